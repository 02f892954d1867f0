// Host-side helpers shared by the translation units behind the C ABI.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include "../../include/refeff_fms.h"

namespace rfx {
// Records the message returned by refeff_fms_last_error for this context.
void set_last_error(refeff_fms_context* ctx, const std::string& msg);
// Plans and models hold a reference on their context (released on destroy).
void context_retain(refeff_fms_context* ctx);
void context_release(refeff_fms_context* ctx);
// The context's device ordinal and its (non-blocking) stream.
int context_device(const refeff_fms_context* ctx);
cudaStream_t context_stream(const refeff_fms_context* ctx);
// FEFF bcoef transition matrix (mkgtr.cu); the arguments of refeff_fms_transition_matrix.
int mkgtr_transition_matrix(int lmax, int kinit, int polarization, const refeff_complex128* ptz9, int multipole,
                            int trace_orbital, int spin, int nsp, double angks, refeff_complex128* out,
                            int32_t* lind, int32_t* kiind);
// geom.dat text (FEFF rdinp's write_geom_dat) for the cluster of a feff.inp (feff_inp.cu).
int geom_dat_from_feff_inp(const std::string& path, std::string& text, std::string& err);
}  // namespace rfx
