"""GB300-native (sm_103a) implementation of refeff's real-space FMS hot path.

The compute lives in librefeff_fms.so (CUDA kernels + C ABI, include/refeff_fms.h);
this package is the Python mirror of the reference interface used by tests and
benchmarks.  There is no CPU fallback.
"""
from .fms import (  # noqa: F401
    FORM_BICGSTAB,
    FORM_FP32_REFINED,
    FORM_FP64_LU,
    Context,
    FmsError,
    FmsRealSpacePlan,
    PrecondModel,
    complex_lu_solve_batched,
    debye_sigma2_table,
    ff2x_read_xsect_dat,
    ff2x_xanes_mu,
    ff2x_xscorr,
    fms_full_scattering_spectrum,
    fms_real_space_plan,
    fms_real_space_spectrum,
    fms_real_space_spectrum_device,
    fms_real_space_spectrum_multi,
    fms_yprep_cluster,
    gg_section,
    load,
    mkgtr_trace,
    mkgtr_trace_device,
    read_phase_bin,
    reciprocal_core_hole,
    reciprocal_integrate,
    run_fms_in_dir,
    run_mkgtr_in_dir,
    transition_matrix,
    write_fms_bin,
    write_gg_dat,
    write_gg_diag_bin,
    write_gg_slice_bin,
    write_gtr_dat,
)

__all__ = [
    "FORM_BICGSTAB", "FORM_FP32_REFINED", "FORM_FP64_LU", "Context", "FmsError", "FmsRealSpacePlan", "PrecondModel", "complex_lu_solve_batched",
    "debye_sigma2_table", "ff2x_read_xsect_dat", "ff2x_xanes_mu", "ff2x_xscorr", "fms_full_scattering_spectrum",
    "fms_real_space_plan", "fms_real_space_spectrum", "fms_real_space_spectrum_device", "fms_real_space_spectrum_multi",
    "fms_yprep_cluster",
    "gg_section", "load", "mkgtr_trace", "mkgtr_trace_device", "read_phase_bin", "reciprocal_core_hole",
    "reciprocal_integrate", "run_fms_in_dir", "run_mkgtr_in_dir",
    "transition_matrix", "write_fms_bin", "write_gg_dat", "write_gg_diag_bin", "write_gg_slice_bin",
    "write_gtr_dat",
]
