// Host-side helpers shared by the translation units behind the C ABI.
#pragma once
#include <string>
#include "../../include/refeff_fms.h"

namespace rfx {
// Records the message returned by refeff_fms_last_error for this context.
void set_last_error(refeff_fms_context* ctx, const std::string& msg);
}  // namespace rfx
