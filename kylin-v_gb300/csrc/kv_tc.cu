// Mixed-precision grouped complex GEMM (tcgen05, 3M with TF32 hi/lo split).
#include "kv_internal.h"

namespace kv {

void launch_gemm_mixed(const GemmPlan &, const double2 *, const double2 *, double2 *, double, const int *) {
    throw Error(KV_EINVAL, "mixed-precision GEMM is not built yet");
}

}  // namespace kv
