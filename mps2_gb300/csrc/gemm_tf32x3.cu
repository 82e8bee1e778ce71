// Split-precision grouped GEMM (3xTF32 on tcgen05) -- entry points.
#include "gq_runtime.hpp"

namespace gq {

int gemm_tile_m(Precision) { return 64; }
int gemm_tile_n(Precision) { return 64; }

void launch_gemm_tf32x3(const ContractPlan &, const double *, const double *, double *) {
  fail(kInvalidArgument, "the 3xTF32 contraction kernel is not available in this build");
}

}  // namespace gq
