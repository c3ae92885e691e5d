// The BF16 variant of the tensor-core fused kernel.
#include "tdg_fused_tc.cuh"

namespace tdg {

cudaError_t launch_tc_bf16(const FusedArgs& a, const TcLaunch& t, int n_ctas, cudaStream_t s) {
  return launch_variant<true, false>(a, t, n_ctas, s);
}

}  // namespace tdg
