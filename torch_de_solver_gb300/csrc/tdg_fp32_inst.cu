// One variant of the FP32 fused kernel: main site class TDG_F32_CLS (0..10, tdg_jetcls.h). The
// build compiles this file once per class with -DTDG_F32_CLS=...
#include "tdg_fused_fp32.cuh"

#if !defined(TDG_F32_CLS)
#error "tdg_fp32_inst.cu is compiled once per site class with TDG_F32_CLS"
#endif

namespace tdg {

cudaError_t TDG_F32_FN(TDG_F32_CLS)(const FusedArgs& a, int n_ctas, cudaStream_t s) {
  return launch_fp32_variant<TDG_F32_CLS>(a, n_ctas, s);
}

}  // namespace tdg
