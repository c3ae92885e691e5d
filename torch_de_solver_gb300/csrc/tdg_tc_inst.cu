// One variant of the tensor-core fused kernel: precision TDG_TC_PREC (tf32 | bf16 | 3x) and main
// site class TDG_TC_CLS (0..10, tdg_jetcls.h). The build compiles this file once per variant with
// -DTDG_TC_PREC=... -DTDG_TC_BF16=... -DTDG_TC_X3=... -DTDG_TC_CLS=...
#include "tdg_fused_tc.cuh"

#if !defined(TDG_TC_PREC) || !defined(TDG_TC_BF16) || !defined(TDG_TC_X3) || !defined(TDG_TC_CLS)
#error "tdg_tc_inst.cu is compiled once per variant with TDG_TC_PREC, TDG_TC_BF16, TDG_TC_X3, TDG_TC_CLS"
#endif

namespace tdg {

cudaError_t TDG_TC_FN(TDG_TC_PREC, TDG_TC_CLS)(const FusedArgs& a, const TcLaunch& t, int n_ctas,
                                               cudaStream_t s) {
  return launch_variant<TDG_TC_BF16 != 0, TDG_TC_X3 != 0, TDG_TC_CLS>(a, t, n_ctas, s);
}

}  // namespace tdg
