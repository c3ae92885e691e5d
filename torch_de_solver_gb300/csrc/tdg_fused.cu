// FP32 fused kernel: the dispatch to the variant of the plan's main site class (the kernel is
// tdg_fused_fp32.cuh, instantiated once per class from tdg_fp32_inst.cu).
#include "tdg_internal.h"
#include "tdg_jetcls.h"

namespace tdg {

namespace {
using F32Fn = cudaError_t (*)(const FusedArgs&, int, cudaStream_t);
#define TDG_F32_ENTRY(P, C) TDG_F32_FN(C),
const F32Fn kF32[] = {TDG_TC_EACH_CLASS(TDG_F32_ENTRY, fp32)};
#undef TDG_F32_ENTRY
static_assert(sizeof(kF32) / sizeof(kF32[0]) == jetcls::N_CLASSES, "one variant per site class");
}  // namespace

cudaError_t launch_fused_fp32(const FusedArgs& a, int cls_main, int n_ctas, cudaStream_t s) {
  const int c = cls_main >= 0 && cls_main < jetcls::N_CLASSES ? cls_main : 0;
  return kF32[c](a, n_ctas, s);
}

}  // namespace tdg
