// Tensor-core fused kernel: shared-memory size, the bounded-wait self-test and the dispatch to
// the variants of each precision and main site class (instantiated from tdg_tc_inst.cu).
#include "tdg_fused_tc.cuh"

namespace tdg {

size_t fused_tc_smem_bytes() {
  return 2 * (size_t)OPB + sizeof(float) * (RMAX * LDS + 2 * RMAX * MAX_OUT + RMAX * TDG_MAX_DIN + PBUF) +
         sizeof(DevGroup) + sizeof(double) * (MAX_OUT + (NTC / 32) * MAX_OUT) + 3 * sizeof(uint64_t) + 16 + 3 * 128;
}

// Self-test of the bounded wait: one thread waits on an mbarrier that nothing arrives at and
// records whether the wait gave up (it must) instead of spinning forever.
namespace {
__global__ void bounded_wait_selftest_kernel(int max_polls, int* gave_up) {
  __shared__ __align__(8) uint64_t bar;
  mbar_init(&bar, 1);
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  *gave_up = mbar_wait(&bar, 0, max_polls) ? 0 : 1;
}
}  // namespace

cudaError_t launch_bounded_wait_selftest(int max_polls, int* gave_up, cudaStream_t s) {
  bounded_wait_selftest_kernel<<<1, 1, 0, s>>>(max_polls, gave_up);
  count_launch();
  return cudaGetLastError();
}

namespace {
using TcFn = cudaError_t (*)(const FusedArgs&, const TcLaunch&, int, cudaStream_t);
#define TDG_TC_ENTRY(P, C) TDG_TC_FN(P, C),
const TcFn kTcTf32[] = {TDG_TC_EACH_CLASS(TDG_TC_ENTRY, tf32)};
const TcFn kTcBf16[] = {TDG_TC_EACH_CLASS(TDG_TC_ENTRY, bf16)};
const TcFn kTc3x[] = {TDG_TC_EACH_CLASS(TDG_TC_ENTRY, 3x)};
#undef TDG_TC_ENTRY
static_assert(sizeof(kTcTf32) / sizeof(kTcTf32[0]) == jetcls::N_CLASSES, "one variant per site class");
}  // namespace

cudaError_t launch_fused_tc(const FusedArgs& a, const TcLaunch& t, int n_ctas, cudaStream_t s) {
  const int c = t.cls_main >= 0 && t.cls_main < jetcls::N_CLASSES ? t.cls_main : 0;
  if (t.x3) return kTc3x[c](a, t, n_ctas, s);
  if (t.bf16) return kTcBf16[c](a, t, n_ctas, s);
  return kTcTf32[c](a, t, n_ctas, s);
}

}  // namespace tdg
