// tdg_dot_f64_noalloc: the FP64 dot product (used by the L-BFGS two-loop recursion) for callers
// that must not have this library allocate device memory.
//
// Who needs it: a host that owns all device memory itself, such as a framework whose caching
// allocator has already reserved the GPU, or a foreign-language runtime that binds this C ABI
// under a fixed device-memory budget. tdg_dot_f64 calls cudaMalloc for its partial sums the first
// time it runs on a device; such callers cannot allow that, because the allocation can fail when
// memory is reserved elsewhere and it escapes their accounting.
//
// How: the per-block partial sums live in a file-scope static __device__ array of
// TDG_DOT_NOALLOC_MAX_BLOCKS doubles (32 KiB), which every GPU that loads the library holds until
// the process exits. Host code cannot use the array's name as a device address, so the first
// call on each device looks the address up with cudaGetSymbolAddress while that device is
// current and caches it. Each call writes every partial it later reads, so nothing needs
// clearing. All calls share the one array: calls that overlap on the GPU (for example on two
// streams at once) race on it and must be ordered by the caller.
#include <cstdio>
#include <mutex>

#include "tdg_internal.h"

namespace tdg {

namespace {

constexpr int kThreads = 256;
constexpr int64_t kChunk = TDG_DOT_NOALLOC_CHUNK;   // elements summed by one block

static __device__ __align__(256) double g_dot_partials[TDG_DOT_NOALLOC_MAX_BLOCKS];

// block b sums a[i] * b[i] over its chunk [b * kChunk, (b + 1) * kChunk) in FP64
__global__ void dot_chunk_kernel(const float* __restrict__ a, const float* __restrict__ b,
                                 int64_t n, double* __restrict__ partials) {
  const int64_t begin = (int64_t)blockIdx.x * kChunk;
  const int64_t end = begin + kChunk < n ? begin + kChunk : n;
  double s = 0.0;
  for (int64_t i = begin + threadIdx.x; i < end; i += kThreads) s += (double)a[i] * (double)b[i];
  for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
  __shared__ double w[kThreads / 32];
  if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < kThreads / 32; ++i) t += w[i];
    partials[blockIdx.x] = t;
  }
}

// one warp adds the partials in a fixed order
__global__ void dot_partials_sum_kernel(const double* __restrict__ partials, int n_blocks,
                                        double* __restrict__ out) {
  double s = 0.0;
  for (int i = threadIdx.x; i < n_blocks; i += 32) s += partials[i];
  for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
  if (threadIdx.x == 0) *out = s;
}

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_scratch[kMaxDevices] = {nullptr};

// Device address of g_dot_partials on the current device, looked up once per device.
cudaError_t scratch_on_current_device(double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_dot_partials);
    if (e != cudaSuccess) return e;
    g_scratch[dev] = static_cast<double*>(p);
  }
  *out = g_scratch[dev];
  return cudaSuccess;
}

}  // namespace

}  // namespace tdg

extern "C" tdg_status tdg_dot_f64_noalloc(const float* a, const float* b, int64_t n, double* out,
                                          tdg_stream_t stream) {
  using namespace tdg;
  if (!a || !b || !out) return record_error(TDG_ERR_INVALID, "tdg_dot_f64_noalloc: null argument");
  if (n < 0) return record_error(TDG_ERR_SHAPE, "tdg_dot_f64_noalloc: negative length");
  if (n > TDG_DOT_NOALLOC_MAX_N)
    return record_error(TDG_ERR_SHAPE,
                        "tdg_dot_f64_noalloc: n = %lld exceeds the static scratch limit of %lld "
                        "elements (%d partial sums of %lld elements); use tdg_dot_f64",
                        (long long)n, (long long)TDG_DOT_NOALLOC_MAX_N,
                        TDG_DOT_NOALLOC_MAX_BLOCKS, (long long)TDG_DOT_NOALLOC_CHUNK);
  double* partials = nullptr;
  cudaError_t e = scratch_on_current_device(&partials);
  if (e != cudaSuccess)
    return record_error(TDG_ERR_CUDA, "tdg_dot_f64_noalloc: cudaGetSymbolAddress: %s",
                        cudaGetErrorString(e));
  const int n_blocks = n == 0 ? 1 : (int)((n + TDG_DOT_NOALLOC_CHUNK - 1) / TDG_DOT_NOALLOC_CHUNK);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  dot_chunk_kernel<<<n_blocks, kThreads, 0, s>>>(a, b, n, partials);
  dot_partials_sum_kernel<<<1, 32, 0, s>>>(partials, n_blocks, out);
  count_launch(2);
  e = cudaGetLastError();
  if (e != cudaSuccess) return record_error(TDG_ERR_CUDA, "tdg_dot_f64_noalloc launch: %s", cudaGetErrorString(e));
  return TDG_OK;
}
