// Reduction, optimizer and dot-product kernels around the fused loss/gradient kernel.
#include <mutex>

#include "tdg_internal.h"

namespace tdg {

namespace {

// grad[p][j] = sum over the problem's segments (fixed order) of partial[seg][j]
__global__ void reduce_grad_kernel(const float* __restrict__ partial, int64_t stride,
                                   const int32_t* __restrict__ seg_begin,
                                   const int32_t* __restrict__ seg_list, int64_t n_params,
                                   float* __restrict__ grad) {
  const int p = blockIdx.y;
  const int b = seg_begin[p], e = seg_begin[p + 1];
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n_params;
       j += (int64_t)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int i = b; i < e; ++i) s += partial[(int64_t)seg_list[i] * stride + j];
    grad[(int64_t)p * n_params + j] = s;
  }
}

// loss[2p] = sum_slots w * sum_cta slot_partial; loss[2p+1] with the normalized weights.
__global__ void reduce_loss_kernel(const double* __restrict__ slot_partial, int n_ctas, int n_slots,
                                   const int32_t* __restrict__ slot_problem,
                                   const double* __restrict__ slot_w,
                                   const double* __restrict__ slot_wn, int n_problems,
                                   double* __restrict__ loss) {
  extern __shared__ double sums[];
  for (int s = threadIdx.x; s < n_slots; s += blockDim.x) {
    double v = 0.0;
    for (int c = 0; c < n_ctas; ++c) v += slot_partial[(int64_t)c * n_slots + s];
    sums[s] = v;
  }
  __syncthreads();
  for (int p = threadIdx.x; p < n_problems; p += blockDim.x) {
    double l = 0.0, ln = 0.0;
    for (int s = 0; s < n_slots; ++s)
      if (slot_problem[s] == p) {
        l += slot_w[s] * sums[s];
        ln += slot_wn[s] * sums[s];
      }
    loss[2 * p] = l;
    loss[2 * p + 1] = ln;
  }
}

// torch.optim.Adam (non-amsgrad): m.lerp_(g, 1-b1); v = v*b2 + (1-b2) g g;
// p -= lr / (1 - b1^t) * m / (sqrt(v) / sqrt(1 - b2^t) + eps)
__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g,
                            float* __restrict__ m, float* __restrict__ v,
                            const float* __restrict__ step, int64_t n, tdg_adam_desc hp) {
  const double t = (double)(*step) + 1.0;
  const double bc1 = 1.0 - pow((double)hp.beta1, t);
  const double bc2 = 1.0 - pow((double)hp.beta2, t);
  const float step_size = (float)((double)hp.lr / bc1);
  const float bc2_sqrt = (float)sqrt(bc2);
  const float w1 = (float)(1.0 - (double)hp.beta1);
  const float w2 = (float)(1.0 - (double)hp.beta2);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float gi = hp.maximize ? -g[i] : g[i];
    if (hp.weight_decay != 0.f) gi = gi + hp.weight_decay * p[i];
    const float mi = m[i] + w1 * (gi - m[i]);
    const float vi = v[i] * hp.beta2 + w2 * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float denom = sqrtf(vi) / bc2_sqrt + hp.eps;
    p[i] = p[i] - step_size * (mi / denom);
  }
}

__global__ void adam_step_inc(float* step) { *step += 1.f; }

__global__ void dot_f64_kernel(const float* __restrict__ a, const float* __restrict__ b, int64_t n,
                               double* __restrict__ partial) {
  double s = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    s += (double)a[i] * (double)b[i];
  for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
  __shared__ double w[32];
  if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += w[i];
    partial[blockIdx.x] = t;
  }
}

__global__ void dot_finish_kernel(const double* __restrict__ partial, int n, double* out) {
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < n; ++i) t += partial[i];
    *out = t;
  }
}

// one thread per column k of the [n_t][rest] time-slice layout: a running FP64 sum of the
// squared residuals of the earlier slices (rows of one slice are adjacent, so a warp's loads of
// one slice are coalesced)
__global__ void causal_weights_kernel(const float* __restrict__ op, int64_t rest, int n_eq,
                                      int64_t n_t, float tol, float* __restrict__ w) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < rest;
       k += (int64_t)gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int64_t s = 0; s < n_t; ++s) {
      const int64_t i = s * rest + k;
      w[i] = expf(-tol * (float)acc);
      double r = 0.0;
      for (int e = 0; e < n_eq; ++e) {
        const double v = op[i * n_eq + e];
        r += v * v;
      }
      acc += r;
    }
  }
}

__global__ void gather_rows_kernel(const float* __restrict__ src, int64_t n_src,
                                   const int64_t* __restrict__ index, int64_t n, int row_len,
                                   float* __restrict__ dst) {
  const int64_t total = n * row_len;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / row_len, c = e - r * row_len;
    const int64_t j = index[r];
    dst[e] = (j >= 0 && j < n_src) ? src[j * row_len + c] : 0.f;
  }
}

}  // namespace

cudaError_t launch_causal_weights(const float* op, int64_t n_rows, int n_eq, int64_t n_t,
                                  float tol, float* w, cudaStream_t s) {
  const int64_t rest = n_rows / n_t;
  int64_t blocks = (rest + 127) / 128;
  if (blocks > 1216) blocks = 1216;
  causal_weights_kernel<<<(int)blocks, 128, 0, s>>>(op, rest, n_eq, n_t, tol, w);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_gather_rows(const float* src, int64_t n_src, const int64_t* index, int64_t n,
                               int row_len, float* dst, cudaStream_t s) {
  int64_t blocks = (n * row_len + 255) / 256;
  if (blocks > 1216) blocks = 1216;
  gather_rows_kernel<<<(int)blocks, 256, 0, s>>>(src, n_src, index, n, row_len, dst);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_reduce_grad(const float* partial, int64_t part_stride, const int32_t* seg_begin,
                               const int32_t* seg_list, int n_problems, int64_t n_params,
                               float* grad, cudaStream_t s) {
  int bx = (int)((n_params + 255) / 256);
  if (bx > 1024) bx = 1024;
  reduce_grad_kernel<<<dim3(bx, n_problems), 256, 0, s>>>(partial, part_stride, seg_begin, seg_list,
                                                           n_params, grad);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_reduce_loss(const double* slot_partial, int n_ctas, int n_slots,
                               const int32_t* slot_problem, const double* slot_w,
                               const double* slot_wn, int n_problems, double* loss,
                               cudaStream_t s) {
  reduce_loss_kernel<<<1, 256, sizeof(double) * n_slots, s>>>(slot_partial, n_ctas, n_slots,
                                                              slot_problem, slot_w, slot_wn,
                                                              n_problems, loss);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_adam(float* p, const float* g, float* m, float* v, float* step, int64_t n,
                        const tdg_adam_desc& hp, cudaStream_t s) {
  int blocks = (int)((n + 255) / 256);
  if (blocks > 4096) blocks = 4096;
  adam_kernel<<<blocks, 256, 0, s>>>(p, g, m, v, step, n, hp);
  adam_step_inc<<<1, 1, 0, s>>>(step);
  count_launch(2);
  return cudaGetLastError();
}

// scratch for the two-pass dot product lives in a small per-device buffer allocated once; the
// first call on a device allocates it under a lock, so concurrent first calls from several host
// threads neither leak nor hand a kernel a pointer that is still being written. Every later call
// on that device shares the buffer: calls that overlap on the GPU race on it.
namespace {
std::mutex g_dot_mu;
double* g_dot_partial[64] = {nullptr};
}  // namespace

cudaError_t launch_dot_f64(const float* a, const float* b, int64_t n, double* out,
                           cudaStream_t s) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  constexpr int kBlocks = 304;
  double* partial = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_dot_mu);
    if (!g_dot_partial[dev]) {
      e = cudaMalloc(&g_dot_partial[dev], kBlocks * sizeof(double));
      if (e != cudaSuccess) {
        g_dot_partial[dev] = nullptr;
        return e;
      }
    }
    partial = g_dot_partial[dev];
  }
  dot_f64_kernel<<<kBlocks, 256, 0, s>>>(a, b, n, partial);
  dot_finish_kernel<<<1, 32, 0, s>>>(partial, kBlocks, out);
  count_launch(2);
  return cudaGetLastError();
}

}  // namespace tdg
