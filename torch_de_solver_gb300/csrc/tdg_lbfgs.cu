// Device-resident L-BFGS (the optimizer the reference selects as torch.optim.LBFGS,
// tedeous/optimizers/optimizer.py:50-51): the curvature history, the two-loop recursion and the
// convergence statistics stay on the device, every dot product in FP64.
//
// State: a ring of history_size + 1 slots of (s, y) pairs, n floats each. The slot at `head` is
// always free, so a new pair is written there first and committed (head advanced) only when its
// curvature y.s passes the test; a rejected pair leaves the history as it was, as in
// torch.optim.LBFGS. rho = 1 / y.s of each slot, the two-loop coefficients alpha and the
// diagonal scale H_diag = y.s / y.y are FP64.
//
// Every reduction is two-level and deterministic: each of kBlocks blocks sums a fixed range of
// elements into its own FP64 partial, and the consumer sums the kBlocks partials in block order.
// The two-loop recursion fuses each step's update with the next step's dot: the kernel for
// history entry i sums the partials of (s_i . q) into alpha_i, applies q -= alpha_i y_i to its
// own range, and writes the partials of the next entry's dot over that range. A loop over k
// entries is k + 1 launches with no host synchronisation.
#include <cmath>

#include "tdg_internal.h"

struct tdg_lbfgs {
  int64_t n;
  int32_t hist;          // history_size
  float* s;              // (hist + 1) x n
  float* y;              // (hist + 1) x n
  double* rho;           // hist + 1 (0: slot not holding an accepted pair)
  double* alpha;         // hist
  double* part;          // 4 x kBlocks partial sums
  double* stats;         // statistics written by tdg_lbfgs_stats
  int32_t* ring;         // [0] head (the free slot), [1] count of accepted pairs
  double* hdiag;         // H_diag
};

namespace tdg {
namespace {

constexpr int kThreads = 256;
constexpr int kBlocks = 304;   // 2 per SM

// [begin, end) of block b's contiguous range
__device__ __forceinline__ void block_range(int64_t n, int64_t* b0, int64_t* b1) {
  const int64_t per = (n + kBlocks - 1) / kBlocks;
  *b0 = (int64_t)blockIdx.x * per;
  *b1 = *b0 + per < n ? *b0 + per : n;
}

// block-wide sum of one double per thread (fixed order: warp shuffles, then warps in order)
__device__ __forceinline__ double block_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < kThreads / 32; ++w) t += sh[w];
  __syncthreads();
  return t;
}

__device__ __forceinline__ double block_max(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < kThreads / 32; ++w) t = fmax(t, sh[w]);
  __syncthreads();
  return t;
}

// the sum of the kBlocks partials of one dot, in block order (every thread gets it)
__device__ __forceinline__ double partials_total(const double* p, double* sh) {
  double v = 0.0;
  for (int i = threadIdx.x; i < kBlocks; i += kThreads) v += p[i];
  // per-thread sums are over a fixed set of indices: the order is the same in every call
  v = block_sum(v, sh);
  if (threadIdx.x == 0) sh[kThreads / 32] = v;
  __syncthreads();
  const double t = sh[kThreads / 32];
  __syncthreads();
  return t;
}

// y = g - g_prev, s = t d into the free slot; partials of y.s and y.y
__global__ void push_kernel(tdg_lbfgs h, const float* __restrict__ g, const float* __restrict__ gp,
                            const float* __restrict__ d, double t) {
  __shared__ double sh[kThreads / 32 + 1];
  const int slot = h.ring[0];
  float* s = h.s + (int64_t)slot * h.n;
  float* y = h.y + (int64_t)slot * h.n;
  int64_t b0, b1;
  block_range(h.n, &b0, &b1);
  double ys = 0.0, yy = 0.0;
  for (int64_t i = b0 + threadIdx.x; i < b1; i += kThreads) {
    const float yv = g[i] - gp[i];
    const float sv = (float)(t * (double)d[i]);
    y[i] = yv;
    s[i] = sv;
    ys += (double)yv * (double)sv;
    yy += (double)yv * (double)yv;
  }
  ys = block_sum(ys, sh);
  yy = block_sum(yy, sh);
  if (threadIdx.x == 0) {
    h.part[blockIdx.x] = ys;
    h.part[kBlocks + blockIdx.x] = yy;
  }
}

// accept the pair when y.s > 1e-10 (torch.optim.LBFGS's test): rho, H_diag, advance the ring
__global__ void push_finish_kernel(tdg_lbfgs h) {
  __shared__ double sh[kThreads / 32 + 1];
  const double ys = partials_total(h.part, sh);
  const double yy = partials_total(h.part + kBlocks, sh);
  if (threadIdx.x == 0) {
    h.stats[4] = ys;
    if (ys > 1e-10) {
      const int slot = h.ring[0];
      h.rho[slot] = 1.0 / ys;
      *h.hdiag = ys / yy;
      h.ring[0] = (slot + 1) % (h.hist + 1);
      h.ring[1] = h.ring[1] < h.hist ? h.ring[1] + 1 : h.hist;
    }
  }
}

// slot of the i-th newest accepted pair, or -1 when fewer than i + 1 are stored
__device__ __forceinline__ int slot_of(const tdg_lbfgs& h, int i) {
  if (i >= h.ring[1]) return -1;
  const int m = h.hist + 1;
  return ((h.ring[0] - 1 - i) % m + m) % m;
}

// Loop 1 of the two-loop recursion, newest pair first. mode 0 (entry -1): q = -g and the partials
// of s_0 . q. mode 1 (entry i): alpha_i = rho_i * (s_i . q), q -= alpha_i y_i, then the partials
// of s_{i+1} . q. Absent entries contribute nothing.
__global__ void loop1_kernel(tdg_lbfgs h, const float* __restrict__ g, float* __restrict__ q, int i,
                             int k) {
  __shared__ double sh[kThreads / 32 + 1];
  int64_t b0, b1;
  block_range(h.n, &b0, &b1);
  double* part_cur = h.part + (i & 1) * kBlocks;
  double* part_next = h.part + ((i + 1) & 1) * kBlocks;
  if (i < 0) {
    for (int64_t e = b0 + threadIdx.x; e < b1; e += kThreads) q[e] = -g[e];
  } else {
    const int si = slot_of(h, i);
    if (si >= 0) {
      const double a = h.rho[si] * partials_total(part_cur, sh);
      if (blockIdx.x == 0 && threadIdx.x == 0) h.alpha[i] = a;
      const float* y = h.y + (int64_t)si * h.n;
      for (int64_t e = b0 + threadIdx.x; e < b1; e += kThreads) q[e] = (float)((double)q[e] - a * (double)y[e]);
    } else if (blockIdx.x == 0 && threadIdx.x == 0) {
      h.alpha[i] = 0.0;
    }
  }
  if (i + 1 < k) {
    const int sn = slot_of(h, i + 1);
    double v = 0.0;
    if (sn >= 0) {
      const float* s = h.s + (int64_t)sn * h.n;
      for (int64_t e = b0 + threadIdx.x; e < b1; e += kThreads) v += (double)s[e] * (double)q[e];
    }
    v = block_sum(v, sh);
    if (threadIdx.x == 0) part_next[blockIdx.x] = v;
  }
}

// Loop 2, oldest pair first over j = 0..k-1 (entry i = k - 1 - j). mode j = -1: r = H_diag q and
// the partials of y_{i(0)} . r. Entry j: beta = rho (y . r), r += (alpha - beta) s, then the
// partials of the next entry's y . r.
__global__ void loop2_kernel(tdg_lbfgs h, float* __restrict__ r, int j, int k) {
  __shared__ double sh[kThreads / 32 + 1];
  int64_t b0, b1;
  block_range(h.n, &b0, &b1);
  double* part_cur = h.part + 2 * kBlocks + (j & 1) * kBlocks;
  double* part_next = h.part + 2 * kBlocks + ((j + 1) & 1) * kBlocks;
  if (j < 0) {
    const double hd = *h.hdiag;
    for (int64_t e = b0 + threadIdx.x; e < b1; e += kThreads) r[e] = (float)((double)r[e] * hd);
  } else {
    const int i = k - 1 - j;
    const int si = slot_of(h, i);
    if (si >= 0) {
      const double be = h.rho[si] * partials_total(part_cur, sh);
      const double c = h.alpha[i] - be;
      const float* s = h.s + (int64_t)si * h.n;
      for (int64_t e = b0 + threadIdx.x; e < b1; e += kThreads) r[e] = (float)((double)r[e] + c * (double)s[e]);
    }
  }
  if (j + 1 < k) {
    const int sn = slot_of(h, k - 2 - j);
    double v = 0.0;
    if (sn >= 0) {
      const float* y = h.y + (int64_t)sn * h.n;
      for (int64_t e = b0 + threadIdx.x; e < b1; e += kThreads) v += (double)y[e] * (double)r[e];
    }
    v = block_sum(v, sh);
    if (threadIdx.x == 0) part_next[blockIdx.x] = v;
  }
}

// partials of g.d, sum |g|, max |g|, max |d| (d may be null: its entries then read as 0)
__global__ void stats_kernel(tdg_lbfgs h, const float* __restrict__ g, const float* __restrict__ d) {
  __shared__ double sh[kThreads / 32 + 1];
  int64_t b0, b1;
  block_range(h.n, &b0, &b1);
  double gd = 0.0, g1 = 0.0, gm = 0.0, dm = 0.0;
  for (int64_t e = b0 + threadIdx.x; e < b1; e += kThreads) {
    const double gv = g[e], dv = d ? d[e] : 0.0;
    gd += gv * dv;
    g1 += fabs(gv);
    gm = fmax(gm, fabs(gv));
    dm = fmax(dm, fabs(dv));
  }
  gd = block_sum(gd, sh);
  g1 = block_sum(g1, sh);
  gm = block_max(gm, sh);
  dm = block_max(dm, sh);
  if (threadIdx.x == 0) {
    h.part[blockIdx.x] = gd;
    h.part[kBlocks + blockIdx.x] = g1;
    h.part[2 * kBlocks + blockIdx.x] = gm;
    h.part[3 * kBlocks + blockIdx.x] = dm;
  }
}

__global__ void stats_finish_kernel(tdg_lbfgs h, const float* __restrict__ loss, double* __restrict__ out) {
  __shared__ double sh[kThreads / 32 + 1];
  const double gd = partials_total(h.part, sh);
  const double g1 = partials_total(h.part + kBlocks, sh);
  double gm = 0.0, dm = 0.0;
  for (int i = threadIdx.x; i < kBlocks; i += kThreads) {
    gm = fmax(gm, h.part[2 * kBlocks + i]);
    dm = fmax(dm, h.part[3 * kBlocks + i]);
  }
  gm = block_max(gm, sh);
  dm = block_max(dm, sh);
  if (threadIdx.x == 0) {
    out[0] = gd;
    out[1] = g1;
    out[2] = gm;
    out[3] = dm;
    out[4] = loss ? (double)*loss : 0.0;
  }
}

__global__ void axpy_kernel(const float* __restrict__ x, const float* __restrict__ d, double t,
                            float* __restrict__ out, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (float)((double)x[i] + t * (double)d[i]);
}

__global__ void reset_kernel(tdg_lbfgs h) {
  for (int i = threadIdx.x; i <= h.hist; i += blockDim.x) h.rho[i] = 0.0;
  if (threadIdx.x == 0) {
    h.ring[0] = 0;
    h.ring[1] = 0;
    *h.hdiag = 1.0;
  }
}

tdg_status launched(const char* what) {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return record_error(TDG_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  return TDG_OK;
}

}  // namespace
}  // namespace tdg

extern "C" tdg_status tdg_lbfgs_create(int64_t n, int32_t history_size, tdg_lbfgs** out) {
  using namespace tdg;
  if (!out) return record_error(TDG_ERR_INVALID, "tdg_lbfgs_create: null output");
  *out = nullptr;
  if (n <= 0 || history_size <= 0)
    return record_error(TDG_ERR_SHAPE, "tdg_lbfgs_create: n = %lld and history_size = %d must be "
                        "positive", (long long)n, history_size);
  tdg_lbfgs* h = new tdg_lbfgs{};
  h->n = n;
  h->hist = history_size;
  const size_t vec = sizeof(float) * (size_t)n * (size_t)(history_size + 1);
  cudaError_t e = cudaSuccess;
  void* p[7] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  const size_t sz[7] = {vec, vec, sizeof(double) * (history_size + 1), sizeof(double) * history_size,
                        sizeof(double) * 4 * kBlocks, sizeof(double) * 8, sizeof(int32_t) * 2 + sizeof(double) * 2};
  for (int i = 0; i < 7 && e == cudaSuccess; ++i) e = cudaMalloc(&p[i], sz[i]);
  if (e != cudaSuccess) {
    for (void* q : p)
      if (q) cudaFree(q);
    delete h;
    return record_error(TDG_ERR_NOMEM, "tdg_lbfgs_create: %s", cudaGetErrorString(e));
  }
  h->s = static_cast<float*>(p[0]);
  h->y = static_cast<float*>(p[1]);
  h->rho = static_cast<double*>(p[2]);
  h->alpha = static_cast<double*>(p[3]);
  h->part = static_cast<double*>(p[4]);
  h->stats = static_cast<double*>(p[5]);
  h->ring = static_cast<int32_t*>(p[6]);
  h->hdiag = reinterpret_cast<double*>(static_cast<char*>(p[6]) + 16);
  cudaMemset(h->stats, 0, sizeof(double) * 8);
  reset_kernel<<<1, 256>>>(*h);
  count_launch();
  tdg_status st = launched("tdg_lbfgs_create");
  // the state is ready before any stream (blocking or not) uses it
  if (st == TDG_OK && (e = cudaDeviceSynchronize()) != cudaSuccess)
    st = record_error(TDG_ERR_CUDA, "tdg_lbfgs_create: %s", cudaGetErrorString(e));
  if (st != TDG_OK) {
    for (void* q : p) cudaFree(q);
    delete h;
    return st;
  }
  *out = h;
  return TDG_OK;
}

extern "C" tdg_status tdg_lbfgs_destroy(tdg_lbfgs* h) {
  if (!h) return TDG_OK;
  cudaFree(h->s);
  cudaFree(h->y);
  cudaFree(h->rho);
  cudaFree(h->alpha);
  cudaFree(h->part);
  cudaFree(h->stats);
  cudaFree(h->ring);
  delete h;
  return TDG_OK;
}

extern "C" tdg_status tdg_lbfgs_reset(tdg_lbfgs* h, tdg_stream_t stream) {
  using namespace tdg;
  if (!h) return record_error(TDG_ERR_INVALID, "tdg_lbfgs_reset: null state");
  reset_kernel<<<1, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(*h);
  count_launch();
  return launched("tdg_lbfgs_reset");
}

extern "C" tdg_status tdg_lbfgs_push(tdg_lbfgs* h, const float* g, const float* g_prev, const float* d,
                                     double t, tdg_stream_t stream) {
  using namespace tdg;
  if (!h || !g || !g_prev || !d) return record_error(TDG_ERR_INVALID, "tdg_lbfgs_push: null argument");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  push_kernel<<<kBlocks, kThreads, 0, s>>>(*h, g, g_prev, d, t);
  push_finish_kernel<<<1, kThreads, 0, s>>>(*h);
  count_launch(2);
  return launched("tdg_lbfgs_push");
}

extern "C" tdg_status tdg_lbfgs_direction(tdg_lbfgs* h, const float* g, float* d, int32_t n_pairs_bound,
                                          tdg_stream_t stream) {
  using namespace tdg;
  if (!h || !g || !d) return record_error(TDG_ERR_INVALID, "tdg_lbfgs_direction: null argument");
  if (n_pairs_bound < 0 || n_pairs_bound > h->hist)
    return record_error(TDG_ERR_SHAPE, "tdg_lbfgs_direction: n_pairs_bound = %d outside [0, %d]",
                        n_pairs_bound, h->hist);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const int k = n_pairs_bound;
  for (int i = -1; i < k; ++i) loop1_kernel<<<kBlocks, kThreads, 0, s>>>(*h, g, d, i, k);
  for (int j = -1; j < k; ++j) loop2_kernel<<<kBlocks, kThreads, 0, s>>>(*h, d, j, k);
  count_launch(2 * (k + 1));
  return launched("tdg_lbfgs_direction");
}

extern "C" tdg_status tdg_lbfgs_stats(tdg_lbfgs* h, const float* g, const float* d, const float* loss,
                                      double* out, tdg_stream_t stream) {
  using namespace tdg;
  if (!h || !g || !out) return record_error(TDG_ERR_INVALID, "tdg_lbfgs_stats: null argument");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  stats_kernel<<<kBlocks, kThreads, 0, s>>>(*h, g, d);
  stats_finish_kernel<<<1, kThreads, 0, s>>>(*h, loss, out);
  count_launch(2);
  return launched("tdg_lbfgs_stats");
}

extern "C" tdg_status tdg_axpy(const float* x, const float* d, double t, float* out, int64_t n,
                               tdg_stream_t stream) {
  using namespace tdg;
  if (!x || !d || !out) return record_error(TDG_ERR_INVALID, "tdg_axpy: null argument");
  if (n < 0) return record_error(TDG_ERR_SHAPE, "tdg_axpy: negative length");
  if (n == 0) return TDG_OK;
  int blocks = (int)((n + 255) / 256);
  if (blocks > 1216) blocks = 1216;
  axpy_kernel<<<blocks, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(x, d, t, out, n);
  count_launch();
  return launched("tdg_axpy");
}
