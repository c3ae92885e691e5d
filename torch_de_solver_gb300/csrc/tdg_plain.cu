// Plain form: the same computation as the fused kernels, issued the way a framework issues it -
// one launch per layer operation, every activation of every (point, stream) row materialised in
// device memory. Rows of a group are stream-major: row s * n + i is stream s of point i.
//   forward : input layer -> [tanh jet -> Linear] x (L-2) -> tanh jet -> output layer
//   loss    : operator program, squared errors (FP64 atomics per slot), loss seeds dL/dY
//   backward: output layer -> [jet adjoint -> dW = G^T H, db, dX = G W] ... -> input layer
// It is the baseline the fused kernels are measured against (the reference's GPU path is
// likewise one ATen launch per op with activations in device memory).
#include <algorithm>

#include "tdg_internal.h"

namespace tdg {

namespace {

constexpr int PT = 256;

__device__ __forceinline__ float sgk(int k, float t, float s1, float s2, float s3, float s4) {
  return k == 0 ? t : k == 1 ? s1 : k == 2 ? s2 : k == 3 ? s3 : s4;
}
__device__ __forceinline__ float pw(float x, float p) {
  if (p == 1.f) return x;
  if (p == 2.f) return x * x;
  if (p == 0.f) return 1.f;
  if (p == 3.f) return x * x * x;
  return powf(x, p);
}
__device__ __forceinline__ float dpw(float x, float p) {
  if (p == 1.f) return 1.f;
  if (p == 2.f) return 2.f * x;
  if (p == 0.f) return 0.f;
  if (p == 3.f) return 3.f * x * x;
  return p * powf(x, p - 1.f);
}

// Z1[s*n + i][j] for every stream row
__global__ void plain_input(const DevGroup* __restrict__ G, const float* const* __restrict__ arrays,
                            const float* __restrict__ W0, const float* __restrict__ b0, int d_in,
                            int N, float* __restrict__ Z) {
  const int n = G->n_rows, S = G->S;
  const int64_t total = (int64_t)n * S * N;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(e % N);
    const int64_t r = e / N;
    const int s = (int)(r / n), i = (int)(r % n);
    const int o = G->st_order[s];
    float z = 0.f;
    if (o == 0) {
      const int q = G->st_site[s];
      const float* x = arrays[G->site_points[q]] + (int64_t)i * d_in;
      for (int a = 0; a < d_in; ++a) z = fmaf(W0[j * d_in + a], x[a] + G->site_off[q][a], z);
      z += b0[j];
    } else if (o == 1) {
      z = W0[j * d_in + G->st_axis[s]];
    }
    Z[r * N + j] = z;
  }
}

// H = tanh jet of Z, thread per (point, neuron)
__global__ void plain_jet_fwd(const DevGroup* __restrict__ G, const float* __restrict__ Z,
                              float* __restrict__ H, int N) {
  const int n = G->n_rows;
  const int64_t total = (int64_t)n * N;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(e % N), i = (int)(e / N);
    for (int q = 0; q < G->n_sites; ++q) {
      const int ns = G->site_nstreams[q], base = G->site_streams[q][0];
      const float t = tanhf(Z[((int64_t)base * n + i) * N + j]);
      const float s1 = 1.f - t * t, s2 = -2.f * t * s1, s3 = s1 * (6.f * t * t - 2.f);
      H[((int64_t)base * n + i) * N + j] = t;
      for (int m = 1; m < ns; ++m) {
        const int s = G->site_streams[q][m];
        float h = 0.f;
        for (int u = 0; u < G->st_nrule[s]; ++u) {
          const DevRule& ru = G->rules[s][u];
          float v = (float)ru.mult * sgk(ru.k, t, s1, s2, s3, 0.f);
          for (int f = 0; f < ru.k; ++f) v *= Z[((int64_t)ru.sub[f] * n + i) * N + j];
          h += v;
        }
        H[((int64_t)s * n + i) * N + j] = h;
      }
    }
  }
}

// In place on G: dL/dH -> dL/dZ, thread per (point, neuron), streams of a site in increasing order
__global__ void plain_jet_bwd(const DevGroup* __restrict__ G, const float* __restrict__ Z,
                              float* __restrict__ Gb, int N) {
  const int n = G->n_rows;
  const int64_t total = (int64_t)n * N;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(e % N), i = (int)(e / N);
    for (int q = 0; q < G->n_sites; ++q) {
      const int ns = G->site_nstreams[q], base = G->site_streams[q][0];
      const float t = tanhf(Z[((int64_t)base * n + i) * N + j]);
      const float s1 = 1.f - t * t, s2 = -2.f * t * s1, s3 = s1 * (6.f * t * t - 2.f);
      const float s4 = t * s1 * (16.f - 24.f * t * t);
      for (int m = 0; m < ns; ++m) {
        const int b = G->site_streams[q][m];
        float acc = 0.f;
        for (int u = 0; u < G->st_npull[b]; ++u) {
          const DevPull& pl = G->pulls[G->st_pull_first[b] + u];
          float v = (float)pl.mult * sgk(pl.kk, t, s1, s2, s3, s4) * Gb[((int64_t)pl.alpha * n + i) * N + j];
          for (int f = 0; f < pl.n_oth; ++f) v *= Z[((int64_t)pl.oth[f] * n + i) * N + j];
          acc += v;
        }
        Gb[((int64_t)b * n + i) * N + j] = acc;
      }
    }
  }
}

// Tiled SIMT GEMM, 64x64 output tile, 16x16 threads with 4x4 outputs each.
//   mode 0: C[r][c] = sum_k A[r][k] B[c][k] (+ bias[c] on value rows)    A: R x K, B: N x K
//   mode 1: C[r][c] = sum_k A[r][k] B[k][c]                              A: R x K, B: K x N
//   mode 2: C[r][c] += sum_t A[t][r] B[t][c]  (atomic; rows t split over blockIdx.z)   A: T x R, B: T x N
template <int MODE>
__global__ void plain_gemm(const float* __restrict__ A, const float* __restrict__ B,
                           float* __restrict__ C, const float* __restrict__ bias,
                           const DevGroup* __restrict__ G, int64_t R, int N, int64_t K) {
  __shared__ float As[16][64 + 4];
  __shared__ float Bs[16][64 + 4];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  // modes 0/1: row tiles on grid.x (up to 2^31-1 of them), column tiles on grid.y
  // mode 2: output rows are neurons, so the roles of x and y are the usual ones
  const int64_t r0 = (int64_t)(MODE == 2 ? blockIdx.y : blockIdx.x) * 64;
  const int c0 = (MODE == 2 ? blockIdx.x : blockIdx.y) * 64;
  float acc[4][4] = {};
  int64_t k_begin = 0, k_end = K;
  if (MODE == 2) {
    const int64_t chunk = (K + gridDim.z - 1) / gridDim.z;
    k_begin = blockIdx.z * chunk;
    k_end = k_begin + chunk < K ? k_begin + chunk : K;
  }
  for (int64_t k0 = k_begin; k0 < k_end; k0 += 16) {
    // operands whose K index is contiguous are read along K (16 floats per row), the others along
    // their row index, so every warp reads contiguous runs
    for (int e = threadIdx.x; e < 16 * 64; e += 256) {
      const bool along_k = MODE != 2;
      const int kk = along_k ? e % 16 : e / 64, m = along_k ? e / 16 : e % 64;
      const int64_t k = k0 + kk, r = r0 + m;
      float a = 0.f;
      if (k < k_end && r < R) a = MODE == 2 ? A[k * R + r] : A[r * K + k];
      As[kk][m] = a;
    }
    for (int e = threadIdx.x; e < 16 * 64; e += 256) {
      const bool along_k = MODE == 0;
      const int kk = along_k ? e % 16 : e / 64, m = along_k ? e / 16 : e % 64;
      const int64_t k = k0 + kk;
      const int c = c0 + m;
      float b = 0.f;
      if (k < k_end && c < N) b = MODE == 0 ? B[(int64_t)c * K + k] : B[k * N + c];
      Bs[kk][m] = b;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int64_t r = r0 + ty + 16 * i;
    if (r >= R) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int c = c0 + tx + 16 * j;
      if (c >= N) continue;
      if (MODE == 2) {
        atomicAdd(&C[r * N + c], acc[i][j]);
      } else {
        float v = acc[i][j];
        if (MODE == 0 && bias && G->st_order[r / G->n_rows] == 0) v += bias[c];
        C[r * N + c] = v;
      }
    }
  }
}

// bias gradient: db[j] += sum over value rows of G[r][j]
__global__ void plain_bias_grad(const DevGroup* __restrict__ G, const float* __restrict__ Gb, int N,
                                float* __restrict__ db) {
  const int n = G->n_rows;
  for (int j = blockIdx.x; j < N; j += gridDim.x) {
    float s = 0.f;
    for (int sidx = 0; sidx < G->S; ++sidx) {
      if (G->st_order[sidx] != 0) continue;
      for (int i = threadIdx.x; i < n; i += blockDim.x) s += Gb[((int64_t)sidx * n + i) * N + j];
    }
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    __shared__ float w[PT / 32];
    if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      float t = 0.f;
      for (int k = 0; k < PT / 32; ++k) t += w[k];
      atomicAdd(&db[j], t);
    }
    __syncthreads();
  }
}

// output layer forward: Y[r][o] = H[r] . W[o] (+ b[o] on value rows)
__global__ void plain_output(const DevGroup* __restrict__ G, const float* __restrict__ H,
                             const float* __restrict__ W, const float* __restrict__ b, int K,
                             int d_out, float* __restrict__ Y) {
  const int64_t rows = (int64_t)G->n_rows * G->S;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < rows * d_out;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / d_out;
    const int o = (int)(e % d_out);
    float z = 0.f;
    for (int k = 0; k < K; ++k) z = fmaf(H[r * K + k], W[o * K + k], z);
    if (G->st_order[r / G->n_rows] == 0) z += b[o];
    Y[r * d_out + o] = z;
  }
}

// operator program per point: outputs, squared errors into FP64 slot sums, seeds dL/dY
// (trainable coefficients: values cf[k], gradients accumulated into cgrad[k], k < n_coeff)
__global__ void plain_program(const DevGroup* __restrict__ G, const float* const* __restrict__ arrays,
                              const float* __restrict__ Y, float* __restrict__ GY, int d_out,
                              double* __restrict__ slot_sum, float* __restrict__ outputs,
                              int do_grad, const float* __restrict__ cf, float* __restrict__ cgrad,
                              int n_coeff) {
  const int n = G->n_rows, n_out = G->n_outputs;
  __shared__ double red[MAX_OUT];
  __shared__ float cred[TDG_MAX_COEFF];
  if (threadIdx.x < MAX_OUT) red[threadIdx.x] = 0.0;
  if (threadIdx.x < TDG_MAX_COEFF) cred[threadIdx.x] = 0.f;
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float outv[MAX_OUT] = {};
    for (int t = 0; t < G->n_terms; ++t) {
      const DevTerm& tm = G->terms[t];
      const float c = tm.coeff_param >= 0 ? tm.coeff * cf[tm.coeff_param]
                      : tm.coeff_array >= 0 ? arrays[tm.coeff_array][i] : tm.coeff;
      float prod = 1.f;
      for (int f = 0; f < tm.n_factors; ++f) {
        const DevFactor& fc = G->factors[tm.factor_first + f];
        float F = 0.f;
        for (int u = 0; u < fc.n_parts; ++u) {
          const DevPart& pt = G->parts[fc.part_first + u];
          F = fmaf(Y[((int64_t)pt.stream * n + i) * d_out + fc.var], pt.weight, F);
        }
        prod *= pw(F, fc.power);
      }
      outv[tm.output] += c * prod;
    }
    float seed[MAX_OUT] = {};
    for (int o = 0; o < n_out; ++o) {
      const float tgt = G->target_array >= 0 ? arrays[G->target_array][(int64_t)i * n_out + o] : 0.f;
      const float e = outv[o] - tgt;
      const float rw = G->row_weight_array >= 0 ? arrays[G->row_weight_array][i] : 1.f;
      atomicAdd(&red[o], (double)e * e * (double)rw);
      seed[o] = e * G->seed_scale[o] * rw;
      if (outputs && G->out_offset >= 0) outputs[G->out_offset + (int64_t)i * n_out + o] = outv[o];
    }
    if (!do_grad) continue;
    for (int t = 0; t < G->n_terms; ++t) {
      const DevTerm& tm = G->terms[t];
      const float c = tm.coeff_param >= 0 ? tm.coeff * cf[tm.coeff_param]
                      : tm.coeff_array >= 0 ? arrays[tm.coeff_array][i] : tm.coeff;
      const float dt = seed[tm.output] * c;
      float F[MAX_TERM_FACTORS];
      for (int f = 0; f < tm.n_factors; ++f) {
        const DevFactor& fc = G->factors[tm.factor_first + f];
        float v = 0.f;
        for (int u = 0; u < fc.n_parts; ++u) {
          const DevPart& pt = G->parts[fc.part_first + u];
          v = fmaf(Y[((int64_t)pt.stream * n + i) * d_out + fc.var], pt.weight, v);
        }
        F[f] = v;
      }
      if (tm.coeff_param >= 0) {   // d loss / d coefficient: seed * scale * product
        float prod = 1.f;
        for (int f = 0; f < tm.n_factors; ++f) prod *= pw(F[f], G->factors[tm.factor_first + f].power);
        atomicAdd(&cred[tm.coeff_param], seed[tm.output] * tm.coeff * prod);
      }
      for (int f = 0; f < tm.n_factors; ++f) {
        const DevFactor& fc = G->factors[tm.factor_first + f];
        float d = dt * dpw(F[f], fc.power);
        for (int g = 0; g < tm.n_factors; ++g)
          if (g != f) d *= pw(F[g], G->factors[tm.factor_first + g].power);
        for (int u = 0; u < fc.n_parts; ++u) {
          const DevPart& pt = G->parts[fc.part_first + u];
          GY[((int64_t)pt.stream * n + i) * d_out + fc.var] += d * pt.weight;
        }
      }
    }
  }
  __syncthreads();
  if (threadIdx.x < n_out) atomicAdd(&slot_sum[G->slot_first + threadIdx.x], red[threadIdx.x]);
  if (do_grad && threadIdx.x < n_coeff) atomicAdd(&cgrad[threadIdx.x], cred[threadIdx.x]);
}

// output layer backward: dL/dH[r][k] = sum_o GY[r][o] W[o][k]
__global__ void plain_output_dx(const DevGroup* __restrict__ G, const float* __restrict__ GY,
                                const float* __restrict__ W, int K, int d_out, float* __restrict__ GH) {
  const int64_t rows = (int64_t)G->n_rows * G->S;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < rows * K;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / K;
    const int k = (int)(e % K);
    float s = 0.f;
    for (int o = 0; o < d_out; ++o) s = fmaf(GY[r * d_out + o], W[o * K + k], s);
    GH[r * K + k] = s;
  }
}

// input layer gradients: dW0[j][a] (value rows: G * x, first-order rows of axis a: G), db0[j]
__global__ void plain_input_bwd(const DevGroup* __restrict__ G, const float* const* __restrict__ arrays,
                                const float* __restrict__ Gz, int d_in, int N, float* __restrict__ dW0,
                                float* __restrict__ db0) {
  const int n = G->n_rows;
  for (int j = blockIdx.x; j < N; j += gridDim.x) {
    float sb = 0.f, sw[TDG_MAX_DIN] = {0.f, 0.f, 0.f, 0.f};
    for (int s = 0; s < G->S; ++s) {
      const int o = G->st_order[s];
      if (o > 1) continue;
      const int q = G->st_site[s];
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const float g = Gz[((int64_t)s * n + i) * N + j];
        if (o == 0) {
          sb += g;
          const float* x = arrays[G->site_points[q]] + (int64_t)i * d_in;
          for (int a = 0; a < d_in; ++a) sw[a] = fmaf(g, x[a] + G->site_off[q][a], sw[a]);
        } else {
          const int ax = G->st_axis[s];
          for (int a = 0; a < d_in; ++a) if (a == ax) sw[a] += g;
        }
      }
    }
    __shared__ float red[(1 + TDG_MAX_DIN) * PT];
    red[threadIdx.x] = sb;
    for (int a = 0; a < TDG_MAX_DIN; ++a) red[(1 + a) * PT + threadIdx.x] = sw[a];
    __syncthreads();
    if (threadIdx.x <= d_in) {
      float t = 0.f;
      for (int k = 0; k < PT; ++k) t += red[threadIdx.x * PT + k];
      if (threadIdx.x == 0) atomicAdd(&db0[j], t);
      else atomicAdd(&dW0[j * d_in + threadIdx.x - 1], t);
    }
    __syncthreads();
  }
}

__global__ void plain_output_dw(const DevGroup* __restrict__ G, const float* __restrict__ GY,
                                const float* __restrict__ H, int K, int d_out,
                                float* __restrict__ dW, float* __restrict__ db) {
  const int64_t rows = (int64_t)G->n_rows * G->S;
  // one block per (o, k); a final block row for the bias
  const int o = blockIdx.y;
  for (int k = blockIdx.x; k <= K; k += gridDim.x) {
    float s = 0.f;
    for (int64_t r = threadIdx.x; r < rows; r += blockDim.x) {
      if (k < K) s = fmaf(GY[r * d_out + o], H[r * K + k], s);
      else if (G->st_order[r / G->n_rows] == 0) s += GY[r * d_out + o];
    }
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    __shared__ float w[PT / 32];
    if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      float t = 0.f;
      for (int i = 0; i < PT / 32; ++i) t += w[i];
      if (k < K) atomicAdd(&dW[o * K + k], t); else atomicAdd(&db[o], t);
    }
    __syncthreads();
  }
}

__global__ void plain_finish_loss(const double* __restrict__ slot_sum, int n_slots,
                                  const int32_t* __restrict__ slot_problem,
                                  const double* __restrict__ w, const double* __restrict__ wn,
                                  int n_problems, double* __restrict__ loss) {
  for (int p = threadIdx.x; p < n_problems; p += blockDim.x) {
    double l = 0.0, ln = 0.0;
    for (int s = 0; s < n_slots; ++s)
      if (slot_problem[s] == p) { l += w[s] * slot_sum[s]; ln += wn[s] * slot_sum[s]; }
    loss[2 * p] = l;
    loss[2 * p + 1] = ln;
  }
}

int grid_for(int64_t work) {
  int64_t b = (work + PT - 1) / PT;
  return (int)(b < 1 ? 1 : (b > 65535 * 8 ? 65535 * 8 : b));
}

}  // namespace

cudaError_t run_plain(const PlainArgs& P, cudaStream_t s) {
  const int L = P.n_layers, d_in = P.width[0], d_out = P.width[L];
  cudaError_t e;
  if ((e = cudaMemsetAsync(P.slot_sum, 0, sizeof(double) * P.n_slots, s)) != cudaSuccess) return e;
  if (P.do_grad && (e = cudaMemsetAsync(P.grad, 0, sizeof(float) * P.n_params * P.n_problems, s)) != cudaSuccess) return e;
  for (int gi = 0; gi < P.n_groups; ++gi) {
    const DevGroup* G = P.groups + gi;
    const HostGroupInfo& hg = P.ginfo[gi];
    const int64_t n = hg.n_rows, rows = n * hg.S;
    const float* prm = P.params + (int64_t)hg.problem * P.n_params;
    float* grad = P.grad + (int64_t)hg.problem * P.n_params;
    // Z_l and H_l of every hidden layer l = 1..L-1 (act + off[l])
    float* Zl[TDG_MAX_LAYERS + 1];
    float* Hl[TDG_MAX_LAYERS + 1];
    int64_t off = 0;
    for (int l = 1; l < L; ++l) {
      Zl[l] = P.act + off; off += rows * P.width[l];
      Hl[l] = P.act + off; off += rows * P.width[l];
    }
    plain_input<<<grid_for(rows * P.width[1]), PT, 0, s>>>(G, P.arrays, prm + P.w_off[0], prm + P.b_off[0], d_in, P.width[1], Zl[1]);
    plain_jet_fwd<<<grid_for(n * P.width[1]), PT, 0, s>>>(G, Zl[1], Hl[1], P.width[1]);
    count_launch(2);
    for (int l = 1; l < L - 1; ++l) {
      const int K = P.width[l], N = P.width[l + 1];
      dim3 grid((unsigned)((rows + 63) / 64), (N + 63) / 64);
      plain_gemm<0><<<grid, 256, 0, s>>>(Hl[l], prm + P.w_off[l], Zl[l + 1], prm + P.b_off[l], G, rows, N, K);
      plain_jet_fwd<<<grid_for(n * N), PT, 0, s>>>(G, Zl[l + 1], Hl[l + 1], N);
      count_launch(2);
    }
    const int KL = P.width[L - 1];
    plain_output<<<grid_for(rows * d_out), PT, 0, s>>>(G, Hl[L - 1], prm + P.w_off[L - 1], prm + P.b_off[L - 1], KL, d_out, P.y);
    if ((e = cudaMemsetAsync(P.gy, 0, sizeof(float) * rows * d_out, s)) != cudaSuccess) return e;
    plain_program<<<grid_for(n), PT, 0, s>>>(G, P.arrays, P.y, P.gy, d_out, P.slot_sum, P.outputs, P.do_grad,
                                             prm + P.coeff_off, grad + P.coeff_off, P.n_coeff);
    count_launch(2);
    if (!P.do_grad) continue;
    // backward
    plain_output_dw<<<dim3(128, d_out), PT, 0, s>>>(G, P.gy, Hl[L - 1], KL, d_out, grad + P.w_off[L - 1], grad + P.b_off[L - 1]);
    plain_output_dx<<<grid_for(rows * KL), PT, 0, s>>>(G, P.gy, prm + P.w_off[L - 1], KL, d_out, P.g0);
    count_launch(2);
    float* gcur = P.g0;
    float* gnext = P.g1;
    for (int l = L - 1; l >= 1; --l) {
      const int N = P.width[l];
      plain_jet_bwd<<<grid_for(n * N), PT, 0, s>>>(G, Zl[l], gcur, N);
      count_launch();
      if (l == 1) {
        plain_input_bwd<<<N, PT, 0, s>>>(G, P.arrays, gcur, d_in, N, grad + P.w_off[0], grad + P.b_off[0]);
        count_launch();
        break;
      }
      const int K = P.width[l - 1];
      const int zsplit = (int)std::min<int64_t>(64, (rows + 4095) / 4096);
      dim3 gdw((K + 63) / 64, (N + 63) / 64, zsplit);
      plain_gemm<2><<<gdw, 256, 0, s>>>(gcur, Hl[l - 1], grad + P.w_off[l - 1], nullptr, G, N, K, rows);
      plain_bias_grad<<<N, PT, 0, s>>>(G, gcur, N, grad + P.b_off[l - 1]);
      dim3 gdx((unsigned)((rows + 63) / 64), (K + 63) / 64);
      plain_gemm<1><<<gdx, 256, 0, s>>>(gcur, prm + P.w_off[l - 1], gnext, nullptr, G, rows, K, N);
      count_launch(3);
      float* t = gcur; gcur = gnext; gnext = t;
    }
  }
  plain_finish_loss<<<1, 256, 0, s>>>(P.slot_sum, P.n_slots, P.slot_problem, P.slot_w, P.slot_wn, P.n_problems, P.loss);
  count_launch();
  return cudaGetLastError();
}

}  // namespace tdg
