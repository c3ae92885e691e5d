// Fused FP32 training-step kernel: one persistent CTA per SM walks a contiguous range of tiles.
// For each tile of (point, stream) rows it runs
//   input layer -> [hidden GEMM -> tanh jet] x (L-2) -> output layer        (forward, Taylor mode)
//   operator program (coefficient x product of derivative factors) -> squared error -> loss slot
//   adjoint of the program -> output layer -> [tanh jet adjoint -> dW, dX GEMMs] ... -> input layer
// The residual of the reference's 'autograd' mode (nested autograd.grad, tedeous/derivative.py:74-132)
// is carried as derivative streams through each layer; its 'NN' mode (tedeous/derivative.py:30-58)
// is carried as value streams at shifted sites. Loss (tedeous/losses.py:84-135) is reduced per CTA
// in FP64; parameter gradients are written to per-CTA segments and reduced by a second kernel, so
// the result is deterministic.
//
// The kernel is a template over the plan's main site class CM: each variant carries the
// compile-time jets of the value-only class and of CM (tdg_jetcode.cuh); every other site runs
// the rule tables. tdg_fp32_inst.cu instantiates one variant per class.
#pragma once
#include "tdg_internal.h"
#include "tdg_jetcode.cuh"

namespace tdg {

namespace {

__device__ __forceinline__ float pow_f(float x, float p) {
  if (p == 1.f) return x;
  if (p == 2.f) return x * x;
  if (p == 0.f) return 1.f;
  if (p == 3.f) return x * x * x;
  return powf(x, p);
}

__device__ __forceinline__ float dpow_f(float x, float p) {  // d/dx x^p
  if (p == 1.f) return 1.f;
  if (p == 2.f) return 2.f * x;
  if (p == 0.f) return 0.f;
  if (p == 3.f) return 3.f * x * x;
  return p * powf(x, p - 1.f);
}

// The three SIMT GEMMs of a tile: 16x16 threads, each with an 8x8 register tile of the 128x128
// output. A column guard around the B loads keeps the compiler from issuing them ahead of the
// FMAs, so every width that is a multiple of 16 runs a guard-free instantiation: JN = columns / 16
// column groups per thread (the accumulators of the other groups are never touched), and KC = 128
// makes the reduction length a compile-time constant for the 128-wide layers. JN = 0 is the
// guarded form for the other widths. Every accumulator sees the same operations in the same order
// in all forms, so the results are bitwise the same.

// Z[r][n] = sum_k H[r][k] W[n][k] (+ b[n] on value streams)
template <int JN, int KC>
__device__ __forceinline__ void fwd_acc(const float* __restrict__ H, const float* __restrict__ W,
                                        float (&acc)[8][8], int R, int N, int K) {
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int KK = KC ? KC : K;
  for (int k = 0; k < KK; k += 4) {
    float4 a[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int r = ty + 16 * i;
      a[i] = r < R ? *reinterpret_cast<const float4*>(&H[r * LDS + k]) : make_float4(0, 0, 0, 0);
    }
#pragma unroll
    for (int j = 0; j < (JN ? JN : 8); ++j) {
      const int n = tx + 16 * j;
      if (JN || n < N) {
        const float4 b = *reinterpret_cast<const float4*>(&W[n * LDS + k]);
#pragma unroll
        for (int i = 0; i < 8; ++i) acc[i][j] = fmaf(a[i].x, b.x, acc[i][j]);
#pragma unroll
        for (int i = 0; i < 8; ++i) acc[i][j] = fmaf(a[i].y, b.y, acc[i][j]);
#pragma unroll
        for (int i = 0; i < 8; ++i) acc[i][j] = fmaf(a[i].z, b.z, acc[i][j]);
#pragma unroll
        for (int i = 0; i < 8; ++i) acc[i][j] = fmaf(a[i].w, b.w, acc[i][j]);
      }
    }
  }
}

__device__ void gemm_fwd(const float* __restrict__ H, const float* __restrict__ W,
                         float* __restrict__ Z, const float* __restrict__ bias,
                         const DevGroup& G, int R, int N, int K) {
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  float acc[8][8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
  if (N == 128 && K == 128) fwd_acc<8, 128>(H, W, acc, R, N, K);
  else if (N == 128) fwd_acc<8, 0>(H, W, acc, R, N, K);
  else if (N == 64) fwd_acc<4, 0>(H, W, acc, R, N, K);
  else if (N == 32) fwd_acc<2, 0>(H, W, acc, R, N, K);
  else fwd_acc<0, 0>(H, W, acc, R, N, K);
  const FastDiv fdT(G.T);
  float bj[8];   // this thread's 8 biases, loaded once
#pragma unroll
  for (int j = 0; j < 8; ++j) bj[j] = tx + 16 * j < N ? __ldg(&bias[tx + 16 * j]) : 0.f;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int r = ty + 16 * i;
    if (r >= R) continue;
    const bool val = G.st_order[fdT.div(r)] == 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int n = tx + 16 * j;
      if (n < N) Z[r * LDS + n] = acc[i][j] + (val ? bj[j] : 0.f);
    }
  }
}

// X[r][k] = sum_n G[r][n] W[n][k] (JN = K / 16 column groups of stride 16, NC the reduction length)
template <int JN, int NC>
__device__ __forceinline__ void dx_acc(const float* __restrict__ Gz, const float* __restrict__ W,
                                       float (&acc)[8][8], int R, int N, int K) {
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int NN = NC ? NC : N;
  for (int n = 0; n < NN; n += 4) {
    float4 a[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int r = ty + 16 * i;
      a[i] = r < R ? *reinterpret_cast<const float4*>(&Gz[r * LDS + n]) : make_float4(0, 0, 0, 0);
    }
#pragma unroll
    for (int j = 0; j < (JN ? JN : 8); ++j) {
      const int k = tx + 16 * j;
      if (JN || k < K) {
        const float b0 = W[n * LDS + k], b1 = W[(n + 1) * LDS + k];
        const float b2 = W[(n + 2) * LDS + k], b3 = W[(n + 3) * LDS + k];
#pragma unroll
        for (int i = 0; i < 8; ++i) acc[i][j] = fmaf(a[i].x, b0, acc[i][j]);
#pragma unroll
        for (int i = 0; i < 8; ++i) acc[i][j] = fmaf(a[i].y, b1, acc[i][j]);
#pragma unroll
        for (int i = 0; i < 8; ++i) acc[i][j] = fmaf(a[i].z, b2, acc[i][j]);
#pragma unroll
        for (int i = 0; i < 8; ++i) acc[i][j] = fmaf(a[i].w, b3, acc[i][j]);
      }
    }
  }
}

// The same for K = 64 HN with 4 contiguous columns per half: thread (ty, tx) owns k = 4 tx +
// 64 h + (0..3), so each row of W is read as 16-byte vectors (HN vectors per n instead of 4 HN
// scalar loads); the accumulators see the same FMAs in the same order.
template <int HN, int NC>
__device__ __forceinline__ void dx_acc4(const float* __restrict__ Gz, const float* __restrict__ W,
                                        float (&acc)[8][8], int R, int N) {
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int NN = NC ? NC : N;
  for (int n = 0; n < NN; n += 4) {
    float4 a[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int r = ty + 16 * i;
      a[i] = r < R ? *reinterpret_cast<const float4*>(&Gz[r * LDS + n]) : make_float4(0, 0, 0, 0);
    }
#pragma unroll
    for (int h = 0; h < HN; ++h) {
      const int k = 4 * tx + 64 * h;
      const float4 b0 = *reinterpret_cast<const float4*>(&W[n * LDS + k]);
      const float4 b1 = *reinterpret_cast<const float4*>(&W[(n + 1) * LDS + k]);
      const float4 b2 = *reinterpret_cast<const float4*>(&W[(n + 2) * LDS + k]);
      const float4 b3 = *reinterpret_cast<const float4*>(&W[(n + 3) * LDS + k]);
      const float bx[4][4] = {{b0.x, b1.x, b2.x, b3.x}, {b0.y, b1.y, b2.y, b3.y},
                              {b0.z, b1.z, b2.z, b3.z}, {b0.w, b1.w, b2.w, b3.w}};
#pragma unroll
      for (int c = 0; c < 4; ++c) {
#pragma unroll
        for (int i = 0; i < 8; ++i) acc[i][4 * h + c] = fmaf(a[i].x, bx[c][0], acc[i][4 * h + c]);
#pragma unroll
        for (int i = 0; i < 8; ++i) acc[i][4 * h + c] = fmaf(a[i].y, bx[c][1], acc[i][4 * h + c]);
#pragma unroll
        for (int i = 0; i < 8; ++i) acc[i][4 * h + c] = fmaf(a[i].z, bx[c][2], acc[i][4 * h + c]);
#pragma unroll
        for (int i = 0; i < 8; ++i) acc[i][4 * h + c] = fmaf(a[i].w, bx[c][3], acc[i][4 * h + c]);
      }
    }
  }
}

__device__ void gemm_dx(const float* __restrict__ Gz, const float* __restrict__ W,
                        float* __restrict__ X, int R, int N, int K) {
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  float acc[8][8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
  if (K == 128 || K == 64) {   // 4 contiguous columns per half
    if (N == 128 && K == 128) dx_acc4<2, 128>(Gz, W, acc, R, N);
    else if (K == 128) dx_acc4<2, 0>(Gz, W, acc, R, N);
    else dx_acc4<1, 0>(Gz, W, acc, R, N);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int r = ty + 16 * i;
      if (r >= R) continue;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int k = 4 * tx + 64 * h;
        if (k < K)
          *reinterpret_cast<float4*>(&X[r * LDS + k]) =
              make_float4(acc[i][4 * h], acc[i][4 * h + 1], acc[i][4 * h + 2], acc[i][4 * h + 3]);
      }
    }
    return;
  }
  if (K == 32) dx_acc<2, 0>(Gz, W, acc, R, N, K);
  else dx_acc<0, 0>(Gz, W, acc, R, N, K);
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int r = ty + 16 * i;
    if (r >= R) continue;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int k = tx + 16 * j;
      if (k < K) X[r * LDS + k] = acc[i][j];
    }
  }
}

// dW[n][k] += sum_r G[r][n] H[r][k] over the tile's rows. Thread (ty, tx) owns n = 4 ty + 64 h
// + (0..3) and k = 4 tx + 64 h' + (0..3) for halves h, h' < HN: HN = 1 when both widths are at
// most 64 (the other three quarters would only multiply zeros). FREE: no bounds on the loads
// (N = K = 64 HN; lanes past a width read rows of the 128-wide buffer that nothing stores).
template <int HN, bool FREE>
__device__ __forceinline__ void dw_acc(const float* __restrict__ Gz, const float* __restrict__ H,
                                       float (&acc)[8][8], int R, int N, int K) {
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
#pragma unroll 4
  for (int r = 0; r < R; ++r) {
    float ga[8], hb[8];
#pragma unroll
    for (int h = 0; h < HN; ++h) {
      const int n = 4 * ty + 64 * h;
      const float4 g4 = FREE || n < N ? *reinterpret_cast<const float4*>(&Gz[r * LDS + n])
                                      : make_float4(0, 0, 0, 0);
      ga[4 * h + 0] = g4.x; ga[4 * h + 1] = g4.y; ga[4 * h + 2] = g4.z; ga[4 * h + 3] = g4.w;
      const int k = 4 * tx + 64 * h;
      const float4 h4 = FREE || k < K ? *reinterpret_cast<const float4*>(&H[r * LDS + k])
                                      : make_float4(0, 0, 0, 0);
      hb[4 * h + 0] = h4.x; hb[4 * h + 1] = h4.y; hb[4 * h + 2] = h4.z; hb[4 * h + 3] = h4.w;
    }
#pragma unroll
    for (int i = 0; i < 4 * HN; ++i)
#pragma unroll
      for (int j = 0; j < 4 * HN; ++j) acc[i][j] = fmaf(ga[i], hb[j], acc[i][j]);
  }
}

// dW[n][k] (+)= sum_r G[r][n] H[r][k]; db[n] (+)= sum over value rows of G[r][n].
__device__ void gemm_dw(const float* __restrict__ Gz, const float* __restrict__ H,
                        float* __restrict__ dW, float* __restrict__ db, const DevGroup& G,
                        int R, int N, int K, bool first) {
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  float acc[8][8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
  if (N == 128 && K == 128) dw_acc<2, true>(Gz, H, acc, R, N, K);
  else if (N == 64 && K == 64) dw_acc<1, true>(Gz, H, acc, R, N, K);
  else if (N <= 64 && K <= 64) dw_acc<1, false>(Gz, H, acc, R, N, K);
  else dw_acc<2, false>(Gz, H, acc, R, N, K);
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int n = 4 * ty + 64 * (i >> 2) + (i & 3);
    if (n >= N) continue;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int k = 4 * tx + 64 * h;
      if (k >= K) continue;
      // the segment's first tile stores, the later ones add without waiting for a load (one
      // thread owns each address, so the adds keep their order)
      float* dst = &dW[(int64_t)n * K + k];
      if (first)
        *reinterpret_cast<float4*>(dst) =
            make_float4(acc[i][4 * h], acc[i][4 * h + 1], acc[i][4 * h + 2], acc[i][4 * h + 3]);
      else
        red_add4(dst, acc[i][4 * h], acc[i][4 * h + 1], acc[i][4 * h + 2], acc[i][4 * h + 3]);
    }
  }
  // bias gradient: one thread per neuron, the value streams' rows in ascending order
  const int T = G.T;
  for (int n = threadIdx.x; n < N; n += NT) {
    float s = 0.f;
    for (int st = 0; st * T < R; ++st)
      if (G.st_order[st] == 0)
        for (int r = st * T; r < st * T + T && r < R; ++r) s += Gz[r * LDS + n];
    if (first) db[n] = s;
    else red_add1(&db[n], s);
  }
}

// In place: Z (pre-activations of every stream) -> H (tanh jet). Streams of a site are processed
// from the highest order down so that lower-order Z values are still intact when read.
// d loss / d theta_k summed over each warp's points into cred[warp][k]. The point's program is
// evaluated again (outputs, seeds, then seed * scale * product per trainable term; scale = the
// term's coefficient in the plan, `gterms`), so the kernel's own program loop stays as it is for
// problems without trainable coefficients. Called by every thread of the CTA.
__device__ __noinline__ void coeff_grad_warps(const DevGroup& G, const DevTerm* __restrict__ gterms,
                                              const float* const* arrays, const float* ybuf, int T,
                                              int nvalid, int row0, int n_coeff, float* cred) {
  const int p = threadIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const bool valid = p < T && p < nvalid;
  const int n_out = G.n_outputs;
  float seed[MAX_OUT];
#pragma unroll
  for (int o = 0; o < MAX_OUT; ++o) seed[o] = 0.f;
  if (valid) {
    float outv[MAX_OUT];
#pragma unroll
    for (int o = 0; o < MAX_OUT; ++o) outv[o] = 0.f;
    for (int t = 0; t < G.n_terms; ++t) {
      const DevTerm& tm = G.terms[t];
      const float c = tm.coeff_array >= 0 ? arrays[tm.coeff_array][row0 + p] : tm.coeff;
      float prod = 1.f;
      for (int f = 0; f < tm.n_factors; ++f) {
        const DevFactor& fc = G.factors[tm.factor_first + f];
        float F = 0.f;
        for (int u = 0; u < fc.n_parts; ++u) {
          const DevPart& pt = G.parts[fc.part_first + u];
          F = fmaf(ybuf[(pt.stream * T + p) * MAX_OUT + fc.var], pt.weight, F);
        }
        prod *= pow_f(F, fc.power);
      }
      outv[tm.output] += c * prod;
    }
    for (int o = 0; o < n_out; ++o) {
      const float tgt = G.target_array >= 0 ? arrays[G.target_array][(int64_t)(row0 + p) * n_out + o] : 0.f;
      const float rw = G.row_weight_array >= 0 ? arrays[G.row_weight_array][row0 + p] : 1.f;
      seed[o] = (outv[o] - tgt) * G.seed_scale[o] * rw;
    }
  }
  for (int k = 0; k < n_coeff; ++k) {
    float v = 0.f;
    if (valid)
      for (int t = 0; t < G.n_terms; ++t) {
        const DevTerm& tm = G.terms[t];
        if (tm.coeff_param != k) continue;
        float prod = 1.f;
        for (int f = 0; f < tm.n_factors; ++f) {
          const DevFactor& fc = G.factors[tm.factor_first + f];
          float F = 0.f;
          for (int u = 0; u < fc.n_parts; ++u) {
            const DevPart& pt = G.parts[fc.part_first + u];
            F = fmaf(ybuf[(pt.stream * T + p) * MAX_OUT + fc.var], pt.weight, F);
          }
          prod *= pow_f(F, fc.power);
        }
        v += seed[tm.output] * gterms[t].coeff * prod;
      }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if (lane == 0) cred[warp * TDG_MAX_COEFF + k] = v;
  }
}

template <int C>
__device__ __forceinline__ void jet_fwd_cls32(float* __restrict__ buf, int T, int base, int p, int n) {
  constexpr int NS = rules_of<C>().ns;
  float4 z[NS];
  sfor<NS>([&](auto mc) {
    constexpr int M = decltype(mc)::value;
    z[M] = ld4(&buf[((base + M) * T + p) * LDS + n]);
  });
  Sig sg;
  sg.make(z[0], rules_of<C>().maxk >= 4);
  sfor<NS>([&](auto mc) {
    constexpr int M = decltype(mc)::value;
    float4 h;
    if constexpr (M == 0) h = sg.t;
    else h = cls_rule_sum<C, M>(sg, z);
    st4(&buf[((base + M) * T + p) * LDS + n], h);
  });
}

template <int CM>
__device__ void jet_forward(float* __restrict__ buf, const DevGroup& G, int N) {
  const int T = G.T, N4 = N >> 2;   // the fused forms' widths are multiples of 4
  const FastDiv fdN4(N4);
  for (int e = threadIdx.x; e < T * N4; e += NT) {
    const int p = fdN4.div(e), n = (e - p * N4) * 4;
    for (int q = 0; q < G.n_sites; ++q) {
      const int ns = G.site_nstreams[q];
      const int base = G.site_streams[q][0];
      if (with_class<CM>(G.site_cls[q], [&](auto cc) {
            jet_fwd_cls32<decltype(cc)::value>(buf, T, base, p, n);
            return true;
          }))
        continue;
      // the rule tables: streams from the highest order down, so that the lower-order Z rows a
      // rule reads are still intact
      float* zb = &buf[(base * T + p) * LDS + n];
      Sig sg;
      sg.make(ld4(zb), false);   // forward rules take tanh derivatives up to the third
      for (int m = ns - 1; m >= 1; --m) {
        const int st = G.site_streams[q][m];
        float4 h = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int u = 0; u < G.st_nrule[st]; ++u) {
          const DevRule& ru = G.rules[st][u];
          float4 v = f4scale(sg.sel(ru.k), (float)ru.mult);
          for (int i = 0; i < ru.k; ++i) v = f4mul(v, ld4(&buf[(ru.sub[i] * T + p) * LDS + n]));
          h = f4add(h, v);
        }
        st4(&buf[(st * T + p) * LDS + n], h);
      }
      st4(zb, sg.t);
    }
  }
}

// jet adjoint of a classed site for (point p, neurons n..n+3): dL/dH rows of gbuf -> dL/dZ rows
// in place. Contributions accumulate in the order of the table pulls: the value stream's own
// term, then streams and rules ascending.
template <int C>
__device__ __forceinline__ void jet_bwd_cls32(const float* __restrict__ zbuf, float* __restrict__ gbuf,
                                              int T, int base, int p, int n) {
  constexpr int NS = rules_of<C>().ns;
  float4 z[NS], g[NS], gz[NS];
  sfor<NS>([&](auto mc) {
    constexpr int M = decltype(mc)::value;
    z[M] = ld4(&zbuf[((base + M) * T + p) * LDS + n]);
    g[M] = ld4(&gbuf[((base + M) * T + p) * LDS + n]);
    gz[M] = make_float4(0.f, 0.f, 0.f, 0.f);
  });
  Sig sg;
  sg.make(z[0], rules_of<C>().maxk + 1 >= 4);
  gz[0] = f4mul(g[0], sg.s1);
  sfor<NS>([&](auto mc) {
    constexpr int M = decltype(mc)::value;
    if constexpr (M >= 1) {
      sfor<rules_of<C>().nrule[M]>([&](auto uc) {
        constexpr int U = decltype(uc)::value;
        constexpr int K = rules_of<C>().k[M][U];
        constexpr float MU = (float)rules_of<C>().mult[M][U];
        float4 v = f4mul(g[M], f4scale(sg.sel(K + 1), MU));
        sfor<K>([&](auto fc) { v = f4mul(v, z[rules_of<C>().sub[M][U][decltype(fc)::value]]); });
        gz[0] = f4add(gz[0], v);
        sfor<K>([&](auto ic) {
          constexpr int I = decltype(ic)::value;
          float4 w = f4mul(g[M], f4scale(sg.sel(K), MU));
          sfor<K>([&](auto jc) {
            constexpr int J = decltype(jc)::value;
            if constexpr (J != I) w = f4mul(w, z[rules_of<C>().sub[M][U][J]]);
          });
          constexpr int SI = rules_of<C>().sub[M][U][I];
          gz[SI] = f4add(gz[SI], w);
        });
      });
    }
  });
  sfor<NS>([&](auto mc) {
    constexpr int M = decltype(mc)::value;
    st4(&gbuf[((base + M) * T + p) * LDS + n], gz[M]);
  });
}

// In place: gbuf holds dL/dH of every stream, zbuf the pre-activations; gbuf becomes dL/dZ.
// Table-driven sites process their streams from the value stream up (see DevPull).
template <int CM>
__device__ void jet_backward(const float* __restrict__ zbuf, float* __restrict__ gbuf,
                             const DevGroup& G, int N) {
  const int T = G.T, N4 = N >> 2;
  const FastDiv fdN4(N4);
  for (int e = threadIdx.x; e < T * N4; e += NT) {
    const int p = fdN4.div(e), n = (e - p * N4) * 4;
    for (int q = 0; q < G.n_sites; ++q) {
      const int ns = G.site_nstreams[q];
      const int base = G.site_streams[q][0];
      if (with_class<CM>(G.site_cls[q], [&](auto cc) {
            jet_bwd_cls32<decltype(cc)::value>(zbuf, gbuf, T, base, p, n);
            return true;
          }))
        continue;
      Sig sg;
      sg.make(ld4(&zbuf[(base * T + p) * LDS + n]), ns > 1);
      if (ns == 1) {
        float* g = &gbuf[(base * T + p) * LDS + n];
        st4(g, f4mul(ld4(g), sg.s1));
        continue;
      }
      for (int m = 0; m < ns; ++m) {
        const int b = G.site_streams[q][m];
        float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
        const int pf = G.st_pull_first[b];
        for (int u = 0; u < G.st_npull[b]; ++u) {
          const DevPull& pl = G.pulls[pf + u];
          float4 v = f4mul(ld4(&gbuf[(pl.alpha * T + p) * LDS + n]), f4scale(sg.sel(pl.kk), (float)pl.mult));
          for (int i = 0; i < pl.n_oth; ++i) v = f4mul(v, ld4(&zbuf[(pl.oth[i] * T + p) * LDS + n]));
          acc = f4add(acc, v);
        }
        st4(&gbuf[(b * T + p) * LDS + n], acc);
      }
    }
  }
}

// 16-byte asynchronous copies global -> shared (cp.async, L2 only): a stage is issued ahead and
// lands while other work runs; cp.async.wait_group then the next barrier make it visible.
__device__ __forceinline__ void cp_async16(float* smem, const float* gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;"
               :: "r"((uint32_t)__cvta_generic_to_shared(smem)), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int PENDING>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" :: "n"(PENDING) : "memory");
}

// Stage W [N x K] into shared memory, asynchronously when W is 16-byte aligned; the weights of
// problem p start at p * n_params floats, which is not a multiple of 4 for odd parameter counts,
// so misaligned layers are read element by element (synchronously). Commits one copy group.
__device__ void load_weights(float* __restrict__ wbuf, const float* __restrict__ W, int N, int K) {
  if ((reinterpret_cast<uintptr_t>(W) & 15) == 0) {
    const int K4 = K >> 2;
    const FastDiv fdK4(K4);
    for (int e = threadIdx.x; e < N * K4; e += NT) {
      const int n = fdK4.div(e), k = (e - n * K4) * 4;
      cp_async16(&wbuf[n * LDS + k], &W[(int64_t)n * K + k]);
    }
  } else {
    const FastDiv fdK(K);
    for (int e = threadIdx.x; e < N * K; e += NT) {
      const int n = fdK.div(e), k = e - n * K;
      wbuf[n * LDS + k] = __ldg(&W[(int64_t)n * K + k]);
    }
  }
  cp_async_commit();
}

// rows [R x K] of a saved layer (global scratch, row stride LDS) into shared memory,
// asynchronously; commits one copy group
__device__ void fetch_rows(float* __restrict__ dst, const float* __restrict__ src, int R, int K) {
  const int K4 = K >> 2;
  const FastDiv fdK4(K4);
  for (int e = threadIdx.x; e < R * K4; e += NT) {
    const int r = fdK4.div(e), k = (e - r * K4) * 4;
    cp_async16(&dst[r * LDS + k], &src[r * LDS + k]);
  }
  cp_async_commit();
}

// rows [R x K] of shared memory into the global scratch (row stride LDS)
__device__ void copy_rows(float* __restrict__ dst, const float* __restrict__ src, int R, int K) {
  const int K4 = K >> 2;
  const FastDiv fdK4(K4);
  for (int e = threadIdx.x; e < R * K4; e += NT) {
    const int r = fdK4.div(e), k = (e - r * K4) * 4;
    *reinterpret_cast<float4*>(&dst[r * LDS + k]) = *reinterpret_cast<const float4*>(&src[r * LDS + k]);
  }
}

}  // namespace

template <int CM>
__global__ void __launch_bounds__(NT, 1) fused_fp32_kernel(FusedArgs A) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* bufA = reinterpret_cast<float*>(smem_raw);
  float* bufB = bufA + RMAX * LDS;
  float* wbuf = bufB + RMAX * LDS;
  float* ybuf = wbuf + RMAX * LDS;                  // [RMAX][MAX_OUT]
  float* gybuf = ybuf + RMAX * MAX_OUT;             // [RMAX][MAX_OUT]
  float* xsbuf = gybuf + RMAX * MAX_OUT;            // [RMAX][TDG_MAX_DIN]
  DevGroup* Gs = reinterpret_cast<DevGroup*>(xsbuf + RMAX * TDG_MAX_DIN);
  double* slot_acc = reinterpret_cast<double*>(
      (reinterpret_cast<uintptr_t>(Gs + 1) + 15) & ~uintptr_t(15));
  double* wred = slot_acc + MAX_SLOTS;             // [NT/32][MAX_OUT]
  float* cred = reinterpret_cast<float*>(wred + NT / 32 * MAX_OUT);   // [NT/32][TDG_MAX_COEFF]

  const int tid = threadIdx.x;
  const int cta = blockIdx.x;
  const int L = A.n_layers;
  const int d_in = A.width[0], d_out = A.width[L];
  for (int s = tid; s < A.n_slots; s += NT) slot_acc[s] = 0.0;
  int cur_group = -1;
  float* scr = A.scratch + (int64_t)cta * (L - 1) * RMAX * LDS;

  for (int ti = A.cta_tile_begin[cta]; ti < A.cta_tile_begin[cta + 1]; ++ti) {
    const DevTile tile = A.tiles[ti];
    __syncthreads();
    if (tile.group != cur_group) {
      const int4* src = reinterpret_cast<const int4*>(&A.groups[tile.group]);
      int4* dst = reinterpret_cast<int4*>(Gs);
      for (int e = tid; e < (int)(sizeof(DevGroup) / 16); e += NT) dst[e] = src[e];
      cur_group = tile.group;
      __syncthreads();
      if (A.n_coeff > 0) {   // trainable coefficients: the shared copy carries scale * theta
        const float* theta = A.params + (int64_t)Gs->problem * A.n_params + A.coeff_off;
        for (int t = tid; t < Gs->n_terms; t += NT)
          if (Gs->terms[t].coeff_param >= 0)
            Gs->terms[t].coeff = A.groups[tile.group].terms[t].coeff * theta[Gs->terms[t].coeff_param];
        __syncthreads();
      }
    }
    const DevGroup& G = *Gs;
    const int T = G.T, S = G.S, R = T * S;
    const FastDiv fdT(T);
    const int nvalid = tile.nvalid, row0 = tile.row0;
    const float* prm = A.params + (int64_t)G.problem * A.n_params;
    // the first hidden GEMM's weights land during the coordinates, the input layer and its jets
    // (the weight buffer's last reader, the previous tile's last GEMM, ended at a barrier)
    if (L > 2) load_weights(wbuf, prm + A.w_off[1], A.width[2], A.width[1]);

    // ---- coordinates of every row (site point + FP32 offset), zero for padding points
    for (int e = tid; e < R * d_in; e += NT) {
      const int r = e / d_in, a = e - r * d_in;
      const int s = fdT.div(r), p = r - s * T;
      const int q = G.st_site[s];
      float x = 0.f;
      if (p < nvalid) x = A.arrays[G.site_points[q]][(int64_t)(row0 + p) * d_in + a] + G.site_off[q][a];
      xsbuf[r * TDG_MAX_DIN + a] = x;
    }
    __syncthreads();

    // ---- input layer: value streams W x + b; first-order streams W[:, axis]; higher orders 0
    {
      const int N = A.width[1];
      const float* W0 = prm + A.w_off[0];
      const float* b0 = prm + A.b_off[0];
      const FastDiv fdN(N);
      for (int e = tid; e < R * N; e += NT) {
        const int r = fdN.div(e), n = e - r * N;
        const int s = fdT.div(r);
        const int o = G.st_order[s];
        float z;
        if (o == 0) {
          z = 0.f;
          for (int a = 0; a < d_in; ++a) z = fmaf(__ldg(&W0[n * d_in + a]), xsbuf[r * TDG_MAX_DIN + a], z);
          z += __ldg(&b0[n]);
        } else if (o == 1) {
          z = __ldg(&W0[n * d_in + G.st_axis[s]]);
        } else {
          z = 0.f;
        }
        bufA[r * LDS + n] = z;
      }
    }
    __syncthreads();
    if (A.do_grad) copy_rows(scr, bufA, R, A.width[1]);
    jet_forward<CM>(bufA, G, A.width[1]);
    __syncthreads();

    float* hin = bufA;
    float* hout = bufB;
    // ---- hidden layers
    for (int l = 1; l < L - 1; ++l) {
      const int K = A.width[l], N = A.width[l + 1];
      cp_async_wait<0>();   // W_l, issued after the previous GEMM
      __syncthreads();
      gemm_fwd(hin, wbuf, hout, prm + A.b_off[l], G, R, N, K);
      __syncthreads();
      if (l + 1 < L - 1)    // the next layer's weights land during this layer's jets
        load_weights(wbuf, prm + A.w_off[l + 1], A.width[l + 2], N);
      if (A.do_grad) copy_rows(scr + (int64_t)l * RMAX * LDS, hout, R, N);
      jet_forward<CM>(hout, G, N);
      __syncthreads();
      float* t = hin; hin = hout; hout = t;
    }

    // ---- output layer
    {
      const int K = A.width[L - 1];
      const float* Wl = prm + A.w_off[L - 1];
      const float* bl = prm + A.b_off[L - 1];
      for (int e = tid; e < R * d_out; e += NT) {
        const int r = e / d_out, o = e - r * d_out;
        float z = 0.f;
        const float* h = &hin[r * LDS];
        const float* w = &Wl[(int64_t)o * K];
        for (int k = 0; k < K; k += 4) {
          const float4 hv = *reinterpret_cast<const float4*>(&h[k]);
          z = fmaf(hv.x, __ldg(&w[k]), z);
          z = fmaf(hv.y, __ldg(&w[k + 1]), z);
          z = fmaf(hv.z, __ldg(&w[k + 2]), z);
          z = fmaf(hv.w, __ldg(&w[k + 3]), z);
        }
        if (G.st_order[fdT.div(r)] == 0) z += __ldg(&bl[o]);
        ybuf[r * MAX_OUT + o] = z;
        gybuf[r * MAX_OUT + o] = 0.f;
      }
    }
    __syncthreads();

    // ---- operator program, squared error, loss seeds and program adjoint (one thread per point)
    const int n_out = G.n_outputs;
    float err2[MAX_OUT];
#pragma unroll
    for (int o = 0; o < MAX_OUT; ++o) err2[o] = 0.f;
    if (tid < T) {
      const int p = tid;
      const bool valid = p < nvalid;
      float outv[MAX_OUT];
#pragma unroll
      for (int o = 0; o < MAX_OUT; ++o) outv[o] = 0.f;
      for (int t = 0; t < G.n_terms; ++t) {
        const DevTerm& tm = G.terms[t];
        const float c = tm.coeff_array >= 0 && valid ? A.arrays[tm.coeff_array][row0 + p] : tm.coeff;
        float prod = 1.f;
        for (int f = 0; f < tm.n_factors; ++f) {
          const DevFactor& fc = G.factors[tm.factor_first + f];
          float F = 0.f;
          for (int u = 0; u < fc.n_parts; ++u) {
            const DevPart& pt = G.parts[fc.part_first + u];
            F = fmaf(ybuf[(pt.stream * T + p) * MAX_OUT + fc.var], pt.weight, F);
          }
          prod *= pow_f(F, fc.power);
        }
        const float add = c * prod;
#pragma unroll
        for (int o = 0; o < MAX_OUT; ++o)   // register arrays: constant indices, unconditional
          outv[o] += tm.output == o ? add : 0.f;   // stores (outv is never -0, so + 0 is exact)
      }
      float seed[MAX_OUT];
#pragma unroll
      for (int o = 0; o < MAX_OUT; ++o) seed[o] = 0.f;
#pragma unroll
      for (int o = 0; o < MAX_OUT; ++o) {
        float e = 0.f, rw = 1.f, sc = 0.f;   // outputs past n_out keep zeros
        if (o < n_out) {
          const float tgt = (G.target_array >= 0 && valid)
                                ? A.arrays[G.target_array][(int64_t)(row0 + p) * n_out + o] : 0.f;
          e = valid ? outv[o] - tgt : 0.f;
          rw = (G.row_weight_array >= 0 && valid) ? A.arrays[G.row_weight_array][row0 + p] : 1.f;
          sc = G.seed_scale[o];
          if (A.outputs && G.out_offset >= 0 && valid)
            A.outputs[G.out_offset + (int64_t)(row0 + p) * n_out + o] = outv[o];
        }
        err2[o] = e * e * rw;
        seed[o] = e * sc * rw;   // dL/d(out) = 2 * weight * row weight * (out - target)
      }
      if (A.do_grad) {
        for (int t = 0; t < G.n_terms; ++t) {
          const DevTerm& tm = G.terms[t];
          const float c = tm.coeff_array >= 0 && valid ? A.arrays[tm.coeff_array][row0 + p] : tm.coeff;
          float so = 0.f;
#pragma unroll
          for (int o = 0; o < MAX_OUT; ++o) so = tm.output == o ? seed[o] : so;
          const float dt = so * c;
          if (dt == 0.f) continue;
          // the factors and their powers, each evaluated once (the same values the product
          // rule below multiplies)
          const int nf = tm.n_factors;
          float F[MAX_TERM_FACTORS], PW[MAX_TERM_FACTORS];
#pragma unroll
          for (int f = 0; f < MAX_TERM_FACTORS; ++f) {
            float v = 0.f, pw = 1.f;
            if (f < nf) {
              const DevFactor& fc = G.factors[tm.factor_first + f];
              for (int u = 0; u < fc.n_parts; ++u) {
                const DevPart& pt = G.parts[fc.part_first + u];
                v = fmaf(ybuf[(pt.stream * T + p) * MAX_OUT + fc.var], pt.weight, v);
              }
              pw = pow_f(v, fc.power);
            }
            F[f] = v;
            PW[f] = pw;
          }
#pragma unroll
          for (int f = 0; f < MAX_TERM_FACTORS; ++f) {
            if (f >= nf) continue;
            const DevFactor& fc = G.factors[tm.factor_first + f];
            float d = dt * dpow_f(F[f], fc.power);
#pragma unroll
            for (int g = 0; g < MAX_TERM_FACTORS; ++g)
              if (g < nf && g != f) d *= PW[g];   // (a multiplication by 1 would not change d)
            for (int u = 0; u < fc.n_parts; ++u) {
              const DevPart& pt = G.parts[fc.part_first + u];
              gybuf[(pt.stream * T + p) * MAX_OUT + fc.var] += d * pt.weight;
            }
          }
        }
      }
    }
    // deterministic FP64 reduction of squared errors: warp shuffle, then warps in order
    {
      const int lane = tid & 31, warp = tid >> 5;
#pragma unroll
      for (int o = 0; o < MAX_OUT; ++o) {
        if (o >= n_out) continue;
        double v = (double)err2[o];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
        if (lane == 0) wred[warp * MAX_OUT + o] = v;
      }
      __syncthreads();
      if (tid < n_out) {
        double s = 0.0;
        for (int w = 0; w < NT / 32; ++w) s += wred[w * MAX_OUT + tid];
        slot_acc[G.slot_first + tid] += s;
      }
      if (A.do_grad && A.n_coeff > 0)   // coefficient gradients per warp; warps in order below
        coeff_grad_warps(G, A.groups[tile.group].terms, A.arrays, ybuf, T, nvalid, row0, A.n_coeff, cred);
    }
    if (!A.do_grad) continue;
    __syncthreads();

    // ---- backward: gybuf holds dL/dY of every (point, stream) row
    float* grad = A.partial + (int64_t)tile.seg * A.part_stride;
    const bool first = tile.first_in_seg != 0;
    if (tid < A.n_coeff) {   // every coefficient slot of the segment, written on its first tile
      float s = 0.f;
      for (int w = 0; w < NT / 32; ++w) s += cred[w * TDG_MAX_COEFF + tid];
      float* dst = grad + A.coeff_off + tid;
      if (first) *dst = s;
      else red_add1(dst, s);
    }
    // output layer: dW, db, and dL/dH of the last hidden layer into hout
    {
      const int K = A.width[L - 1];
      const float* Wl = prm + A.w_off[L - 1];
      float* dW = grad + A.w_off[L - 1];
      float* db = grad + A.b_off[L - 1];
      const FastDiv fdK(K);
      for (int e = tid; e < d_out * K; e += NT) {
        const int o = fdK.div(e), k = e - o * K;
        float s = 0.f;
        for (int r = 0; r < R; ++r) s = fmaf(gybuf[r * MAX_OUT + o], hin[r * LDS + k], s);
        if (first) dW[(int64_t)o * K + k] = s;
        else red_add1(&dW[(int64_t)o * K + k], s);
      }
      for (int o = tid; o < d_out; o += NT) {
        float s = 0.f;
        for (int st = 0; st < S; ++st)   // the value streams' rows in ascending order
          if (G.st_order[st] == 0)
            for (int r = st * T; r < st * T + T; ++r) s += gybuf[r * MAX_OUT + o];
        if (first) db[o] = s;
        else red_add1(&db[o], s);
      }
      for (int e = tid; e < R * K; e += NT) {
        const int r = fdK.div(e), k = e - r * K;
        float s = 0.f;
        for (int o = 0; o < d_out; ++o) s = fmaf(gybuf[r * MAX_OUT + o], __ldg(&Wl[(int64_t)o * K + k]), s);
        hout[r * LDS + k] = s;
      }
    }
    __syncthreads();
    float* gcur = hout;   // dL/dH_l
    float* other = hin;
    for (int l = L - 1; l >= 1; --l) {
      // layer l: H_l = jet(Z_l), Z_l = Linear_{l-1}(H_{l-1}); width[l] neurons
      const int N = A.width[l];
      fetch_rows(other, scr + (int64_t)(l - 1) * RMAX * LDS, R, N);
      if (l >= 2) {   // W_{l-1} lands during the jet adjoint (the weight buffer is free)
        load_weights(wbuf, prm + A.w_off[l - 1], N, A.width[l - 1]);
        cp_async_wait<1>();   // Z_l
      } else {
        cp_async_wait<0>();
      }
      __syncthreads();
      jet_backward<CM>(other, gcur, G, N);   // gcur: dL/dZ_l
      __syncthreads();
      if (l >= 2) {
        const int K = A.width[l - 1];
        fetch_rows(other, scr + (int64_t)(l - 2) * RMAX * LDS, R, K);
        cp_async_wait<0>();   // Z_{l-1} and W_{l-1}
        __syncthreads();
        jet_forward<CM>(other, G, K);          // other: H_{l-1}
        __syncthreads();
        gemm_dw(gcur, other, grad + A.w_off[l - 1], grad + A.b_off[l - 1], G, R, N, K, first);
        __syncthreads();
        gemm_dx(gcur, wbuf, other, R, N, K);   // other: dL/dH_{l-1}
        __syncthreads();
        float* t = gcur; gcur = other; other = t;
      } else {
        // input layer gradients
        float* dW0 = grad + A.w_off[0];
        float* db0 = grad + A.b_off[0];
        for (int n = tid; n < N; n += NT) {
          float sb = 0.f;
          float sw[TDG_MAX_DIN] = {0.f, 0.f, 0.f, 0.f};
          // branch-free and unrolled, so that the rows' loads overlap: a value row adds g to the
          // bias and g x_a to column a, a first-derivative row along a adds g to column a (adding
          // zero elsewhere leaves every sum as the per-kind branches would)
#pragma unroll 4
          for (int r = 0; r < R; ++r) {
            const int s = fdT.div(r);
            const int o = G.st_order[s];
            const int ax = o == 1 ? G.st_axis[s] : -1;
            const float g = gcur[r * LDS + n];
            const float gv = o == 0 ? g : 0.f;
            const float4 xv = *reinterpret_cast<const float4*>(&xsbuf[r * TDG_MAX_DIN]);
            const float xa[TDG_MAX_DIN] = {xv.x, xv.y, xv.z, xv.w};
            sb += gv;
#pragma unroll
            for (int a = 0; a < TDG_MAX_DIN; ++a)
              if (a < d_in) sw[a] = fmaf(gv, xa[a], sw[a]) + (a == ax ? g : 0.f);
          }
#pragma unroll
          for (int a = 0; a < TDG_MAX_DIN; ++a)
            if (a < d_in) {
              if (first) dW0[n * d_in + a] = sw[a];
              else red_add1(&dW0[n * d_in + a], sw[a]);
            }
          if (first) db0[n] = sb;
          else red_add1(&db0[n], sb);
        }
      }
    }
  }
  __syncthreads();
  for (int s = tid; s < A.n_slots; s += NT) A.slot_partial[(int64_t)cta * A.n_slots + s] = slot_acc[s];
}

template <int CM>
cudaError_t launch_fp32_variant(const FusedArgs& a, int n_ctas, cudaStream_t s) {
  static bool attr_set = false;
  const size_t smem = fused_smem_bytes();
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(fused_fp32_kernel<CM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  fused_fp32_kernel<CM><<<n_ctas, NT, smem, s>>>(a);
  count_launch();
  return cudaGetLastError();
}

}  // namespace tdg
