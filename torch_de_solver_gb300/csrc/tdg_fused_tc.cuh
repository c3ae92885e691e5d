// Tensor-core fused training-step kernel (sm_103a, tcgen05 + TMEM + bulk copies), as templates.
// Each (precision, main site class) variant is instantiated in its own object, compiled from
// tdg_tc_inst.cu with the variant's -D flags, so that all of them compile in parallel.
//
// Same computation as fused_fp32_kernel (tdg_fused_fp32.cuh): one persistent CTA per SM walks tiles of
// 128 (stream, point) rows through the tanh-jet forward, the operator program and loss, and the
// hand-written adjoint. Every hidden-layer GEMM runs on the tensor cores:
//   forward  Z_{j+1}[rows x N]  = H_j[rows x K] . W_j^T          (A = H, B = W packed K-major)
//   dX       G_H_{l-1}          = G_Z_l . W_{l-1}                 (A = G_Z, B = W^T packed K-major)
//   dW       dW_{l-1}[N x K]    = G_Z_l^T . H_{l-1}               (A = G_Z^T, B = H^T, K = rows)
// with FP32 accumulators in tensor memory (D1: 128 columns, D2: 128 columns). Operands are TF32
// (kind::tf32, rounded with cvt.rna) or BF16 (kind::f16). One thread issues the MMAs and commits
// them to an mbarrier; packed weights and the saved pre-activations are staged into shared memory
// with cp.async.bulk. All mbarrier waits are bounded and report a timeout in a device flag.
// The input layer (d_in <= 4), the output layer (d_out <= 8), the tanh jets and the operator
// program stay on the CUDA cores.
#pragma once
#include <utility>
#include "tdg_internal.h"
#include "tdg_jetcls.h"
#include "tdg_jetcode.cuh"
#include "tdg_tc.cuh"

namespace tdg {

namespace {

using namespace tc;

constexpr int OPB = 128 * 128 * 4;    // bytes of one operand buffer
constexpr int NTC = 512;              // threads of the tensor-core kernel (a multiple of 128)
constexpr int NCG = NTC / 128;        // TMEM column groups: warps sharing one lane quarter
constexpr int NPART = NTC / 128;      // row parts of the per-neuron reductions (128 threads each)
// the small parameters of the current problem, staged in shared memory when the problem changes:
// hidden biases (128 per hidden Linear), W0 and b0 of the input layer, W and b of the output layer
constexpr int PB_HB = 0;
constexpr int PB_W0 = PB_HB + (TDG_MAX_LAYERS - 2) * TDG_MAX_WIDTH;
constexpr int PB_B0 = PB_W0 + TDG_MAX_WIDTH * TDG_MAX_DIN;
constexpr int PB_WL = PB_B0 + TDG_MAX_WIDTH;
constexpr int PB_BL = PB_WL + TDG_MAX_DOUT * TDG_MAX_WIDTH;
constexpr int PB_CF = PB_BL + TDG_MAX_DOUT;                     // trainable coefficients
constexpr int PBUF = PB_CF + TDG_MAX_COEFF;

__device__ __forceinline__ int p16(int w) { return (w + 15) & ~15; }

__device__ __forceinline__ float powf_(float x, float p) {
  if (p == 1.f) return x;
  if (p == 2.f) return x * x;
  if (p == 0.f) return 1.f;
  if (p == 3.f) return x * x * x;
  return powf(x, p);
}

__device__ __forceinline__ float dpowf_(float x, float p) {
  if (p == 1.f) return 1.f;
  if (p == 2.f) return 2.f * x;
  if (p == 0.f) return 0.f;
  if (p == 3.f) return 3.f * x * x;
  return p * powf(x, p - 1.f);
}

// d loss / d theta_k of one tile: per (point, trainable term) seed * scale * product of the factors
// (scale = the term's own coefficient in the plan, `gterms`), into the dead term-value rows `tv`,
// then one thread per coefficient sums its terms and points in a fixed order and adds the sum to
// the tile's gradient segment. Out of line: the kernels without trainable coefficients keep their
// term loops unchanged. Called by every thread of the CTA.
__device__ __noinline__ void coeff_grad_tile(const DevGroup& G, const DevTerm* __restrict__ gterms,
                                             const float* ybuf, const float* seedv, float* tv, int T,
                                             float* cgrad, int n_coeff) {
  const int nt = G.n_terms;
  for (int e = threadIdx.x; e < T * nt; e += blockDim.x) {
    const int p = e % T, t = e / T;
    const DevTerm& tm = G.terms[t];
    if (tm.coeff_param < 0) continue;
    float prod = 1.f;
    for (int f = 0; f < tm.n_factors; ++f) {
      const DevFactor& fc = G.factors[tm.factor_first + f];
      float v = 0.f;
      for (int u = 0; u < fc.n_parts; ++u) {
        const DevPart& pt = G.parts[fc.part_first + u];
        v = fmaf(ybuf[(pt.stream * T + p) * MAX_OUT + fc.var], pt.weight, v);
      }
      prod *= powf_(v, fc.power);
    }
    tv[t * RMAX + p] = seedv[tm.output * RMAX + p] * gterms[t].coeff * prod;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < n_coeff; k += blockDim.x) {
    float sum = 0.f;
    bool used = false;
    for (int t = 0; t < nt; ++t)
      if (G.terms[t].coeff_param == k) {
        used = true;
        for (int p = 0; p < T; ++p) sum += tv[t * RMAX + p];
      }
    if (used) red_add1(&cgrad[k], sum);
  }
}

__device__ __forceinline__ float4 ld4o(const unsigned char* b, uint32_t off) {
  return *reinterpret_cast<const float4*>(b + off);
}

// write 4 consecutive K elements of row i (kp elements per row) into an operand buffer
template <bool BF16>
__device__ __forceinline__ void put4(unsigned char* buf, int i, int k, int kp, float4 v) {
  if (BF16) {
    const uint32_t off = ofs(i, k, kp, 2);
    __nv_bfloat162 a = __floats2bfloat162_rn(v.x, v.y), b = __floats2bfloat162_rn(v.z, v.w);
    uint2 u;
    u.x = *reinterpret_cast<uint32_t*>(&a);
    u.y = *reinterpret_cast<uint32_t*>(&b);
    *reinterpret_cast<uint2*>(buf + off) = u;
  } else {
    const uint32_t off = ofs(i, k, kp, 4);
    *reinterpret_cast<float4*>(buf + off) =
        make_float4(to_tf32(v.x), to_tf32(v.y), to_tf32(v.z), to_tf32(v.w));
  }
}

// bulk copies go through two slots, each an mbarrier with its own phase: slot B (the B operand
// buffer opB; issue / load / ensure / wait_tma) and slot A (the other buffer opA, which holds B
// operands too when the A operands live in tensor memory; issue_a / ensure_a / wait_a)
struct TcCtx {
  uint64_t* bar_mma;
  uint64_t* bar_tma;
  uint64_t* bar_tma_a;
  uint32_t ph_mma, ph_tma, ph_tma_a;
  int* err;
  __device__ __forceinline__ void wait_mma() {
    if (!mbar_wait(bar_mma, ph_mma) && threadIdx.x == 0) atomicExch(err, 1);
    ph_mma ^= 1;
    fence_after();
  }
  bool inflight;     // slot B: a bulk copy issued and not yet waited for
  bool inflight_a;   // slot A
  __device__ __forceinline__ void wait_tma() {
    if (!mbar_wait(bar_tma, ph_tma) && threadIdx.x == 0) atomicExch(err, 2);
    ph_tma ^= 1;
    inflight = false;
  }
  __device__ __forceinline__ void wait_a() {
    if (!mbar_wait(bar_tma_a, ph_tma_a) && threadIdx.x == 0) atomicExch(err, 3);
    ph_tma_a ^= 1;
    inflight_a = false;
  }
  __device__ __forceinline__ void issue_a(void* dst, const void* src, uint32_t bytes) {
    if (threadIdx.x == 0) {
      mbar_expect_tx(bar_tma_a, bytes);
      bulk_g2s(dst, src, bytes, bar_tma_a);
    }
    inflight_a = true;
  }
  __device__ __forceinline__ void ensure_a(void* dst, const void* src, uint32_t bytes) {
    if (!inflight_a) issue_a(dst, src, bytes);
    wait_a();
  }
  // no copy left in flight (before the CTA exits)
  __device__ __forceinline__ void drain() {
    if (inflight) wait_tma();
    if (inflight_a) wait_a();
  }
  // every thread: generic-proxy shared-memory accesses ordered before the async proxy's (MMA
  // operand reads, bulk copies into shared memory), then barrier
  __device__ __forceinline__ void publish() {
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
  }
  // as publish, for global memory too: the saved pre-activations (generic stores) before the
  // bulk copies that read them back
  __device__ __forceinline__ void publish_global() {
    fence_async_all();
    fence_before();
    __syncthreads();
    fence_after();
  }
  // start a bulk copy into shared memory; at most one is in flight
  __device__ __forceinline__ void issue(void* dst, const void* src, uint32_t bytes) {
    if (threadIdx.x == 0) {
      mbar_expect_tx(bar_tma, bytes);
      bulk_g2s(dst, src, bytes, bar_tma);
    }
    inflight = true;
  }
  __device__ __forceinline__ void load(void* dst, const void* src, uint32_t bytes) {
    issue(dst, src, bytes);
    wait_tma();
  }
  // the copy issued ahead of time for this use (issued here when none is in flight), completed
  __device__ __forceinline__ void ensure(void* dst, const void* src, uint32_t bytes) {
    if (!inflight) issue(dst, src, bytes);
    wait_tma();
  }
};

// D[128 x n] = A[128 x k] . B[n x k]^T, issued by thread 0 and committed to bar_mma
template <bool BF16>
__device__ __forceinline__ void gemm_issue(uint32_t d, const unsigned char* a, const unsigned char* b,
                                           int n, int k, uint64_t* bar) {
  if (threadIdx.x != 0) return;
  constexpr int es = BF16 ? 2 : 4, epc = 16 / es, mk = BF16 ? 16 : 8;
  const uint32_t sbo = (uint32_t)(k / epc) * 128;
  const uint32_t idesc = instr_desc<BF16>(128, n);
  const uint32_t a0 = smem_u32(a), b0 = smem_u32(b);
  for (int j = 0; j < k / mk; ++j)
    mma<BF16>(d, smem_desc(a0 + j * 256, 128, sbo), smem_desc(b0 + j * 256, 128, sbo), idesc, j > 0);
  commit(bar);
}

// ---- jet code of the compile-time site classes: the helpers are in tdg_jetcode.cuh

// f(T) with the points per tile T a compile-time constant when the group is a single site of
// class C (then T = 128 / streams); for the value-only class also f(runtime T) for other groups.
// False when neither applies (the table-driven code runs).
template <int C, typename F>
__device__ __forceinline__ bool with_tile_points(const DevGroup& G, F&& f) {
  constexpr int TC = RMAX / rules_of<C>().ns;
  if (G.n_sites == 1 && G.T == TC) {
    f(std::integral_constant<int, TC>{});
    return true;
  }
  if constexpr (C == 0) {
    f(G.T);
    return true;
  }
  return false;
}

// forward jet of one site for (point p, neurons n..n+3): plain Z rows of P -> H rows (in place
// and/or operand rows of `out`)
template <int C, bool BF16>
__device__ __forceinline__ void jet_fwd_cls(float* __restrict__ P, unsigned char* __restrict__ out, int T,
                                            int base, int p, int n, int np, bool inplace, bool write_out,
                                            unsigned char* __restrict__ tsave) {
  constexpr int NS = rules_of<C>().ns;
  float4 z[NS];
  sfor<NS>([&](auto mc) {
    constexpr int M = decltype(mc)::value;
    z[M] = ld4(&P[((base + M) * T + p) * LDS + n]);
  });
  Sig sg;
  sg.make(z[0], rules_of<C>().maxk >= 4);
  if (tsave) *reinterpret_cast<float4*>(tsave + ofs(base * T + p, n, np, 4)) = sg.t;
  sfor<NS>([&](auto mc) {
    constexpr int M = decltype(mc)::value;
    float4 h;
    if constexpr (M == 0) h = sg.t;
    else h = cls_rule_sum<C, M>(sg, z);
    if (inplace) st4(&P[((base + M) * T + p) * LDS + n], h);
    if (write_out) put4<BF16>(out, (base + M) * T + p, n, np, h);
  });
}

// jet adjoint of one site for (point p, neurons n..n+3): dL/dH rows of P1 and the interleaved
// pre-activations zs -> dL/dZ rows in place (and operand rows of opA). Contributions accumulate
// in the order of the table pulls: the value stream's own term, then streams and rules ascending.
template <int C, bool BF16>
__device__ __forceinline__ void jet_bwd_cls(float* __restrict__ P1, const unsigned char* __restrict__ zs,
                                            unsigned char* __restrict__ opA, int T, int base, int p, int n,
                                            int np, bool write_op) {
  constexpr int NS = rules_of<C>().ns;
  float4 z[NS], g[NS], gz[NS];
  sfor<NS>([&](auto mc) {
    constexpr int M = decltype(mc)::value;
    z[M] = ld4o(zs, ofs((base + M) * T + p, n, np, 4));
    g[M] = ld4(&P1[((base + M) * T + p) * LDS + n]);
    gz[M] = make_float4(0.f, 0.f, 0.f, 0.f);
  });
  Sig sg;
  sg.from_t(z[0], rules_of<C>().maxk + 1 >= 4);   // the value row holds t = tanh(z)
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
    st4(&P1[((base + M) * T + p) * LDS + n], gz[M]);
    if (write_op) put4<BF16>(opA, (base + M) * T + p, n, np, gz[M]);
  });
}

// H of every stream of a classed site at (point p, neurons n..n+3) from interleaved FP32 Z rows;
// f(m, h) receives the site's stream m, m ascending
template <int C, typename F>
__device__ __forceinline__ void site_values_cls(const unsigned char* __restrict__ zs, int kp, int T, int base,
                                                int p, int n, F&& f) {
  constexpr int NS = rules_of<C>().ns;
  float4 z[NS];
  sfor<NS>([&](auto mc) {
    constexpr int M = decltype(mc)::value;
    z[M] = ld4o(zs, ofs((base + M) * T + p, n, kp, 4));
  });
  Sig sg;
  sg.from_t(z[0], rules_of<C>().maxk >= 4);   // the value row holds t = tanh(z)
  sfor<NS>([&](auto mc) {
    constexpr int M = decltype(mc)::value;
    if constexpr (M == 0) f(0, sg.t);
    else f(M, cls_rule_sum<C, M>(sg, z));
  });
}

// the same for a site run through the rule tables
template <typename F>
__device__ __forceinline__ void site_values_tab(const DevGroup& G, int q, const unsigned char* __restrict__ zs,
                                                int kp, int p, int n, F&& f) {
  const int T = G.T, ns = G.site_nstreams[q], base = G.site_streams[q][0];
  Sig sg;
  sg.from_t(ld4o(zs, ofs(base * T + p, n, kp, 4)), false);   // the value row holds t = tanh(z)
  for (int m = 0; m < ns; ++m) {
    const int s = base + m;
    float4 h = sg.t;
    if (m > 0) {
      h = make_float4(0.f, 0.f, 0.f, 0.f);
      for (int u = 0; u < G.st_nrule[s]; ++u) {
        const DevRule& ru = G.rules[s][u];
        float4 v = f4scale(sg.sel(ru.k), (float)ru.mult);
        for (int i = 0; i < ru.k; ++i) v = f4mul(v, ld4o(zs, ofs(ru.sub[i] * T + p, n, kp, 4)));
        h = f4add(h, v);
      }
    }
    f(m, h);
  }
}

// the table-driven forward jet of site q (out of line: the compiled classes are the hot path)
template <bool BF16>
__device__ __noinline__ void jet_fwd_tab(float* __restrict__ P, unsigned char* __restrict__ out,
                                         const DevGroup& G, int q, int np, bool inplace, bool also_out,
                                         unsigned char* __restrict__ tsave) {
  const int T = G.T, n4s = np >> 2;
  const int ns = G.site_nstreams[q], base = G.site_streams[q][0];
  for (int e = threadIdx.x; e < T * n4s; e += NTC) {
    const int p = e % T, n = (e / T) * 4;
    Sig sg;
    sg.make(ld4(&P[(base * T + p) * LDS + n]), false);
    if (tsave) *reinterpret_cast<float4*>(tsave + ofs(base * T + p, n, np, 4)) = sg.t;
    for (int m = ns - 1; m >= 0; --m) {
      const int s = G.site_streams[q][m];
      float4 h = sg.t;
      if (m > 0) {
        h = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int u = 0; u < G.st_nrule[s]; ++u) {
          const DevRule& ru = G.rules[s][u];
          float4 v = f4scale(sg.sel(ru.k), (float)ru.mult);
          for (int f = 0; f < ru.k; ++f) v = f4mul(v, ld4(&P[(ru.sub[f] * T + p) * LDS + n]));
          h = f4add(h, v);
        }
      }
      if (inplace) st4(&P[(s * T + p) * LDS + n], h);
      if (!inplace || also_out) put4<BF16>(out, s * T + p, n, np, h);
    }
  }
}

// the table-driven jet adjoint of site q (out of line)
template <bool BF16>
__device__ __noinline__ void jet_bwd_tab(float* __restrict__ P1, const unsigned char* __restrict__ zs,
                                         unsigned char* __restrict__ opA, const DevGroup& G, int q, int np,
                                         bool write_op) {
  const int T = G.T, n4s = np >> 2;
  const int ns = G.site_nstreams[q], base = G.site_streams[q][0];
  for (int e = threadIdx.x; e < T * n4s; e += NTC) {
    const int p = e % T, n = (e / T) * 4;
    Sig sg;
    sg.from_t(ld4o(zs, ofs(base * T + p, n, np, 4)), true);   // the value row holds t
    for (int m = 0; m < ns; ++m) {
      const int b = G.site_streams[q][m];
      float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
      const int pf = G.st_pull_first[b];
      for (int u = 0; u < G.st_npull[b]; ++u) {
        const DevPull& pl = G.pulls[pf + u];
        float4 v = f4mul(ld4(&P1[(pl.alpha * T + p) * LDS + n]), f4scale(sg.sel(pl.kk), (float)pl.mult));
        for (int f = 0; f < pl.n_oth; ++f) v = f4mul(v, ld4o(zs, ofs(pl.oth[f] * T + p, n, np, 4)));
        acc = f4add(acc, v);
      }
      st4(&P1[(b * T + p) * LDS + n], acc);
      if (write_op) put4<BF16>(opA, b * T + p, n, np, acc);
    }
  }
}

// the table-driven H rows of site q from interleaved pre-activations (out of line)
__device__ __noinline__ void rows_from_op_tab(const unsigned char* __restrict__ zs, float* __restrict__ P,
                                              const DevGroup& G, int q, int kp) {
  const int T = G.T, n4s = kp >> 2, base = G.site_streams[q][0];
  for (int e = threadIdx.x; e < T * n4s; e += NTC) {
    const int p = e % T, n = (e / T) * 4;
    site_values_tab(G, q, zs, kp, p, n, [&](int m, float4 h) { st4(&P[((base + m) * T + p) * LDS + n], h); });
  }
}

// thread (p, 4 neurons): H of every (stream, point) row from interleaved FP32 pre-activations zs
// (kp per row) into FP32 rows of P (stride LDS); tanh once per (point, neuron)
template <int CM>
__device__ void jet_rows_from_op(const unsigned char* __restrict__ zs, float* __restrict__ P,
                                 const DevGroup& G, int kp) {
  const int n4s = kp >> 2;
  for (int q = 0; q < G.n_sites; ++q) {
    const int base = G.site_streams[q][0];
    if (with_class<CM>(G.site_cls[q], [&](auto cc) {
          return with_tile_points<decltype(cc)::value>(G, [&](auto tq) {
            const int Tc = tq;
            for (int e = threadIdx.x; e < Tc * n4s; e += NTC) {
              const int p = e % Tc, n = (e / Tc) * 4;
              site_values_cls<decltype(cc)::value>(zs, kp, Tc, base, p, n, [&](int m, float4 h) {
                st4(&P[((base + m) * Tc + p) * LDS + n], h);
              });
            }
          });
        }))
      continue;
    rows_from_op_tab(zs, P, G, q, kp);
  }
}

// rows [r_lo, r_lo + nr) of FP32 rows P (kp neurons) transposed into the K-major operand dst
// (operand rows = neurons, K = the nr rows); rows >= R read as zero. A warp reads 32 neurons of
// one row (conflict-free) and a lane stores 4 rows of its neuron. Split TF32 stores [hi | lo].
template <bool BF16, bool X3>
__device__ void rows_to_opT(const float* __restrict__ P, unsigned char* __restrict__ dst, int kp, int r_lo,
                            int nr, int R, uint32_t lo_off) {
  const bool k128 = kp == 128;   // shifts instead of a runtime division for the common width
  for (int e = threadIdx.x; e < kp * (nr >> 2); e += NTC) {
    const int n = k128 ? e & 127 : e % kp, rl = 4 * (k128 ? e >> 7 : e / kp), r = r_lo + rl;
    float v[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) v[i] = r + i < R ? P[(r + i) * LDS + n] : 0.f;
    if (X3) {   // hi rounded to TF32; lo = x - hi stored as it is (the MMA takes its TF32 bits,
                // as for every other low part)
      const float4 h = make_float4(to_tf32(v[0]), to_tf32(v[1]), to_tf32(v[2]), to_tf32(v[3]));
      *reinterpret_cast<float4*>(dst + ofs(n, rl, nr, 4)) = h;
      *reinterpret_cast<float4*>(dst + lo_off + ofs(n, rl, nr, 4)) =
          make_float4(v[0] - h.x, v[1] - h.y, v[2] - h.z, v[3] - h.w);
    } else {
      put4<BF16>(dst, n, rl, nr, make_float4(v[0], v[1], v[2], v[3]));
    }
  }
}

// split TF32, 128 neurons: rows [0, 64) of P transposed into dst0 and rows [64, 128) into dst1 (each
// [hi | lo], lo at lo_off), as rows_to_opT with compile-time index arithmetic: thread t keeps
// neuron t % 128 and takes the 4-row groups (t / 128) + 4 i of each half
__device__ __forceinline__ void rows_to_opT_x3_128(const float* __restrict__ P, unsigned char* __restrict__ dst0,
                                                   unsigned char* __restrict__ dst1, int R, uint32_t lo_off) {
  static_assert(NTC % 128 == 0, "a thread keeps its neuron");
  const int n = threadIdx.x & 127;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    unsigned char* dst = h ? dst1 : dst0;
#pragma unroll
    for (int i = 0; i < 64 / 4 / (NTC / 128); ++i) {
      const int rl = 4 * ((int)(threadIdx.x >> 7) + (NTC / 128) * i), r = 64 * h + rl;
      float v[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) v[j] = r + j < R ? P[(r + j) * LDS + n] : 0.f;
      const float4 hv = make_float4(to_tf32(v[0]), to_tf32(v[1]), to_tf32(v[2]), to_tf32(v[3]));
      const uint32_t o = ofs(n, rl, 64, 4);
      *reinterpret_cast<float4*>(dst + o) = hv;
      *reinterpret_cast<float4*>(dst + lo_off + o) = make_float4(v[0] - hv.x, v[1] - hv.y, v[2] - hv.z, v[3] - hv.w);
    }
  }
}

// thread (p, 4 neurons): tanh jet of every stream of point p from plain Z rows in P, written as
// operand rows of `out`, or, when `inplace`, back into P as FP32 rows (streams of a site from the
// highest order down, the value stream last, so every Z a rule reads is still intact).
// When tsave is given, t = tanh(z) of every value row is also stored there (the saved
// pre-activations of the layer, interleaved FP32), for the backward pass.
template <bool BF16, int CM>
__device__ void jet_fwd_rows(float* __restrict__ P, unsigned char* __restrict__ out,
                             const DevGroup& G, int np, bool inplace, bool also_out,
                             unsigned char* __restrict__ tsave) {
  const int n4s = np >> 2;
  for (int q = 0; q < G.n_sites; ++q) {
    const int base = G.site_streams[q][0];
    // classed site: one loop per class, the dispatch outside it
    if (with_class<CM>(G.site_cls[q], [&](auto cc) {
          return with_tile_points<decltype(cc)::value>(G, [&](auto tq) {
            const int Tc = tq;
            for (int e = threadIdx.x; e < Tc * n4s; e += NTC)
              jet_fwd_cls<decltype(cc)::value, BF16>(P, out, Tc, base, e % Tc, (e / Tc) * 4, np, inplace,
                                                     !inplace || also_out, tsave);
          });
        }))
      continue;
    jet_fwd_tab<BF16>(P, out, G, q, np, inplace, also_out, tsave);
  }
}

// A operand rows into tensor memory (lane = row, column = K): hi = tf32(x) at a_hi and, for split
// TF32, lo = x - hi at a_lo; rows >= R are zero. Each warp writes its own lane quarter.
template <bool X3>
__device__ void rows_to_tmem(const float* __restrict__ P, uint32_t a_hi, uint32_t a_lo, int kp, int R,
                             uint32_t lane_addr, int lrow, int cgrp) {
  for (int c = 8 * cgrp; c < kp; c += 8 * NCG) {
    float x[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (lrow < R) {
      const float4 x0 = ld4(&P[lrow * LDS + c]), x1 = ld4(&P[lrow * LDS + c + 4]);
      x[0] = x0.x; x[1] = x0.y; x[2] = x0.z; x[3] = x0.w;
      x[4] = x1.x; x[5] = x1.y; x[6] = x1.z; x[7] = x1.w;
    }
    float hi[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) hi[i] = to_tf32(x[i]);
    tmem_st8(a_hi + lane_addr + c, hi);
    if (X3) {
      float lo[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) lo[i] = x[i] - hi[i];
      tmem_st8(a_lo + lane_addr + c, lo);
    }
  }
  tmem_st_wait();
}

// D[128 x n] = A . B^T with A (rows x k) in tensor memory (hi at a_hi, split TF32 lo at a_lo) and
// the packed B from global memory: split TF32 streams K-half 0 ([hi | lo]) through slot A into
// bufA and K-half 1 through slot B into bufB, and issues K-half 0's MMAs while K-half 1 lands;
// TF32 takes all of B through slot A. Copies issued ahead are waited for, not reissued.
template <bool X3, typename F>
__device__ void gemm_tmem_a(TcCtx& cx, uint32_t d, uint32_t a_hi, uint32_t a_lo, unsigned char* bufA,
                            unsigned char* bufB, const unsigned char* b_src, int n, int k, F&& during) {
  const uint32_t idesc = instr_desc<false>(128, n);
  if (X3) {
    const int kh = k / 2;
    const uint32_t hb = (uint32_t)n * kh * 4;   // one of [hi | lo] of a K-half
    const uint32_t sbo = (uint32_t)(kh / 4) * 128;
    cx.ensure_a(bufA, b_src, 2 * hb);
    if (threadIdx.x == 0) {
      fence_after();
      const uint32_t b0 = smem_u32(bufA);
      for (int j = 0; j < kh / 8; ++j) {
        const uint64_t bh = smem_desc(b0 + j * 256, 128, sbo), bl = smem_desc(b0 + hb + j * 256, 128, sbo);
        mma_ts_tf32(d, a_hi + 8 * j, bh, idesc, j > 0);
        mma_ts_tf32(d, a_hi + 8 * j, bl, idesc, true);
        mma_ts_tf32(d, a_lo + 8 * j, bh, idesc, true);
      }
    }
    cx.ensure(bufB, b_src + 2 * hb, 2 * hb);
    if (threadIdx.x == 0) {
      fence_after();
      const uint32_t b0 = smem_u32(bufB);
      for (int j = 0; j < kh / 8; ++j) {
        const int kk = kh + 8 * j;
        const uint64_t bh = smem_desc(b0 + j * 256, 128, sbo), bl = smem_desc(b0 + hb + j * 256, 128, sbo);
        mma_ts_tf32(d, a_hi + kk, bh, idesc, true);
        mma_ts_tf32(d, a_hi + kk, bl, idesc, true);
        mma_ts_tf32(d, a_lo + kk, bh, idesc, true);
      }
      commit(cx.bar_mma);
    }
  } else {
    cx.ensure_a(bufA, b_src, (uint32_t)n * k * 4);
    if (threadIdx.x == 0) {
      fence_after();
      const uint32_t b0 = smem_u32(bufA), sbo = (uint32_t)(k / 4) * 128;
      for (int j = 0; j < k / 8; ++j)
        mma_ts_tf32(d, a_hi + 8 * j, smem_desc(b0 + j * 256, 128, sbo), idesc, j > 0);
      commit(cx.bar_mma);
    }
  }
  during();   // every thread: work that touches neither the operands nor the accumulator
  cx.wait_mma();
}

// dL/dH rows from the dX accumulator (tensor memory) into plain FP32 rows, zero past K and R
__device__ __forceinline__ void d1_to_rows(uint32_t d1, float* __restrict__ P, int kp, int K, int R,
                                           uint32_t lane_addr, int lrow, int cgrp) {
  const bool plain = K == kp && lrow < R;   // nothing to mask
  for (int c = 8 * cgrp; c < kp; c += 8 * NCG) {
    float v[8];
    tmem_ld8(d1 + lane_addr + c, v);
    if (!plain) {
#pragma unroll
      for (int i = 0; i < 8; ++i)
        if (lrow >= R || c + i >= K) v[i] = 0.f;
    }
    st4(&P[lrow * LDS + c], make_float4(v[0], v[1], v[2], v[3]));
    st4(&P[lrow * LDS + c + 4], make_float4(v[4], v[5], v[6], v[7]));
  }
}

// zero rows [r0, 128) of an operand with kp elements per row
template <bool BF16>
__device__ void zero_rows(unsigned char* buf, int r0, int kp, int es) {
  const int n4s = kp >> 2;
  const bool k128 = kp == 128;
  for (int e = threadIdx.x; e < (128 - r0) * n4s; e += NTC) {
    const int r = r0 + (k128 ? e >> 5 : e / n4s), n = (k128 ? e & 31 : e % n4s) * 4;
    if (es == 4) *reinterpret_cast<float4*>(buf + ofs(r, n, kp, 4)) = make_float4(0, 0, 0, 0);
    else *reinterpret_cast<uint2*>(buf + ofs(r, n, kp, 2)) = make_uint2(0, 0);
  }
}

}  // namespace

struct TcArgs {
  const unsigned char* wpack;                 // packed hidden weights of problem 0
  int64_t wpack_stride;                       // bytes per problem
  int64_t wfwd_off[TDG_MAX_LAYERS];           // byte offsets of W_j (forward) per Linear j
  int64_t wbwd_off[TDG_MAX_LAYERS];           // byte offsets of W_j^T
  int* err;                                   // set when a bounded wait gives up
};

template <bool BF16, bool X3, int CM>
__global__ void __launch_bounds__(NTC, 1) fused_tc_kernel(FusedArgs A, TcArgs TA) {
  constexpr int ES = BF16 ? 2 : 4;
  static_assert(!(BF16 && X3), "split TF32 is a TF32 mode");
  // TF32 and split TF32 keep every A operand in tensor memory (hi at AHI, lo at ALO), which
  // leaves both shared-memory operand buffers to the B operands; BF16 keeps A in opA
  constexpr bool TMA_A = !BF16;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* opA = smem_raw;
  unsigned char* opB = smem_raw + OPB;
  float* P1 = reinterpret_cast<float*>(smem_raw + 2 * OPB);
  float* ybuf = P1 + RMAX * LDS;
  float* gybuf = ybuf + RMAX * MAX_OUT;
  float* xsbuf = gybuf + RMAX * MAX_OUT;
  float* pbuf = xsbuf + RMAX * TDG_MAX_DIN;                     // PBUF floats: small parameters
  DevGroup* Gs = reinterpret_cast<DevGroup*>(pbuf + PBUF);
  double* cur_slot = reinterpret_cast<double*>(Gs + 1);        // [MAX_OUT]
  double* wred = cur_slot + MAX_OUT;                           // [NTC/32][MAX_OUT]
  uint64_t* bars = reinterpret_cast<uint64_t*>(wred + (NTC / 32) * MAX_OUT);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 3);
  int8_t* row_s = reinterpret_cast<int8_t*>(tmem_slot + 4);     // [128] stream of a row, -1 padding
  uint8_t* row_v = reinterpret_cast<uint8_t*>(row_s + 128);     // [128] 1 on value-stream rows
  int8_t* row_ax = reinterpret_cast<int8_t*>(row_v + 128);      // [128] -1 value row, axis of a first
                                                                 // derivative row, -2 otherwise

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int cta = blockIdx.x;
  const int L = A.n_layers;
  const int d_in = A.width[0], d_out = A.width[L];
  const int64_t scr_slot = 128 * 128;                         // floats per saved layer
  float* scr = A.scratch + (int64_t)cta * (L - 1) * scr_slot;

  if (tid == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    mbar_init(&bars[2], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) tmem_alloc(tmem_slot, TMA_A ? 512 : 256);
  for (int s = tid; s < A.n_slots; s += NTC) A.slot_partial[(int64_t)cta * A.n_slots + s] = 0.0;
  if (tid < MAX_OUT) cur_slot[tid] = 0.0;
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t D1 = *tmem_slot, D2 = *tmem_slot + 128;
  const uint32_t AHI = *tmem_slot + 256;                    // the A operand (TF32 hi) in TMEM
  const uint32_t ALO = *tmem_slot + (TMA_A ? 384 : 256);    // split TF32: its low part
  TcCtx cx{&bars[0], &bars[1], &bars[2], 0u, 0u, 0u, TA.err, false, false};
  // TMEM lane quarter and column group of this warp in the epilogues
  const int lrow = 32 * (warp & 3) + lane;
  const uint32_t lane_addr = (uint32_t)(32 * (warp & 3)) << 16;
  const int cgrp = warp >> 2;                    // this warp's 8-column chunks c = 8 * (cgrp + NCG * i)
  int cur_group = -1, cur_problem = -1;
  const unsigned char* wpk = TA.wpack;           // the packed weights of the tile's problem
  // the first bulk copy of hidden GEMM j's forward weights (split TF32: the first [hi | lo] half)
  auto wfwd_first = [&](int j) {
    const uint32_t nk = (uint32_t)p16(A.width[j + 1]) * p16(A.width[j]);
    if constexpr (TMA_A) {   // split TF32: K-half 0 -> opA, K-half 1 -> opB; TF32: all -> opA
      cx.issue_a(opA, wpk + TA.wfwd_off[j], nk * 4);
      if (X3) cx.issue(opB, wpk + TA.wfwd_off[j] + nk * 4, nk * 4);
    } else {
      cx.issue(opB, wpk + TA.wfwd_off[j], X3 ? nk * 4 : nk * ES);
    }
  };
  // the first bulk copy of the dX GEMM's B operand (W^T of Linear j): slot A into opA
  auto wbwd_first = [&](int j) {
    const uint32_t nk = (uint32_t)p16(A.width[j + 1]) * p16(A.width[j]);
    cx.issue_a(opA, wpk + TA.wbwd_off[j], nk * 4);
  };

  for (int ti = A.cta_tile_begin[cta]; ti < A.cta_tile_begin[cta + 1]; ++ti) {
    const DevTile tile = A.tiles[ti];
    wpk = TA.wpack + (int64_t)tile.problem * TA.wpack_stride;
    cx.publish();                    // opB's last generic accesses ordered before the copy below
    if (L > 2) wfwd_first(1);        // overlaps the coordinates, input layer and first jets
    if (tile.group != cur_group) {
      if (cur_group >= 0 && tid < Gs->n_outputs) {
        A.slot_partial[(int64_t)cta * A.n_slots + Gs->slot_first + tid] += cur_slot[tid];
        cur_slot[tid] = 0.0;
      }
      __syncthreads();
      const int4* src = reinterpret_cast<const int4*>(&A.groups[tile.group]);
      int4* dst = reinterpret_cast<int4*>(Gs);
      for (int e = tid; e < (int)(sizeof(DevGroup) / 16); e += NTC) dst[e] = src[e];
      cur_group = tile.group;
      __syncthreads();
      if (tid < 128) {
        const int T0 = Gs->T, R0 = Gs->T * Gs->S;
        const int sr = tid < R0 ? tid / T0 : -1;
        row_s[tid] = (int8_t)sr;
        row_v[tid] = (uint8_t)(sr >= 0 && Gs->st_order[sr] == 0);
        row_ax[tid] = (int8_t)(sr < 0 ? -2 : Gs->st_order[sr] == 0 ? -1 : Gs->st_order[sr] == 1 ? Gs->st_axis[sr] : -2);
      }
      if (Gs->problem != cur_problem) {   // stage the problem's small parameters
        cur_problem = Gs->problem;
        const float* pp = A.params + (int64_t)cur_problem * A.n_params;
        for (int j = 1; j < L - 1; ++j)
          for (int n = tid; n < A.width[j + 1]; n += NTC) pbuf[PB_HB + (j - 1) * TDG_MAX_WIDTH + n] = pp[A.b_off[j] + n];
        for (int e = tid; e < A.width[1] * d_in; e += NTC) pbuf[PB_W0 + e] = pp[A.w_off[0] + e];
        for (int n = tid; n < A.width[1]; n += NTC) pbuf[PB_B0 + n] = pp[A.b_off[0] + n];
        for (int e = tid; e < d_out * A.width[L - 1]; e += NTC) pbuf[PB_WL + e] = pp[A.w_off[L - 1] + e];
        for (int o = tid; o < d_out; o += NTC) pbuf[PB_BL + o] = pp[A.b_off[L - 1] + o];
        for (int k = tid; k < A.n_coeff; k += NTC) pbuf[PB_CF + k] = pp[A.coeff_off + k];
      }
      __syncthreads();
      if (A.n_coeff > 0) {   // trainable coefficients: the shared copy carries scale * theta
        for (int t = tid; t < Gs->n_terms; t += NTC)
          if (Gs->terms[t].coeff_param >= 0)
            Gs->terms[t].coeff = A.groups[tile.group].terms[t].coeff * pbuf[PB_CF + Gs->terms[t].coeff_param];
        __syncthreads();
      }
    }
    const DevGroup& G = *Gs;
    const int T = G.T, S = G.S, R = T * S;
    // e / T for 0 <= e < 2^16 as one multiply-high: tmag = ceil(2^32 / T), exact since e T < 2^32
    const uint32_t tmag = 0xFFFFFFFFu / (uint32_t)T + 1u;
    auto divT = [&](int e) { return (int)__umulhi((uint32_t)e, tmag); };
    const int nvalid = tile.nvalid, row0 = tile.row0;


    // ---- input layer -> Z_1 (plain in P1, interleaved FP32 in scratch slot 0)
    {
      const int N = A.width[1], np = p16(N);
      const float* W0 = pbuf + PB_W0;
      const float* b0 = pbuf + PB_B0;
      // a thread keeps one row in every iteration (NTC is a multiple of RMAX): its kind and
      // coordinates load once; W0 and b0 of 4 neurons are 16-byte vectors (widths are multiples
      // of 4); the input width is a compile-time constant of each branch
      static_assert(NTC % RMAX == 0, "a thread keeps its row");
      const int r = tid % RMAX;
      const int ax = row_ax[r];   // a value row: W0 x + b0; d/dx_a: column a of W0; else 0
      unsigned char* s0 = reinterpret_cast<unsigned char*>(scr);
      auto layer = [&](auto din) {
        constexpr int D = decltype(din)::value;
        // the coordinates of this thread's row, loaded by the thread itself (no barrier); the
        // threads of the first 128 also keep them in xsbuf for the input-layer gradients
        float x[D];
#pragma unroll
        for (int a = 0; a < D; ++a) x[a] = 0.f;
        if (r < R) {
          const int s = r / T, p = r - s * T, q = G.st_site[s];
          if (p < nvalid) {
            const float* src = A.arrays[G.site_points[q]] + (int64_t)(row0 + p) * D;
#pragma unroll
            for (int a = 0; a < D; ++a) x[a] = src[a] + G.site_off[q][a];
          }
        }
        if (tid < RMAX) {
#pragma unroll
          for (int a = 0; a < D; ++a) xsbuf[r * TDG_MAX_DIN + a] = x[a];
        }
        for (int e = tid; e < RMAX * (np >> 2); e += NTC) {
          const int n = (e / RMAX) * 4;
          float z[4] = {0.f, 0.f, 0.f, 0.f};
          if (n < N) {
            if (ax == -1) {
              float w[4 * D];
#pragma unroll
              for (int c = 0; c < D; ++c) {
                const float4 wv = ld4(&W0[n * D + 4 * c]);
                w[4 * c] = wv.x; w[4 * c + 1] = wv.y; w[4 * c + 2] = wv.z; w[4 * c + 3] = wv.w;
              }
              const float4 bv = ld4(&b0[n]);
              const float bb[4] = {bv.x, bv.y, bv.z, bv.w};
#pragma unroll
              for (int i = 0; i < 4; ++i) {
                float v = 0.f;
#pragma unroll
                for (int a = 0; a < D; ++a) v = fmaf(w[i * D + a], x[a], v);
                z[i] = v + bb[i];
              }
            } else if (ax >= 0) {
#pragma unroll
              for (int i = 0; i < 4; ++i) z[i] = W0[(n + i) * D + ax];
            }
          }
          const float4 zv = make_float4(z[0], z[1], z[2], z[3]);
          st4(&P1[r * LDS + n], zv);
          if (A.do_grad && ax != -1)   // value rows: the jets save t = tanh(z) instead
            *reinterpret_cast<float4*>(s0 + ofs(r, n, np, 4)) = zv;
        }
      };
      switch (d_in) {
        case 1: layer(std::integral_constant<int, 1>{}); break;
        case 2: layer(std::integral_constant<int, 2>{}); break;
        case 3: layer(std::integral_constant<int, 3>{}); break;
        default: layer(std::integral_constant<int, 4>{}); break;
      }
    }
    __syncthreads();
    unsigned char* t0 = A.do_grad ? reinterpret_cast<unsigned char*>(scr) : nullptr;
    if (L == 2) {
      jet_fwd_rows<BF16, CM>(P1, opA, G, p16(A.width[1]), true, false, t0);   // last hidden layer: rows in P1
    } else if constexpr (TMA_A) {   // H rows in P1, then hi (and lo) into tensor memory
      jet_fwd_rows<BF16, CM>(P1, opA, G, p16(A.width[1]), true, false, t0);
      __syncthreads();
      rows_to_tmem<X3>(P1, AHI, ALO, p16(A.width[1]), R, lane_addr, lrow, cgrp);
    } else {
      jet_fwd_rows<BF16, CM>(P1, opA, G, p16(A.width[1]), false, false, t0);
      zero_rows<BF16>(opA, R, p16(A.width[1]), ES);
    }
    cx.publish();

    // ---- hidden layers on the tensor cores
    for (int j = 1; j < L - 1; ++j) {
      const int K = A.width[j], N = A.width[j + 1];
      const int kp = p16(K), np = p16(N);
      if constexpr (TMA_A) {
        gemm_tmem_a<X3>(cx, D1, AHI, ALO, opA, opB, wpk + TA.wfwd_off[j], np, kp, [] {});
      } else {
        cx.ensure(opB, wpk + TA.wfwd_off[j], (uint32_t)(np * kp * ES));
        gemm_issue<BF16>(D1, opA, opB, np, kp, cx.bar_mma);
        cx.wait_mma();
      }
      if (j + 1 < L - 1) wfwd_first(j + 1);   // the buffers are free: overlaps the epilogue and the jets
      else if (TMA_A && A.do_grad) wbwd_first(L - 2);   // the first dX GEMM's W^T, during the program
      // epilogue: D1 -> +bias -> P1 (plain) and scratch slot j (interleaved FP32)
      {
        const float* bj = pbuf + PB_HB + (j - 1) * TDG_MAX_WIDTH;
        const bool val = row_v[lrow] != 0;
        unsigned char* sj = reinterpret_cast<unsigned char*>(scr + (int64_t)j * scr_slot);
        // a full-width layer and a filled row need no masks: v + 1 * b on value rows, v + 0 * b
        // on the others (the same sums as the masked form)
        const bool plain = N == np && lrow < R;
        const float vb = val ? 1.f : 0.f;
        for (int c = 8 * cgrp; c < np; c += 8 * NCG) {
          float v[8];
          tmem_ld8(D1 + lane_addr + c, v);
          const float4 b0v = ld4(&bj[c]), b1v = ld4(&bj[c + 4]);
          const float bb[8] = {b0v.x, b0v.y, b0v.z, b0v.w, b1v.x, b1v.y, b1v.z, b1v.w};
          if (plain) {
#pragma unroll
            for (int i = 0; i < 8; ++i) v[i] = fmaf(vb, bb[i], v[i]);
          } else {
#pragma unroll
            for (int i = 0; i < 8; ++i) {
              const int n = c + i;
              v[i] = n < N ? v[i] + (val ? bb[i] : 0.f) : 0.f;
              if (lrow >= R) v[i] = 0.f;
            }
          }
          st4(&P1[lrow * LDS + c], make_float4(v[0], v[1], v[2], v[3]));
          st4(&P1[lrow * LDS + c + 4], make_float4(v[4], v[5], v[6], v[7]));
          if (A.do_grad && !val) {   // value rows: the jets save t = tanh(z) instead
            *reinterpret_cast<float4*>(sj + ofs(lrow, c, np, 4)) = make_float4(v[0], v[1], v[2], v[3]);
            *reinterpret_cast<float4*>(sj + ofs(lrow, c + 4, np, 4)) = make_float4(v[4], v[5], v[6], v[7]);
          }
        }
      }
      fence_before();
      __syncthreads();
      unsigned char* tj = A.do_grad ? reinterpret_cast<unsigned char*>(scr + (int64_t)j * scr_slot) : nullptr;
      if (j == L - 2) {
        jet_fwd_rows<BF16, CM>(P1, opA, G, np, true, false, tj);   // last hidden layer: FP32 rows in P1
      } else if constexpr (TMA_A) {
        jet_fwd_rows<BF16, CM>(P1, opA, G, np, true, false, tj);
        __syncthreads();
        rows_to_tmem<X3>(P1, AHI, ALO, np, R, lane_addr, lrow, cgrp);
      } else {
        jet_fwd_rows<BF16, CM>(P1, opA, G, np, false, false, tj);
        zero_rows<BF16>(opA, R, np, ES);
      }
      cx.publish();
    }

    // ---- output layer (H_{L-1} as FP32 rows in P1)
    {
      const int K = A.width[L - 1];
      const float* Wl = pbuf + PB_WL;
      const float* bl = pbuf + PB_BL;
      for (int e = tid; e < RMAX * d_out; e += NTC) {
        const int r = e % RMAX, o = e / RMAX;
        // four independent chains (16-byte chunks c, c + 4, ...), summed pairwise at the end
        float zc[4] = {0.f, 0.f, 0.f, 0.f};
        const float* w = &Wl[(int64_t)o * K];
        for (int k = 0; k < K; k += 16) {
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            if (k + 4 * c < K) {
              const float4 hv = ld4(&P1[r * LDS + k + 4 * c]), wv = ld4(&w[k + 4 * c]);
              zc[c] = fmaf(hv.x, wv.x, zc[c]);
              zc[c] = fmaf(hv.y, wv.y, zc[c]);
              zc[c] = fmaf(hv.z, wv.z, zc[c]);
              zc[c] = fmaf(hv.w, wv.w, zc[c]);
            }
          }
        }
        float z = (zc[0] + zc[1]) + (zc[2] + zc[3]);
        if (row_v[r]) z += bl[o];
        ybuf[r * MAX_OUT + o] = z;
        gybuf[r * MAX_OUT + o] = 0.f;
      }
    }
    __syncthreads();

    // ---- operator program: term values per (point, term), outputs and squared errors per
    // (point, output), the loss seeds, then the program adjoint per (point, term). Scratch lives in
    // opB, which no MMA reads between the last forward GEMM and the first backward bulk copy.
    const int n_out = G.n_outputs;
    {
      float* tv = reinterpret_cast<float*>(opB);           // [MAX_TERMS][T] term values
      float* seedv = tv + MAX_TERMS * RMAX;                 // [MAX_OUT][T] dL/d(output)
      double* e2 = reinterpret_cast<double*>(seedv + MAX_OUT * RMAX);   // [MAX_OUT][T]
      const int nt = G.n_terms;
      for (int e = tid; e < T * nt; e += NTC) {
        const int t = divT(e), p = e - t * T;
        const DevTerm& tm = G.terms[t];
        const bool valid = p < nvalid;
        const float c = tm.coeff_array >= 0 && valid ? A.arrays[tm.coeff_array][row0 + p] : tm.coeff;
        float prod = 1.f;
        for (int f = 0; f < tm.n_factors; ++f) {
          const DevFactor& fc = G.factors[tm.factor_first + f];
          float F = 0.f;
          for (int u = 0; u < fc.n_parts; ++u) {
            const DevPart& pt = G.parts[fc.part_first + u];
            F = fmaf(ybuf[(pt.stream * T + p) * MAX_OUT + fc.var], pt.weight, F);
          }
          prod *= powf_(F, fc.power);
        }
        tv[t * RMAX + p] = c * prod;
      }
      __syncthreads();
      for (int e = tid; e < T * n_out; e += NTC) {
        const int o = divT(e), p = e - o * T;
        const bool valid = p < nvalid;
        float out = 0.f;
        for (int t = 0; t < nt; ++t)
          if (G.terms[t].output == o) out += tv[t * RMAX + p];
        const float tgt = (G.target_array >= 0 && valid)
                              ? A.arrays[G.target_array][(int64_t)(row0 + p) * n_out + o] : 0.f;
        const float err = valid ? out - tgt : 0.f;
        const float rw = (G.row_weight_array >= 0 && valid) ? A.arrays[G.row_weight_array][row0 + p] : 1.f;
        e2[o * RMAX + p] = (double)err * (double)err * (double)rw;   // per-row loss weights (causal loss)
        seedv[o * RMAX + p] = err * G.seed_scale[o] * rw;
        if (A.outputs && G.out_offset >= 0 && valid)
          A.outputs[G.out_offset + (int64_t)(row0 + p) * n_out + o] = out;
      }
      __syncthreads();
      if (warp < n_out) {   // FP64 sum over the tile's points, one warp per output, fixed order:
                            // lane-strided partial sums, then a butterfly
        double sum = 0.0;
        for (int p = lane; p < T; p += 32) sum += e2[warp * RMAX + p];
#pragma unroll
        for (int m = 16; m >= 1; m >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, m);
        if (lane == 0) cur_slot[warp] += sum;
      }
      if (A.do_grad) {
        for (int e = tid; e < T * nt; e += NTC) {
          const int t = divT(e), p = e - t * T;
          const DevTerm& tm = G.terms[t];
          const bool valid = p < nvalid;
          const float c = tm.coeff_array >= 0 && valid ? A.arrays[tm.coeff_array][row0 + p] : tm.coeff;
          const float dt = seedv[tm.output * RMAX + p] * c;
          if (dt == 0.f) continue;
          float F[MAX_TERM_FACTORS];
          for (int f = 0; f < tm.n_factors; ++f) {
            const DevFactor& fc = G.factors[tm.factor_first + f];
            float v = 0.f;
            for (int u = 0; u < fc.n_parts; ++u) {
              const DevPart& pt = G.parts[fc.part_first + u];
              v = fmaf(ybuf[(pt.stream * T + p) * MAX_OUT + fc.var], pt.weight, v);
            }
            F[f] = v;
          }
          for (int f = 0; f < tm.n_factors; ++f) {
            const DevFactor& fc = G.factors[tm.factor_first + f];
            float d = dt * dpowf_(F[f], fc.power);
            for (int g = 0; g < tm.n_factors; ++g)
              if (g != f) d *= powf_(F[g], G.factors[tm.factor_first + g].power);
            for (int u = 0; u < fc.n_parts; ++u) {
              const DevPart& pt = G.parts[fc.part_first + u];
              atomicAdd(&gybuf[(pt.stream * T + p) * MAX_OUT + fc.var], d * pt.weight);
            }
          }
        }
        if (A.n_coeff > 0)
          coeff_grad_tile(G, A.groups[tile.group].terms, ybuf, seedv, tv, T,
                          A.partial + (int64_t)tile.seg * A.part_stride + A.coeff_off, A.n_coeff);
      }
    }
    if (!A.do_grad) continue;
    cx.publish_global();   // opB's program scratch is dead and every Z of the tile stored:
                           // Z_{L-1} overlaps the output layer
    cx.issue(opB, scr + (int64_t)(L - 2) * scr_slot, (uint32_t)(128 * p16(A.width[L - 1]) * 4));

    // this CTA's gradient segment, zeroed before the launch; every per-tile sum is added with a
    // fire-and-forget atomic (one thread owns each address, so the order of the adds is fixed)
    float* grad = A.partial + (int64_t)tile.seg * A.part_stride;
    // ---- output layer backward: dW, db (H_{L-1} in P1), then dL/dH_{L-1} -> P1
    {
      const int K = A.width[L - 1], kp = p16(K);
      const float* Wl = pbuf + PB_WL;
      float* dW = grad + A.w_off[L - 1];
      float* db = grad + A.b_off[L - 1];
      // dW = dL/dY^T . H_{L-1} and db = sums of dL/dY over the value rows, a warp per (output,
      // 32 input neurons) or per output bias. For dW a lane is (row phase c = lane / 8, 4 neurons):
      // it sums rows c, c + 4, ...; the four phases combine by shuffles in a fixed order, so every
      // sum has the same order in every tile (K is a multiple of 4: 16-byte vectors and atomics)
      {
        const int nkb = (K + 31) / 32;
        for (int t = warp; t < d_out * (nkb + 1); t += NTC / 32) {
          const int o = t / (nkb + 1), b = t - o * (nkb + 1);
          if (b < nkb) {
            const int c = lane >> 3, k = 32 * b + 4 * (lane & 7);
            float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
            if (k < K)
#pragma unroll 4
              for (int r = c; r < R; r += 4) {
                const float gy = gybuf[r * MAX_OUT + o];
                const float4 h = ld4(&P1[r * LDS + k]);
                s = make_float4(fmaf(gy, h.x, s.x), fmaf(gy, h.y, s.y), fmaf(gy, h.z, s.z),
                                fmaf(gy, h.w, s.w));
              }
#pragma unroll
            for (int m = 8; m <= 16; m <<= 1) {
              s.x += __shfl_xor_sync(0xffffffffu, s.x, m);
              s.y += __shfl_xor_sync(0xffffffffu, s.y, m);
              s.z += __shfl_xor_sync(0xffffffffu, s.z, m);
              s.w += __shfl_xor_sync(0xffffffffu, s.w, m);
            }
            if (c == 0 && k < K) red_add4(&dW[(int64_t)o * K + k], s.x, s.y, s.z, s.w);
          } else {
            float s = 0.f;
            for (int r = lane; r < R; r += 32)
              if (row_v[r]) s += gybuf[r * MAX_OUT + o];
#pragma unroll
            for (int m = 16; m >= 1; m >>= 1) s += __shfl_xor_sync(0xffffffffu, s, m);
            if (lane == 0) red_add1(&db[o], s);
          }
        }
      }
      __syncthreads();
      // dL/dH_{L-1} = dL/dY . W: consecutive threads take consecutive 4-neuron chunks of one row,
      // so a warp's seed loads are one broadcast and its W loads and row stores are contiguous
      // (conflict-free)
      {
        const int n4s = kp >> 2;
        const bool k128 = kp == 128;   // compile-time index arithmetic for the common width
        for (int e = tid; e < RMAX * n4s; e += NTC) {
          const int r = k128 ? e >> 5 : e / n4s, k = k128 ? (e & 31) * 4 : (e - r * n4s) * 4;
          float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
          if (r < R && k < K) {
#pragma unroll
            for (int o = 0; o < MAX_OUT; ++o)
              if (o < d_out) {
                const float g = gybuf[r * MAX_OUT + o];
                const float4 w = ld4(&Wl[o * K + k]);
                v = make_float4(fmaf(g, w.x, v.x), fmaf(g, w.y, v.y), fmaf(g, w.z, v.z),
                                fmaf(g, w.w, v.w));
              }
          }
          st4(&P1[r * LDS + k], v);
        }
      }
    }
    __syncthreads();

    for (int l = L - 1; l >= 1; --l) {
      const int N = A.width[l], np = p16(N);
      if (l >= 2 && tid == 0)   // warm L2 with the pre-activations the dW operand will need
        prefetch_l2(scr + (int64_t)(l - 2) * scr_slot, (uint32_t)(128 * p16(A.width[l - 1]) * 4));
      // Z_l (scratch slot l-1, interleaved FP32) -> opB, issued ahead
      cx.ensure(opB, scr + (int64_t)(l - 1) * scr_slot, (uint32_t)(128 * np * 4));

      // jet adjoint: P1 (dL/dH_l) -> P1 (dL/dZ_l) in place, streams of a site in increasing order;
      // also the K-major operand copy of dL/dZ_l in opA for the dX GEMM
      {
        const int n4s = np >> 2;
        for (int q = 0; q < G.n_sites; ++q) {
          const int base = G.site_streams[q][0];
          if (with_class<CM>(G.site_cls[q], [&](auto cc) {
                return with_tile_points<decltype(cc)::value>(G, [&](auto tq) {
                  const int Tc = tq;
                  for (int e = tid; e < Tc * n4s; e += NTC)
                    jet_bwd_cls<decltype(cc)::value, BF16>(P1, opB, opA, Tc, base, e % Tc, (e / Tc) * 4, np,
                                                           !TMA_A && l >= 2);
                });
              }))
            continue;
          jet_bwd_tab<BF16>(P1, opB, opA, G, q, np, !TMA_A && l >= 2);
        }
      }
      if (l == 1) {
        __syncthreads();
        // input layer gradients from dL/dZ_1 in P1: 4 row quarters per neuron, then reduced
        float* red = reinterpret_cast<float*>(opA);   // [NPART][640] partials; opA is free at layer 1
        {
          constexpr int RPP = (RMAX + NPART - 1) / NPART;   // rows per part
          const int n = tid & 127, part = tid >> 7;
          float sb = 0.f;
          float sw[TDG_MAX_DIN] = {0.f, 0.f, 0.f, 0.f};
          const int r_end = RPP * part + RPP < R ? RPP * part + RPP : R;
          // branch-free and unrolled, so that the rows' loads overlap: a value row adds g to the
          // bias and g x_a to column a, a first-derivative row along a adds g to column a (adding
          // zero elsewhere leaves every sum bit for bit as the per-kind branches would)
          if (n < N) {
#pragma unroll 4
            for (int r = RPP * part; r < r_end; ++r) {
              const int ax = row_ax[r];   // -1 value row, else the axis of a first derivative
              const float g = P1[r * LDS + n];
              const float gv = ax == -1 ? g : 0.f;
              const float4 xv = ld4(&xsbuf[r * TDG_MAX_DIN]);
              const float xa[TDG_MAX_DIN] = {xv.x, xv.y, xv.z, xv.w};
              sb += gv;
#pragma unroll
              for (int a = 0; a < TDG_MAX_DIN; ++a)
                if (a < d_in) sw[a] = fmaf(gv, xa[a], sw[a]) + (a == ax ? g : 0.f);
            }
          }
          red[part * 640 + n] = sb;
#pragma unroll
          for (int a = 0; a < TDG_MAX_DIN; ++a) red[part * 640 + 128 * (1 + a) + n] = sw[a];
        }
        __syncthreads();
        float* dW0 = grad + A.w_off[0];
        float* db0 = grad + A.b_off[0];
        for (int e = tid; e < N * (1 + d_in); e += NTC) {
          const int n = N == 128 ? e & 127 : e % N, c = N == 128 ? e >> 7 : e / N;   // c = 0: bias, c = 1 + a: weight column a
          float v = red[128 * c + n];
#pragma unroll
          for (int q = 1; q < NPART; ++q) v += red[640 * q + 128 * c + n];
          float* dst = c == 0 ? &db0[n] : &dW0[n * d_in + (c - 1)];
          red_add1(dst, v);
        }
        break;
      }
      const int K = A.width[l - 1], kp = p16(K);
      if constexpr (TMA_A) {
        __syncthreads();
        rows_to_tmem<X3>(P1, AHI, ALO, np, R, lane_addr, lrow, cgrp);   // dL/dZ_l: the dX A operand
        cx.publish();
        if (X3)   // opB (Z_l) is free: K-half 1 of W_{l-1}^T lands while K-half 0's MMAs run
          cx.issue(opB, wpk + TA.wbwd_off[l - 1] + (uint32_t)kp * np * 4, (uint32_t)kp * np * 4);
      } else {
        zero_rows<BF16>(opA, R, np, ES);
        cx.publish();
      }
      // Z_l (scratch slot l-1) reached opB for the last time at the top of this layer: warps
      // other than the MMA issuer's drop its lines from L2 (no write-back to DRAM; the next tile's
      // forward rewrites them) while the dX GEMM's weights land and its MMAs run
      if (warp > 0) {
        const char* zg = reinterpret_cast<const char*>(scr + (int64_t)(l - 1) * scr_slot);
        for (int off = (tid - 32) * 128; off < 128 * np * 4; off += (NTC - 32) * 128) discard_l2(zg + off);
      }
      // dX: D1[rows x kp] = dL/dZ_l[rows x np] . (W_{l-1}^T packed [kp x np])^T
      if constexpr (TMA_A) {
        // while the MMAs run: the bias gradient partials of Linear l-1 (sums of dL/dZ_l over the
        // value rows of row blocks 8 (q + 4 i), q = this thread's part) from P1, into ybuf
        gemm_tmem_a<X3>(cx, D1, AHI, ALO, opA, opB, wpk + TA.wbwd_off[l - 1], kp, np, [&] {
          const int n = tid & 127, q = tid >> 7;
          float sb = 0.f;
          if (n < N) {
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
              for (int rr = 0; rr < 8; ++rr) {
                const int r = 8 * (q + 4 * i) + rr;
                if (row_v[r]) sb += P1[r * LDS + n];
              }
          }
          ybuf[q * 128 + n] = sb;
        });
      } else {
        cx.load(opB, wpk + TA.wbwd_off[l - 1], (uint32_t)(kp * np * ES));
        gemm_issue<BF16>(D1, opA, opB, kp, np, cx.bar_mma);
        cx.wait_mma();
      }
      // opB is free: Z_{l-1} (scratch slot l-2, interleaved FP32) overlaps the dW operand A build
      cx.issue(opB, scr + (int64_t)(l - 2) * scr_slot, (uint32_t)(128 * kp * 4));
      // dW operand A = dL/dZ_l^T [128 (neurons, zero padded) x 128 rows] from P1, and the bias
      // gradient of Linear l-1 (sum of dL/dZ_l over value rows) from the same reads
      {
        float* red = ybuf;   // [NPART][128] bias partials
        const int n = tid & 127;
        float sb = 0.f;
        for (int e = tid; e < 128 * 32; e += NTC) {
          if constexpr (TMA_A && X3) {   // lane = neuron n, columns = rows r..r+7 (the same r for the warp)
            if (e >= 128 * 16) break;
            const int r = (e >> 7) * 8;
            float v[8], h[8];
            if (n < N && r + 8 <= R) {   // a full block of rows: no masks
#pragma unroll
              for (int i = 0; i < 8; ++i) v[i] = P1[(r + i) * LDS + n];
            } else {
#pragma unroll
              for (int i = 0; i < 8; ++i) v[i] = (n < N && r + i < R) ? P1[(r + i) * LDS + n] : 0.f;
            }
#pragma unroll
            for (int i = 0; i < 8; ++i) h[i] = to_tf32(v[i]);
            tmem_st8(AHI + lane_addr + r, h);
            if (X3) {
#pragma unroll
              for (int i = 0; i < 8; ++i) v[i] -= h[i];
              tmem_st8(ALO + lane_addr + r, v);
            }
            continue;
          }
          const int r = (e >> 7) * 4;
          float v[4];
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            v[i] = (n < N && r + i < R) ? P1[(r + i) * LDS + n] : 0.f;
            if (!TMA_A && row_v[r + i]) sb += v[i];
          }
          if constexpr (TMA_A) {   // lane = neuron n, columns = rows r..r+3 (the same r for the warp)
            tmem_st4(AHI + lane_addr + r, to_tf32(v[0]), to_tf32(v[1]), to_tf32(v[2]), to_tf32(v[3]));
          } else {
            put4<BF16>(opA, n, r, 128, make_float4(v[0], v[1], v[2], v[3]));
          }
        }
        if (TMA_A) tmem_st_wait();
        if (!TMA_A) red[(tid >> 7) * 128 + n] = sb;   // TMA_A: written while the dX MMAs ran
        __syncthreads();
        float* db = grad + A.b_off[l - 1];
        for (int m = tid; m < N; m += NTC) {
          float v = red[m];
#pragma unroll
          for (int q = 1; q < NPART; ++q) v += red[128 * q + m];
          red_add1(&db[m], v);
        }
      }
      // no barrier here: the H rows below overwrite P1, which every thread finished reading
      // before the barrier above, and the bias partials are not written again in this layer
      if constexpr (!TMA_A) cx.publish();
      // H_{l-1}: the tanh jets of Z_{l-1} (opB) per (point, 4 neurons), every stream of a site
      // at once, as FP32 rows in P1 (dL/dZ_l there is consumed)
      cx.wait_tma();
      jet_rows_from_op<CM>(opB, P1, G, kp);
      cx.publish();
      if constexpr (TMA_A) {
        // H_{l-1}^T as the B operand (K = rows): split TF32 puts rows 0..63 ([hi | lo]) in opA and
        // rows 64..127 in opB, TF32 all rows in opA; A = dL/dZ_l^T (hi, lo) in tensor memory
        const uint32_t idesc = instr_desc<false>(128, kp);
        if (X3) {
          const uint32_t lo_off = (uint32_t)kp * 64 * 4;
          if (kp == 128) {
            rows_to_opT_x3_128(P1, opA, opB, R, lo_off);
          } else {
            rows_to_opT<false, true>(P1, opA, kp, 0, 64, R, lo_off);
            rows_to_opT<false, true>(P1, opB, kp, 64, 64, R, lo_off);
          }
          cx.publish();
          if (tid == 0) {
            for (int hh = 0; hh < 2; ++hh) {
              const uint32_t b0 = smem_u32(hh ? opB : opA);
              for (int j = 0; j < 8; ++j) {
                const int kk = 64 * hh + 8 * j;
                const uint64_t bh = smem_desc(b0 + j * 256, 128, 2048);
                const uint64_t bl = smem_desc(b0 + lo_off + j * 256, 128, 2048);
                mma_ts_tf32(D2, AHI + kk, bh, idesc, hh > 0 || j > 0);
                mma_ts_tf32(D2, AHI + kk, bl, idesc, true);
                mma_ts_tf32(D2, ALO + kk, bh, idesc, true);
              }
            }
            commit(cx.bar_mma);
          }
        } else {
          rows_to_opT<false, false>(P1, opA, kp, 0, 128, R, 0);
          cx.publish();
          if (tid == 0) {
            const uint32_t b0 = smem_u32(opA);
            for (int j = 0; j < 16; ++j)
              mma_ts_tf32(D2, AHI + 8 * j, smem_desc(b0 + j * 256, 128, 4096), idesc, j > 0);
            commit(cx.bar_mma);
          }
        }
        cx.wait_mma();
        cx.issue(opB, scr + (int64_t)(l - 2) * scr_slot, (uint32_t)(128 * kp * 4));   // next layer's Z
        d1_to_rows(D1, P1, kp, K, R, lane_addr, lrow, cgrp);
      } else {
        rows_to_opT<BF16, false>(P1, opB, kp, 0, 128, R, 0);
        cx.publish();
        // dW: D2[128 x kp] = A[128 x 128] . B[kp x 128]^T
        gemm_issue<BF16>(D2, opA, opB, kp, 128, cx.bar_mma);
        d1_to_rows(D1, P1, kp, K, R, lane_addr, lrow, cgrp);   // overlaps the dW MMA
        cx.wait_mma();
        cx.issue(opB, scr + (int64_t)(l - 2) * scr_slot, (uint32_t)(128 * kp * 4));   // next layer's Z
      }
      // flush dW_{l-1} (TMEM lane = output neuron, columns = input neurons) into this CTA's zeroed
      // gradient segment: staged in opA (free after the dW MMAs) as 128 rows of 32 16-byte
      // chunks, chunk j of row n at j ^ (n & 7) (conflict-free writes and reads), then every warp
      // adds whole rows with coalesced vector atomics. One thread owns each address in every
      // tile, so the accumulation order is fixed.
      {
        float4* stage = reinterpret_cast<float4*>(opA);
        const int sw = lrow & 7;
        auto put = [&](int c, const float (&v)[8]) {
          const int j = c >> 2;
          stage[lrow * 32 + (j ^ sw)] = make_float4(v[0], v[1], v[2], v[3]);
          stage[lrow * 32 + ((j + 1) ^ sw)] = make_float4(v[4], v[5], v[6], v[7]);
        };
        for (int c = 8 * cgrp; c < kp; c += 16 * NCG) {   // two column chunks per wait
          float v[8], w[8];
          if (c + 8 * NCG < kp) {
            tmem_ld8x2(D2 + lane_addr + c, D2 + lane_addr + c + 8 * NCG, v, w);
            put(c, v);
            put(c + 8 * NCG, w);
          } else {
            tmem_ld8(D2 + lane_addr + c, v);
            put(c, v);
          }
        }
        __syncthreads();
        float* dW = grad + A.w_off[l - 1];
        for (int n = warp; n < N; n += NTC / 32)
          if (4 * lane < K) {
            const float4 v = stage[n * 32 + (lane ^ (n & 7))];
            red_add4(&dW[(int64_t)n * K + 4 * lane], v.x, v.y, v.z, v.w);
          }
      }
      if constexpr (TMA_A) {
        cx.publish();                         // the flush's reads of opA before the copy below
        if (l - 1 >= 2) wbwd_first(l - 2);    // the next dX GEMM's W^T (K-half 0), during its jets
      } else {
        fence_before();
        __syncthreads();
      }
    }
  }
  __syncthreads();
  if (cur_group >= 0 && tid < Gs->n_outputs)
    A.slot_partial[(int64_t)cta * A.n_slots + Gs->slot_first + tid] += cur_slot[tid];
  fence_before();
  __syncthreads();
  cx.drain();
  if (warp == 0) tmem_dealloc(*tmem_slot, TMA_A ? 512 : 256);
}

// ---- weight packing: every hidden Linear j into forward (N x K) and transposed (K x N) operands.
// Split TF32 packs each operand as two K-halves, each a [hi | lo] pair of K-major blocks.
namespace {
template <bool BF16, bool X3>
__global__ void pack_weights_kernel(const float* __restrict__ params, TcLaunch t) {
  constexpr int ES = BF16 ? 2 : 4;
  const int j = blockIdx.y + 1;   // hidden Linear layers 1..n_layers-2
  const int K = t.width[j], N = t.width[j + 1];
  const int kp = p16(K), np = p16(N);
  const int prob = blockIdx.z;    // every problem's own weights
  const float* W = params + (int64_t)prob * t.n_params + t.w_off[j];
  unsigned char* f = t.wpack + (int64_t)prob * t.wpack_stride + t.fwd_off[j];
  unsigned char* b = t.wpack + (int64_t)prob * t.wpack_stride + t.bwd_off[j];
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < np * kp; e += gridDim.x * blockDim.x) {
    const int n = e / kp, k = e % kp;
    const float v = (n < N && k < K) ? W[(int64_t)n * K + k] : 0.f;
    if (X3) {
      const float hi = to_tf32(v), lo = to_tf32(v - hi);
      const int kh = kp / 2, nh = np / 2;
      // forward operand [np x kp], halves over k
      {
        const int h = k / kh, kk = k - h * kh;
        unsigned char* base = f + (size_t)h * 2 * np * kh * 4;
        *reinterpret_cast<float*>(base + ofs(n, kk, kh, 4)) = hi;
        *reinterpret_cast<float*>(base + (size_t)np * kh * 4 + ofs(n, kk, kh, 4)) = lo;
      }
      // transposed operand [kp x np], halves over n
      {
        const int h = n / nh, nn = n - h * nh;
        unsigned char* base = b + (size_t)h * 2 * kp * nh * 4;
        *reinterpret_cast<float*>(base + ofs(k, nn, nh, 4)) = hi;
        *reinterpret_cast<float*>(base + (size_t)kp * nh * 4 + ofs(k, nn, nh, 4)) = lo;
      }
    } else {
      put<BF16>(f, ofs(n, k, kp, ES), v);
      put<BF16>(b, ofs(k, n, np, ES), v);
    }
  }
}

template <bool BF16, bool X3, int CM>
cudaError_t launch_variant(const FusedArgs& a, const TcLaunch& t, int n_ctas, cudaStream_t s) {
  static bool attr = false;
  const size_t smem = fused_tc_smem_bytes();
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(fused_tc_kernel<BF16, X3, CM>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  if (a.n_layers > 2) {   // pack this step's hidden weights
    pack_weights_kernel<BF16, X3><<<dim3(16, a.n_layers - 2, t.n_problems), 256, 0, s>>>(a.params, t);
    count_launch();
  }
  TcArgs ta{};
  ta.wpack = t.wpack;
  ta.wpack_stride = t.wpack_stride;
  for (int l = 0; l < TDG_MAX_LAYERS; ++l) { ta.wfwd_off[l] = t.fwd_off[l]; ta.wbwd_off[l] = t.bwd_off[l]; }
  ta.err = t.err;
  fused_tc_kernel<BF16, X3, CM><<<n_ctas, NTC, smem, s>>>(a, ta);
  count_launch();
  return cudaGetLastError();
}
}  // namespace

}  // namespace tdg
