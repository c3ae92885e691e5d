// Internal tables shared by the host-side plan builder (tdg_plan.cu) and the kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "../../include/tdg.h"

namespace tdg {

constexpr int NT = 256;            // threads per CTA of the fused kernel
constexpr int RMAX = 128;          // (point, stream) rows per tile
constexpr int LDS = 132;           // row stride (floats) of shared-memory activation tiles
constexpr int SMAX = TDG_MAX_STREAMS;
constexpr int MAX_SITES = TDG_MAX_SITES;
constexpr int MAX_RULES = 6;       // Faa di Bruno terms of one stream (order <= 3 needs 5)
constexpr int MAX_PULL = 160;      // adjoint contributions of one group
constexpr int MAX_TERMS = 32;
constexpr int MAX_FACTORS = 64;
constexpr int MAX_PARTS = 256;
constexpr int MAX_TERM_FACTORS = 4;
constexpr int MAX_OUT = TDG_MAX_DOUT;   // outputs per group row
constexpr int MAX_SLOTS = 1024;    // loss slots of a plan

// H^alpha = sum_rules mult * tanh^(k)(z_base) * prod_{i<k} Z[sub[i]]
struct DevRule {
  int8_t k, mult;
  int8_t sub[3];
  int8_t pad[3];
};

// adjoint: G_Z[beta] += mult * tanh^(kk)(z_base) * prod_{i<n_oth} Z[oth[i]] * G_H[alpha]
struct DevPull {
  int8_t alpha, kk, mult, n_oth;
  int8_t oth[3];
  int8_t pad;
};

struct DevTerm {
  int16_t factor_first, n_factors, output, coeff_array;
  float coeff;
  int16_t coeff_param, pad;   // trainable coefficient index (-1: none)
};

struct DevFactor {
  int16_t part_first, n_parts, var, pad;
  float power;
};

struct DevPart {
  int16_t stream, pad;
  float weight;
};

// Everything the fused kernel needs about one group, copied to shared memory per tile.
struct alignas(16) DevGroup {
  int32_t n_rows, T, S, n_sites;
  int32_t n_outputs, n_terms, problem, slot_first;
  int32_t target_array, row_weight_array;   // row_weight_array: per-row loss weights (-1: none)
  int64_t out_offset;
  float seed_scale[MAX_OUT];              // 2 * loss weight of each output's slot
  int32_t site_points[MAX_SITES];
  float site_off[MAX_SITES][TDG_MAX_DIN];
  int8_t site_nstreams[MAX_SITES];
  int8_t site_streams[MAX_SITES][SMAX];   // row-stream indices of a site, increasing order; [0] = value
  int8_t site_cls[MAX_SITES];             // compile-time jet class of a site (tdg_jetcls.h), -1: tables
  int8_t st_site[SMAX], st_order[SMAX], st_axis[SMAX], st_nrule[SMAX];
  int8_t st_npull[SMAX];
  int16_t st_pull_first[SMAX];
  DevRule rules[SMAX][MAX_RULES];
  DevPull pulls[MAX_PULL];
  DevTerm terms[MAX_TERMS];
  DevFactor factors[MAX_FACTORS];
  DevPart parts[MAX_PARTS];
};

// e / d for 0 <= e < 2^16 and 1 <= d < 2^16 as one multiply-high by m = ceil(2^32 / d) instead of
// a division by a runtime divisor: exact, since the error term e (m d - 2^32) / (d 2^32) stays
// below e / 2^32 < 1 / d. d = 1 passes e through.
struct FastDiv {
  uint32_t m;
  int d;
  __device__ __forceinline__ explicit FastDiv(int d_)
      : m(d_ > 1 ? 0xFFFFFFFFu / (uint32_t)d_ + 1u : 0u), d(d_) {}
  __device__ __forceinline__ int div(int e) const { return d > 1 ? (int)__umulhi((uint32_t)e, m) : e; }
};

// fire-and-forget add of one float to global memory
__device__ __forceinline__ void red_add1(float* dst, float v) {
  asm volatile("red.global.add.f32 [%0], %1;" :: "l"(dst), "f"(v) : "memory");
}

// fire-and-forget vector add of 4 floats to global memory (16-byte aligned)
__device__ __forceinline__ void red_add4(float* dst, float a, float b, float c, float d) {
  asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};"
               :: "l"(dst), "f"(a), "f"(b), "f"(c), "f"(d) : "memory");
}

struct DevTile {
  int32_t group, row0, nvalid, seg;
  int32_t first_in_seg, problem, pad[2];   // problem: the group's parameter set
};

static_assert(sizeof(DevGroup) % 16 == 0, "DevGroup is copied as int4");

struct FusedArgs {
  const DevGroup* groups;
  const DevTile* tiles;
  const int32_t* cta_tile_begin;      // n_ctas + 1
  const float* const* arrays;         // device table of device pointers
  const float* params;                // n_problems x n_params
  int64_t n_params;                   // per problem
  int64_t coeff_off;                  // the trainable coefficients' offset within a problem's params
  int32_t n_coeff;                    // trainable coefficients per problem
  int64_t part_stride;                // floats per gradient segment (n_params rounded up to 4)
  float* partial;                     // n_segments x part_stride
  double* slot_partial;               // n_ctas x n_slots
  int32_t n_slots;
  int32_t do_grad;
  float* outputs;                     // optional
  float* scratch;                     // n_ctas x (n_layers-1) x RMAX x LDS
  int32_t n_layers;
  int32_t width[TDG_MAX_LAYERS + 1];
  int64_t w_off[TDG_MAX_LAYERS], b_off[TDG_MAX_LAYERS];
};

// shared-memory bytes of the fused FP32 kernel
constexpr size_t fused_smem_bytes() {
  return sizeof(float) * (3 * RMAX * LDS + 2 * RMAX * MAX_OUT + RMAX * TDG_MAX_DIN)
         + sizeof(DevGroup) + sizeof(double) * (MAX_SLOTS + NT / 32 * MAX_OUT)
         + sizeof(float) * (NT / 32) * TDG_MAX_COEFF + 64;
}

// the FP32 fused kernel, variant of the main site class cls_main (tdg_fp32_inst.cu)
cudaError_t launch_fused_fp32(const FusedArgs& a, int cls_main, int n_ctas, cudaStream_t s);

// tensor-core path: packed hidden weights (per problem p and hidden Linear j: W_j as an np x kp
// K-major operand at p * wpack_stride + fwd_off[j] and W_j^T as kp x np at p * wpack_stride +
// bwd_off[j], widths padded to 16) and a timeout flag
struct TcLaunch {
  bool bf16;
  bool x3;     // split TF32 (hi*hi + hi*lo + lo*hi)
  int cls_main;   // the site class (besides the value-only class 0) the kernel variant carries
  unsigned char* wpack;
  int64_t wpack_stride;   // bytes of one problem's packed weights
  int n_problems;
  int64_t n_params;       // parameters of one problem (the stride of `params`)
  int64_t fwd_off[TDG_MAX_LAYERS], bwd_off[TDG_MAX_LAYERS];
  int64_t w_off[TDG_MAX_LAYERS];
  int32_t width[TDG_MAX_LAYERS + 1];
  int* err;
};
size_t fused_tc_smem_bytes();

// plain form: one launch per layer operation, activations of every row kept in device memory
struct HostGroupInfo {
  int64_t n_rows;
  int32_t S, problem;
};
struct PlainArgs {
  const DevGroup* groups;           // device
  const HostGroupInfo* ginfo;       // host
  int32_t n_groups;
  const float* const* arrays;
  const float* params;
  float* grad;
  int64_t n_params;
  int64_t coeff_off;                // the trainable coefficients' offset within a problem's params
  int32_t n_coeff;
  int32_t n_problems;
  int32_t n_layers;
  int32_t width[TDG_MAX_LAYERS + 1];
  int64_t w_off[TDG_MAX_LAYERS], b_off[TDG_MAX_LAYERS];
  float* act;                       // Z_l and H_l of every hidden layer of one group
  float* g0;
  float* g1;                        // dL/dH and dL/dZ ping-pong
  float* y;
  float* gy;                        // MLP outputs and their seeds
  double* slot_sum;
  int32_t n_slots;
  const int32_t* slot_problem;
  const double* slot_w;
  const double* slot_wn;
  double* loss;
  float* outputs;
  int32_t do_grad;
};
cudaError_t run_plain(const PlainArgs& a, cudaStream_t s);
cudaError_t launch_fused_tc(const FusedArgs& a, const TcLaunch& t, int n_ctas, cudaStream_t s);
// the tensor-core kernel's variants: launch_tc_<precision>_c<main site class>
#define TDG_TC_FN_(P, C) launch_tc_##P##_c##C
#define TDG_TC_FN(P, C) TDG_TC_FN_(P, C)
#define TDG_TC_DECLARE(P, C) \
  cudaError_t TDG_TC_FN(P, C)(const FusedArgs& a, const TcLaunch& t, int n_ctas, cudaStream_t s);
#define TDG_TC_EACH_CLASS(M, P) M(P, 0) M(P, 1) M(P, 2) M(P, 3) M(P, 4) M(P, 5) M(P, 6) M(P, 7) M(P, 8) M(P, 9) M(P, 10)
TDG_TC_EACH_CLASS(TDG_TC_DECLARE, tf32)
TDG_TC_EACH_CLASS(TDG_TC_DECLARE, bf16)
TDG_TC_EACH_CLASS(TDG_TC_DECLARE, 3x)
#define TDG_F32_FN_(C) launch_fp32_c##C
#define TDG_F32_FN(C) TDG_F32_FN_(C)
#define TDG_F32_DECLARE(P, C) cudaError_t TDG_F32_FN(C)(const FusedArgs& a, int n_ctas, cudaStream_t s);
TDG_TC_EACH_CLASS(TDG_F32_DECLARE, fp32)
cudaError_t launch_bounded_wait_selftest(int max_polls, int* gave_up, cudaStream_t s);
cudaError_t launch_reduce_grad(const float* partial, int64_t part_stride, const int32_t* seg_begin,
                               const int32_t* seg_list, int n_problems, int64_t n_params,
                               float* grad, cudaStream_t s);
cudaError_t launch_reduce_loss(const double* slot_partial, int n_ctas, int n_slots,
                               const int32_t* slot_problem, const double* slot_w,
                               const double* slot_wn, int n_problems, double* loss,
                               cudaStream_t s);
cudaError_t launch_adam(float* p, const float* g, float* m, float* v, float* step, int64_t n,
                        const tdg_adam_desc& hp, cudaStream_t s);
cudaError_t launch_causal_weights(const float* op, int64_t n_rows, int n_eq, int64_t n_t,
                                  float tol, float* w, cudaStream_t s);
cudaError_t launch_gather_rows(const float* src, int64_t n_src, const int64_t* index, int64_t n,
                               int row_len, float* dst, cudaStream_t s);
cudaError_t launch_dot_f64(const float* a, const float* b, int64_t n, double* out,
                           cudaStream_t s);

void count_launch(int n = 1);
// record the message of a failure for tdg_last_error() and return its status
tdg_status record_error(tdg_status st, const char* fmt, ...);

}  // namespace tdg
