// Jet code shared by the fused kernels (FP32 on the CUDA cores and tensor-core): float4
// arithmetic for (point, 4 neurons) tasks, tanh and its derivatives as functions of t = tanh(z),
// and the compile-time site classes of tdg_jetcls.h, whose Faa di Bruno rules fold into
// straight-line code with every stream value of a task in registers.
#pragma once
#include <utility>
#include "tdg_internal.h"
#include "tdg_jetcls.h"

namespace tdg {

namespace {

__device__ __forceinline__ float4 f4mul(float4 a, float4 b) { return make_float4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
__device__ __forceinline__ float4 f4add(float4 a, float4 b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
__device__ __forceinline__ float4 f4scale(float4 a, float c) { return make_float4(a.x * c, a.y * c, a.z * c, a.w * c); }

struct Sig {   // tanh and its derivatives, as functions of t = tanh(z), for 4 neurons
  float4 t, s1, s2, s3, s4;
  __device__ __forceinline__ void make(const float4 z, bool need4) {
    from_t(make_float4(tanhf(z.x), tanhf(z.y), tanhf(z.z), tanhf(z.w)), need4);
  }
  // from t = tanh(z) saved by the forward pass
  __device__ __forceinline__ void from_t(const float4 tv, bool need4) {
    t = tv;
    const float4 tt = f4mul(t, t);
    s1 = make_float4(1.f - tt.x, 1.f - tt.y, 1.f - tt.z, 1.f - tt.w);
    s2 = f4scale(f4mul(t, s1), -2.f);
    s3 = f4mul(s1, make_float4(6.f * tt.x - 2.f, 6.f * tt.y - 2.f, 6.f * tt.z - 2.f, 6.f * tt.w - 2.f));
    s4 = need4 ? f4mul(f4mul(t, s1), make_float4(16.f - 24.f * tt.x, 16.f - 24.f * tt.y,
                                                  16.f - 24.f * tt.z, 16.f - 24.f * tt.w))
               : make_float4(0.f, 0.f, 0.f, 0.f);
  }
  // the k-th derivative; k is the same for every thread of a group's table entry (uniform branch)
  __device__ __forceinline__ float4 sel(int k) const {
    switch (k) {
      case 0: return t;
      case 1: return s1;
      case 2: return s2;
      case 3: return s3;
      default: return s4;
    }
  }
};

__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ void st4(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }

// ---- jet code of the compile-time site classes (tdg_jetcls.h): rules folded into straight-line
// code, every stream value of a (point, 4 neurons) task in registers
template <int C>
__host__ __device__ constexpr jetcls::Rules rules_of() { return jetcls::make_rules(jetcls::kSiteClasses[C]); }

template <typename F, int... I>
__device__ __forceinline__ void sfor_(F& f, std::integer_sequence<int, I...>) {
  (f(std::integral_constant<int, I>{}), ...);
}
template <int N, typename F>
__device__ __forceinline__ void sfor(F&& f) { sfor_(f, std::make_integer_sequence<int, N>{}); }

// run f(integral_constant<C>) for the site class `cls` when it is one this kernel carries: the
// value-only class 0 and the plan's main class CM (each kernel instantiation carries two, which
// keeps its code small); false otherwise (the table-driven code runs)
template <int CM, typename F>
__device__ __forceinline__ bool with_class(int cls, F&& f) {
  if (cls == 0) return f(std::integral_constant<int, 0>{});
  if constexpr (CM > 0) {
    if (cls == CM) return f(std::integral_constant<int, CM>{});
  }
  return false;
}

// H_M = sum_u mult * tanh^(k)(z_0) * prod Z[sub]  (same operation order as the table rules)
template <int C, int M, int NS>
__device__ __forceinline__ float4 cls_rule_sum(const Sig& sg, const float4 (&z)[NS]) {
  float4 h = make_float4(0.f, 0.f, 0.f, 0.f);
  sfor<rules_of<C>().nrule[M]>([&](auto uc) {
    constexpr int U = decltype(uc)::value;
    constexpr int K = rules_of<C>().k[M][U];
    float4 v = f4scale(sg.sel(K), (float)rules_of<C>().mult[M][U]);
    sfor<K>([&](auto fc) { v = f4mul(v, z[rules_of<C>().sub[M][U][decltype(fc)::value]]); });
    h = f4add(h, v);
  });
  return h;
}

}  // namespace

}  // namespace tdg
