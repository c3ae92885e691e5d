// Compile-time site classes of the tanh-jet code.
//
// A site evaluates the network at one point set and carries derivative streams, each a sorted
// multiset of input axes (the value stream is the empty set). The streams of a site are kept in
// canonical order: by derivative order, then lexicographically (the order the lowering emits,
// closed under sub-derivatives). For the layouts listed in kSiteClasses the kernels run jet code
// whose Faa di Bruno rules are folded at compile time (every stream value held in registers, no
// table walk); every other layout runs the table-driven code. The host tags each site with its
// class index (or -1) when it builds the group tables.
#pragma once

namespace tdg {
namespace jetcls {

constexpr int CS = 8;      // streams of a classed site
constexpr int CR = 6;      // rules of one stream (order <= 3 needs 5)

struct SiteClass {
  int ns;
  int ord[CS];
  int ax[CS][3];
};

// Rules of every stream m >= 1: H_m = sum_u mult * tanh^(k)(z_0) * prod_{i<k} Z[sub[i]].
struct Rules {
  int ns;
  int maxk;                  // largest k of any rule (tanh derivatives the forward needs)
  int nrule[CS];
  int k[CS][CR];
  int mult[CS][CR];
  int sub[CS][CR][3];
};

// The classed layouts. Axis 0 and 1 are the first two input coordinates.
constexpr int N_CLASSES = 11;
constexpr SiteClass kSiteClasses[N_CLASSES] = {
    {1, {0}, {}},                                                     // u
    {2, {0, 1}, {{}, {0}}},                                           // u, u_0
    {2, {0, 1}, {{}, {1}}},                                           // u, u_1
    {3, {0, 1, 1}, {{}, {0}, {1}}},                                   // u, u_0, u_1
    {3, {0, 1, 2}, {{}, {0}, {0, 0}}},                                // u, u_0, u_00
    {4, {0, 1, 1, 2}, {{}, {0}, {1}, {0, 0}}},                        // + u_1 (Burgers-like)
    {4, {0, 1, 1, 2}, {{}, {0}, {1}, {1, 1}}},
    {5, {0, 1, 1, 2, 2}, {{}, {0}, {1}, {0, 0}, {1, 1}}},             // Laplacian / Navier-Stokes
    {5, {0, 1, 1, 2, 3}, {{}, {0}, {1}, {0, 0}, {0, 0, 0}}},          // third order in axis 0
    {5, {0, 1, 1, 2, 3}, {{}, {0}, {1}, {1, 1}, {1, 1, 1}}},
    {6, {0, 1, 1, 2, 2, 2}, {{}, {0}, {1}, {0, 0}, {0, 1}, {1, 1}}},  // full second order in 2-D
};

__host__ __device__ constexpr int find_stream(const SiteClass& c, int ord, const int* ax) {
  for (int m = 0; m < c.ns; ++m) {
    if (c.ord[m] != ord) continue;
    bool same = true;
    for (int i = 0; i < ord; ++i) same = same && c.ax[m][i] == ax[i];
    if (same) return m;
  }
  return -1;
}

// Set partitions of up to 3 positions as restricted growth strings (block label per position).
__host__ __device__ constexpr int n_partitions(int ord) { return ord == 1 ? 1 : ord == 2 ? 2 : 5; }
__host__ __device__ constexpr int partition_label(int ord, int pi, int pos) {
  // order 2: 00, 01; order 3: 000, 001, 010, 011, 012
  return ord == 1 ? 0
       : ord == 2 ? (pi == 0 ? 0 : pos)
       : (pi == 0 ? 0
          : pi == 1 ? (pos == 2 ? 1 : 0)
          : pi == 2 ? (pos == 1 ? 1 : 0)
          : pi == 3 ? (pos == 0 ? 0 : 1)
          : pos);
}

// Faa di Bruno: d^alpha tanh(z) = sum over set partitions pi of alpha's positions of
// tanh^(|pi|)(z) * prod_{B in pi} d^B z; equal (k, sorted sub-stream) terms merged into `mult`.
// A layout that is not closed under sub-derivatives yields ns = 0.
__host__ __device__ constexpr Rules make_rules(const SiteClass& c) {
  Rules R{};
  R.ns = c.ns;
  R.maxk = 1;
  for (int m = 1; m < c.ns; ++m) {
    const int o = c.ord[m];
    for (int pi = 0; pi < n_partitions(o); ++pi) {
      int k = 0;
      for (int pos = 0; pos < o; ++pos) {
        const int lb = partition_label(o, pi, pos);
        if (lb + 1 > k) k = lb + 1;
      }
      int sub[3] = {0, 0, 0};
      for (int b = 0; b < k; ++b) {
        int bax[3] = {0, 0, 0};
        int bo = 0;
        for (int pos = 0; pos < o; ++pos)
          if (partition_label(o, pi, pos) == b) bax[bo++] = c.ax[m][pos];
        for (int i = 1; i < bo; ++i)       // sort the block's axes
          for (int j = i; j > 0 && bax[j - 1] > bax[j]; --j) {
            const int t = bax[j]; bax[j] = bax[j - 1]; bax[j - 1] = t;
          }
        const int s = find_stream(c, bo, bax);
        if (s < 0) { R.ns = 0; return R; }
        sub[b] = s;
      }
      for (int i = 1; i < k; ++i)          // sort the sub-streams
        for (int j = i; j > 0 && sub[j - 1] > sub[j]; --j) {
          const int t = sub[j]; sub[j] = sub[j - 1]; sub[j - 1] = t;
        }
      bool merged = false;
      for (int u = 0; u < R.nrule[m] && !merged; ++u) {
        bool same = R.k[m][u] == k;
        for (int i = 0; i < k; ++i) same = same && R.sub[m][u][i] == sub[i];
        if (same) { R.mult[m][u] += 1; merged = true; }
      }
      if (!merged) {
        const int u = R.nrule[m]++;
        R.k[m][u] = k;
        R.mult[m][u] = 1;
        for (int i = 0; i < 3; ++i) R.sub[m][u][i] = sub[i];
      }
      if (k > R.maxk) R.maxk = k;
    }
  }
  return R;
}

// Class of a site given its streams (orders and sorted axes, canonical order), or -1.
inline int classify(int ns, const int* ord, const int (*ax)[3]) {
  for (int c = 0; c < N_CLASSES; ++c) {
    const SiteClass& sc = kSiteClasses[c];
    if (sc.ns != ns) continue;
    bool same = true;
    for (int m = 0; m < ns && same; ++m) {
      same = sc.ord[m] == ord[m];
      for (int i = 0; i < ord[m] && same; ++i) same = sc.ax[m][i] == ax[m][i];
    }
    if (same) return c;
  }
  return -1;
}

}  // namespace jetcls
}  // namespace tdg
