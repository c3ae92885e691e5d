// Host side of the C ABI declared in include/tdg.h: validates a problem description, derives the
// per-group tables the kernels interpret (Faa di Bruno rules of the tanh jet and their adjoint,
// the operator program), schedules tiles over persistent CTAs and owns the plan's device memory.
#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "tdg_internal.h"
#include "tdg_jetcls.h"

namespace tdg {

static std::atomic<int64_t> g_launches{0};
void count_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

static thread_local std::string g_error;

static tdg_status fail(tdg_status st, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_error = buf;
  return st;
}

tdg_status record_error(tdg_status st, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_error = buf;
  return st;
}

static tdg_status cuda_fail(cudaError_t e, const char* what) {
  return fail(TDG_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

}  // namespace tdg

using namespace tdg;

struct tdg_plan {
  int device = 0;
  int n_layers = 0;
  int width[TDG_MAX_LAYERS + 1] = {0};
  int64_t w_off[TDG_MAX_LAYERS] = {0}, b_off[TDG_MAX_LAYERS] = {0};
  int64_t n_params = 0, part_stride = 0;
  int64_t coeff_off = 0;   // the trainable coefficients follow the MLP's parameters
  int n_coeff = 0;
  int n_problems = 0, n_slots = 0, n_tiles = 0, n_ctas = 0, n_segments = 0, max_streams = 0;
  int precision = 0, form = 0;
  int cls_main = 0;   // the fused kernels' variant: the site class with the most rows
  double flops_hidden = 0, flops_total = 0;
  std::vector<const float*> arrays;
  std::vector<int64_t> array_len;
  // device memory
  DevGroup* d_groups = nullptr;
  DevTile* d_tiles = nullptr;
  int32_t* d_cta_begin = nullptr;
  const float** d_arrays = nullptr;
  int32_t* d_seg_begin = nullptr;
  int32_t* d_seg_list = nullptr;
  float* d_partial = nullptr;
  double* d_slot_partial = nullptr;
  int32_t* d_slot_problem = nullptr;
  double* d_slot_w = nullptr;
  double* d_slot_wn = nullptr;
  float* d_scratch = nullptr;
  unsigned char* d_wpack = nullptr;
  int* d_err = nullptr;
  // plain form
  std::vector<HostGroupInfo> ginfo;
  float* d_act = nullptr;
  float* d_g0 = nullptr;
  float* d_g1 = nullptr;
  float* d_y = nullptr;
  float* d_gy = nullptr;
  double* d_slot_sum = nullptr;
  int64_t wpack_fwd[TDG_MAX_LAYERS] = {0}, wpack_bwd[TDG_MAX_LAYERS] = {0};
  int64_t wpack_stride = 0;
  int64_t workspace_bytes = 0;
  bool arrays_dirty = false;
};

namespace {

using Key = std::vector<int>;   // sorted axes of a derivative stream

// all set partitions of {0..k-1}, each as a list of blocks
void set_partitions(int k, int i, std::vector<std::vector<int>>& cur,
                    std::vector<std::vector<std::vector<int>>>& out) {
  if (i == k) {
    out.push_back(cur);
    return;
  }
  for (size_t b = 0; b < cur.size(); ++b) {
    cur[b].push_back(i);
    set_partitions(k, i + 1, cur, out);
    cur[b].pop_back();
  }
  cur.push_back({i});
  set_partitions(k, i + 1, cur, out);
  cur.pop_back();
}

struct HostRule {
  int k, mult;
  std::vector<int> sub;   // row-stream indices, sorted
};

template <typename T>
tdg_status dev_upload(tdg_plan* p, T** dst, const T* src, size_t n) {
  size_t bytes = sizeof(T) * std::max<size_t>(n, 1);
  cudaError_t e = cudaMalloc((void**)dst, bytes);
  if (e != cudaSuccess) return fail(TDG_ERR_NOMEM, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
  p->workspace_bytes += bytes;
  if (n) {
    e = cudaMemcpy(*dst, src, sizeof(T) * n, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy");
  }
  return TDG_OK;
}

tdg_status dev_alloc(tdg_plan* p, void** dst, size_t bytes) {
  cudaError_t e = cudaMalloc(dst, std::max<size_t>(bytes, 16));
  if (e != cudaSuccess) return fail(TDG_ERR_NOMEM, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
  p->workspace_bytes += bytes;
  return TDG_OK;
}

void free_plan(tdg_plan* p) {
  void* ptrs[] = {p->d_groups, p->d_tiles, p->d_cta_begin, (void*)p->d_arrays, p->d_seg_begin,
                  p->d_seg_list, p->d_partial, p->d_slot_partial, p->d_slot_problem,
                  p->d_slot_w, p->d_slot_wn, p->d_scratch, p->d_wpack, p->d_err,
                  p->d_act, p->d_g0, p->d_g1, p->d_y, p->d_gy, p->d_slot_sum};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  delete p;
}

// Build the DevGroup of one group description.
// Compile-time jet class of the site whose streams are rows [base, base + ns): the class with the
// same stream list whose folded rules equal the tables just built, else -1 (table-driven code).
int site_class(const DevGroup& G, const std::vector<Key>& keys, int base, int ns) {
  if (ns > jetcls::CS) return -1;
  int ord[jetcls::CS] = {0};
  int ax[jetcls::CS][3] = {{0}};
  for (int m = 0; m < ns; ++m) {
    const Key& k = keys[base + m];
    ord[m] = (int)k.size();
    for (size_t i = 0; i < k.size(); ++i) ax[m][i] = k[i];
  }
  const int c = jetcls::classify(ns, ord, ax);
  if (c < 0) return -1;
  const jetcls::Rules R = jetcls::make_rules(jetcls::kSiteClasses[c]);
  if (R.ns != ns) return -1;
  for (int m = 1; m < ns; ++m) {
    const int s = base + m;
    if (R.nrule[m] != G.st_nrule[s]) return -1;
    for (int u = 0; u < R.nrule[m]; ++u) {
      const DevRule& r = G.rules[s][u];
      if (r.k != R.k[m][u] || r.mult != R.mult[m][u]) return -1;
      for (int i = 0; i < r.k; ++i)
        if (r.sub[i] != base + R.sub[m][u][i]) return -1;
    }
  }
  return c;
}

tdg_status build_group(const tdg_problem_desc& d, const tdg_group_desc& g, int d_in, int d_out,
                       bool tables_only, int max_rows, DevGroup& G, int& S_out) {
  memset(&G, 0, sizeof(G));
  if (g.n_sites < 1 || g.n_sites > MAX_SITES) return fail(TDG_ERR_UNSUPPORTED, "group has %d sites (1..%d)", g.n_sites, MAX_SITES);
  if (g.site_first < 0 || g.site_first + g.n_sites > d.n_sites) return fail(TDG_ERR_INVALID, "site range out of bounds");
  if (g.n_outputs < 1 || g.n_outputs > MAX_OUT) return fail(TDG_ERR_UNSUPPORTED, "group has %d outputs (1..%d)", g.n_outputs, MAX_OUT);
  if (g.n_rows < 1) return fail(TDG_ERR_SHAPE, "group with %d rows", g.n_rows);
  int S = 0;
  std::vector<Key> keys;
  std::vector<int> site_base(g.n_sites);
  for (int q = 0; q < g.n_sites; ++q) {
    const tdg_site_desc& st = d.sites[g.site_first + q];
    if (st.points < 0 || st.points >= d.n_arrays) return fail(TDG_ERR_INVALID, "site points array %d out of range", st.points);
    if (d.array_len[st.points] < (int64_t)g.n_rows * d_in)
      return fail(TDG_ERR_SHAPE, "points array %d holds %lld floats, need %lld", st.points,
                  (long long)d.array_len[st.points], (long long)g.n_rows * d_in);
    if (st.n_streams < 1 || st.stream_first < 0 || st.stream_first + st.n_streams > d.n_streams)
      return fail(TDG_ERR_INVALID, "site stream range out of bounds");
    if (S + st.n_streams > SMAX) return fail(TDG_ERR_UNSUPPORTED, "more than %d streams per row", SMAX);
    site_base[q] = S;
    G.site_points[q] = st.points;
    for (int a = 0; a < TDG_MAX_DIN; ++a) G.site_off[q][a] = st.offset[a];
    G.site_nstreams[q] = (int8_t)st.n_streams;
    std::map<Key, int> index;
    int prev_order = 0;
    for (int m = 0; m < st.n_streams; ++m) {
      const tdg_stream_desc& sd = d.streams[st.stream_first + m];
      if (sd.order < 0 || sd.order > TDG_MAX_ORDER) return fail(TDG_ERR_UNSUPPORTED, "derivative order %d (max %d)", sd.order, TDG_MAX_ORDER);
      if (m == 0 && sd.order != 0) return fail(TDG_ERR_INVALID, "first stream of a site must be the value");
      if (sd.order < prev_order) return fail(TDG_ERR_INVALID, "streams of a site must be sorted by order");
      prev_order = sd.order;
      Key k(sd.axes, sd.axes + sd.order);
      for (int a : k) if (a < 0 || a >= d_in) return fail(TDG_ERR_INVALID, "derivative axis %d out of range", a);
      std::sort(k.begin(), k.end());
      if (index.count(k)) return fail(TDG_ERR_INVALID, "duplicate stream in a site");
      const int s = S + m;
      index[k] = s;
      G.site_streams[q][m] = (int8_t)s;
      G.st_site[s] = (int8_t)q;
      G.st_order[s] = (int8_t)sd.order;
      G.st_axis[s] = (int8_t)(sd.order >= 1 ? k[0] : 0);
      keys.push_back(k);
    }
    // Faa di Bruno rules: d^alpha tanh(z) = sum over set partitions pi of alpha's positions
    // of tanh^(|pi|)(z) * prod_{B in pi} d^B z
    for (int m = 1; m < st.n_streams; ++m) {
      const int s = S + m;
      const Key& ax = keys[s];
      std::vector<std::vector<std::vector<int>>> parts;
      std::vector<std::vector<int>> cur;
      set_partitions((int)ax.size(), 0, cur, parts);
      std::vector<HostRule> rules;
      for (auto& pi : parts) {
        HostRule r{(int)pi.size(), 1, {}};
        for (auto& blk : pi) {
          Key sub;
          for (int i : blk) sub.push_back(ax[i]);
          std::sort(sub.begin(), sub.end());
          auto it = index.find(sub);
          if (it == index.end()) return fail(TDG_ERR_INVALID, "stream set of a site is not closed under sub-derivatives");
          r.sub.push_back(it->second);
        }
        std::sort(r.sub.begin(), r.sub.end());
        bool merged = false;
        for (auto& x : rules)
          if (x.k == r.k && x.sub == r.sub) { x.mult += 1; merged = true; break; }
        if (!merged) rules.push_back(r);
      }
      if ((int)rules.size() > MAX_RULES) return fail(TDG_ERR_UNSUPPORTED, "too many jet rules");
      G.st_nrule[s] = (int8_t)rules.size();
      for (size_t u = 0; u < rules.size(); ++u) {
        G.rules[s][u].k = (int8_t)rules[u].k;
        G.rules[s][u].mult = (int8_t)rules[u].mult;
        for (int i = 0; i < rules[u].k; ++i) G.rules[s][u].sub[i] = (int8_t)rules[u].sub[i];
      }
    }
    G.site_cls[q] = (int8_t)(tables_only ? -1 : site_class(G, keys, S, st.n_streams));
    S += st.n_streams;
  }
  // adjoint pull lists: for each stream beta, every (alpha, rule) term whose derivative wrt Z[beta]
  // is nonzero. Pulls for beta are stored contiguously.
  std::vector<std::vector<DevPull>> pulls(S);
  for (int q = 0; q < g.n_sites; ++q) {
    const int base = site_base[q];
    const int ns = G.site_nstreams[q];
    pulls[base].push_back(DevPull{(int8_t)base, 1, 1, 0, {0, 0, 0}, 0});   // H = tanh(z)
    for (int m = 1; m < ns; ++m) {
      const int a = base + m;
      for (int u = 0; u < G.st_nrule[a]; ++u) {
        const DevRule& r = G.rules[a][u];
        DevPull pb{(int8_t)a, (int8_t)(r.k + 1), r.mult, (int8_t)r.k, {0, 0, 0}, 0};
        for (int i = 0; i < r.k; ++i) pb.oth[i] = r.sub[i];
        pulls[base].push_back(pb);
        for (int i = 0; i < r.k; ++i) {
          DevPull pa{(int8_t)a, r.k, r.mult, (int8_t)(r.k - 1), {0, 0, 0}, 0};
          int c = 0;
          for (int j = 0; j < r.k; ++j)
            if (j != i) pa.oth[c++] = r.sub[j];
          pulls[r.sub[i]].push_back(pa);
        }
      }
    }
  }
  int np = 0;
  for (int s = 0; s < S; ++s) {
    G.st_pull_first[s] = (int16_t)np;
    G.st_npull[s] = (int8_t)pulls[s].size();
    for (auto& x : pulls[s]) {
      if (np >= MAX_PULL) return fail(TDG_ERR_UNSUPPORTED, "jet adjoint table too large");
      G.pulls[np++] = x;
    }
  }
  // operator program
  if (g.n_terms < 1 || g.n_terms > MAX_TERMS) return fail(TDG_ERR_UNSUPPORTED, "group has %d terms (1..%d)", g.n_terms, MAX_TERMS);
  if (g.term_first < 0 || g.term_first + g.n_terms > d.n_terms) return fail(TDG_ERR_INVALID, "term range out of bounds");
  int nf = 0, npart = 0;
  for (int t = 0; t < g.n_terms; ++t) {
    const tdg_term_desc& td = d.terms[g.term_first + t];
    if (td.output < 0 || td.output >= g.n_outputs) return fail(TDG_ERR_INVALID, "term output %d out of range", td.output);
    if (td.n_factors < 1 || td.n_factors > MAX_TERM_FACTORS) return fail(TDG_ERR_UNSUPPORTED, "term with %d factors (1..%d)", td.n_factors, MAX_TERM_FACTORS);
    if (td.factor_first < 0 || td.factor_first + td.n_factors > d.n_factors) return fail(TDG_ERR_INVALID, "factor range out of bounds");
    if (td.coeff_array >= d.n_arrays) return fail(TDG_ERR_INVALID, "coefficient array out of range");
    if (td.coeff_array >= 0 && d.array_len[td.coeff_array] < g.n_rows) return fail(TDG_ERR_SHAPE, "coefficient array shorter than the group");
    DevTerm& T = G.terms[t];
    T.factor_first = (int16_t)nf;
    T.n_factors = (int16_t)td.n_factors;
    T.output = (int16_t)td.output;
    T.coeff_array = (int16_t)td.coeff_array;
    T.coeff = td.coeff;
    if (td.coeff_param >= d.n_coeff_params || td.coeff_param < -1)
      return fail(TDG_ERR_INVALID, "term coefficient parameter %d out of range", td.coeff_param);
    if (td.coeff_param >= 0 && td.coeff_array >= 0)
      return fail(TDG_ERR_INVALID, "a term's coefficient is either trainable or a per-row array");
    T.coeff_param = (int16_t)td.coeff_param;
    for (int f = 0; f < td.n_factors; ++f) {
      const tdg_factor_desc& fd = d.factors[td.factor_first + f];
      if (nf >= MAX_FACTORS) return fail(TDG_ERR_UNSUPPORTED, "too many factors in a group");
      if (fd.var < 0 || fd.var >= d_out) return fail(TDG_ERR_INVALID, "factor var %d out of range", fd.var);
      if (fd.n_parts < 1 || fd.part_first < 0 || fd.part_first + fd.n_parts > d.n_parts) return fail(TDG_ERR_INVALID, "part range out of bounds");
      DevFactor& F = G.factors[nf++];
      F.part_first = (int16_t)npart;
      F.n_parts = (int16_t)fd.n_parts;
      F.var = (int16_t)fd.var;
      F.power = fd.power;
      for (int u = 0; u < fd.n_parts; ++u) {
        const tdg_part_desc& pd = d.parts[fd.part_first + u];
        if (npart >= MAX_PARTS) return fail(TDG_ERR_UNSUPPORTED, "too many parts in a group");
        if (pd.site < 0 || pd.site >= g.n_sites) return fail(TDG_ERR_INVALID, "part site out of range");
        if (pd.stream < 0 || pd.stream >= G.site_nstreams[pd.site]) return fail(TDG_ERR_INVALID, "part stream out of range");
        G.parts[npart].stream = (int16_t)(site_base[pd.site] + pd.stream);
        G.parts[npart].weight = pd.weight;
        ++npart;
      }
    }
  }
  if (g.target_array >= d.n_arrays) return fail(TDG_ERR_INVALID, "target array out of range");
  if (g.target_array >= 0 && d.array_len[g.target_array] < (int64_t)g.n_rows * g.n_outputs)
    return fail(TDG_ERR_SHAPE, "target array shorter than rows x outputs");
  if (g.row_weight_array >= d.n_arrays) return fail(TDG_ERR_INVALID, "row weight array out of range");
  if (g.row_weight_array >= 0 && d.array_len[g.row_weight_array] < g.n_rows)
    return fail(TDG_ERR_SHAPE, "row weight array shorter than the group");
  if (g.slot_first < 0 || g.slot_first + g.n_outputs > d.n_slots) return fail(TDG_ERR_INVALID, "slot range out of bounds");
  for (int o = 0; o < g.n_outputs; ++o) {
    const tdg_slot_desc& sl = d.slots[g.slot_first + o];
    if (sl.problem != g.problem) return fail(TDG_ERR_INVALID, "slot belongs to another problem");
    G.seed_scale[o] = (float)(2.0 * sl.weight);
  }
  G.n_rows = g.n_rows;
  G.S = S;
  G.T = max_rows / S;
  G.n_sites = g.n_sites;
  G.n_outputs = g.n_outputs;
  G.n_terms = g.n_terms;
  G.problem = g.problem;
  G.slot_first = g.slot_first;
  G.target_array = g.target_array;
  G.row_weight_array = g.row_weight_array < 0 ? -1 : g.row_weight_array;
  G.out_offset = g.output_offset;
  S_out = S;
  return TDG_OK;
}

}  // namespace

extern "C" {

int32_t tdg_abi_version(void) { return TDG_ABI_VERSION; }
const char* tdg_last_error(void) { return g_error.c_str(); }
int64_t tdg_launch_count(void) { return g_launches.load(); }

int32_t tdg_site_class(int32_t n_streams, const tdg_stream_desc* streams) {
  if (n_streams < 1 || n_streams > jetcls::CS || !streams) return -1;
  int ord[jetcls::CS] = {0};
  int ax[jetcls::CS][3] = {{0}};
  for (int m = 0; m < n_streams; ++m) {
    if (streams[m].order < 0 || streams[m].order > TDG_MAX_ORDER) return -1;
    ord[m] = streams[m].order;
    for (int i = 0; i < ord[m]; ++i) ax[m][i] = streams[m].axes[i];
    std::sort(ax[m], ax[m] + ord[m]);
  }
  const int c = jetcls::classify(n_streams, ord, ax);
  return c >= 0 && jetcls::make_rules(jetcls::kSiteClasses[c]).ns == n_streams ? c : -1;
}

tdg_status tdg_plan_create(const tdg_problem_desc* desc, tdg_plan** out) {
  return tdg_plan_create_scheduled(desc, nullptr, out);
}

tdg_status tdg_plan_create_scheduled(const tdg_problem_desc* desc, const tdg_schedule* sched,
                                     tdg_plan** out) {
  if (!desc || !out) return fail(TDG_ERR_INVALID, "null argument");
  tdg_schedule sc{RMAX, 0, 0, 0};
  if (sched) {
    sc = *sched;
    if (sc.max_rows < 32 || sc.max_rows > RMAX || sc.max_rows % 32)
      return fail(TDG_ERR_INVALID, "schedule max_rows %d (a multiple of 32, 32..%d)", sc.max_rows, RMAX);
    if (sc.n_ctas < 0) return fail(TDG_ERR_INVALID, "schedule n_ctas %d < 0", sc.n_ctas);
    if (sc.balance < 0 || sc.balance > 1) return fail(TDG_ERR_INVALID, "schedule balance %d (0 or 1)", sc.balance);
  }
  *out = nullptr;
  const tdg_problem_desc& d = *desc;
  const int L = d.mlp.n_layers;
  if (L < 2 || L > TDG_MAX_LAYERS) return fail(TDG_ERR_UNSUPPORTED, "MLP with %d Linear layers (2..%d)", L, TDG_MAX_LAYERS);
  const int d_in = d.mlp.width[0], d_out = d.mlp.width[L];
  if (d_in < 1 || d_in > TDG_MAX_DIN) return fail(TDG_ERR_UNSUPPORTED, "input width %d (1..%d)", d_in, TDG_MAX_DIN);
  if (d_out < 1 || d_out > TDG_MAX_DOUT) return fail(TDG_ERR_UNSUPPORTED, "output width %d (1..%d)", d_out, TDG_MAX_DOUT);
  for (int l = 1; l < L; ++l) {
    // the fused kernels keep a layer's rows and operands on chip and move them in 16-byte
    // vectors; the plain form's per-layer kernels take any width
    const int w = d.mlp.width[l];
    if (d.form == TDG_FORM_PLAIN) {
      if (w < 1 || w > TDG_MAX_WIDTH_PLAIN)
        return fail(TDG_ERR_UNSUPPORTED, "hidden width %d (the plain form takes 1..%d)", w, TDG_MAX_WIDTH_PLAIN);
    } else if (w < 4 || w > TDG_MAX_WIDTH || w % 4) {
      return fail(TDG_ERR_UNSUPPORTED,
                  "hidden width %d (the fused form takes a multiple of 4, <= %d; the plain form any width up to %d)",
                  w, TDG_MAX_WIDTH, TDG_MAX_WIDTH_PLAIN);
    }
  }
  if (d.precision < TDG_PREC_FP32 || d.precision > TDG_PREC_BF16)
    return fail(TDG_ERR_UNSUPPORTED, "precision %d not built", d.precision);
  if (d.form != TDG_FORM_FUSED && d.form != TDG_FORM_PLAIN) return fail(TDG_ERR_UNSUPPORTED, "form %d not built", d.form);
  if (d.form == TDG_FORM_PLAIN && d.precision != TDG_PREC_FP32)
    return fail(TDG_ERR_UNSUPPORTED, "the plain form computes in FP32 only");
  if (d.n_problems < 1) return fail(TDG_ERR_INVALID, "n_problems < 1");
  if (d.n_groups < 1) return fail(TDG_ERR_INVALID, "no groups");
  if (d.n_slots < 1 || d.n_slots > MAX_SLOTS) return fail(TDG_ERR_UNSUPPORTED, "%d loss slots (1..%d)", d.n_slots, MAX_SLOTS);
  if (d.n_arrays < 1 || !d.arrays || !d.array_len) return fail(TDG_ERR_INVALID, "no arrays");
  for (int i = 0; i < d.n_arrays; ++i)
    if (!d.arrays[i] && d.array_len[i] > 0) return fail(TDG_ERR_INVALID, "array %d is null", i);

  tdg_plan* p = new tdg_plan();
  cudaError_t ce = cudaGetDevice(&p->device);
  if (ce != cudaSuccess) { free_plan(p); return cuda_fail(ce, "cudaGetDevice"); }
  p->n_layers = L;
  for (int l = 0; l <= L; ++l) p->width[l] = d.mlp.width[l];
  int64_t off = 0;
  for (int l = 0; l < L; ++l) {
    p->w_off[l] = off;
    off += (int64_t)d.mlp.width[l] * d.mlp.width[l + 1];
    p->b_off[l] = off;
    off += d.mlp.width[l + 1];
  }
  if (d.n_coeff_params < 0 || d.n_coeff_params > TDG_MAX_COEFF) {
    free_plan(p);
    return fail(TDG_ERR_UNSUPPORTED, "%d trainable coefficients (0..%d)", d.n_coeff_params, TDG_MAX_COEFF);
  }
  p->coeff_off = off;
  p->n_coeff = d.n_coeff_params;
  off += d.n_coeff_params;
  p->n_params = off;
  p->part_stride = (off + 3) / 4 * 4;
  p->n_problems = d.n_problems;
  p->n_slots = d.n_slots;
  p->precision = d.precision;
  p->form = d.form;
  p->arrays.assign(d.arrays, d.arrays + d.n_arrays);
  p->array_len.assign(d.array_len, d.array_len + d.n_arrays);

  // TDG_JET_TABLES=1 runs every site through the table-driven jet code (to compare both codes)
  const char* jt = std::getenv("TDG_JET_TABLES");
  const bool tables_only = jt && jt[0] == '1';
  std::vector<DevGroup> groups(d.n_groups);
  std::vector<DevTile> tiles;
  double hidden_pairs = 0, all_pairs = 0;
  for (int l = 1; l < L - 1; ++l) hidden_pairs += (double)d.mlp.width[l] * d.mlp.width[l + 1];
  for (int l = 0; l < L; ++l) all_pairs += (double)d.mlp.width[l] * d.mlp.width[l + 1];
  for (int gi = 0; gi < d.n_groups; ++gi) {
    const tdg_group_desc& g = d.groups[gi];
    if (g.problem < 0 || g.problem >= d.n_problems) { free_plan(p); return fail(TDG_ERR_INVALID, "group problem out of range"); }
    int S = 0;
    tdg_status st = build_group(d, g, d_in, d_out, tables_only, sc.max_rows, groups[gi], S);
    if (st != TDG_OK) { free_plan(p); return st; }
    if (sc.max_rows / S < 1) {
      free_plan(p);
      return fail(TDG_ERR_INVALID, "schedule max_rows %d holds no point of a %d-stream group", sc.max_rows, S);
    }
    p->max_streams = std::max(p->max_streams, S);
    p->ginfo.push_back(HostGroupInfo{g.n_rows, S, g.problem});
    const int T = sc.max_rows / S;
    for (int r0 = 0; r0 < g.n_rows; r0 += T)
      tiles.push_back(DevTile{gi, r0, std::min(T, g.n_rows - r0), 0, 0, g.problem, {0, 0}});
    p->flops_hidden += 3.0 * 2.0 * (double)g.n_rows * S * hidden_pairs;
    p->flops_total += 3.0 * 2.0 * (double)g.n_rows * S * all_pairs;
  }
  // the fused kernels' variant: besides the value-only class, it carries the compile-time jets
  // of one site class, the one covering the most rows (other sites run the tables)
  {
    std::vector<int64_t> rows_of_class(jetcls::N_CLASSES, 0);
    for (int gi = 0; gi < d.n_groups; ++gi)
      for (int q = 0; q < groups[gi].n_sites; ++q) {
        const int c = groups[gi].site_cls[q];
        if (c > 0) rows_of_class[c] += (int64_t)d.groups[gi].n_rows * groups[gi].site_nstreams[q];
      }
    for (int c = 1; c < jetcls::N_CLASSES; ++c)
      if (rows_of_class[c] > rows_of_class[p->cls_main]) p->cls_main = c;
  }
  // contiguous partition of the tile list (in group order) over the persistent CTAs, one per SM
  // by default: equal tile counts, or (balance 1) equal estimated work, each tile weighing a fixed
  // share for its layer-by-layer synchronisation plus its filled (stream, point) rows
  int sms = 0;
  ce = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device);
  if (ce != cudaSuccess) { free_plan(p); return cuda_fail(ce, "cudaDeviceGetAttribute"); }
  const int n_tiles = (int)tiles.size();
  const int max_ctas = sc.n_ctas > 0 ? std::min(sc.n_ctas, sms) : sms;
  const int n_ctas = std::max(1, std::min(n_tiles, max_ctas));
  std::vector<int32_t> cta_begin(n_ctas + 1);
  if (sc.balance == 0) {
    for (int c = 0; c <= n_ctas; ++c) cta_begin[c] = (int32_t)((int64_t)n_tiles * c / n_ctas);
  } else {
    std::vector<double> prefix(n_tiles + 1, 0.0);
    for (int t = 0; t < n_tiles; ++t)
      prefix[t + 1] = prefix[t] + 1.0 + (double)tiles[t].nvalid * groups[tiles[t].group].S / RMAX;
    cta_begin[0] = 0;
    int t = 0;
    for (int c = 1; c < n_ctas; ++c) {
      const double target = prefix[n_tiles] * c / n_ctas;
      while (t < n_tiles && prefix[t + 1] <= target) ++t;
      // at least one tile per CTA before and after this cut
      t = std::max(t, (int)cta_begin[c - 1] + 1);
      t = std::min(t, n_tiles - (n_ctas - c));
      cta_begin[c] = t;
    }
    cta_begin[n_ctas] = n_tiles;
  }
  // segments: one per (CTA, problem) pair, in CTA order
  std::vector<std::vector<int32_t>> segs_of(d.n_problems);
  int n_seg = 0;
  for (int c = 0; c < n_ctas; ++c) {
    std::map<int, int> seg_of_problem;
    for (int t = cta_begin[c]; t < cta_begin[c + 1]; ++t) {
      const int prob = groups[tiles[t].group].problem;
      auto it = seg_of_problem.find(prob);
      if (it == seg_of_problem.end()) {
        seg_of_problem[prob] = n_seg;
        segs_of[prob].push_back(n_seg);
        tiles[t].seg = n_seg++;
        tiles[t].first_in_seg = 1;
      } else {
        tiles[t].seg = it->second;
      }
    }
  }
  std::vector<int32_t> seg_begin(d.n_problems + 1, 0), seg_list;
  for (int q = 0; q < d.n_problems; ++q) {
    if (segs_of[q].empty()) { free_plan(p); return fail(TDG_ERR_INVALID, "problem %d has no rows", q); }
    seg_begin[q + 1] = seg_begin[q] + (int)segs_of[q].size();
    seg_list.insert(seg_list.end(), segs_of[q].begin(), segs_of[q].end());
  }
  std::vector<int32_t> slot_problem(d.n_slots);
  std::vector<double> slot_w(d.n_slots), slot_wn(d.n_slots);
  for (int s = 0; s < d.n_slots; ++s) {
    if (d.slots[s].problem < 0 || d.slots[s].problem >= d.n_problems) { free_plan(p); return fail(TDG_ERR_INVALID, "slot problem out of range"); }
    slot_problem[s] = d.slots[s].problem;
    slot_w[s] = d.slots[s].weight;
    slot_wn[s] = d.slots[s].weight_normalized;
  }
  p->n_tiles = n_tiles;
  p->n_ctas = n_ctas;
  p->n_segments = n_seg;

  tdg_status st = TDG_OK;
  if ((st = dev_upload(p, &p->d_groups, groups.data(), groups.size())) ||
      (st = dev_upload(p, &p->d_tiles, tiles.data(), tiles.size())) ||
      (st = dev_upload(p, &p->d_cta_begin, cta_begin.data(), cta_begin.size())) ||
      (st = dev_upload(p, (const float***)&p->d_arrays, p->arrays.data(), p->arrays.size())) ||
      (st = dev_upload(p, &p->d_seg_begin, seg_begin.data(), seg_begin.size())) ||
      (st = dev_upload(p, &p->d_seg_list, seg_list.data(), seg_list.size())) ||
      (st = dev_upload(p, &p->d_slot_problem, slot_problem.data(), slot_problem.size())) ||
      (st = dev_upload(p, &p->d_slot_w, slot_w.data(), slot_w.size())) ||
      (st = dev_upload(p, &p->d_slot_wn, slot_wn.data(), slot_wn.size())) ||
      (st = dev_alloc(p, (void**)&p->d_partial, sizeof(float) * p->part_stride * n_seg)) ||
      (st = dev_alloc(p, (void**)&p->d_slot_partial, sizeof(double) * (size_t)n_ctas * d.n_slots)) ||
      (st = dev_alloc(p, (void**)&p->d_scratch, sizeof(float) * (size_t)n_ctas * (L - 1) * RMAX * LDS)) ||
      (st = dev_alloc(p, (void**)&p->d_err, sizeof(int)))) {
    free_plan(p);
    return st;
  }
  if (cudaMemset(p->d_err, 0, sizeof(int)) != cudaSuccess) { free_plan(p); return fail(TDG_ERR_CUDA, "cudaMemset"); }
  if (d.form == TDG_FORM_PLAIN) {
    int64_t rows_max = 0, wsum = 0, wmax = 0;
    for (auto& gi : p->ginfo) rows_max = std::max<int64_t>(rows_max, gi.n_rows * gi.S);
    for (int l = 1; l < L; ++l) { wsum += 2 * d.mlp.width[l]; wmax = std::max<int64_t>(wmax, d.mlp.width[l]); }
    if ((st = dev_alloc(p, (void**)&p->d_act, sizeof(float) * rows_max * wsum)) ||
        (st = dev_alloc(p, (void**)&p->d_g0, sizeof(float) * rows_max * wmax)) ||
        (st = dev_alloc(p, (void**)&p->d_g1, sizeof(float) * rows_max * wmax)) ||
        (st = dev_alloc(p, (void**)&p->d_y, sizeof(float) * rows_max * d_out)) ||
        (st = dev_alloc(p, (void**)&p->d_gy, sizeof(float) * rows_max * d_out)) ||
        (st = dev_alloc(p, (void**)&p->d_slot_sum, sizeof(double) * d.n_slots))) {
      free_plan(p);
      return st;
    }
  }
  if (d.precision != TDG_PREC_FP32) {
    // packed hidden weights for the tensor-core kernel: forward and transposed operand per layer
    // element bytes; split TF32 stores a hi and a lo value per element
    const int es = d.precision == TDG_PREC_BF16 ? 2 : d.precision == TDG_PREC_3XTF32 ? 8 : 4;
    int64_t off = 0;
    for (int j = 1; j < L - 1; ++j) {
      const int64_t kp = (d.mlp.width[j] + 15) / 16 * 16, np = (d.mlp.width[j + 1] + 15) / 16 * 16;
      p->wpack_fwd[j] = off;
      off += np * kp * es;
      p->wpack_bwd[j] = off;
      off += np * kp * es;
    }
    p->wpack_stride = off;   // every problem has its own weights
    if ((st = dev_alloc(p, (void**)&p->d_wpack, (size_t)std::max<int64_t>(off * d.n_problems, 16)))) {
      free_plan(p);
      return st;
    }
  }
  *out = p;
  return TDG_OK;
}

tdg_status tdg_plan_destroy(tdg_plan* plan) {
  if (plan) free_plan(plan);
  return TDG_OK;
}

tdg_status tdg_plan_get_info(const tdg_plan* p, tdg_plan_info* info) {
  if (!p || !info) return fail(TDG_ERR_INVALID, "null argument");
  info->n_params = p->n_params;
  info->workspace_bytes = p->workspace_bytes;
  info->n_tiles = p->n_tiles;
  info->n_ctas = p->n_ctas;
  info->n_segments = p->n_segments;
  info->max_streams = p->max_streams;
  info->flops_hidden = p->flops_hidden;
  info->flops_total = p->flops_total;
  return TDG_OK;
}

tdg_status tdg_plan_set_array(tdg_plan* p, int32_t index, const float* dev_ptr, int64_t n) {
  if (!p) return fail(TDG_ERR_INVALID, "null plan");
  if (index < 0 || index >= (int)p->arrays.size()) return fail(TDG_ERR_INVALID, "array index %d out of range", index);
  if (n != p->array_len[index]) return fail(TDG_ERR_SHAPE, "array %d: length %lld, plan expects %lld", index, (long long)n, (long long)p->array_len[index]);
  if (!dev_ptr) return fail(TDG_ERR_INVALID, "null array pointer");
  if (p->arrays[index] == dev_ptr) return TDG_OK;
  p->arrays[index] = dev_ptr;
  cudaError_t e = cudaMemcpy(p->d_arrays + index, &p->arrays[index], sizeof(float*), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy");
  return TDG_OK;
}

static tdg_status run(tdg_plan* p, const float* params, float* grad, double* loss, float* outputs,
                      tdg_stream_t stream, bool do_grad) {
  if (!p) return fail(TDG_ERR_INVALID, "null plan");
  if (!params || !loss || (do_grad && !grad)) return fail(TDG_ERR_INVALID, "null device pointer");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  FusedArgs a{};
  a.groups = p->d_groups;
  a.tiles = p->d_tiles;
  a.cta_tile_begin = p->d_cta_begin;
  a.arrays = p->d_arrays;
  a.params = params;
  a.n_params = p->n_params;
  a.coeff_off = p->coeff_off;
  a.n_coeff = p->n_coeff;
  a.part_stride = p->part_stride;
  a.partial = p->d_partial;
  a.slot_partial = p->d_slot_partial;
  a.n_slots = p->n_slots;
  a.do_grad = do_grad ? 1 : 0;
  a.outputs = outputs;
  a.scratch = p->d_scratch;
  a.n_layers = p->n_layers;
  for (int l = 0; l <= p->n_layers; ++l) a.width[l] = p->width[l];
  for (int l = 0; l < p->n_layers; ++l) { a.w_off[l] = p->w_off[l]; a.b_off[l] = p->b_off[l]; }
  cudaError_t e;
  if (p->form == TDG_FORM_PLAIN) {
    PlainArgs pa{};
    pa.groups = p->d_groups;
    pa.ginfo = p->ginfo.data();
    pa.n_groups = (int)p->ginfo.size();
    pa.arrays = p->d_arrays;
    pa.params = params;
    pa.grad = grad;
    pa.n_params = p->n_params;
    pa.coeff_off = p->coeff_off;
    pa.n_coeff = p->n_coeff;
    pa.n_problems = p->n_problems;
    pa.n_layers = p->n_layers;
    for (int l = 0; l <= p->n_layers; ++l) pa.width[l] = p->width[l];
    for (int l = 0; l < p->n_layers; ++l) { pa.w_off[l] = p->w_off[l]; pa.b_off[l] = p->b_off[l]; }
    pa.act = p->d_act; pa.g0 = p->d_g0; pa.g1 = p->d_g1; pa.y = p->d_y; pa.gy = p->d_gy;
    pa.slot_sum = p->d_slot_sum;
    pa.n_slots = p->n_slots;
    pa.slot_problem = p->d_slot_problem;
    pa.slot_w = p->d_slot_w;
    pa.slot_wn = p->d_slot_wn;
    pa.loss = loss;
    pa.outputs = outputs;
    pa.do_grad = do_grad ? 1 : 0;
    e = run_plain(pa, s);
    if (e != cudaSuccess) return cuda_fail(e, "plain form launch");
    return TDG_OK;
  }
  if (p->precision == TDG_PREC_FP32) {
    e = launch_fused_fp32(a, p->cls_main, p->n_ctas, s);
  } else {
    TcLaunch t{};
    t.bf16 = p->precision == TDG_PREC_BF16;
    t.x3 = p->precision == TDG_PREC_3XTF32;
    t.cls_main = p->cls_main;
    t.wpack = p->d_wpack;
    t.wpack_stride = p->wpack_stride;
    t.n_problems = p->n_problems;
    t.n_params = p->n_params;
    for (int l = 0; l < TDG_MAX_LAYERS; ++l) {
      t.fwd_off[l] = p->wpack_fwd[l];
      t.bwd_off[l] = p->wpack_bwd[l];
      t.w_off[l] = p->w_off[l];
    }
    for (int l = 0; l <= p->n_layers; ++l) t.width[l] = p->width[l];
    t.err = p->d_err;
    if (do_grad) {   // the tensor-core kernel accumulates hidden dW with atomic adds
      e = cudaMemsetAsync(p->d_partial, 0, sizeof(float) * p->part_stride * p->n_segments, s);
      if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync");
    }
    e = launch_fused_tc(a, t, p->n_ctas, s);
  }
  if (e != cudaSuccess) return cuda_fail(e, "fused kernel launch");
  if (do_grad) {
    e = launch_reduce_grad(p->d_partial, p->part_stride, p->d_seg_begin, p->d_seg_list,
                           p->n_problems, p->n_params, grad, s);
    if (e != cudaSuccess) return cuda_fail(e, "gradient reduction launch");
  }
  e = launch_reduce_loss(p->d_slot_partial, p->n_ctas, p->n_slots, p->d_slot_problem, p->d_slot_w,
                         p->d_slot_wn, p->n_problems, loss, s);
  if (e != cudaSuccess) return cuda_fail(e, "loss reduction launch");
  return TDG_OK;
}

tdg_status tdg_loss(tdg_plan* p, const float* params, double* loss, float* outputs,
                    tdg_stream_t stream) {
  return run(p, params, nullptr, loss, outputs, stream, false);
}

tdg_status tdg_loss_grad(tdg_plan* p, const float* params, float* grad, double* loss,
                         float* outputs, tdg_stream_t stream) {
  return run(p, params, grad, loss, outputs, stream, true);
}

tdg_status tdg_plan_sync_status(tdg_plan* p) {
  if (!p) return fail(TDG_ERR_INVALID, "null plan");
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceSynchronize");
  int flag = 0;
  e = cudaMemcpy(&flag, p->d_err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy");
  if (flag) return fail(TDG_ERR_TIMEOUT, "a bounded device wait gave up (code %d)", flag);
  return TDG_OK;
}

tdg_status tdg_selftest_bounded_wait(int32_t max_polls) {
  if (max_polls < 1) return fail(TDG_ERR_INVALID, "max_polls < 1");
  int* flag = nullptr;
  cudaError_t e = cudaMalloc(&flag, sizeof(int));
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
  int gave_up = -1;
  e = launch_bounded_wait_selftest(max_polls, flag, nullptr);
  if (e == cudaSuccess) e = cudaMemcpy(&gave_up, flag, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(flag);
  if (e != cudaSuccess) return cuda_fail(e, "bounded wait self-test");
  if (gave_up == 1) return fail(TDG_ERR_TIMEOUT, "bounded wait gave up after %d polls", max_polls);
  return fail(TDG_ERR_INVALID, "bounded wait self-test: the wait completed unexpectedly");
}

tdg_status tdg_adam_step(float* params, const float* grad, float* exp_avg, float* exp_avg_sq,
                         float* step, int64_t n, const tdg_adam_desc* hp, tdg_stream_t stream) {
  if (!params || !grad || !exp_avg || !exp_avg_sq || !step || !hp) return fail(TDG_ERR_INVALID, "null argument");
  if (n < 0) return fail(TDG_ERR_SHAPE, "negative length");
  if (n == 0) return TDG_OK;
  cudaError_t e = launch_adam(params, grad, exp_avg, exp_avg_sq, step, n, *hp,
                              reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "adam launch");
  return TDG_OK;
}

tdg_status tdg_causal_weights(const float* op, int64_t n_rows, int32_t n_eq, int64_t n_t, float tol,
                              float* w, tdg_stream_t stream) {
  if (!op || !w) return fail(TDG_ERR_INVALID, "null argument");
  if (n_rows < 1 || n_eq < 1 || n_t < 1 || n_rows % n_t != 0)
    return fail(TDG_ERR_SHAPE, "causal weights: %lld rows do not form %lld time slices", (long long)n_rows,
                (long long)n_t);
  cudaError_t e = launch_causal_weights(op, n_rows, n_eq, n_t, tol, w, reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "causal weights launch");
  return TDG_OK;
}

tdg_status tdg_gather_rows(const float* src, int64_t n_src, const int64_t* index, int64_t n, int32_t row_len,
                           float* dst, tdg_stream_t stream) {
  if (n < 0 || n_src < 0 || row_len < 1) return fail(TDG_ERR_SHAPE, "gather: bad sizes");
  if (n == 0) return TDG_OK;
  if (!src || !index || !dst) return fail(TDG_ERR_INVALID, "null argument");
  cudaError_t e = launch_gather_rows(src, n_src, index, n, row_len, dst, reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "gather launch");
  return TDG_OK;
}

tdg_status tdg_dot_f64(const float* a, const float* b, int64_t n, double* out, tdg_stream_t stream) {
  if (!a || !b || !out) return fail(TDG_ERR_INVALID, "null argument");
  if (n < 0) return fail(TDG_ERR_SHAPE, "negative length");
  cudaError_t e = launch_dot_f64(a, b, n, out, reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "dot launch");
  return TDG_OK;
}

}  // extern "C"
