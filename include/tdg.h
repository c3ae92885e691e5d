/*
 * tdg.h - C ABI of the GB300 training hot path for TEDEouS-style PINN problems.
 *
 * One call evaluates, for a tanh MLP, the residual of a differential operator and the boundary
 * conditions at all collocation points, the weighted MSE loss, and the gradient of that loss with
 * respect to every MLP parameter. The problem arrives as a flat, plain-old-data description
 * (groups of points, evaluation sites, derivative streams and an operator program), so the same
 * kernels serve the reference's 'NN' finite-difference mode and its 'autograd' mode.
 *
 * Reference interfaces these entry points replace (paths inside the TEDEouS project):
 *   tdg_plan_create / tdg_plan_destroy
 *       Solution.__init__ preparation: tedeous/solution.py:23-88 (Operator, Bounds, Losses built
 *       once per compile); the derivative strategy chosen by Derivative.set_strategy
 *       tedeous/derivative.py:347-363.
 *   tdg_loss
 *       Solution.evaluate(save_graph=False): tedeous/solution.py:129-168 -> Operator.operator_compute
 *       tedeous/eval.py:223-232, Bounds.apply_bcs tedeous/eval.py:433-461,
 *       Losses.compute tedeous/losses.py:230-263.
 *   tdg_loss_grad
 *       Solution.evaluate() followed by loss.backward() inside Closure._closure:
 *       tedeous/optimizers/closure.py:49-64.
 *   tdg_adam_step
 *       the optimizer.step() of torch.optim.Adam selected by Optimizer.optimizer_choice:
 *       tedeous/optimizers/optimizer.py:44-51.
 *   tdg_dot_f64
 *       the dot products of the L-BFGS two-loop recursion (torch.optim.LBFGS selected at
 *       tedeous/optimizers/optimizer.py:50-51), computed in FP64.
 *   tdg_causal_weights
 *       the time weights of the causal loss, Losses._causal_loss: tedeous/losses.py:137-182.
 *   tdg_gather_rows
 *       the mini-batch of collocation points drawn by the DataLoader of Operator:
 *       tedeous/eval.py:119-144 (_pde_compute :172-183).
 *
 * Conventions: every pointer passed to a compute entry point is a device pointer owned by the
 * caller; nothing here frees caller memory. Calls are asynchronous on the given stream and never
 * synchronise the host. A plan is not thread safe: use one plan per stream. Errors are returned
 * as tdg_status codes and the message of the last failure on the calling thread is available
 * from tdg_last_error(). No C++ exception crosses this boundary.
 */
#ifndef TDG_H_
#define TDG_H_

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TDG_ABI_VERSION 3

#define TDG_MAX_LAYERS 12      /* Linear layers of the MLP */
#define TDG_MAX_DIN 4          /* input coordinates per point */
#define TDG_MAX_DOUT 8         /* MLP outputs (dependent variables) */
#define TDG_MAX_WIDTH 128      /* hidden width of the fused forms (a multiple of 4) */
#define TDG_MAX_WIDTH_PLAIN 4096 /* hidden width of the plain form (any width) */
#define TDG_MAX_ORDER 3        /* derivative order of one stream */
#define TDG_MAX_STREAMS 16     /* (site, stream) pairs per row */
#define TDG_MAX_SITES 16       /* evaluation sites per row */
#define TDG_MAX_COEFF 16       /* trainable equation coefficients per problem */

typedef enum {
  TDG_OK = 0,
  TDG_ERR_INVALID = 1,      /* malformed description or argument */
  TDG_ERR_UNSUPPORTED = 2,  /* a feature outside what the kernels implement */
  TDG_ERR_SHAPE = 3,        /* array sizes inconsistent with the description */
  TDG_ERR_CUDA = 4,         /* a CUDA runtime call failed */
  TDG_ERR_TIMEOUT = 5,      /* a bounded device-side wait gave up */
  TDG_ERR_NOMEM = 6         /* device allocation failed */
} tdg_status;

typedef enum {
  TDG_PREC_FP32 = 0,        /* FP32 FMA hidden GEMMs (CUDA cores) */
  TDG_PREC_TF32 = 1,        /* TF32 tensor-core hidden GEMMs, FP32 accumulate */
  TDG_PREC_3XTF32 = 2,      /* split TF32 (hi*hi + hi*lo + lo*hi), FP32 accumulate */
  TDG_PREC_BF16 = 3         /* BF16 tensor-core hidden GEMMs, FP32 accumulate */
} tdg_precision;

typedef enum {
  TDG_FORM_FUSED = 0,       /* one persistent kernel: jet/stencil forward + operator + loss + adjoint */
  TDG_FORM_PLAIN = 1        /* one launch per layer operation, activations kept in device memory */
} tdg_form;

/* tanh MLP: Linear(width[0]->width[1]), Tanh, ..., Linear(width[n-1]->width[n]). Parameters are one
 * flat FP32 buffer in torch.nn.Module.parameters() order: W0 (width[1] x width[0], row-major), b0,
 * W1, b1, ... */
typedef struct {
  int32_t n_layers;
  int32_t width[TDG_MAX_LAYERS + 1];
} tdg_mlp_desc;

/* A derivative stream: d^order u / dx_axes[0] .. dx_axes[order-1]; order 0 is the value. */
typedef struct {
  int32_t order;
  int32_t axes[TDG_MAX_ORDER];
} tdg_stream_desc;

/* An evaluation site: row i of the group is evaluated at points[i] + offset (FP32 add per axis,
 * as the reference builds shifted grids), carrying n_streams derivative streams. */
typedef struct {
  int32_t points;            /* index into tdg_problem_desc.arrays: n_rows x d_in floats */
  int32_t stream_first;      /* into tdg_problem_desc.streams */
  int32_t n_streams;
  float offset[TDG_MAX_DIN];
} tdg_site_desc;

/* part of a factor: weight * MLP_output[var] of stream `stream` at site `site` (indices relative
 * to the group's first site and to that site's first stream). */
typedef struct {
  int32_t site;
  int32_t stream;
  float weight;
} tdg_part_desc;

/* factor of a term: (sum over its parts) ** power, reading MLP output `var`. */
typedef struct {
  int32_t part_first;
  int32_t n_parts;
  int32_t var;
  float power;
} tdg_factor_desc;

/* term: coeff * product of factors, added to the group's output `output`. coeff_array >= 0 names a
 * per-row coefficient array (n_rows floats) that replaces the scalar coeff. coeff_param >= 0 makes
 * the coefficient trainable: the term's coefficient is coeff * theta, theta the problem's parameter
 * n_mlp + coeff_param (n_mlp = the MLP's parameter count), and the gradient gets d loss / d theta
 * at the same index (inverse problems: an nn.Parameter coefficient of the reference,
 * tedeous/solution.py:96-108). */
typedef struct {
  int32_t factor_first;
  int32_t n_factors;
  int32_t output;
  int32_t coeff_array;
  float coeff;
  int32_t coeff_param;
} tdg_term_desc;

/* a group of rows sharing one site/stream layout and one operator program. Output o of row i is
 * compared with target[i * n_outputs + o] (0 when target_array < 0) and its squared error is
 * added to loss slot slot_first + o. row_weight_array >= 0 names an array of n_rows floats w_i that
 * multiply row i's squared errors and, held constant, its gradient (the causal loss's time
 * weights, tedeous/losses.py:137-182; tdg_causal_weights computes them). */
typedef struct {
  int32_t problem;           /* which parameter set (0 for a single solve) */
  int32_t n_rows;
  int32_t site_first, n_sites;
  int32_t term_first, n_terms;
  int32_t n_outputs;
  int32_t slot_first;
  int32_t target_array;
  int32_t row_weight_array;  /* -1: every row weighs 1 */
  int64_t output_offset;     /* where rows' outputs go in the optional outputs buffer; -1: none */
} tdg_group_desc;

/* loss slot: loss += weight * sum(err^2); loss_normalized += weight_normalized * sum(err^2). */
typedef struct {
  int32_t problem;
  double weight;
  double weight_normalized;
} tdg_slot_desc;

typedef struct {
  tdg_mlp_desc mlp;
  int32_t n_problems;
  int32_t n_groups;   const tdg_group_desc* groups;
  int32_t n_sites;    const tdg_site_desc* sites;
  int32_t n_streams;  const tdg_stream_desc* streams;
  int32_t n_terms;    const tdg_term_desc* terms;
  int32_t n_factors;  const tdg_factor_desc* factors;
  int32_t n_parts;    const tdg_part_desc* parts;
  int32_t n_slots;    const tdg_slot_desc* slots;
  int32_t n_arrays;   const float* const* arrays;   /* device pointers */
  const int64_t* array_len;                         /* element counts of arrays[] */
  int32_t precision;  /* tdg_precision */
  int32_t form;       /* tdg_form */
  int32_t n_coeff_params;   /* trainable coefficients per problem, stored after the MLP's parameters */
} tdg_problem_desc;

typedef struct {
  int64_t n_params;           /* parameters of one problem: the MLP's, then the trainable coefficients */
  int64_t workspace_bytes;    /* device memory owned by the plan */
  int32_t n_tiles;
  int32_t n_ctas;
  int32_t n_segments;
  int32_t max_streams;
  double flops_hidden;        /* algorithmic hidden->hidden GEMM flops of one loss+gradient call */
  double flops_total;         /* all layers, forward + backward */
} tdg_plan_info;

typedef struct {
  float lr, beta1, beta2, eps, weight_decay;
  int32_t maximize;
} tdg_adam_desc;

typedef struct tdg_plan tdg_plan;
typedef struct CUstream_st* tdg_stream_t;   /* a cudaStream_t */

int32_t tdg_abi_version(void);
const char* tdg_last_error(void);
int64_t tdg_launch_count(void);             /* kernels launched by this library so far */
/* Compile-time jet class of a site with these streams (value first, then by order and axes, the
 * order the lowering emits), or -1 when the site runs the table-driven jet code. Host only. */
int32_t tdg_site_class(int32_t n_streams, const tdg_stream_desc* streams);

/* Validate the description, build tile schedules and device tables, allocate the workspace. */
tdg_status tdg_plan_create(const tdg_problem_desc* desc, tdg_plan** plan);

/* How a plan cuts its rows into tiles and spreads the tiles over persistent CTAs; the knobs the
 * autotuner (torch_de_solver_gb300.autotune) searches for a problem shape. max_rows caps the
 * (stream, point) rows of a tile (a multiple of 32, at most 128): a group of S streams runs
 * floor(max_rows / S) points per tile. n_ctas is the number of persistent CTAs (0: one per SM;
 * at most the SM count). balance 0 gives every CTA an equal number of consecutive tiles, balance 1
 * an equal share of estimated work (a fixed cost per tile plus its filled rows). */
typedef struct {
  int32_t max_rows;
  int32_t n_ctas;
  int32_t balance;
  int32_t reserved;
} tdg_schedule;
/* tdg_plan_create with a schedule (NULL: {128, 0, 0}, the tdg_plan_create default). Same
 * replacement as tdg_plan_create (tedeous/solution.py:23-88): no counterpart of the schedule in
 * the reference, which evaluates every point set in one batch. */
tdg_status tdg_plan_create_scheduled(const tdg_problem_desc* desc, const tdg_schedule* schedule,
                                     tdg_plan** plan);
tdg_status tdg_plan_destroy(tdg_plan* plan);
tdg_status tdg_plan_get_info(const tdg_plan* plan, tdg_plan_info* info);
/* Replace the device pointer of array `index` (same length), e.g. freshly copied points. */
tdg_status tdg_plan_set_array(tdg_plan* plan, int32_t index, const float* dev_ptr, int64_t n);

/* loss[2*p] = loss, loss[2*p+1] = loss_normalized of problem p (device doubles). outputs, when
 * not NULL, receives every group's per-row outputs at the groups' output_offset. */
tdg_status tdg_loss(tdg_plan* plan, const float* params, double* loss, float* outputs,
                    tdg_stream_t stream);
/* As tdg_loss, and grad[p * n_params + j] = d loss_p / d params[p * n_params + j]. */
tdg_status tdg_loss_grad(tdg_plan* plan, const float* params, float* grad, double* loss,
                         float* outputs, tdg_stream_t stream);

/* Synchronise the device and report TDG_ERR_TIMEOUT if a kernel of this plan gave up a bounded
 * wait on an mbarrier (the tensor-core path never spins without a limit). */
tdg_status tdg_plan_sync_status(tdg_plan* plan);

/* Failure-detection self-test: launch one thread that waits, with at most max_polls polls, on an
 * mbarrier that nothing arrives at. Returns TDG_ERR_TIMEOUT when the wait gives up as designed
 * (the kernels' waits on tensor-core and copy completion use the same bounded wait), leaving the
 * CUDA context usable. Synchronises the device. */
tdg_status tdg_selftest_bounded_wait(int32_t max_polls);

/* In-place Adam (torch.optim.Adam semantics, L2 weight_decay) on n floats; step is a device
 * float counter incremented by the call, so the call can be replayed from a CUDA graph. */
tdg_status tdg_adam_step(float* params, const float* grad, float* exp_avg, float* exp_avg_sq,
                         float* step, int64_t n, const tdg_adam_desc* hp, tdg_stream_t stream);

/* out[0] = sum_i a[i] * b[i] accumulated in FP64 (device double). The first call on a device
 * allocates a 2.4 KB partial-sum buffer (under a lock, safe from several host threads) that every
 * later call on that device shares: calls that overlap on the GPU race on it. */
tdg_status tdg_dot_f64(const float* a, const float* b, int64_t n, double* out,
                       tdg_stream_t stream);

/* Device-resident L-BFGS, replacing the torch.optim.LBFGS that the reference selects
 * (tedeous/optimizers/optimizer.py:50-51) in its two-loop recursion and curvature updates.
 * The history is a ring of history_size + 1 (s, y) pairs of n floats on the device with FP64
 * rho = 1 / y.s, FP64 two-loop coefficients and the FP64 scale H_diag = y.s / y.y; every dot
 * product accumulates in FP64 with fixed-order (deterministic) sums. No call synchronises the host
 * except tdg_lbfgs_create. A state is not thread safe: one per optimizer and stream. */
typedef struct tdg_lbfgs tdg_lbfgs;
tdg_status tdg_lbfgs_create(int64_t n, int32_t history_size, tdg_lbfgs** out);
tdg_status tdg_lbfgs_destroy(tdg_lbfgs* h);
/* Forget every stored pair; H_diag = 1. */
tdg_status tdg_lbfgs_reset(tdg_lbfgs* h, tdg_stream_t stream);
/* The pair y = g - g_prev, s = t d, stored (the oldest dropped when the ring is full) when
 * y.s > 1e-10, as torch.optim.LBFGS does; otherwise the history is unchanged. */
tdg_status tdg_lbfgs_push(tdg_lbfgs* h, const float* g, const float* g_prev, const float* d,
                          double t, tdg_stream_t stream);
/* d = -H g by the two-loop recursion over the stored pairs (newest first, then oldest first).
 * n_pairs_bound (<= history_size) is an upper bound on the stored pairs, e.g. the number of pushes
 * so far: the host need not know how many were accepted. 2 (n_pairs_bound + 1) launches. */
tdg_status tdg_lbfgs_direction(tdg_lbfgs* h, const float* g, float* d, int32_t n_pairs_bound,
                               tdg_stream_t stream);
/* out[0..4] (device doubles) = g.d, sum |g_i|, max |g_i|, max |d_i|, *loss: the quantities of
 * torch.optim.LBFGS's step-size and stopping tests, for one device-to-host read. d and loss may
 * be NULL (read as 0). */
tdg_status tdg_lbfgs_stats(tdg_lbfgs* h, const float* g, const float* d, const float* loss,
                           double* out, tdg_stream_t stream);
/* out = x + t d (out may alias x): the parameter update of an L-BFGS step or line-search trial. */
tdg_status tdg_axpy(const float* x, const float* d, double t, float* out, int64_t n,
                    tdg_stream_t stream);

/* Allocation-free variant of tdg_dot_f64. No counterpart in the reference: it serves callers that
 * own all device memory themselves (a framework allocator that has reserved the GPU, or a
 * foreign-language host binding this ABI under a fixed device-memory budget) and so cannot let
 * the library call cudaMalloc, which tdg_dot_f64 does on its first call on each device.
 * Partial sums live in a static device array of TDG_DOT_NOALLOC_MAX_BLOCKS doubles (32 KiB,
 * held by every GPU that loads the library until exit); n above TDG_DOT_NOALLOC_MAX_N is
 * rejected with TDG_ERR_SHAPE. The first call on each device looks up the array's device address
 * (cudaGetSymbolAddress) with that device current; make that first call before any stream
 * capture. All calls share the array, so calls that overlap on the GPU race on it. */
#define TDG_DOT_NOALLOC_MAX_BLOCKS 4096
#define TDG_DOT_NOALLOC_CHUNK 16384LL
#define TDG_DOT_NOALLOC_MAX_N (TDG_DOT_NOALLOC_MAX_BLOCKS * TDG_DOT_NOALLOC_CHUNK)
tdg_status tdg_dot_f64_noalloc(const float* a, const float* b, int64_t n, double* out,
                               tdg_stream_t stream);

/* Causal-loss weights of a residual field op[n_rows][n_eq] (row-major floats) whose rows form n_t
 * time slices of rest = n_rows / n_t adjacent rows: with res_i = sum_e op[i][e]^2 and row
 * i = s * rest + k, w[i] = exp(-tol * sum over s' < s of res[s' * rest + k]), the sum in FP64
 * (tedeous/losses.py:160-168). n_rows must be a multiple of n_t (TDG_ERR_SHAPE otherwise). */
tdg_status tdg_causal_weights(const float* op, int64_t n_rows, int32_t n_eq, int64_t n_t, float tol,
                              float* w, tdg_stream_t stream);

/* dst[r][c] = src[index[r]][c] for r < n and c < row_len (device arrays; index is int64). An
 * index outside [0, n_src) gives a zero row. */
tdg_status tdg_gather_rows(const float* src, int64_t n_src, const int64_t* index, int64_t n,
                           int32_t row_len, float* dst, tdg_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* TDG_H_ */
