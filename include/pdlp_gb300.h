/*
 * pdlp_gb300.h -- additions of the GB300 solver beyond the reference C API.
 *
 * Nothing here replaces a reference entry point; these are new, namespaced
 * functions: solve diagnostics and precision options, problems resident in
 * HBM, the batch / serving runtime, the binary problem format, seeded
 * problem generators, and the device-level hooks the parity tests call.
 * They take plain pointers and sizes (host memory unless a function says
 * device).
 * Errors: functions returning int give 0 on success and a negative code on
 * failure; pdlp_last_error() then describes the failure of the calling thread.
 */
#ifndef PDLP_GB300_H
#define PDLP_GB300_H

#include "cupdlpx_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Diagnostics of one solve. */
typedef struct {
  int power_iterations;       /* iterations of the step-size power method */
  double sigma_max;           /* estimated largest singular value of scaled A */
  double setup_seconds;       /* upload + transpose + plans + GPU rescaling */
  double rescale_seconds;     /* GPU rescaling alone */
  double power_seconds;       /* power method */
  double loop_seconds;        /* PDHG loop, wall clock */
  double total_seconds;       /* whole solve_lp_problem call */
  int graphs;                 /* distinct iteration-chunk CUDA graphs */
  long long kernel_launches;  /* kernels launched by the solve */
  double device_seconds;      /* CUDA events on the solve's stream, from the
                                 first copy/kernel to the result on the host */
  int refinement_rounds;      /* FP32 rounds of a mixed-precision solve */
  int precision;              /* PDLP_PRECISION_* the solve ran in */
  double primal_step_ms;      /* average device time of an ordinary primal-step
                                 launch (A^T SpMV + update) inside the loop,
                                 from CUDA events in one iteration per
                                 100-iteration chunk */
  double dual_step_ms;        /* the same for the dual step (A SpMV + update) */
  int timed_chunks;           /* chunks those averages cover (0: none) */
  int fp64_finish;            /* 1 when a mixed-precision solve ended with FP64
                                 PDHG warm-started from its best FP64 point */
  int spmv_kernel_A;          /* SpMV kernel of A (dual step and its other
                                 products): 0 fused, 1 pipelined */
  int spmv_kernel_AT;         /* the same for A^T (primal step) */
  double tune_ms[4];          /* the measurement that chose them, ms per
                                 launch: A fused, A pipelined, A^T fused, A^T
                                 pipelined (zeros when the choice was reused
                                 from an earlier solve of the problem) */
} pdlp_solve_info_t;

/* Arithmetic of the PDHG iteration.
 * FP64: every operation in FP64, as the reference.
 * FP32_REFINE: matrix values, iterates, SpMVs and updates in FP32 (FP32
 *   accumulation); KKT / gap / restart / primal-weight reductions, objective
 *   values and the refinement residuals in FP64.  Rounds of iterative
 *   refinement re-centre the LP at the FP64 point until the FP64 KKT of the
 *   original problem meets the requested tolerances; when a round cannot
 *   improve the point (an FP32 precision floor), FP64 PDHG finishes from the
 *   best FP64 point.
 * The drop-in solve_lp_problem() uses FP64 unless the environment variable
 * PDLP_PRECISION is "fp32" (FP32_REFINE) or "fp32m" (FP32_MATRIX). */
#define PDLP_PRECISION_FP64 0
#define PDLP_PRECISION_FP32_REFINE 1
/* FP32_MATRIX: matrix values, SpMV products and their accumulation in FP32;
 * iterates and the per-element updates in FP64 (no FP32 absorption floor);
 * reductions in FP64.  Same refinement rounds as FP32_REFINE when the FP64
 * KKT of the original LP misses the tolerances. */
#define PDLP_PRECISION_FP32_MATRIX 2

typedef struct {
  int precision;          /* PDLP_PRECISION_* */
  int max_refinements;    /* FP32 rounds (0: 8) */
  double inner_eps;       /* tolerance of rounds after the first (0: the
                             requested tolerances) */
} pdlp_options_t;

/* solve_lp_problem with explicit options (NULL: FP64). */
cupdlpx_result_t *pdlp_solve_opts(const lp_problem_t *prob,
                                  const pdhg_parameters_t *params,
                                  const pdlp_options_t *opts,
                                  pdlp_solve_info_t *info);

/* Number of doubles per trace record written by pdlp_solve_ex: iteration,
 * rel. primal residual, rel. dual residual, rel. gap, primal objective,
 * dual objective, primal weight, fixed-point error, step size, inner count. */
#define PDLP_TRACE_WIDTH 10

/* solve_lp_problem plus optional per-evaluation trace and diagnostics
 * (trace/info may be NULL).  Same result ownership as solve_lp_problem. */
cupdlpx_result_t *pdlp_solve_ex(const lp_problem_t *prob,
                                const pdhg_parameters_t *params, double *trace,
                                int trace_cap, int *trace_len,
                                pdlp_solve_info_t *info);

/* ---- problems resident in HBM ----------------------------------------
 * An uploaded problem keeps A, its transpose (CSR), the SpMV plans, bounds
 * and objective on the current device, unscaled, so that any number of
 * solves can start from HBM without a host copy.  Solves from one handle
 * may run one after another or concurrently from different threads. */
typedef struct pdlp_device_problem pdlp_device_problem_t;

pdlp_device_problem_t *pdlp_device_problem_create(const lp_problem_t *prob);
void pdlp_device_problem_free(pdlp_device_problem_t *dp);
/* Bytes of HBM the handle holds. */
long long pdlp_device_problem_bytes(const pdlp_device_problem_t *dp);
/* Solve from the resident problem (result copied to host, as from
 * solve_lp_problem). */
cupdlpx_result_t *pdlp_device_problem_solve(pdlp_device_problem_t *dp,
                                            const pdhg_parameters_t *params,
                                            pdlp_solve_info_t *info);
/* pdlp_device_problem_solve with explicit options (NULL: FP64). */
cupdlpx_result_t *pdlp_device_problem_solve_opts(pdlp_device_problem_t *dp,
                                                 const pdhg_parameters_t *params,
                                                 const pdlp_options_t *opts,
                                                 pdlp_solve_info_t *info);
/* Average device milliseconds per launch of the iteration kernels, timed
 * with CUDA events on the solve's stream over `reps` launches each:
 * ms[0] primal step (A^T SpMV + projection + Halpern), ms[1] dual step
 * (A SpMV + projection + Halpern), ms[2] evaluation over A, ms[3]
 * evaluation over A^T. */
int pdlp_device_problem_time_kernels(pdlp_device_problem_t *dp,
                                     const pdhg_parameters_t *params, int reps,
                                     double *ms);
/* As above for the given PDLP_PRECISION_* iteration type. */
int pdlp_device_problem_time_kernels_prec(pdlp_device_problem_t *dp,
                                          const pdhg_parameters_t *params,
                                          int precision, int reps, double *ms);

/* ---- batched and served solves of independent LPs ----------------------
 * No counterpart in the reference, which solves one LP per call
 * (src/cupdlpx.c:174-198); each request runs that solve.
 *
 * A server runs `workers` host threads, each with its own CUDA stream, over
 * one FIFO queue of submitted LPs (deep copies).  The head request is
 * admitted when its estimated device footprint
 * (pdlp_estimate_device_bytes) fits in what is left of the memory budget
 * (mem_budget_bytes <= 0: 80% of the device memory free at creation); a
 * request larger than the whole budget is admitted alone.  LPs in flight
 * overlap on the GPU.  Each LP's arithmetic depends on its own data only, so
 * its result is bitwise the same solved alone or in any mix.  All solves use
 * `params` (NULL: defaults) and `opts` (NULL: FP64). */
typedef struct pdlp_server pdlp_server_t;

typedef struct {
  double queued_seconds;    /* submit -> admission */
  double solve_seconds;     /* admission -> result (upload, solve, copy back) */
  double latency_seconds;   /* submit -> result */
  int worker;               /* worker thread that solved it */
  long long device_bytes;   /* footprint the admission charged */
  double upload_seconds;    /* host time of the upload (checks, transpose,
                               plans, copies enqueued) */
  double device_seconds;    /* the solve on the worker's stream, from CUDA
                               events (waits behind other requests' kernels
                               included) */
} pdlp_request_info_t;

typedef struct {
  long long completed;      /* requests finished (solved or failed) */
  long long failed;         /* requests whose solve returned no result */
  long long queued;         /* requests waiting for admission */
  int in_flight;            /* requests being solved now */
  int max_in_flight;        /* most requests in flight at once */
  long long iterations;     /* PDHG iterations summed over finished requests */
  long long device_bytes_in_use; /* footprint of the requests in flight */
  double busy_seconds;      /* first admission to last finish */
  long long rejected;       /* submissions refused by the queue bound */
  long long queued_host_bytes; /* host bytes of the waiting requests' copies */
} pdlp_server_stats_t;

/* Estimated device bytes of one solve (problem plus solve workspace). */
long long pdlp_estimate_device_bytes(int m, int n, long long nnz, int precision);

pdlp_server_t *pdlp_server_create(const pdhg_parameters_t *params,
                                  const pdlp_options_t *opts, int workers,
                                  long long mem_budget_bytes);
/* Queue a copy of prob; returns the request id (>= 0), -1 on failure, or
 * -2 when the queue bound refuses it (pdlp_server_set_queue_limit). */
long long pdlp_server_submit(pdlp_server_t *s, const lp_problem_t *prob);
/* Bound the queue: a submission whose copy would take the requests waiting
 * for admission past max_queued_host_bytes of host memory is refused (-2)
 * unless the queue is empty; 0 (the default) removes the bound.  Under an
 * arrival rate above the GPU's capacity this keeps the host memory of the
 * backlog bounded; refused requests are counted in the stats. */
int pdlp_server_set_queue_limit(pdlp_server_t *s, long long max_queued_host_bytes);
/* Block until request `id` is solved; the result (NULL on failure, see
 * pdlp_last_error) belongs to the caller; info may be NULL.  Each id can be
 * collected once. */
cupdlpx_result_t *pdlp_server_wait(pdlp_server_t *s, long long id,
                                   pdlp_request_info_t *info);
int pdlp_server_stats(pdlp_server_t *s, pdlp_server_stats_t *stats);
/* Finish every queued request, stop the workers and free what was not
 * collected. */
void pdlp_server_destroy(pdlp_server_t *s);

typedef struct {
  int lps;                  /* LPs submitted */
  int failed;               /* LPs without a result */
  double wall_seconds;      /* first submission to last result */
  double lps_per_second;    /* solved LPs / wall_seconds */
  long long iterations;     /* PDHG iterations summed over the LPs */
  int max_concurrent;       /* most LPs in flight at once */
} pdlp_batch_info_t;

/* Solve `count` LPs through a server of `workers` workers; results[i] is the
 * result of probs[i] (caller frees each).  Returns 0, or -3 when some LP
 * failed (its result NULL), -1/-2 on bad arguments / no server. */
int pdlp_batch_solve(const lp_problem_t *const *probs, int count,
                     const pdhg_parameters_t *params, const pdlp_options_t *opts,
                     int workers, long long mem_budget_bytes,
                     cupdlpx_result_t **results, pdlp_batch_info_t *info);

/* ---- binary problem format ----------------------------------------------
 * The byte layout of the reference's serialize_lp_problem_to_ptr
 * (src/distribution_utils.cu:279-405), for request payloads and stored
 * instances: int32 n, m, nnz; float64 objective constant; float64 c[n],
 * lv[n], uv[n], lc[m], uc[m]; int32 row_ptr[m+1], col[nnz]; float64
 * val[nnz]; int32 has_primal_start, has_dual_start; then the start vectors
 * present.  Host byte order, packed. */
long long pdlp_problem_wire_size(const lp_problem_t *lp);
/* Write lp into buf (capacity bytes); returns the bytes written or -1. */
long long pdlp_problem_serialize(const lp_problem_t *lp, void *buf, long long capacity);
/* Read a payload of `length` bytes; NULL when it is truncated or its CSR is
 * inconsistent.  Free with lp_problem_free. */
lp_problem_t *pdlp_problem_deserialize(const void *buf, long long length);
/* pdlp_server_submit of a payload in that format. */
long long pdlp_server_submit_bytes(pdlp_server_t *s, const void *buf, long long length);

/* Return the device memory cached by the library's pool. */
void pdlp_release_pooled_memory(void);

/* Message of the last failure in this thread ("" if none). */
const char *pdlp_last_error(void);

/* Name of a termination reason (reference src/utils.cu:173-194). */
const char *pdlp_termination_reason_to_string(termination_reason_t reason);

/* ---- seeded synthetic LPs (SplitMix64 streams; identical on every host).
 * All return a problem owned by the caller (lp_problem_free), or NULL. */

/* Uniform random positions (distinct), values N(0,1); x0 ~ U[0,1]^n feasible;
 * 30% of rows equality l = u = A x0, the rest l = A x0 - U[0,1], u = +inf;
 * 0 <= x <= 10; c ~ U[-1,1]. */
lp_problem_t *pdlp_generate_random_lp(int m, int n, long long nnz,
                                      unsigned long long seed);

/* As above, but column degrees follow a rank Zipf law d_r = max(1, min(cap,
 * round(C r^-s))) with C chosen so the degrees sum to about nnz_target,
 * assigned to a random column permutation; rows uniform within a column;
 * values N(0,1) with 5% of entries +-1. */
lp_problem_t *pdlp_generate_powerlaw_lp(int m, int n, long long nnz_target,
                                        double zipf_s, int max_degree,
                                        unsigned long long seed);

/* Balanced transportation LP: sources x sinks arcs, one equality row per
 * source (supply ~ U[1,100]) and per sink (demand ~ U[1,100] rescaled to
 * the total supply), costs ~ U[0,1], x >= 0. */
lp_problem_t *pdlp_generate_transport_lp(int sources, int sinks,
                                         unsigned long long seed);

/* ---- device-level hooks (inputs and outputs in host memory) ----------- */

/* GPU rescaling of prob (upload, transpose, Ruiz/PC/bound-objective) with
 * the scaled problem copied back.  Output sizes: vals nnz, c/lv/uv/var n,
 * lc/uc/con m. */
int pdlp_gpu_rescale(const lp_problem_t *prob, const pdhg_parameters_t *params,
                     double *vals, double *c, double *lv, double *uv,
                     double *lc, double *uc, double *con_rescale,
                     double *var_rescale, double *con_bound_rescale,
                     double *obj_vec_rescale);

/* y = A x with the fused SpMV kernel and a plan of the given tile
 * (512 or 2048 non-zeros per thread block). */
int pdlp_gpu_spmv(int rows, int cols, const int *row_ptr, const int *col_ind,
                  const double *vals, const double *x, double *y, int tile);

/* As pdlp_gpu_spmv, with tile 512, 1024 or 2048 and a kernel variant:
 * 0 staged, 1 register path for short-row tiles (tile 1024 only), 2 the
 * register path with column and value arrays placed off 16-byte boundaries
 * (its scalar-load fallback). */
int pdlp_gpu_spmv_variant(int rows, int cols, const int *row_ptr, const int *col_ind,
                          const double *vals, const double *x, double *y, int tile,
                          int variant);

/* The SpMV plan the solver builds for a CSR matrix of `rows` rows: tiles of
 * `tile` non-zeros (512, 1024 or 2048), long rows in chunks of `chunk`
 * (>= tile; 0: the solver's default).  Writes up to `cap` blocks as
 * {first row, end row or -(long row id + 1), first non-zero, end non-zero}
 * into `blocks` (may be NULL), and the block count, long-row count and the
 * register-path choice (1 or 0, tiles of 1024 only).  Returns 0, or -1 on
 * invalid arguments or a malformed row pointer. */
int pdlp_spmv_plan(int rows, const int *row_ptr, int tile, int chunk, int *blocks,
                   int cap, int *nblk, int *nlong, int *direct);

/* Tiling of the pipelined step kernel for a matrix of `rows` rows whose step
 * epilogue stages nv per-row vectors: *ntile tiles of 4 ints {r0, r1 or
 * -(long row id + 1), k0, k1} into tiles (up to cap) and, per tile, the stage
 * bytes its copy ranges take in the largest precision into bytes (up to
 * cap; either may be NULL); limits (may be NULL) receives {rows per tile,
 * non-zeros per tile, longest row packed with others, stage bytes}.
 * Returns 0, or -1 on invalid arguments or a malformed row pointer. */
int pdlp_spmv_pipe_plan(int rows, const int *row_ptr, int nv, int *tiles, int *bytes,
                        int cap, int *ntile, int *nlong, int *limits);

/* The host transpose (the order the device transpose reproduces): A (m x n CSR) to A^T (n x m CSR),
 * entries of each column in row order.  Outputs: t_row_ptr n+1, t_col_ind
 * and t_vals nnz.  Returns 0, or -1 on invalid sizes, a NULL pointer, a
 * malformed row pointer or a column index outside [0, n). */
int pdlp_host_transpose(int m, int n, const int *row_ptr, const int *col_ind,
                        const double *vals, int *t_row_ptr, int *t_col_ind,
                        double *t_vals);

/* The device transpose of the upload path (the stable transpose above,
 * built on the GPU by a radix sort of the column indices), on host arrays
 * copied in and out.  Returns 0, -1 as pdlp_host_transpose, -2 on a CUDA
 * error. */
int pdlp_gpu_transpose(int m, int n, const int *row_ptr, const int *col_ind,
                       const double *vals, int *t_row_ptr, int *t_col_ind,
                       double *t_vals);

/* Power method of the solver on the scaled problem of prob; returns the
 * step-size estimate sigma_max and the iteration count. */
int pdlp_gpu_power_method(const lp_problem_t *prob,
                          const pdhg_parameters_t *params, double *sigma_max,
                          int *iterations);

/* ---- SpMV that allocates nothing ---------------------------------------
 * No counterpart in the reference: an addition of this library for callers
 * that cannot call cudaMalloc -- a host application whose own pool
 * allocator has already reserved the device memory (a further cudaMalloc
 * fails or breaks its accounting), or a latency-critical loop that must not
 * take the device-wide synchronisation that cudaMalloc / cudaFree imply.
 *
 * y = A x for a CSR matrix (rows x cols, nnz non-zeros) with row_ptr,
 * col_ind, vals, x and y all in DEVICE memory owned by the caller; stream is
 * a cudaStream_t (NULL: the legacy default stream).  The call returns after
 * the product is complete on that stream.  Its only scratch (per-tile
 * partial sums of rows that cross 2048-non-zero tiles, and an error flag) is
 * a 1.3 MB array in device global memory that each GPU loading this library
 * holds until the process exits; no cudaMalloc, cudaFree or allocating
 * library routine is called.
 *
 * Limits and sharing: nnz may be at most PDLP_NOALLOC_MAX_TILES * 2048
 * (134,217,728); larger inputs return -3 without launching.  All calls share
 * the one scratch array per device, so calls that overlap on the GPU (other
 * streams, other host threads) race and must be serialised by the caller.
 * The first successful call on each device looks up the array's device
 * address with that device current.  Every call waits for its own product
 * (it reads the error flag back and synchronises the stream), so it must not
 * be called while that stream is being captured into a CUDA graph.
 *
 * Returns 0 on success; -1 bad arguments (negative sizes, NULL buffers,
 * non-zeros without rows), -2 CUDA error, -3 size above the
 * limit, -4 malformed CSR (row pointers or column indices, detected on the
 * device; y is then unspecified).  pdlp_spmv_noalloc_error() gives the
 * message of the calling thread's last failure. */
#define PDLP_NOALLOC_MAX_TILES 65536
int pdlp_spmv_noalloc(int rows, int cols, int nnz, const int *row_ptr,
                      const int *col_ind, const double *vals, const double *x,
                      double *y, void *stream);
const char *pdlp_spmv_noalloc_error(void);

#ifdef __cplusplus
}
#endif
#endif
