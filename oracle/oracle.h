/*
 * oracle.h -- CPU FP64 restatement of the reference's single-GPU PDHG solve.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle of the CUDA solver's
 * parity tests and the timed CPU baseline; the product never links, loads or
 * calls it.  Each function cites the reference code (D-PDLP, path:line) that
 * it restates.
 */
#ifndef PDLP_ORACLE_H
#define PDLP_ORACLE_H

#include "cupdlpx_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* One record per evaluation iteration, in this order. */
enum {
  ORACLE_TR_ITER = 0,
  ORACLE_TR_REL_PRIMAL,
  ORACLE_TR_REL_DUAL,
  ORACLE_TR_REL_GAP,
  ORACLE_TR_PRIMAL_OBJ,
  ORACLE_TR_DUAL_OBJ,
  ORACLE_TR_PRIMAL_WEIGHT,
  ORACLE_TR_FIXED_POINT_ERROR,
  ORACLE_TR_STEP_SIZE,
  ORACLE_TR_INNER_COUNT,
  ORACLE_TR_WIDTH
};

/* Full solve: rescale -> power method -> restarted Halpern PDHG -> unscale
 * (reference src/solver.cu:32-127 with presolve off).  nthreads <= 0 uses
 * every OpenMP thread.  trace (may be NULL) receives up to trace_cap records
 * of ORACLE_TR_WIDTH doubles; *trace_len the number written.  The result is
 * released with oracle_result_free. */
cupdlpx_result_t *oracle_solve(const lp_problem_t *prob,
                               const pdhg_parameters_t *params, int nthreads,
                               double *trace, int trace_cap, int *trace_len);
void oracle_result_free(cupdlpx_result_t *r);

/* Defaults (reference src/utils.cu:295-329). */
void oracle_default_parameters(pdhg_parameters_t *p);

/* Rescaling (reference src/preconditioner.c:197-273).  Outputs are caller
 * buffers: scaled CSR values (nnz), c (n), lv, uv (n), lc, uc (m),
 * con_rescale (m), var_rescale (n), and the two scalars. */
void oracle_rescale(const lp_problem_t *prob, const pdhg_parameters_t *params,
                    double *vals, double *c, double *lv, double *uv,
                    double *lc, double *uc, double *con_rescale,
                    double *var_rescale, double *con_bound_rescale,
                    double *obj_vec_rescale);

/* Stable CSR transpose (what cusparseCsr2cscEx2 produces in
 * src/pdlp_core_op.cu:109-130): rows of A^T sorted by original row. */
void oracle_transpose(int m, int n, const int *ap, const int *aj,
                      const double *ax, int *tp, int *tj, double *tx);

/* y = A x, one sequential sum per row in CSR order. */
void oracle_spmv(int rows, const int *ap, const int *aj, const double *ax,
                 const double *x, double *y, int nthreads);

/* Power method on A A^T (reference src/utils.cu:66-171) started from the
 * given vector v0 (length m).  Returns sigma_max; *iters_out the number of
 * iterations run. */
double oracle_power_method(int m, int n, const int *ap, const int *aj,
                           const double *ax, const double *v0, int max_iter,
                           double tol, int *iters_out, int nthreads);

/* Start vector of the reference power method: m draws of N(0,1) from a
 * fresh std::mt19937(1) (reference src/utils.cu:29-30, :79-82). */
void oracle_power_start_vector(int m, double *v);

/* Format converters (reference src/utils.cu:826-1013).  Output arrays are
 * malloc'ed and freed by the caller with free().  Return 0 on success. */
int oracle_dense_to_csr(const matrix_desc_t *d, int **rp, int **ci,
                        double **v, int *nnz);
int oracle_csc_to_csr(const matrix_desc_t *d, int **rp, int **ci, double **v,
                      int *nnz);
int oracle_coo_to_csr(const matrix_desc_t *d, int **rp, int **ci, double **v,
                      int *nnz);

/* Bounded samples for the CPU baseline: a session holds one prepared solve.
 * create: rescale + transpose + norms (timed, seconds in *setup_sec);
 * power: `iters` power-method iterations from the reference start vector,
 *        returns seconds;
 * iterate: `iters` iterations of the driver loop (evaluations, restarts and
 *        all) continuing from the current state, returns seconds. */
typedef struct oracle_session oracle_session_t;
oracle_session_t *oracle_session_create(const lp_problem_t *prob,
                                        const pdhg_parameters_t *params,
                                        int nthreads, double *setup_sec);
double oracle_session_power(oracle_session_t *s, int iters);
double oracle_session_iterate(oracle_session_t *s, int iters);
void oracle_session_free(oracle_session_t *s);

/* Evaluation cadence (reference src/utils.cu:492-501). */
int oracle_print_frequency(int iter);

/* Termination reason for one evaluation's scalars (reference
 * src/utils.cu:214-263); TERMINATION_REASON_UNSPECIFIED when none holds. */
int oracle_termination_decision(const termination_criteria_t *tc, double rel_p,
                                double rel_d, double rel_gap, double dray_obj,
                                double max_dray, double pray_obj, double max_pray,
                                int total, double cum_time);

/* Adaptive restart test (reference src/utils.cu:265-293); updates
 * *last_fpe as the reference updates last_trial_fixed_point_error. */
int oracle_restart_decision(const restart_parameters_t *rp, int F, int total,
                            int inner, double fpe, double init_fpe,
                            double *last_fpe);

/* The seeded LP generators of the benchmarks (d-pdlp_gb300/csrc/lpgen.cpp,
 * compiled into this library under these names), so CPU baselines and the
 * reference's own solve get their problems without loading the product
 * library.  Problems are released with oracle_problem_free. */
lp_problem_t *oracle_generate_random_lp(int m, int n, long long nnz, unsigned long long seed);
lp_problem_t *oracle_generate_powerlaw_lp(int m, int n, long long nnz_target, double zipf_s,
                                          int max_degree, unsigned long long seed);
lp_problem_t *oracle_generate_transport_lp(int sources, int sinks, unsigned long long seed);
void oracle_problem_free(lp_problem_t *p);

#ifdef __cplusplus
}
#endif
#endif
