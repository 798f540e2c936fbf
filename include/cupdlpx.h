/*
 * cupdlpx.h -- the drop-in C API of the GB300 PDHG LP solver.
 *
 * Same six entry points, argument meaning, ownership and NULL conventions as
 * the reference's single-GPU API (D-PDLP include/cupdlpx.h:26-45,
 * src/cupdlpx.c:26-198).  Differences, all in the caller's favour:
 *  - CUDA failures return NULL from solve_lp_problem (message on stderr)
 *    instead of exit(EXIT_FAILURE) (reference internal/utils.h:30-58);
 *  - the solve is re-entrant: fresh power-method seed per call, one CUDA
 *    stream per solve, no process-global state;
 *  - cupdlpx_result_free also releases reduced_cost;
 *  - presolve=true prints a one-line notice and solves without presolve
 *    (the PSLP presolver the reference links is not part of this library).
 */
#ifndef CUPDLPX_GB300_H
#define CUPDLPX_GB300_H

#include "cupdlpx_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Deep-copies the inputs into a new host problem (CSR).  NULL objective
 * gives zeros, NULL bounds give -inf/+inf, NULL constant gives 0.  Returns
 * NULL for an unsupported format or an out-of-range index.
 * Replaces reference include/cupdlpx.h:26-30 (src/cupdlpx.c:26-117). */
lp_problem_t *create_lp_problem(const double *objective_c,
                                const matrix_desc_t *A_desc,
                                const double *con_lb, const double *con_ub,
                                const double *var_lb, const double *var_ub,
                                const double *objective_constant);

/* Copies a warm start into the problem, replacing any previous one; either
 * pointer may be NULL.  Replaces reference include/cupdlpx.h:33-34
 * (src/cupdlpx.c:146-172). */
void set_start_values(lp_problem_t *prob, const double *primal,
                      const double *dual);

/* Solves the LP on the current CUDA device with restarted Halpern PDHG.
 * params == NULL uses set_default_parameters().  prob is not modified.
 * Returns NULL on a NULL problem or a CUDA failure.
 * Replaces reference include/cupdlpx.h:37-38 (src/cupdlpx.c:174-198). */
cupdlpx_result_t *solve_lp_problem(const lp_problem_t *prob,
                                   const pdhg_parameters_t *params);

/* Fills every field with the reference defaults (reference src/utils.cu:
 * 295-329), and also the fields the reference leaves unset
 * (grid_size.row_dims/col_dims = 1, permute_block_size = 256).
 * Replaces reference include/cupdlpx.h:41. */
void set_default_parameters(pdhg_parameters_t *params);

/* Frees a result and its three arrays.  Replaces include/cupdlpx.h:43. */
void cupdlpx_result_free(cupdlpx_result_t *results);

/* Frees a problem made by create_lp_problem.  Replaces include/cupdlpx.h:45. */
void lp_problem_free(lp_problem_t *prob);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* CUPDLPX_GB300_H */
