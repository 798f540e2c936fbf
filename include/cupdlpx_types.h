/*
 * cupdlpx_types.h -- public data types of the GB300 PDHG LP solver.
 *
 * Every struct and enum here is layout-compatible with the reference's
 * public types header (D-PDLP include/cupdlpx_types.h:27-197), so that a C
 * program compiled against the reference header links against this library
 * unchanged: same field names, same order, same C types (C99 `bool` is one
 * byte, enums are `int`).  The reference header also includes the PSLP
 * presolve stats header (cupdlpx_types.h:19); the only type it would use
 * (`PresolveStats`) is commented out of the result struct (:135), so this
 * header does not include it.
 *
 * Problem form:   min c'x + c0   s.t.   lc <= A x <= uc,   lv <= x <= uv.
 */
#ifndef CUPDLPX_GB300_TYPES_H
#define CUPDLPX_GB300_TYPES_H

#include <stdbool.h>
#include <stdlib.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Outcome of a solve (reference cupdlpx_types.h:27-36). */
typedef enum {
  TERMINATION_REASON_UNSPECIFIED,
  TERMINATION_REASON_OPTIMAL,
  TERMINATION_REASON_PRIMAL_INFEASIBLE,
  TERMINATION_REASON_DUAL_INFEASIBLE,
  TERMINATION_REASON_INFEASIBLE_OR_UNBOUNDED,
  TERMINATION_REASON_TIME_LIMIT,
  TERMINATION_REASON_ITERATION_LIMIT,
  TERMINATION_REASON_FEAS_POLISH_SUCCESS
} termination_reason_t;

/* Norm used by the optimality measures (reference :38). */
typedef enum { NORM_TYPE_L2 = 0, NORM_TYPE_L_INF = 1 } norm_type_t;

/* An LP held in host memory, constraint matrix in CSR (reference :40-58).
 * Produced by create_lp_problem(), released by lp_problem_free(). */
typedef struct {
  int num_variables;
  int num_constraints;
  double *variable_lower_bound;
  double *variable_upper_bound;
  double *objective_vector;
  double objective_constant;

  int *constraint_matrix_row_pointers;
  int *constraint_matrix_col_indices;
  double *constraint_matrix_values;
  int constraint_matrix_num_nonzeros;

  double *constraint_lower_bound;
  double *constraint_upper_bound;

  double *primal_start; /* optional warm start, length num_variables */
  double *dual_start;   /* optional warm start, length num_constraints */
} lp_problem_t;

/* Adaptive-restart and primal-weight PID settings (reference :60-68). */
typedef struct {
  double artificial_restart_threshold;
  double sufficient_reduction_for_restart;
  double necessary_reduction_for_restart;
  double k_p;
  double k_i;
  double k_d;
  double i_smooth;
} restart_parameters_t;

/* Stopping rules (reference :70-77). */
typedef struct {
  double eps_optimal_relative;
  double eps_feasible_relative;
  double eps_feas_polish_relative;
  double eps_infeasible;
  double time_sec_limit;
  int iteration_limit;
} termination_criteria_t;

/* Multi-GPU partitioning choices.  Kept for layout compatibility; this
 * single-GPU build accepts and ignores them (reference :79-94). */
typedef enum {
  UNIFORM_PARTITION,
  NNZ_BALANCE_PARTITION,
} partition_method_t;

typedef enum {
  NO_PERMUTATION,
  FULL_RANDOM_PERMUTATION,
  BLOCK_RANDOM_PERMUTATION,
} permute_method_t;

typedef struct {
  int row_dims;
  int col_dims;
  bool decided;
} grid_size_t;

/* Solver parameters (reference :96-115); defaults from
 * set_default_parameters(). */
typedef struct {
  int l_inf_ruiz_iterations;
  bool has_pock_chambolle_alpha;
  double pock_chambolle_alpha;
  bool bound_objective_rescaling;
  bool verbose;
  int termination_evaluation_frequency;
  int sv_max_iter;
  double sv_tol;
  termination_criteria_t termination_criteria;
  restart_parameters_t restart_params;
  double reflection_coefficient;
  bool feasibility_polishing;
  norm_type_t optimality_norm;
  bool presolve;
  partition_method_t partition_method;
  permute_method_t permute_method;
  grid_size_t grid_size;
  int permute_block_size;
} pdhg_parameters_t;

/* Result of solve_lp_problem() (reference :117-152).  The three arrays are
 * malloc'ed, sized to the original problem, and released (all three) by
 * cupdlpx_result_free(). */
typedef struct {
  int num_variables;
  int num_constraints;
  int num_nonzeros;

  int num_reduced_variables;
  int num_reduced_constraints;
  int num_reduced_nonzeros;

  double *primal_solution;
  double *dual_solution;
  double *reduced_cost;

  int total_count;
  double rescaling_time_sec;
  double cumulative_time_sec;
  double presolve_time;
  int presolve_status;

  double absolute_primal_residual;
  double relative_primal_residual;
  double absolute_dual_residual;
  double relative_dual_residual;
  double primal_objective_value;
  double dual_objective_value;
  double objective_gap;
  double relative_objective_gap;
  double max_primal_ray_infeasibility;
  double max_dual_ray_infeasibility;
  double primal_ray_linear_objective;
  double dual_ray_objective;
  termination_reason_t termination_reason;
  double feasibility_polishing_time;
  int feasibility_iteration;
} cupdlpx_result_t;

/* Input matrix formats accepted by create_lp_problem (reference :155-160). */
typedef enum {
  matrix_dense = 0,
  matrix_csr = 1,
  matrix_csc = 2,
  matrix_coo = 3
} matrix_format_t;

/* Borrowed view of a constraint matrix (reference :163-197). */
typedef struct {
  int m; /* num_constraints */
  int n; /* num_variables */
  matrix_format_t fmt;

  /* entries with |a| <= zero_tolerance are dropped (dense default 1e-12,
   * CSC/COO default 0, CSR copied as given) */
  double zero_tolerance;

  union MatrixData {
    struct MatrixDense { /* row-major m*n */
      const double *A;
    } dense;

    struct MatrixCSR {
      int nnz;
      const int *row_ptr;
      const int *col_ind;
      const double *vals;
    } csr;

    struct MatrixCSC {
      int nnz;
      const int *col_ptr;
      const int *row_ind;
      const double *vals;
    } csc;

    struct MatrixCOO {
      int nnz;
      const int *row_ind;
      const int *col_ind;
      const double *vals;
    } coo;
  } data;
} matrix_desc_t;

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* CUPDLPX_GB300_TYPES_H */
