/* ref_solve -- runs the reference's own single-GPU solve (cuSPARSE/cuBLAS,
 * FP64) on one LP read from a file, as a baseline and parity oracle.
 *
 * TEST AND BENCHMARK INFRASTRUCTURE ONLY: linked with the reference's
 * sources (src/cupdlpx.c, solver.cu, pdlp_core_op.cu, utils.cu,
 * preconditioner.c), never with this project's solver.
 *
 *   ref_solve LP_FILE OUT_FILE [--eps E] [--iter-limit N] [--time-limit S]
 *                              [--verbose]
 *
 * The problem goes through the reference's public API as a caller would:
 * create_lp_problem (matrix_csr) and solve_lp_problem with presolve off
 * (reference include/cupdlpx.h:26-38).  The first solve in a process uses the
 * reference's power-method start vector, the first draws of its global
 * mt19937(1) (src/utils.cu:29-30), so one process runs one solve.
 *
 * LP_FILE layout (little-endian, written by tests/oracle_lib.py):
 *   char magic[8] = "PDLPLP1\0"; int32 m, n, nnz, 0; double c0;
 *   double c[n], lv[n], uv[n], lc[m], uc[m]; int32 row_ptr[m+1], col[nnz];
 *   double val[nnz]
 * OUT_FILE: double x[n], y[m], reduced_cost[n].
 * stdout, last line: "REF_RESULT {json}" with the result scalars and the
 * wall time of solve_lp_problem (host rescaling, upload, transpose, power
 * method, loop and result copy; the CUDA context is created before it). */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include <cuda_runtime_api.h>

#include "cupdlpx.h"

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static int read_all(FILE *f, void *dst, size_t elem, size_t count) {
  return count == 0 || fread(dst, elem, count, f) == count;
}

static const char *reason_name(termination_reason_t r) {
  switch (r) {
    case TERMINATION_REASON_OPTIMAL: return "OPTIMAL";
    case TERMINATION_REASON_PRIMAL_INFEASIBLE: return "PRIMAL_INFEASIBLE";
    case TERMINATION_REASON_DUAL_INFEASIBLE: return "DUAL_INFEASIBLE";
    case TERMINATION_REASON_TIME_LIMIT: return "TIME_LIMIT";
    case TERMINATION_REASON_ITERATION_LIMIT: return "ITERATION_LIMIT";
    case TERMINATION_REASON_FEAS_POLISH_SUCCESS: return "FEAS_POLISH_SUCCESS";
    default: return "UNSPECIFIED";
  }
}

int main(int argc, char **argv) {
  if (argc < 3) {
    fprintf(stderr, "usage: %s LP_FILE OUT_FILE [--eps E] [--iter-limit N] "
                    "[--time-limit S] [--verbose]\n", argv[0]);
    return 2;
  }
  double eps = 1e-4, time_limit = -1.0;
  int iter_limit = -1, verbose = 0;
  for (int i = 3; i < argc; ++i) {
    if (!strcmp(argv[i], "--eps") && i + 1 < argc) eps = atof(argv[++i]);
    else if (!strcmp(argv[i], "--iter-limit") && i + 1 < argc) iter_limit = atoi(argv[++i]);
    else if (!strcmp(argv[i], "--time-limit") && i + 1 < argc) time_limit = atof(argv[++i]);
    else if (!strcmp(argv[i], "--verbose")) verbose = 1;
    else {
      fprintf(stderr, "unknown argument %s\n", argv[i]);
      return 2;
    }
  }
  FILE *f = fopen(argv[1], "rb");
  if (!f) {
    perror(argv[1]);
    return 2;
  }
  char magic[8];
  int hdr[4];
  double c0 = 0.0;
  if (!read_all(f, magic, 1, 8) || memcmp(magic, "PDLPLP1", 8) != 0 ||
      !read_all(f, hdr, sizeof(int), 4) || !read_all(f, &c0, sizeof(double), 1)) {
    fprintf(stderr, "%s: not an LP file\n", argv[1]);
    fclose(f);
    return 2;
  }
  const int m = hdr[0], n = hdr[1], nnz = hdr[2];
  if (m < 0 || n < 0 || nnz < 0) {
    fprintf(stderr, "%s: bad sizes\n", argv[1]);
    fclose(f);
    return 2;
  }
  double *c = malloc(sizeof(double) * (n ? n : 1));
  double *lv = malloc(sizeof(double) * (n ? n : 1));
  double *uv = malloc(sizeof(double) * (n ? n : 1));
  double *lc = malloc(sizeof(double) * (m ? m : 1));
  double *uc = malloc(sizeof(double) * (m ? m : 1));
  int *rp = malloc(sizeof(int) * ((size_t)m + 1));
  int *cj = malloc(sizeof(int) * (nnz ? nnz : 1));
  double *av = malloc(sizeof(double) * (nnz ? nnz : 1));
  if (!c || !lv || !uv || !lc || !uc || !rp || !cj || !av) {
    fprintf(stderr, "out of host memory\n");
    return 2;
  }
  int ok = read_all(f, c, 8, n) && read_all(f, lv, 8, n) && read_all(f, uv, 8, n) &&
           read_all(f, lc, 8, m) && read_all(f, uc, 8, m) && read_all(f, rp, 4, (size_t)m + 1) &&
           read_all(f, cj, 4, nnz) && read_all(f, av, 8, nnz);
  fclose(f);
  if (!ok || rp[0] != 0 || rp[m] != nnz) {
    fprintf(stderr, "%s: truncated or inconsistent LP file\n", argv[1]);
    return 2;
  }
  for (int r = 0; r < m; ++r)
    if (rp[r] > rp[r + 1]) {
      fprintf(stderr, "%s: row pointers decrease at row %d\n", argv[1], r);
      return 2;
    }
  for (int k = 0; k < nnz; ++k)
    if (cj[k] < 0 || cj[k] >= n) {
      fprintf(stderr, "%s: column index out of range at %d\n", argv[1], k);
      return 2;
    }

  matrix_desc_t d;
  memset(&d, 0, sizeof(d));
  d.m = m;
  d.n = n;
  d.fmt = matrix_csr;
  d.zero_tolerance = 0.0;
  d.data.csr.nnz = nnz;
  d.data.csr.row_ptr = rp;
  d.data.csr.col_ind = cj;
  d.data.csr.vals = av;
  lp_problem_t *prob = create_lp_problem(c, &d, lc, uc, lv, uv, &c0);
  if (!prob) {
    fprintf(stderr, "create_lp_problem failed\n");
    return 3;
  }
  pdhg_parameters_t p;
  memset(&p, 0, sizeof(p));  /* the reference leaves some fields unset */
  set_default_parameters(&p);
  p.presolve = false;
  p.verbose = verbose != 0;
  p.termination_criteria.eps_optimal_relative = eps;
  p.termination_criteria.eps_feasible_relative = eps;
  if (iter_limit > 0) p.termination_criteria.iteration_limit = iter_limit;
  if (time_limit > 0) p.termination_criteria.time_sec_limit = time_limit;

  cudaFree(0); /* context creation stays outside the timed call */
  const double t0 = now_s();
  cupdlpx_result_t *r = solve_lp_problem(prob, &p);
  const double wall = now_s() - t0;
  if (!r) {
    fprintf(stderr, "solve_lp_problem returned NULL\n");
    return 4;
  }
  FILE *o = fopen(argv[2], "wb");
  if (!o) {
    perror(argv[2]);
    return 2;
  }
  int wok = fwrite(r->primal_solution, 8, n, o) == (size_t)n &&
            fwrite(r->dual_solution, 8, m, o) == (size_t)m &&
            fwrite(r->reduced_cost, 8, n, o) == (size_t)n;
  fclose(o);
  if (!wok) {
    fprintf(stderr, "%s: write failed\n", argv[2]);
    return 2;
  }
  fflush(stdout);
  printf("REF_RESULT {\"status\": \"%s\", \"total_count\": %d, \"wall_s\": %.6f, "
         "\"cumulative_time_sec\": %.6f, \"rescaling_time_sec\": %.6f, "
         "\"primal_objective_value\": %.17g, \"dual_objective_value\": %.17g, "
         "\"relative_primal_residual\": %.17g, \"relative_dual_residual\": %.17g, "
         "\"relative_objective_gap\": %.17g, \"absolute_primal_residual\": %.17g, "
         "\"absolute_dual_residual\": %.17g, \"objective_gap\": %.17g, "
         "\"m\": %d, \"n\": %d, \"nnz\": %d, \"eps\": %.3g}\n",
         reason_name(r->termination_reason), r->total_count, wall, r->cumulative_time_sec,
         r->rescaling_time_sec, r->primal_objective_value, r->dual_objective_value,
         r->relative_primal_residual, r->relative_dual_residual, r->relative_objective_gap,
         r->absolute_primal_residual, r->absolute_dual_residual, r->objective_gap, m, n, nnz,
         eps);
  fflush(stdout);
  /* the result's reduced_cost is freed here: the reference's
   * cupdlpx_result_free leaves it allocated (src/cupdlpx.c:119-127) */
  free(r->reduced_cost);
  r->reduced_cost = NULL;
  cupdlpx_result_free(r);
  lp_problem_free(prob);
  free(c); free(lv); free(uv); free(lc); free(uc); free(rp); free(cj); free(av);
  return 0;
}
