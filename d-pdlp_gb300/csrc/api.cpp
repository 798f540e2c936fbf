// api.cpp -- the drop-in C API (include/cupdlpx.h) and its extensions
// (include/pdlp_gb300.h).
//
// Interface follows the reference src/cupdlpx.c:26-198 and the host helpers
// of src/utils.cu:295-501, :816-1013.  Every CUDA failure becomes a NULL /
// negative return with a message (stderr and pdlp_last_error()) instead of
// exit().
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <chrono>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "cupdlpx.h"
#include "pdlp_gb300.h"
#include "runtime.h"
#include "solver.cuh"

struct pdlp_device_problem {
  std::unique_ptr<pdlp::DevProblem> P;
};

namespace {

thread_local std::string g_last_error;

void set_error(const std::string &msg) {
  g_last_error = msg;
  fprintf(stderr, "[cupdlpx-gb300] %s\n", msg.c_str());
}

template <class T>
T *xmalloc(size_t count) {
  T *p = (T *)malloc(sizeof(T) * (count ? count : 1));
  if (!p) throw std::bad_alloc();
  return p;
}

void fill_or_copy(double **dst, int n, const double *src, double fill) {
  *dst = xmalloc<double>((size_t)n);
  if (src) memcpy(*dst, src, (size_t)n * sizeof(double));
  else
    for (int i = 0; i < n; ++i) (*dst)[i] = fill;
}

// dense (row-major) -> CSR, |a| > tol kept, default tol 1e-12
// (reference src/utils.cu:826-859)
int dense_to_csr(const matrix_desc_t *d, int **rp, int **ci, double **v, int *nnz_out) {
  const int m = d->m, n = d->n;
  const double tol = d->zero_tolerance > 0 ? d->zero_tolerance : 1e-12;
  const double *A = d->data.dense.A;
  long nnz = 0;
  for (long i = 0; i < (long)m * n; ++i)
    if (fabs(A[i]) > tol) ++nnz;
  *rp = xmalloc<int>((size_t)m + 1);
  *ci = xmalloc<int>((size_t)nnz);
  *v = xmalloc<double>((size_t)nnz);
  int k = 0;
  for (int i = 0; i < m; ++i) {
    (*rp)[i] = k;
    const double *row = A + (long)i * n;
    for (int j = 0; j < n; ++j)
      if (fabs(row[j]) > tol) {
        (*ci)[k] = j;
        (*v)[k] = row[j];
        ++k;
      }
  }
  (*rp)[m] = k;
  *nnz_out = k;
  return 0;
}

// CSC -> CSR by counting sort over rows, default tol 0 (keep everything)
// (reference src/utils.cu:862-922)
int csc_to_csr(const matrix_desc_t *d, int **rp, int **ci, double **v, int *nnz_out) {
  const int m = d->m, n = d->n;
  const int *cp = d->data.csc.col_ptr, *ri = d->data.csc.row_ind;
  const double *x = d->data.csc.vals;
  const double tol = d->zero_tolerance > 0 ? d->zero_tolerance : 0.0;
  // the column pointer must describe n columns over the declared non-zeros
  if (!cp || cp[0] != 0 || cp[n] != d->data.csc.nnz) return -1;
  for (int j = 0; j < n; ++j)
    if (cp[j] > cp[j + 1]) return -1;
  std::vector<int> cnt((size_t)m + 1, 0);
  int nnz = 0;
  for (int j = 0; j < n; ++j)
    for (int k = cp[j]; k < cp[j + 1]; ++k) {
      if (ri[k] < 0 || ri[k] >= m) return -1;
      if (tol > 0 && fabs(x[k]) <= tol) continue;
      ++cnt[ri[k] + 1];
      ++nnz;
    }
  for (int i = 0; i < m; ++i) cnt[i + 1] += cnt[i];
  *rp = xmalloc<int>((size_t)m + 1);
  *ci = xmalloc<int>((size_t)nnz);
  *v = xmalloc<double>((size_t)nnz);
  memcpy(*rp, cnt.data(), ((size_t)m + 1) * sizeof(int));
  for (int j = 0; j < n; ++j)
    for (int k = cp[j]; k < cp[j + 1]; ++k) {
      if (tol > 0 && fabs(x[k]) <= tol) continue;
      int pos = cnt[ri[k]]++;
      (*ci)[pos] = j;
      (*v)[pos] = x[k];
    }
  *nnz_out = nnz;
  return 0;
}

// COO -> CSR, stable in input order within a row, default tol 0
// (reference src/utils.cu:925-1013)
int coo_to_csr(const matrix_desc_t *d, int **rp, int **ci, double **v, int *nnz_out) {
  const int m = d->m, n = d->n, nin = d->data.coo.nnz;
  const int *r = d->data.coo.row_ind, *c = d->data.coo.col_ind;
  const double *x = d->data.coo.vals;
  const double tol = d->zero_tolerance > 0 ? d->zero_tolerance : 0.0;
  std::vector<int> cnt((size_t)m + 1, 0);
  int nnz = 0;
  for (int k = 0; k < nin; ++k) {
    if (tol > 0 && fabs(x[k]) <= tol) continue;
    if (r[k] < 0 || r[k] >= m || c[k] < 0 || c[k] >= n) return -1;
    ++cnt[r[k] + 1];
    ++nnz;
  }
  for (int i = 0; i < m; ++i) cnt[i + 1] += cnt[i];
  *rp = xmalloc<int>((size_t)m + 1);
  *ci = xmalloc<int>((size_t)nnz);
  *v = xmalloc<double>((size_t)nnz);
  memcpy(*rp, cnt.data(), ((size_t)m + 1) * sizeof(int));
  for (int k = 0; k < nin; ++k) {
    if (tol > 0 && fabs(x[k]) <= tol) continue;
    int pos = cnt[r[k]]++;
    (*ci)[pos] = c[k];
    (*v)[pos] = x[k];
  }
  *nnz_out = nnz;
  return 0;
}

const char *reason_name(termination_reason_t r) {
  switch (r) {
    case TERMINATION_REASON_OPTIMAL: return "OPTIMAL";
    case TERMINATION_REASON_PRIMAL_INFEASIBLE: return "PRIMAL_INFEASIBLE";
    case TERMINATION_REASON_DUAL_INFEASIBLE: return "DUAL_INFEASIBLE";
    case TERMINATION_REASON_INFEASIBLE_OR_UNBOUNDED: return "INFEASIBLE_OR_UNBOUNDED";
    case TERMINATION_REASON_TIME_LIMIT: return "TIME_LIMIT";
    case TERMINATION_REASON_ITERATION_LIMIT: return "ITERATION_LIMIT";
    case TERMINATION_REASON_UNSPECIFIED: return "UNSPECIFIED";
    case TERMINATION_REASON_FEAS_POLISH_SUCCESS: return "FEAS_POLISH_SUCCESS";
    default: return "UNKNOWN";
  }
}

const char *kRule =
    "---------------------------------------------------------------------------------------\n";

// Banner and non-default settings (reference src/utils.cu:352-423)
void print_initial_info(const pdhg_parameters_t *p, const lp_problem_t *prob) {
  if (!p->verbose) return;
  pdhg_parameters_t def;
  set_default_parameters(&def);
  printf("%s", kRule);
  printf("                   D-PDLP drop-in: restarted Halpern PDHG on GB300 (sm_103a)\n");
  printf("%s", kRule);
  printf("problem: %d rows, %d columns, %d nonzeros\n", prob->num_constraints,
         prob->num_variables, prob->constraint_matrix_num_nonzeros);
  printf("settings:\n");
  printf("  iter_limit         : %d\n", p->termination_criteria.iteration_limit);
  printf("  time_limit         : %.2f sec\n", p->termination_criteria.time_sec_limit);
  printf("  eps_opt            : %.1e\n", p->termination_criteria.eps_optimal_relative);
  printf("  eps_feas           : %.1e\n", p->termination_criteria.eps_feasible_relative);
  printf("  eps_infeas_detect  : %.1e\n", p->termination_criteria.eps_infeasible);
  if (p->optimality_norm != def.optimality_norm)
    printf("  optimality_norm    : %s\n", p->optimality_norm == NORM_TYPE_L_INF ? "L_inf" : "L2");
  auto di = [](const char *name, int cur, int dv) {
    if (cur != dv) printf("  %-18s : %d\n", name, cur);
  };
  auto dd = [](const char *name, double cur, double dv) {
    if (fabs(cur - dv) > 1e-9) printf("  %-18s : %.1e\n", name, cur);
  };
  auto db = [](const char *name, bool cur, bool dv) {
    if (cur != dv) printf("  %-18s : %s\n", name, cur ? "on" : "off");
  };
  di("l_inf_ruiz_iter", p->l_inf_ruiz_iterations, def.l_inf_ruiz_iterations);
  dd("pock_chambolle_alpha", p->pock_chambolle_alpha, def.pock_chambolle_alpha);
  db("has_pock_chambolle_alpha", p->has_pock_chambolle_alpha, def.has_pock_chambolle_alpha);
  db("bound_obj_rescaling", p->bound_objective_rescaling, def.bound_objective_rescaling);
  di("sv_max_iter", p->sv_max_iter, def.sv_max_iter);
  dd("sv_tol", p->sv_tol, def.sv_tol);
  di("evaluation_freq", p->termination_evaluation_frequency,
     def.termination_evaluation_frequency);
  db("feasibility_polishing", p->feasibility_polishing, def.feasibility_polishing);
  dd("eps_feas_polish_relative", p->termination_criteria.eps_feas_polish_relative,
     def.termination_criteria.eps_feas_polish_relative);
  printf("%s", kRule);
  printf("%s | %s | %s | %s \n", "   runtime    ", "    objective     ",
         "  absolute residuals   ", "  relative residuals   ");
  printf("%s %s | %s %s | %s %s %s | %s %s %s \n", "  iter", "  time ", " pr obj ",
         "  du obj ", " pr res", " du res", "  gap  ", " pr res", " du res", "  gap  ");
  printf("%s", kRule);
}

// Summary (reference src/utils.cu:427-476); printed for every solve, as the
// reference does.
void final_log(const cupdlpx_result_t *r, const pdhg_parameters_t *p) {
  if (p->verbose) printf("%s", kRule);
  printf("Solution Summary\n");
  printf("  Status             : %s\n", reason_name(r->termination_reason));
  if (p->presolve) printf("  Presolve time      : %.3g sec\n", r->presolve_time);
  printf("  Solve time         : %.3g sec\n", r->cumulative_time_sec);
  printf("  Iterations         : %d\n", r->total_count);
  printf("  Primal objective   : %.10g\n", r->primal_objective_value);
  printf("  Dual objective     : %.10g\n", r->dual_objective_value);
  printf("  Objective gap      : %.3e\n", r->relative_objective_gap);
  printf("  Primal infeas      : %.3e\n", r->relative_primal_residual);
  printf("  Dual infeas        : %.3e\n", r->relative_dual_residual);
  fflush(stdout);
}

std::once_flag g_presolve_notice;

bool quiet_summary() {
  const char *e = getenv("PDLP_QUIET");
  return e && e[0] && e[0] != '0';
}

struct StreamGuard {
  cudaStream_t s = nullptr;
  StreamGuard() { PDLP_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)); }
  ~StreamGuard() {
    if (s) cudaStreamDestroy(s);
  }
};

// Feasibility polishing after an FP64 solve (reference src/pdlp_core_op.cu:
// 862-930): when the solve's relative residuals are not both below
// eps_feas_polish_relative, PDHG runs on the primal feasibility problem
// (objective 0) and then on the dual one (finite bounds 0), each from the
// solve's iterates with the initial primal weight, and the solve adopts each
// side that reaches the tolerance.
void feasibility_polish(const pdlp::DevProblem &P, const pdhg_parameters_t &p, cudaStream_t st,
                        pdlp::Solve<double> &s, double &seconds, int &iterations) {
  auto t0 = std::chrono::steady_clock::now();
  const double eps = p.termination_criteria.eps_feas_polish_relative;
  pdlp::Kkt k = s.last_kkt();
  if (k.rel_p < eps && k.rel_d < eps) {
    if (!quiet_summary())
      printf("Skipping feasibility polishing as the solution is already sufficiently feasible.\n");
    return;
  }
  const double w0 = p.bound_objective_rescaling
                        ? 1.0
                        : (s.dev().cnorm + 1.0) / (s.dev().bnorm + 1.0);
  for (int mode = 1; mode <= 2; ++mode) {
    pdlp::Solve<double> ps(p, st, P, 0);
    ps.prepare();
    ps.init_step(s.sigma_max(), w0);
    ps.polish_init(s, mode);
    ps.run();
    if (ps.reason() == TERMINATION_REASON_FEAS_POLISH_SUCCESS) s.adopt_polish(ps, mode);
    iterations += ps.total_count() - 1;
  }
  s.finish_polish();
  seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

cupdlpx_result_t *run_solve(const pdlp::DevProblem &P, const pdhg_parameters_t &p,
                            cudaStream_t st, double *trace, int trace_cap, int *trace_len,
                            pdlp_solve_info_t *info,
                            std::chrono::steady_clock::time_point t0) {
  pdlp::Solve<double> s(p, st, P, trace ? trace_cap : 0);
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  if (info) {
    PDLP_CUDA(cudaEventCreate(&ev0));
    PDLP_CUDA(cudaEventCreate(&ev1));
    PDLP_CUDA(cudaEventRecord(ev0, st));
  }
  s.prepare();
  auto t1 = std::chrono::steady_clock::now();
  s.init_step();
  auto t2 = std::chrono::steady_clock::now();
  s.run();
  double polish_sec = 0.0;
  int polish_iters = 0;
  const int why = s.reason();
  if (p.feasibility_polishing && why != TERMINATION_REASON_PRIMAL_INFEASIBLE &&
      why != TERMINATION_REASON_DUAL_INFEASIBLE)
    feasibility_polish(P, p, st, s, polish_sec, polish_iters);
  cupdlpx_result_t *r = s.result();
  if (r) {
    r->feasibility_polishing_time = polish_sec;
    r->feasibility_iteration = polish_iters;
  }
  auto t3 = std::chrono::steady_clock::now();
  if (info) {
    PDLP_CUDA(cudaEventRecord(ev1, st));
    PDLP_CUDA(cudaEventSynchronize(ev1));
    float ms = 0.f;
    PDLP_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
    info->device_seconds = ms * 1e-3;
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
  }
  if (trace && trace_len) {
    std::vector<double> tr = s.trace();
    int len = (int)(tr.size() / PDLP_TRACE_WIDTH);
    if (len > trace_cap) len = trace_cap;
    memcpy(trace, tr.data(), (size_t)len * PDLP_TRACE_WIDTH * sizeof(double));
    *trace_len = len;
  }
  if (info) {
    info->power_iterations = s.power_iterations();
    info->sigma_max = s.sigma_max();
    info->setup_seconds = std::chrono::duration<double>(t1 - t0).count();
    info->rescale_seconds = s.rescale_seconds();
    info->power_seconds = std::chrono::duration<double>(t2 - t1).count();
    info->loop_seconds = s.loop_seconds();
    info->total_seconds = std::chrono::duration<double>(t3 - t0).count();
    info->graphs = s.graph_count();
    info->kernel_launches = s.kernel_launches();
    info->precision = PDLP_PRECISION_FP64;
    info->primal_step_ms = s.live_primal_ms();
    info->dual_step_ms = s.live_dual_ms();
    info->timed_chunks = s.live_samples();
    info->spmv_kernel_A = s.pipe_A() ? 1 : 0;
    info->spmv_kernel_AT = s.pipe_AT() ? 1 : 0;
    for (int i = 0; i < 4; ++i) info->tune_ms[i] = s.tune_ms(i);
  }
  return r;
}

cupdlpx_result_t *run_refined(const pdlp::DevProblem &P, const pdhg_parameters_t &p,
                              const pdlp_options_t &o, cudaStream_t st,
                              pdlp_solve_info_t *info,
                              std::chrono::steady_clock::time_point t0) {
  pdlp::RefineOptions ro;
  if (o.max_refinements > 0) ro.max_rounds = o.max_refinements;
  ro.inner_eps = o.inner_eps;
  ro.fp64_iterates = o.precision == PDLP_PRECISION_FP32_MATRIX;
  pdlp::RefineReport rep;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  PDLP_CUDA(cudaEventCreate(&ev0));
  PDLP_CUDA(cudaEventCreate(&ev1));
  PDLP_CUDA(cudaEventRecord(ev0, st));
  cupdlpx_result_t *r = pdlp::solve_refined(P, p, ro, st, &rep);
  PDLP_CUDA(cudaEventRecord(ev1, st));
  PDLP_CUDA(cudaEventSynchronize(ev1));
  float ms = 0.f;
  PDLP_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  if (info) {
    info->device_seconds = ms * 1e-3;
    info->loop_seconds = rep.seconds;
    info->total_seconds =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    info->kernel_launches = rep.kernel_launches;
    info->refinement_rounds = rep.rounds;
    info->power_iterations = rep.power_iterations;
    info->sigma_max = rep.sigma_max;
    info->precision = o.precision;
    info->timed_chunks = rep.timed_chunks;
    info->fp64_finish = rep.fp64_finish ? 1 : 0;
    info->spmv_kernel_A = rep.kernel_A;
    info->spmv_kernel_AT = rep.kernel_AT;
    for (int q = 0; q < 4; ++q) info->tune_ms[q] = rep.tune_ms[q];
    if (rep.timed_chunks > 0) {
      info->primal_step_ms = rep.timed_primal_ms_sum / rep.timed_chunks;
      info->dual_step_ms = rep.timed_dual_ms_sum / rep.timed_chunks;
    }
  }
  return r;
}

pdlp_options_t env_options() {
  pdlp_options_t o;
  memset(&o, 0, sizeof(o));
  const char *e = getenv("PDLP_PRECISION");
  if (e && (strcmp(e, "fp32") == 0 || strcmp(e, "FP32") == 0))
    o.precision = PDLP_PRECISION_FP32_REFINE;
  if (e && (strcmp(e, "fp32m") == 0 || strcmp(e, "FP32M") == 0))
    o.precision = PDLP_PRECISION_FP32_MATRIX;
  return o;
}

bool prepare_params(const pdhg_parameters_t *params, pdhg_parameters_t &p) {
  if (params) p = *params;
  else set_default_parameters(&p);
  if (p.termination_evaluation_frequency <= 0) {
    set_error("solve: termination_evaluation_frequency must be positive.");
    return false;
  }
  if (p.presolve)
    std::call_once(g_presolve_notice, [] {
      fprintf(stderr,
              "[cupdlpx-gb300] presolve requested: this library has no presolver; "
              "solving the original problem.\n");
    });
  return true;
}

cupdlpx_result_t *solve_impl(const lp_problem_t *prob, const pdhg_parameters_t *params,
                             double *trace, int trace_cap, int *trace_len,
                             pdlp_solve_info_t *info, const pdlp_options_t *opts) {
  if (!prob) {
    set_error("solve_lp_problem: invalid arguments.");
    return nullptr;
  }
  pdhg_parameters_t p;
  if (!prepare_params(params, p)) return nullptr;
  auto t0 = std::chrono::steady_clock::now();
  try {
    print_initial_info(&p, prob);
    StreamGuard sg;
    std::unique_ptr<pdlp::DevProblem> P(pdlp::upload_problem(prob, sg.s));
    pdlp_options_t o = opts ? *opts : env_options();
    cupdlpx_result_t *r =
        o.precision != PDLP_PRECISION_FP64
            ? run_refined(*P, p, o, sg.s, info, t0)
            : run_solve(*P, p, sg.s, trace, trace_cap, trace_len, info, t0);
    if (!quiet_summary()) final_log(r, &p);
    return r;
  } catch (const std::exception &e) {
    set_error(std::string("solve failed: ") + e.what());
    cudaGetLastError();  // clear a sticky launch error of this thread
    return nullptr;
  }
}

}  // namespace

namespace pdlp {

cupdlpx_result_t *solve_uploaded(const DevProblem &P, const pdhg_parameters_t &p,
                                 const pdlp_options_t &o, cudaStream_t st,
                                 pdlp_solve_info_t *info) {
  auto t0 = std::chrono::steady_clock::now();
  return o.precision != PDLP_PRECISION_FP64
             ? run_refined(P, p, o, st, info, t0)
             : run_solve(P, p, st, nullptr, 0, nullptr, info, t0);
}

bool resolve_parameters(const pdhg_parameters_t *params, pdhg_parameters_t &p) {
  return prepare_params(params, p);
}

void record_error(const std::string &msg) { set_error(msg); }

}  // namespace pdlp

extern "C" {

lp_problem_t *create_lp_problem(const double *objective_c, const matrix_desc_t *A_desc,
                                const double *con_lb, const double *con_ub,
                                const double *var_lb, const double *var_ub,
                                const double *objective_constant) {
  if (!A_desc || A_desc->m < 0 || A_desc->n < 0) {
    set_error("create_lp_problem: invalid matrix descriptor.");
    return nullptr;
  }
  lp_problem_t *prob = (lp_problem_t *)calloc(1, sizeof(lp_problem_t));
  if (!prob) return nullptr;
  try {
    prob->num_variables = A_desc->n;
    prob->num_constraints = A_desc->m;
    int rc = 0;
    switch (A_desc->fmt) {
      case matrix_dense:
        rc = dense_to_csr(A_desc, &prob->constraint_matrix_row_pointers,
                          &prob->constraint_matrix_col_indices,
                          &prob->constraint_matrix_values,
                          &prob->constraint_matrix_num_nonzeros);
        break;
      case matrix_csc:
        rc = csc_to_csr(A_desc, &prob->constraint_matrix_row_pointers,
                        &prob->constraint_matrix_col_indices, &prob->constraint_matrix_values,
                        &prob->constraint_matrix_num_nonzeros);
        if (rc) set_error("CSC->CSR failed: row index out of range.");
        break;
      case matrix_coo:
        rc = coo_to_csr(A_desc, &prob->constraint_matrix_row_pointers,
                        &prob->constraint_matrix_col_indices, &prob->constraint_matrix_values,
                        &prob->constraint_matrix_num_nonzeros);
        if (rc) set_error("COO->CSR failed: index out of range.");
        break;
      case matrix_csr: {
        const int m = A_desc->m, nnz = A_desc->data.csr.nnz;
        prob->constraint_matrix_num_nonzeros = nnz;
        prob->constraint_matrix_row_pointers = xmalloc<int>((size_t)m + 1);
        prob->constraint_matrix_col_indices = xmalloc<int>((size_t)nnz);
        prob->constraint_matrix_values = xmalloc<double>((size_t)nnz);
        memcpy(prob->constraint_matrix_row_pointers, A_desc->data.csr.row_ptr,
               ((size_t)m + 1) * sizeof(int));
        if (nnz) {
          memcpy(prob->constraint_matrix_col_indices, A_desc->data.csr.col_ind,
                 (size_t)nnz * sizeof(int));
          memcpy(prob->constraint_matrix_values, A_desc->data.csr.vals,
                 (size_t)nnz * sizeof(double));
        }
        break;
      }
      default:
        set_error("create_lp_problem: unsupported matrix format " +
                  std::to_string((int)A_desc->fmt) + ".");
        rc = -1;
    }
    if (rc) {
      lp_problem_free(prob);
      return nullptr;
    }
    prob->objective_constant = objective_constant ? *objective_constant : 0.0;
    fill_or_copy(&prob->objective_vector, prob->num_variables, objective_c, 0.0);
    fill_or_copy(&prob->variable_lower_bound, prob->num_variables, var_lb, -INFINITY);
    fill_or_copy(&prob->variable_upper_bound, prob->num_variables, var_ub, INFINITY);
    fill_or_copy(&prob->constraint_lower_bound, prob->num_constraints, con_lb, -INFINITY);
    fill_or_copy(&prob->constraint_upper_bound, prob->num_constraints, con_ub, INFINITY);
    return prob;
  } catch (const std::bad_alloc &) {
    set_error("create_lp_problem: out of host memory.");
    lp_problem_free(prob);
    return nullptr;
  }
}

void set_start_values(lp_problem_t *prob, const double *primal, const double *dual) {
  if (!prob) return;
  free(prob->primal_start);
  free(prob->dual_start);
  prob->primal_start = nullptr;
  prob->dual_start = nullptr;
  if (primal) {
    prob->primal_start = (double *)malloc(sizeof(double) * (prob->num_variables ? prob->num_variables : 1));
    if (prob->primal_start)
      memcpy(prob->primal_start, primal, sizeof(double) * (size_t)prob->num_variables);
  }
  if (dual) {
    prob->dual_start = (double *)malloc(sizeof(double) * (prob->num_constraints ? prob->num_constraints : 1));
    if (prob->dual_start)
      memcpy(prob->dual_start, dual, sizeof(double) * (size_t)prob->num_constraints);
  }
}

cupdlpx_result_t *solve_lp_problem(const lp_problem_t *prob, const pdhg_parameters_t *params) {
  return solve_impl(prob, params, nullptr, 0, nullptr, nullptr, nullptr);
}

cupdlpx_result_t *pdlp_solve_opts(const lp_problem_t *prob, const pdhg_parameters_t *params,
                                  const pdlp_options_t *opts, pdlp_solve_info_t *info) {
  if (info) memset(info, 0, sizeof(*info));
  pdlp_options_t o;
  memset(&o, 0, sizeof(o));
  return solve_impl(prob, params, nullptr, 0, nullptr, info, opts ? opts : &o);
}

void set_default_parameters(pdhg_parameters_t *p) {
  if (!p) return;
  memset(p, 0, sizeof(*p));
  p->l_inf_ruiz_iterations = 10;
  p->has_pock_chambolle_alpha = true;
  p->pock_chambolle_alpha = 1.0;
  p->bound_objective_rescaling = true;
  p->verbose = false;
  p->termination_evaluation_frequency = 200;
  p->feasibility_polishing = false;
  p->reflection_coefficient = 1.0;
  p->sv_max_iter = 5000;
  p->sv_tol = 1e-4;
  p->termination_criteria.eps_optimal_relative = 1e-4;
  p->termination_criteria.eps_feasible_relative = 1e-4;
  p->termination_criteria.eps_infeasible = 1e-10;
  p->termination_criteria.time_sec_limit = 3600.0;
  p->termination_criteria.iteration_limit = 2147483647;
  p->termination_criteria.eps_feas_polish_relative = 1e-6;
  p->restart_params.artificial_restart_threshold = 0.36;
  p->restart_params.sufficient_reduction_for_restart = 0.2;
  p->restart_params.necessary_reduction_for_restart = 0.5;
  p->restart_params.k_p = 0.99;
  p->restart_params.k_i = 0.01;
  p->restart_params.k_d = 0.0;
  p->restart_params.i_smooth = 0.3;
  p->optimality_norm = NORM_TYPE_L2;
  p->presolve = true;
  p->grid_size.row_dims = 1;
  p->grid_size.col_dims = 1;
  p->grid_size.decided = false;
  p->partition_method = NNZ_BALANCE_PARTITION;
  p->permute_method = BLOCK_RANDOM_PERMUTATION;
  p->permute_block_size = 256;
}

void cupdlpx_result_free(cupdlpx_result_t *r) {
  if (!r) return;
  free(r->primal_solution);
  free(r->dual_solution);
  free(r->reduced_cost);
  free(r);
}

void lp_problem_free(lp_problem_t *prob) {
  if (!prob) return;
  free(prob->constraint_matrix_row_pointers);
  free(prob->constraint_matrix_col_indices);
  free(prob->constraint_matrix_values);
  free(prob->variable_lower_bound);
  free(prob->variable_upper_bound);
  free(prob->objective_vector);
  free(prob->constraint_lower_bound);
  free(prob->constraint_upper_bound);
  free(prob->primal_start);
  free(prob->dual_start);
  memset(prob, 0, sizeof(*prob));
  free(prob);
}

cupdlpx_result_t *pdlp_solve_ex(const lp_problem_t *prob, const pdhg_parameters_t *params,
                                double *trace, int trace_cap, int *trace_len,
                                pdlp_solve_info_t *info) {
  if (trace_len) *trace_len = 0;
  if (info) memset(info, 0, sizeof(*info));
  pdlp_options_t o;
  memset(&o, 0, sizeof(o));
  return solve_impl(prob, params, trace, trace_cap, trace_len, info, &o);
}

const char *pdlp_last_error(void) { return g_last_error.c_str(); }

const char *pdlp_termination_reason_to_string(termination_reason_t r) { return reason_name(r); }

int pdlp_gpu_rescale(const lp_problem_t *prob, const pdhg_parameters_t *params, double *vals,
                     double *c, double *lv, double *uv, double *lc, double *uc, double *con,
                     double *var, double *cbr, double *obr) {
  if (!prob || !params) return -1;
  try {
    StreamGuard sg;
    std::unique_ptr<pdlp::DevProblem> P(pdlp::upload_problem(prob, sg.s));
    pdlp::Solve<double> s(*params, sg.s, *P, 0);
    s.prepare();
    const pdlp::Dev<double> &d = s.dev();
    const int n = d.n, m = d.m, nnz = s.A().nnz;
    auto get = [&](double *dst, const double *src, int cnt) {
      if (cnt > 0) {
        PDLP_CUDA(cudaMemcpyAsync(dst, src, (size_t)cnt * 8, cudaMemcpyDeviceToHost, sg.s));
        PDLP_CUDA(cudaStreamSynchronize(sg.s));
      }
    };
    get(vals, s.A64().val, nnz);
    get(c, d.c, n);
    get(lv, d.lv, n);
    get(uv, d.uv, n);
    get(lc, d.lc, m);
    get(uc, d.uc, m);
    get(con, d.Dr, m);
    get(var, d.Dc, n);
    *cbr = d.cb;
    *obr = d.ob;
    return 0;
  } catch (const std::exception &e) {
    set_error(std::string("pdlp_gpu_rescale: ") + e.what());
    return -2;
  }
}

int pdlp_gpu_power_method(const lp_problem_t *prob, const pdhg_parameters_t *params,
                          double *sigma_max, int *iterations) {
  if (!prob || !params) return -1;
  try {
    StreamGuard sg;
    std::unique_ptr<pdlp::DevProblem> P(pdlp::upload_problem(prob, sg.s));
    pdlp::Solve<double> s(*params, sg.s, *P, 0);
    s.prepare();
    s.init_step();
    *sigma_max = s.sigma_max();
    *iterations = s.power_iterations();
    return 0;
  } catch (const std::exception &e) {
    set_error(std::string("pdlp_gpu_power_method: ") + e.what());
    return -2;
  }
}

pdlp_device_problem_t *pdlp_device_problem_create(const lp_problem_t *prob) {
  if (!prob) {
    set_error("pdlp_device_problem_create: NULL problem.");
    return nullptr;
  }
  try {
    StreamGuard sg;
    auto dp = std::make_unique<pdlp_device_problem>();
    dp->P.reset(pdlp::upload_problem(prob, sg.s));
    dp->P->owner = cudaStreamPerThread;  // sg.s ends here; the upload has finished
    return dp.release();
  } catch (const std::exception &e) {
    set_error(std::string("pdlp_device_problem_create: ") + e.what());
    cudaGetLastError();
    return nullptr;
  }
}

void pdlp_device_problem_free(pdlp_device_problem_t *dp) { delete dp; }

long long pdlp_device_problem_bytes(const pdlp_device_problem_t *dp) {
  return dp && dp->P ? (long long)dp->P->bytes : 0;
}

cupdlpx_result_t *pdlp_device_problem_solve(pdlp_device_problem_t *dp,
                                            const pdhg_parameters_t *params,
                                            pdlp_solve_info_t *info) {
  pdlp_options_t o;
  memset(&o, 0, sizeof(o));
  return pdlp_device_problem_solve_opts(dp, params, &o, info);
}

cupdlpx_result_t *pdlp_device_problem_solve_opts(pdlp_device_problem_t *dp,
                                                 const pdhg_parameters_t *params,
                                                 const pdlp_options_t *opts,
                                                 pdlp_solve_info_t *info) {
  if (!dp || !dp->P) {
    set_error("pdlp_device_problem_solve: NULL handle.");
    return nullptr;
  }
  if (info) memset(info, 0, sizeof(*info));
  pdhg_parameters_t p;
  if (!prepare_params(params, p)) return nullptr;
  auto t0 = std::chrono::steady_clock::now();
  try {
    StreamGuard sg;
    pdlp_options_t o;
    memset(&o, 0, sizeof(o));
    if (opts) o = *opts;
    cupdlpx_result_t *r = o.precision != PDLP_PRECISION_FP64
                              ? run_refined(*dp->P, p, o, sg.s, info, t0)
                              : run_solve(*dp->P, p, sg.s, nullptr, 0, nullptr, info, t0);
    if (!quiet_summary()) final_log(r, &p);
    return r;
  } catch (const std::exception &e) {
    set_error(std::string("pdlp_device_problem_solve: ") + e.what());
    cudaGetLastError();
    return nullptr;
  }
}

int pdlp_device_problem_time_kernels(pdlp_device_problem_t *dp, const pdhg_parameters_t *params,
                                     int reps, double *ms) {
  return pdlp_device_problem_time_kernels_prec(dp, params, PDLP_PRECISION_FP64, reps, ms);
}

int pdlp_device_problem_time_kernels_prec(pdlp_device_problem_t *dp,
                                          const pdhg_parameters_t *params, int precision,
                                          int reps, double *ms) {
  if (!dp || !dp->P || !ms || reps <= 0) return -1;
  pdhg_parameters_t p;
  if (!prepare_params(params, p)) return -1;
  try {
    StreamGuard sg;
    if (precision == PDLP_PRECISION_FP32_MATRIX) {
      pdlp::Solve<double, float> s(p, sg.s, *dp->P, 0);
      s.prepare();
      s.init_step();
      s.time_kernels(reps, ms);
    } else if (precision == PDLP_PRECISION_FP32_REFINE) {
      pdlp::Solve<float> s(p, sg.s, *dp->P, 0);
      s.prepare();
      s.init_step();
      s.time_kernels(reps, ms);
    } else {
      pdlp::Solve<double> s(p, sg.s, *dp->P, 0);
      s.prepare();
      s.init_step();
      s.time_kernels(reps, ms);
    }
    return 0;
  } catch (const std::exception &e) {
    set_error(std::string("pdlp_device_problem_time_kernels: ") + e.what());
    cudaGetLastError();
    return -2;
  }
}

}  // extern "C"
