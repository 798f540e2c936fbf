// oracle.cpp -- CPU FP64 restatement of the reference's single-GPU PDHG solve.
//
// TEST INFRASTRUCTURE ONLY: the oracle of the CUDA solver's parity tests and
// the timed CPU baseline.  Nothing in the product links or calls this file.
//
// It restates, in plain loops:
//   rescaling            reference src/preconditioner.c:89-273
//   state set-up         reference src/pdlp_core_op.cu:42-391
//   step size / power    reference src/pdlp_core_op.cu:638-656, src/utils.cu:66-171
//   PDHG iteration ops   reference src/pdlp_core_op.cu:393-696
//   KKT / infeasibility  reference src/utils.cu:503-813
//   criteria / defaults  reference src/utils.cu:214-329, :492-501
//   driver loop          reference src/solver.cu:32-127
//   result extraction    reference src/pdlp_core_op.cu:31-40, :464-480, :789-859
//   input converters     reference src/utils.cu:816-1013
//
// Library reductions of the reference (cuBLAS nrm2/dot/idamax) are restated
// as sums in a fixed chunk order, so the oracle's own results do not depend
// on the thread count; they differ from cuBLAS only in rounding.
#include "oracle.h"

#include <omp.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>

namespace {

using vec = std::vector<double>;
constexpr long kChunk = 4096;

// Deterministic sum of f(i), i in [0, n): fixed chunks, chunk partials summed
// in order.  Independent of the OpenMP thread count.
template <class F>
double det_sum(long n, F f) {
  if (n <= 0) return 0.0;
  long nch = (n + kChunk - 1) / kChunk;
  std::vector<double> part(nch, 0.0);
#pragma omp parallel for schedule(static)
  for (long c = 0; c < nch; ++c) {
    long lo = c * kChunk, hi = std::min(n, lo + kChunk);
    double s = 0.0;
    for (long i = lo; i < hi; ++i) s += f(i);
    part[c] = s;
  }
  double s = 0.0;
  for (long c = 0; c < nch; ++c) s += part[c];
  return s;
}

template <class F>
double det_max(long n, F f) {  // max of f(i) >= 0
  if (n <= 0) return 0.0;
  long nch = (n + kChunk - 1) / kChunk;
  std::vector<double> part(nch, 0.0);
#pragma omp parallel for schedule(static)
  for (long c = 0; c < nch; ++c) {
    long lo = c * kChunk, hi = std::min(n, lo + kChunk);
    double s = 0.0;
    for (long i = lo; i < hi; ++i) s = std::max(s, f(i));
    part[c] = s;
  }
  double s = 0.0;
  for (long c = 0; c < nch; ++c) s = std::max(s, part[c]);
  return s;
}

double nrm2(const vec &v) {
  return std::sqrt(det_sum((long)v.size(), [&](long i) { return v[i] * v[i]; }));
}
double inf_norm(const vec &v) {
  return det_max((long)v.size(), [&](long i) { return std::fabs(v[i]); });
}
double dot(const vec &a, const vec &b) {
  return det_sum((long)a.size(), [&](long i) { return a[i] * b[i]; });
}
double vsum(const vec &v) {
  return det_sum((long)v.size(), [&](long i) { return v[i]; });
}

struct Csr {
  int rows = 0, cols = 0;
  std::vector<int> p, j;
  vec x;
};

void spmv(const Csr &A, const double *in, double *out) {
#pragma omp parallel for schedule(dynamic, 512)
  for (int r = 0; r < A.rows; ++r) {
    double s = 0.0;
    for (int k = A.p[r]; k < A.p[r + 1]; ++k) s += A.x[k] * in[A.j[k]];
    out[r] = s;
  }
}

void transpose(const Csr &A, Csr &T) {
  T.rows = A.cols;
  T.cols = A.rows;
  int nnz = A.p[A.rows];
  T.p.assign(A.cols + 1, 0);
  T.j.resize(nnz);
  T.x.resize(nnz);
  for (int k = 0; k < nnz; ++k) T.p[A.j[k] + 1]++;
  for (int c = 0; c < A.cols; ++c) T.p[c + 1] += T.p[c];
  std::vector<int> next(T.p.begin(), T.p.end() - 1);
  for (int r = 0; r < A.rows; ++r)
    for (int k = A.p[r]; k < A.p[r + 1]; ++k) {
      int pos = next[A.j[k]]++;
      T.j[pos] = r;
      T.x[pos] = A.x[k];
    }
}

int print_frequency(int iter) {  // reference src/utils.cu:492-501
  int step = 10;
  long long threshold = 1000;
  while (iter >= threshold) {
    step *= 10;
    threshold *= 10;
  }
  return step;
}

// ---------------------------------------------------------------- rescaling
struct Scaled {
  Csr A;  // scaled A (CSR, m x n)
  vec c, lv, uv, lc, uc;
  vec con, var;  // cumulative row / column scalings
  double cb = 1.0, ob = 1.0;
  double seconds = 0.0;
};

// reference src/preconditioner.c:89-110
void scale_problem(Scaled &s, const vec &con, const vec &var) {
  int n = s.A.cols, m = s.A.rows;
  for (int i = 0; i < n; ++i) {
    s.c[i] /= var[i];
    s.uv[i] *= var[i];
    s.lv[i] *= var[i];
  }
  for (int i = 0; i < m; ++i) {
    s.lc[i] /= con[i];
    s.uc[i] /= con[i];
  }
#pragma omp parallel for schedule(dynamic, 512)
  for (int r = 0; r < m; ++r)
    for (int k = s.A.p[r]; k < s.A.p[r + 1]; ++k)
      s.A.x[k] /= (con[r] * var[s.A.j[k]]);
}

constexpr double kScalingEps = 1e-12;  // reference preconditioner.c:24

// reference src/preconditioner.c:112-160 (column maxima taken over the
// transpose pattern; max is order-free, so the result is the same)
void ruiz(Scaled &s, int iters) {
  int n = s.A.cols, m = s.A.rows;
  vec con(m), var(n);
  for (int it = 0; it < iters; ++it) {
    std::fill(var.begin(), var.end(), 0.0);
    std::fill(con.begin(), con.end(), 0.0);
    for (int r = 0; r < m; ++r)
      for (int k = s.A.p[r]; k < s.A.p[r + 1]; ++k) {
        double v = std::fabs(s.A.x[k]);
        int col = s.A.j[k];
        if (v > var[col]) var[col] = v;
        if (v > con[r]) con[r] = v;
      }
    for (int i = 0; i < n; ++i) var[i] = var[i] < kScalingEps ? 1.0 : std::sqrt(var[i]);
    for (int i = 0; i < m; ++i) con[i] = con[i] < kScalingEps ? 1.0 : std::sqrt(con[i]);
    scale_problem(s, con, var);
    for (int i = 0; i < n; ++i) s.var[i] *= var[i];
    for (int i = 0; i < m; ++i) s.con[i] *= con[i];
  }
}

// reference src/preconditioner.c:162-195 (sums accumulated in CSR row order,
// as the reference does)
void pock_chambolle(Scaled &s, double alpha) {
  int n = s.A.cols, m = s.A.rows;
  vec con(m, 0.0), var(n, 0.0);
  for (int r = 0; r < m; ++r)
    for (int k = s.A.p[r]; k < s.A.p[r + 1]; ++k) {
      double v = std::fabs(s.A.x[k]);
      var[s.A.j[k]] += std::pow(v, 2.0 - alpha);
      con[r] += std::pow(v, alpha);
    }
  for (int i = 0; i < n; ++i) var[i] = var[i] < kScalingEps ? 1.0 : std::sqrt(var[i]);
  for (int i = 0; i < m; ++i) con[i] = con[i] < kScalingEps ? 1.0 : std::sqrt(con[i]);
  scale_problem(s, con, var);
  for (int i = 0; i < n; ++i) s.var[i] *= var[i];
  for (int i = 0; i < m; ++i) s.con[i] *= con[i];
}

// reference src/preconditioner.c:197-273
void rescale(const lp_problem_t *p, const pdhg_parameters_t *prm, Scaled &s) {
  auto t0 = std::chrono::steady_clock::now();
  int n = p->num_variables, m = p->num_constraints;
  int nnz = p->constraint_matrix_num_nonzeros;
  s.A.rows = m;
  s.A.cols = n;
  s.A.p.assign(p->constraint_matrix_row_pointers, p->constraint_matrix_row_pointers + m + 1);
  s.A.j.assign(p->constraint_matrix_col_indices, p->constraint_matrix_col_indices + nnz);
  s.A.x.assign(p->constraint_matrix_values, p->constraint_matrix_values + nnz);
  s.c.assign(p->objective_vector, p->objective_vector + n);
  s.lv.assign(p->variable_lower_bound, p->variable_lower_bound + n);
  s.uv.assign(p->variable_upper_bound, p->variable_upper_bound + n);
  s.lc.assign(p->constraint_lower_bound, p->constraint_lower_bound + m);
  s.uc.assign(p->constraint_upper_bound, p->constraint_upper_bound + m);
  s.con.assign(m, 1.0);
  s.var.assign(n, 1.0);
  if (prm->l_inf_ruiz_iterations > 0) ruiz(s, prm->l_inf_ruiz_iterations);
  if (prm->has_pock_chambolle_alpha) pock_chambolle(s, prm->pock_chambolle_alpha);
  if (prm->bound_objective_rescaling) {
    double bsq = 0.0;
    for (int i = 0; i < m; ++i) {
      if (std::isfinite(s.lc[i]) && s.lc[i] != s.uc[i]) bsq += s.lc[i] * s.lc[i];
      if (std::isfinite(s.uc[i])) bsq += s.uc[i] * s.uc[i];
    }
    double osq = 0.0;
    for (int i = 0; i < n; ++i) osq += s.c[i] * s.c[i];
    s.cb = 1.0 / (std::sqrt(bsq) + 1.0);
    s.ob = 1.0 / (std::sqrt(osq) + 1.0);
    for (int i = 0; i < m; ++i) {
      s.lc[i] *= s.cb;
      s.uc[i] *= s.cb;
    }
    for (int i = 0; i < n; ++i) {
      s.lv[i] *= s.cb;
      s.uv[i] *= s.cb;
      s.c[i] *= s.ob;
    }
  } else {
    s.cb = 1.0;
    s.ob = 1.0;
  }
  s.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

void power_start(int m, vec &v) {
  std::mt19937 gen(1);
  std::normal_distribution<double> dist(0.0, 1.0);
  v.resize(m);
  for (int i = 0; i < m; ++i) v[i] = dist(gen);
}

// reference src/utils.cu:66-171
double power_method(const Csr &A, const Csr &AT, const vec &v0, int max_iter,
                    double tol, int *iters_out) {
  int m = A.rows, n = A.cols;
  vec v = v0, q(m), g(n), r(m);
  double sigma_sq = 1.0;
  int it = 0;
  for (it = 0; it < max_iter; ++it) {
    q = v;
    double nv = nrm2(q);
    double inv = 1.0 / nv;
    for (int i = 0; i < m; ++i) q[i] = inv * q[i];
    spmv(AT, q.data(), g.data());
    spmv(A, g.data(), v.data());
    sigma_sq = dot(q, v);
    double neg = -sigma_sq;
    for (int i = 0; i < m; ++i) r[i] = neg * q[i];
    for (int i = 0; i < m; ++i) r[i] = 1.0 * v[i] + r[i];
    double res = nrm2(r);
    if (res < tol) {
      ++it;
      break;
    }
  }
  if (iters_out) *iters_out = it;
  return std::sqrt(sigma_sq);
}

// ---------------------------------------------------------- scalar criteria
// reference src/utils.cu:214-263 (optimality, primal / dual infeasibility,
// iteration and time limits, in that order of precedence)
extern "C" int oracle_termination_decision(const termination_criteria_t *tc, double rel_p,
                                           double rel_d, double rel_gap, double dray_obj,
                                           double max_dray, double pray_obj, double max_pray,
                                           int total, double cum_time) {
  if (rel_d < tc->eps_feasible_relative && rel_p < tc->eps_feasible_relative &&
      rel_gap < tc->eps_optimal_relative)
    return TERMINATION_REASON_OPTIMAL;
  if (dray_obj > 0.0 && max_dray / dray_obj <= tc->eps_infeasible)
    return TERMINATION_REASON_PRIMAL_INFEASIBLE;
  if (pray_obj < 0.0 && max_pray / (-pray_obj) <= tc->eps_infeasible)
    return TERMINATION_REASON_DUAL_INFEASIBLE;
  if (total >= tc->iteration_limit) return TERMINATION_REASON_ITERATION_LIMIT;
  if (cum_time >= tc->time_sec_limit) return TERMINATION_REASON_TIME_LIMIT;
  return TERMINATION_REASON_UNSPECIFIED;
}

// reference src/utils.cu:265-293: restart at the first major evaluation,
// then on sufficient decay, on necessary decay with no progress since the
// last trial, or when the inner count passes the artificial threshold;
// *last_fpe becomes fpe
extern "C" int oracle_restart_decision(const restart_parameters_t *rp, int F, int total,
                                       int inner, double fpe, double init_fpe,
                                       double *last_fpe) {
  bool r = false;
  if (total == F) {
    r = true;
  } else if (total > F) {
    if (fpe <= rp->sufficient_reduction_for_restart * init_fpe) r = true;
    if (fpe <= rp->necessary_reduction_for_restart * init_fpe && fpe > *last_fpe) r = true;
    if (inner >= rp->artificial_restart_threshold * total) r = true;
  }
  *last_fpe = fpe;
  return r ? 1 : 0;
}

// ------------------------------------------------------------------- solver
struct Solver {
  const pdhg_parameters_t &prm;
  int n = 0, m = 0;
  Csr A, AT;
  vec c, lv, uv, lc, uc, lvf, uvf, lcf, ucf, Dr, Dc;
  double cb = 1, ob = 1, c0 = 0, cnorm = 0, bnorm = 0, rescale_sec = 0;
  // iterates and work vectors (names follow the reference state fields)
  vec x0, x, xhat, xref, dprod, lam, dres, dx;
  vec y0, y, yhat, yref, pprod, pslack, pres, dy;
  double eta = 0, omega = 1, best_omega = 1, best_gap = INFINITY;
  double pw_err_sum = 0, pw_last_err = 0;
  double fpe = 0, init_fpe = 0, last_fpe = INFINITY;
  int total = 0, inner = 0;
  bool is_major = false;
  double abs_p = 0, rel_p = 0, abs_d = 0, rel_d = 0, pobj = 0, dobj = 0;
  double gap = 0, rel_gap = 0;
  double max_pray = 0, max_dray = 0, pray_obj = 0, dray_obj = 0;
  double cum_time = 0;
  termination_reason_t reason = TERMINATION_REASON_UNSPECIFIED;

  explicit Solver(const pdhg_parameters_t &p) : prm(p) {}

  // reference src/pdlp_core_op.cu:42-391
  void init(const lp_problem_t *p) {
    Scaled s;
    rescale(p, &prm, s);
    n = p->num_variables;
    m = p->num_constraints;
    A = std::move(s.A);
    transpose(A, AT);
    c = s.c; lv = s.lv; uv = s.uv; lc = s.lc; uc = s.uc;
    Dr = s.con; Dc = s.var; cb = s.cb; ob = s.ob;
    rescale_sec = s.seconds;
    c0 = p->objective_constant;
    auto fin = [](const vec &a) {
      vec o(a.size());
      for (size_t i = 0; i < a.size(); ++i) o[i] = std::isfinite(a[i]) ? a[i] : 0.0;
      return o;
    };
    lcf = fin(lc); ucf = fin(uc); lvf = fin(lv); uvf = fin(uv);
    x0.assign(n, 0); x.assign(n, 0); xhat.assign(n, 0); xref.assign(n, 0);
    dprod.assign(n, 0); lam.assign(n, 0); dres.assign(n, 0); dx.assign(n, 0);
    y0.assign(m, 0); y.assign(m, 0); yhat.assign(m, 0); yref.assign(m, 0);
    pprod.assign(m, 0); pslack.assign(m, 0); pres.assign(m, 0); dy.assign(m, 0);
    if (p->primal_start)
      for (int i = 0; i < n; ++i)
        x0[i] = x[i] = xhat[i] = p->primal_start[i] * Dc[i] * cb;
    if (p->dual_start)
      for (int i = 0; i < m; ++i)
        y0[i] = y[i] = yhat[i] = p->dual_start[i] * Dr[i] * ob;
    // norms of the unscaled data (reference :232-286)
    bool linf = prm.optimality_norm == NORM_TYPE_L_INF;
    double ss = 0, mx = 0;
    for (int i = 0; i < n; ++i) {
      double v = p->objective_vector[i];
      if (linf) mx = std::max(mx, std::fabs(v));
      else ss += v * v;
    }
    cnorm = linf ? mx : std::sqrt(ss);
    ss = 0; mx = 0;
    for (int i = 0; i < m; ++i) {
      double lo = p->constraint_lower_bound[i], up = p->constraint_upper_bound[i];
      if (linf) {
        if (std::isfinite(lo) && lo != up) mx = std::max(mx, std::fabs(lo));
        if (std::isfinite(up)) mx = std::max(mx, std::fabs(up));
      } else {
        if (std::isfinite(lo) && lo != up) ss += lo * lo;
        if (std::isfinite(up)) ss += up * up;
      }
    }
    bnorm = linf ? mx : std::sqrt(ss);
  }

  // reference src/pdlp_core_op.cu:638-656
  void init_step() {
    if (A.p[m] == 0) {
      eta = 1.0;
    } else {
      vec v0;
      power_start(m, v0);
      double smax = power_method(A, AT, v0, prm.sv_max_iter, prm.sv_tol, nullptr);
      eta = 0.998 / smax;
    }
    omega = prm.bound_objective_rescaling ? 1.0 : (cnorm + 1.0) / (bnorm + 1.0);
    best_omega = omega;
  }

  double norm(const vec &v) const {
    return prm.optimality_norm == NORM_TYPE_L_INF ? inf_norm(v) : nrm2(v);
  }

  // reference src/utils.cu:503-531, :639-719
  void compute_residual() {
    spmv(A, xhat.data(), pprod.data());
    spmv(AT, yhat.data(), dprod.data());
#pragma omp parallel for schedule(static)
    for (int i = 0; i < m; ++i) {
      double cl = std::fmax(lc[i], std::fmin(pprod[i], uc[i]));
      pres[i] = (pprod[i] - cl) * Dr[i];
      pslack[i] = std::fmax(yhat[i], 0.0) * lcf[i] + std::fmin(yhat[i], 0.0) * ucf[i];
    }
#pragma omp parallel for schedule(static)
    for (int j = 0; j < n; ++j) dres[j] = (c[j] - dprod[j] - lam[j]) * Dc[j];
    abs_p = norm(pres) / cb;
    abs_d = norm(dres) / ob;
    pobj = dot(c, xhat) / (cb * ob) + c0;
    double base = dot(lam, xhat);
    double ssum = vsum(pslack);
    dobj = (base + ssum) / (cb * ob) + c0;
    rel_p = abs_p / (1.0 + bnorm);
    rel_d = abs_d / (1.0 + cnorm);
    gap = std::fabs(pobj - dobj);
    rel_gap = gap / (1.0 + std::fabs(pobj) + std::fabs(dobj));
  }

  // reference src/utils.cu:533-614, :721-813
  void compute_infeasibility() {
    for (int j = 0; j < n; ++j) {
      if (std::isfinite(lv[j])) dx[j] = std::fmax(dx[j], 0.0);
      if (std::isfinite(uv[j])) dx[j] = std::fmin(dx[j], 0.0);
    }
    for (int i = 0; i < m; ++i) {
      if (!std::isfinite(lc[i])) dy[i] = std::fmin(dy[i], 0.0);
      if (!std::isfinite(uc[i])) dy[i] = std::fmax(dy[i], 0.0);
    }
    double pinf = inf_norm(dx);
    if (pinf > 0.0) {
      double sc = 1.0 / pinf;
      for (int j = 0; j < n; ++j) dx[j] = sc * dx[j];
    }
    double dinf = inf_norm(dy);
    spmv(A, dx.data(), pprod.data());
    spmv(AT, dy.data(), dprod.data());
    pray_obj = dot(c, dx) / (cb * ob);
    vec dsl(n);
    for (int i = 0; i < m; ++i)
      pslack[i] = std::fmax(dy[i], 0.0) * lcf[i] + std::fmin(dy[i], 0.0) * ucf[i];
    for (int j = 0; j < n; ++j)
      dsl[j] = std::fmax(-dprod[j], 0.0) * lvf[j] + std::fmin(-dprod[j], 0.0) * uvf[j];
    double sp = vsum(pslack), sd = vsum(dsl);
    dray_obj = (sp + sd) / (cb * ob);
    for (int i = 0; i < m; ++i) {
      double v = pprod[i];
      pslack[i] = (std::fmax(0.0, -v) * (double)std::isfinite(lc[i]) +
                   std::fmax(0.0, v) * (double)std::isfinite(uc[i])) * Dr[i];
    }
    for (int j = 0; j < n; ++j) {
      double v = -dprod[j];
      dsl[j] = (std::fmax(0.0, v) * (double)!std::isfinite(lv[j]) -
                std::fmin(0.0, v) * (double)!std::isfinite(uv[j])) * Dc[j];
    }
    max_pray = inf_norm(pslack);
    double dsn = inf_norm(dsl);
    max_dray = dsn;
    double scale = std::fmax(dinf, dsn);
    if (scale > 0.0) {
      max_dray /= scale;
      dray_obj /= scale;
    } else {
      max_dray = 0.0;
      dray_obj = 0.0;
    }
  }

  void check_termination() {
    int r = oracle_termination_decision(&prm.termination_criteria, rel_p, rel_d, rel_gap,
                                        dray_obj, max_dray, pray_obj, max_pray, total, cum_time);
    if (r != TERMINATION_REASON_UNSPECIFIED) reason = (termination_reason_t)r;
  }

  bool should_restart() {
    return oracle_restart_decision(&prm.restart_params, prm.termination_evaluation_frequency,
                                   total, inner, fpe, init_fpe, &last_fpe) != 0;
  }

  // reference src/pdlp_core_op.cu:577-636
  void perform_restart() {
    const auto &rp = prm.restart_params;
    double pd = std::sqrt(det_sum(n, [&](long j) { double d = xhat[j] - x0[j]; return d * d; }));
    double dd = std::sqrt(det_sum(m, [&](long i) { double d = yhat[i] - y0[i]; return d * d; }));
    double ratio = rel_d / rel_p;
    if (pd > 1e-16 && dd > 1e-16 && pd < 1e12 && dd < 1e12 && ratio > 1e-8 && ratio < 1e8) {
      double err = std::log(dd) - std::log(pd) - std::log(omega);
      pw_err_sum *= rp.i_smooth;
      pw_err_sum += err;
      double derr = err - pw_last_err;
      omega *= std::exp(rp.k_p * err + rp.k_i * pw_err_sum + rp.k_d * derr);
      pw_last_err = err;
    } else {
      omega = best_omega;
      pw_err_sum = 0.0;
      pw_last_err = 0.0;
    }
    double g = std::fabs(std::log10(rel_d / rel_p));
    if (g < best_gap) {
      best_gap = g;
      best_omega = omega;
    }
    x0 = xhat; x = xhat; y0 = yhat; y = yhat;
    inner = 0;
    last_fpe = INFINITY;
  }

  // reference src/pdlp_core_op.cu:393-418, :495-526
  void primal_step(bool major) {
    spmv(AT, y.data(), dprod.data());
    double step = eta / omega;
#pragma omp parallel for schedule(static)
    for (int j = 0; j < n; ++j) {
      double t = x[j] - step * (c[j] - dprod[j]);
      if (major) {
        xhat[j] = std::fmax(lv[j], std::fmin(t, uv[j]));
        lam[j] = (xhat[j] - t) / step;
        xref[j] = 2.0 * xhat[j] - x[j];
      } else {
        double pr = std::fmax(lv[j], std::fmin(t, uv[j]));
        xref[j] = 2.0 * pr - x[j];
      }
    }
  }

  // reference src/pdlp_core_op.cu:420-443, :528-557
  void dual_step(bool major) {
    spmv(A, xref.data(), pprod.data());
    double step = eta * omega;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < m; ++i) {
      double t = y[i] / step - pprod[i];
      double pr = std::fmax(-uc[i], std::fmin(t, -lc[i]));
      if (major) {
        yhat[i] = (t - pr) * step;
        yref[i] = 2.0 * yhat[i] - y[i];
      } else {
        yref[i] = 2.0 * (t - pr) * step - y[i];
      }
    }
  }

  // reference src/pdlp_core_op.cu:658-696
  void fixed_point_error() {
#pragma omp parallel for schedule(static)
    for (int j = 0; j < n; ++j) dx[j] = xref[j] - x[j];
#pragma omp parallel for schedule(static)
    for (int i = 0; i < m; ++i) dy[i] = yref[i] - y[i];
    spmv(AT, dy.data(), dprod.data());
    double dn = nrm2(dy), pn = nrm2(dx);
    double movement = pn * pn * omega + dn * dn / omega;
    double cross = dot(dprod, dx);
    double interaction = 2 * eta * cross;
    fpe = std::sqrt(movement + interaction);
  }

  // reference src/pdlp_core_op.cu:445-462, :559-567
  void halpern() {
    double w = (double)(inner + 1) / (inner + 2);
    double rc = prm.reflection_coefficient;
#pragma omp parallel for schedule(static)
    for (int j = 0; j < n; ++j) {
      double r = rc * xref[j] + (1.0 - rc) * x[j];
      x[j] = w * r + (1.0 - w) * x0[j];
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < m; ++i) {
      double r = rc * yref[i] + (1.0 - rc) * y[i];
      y[i] = w * r + (1.0 - w) * y0[i];
    }
  }

  void record(double *tr, int cap, int *len) {
    if (!tr || !len || *len >= cap) return;
    double *r = tr + (long)(*len) * ORACLE_TR_WIDTH;
    r[ORACLE_TR_ITER] = total;
    r[ORACLE_TR_REL_PRIMAL] = rel_p;
    r[ORACLE_TR_REL_DUAL] = rel_d;
    r[ORACLE_TR_REL_GAP] = rel_gap;
    r[ORACLE_TR_PRIMAL_OBJ] = pobj;
    r[ORACLE_TR_DUAL_OBJ] = dobj;
    r[ORACLE_TR_PRIMAL_WEIGHT] = omega;
    r[ORACLE_TR_FIXED_POINT_ERROR] = fpe;
    r[ORACLE_TR_STEP_SIZE] = eta;
    r[ORACLE_TR_INNER_COUNT] = inner;
    ++*len;
  }

  bool do_restart = false;

  // reference src/solver.cu:54-109; stops early after `budget` iterations
  // (budget < 0: no budget) so a session can run bounded samples.
  void run(double *tr, int cap, int *len, long budget = -1) {
    int F = prm.termination_evaluation_frequency;
    auto t0 = std::chrono::steady_clock::now();
    long done_here = 0;
    while (total < prm.termination_criteria.iteration_limit) {
      if (budget >= 0 && done_here >= budget) return;
      ++done_here;
      if (is_major || total == 0 || total % print_frequency(total) == 0) {
        compute_residual();
        if (is_major && total < 3 * F) compute_infeasibility();
        cum_time = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        check_termination();
        record(tr, cap, len);
        if (reason != TERMINATION_REASON_UNSPECIFIED) break;
      }
      if (is_major || total == 0) {
        do_restart = should_restart();
        if (do_restart) perform_restart();
      }
      is_major = ((total + 1) % F) == 0;
      bool major_kernel = is_major || ((total + 2) % print_frequency(total + 2)) == 0;
      primal_step(major_kernel);
      dual_step(major_kernel);
      if (is_major || do_restart) {
        fixed_point_error();
        if (do_restart) {
          init_fpe = fpe;
          do_restart = false;
        }
      }
      halpern();
      ++inner;
      ++total;
    }
    if (reason == TERMINATION_REASON_UNSPECIFIED) {
      reason = TERMINATION_REASON_ITERATION_LIMIT;
      compute_residual();
      record(tr, cap, len);
    }
    cum_time = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }

  // ----------------------------------------------------- feasibility polishing
  // reference src/pdlp_core_op.cu:861-1360, src/utils.cu:1015-1040, :1110-1229
  int polish_mode = 0;  // 1: primal feasibility problem, 2: dual
  double feas_time = 0.0;
  int feas_iter = 0;

  // reference initialize_primal / initialize_dual_feas_polish_state
  void setup_polish(int mode, double w0) {
    polish_mode = mode;
    auto zero = [](vec &v) { std::fill(v.begin(), v.end(), 0.0); };
    auto zero_finite = [](vec &v) {
      for (double &a : v)
        if (std::isfinite(a)) a = 0.0;
    };
    if (mode == 1) {
      zero(c);
      c0 = 0.0;  // the reference's primal polish state drops the objective constant
      zero(y0); zero(y); zero(yhat); zero(yref); zero(dprod);
    } else {
      zero_finite(lc); zero_finite(uc); zero_finite(lv); zero_finite(uv);
      zero(lcf); zero(ucf); zero(lvf); zero(uvf);
      zero(x0); zero(x); zero(xhat); zero(xref); zero(pprod);
    }
    if (mode == 1) zero(lam);
    zero(pslack); zero(dres); zero(pres); zero(dx); zero(dy);
    pw_err_sum = 0.0;
    pw_last_err = 0.0;
    fpe = init_fpe = last_fpe = INFINITY;
    omega = best_omega = w0;
    is_major = false;
    total = inner = 0;
    reason = TERMINATION_REASON_UNSPECIFIED;
    cum_time = 0.0;
    best_gap = INFINITY;
    if (mode == 1) rel_d = abs_d = rel_gap = gap = 0.0;
    else rel_p = abs_p = rel_gap = gap = 0.0;
  }

  // reference compute_primal_feas_polish_residual / compute_dual_...
  void polish_residual(const Solver &ori) {
    if (polish_mode == 1) {
      spmv(A, xhat.data(), pprod.data());
#pragma omp parallel for schedule(static)
      for (int i = 0; i < m; ++i) {
        double cl = std::fmax(lc[i], std::fmin(pprod[i], uc[i]));
        pres[i] = (pprod[i] - cl) * Dr[i];
      }
      abs_p = norm(pres) / cb;
      rel_p = abs_p / (1.0 + bnorm);
      pobj = dot(ori.c, xhat) / (cb * ob) + c0;
    } else {
      spmv(AT, yhat.data(), dprod.data());
#pragma omp parallel for schedule(static)
      for (int j = 0; j < n; ++j) dres[j] = (c[j] - dprod[j] - lam[j]) * Dc[j];
#pragma omp parallel for schedule(static)
      for (int i = 0; i < m; ++i)
        pslack[i] = std::fmax(yhat[i], 0.0) * ori.lcf[i] + std::fmin(yhat[i], 0.0) * ori.ucf[i];
      abs_d = norm(dres) / ob;
      rel_d = abs_d / (1.0 + cnorm);
      double base = dot(lam, ori.xhat);
      dobj = (base + vsum(pslack)) / (cb * ob) + c0;
    }
  }

  // reference src/utils.cu:1015-1039
  void polish_termination() {
    const auto &tc = prm.termination_criteria;
    double r = polish_mode == 1 ? rel_p : rel_d;
    if (r <= tc.eps_feas_polish_relative) reason = TERMINATION_REASON_FEAS_POLISH_SUCCESS;
    else if (total >= tc.iteration_limit) reason = TERMINATION_REASON_ITERATION_LIMIT;
    else if (cum_time >= tc.time_sec_limit) reason = TERMINATION_REASON_TIME_LIMIT;
  }

  // reference primal_feasibility_polish / dual_feasibility_polish: the loop
  // of the solve with one-sided restarts and fixed-point error; like the
  // reference, the iteration in progress completes after termination
  void polish_loop(const Solver &ori) {
    int F = prm.termination_evaluation_frequency;
    auto t0 = std::chrono::steady_clock::now();
    bool restart = false;
    while (reason == TERMINATION_REASON_UNSPECIFIED) {
      if (is_major || total == 0 || total % print_frequency(total) == 0) {
        polish_residual(ori);
        cum_time = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        polish_termination();
      }
      if (is_major || total == 0) {
        restart = should_restart();
        if (restart) {  // reference perform_primal_restart / perform_dual_restart
          if (polish_mode == 1) x0 = x = xhat;
          else y0 = y = yhat;
          inner = 0;
          last_fpe = INFINITY;
        }
      }
      is_major = ((total + 1) % F) == 0;
      bool major_kernel = is_major || ((total + 2) % print_frequency(total + 2)) == 0;
      primal_step(major_kernel);
      dual_step(major_kernel);
      if (is_major || restart) {  // reference compute_primal/dual_fixed_point_error
        if (polish_mode == 1) {
#pragma omp parallel for schedule(static)
          for (int j = 0; j < n; ++j) dx[j] = xref[j] - x[j];
          double pn = nrm2(dx);
          fpe = pn * pn * omega;
        } else {
#pragma omp parallel for schedule(static)
          for (int i = 0; i < m; ++i) dy[i] = yref[i] - y[i];
          double dn = nrm2(dy);
          fpe = dn * dn / omega;
        }
        if (restart) {
          init_fpe = fpe;
          restart = false;
        }
      }
      halpern();
      ++inner;
      ++total;
    }
  }

  // reference feasibility_polish (src/pdlp_core_op.cu:862-930)
  void feasibility_polish() {
    auto t0 = std::chrono::steady_clock::now();
    const double eps = prm.termination_criteria.eps_feas_polish_relative;
    if (rel_p < eps && rel_d < eps) return;
    double w0 = prm.bound_objective_rescaling ? 1.0 : (cnorm + 1.0) / (bnorm + 1.0);
    Solver ps = *this;
    ps.setup_polish(1, w0);
    ps.polish_loop(*this);
    if (ps.reason == TERMINATION_REASON_FEAS_POLISH_SUCCESS) {
      xhat = ps.xhat;
      abs_p = ps.abs_p;
      rel_p = ps.rel_p;
      pobj = ps.pobj;
    }
    feas_iter += ps.total - 1;
    Solver ds = *this;
    ds.setup_polish(2, w0);
    ds.polish_loop(*this);
    if (ds.reason == TERMINATION_REASON_FEAS_POLISH_SUCCESS) {
      yhat = ds.yhat;
      abs_d = ds.abs_d;
      rel_d = ds.rel_d;
      dobj = ds.dobj;
    }
    feas_iter += ds.total - 1;
    gap = std::fabs(pobj - dobj);
    rel_gap = gap / (1.0 + std::fabs(pobj) + std::fabs(dobj));
    feas_time = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }

  // reference src/pdlp_core_op.cu:789-859
  cupdlpx_result_t *result(const lp_problem_t *p) {
    auto *r = (cupdlpx_result_t *)calloc(1, sizeof(cupdlpx_result_t));
    spmv(AT, yhat.data(), dprod.data());
    r->primal_solution = (double *)malloc(sizeof(double) * (n ? n : 1));
    r->dual_solution = (double *)malloc(sizeof(double) * (m ? m : 1));
    r->reduced_cost = (double *)malloc(sizeof(double) * (n ? n : 1));
    for (int j = 0; j < n; ++j) {
      r->reduced_cost[j] = (c[j] - dprod[j]) * Dc[j] / ob;
      r->primal_solution[j] = xhat[j] / Dc[j] / cb;
    }
    for (int i = 0; i < m; ++i) r->dual_solution[i] = yhat[i] / Dr[i] / ob;
    r->num_variables = p->num_variables;
    r->num_constraints = p->num_constraints;
    r->num_nonzeros = p->constraint_matrix_num_nonzeros;
    r->num_reduced_variables = p->num_variables;
    r->num_reduced_constraints = p->num_constraints;
    r->num_reduced_nonzeros = p->constraint_matrix_num_nonzeros;
    r->total_count = total;
    r->rescaling_time_sec = rescale_sec;
    r->cumulative_time_sec = cum_time;
    r->absolute_primal_residual = abs_p;
    r->relative_primal_residual = rel_p;
    r->absolute_dual_residual = abs_d;
    r->relative_dual_residual = rel_d;
    r->primal_objective_value = pobj;
    r->dual_objective_value = dobj;
    r->objective_gap = gap;
    r->relative_objective_gap = rel_gap;
    r->max_primal_ray_infeasibility = max_pray;
    r->max_dual_ray_infeasibility = max_dray;
    r->primal_ray_linear_objective = pray_obj;
    r->dual_ray_objective = dray_obj;
    r->termination_reason = reason;
    r->feasibility_polishing_time = feas_time;
    r->feasibility_iteration = feas_iter;
    return r;
  }
};

struct ThreadScope {
  int saved;
  explicit ThreadScope(int n) : saved(omp_get_max_threads()) {
    if (n > 0) omp_set_num_threads(n);
  }
  ~ThreadScope() { omp_set_num_threads(saved); }
};

Csr make_csr(int rows, int cols, const int *p, const int *j, const double *x) {
  Csr A;
  A.rows = rows;
  A.cols = cols;
  int nnz = p[rows];
  A.p.assign(p, p + rows + 1);
  A.j.assign(j, j + nnz);
  A.x.assign(x, x + nnz);
  return A;
}

}  // namespace

extern "C" {

void oracle_default_parameters(pdhg_parameters_t *p) {
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
  p->grid_size.decided = false;
  p->partition_method = NNZ_BALANCE_PARTITION;
  p->permute_method = BLOCK_RANDOM_PERMUTATION;
}

cupdlpx_result_t *oracle_solve(const lp_problem_t *prob,
                               const pdhg_parameters_t *params, int nthreads,
                               double *trace, int trace_cap, int *trace_len) {
  if (!prob) return nullptr;
  ThreadScope ts(nthreads);
  pdhg_parameters_t local;
  if (params) local = *params;
  else oracle_default_parameters(&local);
  if (trace_len) *trace_len = 0;
  Solver s(local);
  s.init(prob);
  s.init_step();
  s.run(trace, trace_cap, trace_len);
  // reference src/solver.cu:111-115
  if (local.feasibility_polishing && s.reason != TERMINATION_REASON_DUAL_INFEASIBLE &&
      s.reason != TERMINATION_REASON_PRIMAL_INFEASIBLE)
    s.feasibility_polish();
  return s.result(prob);
}

void oracle_result_free(cupdlpx_result_t *r) {
  if (!r) return;
  free(r->primal_solution);
  free(r->dual_solution);
  free(r->reduced_cost);
  free(r);
}

void oracle_rescale(const lp_problem_t *prob, const pdhg_parameters_t *params,
                    double *vals, double *c, double *lv, double *uv,
                    double *lc, double *uc, double *con_rescale,
                    double *var_rescale, double *cbr, double *obr) {
  Scaled s;
  rescale(prob, params, s);
  std::copy(s.A.x.begin(), s.A.x.end(), vals);
  std::copy(s.c.begin(), s.c.end(), c);
  std::copy(s.lv.begin(), s.lv.end(), lv);
  std::copy(s.uv.begin(), s.uv.end(), uv);
  std::copy(s.lc.begin(), s.lc.end(), lc);
  std::copy(s.uc.begin(), s.uc.end(), uc);
  std::copy(s.con.begin(), s.con.end(), con_rescale);
  std::copy(s.var.begin(), s.var.end(), var_rescale);
  *cbr = s.cb;
  *obr = s.ob;
}

void oracle_transpose(int m, int n, const int *ap, const int *aj,
                      const double *ax, int *tp, int *tj, double *tx) {
  Csr A = make_csr(m, n, ap, aj, ax), T;
  transpose(A, T);
  std::copy(T.p.begin(), T.p.end(), tp);
  std::copy(T.j.begin(), T.j.end(), tj);
  std::copy(T.x.begin(), T.x.end(), tx);
}

void oracle_spmv(int rows, const int *ap, const int *aj, const double *ax,
                 const double *x, double *y, int nthreads) {
  ThreadScope ts(nthreads);
#pragma omp parallel for schedule(dynamic, 512)
  for (int r = 0; r < rows; ++r) {
    double s = 0.0;
    for (int k = ap[r]; k < ap[r + 1]; ++k) s += ax[k] * x[aj[k]];
    y[r] = s;
  }
}

void oracle_power_start_vector(int m, double *v) {
  vec t;
  power_start(m, t);
  std::copy(t.begin(), t.end(), v);
}

double oracle_power_method(int m, int n, const int *ap, const int *aj,
                           const double *ax, const double *v0, int max_iter,
                           double tol, int *iters_out, int nthreads) {
  ThreadScope ts(nthreads);
  Csr A = make_csr(m, n, ap, aj, ax), T;
  transpose(A, T);
  vec v(v0, v0 + m);
  return power_method(A, T, v, max_iter, tol, iters_out);
}

int oracle_print_frequency(int iter) { return print_frequency(iter); }

// reference src/utils.cu:826-859
int oracle_dense_to_csr(const matrix_desc_t *d, int **rp, int **ci, double **v,
                        int *nnz_out) {
  int m = d->m, n = d->n;
  double tol = d->zero_tolerance > 0 ? d->zero_tolerance : 1e-12;
  const double *A = d->data.dense.A;
  int nnz = 0;
  for (long i = 0; i < (long)m * n; ++i)
    if (std::fabs(A[i]) > tol) ++nnz;
  *rp = (int *)malloc(sizeof(int) * (m + 1));
  *ci = (int *)malloc(sizeof(int) * (nnz ? nnz : 1));
  *v = (double *)malloc(sizeof(double) * (nnz ? nnz : 1));
  int k = 0;
  for (int i = 0; i < m; ++i) {
    (*rp)[i] = k;
    for (int j = 0; j < n; ++j) {
      double a = A[(long)i * n + j];
      if (std::fabs(a) > tol) {
        (*ci)[k] = j;
        (*v)[k] = a;
        ++k;
      }
    }
  }
  (*rp)[m] = k;
  *nnz_out = k;
  return 0;
}

// reference src/utils.cu:862-922
int oracle_csc_to_csr(const matrix_desc_t *d, int **rp, int **ci, double **v,
                      int *nnz_out) {
  int m = d->m, n = d->n;
  const int *cp = d->data.csc.col_ptr, *ri = d->data.csc.row_ind;
  const double *x = d->data.csc.vals;
  double tol = d->zero_tolerance > 0 ? d->zero_tolerance : 0.0;
  std::vector<int> cnt(m + 1, 0);
  int nnz = 0;
  for (int j = 0; j < n; ++j)
    for (int k = cp[j]; k < cp[j + 1]; ++k) {
      if (ri[k] < 0 || ri[k] >= m) return -1;
      if (tol > 0 && std::fabs(x[k]) <= tol) continue;
      cnt[ri[k] + 1]++;
      ++nnz;
    }
  for (int i = 0; i < m; ++i) cnt[i + 1] += cnt[i];
  *rp = (int *)malloc(sizeof(int) * (m + 1));
  *ci = (int *)malloc(sizeof(int) * (nnz ? nnz : 1));
  *v = (double *)malloc(sizeof(double) * (nnz ? nnz : 1));
  std::copy(cnt.begin(), cnt.end(), *rp);
  std::vector<int> next(cnt.begin(), cnt.end() - 1);
  for (int j = 0; j < n; ++j)
    for (int k = cp[j]; k < cp[j + 1]; ++k) {
      if (tol > 0 && std::fabs(x[k]) <= tol) continue;
      int pos = next[ri[k]]++;
      (*ci)[pos] = j;
      (*v)[pos] = x[k];
    }
  *nnz_out = nnz;
  return 0;
}

// reference src/utils.cu:925-1013
int oracle_coo_to_csr(const matrix_desc_t *d, int **rp, int **ci, double **v,
                      int *nnz_out) {
  int m = d->m, n = d->n, nin = d->data.coo.nnz;
  const int *r = d->data.coo.row_ind, *cc = d->data.coo.col_ind;
  const double *x = d->data.coo.vals;
  double tol = d->zero_tolerance > 0 ? d->zero_tolerance : 0.0;
  std::vector<int> cnt(m + 1, 0);
  int nnz = 0;
  for (int k = 0; k < nin; ++k) {
    if (tol > 0 && std::fabs(x[k]) <= tol) continue;
    if (r[k] < 0 || r[k] >= m) return -1;
    if (cc[k] < 0 || cc[k] >= n) return -1;
    cnt[r[k] + 1]++;
    ++nnz;
  }
  for (int i = 0; i < m; ++i) cnt[i + 1] += cnt[i];
  *rp = (int *)malloc(sizeof(int) * (m + 1));
  *ci = (int *)malloc(sizeof(int) * (nnz ? nnz : 1));
  *v = (double *)malloc(sizeof(double) * (nnz ? nnz : 1));
  std::copy(cnt.begin(), cnt.end(), *rp);
  std::vector<int> next(cnt.begin(), cnt.end() - 1);
  for (int k = 0; k < nin; ++k) {
    if (tol > 0 && std::fabs(x[k]) <= tol) continue;
    int pos = next[r[k]]++;
    (*ci)[pos] = cc[k];
    (*v)[pos] = x[k];
  }
  *nnz_out = nnz;
  return 0;
}

struct oracle_session {
  pdhg_parameters_t prm;
  Solver *s;
  int nthreads;
};

oracle_session_t *oracle_session_create(const lp_problem_t *prob,
                                        const pdhg_parameters_t *params, int nthreads,
                                        double *setup_sec) {
  auto *ss = new oracle_session;
  if (params) ss->prm = *params;
  else oracle_default_parameters(&ss->prm);
  ss->nthreads = nthreads;
  ThreadScope ts(nthreads);
  auto t0 = std::chrono::steady_clock::now();
  ss->s = new Solver(ss->prm);
  ss->s->init(prob);
  if (setup_sec)
    *setup_sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  // step size from a short power run so the loop can proceed
  ss->s->eta = 1.0;
  ss->s->omega = 1.0;
  ss->s->best_omega = 1.0;
  return ss;
}

double oracle_session_power(oracle_session_t *ss, int iters) {
  ThreadScope ts(ss->nthreads);
  Solver &s = *ss->s;
  vec v0;
  power_start(s.m, v0);
  auto t0 = std::chrono::steady_clock::now();
  double smax = power_method(s.A, s.AT, v0, iters, 0.0, nullptr);
  double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (smax > 0) s.eta = 0.998 / smax;
  return sec;
}

double oracle_session_iterate(oracle_session_t *ss, int iters) {
  ThreadScope ts(ss->nthreads);
  auto t0 = std::chrono::steady_clock::now();
  ss->s->run(nullptr, 0, nullptr, iters);
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

void oracle_session_free(oracle_session_t *ss) {
  if (!ss) return;
  delete ss->s;
  delete ss;
}

void oracle_problem_free(lp_problem_t *p) {
  if (!p) return;
  free(p->constraint_matrix_row_pointers);
  free(p->constraint_matrix_col_indices);
  free(p->constraint_matrix_values);
  free(p->objective_vector);
  free(p->variable_lower_bound);
  free(p->variable_upper_bound);
  free(p->constraint_lower_bound);
  free(p->constraint_upper_bound);
  free(p->primal_start);
  free(p->dual_start);
  free(p);
}

}  // extern "C"
