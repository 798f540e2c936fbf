// refine.cu -- FP32 PDHG with FP64 iterative refinement.
//
// Round 0 solves the LP with FP32 iterates (FP32 SpMVs and updates, FP64
// reductions).  If the FP64 KKT of the result, evaluated on the original
// problem, misses the tolerance, each further round re-centres the problem
// at the FP64 point (xbar, ybar) and solves the correction LP
//     min (c - A^T ybar)' z
//     s.t. lc - A xbar <= A z <= uc - A xbar,  lv - xbar <= z <= uv - xbar
// in FP32, then accumulates xbar += z, ybar += w (w the correction dual) and
// takes the correction's dual slack as the new one; the correction's KKT
// residuals are exactly the original residuals of (xbar + z, ybar + w), so
// its termination test uses the original's bound / objective norms.  FP32
// only has to represent the correction, which shrinks round after round.
// Residuals, corrections and the final KKT are FP64 throughout.
//
// Tolerances below 1e-4: round 0 stops at a relaxed tolerance (30 x eps,
// within [1e-5, 1e-4]) and an FP64 PDHG solve warm-started at the FP64 point
// with a cold primal weight (the FP64 finish) completes the solve; the
// correction rounds then serve the cases where round 0 stalls above it.
// Every path ends with the FP64 finish when the rounds miss the tolerance.
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <chrono>

#include "iter_kernels.cuh"

namespace pdlp {

// over A: s = (A xbar)_i -> shifted constraint bounds
struct CorrAEpi {
  using val_t = double;
  using acc_t = double;
  static constexpr int NF = 0;
  static constexpr unsigned MAXMASK = 0;
  const double *xbar, *lc, *uc;
  double *lc2, *uc2;
  double dp;
  PDLP_NO_BLOCK_SCALARS
  __device__ bool init() { return true; }
  __device__ double gather(int j) const { return xbar[j]; }
  __device__ void row(int i, double s, double *) const {
    lc2[i] = dp * (lc[i] - s);
    uc2[i] = dp * (uc[i] - s);
  }
};

// over A^T: s = (A^T ybar)_j -> reduced-cost objective, shifted variable bounds
struct CorrATEpi {
  using val_t = double;
  using acc_t = double;
  static constexpr int NF = 0;
  static constexpr unsigned MAXMASK = 0;
  const double *ybar, *c, *lv, *uv, *xbar;
  double *c2, *lv2, *uv2;
  double dp, dd;
  PDLP_NO_BLOCK_SCALARS
  __device__ bool init() { return true; }
  __device__ double gather(int i) const { return ybar[i]; }
  __device__ void row(int j, double s, double *) const {
    c2[j] = dd * (c[j] - s);
    double xb = xbar[j];
    lv2[j] = dp * (lv[j] - xb);
    uv2[j] = dp * (uv[j] - xb);
  }
};

// reduced cost rc = c - A^T y of the FP64 point, and the dual slack taken as
// its projection onto the cone the bounds allow: rc_j where both bounds are
// finite, max(rc_j, 0) with only a lower bound, min(rc_j, 0) with only an
// upper bound, 0 for a free variable.  This is the limit of the iteration's
// (x_hat - t) / tau and, unlike a dual slack carried over from an FP32
// round, has FP64 accuracy.
struct RcEpi {
  using val_t = double;
  using acc_t = double;
  static constexpr int NF = 0;
  static constexpr unsigned MAXMASK = 0;
  const double *y, *c, *lv, *uv;
  double *rc, *lam;
  PDLP_NO_BLOCK_SCALARS
  __device__ bool init() { return true; }
  __device__ double gather(int i) const { return y[i]; }
  __device__ void row(int j, double s, double *) const {
    double r = c[j] - s;
    rc[j] = r;
    bool lo = isfinite(lv[j]), up = isfinite(uv[j]);
    lam[j] = lo && up ? r : lo ? fmax(r, 0.0) : up ? fmin(r, 0.0) : 0.0;
  }
};

__global__ void k_finite(int m, const double *lc, const double *uc, double *lcf, double *ucf) {
  long stride = (long)gridDim.x * blockDim.x;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < m; i += stride) {
    lcf[i] = isfinite(lc[i]) ? lc[i] : 0.0;
    ucf[i] = isfinite(uc[i]) ? uc[i] : 0.0;
  }
}

// xbar += z, ybar += w, keeping the previous point for a rollback
__global__ void k_accumulate(int n, int m, double *xbar, double *ybar, double *xold,
                             double *yold, const double *z, const double *w, double dpi,
                             double ddi) {
  long stride = (long)gridDim.x * blockDim.x;
  for (long j = blockIdx.x * (long)blockDim.x + threadIdx.x; j < n; j += stride) {
    xold[j] = xbar[j];
    xbar[j] += z[j] * dpi;
  }
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < m; i += stride) {
    yold[i] = ybar[i];
    ybar[i] += w[i] * ddi;
  }
}

__global__ void k_rollback(int n, int m, double *xbar, double *ybar, const double *xold,
                           const double *yold) {
  long stride = (long)gridDim.x * blockDim.x;
  for (long j = blockIdx.x * (long)blockDim.x + threadIdx.x; j < n; j += stride) xbar[j] = xold[j];
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < m; i += stride) ybar[i] = yold[i];
}

namespace {
size_t a256(size_t b) { return (b + 255) & ~(size_t)255; }
}  // namespace

cupdlpx_result_t *solve_refined(const DevProblem &P, const pdhg_parameters_t &params,
                                const RefineOptions &opt, cudaStream_t st,
                                RefineReport *report) {
  auto t0 = std::chrono::steady_clock::now();
  const int n = P.n, m = P.m, nnz = P.nnz;
  const double eps_feas = params.termination_criteria.eps_feasible_relative;
  const double eps_opt = params.termination_criteria.eps_optimal_relative;
  const bool linf = params.optimality_norm == NORM_TYPE_L_INF;

  // device workspace: FP64 point, correction, correction problem vectors,
  // SpMV scratch for the original matrices
  size_t bytes = 0;
  const size_t vn = n, vm = m;
  auto need = [&](size_t b) { bytes += a256(b + 1); };
  for (int i = 0; i < 9; ++i) need(vn * 8);  // xbar lam z lz c2 lv2 uv2 rc xold
  for (int i = 0; i < 7; ++i) need(vm * 8);  // ybar w lc2 uc2 lcf ucf yold
  for (const DevCsr *W : {&P.A, &P.AT}) {
    need((size_t)W->plan.nlong * 4); need((size_t)W->plan.nblk * 8);
    need((size_t)W->pipe.nlong * 4); need((size_t)W->pipe.ntile * 8); need(4);
  }
  char *mem = (char *)dev_alloc(bytes, st);
  struct Free {
    char *p;
    cudaStream_t s;
    ~Free() { dev_free(p, s); }
  } guard{mem, st};
  size_t off = 0;
  auto take = [&](size_t b) {
    char *p = mem + off;
    off += a256(b + 1);
    return p;
  };
  double *xbar = (double *)take(vn * 8), *lam = (double *)take(vn * 8);
  double *z = (double *)take(vn * 8), *lz = (double *)take(vn * 8);
  double *c2 = (double *)take(vn * 8), *lv2 = (double *)take(vn * 8);
  double *uv2 = (double *)take(vn * 8), *rc = (double *)take(vn * 8);
  double *xold = (double *)take(vn * 8), *yold = (double *)take(vm * 8);
  double *ybar = (double *)take(vm * 8), *w = (double *)take(vm * 8);
  double *lc2 = (double *)take(vm * 8), *uc2 = (double *)take(vm * 8);
  double *olcf = (double *)take(vm * 8), *oucf = (double *)take(vm * 8);
  if (m) k_finite<<<grid_for(m), kThreads, 0, st>>>(m, P.lc, P.uc, olcf, oucf);
  DevCsr A = P.A, AT = P.AT;
  A.plan.lcnt = (unsigned *)take((size_t)P.A.plan.nlong * 4);
  A.plan.lsum = (double *)take((size_t)P.A.plan.nblk * 8);
  AT.plan.lcnt = (unsigned *)take((size_t)P.AT.plan.nlong * 4);
  AT.plan.lsum = (double *)take((size_t)P.AT.plan.nblk * 8);
  if (P.A.plan.nlong) PDLP_CUDA(cudaMemsetAsync(A.plan.lcnt, 0, (size_t)P.A.plan.nlong * 4, st));
  if (P.AT.plan.nlong) PDLP_CUDA(cudaMemsetAsync(AT.plan.lcnt, 0, (size_t)P.AT.plan.nlong * 4, st));
  for (DevCsr *W : {&A, &AT}) {  // the pipelined kernel's scratch
    W->pipe.lcnt = (unsigned *)take((size_t)W->pipe.nlong * 4);
    W->pipe.lsum = (double *)take((size_t)W->pipe.ntile * 8);
    W->pipe.err = (int *)take(4);
    if (W->pipe.nlong)
      PDLP_CUDA(cudaMemsetAsync(W->pipe.lcnt, 0, (size_t)W->pipe.nlong * 4, st));
    PDLP_CUDA(cudaMemsetAsync(W->pipe.err, 0, sizeof(int), st));
  }
  if (n) {
    PDLP_CUDA(cudaMemsetAsync(xbar, 0, vn * 8, st));
    PDLP_CUDA(cudaMemsetAsync(lam, 0, vn * 8, st));
  }
  if (m) PDLP_CUDA(cudaMemsetAsync(ybar, 0, vm * 8, st));

  // FP64 evaluator of the original problem (KKT is scaling invariant, so no
  // rescaling is needed)
  pdhg_parameters_t pe = params;
  pe.l_inf_ruiz_iterations = 0;
  pe.has_pock_chambolle_alpha = false;
  pe.bound_objective_rescaling = false;
  Solve<double> ev(pe, st, P, 0);
  ev.prepare();

  // the correction problem: a view of P's matrices with its own vectors
  DevProblem Q;
  Q.m = m;
  Q.n = n;
  Q.nnz = nnz;
  Q.tile = P.tile;
  Q.A = P.A;
  Q.AT = P.AT;
  Q.shape_key = P.shape_key;  // same structure: the rounds run round 0's kernels
  Q.c = c2;
  Q.lv = lv2;
  Q.uv = uv2;
  Q.lc = lc2;
  Q.uc = uc2;
  // original norms: the correction's relative residuals equal the original's
  Q.cnorm_l2 = P.cnorm_l2;
  Q.cnorm_linf = P.cnorm_linf;
  Q.bnorm_l2 = P.bnorm_l2;
  Q.bnorm_linf = P.bnorm_linf;
  Q.c0 = 0.0;
  Q.shift_x = xbar;
  Q.shift_y = ybar;
  Q.orig_c = P.c;
  Q.orig_lcf = olcf;
  Q.orig_ucf = oucf;
  Q.orig_c0 = P.c0;

  // stall rule of the FP32 rounds: once a round's relative KKT error is
  // below 2e-5 -- about where FP32 iterates (unit roundoff 6e-8) meet the
  // cancellation of long rows -- the round ends when the error has not
  // improved by 10% within max(10000, t / 2) iterations.  Above that level a
  // plateau is the method's own (the 20M-nnz power-law LP, FP64 or FP32,
  // spends 10,000+ iterations near 2e-4; FP32 alone reaches 1e-4 there in
  // 57,000 iterations) and stopping there would hand an unconverged point to
  // refinement.  PDLP_STALL_MIN / _FRAC / _FLOOR override the three numbers.
  int stall_min = 10000;
  double stall_frac = 0.5, stall_floor = 2e-5;
  if (const char *e = getenv("PDLP_STALL_MIN")) stall_min = atoi(e);
  if (const char *e = getenv("PDLP_STALL_FRAC")) stall_frac = atof(e);
  if (const char *e = getenv("PDLP_STALL_FLOOR")) stall_floor = atof(e);
  RefineReport rep;
  double sigma = 0.0;
  int reason = TERMINATION_REASON_UNSPECIFIED;
  long iters = 0, launches = 0;
  (void)reason;
  int limit = params.termination_criteria.iteration_limit;
  Kkt kkt{};
  double best_err = INFINITY;
  double omega0 = 1.0, cb0 = 1.0, ob0 = 1.0, dp = 1.0, dd = 1.0;
  reason = TERMINATION_REASON_ITERATION_LIMIT;  // unless a round meets the tolerances
  cupdlpx_result_t *ray_result = nullptr;
  double rescale_sec = 0.0;
  // Round 0's tolerance.  Below 1e-4, FP32 runs only the first part of the
  // way: to 30 x eps (at least 1e-5, at most 1e-4), where FP32 iterates are
  // still reliable, and the FP64 finish below takes the point the rest of
  // the way.  Measured on the 20M-nnz transport LP at eps 1e-6 (GB300): FP32
  // to 3e-5 (28,600 iterations) then 9,300 FP64 iterations, 9.3 s, against
  // 29.4 s for FP64 alone (100,600 iterations); FP32 alone stalls near 5e-6
  // (197,000 iterations), and correction rounds from the 1e-5 point cost
  // more than they gained.
  const double eps_min = fmin(eps_feas, eps_opt);
  const double eps0 = eps_min < 1e-4 ? fmin(1e-4, fmax(30.0 * eps_min, 1e-5)) : 0.0;
  for (int round = 0; round < opt.max_rounds; ++round) {
    const DevProblem &R = round == 0 ? P : Q;
    bool stop = false;
    if (round > 0) {
      // unit-size correction: scale by the inverse of the current relative
      // residuals (primal / dual+gap), never below 1
      dp = 1.0 / fmax(fmax(kkt.rel_p, kkt.rel_gap), 0.1 * eps_feas);
      dd = 1.0 / fmax(fmax(kkt.rel_d, kkt.rel_gap), 0.1 * eps_feas);
      dp = fmax(dp, 1.0);
      dd = fmax(dd, 1.0);
      Q.delta_p = dp;
      Q.delta_d = dd;
      Q.cnorm_l2 = dd * (1.0 + P.cnorm_l2) - 1.0;
      Q.cnorm_linf = dd * (1.0 + P.cnorm_linf) - 1.0;
      Q.bnorm_l2 = dp * (1.0 + P.bnorm_l2) - 1.0;
      Q.bnorm_linf = dp * (1.0 + P.bnorm_linf) - 1.0;
      launch_spmv(A, CorrAEpi{xbar, P.lc, P.uc, lc2, uc2, dp}, nullptr, nullptr, st);
      launch_spmv(AT, CorrATEpi{ybar, P.c, P.lv, P.uv, xbar, c2, lv2, uv2, dp, dd}, nullptr,
                  nullptr, st);
      launches += 2;
    }
    pdhg_parameters_t pi = params;
    if (round == 0 && eps0 > 0.0) {
      pi.termination_criteria.eps_feasible_relative = fmax(eps_feas, eps0);
      pi.termination_criteria.eps_optimal_relative = fmax(eps_opt, eps0);
    }
    // the FP32 rounds leave 3 evaluation periods of the iteration limit to
    // the FP64 finish: its infeasibility window (the first 3 periods, as in
    // the reference's loop, src/solver.cu:62-65) certifies rays at
    // eps_infeasible, which FP32 iterates cannot resolve
    const long reserve = std::min<long>(3L * std::max(1, params.termination_evaluation_frequency),
                                        limit / 2);
    pi.termination_criteria.iteration_limit = (int)std::max<long>(0, limit - iters - reserve);
    double elapsed = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    pi.termination_criteria.time_sec_limit = params.termination_criteria.time_sec_limit - elapsed;
    if (round > 0) {
      // a margin below the target, so a round never stops at its first
      // evaluation on a point the FP64 check just rejected
      double e = opt.inner_eps > 0.0 ? opt.inner_eps : 0.5;
      pi.termination_criteria.eps_feasible_relative = opt.inner_eps > 0.0 ? e : e * eps_feas;
      pi.termination_criteria.eps_optimal_relative = opt.inner_eps > 0.0 ? e : e * eps_opt;
    }
    // one round with either FP32 iterates or FP64 iterates over an FP32 matrix;
    // returns true when the refinement should stop
    auto round_body = [&](auto &s) -> bool {
      // corrections keep the first round's bound / objective scaling, so the
      // scaled correction looks like the scaled original near its optimum
      if (round > 0) s.set_fixed_scaling(cb0, ob0);
      s.prepare();
      if (round == 0) rescale_sec = s.rescale_seconds();
      // the primal weight balances the scaled dual and primal distances, which
      // the correction multiplies by dd and dp
      double omega = round == 0 ? 0.0 : omega0 * dd / dp;
      s.init_step(sigma, omega);
      if (round == 0) {
        sigma = s.sigma_max();
        rep.power_iterations = s.power_iterations();
        rep.sigma_max = sigma;
      }
      s.set_stall_rule(stall_min, stall_frac, stall_floor);  // a floor ends a round, never a hang
      s.enable_snapshot();
      s.run();
      if (round == 0) {
        rep.kernel_A = s.pipe_A() ? 1 : 0;
        rep.kernel_AT = s.pipe_AT() ? 1 : 0;
        for (int q = 0; q < 4; ++q) rep.tune_ms[q] = s.tune_ms(q);
        omega0 = s.primal_weight();
        cb0 = s.cb();
        ob0 = s.ob();
      }
      int r = s.reason();
      iters += s.total_count();
      launches += s.kernel_launches();
      rep.rounds = round + 1;
      rep.timed_primal_ms_sum += s.live_primal_ms() * s.live_samples();
      rep.timed_dual_ms_sum += s.live_dual_ms() * s.live_samples();
      rep.timed_chunks += s.live_samples();
      if (r == TERMINATION_REASON_PRIMAL_INFEASIBLE || r == TERMINATION_REASON_DUAL_INFEASIBLE) {
        // infeasibility certificates come from the first round's rays
        ray_result = s.result();
        reason = r;
        return true;
      }
      s.result_device(z, w, lz);
      k_accumulate<<<grid_for((long)n + m), kThreads, 0, st>>>(n, m, xbar, ybar, xold, yold, z,
                                                               w, 1.0 / dp, 1.0 / dd);
      PDLP_LAUNCH_CHECK();
      launch_spmv(AT, RcEpi{ybar, P.c, P.lv, P.uv, rc, lam}, nullptr, nullptr, st);
      launches += 2;
      Kkt k = ev.evaluate(xbar, ybar, lam);
      launches += 4;
      double err = fmax(k.rel_p / eps_feas, fmax(k.rel_d / eps_feas, k.rel_gap / eps_opt));
      if (params.verbose)
        printf("refinement round %d: dp %.3g dd %.3g, %d iterations (reason %d, primal "
               "weight %.3g) -> FP64 rel primal %.3e rel dual %.3e rel gap %.3e\n",
               round, dp, dd, s.total_count(), r, s.primal_weight(), k.rel_p, k.rel_d,
               k.rel_gap);
      if (round > 0 && err >= best_err) {
        // the round did not improve the FP64 point: keep the previous one
        k_rollback<<<grid_for((long)n + m), kThreads, 0, st>>>(n, m, xbar, ybar, xold, yold);
        launch_spmv(AT, RcEpi{ybar, P.c, P.lv, P.uv, rc, lam}, nullptr, nullptr, st);
        PDLP_LAUNCH_CHECK();
        launches += 2;
        return true;
      }
      // a correction that gains less than 10x has met the FP32 floor of its
      // own solve: keep its point, but hand over to the FP64 finish
      const bool weak = round > 0 && err > 0.1 * best_err;
      best_err = err;
      kkt = k;
      if (err < 1.0) {
        reason = TERMINATION_REASON_OPTIMAL;
        return true;
      }
      if (r == TERMINATION_REASON_ITERATION_LIMIT || r == TERMINATION_REASON_TIME_LIMIT ||
          iters >= limit) {
        reason = r == TERMINATION_REASON_TIME_LIMIT ? r : TERMINATION_REASON_ITERATION_LIMIT;
        return true;
      }
      // round 0 met its relaxed tolerance: the FP64 finish takes it from here
      if (round == 0 && eps0 > 0.0 && r == TERMINATION_REASON_OPTIMAL) return true;
      return weak;
    };
    if (opt.fp64_iterates) {
      Solve<double, float> s(pi, st, R, 0);
      stop = round_body(s);
    } else {
      Solve<float, float> s(pi, st, R, 0);
      stop = round_body(s);
    }
    if (stop) break;
  }
  (void)linf;
  // FP64 finish: when a correction round could not improve the point, or the
  // rounds ran out, FP64 PDHG (the reference's arithmetic) continues from the
  // best FP64 point with round 0's step size and primal weight, so the
  // requested tolerance stays reachable whatever floor FP32 met.
  const double left_sec = params.termination_criteria.time_sec_limit -
                          std::chrono::duration<double>(std::chrono::steady_clock::now() - t0)
                              .count();
  if (!ray_result && reason != TERMINATION_REASON_OPTIMAL &&
      reason != TERMINATION_REASON_TIME_LIMIT && iters < limit && left_sec > 0.0) {
    DevProblem W;  // a view of P warm-started at the FP64 point
    W.m = m;
    W.n = n;
    W.nnz = nnz;
    W.tile = P.tile;
    W.A = P.A;
    W.AT = P.AT;
    W.shape_key = P.shape_key;
    W.c = P.c;
    W.lv = P.lv;
    W.uv = P.uv;
    W.lc = P.lc;
    W.uc = P.uc;
    W.cnorm_l2 = P.cnorm_l2;
    W.cnorm_linf = P.cnorm_linf;
    W.bnorm_l2 = P.bnorm_l2;
    W.bnorm_linf = P.bnorm_linf;
    W.c0 = P.c0;
    W.xs = xbar;
    W.ys = ybar;
    pdhg_parameters_t pf = params;
    pf.termination_criteria.iteration_limit = (int)(limit - iters);
    pf.termination_criteria.time_sec_limit = left_sec;
    Solve<double> s(pf, st, W, 0);
    s.prepare();
    // a cold primal weight: the FP32 rounds' weight has drifted under FP32
    // noise in the distances it balances (the 20M transport LP at 1e-6: from
    // a point at 2.3e-6, 220,200 FP64 iterations with round 0's weight
    // 1.5e-6, 4,200 with the cold one)
    s.init_step(sigma, 0.0);
    s.run();
    iters += s.total_count();
    launches += s.kernel_launches();
    const int r = s.reason();
    s.result_device(xbar, ybar, lz);
    launch_spmv(AT, RcEpi{ybar, P.c, P.lv, P.uv, rc, lam}, nullptr, nullptr, st);
    launches += 1;
    Kkt k = ev.evaluate(xbar, ybar, lam);
    double err = fmax(k.rel_p / eps_feas, fmax(k.rel_d / eps_feas, k.rel_gap / eps_opt));
    if (err >= 1.0) {
      // the solve's own dual slack, when the projected reduced cost is worse
      Kkt k2 = ev.evaluate(xbar, ybar, lz);
      double err2 = fmax(k2.rel_p / eps_feas, fmax(k2.rel_d / eps_feas, k2.rel_gap / eps_opt));
      if (err2 < err) {
        k = k2;
        err = err2;
        PDLP_CUDA(cudaMemcpyAsync(lam, lz, vn * 8, cudaMemcpyDeviceToDevice, st));
      }
    }
    launches += 8;
    kkt = k;
    rep.rounds += 1;
    rep.fp64_finish = true;
    reason = err < 1.0 || r == TERMINATION_REASON_OPTIMAL ? TERMINATION_REASON_OPTIMAL : r;
    if (params.verbose)
      printf("FP64 finish: %d iterations (reason %d) -> FP64 rel primal %.3e rel dual %.3e "
             "rel gap %.3e\n", s.total_count(), r, k.rel_p, k.rel_d, k.rel_gap);
  }
  double seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  rep.inner_iterations = iters;
  rep.kernel_launches = launches;
  rep.seconds = seconds;
  rep.kkt = kkt;
  if (report) *report = rep;
  if (ray_result) {
    ray_result->total_count = (int)iters;
    ray_result->cumulative_time_sec = seconds;
    return ray_result;
  }

  auto *res = (cupdlpx_result_t *)calloc(1, sizeof(cupdlpx_result_t));
  if (!res) throw std::bad_alloc();
  res->primal_solution = (double *)malloc(sizeof(double) * (n ? n : 1));
  res->dual_solution = (double *)malloc(sizeof(double) * (m ? m : 1));
  res->reduced_cost = (double *)malloc(sizeof(double) * (n ? n : 1));
  if (!res->primal_solution || !res->dual_solution || !res->reduced_cost) {
    free(res->primal_solution);
    free(res->dual_solution);
    free(res->reduced_cost);
    free(res);
    throw std::bad_alloc();
  }
  if (n) {
    PDLP_CUDA(cudaMemcpyAsync(res->primal_solution, xbar, vn * 8, cudaMemcpyDeviceToHost, st));
    PDLP_CUDA(cudaMemcpyAsync(res->reduced_cost, rc, vn * 8, cudaMemcpyDeviceToHost, st));
  }
  if (m) PDLP_CUDA(cudaMemcpyAsync(res->dual_solution, ybar, vm * 8, cudaMemcpyDeviceToHost, st));
  PDLP_CUDA(cudaStreamSynchronize(st));
  res->num_variables = n;
  res->num_constraints = m;
  res->num_nonzeros = nnz;
  res->num_reduced_variables = n;
  res->num_reduced_constraints = m;
  res->num_reduced_nonzeros = nnz;
  res->total_count = (int)iters;
  res->rescaling_time_sec = rescale_sec;
  res->cumulative_time_sec = seconds;
  res->absolute_primal_residual = kkt.abs_p;
  res->relative_primal_residual = kkt.rel_p;
  res->absolute_dual_residual = kkt.abs_d;
  res->relative_dual_residual = kkt.rel_d;
  res->primal_objective_value = kkt.pobj;
  res->dual_objective_value = kkt.dobj;
  res->objective_gap = kkt.gap;
  res->relative_objective_gap = kkt.rel_gap;
  res->termination_reason = (termination_reason_t)reason;
  return res;
}

}  // namespace pdlp
