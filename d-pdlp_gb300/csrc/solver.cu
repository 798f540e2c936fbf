// solver.cu -- restarted Halpern PDHG on one GPU, FP64.
//
// Per iteration two kernels run (reference src/solver.cu:85-102):
//   primal : g = A^T y (fused SpMV) -> x_hat = proj(x - tau (c - g)),
//            x_ref = 2 x_hat - x, Halpern x_next = w x_ref + (1-w) x0
//            (reference pdlp_core_op.cu:393-418, :445-462, :495-526)
//   dual   : h = A x_ref (fused SpMV) -> y_hat = sigma (t - proj(t)),
//            t = y/sigma - h, y_ref = 2 y_hat - y, Halpern y_next
//            (reference pdlp_core_op.cu:420-443, :528-557)
// The Halpern update of the reference is a separate pass after both steps;
// it only reads z_ref, z and z0 element-wise, so it is folded into the two
// epilogues, with z ping-ponged between two buffers.
//
// Evaluations, restarts, the fixed-point error and the termination test run
// on the device at the iterations the reference schedules them
// (reference src/solver.cu:58-103), so no iteration waits on the host.
#include <math.h>
#include <string.h>

#include <chrono>
#include <random>

#include "solver.cuh"

namespace pdlp {

// ======================================================= SpMV epilogues
// Epilogues without per-block scalars.
#define PDLP_NO_BLOCK_SCALARS                        \
  __device__ void prologue(double *) const {}        \
  __device__ void bind(const double *) {}

// Halpern weight w = (k+1)/(k+2), k = inner iteration count
// (reference pdlp_core_op.cu:559-567), formed once per block.
__device__ __forceinline__ void halpern_weight(const Ctl *c, int off, double *sc) {
  int k = c->t_base + off - c->restart_t;
  double w = (double)(k + 1) / (double)(k + 2);
  sc[0] = w;
  sc[1] = 1.0 - w;
}

template <bool MAJOR, bool FPE>
struct PrimalEpi {
  using val_t = double;
  using acc_t = double;
  static constexpr int NF = FPE ? 1 : 0;
  static constexpr unsigned MAXMASK = 0;
  Dev d;
  int off;
  const double *xcur, *ycur;
  double *xnext;
  double tau, w, omw;
  __device__ bool init() {
    const Ctl *c = d.ctl;
    if (c->done) return false;
    tau = c->tau;
    return true;
  }
  __device__ void prologue(double *sc) const { halpern_weight(d.ctl, off, sc); }
  __device__ void bind(const double *sc) {
    w = sc[0];
    omw = sc[1];
  }
  __device__ double gather(int i) const { return ycur[i]; }
  __device__ void row(int j, double s, double *acc) const {
    double xc = xcur[j];
    double t = xc - tau * (d.c[j] - s);
    double xh = fmax(d.lv[j], fmin(t, d.uv[j]));
    if (MAJOR) {
      d.xhat[j] = xh;
      d.lam[j] = (xh - t) / tau;
    }
    double xr = 2.0 * xh - xc;
    d.xref[j] = xr;
    if (FPE) {
      double dd = xr - xc;
      d.dx[j] = dd;
      acc[0] += dd * dd;
    }
    double refl = d.rho_is_one ? xr : d.rho * xr + d.one_minus_rho * xc;
    xnext[j] = w * refl + omw * d.x0[j];
  }
};

template <bool MAJOR, bool FPE>
struct DualEpi {
  using val_t = double;
  using acc_t = double;
  static constexpr int NF = FPE ? 1 : 0;
  static constexpr unsigned MAXMASK = 0;
  Dev d;
  int off;
  const double *ycur;
  double *ynext;
  double sigma, inv_sigma, w, omw;
  __device__ bool init() {
    const Ctl *c = d.ctl;
    if (c->done) return false;
    sigma = c->sigma;
    inv_sigma = c->inv_sigma;
    return true;
  }
  __device__ void prologue(double *sc) const { halpern_weight(d.ctl, off, sc); }
  __device__ void bind(const double *sc) {
    w = sc[0];
    omw = sc[1];
  }
  __device__ double gather(int j) const { return d.xref[j]; }
  __device__ void row(int i, double s, double *acc) const {
    double yc = ycur[i];
    // the reference divides by sigma; one reciprocal per launch instead
    // (at most 1 ulp apart; an FP64 division costs ~10 FP64 issue slots)
    double t = yc * inv_sigma - s;
    double tp = fmax(-d.uc[i], fmin(t, -d.lc[i]));
    double yh = (t - tp) * sigma;
    if (MAJOR) d.yhat[i] = yh;
    double yr = 2.0 * yh - yc;
    if (FPE) {
      double dd = yr - yc;
      d.dy[i] = dd;
      acc[0] += dd * dd;
    }
    double refl = d.rho_is_one ? yr : d.rho * yr + d.one_minus_rho * yc;
    ynext[i] = w * refl + omw * d.y0[i];
  }
};

// cross term <A^T dy, dx> of the fixed-point error (pdlp_core_op.cu:658-696)
template <bool RESTART_ONLY>
struct FpeEpi {
  using val_t = double;
  using acc_t = double;
  static constexpr int NF = 1;
  static constexpr unsigned MAXMASK = 0;
  Dev d;
  PDLP_NO_BLOCK_SCALARS
  __device__ bool init() {
    if (d.ctl->done) return false;
    if (RESTART_ONLY && !d.ctl->do_restart) return false;
    return true;
  }
  __device__ double gather(int i) const { return d.dy[i]; }
  __device__ void row(int j, double s, double *acc) const { acc[0] += s * d.dx[j]; }
};

// KKT over A x_hat (utils.cu:503-531 constraint half)
template <bool LINF>
struct EvalAEpi {
  using val_t = double;
  using acc_t = double;
  static constexpr int NF = 2;
  static constexpr unsigned MAXMASK = LINF ? 1u : 0u;
  Dev d;
  PDLP_NO_BLOCK_SCALARS
  __device__ bool init() { return !d.ctl->done; }
  __device__ double gather(int j) const { return d.xhat[j]; }
  __device__ void row(int i, double s, double *acc) const {
    double cl = fmax(d.lc[i], fmin(s, d.uc[i]));
    double pr = (s - cl) * d.Dr[i];
    acc[0] = LINF ? fmax(acc[0], fabs(pr)) : acc[0] + pr * pr;
    double yh = d.yhat[i];
    acc[1] += fmax(yh, 0.0) * d.lcf[i] + fmin(yh, 0.0) * d.ucf[i];
  }
};

// KKT over A^T y_hat (utils.cu:503-531 variable half, plus objective dots)
template <bool LINF>
struct EvalATEpi {
  using val_t = double;
  using acc_t = double;
  static constexpr int NF = 3;
  static constexpr unsigned MAXMASK = LINF ? 1u : 0u;
  Dev d;
  PDLP_NO_BLOCK_SCALARS
  __device__ bool init() { return !d.ctl->done; }
  __device__ double gather(int i) const { return d.yhat[i]; }
  __device__ void row(int j, double s, double *acc) const {
    double lam = d.lam[j];
    double dr = (d.c[j] - s - lam) * d.Dc[j];
    acc[0] = LINF ? fmax(acc[0], fabs(dr)) : acc[0] + dr * dr;
    double xh = d.xhat[j];
    acc[1] += d.c[j] * xh;
    acc[2] += lam * xh;
  }
};

__device__ __forceinline__ double ray_scale(const Ctl *c) {
  double p = c->ray_primal_inf_norm;
  return p > 0.0 ? 1.0 / p : 1.0;
}

// primal ray over A (utils.cu:561-572, :588-600)
struct InfAEpi {
  using val_t = double;
  using acc_t = double;
  static constexpr int NF = 2;
  static constexpr unsigned MAXMASK = 1u;
  Dev d;
  double sc;
  PDLP_NO_BLOCK_SCALARS
  __device__ bool init() {  // runs twice per solve: a per-thread division is fine
    if (d.ctl->done) return false;
    sc = ray_scale(d.ctl);
    return true;
  }
  __device__ double gather(int j) const { return sc * d.dx[j]; }
  __device__ void row(int i, double s, double *acc) const {
    double pi = (fmax(0.0, -s) * (double)isfinite(d.lc[i]) +
                 fmax(0.0, s) * (double)isfinite(d.uc[i])) * d.Dr[i];
    acc[0] = fmax(acc[0], fabs(pi));
    double dy = d.dy[i];
    acc[1] += fmax(dy, 0.0) * d.lcf[i] + fmin(dy, 0.0) * d.ucf[i];
  }
};

// dual ray over A^T (utils.cu:574-586, :602-614; the slack slot holds A^T dy
// as in the reference call at utils.cu:772-776)
struct InfATEpi {
  using val_t = double;
  using acc_t = double;
  static constexpr int NF = 3;
  static constexpr unsigned MAXMASK = 2u;
  Dev d;
  double sc;
  PDLP_NO_BLOCK_SCALARS
  __device__ bool init() {
    if (d.ctl->done) return false;
    sc = ray_scale(d.ctl);
    return true;
  }
  __device__ double gather(int i) const { return d.dy[i]; }
  __device__ void row(int j, double s, double *acc) const {
    double ns = -s;
    acc[0] += fmax(ns, 0.0) * d.lvf[j] + fmin(ns, 0.0) * d.uvf[j];
    double di = (fmax(0.0, ns) * (double)!isfinite(d.lv[j]) -
                 fmin(0.0, ns) * (double)!isfinite(d.uv[j])) * d.Dc[j];
    acc[1] = fmax(acc[1], fabs(di));
    acc[2] += d.c[j] * (sc * d.dx[j]);
  }
};

// reduced cost (pdlp_core_op.cu:31-40)
struct ReducedCostEpi {
  using val_t = double;
  using acc_t = double;
  static constexpr int NF = 0;
  static constexpr unsigned MAXMASK = 0;
  Dev d;
  PDLP_NO_BLOCK_SCALARS
  __device__ bool init() { return true; }
  __device__ double gather(int i) const { return d.yhat[i]; }
  __device__ void row(int j, double s, double *) const {
    d.auxn[j] = (d.c[j] - s) * d.Dc[j] / d.ob;
  }
};

// power method: g = A^T (inv * v)   (utils.cu:127-136)
struct PowAtEpi {
  using val_t = double;
  using acc_t = double;
  static constexpr int NF = 0;
  static constexpr unsigned MAXMASK = 0;
  Dev d;
  const double *v;
  double inv;
  PDLP_NO_BLOCK_SCALARS
  __device__ bool init() {
    if (d.ctl->pm_done) return false;
    inv = d.ctl->pm_inv_norm;
    return true;
  }
  __device__ double gather(int i) const { return inv * v[i]; }
  __device__ void row(int j, double s, double *) const { d.pm_g[j] = s; }
};

// power method: v' = A g, sum q.v', sum v'^2   (utils.cu:138-144)
struct PowAEpi {
  using val_t = double;
  using acc_t = double;
  static constexpr int NF = 2;
  static constexpr unsigned MAXMASK = 0;
  Dev d;
  const double *v;
  double *vnext;
  double inv;
  PDLP_NO_BLOCK_SCALARS
  __device__ bool init() {
    if (d.ctl->pm_done) return false;
    inv = d.ctl->pm_inv_norm;
    return true;
  }
  __device__ double gather(int j) const { return d.pm_g[j]; }
  __device__ void row(int i, double s, double *acc) const {
    vnext[i] = s;
    double q = inv * v[i];
    acc[0] += q * s;
    acc[1] += s * s;
  }
};

// step sizes derived from eta and omega (reference pdlp_core_op.cu:512, :545)
__device__ __forceinline__ void set_steps(Ctl *c) {
  c->tau = c->step_size / c->primal_weight;
  c->sigma = c->step_size * c->primal_weight;
  c->inv_sigma = 1.0 / c->sigma;
}
__global__ void k_set_steps(Ctl *c) { set_steps(c); }

// ================================================================ launch
template <class Epi>
void launch_spmv(const DevCsr &M, const Epi &epi, double *part, double *lpart,
                 cudaStream_t st) {
  if (M.plan.nblk == 0) return;
  if (M.plan.tile == 2048)
    spmv_fused<2048, Epi><<<M.plan.nblk, kThreads, 0, st>>>(M.ptr, M.col, M.val, M.plan,
                                                             part, lpart, epi);
  else if (M.plan.tile == 1024)
    spmv_fused<1024, Epi><<<M.plan.nblk, kThreads, 0, st>>>(M.ptr, M.col, M.val, M.plan,
                                                             part, lpart, epi);
  else
    spmv_fused<512, Epi><<<M.plan.nblk, kThreads, 0, st>>>(M.ptr, M.col, M.val, M.plan,
                                                            part, lpart, epi);
  PDLP_LAUNCH_CHECK();
}

// ======================================================= element kernels
__global__ void k_set_tbase(Ctl *ctl, int t) { ctl->t_base = t; }

__global__ void k_loop_start(Ctl *ctl) { ctl->t_start_ns = global_ns(); }

// Ray projection + infinity norms (utils.cu:533-559, :744-748)
__global__ void __launch_bounds__(kThreads) k_ray_project(Dev d) {
  if (d.ctl->done) return;
  __shared__ double red[24];
  double a[2] = {0.0, 0.0};
  long stride = (long)gridDim.x * kThreads;
  for (long j = blockIdx.x * (long)kThreads + threadIdx.x; j < d.n; j += stride) {
    double v = d.dx[j];
    if (isfinite(d.lv[j])) v = fmax(v, 0.0);
    if (isfinite(d.uv[j])) v = fmin(v, 0.0);
    d.dx[j] = v;
    a[0] = fmax(a[0], fabs(v));
  }
  for (long i = blockIdx.x * (long)kThreads + threadIdx.x; i < d.m; i += stride) {
    double v = d.dy[i];
    if (!isfinite(d.lc[i])) v = fmin(v, 0.0);
    if (!isfinite(d.uc[i])) v = fmax(v, 0.0);
    d.dy[i] = v;
    a[1] = fmax(a[1], fabs(v));
  }
  block_reduce_fields<2, 3u>(a, red);
  if (threadIdx.x == 0) {
    d.p_i0[blockIdx.x] = a[0];
    d.p_i0[gridDim.x + blockIdx.x] = a[1];
  }
}

__global__ void __launch_bounds__(kThreads) k_ray_project_fin(Dev d) {
  if (d.ctl->done) return;
  __shared__ double sm[32];
  double p = block_fold<true>(d.p_i0, d.ew_grid, sm);
  double q = block_fold<true>(d.p_i0 + d.ew_grid, d.ew_grid, sm);
  if (threadIdx.x == 0) {
    d.ctl->ray_primal_inf_norm = p;
    d.ctl->ray_dual_inf_norm = q;
  }
}

// Restart copy + distances (pdlp_core_op.cu:577-591, :621-632)
__global__ void __launch_bounds__(kThreads)
    k_restart(Dev d, double *xcur, double *ycur) {
  if (d.ctl->done || !d.ctl->do_restart) return;
  __shared__ double red[24];
  double a[2] = {0.0, 0.0};
  long stride = (long)gridDim.x * kThreads;
  for (long j = blockIdx.x * (long)kThreads + threadIdx.x; j < d.n; j += stride) {
    double xh = d.xhat[j];
    double dd = xh - d.x0[j];
    a[0] += dd * dd;
    d.x0[j] = xh;
    xcur[j] = xh;
  }
  for (long i = blockIdx.x * (long)kThreads + threadIdx.x; i < d.m; i += stride) {
    double yh = d.yhat[i];
    double dd = yh - d.y0[i];
    a[1] += dd * dd;
    d.y0[i] = yh;
    ycur[i] = yh;
  }
  block_reduce_fields<2, 0u>(a, red);
  if (threadIdx.x == 0) {
    d.p_rs[blockIdx.x] = a[0];
    d.p_rs[gridDim.x + blockIdx.x] = a[1];
  }
}

// PID primal-weight update (pdlp_core_op.cu:593-619)
__global__ void __launch_bounds__(kThreads) k_restart_fin(Dev d, int off) {
  Ctl *c = d.ctl;
  if (c->done || !c->do_restart) return;
  __shared__ double sm[32];
  double ps = block_fold<false>(d.p_rs, d.ew_grid, sm);
  double ds = block_fold<false>(d.p_rs + d.ew_grid, d.ew_grid, sm);
  if (threadIdx.x != 0) return;
  double pd = sqrt(ps), dd = sqrt(ds);
  double ratio = c->rel_dual_res / c->rel_primal_res;
  if (pd > 1e-16 && dd > 1e-16 && pd < 1e12 && dd < 1e12 && ratio > 1e-8 && ratio < 1e8) {
    double err = log(dd) - log(pd) - log(c->primal_weight);
    c->pw_error_sum *= d.ismooth;
    c->pw_error_sum += err;
    double derr = err - c->pw_last_error;
    c->primal_weight *= exp(d.kp * err + d.ki * c->pw_error_sum + d.kd * derr);
    c->pw_last_error = err;
  } else {
    c->primal_weight = c->best_primal_weight;
    c->pw_error_sum = 0.0;
    c->pw_last_error = 0.0;
  }
  double g = fabs(log10(c->rel_dual_res / c->rel_primal_res));
  if (g < c->best_gap) {
    c->best_gap = g;
    c->best_primal_weight = c->primal_weight;
  }
  set_steps(c);
  c->restart_t = c->t_base + off;
  c->last_trial_fixed_point_error = INFINITY;
}

// Fixed-point error (pdlp_core_op.cu:677-695) + restart bookkeeping
// (solver.cu:89-95)
__global__ void __launch_bounds__(kThreads) k_fpe_fin(Dev d, int restart_only) {
  Ctl *c = d.ctl;
  if (c->done) return;
  if (restart_only && !c->do_restart) return;
  __shared__ double sm[32];
  double pn2 = fold_site<false>(d.p_pstep, d.nblkT, d.lp_pstep, d.nlongT, 0, sm);
  double dn2 = fold_site<false>(d.p_dstep, d.nblkA, d.lp_dstep, d.nlongA, 0, sm);
  double cross = fold_site<false>(d.p_fpe, d.nblkT, d.lp_fpe, d.nlongT, 0, sm);
  if (threadIdx.x != 0) return;
  double pn = sqrt(pn2), dn = sqrt(dn2);
  double w = c->primal_weight;
  double movement = pn * pn * w + dn * dn / w;
  double interaction = 2 * c->step_size * cross;
  c->fixed_point_error = sqrt(movement + interaction);
  if (c->do_restart) {
    c->initial_fixed_point_error = c->fixed_point_error;
    c->do_restart = 0;
  }
}

// Evaluation: KKT scalars, optional ray statistics, termination test,
// restart decision, trace record (utils.cu:639-813, :239-293; solver.cu:59-83)
__global__ void __launch_bounds__(kThreads)
    k_eval_fin(Dev d, int off, int infeas, int restart_check, int final_eval) {
  Ctl *c = d.ctl;
  if (c->done) return;
  __shared__ double sm[32];
  const bool L = d.linf != 0;
  double pr = L ? fold_site<true>(d.p_e1, d.nblkA, d.lp_e1, d.nlongA, 0, sm)
                : fold_site<false>(d.p_e1, d.nblkA, d.lp_e1, d.nlongA, 0, sm);
  double qsum = fold_site<false>(d.p_e1, d.nblkA, d.lp_e1, d.nlongA, 1, sm);
  double dr = L ? fold_site<true>(d.p_e2, d.nblkT, d.lp_e2, d.nlongT, 0, sm)
                : fold_site<false>(d.p_e2, d.nblkT, d.lp_e2, d.nlongT, 0, sm);
  double cx = fold_site<false>(d.p_e2, d.nblkT, d.lp_e2, d.nlongT, 1, sm);
  double lx = fold_site<false>(d.p_e2, d.nblkT, d.lp_e2, d.nlongT, 2, sm);
  double i1max = 0, i1sum = 0, i2sum = 0, i2max = 0, i2c = 0;
  if (infeas) {
    i1max = fold_site<true>(d.p_i1, d.nblkA, d.lp_i1, d.nlongA, 0, sm);
    i1sum = fold_site<false>(d.p_i1, d.nblkA, d.lp_i1, d.nlongA, 1, sm);
    i2sum = fold_site<false>(d.p_i2, d.nblkT, d.lp_i2, d.nlongT, 0, sm);
    i2max = fold_site<true>(d.p_i2, d.nblkT, d.lp_i2, d.nlongT, 1, sm);
    i2c = fold_site<false>(d.p_i2, d.nblkT, d.lp_i2, d.nlongT, 2, sm);
  }
  if (threadIdx.x != 0) return;
  const int t = c->t_base + off;
  const double cbo = d.cb * d.ob;
  c->abs_primal_res = (L ? pr : sqrt(pr)) / d.cb;
  c->abs_dual_res = (L ? dr : sqrt(dr)) / d.ob;
  c->primal_obj = cx / cbo + d.c0;
  c->dual_obj = (lx + qsum) / cbo + d.c0;
  c->rel_primal_res = c->abs_primal_res / (1.0 + d.bnorm);
  c->rel_dual_res = c->abs_dual_res / (1.0 + d.cnorm);
  c->gap = fabs(c->primal_obj - c->dual_obj);
  c->rel_gap = c->gap / (1.0 + fabs(c->primal_obj) + fabs(c->dual_obj));
  if (infeas) {
    c->primal_ray_obj = i2c / cbo;
    c->dual_ray_obj = (i1sum + i2sum) / cbo;
    c->max_primal_ray_inf = i1max;
    c->max_dual_ray_inf = i2max;
    double scale = fmax(c->ray_dual_inf_norm, i2max);
    if (scale > 0.0) {
      c->max_dual_ray_inf /= scale;
      c->dual_ray_obj /= scale;
    } else {
      c->max_dual_ray_inf = 0.0;
      c->dual_ray_obj = 0.0;
    }
  }
  c->cum_time = (double)(global_ns() - c->t_start_ns) * 1e-9;
  int reason = TERMINATION_REASON_UNSPECIFIED;
  if (final_eval) {
    reason = TERMINATION_REASON_ITERATION_LIMIT;
  } else if (c->rel_dual_res < d.eps_feas && c->rel_primal_res < d.eps_feas &&
             c->rel_gap < d.eps_opt) {
    reason = TERMINATION_REASON_OPTIMAL;
  } else if (c->dual_ray_obj > 0.0 && c->max_dual_ray_inf / c->dual_ray_obj <= d.eps_inf) {
    reason = TERMINATION_REASON_PRIMAL_INFEASIBLE;
  } else if (c->primal_ray_obj < 0.0 &&
             c->max_primal_ray_inf / (-c->primal_ray_obj) <= d.eps_inf) {
    reason = TERMINATION_REASON_DUAL_INFEASIBLE;
  } else if (c->cum_time >= d.time_limit) {
    reason = TERMINATION_REASON_TIME_LIMIT;
  }
  if (d.trace && c->trace_len < d.trace_cap) {
    double *r = d.trace + (long)c->trace_len * 10;
    r[0] = t;
    r[1] = c->rel_primal_res;
    r[2] = c->rel_dual_res;
    r[3] = c->rel_gap;
    r[4] = c->primal_obj;
    r[5] = c->dual_obj;
    r[6] = c->primal_weight;
    r[7] = c->fixed_point_error;
    r[8] = c->step_size;
    r[9] = t - c->restart_t;
    c->trace_len++;
  }
  if (d.verbose && t % print_frequency(t) == 0)
    printf("%6d %.1e | %8.1e  %8.1e | %.1e %.1e %.1e | %.1e %.1e %.1e \n", t, c->cum_time,
           c->primal_obj, c->dual_obj, c->abs_primal_res, c->abs_dual_res, c->gap,
           c->rel_primal_res, c->rel_dual_res, c->rel_gap);
  if (reason != TERMINATION_REASON_UNSPECIFIED) {
    c->reason = reason;
    c->final_t = t;
    c->done = 1;
    __threadfence_system();
    d.hflag->done = 1;
    return;
  }
  if (restart_check) {
    // should_do_adaptive_restart (utils.cu:265-293)
    bool r = false;
    int inner = t - c->restart_t;
    if (t == d.F) {
      r = true;
    } else if (t > d.F) {
      double f = c->fixed_point_error, f0 = c->initial_fixed_point_error;
      if (f <= d.suff * f0) r = true;
      if (f <= d.nec * f0 && f > c->last_trial_fixed_point_error) r = true;
      if (inner >= d.art * t) r = true;
    }
    c->last_trial_fixed_point_error = c->fixed_point_error;
    c->do_restart = r ? 1 : 0;
  }
}

// ---- power method element kernels (utils.cu:107-153)
__global__ void __launch_bounds__(kThreads) k_pm_norm(Dev d, const double *v) {
  if (d.ctl->pm_done) return;
  __shared__ double red[16];
  double a[1] = {0.0};
  long stride = (long)gridDim.x * kThreads;
  for (long i = blockIdx.x * (long)kThreads + threadIdx.x; i < d.m; i += stride)
    a[0] += v[i] * v[i];
  block_reduce_fields<1, 0u>(a, red);
  if (threadIdx.x == 0) d.p_pr[blockIdx.x] = a[0];
}

__global__ void __launch_bounds__(kThreads) k_pm_norm_fin(Dev d) {
  if (d.ctl->pm_done) return;
  __shared__ double sm[32];
  double s = block_fold<false>(d.p_pr, d.ew_grid, sm);
  if (threadIdx.x == 0) d.ctl->pm_inv_norm = 1.0 / sqrt(s);
}

__global__ void __launch_bounds__(kThreads) k_pm_dot_fin(Dev d) {
  Ctl *c = d.ctl;
  if (c->pm_done) return;
  __shared__ double sm[32];
  double dotqv = fold_site<false>(d.p_pa, d.nblkA, d.lp_pa, d.nlongA, 0, sm);
  double vv = fold_site<false>(d.p_pa, d.nblkA, d.lp_pa, d.nlongA, 1, sm);
  if (threadIdx.x == 0) {
    c->pm_sigma_sq = dotqv;
    c->pm_res = vv;  // |v'|^2, turned into 1/|v'| after the residual
  }
}

__global__ void __launch_bounds__(kThreads)
    k_pm_resid(Dev d, const double *v, const double *vnext) {
  if (d.ctl->pm_done) return;
  __shared__ double red[16];
  double inv = d.ctl->pm_inv_norm, ns = -d.ctl->pm_sigma_sq;
  double a[1] = {0.0};
  long stride = (long)gridDim.x * kThreads;
  for (long i = blockIdx.x * (long)kThreads + threadIdx.x; i < d.m; i += stride) {
    double q = inv * v[i];
    double r = 1.0 * vnext[i] + ns * q;
    a[0] += r * r;
  }
  block_reduce_fields<1, 0u>(a, red);
  if (threadIdx.x == 0) d.p_pr[blockIdx.x] = a[0];
}

__global__ void __launch_bounds__(kThreads) k_pm_resid_fin(Dev d) {
  Ctl *c = d.ctl;
  if (c->pm_done) return;
  __shared__ double sm[32];
  double s = block_fold<false>(d.p_pr, d.ew_grid, sm);
  if (threadIdx.x == 0) {
    c->pm_iters++;
    double res = sqrt(s);
    c->pm_inv_norm = 1.0 / sqrt(c->pm_res);
    c->pm_res = res;
    if (res < d.sv_tol) {
      c->pm_done = 1;
      __threadfence_system();
      d.hflag->pm_done = 1;
    }
  }
}

// Unscale (pdlp_core_op.cu:464-480)
__global__ void k_unscale(Dev d) {
  long stride = (long)gridDim.x * blockDim.x;
  for (long j = blockIdx.x * (long)blockDim.x + threadIdx.x; j < d.n; j += stride)
    d.xhat[j] = d.xhat[j] / d.Dc[j] / d.cb;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < d.m; i += stride)
    d.yhat[i] = d.yhat[i] / d.Dr[i] / d.ob;
}

// Finite copies of the scaled bounds (pdlp_core_op.cu:203-230)
__global__ void k_finite_copies(int n, int m, const double *lv, const double *uv,
                                const double *lc, const double *uc, double *lvf,
                                double *uvf, double *lcf, double *ucf) {
  long stride = (long)gridDim.x * blockDim.x;
  for (long j = blockIdx.x * (long)blockDim.x + threadIdx.x; j < n; j += stride) {
    lvf[j] = isfinite(lv[j]) ? lv[j] : 0.0;
    uvf[j] = isfinite(uv[j]) ? uv[j] : 0.0;
  }
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < m; i += stride) {
    lcf[i] = isfinite(lc[i]) ? lc[i] : 0.0;
    ucf[i] = isfinite(uc[i]) ? uc[i] : 0.0;
  }
}

// Warm start scaling (pdlp_core_op.cu:174-201)
__global__ void k_warm_start(int n, int m, const double *xs, const double *ys,
                             const double *Dc, const double *Dr, double cb, double ob,
                             double *x0, double *x, double *xhat, double *y0, double *y,
                             double *yhat) {
  long stride = (long)gridDim.x * blockDim.x;
  if (xs)
    for (long j = blockIdx.x * (long)blockDim.x + threadIdx.x; j < n; j += stride) {
      double v = xs[j] * Dc[j] * cb;
      x0[j] = v;
      x[j] = v;
      xhat[j] = v;
    }
  if (ys)
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < m; i += stride) {
      double v = ys[i] * Dr[i] * ob;
      y0[i] = v;
      y[i] = v;
      yhat[i] = v;
    }
}

// ============================================================ host side
namespace {
size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

struct Arena {
  char *base = nullptr;
  size_t off = 0;
  template <class T>
  T *take(size_t count) {
    T *p = reinterpret_cast<T *>(base + off);
    off += align256(count * sizeof(T) + 1);
    return p;
  }
};

struct Sizer {
  size_t bytes = 0;
  void add(size_t b) { bytes += align256(b + 1); }
};
}  // namespace

void host_transpose(int m, int n, const int *ap, const int *aj, const double *ax,
                    std::vector<int> &tp, std::vector<int> &tj,
                    std::vector<double> &tx) {
  int nnz = ap[m];
  tp.assign((size_t)n + 1, 0);
  tj.resize(nnz);
  tx.resize(nnz);
  for (int k = 0; k < nnz; ++k) tp[aj[k] + 1]++;
  for (int c = 0; c < n; ++c) tp[c + 1] += tp[c];
  std::vector<int> next(tp.begin(), tp.end() - 1);
  for (int r = 0; r < m; ++r)
    for (int k = ap[r]; k < ap[r + 1]; ++k) {
      int pos = next[aj[k]]++;
      tj[pos] = r;
      tx[pos] = ax[k];
    }
}

// Non-zeros per thread-block tile.  PDLP_SPMV_TILE (512, 1024 or 2048)
// overrides the size rule.
static int pick_tile(long nnz) {
  if (const char *e = getenv("PDLP_SPMV_TILE")) {
    int t = atoi(e);
    if (t == 512 || t == 1024 || t == 2048) return t;
  }
  return nnz >= 2000000 ? 2048 : 512;
}

DevProblem::~DevProblem() {
  if (arena) cudaFree(arena);
}

DevProblem *upload_problem(const lp_problem_t *prob, cudaStream_t st) {
  const int n = prob->num_variables, m = prob->num_constraints;
  const int nnz = prob->constraint_matrix_num_nonzeros;
  // A malformed CSR must never reach the host transpose or a device gather.
  {
    const int *rp = prob->constraint_matrix_row_pointers;
    const int *cj = prob->constraint_matrix_col_indices;
    bool ok = n >= 0 && m >= 0 && nnz >= 0 && rp &&
              (nnz == 0 || (cj && prob->constraint_matrix_values)) &&
              (n == 0 || (prob->objective_vector && prob->variable_lower_bound &&
                          prob->variable_upper_bound)) &&
              (m == 0 || (prob->constraint_lower_bound && prob->constraint_upper_bound));
    if (ok) ok = rp[0] == 0 && rp[m] == nnz;
    for (int r = 0; ok && r < m; ++r) ok = rp[r] <= rp[r + 1];
    for (int k = 0; ok && k < nnz; ++k) ok = cj[k] >= 0 && cj[k] < n;
    if (!ok) throw std::runtime_error("invalid CSR matrix (row pointers or column indices)");
  }
  auto P = std::make_unique<DevProblem>();
  P->m = m;
  P->n = n;
  P->nnz = nnz;
  P->tile = pick_tile(nnz);
  P->c0 = prob->objective_constant;
  std::vector<int> tp, tj;
  std::vector<double> tx;
  host_transpose(m, n, prob->constraint_matrix_row_pointers, prob->constraint_matrix_col_indices,
                 prob->constraint_matrix_values, tp, tj, tx);
  std::vector<int4> blkA, blkT;
  std::vector<int2> lrA, lrT;
  build_plan_host(m, prob->constraint_matrix_row_pointers, P->tile, blkA, lrA);
  build_plan_host(n, tp.data(), P->tile, blkT, lrT);
  // norms of the unscaled objective and bounds (reference pdlp_core_op.cu:232-286)
  {
    double ss = 0, mx = 0;
    for (int i = 0; i < n; ++i) {
      double v = prob->objective_vector[i];
      mx = fmax(mx, fabs(v));
      ss += v * v;
    }
    P->cnorm_l2 = sqrt(ss);
    P->cnorm_linf = mx;
    ss = 0;
    mx = 0;
    for (int i = 0; i < m; ++i) {
      double lo = prob->constraint_lower_bound[i], up = prob->constraint_upper_bound[i];
      if (isfinite(lo) && lo != up) {
        mx = fmax(mx, fabs(lo));
        ss += lo * lo;
      }
      if (isfinite(up)) {
        mx = fmax(mx, fabs(up));
        ss += up * up;
      }
    }
    P->bnorm_l2 = sqrt(ss);
    P->bnorm_linf = mx;
  }
  const size_t vn = n, vm = m;
  Sizer z;
  z.add((vm + 1) * 4); z.add((size_t)nnz * 4); z.add((size_t)nnz * 8);
  z.add((vn + 1) * 4); z.add((size_t)nnz * 4); z.add((size_t)nnz * 8);
  z.add(blkA.size() * 16); z.add(lrA.size() * 8);
  z.add(blkT.size() * 16); z.add(lrT.size() * 8);
  for (int i = 0; i < 3; ++i) z.add(vn * 8);
  for (int i = 0; i < 2; ++i) z.add(vm * 8);
  if (prob->primal_start) z.add(vn * 8);
  if (prob->dual_start) z.add(vm * 8);
  PDLP_CUDA(cudaMalloc(&P->arena, z.bytes));
  P->bytes = z.bytes;
  Arena ar{(char *)P->arena, 0};
  auto mat = [&](DevCsr &M, int rows, int cols, std::vector<int4> &blk, std::vector<int2> &lr) {
    M.rows = rows;
    M.cols = cols;
    M.nnz = nnz;
    M.ptr = ar.take<int>((size_t)rows + 1);
    M.col = ar.take<int>(nnz);
    M.val = ar.take<double>(nnz);
    M.plan.rows = rows;
    M.plan.nblk = (int)blk.size();
    M.plan.nlong = (int)lr.size();
    M.plan.tile = P->tile;
    M.plan.blk = ar.take<int4>(blk.size());
    M.plan.lrow = ar.take<int2>(lr.size());
    if (!blk.empty())
      PDLP_CUDA(cudaMemcpyAsync(M.plan.blk, blk.data(), blk.size() * 16, cudaMemcpyHostToDevice, st));
    if (!lr.empty())
      PDLP_CUDA(cudaMemcpyAsync(M.plan.lrow, lr.data(), lr.size() * 8, cudaMemcpyHostToDevice, st));
  };
  mat(P->A, m, n, blkA, lrA);
  mat(P->AT, n, m, blkT, lrT);
  P->c = ar.take<double>(vn);
  P->lv = ar.take<double>(vn);
  P->uv = ar.take<double>(vn);
  P->lc = ar.take<double>(vm);
  P->uc = ar.take<double>(vm);
  auto h2d = [&](void *dst, const void *src, size_t b) {
    if (b) PDLP_CUDA(cudaMemcpyAsync(dst, src, b, cudaMemcpyHostToDevice, st));
  };
  h2d(P->A.ptr, prob->constraint_matrix_row_pointers, (vm + 1) * 4);
  h2d(P->A.col, prob->constraint_matrix_col_indices, (size_t)nnz * 4);
  h2d(P->A.val, prob->constraint_matrix_values, (size_t)nnz * 8);
  h2d(P->AT.ptr, tp.data(), (vn + 1) * 4);
  h2d(P->AT.col, tj.data(), (size_t)nnz * 4);
  h2d(P->AT.val, tx.data(), (size_t)nnz * 8);
  h2d(P->c, prob->objective_vector, vn * 8);
  h2d(P->lv, prob->variable_lower_bound, vn * 8);
  h2d(P->uv, prob->variable_upper_bound, vn * 8);
  h2d(P->lc, prob->constraint_lower_bound, vm * 8);
  h2d(P->uc, prob->constraint_upper_bound, vm * 8);
  if (prob->primal_start) {
    P->xs = ar.take<double>(vn);
    h2d(P->xs, prob->primal_start, vn * 8);
  }
  if (prob->dual_start) {
    P->ys = ar.take<double>(vm);
    h2d(P->ys, prob->dual_start, vm * 8);
  }
  PDLP_CUDA(cudaStreamSynchronize(st));  // host staging (tp/tj/tx) must outlive the copies
  return P.release();
}

Solve::Solve(const pdhg_parameters_t &params, cudaStream_t stream, const DevProblem &prob,
             int trace_cap)
    : p_(params), st_(stream), P_(prob), trace_cap_(trace_cap) {
  alloc();
}

Solve::~Solve() {
  for (auto &kv : graphs_) cudaGraphExecDestroy(kv.second);
  for (auto g : raw_graphs_) cudaGraphDestroy(g);
  if (arena_) cudaFree(arena_);
  if (hflag_) cudaFreeHost(hflag_);
}

void Solve::alloc() {
  const int n = P_.n, m = P_.m, nnz = P_.nnz;
  const int ew = grid_for((long)n + m, 4);
  const size_t vn = n, vm = m;
  const size_t nbA = P_.A.plan.nblk, nbT = P_.AT.plan.nblk;
  const size_t nlA = P_.A.plan.nlong, nlT = P_.AT.plan.nlong;
  Sizer z;
  z.add((size_t)nnz * 8); z.add((size_t)nnz * 8);           // scaled values
  z.add(nlA * 4); z.add(nbA * 8); z.add(nlT * 4); z.add(nbT * 8);  // per-solve plan scratch
  for (int i = 0; i < 6; ++i) z.add(vn * 8);  // c lv uv lvf uvf Dc
  for (int i = 0; i < 5; ++i) z.add(vm * 8);  // lc uc lcf ucf Dr
  for (int i = 0; i < 8; ++i) z.add(vn * 8);  // x[2] x0 xref xhat lam dx auxn
  for (int i = 0; i < 6; ++i) z.add(vm * 8);  // y[2] y0 yhat dy auxm
  z.add(vm * 8); z.add(vm * 8); z.add(vn * 8);  // power v[2], g
  size_t pa = nbA + nlA + 2, pt = nbT + nlT + 2;
  z.add(pt * 8); z.add(pa * 8); z.add(pt * 8);  // pstep dstep fpe
  z.add(pa * 16); z.add(pt * 24);               // e1 e2
  z.add((size_t)ew * 16);                       // i0
  z.add(pa * 16); z.add(pt * 24);               // i1 i2
  z.add((size_t)ew * 16);                       // rs
  z.add(pa * 16); z.add((size_t)ew * 8);        // pa pr
  z.add((size_t)kMiscPart * 8);
  z.add(sizeof(Ctl)); z.add((size_t)trace_cap_ * 80 + 8);
  PDLP_CUDA(cudaMalloc(&arena_, z.bytes));
  Arena ar{(char *)arena_, 0};

  auto mat = [&](DevCsr &W, const DevCsr &S) {
    W = S;
    W.val = ar.take<double>(nnz);
    W.plan.lcnt = ar.take<unsigned>(S.plan.nlong);
    W.plan.lsum = ar.take<double>(S.plan.nblk);
    if (S.plan.nlong)
      PDLP_CUDA(cudaMemsetAsync(W.plan.lcnt, 0, (size_t)S.plan.nlong * 4, st_));
  };
  mat(A_, P_.A);
  mat(AT_, P_.AT);

  Dev &d = d_;
  d.n = n;
  d.m = m;
  d.c = ar.take<double>(vn); d.lv = ar.take<double>(vn); d.uv = ar.take<double>(vn);
  d.lvf = ar.take<double>(vn); d.uvf = ar.take<double>(vn); d.Dc = ar.take<double>(vn);
  d.lc = ar.take<double>(vm); d.uc = ar.take<double>(vm); d.lcf = ar.take<double>(vm);
  d.ucf = ar.take<double>(vm); d.Dr = ar.take<double>(vm);
  d.x[0] = ar.take<double>(vn); d.x[1] = ar.take<double>(vn); d.x0 = ar.take<double>(vn);
  d.xref = ar.take<double>(vn); d.xhat = ar.take<double>(vn); d.lam = ar.take<double>(vn);
  d.dx = ar.take<double>(vn); d.auxn = ar.take<double>(vn);
  d.y[0] = ar.take<double>(vm); d.y[1] = ar.take<double>(vm); d.y0 = ar.take<double>(vm);
  d.yhat = ar.take<double>(vm); d.dy = ar.take<double>(vm); d.auxm = ar.take<double>(vm);
  d.pm_v[0] = ar.take<double>(vm); d.pm_v[1] = ar.take<double>(vm); d.pm_g = ar.take<double>(vn);
  d.nblkA = (int)nbA; d.nlongA = (int)nlA; d.nblkT = (int)nbT; d.nlongT = (int)nlT;
  d.ew_grid = ew;
  auto split = [&](double *&p, double *&lp, size_t nb, size_t nl, int nf) {
    double *base = ar.take<double>((nb + nl + 2) * nf);
    p = base;
    lp = base + nb * nf;
  };
  split(d.p_pstep, d.lp_pstep, nbT, nlT, 1);
  split(d.p_dstep, d.lp_dstep, nbA, nlA, 1);
  split(d.p_fpe, d.lp_fpe, nbT, nlT, 1);
  split(d.p_e1, d.lp_e1, nbA, nlA, 2);
  split(d.p_e2, d.lp_e2, nbT, nlT, 3);
  d.p_i0 = ar.take<double>((size_t)ew * 2);
  split(d.p_i1, d.lp_i1, nbA, nlA, 2);
  split(d.p_i2, d.lp_i2, nbT, nlT, 3);
  d.p_rs = ar.take<double>((size_t)ew * 2);
  split(d.p_pa, d.lp_pa, nbA, nlA, 2);
  d.p_pr = ar.take<double>((size_t)ew);
  d.p_misc = ar.take<double>((size_t)kMiscPart);
  d.ctl = ar.take<Ctl>(1);
  d.trace = trace_cap_ > 0 ? ar.take<double>((size_t)trace_cap_ * 10) : nullptr;
  d.trace_cap = trace_cap_;

  PDLP_CUDA(cudaHostAlloc((void **)&hflag_, sizeof(HostFlag), cudaHostAllocMapped));
  hflag_->done = 0;
  hflag_->pm_done = 0;
  HostFlag *dflag = nullptr;
  PDLP_CUDA(cudaHostGetDevicePointer((void **)&dflag, hflag_, 0));
  d.hflag = dflag;
}

void Solve::prepare() {
  Dev &d = d_;
  const int n = d.n, m = d.m, nnz = P_.nnz;
  auto t0 = std::chrono::steady_clock::now();
  d.c0 = P_.c0;
  d.rho = p_.reflection_coefficient;
  d.one_minus_rho = 1.0 - d.rho;
  d.rho_is_one = d.rho == 1.0;
  d.F = p_.termination_evaluation_frequency > 0 ? p_.termination_evaluation_frequency : 1;
  d.linf = p_.optimality_norm == NORM_TYPE_L_INF;
  d.cnorm = d.linf ? P_.cnorm_linf : P_.cnorm_l2;
  d.bnorm = d.linf ? P_.bnorm_linf : P_.bnorm_l2;
  d.verbose = p_.verbose;
  d.eps_opt = p_.termination_criteria.eps_optimal_relative;
  d.eps_feas = p_.termination_criteria.eps_feasible_relative;
  d.eps_inf = p_.termination_criteria.eps_infeasible;
  d.time_limit = p_.termination_criteria.time_sec_limit;
  d.art = p_.restart_params.artificial_restart_threshold;
  d.suff = p_.restart_params.sufficient_reduction_for_restart;
  d.nec = p_.restart_params.necessary_reduction_for_restart;
  d.kp = p_.restart_params.k_p;
  d.ki = p_.restart_params.k_i;
  d.kd = p_.restart_params.k_d;
  d.ismooth = p_.restart_params.i_smooth;
  d.sv_tol = p_.sv_tol;
  auto d2d = [&](const void *dst, const void *src, size_t b) {
    if (b) PDLP_CUDA(cudaMemcpyAsync((void *)dst, src, b, cudaMemcpyDeviceToDevice, st_));
  };
  d2d(A_.val, P_.A.val, (size_t)nnz * 8);
  d2d(AT_.val, P_.AT.val, (size_t)nnz * 8);
  d2d(d.c, P_.c, (size_t)n * 8);
  d2d(d.lv, P_.lv, (size_t)n * 8);
  d2d(d.uv, P_.uv, (size_t)n * 8);
  d2d(d.lc, P_.lc, (size_t)m * 8);
  d2d(d.uc, P_.uc, (size_t)m * 8);
  gpu_rescale(p_, A_, AT_, (double *)d.c, (double *)d.lv, (double *)d.uv, (double *)d.lc,
              (double *)d.uc, (double *)d.Dr, (double *)d.Dc, &d.cb, &d.ob, d.auxn, d.auxm,
              d.p_misc, st_);
  rescale_sec_ = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  int g = grid_for((long)n + m);
  k_finite_copies<<<g, kThreads, 0, st_>>>(n, m, d.lv, d.uv, d.lc, d.uc, (double *)d.lvf,
                                           (double *)d.uvf, (double *)d.lcf, (double *)d.ucf);
  PDLP_LAUNCH_CHECK();
  for (double *p : {d.x[0], d.x[1], d.x0, d.xref, d.xhat, d.lam, d.dx})
    if (n) PDLP_CUDA(cudaMemsetAsync(p, 0, (size_t)n * 8, st_));
  for (double *p : {d.y[0], d.y[1], d.y0, d.yhat, d.dy})
    if (m) PDLP_CUDA(cudaMemsetAsync(p, 0, (size_t)m * 8, st_));
  if (P_.xs || P_.ys) {
    k_warm_start<<<g, kThreads, 0, st_>>>(n, m, P_.xs, P_.ys, d.Dc, d.Dr, d.cb, d.ob, d.x0,
                                          d.x[0], d.xhat, d.y0, d.y[0], d.yhat);
    PDLP_LAUNCH_CHECK();
  }
  Ctl c0;
  memset(&c0, 0, sizeof(c0));
  c0.best_gap = INFINITY;
  c0.last_trial_fixed_point_error = INFINITY;
  c0.reason = TERMINATION_REASON_UNSPECIFIED;
  PDLP_CUDA(cudaMemcpyAsync(d.ctl, &c0, sizeof(Ctl), cudaMemcpyHostToDevice, st_));
  PDLP_CUDA(cudaStreamSynchronize(st_));
  hflag_->done = 0;
  hflag_->pm_done = 0;
}

void Solve::power_method() {
  Dev &d = d_;
  const int m = d.m;
  // start vector: m draws of N(0,1) from a fresh mt19937(1), like the
  // reference's first solve in a process (utils.cu:29-30, :79-82)
  std::vector<double> v0(m);
  {
    std::mt19937 gen(1);
    std::normal_distribution<double> dist(0.0, 1.0);
    for (int i = 0; i < m; ++i) v0[i] = dist(gen);
  }
  PDLP_CUDA(cudaMemcpyAsync(d.pm_v[0], v0.data(), (size_t)m * 8, cudaMemcpyHostToDevice, st_));
  k_pm_norm<<<d.ew_grid, kThreads, 0, st_>>>(d, d.pm_v[0]);
  k_pm_norm_fin<<<1, kThreads, 0, st_>>>(d);
  PDLP_LAUNCH_CHECK();
  // chunks of power iterations, captured once and replayed until converged
  const int CH = 16;
  auto enqueue = [&](int it) {
    const double *v = d.pm_v[it & 1];
    double *vn = d.pm_v[(it + 1) & 1];
    PowAtEpi e1{d, v, 0.0};
    launch_spmv(AT_, e1, nullptr, nullptr, st_);
    PowAEpi e2{d, v, vn, 0.0};
    launch_spmv(A_, e2, d.p_pa, d.lp_pa, st_);
    k_pm_dot_fin<<<1, kThreads, 0, st_>>>(d);
    k_pm_resid<<<d.ew_grid, kThreads, 0, st_>>>(d, v, vn);
    k_pm_resid_fin<<<1, kThreads, 0, st_>>>(d);
    PDLP_LAUNCH_CHECK();
  };
  cudaGraph_t graph;
  cudaGraphExec_t exec;
  PDLP_CUDA(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal));
  for (int i = 0; i < CH; ++i) enqueue(i);
  PDLP_CUDA(cudaStreamEndCapture(st_, &graph));
  PDLP_CUDA(cudaGraphInstantiate(&exec, graph, 0));
  int launched = 0;
  const int maxit = p_.sv_max_iter;
  // the chunk runs CH iterations; the last partial chunk is run unrolled
  while (launched + CH <= maxit) {
    PDLP_CUDA(cudaGraphLaunch(exec, st_));
    launched += CH;
    launches_ += CH * 5;
    PDLP_CUDA(cudaStreamSynchronize(st_));
    if (hflag_->pm_done) break;
  }
  if (!hflag_->pm_done)
    for (int i = launched; i < maxit; ++i) enqueue(i - launched);  // parity restarts at 0: even CH
  cudaGraphExecDestroy(exec);
  cudaGraphDestroy(graph);
  Ctl c;
  PDLP_CUDA(cudaMemcpyAsync(&c, d.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st_));
  PDLP_CUDA(cudaStreamSynchronize(st_));
  pm_iters_ = c.pm_iters;
  sigma_max_ = sqrt(c.pm_sigma_sq);
}

void Solve::init_step() {
  Dev &d = d_;
  double eta = 1.0;
  if (A_.nnz > 0 && d.m > 0) {
    power_method();
    eta = 0.998 / sigma_max_;
  }
  double omega = p_.bound_objective_rescaling ? 1.0 : (d.cnorm + 1.0) / (d.bnorm + 1.0);
  // ctl offsets of step_size/primal_weight/best_primal_weight are the first 3 doubles
  double s[3] = {eta, omega, omega};
  PDLP_CUDA(cudaMemcpyAsync(d.ctl, s, sizeof(s), cudaMemcpyHostToDevice, st_));
  k_set_steps<<<1, 1, 0, st_>>>(d.ctl);
  PDLP_LAUNCH_CHECK();
  PDLP_CUDA(cudaStreamSynchronize(st_));
}

void Solve::enqueue_eval(int t, int off, bool infeas, bool restart_check, bool final_eval) {
  (void)t;
  Dev &d = d_;
  if (d.linf) {
    launch_spmv(A_, EvalAEpi<true>{d}, d.p_e1, d.lp_e1, st_);
    launch_spmv(AT_, EvalATEpi<true>{d}, d.p_e2, d.lp_e2, st_);
  } else {
    launch_spmv(A_, EvalAEpi<false>{d}, d.p_e1, d.lp_e1, st_);
    launch_spmv(AT_, EvalATEpi<false>{d}, d.p_e2, d.lp_e2, st_);
  }
  launches_ += 2;
  if (infeas) {
    k_ray_project<<<d.ew_grid, kThreads, 0, st_>>>(d);
    k_ray_project_fin<<<1, kThreads, 0, st_>>>(d);
    launch_spmv(A_, InfAEpi{d, 0.0}, d.p_i1, d.lp_i1, st_);
    launch_spmv(AT_, InfATEpi{d, 0.0}, d.p_i2, d.lp_i2, st_);
    launches_ += 4;
  }
  k_eval_fin<<<1, kThreads, 0, st_>>>(d, off, infeas, restart_check, final_eval);
  PDLP_LAUNCH_CHECK();
  launches_ += 1;
}

void Solve::enqueue_iteration(int t, int off, bool) {
  Dev &d = d_;
  IterFlags f = iteration_flags(t, d.F);
  const int par = t & 1;
  double *xc = d.x[par], *xn = d.x[par ^ 1];
  double *yc = d.y[par], *yn = d.y[par ^ 1];
  if (f.eval) enqueue_eval(t, off, f.infeas, f.restart_check, false);
  if (f.maybe_restart) {
    k_restart<<<d.ew_grid, kThreads, 0, st_>>>(d, xc, yc);
    k_restart_fin<<<1, kThreads, 0, st_>>>(d, off);
    PDLP_LAUNCH_CHECK();
    launches_ += 2;
  }
#define PDLP_STEPS(MAJ, FP)                                                         \
  {                                                                                 \
    PrimalEpi<MAJ, FP> pe{d, off, xc, yc, xn, 0.0, 0.0, 0.0};                       \
    launch_spmv(AT_, pe, d.p_pstep, d.lp_pstep, st_);                               \
    DualEpi<MAJ, FP> de{d, off, yc, yn, 0.0, 0.0, 0.0, 0.0};                        \
    launch_spmv(A_, de, d.p_dstep, d.lp_dstep, st_);                                \
  }
  if (f.major_kernel) {
    if (f.fpe) PDLP_STEPS(true, true) else PDLP_STEPS(true, false)
  } else {
    if (f.fpe) PDLP_STEPS(false, true) else PDLP_STEPS(false, false)
  }
#undef PDLP_STEPS
  launches_ += 2;
  if (f.fpe) {
    if (f.fpe_restart_only) launch_spmv(AT_, FpeEpi<true>{d}, d.p_fpe, d.lp_fpe, st_);
    else launch_spmv(AT_, FpeEpi<false>{d}, d.p_fpe, d.lp_fpe, st_);
    k_fpe_fin<<<1, kThreads, 0, st_>>>(d, f.fpe_restart_only ? 1 : 0);
    PDLP_LAUNCH_CHECK();
    launches_ += 2;
  }
}

cudaGraphExec_t Solve::chunk_graph(int t0, int t1) {
  std::string key;
  key.reserve((size_t)(t1 - t0) * 8 + 8);
  key += (char)('0' + (t0 & 1));
  for (int t = t0; t < t1; ++t) {
    IterFlags f = iteration_flags(t, d_.F);
    key += (char)('A' + (f.eval) + 2 * f.infeas + 4 * f.restart_check + 8 * f.maybe_restart);
    key += (char)('A' + (f.major_kernel) + 2 * f.fpe + 4 * f.fpe_restart_only);
  }
  auto it = graphs_.find(key);
  if (it != graphs_.end()) return it->second;
  cudaGraph_t g;
  cudaGraphExec_t e;
  long saved = launches_;
  PDLP_CUDA(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal));
  for (int t = t0; t < t1; ++t) enqueue_iteration(t, t - t0, true);
  PDLP_CUDA(cudaStreamEndCapture(st_, &g));
  PDLP_CUDA(cudaGraphInstantiate(&e, g, 0));
  launches_ = saved;
  raw_graphs_.push_back(g);
  graphs_[key] = e;
  return e;
}

void Solve::run() {
  Dev &d = d_;
  const int L = p_.termination_criteria.iteration_limit;
  const int CH = 100;
  auto t0 = std::chrono::steady_clock::now();
  k_loop_start<<<1, 1, 0, st_>>>(d.ctl);
  PDLP_LAUNCH_CHECK();
  cudaEvent_t ev[2];
  PDLP_CUDA(cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming));
  PDLP_CUDA(cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming));
  int t = 0, k = 0;
  while (t < L) {
    if (hflag_->done) break;
    int t1 = (int)std::min<long>((long)L, ((long)t / CH + 1) * CH);
    cudaGraphExec_t g = chunk_graph(t, t1);
    if (k >= 2) PDLP_CUDA(cudaEventSynchronize(ev[k & 1]));
    if (hflag_->done) break;
    k_set_tbase<<<1, 1, 0, st_>>>(d.ctl, t);
    PDLP_LAUNCH_CHECK();
    PDLP_CUDA(cudaGraphLaunch(g, st_));
    PDLP_CUDA(cudaEventRecord(ev[k & 1], st_));
    // count kernels of the chunk (device-side early exits still launch)
    for (int tt = t; tt < t1; ++tt) {
      IterFlags f = iteration_flags(tt, d.F);
      launches_ += 2 + (f.eval ? 3 + (f.infeas ? 4 : 0) : 0) + (f.maybe_restart ? 2 : 0) +
                   (f.fpe ? 2 : 0);
    }
    launches_ += 1;
    ++k;
    t = t1;
  }
  PDLP_CUDA(cudaStreamSynchronize(st_));
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
  if (!hflag_->done) {
    // iteration limit: one more evaluation at total_count = L (solver.cu:105-109)
    k_set_tbase<<<1, 1, 0, st_>>>(d.ctl, L);
    enqueue_eval(L, 0, false, false, true);
    PDLP_CUDA(cudaStreamSynchronize(st_));
  }
  loop_sec_ = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

void Solve::time_kernels(int reps, double *ms) {
  Dev &d = d_;
  cudaEvent_t e0, e1;
  PDLP_CUDA(cudaEventCreate(&e0));
  PDLP_CUDA(cudaEventCreate(&e1));
  auto timed = [&](auto &&launch) {
    launch();  // warm
    PDLP_CUDA(cudaEventRecord(e0, st_));
    for (int i = 0; i < reps; ++i) launch();
    PDLP_CUDA(cudaEventRecord(e1, st_));
    PDLP_CUDA(cudaEventSynchronize(e1));
    float t = 0;
    PDLP_CUDA(cudaEventElapsedTime(&t, e0, e1));
    return (double)t / reps;
  };
  PrimalEpi<false, false> pe{d, 0, d.x[0], d.y[0], d.x[1], 0.0, 0.0, 0.0};
  DualEpi<false, false> de{d, 0, d.y[0], d.y[1], 0.0, 0.0, 0.0, 0.0};
  ms[0] = timed([&] { launch_spmv(AT_, pe, nullptr, nullptr, st_); });
  ms[1] = timed([&] { launch_spmv(A_, de, d.p_dstep, d.lp_dstep, st_); });
  ms[2] = timed([&] { launch_spmv(A_, EvalAEpi<false>{d}, d.p_e1, d.lp_e1, st_); });
  ms[3] = timed([&] { launch_spmv(AT_, EvalATEpi<false>{d}, d.p_e2, d.lp_e2, st_); });
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
}

std::vector<double> Solve::trace() const {
  Ctl c;
  PDLP_CUDA(cudaMemcpy(&c, d_.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost));
  std::vector<double> tr((size_t)c.trace_len * 10);
  if (c.trace_len)
    PDLP_CUDA(cudaMemcpy(tr.data(), d_.trace, tr.size() * 8, cudaMemcpyDeviceToHost));
  return tr;
}

cupdlpx_result_t *Solve::result() {
  Dev &d = d_;
  const int n = d.n, m = d.m;
  launch_spmv(AT_, ReducedCostEpi{d}, nullptr, nullptr, st_);
  k_unscale<<<grid_for((long)n + m), kThreads, 0, st_>>>(d);
  PDLP_LAUNCH_CHECK();
  auto *r = (cupdlpx_result_t *)calloc(1, sizeof(cupdlpx_result_t));
  if (!r) throw std::bad_alloc();
  r->primal_solution = (double *)malloc(sizeof(double) * (n ? n : 1));
  r->dual_solution = (double *)malloc(sizeof(double) * (m ? m : 1));
  r->reduced_cost = (double *)malloc(sizeof(double) * (n ? n : 1));
  if (!r->primal_solution || !r->dual_solution || !r->reduced_cost) {
    free(r->primal_solution);
    free(r->dual_solution);
    free(r->reduced_cost);
    free(r);
    throw std::bad_alloc();
  }
  if (n) {
    PDLP_CUDA(cudaMemcpyAsync(r->primal_solution, d.xhat, (size_t)n * 8, cudaMemcpyDeviceToHost, st_));
    PDLP_CUDA(cudaMemcpyAsync(r->reduced_cost, d.auxn, (size_t)n * 8, cudaMemcpyDeviceToHost, st_));
  }
  if (m)
    PDLP_CUDA(cudaMemcpyAsync(r->dual_solution, d.yhat, (size_t)m * 8, cudaMemcpyDeviceToHost, st_));
  Ctl c;
  PDLP_CUDA(cudaMemcpyAsync(&c, d.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st_));
  PDLP_CUDA(cudaStreamSynchronize(st_));
  r->num_variables = n;
  r->num_constraints = m;
  r->num_nonzeros = P_.nnz;
  r->num_reduced_variables = n;
  r->num_reduced_constraints = m;
  r->num_reduced_nonzeros = P_.nnz;
  r->total_count = c.final_t;
  r->rescaling_time_sec = rescale_sec_;
  r->cumulative_time_sec = c.cum_time;
  r->presolve_time = 0.0;
  r->presolve_status = 0;
  r->absolute_primal_residual = c.abs_primal_res;
  r->relative_primal_residual = c.rel_primal_res;
  r->absolute_dual_residual = c.abs_dual_res;
  r->relative_dual_residual = c.rel_dual_res;
  r->primal_objective_value = c.primal_obj;
  r->dual_objective_value = c.dual_obj;
  r->objective_gap = c.gap;
  r->relative_objective_gap = c.rel_gap;
  r->max_primal_ray_infeasibility = c.max_primal_ray_inf;
  r->max_dual_ray_infeasibility = c.max_dual_ray_inf;
  r->primal_ray_linear_objective = c.primal_ray_obj;
  r->dual_ray_objective = c.dual_ray_obj;
  r->termination_reason = (termination_reason_t)c.reason;
  r->feasibility_polishing_time = 0.0;
  r->feasibility_iteration = 0;
  return r;
}

}  // namespace pdlp
