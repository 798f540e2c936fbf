// solver_impl.cuh -- restarted Halpern PDHG on one GPU (FP64 or FP32 iterates).
// Template definitions, instantiated once per arithmetic in solver.cu,
// solver_f32.cu and solver_mix.cu (compiled in parallel).
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
// Chunks of iterations are captured once as CUDA graphs and replayed.
#pragma once

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <chrono>
#include <random>

#include <type_traits>

#include "iter_kernels.cuh"

namespace pdlp {

// Non-template kernels, defined in solver.cu.
__global__ void k_set_tbase(Ctl *ctl, int t);
__global__ void k_halpern_table(double *hw, int len);
__global__ void k_loop_start(Ctl *ctl);
__global__ void k_set_steps(Ctl *c);
__global__ void k_pm_norm(PowDev d, const double *v);
__global__ void k_pm_norm_fin(PowDev d);
__global__ void k_pm_dot_fin(PowDev d);
__global__ void k_pm_resid(PowDev d, const double *v, const double *vnext);
__global__ void k_pm_resid_fin(PowDev d);


// Evaluation modes of k_eval_fin.
enum EvalMode { kEvalCheck = 0, kEvalIterLimit = 1, kEvalOnly = 2 };

// ======================================================= element kernels

// Ray projection + infinity norms (utils.cu:533-559, :744-748)
template <class T>
__global__ void __launch_bounds__(kThreads) k_ray_project(Dev<T> d) {
  if (d.ctl->done) return;
  __shared__ double red[24];
  double a[2] = {0.0, 0.0};
  long stride = (long)gridDim.x * kThreads;
  for (long j = blockIdx.x * (long)kThreads + threadIdx.x; j < d.n; j += stride) {
    T v = d.dx[j];
    if (isfinite(d.lv[j])) v = fmax(v, T(0));
    if (isfinite(d.uv[j])) v = fmin(v, T(0));
    d.dx[j] = v;
    a[0] = fmax(a[0], fabs((double)v));
  }
  for (long i = blockIdx.x * (long)kThreads + threadIdx.x; i < d.m; i += stride) {
    T v = d.dy[i];
    if (!isfinite(d.lc[i])) v = fmin(v, T(0));
    if (!isfinite(d.uc[i])) v = fmax(v, T(0));
    d.dy[i] = v;
    a[1] = fmax(a[1], fabs((double)v));
  }
  block_reduce_fields<2, 3u>(a, red);
  if (threadIdx.x == 0) {
    d.p_i0[blockIdx.x] = a[0];
    d.p_i0[gridDim.x + blockIdx.x] = a[1];
  }
}

template <class T>
__global__ void __launch_bounds__(kThreads) k_ray_project_fin(Dev<T> d) {
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
template <class T>
__global__ void __launch_bounds__(kThreads) k_restart(Dev<T> d, T *xcur, T *ycur) {
  if (d.ctl->done || !d.ctl->do_restart) return;
  __shared__ double red[24];
  double a[2] = {0.0, 0.0};
  long stride = (long)gridDim.x * kThreads;
  // polishing restarts one side (reference perform_primal / dual_restart)
  if (d.polish != 2)
    for (long j = blockIdx.x * (long)kThreads + threadIdx.x; j < d.n; j += stride) {
      T xh = d.xhat[j];
      double dd = (double)xh - (double)d.x0[j];
      a[0] += dd * dd;
      d.x0[j] = xh;
      xcur[j] = xh;
    }
  if (d.polish != 1)
    for (long i = blockIdx.x * (long)kThreads + threadIdx.x; i < d.m; i += stride) {
      T yh = d.yhat[i];
      double dd = (double)yh - (double)d.y0[i];
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
template <class T>
__global__ void __launch_bounds__(kThreads) k_restart_fin(Dev<T> d, int off) {
  Ctl *c = d.ctl;
  if (c->done || !c->do_restart) return;
  __shared__ double sm[32];
  double ps = block_fold<false>(d.p_rs, d.ew_grid, sm);
  double ds = block_fold<false>(d.p_rs + d.ew_grid, d.ew_grid, sm);
  if (threadIdx.x != 0) return;
  if (d.polish) {  // polishing keeps the primal weight
    c->restart_t = c->t_base + off;
    c->last_trial_fixed_point_error = INFINITY;
    return;
  }
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
template <class T>
__global__ void __launch_bounds__(kThreads) k_fpe_fin(Dev<T> d, int restart_only) {
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
  if (d.polish == 1) {  // reference compute_primal_fixed_point_error
    c->fixed_point_error = pn * pn * w;
  } else if (d.polish == 2) {  // reference compute_dual_fixed_point_error
    c->fixed_point_error = dn * dn / w;
  } else {
    double movement = pn * pn * w + dn * dn / w;
    double interaction = 2 * c->step_size * cross;
    c->fixed_point_error = sqrt(movement + interaction);
  }
  if (c->do_restart) {
    c->initial_fixed_point_error = c->fixed_point_error;
    c->do_restart = 0;
  }
}

// Evaluation: KKT scalars, optional ray statistics, termination test,
// restart decision, trace record (utils.cu:639-813, :239-293; solver.cu:59-83)
template <class T>
__global__ void __launch_bounds__(kThreads)
    k_eval_fin(Dev<T> d, int off, int infeas, int restart_check, int mode) {
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
  if (d.shifted) {  // terms already in original units
    c->primal_obj = cx + d.oc0;
    c->dual_obj = lx + qsum + d.oc0;
  } else {
    c->primal_obj = cx / cbo + d.c0;
    c->dual_obj = (lx + qsum) / cbo + d.c0;
  }
  c->rel_primal_res = c->abs_primal_res / (1.0 + d.bnorm);
  c->rel_dual_res = c->abs_dual_res / (1.0 + d.cnorm);
  c->gap = fabs(c->primal_obj - c->dual_obj);
  c->rel_gap = c->gap / (1.0 + fabs(c->primal_obj) + fabs(c->dual_obj));
  if (mode == kEvalOnly) return;
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
  bool stalled = false;
  if (d.polish) {
    // reference check_feas_polishing_termination_criteria (utils.cu:1015-1039);
    // the other side's residual and the gap are not measured
    if (d.polish == 1) c->abs_dual_res = c->rel_dual_res = 0.0;
    else c->abs_primal_res = c->rel_primal_res = 0.0;
    c->gap = c->rel_gap = 0.0;
    const double r = d.polish == 1 ? c->rel_primal_res : c->rel_dual_res;
    if (r <= d.eps_polish) reason = TERMINATION_REASON_FEAS_POLISH_SUCCESS;
    else if (mode == kEvalIterLimit) reason = TERMINATION_REASON_ITERATION_LIMIT;
    else if (c->cum_time >= d.time_limit) reason = TERMINATION_REASON_TIME_LIMIT;
  } else {
    if (d.stall_min > 0 && mode == kEvalCheck) {
      // best-iterate snapshot and stall rule of the refinement rounds
      double err = fmax(c->rel_primal_res, fmax(c->rel_dual_res, c->rel_gap));
      c->snap_now = err < c->snap_err ? 1 : 0;
      if (c->snap_now) c->snap_err = err;
      if (err < 0.9 * c->best_err) {
        c->best_err = err;
        c->best_err_t = t;
      } else if (c->best_err < d.stall_floor &&
                 t - c->best_err_t > max(d.stall_min, (int)(d.stall_frac * t))) {
        stalled = true;
      }
    }
    if (mode == kEvalIterLimit) {
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
    } else if (stalled) {
      reason = kReasonStalled;
    }
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
    // a polish loop completes the iteration in progress before it stops
    c->final_t = d.polish ? t + 1 : t;
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

// Copy the evaluated iterate into the snapshot when it is the best so far.
template <class T>
__global__ void k_snapshot(Dev<T> d) {
  if (!d.ctl->snap_now) return;
  long stride = (long)gridDim.x * blockDim.x;
  for (long j = blockIdx.x * (long)blockDim.x + threadIdx.x; j < d.n; j += stride) {
    d.bx[j] = d.xhat[j];
    d.bl[j] = d.lam[j];
  }
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < d.m; i += stride)
    d.by[i] = d.yhat[i];
}

// Unscale (pdlp_core_op.cu:464-480) into FP64 outputs; the dual slack maps
// back like the reduced cost (times Dc / ob).
template <class T>
__global__ void k_unscale(Dev<T> d, double *x, double *y, double *lam) {
  long stride = (long)gridDim.x * blockDim.x;
  for (long j = blockIdx.x * (long)blockDim.x + threadIdx.x; j < d.n; j += stride) {
    x[j] = (double)d.xhat[j] / d.Dc[j] / d.cb;
    if (lam) lam[j] = (double)d.lam[j] * d.Dc[j] / d.ob;
  }
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < d.m; i += stride)
    y[i] = (double)d.yhat[i] / d.Dr[i] / d.ob;
}

// Scale an original-units point into this solve's scaled space.
template <class T>
__global__ void k_scale_point(Dev<T> d, const double *x, const double *y, const double *lam) {
  long stride = (long)gridDim.x * blockDim.x;
  for (long j = blockIdx.x * (long)blockDim.x + threadIdx.x; j < d.n; j += stride) {
    d.xhat[j] = (T)(x[j] * d.Dc[j] * d.cb);
    d.lam[j] = (T)(lam[j] * d.ob / d.Dc[j]);
  }
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < d.m; i += stride)
    d.yhat[i] = (T)(y[i] * d.Dr[i] * d.ob);
}

// Finite copies of the scaled bounds (pdlp_core_op.cu:203-230)
template <class T>
__global__ void k_finite_copies(int n, int m, const T *lv, const T *uv, const T *lc,
                                const T *uc, T *lvf, T *uvf, T *lcf, T *ucf) {
  long stride = (long)gridDim.x * blockDim.x;
  for (long j = blockIdx.x * (long)blockDim.x + threadIdx.x; j < n; j += stride) {
    lvf[j] = isfinite(lv[j]) ? lv[j] : T(0);
    uvf[j] = isfinite(uv[j]) ? uv[j] : T(0);
  }
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < m; i += stride) {
    lcf[i] = isfinite(lc[i]) ? lc[i] : T(0);
    ucf[i] = isfinite(uc[i]) ? uc[i] : T(0);
  }
}

// Warm start scaling (pdlp_core_op.cu:174-201)
template <class T>
__global__ void k_warm_start(int n, int m, const double *xs, const double *ys,
                             const double *Dc, const double *Dr, double cb, double ob, T *x0,
                             T *x, T *xhat, T *y0, T *y, T *yhat) {
  long stride = (long)gridDim.x * blockDim.x;
  if (xs)
    for (long j = blockIdx.x * (long)blockDim.x + threadIdx.x; j < n; j += stride) {
      T v = (T)(xs[j] * Dc[j] * cb);
      x0[j] = v;
      x[j] = v;
      xhat[j] = v;
    }
  if (ys)
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < m; i += stride) {
      T v = (T)(ys[i] * Dr[i] * ob);
      y0[i] = v;
      y[i] = v;
      yhat[i] = v;
    }
}

// FP64 -> T copy (rounding to nearest)
template <class T>
__global__ void k_convert(long n, const double *__restrict__ src, T *__restrict__ dst) {
  long stride = (long)gridDim.x * blockDim.x;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += stride)
    dst[i] = (T)src[i];
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
  template <class T>
  void add(size_t count) {
    bytes += align256(count * sizeof(T) + 1);
  }
};
}  // namespace

template <class T, class M>
Solve<T, M>::Solve(const pdhg_parameters_t &params, cudaStream_t stream, const DevProblem &prob,
                int trace_cap)
    : p_(params), st_(stream), P_(prob), trace_cap_(trace_cap) {
  alloc();
}

template <class T, class M>
Solve<T, M>::~Solve() {
  if (snap_mem_) dev_free(snap_mem_, st_);
  for (auto &slot : tev_)
    for (auto ev : slot)
      if (ev) cudaEventDestroy(ev);
  for (auto &kv : graphs_) cudaGraphExecDestroy(kv.second);
  for (auto g : raw_graphs_) cudaGraphDestroy(g);
  if (arena_) dev_free(arena_, st_);
  hostflag_release(hflag_);
}

template <class T, class M>
void Solve<T, M>::alloc() {
  constexpr bool F64 = sizeof(T) == 8;   // iterates in FP64
  constexpr bool M64 = sizeof(M) == 8;   // matrix in FP64
  const int n = P_.n, m = P_.m, nnz = P_.nnz;
  const int ew = grid_for((long)n + m, 4);
  const size_t vn = n, vm = m;
  // reduction partials of an SpMV site: one per CTA of the pipelined kernel
  // (or per block of the fused kernel) plus one per long row
  const size_t nbA = spmv_partials_max(P_.A), nbT = spmv_partials_max(P_.AT);
  const size_t nlA = spmv_long_rows_max(P_.A), nlT = spmv_long_rows_max(P_.AT);
  Sizer z;
  z.add<double>(nnz); z.add<double>(nnz);                      // FP64 scaled values
  if (!M64) { z.add<M>(nnz); z.add<M>(nnz); }                  // iteration values
  for (const DevCsr *W : {&P_.A, &P_.AT}) {                    // SpMV scratch of both kernels
    z.add<unsigned>(W->plan.nlong); z.add<double>(W->plan.nblk);
    z.add<unsigned>(W->pipe.nlong); z.add<double>(W->pipe.ntile); z.add<int>(1);
  }
  for (int i = 0; i < 3; ++i) z.add<double>(vn);               // c lv uv (FP64 scaled)
  for (int i = 0; i < 2; ++i) z.add<double>(vm);               // lc uc
  z.add<double>(vn); z.add<double>(vm);                        // Dc Dr
  if (!F64) {
    for (int i = 0; i < 3; ++i) z.add<T>(vn);
    for (int i = 0; i < 2; ++i) z.add<T>(vm);
  }
  for (int i = 0; i < 2; ++i) z.add<T>(vn);                    // lvf uvf
  for (int i = 0; i < 2; ++i) z.add<T>(vm);                    // lcf ucf
  for (int i = 0; i < 8; ++i) z.add<T>(vn);                    // x[2] x0 xref xhat lam dx auxn
  for (int i = 0; i < 6; ++i) z.add<T>(vm);                    // y[2] y0 yhat dy auxm
  z.add<double>(vm); z.add<double>(vm); z.add<double>(vn);     // power v[2], g
  z.add<double>(vn); z.add<double>(vm); z.add<double>(vn);     // FP64 outputs x, y, rc/lam
  size_t pa = nbA + nlA + 2, pt = nbT + nlT + 2;
  z.add<double>(pt); z.add<double>(pa); z.add<double>(pt);    // pstep dstep fpe
  z.add<double>(pa * 2); z.add<double>(pt * 3);               // e1 e2
  z.add<double>((size_t)ew * 2);                               // i0
  z.add<double>(pa * 2); z.add<double>(pt * 3);               // i1 i2
  z.add<double>((size_t)ew * 2);                               // rs
  z.add<double>(pa * 2); z.add<double>((size_t)ew);           // power partials
  z.add<double>((size_t)kMiscPart);
  z.add<double>((size_t)kHalpernTable);
  z.add<Ctl>(1); z.add<double>((size_t)trace_cap_ * 10 + 1);
  arena_ = dev_alloc(z.bytes, st_);
  Arena ar{(char *)arena_, 0};

  auto mat64 = [&](DevCsr &W, const DevCsr &S) {
    W = S;
    W.val = ar.take<double>(nnz);
    W.plan.lcnt = ar.take<unsigned>(S.plan.nlong);
    W.plan.lsum = ar.take<double>(S.plan.nblk);
    if (S.plan.nlong) PDLP_CUDA(cudaMemsetAsync(W.plan.lcnt, 0, (size_t)S.plan.nlong * 4, st_));
    W.pipe.lcnt = ar.take<unsigned>(S.pipe.nlong);
    W.pipe.lsum = ar.take<double>(S.pipe.ntile);
    W.pipe.err = ar.take<int>(1);
    if (S.pipe.nlong) PDLP_CUDA(cudaMemsetAsync(W.pipe.lcnt, 0, (size_t)S.pipe.nlong * 4, st_));
    PDLP_CUDA(cudaMemsetAsync(W.pipe.err, 0, sizeof(int), st_));
  };
  mat64(A64_, P_.A);
  mat64(AT64_, P_.AT);
  auto matT = [&](DevCsrT<M> &W, const DevCsr &S64) {
    W.rows = S64.rows;
    W.cols = S64.cols;
    W.nnz = S64.nnz;
    W.ptr = S64.ptr;
    W.col = S64.col;
    W.plan = S64.plan;  // shares the per-solve scratch of the FP64 copy
    W.pipe = S64.pipe;
    if constexpr (M64) W.val = (M *)S64.val;
    else W.val = ar.take<M>(nnz);
  };
  matT(A_, A64_);
  matT(AT_, AT64_);

  Dev<T> &d = d_;
  d.n = n;
  d.m = m;
  c64_ = ar.take<double>(vn); lv64_ = ar.take<double>(vn); uv64_ = ar.take<double>(vn);
  lc64_ = ar.take<double>(vm); uc64_ = ar.take<double>(vm);
  d.Dc = ar.take<double>(vn);
  d.Dr = ar.take<double>(vm);
  if constexpr (F64) {
    d.c = (const T *)c64_; d.lv = (const T *)lv64_; d.uv = (const T *)uv64_;
    d.lc = (const T *)lc64_; d.uc = (const T *)uc64_;
  } else {
    d.c = ar.take<T>(vn); d.lv = ar.take<T>(vn); d.uv = ar.take<T>(vn);
    d.lc = ar.take<T>(vm); d.uc = ar.take<T>(vm);
  }
  d.lvf = ar.take<T>(vn); d.uvf = ar.take<T>(vn);
  d.lcf = ar.take<T>(vm); d.ucf = ar.take<T>(vm);
  d.x[0] = ar.take<T>(vn); d.x[1] = ar.take<T>(vn); d.x0 = ar.take<T>(vn);
  d.xref = ar.take<T>(vn); d.xhat = ar.take<T>(vn); d.lam = ar.take<T>(vn);
  d.dx = ar.take<T>(vn); d.auxn = ar.take<T>(vn);
  d.y[0] = ar.take<T>(vm); d.y[1] = ar.take<T>(vm); d.y0 = ar.take<T>(vm);
  d.yhat = ar.take<T>(vm); d.dy = ar.take<T>(vm); d.auxm = ar.take<T>(vm);
  pw_.v[0] = ar.take<double>(vm); pw_.v[1] = ar.take<double>(vm); pw_.g = ar.take<double>(vn);
  outx_ = ar.take<double>(vn); outy_ = ar.take<double>(vm); outl_ = ar.take<double>(vn);
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
  split(pw_.p_pa, pw_.lp_pa, nbA, nlA, 2);
  pw_.p_pr = ar.take<double>((size_t)ew);
  d.p_misc = ar.take<double>((size_t)kMiscPart);
  {
    double *hw = ar.take<double>((size_t)kHalpernTable);
    k_halpern_table<<<grid_for(kHalpernTable), kThreads, 0, st_>>>(hw, kHalpernTable);
    PDLP_LAUNCH_CHECK();
    launches_ += 1;
    d.hw = hw;
    d.hw_len = kHalpernTable;
  }
  d.ctl = ar.take<Ctl>(1);
  d.trace = trace_cap_ > 0 ? ar.take<double>((size_t)trace_cap_ * 10) : nullptr;
  d.trace_cap = trace_cap_;

  hflag_ = hostflag_acquire();
  hflag_->done = 0;
  hflag_->pm_done = 0;
  HostFlag *dflag = nullptr;
  PDLP_CUDA(cudaHostGetDevicePointer((void **)&dflag, hflag_, 0));
  d.hflag = dflag;

  pw_.n = n;
  pw_.m = m;
  pw_.ctl = d.ctl;
  pw_.hflag = dflag;
  pw_.ew_grid = ew;
  // kernels: the problem's measured choice for this precision, a forced one,
  // or the fused kernel until run() measures both
  int cA = 0, cT = 0;
  {
    std::lock_guard<std::mutex> lk(P_.tune_mu);
    const int *ch = P_.kernel_choice[precision_index()];
    if (kernel_override() >= 0) {
      cA = cT = kernel_override();
      tuned_ = true;
    } else if (ch[0] >= 0 && ch[1] >= 0) {
      cA = ch[0];
      cT = ch[1];
      tuned_ = true;
    }
  }
  apply_kernels(cA != 0, cT != 0);
}

template <class T, class M>
void Solve<T, M>::apply_kernels(bool pipe_A, bool pipe_T) {
  Dev<T> &d = d_;
  A64_.pipe_on = A_.pipe_on = pipe_A && P_.A.pipe.ntile > 0;
  AT64_.pipe_on = AT_.pipe_on = pipe_T && P_.AT.pipe.ntile > 0;
  d.nblkA = (int)spmv_partials(A64_);
  d.nlongA = (int)spmv_long_rows(A64_);
  d.nblkT = (int)spmv_partials(AT64_);
  d.nlongT = (int)spmv_long_rows(AT64_);
  pw_.nblkA = d.nblkA;
  pw_.nlongA = d.nlongA;
}

// The SpMV kernel of each matrix, chosen once per problem and precision.
// Below kTuneMinNnz non-zeros both matrices take the fused kernel (launches
// of a few microseconds, where it is never slower).  Above, the step kernel
// of each matrix (primal step over A^T, dual step over A) is timed on both
// kernels, 2 warm and 5 timed launches each, CUDA events on the solve's
// stream, and the pipelined kernel is kept where it is at least 3% faster.
// The choice is recorded for the structure (settle_kernel_choice), so every
// later solve of a matrix of that structure in the process runs the same
// kernels and returns the same bits.  Runs before the first iteration (the
// step kernels only write the next iterates and x_ref, which the loop
// writes before it reads them).
constexpr long kTuneMinNnz = 1L << 22;

template <class T, class M>
void Solve<T, M>::tune_kernels() {
  if (tuned_) return;
  tuned_ = true;
  std::lock_guard<std::mutex> lk(P_.tune_mu);
  int *ch = P_.kernel_choice[precision_index()];
  if (ch[0] < 0 || ch[1] < 0) {
    if (P_.nnz < kTuneMinNnz) {
      ch[0] = ch[1] = 0;
    } else if (!lookup_kernel_choice(P_.shape_key, precision_index(), ch)) {
      Dev<T> &d = d_;
      cudaEvent_t e0, e1;
      PDLP_CUDA(cudaEventCreate(&e0));
      PDLP_CUDA(cudaEventCreate(&e1));
      auto timed = [&](auto &&launch) {
        for (int i = 0; i < 2; ++i) launch();
        PDLP_CUDA(cudaEventRecord(e0, st_));
        for (int i = 0; i < 5; ++i) launch();
        PDLP_CUDA(cudaEventRecord(e1, st_));
        PDLP_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        PDLP_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        return ms;
      };
      PrimalEpi<T, M, false, false, true> pe{d, 0, d.x[0], d.y[0], d.x[1], T(0), T(0), T(0)};
      DualEpi<T, M, false, false, true> de{d, 0, d.y[0], d.y[1], T(0), T(0), T(0), T(0)};
      float tf[2] = {0.f, 0.f}, tp[2] = {0.f, 0.f};
      for (int k = 0; k < 2; ++k) {
        apply_kernels(k != 0, k != 0);
        float a = timed([&] { launch_spmv(A_, de, d.p_dstep, d.lp_dstep, st_); });
        float t = timed([&] { launch_spmv(AT_, pe, d.p_pstep, d.lp_pstep, st_); });
        (k ? tp : tf)[0] = a;
        (k ? tp : tf)[1] = t;
      }
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      ch[0] = P_.A.pipe.ntile > 0 && tp[0] < 0.97f * tf[0] ? 1 : 0;
      ch[1] = P_.AT.pipe.ntile > 0 && tp[1] < 0.97f * tf[1] ? 1 : 0;
      settle_kernel_choice(P_.shape_key, precision_index(), ch);
      tune_ms_[0] = tf[0] / 5; tune_ms_[1] = tp[0] / 5;
      tune_ms_[2] = tf[1] / 5; tune_ms_[3] = tp[1] / 5;
    }
  }
  apply_kernels(ch[0] != 0, ch[1] != 0);
}

template <class T, class M>
void Solve<T, M>::prepare() {
  Dev<T> &d = d_;
  const int n = d.n, m = d.m, nnz = P_.nnz;
  auto t0 = std::chrono::steady_clock::now();
  d.c0 = P_.c0;
  d.shifted = P_.shift_x != nullptr;
  d.sx = P_.shift_x;
  d.sy = P_.shift_y;
  d.oc = P_.orig_c;
  d.olcf = P_.orig_lcf;
  d.oucf = P_.orig_ucf;
  d.oc0 = P_.orig_c0;
  d.sdp_inv = 1.0 / P_.delta_p;
  d.sdd_inv = 1.0 / P_.delta_d;
  d.polish = 0;
  d.eps_polish = p_.termination_criteria.eps_feas_polish_relative;
  d.c_obj = d.c;
  d.x_obj = d.xhat;
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
  pw_.sv_tol = p_.sv_tol;
  auto d2d = [&](const void *dst, const void *src, size_t b) {
    if (b) PDLP_CUDA(cudaMemcpyAsync((void *)dst, src, b, cudaMemcpyDeviceToDevice, st_));
  };
  d2d(A64_.val, P_.A.val, (size_t)nnz * 8);
  d2d(AT64_.val, P_.AT.val, (size_t)nnz * 8);
  d2d(c64_, P_.c, (size_t)n * 8);
  d2d(lv64_, P_.lv, (size_t)n * 8);
  d2d(uv64_, P_.uv, (size_t)n * 8);
  d2d(lc64_, P_.lc, (size_t)m * 8);
  d2d(uc64_, P_.uc, (size_t)m * 8);
  gpu_rescale(p_, A64_, AT64_, c64_, lv64_, uv64_, lc64_, uc64_, (double *)d.Dr,
              (double *)d.Dc, &d.cb, &d.ob, outx_, outy_, d.p_misc, st_, fixed_cb_, fixed_ob_);
  int g = grid_for((long)n + m);
  if constexpr (sizeof(M) != 8) {
    int gz = grid_for(nnz);
    k_convert<M><<<gz, kThreads, 0, st_>>>(nnz, A64_.val, A_.val);
    k_convert<M><<<gz, kThreads, 0, st_>>>(nnz, AT64_.val, AT_.val);
    PDLP_LAUNCH_CHECK();
  }
  if constexpr (sizeof(T) != 8) {
    int gn = grid_for(n), gm = grid_for(m);
    k_convert<T><<<gn, kThreads, 0, st_>>>(n, c64_, (T *)d.c);
    k_convert<T><<<gn, kThreads, 0, st_>>>(n, lv64_, (T *)d.lv);
    k_convert<T><<<gn, kThreads, 0, st_>>>(n, uv64_, (T *)d.uv);
    k_convert<T><<<gm, kThreads, 0, st_>>>(m, lc64_, (T *)d.lc);
    k_convert<T><<<gm, kThreads, 0, st_>>>(m, uc64_, (T *)d.uc);
    PDLP_LAUNCH_CHECK();
  }
  k_finite_copies<T><<<g, kThreads, 0, st_>>>(n, m, d.lv, d.uv, d.lc, d.uc, (T *)d.lvf,
                                              (T *)d.uvf, (T *)d.lcf, (T *)d.ucf);
  PDLP_LAUNCH_CHECK();
  for (T *p : {d.x[0], d.x[1], d.x0, d.xref, d.xhat, d.lam, d.dx})
    if (n) PDLP_CUDA(cudaMemsetAsync(p, 0, (size_t)n * sizeof(T), st_));
  for (T *p : {d.y[0], d.y[1], d.y0, d.yhat, d.dy})
    if (m) PDLP_CUDA(cudaMemsetAsync(p, 0, (size_t)m * sizeof(T), st_));
  if (P_.xs || P_.ys) {
    k_warm_start<T><<<g, kThreads, 0, st_>>>(n, m, P_.xs, P_.ys, d.Dc, d.Dr, d.cb, d.ob, d.x0,
                                             d.x[0], d.xhat, d.y0, d.y[0], d.yhat);
    PDLP_LAUNCH_CHECK();
  }
  Ctl c0;
  memset(&c0, 0, sizeof(c0));
  c0.best_gap = INFINITY;
  c0.last_trial_fixed_point_error = INFINITY;
  c0.reason = TERMINATION_REASON_UNSPECIFIED;
  c0.step_size = 1.0;
  c0.primal_weight = 1.0;
  c0.best_primal_weight = 1.0;
  c0.tau = c0.sigma = c0.inv_sigma = 1.0;
  c0.best_err = INFINITY;
  c0.snap_err = INFINITY;
  PDLP_CUDA(cudaMemcpyAsync(d.ctl, &c0, sizeof(Ctl), cudaMemcpyHostToDevice, st_));
  PDLP_CUDA(cudaStreamSynchronize(st_));
  hflag_->done = 0;
  hflag_->pm_done = 0;
  rescale_sec_ = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

template <class T, class M>
void Solve<T, M>::power_method() {
  PowDev &w = pw_;
  const int m = w.m;
  // start vector: m draws of N(0,1) from a fresh mt19937(1), like the
  // reference's first solve in a process (utils.cu:29-30, :79-82)
  std::vector<double> v0(m);
  {
    std::mt19937 gen(1);
    std::normal_distribution<double> dist(0.0, 1.0);
    for (int i = 0; i < m; ++i) v0[i] = dist(gen);
  }
  PDLP_CUDA(cudaMemcpyAsync(w.v[0], v0.data(), (size_t)m * 8, cudaMemcpyHostToDevice, st_));
  k_pm_norm<<<w.ew_grid, kThreads, 0, st_>>>(w, w.v[0]);
  k_pm_norm_fin<<<1, kThreads, 0, st_>>>(w);
  PDLP_LAUNCH_CHECK();
  launches_ += 2;
  // chunks of power iterations, captured once and replayed until converged
  const int CH = 16;
  auto enqueue = [&](int it) {
    const double *v = w.v[it & 1];
    double *vn = w.v[(it + 1) & 1];
    launch_spmv(AT64_, PowAtEpi{w, v, 0.0}, nullptr, nullptr, st_);
    launch_spmv(A64_, PowAEpi{w, v, vn, 0.0}, w.p_pa, w.lp_pa, st_);
    k_pm_dot_fin<<<1, kThreads, 0, st_>>>(w);
    k_pm_resid<<<w.ew_grid, kThreads, 0, st_>>>(w, v, vn);
    k_pm_resid_fin<<<1, kThreads, 0, st_>>>(w);
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
  while (launched + CH <= maxit) {
    PDLP_CUDA(cudaGraphLaunch(exec, st_));
    launched += CH;
    launches_ += CH * 5;
    PDLP_CUDA(cudaStreamSynchronize(st_));
    if (hflag_->pm_done) break;
  }
  if (!hflag_->pm_done)
    for (int i = launched; i < maxit; ++i) {  // even CH: parity restarts at 0
      enqueue(i - launched);
      launches_ += 5;
    }
  cudaGraphExecDestroy(exec);
  cudaGraphDestroy(graph);
  Ctl c;
  PDLP_CUDA(cudaMemcpyAsync(&c, w.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st_));
  PDLP_CUDA(cudaStreamSynchronize(st_));
  pm_iters_ = c.pm_iters;
  sigma_max_ = sqrt(c.pm_sigma_sq);
}

template <class T, class M>
void Solve<T, M>::init_step(double known_sigma, double known_omega) {
  Dev<T> &d = d_;
  double eta = 1.0;
  if (A64_.nnz > 0 && d.m > 0) {
    if (known_sigma > 0.0) sigma_max_ = known_sigma;
    else power_method();
    eta = 0.998 / sigma_max_;
  }
  double omega = p_.bound_objective_rescaling ? 1.0 : (d.cnorm + 1.0) / (d.bnorm + 1.0);
  if (known_omega > 0.0) omega = known_omega;
  // ctl offsets of step_size/primal_weight/best_primal_weight are the first 3 doubles
  double s[3] = {eta, omega, omega};
  PDLP_CUDA(cudaMemcpyAsync(d.ctl, s, sizeof(s), cudaMemcpyHostToDevice, st_));
  k_set_steps<<<1, 1, 0, st_>>>(d.ctl);
  PDLP_LAUNCH_CHECK();
  PDLP_CUDA(cudaStreamSynchronize(st_));
}

template <class T, class M>
void Solve<T, M>::enqueue_eval(int off, bool infeas, bool restart_check, int mode) {
  Dev<T> &d = d_;
  // KKT evaluation on the FP64 scaled matrix in every precision: an FP32
  // round then stops when the FP64 KKT of its own point meets the tolerance,
  // not when rounding in long cancelling rows lets it (evaluations are about
  // 1% of the SpMVs)
  if (d.linf) {
    launch_spmv(A64_, EvalAEpi<T, double, true>{d}, d.p_e1, d.lp_e1, st_);
    launch_spmv(AT64_, EvalATEpi<T, double, true>{d}, d.p_e2, d.lp_e2, st_);
  } else {
    launch_spmv(A64_, EvalAEpi<T, double, false>{d}, d.p_e1, d.lp_e1, st_);
    launch_spmv(AT64_, EvalATEpi<T, double, false>{d}, d.p_e2, d.lp_e2, st_);
  }
  if (infeas) {
    // the ray statistics likewise on the FP64 matrix: the infeasibility test
    // compares them with eps_infeasible (1e-10 by default), below what FP32
    // sums over long rows resolve
    k_ray_project<T><<<d.ew_grid, kThreads, 0, st_>>>(d);
    k_ray_project_fin<T><<<1, kThreads, 0, st_>>>(d);
    launch_spmv(A64_, InfAEpi<T, double>{d, T(0)}, d.p_i1, d.lp_i1, st_);
    launch_spmv(AT64_, InfATEpi<T, double>{d, T(0)}, d.p_i2, d.lp_i2, st_);
  }
  k_eval_fin<T><<<1, kThreads, 0, st_>>>(d, off, infeas, restart_check, mode);
  PDLP_LAUNCH_CHECK();
  if (snapshot_ && mode == kEvalCheck) {
    k_snapshot<T><<<d.ew_grid, kThreads, 0, st_>>>(d);
    PDLP_LAUNCH_CHECK();
  }
}

template <class T, class M>
void Solve<T, M>::enable_snapshot() {
  if (snapshot_) return;
  Dev<T> &d = d_;
  size_t bytes = ((size_t)d.n * 2 + d.m) * sizeof(T) + 1024;
  void *mem = dev_alloc(bytes, st_);
  snap_mem_ = mem;
  d.bx = (T *)mem;
  d.bl = d.bx + d.n;
  d.by = d.bl + d.n;
  snapshot_ = true;
}

template <class T, class M>
double Solve<T, M>::primal_weight() const {
  Ctl c;
  read_ctl(c);
  return c.primal_weight;
}

template <class T, class M>
void Solve<T, M>::enqueue_iteration(int t, int off, bool timed) {
  Dev<T> &d = d_;
  IterFlags f = flags(t);
  const int par = t & 1;
  T *xc = d.x[par], *xn = d.x[par ^ 1];
  T *yc = d.y[par], *yn = d.y[par ^ 1];
  if (f.eval) enqueue_eval(off, f.infeas, f.restart_check, kEvalCheck);
  if (f.maybe_restart) {
    k_restart<T><<<d.ew_grid, kThreads, 0, st_>>>(d, xc, yc);
    k_restart_fin<T><<<1, kThreads, 0, st_>>>(d, off);
    PDLP_LAUNCH_CHECK();
  }
#define PDLP_STEPS_R(MAJ, FP, R1)                                           \
  {                                                                         \
    PrimalEpi<T, M, MAJ, FP, R1> pe{d, off, xc, yc, xn, T(0), T(0), T(0)};     \
    launch_spmv(AT_, pe, d.p_pstep, d.lp_pstep, st_);                       \
    DualEpi<T, M, MAJ, FP, R1> de{d, off, yc, yn, T(0), T(0), T(0), T(0)};     \
    launch_spmv(A_, de, d.p_dstep, d.lp_dstep, st_);                        \
  }
#define PDLP_STEPS(MAJ, FP)                                                 \
  {                                                                         \
    if (d.rho_is_one) PDLP_STEPS_R(MAJ, FP, true) else PDLP_STEPS_R(MAJ, FP, false) \
  }
  if (f.major_kernel) {
    if (f.fpe) PDLP_STEPS(true, true) else PDLP_STEPS(true, false)
  } else if (f.fpe) {
    PDLP_STEPS(false, true)
  } else if (timed) {
    // ordinary iteration sampled for the in-loop kernel timing; external
    // records become event-record nodes of the captured graph
    auto steps = [&](auto r1) {
      constexpr bool R1 = decltype(r1)::value;
      PrimalEpi<T, M, false, false, R1> pe{d, off, xc, yc, xn, T(0), T(0), T(0)};
      DualEpi<T, M, false, false, R1> de{d, off, yc, yn, T(0), T(0), T(0), T(0)};
      PDLP_CUDA(cudaEventRecordWithFlags(tev_[0][0], st_, cudaEventRecordExternal));
      launch_spmv(AT_, pe, d.p_pstep, d.lp_pstep, st_);
      PDLP_CUDA(cudaEventRecordWithFlags(tev_[0][1], st_, cudaEventRecordExternal));
      launch_spmv(A_, de, d.p_dstep, d.lp_dstep, st_);
      PDLP_CUDA(cudaEventRecordWithFlags(tev_[0][2], st_, cudaEventRecordExternal));
    };
    if (d.rho_is_one) steps(std::true_type{});
    else steps(std::false_type{});
  } else {
    PDLP_STEPS(false, false)
  }
#undef PDLP_STEPS
#undef PDLP_STEPS_R
  if (f.fpe) {
    if (f.fpe_restart_only) launch_spmv(AT_, FpeEpi<T, M, true>{d}, d.p_fpe, d.lp_fpe, st_);
    else launch_spmv(AT_, FpeEpi<T, M, false>{d}, d.p_fpe, d.lp_fpe, st_);
    k_fpe_fin<T><<<1, kThreads, 0, st_>>>(d, f.fpe_restart_only ? 1 : 0);
    PDLP_LAUNCH_CHECK();
  }
}

// kernels one iteration launches (early exits included)
static long iteration_launches(const IterFlags &f) {
  return 2 + (f.eval ? 3 + (f.infeas ? 4 : 0) : 0) + (f.maybe_restart ? 2 : 0) + (f.fpe ? 2 : 0);
}

template <class T, class M>
cudaGraphExec_t Solve<T, M>::chunk_graph(int t0, int t1) {
  std::string key;
  key.reserve((size_t)(t1 - t0) * 2 + 2);
  key += (char)('0' + (t0 & 1));
  for (int t = t0; t < t1; ++t) {
    IterFlags f = flags(t);
    key += (char)('A' + (f.eval) + 2 * f.infeas + 4 * f.restart_check + 8 * f.maybe_restart);
    key += (char)('A' + (f.major_kernel) + 2 * f.fpe + 4 * f.fpe_restart_only);
  }
  auto it = graphs_.find(key);
  if (it != graphs_.end()) return it->second;
  const int tt = timed_iteration(t0, t1);
  if (tt >= 0 && !tev_[0][0])
    for (auto &slot : tev_)
      for (auto &ev : slot) PDLP_CUDA(cudaEventCreate(&ev));
  cudaGraph_t g;
  cudaGraphExec_t e;
  PDLP_CUDA(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal));
  for (int t = t0; t < t1; ++t) enqueue_iteration(t, t - t0, t == tt);
  PDLP_CUDA(cudaStreamEndCapture(st_, &g));
  PDLP_CUDA(cudaGraphInstantiate(&e, g, 0));
  raw_graphs_.push_back(g);
  graphs_[key] = e;
  if (tt >= 0) {
    // the event-record nodes, identified by the event each one records
    size_t nn = 0;
    PDLP_CUDA(cudaGraphGetNodes(g, nullptr, &nn));
    std::vector<cudaGraphNode_t> nodes(nn);
    PDLP_CUDA(cudaGraphGetNodes(g, nodes.data(), &nn));
    std::array<cudaGraphNode_t, 3> tn{};
    int found = 0;
    for (cudaGraphNode_t nd : nodes) {
      cudaGraphNodeType ty;
      PDLP_CUDA(cudaGraphNodeGetType(nd, &ty));
      if (ty != cudaGraphNodeTypeEventRecord) continue;
      cudaEvent_t ev;
      PDLP_CUDA(cudaGraphEventRecordNodeGetEvent(nd, &ev));
      for (int i = 0; i < 3; ++i)
        if (ev == tev_[0][i]) {
          tn[i] = nd;
          ++found;
        }
    }
    if (found == 3) tnodes_[e] = tn;
  }
  return e;
}

// An ordinary iteration (no evaluation, restart, major or fixed-point-error
// kernels) in the second half of the chunk, or -1.
template <class T, class M>
int Solve<T, M>::timed_iteration(int t0, int t1) const {
  for (int t = t0 + (t1 - t0) / 2; t < t1; ++t) {
    IterFlags f = flags(t);
    if (!f.eval && !f.maybe_restart && !f.major_kernel && !f.fpe) return t;
  }
  return -1;
}

template <class T, class M>
void Solve<T, M>::read_timing(int slot) {
  if (tpending_[slot] < 0) return;
  float a = 0.f, b = 0.f;
  if (cudaEventElapsedTime(&a, tev_[slot][0], tev_[slot][1]) == cudaSuccess &&
      cudaEventElapsedTime(&b, tev_[slot][1], tev_[slot][2]) == cudaSuccess)
    tsamples_.push_back({tpending_[slot], a, b});
  else
    cudaGetLastError();
  tpending_[slot] = -1;
}

template <class T, class M>
double Solve<T, M>::live_primal_ms() const {
  double s = 0;
  int k = 0;
  for (const auto &x : tsamples_)
    if (x.t + 10 < final_count_) s += x.primal_ms, ++k;
  return k ? s / k : 0.0;
}

template <class T, class M>
double Solve<T, M>::live_dual_ms() const {
  double s = 0;
  int k = 0;
  for (const auto &x : tsamples_)
    if (x.t + 10 < final_count_) s += x.dual_ms, ++k;
  return k ? s / k : 0.0;
}

template <class T, class M>
int Solve<T, M>::live_samples() const {
  int k = 0;
  for (const auto &x : tsamples_) k += x.t + 10 < final_count_;
  return k;
}

template <class T, class M>
void Solve<T, M>::run() {
  Dev<T> &d = d_;
  const int L = p_.termination_criteria.iteration_limit;
  const int CH = 100;
  tune_kernels();
  auto t0 = std::chrono::steady_clock::now();
  k_loop_start<<<1, 1, 0, st_>>>(d.ctl);
  PDLP_LAUNCH_CHECK();
  launches_ += 1;
  cudaEvent_t ev[2];
  PDLP_CUDA(cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming));
  PDLP_CUDA(cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming));
  int t = 0, k = 0;
  while (t < L) {
    if (hflag_->done) break;
    int t1 = (int)std::min<long>((long)L, ((long)t / CH + 1) * CH);
    cudaGraphExec_t g = chunk_graph(t, t1);
    const int slot = k & 1;
    if (k >= 2) {
      PDLP_CUDA(cudaEventSynchronize(ev[slot]));
      read_timing(slot);  // chunk k-2 used this slot's events and has finished
    }
    if (hflag_->done) break;
    auto tn = tnodes_.find(g);
    if (tn != tnodes_.end()) {
      for (int i = 0; i < 3; ++i)
        PDLP_CUDA(cudaGraphExecEventRecordNodeSetEvent(g, tn->second[i], tev_[slot][i]));
      tpending_[slot] = timed_iteration(t, t1);
    }
    k_set_tbase<<<1, 1, 0, st_>>>(d.ctl, t);
    PDLP_LAUNCH_CHECK();
    PDLP_CUDA(cudaGraphLaunch(g, st_));
    PDLP_CUDA(cudaEventRecord(ev[k & 1], st_));
    for (int tt = t; tt < t1; ++tt) launches_ += iteration_launches(flags(tt));
    launches_ += 1;
    ++k;
    t = t1;
  }
  PDLP_CUDA(cudaStreamSynchronize(st_));
  read_timing(0);
  read_timing(1);
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
  if (!hflag_->done) {
    // iteration limit: one more evaluation at total_count = L (solver.cu:105-109)
    k_set_tbase<<<1, 1, 0, st_>>>(d.ctl, L);
    enqueue_eval(0, false, false, kEvalIterLimit);
    launches_ += 4;
    PDLP_CUDA(cudaStreamSynchronize(st_));
  }
  loop_sec_ = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  final_count_ = total_count();
  check_pipe_errors();
}

// A stage wait of the pipelined kernel that timed out leaves a flag (the
// kernel then stopped early, so the iterates are not to be trusted).
template <class T, class M>
void Solve<T, M>::check_pipe_errors() const {
  int e[2] = {0, 0};
  const int *flags[2] = {A64_.pipe.err, AT64_.pipe.err};
  for (int i = 0; i < 2; ++i)
    if (flags[i]) PDLP_CUDA(cudaMemcpyAsync(&e[i], flags[i], sizeof(int), cudaMemcpyDeviceToHost, st_));
  PDLP_CUDA(cudaStreamSynchronize(st_));
  if (e[0] || e[1])
    throw std::runtime_error("pipelined SpMV: a tile copy did not complete within its wait limit");
}

// finite entries -> 0 (the dual feasibility problem's bounds)
template <class T>
__global__ void k_zero_finite(long n, T *v) {
  long stride = (long)gridDim.x * blockDim.x;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += stride)
    if (isfinite((double)v[i])) v[i] = T(0);
}

template <class T, class M>
void Solve<T, M>::polish_init(const Solve &main, int mode) {
  Dev<T> &d = d_;
  const Dev<T> &md = main.d_;
  const int n = d.n, m = d.m;
  const int cur = main.final_count_ & 1;  // main's current iterate at termination
  auto copy = [&](T *dst, const T *src, int k) {
    if (k) PDLP_CUDA(cudaMemcpyAsync(dst, src, (size_t)k * sizeof(T), cudaMemcpyDeviceToDevice, st_));
  };
  auto zero = [&](T *p, int k) {
    if (k) PDLP_CUDA(cudaMemsetAsync(p, 0, (size_t)k * sizeof(T), st_));
  };
  d.polish = mode;
  if (mode == 1) {
    // objective 0 (and no objective constant, as the reference's polish state);
    // primal iterates from the solve, dual iterates 0
    zero((T *)d.c, n);
    d.c_obj = md.c;
    d.c0 = 0.0;
    copy(d.x0, md.x0, n);
    copy(d.x[0], md.x[cur], n);
    copy(d.xhat, md.xhat, n);
    copy(d.xref, md.xref, n);
    T *const ys[] = {d.y0, d.y[0], d.y[1], d.yhat};
    for (T *p : ys) zero(p, m);
    zero(d.lam, n);
  } else {
    // finite bounds 0; the dual objective keeps the solve's finite bounds and
    // primal point; dual iterates and dual slack from the solve, primal 0
    const int gn = grid_for(n), gm = grid_for(m);
    if (n) {
      k_zero_finite<T><<<gn, kThreads, 0, st_>>>(n, (T *)d.lv);
      k_zero_finite<T><<<gn, kThreads, 0, st_>>>(n, (T *)d.uv);
    }
    if (m) {
      k_zero_finite<T><<<gm, kThreads, 0, st_>>>(m, (T *)d.lc);
      k_zero_finite<T><<<gm, kThreads, 0, st_>>>(m, (T *)d.uc);
    }
    PDLP_LAUNCH_CHECK();
    launches_ += 4;
    d.lcf = md.lcf;
    d.ucf = md.ucf;
    d.x_obj = md.xhat;
    copy(d.y0, md.y0, m);
    copy(d.y[0], md.y[cur], m);
    copy(d.yhat, md.yhat, m);
    copy(d.lam, md.lam, n);
    T *const xs[] = {d.x0, d.x[0], d.x[1], d.xhat, d.xref};
    for (T *p : xs) zero(p, n);
  }
  Ctl c;
  read_ctl(c);
  c.fixed_point_error = c.initial_fixed_point_error = c.last_trial_fixed_point_error = INFINITY;
  c.pw_error_sum = c.pw_last_error = 0.0;
  c.best_gap = INFINITY;
  PDLP_CUDA(cudaMemcpyAsync(d.ctl, &c, sizeof(Ctl), cudaMemcpyHostToDevice, st_));
  PDLP_CUDA(cudaStreamSynchronize(st_));
}

template <class T, class M>
void Solve<T, M>::adopt_polish(const Solve &ps, int mode) {
  Dev<T> &d = d_;
  Ctl c, pc;
  read_ctl(c);
  ps.read_ctl(pc);
  if (mode == 1) {
    if (d.n)
      PDLP_CUDA(cudaMemcpyAsync(d.xhat, ps.d_.xhat, (size_t)d.n * sizeof(T),
                                cudaMemcpyDeviceToDevice, st_));
    c.abs_primal_res = pc.abs_primal_res;
    c.rel_primal_res = pc.rel_primal_res;
    c.primal_obj = pc.primal_obj;
  } else {
    if (d.m)
      PDLP_CUDA(cudaMemcpyAsync(d.yhat, ps.d_.yhat, (size_t)d.m * sizeof(T),
                                cudaMemcpyDeviceToDevice, st_));
    c.abs_dual_res = pc.abs_dual_res;
    c.rel_dual_res = pc.rel_dual_res;
    c.dual_obj = pc.dual_obj;
  }
  PDLP_CUDA(cudaMemcpyAsync(d.ctl, &c, sizeof(Ctl), cudaMemcpyHostToDevice, st_));
  PDLP_CUDA(cudaStreamSynchronize(st_));
}

template <class T, class M>
void Solve<T, M>::finish_polish() {
  Ctl c;
  read_ctl(c);
  c.gap = fabs(c.primal_obj - c.dual_obj);
  c.rel_gap = c.gap / (1.0 + fabs(c.primal_obj) + fabs(c.dual_obj));
  PDLP_CUDA(cudaMemcpyAsync(d_.ctl, &c, sizeof(Ctl), cudaMemcpyHostToDevice, st_));
  PDLP_CUDA(cudaStreamSynchronize(st_));
}

template <class T, class M>
Kkt Solve<T, M>::last_kkt() const {
  Ctl c;
  read_ctl(c);
  return Kkt{c.abs_primal_res, c.rel_primal_res, c.abs_dual_res, c.rel_dual_res,
             c.primal_obj,     c.dual_obj,       c.gap,          c.rel_gap};
}

template <class T, class M>
void Solve<T, M>::time_kernels(int reps, double *ms) {
  Dev<T> &d = d_;
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
  // the default reflection coefficient (1) selects the kernels of a solve
  PrimalEpi<T, M, false, false, true> pe{d, 0, d.x[0], d.y[0], d.x[1], T(0), T(0), T(0)};
  DualEpi<T, M, false, false, true> de{d, 0, d.y[0], d.y[1], T(0), T(0), T(0), T(0)};
  ms[0] = timed([&] { launch_spmv(AT_, pe, nullptr, nullptr, st_); });
  ms[1] = timed([&] { launch_spmv(A_, de, d.p_dstep, d.lp_dstep, st_); });
  ms[2] = timed([&] { launch_spmv(A64_, EvalAEpi<T, double, false>{d}, d.p_e1, d.lp_e1, st_); });
  ms[3] = timed([&] { launch_spmv(AT64_, EvalATEpi<T, double, false>{d}, d.p_e2, d.lp_e2, st_); });
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
}

template <class T, class M>
int Solve<T, M>::reason() const {
  Ctl c;
  read_ctl(c);
  return c.reason;
}

template <class T, class M>
int Solve<T, M>::total_count() const {
  Ctl c;
  read_ctl(c);
  return c.final_t;
}

template <class T, class M>
std::vector<double> Solve<T, M>::trace() const {
  Ctl c;
  read_ctl(c);
  std::vector<double> tr((size_t)c.trace_len * 10);
  if (c.trace_len)
    PDLP_CUDA(cudaMemcpyAsync(tr.data(), d_.trace, tr.size() * 8, cudaMemcpyDeviceToHost, st_));
    PDLP_CUDA(cudaStreamSynchronize(st_));
  return tr;
}

template <class T, class M>
void Solve<T, M>::result_device(double *x, double *y, double *lam) {
  Dev<T> d = d_;
  if (snapshot_) {  // the best evaluated iterate of the run
    Ctl c;
    PDLP_CUDA(cudaMemcpyAsync(&c, d.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st_));
    PDLP_CUDA(cudaStreamSynchronize(st_));
    if (c.snap_err < INFINITY) {
      d.xhat = d.bx;
      d.yhat = d.by;
      d.lam = d.bl;
    }
  }
  k_unscale<T><<<grid_for((long)d.n + d.m), kThreads, 0, st_>>>(d, x, y, lam);
  PDLP_LAUNCH_CHECK();
}

template <class T, class M>
Kkt Solve<T, M>::evaluate(const double *x, const double *y, const double *lam) {
  Dev<T> &d = d_;
  k_scale_point<T><<<grid_for((long)d.n + d.m), kThreads, 0, st_>>>(d, x, y, lam);
  PDLP_LAUNCH_CHECK();
  k_set_tbase<<<1, 1, 0, st_>>>(d.ctl, 0);
  enqueue_eval(0, false, false, kEvalOnly);
  Ctl c;
  PDLP_CUDA(cudaMemcpyAsync(&c, d.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st_));
  PDLP_CUDA(cudaStreamSynchronize(st_));
  return Kkt{c.abs_primal_res, c.rel_primal_res, c.abs_dual_res, c.rel_dual_res,
             c.primal_obj,     c.dual_obj,       c.gap,          c.rel_gap};
}

template <class T, class M>
cupdlpx_result_t *Solve<T, M>::result() {
  Dev<T> &d = d_;
  const int n = d.n, m = d.m;
  launch_spmv(AT_, ReducedCostEpi<T, M>{d, outl_}, nullptr, nullptr, st_);
  result_device(outx_, outy_, nullptr);
  launches_ += 2;
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
    PDLP_CUDA(cudaMemcpyAsync(r->primal_solution, outx_, (size_t)n * 8, cudaMemcpyDeviceToHost, st_));
    PDLP_CUDA(cudaMemcpyAsync(r->reduced_cost, outl_, (size_t)n * 8, cudaMemcpyDeviceToHost, st_));
  }
  if (m)
    PDLP_CUDA(cudaMemcpyAsync(r->dual_solution, outy_, (size_t)m * 8, cudaMemcpyDeviceToHost, st_));
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
