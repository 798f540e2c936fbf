// iter_kernels.cuh -- device code of the PDHG iteration: SpMV epilogues,
// element kernels and the single-block finalisers that hold the driver's
// scalar logic (termination, restart, primal-weight PID, fixed-point error).
//
// Every kernel is templated on T (double: FP64 path, float: FP32 path).  The
// per-element PDHG arithmetic runs in T; residuals, objective terms and every
// reduction run in FP64.
#pragma once

#include <math.h>

#include "solver.cuh"
#include "spmv_pipe.cuh"

namespace pdlp {

// Epilogues without per-block scalars.
#define PDLP_NO_BLOCK_SCALARS                 \
  __device__ void prologue(double *) const {} \
  __device__ void bind(const double *) {}

// Halpern weight w = (k+1)/(k+2), k = inner iteration count
// (reference pdlp_core_op.cu:559-567), once per block: from the solve's table
// (the same quotients, computed once) or, past its end, by division.
__device__ __forceinline__ void halpern_weight(const Ctl *c, const double *hw, int hw_len,
                                               int off, double *sc) {
  int k = c->t_base + off - c->restart_t;
  double w = (k >= 0 && k < hw_len) ? hw[k] : (double)(k + 1) / (double)(k + 2);
  sc[0] = w;
  sc[1] = 1.0 - w;
}

// primal step: x_hat = proj(x - tau (c - A^T y)), x_ref = 2 x_hat - x, Halpern
// (reference pdlp_core_op.cu:393-418, :445-462, :495-526).  RHO1: the
// reflection coefficient is 1 (the default), so the reflected point is x_ref
// itself.
template <class T, class M, bool MAJOR, bool FPE, bool RHO1>
struct PrimalEpi {
  using val_t = M;
  using acc_t = M;
  static constexpr int NF = FPE ? 1 : 0;
  static constexpr unsigned MAXMASK = 0;
  Dev<T> d;
  int off;
  const T *xcur, *ycur;
  T *xnext;
  T tau, w, omw;
  __device__ bool init() {
    const Ctl *c = d.ctl;
    if (c->done) return false;
    tau = (T)c->tau;
    return true;
  }
  __device__ void prologue(double *sc) const { halpern_weight(d.ctl, d.hw, d.hw_len, off, sc); }
  __device__ void bind(const double *sc) {
    w = (T)sc[0];
    omw = (T)sc[1];
  }
  __device__ M gather(int i) const { return (M)ycur[i]; }
  struct Pre {
    T xc, c, lv, uv, x0;
  };
  // per-row vectors of the pipelined kernel, in Pre order
  using vec_t = T;
  static constexpr int NV = 5;
  __device__ void vecs(const T *(&v)[NV]) const {
    v[0] = xcur;
    v[1] = d.c;
    v[2] = d.lv;
    v[3] = d.uv;
    v[4] = d.x0;
  }
  __device__ Pre make_pre(const T (&v)[NV]) const { return Pre{v[0], v[1], v[2], v[3], v[4]}; }
  __device__ void preload(int j, Pre &p) const {
    p.xc = xcur[j];
    p.c = d.c[j];
    p.lv = d.lv[j];
    p.uv = d.uv[j];
    p.x0 = d.x0[j];
  }
  __device__ void row(int j, M sm, double *acc) const {
    Pre p;
    preload(j, p);
    row_pre(j, sm, p, acc);
  }
  __device__ void row_pre(int j, M sm, const Pre &p, double *acc) const {
    T s = (T)sm;
    T xc = p.xc;
    T t = xc - tau * (p.c - s);
    T xh = clamp_to(t, p.lv, p.uv);
    if (MAJOR) {
      d.xhat[j] = xh;
      d.lam[j] = (xh - t) / tau;
    }
    T xr = T(2) * xh - xc;
    d.xref[j] = xr;
    if (FPE) {
      T dd = xr - xc;
      d.dx[j] = dd;
      acc[0] += (double)dd * (double)dd;
    }
    T refl = RHO1 ? xr : (T)d.rho * xr + (T)d.one_minus_rho * xc;
    xnext[j] = w * refl + omw * p.x0;
  }
};

// dual step: t = y/sigma - A x_ref, y_hat = sigma (t - proj(t)), Halpern
// (reference pdlp_core_op.cu:420-443, :528-557)
template <class T, class M, bool MAJOR, bool FPE, bool RHO1>
struct DualEpi {
  using val_t = M;
  using acc_t = M;
  static constexpr int NF = FPE ? 1 : 0;
  static constexpr unsigned MAXMASK = 0;
  Dev<T> d;
  int off;
  const T *ycur;
  T *ynext;
  T sigma, inv_sigma, w, omw;
  __device__ bool init() {
    const Ctl *c = d.ctl;
    if (c->done) return false;
    sigma = (T)c->sigma;
    inv_sigma = (T)c->inv_sigma;
    return true;
  }
  __device__ void prologue(double *sc) const { halpern_weight(d.ctl, d.hw, d.hw_len, off, sc); }
  __device__ void bind(const double *sc) {
    w = (T)sc[0];
    omw = (T)sc[1];
  }
  __device__ M gather(int j) const { return (M)d.xref[j]; }
  struct Pre {
    T yc, lc, uc, y0;
  };
  using vec_t = T;
  static constexpr int NV = 4;
  __device__ void vecs(const T *(&v)[NV]) const {
    v[0] = ycur;
    v[1] = d.lc;
    v[2] = d.uc;
    v[3] = d.y0;
  }
  __device__ Pre make_pre(const T (&v)[NV]) const { return Pre{v[0], v[1], v[2], v[3]}; }
  __device__ void preload(int i, Pre &p) const {
    p.yc = ycur[i];
    p.lc = d.lc[i];
    p.uc = d.uc[i];
    p.y0 = d.y0[i];
  }
  __device__ void row(int i, M sm, double *acc) const {
    Pre p;
    preload(i, p);
    row_pre(i, sm, p, acc);
  }
  __device__ void row_pre(int i, M sm, const Pre &p, double *acc) const {
    T s = (T)sm;
    T yc = p.yc;
    // the reference divides by sigma; one reciprocal per launch instead
    // (at most 1 ulp apart; an FP64 division costs ~10 FP64 issue slots)
    T t = yc * inv_sigma - s;
    T tp = clamp_to(t, -p.uc, -p.lc);
    T yh = (t - tp) * sigma;
    if (MAJOR) d.yhat[i] = yh;
    T yr = T(2) * yh - yc;
    if (FPE) {
      T dd = yr - yc;
      d.dy[i] = dd;
      acc[0] += (double)dd * (double)dd;
    }
    T refl = RHO1 ? yr : (T)d.rho * yr + (T)d.one_minus_rho * yc;
    ynext[i] = w * refl + omw * p.y0;
  }
};

// cross term <A^T dy, dx> of the fixed-point error (pdlp_core_op.cu:658-696)
template <class T, class M, bool RESTART_ONLY>
struct FpeEpi {
  using val_t = M;
  using acc_t = M;
  static constexpr int NF = 1;
  static constexpr unsigned MAXMASK = 0;
  Dev<T> d;
  PDLP_NO_BLOCK_SCALARS
  __device__ bool init() {
    if (d.ctl->done) return false;
    if (RESTART_ONLY && !d.ctl->do_restart) return false;
    return true;
  }
  __device__ M gather(int i) const { return (M)d.dy[i]; }
  __device__ void row(int j, M s, double *acc) const { acc[0] += (double)s * (double)d.dx[j]; }
};

// KKT over A x_hat (utils.cu:503-531 constraint half), FP64 terms
template <class T, class M, bool LINF>
struct EvalAEpi {
  using val_t = M;
  using acc_t = M;
  static constexpr int NF = 2;
  static constexpr unsigned MAXMASK = LINF ? 1u : 0u;
  Dev<T> d;
  PDLP_NO_BLOCK_SCALARS
  __device__ bool init() { return !d.ctl->done; }
  __device__ M gather(int j) const { return (M)d.xhat[j]; }
  __device__ void row(int i, M s, double *acc) const {
    double sd = s;
    double cl = fmax((double)d.lc[i], fmin(sd, (double)d.uc[i]));
    double pr = (sd - cl) * d.Dr[i];
    acc[0] = LINF ? fmax(acc[0], fabs(pr)) : acc[0] + pr * pr;
    if (d.shifted) {  // original-units dual at the centre plus the correction
      double yo = d.sy[i] + (double)d.yhat[i] / (d.Dr[i] * d.ob) * d.sdd_inv;
      acc[1] += fmax(yo, 0.0) * d.olcf[i] + fmin(yo, 0.0) * d.oucf[i];
    } else {
      double yh = d.yhat[i];
      acc[1] += fmax(yh, 0.0) * (double)d.lcf[i] + fmin(yh, 0.0) * (double)d.ucf[i];
    }
  }
};

// KKT over A^T y_hat (utils.cu:503-531 variable half, plus objective dots)
template <class T, class M, bool LINF>
struct EvalATEpi {
  using val_t = M;
  using acc_t = M;
  static constexpr int NF = 3;
  static constexpr unsigned MAXMASK = LINF ? 1u : 0u;
  Dev<T> d;
  PDLP_NO_BLOCK_SCALARS
  __device__ bool init() { return !d.ctl->done; }
  __device__ M gather(int i) const { return (M)d.yhat[i]; }
  __device__ void row(int j, M s, double *acc) const {
    double lam = d.lam[j], c = d.c[j];
    double dr = (c - (double)s - lam) * d.Dc[j];
    acc[0] = LINF ? fmax(acc[0], fabs(dr)) : acc[0] + dr * dr;
    if (d.shifted) {  // original objective at the centre plus the correction
      double xo = d.sx[j] + (double)d.xhat[j] / (d.Dc[j] * d.cb) * d.sdp_inv;
      acc[1] += d.oc[j] * xo;
      acc[2] += lam * d.Dc[j] / d.ob * d.sdd_inv * xo;
    } else {
      double xh = d.xhat[j];
      acc[1] += (double)d.c_obj[j] * xh;
      acc[2] += lam * (double)d.x_obj[j];
    }
  }
};

__device__ __forceinline__ double ray_scale(const Ctl *c) {
  double p = c->ray_primal_inf_norm;
  return p > 0.0 ? 1.0 / p : 1.0;
}

// primal ray over A (utils.cu:561-572, :588-600)
template <class T, class M>
struct InfAEpi {
  using val_t = M;
  using acc_t = M;
  static constexpr int NF = 2;
  static constexpr unsigned MAXMASK = 1u;
  Dev<T> d;
  T sc;
  PDLP_NO_BLOCK_SCALARS
  __device__ bool init() {  // runs twice per solve: a per-thread division is fine
    if (d.ctl->done) return false;
    sc = (T)ray_scale(d.ctl);
    return true;
  }
  __device__ M gather(int j) const { return (M)(sc * d.dx[j]); }
  __device__ void row(int i, M s, double *acc) const {
    double sd = s;
    double pi = (fmax(0.0, -sd) * (double)isfinite(d.lc[i]) +
                 fmax(0.0, sd) * (double)isfinite(d.uc[i])) * d.Dr[i];
    acc[0] = fmax(acc[0], fabs(pi));
    double dy = d.dy[i];
    acc[1] += fmax(dy, 0.0) * (double)d.lcf[i] + fmin(dy, 0.0) * (double)d.ucf[i];
  }
};

// dual ray over A^T (utils.cu:574-586, :602-614; the slack slot holds A^T dy
// as in the reference call at utils.cu:772-776)
template <class T, class M>
struct InfATEpi {
  using val_t = M;
  using acc_t = M;
  static constexpr int NF = 3;
  static constexpr unsigned MAXMASK = 2u;
  Dev<T> d;
  T sc;
  PDLP_NO_BLOCK_SCALARS
  __device__ bool init() {
    if (d.ctl->done) return false;
    sc = (T)ray_scale(d.ctl);
    return true;
  }
  __device__ M gather(int i) const { return (M)d.dy[i]; }
  __device__ void row(int j, M s, double *acc) const {
    double ns = -(double)s;
    acc[0] += fmax(ns, 0.0) * (double)d.lvf[j] + fmin(ns, 0.0) * (double)d.uvf[j];
    double di = (fmax(0.0, ns) * (double)!isfinite(d.lv[j]) -
                 fmin(0.0, ns) * (double)!isfinite(d.uv[j])) * d.Dc[j];
    acc[1] = fmax(acc[1], fabs(di));
    acc[2] += (double)d.c[j] * (double)(sc * d.dx[j]);
  }
};

// reduced cost (pdlp_core_op.cu:31-40), FP64 output in original units
template <class T, class M>
struct ReducedCostEpi {
  using val_t = M;
  using acc_t = M;
  static constexpr int NF = 0;
  static constexpr unsigned MAXMASK = 0;
  Dev<T> d;
  double *out;
  PDLP_NO_BLOCK_SCALARS
  __device__ bool init() { return true; }
  __device__ M gather(int i) const { return (M)d.yhat[i]; }
  __device__ void row(int j, M s, double *) const {
    out[j] = ((double)d.c[j] - (double)s) * d.Dc[j] / d.ob;
  }
};

// power method: g = A^T (inv * v)   (utils.cu:127-136)
struct PowAtEpi {
  using val_t = double;
  using acc_t = double;
  static constexpr int NF = 0;
  static constexpr unsigned MAXMASK = 0;
  PowDev d;
  const double *v;
  double inv;
  PDLP_NO_BLOCK_SCALARS
  __device__ bool init() {
    if (d.ctl->pm_done) return false;
    inv = d.ctl->pm_inv_norm;
    return true;
  }
  __device__ double gather(int i) const { return inv * v[i]; }
  __device__ void row(int j, double s, double *) const { d.g[j] = s; }
};

// power method: v' = A g, sum q.v', sum v'^2   (utils.cu:138-144)
struct PowAEpi {
  using val_t = double;
  using acc_t = double;
  static constexpr int NF = 2;
  static constexpr unsigned MAXMASK = 0;
  PowDev d;
  const double *v;
  double *vnext;
  double inv;
  PDLP_NO_BLOCK_SCALARS
  __device__ bool init() {
    if (d.ctl->pm_done) return false;
    inv = d.ctl->pm_inv_norm;
    return true;
  }
  __device__ double gather(int j) const { return d.g[j]; }
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

// Each matrix of a solve runs every SpMV on one of the two kernels: the
// pipelined one (M.pipe_on) or the fused one.  The choice is made per matrix
// by timing both on the step epilogue (Solve::tune_kernels), or forced by
// PDLP_STEP_KERNEL=pipe / fused; reduction partials are sized for either
// and folded with the counts of the kernel in use.
// 1: forced pipelined, 0: forced fused, -1: measured per matrix
int kernel_override();

template <class V>
inline bool use_pipe(const DevCsrT<V> &M) {
  return M.pipe_on && M.pipe.ntile > 0;
}
template <class V>
inline size_t spmv_partials(const DevCsrT<V> &M) {
  return use_pipe(M) ? (size_t)M.pipe.grid : (size_t)M.plan.nblk;
}
template <class V>
inline size_t spmv_long_rows(const DevCsrT<V> &M) {
  return use_pipe(M) ? (size_t)M.pipe.nlong : (size_t)M.plan.nlong;
}
// partial buffers large enough for either kernel
template <class V>
inline size_t spmv_partials_max(const DevCsrT<V> &M) {
  return (size_t)(M.pipe.grid > M.plan.nblk ? M.pipe.grid : M.plan.nblk);
}
template <class V>
inline size_t spmv_long_rows_max(const DevCsrT<V> &M) {
  return (size_t)(M.pipe.nlong > M.plan.nlong ? M.pipe.nlong : M.plan.nlong);
}

template <class Epi>
void set_pipe_smem() {
  static const cudaError_t e = cudaFuncSetAttribute(
      spmv_pipe<Epi>, cudaFuncAttributeMaxDynamicSharedMemorySize, kPipeSmem);
  PDLP_CUDA(e);
}

template <class Epi, class V>
void launch_spmv(const DevCsrT<V> &M, const Epi &epi, double *part, double *lpart,
                 cudaStream_t st) {
  if (use_pipe(M)) {
    set_pipe_smem<Epi>();
    spmv_pipe<Epi><<<M.pipe.grid, kPipeBlock, kPipeSmem, st>>>(M.ptr, M.col, M.val, M.pipe,
                                                                 part, lpart, epi);
    PDLP_LAUNCH_CHECK();
    return;
  }
  if (M.plan.nblk == 0) return;
  if (M.plan.tile == 2048)
    spmv_fused<2048, Epi><<<M.plan.nblk, kThreads, 0, st>>>(M.ptr, M.col, M.val, M.plan,
                                                             part, lpart, epi);
  else if (M.plan.tile == 1024 && M.plan.direct)
    spmv_fused<1024, Epi, true><<<M.plan.nblk, kThreads, 0, st>>>(M.ptr, M.col, M.val, M.plan,
                                                                   part, lpart, epi);
  else if (M.plan.tile == 1024)
    spmv_fused<1024, Epi><<<M.plan.nblk, kThreads, 0, st>>>(M.ptr, M.col, M.val, M.plan,
                                                             part, lpart, epi);
  else
    spmv_fused<512, Epi><<<M.plan.nblk, kThreads, 0, st>>>(M.ptr, M.col, M.val, M.plan,
                                                            part, lpart, epi);
  PDLP_LAUNCH_CHECK();
}

}  // namespace pdlp
