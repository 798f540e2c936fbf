// precond.cu -- diagonal rescaling of the LP on the GPU.
//
// Restates the reference's host preconditioner (src/preconditioner.c:89-273)
// as device sweeps over A (CSR) and A^T (CSR of the transpose):
//   Ruiz L-inf, l_inf_ruiz_iterations times: row maxima over A, column maxima
//     over A^T rows, r = sqrt(max) (1 where max < 1e-12), then
//     a_ij /= r_i * s_j, c /= s, bounds of x *= s, bounds of Ax /= r;
//   Pock-Chambolle: row sums of |a|^alpha over A, column sums of
//     |a|^(2-alpha) over A^T rows, sqrt, same scaling;
//   bound / objective rescaling: cb = 1/(|b| + 1), ob = 1/(|c| + 1).
// Maxima are order-free and every PC sum runs sequentially in the reference's
// accumulation order (row order of the CSR for rows, increasing row index for
// columns, which is the row order of A^T), so the scaled matrix, c, bounds
// and cumulative scalings are bit-identical to the host algorithm; only the
// two bound/objective norms are tree sums.
#include <math.h>

#include "solver.cuh"

namespace pdlp {

constexpr double kScalingEps = 1e-12;

// one warp per row: out[r] = transform(max_k |val_k|)
__global__ void k_row_absmax(int rows, const int *__restrict__ ptr,
                             const double *__restrict__ val, double *__restrict__ out) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int r = warp; r < rows; r += nwarps) {
    double mx = 0.0;
    for (int k = ptr[r] + lane; k < ptr[r + 1]; k += 32) mx = fmax(mx, fabs(val[k]));
    mx = warp_max(mx);
    if (lane == 0) out[r] = mx < kScalingEps ? 1.0 : sqrt(mx);
  }
}

__device__ __forceinline__ double pow_exact(double v, double e) {
  if (e == 1.0) return v;
  if (e == 2.0) return v * v;
  if (e == 0.0) return 1.0;
  return pow(v, e);
}

// one thread per row, sequential sum in row order
__global__ void k_row_powsum(int rows, const int *__restrict__ ptr,
                             const double *__restrict__ val, double e,
                             double *__restrict__ out) {
  long stride = (long)gridDim.x * blockDim.x;
  for (long r = blockIdx.x * (long)blockDim.x + threadIdx.x; r < rows; r += stride) {
    double s = 0.0;
    for (int k = ptr[r]; k < ptr[r + 1]; ++k) s += pow_exact(fabs(val[k]), e);
    out[r] = s < kScalingEps ? 1.0 : sqrt(s);
  }
}

// a_k /= rs[row] * cs[col]   (products commute exactly, so A and A^T agree)
__global__ void k_scale_rows(int rows, const int *__restrict__ ptr,
                             const int *__restrict__ col, double *__restrict__ val,
                             const double *__restrict__ rs, const double *__restrict__ cs) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int r = warp; r < rows; r += nwarps) {
    double a = rs[r];
    for (int k = ptr[r] + lane; k < ptr[r + 1]; k += 32) val[k] /= (a * cs[col[k]]);
  }
}

// vectors and cumulative scalings (preconditioner.c:91-99, :149-152)
__global__ void k_scale_vectors(int n, int m, double *c, double *lv, double *uv,
                                double *lc, double *uc, double *Dc, double *Dr,
                                const double *var, const double *con) {
  long stride = (long)gridDim.x * blockDim.x;
  for (long j = blockIdx.x * (long)blockDim.x + threadIdx.x; j < n; j += stride) {
    double s = var[j];
    c[j] /= s;
    uv[j] *= s;
    lv[j] *= s;
    Dc[j] *= s;
  }
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < m; i += stride) {
    double s = con[i];
    lc[i] /= s;
    uc[i] /= s;
    Dr[i] *= s;
  }
}

__global__ void k_fill(long n, double *p, double v) {
  long stride = (long)gridDim.x * blockDim.x;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += stride) p[i] = v;
}

// squared norms for the bound / objective rescaling (preconditioner.c:226-246)
__global__ void __launch_bounds__(kThreads)
    k_bound_obj_norms(int n, int m, const double *c, const double *lc, const double *uc,
                      double *part) {
  __shared__ double red[24];
  double a[2] = {0.0, 0.0};
  long stride = (long)gridDim.x * kThreads;
  for (long i = blockIdx.x * (long)kThreads + threadIdx.x; i < m; i += stride) {
    double lo = lc[i], up = uc[i];
    if (isfinite(lo) && lo != up) a[0] += lo * lo;
    if (isfinite(up)) a[0] += up * up;
  }
  for (long j = blockIdx.x * (long)kThreads + threadIdx.x; j < n; j += stride)
    a[1] += c[j] * c[j];
  block_reduce_fields<2, 0u>(a, red);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = a[0];
    part[gridDim.x + blockIdx.x] = a[1];
  }
}

__global__ void __launch_bounds__(kThreads) k_bound_obj_fin(int g, const double *part,
                                                            double *out) {
  __shared__ double sm[32];
  double b = block_fold<false>(part, g, sm);
  double o = block_fold<false>(part + g, g, sm);
  if (threadIdx.x == 0) {
    out[0] = 1.0 / (sqrt(b) + 1.0);
    out[1] = 1.0 / (sqrt(o) + 1.0);
  }
}

__global__ void k_scale_bounds_obj(int n, int m, double *c, double *lv, double *uv,
                                   double *lc, double *uc, const double *cbob) {
  double cb = cbob[0], ob = cbob[1];
  long stride = (long)gridDim.x * blockDim.x;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < m; i += stride) {
    lc[i] *= cb;
    uc[i] *= cb;
  }
  for (long j = blockIdx.x * (long)blockDim.x + threadIdx.x; j < n; j += stride) {
    lv[j] *= cb;
    uv[j] *= cb;
    c[j] *= ob;
  }
}

static int warp_grid(int rows) {
  long w = rows;  // one warp per row
  long b = (w * 32 + kThreads - 1) / kThreads;
  if (b < 1) b = 1;
  long cap = (long)kNumSms * 16;
  return (int)(b < cap ? b : cap);
}

void gpu_rescale(const pdhg_parameters_t &p, DevCsr &A, DevCsr &AT, double *c, double *lv,
                 double *uv, double *lc, double *uc, double *Dr, double *Dc, double *cb,
                 double *ob, double *tmp_n, double *tmp_m, double *part, cudaStream_t st,
                 double fixed_cb, double fixed_ob) {
  const int n = A.cols, m = A.rows;
  const int gv = grid_for((long)n + m);
  k_fill<<<grid_for(m), kThreads, 0, st>>>(m, Dr, 1.0);
  k_fill<<<grid_for(n), kThreads, 0, st>>>(n, Dc, 1.0);
  PDLP_LAUNCH_CHECK();
  auto apply = [&](double *con, double *var) {
    k_scale_vectors<<<gv, kThreads, 0, st>>>(n, m, c, lv, uv, lc, uc, Dc, Dr, var, con);
    if (m) k_scale_rows<<<warp_grid(m), kThreads, 0, st>>>(m, A.ptr, A.col, A.val, con, var);
    if (n) k_scale_rows<<<warp_grid(n), kThreads, 0, st>>>(n, AT.ptr, AT.col, AT.val, var, con);
    PDLP_LAUNCH_CHECK();
  };
  for (int it = 0; it < p.l_inf_ruiz_iterations; ++it) {
    if (m) k_row_absmax<<<warp_grid(m), kThreads, 0, st>>>(m, A.ptr, A.val, tmp_m);
    if (n) k_row_absmax<<<warp_grid(n), kThreads, 0, st>>>(n, AT.ptr, AT.val, tmp_n);
    PDLP_LAUNCH_CHECK();
    apply(tmp_m, tmp_n);
  }
  if (p.has_pock_chambolle_alpha) {
    double a = p.pock_chambolle_alpha;
    if (m) k_row_powsum<<<grid_for(m), kThreads, 0, st>>>(m, A.ptr, A.val, a, tmp_m);
    if (n) k_row_powsum<<<grid_for(n), kThreads, 0, st>>>(n, AT.ptr, AT.val, 2.0 - a, tmp_n);
    PDLP_LAUNCH_CHECK();
    apply(tmp_m, tmp_n);
  }
  if (fixed_cb > 0.0 && fixed_ob > 0.0) {
    // refinement rounds keep the first round's bound / objective scaling
    double h[2] = {fixed_cb, fixed_ob};
    double *out = part;
    PDLP_CUDA(cudaMemcpyAsync(out, h, sizeof(h), cudaMemcpyHostToDevice, st));
    k_scale_bounds_obj<<<gv, kThreads, 0, st>>>(n, m, c, lv, uv, lc, uc, out);
    PDLP_LAUNCH_CHECK();
    PDLP_CUDA(cudaStreamSynchronize(st));
    *cb = fixed_cb;
    *ob = fixed_ob;
  } else if (p.bound_objective_rescaling) {
    int g = grid_for((long)n + m);
    if (g > kMiscPart / 2 - 2) g = kMiscPart / 2 - 2;
    double *out = part + 2 * g;
    k_bound_obj_norms<<<g, kThreads, 0, st>>>(n, m, c, lc, uc, part);
    k_bound_obj_fin<<<1, kThreads, 0, st>>>(g, part, out);
    k_scale_bounds_obj<<<gv, kThreads, 0, st>>>(n, m, c, lv, uv, lc, uc, out);
    PDLP_LAUNCH_CHECK();
    double h[2];
    PDLP_CUDA(cudaMemcpyAsync(h, out, sizeof(h), cudaMemcpyDeviceToHost, st));
    PDLP_CUDA(cudaStreamSynchronize(st));
    *cb = h[0];
    *ob = h[1];
  } else {
    *cb = 1.0;
    *ob = 1.0;
  }
}

}  // namespace pdlp
