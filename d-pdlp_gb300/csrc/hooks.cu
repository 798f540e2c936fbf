// hooks.cu -- device-level and host entry points used by the parity tests
// (declared in include/pdlp_gb300.h).
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "pdlp_gb300.h"
#include "solver.cuh"

namespace pdlp {

// y[r] = sum_k a_rk x_k
struct PlainEpi {
  using val_t = double;
  using acc_t = double;
  static constexpr int NF = 0;
  static constexpr unsigned MAXMASK = 0;
  const double *x;
  double *y;
  __device__ bool init() { return true; }
  __device__ void prologue(double *) const {}
  __device__ void bind(const double *) {}
  __device__ double gather(int j) const { return x[j]; }
  __device__ void row(int r, double s, double *) const { y[r] = s; }
};

}  // namespace pdlp

extern "C" int pdlp_gpu_spmv_variant(int rows, int cols, const int *row_ptr,
                                     const int *col_ind, const double *vals, const double *x,
                                     double *y, int tile, int variant) {
  using namespace pdlp;
  if (rows < 0 || cols < 0 || !row_ptr || (tile != 512 && tile != 1024 && tile != 2048))
    return -1;
  if (variant < 0 || variant > 2 || (variant > 0 && tile != 1024)) return -1;
  const int nnz = row_ptr[rows];
  for (int r = 0; r < rows; ++r)
    if (row_ptr[r] > row_ptr[r + 1]) return -1;
  for (int k = 0; k < nnz; ++k)
    if (col_ind[k] < 0 || col_ind[k] >= cols) return -1;
  std::vector<int4> blk;
  std::vector<int2> lr;
  build_plan_host(rows, row_ptr, tile, blk, lr);
  void *mem = nullptr;
  try {
    size_t bytes = ((size_t)rows + 1) * 4 + (size_t)nnz * 12 + (size_t)cols * 8 +
                   (size_t)rows * 8 + blk.size() * 24 + lr.size() * 12 + 4096;
    PDLP_CUDA(cudaMalloc(&mem, bytes));
    char *p = (char *)mem;
    auto take = [&](size_t b) {
      char *q = p;
      p += (b + 255) & ~(size_t)255;
      return q;
    };
    int *dptr = (int *)take(((size_t)rows + 1) * 4);
    // variant 2: column and value arrays 4 and 8 bytes past a 16-byte boundary
    int *dcol = (int *)take((size_t)nnz * 4 + 4) + (variant == 2 ? 1 : 0);
    double *dval = (double *)take((size_t)nnz * 8 + 8) + (variant == 2 ? 1 : 0);
    double *dx = (double *)take((size_t)cols * 8 + 8);
    double *dy = (double *)take((size_t)rows * 8 + 8);
    SpmvPlan plan;
    plan.rows = rows;
    plan.nblk = (int)blk.size();
    plan.nlong = (int)lr.size();
    plan.tile = tile;
    plan.direct = variant > 0;
    plan.blk = (int4 *)take(blk.size() * 16 + 16);
    plan.lrow = (int2 *)take(lr.size() * 8 + 8);
    plan.lcnt = (unsigned *)take(lr.size() * 4 + 4);
    plan.lsum = (double *)take(blk.size() * 8 + 8);
    PDLP_CUDA(cudaMemcpy(dptr, row_ptr, ((size_t)rows + 1) * 4, cudaMemcpyHostToDevice));
    if (nnz) {
      PDLP_CUDA(cudaMemcpy(dcol, col_ind, (size_t)nnz * 4, cudaMemcpyHostToDevice));
      PDLP_CUDA(cudaMemcpy(dval, vals, (size_t)nnz * 8, cudaMemcpyHostToDevice));
    }
    if (cols) PDLP_CUDA(cudaMemcpy(dx, x, (size_t)cols * 8, cudaMemcpyHostToDevice));
    if (!blk.empty())
      PDLP_CUDA(cudaMemcpy(plan.blk, blk.data(), blk.size() * 16, cudaMemcpyHostToDevice));
    if (!lr.empty()) {
      PDLP_CUDA(cudaMemcpy(plan.lrow, lr.data(), lr.size() * 8, cudaMemcpyHostToDevice));
      PDLP_CUDA(cudaMemset(plan.lcnt, 0, lr.size() * 4));
    }
    PlainEpi e{dx, dy};
    if (plan.nblk > 0) {
      if (tile == 2048)
        spmv_fused<2048, PlainEpi><<<plan.nblk, kThreads>>>(dptr, dcol, dval, plan, nullptr,
                                                            nullptr, e);
      else if (tile == 1024 && plan.direct)
        spmv_fused<1024, PlainEpi, true><<<plan.nblk, kThreads>>>(dptr, dcol, dval, plan,
                                                                  nullptr, nullptr, e);
      else if (tile == 1024)
        spmv_fused<1024, PlainEpi><<<plan.nblk, kThreads>>>(dptr, dcol, dval, plan, nullptr,
                                                            nullptr, e);
      else
        spmv_fused<512, PlainEpi><<<plan.nblk, kThreads>>>(dptr, dcol, dval, plan, nullptr,
                                                           nullptr, e);
      PDLP_LAUNCH_CHECK();
    }
    if (rows) PDLP_CUDA(cudaMemcpy(y, dy, (size_t)rows * 8, cudaMemcpyDeviceToHost));
    cudaFree(mem);
    return 0;
  } catch (const std::exception &e) {
    if (mem) cudaFree(mem);
    fprintf(stderr, "[cupdlpx-gb300] pdlp_gpu_spmv: %s\n", e.what());
    return -2;
  }
}

extern "C" int pdlp_gpu_spmv(int rows, int cols, const int *row_ptr, const int *col_ind,
                             const double *vals, const double *x, double *y, int tile) {
  if (tile != 512 && tile != 2048) return -1;
  return pdlp_gpu_spmv_variant(rows, cols, row_ptr, col_ind, vals, x, y, tile, 0);
}

extern "C" int pdlp_host_transpose(int m, int n, const int *row_ptr, const int *col_ind,
                                   const double *vals, int *t_row_ptr, int *t_col_ind,
                                   double *t_vals) {
  if (m < 0 || n < 0 || !row_ptr || !t_row_ptr || row_ptr[0] != 0) return -1;
  for (int r = 0; r < m; ++r)
    if (row_ptr[r] > row_ptr[r + 1]) return -1;
  const int nnz = row_ptr[m];
  if (nnz > 0 && (!col_ind || !vals || !t_col_ind || !t_vals)) return -1;
  for (int k = 0; k < nnz; ++k)
    if (col_ind[k] < 0 || col_ind[k] >= n) return -1;
  std::vector<int> tp;
  pdlp::host_buf<int> tj;
  pdlp::host_buf<double> tx;
  pdlp::host_transpose(m, n, row_ptr, col_ind, vals, tp, tj, tx);
  memcpy(t_row_ptr, tp.data(), sizeof(int) * ((size_t)n + 1));
  if (nnz) {
    memcpy(t_col_ind, tj.data(), sizeof(int) * (size_t)nnz);
    memcpy(t_vals, tx.data(), sizeof(double) * (size_t)nnz);
  }
  return 0;
}

extern "C" int pdlp_gpu_transpose(int m, int n, const int *row_ptr, const int *col_ind,
                                  const double *vals, int *t_row_ptr, int *t_col_ind,
                                  double *t_vals) {
  if (m < 0 || n < 0 || !row_ptr || !t_row_ptr || row_ptr[0] != 0) return -1;
  for (int r = 0; r < m; ++r)
    if (row_ptr[r] > row_ptr[r + 1]) return -1;
  const int nnz = row_ptr[m];
  if (nnz > 0 && (!col_ind || !vals || !t_col_ind || !t_vals)) return -1;
  for (int k = 0; k < nnz; ++k)
    if (col_ind[k] < 0 || col_ind[k] >= n) return -1;
  try {
    using namespace pdlp;
    const size_t nz = (size_t)nnz;
    auto a256 = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t bytes = a256(((size_t)m + 1) * 4) + a256(nz * 4) + a256(nz * 8) +
                         a256(((size_t)n + 1) * 4) + a256(nz * 4) + a256(nz * 8);
    struct Free {
      void *p = nullptr;
      ~Free() {
        if (p) cudaFree(p);
      }
    } mem, scr;
    PDLP_CUDA(cudaMalloc(&mem.p, bytes));
    PDLP_CUDA(cudaMalloc(&scr.p, device_transpose_scratch_bytes(n, nnz)));
    char *p = (char *)mem.p;
    int *dptr = (int *)p; p += a256(((size_t)m + 1) * 4);
    int *dcol = (int *)p; p += a256(nz * 4);
    double *dval = (double *)p; p += a256(nz * 8);
    int *tptr = (int *)p; p += a256(((size_t)n + 1) * 4);
    int *tcol = (int *)p; p += a256(nz * 4);
    double *tval = (double *)p;
    PDLP_CUDA(cudaMemcpy(dptr, row_ptr, ((size_t)m + 1) * 4, cudaMemcpyHostToDevice));
    if (nnz) {
      PDLP_CUDA(cudaMemcpy(dcol, col_ind, nz * 4, cudaMemcpyHostToDevice));
      PDLP_CUDA(cudaMemcpy(dval, vals, nz * 8, cudaMemcpyHostToDevice));
    }
    device_transpose(m, n, nnz, dptr, dcol, dval, tptr, tcol, tval, scr.p, 0);
    PDLP_CUDA(cudaMemcpy(t_row_ptr, tptr, ((size_t)n + 1) * 4, cudaMemcpyDeviceToHost));
    if (nnz) {
      PDLP_CUDA(cudaMemcpy(t_col_ind, tcol, nz * 4, cudaMemcpyDeviceToHost));
      PDLP_CUDA(cudaMemcpy(t_vals, tval, nz * 8, cudaMemcpyDeviceToHost));
    }
    return 0;
  } catch (const std::exception &e) {
    fprintf(stderr, "[cupdlpx-gb300] pdlp_gpu_transpose: %s\n", e.what());
    cudaGetLastError();
    return -2;
  }
}

extern "C" int pdlp_spmv_plan(int rows, const int *row_ptr, int tile, int chunk, int *blocks,
                              int cap, int *nblk, int *nlong, int *direct) {
  using namespace pdlp;
  if (rows < 0 || !row_ptr || !nblk || !nlong || !direct) return -1;
  if (tile != 512 && tile != 1024 && tile != 2048) return -1;
  if (row_ptr[0] != 0) return -1;
  for (int r = 0; r < rows; ++r)
    if (row_ptr[r] > row_ptr[r + 1]) return -1;
  if (chunk <= 0) chunk = tile * 8 < 8192 ? tile * 8 : 8192;
  std::vector<int4> blk;
  std::vector<int2> lr;
  build_plan_host(rows, row_ptr, tile, blk, lr, chunk);
  *nblk = (int)blk.size();
  *nlong = (int)lr.size();
  *direct = tile == 1024 && plan_direct(blk, row_ptr[rows]);
  if (blocks)
    for (int i = 0; i < (int)blk.size() && i < cap; ++i) {
      blocks[4 * i] = blk[i].x;
      blocks[4 * i + 1] = blk[i].y;
      blocks[4 * i + 2] = blk[i].z;
      blocks[4 * i + 3] = blk[i].w;
    }
  return 0;
}

extern "C" int pdlp_spmv_pipe_plan(int rows, const int *row_ptr, int nv, int *tiles, int *bytes,
                                   int cap, int *ntile, int *nlong, int *limits) {
  using namespace pdlp;
  if (rows < 0 || !row_ptr || !ntile || !nlong || nv < 0) return -1;
  if (row_ptr[0] != 0) return -1;
  for (int r = 0; r < rows; ++r)
    if (row_ptr[r] > row_ptr[r + 1]) return -1;
  std::vector<int4> blk;
  std::vector<int2> lr;
  build_pipe_plan_host(rows, row_ptr, nv, blk, lr);
  *ntile = (int)blk.size();
  *nlong = (int)lr.size();
  if (limits) {
    limits[0] = kPipeRows;
    limits[1] = kPipeTile;
    limits[2] = kPipeMedRows;
    limits[3] = kPipeTileBytes;
  }
  for (int i = 0; i < (int)blk.size() && i < cap; ++i) {
    if (tiles) {
      tiles[4 * i] = blk[i].x;
      tiles[4 * i + 1] = blk[i].y;
      tiles[4 * i + 2] = blk[i].z;
      tiles[4 * i + 3] = blk[i].w;
    }
    if (bytes) bytes[i] = pipe_tile_bytes(blk[i], nv);
  }
  return 0;
}
