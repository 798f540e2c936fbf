// noalloc.cu -- y = A x on caller-owned device buffers, allocating nothing.
//
// Some callers cannot let a library allocate device memory: a host
// application that hands all of HBM to its own pool allocator at start-up
// (a further cudaMalloc fails or breaks its accounting), or code that must
// not take the device-wide synchronisation that cudaMalloc / cudaFree imply
// in the middle of a latency-critical loop.
// pdlp_spmv_noalloc serves them: the caller passes the CSR matrix and the
// vectors already in device memory, and the only scratch the product needs
// (per-tile partial sums of rows that cross tile boundaries, and an error
// flag) lives in the file-scope device array below, which every GPU that
// loads this library holds until the process exits.
//
// It is a variant of the fused SpMV of the solver: tiles of kTile non-zeros
// staged with coalesced loads, the rows starting in a tile folded from shared
// memory; tiles are cut at fixed non-zero offsets, so no row plan has to be
// built or stored.  A row that continues past its tile leaves one partial per
// tile in the scratch array, and a second kernel adds them in tile order, so
// the result is bitwise reproducible.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <mutex>
#include <string>

#include "common.cuh"
#include "pdlp_gb300.h"

namespace {

constexpr int kTile = 2048;  // non-zeros per thread block
constexpr int kMaxTiles = PDLP_NOALLOC_MAX_TILES;

// Scratch of every call: own[t] (partial of the row that starts in tile t and
// runs past it), in[t] (partial of the row that reached tile t from an
// earlier tile), own_row[t] (that row, or -1), and the error flag.
struct Scratch {
  double own[kMaxTiles];
  double in[kMaxTiles];
  int own_row[kMaxTiles];
  int error;
};

static __device__ __align__(256) Scratch g_scratch;

__device__ __forceinline__ int lower_bound_rows(const int *ptr, int rows, int key) {
  int lo = 0, hi = rows;  // first r in [0, rows) with ptr[r] >= key, else rows
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (ptr[mid] < key) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

__global__ void __launch_bounds__(pdlp::kThreads)
    k_spmv_tiles(int rows, int cols, int nnz, int ntiles, const int *__restrict__ ptr,
                 const int *__restrict__ col, const double *__restrict__ val,
                 const double *__restrict__ x, double *__restrict__ y, Scratch *s) {
  __shared__ double sv[kTile];
  __shared__ double sx[kTile];
  __shared__ int s_rows[2];
  const int t = blockIdx.x;
  const int k0 = t * kTile;
  const int k1 = min(nnz, k0 + kTile);
  const int len = k1 > k0 ? k1 - k0 : 0;
  // row pointers are validated over all rows (grid-stride), so a malformed
  // CSR always raises the flag; every access below stays in bounds either way
  for (long r = (long)t * pdlp::kThreads + threadIdx.x; r < rows;
       r += (long)ntiles * pdlp::kThreads)
    if (ptr[r] > ptr[r + 1]) atomicOr(&s->error, 1);
  if (threadIdx.x == 0) {
    if (t == 0 && (ptr[0] != 0 || ptr[rows] != nnz)) atomicOr(&s->error, 1);
    s_rows[0] = t == 0 ? 0 : lower_bound_rows(ptr, rows, k0);
    s_rows[1] = t == ntiles - 1 ? rows : lower_bound_rows(ptr, rows, k1);
    s->own_row[t] = -1;  // set below by the row that runs past k1, if any
  }
  for (int i = threadIdx.x; i < len; i += pdlp::kThreads) {
    int c = col[k0 + i];
    double xv = 0.0;
    if (c >= 0 && c < cols) xv = x[c];
    else atomicOr(&s->error, 2);  // bad column: flagged, never dereferenced
    sv[i] = val[k0 + i];
    sx[i] = xv;
  }
  __syncthreads();
  const int rA = s_rows[0], rB = s_rows[1];
  // rows starting in this tile; the one running past k1 leaves its partial
  for (int r = rA + threadIdx.x; r < rB; r += pdlp::kThreads) {
    int a = ptr[r], e = ptr[r + 1];
    if (a > e || a < 0 || e > nnz) continue;  // flagged by the validation loop
    int lo = max(a, k0) - k0, hi = min(e, k1) - k0;
    double sum = 0.0;
    for (int i = lo; i < hi; ++i) sum = fma(sv[i], sx[i], sum);
    if (e > k1) {
      s->own[t] = sum;
      s->own_row[t] = r;
    } else {
      y[r] = sum;
    }
  }
  // partial of the row (started in an earlier tile) that runs into this one
  if (threadIdx.x == 0) {
    double inc = 0.0;
    if (t > 0 && rA > 0) {
      int end = min(ptr[rA], k1);  // row rA-1 ends where row rA starts
      for (int i = 0; i < end - k0; ++i) inc = fma(sv[i], sx[i], inc);
    }
    s->in[t] = inc;
  }
}

// y[r] for a row crossing tiles: its own partial plus the partials of the
// tiles it runs into, added in tile order
__global__ void k_spmv_tiles_fix(int ntiles, const int *__restrict__ ptr, double *__restrict__ y,
                                 const Scratch *__restrict__ s) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntiles) return;
  int r = s->own_row[t];
  if (r < 0) return;
  double tot = s->own[t];
  int end = ptr[r + 1];
  for (int u = t + 1; u < ntiles && (long)u * kTile < end; ++u) tot += s->in[u];
  y[r] = tot;
}

// Device address of the scratch array, per device.  Only a successful
// lookup is kept: a lookup that failed (say, before the device could be
// used) is tried again by the next call.
constexpr int kMaxDevices = 64;
Scratch *g_addr[kMaxDevices] = {};
std::mutex g_addr_mu;

thread_local std::string g_err;

int fail(int code, const std::string &msg) {
  g_err = msg;
  fprintf(stderr, "[cupdlpx-gb300] pdlp_spmv_noalloc: %s\n", msg.c_str());
  return code;
}

}  // namespace

extern "C" const char *pdlp_spmv_noalloc_error(void) { return g_err.c_str(); }

extern "C" int pdlp_spmv_noalloc(int rows, int cols, int nnz, const int *row_ptr,
                                 const int *col_ind, const double *vals, const double *x,
                                 double *y, void *stream) {
  if (rows < 0 || cols < 0 || nnz < 0)
    return fail(-1, "negative size");
  const long ntiles_l = nnz > 0 ? ((long)nnz + kTile - 1) / kTile : 1;
  if (ntiles_l > kMaxTiles)
    return fail(-3, "nnz " + std::to_string(nnz) + " exceeds the maximum of " +
                        std::to_string((long)kMaxTiles * kTile) +
                        " non-zeros (PDLP_NOALLOC_MAX_TILES tiles of 2048)");
  if (rows == 0) {
    if (nnz > 0) return fail(-1, "non-zeros given for a matrix without rows");
    return 0;
  }
  if (!row_ptr || !y || (nnz > 0 && (!col_ind || !vals || !x)))
    return fail(-1, "NULL buffer");
  const int ntiles = (int)ntiles_l;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return fail(-2, std::string("no usable CUDA device: ") + cudaGetErrorString(e));
  // set-up, once per device, with that device current
  Scratch *s = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_addr_mu);
    if (!g_addr[dev]) {
      void *p = nullptr;
      e = cudaGetSymbolAddress(&p, g_scratch);
      if (e != cudaSuccess || !p) {
        cudaGetLastError();
        return fail(-2, std::string("cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
      }
      g_addr[dev] = (Scratch *)p;
    }
    s = g_addr[dev];
  }
  cudaStream_t st = (cudaStream_t)stream;
  // the error flag must start at zero; every other slot a call reads, the
  // same call writes first
  e = cudaMemsetAsync(&s->error, 0, sizeof(int), st);
  if (e != cudaSuccess) return fail(-2, std::string("memset: ") + cudaGetErrorString(e));
  k_spmv_tiles<<<ntiles, pdlp::kThreads, 0, st>>>(rows, cols, nnz, ntiles, row_ptr, col_ind,
                                                  vals, x, y, s);
  k_spmv_tiles_fix<<<(ntiles + pdlp::kThreads - 1) / pdlp::kThreads, pdlp::kThreads, 0, st>>>(
      ntiles, row_ptr, y, s);
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(-2, std::string("launch: ") + cudaGetErrorString(e));
  int flag = 0;
  e = cudaMemcpyAsync(&flag, &s->error, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return fail(-2, std::string("sync: ") + cudaGetErrorString(e));
  if (flag & 2) return fail(-4, "column index out of range");
  if (flag & 1) return fail(-4, "malformed row pointers");
  return 0;
}
