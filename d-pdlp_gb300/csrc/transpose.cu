// transpose.cu -- A^T of an uploaded CSR matrix, built on the device.
//
// Replaces the reference's cusparseCsr2cscEx2 (src/pdlp_core_op.cu:109-130)
// and this library's former host transpose on the upload path.  The result
// is the stable transpose: row j of A^T lists the entries of column j of A
// in increasing row order (equal rows -- duplicate entries -- in input
// order), bit for bit what a stable counting sort gives.
//
// Method: an LSD radix sort of the keys col[k] carrying the positions k,
// 8 bits a pass (ceil(log2 n / 8) passes), each pass stable:
//   1. k_digit_hist: per tile of kTileKeys keys, the count of each digit;
//   2. k_scan_hist: exclusive scan of the counts in (digit, tile) order;
//   3. k_scatter: every key goes to scan[digit][tile] + (keys of the same
//      digit before it in its tile), the in-tile rank found warp by warp
//      with __match_any_sync in input order.
// Then A^T's columns are the rows of the carried positions, its values the
// values at those positions, and its row pointers the first position of
// each key (binary search in the sorted keys).
#include <cuda_runtime.h>

#include <utility>

#include "common.cuh"
#include "solver.cuh"

namespace pdlp {

namespace {

constexpr int kRadixBits = 8;
constexpr int kDigits = 1 << kRadixBits;
constexpr int kKeysPerLane = 8;
constexpr int kWarps = kThreads / 32;
constexpr int kTileKeys = kThreads * kKeysPerLane;  // 2048 keys per tile

// row of every position: the r with ptr[r] <= k < ptr[r + 1]
__global__ void k_row_of(int m, int nnz, const int *__restrict__ ptr, int *__restrict__ rowk) {
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < nnz;
       k += (long)gridDim.x * blockDim.x) {
    int lo = 0, hi = m;  // last r in [0, m) with ptr[r] <= k
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (ptr[mid] <= (int)k) lo = mid;
      else hi = mid;
    }
    rowk[k] = lo;
  }
}

__global__ void k_iota(int nnz, int *__restrict__ v) {
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < nnz;
       k += (long)gridDim.x * blockDim.x)
    v[k] = (int)k;
}

__global__ void __launch_bounds__(kThreads)
    k_digit_hist(int nnz, int shift, const int *__restrict__ keys, int ntiles,
                 int *__restrict__ hist) {
  __shared__ int cnt[kDigits];
  for (int d = threadIdx.x; d < kDigits; d += kThreads) cnt[d] = 0;
  __syncthreads();
  const long base = (long)blockIdx.x * kTileKeys;
  for (int u = 0; u < kKeysPerLane; ++u) {
    const long k = base + u * kThreads + threadIdx.x;
    if (k < nnz) atomicAdd(&cnt[(keys[k] >> shift) & (kDigits - 1)], 1);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < kDigits; d += kThreads)
    hist[(long)d * ntiles + blockIdx.x] = cnt[d];
}

// Exclusive scan of total = kDigits * ntiles counts by one block: each
// thread scans a contiguous run, the run totals are scanned in shared memory.
__global__ void __launch_bounds__(1024) k_scan_hist(long total, int *__restrict__ hist) {
  __shared__ long run[1024];
  const long per = (total + 1023) / 1024;
  const long a = threadIdx.x * per, e = a + per < total ? a + per : total;
  long s = 0;
  for (long i = a; i < e; ++i) s += hist[i];
  run[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    long acc = 0;
    for (int t = 0; t < 1024; ++t) {
      const long v = run[t];
      run[t] = acc;
      acc += v;
    }
  }
  __syncthreads();
  long acc = run[threadIdx.x];
  for (long i = a; i < e; ++i) {
    const int v = hist[i];
    hist[i] = (int)acc;
    acc += v;
  }
}

__global__ void __launch_bounds__(kThreads)
    k_scatter(int nnz, int shift, const int *__restrict__ kin, const int *__restrict__ vin,
              int *__restrict__ kout, int *__restrict__ vout, int ntiles,
              const int *__restrict__ scan) {
  __shared__ int wcnt[kWarps][kDigits];  // per warp: count, then its offset
  for (int i = threadIdx.x; i < kWarps * kDigits; i += kThreads) (&wcnt[0][0])[i] = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const unsigned lt = (1u << lane) - 1u;
  // warp w owns the contiguous keys [base, base + 32 * kKeysPerLane) of the
  // tile, taken 32 at a time in order
  const long base = (long)blockIdx.x * kTileKeys + (long)w * 32 * kKeysPerLane;
  int key[kKeysPerLane], rank[kKeysPerLane];
#pragma unroll
  for (int u = 0; u < kKeysPerLane; ++u) {
    const long k = base + u * 32 + lane;
    key[u] = k < nnz ? kin[k] : 0;
    // past the end: digit kDigits matches only other such lanes, counts nothing
    const int d = k < nnz ? (key[u] >> shift) & (kDigits - 1) : kDigits;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int before = __popc(peers & lt);
    int start = 0;
    if (d < kDigits) start = wcnt[w][d];
    __syncwarp();
    if (d < kDigits && before == 0) wcnt[w][d] = start + __popc(peers);
    __syncwarp();
    rank[u] = start + before;
  }
  __syncthreads();
  // counts -> offsets: warps in order within each digit
  for (int d = threadIdx.x; d < kDigits; d += kThreads) {
    int acc = 0;
    for (int q = 0; q < kWarps; ++q) {
      const int c = wcnt[q][d];
      wcnt[q][d] = acc;
      acc += c;
    }
  }
  __syncthreads();
#pragma unroll
  for (int u = 0; u < kKeysPerLane; ++u) {
    const long k = base + u * 32 + lane;
    if (k < nnz) {
      const int d = (key[u] >> shift) & (kDigits - 1);
      const long pos = (long)scan[(long)d * ntiles + blockIdx.x] + wcnt[w][d] + rank[u];
      kout[pos] = key[u];
      vout[pos] = vin[k];
    }
  }
}

// A^T: row pointers from the sorted keys, columns (rows of A) and values
__global__ void k_transpose_out(int n, int nnz, const int *__restrict__ skeys,
                                const int *__restrict__ spos, const int *__restrict__ rowk,
                                const double *__restrict__ val, int *__restrict__ tptr,
                                int *__restrict__ tcol, double *__restrict__ tval) {
  const long stride = (long)gridDim.x * blockDim.x;
  for (long j = blockIdx.x * (long)blockDim.x + threadIdx.x; j <= n; j += stride) {
    int lo = 0, hi = nnz;  // first position with key >= j
    while (lo < hi) {
      const int mid = (int)(((long)lo + hi) >> 1);
      if (skeys[mid] < (int)j) lo = mid + 1;
      else hi = mid;
    }
    tptr[j] = lo;
  }
  for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < nnz; p += stride) {
    const int k = spos[p];
    tcol[p] = rowk[k];
    tval[p] = val[k];
  }
}

}  // namespace

size_t device_transpose_scratch_bytes(int n, int nnz) {
  (void)n;
  const long ntiles = ((long)nnz + kTileKeys - 1) / kTileKeys;
  return 5 * ((size_t)nnz * 4 + 256) + (size_t)kDigits * (ntiles > 0 ? ntiles : 1) * 4 + 256;
}

void device_transpose(int m, int n, int nnz, const int *ptr, const int *col, const double *val,
                      int *tptr, int *tcol, double *tval, void *scratch, cudaStream_t st) {
  auto a256 = [](size_t b) { return (b + 255) & ~(size_t)255; };
  char *p = (char *)scratch;
  int *k0 = (int *)p; p += a256((size_t)nnz * 4);
  int *k1 = (int *)p; p += a256((size_t)nnz * 4);
  int *v0 = (int *)p; p += a256((size_t)nnz * 4);
  int *v1 = (int *)p; p += a256((size_t)nnz * 4);
  int *rowk = (int *)p; p += a256((size_t)nnz * 4);
  int *hist = (int *)p;
  const int ntiles = (int)(((long)nnz + kTileKeys - 1) / kTileKeys);
  const int g = grid_for(nnz > n + 1 ? nnz : n + 1);
  if (nnz > 0) {
    PDLP_CUDA(cudaMemcpyAsync(k0, col, (size_t)nnz * 4, cudaMemcpyDeviceToDevice, st));
    k_iota<<<g, kThreads, 0, st>>>(nnz, v0);
    k_row_of<<<g, kThreads, 0, st>>>(m, nnz, ptr, rowk);
    PDLP_LAUNCH_CHECK();
    int bits = 0;
    while (bits < 31 && (1L << bits) < (long)n) ++bits;
    for (int shift = 0; shift < bits; shift += kRadixBits) {
      k_digit_hist<<<ntiles, kThreads, 0, st>>>(nnz, shift, k0, ntiles, hist);
      k_scan_hist<<<1, 1024, 0, st>>>((long)kDigits * ntiles, hist);
      k_scatter<<<ntiles, kThreads, 0, st>>>(nnz, shift, k0, v0, k1, v1, ntiles, hist);
      PDLP_LAUNCH_CHECK();
      std::swap(k0, k1);
      std::swap(v0, v1);
    }
  }
  k_transpose_out<<<g, kThreads, 0, st>>>(n, nnz, k0, v0, rowk, val, tptr, tcol, tval);
  PDLP_LAUNCH_CHECK();
}

}  // namespace pdlp
