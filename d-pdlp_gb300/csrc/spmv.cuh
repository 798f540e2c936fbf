// spmv.cuh -- row-binned ("CSR-adaptive") sparse matrix-vector product with a
// fused per-row epilogue.
//
// Replaces the reference's cusparseSpMV(CSR_ALG2) calls
// (src/pdlp_core_op.cu:501-504, :534-537, :671-674, :801-804;
// src/utils.cu:134-140, :645-653, :750-758) and the elementwise kernel that
// follows each of them.
//
// Layout: the matrix stays in CSR (int32 row_ptr / col, value array).  A plan
// cuts the rows into thread-block tiles of at most TILE non-zeros:
//   * light tile : consecutive rows [r0, r1) whose non-zeros fit in TILE; the
//                  block streams the tile's values and column indices with
//                  coalesced loads, gathers x and stages (value, x) pairs in
//                  shared memory.  Short rows (at most 64 non-zeros on
//                  average): each lane folds 8 consecutive pairs, then each
//                  row adds its 1-3 segment partials -- every FP64 instruction
//                  runs with all 32 lanes.  Few long rows: a group of G lanes
//                  per row (G = 256 / rows, power of two, at most 32); a tile
//                  with one row uses the whole block.  In the DIRECT variant
//                  (chosen per matrix), short rows of 16 or more non-zeros
//                  skip the staging: each lane loads, gathers and folds an
//                  aligned group of 4 elements in registers;
//   * long row   : a row with more than TILE non-zeros is cut into chunks (up
//                  to 8 tiles long), one block each, folded in passes of TILE
//                  non-zeros; the last block to finish (atomic ticket) sums
//                  the chunk partials in chunk order and runs the epilogue.
// Every sum has a fixed order for a given plan, so results are bitwise
// reproducible run to run.  The epilogue of row r runs once, in one thread,
// and may add to NF per-block reduction fields (sums, or maxima where bit f
// of Epi::MAXMASK is set); the block writes them to part[f * nblk + block],
// and long-row contributions to lpart[f * nlong + long_row], for a
// single-block finaliser to fold in a fixed order.
#pragma once

#include <type_traits>
#include <vector>

#include "common.cuh"

namespace pdlp {

constexpr int kMaxRowsPerTile = 1024;

struct SpmvPlan {
  int rows = 0, nblk = 0, nlong = 0, tile = 0;
  int direct = 0;             // launch the register-path variant (see plan_direct)
  int4 *blk = nullptr;        // {r0, r1 | -(long_id+1), k0, k1}
  int2 *lrow = nullptr;       // per long row {first block, chunk count}
  unsigned *lcnt = nullptr;   // per long row arrival counter (kept at 0)
  double *lsum = nullptr;     // per block chunk partial (long rows)
};

// Host: cut rows into tiles.  `ptr` is the host copy of the row pointer.
// Rows longer than `tile` are cut into chunks of `chunk` (>= tile) non-zeros.
inline void build_plan_host(int rows, const int *ptr, int tile,
                            std::vector<int4> &blk, std::vector<int2> &lrow, int chunk = 0) {
  blk.clear();
  lrow.clear();
  if (chunk < tile) chunk = tile;
  int r = 0;
  while (r < rows) {
    int len = ptr[r + 1] - ptr[r];
    if (len > tile) {
      int nch = (len + chunk - 1) / chunk;
      int lid = (int)lrow.size();
      lrow.push_back(make_int2((int)blk.size(), nch));
      for (int c = 0; c < nch; ++c) {
        int k0 = ptr[r] + c * chunk;
        int k1 = k0 + chunk < ptr[r + 1] ? k0 + chunk : ptr[r + 1];
        blk.push_back(make_int4(r, -(lid + 1), k0, k1));
      }
      ++r;
    } else {
      int r0 = r, k0 = ptr[r];
      while (r < rows && (r - r0) < kMaxRowsPerTile && ptr[r + 1] - k0 <= tile) ++r;
      blk.push_back(make_int4(r0, r, k0, ptr[r]));
    }
  }
}

// Light tiles whose rows hold at least this many non-zeros on average take
// the register path (4-element groups per lane) in the DIRECT variant of the
// kernel; shorter rows are staged through shared memory.
constexpr int kDirectMinAvg = 16;

// Host: whether a matrix should run the register-path variant -- when at least
// half of its non-zeros sit in short-row tiles of kDirectMinAvg or more
// non-zeros per row.  Measured per step with tiles of 1024 (FP64): the
// power-law LP's A (m = 1M, rows of ~20) 0.151 -> 0.135 ms; a random LP's A
// (m = 200k, rows of ~25) 0.049 ms either way; rows of ~10 (that LP's
// transpose) 0.047 -> 0.051 ms and rows of 1-4 0.153 -> 0.170 ms, so those
// stay on the staged kernel at 6 blocks per SM.
inline bool plan_direct(const std::vector<int4> &blk, long nnz) {
  long in = 0;
  for (const int4 &b : blk) {
    const int R = b.y - b.x, len = b.w - b.z;
    if (b.y >= 0 && R > 1 && len <= 64 * R && len >= kDirectMinAvg * R) in += len;
  }
  return nnz > 0 && 2 * in >= nnz;
}

template <class T>
__device__ __forceinline__ T ld_stream(const T *p) {
  return __ldcs(p);  // matrix data is read once per sweep: evict first
}

template <int NF, unsigned MAXMASK>
__device__ __forceinline__ void block_reduce_fields(double (&acc)[NF > 0 ? NF : 1],
                                                    double *red) {
  if constexpr (NF > 0) {
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int f = 0; f < NF; ++f)
      acc[f] = ((MAXMASK >> f) & 1u) ? warp_max(acc[f]) : warp_sum(acc[f]);
    if (lane == 0) {
#pragma unroll
      for (int f = 0; f < NF; ++f) red[f * 8 + wid] = acc[f];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
      for (int f = 0; f < NF; ++f) {
        double s = 0.0;
#pragma unroll
        for (int w = 0; w < kThreads / 32; ++w)
          s = ((MAXMASK >> f) & 1u) ? fmax(s, red[f * 8 + w]) : s + red[f * 8 + w];
        acc[f] = s;
      }
    }
  }
}

// Epi must provide:
//   using val_t;  (matrix value and gathered vector type)
//   using acc_t;  (accumulation type of the row sums)
//   static constexpr int NF; static constexpr unsigned MAXMASK;
//   __device__ bool init();                   // all threads; false: skip (uniform)
//   __device__ void prologue(double *sc);     // thread 0: per-block scalars
//   __device__ void bind(const double *sc);   // all threads, after the barrier
//   __device__ val_t gather(int col) const;   // x[col] (any transform)
//   __device__ void row(int r, acc_t sum, double *acc) const;
//
// GB300 executes FP64 at about 2 lanes per clock per SM, so an FP64 sweep is
// bound by FP64 issue as much as by HBM.  The kernel therefore spends exactly
// one fused multiply-add per non-zero: phase 1 stages (value, x[col]) pairs
// in shared memory with coalesced loads, phase 2 folds each row with FMA, and
// scalars that need a division (step sizes, Halpern weight) are formed once
// per block by thread 0.
// Shared-memory swizzle for the staged (value, x) pairs: phase 1 writes
// consecutive elements per lane, the staged stream phase reads 8 consecutive
// elements per lane (lane stride 8); XOR-ing the low 3 bits with higher index
// bits makes both patterns bank-conflict free for 4- and 8-byte elements.
template <class T>
__device__ __forceinline__ int swz(int i) {
  return i ^ ((i >> (sizeof(T) == 8 ? 4 : 5)) & 7);
}

// Epilogues may define `struct Pre`, `preload(r, Pre&)` and
// `row_pre(r, sum, const Pre&, acc)`: the stream path then issues each row's
// vector loads in phase 1, next to the matrix stream, instead of after it.
template <class E, class = void>
struct has_preload : std::false_type {};
template <class E>
struct has_preload<E, std::void_t<typename E::Pre>> : std::true_type {};
template <class E, bool = has_preload<E>::value>
struct pre_of {
  struct type {};
};
template <class E>
struct pre_of<E, true> {
  using type = typename E::Pre;
};

// Resident blocks per SM the register allocation must allow.  The kernel is
// latency-bound (dependent col -> gather -> FMA chains, per-row vector loads),
// so residency pays: 6 blocks of 256 threads (40 registers) for FP64 tiles of
// up to 1024 non-zeros, 8 blocks (32 registers, up to 28 bytes of L1-resident
// spills) for FP32 values -- measured on GB300 against 6 blocks: the 20M-nnz
// power-law primal step 0.115 -> 0.102 ms, the transport primal step 0.163
// -> 0.131 ms and its dual step 0.079 -> 0.073 ms.  2048-element tiles need
// their registers (the long-row path keeps 8 loads per thread in flight) and
// run at 4 blocks.  The register-path variant holds a group's columns and
// values across the first barrier and runs at 5 blocks (48 registers).  In
// FP32 it is faster at 8 (the power-law dual step 0.107 ms at 5 blocks, 0.093
// at 8), but then the per-matrix choice on the 20M-nnz power-law LP takes it
// for A instead of the pipelined kernel, and with its rounding that LP's FP32
// trajectory needs 69,400 iterations to 1e-4 against 55,200: 14.4 s against
// 11.5 s end to end, so 5 stays the default.
// FP64 tiles stay at 6: at 8 (32 registers, 120 bytes of spills) the
// power-law primal step goes from 0.153 to 0.183 ms, the FP64 pipe being
// the other bound there.  PDLP_FUSED_FP32_BLOCKS, PDLP_DIRECT_FP32_BLOCKS and
// PDLP_FUSED_FP64_BLOCKS override the counts at build time.
#ifndef PDLP_FUSED_FP32_BLOCKS
#define PDLP_FUSED_FP32_BLOCKS 8
#endif
#ifndef PDLP_FUSED_FP64_BLOCKS
#define PDLP_FUSED_FP64_BLOCKS 6
#endif
#ifndef PDLP_DIRECT_FP32_BLOCKS
#define PDLP_DIRECT_FP32_BLOCKS 5
#endif
template <int TILE, bool DIRECT = false, int VBYTES = 8>
constexpr int spmv_min_blocks() {
  return TILE >= 2048 ? 1
         : DIRECT     ? (VBYTES == 4 ? PDLP_DIRECT_FP32_BLOCKS : 5)
         : VBYTES == 4 ? PDLP_FUSED_FP32_BLOCKS
                       : PDLP_FUSED_FP64_BLOCKS;
}

template <int TILE, class Epi, bool DIRECT = false>
__global__ void __launch_bounds__(kThreads,
                                  spmv_min_blocks<TILE, DIRECT, sizeof(typename Epi::val_t)>())
    spmv_fused(const int *__restrict__ ptr, const int *__restrict__ col,
               const typename Epi::val_t *__restrict__ val, SpmvPlan plan,
               double *__restrict__ part, double *__restrict__ lpart, Epi epi) {
  using T = typename Epi::val_t;
  using A = typename Epi::acc_t;
  constexpr int NF = Epi::NF;
  constexpr int IPT = TILE / kThreads;
  static_assert(sizeof(A) == sizeof(T), "run partials share the value buffer");
  __shared__ __align__(16) T sv[TILE + 8];  // values; run partials of short rows;
                                             // chunk partials of a long row (as doubles)
  __shared__ __align__(16) T sx[TILE];      // gathered x; start rows of short-row groups
  __shared__ int soff[kMaxRowsPerTile + 1];
  __shared__ double red[8 * (NF > 0 ? NF : 1) + 8];
  __shared__ double sc[4];
  __shared__ int s_last;

  if (!epi.init()) return;
  if (threadIdx.x == 0) epi.prologue(sc);
  const int4 b = plan.blk[blockIdx.x];
  const int k0 = b.z, len = b.w - b.z;
  const int R = b.y >= 0 ? b.y - b.x : 0;
  double acc[NF > 0 ? NF : 1];
#pragma unroll
  for (int f = 0; f < (NF > 0 ? NF : 1); ++f) acc[f] = 0.0;

  if (b.y < 0) {
    // Chunk of a long row: each thread folds its IPT elements straight from
    // global memory (coalesced loads, no shared staging); the 256 partials are
    // summed in FP64 through shared memory -- warp 0 adds 8 per lane, then
    // shuffles -- 13 FP64 warp instructions instead of a shuffle tree in every
    // warp.  Rows of up to ~10^5 terms with cancellation keep every sum across
    // threads, warps and chunks in FP64.
    A s = A(0);
    // the chunk (any length) in passes of IPT elements per thread
    for (int base = 0; base < len; base += IPT * kThreads) {
      int cidx[IPT];
      T v[IPT], xg[IPT];
#pragma unroll
      for (int u = 0; u < IPT; ++u) {
        int i = base + threadIdx.x + u * kThreads;
        if (i < len) {
          cidx[u] = ld_stream(col + k0 + i);
          v[u] = ld_stream(val + k0 + i);
        }
      }
#pragma unroll
      for (int u = 0; u < IPT; ++u)
        if (base + threadIdx.x + u * kThreads < len) xg[u] = epi.gather(cidx[u]);
#pragma unroll
      for (int u = 0; u < IPT; ++u)
        if (base + threadIdx.x + u * kThreads < len) s = fma((A)v[u], (A)xg[u], s);
    }
    double *tp = reinterpret_cast<double *>(sv);
    tp[threadIdx.x] = (double)s;
    __syncthreads();
    epi.bind(sc);
    const int lid = -b.y - 1;
    if (threadIdx.x < 32) {
      double t = 0.0;
#pragma unroll
      for (int w = 0; w < kThreads / 32; ++w) t += tp[threadIdx.x + 32 * w];
      t = warp_sum(t);
      if (threadIdx.x == 0) {
        plan.lsum[blockIdx.x] = t;
        __threadfence();
        unsigned prev = atomicAdd(plan.lcnt + lid, 1u);
        s_last = (prev == (unsigned)plan.lrow[lid].y - 1u);
      }
    }
    __syncthreads();
    if (s_last && threadIdx.x == 0) {
      __threadfence();
      const int2 L = plan.lrow[lid];
      double tot = 0.0;
      for (int c = 0; c < L.y; ++c) tot += __ldcg(plan.lsum + L.x + c);
      double lacc[NF > 0 ? NF : 1];
#pragma unroll
      for (int f = 0; f < (NF > 0 ? NF : 1); ++f) lacc[f] = 0.0;
      epi.row(b.x, (A)tot, lacc);
      if constexpr (NF > 0) {
#pragma unroll
        for (int f = 0; f < NF; ++f) lpart[f * plan.nlong + lid] = lacc[f];
      }
      plan.lcnt[lid] = 0u;  // ready for the next launch
    }
    if constexpr (NF > 0) {
      if (threadIdx.x == 0) {
#pragma unroll
        for (int f = 0; f < NF; ++f) part[f * plan.nblk + blockIdx.x] = 0.0;
      }
    }
    return;
  }

  const bool stream = R > 1 && len <= 64 * R;
  [[maybe_unused]] typename pre_of<Epi>::type pre;
  if (DIRECT && stream && len >= kDirectMinAvg * R) {
    // Register path, rows of kDirectMinAvg or more non-zeros on average: lane
    // g owns the aligned group [kb + 4g, kb + 4g + 4) of the matrix arrays
    // (kb = k0 rounded down to a multiple of 4; elements outside [k0, k0 +
    // len) are skipped).  It loads the group with 16-byte vector loads (scalar
    // loads for a partial group or arrays off 16-byte boundaries) straight
    // into registers, gathers x and folds it with FMA; only the row offsets,
    // the start row of each group and the partial of each run (a row's
    // elements inside one group) pass through shared memory, and the first
    // barrier waits for row offsets only, not for the matrix stream.
    constexpr int GRP = 4;
    A *runp = reinterpret_cast<A *>(sv);      // run partials by position - kb
    int *srow = reinterpret_cast<int *>(sx);  // row holding position GRP * g
    const int k1 = k0 + len, kb = k0 & ~(GRP - 1);
    const int ngrp = (k1 - kb + GRP - 1) / GRP;
    const bool vec =
        ((reinterpret_cast<uintptr_t>(col) | reinterpret_cast<uintptr_t>(val)) & 15) == 0;
    auto load_group = [&](int g, int (&c)[GRP], T (&v)[GRP]) {
      const int base = kb + GRP * g;
      if (vec && base >= k0 && base + GRP <= k1) {
        const int4 c4 = __ldcs(reinterpret_cast<const int4 *>(col + base));
        c[0] = c4.x; c[1] = c4.y; c[2] = c4.z; c[3] = c4.w;
        if constexpr (sizeof(T) == 8) {
          const double2 v0 = __ldcs(reinterpret_cast<const double2 *>(val + base));
          const double2 v1 = __ldcs(reinterpret_cast<const double2 *>(val + base) + 1);
          v[0] = v0.x; v[1] = v0.y; v[2] = v1.x; v[3] = v1.y;
        } else {
          const float4 v4 = __ldcs(reinterpret_cast<const float4 *>(val + base));
          v[0] = v4.x; v[1] = v4.y; v[2] = v4.z; v[3] = v4.w;
        }
      } else {
#pragma unroll
        for (int u = 0; u < GRP; ++u) {
          const int e = base + u;
          if (e >= k0 && e < k1) {
            c[u] = ld_stream(col + e);
            v[u] = ld_stream(val + e);
          }
        }
      }
    };
    auto fold_group = [&](int g, const int (&c)[GRP], const T (&v)[GRP]) {
      const int base = GRP * g;  // relative to kb
      const int lo = (k0 - kb) > base ? (k0 - kb) : base;
      const int hi = (k1 - kb) < base + GRP ? (k1 - kb) : base + GRP;
      T xg[GRP];
#pragma unroll
      for (int u = 0; u < GRP; ++u)
        if (base + u >= lo && base + u < hi) xg[u] = epi.gather(c[u]);
      // group 0 may start before the tile: begin at row 0 and step over
      // empty rows; later groups start inside the row that srow names
      int j = g == 0 ? 0 : srow[g];
      int nb = soff[j + 1], segs = lo;
      A s = A(0);
#pragma unroll
      for (int u = 0; u < GRP; ++u) {
        const int e = base + u;
        if (e >= lo && e < hi) {
          while (e == nb) {
            if (segs < e) runp[segs] = s;
            s = A(0);
            segs = e;
            ++j;
            nb = soff[j + 1];
          }
          s = fma((A)v[u], (A)xg[u], s);
        }
      }
      if (lo < hi) runp[segs] = s;
    };

    int c[GRP];
    T v[GRP];
    if ((int)threadIdx.x < ngrp) load_group(threadIdx.x, c, v);
    if constexpr (has_preload<Epi>::value) {
      if ((int)threadIdx.x < R) epi.preload(b.x + threadIdx.x, pre);
    }
    for (int j = threadIdx.x; j <= R; j += kThreads) {
      const int a = ptr[b.x + j] - kb;
      soff[j] = a;
      if (j < R) {
        const int e = ptr[b.x + j + 1] - kb;
        for (int q = (a + GRP - 1) & ~(GRP - 1); q < e; q += GRP) srow[q / GRP] = j;
      }
    }
    __syncthreads();
    epi.bind(sc);
    for (int g = threadIdx.x; g < ngrp; g += kThreads) {
      if (g != (int)threadIdx.x) load_group(g, c, v);  // tiles of more than 256 groups
      fold_group(g, c, v);
    }
    __syncthreads();
    // Row fold: the run at the row start, then one per group boundary inside.
    for (int j = threadIdx.x; j < R; j += kThreads) {
      const int a = soff[j], e = soff[j + 1];
      A sum = A(0);
      if (a < e) {
        sum = runp[a];
        for (int q = (a & ~(GRP - 1)) + GRP; q < e; q += GRP) sum += runp[q];
      }
      if constexpr (has_preload<Epi>::value) {
        if (j == (int)threadIdx.x) epi.row_pre(b.x + j, sum, pre, acc);
        else epi.row(b.x + j, sum, acc);
      } else {
        epi.row(b.x + j, sum, acc);
      }
    }
  } else {
    // Phase 1: coalesced stream of values / columns, gather of x, row offsets.
    {
      int cidx[IPT];
#pragma unroll
      for (int u = 0; u < IPT; ++u) {
        int i = threadIdx.x + u * kThreads;
        if (i < len) {
          cidx[u] = ld_stream(col + k0 + i);
          sv[swz<T>(i)] = ld_stream(val + k0 + i);
        }
      }
      if constexpr (has_preload<Epi>::value) {
        if (stream && threadIdx.x < R) epi.preload(b.x + threadIdx.x, pre);
      }
      for (int j = threadIdx.x; j <= R; j += kThreads) soff[j] = ptr[b.x + j] - k0;
#pragma unroll
      for (int u = 0; u < IPT; ++u) {
        int i = threadIdx.x + u * kThreads;
        if (i < len) sx[swz<T>(i)] = epi.gather(cidx[u]);
      }
    }
    __syncthreads();
    epi.bind(sc);
    const int r0 = b.x;
    if (stream) {
      // Very short rows: lane t folds staged elements [8t, 8t+8) with FMA, all
      // lanes busy; each finished segment's partial goes to sv[swz(start)], a
      // slot the lane has already consumed.
      constexpr int SEG = 8;
      const int beg = threadIdx.x * SEG;
      if (beg < len) {
        const int end = beg + SEG < len ? beg + SEG : len;
        int lo = 0, hi = R;  // row j with soff[j] <= beg < soff[j+1]
        while (hi - lo > 1) {
          int mid = (lo + hi) >> 1;
          if (soff[mid] <= beg) lo = mid;
          else hi = mid;
        }
        int j = lo, nb = soff[j + 1], segs = beg;
        A s = A(0);
        for (int e = beg; e < end; ++e) {
          while (e == nb) {
            if (segs < e) sv[swz<T>(segs)] = (T)s;
            s = A(0);
            segs = e;
            ++j;
            nb = soff[j + 1];
          }
          s = fma((A)sv[swz<T>(e)], (A)sx[swz<T>(e)], s);
        }
        sv[swz<T>(segs)] = (T)s;
      }
      __syncthreads();
      // Row fold: segment at the row start, then one per lane boundary inside.
      for (int j = threadIdx.x; j < R; j += kThreads) {
        const int a = soff[j], e = soff[j + 1];
        A sum = A(0);
        if (a < e) {
          sum = (A)sv[swz<T>(a)];
          for (int q = (a / SEG + 1) * SEG; q < e; q += SEG) sum += (A)sv[swz<T>(q)];
        }
        if constexpr (has_preload<Epi>::value) {
          if (j == (int)threadIdx.x) epi.row_pre(b.x + j, sum, pre, acc);
          else epi.row(b.x + j, sum, acc);
        } else {
          epi.row(b.x + j, sum, acc);
        }
      }
    } else if (R == 1) {
      // one long light row: lane chains in A, cross-lane sums in FP64
      A s = A(0);
      for (int i = threadIdx.x; i < len; i += kThreads)
        s = fma((A)sv[swz<T>(i)], (A)sx[swz<T>(i)], s);
      double v = warp_sum((double)s);
      int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
      if (lane == 0) red[wid] = v;
      __syncthreads();
      if (threadIdx.x == 0) {
        double tot = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) tot += red[w];
        epi.row(r0, (A)tot, acc);
      }
    } else if (R > 1) {
      // few long rows: a group of G lanes per row
      int g = kThreads / R;
      int G = 1;
      while (G * 2 <= g && G < 32) G *= 2;
      int grp = threadIdx.x / G, li = threadIdx.x & (G - 1);
      A s = A(0);
      if (grp < R) {
        int beg = soff[grp], end = soff[grp + 1];
        for (int i = beg + li; i < end; i += G) s = fma((A)sv[swz<T>(i)], (A)sx[swz<T>(i)], s);
      }
      double sd = s;  // cross-lane sums in FP64
      for (int o = G >> 1; o > 0; o >>= 1) sd += __shfl_xor_sync(0xffffffffu, sd, o);
      if (li == 0 && grp < R) epi.row(r0 + grp, (A)sd, acc);
    }
  }

  if constexpr (NF > 0) {
    __syncthreads();
    block_reduce_fields<NF, Epi::MAXMASK>(acc, red);
    if (threadIdx.x == 0) {
#pragma unroll
      for (int f = 0; f < NF; ++f) part[f * plan.nblk + blockIdx.x] = acc[f];
    }
  }
}

// Fold per-block and long-row partials of field f of one SpMV site.
template <bool IS_MAX>
__device__ double fold_site(const double *part, int nblk, const double *lpart,
                            int nlong, int f, double *smem) {
  double a = block_fold<IS_MAX>(part + (long)f * nblk, nblk, smem);
  double b = block_fold<IS_MAX>(lpart + (long)f * nlong, nlong, smem);
  return IS_MAX ? fmax(a, b) : a + b;
}

}  // namespace pdlp
