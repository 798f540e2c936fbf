// spmv_pipe.cuh -- the PDHG step kernels' SpMV: a persistent, TMA-fed
// pipeline over byte-budget tiles, with the row epilogue fused.
//
// Replaces, for the two step launches of every iteration, the reference's
// cusparseSpMV(CSR_ALG2) and the element kernel after it
// (src/pdlp_core_op.cu:495-526 primal, :528-557 dual).
//
// Why: a step is one pass over the matrix (col, val), its row pointers and
// the step's per-row vectors (x, c, bounds, anchor for the primal step; y,
// bounds, anchor for the dual step), all of them contiguous ranges per tile,
// plus a gather of the other side's iterate (L2-resident).  Loaded by threads
// these streams come in dependent rounds (plan -> offsets -> elements ->
// gather -> row vectors), so the kernel waits on memory latency instead of
// streaming.  Here every contiguous range of a tile is one bulk copy
// (cp.async.bulk, global -> shared, completion counted on an mbarrier) issued
// STAGES tiles ahead by one thread, so HBM sees long streams in flight
// without registers or extra blocks, and threads touch global memory only
// for the gather and the row outputs.
//
// Tiles (host plan, build_pipe_plan_host): consecutive rows [r0, r1) packed
// while at most kPipeRows rows, kPipeTile non-zeros and kPipeTileBytes of
// stage buffer (all ranges, padded to their 16-byte copy boundaries) fit;
// a row of more than kPipeMedRows non-zeros gets a tile of its own (one
// block-wide sum); a row of more than kPipeTile non-zeros is cut into chunks
// of kPipeTile, each summed by one tile, the last chunk to finish (atomic
// ticket, checked by the CTA at its next tile) adding the chunk sums in
// chunk order and running the epilogue.
// Tile t runs on CTA t % grid, in increasing t: every sum has a fixed order,
// so results are bitwise reproducible.
//
// Arithmetic per packed tile: lane l folds E consecutive elements (E the
// odd number at or above len / 256, so the lanes' stride-E reads of the
// linearly copied stage are free of bank conflicts) with one FMA each (all
// lanes busy: GB300 issues an FP64 warp instruction at the same cost whether
// 1 or 32 lanes are active), leaving the partial of each row run in shared
// memory; then thread j adds the run partials of row j and runs the
// epilogue on the row's vectors from the stage buffer.  A tile of one row,
// or one chunk of a long row, is summed with lanes striding the elements.
//
// Copy ranges start on 16-byte boundaries below the tile's first element and
// end on the boundary above its last, so a copy reads up to 15 bytes outside
// the range: every array this kernel reads is a 256-byte-aligned allocation
// padded to a multiple of 256 bytes (Arena::take), which keeps those bytes
// inside the allocation.
#pragma once

#include <stdint.h>

#include <type_traits>
#include <vector>

#include "bulk.cuh"
#include "spmv.cuh"

namespace pdlp {

// Shape of the pipeline (PDLP_PIPE_TILE / _STAGES / _CTAS override them at
// build time): tiles of up to kPipeTile non-zeros in stage buffers of
// kPipeStageBytes, kPipeStages stages a CTA (so kPipeStages - 1 tiles are in
// flight while one is processed), kPipeCtasPerSm CTAs resident on an SM.
#ifndef PDLP_PIPE_TILE
#define PDLP_PIPE_TILE 2048
#endif
#ifndef PDLP_PIPE_STAGES
#define PDLP_PIPE_STAGES 2
#endif
#ifndef PDLP_PIPE_CTAS
#define PDLP_PIPE_CTAS 3
#endif
constexpr int kPipeRows = kThreads;      // rows per packed tile (one per thread)
constexpr int kPipeTile = PDLP_PIPE_TILE;
// elements per lane: the odd number at or above kPipeTile / 256
constexpr int kPipeMaxE = ((kPipeTile + kThreads - 1) / kThreads) | 1;
constexpr int kPipeMedRows = 128;        // longer rows get a tile of their own
// a tile's copies: a chunk of kPipeTile 8-byte values and their columns,
// plus copy padding; the stage adds room for the 256 lane sums of a one-row
// tile (a double, or a float pair)
constexpr int kPipeTileBytes = kPipeTile * 12 + 1024;
constexpr int kPipeStageBytes = kPipeTileBytes + kThreads * 8;
static_assert(kPipeStageBytes - kPipeTileBytes >= kThreads * 8 &&
                  kPipeStageBytes - kPipeTileBytes >= kThreads * 2 * 4,
              "lane-sum area of a stage");
constexpr int kPipeStages = PDLP_PIPE_STAGES;
constexpr int kPipeCtasPerSm = PDLP_PIPE_CTAS;

// Byte layout of one tile in a stage buffer: row pointers [r0, r1], columns
// and values [k0, k1), NV vectors [r0, r1); each range widened to 16-byte
// copy boundaries.  SM: bytes per matrix value, ST: per vector element.
struct PipeLayout {
  int a_ptr, a_col, a_val, a_vec;   // first element index copied, per range
  int b_ptr, b_col, b_val, b_vec;   // bytes per range (b_vec: per vector)
  int o_col, o_val, o_vec;          // byte offsets in the stage (ptr at 0)
  int total;
};

__host__ __device__ inline PipeLayout pipe_layout(int4 b, int SM, int ST, int NV) {
  PipeLayout L{};
  const int k0 = b.z, k1 = b.w;
  const bool packed = b.y >= 0;
  const int len = k1 - k0;
  if (packed) {
    const int r0 = b.x, r1 = b.y;
    L.a_ptr = r0 & ~3;
    L.b_ptr = (((r1 + 1) + 3) & ~3) * 4 - L.a_ptr * 4;
    const int tv = 16 / ST;
    L.a_vec = r0 & ~(tv - 1);
    L.b_vec = r1 > r0 ? ((((r1 + tv - 1) & ~(tv - 1)) - L.a_vec) * ST) : 0;
  }
  if (len > 0) {
    L.a_col = k0 & ~3;
    L.b_col = (((k1 + 3) & ~3) - L.a_col) * 4;
    const int mv = 16 / SM;
    L.a_val = k0 & ~(mv - 1);
    L.b_val = (((k1 + mv - 1) & ~(mv - 1)) - L.a_val) * SM;
  }
  L.o_col = L.b_ptr;
  L.o_val = L.o_col + L.b_col;
  L.o_vec = L.o_val + L.b_val;
  L.total = L.o_vec + NV * L.b_vec;
  return L;
}

// Largest stage a tile needs in any precision the solver runs (FP64, FP32,
// FP32 matrix with FP64 vectors).
inline int pipe_tile_bytes(int4 b, int NV) {
  int a = pipe_layout(b, 8, 8, NV).total;
  int c = pipe_layout(b, 4, 4, NV).total;
  int d = pipe_layout(b, 4, 8, NV).total;
  return a > c ? (a > d ? a : d) : (c > d ? c : d);
}

// Host: tiles of the pipelined kernel for a matrix whose step epilogue has NV
// per-row vectors.  Same descriptor as the fused kernel's plan:
// {r0, r1 | -(long_id + 1), k0, k1}, lrow[long_id] = {first tile, chunks}.
inline void build_pipe_plan_host(int rows, const int *ptr, int NV, std::vector<int4> &blk,
                                 std::vector<int2> &lrow) {
  blk.clear();
  lrow.clear();
  int r = 0;
  while (r < rows) {
    const int len = ptr[r + 1] - ptr[r];
    if (len > kPipeTile) {
      const int nch = (len + kPipeTile - 1) / kPipeTile;
      const int lid = (int)lrow.size();
      lrow.push_back(make_int2((int)blk.size(), nch));
      for (int c = 0; c < nch; ++c) {
        const int k0 = ptr[r] + c * kPipeTile;
        const int k1 = k0 + kPipeTile < ptr[r + 1] ? k0 + kPipeTile : ptr[r + 1];
        blk.push_back(make_int4(r, -(lid + 1), k0, k1));
      }
      ++r;
      continue;
    }
    const int r0 = r;
    ++r;  // the first row always fits (len <= kPipeTile)
    if (len <= kPipeMedRows) {
      while (r < rows && r - r0 < kPipeRows) {
        const int l2 = ptr[r + 1] - ptr[r];
        if (l2 > kPipeMedRows || ptr[r + 1] - ptr[r0] > kPipeTile) break;
        if (pipe_tile_bytes(make_int4(r0, r + 1, ptr[r0], ptr[r + 1]), NV) > kPipeTileBytes) break;
        ++r;
      }
    }
    blk.push_back(make_int4(r0, r, ptr[r0], ptr[r]));
  }
}

// ticket of a long row's chunk: counts the arrival after this thread's
// earlier writes (the chunk sum) are visible; returns the previous count
__device__ __forceinline__ unsigned ticket_release(unsigned *p) {
  unsigned prev;
  asm volatile("atom.add.release.gpu.u32 %0, [%1], 1;" : "=r"(prev) : "l"(p) : "memory");
  return prev;
}

// Per-lane accumulation of a run of products.  FP64 matrices: one FMA per
// non-zero.  FP32 matrices: a compensated (double-float) sum -- each product
// split exactly with an FMA, each addition with its rounding error (2Sum,
// Knuth) -- so rows of tens of thousands of cancelling terms keep close to
// FP64 accuracy at about 9 FP32 instructions per non-zero, which GB300's
// FP32 pipe (64x its FP64 rate) absorbs.  The _rn intrinsics keep the
// compiler from contracting the error terms into FMAs.
template <class M>
struct LaneAcc;
template <>
struct LaneAcc<double> {
  double s = 0.0;
  __device__ __forceinline__ void add(double a, double x) { s = fma(a, x, s); }
  __device__ __forceinline__ void add_pair(double h, double) { s += h; }
  __device__ __forceinline__ double hi() const { return s; }
  __device__ __forceinline__ double lo() const { return 0.0; }
  __device__ __forceinline__ double total() const { return s; }
  __device__ __forceinline__ double rounded() const { return s; }
};
template <>
struct LaneAcc<float> {
  float h = 0.f, l = 0.f;
  __device__ __forceinline__ void two_sum(float b) {
    const float s = __fadd_rn(h, b);
    const float bb = __fsub_rn(s, h);
    const float e = __fadd_rn(__fsub_rn(h, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    h = s;
    l = __fadd_rn(l, e);
  }
  __device__ __forceinline__ void add(float a, float x) {
    const float p = __fmul_rn(a, x);
    const float pe = fmaf(a, x, -p);  // exact: a x = p + pe
    two_sum(p);
    l = __fadd_rn(l, pe);
  }
  __device__ __forceinline__ void add_pair(float hb, float lb) {
    two_sum(hb);
    l = __fadd_rn(l, lb);
  }
  __device__ __forceinline__ float hi() const { return h; }
  __device__ __forceinline__ float lo() const { return l; }
  __device__ __forceinline__ double total() const { return (double)h + (double)l; }
  __device__ __forceinline__ float rounded() const { return __fadd_rn(h, l); }
};

// The pipelined step kernel's plan (per matrix): tiles, long rows, grid.
struct PipePlan {
  int ntile = 0, nlong = 0, grid = 0;
  int4 *blk = nullptr;        // tile descriptors
  int2 *lrow = nullptr;       // per long row {first tile, chunk count}
  unsigned *lcnt = nullptr;   // per long row arrival counter (per solve, kept at 0)
  double *lsum = nullptr;     // per tile chunk sum (per solve)
  int *err = nullptr;         // per solve: set when a stage wait timed out
};

// Threads of the pipelined kernel: kThreads consumers (8 warps) and one
// producer warp that issues the stage copies.
constexpr int kPipeBlock = kThreads + 32;

// The consumers' barrier (named barrier 1, kThreads threads): the producer
// warp never waits on it.
__device__ __forceinline__ void consumers_sync() {
  asm volatile("bar.sync 1, %0;" ::"n"(kThreads) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// Epi has the fused kernel's interface; the step epilogues also declare
// `static constexpr int NV`, `vec_t`, `vecs(const vec_t *(&)[NV])` (the
// per-row vectors, each read at the row index) and
// `make_pre(const vec_t (&)[NV])` (the row's preloaded values), and then get
// those vectors from the stage buffer.
//
// Roles: the producer warp's lane 0 issues tile i's copies into stage
// i % kPipeStages once the consumers have released that stage (empty
// mbarrier, one arrival per consumer warp); the 8 consumer warps wait for
// the stage (full mbarrier, completed by the copies' byte count), process
// the tile with one consumers-only barrier in the middle, and release it.
// Every wait is bounded: a consumer whose stage never arrives marks itself
// bad, skips the work that reads the stage but keeps to the barriers (so no
// barrier waits on a thread that left), and the CTA reports the timeout in
// plan.err.
template <class Epi>
__global__ void __launch_bounds__(kPipeBlock, kPipeCtasPerSm)
    spmv_pipe(const int *__restrict__ ptr, const int *__restrict__ col,
              const typename Epi::val_t *__restrict__ val, PipePlan plan,
              double *__restrict__ part, double *__restrict__ lpart, Epi epi) {
  using M = typename Epi::val_t;
  using A = typename Epi::acc_t;
  using T = typename step_vectors<Epi>::vec_t;
  constexpr int NF = Epi::NF;
  constexpr int NV = step_vectors<Epi>::NV;
  static_assert(sizeof(A) == sizeof(M), "run partials share the value buffer");
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t full[kPipeStages];
  __shared__ __align__(8) uint64_t empty[kPipeStages];
  __shared__ double red[8 * (NF > 0 ? NF : 1) + 8];
  __shared__ double sc[4];

  if (!epi.init()) return;
  const int tid = threadIdx.x;
  const int G = gridDim.x;
  const int first = blockIdx.x;
  const int mine = first < plan.ntile ? (plan.ntile - 1 - first) / G + 1 : 0;

  if (tid == 0) {
    for (int q = 0; q < kPipeStages; ++q) {
      mbar_init(&full[q], 1);
      mbar_init(&empty[q], kThreads / 32);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    epi.prologue(sc);
  }
  __syncthreads();
  epi.bind(sc);

  if (tid >= kThreads) {
    // producer warp
    if (tid == kThreads) {
      const uint64_t pol = l2_evict_first();
      const T *vbase[NV > 0 ? NV : 1];
      if constexpr (NV > 0) epi.vecs(vbase);
      for (int i = 0; i < mine; ++i) {
        const int q = i % kPipeStages;
        if (i >= kPipeStages &&
            !mbar_wait_bounded(&empty[q], (unsigned)((i / kPipeStages - 1) & 1))) {
          atomicOr(plan.err, 1);  // the consumers' waits then time out too
          break;
        }
        const int4 b = plan.blk[first + i * G];
        const PipeLayout L = pipe_layout(b, (int)sizeof(M), (int)sizeof(T), NV);
        unsigned char *st = smem + (size_t)q * kPipeStageBytes;
        uint64_t *bar = &full[q];
        const int nvec = b.y >= 0 && L.b_vec > 0 ? NV : 0;
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_arrive_expect_tx(bar, (unsigned)(L.b_ptr + L.b_col + L.b_val + nvec * L.b_vec));
        if (L.b_ptr) bulk_g2s(st, ptr + L.a_ptr, L.b_ptr, bar, pol);
        if (L.b_col) bulk_g2s(st + L.o_col, col + L.a_col, L.b_col, bar, pol);
        if (L.b_val) bulk_g2s(st + L.o_val, val + L.a_val, L.b_val, bar, pol);
        for (int v = 0; v < nvec; ++v)
          bulk_g2s(st + L.o_vec + v * L.b_vec, vbase[v] + L.a_vec, L.b_vec, bar, pol);
      }
    }
    return;
  }

  // ---------------------------------------------------------- consumers
  const int lane = tid & 31, warp = tid >> 5;
  bool bad = false;
  // A long row's chunk counts its arrival without waiting for the count
  // (thread 0 keeps the ticket); the check, and for the last chunk the
  // row's sum and epilogue, run at the start of the CTA's next tile.
  int pend_lid = -1, pend_row = 0;
  unsigned pend_prev = 0;
  int2 pend_lr = make_int2(0, 0);
  auto finish_long = [&]() {
    if (pend_lid < 0) return;
    const int lid = pend_lid;
    pend_lid = -1;
    if (pend_prev != (unsigned)pend_lr.y - 1u) return;
    asm volatile("fence.acq_rel.gpu;" ::: "memory");  // every chunk sum is visible
    double sum = 0.0;
#pragma unroll 4
    for (int c = 0; c < pend_lr.y; ++c) sum += __ldcg(plan.lsum + pend_lr.x + c);
    double lacc[NF > 0 ? NF : 1];
#pragma unroll
    for (int f = 0; f < (NF > 0 ? NF : 1); ++f) lacc[f] = 0.0;
    epi.row(pend_row, (A)sum, lacc);
    if constexpr (NF > 0) {
#pragma unroll
      for (int f = 0; f < NF; ++f) lpart[f * plan.nlong + lid] = lacc[f];
    }
    plan.lcnt[lid] = 0u;  // ready for the next launch
  };

  double acc[NF > 0 ? NF : 1];
#pragma unroll
  for (int f = 0; f < (NF > 0 ? NF : 1); ++f) acc[f] = 0.0;

  int4 b_next = mine > 0 ? plan.blk[first] : make_int4(0, 0, 0, 0);
  for (int i = 0; i < mine; ++i) {
    const int t = first + i * G;
    const int q = i % kPipeStages;
    const int4 b = b_next;
    if (i + 1 < mine) b_next = plan.blk[t + G];  // in flight while this tile runs
    if (tid == 0 && !bad) finish_long();
    const PipeLayout L = pipe_layout(b, (int)sizeof(M), (int)sizeof(T), NV);
    unsigned char *st = smem + (size_t)q * kPipeStageBytes;
    if (!bad && !mbar_wait_bounded(&full[q], (unsigned)((i / kPipeStages) & 1))) {
      bad = true;
      atomicOr(plan.err, 1);
    }
    const int *sptr = reinterpret_cast<const int *>(st);
    const int *scol = reinterpret_cast<const int *>(st + L.o_col) + (b.z - L.a_col);
    M *sval = reinterpret_cast<M *>(st + L.o_val) + (b.z - L.a_val);
    const int k0 = b.z, len = b.w - b.z;
    if (b.y < 0 || b.y - b.x == 1) {
      // one row (or one chunk of a long row): lane l takes elements l,
      // l + 256, ... (consecutive lanes, consecutive words: no bank
      // conflicts), sums them in a fixed order; rounds past the tile's end
      // are left by a block-uniform break, not predicated (GB300 charges an
      // FP64 issue slot per warp instruction however many lanes are active)
      LaneAcc<M> s;
      if (!bad) {
        M xg[kPipeMaxE];
#pragma unroll
        for (int u = 0; u < kPipeMaxE; ++u) {
          if (u * kThreads >= len) break;
          if (tid + u * kThreads < len) xg[u] = epi.gather(scol[tid + u * kThreads]);
        }
#pragma unroll
        for (int u = 0; u < kPipeMaxE; ++u) {
          if (u * kThreads >= len) break;
          if (tid + u * kThreads < len) s.add(sval[tid + u * kThreads], xg[u]);
        }
      }
      // the 256 lane sums go to the stage's partials area; warp 0 adds 8
      // per lane, then one shuffle tree (13 warp instructions, on the FP32
      // pipe in double-float for FP32 matrices)
      // (area of kThreads * 8 bytes: one double per lane, or for FP32 the
      // high floats then the low floats)
      M *ph = reinterpret_cast<M *>(st + kPipeTileBytes);
      float *pl = reinterpret_cast<float *>(ph + kThreads);  // FP32 only
      ph[tid] = (M)s.hi();
      if constexpr (sizeof(M) == 4) pl[tid] = (float)s.lo();
      consumers_sync();
      if (warp == 0) {
        if (!bad) {
          LaneAcc<M> r;
#pragma unroll
          for (int w = 0; w < kThreads / 32; ++w) {
            if constexpr (sizeof(M) == 4) r.add_pair(ph[lane + 32 * w], pl[lane + 32 * w]);
            else r.add_pair(ph[lane + 32 * w], M(0));
          }
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) {
            const M hb = __shfl_xor_sync(0xffffffffu, r.hi(), o);
            const M lb = __shfl_xor_sync(0xffffffffu, r.lo(), o);
            r.add_pair(hb, lb);
          }
          if (lane == 0) {
            const double tot = r.total();
            if (b.y >= 0) {
              // a row of its own: vectors from the stage
              if constexpr (NV > 0) {
                const T *sv0 = reinterpret_cast<const T *>(st + L.o_vec);
                T pv[NV];
#pragma unroll
                for (int v = 0; v < NV; ++v)
                  pv[v] = sv0[(size_t)v * (L.b_vec / sizeof(T)) + (b.x - L.a_vec)];
                epi.row_pre(b.x, (A)tot, epi.make_pre(pv), acc);
              } else {
                epi.row(b.x, (A)tot, acc);
              }
            } else {
              const int lid = -b.y - 1;
              plan.lsum[t] = tot;
              pend_prev = ticket_release(plan.lcnt + lid);
              pend_lr = plan.lrow[lid];  // both in flight until the next tile
              pend_lid = lid;
              pend_row = b.x;
            }
          }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[q]);
      } else if (lane == 0) {
        mbar_arrive(&empty[q]);
      }
    } else {
      // packed rows: lane l folds the E consecutive elements [lE, lE + E)
      // with E odd -- a stride of E words (or 2E for 8-byte values) across a
      // warp then hits every bank once -- leaving run partials; then one
      // thread per row
      int E = (len + kThreads - 1) / kThreads;
      E |= 1;  // <= kPipeMaxE for len <= kPipeTile
      const int beg = tid * E;
      const int r0 = b.x, R = b.y - b.x;
      const int *soff = sptr + (r0 - L.a_ptr);  // soff[j] - k0: row j's first element
      // run partials: the high part in the value slot of the run's first
      // element, the low part (compensated FP32 sums) in its column slot --
      // both already consumed by this lane
      float *slo = reinterpret_cast<float *>(
          reinterpret_cast<int *>(st + L.o_col) + (b.z - L.a_col));
      if (!bad && beg < len) {
        M xg[kPipeMaxE];
#pragma unroll
        for (int u = 0; u < kPipeMaxE; ++u) {
          if (u >= E) break;  // block-uniform
          if (beg + u < len) xg[u] = epi.gather(scol[beg + u]);
        }
        const int end = beg + E < len ? beg + E : len;
        int lo = 0, hi = R;  // row j with soff[j] - k0 <= beg < soff[j + 1] - k0
        while (hi - lo > 1) {
          const int mid = (lo + hi) >> 1;
          if (soff[mid] - k0 <= beg) lo = mid;
          else hi = mid;
        }
        int nb = soff[lo + 1] - k0, j = lo, segs = beg;
        LaneAcc<M> s;
        auto flush = [&](int at) {
          sval[at] = (M)s.hi();
          if constexpr (sizeof(M) == 4) slo[at] = (float)s.lo();
        };
#pragma unroll
        for (int u = 0; u < kPipeMaxE; ++u) {
          if (u >= E) break;  // block-uniform
          const int e = beg + u;
          if (e < end) {
            while (e == nb) {  // a row ends before element e
              if (segs < e) flush(segs);
              s = LaneAcc<M>();
              segs = e;
              ++j;
              nb = soff[j + 1] - k0;
            }
            s.add(sval[e], xg[u]);
          }
        }
        flush(segs);
      }
      consumers_sync();
      if (!bad && tid < R) {
        const int a = soff[tid] - k0, e = soff[tid + 1] - k0;
        LaneAcc<M> sum;
        if (a < e) {
          auto part_at = [&](int qq) {
            if constexpr (sizeof(M) == 4) sum.add_pair(sval[qq], slo[qq]);
            else sum.add_pair(sval[qq], M(0));
          };
          part_at(a);
          for (int qq = (a / E + 1) * E; qq < e; qq += E) part_at(qq);
        }
        if constexpr (NV > 0) {
          const T *sv0 = reinterpret_cast<const T *>(st + L.o_vec);
          T pv[NV];
#pragma unroll
          for (int v = 0; v < NV; ++v)
            pv[v] = sv0[(size_t)v * (L.b_vec / sizeof(T)) + (r0 + tid - L.a_vec)];
          epi.row_pre(r0 + tid, (A)sum.rounded(), epi.make_pre(pv), acc);
        } else {
          epi.row(r0 + tid, (A)sum.rounded(), acc);
        }
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[q]);
    }
  }
  if (tid == 0 && !bad) finish_long();
  if constexpr (NF > 0) {
    // consumers-only block reduction of the per-thread fields
#pragma unroll
    for (int f = 0; f < NF; ++f)
      acc[f] = ((Epi::MAXMASK >> f) & 1u) ? warp_max(acc[f]) : warp_sum(acc[f]);
    if (lane == 0) {
#pragma unroll
      for (int f = 0; f < NF; ++f) red[f * 8 + warp] = acc[f];
    }
    consumers_sync();
    if (tid == 0) {
#pragma unroll
      for (int f = 0; f < NF; ++f) {
        double r = 0.0;
#pragma unroll
        for (int w = 0; w < kThreads / 32; ++w)
          r = ((Epi::MAXMASK >> f) & 1u) ? fmax(r, red[f * 8 + w]) : r + red[f * 8 + w];
        part[f * G + blockIdx.x] = r;
      }
    }
  }
}

// Dynamic shared memory of the pipelined kernel.
constexpr int kPipeSmem = kPipeStages * kPipeStageBytes;
// kPipeCtasPerSm CTAs (each with ~2 KB of static shared memory and the 1 KB
// the SM reserves per CTA) must fit the SM's 228 KB, or the grid would run
// in two waves.
static_assert(kPipeCtasPerSm * (kPipeSmem + 2 * 1024) <= 228 * 1024,
              "pipeline stages do not fit kPipeCtasPerSm CTAs per SM");

}  // namespace pdlp
