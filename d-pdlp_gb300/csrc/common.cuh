// common.cuh -- shared device helpers, error handling and the device-resident
// control block of one PDHG solve.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <stdexcept>
#include <string>

namespace pdlp {

// Host-side CUDA error check: throws, so every public entry point can turn
// a failure into a NULL / error return instead of exiting the process (the
// reference exits, internal/utils.h:30-58).
struct CudaError : std::runtime_error {
  cudaError_t code;
  CudaError(cudaError_t c, const std::string &what)
      : std::runtime_error(what), code(c) {}
};

#define PDLP_CUDA(call)                                                     \
  do {                                                                      \
    cudaError_t e_ = (call);                                                \
    if (e_ != cudaSuccess)                                                  \
      throw ::pdlp::CudaError(e_, std::string(#call) + " -> " +             \
                                      cudaGetErrorString(e_) + " at " +     \
                                      __FILE__ + ":" +                      \
                                      std::to_string(__LINE__));            \
  } while (0)

#define PDLP_LAUNCH_CHECK() PDLP_CUDA(cudaGetLastError())

constexpr int kThreads = 256;  // every kernel of the solver uses 256 threads
constexpr int kNumSms = 152;   // GB300

// Evaluation cadence of the reference driver (src/utils.cu:492-501).
__host__ __device__ inline int print_frequency(int iter) {
  int step = 10;
  long long threshold = 1000;
  while (iter >= threshold) {
    step *= 10;
    threshold *= 10;
  }
  return step;
}

// ------------------------------------------------------------------ control
// Every scalar of the iteration lives here, in device memory, so that whole
// chunks of iterations run without a host round trip.  Field meanings follow
// the reference's pdhg_solver_state_t (internal/internal_types.h:50-145).
struct Ctl {
  // step size / primal weight (reference pdlp_core_op.cu:577-656)
  double step_size;       // eta
  double primal_weight;   // omega
  double best_primal_weight;
  double tau, sigma, inv_sigma;  // eta/omega, eta*omega, 1/sigma
  double best_gap;        // best |log10(rel_d/rel_p)|
  double pw_error_sum;
  double pw_last_error;
  // restart bookkeeping (reference utils.cu:265-293)
  double fixed_point_error;
  double initial_fixed_point_error;
  double last_trial_fixed_point_error;
  // KKT measures (reference utils.cu:639-719)
  double abs_primal_res, rel_primal_res, abs_dual_res, rel_dual_res;
  double primal_obj, dual_obj, gap, rel_gap;
  // infeasibility (reference utils.cu:721-813)
  double max_primal_ray_inf, max_dual_ray_inf, primal_ray_obj, dual_ray_obj;
  double ray_primal_inf_norm, ray_dual_inf_norm;  // scratch
  double cum_time;
  double best_err;  // best max(rel_p, rel_d, rel_gap) seen (stall detection)
  double snap_err;  // error of the snapshot iterate (refinement rounds)
  // iteration counters
  int t_base;       // iteration number of the first iteration of the chunk
  int restart_t;    // total_count at the last restart (inner = t - restart_t)
  int do_restart;   // decided at an evaluation, consumed by restart + FPE
  int done;         // 1 once a termination reason is set
  int reason;       // termination_reason_t
  int final_t;      // total_count at termination
  int trace_len;
  int best_err_t;   // iteration of the last 10% improvement of best_err
  int snap_now;     // 1: the evaluation just made is the best so far
  unsigned long long t_start_ns;  // %globaltimer at loop start
  // power method (reference utils.cu:66-171)
  double pm_inv_norm;
  double pm_sigma_sq;
  double pm_res;
  int pm_done;
  int pm_iters;
};

// Host-visible mirror written by the device when a solve finishes.
struct HostFlag {
  volatile int done;
  volatile int pm_done;
};

// Device memory of the solve path: a stream-ordered pool owned by the library
// (no device-wide synchronisation, unlike cudaMalloc / cudaFree); a block
// freed on a stream is reused by later allocations (memory.cu).
void *dev_alloc(size_t bytes, cudaStream_t st);
void dev_free(void *p, cudaStream_t st);
// Mapped pinned termination flags from a slab allocated once.
HostFlag *hostflag_acquire();
void hostflag_release(HostFlag *f);
// Return the pool's cached blocks to the device.
void release_pooled_memory();

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// ------------------------------------------------------------- reductions
// All reductions are deterministic: a fixed tree inside a block, and block
// partials combined in block order by a single-block finaliser.
template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
// max(lo, min(t, hi)), the projection onto [lo, hi] in the reference's
// operand order (a crossed interval yields lo).  For doubles it compares
// order-preserving integer keys -- for IEEE values, flipping the magnitude
// bits of negatives makes signed 64-bit order equal numeric order (-0 sorts
// below +0) -- so the projection issues on the integer pipe instead of
// GB300's FP64 pipe, where min/max cost a full FP64 issue slot each.
__device__ __forceinline__ long long order_key(double v) {
  long long b = __double_as_longlong(v);
  return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
__device__ __forceinline__ double clamp_to(double t, double lo, double hi) {
  long long kt = order_key(t), kh = order_key(hi);
  double r = kt > kh ? hi : t;
  long long kr = kt > kh ? kh : kt;
  return kr < order_key(lo) ? lo : r;
}
__device__ __forceinline__ float clamp_to(float t, float lo, float hi) {
  return fmaxf(lo, fminf(t, hi));
}

template <class T>
__device__ __forceinline__ T warp_max(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Block-wide sum of NF doubles; result valid in thread 0.
template <int NF>
__device__ __forceinline__ void block_sum(double (&v)[NF], double *smem /*>= 8*NF*/) {
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int f = 0; f < NF; ++f) v[f] = warp_sum(v[f]);
  if (lane == 0) {
#pragma unroll
    for (int f = 0; f < NF; ++f) smem[f * 8 + wid] = v[f];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int f = 0; f < NF; ++f) {
      double s = 0.0;
#pragma unroll
      for (int w = 0; w < kThreads / 32; ++w) s += smem[f * 8 + w];
      v[f] = s;
    }
  }
  __syncthreads();
}

// Sum (or max, when IS_MAX) of part[0..n) by one block of kThreads threads,
// in a fixed order.  Result returned to every thread.
template <bool IS_MAX>
__device__ double block_fold(const double *part, int n, double *smem) {
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += kThreads)
    s = IS_MAX ? fmax(s, part[i]) : s + part[i];
  s = IS_MAX ? warp_max(s) : warp_sum(s);
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) smem[wid] = s;
  __syncthreads();
  double r = 0.0;
  for (int w = 0; w < kThreads / 32; ++w) r = IS_MAX ? fmax(r, smem[w]) : r + smem[w];
  __syncthreads();
  return r;
}

inline int grid_for(long n, int per_thread = 1) {
  long b = (n + (long)kThreads * per_thread - 1) / ((long)kThreads * per_thread);
  if (b < 1) b = 1;
  long cap = (long)kNumSms * 16;
  return (int)(b < cap ? b : cap);
}

}  // namespace pdlp
