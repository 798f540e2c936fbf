// solver.cu -- problem upload and the FP64 instantiation of the PDHG solve.
//
// The iteration itself (kernels and the Solve driver) lives in
// solver_impl.cuh; this file holds the pieces defined once: the non-template
// kernels, the host transpose, the device-resident problem, and
// Solve<double, double>.
#include <string.h>

#include <algorithm>
#include <atomic>
#include <exception>
#include <thread>

#include "solver_impl.cuh"

namespace pdlp {

__global__ void k_set_tbase(Ctl *ctl, int t) { ctl->t_base = t; }
__global__ void k_loop_start(Ctl *ctl) { ctl->t_start_ns = global_ns(); }
__global__ void k_set_steps(Ctl *c) { set_steps(c); }
// Halpern weights (k+1)/(k+2), the quotients the iteration would form
__global__ void k_halpern_table(double *hw, int len) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < len) hw[k] = (double)(k + 1) / (double)(k + 2);
}

// ---- power method element kernels (utils.cu:107-153), FP64
__global__ void __launch_bounds__(kThreads) k_pm_norm(PowDev d, const double *v) {
  if (d.ctl->pm_done) return;
  __shared__ double red[16];
  double a[1] = {0.0};
  long stride = (long)gridDim.x * kThreads;
  for (long i = blockIdx.x * (long)kThreads + threadIdx.x; i < d.m; i += stride)
    a[0] += v[i] * v[i];
  block_reduce_fields<1, 0u>(a, red);
  if (threadIdx.x == 0) d.p_pr[blockIdx.x] = a[0];
}

__global__ void __launch_bounds__(kThreads) k_pm_norm_fin(PowDev d) {
  if (d.ctl->pm_done) return;
  __shared__ double sm[32];
  double s = block_fold<false>(d.p_pr, d.ew_grid, sm);
  if (threadIdx.x == 0) d.ctl->pm_inv_norm = 1.0 / sqrt(s);
}

__global__ void __launch_bounds__(kThreads) k_pm_dot_fin(PowDev d) {
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
    k_pm_resid(PowDev d, const double *v, const double *vnext) {
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

__global__ void __launch_bounds__(kThreads) k_pm_resid_fin(PowDev d) {
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

// A^T in CSR, entries of each column in row order (a stable counting sort).
// Matrices of 4M+ non-zeros are transposed by up to 8 threads, each owning a
// range of columns (balanced by non-zeros) and scanning every row in order,
// so the result is the serial one, bit for bit.
void host_transpose(int m, int n, const int *ap, const int *aj, const double *ax,
                    std::vector<int> &tp, host_buf<int> &tj, host_buf<double> &tx) {
  const int nnz = ap[m];
  tp.assign((size_t)n + 1, 0);
  tj.resize(nnz);
  tx.resize(nnz);
  const unsigned hw = std::thread::hardware_concurrency();
  const int T = nnz >= 4000000 && n > 0 ? (int)std::min(8u, hw ? hw : 1u) : 1;
  auto run = [&](auto &&f) {
    std::vector<std::thread> th;
    for (int t = 1; t < T; ++t) th.emplace_back(f, t);
    f(0);
    for (auto &x : th) x.join();
  };
  // column counts: thread t owns columns [n t / T, n (t+1) / T)
  run([&](int t) {
    const int c0 = (int)((long)n * t / T), c1 = (int)((long)n * (t + 1) / T);
    for (int k = 0; k < nnz; ++k) {
      const int c = aj[k];
      if (c >= c0 && c < c1) tp[c + 1]++;
    }
  });
  for (int c = 0; c < n; ++c) tp[c + 1] += tp[c];
  // scatter: column ranges of about nnz / T entries each
  std::vector<int> cut(T + 1, n);
  cut[0] = 0;
  for (int t = 1; t < T; ++t)
    cut[t] = std::max(cut[t - 1], (int)(std::lower_bound(tp.begin(), tp.end(),
                                                         (int)((long)nnz * t / T)) - tp.begin()));
  cut[T] = n;
  run([&](int t) {
    const int c0 = std::min(cut[t], n), c1 = std::min(cut[t + 1], n);
    if (c0 >= c1) return;
    std::vector<int> next(tp.begin() + c0, tp.begin() + c1);
    for (int r = 0; r < m; ++r)
      for (int k = ap[r]; k < ap[r + 1]; ++k) {
        const int c = aj[k];
        if (c >= c0 && c < c1) {
          const int pos = next[c - c0]++;
          tj[pos] = r;
          tx[pos] = ax[k];
        }
      }
  });
}

// Non-zeros per thread-block tile.  PDLP_SPMV_TILE (512, 1024 or 2048)
// overrides the size rule (1024 measured fastest on the 20M-nnz power-law and
// transport LPs at 6 resident blocks per SM).
static int pick_tile(long nnz) {
  if (const char *e = getenv("PDLP_SPMV_TILE")) {
    int t = atoi(e);
    if (t == 512 || t == 1024 || t == 2048) return t;
  }
  return nnz >= 2000000 ? 1024 : 512;
}

// Non-zeros per block of a row longer than a tile: 8192 (at most 8 tiles).
// Long chunks amortise the block's FP64 reduction, barriers and ticket over
// more non-zeros (measured on the 20M-nnz LPs: power-law primal step -12%,
// transport dual step -25% against one tile per chunk; 16384 loses to load
// imbalance).  PDLP_SPMV_CHUNK (a multiple of the tile, at most 16384)
// overrides the default.
static int pick_chunk(int tile) {
  if (const char *e = getenv("PDLP_SPMV_CHUNK")) {
    int c = atoi(e);
    if (c >= tile && c <= 16384 && c % tile == 0) return c;
  }
  return tile * 8 < 8192 ? tile * 8 : 8192;
}

int kernel_override() {
  static const int v = [] {
    const char *e = getenv("PDLP_STEP_KERNEL");
    if (e && strcmp(e, "pipe") == 0) return 1;
    if (e && strcmp(e, "fused") == 0) return 0;
    return -1;
  }();
  return v;
}

namespace {
std::mutex g_choice_mu;
std::map<uint64_t, std::array<int, 2>> g_choice[3];

// FNV-1a over 32-bit words (the fingerprint only has to separate structures
// within one process)
uint64_t fnv1a(uint64_t h, const int *v, size_t count) {
  for (size_t i = 0; i < count; ++i) h = (h ^ (uint32_t)v[i]) * 1099511628211ull;
  return h;
}

// Host threads for the upload's passes over the non-zeros (LPs of 2M+
// non-zeros; smaller ones stay on the calling thread).
int upload_threads(long nnz) {
  const unsigned hw = std::thread::hardware_concurrency();
  return nnz >= (1L << 21) ? (int)std::min(16u, hw ? hw : 1u) : 1;
}

// f(begin, end) over [0, count) in T contiguous slices, slice 0 on this thread
template <class F>
void parallel_slices(int T, long count, F &&f) {
  if (T <= 1) {
    f(0L, count);
    return;
  }
  std::vector<std::thread> th;
  for (int t = 1; t < T; ++t) th.emplace_back([&f, t, T, count] { f(count * t / T, count * (t + 1) / T); });
  f(0L, count / T);
  for (auto &x : th) x.join();
}
}  // namespace

bool lookup_kernel_choice(uint64_t key, int prec, int c[2]) {
  std::lock_guard<std::mutex> lk(g_choice_mu);
  auto it = g_choice[prec].find(key);
  if (it == g_choice[prec].end()) return false;
  c[0] = it->second[0];
  c[1] = it->second[1];
  return true;
}

void settle_kernel_choice(uint64_t key, int prec, int c[2]) {
  std::lock_guard<std::mutex> lk(g_choice_mu);
  auto it = g_choice[prec].emplace(key, std::array<int, 2>{c[0], c[1]}).first;
  c[0] = it->second[0];
  c[1] = it->second[1];
}

DevProblem::~DevProblem() {
  if (arena) dev_free(arena, owner);
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
    if (ok) {
      std::atomic<bool> bad{false};
      parallel_slices(upload_threads(nnz), nnz, [&](long a, long b) {
        for (long k = a; k < b; ++k)
          if (cj[k] < 0 || cj[k] >= n) {
            bad.store(true, std::memory_order_relaxed);
            return;
          }
      });
      ok = !bad.load();
    }
    if (!ok) throw std::runtime_error("invalid CSR matrix (row pointers or column indices)");
  }
  auto P = std::make_unique<DevProblem>();
  P->owner = st;
  P->m = m;
  P->n = n;
  P->nnz = nnz;
  P->tile = pick_tile(nnz);
  P->c0 = prob->objective_constant;
  // row pointers of A^T (column counts of A, prefix-summed) for the plans;
  // A^T itself is built on the device after A is uploaded
  std::vector<int> tp((size_t)n + 1, 0);
  {
    const int *cj = prob->constraint_matrix_col_indices;
    int *cnt = tp.data() + 1;
    const int T = upload_threads(nnz);
    if (T > 1) {
      parallel_slices(T, nnz, [&](long a, long b) {
        for (long k = a; k < b; ++k) __atomic_fetch_add(cnt + cj[k], 1, __ATOMIC_RELAXED);
      });
    } else {
      for (int k = 0; k < nnz; ++k) cnt[cj[k]]++;
    }
    for (int c = 0; c < n; ++c) tp[c + 1] += tp[c];
  }
  {
    const int dims[3] = {m, n, nnz};
    uint64_t h = fnv1a(1469598103934665603ull, dims, 3);
    h = fnv1a(h, prob->constraint_matrix_row_pointers, (size_t)m + 1);
    P->shape_key = fnv1a(h, tp.data(), (size_t)n + 1);
  }
  std::vector<int4> blkA, blkT;
  std::vector<int2> lrA, lrT;
  const int chunk = pick_chunk(P->tile);
  // pipelined step kernel: the dual step (A) stages 4 row vectors, the
  // primal step (A^T) 5.  A's plans are built on a second thread for large
  // LPs, beside A^T's.
  std::vector<int4> pblkA, pblkT;
  std::vector<int2> plrA, plrT;
  auto plans_A = [&] {
    build_plan_host(m, prob->constraint_matrix_row_pointers, P->tile, blkA, lrA, chunk);
    build_pipe_plan_host(m, prob->constraint_matrix_row_pointers, 4, pblkA, plrA);
  };
  std::exception_ptr failed_A;
  std::thread thread_A;
  if (upload_threads(nnz) > 1)
    thread_A = std::thread([&] {
      try {
        plans_A();
      } catch (...) {
        failed_A = std::current_exception();
      }
    });
  else
    plans_A();
  try {
    build_plan_host(n, tp.data(), P->tile, blkT, lrT, chunk);
    build_pipe_plan_host(n, tp.data(), 5, pblkT, plrT);
  } catch (...) {
    if (thread_A.joinable()) thread_A.join();
    throw;
  }
  if (thread_A.joinable()) thread_A.join();
  if (failed_A) std::rethrow_exception(failed_A);
  int dev = 0, nsm = kNumSms;
  PDLP_CUDA(cudaGetDevice(&dev));
  PDLP_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
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
  z.add<int>(vm + 1); z.add<int>(nnz); z.add<double>(nnz);
  z.add<int>(vn + 1); z.add<int>(nnz); z.add<double>(nnz);
  z.add<int4>(blkA.size()); z.add<int2>(lrA.size());
  z.add<int4>(blkT.size()); z.add<int2>(lrT.size());
  z.add<int4>(pblkA.size()); z.add<int2>(plrA.size());
  z.add<int4>(pblkT.size()); z.add<int2>(plrT.size());
  for (int i = 0; i < 3; ++i) z.add<double>(vn);
  for (int i = 0; i < 2; ++i) z.add<double>(vm);
  if (prob->primal_start) z.add<double>(vn);
  if (prob->dual_start) z.add<double>(vm);
  P->arena = dev_alloc(z.bytes, st);
  P->bytes = z.bytes;
  Arena ar{(char *)P->arena, 0};
  auto mat = [&](DevCsr &M, int rows, int cols, std::vector<int4> &blk, std::vector<int2> &lr,
                 std::vector<int4> &pblk, std::vector<int2> &plr) {
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
    // register-path kernel variant for matrices of short rows of 16+ non-zeros
    // (tiles of 1024 only); PDLP_SPMV_DIRECT=0/1 overrides the rule
    M.plan.direct = P->tile == 1024 && plan_direct(blk, nnz);
    if (const char *e = getenv("PDLP_SPMV_DIRECT")) M.plan.direct = P->tile == 1024 && atoi(e) != 0;
    M.plan.blk = ar.take<int4>(blk.size());
    M.plan.lrow = ar.take<int2>(lr.size());
    if (!blk.empty())
      PDLP_CUDA(cudaMemcpyAsync(M.plan.blk, blk.data(), blk.size() * 16, cudaMemcpyHostToDevice, st));
    if (!lr.empty())
      PDLP_CUDA(cudaMemcpyAsync(M.plan.lrow, lr.data(), lr.size() * 8, cudaMemcpyHostToDevice, st));
    M.pipe.ntile = (int)pblk.size();
    M.pipe.nlong = (int)plr.size();
    const long cap = (long)nsm * kPipeCtasPerSm;
    M.pipe.grid = (int)(M.pipe.ntile < cap ? M.pipe.ntile : cap);
    M.pipe.blk = ar.take<int4>(pblk.size());
    M.pipe.lrow = ar.take<int2>(plr.size());
    if (!pblk.empty())
      PDLP_CUDA(cudaMemcpyAsync(M.pipe.blk, pblk.data(), pblk.size() * 16, cudaMemcpyHostToDevice, st));
    if (!plr.empty())
      PDLP_CUDA(cudaMemcpyAsync(M.pipe.lrow, plr.data(), plr.size() * 8, cudaMemcpyHostToDevice, st));
  };
  mat(P->A, m, n, blkA, lrA, pblkA, plrA);
  mat(P->AT, n, m, blkT, lrT, pblkT, plrT);
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
  {
    // stable transpose on the device (reference: cusparseCsr2cscEx2,
    // src/pdlp_core_op.cu:109-130), scratch released on this stream
    void *scratch = dev_alloc(device_transpose_scratch_bytes(n, nnz), st);
    device_transpose(m, n, nnz, P->A.ptr, P->A.col, P->A.val, P->AT.ptr, P->AT.col, P->AT.val,
                     scratch, st);
    dev_free(scratch, st);
  }
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
  PDLP_CUDA(cudaStreamSynchronize(st));  // host staging (plans) must outlive the copies
  return P.release();
}


template class Solve<double, double>;

}  // namespace pdlp
