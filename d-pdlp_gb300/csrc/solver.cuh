// solver.cuh -- device-side data of one PDHG solve and the host driver class.
//
// The iteration is templated on T, the type of the matrix values, iterates
// and per-element arithmetic: double for the FP64 path, float for the FP32
// path.  In both, every reduction (KKT, fixed-point error, restart distances,
// power method), every scalar of the control block, the rescaling and the
// unscaling run in FP64.
#pragma once

#include <array>
#include <map>
#include <mutex>
#include <memory>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "common.cuh"
#include "cupdlpx_types.h"
#include "spmv.cuh"
#include "spmv_pipe.cuh"

namespace pdlp {

// A sparse matrix resident in HBM (CSR, int32 indices, values of type T),
// with the plans of the fused kernel and of the pipelined step kernel.
template <class T>
struct DevCsrT {
  int rows = 0, cols = 0, nnz = 0;
  int *ptr = nullptr, *col = nullptr;
  T *val = nullptr;
  SpmvPlan plan;
  PipePlan pipe;
  bool pipe_on = false;  // this matrix's SpMVs run on the pipelined kernel
};
using DevCsr = DevCsrT<double>;

// Everything a kernel of the iteration needs, passed by value (kernel
// parameter space), so concurrent solves never share a global.
template <class T>
struct Dev {
  int n, m;
  // scaled problem (reference rescale_info_t / solver state)
  const T *c, *lv, *uv, *lc, *uc;
  const T *lvf, *uvf, *lcf, *ucf;  // bounds with +-inf replaced by 0
  const double *Dr, *Dc;           // cumulative row / column scaling (FP64)
  // iterates
  T *x[2], *x0, *xref, *xhat, *lam, *dx, *auxn;
  T *y[2], *y0, *yhat, *dy, *auxm;
  Ctl *ctl;
  HostFlag *hflag;  // mapped pinned host memory
  double *trace;
  int trace_cap;
  // constants
  double cb, ob, c0, cnorm, bnorm, rho, one_minus_rho;
  int rho_is_one;
  int F, linf, verbose;
  double eps_opt, eps_feas, eps_inf, time_limit;
  double art, suff, nec, kp, ki, kd, ismooth;
  // stall rule (FP32 rounds of the refinement): once the KKT error is below
  // stall_floor (near the resolution of FP32 iterates), stop when it has not
  // improved by 10% within max(stall_min, stall_frac * t) iterations; above
  // the floor a plateau is ordinary PDHG progress and the round goes on;
  // stall_min = 0 disables the rule
  int stall_min;
  double stall_frac, stall_floor;
  // shifted evaluation (refinement rounds): the solve works on a correction
  // LP centred at (sx, sy); the objectives are then those of the original
  // LP at (sx + x, sy + y), from its objective and finite bounds
  int shifted;
  const double *sx, *sy, *oc, *olcf, *oucf;
  double oc0, sdp_inv, sdd_inv;  // 1/Delta_p, 1/Delta_d of the correction
  // best-iterate snapshot (refinement rounds): copies of x_hat, y_hat, lam
  T *bx, *by, *bl;
  // reduction partials, one buffer per launch site
  int nblkA, nlongA, nblkT, nlongT, ew_grid;
  double *p_pstep, *lp_pstep;  // primal step: sum dx^2
  double *p_dstep, *lp_dstep;  // dual step: sum dy^2
  double *p_fpe, *lp_fpe;      // FPE cross term
  double *p_e1, *lp_e1;        // eval over A (2 fields)
  double *p_e2, *lp_e2;        // eval over A^T (3 fields)
  double *p_i0;                // ray projection maxima (2 x ew_grid)
  double *p_i1, *lp_i1;        // ray over A (2)
  double *p_i2, *lp_i2;        // ray over A^T (3)
  double *p_rs;                // restart distances (2 x ew_grid)
  double *p_misc;              // kMiscPart doubles for set-up reductions
  // feasibility polishing (reference src/pdlp_core_op.cu:861-1360): 0 for a
  // solve, 1 / 2 for the primal / dual feasibility problem, which evaluate
  // and restart one side only; c_obj / x_obj are the objective and primal
  // point the objective terms use (c and x_hat, or the solve's for polishing)
  int polish;
  double eps_polish;
  const T *c_obj, *x_obj;
  // Halpern weights w_k = (k+1)/(k+2) for k < hw_len, filled once per solve
  // so the iteration kernels load them instead of dividing per block
  const double *hw;
  int hw_len;
};

// The power method always runs in FP64 on the FP64 scaled matrix.
struct PowDev {
  int n, m;
  Ctl *ctl;
  HostFlag *hflag;
  double *v[2], *g;
  double *p_pa, *lp_pa, *p_pr;
  int nblkA, nlongA, ew_grid;
  double sv_tol;
};

constexpr int kMiscPart = 4096;
constexpr int kHalpernTable = 1 << 16;

// Termination reason of an FP32 refinement round that stopped improving;
// internal, never returned to callers.
constexpr int kReasonStalled = 100;

// Host flags describing one iteration of the reference driver loop
// (reference src/solver.cu:58-103).
struct IterFlags {
  bool eval, infeas, restart_check, maybe_restart, major_kernel, fpe, fpe_restart_only;
};

inline IterFlags iteration_flags(int t, int F) {
  IterFlags f;
  bool top_major = t > 0 && t % F == 0;  // is_this_major_iteration at loop top
  f.eval = top_major || t == 0 || t % print_frequency(t) == 0;
  f.infeas = top_major && t < 3 * F;
  f.restart_check = top_major || t == 0;
  f.maybe_restart = f.restart_check && t >= F;
  bool major_next = ((long)t + 1) % F == 0;
  f.major_kernel = major_next || ((long)t + 2) % print_frequency(t + 2) == 0;
  f.fpe = major_next || f.maybe_restart;
  f.fpe_restart_only = !major_next && f.maybe_restart;
  return f;
}

// An LP resident in HBM, as the caller gave it (unscaled): A and its
// transpose in CSR with their SpMV plans, bounds, objective, warm start.
// Read-only once built; any number of solves can run from it.  A derived
// problem (refinement) shares the matrices of its parent and owns only its
// vectors.
struct DevProblem {
  int m = 0, n = 0, nnz = 0, tile = 0;
  DevCsr A, AT;  // original values; plan scratch (lcnt/lsum) is per solve
  double *c = nullptr, *lv = nullptr, *uv = nullptr, *lc = nullptr, *uc = nullptr;
  double *xs = nullptr, *ys = nullptr;  // warm start (unscaled) or null
  double cnorm_l2 = 0, cnorm_linf = 0, bnorm_l2 = 0, bnorm_linf = 0, c0 = 0;
  // correction LP of a refinement round: centre and original objective data
  const double *shift_x = nullptr, *shift_y = nullptr, *orig_c = nullptr;
  const double *orig_lcf = nullptr, *orig_ucf = nullptr;
  double orig_c0 = 0;
  double delta_p = 1.0, delta_d = 1.0;  // correction scalings (x - xbar) Delta_p, ...
  void *arena = nullptr;  // owned device memory (null for a view)
  size_t bytes = 0;
  // Stream the arena is released on: the stream that uploaded it, so on an
  // error path (uploads or solve kernels still queued there) the release is
  // ordered after that work.  A handle that outlives its upload stream
  // (pdlp_device_problem_t) switches to the per-thread stream: its solves
  // return only after their work on the problem has finished.
  cudaStream_t owner = cudaStreamPerThread;
  // SpMV kernel per matrix and precision (index: 0 FP64, 1 FP32, 2 FP32
  // matrix), chosen by the first solve of each precision: -1 not yet
  // chosen, 0 fused, 1 pipelined; {A, A^T}
  mutable int kernel_choice[3][2] = {{-1, -1}, {-1, -1}, {-1, -1}};
  // fingerprint of the structure the kernel choice depends on: m, n, nnz
  // and the row lengths of A and A^T (FNV-1a over both row-pointer arrays)
  uint64_t shape_key = 0;
  mutable std::mutex tune_mu;
  ~DevProblem();
};

// Validate, transpose (host), plan and upload.  Throws on a malformed CSR.
DevProblem *upload_problem(const lp_problem_t *prob, cudaStream_t st);

// Kernel choices of this process by structure fingerprint and precision
// index: every problem of one structure runs the kernels the first timed
// solve of that structure chose.  lookup fills c and returns true when a
// choice is recorded; settle records c unless one is already recorded, and
// returns the recorded choice in c.
bool lookup_kernel_choice(uint64_t key, int prec, int c[2]);
void settle_kernel_choice(uint64_t key, int prec, int c[2]);

// KKT measures of a point, in the reference's definitions.
struct Kkt {
  double abs_p, rel_p, abs_d, rel_d, pobj, dobj, gap, rel_gap;
};

// One single-LP solve on one stream.  T is the type of the iterates and of
// the per-element update arithmetic, M the type of the matrix values and of
// the SpMV products and accumulation:
//   <double, double>  FP64 path (the reference's arithmetic)
//   <float,  float>   FP32 path (iterates and SpMVs in FP32)
//   <double, float>   FP32 matrix and SpMVs, FP64 iterates and updates
// Reductions, control scalars, rescaling and unscaling are FP64 in all three.
template <class T, class M = T>
class Solve {
 public:
  Solve(const pdhg_parameters_t &params, cudaStream_t stream, const DevProblem &prob,
        int trace_cap = 0);
  // Use these bound / objective scalings instead of the reference rule
  // (before prepare()).
  void set_fixed_scaling(double cb, double ob) {
    fixed_cb_ = cb;
    fixed_ob_ = ob;
  }
  // Enable the stall rule (before run()).
  void set_stall_rule(int min_iters, double frac, double floor) {
    d_.stall_min = min_iters;
    d_.stall_frac = frac;
    d_.stall_floor = floor;
  }
  ~Solve();
  // Working copy of the problem, GPU rescaling, finite bounds, warm start.
  void prepare();
  // Power method -> step size (skipped when known_sigma > 0); initial primal
  // weight (known_omega > 0 overrides the reference's choice).
  void init_step(double known_sigma = 0.0, double known_omega = 0.0);
  // Keep the best-KKT iterate of the run (refinement rounds); result_device
  // then returns it.  Call before run().
  void enable_snapshot();
  // scalings and final primal weight (after prepare / run)
  double cb() const { return d_.cb; }
  double ob() const { return d_.ob; }
  double primal_weight() const;
  // Main loop until termination or iteration limit.
  void run();
  // Reduced cost, unscale, copy to a malloc'ed result.
  cupdlpx_result_t *result();
  // Unscaled FP64 primal, dual and dual slack into device buffers.
  void result_device(double *x, double *y, double *lam);
  // KKT of the given unscaled point (device buffers) on this solve's problem;
  // meaningful for a solve prepared without rescaling.
  Kkt evaluate(const double *x, const double *y, const double *lam);
  // Average device time (ms) of the plain-iteration kernels, measured with
  // CUDA events on the solve's stream over `reps` launches each:
  // ms[0] primal step (A^T SpMV + update), ms[1] dual step (A SpMV + update),
  // ms[2] evaluation over A, ms[3] evaluation over A^T.
  void time_kernels(int reps, double *ms);

  // In-loop timing of the plain iteration kernels: in every 100-iteration
  // chunk one ordinary iteration's primal and dual launches are bracketed by
  // CUDA events captured into the chunk graph; the averages cover the chunks
  // that ran before termination (after run()).
  double live_primal_ms() const;
  double live_dual_ms() const;
  int live_samples() const;

  // Feasibility polishing (reference src/pdlp_core_op.cu:861-1360).  After
  // prepare() and init_step(main's sigma, w0): turn this solve into the
  // primal (mode 1: objective 0, dual iterates 0) or dual (mode 2: finite
  // bounds 0, primal iterates 0) feasibility problem of `main`, starting
  // from main's final iterates.
  void polish_init(const Solve &main, int mode);
  // Take a successful polish's point and residuals (mode 1 primal, 2 dual);
  // finish_polish() then recomputes the gap from the objectives.
  void adopt_polish(const Solve &ps, int mode);
  void finish_polish();
  // FP64 KKT scalars of the last evaluation (scaled problem, original units)
  Kkt last_kkt() const;

  // diagnostics
  int power_iterations() const { return pm_iters_; }
  double sigma_max() const { return sigma_max_; }
  std::vector<double> trace() const;
  double rescale_seconds() const { return rescale_sec_; }
  double loop_seconds() const { return loop_sec_; }
  int graph_count() const { return (int)graphs_.size(); }
  long kernel_launches() const { return launches_; }
  // termination reason and iteration count after run()
  int reason() const;
  int total_count() const;
  const Dev<T> &dev() const { return d_; }
  const DevCsrT<M> &A() const { return A_; }
  const DevCsr &A64() const { return A64_; }
  // scaled FP64 vectors (valid after prepare)
  const double *c64() const { return c64_; }
  const double *lv64() const { return lv64_; }
  const double *uv64() const { return uv64_; }
  const double *lc64() const { return lc64_; }
  const double *uc64() const { return uc64_; }

 private:
  void alloc();
  // schedule of iteration t (polishing never runs infeasibility detection)
  IterFlags flags(int t) const {
    IterFlags f = iteration_flags(t, d_.F);
    if (d_.polish) f.infeas = false;
    return f;
  }
  void read_ctl(Ctl &c) const {
    PDLP_CUDA(cudaMemcpyAsync(&c, d_.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st_));
    PDLP_CUDA(cudaStreamSynchronize(st_));
  }
  void enqueue_iteration(int t, int off, bool timed = false);
  void enqueue_eval(int off, bool infeas, bool restart_check, int mode);
  cudaGraphExec_t chunk_graph(int t0, int t1);
  int timed_iteration(int t0, int t1) const;
  void read_timing(int slot);
  void power_method();
  void check_pipe_errors() const;
  // kernel choice per matrix: apply (pipe_A, pipe_T) to the matrices and the
  // fold counts; tune_kernels times both kernels on the step epilogues
  void apply_kernels(bool pipe_A, bool pipe_T);
  void tune_kernels();
  int precision_index() const { return sizeof(T) == 4 ? 1 : sizeof(M) == 4 ? 2 : 0; }
  bool tuned_ = false;

 public:
  // kernels per matrix after tuning (pipelined or not) and the tuning's
  // measured ms per launch: {A fused, A pipelined, A^T fused, A^T pipelined}
  // (zeros when the choice came from the problem's cache or an override)
  bool pipe_A() const { return A64_.pipe_on; }
  bool pipe_AT() const { return AT64_.pipe_on; }
  double tune_ms(int i) const { return tune_ms_[i]; }

 private:
  double tune_ms_[4] = {0, 0, 0, 0};

  pdhg_parameters_t p_;
  cudaStream_t st_;
  const DevProblem &P_;
  Dev<T> d_{};
  PowDev pw_{};
  DevCsr A64_, AT64_;   // FP64 scaled working copies (rescaling, power method)
  DevCsrT<M> A_, AT_;   // iteration matrices (== A64_/AT64_ for M = double)
  double *c64_ = nullptr, *lv64_ = nullptr, *uv64_ = nullptr, *lc64_ = nullptr,
         *uc64_ = nullptr;
  double *outx_ = nullptr, *outy_ = nullptr, *outl_ = nullptr;  // FP64 results
  void *arena_ = nullptr;
  HostFlag *hflag_ = nullptr;
  int trace_cap_ = 0;
  std::map<std::string, cudaGraphExec_t> graphs_;
  // timing: the 3 event-record nodes of each timed chunk graph, pointed at
  // the events of the chunk's parity slot before each launch
  std::map<cudaGraphExec_t, std::array<cudaGraphNode_t, 3>> tnodes_;
  cudaEvent_t tev_[2][3] = {};
  int tpending_[2] = {-1, -1};  // timed iteration recorded in each slot
  struct TimingSample {
    int t;
    float primal_ms, dual_ms;
  };
  std::vector<TimingSample> tsamples_;
  int final_count_ = 0;
  std::vector<cudaGraph_t> raw_graphs_;
  int pm_iters_ = 0;
  double sigma_max_ = 0.0;
  double rescale_sec_ = 0.0, loop_sec_ = 0.0;
  long launches_ = 0;
  bool snapshot_ = false;
  void *snap_mem_ = nullptr;
  double fixed_cb_ = 0.0, fixed_ob_ = 0.0;
};

extern template class Solve<double, double>;
extern template class Solve<float, float>;
extern template class Solve<double, float>;

// GPU rescaling (precond.cu): Ruiz, Pock-Chambolle, bound/objective scaling
// on the device copies of A, A^T, c, bounds.  Fills Dr, Dc, cb, ob.
void gpu_rescale(const pdhg_parameters_t &p, DevCsr &A, DevCsr &AT, double *c,
                 double *lv, double *uv, double *lc, double *uc, double *Dr,
                 double *Dc, double *cb, double *ob, double *tmp_n, double *tmp_m,
                 double *part, cudaStream_t st, double fixed_cb = 0.0,
                 double fixed_ob = 0.0);

// Host buffer whose elements are left uninitialised on resize (filled
// right after, by several threads: no serial zero-fill first).
template <class T>
struct uninit_alloc : std::allocator<T> {
  template <class U>
  struct rebind {
    using other = uninit_alloc<U>;
  };
  template <class U>
  void construct(U *) noexcept {}
  template <class U, class... Args>
  void construct(U *p, Args &&...args) {
    ::new ((void *)p) U(std::forward<Args>(args)...);
  }
};
template <class T>
using host_buf = std::vector<T, uninit_alloc<T>>;

// Stable transpose of a device CSR (rows of A^T ordered by original row),
// bit for bit the host transpose below; scratch of
// device_transpose_scratch_bytes(n, nnz) bytes, all work on stream st.
size_t device_transpose_scratch_bytes(int n, int nnz);
void device_transpose(int m, int n, int nnz, const int *ptr, const int *col, const double *val,
                      int *tptr, int *tcol, double *tval, void *scratch, cudaStream_t st);

// Stable transpose of a host CSR (rows of A^T ordered by original row).
void host_transpose(int m, int n, const int *ap, const int *aj, const double *ax,
                    std::vector<int> &tp, host_buf<int> &tj, host_buf<double> &tx);

// Options of the mixed-precision solve (refine.cu).
struct RefineOptions {
  int max_rounds = 8;       // outer refinement rounds
  double inner_eps = 0.0;   // tolerance of each FP32 solve (0: automatic)
  bool fp64_iterates = false;  // rounds run Solve<double, float> instead of <float, float>
};

struct RefineReport {
  int kernel_A = 0, kernel_AT = 0;  // SpMV kernels of the FP32 rounds (1: pipelined)
  double tune_ms[4] = {0, 0, 0, 0};
  int rounds = 0;
  int power_iterations = 0;
  double sigma_max = 0.0;
  long inner_iterations = 0;
  long kernel_launches = 0;
  double seconds = 0.0;
  Kkt kkt{};
  bool fp64_finish = false;  // the last round ran FP64 PDHG from the best point
  // in-loop kernel timing summed over the FP32 rounds (ms x chunks)
  double timed_primal_ms_sum = 0.0, timed_dual_ms_sum = 0.0;
  int timed_chunks = 0;
};

// FP32 PDHG with FP64 iterative refinement on a resident problem; returns
// a result in the layout of solve_lp_problem.
cupdlpx_result_t *solve_refined(const DevProblem &P, const pdhg_parameters_t &params,
                                const RefineOptions &opt, cudaStream_t st,
                                RefineReport *report);

}  // namespace pdlp
