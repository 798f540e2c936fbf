// solver.cuh -- device-side data of one PDHG solve and the host driver class.
#pragma once

#include <map>
#include <memory>
#include <string>
#include <vector>

#include "common.cuh"
#include "cupdlpx_types.h"
#include "spmv.cuh"

namespace pdlp {

// A sparse matrix resident in HBM (CSR, int32 indices, FP64 values).
struct DevCsr {
  int rows = 0, cols = 0, nnz = 0;
  int *ptr = nullptr, *col = nullptr;
  double *val = nullptr;
  SpmvPlan plan;
};

// Everything a kernel of the iteration needs, passed by value (kernel
// parameter space), so concurrent solves never share a global.
struct Dev {
  int n, m;
  // scaled problem (reference rescale_info_t / solver state)
  const double *c, *lv, *uv, *lc, *uc;
  const double *lvf, *uvf, *lcf, *ucf;  // bound with +-inf replaced by 0
  const double *Dr, *Dc;                // cumulative row / column scaling
  // iterates
  double *x[2], *x0, *xref, *xhat, *lam, *dx, *auxn;
  double *y[2], *y0, *yhat, *dy, *auxm;
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
  double sv_tol;
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
  double *p_pa, *lp_pa;        // power A (2)
  double *p_pr;                // power residual / norm (1 x ew_grid)
  double *pm_v[2], *pm_g;      // power vectors (m, m, n)
  double *p_misc;              // kMiscPart doubles for set-up reductions
};

constexpr int kMiscPart = 4096;

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
// Read-only once built; any number of solves can run from it.
struct DevProblem {
  int m = 0, n = 0, nnz = 0, tile = 0;
  DevCsr A, AT;  // original values; plan scratch (lcnt/lsum) is per solve
  double *c = nullptr, *lv = nullptr, *uv = nullptr, *lc = nullptr, *uc = nullptr;
  double *xs = nullptr, *ys = nullptr;  // warm start (unscaled) or null
  double cnorm_l2 = 0, cnorm_linf = 0, bnorm_l2 = 0, bnorm_linf = 0, c0 = 0;
  void *arena = nullptr;
  size_t bytes = 0;
  ~DevProblem();
};

// Validate, transpose (host), plan and upload.  Throws on a malformed CSR.
DevProblem *upload_problem(const lp_problem_t *prob, cudaStream_t st);

// One single-LP FP64 solve on one stream.
class Solve {
 public:
  Solve(const pdhg_parameters_t &params, cudaStream_t stream, const DevProblem &prob,
        int trace_cap = 0);
  ~Solve();
  // Working copy of the problem, GPU rescaling, finite bounds, warm start.
  void prepare();
  // Power method -> step size; initial primal weight.
  void init_step();
  // Main loop until termination or iteration limit.
  void run();
  // Reduced cost, unscale, copy to a malloc'ed result.
  cupdlpx_result_t *result();

  // Average device time (ms) of the plain-iteration kernels, measured with
  // CUDA events on the solve's stream over `reps` launches each:
  // ms[0] primal step (A^T SpMV + update), ms[1] dual step (A SpMV + update),
  // ms[2] evaluation over A, ms[3] evaluation over A^T.
  void time_kernels(int reps, double *ms);

  // diagnostics
  int power_iterations() const { return pm_iters_; }
  double sigma_max() const { return sigma_max_; }
  std::vector<double> trace() const;
  double rescale_seconds() const { return rescale_sec_; }
  double loop_seconds() const { return loop_sec_; }
  int graph_count() const { return (int)graphs_.size(); }
  long kernel_launches() const { return launches_; }
  const Dev &dev() const { return d_; }
  const DevCsr &A() const { return A_; }
  const DevCsr &AT() const { return AT_; }

 private:
  void alloc();
  void enqueue_iteration(int t, int off, bool capture);
  void enqueue_eval(int t, int off, bool infeas, bool restart_check, bool final_eval);
  cudaGraphExec_t chunk_graph(int t0, int t1);
  void power_method();

  pdhg_parameters_t p_;
  cudaStream_t st_;
  const DevProblem &P_;
  Dev d_{};
  DevCsr A_, AT_;
  void *arena_ = nullptr;
  HostFlag *hflag_ = nullptr;
  int trace_cap_ = 0;
  std::map<std::string, cudaGraphExec_t> graphs_;
  std::vector<cudaGraph_t> raw_graphs_;
  int pm_iters_ = 0;
  double sigma_max_ = 0.0;
  double rescale_sec_ = 0.0, loop_sec_ = 0.0;
  long launches_ = 0;
  bool counting_ = true;
};

// GPU rescaling (precond.cu): Ruiz, Pock-Chambolle, bound/objective scaling
// on the device copies of A, A^T, c, bounds.  Fills Dr, Dc, cb, ob.
void gpu_rescale(const pdhg_parameters_t &p, DevCsr &A, DevCsr &AT, double *c,
                 double *lv, double *uv, double *lc, double *uc, double *Dr,
                 double *Dc, double *cb, double *ob, double *tmp_n, double *tmp_m,
                 double *part, cudaStream_t st);

// Stable transpose of a host CSR (rows of A^T ordered by original row).
void host_transpose(int m, int n, const int *ap, const int *aj, const double *ax,
                    std::vector<int> &tp, std::vector<int> &tj,
                    std::vector<double> &tx);

}  // namespace pdlp
