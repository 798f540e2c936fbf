// cli.cpp -- command-line solver: cupdlpx [OPTIONS] <mps_file> <output_dir>
//
// The single-GPU mode of the reference's command-line tool (src/cli.c:32-350):
// the same options, and the same three output files in <output_dir>:
//   <name>_summary.txt          termination reason, time, iterations,
//                               objectives, residuals, gap, sizes
//   <name>_primal_solution.txt  one value per line (%.10g)
//   <name>_dual_solution.txt    one value per line (%.10g)
// where <name> is the file name up to its first '.'.  One addition:
// --precision fp64|fp32|fp32m selects the arithmetic of the PDHG iteration.
#include <getopt.h>
#include <libgen.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>

#include "cupdlpx.h"
#include "mps_parser.h"
#include "pdlp_gb300.h"

namespace {

std::string instance_name(const char *path) {
  std::string copy(path);
  std::string base = basename(&copy[0]);
  size_t dot = base.find('.');
  return dot == std::string::npos ? base : base.substr(0, dot);
}

bool write_vector(const std::string &path, const double *v, int n) {
  FILE *f = fopen(path.c_str(), "w");
  if (!f) {
    perror(("cannot write " + path).c_str());
    return false;
  }
  for (int i = 0; i < n; ++i) fprintf(f, "%.10g\n", v[i]);
  fclose(f);
  return true;
}

bool write_summary(const std::string &path, const cupdlpx_result_t *r) {
  FILE *f = fopen(path.c_str(), "w");
  if (!f) {
    perror(("cannot write " + path).c_str());
    return false;
  }
  fprintf(f, "Termination Reason: %s\n", pdlp_termination_reason_to_string(r->termination_reason));
  fprintf(f, "Runtime (sec): %e\n", r->cumulative_time_sec);
  fprintf(f, "Iterations Count: %d\n", r->total_count);
  fprintf(f, "Primal Objective Value: %e\n", r->primal_objective_value);
  fprintf(f, "Dual Objective Value: %e\n", r->dual_objective_value);
  fprintf(f, "Relative Primal Residual: %e\n", r->relative_primal_residual);
  fprintf(f, "Relative Dual Residual: %e\n", r->relative_dual_residual);
  fprintf(f, "Absolute Objective Gap: %e\n", r->objective_gap);
  fprintf(f, "Relative Objective Gap: %e\n", r->relative_objective_gap);
  fprintf(f, "Rows: %d\n", r->num_constraints);
  fprintf(f, "Columns: %d\n", r->num_variables);
  fprintf(f, "Nonzeros: %d\n", r->num_nonzeros);
  if (r->feasibility_polishing_time > 0.0) {
    fprintf(f, "Feasibility Polishing Time (sec): %e\n", r->feasibility_polishing_time);
    fprintf(f, "Feasibility Polishing Iteration Count: %d\n", r->feasibility_iteration);
  }
  fclose(f);
  return true;
}

void usage(const char *prog) {
  fprintf(stderr,
          "Usage: %s [OPTIONS] <mps_file> <output_dir>\n\n"
          "Arguments:\n"
          "  <mps_file>    problem in MPS format (.mps, or .mps.gz with zlib)\n"
          "  <output_dir>  receives <name>_summary.txt, <name>_primal_solution.txt and\n"
          "                <name>_dual_solution.txt\n\n"
          "Options:\n"
          "  -h, --help                          this message\n"
          "  -v, --verbose                       log the solve\n"
          "      --time_limit <seconds>          default 3600\n"
          "      --iter_limit <iterations>       default %d\n"
          "      --eps_opt <tolerance>           relative optimality, default 1e-4\n"
          "      --eps_feas <tolerance>          relative feasibility, default 1e-4\n"
          "      --eps_infeas_detect <tolerance> infeasibility detection, default 1e-10\n"
          "      --l_inf_ruiz_iter <int>         Ruiz iterations, default 10\n"
          "      --no_pock_chambolle             disable Pock-Chambolle rescaling\n"
          "      --pock_chambolle_alpha <float>  default 1.0\n"
          "      --no_bound_obj_rescaling        disable bound/objective rescaling\n"
          "      --eval_freq <int>               termination evaluation frequency, default 200\n"
          "      --sv_max_iter <int>             power-method iterations, default 5000\n"
          "      --sv_tol <float>                power-method tolerance, default 1e-4\n"
          "  -f, --feasibility_polishing         polish primal and dual feasibility\n"
          "      --eps_feas_polish <tolerance>   polishing tolerance, default 1e-6\n"
          "      --opt_norm <l2|linf>            norm of the optimality criteria, default l2\n"
          "      --no_presolve                   (this library has no presolver)\n"
          "      --precision <fp64|fp32|fp32m>   iteration arithmetic, default fp64\n",
          prog, INT32_MAX);
}

}  // namespace

int main(int argc, char **argv) {
  pdhg_parameters_t p;
  set_default_parameters(&p);
  pdlp_options_t o;
  memset(&o, 0, sizeof(o));
  static const option longopts[] = {{"help", no_argument, 0, 'h'},
                                    {"verbose", no_argument, 0, 'v'},
                                    {"time_limit", required_argument, 0, 1001},
                                    {"iter_limit", required_argument, 0, 1002},
                                    {"eps_opt", required_argument, 0, 1003},
                                    {"eps_feas", required_argument, 0, 1004},
                                    {"eps_infeas_detect", required_argument, 0, 1005},
                                    {"eps_feas_polish", required_argument, 0, 1006},
                                    {"feasibility_polishing", no_argument, 0, 'f'},
                                    {"l_inf_ruiz_iter", required_argument, 0, 1007},
                                    {"pock_chambolle_alpha", required_argument, 0, 1008},
                                    {"no_pock_chambolle", no_argument, 0, 1009},
                                    {"no_bound_obj_rescaling", no_argument, 0, 1010},
                                    {"sv_max_iter", required_argument, 0, 1011},
                                    {"sv_tol", required_argument, 0, 1012},
                                    {"eval_freq", required_argument, 0, 1013},
                                    {"opt_norm", required_argument, 0, 1014},
                                    {"no_presolve", no_argument, 0, 1015},
                                    {"precision", required_argument, 0, 1016},
                                    {0, 0, 0, 0}};
  int c;
  while ((c = getopt_long(argc, argv, "hvf", longopts, nullptr)) != -1) {
    switch (c) {
      case 'h': usage(argv[0]); return 0;
      case 'v': p.verbose = true; break;
      case 1001: p.termination_criteria.time_sec_limit = atof(optarg); break;
      case 1002: p.termination_criteria.iteration_limit = atoi(optarg); break;
      case 1003: p.termination_criteria.eps_optimal_relative = atof(optarg); break;
      case 1004: p.termination_criteria.eps_feasible_relative = atof(optarg); break;
      case 1005: p.termination_criteria.eps_infeasible = atof(optarg); break;
      case 1006: p.termination_criteria.eps_feas_polish_relative = atof(optarg); break;
      case 'f': p.feasibility_polishing = true; break;
      case 1007: p.l_inf_ruiz_iterations = atoi(optarg); break;
      case 1008: p.pock_chambolle_alpha = atof(optarg); break;
      case 1009: p.has_pock_chambolle_alpha = false; break;
      case 1010: p.bound_objective_rescaling = false; break;
      case 1011: p.sv_max_iter = atoi(optarg); break;
      case 1012: p.sv_tol = atof(optarg); break;
      case 1013: p.termination_evaluation_frequency = atoi(optarg); break;
      case 1014:
        if (!strcmp(optarg, "l2")) p.optimality_norm = NORM_TYPE_L2;
        else if (!strcmp(optarg, "linf")) p.optimality_norm = NORM_TYPE_L_INF;
        else {
          fprintf(stderr, "Error: opt_norm must be 'l2' or 'linf'\n");
          return 1;
        }
        break;
      case 1015: p.presolve = false; break;
      case 1016:
        if (!strcmp(optarg, "fp64")) o.precision = PDLP_PRECISION_FP64;
        else if (!strcmp(optarg, "fp32")) o.precision = PDLP_PRECISION_FP32_REFINE;
        else if (!strcmp(optarg, "fp32m")) o.precision = PDLP_PRECISION_FP32_MATRIX;
        else {
          fprintf(stderr, "Error: precision must be fp64, fp32 or fp32m\n");
          return 1;
        }
        break;
      default: return 1;
    }
  }
  if (argc - optind != 2) {
    fprintf(stderr, "Error: You must specify an input file and an output directory.\n\n");
    usage(argv[0]);
    return 1;
  }
  const char *file = argv[optind];
  const std::string dir = argv[optind + 1];
  const std::string name = instance_name(file);
  lp_problem_t *prob = read_mps_file(file);
  if (!prob) {
    fprintf(stderr, "Failed to read or parse the file.\n");
    return 1;
  }
  cupdlpx_result_t *r = pdlp_solve_opts(prob, &p, &o, nullptr);
  int rc = 0;
  if (!r) {
    fprintf(stderr, "Solver failed: %s\n", pdlp_last_error());
    rc = 1;
  } else {
    bool ok = write_summary(dir + "/" + name + "_summary.txt", r);
    ok = write_vector(dir + "/" + name + "_primal_solution.txt", r->primal_solution,
                      prob->num_variables) && ok;
    ok = write_vector(dir + "/" + name + "_dual_solution.txt", r->dual_solution,
                      prob->num_constraints) && ok;
    if (!ok) rc = 1;
    cupdlpx_result_free(r);
  }
  lp_problem_free(prob);
  return rc;
}
