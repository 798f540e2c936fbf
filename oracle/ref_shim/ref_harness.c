/* ref_harness.c -- plain-argument wrappers around the reference's own
 * scalar decisions, so the tests can compare the oracle with them.
 *
 * Test infrastructure only: linked into oracle/_ref/libref_host.so together
 * with the reference's sources, which exist only in the build container.
 * check_termination_criteria and should_do_adaptive_restart (reference
 * src/utils.cu:239-293) read a handful of pdhg_solver_state_t fields; each
 * wrapper fills those fields of a zeroed state and returns the decision. */
#include <stdlib.h>

#include "internal_types.h"
#include "utils.h"

int ref_h_termination(const termination_criteria_t *tc, double rel_p, double rel_d,
                      double rel_gap, double dray_obj, double max_dray, double pray_obj,
                      double max_pray, int total, double cum_time) {
  pdhg_solver_state_t *s = (pdhg_solver_state_t *)calloc(1, sizeof(*s));
  if (!s) return -1;
  s->relative_primal_residual = rel_p;
  s->relative_dual_residual = rel_d;
  s->relative_objective_gap = rel_gap;
  s->dual_ray_objective = dray_obj;
  s->max_dual_ray_infeasibility = max_dray;
  s->primal_ray_linear_objective = pray_obj;
  s->max_primal_ray_infeasibility = max_pray;
  s->total_count = total;
  s->cumulative_time_sec = cum_time;
  s->termination_reason = TERMINATION_REASON_UNSPECIFIED;
  check_termination_criteria(s, tc);
  int r = (int)s->termination_reason;
  free(s);
  return r;
}

int ref_h_restart(const restart_parameters_t *rp, int F, int total, int inner, double fpe,
                  double init_fpe, double *last_fpe) {
  pdhg_solver_state_t *s = (pdhg_solver_state_t *)calloc(1, sizeof(*s));
  if (!s) return -1;
  s->total_count = total;
  s->inner_count = inner;
  s->fixed_point_error = fpe;
  s->initial_fixed_point_error = init_fpe;
  s->last_trial_fixed_point_error = *last_fpe;
  int r = should_do_adaptive_restart(s, rp, F) ? 1 : 0;
  *last_fpe = s->last_trial_fixed_point_error;
  free(s);
  return r;
}
