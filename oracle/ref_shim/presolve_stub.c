/* Link stubs for the presolve entry points that the reference's optimize()
 * names (src/solver.cu:38-48, :115-118).  The baseline always runs with
 * params->presolve = false, so none of them is reached; each reports that
 * presolve is unavailable should it ever be called. */
#include <stdio.h>
#include <stdlib.h>

#include "presolve.h"

cupdlpx_presolve_info_t *pslp_presolve(const lp_problem_t *original_prob,
                                       const pdhg_parameters_t *params) {
  (void)original_prob;
  (void)params;
  fprintf(stderr, "presolve is not available in this baseline build\n");
  exit(2);
}

cupdlpx_result_t *create_result_from_presolve(const cupdlpx_presolve_info_t *info,
                                              const lp_problem_t *original_prob) {
  (void)info;
  (void)original_prob;
  return NULL;
}

const char *get_presolve_status_str(enum PresolveStatus_ status) {
  (void)status;
  return "unavailable";
}

void pslp_postsolve(const cupdlpx_presolve_info_t *info, cupdlpx_result_t *reduced_result,
                    const lp_problem_t *original_prob) {
  (void)info;
  (void)reduced_result;
  (void)original_prob;
}

void cupdlpx_presolve_info_free(cupdlpx_presolve_info_t *info) { (void)info; }
