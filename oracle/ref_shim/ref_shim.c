/* Link stubs for building the reference's host-side code as a test oracle.
 * The reference's GPU loop (optimize) is not built: the oracle uses only its
 * host-side code (rescaling, converters, defaults, criteria, MPS reader). */
#include <stddef.h>
typedef struct cupdlpx_result_t_opaque cupdlpx_result_t;
cupdlpx_result_t *optimize(const void *params, const void *prob) {
  (void)params;
  (void)prob;
  return NULL;
}
