/* Link stubs for building the reference's host-side code as a test oracle.
 * The GPU driver (optimize) is not built here: there is no GPU in the build
 * container and the reference sources are not present on the GPU machine. */
#include <stddef.h>
typedef struct cupdlpx_result_t_opaque cupdlpx_result_t;
cupdlpx_result_t *optimize(const void *params, const void *prob) {
  (void)params;
  (void)prob;
  return NULL;
}
