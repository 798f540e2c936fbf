/*
 * mps_parser.h -- MPS reader of the GB300 solver.
 *
 * Replaces reference include/mps_parser.h:21 (src/mps_parser.c:365-777):
 * same entry point and reading of the free-format MPS file (.mps, and .mps.gz
 * where the library was built with zlib).  The problem is returned as a
 * minimisation (OBJSENSE MAX negates the objective and its constant) and is
 * freed with lp_problem_free.  NULL when the file cannot be opened or parsed.
 */
#ifndef PDLP_GB300_MPS_PARSER_H
#define PDLP_GB300_MPS_PARSER_H

#include "cupdlpx_types.h"

#ifdef __cplusplus
extern "C" {
#endif

lp_problem_t *read_mps_file(const char *filename);

#ifdef __cplusplus
}
#endif
#endif
