/* Empty stand-in for the PSLP presolve stats header that the reference's
 * public types header includes; no type from it is used on the single-GPU
 * path (the stats field of the result struct is commented out). */
#ifndef PDLP_REF_SHIM_PSLP_STATS_H
#define PDLP_REF_SHIM_PSLP_STATS_H
#endif
