/* Type-only stand-in for the PSLP presolve API header, which the reference
 * does not vendor.  The single-GPU baseline runs with presolve off, so only
 * the names its presolve.h mentions need to exist. */
#ifndef PDLP_REF_SHIM_PSLP_API_H
#define PDLP_REF_SHIM_PSLP_API_H
typedef struct Presolver Presolver;
typedef struct Settings Settings;
enum PresolveStatus_ { PRESOLVE_STATUS_UNUSED = 0 };
#endif
