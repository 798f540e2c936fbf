/* Type-only stand-in for <nccl.h>, used solely to compile the reference's
 * single-GPU sources as a baseline: its internal_types.h includes <nccl.h>
 * unconditionally, but the single-GPU solve calls no NCCL function. */
#ifndef PDLP_REF_SHIM_NCCL_H
#define PDLP_REF_SHIM_NCCL_H
typedef struct ncclComm *ncclComm_t;
#endif
