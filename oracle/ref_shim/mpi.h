/* Type-only stand-in for <mpi.h>, used solely to compile the reference's
 * single-GPU host sources for the test oracle (its internal_types.h includes
 * <mpi.h> unconditionally but the single-GPU path calls no MPI function). */
#ifndef PDLP_REF_SHIM_MPI_H
#define PDLP_REF_SHIM_MPI_H
typedef int MPI_Comm;
typedef int MPI_Request;
#endif
