/* Single-process stand-in for the four MPI calls the reference's MPI RTM
 * program makes (2D-vti-fd+rtm-mpi/Toa_rtm_vti_adcig_cdp.c:242-480).  Rank 0
 * of a world of one: barriers are no-ops and MPI_Reduce(SUM) is a copy.  Used
 * only to compile the reference's own source for the oracle pin. */
#ifndef GEO_MPI_SHIM_H
#define GEO_MPI_SHIM_H
#include <string.h>
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
#define MPI_COMM_WORLD 0
#define MPI_FLOAT 4
#define MPI_SUM 0
static inline int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = 1; return 0; }
static inline int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
static inline int MPI_Reduce(const void *in, void *out, int n, MPI_Datatype t, MPI_Op op, int root, MPI_Comm c)
{ (void)op; (void)root; (void)c; memcpy(out, in, (size_t)n * (size_t)t); return 0; }
#endif
