/* Single-rank stand-in for the MPI subset that the Landau-Poisson reference
 * (source/LP_ompi.h:18) includes.  It exists only so the reference's own C++
 * sources compile here, unmodified, as a test oracle: with one rank every
 * collective is the identity, point-to-point sends have no receiver (the
 * reference only sends from ranks >= 1), and MPI_Wtime is omp_get_wtime.
 * Test infrastructure, never part of the shipped library. */
#ifndef LP_SHIM_MPI_H
#define LP_SHIM_MPI_H
#include <omp.h>
#include <stddef.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 1
#define MPI_INT 2
#define MPI_THREAD_SINGLE 0
#define MPI_THREAD_FUNNELED 1
#define MPI_THREAD_SERIALIZED 2
#define MPI_THREAD_MULTIPLE 3
#define MPI_SUCCESS 0

static inline int MPI_Init_thread(int *argc, char ***argv, int required, int *provided)
{ (void)argc; (void)argv; *provided = required; return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return MPI_SUCCESS; }
static inline int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = 1; return MPI_SUCCESS; }
static inline int MPI_Finalize(void) { return MPI_SUCCESS; }
static inline int MPI_Barrier(MPI_Comm c) { (void)c; return MPI_SUCCESS; }
static inline int MPI_Bcast(void *b, int n, MPI_Datatype t, int root, MPI_Comm c)
{ (void)b; (void)n; (void)t; (void)root; (void)c; return MPI_SUCCESS; }
static inline int MPI_Send(const void *b, int n, MPI_Datatype t, int dst, int tag, MPI_Comm c)
{ (void)b; (void)n; (void)t; (void)dst; (void)tag; (void)c; return MPI_SUCCESS; }
static inline int MPI_Recv(void *b, int n, MPI_Datatype t, int src, int tag, MPI_Comm c, MPI_Status *s)
{ (void)b; (void)n; (void)t; (void)src; (void)tag; (void)c; (void)s; return MPI_SUCCESS; }
static inline double MPI_Wtime(void) { return omp_get_wtime(); }
#endif
