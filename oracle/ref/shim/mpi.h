/* Stand-in for mpi.h (oracle/_ref only): one process, rank 0 of 1. */
#ifndef ORACLE_REF_SHIM_MPI_H
#define ORACLE_REF_SHIM_MPI_H
typedef int MPI_Comm;
#define MPI_COMM_WORLD 0
static inline int MPI_Comm_rank(MPI_Comm c, int* r) { (void)c; *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int* s) { (void)c; *s = 1; return 0; }
static inline int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
static inline int MPI_Init(int* argc, char*** argv) { (void)argc; (void)argv; return 0; }
static inline int MPI_Finalize(void) { return 0; }
#endif
