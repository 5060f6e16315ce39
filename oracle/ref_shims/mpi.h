/* Single-rank stand-in for the MPI calls in the reference's src_par/do_newton.cpp.
 * Test infrastructure only: the oracle's drivers call the serial
 * System_of_eqs::do_newton_seq (src_par/do_newton.cpp:519), never the
 * ScaLAPACK do_newton, so one rank is all that is needed for the file to
 * compile and link.  Implemented in ref_shims.cpp. */
#ifndef KD_REF_SHIM_MPI_H
#define KD_REF_SHIM_MPI_H

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;

#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 1
#define MPI_INT 2
#define MPI_SUM 0
#define MPI_MAX 1
#define MPI_MIN 2
#define MPI_SUCCESS 0

int MPI_Init(int* argc, char*** argv);
int MPI_Finalize(void);
int MPI_Comm_rank(MPI_Comm c, int* rank);
int MPI_Comm_size(MPI_Comm c, int* size);
int MPI_Barrier(MPI_Comm c);
int MPI_Allreduce(const void* in, void* out, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c);
int MPI_Reduce(const void* in, void* out, int n, MPI_Datatype t, MPI_Op op, int root, MPI_Comm c);
int MPI_Allgatherv(const void* in, int n, MPI_Datatype t, void* out, const int* counts, const int* displs,
                   MPI_Datatype rt, MPI_Comm c);
int MPI_Bcast(void* buf, int n, MPI_Datatype t, int root, MPI_Comm c);

#ifdef __cplusplus
}
#endif
#endif
