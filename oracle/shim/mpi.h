/* Test infrastructure (oracle): single-rank stand-in for the MPI calls made by
 * the reference's solver.cpp / FFT.cpp / parallel.cpp, so those files compile
 * unmodified into the CPU oracle.  One rank only: MPI_Alltoall is a copy. */
#pragma once
#include <cstddef>
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Info;
#define MPI_COMM_WORLD 0
#define MPI_INFO_NULL 0
#define MPI_DOUBLE 8
#define MPI_UNSIGNED 4
#define MPI_DOUBLE_COMPLEX 16
int MPI_Init(int *argc, char ***argv);
int MPI_Finalize();
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Comm_split(MPI_Comm comm, int color, int key, MPI_Comm *out);
int MPI_Barrier(MPI_Comm comm);
int MPI_Bcast(void *buf, int count, MPI_Datatype type, int root, MPI_Comm comm);
int MPI_Alltoall(const void *send, int scount, MPI_Datatype stype, void *recv, int rcount,
                 MPI_Datatype rtype, MPI_Comm comm);
int MPI_Abort(MPI_Comm comm, int code);
double MPI_Wtime();
