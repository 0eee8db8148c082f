/* Declarations-only stand-in for <mpi.h>, used solely to compile the
 * reference's FunctionOnGPU.cu into a device-code cubin (no host code from
 * that file is linked or run) and its CPU I/O files into the golden-vector
 * generator.  The MPI calls themselves are never executed. */
#ifndef ORACLE_REF_SHIM_MPI_H
#define ORACLE_REF_SHIM_MPI_H
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
#define MPI_COMM_WORLD 0
#define MPI_FLOAT 1
#define MPI_DOUBLE 2
#define MPI_INT 3
#define MPI_CHAR 4
#define MPI_SUM 1
#define MPI_MIN 2
#define MPI_MAX 3
int MPI_Barrier(MPI_Comm);
int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm);
int MPI_Reduce(const void*, void*, int, MPI_Datatype, MPI_Op, int, MPI_Comm);
#endif
