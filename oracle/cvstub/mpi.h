// mpi.h -- TEST INFRASTRUCTURE ONLY: stand-in declaring the one MPI type
// the reference headers name; the UCM sources make no MPI call.
#ifndef GPB_CVSTUB_MPI_H
#define GPB_CVSTUB_MPI_H
typedef int MPI_Datatype;
#endif
