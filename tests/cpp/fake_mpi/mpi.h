/* A stand-in for <mpi.h> in the distributed drop-in's tests (no MPI in
 * this image): a communicator is its number of ranks. */
#ifndef PALIWA_TEST_FAKE_MPI_H
#define PALIWA_TEST_FAKE_MPI_H
typedef int MPI_Comm;
#define MPI_SUCCESS 0
#define MPI_COMM_SELF 1
static inline int MPI_Comm_size(MPI_Comm comm, int *size) {
  *size = comm;
  return MPI_SUCCESS;
}
#endif
