/*
 * single_process_mpi/mpi.h — the MPI calls of a Formura driver, for one process
 * on one GPU.
 *
 * The reference's drivers include <mpi.h> and call MPI_Init, MPI_Comm_rank,
 * MPI_Barrier and MPI_Finalize around Formura_Init / Formura_Forward
 * (examples/diffusion-main.cpp:1-16, examples/pearson-3d-main.cpp:160-245).
 * On one GPU the engine makes no MPI call (the halo exchange is an in-device
 * periodic wrap), so a driver built with `-I include/single_process_mpi`
 * compiles unchanged without an MPI installation: this header supplies the
 * communicator type (formura_mpi_stub.h) and these calls for a world of one
 * rank.  A build with a real MPI uses that MPI's <mpi.h> instead.
 */
#ifndef FORMURA_SINGLE_PROCESS_MPI_H
#define FORMURA_SINGLE_PROCESS_MPI_H

#include "../formura_mpi_stub.h"

#ifndef MPI_SUCCESS
#define MPI_SUCCESS 0
#endif

static inline int MPI_Init(int *argc, char ***argv) {
  (void)argc;
  (void)argv;
  return MPI_SUCCESS;
}
static inline int MPI_Finalize(void) { return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm comm, int *rank) {
  (void)comm;
  *rank = 0;
  return MPI_SUCCESS;
}
static inline int MPI_Comm_size(MPI_Comm comm, int *size) {
  (void)comm;
  *size = 1;
  return MPI_SUCCESS;
}
static inline int MPI_Barrier(MPI_Comm comm) {
  (void)comm;
  return MPI_SUCCESS;
}

#endif /* FORMURA_SINGLE_PROCESS_MPI_H */
