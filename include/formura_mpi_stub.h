/*
 * formura_mpi_stub.h — the MPI_Comm type for one-GPU builds without MPI.
 *
 * Formura's generated header includes <mpi.h> only for the MPI_Comm type of
 * Formura_Init's second argument and of Formura_Navigator::mpi_comm
 * (src/Formura/MPICxx/Translate.hs:1011, 1042, 1070).  On one GPU the halo
 * exchange is an in-device periodic wrap, so no MPI call is made and the
 * communicator is stored but never used.  The emitted host code is compiled
 * with this stub; code that includes a real <mpi.h> first keeps that
 * definition (the engine never dereferences the field).
 */
#ifndef FORMURA_MPI_STUB_H
#define FORMURA_MPI_STUB_H
#if !defined(MPI_VERSION) && !defined(FORMURA_HAVE_MPI_COMM)
#define FORMURA_HAVE_MPI_COMM 1
typedef int MPI_Comm;
#ifndef MPI_COMM_WORLD
#define MPI_COMM_WORLD 0
#endif
#endif
#endif
