/* Stand-in for <mpi.h> so that the reference's generated C compiles without
 * MPI.  The generated examples-generated/pearson.c names MPI_Comm only as the
 * type of Formura_Init's second argument; it makes no MPI call. */
#pragma once
typedef int MPI_Comm;
