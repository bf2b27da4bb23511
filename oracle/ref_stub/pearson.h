/* Header for the reference's examples-generated/pearson.c, which ships
 * without one.  Reconstructed from what pearson.c uses: the navigator fields
 * it writes (pearson.c:75-85) and the state arrays it defines (pearson.c:9-10;
 * 600x600 cells stored at offset +2 in a 604x604 box). */
#pragma once
#include <mpi.h>
struct Formura_Navigator {
  int time_step;
  int lower_x, upper_x, offset_x;
  int lower_y, upper_y, offset_y;
};
extern double U[604][604];
extern double V[604][604];
int Formura_Init(struct Formura_Navigator *navi, MPI_Comm comm);
int Formura_Forward(struct Formura_Navigator *navi);
