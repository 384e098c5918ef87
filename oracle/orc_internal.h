/* ORACLE internals shared between orc_dg.c and orc_weno.c (test
 * infrastructure only). */
#ifndef MCFD_ORACLE_ORC_INTERNAL_H_
#define MCFD_ORACLE_ORC_INTERNAL_H_

#include <stdint.h>

#include "orc.h"

int orc_mesh_degree(const orc_mesh *m);
int64_t orc_mesh_cells(const orc_mesh *m);
int64_t orc_mesh_faces(const orc_mesh *m);
const int64_t *orc_mesh_face_cells(const orc_mesh *m);
const double *orc_mesh_face_shift(const orc_mesh *m);
/* Hex8 LocalToGlobal(0, 0, 0) of every cell, [cells][3]. */
void orc_cell_centers(const orc_mesh *m, double *center);

#endif /* MCFD_ORACLE_ORC_INTERNAL_H_ */
