/* Free-slip lateral faces: the project's option beside the reference's periodic
 * y (and z without a floor) wrap; there is no counterpart in the reference.
 * Test infrastructure: the CPU oracle of the GPU kernels' free-slip rule.
 *
 * slip bit 0: the y faces, bit 1: the z faces.  A link whose pull source lies
 * beyond a slip face reflects specularly at the halfway plane: direction i of
 * cell (x, y, z) then takes post-collision direction k, i with the crossed
 * velocity components reversed, from the in-plane neighbour (source offset with
 * the crossed components zeroed).  Wall links across a slip face do not exist.
 */
#ifndef PW_ORACLE_SLIP_H
#define PW_ORACLE_SLIP_H

static const int SLIP_CX[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0};
static const int SLIP_CY[19] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 1, -1};
static const int SLIP_CZ[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, -1, 1, -1, 1};

static inline int slip_direction(int cx, int cy, int cz) {
  for (int k = 0; k < 19; k++)
    if (SLIP_CX[k] == cx && SLIP_CY[k] == cy && SLIP_CZ[k] == cz) return k;
  return -1;
}

/* Returns 1 when direction i of cell (y, z) is pulled across a slip face; then
 * *k is the reflected direction and (*oy, *oz) the source offsets in y and z
 * (the x offset stays -cx). */
static inline int slip_pull(int slip, int ny, int nz, int y, int z, int i, int *k, int *oy, int *oz) {
  int cy = SLIP_CY[i], cz = SLIP_CZ[i];
  int sy = y - cy, sz = z - cz;
  int ry = (slip & 1) && cy != 0 && (sy < 0 || sy >= ny);
  int rz = (slip & 2) && cz != 0 && (sz < 0 || sz >= nz);
  if (!ry && !rz) return 0;
  *k = slip_direction(SLIP_CX[i], ry ? -cy : cy, rz ? -cz : cz);
  *oy = ry ? 0 : -cy;
  *oz = rz ? 0 : -cz;
  return 1;
}

#endif
