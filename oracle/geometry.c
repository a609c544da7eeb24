/*
 * FP64 restatement of the reference voxelizer -- TEST ORACLE ONLY.
 *
 * Follows src/geometry/voxelize.ts:1-199 (three parity projections, majority
 * vote, boundaries, counts), src/geometry/wall-links.ts:1-131 (pull masks,
 * q offsets and fractions, body boundary list) and
 * src/geometry/triangle-bins.ts:1-162 (four-cell triangle bins, Moller-Trumbore
 * link intersection) in IEEE binary64, the arithmetic of JavaScript numbers,
 * so the cell flags come out bit for bit as the reference computes them.
 */
#include "pw_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

enum { FLUID = 0, SOLID = 1, SUPPORT = 2, FLOOR = 3, EQ = 4 };
#define NO_Q 0xffffffffu
static const int DIR[19][3] = {{0, 0, 0},  {1, 0, 0},   {-1, 0, 0}, {0, 1, 0},  {0, -1, 0},
                               {0, 0, 1},  {0, 0, -1},  {1, 1, 0},  {-1, -1, 0}, {1, 0, 1},
                               {-1, 0, -1}, {0, 1, 1},  {0, -1, -1}, {1, -1, 0}, {-1, 1, 0},
                               {1, 0, -1}, {-1, 0, 1},  {0, 1, -1}, {0, -1, 1}};

void ov_free(void *p) { free(p); }

/* voxelize.ts:23-25 */
static inline double edge(const double *a, const double *b, double u, double v) {
  return (b[0] - a[0]) * (v - a[1]) - (b[1] - a[1]) * (u - a[0]);
}

/* voxelize.ts:27-30 */
static inline int owns_edge(double value, const double *a, const double *b) {
  return value > 0 || (value == 0 && (b[1] < a[1] || (b[1] == a[1] && b[0] > a[0])));
}

static inline double min3(double a, double b, double c) { double m = a < b ? a : b; return m < c ? m : c; }
static inline double max3(double a, double b, double c) { double m = a > b ? a : b; return m > c ? m : c; }

typedef struct {
  uint32_t *count;  /* hits per column */
  uint32_t *offset; /* start of each column in hits */
  double *hits;
  int filling;
} columns_t;

/* voxelize.ts:32-60; in the counting pass only the number of hits is kept. */
static void rasterize_triangle(const double *a, const double *second, const double *third, int nu,
                               int nv, columns_t *cols) {
  double signed_area = edge(a, second, third[0], third[1]);
  if (signed_area == 0) return;
  const double *b = signed_area > 0 ? second : third;
  const double *c = signed_area > 0 ? third : second;
  double area = fabs(signed_area);
  double lo_u = ceil(min3(a[0], b[0], c[0])), hi_u = floor(max3(a[0], b[0], c[0]));
  double lo_v = ceil(min3(a[1], b[1], c[1])), hi_v = floor(max3(a[1], b[1], c[1]));
  long min_u = lo_u < 0 ? 0 : (long)lo_u;
  long max_u = hi_u > nu - 1 ? nu - 1 : (long)hi_u;
  long min_v = lo_v < 0 ? 0 : (long)lo_v;
  long max_v = hi_v > nv - 1 ? nv - 1 : (long)hi_v;
  for (long v = min_v; v <= max_v; v++) {
    for (long u = min_u; u <= max_u; u++) {
      double wa = edge(b, c, (double)u, (double)v);
      double wb = edge(c, a, (double)u, (double)v);
      double wc = edge(a, b, (double)u, (double)v);
      if (owns_edge(wa, b, c) && owns_edge(wb, c, a) && owns_edge(wc, a, b)) {
        size_t col = (size_t)u + (size_t)nu * (size_t)v;
        if (cols->filling) {
          cols->hits[cols->offset[col] + cols->count[col]] = (wa * a[2] + wb * b[2] + wc * c[2]) / area;
        }
        cols->count[col]++;
      }
    }
  }
}

static int cmp_double(const void *x, const void *y) {
  double a = *(const double *)x, b = *(const double *)y;
  return (a > b) - (a < b);
}

static const int PROJ[3][3] = {{0, 1, 2}, {1, 2, 0}, {2, 0, 1}};

/* voxelize.ts:88-121 */
static int vote_mesh(const float *mesh, uint32_t ntri, const uint32_t size[3], uint32_t *flags,
                     uint32_t type) {
  size_t cells = (size_t)size[0] * size[1] * size[2];
  const size_t strides[3] = {1, size[0], (size_t)size[0] * size[1]};
  uint8_t *votes = (uint8_t *)calloc(cells, 1);
  int watertight = 1;
  for (int p = 0; p < 3; p++) {
    int u = PROJ[p][0], v = PROJ[p][1], axis = PROJ[p][2];
    size_t ncol = (size_t)size[u] * size[v];
    columns_t cols;
    cols.count = (uint32_t *)calloc(ncol, sizeof(uint32_t));
    cols.offset = (uint32_t *)calloc(ncol + 1, sizeof(uint32_t));
    cols.hits = NULL;
    for (int pass = 0; pass < 2; pass++) {
      cols.filling = pass;
      if (pass == 1) {
        size_t total = 0;
        for (size_t k = 0; k < ncol; k++) { cols.offset[k] = (uint32_t)total; total += cols.count[k]; }
        cols.offset[ncol] = (uint32_t)total;
        cols.hits = (double *)malloc((total ? total : 1) * sizeof(double));
        memset(cols.count, 0, ncol * sizeof(uint32_t));
      }
      for (uint32_t t = 0; t < ntri; t++) {
        const float *q = mesh + 9 * (size_t)t;
        double A[3] = {q[u], q[v], q[axis]};
        double B[3] = {q[3 + u], q[3 + v], q[3 + axis]};
        double C[3] = {q[6 + u], q[6 + v], q[6 + axis]};
        rasterize_triangle(A, B, C, (int)size[u], (int)size[v], &cols);
      }
    }
    /* fillColumns, voxelize.ts:62-86 */
    for (size_t col = 0; col < ncol; col++) {
      uint32_t n = cols.count[col];
      if (n == 0) continue;
      double *h = cols.hits + cols.offset[col];
      qsort(h, n, sizeof(double), cmp_double);
      if (n % 2 != 0) watertight = 0;
      size_t base = (col % size[u]) * strides[u] + (col / size[u]) * strides[v];
      for (uint32_t pair = 0; pair + 1 < n; pair += 2) {
        double s0 = ceil(h[pair]), s1 = ceil(h[pair + 1]);
        long start = s0 < 0 ? 0 : (long)s0;
        long end = s1 > (double)size[axis] ? (long)size[axis] : (long)s1;
        for (long c = start; c < end; c++) votes[base + (size_t)c * strides[axis]]++;
      }
    }
    free(cols.count); free(cols.offset); free(cols.hits);
  }
  for (size_t cell = 0; cell < cells; cell++)
    if (votes[cell] >= 2 && flags[cell] == FLUID) flags[cell] = type;
  free(votes);
  return watertight;
}

/* voxelize.ts:123-135 */
static void apply_boundaries(uint32_t *flags, uint32_t nx, uint32_t ny, uint32_t nz, int floor_on) {
  for (uint32_t z = 0; z < nz; z++)
    for (uint32_t y = 0; y < ny; y++) {
      size_t row = (size_t)nx * (y + (size_t)ny * z);
      flags[row] = EQ;
      flags[row + nx - 1] = EQ;
    }
  if (floor_on) {
    for (size_t c = 0; c < (size_t)nx * ny; c++) flags[c] = FLOOR;
    for (size_t c = (size_t)nx * ny * (nz - 1); c < (size_t)nx * ny * nz; c++) flags[c] = EQ;
  }
}

/* ---- triangle bins, triangle-bins.ts:1-162 ---- */
#define BIN 4
typedef struct {
  const float *mesh;
  uint32_t ntri;
  float *bounds;
  uint32_t *bin_start, *bin_items; /* CSR of triangle offsets per bin */
  int nx, ny, nz;
} bins_t;

static void bins_build(bins_t *b, const float *mesh, uint32_t ntri, uint32_t lx, uint32_t ly, uint32_t lz) {
  b->mesh = mesh; b->ntri = ntri;
  b->nx = (int)((lx + BIN - 1) / BIN); b->ny = (int)((ly + BIN - 1) / BIN); b->nz = (int)((lz + BIN - 1) / BIN);
  size_t nb = (size_t)b->nx * b->ny * b->nz;
  b->bounds = (float *)malloc((ntri ? ntri : 1) * 6 * sizeof(float));
  uint32_t *count = (uint32_t *)calloc(nb + 1, sizeof(uint32_t));
  for (int pass = 0; pass < 2; pass++) {
    if (pass == 1) {
      b->bin_start = (uint32_t *)calloc(nb + 1, sizeof(uint32_t));
      size_t total = 0;
      for (size_t k = 0; k < nb; k++) { b->bin_start[k] = (uint32_t)total; total += count[k]; }
      b->bin_start[nb] = (uint32_t)total;
      b->bin_items = (uint32_t *)malloc((total ? total : 1) * sizeof(uint32_t));
      memset(count, 0, (nb + 1) * sizeof(uint32_t));
    }
    for (uint32_t t = 0; t < ntri; t++) {
      const float *p = mesh + 9 * (size_t)t;
      double lo[3], hi[3];
      for (int a = 0; a < 3; a++) {
        double x = p[a], y = p[a + 3], z = p[a + 6];
        lo[a] = min3(x, y, z); hi[a] = max3(x, y, z);
      }
      for (int a = 0; a < 3; a++) { b->bounds[6 * t + a] = (float)lo[a]; b->bounds[6 * t + 3 + a] = (float)hi[a]; }
      long mn[3], mx[3];
      for (int a = 0; a < 3; a++) { mn[a] = (long)floor(lo[a] / BIN); mx[a] = (long)floor(hi[a] / BIN); }
      long z0 = mn[2] < 0 ? 0 : mn[2], z1 = mx[2] > b->nz - 1 ? b->nz - 1 : mx[2];
      long y0 = mn[1] < 0 ? 0 : mn[1], y1 = mx[1] > b->ny - 1 ? b->ny - 1 : mx[1];
      long x0 = mn[0] < 0 ? 0 : mn[0], x1 = mx[0] > b->nx - 1 ? b->nx - 1 : mx[0];
      for (long z = z0; z <= z1; z++)
        for (long y = y0; y <= y1; y++)
          for (long x = x0; x <= x1; x++) {
            size_t k = (size_t)x + (size_t)b->nx * ((size_t)y + (size_t)b->ny * (size_t)z);
            if (pass == 1) b->bin_items[b->bin_start[k] + count[k]] = 9 * t;
            count[k]++;
          }
    }
  }
  free(count);
}

static void bins_free(bins_t *b) { free(b->bounds); free(b->bin_start); free(b->bin_items); }

/* triangle-bins.ts:60-94; returns 1 with *t on a hit */
static int intersection(const float *p, uint32_t offset, const double *o, const double *d, double *t) {
  const double EPS = 1e-9;
  double ax = p[offset], ay = p[offset + 1], az = p[offset + 2];
  double bx = p[offset + 3], by = p[offset + 4], bz = p[offset + 5];
  double cx = p[offset + 6], cy = p[offset + 7], cz = p[offset + 8];
  double e1x = bx - ax, e1y = by - ay, e1z = bz - az;
  double e2x = cx - ax, e2y = cy - ay, e2z = cz - az;
  double px = d[1] * e2z - d[2] * e2y;
  double py = d[2] * e2x - d[0] * e2z;
  double pz = d[0] * e2y - d[1] * e2x;
  double det = e1x * px + e1y * py + e1z * pz;
  if (fabs(det) < 2.220446049250313e-16) return 0;
  double tx = o[0] - ax, ty = o[1] - ay, tz = o[2] - az;
  double u = (tx * px + ty * py + tz * pz) / det;
  if (u < -EPS || u > 1 + EPS) return 0;
  double qx = ty * e1z - tz * e1y;
  double qy = tz * e1x - tx * e1z;
  double qz = tx * e1y - ty * e1x;
  double v = (d[0] * qx + d[1] * qy + d[2] * qz) / det;
  if (v < -EPS || u + v > 1 + EPS) return 0;
  double tt = (e2x * qx + e2y * qy + e2z * qz) / det;
  if (tt >= -EPS && tt <= 1 + EPS) { *t = tt; return 1; }
  return 0;
}

/* triangle-bins.ts:136-161 */
static int nearest_link_hit(const bins_t *b, const double *o, const double *d, double *t) {
  double lo[3], hi[3];
  long mn[3], mx[3];
  for (int a = 0; a < 3; a++) {
    double e = o[a] + d[a];
    lo[a] = o[a] < e ? o[a] : e;
    hi[a] = o[a] > e ? o[a] : e;
    mn[a] = (long)floor(lo[a] / BIN);
    mx[a] = (long)floor(hi[a] / BIN);
  }
  double nearest = INFINITY;
  long z0 = mn[2] < 0 ? 0 : mn[2], z1 = mx[2] > b->nz - 1 ? b->nz - 1 : mx[2];
  long y0 = mn[1] < 0 ? 0 : mn[1], y1 = mx[1] > b->ny - 1 ? b->ny - 1 : mx[1];
  long x0 = mn[0] < 0 ? 0 : mn[0], x1 = mx[0] > b->nx - 1 ? b->nx - 1 : mx[0];
  for (long z = z0; z <= z1; z++)
    for (long y = y0; y <= y1; y++)
      for (long x = x0; x <= x1; x++) {
        size_t k = (size_t)x + (size_t)b->nx * ((size_t)y + (size_t)b->ny * (size_t)z);
        for (uint32_t it = b->bin_start[k]; it < b->bin_start[k + 1]; it++) {
          uint32_t off = b->bin_items[it];
          const float *bd = b->bounds + 6 * (off / 9);
          if (!((double)bd[0] <= hi[0] && (double)bd[3] >= lo[0] && (double)bd[1] <= hi[1] &&
                (double)bd[4] >= lo[1] && (double)bd[2] <= hi[2] && (double)bd[5] >= lo[2]))
            continue;
          double tt;
          if (intersection(b->mesh, off, o, d, &tt) && tt < nearest) nearest = tt;
        }
      }
  if (nearest == INFINITY) return 0;
  *t = nearest;
  return 1;
}

int ov_nearest_link_hit(const float *mesh, uint32_t ntri, uint32_t nx, uint32_t ny, uint32_t nz,
                        const double origin[3], const double dir[3], double *t) {
  bins_t b;
  bins_build(&b, mesh, ntri, nx, ny, nz);
  int hit = nearest_link_hit(&b, origin, dir, t);
  bins_free(&b);
  return hit;
}

/* wall-links.ts:24-28 */
static long neighbour(long x, long y, long z, uint32_t nx, uint32_t ny, uint32_t nz, int floor_on) {
  if (x < 0 || x >= (long)nx || (floor_on && (z < 0 || z >= (long)nz))) return -1;
  return x + (long)nx * ((((y + (long)ny) % (long)ny)) + (long)ny * ((z + (long)nz) % (long)nz));
}

static int is_wall(uint32_t t) { return t >= SOLID && t <= FLOOR; }

int ov_build_wall_links(uint32_t *flags, const float *body, uint32_t ntri, const float *supports,
                        uint32_t nsup, int has_supports, uint32_t nx, uint32_t ny, uint32_t nz,
                        int floor_on, int measure, uint32_t **geometry_out, uint32_t **boundary_out,
                        ov_stats *stats) {
  size_t cells = (size_t)nx * ny * nz;
  /* markWalls, wall-links.ts:34-51 */
  uint8_t *body_boundary = (uint8_t *)calloc(cells, 1);
  for (size_t wall = 0; wall < cells; wall++) {
    uint32_t type = flags[wall] & 7u;
    if (!is_wall(type)) continue;
    long x = (long)(wall % nx), y = (long)((wall / nx) % ny), z = (long)(wall / ((size_t)nx * ny));
    for (int i = 0; i < 19; i++) {
      long fl = neighbour(x + DIR[i][0], y + DIR[i][1], z + DIR[i][2], nx, ny, nz, floor_on);
      if (fl < 0 || (flags[fl] & 7u) != FLUID) continue;
      flags[fl] |= 1u << (3 + i);
      if (type == SOLID) body_boundary[fl] = 1;
    }
  }
  bins_t body_bins, support_bins;
  int have_body_bins = 0, have_support_bins = 0;
  if (measure) { bins_build(&body_bins, body, ntri, nx, ny, nz); have_body_bins = 1; }
  if (has_supports) { bins_build(&support_bins, supports, nsup, nx, ny, nz); have_support_bins = 1; }
  /* count links first */
  size_t nfrac = 0, nb = 0;
  for (size_t cell = 0; cell < cells; cell++) {
    uint32_t flag = flags[cell];
    if ((flag >> 3) == 0) continue;
    nfrac += (size_t)__builtin_popcount(flag >> 3);
    if (body_boundary[cell]) nb++;
  }
  uint32_t *geometry = (uint32_t *)malloc((2 * cells + nfrac) * sizeof(uint32_t));
  uint32_t *boundary = (uint32_t *)malloc((nb ? nb : 1) * sizeof(uint32_t));
  memcpy(geometry, flags, cells * sizeof(uint32_t));
  size_t f = 0, b = 0;
  uint32_t missed = 0;
  for (size_t cell = 0; cell < cells; cell++) {
    uint32_t flag = flags[cell];
    if ((flag >> 3) == 0) { geometry[cells + cell] = NO_Q; continue; }
    geometry[cells + cell] = (uint32_t)f;
    if (body_boundary[cell]) boundary[b++] = (uint32_t)cell;
    long x = (long)(cell % nx), y = (long)((cell / nx) % ny), z = (long)(cell / ((size_t)nx * ny));
    for (int i = 0; i < 19; i++) {
      if ((flag & (1u << (3 + i))) == 0) continue;
      /* linkFraction, wall-links.ts:53-80 */
      double q = 0.5;
      int hit = 1;
      if (have_body_bins) {
        long wall = neighbour(x - DIR[i][0], y - DIR[i][1], z - DIR[i][2], nx, ny, nz, floor_on);
        uint32_t type = flags[wall] & 7u;
        if (type != FLOOR) {
          const bins_t *bins = type == SUPPORT ? (have_support_bins ? &support_bins : NULL) : &body_bins;
          double origin[3] = {(double)(wall % nx) + DIR[i][0], (double)((wall / nx) % ny) + DIR[i][1],
                              (double)(wall / ((long)nx * ny)) + DIR[i][2]};
          double dir[3] = {-DIR[i][0], -DIR[i][1], -DIR[i][2]};
          double t = 0;
          hit = bins ? nearest_link_hit(bins, origin, dir, &t) : 0;
          q = hit ? t : 0.5;
        }
      }
      missed += hit ? 0u : 1u;
      double clamped = q < 1 ? q : 1;
      clamped = clamped > 1e-3 ? clamped : 1e-3;
      float qf = (float)clamped;
      memcpy(&geometry[2 * cells + f], &qf, 4);
      f++;
    }
  }
  if (have_body_bins) bins_free(&body_bins);
  if (have_support_bins) bins_free(&support_bins);
  free(body_boundary);
  *geometry_out = geometry;
  *boundary_out = boundary;
  stats->missed_links = missed;
  stats->geometry_len = 2 * cells + nfrac;
  stats->nboundary = nb;
  return 0;
}

static int valid_mesh(const float *m, uint32_t ntri) {
  for (size_t k = 0; k < 9 * (size_t)ntri; k++)
    if (!isfinite(m[k])) return 0;
  return 1;
}

/* voxelize.ts:172-199 */
int ov_voxelize(const float *body, uint32_t ntri, const float *supports, uint32_t nsup,
                int has_supports, uint32_t nx, uint32_t ny, uint32_t nz, int floor_on,
                int link_fractions, uint32_t **geometry, uint32_t **boundary, ov_stats *stats,
                char *err, size_t errlen) {
  if (nx < 2 || ny < 2 || nz < 2) {
    snprintf(err, errlen, "Grid dimensions must be integers of at least two cells.");
    return -1;
  }
  if (!valid_mesh(body, ntri) || (has_supports && !valid_mesh(supports, nsup))) {
    snprintf(err, errlen, "Mesh coordinates must be finite.");
    return -1;
  }
  size_t cells = (size_t)nx * ny * nz;
  uint32_t size[3] = {nx, ny, nz};
  uint32_t *flags = (uint32_t *)calloc(cells, sizeof(uint32_t));
  int body_closed = vote_mesh(body, ntri, size, flags, SOLID);
  int supports_closed = has_supports ? vote_mesh(supports, nsup, size, flags, SUPPORT) : 1;
  apply_boundaries(flags, nx, ny, nz, floor_on);
  /* countCells, voxelize.ts:137-154 */
  uint8_t *body_proj = (uint8_t *)calloc((size_t)ny * nz, 1);
  uint8_t *wall_proj = (uint8_t *)calloc((size_t)ny * nz, 1);
  uint32_t solid = 0;
  for (size_t c = 0; c < cells; c++) {
    uint32_t t = flags[c] & 7u;
    if (t == SOLID) { solid++; body_proj[c / nx] = 1; }
    if (t == SOLID || t == SUPPORT) wall_proj[c / nx] = 1;
  }
  uint32_t frontal = 0, blocked = 0;
  for (size_t k = 0; k < (size_t)ny * nz; k++) { frontal += body_proj[k]; blocked += wall_proj[k]; }
  free(body_proj); free(wall_proj);
  memset(stats, 0, sizeof(*stats));
  stats->solid_cells = solid;
  stats->frontal_cells = frontal;
  stats->blockage = (double)blocked / ((double)ny * nz);
  stats->watertight = (uint32_t)(body_closed && supports_closed);
  ov_build_wall_links(flags, body, ntri, supports, nsup, has_supports, nx, ny, nz, floor_on,
                      link_fractions, geometry, boundary, stats);
  free(flags);
  return 0;
}
