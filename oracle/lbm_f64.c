/*
 * FP64 restatement of the reference's CPU solver -- TEST ORACLE ONLY.
 *
 * Follows src/lbm/reference/cpu-solver.ts:1-323 (CpuSolver: sources table,
 * wall links, Bouzidi wall values, EQ/outlet cells, momentum exchange) and
 * src/lbm/reference/collision.ts:1-224 (equilibrium, moments, TRT/BGK/REG
 * collisions with optional Smagorinsky tau, the Werner-Wengle wall cell) in
 * IEEE binary64, the arithmetic of JavaScript numbers.
 */
#include "pw_oracle.h"
#include "slip.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static const int CX[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0};
static const int CY[19] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 1, -1};
static const int CZ[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, -1, 1, -1, 1};
static const double WD[19] = {1.0 / 3,  1.0 / 18, 1.0 / 18, 1.0 / 18, 1.0 / 18,
                              1.0 / 18, 1.0 / 18, 1.0 / 36, 1.0 / 36, 1.0 / 36,
                              1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36,
                              1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36};
enum { FLUID = 0, SOLID = 1, SUPPORT = 2, FLOOR = 3, EQ = 4 };
enum { OP_TRT = 0, OP_REG = 1, OP_BGK = 2 };
#define NO_Q 0xffffffffu
static const double LAMBDA = 3.0 / 16.0;
static const double SMAGORINSKY_CS = 0.1;
static const double HALFWAY_Q = 0.5;

static inline int opp(int i) { return i == 0 ? 0 : ((i & 1) ? i + 1 : i - 1); }

typedef struct { double xx, yy, zz, xy, xz, yz; } stress_t;

/* collision.ts:21-32 */
void oc_equilibrium(double *target, double rho, const double u[3]) {
  double ux = u[0], uy = u[1], uz = u[2];
  double speed_squared = ux * ux + uy * uy + uz * uz;
  for (int i = 0; i < 19; i++) {
    double cu = CX[i] * ux + CY[i] * uy + CZ[i] * uz;
    target[i] = WD[i] * (rho - 1 + rho * (3 * cu + 4.5 * cu * cu - 1.5 * speed_squared));
  }
}

/* collision.ts:34-47 */
void oc_moments(const double *g, double out[4]) {
  double rho = 1, ux = 0, uy = 0, uz = 0;
  for (int i = 0; i < 19; i++) {
    rho += g[i];
    ux += CX[i] * g[i];
    uy += CY[i] * g[i];
    uz += CZ[i] * g[i];
  }
  out[0] = rho; out[1] = ux / rho; out[2] = uy / rho; out[3] = uz / rho;
}

/* collision.ts:49-66 */
static stress_t non_equilibrium_stress(const double *g, const double *geq) {
  stress_t s = {0, 0, 0, 0, 0, 0};
  for (int i = 0; i < 19; i++) {
    double cx = CX[i], cy = CY[i], cz = CZ[i];
    double neq = g[i] - geq[i];
    s.xx += cx * cx * neq;
    s.yy += cy * cy * neq;
    s.zz += cz * cz * neq;
    s.xy += cx * cy * neq;
    s.xz += cx * cz * neq;
    s.yz += cy * cz * neq;
  }
  return s;
}

/* collision.ts:68-74 */
static double relaxation_time(double tau0, double rho, stress_t s) {
  double q = s.xx * s.xx + s.yy * s.yy + s.zz * s.zz + 2 * (s.xy * s.xy + s.xz * s.xz + s.yz * s.yz);
  double cs2 = SMAGORINSKY_CS * SMAGORINSKY_CS;
  return 0.5 * (tau0 + sqrt(tau0 * tau0 + (18 * 1.4142135623730951 * cs2 * sqrt(q)) / rho));
}

/* collision.ts:77-96 */
static void regularize(double *g, const double *geq, double rho, double omega_plus, stress_t s,
                       const double *force_terms) {
  double trace_third = (s.xx + s.yy + s.zz) / 3;
  for (int i = 0; i < 19; i++) {
    double cx = CX[i], cy = CY[i], cz = CZ[i];
    double projected = cx * cx * s.xx + cy * cy * s.yy + cz * cz * s.zz +
                       2 * (cx * cy * s.xy + cx * cz * s.xz + cy * cz * s.yz) - trace_third;
    double force = i == 0 ? 0 : rho * force_terms[i];
    g[i] = geq[i] + (1 - omega_plus) * 4.5 * WD[i] * projected + force;
  }
}

/* collision.ts:99-119 */
static void relax_pairs(double *g, const double *geq, double rho, double omega_plus,
                        double omega_minus, const double *force_terms) {
  g[0] = g[0] - omega_plus * (g[0] - geq[0]);
  for (int i = 1; i < 19; i += 2) {
    int j = i + 1;
    double gi = g[i], gj = g[j], eqi = geq[i], eqj = geq[j];
    double even = 0.5 * omega_plus * (gi + gj - eqi - eqj);
    double odd = 0.5 * omega_minus * (gi - gj - eqi + eqj);
    g[i] = gi - even - odd + rho * force_terms[i];
    g[j] = gj - even + odd + rho * force_terms[j];
  }
}

/* collision.ts:122-140 */
void oc_collide(double *g, const double *geq, double rho, double tau0, int op, int les,
                const double *force_terms) {
  int need_stress = les || op == OP_REG;
  stress_t s = {0, 0, 0, 0, 0, 0};
  if (need_stress) s = non_equilibrium_stress(g, geq);
  double tau = (les && need_stress) ? relaxation_time(tau0, rho, s) : tau0;
  double omega_plus = 1 / tau;
  if (op == OP_REG && need_stress) {
    regularize(g, geq, rho, omega_plus, s, force_terms);
    return;
  }
  double omega_minus = op == OP_BGK ? omega_plus : 1 / (LAMBDA / (tau - 0.5) + 0.5);
  relax_pairs(g, geq, rho, omega_plus, omega_minus, force_terms);
}

/* collision.ts:150-154 */
double oc_friction_velocity(double speed, double viscosity) {
  const double WALL_A = 8.3, WALL_B = 1.0 / 7, WALL_SUBLAYER = 11.81, WALL_DISTANCE = 0.5;
  double viscous = sqrt((viscosity * speed) / WALL_DISTANCE);
  if ((WALL_DISTANCE * viscous) / viscosity <= WALL_SUBLAYER) return viscous;
  return pow((speed * pow(viscosity / WALL_DISTANCE, WALL_B)) / WALL_A, 1 / (1 + WALL_B));
}

/* Math.hypot: the scaled formula; exact agreement with V8 in the last ulp is
 * not needed by any pinned value (the results feed thresholds and a unit
 * normalisation). */
static double hypot3(double a, double b, double c) { return sqrt(a * a + b * b + c * c); }

/* collision.ts:162-224 */
int oc_collide_wall(double *g, const double *geq, double rho, const double u[3],
                    const int *wall_incoming, int nwall, double viscosity,
                    const double *force_terms) {
  double nx = 0, ny = 0, nz = 0, exposed = 0;
  for (int k = 0; k < nwall; k++) {
    int i = wall_incoming[k];
    double w = WD[i];
    nx += w * CX[i];
    ny += w * CY[i];
    nz += w * CZ[i];
    exposed += w;
  }
  double sx = u[0], sy = u[1], sz = u[2];
  double normal_length = hypot3(nx, ny, nz);
  if (normal_length > 1e-3) {
    double normal = (sx * nx + sy * ny + sz * nz) / (normal_length * normal_length);
    sx -= normal * nx;
    sy -= normal * ny;
    sz -= normal * nz;
  }
  double speed = hypot3(sx, sy, sz);
  if (speed < 1e-7) return 0;
  double tx = sx / speed, ty = sy / speed, tz = sz / speed;
  double u_tau = oc_friction_velocity(speed, viscosity);
  double shear = 6 * exposed * rho * u_tau * u_tau;
  double flux = 0;
  stress_t b = {0, 0, 0, 0, 0, 0};
  for (int k = 0; k < nwall; k++) {
    int j = opp(wall_incoming[k]);
    double cx = CX[j], cy = CY[j], cz = CZ[j];
    double along = cx * tx + cy * ty + cz * tz;
    flux += 2 * along * (geq[j] + WD[j]);
    double s = 9 * WD[j] * along;
    b.xx += s * (cx * cx - 1.0 / 3);
    b.yy += s * (cy * cy - 1.0 / 3);
    b.zz += s * (cz * cz - 1.0 / 3);
    b.xy += s * cx * cy;
    b.xz += s * cx * cz;
    b.yz += s * cy * cz;
  }
  double norm = b.xx * b.xx + b.yy * b.yy + b.zz * b.zz + 2 * (b.xy * b.xy + b.xz * b.xz + b.yz * b.yz);
  if (norm < 0.05) return 0;
  double post[19];
  regularize(post, geq, rho, 1 - (shear - flux) / norm, b, force_terms);
  for (int i = 0; i < 19; i++)
    if (post[i] + WD[i] < 0) return 0;
  memcpy(g, post, sizeof(post));
  return 1;
}

typedef struct { uint32_t cell; int incoming; int type; double q; int64_t second; } wall_link;

struct oc_solver {
  uint32_t nx, ny, nz, cells;
  int slip; /* free-slip faces, slip.h */
  size_t links_cap;
  double tau0;
  int op, les, walls, threads;
  uint8_t *types;
  int32_t *sources;
  wall_link *links;
  size_t nlinks;
  int32_t *first_link;
  double eq_cell[19];
  double force_terms[19];
  double *current, *next;
};

static void coords(const oc_solver *s, uint32_t cell, uint32_t *x, uint32_t *y, uint32_t *z) {
  *x = cell % s->nx; *y = (cell / s->nx) % s->ny; *z = cell / (s->nx * s->ny);
}

static uint32_t wrapped(const oc_solver *s, uint32_t cell, int cx, int cy, int cz) {
  uint32_t x, y, z;
  coords(s, cell, &x, &y, &z);
  int nx = (int)s->nx, ny = (int)s->ny, nz = (int)s->nz;
  return (uint32_t)(((int)x + cx + nx) % nx + nx * ((((int)y + cy + ny) % ny) + ny * (((int)z + cz + nz) % nz)));
}

static int valid_state(const double st[4]) {
  if (!isfinite(st[0]) || st[0] <= 0) return -1;
  for (int k = 1; k < 4; k++)
    if (!isfinite(st[k])) return -2;
  return 0;
}

static float f32_at(const uint32_t *geometry, size_t index) {
  float f;
  memcpy(&f, &geometry[index], 4);
  return f;
}

static void build_sources(oc_solver *s, const uint32_t *geometry, size_t flags_len, char *err, size_t errlen);

oc_solver *oc_create(uint32_t nx, uint32_t ny, uint32_t nz, double tau0, int op, int les,
                     const double body_force[3], int walls, const uint32_t *flags,
                     size_t flags_len, const double eq_state[4], const double *init_state,
                     int threads, char *err, size_t errlen) {
#define FAIL(msg) do { snprintf(err, errlen, "%s", msg); oc_destroy(s); return NULL; } while (0)
  oc_solver *s = (oc_solver *)calloc(1, sizeof(oc_solver));
  if (!s) return NULL;
  /* referenceCellCount, cpu-solver.ts:45-66 */
  if (nx < 1 || ny < 1 || nz < 1) FAIL("Grid dimensions must be positive safe integers.");
  if (!isfinite(tau0) || tau0 <= 0.5) FAIL("Relaxation time must be finite and greater than 0.5.");
  size_t cells = (size_t)nx * ny * nz;
  if (cells * 19 > 0x7fffffffu) FAIL("Reference grid exceeds signed population indexing.");
  if (flags && flags_len != cells && flags_len < 2 * cells)
    FAIL("Flags must contain one entry per cell or the packed geometry.");
  if (walls == 1 && (flags ? flags_len : 0) < 2 * cells)
    FAIL("Interpolated walls need the packed geometry with q offsets.");
  s->nx = nx; s->ny = ny; s->nz = nz; s->cells = (uint32_t)cells;
  s->tau0 = tau0; s->op = op; s->les = les; s->walls = walls;
  s->threads = threads > 0 ? threads : 1;
  s->types = (uint8_t *)calloc(cells, 1);
  s->sources = (int32_t *)calloc(cells * 19, sizeof(int32_t));
  s->first_link = (int32_t *)calloc(cells + 1, sizeof(int32_t));
  s->current = (double *)calloc(cells * 19, sizeof(double));
  s->next = (double *)calloc(cells * 19, sizeof(double));
  s->links = (wall_link *)malloc(sizeof(wall_link) * 64);
  s->links_cap = 64;
  double rest[4] = {1, 0, 0, 0};
  const double *eqs = eq_state ? eq_state : rest;
  int bad = valid_state(eqs);
  if (bad == -1) FAIL("Initial density must be finite and positive.");
  if (bad == -2) FAIL("Initial velocity must be finite.");
  oc_equilibrium(s->eq_cell, eqs[0], eqs + 1);
  double g[3] = {0, 0, 0};
  if (body_force) { g[0] = body_force[0]; g[1] = body_force[1]; g[2] = body_force[2]; }
  if (!isfinite(g[0]) || !isfinite(g[1]) || !isfinite(g[2])) FAIL("Body acceleration must be finite.");
  for (int i = 0; i < 19; i++) s->force_terms[i] = 3 * WD[i] * (CX[i] * g[0] + CY[i] * g[1] + CZ[i] * g[2]);
  /* initialize, cpu-solver.ts:114-132 */
  double geq[19];
  for (size_t cell = 0; cell < cells; cell++) {
    uint32_t type = (flags ? flags[cell] : FLUID) & 7u;
    if (type > EQ) FAIL("Unknown cell type.");
    s->types[cell] = (uint8_t)type;
    const double *st = init_state ? init_state + 4 * cell : eqs;
    bad = valid_state(st);
    if (bad == -1) FAIL("Initial density must be finite and positive.");
    if (bad == -2) FAIL("Initial velocity must be finite.");
    if (type >= SOLID && type <= FLOOR) continue;
    oc_equilibrium(geq, st[0], st + 1);
    for (int i = 0; i < 19; i++) s->current[(size_t)i * cells + cell] = type == EQ ? s->eq_cell[i] : geq[i];
  }
  memcpy(s->next, s->current, cells * 19 * sizeof(double));
  /* buildSources, cpu-solver.ts:144-197 */
  const uint32_t *geometry = walls == 1 ? flags : NULL;
  build_sources(s, geometry, flags_len, err, errlen);
  if (err && err[0]) { oc_destroy(s); return NULL; }
  return s;
#undef FAIL
}

/* buildSources (cpu-solver.ts:144-197), with free-slip faces (slip.h) */
static void build_sources(oc_solver *s, const uint32_t *geometry, size_t flags_len, char *err, size_t errlen) {
  size_t cells = s->cells;
  if (err && errlen) err[0] = 0;
  s->nlinks = 0;
  for (size_t cell = 0; cell < cells; cell++) {
    s->first_link[cell] = (int32_t)s->nlinks;
    if (s->types[cell] != FLUID) continue;
    int rank = 0;
    uint32_t cx, cy, cz;
    coords(s, (uint32_t)cell, &cx, &cy, &cz);
    for (int i = 0; i < 19; i++) {
      int k, oy, oz;
      if (s->slip && slip_pull(s->slip, (int)s->ny, (int)s->nz, (int)cy, (int)cz, i, &k, &oy, &oz)) {
        s->sources[(size_t)i * cells + cell] = (int32_t)((size_t)k * cells + wrapped(s, (uint32_t)cell, -CX[i], oy, oz));
        continue;
      }
      uint32_t nb = wrapped(s, (uint32_t)cell, -CX[i], -CY[i], -CZ[i]);
      int type = s->types[nb];
      int wall = type >= SOLID && type <= FLOOR;
      s->sources[(size_t)i * cells + cell] = wall ? (int32_t)(opp(i) * cells + cell) : (int32_t)(i * cells + nb);
      if (!wall) continue;
      double q = HALFWAY_Q;
      if (geometry) {
        uint32_t base = geometry[cells + cell];
        if (base != NO_Q) {
          size_t index = 2 * cells + base + (size_t)rank;
          if (index >= flags_len) { snprintf(err, errlen, "Wall-link fraction is missing."); return; }
          double fq = (double)f32_at(geometry, index);
          if (!(fq > 0 && fq <= 1)) { snprintf(err, errlen, "Wall-link fraction must be in (0, 1]."); return; }
          q = fq;
        }
      }
      uint32_t second = wrapped(s, (uint32_t)cell, CX[i], CY[i], CZ[i]);
      int short_link = q < HALFWAY_Q && s->types[second] == FLUID;
      if (s->nlinks == s->links_cap) {
        s->links_cap *= 2;
        s->links = (wall_link *)realloc(s->links, s->links_cap * sizeof(wall_link));
      }
      wall_link L = {(uint32_t)cell, i, type, q, short_link ? (int64_t)second : -1};
      s->links[s->nlinks++] = L;
      rank += 1;
    }
  }
  s->first_link[cells] = (int32_t)s->nlinks;
}

void oc_set_lateral(oc_solver *s, int slip, const uint32_t *flags, size_t flags_len, char *err, size_t errlen) {
  s->slip = slip;
  build_sources(s, s->walls == 1 ? flags : NULL, flags_len, err, errlen);
}

void oc_destroy(oc_solver *s) {
  if (!s) return;
  free(s->types); free(s->sources); free(s->first_link); free(s->current); free(s->next);
  free(s->links); free(s);
}

/* cpu-solver.ts:200-208 */
static double wall_value(const oc_solver *s, const wall_link *L, const double *state) {
  size_t cells = s->cells;
  int i = L->incoming;
  double reflected = state[(size_t)opp(i) * cells + L->cell];
  if (L->q == HALFWAY_Q) return reflected;
  if (L->q < HALFWAY_Q) {
    if (L->second < 0) return reflected;
    return 2 * L->q * reflected + (1 - 2 * L->q) * state[(size_t)opp(i) * cells + (size_t)L->second];
  }
  return (reflected + (2 * L->q - 1) * state[(size_t)i * cells + L->cell]) / (2 * L->q);
}

void oc_macroscopic(oc_solver *s, uint32_t cell, double out[4]) {
  double g[19];
  for (int i = 0; i < 19; i++) g[i] = s->current[(size_t)i * s->cells + cell];
  oc_moments(g, out);
}

static void advance_fluid(oc_solver *s, uint32_t cell) {
  size_t cells = s->cells;
  double g[19], geq[19], m[4];
  for (int i = 0; i < 19; i++) g[i] = s->current[s->sources[(size_t)i * cells + cell]];
  int32_t first = s->first_link[cell], end = s->first_link[cell + 1];
  if (s->walls == 1)
    for (int32_t l = first; l < end; l++) g[s->links[l].incoming] = wall_value(s, &s->links[l], s->current);
  oc_moments(g, m);
  oc_equilibrium(geq, m[0], m + 1);
  int done = 0;
  if (s->les && end != first) {
    int incoming[19], nw = 0;
    for (int32_t l = first; l < end; l++) incoming[nw++] = s->links[l].incoming;
    double viscosity = (s->tau0 - 0.5) / 3;
    done = oc_collide_wall(g, geq, m[0], m + 1, incoming, nw, viscosity, s->force_terms);
  }
  if (!done) oc_collide(g, geq, m[0], s->tau0, s->op, s->les, s->force_terms);
  for (int i = 0; i < 19; i++) s->next[(size_t)i * cells + cell] = g[i];
}

/* cpu-solver.ts:222-244 */
void oc_step(oc_solver *s) {
  long cells = (long)s->cells;
#pragma omp parallel for schedule(static) num_threads(s->threads)
  for (long c = 0; c < cells; c++) {
    uint32_t cell = (uint32_t)c;
    int type = s->types[cell];
    if (type == EQ) {
      double geq[19];
      const double *src = s->eq_cell;
      if (s->nx >= 2 && cell % s->nx == s->nx - 1) {
        double m[4];
        double g[19];
        for (int i = 0; i < 19; i++) g[i] = s->current[(size_t)i * s->cells + cell - 1];
        oc_moments(g, m);
        oc_equilibrium(geq, 1.0, m + 1);
        src = geq;
      }
      for (int i = 0; i < 19; i++) s->next[(size_t)i * s->cells + cell] = src[i];
    } else if (type == FLUID) {
      advance_fluid(s, cell);
    }
  }
  double *t = s->current; s->current = s->next; s->next = t;
}

static void exchange(const oc_solver *s, const double *state, double f[3]) {
  f[0] = f[1] = f[2] = 0;
  for (size_t l = 0; l < s->nlinks; l++) {
    const wall_link *L = &s->links[l];
    if (L->type != SOLID) continue;
    int j = opp(L->incoming);
    double outgoing = state[(size_t)j * s->cells + L->cell];
    double ex = outgoing + (s->walls == 1 ? wall_value(s, L, state) : outgoing);
    f[0] += CX[j] * ex;
    f[1] += CY[j] * ex;
    f[2] += CZ[j] * ex;
  }
}

/* cpu-solver.ts:296-322 */
void oc_momentum_exchange(const oc_solver *s, double out[3]) {
  double a[3], b[3];
  exchange(s, s->current, a);
  exchange(s, s->next, b);
  for (int k = 0; k < 3; k++) out[k] = 0.5 * (a[k] + b[k]);
}

double *oc_populations(oc_solver *s) { return s->current; }
size_t oc_cells(const oc_solver *s) { return s->cells; }
