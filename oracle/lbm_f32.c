/*
 * FP32 restatement of the reference's WGSL solver kernels -- TEST ORACLE ONLY.
 *
 * Follows, statement for statement and in the same evaluation order:
 *   src/lbm/shaders/common.wgsl:1-150      (C, W, idx_wrapped, geq, stress, tau, load/store)
 *   src/lbm/shaders/stream_collide.wgsl:1-136 (wall law, outlet, main)
 *   src/lbm/shaders/walls.wgsl:1-21        (halfway / Bouzidi wall_value)
 *   src/lbm/shaders/collide-trt.wgsl:1-15, collide-reg.wgsl:1-18
 *   src/lbm/shaders/prelude-f16.wgsl:1-22, prelude-f32.wgsl:1-5
 *   src/lbm/shaders/init.wgsl:1-8, force.wgsl:1-40, reduce.wgsl:1-18
 * with the A/B ping-pong of src/lbm/gpu-solver.ts:216-219,378-395 and the
 * uniform packing of packSolverParams (gpu-solver.ts:80-116).
 *
 * Must be compiled with -ffp-contract=off and without -ffast-math: every
 * product and sum is a separate IEEE binary32 operation, as in WGSL.
 */
#include "pw_oracle.h"
#include "slip.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

static const int CX[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0};
static const int CY[19] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 1, -1};
static const int CZ[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, -1, 1, -1, 1};

enum { FLUID = 0, SOLID = 1, SUPPORT = 2, FLOOR = 3, EQ = 4 };
#define NO_Q 0xffffffffu

static float WF[19];
static int tables_ready = 0;
static void init_tables(void) {
  if (tables_ready) return;
  for (int i = 0; i < 19; i++) {
    /* WGSL const-expression 1.0/3.0 etc. is evaluated exactly and rounded once. */
    WF[i] = (float)(i == 0 ? 1.0 / 3.0 : (i < 7 ? 1.0 / 18.0 : 1.0 / 36.0));
  }
  tables_ready = 1;
}

static inline uint32_t fbits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static inline float bitsf(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static inline int opp(int i) { return i == 0 ? 0 : ((i & 1) ? i + 1 : i - 1); }

/* ---------------- storage codecs ---------------- */

uint16_t ow_f32_to_f16_rne(float f) {
  uint32_t x = fbits(f);
  uint32_t sign = (x >> 16) & 0x8000u;
  uint32_t mag = x & 0x7fffffffu;
  if (mag >= 0x7f800000u) return (uint16_t)(sign | (mag > 0x7f800000u ? 0x7e00u : 0x7c00u));
  if (mag >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u);
  if (mag >= 0x38800000u) {
    uint32_t m = mag - 0x38000000u;
    m += 0xfffu + ((m >> 13) & 1u);
    return (uint16_t)(sign | (m >> 13));
  }
  if (mag < 0x33000000u) return (uint16_t)sign;
  uint32_t e = mag >> 23;
  uint32_t mant = (mag & 0x7fffffu) | 0x800000u;
  uint32_t shift = 126u - e;
  uint32_t m = mant >> shift;
  uint32_t rem = mant & ((1u << shift) - 1u);
  uint32_t half = 1u << (shift - 1u);
  if (rem > half || (rem == half && (m & 1u))) m++;
  return (uint16_t)(sign | m);
}

float ow_f16_to_f32(uint16_t h) {
  uint32_t sign = ((uint32_t)h & 0x8000u) << 16;
  uint32_t e = (h >> 10) & 0x1fu;
  uint32_t m = h & 0x3ffu;
  if (e == 0) {
    /* subnormal: m * 2^-24, exact in binary32 */
    float v = (float)m * 5.9604644775390625e-08f;
    return bitsf(fbits(v) | sign);
  }
  if (e == 31) return bitsf(sign | 0x7f800000u | (m << 13));
  return bitsf(sign | ((e + 112u) << 23) | (m << 13));
}

uint16_t ow_f32_to_bf16_rne(float f) {
  uint32_t x = fbits(f);
  if ((x & 0x7fffffffu) > 0x7f800000u) return (uint16_t)((x >> 16) | 0x40u);
  x += 0x7fffu + ((x >> 16) & 1u);
  return (uint16_t)(x >> 16);
}

float ow_bf16_to_f32(uint16_t h) { return bitsf((uint32_t)h << 16); }

static inline uint32_t lowbias32(uint32_t bits, uint32_t i, uint32_t n) {
  uint32_t r = bits ^ (n * 0x9e3779b9u) ^ (i * 0x85ebca6bu);
  r = (r ^ (r >> 16)) * 0x7feb352du;
  r = (r ^ (r >> 15)) * 0x846ca68bu;
  r ^= r >> 16;
  return r;
}

/* prelude-f16.wgsl:7-22: hash-dithered rounding of the 13 discarded bits. */
uint16_t ow_encode_f16(float value, uint32_t i, uint32_t n) {
  uint32_t bits = fbits(value);
  uint32_t random = lowbias32(bits, i, n);
  uint32_t magnitude = bits & 0x7fffffffu;
  if (magnitude < 0x38800000u) return ow_f32_to_f16_rne(value);
  uint32_t increment = ((random & 0x1fffu) < (magnitude & 0x1fffu)) ? 0x2000u : 0u;
  uint32_t rounded = (magnitude & 0xffffe000u) + increment;
  return ow_f32_to_f16_rne(bitsf((bits & 0x80000000u) | rounded));
}

/* The same dithering over the 16 bits bfloat16 discards; the reference has no
 * bf16 path, so this is the project's own rule (no scale is needed: bf16 keeps
 * the binary32 exponent range). */
uint16_t ow_encode_bf16(float value, uint32_t i, uint32_t n) {
  uint32_t bits = fbits(value);
  uint32_t random = lowbias32(bits, i, n);
  uint32_t magnitude = bits & 0x7fffffffu;
  if (magnitude < 0x00800000u || magnitude >= 0x7f800000u) return ow_f32_to_bf16_rne(value);
  uint32_t increment = ((random & 0xffffu) < (magnitude & 0xffffu)) ? 0x10000u : 0u;
  uint32_t rounded = (magnitude & 0xffff0000u) + increment;
  return (uint16_t)(((bits & 0x80000000u) | rounded) >> 16);
}

/* ---------------- solver ---------------- */

struct ow_solver {
  uint32_t nx, ny, nz, cells;
  int slip; /* free-slip faces, slip.h */
  float u_in, nu, cs_term, lambda;
  int les, op, walls, storage, threads;
  uint32_t *geometry;
  size_t geometry_len;
  uint32_t *boundary;
  size_t nboundary;
  void *state[2];
  float *macros;
  int current; /* index of the latest post-collision state */
};

typedef struct {
  const ow_solver *s;
  const void *in;
  void *out;
  float u_in;
  int write_macro;
} ctx_t;

static inline float load_in(const ow_solver *s, const void *st, int i, uint32_t n) {
  size_t k = (size_t)i * s->cells + n;
  switch (s->storage) {
    case 1: return ow_f16_to_f32(((const uint16_t *)st)[k]) / 32768.0f;
    case 2: return ow_bf16_to_f32(((const uint16_t *)st)[k]) / 1.0f;
    default: return ((const float *)st)[k] / 1.0f;
  }
}

static inline void store_out(const ow_solver *s, void *st, int i, uint32_t n, float value) {
  size_t k = (size_t)i * s->cells + n;
  switch (s->storage) {
    case 1: ((uint16_t *)st)[k] = ow_encode_f16(value * 32768.0f, (uint32_t)i, n); break;
    case 2: ((uint16_t *)st)[k] = ow_encode_bf16(value * 1.0f, (uint32_t)i, n); break;
    default: ((float *)st)[k] = value * 1.0f; break;
  }
}

static inline uint32_t idx(const ow_solver *s, uint32_t x, uint32_t y, uint32_t z) {
  return x + s->nx * (y + s->ny * z);
}

static inline uint32_t idx_wrapped(const ow_solver *s, uint32_t x, uint32_t y, uint32_t z,
                                   int ox, int oy, int oz) {
  int sx = ((int)x + ox + (int)s->nx) % (int)s->nx;
  int sy = ((int)y + oy + (int)s->ny) % (int)s->ny;
  int sz = ((int)z + oz + (int)s->nz) % (int)s->nz;
  return idx(s, (uint32_t)sx, (uint32_t)sy, (uint32_t)sz);
}

static inline int is_wall(uint32_t kind) { return kind == SOLID || kind == SUPPORT || kind == FLOOR; }
static inline int has_wall(uint32_t flag, int i) { return (flag & (1u << (3 + i))) != 0u; }

static inline float dot3(float ax, float ay, float az, float bx, float by, float bz) {
  return (ax * bx + ay * by) + az * bz;
}

/* common.wgsl:84-88 */
static inline float geq(int i, float rho_delta, const float v[3]) {
  float cu = dot3((float)CX[i], (float)CY[i], (float)CZ[i], v[0], v[1], v[2]);
  float uu = dot3(v[0], v[1], v[2], v[0], v[1], v[2]);
  return WF[i] * (rho_delta + (1.0f + rho_delta) * (3.0f * cu + 4.5f * cu * cu - 1.5f * uu));
}

typedef struct { float xx, yy, zz, xy, xz, yz; } stress_t;

/* common.wgsl:100-113 */
static stress_t non_equilibrium_stress(const float *g, const float *eq) {
  stress_t st = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
  for (int i = 0; i < 19; i++) {
    float cx = (float)CX[i], cy = (float)CY[i], cz = (float)CZ[i];
    float neq = g[i] - eq[i];
    st.xx += cx * cx * neq;
    st.yy += cy * cy * neq;
    st.zz += cz * cz * neq;
    st.xy += cx * cy * neq;
    st.xz += cx * cz * neq;
    st.yz += cy * cz * neq;
  }
  return st;
}

/* common.wgsl:115-122 */
static float relaxation_time(const ow_solver *s, const float *g, const float *eq, float rho) {
  float tau0 = 3.0f * s->nu + 0.5f;
  if (!s->les) return tau0;
  stress_t pi = non_equilibrium_stress(g, eq);
  float q = pi.xx * pi.xx + pi.yy * pi.yy + pi.zz * pi.zz +
            2.0f * (pi.xy * pi.xy + pi.xz * pi.xz + pi.yz * pi.yz);
  return 0.5f * (tau0 + sqrtf(tau0 * tau0 + s->cs_term * sqrtf(q) / rho));
}

/* collide-trt.wgsl:1-15 and collide-reg.wgsl:3-18 */
static void collide(const ow_solver *s, const float *g, const float *eq, float rho, float *post) {
  float tau = relaxation_time(s, g, eq, rho);
  float omega_plus = 1.0f / tau;
  if (s->op == 1) {
    stress_t pi = non_equilibrium_stress(g, eq);
    float trace = pi.xx + pi.yy + pi.zz;
    for (int i = 0; i < 19; i++) {
      float cx = (float)CX[i], cy = (float)CY[i], cz = (float)CZ[i];
      float projected = cx * cx * pi.xx + cy * cy * pi.yy + cz * cz * pi.zz +
                        2.0f * (cx * cy * pi.xy + cx * cz * pi.xz + cy * cz * pi.yz) -
                        trace / 3.0f;
      post[i] = eq[i] + (1.0f - omega_plus) * 4.5f * WF[i] * projected;
    }
    return;
  }
  float omega_minus = 1.0f / (s->lambda / (tau - 0.5f) + 0.5f);
  post[0] = g[0] - omega_plus * (g[0] - eq[0]);
  for (int i = 1; i < 19; i += 2) {
    int j = opp(i);
    float even = 0.5f * omega_plus * (g[i] + g[j] - eq[i] - eq[j]);
    float odd = 0.5f * omega_minus * (g[i] - g[j] - eq[i] + eq[j]);
    post[i] = g[i] - even - odd;
    post[j] = g[j] - even + odd;
  }
}

/* stream_collide.wgsl:8-12 */
static float friction_velocity(const ow_solver *s, float speed) {
  const float WALL_A = 8.3f;
  const float WALL_B = (float)(1.0 / 7.0);
  const float WALL_SUBLAYER = 11.81f;
  const float WALL_DISTANCE = 0.5f;
  float viscous = sqrtf(s->nu * speed / WALL_DISTANCE);
  if (WALL_DISTANCE * viscous / s->nu <= WALL_SUBLAYER) return viscous;
  return powf(speed * powf(s->nu / WALL_DISTANCE, WALL_B) / WALL_A, 1.0f / (1.0f + WALL_B));
}

/* stream_collide.wgsl:18-80 */
static void collide_wall(const ow_solver *s, const float *g, const float *eq, float rho,
                         const float v[3], uint32_t flag, float *post) {
  float normal[3] = {0.0f, 0.0f, 0.0f};
  float exposed = 0.0f;
  for (int i = 1; i < 19; i++) {
    if (has_wall(flag, i)) {
      normal[0] += WF[i] * (float)CX[i];
      normal[1] += WF[i] * (float)CY[i];
      normal[2] += WF[i] * (float)CZ[i];
      exposed += WF[i];
    }
  }
  float slip[3] = {v[0], v[1], v[2]};
  float normal_length = sqrtf(dot3(normal[0], normal[1], normal[2], normal[0], normal[1], normal[2]));
  if (normal_length > 1e-3f) {
    float n[3] = {normal[0] / normal_length, normal[1] / normal_length, normal[2] / normal_length};
    float d = dot3(v[0], v[1], v[2], n[0], n[1], n[2]);
    slip[0] -= d * n[0];
    slip[1] -= d * n[1];
    slip[2] -= d * n[2];
  }
  float speed = sqrtf(dot3(slip[0], slip[1], slip[2], slip[0], slip[1], slip[2]));
  if (speed < 1e-7f) { collide(s, g, eq, rho, post); return; }
  float t[3] = {slip[0] / speed, slip[1] / speed, slip[2] / speed};
  float u_tau = friction_velocity(s, speed);
  float shear = 6.0f * exposed * rho * u_tau * u_tau;
  float flux = 0.0f;
  stress_t b = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
  const float third = (float)(1.0 / 3.0);
  for (int i = 1; i < 19; i++) {
    if (!has_wall(flag, i)) continue;
    int j = opp(i);
    float cx = (float)CX[j], cy = (float)CY[j], cz = (float)CZ[j];
    float along = dot3(cx, cy, cz, t[0], t[1], t[2]);
    flux += 2.0f * along * (eq[j] + WF[j]);
    float sj = 9.0f * WF[j] * along;
    b.xx += sj * (cx * cx - third);
    b.yy += sj * (cy * cy - third);
    b.zz += sj * (cz * cz - third);
    b.xy += sj * cx * cy;
    b.xz += sj * cx * cz;
    b.yz += sj * cy * cz;
  }
  float norm = b.xx * b.xx + b.yy * b.yy + b.zz * b.zz +
               2.0f * (b.xy * b.xy + b.xz * b.xz + b.yz * b.yz);
  if (norm < 0.05f) { collide(s, g, eq, rho, post); return; }
  float scale = 4.5f * (shear - flux) / norm;
  float trace = b.xx + b.yy + b.zz;
  for (int i = 0; i < 19; i++) {
    float cx = (float)CX[i], cy = (float)CY[i], cz = (float)CZ[i];
    float projected = cx * cx * b.xx + cy * cy * b.yy + cz * cz * b.zz +
                      2.0f * (cx * cy * b.xy + cx * cz * b.xz + cy * cz * b.yz) - trace / 3.0f;
    post[i] = eq[i] + scale * WF[i] * projected;
    if (post[i] + WF[i] < 0.0f) { collide(s, g, eq, rho, post); return; }
  }
}

/* walls.wgsl:6-21 */
static float wall_value(const ow_solver *s, const void *st, int i, uint32_t n, uint32_t x,
                        uint32_t y, uint32_t z, uint32_t flag) {
  int j = opp(i);
  float reflected = load_in(s, st, j, n);
  if (s->walls == 0) return reflected;
  uint32_t base = s->geometry[s->cells + n];
  if (base == NO_Q) return reflected;
  uint32_t rank = (uint32_t)__builtin_popcount((flag >> 3) & ((1u << i) - 1u));
  float q = bitsf(s->geometry[2u * s->cells + base + rank]);
  if (q == 0.5f) return reflected;
  if (q < 0.5f) {
    uint32_t second = idx_wrapped(s, x, y, z, CX[i], CY[i], CZ[i]);
    if ((s->geometry[second] & 7u) != FLUID) return reflected;
    return 2.0f * q * reflected + (1.0f - 2.0f * q) * load_in(s, st, j, second);
  }
  return (reflected + (2.0f * q - 1.0f) * load_in(s, st, i, n)) / (2.0f * q);
}

/* stream_collide.wgsl:83-93 */
static void outlet_velocity(const ow_solver *s, const void *st, uint32_t x, uint32_t y,
                            uint32_t z, float out[3]) {
  uint32_t upstream = idx(s, x - 1u, y, z);
  float mass = 1.0f;
  float m[3] = {0.0f, 0.0f, 0.0f};
  for (int i = 0; i < 19; i++) {
    float value = load_in(s, st, i, upstream);
    mass += value;
    m[0] += (float)CX[i] * value;
    m[1] += (float)CY[i] * value;
    m[2] += (float)CZ[i] * value;
  }
  out[0] = m[0] / mass;
  out[1] = m[1] / mass;
  out[2] = m[2] / mass;
}

/* common.wgsl:145-150 */
static void store_equilibrium(const ow_solver *s, void *out, float *macros, int write_macro,
                              uint32_t n, float rho_delta, const float v[3]) {
  for (int i = 0; i < 19; i++) store_out(s, out, i, n, geq(i, rho_delta, v));
  if (write_macro) {
    macros[4 * (size_t)n + 0] = 1.0f + rho_delta;
    macros[4 * (size_t)n + 1] = v[0];
    macros[4 * (size_t)n + 2] = v[1];
    macros[4 * (size_t)n + 3] = v[2];
  }
}

/* stream_collide.wgsl:95-136 for one cell */
static void cell_step(const ctx_t *c, uint32_t n) {
  const ow_solver *s = c->s;
  uint32_t x = n % s->nx, y = (n / s->nx) % s->ny, z = n / (s->nx * s->ny);
  uint32_t flag = s->geometry[n];
  uint32_t kind = flag & 7u;
  if (is_wall(kind)) return;
  if (kind == EQ) {
    float inflow[3] = {c->u_in, 0.0f, 0.0f};
    if (x == s->nx - 1u && x > 0u) outlet_velocity(s, c->in, x, y, z, inflow);
    store_equilibrium(s, c->out, s->macros, c->write_macro, n, 0.0f, inflow);
    return;
  }
  float g[19], eq[19], post[19];
  g[0] = load_in(s, c->in, 0, n);
  for (int i = 1; i < 19; i++) {
    int k, oy, oz;
    if (s->slip && slip_pull(s->slip, (int)s->ny, (int)s->nz, (int)y, (int)z, i, &k, &oy, &oz))
      g[i] = load_in(s, c->in, k, idx_wrapped(s, x, y, z, -CX[i], oy, oz));
    else if (has_wall(flag, i)) g[i] = wall_value(s, c->in, i, n, x, y, z, flag);
    else g[i] = load_in(s, c->in, i, idx_wrapped(s, x, y, z, -CX[i], -CY[i], -CZ[i]));
  }
  float rho_delta = 0.0f;
  float m[3] = {0.0f, 0.0f, 0.0f};
  for (int i = 0; i < 19; i++) {
    rho_delta += g[i];
    m[0] += (float)CX[i] * g[i];
    m[1] += (float)CY[i] * g[i];
    m[2] += (float)CZ[i] * g[i];
  }
  float rho = 1.0f + rho_delta;
  float v[3] = {m[0] / rho, m[1] / rho, m[2] / rho};
  for (int i = 0; i < 19; i++) eq[i] = geq(i, rho_delta, v);
  if (s->les && (flag >> 3) != 0u) collide_wall(s, g, eq, rho, v, flag, post);
  else collide(s, g, eq, rho, post);
  for (int i = 0; i < 19; i++) store_out(s, c->out, i, n, post[i]);
  if (c->write_macro) {
    s->macros[4 * (size_t)n + 0] = rho;
    s->macros[4 * (size_t)n + 1] = v[0];
    s->macros[4 * (size_t)n + 2] = v[1];
    s->macros[4 * (size_t)n + 3] = v[2];
  }
}

static size_t storage_bytes(int storage) { return storage == 0 ? 4 : 2; }

ow_solver *ow_create(uint32_t nx, uint32_t ny, uint32_t nz, float tau0, float u_in, int les,
                     int op, int walls, int storage, const uint32_t *geometry,
                     size_t geometry_len, const uint32_t *boundary, size_t nboundary,
                     int threads) {
  init_tables();
  ow_solver *s = (ow_solver *)calloc(1, sizeof(ow_solver));
  if (!s) return NULL;
  s->nx = nx; s->ny = ny; s->nz = nz; s->cells = nx * ny * nz;
  s->u_in = u_in;
  /* packSolverParams: nu = fround((fround(tau0) - 0.5) / 3) */
  s->nu = (float)(((double)tau0 - 0.5) / 3.0);
  s->cs_term = (float)(18.0 * 1.4142135623730951 * (0.1 * 0.1));
  s->lambda = (float)(3.0 / 16.0);
  s->les = les; s->op = op; s->walls = walls; s->storage = storage;
  s->threads = threads > 0 ? threads : 1;
  s->geometry = (uint32_t *)malloc(geometry_len * sizeof(uint32_t));
  memcpy(s->geometry, geometry, geometry_len * sizeof(uint32_t));
  s->geometry_len = geometry_len;
  s->boundary = (uint32_t *)malloc((nboundary ? nboundary : 1) * sizeof(uint32_t));
  if (nboundary) memcpy(s->boundary, boundary, nboundary * sizeof(uint32_t));
  s->nboundary = nboundary;
  size_t bytes = 19 * (size_t)s->cells * storage_bytes(storage);
  s->state[0] = calloc(1, bytes);
  s->state[1] = calloc(1, bytes);
  s->macros = (float *)calloc(4 * (size_t)s->cells, sizeof(float));
  ow_reset(s, u_in);
  return s;
}

void ow_set_lateral(ow_solver *s, int slip) { s->slip = slip; }

void ow_destroy(ow_solver *s) {
  if (!s) return;
  free(s->geometry); free(s->boundary); free(s->state[0]); free(s->state[1]); free(s->macros);
  free(s);
}

/* init.wgsl:1-8 dispatched into both states (GpuSolver.reset, gpu-solver.ts:347-355) */
void ow_reset(ow_solver *s, float u_in_init) {
  for (int k = 0; k < 2; k++) {
    for (uint32_t n = 0; n < s->cells; n++) {
      uint32_t kind = s->geometry[n] & 7u;
      float v[3] = {u_in_init, 0.0f, 0.0f};
      if (is_wall(kind)) v[0] = 0.0f;
      store_equilibrium(s, s->state[k], s->macros, 1, n, 0.0f, v);
    }
  }
  s->current = 0;
}

void ow_step(ow_solver *s, float u_in, int write_macro) {
  ctx_t c = {s, s->state[s->current], s->state[1 - s->current], u_in, write_macro};
  long cells = (long)s->cells;
#pragma omp parallel for schedule(static) num_threads(s->threads)
  for (long n = 0; n < cells; n++) cell_step(&c, (uint32_t)n);
  s->current = 1 - s->current;
}

/* force.wgsl:7-40: per state, sum c_j (g*_j + wall_value) over SOLID links of
 * the boundary cells, halve, and add both states (reduce.wgsl).  The link
 * terms are binary32 as in WGSL; the sum is carried in binary64. */
void ow_force(const ow_solver *s, double out[3]) {
  double f[3] = {0.0, 0.0, 0.0};
  for (int k = 0; k < 2; k++) {
    const void *st = s->state[k];
    double part[3] = {0.0, 0.0, 0.0};
    for (size_t item = 0; item < s->nboundary; item++) {
      uint32_t n = s->boundary[item];
      uint32_t flag = s->geometry[n];
      uint32_t x = n % s->nx, y = (n / s->nx) % s->ny, z = n / (s->nx * s->ny);
      for (int i = 1; i < 19; i++) {
        if (!has_wall(flag, i)) continue;
        int k, oy, oz;
        if (s->slip && slip_pull(s->slip, (int)s->ny, (int)s->nz, (int)y, (int)z, i, &k, &oy, &oz)) continue;
        uint32_t nb = idx_wrapped(s, x, y, z, -CX[i], -CY[i], -CZ[i]);
        if ((s->geometry[nb] & 7u) != SOLID) continue;
        int j = opp(i);
        float term = load_in(s, st, j, n) + wall_value(s, st, i, n, x, y, z, flag);
        part[0] += (double)CX[j] * (double)term;
        part[1] += (double)CY[j] * (double)term;
        part[2] += (double)CZ[j] * (double)term;
      }
    }
    f[0] += 0.5 * part[0];
    f[1] += 0.5 * part[1];
    f[2] += 0.5 * part[2];
  }
  out[0] = f[0]; out[1] = f[1]; out[2] = f[2];
}

void ow_populations(const ow_solver *s, float *out) {
  const void *st = s->state[s->current];
  for (int i = 0; i < 19; i++)
    for (uint32_t n = 0; n < s->cells; n++) out[(size_t)i * s->cells + n] = load_in(s, st, i, n);
}

void ow_populations_raw(const ow_solver *s, void *out) {
  memcpy(out, s->state[s->current], 19 * (size_t)s->cells * storage_bytes(s->storage));
}

void ow_macros(const ow_solver *s, float *out) {
  memcpy(out, s->macros, 4 * (size_t)s->cells * sizeof(float));
}

void ow_poke(ow_solver *s, uint32_t i, uint32_t n, float value) {
  store_out(s, s->state[s->current], (int)i, n, value);
}

void ow_params(const ow_solver *s, float out[4]) {
  out[0] = s->u_in; out[1] = s->nu; out[2] = s->cs_term; out[3] = s->lambda;
}
