/*
 * FP32 restatement of the reference tracer kernels -- TEST ORACLE ONLY.
 *
 *   ot_particles_update: src/render/shaders/particles_update.wgsl:1-60
 *                        (trilinear velocity, capped Euler step, hash respawn)
 *   ot_plate_smoke:      src/render/shaders/plate_smoke.wgsl:1-85
 *                        (2-D RK2 smoke on one y plane, slide and settle rule)
 *   ot_streaks:          the project's 3-D streaklines: the rake, ring, release,
 *                        sub-step, step-cap, slide and settle rules of
 *                        plate_smoke.wgsl, with particles_update.wgsl's
 *                        trilinear sampler in place of the bilinear one.
 * WGSL mix(a, b, t) is a * (1 - t) + b * t; compile with -ffp-contract=off.
 */
#include "pw_oracle.h"

#include <math.h>
#include <string.h>

static inline float mixf(float a, float b, float t) { return a * (1.0f - t) + b * t; }
static inline float clampf(float v, float lo, float hi) { return fminf(fmaxf(v, lo), hi); }

uint32_t ot_hash(uint32_t value) {
  uint32_t h = value;
  h = (h ^ (h >> 16)) * 0x7feb352du;
  h = (h ^ (h >> 15)) * 0x846ca68bu;
  return h ^ (h >> 16);
}

typedef struct {
  uint32_t nx, ny, nz;
  const float *macros;
  const uint32_t *flags;
} field_t;

static inline uint32_t cell_index(const field_t *f, uint32_t x, uint32_t y, uint32_t z) {
  return x + f->nx * (y + f->ny * z);
}

/* particles_update.wgsl:26-36 */
static void velocity3(const field_t *f, const float p[3], float out[3]) {
  float size1[3] = {(float)(f->nx - 1u), (float)(f->ny - 1u), (float)(f->nz - 1u)};
  float point[3], w[3];
  uint32_t lo[3], hi[3];
  uint32_t lim[3] = {f->nx - 1u, f->ny - 1u, f->nz - 1u};
  for (int a = 0; a < 3; a++) {
    point[a] = clampf(p[a], 0.0f, size1[a]);
    lo[a] = (uint32_t)floorf(point[a]);
    hi[a] = lo[a] + 1u < lim[a] ? lo[a] + 1u : lim[a];
    w[a] = point[a] - floorf(point[a]);
  }
  const float *m = f->macros;
#define M(X, Y, Z, C) m[4 * (size_t)cell_index(f, X, Y, Z) + 1 + (C)]
  for (int c = 0; c < 3; c++) {
    float x00 = mixf(M(lo[0], lo[1], lo[2], c), M(hi[0], lo[1], lo[2], c), w[0]);
    float x10 = mixf(M(lo[0], hi[1], lo[2], c), M(hi[0], hi[1], lo[2], c), w[0]);
    float x01 = mixf(M(lo[0], lo[1], hi[2], c), M(hi[0], lo[1], hi[2], c), w[0]);
    float x11 = mixf(M(lo[0], hi[1], hi[2], c), M(hi[0], hi[1], hi[2], c), w[0]);
    out[c] = mixf(mixf(x00, x10, w[1]), mixf(x01, x11, w[1]), w[2]);
  }
#undef M
}

/* particles_update.wgsl:20-24 */
static int fluid3(const field_t *f, const float p[3]) {
  float size1[3] = {(float)(f->nx - 1u), (float)(f->ny - 1u), (float)(f->nz - 1u)};
  for (int a = 0; a < 3; a++)
    if (p[a] < 0.0f || p[a] >= size1[a]) return 0;
  uint32_t x = (uint32_t)floorf(p[0] + 0.5f), y = (uint32_t)floorf(p[1] + 0.5f), z = (uint32_t)floorf(p[2] + 0.5f);
  return (f->flags[cell_index(f, x, y, z)] & 7u) == 0u;
}

static inline float len3(const float v[3]) { return sqrtf((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]); }

void ot_particles_update(float *particles, uint32_t count, const float *macros, const uint32_t *flags,
                         uint32_t nx, uint32_t ny, uint32_t nz, uint32_t seed, float steps,
                         const float cs[4], const float fallback[2]) {
  field_t f = {nx, ny, nz, macros, flags};
  for (uint32_t id = 0; id < count; id++) {
    float *pt = particles + 8 * (size_t)id;
    float pos[3] = {pt[0], pt[1], pt[2]};
    float v[3];
    velocity3(&f, pos, v);
    float delta[3] = {v[0] * steps, v[1] * steps, v[2] * steps};
    float l = fmaxf(1.0f, len3(delta));
    for (int a = 0; a < 3; a++) delta[a] /= l;
    float point[3] = {pos[0] + delta[0], pos[1] + delta[1], pos[2] + delta[2]};
    float age = pt[3] + 1.0f;
    if (point[0] >= (float)(nx - 2u) || !fluid3(&f, point) || age > 4000.0f) {
      /* respawn, particles_update.wgsl:37-45 */
      float generation = pt[7] + 1.0f;
      uint32_t h = ot_hash(id + seed + (uint32_t)generation * 0x9e3779b9u);
      float r0 = (float)(h >> 8) / 16777216.0f, r1 = (float)(ot_hash(h) >> 8) / 16777216.0f;
      float q[3] = {2.0f, mixf(cs[0], cs[2], r0), mixf(cs[1], cs[3], r1)};
      if (!fluid3(&f, q)) { q[1] = fallback[0]; q[2] = fallback[1]; }
      float rec[8] = {q[0], q[1], q[2], 0.0f, q[0], q[1], q[2], generation};
      memcpy(pt, rec, sizeof(rec));
    } else {
      float rec[8] = {point[0], point[1], point[2], age, pos[0], pos[1], pos[2], pt[7]};
      memcpy(pt, rec, sizeof(rec));
    }
  }
}

/* ---------------- plate_smoke.wgsl ---------------- */
typedef struct {
  uint32_t nx, ny, nz, plane;
  const float *macros;
  const uint32_t *flags;
} plate_t;

static inline uint32_t pcell(const plate_t *s, uint32_t x, uint32_t z) { return x + s->nx * (s->plane + s->ny * z); }

static int solid2(const plate_t *s, float px, float pz) {
  if (px < 0.0f || pz < 0.0f || px > (float)(s->nx - 1u) || pz > (float)(s->nz - 1u)) return 1;
  uint32_t x = (uint32_t)floorf(px + 0.5f), z = (uint32_t)floorf(pz + 0.5f);
  return (s->flags[pcell(s, x, z)] & 7u) != 0u;
}

static void velocity2(const plate_t *s, float px, float pz, float out[2]) {
  float qx = clampf(px, 0.0f, (float)(s->nx - 2u)), qz = clampf(pz, 0.0f, (float)(s->nz - 2u));
  uint32_t lx = (uint32_t)floorf(qx), lz = (uint32_t)floorf(qz);
  float fx = qx - (float)lx, fz = qz - (float)lz;
  const float *m = s->macros;
  size_t a = 4 * (size_t)pcell(s, lx, lz), b = 4 * (size_t)pcell(s, lx + 1u, lz);
  size_t c = 4 * (size_t)pcell(s, lx, lz + 1u), d = 4 * (size_t)pcell(s, lx + 1u, lz + 1u);
  /* .yw: x and z velocity */
  out[0] = mixf(mixf(m[a + 1], m[b + 1], fx), mixf(m[c + 1], m[d + 1], fx), fz);
  out[1] = mixf(mixf(m[a + 3], m[b + 3], fx), mixf(m[c + 3], m[d + 3], fx), fz);
}

static void carry2(const plate_t *s, float st[3], float h, float settle) {
  float first[2], mid[2];
  velocity2(s, st[0], st[1], first);
  velocity2(s, st[0] + 0.5f * h * first[0], st[1] + 0.5f * h * first[1], mid);
  float step[2] = {h * mid[0], h * mid[1]};
  float l = fmaxf(1.0f, sqrtf(step[0] * step[0] + step[1] * step[1]));
  step[0] /= l; step[1] /= l;
  float nx_ = st[0] + step[0], nz_ = st[1] + step[1];
  float density = st[2];
  if (solid2(s, nx_, nz_)) {
    density *= settle;
    if (!solid2(s, nx_, st[1])) nz_ = st[1];
    else if (!solid2(s, st[0], nz_)) nx_ = st[0];
    else { nx_ = -1.0f; nz_ = -1.0f; }
  }
  st[0] = nx_; st[1] = nz_; st[2] = density;
}

void ot_plate_smoke(float *smoke, uint32_t threads, uint32_t slots, uint32_t release, int releasing,
                    const float rake[4], uint32_t nx, uint32_t ny, uint32_t nz, uint32_t plane,
                    const float *macros, const uint32_t *flags, const float *ports, uint32_t nports) {
  plate_t s = {nx, ny, nz, plane, macros, flags};
  for (uint32_t id = 0; id < threads * slots; id++) {
    uint32_t thread = id / slots;
    float *rec = smoke + 4 * (size_t)id;
    if (releasing && id % slots == release % slots) {
      uint32_t rk = threads - nports;
      if (thread < rk) {
        uint32_t den = (rk > 2u ? rk : 2u) - 1u;
        float height = mixf(rake[1], rake[2], (float)thread / (float)den);
        rec[0] = rake[0]; rec[1] = height; rec[2] = (float)release; rec[3] = 1.0f;
      } else {
        const float *port = ports + 2 * (size_t)(thread - rk);
        rec[0] = port[0]; rec[1] = port[1]; rec[2] = (float)release; rec[3] = port[0] >= 0.0f ? 1.0f : 0.0f;
      }
      continue;
    }
    if (rec[3] == 0.0f) continue;
    float h = rake[3];
    float u[2];
    velocity2(&s, rec[0], rec[1], u);
    float speed = sqrtf(u[0] * u[0] + u[1] * u[1]);
    uint32_t count = (uint32_t)clampf(ceilf(2.0f * h * speed), 1.0f, 16.0f);
    float settle = powf(0.85f, 1.0f / (float)count);
    float st[3] = {rec[0], rec[1], rec[3]};
    for (uint32_t i = 0; i < count && st[0] >= 0.0f; i++) carry2(&s, st, h / (float)count, settle);
    int finite = st[0] == st[0] && st[1] == st[1] && st[2] == st[2];
    int alive = finite && st[0] >= 0.0f && st[0] < (float)(nx - 2u) && st[2] > 0.02f;
    rec[0] = st[0]; rec[1] = st[1]; rec[3] = alive ? st[2] : 0.0f;
  }
}

/* ---------------- 3-D streaklines ---------------- */
static int solid3(const field_t *f, const float p[3]) {
  float lim[3] = {(float)(f->nx - 1u), (float)(f->ny - 1u), (float)(f->nz - 1u)};
  for (int a = 0; a < 3; a++)
    if (p[a] < 0.0f || p[a] > lim[a]) return 1;
  uint32_t x = (uint32_t)floorf(p[0] + 0.5f), y = (uint32_t)floorf(p[1] + 0.5f), z = (uint32_t)floorf(p[2] + 0.5f);
  return (f->flags[cell_index(f, x, y, z)] & 7u) != 0u;
}

/* The slide candidates keep two, then one, of the three step components, in
 * the order of plate_smoke.wgsl:45-51 (drop the vertical first). */
static const uint8_t KEEP[6][3] = {{1, 1, 0}, {1, 0, 1}, {0, 1, 1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};

static void carry3(const field_t *f, float st[4], float h, float settle) {
  float first[3], mid[3];
  velocity3(f, st, first);
  float half[3] = {st[0] + 0.5f * h * first[0], st[1] + 0.5f * h * first[1], st[2] + 0.5f * h * first[2]};
  velocity3(f, half, mid);
  float step[3] = {h * mid[0], h * mid[1], h * mid[2]};
  float l = fmaxf(1.0f, len3(step));
  for (int a = 0; a < 3; a++) step[a] /= l;
  float next[3] = {st[0] + step[0], st[1] + step[1], st[2] + step[2]};
  float density = st[3];
  if (solid3(f, next)) {
    density *= settle;
    int moved = 0;
    for (int k = 0; k < 6 && !moved; k++) {
      float cand[3];
      for (int a = 0; a < 3; a++) cand[a] = KEEP[k][a] ? next[a] : st[a];
      if (!solid3(f, cand)) { memcpy(next, cand, sizeof(cand)); moved = 1; }
    }
    if (!moved) { next[0] = -1.0f; next[1] = -1.0f; next[2] = -1.0f; }
  }
  st[0] = next[0]; st[1] = next[1]; st[2] = next[2]; st[3] = density;
}

void ot_streaks(float *puffs, uint32_t *release_of, uint32_t ry, uint32_t rz, uint32_t slots,
                uint32_t release, int releasing, const float rake[5], float h, uint32_t nx,
                uint32_t ny, uint32_t nz, const float *macros, const uint32_t *flags) {
  field_t f = {nx, ny, nz, macros, flags};
  uint32_t threads = ry * rz;
  for (uint32_t id = 0; id < threads * slots; id++) {
    uint32_t thread = id / slots;
    float *rec = puffs + 4 * (size_t)id;
    if (releasing && id % slots == release % slots) {
      uint32_t iy = thread % ry, iz = thread / ry;
      float ty = (float)iy / (float)((ry > 2u ? ry : 2u) - 1u);
      float tz = (float)iz / (float)((rz > 2u ? rz : 2u) - 1u);
      rec[0] = rake[0];
      rec[1] = mixf(rake[1], rake[2], ty);
      rec[2] = mixf(rake[3], rake[4], tz);
      rec[3] = 1.0f;
      release_of[id] = release;
      continue;
    }
    if (rec[3] == 0.0f) continue;
    float u[3];
    velocity3(&f, rec, u);
    uint32_t count = (uint32_t)clampf(ceilf(2.0f * h * len3(u)), 1.0f, 16.0f);
    float settle = powf(0.85f, 1.0f / (float)count);
    float st[4] = {rec[0], rec[1], rec[2], rec[3]};
    for (uint32_t i = 0; i < count && st[0] >= 0.0f; i++) carry3(&f, st, h / (float)count, settle);
    int finite = st[0] == st[0] && st[1] == st[1] && st[2] == st[2] && st[3] == st[3];
    int alive = finite && st[0] >= 0.0f && st[0] < (float)(nx - 2u) && st[3] > 0.02f;
    rec[0] = st[0]; rec[1] = st[1]; rec[2] = st[2]; rec[3] = alive ? st[3] : 0.0f;
  }
}
