// Tracer advection on the solver's macro field (compiled with -fmad=false so the
// binary32 sampler and integrators round as the reference's WGSL does).
//   particles: src/render/shaders/particles_update.wgsl:1-60
//   plate:     src/render/shaders/plate_smoke.wgsl:1-85
//   streaks:   plate_smoke's rake/ring/sub-step/cap/slide/settle rules in 3-D with
//              particles_update's trilinear sampler and an RK2 midpoint step.
// WGSL mix(a, b, t) = a * (1 - t) + b * t.
#include <cuda_runtime.h>

#include "pw_internal.h"

using namespace pwhost;

namespace {

__device__ __forceinline__ float mixf(float a, float b, float t) { return a * (1.0f - t) + b * t; }
__device__ __forceinline__ float clampf(float v, float lo, float hi) { return fminf(fmaxf(v, lo), hi); }

struct Field {
  const float4 *macros;
  const uint32_t *flags;
  uint32_t nx, ny, nz;
  __device__ __forceinline__ uint32_t cell(uint32_t x, uint32_t y, uint32_t z) const { return x + nx * (y + ny * z); }
};

__device__ __forceinline__ uint32_t hash32(uint32_t value) {
  uint32_t h = value;
  h = (h ^ (h >> 16)) * 0x7feb352du;
  h = (h ^ (h >> 15)) * 0x846ca68bu;
  return h ^ (h >> 16);
}

// particles_update.wgsl:26-36
__device__ float3 velocity3(const Field &f, float px, float py, float pz) {
  float sx = (float)(f.nx - 1u), sy = (float)(f.ny - 1u), sz = (float)(f.nz - 1u);
  float qx = clampf(px, 0.f, sx), qy = clampf(py, 0.f, sy), qz = clampf(pz, 0.f, sz);
  uint32_t lx = (uint32_t)floorf(qx), ly = (uint32_t)floorf(qy), lz = (uint32_t)floorf(qz);
  uint32_t hx = min(lx + 1u, f.nx - 1u), hy = min(ly + 1u, f.ny - 1u), hz = min(lz + 1u, f.nz - 1u);
  float wx = qx - floorf(qx), wy = qy - floorf(qy), wz = qz - floorf(qz);
  float4 a = f.macros[f.cell(lx, ly, lz)], b = f.macros[f.cell(hx, ly, lz)];
  float4 c = f.macros[f.cell(lx, hy, lz)], d = f.macros[f.cell(hx, hy, lz)];
  float4 e = f.macros[f.cell(lx, ly, hz)], g = f.macros[f.cell(hx, ly, hz)];
  float4 h = f.macros[f.cell(lx, hy, hz)], k = f.macros[f.cell(hx, hy, hz)];
  float3 out;
  float y_, z_, w_;
  {
    float x00 = mixf(a.y, b.y, wx), x10 = mixf(c.y, d.y, wx), x01 = mixf(e.y, g.y, wx), x11 = mixf(h.y, k.y, wx);
    y_ = mixf(mixf(x00, x10, wy), mixf(x01, x11, wy), wz);
  }
  {
    float x00 = mixf(a.z, b.z, wx), x10 = mixf(c.z, d.z, wx), x01 = mixf(e.z, g.z, wx), x11 = mixf(h.z, k.z, wx);
    z_ = mixf(mixf(x00, x10, wy), mixf(x01, x11, wy), wz);
  }
  {
    float x00 = mixf(a.w, b.w, wx), x10 = mixf(c.w, d.w, wx), x01 = mixf(e.w, g.w, wx), x11 = mixf(h.w, k.w, wx);
    w_ = mixf(mixf(x00, x10, wy), mixf(x01, x11, wy), wz);
  }
  out.x = y_;
  out.y = z_;
  out.z = w_;
  return out;
}

// particles_update.wgsl:20-24
__device__ bool fluid3(const Field &f, float px, float py, float pz) {
  if (px < 0.f || py < 0.f || pz < 0.f) return false;
  if (px >= (float)(f.nx - 1u) || py >= (float)(f.ny - 1u) || pz >= (float)(f.nz - 1u)) return false;
  uint32_t x = (uint32_t)floorf(px + 0.5f), y = (uint32_t)floorf(py + 0.5f), z = (uint32_t)floorf(pz + 0.5f);
  return (f.flags[f.cell(x, y, z)] & 7u) == 0u;
}

__device__ __forceinline__ float len3(float x, float y, float z) { return sqrtf((x * x + y * y) + z * z); }

struct ParticleParams {
  uint32_t count, seed;
  float steps;
  float cs[4];
  float fallback[2];
};

// particles_update.wgsl:46-60
__global__ void particles_kernel(Field f, ParticleParams P, float4 *rec) {
  uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= P.count) return;
  float4 pos = rec[2 * id], prev = rec[2 * id + 1];
  float3 v = velocity3(f, pos.x, pos.y, pos.z);
  float dx = v.x * P.steps, dy = v.y * P.steps, dz = v.z * P.steps;
  float l = fmaxf(1.0f, len3(dx, dy, dz));
  dx /= l; dy /= l; dz /= l;
  float qx = pos.x + dx, qy = pos.y + dy, qz = pos.z + dz;
  float age = pos.w + 1.0f;
  if (qx >= (float)(f.nx - 2u) || !fluid3(f, qx, qy, qz) || age > 4000.0f) {
    float generation = prev.w + 1.0f;
    uint32_t h = hash32(id + P.seed + (uint32_t)generation * 0x9e3779b9u);
    float r0 = (float)(h >> 8) / 16777216.0f, r1 = (float)(hash32(h) >> 8) / 16777216.0f;
    float py = mixf(P.cs[0], P.cs[2], r0), pz = mixf(P.cs[1], P.cs[3], r1);
    if (!fluid3(f, 2.0f, py, pz)) { py = P.fallback[0]; pz = P.fallback[1]; }
    rec[2 * id] = make_float4(2.0f, py, pz, 0.0f);
    rec[2 * id + 1] = make_float4(2.0f, py, pz, generation);
  } else {
    rec[2 * id] = make_float4(qx, qy, qz, age);
    rec[2 * id + 1] = make_float4(pos.x, pos.y, pos.z, prev.w);
  }
}

// ---------------------------------------------------------------- plate_smoke.wgsl
struct PlateParams {
  uint32_t nx, ny, nz, plane;
  uint32_t threads, slots, release, releasing;
  float rake[4];
  uint32_t nports;
};

struct Plate {
  const float4 *macros;
  const uint32_t *flags;
  PlateParams s;
  __device__ __forceinline__ uint32_t cell(uint32_t x, uint32_t z) const { return x + s.nx * (s.plane + s.ny * z); }
  __device__ bool solid(float px, float pz) const {
    if (px < 0.f || pz < 0.f || px > (float)(s.nx - 1u) || pz > (float)(s.nz - 1u)) return true;
    uint32_t x = (uint32_t)floorf(px + 0.5f), z = (uint32_t)floorf(pz + 0.5f);
    return (flags[cell(x, z)] & 7u) != 0u;
  }
  __device__ float2 velocity(float px, float pz) const {
    float qx = clampf(px, 0.f, (float)(s.nx - 2u)), qz = clampf(pz, 0.f, (float)(s.nz - 2u));
    uint32_t lx = (uint32_t)floorf(qx), lz = (uint32_t)floorf(qz);
    float fx = qx - (float)lx, fz = qz - (float)lz;
    float4 a = macros[cell(lx, lz)], b = macros[cell(lx + 1u, lz)];
    float4 c = macros[cell(lx, lz + 1u)], d = macros[cell(lx + 1u, lz + 1u)];
    return make_float2(mixf(mixf(a.y, b.y, fx), mixf(c.y, d.y, fx), fz),
                       mixf(mixf(a.w, b.w, fx), mixf(c.w, d.w, fx), fz));
  }
  // plate_smoke.wgsl:37-54
  __device__ void carry(float &x, float &z, float &density, float h, float settle) const {
    float2 first = velocity(x, z);
    float2 mid = velocity(x + 0.5f * h * first.x, z + 0.5f * h * first.y);
    float sx = h * mid.x, sz = h * mid.y;
    float l = fmaxf(1.0f, sqrtf(sx * sx + sz * sz));
    sx /= l; sz /= l;
    float nx_ = x + sx, nz_ = z + sz;
    if (solid(nx_, nz_)) {
      density *= settle;
      if (!solid(nx_, z)) nz_ = z;
      else if (!solid(x, nz_)) nx_ = x;
      else { nx_ = -1.0f; nz_ = -1.0f; }
    }
    x = nx_; z = nz_;
  }
};

__global__ void plate_kernel(Plate pl, float4 *smoke, const float2 *ports) {
  const PlateParams &s = pl.s;
  uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= s.threads * s.slots) return;
  uint32_t thread = id / s.slots;
  if (s.releasing == 1u && id % s.slots == s.release % s.slots) {
    uint32_t rake = s.threads - s.nports;
    if (thread < rake) {
      float height = mixf(s.rake[1], s.rake[2], (float)thread / (float)(max(rake, 2u) - 1u));
      smoke[id] = make_float4(s.rake[0], height, (float)s.release, 1.0f);
    } else {
      float2 port = ports[thread - rake];
      smoke[id] = make_float4(port.x, port.y, (float)s.release, port.x >= 0.0f ? 1.0f : 0.0f);
    }
    return;
  }
  float4 puff = smoke[id];
  if (puff.w == 0.0f) return;
  float h = s.rake[3];
  float2 u = pl.velocity(puff.x, puff.y);
  uint32_t count = (uint32_t)clampf(ceilf(2.0f * h * sqrtf(u.x * u.x + u.y * u.y)), 1.0f, 16.0f);
  float settle = powf(0.85f, 1.0f / (float)count);
  float x = puff.x, z = puff.y, density = puff.w;
  for (uint32_t i = 0; i < count && x >= 0.0f; i++) pl.carry(x, z, density, h / (float)count, settle);
  bool finite = x == x && z == z && density == density;
  bool alive = finite && x >= 0.0f && x < (float)(s.nx - 2u) && density > 0.02f;
  smoke[id] = make_float4(x, z, puff.z, alive ? density : 0.0f);
}

// ---------------------------------------------------------------- 3-D streaklines
struct StreakParams {
  uint32_t ry, rz, slots, release, releasing;
  float rake[5];
  float h;
};

__device__ bool solid3(const Field &f, float px, float py, float pz) {
  if (px < 0.f || py < 0.f || pz < 0.f) return true;
  if (px > (float)(f.nx - 1u) || py > (float)(f.ny - 1u) || pz > (float)(f.nz - 1u)) return true;
  uint32_t x = (uint32_t)floorf(px + 0.5f), y = (uint32_t)floorf(py + 0.5f), z = (uint32_t)floorf(pz + 0.5f);
  return (f.flags[f.cell(x, y, z)] & 7u) != 0u;
}

__device__ void carry3(const Field &f, float st[4], float h, float settle) {
  float3 first = velocity3(f, st[0], st[1], st[2]);
  float3 mid = velocity3(f, st[0] + 0.5f * h * first.x, st[1] + 0.5f * h * first.y, st[2] + 0.5f * h * first.z);
  float sx = h * mid.x, sy = h * mid.y, sz = h * mid.z;
  float l = fmaxf(1.0f, len3(sx, sy, sz));
  sx /= l; sy /= l; sz /= l;
  float next[3] = {st[0] + sx, st[1] + sy, st[2] + sz};
  float density = st[3];
  if (solid3(f, next[0], next[1], next[2])) {
    density *= settle;
    // keep two components (drop z, then y, then x), then one, as the slide candidates
    const uint8_t keep[6][3] = {{1, 1, 0}, {1, 0, 1}, {0, 1, 1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    bool moved = false;
    for (int k = 0; k < 6 && !moved; k++) {
      float c0 = keep[k][0] ? next[0] : st[0], c1 = keep[k][1] ? next[1] : st[1], c2 = keep[k][2] ? next[2] : st[2];
      if (!solid3(f, c0, c1, c2)) { next[0] = c0; next[1] = c1; next[2] = c2; moved = true; }
    }
    if (!moved) { next[0] = -1.0f; next[1] = -1.0f; next[2] = -1.0f; }
  }
  st[0] = next[0]; st[1] = next[1]; st[2] = next[2]; st[3] = density;
}

__global__ void streak_kernel(Field f, StreakParams P, float4 *puffs, uint32_t *release_of) {
  uint32_t threads = P.ry * P.rz;
  uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= threads * P.slots) return;
  uint32_t thread = id / P.slots;
  if (P.releasing && id % P.slots == P.release % P.slots) {
    uint32_t iy = thread % P.ry, iz = thread / P.ry;
    float ty = (float)iy / (float)(max(P.ry, 2u) - 1u);
    float tz = (float)iz / (float)(max(P.rz, 2u) - 1u);
    puffs[id] = make_float4(P.rake[0], mixf(P.rake[1], P.rake[2], ty), mixf(P.rake[3], P.rake[4], tz), 1.0f);
    release_of[id] = P.release;
    return;
  }
  float4 p = puffs[id];
  if (p.w == 0.0f) return;
  float3 u = velocity3(f, p.x, p.y, p.z);
  uint32_t count = (uint32_t)clampf(ceilf(2.0f * P.h * len3(u.x, u.y, u.z)), 1.0f, 16.0f);
  float settle = powf(0.85f, 1.0f / (float)count);
  float st[4] = {p.x, p.y, p.z, p.w};
  for (uint32_t i = 0; i < count && st[0] >= 0.0f; i++) carry3(f, st, P.h / (float)count, settle);
  bool finite = st[0] == st[0] && st[1] == st[1] && st[2] == st[2] && st[3] == st[3];
  bool alive = finite && st[0] >= 0.0f && st[0] < (float)(f.nx - 2u) && st[3] > 0.02f;
  puffs[id] = make_float4(st[0], st[1], st[2], alive ? st[3] : 0.0f);
}

}  // namespace

struct pw_particles {
  pw_domain *dom;
  Field field;
  ParticleParams P;
  float4 *rec = nullptr;
  cudaStream_t stream;
};

struct pw_plate_smoke {
  pw_domain *dom;
  Plate plate;
  float4 *smoke = nullptr;
  float2 *ports = nullptr;
  cudaStream_t stream;
};

struct pw_streaks {
  pw_domain *dom;
  Field field;
  StreakParams P;
  float4 *puffs = nullptr;
  uint32_t *release_of = nullptr;
  cudaStream_t stream;
};

static int field_of(pw_domain *dom, Field *f, cudaStream_t *s) {
  void *macros = nullptr, *flags = nullptr, *stream = nullptr;
  int rc = pw_domain_buffers(dom, &macros, &flags, &stream);
  if (rc != PW_OK) return rc;
  domain_dims(dom, &f->nx, &f->ny, &f->nz);
  f->macros = (const float4 *)macros;
  f->flags = (const uint32_t *)flags;
  *s = (cudaStream_t)stream;
  return PW_OK;
}

extern "C" {

int pw_particles_create(pw_domain *dom, const float *records, uint32_t count, uint32_t seed,
                        const float cs[4], const float fallback[2], pw_particles **out) {
  if (!dom || !records || !cs || !fallback || !out || count == 0) { set_error("invalid particle arguments"); return PW_ERR_INVALID; }
  *out = nullptr;
  pw_particles *p = new pw_particles();
  p->dom = dom;
  int rc = field_of(dom, &p->field, &p->stream);
  if (rc != PW_OK) { delete p; return rc; }
  cudaError_t e = cudaMalloc(&p->rec, (size_t)count * 32);
  if (e != cudaSuccess) { delete p; return cuda_status(e, "pw_particles_create"); }
  p->P.count = count;
  p->P.seed = seed;
  for (int k = 0; k < 4; k++) p->P.cs[k] = cs[k];
  p->P.fallback[0] = fallback[0];
  p->P.fallback[1] = fallback[1];
  *out = p;
  return pw_particles_write(p, records);
}

int pw_particles_write(pw_particles *p, const float *records) {
  if (!p || !records) { set_error("NULL argument"); return PW_ERR_INVALID; }
  PW_TRY(cudaMemcpyAsync(p->rec, records, (size_t)p->P.count * 32, cudaMemcpyHostToDevice, p->stream));
  PW_TRY(cudaStreamSynchronize(p->stream));
  return PW_OK;
}

int pw_particles_update(pw_particles *p, float steps) {
  if (!p || !(steps >= 0.0f)) { set_error("Particle advection needs non-negative finite solver steps."); return PW_ERR_INVALID; }
  p->P.steps = steps;
  particles_kernel<<<(p->P.count + 127) / 128, 128, 0, p->stream>>>(p->field, p->P, p->rec);
  PW_TRY(cudaGetLastError());
  return PW_OK;
}

int pw_particles_read(pw_particles *p, float *out) {
  if (!p || !out) { set_error("NULL argument"); return PW_ERR_INVALID; }
  PW_TRY(cudaMemcpyAsync(out, p->rec, (size_t)p->P.count * 32, cudaMemcpyDeviceToHost, p->stream));
  PW_TRY(cudaStreamSynchronize(p->stream));
  return PW_OK;
}

void pw_particles_destroy(pw_particles *p) {
  if (!p) return;
  // cudaFree waits for pending work; the owning domain (and its stream) may be gone.
  cudaFree(p->rec);
  delete p;
}

int pw_plate_create(pw_domain *dom, uint32_t plane, uint32_t rake_threads, uint32_t slots, const float *ports,
                    uint32_t nports, pw_plate_smoke **out) {
  if (!dom || !out || slots == 0 || (nports && !ports)) { set_error("invalid plate arguments"); return PW_ERR_INVALID; }
  *out = nullptr;
  pw_plate_smoke *s = new pw_plate_smoke();
  s->dom = dom;
  Field f;
  int rc = field_of(dom, &f, &s->stream);
  if (rc != PW_OK) { delete s; return rc; }
  s->plate.macros = f.macros;
  s->plate.flags = f.flags;
  s->plate.s.nx = f.nx; s->plate.s.ny = f.ny; s->plate.s.nz = f.nz;
  if (plane >= f.ny) { delete s; set_error("Smoke needs a plane inside the grid and a release index below 2^24."); return PW_ERR_INVALID; }
  s->plate.s.plane = plane;
  s->plate.s.threads = rake_threads + nports;
  s->plate.s.slots = slots;
  s->plate.s.nports = nports;
  size_t n = (size_t)s->plate.s.threads * slots;
  cudaError_t e = cudaMalloc(&s->smoke, n * 16);
  if (e == cudaSuccess) e = cudaMalloc(&s->ports, (nports ? nports : 1) * 8);
  if (e == cudaSuccess) e = cudaMemsetAsync(s->smoke, 0, n * 16, s->stream);
  if (e == cudaSuccess && nports) e = cudaMemcpyAsync(s->ports, ports, (size_t)nports * 8, cudaMemcpyHostToDevice, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) { cudaFree(s->smoke); cudaFree(s->ports); delete s; return cuda_status(e, "pw_plate_create"); }
  *out = s;
  return PW_OK;
}

int pw_plate_advance(pw_plate_smoke *s, uint32_t release, int releasing, const float rake[4]) {
  if (!s || !rake) { set_error("NULL argument"); return PW_ERR_INVALID; }
  if (release >= (1u << 24) || !(rake[3] >= 0.0f)) {
    set_error("Smoke needs a plane inside the grid and a release index below 2^24.");
    return PW_ERR_INVALID;
  }
  s->plate.s.release = release;
  s->plate.s.releasing = releasing ? 1u : 0u;
  for (int k = 0; k < 4; k++) s->plate.s.rake[k] = rake[k];
  size_t n = (size_t)s->plate.s.threads * s->plate.s.slots;
  plate_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s->stream>>>(s->plate, s->smoke, s->ports);
  PW_TRY(cudaGetLastError());
  return PW_OK;
}

int pw_plate_read(pw_plate_smoke *s, float *out) {
  if (!s || !out) { set_error("NULL argument"); return PW_ERR_INVALID; }
  size_t n = (size_t)s->plate.s.threads * s->plate.s.slots;
  PW_TRY(cudaMemcpyAsync(out, s->smoke, n * 16, cudaMemcpyDeviceToHost, s->stream));
  PW_TRY(cudaStreamSynchronize(s->stream));
  return PW_OK;
}

void pw_plate_destroy(pw_plate_smoke *s) {
  if (!s) return;
  cudaFree(s->smoke);
  cudaFree(s->ports);
  delete s;
}

int pw_streaks_create(pw_domain *dom, uint32_t ry, uint32_t rz, uint32_t slots, const float rake[5], pw_streaks **out) {
  if (!dom || !rake || !out || ry == 0 || rz == 0 || slots == 0) { set_error("invalid streak arguments"); return PW_ERR_INVALID; }
  *out = nullptr;
  pw_streaks *s = new pw_streaks();
  s->dom = dom;
  int rc = field_of(dom, &s->field, &s->stream);
  if (rc != PW_OK) { delete s; return rc; }
  s->P.ry = ry; s->P.rz = rz; s->P.slots = slots;
  for (int k = 0; k < 5; k++) s->P.rake[k] = rake[k];
  size_t n = (size_t)ry * rz * slots;
  cudaError_t e = cudaMalloc(&s->puffs, n * 16);
  if (e == cudaSuccess) e = cudaMalloc(&s->release_of, n * 4);
  if (e == cudaSuccess) e = cudaMemsetAsync(s->puffs, 0, n * 16, s->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(s->release_of, 0, n * 4, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) { cudaFree(s->puffs); cudaFree(s->release_of); delete s; return cuda_status(e, "pw_streaks_create"); }
  *out = s;
  return PW_OK;
}

int pw_streaks_advance(pw_streaks *s, float h_steps, uint32_t release, int releasing) {
  if (!s || !(h_steps >= 0.0f)) { set_error("Streaklines need non-negative finite solver steps."); return PW_ERR_INVALID; }
  s->P.h = h_steps;
  s->P.release = release;
  s->P.releasing = releasing ? 1u : 0u;
  size_t n = (size_t)s->P.ry * s->P.rz * s->P.slots;
  streak_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s->stream>>>(s->field, s->P, s->puffs, s->release_of);
  PW_TRY(cudaGetLastError());
  return PW_OK;
}

int pw_streaks_read(pw_streaks *s, float *puffs, uint32_t *release_of) {
  if (!s || !puffs) { set_error("NULL argument"); return PW_ERR_INVALID; }
  size_t n = (size_t)s->P.ry * s->P.rz * s->P.slots;
  PW_TRY(cudaMemcpyAsync(puffs, s->puffs, n * 16, cudaMemcpyDeviceToHost, s->stream));
  if (release_of) PW_TRY(cudaMemcpyAsync(release_of, s->release_of, n * 4, cudaMemcpyDeviceToHost, s->stream));
  PW_TRY(cudaStreamSynchronize(s->stream));
  return PW_OK;
}

void pw_streaks_destroy(pw_streaks *s) {
  if (!s) return;
  cudaFree(s->puffs);
  cudaFree(s->release_of);
  delete s;
}

}  // extern "C"
