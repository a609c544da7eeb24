// Fused D3Q19 stream-collide with in-place AA streaming, momentum-exchange drag,
// density guard and outlet plane, for one GB300 (sm_103a).
//
// Included twice: by pw_kernels_fast.cu (PW_STRICT 0, compiled with fused
// multiply-add and hand-simplified moment algebra) and by pw_kernels_strict.cu
// (PW_STRICT 1, compiled with -fmad=false and the reference's own expression
// order, so its binary32 results equal a binary32 restatement bit for bit).
//
// Semantics follow the reference's pull kernel src/lbm/shaders/stream_collide.wgsl
// (one dispatch per step, A/B ping-pong, src/lbm/gpu-solver.ts:378-395).  The
// storage pattern is GB300-first instead: ONE population array updated in place.
//
//   P_t(j, n) = post-collision population j of cell n after step t.
//   Even t ("layout E"): P_t(j, n) at slot opp(j) of cell n.
//   Odd  t ("layout O"): P_t(j, n) at slot j of cell n + c_j (pre-streamed).
//   Odd step  (reads E): g_i(n) = slot opp(i) of n - c_i; writes P(j,n) to slot j of n + c_j.
//   Even step (reads O): g_i(n) = slot i of n;            writes P(j,n) to slot opp(j) of n.
// Each cell reads exactly the slots it writes, so the update is race free.
// Halfway bounce-back: a wall cell w never runs, so its slots keep what was
// pushed into them.  For a fluid cell n with wall link i (w = n - c_i) the pull
// needs P_prev(opp(i), n), which the AA pattern leaves in a slot no cell rewrites
// during the step that reads it: after an odd step it is the slot opp(i) of w
// (n's own push), after an even step the slot i of n (n's own write).  So a
// boundary cell reads those two slots for its wall links and otherwise streams
// as every other cell; nothing is written twice and walls are never written.
// The pressure outlet reads its upstream cell's previous state, which the AA
// update overwrites concurrently, so cells at x = nx-2 publish their velocity
// (computed exactly as stream_collide.wgsl:83-93 does from the stored codes)
// into a double-buffered (ny*nz) plane that the next step's outlet reads.
#include "pw_common.cuh"
#include "pw_launch.h"

#ifndef PW_NS
#error "define PW_NS before including pw_lbm.cuh"
#endif

namespace PW_NS {
using namespace pw;

constexpr int BX = kBlockX;
constexpr int BY = kBlockY;
constexpr int NTHREADS = BX * BY;

// ---------------------------------------------------------------- reference-order math
__device__ __forceinline__ float dot3(float ax, float ay, float az, float bx, float by, float bz) {
  return (ax * bx + ay * by) + az * bz;
}

// common.wgsl:84-88
__device__ __forceinline__ float geq_ref(int i, float rd, float vx, float vy, float vz) {
  float cu = dot3((float)cx_of(i), (float)cy_of(i), (float)cz_of(i), vx, vy, vz);
  float uu = dot3(vx, vy, vz, vx, vy, vz);
  return w_of(i) * (rd + (1.0f + rd) * (3.0f * cu + 4.5f * cu * cu - 1.5f * uu));
}

struct Stress { float xx, yy, zz, xy, xz, yz; };

// common.wgsl:100-113
__device__ __forceinline__ Stress neq_stress_ref(const float *g, const float *eq) {
  Stress s = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
  for (int i = 0; i < 19; i++) {
    float cx = (float)cx_of(i), cy = (float)cy_of(i), cz = (float)cz_of(i);
    float neq = g[i] - eq[i];
    s.xx += cx * cx * neq;
    s.yy += cy * cy * neq;
    s.zz += cz * cz * neq;
    s.xy += cx * cy * neq;
    s.xz += cx * cz * neq;
    s.yz += cy * cz * neq;
  }
  return s;
}

// common.wgsl:115-122
template <bool LES>
__device__ __forceinline__ float relaxation_time_ref(const StepParams &p, const float *g,
                                                     const float *eq, float rho) {
  float tau0 = 3.0f * p.nu + 0.5f;
  if (!LES) return tau0;
  Stress pi = neq_stress_ref(g, eq);
  float q = pi.xx * pi.xx + pi.yy * pi.yy + pi.zz * pi.zz +
            2.0f * (pi.xy * pi.xy + pi.xz * pi.xz + pi.yz * pi.yz);
  return 0.5f * (tau0 + sqrtf(tau0 * tau0 + p.cs_term * sqrtf(q) / rho));
}

// collide-trt.wgsl:1-15, collide-reg.wgsl:3-18
template <int OP, bool LES>
__device__ __forceinline__ void collide_ref(const StepParams &p, const float *g, const float *eq,
                                            float rho, float *post) {
  float tau = relaxation_time_ref<LES>(p, g, eq, rho);
  float omega_plus = 1.0f / tau;
  if (OP == OP_REG) {
    Stress pi = neq_stress_ref(g, eq);
    float trace = pi.xx + pi.yy + pi.zz;
#pragma unroll
    for (int i = 0; i < 19; i++) {
      float cx = (float)cx_of(i), cy = (float)cy_of(i), cz = (float)cz_of(i);
      float projected = cx * cx * pi.xx + cy * cy * pi.yy + cz * cz * pi.zz +
                        2.0f * (cx * cy * pi.xy + cx * cz * pi.xz + cy * cz * pi.yz) - trace / 3.0f;
      post[i] = eq[i] + (1.0f - omega_plus) * 4.5f * w_of(i) * projected;
    }
  } else {
    float omega_minus = 1.0f / (p.lambda / (tau - 0.5f) + 0.5f);
    post[0] = g[0] - omega_plus * (g[0] - eq[0]);
#pragma unroll
    for (int i = 1; i < 19; i += 2) {
      int j = i + 1;
      float even = 0.5f * omega_plus * (g[i] + g[j] - eq[i] - eq[j]);
      float odd = 0.5f * omega_minus * (g[i] - g[j] - eq[i] + eq[j]);
      post[i] = g[i] - even - odd;
      post[j] = g[j] - even + odd;
    }
  }
}

// stream_collide.wgsl:8-12
__device__ __forceinline__ float friction_velocity(const StepParams &p, float speed) {
  const float WALL_A = 8.3f, WALL_SUBLAYER = 11.81f, WALL_DISTANCE = 0.5f;
  const float WALL_B = 0.142857149243354797f;  // binary32 of 1/7
  float viscous = sqrtf(p.nu * speed / WALL_DISTANCE);
  if (WALL_DISTANCE * viscous / p.nu <= WALL_SUBLAYER) return viscous;
  return powf(speed * powf(p.nu / WALL_DISTANCE, WALL_B) / WALL_A, 1.0f / (1.0f + WALL_B));
}

// stream_collide.wgsl:18-80 (the LES wall cell), reference order in both builds.
template <int OP>
__device__ void collide_wall_ref(const StepParams &p, const float *g, const float *eq, float rho,
                                 float vx, float vy, float vz, uint32_t flag, float *post) {
  float nx_ = 0.f, ny_ = 0.f, nz_ = 0.f, exposed = 0.f;
#pragma unroll
  for (int i = 1; i < 19; i++) {
    if (flag & (1u << (3 + i))) {
      nx_ += w_of(i) * (float)cx_of(i);
      ny_ += w_of(i) * (float)cy_of(i);
      nz_ += w_of(i) * (float)cz_of(i);
      exposed += w_of(i);
    }
  }
  float sx = vx, sy = vy, sz = vz;
  float normal_length = sqrtf(dot3(nx_, ny_, nz_, nx_, ny_, nz_));
  if (normal_length > 1e-3f) {
    float ux = nx_ / normal_length, uy = ny_ / normal_length, uz = nz_ / normal_length;
    float d = dot3(vx, vy, vz, ux, uy, uz);
    sx -= d * ux;
    sy -= d * uy;
    sz -= d * uz;
  }
  float speed = sqrtf(dot3(sx, sy, sz, sx, sy, sz));
  if (speed < 1e-7f) { collide_ref<OP, true>(p, g, eq, rho, post); return; }
  float tx = sx / speed, ty = sy / speed, tz = sz / speed;
  float u_tau = friction_velocity(p, speed);
  float shear = 6.0f * exposed * rho * u_tau * u_tau;
  float flux = 0.f;
  Stress b = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  const float third = 0.333333343267440796f;
#pragma unroll
  for (int i = 1; i < 19; i++) {
    if (!(flag & (1u << (3 + i)))) continue;
    const int j = opp_of(i);
    float cx = (float)cx_of(j), cy = (float)cy_of(j), cz = (float)cz_of(j);
    float along = dot3(cx, cy, cz, tx, ty, tz);
    flux += 2.0f * along * (eq[j] + w_of(j));
    float sj = 9.0f * w_of(j) * along;
    b.xx += sj * (cx * cx - third);
    b.yy += sj * (cy * cy - third);
    b.zz += sj * (cz * cz - third);
    b.xy += sj * cx * cy;
    b.xz += sj * cx * cz;
    b.yz += sj * cy * cz;
  }
  float norm = b.xx * b.xx + b.yy * b.yy + b.zz * b.zz + 2.0f * (b.xy * b.xy + b.xz * b.xz + b.yz * b.yz);
  if (norm < 0.05f) { collide_ref<OP, true>(p, g, eq, rho, post); return; }
  float scale = 4.5f * (shear - flux) / norm;
  float trace = b.xx + b.yy + b.zz;
#pragma unroll
  for (int i = 0; i < 19; i++) {
    float cx = (float)cx_of(i), cy = (float)cy_of(i), cz = (float)cz_of(i);
    float projected = cx * cx * b.xx + cy * cy * b.yy + cz * cz * b.zz +
                      2.0f * (cx * cy * b.xy + cx * cz * b.xz + cy * cz * b.yz) - trace / 3.0f;
    post[i] = eq[i] + scale * w_of(i) * projected;
  }
#pragma unroll
  for (int i = 0; i < 19; i++) {
    if (post[i] + w_of(i) < 0.0f) { collide_ref<OP, true>(p, g, eq, rho, post); return; }
  }
}

// Full reference-order cell update: moments, equilibrium, collision
// (stream_collide.wgsl:114-133).  Returns rho and velocity for macros.
template <int OP, bool LES>
__device__ __forceinline__ void update_ref(const StepParams &p, const float *g, uint32_t flag,
                                           float *post, float &rho, float &vx, float &vy, float &vz) {
  float rd = 0.f, mx = 0.f, my = 0.f, mz = 0.f;
#pragma unroll
  for (int i = 0; i < 19; i++) {
    rd += g[i];
    mx += (float)cx_of(i) * g[i];
    my += (float)cy_of(i) * g[i];
    mz += (float)cz_of(i) * g[i];
  }
  rho = 1.0f + rd;
  vx = mx / rho;
  vy = my / rho;
  vz = mz / rho;
  float eq[19];
#pragma unroll
  for (int i = 0; i < 19; i++) eq[i] = geq_ref(i, rd, vx, vy, vz);
  if (LES && (flag >> 3) != 0u) collide_wall_ref<OP>(p, g, eq, rho, vx, vy, vz, flag, post);
  else collide_ref<OP, LES>(p, g, eq, rho, post);
}

// ---------------------------------------------------------------- fast math
// Same operator, fewer instructions: moments from the sums s_k and differences
// d_k of the nine opposite pairs, equilibrium split into even/odd parts per pair,
// non-equilibrium stress from the second moment minus its closed-form
// equilibrium value (sum_i w_i c_a c_b g_eq,i = delta_ab rd/3 + rho u_a u_b),
// reciprocals and square roots from the hardware approximations (a few ulp).
// g holds populations in units of 1/scale (scale = 2^15 for f16 storage, so the
// stored codes enter without a multiply); outputs are written back in those units.
//
// Pairs k = 1..9 are directions (2k-1, 2k) with velocities
// x, y, z, x+y, x+z, y+z, x-y, x-z, y-z.
// A relaxation-time hook of the LES branch: given the Smagorinsky relaxation
// time and the cell's state, return the relaxation time to use.  NoHook keeps
// Smagorinsky; the learned closure scales its eddy viscosity.
struct NoHook {
  __device__ __forceinline__ float operator()(const StepParams &, float tau_s, float, float, float, float, float,
                                              float, float, float, float, float) const {
    return tau_s;
  }
};

// Returns the cell's omega+ (binary32), which is finite exactly when the
// LES relaxation time is.
template <int OP, bool LES, class Hook = NoHook>
__device__ __forceinline__ float update_fast(const StepParams &p, float *g, float &rho, float &vx, float &vy,
                                             float &vz, const float scale = 1.0f, const float inv_scale = 1.0f,
                                             const Hook &hook = Hook()) {
  float s[10], d[10];
#pragma unroll
  for (int k = 1; k <= 9; k++) {
    s[k] = g[2 * k - 1] + g[2 * k];
    d[k] = g[2 * k - 1] - g[2 * k];
  }
  const float rd = ((g[0] + (s[1] + s[2] + s[3])) + ((s[4] + s[5] + s[6]) + (s[7] + s[8] + s[9]))) * inv_scale;
  const float jx = (d[1] + d[4]) + (d[5] + d[7]) + d[8];
  const float jy = (d[2] + d[4]) + (d[6] - d[7]) + d[9];
  const float jz = (d[3] + d[5]) + (d[6] - d[8]) - d[9];
  rho = 1.0f + rd;
  const float inv = __fdividef(1.0f, rho);
  const float vs = inv * inv_scale;
  vx = jx * vs;
  vy = jy * vs;
  vz = jz * vs;
  const float uu = vx * vx + vy * vy + vz * vz;
  const float K = rd - 1.5f * rho * uu;  // rd + rho(-1.5 uu): the cu-free part of the equilibrium
  float om_p = p.omega_plus, om_m = p.omega_minus;
  float pxx = 0.f, pyy = 0.f, pzz = 0.f, pxy = 0.f, pxz = 0.f, pyz = 0.f;
  if (LES || OP == OP_REG) {
    const float rd3 = rd * (1.0f / 3.0f);
    pxx = (s[1] + s[4] + s[5] + s[7] + s[8]) * inv_scale - (rd3 + rho * vx * vx);
    pyy = (s[2] + s[4] + s[6] + s[7] + s[9]) * inv_scale - (rd3 + rho * vy * vy);
    pzz = (s[3] + s[5] + s[6] + s[8] + s[9]) * inv_scale - (rd3 + rho * vz * vz);
    pxy = (s[4] - s[7]) * inv_scale - rho * vx * vy;
    pxz = (s[5] - s[8]) * inv_scale - rho * vx * vz;
    pyz = (s[6] - s[9]) * inv_scale - rho * vy * vz;
    if (LES) {
      const float q = pxx * pxx + pyy * pyy + pzz * pzz + 2.0f * (pxy * pxy + pxz * pxz + pyz * pyz);
      const float t0 = p.tau0;
      const float norm = q > 0.0f ? q * rsqrtf(q) : 0.0f;
      const float arg = t0 * t0 + p.cs_term * norm * inv;
      const float tau_plus = hook(p, 0.5f * (t0 + arg * rsqrtf(arg)), rho, vx, vy, vz, pxx, pyy, pzz, pxy, pxz, pyz);
      om_p = __fdividef(1.0f, tau_plus);
      om_m = __fdividef(1.0f, p.lambda * __fdividef(1.0f, tau_plus - 0.5f) + 0.5f);
    }
  }
  if (OP == OP_REG) {
    const float c = (1.0f - om_p) * 4.5f;
    const float tr3 = (pxx + pyy + pzz) * (1.0f / 3.0f);
    const float r3 = 3.0f * rho, r45 = 4.5f * rho;
    // rest
    g[0] = (w_of(0) * scale) * (K + c * (-tr3));
#define PW_REG_PAIR(I, CU, PROJ)                                        \
  {                                                                     \
    const float cu_ = (CU);                                             \
    const float ev_ = K + r45 * cu_ * cu_ + c * (PROJ);                 \
    const float od_ = r3 * cu_;                                         \
    g[I] = (w_of(I) * scale) * (ev_ + od_);                             \
    g[I + 1] = (w_of(I) * scale) * (ev_ - od_);                         \
  }
    PW_REG_PAIR(1, vx, pxx - tr3)
    PW_REG_PAIR(3, vy, pyy - tr3)
    PW_REG_PAIR(5, vz, pzz - tr3)
    PW_REG_PAIR(7, vx + vy, pxx + pyy + 2.0f * pxy - tr3)
    PW_REG_PAIR(9, vx + vz, pxx + pzz + 2.0f * pxz - tr3)
    PW_REG_PAIR(11, vy + vz, pyy + pzz + 2.0f * pyz - tr3)
    PW_REG_PAIR(13, vx - vy, pxx + pyy - 2.0f * pxy - tr3)
    PW_REG_PAIR(15, vx - vz, pxx + pzz - 2.0f * pxz - tr3)
    PW_REG_PAIR(17, vy - vz, pyy + pzz - 2.0f * pyz - tr3)
#undef PW_REG_PAIR
  } else {
    const float r3 = 3.0f * rho, r45 = 4.5f * rho;
    const float hp = 0.5f * om_p, hm = 0.5f * om_m;
    g[0] = g[0] - om_p * (g[0] - (w_of(0) * scale) * K);
#define PW_TRT_PAIR(I, CU)                                              \
  {                                                                     \
    const float cu_ = (CU);                                             \
    const float ep_ = (w_of(I) * scale) * (K + r45 * cu_ * cu_);        \
    const float em_ = (w_of(I) * scale) * (r3 * cu_);                   \
    const float a_ = hp * (s[(I + 1) / 2] - 2.0f * ep_);                \
    const float b_ = hm * (d[(I + 1) / 2] - 2.0f * em_);                \
    g[I] = g[I] - a_ - b_;                                              \
    g[I + 1] = g[I + 1] - a_ + b_;                                      \
  }
    PW_TRT_PAIR(1, vx)
    PW_TRT_PAIR(3, vy)
    PW_TRT_PAIR(5, vz)
    PW_TRT_PAIR(7, vx + vy)
    PW_TRT_PAIR(9, vx + vz)
    PW_TRT_PAIR(11, vy + vz)
    PW_TRT_PAIR(13, vx - vy)
    PW_TRT_PAIR(15, vx - vz)
    PW_TRT_PAIR(17, vy - vz)
#undef PW_TRT_PAIR
  }
  return om_p;
}

// ---------------------------------------------------------------- two cells at once
#if !PW_STRICT
// update_fast on two cells held as the .x and .y lanes of float2 values, with
// Blackwell's packed binary32 arithmetic (one FADD2 / FMUL2 / FFMA2 per two
// cells); the reciprocals and square roots stay per lane.  Same formulas and
// expression order as update_fast.
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, neg2(b)); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 rcp2(float2 a) { return make_float2(__fdividef(1.0f, a.x), __fdividef(1.0f, a.y)); }

// Lanes flagged in eq (bit 0: .x, bit 1: .y) come out at the equilibrium of
// rho 1 and velocity (eux, euy, euz) instead: their moments are replaced and
// their relaxation rates set to 1 before the reconstruction.  For TRT their
// loaded values are zeroed first: on odd steps an x-face EQ cell's c_x = +-1
// loads fall outside its row, on slots that another EQ cell may be writing in
// the same step, and TRT's s - (s - 2 e) would carry their rounding into the
// result (REG multiplies them by an exact zero).  Hook (LES) maps
// both lanes' Smagorinsky relaxation time to the one used, as update_fast's
// hook does for one cell; every thread of a block calls it once.
struct NoHook2 {
  __device__ __forceinline__ float2 operator()(const StepParams &, float2 tau_s, float2, float2, float2, float2,
                                               float2, float2, float2, float2, float2, float2) const {
    return tau_s;
  }
};

template <int OP, bool LES, class Hook = NoHook2>
__device__ __forceinline__ float2 update_fast2(const StepParams &p, float2 *g, float2 &rho, float2 &vx, float2 &vy,
                                               float2 &vz, const float scale, const float inv_scale, uint32_t eq,
                                               float2 eux, float2 euy, float2 euz, const Hook &hook = Hook()) {
  if constexpr (OP == OP_TRT) {
    if (eq) {
#pragma unroll
      for (int i = 0; i < 19; i++) {
        if (eq & 1u) g[i].x = 0.0f;
        if (eq & 2u) g[i].y = 0.0f;
      }
    }
  }
  float2 s[10], d[10];
#pragma unroll
  for (int k = 1; k <= 9; k++) {
    s[k] = add2(g[2 * k - 1], g[2 * k]);
    d[k] = sub2(g[2 * k - 1], g[2 * k]);
  }
  const float2 is = f2(inv_scale);
  float2 rd = mul2(add2(add2(g[0], add2(add2(s[1], s[2]), s[3])),
                        add2(add2(add2(s[4], s[5]), s[6]), add2(add2(s[7], s[8]), s[9]))),
                   is);
  if (eq & 1u) rd.x = 0.0f;
  if (eq & 2u) rd.y = 0.0f;
  const float2 jx = add2(add2(add2(d[1], d[4]), add2(d[5], d[7])), d[8]);
  const float2 jy = add2(add2(add2(d[2], d[4]), sub2(d[6], d[7])), d[9]);
  const float2 jz = sub2(add2(add2(d[3], d[5]), sub2(d[6], d[8])), d[9]);
  rho = add2(f2(1.0f), rd);
  const float2 inv = rcp2(rho);
  const float2 vs = mul2(inv, is);
  vx = mul2(jx, vs);
  vy = mul2(jy, vs);
  vz = mul2(jz, vs);
  if (eq & 1u) { vx.x = eux.x; vy.x = euy.x; vz.x = euz.x; }
  if (eq & 2u) { vx.y = eux.y; vy.y = euy.y; vz.y = euz.y; }
  const float2 uu = fma2(vx, vx, fma2(vy, vy, mul2(vz, vz)));
  const float2 K = fma2(mul2(f2(-1.5f), rho), uu, rd);
  float2 om_p = f2(p.omega_plus), om_m = f2(p.omega_minus);
  float2 pxx = f2(0.f), pyy = f2(0.f), pzz = f2(0.f), pxy = f2(0.f), pxz = f2(0.f), pyz = f2(0.f);
  if (LES || OP == OP_REG) {
    const float2 rd3 = mul2(rd, f2(1.0f / 3.0f));
    const float2 rvx = mul2(rho, vx), rvy = mul2(rho, vy), rvz = mul2(rho, vz);
    pxx = fma2(add2(add2(add2(s[1], s[4]), add2(s[5], s[7])), s[8]), is, neg2(fma2(rvx, vx, rd3)));
    pyy = fma2(add2(add2(add2(s[2], s[4]), add2(s[6], s[7])), s[9]), is, neg2(fma2(rvy, vy, rd3)));
    pzz = fma2(add2(add2(add2(s[3], s[5]), add2(s[6], s[8])), s[9]), is, neg2(fma2(rvz, vz, rd3)));
    pxy = fma2(sub2(s[4], s[7]), is, neg2(mul2(rvx, vy)));
    pxz = fma2(sub2(s[5], s[8]), is, neg2(mul2(rvx, vz)));
    pyz = fma2(sub2(s[6], s[9]), is, neg2(mul2(rvy, vz)));
    if (LES) {
      const float2 q = fma2(pxx, pxx, fma2(pyy, pyy, fma2(pzz, pzz, mul2(f2(2.0f),
                           fma2(pxy, pxy, fma2(pxz, pxz, mul2(pyz, pyz)))))));
      const float t0 = p.tau0;
      const float2 norm = make_float2(q.x > 0.0f ? q.x * rsqrtf(q.x) : 0.0f, q.y > 0.0f ? q.y * rsqrtf(q.y) : 0.0f);
      const float2 arg = fma2(f2(p.cs_term), mul2(norm, inv), f2(t0 * t0));
      const float2 tau_plus =
          hook(p, mul2(f2(0.5f), add2(f2(t0), make_float2(arg.x * rsqrtf(arg.x), arg.y * rsqrtf(arg.y)))), rho, vx,
               vy, vz, pxx, pyy, pzz, pxy, pxz, pyz);
      om_p = rcp2(tau_plus);
      om_m = rcp2(fma2(f2(p.lambda), rcp2(sub2(tau_plus, f2(0.5f))), f2(0.5f)));
    }
  }
  if (eq & 1u) { om_p.x = 1.0f; om_m.x = 1.0f; }
  if (eq & 2u) { om_p.y = 1.0f; om_m.y = 1.0f; }
  const float2 r3 = mul2(f2(3.0f), rho), r45 = mul2(f2(4.5f), rho);
  if (OP == OP_REG) {
    const float2 c = fma2(om_p, f2(-4.5f), f2(4.5f));
    const float2 tr3 = mul2(add2(add2(pxx, pyy), pzz), f2(1.0f / 3.0f));
    g[0] = mul2(f2(w_of(0) * scale), fma2(c, neg2(tr3), K));
#define PW_REG_PAIR2(I, CU, PROJ)                                       \
  {                                                                     \
    const float2 cu_ = (CU);                                            \
    const float2 ev_ = fma2(c, (PROJ), fma2(mul2(r45, cu_), cu_, K));   \
    const float2 od_ = mul2(r3, cu_);                                   \
    g[I] = mul2(f2(w_of(I) * scale), add2(ev_, od_));                   \
    g[I + 1] = mul2(f2(w_of(I) * scale), sub2(ev_, od_));               \
  }
    const float2 axx = sub2(pxx, tr3), ayy = sub2(pyy, tr3), azz = sub2(pzz, tr3);
    const float2 txy = sub2(add2(pxx, pyy), tr3), txz = sub2(add2(pxx, pzz), tr3), tyz = sub2(add2(pyy, pzz), tr3);
    PW_REG_PAIR2(1, vx, axx)
    PW_REG_PAIR2(3, vy, ayy)
    PW_REG_PAIR2(5, vz, azz)
    PW_REG_PAIR2(7, add2(vx, vy), fma2(f2(2.0f), pxy, txy))
    PW_REG_PAIR2(9, add2(vx, vz), fma2(f2(2.0f), pxz, txz))
    PW_REG_PAIR2(11, add2(vy, vz), fma2(f2(2.0f), pyz, tyz))
    PW_REG_PAIR2(13, sub2(vx, vy), fma2(f2(-2.0f), pxy, txy))
    PW_REG_PAIR2(15, sub2(vx, vz), fma2(f2(-2.0f), pxz, txz))
    PW_REG_PAIR2(17, sub2(vy, vz), fma2(f2(-2.0f), pyz, tyz))
#undef PW_REG_PAIR2
  } else {
    // TRT on the pair sums and differences: s' = s - om+ (s - 2 e+),
    // d' = d - om- (d - 2 e-), post = (s' +- d') / 2 (only g[0] is kept).
    g[0] = fma2(neg2(om_p), fma2(f2(-w_of(0) * scale), K, g[0]), g[0]);
#define PW_TRT_PAIR2(I, CU)                                             \
  {                                                                     \
    const float2 cu_ = (CU);                                            \
    const float2 ep_ = mul2(f2(w_of(I) * scale), fma2(mul2(r45, cu_), cu_, K)); \
    const float2 em_ = mul2(f2(w_of(I) * scale), mul2(r3, cu_));        \
    const float2 sp_ = fma2(neg2(om_p), fma2(f2(-2.0f), ep_, s[(I + 1) / 2]), s[(I + 1) / 2]); \
    const float2 dp_ = fma2(neg2(om_m), fma2(f2(-2.0f), em_, d[(I + 1) / 2]), d[(I + 1) / 2]); \
    g[I] = mul2(f2(0.5f), add2(sp_, dp_));                              \
    g[I + 1] = mul2(f2(0.5f), sub2(sp_, dp_));                          \
  }
    PW_TRT_PAIR2(1, vx)
    PW_TRT_PAIR2(3, vy)
    PW_TRT_PAIR2(5, vz)
    PW_TRT_PAIR2(7, add2(vx, vy))
    PW_TRT_PAIR2(9, add2(vx, vz))
    PW_TRT_PAIR2(11, add2(vy, vz))
    PW_TRT_PAIR2(13, sub2(vx, vy))
    PW_TRT_PAIR2(15, sub2(vx, vz))
    PW_TRT_PAIR2(17, sub2(vy, vz))
#undef PW_TRT_PAIR2
  }
  return om_p;
}

// The LES wall cell (stream_collide.wgsl:18-80) of cells whose only wall links
// are the five floor links (their pull sources lie at z - 1: a flat wall
// below), two cells at once, g in stored units.  For these links the wall
// normal is (0, 0, 1) and the exposed weight 1/18 + 4/36 = 1/6, the slip velocity is
// (ux, uy, 0) with unit tangent t, the link stress B has only the components
// B_xz = -tx/2 and B_yz = -ty/2 (|B|^2 = 1/2, trace 0), and the flux
// 2 sum_j (c_j . t)(eq_j + w_j) over the opposite links reduces to
// rho (1 - 3 uz) |u_t| / 3.  The post-collision state is then
//   eq_i - 9 (shear - flux) w_i c_iz (c_ix tx + c_iy ty),
// shear = 6 * (1/6) * rho * u_tau^2 (Werner-Wengle u_tau, stream_collide.wgsl:8-12).
__device__ __forceinline__ float floor_u_tau(const StepParams &p, float speed) {
  const float viscous = sqrtf(2.0f * p.nu * speed);  // sqrt(nu speed / y), y = 1/2
  if (0.5f * viscous <= 11.81f * p.nu) return viscous;
  return exp2f(p.wall_e * __log2f(speed * p.wall_c));  // (speed (nu/y)^B / A)^(1/(1+B))
}

// What a floor cell's post-collision state depends on: density, velocity,
// K = rd - 1.5 rho u.u, and the stress term along x and y (A tx, A ty).
struct FloorState {
  float2 rho, vx, vy, vz, K, atx, aty;
};

// The post-collision values of floor cells for the cells in `lanes` (bits 0
// and 1) into g, in stored units; returns the smallest f = g + w of each cell.
__device__ __forceinline__ float2 floor_post2(float2 *g, const FloorState &w, const float scale, uint32_t lanes) {
  const float2 r3 = mul2(f2(3.0f), w.rho), r45 = mul2(f2(4.5f), w.rho), z2 = f2(0.0f);
  float2 lo = f2(INFINITY);
  const auto put = [&](int i, float2 v) {
    if (lanes & 1u) g[i].x = v.x;
    if (lanes & 2u) g[i].y = v.y;
    lo = make_float2(fminf(lo.x, v.x + w_of(i) * scale), fminf(lo.y, v.y + w_of(i) * scale));
  };
  put(0, mul2(f2(w_of(0) * scale), w.K));
  // pair by pair: the equilibrium along cu, plus the stress term on the eight
  // sloped links:  9 = (1,0,1), 10 = (-1,0,-1): - A tx;  15 = (1,0,-1),
  // 16 = (-1,0,1): + A tx;  11 = (0,1,1), 12 = (0,-1,-1): - A ty;
  // 17 = (0,1,-1), 18 = (0,-1,1): + A ty
#define PW_FLOOR_PAIR(I, CU, EXTRA)                                         \
  {                                                                         \
    const float2 cu_ = (CU);                                                \
    const float2 ev_ = fma2(mul2(r45, cu_), cu_, w.K);                      \
    const float2 od_ = mul2(r3, cu_);                                       \
    put(I, fma2(f2(w_of(I) * scale), add2(ev_, od_), EXTRA));               \
    put(I + 1, fma2(f2(w_of(I) * scale), sub2(ev_, od_), EXTRA));           \
  }
  PW_FLOOR_PAIR(1, w.vx, z2)
  PW_FLOOR_PAIR(3, w.vy, z2)
  PW_FLOOR_PAIR(5, w.vz, z2)
  PW_FLOOR_PAIR(7, add2(w.vx, w.vy), z2)
  PW_FLOOR_PAIR(9, add2(w.vx, w.vz), neg2(w.atx))
  PW_FLOOR_PAIR(11, add2(w.vy, w.vz), neg2(w.aty))
  PW_FLOOR_PAIR(13, sub2(w.vx, w.vy), z2)
  PW_FLOOR_PAIR(15, sub2(w.vx, w.vz), w.atx)
  PW_FLOOR_PAIR(17, sub2(w.vy, w.vz), w.aty)
#undef PW_FLOOR_PAIR
  return lo;
}

// The wall-model post-collision state of both cells replaces g.  Returns in
// bits 0 and 1 the cells for which the reference keeps its plain collision
// instead (slip speed below 1e-7, or a population the stress would make
// negative, stream_collide.wgsl:39,76-77): the caller reloads and collides them.
__device__ __forceinline__ uint32_t floor_wall2(const StepParams &p, float2 *g, FloorState &w, const float scale,
                                                const float inv_scale) {
  float2 d[10], rs = g[0];
#pragma unroll
  for (int k = 1; k <= 9; k++) {
    rs = add2(rs, add2(g[2 * k - 1], g[2 * k]));
    d[k] = sub2(g[2 * k - 1], g[2 * k]);
  }
  const float2 is = f2(inv_scale);
  const float2 rd = mul2(rs, is);
  const float2 jx = add2(add2(add2(d[1], d[4]), add2(d[5], d[7])), d[8]);
  const float2 jy = add2(add2(add2(d[2], d[4]), sub2(d[6], d[7])), d[9]);
  const float2 jz = sub2(add2(add2(d[3], d[5]), sub2(d[6], d[8])), d[9]);
  w.rho = add2(f2(1.0f), rd);
  const float2 vs = mul2(rcp2(w.rho), is);
  w.vx = mul2(jx, vs);
  w.vy = mul2(jy, vs);
  w.vz = mul2(jz, vs);
  const float2 uu = fma2(w.vx, w.vx, fma2(w.vy, w.vy, mul2(w.vz, w.vz)));
  w.K = fma2(mul2(f2(-1.5f), w.rho), uu, rd);
  const float2 sp2 = fma2(w.vx, w.vx, mul2(w.vy, w.vy));
  uint32_t fb = 0u;
#pragma unroll
  for (int l = 0; l < 2; l++) {
    const float q = l ? sp2.y : sp2.x;
    const float sp = q > 0.0f ? q * rsqrtf(q) : 0.0f;
    const float r = l ? w.rho.y : w.rho.x, uz = l ? w.vz.y : w.vz.x;
    if (!(sp >= 1e-7f)) fb |= 1u << l;  // also a NaN speed
    const float inv = __fdividef(1.0f, sp);
    const float ut = floor_u_tau(p, sp);
    const float shear = r * ut * ut;
    const float flux = (1.0f / 3.0f) * r * (1.0f - 3.0f * uz) * sp;
    const float a = 9.0f * (shear - flux) * (w_of(7) * scale) * inv;
    if (l) { w.atx.y = a * w.vx.y; w.aty.y = a * w.vy.y; }
    else { w.atx.x = a * w.vx.x; w.aty.x = a * w.vy.x; }
  }
  const float2 lo = floor_post2(g, w, scale, 3u);
  if (!(lo.x >= 0.0f)) fb |= 1u;  // also a NaN state
  if (!(lo.y >= 0.0f)) fb |= 2u;
  return fb;
}

#endif

// ---------------------------------------------------------------- cell addressing
struct Nbr {
  uint32_t xm, x, xp;     // x - 1, x, x + 1 (periodic)
  uint32_t ym, y, yp;     // row offsets: (y-1)*nx, y*nx, (y+1)*nx
  uint32_t zm, z, zp;     // plane offsets
  bool sym, syp, szm, szp;  // the -y / +y / -z / +z neighbour lies beyond a free-slip face
  __device__ __forceinline__ uint32_t at(int dx, int dy, int dz) const {
    return (dx < 0 ? xm : (dx > 0 ? xp : x)) + (dy < 0 ? ym : (dy > 0 ? yp : y)) +
           (dz < 0 ? zm : (dz > 0 ? zp : z));
  }
  // Odd steps push P(j, n) into slot j of n + c_j; across a free-slip face the
  // population reflects: slot mirror(j) of the in-plane neighbour.  This is also
  // where P(j, n) sits after an odd step (the readout map).
  __device__ __forceinline__ pidx push(int j, uint32_t stride) const {
    const int cy = cy_of(j), cz = cz_of(j);
    const bool ry = (cy > 0 && syp) || (cy < 0 && sym);
    const bool rz = (cz > 0 && szp) || (cz < 0 && szm);
    const int k = ry ? (rz ? mirror_yz(j) : mirror_y(j)) : (rz ? mirror_z(j) : j);
    return (pidx)k * stride + at(cx_of(j), ry ? 0 : cy, rz ? 0 : cz);
  }
  // Odd steps pull direction i from slot opp(i) of n - c_i; across a free-slip
  // face from slot opp(mirror(i)) of the in-plane neighbour, where that
  // neighbour's even step left P(mirror(i)).
  __device__ __forceinline__ pidx pull(int i, uint32_t stride) const {
    const int cy = -cy_of(i), cz = -cz_of(i);
    const bool ry = (cy > 0 && syp) || (cy < 0 && sym);
    const bool rz = (cz > 0 && szp) || (cz < 0 && szm);
    const int k = ry ? (rz ? mirror_yz(i) : mirror_y(i)) : (rz ? mirror_z(i) : i);
    return (pidx)opp_of(k) * stride + at(-cx_of(i), ry ? 0 : cy, rz ? 0 : cz);
  }
};

__device__ __forceinline__ Nbr make_nbr(const StepParams &p, uint32_t x, uint32_t y, uint32_t z) {
  Nbr b;
  uint32_t plane = p.nx * p.ny;
  b.x = x;
  b.xm = x == 0 ? p.nx - 1 : x - 1;
  b.xp = x + 1 == p.nx ? 0 : x + 1;
  b.y = y * p.nx;
  b.ym = (y == 0 ? p.ny - 1 : y - 1) * p.nx;
  b.yp = (y + 1 == p.ny ? 0 : y + 1) * p.nx;
  b.z = z * plane;
  b.zm = (z == 0 ? p.nz - 1 : z - 1) * plane;
  b.zp = (z + 1 == p.nz ? 0 : z + 1) * plane;
  b.sym = (p.slip & 1u) && y == 0;
  b.syp = (p.slip & 1u) && y + 1 == p.ny;
  b.szm = (p.slip & 2u) && z == 0;
  b.szp = (p.slip & 2u) && z + 1 == p.nz;
  return b;
}

// Location of P(j, n) after a step of the given parity (the readout map).
template <bool ODD_LAYOUT>
__device__ __forceinline__ pidx slot_of(const Nbr &b, int j, uint32_t stride, uint32_t n) {
  if (ODD_LAYOUT) return b.push(j, stride);
  return (pidx)opp_of(j) * stride + n;
}

// The velocity the outlet takes from its upstream cell: stream_collide.wgsl:83-93
// evaluated on the stored codes of this cell's new state.
template <int ST>
__device__ __forceinline__ float4 outlet_velocity_of(const typename Store<ST>::T *codes) {
  float mass = 1.0f, mx = 0.f, my = 0.f, mz = 0.f;
#pragma unroll
  for (int i = 0; i < 19; i++) {
    float value = Store<ST>::decode(codes[i]);
    mass += value;
    mx += (float)cx_of(i) * value;
    my += (float)cy_of(i) * value;
    mz += (float)cz_of(i) * value;
  }
  return make_float4(mx / mass, my / mass, mz / mass, 0.f);
}

// Block reduction of the momentum exchange into this block's partial slot.
// Block reduction of the momentum exchange into partial slot `slot`; t is the
// thread's index in its block of NTHREADS.
__device__ __forceinline__ void reduce_force_at(bool any, double fx, double fy, double fz, double *partials,
                                                size_t slot, uint32_t t) {
  if (partials == nullptr) return;  // uniform: a kernel parameter
  if (!__syncthreads_or(any)) return;
  __shared__ double red[NTHREADS / 32][3];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    fx += __shfl_down_sync(0xffffffffu, fx, o);
    fy += __shfl_down_sync(0xffffffffu, fy, o);
    fz += __shfl_down_sync(0xffffffffu, fz, o);
  }
  if ((t & 31) == 0) { red[t >> 5][0] = fx; red[t >> 5][1] = fy; red[t >> 5][2] = fz; }
  __syncthreads();
  if (t == 0) {
    double a = 0, b = 0, c = 0;
#pragma unroll
    for (int w = 0; w < NTHREADS / 32; w++) { a += red[w][0]; b += red[w][1]; c += red[w][2]; }
    partials[3 * slot + 0] = a;
    partials[3 * slot + 1] = b;
    partials[3 * slot + 2] = c;
  }
}

// Block reduction of the momentum exchange into this block's partial slot.
__device__ __forceinline__ void reduce_force(bool any, double fx, double fy, double fz, double *partials) {
  size_t blk = blockIdx.x + (size_t)gridDim.x * (blockIdx.y + (size_t)gridDim.y * blockIdx.z);
  reduce_force_at(any, fx, fy, fz, partials, blk, threadIdx.x + BX * threadIdx.y);
}

// ---------------------------------------------------------------- interpolated walls
// wall_value (walls.wgsl:6-21) for every wall link of one fluid cell, in link-rank
// order.  On entry g[i] of a link holds the halfway value f*_j(n) (j = opp(i)) of
// the state being read, and g[j] holds f*_j(n + c_i) whenever n + c_i is fluid (it
// is then n's ordinary pull source for j in both parities); own(i, k) gives the
// cell's own f*_i(n).  Each link's value replaces g[i]; links into SOLID add
// c_j (f*_j(n) + value) of that state to fx..fz (force.wgsl:20-29).
template <class Own>
__device__ __forceinline__ void interpolated_links(const StepParams &p, const Nbr &b, uint32_t n, uint32_t flag,
                                                   float *g, const Own &own, double &fx, double &fy, double &fz,
                                                   bool &force_any) {
  const uint32_t base = __ldg(&p.qoff[n]);
  uint32_t k = base;
#pragma unroll
  for (int i = 1; i < 19; i++) {
    if (!(flag & (1u << (3 + i)))) continue;
    const int j = opp_of(i);
    const float reflected = g[i];
    float value = reflected;
    if (base != NO_Q) {
      const float q = __ldg(&p.q[k]);
      if (q != 0.5f) {
        if (q < 0.5f) {
          const uint32_t second = b.at(cx_of(i), cy_of(i), cz_of(i));
          if ((__ldg(&p.flags[second]) & 7u) == FLUID) value = 2.0f * q * reflected + (1.0f - 2.0f * q) * g[j];
        } else {
          value = (reflected + (2.0f * q - 1.0f) * own(i, k)) / (2.0f * q);
        }
      }
      k++;
    }
    const uint32_t w = b.at(-cx_of(i), -cy_of(i), -cz_of(i));
    if ((__ldg(&p.flags[w]) & 7u) == SOLID) {
      double term = (double)(reflected + value);
      fx += (double)cx_of(j) * term;
      fy += (double)cy_of(j) * term;
      fz += (double)cz_of(j) * term;
      force_any = true;
    }
    g[i] = value;
  }
}

template <int ST>
struct OwnFromHist {
  const typename Store<ST>::T *hist;
  __device__ __forceinline__ float operator()(int, uint32_t k) const { return Store<ST>::decode(hist[k]); }
};

// ---------------------------------------------------------------- the step
// One cell of a step.  ODD: this step reads layout E and writes layout O;
// otherwise the reverse.  flag is the cell's packed flags (0 for plain fluid).
template <int ST, int OP, bool LES, bool ODD, class Hook = NoHook>
__device__ __forceinline__ void general_cell(const StepParams &p, uint32_t x, uint32_t y, uint32_t z, uint32_t n,
                                             uint32_t flag, double &fx, double &fy, double &fz, bool &force_any,
                                             const Hook &hook = Hook()) {
  using S = Store<ST>;
  using T = typename S::T;
  T *f = reinterpret_cast<T *>(p.f);
  const uint32_t S_ = p.stride;
  const uint32_t kind = flag & 7u;
  if (is_wall_kind(kind)) return;
  const Nbr b = make_nbr(p, x, y, z);
  float post[19];
  float rho = 1.0f, vx = 0.f, vy = 0.f, vz = 0.f;
  if (kind == EQ) {
    // stream_collide.wgsl:102-107: inlet at u_in, outlet (x = nx-1 > 0) at rho 1
    // with the upstream velocity published by the previous step.
    vx = p.u_in;
    if (x == p.nx - 1 && x > 0) {
      float4 u = p.plane_in[y + p.ny * z];
      vx = u.x; vy = u.y; vz = u.z;
    }
#pragma unroll
    for (int i = 0; i < 19; i++) post[i] = geq_ref(i, 0.0f, vx, vy, vz);
    rho = 1.0f + 0.0f;
  } else {
    float g[19];
#pragma unroll
    for (int i = 0; i < 19; i++) {
      pidx src;
      if (ODD) src = b.pull(i, S_);
      else src = (pidx)i * S_ + n;
      if (i > 0 && (flag & (1u << (3 + i)))) {  // wall link i: the slot nobody rewrites this step
        if (ODD) src = (pidx)i * S_ + n;
        else src = (pidx)opp_of(i) * S_ + b.at(-cx_of(i), -cy_of(i), -cz_of(i));
      }
      g[i] = S::decode(f[src]);
    }
    if (p.qoff != nullptr && (flag >> 3) != 0u)
      interpolated_links(p, b, n, flag, g, OwnFromHist<ST>{reinterpret_cast<const T *>(p.hist)}, fx, fy, fz,
                         force_any);
#if PW_STRICT
    update_ref<OP, LES>(p, g, flag, post, rho, vx, vy, vz);
#else
    if (LES && (flag >> 3) != 0u) {
      update_ref<OP, LES>(p, g, flag, post, rho, vx, vy, vz);
    } else {
      update_fast<OP, LES, Hook>(p, g, rho, vx, vy, vz, 1.0f, 1.0f, hook);
#pragma unroll
      for (int i = 0; i < 19; i++) post[i] = g[i];
    }
#endif
    if (p.write_macro) {
      bool bad = !(rho >= 0.5f && rho <= 1.5f);  // also catches NaN
      if (bad) atomicOr(p.status, 1u);
    }
  }
  T code[19];
#pragma unroll
  for (int j = 0; j < 19; j++) code[j] = S::encode(post[j], (uint32_t)j, n);
#pragma unroll
  for (int j = 0; j < 19; j++) {
    pidx dst;
    if (ODD) dst = b.push(j, S_);
    else dst = (pidx)opp_of(j) * S_ + n;
    f[dst] = code[j];
  }
  if (p.qoff != nullptr && (flag >> 3) != 0u) {
    // keep this step's f*_i(n) of every wall link for the next step's wall values
    const uint32_t base = __ldg(&p.qoff[n]);
    if (base != NO_Q) {
      T *hist = reinterpret_cast<T *>(p.hist);
      uint32_t k = base;
#pragma unroll
      for (int i = 1; i < 19; i++)
        if (flag & (1u << (3 + i))) hist[k++] = code[i];
    }
  } else if (flag >> 3) {
    // SOLID links add 2 c_j g*_j to the drag (force.wgsl:20-29, halfway walls).
#pragma unroll
    for (int i = 1; i < 19; i++) {
      if (!(flag & (1u << (3 + i)))) continue;
      const int j = opp_of(i);
      const uint32_t w = b.at(-cx_of(i), -cy_of(i), -cz_of(i));
      if ((__ldg(&p.flags[w]) & 7u) == SOLID) {
        float v = S::decode(code[j]);
        double term = (double)(v + v);
        fx += (double)cx_of(j) * term;
        fy += (double)cy_of(j) * term;
        fz += (double)cz_of(j) * term;
        force_any = true;
      }
    }
  }
  if (p.write_macro) p.macros[n] = make_float4(rho, vx, vy, vz);
  if (x + 2 == p.nx) p.plane_out[y + p.ny * z] = outlet_velocity_of<ST>(code);
}

// Every cell, one per thread, 32 x 4 cells per block (the strict build's step).
template <int ST, int OP, bool LES, bool ODD>
__global__ void __launch_bounds__(NTHREADS) aa_step(StepParams p) {
  const uint32_t x = blockIdx.x * BX + threadIdx.x;
  const uint32_t y = blockIdx.y * BY + threadIdx.y;
  const uint32_t z = blockIdx.z;
  bool force_any = false;
  double fx = 0.0, fy = 0.0, fz = 0.0;
  if (x < p.nx && y < p.ny) {
    const uint32_t n = x + p.nx * (y + p.ny * z);
    const bool special = (__ldg(&p.special[n >> 5]) >> (n & 31u)) & 1u;
    const uint32_t flag = special ? __ldg(&p.flags[n]) : 0u;
    general_cell<ST, OP, LES, ODD>(p, x, y, z, n, flag, fx, fy, fz, force_any);
  }
  reduce_force(force_any, fx, fy, fz, p.partials);
}

#if !PW_STRICT
// The step of the fast build runs as two launches over disjoint cells; in the
// in-place pattern each cell reads and writes only its own slots, so the two
// commute.  aa_step_fast takes the plain cells (not special, 1 <= x <= nx-2):
// direction i is read from element n + ld[i] and written to element n + st[i],
// the arithmetic runs in stored units (populations times 2^15 for f16, so the
// codes enter and leave without a multiply), and 16-bit codes are rounded by
// encode_fast: the reference's unbiased dithering of the discarded bits, drawn
// from a cheaper hash.  EQ cells without wall links ride along in the same
// warps (their stores then share sectors with the row's plain cells).
// aa_step_edges takes the listed remaining cells (wall links, periodic x faces)
// through general_cell and owns the force.
template <int ST, int OP, bool LES, bool ODD>
__device__ __forceinline__ void plain_cell(const StepParams &p, uint32_t n, uint32_t x, uint32_t y, uint32_t z,
                                           const int64_t *ld, const int64_t *st) {
  using S = Store<ST>;
  using T = typename S::T;
  T *f = reinterpret_cast<T *>(p.f);
  float g[19];
#pragma unroll
  for (int i = 0; i < 19; i++) g[i] = S::raw(f[n + ld[i]]);
  float rho, vx, vy, vz;
  const float om = update_fast<OP, LES>(p, g, rho, vx, vy, vz, S::kScale, S::kInvScale);
  if (ST != STORE_F32 && !(fabsf(rho + om) < INFINITY)) {
    // a non-finite state is stored as NaN, as the reference's GPUs store it
#pragma unroll
    for (int j = 0; j < 19; j++) g[j] = __uint_as_float(0x7fc00000u);
  }
  const uint32_t nk = n * 0x9e3779b9u;
#pragma unroll
  for (int j = 0; j < 19; j++) f[n + st[j]] = S::encode_fast(g[j], dither_mul(j), nk);
  if (p.write_macro) {
    if (!(rho >= 0.5f && rho <= 1.5f)) atomicOr(p.status, 1u);
    p.macros[n] = make_float4(rho, vx, vy, vz);
  }
  if (x + 2 == p.nx) {
    // the outlet's upstream plane publishes the velocity of its stored codes
    // (outlet_velocity_of, accumulated as they are read back)
    // (addresses from the readout map, so the store addresses need not stay live)
    const Nbr b = make_nbr(p, x, y, z);
    float mass = 1.0f, mx = 0.f, my = 0.f, mz = 0.f;
#pragma unroll
    for (int j = 0; j < 19; j++) {
      const float v = S::decode(f[slot_of<ODD>(b, j, p.stride, n)]);
      mass += v;
      mx += (float)cx_of(j) * v;
      my += (float)cy_of(j) * v;
      mz += (float)cz_of(j) * v;
    }
    const float inv = __fdividef(1.0f, mass);
    p.plane_out[y + p.ny * z] = make_float4(mx * inv, my * inv, mz * inv, 0.f);
  }
}

// An EQ cell without wall links on a seam row (odd steps): stream_collide.wgsl:102-107
// as in general_cell, stored through the seam kernel's wrapped offsets st.
template <int ST, bool ODD>
__device__ __forceinline__ void eq_cell(const StepParams &p, uint32_t n, uint32_t x, uint32_t y, uint32_t z,
                                        const int64_t *st) {
  using S = Store<ST>;
  using T = typename S::T;
  T *f = reinterpret_cast<T *>(p.f);
  float vx = p.u_in, vy = 0.f, vz = 0.f;
  if (x == p.nx - 1 && x > 0) {
    const float4 u = p.plane_in[y + p.ny * z];
    vx = u.x; vy = u.y; vz = u.z;
  }
  const uint32_t nk = n * 0x9e3779b9u;
#pragma unroll
  for (int j = 0; j < 19; j++)
    f[n + st[j]] = S::encode_fast(geq_ref(j, 0.0f, vx, vy, vz) * S::kScale, dither_mul(j), nk);
  if (p.write_macro) p.macros[n] = make_float4(1.0f + 0.0f, vx, vy, vz);
  if (x + 2 == p.nx) {
    const Nbr b = make_nbr(p, x, y, z);
    T code[19];
#pragma unroll
    for (int j = 0; j < 19; j++) code[j] = f[slot_of<ODD>(b, j, p.stride, n)];
    p.plane_out[y + p.ny * z] = outlet_velocity_of<ST>(code);
  }
}

// The stored codes of one direction of the cell pair in v (.x, .y): 16-bit
// storages round both with one paired stochastic conversion.
template <int ST>
__device__ __forceinline__ void encode_two(float2 v, int j, uint32_t nk, uint32_t nk2, typename Store<ST>::T &a,
                                           typename Store<ST>::T &b) {
  using S = Store<ST>;
  if constexpr (ST == STORE_F32) {
    a = S::encode_fast(v.x, dither_mul(j), nk);
    b = S::encode_fast(v.y, dither_mul(j), nk2);
  } else {
    const uint32_t w = S::encode_pair(v.y, v.x, pair_dither<ST>(v.y, v.x, dither_mul(j), nk2, nk));
    if constexpr (ST == STORE_F16) {
      a = __ushort_as_half((unsigned short)(w & 0xffffu));
      b = __ushort_as_half((unsigned short)(w >> 16));
    } else {
      a = __ushort_as_bfloat16((unsigned short)(w & 0xffffu));
      b = __ushort_as_bfloat16((unsigned short)(w >> 16));
    }
  }
}

// Cells n and n + 32 (x and x + 32 of one row) per thread, the arithmetic in
// packed pairs and the second cell's elements 32 away from the first's.  ok
// (bit 0: n, bit 1: n + 32) marks the lanes that are stored: plain cells, and
// EQ cells without wall links (eq), which take the equilibrium of rho 1 and
// the inlet or outlet velocity through the same reconstruction
// (stream_collide.wgsl:102-107).  Other lanes compute on the elements they
// read (inside the padded array) and store nothing.
template <int ST, int OP, bool LES, bool ODD>
__device__ __forceinline__ void plain_pair(const StepParams &p, uint32_t n, uint32_t x, uint32_t y, uint32_t z,
                                           uint32_t ok, uint32_t eq) {
  using S = Store<ST>;
  using T = typename S::T;
  T *f = reinterpret_cast<T *>(p.f);
  float2 eux = f2(p.u_in), euy = f2(0.f), euz = f2(0.f);
  if (eq) {
    const uint32_t row = y + p.ny * z;
    if ((eq & 1u) && x == p.nx - 1 && x > 0) {
      const float4 u = p.plane_in[row];
      eux.x = u.x; euy.x = u.y; euz.x = u.z;
    }
    if ((eq & 2u) && x + 32u == p.nx - 1) {
      const float4 u = p.plane_in[row];
      eux.y = u.x; euy.y = u.y; euz.y = u.z;
    }
  }
  float2 g[19];
#pragma unroll
  for (int i = 0; i < 19; i++) {
    const T *a = f + (n + p.ld[i]);
    g[i] = make_float2(S::raw(a[0]), S::raw(a[32]));
  }
  float2 rho, vx, vy, vz;
  const float2 om = update_fast2<OP, LES>(p, g, rho, vx, vy, vz, S::kScale, S::kInvScale, eq, eux, euy, euz);
  if (ST != STORE_F32) {
    // a non-finite state is stored as NaN, as the reference's GPUs store it
    if (!(fabsf(rho.x + om.x) < INFINITY)) {
#pragma unroll
      for (int j = 0; j < 19; j++) g[j].x = __uint_as_float(0x7fc00000u);
    }
    if (!(fabsf(rho.y + om.y) < INFINITY)) {
#pragma unroll
      for (int j = 0; j < 19; j++) g[j].y = __uint_as_float(0x7fc00000u);
    }
  }
  const uint32_t nk = n * 0x9e3779b9u, nk2 = nk + 32u * 0x9e3779b9u;
  // EQ lanes at x = 0 or nx - 1 store to n + c_j, which wraps in x on odd steps;
  // a warp with such a lane takes the wrapping stores as a whole
  const bool wrap = ODD && __any_sync(__activemask(), eq && (x == 0u || x + 33u >= p.nx));
  if (!wrap) {
#pragma unroll
    for (int j = 0; j < 19; j++) {
      T *a = f + (n + p.st[j]);
      T ca, cb;
      encode_two<ST>(g[j], j, nk, nk2, ca, cb);
      if (ok & 1u) a[0] = ca;
      if (ok & 2u) a[32] = cb;
    }
  } else {
    const uint32_t xa = x, xb = x + 32u;
#pragma unroll
    for (int j = 0; j < 19; j++) {
      // signed: added to 64-bit element indices
      const int64_t wa = cx_of(j) < 0 && xa == 0u ? (int64_t)p.nx : (cx_of(j) > 0 && xa + 1u == p.nx ? -(int64_t)p.nx : 0);
      const int64_t wb = cx_of(j) > 0 && xb + 1u == p.nx ? -(int64_t)p.nx : 0;
      T ca, cb;
      encode_two<ST>(g[j], j, nk, nk2, ca, cb);
      if (ok & 1u) f[n + p.st[j] + wa] = ca;
      if (ok & 2u) f[n + 32u + p.st[j] + wb] = cb;
    }
  }
  if (p.write_macro) {
    const bool bad_a = (ok & ~eq & 1u) && !(rho.x >= 0.5f && rho.x <= 1.5f);
    const bool bad_b = (ok & ~eq & 2u) && !(rho.y >= 0.5f && rho.y <= 1.5f);
    if (bad_a || bad_b) atomicOr(p.status, 1u);
    if (ok & 1u) p.macros[n] = make_float4(rho.x, vx.x, vy.x, vz.x);
    if (ok & 2u) p.macros[n + 32] = make_float4(rho.y, vx.y, vy.y, vz.y);
  }
  const bool pub_a = (ok & 1u) && x + 2u == p.nx, pub_b = (ok & 2u) && x + 34u == p.nx;
  if (pub_a || pub_b) {
    // the outlet's upstream plane publishes the velocity of its stored codes
    const uint32_t xo = pub_a ? x : x + 32u, no = n + (xo - x);
    const Nbr b = make_nbr(p, xo, y, z);
    T code[19];
#pragma unroll
    for (int j = 0; j < 19; j++) code[j] = f[slot_of<ODD>(b, j, p.stride, no)];
    p.plane_out[y + p.ny * z] = outlet_velocity_of<ST>(code);
  }
}

// Plain cells and wall-free EQ cells of the whole grid (even steps, which
// touch only the cell's own slots) or of the rows off the periodic y and z
// seams (odd steps: y and z from 1 to n-2); threads take x and x + 32 of a
// 64-cell run of a row.
// One thread of the plain kernel: cells x and x + 32 of row (y, z).
template <int ST, int OP, bool LES, bool ODD>
__device__ __forceinline__ void plain_thread(const StepParams &p, uint32_t x, uint32_t y, uint32_t z) {
  const uint32_t n = x + p.nx * (y + p.ny * z);
  uint32_t ok = 0u, eq = 0u;
#pragma unroll
  for (uint32_t k = 0; k < 2u; k++) {
    const uint32_t xk = x + 32u * k, nk = n + 32u * k;
    if (xk >= p.nx) continue;
    if (!((__ldg(&p.special[nk >> 5]) >> (nk & 31u)) & 1u)) {
      if (is_plain_position(xk, p.nx)) ok |= 1u << k;
    } else if (__ldg(&p.flags[nk]) == EQ) {
      ok |= 1u << k;
      eq |= 1u << k;
    }
  }
  if (ok) plain_pair<ST, OP, LES, ODD>(p, n, x, y, z, ok, eq);
}

template <int ST, int OP, bool LES, bool ODD>
__global__ void __launch_bounds__(NTHREADS) aa_step_fast(StepParams p) {
  const uint32_t x = blockIdx.x * (2 * BX) + threadIdx.x;
  const uint32_t y = blockIdx.y * BY + threadIdx.y + (ODD ? 1u : 0u);
  const uint32_t z = blockIdx.z + (ODD ? 1u : 0u);
  if (y + (ODD ? 1u : 0u) >= p.ny) return;
  plain_thread<ST, OP, LES, ODD>(p, x, y, z);
}

// ---------------------------------------------------------------- 16-bit cell pairs
// The 16-bit storages' plain kernel (nx even): lane t of a warp takes the
// adjacent cells x0 = 64 r + 2t and x0 + 1 of a 64-cell run r of a row, so a
// pair is one aligned 32-bit word of every direction plane.  Even steps touch
// only the cell's own slots: each direction is one 32-bit load and one 32-bit
// store of both cells' codes (whole 128-byte lines per warp), and the store
// word comes straight out of the paired stochastic conversion.  On odd steps
// the directions with c_x = 0 stay on the word grid and move as words; the
// ten with c_x = +-1 sit one element off it and move as two 16-bit accesses,
// one per cell (no shuffles, no divergence: 58 memory instructions per pair
// instead of 76).  A word whose two cells are not both stored here (an
// x-face or wall-link neighbour belongs to the edge kernel) is written half by
// half.
__device__ __forceinline__ uint32_t ld_word(const void *a) {
  uint32_t v;
  asm("ld.global.L2::256B.b32 %0, [%1];" : "=r"(v) : "l"(a));
  return v;
}
__device__ __forceinline__ uint32_t ld_half(const void *a) {
  unsigned short v;
  asm("ld.global.b16 %0, [%1];" : "=h"(v) : "l"(a));
  return v;
}
__device__ __forceinline__ void st_word(void *a, uint32_t v) {
  asm volatile("st.global.b32 [%0], %1;" ::"l"(a), "r"(v) : "memory");
}
__device__ __forceinline__ void st_half(void *a, uint32_t v) {
  asm volatile("st.global.b16 [%0], %1;" ::"l"(a), "h"((unsigned short)v) : "memory");
}

template <int ST>
__device__ __forceinline__ float raw_of_bits(uint32_t b) {
  if (ST == STORE_F16) return __half2float(__ushort_as_half((unsigned short)b));
  return __uint_as_float(b << 16);
}

// Both codes of a 32-bit word as binary32 (.x the low code).
template <int ST>
__device__ __forceinline__ float2 raw_of_word(uint32_t w) {
  if constexpr (ST == STORE_F16) {
    __half2 h;
    memcpy(&h, &w, sizeof(h));
    return __half22float2(h);
  } else {
    return make_float2(__uint_as_float(w << 16), __uint_as_float(w & 0xffff0000u));
  }
}

// The update and stores of a cell pair whose 19 direction values (both cells,
// stored units) are in g: collision, rounding, the stores, the outlet's
// upstream plane and the macros.
// The periodic wrap of an odd step's pulls on a seam row (y = 0 or ny - 1,
// z = 0 or nz - 1), in bytes per direction: the pull from y - 1 on y = 0
// lands ny rows further on, the one from y + 1 on y = ny - 1 ny rows back,
// and the same with planes in z.  The same for every cell of a row; zero off
// the seams.  The store of direction j goes where direction opp(j) was loaded,
// so it takes opp(j)'s correction.
struct SeamWrap {
  int64_t y_lo = 0, y_hi = 0, z_lo = 0, z_hi = 0;
  __device__ __forceinline__ SeamWrap() {}
  __device__ __forceinline__ SeamWrap(const StepParams &p, uint32_t y, uint32_t z, int64_t esize) {
    const int64_t rows = (int64_t)p.nx * p.ny, planes = rows * p.nz;
    y_lo = y == 0u ? rows * esize : 0;
    y_hi = y + 1u == p.ny ? -rows * esize : 0;
    z_lo = z == 0u ? planes * esize : 0;
    z_hi = z + 1u == p.nz ? -planes * esize : 0;
  }
  __device__ __forceinline__ int64_t of(int i) const {
    return (cy_of(i) > 0 ? y_lo : (cy_of(i) < 0 ? y_hi : 0)) + (cz_of(i) > 0 ? z_lo : (cz_of(i) < 0 ? z_hi : 0));
  }
};

// A cell pair's inputs read again (the floor cells' rare fallback); the pair's
// slots are not written before its stores, so a second read returns them.
struct NoReload {
  __device__ __forceinline__ void operator()(float2 *) const {}
};

template <int ST, int OP, bool LES, bool ODD, bool FLOOR = false, bool SEAM = false, class Reload = NoReload>
__device__ __forceinline__ void pair_finish(const StepParams &p, uint32_t n, uint32_t x, uint32_t y, uint32_t z,
                                            uint32_t ok, uint32_t eq, float2 *g, const Reload &reload = Reload(),
                                            const SeamWrap &sw = SeamWrap()) {
  using S = Store<ST>;
  float2 eux = f2(p.u_in), euy = f2(0.f), euz = f2(0.f);
  if ((eq & 2u) && x + 2u == p.nx) {  // the outlet is the pair's second cell (x even, nx even)
    const float4 u = p.plane_in[y + p.ny * z];
    eux.y = u.x; euy.y = u.y; euz.y = u.z;
  }
  float2 rho, vx, vy, vz, om;
  if constexpr (FLOOR && LES) {
    // floor cells: the reference's LES wall cell; a cell for which it keeps
    // the plain collision takes that instead (rare: no slip, or a population
    // the wall stress would make negative)
    FloorState w;
    const uint32_t fb = floor_wall2(p, g, w, S::kScale, S::kInvScale);
    rho = w.rho; vx = w.vx; vy = w.vy; vz = w.vz;
    om = rho;  // finite exactly when the state is
    if (fb) {
      float2 r2, x2, y2, z2;
      reload(g);
      update_fast2<OP, LES>(p, g, r2, x2, y2, z2, S::kScale, S::kInvScale, 0u, eux, euy, euz);
      floor_post2(g, w, S::kScale, ~fb & 3u);
    }
  } else {
    om = update_fast2<OP, LES>(p, g, rho, vx, vy, vz, S::kScale, S::kInvScale, eq, eux, euy, euz);
  }
  // a non-finite state is stored as NaN, as the reference's GPUs store it
  if (!(fabsf(rho.x + om.x) < INFINITY)) {
#pragma unroll
    for (int j = 0; j < 19; j++) g[j].x = __uint_as_float(0x7fc00000u);
  }
  if (!(fabsf(rho.y + om.y) < INFINITY)) {
#pragma unroll
    for (int j = 0; j < 19; j++) g[j].y = __uint_as_float(0x7fc00000u);
  }
  const uint32_t nk = n * 0x9e3779b9u, nk2 = nk + 0x9e3779b9u;
  // odd steps: the EQ cell at x = 0 pushes c_x = -1 to x = nx - 1 and the one at
  // x = nx - 1 pushes c_x = +1 to x = 0 (periodic in x, as idx_wrapped)
  // (signed byte offsets: they are added to the pointer on their own)
  const int wrap_lo = ODD && (eq & 1u) && x == 0u ? 2 * (int)p.nx : 0;
  const int wrap_hi = ODD && (eq & 2u) && x + 2u == p.nx ? -2 * (int)p.nx : 0;
  // the outlet's upstream cell (x = nx - 2, the first of its pair) publishes the
  // velocity of its stored codes
  const bool pub = (ok & 1u) && x + 2u == p.nx;
  float mass = 1.0f, mx = 0.f, my = 0.f, mz = 0.f;
  uint32_t w[19];
#pragma unroll
  for (int j = 0; j < 19; j++) {
    w[j] = S::encode_pair(g[j].y, g[j].x, pair_dither<ST>(g[j].y, g[j].x, dither_mul(j), nk2, nk));
    if (pub) {
      const float v = raw_of_bits<ST>(w[j] & 0xffffu) * S::kInvScale;
      mass += v;
      mx += (float)cx_of(j) * v;
      my += (float)cy_of(j) * v;
      mz += (float)cz_of(j) * v;
    }
  }
  char *obase = reinterpret_cast<char *>(p.f) + 2 * (size_t)n;
  if (ok == 3u && !wrap_lo && !wrap_hi) {
    // both cells stored here (nearly every pair): one branch for all directions
#pragma unroll
    for (int j = 0; j < 19; j++) {
      char *a = obase + p.stb[j] + (SEAM ? sw.of(opp_of(j)) : 0);
      if (ODD && cx_of(j) != 0) {
        st_half(a, w[j] & 0xffffu);
        st_half(a + 2, w[j] >> 16);
      } else {
        st_word(a, w[j]);
      }
    }
  } else {
#pragma unroll
    for (int j = 0; j < 19; j++) {
      char *a = obase + p.stb[j] + (SEAM ? sw.of(opp_of(j)) : 0);
      if (ODD && cx_of(j) != 0) {
        if (ok & 1u) st_half(a + (cx_of(j) < 0 ? wrap_lo : 0), w[j] & 0xffffu);
        if (ok & 2u) st_half(a + 2 + (cx_of(j) > 0 ? wrap_hi : 0), w[j] >> 16);
      } else {
        if (ok & 1u) st_half(a, w[j] & 0xffffu);
        if (ok & 2u) st_half(a + 2, w[j] >> 16);
      }
    }
  }
  if (pub) {
    const float inv = __fdividef(1.0f, mass);
    p.plane_out[y + p.ny * z] = make_float4(mx * inv, my * inv, mz * inv, 0.f);
  }
  if (p.write_macro) {
    const bool bad_a = (ok & ~eq & 1u) && !(rho.x >= 0.5f && rho.x <= 1.5f);
    const bool bad_b = (ok & ~eq & 2u) && !(rho.y >= 0.5f && rho.y <= 1.5f);
    if (bad_a || bad_b) atomicOr(p.status, 1u);
    if (ok & 1u) p.macros[n] = make_float4(rho.x, vx.x, vy.x, vz.x);
    if (ok & 2u) p.macros[n + 1] = make_float4(rho.y, vx.y, vy.y, vz.y);
  }
}

// Whether direction i of a cell pair is read one element off the word grid:
// the odd steps' pulls along c_x = +-1, and for a floor cell's links (read
// where the opposite parity pulls from) the even steps'.
template <bool ODD, bool LINK>
__host__ __device__ constexpr bool shifted_read(int i) {
  return cx_of(i) != 0 && (LINK ? !ODD : ODD);
}

// A cell pair of the one-shot cell-pair kernels, its codes loaded straight
// from HBM.  FLOOR: both cells are floor cells, whose five floor links read
// the slots that nobody rewrites this step (halfway bounce-back).
template <int ST, int OP, bool LES, bool ODD, bool FLOOR = false, bool SEAM = false>
__device__ __forceinline__ void pair_cells(const StepParams &p, uint32_t n, uint32_t x, uint32_t y, uint32_t z,
                                           uint32_t ok, uint32_t eq) {
  // one 64-bit base per thread; each direction adds its byte offset from the
  // kernel parameters (and on a seam row its wrap)
  const char *base = reinterpret_cast<const char *>(p.f) + 2 * (size_t)n;
  const SeamWrap sw = SEAM ? SeamWrap(p, y, z, 2) : SeamWrap();
  const auto load = [&](float2 *v) {
#pragma unroll
    for (int i = 0; i < 19; i++) {
      const bool link = FLOOR && cz_of(i) == 1;
      const char *a = base + (link ? p.wb[i] : p.ldb[i]) + (SEAM ? sw.of(i) : 0);
      if (link ? shifted_read<ODD, true>(i) : shifted_read<ODD, false>(i)) {
        v[i] = make_float2(raw_of_bits<ST>(ld_half(a)), raw_of_bits<ST>(ld_half(a + 2)));
      } else {
        v[i] = raw_of_word<ST>(ld_word(a));
      }
    }
  };
  float2 g[19];
  load(g);
  pair_finish<ST, OP, LES, ODD, FLOOR, SEAM>(p, n, x, y, z, ok, eq, g, load, sw);
}

// The floor layer of a domain with floor rows (is_floor_cell): the z = 1 rows
// off the y seams, a lane per cell pair; it runs beside the cell-pair kernel
// on the side stream.  Floor cells link only to FLOOR cells, which add
// nothing to the drag.
template <int ST, int OP, bool LES, bool ODD>
__global__ void __launch_bounds__(NTHREADS, 5) aa_step_floor(StepParams p) {
  const uint32_t x = blockIdx.x * (2 * BX) + 2u * threadIdx.x;
  const uint32_t y = 1u + blockIdx.y * BY + threadIdx.y;
  if (x >= p.nx || y + 2u > p.ny) return;
  const uint32_t n = x + p.nx * (y + p.ny);
  const uint32_t ok = (__ldg(&p.flags[n]) == kFloorFlag ? 1u : 0u) | (__ldg(&p.flags[n + 1]) == kFloorFlag ? 2u : 0u);
  if (ok) pair_cells<ST, OP, LES, ODD, true>(p, n, x, y, 1u, ok, 0u);
}

template <int ST, int OP, bool LES, bool ODD>
__device__ __forceinline__ void pair_thread(const StepParams &p, uint32_t x, uint32_t y, uint32_t z) {
  if (x >= p.nx) return;
  const uint32_t n = x + p.nx * (y + p.ny * z);
  const uint32_t word = __ldg(&p.special[n >> 5]);
  uint32_t ok = 0u, eq = 0u;
#pragma unroll
  for (uint32_t k = 0; k < 2u; k++) {
    const uint32_t xk = x + k, nk = n + k;
    if (!((word >> (nk & 31u)) & 1u)) {
      if (is_plain_position(xk, p.nx)) ok |= 1u << k;
    } else if (__ldg(&p.flags[nk]) == EQ) {
      ok |= 1u << k;
      eq |= 1u << k;
    }
  }
  if (ok) pair_cells<ST, OP, LES, ODD>(p, n, x, y, z, ok, eq);
}

// One warp per 64-cell run of a row: every row on even steps, the rows off the
// periodic y and z seams on odd steps.  Held to 64 registers (8 blocks per SM):
// the few spilled words cost less than the lost occupancy (measured 1%).
template <int ST, int OP, bool LES, bool ODD>
__global__ void __launch_bounds__(NTHREADS, 8) aa_step_pairs(StepParams p) {
  const uint32_t x = blockIdx.x * (2 * BX) + 2u * threadIdx.x;
  const uint32_t y = blockIdx.y * BY + threadIdx.y + (ODD ? 1u : 0u);
  const uint32_t z = blockIdx.z + (ODD ? 1u : 0u);
  if (y + (ODD ? 1u : 0u) >= p.ny) return;
  pair_thread<ST, OP, LES, ODD>(p, x, y, z);
}

// Odd steps on the seam rows: every row of the planes z = 0 and z = nz-1, then
// the rows y = 0 and y = ny-1 of the planes between; one row per block row.
// Neighbour offsets wrap around the domain.
__host__ __device__ __forceinline__ uint32_t seam_rows(uint32_t ny, uint32_t nz) {
  const uint32_t zs = nz > 1u ? 2u : 1u, ys = ny > 1u ? 2u : 1u;
  return zs * ny + (nz - zs) * ys;
}

template <int ST, int OP, bool LES>
__device__ __forceinline__ void seam_thread(const StepParams &p, uint32_t x, uint32_t r) {
  const uint32_t zs = p.nz > 1u ? 2u : 1u, ys = p.ny > 1u ? 2u : 1u;
  uint32_t y, z;
  if (r < zs * p.ny) {
    z = r < p.ny ? 0u : p.nz - 1u;
    y = r < p.ny ? r : r - p.ny;
  } else {
    r -= zs * p.ny;
    z = 1u + r / ys;
    y = (r % ys) ? p.ny - 1u : 0u;
  }
  const uint32_t n = x + p.nx * (y + p.ny * z);
  if (x >= p.nx) return;
  const bool special = (__ldg(&p.special[n >> 5]) >> (n & 31u)) & 1u;
  if (special ? __ldg(&p.flags[n]) != EQ : !is_plain_position(x, p.nx)) return;
  // offsets relative to n of the wrapped (or reflected, on free-slip faces) slots
  const Nbr b = make_nbr(p, x, y, z);
  int64_t ld[19], st[19];
#pragma unroll
  for (int i = 0; i < 19; i++) {
    ld[i] = (int64_t)b.pull(i, p.stride) - (int64_t)n;
    st[i] = (int64_t)b.push(i, p.stride) - (int64_t)n;
  }
  if (special) eq_cell<ST, true>(p, n, x, y, z, st);
  else plain_cell<ST, OP, LES, true>(p, n, x, y, z, ld, st);
}

template <int ST, int OP, bool LES>
__global__ void __launch_bounds__(BX) aa_step_seam(StepParams p) {
  seam_thread<ST, OP, LES>(p, blockIdx.x * BX + threadIdx.x, blockIdx.y);
}

// Odd steps on the seam rows with periodic y and z faces, as cell pairs (16-bit
// storage, nx even): the rows of seam_thread, four per block, each direction
// pulled and pushed across the wrap by its row's SeamWrap correction.
template <int ST, int OP, bool LES>
__device__ __forceinline__ void seam_pair_thread(const StepParams &p, uint32_t x, uint32_t r) {
  if (r >= seam_rows(p.ny, p.nz) || x >= p.nx) return;
  const uint32_t zs = p.nz > 1u ? 2u : 1u, ys = p.ny > 1u ? 2u : 1u;
  uint32_t y, z;
  if (r < zs * p.ny) {
    z = r < p.ny ? 0u : p.nz - 1u;
    y = r < p.ny ? r : r - p.ny;
  } else {
    r -= zs * p.ny;
    z = 1u + r / ys;
    y = (r % ys) ? p.ny - 1u : 0u;
  }
  const uint32_t n = x + p.nx * (y + p.ny * z);
  const uint32_t word = __ldg(&p.special[n >> 5]);
  uint32_t ok = 0u, eq = 0u;
#pragma unroll
  for (uint32_t k = 0; k < 2u; k++) {
    const uint32_t xk = x + k, nk = n + k;
    if (!((word >> (nk & 31u)) & 1u)) {
      if (is_plain_position(xk, p.nx)) ok |= 1u << k;
    } else if (__ldg(&p.flags[nk]) == EQ) {
      ok |= 1u << k;
      eq |= 1u << k;
    }
  }
  if (ok) pair_cells<ST, OP, LES, true, false, true>(p, n, x, y, z, ok, eq);
}

template <int ST, int OP, bool LES>
__global__ void __launch_bounds__(NTHREADS, 5) aa_step_seam_pairs(StepParams p) {
  seam_pair_thread<ST, OP, LES>(p, blockIdx.x * (2 * BX) + 2u * threadIdx.x, blockIdx.y * BY + threadIdx.y);
}

__device__ __forceinline__ void cell_coords(const StepParams &p, uint32_t n, uint32_t &x, uint32_t &y, uint32_t &z) {
  const uint32_t row = n / p.nx;
  x = n - row * p.nx;
  z = row / p.ny;
  y = row - z * p.ny;
}

// One listed cell per thread; block b's force partial goes to slot b.
template <int ST, int OP, bool LES, bool ODD>
__device__ __forceinline__ void edge_block(const StepParams &p, const uint32_t *list, uint32_t count, uint32_t blk,
                                           uint32_t tid) {
  const uint32_t t = blk * NTHREADS + tid;
  bool force_any = false;
  double fx = 0.0, fy = 0.0, fz = 0.0;
  if (t < count) {
    const uint32_t n = __ldg(&list[t]);
    uint32_t x, y, z;
    cell_coords(p, n, x, y, z);
    const uint32_t flag = __ldg(&p.flags[n]);
    // with floor rows on, the floor kernel updates the floor layer
    if (!(p.floor_rows && is_floor_cell(flag, y, z, p.ny)))
      general_cell<ST, OP, LES, ODD>(p, x, y, z, n, flag, fx, fy, fz, force_any);
  }
  reduce_force_at(force_any, fx, fy, fz, p.partials, blk, tid);
}

// Held to 64 registers (8 blocks per SM) although it spills: it runs beside the
// plain kernel, and its smaller register share leaves that kernel more warps
// (the step measured 1.2% faster than at its natural 96 registers).
template <int ST, int OP, bool LES, bool ODD>
__global__ void __launch_bounds__(NTHREADS, 8) aa_step_edges(StepParams p, const uint32_t *list, uint32_t count) {
  edge_block<ST, OP, LES, ODD>(p, list, count, blockIdx.x, threadIdx.x);
}
#endif

// ---------------------------------------------------------------- init (layout E)
// init.wgsl:1-8 into the even layout, after the array was cleared: equilibrium
// at u_start in fluid and EQ cells, macros everywhere (walls at rest),
// both outlet planes and both force partials of the start state.
template <int ST>
__device__ __forceinline__ void init_cell(const StepParams &p, uint32_t x, uint32_t y, uint32_t z, float4 *plane_b,
                                          double &fx, double &fy, double &fz, bool &any) {
  using S = Store<ST>;
  using T = typename S::T;
  T *f = reinterpret_cast<T *>(p.f);
  const uint32_t n = x + p.nx * (y + p.ny * z);
  const uint32_t flag = p.flags[n];
  const uint32_t kind = flag & 7u;
  const Nbr b = make_nbr(p, x, y, z);
  const float vx = is_wall_kind(kind) ? 0.0f : p.u_in;
  T code[19];
#pragma unroll
  for (int j = 0; j < 19; j++) code[j] = S::encode(geq_ref(j, 0.0f, vx, 0.f, 0.f), (uint32_t)j, n);
  if (!is_wall_kind(kind)) {
#pragma unroll
    for (int j = 0; j < 19; j++) f[(pidx)opp_of(j) * p.stride + n] = code[j];
    if (kind == FLUID && (flag >> 3)) {
#pragma unroll
      for (int i = 1; i < 19; i++) {
        if (!(flag & (1u << (3 + i)))) continue;
        const int j = opp_of(i);
        const uint32_t w = b.at(-cx_of(i), -cy_of(i), -cz_of(i));
        if ((p.flags[w] & 7u) == SOLID) {
          float v = S::decode(code[j]);
          double term = (double)(v + v);
          fx += (double)cx_of(j) * term;
          fy += (double)cy_of(j) * term;
          fz += (double)cz_of(j) * term;
          any = true;
        }
      }
    }
  }
  p.macros[n] = make_float4(1.0f + 0.0f, vx, 0.f, 0.f);
  if (x + 2 == p.nx) {
    float4 u = make_float4(0.f, 0.f, 0.f, 0.f);
    if (!is_wall_kind(kind)) u = outlet_velocity_of<ST>(code);
    p.plane_out[y + p.ny * z] = u;
    plane_b[y + p.ny * z] = u;
  }
}

__device__ __forceinline__ void copy_partial(double *partials_a, double *partials_b) {
  if (partials_a == nullptr || partials_b == nullptr) return;
  __syncthreads();
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    size_t blk = blockIdx.x + (size_t)gridDim.x * (blockIdx.y + (size_t)gridDim.y * blockIdx.z);
    for (int k = 0; k < 3; k++) partials_b[3 * blk + k] = partials_a[3 * blk + k];
  }
}

// Tile mapping of aa_step: one cell per thread, 32 x 4 cells per block.
template <int ST>
__global__ void __launch_bounds__(NTHREADS) aa_init(StepParams p, float4 *plane_b, double *partials_b) {
  const uint32_t x = blockIdx.x * BX + threadIdx.x;
  const uint32_t y = blockIdx.y * BY + threadIdx.y;
  const uint32_t z = blockIdx.z;
  bool any = false;
  double fx = 0, fy = 0, fz = 0;
  if (x < p.nx && y < p.ny) init_cell<ST>(p, x, y, z, plane_b, fx, fy, fz, any);
  if (__syncthreads_or(any)) {
    reduce_force(any, fx, fy, fz, p.partials);
    copy_partial(p.partials, partials_b);
  }
}

// Linear mapping of the tiled step: block b owns cells [b * cpb, (b + 1) * cpb).
template <int ST>
__global__ void __launch_bounds__(NTHREADS) aa_init_lin(StepParams p, float4 *plane_b, double *partials_b,
                                                      uint32_t cpb) {
  const size_t cells = (size_t)p.nx * p.ny * p.nz;
  bool any = false;
  double fx = 0, fy = 0, fz = 0;
  const size_t base = (size_t)blockIdx.x * cpb;
  for (uint32_t c = threadIdx.x; c < cpb; c += NTHREADS) {
    size_t n = base + c;
    if (n < cells) {
      uint32_t x = (uint32_t)(n % p.nx), y = (uint32_t)((n / p.nx) % p.ny), z = (uint32_t)(n / ((size_t)p.nx * p.ny));
      init_cell<ST>(p, x, y, z, plane_b, fx, fy, fz, any);
    }
  }
  if (__syncthreads_or(any)) {
    reduce_force(any, fx, fy, fz, p.partials);
    copy_partial(p.partials, partials_b);
  }
}

// ---------------------------------------------------------------- readout / write-in
// mode 0: decoded float; mode 1: raw codes.  odd_layout: parity of the latest step.
template <int ST>
__global__ void aa_read(StepParams p, int odd_layout, int mode, void *out) {
  using S = Store<ST>;
  using T = typename S::T;
  const T *f = reinterpret_cast<const T *>(p.f);
  const uint32_t x = blockIdx.x * BX + threadIdx.x;
  const uint32_t y = blockIdx.y * BY + threadIdx.y;
  const uint32_t z = blockIdx.z;
  if (x >= p.nx || y >= p.ny) return;
  const uint32_t cells = p.nx * p.ny * p.nz;
  const uint32_t n = x + p.nx * (y + p.ny * z);
  const bool wall = is_wall_kind(p.flags[n] & 7u);
  const Nbr b = make_nbr(p, x, y, z);
#pragma unroll
  for (int j = 0; j < 19; j++) {
    T code;
    if (wall) code = S::encode(0.0f, 0u, 0u);
    else code = f[odd_layout ? slot_of<true>(b, j, p.stride, n) : slot_of<false>(b, j, p.stride, n)];
    size_t k = (size_t)j * cells + n;
    if (mode == 0) reinterpret_cast<float *>(out)[k] = wall ? 0.0f : S::decode(code);
    else reinterpret_cast<T *>(out)[k] = code;
  }
}

// Write a canonical state into the AA layout of the given parity; mode 0
// encodes decoded floats, mode 1 copies codes.
template <int ST>
__global__ void aa_write(StepParams p, int odd_layout, int mode, const void *in) {
  using S = Store<ST>;
  using T = typename S::T;
  T *f = reinterpret_cast<T *>(p.f);
  const uint32_t x = blockIdx.x * BX + threadIdx.x;
  const uint32_t y = blockIdx.y * BY + threadIdx.y;
  const uint32_t z = blockIdx.z;
  if (x >= p.nx || y >= p.ny) return;
  const uint32_t cells = p.nx * p.ny * p.nz;
  const uint32_t n = x + p.nx * (y + p.ny * z);
  const uint32_t flag = p.flags[n];
  if (is_wall_kind(flag & 7u)) return;
  const Nbr b = make_nbr(p, x, y, z);
#pragma unroll
  for (int j = 0; j < 19; j++) {
    size_t k = (size_t)j * cells + n;
    T code = mode == 0 ? S::encode(reinterpret_cast<const float *>(in)[k], (uint32_t)j, n)
                       : reinterpret_cast<const T *>(in)[k];
    f[odd_layout ? slot_of<true>(b, j, p.stride, n) : slot_of<false>(b, j, p.stride, n)] = code;
  }
}

// Recompute the outlet plane and this parity's force partial from the latest
// state (after a write-in).
template <int ST>
__device__ __forceinline__ void refresh_cell(const StepParams &p, int odd_layout, uint32_t x, uint32_t y, uint32_t z,
                                             double &fx, double &fy, double &fz, bool &any) {
  using S = Store<ST>;
  using T = typename S::T;
  const T *f = reinterpret_cast<const T *>(p.f);
  const uint32_t n = x + p.nx * (y + p.ny * z);
  const uint32_t flag = p.flags[n];
  const Nbr b = make_nbr(p, x, y, z);
  if (is_wall_kind(flag & 7u)) return;
  T code[19];
#pragma unroll
  for (int j = 0; j < 19; j++)
    code[j] = f[odd_layout ? slot_of<true>(b, j, p.stride, n) : slot_of<false>(b, j, p.stride, n)];
  if (x + 2 == p.nx) p.plane_out[y + p.ny * z] = outlet_velocity_of<ST>(code);
  if ((flag & 7u) == FLUID && (flag >> 3)) {
#pragma unroll
    for (int i = 1; i < 19; i++) {
      if (!(flag & (1u << (3 + i)))) continue;
      const int j = opp_of(i);
      if ((p.flags[b.at(-cx_of(i), -cy_of(i), -cz_of(i))] & 7u) != SOLID) continue;
      float v = S::decode(code[j]);
      double term = (double)(v + v);
      fx += (double)cx_of(j) * term;
      fy += (double)cy_of(j) * term;
      fz += (double)cz_of(j) * term;
      any = true;
    }
  }
}

template <int ST>
__global__ void __launch_bounds__(NTHREADS) aa_refresh(StepParams p, int odd_layout) {
  const uint32_t x = blockIdx.x * BX + threadIdx.x;
  const uint32_t y = blockIdx.y * BY + threadIdx.y;
  const uint32_t z = blockIdx.z;
  bool any = false;
  double fx = 0, fy = 0, fz = 0;
  if (x < p.nx && y < p.ny) refresh_cell<ST>(p, odd_layout, x, y, z, fx, fy, fz, any);
  reduce_force(any, fx, fy, fz, p.partials);
}

template <int ST>
__global__ void __launch_bounds__(NTHREADS) aa_refresh_lin(StepParams p, int odd_layout, uint32_t cpb) {
  const size_t cells = (size_t)p.nx * p.ny * p.nz;
  bool any = false;
  double fx = 0, fy = 0, fz = 0;
  const size_t base = (size_t)blockIdx.x * cpb;
  for (uint32_t c = threadIdx.x; c < cpb; c += NTHREADS) {
    size_t n = base + c;
    if (n < cells) {
      uint32_t x = (uint32_t)(n % p.nx), y = (uint32_t)((n / p.nx) % p.ny), z = (uint32_t)(n / ((size_t)p.nx * p.ny));
      refresh_cell<ST>(p, odd_layout, x, y, z, fx, fy, fz, any);
    }
  }
  reduce_force(any, fx, fy, fz, p.partials);
}

#if !PW_STRICT
// Outlet plane and force partials of the latest state over the fast step's
// edge list, in aa_step_edges' slot mapping.
template <int ST>
__global__ void __launch_bounds__(NTHREADS) aa_refresh_edges(StepParams p, int odd_layout, const uint32_t *list,
                                                           uint32_t count) {
  const uint32_t t = blockIdx.x * NTHREADS + threadIdx.x;
  bool any = false;
  double fx = 0, fy = 0, fz = 0;
  if (t < count) {
    uint32_t x, y, z;
    cell_coords(p, __ldg(&list[t]), x, y, z);
    refresh_cell<ST>(p, odd_layout, x, y, z, fx, fy, fz, any);
  }
  reduce_force(any, fx, fy, fz, p.partials);
}
#endif

// ---------------------------------------------------------------- interpolated walls: state pass
// The momentum exchange of the latest state with interpolated walls, as the next
// step will evaluate its wall values (force.wgsl:20-29 over walls.wgsl:6-21), into
// p.partials; with refresh, each link's f*_i(n) is first copied out of the layout
// into hist (after an init or a write of the state).
template <int ST>
__device__ __forceinline__ void interpolated_state_cell(const StepParams &p, int odd_layout, int refresh, uint32_t x,
                                                        uint32_t y, uint32_t z, double &fx, double &fy, double &fz,
                                                        bool &any) {
  using S = Store<ST>;
  using T = typename S::T;
  const T *f = reinterpret_cast<const T *>(p.f);
  const uint32_t n = x + p.nx * (y + p.ny * z);
  const uint32_t flag = __ldg(&p.flags[n]);
  if ((flag & 7u) != FLUID || (flag >> 3) == 0u) return;
  const Nbr b = make_nbr(p, x, y, z);
  const uint32_t S_ = p.stride;
  T *hist = reinterpret_cast<T *>(p.hist);
  const uint32_t base = __ldg(&p.qoff[n]);
  if (refresh && base != NO_Q) {
    uint32_t k = base;
#pragma unroll
    for (int i = 1; i < 19; i++)
      if (flag & (1u << (3 + i))) hist[k++] = f[odd_layout ? slot_of<true>(b, i, S_, n) : slot_of<false>(b, i, S_, n)];
  }
  // what the next step reads: it is even after an odd layout, odd after an even one
  float g[19];
#pragma unroll
  for (int i = 0; i < 19; i++) {
    pidx src = odd_layout ? (pidx)i * S_ + n : b.pull(i, S_);
    if (i > 0 && (flag & (1u << (3 + i))))
      src = odd_layout ? (pidx)opp_of(i) * S_ + b.at(-cx_of(i), -cy_of(i), -cz_of(i)) : (pidx)i * S_ + n;
    g[i] = S::decode(f[src]);
  }
  interpolated_links(p, b, n, flag, g, OwnFromHist<ST>{hist}, fx, fy, fz, any);
}

template <int ST>
__global__ void __launch_bounds__(NTHREADS) aa_interp_state(StepParams p, int odd_layout, int refresh) {
  const uint32_t x = blockIdx.x * BX + threadIdx.x;
  const uint32_t y = blockIdx.y * BY + threadIdx.y;
  const uint32_t z = blockIdx.z;
  bool any = false;
  double fx = 0, fy = 0, fz = 0;
  if (x < p.nx && y < p.ny) interpolated_state_cell<ST>(p, odd_layout, refresh, x, y, z, fx, fy, fz, any);
  reduce_force(any, fx, fy, fz, p.partials);
}

#if !PW_STRICT
template <int ST>
__global__ void __launch_bounds__(NTHREADS) aa_interp_state_edges(StepParams p, int odd_layout, int refresh,
                                                                  const uint32_t *list, uint32_t count) {
  const uint32_t t = blockIdx.x * NTHREADS + threadIdx.x;
  bool any = false;
  double fx = 0, fy = 0, fz = 0;
  if (t < count) {
    uint32_t x, y, z;
    cell_coords(p, __ldg(&list[t]), x, y, z);
    interpolated_state_cell<ST>(p, odd_layout, refresh, x, y, z, fx, fy, fz, any);
  }
  reduce_force(any, fx, fy, fz, p.partials);
}
#endif

// FP64 mass deviation and momentum of the latest state over non-wall cells.
template <int ST>
__global__ void __launch_bounds__(NTHREADS) aa_totals(StepParams p, int odd_layout, double *out) {
  using S = Store<ST>;
  using T = typename S::T;
  const T *f = reinterpret_cast<const T *>(p.f);
  const uint32_t x = blockIdx.x * BX + threadIdx.x;
  const uint32_t y = blockIdx.y * BY + threadIdx.y;
  const uint32_t z = blockIdx.z;
  double m = 0, jx = 0, jy = 0, jz = 0;
  if (x < p.nx && y < p.ny) {
    const uint32_t n = x + p.nx * (y + p.ny * z);
    if (!is_wall_kind(p.flags[n] & 7u)) {
      const Nbr b = make_nbr(p, x, y, z);
#pragma unroll
      for (int j = 0; j < 19; j++) {
        double v = S::decode(f[odd_layout ? slot_of<true>(b, j, p.stride, n) : slot_of<false>(b, j, p.stride, n)]);
        m += v;
        jx += cx_of(j) * v;
        jy += cy_of(j) * v;
        jz += cz_of(j) * v;
      }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    m += __shfl_down_sync(0xffffffffu, m, o);
    jx += __shfl_down_sync(0xffffffffu, jx, o);
    jy += __shfl_down_sync(0xffffffffu, jy, o);
    jz += __shfl_down_sync(0xffffffffu, jz, o);
  }
  if (((threadIdx.x + BX * threadIdx.y) & 31) == 0) {
    atomicAdd(out + 0, m);
    atomicAdd(out + 1, jx);
    atomicAdd(out + 2, jy);
    atomicAdd(out + 3, jz);
  }
}

// ---------------------------------------------------------------- launchers
#ifdef PW_DEFINE_LAUNCHERS
template <int ST, int OP, bool LES>
static void step3(const StepParams &p, bool odd, dim3 g, cudaStream_t s) {
  dim3 blk(BX, BY);
#if PW_STRICT
  if (odd) aa_step<ST, OP, LES, true><<<g, blk, 0, s>>>(p);
  else aa_step<ST, OP, LES, false><<<g, blk, 0, s>>>(p);
#else
  if (odd) aa_step_fast<ST, OP, LES, true><<<g, blk, 0, s>>>(p);
  else aa_step_fast<ST, OP, LES, false><<<g, blk, 0, s>>>(p);
#endif
}
template <int ST>
static void step2(const StepParams &p, int op, int les, bool odd, dim3 g, cudaStream_t s) {
  if (op == OP_REG) { if (les) step3<ST, OP_REG, true>(p, odd, g, s); else step3<ST, OP_REG, false>(p, odd, g, s); }
  else { if (les) step3<ST, OP_TRT, true>(p, odd, g, s); else step3<ST, OP_TRT, false>(p, odd, g, s); }
}
void launch_step(const StepParams &p, int storage, int op, int les, bool odd, dim3 g, cudaStream_t s) {
  switch (storage) {
    case STORE_F16: step2<STORE_F16>(p, op, les, odd, g, s); break;
    case STORE_BF16: step2<STORE_BF16>(p, op, les, odd, g, s); break;
    default: step2<STORE_F32>(p, op, les, odd, g, s); break;
  }
}
#define PW_DISPATCH(storage, CALL)                         \
  switch (storage) {                                       \
    case STORE_F16: { constexpr int ST = STORE_F16; CALL; break; } \
    case STORE_BF16: { constexpr int ST = STORE_BF16; CALL; break; } \
    default: { constexpr int ST = STORE_F32; CALL; break; } \
  }
#if !PW_STRICT
static inline void mark(const cudaEvent_t *ev, int k, cudaStream_t s) {
  if (ev) cudaEventRecord(ev[k], s);
}
// The seam rows of an odd step: as cell pairs with periodic faces (16-bit
// storage, nx even), else one cell per thread (free-slip faces reflect).
template <int ST, int OP, bool LES>
static void launch_seam(const StepParams &p, dim3 g, cudaStream_t s) {
  const uint32_t rows = seam_rows(p.ny, p.nz);
  if constexpr (ST != STORE_F32) {
    if ((p.nx & 1u) == 0u && p.slip == 0u) {
      const dim3 grid((p.nx + 2 * BX - 1) / (2 * BX), (rows + BY - 1) / BY);
      aa_step_seam_pairs<ST, OP, LES><<<grid, dim3(BX, BY), 0, s>>>(p);
      return;
    }
  }
  aa_step_seam<ST, OP, LES><<<dim3(g.x, rows), BX, 0, s>>>(p);
}

// The floor layer's kernel, when the domain's floor rows are on (16-bit
// storage with nx even only: the floor rows are decided at domain creation).
template <int ST, int OP, bool LES>
static void launch_floor(const StepParams &p, bool odd, cudaStream_t s) {
  if constexpr (ST != STORE_F32) {
    if (!p.floor_rows || p.ny < 3u) return;
    const dim3 grid((p.nx + 2 * BX - 1) / (2 * BX), (p.ny - 2u + BY - 1u) / BY);
    if (odd) aa_step_floor<ST, OP, LES, true><<<grid, dim3(BX, BY), 0, s>>>(p);
    else aa_step_floor<ST, OP, LES, false><<<grid, dim3(BX, BY), 0, s>>>(p);
  } else {
    (void)p; (void)odd; (void)s;
  }
}

template <int ST, int OP, bool LES>
static void step_split3(const StepParams &p, bool odd, dim3 g, const uint32_t *list, uint32_t count, cudaStream_t s,
                        const cudaEvent_t *ev, const SideStream *side) {
  const bool plain = g.x && g.y && g.z;
  // the seam and edge kernels: on the side stream when there is one
  cudaStream_t t = side ? side->stream : s;
  if (side) {
    cudaEventRecord(side->fork, s);
    cudaStreamWaitEvent(t, side->fork, 0);
  }
  if (side) {
    // launched first so their few blocks start before the plain grid fills the GPU
    if (plain && odd) launch_seam<ST, OP, LES>(p, g, t);
    launch_floor<ST, OP, LES>(p, odd, t);
    if (count) {
      unsigned blocks = (count + NTHREADS - 1) / NTHREADS;
      if (odd) aa_step_edges<ST, OP, LES, true><<<blocks, NTHREADS, 0, t>>>(p, list, count);
      else aa_step_edges<ST, OP, LES, false><<<blocks, NTHREADS, 0, t>>>(p, list, count);
    }
  }
  if (plain) {
    const unsigned runs = (p.nx + 2 * BX - 1) / (2 * BX);  // 64-cell runs per row
    // 16-bit storage with whole 32-bit pairs in a row: the pair kernel
    const bool pairs = ST != STORE_F32 && (p.nx & 1u) == 0u;
    if (odd) {
      dim3 inner(runs, p.ny > 2u ? (p.ny - 2u + BY - 1u) / BY : 0u, p.nz > 2u ? p.nz - 2u : 0u);
      mark(ev, 0, s);
      if (inner.y && inner.z) {
        if constexpr (ST != STORE_F32) {
          if (pairs) aa_step_pairs<ST, OP, LES, true><<<inner, dim3(BX, BY), 0, s>>>(p);
          else aa_step_fast<ST, OP, LES, true><<<inner, dim3(BX, BY), 0, s>>>(p);
        } else {
          aa_step_fast<ST, OP, LES, true><<<inner, dim3(BX, BY), 0, s>>>(p);
        }
      }
      mark(ev, 1, s);
      mark(ev, 2, s);
      if (!side) launch_seam<ST, OP, LES>(p, g, s);
      mark(ev, 3, s);
    } else {
      mark(ev, 0, s);
      if constexpr (ST != STORE_F32) {
        if (pairs) aa_step_pairs<ST, OP, LES, false><<<dim3(runs, g.y, g.z), dim3(BX, BY), 0, s>>>(p);
        else aa_step_fast<ST, OP, LES, false><<<dim3(runs, g.y, g.z), dim3(BX, BY), 0, s>>>(p);
      } else {
        (void)pairs;
        aa_step_fast<ST, OP, LES, false><<<dim3(runs, g.y, g.z), dim3(BX, BY), 0, s>>>(p);
      }
      mark(ev, 1, s);
      mark(ev, 2, s);
      mark(ev, 3, s);
    }
  }
  if (side) {
    cudaEventRecord(side->join, t);
    cudaStreamWaitEvent(s, side->join, 0);
    return;
  }
  mark(ev, 4, s);
  launch_floor<ST, OP, LES>(p, odd, s);
  if (count) {
    unsigned blocks = (count + NTHREADS - 1) / NTHREADS;
    if (odd) aa_step_edges<ST, OP, LES, true><<<blocks, NTHREADS, 0, s>>>(p, list, count);
    else aa_step_edges<ST, OP, LES, false><<<blocks, NTHREADS, 0, s>>>(p, list, count);
  }
  mark(ev, 5, s);
}
template <int ST>
static void step_split2(const StepParams &p, int op, int les, bool odd, dim3 g, const uint32_t *list, uint32_t count,
                        cudaStream_t s, const cudaEvent_t *ev, const SideStream *side) {
  if (op == OP_REG) {
    if (les) step_split3<ST, OP_REG, true>(p, odd, g, list, count, s, ev, side);
    else step_split3<ST, OP_REG, false>(p, odd, g, list, count, s, ev, side);
  } else {
    if (les) step_split3<ST, OP_TRT, true>(p, odd, g, list, count, s, ev, side);
    else step_split3<ST, OP_TRT, false>(p, odd, g, list, count, s, ev, side);
  }
}
void launch_step_split(const StepParams &p, int storage, int op, int les, bool odd, dim3 plain_grid,
                       const uint32_t *list, uint32_t count, cudaStream_t s, const cudaEvent_t *ev,
                       const SideStream *side) {
  if (ev) side = nullptr;  // per-kernel timing runs the kernels one after another
  switch (storage) {
    case STORE_F16: step_split2<STORE_F16>(p, op, les, odd, plain_grid, list, count, s, ev, side); break;
    case STORE_BF16: step_split2<STORE_BF16>(p, op, les, odd, plain_grid, list, count, s, ev, side); break;
    default: step_split2<STORE_F32>(p, op, les, odd, plain_grid, list, count, s, ev, side); break;
  }
}
#endif
void launch_init(const StepParams &p, float4 *plane_b, double *partials_b, int storage, dim3 g, cudaStream_t s) {
  PW_DISPATCH(storage, (aa_init<ST><<<g, dim3(BX, BY), 0, s>>>(p, plane_b, partials_b)))
}
void launch_init_lin(const StepParams &p, float4 *plane_b, double *partials_b, int storage, unsigned blocks,
                     uint32_t cpb, cudaStream_t s) {
  PW_DISPATCH(storage, (aa_init_lin<ST><<<blocks, NTHREADS, 0, s>>>(p, plane_b, partials_b, cpb)))
}
#if !PW_STRICT
void launch_refresh_edges(const StepParams &p, int odd_layout, int storage, const uint32_t *list, uint32_t count,
                          cudaStream_t s) {
  if (!count) return;
  unsigned blocks = (count + NTHREADS - 1) / NTHREADS;
  PW_DISPATCH(storage, (aa_refresh_edges<ST><<<blocks, NTHREADS, 0, s>>>(p, odd_layout, list, count)))
}
#endif
void launch_refresh_lin(const StepParams &p, int odd_layout, int storage, unsigned blocks, uint32_t cpb,
                        cudaStream_t s) {
  PW_DISPATCH(storage, (aa_refresh_lin<ST><<<blocks, NTHREADS, 0, s>>>(p, odd_layout, cpb)))
}
void launch_read(const StepParams &p, int odd_layout, int mode, void *out, int storage, dim3 g, cudaStream_t s) {
  PW_DISPATCH(storage, (aa_read<ST><<<g, dim3(BX, BY), 0, s>>>(p, odd_layout, mode, out)))
}
void launch_write(const StepParams &p, int odd_layout, int mode, const void *in, int storage, dim3 g, cudaStream_t s) {
  PW_DISPATCH(storage, (aa_write<ST><<<g, dim3(BX, BY), 0, s>>>(p, odd_layout, mode, in)))
}
void launch_refresh(const StepParams &p, int odd_layout, int storage, dim3 g, cudaStream_t s) {
  PW_DISPATCH(storage, (aa_refresh<ST><<<g, dim3(BX, BY), 0, s>>>(p, odd_layout)))
}
void launch_interp_state(const StepParams &p, int odd_layout, int refresh, int storage, dim3 g, const uint32_t *list,
                         uint32_t count, cudaStream_t s) {
#if !PW_STRICT
  if (list) {
    if (!count) return;
    unsigned blocks = (count + NTHREADS - 1) / NTHREADS;
    PW_DISPATCH(storage, (aa_interp_state_edges<ST><<<blocks, NTHREADS, 0, s>>>(p, odd_layout, refresh, list, count)))
    return;
  }
#endif
  PW_DISPATCH(storage, (aa_interp_state<ST><<<g, dim3(BX, BY), 0, s>>>(p, odd_layout, refresh)))
}
void launch_totals(const StepParams &p, int odd_layout, double *out, int storage, dim3 g, cudaStream_t s) {
  PW_DISPATCH(storage, (aa_totals<ST><<<g, dim3(BX, BY), 0, s>>>(p, odd_layout, out)))
}
#undef PW_DISPATCH
#endif

}  // namespace PW_NS
