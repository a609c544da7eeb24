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
// Same operator, fewer instructions: moments as signed direction sums,
// equilibrium split into even/odd parts per opposite pair, non-equilibrium
// stress from the second moment minus its closed-form equilibrium value
// (sum_i w_i c_a c_b g_eq,i = delta_ab rd/3 + rho u_a u_b).
template <int OP, bool LES>
__device__ __forceinline__ void update_fast(const StepParams &p, float *g, float &rho, float &vx,
                                            float &vy, float &vz) {
  float rd = ((g[0] + g[1]) + (g[2] + g[3])) + ((g[4] + g[5]) + (g[6] + g[7])) +
             ((g[8] + g[9]) + (g[10] + g[11])) + ((g[12] + g[13]) + (g[14] + g[15])) +
             ((g[16] + g[17]) + g[18]);
  float jx = ((g[1] - g[2]) + (g[7] - g[8])) + ((g[9] - g[10]) + (g[13] - g[14])) + (g[15] - g[16]);
  float jy = ((g[3] - g[4]) + (g[7] - g[8])) + ((g[11] - g[12]) + (g[14] - g[13])) + (g[17] - g[18]);
  float jz = ((g[5] - g[6]) + (g[9] - g[10])) + ((g[11] - g[12]) + (g[16] - g[15])) + (g[18] - g[17]);
  rho = 1.0f + rd;
  float inv = __frcp_rn(rho);
  vx = jx * inv;
  vy = jy * inv;
  vz = jz * inv;
  float uu = vx * vx + vy * vy + vz * vz;
  float K = rd - 1.5f * rho * uu;  // rd + rho(-1.5 uu): the cu-free part of the equilibrium
  float tau_plus = p.tau0, om_p = p.omega_plus, om_m = p.omega_minus;
  float pxx = 0.f, pyy = 0.f, pzz = 0.f, pxy = 0.f, pxz = 0.f, pyz = 0.f;
  if (LES || OP == OP_REG) {
    float sxx = ((g[1] + g[2]) + (g[7] + g[8])) + ((g[9] + g[10]) + (g[13] + g[14])) + (g[15] + g[16]);
    float syy = ((g[3] + g[4]) + (g[7] + g[8])) + ((g[11] + g[12]) + (g[13] + g[14])) + (g[17] + g[18]);
    float szz = ((g[5] + g[6]) + (g[9] + g[10])) + ((g[11] + g[12]) + (g[15] + g[16])) + (g[17] + g[18]);
    float sxy = (g[7] + g[8]) - (g[13] + g[14]);
    float sxz = (g[9] + g[10]) - (g[15] + g[16]);
    float syz = (g[11] + g[12]) - (g[17] + g[18]);
    float rd3 = rd * (1.0f / 3.0f);
    pxx = sxx - (rd3 + rho * vx * vx);
    pyy = syy - (rd3 + rho * vy * vy);
    pzz = szz - (rd3 + rho * vz * vz);
    pxy = sxy - rho * vx * vy;
    pxz = sxz - rho * vx * vz;
    pyz = syz - rho * vy * vz;
    if (LES) {
      float q = pxx * pxx + pyy * pyy + pzz * pzz + 2.0f * (pxy * pxy + pxz * pxz + pyz * pyz);
      float t0 = p.tau0;
      tau_plus = 0.5f * (t0 + sqrtf(t0 * t0 + p.cs_term * sqrtf(q) * inv));
      om_p = __frcp_rn(tau_plus);
      om_m = __frcp_rn(p.lambda * __frcp_rn(tau_plus - 0.5f) + 0.5f);
    }
  }
  if (OP == OP_REG) {
    const float c = (1.0f - om_p) * 4.5f;
    const float tr3 = (pxx + pyy + pzz) * (1.0f / 3.0f);
    const float r3 = 3.0f * rho, r45 = 4.5f * rho;
    // rest
    g[0] = w_of(0) * (K + c * (-tr3));
#define PW_REG_PAIR(I, CU, PROJ)                                        \
  {                                                                     \
    const float cu_ = (CU);                                             \
    const float ev_ = K + r45 * cu_ * cu_ + c * (PROJ);                 \
    const float od_ = r3 * cu_;                                         \
    g[I] = w_of(I) * (ev_ + od_);                                       \
    g[I + 1] = w_of(I) * (ev_ - od_);                                   \
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
    g[0] = g[0] - om_p * (g[0] - w_of(0) * K);
#define PW_TRT_PAIR(I, CU)                                              \
  {                                                                     \
    const float cu_ = (CU);                                             \
    const float ep_ = w_of(I) * (K + r45 * cu_ * cu_);                  \
    const float em_ = w_of(I) * (r3 * cu_);                             \
    const float gi_ = g[I], gj_ = g[I + 1];                             \
    const float a_ = hp * ((gi_ + gj_) - 2.0f * ep_);                   \
    const float b_ = hm * ((gi_ - gj_) - 2.0f * em_);                   \
    g[I] = gi_ - a_ - b_;                                               \
    g[I + 1] = gj_ - a_ + b_;                                           \
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
}

// ---------------------------------------------------------------- cell addressing
struct Nbr {
  uint32_t xm, x, xp;     // x - 1, x, x + 1 (periodic)
  uint32_t ym, y, yp;     // row offsets: (y-1)*nx, y*nx, (y+1)*nx
  uint32_t zm, z, zp;     // plane offsets
  __device__ __forceinline__ uint32_t at(int dx, int dy, int dz) const {
    return (dx < 0 ? xm : (dx > 0 ? xp : x)) + (dy < 0 ? ym : (dy > 0 ? yp : y)) +
           (dz < 0 ? zm : (dz > 0 ? zp : z));
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
  return b;
}

// Location of P(j, n) after a step of the given parity (the readout map).
template <bool ODD_LAYOUT>
__device__ __forceinline__ uint32_t slot_of(const Nbr &b, int j, uint32_t stride, uint32_t n) {
  if (ODD_LAYOUT) return (uint32_t)j * stride + b.at(cx_of(j), cy_of(j), cz_of(j));
  return (uint32_t)opp_of(j) * stride + n;
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
__device__ __forceinline__ void reduce_force(bool any, double fx, double fy, double fz, double *partials) {
  if (!__syncthreads_or(any)) return;
  __shared__ double red[NTHREADS / 32][3];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    fx += __shfl_down_sync(0xffffffffu, fx, o);
    fy += __shfl_down_sync(0xffffffffu, fy, o);
    fz += __shfl_down_sync(0xffffffffu, fz, o);
  }
  int t = threadIdx.x + BX * threadIdx.y;
  if ((t & 31) == 0) { red[t >> 5][0] = fx; red[t >> 5][1] = fy; red[t >> 5][2] = fz; }
  __syncthreads();
  if (t == 0) {
    double a = 0, b = 0, c = 0;
#pragma unroll
    for (int w = 0; w < NTHREADS / 32; w++) { a += red[w][0]; b += red[w][1]; c += red[w][2]; }
    size_t blk = blockIdx.x + (size_t)gridDim.x * (blockIdx.y + (size_t)gridDim.y * blockIdx.z);
    partials[3 * blk + 0] = a;
    partials[3 * blk + 1] = b;
    partials[3 * blk + 2] = c;
  }
}

// ---------------------------------------------------------------- the step
// ODD: this step reads layout E and writes layout O; otherwise the reverse.
template <int ST, int OP, bool LES, bool ODD>
__global__ void __launch_bounds__(NTHREADS) aa_step(StepParams p) {
  using S = Store<ST>;
  using T = typename S::T;
  T *f = reinterpret_cast<T *>(p.f);
  const uint32_t x = blockIdx.x * BX + threadIdx.x;
  const uint32_t y = blockIdx.y * BY + threadIdx.y;
  const uint32_t z = blockIdx.z;
  const uint32_t S_ = p.stride;
  bool force_any = false;
  double fx = 0.0, fy = 0.0, fz = 0.0;
  if (x < p.nx && y < p.ny) {
    const uint32_t n = x + p.nx * (y + p.ny * z);
    const bool special = (__ldg(&p.special[n >> 5]) >> (n & 31u)) & 1u;
    const uint32_t flag = special ? __ldg(&p.flags[n]) : 0u;
    const uint32_t kind = flag & 7u;
    const Nbr b = make_nbr(p, x, y, z);
    if (!is_wall_kind(kind)) {
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
          uint32_t src;
          if (ODD) src = (uint32_t)opp_of(i) * S_ + b.at(-cx_of(i), -cy_of(i), -cz_of(i));
          else src = (uint32_t)i * S_ + n;
          if (i > 0 && (flag & (1u << (3 + i)))) {  // wall link i: the slot nobody rewrites this step
            if (ODD) src = (uint32_t)i * S_ + n;
            else src = (uint32_t)opp_of(i) * S_ + b.at(-cx_of(i), -cy_of(i), -cz_of(i));
          }
          g[i] = S::decode(f[src]);
        }
#if PW_STRICT
        update_ref<OP, LES>(p, g, flag, post, rho, vx, vy, vz);
#else
        if (LES && (flag >> 3) != 0u) {
          update_ref<OP, LES>(p, g, flag, post, rho, vx, vy, vz);
        } else {
          update_fast<OP, LES>(p, g, rho, vx, vy, vz);
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
        uint32_t dst;
        if (ODD) dst = (uint32_t)j * S_ + b.at(cx_of(j), cy_of(j), cz_of(j));
        else dst = (uint32_t)opp_of(j) * S_ + n;
        f[dst] = code[j];
      }
      if (flag >> 3) {
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
  }
  reduce_force(force_any, fx, fy, fz, p.partials);
}

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
    for (int j = 0; j < 19; j++) f[(uint32_t)opp_of(j) * p.stride + n] = code[j];
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
  if (odd) aa_step<ST, OP, LES, true><<<g, blk, 0, s>>>(p);
  else aa_step<ST, OP, LES, false><<<g, blk, 0, s>>>(p);
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
void launch_init(const StepParams &p, float4 *plane_b, double *partials_b, int storage, dim3 g, cudaStream_t s) {
  PW_DISPATCH(storage, (aa_init<ST><<<g, dim3(BX, BY), 0, s>>>(p, plane_b, partials_b)))
}
void launch_init_lin(const StepParams &p, float4 *plane_b, double *partials_b, int storage, unsigned blocks,
                     uint32_t cpb, cudaStream_t s) {
  PW_DISPATCH(storage, (aa_init_lin<ST><<<blocks, NTHREADS, 0, s>>>(p, plane_b, partials_b, cpb)))
}
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
void launch_totals(const StepParams &p, int odd_layout, double *out, int storage, dim3 g, cudaStream_t s) {
  PW_DISPATCH(storage, (aa_totals<ST><<<g, dim3(BX, BY), 0, s>>>(p, odd_layout, out)))
}
#undef PW_DISPATCH
#endif

}  // namespace PW_NS
