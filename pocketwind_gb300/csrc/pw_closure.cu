// The learned subgrid closure (pw_closure_*): training data from the solver's
// own fine-grid fields, hand-written training (forward, backward, Adam), and
// inference fused into a step kernel on the tensor cores.  No counterpart in
// the reference.
//
// Data: a fine run's macros are box-filtered 2x2x2 onto the coarse grid; the
// target is the eddy viscosity that best reproduces the subgrid stress of the
// filtered fields, nu* = max(0, -tau_sgs : S / (2 S : S)), with
// tau_sgs = mean((u - ubar)(u - ubar)) and S the finite-difference strain of the
// filtered velocity, expressed as c* = nu* / nu_smag - 1 (clipped to [-1, 3]),
// nu_smag = (0.1)^2 |S| the Smagorinsky viscosity of the same strain.  Cells
// within two coarse cells of a wall or of the x faces are left out (the wall
// model owns the wall cells).
//
// Inference, periodic faces (closure_pairs): the plain step's two-cell update
// (update_fast2) with a hook between the Smagorinsky relaxation time and the
// reconstruction.  Each thread takes cells x and x + 32 of a row, a block the
// 256 cells of four rows; the hook takes each plain LES cell's strain
// S = -3 Pi_neq / (2 rho tau_s) and its nine inputs, and the block runs the
// network for its cells on the 5th-generation tensor cores as two tiles of
// M = 128 cells: each layer is one tcgen05.mma per tile of N = 32 outputs
// (K = 16 inputs, or two of K = 16 hidden units), bf16 operands in shared
// memory, binary32 accumulators in tensor memory, issued by one thread and
// read back by every thread for its own cells (tcgen05.ld); the update then
// goes on with tau = tau0 + (tau_s - tau0) max(0, 1 + c).  The wall-link cells
// and the floor layer run in the edge and floor kernels beside it with plain
// Smagorinsky and the reference's wall model, as in a step without the closure.
// Free-slip faces (closure_step): one cell per thread over every cell, 128
// cells per block, the same network on one tile; for the regularized operator
// the first pass's Smagorinsky post-collision state is corrected in place
// (finish_plain_reg), for TRT the cell goes through the one-cell path again.
#define PW_NS pwclosure
#define PW_STRICT 0
#include <algorithm>
#include <cmath>
#include <vector>

#include "pw_internal.h"
#include "pw_lbm.cuh"
#include "pw_closure.cuh"
#include "pw_launch.h"

using namespace pwhost;
using pw::StepParams;
using namespace pwcl;

namespace {

constexpr int kTrainThreads = 128;

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t *>(&v);
}

// ---------------------------------------------------------------- tensor-core operands
// K-major operands without swizzle: 8-row x 16-byte core matrices, element
// (row r, k) at byte (r % 8) * 16 + (r / 8) * SBO + (k / 8) * LBO + (k % 8) * 2
// (LBO: the next 8 elements of K; SBO: the next 8 rows).
constexpr uint32_t kLbo = 128;
__host__ __device__ constexpr uint32_t cm_offset(uint32_t r, uint32_t k, uint32_t sbo) {
  return (r & 7u) * 16u + (r >> 3) * sbo + (k >> 3) * kLbo + (k & 7u) * 2u;
}
constexpr uint32_t kSbo1 = 2 * kLbo, kSbo2 = 4 * kLbo;  // K = 16 (layer 1), K = 32 (layer 2)
// The network's image in global memory, copied to shared memory by each block:
// W1 (32 x 16, inputs 9..15 zero) and W2 (32 x 32) as bf16 operands, then b1,
// b2, W3 (bf16-rounded) and b3 as binary32.
constexpr uint32_t kImgW1 = 0, kImgW2 = 1024, kImgB1 = 3072, kImgB2 = kImgB1 + 128, kImgW3 = kImgB2 + 128,
                   kImgB3 = kImgW3 + 128, kImgBytes = kImgB3 + 16;
constexpr uint32_t kFragWords = 48;  // the image's buffer: 32 x 48 words (>= kImgBytes / 4)
static_assert(kImgBytes <= 4 * 32 * kFragWords, "network image does not fit its buffer");

__global__ void build_fragments(const float *w, uint32_t *frag) {
  unsigned char *img = reinterpret_cast<unsigned char *>(frag);
  for (uint32_t i = threadIdx.x; i < 32u * 16u; i += blockDim.x) {
    const uint32_t n = i >> 4, k = i & 15u;
    const float v = k < (uint32_t)kIn ? w[kW1 + n * kIn + k] : 0.0f;
    *reinterpret_cast<__nv_bfloat16 *>(img + kImgW1 + cm_offset(n, k, kSbo1)) = __float2bfloat16_rn(v);
  }
  for (uint32_t i = threadIdx.x; i < 32u * 32u; i += blockDim.x) {
    const uint32_t n = i >> 5, k = i & 31u;
    *reinterpret_cast<__nv_bfloat16 *>(img + kImgW2 + cm_offset(n, k, kSbo2)) =
        __float2bfloat16_rn(w[kW2 + n * kHidden + k]);
  }
  for (uint32_t j = threadIdx.x; j < 32u; j += blockDim.x) {
    reinterpret_cast<float *>(img + kImgB1)[j] = w[kB1 + j];
    reinterpret_cast<float *>(img + kImgB2)[j] = w[kB2 + j];
    reinterpret_cast<float *>(img + kImgW3)[j] = bf16_round(w[kW3 + j]);
  }
  if (threadIdx.x == 0) reinterpret_cast<float *>(img + kImgB3)[0] = w[kB3];
}

// tcgen05 instruction descriptor (kind::f16): binary32 accumulator, bf16 A and
// B, both K-major, N = 32, M = 128.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((32u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ uint32_t smem_u32(const void *ptr) { return (uint32_t)__cvta_generic_to_shared(ptr); }
// Shared-memory matrix descriptor: start, LBO, SBO (each in 16-byte units),
// the fixed version 1 at bit 46, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3fffu) | ((uint64_t)((kLbo >> 4) & 0x3fffu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3fffu) << 32) | ((uint64_t)1 << 46);
}
__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          tmem_d),
      "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void tc_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tc_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// 8 binary32 columns from column col of this thread's TMEM lane (warp w reads
// lanes 32w..32w+31), waited for.
__device__ __forceinline__ void tc_load8(uint32_t taddr, float *v) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 8; j++) v[j] = __uint_as_float(r[j]);
}

// Shared state of a block's network evaluation.
struct TcShared {
  __align__(128) unsigned char img[kImgBytes];   // the network image
  __align__(128) unsigned char a1[128 * 32];     // layer-1 operand: 128 cells x 16 inputs, bf16
  __align__(128) unsigned char a2[128 * 64];     // layer-2 operand: 128 cells x 32 hidden units, bf16
  __align__(8) uint64_t bar;                     // MMA completion
  uint32_t tmem;                                 // base of the block's 64 TMEM columns
  uint32_t failed;                               // a completion wait ran out
};

// Bounded wait on the MMA barrier's phase `parity`; false when it ran out
// (the caller then skips the network and keeps plain Smagorinsky, c = 0).
// Before returning false it waits once more, also bounded, so that an MMA
// still in flight can finish before its operands or columns are reused.
__device__ __forceinline__ bool tc_wait_once(uint64_t *bar, uint32_t parity) {
  for (uint32_t it = 0; it < (1u << 22); it++) {
    uint32_t ok;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(ok)
                 : "r"(smem_u32(bar)), "r"(parity)
                 : "memory");
    if (ok) return true;
  }
  return false;
}
__device__ __noinline__ void tc_drain(uint64_t *bar, uint32_t parity) { tc_wait_once(bar, parity); }
__device__ __forceinline__ bool tc_wait(uint64_t *bar, uint32_t parity) {
  if (tc_wait_once(bar, parity)) return true;
  tc_drain(bar, parity);  // out of line: the kernels' code stays small for the instruction cache
  return false;
}

// Block start: copy the image, set up the barrier, allocate 64 TMEM columns
// (warp 0).  All 128 threads call it.
template <class Sh>
__device__ void tc_setup(Sh &sh, const uint32_t *frag) {
  const uint32_t tid = threadIdx.x + 32u * threadIdx.y;
  const uint32_t *src = frag;
  uint32_t *dst = reinterpret_cast<uint32_t *>(sh.img);
  for (uint32_t i = tid; i < kImgBytes / 4u; i += 128u) dst[i] = __ldg(&src[i]);
  if (tid == 0) {
    sh.failed = 0u;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&sh.bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (tid < 32u) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 64;" ::"r"(smem_u32(&sh.tmem))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_before_sync();
  __syncthreads();
  tc_after_sync();
}

// Block end: free the TMEM columns (warp 0), after every thread's last read.
template <class Sh>
__device__ void tc_teardown(Sh &sh) {
  tc_before_sync();
  __syncthreads();
  tc_after_sync();
  if (threadIdx.x + 32u * threadIdx.y < 32u)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 64;" ::"r"(sh.tmem) : "memory");
}

// The network on the block's 128 cells: every thread passes its cell's inputs
// x (zeros for cells without a closure) and gets its c.  `phase` counts the
// barrier's completions (two per call).  Rounding as forward_scalar: inputs,
// weights and hidden activations in bf16, binary32 accumulation.
__device__ float block_mlp(TcShared &sh, const float x[kIn], uint32_t &phase) {
  const uint32_t tid = threadIdx.x + 32u * threadIdx.y, warp = tid >> 5;
  const uint32_t lane_addr = sh.tmem + ((warp * 32u) << 16);
  // layer-1 operand row: inputs 0..7 and 8..15 (9..15 zero) as two 16-byte pieces
  {
    uint4 lo, hi;
    lo.x = pack_bf16(x[0], x[1]); lo.y = pack_bf16(x[2], x[3]); lo.z = pack_bf16(x[4], x[5]);
    lo.w = pack_bf16(x[6], x[7]);
    hi.x = pack_bf16(x[8], 0.0f); hi.y = 0u; hi.z = 0u; hi.w = 0u;
    *reinterpret_cast<uint4 *>(sh.a1 + cm_offset(tid, 0, kSbo1)) = lo;
    *reinterpret_cast<uint4 *>(sh.a1 + cm_offset(tid, 8, kSbo1)) = hi;
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  tc_before_sync();
  __syncthreads();
  tc_after_sync();
  const bool live = sh.failed == 0u;
  if (tid == 0 && live) {
    tc_mma(sh.tmem, smem_desc(smem_u32(sh.a1), kSbo1), smem_desc(smem_u32(sh.img + kImgW1), kSbo1), 0u);
    tc_commit(&sh.bar);
  }
  // each warp reads TMEM only when all its lanes saw the layer complete
  const bool done1 = __all_sync(0xffffffffu, live && tc_wait(&sh.bar, phase & 1u));
  phase++;
  tc_after_sync();
  if (!done1 && live) atomicOr(&sh.failed, 1u);
  const float *b1 = reinterpret_cast<const float *>(sh.img + kImgB1);
#pragma unroll
  for (int k = 0; k < 32; k += 8) {  // eight columns at a time: fewer live registers
    float h[8];
    if (done1) {
      tc_load8(lane_addr + (uint32_t)k, h);
    } else {
#pragma unroll
      for (int j = 0; j < 8; j++) h[j] = 0.0f;
    }
    uint4 v;
    v.x = pack_bf16(tanh_fast(h[0] + b1[k]), tanh_fast(h[1] + b1[k + 1]));
    v.y = pack_bf16(tanh_fast(h[2] + b1[k + 2]), tanh_fast(h[3] + b1[k + 3]));
    v.z = pack_bf16(tanh_fast(h[4] + b1[k + 4]), tanh_fast(h[5] + b1[k + 5]));
    v.w = pack_bf16(tanh_fast(h[6] + b1[k + 6]), tanh_fast(h[7] + b1[k + 7]));
    *reinterpret_cast<uint4 *>(sh.a2 + cm_offset(tid, k, kSbo2)) = v;
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  tc_before_sync();
  __syncthreads();
  tc_after_sync();
  const bool live2 = sh.failed == 0u;
  if (tid == 0 && live2) {
    const uint32_t a2 = smem_u32(sh.a2), w2 = smem_u32(sh.img + kImgW2);
    tc_mma(sh.tmem + 32u, smem_desc(a2, kSbo2), smem_desc(w2, kSbo2), 0u);
    tc_mma(sh.tmem + 32u, smem_desc(a2 + 2u * kLbo, kSbo2), smem_desc(w2 + 2u * kLbo, kSbo2), 1u);
    tc_commit(&sh.bar);
  }
  const bool done2 = __all_sync(0xffffffffu, live2 && tc_wait(&sh.bar, phase & 1u));
  phase++;
  tc_after_sync();
  if (!done2) {
    if (live2) atomicOr(&sh.failed, 1u);
    return 0.0f;
  }
  const float *b2 = reinterpret_cast<const float *>(sh.img + kImgB2);
  const float *w3 = reinterpret_cast<const float *>(sh.img + kImgW3);
  float out = 0.0f;
#pragma unroll
  for (int k = 0; k < 32; k += 8) {
    float h[8];
    tc_load8(lane_addr + 32u + (uint32_t)k, h);
#pragma unroll
    for (int j = 0; j < 8; j++) out = fmaf(w3[k + j], bf16_round(tanh_fast(h[j] + b2[k + j])), out);
  }
  return out + reinterpret_cast<const float *>(sh.img + kImgB3)[0];
}

// Records the Smagorinsky state of a cell (first pass).
struct CaptureHook {
  float *s;  // tau_s, rho, ux, uy, uz, pxx, pyy, pzz, pxy, pxz, pyz
  __device__ __forceinline__ float operator()(const StepParams &, float tau_s, float rho, float vx, float vy, float vz,
                                              float pxx, float pyy, float pzz, float pxy, float pxz,
                                              float pyz) const {
    s[0] = tau_s; s[1] = rho; s[2] = vx; s[3] = vy; s[4] = vz;
    s[5] = pxx; s[6] = pyy; s[7] = pzz; s[8] = pxy; s[9] = pxz; s[10] = pyz;
    return tau_s;
  }
};

// Scales the Smagorinsky eddy viscosity by max(0, 1 + c) (second pass).
struct ClosureHook {
  float c;
  __device__ __forceinline__ float operator()(const StepParams &p, float tau_s, float, float, float, float, float,
                                              float, float, float, float, float) const {
    return p.tau0 + (tau_s - p.tau0) * fmaxf(0.0f, 1.0f + c);
  }
};

// Inputs of a cell from its Smagorinsky state (strain from the stress).
__device__ __forceinline__ void cell_inputs(const StepParams &p, const float *st, float wall, float x[kIn]) {
  const float tau_s = st[0], rho = st[1];
  const float k = -1.5f / (rho * tau_s);  // S = -Pi / (2 rho c_s^2 tau), c_s^2 = 1/3
  const float s[6] = {k * st[5], k * st[6], k * st[7], k * st[8], k * st[9], k * st[10]};
  const float nu_s = (tau_s - p.tau0) * (1.0f / 3.0f);
  features(s, rho, st[2], st[3], st[4], wall, p.nu, nu_s, p.u_in, x);
}

// REG collision of a plain cell with the closure's relaxation time, from its
// Smagorinsky post-collision state post (first pass): in the regularized
// operator the relaxation time enters only through (1 - omega) 4.5 w_i Q_i:Pi,
// so the closure's state is post_i + 4.5 (omega_s - omega) w_i Q_i:Pi (Q_i:Pi
// with the trace removed, as update_fast projects it).  Then the cell's
// rounding, stores, macros and outlet plane, as general_cell ends.
template <int ST, bool ODD>
__device__ __forceinline__ void finish_plain_reg(const StepParams &p, uint32_t x, uint32_t y, uint32_t z, uint32_t n,
                                                 const float *st, float c, float *post, bool interior) {
  using S = pw::Store<ST>;
  using T = typename S::T;
  const float tau_s = st[0];
  const float tau = p.tau0 + (tau_s - p.tau0) * fmaxf(0.0f, 1.0f + c);
  const float dc = 4.5f * (__fdividef(1.0f, tau_s) - __fdividef(1.0f, tau));
  const float pxx = st[5], pyy = st[6], pzz = st[7], pxy = st[8], pxz = st[9], pyz = st[10];
  const float tr3 = (pxx + pyy + pzz) * (1.0f / 3.0f);
  const float proj[10] = {-tr3,
                          pxx - tr3,
                          pyy - tr3,
                          pzz - tr3,
                          pxx + pyy + 2.0f * pxy - tr3,
                          pxx + pzz + 2.0f * pxz - tr3,
                          pyy + pzz + 2.0f * pyz - tr3,
                          pxx + pyy - 2.0f * pxy - tr3,
                          pxx + pzz - 2.0f * pxz - tr3,
                          pyy + pzz - 2.0f * pyz - tr3};
  post[0] = fmaf(dc * pw::w_of(0), proj[0], post[0]);
#pragma unroll
  for (int i = 1; i < 19; i++) post[i] = fmaf(dc * pw::w_of(i), proj[(i + 1) / 2], post[i]);
  const float rho = st[1];
  if (p.write_macro && !(rho >= 0.5f && rho <= 1.5f)) atomicOr(p.status, 1u);  // also catches NaN
  T *f = reinterpret_cast<T *>(p.f);
  T code[19];
#pragma unroll
  for (int j = 0; j < 19; j++) code[j] = S::encode(post[j], (uint32_t)j, n);
  if (interior) {
#pragma unroll
    for (int j = 0; j < 19; j++) f[n + p.st[j]] = code[j];
  } else {
    const pwclosure::Nbr b = pwclosure::make_nbr(p, x, y, z);
#pragma unroll
    for (int j = 0; j < 19; j++) f[ODD ? b.push(j, p.stride) : (pw::pidx)pw::opp_of(j) * p.stride + n] = code[j];
  }
  if (p.write_macro) p.macros[n] = make_float4(rho, st[2], st[3], st[4]);
  if (x + 2 == p.nx) p.plane_out[y + p.ny * z] = pwclosure::outlet_velocity_of<ST>(code);
}

// A persistent grid (four blocks per SM): each block sets up the network image
// and its TMEM columns once, then walks tiles of 32 x 4 cells of one z-plane,
// tiles W apart for W blocks.
template <int ST, int OP, bool ODD>
__global__ void __launch_bounds__(128, 4) closure_step(StepParams p, const uint32_t *frag, const uint8_t *wall_dist,
                                                       uint32_t tiles_x, uint32_t tiles_y) {
  using S = pw::Store<ST>;
  using T = typename S::T;
  __shared__ TcShared sh;
  __shared__ float post_s[OP == pw::OP_REG ? 19 : 1][128];  // REG: plain cells' Smagorinsky post-collision state
  tc_setup(sh, frag);
  uint32_t phase = 0;
  const uint32_t tid = threadIdx.x + 32u * threadIdx.y;
  const uint32_t tiles = tiles_x * tiles_y * p.nz;
  for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const uint32_t bx = tile % tiles_x, by = (tile / tiles_x) % tiles_y, z = tile / (tiles_x * tiles_y);
    const uint32_t x = bx * 32 + threadIdx.x;
    const uint32_t y = by * 4 + threadIdx.y;
    const bool in = x < p.nx && y < p.ny;
    const uint32_t n = in ? x + p.nx * (y + p.ny * z) : 0u;
    const uint32_t flag = in ? __ldg(&p.flags[n]) : (uint32_t)pw::SOLID;
    float xin[kIn], st[11];
#pragma unroll
    for (int k = 0; k < kIn; k++) xin[k] = 0.0f;
    const bool plain = in && flag == pw::FLUID;  // fluid without wall links
    // cells whose neighbours need no periodic wrap take the step's element
    // offsets from the kernel parameters (the wrap arithmetic otherwise)
    const bool interior = x >= 1u && x + 2u <= p.nx && y >= 1u && y + 2u <= p.ny && z >= 1u && z + 2u <= p.nz &&
                          p.slip == 0u;
    if (plain) {
      const T *f = reinterpret_cast<const T *>(p.f);
      float g[19];
      if (interior) {
#pragma unroll
        for (int i = 0; i < 19; i++) g[i] = S::decode(f[n + p.ld[i]]);
      } else {
        const pwclosure::Nbr b = pwclosure::make_nbr(p, x, y, z);
#pragma unroll
        for (int i = 0; i < 19; i++) g[i] = S::decode(f[ODD ? b.pull(i, p.stride) : (pw::pidx)i * p.stride + n]);
      }
      float rho, vx, vy, vz;
      pwclosure::update_fast<OP, true, CaptureHook>(p, g, rho, vx, vy, vz, 1.0f, 1.0f, CaptureHook{st});
      cell_inputs(p, st, (float)wall_dist[n], xin);
      if (OP == pw::OP_REG) {
#pragma unroll
        for (int i = 0; i < 19; i++) post_s[i][tid] = g[i];
      }
    }
    const float c = block_mlp(sh, xin, phase);
    bool any = false;
    double fx = 0.0, fy = 0.0, fz = 0.0;
    if (OP == pw::OP_REG && plain) {
      // single pass: the Smagorinsky state corrected to the closure's relaxation time
      float post[19];
#pragma unroll
      for (int i = 0; i < 19; i++) post[i] = post_s[OP == pw::OP_REG ? i : 0][tid];
      finish_plain_reg<ST, ODD>(p, x, y, z, n, st, c, post, interior);
    } else if (in) {
      pwclosure::general_cell<ST, OP, true, ODD, ClosureHook>(p, x, y, z, n, flag, fx, fy, fz, any, ClosureHook{c});
    }
    // the partial slot of tile (x block, y block, z), as the cell kernels number them
    const size_t slot = tile;
    pwclosure::reduce_force_at(any, fx, fy, fz, p.partials, slot, threadIdx.x + 32 * threadIdx.y);
  }
  if (threadIdx.x == 0 && threadIdx.y == 0 && sh.failed) atomicOr(p.status, 4u);
  tc_teardown(sh);
}

// ---------------------------------------------------------------- cell-pair closure step
// The closure step on the plain step's two-cell arithmetic (update_fast2):
// each thread takes cells x and x + 32 of a 64-cell run, as aa_step_fast does
// for every storage, and a block the 256 cells of four rows, so its network
// runs as two M = 128 tiles, the threads' first cells and their second cells.
// Every row of both parities runs here, the seam rows with their periodic
// wrap as per-row offsets (SeamWrap); the wall-link cells and the floor layer
// run in the edge and floor kernels beside it, with the reference's wall
// model, as in a step without the closure.
struct TcPair {
  __align__(128) unsigned char img[kImgBytes];   // the network image
  // the layer-2 operands of the two tiles (128 x 32 bf16 each); the two
  // layer-1 operands (128 x 16 each) share the first tile's, which layer 1's
  // MMAs have read by the time their outputs come back
  __align__(128) unsigned char a2[2][128 * 64];
  __align__(8) uint64_t bar;                     // MMA completion
  uint32_t tmem;                                 // 64 TMEM columns: tile t's layer output at column 32 t
  uint32_t failed;                               // a completion wait ran out
  __device__ __forceinline__ unsigned char *a1(int t) { return a2[0] + t * (128 * 32); }
};

__device__ __forceinline__ void put_inputs(unsigned char *a1, uint32_t row, const float x[kIn]) {
  uint4 lo, hi;
  lo.x = pack_bf16(x[0], x[1]); lo.y = pack_bf16(x[2], x[3]); lo.z = pack_bf16(x[4], x[5]);
  lo.w = pack_bf16(x[6], x[7]);
  hi.x = pack_bf16(x[8], 0.0f); hi.y = 0u; hi.z = 0u; hi.w = 0u;
  *reinterpret_cast<uint4 *>(a1 + cm_offset(row, 0, kSbo1)) = lo;
  *reinterpret_cast<uint4 *>(a1 + cm_offset(row, 8, kSbo1)) = hi;
}

// block_mlp for the block's two tiles: c of the thread's first (.x) and
// second (.y) cell.  Layer 2 writes the columns layer 1's outputs were read
// from, after the block barrier that follows those reads.  The loops over
// the two tiles stay rolled: the smaller kernel measured 3.7% faster (its
// warps had waited on instruction fetch more than on anything else).
__device__ float2 block_mlp2(TcPair &sh, const float xa[kIn], const float xb[kIn], uint32_t &phase) {
  const uint32_t tid = threadIdx.x + 32u * threadIdx.y, warp = tid >> 5;
  const uint32_t lane_addr = sh.tmem + ((warp * 32u) << 16);
  put_inputs(sh.a1(0), tid, xa);
  put_inputs(sh.a1(1), tid, xb);
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  tc_before_sync();
  __syncthreads();
  tc_after_sync();
  const bool live = sh.failed == 0u;
  if (tid == 0 && live) {
    const uint64_t w1 = smem_desc(smem_u32(sh.img + kImgW1), kSbo1);
    tc_mma(sh.tmem, smem_desc(smem_u32(sh.a1(0)), kSbo1), w1, 0u);
    tc_mma(sh.tmem + 32u, smem_desc(smem_u32(sh.a1(1)), kSbo1), w1, 0u);
    tc_commit(&sh.bar);
  }
  const bool done1 = __all_sync(0xffffffffu, live && tc_wait(&sh.bar, phase & 1u));
  phase++;
  tc_after_sync();
  if (!done1 && live) atomicOr(&sh.failed, 1u);
  const float *b1 = reinterpret_cast<const float *>(sh.img + kImgB1);
#pragma unroll 1
  for (int t = 0; t < 2; t++) {
#pragma unroll
    for (int k = 0; k < 32; k += 8) {
      float h[8];
      if (done1) {
        tc_load8(lane_addr + 32u * t + (uint32_t)k, h);
      } else {
#pragma unroll
        for (int j = 0; j < 8; j++) h[j] = 0.0f;
      }
      uint4 v;
      v.x = pack_bf16(tanh_fast(h[0] + b1[k]), tanh_fast(h[1] + b1[k + 1]));
      v.y = pack_bf16(tanh_fast(h[2] + b1[k + 2]), tanh_fast(h[3] + b1[k + 3]));
      v.z = pack_bf16(tanh_fast(h[4] + b1[k + 4]), tanh_fast(h[5] + b1[k + 5]));
      v.w = pack_bf16(tanh_fast(h[6] + b1[k + 6]), tanh_fast(h[7] + b1[k + 7]));
      *reinterpret_cast<uint4 *>(sh.a2[t] + cm_offset(tid, k, kSbo2)) = v;
    }
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  tc_before_sync();
  __syncthreads();
  tc_after_sync();
  const bool live2 = sh.failed == 0u;
  if (tid == 0 && live2) {
    const uint32_t w2 = smem_u32(sh.img + kImgW2);
#pragma unroll
    for (int t = 0; t < 2; t++) {
      const uint32_t a2 = smem_u32(sh.a2[t]);
      tc_mma(sh.tmem + 32u * t, smem_desc(a2, kSbo2), smem_desc(w2, kSbo2), 0u);
      tc_mma(sh.tmem + 32u * t, smem_desc(a2 + 2u * kLbo, kSbo2), smem_desc(w2 + 2u * kLbo, kSbo2), 1u);
    }
    tc_commit(&sh.bar);
  }
  const bool done2 = __all_sync(0xffffffffu, live2 && tc_wait(&sh.bar, phase & 1u));
  phase++;
  tc_after_sync();
  if (!done2) {
    if (live2) atomicOr(&sh.failed, 1u);
    return make_float2(0.0f, 0.0f);
  }
  const float *b2 = reinterpret_cast<const float *>(sh.img + kImgB2);
  const float *w3 = reinterpret_cast<const float *>(sh.img + kImgW3);
  float out0 = 0.0f, out1 = 0.0f;
#pragma unroll 1
  for (int t = 0; t < 2; t++) {
    float o = 0.0f;
#pragma unroll
    for (int k = 0; k < 32; k += 8) {
      float h[8];
      tc_load8(lane_addr + 32u * t + (uint32_t)k, h);
#pragma unroll
      for (int j = 0; j < 8; j++) o = fmaf(w3[k + j], bf16_round(tanh_fast(h[j] + b2[k + j])), o);
    }
    if (t == 0) out0 = o; else out1 = o;
  }
  const float b3 = reinterpret_cast<const float *>(sh.img + kImgB3)[0];
  return make_float2(out0 + b3, out1 + b3);
}

// update_fast2's hook: the network's relaxation time for the lanes in live
// (bit 0 .x, bit 1 .y: plain LES cells), the Smagorinsky one for the others.
struct ClosureHook2 {
  TcPair *sh;
  uint32_t *phase;
  float2 wall;
  uint32_t live;
  __device__ __forceinline__ float2 operator()(const StepParams &p, float2 tau_s, float2 rho, float2 vx, float2 vy,
                                               float2 vz, float2 pxx, float2 pyy, float2 pzz, float2 pxy, float2 pxz,
                                               float2 pyz) const {
    float xa[kIn], xb[kIn];
#pragma unroll
    for (int k = 0; k < kIn; k++) xa[k] = xb[k] = 0.0f;
    if (live & 1u) {
      const float st[11] = {tau_s.x, rho.x, vx.x, vy.x, vz.x, pxx.x, pyy.x, pzz.x, pxy.x, pxz.x, pyz.x};
      cell_inputs(p, st, wall.x, xa);
    }
    if (live & 2u) {
      const float st[11] = {tau_s.y, rho.y, vx.y, vy.y, vz.y, pxx.y, pyy.y, pzz.y, pxy.y, pxz.y, pyz.y};
      cell_inputs(p, st, wall.y, xb);
    }
    const float2 c = block_mlp2(*sh, xa, xb, *phase);
    float2 tau = tau_s;
    if (live & 1u) tau.x = p.tau0 + (tau_s.x - p.tau0) * fmaxf(0.0f, 1.0f + c.x);
    if (live & 2u) tau.y = p.tau0 + (tau_s.y - p.tau0) * fmaxf(0.0f, 1.0f + c.y);
    return tau;
  }
};

// A persistent grid: each block sets up the network image and its TMEM
// columns once, then walks tiles of 64 x 4 cells of one z-plane, tiles W apart
// for W blocks.  Plain cells and EQ cells without wall links are stored, as in
// aa_step_fast; every thread takes part in each tile's network.
// Eight blocks per SM (64 registers; all 512 TMEM columns): measured 6%
// faster than six (80 registers) and 9% faster than four.
#ifndef PW_CLOSURE_PAIR_BLOCKS
#define PW_CLOSURE_PAIR_BLOCKS 8
#endif
static_assert(PW_CLOSURE_PAIR_BLOCKS * 64 <= 512, "the blocks of an SM must fit its 512 TMEM columns");
template <int ST, int OP, bool ODD>
__global__ void __launch_bounds__(128, PW_CLOSURE_PAIR_BLOCKS) closure_pairs(StepParams p, const uint32_t *frag, const uint8_t *wall_dist,
                                                        uint32_t runs, uint32_t row_blocks) {
  using S = pw::Store<ST>;
  using T = typename S::T;
  __shared__ TcPair sh;
  tc_setup(sh, frag);
  uint32_t phase = 0;
  T *f = reinterpret_cast<T *>(p.f);
  const uint32_t tiles = runs * row_blocks * p.nz;
  for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const uint32_t run = tile % runs, rest = tile / runs;
    const uint32_t x = run * 64u + threadIdx.x, y = (rest % row_blocks) * 4u + threadIdx.y, z = rest / row_blocks;
    const bool row_in = y < p.ny;
    const uint32_t n = x + p.nx * ((row_in ? y : 0u) + p.ny * z);
    uint32_t ok = 0u, eq = 0u;
    if (row_in) {
#pragma unroll
      for (uint32_t k = 0; k < 2u; k++) {
        const uint32_t xk = x + 32u * k, nk = n + 32u * k;
        if (xk >= p.nx) continue;
        if (!((__ldg(&p.special[nk >> 5]) >> (nk & 31u)) & 1u)) {
          if (pwclosure::is_plain_position(xk, p.nx)) ok |= 1u << k;
        } else if (__ldg(&p.flags[nk]) == pw::EQ) {
          ok |= 1u << k;
          eq |= 1u << k;
        }
      }
    }
    const uint32_t live = ok & ~eq;
    // odd steps pull across the periodic y and z faces on the seam rows (the
    // offsets are zero on the other rows: one code path keeps the kernel small,
    // measured 3.7% faster than a separate path for the seam rows)
    const pwclosure::SeamWrap sw = ODD && row_in ? pwclosure::SeamWrap(p, y, z, 1) : pwclosure::SeamWrap();
    float2 g[19];
    if (row_in) {
#pragma unroll
      for (int i = 0; i < 19; i++) {
        const T *a = f + (n + p.ld[i] + sw.of(i));
        g[i] = make_float2(S::raw(a[0]), S::raw(a[32]));
      }
    } else {
#pragma unroll
      for (int i = 0; i < 19; i++) g[i] = make_float2(0.0f, 0.0f);
    }
    float2 eux = pwclosure::f2(p.u_in), euy = pwclosure::f2(0.f), euz = pwclosure::f2(0.f);
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
    const float2 wall = make_float2((live & 1u) ? (float)wall_dist[n] : 0.0f, (live & 2u) ? (float)wall_dist[n + 32] : 0.0f);
    float2 rho, vx, vy, vz;
    const float2 om = pwclosure::update_fast2<OP, true, ClosureHook2>(
        p, g, rho, vx, vy, vz, S::kScale, S::kInvScale, eq, eux, euy, euz, ClosureHook2{&sh, &phase, wall, live});
    if (!ok) continue;
    if (ST != pw::STORE_F32) {
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
    const uint32_t xa = x, xb = x + 32u;
#pragma unroll
    for (int j = 0; j < 19; j++) {
      // odd steps: the EQ cell at x = 0 pushes c_x = -1 to x = nx - 1 and the
      // one at x = nx - 1 pushes c_x = +1 to x = 0 (signed element offsets)
      const int cx = pw::cx_of(j);
      const int64_t wa = !ODD ? 0 : (cx < 0 && xa == 0u ? (int64_t)p.nx : (cx > 0 && xa + 1u == p.nx ? -(int64_t)p.nx : 0));
      const int64_t wb = ODD && cx > 0 && xb + 1u == p.nx ? -(int64_t)p.nx : 0;
      T ca, cb;
      pwclosure::encode_two<ST>(g[j], j, nk, nk2, ca, cb);
      T *a = f + (n + p.st[j] + sw.of(pw::opp_of(j)));
      if (ok & 1u) a[wa] = ca;
      if (ok & 2u) a[32 + wb] = cb;
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
      const pwclosure::Nbr b = pwclosure::make_nbr(p, xo, y, z);
      T code[19];
#pragma unroll
      for (int j = 0; j < 19; j++) code[j] = f[pwclosure::slot_of<ODD>(b, j, p.stride, no)];
      p.plane_out[y + p.ny * z] = pwclosure::outlet_velocity_of<ST>(code);
    }
  }
  if (threadIdx.x == 0 && threadIdx.y == 0 && sh.failed) atomicOr(p.status, 4u);
  tc_teardown(sh);
}

// Network outputs for given inputs through the same tensor-core path (tests);
// *status gets bit 0 if a completion wait ran out.
__global__ void __launch_bounds__(128) eval_kernel(const uint32_t *frag, const float *xin, uint32_t count, float *out,
                                                   uint32_t *status) {
  __shared__ TcShared sh;
  tc_setup(sh, frag);
  uint32_t phase = 0;
  const uint32_t i = blockIdx.x * 128 + threadIdx.x;
  float x[kIn];
#pragma unroll
  for (int k = 0; k < kIn; k++) x[k] = i < count ? xin[(size_t)i * kIn + k] : 0.0f;
  const float c = block_mlp(sh, x, phase);
  if (i < count) out[i] = c;
  if (threadIdx.x == 0 && sh.failed) atomicOr(status, 1u);
  tc_teardown(sh);
}

// ---------------------------------------------------------------- wall distance
// Cells to the nearest wall cell (6-neighbour steps, capped at kWallCap): x
// bounded, y and z periodic as the lattice.
__global__ void dist_init(const uint32_t *flags, size_t cells, uint8_t *d) {
  const size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n < cells) d[n] = pw::is_wall_kind(flags[n] & 7u) ? 0 : 255;
}
__global__ void dist_from_solid(const uint8_t *solid, size_t cells, uint8_t *d) {
  const size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n < cells) d[n] = solid[n] ? 0 : 255;
}
__global__ void dist_step(const uint8_t *in, uint8_t *out, uint32_t nx, uint32_t ny, uint32_t nz) {
  const size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= (size_t)nx * ny * nz) return;
  const uint32_t x = (uint32_t)(n % nx), y = (uint32_t)((n / nx) % ny), z = (uint32_t)(n / ((size_t)nx * ny));
  const size_t plane = (size_t)nx * ny;
  uint32_t v = in[n];
  if (x > 0) v = min(v, in[n - 1] + 1u);
  if (x + 1 < nx) v = min(v, in[n + 1] + 1u);
  v = min(v, in[n - (size_t)y * nx + (size_t)((y + ny - 1) % ny) * nx] + 1u);
  v = min(v, in[n - (size_t)y * nx + (size_t)((y + 1) % ny) * nx] + 1u);
  v = min(v, in[n - (size_t)z * plane + (size_t)((z + nz - 1) % nz) * plane] + 1u);
  v = min(v, in[n - (size_t)z * plane + (size_t)((z + 1) % nz) * plane] + 1u);
  out[n] = (uint8_t)min(v, 255u);
}

int wall_distance(uint8_t *d, uint8_t *tmp, uint32_t nx, uint32_t ny, uint32_t nz, cudaStream_t s) {
  const size_t cells = (size_t)nx * ny * nz;
  const unsigned blocks = (unsigned)((cells + 255) / 256);
  for (int k = 0; k < (int)kWallCap; k += 2) {
    dist_step<<<blocks, 256, 0, s>>>(d, tmp, nx, ny, nz);
    dist_step<<<blocks, 256, 0, s>>>(tmp, d, nx, ny, nz);
  }
  PW_TRY(cudaGetLastError());
  return PW_OK;
}

// ---------------------------------------------------------------- training data
// coarse[q][N]: rho, ux, uy, uz and the subgrid stress mean((u - ubar)(u - ubar)):
// xx, yy, zz, xy, xz, yz (taken from the deviations, free of the cancellation
// of mean(u u) - ubar ubar in binary32).
__global__ void coarsen_kernel(const float4 *macros, const uint32_t *flags, uint32_t nx, uint32_t ny, uint32_t nz,
                               float *coarse, uint8_t *solid) {
  const uint32_t cx = nx / 2, cy = ny / 2, cz = nz / 2;
  const size_t nc = (size_t)cx * cy * cz;
  const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  const uint32_t X = (uint32_t)(c % cx), Y = (uint32_t)((c / cx) % cy), Z = (uint32_t)(c / ((size_t)cx * cy));
  float4 m[8];
  float mean[4] = {0, 0, 0, 0};
  uint32_t walls = 0;
  for (uint32_t k = 0; k < 8; k++) {
    const size_t n = (2 * X + (k & 1)) + (size_t)nx * ((2 * Y + ((k >> 1) & 1)) + (size_t)ny * (2 * Z + (k >> 2)));
    m[k] = macros[n];
    walls += pw::is_wall_kind(flags[n] & 7u) ? 1u : 0u;
    mean[0] += m[k].x; mean[1] += m[k].y; mean[2] += m[k].z; mean[3] += m[k].w;
  }
  for (int q = 0; q < 4; q++) mean[q] *= 0.125f;
  float t[6] = {0, 0, 0, 0, 0, 0};
  for (uint32_t k = 0; k < 8; k++) {
    const float dx = m[k].y - mean[1], dy = m[k].z - mean[2], dz = m[k].w - mean[3];
    t[0] += dx * dx; t[1] += dy * dy; t[2] += dz * dz; t[3] += dx * dy; t[4] += dx * dz; t[5] += dy * dz;
  }
  for (int q = 0; q < 4; q++) coarse[(size_t)q * nc + c] = mean[q];
  for (int q = 0; q < 6; q++) coarse[(size_t)(4 + q) * nc + c] = 0.125f * t[q];
  solid[c] = walls ? 1 : 0;
}

// Target and inputs of coarse cell c, or false when it is left out.
__device__ __forceinline__ bool coarse_sample(const float *co, const uint8_t *dist, uint32_t cx, uint32_t cy,
                                              uint32_t cz, size_t c, float nu0, float u_in, float x[kIn], float *y) {
  const size_t nc = (size_t)cx * cy * cz;
  const uint32_t X = (uint32_t)(c % cx), Y = (uint32_t)((c / cx) % cy), Z = (uint32_t)(c / ((size_t)cx * cy));
  if (X < 2 || X + 3 > cx || dist[c] < 2) return false;
  const size_t plane = (size_t)cx * cy;
  const size_t xm = c - 1, xp = c + 1;
  const size_t ym = c - (size_t)Y * cx + (size_t)((Y + cy - 1) % cy) * cx, yp = c - (size_t)Y * cx + (size_t)((Y + 1) % cy) * cx;
  const size_t zm = c - (size_t)Z * plane + (size_t)((Z + cz - 1) % cz) * plane;
  const size_t zp = c - (size_t)Z * plane + (size_t)((Z + 1) % cz) * plane;
  auto u = [&](int comp, size_t at) { return co[(size_t)(1 + comp) * nc + at]; };
  float grad[3][3];  // grad[a][b] = d u_b / d x_a
  for (int b = 0; b < 3; b++) {
    grad[0][b] = 0.5f * (u(b, xp) - u(b, xm));
    grad[1][b] = 0.5f * (u(b, yp) - u(b, ym));
    grad[2][b] = 0.5f * (u(b, zp) - u(b, zm));
  }
  const float s[6] = {grad[0][0], grad[1][1], grad[2][2], 0.5f * (grad[0][1] + grad[1][0]),
                      0.5f * (grad[0][2] + grad[2][0]), 0.5f * (grad[1][2] + grad[2][1])};
  const float ux = u(0, c), uy = u(1, c), uz = u(2, c);
  const float tsgs[6] = {co[4 * nc + c], co[5 * nc + c], co[6 * nc + c], co[7 * nc + c], co[8 * nc + c],
                         co[9 * nc + c]};
  const float ss = s[0] * s[0] + s[1] * s[1] + s[2] * s[2] + 2.0f * (s[3] * s[3] + s[4] * s[4] + s[5] * s[5]);
  const float ts = tsgs[0] * s[0] + tsgs[1] * s[1] + tsgs[2] * s[2] + 2.0f * (tsgs[3] * s[3] + tsgs[4] * s[4] + tsgs[5] * s[5]);
  const float nu_s = 0.01f * sqrtf(2.0f * ss);
  if (!(nu_s > 1e-9f)) return false;
  const float nu_t = fmaxf(0.0f, -ts / (2.0f * ss));
  *y = fminf(3.0f, fmaxf(-1.0f, nu_t / nu_s - 1.0f));
  features(s, co[c], ux, uy, uz, (float)dist[c], nu0, nu_s, u_in, x);
  return true;
}

constexpr int kScanBlock = 1024;

__global__ void sample_count(const float *co, const uint8_t *dist, uint32_t cx, uint32_t cy, uint32_t cz, float nu0,
                             float u_in, uint32_t *block_counts) {
  __shared__ uint32_t warp_counts[kScanBlock / 32];
  const size_t c = (size_t)blockIdx.x * kScanBlock + threadIdx.x;
  float x[kIn], y;
  const bool ok = c < (size_t)cx * cy * cz && coarse_sample(co, dist, cx, cy, cz, c, nu0, u_in, x, &y);
  const uint32_t ballot = __ballot_sync(0xffffffffu, ok);
  if ((threadIdx.x & 31) == 0) warp_counts[threadIdx.x >> 5] = __popc(ballot);
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int w = 0; w < kScanBlock / 32; w++) t += warp_counts[w];
    block_counts[blockIdx.x] = t;
  }
}

__global__ void scan_counts(uint32_t *counts, uint32_t nblk, uint32_t *total) {
  __shared__ uint32_t sh[kScanBlock];
  uint32_t carry = 0;
  for (uint32_t base = 0; base < nblk; base += kScanBlock) {
    const uint32_t i = base + threadIdx.x;
    const uint32_t v = i < nblk ? counts[i] : 0u;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < kScanBlock; o <<= 1) {
      const uint32_t add = threadIdx.x >= (unsigned)o ? sh[threadIdx.x - o] : 0u;
      __syncthreads();
      sh[threadIdx.x] += add;
      __syncthreads();
    }
    if (i < nblk) counts[i] = carry + sh[threadIdx.x] - v;
    carry += sh[kScanBlock - 1];
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

__global__ void sample_write(const float *co, const uint8_t *dist, uint32_t cx, uint32_t cy, uint32_t cz, float nu0,
                             float u_in, const uint32_t *offsets, uint64_t base, uint64_t cap, float *X, float *Y) {
  __shared__ uint32_t warp_base[kScanBlock / 32];
  const size_t c = (size_t)blockIdx.x * kScanBlock + threadIdx.x;
  float x[kIn], y = 0.0f;
  const bool ok = c < (size_t)cx * cy * cz && coarse_sample(co, dist, cx, cy, cz, c, nu0, u_in, x, &y);
  const uint32_t ballot = __ballot_sync(0xffffffffu, ok);
  const uint32_t lane = threadIdx.x & 31;
  if (lane == 0) warp_base[threadIdx.x >> 5] = __popc(ballot);
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = offsets[blockIdx.x];
    for (int w = 0; w < kScanBlock / 32; w++) { const uint32_t k = warp_base[w]; warp_base[w] = t; t += k; }
  }
  __syncthreads();
  if (!ok) return;
  const uint64_t at = base + warp_base[threadIdx.x >> 5] + __popc(ballot & ((1u << lane) - 1u));
  if (at >= cap) return;
  for (int k = 0; k < kIn; k++) X[at * kIn + k] = x[k];
  Y[at] = y;
}

// ---------------------------------------------------------------- training
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// One block of kTrainThreads samples: forward with the network's rounding,
// squared error against the target, backward (the bf16 roundings pass
// gradients through unchanged; tanh' = 1 - h^2 of the rounded activation),
// and the block's parameter-gradient sums and loss sum in partial[block].
// sample index: explicit list `idx` when given, else mix64(seed + step * 2^32 + i) mod n.
__global__ void __launch_bounds__(kTrainThreads) train_block(const float *w, const float *X, const float *Y, uint64_t n,
                                                             uint32_t batch, uint64_t seed, const uint32_t *step,
                                                             const uint32_t *idx, float *partial) {
  extern __shared__ float sm[];
  float *wr = sm;                                     // kParams rounded weights (biases kept)
  float *xs = wr + kParams + 3;                       // [kTrainThreads][kIn]
  float *h1s = xs + kTrainThreads * kIn;              // [kTrainThreads][32]
  float *d1s = h1s + kTrainThreads * kHidden;
  float *h2s = d1s + kTrainThreads * kHidden;
  float *d2s = h2s + kTrainThreads * kHidden;
  float *d3s = d2s + kTrainThreads * kHidden;         // [kTrainThreads]
  float *ls = d3s + kTrainThreads;                    // [kTrainThreads]
  const uint32_t tid = threadIdx.x;
  for (int k = tid; k < kParams; k += kTrainThreads) {
    const bool bias = (k >= kB1 && k < kW2) || (k >= kB2 && k < kW3) || k == kB3;
    wr[k] = bias ? w[k] : bf16_round(w[k]);
  }
  __syncthreads();
  const uint32_t i = blockIdx.x * kTrainThreads + tid;
  const bool live = i < batch;
  uint64_t s = 0;
  if (live) s = idx ? idx[i] : mix64(seed + ((uint64_t)*step << 32) + i) % n;
  float x[kIn], h1[kHidden];
#pragma unroll
  for (int k = 0; k < kIn; k++) x[k] = live ? bf16_round(X[s * kIn + k]) : 0.0f;
  for (int j = 0; j < kHidden; j++) {
    float a = 0.0f;
#pragma unroll
    for (int k = 0; k < kIn; k++) a = fmaf(wr[kW1 + j * kIn + k], x[k], a);
    h1[j] = bf16_round(tanh_fast(a + wr[kB1 + j]));
  }
  float out = 0.0f;
  for (int j = 0; j < kHidden; j++) {
    float a = 0.0f;
    for (int k = 0; k < kHidden; k++) a = fmaf(wr[kW2 + j * kHidden + k], h1[k], a);
    const float h2 = bf16_round(tanh_fast(a + wr[kB2 + j]));
    h2s[tid * kHidden + j] = h2;
    out = fmaf(wr[kW3 + j], h2, out);
  }
  out += wr[kB3];
  const float err = live ? out - Y[s] : 0.0f;
  const float d3 = live ? 2.0f * err / (float)batch : 0.0f;
  ls[tid] = err * err;
  d3s[tid] = d3;
  for (int j = 0; j < kHidden; j++) {
    const float h2 = h2s[tid * kHidden + j];
    d2s[tid * kHidden + j] = d3 * wr[kW3 + j] * (1.0f - h2 * h2);
  }
  for (int k = 0; k < kHidden; k++) {
    float a = 0.0f;
    for (int j = 0; j < kHidden; j++) a = fmaf(d2s[tid * kHidden + j], wr[kW2 + j * kHidden + k], a);
    d1s[tid * kHidden + k] = a * (1.0f - h1[k] * h1[k]);
    h1s[tid * kHidden + k] = h1[k];
  }
#pragma unroll
  for (int k = 0; k < kIn; k++) xs[tid * kIn + k] = x[k];
  __syncthreads();
  float *out_p = partial + (size_t)blockIdx.x * (kParams + 1);
  for (int q = tid; q < kParams + 1; q += kTrainThreads) {
    float acc = 0.0f;
    if (q < kB1) {
      const int j = q / kIn, k = q % kIn;
      for (int r = 0; r < kTrainThreads; r++) acc = fmaf(d1s[r * kHidden + j], xs[r * kIn + k], acc);
    } else if (q < kW2) {
      for (int r = 0; r < kTrainThreads; r++) acc += d1s[r * kHidden + (q - kB1)];
    } else if (q < kB2) {
      const int j = (q - kW2) / kHidden, k = (q - kW2) % kHidden;
      for (int r = 0; r < kTrainThreads; r++) acc = fmaf(d2s[r * kHidden + j], h1s[r * kHidden + k], acc);
    } else if (q < kW3) {
      for (int r = 0; r < kTrainThreads; r++) acc += d2s[r * kHidden + (q - kB2)];
    } else if (q < kB3) {
      for (int r = 0; r < kTrainThreads; r++) acc = fmaf(d3s[r], h2s[r * kHidden + (q - kW3)], acc);
    } else if (q == kB3) {
      for (int r = 0; r < kTrainThreads; r++) acc += d3s[r];
    } else {
      for (int r = 0; r < kTrainThreads; r++) acc += ls[r];
    }
    out_p[q] = acc;
  }
}

// Fixed-order sums of the block partials: grad[q], q < kParams; grad[kParams] = loss sum.
__global__ void train_reduce(const float *partial, uint32_t blocks, float *grad) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q > (uint32_t)kParams) return;
  float acc = 0.0f;
  for (uint32_t b = 0; b < blocks; b++) acc += partial[(size_t)b * (kParams + 1) + q];
  grad[q] = acc;
}

// Adam (beta1 0.9, beta2 0.999, eps 1e-8) on the binary32 master weights; one
// block, which then advances the step counter and records the batch loss.
__global__ void train_adam(float *w, float *m, float *v, const float *grad, uint32_t *step, float lr, uint32_t batch,
                           float *loss) {
  const uint32_t t = *step + 1;
  const float c1 = 1.0f - powf(0.9f, (float)t), c2 = 1.0f - powf(0.999f, (float)t);
  for (int q = threadIdx.x; q < kParams; q += blockDim.x) {
    const float gq = grad[q];
    const float mq = 0.9f * m[q] + 0.1f * gq;
    const float vq = 0.999f * v[q] + 0.001f * gq * gq;
    m[q] = mq;
    v[q] = vq;
    w[q] -= lr * (mq / c1) / (sqrtf(vq / c2) + 1e-8f);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    *loss = grad[kParams] / (float)batch;
    *step = t;
  }
}

}  // namespace

struct pw_closure {
  float *w = nullptr, *m = nullptr, *v = nullptr, *grad = nullptr, *partial = nullptr, *loss = nullptr;
  uint32_t *frag = nullptr, *step = nullptr;
  float *X = nullptr, *Y = nullptr;
  uint64_t n = 0, cap = 0;
  uint32_t partial_blocks = 0;
  cudaStream_t stream = nullptr;
};

namespace {

size_t train_smem() {
  return sizeof(float) * (kParams + 3 + kTrainThreads * (kIn + 4 * kHidden + 2));
}

int ensure_partials(pw_closure *c, uint32_t blocks) {
  if (blocks <= c->partial_blocks) return PW_OK;
  cudaFree(c->partial);
  c->partial = nullptr;
  c->partial_blocks = 0;
  PW_TRY(cudaMalloc(&c->partial, (size_t)blocks * (kParams + 1) * sizeof(float)));
  c->partial_blocks = blocks;
  return PW_OK;
}

int refresh_fragments(pw_closure *c) {
  build_fragments<<<1, 32, 0, c->stream>>>(c->w, c->frag);
  PW_TRY(cudaGetLastError());
  return PW_OK;
}

}  // namespace

namespace pwclosure_host {
// Multiprocessors of the current device, cached per device (1 when unknown).
static int sm_count() {
  static int sms[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) { cudaGetLastError(); dev = 0; }
  if (!sms[dev] && cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    sms[dev] = 1;
  }
  return std::max(sms[dev], 1);
}

// The closure step for a domain with an attached closure (pw_domain.cu).
void launch_closure_step(const StepParams &p, int storage, int op, bool odd, dim3 grid, const uint32_t *frag,
                         const uint8_t *wall, cudaStream_t s) {
  const dim3 blk(32, 4);
  const uint32_t tiles = grid.x * grid.y * grid.z;
  const unsigned g = (unsigned)std::min<uint32_t>(tiles, 4u * (uint32_t)sm_count());
#define PW_CL_LAUNCH(ST, OPV)                                                                  \
  do {                                                                                        \
    if (odd) closure_step<ST, OPV, true><<<g, blk, 0, s>>>(p, frag, wall, grid.x, grid.y);    \
    else closure_step<ST, OPV, false><<<g, blk, 0, s>>>(p, frag, wall, grid.x, grid.y);       \
  } while (0)
  if (op == pw::OP_REG) {
    if (storage == pw::STORE_F16) PW_CL_LAUNCH(pw::STORE_F16, pw::OP_REG);
    else if (storage == pw::STORE_BF16) PW_CL_LAUNCH(pw::STORE_BF16, pw::OP_REG);
    else PW_CL_LAUNCH(pw::STORE_F32, pw::OP_REG);
  } else {
    if (storage == pw::STORE_F16) PW_CL_LAUNCH(pw::STORE_F16, pw::OP_TRT);
    else if (storage == pw::STORE_BF16) PW_CL_LAUNCH(pw::STORE_BF16, pw::OP_TRT);
    else PW_CL_LAUNCH(pw::STORE_F32, pw::OP_TRT);
  }
#undef PW_CL_LAUNCH
}

template <int ST, int OP, bool ODD>
static void closure_pairs_step(const StepParams &p, const uint32_t *frag, const uint8_t *wall, const uint32_t *list,
                               uint32_t count, cudaStream_t s, cudaStream_t t) {
  // the grid is the blocks that fit at once: the launch bound's count per SM
  // (registers; 20 KB of shared memory and 64 TMEM columns a block leave room
  // for more).  No occupancy query: the first step may run under stream capture.
  const int blocks_per_sm = PW_CLOSURE_PAIR_BLOCKS;
  // the floor layer and the wall-link cells beside the plain cells
  if constexpr (ST != pw::STORE_F32) {
    if (p.floor_rows && p.ny >= 3u) {
      const dim3 grid((p.nx + 2 * pwclosure::BX - 1) / (2 * pwclosure::BX), (p.ny - 2u + pwclosure::BY - 1u) / pwclosure::BY);
      pwclosure::aa_step_floor<ST, OP, true, ODD><<<grid, dim3(pwclosure::BX, pwclosure::BY), 0, t>>>(p);
    }
  }
  if (count)
    pwclosure::aa_step_edges<ST, OP, true, ODD>
        <<<(count + pwclosure::NTHREADS - 1) / pwclosure::NTHREADS, pwclosure::NTHREADS, 0, t>>>(p, list, count);
  const uint32_t runs = (p.nx + 63u) / 64u, row_blocks = (p.ny + 3u) / 4u;
  const uint32_t tiles = runs * row_blocks * p.nz;
  const unsigned g = (unsigned)std::min<uint32_t>(tiles, (uint32_t)blocks_per_sm * (uint32_t)sm_count());
  closure_pairs<ST, OP, ODD><<<g, dim3(32, 4), 0, s>>>(p, frag, wall, runs, row_blocks);
}

void launch_closure_pairs(const StepParams &p, int storage, int op, bool odd, const uint32_t *frag,
                          const uint8_t *wall, const uint32_t *list, uint32_t count, cudaStream_t s,
                          const pwfast::SideStream *side) {
  cudaStream_t t = side ? side->stream : s;
  if (side) {
    cudaEventRecord(side->fork, s);
    cudaStreamWaitEvent(t, side->fork, 0);
  }
#define PW_CLP(ST, OPV)                                                             \
  do {                                                                              \
    if (odd) closure_pairs_step<ST, OPV, true>(p, frag, wall, list, count, s, t);   \
    else closure_pairs_step<ST, OPV, false>(p, frag, wall, list, count, s, t);      \
  } while (0)
  if (op == pw::OP_REG) {
    if (storage == pw::STORE_F16) PW_CLP(pw::STORE_F16, pw::OP_REG);
    else if (storage == pw::STORE_BF16) PW_CLP(pw::STORE_BF16, pw::OP_REG);
    else PW_CLP(pw::STORE_F32, pw::OP_REG);
  } else {
    if (storage == pw::STORE_F16) PW_CLP(pw::STORE_F16, pw::OP_TRT);
    else if (storage == pw::STORE_BF16) PW_CLP(pw::STORE_BF16, pw::OP_TRT);
    else PW_CLP(pw::STORE_F32, pw::OP_TRT);
  }
#undef PW_CLP
  if (side) {
    cudaEventRecord(side->join, t);
    cudaStreamWaitEvent(s, side->join, 0);
  }
}

int wall_distance_of(const uint32_t *flags, uint32_t nx, uint32_t ny, uint32_t nz, uint8_t *out, cudaStream_t s) {
  const size_t cells = (size_t)nx * ny * nz;
  uint8_t *tmp = nullptr;
  PW_TRY(cudaMalloc(&tmp, cells));
  dist_init<<<(unsigned)((cells + 255) / 256), 256, 0, s>>>(flags, cells, out);
  int rc = wall_distance(out, tmp, nx, ny, nz, s);
  cudaStreamSynchronize(s);
  cudaFree(tmp);
  return rc;
}

const uint32_t *fragments(const pw_closure *c) { return c->frag; }
}  // namespace pwclosure_host

extern "C" {

int pw_closure_create(uint64_t seed, pw_closure **out) {
  if (!out) { set_error("NULL argument"); return PW_ERR_INVALID; }
  *out = nullptr;
  pw_closure *c = new pw_closure();
  cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&c->w, kParams * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&c->m, kParams * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&c->v, kParams * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&c->grad, (kParams + 1) * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&c->loss, sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&c->frag, 32 * kFragWords * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMalloc(&c->step, sizeof(uint32_t));
  if (e != cudaSuccess) {
    int rc = cuda_status(e, "pw_closure_create");
    pw_closure_destroy(c);
    return rc;
  }
  // Glorot-uniform hidden layers (seeded), zero biases, zero output layer: the
  // untrained network outputs c = 0, plain Smagorinsky.
  std::vector<float> w(kParams, 0.0f);
  uint64_t state = seed;
  auto uniform = [&]() {
    state += 0x9E3779B97F4A7C15ull;
    uint64_t z = state;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
  };
  const double a1 = std::sqrt(6.0 / (kIn + kHidden)), a2 = std::sqrt(6.0 / (2 * kHidden));
  for (int k = 0; k < kHidden * kIn; k++) w[kW1 + k] = (float)(a1 * uniform());
  for (int k = 0; k < kHidden * kHidden; k++) w[kW2 + k] = (float)(a2 * uniform());
  e = cudaMemcpy(c->w, w.data(), kParams * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(c->m, 0, kParams * sizeof(float));
  if (e == cudaSuccess) e = cudaMemset(c->v, 0, kParams * sizeof(float));
  if (e == cudaSuccess) e = cudaMemset(c->step, 0, sizeof(uint32_t));
  if (e != cudaSuccess) {
    int rc = cuda_status(e, "pw_closure_create");
    pw_closure_destroy(c);
    return rc;
  }
  int rc = refresh_fragments(c);
  if (rc == PW_OK) rc = cudaStreamSynchronize(c->stream) == cudaSuccess ? PW_OK : PW_ERR_CUDA;
  if (rc != PW_OK) { pw_closure_destroy(c); return rc; }
  *out = c;
  return PW_OK;
}

void pw_closure_destroy(pw_closure *c) {
  if (!c) return;
  if (c->stream) cudaStreamSynchronize(c->stream);
  cudaFree(c->w); cudaFree(c->m); cudaFree(c->v); cudaFree(c->grad); cudaFree(c->loss);
  cudaFree(c->frag); cudaFree(c->step); cudaFree(c->partial); cudaFree(c->X); cudaFree(c->Y);
  if (c->stream) cudaStreamDestroy(c->stream);
  cudaGetLastError();
  delete c;
}

int pw_closure_get_params(pw_closure *c, float *out) {
  if (!c || !out) { set_error("NULL argument"); return PW_ERR_INVALID; }
  PW_TRY(cudaMemcpyAsync(out, c->w, kParams * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  PW_TRY(cudaStreamSynchronize(c->stream));
  return PW_OK;
}

int pw_closure_set_params(pw_closure *c, const float *in) {
  if (!c || !in) { set_error("NULL argument"); return PW_ERR_INVALID; }
  for (int k = 0; k < kParams; k++)
    if (!std::isfinite(in[k])) { set_error("Closure parameters must be finite."); return PW_ERR_INVALID; }
  PW_TRY(cudaMemcpyAsync(c->w, in, kParams * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  PW_TRY(cudaMemsetAsync(c->m, 0, kParams * sizeof(float), c->stream));
  PW_TRY(cudaMemsetAsync(c->v, 0, kParams * sizeof(float), c->stream));
  PW_TRY(cudaMemsetAsync(c->step, 0, sizeof(uint32_t), c->stream));
  int rc = refresh_fragments(c);
  if (rc != PW_OK) return rc;
  PW_TRY(cudaStreamSynchronize(c->stream));
  return PW_OK;
}

int pw_closure_eval(pw_closure *c, const float *x, uint32_t count, float *out) {
  if (!c || (!x && count) || (!out && count)) { set_error("NULL argument"); return PW_ERR_INVALID; }
  if (!count) return PW_OK;
  float *dx = nullptr, *dy = nullptr;
  uint32_t *dstatus = nullptr, status = 0;
  PW_TRY(cudaMalloc(&dx, (size_t)count * kIn * sizeof(float)));
  cudaError_t e = cudaMalloc(&dy, (size_t)count * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&dstatus, sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMemsetAsync(dstatus, 0, sizeof(uint32_t), c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dx, x, (size_t)count * kIn * sizeof(float), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) {
    eval_kernel<<<(count + 127) / 128, 128, 0, c->stream>>>(c->frag, dx, count, dy, dstatus);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, dy, (size_t)count * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&status, dstatus, sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  cudaFree(dx);
  cudaFree(dy);
  cudaFree(dstatus);
  if (e != cudaSuccess) return cuda_status(e, "pw_closure_eval");
  if (status) {
    set_error("pw_closure_eval: a tensor-core layer did not complete in time");
    return PW_ERR_TIMEOUT;
  }
  return PW_OK;
}

int pw_closure_gradients(pw_closure *c, const float *x, const float *y, uint32_t count, float *grad, float *loss) {
  if (!c || !x || !y || !grad || count == 0) { set_error("NULL argument or no samples"); return PW_ERR_INVALID; }
  float *dx = nullptr, *dy = nullptr;
  uint32_t *idx = nullptr;
  const uint32_t blocks = (count + kTrainThreads - 1) / kTrainThreads;
  int rc = ensure_partials(c, blocks);
  if (rc != PW_OK) return rc;
  PW_TRY(cudaFuncSetAttribute(train_block, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)train_smem()));
  cudaError_t e = cudaMalloc(&dx, (size_t)count * kIn * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&dy, (size_t)count * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&idx, (size_t)count * sizeof(uint32_t));
  std::vector<uint32_t> seq(count);
  for (uint32_t i = 0; i < count; i++) seq[i] = i;
  if (e == cudaSuccess) e = cudaMemcpyAsync(dx, x, (size_t)count * kIn * sizeof(float), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dy, y, (size_t)count * sizeof(float), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(idx, seq.data(), (size_t)count * sizeof(uint32_t), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) {
    train_block<<<blocks, kTrainThreads, train_smem(), c->stream>>>(c->w, dx, dy, count, count, 0, c->step, idx,
                                                                    c->partial);
    train_reduce<<<(kParams + 1 + 255) / 256, 256, 0, c->stream>>>(c->partial, blocks, c->grad);
    e = cudaGetLastError();
  }
  std::vector<float> h(kParams + 1);
  if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), c->grad, (kParams + 1) * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  cudaFree(dx); cudaFree(dy); cudaFree(idx);
  if (e != cudaSuccess) return cuda_status(e, "pw_closure_gradients");
  std::copy(h.begin(), h.begin() + kParams, grad);
  if (loss) *loss = h[kParams] / (float)count;
  return PW_OK;
}

int pw_closure_dataset_clear(pw_closure *c) {
  if (!c) { set_error("NULL argument"); return PW_ERR_INVALID; }
  c->n = 0;
  return PW_OK;
}

int pw_closure_dataset_reserve(pw_closure *c, uint64_t capacity) {
  if (!c) { set_error("NULL argument"); return PW_ERR_INVALID; }
  if (capacity <= c->cap) return PW_OK;
  float *nx = nullptr, *ny = nullptr;
  PW_TRY(cudaMalloc(&nx, capacity * kIn * sizeof(float)));
  cudaError_t e = cudaMalloc(&ny, capacity * sizeof(float));
  if (e == cudaSuccess && c->n) e = cudaMemcpy(nx, c->X, c->n * kIn * sizeof(float), cudaMemcpyDeviceToDevice);
  if (e == cudaSuccess && c->n) e = cudaMemcpy(ny, c->Y, c->n * sizeof(float), cudaMemcpyDeviceToDevice);
  if (e != cudaSuccess) { cudaFree(nx); cudaFree(ny); return cuda_status(e, "pw_closure_dataset_reserve"); }
  cudaFree(c->X); cudaFree(c->Y);
  c->X = nx; c->Y = ny; c->cap = capacity;
  return PW_OK;
}

int pw_closure_dataset_write(pw_closure *c, const float *x, const float *y, uint64_t count) {
  if (!c || (count && (!x || !y))) { set_error("NULL argument"); return PW_ERR_INVALID; }
  int rc = pw_closure_dataset_reserve(c, count ? count : 1);
  if (rc != PW_OK) return rc;
  if (count) {
    PW_TRY(cudaMemcpy(c->X, x, count * kIn * sizeof(float), cudaMemcpyHostToDevice));
    PW_TRY(cudaMemcpy(c->Y, y, count * sizeof(float), cudaMemcpyHostToDevice));
  }
  c->n = count;
  return PW_OK;
}

int pw_closure_dataset_size(const pw_closure *c, uint64_t *n) {
  if (!c || !n) { set_error("NULL argument"); return PW_ERR_INVALID; }
  *n = c->n;
  return PW_OK;
}

int pw_closure_dataset_read(pw_closure *c, uint64_t first, uint64_t count, float *x, float *y) {
  if (!c || (count && (!x || !y))) { set_error("NULL argument"); return PW_ERR_INVALID; }
  if (first + count > c->n) { set_error("Dataset range beyond its %llu samples.", (unsigned long long)c->n); return PW_ERR_INVALID; }
  if (!count) return PW_OK;
  PW_TRY(cudaMemcpy(x, c->X + first * kIn, count * kIn * sizeof(float), cudaMemcpyDeviceToHost));
  PW_TRY(cudaMemcpy(y, c->Y + first, count * sizeof(float), cudaMemcpyDeviceToHost));
  return PW_OK;
}

// Append the samples of a fine domain's latest macros (the last step must have
// written them) at the given coarse molecular viscosity.
int pw_closure_dataset_add(pw_closure *c, pw_domain *fine, double nu0_coarse, uint64_t *added) {
  if (!c || !fine) { set_error("NULL argument"); return PW_ERR_INVALID; }
  uint32_t nx, ny, nz;
  domain_dims(fine, &nx, &ny, &nz);
  if (nx % 2 || ny % 2 || nz % 2 || nx < 10 || ny < 4 || nz < 4) {
    set_error("The fine grid must have even dimensions of at least 10 x 4 x 4.");
    return PW_ERR_INVALID;
  }
  if (!(nu0_coarse > 0.0) || !std::isfinite(nu0_coarse)) { set_error("The coarse viscosity must be positive."); return PW_ERR_INVALID; }
  void *macros = nullptr, *flags = nullptr, *stream = nullptr;
  int rc = pw_domain_buffers(fine, &macros, &flags, &stream);
  if (rc != PW_OK) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  const uint32_t cx = nx / 2, cy = ny / 2, cz = nz / 2;
  const size_t nc = (size_t)cx * cy * cz;
  float *co = nullptr;
  uint8_t *solid = nullptr, *dist = nullptr, *tmp = nullptr;
  uint32_t *counts = nullptr;
  const uint32_t nblk = (uint32_t)((nc + kScanBlock - 1) / kScanBlock);
  cudaError_t e = cudaMalloc(&co, 10 * nc * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&solid, nc);
  if (e == cudaSuccess) e = cudaMalloc(&dist, nc);
  if (e == cudaSuccess) e = cudaMalloc(&tmp, nc);
  if (e == cudaSuccess) e = cudaMalloc(&counts, (nblk + 1) * sizeof(uint32_t));
  uint32_t total = 0;
  float u_in = 0.0f;
  if (e == cudaSuccess) {
    pw::StepParams p = member_params(fine, 2, 0);
    u_in = p.u_in;
    coarsen_kernel<<<(unsigned)((nc + 255) / 256), 256, 0, s>>>((const float4 *)macros, (const uint32_t *)flags, nx, ny,
                                                                 nz, co, solid);
    dist_from_solid<<<(unsigned)((nc + 255) / 256), 256, 0, s>>>(solid, nc, dist);
    rc = wall_distance(dist, tmp, cx, cy, cz, s);
    sample_count<<<nblk, kScanBlock, 0, s>>>(co, dist, cx, cy, cz, (float)nu0_coarse, u_in, counts);
    scan_counts<<<1, kScanBlock, 0, s>>>(counts, nblk, counts + nblk);
    e = cudaMemcpyAsync(&total, counts + nblk, 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  if (e == cudaSuccess && rc == PW_OK) {
    const uint64_t need = c->n + total;
    if (need > c->cap) rc = pw_closure_dataset_reserve(c, std::max<uint64_t>(need, c->cap * 2));
  }
  if (e == cudaSuccess && rc == PW_OK) {
    sample_write<<<nblk, kScanBlock, 0, s>>>(co, dist, cx, cy, cz, (float)nu0_coarse, u_in, counts, c->n, c->cap,
                                             c->X, c->Y);
    e = cudaStreamSynchronize(s);
  }
  cudaFree(co); cudaFree(solid); cudaFree(dist); cudaFree(tmp); cudaFree(counts);
  if (e != cudaSuccess) return cuda_status(e, "pw_closure_dataset_add");
  if (rc != PW_OK) return rc;
  c->n += total;
  if (added) *added = total;
  return PW_OK;
}

// Adam over `steps` minibatches of `batch` samples drawn by a seeded hash from
// the dataset; first and last batch losses (mean squared error of c).
int pw_closure_train(pw_closure *c, uint32_t steps, uint32_t batch, float lr, uint64_t seed, float *loss_first,
                     float *loss_last) {
  if (!c || steps == 0 || batch == 0 || !(lr > 0.0f)) { set_error("Training needs steps, a batch and a positive rate."); return PW_ERR_INVALID; }
  if (c->n == 0) { set_error("The closure dataset is empty."); return PW_ERR_INVALID; }
  const uint32_t blocks = (batch + kTrainThreads - 1) / kTrainThreads;
  int rc = ensure_partials(c, blocks);
  if (rc != PW_OK) return rc;
  PW_TRY(cudaFuncSetAttribute(train_block, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)train_smem()));
  auto one = [&](cudaStream_t s) {
    train_block<<<blocks, kTrainThreads, train_smem(), s>>>(c->w, c->X, c->Y, c->n, batch, seed, c->step, nullptr,
                                                            c->partial);
    train_reduce<<<(kParams + 1 + 255) / 256, 256, 0, s>>>(c->partial, blocks, c->grad);
    train_adam<<<1, 1024, 0, s>>>(c->w, c->m, c->v, c->grad, c->step, lr, batch, c->loss);
  };
  one(c->stream);
  PW_TRY(cudaGetLastError());
  if (loss_first) PW_TRY(cudaMemcpyAsync(loss_first, c->loss, sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  // the rest as replays of a captured 100-step graph
  uint32_t done = 1;
  const uint32_t chunk = 100;
  cudaGraphExec_t exec = nullptr;
  if (steps - done >= chunk) {
    cudaStream_t cap;
    PW_TRY(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    cudaGraph_t graph = nullptr;
    if (cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      for (uint32_t k = 0; k < chunk; k++) one(cap);
      if (cudaStreamEndCapture(cap, &graph) == cudaSuccess && graph) {
        if (cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) exec = nullptr;
        cudaGraphDestroy(graph);
      }
    }
    cudaStreamDestroy(cap);
    cudaGetLastError();
  }
  while (exec && steps - done >= chunk) {
    if (cudaGraphLaunch(exec, c->stream) != cudaSuccess) break;
    done += chunk;
  }
  if (exec) cudaGraphExecDestroy(exec);
  for (; done < steps; done++) one(c->stream);
  PW_TRY(cudaGetLastError());
  if (loss_last) PW_TRY(cudaMemcpyAsync(loss_last, c->loss, sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  rc = refresh_fragments(c);
  if (rc != PW_OK) return rc;
  PW_TRY(cudaStreamSynchronize(c->stream));
  return PW_OK;
}

}  // extern "C"
