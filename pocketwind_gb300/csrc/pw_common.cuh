// Shared device definitions of the D3Q19 solver: lattice tables, storage codecs,
// kernel parameter blocks.  Lattice order and weights follow
// src/lbm/lattice.ts:1-52 and src/lbm/shaders/common.wgsl:1-22 of the reference.
#pragma once
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include <stdint.h>

namespace pw {

enum : uint32_t { FLUID = 0, SOLID = 1, SUPPORT = 2, FLOOR = 3, EQ = 4 };
constexpr uint32_t NO_Q = 0xffffffffu;  // cell without packed link fractions
// Element index into the population array: plane * stride + cell, which passes
// 2^32 on domains above 226 M cells (cell indices themselves stay below 2^32).
typedef uint64_t pidx;
enum : int { STORE_F32 = 0, STORE_F16 = 1, STORE_BF16 = 2 };
enum : int { OP_TRT = 0, OP_REG = 1 };

// Direction i: velocity (CX, CY, CZ); opposite pairs are (1,2), (3,4), ...
__host__ __device__ constexpr int cx_of(int i) {
  return i == 1 || i == 7 || i == 9 || i == 13 || i == 15 ? 1
         : (i == 2 || i == 8 || i == 10 || i == 14 || i == 16 ? -1 : 0);
}
__host__ __device__ constexpr int cy_of(int i) {
  return i == 3 || i == 7 || i == 11 || i == 14 || i == 17 ? 1
         : (i == 4 || i == 8 || i == 12 || i == 13 || i == 18 ? -1 : 0);
}
__host__ __device__ constexpr int cz_of(int i) {
  return i == 5 || i == 9 || i == 11 || i == 16 || i == 18 ? 1
         : (i == 6 || i == 10 || i == 12 || i == 15 || i == 17 ? -1 : 0);
}
__host__ __device__ constexpr int opp_of(int i) { return i == 0 ? 0 : ((i & 1) ? i + 1 : i - 1); }
__host__ __device__ constexpr int dir_of(int cx, int cy, int cz, int k = 0) {
  return k == 19 ? -1 : (cx_of(k) == cx && cy_of(k) == cy && cz_of(k) == cz ? k : dir_of(cx, cy, cz, k + 1));
}
// Direction i with its y (or z, or both) velocity component reversed: the
// specular reflection at a free-slip face.
__host__ __device__ constexpr int mirror_y(int i) { return dir_of(cx_of(i), -cy_of(i), cz_of(i)); }
__host__ __device__ constexpr int mirror_z(int i) { return dir_of(cx_of(i), cy_of(i), -cz_of(i)); }
__host__ __device__ constexpr int mirror_yz(int i) { return dir_of(cx_of(i), -cy_of(i), -cz_of(i)); }
// binary32 weights, each 1/3, 1/18 or 1/36 rounded once (WGSL const-expression).
__host__ __device__ constexpr float w_of(int i) {
  return i == 0 ? 0.333333343267440796f : (i < 7 ? 0.0555555559694766998f : 0.0277777779847383499f);
}

__device__ __forceinline__ bool is_wall_kind(uint32_t k) { return k >= SOLID && k <= FLOOR; }

// The packed flag of a fluid cell whose only wall links are the five whose
// pull sources lie at z - 1 (c_z = +1): the first fluid layer over a flat floor.
__host__ __device__ constexpr uint32_t floor_links(int i = 1) {
  return i == 19 ? 0u : ((cz_of(i) == 1 ? 1u << (3 + i) : 0u) | floor_links(i + 1));
}
constexpr uint32_t kFloorFlag = FLUID | floor_links();
// A floor cell of a domain with floor rows: the z = 1 layer over an all-FLOOR
// z = 0 plane, off the periodic y seams (those rows belong to the seam kernel
// on odd steps).
__host__ __device__ __forceinline__ bool is_floor_cell(uint32_t flag, uint32_t y, uint32_t z, uint32_t ny) {
  return z == 1u && y >= 1u && y + 2u <= ny && flag == kFloorFlag;
}

// Positions whose x-neighbours are reached without the periodic wrap in x; a
// non-special cell there is a plain cell of the fast step (the y and z seams
// are handled in the plain kernel).
__host__ __device__ __forceinline__ bool is_plain_position(uint32_t x, uint32_t nx) {
  return x >= 1u && x + 2u <= nx;
}

// ------------------------------------------------------------ storage codecs
// lowbias32 dithering of the discarded bits (src/lbm/shaders/prelude-f16.wgsl:7-22).
__device__ __forceinline__ uint32_t lowbias32(uint32_t bits, uint32_t i, uint32_t n) {
  uint32_t r = bits ^ (n * 0x9e3779b9u) ^ (i * 0x85ebca6bu);
  r = (r ^ (r >> 16)) * 0x7feb352du;
  r = (r ^ (r >> 15)) * 0x846ca68bu;
  r ^= r >> 16;
  return r;
}

// Odd per-direction multipliers of the fast build's dither hash.
__host__ __device__ constexpr uint32_t dither_mul(int i) { return (0x9e3779b1u ^ ((uint32_t)i * 0x85ebca6bu)) | 1u; }

// Random bits for encode_pair of two codes of direction i: for each value the
// upper half of its own hash bits * dither_mul(i) + nk (nk = n * 0x9e3779b9
// of its cell), so a code's rounding depends on its own value, cell and
// direction only, never on its partner's.  One byte permute puts h_lo[31:16]
// in the low half and h_hi[31:16] in the high half: bfloat16 adds all 16 bits
// of each half, f16 the 13 bits 12:0 and 28:16, that is hash bits 28:16 (the
// one-code encode_fast takes bits 31:19 of the same hash: the same rounding
// probabilities, another realization).
template <int ST>
__device__ __forceinline__ uint32_t pair_dither(float hi, float lo, uint32_t mj, uint32_t nk_hi, uint32_t nk_lo) {
  const uint32_t h_hi = __float_as_uint(hi) * mj + nk_hi;
  const uint32_t h_lo = __float_as_uint(lo) * mj + nk_lo;
  return __byte_perm(h_lo, h_hi, 0x7632u);
}

template <int S> struct Store;

template <> struct Store<STORE_F32> {
  using T = float;
  static constexpr float kScale = 1.0f;
  static constexpr float kInvScale = 1.0f;
  __device__ __forceinline__ static float decode(float v) { return v; }
  __device__ __forceinline__ static float raw(float v) { return v; }
  __device__ __forceinline__ static float encode(float v, uint32_t, uint32_t) { return v; }
  __device__ __forceinline__ static float encode_fast(float v, uint32_t, uint32_t) { return v; }
};

template <> struct Store<STORE_F16> {
  using T = __half;
  static constexpr float kScale = 32768.0f;
  static constexpr float kInvScale = 1.0f / 32768.0f;
  // Division by a power of two is exact, so this equals f32(h) / 2^15.
  __device__ __forceinline__ static float decode(__half h) { return __half2float(h) * kInvScale; }
  __device__ __forceinline__ static float raw(__half h) { return __half2float(h); }
  // The fast build's rounding of a value already multiplied by 2^15: the same
  // unbiased dithering of the 13 discarded bits (round up with probability
  // discarded / 2^13, as "add a dither in [0, 2^13) and truncate"), with the
  // dither taken from a one-multiply hash of (value bits, cell, direction):
  // the top 13 bits of bits * mj + nk, where mj = dither_mul(i) and
  // nk = n * 0x9e3779b9.  The truncation is the conversion's round-toward-zero.
  // Below 2^-14 (stored units) the dither acts on the subnormal step instead,
  // and values beyond the f16 range saturate at 65504 rather than reaching
  // infinity (a population of 2, far outside the density guard's bounds).  The
  // caller passes NaN as the quiet NaN 0x7fc00000, which this keeps.
  __device__ __forceinline__ static __half encode_fast(float scaled, uint32_t mj, uint32_t nk) {
    const uint32_t bits = __float_as_uint(scaled);
    const uint32_t r = bits * mj + nk;
    return __float2half_rz(__uint_as_float(bits + (r >> 19)));
  }
  // Two codes at once by the hardware's stochastic conversion (cvt.rs, sm_100
  // family): it adds rbits[28:16] to the 13 bits that hi discards and rbits[12:0]
  // to those of lo, then truncates: the rule of encode_fast with the dither
  // supplied.  .satfinite keeps overflow at 65504 and NaN a NaN.  Returns
  // code(hi) << 16 | code(lo).
  __device__ __forceinline__ static uint32_t encode_pair(float hi, float lo, uint32_t rbits) {
    uint32_t d;
    asm("cvt.rs.satfinite.f16x2.f32 %0, %1, %2, %3;" : "=r"(d) : "f"(hi), "f"(lo), "r"(rbits));
    return d;
  }
  __device__ __forceinline__ static __half encode(float value, uint32_t i, uint32_t n) {
    float scaled = value * kScale;
    // CUDA's NaN (0x7fffffff) would carry into the sign below and become -0; the
    // reference's GPUs produce 0x7fc00000, which stays NaN.  Keep NaN a NaN.
    if (scaled != scaled) return __ushort_as_half((unsigned short)0x7e00u);
    uint32_t bits = __float_as_uint(scaled);
    uint32_t magnitude = bits & 0x7fffffffu;
    if (magnitude < 0x38800000u) return __float2half_rn(scaled);
    uint32_t random = lowbias32(bits, i, n);
    uint32_t increment = ((random & 0x1fffu) < (magnitude & 0x1fffu)) ? 0x2000u : 0u;
    uint32_t rounded = (magnitude & 0xffffe000u) + increment;
    return __float2half_rn(__uint_as_float((bits & 0x80000000u) | rounded));
  }
};

template <> struct Store<STORE_BF16> {
  using T = __nv_bfloat16;
  static constexpr float kScale = 1.0f;
  static constexpr float kInvScale = 1.0f;
  __device__ __forceinline__ static float decode(__nv_bfloat16 h) { return __bfloat162float(h); }
  __device__ __forceinline__ static float raw(__nv_bfloat16 h) { return __bfloat162float(h); }
  // The fast build's rounding: encode_fast of the f16 codec on the 16 bits that
  // bfloat16 discards.
  __device__ __forceinline__ static __nv_bfloat16 encode_fast(float value, uint32_t mj, uint32_t nk) {
    const uint32_t bits = __float_as_uint(value);
    const uint32_t r = bits * mj + nk;
    return __float2bfloat16_rz(__uint_as_float(bits + (r >> 16)));
  }
  // encode_pair of the f16 codec for bfloat16: rbits[31:16] and rbits[15:0] are
  // added to the 16 discarded bits of hi and lo.
  __device__ __forceinline__ static uint32_t encode_pair(float hi, float lo, uint32_t rbits) {
    uint32_t d;
    asm("cvt.rs.bf16x2.f32 %0, %1, %2, %3;" : "=r"(d) : "f"(hi), "f"(lo), "r"(rbits));
    return d;
  }
  // The f16 dithering rule applied to the 16 bits bfloat16 discards.
  __device__ __forceinline__ static __nv_bfloat16 encode(float value, uint32_t i, uint32_t n) {
    uint32_t bits = __float_as_uint(value);
    uint32_t magnitude = bits & 0x7fffffffu;
    if (magnitude < 0x00800000u || magnitude >= 0x7f800000u) return __float2bfloat16_rn(value);
    uint32_t random = lowbias32(bits, i, n);
    uint32_t increment = ((random & 0xffffu) < (magnitude & 0xffffu)) ? 0x10000u : 0u;
    uint32_t rounded = (magnitude & 0xffff0000u) + increment;
    return __ushort_as_bfloat16((unsigned short)(((bits & 0x80000000u) | rounded) >> 16));
  }
};

// Step kernels run blocks of one warp along x by kBlockY rows.
constexpr int kBlockX = 32;
constexpr int kBlockY = 4;

// ------------------------------------------------------------ parameter blocks
struct StepParams {
  void *f;                 // 19 * stride population codes (AA layout)
  float4 *macros;          // (rho, ux, uy, uz) per cell
  const float4 *plane_in;  // outlet upstream velocity written by the previous step
  float4 *plane_out;       // this step's upstream velocity
  const uint32_t *flags;   // packed flags (kind | wall bits << 3)
  const uint32_t *special; // bit per cell: anything but plain fluid without wall links
  double *partials;        // 3 doubles per block: momentum exchange of this step's output
  uint32_t *status;        // bit 0: density guard tripped on a macro step
  uint32_t nx, ny, nz;
  uint32_t stride;         // elements between direction planes
  float u_in;              // inlet speed of this step
  float nu, cs_term, lambda;
  float tau0, omega_plus, omega_minus;  // binary32 constants of the LES-free operator
  int write_macro;
  uint32_t slip;           // free-slip faces: bit 0 the y faces, bit 1 the z faces (0: periodic)
  // Plain cells (no periodic wrap in reach): direction i is loaded from element
  // n + ld[i] and stored to element n + st[i] of f, offsets for this step's parity.
  int64_t ld[19];
  int64_t st[19];
  // The same offsets in bytes (element offsets times the element size), added
  // to a per-thread base pointer by the cell-pair kernels.
  int64_t ldb[19];
  int64_t stb[19];
  // The other parity's load offsets in bytes: a wall link i reads the slot
  // that nobody rewrites during the step, which is where the opposite parity
  // pulls from (odd steps: slot i of n; even steps: slot opp(i) of n - c_i).
  int64_t wb[19];
  // Floor rows: the floor kernel updates the cells of the z = 1 rows off the
  // y seams whose only wall links are the five floor links (is_floor_cell),
  // and the edge kernel leaves them out.
  uint32_t floor_rows;
  float wall_c, wall_e;    // Werner-Wengle: (nu / (1/2))^(1/7) / 8.3 and 1 / (1 + 1/7)
  // Interpolated walls (walls.wgsl:6-21); null qoff means halfway bounce-back.
  // qoff[n]: index of cell n's first wall-link fraction (PW_NO_Q without); q: the
  // fractions in link-rank order; hist: per link, the cell's own post-collision
  // code in the link's direction from the latest step (the AA pattern overwrites
  // that population in place, so the cell keeps a copy).  With interpolated walls
  // a step's force partials hold the momentum exchange of the state it read.
  const uint32_t *qoff;
  const float *q;
  void *hist;
};

}  // namespace pw
