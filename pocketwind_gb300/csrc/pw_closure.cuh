// The learned subgrid closure: a 9 -> 32 -> 32 -> 1 network whose output c
// scales the Smagorinsky eddy viscosity, nu_t = nu_smag * max(0, 1 + c), so
// c = 0 is plain Smagorinsky.  No counterpart in the reference.
//
// Parameters, packed as floats in this order (kParams in all):
//   W1[32][9]  b1[32]  W2[32][32]  b2[32]  W3[32]  b3
// The forward pass rounds inputs, weights and hidden activations to bfloat16
// and accumulates in binary32, with the hardware tanh approximation; training
// and the fused inference use the same rounding.
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>
#include <string.h>

namespace pwcl {

constexpr int kIn = 9, kHidden = 32;
constexpr int kW1 = 0, kB1 = kW1 + kHidden * kIn, kW2 = kB1 + kHidden, kB2 = kW2 + kHidden * kHidden,
              kW3 = kB2 + kHidden, kB3 = kW3 + kHidden, kParams = kB3 + 1;  // 1409
constexpr float kWallCap = 8.0f;

__device__ __forceinline__ float tanh_fast(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__host__ __device__ __forceinline__ float bf16_round(float x) {
#ifdef __CUDA_ARCH__
  return __bfloat162float(__float2bfloat16_rn(x));
#else
  uint32_t u;
  memcpy(&u, &x, 4);
  if ((u & 0x7fffffffu) > 0x7f800000u) return x;
  u = (u + 0x7fffu + ((u >> 16) & 1u)) & 0xffff0000u;
  float y;
  memcpy(&y, &u, 4);
  return y;
#endif
}

// Strain rate S (xx, yy, zz, xy, xz, yz), density, velocity, wall distance
// (cells), molecular viscosity nu0 and the Smagorinsky eddy viscosity nu_s of
// the cell, inlet speed u_in -> the nine inputs.  The same function serves the
// training data (S from finite differences of filtered fields) and the fused
// inference (S from the non-equilibrium stress).
__host__ __device__ __forceinline__ void features(const float s[6], float rho, float ux, float uy, float uz,
                                                  float wall, float nu0, float nu_s, float u_in, float x[kIn]) {
  const float ss = s[0] * s[0] + s[1] * s[1] + s[2] * s[2] + 2.0f * (s[3] * s[3] + s[4] * s[4] + s[5] * s[5]);
  const float off = 2.0f * (s[3] * s[3] + s[4] * s[4] + s[5] * s[5]);
  // tr(S^3) of the symmetric S [[a, d, e], [d, b, f], [e, f, c]]
  const float t3 = s[0] * s[0] * s[0] + s[1] * s[1] * s[1] + s[2] * s[2] * s[2] +
                   3.0f * ((s[0] + s[1]) * s[3] * s[3] + (s[0] + s[2]) * s[4] * s[4] + (s[1] + s[2]) * s[5] * s[5]) +
                   6.0f * s[3] * s[4] * s[5];
  const float mag = sqrtf(2.0f * ss);
  const float inv_u = 1.0f / u_in;
  const float uu = sqrtf(ux * ux + uy * uy + uz * uz);
  x[0] = 100.0f * mag;
  x[1] = t3 / (ss * sqrtf(ss) + 1e-30f);
  x[2] = off / (ss + 1e-30f);
  x[3] = uu * inv_u;
  x[4] = ux * inv_u;
  x[5] = 0.1f * (rho - 1.0f) * inv_u * inv_u;
  x[6] = fminf(wall, kWallCap) * (1.0f / kWallCap);
  x[7] = 10.0f * nu_s / nu0;
  x[8] = 200.0f * nu0;
}

// Scalar forward pass with the network's rounding (host oracle mirrors and
// small device uses); `w` holds kParams floats.
__device__ __forceinline__ float forward_scalar(const float *w, const float x[kIn]) {
  float xb[kIn], h1[kHidden];
#pragma unroll
  for (int k = 0; k < kIn; k++) xb[k] = bf16_round(x[k]);
#pragma unroll 4
  for (int j = 0; j < kHidden; j++) {
    float a = 0.0f;
#pragma unroll
    for (int k = 0; k < kIn; k++) a = fmaf(bf16_round(w[kW1 + j * kIn + k]), xb[k], a);
    h1[j] = bf16_round(tanh_fast(a + w[kB1 + j]));
  }
  float out = 0.0f;
#pragma unroll 4
  for (int j = 0; j < kHidden; j++) {
    float a = 0.0f;
#pragma unroll 8
    for (int k = 0; k < kHidden; k++) a = fmaf(bf16_round(w[kW2 + j * kHidden + k]), h1[k], a);
    const float h2 = bf16_round(tanh_fast(a + w[kB2 + j]));
    out = fmaf(bf16_round(w[kW3 + j]), h2, out);
  }
  return out + w[kB3];
}

}  // namespace pwcl
