// TMA-staged form of the fused AA stream-collide.
//
// Included after pw_lbm.cuh by both builds (PW_NS, PW_STRICT).  Same semantics and
// per-cell arithmetic as aa_step; only the data movement differs, so the strict
// build's tile kernel reproduces the binary32 restatement bit for bit like the
// one-cell-per-thread strict kernel does.  A block owns R whole x-rows (consecutive in y, then z).  For
// each of the 19 slots s it stages the R rows that its cells pull slot s from --
// the block's own rows on even steps, the rows shifted by (c_s.y, c_s.z) on odd
// steps -- with one bulk TMA copy per row (cp.async.bulk, completion counted on
// an mbarrier), so a block keeps 19 * R * nx * s bytes in flight without holding
// them in registers.  Whole rows make the periodic x shift an index wrap inside
// shared memory.  Each thread then updates one cell at a time in place (a cell
// writes exactly the shared elements it read), and the rows go back to HBM with
// bulk stores.  Different blocks stage disjoint (slot, row) pairs, so the
// in-place update stays race free.
//
// Wall cells are never updated, so their staged elements return unchanged; the
// boundary cells' redirected wall-link reads (pw_lbm.cuh) fetch slots that no
// block changes in that step straight from HBM.
//
// Every wait on the mbarrier is bounded: past the limit the block raises bit 1
// of the status word, skips its update and returns.
#include "pw_common.cuh"

namespace PW_NS {
using namespace pw;

constexpr int TILE_THREADS = NTHREADS;  // 128: the force-partial reduction's block size

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// global -> shared, counted on the mbarrier (size and both addresses 16-byte aligned)
__device__ __forceinline__ void bulk_load(void *dst_smem, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst_smem)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}
// shared -> global in a bulk group
__device__ __forceinline__ void bulk_store(void *dst, const void *src_smem, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_addr(src_smem)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Element offset of x = 0 of the row that slot s of tile row tr is staged from.
__device__ __forceinline__ uint32_t staged_row(const StepParams &p, int s, uint32_t row, bool odd) {
  uint32_t y = row % p.ny, z = row / p.ny;
  if (odd) {
    const int cy = cy_of(s), cz = cz_of(s);
    y = cy > 0 ? (y + 1 == p.ny ? 0 : y + 1) : (cy < 0 ? (y == 0 ? p.ny - 1 : y - 1) : y);
    z = cz > 0 ? (z + 1 == p.nz ? 0 : z + 1) : (cz < 0 ? (z == 0 ? p.nz - 1 : z - 1) : z);
  }
  return (uint32_t)s * p.stride + (y + p.ny * z) * p.nx;
}

// The LES wall cell (rare: boundary cells only) out of line, so the common path
// keeps its registers.
template <int OP>
__device__ __noinline__ void wall_cell_update(const StepParams &p, const float *g, uint32_t flag, float *post,
                                              float *m4) {
  float rho, vx, vy, vz;
  update_ref<OP, true>(p, g, flag, post, rho, vx, vy, vz);
  m4[0] = rho; m4[1] = vx; m4[2] = vy; m4[3] = vz;
}

template <int ST, int OP, bool LES, bool ODD>
__global__ void __launch_bounds__(TILE_THREADS, 4) aa_step_tile(StepParams p, uint32_t rows_per_tile) {
  using S = Store<ST>;
  using T = typename S::T;
  extern __shared__ __align__(128) unsigned char tile_smem[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ int timed_out;
  T *buf = reinterpret_cast<T *>(tile_smem);  // [19][R][nx]
  T *f = reinterpret_cast<T *>(p.f);
  const uint32_t nx = p.nx;
  const uint32_t rows = p.ny * p.nz;
  const uint32_t R0 = blockIdx.x * rows_per_tile;
  const uint32_t R = min(rows_per_tile, rows - R0);
  const uint32_t row_bytes = nx * (uint32_t)sizeof(T);
  const uint32_t copies = 19u * R;

  // ---------------------------------------------------------------- stage
  if (threadIdx.x == 0) {
    timed_out = 0;
    mbar_init(&bar, 1);
    mbar_fence_init();
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    if (threadIdx.x == 0) mbar_arrive_expect_tx(&bar, copies * row_bytes);
    __syncwarp();
    for (uint32_t k = threadIdx.x; k < copies; k += 32) {
      const int s = (int)(k / R);
      const uint32_t tr = k - (uint32_t)s * R;
      bulk_load(buf + ((size_t)s * rows_per_tile + tr) * nx, f + staged_row(p, s, R0 + tr, ODD), row_bytes, &bar);
    }
  }
  {
    // bounded wait: about two seconds at 2 GHz before the block gives up
    const long long t0 = clock64();
    bool done = false;
    while (!(done = mbar_try_wait(&bar, 0))) {
      if (clock64() - t0 > (4ll << 30)) break;
    }
    if (!done) atomicExch(&timed_out, 1);
  }
  __syncthreads();
  if (timed_out) {
    if (threadIdx.x == 0) atomicOr(p.status, 2u);
    // the copies may still land: give them another bounded wait before the shared memory is released
    const long long t0 = clock64();
    while (!mbar_try_wait(&bar, 0) && clock64() - t0 < (1ll << 30)) {
    }
    return;
  }

  // ---------------------------------------------------------------- update in place
  bool force_any = false;
  double fx = 0.0, fy = 0.0, fz = 0.0;
  const uint32_t tile_cells = R * nx;
  const uint32_t plane = nx * p.ny;
  for (uint32_t c = threadIdx.x; c < tile_cells; c += TILE_THREADS) {
    const uint32_t tr = c / nx;
    const uint32_t x = c - tr * nx;
    const uint32_t row = R0 + tr;
    const uint32_t y = row % p.ny, z = row / p.ny;
    const uint32_t n = x + nx * row;
    const bool special = (__ldg(&p.special[n >> 5]) >> (n & 31u)) & 1u;
    const uint32_t flag = special ? __ldg(&p.flags[n]) : 0u;
    const uint32_t kind = flag & 7u;
    if (is_wall_kind(kind)) continue;
    const uint32_t xm = x == 0 ? nx - 1 : x - 1;
    const uint32_t xp = x + 1 == nx ? 0 : x + 1;
    T *rowbuf = buf + (size_t)tr * nx;
    const size_t slot_pitch = (size_t)rows_per_tile * nx;
    // shared element of slot s for this cell: odd steps read/write it at x + c_s.x
    auto elem = [&](int s) -> T * {
      const uint32_t xs = ODD ? (cx_of(s) > 0 ? xp : (cx_of(s) < 0 ? xm : x)) : x;
      return rowbuf + (size_t)s * slot_pitch + xs;
    };
    float post[19];
    float rho = 1.0f, vx = 0.f, vy = 0.f, vz = 0.f;
    if (kind == EQ) {
      vx = p.u_in;
      if (x == nx - 1 && x > 0) {
        float4 u = p.plane_in[y + p.ny * z];
        vx = u.x; vy = u.y; vz = u.z;
      }
#pragma unroll
      for (int j = 0; j < 19; j++) post[j] = geq_ref(j, 0.0f, vx, vy, vz);
    } else {
      float g[19];
#pragma unroll
      for (int i = 0; i < 19; i++) {
        // odd: g_i from slot opp(i) at n - c_i = n + c_opp(i); even: slot i at n
        const int s = ODD ? opp_of(i) : i;
        g[i] = S::decode(*elem(s));
      }
      if (flag >> 3) {
#pragma unroll
        for (int i = 1; i < 19; i++) {
          if (!(flag & (1u << (3 + i)))) continue;
          uint32_t src;
          if (ODD) {
            src = (uint32_t)i * p.stride + n;
          } else {
            const uint32_t wx = cx_of(i) > 0 ? xm : (cx_of(i) < 0 ? xp : x);
            const uint32_t wy = cy_of(i) > 0 ? (y == 0 ? p.ny - 1 : y - 1) : (cy_of(i) < 0 ? (y + 1 == p.ny ? 0 : y + 1) : y);
            const uint32_t wz = cz_of(i) > 0 ? (z == 0 ? p.nz - 1 : z - 1) : (cz_of(i) < 0 ? (z + 1 == p.nz ? 0 : z + 1) : z);
            src = (uint32_t)opp_of(i) * p.stride + wx + nx * wy + plane * wz;
          }
          g[i] = S::decode(f[src]);
        }
      }
#if PW_STRICT
      update_ref<OP, LES>(p, g, flag, post, rho, vx, vy, vz);
#else
      if (LES && (flag >> 3) != 0u) {
        float m4[4];
        wall_cell_update<OP>(p, g, flag, post, m4);
        rho = m4[0]; vx = m4[1]; vy = m4[2]; vz = m4[3];
      } else {
        update_fast<OP, LES>(p, g, rho, vx, vy, vz);
#pragma unroll
        for (int j = 0; j < 19; j++) post[j] = g[j];
      }
#endif
      if (p.write_macro) {
        bool bad = !(rho >= 0.5f && rho <= 1.5f);
        if (bad) atomicOr(p.status, 1u);
      }
    }
    T code[19];
#pragma unroll
    for (int j = 0; j < 19; j++) {
      code[j] = S::encode(post[j], (uint32_t)j, n);
      // odd: P(j, n) to slot j at n + c_j; even: to slot opp(j) at n
      *elem(ODD ? j : opp_of(j)) = code[j];
    }
    if (flag >> 3) {
#pragma unroll
      for (int i = 1; i < 19; i++) {
        if (!(flag & (1u << (3 + i)))) continue;
        const int j = opp_of(i);
        const uint32_t wx = cx_of(i) > 0 ? xm : (cx_of(i) < 0 ? xp : x);
        const uint32_t wy = cy_of(i) > 0 ? (y == 0 ? p.ny - 1 : y - 1) : (cy_of(i) < 0 ? (y + 1 == p.ny ? 0 : y + 1) : y);
        const uint32_t wz = cz_of(i) > 0 ? (z == 0 ? p.nz - 1 : z - 1) : (cz_of(i) < 0 ? (z + 1 == p.nz ? 0 : z + 1) : z);
        if ((__ldg(&p.flags[wx + nx * wy + plane * wz]) & 7u) == SOLID) {
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
    if (x + 2 == nx) p.plane_out[y + p.ny * z] = outlet_velocity_of<ST>(code);
  }

  // ---------------------------------------------------------------- write back
  fence_proxy_async_smem();
  __syncthreads();
  if (threadIdx.x < 32) {
    for (uint32_t k = threadIdx.x; k < copies; k += 32) {
      const int s = (int)(k / R);
      const uint32_t tr = k - (uint32_t)s * R;
      bulk_store(f + staged_row(p, s, R0 + tr, ODD), buf + ((size_t)s * rows_per_tile + tr) * nx, row_bytes);
    }
    bulk_commit();
    bulk_wait_all();
  }
  reduce_force(force_any, fx, fy, fz, p.partials);
}

// Rows per tile for a domain: about `target` bytes of staged rows, at least one row.
inline uint32_t tile_rows(uint32_t nx, uint32_t rows, size_t elem_bytes, size_t target) {
  size_t per_row = 19 * (size_t)nx * elem_bytes;
  size_t r = target / per_row;
  if (r < 1) r = 1;
  if (r > rows) r = rows;
  return (uint32_t)r;
}

#ifdef PW_DEFINE_LAUNCHERS
static size_t elem_bytes(int storage) { return storage == STORE_F32 ? 4 : 2; }

uint32_t tile_rows_for(uint32_t nx, uint32_t rows, int storage) {
  return tile_rows(nx, rows, elem_bytes(storage), (size_t)40 << 10);
}

size_t tile_smem_bytes(uint32_t nx, uint32_t rows_per_tile, int storage) {
  return 19 * (size_t)rows_per_tile * nx * elem_bytes(storage);
}

template <int ST, int OP, bool LES>
static cudaError_t allow_smem(size_t bytes) {
  cudaError_t e = cudaFuncSetAttribute(aa_step_tile<ST, OP, LES, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(aa_step_tile<ST, OP, LES, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)bytes);
  return e;
}

template <int ST>
static cudaError_t allow_smem_all(size_t bytes) {
  cudaError_t e = allow_smem<ST, OP_TRT, false>(bytes);
  if (e == cudaSuccess) e = allow_smem<ST, OP_TRT, true>(bytes);
  if (e == cudaSuccess) e = allow_smem<ST, OP_REG, false>(bytes);
  if (e == cudaSuccess) e = allow_smem<ST, OP_REG, true>(bytes);
  return e;
}

cudaError_t prepare_tile_kernels(size_t smem_bytes) {
  cudaError_t e = allow_smem_all<STORE_F32>(smem_bytes);
  if (e == cudaSuccess) e = allow_smem_all<STORE_F16>(smem_bytes);
  if (e == cudaSuccess) e = allow_smem_all<STORE_BF16>(smem_bytes);
  return e;
}

template <int ST, int OP, bool LES>
static void tile3(const StepParams &p, bool odd, uint32_t rpt, unsigned blocks, size_t smem, cudaStream_t s) {
  if (odd) aa_step_tile<ST, OP, LES, true><<<blocks, TILE_THREADS, smem, s>>>(p, rpt);
  else aa_step_tile<ST, OP, LES, false><<<blocks, TILE_THREADS, smem, s>>>(p, rpt);
}
template <int ST>
static void tile2(const StepParams &p, int op, int les, bool odd, uint32_t rpt, unsigned blocks, size_t smem,
                  cudaStream_t s) {
  if (op == OP_REG) {
    if (les) tile3<ST, OP_REG, true>(p, odd, rpt, blocks, smem, s);
    else tile3<ST, OP_REG, false>(p, odd, rpt, blocks, smem, s);
  } else {
    if (les) tile3<ST, OP_TRT, true>(p, odd, rpt, blocks, smem, s);
    else tile3<ST, OP_TRT, false>(p, odd, rpt, blocks, smem, s);
  }
}
void launch_step_tile(const StepParams &p, int storage, int op, int les, bool odd, uint32_t rpt, unsigned blocks,
                      size_t smem, cudaStream_t s) {
  switch (storage) {
    case STORE_F16: tile2<STORE_F16>(p, op, les, odd, rpt, blocks, smem, s); break;
    case STORE_BF16: tile2<STORE_BF16>(p, op, les, odd, rpt, blocks, smem, s); break;
    default: tile2<STORE_F32>(p, op, les, odd, rpt, blocks, smem, s); break;
  }
}
#endif

}  // namespace PW_NS
