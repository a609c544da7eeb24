// Fast build of the stream-collide kernels: fused multiply-add allowed and the
// hand-simplified moment algebra of update_fast().
#define PW_NS pwfast
#define PW_STRICT 0
#define PW_DEFINE_LAUNCHERS
#include "pw_lbm.cuh"

#include "pw_lbm_tile.cuh"

namespace pwfast {

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

}  // namespace pwfast
