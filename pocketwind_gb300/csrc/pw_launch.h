// Host-side launchers of the stream-collide kernels, one set per build
// (pwfast: fused multiply-add and simplified algebra; pwstrict: reference order).
#pragma once
#include <cuda_runtime.h>

#include "pw_common.cuh"

#define PW_DECLARE_LAUNCHERS(NS)                                                                   \
  namespace NS {                                                                                   \
  void launch_step(const pw::StepParams &p, int storage, int op, int les, bool odd, dim3 grid,     \
                   cudaStream_t s);                                                                \
  void launch_init(const pw::StepParams &p, float4 *plane_b, double *partials_b, int storage,      \
                   dim3 grid, cudaStream_t s);                                                     \
  void launch_read(const pw::StepParams &p, int odd_layout, int mode, void *out, int storage,      \
                   dim3 grid, cudaStream_t s);                                                     \
  void launch_write(const pw::StepParams &p, int odd_layout, int mode, const void *in,            \
                    int storage, dim3 grid, cudaStream_t s);                                       \
  void launch_refresh(const pw::StepParams &p, int odd_layout, int storage, dim3 grid,             \
                      cudaStream_t s);                                                             \
  void launch_totals(const pw::StepParams &p, int odd_layout, double *out, int storage, dim3 grid, \
                     cudaStream_t s);                                                              \
  /* interpolated walls: force of the latest state into p.partials (grid mapping, or the edge     \
     list's when list is set), after copying each link's own population to hist when refresh */  \
  void launch_interp_state(const pw::StepParams &p, int odd_layout, int refresh, int storage,      \
                           dim3 grid, const uint32_t *list, uint32_t count, cudaStream_t s);       \
  void launch_init_lin(const pw::StepParams &p, float4 *plane_b, double *partials_b, int storage,  \
                       unsigned blocks, uint32_t cpb, cudaStream_t s);                             \
  void launch_refresh_lin(const pw::StepParams &p, int odd_layout, int storage, unsigned blocks,   \
                          uint32_t cpb, cudaStream_t s);                                           \
  /* TMA-staged rows: blocks of 128 threads owning rows_per_tile whole x-rows */                  \
  uint32_t tile_rows_for(uint32_t nx, uint32_t rows, int storage);                                 \
  size_t tile_smem_bytes(uint32_t nx, uint32_t rows_per_tile, int storage);                        \
  cudaError_t prepare_tile_kernels(size_t smem_bytes);                                             \
  void launch_step_tile(const pw::StepParams &p, int storage, int op, int les, bool odd,           \
                        uint32_t rows_per_tile, unsigned blocks, size_t smem_bytes, cudaStream_t s); \
  }

PW_DECLARE_LAUNCHERS(pwfast)
namespace pwfast {
// A second stream for the edge and seam-row kernels of a split step, forked
// from and joined back to the step's stream by the two events.
struct SideStream {
  cudaStream_t stream = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
};
// The fast build's split step: plain cells over plain_grid (the cell grid),
// the seam rows (odd steps) and the listed edge cells, whose blocks own the
// force partials.  The three kernels update disjoint cells, and in the in-place
// pattern no cell reads a slot that another writes within a step, so with side
// the seam and edge kernels run on side.stream concurrently with the plain
// kernel and join before the step ends.  With ev (6 events, no side stream) it
// records around the plain kernel (0, 1), the seam-row kernel (2, 3) and the
// edge kernel (4, 5).
void launch_step_split(const pw::StepParams &p, int storage, int op, int les, bool odd, dim3 plain_grid,
                       const uint32_t *list, uint32_t count, cudaStream_t s, const cudaEvent_t *ev = nullptr,
                       const SideStream *side = nullptr);
void launch_refresh_edges(const pw::StepParams &p, int odd_layout, int storage, const uint32_t *list,
                          uint32_t count, cudaStream_t s);
}
PW_DECLARE_LAUNCHERS(pwstrict)


struct pw_closure;
// The learned closure's step (pw_closure.cu) for a domain with a closure attached:
// one cell per thread over the tile grid, network inference on the tensor cores
// (free-slip faces).
namespace pwclosure_host {
void launch_closure_step(const pw::StepParams &p, int storage, int op, bool odd, dim3 grid, const uint32_t *frag,
                         const uint8_t *wall, cudaStream_t s);
// The same step for periodic faces in the cell-pair form: every row's plain
// cells two per thread with the network on the block's two 128-cell tiles, and
// the listed edge cells (and the floor layer) beside them on side's stream.
void launch_closure_pairs(const pw::StepParams &p, int storage, int op, bool odd, const uint32_t *frag,
                          const uint8_t *wall, const uint32_t *list, uint32_t count, cudaStream_t s,
                          const pwfast::SideStream *side);
int wall_distance_of(const uint32_t *flags, uint32_t nx, uint32_t ny, uint32_t nz, uint8_t *out, cudaStream_t s);
const uint32_t *fragments(const pw_closure *c);
}
