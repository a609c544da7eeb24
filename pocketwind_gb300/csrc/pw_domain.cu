// Solver domain: the C-ABI counterpart of the reference's GpuSolver and GpuForce
// (src/lbm/gpu-solver.ts:135-465, src/lbm/gpu-force.ts:45-216).
//
// Memory (one GB300, everything resident in HBM):
//   f         19 * stride population codes, updated in place (AA pattern)
//   macros    float4 per cell
//   plane[2]  float4 per (y, z): outlet upstream velocity, double-buffered by step parity
//   flags     u32 per cell; special: 1 bit per cell (non-plain cells)
//   partials[2] 3 doubles per step block: momentum exchange of the even / odd states
// Stepping queues one fused kernel per step on the domain's stream; runs of
// steps without ramping are replayed from captured CUDA graphs.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <tuple>

#include "pw_internal.h"

#include "pw_launch.h"

using namespace pwhost;

namespace {

constexpr int kGraphChunk = 64;  // steps per captured graph

__global__ void special_kernel(const uint32_t *flags, size_t cells, uint32_t *special) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t bit = 0;
  if (i < cells) {
    uint32_t f = flags[i];
    bit = (f & 7u) != pw::FLUID || (f >> 3) != 0u;
  }
  uint32_t word = __ballot_sync(0xffffffffu, bit);
  if ((threadIdx.x & 31) == 0 && i < cells) special[i >> 5] = word;
}

// Counts the cells of the z = 0 plane that are not FLOOR.
__global__ void floor_plane_kernel(const uint32_t *flags, uint32_t cells, uint32_t *not_floor) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < cells && (flags[i] & 7u) != pw::FLOOR) atomicAdd(not_floor, 1u);
}

// The fast step's edge list: non-wall cells that are special or on the x faces,
// except EQ cells without wall links, in ascending cell order (so its force
// partials sum in a fixed order).
// With floor rows the list is partitioned: part 0 the other edge cells, part 1
// the floor cells (is_floor_cell), which the floor kernel updates in a
// domain's own step and a batch's edge items take with the rest.
__device__ __forceinline__ bool is_edge_cell(const uint32_t *flags, const uint32_t *special, uint32_t n, uint32_t nx,
                                             uint32_t ny, uint32_t nz, int floor_rows, int part) {
  const uint32_t flag = flags[n];
  if (pw::is_wall_kind(flag & 7u) || flag == pw::EQ) return false;  // EQ without wall links: plain kernels
  if (!pw::is_plain_position(n % nx, nx) || ((special[n >> 5] >> (n & 31u)) & 1u)) {
    const bool floor = floor_rows && pw::is_floor_cell(flag, (n / nx) % ny, n / nx / ny, ny);
    return part ? floor : !floor;
  }
  return false;
}

constexpr int kEdgeBlock = 1024;

__global__ void edge_count_kernel(const uint32_t *flags, const uint32_t *special, uint32_t nx, uint32_t ny,
                                  uint32_t nz, uint32_t cells, int floor_rows, int part, uint32_t *block_counts) {
  __shared__ uint32_t warp_counts[kEdgeBlock / 32];
  const uint32_t n = blockIdx.x * kEdgeBlock + threadIdx.x;
  const bool pred = n < cells && is_edge_cell(flags, special, n, nx, ny, nz, floor_rows, part);
  const uint32_t ballot = __ballot_sync(0xffffffffu, pred);
  if ((threadIdx.x & 31) == 0) warp_counts[threadIdx.x >> 5] = __popc(ballot);
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int w = 0; w < kEdgeBlock / 32; w++) t += warp_counts[w];
    block_counts[blockIdx.x] = t;
  }
}

// Exclusive scan of the block counts in place (one block); total into *total.
__global__ void edge_scan_kernel(uint32_t *counts, uint32_t nblk, uint32_t *total) {
  __shared__ uint32_t sh[kEdgeBlock];
  uint32_t carry = 0;
  for (uint32_t base = 0; base < nblk; base += kEdgeBlock) {
    const uint32_t i = base + threadIdx.x;
    const uint32_t v = i < nblk ? counts[i] : 0u;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < kEdgeBlock; o <<= 1) {
      uint32_t add = threadIdx.x >= (unsigned)o ? sh[threadIdx.x - o] : 0u;
      __syncthreads();
      sh[threadIdx.x] += add;
      __syncthreads();
    }
    if (i < nblk) counts[i] = carry + sh[threadIdx.x] - v;
    carry += sh[kEdgeBlock - 1];
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

__global__ void edge_write_kernel(const uint32_t *flags, const uint32_t *special, uint32_t nx, uint32_t ny,
                                  uint32_t nz, uint32_t cells, int floor_rows, int part, const uint32_t *offsets,
                                  uint32_t *list) {
  __shared__ uint32_t warp_base[kEdgeBlock / 32];
  const uint32_t n = blockIdx.x * kEdgeBlock + threadIdx.x;
  const bool pred = n < cells && is_edge_cell(flags, special, n, nx, ny, nz, floor_rows, part);
  const uint32_t ballot = __ballot_sync(0xffffffffu, pred);
  const uint32_t lane = threadIdx.x & 31;
  if (lane == 0) warp_base[threadIdx.x >> 5] = __popc(ballot);
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = offsets[blockIdx.x];
    for (int w = 0; w < kEdgeBlock / 32; w++) { uint32_t c = warp_base[w]; warp_base[w] = t; t += c; }
  }
  __syncthreads();
  if (pred) list[warp_base[threadIdx.x >> 5] + __popc(ballot & ((1u << lane) - 1u))] = n;
}

// Free-slip faces reflect instead of wrapping, so a wall link whose pull source
// lies beyond one (a wall reached through the periodic wrap) does not exist.
__global__ void clear_slip_links_kernel(uint32_t *flags, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t slip,
                                        size_t cells) {
  const size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= cells) return;
  uint32_t f = flags[n];
  if ((f >> 3) == 0u) return;
  const uint32_t y = (uint32_t)((n / nx) % ny), z = (uint32_t)(n / ((size_t)nx * ny));
  for (int i = 1; i < 19; i++) {
    const int sy = (int)y - pw::cy_of(i), sz = (int)z - pw::cz_of(i);
    const bool cross = ((slip & 1u) && (sy < 0 || sy >= (int)ny)) || ((slip & 2u) && (sz < 0 || sz >= (int)nz));
    if (cross) f &= ~(1u << (3 + i));
  }
  flags[n] = f;
}

__global__ void first_fluid_kernel(const uint32_t *flags, size_t cells, unsigned long long *out) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < cells && (flags[i] & 7u) == pw::FLUID) atomicMin(out, (unsigned long long)i);
}

// Sum both parities' partials: 0.5 * (F(even state) + F(odd state)) (force.wgsl:31-32,
// reduce.wgsl), binary64, fixed order.
__global__ void force_reduce_kernel(const double *a, const double *b, size_t nblocks, double *out) {
  __shared__ double sh[256][3];
  double s0 = 0, s1 = 0, s2 = 0;
  for (size_t k = threadIdx.x; k < nblocks; k += 256) {
    s0 += a[3 * k] + b[3 * k];
    s1 += a[3 * k + 1] + b[3 * k + 1];
    s2 += a[3 * k + 2] + b[3 * k + 2];
  }
  sh[threadIdx.x][0] = s0; sh[threadIdx.x][1] = s1; sh[threadIdx.x][2] = s2;
  __syncthreads();
  for (int st = 128; st > 0; st >>= 1) {
    if (threadIdx.x < (unsigned)st)
      for (int c = 0; c < 3; c++) sh[threadIdx.x][c] += sh[threadIdx.x + st][c];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int c = 0; c < 3; c++) out[c] = 0.5 * sh[0][c];
}

enum ForceState { FORCE_IDLE = 0, FORCE_ENCODED = 1 };

}  // namespace

struct pw_domain {
  pw_domain_desc desc{};
  uint32_t nx = 0, ny = 0, nz = 0;
  size_t cells = 0;
  uint32_t stride = 0;
  size_t esize = 4;
  int device = 0;                 // current device at creation: the domain's memory and streams live there
  void *f = nullptr;
  float4 *macros = nullptr;
  float4 *plane[2] = {nullptr, nullptr};
  uint32_t *flags = nullptr, *special = nullptr;
  bool floor_rows = false;        // the floor kernel updates the floor layer (is_floor_cell)
  float wall_c = 0, wall_e = 0;   // Werner-Wengle constants of the floor cells' wall model
  double *partials[2] = {nullptr, nullptr};
  size_t nblocks = 0;
  double *force_dev = nullptr;
  double *force_host = nullptr;   // pinned staging slot
  uint32_t *status_dev = nullptr;
  uint32_t *status_host = nullptr;
  double *totals_dev = nullptr;
  void *scratch = nullptr;        // readout / write-in buffer, allocated on first use
  uint64_t first_fluid = ~0ull;
  cudaStream_t stream = nullptr;
  cudaEvent_t force_event = nullptr;
  pwfast::SideStream side;        // edge and seam kernels of split steps run here, beside the plain kernel
  uint64_t steps = 0;
  int force_state = FORCE_IDLE;
  uint64_t force_step = 0;
  float u_in = 0, nu = 0, cs_term = 0, lambda = 0, tau0 = 0, om_p = 0, om_m = 0;
  dim3 grid;
  uint32_t slip = 0;              // free-slip faces (bit 0 y, bit 1 z)
  bool split = false;             // fast build, one cell per thread: plain kernel + edge list
  uint32_t *edges = nullptr;      // edge cells in ascending order
  uint32_t edge_count = 0;
  uint32_t edge_own = 0;          // the list's head that a domain's own step runs (all but its floor cells)
  dim3 plain_grid;                // the cell grid, or empty when no plain position exists
  const uint32_t *closure_frag = nullptr;  // attached learned closure (its weight fragments)
  uint8_t *wall_dist = nullptr;   // cells to the nearest wall, for the closure's inputs
  bool interp = false;            // interpolated (Bouzidi) walls
  uint32_t *qoff = nullptr;       // per cell: first wall-link fraction (interpolated walls)
  float *qfrac = nullptr;         // wall-link fractions in link-rank order
  void *hist = nullptr;           // per link: the cell's own latest post-collision code
  bool tiled = false;             // TMA-staged row tiles
  uint32_t rows_per_tile = 0;
  unsigned tile_blocks = 0;
  size_t tile_smem = 0;
  // captured step runs: key (start parity, write macro on last) -> graph of kGraphChunk steps
  std::map<std::pair<int, int>, cudaGraphExec_t> graphs;
};

namespace pwhost {
void domain_dims(const pw_domain *d, uint32_t *nx, uint32_t *ny, uint32_t *nz) {
  *nx = d->nx; *ny = d->ny; *nz = d->nz;
}
DomainView domain_view(const pw_domain *d) {
  return DomainView{d->f, d->flags, d->nx, d->ny, d->nz, d->stride, d->steps, d->desc.storage, d->stream, d->slip,
                    d->device};
}
}  // namespace pwhost

namespace {

pw::StepParams params_for(const pw_domain *d, uint64_t step, float u_in, int write_macro) {
  pw::StepParams p{};
  int par = (int)(step & 1);
  p.f = d->f;
  p.macros = d->macros;
  p.plane_in = d->plane[par ^ 1];
  p.plane_out = d->plane[par];
  p.flags = d->flags;
  p.special = d->special;
  p.partials = d->partials[par];
  p.status = d->status_dev;
  p.nx = d->nx; p.ny = d->ny; p.nz = d->nz;
  p.stride = d->stride;
  p.u_in = u_in;
  p.nu = d->nu; p.cs_term = d->cs_term; p.lambda = d->lambda;
  p.tau0 = d->tau0; p.omega_plus = d->om_p; p.omega_minus = d->om_m;
  p.write_macro = write_macro;
  p.slip = d->slip;
  if (d->interp) {
    // a step evaluates the wall values of the state it reads, so its partials
    // hold that (previous) state's momentum exchange
    p.qoff = d->qoff;
    p.q = d->qfrac;
    p.hist = d->hist;
    p.partials = d->partials[par ^ 1];
  }
  // Per-direction element offsets of the plain cells.  Even steps read slot i
  // and write slot opp(j) of the cell itself; odd steps read slot opp(i) of
  // n - c_i and write slot j of n + c_j.  Every offset is non-negative
  // (stride >= cells) and n + offset < 19 * stride (64-bit element indices).
  const int64_t S = d->stride;
  const int64_t nx = d->nx, nxy = (int64_t)d->nx * d->ny;
  for (int i = 0; i < 19; i++) {
    const int64_t off = pw::cx_of(i) + nx * pw::cy_of(i) + nxy * pw::cz_of(i);
    p.ld[i] = par ? pw::opp_of(i) * S - off : i * S;
    p.st[i] = par ? i * S + off : pw::opp_of(i) * S;
    p.ldb[i] = (int64_t)p.ld[i] * (int64_t)d->esize;
    p.stb[i] = (int64_t)p.st[i] * (int64_t)d->esize;
    p.wb[i] = (par ? i * S : pw::opp_of(i) * S - off) * (int64_t)d->esize;
  }
  p.floor_rows = d->floor_rows ? 1u : 0u;
  p.wall_c = d->wall_c;
  p.wall_e = d->wall_e;
  return p;
}

// Queue step number `step` (1-based) with the given inlet speed.
void enqueue_step(pw_domain *d, uint64_t step, float u_in, int write_macro) {
  pw::StepParams p = params_for(d, step, u_in, write_macro);
  if (write_macro) cudaMemsetAsync(d->status_dev, 0, 4, d->stream);
  bool odd = (step & 1) != 0;
  if (d->tiled && d->desc.strict)
    pwstrict::launch_step_tile(p, d->desc.storage, d->desc.op, d->desc.les, odd, d->rows_per_tile, d->tile_blocks,
                               d->tile_smem, d->stream);
  else if (d->tiled)
    pwfast::launch_step_tile(p, d->desc.storage, d->desc.op, d->desc.les, odd, d->rows_per_tile, d->tile_blocks,
                             d->tile_smem, d->stream);
  else if (d->desc.strict)
    pwstrict::launch_step(p, d->desc.storage, d->desc.op, d->desc.les, odd, d->grid, d->stream);
  else if (d->closure_frag && d->split)
    pwclosure_host::launch_closure_pairs(p, d->desc.storage, d->desc.op, odd, d->closure_frag, d->wall_dist, d->edges,
                                         d->edge_own, d->stream, &d->side);
  else if (d->closure_frag)
    pwclosure_host::launch_closure_step(p, d->desc.storage, d->desc.op, odd, d->grid, d->closure_frag, d->wall_dist,
                                        d->stream);
  else if (d->split)
    pwfast::launch_step_split(p, d->desc.storage, d->desc.op, d->desc.les, odd, d->plain_grid, d->edges,
                              d->edge_own, d->stream, nullptr, &d->side);
  else
    pwfast::launch_step(p, d->desc.storage, d->desc.op, d->desc.les, odd, d->grid, d->stream);
}

// rampFactor (gpu-solver.ts:119-123) and the f32 rounding of packSolverParams.
float ramp_speed(const pw_domain *d, uint64_t step) {
  uint32_t r = d->desc.ramp_steps;
  if (r == 0) return d->u_in;
  double factor = step == 0 ? 0.0 : (step >= r ? 1.0 : (double)step / (double)r);
  return (float)(d->desc.u_in * factor);
}

// Interpolated walls: the momentum exchange of the state after `steps` steps into
// that parity's partials, in the step kernels' slot mapping; refresh also copies
// each link's own population into hist.
void interp_state(pw_domain *d, uint64_t steps, int refresh) {
  pw::StepParams p = params_for(d, steps, d->u_in, 0);
  int odd = (int)(steps & 1);
  p.partials = d->partials[odd];
  if (d->desc.strict) pwstrict::launch_interp_state(p, odd, refresh, d->desc.storage, d->grid, nullptr, 0, d->stream);
  // the partials in the numbering of the step kernels that run: the edge
  // list's blocks (split step) or the cell tiles (closure step)
  else if (d->split) pwfast::launch_interp_state(p, odd, refresh, d->desc.storage, d->grid, d->edges, d->edge_count, d->stream);
  else pwfast::launch_interp_state(p, odd, refresh, d->desc.storage, d->grid, nullptr, 0, d->stream);
}

int launch_init(pw_domain *d) {
  float u0 = d->desc.ramp_steps > 0 ? 0.0f : d->u_in;
  PW_TRY(cudaMemsetAsync(d->f, 0, (size_t)19 * d->stride * d->esize, d->stream));
  pw::StepParams p = params_for(d, 0, u0, 1);
  if (d->tiled && d->desc.strict)
    pwstrict::launch_init_lin(p, d->plane[1], d->partials[1], d->desc.storage, d->tile_blocks,
                              d->rows_per_tile * d->nx, d->stream);
  else if (d->tiled)
    pwfast::launch_init_lin(p, d->plane[1], d->partials[1], d->desc.storage, d->tile_blocks,
                            d->rows_per_tile * d->nx, d->stream);
  else if (d->desc.strict || !d->split)
    (d->desc.strict ? pwstrict::launch_init : pwfast::launch_init)(p, d->plane[1], d->partials[1], d->desc.storage,
                                                                   d->grid, d->stream);
  else {
    // the edge list's blocks own the partials: initialise the state, then take
    // both parities' partials of the start state in that mapping
    pw::StepParams q = p;
    q.partials = nullptr;
    pwfast::launch_init(q, d->plane[1], nullptr, d->desc.storage, d->grid, d->stream);
    pwfast::launch_refresh_edges(p, 0, d->desc.storage, d->edges, d->edge_count, d->stream);
    PW_TRY(cudaMemcpyAsync(d->partials[1], d->partials[0], d->nblocks * 3 * sizeof(double),
                           cudaMemcpyDeviceToDevice, d->stream));
  }
  if (d->interp) {
    // both parities start as the start state's momentum exchange with its wall values
    interp_state(d, 0, 1);
    PW_TRY(cudaMemcpyAsync(d->partials[1], d->partials[0], d->nblocks * 3 * sizeof(double),
                           cudaMemcpyDeviceToDevice, d->stream));
  }
  PW_TRY(cudaGetLastError());
  return PW_OK;
}

void destroy_side(pw_domain *d) {
  if (d->side.stream) cudaStreamDestroy(d->side.stream);
  if (d->side.fork) cudaEventDestroy(d->side.fork);
  if (d->side.join) cudaEventDestroy(d->side.join);
  d->side = pwfast::SideStream();
}

int ensure_scratch(pw_domain *d) {
  if (d->scratch) return PW_OK;
  PW_TRY(cudaMalloc(&d->scratch, (size_t)19 * d->cells * 4));
  return PW_OK;
}

bool alive(const pw_domain *d) {
  if (!d) { set_error("The solver handle is NULL."); return false; }
  return true;
}

void drop_graphs(pw_domain *d) {
  for (auto &kv : d->graphs) cudaGraphExecDestroy(kv.second);
  d->graphs.clear();
}

// A captured run of kGraphChunk steps beginning at an odd (parity 1) or even step.
cudaGraphExec_t graph_for(pw_domain *d, int start_parity, int macro_last) {
  auto key = std::make_pair(start_parity, macro_last);
  auto it = d->graphs.find(key);
  if (it != d->graphs.end()) return it->second;
  cudaStream_t cap;
  if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess) { cudaGetLastError(); return nullptr; }
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t saved = d->stream;
  d->stream = cap;
  if (cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
    for (int k = 0; k < kGraphChunk; k++) {
      uint64_t step = (uint64_t)start_parity + (uint64_t)k;  // only the parity matters
      enqueue_step(d, step == 0 ? 2 : step, d->u_in, macro_last && k == kGraphChunk - 1);
    }
    if (cudaStreamEndCapture(cap, &graph) == cudaSuccess && graph) {
      if (cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) exec = nullptr;
      cudaGraphDestroy(graph);
    }
  }
  d->stream = saved;
  cudaStreamDestroy(cap);
  cudaGetLastError();
  if (exec) d->graphs[key] = exec;
  return exec;
}

// The fast step's edge list and its launch shapes; nblocks becomes the edge
// kernel's block count (at least 1), within the partial arrays' allocation.
// Force partial slots of a split step: one per block of the edge kernel.
size_t edge_blocks(const pw_domain *d) {
  return d->edge_count ? (d->edge_count + pw::kBlockX * pw::kBlockY - 1) / (pw::kBlockX * pw::kBlockY) : 1;
}

int build_edge_list(pw_domain *d, Allocs &a) {
  const uint32_t cells = (uint32_t)d->cells;
  const uint32_t nblk = (cells + kEdgeBlock - 1) / kEdgeBlock;
  const int floor = d->floor_rows ? 1 : 0;
  uint32_t *counts = nullptr, total[2] = {0u, 0u};
  cudaError_t e = cudaMalloc((void **)&counts, (2 * (size_t)nblk + 2) * 4);
  if (e != cudaSuccess) return cuda_status(e, "pw_domain_create edge list");
  for (int part = 0; part <= floor; part++) {
    uint32_t *c = counts + (size_t)part * (nblk + 1);
    edge_count_kernel<<<nblk, kEdgeBlock, 0, d->stream>>>(d->flags, d->special, d->nx, d->ny, d->nz, cells, floor,
                                                          part, c);
    edge_scan_kernel<<<1, kEdgeBlock, 0, d->stream>>>(c, nblk, c + nblk);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&total[part], c + nblk, 4, cudaMemcpyDeviceToHost, d->stream);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(d->stream);
  if (e == cudaSuccess) e = a.alloc((void **)&d->edges, ((size_t)total[0] + total[1]) * 4);
  for (int part = 0; part <= floor && e == cudaSuccess; part++)
    edge_write_kernel<<<nblk, kEdgeBlock, 0, d->stream>>>(d->flags, d->special, d->nx, d->ny, d->nz, cells, floor,
                                                          part, counts + (size_t)part * (nblk + 1),
                                                          d->edges + (part ? total[0] : 0u));
  if (e == cudaSuccess) e = cudaStreamSynchronize(d->stream);
  cudaFree(counts);
  if (e != cudaSuccess) return cuda_status(e, "pw_domain_create edge list");
  d->edge_count = total[0] + total[1];
  d->edge_own = total[0];
  d->nblocks = edge_blocks(d);
  d->plain_grid = d->nx >= 3 ? d->grid : dim3(0, 0, 0);
  return PW_OK;
}

// The checks of a domain description that need no device, in the order
// pw_domain_create applies them: the enumerations, then packSolverParams's
// (gpu-solver.ts:88-105) relaxation time and inlet speed in binary32, then the
// size.  Writes the binary32 viscosity and inlet speed when asked.
int check_desc(const pw_domain_desc *desc, float *nu_out, float *uin_out) {
  if (desc->nx < 1 || desc->ny < 1 || desc->nz < 1) {
    set_error("Grid dimensions must be positive safe integers.");
    return PW_ERR_INVALID;
  }
  if (desc->storage < 0 || desc->storage > 2) { set_error("Unknown population storage."); return PW_ERR_INVALID; }
  if (desc->kernel < PW_KERNEL_AUTO || desc->kernel > PW_KERNEL_TILE) { set_error("Unknown kernel choice."); return PW_ERR_INVALID; }
  if (desc->lateral != PW_LATERAL_PERIODIC && desc->lateral != PW_LATERAL_FREE_SLIP) {
    set_error("Unknown lateral boundary.");
    return PW_ERR_INVALID;
  }
  if (desc->lateral == PW_LATERAL_FREE_SLIP && desc->kernel == PW_KERNEL_TILE) {
    set_error("PW_KERNEL_TILE supports periodic lateral faces only.");
    return PW_ERR_INVALID;
  }
  if (desc->op != PW_OP_TRT && desc->op != PW_OP_REG) { set_error("Unknown collision operator."); return PW_ERR_INVALID; }
  if (desc->walls != PW_WALLS_BB && desc->walls != PW_WALLS_BOUZIDI) { set_error("Unknown wall rule."); return PW_ERR_INVALID; }
  if (desc->walls == PW_WALLS_BOUZIDI && (desc->kernel == PW_KERNEL_TILE || desc->lateral != PW_LATERAL_PERIODIC)) {
    set_error("Interpolated (Bouzidi) walls run with the one-cell-per-thread kernels and periodic lateral faces.");
    return PW_ERR_INVALID;
  }
  // packSolverParams (gpu-solver.ts:94-105)
  float tau0f = (float)desc->tau0;
  float uin = (float)desc->u_in;
  float nu = (float)(((double)tau0f - 0.5) / 3.0);
  float shader_tau = (float)((float)(3.0 * (double)nu) + 0.5);
  if (!std::isfinite(tau0f) || !std::isfinite(shader_tau) || shader_tau <= 0.5f || !std::isfinite(uin)) {
    set_error("Relaxation time must exceed 0.5 and inlet speed must be finite.");
    return PW_ERR_INVALID;
  }
  const size_t cells = (size_t)desc->nx * desc->ny * desc->nz;
  // cell indices and the plane stride (cells rounded up to 64) stay 32-bit;
  // element indices into the population array are 64-bit
  if (cells > 0xffffffffull - 64) { set_error("The grid exceeds 2^32 cells."); return PW_ERR_INVALID; }
  if (nu_out) *nu_out = nu;
  if (uin_out) *uin_out = uin;
  return PW_OK;
}

}  // namespace

extern "C" {

int pw_validate_desc(const pw_domain_desc *desc) {
  if (!desc) { set_error("NULL argument"); return PW_ERR_INVALID; }
  return check_desc(desc, nullptr, nullptr);
}

int pw_domain_create(const pw_domain_desc *desc, const pw_grid *grid, pw_domain **out) {
  if (!desc || !grid || !out) { set_error("NULL argument"); return PW_ERR_INVALID; }
  *out = nullptr;
  if (desc->nx != grid->nx || desc->ny != grid->ny || desc->nz != grid->nz) {
    set_error("Geometry must match the solver layout and contain flags and q offsets.");
    return PW_ERR_INVALID;
  }
  float nu = 0.0f, uin = 0.0f;
  const int checked = check_desc(desc, &nu, &uin);
  if (checked != PW_OK) return checked;
  size_t cells = grid->cells;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); set_error("No CUDA device is available."); return PW_ERR_CUDA; }

  pw_domain *d = new pw_domain();
  d->desc = *desc;
  d->device = dev;
  d->nx = desc->nx; d->ny = desc->ny; d->nz = desc->nz;
  d->cells = cells;
  d->stride = (uint32_t)((cells + 63) / 64 * 64);
  d->esize = desc->storage == PW_STORE_F32 ? 4 : 2;
  d->slip = desc->lateral == PW_LATERAL_FREE_SLIP ? 3u : 0u;
  d->u_in = uin;
  d->nu = nu;
  d->cs_term = (float)(18.0 * 1.4142135623730951 * (0.1 * 0.1));
  d->lambda = 0.1875f;
  // binary32 constants of the LES-free operator (collide-trt.wgsl:2-4, common.wgsl:116)
  d->tau0 = 3.0f * nu + 0.5f;
  d->om_p = 1.0f / d->tau0;
  d->om_m = 1.0f / (d->lambda / (d->tau0 - 0.5f) + 0.5f);
  d->grid = dim3((d->nx + pw::kBlockX - 1) / pw::kBlockX, (d->ny + pw::kBlockY - 1) / pw::kBlockY, d->nz);
  d->nblocks = (size_t)d->grid.x * d->grid.y * d->grid.z;
  // Staged row tiles: rows must be whole 16-byte multiples for the bulk copies and fit in shared memory.
  if (desc->kernel == PW_KERNEL_TILE) {
    if ((size_t)19 * d->stride > 0xffffffffull) {
      set_error("PW_KERNEL_TILE indexes the populations with 32 bits: at most 226 M cells.");
      delete d;
      return PW_ERR_INVALID;
    }
    if ((d->nx * d->esize) % 16 != 0) {
      set_error("PW_KERNEL_TILE needs nx * element bytes to be a multiple of 16.");
      delete d;
      return PW_ERR_INVALID;
    }
    uint32_t rows = d->ny * d->nz;
    uint32_t rpt = pwfast::tile_rows_for(d->nx, rows, desc->storage);
    size_t smem = pwfast::tile_smem_bytes(d->nx, rpt, desc->storage);
    cudaError_t pe = desc->strict ? pwstrict::prepare_tile_kernels(smem) : pwfast::prepare_tile_kernels(smem);
    cudaGetLastError();
    if (smem > (size_t)200 << 10 || pe != cudaSuccess) {
      set_error("PW_KERNEL_TILE: one x-row tile does not fit in shared memory.");
      delete d;
      return PW_ERR_INVALID;
    }
    d->tiled = true;
    d->rows_per_tile = rpt;
    d->tile_smem = smem;
    d->tile_blocks = (rows + rpt - 1) / rpt;
    d->nblocks = d->tile_blocks;
  }
  size_t plane_n = (size_t)d->ny * d->nz;

  Allocs a;
  cudaError_t e = cudaStreamCreateWithFlags(&d->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&d->force_event, cudaEventDisableTiming);
  // the side stream takes the highest priority, so the edge kernel's few blocks
  // are dispatched ahead of the plain kernel's grid instead of after it
  int lo_prio = 0, hi_prio = 0;
  if (e == cudaSuccess) e = cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio);
  if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&d->side.stream, cudaStreamNonBlocking, hi_prio);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&d->side.fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&d->side.join, cudaEventDisableTiming);
  // The fast step's two-cell kernel reads (and discards) elements up to
  // nx * ny + nx + 64 past the 19 direction planes.
  if (e == cudaSuccess)
    e = a.alloc(&d->f, ((size_t)19 * d->stride + (size_t)d->nx * d->ny + d->nx + 64) * d->esize);
  if (e == cudaSuccess) e = a.alloc((void **)&d->macros, cells * sizeof(float4));
  if (e == cudaSuccess) e = a.alloc((void **)&d->plane[0], plane_n * sizeof(float4));
  if (e == cudaSuccess) e = a.alloc((void **)&d->plane[1], plane_n * sizeof(float4));
  if (e == cudaSuccess) e = a.alloc((void **)&d->flags, cells * 4);
  if (e == cudaSuccess) e = a.alloc((void **)&d->special, ((cells + 31) / 32 + 1) * 4);
  d->interp = desc->walls == PW_WALLS_BOUZIDI;
  if (d->interp && e == cudaSuccess) e = a.alloc((void **)&d->qoff, cells * 4);
  if (d->interp && e == cudaSuccess) e = a.alloc((void **)&d->qfrac, (grid->nfrac ? grid->nfrac : 1) * 4);
  if (d->interp && e == cudaSuccess) e = a.alloc(&d->hist, (grid->nfrac ? grid->nfrac : 1) * d->esize);
  if (e == cudaSuccess) e = a.alloc((void **)&d->partials[0], d->nblocks * 3 * sizeof(double));
  if (e == cudaSuccess) e = a.alloc((void **)&d->partials[1], d->nblocks * 3 * sizeof(double));
  if (e == cudaSuccess) e = a.alloc((void **)&d->force_dev, 4 * sizeof(double));
  if (e == cudaSuccess) e = a.alloc((void **)&d->status_dev, 16);
  if (e == cudaSuccess) e = a.alloc((void **)&d->totals_dev, 4 * sizeof(double));
  if (e == cudaSuccess) e = cudaMallocHost((void **)&d->force_host, 4 * sizeof(double));
  if (e == cudaSuccess) e = cudaMallocHost((void **)&d->status_host, 16);
  if (e != cudaSuccess) {
    int rc = cuda_status(e, "pw_domain_create");
    if (d->force_host) cudaFreeHost(d->force_host);
    if (d->status_host) cudaFreeHost(d->status_host);
    if (d->force_event) cudaEventDestroy(d->force_event);
    destroy_side(d);
    if (d->stream) cudaStreamDestroy(d->stream);
    delete d;
    return rc;
  }
  cudaStream_t s = d->stream;
  unsigned long long *ff = reinterpret_cast<unsigned long long *>(d->totals_dev);
  unsigned long long none = ~0ull;
  cudaMemcpyAsync(d->flags, grid->flags, cells * 4, cudaMemcpyDeviceToDevice, s);
  if (d->interp) {
    cudaMemcpyAsync(d->qoff, grid->qoff, cells * 4, cudaMemcpyDeviceToDevice, s);
    if (grid->nfrac) cudaMemcpyAsync(d->qfrac, grid->fractions, grid->nfrac * 4, cudaMemcpyDeviceToDevice, s);
  }
  cudaMemsetAsync(d->partials[0], 0, d->nblocks * 3 * sizeof(double), s);
  cudaMemsetAsync(d->partials[1], 0, d->nblocks * 3 * sizeof(double), s);
  cudaMemsetAsync(d->plane[0], 0, plane_n * sizeof(float4), s);
  cudaMemsetAsync(d->plane[1], 0, plane_n * sizeof(float4), s);
  cudaMemsetAsync(d->status_dev, 0, 16, s);
  if (d->slip)
    clear_slip_links_kernel<<<(unsigned)((cells + 255) / 256), 256, 0, s>>>(d->flags, d->nx, d->ny, d->nz, d->slip,
                                                                           cells);
  special_kernel<<<(unsigned)((cells + 255) / 256), 256, 0, s>>>(d->flags, cells, d->special);
  // Floor rows: in the fast build with 16-bit storage and nx even (the cell
  // pairs) and halfway walls, the floor kernel takes the first fluid layer over
  // a floor when the whole z = 0 plane is FLOOR (the voxelizer's floor option).
  if (!d->tiled && !desc->strict && desc->storage != PW_STORE_F32 && (d->nx & 1u) == 0u && !d->interp &&
      d->ny >= 3 && d->nz >= 3) {
    uint32_t *count = reinterpret_cast<uint32_t *>(d->status_dev) + 2, not_floor = 1;
    const uint32_t plane = d->nx * d->ny;
    cudaMemsetAsync(count, 0, 4, s);
    floor_plane_kernel<<<(plane + 255) / 256, 256, 0, s>>>(d->flags, plane, count);
    if (cudaMemcpyAsync(&not_floor, count, 4, cudaMemcpyDeviceToHost, s) == cudaSuccess &&
        cudaStreamSynchronize(s) == cudaSuccess)
      d->floor_rows = not_floor == 0;
    cudaMemsetAsync(count, 0, 4, s);
    cudaGetLastError();
  }
  d->wall_c = powf(d->nu / 0.5f, 0.142857149243354797f) / 8.3f;
  d->wall_e = 1.0f / (1.0f + 0.142857149243354797f);
  cudaMemcpyAsync(ff, &none, 8, cudaMemcpyHostToDevice, s);
  first_fluid_kernel<<<(unsigned)((cells + 255) / 256), 256, 0, s>>>(d->flags, cells, ff);
  cudaMemcpyAsync(&d->first_fluid, ff, 8, cudaMemcpyDeviceToHost, s);
  int rc = PW_OK;
  if (!d->tiled && !desc->strict) {
    d->split = true;
    rc = build_edge_list(d, a);
  }
  if (rc == PW_OK) rc = launch_init(d);
  if (rc == PW_OK) {
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) rc = cuda_status(e, "pw_domain_create init");
  }
  if (rc != PW_OK) {
    cudaFreeHost(d->force_host);
    cudaFreeHost(d->status_host);
    cudaEventDestroy(d->force_event);
    destroy_side(d);
    cudaStreamDestroy(d->stream);
    delete d;
    return rc;
  }
  a.keep = true;
  noalloc_prepare_device();
  *out = d;
  return PW_OK;
}

void pw_domain_destroy(pw_domain *d) {
  if (!d) return;
  cudaStreamSynchronize(d->stream);
  drop_graphs(d);
  cudaFree(d->f); cudaFree(d->macros); cudaFree(d->plane[0]); cudaFree(d->plane[1]);
  cudaFree(d->flags); cudaFree(d->special); cudaFree(d->partials[0]); cudaFree(d->partials[1]);
  cudaFree(d->force_dev); cudaFree(d->status_dev); cudaFree(d->totals_dev); cudaFree(d->scratch);
  cudaFree(d->edges);
  cudaFree(d->wall_dist);
  cudaFree(d->qoff); cudaFree(d->qfrac); cudaFree(d->hist);
  cudaFreeHost(d->force_host); cudaFreeHost(d->status_host);
  cudaEventDestroy(d->force_event);
  destroy_side(d);
  cudaStreamDestroy(d->stream);
  cudaGetLastError();
  delete d;
}

int pw_reset(pw_domain *d) {
  if (!alive(d)) return PW_ERR_INVALID;
  int rc = launch_init(d);
  if (rc != PW_OK) return rc;
  d->steps = 0;
  if (d->force_state == FORCE_ENCODED) d->force_state = FORCE_IDLE;  // GpuForce.reset
  return PW_OK;
}

int pw_step(pw_domain *d, uint64_t count, int write_macro_on_last) {
  if (!alive(d)) return PW_ERR_INVALID;
  if (count > (1ull << 53) || d->steps + count > (1ull << 53)) {
    set_error("Step count must be a non-negative safe integer.");
    return PW_ERR_INVALID;
  }
  uint64_t k = 0;
  // ramped steps, one launch each with its own inlet speed
  while (k < count && d->desc.ramp_steps > 0 && d->steps < d->desc.ramp_steps) {
    uint64_t step = d->steps + 1;
    enqueue_step(d, step, ramp_speed(d, step), write_macro_on_last && k == count - 1);
    d->steps++;
    k++;
  }
  // full-speed steps: graph chunks when the domain is small enough to be launch bound
  const bool use_graphs = d->cells <= (size_t)8 << 20;
  while (use_graphs && count - k >= (uint64_t)kGraphChunk) {
    int macro_last = write_macro_on_last && (count - k == (uint64_t)kGraphChunk);
    cudaGraphExec_t g = graph_for(d, (int)((d->steps + 1) & 1), macro_last);
    if (!g) break;
    if (cudaGraphLaunch(g, d->stream) != cudaSuccess) { cudaGetLastError(); break; }
    d->steps += kGraphChunk;
    k += kGraphChunk;
  }
  for (; k < count; k++) {
    uint64_t step = d->steps + 1;
    enqueue_step(d, step, d->u_in, write_macro_on_last && k == count - 1);
    d->steps++;
  }
  PW_TRY(cudaGetLastError());
  return PW_OK;
}

int pw_step_count(const pw_domain *d, uint64_t *out) {
  if (!d || !out) { set_error("NULL argument"); return PW_ERR_INVALID; }
  *out = d->steps;
  return PW_OK;
}

int pw_encode_force(pw_domain *d) {
  if (!alive(d)) return PW_ERR_INVALID;
  if (d->force_state != FORCE_IDLE) return PW_OK;  // occupied slot skips the sample
  if (d->interp) interp_state(d, d->steps, 0);  // the latest state; the last step gave the one before
  force_reduce_kernel<<<1, 256, 0, d->stream>>>(d->partials[0], d->partials[1], d->nblocks, d->force_dev);
  PW_TRY(cudaMemcpyAsync(d->force_host, d->force_dev, 3 * sizeof(double), cudaMemcpyDeviceToHost, d->stream));
  PW_TRY(cudaEventRecord(d->force_event, d->stream));
  d->force_state = FORCE_ENCODED;
  d->force_step = d->steps;
  return PW_OK;
}

int pw_read_force(pw_domain *d, pw_force_sample *out) {
  if (!alive(d) || !out) { set_error("NULL argument"); return PW_ERR_INVALID; }
  if (d->force_state != FORCE_ENCODED) return PW_ERR_BUSY;
  d->force_state = FORCE_IDLE;
  PW_TRY(cudaEventSynchronize(d->force_event));
  out->step = d->force_step;
  out->fx = d->force_host[0];
  out->fy = d->force_host[1];
  out->fz = d->force_host[2];
  return PW_OK;
}

int pw_read_macros(pw_domain *d, float *out) {
  if (!alive(d) || !out) { set_error("NULL argument"); return PW_ERR_INVALID; }
  PW_TRY(cudaMemcpyAsync(out, d->macros, d->cells * sizeof(float4), cudaMemcpyDeviceToHost, d->stream));
  PW_TRY(cudaStreamSynchronize(d->stream));
  return PW_OK;
}

int pw_write_macros(pw_domain *d, const float *in) {
  if (!alive(d) || !in) { set_error("NULL argument"); return PW_ERR_INVALID; }
  PW_TRY(cudaMemcpyAsync(d->macros, in, d->cells * sizeof(float4), cudaMemcpyHostToDevice, d->stream));
  PW_TRY(cudaStreamSynchronize(d->stream));
  return PW_OK;
}

static int read_pops(pw_domain *d, void *out, int mode) {
  if (!alive(d) || !out) { set_error("NULL argument"); return PW_ERR_INVALID; }
  int rc = ensure_scratch(d);
  if (rc != PW_OK) return rc;
  pw::StepParams p = params_for(d, d->steps, d->u_in, 0);
  int odd = (int)(d->steps & 1);
  if (d->desc.strict) pwstrict::launch_read(p, odd, mode, d->scratch, d->desc.storage, d->grid, d->stream);
  else pwfast::launch_read(p, odd, mode, d->scratch, d->desc.storage, d->grid, d->stream);
  size_t bytes = (size_t)19 * d->cells * (mode == 0 ? 4 : d->esize);
  PW_TRY(cudaMemcpyAsync(out, d->scratch, bytes, cudaMemcpyDeviceToHost, d->stream));
  PW_TRY(cudaStreamSynchronize(d->stream));
  return PW_OK;
}

int pw_read_populations(pw_domain *d, float *out) { return read_pops(d, out, 0); }
int pw_read_populations_raw(pw_domain *d, void *out) { return read_pops(d, out, 1); }

static int write_pops(pw_domain *d, const void *in, int mode) {
  if (!alive(d) || !in) { set_error("NULL argument"); return PW_ERR_INVALID; }
  int rc = ensure_scratch(d);
  if (rc != PW_OK) return rc;
  size_t bytes = (size_t)19 * d->cells * (mode == 0 ? 4 : d->esize);
  PW_TRY(cudaMemcpyAsync(d->scratch, in, bytes, cudaMemcpyHostToDevice, d->stream));
  pw::StepParams p = params_for(d, d->steps, d->u_in, 0);
  int odd = (int)(d->steps & 1);
  if (d->interp) p.partials = nullptr;  // the state pass below takes the force
  if (d->desc.strict && d->tiled) {
    pwstrict::launch_write(p, odd, mode, d->scratch, d->desc.storage, d->grid, d->stream);
    pwstrict::launch_refresh_lin(p, odd, d->desc.storage, d->tile_blocks, d->rows_per_tile * d->nx, d->stream);
  } else if (d->desc.strict) {
    pwstrict::launch_write(p, odd, mode, d->scratch, d->desc.storage, d->grid, d->stream);
    pwstrict::launch_refresh(p, odd, d->desc.storage, d->grid, d->stream);
  } else if (d->tiled) {
    pwfast::launch_write(p, odd, mode, d->scratch, d->desc.storage, d->grid, d->stream);
    pwfast::launch_refresh_lin(p, odd, d->desc.storage, d->tile_blocks, d->rows_per_tile * d->nx, d->stream);
  } else if (d->split) {
    pwfast::launch_write(p, odd, mode, d->scratch, d->desc.storage, d->grid, d->stream);
    pwfast::launch_refresh_edges(p, odd, d->desc.storage, d->edges, d->edge_count, d->stream);
  } else {
    pwfast::launch_write(p, odd, mode, d->scratch, d->desc.storage, d->grid, d->stream);
    pwfast::launch_refresh(p, odd, d->desc.storage, d->grid, d->stream);
  }
  if (d->interp) interp_state(d, d->steps, 1);
  PW_TRY(cudaStreamSynchronize(d->stream));
  return PW_OK;
}

int pw_write_populations(pw_domain *d, const float *g) { return write_pops(d, g, 0); }
int pw_write_populations_raw(pw_domain *d, const void *raw) { return write_pops(d, raw, 1); }

int pw_read_totals(pw_domain *d, double out[4]) {
  if (!alive(d) || !out) { set_error("NULL argument"); return PW_ERR_INVALID; }
  PW_TRY(cudaMemsetAsync(d->totals_dev, 0, 4 * sizeof(double), d->stream));
  pw::StepParams p = params_for(d, d->steps, d->u_in, 0);
  int odd = (int)(d->steps & 1);
  if (d->desc.strict) pwstrict::launch_totals(p, odd, d->totals_dev, d->desc.storage, d->grid, d->stream);
  else pwfast::launch_totals(p, odd, d->totals_dev, d->desc.storage, d->grid, d->stream);
  PW_TRY(cudaMemcpyAsync(out, d->totals_dev, 4 * sizeof(double), cudaMemcpyDeviceToHost, d->stream));
  PW_TRY(cudaStreamSynchronize(d->stream));
  return PW_OK;
}

int pw_guard_check(pw_domain *d, int *unstable) {
  if (!alive(d) || !unstable) { set_error("NULL argument"); return PW_ERR_INVALID; }
  PW_TRY(cudaMemcpyAsync(d->status_host, d->status_dev, 4, cudaMemcpyDeviceToHost, d->stream));
  PW_TRY(cudaStreamSynchronize(d->stream));
  *unstable = (d->status_host[0] & 1u) ? 1 : 0;
  if (d->status_host[0] & 2u) {
    set_error("A step's staged copies did not complete in time (the step's state is not valid).");
    return PW_ERR_TIMEOUT;
  }
  return PW_OK;
}

int pw_inject_nan(pw_domain *d) {
  if (!alive(d)) return PW_ERR_INVALID;
  if (d->first_fluid == ~0ull) return PW_OK;
  // The rest population of a cell sits in slot 0 of the cell in both layouts.
  uint32_t f32nan = 0x7fc00000u;
  uint16_t h16nan = d->desc.storage == PW_STORE_F16 ? 0x7e00u : 0x7fc0u;
  char *base = reinterpret_cast<char *>(d->f) + d->first_fluid * d->esize;
  const void *src = d->esize == 4 ? (const void *)&f32nan : (const void *)&h16nan;
  PW_TRY(cudaMemcpyAsync(base, src, d->esize, cudaMemcpyHostToDevice, d->stream));
  PW_TRY(cudaStreamSynchronize(d->stream));
  return PW_OK;
}

int pw_domain_buffers(pw_domain *d, void **macros, void **flags, void **stream) {
  if (!alive(d)) return PW_ERR_INVALID;
  if (macros) *macros = d->macros;
  if (flags) *flags = d->flags;
  if (stream) *stream = d->stream;
  return PW_OK;
}

int pw_profile_steps(pw_domain *d, uint64_t count, float kernel_ms[3]) {
  if (!alive(d) || !kernel_ms) { set_error("NULL argument"); return PW_ERR_INVALID; }
  kernel_ms[0] = kernel_ms[1] = kernel_ms[2] = 0.0f;
  constexpr int kBatch = 32;
  cudaEvent_t ev[kBatch][6];
  int made = 0;
  cudaError_t e = cudaSuccess;
  for (; made < kBatch * 6 && e == cudaSuccess; made++) e = cudaEventCreate(&ev[made / 6][made % 6]);
  uint64_t k = 0;
  while (e == cudaSuccess && k < count) {
    const int n = (int)std::min<uint64_t>(kBatch, count - k);
    for (int b = 0; b < n; b++) {
      const uint64_t step = d->steps + 1;
      pw::StepParams p = params_for(d, step, ramp_speed(d, step), 0);
      const bool odd = (step & 1) != 0;
      if (d->split && !d->closure_frag) {
        pwfast::launch_step_split(p, d->desc.storage, d->desc.op, d->desc.les, odd, d->plain_grid, d->edges,
                                  d->edge_own, d->stream, ev[b]);
      } else {
        cudaEventRecord(ev[b][0], d->stream);
        enqueue_step(d, step, ramp_speed(d, step), 0);
        for (int m = 1; m < 6; m++) cudaEventRecord(ev[b][m], d->stream);
      }
      d->steps++;
    }
    e = cudaEventSynchronize(ev[n - 1][5]);
    for (int b = 0; b < n && e == cudaSuccess; b++) {
      for (int c = 0; c < 3 && e == cudaSuccess; c++) {
        float t = 0.0f;
        e = cudaEventElapsedTime(&t, ev[b][2 * c], ev[b][2 * c + 1]);
        kernel_ms[c] += t;
      }
    }
    k += (uint64_t)n;
  }
  for (int m = 0; m < made; m++) cudaEventDestroy(ev[m / 6][m % 6]);
  if (e != cudaSuccess) return cuda_status(e, "pw_profile_steps");
  return PW_OK;
}

int pw_time_steps(pw_domain *d, uint64_t count, float *ms) {
  if (!alive(d) || !ms) { set_error("NULL argument"); return PW_ERR_INVALID; }
  cudaEvent_t a, b;
  PW_TRY(cudaEventCreate(&a));
  PW_TRY(cudaEventCreate(&b));
  cudaEventRecord(a, d->stream);
  int rc = pw_step(d, count, 0);
  cudaEventRecord(b, d->stream);
  cudaError_t e = cudaEventSynchronize(b);
  if (e == cudaSuccess) e = cudaEventElapsedTime(ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (rc != PW_OK) return rc;
  if (e != cudaSuccess) return cuda_status(e, "pw_time_steps");
  return PW_OK;
}

}  // extern "C"

namespace pwhost {
MemberView member_view(const pw_domain *d) {
  MemberView v;
  v.split = d->split;
  v.closure = d->closure_frag != nullptr;
  v.storage = d->desc.storage;
  v.op = d->desc.op;
  v.les = d->desc.les;
  v.nx = d->nx; v.ny = d->ny; v.nz = d->nz;
  v.steps = d->steps;
  v.ramping = d->desc.ramp_steps > 0 && d->steps < d->desc.ramp_steps;
  v.interpolated = d->interp;
  v.edges = d->edges;
  v.edge_count = d->edge_count;
  v.slip = d->slip;
  v.status = d->status_dev;
  v.stream = d->stream;
  return v;
}
pw::StepParams member_params(const pw_domain *d, uint64_t step, int write_macro) {
  pw::StepParams p = params_for(d, step, d->u_in, write_macro);
  p.floor_rows = 0;  // a batch's edge items take the floor layer through the general path
  return p;
}
void member_advance(pw_domain *d, uint64_t n) { d->steps += n; }
}  // namespace pwhost

extern "C" int pw_closure_attach(pw_domain *d, const pw_closure *c) {
  if (!alive(d)) return PW_ERR_INVALID;
  if (c) {
    if (d->desc.strict || d->tiled || !d->desc.les) {
      set_error("A closure needs an LES domain on the fast build's one-cell-per-thread path.");
      return PW_ERR_INVALID;
    }
    if (!d->wall_dist) {
      PW_TRY(cudaMalloc(&d->wall_dist, d->cells));
      int rc = pwclosure_host::wall_distance_of(d->flags, d->nx, d->ny, d->nz, d->wall_dist, d->stream);
      if (rc != PW_OK) return rc;
    }
    d->closure_frag = pwclosure_host::fragments(c);
    // periodic faces: the cell-pair closure step with the edge list beside it
    // (the split step's partials); free-slip faces: the one-cell closure step
    // over the cell tiles
    d->split = d->slip == 0u;
    d->nblocks = d->split ? edge_blocks(d) : (size_t)d->grid.x * d->grid.y * d->grid.z;
  } else {
    if (!d->closure_frag) return PW_OK;
    d->closure_frag = nullptr;
    d->split = true;
    d->nblocks = edge_blocks(d);
  }
  drop_graphs(d);
  PW_TRY(cudaMemsetAsync(d->partials[0], 0, (size_t)d->grid.x * d->grid.y * d->grid.z * 3 * sizeof(double), d->stream));
  PW_TRY(cudaMemsetAsync(d->partials[1], 0, (size_t)d->grid.x * d->grid.y * d->grid.z * 3 * sizeof(double), d->stream));
  int rc = launch_init(d);
  if (rc != PW_OK) return rc;
  d->steps = 0;
  if (d->force_state == FORCE_ENCODED) d->force_state = FORCE_IDLE;
  PW_TRY(cudaStreamSynchronize(d->stream));
  return PW_OK;
}

// ---------------------------------------------------------------- field export, checkpoint
namespace {

// The macros of a box of cells, x fastest, into a packed device buffer.
__global__ void macro_box_kernel(const float4 *macros, uint32_t nx, uint32_t ny, uint32_t x0, uint32_t y0,
                                 uint32_t z0, uint32_t wx, uint32_t wy, uint32_t wz, float4 *out) {
  const size_t total = (size_t)wx * wy * wz;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += (size_t)gridDim.x * blockDim.x) {
    const size_t x = k % wx, y = (k / wx) % wy, z = k / ((size_t)wx * wy);
    out[k] = macros[(x0 + x) + (size_t)nx * ((y0 + y) + (size_t)ny * (z0 + z))];
  }
}

__device__ __forceinline__ uint32_t big_endian(float v) { return __byte_perm(__float_as_uint(v), 0u, 0x0123u); }

// The bytes of writeVtk (src/io/vtk.ts:56-80) after the header, with latticeToField's
// velocity scale (src/io/field-export.ts:22-29): rho as big-endian binary32; a newline and
// "VECTORS velocity float\n" (24 bytes, so the velocity block starts on a word); the
// velocity triples, each the binary64 product value * scale rounded to binary32; a newline.
__global__ void vtk_body_kernel(const float4 *macros, size_t cells, double scale, uint32_t *out) {
  const size_t vel = cells + 6;
  for (size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x; n < cells; n += (size_t)gridDim.x * blockDim.x) {
    float4 m = macros[n];
    out[n] = big_endian(m.x);
    out[vel + 3 * n] = big_endian((float)((double)m.y * scale));
    out[vel + 3 * n + 1] = big_endian((float)((double)m.z * scale));
    out[vel + 3 * n + 2] = big_endian((float)((double)m.w * scale));
  }
  if (blockIdx.x == 0 && threadIdx.x < 24) {
    const char text[25] = "\nVECTORS velocity float\n";
    reinterpret_cast<char *>(out + cells)[threadIdx.x] = text[threadIdx.x];
    if (threadIdx.x == 0) reinterpret_cast<char *>(out + vel + 3 * cells)[0] = '\n';
  }
}

// Solver-state checkpoint: this header, then the populations (direction-major, in the
// storage's own codes, read at the saved step's parity), the macros (float4 per cell),
// and both parities' force partials.  Little-endian; the checksum covers header and payload.
struct CheckpointHeader {
  char magic[8];
  uint32_t version;
  uint32_t header_bytes;
  uint32_t nx, ny, nz;
  int32_t storage, op, les, walls, lateral, strict;
  uint32_t status;
  uint64_t steps;
  uint64_t population_bytes, macro_bytes, partial_bytes;
  float tau0, u_in;
  uint32_t ramp_steps, reserved;
  uint64_t checksum;
};
static_assert(sizeof(CheckpointHeader) == 112, "checkpoint header layout");
constexpr char kCheckpointMagic[8] = {'P', 'W', 'S', 'T', 'A', 'T', 'E', '\0'};
constexpr uint32_t kCheckpointVersion = 1;

// 64-bit words folded with a multiply-xorshift per word (the tail bytes zero-padded).
uint64_t fold_words(uint64_t h, const unsigned char *p, size_t bytes) {
  size_t k = 0;
  for (; k + 8 <= bytes; k += 8) {
    uint64_t w;
    std::memcpy(&w, p + k, 8);
    h = (h ^ w) * 0x9e3779b97f4a7c15ull;
    h ^= h >> 29;
  }
  if (k < bytes) {
    uint64_t w = 0;
    std::memcpy(&w, p + k, bytes - k);
    h = (h ^ w) * 0x9e3779b97f4a7c15ull;
    h ^= h >> 29;
  }
  return h;
}

// Checksum of the header (its checksum field taken as zero) and the payload.
uint64_t checkpoint_checksum(CheckpointHeader h, const unsigned char *payload, size_t bytes) {
  h.checksum = 0;
  uint64_t s = fold_words(0x243f6a8885a308d3ull, reinterpret_cast<const unsigned char *>(&h), sizeof h);
  return fold_words(s, payload, bytes);
}

CheckpointHeader header_of(const pw_domain *d) {
  CheckpointHeader h{};
  std::memcpy(h.magic, kCheckpointMagic, 8);
  h.version = kCheckpointVersion;
  h.header_bytes = sizeof(CheckpointHeader);
  h.nx = d->nx; h.ny = d->ny; h.nz = d->nz;
  h.storage = d->desc.storage; h.op = d->desc.op; h.les = d->desc.les;
  h.walls = d->desc.walls; h.lateral = d->desc.lateral; h.strict = d->desc.strict;
  h.steps = d->steps;
  h.population_bytes = (uint64_t)19 * d->cells * d->esize;
  h.macro_bytes = (uint64_t)d->cells * sizeof(float4);
  h.partial_bytes = (uint64_t)2 * d->nblocks * 3 * sizeof(double);
  h.tau0 = d->tau0; h.u_in = (float)d->desc.u_in;
  h.ramp_steps = d->desc.ramp_steps;
  return h;
}

}  // namespace

extern "C" {

int pw_field_vtk_body(pw_domain *d, double velocity_scale, void *out, size_t capacity) {
  if (!alive(d) || !out) { set_error("NULL argument"); return PW_ERR_INVALID; }
  if (!std::isfinite(velocity_scale) || velocity_scale <= 0) {
    set_error("speedMps must be a positive finite number.");
    return PW_ERR_INVALID;
  }
  size_t bytes = 16 * d->cells + 25;
  if (capacity < bytes) { set_error("The output buffer is smaller than the field's VTK body."); return PW_ERR_INVALID; }
  int rc = ensure_scratch(d);
  if (rc != PW_OK) return rc;
  unsigned blocks = (unsigned)std::min<size_t>((d->cells + 255) / 256, (size_t)152 * 16);
  vtk_body_kernel<<<blocks, 256, 0, d->stream>>>(d->macros, d->cells, velocity_scale,
                                                 reinterpret_cast<uint32_t *>(d->scratch));
  PW_TRY(cudaGetLastError());
  PW_TRY(cudaMemcpyAsync(out, d->scratch, bytes, cudaMemcpyDeviceToHost, d->stream));
  PW_TRY(cudaStreamSynchronize(d->stream));
  return PW_OK;
}

int pw_read_macros_box(pw_domain *d, uint32_t x0, uint32_t y0, uint32_t z0, uint32_t wx, uint32_t wy, uint32_t wz,
                       float *out) {
  if (!alive(d) || !out) { set_error("NULL argument"); return PW_ERR_INVALID; }
  if (wx == 0 || wy == 0 || wz == 0 || (uint64_t)x0 + wx > d->nx || (uint64_t)y0 + wy > d->ny ||
      (uint64_t)z0 + wz > d->nz) {
    set_error("The box must be non-empty and inside the grid.");
    return PW_ERR_INVALID;
  }
  const size_t total = (size_t)wx * wy * wz;
  float4 *buf = nullptr;
  PW_TRY(cudaMallocAsync((void **)&buf, total * sizeof(float4), d->stream));
  unsigned blocks = (unsigned)std::min<size_t>((total + 255) / 256, (size_t)152 * 16);
  macro_box_kernel<<<blocks, 256, 0, d->stream>>>(d->macros, d->nx, d->ny, x0, y0, z0, wx, wy, wz, buf);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, buf, total * sizeof(float4), cudaMemcpyDeviceToHost, d->stream);
  cudaFreeAsync(buf, d->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(d->stream);
  if (e != cudaSuccess) return cuda_status(e, "pw_read_macros_box");
  return PW_OK;
}

int pw_checkpoint_size(const pw_domain *d, size_t *bytes) {
  if (!alive(d) || !bytes) { set_error("NULL argument"); return PW_ERR_INVALID; }
  CheckpointHeader h = header_of(d);
  *bytes = sizeof(CheckpointHeader) + h.population_bytes + h.macro_bytes + h.partial_bytes;
  return PW_OK;
}

int pw_checkpoint_save(pw_domain *d, void *out, size_t capacity) {
  if (!alive(d) || !out) { set_error("NULL argument"); return PW_ERR_INVALID; }
  CheckpointHeader h = header_of(d);
  size_t total = sizeof(CheckpointHeader) + h.population_bytes + h.macro_bytes + h.partial_bytes;
  if (capacity < total) { set_error("The output buffer is smaller than the checkpoint."); return PW_ERR_INVALID; }
  unsigned char *base = static_cast<unsigned char *>(out);
  unsigned char *pops = base + sizeof(CheckpointHeader);
  int rc = read_pops(d, pops, 1);
  if (rc != PW_OK) return rc;
  unsigned char *mac = pops + h.population_bytes;
  unsigned char *part = mac + h.macro_bytes;
  PW_TRY(cudaMemcpyAsync(mac, d->macros, h.macro_bytes, cudaMemcpyDeviceToHost, d->stream));
  PW_TRY(cudaMemcpyAsync(part, d->partials[0], h.partial_bytes / 2, cudaMemcpyDeviceToHost, d->stream));
  PW_TRY(cudaMemcpyAsync(part + h.partial_bytes / 2, d->partials[1], h.partial_bytes / 2, cudaMemcpyDeviceToHost,
                         d->stream));
  PW_TRY(cudaMemcpyAsync(&h.status, d->status_dev, 4, cudaMemcpyDeviceToHost, d->stream));
  PW_TRY(cudaStreamSynchronize(d->stream));
  h.checksum = checkpoint_checksum(h, pops, total - sizeof(CheckpointHeader));
  std::memcpy(base, &h, sizeof h);
  return PW_OK;
}

int pw_checkpoint_load(pw_domain *d, const void *in, size_t size) {
  if (!alive(d) || !in) { set_error("NULL argument"); return PW_ERR_INVALID; }
  CheckpointHeader h;
  if (size < sizeof h) { set_error("The checkpoint is truncated."); return PW_ERR_INVALID; }
  std::memcpy(&h, in, sizeof h);
  if (std::memcmp(h.magic, kCheckpointMagic, 8) != 0 || h.header_bytes != sizeof h) {
    set_error("The data is not a solver checkpoint.");
    return PW_ERR_INVALID;
  }
  if (h.version != kCheckpointVersion) { set_error("Unsupported checkpoint version."); return PW_ERR_INVALID; }
  CheckpointHeader mine = header_of(d);
  if (h.nx != mine.nx || h.ny != mine.ny || h.nz != mine.nz || h.storage != mine.storage || h.op != mine.op ||
      h.les != mine.les || h.walls != mine.walls || h.lateral != mine.lateral || h.strict != mine.strict ||
      h.tau0 != mine.tau0 || h.u_in != mine.u_in || h.ramp_steps != mine.ramp_steps) {
    set_error("The checkpoint was saved by a solver with another layout or other parameters.");
    return PW_ERR_INVALID;
  }
  if (h.population_bytes != mine.population_bytes || h.macro_bytes != mine.macro_bytes ||
      h.partial_bytes != mine.partial_bytes) {
    set_error("The checkpoint's sections do not match this solver's kernel layout.");
    return PW_ERR_INVALID;
  }
  if (h.steps > (1ull << 53)) { set_error("The checkpoint's step count is out of range."); return PW_ERR_INVALID; }
  size_t total = sizeof h + h.population_bytes + h.macro_bytes + h.partial_bytes;
  if (size < total) { set_error("The checkpoint is truncated."); return PW_ERR_INVALID; }
  const unsigned char *pops = static_cast<const unsigned char *>(in) + sizeof h;
  if (checkpoint_checksum(h, pops, total - sizeof h) != h.checksum) {
    set_error("The checkpoint's checksum does not match its contents.");
    return PW_ERR_INVALID;
  }
  uint64_t old_steps = d->steps;
  d->steps = h.steps;
  int rc = write_pops(d, pops, 1);
  if (rc != PW_OK) { d->steps = old_steps; return rc; }
  const unsigned char *mac = pops + h.population_bytes;
  const unsigned char *part = mac + h.macro_bytes;
  PW_TRY(cudaMemcpyAsync(d->macros, mac, h.macro_bytes, cudaMemcpyHostToDevice, d->stream));
  PW_TRY(cudaMemcpyAsync(d->partials[0], part, h.partial_bytes / 2, cudaMemcpyHostToDevice, d->stream));
  PW_TRY(cudaMemcpyAsync(d->partials[1], part + h.partial_bytes / 2, h.partial_bytes / 2, cudaMemcpyHostToDevice,
                         d->stream));
  PW_TRY(cudaMemcpyAsync(d->status_dev, &h.status, 4, cudaMemcpyHostToDevice, d->stream));
  PW_TRY(cudaStreamSynchronize(d->stream));
  if (d->force_state == FORCE_ENCODED) d->force_state = FORCE_IDLE;
  return PW_OK;
}

}  // extern "C"
