// Batched stepping of many independent domains: two concurrent persistent
// launches per step over the work of every member, replayed from captured CUDA
// graphs, with the launch shape chosen by timing (pw_batch_tune).  No counterpart in the
// reference, which runs one solver at a time (src/app/solver-slot.ts).
//
// Work items (per step parity):
//   plain  R rows x 64 cells of one member (two cells per thread: the 32-bit
//          cell-pair kernel for 16-bit storage, x / x + 32 else;
//          even steps every row, odd steps the rows off the y/z seams);
//   seam   16 seam rows x 64 cells as cell pairs with periodic wrap corrections
//          (odd steps, 16-bit storage, every nx even, periodic faces;
//          seam_pair_thread), else 16 rows x 32 cells one per thread (seam_thread);
//   edge   128 listed cells (edge_block), whose force partial goes to the
//          member's slot of that block, exactly as its own edge kernel does.
// A step is two persistent launches, as a single domain's step is: the plain
// items, and the seam and edge items on a high-priority side stream beside
// them (disjoint cells, so they may run together), each kernel with only its
// own code path and registers.  A block loads its item's member parameters
// into shared memory and runs the same device code as the member's own
// kernels, so a member stepped in a batch follows the same arithmetic as one
// stepped alone.
#define PW_NS pwbatch
#define PW_STRICT 0
#include <algorithm>
#include <map>
#include <vector>

#include "pw_internal.h"
#include "pw_lbm.cuh"

using namespace pwhost;

namespace {

using pw::StepParams;

struct BatchSeg {
  uint32_t first;   // first global work index of this segment
  uint32_t member;
  uint32_t kind;    // 0 plain, 1 seam, 2 edge
  uint32_t count;
};

constexpr int kBatchThreads = pwbatch::NTHREADS;  // 128
constexpr int kChunk = 50;                        // steps per captured graph
// Seam rows per seam item (four per warp): an item's block barriers and its
// member's parameter load are shared by 16 rows, not 4 (0.7% faster on the
// 64-tunnel batch, whose seam rows are 5% of its cells on odd steps; the seam
// items in the plain kernel instead, under its register cap, no faster).
constexpr uint32_t kSeamRowsPerItem = 16;

// PLAIN: the plain items (PAIRS: through the 32-bit cell-pair kernel, which
// needs 16-bit storage and every member's nx even); otherwise
// the seam and edge items.
// The plain kernels are held to 72 registers (7 blocks per SM): the member's
// offset tables sit in shared memory and are reloaded rather than kept live.
// Measured on the 64-tunnel batch: 6 blocks (85 registers) 0.8% slower, 8
// blocks (64 registers, 140 bytes spilled per thread) 4% slower.
#ifndef PW_BATCH_PLAIN_BLOCKS
#define PW_BATCH_PLAIN_BLOCKS 7
#endif
template <int ST, int OP, bool LES, bool ODD, bool PLAIN, bool PAIRS>
__global__ void __launch_bounds__(kBatchThreads, PLAIN ? PW_BATCH_PLAIN_BLOCKS : 1) batch_step(const StepParams *params, const BatchSeg *segs,
                                                             const uint32_t *item_seg, uint32_t total,
                                                             const uint32_t *const *lists, const uint32_t *counts,
                                                             uint32_t rows) {
  __shared__ StepParams sp;
  __shared__ BatchSeg cur;
  const uint32_t tid = threadIdx.x;
  for (uint32_t w = blockIdx.x; w < total; w += gridDim.x) {
    __syncthreads();  // the previous item is done with sp
    if (tid == 0) cur = segs[__ldg(&item_seg[w])];
    __syncthreads();
    const uint32_t m = cur.member, local = w - cur.first, kind = cur.kind;
    {
      const uint32_t *src = reinterpret_cast<const uint32_t *>(&params[m]);
      uint32_t *dst = reinterpret_cast<uint32_t *>(&sp);
      for (uint32_t i = tid; i < sizeof(StepParams) / 4; i += kBatchThreads) dst[i] = src[i];
    }
    __syncthreads();
    if (PLAIN) {
      const uint32_t off = ODD ? 1u : 0u;
      const uint32_t runs = (sp.nx + 63u) / 64u;
      const uint32_t ny_rows = sp.ny - 2u * off;
      const uint32_t yblocks = (ny_rows + rows - 1u) / rows;
      const uint32_t run = local % runs, t = local / runs;
      const uint32_t yb = t % yblocks, zb = t / yblocks;
      for (uint32_t r = tid >> 5; r < rows; r += kBatchThreads / 32) {
        const uint32_t yr = yb * rows + r;
        if (yr >= ny_rows) continue;
        if constexpr (PAIRS && ST != pw::STORE_F32)
          pwbatch::pair_thread<ST, OP, LES, ODD>(sp, run * 64u + 2u * (tid & 31u), yr + off, zb + off);
        else
          pwbatch::plain_thread<ST, OP, LES, ODD>(sp, run * 64u + (tid & 31u), yr + off, zb + off);
      }
    } else if (kind == 1) {
      bool paired = false;
      if constexpr (PAIRS && ST != pw::STORE_F32) {
        if (sp.slip == 0u) {  // cell pairs with periodic wrap corrections
          paired = true;
          const uint32_t runs = (sp.nx + 63u) / 64u;
          const uint32_t run = local % runs, g = local / runs;
          for (uint32_t r = tid >> 5; r < kSeamRowsPerItem; r += kBatchThreads / 32)
            pwbatch::seam_pair_thread<ST, OP, LES>(sp, run * 64u + 2u * (tid & 31u), g * kSeamRowsPerItem + r);
        }
      }
      if (!paired) {
        const uint32_t runs = (sp.nx + 31u) / 32u;
        const uint32_t run = local % runs, g = local / runs;
        for (uint32_t r = tid >> 5; r < kSeamRowsPerItem; r += kBatchThreads / 32) {
          const uint32_t row = g * kSeamRowsPerItem + r;
          if (row < pwbatch::seam_rows(sp.ny, sp.nz)) pwbatch::seam_thread<ST, OP, LES>(sp, run * 32u + (tid & 31u), row);
        }
      }
    } else {
      pwbatch::edge_block<ST, OP, LES, ODD>(sp, lists[m], counts[m], local, tid);
    }
  }
}

template <int ST, int OP, bool LES>
void launch3(bool odd, bool plain, bool pairs, unsigned blocks, cudaStream_t s, const StepParams *params,
             const BatchSeg *segs, const uint32_t *item_seg, uint32_t total, const uint32_t *const *lists,
             const uint32_t *counts, uint32_t rows) {
#define PW_BATCH_LAUNCH(O, P, Q) \
  batch_step<ST, OP, LES, O, P, Q><<<blocks, kBatchThreads, 0, s>>>(params, segs, item_seg, total, lists, counts, rows)
  if (plain) {
    if (pairs && ST != pw::STORE_F32) {
      if (odd) PW_BATCH_LAUNCH(true, true, true);
      else PW_BATCH_LAUNCH(false, true, true);
    } else {
      if (odd) PW_BATCH_LAUNCH(true, true, false);
      else PW_BATCH_LAUNCH(false, true, false);
    }
  } else if (pairs && ST != pw::STORE_F32) {
    if (odd) PW_BATCH_LAUNCH(true, false, true);
    else PW_BATCH_LAUNCH(false, false, true);
  } else {
    if (odd) PW_BATCH_LAUNCH(true, false, false);
    else PW_BATCH_LAUNCH(false, false, false);
  }
#undef PW_BATCH_LAUNCH
}

template <int ST>
void launch2(int op, int les, bool odd, bool plain, bool pairs, unsigned blocks, cudaStream_t s,
             const StepParams *params, const BatchSeg *segs, const uint32_t *item_seg, uint32_t total,
             const uint32_t *const *lists, const uint32_t *counts, uint32_t rows) {
  if (op == pw::OP_REG) {
    if (les) launch3<ST, pw::OP_REG, true>(odd, plain, pairs, blocks, s, params, segs, item_seg, total, lists, counts, rows);
    else launch3<ST, pw::OP_REG, false>(odd, plain, pairs, blocks, s, params, segs, item_seg, total, lists, counts, rows);
  } else {
    if (les) launch3<ST, pw::OP_TRT, true>(odd, plain, pairs, blocks, s, params, segs, item_seg, total, lists, counts, rows);
    else launch3<ST, pw::OP_TRT, false>(odd, plain, pairs, blocks, s, params, segs, item_seg, total, lists, counts, rows);
  }
}

}  // namespace

struct pw_batch {
  std::vector<pw_domain *> members;
  int storage = 0, op = 0, les = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  std::vector<cudaEvent_t> member_ready;
  // [parity][write_macro] member parameter arrays; [parity][plain items, seam and
  // edge items] work segments
  StepParams *params[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
  BatchSeg *segs[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
  // the segment of every work item, so a block finds its item's member with
  // one load instead of a search over the segments
  uint32_t *item_seg[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
  uint32_t total[2][2] = {{0, 0}, {0, 0}};
  cudaStream_t side = nullptr;    // the seam and edge items, beside the plain items
  cudaEvent_t fork = nullptr, join = nullptr;
  unsigned sms = 1;               // multiprocessors of the device
  bool pairs = false;             // every member's nx is even: the plain items use the cell-pair kernel
  const uint32_t **lists = nullptr;
  uint32_t *counts = nullptr;
  uint32_t rows = 4;       // plain rows per work item
  unsigned blocks = 0;     // persistent grid
  uint64_t steps = 0;
  std::map<std::pair<int, int>, cudaGraphExec_t> graphs;
};

namespace {

void drop_graphs(pw_batch *b) {
  for (auto &kv : b->graphs) cudaGraphExecDestroy(kv.second);
  b->graphs.clear();
}

// Work segments of both parities for the current rows-per-item.
int build_segments(pw_batch *b) {
  for (int par = 0; par < 2; par++) {
    std::vector<BatchSeg> segs[2];
    uint32_t first[2] = {0, 0};
    for (uint32_t m = 0; m < b->members.size(); m++) {
      const MemberView v = member_view(b->members[m]);
      const uint32_t off = par ? 1u : 0u;
      const uint32_t runs = (v.nx + 63u) / 64u;
      const uint32_t nyr = v.ny > 2u * off ? v.ny - 2u * off : 0u, nzr = v.nz > 2u * off ? v.nz - 2u * off : 0u;
      const uint32_t plain = v.nx >= 3u ? runs * ((nyr + b->rows - 1u) / b->rows) * nzr : 0u;
      // seam items: kSeamRowsPerItem rows of 64 cells as cell pairs (16-bit
      // storage, nx even, periodic faces), else of 32 cells one per thread
      const bool paired = b->pairs && v.storage != pw::STORE_F32 && v.slip == 0u;
      const uint32_t seam_run = paired ? 64u : 32u;
      const uint32_t seam = par && v.nx >= 3u ? ((v.nx + seam_run - 1u) / seam_run) *
                                                    ((pwbatch::seam_rows(v.ny, v.nz) + kSeamRowsPerItem - 1u) /
                                                     kSeamRowsPerItem)
                                              : 0u;
      const uint32_t edge = (v.edge_count + kBatchThreads - 1u) / kBatchThreads;
      const uint32_t kinds[3] = {plain, seam, edge};
      for (uint32_t k = 0; k < 3; k++) {
        if (!kinds[k]) continue;
        const int list = k == 0 ? 0 : 1;
        segs[list].push_back(BatchSeg{first[list], m, k, kinds[k]});
        first[list] += kinds[k];
      }
    }
    for (int list = 0; list < 2; list++) {
      if (segs[list].empty()) segs[list].push_back(BatchSeg{0, 0, (uint32_t)list, 0});
      cudaFree(b->segs[par][list]);
      b->segs[par][list] = nullptr;
      PW_TRY(cudaMalloc(&b->segs[par][list], segs[list].size() * sizeof(BatchSeg)));
      PW_TRY(cudaMemcpy(b->segs[par][list], segs[list].data(), segs[list].size() * sizeof(BatchSeg),
                        cudaMemcpyHostToDevice));
      std::vector<uint32_t> table(std::max<uint32_t>(1u, first[list]), 0u);
      for (uint32_t k = 0; k < segs[list].size(); k++)
        for (uint32_t i = 0; i < segs[list][k].count; i++) table[segs[list][k].first + i] = k;
      cudaFree(b->item_seg[par][list]);
      b->item_seg[par][list] = nullptr;
      PW_TRY(cudaMalloc(&b->item_seg[par][list], table.size() * sizeof(uint32_t)));
      PW_TRY(cudaMemcpy(b->item_seg[par][list], table.data(), table.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
      b->total[par][list] = first[list];
    }
  }
  return PW_OK;
}

// Member parameters of both parities, with and without the macro write.  The
// partial, plane and offset fields depend only on the parity, so one set per
// parity serves every step of the batch.
int upload_params(pw_batch *b) {
  const size_t n = b->members.size();
  std::vector<StepParams> host(n);
  for (int par = 0; par < 2; par++) {
    for (int macro = 0; macro < 2; macro++) {
      for (size_t m = 0; m < n; m++) host[m] = member_params(b->members[m], 2 + (uint64_t)par, macro);
      PW_TRY(cudaMemcpy(b->params[par][macro], host.data(), n * sizeof(StepParams), cudaMemcpyHostToDevice));
    }
  }
  return PW_OK;
}

void launch_items(pw_batch *b, bool odd, int macro, bool plain, unsigned blocks, cudaStream_t s) {
  const int par = odd ? 1 : 0, list = plain ? 0 : 1;
  const StepParams *params = b->params[par][macro];
  const BatchSeg *segs = b->segs[par][list];
  const uint32_t *item_seg = b->item_seg[par][list];
  const uint32_t total = b->total[par][list];
  switch (b->storage) {
    case pw::STORE_F16:
      launch2<pw::STORE_F16>(b->op, b->les, odd, plain, b->pairs, blocks, s, params, segs, item_seg, total, b->lists,
                             b->counts, b->rows);
      break;
    case pw::STORE_BF16:
      launch2<pw::STORE_BF16>(b->op, b->les, odd, plain, b->pairs, blocks, s, params, segs, item_seg, total, b->lists,
                              b->counts, b->rows);
      break;
    default:
      launch2<pw::STORE_F32>(b->op, b->les, odd, plain, b->pairs, blocks, s, params, segs, item_seg, total, b->lists,
                             b->counts, b->rows);
      break;
  }
}

void enqueue(pw_batch *b, bool odd, int macro) {
  const int par = odd ? 1 : 0;
  if (macro)
    for (pw_domain *d : b->members) cudaMemsetAsync(member_view(d).status, 0, 4, b->stream);
  const uint32_t rest = b->total[par][1];
  if (rest) {
    // seam and edge items on the side stream, forked from and joined back to the batch stream
    cudaEventRecord(b->fork, b->stream);
    cudaStreamWaitEvent(b->side, b->fork, 0);
    const unsigned rblocks = std::max(1u, std::min<unsigned>(rest, b->sms * 8u));
    launch_items(b, odd, macro, false, rblocks, b->side);
  }
  const unsigned blocks = std::max(1u, std::min<unsigned>(b->blocks, std::max(1u, b->total[par][0])));
  if (b->total[par][0]) launch_items(b, odd, macro, true, blocks, b->stream);
  if (rest) {
    cudaEventRecord(b->join, b->side);
    cudaStreamWaitEvent(b->stream, b->join, 0);
  }
}

cudaGraphExec_t graph_for(pw_batch *b, int start_parity, int macro_last) {
  auto key = std::make_pair(start_parity, macro_last);
  auto it = b->graphs.find(key);
  if (it != b->graphs.end()) return it->second;
  cudaStream_t cap;
  if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess) { cudaGetLastError(); return nullptr; }
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t saved = b->stream;
  b->stream = cap;
  if (cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
    for (int k = 0; k < kChunk; k++) enqueue(b, ((start_parity + k) & 1) != 0, macro_last && k == kChunk - 1);
    if (cudaStreamEndCapture(cap, &graph) == cudaSuccess && graph) {
      if (cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) exec = nullptr;
      cudaGraphDestroy(graph);
    }
  }
  b->stream = saved;
  cudaStreamDestroy(cap);
  cudaGetLastError();
  if (exec) b->graphs[key] = exec;
  return exec;
}

// Order the batch stream after each member's queued work, and each member's
// stream after the batch's.
void members_to_batch(pw_batch *b) {
  for (size_t m = 0; m < b->members.size(); m++) {
    cudaEventRecord(b->member_ready[m], member_view(b->members[m]).stream);
    cudaStreamWaitEvent(b->stream, b->member_ready[m], 0);
  }
}
void batch_to_members(pw_batch *b) {
  cudaEventRecord(b->done, b->stream);
  for (pw_domain *d : b->members) cudaStreamWaitEvent(member_view(d).stream, b->done, 0);
}

int queue_steps(pw_batch *b, uint64_t count, int macro_last) {
  uint64_t k = 0;
  while (count - k >= (uint64_t)kChunk) {
    const int macro = macro_last && count - k == (uint64_t)kChunk;
    cudaGraphExec_t g = graph_for(b, (int)((b->steps + 1) & 1), macro);
    if (!g) break;
    if (cudaGraphLaunch(g, b->stream) != cudaSuccess) { cudaGetLastError(); break; }
    b->steps += kChunk;
    k += kChunk;
  }
  for (; k < count; k++) {
    enqueue(b, ((b->steps + 1) & 1) != 0, macro_last && k == count - 1);
    b->steps++;
  }
  PW_TRY(cudaGetLastError());
  return PW_OK;
}

int max_blocks() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return std::max(1, sms);
}

}  // namespace

extern "C" {

int pw_batch_create(pw_domain *const *members, uint32_t count, pw_batch **out) {
  if (!members || !out || count == 0) { set_error("A batch needs at least one member domain."); return PW_ERR_INVALID; }
  *out = nullptr;
  MemberView first = member_view(members[0]);
  for (uint32_t m = 0; m < count; m++) {
    if (!members[m]) { set_error("NULL member domain."); return PW_ERR_INVALID; }
    for (uint32_t k = 0; k < m; k++)
      if (members[k] == members[m]) { set_error("A domain can join a batch only once."); return PW_ERR_INVALID; }
    const MemberView v = member_view(members[m]);
    if (!v.split) {
      set_error("Batch members must use the fast build's one-cell-per-thread kernels (strict = 0, kernel AUTO/CELL).");
      return PW_ERR_INVALID;
    }
    if (v.closure) {
      set_error("Batch members cannot have a learned closure attached.");
      return PW_ERR_INVALID;
    }
    if (v.storage != first.storage || v.op != first.op || v.les != first.les) {
      set_error("Batch members must share storage, collision operator and LES.");
      return PW_ERR_INVALID;
    }
    if (v.interpolated) {
      set_error("Batch members must use halfway bounce-back walls.");
      return PW_ERR_INVALID;
    }
    if (v.steps != first.steps) { set_error("Batch members must have taken the same number of steps."); return PW_ERR_INVALID; }
    if (v.ramping) { set_error("Batch members must have finished their inlet ramp."); return PW_ERR_INVALID; }
  }
  pw_batch *b = new pw_batch();
  b->members.assign(members, members + count);
  b->pairs = true;
  for (uint32_t m = 0; m < count; m++) b->pairs = b->pairs && (member_view(members[m]).nx & 1u) == 0u;
  b->storage = first.storage; b->op = first.op; b->les = first.les;
  b->steps = first.steps;
  b->sms = (unsigned)max_blocks();
  b->blocks = b->sms * 4u;
  auto fail = [&](int rc) {
    pw_batch_destroy(b);
    return rc;
  };
  cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  int lo_prio = 0, hi_prio = 0;
  if (e == cudaSuccess) e = cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio);
  if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&b->side, cudaStreamNonBlocking, hi_prio);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming);
  b->member_ready.assign(count, nullptr);
  for (uint32_t m = 0; m < count && e == cudaSuccess; m++)
    e = cudaEventCreateWithFlags(&b->member_ready[m], cudaEventDisableTiming);
  for (int par = 0; par < 2 && e == cudaSuccess; par++)
    for (int macro = 0; macro < 2 && e == cudaSuccess; macro++)
      e = cudaMalloc(&b->params[par][macro], count * sizeof(StepParams));
  if (e == cudaSuccess) e = cudaMalloc((void **)&b->lists, count * sizeof(uint32_t *));
  if (e == cudaSuccess) e = cudaMalloc((void **)&b->counts, count * sizeof(uint32_t));
  if (e != cudaSuccess) return fail(cuda_status(e, "pw_batch_create"));
  std::vector<const uint32_t *> lists(count);
  std::vector<uint32_t> counts(count);
  for (uint32_t m = 0; m < count; m++) {
    const MemberView v = member_view(members[m]);
    lists[m] = v.edges;
    counts[m] = v.edge_count;
  }
  e = cudaMemcpy(b->lists, lists.data(), count * sizeof(uint32_t *), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b->counts, counts.data(), count * sizeof(uint32_t), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return fail(cuda_status(e, "pw_batch_create"));
  int rc = upload_params(b);
  if (rc == PW_OK) rc = build_segments(b);
  if (rc != PW_OK) return fail(rc);
  *out = b;
  return PW_OK;
}

void pw_batch_destroy(pw_batch *b) {
  if (!b) return;
  if (b->stream) cudaStreamSynchronize(b->stream);
  drop_graphs(b);
  for (int par = 0; par < 2; par++) {
    for (int macro = 0; macro < 2; macro++) cudaFree(b->params[par][macro]);
    for (int list = 0; list < 2; list++) {
      cudaFree(b->segs[par][list]);
      cudaFree(b->item_seg[par][list]);
    }
  }
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->join) cudaEventDestroy(b->join);
  if (b->side) cudaStreamDestroy(b->side);
  cudaFree(b->lists);
  cudaFree(b->counts);
  for (cudaEvent_t ev : b->member_ready)
    if (ev) cudaEventDestroy(ev);
  if (b->done) cudaEventDestroy(b->done);
  if (b->stream) cudaStreamDestroy(b->stream);
  cudaGetLastError();
  delete b;
}

int pw_batch_step(pw_batch *b, uint64_t count, int write_macro_on_last) {
  if (!b) { set_error("The batch handle is NULL."); return PW_ERR_INVALID; }
  for (pw_domain *d : b->members)
    if (member_view(d).steps != b->steps) {
      set_error("A batch member was stepped on its own; members must step only through the batch.");
      return PW_ERR_INVALID;
    }
  if (count == 0) return PW_OK;
  members_to_batch(b);
  int rc = queue_steps(b, count, write_macro_on_last);
  batch_to_members(b);
  for (pw_domain *d : b->members) member_advance(d, count);
  return rc;
}

int pw_batch_time_steps(pw_batch *b, uint64_t count, float *ms) {
  if (!b || !ms) { set_error("NULL argument"); return PW_ERR_INVALID; }
  cudaEvent_t t0, t1;
  PW_TRY(cudaEventCreate(&t0));
  PW_TRY(cudaEventCreate(&t1));
  members_to_batch(b);
  cudaEventRecord(t0, b->stream);
  int rc = PW_OK;
  for (pw_domain *d : b->members)
    if (member_view(d).steps != b->steps) rc = PW_ERR_INVALID;
  if (rc == PW_OK) rc = queue_steps(b, count, 0);
  cudaEventRecord(t1, b->stream);
  batch_to_members(b);
  if (rc == PW_OK)
    for (pw_domain *d : b->members) member_advance(d, count);
  cudaError_t e = cudaEventSynchronize(t1);
  if (e == cudaSuccess) e = cudaEventElapsedTime(ms, t0, t1);
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  if (rc != PW_OK) { set_error("A batch member was stepped on its own."); return rc; }
  if (e != cudaSuccess) return cuda_status(e, "pw_batch_time_steps");
  return PW_OK;
}

// Time every candidate launch shape (persistent grid of 2, 4, 8, 16 or 32 blocks
// per SM, and 8, 16, 32 or 64 plain rows per work item) over `trial_steps` real
// steps each (an even number, after two warm-up steps) and keep the fastest.
// The trial steps advance the members.
int pw_batch_tune(pw_batch *b, uint32_t trial_steps, pw_batch_tuning *out) {
  if (!b || trial_steps == 0) { set_error("The batch handle is NULL or the trial has no steps."); return PW_ERR_INVALID; }
  trial_steps += trial_steps & 1u;
  const unsigned sms = (unsigned)max_blocks();
  const unsigned grid_mult[] = {2, 4, 8, 16, 32};
  const uint32_t row_opts[] = {8, 16, 32, 64};
  float best = 1e30f;
  unsigned best_blocks = b->blocks;
  uint32_t best_rows = b->rows, tried = 0;
  for (uint32_t rows : row_opts) {
    b->rows = rows;
    drop_graphs(b);
    int rc = build_segments(b);
    if (rc != PW_OK) return rc;
    for (unsigned g : grid_mult) {
      b->blocks = sms * g;
      drop_graphs(b);
      rc = pw_batch_step(b, 2, 0);
      if (rc != PW_OK) return rc;
      float ms = 0.0f;
      rc = pw_batch_time_steps(b, trial_steps, &ms);
      if (rc != PW_OK) return rc;
      tried++;
      if (ms < best) { best = ms; best_blocks = b->blocks; best_rows = rows; }
    }
  }
  b->rows = best_rows;
  b->blocks = best_blocks;
  drop_graphs(b);
  int rc = build_segments(b);
  if (rc != PW_OK) return rc;
  if (out) {
    out->blocks = best_blocks;
    out->rows_per_item = best_rows;
    out->ms_per_step = best / (float)trial_steps;
    out->candidates = tried;
  }
  return PW_OK;
}

int pw_batch_reset(pw_batch *b) {
  if (!b) { set_error("The batch handle is NULL."); return PW_ERR_INVALID; }
  members_to_batch(b);
  PW_TRY(cudaStreamSynchronize(b->stream));
  for (pw_domain *d : b->members) {
    int rc = pw_reset(d);
    if (rc != PW_OK) return rc;
  }
  b->steps = 0;
  return PW_OK;
}

}  // extern "C"
