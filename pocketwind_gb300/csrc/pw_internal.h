// Internal host-side definitions shared by the C-ABI translation units.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>

#include "../../include/pocketwind.h"
#include "pw_common.cuh"

namespace pwhost {

void set_error(const char *fmt, ...);
int cuda_status(cudaError_t e, const char *what);  // PW_ERR_OOM / PW_ERR_CUDA with message

#define PW_TRY(call)                                           \
  do {                                                         \
    cudaError_t e_ = (call);                                   \
    if (e_ != cudaSuccess) return pwhost::cuda_status(e_, #call); \
  } while (0)

void domain_dims(const pw_domain *d, uint32_t *nx, uint32_t *ny, uint32_t *nz);

// Read-only view of a domain's device state for kernels outside pw_domain.cu.
struct DomainView {
  void *f;
  const uint32_t *flags;
  uint32_t nx, ny, nz, stride;
  uint64_t steps;
  int storage;
  cudaStream_t stream;
  uint32_t slip;  // free-slip faces (bit 0 y, bit 1 z)
  int device;     // the device the domain was created on
};
DomainView domain_view(const pw_domain *d);
// Load the allocation-free readout's code and fixed array onto the current
// device and look up the array's address (pw_noalloc.cu).  pw_domain_create
// calls it, so that the readout itself never loads a module later, when the
// device's memory may already be taken.  Failures are left for the readout
// to report.
void noalloc_prepare_device();

// What a batch needs of a member domain (pw_batch.cu).
struct MemberView {
  bool split;                // fast build, one cell per thread (plain kernels + edge list)
  bool closure;              // a learned closure is attached
  int storage, op, les;
  uint32_t nx, ny, nz;
  uint64_t steps;
  bool ramping;              // inlet ramp still in progress
  bool interpolated;         // interpolated (Bouzidi) walls
  uint32_t slip;             // free-slip faces (bit 0 y, bit 1 z)
  const uint32_t *edges;
  uint32_t edge_count;
  uint32_t *status;
  cudaStream_t stream;
};
MemberView member_view(const pw_domain *d);
// The step parameters of step `step` (1-based) at the domain's full inlet speed.
pw::StepParams member_params(const pw_domain *d, uint64_t step, int write_macro);
// Count `n` steps run for the domain by a batch.
void member_advance(pw_domain *d, uint64_t n);

// Device-resident packed geometry (the reference's VoxelGrid).
struct Grid {
  uint32_t nx = 0, ny = 0, nz = 0;
  size_t cells = 0;
  uint32_t *flags = nullptr;      // cells
  uint32_t *qoff = nullptr;       // cells
  float *fractions = nullptr;     // nfrac
  uint32_t *boundary = nullptr;   // nboundary
  size_t nfrac = 0, nboundary = 0;
  pw_grid_stats stats{};
  ~Grid();
};

// Allocation helper: frees everything it handed out unless released.
struct Allocs {
  void *ptrs[32];
  int n = 0;
  bool keep = false;
  cudaError_t alloc(void **p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
    if (e == cudaSuccess) ptrs[n++] = *p;
    return e;
  }
  ~Allocs() {
    if (!keep)
      for (int i = 0; i < n; i++) cudaFree(ptrs[i]);
  }
};

}  // namespace pwhost

struct pw_grid : pwhost::Grid {};
