// Population readout that allocates no device memory.
//
// pw_read_populations turns the in-place layout into direction-major order in a
// device buffer as large as the whole state, which it allocates on first use
// (19 x cells x 4 bytes: 2.5 GB for the 33.5 M-cell tunnel).  Some callers cannot
// allocate at that point: a host that has already given nearly all of the GPU's
// memory to its domains (a 33.5 M-cell f32 domain plus other tenants on the same
// device leaves no room for another 2.5 GB), and hosts whose device memory is
// budgeted once up front by an embedding runtime, as pocketwind's browser tiers
// budget theirs (src/lbm/tier-probe.ts), so that a mid-run allocation is not
// allowed.  For them this file converts the state one direction and a slab of
// z-planes at a time through a fixed 4 MiB array that lives in the library's
// own device image (a file-scope __device__ array), so the readout needs no
// cudaMalloc, cudaFree or allocating library call.
//
// Limits and sharing:
//   - one x-y plane of one direction (nx * ny * 4 bytes) must fit in the 4 MiB
//     array, i.e. nx * ny <= 1,048,576 cells; larger planes are rejected;
//   - CUDA loads a module's code and its __device__ arrays lazily, on first
//     use, and that load takes device memory.  So creating a domain
//     (pw_domain_create) loads this file's readout kernels and array onto its
//     device and looks up the array's device address for that device
//     (cudaGetSymbolAddress, with that device current): the readout itself
//     then loads nothing.  The readout's own first call on a device repeats
//     the lookup only if that preparation failed; it should come before any
//     stream capture;
//   - the domain's device must be current when the readout is called;
//   - every call shares the array and leaves the last call's slab in it; two
//     calls that overlap on the GPU (from different threads or streams) race.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "pw_internal.h"

#define PW_NS pwnoalloc
#include "pw_lbm.cuh"
#undef PW_NS

using namespace pwhost;

namespace {

constexpr size_t kScratchBytes = (size_t)4 << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_readout_scratch[kScratchBytes];

std::mutex g_mutex;
void *g_scratch_addr[kMaxDevices] = {};

// Device address of g_readout_scratch on the current device, looked up once per device.
int scratch_address(void **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_status(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("device ordinal %d is outside the readout table", dev);
    return PW_ERR_CUDA;
  }
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_scratch_addr[dev]) {
    void *addr = nullptr;
    e = cudaGetSymbolAddress(&addr, g_readout_scratch);
    if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(g_readout_scratch)");
    g_scratch_addr[dev] = addr;
  }
  *out = g_scratch_addr[dev];
  return PW_OK;
}

// The readout kernel (pwfast/pwstrict aa_read) restricted to one direction j and
// the z-planes [z0, z0 + gridDim.z), writing decoded deviations into `slab`.
template <int ST>
__global__ void read_slab_kernel(pw::StepParams p, int odd_layout, int j, uint32_t z0, float *slab) {
  using S = pw::Store<ST>;
  using T = typename S::T;
  const T *f = reinterpret_cast<const T *>(p.f);
  const uint32_t x = blockIdx.x * pwnoalloc::BX + threadIdx.x;
  const uint32_t y = blockIdx.y * pwnoalloc::BY + threadIdx.y;
  const uint32_t z = z0 + blockIdx.z;
  if (x >= p.nx || y >= p.ny) return;
  const uint32_t n = x + p.nx * (y + p.ny * z);
  float v = 0.0f;
  if (!pw::is_wall_kind(p.flags[n] & 7u)) {
    const pwnoalloc::Nbr b = pwnoalloc::make_nbr(p, x, y, z);
    pw::pidx k = odd_layout ? pwnoalloc::slot_of<true>(b, j, p.stride, n)
                            : pwnoalloc::slot_of<false>(b, j, p.stride, n);
    v = S::decode(f[k]);
  }
  slab[(size_t)blockIdx.z * p.nx * p.ny + x + (size_t)p.nx * y] = v;
}

// Force the lazy loader to bring in the three readout kernels now.
cudaError_t load_readout_kernels() {
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, read_slab_kernel<pw::STORE_F32>);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, read_slab_kernel<pw::STORE_F16>);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, read_slab_kernel<pw::STORE_BF16>);
  return e;
}

}  // namespace

namespace pwhost {
void noalloc_prepare_device() {
  void *addr = nullptr;
  if (load_readout_kernels() != cudaSuccess || scratch_address(&addr) != PW_OK) cudaGetLastError();
}
}  // namespace pwhost

extern "C" {

int pw_read_populations_noalloc(pw_domain *dom, float *out) {
  if (!dom || !out) { set_error("NULL argument"); return PW_ERR_INVALID; }
  DomainView v = domain_view(dom);
  const size_t plane = (size_t)v.nx * v.ny;
  const size_t plane_bytes = plane * sizeof(float);
  if (plane_bytes > kScratchBytes) {
    set_error("pw_read_populations_noalloc: an x-y plane of %zu cells needs %zu bytes, more than its "
              "fixed %zu-byte readout array holds (nx * ny must be at most %zu)",
              plane, plane_bytes, kScratchBytes, kScratchBytes / sizeof(float));
    return PW_ERR_INVALID;
  }
  int current = -1;
  PW_TRY(cudaGetDevice(&current));
  if (current != v.device) {
    set_error("pw_read_populations_noalloc: the domain lives on device %d but device %d is current; make the "
              "domain's device current first", v.device, current);
    return PW_ERR_INVALID;
  }
  void *scratch = nullptr;
  int rc = scratch_address(&scratch);
  if (rc != PW_OK) return rc;
  pw::StepParams p{};
  p.f = v.f;
  p.flags = v.flags;
  p.nx = v.nx; p.ny = v.ny; p.nz = v.nz;
  p.stride = v.stride;
  p.slip = v.slip;
  const int odd = (int)(v.steps & 1);
  const size_t cells = plane * v.nz;
  const uint32_t zc = (uint32_t)std::min<size_t>(v.nz, kScratchBytes / plane_bytes);
  const dim3 block(pwnoalloc::BX, pwnoalloc::BY);
  for (int j = 0; j < 19; j++) {
    for (uint32_t z0 = 0; z0 < v.nz; z0 += zc) {
      uint32_t nzs = std::min<uint32_t>(zc, v.nz - z0);
      dim3 grid((v.nx + pwnoalloc::BX - 1) / pwnoalloc::BX, (v.ny + pwnoalloc::BY - 1) / pwnoalloc::BY, nzs);
      float *slab = reinterpret_cast<float *>(scratch);
      switch (v.storage) {
        case PW_STORE_F16: read_slab_kernel<pw::STORE_F16><<<grid, block, 0, v.stream>>>(p, odd, j, z0, slab); break;
        case PW_STORE_BF16: read_slab_kernel<pw::STORE_BF16><<<grid, block, 0, v.stream>>>(p, odd, j, z0, slab); break;
        default: read_slab_kernel<pw::STORE_F32><<<grid, block, 0, v.stream>>>(p, odd, j, z0, slab); break;
      }
      PW_TRY(cudaGetLastError());
      PW_TRY(cudaMemcpyAsync(out + (size_t)j * cells + (size_t)z0 * plane, slab, nzs * plane_bytes,
                             cudaMemcpyDeviceToHost, v.stream));
      // the next slab reuses the array: wait for this copy first
      PW_TRY(cudaStreamSynchronize(v.stream));
    }
  }
  return PW_OK;
}

}  // extern "C"
