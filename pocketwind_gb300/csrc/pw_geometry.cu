// GPU voxelizer and packed-geometry validation (compiled with -fmad=false so every
// binary64 edge function and hit depth rounds exactly as the reference computes it).
//
// Follows src/geometry/voxelize.ts:1-199 and src/geometry/wall-links.ts:1-131:
//   per projection (u, v, axis) in {(x,y,z), (y,z,x), (z,x,y)}: rasterize every
//   triangle onto integer (u, v) columns with the half-open edge rule, collect the
//   hit depths per column, sort them, fill [ceil(h0), ceil(h1)) spans into a vote;
//   a cell is the mesh's kind when two of three projections agree and it is still
//   fluid (body before supports); then EQ x faces, FLOOR/EQ z faces, counts,
//   pull-direction wall masks, q offsets (halfway fractions) and the ascending
//   list of fluid cells next to the body.
// GPU shape: one block per triangle (threads stride over its pixel box) for the
// counting and filling passes, one thread per column for sort-and-fill, one
// thread per cell for the rest; prefix sums give CSR column offsets, q offsets and
// the boundary list in cell order.
#include <cuda_runtime.h>
#include <math_constants.h>

#include <cmath>
#include <cstdarg>
#include <cstring>
#include <vector>

#include "pw_internal.h"

namespace pwhost {

static thread_local std::string g_error;

void set_error(const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_error = buf;
}

const char *last_error() { return g_error.c_str(); }

int cuda_status(cudaError_t e, const char *what) {
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    set_error("device allocation failed (%s)", what);
    return PW_ERR_OOM;
  }
  set_error("CUDA error %s in %s", cudaGetErrorString(e), what);
  return PW_ERR_CUDA;
}

// Temporaries of one voxelization come from the stream-ordered pool: freeing
// one never waits for the whole device, and the pool keeps up to 256 MB mapped
// between calls.
static cudaError_t tmp_alloc(void *p, size_t bytes, cudaStream_t s) {
  static bool pool_set = false;
  if (!pool_set) {
    int dev = 0;
    cudaMemPool_t pool;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      uint64_t keep = 256ull << 20;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    cudaGetLastError();
    pool_set = true;
  }
  return cudaMallocAsync(reinterpret_cast<void **>(p), bytes, s);
}
static void tmp_free(void *p, cudaStream_t s) {
  if (p) cudaFreeAsync(p, s);
}

Grid::~Grid() {
  cudaFree(flags);
  cudaFree(qoff);
  cudaFree(fractions);
  cudaFree(boundary);
}

// ------------------------------------------------------------------ scan
// Exclusive prefix sum of n uint32 values (in place into out), total returned.
__global__ void scan_blocks(const uint32_t *in, uint32_t *out, uint32_t *block_sums, size_t n) {
  __shared__ uint32_t sh[1024];
  size_t base = (size_t)blockIdx.x * 4096;
  uint32_t v[4];
  uint32_t local = 0;
  for (int k = 0; k < 4; k++) {
    size_t i = base + threadIdx.x * 4 + k;
    v[k] = i < n ? in[i] : 0u;
    local += v[k];
  }
  sh[threadIdx.x] = local;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    uint32_t t = threadIdx.x >= (unsigned)off ? sh[threadIdx.x - off] : 0u;
    __syncthreads();
    sh[threadIdx.x] += t;
    __syncthreads();
  }
  uint32_t run = sh[threadIdx.x] - local;
  for (int k = 0; k < 4; k++) {
    size_t i = base + threadIdx.x * 4 + k;
    if (i < n) out[i] = run;
    run += v[k];
  }
  if (threadIdx.x == 1023) block_sums[blockIdx.x] = sh[1023];
}

__global__ void scan_add(uint32_t *out, const uint32_t *block_offsets, size_t n) {
  size_t i = (size_t)blockIdx.x * 4096 + threadIdx.x;
  for (int k = 0; k < 4; k++, i += 1024)
    if (i < n) out[i] += block_offsets[blockIdx.x];
}

static int exclusive_scan(const uint32_t *in, uint32_t *out, size_t n, uint64_t *total, cudaStream_t s) {
  if (n == 0) { *total = 0; return PW_OK; }
  size_t blocks = (n + 4095) / 4096;
  uint32_t *sums = nullptr, *offs = nullptr;
  PW_TRY(tmp_alloc(&sums, (blocks + 1) * sizeof(uint32_t), s));
  cudaError_t e = tmp_alloc(&offs, (blocks + 1) * sizeof(uint32_t), s);
  if (e != cudaSuccess) { tmp_free(sums, s); return cuda_status(e, "scan"); }
  scan_blocks<<<(unsigned)blocks, 1024, 0, s>>>(in, out, sums, n);
  int rc = PW_OK;
  if (blocks > 1) {
    uint64_t sub = 0;
    rc = exclusive_scan(sums, offs, blocks, &sub, s);
    if (rc == PW_OK) scan_add<<<(unsigned)blocks, 1024, 0, s>>>(out, offs, n);
  }
  // total = last exclusive value + last input
  uint32_t last_out = 0, last_in = 0;
  if (rc == PW_OK) {
    e = cudaMemcpyAsync(&last_out, out + n - 1, 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&last_in, in + n - 1, 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) rc = cuda_status(e, "scan total");
  }
  tmp_free(sums, s);
  tmp_free(offs, s);
  *total = (uint64_t)last_out + last_in;
  return rc;
}

// ------------------------------------------------------------------ raster
struct Proj { int u, v, axis; uint32_t su, sv, sa; size_t stu, stv, sta; };

__device__ __forceinline__ double edge_fn(const double *a, const double *b, double u, double v) {
  return (b[0] - a[0]) * (v - a[1]) - (b[1] - a[1]) * (u - a[0]);
}

__device__ __forceinline__ bool owns_edge(double value, const double *a, const double *b) {
  return value > 0 || (value == 0 && (b[1] < a[1] || (b[1] == a[1] && b[0] > a[0])));
}

// mode 0: count hits per column; mode 1: write hit depths at cursor positions.
__global__ void raster_kernel(const float *mesh, Proj P, uint32_t *count, const uint32_t *offset,
                              uint32_t *cursor, double *hits, int mode) {
  const float *q = mesh + 9 * (size_t)blockIdx.x;
  double A[3] = {q[P.u], q[P.v], q[P.axis]};
  double B0[3] = {q[3 + P.u], q[3 + P.v], q[3 + P.axis]};
  double C0[3] = {q[6 + P.u], q[6 + P.v], q[6 + P.axis]};
  double signed_area = edge_fn(A, B0, C0[0], C0[1]);
  if (signed_area == 0) return;
  const double *B = signed_area > 0 ? B0 : C0;
  const double *C = signed_area > 0 ? C0 : B0;
  double area = fabs(signed_area);
  double lu = ceil(fmin(fmin(A[0], B[0]), C[0])), hu = floor(fmax(fmax(A[0], B[0]), C[0]));
  double lv = ceil(fmin(fmin(A[1], B[1]), C[1])), hv = floor(fmax(fmax(A[1], B[1]), C[1]));
  lu = fmax(0.0, lu); lv = fmax(0.0, lv);
  hu = fmin((double)P.su - 1.0, hu); hv = fmin((double)P.sv - 1.0, hv);
  if (lu > hu || lv > hv) return;
  long long u0 = (long long)lu, v0 = (long long)lv;
  long long w = (long long)hu - u0 + 1, h = (long long)hv - v0 + 1;
  for (long long k = threadIdx.x; k < w * h; k += blockDim.x) {
    long long u = u0 + k % w, v = v0 + k / w;
    double wa = edge_fn(B, C, (double)u, (double)v);
    double wb = edge_fn(C, A, (double)u, (double)v);
    double wc = edge_fn(A, B, (double)u, (double)v);
    if (owns_edge(wa, B, C) && owns_edge(wb, C, A) && owns_edge(wc, A, B)) {
      size_t col = (size_t)u + (size_t)P.su * (size_t)v;
      if (mode == 0) {
        atomicAdd(&count[col], 1u);
      } else {
        uint32_t at = atomicAdd(&cursor[col], 1u);
        hits[offset[col] + at] = (wa * A[2] + wb * B[2] + wc * C[2]) / area;
      }
    }
  }
}

__global__ void column_kernel(Proj P, const uint32_t *count, const uint32_t *offset, double *hits,
                              uint8_t *votes, uint32_t *closed) {
  size_t col = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= (size_t)P.su * P.sv) return;
  uint32_t n = count[col];
  if (n == 0) return;
  double *h = hits + offset[col];
  for (uint32_t i = 1; i < n; i++) {  // insertion sort: columns hold few hits
    double key = h[i];
    int j = (int)i - 1;
    while (j >= 0 && h[j] > key) { h[j + 1] = h[j]; j--; }
    h[j + 1] = key;
  }
  if (n % 2) *closed = 0u;
  size_t base = (col % P.su) * P.stu + (col / P.su) * P.stv;
  for (uint32_t pair = 0; pair + 1 < n; pair += 2) {
    double s0 = fmax(0.0, ceil(h[pair]));
    double s1 = fmin((double)P.sa, ceil(h[pair + 1]));
    for (long long c = (long long)s0; c < (long long)s1; c++) votes[base + (size_t)c * P.sta]++;
  }
}

__global__ void classify_kernel(const uint8_t *votes, uint32_t *flags, size_t cells, uint32_t type) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < cells && votes[i] >= 2 && flags[i] == pw::FLUID) flags[i] = type;
}

// voxelize.ts:123-135 (x faces, then the floor plane and the top plane)
__global__ void boundary_kernel(uint32_t *flags, uint32_t nx, uint32_t ny, uint32_t nz, int floor_on) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  size_t cells = (size_t)nx * ny * nz;
  if (i >= cells) return;
  uint32_t x = (uint32_t)(i % nx);
  uint32_t z = (uint32_t)(i / ((size_t)nx * ny));
  if (floor_on && z == 0) flags[i] = pw::FLOOR;
  else if (floor_on && z == nz - 1) flags[i] = pw::EQ;
  else if (x == 0 || x == nx - 1) flags[i] = pw::EQ;
}

// countCells, voxelize.ts:137-154
__global__ void count_kernel(const uint32_t *flags, size_t cells, uint32_t nx, uint32_t *solid,
                             uint8_t *body_proj, uint8_t *wall_proj) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= cells) return;
  uint32_t t = flags[i] & 7u;
  if (t == pw::SOLID) { atomicAdd(solid, 1u); body_proj[i / nx] = 1; }
  if (t == pw::SOLID || t == pw::SUPPORT) wall_proj[i / nx] = 1;
}

__global__ void sum_u8_kernel(const uint8_t *v, size_t n, uint32_t *out) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t x = i < n ? v[i] : 0u;
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  if ((threadIdx.x & 31) == 0 && x) atomicAdd(out, x);
}

// markWalls, wall-links.ts:34-51, gathered per fluid cell: bit (3+i) when the
// pull source x - c_i (x bounded, y periodic, z bounded with a floor) is a wall.
// Only fluid words change and their type bits stay, so concurrent readers of a
// neighbour's type see the same kind before and after its write.
__global__ void wall_mask_kernel(uint32_t *flags, uint32_t nx, uint32_t ny, uint32_t nz, int floor_on,
                                 uint32_t *link_count, uint32_t *is_boundary) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  size_t cells = (size_t)nx * ny * nz;
  if (i >= cells) return;
  uint32_t f = flags[i];
  uint32_t mask = 0, body = 0;
  if ((f & 7u) == pw::FLUID) {
    long x = (long)(i % nx), y = (long)((i / nx) % ny), z = (long)(i / ((size_t)nx * ny));
#pragma unroll
    for (int d = 1; d < 19; d++) {
      long sx = x - pw::cx_of(d), sy = y - pw::cy_of(d), sz = z - pw::cz_of(d);
      if (sx < 0 || sx >= (long)nx) continue;
      if (floor_on && (sz < 0 || sz >= (long)nz)) continue;
      sy = (sy + ny) % ny;
      sz = (sz + nz) % nz;
      uint32_t t = flags[(size_t)sx + (size_t)nx * ((size_t)sy + (size_t)ny * (size_t)sz)] & 7u;
      if (t >= pw::SOLID && t <= pw::FLOOR) {
        mask |= 1u << (3 + d);
        if (t == pw::SOLID) body = 1;
      }
    }
    if (mask) flags[i] = f | mask;
  }
  link_count[i] = __popc(mask);
  is_boundary[i] = body;
}

__global__ void qoff_kernel(const uint32_t *link_count, const uint32_t *scan, uint32_t *qoff, size_t cells) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < cells) qoff[i] = link_count[i] ? scan[i] : PW_NO_Q;
}

__global__ void compact_kernel(const uint32_t *is_boundary, const uint32_t *scan, uint32_t *out, size_t cells) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < cells && is_boundary[i]) out[scan[i]] = (uint32_t)i;
}

__global__ void fill_float_kernel(float *p, size_t n, float v) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

static inline unsigned nblk(size_t n, unsigned b = 256) { return (unsigned)((n + b - 1) / b); }

static int vote_mesh(const float *d_mesh, uint32_t ntri, uint32_t nx, uint32_t ny, uint32_t nz,
                     uint32_t *flags, uint32_t type, bool *watertight, cudaStream_t s) {
  size_t cells = (size_t)nx * ny * nz;
  uint32_t sizes[3] = {nx, ny, nz};
  size_t strides[3] = {1, nx, (size_t)nx * ny};
  const int PROJS[3][3] = {{0, 1, 2}, {1, 2, 0}, {2, 0, 1}};
  uint8_t *votes = nullptr;
  uint32_t *closed = nullptr;
  PW_TRY(tmp_alloc(&votes, cells, s));
  cudaError_t e = tmp_alloc(&closed, 4, s);
  if (e != cudaSuccess) { tmp_free(votes, s); return cuda_status(e, "voxelize"); }
  int rc = PW_OK;
  uint32_t one = 1u;
  cudaMemsetAsync(votes, 0, cells, s);
  cudaMemcpyAsync(closed, &one, 4, cudaMemcpyHostToDevice, s);
  for (int p = 0; p < 3 && rc == PW_OK && ntri > 0; p++) {
    Proj P;
    P.u = PROJS[p][0]; P.v = PROJS[p][1]; P.axis = PROJS[p][2];
    P.su = sizes[P.u]; P.sv = sizes[P.v]; P.sa = sizes[P.axis];
    P.stu = strides[P.u]; P.stv = strides[P.v]; P.sta = strides[P.axis];
    size_t ncol = (size_t)P.su * P.sv;
    uint32_t *count = nullptr, *offset = nullptr, *cursor = nullptr;
    double *hits = nullptr;
    uint64_t total = 0;
    e = tmp_alloc(&count, ncol * 4, s);
    if (e == cudaSuccess) e = tmp_alloc(&offset, ncol * 4, s);
    if (e == cudaSuccess) e = tmp_alloc(&cursor, ncol * 4, s);
    if (e != cudaSuccess) rc = cuda_status(e, "voxelize columns");
    if (rc == PW_OK) {
      cudaMemsetAsync(count, 0, ncol * 4, s);
      cudaMemsetAsync(cursor, 0, ncol * 4, s);
      raster_kernel<<<ntri, 128, 0, s>>>(d_mesh, P, count, nullptr, nullptr, nullptr, 0);
      rc = exclusive_scan(count, offset, ncol, &total, s);
    }
    if (rc == PW_OK) {
      e = tmp_alloc(&hits, (total ? total : 1) * sizeof(double), s);
      if (e != cudaSuccess) rc = cuda_status(e, "voxelize hits");
    }
    if (rc == PW_OK) {
      raster_kernel<<<ntri, 128, 0, s>>>(d_mesh, P, count, offset, cursor, hits, 1);
      column_kernel<<<nblk(ncol), 256, 0, s>>>(P, count, offset, hits, votes, closed);
    }
    tmp_free(count, s); tmp_free(offset, s); tmp_free(cursor, s); tmp_free(hits, s);
  }
  uint32_t closed_h = 1;
  if (rc == PW_OK) {
    classify_kernel<<<nblk(cells), 256, 0, s>>>(votes, flags, cells, type);
    e = cudaMemcpyAsync(&closed_h, closed, 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) rc = cuda_status(e, "voxelize vote");
  }
  *watertight = closed_h != 0;
  tmp_free(votes, s);
  tmp_free(closed, s);
  return rc;
}

// ------------------------------------------------------------------ link fractions
// binTriangles / nearestLinkHit / intersection (src/geometry/triangle-bins.ts:1-162)
// and linkFraction (src/geometry/wall-links.ts:53-80) in binary64: four-cell bins
// of triangle offsets, then one thread per fluid cell casts each wall link's segment
// from the cell centre toward the wall and keeps the nearest Moller-Trumbore hit.
// The minimum does not depend on the order of a bin's items, so bins fill with
// atomics and the fractions match the sequential reference bit for bit.
constexpr int kBin = 4;

struct DevBins {
  const float *mesh = nullptr;
  float *bounds = nullptr;      // 6 per triangle: float lo, hi
  uint32_t *start = nullptr;    // nbins + 1
  uint32_t *items = nullptr;    // 9 * triangle per entry
  int bx = 0, by = 0, bz = 0;
};

__device__ __forceinline__ void bin_range(const double *lo, const double *hi, const DevBins &B, long *r) {
  const int dims[3] = {B.bx, B.by, B.bz};
  for (int a = 0; a < 3; a++) {
    long mn = (long)floor(lo[a] / kBin), mx = (long)floor(hi[a] / kBin);
    r[2 * a] = mn < 0 ? 0 : mn;
    r[2 * a + 1] = mx > dims[a] - 1 ? dims[a] - 1 : mx;
  }
}

// pass 0 counts the bins each triangle's box touches, pass 1 files the triangle.
__global__ void bin_triangles_kernel(DevBins B, uint32_t ntri, uint32_t *count, int pass) {
  uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntri) return;
  const float *p = B.mesh + 9 * (size_t)t;
  double lo[3], hi[3];
  for (int a = 0; a < 3; a++) {
    double x = p[a], y = p[a + 3], z = p[a + 6];
    lo[a] = fmin(fmin(x, y), z);
    hi[a] = fmax(fmax(x, y), z);
  }
  if (pass == 0)
    for (int a = 0; a < 3; a++) { B.bounds[6 * t + a] = (float)lo[a]; B.bounds[6 * t + 3 + a] = (float)hi[a]; }
  long r[6];
  bin_range(lo, hi, B, r);
  for (long z = r[4]; z <= r[5]; z++)
    for (long y = r[2]; y <= r[3]; y++)
      for (long x = r[0]; x <= r[1]; x++) {
        size_t k = (size_t)x + (size_t)B.bx * ((size_t)y + (size_t)B.by * (size_t)z);
        uint32_t slot = atomicAdd(&count[k], 1u);
        if (pass == 1) B.items[B.start[k] + slot] = 9u * t;
      }
}

__global__ void set_u32_kernel(uint32_t *p, uint32_t v) { *p = v; }

// intersection, triangle-bins.ts:60-94: the hit depth t along d, or false.
__device__ bool segment_hit(const float *p, uint32_t off, const double *o, const double *d, double *t) {
  const double EPS = 1e-9;
  double ax = p[off], ay = p[off + 1], az = p[off + 2];
  double e1x = (double)p[off + 3] - ax, e1y = (double)p[off + 4] - ay, e1z = (double)p[off + 5] - az;
  double e2x = (double)p[off + 6] - ax, e2y = (double)p[off + 7] - ay, e2z = (double)p[off + 8] - az;
  double px = d[1] * e2z - d[2] * e2y;
  double py = d[2] * e2x - d[0] * e2z;
  double pz = d[0] * e2y - d[1] * e2x;
  double det = e1x * px + e1y * py + e1z * pz;
  if (fabs(det) < 2.220446049250313e-16) return false;
  double tx = o[0] - ax, ty = o[1] - ay, tz = o[2] - az;
  double u = (tx * px + ty * py + tz * pz) / det;
  if (u < -EPS || u > 1 + EPS) return false;
  double qx = ty * e1z - tz * e1y;
  double qy = tz * e1x - tx * e1z;
  double qz = tx * e1y - ty * e1x;
  double v = (d[0] * qx + d[1] * qy + d[2] * qz) / det;
  if (v < -EPS || u + v > 1 + EPS) return false;
  double tt = (e2x * qx + e2y * qy + e2z * qz) / det;
  if (tt >= -EPS && tt <= 1 + EPS) { *t = tt; return true; }
  return false;
}

// nearestLinkHit, triangle-bins.ts:136-161.
__device__ bool nearest_link_hit(const DevBins &B, const double *o, const double *d, double *t) {
  double lo[3], hi[3];
  for (int a = 0; a < 3; a++) {
    double e = o[a] + d[a];
    lo[a] = o[a] < e ? o[a] : e;
    hi[a] = o[a] > e ? o[a] : e;
  }
  long r[6];
  bin_range(lo, hi, B, r);
  double nearest = CUDART_INF;
  for (long z = r[4]; z <= r[5]; z++)
    for (long y = r[2]; y <= r[3]; y++)
      for (long x = r[0]; x <= r[1]; x++) {
        size_t k = (size_t)x + (size_t)B.bx * ((size_t)y + (size_t)B.by * (size_t)z);
        for (uint32_t it = B.start[k]; it < B.start[k + 1]; it++) {
          uint32_t off = B.items[it];
          const float *bd = B.bounds + 6 * (off / 9);
          if (!((double)bd[0] <= hi[0] && (double)bd[3] >= lo[0] && (double)bd[1] <= hi[1] &&
                (double)bd[4] >= lo[1] && (double)bd[2] <= hi[2] && (double)bd[5] >= lo[2]))
            continue;
          double tt;
          if (segment_hit(B.mesh, off, o, d, &tt) && tt < nearest) nearest = tt;
        }
      }
  if (nearest == CUDART_INF) return false;
  *t = nearest;
  return true;
}

// linkFraction per wall link of a fluid cell, in link-rank order from its q offset:
// FLOOR links keep 1/2; SOLID links cast against the body, SUPPORT links against
// the supports; a miss keeps 1/2 and counts; hits clamp to [1e-3, 1].
__global__ void link_fraction_kernel(const uint32_t *flags, const uint32_t *qoff, float *fractions, uint32_t nx,
                                     uint32_t ny, uint32_t nz, int floor_on, DevBins body, DevBins sup, int has_sup,
                                     uint32_t *missed) {
  size_t cell = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  size_t cells = (size_t)nx * ny * nz;
  if (cell >= cells) return;
  uint32_t flag = flags[cell];
  if ((flag >> 3) == 0) return;
  uint32_t f = qoff[cell];
  long x = (long)(cell % nx), y = (long)((cell / nx) % ny), z = (long)(cell / ((size_t)nx * ny));
  uint32_t miss = 0;
  for (int i = 1; i < 19; i++) {
    if (!(flag & (1u << (3 + i)))) continue;
    const int cx = pw::cx_of(i), cy = pw::cy_of(i), cz = pw::cz_of(i);
    // the wall x - c_i: x bounded, y periodic, z periodic unless a floor bounds it
    long wx = x - cx, wy = (y - cy + (long)ny) % (long)ny, wz = (z - cz + (long)nz) % (long)nz;
    size_t wall = (size_t)wx + (size_t)nx * ((size_t)wy + (size_t)ny * (size_t)wz);
    uint32_t type = flags[wall] & 7u;
    double q = 0.5;
    bool hit = true;
    if (type != pw::FLOOR) {
      const DevBins *bins = type == pw::SUPPORT ? (has_sup ? &sup : nullptr) : &body;
      double o[3] = {(double)wx + cx, (double)wy + cy, (double)wz + cz};
      double d[3] = {(double)-cx, (double)-cy, (double)-cz};
      double t = 0;
      hit = bins ? nearest_link_hit(*bins, o, d, &t) : false;
      q = hit ? t : 0.5;
    }
    miss += hit ? 0u : 1u;
    double c = q < 1 ? q : 1;
    c = c > 1e-3 ? c : 1e-3;
    fractions[f++] = (float)c;
  }
  if (miss) atomicAdd(missed, miss);
}

static void free_bins(DevBins &B, cudaStream_t s) {
  tmp_free(B.bounds, s); tmp_free(B.start, s); tmp_free(B.items, s);
  B = DevBins();
}

static int build_bins(const float *d_mesh, uint32_t ntri, uint32_t nx, uint32_t ny, uint32_t nz, DevBins *out,
                      cudaStream_t s) {
  DevBins B;
  B.mesh = d_mesh;
  B.bx = (int)((nx + kBin - 1) / kBin); B.by = (int)((ny + kBin - 1) / kBin); B.bz = (int)((nz + kBin - 1) / kBin);
  size_t nb = (size_t)B.bx * B.by * B.bz;
  uint32_t *count = nullptr;
  uint64_t total = 0;
  cudaError_t e = tmp_alloc(&B.bounds, (ntri ? ntri : 1) * 6 * sizeof(float), s);
  if (e == cudaSuccess) e = tmp_alloc(&B.start, (nb + 1) * 4, s);
  if (e == cudaSuccess) e = tmp_alloc(&count, nb * 4, s);
  int rc = e == cudaSuccess ? PW_OK : cuda_status(e, "triangle bins");
  if (rc == PW_OK) {
    cudaMemsetAsync(count, 0, nb * 4, s);
    if (ntri) bin_triangles_kernel<<<nblk(ntri, 128), 128, 0, s>>>(B, ntri, count, 0);
    rc = exclusive_scan(count, B.start, nb, &total, s);
  }
  if (rc == PW_OK) {
    set_u32_kernel<<<1, 1, 0, s>>>(B.start + nb, (uint32_t)total);
    e = tmp_alloc(&B.items, (total ? total : 1) * 4, s);
    if (e != cudaSuccess) rc = cuda_status(e, "triangle bins");
  }
  if (rc == PW_OK) {
    cudaMemsetAsync(count, 0, nb * 4, s);
    if (ntri) bin_triangles_kernel<<<nblk(ntri, 128), 128, 0, s>>>(B, ntri, count, 1);
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) rc = cuda_status(e, "triangle bins");
  }
  tmp_free(count, s);
  if (rc != PW_OK) { free_bins(B, s); return rc; }
  *out = B;
  return PW_OK;
}

// Measured fractions for every wall link of a finished grid (buildWallLinks with
// measureFractions, wall-links.ts:99-131); sets stats.missed_links.
static int measure_links(pw_grid *g, const float *d_body, uint32_t nbody, const float *d_sup, uint32_t nsup,
                         bool has_sup, int floor_on, cudaStream_t s) {
  DevBins body, sup;
  int rc = build_bins(d_body, nbody, g->nx, g->ny, g->nz, &body, s);
  if (rc == PW_OK && has_sup) rc = build_bins(d_sup, nsup, g->nx, g->ny, g->nz, &sup, s);
  uint32_t *missed = nullptr;
  uint32_t missed_h = 0;
  if (rc == PW_OK) {
    cudaError_t e = tmp_alloc(&missed, 4, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(missed, 0, 4, s);
    if (e == cudaSuccess) {
      link_fraction_kernel<<<nblk(g->cells, 128), 128, 0, s>>>(g->flags, g->qoff, g->fractions, g->nx, g->ny, g->nz,
                                                               floor_on, body, sup, has_sup ? 1 : 0, missed);
      e = cudaMemcpyAsync(&missed_h, missed, 4, cudaMemcpyDeviceToHost, s);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) rc = cuda_status(e, "link fractions");
  }
  tmp_free(missed, s);
  free_bins(body, s);
  free_bins(sup, s);
  if (rc == PW_OK) g->stats.missed_links = missed_h;
  return rc;
}

static bool finite_mesh(const float *m, uint32_t ntri) {
  for (size_t k = 0; k < 9 * (size_t)ntri; k++)
    if (!std::isfinite(m[k])) return false;
  return true;
}

// Shared tail: wall masks, q offsets, halfway fractions, boundary list, counts.
static int finish_grid(pw_grid *g, int floor_on, bool body_closed, bool supports_closed, cudaStream_t s) {
  size_t cells = g->cells;
  uint32_t *link_count = nullptr, *is_boundary = nullptr, *scan = nullptr, *solid = nullptr;
  uint8_t *proj = nullptr;
  size_t plane = (size_t)g->ny * g->nz;
  cudaError_t e = tmp_alloc(&link_count, cells * 4, s);
  if (e == cudaSuccess) e = tmp_alloc(&is_boundary, cells * 4, s);
  if (e == cudaSuccess) e = tmp_alloc(&scan, cells * 4, s);
  if (e == cudaSuccess) e = tmp_alloc(&solid, 16, s);
  if (e == cudaSuccess) e = tmp_alloc(&proj, 2 * plane, s);
  int rc = e == cudaSuccess ? PW_OK : cuda_status(e, "voxelize counts");
  uint32_t counts[4] = {0, 0, 0, 0};
  if (rc == PW_OK) {
    cudaMemsetAsync(solid, 0, 16, s);
    cudaMemsetAsync(proj, 0, 2 * plane, s);
    count_kernel<<<nblk(cells), 256, 0, s>>>(g->flags, cells, g->nx, solid, proj, proj + plane);
    sum_u8_kernel<<<nblk(plane), 256, 0, s>>>(proj, plane, solid + 1);
    sum_u8_kernel<<<nblk(plane), 256, 0, s>>>(proj + plane, plane, solid + 2);
    wall_mask_kernel<<<nblk(cells), 256, 0, s>>>(g->flags, g->nx, g->ny, g->nz, floor_on, link_count, is_boundary);
    uint64_t nfrac = 0, nb = 0;
    rc = exclusive_scan(link_count, scan, cells, &nfrac, s);
    if (rc == PW_OK) {
      e = cudaMalloc(&g->qoff, cells * 4);
      if (e == cudaSuccess) e = cudaMalloc(&g->fractions, (nfrac ? nfrac : 1) * 4);
      if (e != cudaSuccess) rc = cuda_status(e, "voxelize q");
    }
    if (rc == PW_OK) {
      qoff_kernel<<<nblk(cells), 256, 0, s>>>(link_count, scan, g->qoff, cells);
      if (nfrac) fill_float_kernel<<<nblk(nfrac), 256, 0, s>>>(g->fractions, nfrac, 0.5f);
      g->nfrac = nfrac;
      rc = exclusive_scan(is_boundary, scan, cells, &nb, s);
    }
    if (rc == PW_OK) {
      e = cudaMalloc(&g->boundary, (nb ? nb : 1) * 4);
      if (e != cudaSuccess) rc = cuda_status(e, "voxelize boundary");
    }
    if (rc == PW_OK) {
      compact_kernel<<<nblk(cells), 256, 0, s>>>(is_boundary, scan, g->boundary, cells);
      g->nboundary = nb;
      e = cudaMemcpyAsync(counts, solid, 12, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) rc = cuda_status(e, "voxelize finish");
    }
  }
  tmp_free(link_count, s); tmp_free(is_boundary, s); tmp_free(scan, s); tmp_free(solid, s); tmp_free(proj, s);
  if (rc != PW_OK) return rc;
  pw_grid_stats &st = g->stats;
  st.nx = g->nx; st.ny = g->ny; st.nz = g->nz;
  st.solid_cells = counts[0];
  st.frontal_cells = counts[1];
  st.blockage = (double)counts[2] / ((double)g->ny * g->nz);
  st.watertight = body_closed && supports_closed;
  st.missed_links = 0;
  st.geometry_len = 2 * (uint64_t)cells + g->nfrac;
  st.boundary_cells = g->nboundary;
  return PW_OK;
}

// ------------------------------------------------------------------ validation
// validateGeometry's mask rule (geometry-contract.ts:20-58) with every axis
// periodic: non-fluid cells carry their kind alone, fluid cells exactly the
// walls among their wrapped pull sources.
__global__ void validate_kernel(const uint32_t *flags, uint32_t nx, uint32_t ny, uint32_t nz,
                                unsigned long long *first_bad) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  size_t cells = (size_t)nx * ny * nz;
  if (i >= cells) return;
  uint32_t f = flags[i], kind = f & 7u;
  uint32_t expected = 0;
  if (kind == pw::FLUID) {
    long x = (long)(i % nx), y = (long)((i / nx) % ny), z = (long)(i / ((size_t)nx * ny));
#pragma unroll
    for (int d = 1; d < 19; d++) {
      long sx = (x - pw::cx_of(d) + nx) % nx, sy = (y - pw::cy_of(d) + ny) % ny, sz = (z - pw::cz_of(d) + nz) % nz;
      uint32_t t = flags[(size_t)sx + (size_t)nx * ((size_t)sy + (size_t)ny * (size_t)sz)] & 7u;
      if (t >= pw::SOLID && t <= pw::FLOOR) expected |= 1u << (3 + d);
    }
  }
  if (kind > pw::EQ || f != (kind | expected)) atomicMin(first_bad, (unsigned long long)i);
}

}  // namespace pwhost

using namespace pwhost;

extern "C" {

const char *pw_last_error(void) { return pwhost::last_error(); }
const char *pw_version(void) { return "pocketwind_gb300 0.1 (sm_103a)"; }

int pw_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) { cudaGetLastError(); return 0; }
  return n;
}

int pw_voxelize(const float *body, uint32_t body_triangles, const float *supports,
                uint32_t support_triangles, uint32_t nx, uint32_t ny, uint32_t nz, int floor_on,
                pw_grid **out) {
  return pw_voxelize_opts(body, body_triangles, supports, support_triangles, nx, ny, nz, floor_on, 0, out);
}

int pw_voxelize_opts(const float *body, uint32_t body_triangles, const float *supports,
                     uint32_t support_triangles, uint32_t nx, uint32_t ny, uint32_t nz, int floor_on,
                     int link_fractions, pw_grid **out) {
  if (!out) { set_error("out is NULL"); return PW_ERR_INVALID; }
  *out = nullptr;
  if (nx < 2 || ny < 2 || nz < 2) {
    set_error("Grid dimensions must be integers of at least two cells.");
    return PW_ERR_INVALID;
  }
  size_t cells = (size_t)nx * ny * nz;
  if (cells > 0xffffffffull - 64) {
    set_error("The grid exceeds 2^32 cells.");
    return PW_ERR_INVALID;
  }
  if ((body_triangles && !body) || (support_triangles && !supports)) {
    set_error("Mesh positions must match a non-negative triangle count.");
    return PW_ERR_INVALID;
  }
  if (!finite_mesh(body, body_triangles) || (supports && !finite_mesh(supports, support_triangles))) {
    set_error("Mesh coordinates must be finite.");
    return PW_ERR_INVALID;
  }
  cudaStream_t s;
  PW_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  pw_grid *g = new pw_grid();
  g->nx = nx; g->ny = ny; g->nz = nz; g->cells = cells;
  float *d_mesh = nullptr;
  int rc = PW_OK;
  bool body_closed = true, sup_closed = true;
  cudaError_t e = cudaMalloc(&g->flags, cells * 4);
  float *d_sup = nullptr;
  if (e == cudaSuccess) e = tmp_alloc(&d_mesh, (body_triangles ? body_triangles : 1) * 36, s);
  if (e == cudaSuccess) e = tmp_alloc(&d_sup, (support_triangles ? support_triangles : 1) * 36, s);
  if (e != cudaSuccess) rc = cuda_status(e, "pw_voxelize");
  if (rc == PW_OK) {
    cudaMemsetAsync(g->flags, 0, cells * 4, s);
    if (body_triangles) cudaMemcpyAsync(d_mesh, body, (size_t)body_triangles * 36, cudaMemcpyHostToDevice, s);
    rc = vote_mesh(d_mesh, body_triangles, nx, ny, nz, g->flags, pw::SOLID, &body_closed, s);
  }
  if (rc == PW_OK && supports) {
    if (support_triangles) cudaMemcpyAsync(d_sup, supports, (size_t)support_triangles * 36, cudaMemcpyHostToDevice, s);
    rc = vote_mesh(d_sup, support_triangles, nx, ny, nz, g->flags, pw::SUPPORT, &sup_closed, s);
  }
  if (rc == PW_OK) {
    boundary_kernel<<<nblk(cells), 256, 0, s>>>(g->flags, nx, ny, nz, floor_on);
    rc = finish_grid(g, floor_on, body_closed, sup_closed, s);
  }
  if (rc == PW_OK && link_fractions && g->nfrac)
    rc = measure_links(g, d_mesh, body_triangles, d_sup, support_triangles, supports != nullptr, floor_on, s);
  tmp_free(d_mesh, s);
  tmp_free(d_sup, s);
  cudaStreamSynchronize(s);
  cudaStreamDestroy(s);
  if (rc != PW_OK) { delete g; return rc; }
  *out = g;
  return PW_OK;
}

int pw_grid_from_host(uint32_t nx, uint32_t ny, uint32_t nz, const uint32_t *geometry,
                      size_t geometry_len, const uint32_t *boundary, size_t nboundary, pw_grid **out) {
  if (!out) { set_error("out is NULL"); return PW_ERR_INVALID; }
  *out = nullptr;
  if (nx < 1 || ny < 1 || nz < 1) { set_error("Grid dimensions must be positive safe integers."); return PW_ERR_INVALID; }
  size_t cells = (size_t)nx * ny * nz;
  if (cells > 0xffffffffull - 64) { set_error("The grid exceeds 2^32 cells."); return PW_ERR_INVALID; }
  if (!geometry || geometry_len < 2 * cells) {
    set_error("Geometry must match the solver layout and contain flags and q offsets.");
    return PW_ERR_INVALID;
  }
  // q offsets and fraction count (geometry-contract.ts:7-18,50-65)
  size_t fractions = 0;
  for (size_t c = 0; c < cells; c++) {
    uint32_t flag = geometry[c], kind = flag & 7u;
    if (kind > pw::EQ) { set_error("Unknown geometry cell kind at cell %zu.", c); return PW_ERR_INVALID; }
    uint32_t off = geometry[cells + c];
    if (off == PW_NO_Q) continue;
    uint32_t mask = kind == pw::FLUID ? (flag & ~7u) : 0u;
    if (mask == 0 || off != fractions) { set_error("Invalid geometry q offset at cell %zu.", c); return PW_ERR_INVALID; }
    fractions += (size_t)__builtin_popcount(mask >> 4);
  }
  if (geometry_len != 2 * cells + fractions) {
    set_error("Geometry length must match its cell planes and packed wall-link fractions.");
    return PW_ERR_INVALID;
  }
  for (size_t k = 0; k < nboundary; k++) {
    uint32_t c = boundary[k];
    if (c >= cells || (geometry[c] & 7u) != pw::FLUID || (geometry[c] >> 4) == 0) {
      set_error("Boundary cells must index fluid cells with wall links.");
      return PW_ERR_INVALID;
    }
  }
  cudaStream_t s;
  PW_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  pw_grid *g = new pw_grid();
  g->nx = nx; g->ny = ny; g->nz = nz; g->cells = cells;
  unsigned long long *bad = nullptr;
  unsigned long long bad_h = ~0ull;
  cudaError_t e = cudaMalloc(&g->flags, cells * 4);
  if (e == cudaSuccess) e = cudaMalloc(&g->qoff, cells * 4);
  if (e == cudaSuccess) e = cudaMalloc(&g->fractions, (fractions ? fractions : 1) * 4);
  if (e == cudaSuccess) e = cudaMalloc(&g->boundary, (nboundary ? nboundary : 1) * 4);
  if (e == cudaSuccess) e = cudaMalloc(&bad, 8);
  if (e == cudaSuccess) e = cudaMemcpyAsync(g->flags, geometry, cells * 4, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(g->qoff, geometry + cells, cells * 4, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && fractions)
    e = cudaMemcpyAsync(g->fractions, geometry + 2 * cells, fractions * 4, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && nboundary) e = cudaMemcpyAsync(g->boundary, boundary, nboundary * 4, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(bad, &bad_h, 8, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    validate_kernel<<<nblk(cells), 256, 0, s>>>(g->flags, nx, ny, nz, bad);
    e = cudaMemcpyAsync(&bad_h, bad, 8, cudaMemcpyDeviceToHost, s);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(bad);
  cudaStreamDestroy(s);
  if (e != cudaSuccess) { delete g; return cuda_status(e, "pw_grid_from_host"); }
  if (bad_h != ~0ull) {
    delete g;
    set_error("Inconsistent wall mask at cell %llu.", bad_h);
    return PW_ERR_INVALID;
  }
  g->nfrac = fractions;
  g->nboundary = nboundary;
  // statistics as countCells would report them (voxelize.ts:137-154)
  uint32_t solid = 0, frontal = 0, blocked = 0;
  std::vector<uint8_t> bp((size_t)ny * nz, 0), wp((size_t)ny * nz, 0);
  for (size_t c = 0; c < cells; c++) {
    uint32_t t = geometry[c] & 7u;
    if (t == pw::SOLID) { solid++; bp[c / nx] = 1; }
    if (t == pw::SOLID || t == pw::SUPPORT) wp[c / nx] = 1;
  }
  for (size_t k = 0; k < bp.size(); k++) { frontal += bp[k]; blocked += wp[k]; }
  pw_grid_stats &st = g->stats;
  st.nx = nx; st.ny = ny; st.nz = nz;
  st.solid_cells = solid; st.frontal_cells = frontal;
  st.blockage = (double)blocked / ((double)ny * nz);
  st.watertight = 1; st.missed_links = 0;
  st.geometry_len = geometry_len; st.boundary_cells = nboundary;
  *out = g;
  return PW_OK;
}

int pw_grid_stats_get(const pw_grid *grid, pw_grid_stats *out) {
  if (!grid || !out) { set_error("NULL argument"); return PW_ERR_INVALID; }
  *out = grid->stats;
  return PW_OK;
}

int pw_grid_read_geometry(const pw_grid *g, uint32_t *out, size_t capacity) {
  if (!g || !out) { set_error("NULL argument"); return PW_ERR_INVALID; }
  if (capacity < 2 * g->cells + g->nfrac) { set_error("geometry buffer too small"); return PW_ERR_INVALID; }
  PW_TRY(cudaMemcpy(out, g->flags, g->cells * 4, cudaMemcpyDeviceToHost));
  PW_TRY(cudaMemcpy(out + g->cells, g->qoff, g->cells * 4, cudaMemcpyDeviceToHost));
  if (g->nfrac) PW_TRY(cudaMemcpy(out + 2 * g->cells, g->fractions, g->nfrac * 4, cudaMemcpyDeviceToHost));
  return PW_OK;
}

int pw_grid_read_boundary(const pw_grid *g, uint32_t *out, size_t capacity) {
  if (!g || (!out && g->nboundary)) { set_error("NULL argument"); return PW_ERR_INVALID; }
  if (capacity < g->nboundary) { set_error("boundary buffer too small"); return PW_ERR_INVALID; }
  if (g->nboundary) PW_TRY(cudaMemcpy(out, g->boundary, g->nboundary * 4, cudaMemcpyDeviceToHost));
  return PW_OK;
}

void pw_grid_destroy(pw_grid *grid) { delete grid; }

}  // extern "C"
