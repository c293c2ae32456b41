// mdg_observe_noalloc: the observers of mdg_observe for callers that cannot
// allocate device memory.
//
// Who needs it: code that runs where cudaMalloc is unavailable or unsafe --
// inside a memory-pool-managed host application that forbids CUDA
// allocations, inside a host callback or a stream-ordered section that must
// not synchronise the device, or a caller that already owns its particle
// arrays on the device and has no mdg handle (creating one allocates the
// whole pair-list machinery).  Such a caller passes its own device arrays and
// receives the three observer sums in its own device buffer.
//
// How: the kernels are a variant of the handle's observe kernel (same pair
// energy and virial expressions, same reference rounding of r^2), but instead
// of reading the handle's neighbour list they bin the particles into cells of
// width >= cutoff and scan the 27 neighbouring cells.  All working memory --
// cell counts, cell starts, the particle order and the per-block partial
// sums -- is one file-scope __device__ array of fixed size (every GPU that
// loads this library holds it until the process exits).  Its device address
// is looked up once per device with cudaGetSymbolAddress on that device's
// first call; nothing is allocated or freed, ever.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <mutex>

#include "mdg_internal.cuh"

namespace mdg {
namespace noalloc {

constexpr int kMaxParticles = 1 << 20;  // 1,048,576
constexpr int kMaxCells = 1 << 18;      // 262,144
constexpr int kThreads = 128;
constexpr int kMaxBlocks = kMaxParticles / kThreads;
constexpr int kMaxDevices = 64;

// Layout of the scratch array, in 8-byte words.
constexpr size_t kOffCount = 0;                                   // int[kMaxCells]
constexpr size_t kOffStart = kOffCount + kMaxCells / 2;           // int[kMaxCells + 2]
constexpr size_t kOffFill = kOffStart + kMaxCells / 2 + 1;        // int[kMaxCells]
constexpr size_t kOffCellOf = kOffFill + kMaxCells / 2;           // int[kMaxParticles]
constexpr size_t kOffOrder = kOffCellOf + kMaxParticles / 2;      // int[kMaxParticles]
constexpr size_t kOffPartial = kOffOrder + kMaxParticles / 2;     // double[3 * kMaxBlocks]
constexpr size_t kWords = kOffPartial + 3 * (size_t)kMaxBlocks;   // 1,409,025 words = 11.3 MB

static __device__ __align__(256) unsigned long long g_scratch[kWords];

struct Box {
  double L[3], inv_w[3];
  int nc[3], ncell, n;
  double rc2, c0, c2, c2x8;
};

struct Scratch {
  int *count, *start, *fill, *cell_of, *order;
  double *partial;
};

__global__ void k_clear(Box b, Scratch s) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < b.ncell; c += gridDim.x * blockDim.x) {
    s.count[c] = 0;
    s.fill[c] = 0;
  }
}

__device__ __forceinline__ double wrap1(double x, double L) {
  if (x < 0.0) x += L;
  else if (x >= L) x -= L;
  if (x < 0.0 || x >= L) x -= L * floor(x / L);
  return x;
}

__global__ void k_bin(Box b, Scratch s, const double4_32a *q) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b.n) return;
  const double4_32a v = q[i];
  const double x[3] = {wrap1(v.x, b.L[0]), wrap1(v.y, b.L[1]), wrap1(v.z, b.L[2])};
  int c[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    int ci = (int)(x[k] * b.inv_w[k]);
    c[k] = ci < 0 ? 0 : (ci >= b.nc[k] ? b.nc[k] - 1 : ci);
  }
  const int cc = (c[2] * b.nc[1] + c[1]) * b.nc[0] + c[0];
  s.cell_of[i] = cc;
  atomicAdd(&s.count[cc], 1);
}

// One block of 1024 threads: exclusive scan over all cells in tiles of 1024.
__global__ void __launch_bounds__(1024) k_scan(Box b, Scratch s) {
  __shared__ int warp_tot[32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int base = 0; base < b.ncell; base += 1024) {
    const int c = base + threadIdx.x;
    const int v = c < b.ncell ? s.count[c] : 0;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[wid] = x;
    __syncthreads();
    if (wid == 0) {
      int t = warp_tot[lane];
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, t, o);
        if (lane >= o) t += y;
      }
      warp_tot[lane] = t;
    }
    __syncthreads();
    const int excl = carry + (wid ? warp_tot[wid - 1] : 0) + x - v;
    if (c < b.ncell) s.start[c] = excl;
    __syncthreads();
    if (threadIdx.x == 0) carry += warp_tot[31];
    __syncthreads();
  }
  if (threadIdx.x == 0) s.start[b.ncell] = carry;
}

__global__ void k_scatter(Box b, Scratch s) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b.n) return;
  const int c = s.cell_of[i];
  s.order[s.start[c] + atomicAdd(&s.fill[c], 1)] = i;
}

__device__ __forceinline__ double block_sum(double v, double *sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sh[w];
  __syncthreads();
  return t;
}

// Observers of observer.cc:5-79 over every image pair within the cut-off,
// each pair weighted 1/2 (it is met from both sides).
__global__ void __launch_bounds__(kThreads) k_observe(Box b, Scratch s, const double4_32a *q, const double4_32a *p) {
  __shared__ double sh[kThreads / 32];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double ke = 0.0, pe = 0.0, vir = 0.0;
  if (i < b.n) {
    const double4_32a pi = p[i];
    ke = 0.5 * pi.x * pi.x + 0.5 * pi.y * pi.y + 0.5 * pi.z * pi.z + 0.5 * pi.w * pi.w;
    const double4_32a qr = q[i];
    const double xi = wrap1(qr.x, b.L[0]), yi = wrap1(qr.y, b.L[1]), zi = wrap1(qr.z, b.L[2]);
    const int c = s.cell_of[i];
    const int cx = c % b.nc[0], t = c / b.nc[0], cy = t % b.nc[1], cz = t / b.nc[1];
    for (int oz = -1; oz <= 1; oz++) {
      int nz = cz + oz, sz = 0;
      if (nz < 0) { nz += b.nc[2]; sz = -1; } else if (nz >= b.nc[2]) { nz -= b.nc[2]; sz = 1; }
      for (int oy = -1; oy <= 1; oy++) {
        int ny = cy + oy, sy = 0;
        if (ny < 0) { ny += b.nc[1]; sy = -1; } else if (ny >= b.nc[1]) { ny -= b.nc[1]; sy = 1; }
        for (int ox = -1; ox <= 1; ox++) {
          int nx = cx + ox, sx = 0;
          if (nx < 0) { nx += b.nc[0]; sx = -1; } else if (nx >= b.nc[0]) { nx -= b.nc[0]; sx = 1; }
          const int cc = (nz * b.nc[1] + ny) * b.nc[0] + nx;
          const int a = s.start[cc], e = s.start[cc + 1];
          for (int k = a; k < e; k++) {
            const int j = s.order[k];
            if (j == i && !(sx | sy | sz)) continue;
            const double4_32a qj = q[j];
            double xj = wrap1(qj.x, b.L[0]), yj = wrap1(qj.y, b.L[1]), zj = wrap1(qj.z, b.L[2]);
            if (sx) xj = __dadd_rn(xj, sx > 0 ? b.L[0] : -b.L[0]);
            if (sy) yj = __dadd_rn(yj, sy > 0 ? b.L[1] : -b.L[1]);
            if (sz) zj = __dadd_rn(zj, sz > 0 ? b.L[2] : -b.L[2]);
            const double dx = __dsub_rn(xi, xj), dy = __dsub_rn(yi, yj), dz = __dsub_rn(zi, zj);
            const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
            if (r2 > b.rc2) continue;
            const double r4 = __dmul_rn(r2, r2), r6 = __dmul_rn(r4, r2), r8 = __dmul_rn(r6, r2),
                         r10 = __dmul_rn(r8, r2), r12 = __dmul_rn(r10, r2);
            const double e_ij = 4.0 * (1.0 / r12 - 1.0 / r6 + __dmul_rn(b.c2, r2) + b.c0);
            const double df = (__dsub_rn(__dmul_rn(24.0, r6), 48.0) / (__dmul_rn(__dmul_rn(r6, r6), r2)) + b.c2x8) * r2;
            pe += 0.5 * e_ij;
            vir += 0.5 * df;
          }
        }
      }
    }
  }
  const double ta = block_sum(ke, sh), tb = block_sum(pe, sh), tc = block_sum(vir, sh);
  if (threadIdx.x == 0) {
    s.partial[3 * blockIdx.x + 0] = ta;
    s.partial[3 * blockIdx.x + 1] = tb;
    s.partial[3 * blockIdx.x + 2] = tc;
  }
}

__global__ void k_final(Scratch s, int nparts, double *out) {
  __shared__ double sh[32];
  double a = 0.0, b2 = 0.0, c = 0.0;
  for (int k = threadIdx.x; k < nparts; k += blockDim.x) {
    a += s.partial[3 * k + 0];
    b2 += s.partial[3 * k + 1];
    c += s.partial[3 * k + 2];
  }
  const double ta = block_sum(a, sh), tb = block_sum(b2, sh), tc = block_sum(c, sh);
  if (threadIdx.x == 0) {
    out[0] = ta;
    out[1] = tb;
    out[2] = tc / 3.0;
  }
}

std::mutex g_mu;
unsigned long long *g_addr[kMaxDevices] = {};

// Device address of g_scratch on the current device, looked up on the first call.
cudaError_t scratch_address(int dev, unsigned long long **out) {
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[dev]) {
    void *ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_scratch);
    if (e != cudaSuccess) return e;
    g_addr[dev] = static_cast<unsigned long long *>(ptr);
  }
  *out = g_addr[dev];
  return cudaSuccess;
}

}  // namespace noalloc
}  // namespace mdg

extern "C" int mdg_observe_noalloc(const double *q4_dev, const double *p4_dev, int32_t n, const double box[3],
                                   double cutoff, double *out3_dev, void *stream) {
  using namespace mdg::noalloc;
  if (!q4_dev || !p4_dev || !box || !out3_dev || n <= 0 || !(cutoff > 0.0)) return MDG_ERR_INVALID;
  // the state is read as 32-byte vectors, the sums written as doubles
  if ((((uintptr_t)q4_dev | (uintptr_t)p4_dev) & 31u) != 0 || ((uintptr_t)out3_dev & 7u) != 0) {
    fprintf(stderr, "mdg_observe_noalloc: q4_dev and p4_dev must be 32-byte aligned, out3_dev 8-byte aligned\n");
    return MDG_ERR_INVALID;
  }
  if (n > kMaxParticles) {
    fprintf(stderr, "mdg_observe_noalloc: %d particles exceed the fixed maximum of %d\n", n, kMaxParticles);
    return MDG_ERR_CAPACITY;
  }
  Box b;
  long long ncell = 1;
  for (int k = 0; k < 3; k++) {
    if (!(box[k] > 2.0 * cutoff) || !std::isfinite(box[k])) return MDG_ERR_INVALID;
    // the cell count is bounded before any conversion or product can overflow
    const double ratio = box[k] / cutoff;
    if (!(ratio <= (double)kMaxCells)) {
      fprintf(stderr, "mdg_observe_noalloc: box side %g / cutoff %g exceeds the fixed maximum of %d cells\n",
              box[k], cutoff, kMaxCells);
      return MDG_ERR_CAPACITY;
    }
    int nc = (int)ratio;
    while (nc > 0 && box[k] / (double)nc < cutoff * (1.0 + 1e-12)) nc--;
    if (nc < 2) return MDG_ERR_INVALID;
    b.L[k] = box[k];
    b.nc[k] = nc;
    b.inv_w[k] = 1.0 / (box[k] / (double)nc);
    if (ncell > kMaxCells / nc) {
      fprintf(stderr, "mdg_observe_noalloc: more cells than the fixed maximum of %d\n", kMaxCells);
      return MDG_ERR_CAPACITY;
    }
    ncell *= nc;
  }
  if (ncell > kMaxCells) {
    fprintf(stderr, "mdg_observe_noalloc: %lld cells exceed the fixed maximum of %d\n", ncell, kMaxCells);
    return MDG_ERR_CAPACITY;
  }
  b.ncell = (int)ncell;
  b.n = n;
  b.rc2 = cutoff * cutoff;
  const double s2 = 1.0 / (cutoff * cutoff);  // Variables::Variables (variables.cc:16-28)
  const double s6 = s2 * s2 * s2, s8 = s6 * s2, s12 = s6 * s6, s14 = s12 * s2;
  b.c2 = 6.0 * s14 - 3.0 * s8;
  b.c0 = -s12 + s6 - b.c2 / s2;
  b.c2x8 = b.c2 * 8.0;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return MDG_ERR_CUDA;
  unsigned long long *base = nullptr;
  if (scratch_address(dev, &base) != cudaSuccess) return MDG_ERR_CUDA;
  Scratch s;
  s.count = reinterpret_cast<int *>(base + kOffCount);
  s.start = reinterpret_cast<int *>(base + kOffStart);
  s.fill = reinterpret_cast<int *>(base + kOffFill);
  s.cell_of = reinterpret_cast<int *>(base + kOffCellOf);
  s.order = reinterpret_cast<int *>(base + kOffOrder);
  s.partial = reinterpret_cast<double *>(base + kOffPartial);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int grid = (n + kThreads - 1) / kThreads;
  const auto *q = reinterpret_cast<const double4_32a *>(q4_dev);
  const auto *p = reinterpret_cast<const double4_32a *>(p4_dev);
  k_clear<<<(b.ncell + 255) / 256, 256, 0, st>>>(b, s);
  k_bin<<<grid, kThreads, 0, st>>>(b, s, q);
  k_scan<<<1, 1024, 0, st>>>(b, s);
  k_scatter<<<grid, kThreads, 0, st>>>(b, s);
  k_observe<<<grid, kThreads, 0, st>>>(b, s, q, p);
  k_final<<<1, 1024, 0, st>>>(s, grid, out3_dev);
  return cudaGetLastError() == cudaSuccess ? MDG_OK : MDG_ERR_CUDA;
}
