// Initial conditions of the reference's configuration makers, generated on the
// device:
//   ConfigurationMaker (confmaker.cc:9-44): FCC sites with a 1e-7 offset;
//   ExtractConfigurationMaker (confmaker.cc:174-252): the FCC lattice of
//     floor(w/s) + 1 cells per side, thinned to floor(w^3 rho) sites by deleting
//     the first n_delete distinct sites drawn from mt19937(unit id) through
//     uniform_real_distribution<double>(0, 1);
//   DropletMaker (burst.cc:10-61): FCC sites inside a sphere at the box centre;
//   BallAdder (collision.cc:8-51) as Collision::Run places it (collision.cc:55-63):
//     two balls of a simple-cubic lattice with three half-shifted sites per
//     cell, moving at +speed and -speed along x;
//   Variables::SetInitialVelocity (variables.cc:82-108): speed V0 in directions
//     drawn from mt19937(seed), minus the mean.
// Positions are bit-identical to the reference's: the same double operations
// site by site, and the same random draws.  The random stream is MT19937
// (Matsumoto and Nishimura, 1998), generated by one block: the 624-word state
// is twisted in four sub-ranges whose inputs are already final, then tempered
// in parallel.  A double is made of two words as the C++ standard's
// generate_canonical<double, 53> does for a 32-bit engine, (w0 + w1 2^32) / 2^64,
// with the result held below 1 as libstdc++ does.  The reference finds distinct
// deletion sites with a linear search per draw (quadratic in the number of
// deletions: 3.5 s for 4M atoms on one host core); here every draw's first
// occurrence comes from an atomicMin per site and a prefix count, which gives
// the same set.  Velocity
// directions use the device's cos/sin, so velocities agree with the reference's
// to a few ulps rather than bit for bit.
#include <cuda_runtime.h>

#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mdg.h"
#include "mdg_internal.cuh"

namespace mdg {
namespace init {

constexpr int kMtN = 624, kMtM = 397;
constexpr uint32_t kMtA = 0x9908b0dfu, kUpper = 0x80000000u, kLower = 0x7fffffffu;
constexpr int kT = 256;

__device__ __forceinline__ uint32_t mt_temper(uint32_t y) {
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return y;
}

__device__ __forceinline__ uint32_t mt_next(const uint32_t *mt, int i, int j, int k) {
  const uint32_t y = (mt[i] & kUpper) | (mt[j] & kLower);
  return mt[k] ^ (y >> 1) ^ ((y & 1u) ? kMtA : 0u);
}

// The first `count` outputs of mt19937(seed), one block of >= 624 threads.
__global__ void k_mt_words(uint32_t seed, long long count, uint32_t *out) {
  __shared__ uint32_t mt[kMtN];
  const int t = threadIdx.x;
  if (t == 0) {
    mt[0] = seed;
    for (int i = 1; i < kMtN; i++) mt[i] = 1812433253u * (mt[i - 1] ^ (mt[i - 1] >> 30)) + (uint32_t)i;
  }
  __syncthreads();
  for (long long base = 0; base < count; base += kMtN) {
    // in-place twist i = 0..623 in order: i < 227 reads old words only;
    // 227 <= i < 454 reads the new words of the first range; 454 <= i < 623
    // those of the second; i = 623 reads new words 0 and 396
    uint32_t v = 0;
    if (t < 227) v = mt_next(mt, t, t + 1, t + kMtM);
    __syncthreads();
    if (t < 227) mt[t] = v;
    __syncthreads();
    if (t >= 227 && t < 454) v = mt_next(mt, t, t + 1, t - 227);
    __syncthreads();
    if (t >= 227 && t < 454) mt[t] = v;
    __syncthreads();
    if (t >= 454 && t < 623) v = mt_next(mt, t, t + 1, t - 227);
    __syncthreads();
    if (t >= 454 && t < 623) mt[t] = v;
    __syncthreads();
    if (t == 0) mt[623] = mt_next(mt, 623, 0, 396);
    __syncthreads();
    if (t < kMtN && base + t < count) out[base + t] = mt_temper(mt[t]);
    __syncthreads();
  }
}

// uniform_real_distribution<double>(0, 1) of draw k: words 2k, 2k + 1.
__device__ __forceinline__ double canonical(const uint32_t *w, long long k) {
  const double sum = __dadd_rn((double)w[2 * k], __dmul_rn((double)w[2 * k + 1], 4294967296.0));
  const double r = sum * 5.421010862427522170037e-20;  // 2^-64, exact
  return r >= 1.0 ? 0.99999999999999988898 : r;        // nextafter(1, 0)
}

// Site v of each deletion draw and the earliest draw of every site.
__global__ void k_draw_sites(const uint32_t *w, long long draws, int n_full, int *site, int *first) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < draws; k += (long long)gridDim.x * blockDim.x) {
    int v = (int)(unsigned long)(__dmul_rn((double)n_full, canonical(w, k)));
    v = v < n_full ? v : n_full - 1;  // bounds guard; a draw this close to 1 has probability 2^-64
    site[k] = v;
    atomicMin(&first[v], (int)k);
  }
}

__global__ void k_fill(int *a, long long n, int v) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    a[i] = v;
}

// flag[k] = draw k is the first draw of its site
__global__ void k_first_flags(const int *site, const int *first, long long draws, int *flag) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < draws; k += (long long)gridDim.x * blockDim.x)
    flag[k] = first[site[k]] == (int)k ? 1 : 0;
}

// Inclusive scan of a[0..n) in place (block sums in aux, sized for the grid).
__global__ void k_scan_blocks(int *a, long long n, int *aux) {
  __shared__ int sh[kT];
  const long long i = blockIdx.x * (long long)kT + threadIdx.x;
  int x = i < n ? a[i] : 0;
  sh[threadIdx.x] = x;
  __syncthreads();
  for (int o = 1; o < kT; o <<= 1) {
    const int y = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
    __syncthreads();
    sh[threadIdx.x] += y;
    __syncthreads();
  }
  if (i < n) a[i] = sh[threadIdx.x];
  if (threadIdx.x == kT - 1) aux[blockIdx.x] = sh[kT - 1];
}

__global__ void k_scan_add(int *a, long long n, const int *aux_scanned) {
  const long long i = blockIdx.x * (long long)kT + threadIdx.x;
  if (i < n && blockIdx.x > 0) a[i] += aux_scanned[blockIdx.x - 1];
}

// The draw at which the n_delete-th distinct site appears: flag_scan is the
// inclusive count of first draws.
__global__ void k_cut(const int *flag_scan, const int *flag, long long draws, int n_delete, long long *cut) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < draws; k += (long long)gridDim.x * blockDim.x)
    if (flag[k] && flag_scan[k] == n_delete) *cut = k + 1;
}

struct Lattice {
  double s, hs, e;    // spacing (the makers use one spacing for all axes), half, offset
  double ox, oy, oz;  // unit origin
  int sx, sy, sz;     // cells per side
  int pad;
  // collision maker: two balls of radius br at centres bc[0], bc[1], each with
  // per_ball sites; the box [0, L) the reference's unit accepts
  double bc[2][3], br, L[3];
  long long per_ball;
};

// Position of site n in the makers' loop order (iz, iy, ix, then the four
// sub-sites), with the reference's operations.
__device__ __forceinline__ void site_pos(const Lattice &l, long long n, double x[3]) {
  const int sub = (int)(n & 3);
  const long long c = n >> 2;
  const int ix = (int)(c % l.sx);
  const long long r = c / l.sx;
  const int iy = (int)(r % l.sy), iz = (int)(r / l.sy);
  // every product and sum rounded on its own, as the reference computes them
  const double bx = __dadd_rn(l.ox, __dmul_rn((double)ix, l.s)), by = __dadd_rn(l.oy, __dmul_rn((double)iy, l.s)),
               bz = __dadd_rn(l.oz, __dmul_rn((double)iz, l.s));
  const bool hx = sub >= 2, hy = sub == 1 || sub == 3, hz = sub == 1 || sub == 2;
  // the half spacing is added only to the shifted coordinates, then e
  x[0] = hx ? __dadd_rn(bx, l.hs) : bx;
  x[1] = hy ? __dadd_rn(by, l.hs) : by;
  x[2] = hz ? __dadd_rn(bz, l.hs) : bz;
  if (l.e != 0.0) {
    x[0] = __dadd_rn(x[0], l.e);
    x[1] = __dadd_rn(x[1], l.e);
    x[2] = __dadd_rn(x[2], l.e);
  }
}

// Site n of the collision maker (BallAdder::Execute, collision.cc:34-50): the
// first ball's sites, then the second's; per ball is^3 cells in (iz, iy, ix)
// order, each giving its corner x1 = ix s - r + c, then x1 shifted by s/2
// along x, along y, along z.  Returns the ball.
__device__ __forceinline__ int ball_pos(const Lattice &l, long long n, double x[3]) {
  const int b = n >= l.per_ball ? 1 : 0;
  const long long m = b ? n - l.per_ball : n;
  const int sub = (int)(m & 3);
  const long long c = m >> 2;
  const int ix = (int)(c % l.sx);
  const long long r = c / l.sx;
  const int iy = (int)(r % l.sx), iz = (int)(r / l.sx);
  const double *cb = l.bc[b];
  x[0] = __dadd_rn(__dsub_rn(__dmul_rn((double)ix, l.s), l.br), cb[0]);
  x[1] = __dadd_rn(__dsub_rn(__dmul_rn((double)iy, l.s), l.br), cb[1]);
  x[2] = __dadd_rn(__dsub_rn(__dmul_rn((double)iz, l.s), l.br), cb[2]);
  if (sub > 0) x[sub - 1] = __dadd_rn(x[sub - 1], l.hs);
  return b;
}

// keep[n] for every site: 0 deleted / outside, 1 kept.
__global__ void k_keep(Lattice l, long long n_sites, int mode, const int *first, long long cut, double cx, double r2max,
                       int *keep) {
  for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < n_sites;
       n += (long long)gridDim.x * blockDim.x) {
    int k = 1;
    if (mode == 1) {
      k = first[n] < cut ? 0 : 1;
    } else if (mode == 2) {
      double x[3];
      site_pos(l, n, x);
      const double dx = __dsub_rn(x[0], cx), dy = __dsub_rn(x[1], cx), dz = __dsub_rn(x[2], cx);
      k = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)) < r2max ? 1 : 0;
    } else if (mode == 3) {
      // BallAdder::Add (collision.cc:23-31): r^2 <= r*r, then MDUnit::AddParticle's
      // MDRect::IsInside (mdunit.cc:44-49, mdrect.h:35-38) for the unit [0, L)
      double x[3];
      const double *c = l.bc[ball_pos(l, n, x)];
      const double dx = __dsub_rn(x[0], c[0]), dy = __dsub_rn(x[1], c[1]), dz = __dsub_rn(x[2], c[2]);
      const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
      const bool inside = 0.0 <= x[0] && x[0] < l.L[0] && 0.0 <= x[1] && x[1] < l.L[1] && 0.0 <= x[2] && x[2] < l.L[2];
      k = (!(r2 > r2max) && inside) ? 1 : 0;
    }
    keep[n] = k;
  }
}

// Writes the kept sites in order; p4 (when given) receives the velocities the
// maker sets: (+speed, 0, 0) for the first ball and (-speed, 0, 0) for the
// second (mode 3), zero otherwise.
__global__ void k_emit(Lattice l, long long n_sites, int mode, const int *keep, const int *keep_scan, double4_32a *q4,
                       double4_32a *p4, double speed, int cap) {
  for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < n_sites;
       n += (long long)gridDim.x * blockDim.x) {
    if (!keep[n]) continue;
    const int slot = keep_scan[n] - 1;
    if (slot >= cap) continue;
    double x[3];
    double vx = 0.0;
    if (mode == 3) {
      vx = ball_pos(l, n, x) == 0 ? speed : -speed;
    } else {
      site_pos(l, n, x);
    }
    q4[slot] = make_double4_32a(x[0], x[1], x[2], 0.0);
    if (p4) p4[slot] = make_double4_32a(vx, 0.0, 0.0, 0.0);
  }
}

// SetInitialVelocity: draws 2i (z) and 2i + 1 (phi) of mt19937(seed).
__global__ void k_velocity(const uint32_t *w, int n, double v0, double4_32a *p4) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double z = __dsub_rn(__dmul_rn(canonical(w, 2LL * i), 2.0), 1.0);
    const double phi = __dmul_rn(__dmul_rn(canonical(w, 2LL * i + 1), 2.0), 3.14159265358979323846);
    const double sz = sqrt(__dsub_rn(1.0, __dmul_rn(z, z)));
    p4[i] = make_double4_32a(v0 * sz * cos(phi), v0 * sz * sin(phi), v0 * z, 0.0);
  }
}

__global__ void k_mean_sub(double4_32a *p4, int n) {
  __shared__ double sh[3][32];
  __shared__ double mean[3];
  double s[3] = {0.0, 0.0, 0.0};
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double4_32a v = p4[i];
    s[0] += v.x;
    s[1] += v.y;
    s[2] += v.z;
  }
  for (int d = 0; d < 3; d++) {
    double v = s[d];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sh[d][threadIdx.x >> 5] = v;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sh[threadIdx.x][w];
    mean[threadIdx.x] = t / (double)n;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double4_32a v = p4[i];
    v.x -= mean[0];
    v.y -= mean[1];
    v.z -= mean[2];
    p4[i] = v;
  }
}

int grid_for(long long n) {
  long long g = (n + kT - 1) / kT;
  return (int)(g < 1 ? 1 : (g > 4096 ? 4096 : g));
}

struct Buf {
  std::vector<void *> ptrs;
  ~Buf() {
    for (void *p : ptrs) cudaFree(p);
  }
  template <class T>
  cudaError_t get(T **p, size_t n) {
    cudaError_t e = cudaMalloc((void **)p, (n ? n : 1) * sizeof(T));
    if (e == cudaSuccess) ptrs.push_back(*p);
    return e;
  }
};

// Inclusive scan of a[0..n) on the stream (recursive over block sums).
cudaError_t scan(int *a, long long n, cudaStream_t s, Buf &buf) {
  const long long nb = (n + kT - 1) / kT;
  int *aux = nullptr;
  cudaError_t e = buf.get(&aux, (size_t)nb);
  if (e != cudaSuccess) return e;
  k_scan_blocks<<<(unsigned)nb, kT, 0, s>>>(a, n, aux);
  if (nb > 1) {
    e = scan(aux, nb, s, buf);
    if (e != cudaSuccess) return e;
    k_scan_add<<<(unsigned)nb, kT, 0, s>>>(a, n, aux);
  }
  return cudaGetLastError();
}

cudaError_t mt_words(uint32_t seed, long long count, uint32_t *out, cudaStream_t s) {
  k_mt_words<<<1, 640, 0, s>>>(seed, count, out);
  return cudaGetLastError();
}

}  // namespace init
}  // namespace mdg

using namespace mdg::init;

extern "C" {

int mdg_make_configuration(const double box[3], int32_t maker, double density, double radius, int32_t unit_id,
                           double speed, double *q4_dev, double *p4_dev, int32_t capacity, int32_t *n, void *stream) {
  if (!box || !n || !(density > 0.0) || capacity < 0 || maker < MDG_MAKER_FCC || maker > MDG_MAKER_COLLISION)
    return MDG_ERR_INVALID;
  if (maker == MDG_MAKER_COLLISION && !(radius > 0.0)) return MDG_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  Buf buf;
  Lattice l;
  memset(&l, 0, sizeof l);
  // lattice spacing from the density: s = 1 / (rho / 4)^(1/3) (confmaker.cc:12)
  const double s0 = 1.0 / pow(density * 0.25, 1.0 / 3.0);
  long long n_sites = 0;
  int mode = 0;
  const int *first = nullptr;
  long long cut = 0;
  if (maker == MDG_MAKER_EXTRACT) {
    // a unit that spans the box: w = L, origin 0 (confmaker.cc:176-252)
    const double *w = box;
    l.sx = (int)(unsigned long)(w[0] / s0) + 1;
    l.sy = (int)(unsigned long)(w[1] / s0) + 1;
    l.sz = (int)(unsigned long)(w[2] / s0) + 1;
    const long long nf = (long long)l.sx * l.sy * l.sz * 4;
    if (nf > INT_MAX) return MDG_ERR_CAPACITY;
    const int n_full = (int)nf;
    const int n_exact = (int)(w[0] * w[1] * w[2] * density);
    const int n_delete = n_full - n_exact;
    l.s = w[0] / (double)l.sx;
    l.hs = l.s * 0.5;
    l.e = 0.0;
    n_sites = n_full;
    mode = 1;
    int *d_first = nullptr;
    if (buf.get(&d_first, (size_t)n_full) != cudaSuccess) return MDG_ERR_CUDA;
    k_fill<<<grid_for(n_full), kT, 0, s>>>(d_first, n_full, INT_MAX);
    if (n_delete > 0) {
      // enough draws for n_delete distinct sites: grow until found
      for (long long draws = 2LL * n_delete + 4096;; draws *= 2) {
        if (draws > (1LL << 31)) return MDG_ERR_CAPACITY;
        Buf round;
        uint32_t *words = nullptr;
        int *site = nullptr, *flag = nullptr, *scanned = nullptr;
        long long *d_cut = nullptr;
        if (round.get(&words, (size_t)(2 * draws)) != cudaSuccess || round.get(&site, (size_t)draws) != cudaSuccess ||
            round.get(&flag, (size_t)draws) != cudaSuccess || round.get(&scanned, (size_t)draws) != cudaSuccess ||
            round.get(&d_cut, 1) != cudaSuccess)
          return MDG_ERR_CUDA;
        k_fill<<<grid_for(n_full), kT, 0, s>>>(d_first, n_full, INT_MAX);
        if (mt_words((uint32_t)unit_id, 2 * draws, words, s) != cudaSuccess) return MDG_ERR_CUDA;
        k_draw_sites<<<grid_for(draws), kT, 0, s>>>(words, draws, n_full, site, d_first);
        k_first_flags<<<grid_for(draws), kT, 0, s>>>(site, d_first, draws, flag);
        if (cudaMemcpyAsync(scanned, flag, (size_t)draws * sizeof(int), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
          return MDG_ERR_CUDA;
        if (scan(scanned, draws, s, round) != cudaSuccess) return MDG_ERR_CUDA;
        long long zero = 0;
        if (cudaMemcpyAsync(d_cut, &zero, sizeof zero, cudaMemcpyHostToDevice, s) != cudaSuccess) return MDG_ERR_CUDA;
        k_cut<<<grid_for(draws), kT, 0, s>>>(scanned, flag, draws, n_delete, d_cut);
        if (cudaMemcpyAsync(&cut, d_cut, sizeof cut, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
          return MDG_ERR_CUDA;
        if (cut > 0) break;
      }
    }
    first = d_first;
  } else if (maker == MDG_MAKER_COLLISION) {
    // Collision::Run (collision.cc:55-63): balls at (L/4, L/2, L/2) and
    // (3L/4, L/2, L/2); BallAdder::Execute: is = int(2 r / s) cells per side
    const double is = 2.0 * radius / s0;
    if (!(is < 1024.0)) return MDG_ERR_CAPACITY;
    l.sx = l.sy = l.sz = (int)is;
    l.s = s0;
    l.hs = s0 * 0.5;
    l.br = radius;
    for (int d = 0; d < 3; d++) {
      l.bc[0][d] = box[d] * (d == 0 ? 0.25 : 0.5);
      l.bc[1][d] = box[d] * (d == 0 ? 0.75 : 0.5);
      l.L[d] = box[d];
    }
    l.per_ball = (long long)l.sx * l.sx * l.sx * 4;
    n_sites = 2 * l.per_ball;
    mode = 3;
  } else {
    // ConfigurationMaker / DropletMaker: floor(L / s) cells per side, offset 1e-7
    l.sx = (int)(box[0] / s0);
    l.sy = (int)(box[1] / s0);
    l.sz = (int)(box[2] / s0);
    l.s = s0;
    l.hs = s0 * 0.5;
    l.e = 0.0000001;
    n_sites = (long long)l.sx * l.sy * l.sz * 4;
    mode = maker == MDG_MAKER_DROPLET ? 2 : 0;
  }
  if (n_sites > INT_MAX) return MDG_ERR_CAPACITY;
  int *keep = nullptr, *keep_scan = nullptr;
  if (buf.get(&keep, (size_t)n_sites) != cudaSuccess || buf.get(&keep_scan, (size_t)n_sites) != cudaSuccess)
    return MDG_ERR_CUDA;
  const double c = box[0] * 0.5;
  if (n_sites > 0) k_keep<<<grid_for(n_sites), kT, 0, s>>>(l, n_sites, mode, first, cut, c, radius * radius, keep);
  if (cudaMemcpyAsync(keep_scan, keep, (size_t)n_sites * sizeof(int), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
    return MDG_ERR_CUDA;
  if (n_sites > 0 && scan(keep_scan, n_sites, s, buf) != cudaSuccess) return MDG_ERR_CUDA;
  int count = 0;
  if (n_sites > 0 &&
      cudaMemcpyAsync(&count, keep_scan + (n_sites - 1), sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return MDG_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return MDG_ERR_CUDA;
  *n = count;
  if (count > capacity) return MDG_ERR_CAPACITY;
  if (count > 0) {
    if (!q4_dev) return MDG_ERR_INVALID;
    k_emit<<<grid_for(n_sites), kT, 0, s>>>(l, n_sites, mode, keep, keep_scan, (double4_32a *)q4_dev,
                                            (double4_32a *)p4_dev, speed, capacity);
  }
  if (cudaStreamSynchronize(s) != cudaSuccess) return MDG_ERR_CUDA;
  return cudaGetLastError() == cudaSuccess ? MDG_OK : MDG_ERR_CUDA;
}

int mdg_make_velocity(double v0, int32_t seed, double *p4_dev, int32_t n, void *stream) {
  if (!p4_dev || n <= 0) return MDG_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  Buf buf;
  uint32_t *words = nullptr;
  if (buf.get(&words, (size_t)4 * n) != cudaSuccess) return MDG_ERR_CUDA;
  if (mt_words((uint32_t)seed, 4LL * n, words, s) != cudaSuccess) return MDG_ERR_CUDA;
  k_velocity<<<grid_for(n), kT, 0, s>>>(words, n, v0, (double4_32a *)p4_dev);
  k_mean_sub<<<1, 1024, 0, s>>>((double4_32a *)p4_dev, n);
  if (cudaStreamSynchronize(s) != cudaSuccess) return MDG_ERR_CUDA;
  return cudaGetLastError() == cudaSuccess ? MDG_OK : MDG_ERR_CUDA;
}

}  // extern "C"
