// Pair-list rebuild, part 2: the padded neighbour list.
//
// Replaces MeshList::SearchMesh / AppendList / RegisterPair and the COO->CSR
// step of MeshList::MakeList (meshlist.cc:57-87, 207-310) together with the
// ghost images of MDManager::MakePairList (mdmanager.cc:262-280,
// mdunit.cc:125-191).  Instead of ghost copies each slot scans the 27 cells
// around its own with periodic wrap and records every partner image within
// the search length rc + margin: a full (both directions) list, so the force
// kernel gathers without atomics.
//
// Acceptance is decided exactly as the reference decides it: the image
// position is formed first, q_j +- L (mdunit.cc:167), then the difference and
// r2 = dx*dx + dy*dy + dz*dz with every operation rounded separately
// (meshlist.cc:262-266), accepted when r2 <= SL^2.  Candidates are first
// measured in float from home-cell-local positions, whose r2 is within 1e-5
// of the exact value; only those within 1e-4 of SL^2 take the double test,
// so the result is the exact set at float cost.  The order of the entries in
// a row (stencil cell by cell, near side first) carries no meaning.
#include "mdg_internal.cuh"

namespace mdg {

namespace {

// Threads per block of the list build.  A block's slots are consecutive in
// cell order, so larger blocks keep more neighbouring cells on one SM and
// their candidate loads hit L1; at 78 registers two 384-thread blocks fit an
// SM (forced rebuild of the 4M-atom liquid box: 128 threads 3.70 ms, 256
// 3.58, 384 3.49, 512 3.81 with one block per SM).
#ifndef MDG_LIST_THREADS
#define MDG_LIST_THREADS 384
#endif
constexpr int kListThreads = MDG_LIST_THREADS;
#ifndef MDG_LIST_MIN_BLOCKS
#define MDG_LIST_MIN_BLOCKS 1
#endif
#ifndef MDG_LIST_UNROLL
#define MDG_LIST_UNROLL 4
#endif
constexpr int kListUnroll = MDG_LIST_UNROLL;

// Exact acceptance of a candidate in the float band: the reference's image
// and rounding order (mdunit.cc:167, meshlist.cc:262-266).
__device__ __forceinline__ bool exact_within(const Geom &g, const double4_32a &qi, const double4_32a &qj, int sx, int sy,
                                             int sz) {
  const double xj = sx ? __dadd_rn(qj.x, sx > 0 ? g.L[0] : -g.L[0]) : qj.x;
  const double yj = sy ? __dadd_rn(qj.y, sy > 0 ? g.L[1] : -g.L[1]) : qj.y;
  const double zj = sz ? __dadd_rn(qj.z, sz > 0 ? g.L[2] : -g.L[2]) : qj.z;
  const double dx = __dsub_rn(qi.x, xj), dy = __dsub_rn(qi.y, yj), dz = __dsub_rn(qi.z, zj);
  const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
  return r2 <= g.sl2;
}

// One thread per slot; each stencil cell's candidates are read kListUnroll at
// a time (independent loads in flight), then tested in order.
__global__ void __launch_bounds__(kListThreads, MDG_LIST_MIN_BLOCKS) k_build_list(Geom g, Dev d) {
  DevFlags *f = d.flags;
  // one read for the whole block: another block may set the halt meanwhile
  __shared__ int s_run;
  if (threadIdx.x == 0) s_run = f->halt == 0 && f->rebuild != 0;
  __syncthreads();
  if (!s_run) return;
  unsigned long long tot = 0;
  int mx = 0;
  const float acc_lo = g.acc_lo, acc_hi = g.acc_hi;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < g.n; i += gridDim.x * blockDim.x) {
    int cnt = 0;
    const float4 fi = d.qf[i];
    int cx, cy, cz;
    cell_unpack(fi.w, cx, cy, cz);
    uint32_t *row = d.nl + i;
    const size_t stride = (size_t)g.stride;
    const int cap = g.list_cap;
    for (int oz = -1; oz <= 1; oz++) {
      int nz = cz + oz, sz = 0;
      if (nz < 0) { nz += g.nc[2]; sz = -1; } else if (nz >= g.nc[2]) { nz -= g.nc[2]; sz = 1; }
      // offset of the partner cell's centre: oz*w + sz*(L - nc*w)
      const float fz = (float)oz * g.w32[2] + (float)sz * g.dl32[2] - fi.z;
      for (int oy = -1; oy <= 1; oy++) {
        int ny = cy + oy, sy = 0;
        if (ny < 0) { ny += g.nc[1]; sy = -1; } else if (ny >= g.nc[1]) { ny -= g.nc[1]; sy = 1; }
        const float fy = (float)oy * g.w32[1] + (float)sy * g.dl32[1] - fi.y;
        for (int ox = -1; ox <= 1; ox++) {
          int nx = cx + ox, sx = 0;
          if (nx < 0) { nx += g.nc[0]; sx = -1; } else if (nx >= g.nc[0]) { nx -= g.nc[0]; sx = 1; }
          const float fx = (float)ox * g.w32[0] + (float)sx * g.dl32[0] - fi.x;
          const int cc = cell_rank(g, nx, ny, nz);
          if (!MDG_IN_RANGE(f, kCheckBuildCell, cc, g.nrank)) continue;
          int a = d.cell_start[cc], b = d.cell_start[cc + 1];
          if (!MDG_IN_RANGE(f, kCheckBuildRange, b, g.n + 1) || !MDG_IN_RANGE(f, kCheckBuildRange, a, b + 1)) a = b = 0;
          const uint32_t code = entry_pack(0, ox, oy, oz);
          for (int j0 = a; j0 < b; j0 += kListUnroll) {
            float4 fj[kListUnroll];
#pragma unroll
            for (int u = 0; u < kListUnroll; u++)
              fj[u] = j0 + u < b ? d.qf[j0 + u] : make_float4(1e30f, 0.f, 0.f, 0.f);
#pragma unroll
            for (int u = 0; u < kListUnroll; u++) {
              const int j = j0 + u;
              const float ex = fj[u].x + fx, ey = fj[u].y + fy, ez = fj[u].z + fz;
              const float r2f = fmaf(ez, ez, fmaf(ey, ey, ex * ex));
              if (r2f > acc_hi || j == i) continue;
              bool take = r2f < acc_lo;
              if (!take) take = exact_within(g, d.q_end[i], d.q_end[j], sx, sy, sz);
              if (take) {
                if (cnt < cap) row[(size_t)cnt * stride] = ((uint32_t)j << kCodeBits) | code;
                cnt++;
              }
            }
          }
        }
      }
    }
    d.ncount[i] = cnt < g.list_cap ? cnt : g.list_cap;
    if (cnt > g.list_cap) {
      atomicMax(&f->overflow_max, cnt);
      halt_with(f, kHaltOverflow);
    }
    tot += (unsigned long long)(cnt < g.list_cap ? cnt : g.list_cap);
    mx = max(mx, cnt);
  }
  // block totals -> one atomic each
  __shared__ unsigned long long s_sum[kListThreads / 32];
  __shared__ int s_max[kListThreads / 32];
  unsigned long long v = tot;
  int m = mx;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v += __shfl_down_sync(0xffffffffu, v, o);
    m = max(m, __shfl_down_sync(0xffffffffu, m, o));
  }
  if ((threadIdx.x & 31) == 0) { s_sum[threadIdx.x >> 5] = v; s_max[threadIdx.x >> 5] = m; }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long tv = 0;
    int tm = 0;
    for (int w = 0; w < kListThreads / 32; w++) { tv += s_sum[w]; tm = max(tm, s_max[w]); }
    atomicAdd(&f->pairs, tv);
    atomicMax(&f->max_count, tm);
  }
}

// A new outer list always gets a fresh inner list: in this step's kernel
// when the rebuild ran inside a step, otherwise in the next step's.
__global__ void k_rebuild_done(DevFlags *f, int in_step) {
  if (f->halt == 0 && f->rebuild) {
    f->rebuild = 0;
    f->rebuilds += 1;
    if (!in_step) {
      f->prune_next = 1;
    } else if (!f->prune_now) {
      f->prune_now = 1;
      f->prunes += 1;
      f->inner_pairs = 0;
    }
  }
}

__global__ void k_list_prepare(DevFlags *f) {
  if (f->halt == 0 && f->rebuild) {
    f->pairs = 0;
    f->max_count = 0;
  }
}

}  // namespace

void launch_build_list(const Geom &g, const Dev &d, int num_sms, cudaStream_t s, bool in_step) {
  k_list_prepare<<<1, 1, 0, s>>>(d.flags);
  // one slot per thread: the blocks' work is uneven (denser regions have more
  // candidates), and many blocks balance it where a grid of 16 blocks per SM
  // striding over the slots did not (128-thread blocks, forced rebuild of the
  // 4M-atom liquid box: 3.70 against 3.98 ms; one wave of resident blocks:
  // 4.67 ms)
  (void)num_sms;
  const int grid = (g.n + kListThreads - 1) / kListThreads;
  k_build_list<<<grid > 0 ? grid : 1, kListThreads, 0, s>>>(g, d);
  k_rebuild_done<<<1, 1, 0, s>>>(d.flags, in_step ? 1 : 0);
}

}  // namespace mdg
