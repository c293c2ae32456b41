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
// so the result is the exact set at float cost.
#include "mdg_internal.cuh"

namespace mdg {

namespace {

constexpr int kListThreads = 128;

__global__ void __launch_bounds__(kListThreads) k_build_list(Geom g, Dev d) {
  DevFlags *f = d.flags;
  if (f->halt != 0 || f->rebuild == 0) return;
  unsigned long long tot = 0;
  int mx = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < g.n; i += gridDim.x * blockDim.x) {
    int cnt = 0;
    const float4 fi = d.qf[i];
    const int c = d.cell[i];
    const int cx = c % g.nc[0], t = c / g.nc[0], cy = t % g.nc[1], cz = t / g.nc[1];
    for (int oz = -1; oz <= 1; oz++) {
      int nz = cz + oz, sz = 0;
      if (nz < 0) { nz += g.nc[2]; sz = -1; } else if (nz >= g.nc[2]) { nz -= g.nc[2]; sz = 1; }
      // offset of the partner cell's centre: oz*w + sz*(L - nc*w)
      const float offz = (float)oz * g.w32[2] + (float)sz * g.dl32[2];
      for (int oy = -1; oy <= 1; oy++) {
        int ny = cy + oy, sy = 0;
        if (ny < 0) { ny += g.nc[1]; sy = -1; } else if (ny >= g.nc[1]) { ny -= g.nc[1]; sy = 1; }
        const float offy = (float)oy * g.w32[1] + (float)sy * g.dl32[1];
        for (int ox = -1; ox <= 1; ox++) {
          int nx = cx + ox, sx = 0;
          if (nx < 0) { nx += g.nc[0]; sx = -1; } else if (nx >= g.nc[0]) { nx -= g.nc[0]; sx = 1; }
          const float offx = (float)ox * g.w32[0] + (float)sx * g.dl32[0];
          const int cc = (nz * g.nc[1] + ny) * g.nc[0] + nx;
          const int a = d.cell_start[cc], b = d.cell_start[cc + 1];
          const float fx = offx - fi.x, fy = offy - fi.y, fz = offz - fi.z;
          const uint32_t code = entry_pack(0, ox, oy, oz);
          const bool self_cell = (sx | sy | sz) == 0;
          for (int j = a; j < b; j++) {
            const float4 fj = d.qf[j];
            const float ex = fj.x + fx, ey = fj.y + fy, ez = fj.z + fz;
            const float r2f = ex * ex + ey * ey + ez * ez;
            if (r2f > g.acc_hi) continue;
            if (self_cell && j == i) continue;
            if (r2f < g.acc_lo) {
              if (cnt < g.list_cap) d.nl[(size_t)cnt * g.stride + i] = ((uint32_t)j << kCodeBits) | code;
              cnt++;
              continue;
            }
            const double4_32a qi = d.q_end[i];
            const double4_32a qj = d.q_end[j];
            const double xj = sx ? __dadd_rn(qj.x, sx > 0 ? g.L[0] : -g.L[0]) : qj.x;
            const double yj = sy ? __dadd_rn(qj.y, sy > 0 ? g.L[1] : -g.L[1]) : qj.y;
            const double zj = sz ? __dadd_rn(qj.z, sz > 0 ? g.L[2] : -g.L[2]) : qj.z;
            const double dx = __dsub_rn(qi.x, xj), dy = __dsub_rn(qi.y, yj), dz = __dsub_rn(qi.z, zj);
            const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
            if (r2 > g.sl2) continue;
            if (cnt < g.list_cap) d.nl[(size_t)cnt * g.stride + i] = ((uint32_t)j << kCodeBits) | code;
            cnt++;
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
  int grid = (g.n + kListThreads - 1) / kListThreads;
  if (grid > num_sms * 16) grid = num_sms * 16;
  k_build_list<<<grid > 0 ? grid : 1, kListThreads, 0, s>>>(g, d);
  k_rebuild_done<<<1, 1, 0, s>>>(d.flags, in_step ? 1 : 0);
}

}  // namespace mdg
