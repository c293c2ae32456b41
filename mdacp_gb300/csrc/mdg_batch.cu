// Batched replicas: many independent periodic LJ boxes of uneven size,
// density and temperature advanced together, one persistent kernel per step.
//
// No reference counterpart (a new pattern on top of the drop-in): each box is
// what one MDACP run does (NVE drift-kick-drift, cell list + Verlet list with a
// margin, the same smoothly truncated potential), but a thousand of them share
// the GPU.  Design:
//   * the grid is a few CTAs per SM; each CTA owns a fixed list of boxes
//     assigned longest-first to the least-loaded CTA (host, deterministic);
//   * a CTA advances each of its boxes by one step (the fused force/kick/
//     drift over the box);
//   * a box whose displacement test fired is rebuilt at the start of the next
//     step by kernels ahead of the persistent one: k_batch_rebuild_set (the
//     rebuilding boxes and their slot prefix), k_batch_bin (one thread per
//     particle of every rebuilding box: wrap and home cell), k_batch_sort (one
//     CTA per rebuilding box: counting sort with the cell counters in shared
//     memory, each cell in id order), k_batch_place (one thread per particle:
//     the reordered state and its float positions) and k_batch_list (one
//     thread per particle, same float-first exact acceptance test as the
//     single-box path), so a rebuild is spread over the whole GPU instead of
//     stalling the CTA that steps the box;
//   * lanes-per-particle (1, 2 or 4 lanes share one particle's row and reduce
//     with shuffles), threads per CTA and CTAs per SM are chosen by the
//     autotuner (mdg_batch_tune);
//   * a box whose row overflows stops (its step counter does not advance) while
//     the others continue; the host regrows the rows and runs catch-up steps
//     that advance only the boxes behind the goal.  No kernel waits on another.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "mdg_internal.cuh"

namespace mdg {
namespace batch {

constexpr int kMaxCellsPerBox = 4096;  // cell counters and starts live in shared memory
constexpr int kErrOverflow = 1, kErrBadState = 2;

struct BoxDesc {
  double L[3];
  double inv_w[3];
  float w32[3];
  float dl32[3];
  int nc[3];
  int ncell;
  int n;
  int atom_off;
  long long list_off;  // first entry of the box in the list pool (n * cap entries)
  int cell_off;        // first cell start of the box (ncell + 1 entries)
  int pad;
};

struct Params {
  double sl2, rc2, c2x8, dt, dt2, half_margin2;
  float acc_lo, acc_hi, rc2f, c2x8f;
  int list_cap;
  int nbox;
  int total;  // particles of all boxes
  // inner list (one lane per particle): the listed pairs within rc + buffer,
  // re-selected when a particle of the box moved buffer / 2 since the last
  // selection, and after every rebuild
  int inner;
  float prune_thr2f, half_prune2;
  double prune_thr2d;
  // mixed forms: q_mid relative to the centre of the slot's home cell, the
  // build and prune references packed in the padding words of q_mid and p
  // (21-bit fixed point per axis in units of w / (2^20 - 1)), q_end not
  // written by the step; the displacement thresholds lowered by two units of
  // the largest cell width
  int local_pos;
  float half_margin2_ref, half_prune2_ref;
};

struct Dev {
  BoxDesc *boxes;
  int *cta_start, *cta_boxes;
  double4_32a *q_end, *q_mid[2], *p, *q_build, *t_q, *t_p;
  float4 *qf, *loc[2];
  int *id, *cell, *t_id, *t_cell, *order, *cell_start;
  uint32_t *nl, *pl;  // outer rows; inner rows in the same layout
  int *ncount, *pcount;
  float4 *loc_p;       // local positions at the last inner-list selection
  int *box_rebuild, *box_err, *box_need, *box_prune;
  // flat layout: raised (plain stores of 1) by any particle of the box during
  // the step, applied by k_batch_finish after it
  int *box_req, *box_preq;
  long long *box_steps, *box_rebuilds, *goal;
  // mixed forms: -1 when the box's q_end is current, else the q_mid slot
  // (0 or 1) its last step wrote, from which q_end is formed when needed
  int *box_mid;
  double *partials;  // per box: KE, PE, virial
  const int *box_of_slot;
  // this step's rebuilding boxes in box order and their first atom in the
  // concatenation of their slots (rb_start[rb_count] = atoms to list)
  int *rb_boxes, *rb_start, *rb_count;
};

// A box takes part in this step's rebuild: flagged, healthy, behind the goal.
__device__ __forceinline__ bool rebuilding(const Dev &d, int bi, long long goal) {
  return d.box_rebuild[bi] != 0 && d.box_err[bi] == 0 && d.box_steps[bi] < goal;
}

__device__ __forceinline__ double rcp_hh3(double x) {
  double y;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  const double e = fma(-x, y, 1.0);
  return fma(y, fma(e, e, e), y);
}

__device__ __forceinline__ void cell_xyz(const BoxDesc &b, int c, int &cx, int &cy, int &cz) {
  cx = c % b.nc[0];
  const int t = c / b.nc[0];
  cy = t % b.nc[1];
  cz = t / b.nc[1];
}

// Centre of the box's cell c along axis k, exact in double.
__device__ __forceinline__ double box_cell_centre(const BoxDesc &b, int k, int c) {
  return ((double)c + 0.5) * (double)b.w32[k];
}

// Mixed forms: a home-cell-local position (|x| < w per axis) packed into the
// bits of a double, 21-bit two's complement fields at bits 0, 21, 42; the
// value is only ever moved, never used in arithmetic.
__device__ __forceinline__ double pack_box_ref(const BoxDesc &b, float x, float y, float z) {
  const long long u = (long long)__float2int_rn(x * (1048575.0f / b.w32[0])) & 0x1FFFFF;
  const long long v = (long long)__float2int_rn(y * (1048575.0f / b.w32[1])) & 0x1FFFFF;
  const long long w = (long long)__float2int_rn(z * (1048575.0f / b.w32[2])) & 0x1FFFFF;
  return __longlong_as_double(u | (v << 21) | (w << 42));
}

__device__ __forceinline__ void unpack_box_ref(const BoxDesc &b, double r, float &x, float &y, float &z) {
  const long long u = __double_as_longlong(r);
  x = (float)(int)((u << 43) >> 43) * (b.w32[0] * (1.0f / 1048575.0f));
  y = (float)(int)((u << 22) >> 43) * (b.w32[1] * (1.0f / 1048575.0f));
  z = (float)(int)((u << 1) >> 43) * (b.w32[2] * (1.0f / 1048575.0f));
}

// Mixed forms: the step-boundary position of slot s from its home-cell-local
// mid-step position in q_mid[mid]: the cell centre plus (q_mid - p dt/2).
__device__ __forceinline__ double4_32a box_end_from_mid(const Params &P, const Dev &d, const BoxDesc &b, int s,
                                                        int mid) {
  const double4_32a u = d.q_mid[mid][s], p = d.p[s];
  int cx, cy, cz;
  cell_xyz(b, d.cell[s], cx, cy, cz);
  double4_32a q = u;
  q.x = box_cell_centre(b, 0, cx) + fma(-p.x, P.dt2, u.x);
  q.y = box_cell_centre(b, 1, cy) + fma(-p.y, P.dt2, u.y);
  q.z = box_cell_centre(b, 2, cz) + fma(-p.z, P.dt2, u.z);
  q.w = 0.0;
  return q;
}

// Exclusive scan over cnt[0..m) in shared memory by the whole CTA; writes the
// starts to out[0..m] (out[m] = total) and zeroes cnt.
__device__ void cta_scan(int *cnt, int *out, int m) {
  __shared__ int warp_tot[32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  for (int base = 0; base < m; base += blockDim.x) {
    const int c = base + threadIdx.x;
    const int v = c < m ? cnt[c] : 0;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[wid] = x;
    __syncthreads();
    if (wid == 0) {
      int t = lane < nw ? warp_tot[lane] : 0;
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, t, o);
        if (lane >= o) t += y;
      }
      if (lane < nw) warp_tot[lane] = t;
    }
    __syncthreads();
    if (c < m) {
      out[c] = carry + (wid ? warp_tot[wid - 1] : 0) + x - v;
      cnt[c] = 0;
    }
    __syncthreads();
    if (threadIdx.x == 0) carry += warp_tot[nw - 1];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[m] = carry;
  __syncthreads();
}

// Slot t of this step's rebuilding boxes (their particles side by side):
// the index k into rb_boxes / rb_start with rb_start[k] <= t < rb_start[k + 1].
__device__ __forceinline__ int rb_find(const Dev &d, int nb, int t) {
  int lo = 0, hi = nb - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (d.rb_start[mid] <= t) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Rebuild part 1, one thread per particle of every rebuilding box (the FP64
// work of a rebuild spread over the GPU: at 1/64 of the FP32 rate one SM
// per box would take ~100 us for 8,000 particles): wrap (one +-L per
// component) and home cell.  A particle outside [-L, 2L) fails its box.
__device__ void bin_particle(const Params &P, const Dev &d, const BoxDesc &b, int bi, int a) {
  const int o = b.atom_off;
  const int mid = d.box_mid[bi];
  double4_32a q = mid >= 0 ? box_end_from_mid(P, d, b, o + a, mid) : d.q_end[o + a];
  double x[3] = {q.x, q.y, q.z};
  int ci[3];
  bool bad = false;
  for (int k = 0; k < 3; k++) {
    double v = x[k];
    if (v < 0.0) v += b.L[k];
    else if (v > b.L[k]) v -= b.L[k];
    if (!(v >= 0.0 && v <= b.L[k])) bad = true;
    x[k] = v;
    int c = bad ? 0 : (int)(v * b.inv_w[k]);
    ci[k] = c < 0 ? 0 : (c >= b.nc[k] ? b.nc[k] - 1 : c);
  }
  if (bad) atomicExch(&d.box_err[bi], kErrBadState);
  q.x = x[0]; q.y = x[1]; q.z = x[2];
  d.q_end[o + a] = q;
  d.cell[o + a] = (ci[2] * b.nc[1] + ci[1]) * b.nc[0] + ci[0];
}

// Rebuild part 2, one CTA per rebuilding box: the integer reorder.  Cell
// counts in shared memory, their scan, then each cell's particles in id order
// (slots and ids scattered per cell, then one thread per particle counting
// the cell's smaller ids: ids are distinct), cell starts, and the particles
// gathered in the new order into the temporaries.
__device__ void sort_box(const Dev &d, const BoxDesc &b, int *s_cnt, int *s_start) {
  const int n = b.n, o = b.atom_off;
  for (int c = threadIdx.x; c < b.ncell; c += blockDim.x) s_cnt[c] = 0;
  __syncthreads();
  for (int a = threadIdx.x; a < n; a += blockDim.x) atomicAdd(&s_cnt[d.cell[o + a]], 1);
  __syncthreads();
  cta_scan(s_cnt, s_start, b.ncell);
  for (int a = threadIdx.x; a < n; a += blockDim.x) {
    const int c = d.cell[o + a];
    const int k = o + s_start[c] + atomicAdd(&s_cnt[c], 1);
    d.t_cell[k] = a;
    d.t_id[k] = d.id[o + a];
  }
  for (int c = threadIdx.x; c < b.ncell; c += blockDim.x) d.cell_start[b.cell_off + c] = s_start[c];
  if (threadIdx.x == 0) d.cell_start[b.cell_off + b.ncell] = n;
  __syncthreads();
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const int v = d.t_cell[o + k], key = d.t_id[o + k];
    const int c = d.cell[o + v];
    const int lo = s_start[c], hi = s_start[c + 1];
    int r = 0;
    for (int m = lo; m < hi; m++) r += d.t_id[o + m] < key ? 1 : 0;
    d.order[o + lo + r] = v;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const int src = o + d.order[o + k];
    d.t_q[o + k] = d.q_end[src];
    d.t_p[o + k] = d.p[src];
    d.t_id[o + k] = d.id[src];
    d.t_cell[o + k] = d.cell[src];
  }
}

// Rebuild part 3, one thread per particle of every rebuilding box: the
// reordered state back in place, with the build-time and mid-step positions.
// Mixed forms: q_mid relative to the home-cell centre, (q - c) + p dt/2,
// with the build position packed in q_mid.w (the rebuild test's reference)
// and in p.w (the prune reference until the step's re-selection records its
// own); q_end is current until the box steps.
__device__ void place_particle(const Params &P, const Dev &d, const BoxDesc &b, int bi, int k, int par) {
  const int o = b.atom_off;
  const double4_32a q = d.t_q[o + k];
  double4_32a p = d.t_p[o + k];
  const int c = d.t_cell[o + k];
  d.q_end[o + k] = q;
  d.id[o + k] = d.t_id[o + k];
  d.cell[o + k] = c;
  if (k == 0) d.box_mid[bi] = -1;
  int cx, cy, cz;
  cell_xyz(b, c, cx, cy, cz);
  const double ox = box_cell_centre(b, 0, cx), oy = box_cell_centre(b, 1, cy), oz = box_cell_centre(b, 2, cz);
  const float4 lb = make_float4((float)(q.x - ox), (float)(q.y - oy), (float)(q.z - oz), 0.0f);
  d.qf[o + k] = lb;
  double4_32a m = q;
  if (P.local_pos) {
    m.x = __dadd_rn(q.x - ox, __dmul_rn(p.x, P.dt2));
    m.y = __dadd_rn(q.y - oy, __dmul_rn(p.y, P.dt2));
    m.z = __dadd_rn(q.z - oz, __dmul_rn(p.z, P.dt2));
    m.w = pack_box_ref(b, lb.x, lb.y, lb.z);
    p.w = m.w;
    d.q_mid[par][o + k] = m;
    d.loc[par][o + k] = make_float4((float)m.x, (float)m.y, (float)m.z, 0.0f);
  } else {
    d.q_build[o + k] = q;
    m.x = __dadd_rn(q.x, __dmul_rn(p.x, P.dt2));
    m.y = __dadd_rn(q.y, __dmul_rn(p.y, P.dt2));
    m.z = __dadd_rn(q.z, __dmul_rn(p.z, P.dt2));
    d.q_mid[par][o + k] = m;
    d.loc[par][o + k] = make_float4((float)(m.x - ox), (float)(m.y - oy), (float)(m.z - oz), 0.0f);
  }
  d.p[o + k] = p;
}

// Pair-list row of local particle a of box b (the box's cell starts and
// build-time positions are in place): the 27 stencil cells with periodic
// wrap, float-first exact acceptance.  Returns the row length (rows longer
// than the capacity are truncated and flag the box).
__device__ int build_row(const Params &P, const Dev &d, const BoxDesc &b, int bi, int a) {
  const int n = b.n, o = b.atom_off;
  const int *cstart = d.cell_start + b.cell_off;
  const float4 fi = d.qf[o + a];
  int cx, cy, cz;
  cell_xyz(b, d.cell[o + a], cx, cy, cz);
  int cnt = 0;
  for (int oz = -1; oz <= 1; oz++) {
    int nz = cz + oz, sz = 0;
    if (nz < 0) { nz += b.nc[2]; sz = -1; } else if (nz >= b.nc[2]) { nz -= b.nc[2]; sz = 1; }
    const float offz = (float)oz * b.w32[2] + (float)sz * b.dl32[2];
    for (int oy = -1; oy <= 1; oy++) {
      int ny = cy + oy, sy = 0;
      if (ny < 0) { ny += b.nc[1]; sy = -1; } else if (ny >= b.nc[1]) { ny -= b.nc[1]; sy = 1; }
      const float offy = (float)oy * b.w32[1] + (float)sy * b.dl32[1];
      for (int ox = -1; ox <= 1; ox++) {
        int nx = cx + ox, sx = 0;
        if (nx < 0) { nx += b.nc[0]; sx = -1; } else if (nx >= b.nc[0]) { nx -= b.nc[0]; sx = 1; }
        const float offx = (float)ox * b.w32[0] + (float)sx * b.dl32[0];
        const int cc = (nz * b.nc[1] + ny) * b.nc[0] + nx;
        const int lo = cstart[cc], hi = cstart[cc + 1];
        const uint32_t code = entry_pack(0, ox, oy, oz);
        const bool self_cell = (sx | sy | sz) == 0;
        const float fx = offx - fi.x, fy = offy - fi.y, fz = offz - fi.z;
        for (int j = lo; j < hi; j++) {
          const float4 fj = d.qf[o + j];
          const float ex = fj.x + fx, ey = fj.y + fy, ez = fj.z + fz;
          const float r2f = ex * ex + ey * ey + ez * ez;
          if (r2f > P.acc_hi) continue;
          if (self_cell && j == a) continue;
          bool take = r2f < P.acc_lo;
          if (!take) {
            const double4_32a qi = d.q_end[o + a], qj = d.q_end[o + j];
            const double xj = sx ? __dadd_rn(qj.x, sx > 0 ? b.L[0] : -b.L[0]) : qj.x;
            const double yj = sy ? __dadd_rn(qj.y, sy > 0 ? b.L[1] : -b.L[1]) : qj.y;
            const double zj = sz ? __dadd_rn(qj.z, sz > 0 ? b.L[2] : -b.L[2]) : qj.z;
            const double dx = __dsub_rn(qi.x, xj), dy = __dsub_rn(qi.y, yj), dz = __dsub_rn(qi.z, zj);
            const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
            take = r2 <= P.sl2;
          }
          if (take) {
            if (cnt < P.list_cap) d.nl[b.list_off + (long long)cnt * n + a] = ((uint32_t)j << kCodeBits) | code;
            cnt++;
          }
        }
      }
    }
  }
  d.ncount[o + a] = cnt < P.list_cap ? cnt : P.list_cap;
  return cnt;
}

// Rebuild part 1 for every box that rebuilds this step: one CTA per box.
// One CTA per rebuilding box; the largest box's serial phases bound the
// kernel, so the CTA is as wide as possible: 1,024 threads measured 1.04 ms per
// step on 1,024 boxes against 1.09 (512) and 1.15 (256).
#ifndef MDG_BATCH_PREP_THREADS
#define MDG_BATCH_PREP_THREADS 1024
#endif
constexpr int kPrepThreads = MDG_BATCH_PREP_THREADS;
constexpr int kBatchKernelsPerStep = 6;  // rebuild set, bin, sort, place, list, step (+ finish in the flat layout)

__global__ void __launch_bounds__(128) k_batch_bin(Params P, Dev d) {
  const int nb = *d.rb_count;
  if (nb == 0) return;
  const int total = d.rb_start[nb];
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
    const int k = rb_find(d, nb, t), bi = d.rb_boxes[k];
    bin_particle(P, d, d.boxes[bi], bi, t - d.rb_start[k]);
  }
}

__global__ void __launch_bounds__(kPrepThreads) k_batch_sort(Dev d) {
  __shared__ int s_cnt[kMaxCellsPerBox];
  __shared__ int s_start[kMaxCellsPerBox + 1];
  const int bi = blockIdx.x;
  if (!rebuilding(d, bi, *d.goal)) return;  // uniform over the CTA; a box failed by k_batch_bin stops here
  const BoxDesc b = d.boxes[bi];
  sort_box(d, b, s_cnt, s_start);
}

__global__ void __launch_bounds__(128) k_batch_place(Params P, Dev d, int par) {
  const int nb = *d.rb_count;
  if (nb == 0) return;
  const int total = d.rb_start[nb];
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
    const int k = rb_find(d, nb, t), bi = d.rb_boxes[k];
    if (d.box_err[bi] == 0) place_particle(P, d, d.boxes[bi], bi, t - d.rb_start[k], par);
  }
}

// Ahead of the rebuild parts: the boxes that rebuild this step, in box order,
// and the prefix of their particle counts (a box the rebuild then fails stays
// in the set; the later parts skip it).  One CTA of 1,024 threads.
__global__ void __launch_bounds__(1024) k_batch_rebuild_set(Params P, Dev d) {
  __shared__ int carry_n, carry_k;
  __shared__ long long wsum[32];
  const long long goal = *d.goal;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (threadIdx.x == 0) carry_n = carry_k = 0;
  __syncthreads();
  for (int base = 0; base < P.nbox; base += blockDim.x) {
    const int bi = base + threadIdx.x;
    const bool on = bi < P.nbox && rebuilding(d, bi, goal);
    const int n = on ? d.boxes[bi].n : 0;
    // inclusive scans of n and of the flag over the CTA, packed in one pass
    long long x = ((long long)n << 20) | (on ? 1 : 0);
    for (int o = 1; o < 32; o <<= 1) {
      const long long y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wsum[wid] = x;
    __syncthreads();
    if (wid == 0) {
      long long t = lane < nw ? wsum[lane] : 0;
      for (int o = 1; o < 32; o <<= 1) {
        const long long y = __shfl_up_sync(0xffffffffu, t, o);
        if (lane >= o) t += y;
      }
      wsum[lane] = t;
    }
    __syncthreads();
    const long long incl = x + (wid ? wsum[wid - 1] : 0);
    const int k = carry_k + (int)(incl & 0xfffff) - 1, start = carry_n + (int)(incl >> 20) - n;
    if (on) {
      d.rb_boxes[k] = bi;
      d.rb_start[k] = start;
    }
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) {
      carry_k += (int)(incl & 0xfffff);
      carry_n += (int)(incl >> 20);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    *d.rb_count = carry_k;
    d.rb_start[carry_k] = carry_n;
  }
}

// Rebuild part 2: one thread per particle slot of every rebuilding box, so a
// box's list is built by the whole GPU rather than by the CTA that steps it.
// A fixed grid walks the concatenated slots of this step's rebuilding boxes.
__global__ void __launch_bounds__(128) k_batch_list(Params P, Dev d) {
  const int nb = *d.rb_count;
  if (nb == 0) return;
  const int total = d.rb_start[nb];
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
    const int lo = rb_find(d, nb, t), bi = d.rb_boxes[lo];
    if (d.box_err[bi] == kErrBadState) continue;
    const BoxDesc &b = d.boxes[bi];
    const int cnt = build_row(P, d, b, bi, t - d.rb_start[lo]);
    if (cnt > P.list_cap) {
      atomicMax(&d.box_need[bi], cnt);
      atomicExch(&d.box_err[bi], kErrOverflow);
    }
  }
}

// Force on local particle a of box b from its row, lanes l = 0..LPI-1 of a group
// taking every LPI-th entry; returns the group sum on every lane.  MODE 0 walks
// the outer row; MODE 1 (one lane per particle) walks the outer row and, when
// `select` is set, copies the entries within the inner radius to the inner row
// (*kept: their number); MODE 2 walks the inner row.
template <int MIXED, int LPI, int MODE>
__device__ __forceinline__ double3 box_force(const Params &P, const Dev &d, const BoxDesc &b, int a, int lane, int par,
                                             bool select = false, int *kept = nullptr) {
  static_assert(MODE == 0 || LPI == 1, "the inner list is kept for one lane per particle");
  const int o = b.atom_off, n = b.n;
  int cx, cy, cz;
  cell_xyz(b, d.cell[o + a], cx, cy, cz);
  const int cnt = MODE == 2 ? d.pcount[o + a] : d.ncount[o + a];
  const uint32_t *row = (MODE == 2 ? d.pl : d.nl) + b.list_off + a;
  uint32_t *prow = d.pl + b.list_off + a;
  int m = 0;
  double fx = 0.0, fy = 0.0, fz = 0.0;
  if (MIXED) {
    const float4 li = d.loc[par][o + a];
    const AxisQuad qx = axis_quad(b.w32[0], b.dl32[0], cx == 0, cx == b.nc[0] - 1, li.x, 1.0f);
    const AxisQuad qy = axis_quad(b.w32[1], b.dl32[1], cy == 0, cy == b.nc[1] - 1, li.y, 0.25f);
    const AxisQuad qz = axis_quad(b.w32[2], b.dl32[2], cz == 0, cz == b.nc[2] - 1, li.z, 0.0625f);
    float sx = 0.f, sy = 0.f, sz = 0.f;
    float cx_ = 0.f, cy_ = 0.f, cz_ = 0.f;  // Kahan corrections (MDG_MIXED)
    const float4 *loc = d.loc[par] + o;
    auto pair = [&](uint32_t e, const float4 &lj) {
      const float tx = step_float(e, 0x03u, 8388609.0f), ty = step_float(e, 0x0Cu, 8388612.0f),
                  tz = step_float(e, 0x30u, 8388624.0f);
      const float dx = lj.x + fmaf(fmaf(qx.b, tx, qx.a), tx, qx.c);
      const float dy = lj.y + fmaf(fmaf(qy.b, ty, qy.a), ty, qy.c);
      const float dz = lj.z + fmaf(fmaf(qz.b, tz, qz.a), tz, qz.c);
      const float r2 = dx * dx + dy * dy + dz * dz;
      if (MODE == 1 && select && r2 <= P.prune_thr2f) prow[(long long)(m++) * n] = e;
      float inv;
      asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(inv) : "f"(r2));
      const float i6 = inv * inv * inv;
      float df = (i6 * inv) * fmaf(-48.0f, i6, 24.0f) + P.c2x8f;
      df = r2 <= P.rc2f ? df : 0.0f;
      if (MIXED == MDG_MIXED) {  // compensated sums, as the single-box mixed form
        kahan_fma(sx, cx_, df, dx);
        kahan_fma(sy, cy_, df, dy);
        kahan_fma(sz, cz_, df, dz);
      } else {
        sx = fmaf(df, dx, sx);
        sy = fmaf(df, dy, sy);
        sz = fmaf(df, dz, sz);
      }
    };
    // this lane's entries lane, lane + LPI, ... in batches of four: the next
    // batch's entries are requested before this batch's positions are used,
    // and the last full batch requests the remainder
    const int mine = cnt > lane ? (cnt - lane + LPI - 1) / LPI : 0;
    const int full = mine - mine % 4;
    uint32_t en[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const int kn = lane + u * LPI;
      en[u] = kn < cnt ? __ldg(row + (long long)kn * n) : 0u;
    }
    int k = lane;
    for (int j = 0; j < full; j += 4, k += 4 * LPI) {
      uint32_t e[4];
      float4 l[4];
#pragma unroll
      for (int u = 0; u < 4; u++) e[u] = en[u];
#pragma unroll
      for (int u = 0; u < 4; u++) l[u] = __ldg(loc + entry_slot(e[u]));
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const int kn = k + (4 + u) * LPI;
        en[u] = kn < cnt ? __ldg(row + (long long)kn * n) : 0u;
      }
#pragma unroll
      for (int u = 0; u < 4; u++) pair(e[u], l[u]);
    }
    if (full < mine) {
      // missing entries get a partner at 1e30: r^2 overflows to +inf, no force
      float4 l[3];
#pragma unroll
      for (int u = 0; u < 3; u++)
        l[u] = k + u * LPI < cnt ? __ldg(loc + entry_slot(en[u])) : make_float4(1e30f, 1e30f, 1e30f, 0.f);
#pragma unroll
      for (int u = 0; u < 3; u++) pair(en[u], l[u]);
    }
    fx = (double)(sx - cx_);
    fy = (double)(sy - cy_);
    fz = (double)(sz - cz_);
  } else {
    const double4_32a qi = d.q_mid[par][o + a];
    const bool edge = cx == 0 || cy == 0 || cz == 0 || cx == b.nc[0] - 1 || cy == b.nc[1] - 1 || cz == b.nc[2] - 1;
    for (int k = lane; k < cnt; k += LPI) {
      const uint32_t e = __ldg(row + (long long)k * n);
      double4_32a qj = ldg4(d.q_mid[par] + o + entry_slot(e));
      if (edge) {
        const int ox = entry_sx(e), oy = entry_sy(e), oz = entry_sz(e);
        if (ox == 0 && cx == 0) qj.x -= b.L[0]; else if (ox == 2 && cx == b.nc[0] - 1) qj.x += b.L[0];
        if (oy == 0 && cy == 0) qj.y -= b.L[1]; else if (oy == 2 && cy == b.nc[1] - 1) qj.y += b.L[1];
        if (oz == 0 && cz == 0) qj.z -= b.L[2]; else if (oz == 2 && cz == b.nc[2] - 1) qj.z += b.L[2];
      }
      const double dx = qj.x - qi.x, dy = qj.y - qi.y, dz = qj.z - qi.z;
      const double r2 = dx * dx + dy * dy + dz * dz;
      // bit-pattern comparisons of r2 >= +0: the integer pipe, not the FP64 one
      const long long r2_bits = __double_as_longlong(r2);
      if (MODE == 1 && select && r2_bits <= __double_as_longlong(P.prune_thr2d)) prow[(long long)(m++) * n] = e;
      if (r2_bits <= __double_as_longlong(P.rc2)) {
        const double inv = rcp_hh3(r2);
        const double i6 = inv * inv * inv;
        const double df = (i6 * inv) * fma(-48.0, i6, 24.0) + P.c2x8;
        fx = fma(df, dx, fx);
        fy = fma(df, dy, fy);
        fz = fma(df, dz, fz);
      }
    }
  }
  if (MODE == 1 && kept) *kept = m;
  if (LPI > 1) {
#pragma unroll
    for (int off = LPI / 2; off > 0; off >>= 1) {
      fx += __shfl_xor_sync(0xffffffffu, fx, off, LPI);
      fy += __shfl_xor_sync(0xffffffffu, fy, off, LPI);
      fz += __shfl_xor_sync(0xffffffffu, fz, off, LPI);
    }
  }
  return make_double3(fx, fy, fz);
}

// Kick, both half-drifts, the displacement and inner-list tests and the
// stores of slot s after its force F (one lane per particle does this).
template <int MIXED, bool INNER>
__device__ __forceinline__ void advance_particle(const Params &P, const Dev &d, const BoxDesc &b, int s,
                                                 const double3 &F, int par, bool sel, int kept, bool &rebuild,
                                                 bool &reselect) {
  const bool inner = INNER;
  double4_32a p = d.p[s];
  p.x += F.x * P.dt;
  p.y += F.y * P.dt;
  p.z += F.z * P.dt;
  const double4_32a q0 = d.q_mid[par][s];
  double4_32a qe = q0, q1 = q0;
  float4 ln;
  if (MIXED) {
    // as the single-box mixed form: one rounding per half-drift (fused) on
    // home-cell-local positions, the new local position one conversion, the
    // displacement since the build tested in float against the build
    // position packed in q_mid.w, q_end left for box_end_from_mid
    qe.x = fma(p.x, P.dt2, q0.x);
    qe.y = fma(p.y, P.dt2, q0.y);
    qe.z = fma(p.z, P.dt2, q0.z);
    q1.x = fma(p.x, P.dt2, qe.x);
    q1.y = fma(p.y, P.dt2, qe.y);
    q1.z = fma(p.z, P.dt2, qe.z);
    ln = make_float4((float)q1.x, (float)q1.y, (float)q1.z, 0.0f);
    float bx, by, bz;
    unpack_box_ref(b, q0.w, bx, by, bz);
    const float fx = ln.x - bx, fy = ln.y - by, fz = ln.z - bz;
    if (fx * fx + fy * fy + fz * fz > P.half_margin2_ref || !(fx == fx && fy == fy && fz == fz)) rebuild = true;
  } else {
    qe.x = __dadd_rn(q0.x, __dmul_rn(p.x, P.dt2));
    qe.y = __dadd_rn(q0.y, __dmul_rn(p.y, P.dt2));
    qe.z = __dadd_rn(q0.z, __dmul_rn(p.z, P.dt2));
    q1.x = __dadd_rn(qe.x, __dmul_rn(p.x, P.dt2));
    q1.y = __dadd_rn(qe.y, __dmul_rn(p.y, P.dt2));
    q1.z = __dadd_rn(qe.z, __dmul_rn(p.z, P.dt2));
    const double4_32a qb = d.q_build[s];
    const double ux = q1.x - qb.x, uy = q1.y - qb.y, uz = q1.z - qb.z;
    if (ux * ux + uy * uy + uz * uz > P.half_margin2 || !(q1.x == q1.x && q1.y == q1.y && q1.z == q1.z))
      rebuild = true;
    const float4 lb = d.qf[s];
    ln = make_float4(lb.x + (float)ux, lb.y + (float)uy, lb.z + (float)uz, 0.0f);
  }
  d.loc[par ^ 1][s] = ln;
  if (inner) {
    // inner-list reference: this force evaluation's positions when the
    // rows were re-selected now, else those of the last selection (mixed:
    // packed in p.w)
    float4 lp;
    if (sel) {
      lp = d.loc[par][s];
      if (MIXED) p.w = pack_box_ref(b, lp.x, lp.y, lp.z);
      else d.loc_p[s] = lp;
      d.pcount[s] = kept;
    } else if (MIXED) {
      unpack_box_ref(b, p.w, lp.x, lp.y, lp.z);
    } else {
      lp = d.loc_p[s];
    }
    const float vx = ln.x - lp.x, vy = ln.y - lp.y, vz = ln.z - lp.z;
    if (vx * vx + vy * vy + vz * vz > (MIXED ? P.half_prune2_ref : P.half_prune2)) reselect = true;
  }
  d.p[s] = p;
  if (!MIXED) d.q_end[s] = qe;
  d.q_mid[par ^ 1][s] = q1;
}

// The advance of every box by one step, one persistent kernel: each CTA
// steps its boxes in turn.  The lists of the boxes that rebuilt this step
// were made by the rebuild kernels just before.
// Resident 512-thread blocks per SM the mixed step is compiled for: 2 (64
// registers) measured 9 % faster on 1,024 boxes than 3 (40 registers); the
// FP64 form stays at 2 (it spills at 40 registers).
#ifndef MDG_BATCH_MIN_BLOCKS
#define MDG_BATCH_MIN_BLOCKS 2
#endif
template <int MIXED, int LPI, int INNER>
__global__ void __launch_bounds__(512, MIXED ? MDG_BATCH_MIN_BLOCKS : 2) k_batch_step(Params P, Dev d, int par) {
  __shared__ int s_flag[3];
  const long long goal = *d.goal;
  static_assert(INNER == 0 || LPI == 1, "the inner list is kept for one lane per particle");
  constexpr bool inner = INNER != 0;
  for (int t = d.cta_start[blockIdx.x]; t < d.cta_start[blockIdx.x + 1]; t++) {
    const int bi = d.cta_boxes[t];
    if (threadIdx.x == 0) {
      s_flag[0] = (d.box_err[bi] == 0 && d.box_steps[bi] < goal) ? 1 : 0;
      s_flag[1] = d.box_rebuild[bi];
      s_flag[2] = d.box_prune[bi];
    }
    __syncthreads();
    const int go = s_flag[0], rb = s_flag[1];
    // this step re-selects the box's inner rows (after a rebuild, or when a
    // particle moved half the buffer since the last selection)
    const bool sel = rb != 0 || s_flag[2] != 0;
    __syncthreads();
    if (!go) continue;
    const BoxDesc b = d.boxes[bi];
    if (rb && threadIdx.x == 0) {  // the rebuild of this step completed
      d.box_rebuild[bi] = 0;
      d.box_rebuilds[bi] += 1;
    }
    const int o = b.atom_off, n = b.n;
    const int groups = blockDim.x / LPI, lane = threadIdx.x % LPI;
    bool rebuild = false, reselect = false;
    // all lanes of a group stay together: loop bound rounded to whole groups
    for (int a0 = threadIdx.x / LPI; a0 < ((n + groups - 1) / groups) * groups; a0 += groups) {
      const int a = a0 < n ? a0 : n - 1;
      double3 F;
      int kept = 0;
      if constexpr (INNER != 0) {
        if (sel) F = box_force<MIXED, 1, 1>(P, d, b, a, lane, par, a0 < n, &kept);
        else F = box_force<MIXED, 1, 2>(P, d, b, a, lane, par);
      } else {
        F = box_force<MIXED, LPI, 0>(P, d, b, a, lane, par);
      }
      if (lane != 0 || a0 >= n) continue;
      advance_particle<MIXED, inner>(P, d, b, o + a, F, par, sel, kept, rebuild, reselect);
    }
    const int any = __syncthreads_or(rebuild ? 1 : 0);
    const int anyp = __syncthreads_or(reselect ? 1 : 0);
    if (threadIdx.x == 0) {
      if (any) d.box_rebuild[bi] = 1;
      if (inner) d.box_prune[bi] = anyp;
      if (MIXED) d.box_mid[bi] = par ^ 1;
      d.box_steps[bi] += 1;
    }
    __syncthreads();
  }
}

// The same step in the flat layout: the grid (only as many CTAs as are
// resident at once) strides over the particles of all boxes, one thread per
// particle, so no CTA waits for the slowest warp of a box before the next,
// the work of a box spreads over the whole GPU and the kernel holds no box
// description in registers (its fields are read where they are used, from
// L1).  A particle whose displacement test fires raises its box's request
// with a plain store of 1; k_batch_finish applies the requests and counts the
// box's step after the kernel.  The box state the step reads (error, step
// count, rebuild and re-selection flags) is not written during it.
// Resident 256-thread CTAs per SM the flat kernel is compiled for: 4 gives
// 64 registers, where the inner-list variant runs without spills and beats
// the outer-list walk (1,024 boxes, mixed: 5.18e9 atom-steps/s at 128 x 8
// with the inner list, against 4.56e9 for the outer list at 48 registers
// (5 CTAs), where the inner variant lost; 3 CTAs, up to 80 registers: 4.96e9).
#ifndef MDG_BATCH_FLAT_MIN_BLOCKS
#define MDG_BATCH_FLAT_MIN_BLOCKS 4
#endif
constexpr int kFlatMaxThreads = 256;
template <int MIXED, int INNER>
__global__ void __launch_bounds__(kFlatMaxThreads, MDG_BATCH_FLAT_MIN_BLOCKS) k_batch_step_flat(Params P, Dev d,
                                                                                            int par) {
  const long long goal = *d.goal;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < P.total; s += gridDim.x * blockDim.x) {
    const int bi = d.box_of_slot[s];
    if (d.box_err[bi] != 0 || d.box_steps[bi] >= goal) continue;
    const BoxDesc &b = d.boxes[bi];
    const int a = s - b.atom_off;
    const bool sel = d.box_rebuild[bi] != 0 || d.box_prune[bi] != 0;
    double3 F;
    int kept = 0;
    if constexpr (INNER != 0) {
      if (sel) F = box_force<MIXED, 1, 1>(P, d, b, a, 0, par, true, &kept);
      else F = box_force<MIXED, 1, 2>(P, d, b, a, 0, par);
    } else {
      F = box_force<MIXED, 1, 0>(P, d, b, a, 0, par);
    }
    bool rebuild = false, reselect = false;
    advance_particle<MIXED, INNER != 0>(P, d, b, s, F, par, sel, kept, rebuild, reselect);
    if (rebuild) d.box_req[bi] = 1;
    if (INNER != 0 && reselect) d.box_preq[bi] = 1;
  }
}

// After the flat step, one thread per box (the same participation test as
// the step): the rebuild this step consumed is counted, the requests become
// the next step's flags, the box's step count advances.
template <int INNER>
__global__ void k_batch_finish(Params P, Dev d, int par) {
  const int bi = blockIdx.x * blockDim.x + threadIdx.x;
  if (bi >= P.nbox) return;
  if (d.box_err[bi] != 0 || d.box_steps[bi] >= *d.goal) return;
  if (d.box_rebuild[bi]) {
    d.box_rebuild[bi] = 0;
    d.box_rebuilds[bi] += 1;
  }
  if (d.box_req[bi]) {
    d.box_rebuild[bi] = 1;
    d.box_req[bi] = 0;
  }
  if (INNER != 0) {
    d.box_prune[bi] = d.box_preq[bi];
    d.box_preq[bi] = 0;
  }
  if (P.local_pos) d.box_mid[bi] = par ^ 1;
  d.box_steps[bi] += 1;
}

// Per-box observer sums at q_end (observer.cc:5-79 expressions, pairs 1/2 each).
__global__ void k_batch_observe(Params P, Dev d) {
  __shared__ double sh[3][32];
  const int bi = blockIdx.x;
  const BoxDesc b = d.boxes[bi];
  const int o = b.atom_off, n = b.n;
  double ke = 0.0, pe = 0.0, vir = 0.0;
  for (int a = threadIdx.x; a < n; a += blockDim.x) {
    const double4_32a p = d.p[o + a];
    ke += 0.5 * p.x * p.x + 0.5 * p.y * p.y + 0.5 * p.z * p.z;  // w is padding
    const double4_32a qi = d.q_end[o + a];
    int cx, cy, cz;
    cell_xyz(b, d.cell[o + a], cx, cy, cz);
    const int cnt = d.ncount[o + a];
    for (int k = 0; k < cnt; k++) {
      const uint32_t e = d.nl[b.list_off + (long long)k * n + a];
      double4_32a qj = d.q_end[o + entry_slot(e)];
      const int ox = entry_sx(e), oy = entry_sy(e), oz = entry_sz(e);
      if (ox == 0 && cx == 0) qj.x -= b.L[0]; else if (ox == 2 && cx == b.nc[0] - 1) qj.x += b.L[0];
      if (oy == 0 && cy == 0) qj.y -= b.L[1]; else if (oy == 2 && cy == b.nc[1] - 1) qj.y += b.L[1];
      if (oz == 0 && cz == 0) qj.z -= b.L[2]; else if (oz == 2 && cz == b.nc[2] - 1) qj.z += b.L[2];
      const double dx = __dsub_rn(qi.x, qj.x), dy = __dsub_rn(qi.y, qj.y), dz = __dsub_rn(qi.z, qj.z);
      const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
      if (r2 > P.rc2) continue;
      const double r4 = __dmul_rn(r2, r2), r6 = __dmul_rn(r4, r2), r8 = __dmul_rn(r6, r2), r10 = __dmul_rn(r8, r2),
                   r12 = __dmul_rn(r10, r2);
      const double c2 = P.c2x8 / 8.0;
      const double c0 = -1.0 / (P.rc2 * P.rc2 * P.rc2 * P.rc2 * P.rc2 * P.rc2) + 1.0 / (P.rc2 * P.rc2 * P.rc2) -
                        c2 * P.rc2;
      pe += 0.5 * (4.0 * (1.0 / r12 - 1.0 / r6 + __dmul_rn(c2, r2) + c0));
      vir += 0.5 * ((__dsub_rn(__dmul_rn(24.0, r6), 48.0) / (__dmul_rn(__dmul_rn(r6, r6), r2)) + P.c2x8) * r2);
    }
  }
  double v[3] = {ke, pe, vir};
  for (int k = 0; k < 3; k++)
    for (int off = 16; off > 0; off >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], off);
  if ((threadIdx.x & 31) == 0)
    for (int k = 0; k < 3; k++) sh[k][threadIdx.x >> 5] = v[k];
  __syncthreads();
  if (threadIdx.x == 0) {
    double t[3] = {0, 0, 0};
    for (int w = 0; w < (int)(blockDim.x >> 5); w++)
      for (int k = 0; k < 3; k++) t[k] += sh[k][w];
    d.partials[3 * bi + 0] = t[0];
    d.partials[3 * bi + 1] = t[1];
    d.partials[3 * bi + 2] = t[2] / 3.0;
  }
}

// The caller's arrays in the caller's order; the fourth lane is padding and
// comes back zero (the mixed forms keep packed reference positions in it).
__global__ void k_batch_unsort(Dev d, int total, double4_32a *qo, double4_32a *po, const int *box_of_slot) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= total) return;
  const int bi = box_of_slot[s];
  const int dst = d.boxes[bi].atom_off + d.id[s];
  if (qo) {
    double4_32a q = d.q_end[s];
    q.w = 0.0;
    qo[dst] = q;
  }
  if (po) {
    double4_32a p = d.p[s];
    p.w = 0.0;
    po[dst] = p;
  }
}

// Mixed forms: q_end of every slot whose box has stepped since it was last
// current, from that box's q_mid slot; k_batch_end_current then records that
// every box's q_end is current (a separate kernel, so no thread clears a
// box's slot while others still read it).
__global__ void k_batch_end_from_mid(Params P, Dev d, const int *box_of_slot) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= P.total) return;
  const int bi = box_of_slot[s];
  const int mid = d.box_mid[bi];
  if (mid >= 0) d.q_end[s] = box_end_from_mid(P, d, d.boxes[bi], s, mid);
}

__global__ void k_batch_end_current(Params P, Dev d) {
  const int bi = blockIdx.x * blockDim.x + threadIdx.x;
  if (bi < P.nbox) d.box_mid[bi] = -1;
}

}  // namespace batch
}  // namespace mdg

// ---------------------------------------------------------------- C ABI
using namespace mdg::batch;

struct mdg_batch {
  mdg_batch_params prm;
  std::string err;
  int nbox = 0, total = 0, num_sms = 0;
  int threads = 256, lpi = 1, ctas_per_sm = 2;
  int use_inner = 1;  // one lane per particle walks the inner list (when the buffer is > 0)
  int flat = 0;       // 1: the flat layout of the step (k_batch_step_flat + k_batch_finish)
  double buffer = 0.0;  // inner-list buffer in use
  double ref_unit = 0.0;  // mixed forms: the largest packed-position unit, w / (2^20 - 1), over the boxes
  cudaStream_t stream = nullptr;
  Params P;
  Dev d;
  std::vector<BoxDesc> boxes;
  std::vector<int> box_of_slot;
  int *d_box_of_slot = nullptr;
  int par = 0;
  long long steps = 0;  // goal reached by every box
  cudaGraphExec_t gx[2] = {nullptr, nullptr};
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double last_ms = 0.0;
  long long launches = 0;
  int grid = 0;
};

namespace {

int bfail(mdg_batch *b, int code, const std::string &m) {
  if (b) b->err = m;
  return code;
}

#define MDG_BCK(call)                                                                               \
  do {                                                                                              \
    cudaError_t e_ = (call);                                                                        \
    if (e_ != cudaSuccess) return bfail(b, MDG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

void drop_batch_graphs(mdg_batch *b) {
  for (int k = 0; k < 2; k++)
    if (b->gx[k]) {
      cudaGraphExecDestroy(b->gx[k]);
      b->gx[k] = nullptr;
    }
}

template <class T>
cudaError_t balloc(T **p, size_t count) {
  *p = nullptr;
  return cudaMalloc((void **)p, (count ? count : 1) * sizeof(T));
}

// The persistent step kernel the shape selects (as launch_batch_step does).
const void *step_kernel_fn(int prec, int lpi, bool inner, bool flat) {
  if (flat) {
    if (prec == MDG_MIXED) return inner ? reinterpret_cast<const void *>(&k_batch_step_flat<MDG_MIXED, 1>)
                                        : reinterpret_cast<const void *>(&k_batch_step_flat<MDG_MIXED, 0>);
    if (prec == MDG_MIXED_PLAIN)
      return inner ? reinterpret_cast<const void *>(&k_batch_step_flat<MDG_MIXED_PLAIN, 1>)
                   : reinterpret_cast<const void *>(&k_batch_step_flat<MDG_MIXED_PLAIN, 0>);
    return inner ? reinterpret_cast<const void *>(&k_batch_step_flat<MDG_FP64, 1>)
                 : reinterpret_cast<const void *>(&k_batch_step_flat<MDG_FP64, 0>);
  }
#define MDG_BFN(M, L, I) reinterpret_cast<const void *>(&k_batch_step<M, L, I>)
  if (prec == MDG_MIXED)
    return lpi == 4 ? MDG_BFN(MDG_MIXED, 4, 0) : lpi == 2 ? MDG_BFN(MDG_MIXED, 2, 0)
           : inner  ? MDG_BFN(MDG_MIXED, 1, 1) : MDG_BFN(MDG_MIXED, 1, 0);
  if (prec == MDG_MIXED_PLAIN)
    return lpi == 4 ? MDG_BFN(MDG_MIXED_PLAIN, 4, 0) : lpi == 2 ? MDG_BFN(MDG_MIXED_PLAIN, 2, 0)
           : inner  ? MDG_BFN(MDG_MIXED_PLAIN, 1, 1) : MDG_BFN(MDG_MIXED_PLAIN, 1, 0);
  return lpi == 4 ? MDG_BFN(MDG_FP64, 4, 0) : lpi == 2 ? MDG_BFN(MDG_FP64, 2, 0)
         : inner  ? MDG_BFN(MDG_FP64, 1, 1) : MDG_BFN(MDG_FP64, 1, 0);
#undef MDG_BFN
}

// CTAs of `threads` threads of the selected step kernel that fit on one SM
// at once (registers, shared memory, thread slots): the persistent kernel's
// grid must not exceed this, or its CTAs run in waves.
int resident_ctas(const mdg_batch *b, int threads) {
  const bool inner = b->P.inner && b->lpi == 1 && b->use_inner;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, step_kernel_fn(b->prm.precision, b->lpi, inner, b->flat != 0),
                                                    threads,
                                                    0) != cudaSuccess)
    return 1;
  return nb > 0 ? nb : 1;
}

// The inner-list buffer b: rows keep the listed pairs within rc + b and are
// re-selected when a particle of the box moved b / 2 since the last selection.
void set_prune_buffer(mdg_batch *b, double buffer) {
  Params &P = b->P;
  const double rb = b->prm.cutoff + buffer;
  P.prune_thr2d = rb * rb;
  P.prune_thr2f = (float)(rb * rb + 1e-4);  // float r2 of local positions is within ~1e-5
  P.half_prune2 = (float)(0.25 * buffer * buffer * (1.0 - 1e-4));
  const double hp = 0.5 * buffer - 2.0 * b->ref_unit;
  P.half_prune2_ref = buffer > 0.0 ? (float)(hp > 0.0 ? hp * hp * (1.0 - 1e-4) : 0.0) : 3.0e38f;
  b->buffer = buffer;
  drop_batch_graphs(b);  // the graphs hold the parameters by value
}

// Mixed forms: every box's q_end from its last q_mid (the steps leave it
// behind), before anything reads q_end from outside a rebuild.
void make_end_current(mdg_batch *b) {
  if (!b->P.local_pos) return;
  k_batch_end_from_mid<<<(b->total + 255) / 256, 256, 0, b->stream>>>(b->P, b->d, b->d_box_of_slot);
  k_batch_end_current<<<(b->nbox + 255) / 256, 256, 0, b->stream>>>(b->P, b->d);
  b->launches += 2;
}

// Longest-first assignment of boxes to grid CTAs (work ~ n * list capacity).
// The CTAs per SM are capped by what is resident at once, so every CTA of the
// persistent kernel runs from the start.
int assign(mdg_batch *b) {
  b->ctas_per_sm = std::min(b->ctas_per_sm, resident_ctas(b, b->threads));
  const int G = b->num_sms * b->ctas_per_sm;
  std::vector<int> idx(b->nbox);
  std::iota(idx.begin(), idx.end(), 0);
  std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) { return b->boxes[x].n > b->boxes[y].n; });
  std::vector<long long> load(G, 0);
  std::vector<std::vector<int>> own(G);
  for (int k : idx) {
    int best = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    own[best].push_back(k);
    load[best] += b->boxes[k].n;
  }
  std::vector<int> start(G + 1, 0), flat;
  for (int g = 0; g < G; g++) {
    start[g + 1] = start[g] + (int)own[g].size();
    flat.insert(flat.end(), own[g].begin(), own[g].end());
  }
  if (b->d.cta_start) cudaFree(b->d.cta_start);
  if (b->d.cta_boxes) cudaFree(b->d.cta_boxes);
  MDG_BCK(balloc(&b->d.cta_start, G + 1));
  MDG_BCK(balloc(&b->d.cta_boxes, b->nbox));
  MDG_BCK(cudaMemcpy(b->d.cta_start, start.data(), (G + 1) * sizeof(int), cudaMemcpyHostToDevice));
  MDG_BCK(cudaMemcpy(b->d.cta_boxes, flat.data(), b->nbox * sizeof(int), cudaMemcpyHostToDevice));
  b->grid = G;
  // the inner rows are kept only under one lane per particle: a new shape
  // starts from a fresh selection
  MDG_BCK(cudaMemset(b->d.box_prune, 1, b->nbox * sizeof(int)));
  drop_batch_graphs(b);
  return MDG_OK;
}

// (Re)allocates the list pool for capacity `cap` and uploads box descriptors.
int alloc_batch_list(mdg_batch *b, int cap) {
  long long off = 0;
  for (auto &bx : b->boxes) {
    bx.list_off = off;
    off += (long long)bx.n * cap;
  }
  if (b->d.nl) cudaFree(b->d.nl);
  if (b->d.pl) cudaFree(b->d.pl);
  b->d.nl = b->d.pl = nullptr;
  MDG_BCK(balloc(&b->d.nl, (size_t)off));
  if (b->P.inner) MDG_BCK(balloc(&b->d.pl, (size_t)off));
  b->P.list_cap = cap;
  MDG_BCK(cudaMemcpy(b->d.boxes, b->boxes.data(), b->nbox * sizeof(BoxDesc), cudaMemcpyHostToDevice));
  std::vector<int> ones(b->nbox, 1);
  MDG_BCK(cudaMemcpy(b->d.box_rebuild, ones.data(), b->nbox * sizeof(int), cudaMemcpyHostToDevice));
  drop_batch_graphs(b);
  return MDG_OK;
}

void launch_batch_step(mdg_batch *b, int par) {
  const int T = b->threads;
  const int prec = b->prm.precision;
  k_batch_rebuild_set<<<1, 1024, 0, b->stream>>>(b->P, b->d);
  k_batch_bin<<<b->num_sms * 16, 128, 0, b->stream>>>(b->P, b->d);
  k_batch_sort<<<b->nbox, kPrepThreads, 0, b->stream>>>(b->d);
  k_batch_place<<<b->num_sms * 16, 128, 0, b->stream>>>(b->P, b->d, par);
  k_batch_list<<<b->num_sms * 16, 128, 0, b->stream>>>(b->P, b->d);
#define MDG_BSTEP(M, L, I) k_batch_step<M, L, I><<<b->grid, T, 0, b->stream>>>(b->P, b->d, par)
  const bool inner = b->P.inner && b->lpi == 1 && b->use_inner;
  if (b->flat) {
#define MDG_FSTEP(M, I) k_batch_step_flat<M, I><<<b->grid, T, 0, b->stream>>>(b->P, b->d, par)
    if (prec == MDG_MIXED) { if (inner) MDG_FSTEP(MDG_MIXED, 1); else MDG_FSTEP(MDG_MIXED, 0); }
    else if (prec == MDG_MIXED_PLAIN) { if (inner) MDG_FSTEP(MDG_MIXED_PLAIN, 1); else MDG_FSTEP(MDG_MIXED_PLAIN, 0); }
    else { if (inner) MDG_FSTEP(MDG_FP64, 1); else MDG_FSTEP(MDG_FP64, 0); }
#undef MDG_FSTEP
    const int fg = (b->nbox + 255) / 256;
    if (inner) k_batch_finish<1><<<fg, 256, 0, b->stream>>>(b->P, b->d, par);
    else k_batch_finish<0><<<fg, 256, 0, b->stream>>>(b->P, b->d, par);
    b->launches += kBatchKernelsPerStep + 1;
    return;
  }
  if (prec == MDG_MIXED) {
    if (b->lpi == 4) MDG_BSTEP(MDG_MIXED, 4, 0); else if (b->lpi == 2) MDG_BSTEP(MDG_MIXED, 2, 0);
    else if (inner) MDG_BSTEP(MDG_MIXED, 1, 1); else MDG_BSTEP(MDG_MIXED, 1, 0);
  } else if (prec == MDG_MIXED_PLAIN) {
    if (b->lpi == 4) MDG_BSTEP(MDG_MIXED_PLAIN, 4, 0); else if (b->lpi == 2) MDG_BSTEP(MDG_MIXED_PLAIN, 2, 0);
    else if (inner) MDG_BSTEP(MDG_MIXED_PLAIN, 1, 1); else MDG_BSTEP(MDG_MIXED_PLAIN, 1, 0);
  } else {
    if (b->lpi == 4) MDG_BSTEP(0, 4, 0); else if (b->lpi == 2) MDG_BSTEP(0, 2, 0);
    else if (inner) MDG_BSTEP(0, 1, 1); else MDG_BSTEP(0, 1, 0);
  }
#undef MDG_BSTEP
  b->launches += kBatchKernelsPerStep;
}

int run_steps(mdg_batch *b, int nsteps) {
  if (!b->prm.use_graphs) {
    for (int k = 0; k < nsteps; k++) {
      launch_batch_step(b, b->par);
      b->par ^= 1;
    }
    return cudaGetLastError() == cudaSuccess ? MDG_OK : bfail(b, MDG_ERR_CUDA, "launch failed");
  }
  int left = nsteps;
  while (left > 0) {
    const int par = b->par;
    if (left >= 2) {
      if (!b->gx[par]) {
        cudaGraph_t g = nullptr;
        MDG_BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        const long long l0 = b->launches;
        launch_batch_step(b, par);
        launch_batch_step(b, par ^ 1);
        b->launches = l0;
        MDG_BCK(cudaStreamEndCapture(b->stream, &g));
        cudaError_t e = cudaGraphInstantiate(&b->gx[par], g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return bfail(b, MDG_ERR_CUDA, cudaGetErrorString(e));
      }
      MDG_BCK(cudaGraphLaunch(b->gx[par], b->stream));
      b->launches += 2 * (kBatchKernelsPerStep + (b->flat ? 1 : 0));
      left -= 2;
    } else {
      launch_batch_step(b, par);
      b->par ^= 1;
      left -= 1;
    }
  }
  return MDG_OK;
}

}  // namespace

extern "C" {

void mdg_batch_params_default(mdg_batch_params *p) {
  if (!p) return;
  memset(p, 0, sizeof(*p));
  p->precision = MDG_FP64;
  p->cutoff = 2.5;
  p->margin = 0.4;
  p->dt = 0.002;
  p->list_capacity = 0;
  p->use_graphs = 1;
  p->prune_buffer = -1.0;
}

int mdg_batch_create(const mdg_batch_params *p, int32_t nbox, const int32_t *n_per_box, const double *box_lengths,
                     mdg_batch **out) {
  if (!p || !out || nbox <= 0 || !n_per_box || !box_lengths) return MDG_ERR_INVALID;
  *out = nullptr;
  if (p->precision < MDG_FP64 || p->precision > MDG_MIXED_PLAIN) return MDG_ERR_INVALID;
  mdg_batch *b = new mdg_batch();
  b->prm = *p;
  b->nbox = nbox;
  memset(&b->d, 0, sizeof(b->d));
  const double sl = p->cutoff + p->margin;
  long long total = 0, cells = 0;
  double max_rho = 0.0;
  for (int k = 0; k < nbox; k++) {
    BoxDesc bx;
    memset(&bx, 0, sizeof bx);
    bx.n = n_per_box[k];
    if (bx.n <= 0) {
      delete b;
      return MDG_ERR_INVALID;
    }
    long long nc_tot = 1;
    for (int a = 0; a < 3; a++) {
      const double L = box_lengths[3 * k + a];
      int nc = (int)(L / sl);
      while (nc > 0 && L / (double)nc < sl * (1.0 + 1e-12)) nc--;
      if (nc < 2 || !(L > 2.0 * sl)) {
        delete b;
        return MDG_ERR_INVALID;
      }
      const double w = L / (double)nc;
      bx.L[a] = L;
      bx.nc[a] = nc;
      bx.inv_w[a] = 1.0 / w;
      bx.w32[a] = (float)w;
      bx.dl32[a] = (float)(L - (double)nc * (double)bx.w32[a]);
      nc_tot *= nc;
    }
    if (nc_tot > kMaxCellsPerBox) {
      delete b;
      return MDG_ERR_CAPACITY;
    }
    bx.ncell = (int)nc_tot;
    bx.atom_off = (int)total;
    bx.cell_off = (int)cells;
    total += bx.n;
    cells += nc_tot + 1;
    max_rho = std::max(max_rho, bx.n / (bx.L[0] * bx.L[1] * bx.L[2]));
    b->boxes.push_back(bx);
  }
  if (total > (1LL << 30)) {
    delete b;
    return MDG_ERR_CAPACITY;
  }
  b->total = (int)total;
  for (int k = 0; k < nbox; k++)
    for (int a = 0; a < b->boxes[k].n; a++) b->box_of_slot.push_back(k);
  Params &P = b->P;
  P.sl2 = sl * sl;
  P.rc2 = p->cutoff * p->cutoff;
  const double s2 = 1.0 / P.rc2, s6 = s2 * s2 * s2, s8 = s6 * s2, s12 = s6 * s6, s14 = s12 * s2;
  P.c2x8 = (6.0 * s14 - 3.0 * s8) * 8.0;
  (void)s12;
  P.c2x8f = (float)P.c2x8;
  P.rc2f = (float)P.rc2;
  P.acc_lo = (float)(sl * sl - 1e-4);
  P.acc_hi = (float)(sl * sl + 1e-4);
  P.dt = p->dt;
  P.dt2 = p->dt * 0.5;
  P.half_margin2 = 0.25 * p->margin * p->margin;
  P.nbox = nbox;
  P.total = (int)total;
  P.local_pos = p->precision != MDG_FP64 ? 1 : 0;
  for (const auto &bx : b->boxes)
    for (int a = 0; a < 3; a++) b->ref_unit = std::fmax(b->ref_unit, (double)bx.w32[a] / 1048575.0);
  const double hm = 0.5 * p->margin - 2.0 * b->ref_unit;
  P.half_margin2_ref = (float)(hm > 0.0 ? hm * hm : 0.0);
  // inner-list buffer: negative = min(0.1, margin / 2), as the single-box
  // form (the autotuner may then pick margin / 2 instead)
  const double buffer = p->prune_buffer < 0.0 ? std::fmin(0.1, 0.5 * p->margin) : p->prune_buffer;
  P.inner = buffer > 0.0 ? 1 : 0;
  set_prune_buffer(b, buffer);
  int cap = p->list_capacity > 0 ? p->list_capacity : (int)(max_rho * 4.18879020478639 * sl * sl * sl * 1.5 + 24);
  cap = (cap + 7) & ~7;
  cudaError_t e = cudaSetDevice(p->device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&b->num_sms, cudaDevAttrMultiProcessorCount, p->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&b->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&b->ev1);
  Dev &d = b->d;
  const size_t n = (size_t)total;
  if (e == cudaSuccess) e = balloc(&d.boxes, nbox);
  if (e == cudaSuccess) e = balloc(&d.q_end, n);
  if (e == cudaSuccess) e = balloc(&d.q_mid[0], n);
  if (e == cudaSuccess) e = balloc(&d.q_mid[1], n);
  if (e == cudaSuccess) e = balloc(&d.p, n);
  if (e == cudaSuccess) e = balloc(&d.q_build, n);
  if (e == cudaSuccess) e = balloc(&d.t_q, n);
  if (e == cudaSuccess) e = balloc(&d.t_p, n);
  if (e == cudaSuccess) e = balloc(&d.qf, n);
  if (e == cudaSuccess) e = balloc(&d.loc[0], n);
  if (e == cudaSuccess) e = balloc(&d.loc[1], n);
  if (e == cudaSuccess) e = balloc(&d.id, n);
  if (e == cudaSuccess) e = balloc(&d.cell, n);
  if (e == cudaSuccess) e = balloc(&d.t_id, n);
  if (e == cudaSuccess) e = balloc(&d.t_cell, n);
  if (e == cudaSuccess) e = balloc(&d.order, n);
  if (e == cudaSuccess) e = balloc(&d.ncount, n);
  if (e == cudaSuccess) e = balloc(&d.pcount, n);
  if (e == cudaSuccess) e = balloc(&d.loc_p, n);
  if (e == cudaSuccess) e = balloc(&d.box_prune, nbox);
  if (e == cudaSuccess) e = balloc(&d.box_req, nbox);
  if (e == cudaSuccess) e = balloc(&d.box_preq, nbox);
  if (e == cudaSuccess) e = cudaMemset(d.box_req, 0, nbox * sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(d.box_preq, 0, nbox * sizeof(int));
  if (e == cudaSuccess) e = balloc(&d.box_mid, nbox);
  if (e == cudaSuccess) e = cudaMemset(d.box_mid, 0xFF, nbox * sizeof(int));  // -1: q_end current
  if (e == cudaSuccess) e = balloc(&d.rb_boxes, nbox);
  if (e == cudaSuccess) e = balloc(&d.rb_start, (size_t)nbox + 1);
  if (e == cudaSuccess) e = balloc(&d.rb_count, 1);
  if (e == cudaSuccess) e = balloc(&d.cell_start, (size_t)cells);
  if (e == cudaSuccess) e = balloc(&d.box_rebuild, nbox);
  if (e == cudaSuccess) e = balloc(&d.box_err, nbox);
  if (e == cudaSuccess) e = balloc(&d.box_need, nbox);
  if (e == cudaSuccess) e = balloc(&d.box_steps, nbox);
  if (e == cudaSuccess) e = balloc(&d.box_rebuilds, nbox);
  if (e == cudaSuccess) e = balloc(&d.goal, 1);
  if (e == cudaSuccess) e = balloc(&d.partials, 3 * (size_t)nbox);
  if (e == cudaSuccess) e = balloc(&b->d_box_of_slot, n);
  if (e == cudaSuccess) e = cudaMemcpy(b->d_box_of_slot, b->box_of_slot.data(), n * sizeof(int), cudaMemcpyHostToDevice);
  d.box_of_slot = b->d_box_of_slot;
  if (e != cudaSuccess) {
    fprintf(stderr, "mdg_batch_create: %s\n", cudaGetErrorString(e));
    mdg_batch_destroy(b);
    return MDG_ERR_CUDA;
  }
  if (alloc_batch_list(b, cap) != MDG_OK || assign(b) != MDG_OK) {
    fprintf(stderr, "mdg_batch_create: %s\n", b->err.c_str());
    mdg_batch_destroy(b);
    return MDG_ERR_CUDA;
  }
  *out = b;
  return MDG_OK;
}

int mdg_batch_destroy(mdg_batch *b) {
  if (!b) return MDG_OK;
  cudaSetDevice(b->prm.device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  drop_batch_graphs(b);
  Dev &d = b->d;
  void *ptrs[] = {d.boxes, d.cta_start, d.cta_boxes, d.q_end, d.q_mid[0], d.q_mid[1], d.p, d.q_build, d.t_q, d.t_p,
                  d.qf, d.loc[0], d.loc[1], d.id, d.cell, d.t_id, d.t_cell, d.order, d.cell_start, d.nl, d.ncount,
                  d.pl, d.pcount, d.loc_p, d.box_prune, d.box_req, d.box_preq, d.rb_boxes, d.rb_start, d.rb_count,
                  d.box_rebuild, d.box_err, d.box_need, d.box_steps, d.box_rebuilds, d.goal, d.partials,
                  d.box_mid, b->d_box_of_slot};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return MDG_OK;
}

const char *mdg_batch_last_error(const mdg_batch *b) { return b ? b->err.c_str() : "null batch"; }

int mdg_batch_set_state(mdg_batch *b, const double *q4, const double *p4) {
  if (!b || !q4 || !p4) return MDG_ERR_INVALID;
  cudaSetDevice(b->prm.device);
  const size_t bytes = (size_t)b->total * 32;
  MDG_BCK(cudaMemcpyAsync(b->d.q_end, q4, bytes, cudaMemcpyHostToDevice, b->stream));
  MDG_BCK(cudaMemcpyAsync(b->d.p, p4, bytes, cudaMemcpyHostToDevice, b->stream));
  std::vector<int> ids(b->total);
  for (int k = 0; k < b->nbox; k++)
    for (int a = 0; a < b->boxes[k].n; a++) ids[b->boxes[k].atom_off + a] = a;
  MDG_BCK(cudaMemcpyAsync(b->d.id, ids.data(), ids.size() * sizeof(int), cudaMemcpyHostToDevice, b->stream));
  std::vector<int> ones(b->nbox, 1), zeros(b->nbox, 0);
  std::vector<long long> lz(b->nbox, 0);
  MDG_BCK(cudaMemcpyAsync(b->d.box_rebuild, ones.data(), b->nbox * sizeof(int), cudaMemcpyHostToDevice, b->stream));
  MDG_BCK(cudaMemcpyAsync(b->d.box_err, zeros.data(), b->nbox * sizeof(int), cudaMemcpyHostToDevice, b->stream));
  MDG_BCK(cudaMemcpyAsync(b->d.box_need, zeros.data(), b->nbox * sizeof(int), cudaMemcpyHostToDevice, b->stream));
  MDG_BCK(cudaMemcpyAsync(b->d.box_steps, lz.data(), b->nbox * sizeof(long long), cudaMemcpyHostToDevice, b->stream));
  MDG_BCK(cudaMemcpyAsync(b->d.box_rebuilds, lz.data(), b->nbox * sizeof(long long), cudaMemcpyHostToDevice, b->stream));
  MDG_BCK(cudaMemcpyAsync(b->d.box_req, zeros.data(), b->nbox * sizeof(int), cudaMemcpyHostToDevice, b->stream));
  MDG_BCK(cudaMemcpyAsync(b->d.box_preq, zeros.data(), b->nbox * sizeof(int), cudaMemcpyHostToDevice, b->stream));
  MDG_BCK(cudaMemsetAsync(b->d.box_mid, 0xFF, b->nbox * sizeof(int), b->stream));  // q_end current
  MDG_BCK(cudaStreamSynchronize(b->stream));
  b->steps = 0;
  b->par = 0;
  drop_batch_graphs(b);
  return MDG_OK;
}

int mdg_batch_get_state(mdg_batch *b, double *q4, double *p4) {
  if (!b) return MDG_ERR_INVALID;
  cudaSetDevice(b->prm.device);
  double4_32a *tq = b->d.t_q, *tp = b->d.t_p;  // staging (free outside rebuilds)
  make_end_current(b);
  k_batch_unsort<<<(b->total + 255) / 256, 256, 0, b->stream>>>(b->d, b->total, q4 ? tq : nullptr,
                                                                 p4 ? tp : nullptr, b->d_box_of_slot);
  const size_t bytes = (size_t)b->total * 32;
  if (q4) MDG_BCK(cudaMemcpyAsync(q4, tq, bytes, cudaMemcpyDeviceToHost, b->stream));
  if (p4) MDG_BCK(cudaMemcpyAsync(p4, tp, bytes, cudaMemcpyDeviceToHost, b->stream));
  MDG_BCK(cudaStreamSynchronize(b->stream));
  return MDG_OK;
}

int mdg_batch_calculate(mdg_batch *b, int32_t nsteps) {
  if (!b || nsteps < 0) return MDG_ERR_INVALID;
  cudaSetDevice(b->prm.device);
  if (nsteps == 0) return MDG_OK;
  const long long goal = b->steps + nsteps;
  MDG_BCK(cudaMemcpyAsync(b->d.goal, &goal, sizeof goal, cudaMemcpyHostToDevice, b->stream));
  MDG_BCK(cudaEventRecord(b->ev0, b->stream));
  int rc = run_steps(b, nsteps);
  if (rc) return rc;
  for (int round = 0; round < 32; round++) {
    std::vector<int> err(b->nbox), need(b->nbox);
    std::vector<long long> st(b->nbox);
    MDG_BCK(cudaMemcpyAsync(err.data(), b->d.box_err, b->nbox * sizeof(int), cudaMemcpyDeviceToHost, b->stream));
    MDG_BCK(cudaMemcpyAsync(need.data(), b->d.box_need, b->nbox * sizeof(int), cudaMemcpyDeviceToHost, b->stream));
    MDG_BCK(cudaMemcpyAsync(st.data(), b->d.box_steps, b->nbox * sizeof(long long), cudaMemcpyDeviceToHost, b->stream));
    MDG_BCK(cudaStreamSynchronize(b->stream));
    long long behind = 0;
    int maxneed = 0;
    for (int k = 0; k < b->nbox; k++) {
      if (err[k] == kErrBadState) return bfail(b, MDG_ERR_STATE, "box " + std::to_string(k) + ": bad coordinate");
      behind = std::max(behind, goal - st[k]);
      if (err[k] == kErrOverflow) maxneed = std::max(maxneed, need[k]);
    }
    if (behind == 0) break;
    if (maxneed > 0) {
      int cap = ((int)(maxneed * 1.25) + 15) & ~7;
      rc = alloc_batch_list(b, cap);  // every box rebuilds its list at the new capacity
      if (rc) return rc;
      std::vector<int> zeros(b->nbox, 0);
      MDG_BCK(cudaMemcpyAsync(b->d.box_err, zeros.data(), b->nbox * sizeof(int), cudaMemcpyHostToDevice, b->stream));
      MDG_BCK(cudaMemcpyAsync(b->d.box_need, zeros.data(), b->nbox * sizeof(int), cudaMemcpyHostToDevice, b->stream));
    }
    // catch-up: only boxes behind the goal advance
    for (long long k = 0; k < behind; k++) {
      launch_batch_step(b, b->par);
      b->par ^= 1;
    }
    drop_batch_graphs(b);
    b->par = 0;  // parity is re-established by the rebuild of every box
    std::vector<int> ones(b->nbox, 1);
    MDG_BCK(cudaMemcpyAsync(b->d.box_rebuild, ones.data(), b->nbox * sizeof(int), cudaMemcpyHostToDevice, b->stream));
  }
  MDG_BCK(cudaEventRecord(b->ev1, b->stream));
  MDG_BCK(cudaEventSynchronize(b->ev1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, b->ev0, b->ev1);
  b->last_ms = ms;
  b->steps = goal;
  return MDG_OK;
}

int mdg_batch_observe(mdg_batch *b, double *out) {
  if (!b || !out) return MDG_ERR_INVALID;
  cudaSetDevice(b->prm.device);
  make_end_current(b);
  k_batch_observe<<<b->nbox, 256, 0, b->stream>>>(b->P, b->d);
  MDG_BCK(cudaMemcpyAsync(out, b->d.partials, 3 * (size_t)b->nbox * sizeof(double), cudaMemcpyDeviceToHost,
                          b->stream));
  MDG_BCK(cudaStreamSynchronize(b->stream));
  return MDG_OK;
}

int mdg_batch_tune(mdg_batch *b, int32_t trial_steps, int32_t *threads, int32_t *lanes_per_particle,
                   int32_t *ctas_per_sm) {
  if (!b || trial_steps <= 0) return MDG_ERR_INVALID;
  cudaSetDevice(b->prm.device);
  // work on a copy of the state and restore it afterwards
  const size_t n = (size_t)b->total;
  double4_32a *sq = nullptr, *sp = nullptr;
  int *sid = nullptr;
  MDG_BCK(balloc(&sq, n));
  MDG_BCK(balloc(&sp, n));
  MDG_BCK(balloc(&sid, n));
  make_end_current(b);
  MDG_BCK(cudaMemcpyAsync(sq, b->d.q_end, n * 32, cudaMemcpyDeviceToDevice, b->stream));
  MDG_BCK(cudaMemcpyAsync(sp, b->d.p, n * 32, cudaMemcpyDeviceToDevice, b->stream));
  MDG_BCK(cudaMemcpyAsync(sid, b->d.id, n * sizeof(int), cudaMemcpyDeviceToDevice, b->stream));
  std::vector<long long> st0(b->nbox);
  MDG_BCK(cudaMemcpy(st0.data(), b->d.box_steps, b->nbox * sizeof(long long), cudaMemcpyDeviceToHost));
  const long long steps0 = b->steps;
  // one trial: the shape from the saved state with fresh lists; *ms receives
  // the device time of `steps` steps after the two that build the lists
  auto trial = [&](int T, int Lp, int C, int I, int F, int steps, double *ms) -> int {
    b->threads = T;
    b->lpi = Lp;
    b->ctas_per_sm = C;
    b->use_inner = I;
    b->flat = F;
    int rc = assign(b);
    if (rc) return rc;
    MDG_BCK(cudaMemcpyAsync(b->d.q_end, sq, n * 32, cudaMemcpyDeviceToDevice, b->stream));
    MDG_BCK(cudaMemcpyAsync(b->d.p, sp, n * 32, cudaMemcpyDeviceToDevice, b->stream));
    MDG_BCK(cudaMemcpyAsync(b->d.id, sid, n * sizeof(int), cudaMemcpyDeviceToDevice, b->stream));
    MDG_BCK(cudaMemsetAsync(b->d.box_mid, 0xFF, b->nbox * sizeof(int), b->stream));  // q_end restored, current
    std::vector<int> ones(b->nbox, 1);
    MDG_BCK(cudaMemcpyAsync(b->d.box_rebuild, ones.data(), b->nbox * sizeof(int), cudaMemcpyHostToDevice, b->stream));
    MDG_BCK(cudaMemcpyAsync(b->d.box_steps, st0.data(), b->nbox * sizeof(long long), cudaMemcpyHostToDevice, b->stream));
    b->steps = steps0;
    b->par = 0;
    rc = mdg_batch_calculate(b, 2);  // builds lists
    if (rc) return rc;
    rc = mdg_batch_calculate(b, steps);
    if (rc) return rc;
    *ms = b->last_ms;
    return MDG_OK;
  };
  const int Ts[] = {128, 256, 512}, Ls[] = {1, 2, 4}, Cs[] = {1, 2, 3, 4};
  double best = 1e300;
  int bt = b->threads, bl = b->lpi, bc = b->ctas_per_sm, bi = 0, bf = 0;
  for (int T : Ts)
    for (int Lp : Ls)
      for (int C : Cs) {
        if (T * C > 2048) continue;
        b->lpi = Lp;
        b->use_inner = 0;
        b->flat = 0;
        if (C > resident_ctas(b, T)) continue;  // would run in waves (assign would cap it)
        double ms = 0.0;
        int rc = trial(T, Lp, C, 0, 0, trial_steps, &ms);
        if (rc) return rc;
        if (ms < best) {
          best = ms;
          bt = T;
          bl = Lp;
          bc = C;
          bf = 0;
        }
      }
  // the flat layout, one lane per particle, with every resident CTA
  for (int T : {128, 256}) {
    b->lpi = 1;
    b->use_inner = 0;
    b->flat = 1;
    const int C = resident_ctas(b, T);
    double ms = 0.0;
    int rc = trial(T, 1, C, 0, 1, trial_steps, &ms);
    if (rc) return rc;
    if (ms < best) {
      best = ms;
      bt = T;
      bl = 1;
      bc = C;
      bf = 1;
    }
  }
  // the inner list (one lane per particle) on and off over longer trials: it
  // pays when the boxes re-select their inner rows rarely (small steps,
  // FP64), which short trials from fresh lists cannot show.  With the
  // automatic buffer, half the margin is tried beside min(0.1, margin / 2):
  // a longer inner row, re-selected about half as often
  if (bl == 1 && b->P.inner) {
    const int longer = std::max((int)trial_steps, 60);
    double off = 0.0, best_on = 1e300;
    int rc = trial(bt, 1, bc, 0, bf, longer, &off);
    if (rc) return rc;
    const double buf0 = b->buffer;
    double best_buf = buf0;
    std::vector<double> bufs{buf0};
    if (b->prm.prune_buffer < 0.0 && 0.5 * b->prm.margin > buf0 * (1.0 + 1e-9)) bufs.push_back(0.5 * b->prm.margin);
    for (double buf : bufs) {
      set_prune_buffer(b, buf);
      double on = 0.0;
      rc = trial(bt, 1, bc, 1, bf, longer, &on);
      if (rc) return rc;
      if (on < best_on) {
        best_on = on;
        best_buf = buf;
      }
    }
    set_prune_buffer(b, best_buf);
    bi = best_on < off ? 1 : 0;
  }
  b->threads = bt;
  b->lpi = bl;
  b->ctas_per_sm = bc;
  b->use_inner = bi;
  b->flat = bf;
  int rc = assign(b);
  if (rc) return rc;
  MDG_BCK(cudaMemcpyAsync(b->d.q_end, sq, n * 32, cudaMemcpyDeviceToDevice, b->stream));
  MDG_BCK(cudaMemcpyAsync(b->d.p, sp, n * 32, cudaMemcpyDeviceToDevice, b->stream));
  MDG_BCK(cudaMemcpyAsync(b->d.id, sid, n * sizeof(int), cudaMemcpyDeviceToDevice, b->stream));
  MDG_BCK(cudaMemsetAsync(b->d.box_mid, 0xFF, b->nbox * sizeof(int), b->stream));  // q_end restored, current
  std::vector<int> ones(b->nbox, 1);
  MDG_BCK(cudaMemcpyAsync(b->d.box_rebuild, ones.data(), b->nbox * sizeof(int), cudaMemcpyHostToDevice, b->stream));
  MDG_BCK(cudaMemcpyAsync(b->d.box_steps, st0.data(), b->nbox * sizeof(long long), cudaMemcpyHostToDevice, b->stream));
  MDG_BCK(cudaStreamSynchronize(b->stream));
  b->steps = steps0;
  b->par = 0;
  cudaFree(sq);
  cudaFree(sp);
  cudaFree(sid);
  if (threads) *threads = bt;
  if (lanes_per_particle) *lanes_per_particle = bl;
  if (ctas_per_sm) *ctas_per_sm = bc;
  return MDG_OK;
}

int mdg_batch_set_shape(mdg_batch *b, int32_t threads, int32_t lanes_per_particle, int32_t ctas_per_sm) {
  if (!b || (threads != 128 && threads != 256 && threads != 512 && threads != 1024) ||
      (lanes_per_particle != 1 && lanes_per_particle != 2 && lanes_per_particle != 4) || ctas_per_sm < 1 ||
      threads * ctas_per_sm > 2048 || (b->flat && (lanes_per_particle != 1 || threads > kFlatMaxThreads)))
    return MDG_ERR_INVALID;
  b->threads = threads;
  b->lpi = lanes_per_particle;
  b->ctas_per_sm = ctas_per_sm;
  return assign(b);
}

int mdg_batch_set_inner(mdg_batch *b, int32_t on) {
  if (!b) return MDG_ERR_INVALID;
  b->use_inner = on ? 1 : 0;
  return assign(b);  // fresh selections, graphs captured again
}

int mdg_batch_set_flat(mdg_batch *b, int32_t on) {
  if (!b) return MDG_ERR_INVALID;
  if (on && (b->lpi != 1 || b->threads > kFlatMaxThreads))
    return bfail(b, MDG_ERR_INVALID, "the flat layout takes one lane per particle and at most 256 threads per CTA");
  b->flat = on ? 1 : 0;
  return assign(b);
}

int mdg_batch_get_stats(mdg_batch *b, mdg_batch_stats *s) {
  if (!b || !s) return MDG_ERR_INVALID;
  memset(s, 0, sizeof(*s));
  std::vector<long long> rb(b->nbox);
  MDG_BCK(cudaMemcpy(rb.data(), b->d.box_rebuilds, b->nbox * sizeof(long long), cudaMemcpyDeviceToHost));
  s->steps = b->steps;
  for (long long v : rb) s->rebuilds += v;
  s->particles = b->total;
  s->boxes = b->nbox;
  s->list_capacity = b->P.list_cap;
  s->threads = b->threads;
  s->lanes_per_particle = b->lpi;
  s->ctas_per_sm = b->ctas_per_sm;
  s->inner_list = (b->P.inner && b->lpi == 1 && b->use_inner) ? 1 : 0;
  s->flat = b->flat;
  s->prune_buffer = b->P.inner ? b->buffer : 0.0;
  s->elapsed_ms = b->last_ms;
  s->kernel_launches = b->launches;
  return MDG_OK;
}

}  // extern "C"
