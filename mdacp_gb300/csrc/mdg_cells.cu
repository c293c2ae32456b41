// Pair-list rebuild, part 1: periodic wrap, cell binning and the stable
// reorder of particles by cell.
//
// Replaces MeshList::MakeMesh (meshlist.cc:153-205, counting sort into
// cells), MeshList::Sort (meshlist.cc:117-150, reorder of q/p by cell) and the
// wrap of Variables::AdjustPeriodicBoundary (variables.cc:59-79, applied only
// at a rebuild).  Every kernel here is a no-op unless flags->rebuild is set, so
// the whole sequence can sit in every captured step and cost one near-empty
// wave when no rebuild is due.  Grids are a few waves of the SM count with
// grid-stride loops.
//
// Cells are stored in the order of cell_rank.  Order inside a cell is by
// caller particle index, which makes the slot order (and with it every later
// summation order) independent of the atomics used to fill the cells.
#include "mdg_internal.cuh"

namespace mdg {

namespace {

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ bool rebuild_off(const DevFlags *f) { return f->halt != 0 || f->rebuild == 0; }

// Exclusive scan of one int per thread over a 1024-thread block; returns the
// block total in *total.
__device__ int block_exclusive_scan(int v, int *total) {
  __shared__ int warp_tot[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int t = (lane < (int)(blockDim.x >> 5)) ? warp_tot[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    warp_tot[lane] = t;  // inclusive
  }
  __syncthreads();
  const int warp_off = wid ? warp_tot[wid - 1] : 0;
  *total = warp_tot[(blockDim.x >> 5) - 1];
  __syncthreads();
  return warp_off + x - v;
}

// Start of a step: step and Langevin counters; the inner-list re-selection
// requested by the last step (or by a rebuild outside a step) is handed to
// this step's kernel.
__device__ __forceinline__ void start_step(DevFlags *f, int lang_step) {
  f->steps += 1;
  if (lang_step) f->lang += 1;
  f->prune_now = f->prune_next;
  f->prune_next = 0;
  if (f->prune_now) {
    f->prunes += 1;
    f->inner_pairs = 0;
  }
}

// Step-boundary position of slot i in the mixed form from the home-cell-local
// mid-step position: the centre of the home cell plus (q_mid - p dt/2), the
// inverse of the step's last half-drift.
__device__ __forceinline__ double4_32a end_from_mid(const Geom &g, const Dev &d, int i, int mid) {
  const double4_32a u = d.q_mid[mid][i], p = d.p[i];
  int cx, cy, cz;
  cell_unkey(d.cell[i], cx, cy, cz);
  double4_32a q = u;
  q.x = cell_centre(g, 0, cx) + fma(-p.x, g.dt2, u.x);
  q.y = cell_centre(g, 1, cy) + fma(-p.y, g.dt2, u.y);
  q.z = cell_centre(g, 2, cz) + fma(-p.z, g.dt2, u.z);
  return q;
}

// Wraps q_end into the box with the reference rule (one +-L per component),
// bins it and counts cell occupancy.  Thread 0 also advances the step and
// Langevin counters of a step that is starting.  In the mixed form q_end is
// first taken from q_mid[mid] when the steps left it behind.
__global__ void k_wrap_bin(Geom g, Dev d, int count_step, int lang_step, int mid) {
  DevFlags *f = d.flags;
  if (count_step && blockIdx.x == 0 && threadIdx.x == 0 && f->halt == 0) start_step(f, lang_step);
  if (rebuild_off(f)) return;
  const bool from_mid = g.local_pos && f->end_stale;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < g.n; i += gridDim.x * blockDim.x) {
    double4_32a q = from_mid ? end_from_mid(g, d, i, mid) : d.q_end[i];
    double x[3] = {q.x, q.y, q.z};
    int c[3];
    bool bad = false;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      double v = x[k];
      if (v < 0.0) v += g.L[k];
      else if (v > g.L[k]) v -= g.L[k];
      if (!(v >= 0.0 && v <= g.L[k])) bad = true;  // also catches NaN
      x[k] = v;
      int ci = bad ? 0 : (int)(v * g.inv_w[k]);
      c[k] = ci < 0 ? 0 : (ci >= g.nc[k] ? g.nc[k] - 1 : ci);
    }
    if (bad) {
      halt_with(f, kHaltBadState);
      atomicMin(&f->bad_slot, i);
      continue;
    }
    q.x = x[0]; q.y = x[1]; q.z = x[2];
    d.q_end[i] = q;
    d.cell[i] = cell_key(c[0], c[1], c[2]);
    atomicAdd(&d.cell_count[cell_rank(g, c[0], c[1], c[2])], 1);
  }
}

__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(Geom g, Dev d) {
  if (rebuild_off(d.flags)) return;
  const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  int s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; k++)
    if (base + k < g.nrank) s += d.cell_count[base + k];
  int total;
  block_exclusive_scan(s, &total);
  if (threadIdx.x == 0) d.block_sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_top(int nblocks, Dev d) {
  if (rebuild_off(d.flags)) return;
  const int base = threadIdx.x * kScanItems;
  int v[kScanItems], s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    v[k] = (base + k < nblocks) ? d.block_sums[base + k] : 0;
    s += v[k];
  }
  int total;
  int off = block_exclusive_scan(s, &total);
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    if (base + k < nblocks) d.block_sums[base + k] = off;
    off += v[k];
  }
}

__global__ void __launch_bounds__(kScanThreads) k_scan_apply(Geom g, Dev d) {
  if (rebuild_off(d.flags)) return;
  const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  int v[kScanItems], s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    v[k] = (base + k < g.nrank) ? d.cell_count[base + k] : 0;
    s += v[k];
  }
  int total;
  int off = block_exclusive_scan(s, &total) + d.block_sums[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    if (base + k < g.nrank) {
      d.cell_start[base + k] = off;
      d.cell_count[base + k] = 0;
      d.cell_fill[base + k] = 0;
    }
    off += v[k];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) d.cell_start[g.nrank] = g.n;
}

__global__ void k_scatter(Geom g, Dev d) {
  if (rebuild_off(d.flags)) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < g.n; i += gridDim.x * blockDim.x) {
    int cx, cy, cz;
    cell_unkey(d.cell[i], cx, cy, cz);
    const int c = cell_rank(g, cx, cy, cz);
    const int dst = d.cell_start[c] + atomicAdd(&d.cell_fill[c], 1);
    if (MDG_IN_RANGE(d.flags, kCheckScatter, dst, g.n)) d.order[dst] = i;
  }
}

// Insertion sort of each cell's slots by caller index (cells hold tens of
// particles): the order is a function of the state alone.
__global__ void k_cell_sort(Geom g, Dev d) {
  if (rebuild_off(d.flags)) return;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < g.nrank; c += gridDim.x * blockDim.x) {
    const int a = d.cell_start[c], b = d.cell_start[c + 1];
    for (int k = a + 1; k < b; k++) {
      const int v = d.order[k], key = d.id[v];
      int m = k - 1;
      while (m >= a && d.id[d.order[m]] > key) {
        d.order[m + 1] = d.order[m];
        m--;
      }
      d.order[m + 1] = v;
    }
  }
}

__global__ void k_reorder(Geom g, Dev d) {
  if (rebuild_off(d.flags)) return;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < g.n; k += gridDim.x * blockDim.x) {
    const int o = d.order[k];
    d.t_q[k] = d.q_end[o];
    d.t_p[k] = d.p[o];
    d.t_id[k] = d.id[o];
    d.t_cell[k] = d.cell[o];
  }
}

// Copies the sorted staging back, records the build positions and derives the
// positions the next force evaluation uses: q_mid = q + p dt/2 (the first
// half-drift, fcalculator.cc:21-32, rounded as two separate operations).  In
// the mixed form q_mid is kept relative to the centre of the new home cell,
// (q - centre) + p dt/2, and q_end is current again.
__global__ void k_finalize(Geom g, Dev d, int q_mid_dst) {
  double4_32a *q_mid = d.q_mid[q_mid_dst];
  if (rebuild_off(d.flags)) return;
  // k_wrap_bin, the only reader of end_stale in the rebuild, has finished;
  // a new list starts the reference policy's budget (PairList::Init,
  // pairlist.cc:11-23)
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    d.flags->end_stale = 0;
    d.flags->buffer_length = g.margin;
    d.flags->lifetime = 0;
    d.flags->need_check = 0;
  }
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < g.n; k += gridDim.x * blockDim.x) {
    const double4_32a q = d.t_q[k];
    double4_32a p = d.t_p[k];
    const int id = d.t_id[k], c = d.t_cell[k];
    d.q_end[k] = q;
    d.id[k] = id;
    d.cell[k] = c;
    d.inv[id] = k;
    int cx, cy, cz;
    cell_unkey(c, cx, cy, cz);
    const float cw = __int_as_float(c);
    const double ox = cell_centre(g, 0, cx), oy = cell_centre(g, 1, cy), oz = cell_centre(g, 2, cz);
    const float4 lb = make_float4((float)(q.x - ox), (float)(q.y - oy), (float)(q.z - oz), cw);
    d.qf[k] = lb;
    double4_32a m = q;
    if (g.local_pos) {
      m.x = __dadd_rn(q.x - ox, __dmul_rn(p.x, g.dt2));
      m.y = __dadd_rn(q.y - oy, __dmul_rn(p.y, g.dt2));
      m.z = __dadd_rn(q.z - oz, __dmul_rn(p.z, g.dt2));
      // the build reference (for the rebuild test) in q_mid's padding word, and
      // the same position as the prune reference in p's until the step's
      // re-selection records its own
      m.w = pack_ref(g, lb.x, lb.y, lb.z);
      p.w = m.w;
      q_mid[k] = m;
      d.p[k] = p;
      d.loc[q_mid_dst][k] = make_float4((float)m.x, (float)m.y, (float)m.z, cw);
    } else {
      d.p[k] = p;
      d.q_build[k] = q;
      m.x = __dadd_rn(q.x, __dmul_rn(p.x, g.dt2));
      m.y = __dadd_rn(q.y, __dmul_rn(p.y, g.dt2));
      m.z = __dadd_rn(q.z, __dmul_rn(p.z, g.dt2));
      q_mid[k] = m;
      d.loc[q_mid_dst][k] = make_float4((float)(m.x - ox), (float)(m.y - oy), (float)(m.z - oz), cw);
    }
  }
}

// Mixed form: q_end from q_mid[mid] and p for every slot while the steps have
// left it behind; k_end_current then records that it is current (a separate
// kernel, so no thread clears the flag while others still read it).
__global__ void k_end_from_mid(Geom g, Dev d, int mid) {
  if (!d.flags->end_stale) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < g.n; i += gridDim.x * blockDim.x)
    d.q_end[i] = end_from_mid(g, d, i, mid);
}

__global__ void k_end_current(DevFlags *f) { f->end_stale = 0; }

__global__ void k_set_rebuild(DevFlags *f) {
  if (f->halt == 0) f->rebuild = 1;
}

// Graph path: the step-start bookkeeping of k_wrap_bin and the conditions of
// the step's nodes, all decided before the rebuild: a rebuild inside a step
// always re-selects the inner list (k_rebuild_done), and after a halt every
// later kernel is a no-op.  Two forms:
//   rebuild_cond (IF: run the rebuild body) and variant_cond (SWITCH: 0 the
//   ordinary step, 1 the re-selecting one, 2 none), for the timed graphs,
//   which record events between the nodes;
//   step_cond alone (SWITCH: 0 ordinary, 1 re-selecting, 2 rebuild then
//   re-selecting, 3 none), one conditional node per step.
__global__ void k_prelude(DevFlags *f, int lang_step, cudaGraphConditionalHandle rebuild_cond,
                          cudaGraphConditionalHandle variant_cond, cudaGraphConditionalHandle step_cond, int split) {
  if (f->halt == 0) start_step(f, lang_step);
  const bool run = f->halt == 0, rebuild = run && f->rebuild != 0;
  const unsigned variant = !run ? 2u : ((rebuild || f->prune_now) ? 1u : 0u);
  if (split) {
    cudaGraphSetConditional(rebuild_cond, rebuild ? 1u : 0u);
    cudaGraphSetConditional(variant_cond, variant);
  } else {
    cudaGraphSetConditional(step_cond, !run ? 3u : (rebuild ? 2u : variant));
  }
}

}  // namespace

// ----------------------------------------------------------------------------
// The reference's rebuild policy, PairList::IsPairListExpired with
// CheckByDisplacement (pairlist.cc:26-121), evaluated at the start of a step
// (MDManager::Calculate, mdmanager.cc:116-148): the budget starts at the
// margin at every build (PairList::Init, pairlist.cc:11-23) and loses
// 2 max|p| dt per step; once it is negative, every step checks the entries
// displaced by more than (margin - max displacement) since the build: more
// than min(CheckListLength, entries) of them, or one pair of them that was
// outside the search length at the build and is now inside the cut-off,
// expires the list.  The reference runs the check over its local particles
// and their ghost images (GetTotalParticleNumber): a particle within SL of a
// face at the build has an image shifted by +-L across it, cascading over the
// axes (FindBorderParticles, mdunit.cc:125-191).  Ghost positions are
// refreshed after the first half-drift of a step (SendBorderParticles), so at
// the next step's check an image stands at its original's previous mid-step
// position, shifted: here q_mid of the other parity, which the coming step
// has not yet overwritten.  Each entry is scored on its own positions, every
// shifted coordinate formed by one addition as the ghost's is.
namespace {

constexpr int kPolicyThreads = 256;

__device__ __forceinline__ double block_sum_d(double v, double *sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sh[w];
  __syncthreads();
  return t;
}

__device__ __forceinline__ double block_max(double v, double *sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t = fmax(t, sh[w]);
  __syncthreads();
  return t;
}

// Slot i in box coordinates: at the step boundary (the local entry) and at
// the last build; at the previous mid-step (its images) only when it has
// images (`with_mid`).  The mixed forms: home-cell centre plus
// q_mid - p dt/2, plus qf, plus the other q_mid.
struct PolicyPos {
  double end[3], mid[3], bld[3];
};

__device__ __forceinline__ PolicyPos policy_positions(const Geom &g, const Dev &d, int i, int par) {
  PolicyPos r;
  if (g.local_pos) {
    int cx, cy, cz;
    cell_unkey(d.cell[i], cx, cy, cz);
    const double o[3] = {cell_centre(g, 0, cx), cell_centre(g, 1, cy), cell_centre(g, 2, cz)};
    const double4_32a u = d.q_mid[par][i], p = d.p[i];
    const float4 b = d.qf[i];
    r.end[0] = o[0] + fma(-p.x, g.dt2, u.x);
    r.end[1] = o[1] + fma(-p.y, g.dt2, u.y);
    r.end[2] = o[2] + fma(-p.z, g.dt2, u.z);
    r.bld[0] = o[0] + (double)b.x;
    r.bld[1] = o[1] + (double)b.y;
    r.bld[2] = o[2] + (double)b.z;
  } else {
    const double4_32a q = d.q_end[i], b = d.q_build[i];
    r.end[0] = q.x; r.end[1] = q.y; r.end[2] = q.z;
    r.bld[0] = b.x; r.bld[1] = b.y; r.bld[2] = b.z;
  }
  r.mid[0] = r.mid[1] = r.mid[2] = 0.0;
  return r;
}

__device__ __forceinline__ void with_mid(const Geom &g, const Dev &d, int i, int par, PolicyPos &r) {
  const double4_32a v = d.q_mid[par ^ 1][i];
  if (g.local_pos) {
    int cx, cy, cz;
    cell_unkey(d.cell[i], cx, cy, cz);
    r.mid[0] = cell_centre(g, 0, cx) + v.x;
    r.mid[1] = cell_centre(g, 1, cy) + v.y;
    r.mid[2] = cell_centre(g, 2, cz) + v.z;
  } else {
    r.mid[0] = v.x; r.mid[1] = v.y; r.mid[2] = v.z;
  }
}

// Image shifts of a particle along each axis (0, and +1 / -1 when its build
// position lies within SL of the lower / upper face, strictly inside the
// box: find_ghosts' inside_edge rule); its entries are the combinations,
// numbered e = (ax * ny + ay) * nz + az, entry 0 the particle itself.
struct Images {
  int s[3][3];
  int n[3];
};

__device__ __forceinline__ Images images_of(const Geom &g, const double bld[3]) {
  Images im;
  const double sl = g.sl;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    int c = 0;
    im.s[k][c++] = 0;
    if (bld[k] > 0.0 && bld[k] < sl) im.s[k][c++] = 1;
    if (bld[k] > g.L[k] - sl && bld[k] < g.L[k]) im.s[k][c++] = -1;
    im.n[k] = c;
  }
  return im;
}

// Entry e's build and current positions.
__device__ __forceinline__ void entry_positions(const Geom &g, const PolicyPos &pp, const Images &im, int e,
                                                double b[3], double c[3]) {
  const int az = e % im.n[2], ay = (e / im.n[2]) % im.n[1], ax = e / (im.n[2] * im.n[1]);
  const int sh[3] = {im.s[0][ax], im.s[1][ay], im.s[2][az]};
  const double *cur = e == 0 ? pp.end : pp.mid;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    b[k] = sh[k] ? pp.bld[k] + sh[k] * g.L[k] : pp.bld[k];
    c[k] = sh[k] ? cur[k] + sh[k] * g.L[k] : cur[k];
  }
}

__device__ __forceinline__ double entry_disp(const double b[3], const double c[3]) {
  const double dx = b[0] - c[0], dy = b[1] - c[1], dz = b[2] - c[2];
  return dx * dx + dy * dy + dz * dz;
}

// A particle outside the cells at the faces has no image (cells are at least
// SL wide), and its one entry's displacement needs no box coordinates: the
// build minus the step-boundary position, home-cell-local in the mixed forms.
__device__ __forceinline__ bool face_cell(const Geom &g, const Dev &d, int i) {
  int cx, cy, cz;
  cell_unkey(d.cell[i], cx, cy, cz);
  return cx == 0 || cy == 0 || cz == 0 || cx == g.nc[0] - 1 || cy == g.nc[1] - 1 || cz == g.nc[2] - 1;
}

__device__ __forceinline__ double local_disp(const Geom &g, const Dev &d, int i, int par) {
  double dx, dy, dz;
  if (g.local_pos) {
    const double4_32a u = d.q_mid[par][i], p = d.p[i];
    const float4 b = d.qf[i];
    dx = (double)b.x - fma(-p.x, g.dt2, u.x);
    dy = (double)b.y - fma(-p.y, g.dt2, u.y);
    dz = (double)b.z - fma(-p.z, g.dt2, u.z);
  } else {
    const double4_32a q = d.q_end[i], b = d.q_build[i];
    dx = b.x - q.x;
    dy = b.y - q.y;
    dz = b.z - q.z;
  }
  return dx * dx + dy * dy + dz * dz;
}

// The policy is not evaluated when a rebuild is already due (the reference's
// uninitialized list) or after a halt.
__device__ __forceinline__ bool policy_off(const DevFlags *f) { return f->halt != 0 || f->rebuild != 0; }

__global__ void __launch_bounds__(kPolicyThreads) k_policy_vmax(Geom g, Dev d) {
  __shared__ double sh[kPolicyThreads / 32];
  if (policy_off(d.flags)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double v = 0.0;
  if (i < g.n) {
    const double4_32a p = d.p[i];
    v = p.x * p.x + p.y * p.y + p.z * p.z;
  }
  const double m = block_max(v, sh);
  if (threadIdx.x == 0) d.vpart[blockIdx.x] = m;
}

// The budget: lifetime, vmax, the too-fast abort, the budget's decrease, and
// whether this step checks displacements (pairlist.cc:26-65).
__global__ void __launch_bounds__(1024) k_policy_budget(Geom g, Dev d, int nparts, cudaGraphConditionalHandle check_cond,
                                                        int use_cond) {
  __shared__ double sh[32];
  DevFlags *f = d.flags;
  const bool off = policy_off(f);
  double v = 0.0;
  if (!off)
    for (int k = threadIdx.x; k < nparts; k += blockDim.x) v = fmax(v, d.vpart[k]);
  const double vmax2 = block_max(v, sh);
  if (threadIdx.x != 0) return;
  int need = 0;
  if (!off) {
    f->lifetime += 1;
    double buf = f->buffer_length;
    if (buf > 0.0) {
      const double vmax = sqrt(vmax2);
      f->vmax = vmax;
      if (vmax * 2.0 * g.dt > g.margin) {
        halt_with(f, kHaltTooFast);
      } else {
        buf = buf - vmax * 2.0 * g.dt;
        f->buffer_length = buf;
      }
    }
    need = f->halt == 0 && buf < 0.0;
    if (need) f->checks += 1;
  }
  f->need_check = need;
  if (use_cond) cudaGraphSetConditional(check_cond, need ? 1u : 0u);
}

// Per slot the local entry's displacement (t_q.x) and the largest of its
// images' (t_q.y; the images are scored only for particles that have any);
// per block the largest displacement and the entry count, the latter in
// vpart[nparts + block].
__global__ void __launch_bounds__(kPolicyThreads) k_policy_disp(Geom g, Dev d, int par) {
  __shared__ double sh[kPolicyThreads / 32];
  if (!d.flags->need_check) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double dmax = 0.0, entries = 0.0;
  if (i < g.n && !face_cell(g, d, i)) {
    const double d0 = local_disp(g, d, i, par);
    d.t_q[i].x = d0;
    d.t_q[i].y = 0.0;
    dmax = d0;
    entries = 1.0;
  } else if (i < g.n) {
    PolicyPos pp = policy_positions(g, d, i, par);
    const Images im = images_of(g, pp.bld);
    const int ne = im.n[0] * im.n[1] * im.n[2];
    if (ne > 1) with_mid(g, d, i, par, pp);
    double b[3], c[3];
    entry_positions(g, pp, im, 0, b, c);
    const double d0 = entry_disp(b, c);
    double dimg = 0.0;
    for (int e = 1; e < ne; e++) {
      entry_positions(g, pp, im, e, b, c);
      dimg = fmax(dimg, entry_disp(b, c));
    }
    d.t_q[i].x = d0;  // staging: free until a rebuild reorders
    d.t_q[i].y = dimg;
    dmax = fmax(d0, dimg);
    entries = (double)ne;
  }
  const double m = block_max(dmax, sh);
  const double t = block_sum_d(entries, sh);
  if (threadIdx.x == 0) {
    d.vpart[blockIdx.x] = m;
    d.vpart[gridDim.x + blockIdx.x] = t;
  }
}

__global__ void __launch_bounds__(1024) k_policy_threshold(Geom g, Dev d, int nparts) {
  __shared__ double sh[32];
  DevFlags *f = d.flags;
  if (!f->need_check) return;
  double v = 0.0, e = 0.0;
  for (int k = threadIdx.x; k < nparts; k += blockDim.x) {
    v = fmax(v, d.vpart[k]);
    e += d.vpart[nparts + k];
  }
  const double dr2_max = block_max(v, sh);
  const double entries = block_sum_d(e, sh);
  if (threadIdx.x == 0) {
    f->entries = (int)entries;
    const double c_distance = g.margin - sqrt(dr2_max);
    f->c_d2 = c_distance * c_distance;
    f->cand_count = 0;
    f->cand_slots = 0;
  }
}

// Candidate entries (any order: the outcome depends on their set alone):
// counted toward the limit; each particle with any is recorded with the mask
// of its candidate entries.
__global__ void __launch_bounds__(kPolicyThreads) k_policy_candidates(Geom g, Dev d, int par) {
  DevFlags *f = d.flags;
  if (!f->need_check) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n) return;
  const double c_d2 = f->c_d2;
  if (!(d.t_q[i].x > c_d2) && !(d.t_q[i].y > c_d2)) return;  // no entry of this particle
  unsigned mask = 0;
  if (!face_cell(g, d, i)) {
    mask = 1u;  // its only entry, scored by k_policy_disp
  } else {
    PolicyPos pp = policy_positions(g, d, i, par);
    const Images im = images_of(g, pp.bld);
    const int ne = im.n[0] * im.n[1] * im.n[2];
    if (ne > 1) with_mid(g, d, i, par, pp);
    for (int e = 0; e < ne; e++) {
      double b[3], c[3];
      entry_positions(g, pp, im, e, b, c);
      if (entry_disp(b, c) > c_d2) mask |= 1u << e;
    }
  }
  if (!mask) return;
  atomicAdd(&f->cand_count, __popc(mask));
  const int k = atomicAdd(&f->cand_slots, 1);
  if (k < g.check_list) {
    d.cand[k] = i;
    d.cand[g.check_list + k] = (int)mask;
  }
}

// Expired when the candidate entries reached min(CheckListLength, entries),
// or when a pair of candidate entries outside the search length at the build
// is inside the cut-off now (two entries of one particle are a box length
// apart and never are).  Block a takes the pairs (a, b > a) of the recorded
// candidate particles, its threads striding over b; any block that finds one
// sets the rebuild flag (a plain store of 1).
__global__ void __launch_bounds__(kPolicyThreads) k_policy_pairs(Geom g, Dev d, int par) {
  DevFlags *f = d.flags;
  if (!f->need_check) return;
  const int nl = min(g.check_list, f->entries);
  const int cnt = f->cand_count, np = f->cand_slots;
  if (cnt >= nl) {
    if (blockIdx.x == 0 && threadIdx.x == 0) f->rebuild = 1;
    return;
  }
  const int a = blockIdx.x;
  if (a >= np) return;
  const int ia = d.cand[a];
  const unsigned ma = (unsigned)d.cand[g.check_list + a];
  PolicyPos pa = policy_positions(g, d, ia, par);
  const Images ima = images_of(g, pa.bld);
  if (ima.n[0] * ima.n[1] * ima.n[2] > 1) with_mid(g, d, ia, par, pa);
  int expired = 0;
  for (int b = a + 1 + threadIdx.x; b < np && !expired; b += blockDim.x) {
    const int ib = d.cand[b];
    const unsigned mb = (unsigned)d.cand[g.check_list + b];
    PolicyPos pb = policy_positions(g, d, ib, par);
    const Images imb = images_of(g, pb.bld);
    if (imb.n[0] * imb.n[1] * imb.n[2] > 1) with_mid(g, d, ib, par, pb);
    for (unsigned xa = ma; xa && !expired; xa &= xa - 1) {
      double ba[3], ca[3];
      entry_positions(g, pa, ima, __ffs(xa) - 1, ba, ca);
      for (unsigned xb = mb; xb && !expired; xb &= xb - 1) {
        double bb[3], cb[3];
        entry_positions(g, pb, imb, __ffs(xb) - 1, bb, cb);
        double dx = ba[0] - bb[0], dy = ba[1] - bb[1], dz = ba[2] - bb[2];
        if (dx * dx + dy * dy + dz * dz < g.sl2) continue;
        dx = ca[0] - cb[0];
        dy = ca[1] - cb[1];
        dz = ca[2] - cb[2];
        if (dx * dx + dy * dy + dz * dz < g.rc2) expired = 1;
      }
    }
  }
  if (expired) f->rebuild = 1;
}

}  // namespace

void launch_policy(const Geom &g, const Dev &d, cudaStream_t s, cudaGraphConditionalHandle check_cond, int use_cond) {
  const int grid = g.n > 0 ? (g.n + kPolicyThreads - 1) / kPolicyThreads : 1;
  k_policy_vmax<<<grid, kPolicyThreads, 0, s>>>(g, d);
  k_policy_budget<<<1, 1024, 0, s>>>(g, d, grid, check_cond, use_cond);
}

void launch_policy_check(const Geom &g, const Dev &d, int par, cudaStream_t s) {
  const int grid = g.n > 0 ? (g.n + kPolicyThreads - 1) / kPolicyThreads : 1;
  k_policy_disp<<<grid, kPolicyThreads, 0, s>>>(g, d, par);
  k_policy_threshold<<<1, 1024, 0, s>>>(g, d, grid);
  k_policy_candidates<<<grid, kPolicyThreads, 0, s>>>(g, d, par);
  // one block per candidate particle the check can record
  k_policy_pairs<<<g.check_list, kPolicyThreads, 0, s>>>(g, d, par);
}

// Declared in mdg_list.cu.
void launch_build_list(const Geom &g, const Dev &d, int num_sms, cudaStream_t s, bool in_step);

void launch_set_rebuild(const Dev &d, cudaStream_t s) { k_set_rebuild<<<1, 1, 0, s>>>(d.flags); }

void launch_end_from_mid(const Geom &g, const Dev &d, int par, cudaStream_t s) {
  const int threads = 256;
  int grid = (g.n + threads - 1) / threads;
  if (grid < 1) grid = 1;
  k_end_from_mid<<<grid, threads, 0, s>>>(g, d, par);
  k_end_current<<<1, 1, 0, s>>>(d.flags);
}

void launch_prelude_split(const Dev &d, int lang_step, cudaGraphConditionalHandle rebuild_cond,
                          cudaGraphConditionalHandle variant_cond, cudaStream_t s) {
  k_prelude<<<1, 1, 0, s>>>(d.flags, lang_step, rebuild_cond, variant_cond, 0, 1);
}

void launch_prelude(const Dev &d, int lang_step, cudaGraphConditionalHandle step_cond, cudaStream_t s) {
  k_prelude<<<1, 1, 0, s>>>(d.flags, lang_step, 0, 0, step_cond, 0);
}

void launch_rebuild(const Geom &g, const Dev &d, int q_mid_dst, int num_sms, cudaStream_t s, bool count_step,
                    bool lang_step, bool in_step) {
  const int threads = 256;
  int grid = (g.n + threads - 1) / threads;
  const int cap = num_sms * 8;
  if (grid > cap) grid = cap;
  if (grid < 1) grid = 1;
  int cgrid = (g.nrank + threads - 1) / threads;
  if (cgrid > cap) cgrid = cap;
  const int nb = (g.nrank + kScanTile - 1) / kScanTile;
  k_wrap_bin<<<grid, threads, 0, s>>>(g, d, count_step ? 1 : 0, lang_step ? 1 : 0, q_mid_dst);
  k_scan_reduce<<<nb, kScanThreads, 0, s>>>(g, d);
  k_scan_top<<<1, kScanThreads, 0, s>>>(nb, d);
  k_scan_apply<<<nb, kScanThreads, 0, s>>>(g, d);
  k_scatter<<<grid, threads, 0, s>>>(g, d);
  k_cell_sort<<<cgrid, threads, 0, s>>>(g, d);
  k_reorder<<<grid, threads, 0, s>>>(g, d);
  k_finalize<<<grid, threads, 0, s>>>(g, d, q_mid_dst);
  launch_build_list(g, d, num_sms, s, in_step);
}

}  // namespace mdg
