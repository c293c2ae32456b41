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
  // k_wrap_bin, the only reader of end_stale in the rebuild, has finished
  if (blockIdx.x == 0 && threadIdx.x == 0) d.flags->end_stale = 0;
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
