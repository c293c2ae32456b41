// One MD step as one kernel, plus the observers and the state exchange.
//
// k_step replaces, for one step of MDManager::Calculate (mdmanager.cc:116-148):
//   ForceCalculator::CalculateForce (fcalculator.cc:35-50, 229-290): the LJ
//     pair force of the smoothly truncated potential, applied as p += F dt;
//   the thermostat of MDManager::CalculateLangevin / CalculateNoseHoover
//     (mdmanager.cc:160-192, fcalculator.cc:743-778);
//   the second half-drift ForceCalculator::UpdatePositionHalf (fcalculator.cc:21-32)
//     and the first half-drift of the following step;
//   the expiry test of PairList::IsPairListExpired (pairlist.cc:26-45), here the
//     displacement criterion: moved more than margin/2 since the build.
// It is a gather over the full neighbour list: one thread per particle, no
// atomics, no reaction scatter (the "Reactless" form, fcalculator.cc:504-542).
//
// FP64 form: the pair force is evaluated in double precision.  1/r^2 comes
// from the hardware reciprocal estimate (rcp.approx.ftz.f64) refined by one
// Householder step of order three, y <- y (1 + e + e^2), e = 1 - r^2 y, which
// cubes the relative error of the estimate.
// Mixed form (MDG_MIXED): particle positions relative to their home-cell
// centre in float; the pair force in float; the per-particle force sum in
// compensated float (Kahan: each term's lost low part carried in a second
// float, four float operations per component and pair), so the sum's error
// does not grow with the number of partners; converted to double once per
// particle; momentum and position updates in double with fused multiply-adds,
// the mid-step positions kept relative to the centre of the home cell (so the
// float position partners gather is one conversion and the displacement since
// the build is tested in float against the build's local position, which
// travels packed in q_mid's padding word, as the prune reference does in p's)
// and the step-boundary positions not written (the readers rebuild them from
// q_mid and p).  MDG_MIXED_PLAIN sums the pair forces in plain float instead (an
// error near u sqrt(40) |f_ij|, u = 2^-24, over about 40 terms).  GB300 runs
// double precision at 1/64 of the float rate, so the per-particle double work
// (momentum, two half-drifts) is kept to one operation per component each,
// and the per-pair work stays in float.
#include "mdg_internal.cuh"

namespace mdg {

namespace {

constexpr int kStepThreads = 128;  // observers, forces, state exchange
// Threads per block of the mixed-form step kernel: 128 for the ordinary
// variant, 384 for the re-selecting one, which walks the outer rows and
// writes the inner rows of consecutive slots (4M atoms, mean step kernel of
// a 20-step window 5 steps after a fresh list / of 400 steps with their
// rebuilds and re-selections, in ms: ordinary/re-selecting 128/128 0.4314 /
// 0.4473; 128/128 at 80 registers for the re-selecting variant 0.4278 /
// 0.4445; 384/384 0.4202 / 0.4322; 256/384 0.4150 / 0.4275; 128/512 0.4132 /
// 0.4261; 128/384 0.4119 / 0.4238).  The FP64 form (FP64-pipe bound) keeps
// 128 for both: 5.795 against 5.831 ms at 384.
#ifndef MDG_STEP_THREADS_MIXED
#define MDG_STEP_THREADS_MIXED 128
#endif
#ifndef MDG_PRUNE_THREADS_MIXED
#define MDG_PRUNE_THREADS_MIXED 384
#endif
// (Nose-Hoover: one size for both variants, whose block sums k_nh_update adds)
template <int THERMO, int MIXED, int PMODE>
__host__ __device__ constexpr int step_threads() {
  return !MIXED ? kStepThreads
                : (PMODE == 1 || THERMO == MDG_NOSEHOOVER ? MDG_STEP_THREADS_MIXED : MDG_PRUNE_THREADS_MIXED);
}
// Resident blocks per SM requested for the ordinary step variant (the
// register budget follows: 65536 / (blocks * 128) per thread).  The kernel
// waits on gathers, so occupancy pays: 12 blocks (40 registers, 48 warps per
// SM) ran 16 % faster than the unconstrained 61-register build at 4M atoms.
#ifndef MDG_STEP_MIN_BLOCKS
#define MDG_STEP_MIN_BLOCKS 12
#endif
// The same for the compensated mixed form.  Its three correction terms fit
// in 40 registers since the build reference is no longer held across the
// pair loop (it travels packed in q_mid.w); before, 12 blocks with a 48-byte
// spill still measured 6 % faster than 10 blocks at 48 registers without it
// (4M atoms, 400 steps: 0.472 against 0.501 ms per step kernel).
#ifndef MDG_STEP_MIN_BLOCKS_KAHAN
#define MDG_STEP_MIN_BLOCKS_KAHAN 12
#endif
#ifndef MDG_PRUNE_MIN_BLOCKS
#define MDG_PRUNE_MIN_BLOCKS 8
#endif
// Neighbour-list entries whose index and position loads are issued together
// in the mixed-form force loop.
#ifndef MDG_STEP_UNROLL
#define MDG_STEP_UNROLL 4
#endif
constexpr int kUnroll = MDG_STEP_UNROLL;

// List rows requested into L2 this many entries ahead of the pair loop (0:
// none).  16 measured best at 4M atoms (step kernel 0.476 -> 0.440 ms; 8: 0.472,
// 12: 0.472, 20: 0.442, 24: 0.445, 32: 0.452, 64: 0.458).
#ifndef MDG_ENTRY_L2_AHEAD
#define MDG_ENTRY_L2_AHEAD 16
#endif
constexpr int kEntryAhead = MDG_ENTRY_L2_AHEAD;

__device__ __forceinline__ double rcp_hh3(double x) {
  double y;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  const double e = fma(-x, y, 1.0);
  return fma(y, fma(e, e, e), y);
}

struct CellPos {
  int cx, cy, cz;
  bool edge;
};

__device__ __forceinline__ CellPos cell_pos(const Geom &g, int key) {
  CellPos r;
  cell_unkey(key, r.cx, r.cy, r.cz);
  r.edge = r.cx == 0 || r.cy == 0 || r.cz == 0 || r.cx == g.nc[0] - 1 || r.cy == g.nc[1] - 1 || r.cz == g.nc[2] - 1;
  return r;
}

// The same from the coordinates packed in the w word of qf / loc (equal
// between the two: both are written with the home cell of the last build).
__device__ __forceinline__ CellPos cell_pos_packed(const Geom &g, float w) {
  CellPos r;
  cell_unpack(w, r.cx, r.cy, r.cz);
  r.edge = r.cx == 0 || r.cy == 0 || r.cz == 0 || r.cx == g.nc[0] - 1 || r.cy == g.nc[1] - 1 || r.cz == g.nc[2] - 1;
  return r;
}

// Image of partner position qj seen from a particle in cell cp through stencil
// offset bits of entry e: +-L where the offset crosses the periodic boundary.
__device__ __forceinline__ void apply_image(const Geom &g, const CellPos &cp, uint32_t e, double4_32a &qj) {
  const int ox = entry_sx(e), oy = entry_sy(e), oz = entry_sz(e);
  if (ox == 0 && cp.cx == 0) qj.x -= g.L[0];
  else if (ox == 2 && cp.cx == g.nc[0] - 1) qj.x += g.L[0];
  if (oy == 0 && cp.cy == 0) qj.y -= g.L[1];
  else if (oy == 2 && cp.cy == g.nc[1] - 1) qj.y += g.L[1];
  if (oz == 0 && cp.cz == 0) qj.z -= g.L[2];
  else if (oz == 2 && cp.cz == g.nc[2] - 1) qj.z += g.L[2];
}

// Sum over the row of slot i of f(r) (q_j - q_i), f(r) = 24 r^-8 - 48 r^-14 + 8 C2,
// the force on i (fcalculator.cc:263-277 without the dt factor).
// `list`/`counts` is the inner (pruned) list in an ordinary step and the outer
// list for a stand-alone force evaluation.  With PRUNE the outer list is
// walked and every entry within the prune radius is copied to the inner row
// of slot i (d.pl); *kept receives the new row length.
template <bool PRUNE>
__device__ __forceinline__ double3 force_fp64(const Geom &g, const Dev &d, const double4_32a *__restrict__ pos, int i,
                                              const CellPos &cp, const uint32_t *__restrict__ list,
                                              const int *__restrict__ counts, int *kept) {
  const double4_32a qi = pos[i];
  int cnt = counts[i];
  if (!MDG_IN_RANGE(d.flags, kCheckStepRow, cnt, g.list_cap + 1)) cnt = 0;
  const uint32_t *row = list + i;
  const double thr = (double)g.prune_thr2;
  // r2 >= +0, so its bit pattern orders like the value (a NaN compares above
  // every finite bound): the cutoff tests run on the integer pipe instead of
  // the FP64 pipe (1/64 of the FP32 rate; 6 % of the FP64 step at 4M atoms)
  const long long rc2_bits = __double_as_longlong(g.rc2), thr_bits = __double_as_longlong(thr);
  int m = 0;
  double fx = 0.0, fy = 0.0, fz = 0.0;
  for (int k = 0; k < cnt; k++) {
    const uint32_t e = __ldg(row + (size_t)k * g.stride);
    if (!MDG_IN_RANGE(d.flags, kCheckStepSlot, entry_slot(e), g.n)) continue;
    double4_32a qj = ldg4(pos + entry_slot(e));
    if (cp.edge) apply_image(g, cp, e, qj);
    const double dx = qj.x - qi.x, dy = qj.y - qi.y, dz = qj.z - qi.z;
    const double r2 = dx * dx + dy * dy + dz * dz;
    if (PRUNE && __double_as_longlong(r2) <= thr_bits) d.pl[(size_t)(m++) * g.stride + i] = e;
    if (__double_as_longlong(r2) <= rc2_bits) {
      const double inv = rcp_hh3(r2);
      const double i6 = inv * inv * inv;
      const double df = (i6 * inv) * fma(-48.0, i6, 24.0) + g.c2x8;
      fx = fma(df, dx, fx);
      fy = fma(df, dy, fy);
      fz = fma(df, dz, fz);
    }
  }
  if (PRUNE) *kept = m;
  return make_double3(fx, fy, fz);
}

// Walks the row of slot i on home-cell-local float positions and hands each
// entry's partner offset q_j - q_i and its r^2 to pair(e, dx, dy, dz, r2).
// The offset between the home cells of i and j is ox*w + s*(L - nc*w) per
// axis, s the periodic wrap of the stencil step, evaluated as the quadratic
// of axis_quad.  EDGE: the home cell touches the periodic boundary, so the
// offset is the quadratic; otherwise it is linear with the cell width as
// slope (b = 0, a = w: fmaf(fmaf(0, t, a), t, c) = fmaf(a, t, c) exactly), the
// width coming from the kernel parameters instead of two registers per axis.
// An entry whose slot a checked build rejects (code `site`) and the padding of
// the last batch get a partner at 1e30, whose r^2 overflows to +inf.
template <bool EDGE, int SITE, class Pair>
__device__ __forceinline__ void walk_row(const Geom &g, const Dev &d, const float4 *__restrict__ loc, int i,
                                         const float4 &li, const CellPos &cp, const uint32_t *__restrict__ list,
                                         int cnt, Pair &&pair) {
  AxisQuad qx, qy, qz;
  if (EDGE) {
    qx = axis_quad(g.w32[0], g.dl32[0], cp.cx == 0, cp.cx == g.nc[0] - 1, li.x, 1.0f);
    qy = axis_quad(g.w32[1], g.dl32[1], cp.cy == 0, cp.cy == g.nc[1] - 1, li.y, 0.25f);
    qz = axis_quad(g.w32[2], g.dl32[2], cp.cz == 0, cp.cz == g.nc[2] - 1, li.z, 0.0625f);
  } else {
    qx.a = g.w32[0];
    qy.a = 0.25f * g.w32[1];
    qz.a = 0.0625f * g.w32[2];
    qx.b = qy.b = qz.b = 0.0f;
    qx.c = -li.x;
    qy.c = -li.y;
    qz.c = -li.z;
  }
  const uint32_t *row = list + i;
  const size_t stride = (size_t)g.stride;
  auto gather = [&](uint32_t e) -> float4 {
    const int j = entry_slot(e);
    if (!MDG_IN_RANGE(d.flags, SITE, j, g.n)) return make_float4(1e30f, 1e30f, 1e30f, 0.f);
    return __ldg(loc + j);
  };
  auto offset = [&](uint32_t e, const float4 &lj) {
    const float tx = step_float(e, 0x03u, 8388609.0f);   // t
    const float ty = step_float(e, 0x0Cu, 8388612.0f);   // 4 t
    const float tz = step_float(e, 0x30u, 8388624.0f);   // 16 t
    float dx, dy, dz;
    if (EDGE) {
      dx = lj.x + fmaf(fmaf(qx.b, tx, qx.a), tx, qx.c);
      dy = lj.y + fmaf(fmaf(qy.b, ty, qy.a), ty, qy.c);
      dz = lj.z + fmaf(fmaf(qz.b, tz, qz.a), tz, qz.c);
    } else {
      dx = lj.x + fmaf(qx.a, tx, qx.c);
      dy = lj.y + fmaf(qy.a, ty, qy.c);
      dz = lj.z + fmaf(qz.a, tz, qz.c);
    }
    pair(e, dx, dy, dz, dx * dx + dy * dy + dz * dz);
  };
  int k = 0;
  // the next batch's list entries are requested before this batch's partner
  // positions are used, so the entry load (from DRAM) overlaps the gathers;
  // the last full batch requests the row's remaining (< kUnroll) entries
  const int full = cnt - cnt % kUnroll;
  uint32_t en[kUnroll];
#pragma unroll
  for (int u = 0; u < kUnroll; u++) en[u] = u < cnt ? __ldg(row + (size_t)u * stride) : 0u;
#pragma unroll 1
  for (; k < full; k += kUnroll) {
    uint32_t e[kUnroll];
    float4 l[kUnroll];
#pragma unroll
    for (int u = 0; u < kUnroll; u++) e[u] = en[u];
#pragma unroll
    for (int u = 0; u < kUnroll; u++) l[u] = gather(e[u]);
#pragma unroll
    for (int u = 0; u < kUnroll; u++) {
      const int kn = k + kUnroll + u;
      en[u] = kn < cnt ? __ldg(row + (size_t)kn * stride) : 0u;
    }
    if (kEntryAhead > 0) {
      // rows kEntryAhead further on, into L2: lane l requests row
      // k + kEntryAhead + (l mod 4) of its own column, so one instruction
      // covers the warp's four next rows, one 128-byte line each
      const int kp = k + kEntryAhead + (int)(threadIdx.x & 3);
      if (kp < cnt) asm volatile("prefetch.global.L2 [%0];" ::"l"(row + (size_t)kp * stride));
    }
#pragma unroll
    for (int u = 0; u < kUnroll; u++) offset(e[u], l[u]);
  }
  if (k < cnt) {
    // the remainder as one batch
    constexpr int kTail = kUnroll > 1 ? kUnroll - 1 : 1;
    float4 l[kTail];
#pragma unroll
    for (int u = 0; u < kTail; u++)
      l[u] = k + u < cnt ? gather(en[u]) : make_float4(1e30f, 1e30f, 1e30f, 0.f);
#pragma unroll
    for (int u = 0; u < kTail; u++) offset(en[u], l[u]);
  }
}

// Mixed form of force_fp64: the sum over the row of slot i of f(r) (q_j - q_i)
// in float.  KAHAN: the per-particle sums compensated (MDG_MIXED), else plain
// float (MDG_MIXED_PLAIN).  With PRUNE every entry within the prune radius is
// copied to the inner row of slot i, as in force_fp64.
template <bool PRUNE, bool KAHAN, bool EDGE>
__device__ __forceinline__ double3 pair_loop(const Geom &g, const Dev &d, const float4 *__restrict__ loc, int i,
                                             const float4 &li, const CellPos &cp, const uint32_t *__restrict__ list,
                                             const int *__restrict__ counts, int *kept) {
  int cnt = counts[i];
  if (!MDG_IN_RANGE(d.flags, kCheckStepRow, cnt, g.list_cap + 1)) cnt = 0;
  const size_t stride = (size_t)g.stride;
  float sx = 0.f, sy = 0.f, sz = 0.f;
  float cx = 0.f, cy = 0.f, cz = 0.f;  // Kahan corrections
  const float rc2 = g.rc2f, c2x8 = g.c2x8f, thr = g.prune_thr2;
  int m = 0;
  walk_row<EDGE, kCheckStepSlot>(g, d, loc, i, li, cp, list, cnt, [&](uint32_t e, float dx, float dy, float dz, float r2) {
    if (PRUNE && r2 <= thr) d.pl[(size_t)(m++) * stride + i] = e;
    // evaluated for every entry and masked: no divergent branch per pair
    float inv;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(inv) : "f"(r2));
    const float i6 = inv * inv * inv;
    float df = (i6 * inv) * fmaf(-48.0f, i6, 24.0f) + c2x8;
    df = r2 <= rc2 ? df : 0.0f;
    if (KAHAN) {
      // a zero term (a pair beyond rc) leaves s - c unchanged as a real
      // number (t - s is exact, and so is the new correction), but it moves
      // the correction into s and the later additions round differently:
      // lists that differ only by pairs beyond rc give forces that agree to
      // about one float rounding, not bit for bit
      kahan_fma(sx, cx, df, dx);
      kahan_fma(sy, cy, df, dy);
      kahan_fma(sz, cz, df, dz);
    } else {
      sx = fmaf(df, dx, sx);
      sy = fmaf(df, dy, sy);
      sz = fmaf(df, dz, sz);
    }
  });
  if (PRUNE) *kept = m;
  // the compensated sum rounded once to float (relative 6e-8 of the force),
  // then one conversion per component: GB300 runs double at 1/64 of float
  if (KAHAN) return make_double3((double)(sx - cx), (double)(sy - cy), (double)(sz - cz));
  return make_double3((double)sx, (double)sy, (double)sz);
}

// The pair loop for the calling warp: the linear offset when no active lane's
// home cell touches the periodic boundary (about four warps in five at 66
// cells a side), the quadratic otherwise; both give the same forces bit for
// bit.  Registers are allocated for the larger loop, but the interior one
// needs six fewer and runs without the other's spills.
template <bool PRUNE, bool KAHAN>
__device__ __forceinline__ double3 force_mixed(const Geom &g, const Dev &d, const float4 *__restrict__ loc, int i,
                                               const float4 &li, const CellPos &cp, const uint32_t *__restrict__ list,
                                               const int *__restrict__ counts, int *kept) {
  if (__all_sync(__activemask(), !cp.edge)) return pair_loop<PRUNE, KAHAN, false>(g, d, loc, i, li, cp, list, counts, kept);
  return pair_loop<PRUNE, KAHAN, true>(g, d, loc, i, li, cp, list, counts, kept);
}

__device__ __forceinline__ uint32_t mulhi32(uint32_t a, uint32_t b) { return __umulhi(a, b); }

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) and Box-Muller in float:
// the Langevin noise stream, keyed by seed, counted by (particle, step).
__device__ __forceinline__ void langevin_normals(uint64_t seed, uint32_t id, uint64_t step, double z[3]) {
  uint32_t c0 = id, c1 = (uint32_t)step, c2 = (uint32_t)(step >> 32), c3 = 0x4C4A4D44u;
  uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
#pragma unroll
  for (int r = 0; r < 10; r++) {
    if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
    const uint32_t hi0 = mulhi32(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
    const uint32_t hi1 = mulhi32(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
    const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
  }
  const float s24 = 5.9604644775390625e-08f;
  const float u1 = (float)((c0 >> 8) + 1u) * s24, u2 = (float)(c1 >> 8) * s24;
  const float u3 = (float)((c2 >> 8) + 1u) * s24, u4 = (float)(c3 >> 8) * s24;
  const float twopi = 6.28318530717958647692f;
  const float ra = sqrtf(-2.0f * logf(u1)), rb = sqrtf(-2.0f * logf(u3));
  z[0] = (double)(ra * cosf(twopi * u2));
  z[1] = (double)(ra * sinf(twopi * u2));
  z[2] = (double)(rb * cosf(twopi * u4));
}

__device__ __forceinline__ double block_sum(double v, double *sh) {
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

// PMODE: 0 = decide from flags->prune_now in the kernel (both paths compiled);
// 1 = ordinary step only, 2 = re-selecting step only (each a no-op when the
// flag says otherwise, so the graph path can run the lighter variant).
template <int THERMO, int COMPAT, int MIXED, int PMODE>
// The resident-block counts of the launch bounds are for 128-thread blocks.
__global__ void __launch_bounds__(step_threads<THERMO, MIXED, PMODE>(), (PMODE != 1          ? MDG_PRUNE_MIN_BLOCKS
                                                         : MIXED == MDG_MIXED ? MDG_STEP_MIN_BLOCKS_KAHAN
                                                                              : MDG_STEP_MIN_BLOCKS) *
                                                            128 / step_threads<THERMO, MIXED, PMODE>())
    k_step(Geom g, Dev d, int par) {
  const DevFlags *f = d.flags;
  if (f->halt != 0) return;
  if (PMODE == 1 && f->prune_now != 0) return;
  if (PMODE == 2 && f->prune_now == 0) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = i < g.n;
  const double4_32a *qm = d.q_mid[par];
  double4_32a *qn = d.q_mid[par ^ 1];
  double ke = 0.0;
  // inner-list re-selection: the same for the whole grid this step
  const bool prune = PMODE == 2 ? true : (PMODE == 1 ? false : f->prune_now != 0);
  int kept = 0;
  if (active) {
    // mixed: this force evaluation's local position (partners gather the
    // same array); FP64: the build-time local position.  The w word of
    // either holds the home-cell coordinates
    const float4 lb = MIXED ? d.loc[par][i] : d.qf[i];
    const CellPos cp = cell_pos_packed(g, lb.w);
    double3 F;
    if (prune)
      F = MIXED ? force_mixed<true, MIXED == MDG_MIXED>(g, d, d.loc[par], i, lb, cp, d.nl, d.ncount, &kept)
                : force_fp64<true>(g, d, qm, i, cp, d.nl, d.ncount, &kept);
    else
      F = MIXED ? force_mixed<false, MIXED == MDG_MIXED>(g, d, d.loc[par], i, lb, cp, d.pl, d.pcount, nullptr)
                : force_fp64<false>(g, d, qm, i, cp, d.pl, d.pcount, nullptr);
    // the w words are padding (zero in the FP64 form, packed reference
    // positions in the mixed form): never scaled, never in the kinetic energy
    double4_32a p = d.p[i];
    if (THERMO == MDG_NOSEHOOVER) {
      const double e1 = f->exp1;
      p.x *= e1; p.y *= e1; p.z *= e1;
      p.x += F.x * g.dt; p.y += F.y * g.dt; p.z += F.z * g.dt;
      p.x *= e1; p.y *= e1; p.z *= e1;
    } else {
      p.x += F.x * g.dt; p.y += F.y * g.dt; p.z += F.z * g.dt;
    }
    if (THERMO == MDG_LANGEVIN) {
      double z[3];
      langevin_normals(g.seed, (uint32_t)d.id[i], f->lang - 1ull, z);
      p.x += (-g.gamma * p.x + g.hb_d * z[0]) * g.dt;
      p.y += (-g.gamma * p.y + g.hb_d * z[1]) * g.dt;
      p.z += (-g.gamma * p.z + g.hb_d * z[2]) * g.dt;
    }
    const double4_32a q0 = qm[i];
    double4_32a qe = q0, q1;
    if (MIXED) {  // one rounding per half-drift (fused)
      if (!(THERMO == MDG_LANGEVIN && COMPAT)) {
        qe.x = fma(p.x, g.dt2, q0.x);
        qe.y = fma(p.y, g.dt2, q0.y);
        qe.z = fma(p.z, g.dt2, q0.z);
      }
      q1 = qe;
      q1.x = fma(p.x, g.dt2, qe.x);
      q1.y = fma(p.y, g.dt2, qe.y);
      q1.z = fma(p.z, g.dt2, qe.z);
    } else {  // the reference's separate product and sum
      if (!(THERMO == MDG_LANGEVIN && COMPAT)) {
        qe.x = __dadd_rn(q0.x, __dmul_rn(p.x, g.dt2));
        qe.y = __dadd_rn(q0.y, __dmul_rn(p.y, g.dt2));
        qe.z = __dadd_rn(q0.z, __dmul_rn(p.z, g.dt2));
      }
      q1 = qe;
      q1.x = __dadd_rn(qe.x, __dmul_rn(p.x, g.dt2));
      q1.y = __dadd_rn(qe.y, __dmul_rn(p.y, g.dt2));
      q1.z = __dadd_rn(qe.z, __dmul_rn(p.z, g.dt2));
    }
    float4 ln;
    if (MIXED) {
      // positions relative to the home-cell centre: the new local position is
      // one conversion, and the displacement since the build is measured in
      // float against the build's local position, packed in q_mid.w
      ln = make_float4((float)q1.x, (float)q1.y, (float)q1.z, lb.w);
      float bx, by, bz;
      unpack_ref(g, q0.w, bx, by, bz);
      const float fx = ln.x - bx, fy = ln.y - by, fz = ln.z - bz;
      // the half-margin rule, or a non-finite position (the rebuild's wrap
      // reports it) under either policy
      if ((g.rebuild_policy == MDG_REBUILD_HALFMARGIN && fx * fx + fy * fy + fz * fz > g.half_margin2_ref) ||
          !(fx == fx && fy == fy && fz == fz))
        d.flags->rebuild = 1;
    } else {
      const double4_32a qb = d.q_build[i];
      const double ux = q1.x - qb.x, uy = q1.y - qb.y, uz = q1.z - qb.z;
      // displacement since the build: in double for the rebuild test, in
      // float for the new home-cell-local position (qf holds the local
      // position at the build) and the inner-list test
      ln = make_float4(lb.x + (float)ux, lb.y + (float)uy, lb.z + (float)uz, lb.w);
      if ((g.rebuild_policy == MDG_REBUILD_HALFMARGIN && ux * ux + uy * uy + uz * uz > g.half_margin2) ||
          !(q1.x == q1.x && q1.y == q1.y && q1.z == q1.z))
        d.flags->rebuild = 1;
    }
    d.loc[par ^ 1][i] = ln;
    // prune reference: the positions of this force evaluation when the
    // inner list was re-selected now, else those of the last selection
    // (mixed: packed in p.w)
    float4 lp;
    if (prune) {
      lp = MIXED ? lb : d.loc[par][i];
      if (MIXED) p.w = pack_ref(g, lp.x, lp.y, lp.z);
      else d.loc_p[i] = lp;
      d.pcount[i] = kept;
    } else if (MIXED) {
      unpack_ref(g, p.w, lp.x, lp.y, lp.z);
    } else {
      lp = d.loc_p[i];
    }
    const float vx = ln.x - lp.x, vy = ln.y - lp.y, vz = ln.z - lp.z;
    if (vx * vx + vy * vy + vz * vz > (MIXED ? g.half_prune2_ref : g.half_prune2)) d.flags->prune_next = 1;
    d.p[i] = p;
    // the mixed form leaves q_end behind: q_mid - p dt/2 gives it back when a
    // rebuild or a reader needs it (32 bytes a particle fewer per step)
    if (!MIXED) d.q_end[i] = qe;
    qn[i] = q1;
    if (THERMO == MDG_NOSEHOOVER) ke = 0.5 * p.x * p.x + 0.5 * p.y * p.y + 0.5 * p.z * p.z;
  }
  if (MIXED && i == 0) d.flags->end_stale = 1;
  if (THERMO == MDG_NOSEHOOVER) {
    __shared__ double sh[step_threads<THERMO, MIXED, PMODE>() / 32];
    const double t = block_sum(ke, sh);
    if (threadIdx.x == 0) d.partials[blockIdx.x] = t;
  }
  if (prune) {  // inner-list size for the statistics (uniform branch)
    unsigned long long v = (unsigned long long)kept;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(&d.flags->inner_pairs, v);
  }
}

// Nose-Hoover bookkeeping after a step (mdmanager.cc:169-174) and before the
// next (mdmanager.cc:161-164): T from the block sums in fixed order.
__global__ void k_nh_update(Geom g, Dev d, int nparts, int first) {
  DevFlags *f = d.flags;
  if (f->halt != 0) return;
  __shared__ double sh[32];
  double v = 0.0;
  for (int b = threadIdx.x; b < nparts; b += blockDim.x) v += d.partials[b];
  const double ke = block_sum(v, sh);
  if (threadIdx.x == 0) {
    const double T = ke / (double)g.n / 1.5;
    const double dt2 = g.dt * 0.5;
    const double t1 = (T - g.temperature) / (g.tau * g.tau);
    const double zeta = first ? f->zeta : f->zeta_a + t1 * dt2;
    f->zeta = zeta;
    f->t_cur = T;
    f->zeta_a = zeta + t1 * dt2;
    f->exp1 = exp(-dt2 * f->zeta_a);
  }
}

__global__ void __launch_bounds__(kStepThreads) k_kinetic(Geom g, Dev d) {
  __shared__ double sh[kStepThreads / 32];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double ke = 0.0;
  if (i < g.n) {
    const double4_32a p = d.p[i];
    ke = 0.5 * p.x * p.x + 0.5 * p.y * p.y + 0.5 * p.z * p.z;
  }
  const double t = block_sum(ke, sh);
  if (threadIdx.x == 0) d.partials[blockIdx.x] = t;
}

// Observers at the step-boundary positions q_end: kinetic energy
// (observer.cc:5-15), pair energy (observer.cc:17-48) and virial
// (observer.cc:50-79), each pair evaluated with the reference's expression
// and rounding and weighted 1/2 (each pair is listed from both sides).
__global__ void __launch_bounds__(kStepThreads) k_observe(Geom g, Dev d) {
  __shared__ double sh[kStepThreads / 32];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double ke = 0.0, pe = 0.0, vir = 0.0;
  if (i < g.n) {
    const double4_32a p = d.p[i];
    ke = 0.5 * p.x * p.x + 0.5 * p.y * p.y + 0.5 * p.z * p.z;
    const double4_32a qi = d.q_end[i];
    const CellPos cp = cell_pos(g, d.cell[i]);
    const int cnt = d.ncount[i];
    for (int k = 0; k < cnt; k++) {
      const uint32_t e = d.nl[(size_t)k * g.stride + i];
      if (!MDG_IN_RANGE(d.flags, kCheckObserve, entry_slot(e), g.n)) continue;
      double4_32a qj = d.q_end[entry_slot(e)];
      if (cp.edge) apply_image(g, cp, e, qj);
      const double dx = __dsub_rn(qi.x, qj.x), dy = __dsub_rn(qi.y, qj.y), dz = __dsub_rn(qi.z, qj.z);
      const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
      if (r2 > g.rc2) continue;
      const double r4 = __dmul_rn(r2, r2), r6 = __dmul_rn(r4, r2), r8 = __dmul_rn(r6, r2), r10 = __dmul_rn(r8, r2),
                   r12 = __dmul_rn(r10, r2);
      const double e_ij = 4.0 * (1.0 / r12 - 1.0 / r6 + __dmul_rn(g.c2, r2) + g.c0);
      const double df = (__dsub_rn(__dmul_rn(24.0, r6), 48.0) / (__dmul_rn(__dmul_rn(r6, r6), r2)) + g.c2x8) * r2;
      pe += 0.5 * e_ij;
      vir += 0.5 * df;
    }
  }
  const double a = block_sum(ke, sh);
  const double b = block_sum(pe, sh);
  const double c = block_sum(vir, sh);
  if (threadIdx.x == 0) {
    d.partials[3 * blockIdx.x + 0] = a;
    d.partials[3 * blockIdx.x + 1] = b;
    d.partials[3 * blockIdx.x + 2] = c;
  }
}

// Mixed-form observers: the same sums with each pair's energy and virial
// term evaluated in float (from the home-cell-local float positions of q_end,
// as the mixed force) and summed over the row in compensated float, walked
// like the step kernel's row; the rows are added in double.  The FP64 form
// keeps k_observe's reference rounding.
template <bool EDGE>
__device__ __forceinline__ void observe_row(const Geom &g, const Dev &d, const float4 *__restrict__ loc, int i,
                                            const float4 &li, const CellPos &cp, int cnt, double &pe, double &vir) {
  const float rc2 = g.rc2f, c2 = (float)g.c2, c0 = (float)g.c0, c2x8 = g.c2x8f;
  // compensated sums: the error of each row sum stays near one float
  // rounding of the sum, whatever the row length (GB300 runs double, and
  // conversions to 64-bit types, at 1/64 of the float rate)
  float se = 0.f, ce = 0.f, sv = 0.f, cv = 0.f;
  walk_row<EDGE, kCheckObserve>(g, d, loc, i, li, cp, d.nl, cnt,
                                [&](uint32_t, float, float, float, float r2) {
    float inv;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(inv) : "f"(r2));
    const float i6 = inv * inv * inv;
    float e_ij = 4.0f * (i6 * i6 - i6 + fmaf(c2, r2, c0));
    float v_ij = ((i6 * inv) * fmaf(-48.0f, i6, 24.0f) + c2x8) * r2;
    // masked, not branched; a padding partner's inf / NaN terms drop here
    e_ij = r2 <= rc2 ? e_ij : 0.0f;
    v_ij = r2 <= rc2 ? v_ij : 0.0f;
    kahan_fma(se, ce, e_ij, 1.0f);
    kahan_fma(sv, cv, v_ij, 1.0f);
  });
  pe = 0.5 * (double)(se - ce);
  vir = 0.5 * (double)(sv - cv);
}

__global__ void __launch_bounds__(kStepThreads) k_observe_mixed(Geom g, Dev d, const float4 *__restrict__ loc) {
  __shared__ double sh[kStepThreads / 32];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double ke = 0.0, pe = 0.0, vir = 0.0;
  if (i < g.n) {
    const double4_32a p = d.p[i];
    ke = 0.5 * p.x * p.x + 0.5 * p.y * p.y + 0.5 * p.z * p.z;
    const float4 li = loc[i];
    const CellPos cp = cell_pos_packed(g, li.w);
    int cnt = d.ncount[i];
    if (!MDG_IN_RANGE(d.flags, kCheckObserve, cnt, g.list_cap + 1)) cnt = 0;
    // the linear offset for warps with no lane at the periodic boundary
    if (__all_sync(__activemask(), !cp.edge)) observe_row<false>(g, d, loc, i, li, cp, cnt, pe, vir);
    else observe_row<true>(g, d, loc, i, li, cp, cnt, pe, vir);
  }
  const double a = block_sum(ke, sh);
  const double b = block_sum(pe, sh);
  const double c = block_sum(vir, sh);
  if (threadIdx.x == 0) {
    d.partials[3 * blockIdx.x + 0] = a;
    d.partials[3 * blockIdx.x + 1] = b;
    d.partials[3 * blockIdx.x + 2] = c;
  }
}

__global__ void k_observe_final(Dev d, int nparts, double *out) {
  __shared__ double sh[32];
  double a = 0.0, b = 0.0, c = 0.0;
  for (int k = threadIdx.x; k < nparts; k += blockDim.x) {
    a += d.partials[3 * k + 0];
    b += d.partials[3 * k + 1];
    c += d.partials[3 * k + 2];
  }
  const double ta = block_sum(a, sh), tb = block_sum(b, sh), tc = block_sum(c, sh);
  if (threadIdx.x == 0) {
    out[0] = ta;
    out[1] = tb;
    out[2] = tc / 3.0;
  }
}

// Forces at q_end in the handle's precision, written in caller order to io4.
template <int MIXED>
__global__ void __launch_bounds__(kStepThreads) k_forces(Geom g, Dev d, const float4 *loc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n) return;
  const CellPos cp = cell_pos(g, d.cell[i]);
  const double3 F = MIXED ? force_mixed<false, MIXED == MDG_MIXED>(g, d, loc, i, loc[i], cp, d.nl, d.ncount, nullptr)
                          : force_fp64<false>(g, d, d.q_end, i, cp, d.nl, d.ncount, nullptr);
  d.io4[d.id[i]] = make_double4_32a(F.x, F.y, F.z, 0.0);
}

// Float positions of q_end relative to the home-cell centres (k_forces<1> input).
// In the mixed form q_mid[par] is already home-cell-local: the step-boundary
// local position is q_mid - p dt/2, with no box coordinates in between.
__global__ void k_loc_from_end(Geom g, Dev d, float4 *loc, int par) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n) return;
  int cx, cy, cz;
  cell_unkey(d.cell[i], cx, cy, cz);
  if (g.local_pos) {
    const double4_32a u = d.q_mid[par][i], p = d.p[i];
    loc[i] = make_float4((float)fma(-p.x, g.dt2, u.x), (float)fma(-p.y, g.dt2, u.y), (float)fma(-p.z, g.dt2, u.z),
                         cell_pack(cx, cy, cz));
    return;
  }
  const double4_32a q = d.q_end[i];
  loc[i] = make_float4((float)(q.x - cell_centre(g, 0, cx)), (float)(q.y - cell_centre(g, 1, cy)),
                       (float)(q.z - cell_centre(g, 2, cz)), cell_pack(cx, cy, cz));
}

// The caller's arrays in the caller's order; their fourth lane is padding
// and comes back zero (the mixed form keeps packed reference positions in it).
__global__ void k_unsort(Geom g, Dev d, double4_32a *qo, double4_32a *po) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n) return;
  const int id = d.id[i];
  if (qo) {
    double4_32a q = d.q_end[i];
    q.w = 0.0;
    qo[id] = q;
  }
  if (po) {
    double4_32a p = d.p[i];
    p.w = 0.0;
    po[id] = p;
  }
}

__global__ void k_sort_in(Geom g, Dev d, const double4_32a *qi, const double4_32a *pi) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n) return;
  double4_32a q = qi[i], p = pi[i];
  q.w = 0.0;
  p.w = 0.0;
  d.q_end[i] = q;
  d.p[i] = p;
  d.id[i] = i;
  d.inv[i] = i;
}

__global__ void k_pairs(Geom g, Dev d, const long long *row_off, int32_t *rec) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n) return;
  const CellPos cp = cell_pos(g, d.cell[i]);
  const int cnt = d.ncount[i];
  long long o = row_off[i];
  for (int k = 0; k < cnt; k++) {
    const uint32_t e = d.nl[(size_t)k * g.stride + i];
    const int j = (int)entry_slot(e);
    const int ox = entry_sx(e), oy = entry_sy(e), oz = entry_sz(e);
    const int sx = (ox == 0 && cp.cx == 0) ? -1 : ((ox == 2 && cp.cx == g.nc[0] - 1) ? 1 : 0);
    const int sy = (oy == 0 && cp.cy == 0) ? -1 : ((oy == 2 && cp.cy == g.nc[1] - 1) ? 1 : 0);
    const int sz = (oz == 0 && cp.cz == 0) ? -1 : ((oz == 2 && cp.cz == g.nc[2] - 1) ? 1 : 0);
    rec[3 * (o + k) + 0] = d.id[i];
    rec[3 * (o + k) + 1] = d.id[j];
    rec[3 * (o + k) + 2] = (sx + 1) + 3 * (sy + 1) + 9 * (sz + 1);
  }
}

inline int blocks_for(int n) { return n > 0 ? (n + kStepThreads - 1) / kStepThreads : 1; }

}  // namespace

template <int T, int C, int M>
void launch_step_variant(const Geom &g, const Dev &d, int par, int pmode, cudaStream_t s) {
  constexpr int t0 = step_threads<T, M, 0>(), t1 = step_threads<T, M, 1>(), t2 = step_threads<T, M, 2>();
  auto grid = [&](int threads) { return g.n > 0 ? (g.n + threads - 1) / threads : 1; };
  if (pmode == 0) k_step<T, C, M, 0><<<grid(t0), t0, 0, s>>>(g, d, par);
  if (pmode == 1 || pmode == 3) k_step<T, C, M, 1><<<grid(t1), t1, 0, s>>>(g, d, par);
  if (pmode == 2 || pmode == 3) k_step<T, C, M, 2><<<grid(t2), t2, 0, s>>>(g, d, par);
  // the Nose-Hoover block sums of this step: one per block of the variant that ran
  static_assert(T != MDG_NOSEHOOVER || (t0 == t1 && t1 == t2), "one partial-sum count for every variant");
  if (T == MDG_NOSEHOOVER) k_nh_update<<<1, 1024, 0, s>>>(g, d, grid(t1), 0);
}

template <int T, int C>
void launch_step_precision(const Geom &g, const Dev &d, int par, int precision, int pmode, cudaStream_t s) {
  if (precision == MDG_MIXED) launch_step_variant<T, C, MDG_MIXED>(g, d, par, pmode, s);
  else if (precision == MDG_MIXED_PLAIN) launch_step_variant<T, C, MDG_MIXED_PLAIN>(g, d, par, pmode, s);
  else launch_step_variant<T, C, MDG_FP64>(g, d, par, pmode, s);
}

// pmode: 0 one kernel deciding on the device; 1 / 2 only the ordinary / the
// re-selecting variant (graph conditional bodies); 3 both variants in turn.
// mixed: the handle's mdg_precision.
void launch_step(const Geom &g, const Dev &d, int par, int thermostat, int compat, int mixed, cudaStream_t s,
                 int pmode) {
  if (thermostat == MDG_LANGEVIN) {
    if (compat) launch_step_precision<MDG_LANGEVIN, 1>(g, d, par, mixed, pmode, s);
    else launch_step_precision<MDG_LANGEVIN, 0>(g, d, par, mixed, pmode, s);
  } else if (thermostat == MDG_NOSEHOOVER) {
    launch_step_precision<MDG_NOSEHOOVER, 0>(g, d, par, mixed, pmode, s);
  } else {
    launch_step_precision<MDG_NVE, 0>(g, d, par, mixed, pmode, s);
  }
}

void launch_nh_init(const Geom &g, const Dev &d, cudaStream_t s) {
  const int grid = blocks_for(g.n);
  k_kinetic<<<grid, kStepThreads, 0, s>>>(g, d);
  k_nh_update<<<1, 1024, 0, s>>>(g, d, grid, 1);
}

void launch_observe(const Geom &g, const Dev &d, double *out_dev, cudaStream_t s, int mixed, int par) {
  const int grid = blocks_for(g.n);
  if (mixed) {
    // the buffer the next step overwrites before reading it
    k_loc_from_end<<<grid, kStepThreads, 0, s>>>(g, d, d.loc[par ^ 1], par);
    k_observe_mixed<<<grid, kStepThreads, 0, s>>>(g, d, d.loc[par ^ 1]);
  } else {
    k_observe<<<grid, kStepThreads, 0, s>>>(g, d);
  }
  k_observe_final<<<1, 1024, 0, s>>>(d, grid, out_dev);
}

void launch_forces(const Geom &g, const Dev &d, int mixed, int par, cudaStream_t s) {
  const int grid = blocks_for(g.n);
  if (mixed) {
    // the buffer the next step overwrites before reading it
    k_loc_from_end<<<grid, kStepThreads, 0, s>>>(g, d, d.loc[par ^ 1], par);
    if (mixed == MDG_MIXED_PLAIN) k_forces<MDG_MIXED_PLAIN><<<grid, kStepThreads, 0, s>>>(g, d, d.loc[par ^ 1]);
    else k_forces<MDG_MIXED><<<grid, kStepThreads, 0, s>>>(g, d, d.loc[par ^ 1]);
  } else {
    k_forces<0><<<grid, kStepThreads, 0, s>>>(g, d, nullptr);
  }
}

void launch_unsort(const Geom &g, const Dev &d, int par, double4_32a *qo, double4_32a *po, cudaStream_t s) {
  if (g.local_pos) launch_end_from_mid(g, d, par, s);
  k_unsort<<<blocks_for(g.n), kStepThreads, 0, s>>>(g, d, qo, po);
}

void launch_sort_in(const Geom &g, const Dev &d, const double4_32a *qi, const double4_32a *pi, cudaStream_t s) {
  k_sort_in<<<blocks_for(g.n), kStepThreads, 0, s>>>(g, d, qi, pi);
}

void launch_pairs(const Geom &g, const Dev &d, const long long *row_off, int32_t *rec, cudaStream_t s) {
  k_pairs<<<blocks_for(g.n), kStepThreads, 0, s>>>(g, d, row_off, rec);
}

}  // namespace mdg
