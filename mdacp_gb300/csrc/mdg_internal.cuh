// Internal declarations shared by the mdg CUDA translation units.
//
// Device data layout (one box, n particles, slots sorted by cell):
//   q_end[n]   double4_32a  positions at the step boundary (the reference's q);
//                       in the mixed form only current after a rebuild or
//                       launch_end_from_mid (flags->end_stale says which)
//   q_mid[2][n] double4_32a positions after the first half-drift; the step kernel
//                       reads one buffer and writes the other.  Mixed form:
//                       relative to the centre of the slot's home cell
//   p[n]       double4_32a  momenta (= velocities, m = 1)
//   q_build[n] double4_32a  positions at the last list build (the FP64 form's
//                       displacement check; the mixed form tests against qf)
//   id[n]      int      caller's particle index of each slot; inv[id] = slot
//   cell[n]    int      home cell of each slot at the last build
//   nl[cap*n]  uint32   neighbour list, ELL layout: entry k of slot i at k*stride+i
//                       bits 0..5 stencil step (ox+1) | (oy+1)<<2 | (oz+1)<<4,
//                       bits 6..31 partner slot
//   ncount[n]  int      entries in row i
//   loc[n]     float4   (mixed form) position relative to the home-cell centre
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/mdg.h"

namespace mdg {

// 32-byte read-only load of a double4_32a as two 16-byte non-coherent loads.
__device__ __forceinline__ double4_32a ldg4(const double4_32a *p) {
  const double2 a = __ldg(reinterpret_cast<const double2 *>(p));
  const double2 b = __ldg(reinterpret_cast<const double2 *>(p) + 1);
  return make_double4_32a(a.x, a.y, b.x, b.y);
}

constexpr int kJBits = 26;     // partner-slot bits of a list entry
constexpr int kCodeBits = 6;   // stencil-step bits below them
constexpr int kMaxParticles = 1 << kJBits;

// List entry of partner slot j reached through stencil step (ox, oy, oz), each -1..1.
__device__ __forceinline__ uint32_t entry_pack(int j, int ox, int oy, int oz) {
  return ((uint32_t)j << kCodeBits) | (uint32_t)((ox + 1) | ((oy + 1) << 2) | ((oz + 1) << 4));
}
__device__ __forceinline__ int entry_slot(uint32_t e) { return (int)(e >> kCodeBits); }
// stencil step + 1 (0, 1, 2) per axis
__device__ __forceinline__ int entry_sx(uint32_t e) { return (int)(e & 3u); }
__device__ __forceinline__ int entry_sy(uint32_t e) { return (int)((e >> 2) & 3u); }
__device__ __forceinline__ int entry_sz(uint32_t e) { return (int)((e >> 4) & 3u); }

// halt codes
constexpr int kHaltOverflow = 1;
constexpr int kHaltBadState = 2;
constexpr int kHaltCheck = 3;  // checked builds: a bounds check failed
constexpr int kHaltTooFast = 4;  // reference rebuild policy: 2 max|p| dt above the margin

struct DevFlags {
  int rebuild;                  // rebuild the list at the start of the next step
  int halt;                     // nonzero: an error stopped the run; kernels are no-ops
  int overflow_max;             // largest row requested when a row overflowed
  int max_count;                // largest row at the last build
  unsigned long long steps;     // steps begun since the state was set
  unsigned long long lang;      // Langevin stream position (applications begun)
  unsigned long long rebuilds;  // completed list builds
  unsigned long long pairs;     // directed pairs at the last build
  int bad_slot;
  int check_site;               // checked builds: which bounds check failed
  double zeta;                  // Nose-Hoover zeta (Variables::Zeta) after the last step
  double zeta_a;                // zeta after the first update of the coming step
  double exp1;                  // exp(-dt/2 * zeta_a)
  double t_cur;                 // temperature of the current momenta
  int prune_now;                // this step's kernel re-selects the inner list (set by the prelude)
  int prune_next;               // a particle left its prune buffer: re-select at the next step
  unsigned long long prunes;    // completed prunes
  unsigned long long inner_pairs;  // directed pairs in the inner list at the last prune
  int end_stale;                // mixed form: q_end is behind the steps (rebuilt from q_mid and p on demand)
  // reference rebuild policy (PairList, pairlist.cc:26-121)
  double buffer_length;         // what is left of the margin's budget since the build
  double c_d2;                  // candidate threshold of the displacement check
  unsigned long long lifetime;  // steps since the build
  unsigned long long checks;    // displacement checks run
  int need_check;               // this step runs the displacement check
  int cand_count;               // candidate entries (particles and their images) found by it
  int cand_slots;               // candidate particles recorded
  int entries;                  // particles and their images (the reference's local + ghost count)
  double vmax;                  // max |p| at the last policy evaluation
};

struct Geom {
  double L[3];
  double w[3];        // cell widths
  double inv_w[3];
  int nc[3];
  int ncell;
  int nt[3];          // cell tiles per side (rounded up)
  int nrank;          // tiles * cells per tile: length of the cell counters and starts
  int n;              // particles
  int stride;         // ELL row stride (allocated particle capacity)
  int list_cap;       // entries per row
  double sl2, rc2;    // (rc+margin)^2, rc^2
  float acc_lo, acc_hi;  // float r2 below acc_lo: inside SL; above acc_hi: outside; between: exact test
  float rc2f;
  double c0, c2, c2x8;
  double dt, dt2;
  double half_margin2;
  // thermostats
  double gamma, temperature, tau, hb_d;  // hb_d = sqrt(2 gamma T / dt)
  uint64_t seed;
  // mixed form
  float w32[3];       // cell widths rounded to float
  float dl32[3];      // L - nc * w32
  float c2x8f;
  // inner (pruned) list: pairs within rc + prune_buffer at the last prune
  float prune_thr2;   // (rc + buffer)^2 + float slack
  float half_prune2;  // (buffer / 2)^2, displacement that forces a re-prune
  // mixed form: q_mid holds positions relative to the centre of the slot's
  // home cell at the last build, and the step kernels do not write q_end
  int local_pos;
  // mixed form: the build and prune reference positions (home-cell-local)
  // travel in the padding words q_mid.w and p.w as 21-bit fixed point per
  // axis, ref_unit = w / (2^20 - 1) apart (|position| < w holds for both);
  // the displacement tests compare against thresholds lowered by twice the
  // largest rounding of a packed position
  float ref_scale[3], ref_unit[3];
  float half_margin2_ref, half_prune2_ref;
  // rebuild policy (mdg_rebuild_policy); the reference policy's margin and
  // candidate limit min(CheckListLength, n)
  int rebuild_policy, check_list;
  double margin, sl;  // margin, search length rc + margin
};

// Home-cell-local position (|x| < w per axis) packed into the bits of a
// double: 21-bit two's complement fields at bits 0, 21, 42.  The value is
// only ever moved, never used in arithmetic.
__device__ __forceinline__ double pack_ref(const Geom &g, float x, float y, float z) {
  const long long a = (long long)__float2int_rn(x * g.ref_scale[0]) & 0x1FFFFF;
  const long long b = (long long)__float2int_rn(y * g.ref_scale[1]) & 0x1FFFFF;
  const long long c = (long long)__float2int_rn(z * g.ref_scale[2]) & 0x1FFFFF;
  return __longlong_as_double(a | (b << 21) | (c << 42));
}

__device__ __forceinline__ void unpack_ref(const Geom &g, double v, float &x, float &y, float &z) {
  const long long u = __double_as_longlong(v);
  x = (float)(int)((u << 43) >> 43) * g.ref_unit[0];
  y = (float)(int)((u << 22) >> 43) * g.ref_unit[1];
  z = (float)(int)((u << 1) >> 43) * g.ref_unit[2];
}

// Centre of home cell (cx, cy, cz) in double, exact: (c + 1/2) w32 has at
// most 36 significant bits.
__host__ __device__ __forceinline__ double cell_centre(const Geom &g, int k, int c) {
  return ((double)c + 0.5) * (double)g.w32[k];
}

struct Dev {
  double4_32a *q_end, *q_mid[2], *p, *q_build;
  double4_32a *t_q, *t_p;   // reorder staging
  float4 *qf;           // float copy of wrapped q_end (list prefilter)
  float4 *loc[2];       // mixed-form local positions at q_mid[0] / q_mid[1]
  int *id, *inv, *cell, *t_id, *t_cell, *order;
  int *cell_count, *cell_fill, *cell_start, *block_sums;
  uint32_t *nl;
  int *ncount;
  uint32_t *pl;         // inner list, same layout and capacity as nl
  int *pcount;
  float4 *loc_p;        // home-cell-local position at the last prune
  double *partials;     // reduction scratch
  int nblocks_red;
  double *vpart;        // reference rebuild policy: per-block maxima
  int *cand;            // reference rebuild policy: the check's candidate particles, then their entry masks
  DevFlags *flags;
  double4_32a *io4;         // caller-order staging for get/set/forces
  double4_32a *io4b;
};

// kernels enqueued by one launch_rebuild and one launch_step call
constexpr int kRebuildKernels = 11;
inline int step_kernels(int thermostat) { return thermostat == MDG_NOSEHOOVER ? 2 : 1; }

// host-side launchers (stream-ordered; none synchronises)
// count_step: the first kernel also starts a step (counters, inner-list
// hand-over); in_step: the rebuild belongs to the step about to run.
void launch_rebuild(const Geom &g, const Dev &d, int q_mid_dst, int num_sms, cudaStream_t s, bool count_step,
                    bool lang_step, bool in_step);
void launch_step(const Geom &g, const Dev &d, int par, int thermostat, int compat, int mixed, cudaStream_t s,
                 int pmode);
// Graph path: step start (counters, hand-over) and the conditions of the
// step's nodes.  Split form (timed graphs): the rebuild condition (IF) and
// the step variant (SWITCH: 0 ordinary, 1 re-selecting, 2 none when halted).
// One-node form: SWITCH 0 ordinary, 1 re-selecting, 2 rebuild then
// re-selecting, 3 none.
void launch_prelude_split(const Dev &d, int lang_step, cudaGraphConditionalHandle rebuild_cond,
                          cudaGraphConditionalHandle variant_cond, cudaStream_t s);
void launch_prelude(const Dev &d, int lang_step, cudaGraphConditionalHandle step_cond, cudaStream_t s);
void launch_nh_init(const Geom &g, const Dev &d, cudaStream_t s);
// Reference rebuild policy at the start of a step that reads q_mid[par]: the
// budget (2 kernels; with a graph handle it sets the check's IF condition)
// and the displacement check (4 kernels, no-ops unless the budget is spent).
constexpr int kPolicyKernels = 2, kPolicyCheckKernels = 4;
void launch_policy(const Geom &g, const Dev &d, cudaStream_t s, cudaGraphConditionalHandle check_cond, int use_cond);
void launch_policy_check(const Geom &g, const Dev &d, int par, cudaStream_t s);
void launch_observe(const Geom &g, const Dev &d, double *out_dev, cudaStream_t s, int mixed, int par);
void launch_forces(const Geom &g, const Dev &d, int mixed, int par, cudaStream_t s);
void launch_unsort(const Geom &g, const Dev &d, int par, double4_32a *qo, double4_32a *po, cudaStream_t s);
void launch_sort_in(const Geom &g, const Dev &d, const double4_32a *qi, const double4_32a *pi, cudaStream_t s);
void launch_pairs(const Geom &g, const Dev &d, const long long *row_off, int32_t *rec, cudaStream_t s);
void launch_set_rebuild(const Dev &d, cudaStream_t s);
// Mixed form: brings q_end up to date from q_mid[par] and p when the steps
// left it behind (two kernels; a no-op when it is current).
void launch_end_from_mid(const Geom &g, const Dev &d, int par, cudaStream_t s);

// Home-cell coordinates of a slot packed in one word: bits 0-10 x, 11-21 y,
// 22-31 z.  `cell[]` holds this key; the w word of the float4 positions (qf,
// loc) holds the same bits, so the step kernel gets them with the position it
// loads anyway.
constexpr int kCellXBits = 11, kCellYBits = 11, kCellZBits = 10;
__device__ __forceinline__ int cell_key(int cx, int cy, int cz) {
  return (int)((uint32_t)cx | ((uint32_t)cy << kCellXBits) | ((uint32_t)cz << (kCellXBits + kCellYBits)));
}
__device__ __forceinline__ float cell_pack(int cx, int cy, int cz) { return __int_as_float(cell_key(cx, cy, cz)); }
__device__ __forceinline__ void cell_unkey(int key, int &cx, int &cy, int &cz) {
  const uint32_t v = (uint32_t)key;
  cx = (int)(v & ((1u << kCellXBits) - 1u));
  cy = (int)((v >> kCellXBits) & ((1u << kCellYBits) - 1u));
  cz = (int)(v >> (kCellXBits + kCellYBits));
}
__device__ __forceinline__ void cell_unpack(float w, int &cx, int &cy, int &cz) { cell_unkey(__float_as_int(w), cx, cy, cz); }

// Storage rank of a cell: cells grouped in tiles of 2^kTileShift cells per
// side, tiles in x-fastest order, cells x-fastest inside a tile (kTileShift 0
// is the plain x-fastest order).  Slots follow this order.
#ifndef MDG_TILE_SHIFT
#define MDG_TILE_SHIFT 0
#endif
constexpr int kTileShift = MDG_TILE_SHIFT;
constexpr int kTileMask = (1 << kTileShift) - 1;
__host__ __device__ __forceinline__ int cell_rank(const Geom &g, int cx, int cy, int cz) {
  const int t = ((cz >> kTileShift) * g.nt[1] + (cy >> kTileShift)) * g.nt[0] + (cx >> kTileShift);
  return (t << (3 * kTileShift)) | ((cz & kTileMask) << (2 * kTileShift)) | ((cy & kTileMask) << kTileShift) |
         (cx & kTileMask);
}

// Mixed-form partner offset.  Per axis, the offset between the home cells of
// i and j minus i's own local coordinate is a quadratic in the stencil step
// t = -1, 0, 1: v(t) = c + a t + b t^2 with c = -l_i,
// a = (off(1) - off(-1)) / 2, b = (off(1) + off(-1)) / 2 (b = 0 away from the
// periodic boundary).  t comes out of the entry's low bits as a float without
// a conversion: OR-ing a small integer m into the mantissa of 2^23 gives the
// float 2^23 + m exactly; the y and z fields sit 2 and 4 bits up, so they
// decode to 4t and 16t and their coefficients carry 1/4 and 1/16 per power.
struct AxisQuad {
  float a, b, c;
};

__device__ __forceinline__ AxisQuad axis_quad(float w, float dl, bool lo, bool hi, float li, float scale) {
  const float m = -w - (lo ? dl : 0.0f), p = w + (hi ? dl : 0.0f);
  AxisQuad q;
  q.a = 0.5f * (p - m) * scale;
  q.b = 0.5f * (p + m) * (scale * scale);
  q.c = -li;
  return q;
}

__device__ __forceinline__ float step_float(uint32_t e, uint32_t mask, float bias) {
  return __int_as_float((int)((e & mask) | 0x4B000000u)) - bias;
}

// Compensated float accumulation (Kahan) of a * b into s: c carries the low
// part each addition lost (with the opposite sign), so the sum is s - c.  The
// product is fused into the first subtraction.
__device__ __forceinline__ void kahan_fma(float &s, float &c, float a, float b) {
  const float y = fmaf(a, b, -c);
  const float t = s + y;
  c = (t - s) - y;
  s = t;
}

// device helpers
__device__ __forceinline__ void halt_with(DevFlags *f, int code) { atomicCAS(&f->halt, 0, code); }

// Checked builds (-DMDG_CHECK=1, libmdg_check.so): index checks on the
// gathers and scatters of the single-box path.  A failed check stops the run
// like any other halt (every later kernel is a no-op), records the site and
// the index, and the access is skipped; nothing traps.  Sites:
enum CheckSite {
  kCheckStepSlot = 1,    // step / force: list entry slot >= n
  kCheckStepRow = 2,     // step / force: row length > list capacity
  kCheckBuildCell = 3,   // list build: stencil cell rank >= cell count
  kCheckBuildRange = 4,  // list build: a cell's slot range outside 0..n
  kCheckScatter = 5,     // binning: destination slot >= n
  kCheckObserve = 6,     // observers: list entry slot >= n
};
#ifndef MDG_CHECK
#define MDG_CHECK 0
#endif
constexpr bool kCheck = MDG_CHECK != 0;

__device__ __noinline__ inline bool check_failed(DevFlags *f, int site, long long index) {
  if (atomicCAS(&f->halt, 0, kHaltCheck) == 0) {
    f->check_site = site;
    f->bad_slot = index > 0x7fffffffLL ? 0x7fffffff : (int)index;
  }
  return false;
}
// true when 0 <= v < n (always in unchecked builds)
#define MDG_IN_RANGE(flags, site, v, n) \
  (!mdg::kCheck || (unsigned long long)(long long)(v) < (unsigned long long)(long long)(n) || \
   mdg::check_failed((flags), (site), (long long)(v)))

}  // namespace mdg
