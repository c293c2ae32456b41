// C ABI of libmdg.so (include/mdg.h): handle life cycle, state exchange and
// the step sequencing that stands in for MDManager::Calculate.
//
// A step is enqueued as the rebuild sequence (a no-op unless the device flag
// says the list expired) followed by the fused step kernel.  Steps are
// replayed from CUDA graphs captured for both parities of the double-buffered
// mid-step positions.  The host synchronises once per mdg_calculate call and
// reads the device flags: a neighbour row that overflowed stops the remaining
// kernels of the call at the step where it happened (they become no-ops), the
// list is regrown and the run continues from that step.
#include <cuda_runtime.h>

#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mdg.h"
#include "mdg_internal.cuh"

using mdg::DevFlags;

struct mdg_handle {
  mdg_params prm;
  std::string err;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  mdg::Geom g;
  mdg::Dev d;
  DevFlags *hflags = nullptr;  // pinned mirror
  double *hobs = nullptr, *dobs = nullptr;
  int cap = 0;
  bool has_state = false;
  bool nh_init = true;
  int par = 0;
  cudaGraphExec_t gx_pair[2] = {nullptr, nullptr};
  cudaGraphExec_t gx_one[2] = {nullptr, nullptr};
  int graph_n = -1;  // particle count the graphs were captured for
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double last_ms = 0.0;
  long long steps_host = 0;  // completed steps as last read from the device
  long long launches = 0;    // kernels enqueued (counting every node of a graph replay)
  long long pending = 0;     // steps enqueued by mdg_calculate and not yet confirmed
  bool ev1_due = false;      // the timing end event is recorded when the steps are confirmed
};

// Steps mdg_calculate may leave enqueued before it waits for them.
constexpr long long kMaxPending = 1024;

namespace {

const char *kVersion = "mdg 0.1 (sm_103a)";

int fail(mdg_handle *h, int code, const std::string &msg) {
  if (h) h->err = msg;
  return code;
}

// Why the calling thread's last mdg_create failed (mdg_last_error(NULL)).
thread_local std::string t_create_err;

int create_fail(int code, const std::string &msg) {
  t_create_err = msg;
  return code;
}

#define MDG_CK(call)                                                                                  \
  do {                                                                                                \
    cudaError_t e_ = (call);                                                                          \
    if (e_ != cudaSuccess)                                                                            \
      return fail(h, MDG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));               \
  } while (0)

void drop_graphs(mdg_handle *h) {
  for (int k = 0; k < 2; k++) {
    if (h->gx_pair[k]) cudaGraphExecDestroy(h->gx_pair[k]);
    if (h->gx_one[k]) cudaGraphExecDestroy(h->gx_one[k]);
    h->gx_pair[k] = h->gx_one[k] = nullptr;
  }
  h->graph_n = -1;
}

template <class T>
cudaError_t dalloc(T **p, size_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  return cudaMalloc((void **)p, count * sizeof(T));
}

void dfree_all(mdg_handle *h) {
  mdg::Dev &d = h->d;
  void *ptrs[] = {d.q_end, d.q_mid[0], d.q_mid[1], d.p, d.q_build, d.t_q, d.t_p, d.qf, d.loc[0], d.loc[1], d.id,
                  d.inv, d.cell, d.t_id, d.t_cell, d.order, d.cell_count, d.cell_fill, d.cell_start, d.block_sums,
                  d.nl, d.ncount, d.pl, d.pcount, d.loc_p, d.partials, d.vpart, d.cand, d.flags, d.io4, d.io4b,
                  h->dobs};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  memset(&h->d, 0, sizeof(h->d));
  h->dobs = nullptr;
}

int lang_on(const mdg_handle *h) { return h->prm.thermostat == MDG_LANGEVIN; }

// Sets the pieces of Geom that depend on the parameters (not on n).
int setup_geometry(mdg_handle *h) {
  mdg::Geom &g = h->g;
  const mdg_params &p = h->prm;
  const double sl = p.cutoff + p.margin;
  long long ncell = 1;
  for (int k = 0; k < 3; k++) {
    g.L[k] = p.box[k];
    // bounded before the conversion: the cell coordinates have 11 or 10 bits
    const double ratio = p.box[k] / sl;
    if (!std::isfinite(p.box[k]) || !(ratio < (double)(1 << mdg::kCellXBits)))
      return fail(h, MDG_ERR_INVALID, "more than 2047 x 2047 x 1023 cells along the box sides");
    int nc = (int)ratio;
    // every pair within sl must lie in neighbouring cells even after rounding
    while (nc > 0 && p.box[k] / (double)nc < sl * (1.0 + 1e-12)) nc--;
    if (nc < 2 || p.box[k] <= 2.0 * sl)
      return fail(h, MDG_ERR_INVALID, "box side must exceed twice the search length cutoff+margin");
    g.nc[k] = nc;
    g.w[k] = p.box[k] / (double)nc;
    g.inv_w[k] = 1.0 / g.w[k];
    g.w32[k] = (float)g.w[k];
    g.dl32[k] = (float)(p.box[k] - (double)nc * (double)g.w32[k]);
    ncell *= nc;
  }
  long long nrank = 1LL << (3 * mdg::kTileShift);
  for (int k = 0; k < 3; k++) {
    g.nt[k] = (g.nc[k] + mdg::kTileMask) >> mdg::kTileShift;
    nrank *= g.nt[k];
  }
  if (ncell > 4096LL * 4096LL || nrank > 4096LL * 4096LL) return fail(h, MDG_ERR_INVALID, "too many cells");
  g.nrank = (int)nrank;
  if (g.nc[0] >= (1 << mdg::kCellXBits) || g.nc[1] >= (1 << mdg::kCellYBits) || g.nc[2] >= (1 << mdg::kCellZBits))
    return fail(h, MDG_ERR_INVALID, "more than 2047 x 2047 x 1023 cells along the box sides");
  g.ncell = (int)ncell;
  g.sl2 = sl * sl;
  g.rc2 = p.cutoff * p.cutoff;
  // Float r2 of home-cell-local positions is within ~1e-5 of the exact value
  // (|local| <= w/2, three roundings per component); a 1e-4 band around SL^2
  // goes to the exact double test.
  g.acc_lo = (float)(sl * sl - 1e-4);
  g.acc_hi = (float)(sl * sl + 1e-4);
  g.rc2f = (float)g.rc2;
  // Variables::Variables (variables.cc:16-28)
  const double s2 = 1.0 / (p.cutoff * p.cutoff);
  const double s6 = s2 * s2 * s2, s8 = s6 * s2, s12 = s6 * s6, s14 = s12 * s2;
  g.c2 = 6.0 * s14 - 3.0 * s8;
  g.c0 = -s12 + s6 - g.c2 / s2;
  g.c2x8 = g.c2 * 8.0;
  g.c2x8f = (float)g.c2x8;
  g.dt = p.dt;
  g.dt2 = p.dt * 0.5;
  g.half_margin2 = 0.25 * p.margin * p.margin;
  // negative: automatic, 0.1 capped by half the margin.  Measured best at both
  // dt = 0.001 (4M atoms NVE) and dt = 0.005 (16.4M atoms Langevin: 3.70 ms
  // per step against 3.98 with a buffer of the whole margin)
  const double buffer = p.prune_buffer < 0.0 ? std::fmin(0.1, 0.5 * p.margin) : p.prune_buffer;
  if (buffer > 0.0) {
    const double rb = p.cutoff + buffer;
    g.prune_thr2 = (float)(rb * rb + 1e-4);  // float r2 of local positions is within ~1e-5
    g.half_prune2 = (float)(0.25 * buffer * buffer * (1.0 - 1e-4));
  } else {
    g.prune_thr2 = 3.0e38f;   // keep every listed pair, select only after a rebuild
    g.half_prune2 = 3.0e38f;
  }
  g.gamma = p.gamma;
  g.temperature = p.temperature;
  g.tau = p.tau;
  g.hb_d = std::sqrt(2.0 * p.gamma * p.temperature / p.dt);
  g.seed = p.seed;
  g.local_pos = p.precision != MDG_FP64 ? 1 : 0;
  g.rebuild_policy = p.rebuild_policy;
  g.check_list = p.check_list_length;
  g.margin = p.margin;
  g.sl = p.cutoff + p.margin;
  // packed reference positions of the mixed form: a packed coordinate is off
  // by at most half a unit plus float rounding, so each displacement
  // threshold is lowered by two units (about 6e-6 at w = 3)
  double unit_max = 0.0;
  for (int k = 0; k < 3; k++) {
    g.ref_scale[k] = (float)(1048575.0 / (double)g.w32[k]);
    g.ref_unit[k] = (float)((double)g.w32[k] / 1048575.0);
    unit_max = std::fmax(unit_max, (double)g.ref_unit[k]);
  }
  const double hm = 0.5 * p.margin - 2.0 * unit_max;
  g.half_margin2_ref = (float)(hm > 0.0 ? hm * hm : 0.0);
  if (buffer > 0.0) {
    const double hp = 0.5 * buffer - 2.0 * unit_max;
    g.half_prune2_ref = (float)(hp > 0.0 ? hp * hp * (1.0 - 1e-4) : 0.0);
  } else {
    g.half_prune2_ref = 3.0e38f;
  }
  return MDG_OK;
}

int estimate_list_cap(const mdg_handle *h, int n) {
  const mdg_params &p = h->prm;
  const double sl = p.cutoff + p.margin;
  const double rho = (double)n / (p.box[0] * p.box[1] * p.box[2]);
  double est = rho * 4.18879020478639 * sl * sl * sl;
  int cap = (int)(est * 1.5 + 24.0);
  return (cap + 7) & ~7;
}

int alloc_list(mdg_handle *h, int list_cap) {
  if (h->d.nl) cudaFree(h->d.nl);
  if (h->d.pl) cudaFree(h->d.pl);
  h->d.nl = h->d.pl = nullptr;
  MDG_CK(dalloc(&h->d.nl, (size_t)list_cap * (size_t)h->cap));
  MDG_CK(dalloc(&h->d.pl, (size_t)list_cap * (size_t)h->cap));
  h->g.list_cap = list_cap;
  drop_graphs(h);
  return MDG_OK;
}

int read_flags(mdg_handle *h) {
  MDG_CK(cudaMemcpyAsync(h->hflags, h->d.flags, sizeof(DevFlags), cudaMemcpyDeviceToHost, h->stream));
  MDG_CK(cudaStreamSynchronize(h->stream));
  return MDG_OK;
}

// After a halt on overflow: undo the counters of the step that did not run,
// regrow the rows and clear the halt (the rebuild request stays set).
int recover_overflow(mdg_handle *h, bool in_step) {
  DevFlags f = *h->hflags;
  if (in_step) {
    f.steps -= 1;
    if (lang_on(h)) f.lang -= 1;
  }
  int need = f.overflow_max;
  int cap = (int)(need * 1.25) + 8;
  cap = (cap + 7) & ~7;
  if (cap <= h->g.list_cap) cap = h->g.list_cap + 8;
  f.halt = 0;
  f.overflow_max = 0;
  f.rebuild = 1;
  MDG_CK(cudaMemcpyAsync(h->d.flags, &f, sizeof(DevFlags), cudaMemcpyHostToDevice, h->stream));
  MDG_CK(cudaStreamSynchronize(h->stream));
  return alloc_list(h, cap);
}

// A bad coordinate stops the run inside the binning kernel, possibly with
// partial cell counts; they are cleared here and the halt stays set (every
// kernel is a no-op) until the next mdg_set_state.
int halt_error(mdg_handle *h) {
  cudaMemsetAsync(h->d.cell_count, 0, (size_t)h->g.nrank * sizeof(int), h->stream);
  cudaMemsetAsync(h->d.cell_fill, 0, (size_t)h->g.nrank * sizeof(int), h->stream);
  cudaStreamSynchronize(h->stream);
  char buf[160];
  if (h->hflags->halt == mdg::kHaltTooFast) {
    snprintf(buf, sizeof buf,
             "too fast particles: 2 max|p| dt = %g exceeds the margin %g (PairList::IsPairListExpired); try a "
             "smaller time step",
             2.0 * h->hflags->vmax * h->prm.dt, h->prm.margin);
    return fail(h, MDG_ERR_STATE, buf);
  }
  if (h->hflags->halt == mdg::kHaltCheck) {
    snprintf(buf, sizeof buf, "bounds check failed (site %d, index %d)", h->hflags->check_site,
             h->hflags->bad_slot);
    return fail(h, MDG_ERR_STATE, buf);
  }
  snprintf(buf, sizeof buf, "particle coordinate non-finite or outside the box at a rebuild (slot %d)",
           h->hflags->bad_slot);
  return fail(h, MDG_ERR_STATE, buf);
}

// Builds the list now if it is due (always when force is set).
int ensure_list(mdg_handle *h, bool force) {
  for (int attempt = 0; attempt < 16; attempt++) {
    if (force) mdg::launch_set_rebuild(h->d, h->stream);
    mdg::launch_rebuild(h->g, h->d, h->par, h->num_sms, h->stream, false, false, false);
    h->launches += mdg::kRebuildKernels + (force ? 1 : 0);
    int rc = read_flags(h);
    if (rc) return rc;
    if (h->hflags->halt == 0) return MDG_OK;
    if (h->hflags->halt != mdg::kHaltOverflow) return halt_error(h);
    rc = recover_overflow(h, false);
    if (rc) return rc;
    force = true;
  }
  return fail(h, MDG_ERR_CAPACITY, "neighbour list could not be sized");
}

int kernels_per_step(const mdg_handle *h) {
  const int policy = h->g.rebuild_policy == MDG_REBUILD_REFERENCE ? mdg::kPolicyKernels + mdg::kPolicyCheckKernels : 0;
  return policy + mdg::kRebuildKernels + mdg::step_kernels(h->prm.thermostat);
}

// Kernels the step graphs executed for `completed` steps with `rebuilds`
// rebuild bodies and `checks` displacement-check bodies: prelude, step
// (+ NH), the reference policy's budget kernels.
long long graph_kernels(const mdg_handle *h, long long completed, long long rebuilds, long long checks) {
  const bool ref = h->g.rebuild_policy == MDG_REBUILD_REFERENCE;
  return completed * (1 + mdg::step_kernels(h->prm.thermostat) + (ref ? mdg::kPolicyKernels : 0)) +
         rebuilds * mdg::kRebuildKernels + checks * mdg::kPolicyCheckKernels;
}

// One step as plain launches: the rebuild sequence (no-ops unless due) and
// the step kernel deciding its variant on the device (pmode 0), or both
// variants in turn with optional events around them (pmode 3, profiled runs).
void enqueue_step(mdg_handle *h, int par, int pmode = 0, cudaEvent_t before = nullptr, cudaEvent_t after = nullptr) {
  if (h->g.rebuild_policy == MDG_REBUILD_REFERENCE) {  // the check's kernels are no-ops unless it is due
    mdg::launch_policy(h->g, h->d, h->stream, 0, 0);
    mdg::launch_policy_check(h->g, h->d, par, h->stream);
  }
  mdg::launch_rebuild(h->g, h->d, par, h->num_sms, h->stream, true, lang_on(h) != 0, true);
  if (before) cudaEventRecord(before, h->stream);
  mdg::launch_step(h->g, h->d, par, h->prm.thermostat, h->prm.langevin_half_drift_compat, h->prm.precision,
                   h->stream, pmode);
  if (after) cudaEventRecord(after, h->stream);
}

// Appends what `enqueue` launches on the handle's stream to graph g after
// node `dep` (none when dep is null); *last receives the final node.
template <class F>
int append_captured(mdg_handle *h, cudaGraph_t g, const cudaGraphNode_t *dep, F enqueue, cudaGraphNode_t *last) {
  MDG_CK(cudaStreamBeginCaptureToGraph(h->stream, g, dep, nullptr, dep ? 1 : 0, cudaStreamCaptureModeThreadLocal));
  enqueue();
  cudaStreamCaptureStatus st;
  const cudaGraphNode_t *deps = nullptr;
  size_t nd = 0;
  cudaError_t e = cudaStreamGetCaptureInfo(h->stream, &st, nullptr, nullptr, &deps, nullptr, &nd);
  cudaGraphNode_t tail = (e == cudaSuccess && nd == 1) ? deps[0] : nullptr;
  cudaGraph_t out = nullptr;
  MDG_CK(cudaStreamEndCapture(h->stream, &out));
  if (e != cudaSuccess || !tail) return fail(h, MDG_ERR_CUDA, "graph capture did not end in one node");
  if (last) *last = tail;
  return MDG_OK;
}

// Adds a conditional node (IF with one body, or SWITCH with `bodies` bodies)
// after `dep` and fills each body with what `fill(k)` launches.
template <class F>
int add_conditional(mdg_handle *h, cudaGraph_t g, cudaGraphNode_t dep, cudaGraphConditionalHandle cond,
                    cudaGraphConditionalNodeType type, int bodies, F fill, cudaGraphNode_t *node) {
  cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};
  np.conditional.handle = cond;
  np.conditional.type = type;
  np.conditional.size = (unsigned)bodies;
  MDG_CK(cudaGraphAddNode(node, g, &dep, nullptr, 1, &np));
  for (int k = 0; k < bodies; k++) {
    cudaGraph_t body = np.conditional.phGraph_out[k];
    MDG_CK(cudaStreamBeginCaptureToGraph(h->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    fill(k);
    cudaGraph_t out = nullptr;
    MDG_CK(cudaStreamEndCapture(h->stream, &out));
  }
  return MDG_OK;
}

// Appends an event-record node after `dep`; *node receives it.
int add_event(mdg_handle *h, cudaGraph_t g, cudaGraphNode_t dep, cudaEvent_t ev, cudaGraphNode_t *node) {
  MDG_CK(cudaGraphAddEventRecordNode(node, g, &dep, 1, ev));
  return MDG_OK;
}

// A graph of nsteps steps starting at parity par.  Per step: a one-thread
// prelude (counters, inner-list hand-over) that sets the step's conditions,
// then one SWITCH { ordinary step | re-selecting step | rebuild (wrap, bin,
// reorder, build) and re-selecting step }: a step without a rebuild runs two
// kernels.  With `ev` (3 nsteps + 1 events, the timed graphs) the rebuild
// and the step are separate nodes, IF(rebuild) then SWITCH(variant), since
// event records cannot sit inside a conditional body: the graph starts by
// recording ev[3 nsteps], and step k records ev[3k] after its prelude,
// ev[3k+1] before its step kernel and ev[3k+2] after it, so the device time
// of each phase of each step is read from the same replay.
int capture(mdg_handle *h, cudaGraphExec_t *out, int par, int nsteps, cudaEvent_t *ev = nullptr) {
  cudaGraph_t g = nullptr;
  MDG_CK(cudaGraphCreate(&g, 0));
  cudaGraphNode_t last = nullptr;
  int rc = MDG_OK;
  if (ev) {
    cudaError_t e = cudaGraphAddEventRecordNode(&last, g, nullptr, 0, ev[3 * nsteps]);
    if (e != cudaSuccess) rc = fail(h, MDG_ERR_CUDA, std::string("cudaGraphAddEventRecordNode: ") + cudaGetErrorString(e));
  }
  const int lang = lang_on(h) != 0;
  for (int k = 0; k < nsteps && rc == MDG_OK; k++) {
    const int p = par ^ (k & 1);
    auto step_kernel = [&](int pmode) {
      mdg::launch_step(h->g, h->d, p, h->prm.thermostat, h->prm.langevin_half_drift_compat, h->prm.precision,
                       h->stream, pmode);
    };
    auto rebuild = [&] { mdg::launch_rebuild(h->g, h->d, p, h->num_sms, h->stream, false, false, true); };
    cudaGraphNode_t pre = nullptr, sw = nullptr;
    if (h->g.rebuild_policy == MDG_REBUILD_REFERENCE) {
      // the reference policy ahead of the step: the budget, then IF (spent)
      // { the displacement check }, which may set the rebuild flag
      cudaGraphConditionalHandle c_chk = 0;
      cudaError_t e = cudaGraphConditionalHandleCreate(&c_chk, g, 0, cudaGraphCondAssignDefault);
      if (e != cudaSuccess) {
        rc = fail(h, MDG_ERR_CUDA, std::string("cudaGraphConditionalHandleCreate: ") + cudaGetErrorString(e));
        break;
      }
      cudaGraphNode_t bud = nullptr, chk = nullptr;
      rc = append_captured(h, g, last ? &last : nullptr, [&] { mdg::launch_policy(h->g, h->d, h->stream, c_chk, 1); },
                           &bud);
      if (rc == MDG_OK)
        rc = add_conditional(h, g, bud, c_chk, cudaGraphCondTypeIf, 1,
                             [&](int) { mdg::launch_policy_check(h->g, h->d, p, h->stream); }, &chk);
      if (rc) break;
      last = chk;
    }
    if (ev) {
      cudaGraphConditionalHandle c_rb = 0, c_var = 0;
      cudaError_t e = cudaGraphConditionalHandleCreate(&c_rb, g, 0, cudaGraphCondAssignDefault);
      if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&c_var, g, 2, cudaGraphCondAssignDefault);
      if (e != cudaSuccess) {
        rc = fail(h, MDG_ERR_CUDA, std::string("cudaGraphConditionalHandleCreate: ") + cudaGetErrorString(e));
        break;
      }
      cudaGraphNode_t cond = nullptr;
      rc = append_captured(h, g, last ? &last : nullptr,
                           [&] { mdg::launch_prelude_split(h->d, lang, c_rb, c_var, h->stream); }, &pre);
      if (rc == MDG_OK) rc = add_event(h, g, pre, ev[3 * k], &pre);
      if (rc == MDG_OK) rc = add_conditional(h, g, pre, c_rb, cudaGraphCondTypeIf, 1, [&](int) { rebuild(); }, &cond);
      if (rc == MDG_OK) rc = add_event(h, g, cond, ev[3 * k + 1], &cond);
      if (rc == MDG_OK)
        rc = add_conditional(h, g, cond, c_var, cudaGraphCondTypeSwitch, 2,
                             [&](int variant) { step_kernel(variant == 0 ? 1 : 2); }, &sw);
      if (rc == MDG_OK) rc = add_event(h, g, sw, ev[3 * k + 2], &sw);
    } else {
      cudaGraphConditionalHandle c_step = 0;
      cudaError_t e = cudaGraphConditionalHandleCreate(&c_step, g, 3, cudaGraphCondAssignDefault);
      if (e != cudaSuccess) {
        rc = fail(h, MDG_ERR_CUDA, std::string("cudaGraphConditionalHandleCreate: ") + cudaGetErrorString(e));
        break;
      }
      rc = append_captured(h, g, last ? &last : nullptr, [&] { mdg::launch_prelude(h->d, lang, c_step, h->stream); },
                           &pre);
      if (rc == MDG_OK)
        rc = add_conditional(h, g, pre, c_step, cudaGraphCondTypeSwitch, 3, [&](int body) {
          if (body == 2) rebuild();
          step_kernel(body == 0 ? 1 : 2);
        }, &sw);
    }
    if (rc) break;
    last = sw;
  }
  if (rc == MDG_OK) {
    cudaError_t e = cudaGraphInstantiate(out, g, 0);
    if (e != cudaSuccess) rc = fail(h, MDG_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
    else h->graph_n = h->g.n;
  }
  cudaGraphDestroy(g);
  return rc;
}

int enqueue_steps(mdg_handle *h, int nsteps) {
  int par = h->par;
  if (!h->prm.use_graphs) {
    for (int k = 0; k < nsteps; k++) {
      enqueue_step(h, par);
      h->launches += kernels_per_step(h);
      par ^= 1;
    }
    h->par = par;
    return cudaGetLastError() == cudaSuccess ? MDG_OK : fail(h, MDG_ERR_CUDA, "kernel launch failed");
  }
  int left = nsteps;
  if (left >= 2) {
    if (!h->gx_pair[par]) {
      int rc = capture(h, &h->gx_pair[par], par, 2);
      if (rc) return rc;
    }
    while (left >= 2) {
      MDG_CK(cudaGraphLaunch(h->gx_pair[par], h->stream));
      left -= 2;
    }
  }
  if (left == 1) {
    if (!h->gx_one[par]) {
      int rc = capture(h, &h->gx_one[par], par, 1);
      if (rc) return rc;
    }
    MDG_CK(cudaGraphLaunch(h->gx_one[par], h->stream));
    par ^= 1;
  }
  h->par = par;
  return MDG_OK;
}

// Confirms the steps mdg_calculate enqueued without waiting: reads the device
// counters once, and after a halt on list overflow (the steps behind the halt
// ran as no-ops) regrows the rows and runs the steps that are still owed.
int settle(mdg_handle *h) {
  if (h->pending == 0) return MDG_OK;
  const long long want = h->pending;
  h->pending = 0;
  long long done = 0;
  for (int attempt = 0; attempt < 64 && done < want; attempt++) {
    const unsigned long long before = (unsigned long long)h->steps_host;
    const unsigned long long rebuilds0 = h->hflags->rebuilds, checks0 = h->hflags->checks;
    if (attempt > 0) {
      int rc = enqueue_steps(h, (int)(want - done));
      if (rc) return rc;
      MDG_CK(cudaEventRecord(h->ev1, h->stream));
    }
    int rc = read_flags(h);
    if (rc) return rc;
    long long completed = (long long)(h->hflags->steps - before);
    if (h->prm.use_graphs)
      h->launches += graph_kernels(h, completed, (long long)(h->hflags->rebuilds - rebuilds0),
                                   (long long)(h->hflags->checks - checks0));
    if (h->hflags->halt == 0) {
      done += completed;
      h->steps_host = (long long)h->hflags->steps;
      continue;
    }
    if (h->hflags->halt != mdg::kHaltOverflow) return halt_error(h);
    done += completed - 1;
    rc = recover_overflow(h, true);
    if (rc) return rc;
    h->steps_host = (long long)h->hflags->steps - 1;
  }
  if (h->ev1_due) MDG_CK(cudaEventRecord(h->ev1, h->stream));
  h->ev1_due = false;
  MDG_CK(cudaEventSynchronize(h->ev1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, h->ev0, h->ev1);
  h->last_ms = ms;
  if (done != want) return fail(h, MDG_ERR_CAPACITY, "neighbour list could not be sized");
  return MDG_OK;
}

// What an entry point does with steps still unconfirmed: confirm them first
// (every reader of the state), leave them (mdg_calculate), or drop the
// bookkeeping because the state is about to be replaced.
enum Pending { kSettle, kKeep, kDrop };

int check_handle(mdg_handle *h, bool need_state, Pending pending = kSettle) {
  if (!h) return MDG_ERR_INVALID;
  if (need_state && !h->has_state) return fail(h, MDG_ERR_NOT_READY, "no particle state loaded");
  cudaError_t e = cudaSetDevice(h->prm.device);
  if (e != cudaSuccess) return fail(h, MDG_ERR_CUDA, cudaGetErrorString(e));
  if (pending == kSettle) return settle(h);
  if (pending == kDrop) h->pending = 0;
  return MDG_OK;
}

}  // namespace

extern "C" {

const char *mdg_version(void) { return kVersion; }

void mdg_params_default(mdg_params *p) {
  if (!p) return;
  memset(p, 0, sizeof(*p));
  p->capacity = 1000000;
  p->precision = MDG_FP64;
  p->box[0] = p->box[1] = p->box[2] = 50.0;
  p->cutoff = 3.0;   // CUTOFF_LENGTH (mdconfig.h:15)
  p->margin = 0.3;   // BufferLength (simulationinfo.cc:6)
  p->dt = 0.001;     // TimeStep default (simulationinfo.cc:9)
  p->thermostat = MDG_NVE;
  p->langevin_half_drift_compat = 1;
  p->temperature = 1.0;  // AimedTemperature default
  p->gamma = 0.1;        // HeatbathGamma default
  p->tau = 0.1;          // HeatbathTau default
  p->seed = 1;
  p->use_graphs = 1;
  p->prune_buffer = -1.0;  // automatic
  p->rebuild_policy = MDG_REBUILD_HALFMARGIN;
  p->check_list_length = 500;  // CheckListLength default (simulationinfo.cc:27)
}

int mdg_create(const mdg_params *p, mdg_handle **out) {
  t_create_err.clear();
  if (!p || !out) return create_fail(MDG_ERR_INVALID, "null parameters or output");
  *out = nullptr;
  if (p->capacity <= 0 || p->capacity > mdg::kMaxParticles)
    return create_fail(MDG_ERR_INVALID, "capacity must be in 1 .. " + std::to_string(mdg::kMaxParticles));
  if (!(p->cutoff > 0.0) || !(p->margin >= 0.0) || !(p->dt > 0.0))
    return create_fail(MDG_ERR_INVALID, "cutoff and dt must be > 0, margin >= 0");
  if (p->precision < MDG_FP64 || p->precision > MDG_MIXED_PLAIN) return create_fail(MDG_ERR_INVALID, "bad precision");
  if (p->thermostat < MDG_NVE || p->thermostat > MDG_NOSEHOOVER) return create_fail(MDG_ERR_INVALID, "bad thermostat");
  if (p->rebuild_policy != MDG_REBUILD_HALFMARGIN && p->rebuild_policy != MDG_REBUILD_REFERENCE)
    return create_fail(MDG_ERR_INVALID, "bad rebuild policy");
  if (p->rebuild_policy == MDG_REBUILD_REFERENCE && p->check_list_length < 1)
    return create_fail(MDG_ERR_INVALID, "check_list_length must be >= 1");
  mdg_handle *h = new mdg_handle();
  h->prm = *p;
  memset(&h->g, 0, sizeof(h->g));
  memset(&h->d, 0, sizeof(h->d));
  int rc = setup_geometry(h);
  if (rc) {
    const std::string msg = h->err;
    delete h;
    return create_fail(rc, msg);
  }
  cudaError_t e = cudaSetDevice(p->device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, p->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&h->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&h->ev1);
  if (e == cudaSuccess) e = cudaMallocHost((void **)&h->hflags, sizeof(DevFlags));
  if (e == cudaSuccess) e = cudaMallocHost((void **)&h->hobs, 4 * sizeof(double));
  const size_t cap = (size_t)p->capacity;
  h->cap = p->capacity;
  mdg::Dev &d = h->d;
  const size_t ncell = (size_t)h->g.nrank;
  const size_t nred = (cap + 127) / 128 + 1;
  if (e == cudaSuccess) e = dalloc(&d.q_end, cap);
  if (e == cudaSuccess) e = dalloc(&d.q_mid[0], cap);
  if (e == cudaSuccess) e = dalloc(&d.q_mid[1], cap);
  if (e == cudaSuccess) e = dalloc(&d.p, cap);
  if (e == cudaSuccess) e = dalloc(&d.q_build, cap);
  if (e == cudaSuccess) e = dalloc(&d.t_q, cap);
  if (e == cudaSuccess) e = dalloc(&d.t_p, cap);
  if (e == cudaSuccess) e = dalloc(&d.qf, cap);
  if (e == cudaSuccess) e = dalloc(&d.loc[0], cap);
  if (e == cudaSuccess) e = dalloc(&d.loc[1], cap);
  if (e == cudaSuccess) e = dalloc(&d.loc_p, cap);
  if (e == cudaSuccess) e = dalloc(&d.pcount, cap);
  if (e == cudaSuccess) e = dalloc(&d.id, cap);
  if (e == cudaSuccess) e = dalloc(&d.inv, cap);
  if (e == cudaSuccess) e = dalloc(&d.cell, cap);
  if (e == cudaSuccess) e = dalloc(&d.t_id, cap);
  if (e == cudaSuccess) e = dalloc(&d.t_cell, cap);
  if (e == cudaSuccess) e = dalloc(&d.order, cap);
  if (e == cudaSuccess) e = dalloc(&d.cell_count, ncell);
  if (e == cudaSuccess) e = dalloc(&d.cell_fill, ncell);
  if (e == cudaSuccess) e = dalloc(&d.cell_start, ncell + 1);
  if (e == cudaSuccess) e = dalloc(&d.block_sums, 4096);
  if (e == cudaSuccess) e = dalloc(&d.ncount, cap);
  if (e == cudaSuccess) e = dalloc(&d.partials, 3 * nred);
  if (e == cudaSuccess) e = dalloc(&d.vpart, 2 * ((cap + 255) / 256 + 1));
  if (e == cudaSuccess)
    e = dalloc(&d.cand, p->rebuild_policy == MDG_REBUILD_REFERENCE ? 2 * (size_t)p->check_list_length : (size_t)2);
  if (e == cudaSuccess) e = dalloc(&d.flags, 1);
  if (e == cudaSuccess) e = dalloc(&d.io4, cap);
  if (e == cudaSuccess) e = dalloc(&d.io4b, cap);
  if (e == cudaSuccess) e = dalloc(&h->dobs, 4);
  if (e == cudaSuccess) e = cudaMemsetAsync(d.cell_count, 0, ncell * sizeof(int), h->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(d.cell_fill, 0, ncell * sizeof(int), h->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(d.flags, 0, sizeof(DevFlags), h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  d.nblocks_red = (int)nred;
  h->g.stride = h->cap;
  if (e != cudaSuccess) {
    std::string msg = cudaGetErrorString(e);
    mdg_destroy(h);
    return create_fail(MDG_ERR_CUDA, msg);
  }
  *out = h;
  return MDG_OK;
}

int mdg_destroy(mdg_handle *h) {
  if (!h) return MDG_OK;
  cudaSetDevice(h->prm.device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  drop_graphs(h);
  dfree_all(h);
  if (h->hflags) cudaFreeHost(h->hflags);
  if (h->hobs) cudaFreeHost(h->hobs);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return MDG_OK;
}

const char *mdg_last_error(const mdg_handle *h) {
  if (h) return h->err.c_str();
  return t_create_err.empty() ? "null handle" : t_create_err.c_str();
}

static int set_state_common(mdg_handle *h, int32_t n) {
  h->g.n = n;
  if (!h->d.nl || h->prm.list_capacity > 0 || h->g.list_cap < 8) {
    int lc = h->prm.list_capacity > 0 ? ((h->prm.list_capacity + 7) & ~7) : estimate_list_cap(h, n);
    if (!h->d.nl || lc != h->g.list_cap) {
      int rc = alloc_list(h, lc);
      if (rc) return rc;
    }
  }
  DevFlags f;
  memset(&f, 0, sizeof f);
  f.rebuild = 1;
  f.bad_slot = INT_MAX;
  f.exp1 = 1.0;
  *h->hflags = f;
  MDG_CK(cudaMemsetAsync(h->d.cell_count, 0, (size_t)h->g.nrank * sizeof(int), h->stream));
  MDG_CK(cudaMemsetAsync(h->d.cell_fill, 0, (size_t)h->g.nrank * sizeof(int), h->stream));
  MDG_CK(cudaMemcpyAsync(h->d.flags, h->hflags, sizeof(DevFlags), cudaMemcpyHostToDevice, h->stream));
  MDG_CK(cudaStreamSynchronize(h->stream));
  // the graphs hold the geometry by value; they stay valid for the same count
  if (h->graph_n != n) drop_graphs(h);
  h->has_state = true;
  h->nh_init = true;
  h->par = 0;
  h->steps_host = 0;
  return MDG_OK;
}

int mdg_set_state(mdg_handle *h, const double *q4, const double *p4, int32_t n) {
  int rc = check_handle(h, false, kDrop);
  if (rc) return rc;
  if (!q4 || !p4 || n <= 0) return fail(h, MDG_ERR_INVALID, "null state or n <= 0");
  if (n > h->cap) return fail(h, MDG_ERR_CAPACITY, "more particles than the handle capacity");
  MDG_CK(cudaMemcpyAsync(h->d.io4, q4, (size_t)n * sizeof(double4_32a), cudaMemcpyHostToDevice, h->stream));
  MDG_CK(cudaMemcpyAsync(h->d.io4b, p4, (size_t)n * sizeof(double4_32a), cudaMemcpyHostToDevice, h->stream));
  h->g.n = n;
  mdg::launch_sort_in(h->g, h->d, h->d.io4, h->d.io4b, h->stream);
  h->launches += 1;
  return set_state_common(h, n);
}

int mdg_set_state_device(mdg_handle *h, const double *q4, const double *p4, int32_t n) {
  int rc = check_handle(h, false, kDrop);
  if (rc) return rc;
  if (!q4 || !p4 || n <= 0) return fail(h, MDG_ERR_INVALID, "null state or n <= 0");
  if (n > h->cap) return fail(h, MDG_ERR_CAPACITY, "more particles than the handle capacity");
  h->g.n = n;
  mdg::launch_sort_in(h->g, h->d, (const double4_32a *)q4, (const double4_32a *)p4, h->stream);
  return set_state_common(h, n);
}

int mdg_make_state(mdg_handle *h, int32_t maker, double density, double radius, double v0) {
  int rc = check_handle(h, false, kDrop);
  if (rc) return rc;
  int32_t n = 0;
  // the collision maker sets its own velocities (speed v0 along x); the other
  // makers leave them zero for SetInitialVelocity
  const bool own_velocity = maker == MDG_MAKER_COLLISION;
  rc = mdg_make_configuration(h->g.L, maker, density, radius, 0, own_velocity ? v0 : 0.0, (double *)h->d.io4,
                              (double *)h->d.io4b, h->cap, &n, h->stream);
  if (rc == MDG_ERR_CAPACITY) return fail(h, rc, "the configuration has more particles than the handle capacity");
  if (rc) return fail(h, rc, "configuration maker failed");
  if (n <= 0) return fail(h, MDG_ERR_INVALID, "the configuration is empty");
  if (!own_velocity && v0 != 0.0) {
    rc = mdg_make_velocity(v0, 0, (double *)h->d.io4b, n, h->stream);
    if (rc) return fail(h, rc, "velocity maker failed");
  }
  h->g.n = n;
  mdg::launch_sort_in(h->g, h->d, h->d.io4, h->d.io4b, h->stream);
  h->launches += 1;
  return set_state_common(h, n);
}

int mdg_get_state(mdg_handle *h, double *q4, double *p4) {
  int rc = check_handle(h, true);
  if (rc) return rc;
  mdg::launch_unsort(h->g, h->d, h->par, q4 ? h->d.io4 : nullptr, p4 ? h->d.io4b : nullptr, h->stream);
  h->launches += h->g.local_pos ? 3 : 1;
  const size_t bytes = (size_t)h->g.n * sizeof(double4_32a);
  if (q4) MDG_CK(cudaMemcpyAsync(q4, h->d.io4, bytes, cudaMemcpyDeviceToHost, h->stream));
  if (p4) MDG_CK(cudaMemcpyAsync(p4, h->d.io4b, bytes, cudaMemcpyDeviceToHost, h->stream));
  MDG_CK(cudaStreamSynchronize(h->stream));
  return MDG_OK;
}

int mdg_get_state_device(mdg_handle *h, double *q4, double *p4) {
  int rc = check_handle(h, true);
  if (rc) return rc;
  mdg::launch_unsort(h->g, h->d, h->par, (double4_32a *)q4, (double4_32a *)p4, h->stream);
  h->launches += h->g.local_pos ? 3 : 1;
  MDG_CK(cudaGetLastError());
  return MDG_OK;
}

int mdg_make_pairlist(mdg_handle *h) {
  int rc = check_handle(h, true);
  if (rc) return rc;
  return ensure_list(h, true);
}

int mdg_calculate(mdg_handle *h, int32_t nsteps) {
  int rc = check_handle(h, true, kKeep);
  if (rc) return rc;
  if (nsteps < 0) return fail(h, MDG_ERR_INVALID, "negative step count");
  if (nsteps == 0) return MDG_OK;
  if (h->prm.thermostat == MDG_NOSEHOOVER && h->nh_init) {
    mdg::launch_nh_init(h->g, h->d, h->stream);
    h->launches += 2;
    h->nh_init = false;
  }
  // A multi-step call is timed on its own: ev0 follows any steps still
  // outstanding in the stream, ev1 its last step.  A run of single-step calls
  // (MDManager::Calculate once per step) records no events between the steps
  // (each record costs about 7 us of device time): it is timed from its first
  // call to the point where it is confirmed.
  if (nsteps > 1 || h->pending == 0) MDG_CK(cudaEventRecord(h->ev0, h->stream));
  rc = enqueue_steps(h, nsteps);
  if (rc) return rc;
  h->ev1_due = nsteps == 1;
  if (!h->ev1_due) MDG_CK(cudaEventRecord(h->ev1, h->stream));
  h->pending += nsteps;
  if (h->pending >= kMaxPending) return settle(h);
  return MDG_OK;
}

int mdg_synchronize(mdg_handle *h) { return check_handle(h, false); }

}  // extern "C"

namespace {

// Steps replayed as the graph mdg_calculate replays, with event-record nodes
// around each step's rebuild phase and step kernel (capture(.., ev)); the
// graph of up to kTimedChunk steps is captured for the call and replayed
// once.  Sums the device time of the step kernels, of the rebuild phases
// and of the whole run, and counts the rebuilds that ran.
constexpr int kTimedChunk = 1024;

int timed_graph_run(mdg_handle *h, int32_t nsteps, double *step_ms, double *rebuild_ms, double *all_ms) {
  std::vector<cudaEvent_t> ev(3 * (size_t)kTimedChunk + 1, nullptr);
  for (auto &e : ev) MDG_CK(cudaEventCreate(&e));
  double t_step = 0.0, t_rebuild = 0.0, t_all = 0.0;
  long long done = 0;
  int status = MDG_OK;
  for (int guard = 0; guard < 4096 && done < nsteps && status == MDG_OK; guard++) {
    const int m = (int)((nsteps - done) < kTimedChunk ? (nsteps - done) : kTimedChunk);
    const unsigned long long before = (unsigned long long)h->steps_host, rebuilds0 = h->hflags->rebuilds,
                             checks0 = h->hflags->checks;
    cudaGraphExec_t gx = nullptr;
    status = capture(h, &gx, h->par, m, ev.data());
    if (status) break;
    cudaError_t e = cudaGraphLaunch(gx, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaGraphExecDestroy(gx);
    if (e != cudaSuccess) {
      status = fail(h, MDG_ERR_CUDA, std::string("timed graph: ") + cudaGetErrorString(e));
      break;
    }
    status = read_flags(h);
    if (status) break;
    const long long completed = (long long)(h->hflags->steps - before);
    h->launches += graph_kernels(h, completed, (long long)(h->hflags->rebuilds - rebuilds0),
                                 (long long)(h->hflags->checks - checks0));
    // a halted step and those behind it ran as no-ops: only the steps that
    // completed are timed
    const int timed = (int)(h->hflags->halt == 0 ? m : completed - 1);
    for (int k = 0; k < timed; k++) {
      float a = 0.f, b = 0.f;
      if (cudaEventElapsedTime(&a, ev[3 * k], ev[3 * k + 1]) == cudaSuccess) t_rebuild += a;
      if (cudaEventElapsedTime(&b, ev[3 * k + 1], ev[3 * k + 2]) == cudaSuccess) t_step += b;
    }
    float w = 0.f;
    if (timed > 0 && cudaEventElapsedTime(&w, ev[3 * m], ev[3 * (timed - 1) + 2]) == cudaSuccess) t_all += w;
    if (h->hflags->halt == 0) {
      done += completed;
      h->steps_host = (long long)h->hflags->steps;
      h->par ^= m & 1;
    } else if (h->hflags->halt == mdg::kHaltOverflow) {
      done += completed - 1;
      status = recover_overflow(h, true);
      h->steps_host = (long long)h->hflags->steps - 1;
      h->par ^= (int)((completed - 1) & 1);
    } else {
      status = halt_error(h);
    }
  }
  for (auto &e : ev) cudaEventDestroy(e);
  if (step_ms) *step_ms = t_step;
  if (rebuild_ms) *rebuild_ms = t_rebuild;
  if (all_ms) *all_ms = t_all;
  if (status == MDG_OK && done != nsteps) return fail(h, MDG_ERR_CAPACITY, "neighbour list could not be sized");
  return status;
}

// Steps as plain launches with three events per step on the handle's stream
// (graphs off): before the rebuild sequence, before the step kernel, after
// it.  Sums the device time of the step kernels (force, kick, drifts), of
// the rebuild sequences (wrap, bin, sort, list build; empty launches when none
// is due) and of the whole run.
int profiled_run(mdg_handle *h, int32_t nsteps, double *step_ms, double *rebuild_ms, double *all_ms) {
  if (h->prm.thermostat == MDG_NOSEHOOVER && h->nh_init) {
    mdg::launch_nh_init(h->g, h->d, h->stream);
    h->launches += 2;
    h->nh_init = false;
  }
  if (h->prm.use_graphs) return timed_graph_run(h, nsteps, step_ms, rebuild_ms, all_ms);
  constexpr int kChunk = 64;
  cudaEvent_t ev[3 * kChunk];
  for (int k = 0; k < 3 * kChunk; k++) MDG_CK(cudaEventCreate(&ev[k]));
  long long done = 0;
  double t_step = 0.0, t_rebuild = 0.0, t_all = 0.0;
  int status = MDG_OK;
  for (int guard = 0; guard < 1000000 && done < nsteps && status == MDG_OK; guard++) {
    const unsigned long long before = (unsigned long long)h->steps_host;
    const int m = (int)((nsteps - done) < kChunk ? (nsteps - done) : kChunk);
    for (int k = 0; k < m; k++) {
      cudaEventRecord(ev[3 * k], h->stream);
      enqueue_step(h, h->par, 3, ev[3 * k + 1], ev[3 * k + 2]);
      h->launches += kernels_per_step(h) + 1;
      h->par ^= 1;
    }
    status = read_flags(h);
    if (status) break;
    for (int k = 0; k < m; k++) {
      float a = 0.f, b = 0.f;
      if (cudaEventElapsedTime(&a, ev[3 * k], ev[3 * k + 1]) == cudaSuccess) t_rebuild += a;
      if (cudaEventElapsedTime(&b, ev[3 * k + 1], ev[3 * k + 2]) == cudaSuccess) t_step += b;
    }
    float w = 0.f;
    if (cudaEventElapsedTime(&w, ev[0], ev[3 * (m - 1) + 2]) == cudaSuccess) t_all += w;
    long long completed = (long long)(h->hflags->steps - before);
    if (h->hflags->halt == 0) {
      done += completed;
      h->steps_host = (long long)h->hflags->steps;
    } else if (h->hflags->halt == mdg::kHaltOverflow) {
      done += completed - 1;
      status = recover_overflow(h, true);
      h->steps_host = (long long)h->hflags->steps - 1;
    } else {
      status = halt_error(h);
    }
  }
  for (int k = 0; k < 3 * kChunk; k++) cudaEventDestroy(ev[k]);
  if (step_ms) *step_ms = t_step;
  if (rebuild_ms) *rebuild_ms = t_rebuild;
  if (all_ms) *all_ms = t_all;
  return status;
}

}  // namespace

extern "C" {

int mdg_calculate_profiled(mdg_handle *h, int32_t nsteps, double *step_kernel_ms) {
  int rc = check_handle(h, true);
  if (rc) return rc;
  if (nsteps < 0 || !step_kernel_ms) return fail(h, MDG_ERR_INVALID, "bad arguments");
  *step_kernel_ms = 0.0;
  return profiled_run(h, nsteps, step_kernel_ms, nullptr, nullptr);
}

int mdg_calculate_phases(mdg_handle *h, int32_t nsteps, double phase_ms[3]) {
  int rc = check_handle(h, true);
  if (rc) return rc;
  if (nsteps < 0 || !phase_ms) return fail(h, MDG_ERR_INVALID, "bad arguments");
  phase_ms[0] = phase_ms[1] = phase_ms[2] = 0.0;
  return profiled_run(h, nsteps, &phase_ms[0], &phase_ms[1], &phase_ms[2]);
}

int mdg_observe(mdg_handle *h, double out[3]) {
  int rc = check_handle(h, true);
  if (rc) return rc;
  if (!out) return fail(h, MDG_ERR_INVALID, "null output");
  rc = ensure_list(h, false);
  if (rc) return rc;
  mdg::launch_observe(h->g, h->d, h->dobs, h->stream, h->prm.precision != MDG_FP64, h->par);
  h->launches += h->prm.precision != MDG_FP64 ? 3 : 2;
  MDG_CK(cudaMemcpyAsync(h->hobs, h->dobs, 3 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  MDG_CK(cudaStreamSynchronize(h->stream));
  out[0] = h->hobs[0];
  out[1] = h->hobs[1];
  out[2] = h->hobs[2];
  return MDG_OK;
}

int mdg_forces(mdg_handle *h, double *f4) {
  int rc = check_handle(h, true);
  if (rc) return rc;
  if (!f4) return fail(h, MDG_ERR_INVALID, "null output");
  rc = ensure_list(h, false);
  if (rc) return rc;
  mdg::launch_forces(h->g, h->d, h->prm.precision, h->par, h->stream);
  h->launches += h->prm.precision != MDG_FP64 ? 2 : 1;
  MDG_CK(cudaMemcpyAsync(f4, h->d.io4, (size_t)h->g.n * sizeof(double4_32a), cudaMemcpyDeviceToHost, h->stream));
  MDG_CK(cudaStreamSynchronize(h->stream));
  return MDG_OK;
}

int mdg_pairs(mdg_handle *h, int32_t *rec, int64_t cap, int64_t *count) {
  int rc = check_handle(h, true);
  if (rc) return rc;
  if (!count) return fail(h, MDG_ERR_INVALID, "null count");
  rc = ensure_list(h, false);
  if (rc) return rc;
  const int n = h->g.n;
  std::vector<int> cnt(n);
  MDG_CK(cudaMemcpyAsync(cnt.data(), h->d.ncount, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  MDG_CK(cudaStreamSynchronize(h->stream));
  std::vector<long long> off(n + 1, 0);
  for (int i = 0; i < n; i++) off[i + 1] = off[i] + cnt[i];
  *count = off[n];
  if (!rec || cap <= 0) return MDG_OK;
  long long *doff = nullptr;
  int32_t *drec = nullptr;
  MDG_CK(dalloc(&doff, (size_t)n + 1));
  cudaError_t e = dalloc(&drec, (size_t)off[n] * 3);
  if (e == cudaSuccess) e = cudaMemcpyAsync(doff, off.data(), (n + 1) * sizeof(long long), cudaMemcpyHostToDevice, h->stream);
  if (e == cudaSuccess) {
    mdg::launch_pairs(h->g, h->d, doff, drec, h->stream);
    const int64_t m = cap < off[n] ? cap : off[n];
    e = cudaMemcpyAsync(rec, drec, (size_t)m * 3 * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  cudaFree(doff);
  cudaFree(drec);
  if (e != cudaSuccess) return fail(h, MDG_ERR_CUDA, cudaGetErrorString(e));
  return MDG_OK;
}

int mdg_set_seed(mdg_handle *h, uint64_t seed) {
  int rc = check_handle(h, false);
  if (rc) return rc;
  h->prm.seed = seed;
  h->g.seed = seed;
  drop_graphs(h);
  return MDG_OK;
}

int mdg_set_thermostat(mdg_handle *h, int32_t thermostat, double temperature) {
  int rc = check_handle(h, false);
  if (rc) return rc;
  if (thermostat < MDG_NVE || thermostat > MDG_NOSEHOOVER) return fail(h, MDG_ERR_INVALID, "bad thermostat");
  h->prm.thermostat = thermostat;
  h->prm.temperature = temperature;
  rc = setup_geometry(h);
  if (rc) return rc;
  h->nh_init = true;
  drop_graphs(h);
  return MDG_OK;
}

int mdg_get_stats(mdg_handle *h, mdg_stats *s) {
  int rc = check_handle(h, false);
  if (rc) return rc;
  if (!s) return fail(h, MDG_ERR_INVALID, "null stats");
  memset(s, 0, sizeof(*s));
  if (h->has_state) {
    rc = read_flags(h);
    if (rc) return rc;
    s->steps = (int64_t)h->hflags->steps;
    s->rebuilds = (int64_t)h->hflags->rebuilds;
    s->max_neighbours = h->hflags->max_count;
    s->listed_pairs = (int64_t)h->hflags->pairs;
    s->zeta = h->hflags->zeta;
    s->inner_pairs = (int64_t)h->hflags->inner_pairs;
    s->prunes = (int64_t)h->hflags->prunes;
  }
  s->list_capacity = h->g.list_cap;
  for (int k = 0; k < 3; k++) s->cells[k] = h->g.nc[k];
  s->particles = h->has_state ? h->g.n : 0;
  s->elapsed_ms = h->last_ms;
  s->kernel_launches = h->launches;
  return MDG_OK;
}

}  // extern "C"
