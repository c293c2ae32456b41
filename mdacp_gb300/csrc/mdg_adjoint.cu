// Adjoint of an NVE trajectory: gradients of a trajectory-averaged observable
// with respect to the LJ parameters (epsilon, sigma) and the initial state.
//
// No reference counterpart (a pattern on top of the drop-in).  The potential
// is the reference's smoothly truncated LJ (variables.cc:16-28) written with
// explicit parameters, V(r) = eps * phi(r / sigma),
//   phi(x) = 4 (x^-12 - x^-6 + C2 x^2 + C0) for x <= xc,
// the cut-off scaling with sigma (xc = cutoff in sigma units).  The step is
// the reference's drift-kick-drift (mdmanager.cc:151-157):
//   qh = q + p dt/2;  p' = p + F(qh) dt;  q' = qh + p' dt/2.
// Objectives J = (1/Ns) sum_{n=1..Ns} j(q_n, p_n) with j = U/N (mean
// potential energy per particle, MDManager::PotentialEnergy) or
// j = P = (2 KE - G) / (3 V), G = sum_pairs f(r) r^2 (MDManager::Pressure).
//
// Discrete adjoint (exact gradient of the discrete trajectory): walking the
// steps backwards, with a_q, a_p the adjoints of (q_n, p_n):
//   a_p += dt/2 a_q;  a_qh = a_q - dt H(qh) a_p;  g_theta += dt a_p . dF/dtheta(qh);
//   a_q = a_qh;  a_p += dt/2 a_qh;  then the objective terms of the earlier state.
// H v is the Hessian-vector product over the same pair list.  States are
// checkpointed every K steps in the forward pass; the backward pass recomputes
// each segment from its checkpoint (storing its K half-step positions and
// states) and then reverses it.  Each checkpoint segment has its own pair
// list (every pair within cutoff*sigma + margin at the segment's first state,
// minimum image), built from the same state in both passes; the forward pass
// verifies that no particle moves more than margin/2 within a segment.  The
// pair kernels give each particle kLanes lanes and evaluate the pair terms
// without divisions (GB300's FP64 rate is 1/64 of FP32).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "mdg_internal.cuh"

namespace mdg {
namespace adj {

constexpr int kT = 128;
// Lanes sharing one particle's row in the pair kernels (FP64 runs at 1/64 of
// the FP32 rate on GB300, so a few thousand particles need several lanes each
// to occupy every SM's FP64 pipes).
#ifndef MDG_ADJ_LANES
#define MDG_ADJ_LANES 8
#endif
constexpr int kLanes = MDG_ADJ_LANES;

struct P {
  double L[3];
  double inv_L[3];
  double eps, sig, dt, dt2;
  double xc2;      // (cutoff in sigma units)^2
  double c0, c2;   // correction constants of phi
  double sl2;      // list radius^2 (absolute)
  double sl2f;     // the float test's radius^2 (widened by 1e-3)
  double half_margin2;
  double volume;
  // eps / sigma^k products used per pair (no division in the pair terms)
  double inv_s2, e_s, e_s2, e_s3, e_s4;
  int n, cap, objective, pad;
};

struct D {
  double4_32a *q, *p, *qh, *F, *aq, *ap, *aqh, *tmp, *q0;
  double4_32a *ckq, *ckp;    // checkpoints
  double4_32a *segq, *segp, *segqh;  // recomputed segment
  int *nbr, *cnt;            // the current segment's list, row-major [n][cap]
  double *part;              // block partials
  double *acc;               // running sums: J, g_eps, g_sig
  int *flag;
  unsigned int *done;        // blocks of the current reduction that wrote their partials
};

__device__ __forceinline__ void min_image(const P &c, double &dx, double &dy, double &dz) {
  dx -= c.L[0] * rint(dx * c.inv_L[0]);
  dy -= c.L[1] * rint(dy * c.inv_L[1]);
  dz -= c.L[2] * rint(dz * c.inv_L[2]);
}

// 1/x from the hardware estimate refined by one cubic Householder step
// (relative error of the estimate cubed, below double rounding).
__device__ __forceinline__ double recip(double x) {
  double y;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  const double e = fma(-x, y, 1.0);
  return fma(y, fma(e, e, e), y);
}

// Per pair at distance r (d = q_j - q_i): the reduced quantities.
struct PairTerms {
  double f;      // V'(r)/r: force on i is f d
  double fpr;    // f'(r)/r
  double phi;    // V(r)
  double fs;     // d f / d sigma
  double dphis;  // d V / d sigma
  double g;      // f r^2
  double gpr;    // g'(r)/r
  double gs;     // d g / d sigma
};

__device__ __forceinline__ bool pair_terms(const P &c, double r2, PairTerms &t) {
  const double x2 = r2 * c.inv_s2;
  // x2 >= +0: compared as bit patterns, on the integer pipe (same order)
  if (__double_as_longlong(x2) > __double_as_longlong(c.xc2)) return false;
  const double ix2 = recip(x2), ix6 = ix2 * ix2 * ix2, ix8 = ix6 * ix2, ix12 = ix6 * ix6, ix14 = ix12 * ix2;
  const double ix10 = ix8 * ix2, ix16 = ix14 * ix2;
  // psi(x) = phi'(x)/x, chi(x) = x^2 psi(x)
  const double psi = -48.0 * ix14 + 24.0 * ix8 + 8.0 * c.c2;
  const double dpsi_x = 672.0 * ix16 - 192.0 * ix10;      // psi'(x)/x
  const double phi = 4.0 * (ix12 - ix6 + c.c2 * x2 + c.c0);
  const double xdphi = 4.0 * (-12.0 * ix12 + 6.0 * ix6 + 2.0 * c.c2 * x2);  // x phi'(x)
  const double chi = x2 * psi;                               // -48 x^-12 + 24 x^-6 + 8 C2 x^2
  const double xdchi = 576.0 * ix12 - 144.0 * ix6 + 16.0 * c.c2 * x2;  // x chi'(x)
  t.f = c.e_s2 * psi;
  t.fpr = c.e_s4 * dpsi_x;
  t.phi = c.eps * phi;
  t.fs = -c.e_s3 * (2.0 * psi + x2 * dpsi_x);
  t.dphis = -c.e_s * xdphi;
  t.g = c.eps * chi;
  t.gpr = c.e_s2 * (xdchi * ix2);
  t.gs = -c.e_s * xdchi;
  return true;
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

// Writes this block's three partials; the last block of the grid to do so
// adds w times their sums (blocks in a fixed order, so the result does not
// depend on which block finished last) to acc[0..2] and rearms the counter.
// No block waits for another.
__device__ void partials_accumulate(const D &d, double A, double B, double E, double w) {
  __shared__ int last;
  __shared__ double sh2[32];
  if (threadIdx.x == 0) {
    d.part[3 * blockIdx.x + 0] = A;
    d.part[3 * blockIdx.x + 1] = B;
    d.part[3 * blockIdx.x + 2] = E;
    __threadfence();
    last = atomicAdd(d.done, 1u) == gridDim.x - 1 ? 1 : 0;
  }
  __syncthreads();
  if (!last) return;
  double a = 0, b = 0, e = 0;
  for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) {
    a += __ldcg(d.part + 3 * k);
    b += __ldcg(d.part + 3 * k + 1);
    e += __ldcg(d.part + 3 * k + 2);
  }
  const double ta = block_sum(a, sh2), tb = block_sum(b, sh2), te = block_sum(e, sh2);
  if (threadIdx.x == 0) {
    d.acc[0] += w * ta;
    d.acc[1] += w * tb;
    d.acc[2] += w * te;
    *d.done = 0;
  }
}

// Sum over the kLanes lanes that share a particle (all lanes hold the total).
__device__ __forceinline__ double lane_sum(double v) {
#pragma unroll
  for (int o = 1; o < kLanes; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Pair list at positions q: every partner within the list radius, minimum
// image.  kLanes lanes share a particle: lane l tests partners j = l, l +
// kLanes, ... (a particle's lanes read neighbouring positions together), first
// counting, then writing at its offset in the row (a prefix sum over the
// lanes), so the row order is fixed: lane 0's partners, then lane 1's, ...
// The test runs in float against a radius widened by 1e-3 (float positions of
// a box of tens of sigma are within 1e-5), so every pair within the exact
// radius is listed; a few more do no harm (the pair terms cut at rc).
__global__ void __launch_bounds__(kT) k_build(P c, D d, const double4_32a *q) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = tid / kLanes, lane = tid % kLanes;
  const bool active = i < c.n;
  float qx = 0.f, qy = 0.f, qz = 0.f;
  if (active) {
    const double4_32a v = q[i];
    qx = (float)v.x;
    qy = (float)v.y;
    qz = (float)v.z;
  }
  const float lx = (float)c.L[0], ly = (float)c.L[1], lz = (float)c.L[2];
  const float ilx = (float)c.inv_L[0], ily = (float)c.inv_L[1], ilz = (float)c.inv_L[2];
  const float sl2f = (float)c.sl2f;
  auto within = [&](int j) {
    const double4_32a v = q[j];
    float dx = (float)v.x - qx, dy = (float)v.y - qy, dz = (float)v.z - qz;
    dx -= lx * rintf(dx * ilx);
    dy -= ly * rintf(dy * ily);
    dz -= lz * rintf(dz * ilz);
    return dx * dx + dy * dy + dz * dz <= sl2f && j != i;
  };
  int m = 0;
  if (active)
    for (int j = lane; j < c.n; j += kLanes) m += within(j) ? 1 : 0;
  // offsets of the lanes' partners in the row
  int incl = m;
#pragma unroll
  for (int o = 1; o < kLanes; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o, kLanes);
    if (lane >= o) incl += v;
  }
  const int total = __shfl_sync(0xffffffffu, incl, kLanes - 1, kLanes);
  if (active) {
    int w = incl - m;
    int *row = d.nbr + (size_t)i * c.cap;
    for (int j = lane; j < c.n; j += kLanes)
      if (within(j)) {
        if (w < c.cap) row[w] = j;
        w++;
      }
    if (lane == 0) {
      d.cnt[i] = total < c.cap ? total : c.cap;
      if (total > c.cap) atomicMax(d.flag, total);
    }
  }
}

// Forces at the half-step positions q; also the segment's displacement check
// (a particle more than margin/2 from where the segment's list was built).
__global__ void k_force(P c, D d, const double4_32a *q, double4_32a *F) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = tid / kLanes, lane = tid % kLanes;
  double fx = 0, fy = 0, fz = 0;
  if (i < c.n) {
    const double4_32a qi = q[i];
    if (lane == 0) {
      const double4_32a z = d.q0[i];
      const double ux = qi.x - z.x, uy = qi.y - z.y, uz = qi.z - z.z;
      if (ux * ux + uy * uy + uz * uz > c.half_margin2) atomicMax(d.flag + 1, 1);
    }
    for (int k = lane; k < d.cnt[i]; k += kLanes) {
      const double4_32a qj = q[d.nbr[(size_t)i * c.cap + k]];
      double dx = qj.x - qi.x, dy = qj.y - qi.y, dz = qj.z - qi.z;
      min_image(c, dx, dy, dz);
      PairTerms t;
      if (!pair_terms(c, dx * dx + dy * dy + dz * dz, t)) continue;
      fx += t.f * dx;
      fy += t.f * dy;
      fz += t.f * dz;
    }
  }
  fx = lane_sum(fx);
  fy = lane_sum(fy);
  fz = lane_sum(fz);
  if (i < c.n && lane == 0) F[i] = make_double4_32a(fx, fy, fz, 0.0);
}

// qh = q + p dt/2: the first half-drift of a trajectory or segment
__global__ void k_drift(P c, const double4_32a *q, const double4_32a *p, double4_32a *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.n) return;
  double4_32a a = q[i];
  const double4_32a b = p[i];
  a.x += b.x * c.dt2;
  a.y += b.y * c.dt2;
  a.z += b.z * c.dt2;
  out[i] = a;
}

// p_out = p_in + F dt; q_out = qh + p_out dt/2; and, when qh_next is given,
// the next step's first half-drift qh_next = q_out + p_out dt/2 (the same
// operations k_drift performs).  Out of place, so a recomputed segment writes
// step k from step k - 1 without copies; qh_next may alias qh.
__global__ void k_kick_drift(P c, const double4_32a *qh, const double4_32a *F, const double4_32a *p_in,
                             double4_32a *q_out, double4_32a *p_out, double4_32a *qh_next) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.n) return;
  double4_32a b = p_in[i];
  const double4_32a f = F[i];
  b.x += f.x * c.dt;
  b.y += f.y * c.dt;
  b.z += f.z * c.dt;
  p_out[i] = b;
  double4_32a a = qh[i];
  a.x += b.x * c.dt2;
  a.y += b.y * c.dt2;
  a.z += b.z * c.dt2;
  q_out[i] = a;
  if (qh_next) {
    a.x += b.x * c.dt2;
    a.y += b.y * c.dt2;
    a.z += b.z * c.dt2;
    qh_next[i] = a;
  }
}

// Objective j at (q, p) into partials (value, d/deps, d/dsigma); with GRAD,
// also adds w * dj/dq to aq and w * dj/dp to ap (w = 1/Ns).  OBJ and GRAD are
// template parameters so that each pass computes only the pair terms it uses
// (the forward pass of the potential-energy objective needs phi and its sigma
// derivative alone).
template <int OBJ, int GRAD>
__global__ void k_objective(P c, D d, const double4_32a *q, const double4_32a *p, double w) {
  constexpr bool grad = GRAD != 0;
  __shared__ double sh[32];
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = tid / kLanes, lane = tid % kLanes;
  double val = 0, ge = 0, gs = 0;
  double gx = 0, gy = 0, gz = 0, u = 0, us = 0, G = 0, Gs = 0;
  if (i < c.n) {
    const double4_32a qi = q[i];
    for (int k = lane; k < d.cnt[i]; k += kLanes) {
      const double4_32a qj = q[d.nbr[(size_t)i * c.cap + k]];
      double dx = qj.x - qi.x, dy = qj.y - qi.y, dz = qj.z - qi.z;
      min_image(c, dx, dy, dz);
      PairTerms t;
      if (!pair_terms(c, dx * dx + dy * dy + dz * dz, t)) continue;
      if (OBJ == 0) {
        u += 0.5 * t.phi;
        us += 0.5 * t.dphis;
        if (grad) {
          gx -= t.f * dx;  // dU/dq_i = -F_i
          gy -= t.f * dy;
          gz -= t.f * dz;
        }
      } else {
        G += 0.5 * t.g;
        Gs += 0.5 * t.gs;
        if (grad) {
          gx += t.gpr * dx;  // dG/dq_i = -sum g'(r) d/r;  dP/dq_i = -(1/3V) dG/dq_i
          gy += t.gpr * dy;
          gz += t.gpr * dz;
        }
      }
    }
  }
  if (grad) {
    gx = lane_sum(gx);
    gy = lane_sum(gy);
    gz = lane_sum(gz);
  }
  if (OBJ == 0) {
    u = lane_sum(u);
    us = lane_sum(us);
  } else {
    G = lane_sum(G);
    Gs = lane_sum(Gs);
  }
  if (i < c.n && lane == 0) {
    const double4_32a pi = p[i];
    const double ke = 0.5 * (pi.x * pi.x + pi.y * pi.y + pi.z * pi.z);
    if (OBJ == 0) {
      const double inv_n = 1.0 / (double)c.n;
      val = u * inv_n;
      ge = u / c.eps * inv_n;
      gs = us * inv_n;
      if (grad) {
        double4_32a a = d.aq[i];
        a.x += w * gx * inv_n;
        a.y += w * gy * inv_n;
        a.z += w * gz * inv_n;
        d.aq[i] = a;
      }
    } else {
      const double inv3v = 1.0 / (3.0 * c.volume);
      val = (2.0 * ke - G) * inv3v;
      ge = -G / c.eps * inv3v;
      gs = -Gs * inv3v;
      if (grad) {
        double4_32a a = d.aq[i], b = d.ap[i];
        a.x += w * gx * inv3v;
        a.y += w * gy * inv3v;
        a.z += w * gz * inv3v;
        b.x += w * 2.0 * pi.x * inv3v;
        b.y += w * 2.0 * pi.y * inv3v;
        b.z += w * 2.0 * pi.z * inv3v;
        d.aq[i] = a;
        d.ap[i] = b;
      }
    }
  }
  const double A = block_sum(val, sh), B = block_sum(ge, sh), E = block_sum(gs, sh);
  partials_accumulate(d, A, B, E, w);
}

// Reverse of one step at half-step positions qh.  In: aq, ap adjoints of
// (q_{n}, p_{n}).  Out: aq, ap adjoints of (q_{n-1}, p_{n-1}); parameter terms
// dt * ap . dF/dtheta into partials (slots 1, 2).
__global__ void k_reverse(P c, D d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < c.n) {
    double4_32a a = d.aq[i], b = d.ap[i];
    // drift q_n = qh + dt/2 p_n : a_p += dt/2 a_q  (done per particle, a_q unchanged)
    b.x += c.dt2 * a.x;
    b.y += c.dt2 * a.y;
    b.z += c.dt2 * a.z;
    d.tmp[i] = b;  // adjoint of p after the kick, needed by the neighbours' H v
    d.aqh[i] = a;
  }
}

__global__ void k_reverse_hvp(P c, D d, const double4_32a *qh) {
  __shared__ double sh[32];
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = tid / kLanes, lane = tid % kLanes;
  double te = 0, ts = 0;
  double hx = 0, hy = 0, hz = 0, fx = 0, fy = 0, fz = 0, sx = 0, sy = 0, sz = 0;
  if (i < c.n) {
    const double4_32a qi = qh[i], vi = d.tmp[i];
    for (int k = lane; k < d.cnt[i]; k += kLanes) {
      const int j = d.nbr[(size_t)i * c.cap + k];
      const double4_32a qj = qh[j], vj = d.tmp[j];
      double dx = qj.x - qi.x, dy = qj.y - qi.y, dz = qj.z - qi.z;
      min_image(c, dx, dy, dz);
      PairTerms t;
      if (!pair_terms(c, dx * dx + dy * dy + dz * dz, t)) continue;
      const double wx = vi.x - vj.x, wy = vi.y - vj.y, wz = vi.z - vj.z;
      const double dw = dx * wx + dy * wy + dz * wz;
      // (H v)_i = sum_j f (v_i - v_j) + (f'/r) d (d . (v_i - v_j))
      hx += t.f * wx + t.fpr * dx * dw;
      hy += t.f * wy + t.fpr * dy * dw;
      hz += t.f * wz + t.fpr * dz * dw;
      fx += t.f * dx;
      fy += t.f * dy;
      fz += t.f * dz;
      sx += t.fs * dx;
      sy += t.fs * dy;
      sz += t.fs * dz;
    }
  }
  hx = lane_sum(hx); hy = lane_sum(hy); hz = lane_sum(hz);
  fx = lane_sum(fx); fy = lane_sum(fy); fz = lane_sum(fz);
  sx = lane_sum(sx); sy = lane_sum(sy); sz = lane_sum(sz);
  if (i < c.n && lane == 0) {
    const double4_32a b = d.tmp[i];
    // parameter terms: dt * a_p . dF_i/deps (= F_i/eps), dt * a_p . dF_i/dsigma
    te = c.dt * (b.x * fx + b.y * fy + b.z * fz) / c.eps;
    ts = c.dt * (b.x * sx + b.y * sy + b.z * sz);
    // kick: a_qh = a_q - dt H a_p ; then drift qh = q + dt/2 p : a_p += dt/2 a_qh
    double4_32a a = d.aqh[i];
    a.x -= c.dt * hx;
    a.y -= c.dt * hy;
    a.z -= c.dt * hz;
    double4_32a pb = b;
    pb.x += c.dt2 * a.x;
    pb.y += c.dt2 * a.y;
    pb.z += c.dt2 * a.z;
    d.aq[i] = a;
    d.ap[i] = pb;
  }
  const double B = block_sum(te, sh), E = block_sum(ts, sh);
  partials_accumulate(d, 0.0, B, E, 1.0);
}

}  // namespace adj
}  // namespace mdg

using namespace mdg::adj;

struct mdg_adjoint {
  mdg_adjoint_params prm;
  std::string err;
  P c;
  D d;
  cudaStream_t s = nullptr;
  int grid = 1;    // one thread per particle
  int gridp = 1;   // kLanes threads per particle (pair kernels)
  int nck = 0;
  bool forward_done = false;
  // the device work of a forward and of a backward pass, captured once and
  // replayed (every pointer is fixed at creation)
  cudaGraphExec_t gx_forward = nullptr, gx_backward = nullptr;
};

namespace {

int afail(mdg_adjoint *a, int code, const std::string &m) {
  if (a) a->err = m;
  return code;
}

#define MDG_ACK(call)                                                                                    \
  do {                                                                                                   \
    cudaError_t e_ = (call);                                                                             \
    if (e_ != cudaSuccess) return afail(a, MDG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

template <class T>
cudaError_t aalloc(T **p, size_t n) {
  *p = nullptr;
  return cudaMalloc((void **)p, (n ? n : 1) * sizeof(T));
}

void launch_objective(mdg_adjoint *a, const double4_32a *q, const double4_32a *p, bool grad, double w) {
  const int obj = a->c.objective;
  if (obj == 0 && !grad) k_objective<0, 0><<<a->gridp, kT, 0, a->s>>>(a->c, a->d, q, p, w);
  else if (obj == 0) k_objective<0, 1><<<a->gridp, kT, 0, a->s>>>(a->c, a->d, q, p, w);
  else if (!grad) k_objective<1, 0><<<a->gridp, kT, 0, a->s>>>(a->c, a->d, q, p, w);
  else k_objective<1, 1><<<a->gridp, kT, 0, a->s>>>(a->c, a->d, q, p, w);
}

// One step from the half-step positions qh (already drifted from step k - 1)
// and p_in: forces, then q_out, p_out and, when given, the next step's qh.
void fwd_step(mdg_adjoint *a, const double4_32a *qh, const double4_32a *p_in, double4_32a *q_out,
              double4_32a *p_out, double4_32a *qh_next) {
  k_force<<<a->gridp, kT, 0, a->s>>>(a->c, a->d, qh, a->d.F);
  k_kick_drift<<<a->grid, kT, 0, a->s>>>(a->c, qh, a->d.F, p_in, q_out, p_out, qh_next);
}

// The horizon from the state in d.q, d.p: per segment its list, per step the
// step and the objective terms, checkpoints every K steps.
int enqueue_forward(mdg_adjoint *a) {
  const size_t N = (size_t)a->c.n, bytes = N * 32;
  D &d = a->d;
  MDG_ACK(cudaMemsetAsync(d.flag, 0, 2 * sizeof(int), a->s));
  MDG_ACK(cudaMemsetAsync(d.acc, 0, 3 * sizeof(double), a->s));
  const int Ns = a->prm.steps, K = a->prm.checkpoint_every;
  const double w = 1.0 / Ns;
  MDG_ACK(cudaMemcpyAsync(d.ckq, d.q, bytes, cudaMemcpyDeviceToDevice, a->s));
  MDG_ACK(cudaMemcpyAsync(d.ckp, d.p, bytes, cudaMemcpyDeviceToDevice, a->s));
  k_drift<<<a->grid, kT, 0, a->s>>>(a->c, d.q, d.p, d.qh);
  for (int n = 1; n <= Ns; n++) {
    if ((n - 1) % K == 0) {  // a checkpoint segment starts: its own list
      MDG_ACK(cudaMemcpyAsync(d.q0, d.q, bytes, cudaMemcpyDeviceToDevice, a->s));
      k_build<<<a->gridp, kT, 0, a->s>>>(a->c, d, d.q);
    }
    fwd_step(a, d.qh, d.p, d.q, d.p, n < Ns ? d.qh : nullptr);
    launch_objective(a, d.q, d.p, false, w);
    if (n % K == 0) {
      MDG_ACK(cudaMemcpyAsync(d.ckq + N * (n / K), d.q, bytes, cudaMemcpyDeviceToDevice, a->s));
      MDG_ACK(cudaMemcpyAsync(d.ckp + N * (n / K), d.p, bytes, cudaMemcpyDeviceToDevice, a->s));
    }
  }
  return cudaGetLastError() == cudaSuccess ? MDG_OK : afail(a, MDG_ERR_CUDA, "adjoint forward launch failed");
}

// Reverse of the horizon, segment by segment from the last: recompute the
// segment from its checkpoint (with the same list), then reverse its steps.
int enqueue_backward(mdg_adjoint *a) {
  const size_t N = (size_t)a->c.n, bytes = N * 32;
  D &d = a->d;
  const int Ns = a->prm.steps, K = a->prm.checkpoint_every;
  const double w = 1.0 / Ns;
  MDG_ACK(cudaMemsetAsync(d.aq, 0, bytes, a->s));
  MDG_ACK(cudaMemsetAsync(d.ap, 0, bytes, a->s));
  MDG_ACK(cudaMemsetAsync(d.acc, 0, 3 * sizeof(double), a->s));
  for (int seg_end = Ns; seg_end > 0;) {
    const int seg_start = ((seg_end - 1) / K) * K;
    const int len = seg_end - seg_start;
    // recompute the segment from its checkpoint: states 0..len, half steps 1..len
    MDG_ACK(cudaMemcpyAsync(d.segq, d.ckq + N * (seg_start / K), bytes, cudaMemcpyDeviceToDevice, a->s));
    MDG_ACK(cudaMemcpyAsync(d.segp, d.ckp + N * (seg_start / K), bytes, cudaMemcpyDeviceToDevice, a->s));
    // the segment's list, built from the same state as in the forward pass
    MDG_ACK(cudaMemcpyAsync(d.q0, d.segq, bytes, cudaMemcpyDeviceToDevice, a->s));
    k_build<<<a->gridp, kT, 0, a->s>>>(a->c, d, d.segq);
    k_drift<<<a->grid, kT, 0, a->s>>>(a->c, d.segq, d.segp, d.segqh + N);
    for (int k = 1; k <= len; k++)
      fwd_step(a, d.segqh + N * k, d.segp + N * (k - 1), d.segq + N * k, d.segp + N * k,
               k < len ? d.segqh + N * (k + 1) : nullptr);
    for (int k = len; k >= 1; k--) {
      // objective terms of state (seg_start + k)
      launch_objective(a, d.segq + N * k, d.segp + N * k, true, w);
      // reverse the step that produced it
      k_reverse<<<a->grid, kT, 0, a->s>>>(a->c, d);
      k_reverse_hvp<<<a->gridp, kT, 0, a->s>>>(a->c, d, d.segqh + N * k);
    }
    seg_end = seg_start;
  }
  return cudaGetLastError() == cudaSuccess ? MDG_OK : afail(a, MDG_ERR_CUDA, "adjoint backward launch failed");
}

// Runs `enqueue` as a CUDA graph captured on first use.
int run_graph(mdg_adjoint *a, cudaGraphExec_t *gx, int (*enqueue)(mdg_adjoint *)) {
  if (!*gx) {
    MDG_ACK(cudaStreamBeginCapture(a->s, cudaStreamCaptureModeThreadLocal));
    const int rc = enqueue(a);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(a->s, &g);
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    MDG_ACK(e);
    const cudaError_t ei = cudaGraphInstantiate(gx, g, 0);
    cudaGraphDestroy(g);
    MDG_ACK(ei);
  }
  MDG_ACK(cudaGraphLaunch(*gx, a->s));
  return MDG_OK;
}

}  // namespace

extern "C" {

void mdg_adjoint_params_default(mdg_adjoint_params *p) {
  if (!p) return;
  memset(p, 0, sizeof(*p));
  p->cutoff = 2.5;
  p->margin = 2.0;
  p->dt = 0.002;
  p->epsilon = 1.0;
  p->sigma = 1.0;
  p->steps = 200;
  p->checkpoint_every = 20;
  p->objective = MDG_OBJ_POTENTIAL;
}

int mdg_adjoint_create(const mdg_adjoint_params *p, int32_t n, mdg_adjoint **out) {
  if (!p || !out || n <= 1 || p->steps <= 0 || p->checkpoint_every <= 0 || !(p->dt > 0) || !(p->epsilon > 0) ||
      !(p->sigma > 0) || (p->objective != MDG_OBJ_POTENTIAL && p->objective != MDG_OBJ_PRESSURE))
    return MDG_ERR_INVALID;
  *out = nullptr;
  const double sl = p->cutoff * p->sigma + p->margin;
  for (int k = 0; k < 3; k++)
    if (!(p->box[k] > 2.0 * sl)) return MDG_ERR_INVALID;
  mdg_adjoint *a = new mdg_adjoint();
  a->prm = *p;
  memset(&a->d, 0, sizeof(a->d));
  P &c = a->c;
  for (int k = 0; k < 3; k++) {
    c.L[k] = p->box[k];
    c.inv_L[k] = 1.0 / p->box[k];
  }
  c.eps = p->epsilon;
  c.sig = p->sigma;
  c.inv_s2 = 1.0 / (p->sigma * p->sigma);
  c.e_s = p->epsilon / p->sigma;
  c.e_s2 = c.e_s / p->sigma;
  c.e_s3 = c.e_s2 / p->sigma;
  c.e_s4 = c.e_s3 / p->sigma;
  c.dt = p->dt;
  c.dt2 = 0.5 * p->dt;
  c.xc2 = p->cutoff * p->cutoff;
  const double s2 = 1.0 / c.xc2, s6 = s2 * s2 * s2, s8 = s6 * s2, s12 = s6 * s6, s14 = s12 * s2;
  c.c2 = 6.0 * s14 - 3.0 * s8;  // variables.cc:16-28 in sigma units
  c.c0 = -s12 + s6 - c.c2 / s2;
  c.sl2 = sl * sl;
  c.sl2f = (sl + 1e-3) * (sl + 1e-3);
  c.half_margin2 = 0.25 * p->margin * p->margin;
  c.volume = p->box[0] * p->box[1] * p->box[2];
  c.n = n;
  c.objective = p->objective;
  const double rho = n / c.volume;
  c.cap = ((int)(rho * 4.18879020478639 * sl * sl * sl * 1.5 + 32) + 7) & ~7;
  a->grid = (n + kT - 1) / kT;
  a->gridp = (int)(((long long)n * kLanes + kT - 1) / kT);
  a->nck = p->steps / p->checkpoint_every + 1;
  const size_t N = (size_t)n, K = (size_t)p->checkpoint_every;
  D &d = a->d;
  cudaError_t e = cudaSetDevice(p->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&a->s, cudaStreamNonBlocking);
  double4_32a **vecs[] = {&d.q, &d.p, &d.qh, &d.F, &d.aq, &d.ap, &d.aqh, &d.tmp, &d.q0};
  for (auto v : vecs)
    if (e == cudaSuccess) e = aalloc(v, N);
  if (e == cudaSuccess) e = aalloc(&d.ckq, N * a->nck);
  if (e == cudaSuccess) e = aalloc(&d.ckp, N * a->nck);
  if (e == cudaSuccess) e = aalloc(&d.segq, N * (K + 1));
  if (e == cudaSuccess) e = aalloc(&d.segp, N * (K + 1));
  if (e == cudaSuccess) e = aalloc(&d.segqh, N * (K + 1));
  if (e == cudaSuccess) e = aalloc(&d.nbr, N * (size_t)c.cap);
  if (e == cudaSuccess) e = aalloc(&d.cnt, N);
  if (e == cudaSuccess) e = aalloc(&d.part, 3 * (size_t)a->gridp);
  if (e == cudaSuccess) e = aalloc(&d.acc, 3);
  if (e == cudaSuccess) e = aalloc(&d.flag, 2);
  if (e == cudaSuccess) e = aalloc(&d.done, 1);
  if (e == cudaSuccess) e = cudaMemset(d.done, 0, sizeof(unsigned int));
  if (e != cudaSuccess) {
    fprintf(stderr, "mdg_adjoint_create: %s\n", cudaGetErrorString(e));
    mdg_adjoint_destroy(a);
    return MDG_ERR_CUDA;
  }
  *out = a;
  return MDG_OK;
}

int mdg_adjoint_destroy(mdg_adjoint *a) {
  if (!a) return MDG_OK;
  cudaSetDevice(a->prm.device);
  if (a->s) cudaStreamSynchronize(a->s);
  if (a->gx_forward) cudaGraphExecDestroy(a->gx_forward);
  if (a->gx_backward) cudaGraphExecDestroy(a->gx_backward);
  D &d = a->d;
  void *ptrs[] = {d.q, d.p, d.qh, d.F, d.aq, d.ap, d.aqh, d.tmp, d.q0, d.ckq, d.ckp, d.segq, d.segp, d.segqh,
                  d.nbr, d.cnt, d.part, d.acc, d.flag, d.done};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  if (a->s) cudaStreamDestroy(a->s);
  delete a;
  return MDG_OK;
}

const char *mdg_adjoint_last_error(const mdg_adjoint *a) { return a ? a->err.c_str() : "null adjoint"; }

int mdg_adjoint_forward(mdg_adjoint *a, const double *q4, const double *p4, double *J) {
  if (!a || !q4 || !p4 || !J) return MDG_ERR_INVALID;
  MDG_ACK(cudaSetDevice(a->prm.device));
  const size_t N = (size_t)a->c.n, bytes = N * 32;
  D &d = a->d;
  MDG_ACK(cudaMemcpyAsync(d.q, q4, bytes, cudaMemcpyHostToDevice, a->s));
  MDG_ACK(cudaMemcpyAsync(d.p, p4, bytes, cudaMemcpyHostToDevice, a->s));
  const int rc = run_graph(a, &a->gx_forward, enqueue_forward);
  if (rc) return rc;
  int flag[2] = {0, 0};
  double acc[3];
  MDG_ACK(cudaMemcpyAsync(acc, d.acc, sizeof acc, cudaMemcpyDeviceToHost, a->s));
  MDG_ACK(cudaMemcpyAsync(flag, d.flag, sizeof flag, cudaMemcpyDeviceToHost, a->s));
  MDG_ACK(cudaStreamSynchronize(a->s));
  if (flag[0]) return afail(a, MDG_ERR_CAPACITY, "adjoint pair list capacity exceeded");
  if (flag[1])
    return afail(a, MDG_ERR_STATE, "a particle moved more than margin/2 within a checkpoint segment; raise margin");
  *J = acc[0];
  a->forward_done = true;
  return MDG_OK;
}

int mdg_adjoint_backward(mdg_adjoint *a, double *dq0, double *dp0, double *deps, double *dsigma) {
  if (!a) return MDG_ERR_INVALID;
  if (!a->forward_done) return afail(a, MDG_ERR_NOT_READY, "run mdg_adjoint_forward first");
  MDG_ACK(cudaSetDevice(a->prm.device));
  const size_t N = (size_t)a->c.n, bytes = N * 32;
  D &d = a->d;
  const int rc = run_graph(a, &a->gx_backward, enqueue_backward);
  if (rc) return rc;
  double acc[3];
  MDG_ACK(cudaMemcpyAsync(acc, d.acc, sizeof acc, cudaMemcpyDeviceToHost, a->s));
  if (dq0) MDG_ACK(cudaMemcpyAsync(dq0, d.aq, bytes, cudaMemcpyDeviceToHost, a->s));
  if (dp0) MDG_ACK(cudaMemcpyAsync(dp0, d.ap, bytes, cudaMemcpyDeviceToHost, a->s));
  MDG_ACK(cudaStreamSynchronize(a->s));
  // acc[1], acc[2]: objective parameter terms (weighted) plus the kick terms
  if (deps) *deps = acc[1];
  if (dsigma) *dsigma = acc[2];
  return MDG_OK;
}

}  // extern "C"
