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
// states) and then reverses it.  Each checkpoint segment starts by wrapping
// the positions into the box (a shift by whole box lengths: forces, objectives
// and adjoints are unchanged) and has its own pair list (every pair within
// cutoff*sigma + margin at the segment's first state, minimum image), built
// from the same state in both passes; the forward pass verifies that no
// particle moves more than margin/2 within a segment.  A list entry keeps the
// pair's image at the segment's first state, which stays the minimum image of
// every pair within the cut-off for the whole segment (box > 2 (rc + margin)),
// so the pair kernels form the separation with one subtraction per axis
// (from q_i, q_i - L or q_i + L, held per lane) instead of a rounding.  The pair kernels give each particle kLanes lanes and evaluate
// the pair terms in Horner form, without divisions (GB300's FP64 rate is 1/64
// of FP32).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <utility>
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
// Lanes sharing one particle in the list build (a warp: the build's float
// test is light, so it needs many warps per SM to hide its load latency).
constexpr int kBuildLanes = 32;

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
  // coefficients of the pair terms in Horner form (pair_terms)
  double kf6, kf0, kfc, kp6, kp0, ke6, ke0, kec2, kec0, kd6, kd0, kdc, ks6, ks0, ksc;
  double kg6, kg0, kgc, kr6, kr0, krc, kq6, kq0, kqc;
  int n, cap, objective, pad;
};

// A list entry: partner index << kImageBits | per axis two bits r + 1, the
// pair's image being q_j - r L (r in {-1, 0, 1}).
constexpr int kImageBits = 6;
constexpr int kMaxAdjointParticles = 1 << (32 - kImageBits);

struct D {
  double4_32a *q, *q2, *p, *qh, *qh2, *aq, *ap, *aqh, *tmp, *tmp2, *q0;
  double4_32a *ckq, *ckp;    // checkpoints
  float4 *qf;                // float copy of the segment's first state (the list test)
  double4_32a *segq, *segp, *segqh;  // recomputed segment
  uint32_t *nbr;             // the current segment's list, row-major [n][cap]
  int *cnt;
  double *part;              // block partials
  double *acc;               // running sums: J, g_eps, g_sig
  int *flag;
  unsigned int *done;        // blocks of the current reduction that wrote their partials
};

// Particle i's position and its images q_i - L, q_i + L per axis.
struct Home {
  double x, y, z, xm, ym, zm, xp, yp, zp;
};

__device__ __forceinline__ Home make_home(const P &c, const double4_32a &q) {
  return Home{q.x, q.y, q.z, q.x - c.L[0], q.y - c.L[1], q.z - c.L[2], q.x + c.L[0], q.y + c.L[1], q.z + c.L[2]};
}

// The partner of entry e and the separation d = q_j - r L - q_i in the
// entry's image, formed as q_j - (q_i + r L).
__device__ __forceinline__ int pair_sep(uint32_t e, const double4_32a *q, const Home &h, double &dx, double &dy,
                                        double &dz) {
  const int j = (int)(e >> kImageBits);
  const double4_32a qj = q[j];
  const uint32_t ix = e & 3u, iy = (e >> 2) & 3u, iz = (e >> 4) & 3u;
  dx = qj.x - (ix == 1u ? h.x : (ix == 0u ? h.xm : h.xp));
  dy = qj.y - (iy == 1u ? h.y : (iy == 0u ? h.ym : h.yp));
  dz = qj.z - (iz == 1u ? h.z : (iz == 0u ? h.zm : h.zp));
  return j;
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

// With x^2 = r^2 / sigma^2, psi(x) = phi'(x)/x = -48 x^-14 + 24 x^-8 + 8 C2,
// chi(x) = x^2 psi(x):
//   f     = eps/s^2 psi              = x^-8 (kf6 x^-6 + kf0) + kfc
//   fpr   = eps/s^4 psi'(x)/x        = x^-10 (kp6 x^-6 + kp0)
//   phi   = eps phi(x)               = x^-6 (ke6 x^-6 + ke0) + (kec2 x^2 + kec0)
//   dphis = -eps/s x phi'(x)         = x^-6 (kd6 x^-6 + kd0) + kdc x^2
//   fs    = -eps/s^3 (2 psi + x psi'(x))  = x^-8 (ks6 x^-6 + ks0) + ksc
//   g     = eps chi(x)               = x^-6 (kg6 x^-6 + kg0) + kgc x^2
//   gpr   = eps/s^2 chi'(x)/x        = x^-8 (kr6 x^-6 + kr0) + krc
//   gs    = -eps/s x chi'(x)         = x^-6 (kq6 x^-6 + kq0) + kqc x^2
// (coefficients set in mdg_adjoint_create; the kernels keep the terms they use).
__device__ __forceinline__ bool pair_terms(const P &c, double r2, PairTerms &t) {
  const double x2 = r2 * c.inv_s2;
  // x2 >= +0: compared as bit patterns, on the integer pipe (same order)
  if (__double_as_longlong(x2) > __double_as_longlong(c.xc2)) return false;
  const double ix2 = recip(x2), ix4 = ix2 * ix2, ix6 = ix4 * ix2, ix8 = ix4 * ix4, ix10 = ix8 * ix2;
  t.f = fma(ix8, fma(c.kf6, ix6, c.kf0), c.kfc);
  t.fpr = ix10 * fma(c.kp6, ix6, c.kp0);
  t.phi = fma(ix6, fma(c.ke6, ix6, c.ke0), fma(c.kec2, x2, c.kec0));
  t.dphis = fma(ix6, fma(c.kd6, ix6, c.kd0), c.kdc * x2);
  t.fs = fma(ix8, fma(c.ks6, ix6, c.ks0), c.ksc);
  t.g = fma(ix6, fma(c.kg6, ix6, c.kg0), c.kgc * x2);
  t.gpr = fma(ix8, fma(c.kr6, ix6, c.kr0), c.krc);
  t.gs = fma(ix6, fma(c.kq6, ix6, c.kq0), c.kqc * x2);
  return true;
}

// Row i's entries k = lane, lane + kLanes, ...: body(t, dx, dy, dz, j) for
// each pair within the cut-off, in the row's order.
template <class Body>
__device__ __forceinline__ void for_pairs(const P &c, const D &d, int i, int lane, const double4_32a *q,
                                          const Home &h, Body body) {
  const int cnt = d.cnt[i];
  const uint32_t *row = d.nbr + (size_t)i * c.cap;
  for (int k = lane; k < cnt; k += kLanes) {
    double dx, dy, dz;
    const int j = pair_sep(row[k], q, h, dx, dy, dz);
    PairTerms t;
    if (pair_terms(c, dx * dx + dy * dy + dz * dz, t)) body(t, dx, dy, dz, j);
  }
}

// Block sums of three values at once (thread 0 holds them).
__device__ __forceinline__ void block_sum3(double &a, double &b, double &e, double *sh) {
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
    e += __shfl_down_sync(0xffffffffu, e, o);
  }
  if ((threadIdx.x & 31) == 0) {
    sh[3 * (threadIdx.x >> 5)] = a;
    sh[3 * (threadIdx.x >> 5) + 1] = b;
    sh[3 * (threadIdx.x >> 5) + 2] = e;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    a = b = e = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
      a += sh[3 * w];
      b += sh[3 * w + 1];
      e += sh[3 * w + 2];
    }
  }
  __syncthreads();
}

// Writes this block's three partials; the last block of the grid to do so
// adds w times their sums (blocks in a fixed order, so the result does not
// depend on which block finished last) to acc[0..2] and rearms the counter.
// No block waits for another.
__device__ void partials_accumulate(const D &d, double A, double B, double E, double w) {
  __shared__ int last;
  __shared__ double sh2[96];
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
  block_sum3(a, b, e, sh2);
  if (threadIdx.x == 0) {
    d.acc[0] += w * a;
    d.acc[1] += w * b;
    d.acc[2] += w * e;
    *d.done = 0;
  }
}

// Sum over the kLanes lanes that share a particle (all lanes hold the total).
__device__ __forceinline__ double lane_sum(double v) {
#pragma unroll
  for (int o = 1; o < kLanes; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Pair list at positions q (wrapped into the box): every partner within the
// list radius, minimum image.  kBuildLanes lanes share a particle: lane l
// tests partners j = l, l + kBuildLanes, ... (a particle's lanes read
// neighbouring positions together), first counting, then writing at its
// offset in the row (a prefix sum over the lanes), so the row order is fixed:
// lane 0's partners, then lane 1's, ...  The test runs in float against a radius widened by 1e-3
// (float positions of a box of tens of sigma are within 1e-5), so every pair
// within the exact radius is listed; a few more do no harm (the pair terms cut
// at rc).  The float positions come from d.qf (k_wrap writes them), so a
// candidate costs one 16-byte load and no conversions.  The recorded image is
// the double-precision minimum image, r = rint((q_j - q_i) / L) per axis, in
// {-1, 0, 1} for wrapped positions.
__global__ void __launch_bounds__(kT) k_build(P c, D d, const double4_32a *q) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = tid / kBuildLanes, lane = tid % kBuildLanes;
  const bool active = i < c.n;
  float qx = 0.f, qy = 0.f, qz = 0.f;
  if (active) {
    const float4 v = d.qf[i];
    qx = v.x;
    qy = v.y;
    qz = v.z;
  }
  const float lx = (float)c.L[0], ly = (float)c.L[1], lz = (float)c.L[2];
  const float sl2f = (float)c.sl2f;
  // wrapped positions differ by at most L per axis, so the minimum-image
  // separation is min(|d|, L - |d|): no rounding instruction per candidate
  auto within = [&](int j) {
    const float4 v = d.qf[j];
    float ax = fabsf(v.x - qx), ay = fabsf(v.y - qy), az = fabsf(v.z - qz);
    ax = fminf(ax, lx - ax);
    ay = fminf(ay, ly - ay);
    az = fminf(az, lz - az);
    return ax * ax + ay * ay + az * az <= sl2f && j != i;
  };
  int m = 0;
  if (active)
    for (int j = lane; j < c.n; j += kBuildLanes) m += within(j) ? 1 : 0;
  // offsets of the lanes' partners in the row
  int incl = m;
#pragma unroll
  for (int o = 1; o < kBuildLanes; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o, kBuildLanes);
    if (lane >= o) incl += v;
  }
  const int total = __shfl_sync(0xffffffffu, incl, kBuildLanes - 1, kBuildLanes);
  if (active) {
    int w = incl - m;
    uint32_t *row = d.nbr + (size_t)i * c.cap;
    const double4_32a qi = q[i];
    for (int j = lane; j < c.n; j += kBuildLanes)
      if (within(j)) {
        if (w < c.cap) {
          const double4_32a v = q[j];
          const int rx = (int)rint((v.x - qi.x) * c.inv_L[0]), ry = (int)rint((v.y - qi.y) * c.inv_L[1]),
                    rz = (int)rint((v.z - qi.z) * c.inv_L[2]);
          row[w] = ((uint32_t)j << kImageBits) | (uint32_t)(rx + 1) | ((uint32_t)(ry + 1) << 2) |
                   ((uint32_t)(rz + 1) << 4);
        }
        w++;
      }
    if (lane == 0) {
      d.cnt[i] = total < c.cap ? total : c.cap;
      if (total > c.cap) atomicMax(d.flag, total);
    }
  }
}

// One step from the half-step positions q: the forces F there (the lanes of
// a particle), then, by its lane 0, p_out = p_in + F dt, q_out = q + p_out dt/2
// and, when qh_next is given, the next step's first half-drift
// qh_next = q_out + p_out dt/2 (the operations k_drift performs).  Out of
// place: q_out and qh_next must not alias q, which other particles' lanes
// still read; p_out may alias p_in.  Also the segment's displacement check
// (a particle more than margin/2 from where the segment's list was built).
// With VAL = 0 or 1 (the potential-energy or pressure objective) the kernel
// also adds w times the objective's value at the previous whole-step state
// (q_obj, p_in) to acc[0], as k_objective<VAL, 0> does (same row walk, lanes
// and reductions, so the same bits); q_obj must be in this step's segment.
template <int VAL>
__global__ void k_step(P c, D d, const double4_32a *q, const double4_32a *p_in, double4_32a *q_out,
                       double4_32a *p_out, double4_32a *qh_next, const double4_32a *q_obj, double w) {
  __shared__ double sh[96];
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = tid / kLanes, lane = tid % kLanes;
  double fx = 0, fy = 0, fz = 0;
  double u = 0, G = 0;
  double4_32a qi = make_double4_32a(0.0, 0.0, 0.0, 0.0);
  if (i < c.n) {
    qi = q[i];
    if (lane == 0) {
      const double4_32a z = d.q0[i];
      const double ux = qi.x - z.x, uy = qi.y - z.y, uz = qi.z - z.z;
      if (ux * ux + uy * uy + uz * uz > c.half_margin2) atomicMax(d.flag + 1, 1);
    }
    const Home h = make_home(c, qi);
    for_pairs(c, d, i, lane, q, h, [&](const PairTerms &t, double dx, double dy, double dz, int) {
      fx += t.f * dx;
      fy += t.f * dy;
      fz += t.f * dz;
    });
    if (VAL >= 0) {
      const Home ho = make_home(c, q_obj[i]);
      for_pairs(c, d, i, lane, q_obj, ho, [&](const PairTerms &t, double, double, double, int) {
        if (VAL == 0) u += 0.5 * t.phi;
        else G += 0.5 * t.g;
      });
    }
  }
  fx = lane_sum(fx);
  fy = lane_sum(fy);
  fz = lane_sum(fz);
  double val = 0.0;
  if (VAL == 0) u = lane_sum(u);
  if (VAL == 1) G = lane_sum(G);
  if (i < c.n && lane == 0) {
    double4_32a b = p_in[i];
    if (VAL == 0) val = u * (1.0 / (double)c.n);
    if (VAL == 1) val = (2.0 * (0.5 * (b.x * b.x + b.y * b.y + b.z * b.z)) - G) * (1.0 / (3.0 * c.volume));
    b.x += fx * c.dt;
    b.y += fy * c.dt;
    b.z += fz * c.dt;
    p_out[i] = b;
    double4_32a a = qi;
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
  if (VAL >= 0) {
    double none1 = 0.0, none2 = 0.0;
    block_sum3(val, none1, none2, sh);
    partials_accumulate(d, val, 0.0, 0.0, w);
  }
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

// A segment's first state: with wrap, positions into the box, q - k L per
// axis with k = floor(q / L) (particles already inside keep their bits); then
// the float copy for the list test.  The backward pass calls it without wrap
// on the checkpoint the forward pass wrapped.
__global__ void k_wrap(P c, double4_32a *q, float4 *qf, int wrap) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.n) return;
  double4_32a a = q[i];
  if (wrap) {
    const double kx = floor(a.x * c.inv_L[0]), ky = floor(a.y * c.inv_L[1]), kz = floor(a.z * c.inv_L[2]);
    if (kx != 0.0) a.x = fma(-kx, c.L[0], a.x);
    if (ky != 0.0) a.y = fma(-ky, c.L[1], a.y);
    if (kz != 0.0) a.z = fma(-kz, c.L[2], a.z);
    q[i] = a;
  }
  qf[i] = make_float4((float)a.x, (float)a.y, (float)a.z, 0.f);
}

// The reverse of a step's second half-drift q_n = qh + dt/2 p_n for particle
// i, from the adjoints a, b of (q_n, p_n): a_p += dt/2 a_q.  tmp receives the
// adjoint of p after the kick (the neighbours' H v reads it), aqh that of qh.
__device__ __forceinline__ void reverse_drift(const P &c, const D &d, int i, const double4_32a &a, double4_32a b,
                                              double4_32a *tmp) {
  b.x += c.dt2 * a.x;
  b.y += c.dt2 * a.y;
  b.z += c.dt2 * a.z;
  tmp[i] = b;
  d.aqh[i] = a;
}

// Particle i's pair sums of the objective at positions q (every lane holds
// them after the lane sums; all threads of the block call it).
struct ObjSums {
  double u, us, G, Gs, gx, gy, gz;
};

template <int OBJ, bool GRAD>
__device__ __forceinline__ ObjSums objective_sums(const P &c, const D &d, int i, int lane, const double4_32a *q) {
  ObjSums r{0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  if (i < c.n) {
    const Home h = make_home(c, q[i]);
    for_pairs(c, d, i, lane, q, h, [&](const PairTerms &t, double dx, double dy, double dz, int) {
      if (OBJ == 0) {
        r.u += 0.5 * t.phi;
        if (GRAD) {
          r.us += 0.5 * t.dphis;
          r.gx -= t.f * dx;  // dU/dq_i = -F_i
          r.gy -= t.f * dy;
          r.gz -= t.f * dz;
        }
      } else {
        r.G += 0.5 * t.g;
        if (GRAD) {
          r.Gs += 0.5 * t.gs;
          r.gx += t.gpr * dx;  // dG/dq_i = -sum g'(r) d/r;  dP/dq_i = -(1/3V) dG/dq_i
          r.gy += t.gpr * dy;
          r.gz += t.gpr * dz;
        }
      }
    });
  }
  if (GRAD) {
    r.gx = lane_sum(r.gx);
    r.gy = lane_sum(r.gy);
    r.gz = lane_sum(r.gz);
  }
  if (OBJ == 0) {
    r.u = lane_sum(r.u);
    if (GRAD) r.us = lane_sum(r.us);
  } else {
    r.G = lane_sum(r.G);
    if (GRAD) r.Gs = lane_sum(r.Gs);
  }
  return r;
}

// Particle i's objective terms from its sums (lane 0): the value and its
// epsilon and sigma derivatives; with GRAD, w dj/dq added to a and w dj/dp
// to b (the adjoints of the state's q and p).
template <int OBJ, bool GRAD>
__device__ __forceinline__ void objective_finish(const P &c, const ObjSums &r, const double4_32a &pi, double w,
                                                 double &val, double &ge, double &gs, double4_32a &a,
                                                 double4_32a &b) {
  if (OBJ == 0) {
    const double inv_n = 1.0 / (double)c.n;
    val = r.u * inv_n;
    ge = r.u / c.eps * inv_n;
    gs = r.us * inv_n;
    if (GRAD) {
      a.x += w * r.gx * inv_n;
      a.y += w * r.gy * inv_n;
      a.z += w * r.gz * inv_n;
    }
  } else {
    const double ke = 0.5 * (pi.x * pi.x + pi.y * pi.y + pi.z * pi.z);
    const double inv3v = 1.0 / (3.0 * c.volume);
    val = (2.0 * ke - r.G) * inv3v;
    ge = -r.G / c.eps * inv3v;
    gs = -r.Gs * inv3v;
    if (GRAD) {
      a.x += w * r.gx * inv3v;
      a.y += w * r.gy * inv3v;
      a.z += w * r.gz * inv3v;
      b.x += w * 2.0 * pi.x * inv3v;
      b.y += w * 2.0 * pi.y * inv3v;
      b.z += w * 2.0 * pi.z * inv3v;
    }
  }
}

// Objective j at (q, p) into partials (value, d/deps, d/dsigma); with GRAD,
// also adds w * dj/dq and w * dj/dp (w = 1/Ns) to the adjoints aq, ap of
// state n and applies the reverse of step n's second half-drift (into tmp
// and aqh, which k_reverse_hvp takes up).  OBJ and GRAD are
// template parameters so that each pass computes only the pair terms it uses:
// the forward pass returns J alone (the parameter terms of the gradient are
// summed in the backward pass), so without GRAD the sigma derivative is left
// out and its partial is zero.
template <int OBJ, int GRAD>
__global__ void k_objective(P c, D d, const double4_32a *q, const double4_32a *p, double w, double4_32a *tmp) {
  constexpr bool grad = GRAD != 0;
  __shared__ double sh[96];
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = tid / kLanes, lane = tid % kLanes;
  double val = 0, ge = 0, gs = 0;
  const ObjSums r = objective_sums<OBJ, grad>(c, d, i, lane, q);
  if (i < c.n && lane == 0) {
    double4_32a a = make_double4_32a(0.0, 0.0, 0.0, 0.0), b = a;
    if (grad) {
      a = d.aq[i];
      b = d.ap[i];
    }
    objective_finish<OBJ, grad>(c, r, p[i], w, val, ge, gs, a, b);
    if (grad) reverse_drift(c, d, i, a, b, tmp);
  }
  block_sum3(val, ge, gs, sh);
  partials_accumulate(d, val, ge, gs, w);
}

// The rest of the reverse of step n at half-step positions qh (kick and
// first half-drift).  In: tmp (read by the neighbours too) and aqh from the
// reverse of its second half-drift.  Out: aq, ap adjoints of (q_{n-1},
// p_{n-1}); parameter terms dt * ap . dF/dtheta into partials (slots 1, 2).
// With OBJ = 0 or 1 the kernel goes on with state n - 1 (in the same
// segment): its objective terms at (q_obj, p_obj), as k_objective<OBJ, 1>
// computes them, and the reverse of step n - 1's second half-drift, into
// tmp_out (not tmp: other particles' lanes still read it) and aqh instead of
// aq, ap.
template <int OBJ>
__global__ void k_reverse_hvp(P c, D d, const double4_32a *qh, const double4_32a *tmp, const double4_32a *q_obj,
                              const double4_32a *p_obj, double w, double4_32a *tmp_out) {
  __shared__ double sh[96];
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = tid / kLanes, lane = tid % kLanes;
  double te = 0, ts = 0;
  double hx = 0, hy = 0, hz = 0, fx = 0, fy = 0, fz = 0, sx = 0, sy = 0, sz = 0;
  if (i < c.n) {
    const double4_32a qi = qh[i], vi = tmp[i];
    const Home h = make_home(c, qi);
    for_pairs(c, d, i, lane, qh, h, [&](const PairTerms &t, double dx, double dy, double dz, int j) {
      const double4_32a vj = tmp[j];
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
    });
  }
  hx = lane_sum(hx); hy = lane_sum(hy); hz = lane_sum(hz);
  fx = lane_sum(fx); fy = lane_sum(fy); fz = lane_sum(fz);
  sx = lane_sum(sx); sy = lane_sum(sy); sz = lane_sum(sz);
  ObjSums r{};
  if (OBJ >= 0) r = objective_sums<(OBJ >= 0 ? OBJ : 0), true>(c, d, i, lane, q_obj);
  double val = 0, ge = 0, gs = 0;
  if (i < c.n && lane == 0) {
    const double4_32a b = tmp[i];
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
    if (OBJ >= 0) {
      objective_finish<(OBJ >= 0 ? OBJ : 0), true>(c, r, p_obj[i], w, val, ge, gs, a, pb);
      reverse_drift(c, d, i, a, pb, tmp_out);
    } else {
      d.aq[i] = a;
      d.ap[i] = pb;
    }
  }
  // the objective's partials carry the weight w, the kick terms 1
  double A = w * val, B = te + w * ge, E = ts + w * gs;
  block_sum3(A, B, E, sh);
  partials_accumulate(d, A, B, E, 1.0);
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
  int gridb = 1;   // kBuildLanes threads per particle (list build)
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

void launch_objective(mdg_adjoint *a, const double4_32a *q, const double4_32a *p, bool grad, double w,
                      double4_32a *tmp = nullptr) {
  const int obj = a->c.objective;
  if (obj == 0 && !grad) k_objective<0, 0><<<a->gridp, kT, 0, a->s>>>(a->c, a->d, q, p, w, tmp);
  else if (obj == 0) k_objective<0, 1><<<a->gridp, kT, 0, a->s>>>(a->c, a->d, q, p, w, tmp);
  else if (!grad) k_objective<1, 0><<<a->gridp, kT, 0, a->s>>>(a->c, a->d, q, p, w, tmp);
  else k_objective<1, 1><<<a->gridp, kT, 0, a->s>>>(a->c, a->d, q, p, w, tmp);
}

// The reverse of step n (half-step positions qh, tmp from its second
// half-drift's reverse), with, when q_obj is given, the objective terms of
// state n - 1 and the reverse of step n - 1's second half-drift into tmp_out.
void launch_reverse(mdg_adjoint *a, const double4_32a *qh, const double4_32a *tmp, const double4_32a *q_obj,
                    const double4_32a *p_obj, double w, double4_32a *tmp_out) {
  const int obj = a->c.objective;
  if (!q_obj) k_reverse_hvp<-1><<<a->gridp, kT, 0, a->s>>>(a->c, a->d, qh, tmp, nullptr, nullptr, 0.0, nullptr);
  else if (obj == 0) k_reverse_hvp<0><<<a->gridp, kT, 0, a->s>>>(a->c, a->d, qh, tmp, q_obj, p_obj, w, tmp_out);
  else k_reverse_hvp<1><<<a->gridp, kT, 0, a->s>>>(a->c, a->d, qh, tmp, q_obj, p_obj, w, tmp_out);
}

// One step from the half-step positions qh (already drifted from step k - 1)
// and p_in: q_out, p_out and, when given, the next step's qh (not qh itself);
// with q_obj, also w times the objective's value at (q_obj, p_in).
void fwd_step(mdg_adjoint *a, const double4_32a *qh, const double4_32a *p_in, double4_32a *q_out,
              double4_32a *p_out, double4_32a *qh_next, const double4_32a *q_obj = nullptr, double w = 0.0) {
  if (!q_obj)
    k_step<-1><<<a->gridp, kT, 0, a->s>>>(a->c, a->d, qh, p_in, q_out, p_out, qh_next, nullptr, 0.0);
  else if (a->c.objective == 0)
    k_step<0><<<a->gridp, kT, 0, a->s>>>(a->c, a->d, qh, p_in, q_out, p_out, qh_next, q_obj, w);
  else
    k_step<1><<<a->gridp, kT, 0, a->s>>>(a->c, a->d, qh, p_in, q_out, p_out, qh_next, q_obj, w);
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
  // half-step and whole-step positions, both written out of place
  double4_32a *qh = d.qh, *qh_alt = d.qh2, *q = d.q, *q_alt = d.q2;
  for (int n = 1; n <= Ns; n++) {
    if ((n - 1) % K == 0) {  // a checkpoint segment starts: wrapped state, checkpoint, its own list
      const size_t ck = (size_t)((n - 1) / K);
      k_wrap<<<a->grid, kT, 0, a->s>>>(a->c, q, d.qf, 1);
      MDG_ACK(cudaMemcpyAsync(d.ckq + N * ck, q, bytes, cudaMemcpyDeviceToDevice, a->s));
      MDG_ACK(cudaMemcpyAsync(d.ckp + N * ck, d.p, bytes, cudaMemcpyDeviceToDevice, a->s));
      MDG_ACK(cudaMemcpyAsync(d.q0, q, bytes, cudaMemcpyDeviceToDevice, a->s));
      k_build<<<a->gridb, kT, 0, a->s>>>(a->c, d, q);
      k_drift<<<a->grid, kT, 0, a->s>>>(a->c, q, d.p, qh);
    }
    // the next step's half-drift here unless a segment starts there (as the
    // backward pass recomputes it: from the wrapped checkpoint); the
    // objective of state n - 1 rides along when that state is in this
    // step's segment (the states are summed in order either way)
    double4_32a *next = n < Ns && n % K != 0 ? qh_alt : nullptr;
    fwd_step(a, qh, d.p, q_alt, d.p, next, n > 1 && (n - 1) % K != 0 ? q : nullptr, w);
    std::swap(q, q_alt);
    if (next) std::swap(qh, qh_alt);
    // the last state of a segment (or of the horizon) with its own list
    if (n % K == 0 || n == Ns) launch_objective(a, q, d.p, false, w);
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
    k_wrap<<<a->grid, kT, 0, a->s>>>(a->c, d.segq, d.qf, 0);
    k_build<<<a->gridb, kT, 0, a->s>>>(a->c, d, d.segq);
    k_drift<<<a->grid, kT, 0, a->s>>>(a->c, d.segq, d.segp, d.segqh + N);
    for (int k = 1; k <= len; k++)
      fwd_step(a, d.segqh + N * k, d.segp + N * (k - 1), d.segq + N * k, d.segp + N * k,
               k < len ? d.segqh + N * (k + 1) : nullptr);
    // objective terms of the segment's last state and the reverse of the
    // second half-drift of the step that produced it; then per step k the
    // rest of its reverse, going on (k > 1) with the objective terms of
    // state k - 1 and the reverse of step k - 1's second half-drift
    double4_32a *tmp = d.tmp, *tmp_alt = d.tmp2;
    launch_objective(a, d.segq + N * len, d.segp + N * len, true, w, tmp);
    for (int k = len; k >= 1; k--) {
      if (k > 1) {
        launch_reverse(a, d.segqh + N * k, tmp, d.segq + N * (k - 1), d.segp + N * (k - 1), w, tmp_alt);
        std::swap(tmp, tmp_alt);
      } else {
        launch_reverse(a, d.segqh + N * k, tmp, nullptr, nullptr, 0.0, nullptr);
      }
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
  if (n >= kMaxAdjointParticles) return MDG_ERR_INVALID;
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
  const double ep = c.eps;
  c.kf6 = -48.0 * c.e_s2; c.kf0 = 24.0 * c.e_s2; c.kfc = 8.0 * c.c2 * c.e_s2;
  c.kp6 = 672.0 * c.e_s4; c.kp0 = -192.0 * c.e_s4;
  c.ke6 = 4.0 * ep; c.ke0 = -4.0 * ep; c.kec2 = 4.0 * ep * c.c2; c.kec0 = 4.0 * ep * c.c0;
  c.kd6 = 48.0 * c.e_s; c.kd0 = -24.0 * c.e_s; c.kdc = -8.0 * c.c2 * c.e_s;
  c.ks6 = -576.0 * c.e_s3; c.ks0 = 144.0 * c.e_s3; c.ksc = -16.0 * c.c2 * c.e_s3;
  c.kg6 = -48.0 * ep; c.kg0 = 24.0 * ep; c.kgc = 8.0 * ep * c.c2;
  c.kr6 = 576.0 * c.e_s2; c.kr0 = -144.0 * c.e_s2; c.krc = 16.0 * c.c2 * c.e_s2;
  c.kq6 = -576.0 * c.e_s; c.kq0 = 144.0 * c.e_s; c.kqc = -16.0 * c.c2 * c.e_s;
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
  a->gridb = (int)(((long long)n * kBuildLanes + kT - 1) / kT);
  a->nck = p->steps / p->checkpoint_every + 1;
  const size_t N = (size_t)n, K = (size_t)p->checkpoint_every;
  D &d = a->d;
  cudaError_t e = cudaSetDevice(p->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&a->s, cudaStreamNonBlocking);
  double4_32a **vecs[] = {&d.q, &d.q2, &d.p, &d.qh, &d.qh2, &d.aq, &d.ap, &d.aqh, &d.tmp, &d.tmp2, &d.q0};
  for (auto v : vecs)
    if (e == cudaSuccess) e = aalloc(v, N);
  if (e == cudaSuccess) e = aalloc(&d.ckq, N * a->nck);
  if (e == cudaSuccess) e = aalloc(&d.ckp, N * a->nck);
  if (e == cudaSuccess) e = aalloc(&d.segq, N * (K + 1));
  if (e == cudaSuccess) e = aalloc(&d.segp, N * (K + 1));
  if (e == cudaSuccess) e = aalloc(&d.segqh, N * (K + 1));
  if (e == cudaSuccess) e = aalloc(&d.nbr, N * (size_t)c.cap);
  if (e == cudaSuccess) e = aalloc(&d.cnt, N);
  if (e == cudaSuccess) e = aalloc(&d.qf, N);
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
  void *ptrs[] = {d.q, d.q2, d.p, d.qh, d.qh2, d.aq, d.ap, d.aqh, d.tmp, d.tmp2, d.q0, d.ckq, d.ckp, d.segq, d.segp, d.segqh,
                  d.nbr, d.cnt, d.qf, d.part, d.acc, d.flag, d.done};
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
