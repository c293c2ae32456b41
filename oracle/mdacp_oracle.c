/*
 * CPU oracle for the MDACP Lennard-Jones hot path — TEST INFRASTRUCTURE ONLY.
 * See mdacp_oracle.h.  Built with -ffp-contract=off so that every expression
 * rounds exactly as the reference's own (FMA-free) build does; with one
 * thread the results are bitwise those of the reference binary.
 */
#include "mdacp_oracle.h"
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum { D_LEFT, D_RIGHT, D_BACK, D_FORWARD, D_DOWN, D_UP };

struct orc_sys {
  orc_params prm;
  double SL, C0, C2;
  int cap, pn, tn;
  double (*q)[4], (*p)[4];
  int *type;
  int *gsrc, *gdir; /* ghost g >= pn: source slot gsrc[g-pn], direction gdir[g-pn] */
  int *border[6], nborder[6];
  /* mesh (meshlist.h:10-31) */
  double mesh_size[3];
  int mx, my, mz, nmesh;
  int *mesh_count, *mesh_index, *mesh_index2, *particle_position, *sortbuf;
  /* pair list */
  long npairs, pair_cap;
  int *key, *partner, *npartners, *key_pointer, *key_pointer2, *sorted_list;
  int *vbuf;
  /* PairList (pairlist.h:10-25) */
  int initialized;
  double buffer_length;
  double (*qb_old)[4];
  double *disp;
  int *cand;
  long lifetime, rebuilds;
  double zeta;        /* Variables::Zeta */
  uint64_t lstep;     /* Langevin step counter of the noise stream */
  double *tacc;       /* per-thread kick accumulators (threads > 1) */
  int tacc_cap;
};

/* ---------------------------------------------------------------- helpers */
static void *xrealloc(void *p, size_t n) {
  void *r = realloc(p, n ? n : 1);
  if (!r) { fprintf(stderr, "oracle: out of memory\n"); abort(); }
  return r;
}

static void grow_particles(orc_sys *s, int need) {
  if (need <= s->cap) return;
  int nc = need + need / 2 + 1024;
  s->q = xrealloc(s->q, sizeof(double[4]) * nc);
  s->p = xrealloc(s->p, sizeof(double[4]) * nc);
  s->qb_old = xrealloc(s->qb_old, sizeof(double[4]) * nc);
  s->type = xrealloc(s->type, sizeof(int) * nc);
  s->gsrc = xrealloc(s->gsrc, sizeof(int) * nc);
  s->gdir = xrealloc(s->gdir, sizeof(int) * nc);
  s->particle_position = xrealloc(s->particle_position, sizeof(int) * nc);
  s->sortbuf = xrealloc(s->sortbuf, sizeof(int) * nc);
  s->npartners = xrealloc(s->npartners, sizeof(int) * nc);
  s->key_pointer = xrealloc(s->key_pointer, sizeof(int) * nc);
  s->key_pointer2 = xrealloc(s->key_pointer2, sizeof(int) * nc);
  s->vbuf = xrealloc(s->vbuf, sizeof(int) * nc);
  s->disp = xrealloc(s->disp, sizeof(double) * nc);
  s->cand = xrealloc(s->cand, sizeof(int) * nc);
  for (int d = 0; d < 6; d++) s->border[d] = xrealloc(s->border[d], sizeof(int) * nc);
  for (int i = s->cap; i < nc; i++) {
    s->q[i][0] = s->q[i][1] = s->q[i][2] = s->q[i][3] = 0.0;
    s->p[i][0] = s->p[i][1] = s->p[i][2] = s->p[i][3] = 0.0;
  }
  s->cap = nc;
}

/* Variables::Variables (variables.cc:16-28). */
void orc_lj_constants(double rc, double *C0, double *C2) {
  const double s2 = 1.0 / (rc * rc);
  const double s6 = s2 * s2 * s2;
  const double s8 = s6 * s2;
  const double s12 = s6 * s6;
  const double s14 = s12 * s2;
  *C2 = 6.0 * s14 - 3.0 * s8;
  *C0 = -s12 + s6 - *C2 / s2;
}

/* MeshList::ChangeScale (meshlist.cc:31-55) for a unit spanning [0, L). */
static void change_scale(orc_sys *s) {
  int ms[3], m[3];
  for (int d = 0; d < 3; d++) {
    const double w = s->prm.L[d];
    ms[d] = (int)(w / s->SL);
    s->mesh_size[d] = w / (double)ms[d];
    m[d] = (int)(w / s->mesh_size[d]) + 2;
  }
  s->mx = m[0]; s->my = m[1]; s->mz = m[2];
  s->nmesh = s->mx * s->my * s->mz;
  s->mesh_count = xrealloc(s->mesh_count, sizeof(int) * s->nmesh);
  s->mesh_index = xrealloc(s->mesh_index, sizeof(int) * s->nmesh);
  s->mesh_index2 = xrealloc(s->mesh_index2, sizeof(int) * s->nmesh);
}

orc_sys *orc_create(const orc_params *prm, int n, const double *qp) {
  orc_sys *s = calloc(1, sizeof(orc_sys));
  s->prm = *prm;
  if (s->prm.check_list_length <= 0) s->prm.check_list_length = 500;
  if (s->prm.threads <= 0) s->prm.threads = 1;
  s->SL = prm->rc + prm->margin; /* simulationinfo.cc:7 */
  orc_lj_constants(prm->rc, &s->C0, &s->C2);
  grow_particles(s, n + 1024);
  for (int i = 0; i < n; i++) { /* Variables::AddParticle (variables.cc:31-42) */
    s->q[i][0] = qp[6 * i + 0]; s->q[i][1] = qp[6 * i + 1]; s->q[i][2] = qp[6 * i + 2];
    s->p[i][0] = qp[6 * i + 3]; s->p[i][1] = qp[6 * i + 4]; s->p[i][2] = qp[6 * i + 5];
    s->type[i] = i;
  }
  s->pn = s->tn = n;
  change_scale(s);
  return s;
}

void orc_destroy(orc_sys *s) {
  if (!s) return;
  free(s->q); free(s->p); free(s->qb_old); free(s->type); free(s->gsrc); free(s->gdir);
  for (int d = 0; d < 6; d++) free(s->border[d]);
  free(s->mesh_count); free(s->mesh_index); free(s->mesh_index2); free(s->particle_position);
  free(s->sortbuf); free(s->key); free(s->partner); free(s->npartners); free(s->key_pointer);
  free(s->key_pointer2); free(s->sorted_list); free(s->vbuf); free(s->disp); free(s->cand);
  free(s->tacc); free(s);
}

/* ------------------------------------------------- migration and wrapping */
/* MDRect::IsOverBoundary (mdrect.cc:5-22) with s = 0, e = L. */
static int over_boundary(const orc_sys *s, int dir, const double *q) {
  const double *L = s->prm.L;
  switch (dir) {
    case D_LEFT: return q[0] < 0.0;
    case D_RIGHT: return q[0] >= L[0];
    case D_BACK: return q[1] < 0.0;
    case D_FORWARD: return q[1] >= L[1];
    case D_DOWN: return q[2] < 0.0;
    default: return q[2] >= L[2];
  }
}

/* MDManager::SendParticles at one unit (mdmanager.cc:195-259; mdunit.cc:78-122):
 * particles past a face are compacted out and re-appended, then wrapped by
 * Variables::AdjustPeriodicBoundary (variables.cc:59-79).  Returns -1 if a
 * particle is still outside the box. */
static int send_particles(orc_sys *s) {
  int n = s->pn;
  double (*sq)[4] = malloc(sizeof(double[4]) * (n + 1));
  double (*sp)[4] = malloc(sizeof(double[4]) * (n + 1));
  int *st = malloc(sizeof(int) * (n + 1));
  for (int dir = 0; dir < 6; dir++) {
    int index = 0, ns = 0;
    for (int i = 0; i < n; i++) {
      if (over_boundary(s, dir, s->q[i])) {
        memcpy(sq[ns], s->q[i], sizeof(double[4]));
        memcpy(sp[ns], s->p[i], sizeof(double[4]));
        st[ns++] = s->type[i];
      } else {
        s->q[index][0] = s->q[i][0]; s->q[index][1] = s->q[i][1]; s->q[index][2] = s->q[i][2];
        s->p[index][0] = s->p[i][0]; s->p[index][1] = s->p[i][1]; s->p[index][2] = s->p[i][2];
        s->type[index] = s->type[i];
        index++;
      }
    }
    for (int k = 0; k < ns; k++) {
      s->q[index][0] = sq[k][0]; s->q[index][1] = sq[k][1]; s->q[index][2] = sq[k][2];
      s->p[index][0] = sp[k][0]; s->p[index][1] = sp[k][1]; s->p[index][2] = sp[k][2];
      s->type[index] = st[k];
      index++;
    }
  }
  free(sq); free(sp); free(st);
  const double *L = s->prm.L;
  for (int i = 0; i < n; i++)
    for (int d = 0; d < 3; d++) {
      if (s->q[i][d] < 0.0) s->q[i][d] += L[d];
      else if (s->q[i][d] > L[d]) s->q[i][d] -= L[d];
    }
  for (int i = 0; i < n; i++)
    for (int d = 0; d < 3; d++)
      if (s->q[i][d] < 0.0 || s->q[i][d] > L[d]) return -1;
  return 0;
}

/* ------------------------------------------------------------------ ghosts */
/* MDRect::IsInsideEdge (mdrect.cc:24-47) with s = 0, e = L. */
static int inside_edge(const orc_sys *s, int dir, const double *q) {
  const double SL = s->SL, *L = s->prm.L;
  switch (dir) {
    case D_LEFT: return q[0] < 0.0 + SL && q[0] > 0.0;
    case D_RIGHT: return q[0] > L[0] - SL && q[0] < L[0];
    case D_BACK: return q[1] < 0.0 + SL && q[1] > 0.0;
    case D_FORWARD: return q[1] > L[1] - SL && q[1] < L[1];
    case D_DOWN: return q[2] < 0.0 + SL && q[2] > 0.0;
    default: return q[2] > L[2] - SL && q[2] < L[2];
  }
}

/* Image shift of a ghost sent in `dir` (mdunit.cc:137-176): the component
 * along dir is +L (left/back/down) or -L (right/forward/up), others 0. */
static void dir_diff(const orc_sys *s, int dir, double diff[3]) {
  const double *L = s->prm.L;
  diff[0] = diff[1] = diff[2] = 0.0;
  switch (dir) {
    case D_LEFT: diff[0] = L[0]; break;
    case D_RIGHT: diff[0] -= L[0]; break;
    case D_BACK: diff[1] = L[1]; break;
    case D_FORWARD: diff[1] = -L[1]; break;
    case D_DOWN: diff[2] = L[2]; break;
    default: diff[2] = -L[2]; break;
  }
}

/* Ghost creation at a rebuild: FindBorderParticles + MakeBufferForBorderParticles
 * + ReceiveBorderParticles per direction, cascading over ghosts already received
 * (mdmanager.cc:269-275, mdunit.cc:125-191). */
static void find_ghosts(orc_sys *s) {
  s->tn = s->pn;
  for (int dir = 0; dir < 6; dir++) {
    int nb = 0;
    for (int i = 0; i < s->tn; i++)
      if (inside_edge(s, dir, s->q[i])) s->border[dir][nb++] = i;
    s->nborder[dir] = nb;
    double diff[3];
    dir_diff(s, dir, diff);
    grow_particles(s, s->tn + nb + 16);
    for (int k = 0; k < nb; k++) {
      const int j = s->border[dir][k], g = s->tn + k;
      s->q[g][0] = s->q[j][0] + diff[0];
      s->q[g][1] = s->q[j][1] + diff[1];
      s->q[g][2] = s->q[j][2] + diff[2];
      s->gsrc[g - s->pn] = j;
      s->gdir[g - s->pn] = dir;
    }
    s->tn += nb;
  }
}

/* MDManager::SendBorderParticles (mdmanager.cc:283-292): ghost positions are
 * re-derived from the border lists of the last rebuild, in the same order. */
static void refresh_ghosts(orc_sys *s) {
  for (int g = s->pn; g < s->tn; g++) {
    double diff[3];
    dir_diff(s, s->gdir[g - s->pn], diff);
    const int j = s->gsrc[g - s->pn];
    s->q[g][0] = s->q[j][0] + diff[0];
    s->q[g][1] = s->q[j][1] + diff[1];
    s->q[g][2] = s->q[j][2] + diff[2];
  }
}

/* --------------------------------------------------------- mesh and search */
/* MeshList::MakeMesh (meshlist.cc:153-205): cell per particle, counting sort. */
static void make_mesh(orc_sys *s) {
  const int pn = s->tn;
  const double imx = 1.0 / s->mesh_size[0], imy = 1.0 / s->mesh_size[1], imz = 1.0 / s->mesh_size[2];
  for (int i = 0; i < s->nmesh; i++) s->mesh_count[i] = 0;
  for (int i = 0; i < pn; i++) {
    int ix = (int)((s->q[i][0] - 0.0) * imx) + 1;
    int iy = (int)((s->q[i][1] - 0.0) * imy) + 1;
    int iz = (int)((s->q[i][2] - 0.0) * imz) + 1;
    if (ix < 0) ix = s->mx - 1; else if (ix >= s->mx) ix = 0;
    if (iy < 0) iy = s->my - 1; else if (iy >= s->my) iy = 0;
    if (iz < 0) iz = s->mz - 1; else if (iz >= s->mz) iz = 0;
    const int index = s->mx * s->my * iz + s->mx * iy + ix;
    s->particle_position[i] = index;
    s->mesh_count[index]++;
  }
  s->mesh_index[0] = 0;
  int sum = 0;
  for (int i = 0; i < s->nmesh - 1; i++) { sum += s->mesh_count[i]; s->mesh_index[i + 1] = sum; }
  for (int i = 0; i < s->nmesh; i++) s->mesh_index2[i] = 0;
  for (int i = 0; i < pn; i++) {
    const int index = s->particle_position[i];
    s->sortbuf[s->mesh_index[index] + s->mesh_index2[index]++] = i;
  }
}

/* MeshList::RegisterPair (meshlist.cc:287-310). */
static void register_pair(orc_sys *s, int a, int b) {
  const int i1 = a < b ? a : b, i2 = a < b ? b : a;
  if (s->npairs >= s->pair_cap) {
    s->pair_cap = s->pair_cap ? s->pair_cap * 2 : (long)s->tn * 32 + 1024;
    s->key = xrealloc(s->key, sizeof(int) * s->pair_cap);
    s->partner = xrealloc(s->partner, sizeof(int) * s->pair_cap);
  }
  s->key[s->npairs] = i1;
  s->partner[s->npairs] = i2;
  s->npartners[i1]++;
  s->npairs++;
}

/* MeshList::AppendList (meshlist.cc:207-217). */
static int append_cell(const orc_sys *s, int ix, int iy, int iz, int *v, int n) {
  if (ix < 0 || ix >= s->mx || iy < 0 || iy >= s->my || iz < 0 || iz >= s->mz) return n;
  const int index = s->mx * s->my * iz + s->mx * iy + ix;
  const int in = s->mesh_count[index], mi = s->mesh_index[index];
  for (int k = 0; k < in; k++) v[n++] = s->sortbuf[mi + k];
  return n;
}

/* MeshList::SearchMesh (meshlist.cc:219-271): self + 13 half-stencil cells,
 * ghost-ghost pairs skipped, accepted when r2 <= SL^2. */
static void search_mesh(orc_sys *s, int index) {
  static const int st[14][3] = {{0, 0, 0},  {1, 0, 0},   {-1, 1, 0}, {0, 1, 0},  {1, 1, 0},
                                {-1, 0, 1}, {0, 0, 1},   {1, 0, 1},  {-1, -1, 1}, {0, -1, 1},
                                {1, -1, 1}, {-1, 1, 1},  {0, 1, 1},  {1, 1, 1}};
  int ix = index % s->mx, t = index / s->mx;
  int iy = t % s->my, iz = t / s->my;
  int *v = s->vbuf, ln = 0;
  for (int k = 0; k < 14; k++) ln = append_cell(s, ix + st[k][0], iy + st[k][1], iz + st[k][2], v, ln);
  const double S2 = s->SL * s->SL;
  const int pn = s->pn, in = s->mesh_count[index];
  for (int i = 0; i < in; i++) {
    const int i1 = v[i];
    const double x1 = s->q[i1][0], y1 = s->q[i1][1], z1 = s->q[i1][2];
    for (int j = i + 1; j < ln; j++) {
      const int i2 = v[j];
      if (i1 >= pn && i2 >= pn) continue;
      const double dx = x1 - s->q[i2][0];
      const double dy = y1 - s->q[i2][1];
      const double dz = z1 - s->q[i2][2];
      const double r2 = (dx * dx + dy * dy + dz * dz);
      if (r2 > S2) continue;
      register_pair(s, i1, i2);
    }
  }
}

/* MeshList::MakeList (meshlist.cc:57-87): search, then COO -> CSR. */
static void make_list(orc_sys *s) {
  const int pn = s->tn;
  s->npairs = 0;
  for (int i = 0; i < pn; i++) s->npartners[i] = 0;
  make_mesh(s);
  for (int i = 0; i < s->nmesh; i++) search_mesh(s, i);
  int pos = 0;
  s->key_pointer[0] = 0;
  for (int i = 0; i < pn - 1; i++) { pos += s->npartners[i]; s->key_pointer[i + 1] = pos; }
  for (int i = 0; i < pn; i++) s->key_pointer2[i] = 0;
  s->sorted_list = xrealloc(s->sorted_list, sizeof(int) * (s->npairs + 1));
  for (long k = 0; k < s->npairs; k++) {
    const int i = s->key[k];
    s->sorted_list[s->key_pointer[i] + s->key_pointer2[i]++] = s->partner[k];
  }
}

/* PairList::Init (pairlist.cc:11-23). */
static void plist_init(orc_sys *s) {
  s->initialized = 1;
  s->buffer_length = s->prm.margin;
  s->lifetime = 0;
  for (int i = 0; i < s->tn; i++) {
    s->qb_old[i][0] = s->q[i][0]; s->qb_old[i][1] = s->q[i][1]; s->qb_old[i][2] = s->q[i][2];
  }
}

/* MDManager::MakePairList (mdmanager.cc:262-280) -> MDUnit::MakePairList (mdunit.cc:194-198). */
void orc_make_pairlist(orc_sys *s) {
  send_particles(s);
  find_ghosts(s);
  plist_init(s);
  make_list(s);
  s->rebuilds++;
}

/* ------------------------------------------------------------ pair list age */
/* PairList::CheckByDisplacement (pairlist.cc:67-121). */
static int check_by_displacement(orc_sys *s) {
  const int pn = s->tn;
  double dr2_max = 0.0;
  for (int i = 0; i < pn; i++) {
    const double dx = s->qb_old[i][0] - s->q[i][0];
    const double dy = s->qb_old[i][1] - s->q[i][1];
    const double dz = s->qb_old[i][2] - s->q[i][2];
    const double dr2 = dx * dx + dy * dy + dz * dz;
    s->disp[i] = dr2;
    if (dr2_max < dr2) dr2_max = dr2;
  }
  const int cl = s->prm.check_list_length;
  const int Nl = (pn > cl) ? cl : pn;
  const double c_distance = s->prm.margin - sqrt(dr2_max);
  const double c_d2 = c_distance * c_distance;
  int l = 0;
  for (int i = 0; i < pn; i++) {
    if (s->disp[i] > c_d2) {
      s->cand[l++] = i;
      if (l >= Nl) return 1;
    }
  }
  const double SL2 = s->SL * s->SL, CL2 = s->prm.rc * s->prm.rc;
  for (int i = 0; i < l - 1; i++)
    for (int j = i + 1; j < l; j++) {
      const int i1 = s->cand[i], i2 = s->cand[j];
      double dx = s->qb_old[i1][0] - s->qb_old[i2][0];
      double dy = s->qb_old[i1][1] - s->qb_old[i2][1];
      double dz = s->qb_old[i1][2] - s->qb_old[i2][2];
      double dr2 = dx * dx + dy * dy + dz * dz;
      if (dr2 < SL2) continue;
      dx = s->q[i1][0] - s->q[i2][0];
      dy = s->q[i1][1] - s->q[i2][1];
      dz = s->q[i1][2] - s->q[i2][2];
      dr2 = dx * dx + dy * dy + dz * dz;
      if (dr2 < CL2) return 1;
    }
  return 0;
}

/* PairList::IsPairListExpired + UpdatePairListValidity (pairlist.cc:26-65).
 * Returns 1 expired, 0 valid, -1 "too fast particles". */
static int is_pairlist_expired(orc_sys *s) {
  if (!s->initialized) return 1;
  if (s->prm.rebuild_policy == ORC_REBUILD_HALFMARGIN) {
    const double h = 0.5 * s->prm.margin, h2 = h * h;
    for (int i = 0; i < s->pn; i++) {
      const double dx = s->q[i][0] - s->qb_old[i][0];
      const double dy = s->q[i][1] - s->qb_old[i][1];
      const double dz = s->q[i][2] - s->qb_old[i][2];
      if (dx * dx + dy * dy + dz * dz > h2) return 1;
    }
    return 0;
  }
  s->lifetime++;
  if (s->buffer_length > 0.0) {
    const double (*p)[4] = (const double (*)[4])s->p;
    double vmax = p[0][0] * p[0][0] + p[0][1] * p[0][1] + p[0][2] * p[0][2];
    for (int i = 1; i < s->pn; i++) {
      const double v = p[i][0] * p[i][0] + p[i][1] * p[i][1] + p[i][2] * p[i][2];
      if (v > vmax) vmax = v;
    }
    vmax = sqrt(vmax);
    if (vmax * 2.0 * s->prm.dt > s->prm.margin) return -1;
    s->buffer_length = s->buffer_length - vmax * 2.0 * s->prm.dt;
  }
  if (s->buffer_length < 0.0) return check_by_displacement(s);
  return 0;
}

/* ------------------------------------------------------------ integration */
/* ForceCalculator::UpdatePositionHalf (fcalculator.cc:21-32). */
static void update_position_half(orc_sys *s) {
  const double dt2 = s->prm.dt * 0.5;
  for (int i = 0; i < s->pn; i++) {
    s->q[i][0] += s->p[i][0] * dt2;
    s->q[i][1] += s->p[i][1] * dt2;
    s->q[i][2] += s->p[i][2] * dt2;
  }
}

/* ForceCalculator::CalculateForceNext (fcalculator.cc:229-290) / CalculateForceSorted
 * (:182-223): half CSR list, kick df*dx into p[i], reaction into p[j].  The two
 * variants round identically; pairs with r2 > rc^2 contribute nothing.  `out`
 * receives the kicks (p itself for a step). */
static void kick_rows(const orc_sys *s, double (*out)[4], double dt, int i0, int i1) {
  const double CL2 = s->prm.rc * s->prm.rc, C2 = s->C2 * 8.0;
  for (int i = i0; i < i1; i++) {
    const double qx_key = s->q[i][0], qy_key = s->q[i][1], qz_key = s->q[i][2];
    double pfx = 0, pfy = 0, pfz = 0;
    const int kp = s->key_pointer[i], np = s->npartners[i];
    for (int k = kp; k < kp + np; k++) {
      const int j = s->sorted_list[k];
      const double dx = s->q[j][0] - qx_key;
      const double dy = s->q[j][1] - qy_key;
      const double dz = s->q[j][2] - qz_key;
      const double r2 = (dx * dx + dy * dy + dz * dz);
      if (r2 > CL2) continue;
      const double r6 = r2 * r2 * r2;
      const double df = ((24.0 * r6 - 48.0) / (r6 * r6 * r2) + C2) * dt;
      pfx += df * dx; pfy += df * dy; pfz += df * dz;
      out[j][0] -= df * dx; out[j][1] -= df * dy; out[j][2] -= df * dz;
    }
    out[i][0] += pfx; out[i][1] += pfy; out[i][2] += pfz;
  }
}

static void apply_kicks(orc_sys *s, double (*out)[4], double dt) {
  const int T = s->prm.threads;
  if (T <= 1) { kick_rows(s, out, dt, 0, s->pn); return; }
#ifdef _OPENMP
  /* Timing-only path: per-thread reaction buffers, summed afterwards. */
  const int tn = s->tn;
  if (s->tacc_cap < tn * T) {
    s->tacc = xrealloc(s->tacc, sizeof(double[4]) * (size_t)tn * T);
    s->tacc_cap = tn * T;
  }
#pragma omp parallel num_threads(T)
  {
    const int t = omp_get_thread_num();
    double (*acc)[4] = (double (*)[4])(s->tacc + (size_t)4 * tn * t);
    memset(acc, 0, sizeof(double[4]) * tn);
    const int chunk = (s->pn + T - 1) / T, a = t * chunk, b = a + chunk < s->pn ? a + chunk : s->pn;
    if (a < b) kick_rows(s, acc, dt, a, b);
#pragma omp barrier
#pragma omp for schedule(static)
    for (int i = 0; i < s->pn; i++)
      for (int u = 0; u < T; u++) {
        const double *a4 = s->tacc + (size_t)4 * tn * u + 4 * i;
        out[i][0] += a4[0]; out[i][1] += a4[1]; out[i][2] += a4[2];
      }
  }
#else
  kick_rows(s, out, dt, 0, s->pn);
#endif
}

/* ForceCalculator::HeatbathZeta / HeatbathMomenta (fcalculator.cc:743-762). */
static double kinetic_sum(const orc_sys *s) {
  double e = 0.0;
  for (int i = 0; i < s->pn; i++)
    for (int d = 0; d < 4; d++) e += 0.5 * s->p[i][d] * s->p[i][d];
  return e;
}
static void heatbath_zeta(orc_sys *s, double t) {
  const double dt2 = s->prm.dt * 0.5, tau = s->prm.tau;
  const double t1 = (t - s->prm.temperature) / (tau * tau);
  s->zeta += t1 * dt2;
}
static void heatbath_momenta(orc_sys *s) {
  const double dt2 = s->prm.dt * 0.5;
  const double exp1 = exp(-dt2 * s->zeta);
  for (int i = 0; i < s->pn; i++)
    for (int d = 0; d < 4; d++) s->p[i][d] *= exp1;
}

/* ---------------------------------------------------- Langevin noise stream */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3], k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; r++) {
    if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
    const uint64_t m0 = (uint64_t)0xD2511F53u * c0, m1 = (uint64_t)0xCD9E8D57u * c2;
    const uint32_t hi0 = (uint32_t)(m0 >> 32), lo0 = (uint32_t)m0;
    const uint32_t hi1 = (uint32_t)(m1 >> 32), lo1 = (uint32_t)m1;
    c0 = hi1 ^ c1 ^ k0; c1 = lo1; c2 = hi0 ^ c3 ^ k1; c3 = lo0;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* Box-Muller on 24-bit uniforms, single precision (the GPU evaluates the same
 * formula with its own logf/sinf/cosf). */
void orc_langevin_normals(uint64_t seed, uint32_t id, uint64_t step, double z[3]) {
  const uint32_t ctr[4] = {id, (uint32_t)step, (uint32_t)(step >> 32), 0x4C4A4D44u};
  const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t r[4];
  orc_philox4x32_10(ctr, key, r);
  const float s24 = 5.9604644775390625e-08f; /* 2^-24 */
  const float u1 = (float)((r[0] >> 8) + 1u) * s24, u2 = (float)(r[1] >> 8) * s24;
  const float u3 = (float)((r[2] >> 8) + 1u) * s24, u4 = (float)(r[3] >> 8) * s24;
  const float twopi = 6.28318530717958647692f;
  const float ra = sqrtf(-2.0f * logf(u1)), rb = sqrtf(-2.0f * logf(u3));
  z[0] = (double)(ra * cosf(twopi * u2));
  z[1] = (double)(ra * sinf(twopi * u2));
  z[2] = (double)(rb * cosf(twopi * u4));
}

/* ForceCalculator::Langevin (fcalculator.cc:764-778) with the shared stream. */
static void langevin(orc_sys *s) {
  const double dt = s->prm.dt, g = s->prm.gamma, T = s->prm.temperature;
  const double hb_D = sqrt(2.0 * g * T / dt);
  for (int i = 0; i < s->pn; i++) {
    double z[3];
    orc_langevin_normals(s->prm.seed, (uint32_t)s->type[i], s->lstep, z);
    s->p[i][0] += (-g * s->p[i][0] + hb_D * z[0]) * dt;
    s->p[i][1] += (-g * s->p[i][1] + hb_D * z[1]) * dt;
    s->p[i][2] += (-g * s->p[i][2] + hb_D * z[2]) * dt;
  }
  s->lstep++;
}

/* MDManager::Calculate (mdmanager.cc:116-148) with CalculateForce (:151-157),
 * CalculateNoseHoover (:160-175) and CalculateLangevin (:186-192). */
int orc_calculate(orc_sys *s) {
  const int e = is_pairlist_expired(s);
  if (e < 0) return -1;
  if (e) orc_make_pairlist(s);
  update_position_half(s);
  refresh_ghosts(s);
  const double dt = s->prm.dt;
  if (s->prm.thermostat == ORC_NOSEHOOVER) {
    double t = kinetic_sum(s) / (double)s->pn / 1.5;
    heatbath_zeta(s, t);
    heatbath_momenta(s);
    apply_kicks(s, s->p, dt);
    heatbath_momenta(s);
    t = kinetic_sum(s) / (double)s->pn / 1.5;
    heatbath_zeta(s, t);
    update_position_half(s);
  } else if (s->prm.thermostat == ORC_LANGEVIN) {
    apply_kicks(s, s->p, dt);
    langevin(s);
    if (!s->prm.langevin_half_drift_compat) update_position_half(s);
  } else {
    apply_kicks(s, s->p, dt);
    update_position_half(s);
  }
  return e ? 1 : 0;
}

/* ------------------------------------------------------------- observers */
void orc_observe(orc_sys *s, double out[3]) {
  refresh_ghosts(s);
  out[0] = kinetic_sum(s); /* KineticEnergyObserver (observer.cc:5-15) */
  const double CL2 = s->prm.rc * s->prm.rc, C2 = s->C2, C0 = s->C0;
  const int pn = s->pn;
  double energy = 0.0, phi = 0.0;
  for (long k = 0; k < s->npairs; k++) { /* PotentialEnergyObserver (observer.cc:17-48) */
    const int i = s->key[k], j = s->partner[k];
    const double dx = s->q[i][0] - s->q[j][0];
    const double dy = s->q[i][1] - s->q[j][1];
    const double dz = s->q[i][2] - s->q[j][2];
    const double r2 = (dx * dx + dy * dy + dz * dz);
    if (r2 > CL2) continue;
    double e = 4.0 * (1.0 / (r2 * r2 * r2 * r2 * r2 * r2) - 1.0 / (r2 * r2 * r2) + C2 * r2 + C0);
    if (i >= pn || j >= pn) e *= 0.5;
    energy += e;
  }
  for (long k = 0; k < s->npairs; k++) { /* VirialObserver (observer.cc:50-79) */
    const int i = s->key[k], j = s->partner[k];
    const double dx = s->q[j][0] - s->q[i][0];
    const double dy = s->q[j][1] - s->q[i][1];
    const double dz = s->q[j][2] - s->q[i][2];
    const double r2 = (dx * dx + dy * dy + dz * dz);
    if (r2 > CL2) continue;
    const double r6 = r2 * r2 * r2;
    double df = ((24.0 * r6 - 48.0) / (r6 * r6 * r2) + C2 * 8.0) * r2;
    if (i >= pn || j >= pn) df *= 0.5;
    phi += df;
  }
  out[1] = energy;
  out[2] = phi / 3.0;
}

void orc_forces(orc_sys *s, double *f) {
  refresh_ghosts(s);
  double (*acc)[4] = calloc((size_t)s->tn, sizeof(double[4]));
  const int T = s->prm.threads;
  s->prm.threads = 1;
  apply_kicks(s, acc, 1.0);
  s->prm.threads = T;
  for (int i = 0; i < s->pn; i++) {
    const int id = s->type[i];
    f[3 * id + 0] = acc[i][0]; f[3 * id + 1] = acc[i][1]; f[3 * id + 2] = acc[i][2];
  }
  free(acc);
}

static int resolve_ghost(const orc_sys *s, int g, int *code) {
  int sh[3] = {0, 0, 0};
  while (g >= s->pn) {
    const int dir = s->gdir[g - s->pn];
    const int axis = dir / 2, sign = (dir % 2 == 0) ? 1 : -1;
    sh[axis] += sign;
    g = s->gsrc[g - s->pn];
  }
  *code = (sh[0] + 1) + 3 * (sh[1] + 1) + 9 * (sh[2] + 1);
  return g;
}

long orc_pairs(orc_sys *s, int32_t *rec, long cap) {
  for (long k = 0; k < s->npairs && k < cap; k++) {
    int code = 13;
    const int a = s->key[k], b = resolve_ghost(s, s->partner[k], &code);
    rec[3 * k + 0] = s->type[a];
    rec[3 * k + 1] = s->type[b];
    rec[3 * k + 2] = code;
  }
  return s->npairs;
}

void orc_get_state(orc_sys *s, double *qp) {
  for (int i = 0; i < s->pn; i++) {
    const int id = s->type[i];
    for (int d = 0; d < 3; d++) { qp[6 * id + d] = s->q[i][d]; qp[6 * id + 3 + d] = s->p[i][d]; }
  }
}

int orc_particle_count(const orc_sys *s) { return s->pn; }
int orc_ghost_count(const orc_sys *s) { return s->tn - s->pn; }
long orc_rebuild_count(const orc_sys *s) { return s->rebuilds; }
double orc_zeta(const orc_sys *s) { return s->zeta; }

/* All directed image pairs by brute force: the partner's image j + code*L is
 * formed first and then subtracted, as the ghost path does (mdunit.cc:167,
 * meshlist.cc:262-266).  Independent of the mesh. */
long orc_bruteforce_pairs(int n, const double *q3, const double L[3], double sl, int32_t *rec, long cap) {
  const double S2 = sl * sl;
  long m = 0;
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      for (int c = 0; c < 27; c++) {
        const int sx = c % 3 - 1, sy = (c / 3) % 3 - 1, sz = c / 9 - 1;
        if (i == j && c == 13) continue;
        const double xj = q3[3 * j + 0] + (sx ? sx * L[0] : 0.0);
        const double yj = q3[3 * j + 1] + (sy ? sy * L[1] : 0.0);
        const double zj = q3[3 * j + 2] + (sz ? sz * L[2] : 0.0);
        const double dx = q3[3 * i + 0] - xj, dy = q3[3 * i + 1] - yj, dz = q3[3 * i + 2] - zj;
        const double r2 = (dx * dx + dy * dy + dz * dz);
        if (r2 > S2) continue;
        if (m < cap) { rec[3 * m] = i; rec[3 * m + 1] = j; rec[3 * m + 2] = c; }
        m++;
      }
  return m;
}
