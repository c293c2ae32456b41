/*
 * CPU oracle for the MDACP Lennard-Jones hot path — TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's single-unit algorithm (one MPI
 * rank, one OpenMP unit whose rectangle is the whole box): ghost images,
 * counting-sort mesh, half-stencil pair search, COO->CSR list, half-list force
 * with Newton's third law, drift-kick-drift stepping, the reference rebuild
 * policy, Langevin / Nose-Hoover thermostats and the observers.  Every
 * function cites the reference file:line it follows.  Only the tests, the
 * smoke check and the benchmark's CPU-baseline leg use it; the GPU library
 * never links or calls it.
 *
 * Pinned against the reference itself: with the same injected state the pair
 * set, forces, observables and a 100-step trajectory are compared with the
 * reference binary built by oracle/build_ref.sh (tests/test_oracle_pin.py and
 * the committed fixtures under tests/golden/).
 */
#ifndef MDACP_ORACLE_H
#define MDACP_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_NVE = 0, ORC_LANGEVIN = 1, ORC_NOSEHOOVER = 2 };
enum { ORC_REBUILD_REFERENCE = 0, ORC_REBUILD_HALFMARGIN = 1 };

typedef struct orc_params {
  double L[3];
  double rc;          /* CUTOFF_LENGTH (mdconfig.h:15) */
  double margin;      /* BufferLength (simulationinfo.cc:6) */
  double dt;          /* TimeStep */
  double gamma;       /* HeatbathGamma */
  double temperature; /* AimedTemperature */
  double tau;         /* HeatbathTau */
  uint64_t seed;      /* Langevin noise stream (Philox4x32-10 key) */
  int thermostat;     /* ORC_NVE / ORC_LANGEVIN / ORC_NOSEHOOVER */
  int rebuild_policy; /* ORC_REBUILD_* */
  int check_list_length;          /* CheckListLength (simulationinfo.cc:27) */
  int langevin_half_drift_compat; /* 1: reference step, no second half-drift */
  int threads;        /* OpenMP threads for the force loop (1 = reference order) */
} orc_params;

typedef struct orc_sys orc_sys;

/* qp: n x 6 doubles {qx,qy,qz,px,py,pz}; particle i gets id i. */
orc_sys *orc_create(const orc_params *prm, int n, const double *qp);
void orc_destroy(orc_sys *s);
/* MDManager::MakePairList (mdmanager.cc:262-280) for one unit. */
void orc_make_pairlist(orc_sys *s);
/* MDManager::Calculate (mdmanager.cc:116-148); returns 1 when the list was rebuilt. */
int orc_calculate(orc_sys *s);
/* Raw KineticEnergy, PotentialEnergy and Virial observer sums (observer.cc:5-79)
 * after a ghost refresh (mdmanager.cc:283-292). */
void orc_observe(orc_sys *s, double out[3]);
/* Forces at the current positions with the current list (p untouched), by id: n x 3. */
void orc_forces(orc_sys *s, double *f);
/* Directed records {key id, partner id, image code} of the half list, code =
 * (sx+1)+3(sy+1)+9(sz+1) for the partner's image.  Returns the count (writes
 * at most cap records). */
long orc_pairs(orc_sys *s, int32_t *rec, long cap);
/* Current real particles by id: n x 6 {q,p}. */
void orc_get_state(orc_sys *s, double *qp);
int orc_particle_count(const orc_sys *s);
int orc_ghost_count(const orc_sys *s);
long orc_rebuild_count(const orc_sys *s);
double orc_zeta(const orc_sys *s);

/* LJ correction constants C0, C2 for cut-off rc (variables.cc:16-28). */
void orc_lj_constants(double rc, double *C0, double *C2);
/* Brute-force directed image pairs within sl of n wrapped positions (meshlist.cc:90-106
 * with periodic images): records {i, j, code}, all ordered pairs.  Returns count. */
long orc_bruteforce_pairs(int n, const double *q3, const double L[3], double sl, int32_t *rec, long cap);
/* The Langevin noise stream shared with the GPU: three standard normals for
 * particle id at Langevin step `step`. */
void orc_langevin_normals(uint64_t seed, uint32_t id, uint64_t step, double z[3]);
/* Philox4x32-10 block (Salmon et al., SC'11). */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

#ifdef __cplusplus
}
#endif
#endif
