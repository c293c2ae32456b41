/*
 * mdg — GB300-native Lennard-Jones short-range engine behind MDACP's call points.
 *
 * C ABI of libmdg.so.  Plain pointers and sizes only.  One handle is one
 * periodic box (one MDACP unit spanning the whole system, as `mpirun -np 1`
 * with one OpenMP unit runs it); it owns all device memory and one CUDA
 * stream.  Every call returns MDG_OK (0) or an error code; mdg_last_error()
 * returns the message of the last failure on that handle, and
 * mdg_last_error(NULL) why the calling thread's last mdg_create failed.  A handle must be
 * used by one host thread at a time.
 *
 * Particle arrays cross the boundary in the reference's layout: `double
 * [n][4]` with the fourth lane as padding (Variables::q / Variables::p,
 * variables.h:16-18), indexed by the caller's particle order: the lane is
 * ignored on input (it never enters the kinetic energy) and returned as
 * zero.  Internally particles are kept sorted by cell; results are returned
 * in the caller's order.
 *
 * Physics (reference semantics): the smoothly truncated LJ potential
 * V(r) = 4(r^-12 - r^-6 + C2 r^2 + C0) with eps = sigma = m = 1 and C0, C2 from
 * the cut-off (variables.cc:16-28); drift-kick-drift stepping
 * (mdmanager.cc:116-157); Langevin without the second half-drift unless
 * langevin_half_drift_compat = 0 (mdmanager.cc:186-192); Nose-Hoover as
 * mdmanager.cc:160-175.  Pair list: every image pair within rc + margin of a
 * particle, formed as the reference forms its ghost pairs (image position
 * first, then the difference; mdunit.cc:167, meshlist.cc:262-266).  A list is
 * rebuilt when a particle has moved more than margin/2 since the last build.
 */
#ifndef MDG_H
#define MDG_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

#define MDG_OK 0
#define MDG_ERR_INVALID 1      /* bad argument or parameter */
#define MDG_ERR_CUDA 2         /* CUDA runtime error */
#define MDG_ERR_CAPACITY 3     /* more particles than the handle's capacity */
#define MDG_ERR_STATE 4        /* non-finite or escaped particle coordinate */
#define MDG_ERR_NOT_READY 5    /* no state loaded */

/* MDG_FP64: the reference's arithmetic.  MDG_MIXED: pair distance and force
 * in FP32 from cell-local positions, per-particle force sums in compensated
 * (Kahan) FP32, positions, momenta, displacement and the energy/virial
 * reductions in FP64.  MDG_MIXED_PLAIN: as MDG_MIXED with plain FP32 force
 * sums (kept for comparison). */
enum mdg_precision { MDG_FP64 = 0, MDG_MIXED = 1, MDG_MIXED_PLAIN = 2 };
enum mdg_thermostat { MDG_NVE = 0, MDG_LANGEVIN = 1, MDG_NOSEHOOVER = 2 };

/* When the pair list is rebuilt (.cfg RebuildPolicy).  HALFMARGIN: as soon
 * as a particle has moved more than half the margin since the build.
 * REFERENCE: PairList::IsPairListExpired (pairlist.cc:26-121): a buffer
 * budget reduced by 2 max|p| dt each step and, once it is spent, the
 * displacement check of at most check_list_length candidates; a step with
 * 2 max|p| dt above the margin fails with MDG_ERR_STATE ("too fast
 * particles", the reference's abort). */
enum mdg_rebuild_policy { MDG_REBUILD_HALFMARGIN = 0, MDG_REBUILD_REFERENCE = 1 };

typedef struct mdg_params {
  int32_t capacity;        /* maximum particles (Variables N, mdconfig.h:11) */
  int32_t precision;       /* mdg_precision (.cfg Precision=fp64|mixed|mixed_plain) */
  double box[3];           /* SystemSizeX/Y/Z (simulationinfo.cc:38-57) */
  double cutoff;           /* CutoffLength; CUTOFF_LENGTH (mdconfig.h:15) */
  double margin;           /* BufferLength (simulationinfo.cc:6) */
  double dt;               /* TimeStep */
  int32_t thermostat;      /* mdg_thermostat (ControlTemperature + HeatbathType) */
  int32_t langevin_half_drift_compat; /* LangevinHalfDriftCompat, 1 = reference */
  double temperature;      /* AimedTemperature */
  double gamma;            /* HeatbathGamma */
  double tau;              /* HeatbathTau */
  uint64_t seed;           /* Seed of the Langevin noise stream */
  int32_t list_capacity;   /* neighbour slots per particle; 0 = sized from the first build */
  int32_t device;          /* CUDA device ordinal */
  int32_t use_graphs;      /* 1 = replay steps as CUDA graphs */
  int32_t rebuild_policy;  /* mdg_rebuild_policy (.cfg RebuildPolicy), default HALFMARGIN */
  double prune_buffer;     /* inner-list buffer: the force kernels walk the pairs within
                              cutoff + prune_buffer, re-selected from the list whenever a
                              particle moved prune_buffer/2 (default -1 = automatic,
                              min(0.1, margin / 2); 0 keeps every listed pair) */
  int32_t check_list_length; /* CheckListLength (simulationinfo.cc:27): the reference
                                policy's candidate limit, default 500 */
  int32_t reserved;
} mdg_params;

typedef struct mdg_stats {
  int64_t steps;           /* steps advanced since the last mdg_set_state */
  int64_t rebuilds;        /* pair-list builds since the last mdg_set_state */
  int32_t list_capacity;   /* current neighbour slots per particle */
  int32_t max_neighbours;  /* largest row at the last build */
  int64_t listed_pairs;    /* directed pairs in the current list */
  int32_t cells[3];        /* cell grid */
  int32_t particles;
  double zeta;             /* Nose-Hoover friction (Variables::Zeta) */
  double elapsed_ms;       /* device time of the steps of the last mdg_calculate call with
                              nsteps > 1; after single-step calls, from the first of them to
                              their confirmation */
  int64_t kernel_launches; /* kernels this handle has enqueued (graph replays count each node) */
  int64_t inner_pairs;     /* directed pairs in the inner list at the last prune */
  int64_t prunes;          /* inner-list selections since the last mdg_set_state */
} mdg_stats;

typedef struct mdg_handle mdg_handle;

/* Library version string. */
const char *mdg_version(void);
/* Fills *p with the reference defaults (rc 3.0, margin 0.3, dt 0.001, NVE, ...). */
void mdg_params_default(mdg_params *p);

/* Replaces MDManager construction (mdmanager.cc:11-47) for one box on one GPU. */
int mdg_create(const mdg_params *p, mdg_handle **out);
int mdg_destroy(mdg_handle *h);
const char *mdg_last_error(const mdg_handle *h);

/* Replaces MDUnit::AddParticle / Variables::q,p filling (mdunit.cc:35-49,
 * variables.cc:31-42): n particles, q4/p4 host arrays [n][4].  Resets the step
 * and rebuild counters and the Langevin stream position. */
int mdg_set_state(mdg_handle *h, const double *q4, const double *p4, int32_t n);
/* Copies the current state back in the caller's order; either pointer may be NULL.
 * Positions are those of the reference at the same point: wrapped at the last
 * rebuild only (variables.cc:59-79). */
int mdg_get_state(mdg_handle *h, double *q4, double *p4);

/* Replaces MDManager::MakePairList (mdmanager.cc:262-280): wrap, bin, build. */
int mdg_make_pairlist(mdg_handle *h);
/* Replaces nsteps calls of MDManager::Calculate (mdmanager.cc:116-148).
 * The steps are enqueued on the handle's stream and the call returns without
 * waiting until 1024 steps are outstanding.  Every other call on the handle
 * first waits for them and confirms them: a list overflow is recovered there
 * (rows regrown, the steps behind it run again), and a particle found outside
 * the box at a rebuild is reported there as MDG_ERR_STATE (the steps after it
 * do nothing).  mdg_set_state and mdg_make_state discard that report. */
int mdg_calculate(mdg_handle *h, int32_t nsteps);
/* Waits for and confirms the steps mdg_calculate left outstanding. */
int mdg_synchronize(mdg_handle *h);
/* mdg_calculate with a CUDA event pair around every step kernel: the steps
 * replay the same step graph as mdg_calculate with event-record nodes added
 * (plain launches with events when use_graphs = 0), and the call waits for
 * them.  *step_kernel_ms receives the summed device time of the step kernels
 * (for roofline accounting). */
int mdg_calculate_profiled(mdg_handle *h, int32_t nsteps, double *step_kernel_ms);
/* The phase times of the reference's StopWatch objects (mdmanager.cc:117-147,
 * stopwatch.h:8-37) for nsteps steps run as in mdg_calculate_profiled:
 * phase_ms[0] = the fused step kernels (force, kick, drifts; "force"),
 * phase_ms[1] = the rebuild sequences (wrap, bin, sort, list build; "pair"),
 * phase_ms[2] = the whole run ("all"), device milliseconds. */
int mdg_calculate_phases(mdg_handle *h, int32_t nsteps, double phase_ms[3]);
/* Replaces KineticEnergyObserver, PotentialEnergyObserver and VirialObserver
 * (observer.cc:5-79) at the current positions: out[0] = sum p^2/2,
 * out[1] = sum of pair energies, out[2] = sum of pair virials / 3. */
int mdg_observe(mdg_handle *h, double out[3]);
/* Forces at the current positions in the handle's precision, caller's order,
 * host [n][4] (ForceCalculator::CalculateForce with p = 0 and dt = 1,
 * fcalculator.cc:35-50). */
int mdg_forces(mdg_handle *h, double *f4);
/* Directed pairs of the current list: rec[3k..3k+2] = {i, j, image code} with
 * code = (sx+1) + 3(sy+1) + 9(sz+1) for the image j + (sx,sy,sz) L of j
 * (the pair set MeshList::SearchMesh registers, meshlist.cc:219-271, both
 * directions).  *count receives the total; at most cap records are written. */
int mdg_pairs(mdg_handle *h, int32_t *rec, int64_t cap, int64_t *count);

/* MDManager::SetSeed (mdmanager.cc:177-183). */
int mdg_set_seed(mdg_handle *h, uint64_t seed);
/* MDManager::SetControlTemperature / SetAimedTemperature (mdmanager.h:77-78)
 * and HeatbathType: thermostat = mdg_thermostat. */
int mdg_set_thermostat(mdg_handle *h, int32_t thermostat, double temperature);
int mdg_get_stats(mdg_handle *h, mdg_stats *s);

/* Device-resident state exchange on the handle's stream (caller-owned device
 * buffers, [n][4] doubles, caller's order). */
int mdg_set_state_device(mdg_handle *h, const double *q4_dev, const double *p4_dev, int32_t n);
int mdg_get_state_device(mdg_handle *h, double *q4_dev, double *p4_dev);

/* ------------------------------------------------------------------------
 * Batched replicas (no reference counterpart; a pattern on top of the
 * drop-in): nbox independent periodic boxes of uneven size and density, each
 * an NVE drift-kick-drift run with its own cell list and Verlet list, all
 * advanced by one persistent kernel per step (replayed from a CUDA graph).
 * Particles are concatenated box after box, [sum n][4] doubles; every box is
 * returned in the order it was given. */
typedef struct mdg_batch_params {
  int32_t precision;      /* mdg_precision */
  int32_t device;
  double cutoff;          /* rc */
  double margin;          /* list margin */
  double dt;
  int32_t list_capacity;  /* neighbour slots per particle; 0 = from the densest box */
  int32_t use_graphs;
  double prune_buffer;    /* inner-list buffer (one lane per particle): the step walks the listed
                             pairs within rc + buffer; negative = min(0.1, margin / 2) (default),
                             0 = walk every listed pair */
} mdg_batch_params;

typedef struct mdg_batch_stats {
  int64_t steps;              /* steps every box has advanced */
  int64_t rebuilds;           /* list builds summed over boxes */
  int64_t particles;
  int32_t boxes;
  int32_t list_capacity;
  int32_t threads;            /* CTA size of the persistent kernel */
  int32_t lanes_per_particle; /* lanes sharing one particle's row */
  int32_t ctas_per_sm;
  int32_t inner_list;         /* 1: the step walks the inner list (chosen by mdg_batch_tune) */
  double elapsed_ms;          /* device time of the last mdg_batch_calculate */
  int64_t kernel_launches;
  int32_t flat;               /* 1: flat layout (see mdg_batch_set_flat) */
  int32_t reserved;
  double prune_buffer;        /* inner-list buffer in use (mdg_batch_tune may pick margin / 2
                                 when the parameters left it automatic); 0 without inner list */
} mdg_batch_stats;

typedef struct mdg_batch mdg_batch;

void mdg_batch_params_default(mdg_batch_params *p);
/* box_lengths: nbox x 3 box sides; each side must exceed 2 (cutoff + margin). */
int mdg_batch_create(const mdg_batch_params *p, int32_t nbox, const int32_t *n_per_box, const double *box_lengths,
                     mdg_batch **out);
int mdg_batch_destroy(mdg_batch *b);
const char *mdg_batch_last_error(const mdg_batch *b);
int mdg_batch_set_state(mdg_batch *b, const double *q4, const double *p4);
int mdg_batch_get_state(mdg_batch *b, double *q4, double *p4);
int mdg_batch_calculate(mdg_batch *b, int32_t nsteps);
/* out: nbox x 3 observer sums (as mdg_observe) at the current positions. */
int mdg_batch_observe(mdg_batch *b, double *out);
/* Autotuner: times trial_steps for every (threads per CTA, lanes per particle,
 * CTAs per SM) shape whose CTAs are all resident at once (occupancy of the
 * step kernel that shape runs) from a copy of the current state, keeps the
 * fastest, and restores the state. */
int mdg_batch_tune(mdg_batch *b, int32_t trial_steps, int32_t *threads, int32_t *lanes_per_particle,
                   int32_t *ctas_per_sm);
/* Fixes the shape by hand; ctas_per_sm is capped at the CTAs of the step
 * kernel that fit on one SM at once (mdg_batch_get_stats reports the value
 * used), so the persistent kernel never runs in waves. */
int mdg_batch_set_shape(mdg_batch *b, int32_t threads, int32_t lanes_per_particle, int32_t ctas_per_sm);
/* Whether one lane per particle walks the inner list (1, the default when the
 * buffer is > 0) or every listed pair (0); mdg_batch_tune chooses it too. */
int mdg_batch_set_inner(mdg_batch *b, int32_t on);
/* Layout of the persistent step kernel: 0 (default) = each CTA steps the
 * boxes assigned to it in turn; 1 = flat: the resident CTAs stride over the
 * particles of all boxes, one thread per particle, and a small per-box kernel
 * after the step applies the boxes' rebuild and re-selection requests.  The
 * flat layout takes one lane per particle and at most 256 threads per CTA;
 * mdg_batch_tune times both layouts. */
int mdg_batch_set_flat(mdg_batch *b, int32_t on);
int mdg_batch_get_stats(mdg_batch *b, mdg_batch_stats *s);

/* ------------------------------------------------------------------------
 * Adjoint (no reference counterpart; a pattern on top of the drop-in):
 * gradients of a trajectory-averaged observable of an NVE drift-kick-drift
 * run with respect to epsilon, sigma and the initial state, by the discrete
 * adjoint (reverse steps with a Hessian-vector product over the same pair
 * list), checkpointing every checkpoint_every steps and recomputing each
 * segment in the backward pass.  V(r) = epsilon phi(r / sigma) with the
 * reference's smoothly truncated phi; the cut-off is cutoff * sigma.  Each
 * checkpoint segment uses the pair list of its first state (all pairs within
 * cutoff * sigma + margin); a particle moving more than margin / 2 within a
 * segment is an error (MDG_ERR_STATE).  FP64 throughout. */
enum mdg_objective { MDG_OBJ_POTENTIAL = 0, MDG_OBJ_PRESSURE = 1 };

typedef struct mdg_adjoint_params {
  double box[3];
  double cutoff;           /* in units of sigma */
  double margin;           /* absolute list margin for one checkpoint segment */
  double dt;
  double epsilon, sigma;
  int32_t steps;           /* horizon */
  int32_t checkpoint_every;
  int32_t objective;       /* MDG_OBJ_POTENTIAL: mean of U/N over steps 1..steps;
                              MDG_OBJ_PRESSURE: mean of (2 KE - sum f r^2) / (3 V) */
  int32_t device;
} mdg_adjoint_params;

typedef struct mdg_adjoint mdg_adjoint;

void mdg_adjoint_params_default(mdg_adjoint_params *p);
/* n particles, 2 <= n < 2^26; every box edge > 2 (cutoff * sigma + margin). */
int mdg_adjoint_create(const mdg_adjoint_params *p, int32_t n, mdg_adjoint **out);
int mdg_adjoint_destroy(mdg_adjoint *a);
const char *mdg_adjoint_last_error(const mdg_adjoint *a);
/* Runs the horizon from host state q4, p4 ([n][4]); *J receives the objective. */
int mdg_adjoint_forward(mdg_adjoint *a, const double *q4, const double *p4, double *J);
/* Gradients of the last forward's objective: dJ/dq0 and dJ/dp0 as host [n][4]
 * (either may be NULL), dJ/depsilon, dJ/dsigma. */
int mdg_adjoint_backward(mdg_adjoint *a, double *dq0, double *dp0, double *depsilon, double *dsigma);

/* Observers without any allocation (this entry point has no counterpart in the
 * reference).  For callers that cannot call cudaMalloc -- applications whose
 * device memory is owned by their own pool, code running in a host callback
 * or a stream-ordered section that must not allocate or synchronise, or a
 * caller that holds its particles on the device and has no handle (creating a
 * handle allocates the whole pair-list machinery).
 *
 * q4_dev, p4_dev: caller-owned device arrays [n][4] (positions in any image;
 * they are wrapped into the box here); out3_dev: caller-owned device buffer of
 * 3 doubles that receives the sums of mdg_observe: sum p^2/2, the pair energy
 * and the pair virial / 3, over every image pair within `cutoff` of the
 * smoothly truncated LJ potential.  Work is enqueued on `stream` (a
 * cudaStream_t; NULL = legacy default stream) and not synchronised.
 *
 * Working memory is one fixed static device array of about 11.3 MB per GPU,
 * held until the process exits: at most 1,048,576 particles and 262,144 cells
 * of width >= cutoff (box side / cutoff, rounded down, per axis); larger
 * inputs return MDG_ERR_CAPACITY with a message on stderr.  The first call on
 * each device looks up that array's device address (cudaGetSymbolAddress), so
 * make the first call on a device outside any stream capture.  Every call
 * reuses the same array: calls that overlap on the GPU (other streams, other
 * host threads) race and give wrong results; serialise them. */
int mdg_observe_noalloc(const double *q4_dev, const double *p4_dev, int32_t n, const double box[3], double cutoff,
                        double *out3_dev, void *stream);

/* ------------------------------------------------------------------------
 * Output and restart formats of the reference, written from host [n][4]
 * arrays (no GPU needed), byte for byte what the reference's writers produce
 * for the same particles in the same order.  append != 0 appends (the
 * reference truncates once and then appends unit by unit). */
/* MDManager::SaveAsDumpFile (mdmanager.cc:475-505): qx qy qz px py pz doubles. */
int mdg_write_dump(const char *path, const double *q4, const double *p4, int32_t n, int32_t append);
/* MDUnit::SaveAsCdview (mdunit.cc:52-67): "0 type qx qy qz px py pz" lines;
 * type may be NULL (all 0, the LJ particle type of AddParticle). */
int mdg_write_cdview(const char *path, const double *q4, const double *p4, const int32_t *type, int32_t n,
                     int32_t append);
/* Variables::SaveConfiguration (variables.cc:45-56): "qx qy qz px py pz" lines
 * (real particles; the reference's file also holds its ghost copies). */
int mdg_write_configuration(const char *path, const double *q4, const double *p4, int32_t n);
/* Variables::SaveToStream (variables.cc:111-118): per particle q[d], p[d] for d = 0..3. */
int mdg_write_stream(const char *path, const double *q4, const double *p4, int32_t n, int32_t append);
/* Variables::LoadFromStream (variables.cc:121-131): int32 count, double time,
 * double zeta, then the stream body.  *n receives the count; MDG_ERR_CAPACITY
 * when it exceeds capacity (nothing else is read). */
int mdg_read_stream(const char *path, double *q4, double *p4, int32_t capacity, int32_t *n, double *time,
                    double *zeta);
/* MDManager::SaveAsDumpFile / SaveAsCdview of a handle's current state
 * (caller order, type 0). */
int mdg_save_dump(mdg_handle *h, const char *path);
int mdg_save_cdview(mdg_handle *h, const char *path);

/* ------------------------------------------------------------------------
 * Initial conditions of the reference's makers, generated on the device.
 * Positions are bit-identical to the reference's for the same box and
 * parameters (same site order); velocities agree to a few ulps (device
 * cos/sin).  The functions allocate temporary device memory and synchronise
 * `stream` (a cudaStream_t; NULL = legacy default stream). */
enum mdg_maker {
  MDG_MAKER_FCC = 0,      /* ConfigurationMaker (confmaker.cc:9-44) */
  MDG_MAKER_EXTRACT = 1,  /* ExtractConfigurationMaker (confmaker.cc:174-252) for one unit spanning the box */
  MDG_MAKER_DROPLET = 2,  /* DropletMaker (burst.cc:10-61): sites within `radius` of the box centre */
  MDG_MAKER_COLLISION = 3 /* BallAdder pair of Collision::Run (collision.cc:8-63): balls of `radius`
                             (the reference uses L_y / 4, density 0.374) at (L_x/4, L_y/2, L_z/2) and
                             (3 L_x/4, L_y/2, L_z/2) moving at +speed and -speed along x */
};
/* Writes the maker's positions to q4_dev ([capacity][4], lane 3 zero); *n
 * receives the count (MDG_ERR_CAPACITY, nothing written, when it exceeds
 * capacity).  p4_dev (NULL to skip) receives the velocities the maker sets
 * itself: (+speed, 0, 0) and (-speed, 0, 0) for the collision maker's two
 * balls, zero for the others.  unit_id seeds ExtractConfigurationMaker's
 * mt19937 as MDUnit::GetID does (0 for the single-unit drop-in). */
int mdg_make_configuration(const double box[3], int32_t maker, double density, double radius, int32_t unit_id,
                           double speed, double *q4_dev, double *p4_dev, int32_t capacity, int32_t *n, void *stream);
/* Variables::SetInitialVelocity (variables.cc:82-108): p4_dev[n][4] <- speed v0,
 * directions from mt19937(seed), mean subtracted. */
int mdg_make_velocity(double v0, int32_t seed, double *p4_dev, int32_t n, void *stream);
/* Both into a handle's state (MDManager's makers + SetInitialVelocity(v0),
 * seed = unit id 0; v0 = 0 leaves the momenta zero).  For the collision maker
 * v0 is the balls' speed and SetInitialVelocity is not applied, as in
 * Collision::Run. */
int mdg_make_state(mdg_handle *h, int32_t maker, double density, double radius, double v0);

#ifdef __cplusplus
}
#endif
#endif
