/*
 * mdsc.h -- C ABI of the GB300 (sm_103a) MD-step library for polydisperse
 * dipolar spherocylinders.  Drop-in for the hot path of mdSpherocyl.
 *
 * The reference's boundary is the set of free functions in
 * v25/functions.hpp:30-54,107-108 that v25/main.cpp calls once per step from one
 * host thread (force_sc, force_dipR, force_dipK, ext_field, self_ener,
 * moveX, moveP, moveTher, neigh_list, check_list, clust_conf).  Each of
 * them has an entry point below that does the same work on the GPU, and
 * mdsc_step() runs the whole loop body (v25/main.cpp:558-708) as one
 * captured CUDA graph.
 *
 * Plain C types only: pointers and sizes, no exceptions across the ABI.
 * All state stays resident in GPU memory between calls; the host sees
 * scalars, except when it uploads or downloads a system.
 *
 * One handle (mdsc_batch) holds one or many independent systems ("batch");
 * every entry point works on all of them at once and returns per-system
 * results in arrays indexed by system.  A batch of one system is the plain
 * path.  Calls on one handle are not thread-safe; different handles are.
 *
 * Units and conventions are the reference's: sigma = epsilon = k_B = 1; O is
 * the 3x3 orientation matrix stored row-major with rows = body axes in the
 * lab frame (row 2 = rod axis, v25/classes.hpp:74); angular momentum l in
 * the lab frame; dipoles are given in the body frame as (offset along the
 * rod axis, direction x, y, z, moment) (v25/classes.cpp:148-173).
 */
#ifndef MDSC_H
#define MDSC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MDSC_ABI_VERSION 3  /* 2: mdsc_observables gained G1, G2, M; 3: mdsc_system_desc.rc_real */
#define MDSC_MAX_DIPOLES 4 /* dipoles per particle */

typedef enum {
  MDSC_OK = 0,
  MDSC_ERR_BAD_ARG = 1,
  MDSC_ERR_CUDA = 2,
  MDSC_ERR_OOM = 3,
  /* force_sc's abort (v25/functions.cpp:1454-1473): a listed pair with
     segment distance^2 < 0.49 sigma^2 or greater than its centre distance^2 */
  MDSC_ERR_OVERLAP = 4,
  MDSC_ERR_NAN = 5,
  /* a dipole pair beyond the reference's table range r > 100.1 sigma
     (v25/functions.cpp:1563,1608-1614; guarded by L_min <= 200 at
     v25/main.cpp:420-425) */
  MDSC_ERR_TABLE_RANGE = 6,
  MDSC_ERR_LIST_OVERFLOW = 7,
  MDSC_ERR_NO_DEVICE = 8,
  MDSC_ERR_TOO_LARGE = 9,
  MDSC_ERR_STATE = 10
} mdsc_status;

/* Everything that defines one system besides its particle state: the
   input.txt parameters the hot path uses (v25/functions.cpp:10-87). */
typedef struct {
  int n;             /* particles */
  int nd;            /* dipoles per particle, 0..MDSC_MAX_DIPOLES */
  double box[3];     /* box edges L_x, L_y, L_z */
  double alpha;      /* Ewald convergence parameter ("Convergence param(a)") */
  int K_max;         /* k-vectors n_x, n_y, n_z in [0, K_max-1] ("No. of Kvectors") */
  int ksq_max;       /* 0: the reference's full cube; > 0: keep |n|^2 <= ksq_max only */
  double sr_cut;     /* "Cutoff dist(SRange)"; 0 -> L_min/2 - d_min (v25/main.cpp:398-399) */
  double dt;         /* time step */
  double temp;       /* thermostat temperature */
  double Q;          /* thermostat mass */
  double gamma;      /* thermostat "shear rate" (Langevin noise on xi); 0 = deterministic */
  double xi0;        /* initial thermostat coordinate (0 in v25, 1 in v25/v251) */
  double B[3];       /* external field */
  double min_s;      /* cluster proximity distance ("proximity dist.") */
  int cl_fr;         /* clustering frequency in steps; 0 = never */
  unsigned long thermo_seed[2]; /* MT19937 seeds of the two thermostats (1, 2 in the driver) */
  unsigned long cluster_seed;   /* MT19937 seed of the cluster generator (1 in the driver) */
  unsigned long cluster_skip;   /* draws already taken from it (e.g. by initialisation) */
  /* Real-space cutoff.  0: every minimum-image dipole pair, as the reference
     sums (v25/functions.cpp:1570-1672).  > 0: the reference's force_dipR
     with its table zeroed beyond rc_real -- entries k with Lh (k + 1) >
     rc_real set to 0 (Lh = 0.5*200.2/32768, v25/functions.cpp:1563,1681),
     so pairs beyond rc_real + Lh contribute nothing -- summed over a
     neighbour list of the system's rods instead of all pairs. */
  double rc_real;
} mdsc_system_desc;

/* Host-side structure-of-arrays view of one system (FP64).  Shapes:
   r, p, l, F, T: n*3; O: n*9; len, dia, mass: n; dip: n*nd*5; clust: n. */
typedef struct {
  double* r;
  double* p;
  double* O;
  double* l;
  double* F;
  double* T;
  const double* len;
  const double* dia;
  const double* mass;
  const double* dip;
  int* clust;
} mdsc_host_state;

/* Per-system results of the last step, as totals over the system (the
   driver divides by N and V, v25/main.cpp:626-649). */
typedef struct {
  double K[2];      /* translational, rotational kinetic energy (moveP) */
  double U_ss, W_ss;
  double U_dipR, U_dipK, U_ext, U_self;
  double PT_kin[9], PT_ss[9], PT_dipR[9], PT_dipK[9];
  double xi[2];     /* thermostat coordinates after the step */
  long long step;   /* steps taken so far */
  int status;       /* mdsc_status of this system */
  int n_clusters;   /* clusters found at the last clustering step */
  int list_builds;  /* neighbour-list rebuilds so far */
  int pad;
  /* oo_params (v25/functions.cpp:2702-2760) of the state after the step, as
     the driver takes them every step (v25/main.cpp:720-728): nematic order
     G2, polar order G1 and the total dipole moment M.  Per-particle terms in
     FP32 (the reference forms Q in FP32 too), float-float sums: M carries
     ~1e-7 of each moment; mdsc_order_params gives it from FP64 terms. */
  double G1, G2;
  double M[3];
} mdsc_observables;

typedef struct mdsc_batch mdsc_batch;

/* ---- lifetime -------------------------------------------------------- */
/* Creates a batch of nsys systems on CUDA device `device` and allocates all
   its GPU memory.  The per-system tables the reference builds once
   (tabul, v25/functions.cpp:1680-1704; wave_v, :1963-1990) are set up here. */
mdsc_status mdsc_create(const mdsc_system_desc* descs, int nsys, int device, mdsc_batch** out);
mdsc_status mdsc_destroy(mdsc_batch* b);
int mdsc_num_systems(const mdsc_batch* b);
/* bytes of GPU memory the batch holds (with the energy criterion's
   candidate lists once a system of it takes that criterion) */
size_t mdsc_device_bytes(const mdsc_batch* b);
/* GPU memory a batch of these systems would need, without creating it.
   mdsc_set_cluster_energy later adds 260 bytes per particle of the batch. */
size_t mdsc_estimate_bytes(const mdsc_system_desc* descs, int nsys);
/* sizeof of the ABI's structures as this library was built (for bindings
   that lay them out by hand): mdsc_system_desc, mdsc_host_state,
   mdsc_observables, mdsc_view.  Any pointer may be NULL. */
void mdsc_abi_sizes(size_t* desc, size_t* host_state, size_t* observables, size_t* view);
/* human-readable detail of the last error on this handle */
mdsc_status mdsc_last_error(const mdsc_batch* b, char* buf, size_t len);

/* ---- state transfer (host SoA <-> GPU) -------------------------------- */
/* Uploads system `sys`.  Shape arrays (len, dia, mass, dip) are read on
   every upload; F and T may be NULL (then zero); clust, if given, sets the
   cluster labels (as chrg_conf reads them) until the next clustering step.
   Rebuilds the neighbour list and the derived single-precision copies. */
mdsc_status mdsc_upload(mdsc_batch* b, int sys, const mdsc_host_state* s);
/* Downloads r, p, O, l, F, T and (if non-NULL) clust of system `sys`. */
mdsc_status mdsc_download(mdsc_batch* b, int sys, mdsc_host_state* s);
/* Uploads / downloads all systems with one host->device (device->host)
   copy each way; arrays are the concatenation of every system's arrays. */
mdsc_status mdsc_upload_all(mdsc_batch* b, const mdsc_host_state* packed);
mdsc_status mdsc_download_all(mdsc_batch* b, mdsc_host_state* packed);
/* Thermostat state: xi, stored normal (v25/classes.hpp:147-151). */
mdsc_status mdsc_set_thermostat(mdsc_batch* b, int sys, const double xi[2], const double strn[2]);
/* The same, read back (either pointer may be NULL): what print_conf writes
   after the particles (v25/functions.cpp:1222-1224). */
mdsc_status mdsc_get_thermostat(mdsc_batch* b, int sys, double xi[2], double strn[2]);

/* ---- the reference's hot-path functions, on every system --------------- */
/* Zero F and T (v25/main.cpp:582-588). */
mdsc_status mdsc_zero_forces(mdsc_batch* b);
/* force_sc (v25/functions.hpp:38-39, v25/functions.cpp:1397-1553): WCA
   core forces and torques over the neighbour list, accumulated into F, T.
   U, W: nsys each; PT: nsys*9.  Returns MDSC_ERR_OVERLAP like the
   reference's false. */
mdsc_status mdsc_force_sc(mdsc_batch* b, double* U, double* W, double* PT);
/* force_dipR (v25/functions.hpp:40-41, v25/functions.cpp:1555-1678):
   real-space Ewald over all minimum-image dipole pairs, accumulated; for a
   system with rc_real > 0, force_dipR with its table zeroed beyond rc_real,
   over the system's neighbour list. */
mdsc_status mdsc_force_dipR(mdsc_batch* b, double* U, double* PT);
/* force_dipK (v25/functions.hpp:42-43, v25/functions.cpp:1706-1961):
   reciprocal-space Ewald, accumulated. */
mdsc_status mdsc_force_dipK(mdsc_batch* b, double* U, double* PT);
/* ext_field (v25/functions.hpp:44, v25/functions.cpp:1992-2025): torques
   accumulated, energies out. */
mdsc_status mdsc_ext_field(mdsc_batch* b, double* U);
/* self_ener (v25/functions.hpp:45, v25/functions.cpp:2027-2069). */
mdsc_status mdsc_self_ener(mdsc_batch* b, double* U);
/* moveX (v25/functions.hpp:50, v25/functions.cpp:2071-2092). */
mdsc_status mdsc_moveX(mdsc_batch* b);
/* moveP (v25/functions.hpp:51-52, v25/functions.cpp:2094-2184); xi: nsys*2
   thermostat coordinates; K: nsys*2; PT: nsys*9. */
mdsc_status mdsc_moveP(mdsc_batch* b, const double* xi, int last, double* K, double* PT);
/* Spherocyl::renorm for every particle (v25/classes.cpp:307-325). */
mdsc_status mdsc_renorm(mdsc_batch* b);
/* neigh_list (v25/functions.hpp:30-31, v25/functions.cpp:1298-1334):
   rebuild every system's Verlet list now. */
mdsc_status mdsc_neigh_list(mdsc_batch* b);
/* check_list (v25/functions.hpp:33-36, v25/functions.cpp:1356-1394):
   rebuild[s] = 1 where the skin was crossed since the last build. */
mdsc_status mdsc_check_list(mdsc_batch* b, int* rebuild);
/* clust_conf (v25/functions.hpp:107-108, v25/functions.cpp:3282-3324):
   labels of system `sys` with the reference's numbering, drawing from the
   system's cluster generator.  labels: n ints (may be NULL). */
mdsc_status mdsc_clust_conf(mdsc_batch* b, int sys, int* labels, int* n_clusters);
/* The bond test of system sys's clusterings (mdsc_clust_conf and the
   clustering every cl_fr steps of mdsc_step).  u_bond_kT = 0: the reference's
   geometric test (the default).  u_bond_kT > 0: an energy criterion, an
   extension the reference does not have: i and j are bonded when
     U_pair = U_WCA (force_sc's pair energy) + sum over their dipole pairs of
              mu_a mu_b (o_a.o_b - 3 (o_a.r)(o_b.r) / r^2) / r^3
   (bare dipole-dipole energy at the minimum image of the dipole sites) is
   below -u_bond_kT * T, T the system's temperature.  Labels are then
   numbered as clust_conf numbers them.  MDSC_ERR_LIST_OVERFLOW from the
   clustering if a particle has more than 16 such bonds (or 64 screened
   candidates) to higher indices.  The first call with u_bond_kT > 0 on a
   batch allocates the candidate lists: 260 bytes per particle of the batch. */
mdsc_status mdsc_set_cluster_energy(mdsc_batch* b, int sys, double u_bond_kT);

/* Moves system ssys of batch src into slot dsys of batch dst (same device,
   same n and nd) without leaving the GPU: particle state, forces, shapes,
   thermostat and generator states, step count and cluster labels.  The
   continuous-batching server uses it to repack running systems when jobs
   finish or arrive.  No counterpart in the reference (one system per run). */
mdsc_status mdsc_transfer(mdsc_batch* dst, int dsys, mdsc_batch* src, int ssys);
/* The same for count systems at once (slot dsys[k] of dst from slot
   ssys[k] of src), without a host synchronization: the copies are ordered
   after src's queued work and before dst's next work, in one kernel
   launch per 256 systems.  src may be destroyed as soon as it returns.
   No counterpart in the reference. */
mdsc_status mdsc_transfer_many(mdsc_batch* dst, mdsc_batch* src, const int* dsys, const int* ssys, int count);
/* System sys takes no more steps once its step count (steps since the
   batch was created, carried by mdsc_transfer) reaches `limit`; limit <= 0
   removes the limit.  In mdsc_step a system at its limit costs nothing:
   every kernel of the step returns at once for it, its state, observables
   and generators stay as they were, and the others go on.  The server uses
   it so that a job that finishes within a tick stops at exactly its step
   count while the batch runs the whole tick.  No counterpart in the
   reference (one system per run). */
mdsc_status mdsc_set_step_limit(mdsc_batch* b, int sys, long long limit);

/* ---- the fused step ---------------------------------------------------- */
/* Advances every system by nsteps steps of the reference's loop body
   (renorm every 100 steps, moveTher 0, moveP, moveTher 1, moveX, forces,
   ext_field, moveP, moveTher 2, list check, clustering every cl_fr steps).
   Observables of the last step go to obs (nsys entries; may be NULL).
   Thermostat noise is drawn on the host from each system's MT19937 pair
   exactly as moveTher does (v25/functions.cpp:2193-2213). */
mdsc_status mdsc_step(mdsc_batch* b, int nsteps, mdsc_observables* obs);
/* A step loop that keeps its state in host memory (the reference's driver
   around its per-function boundary, v25/main.cpp:558-708, with part and
   its Dynvecs on the host): uploads `in` (r, p, O, l and F, T of every
   system, as mdsc_upload_all; NULL keeps the device state), takes nsteps
   steps as mdsc_step, and downloads the updated state into `out` (as
   mdsc_download_all; NULL fields are skipped, NULL out downloads nothing).
   Positions and orientations are final once the last step has moved the
   particles, so they travel to the host while that step's forces are
   computed; momenta, angular momenta, forces and torques as soon as its
   force assembly has written them.
   Observables of the last step go to obs (may be NULL). */
mdsc_status mdsc_step_io(mdsc_batch* b, const mdsc_host_state* in, int nsteps, mdsc_host_state* out,
                         mdsc_observables* obs);
/* Observables of the last step without stepping. */
mdsc_status mdsc_observe(mdsc_batch* b, mdsc_observables* obs);
/* mdsc_step that also returns every step's observables: trace holds
   nsteps x nsys entries, step-major (trace[k * nsys + sys]), as the
   reference's driver reads them after each step (accumulators, output.dat,
   v25/main.cpp:618-650,710-800).  n_clusters changes at clustering steps. */
mdsc_status mdsc_step_trace(mdsc_batch* b, int nsteps, mdsc_observables* trace);
/* The state of a system's generators: which = 0, 1 the translational and
   rotational thermostats (Thermostat::m_ran, v25/classes.cpp:344-367), 2 the
   clustering generator.  MT19937 in GSL's layout: 624 state words and the
   position of the next one (0..624), so the reference's ran_state files
   (gsl_rng_fwrite) round-trip through these two calls. */
mdsc_status mdsc_get_rng(const mdsc_batch* b, int sys, int which, uint32_t mt[624], int* mti);
mdsc_status mdsc_set_rng(mdsc_batch* b, int sys, int which, const uint32_t mt[624], int mti);

/* ---- instrumentation --------------------------------------------------- */
/* Number of kernel launches the last mdsc_step issued per step, and the
   CUDA stream the batch runs on (a cudaStream_t). */
int mdsc_launches_per_step(const mdsc_batch* b);
void* mdsc_stream(const mdsc_batch* b);
/* Device time (ms) of the last mdsc_step call: CUDA events on the batch's
   stream around its noise upload and graph launches. */
double mdsc_last_device_ms(const mdsc_batch* b);
/* Average device time (ms) per launch of each kernel over the last
   mdsc_profile_steps call: names and times in the order of `names`. */
mdsc_status mdsc_profile_steps(mdsc_batch* b, int nsteps, int max_kernels, char* names,
                               size_t name_stride, double* ms_per_launch, int* n_kernels);

/* ---- observables outside the step ----------------------------------------- */
/* Number of histogram bins of system sys for bar width bar_w:
   floor(sqrt(3) Lmin / (2 bar_w)), Lmin the shortest box edge, as the
   reference sizes Hista (v25/main.cpp:251-255); 0 on a bad argument. */
int mdsc_correlation_bins(const mdsc_batch* b, int sys, double bar_w);
/* Species of system sys: nspecies contiguous blocks of counts[k] particles
   (the reference's components, numbered as calc_II / rev_II number them,
   v25/functions.cpp:1158-1179).  Default: one species.  Used by
   mdsc_correlations only. */
mdsc_status mdsc_set_species(mdsc_batch* b, int sys, int nspecies, const int* counts);
/* Doubles mdsc_correlations writes for system sys:
   (nc + nc (nc - 1) / 2) x 4 x nbins, nc its species. */
int mdsc_correlation_size(const mdsc_batch* b, int sys, double bar_w);
/* Replaces acc_correl (v25/functions.cpp:2400-2470): adds every unordered
   pair's terms to the pair-correlation histograms of the current state, at
   bin floor(r / bar_w) of the functions 000, 110, 112 and 220 -- for two
   particles of one species 2, 2 dot, 2 (3 doti dotj - dot), 3 dot^2 - 1 to
   that species' histogram (Hista), otherwise 1, dot, 3 doti dotj - dot,
   (3 dot^2 - 1) / 2 to the species pair's (Histe).  hist holds, system after
   system, its nc species blocks and then its species-pair blocks in the
   order (0,1), (0,2), ..., (1,2), ..., each 4 x nbins doubles
   (function-major; mdsc_correlation_size doubles per system), and is ADDED
   TO, as the reference accumulates over a run.  The counts are exact and a
   pair lands in the reference's bin (an FP64 recheck near bin edges); the
   other three sums carry the FP32 rounding of each pair's term (~1e-7 of
   the count).  Pairs past the last bin (the box's corners) are left out,
   where the reference writes past its matrix. */
mdsc_status mdsc_correlations(mdsc_batch* b, double bar_w, double* hist);
/* Replaces oo_params (v25/functions.cpp:2702-2760) per system: G1[sys],
   G2[sys] (nematic order: the largest |eigenvalue| of
   Q = sum (3 o o^T - 1) / (2 N), and the polar order |sum o . e| / N along its
   eigenvector) and M[3 sys ..] = sum over dipoles of mu o (lab frame).  Each
   argument may be NULL.  The sums are FP64 on the GPU; the reference forms
   Q in FP32, so G1 and G2 agree with it to ~1e-6. */
mdsc_status mdsc_order_params(mdsc_batch* b, double* G1, double* G2, double* M);

/* ---- a new configuration ----------------------------------------------- */
/* ini_pos (v25/functions.cpp:491-675) on the GPU: system sys (shapes
   uploaded) put on the reference's lattice, species by species (nspecies
   contiguous blocks of counts[k] rods, shapes from their first rod), every
   rod along z, sites that come closer than the mean diameter to an earlier
   species skipped, the sites reused from the first when they run out.
   *n_overlaps: the overlapping pairs ini_pos's closing test finds (it reports
   them and the run stops at its first force evaluation).  Momenta are left
   as they are; the reference's 1000 cluster moves (GCAmix) are not made. */
mdsc_status mdsc_lattice(mdsc_batch* b, int sys, int nspecies, const int* counts, int* n_overlaps);
/* Momenta and angular momenta of system sys from the Maxwell-Boltzmann
   distribution at temperature temp, zero total momentum, from a counter-
   based generator seeded by seed (the reference's ini_mom draws differently,
   v25/functions.cpp:677-1147). */
mdsc_status mdsc_thermalize(mdsc_batch* b, int sys, double temp, unsigned long long seed);

/* ---- picture ----------------------------------------------------------- */
/* What mdsc_render draws and from where: the reference viewer's controls
   (v25/graphic.cpp:24-41), with its defaults in brackets. */
typedef struct {
  int width, height;         /* pixels [480 x 480] */
  double theta, phi, dist;   /* camera direction and distance [0.1, 0, 15] */
  double ref[3];             /* the point looked at [0 0 0] */
  double shift[3];           /* added to every position, the viewer's d [0 0 0] */
  int dipoles;               /* draw the dipoles [1] */
  int images;                /* and the 26 periodic images [0] */
  int box;                   /* the box edges [1] */
  int cluster;               /* only the particles with this cluster label; -1 all [-1] */
} mdsc_view;
/* Replaces the SDL/OpenGL viewer (v25/graphic.cpp) without a display: a
   ray-cast picture of system sys in its current state on the GPU -- rods
   grey by species with a blue +axis tip and red/green meridians on the body
   x/y axes, dipoles as blue/red segments, the box edges, on white, from the
   viewer's camera and light -- written to rgb (height x width x 3 bytes,
   rows from the top). */
mdsc_status mdsc_render(mdsc_batch* b, int sys, const mdsc_view* view, unsigned char* rgb);

/* ---- autotuner -------------------------------------------------------- */
/* Chooses the launch mappings (real-space tiles per block, strip-sum block
   size, grid of the FP64 WCA evaluation, k-space gather form) by timing each
   candidate on the batch's current state, and keeps the fastest.  Only
   mappings that leave every result bit-identical are candidates, so a
   system's trajectory does not depend on the choice or on the batch it is
   in.  mdsc_step runs it before its first step unless the environment sets
   MDSC_AUTOTUNE=0; choices are cached per process by the batch's size class
   (force = 1 times again regardless).  No counterpart in the reference. */
mdsc_status mdsc_autotune(mdsc_batch* b, int force);
/* The mappings in use: values[0..4] = tiles per block, strip-sum threads,
   WCA evaluation blocks, gather form (0 packed, 1 one particle per thread),
   tuned (1 once chosen); log: the last tuning's timings (may be NULL). */
mdsc_status mdsc_tuning(const mdsc_batch* b, int* values, char* log, size_t len);
/* Sets the mappings by hand (values[0..3] as above) instead of tuning. */
mdsc_status mdsc_set_tuning(mdsc_batch* b, const int* values);
/* List builds (neigh_list, v25/functions.cpp:1298-1334) on cells (on = 1,
   the default: systems of 4096 rods or more whose box holds at least 3
   cells of the largest list reach along every axis bin their rods and scan
   the 27 cells around each rod, O(N)) or over all pairs (on = 0, O(N^2)).
   Both give the same lists, so the same bits; the switch is for timing and
   tests.  A cell holding more than 64 rods sends its system to the
   all-pairs scan for that build. */
mdsc_status mdsc_set_list_cells(mdsc_batch* b, int on);

/* ---- allocation-free variant ------------------------------------------- */
/* Real-space Ewald forces, torques (without lever arms), energy and
   pressure tensor of one system of ndip dipoles, one per particle, for
   callers that cannot allocate GPU memory at the point of the call (a host
   with a fixed device-memory budget, a real-time loop, a plugin whose host
   owns every buffer).  Inputs and outputs are device pointers the caller
   owns: d_pos, d_mom (ndip*3 doubles each: dipole positions and moment
   vectors mu*o), d_F, d_T (ndip*3 doubles), d_UPT (10 doubles: the energy,
   then the pressure tensor row by row); box, alpha on the host; stream is a
   cudaStream_t (NULL: the default stream).  The call allocates nothing: its
   scratch is a fixed array of this library's device memory (about 6.5 MB
   on every GPU that loads the library, held until the process exits), so
   ndip may not exceed 4096 (MDSC_ERR_TOO_LARGE otherwise).  The first call
   on a device looks up that array's device address; make it before any
   stream capture.  The address is kept per device and CUDA context: after
   cudaDeviceReset the next call looks it up again (so it, too, must come
   before any capture).  A CUDA error already pending on the calling thread
   makes the call return MDSC_ERR_CUDA without launching, and leaves that
   error pending.  Calls share the array and overwrite what they read, so
   calls whose work overlaps on the GPU race.  No counterpart in the
   reference: it is the GPU form of force_dipR's arithmetic for callers
   without an allocator. */
mdsc_status mdsc_force_dipR_noalloc(int ndip, const double* d_pos, const double* d_mom,
                                    const double box[3], double alpha, double* d_F, double* d_T,
                                    double* d_UPT, void* stream);

/* ---- utility ------------------------------------------------------------ */
/* Measured FP32 multiply-add throughput of a device (the bound of the pair
   kernels): `reps` timed launches of independent multiply-add chains in
   scalar (FFMA) and paired (FFMA2, float2 halves) form, best of each, in
   TFLOP/s at 2 FLOP per multiply-add; ms is the best paired launch's device
   time, num_sms the device's multiprocessor count.  No counterpart in the
   reference: it is the roofline denominator of the measurement. */
mdsc_status mdsc_fp32_peak(int device, int reps, double* tflops_ffma, double* tflops_ffma2, double* ms,
                           int* num_sms);


/* Seeded random non-overlapping placement of n rods in a periodic box
   (sequential rejection on the segment distance, gap added to
   (D_i + D_j)/2): centres r (n*3) and orientation matrices O (n*9).  Host
   code, no GPU.  No counterpart on the reference's hot path: the reference
   starts from a lattice plus cluster pivots (v25/functions.cpp:491-1156,
   3328-3409), which stays out of scope.  Returns MDSC_ERR_TOO_LARGE when
   max_attempts + 100 n proposals do not place every rod. */
int mdsc_place_rods(int n, const double* len, const double* dia, const double* box,
                    unsigned long long seed, double gap, int max_attempts, double* r, double* O);

#ifdef __cplusplus
}
#endif
#endif
