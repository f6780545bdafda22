// Device-side layout of a batch of MD systems and the helpers the kernels
// share.  Everything is concatenated over the systems of a batch and
// addressed through per-system offset tables (SysDev).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "softcvt.cuh"

namespace mdsc {

constexpr int kTile = 64;        // real-space tile edge, in dipoles
// real-space tiles with the table in shared memory: warps per block, the
// largest table (entries) a block stages, tiles per block
constexpr int kSmemWarps = 16;
constexpr int kSmemTableMax = 10000;
constexpr int kSmemChunk = 32;
// the analytic tiles interpolate in the reference's table below this
// distance (a short table per system, up to r = kNearTab)
constexpr float kNearTab = 2.0f;
constexpr int kMaxNb = 64;       // Verlet-list capacity per particle
constexpr int kMaxD = 4;         // dipoles per particle (MDSC_MAX_DIPOLES)
constexpr int kPartBlock = 128;  // threads per block of the per-particle kernels
constexpr int kKBlock = 128;     // k-vectors per block of the k-space kernels
constexpr int kKChunk = 256;     // particles per block of the structure-factor kernel
// systems of more strips than this sum their real-space tile energies per
// strip first (real_sum); smaller ones are summed tile by tile
constexpr int kStripRows = 32;
constexpr int kMaxR = 256;       // neighbour-pass list entries per rod (systems with a real-space cutoff)
constexpr int kMaxE = 64;        // energy-criterion candidates (higher index) per rod
constexpr int kMaxC = 16;        // WCA contact candidates of higher index per particle
// cell-binned list builds: rods per cell slot range (a cell with more rods
// sends its system to the all-pairs scan for that build); systems of fewer
// rods than kCellMinRods always scan all pairs (the shared-memory all-pairs
// scan of a 2048-rod system took half the time of its cell scan on GB300;
// at 32,768 rods the cells are 8.7x faster)
constexpr int kCellSlots = 64;
constexpr int kCellMinRods = 4096;

// status bits (OR-ed per system; mapped to mdsc_status on the host)
enum : int {
  kErrOverlap = 1,
  kErrNan = 2,
  kErrTable = 4,
  kErrListOverflow = 8,
};

// modes of the force-assembly kernel
enum : int {
  kMaskWca = 1,
  kMaskReal = 2,
  kMaskK = 4,
  kMaskExt = 8,
  kMaskAll = 15,
  kFlagAccum = 16,  // F, T += components (else F, T = components)
  kFlagMoveP = 32,  // then the second half kick (moveP last)
};
constexpr int kRedGroups = 5;  // blocks per system of the reduction kernel
// modes of the per-system reduction kernel
enum : int { kRedEnergies = 1, kRedStep = 2 };

// Per-system constants (read-only during a step).
struct SysDev {
  int n, nd, ndip;
  int part_off;   // first particle of the system in the batch arrays
  int dip_off;    // first dipole
  int nstrip;     // ceil(ndip / kTile)
  int strip_off;  // first strip of the system in the per-strip energy rows
  long long pp_off;  // real-space partials: nstrip*nstrip*6*kTile floats
  int tile_off, ntile;  // tile list range
  int k_off, nk;        // k-vector range
  int rt_off, rt_n;     // real-space table entries (A, B, C of the reference's tabul)
  int kchunk_off, nkchunk;  // structure-factor partial range (chunks of kKChunk particles)
  int kgs;                  // k-space gather parts: the k tiles split over kgs blocks per particle block
  int kgp_off;              // first partial set of the system (kgs > 1)
  int gch_off, pad_g;       // first chunk of the system in the G-tensor partials
  int blk_off, nblk;        // per-particle block range
  int cl_fr;
  int cl_mode;     // cluster bonds: 0 the reference's geometric test, 1 pair energy
  // cell grid of the list build (set at upload from the shapes): ncell = 0
  // scans all pairs; else cnx x cny x cnz cells of at least the largest
  // reach of a list entry, at cell_off .. cell_off + cell_cap - 1 of the
  // batch's cell arrays
  int ncell, cnx, cny, cnz;
  int cell_off, cell_cap;
  float rl_r2;     // rc_real > 0: squared centre-distance radius of the real-space neighbour list
  double rc_real;  // real-space cutoff (0: all minimum-image pairs, the tiles)
  double cl_ubond; // mode 1: a bond is U_pair < -cl_ubond (the threshold times T)
  double L[3];
  double invL[3];
  double invL32[3];  // 2^32 / L: coordinate to fixed-point box fraction
  double V;
  double ex1;      // exp(-gamma dt / 2)            (moveTher, v25/functions.cpp:2199)
  double cnoise;   // sqrt(2 T gamma dt / Q)        (v25/functions.cpp:2200)
  double ntemp3;   // 3 N T                          (v25/functions.cpp:2204)
  double alpha;
  double dt, temp, Q, gamma;
  double B[3];
  double r_list;   // Verlet-list radius on the segment distance
  double skin;
  double min_s;
  double sig_max;  // largest pair sigma
  double Uself;
  float Lfix[3];   // L / 2^32: fixed-point units to length
  float Lf[3];
  // real-space Ewald constants (FP32; set_real_consts).  The analytic tiles
  // measure lengths in units of 1/s, s = alpha sqrt(log2 e), where
  // exp(-alpha^2 r^2) = 2^(-(s r)^2) and every per-system factor of the
  // pair terms leaves them: A = s^3 A~, B = s^5 B~, C = s^5 C~.
  float Lhi[3], Llo[3];    // L / 2^32 per axis as float-float pairs
  float Shi[3], Slo[3];    // s L / 2^32 per axis as float-float pairs
  float sihh, sihl;        // 1 / (s Lh) as a float-float pair, Lh = 0.5*200.2/32768 (the reference's table spacing)
  float shalfLh2;          // (s Lh)^2 / 2
  float snear;             // s kNearTab
  float sc3[2], sc4[2];    // s^3 and s^4 as float-float pairs: fields, energy, pressure tensor and forces to length units
};

// The real-space constants of a system from its alpha and box (FP64
// arithmetic, on the host or in a kernel).
__host__ __device__ inline void set_real_consts(SysDev& P, double Lh) {
  const double s = P.alpha * 1.2011224087864498;  // alpha sqrt(log2 e)
  for (int a = 0; a < 3; ++a) {
    const double h = P.L[a] / 4294967296.0;
    P.Lhi[a] = (float)h;
    P.Llo[a] = (float)(h - (double)P.Lhi[a]);
    P.Shi[a] = (float)(s * h);
    P.Slo[a] = (float)(s * h - (double)P.Shi[a]);
  }
  const double il = 1.0 / (s * Lh);
  P.sihh = (float)il;
  P.sihl = (float)(il - (double)P.sihh);
  P.shalfLh2 = (float)(0.5 * (s * Lh) * (s * Lh));
  P.snear = (float)(s * (double)kNearTab);
  const double s3 = s * s * s, s4 = s3 * s;
  P.sc3[0] = (float)s3;
  P.sc3[1] = (float)(s3 - (double)P.sc3[0]);
  P.sc4[0] = (float)s4;
  P.sc4[1] = (float)(s4 - (double)P.sc4[0]);
}

// Per-system mutable state.
struct SysState {
  double xi[2];      // thermostat coordinates (trans, rot)
  double strn[2];    // stored normals
  long long step;    // steps since upload
  int status;
  int rebuild;       // the list was rebuilt this step
  int list_builds;
  int iter;          // step index within the current mdsc_step call (noise row)
  int force_list;    // rebuild the Verlet list at the next check regardless of the skin
  int cell_ovf;      // this build: a cell held more than kCellSlots rods (all-pairs scan instead)
  long long stop;    // the step count at which the system stops taking steps (mdsc_set_step_limit)
  double K_first[2]; // kinetic energies after the first half kick
  double xi_mid[2];  // xi used by the second half kick
};

// Per-system observables of the last step (mirrors mdsc_observables).
struct SysObs {
  double K[2];
  double U_ss, W_ss, U_dipR, U_dipK, U_ext, U_self;
  double PT_kin[9], PT_ss[9], PT_dipR[9], PT_dipK[9];
  double xi[2];
  long long step;
  int status, n_clusters, list_builds, pad;
  double osum[12];  // sum o (3), sum o o^T (xx xy xz yy yz zz), sum mu o_dipole (3)
};

// One batch, device pointers.
// Launch mappings the autotuner chooses.  Each one changes only how work
// is grouped into blocks and grids, never the arithmetic or the order of a
// sum, so every choice gives the same bits.
struct Tuning {
  int rp_warps = 1;          // real-space tiles (warps) per block: 1, 2 or 4
  int rsum_threads = 256;    // strip-sum block size: 128, 256 or 512
  int wca_blocks = 0;        // grid of the FP64 WCA evaluation (8 x the SM count until tuned)
  int kg_scalar = 0;         // k-space gather: 0 two particles per thread, 1 one
};

struct Batch {
  int nsys, ntot, ndtot, nktot, ntiles, nblk;
  Tuning tune;
  const SysDev* sys;
  SysState* st;
  SysObs* obs;
  // FP64 master state, AoS per particle
  double* r;     // 3n
  double* p;     // 3n
  double* O;     // 9n
  double* l;     // 3n
  double* F;     // 3n   total force of the last evaluation
  double* T;     // 3n
  double* len;   // n
  double* dia;   // n
  double* mass;  // n
  double* inert; // 3n principal moments (set_inertia)
  double* invm;  // n  1 / mass
  double* invI;  // 3n 1 / inertia
  int* psys;     // n: system of each particle
  // dipoles: body data and owner
  double* dpc;   // ndip: offset along the axis
  double* dob;   // 3 ndip: body-frame direction
  double* dmu;   // ndip: moment
  int* downer;   // ndip: particle (batch index)
  // FP32 / fixed-point working copies written by the integrator
  uint32_t* pfx; // 3n  particle positions, fixed point (x[n], y[n], z[n] blocks)
  float4* pax;   // n   rod axis (xyz) and length
  float* pdia;   // n
  uint32_t* dfx; // 3 ndip dipole positions, fixed point (SoA blocks)
  float* dm;     // 3 ndip dipole moment vectors mu*o (SoA blocks)
  // force components
  float* rpart;  // real-space partials
  const float4* rtab;  // 2 per entry: (A, B, C, dA), (dB, dC, 0, 0); see k_real.cu
  float2* rsum;  // 6 * ndtot: each dipole's real-space force and torque over all strips, float-float, component-major
  float* tileE;  // 10 per tile: U, PT[9]
  double* stripE; // 10 per strip: U, PT[9] of the strip's tiles (I, J >= I) (a float-float sum, hi + lo in FP64)
  int2* bstrips;  // (system, strip) of every strip of the systems of more than kStripRows strips
  int nbstrips;
  int any_rc;     // some system has a real-space cutoff
  int* rnb;       // n * kMaxR: real-space neighbour rods (both directions, ascending) of rc_real systems
  int* rnbc;      // n: their number
  double* rlE;    // 10 per particle block: U, PT of the block's real-space neighbour pairs (rc_real systems)
  int4* tiles;   // (sys, I, J, 0)
  int4* rpwork;  // (sys, first tile, tiles, 0): runs of the tiles whose system's table fits shared memory
  int nrpwork;
  int smem_tn;   // the largest of those tables (entries)
  int* gtile;    // the other tiles, one per warp
  int ngtile;
  int rp_table;  // those tiles read the table from global memory (else the analytic form)
  int2* wlist;   // WCA work list: (candidate slot, system), n * kMaxC at most
  int* wlist_n;  // its length this step
  double* wown;  // n * kMaxC * 6: the lower index's force and torque of each candidate
  double* wev;   // n * kMaxC * 11: U, W, PT of each candidate
  double* wcaE;  // per particle block: U, W, PT (11) of its own candidates
  int* wcand;    // n * kMaxC contact candidates (higher index) of each particle
  int* wcnt;     // n
  int* win;      // n * kMaxC: the candidate slots in which a lower-index particle holds this one
  int* wincnt;   // n: their number (zeroed before each screen)
  double* wrec;  // n * kMaxC * 6: the partner's force and torque of each candidate
  // k-space
  int4* kn;      // (nx, ny, nz, 0) per k
  float4* kv;    // (kx, ky, kz, val) per k
  double* kval;  // val per k (FP64)
  double* kvec;  // 3 per k: the k vector in FP64
  double* kpre;  // pval per k (2 (a4 + 1/k^2)) for the pressure tensor
  float* kpart;  // structure-factor partials: 10 per (chunk, k)
  double* ksum;  // 10 per k: uve (6), self, uvslf (3) -- FP64
  float2* kS;    // val * S(k) per k, FP32 for the gather
  double* kE;    // 10 per k: energy and pressure-tensor terms
  double* kG;    // 6 per particle chunk: sum of m m^T (one dipole per particle)
  double* kGs;   // 6 per system: the chunk sums added in chunk order
  int* kgcnt;    // per system: chunks done this step (the last one adds them)
  int* icnt;     // per system: first-half blocks done this step (the last one sets xi_mid)
  int2* kgwork;  // (particle block, part) of every k-space gather block
  int nkgwork;
  float* kgpart; // partial gather sums of split systems: per (particle block, part) kPartBlock x 12
  int* kgdone;   // per particle block: parts done this launch (the last one combines them)
  float2* Fk;    // 3 ndip: k-space force on each dipole, float-float (hi, lo)
  float2* Tk;    // 3 ndip: k-space torque m x G, float-float
  // integrator partials, per block
  double* kin1;  // 2 per block
  double* kin2;  // 9 per block: K_t, K_r, PTkin xx xy xz yy yz zz, U_ext
  double* dmax;  // 1 per block: largest displacement measure since the last list build
  double* obk;   // 12 per block: the order-parameter terms of SysObs::osum
  int2* blk;     // (sys, first particle) per block
  // cell bins of the list build: per cell its count, and kCellSlots slots
  // of (fixed-point position, batch index) and (axis, length), filled in
  // any order by the binning kernel
  int* ccnt;     // ncellcap
  uint4* cpos;   // ncellcap * kCellSlots
  float4* cax;   // ncellcap * kCellSlots
  int2* cellblk; // per pair of cells of capacity: (system, first cell)
  int ncellblk;
  int cells;     // 1: systems with a cell grid build their lists on it; 0: every system scans all pairs
  int honor_stop; // the step graph: kernels skip the systems at their step limit
  const int* skip; // per system, or null: kernels skip the flagged systems (a force evaluation
                   // for the systems that joined a batch, beside systems that arrived with forces)
  // neighbour list
  int* nb;       // n * kMaxNb
  int* nbc;      // n
  uint32_t* fsave; // 3n fixed-point positions at the last build
  float* usave;     // 3n axes at the last build
  // clusters
  int* comp;     // n component representative
  unsigned char* eflag;  // n * kMaxNb: list entry is a cluster bond
  int* flag;     // 1 changed flag
  int* ebond;    // n * kMaxC: energy-criterion bonds to higher indices
  int* ebcnt;    // n: their number
  int* eovf;     // nsys: a particle had more than kMaxC energy bonds (or kMaxE candidates)
  int* ecand;    // n * kMaxE: energy-criterion candidates of higher index (allocated on first use)
  int* ecnt;     // n: their number
  // thermostat noise: [iter][sys][4] = g0_t, g1_t, g0_r, g1_r
  const double* noise;
};

// Per system, for the pair-correlation histograms: bins, first histogram
// word, number of species.
struct CorrSys {
  int nbins, off, nsp, pad;
};

// ---- small helpers ----------------------------------------------------
// A system at its step limit takes no step: every kernel of the step graph
// returns at once for it (the check is uniform over a block or a warp of
// that system), so it costs nothing until it leaves the batch.
__device__ __forceinline__ bool at_limit(const Batch& b, int s) {
  return (b.honor_stop && b.st[s].step >= b.st[s].stop) || (b.skip && b.skip[s]);
}

__host__ __device__ inline int cdiv(int a, int b) { return (a + b - 1) / b; }

// fixed-point image of a coordinate: fraction of the box in [0, 2^32),
// floor(x 2^32 / L) modulo 2^32 (invL32 = 2^32 / L; the product is the
// exactly scaled x / L, so this equals frac(x / L) 2^32 truncated)
__device__ inline uint32_t to_fix(double x, double invL32) {
  return soft_floor_u32(x * invL32);
}

// slot of a particle block in the per-block partial arrays: blocks are
// launched largest system first, but each system's partials sit in order
// at blk_off .. blk_off + nblk - 1
__device__ __forceinline__ int blk_slot(const SysDev& P, int2 bk) {
  return P.blk_off + (bk.y - P.part_off) / kPartBlock;
}

// minimum-image difference of two fixed-point coordinates, in length units
__device__ inline float fix_diff(uint32_t a, uint32_t b, float scale) {
  return (float)(int32_t)(a - b) * scale;
}

}  // namespace mdsc
