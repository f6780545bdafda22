// Host implementation of the C ABI in include/mdsc.h: batch layout, memory,
// the CUDA-graph step, thermostat noise and cluster-label replay.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <atomic>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "host_util.hpp"
#include "mdsc.h"
#include "mdsc_dev.cuh"

namespace mdsc {
void launch_real_pairs(const Batch& b, bool multi, cudaStream_t s);
cudaError_t prepare_real_pairs();
void launch_real_sum(const Batch& b, cudaStream_t s);
// the cutoff systems' neighbour pass: real space (1), WCA screen (2), both (3)
void launch_near_pass(const Batch& b, int mode, cudaStream_t s);
void launch_kspace(const Batch& b, int maxnd, const int4* kwork, int nkwork, const int2* kowner,
                   double* kE, cudaStream_t s);
void launch_derive(const Batch& b, cudaStream_t s);
void launch_integrate_first(const Batch& b, cudaStream_t s);
void launch_finalize(const Batch& b, int mode, cudaStream_t s);
void launch_reduce_obs(const Batch& b, int mode, cudaStream_t s);
void launch_order_terms(const Batch& b, cudaStream_t s);
void launch_movex(const Batch& b, cudaStream_t s);
void launch_renorm(const Batch& b, cudaStream_t s);
void launch_movep(const Batch& b, const double* xi, int last, cudaStream_t s);
void launch_list_build(const Batch& b, int force_all, cudaStream_t s);
// the WCA screens and FP64 evaluation; near_mode: what the cutoff systems'
// neighbour pass runs besides its WCA screen (1: also their real space)
void launch_wca(const Batch& b, int near_mode, cudaStream_t s);
void launch_cluster_bonds(const Batch& b, cudaStream_t s);
void launch_ebond(const Batch& b, cudaStream_t s);
void launch_cluster_hook(const Batch& b, cudaStream_t s);
void launch_cluster_compress(const Batch& b, cudaStream_t s);
void launch_reset_iter(const Batch& b, cudaStream_t s);
// copies systems (dst slot, src slot) between batches on the destination's stream
cudaError_t launch_transfer(const Batch& dst, const Batch& src, const std::vector<int2>& pairs, cudaStream_t s);
void launch_kspace_parts(const Batch& b, int maxnd, const int4* kwork, int nkwork, const int2* kowner,
                         double* kE, int part, cudaStream_t s);
void launch_correlations(const Batch& b, const CorrSys* cs, const unsigned char* species, double bar_w,
                         int max_bins, unsigned long long* hist, cudaStream_t s);
void launch_order_sums(const Batch& b, double* out, cudaStream_t s);
size_t render_scratch_bytes(int n, int nd, int images);
void launch_lattice_sites(const Batch& b, int sys, double len, double dia, int num1, int num2, int nsites,
                          int prev_first, int prev_n, double* site_r, int* ok, cudaStream_t s);
void launch_overlap_count(const Batch& b, int sys, int n, int* count, cudaStream_t s);
void launch_thermalize(const Batch& b, int sys, int n, double temp, unsigned long long seed, cudaStream_t s);
void launch_render(const Batch& b, int sys, int n, const unsigned char* species, const int* keep, int images,
                   int dipoles, int draw_box, float seg_rad, float box_rad, const float* eye, const float* fwd,
                   const float* right, const float* up, const float* light, float tan_half, int width,
                   int height, void* scratch, unsigned char* rgb, cudaStream_t s);
}  // namespace mdsc

using namespace mdsc;

namespace {

constexpr int kNoiseChunk = 256;  // steps of thermostat noise per upload
// the reference's table covers r <= 0.5 * 200.2 (v25/functions.cpp:1563,1681)
constexpr double kTableRmax = 0.5 * 200 * 1.001;
constexpr double kLh = 0.5 * (200 * 1.001) / 32768;

struct Layout {
  std::vector<SysDev> sys;
  std::vector<int4> tiles, kn, kwork;
  std::vector<float4> kv;
  std::vector<float4> rtab;  // real-space tables of every system (filled by fill_tables)
  size_t rtab_n = 0;         // float4 slots the tables take (2 per entry)
  std::vector<double> kval, kpre, kvec;
  std::vector<int2> blk, kowner;
  std::vector<int2> bstrips;  // strips of the systems whose tile energies are summed per strip
  std::vector<int2> kgwork;   // (particle block, part) of the k-space gather
  std::vector<int2> cellblk;  // (system, first cell) of every block of the cell-binned list build
  std::vector<int4> rpwork;   // runs of tiles whose table is staged in shared memory
  std::vector<int> gtile;     // tiles of the one-tile-per-warp kernel (analytic or global table)
  int smem_tn = 0;
  bool rp_table = false;      // the tiles interpolate in the table (MDSC_REAL_FORM=table)
  int ncellcap = 0;           // cells of capacity over all systems
  long long kgsets = 0;       // partial sets of the split gathers
  int ntot = 0, ndtot = 0, nktot = 0, maxnd = 0, nchunks = 0, nstrips = 0;
  bool any_rc = false;  // some system sums its real space over a neighbour list
  long long rpart = 0, kpart = 0;
  bool multi = false;
};

// distinct +-k representatives of the reference's cube (v25/functions.cpp:1725-1744)
void k_vectors(const mdsc_system_desc& d, std::vector<int4>& kn) {
  const int K = d.K_max;
  for (int nz = 0; nz < K; ++nz)
    for (int ny = -(K - 1); ny < K; ++ny)
      for (int nx = -(K - 1); nx < K; ++nx) {
        const bool half = nz > 0 || (nz == 0 && ny > 0) || (nz == 0 && ny == 0 && nx > 0);
        if (!half) continue;
        if (d.ksq_max > 0 && nx * nx + ny * ny + nz * nz > d.ksq_max) continue;
        // w = 1: n is the previous k-vector's n + (1, 0, 0), so the gathers'
        // phase n . u advances by u_x alone (exactly, modulo 2^32)
        const bool next = !kn.empty() && kn.back().x == nx - 1 && kn.back().y == ny && kn.back().z == nz;
        kn.push_back(make_int4(nx, ny, nz, next ? 1 : 0));
      }
}

std::string check_desc(const mdsc_system_desc& d, int s) {
  char buf[256];
  if (d.n < 0 || d.nd < 0 || d.nd > MDSC_MAX_DIPOLES) {
    snprintf(buf, sizeof buf, "system %d: n=%d nd=%d out of range", s, d.n, d.nd);
    return buf;
  }
  for (int a = 0; a < 3; ++a)
    if (!(d.box[a] > 0)) {
      snprintf(buf, sizeof buf, "system %d: box edge %d not positive", s, a);
      return buf;
    }
  if (d.K_max < 1 || d.alpha <= 0 || d.dt <= 0 || d.Q <= 0) {
    snprintf(buf, sizeof buf, "system %d: K_max, alpha, dt and Q must be positive", s);
    return buf;
  }
  if (!(d.rc_real >= 0.0)) {
    snprintf(buf, sizeof buf, "system %d: rc_real must be 0 (all pairs) or positive", s);
    return buf;
  }
  const double hd = 0.5 * std::sqrt(d.box[0] * d.box[0] + d.box[1] * d.box[1] + d.box[2] * d.box[2]);
  if (hd >= kTableRmax) {
    snprintf(buf, sizeof buf,
             "system %d: half box diagonal %.3f exceeds the reference's real-space table (r <= %.1f)",
             s, hd, kTableRmax);
    return buf;
  }
  return "";
}

// constants of the real-space tiles as float-float pairs: the exponent's
// alpha sqrt(log2 e) and the fixed-point scale L / 2^32, split on the host so
// that the tiles do no FP64 work
// entries 0..n-1 of the reference's table: A, B, C at r = Lh (k + 1), with
// tabul's own expressions and order of operations (v25/functions.cpp:1680-1697)
void table_values(double alpha, int n, double* T) {
  const double extL = 200 * 1.001;
  const double alsq = alpha * alpha;
  const double alft = alsq * alsq;
  const double spi = std::sqrt(M_PI);
  for (int i = 1; i <= n; i++) {
    const double r = 0.5 * extL * i / 32768;
    const double rsq = r * r;
    const double sr1 = 1.0 / r;
    const double sr2 = sr1 * sr1;
    const double sr3 = sr2 * sr1;
    const double ERFC = std::erfc(alpha * r);
    const double aer = 2.0 * alpha * std::exp(-alsq * rsq) / spi;
    const double aa = 2.0 * alsq + 3.0 * sr2;
    T[3 * (i - 1) + 0] = ERFC * sr3 + aer * sr2;
    T[3 * (i - 1) + 1] = (3.0 * ERFC * sr3 + aer * aa) * sr2;
    T[3 * (i - 1) + 2] = 4. * alft * aer;
  }
}

// One system's table as stored on the device: per entry (A, B, C, dA) and
// (dB, dC, 0, 0), the differences to the next entry.  rc > 0: the entries
// beyond the real-space cutoff zeroed (Lh (k + 1) > rc), before the
// differences are taken.  scaled: the short table of the analytic tiles,
// whose pair step measures lengths in units of 1/s (set_real_consts):
// A / s^3, B / s^5 and C / s^5, in FP64 before rounding.
std::vector<float4> table_entries(double alpha, int n, double rc, bool scaled) {
  std::vector<double> T(3 * (size_t)(n + 1));
  table_values(alpha, n + 1, T.data());
  if (rc > 0)
    for (int k = 0; k <= n; ++k)
      if (0.5 * (200 * 1.001) * (k + 1) / 32768 > rc) T[3 * (size_t)k] = T[3 * (size_t)k + 1] = T[3 * (size_t)k + 2] = 0.0;
  if (scaled) {
    const double s = alpha * 1.2011224087864498, s3 = s * s * s, s5 = s3 * s * s;
    for (int k = 0; k <= n; ++k) {
      T[3 * (size_t)k] /= s3;
      T[3 * (size_t)k + 1] /= s5;
      T[3 * (size_t)k + 2] /= s5;
    }
  }
  std::vector<float4> e(2 * (size_t)n);
  for (int k = 0; k < n; ++k) {
    const double* a = &T[3 * (size_t)k];
    const double* b = &T[3 * (size_t)(k + 1)];
    e[2 * (size_t)k] = make_float4((float)a[0], (float)a[1], (float)a[2], (float)(b[0] - a[0]));
    e[2 * (size_t)k + 1] = make_float4((float)(b[1] - a[1]), (float)(b[2] - a[2]), 0.f, 0.f);
  }
  return e;
}

// Tables are a pure function of (alpha, entries) and take ~1 ms each to
// build, so a process keeps the recent ones: a server that rebuilds its
// batch whenever jobs come and go finds the running systems' tables here.
// Least recently used tables leave first, above kTableCacheBytes.
constexpr size_t kTableCacheBytes = size_t(256) << 20;
struct TableCache {
  std::mutex mu;
  std::map<std::tuple<uint64_t, uint64_t, int, bool>, std::pair<std::vector<float4>, uint64_t>> m;  // -> (entries, last use)
  uint64_t clock = 0;
  size_t bytes = 0;
};
TableCache g_tables;

void fill_tables(const mdsc_system_desc* descs, Layout& Lo) {
  Lo.rtab.assign(Lo.rtab_n, make_float4(0.f, 0.f, 0.f, 0.f));
  const int nsys = (int)Lo.sys.size();
  // the analytic tiles' short tables are stored scaled (table_entries)
  auto scaled = [&](int s) { return !Lo.rp_table && !(descs[s].rc_real > 0); };
  auto key_of = [&](int s) {
    uint64_t a, c;
    memcpy(&a, &descs[s].alpha, 8);
    memcpy(&c, &descs[s].rc_real, 8);
    return std::make_tuple(a, c, Lo.sys[s].rt_n, scaled(s));
  };
  // systems whose table is not cached: build them on all host threads
  std::vector<int> miss;
  {
    std::lock_guard<std::mutex> g(g_tables.mu);
    std::map<std::tuple<uint64_t, uint64_t, int, bool>, int> first;
    for (int s = 0; s < nsys; ++s) {
      if (Lo.sys[s].rt_n <= 0) continue;
      const auto k = key_of(s);
      auto it = g_tables.m.find(k);
      if (it != g_tables.m.end()) {
        it->second.second = ++g_tables.clock;
        std::copy(it->second.first.begin(), it->second.first.end(), Lo.rtab.begin() + 2 * (size_t)Lo.sys[s].rt_off);
      } else if (first.emplace(k, s).second) {
        miss.push_back(s);
      }
    }
  }
  if (!miss.empty()) {
    std::vector<std::vector<float4>> built(miss.size());
    const int nth = (int)std::max(1u, std::min<unsigned>(std::thread::hardware_concurrency(), (unsigned)miss.size()));
    std::atomic<int> next{0};
    auto work = [&] {
      for (int q; (q = next.fetch_add(1)) < (int)miss.size();)
        built[q] = table_entries(descs[miss[q]].alpha, Lo.sys[miss[q]].rt_n, descs[miss[q]].rc_real, scaled(miss[q]));
    };
    std::vector<std::thread> th;
    for (int t = 1; t < nth; ++t) th.emplace_back(work);
    work();
    for (auto& t : th) t.join();
    std::lock_guard<std::mutex> g(g_tables.mu);
    for (size_t q = 0; q < miss.size(); ++q) {
      const auto k = key_of(miss[q]);
      if (g_tables.m.count(k)) continue;
      g_tables.bytes += sizeof(float4) * built[q].size();
      g_tables.m[k] = std::make_pair(std::move(built[q]), ++g_tables.clock);
    }
    while (g_tables.bytes > kTableCacheBytes && g_tables.m.size() > 1) {
      auto old = g_tables.m.begin();
      for (auto it = g_tables.m.begin(); it != g_tables.m.end(); ++it)
        if (it->second.second < old->second.second) old = it;
      g_tables.bytes -= sizeof(float4) * old->second.first.size();
      g_tables.m.erase(old);
    }
  }
  // every system, in order, from the cache or a sibling with the same key
  std::lock_guard<std::mutex> g(g_tables.mu);
  for (int s = 0; s < nsys; ++s) {
    if (Lo.sys[s].rt_n <= 0) continue;
    auto it = g_tables.m.find(key_of(s));
    if (it != g_tables.m.end()) {
      std::copy(it->second.first.begin(), it->second.first.end(), Lo.rtab.begin() + 2 * (size_t)Lo.sys[s].rt_off);
    } else {  // evicted at once (cache smaller than this batch's tables): build here
      const std::vector<float4> e = table_entries(descs[s].alpha, Lo.sys[s].rt_n, descs[s].rc_real, scaled(s));
      std::copy(e.begin(), e.end(), Lo.rtab.begin() + 2 * (size_t)Lo.sys[s].rt_off);
    }
  }
}

void make_layout(const mdsc_system_desc* descs, int nsys, Layout& Lo) {
  Lo.sys.resize(nsys);
  const char* form_env = std::getenv("MDSC_REAL_FORM");
  Lo.rp_table = form_env && std::strcmp(form_env, "table") == 0;
  int part = 0, dip = 0, blk = 0;
  long long pp = 0, kp = 0;
  for (int s = 0; s < nsys; ++s) {
    const mdsc_system_desc& d = descs[s];
    SysDev& P = Lo.sys[s];
    memset(&P, 0, sizeof P);
    P.n = d.n;
    P.nd = d.nd;
    P.ndip = d.n * d.nd;
    P.part_off = part;
    P.dip_off = dip;
    // the all-pairs tiles (rc_real = 0) or the neighbour-list pass (rc_real > 0)
    P.rc_real = d.rc_real;
    if (d.rc_real > 0) Lo.any_rc = true;
    P.nstrip = d.rc_real > 0 ? 0 : cdiv(P.ndip, kTile);
    P.strip_off = Lo.nstrips;
    Lo.nstrips += P.nstrip;
    P.pp_off = pp;
    pp += (long long)P.nstrip * P.nstrip * 6 * kTile;
    P.tile_off = (int)Lo.tiles.size();
    for (int I = 0; I < P.nstrip; ++I)
      for (int J = I; J < P.nstrip; ++J) Lo.tiles.push_back(make_int4(s, I, J, 0));
    P.ntile = (int)Lo.tiles.size() - P.tile_off;
    if (P.nstrip > kStripRows)
      for (int X = 0; X < P.nstrip; ++X) Lo.bstrips.push_back(make_int2(s, X));
    // k-vectors and their prefactors (wave_v, v25/functions.cpp:1963-1990)
    P.k_off = (int)Lo.kn.size();
    std::vector<int4> kn;
    if (d.nd > 0) k_vectors(d, kn);
    const double V = d.box[0] * d.box[1] * d.box[2];
    const double c = 4. * d.alpha * d.alpha;
    const double a4 = 1. / (4. * d.alpha);
    for (const int4& n : kn) {
      const double kx = 2. * M_PI / d.box[0] * n.x, ky = 2. * M_PI / d.box[1] * n.y,
                   kz = 2. * M_PI / d.box[2] * n.z;
      const double ksq = kx * kx + ky * ky + kz * kz;
      const double KK = 4. * M_PI * std::exp(-ksq / c) / ksq;
      const double val = 2. * KK / V;
      Lo.kn.push_back(n);
      Lo.kv.push_back(make_float4((float)kx, (float)ky, (float)kz, (float)val));
      Lo.kval.push_back(val);
      Lo.kvec.push_back(kx);
      Lo.kvec.push_back(ky);
      Lo.kvec.push_back(kz);
      Lo.kpre.push_back(2 * (a4 + 1. / ksq));  // pval (v25/functions.cpp:1715,1738)
      Lo.kowner.push_back(make_int2(s, (int)(Lo.kn.size() - 1 - P.k_off)));
    }
    P.nk = (int)kn.size();
    P.nkchunk = P.nk > 0 ? cdiv(d.n, kKChunk) : 0;
    P.kchunk_off = (int)kp;
    kp += (long long)P.nkchunk * P.nk;
    P.gch_off = Lo.nchunks;
    Lo.nchunks += P.nkchunk;
    for (int ch = 0; ch < P.nkchunk; ++ch)
      for (int kt = 0; kt < cdiv(P.nk, kKBlock); ++kt) Lo.kwork.push_back(make_int4(s, ch, kt, 0));
    // cell capacity of the list build: at most one cell per 8 rods (the
    // grid is chosen at upload, when the shapes are known)
    P.cell_off = Lo.ncellcap;
    P.cell_cap = d.n >= kCellMinRods ? d.n / 8 : 0;
    for (int c = 0; c < P.cell_cap; c += 2) Lo.cellblk.push_back(make_int2(s, c));
    Lo.ncellcap += P.cell_cap;
    P.blk_off = blk;
    P.nblk = cdiv(d.n, kPartBlock);
    for (int k = 0; k < P.nblk; ++k) Lo.blk.push_back(make_int2(s, part + k * kPartBlock));
    // the k-space gather of a large single-dipole system runs its k tiles in
    // parts on separate blocks (a function of the system only, so the same
    // bits alone and in any batch); smaller systems fill the GPU as they
    // are (split for every single-dipole system, the 256-replica mix's
    // gather went from 0.107 to 0.117 ms: the parts' partial sums and their
    // combination cost more than the added blocks gained)
    const int ktiles = cdiv(P.nk, kKBlock);
    P.kgs = (d.nd == 1 && d.n >= 4096 && ktiles > 1) ? std::min(8, ktiles) : 1;
    P.kgp_off = (int)Lo.kgsets;
    if (P.kgs > 1) Lo.kgsets += (long long)P.nblk * P.kgs;
    blk += P.nblk;
    P.cl_fr = d.cl_fr;
    for (int a = 0; a < 3; ++a) {
      P.L[a] = d.box[a];
      P.invL[a] = 1.0 / d.box[a];
      P.invL32[a] = P.invL[a] * 4294967296.0;
      P.Lfix[a] = (float)(d.box[a] / 4294967296.0);
      P.Lf[a] = (float)d.box[a];
      P.B[a] = d.B[a];
    }
    P.V = V;
    P.alpha = d.alpha;
    P.dt = d.dt;
    P.temp = d.temp;
    P.Q = d.Q;
    P.gamma = d.gamma;
    P.ex1 = std::exp(-d.gamma * d.dt / 2);
    P.cnoise = std::sqrt(2. * d.temp * d.gamma * d.dt / d.Q);
    P.ntemp3 = 3. * d.n * d.temp;
    P.min_s = d.min_s;
    set_real_consts(P, kLh);
    // the reference's interpolation table (tabul, v25/functions.cpp:1680-1704)
    // in FP64 as tabul computes it, stored as FP32 values and differences to
    // the next entry: over the distances the box can hold for the neighbour
    // pass of a system with a real-space cutoff and for tiles that read it
    // (MDSC_REAL_FORM=table); up to r = kNearTab for the analytic tiles,
    // which interpolate in it for near-contact pairs only
    if (d.nd > 0) {
      const double hd = 0.5 * std::sqrt(d.box[0] * d.box[0] + d.box[1] * d.box[1] + d.box[2] * d.box[2]);
      int n = std::min((int)std::floor(hd / kLh) + 3, 32767);
      if (!Lo.rp_table && !(d.rc_real > 0)) n = std::min(n, (int)std::ceil(kNearTab / kLh) + 3);
      P.rt_off = (int)(Lo.rtab_n / 2);
      P.rt_n = n;
      Lo.rtab_n += 2 * (size_t)n;
    }
    part += d.n;
    dip += P.ndip;
    Lo.maxnd = std::max(Lo.maxnd, d.nd);
    if (d.nd > 1) Lo.multi = true;
  }
  // real-space tiles: one by one, each evaluating the analytic terms with
  // the table's interpolation error added (no lookups: bound by the FP32
  // pipe alone).  MDSC_REAL_FORM=table reads the system's table from
  // global memory instead (one scattered 32-byte lookup per pair, bound by
  // the L1).  With that and MDSC_SMEM_TABLE=1, systems whose table fits a
  // block's shared memory run in runs of kSmemChunk tiles (the longest runs
  // first) on the shared-table form: 11% faster than the global table
  // alone, but its whole-SM blocks wait for free SMs beside the step's
  // other chains, and the step was 10% slower on the 256-replica mix
  const char* smem_env = std::getenv("MDSC_SMEM_TABLE");
  const bool smem_ok = Lo.rp_table && smem_env && smem_env[0] == '1';
  for (int s = 0; s < nsys; ++s) {
    const SysDev& P = Lo.sys[s];
    if (P.ntile == 0) continue;
    if (smem_ok && P.rt_n > 0 && P.rt_n <= kSmemTableMax) {
      for (int t = 0; t < P.ntile; t += kSmemChunk)
        Lo.rpwork.push_back(make_int4(s, P.tile_off + t, std::min(kSmemChunk, P.ntile - t), 0));
      Lo.smem_tn = std::max(Lo.smem_tn, P.rt_n);
    } else {
      for (int t = 0; t < P.ntile; ++t) Lo.gtile.push_back(P.tile_off + t);
    }
  }
  std::stable_sort(Lo.rpwork.begin(), Lo.rpwork.end(), [](const int4& u, const int4& v) { return u.z > v.z; });
  // launch the particle blocks of the largest systems first: their blocks
  // run longest (real-space partials over more strips), so they must not
  // be the last wave on the GPU.  Kernels find a block's partial-sum slot
  // from its particle range (blk_slot), so results do not depend on this
  // order.
  std::stable_sort(Lo.blk.begin(), Lo.blk.end(),
                   [&](const int2& u, const int2& v) { return descs[u.x].n > descs[v.x].n; });
  // the k-space gather's blocks: every part of every particle block, in the
  // launch order above (entries index the sorted block list)
  for (int g = 0; g < (int)Lo.blk.size(); ++g)
    for (int q = 0; q < Lo.sys[Lo.blk[g].x].kgs; ++q) Lo.kgwork.push_back(make_int2(g, q));
  Lo.ntot = part;
  Lo.ndtot = dip;
  Lo.nktot = (int)Lo.kn.size();
  Lo.rpart = pp;
  Lo.kpart = kp;
}

struct Arena {
  size_t off = 0;
  char* base = nullptr;
  template <class T>
  T* take(size_t count) {
    const size_t bytes = ((count * sizeof(T) + 255) / 256) * 256;
    T* p = base ? reinterpret_cast<T*>(base + off) : nullptr;
    off += bytes ? bytes : 256;
    return p;
  }
};

// carves every buffer of a batch out of one allocation (or only sizes it)
void carve(Arena& A, const Layout& Lo, int nsys, Batch& b, int4** kwork, int2** kowner,
           double** noise2, int** skip) {
  const size_t n = std::max(Lo.ntot, 1), nd = std::max(Lo.ndtot, 1), nk = std::max(Lo.nktot, 1);
  const size_t nt = std::max<size_t>(Lo.tiles.size(), 1), nb = std::max<size_t>(Lo.blk.size(), 1);
  b.sys = A.take<SysDev>(nsys);
  b.st = A.take<SysState>(nsys);
  b.obs = A.take<SysObs>(nsys);
  b.r = A.take<double>(3 * n);
  b.p = A.take<double>(3 * n);
  b.O = A.take<double>(9 * n);
  b.l = A.take<double>(3 * n);
  b.F = A.take<double>(3 * n);
  b.T = A.take<double>(3 * n);
  b.len = A.take<double>(n);
  b.dia = A.take<double>(n);
  b.mass = A.take<double>(n);
  b.inert = A.take<double>(3 * n);
  b.invm = A.take<double>(n);
  b.invI = A.take<double>(3 * n);
  b.psys = A.take<int>(n);
  b.dpc = A.take<double>(nd);
  b.dob = A.take<double>(3 * nd);
  b.dmu = A.take<double>(nd);
  b.downer = A.take<int>(nd);
  b.pfx = A.take<uint32_t>(3 * n);
  b.pax = A.take<float4>(n);
  b.pdia = A.take<float>(n);
  b.dfx = A.take<uint32_t>(3 * nd);
  b.dm = A.take<float>(3 * nd);
  b.rpart = A.take<float>(std::max<long long>(Lo.rpart, 1));
  b.rsum = A.take<float2>(6 * (size_t)std::max(Lo.ndtot, 1));
  b.tileE = A.take<float>(10 * nt);
  b.stripE = A.take<double>(10 * (size_t)std::max(Lo.nstrips, 1));
  b.bstrips = A.take<int2>(std::max<size_t>(Lo.bstrips.size(), 1));
  b.kgwork = A.take<int2>(std::max<size_t>(Lo.kgwork.size(), 1));
  b.kgpart = A.take<float>(std::max<long long>(Lo.kgsets, 1) * kPartBlock * 12);
  b.kgdone = A.take<int>(nb);
  b.rnb = A.take<int>(Lo.any_rc ? n * kMaxR : 1);
  b.rnbc = A.take<int>(n);
  b.rlE = A.take<double>(10 * nb);
  b.tiles = A.take<int4>(nt);
  b.rpwork = A.take<int4>(std::max<size_t>(Lo.rpwork.size(), 1));
  b.gtile = A.take<int>(std::max<size_t>(Lo.gtile.size(), 1));
  b.wlist = A.take<int2>(n * kMaxC);
  b.wlist_n = A.take<int>(1);
  b.wown = A.take<double>(n * kMaxC * 6);
  b.wev = A.take<double>(n * kMaxC * 11);
  b.wcaE = A.take<double>(11 * nb);
  b.wcand = A.take<int>(n * kMaxC);
  b.wcnt = A.take<int>(n);
  b.win = A.take<int>(n * kMaxC);
  b.wincnt = A.take<int>(n);
  b.wrec = A.take<double>(n * kMaxC * 6);
  b.kn = A.take<int4>(nk);
  b.kv = A.take<float4>(nk);
  b.rtab = A.take<float4>(std::max<size_t>(Lo.rtab_n, 1));
  b.kval = A.take<double>(nk);
  b.kvec = A.take<double>(3 * nk);
  b.kpre = A.take<double>(nk);
  b.kpart = A.take<float>(10 * std::max<long long>(Lo.kpart, 1));
  b.ksum = A.take<double>(10 * nk);
  b.kS = A.take<float2>(nk);
  b.kE = A.take<double>(10 * nk);
  b.kG = A.take<double>(6 * (size_t)std::max(Lo.nchunks, 1));
  b.kGs = A.take<double>(6 * (size_t)std::max(nsys, 1));
  b.kgcnt = A.take<int>(std::max(nsys, 1));
  b.icnt = A.take<int>(std::max(nsys, 1));
  b.Fk = A.take<float2>(3 * nd);
  b.Tk = A.take<float2>(3 * nd);
  b.kin1 = A.take<double>(2 * nb);
  b.kin2 = A.take<double>(9 * nb);
  b.dmax = A.take<double>(nb);
  b.obk = A.take<double>(12 * nb);
  b.blk = A.take<int2>(nb);
  b.ccnt = A.take<int>(std::max(Lo.ncellcap, 1));
  b.cpos = A.take<uint4>((size_t)std::max(Lo.ncellcap, 1) * kCellSlots);
  b.cax = A.take<float4>((size_t)std::max(Lo.ncellcap, 1) * kCellSlots);
  b.cellblk = A.take<int2>(std::max<size_t>(Lo.cellblk.size(), 1));
  b.nb = A.take<int>(n * kMaxNb);
  b.nbc = A.take<int>(n);
  b.fsave = A.take<uint32_t>(3 * n);
  b.usave = A.take<float>(3 * n);
  b.comp = A.take<int>(n);
  b.eflag = A.take<unsigned char>(n * kMaxNb);
  b.flag = A.take<int>(1);
  b.ebond = A.take<int>(n * kMaxC);
  b.ebcnt = A.take<int>(n);
  b.eovf = A.take<int>(std::max(nsys, 1));
  *kwork = A.take<int4>(std::max<size_t>(Lo.kwork.size(), 1));
  *kowner = A.take<int2>(nk);
  noise2[0] = A.take<double>((size_t)kNoiseChunk * nsys * 4);
  noise2[1] = A.take<double>((size_t)kNoiseChunk * nsys * 4);
  *skip = A.take<int>(std::max(nsys, 1));
}

}  // namespace

struct mdsc_batch {
  int device = 0;
  int num_sms = 0;  // streaming multiprocessors of the device
  int nsys = 0;
  cudaStream_t st = nullptr, s2 = nullptr, s3 = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_j2 = nullptr, ev_j3 = nullptr;
  // mdsc_step_io: the stream that takes positions and orientations home
  // while a step's forces are computed, and the event its graph records
  // once they are final
  cudaStream_t sio = nullptr;
  cudaEvent_t ev_x = nullptr;
  cudaEvent_t ev_f = nullptr;  // recorded by the same graph once the force assembly has run
  std::vector<mdsc_system_desc> desc;
  Layout lo;
  Batch b{};
  int4* kwork = nullptr;
  int2* kowner = nullptr;
  double* noise[2] = {nullptr, nullptr};
  int* d_skip = nullptr;      // per system: skipped by a force evaluation of the others
  double* h_noise = nullptr;  // pinned, the draws of a run of steps (noise buffer 0)
  double* h_noise2 = nullptr; // the same for noise buffer 1: the host draws a run while the last one's copy runs
  cudaEvent_t ev_noise[2] = {nullptr, nullptr};  // the last copy out of each
  SysObs* h_obs = nullptr;    // pinned
  SysObs* h_trace = nullptr;  // pinned, kNoiseChunk x nsys: per-step observables of mdsc_step_trace
  char* arena = nullptr;
  size_t arena_bytes = 0;
  std::vector<Mt19937> thermo_rng;  // 2 per system
  std::vector<Mt19937> clus_rng;    // 1 per system
  std::vector<long long> step_h;
  std::vector<long long> stop_h;  // the systems' step limits (LLONG_MAX: none)
  std::vector<std::vector<int>> labels;
  std::vector<int> n_clusters;
  std::vector<char> uploaded, built, have_forces;
  std::vector<std::vector<int>> species;  // per system: particles per species (contiguous blocks)
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  cudaGraphExec_t graph_io[2] = {nullptr, nullptr};  // the same step, with ev_x after the first half-step
  cudaEvent_t t_beg = nullptr, t_end = nullptr;  // device time of the last mdsc_step
  double last_ms = 0.0;
  int launches = 0;
  int tuned = 0;          // launch mappings chosen (autotuner or cache)
  std::string tune_log;   // the autotuner's timings, for mdsc_tuning
  std::string err;
};

namespace {

mdsc_status fail(mdsc_batch* b, mdsc_status code, const std::string& msg) {
  if (b) b->err = msg;
  return code;
}

#define CU(call)                                                                              \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess)                                                                    \
      return fail(B, e_ == cudaErrorMemoryAllocation ? MDSC_ERR_OOM : MDSC_ERR_CUDA,          \
                  std::string(#call) + ": " + cudaGetErrorString(e_));                        \
  } while (0)

mdsc_status status_from_bits(int bits) {
  if (bits & kErrOverlap) return MDSC_ERR_OVERLAP;
  if (bits & kErrNan) return MDSC_ERR_NAN;
  if (bits & kErrListOverflow) return MDSC_ERR_LIST_OVERFLOW;
  if (bits & kErrTable) return MDSC_ERR_TABLE_RANGE;
  return MDSC_OK;
}

Batch batch_with_noise(const mdsc_batch* B, int which) {
  Batch b = B->b;
  b.noise = B->noise[which];
  return b;
}

// every force term, F and T set from scratch, energies reduced; with a
// skip mask (device, per system) the flagged systems are left as they are
mdsc_status eval_forces(mdsc_batch* B, int force_list, const int* skip = nullptr) {
  Batch b = batch_with_noise(B, 0);
  b.skip = skip;
  launch_derive(b, B->st);
  launch_list_build(b, force_list, B->st);
  launch_wca(b, 1, B->st);  // with the cutoff systems' real space, in the same neighbour pass
  launch_real_pairs(b, B->lo.multi, B->st);
  launch_real_sum(b, B->st);
  launch_kspace(b, B->lo.maxnd, B->kwork, (int)B->lo.kwork.size(), B->kowner, b.kE, B->st);
  launch_finalize(b, kMaskAll, B->st);
  launch_order_terms(b, B->st);
  launch_reduce_obs(b, kRedEnergies, B->st);
  CU(cudaGetLastError());
  for (int s = 0; s < B->nsys; ++s) {
    B->built[s] = 1;
    B->have_forces[s] = 1;
  }
  return MDSC_OK;
}

mdsc_status ensure_forces(mdsc_batch* B);

// ---------------------------------------------------------------------
// autotuner: launch mappings timed on the batch's own state
// ---------------------------------------------------------------------
// Only mappings that leave every result unchanged are tuned (Tuning,
// mdsc_dev.cuh), so a system gives the same bits whatever batch it runs in
// and whatever the tuner picks.  Choices are cached per process by a size
// class of the batch (tiles, particles, k-vectors: half-octaves), so a
// server that repacks batches of similar size tunes once.
struct TuneKey {
  int tiles, parts, ks, maxnd, sms;
  bool operator<(const TuneKey& o) const {
    return std::tie(tiles, parts, ks, maxnd, sms) < std::tie(o.tiles, o.parts, o.ks, o.maxnd, o.sms);
  }
};
std::mutex g_tune_mu;
std::map<TuneKey, Tuning> g_tune_cache;

TuneKey tune_key(const mdsc_batch* B) {
  auto cls = [](long long x) { return x <= 0 ? -1 : (int)std::lround(2.0 * std::log2((double)x)); };
  return TuneKey{cls(B->b.ntiles), cls(B->lo.ntot), cls(B->b.nktot), B->lo.maxnd, B->num_sms};
}

// average device time (ms) of `launch` over `reps` runs after one warm-up
template <class F>
double time_launches(mdsc_batch* B, int reps, F&& launch) {
  launch();
  cudaEventRecord(B->t_beg, B->st);
  for (int r = 0; r < reps; ++r) launch();
  cudaEventRecord(B->t_end, B->st);
  cudaEventSynchronize(B->t_end);
  float t = 0.f;
  cudaEventElapsedTime(&t, B->t_beg, B->t_end);
  return t / reps;
}

mdsc_status autotune(mdsc_batch* B, int force, int reps) {
  const TuneKey key = tune_key(B);
  if (!force) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
      B->b.tune = it->second;
      B->tuned = 1;
      return MDSC_OK;
    }
  }
  mdsc_status st = ensure_forces(B);
  if (st) return st;
  Batch b = batch_with_noise(B, 0);
  Tuning best = b.tune;
  B->tune_log.clear();
  char line[160];
  auto pick = [&](const char* what, const int* cand, int nc, int& field, auto&& launch) {
    double tbest = 1e30;
    int vbest = field;
    for (int k = 0; k < nc; ++k) {
      field = cand[k];
      const double t = time_launches(B, reps, launch);
      snprintf(line, sizeof line, "%s=%d %.4f ms; ", what, cand[k], t);
      B->tune_log += line;
      if (t < tbest) {
        tbest = t;
        vbest = cand[k];
      }
    }
    field = vbest;
  };
  // WCA evaluation grid (the screen runs with it: it refills the work list)
  {
    const int m = B->num_sms;
    const int cand[4] = {m * 2, m * 4, m * 8, m * 16};
    pick("wca_blocks", cand, 4, b.tune.wca_blocks, [&] { launch_wca(b, 0, B->st); });
  }
  // real-space tiles per block, then the strip-sum block size
  if (b.ntiles > 0) {
    const int cand[3] = {1, 2, 4};
    pick("rp_warps", cand, 3, b.tune.rp_warps, [&] { launch_real_pairs(b, B->lo.multi, B->st); });
    const int cand2[3] = {128, 256, 512};
    pick("rsum_threads", cand2, 3, b.tune.rsum_threads, [&] { launch_real_sum(b, B->st); });
  }
  // k-space gather form (single-dipole systems)
  if (b.nktot > 0 && B->lo.maxnd <= 1) {
    launch_kspace_parts(b, B->lo.maxnd, B->kwork, (int)B->lo.kwork.size(), B->kowner, b.kE, 0, B->st);
    launch_kspace_parts(b, B->lo.maxnd, B->kwork, (int)B->lo.kwork.size(), B->kowner, b.kE, 1, B->st);
    const int cand[2] = {0, 1};
    pick("kg_scalar", cand, 2, b.tune.kg_scalar, [&] {
      launch_kspace_parts(b, B->lo.maxnd, B->kwork, (int)B->lo.kwork.size(), B->kowner, b.kE, 2, B->st);
    });
  }
  CU(cudaStreamSynchronize(B->st));
  CU(cudaGetLastError());
  best = b.tune;
  B->b.tune = best;
  B->tuned = 1;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache[key] = best;
  }
  return MDSC_OK;
}

// io: the variant for mdsc_step_io, which also records ev_x (an event
// outside the graph) once the first half-step has moved every particle:
// positions and orientations are final from there on
mdsc_status capture_step(mdsc_batch* B, int which, bool io = false) {
  Batch b = batch_with_noise(B, which);
  b.honor_stop = 1;  // systems at their step limit take no step
  cudaGraph_t g = nullptr;
  CU(cudaStreamBeginCapture(B->st, cudaStreamCaptureModeThreadLocal));
  int launches = 0;
  launch_integrate_first(b, B->st);
  ++launches;
  if (io) cudaEventRecordWithFlags(B->ev_x, B->st, cudaEventRecordExternal);
  cudaEventRecord(B->ev_fork, B->st);
  cudaStreamWaitEvent(B->s2, B->ev_fork, 0);
  cudaStreamWaitEvent(B->s3, B->ev_fork, 0);
  launch_order_terms(b, B->st);
  launch_list_build(b, 0, B->st);
  launch_wca(b, 1, B->st);  // the cutoff systems' real space in their neighbour pass, after their list
  // order terms, the list build's decision and scan (+ the cell binning),
  // the WCA screen and evaluation (+ the cutoff pass)
  launches += 5 + (b.cells && b.ncellblk ? 1 : 0) + (b.any_rc ? 1 : 0);
  launch_real_pairs(b, B->lo.multi, B->s2);
  launch_real_sum(b, B->s2);
  launches += b.ntiles > 0 ? 2 + (b.nbstrips > 0 ? 1 : 0) : 0;
  launch_kspace(b, B->lo.maxnd, B->kwork, (int)B->lo.kwork.size(), B->kowner, b.kE, B->s3);
  launches += b.nktot > 0 ? (B->lo.maxnd > 1 ? 5 : 3) : 0;  // multi-dipole batches: both ksum and kgather forms
  cudaEventRecord(B->ev_j2, B->s2);
  cudaEventRecord(B->ev_j3, B->s3);
  cudaStreamWaitEvent(B->st, B->ev_j2, 0);
  cudaStreamWaitEvent(B->st, B->ev_j3, 0);
  launch_finalize(b, kMaskAll | kFlagMoveP, B->st);
  if (io) cudaEventRecordWithFlags(B->ev_f, B->st, cudaEventRecordExternal);
  launch_reduce_obs(b, kRedStep, B->st);
  launches += 2;
  cudaError_t e = cudaStreamEndCapture(B->st, &g);
  if (e != cudaSuccess) return fail(B, MDSC_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
  e = cudaGraphInstantiate(io ? &B->graph_io[which] : &B->graph[which], g, cudaGraphInstantiateFlagUseNodePriority);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(B, MDSC_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
  if (!io) B->launches = launches;
  return MDSC_OK;
}

// every step graph, to be captured again (new launch mappings or list mode)
void drop_graphs(mdsc_batch* B) {
  for (cudaGraphExec_t* set : {B->graph, B->graph_io})
    for (int w = 0; w < 2; ++w)
      if (set[w]) {
        cudaGraphExecDestroy(set[w]);
        set[w] = nullptr;
      }
}

// thermostat noise of `steps` steps for every system, drawn as moveTher
// mode 0 draws it (v25/functions.cpp:2194-2197): two uniforms per
// thermostat, Box-Muller, first value now, second stored for mode 2
void draw_noise(mdsc_batch* B, int steps, double* h) {
  for (int k = 0; k < steps; ++k)
    for (int s = 0; s < B->nsys; ++s) {
      if (B->step_h[s] + k >= B->stop_h[s]) continue;  // at its step limit: no step, no draw
      double* o = h + ((size_t)k * B->nsys + s) * 4;
      for (int t = 0; t < 2; ++t) {
        Mt19937& g = B->thermo_rng[2 * s + t];
        double r1 = g.uniform(), r2 = g.uniform();
        box_muller(r1, r2);
        o[2 * t] = r1;
        o[2 * t + 1] = r2;
      }
    }
}

// connected components on the GPU, then the reference's labelling order on
// the host: repeatedly draw u, take the floor(u * remaining)-th remaining
// particle in index order, label its whole component (v25/functions.cpp:
// 2950-2970,3282-3313)
mdsc_status run_clusters(mdsc_batch* B, const std::vector<int>& systems) {
  Batch b = B->b;
  launch_cluster_bonds(b, B->st);
  bool energy = false;
  for (int s = 0; s < B->nsys; ++s) energy |= B->lo.sys[s].cl_mode == 1;
  if (energy) {
    CU(cudaMemsetAsync(b.eovf, 0, sizeof(int) * B->nsys, B->st));
    launch_ebond(b, B->st);
    std::vector<int> ovf(B->nsys);
    CU(cudaMemcpyAsync(ovf.data(), b.eovf, sizeof(int) * B->nsys, cudaMemcpyDeviceToHost, B->st));
    CU(cudaStreamSynchronize(B->st));
    for (int s : systems)
      if (ovf[s])
        return fail(B, MDSC_ERR_LIST_OVERFLOW,
                    "system " + std::to_string(s) + ": a particle has more than " + std::to_string(kMaxC) +
                        " energy bonds (or " + std::to_string(kMaxE) + " candidates) to higher indices");
  }
  for (int it = 0; it < 64; ++it) {
    CU(cudaMemsetAsync(b.flag, 0, sizeof(int), B->st));
    launch_cluster_hook(b, B->st);
    launch_cluster_compress(b, B->st);
    int flag = 0;
    CU(cudaMemcpyAsync(&flag, b.flag, sizeof(int), cudaMemcpyDeviceToHost, B->st));
    CU(cudaStreamSynchronize(B->st));
    if (!flag) break;
  }
  CU(cudaGetLastError());
  for (int s : systems) {
    const SysDev& P = B->lo.sys[s];
    std::vector<int> comp(P.n);
    if (P.n)
      CU(cudaMemcpy(comp.data(), b.comp + P.part_off, sizeof(int) * P.n, cudaMemcpyDeviceToHost));
    // members of each component, in index order
    std::vector<int> head(P.n, -1), next(P.n, -1), tail(P.n, -1);
    for (int i = 0; i < P.n; ++i) {
      const int r = comp[i] - P.part_off;
      if (head[r] < 0) head[r] = i;
      else next[tail[r]] = i;
      tail[r] = i;
    }
    Fenwick fw(P.n);
    std::vector<int>& lab = B->labels[s];
    lab.assign(P.n, -1);
    int remaining = P.n, nc = 0;
    Mt19937& g = B->clus_rng[s];
    while (remaining > 0) {
      const double u = g.uniform();
      const int ip = (int)std::floor(u * remaining);
      const int seed = fw.kth(ip);
      const int r = comp[seed] - P.part_off;
      for (int m = head[r]; m >= 0; m = next[m]) {
        lab[m] = nc;
        fw.remove(m);
        --remaining;
      }
      ++nc;
    }
    B->n_clusters[s] = nc;
  }
  return MDSC_OK;
}

void order_params(const double* v, int n, double* G1, double* G2, double* M);

// one system's device observables as the ABI struct
void convert_obs(const SysObs& o, int n, int n_clusters, mdsc_observables& r) {
  memset(&r, 0, sizeof r);
  r.K[0] = o.K[0];
  r.K[1] = o.K[1];
  r.U_ss = o.U_ss;
  r.W_ss = o.W_ss;
  r.U_dipR = o.U_dipR;
  r.U_dipK = o.U_dipK;
  r.U_ext = o.U_ext;
  r.U_self = o.U_self;
  for (int c = 0; c < 9; ++c) {
    r.PT_kin[c] = o.PT_kin[c];
    r.PT_ss[c] = o.PT_ss[c];
    r.PT_dipR[c] = o.PT_dipR[c];
    r.PT_dipK[c] = o.PT_dipK[c];
  }
  r.xi[0] = o.xi[0];
  r.xi[1] = o.xi[1];
  r.step = o.step;
  r.status = status_from_bits(o.status);
  r.n_clusters = n_clusters;
  r.list_builds = o.list_builds;
  order_params(o.osum, n, &r.G1, &r.G2, r.M);
}

// the observables copied to h_obs, to the caller's form and status
mdsc_status finish_obs(mdsc_batch* B, mdsc_observables* out) {
  int bits = 0;
  for (int s = 0; s < B->nsys; ++s) {
    bits |= B->h_obs[s].status;
    if (out) convert_obs(B->h_obs[s], B->lo.sys[s].n, B->n_clusters[s], out[s]);
  }
  const mdsc_status st = status_from_bits(bits);
  if (st != MDSC_OK) return fail(B, st, "a system reported an error (see mdsc_observables.status)");
  return MDSC_OK;
}

mdsc_status read_obs(mdsc_batch* B, mdsc_observables* out) {
  CU(cudaMemcpyAsync(B->h_obs, B->b.obs, sizeof(SysObs) * B->nsys, cudaMemcpyDeviceToHost, B->st));
  CU(cudaStreamSynchronize(B->st));
  return finish_obs(B, out);
}

mdsc_status ensure_forces(mdsc_batch* B) {
  for (int s = 0; s < B->nsys; ++s)
    if (!B->uploaded[s]) return fail(B, MDSC_ERR_STATE, "system " + std::to_string(s) + " has no state yet");
  int missing = 0;
  for (int s = 0; s < B->nsys; ++s) missing += !B->have_forces[s];
  if (missing == 0) return MDSC_OK;
  if (missing == B->nsys) return eval_forces(B, 0);
  // only the systems without forces (those a server just added beside
  // systems moved in with theirs): every kernel returns at once for the
  // others, which keep their forces, lists and bits
  std::vector<int> skip(B->nsys);
  for (int s = 0; s < B->nsys; ++s) skip[s] = B->have_forces[s] ? 1 : 0;
  CU(cudaMemcpyAsync(B->d_skip, skip.data(), sizeof(int) * B->nsys, cudaMemcpyHostToDevice, B->st));
  const mdsc_status st = eval_forces(B, 0, B->d_skip);
  CU(cudaStreamSynchronize(B->st));  // the host flags are read by the copy
  return st;
}

// host-side derived per-particle data of system s from its shape arrays
void shapes_to_host(const mdsc_batch* B, int s, const mdsc_host_state* h, std::vector<double>& inert,
                    std::vector<double>& invm, std::vector<double>& invI, std::vector<double>& dpc,
                    std::vector<double>& dob, std::vector<double>& dmu, std::vector<int>& downer,
                    double& Uself) {
  const SysDev& P = B->lo.sys[s];
  const int n = P.n, nd = P.nd;
  inert.resize(3 * n);
  invm.resize(n);
  invI.resize(3 * n);
  dpc.resize((size_t)n * nd);
  dob.resize((size_t)3 * n * nd);
  dmu.resize((size_t)n * nd);
  downer.resize((size_t)n * nd);
  Uself = 0.0;
  for (int i = 0; i < n; ++i) {
    spherocyl_inertia(h->len[i], h->dia[i], h->mass[i], &inert[3 * i]);
    invm[i] = 1.0 / h->mass[i];
    for (int a = 0; a < 3; ++a) invI[3 * i + a] = 1.0 / inert[3 * i + a];
    for (int w = 0; w < nd; ++w) {
      const double* d = h->dip + ((size_t)i * nd + w) * 5;
      const size_t g = (size_t)i * nd + w;
      dpc[g] = d[0];
      dob[3 * g] = d[1];
      dob[3 * g + 1] = d[2];
      dob[3 * g + 2] = d[3];
      dmu[g] = d[4];
      downer[g] = P.part_off + i;
    }
    // self_ener (v25/functions.cpp:2027-2069): bare dipole-dipole energy of
    // the particle's own dipoles; frame-independent, so the body frame serves
    for (int v = 0; v + 1 < nd; ++v)
      for (int w = v + 1; w < nd; ++w) {
        const double* a = h->dip + ((size_t)i * nd + v) * 5;
        const double* c = h->dip + ((size_t)i * nd + w) * 5;
        const double rij[3] = {0., 0., a[0] - c[0]};
        const double RIJSQ = rij[2] * rij[2];
        const double RIJ = std::sqrt(RIJSQ);
        const double SR2 = 1. / RIJSQ, SR3 = SR2 / RIJ;
        const double UIUJ = a[1] * c[1] + a[2] * c[2] + a[3] * c[3];
        const double UIR = a[3] * rij[2], UJR = c[3] * rij[2];
        Uself += a[4] * c[4] * (UIUJ * SR3 - 3. * UIR * UJR * SR2 * SR3);
      }
  }
}

// ---- observables outside the step: host helpers ------------------------
int corr_bins(const SysDev& P, double bar_w) {
  const double Lmin = std::min(P.L[2], std::min(P.L[1], P.L[0]));
  return (int)std::floor(std::sqrt(3.) * Lmin / (2. * bar_w));
}

// eigenvalues d and eigenvectors (columns of V) of a symmetric 3x3 matrix
// by cyclic Jacobi rotations (Golub & Van Loan, Matrix Computations 8.5)
void sym3_eigen(const double (&A0)[3][3], double (&d)[3], double (&V)[3][3]) {
  double A[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      A[i][j] = A0[i][j];
      V[i][j] = i == j ? 1.0 : 0.0;
    }
  for (int sweep = 0; sweep < 64; ++sweep) {
    const double off = std::fabs(A[0][1]) + std::fabs(A[0][2]) + std::fabs(A[1][2]);
    const double diag = std::fabs(A[0][0]) + std::fabs(A[1][1]) + std::fabs(A[2][2]);
    if (off <= 1e-15 * diag + 1e-300) break;
    for (int p = 0; p < 2; ++p)
      for (int q = p + 1; q < 3; ++q) {
        if (A[p][q] == 0.0) continue;
        const double th = (A[q][q] - A[p][p]) / (2.0 * A[p][q]);
        const double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), sn = t * c;
        for (int k = 0; k < 3; ++k) {
          const double x = A[k][p], y = A[k][q];
          A[k][p] = c * x - sn * y;
          A[k][q] = sn * x + c * y;
        }
        for (int k = 0; k < 3; ++k) {
          const double x = A[p][k], y = A[q][k];
          A[p][k] = c * x - sn * y;
          A[q][k] = sn * x + c * y;
        }
        for (int k = 0; k < 3; ++k) {
          const double x = V[k][p], y = V[k][q];
          V[k][p] = c * x - sn * y;
          V[k][q] = sn * x + c * y;
        }
      }
  }
  for (int i = 0; i < 3; ++i) d[i] = A[i][i];
}

// The eigenvalue of largest magnitude of a symmetric 3x3 matrix and its unit
// eigenvector in closed form: the eigenvalues by the trigonometric solution
// of the characteristic cubic (O. K. Smith, Commun. ACM 4 (1961) 168), the
// eigenvector as the longest cross product of two rows of A - lambda I.
// false when that eigenvalue is within 1e-6 of another (the eigenvector is
// then ill-determined in closed form; the Jacobi sweeps decide it).
bool sym3_dominant(const double (&A)[3][3], double& lam, double (&e)[3]) {
  const double p1 = A[0][1] * A[0][1] + A[0][2] * A[0][2] + A[1][2] * A[1][2];
  const double q = (A[0][0] + A[1][1] + A[2][2]) / 3.0;
  const double p2 = (A[0][0] - q) * (A[0][0] - q) + (A[1][1] - q) * (A[1][1] - q) +
                    (A[2][2] - q) * (A[2][2] - q) + 2.0 * p1;
  const double p = std::sqrt(p2 / 6.0);
  if (!(p > 0)) return false;
  double B[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) B[i][j] = (A[i][j] - (i == j ? q : 0.0)) / p;
  const double det = B[0][0] * (B[1][1] * B[2][2] - B[1][2] * B[2][1]) -
                     B[0][1] * (B[1][0] * B[2][2] - B[1][2] * B[2][0]) +
                     B[0][2] * (B[1][0] * B[2][1] - B[1][1] * B[2][0]);
  const double r = std::fmin(1.0, std::fmax(-1.0, det / 2.0));
  const double phi = std::acos(r) / 3.0;
  const double l1 = q + 2.0 * p * std::cos(phi), l3 = q + 2.0 * p * std::cos(phi + 2.0 * M_PI / 3.0);
  const double ls[3] = {l1, 3.0 * q - l1 - l3, l3};
  int c = 0;
  for (int k = 1; k < 3; ++k)
    if (std::fabs(ls[k]) > std::fabs(ls[c])) c = k;
  lam = ls[c];
  double gap = 1e300;
  for (int k = 0; k < 3; ++k)
    if (k != c) gap = std::fmin(gap, std::fabs(ls[k] - lam));
  if (gap < 1e-6 * (std::fabs(l1) + std::fabs(l3))) return false;
  double R[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) R[i][j] = A[i][j] - (i == j ? lam : 0.0);
  double best = -1.0, v[3] = {0.0, 0.0, 0.0};
  for (int a = 0; a < 2; ++a)
    for (int b2 = a + 1; b2 < 3; ++b2) {
      const double x[3] = {R[a][1] * R[b2][2] - R[a][2] * R[b2][1], R[a][2] * R[b2][0] - R[a][0] * R[b2][2],
                           R[a][0] * R[b2][1] - R[a][1] * R[b2][0]};
      const double n2 = x[0] * x[0] + x[1] * x[1] + x[2] * x[2];
      if (n2 > best) {
        best = n2;
        v[0] = x[0];
        v[1] = x[1];
        v[2] = x[2];
      }
    }
  const double nv = std::sqrt(best);
  if (!(nv > 0)) return false;
  for (int k = 0; k < 3; ++k) e[k] = v[k] / nv;
  return true;
}

// oo_params (v25/functions.cpp:2702-2760) from the sums v[12] over n
// particles: sum o (3), sum o o^T (xx xy xz yy yz zz), sum mu o_dipole (3).
// Q = sum (3 o o^T - 1) / (2 n) (Qmat_3d, :3426-3445); G2 is its eigenvalue
// of largest magnitude, chosen among equal magnitudes as the reference
// chooses (:2738-2748), and G1 = |e . sum o| / n along that eigenvector.
// Closed form when that eigenvalue is distinct (every step of every system
// converts these, so its cost shows), the Jacobi sweeps otherwise.
void order_params(const double* v, int n, double* G1, double* G2, double* M) {
  if (M)
    for (int a = 0; a < 3; ++a) M[a] = v[9 + a];
  if (n <= 0) {
    if (G1) *G1 = 0.0;
    if (G2) *G2 = 0.0;
    return;
  }
  const int ix[3][3] = {{3, 4, 5}, {4, 6, 7}, {5, 7, 8}};
  double Q[3][3], ev[3], V[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) Q[i][j] = (3.0 * v[ix[i][j]] - (i == j ? n : 0.0)) / (2.0 * n);
  double lam, e[3];
  if (sym3_dominant(Q, lam, e)) {  // the common case, in closed form
    if (G2) *G2 = std::fabs(lam);
    if (G1) *G1 = std::fabs(e[0] * v[0] + e[1] * v[1] + e[2] * v[2]) / n;
    return;
  }
  sym3_eigen(Q, ev, V);
  const double e1 = std::fabs(ev[0]), e2 = std::fabs(ev[1]), e3 = std::fabs(ev[2]);
  const int c = (e1 >= e2 && e1 >= e3) ? 0 : (e2 > e1 && e2 >= e3) ? 1 : 2;
  const double nv = std::sqrt(V[0][c] * V[0][c] + V[1][c] * V[1][c] + V[2][c] * V[2][c]);
  if (G2) *G2 = std::fabs(ev[c]);
  if (G1) *G1 = std::fabs((V[0][c] * v[0] + V[1][c] * v[1] + V[2][c] * v[2]) / nv) / n;
}

}  // namespace

// ======================================================================
// C ABI
// ======================================================================
extern "C" {

size_t mdsc_estimate_bytes(const mdsc_system_desc* descs, int nsys) {
  if (!descs || nsys <= 0) return 0;
  Layout lo;
  make_layout(descs, nsys, lo);
  Arena A;
  Batch b{};
  int4* kw;
  int2* ko;
  double* nz[2];
  int* sk;
  carve(A, lo, nsys, b, &kw, &ko, nz, &sk);
  return A.off;
}

mdsc_status mdsc_create(const mdsc_system_desc* descs, int nsys, int device, mdsc_batch** out) {
  if (!out || !descs || nsys <= 0) return MDSC_ERR_BAD_ARG;
  *out = nullptr;
  mdsc_batch* B = new mdsc_batch();
  for (int s = 0; s < nsys; ++s) {
    const std::string e = check_desc(descs[s], s);
    if (!e.empty()) {
      const bool table = e.find("table") != std::string::npos;
      delete B;
      fprintf(stderr, "mdsc_create: %s\n", e.c_str());
      return table ? MDSC_ERR_TABLE_RANGE : MDSC_ERR_BAD_ARG;
    }
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0 || device < 0 || device >= ndev) {
    delete B;
    return MDSC_ERR_NO_DEVICE;
  }
  B->device = device;
  B->nsys = nsys;
  B->desc.assign(descs, descs + nsys);
  cudaSetDevice(device);
  if (cudaDeviceGetAttribute(&B->num_sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
      B->num_sms <= 0 || prepare_real_pairs() != cudaSuccess) {
    delete B;
    return MDSC_ERR_NO_DEVICE;
  }
  make_layout(descs, nsys, B->lo);
  fill_tables(descs, B->lo);
  const Layout& lo = B->lo;
  Arena A;
  carve(A, lo, nsys, B->b, &B->kwork, &B->kowner, B->noise, &B->d_skip);
  B->arena_bytes = A.off;
  B->b.tune.wca_blocks = 8 * B->num_sms;
  cudaError_t e = cudaMalloc(&B->arena, B->arena_bytes);
  if (e != cudaSuccess) {
    delete B;
    return e == cudaErrorMemoryAllocation ? MDSC_ERR_OOM : MDSC_ERR_CUDA;
  }
  A.off = 0;
  A.base = B->arena;
  carve(A, lo, nsys, B->b, &B->kwork, &B->kowner, B->noise, &B->d_skip);
  Batch& b = B->b;
  b.nsys = nsys;
  b.ntot = lo.ntot;
  b.ndtot = lo.ndtot;
  b.nktot = lo.nktot;
  b.ntiles = (int)lo.tiles.size();
  b.nbstrips = (int)lo.bstrips.size();
  b.any_rc = lo.any_rc ? 1 : 0;
  b.nkgwork = (int)lo.kgwork.size();
  b.nblk = (int)lo.blk.size();
  b.ncellblk = (int)lo.cellblk.size();
  b.nrpwork = (int)lo.rpwork.size();
  b.ngtile = (int)lo.gtile.size();
  b.smem_tn = lo.smem_tn;
  b.rp_table = lo.rp_table ? 1 : 0;
  b.cells = 1;
  b.noise = B->noise[0];
  // The step graph forks the real-space tiles (stream s2) from the WCA and
  // k-space chains (st, s3).  The tiles keep the FP32 pipe busy while the
  // others wait on FP64, memory and special functions, so the others run at
  // the higher priority: their blocks are placed first and the tiles fill
  // the SMs around them.
  int prio_lo = 0, prio_hi = 0;
  cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
  if (cudaStreamCreateWithPriority(&B->st, cudaStreamNonBlocking, prio_hi) != cudaSuccess ||
      cudaStreamCreateWithPriority(&B->s2, cudaStreamNonBlocking, prio_lo) != cudaSuccess ||
      cudaStreamCreateWithPriority(&B->s3, cudaStreamNonBlocking, prio_hi) != cudaSuccess ||
      cudaEventCreateWithFlags(&B->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&B->ev_j2, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&B->ev_j3, cudaEventDisableTiming) != cudaSuccess ||
      cudaStreamCreateWithFlags(&B->sio, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&B->ev_x, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&B->ev_f, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreate(&B->t_beg) != cudaSuccess || cudaEventCreate(&B->t_end) != cudaSuccess ||
      cudaMallocHost(&B->h_noise, sizeof(double) * kNoiseChunk * nsys * 4) != cudaSuccess ||
      cudaMallocHost(&B->h_noise2, sizeof(double) * kNoiseChunk * nsys * 4) != cudaSuccess ||
      cudaEventCreateWithFlags(&B->ev_noise[0], cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&B->ev_noise[1], cudaEventDisableTiming) != cudaSuccess ||
      cudaMallocHost(&B->h_obs, sizeof(SysObs) * nsys) != cudaSuccess) {
    mdsc_destroy(B);
    return MDSC_ERR_CUDA;
  }
  // constant tables
  auto up = [&](void* dst, const void* src, size_t bytes) {
    if (bytes) cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, B->st);
  };
  up((void*)b.sys, lo.sys.data(), sizeof(SysDev) * nsys);
  up(b.tiles, lo.tiles.data(), sizeof(int4) * lo.tiles.size());
  if (!lo.rpwork.empty()) up(b.rpwork, lo.rpwork.data(), sizeof(int4) * lo.rpwork.size());
  if (!lo.gtile.empty()) up(b.gtile, lo.gtile.data(), sizeof(int) * lo.gtile.size());
  if (!lo.bstrips.empty()) up(b.bstrips, lo.bstrips.data(), sizeof(int2) * lo.bstrips.size());
  if (!lo.kgwork.empty()) up(b.kgwork, lo.kgwork.data(), sizeof(int2) * lo.kgwork.size());
  up(b.blk, lo.blk.data(), sizeof(int2) * lo.blk.size());
  if (!lo.cellblk.empty()) up(b.cellblk, lo.cellblk.data(), sizeof(int2) * lo.cellblk.size());
  up(b.kn, lo.kn.data(), sizeof(int4) * lo.kn.size());
  up(b.kv, lo.kv.data(), sizeof(float4) * lo.kv.size());
  up((void*)b.rtab, lo.rtab.data(), sizeof(float4) * lo.rtab.size());
  up(b.kval, lo.kval.data(), sizeof(double) * lo.kval.size());
  up(b.kvec, lo.kvec.data(), sizeof(double) * lo.kvec.size());
  up(b.kpre, lo.kpre.data(), sizeof(double) * lo.kpre.size());
  up(B->kwork, lo.kwork.data(), sizeof(int4) * lo.kwork.size());
  up(B->kowner, lo.kowner.data(), sizeof(int2) * lo.kowner.size());
  std::vector<int> psys(std::max(lo.ntot, 1));
  for (int s = 0; s < nsys; ++s)
    for (int i = 0; i < lo.sys[s].n; ++i) psys[lo.sys[s].part_off + i] = s;
  up(b.psys, psys.data(), sizeof(int) * lo.ntot);
  std::vector<SysState> st(nsys);
  memset(st.data(), 0, sizeof(SysState) * nsys);
  for (int s = 0; s < nsys; ++s) {
    st[s].xi[0] = st[s].xi[1] = descs[s].xi0;
    st[s].force_list = 1;
    st[s].stop = LLONG_MAX;
  }
  up(b.st, st.data(), sizeof(SysState) * nsys);
  cudaMemsetAsync(b.obs, 0, sizeof(SysObs) * nsys, B->st);
  cudaMemsetAsync(b.fsave, 0, sizeof(uint32_t) * 3 * std::max(lo.ntot, 1), B->st);
  cudaMemsetAsync(b.usave, 0, sizeof(float) * 3 * std::max(lo.ntot, 1), B->st);
  cudaMemsetAsync(b.nbc, 0, sizeof(int) * std::max(lo.ntot, 1), B->st);
  cudaMemsetAsync(b.wcnt, 0, sizeof(int) * std::max(lo.ntot, 1), B->st);
  cudaMemsetAsync(b.wincnt, 0, sizeof(int) * std::max(lo.ntot, 1), B->st);
  cudaMemsetAsync(b.stripE, 0, sizeof(double) * 10 * std::max(lo.nstrips, 1), B->st);
  cudaMemsetAsync(b.rnbc, 0, sizeof(int) * std::max(lo.ntot, 1), B->st);
  cudaMemsetAsync(b.ccnt, 0, sizeof(int) * std::max(lo.ncellcap, 1), B->st);
  cudaMemsetAsync(b.kgdone, 0, sizeof(int) * std::max<size_t>(lo.blk.size(), 1), B->st);
  cudaMemsetAsync(b.rlE, 0, sizeof(double) * 10 * std::max<size_t>(lo.blk.size(), 1), B->st);
  cudaMemsetAsync(b.kgcnt, 0, sizeof(int) * std::max(nsys, 1), B->st);
  cudaMemsetAsync(b.icnt, 0, sizeof(int) * std::max(nsys, 1), B->st);
  cudaMemsetAsync(b.F, 0, sizeof(double) * 3 * std::max(lo.ntot, 1), B->st);
  cudaMemsetAsync(b.T, 0, sizeof(double) * 3 * std::max(lo.ntot, 1), B->st);
  cudaMemsetAsync(B->noise[0], 0, sizeof(double) * kNoiseChunk * nsys * 4, B->st);
  cudaMemsetAsync(B->noise[1], 0, sizeof(double) * kNoiseChunk * nsys * 4, B->st);
  // rng streams
  for (int s = 0; s < nsys; ++s) {
    const unsigned long s0 = descs[s].thermo_seed[0] ? descs[s].thermo_seed[0] : 1;
    const unsigned long s1 = descs[s].thermo_seed[1] ? descs[s].thermo_seed[1] : 2;
    B->thermo_rng.emplace_back(s0);
    B->thermo_rng.emplace_back(s1);
    B->clus_rng.emplace_back(descs[s].cluster_seed ? descs[s].cluster_seed : 1);
    B->clus_rng.back().discard(descs[s].cluster_skip);
  }
  B->step_h.assign(nsys, 0);
  B->stop_h.assign(nsys, LLONG_MAX);
  B->labels.assign(nsys, std::vector<int>());
  for (int s = 0; s < nsys; ++s) B->labels[s].assign(descs[s].n, 0);
  B->n_clusters.assign(nsys, 0);
  B->uploaded.assign(nsys, 0);
  B->built.assign(nsys, 0);
  B->have_forces.assign(nsys, 0);
  B->species.resize(nsys);
  for (int s = 0; s < nsys; ++s) B->species[s].assign(1, descs[s].n);
  e = cudaStreamSynchronize(B->st);
  if (e != cudaSuccess) {
    mdsc_destroy(B);
    return MDSC_ERR_CUDA;
  }
  std::vector<float4>().swap(B->lo.rtab);  // on the device now; the host copy is not read again
  *out = B;
  return MDSC_OK;
}

mdsc_status mdsc_destroy(mdsc_batch* B) {
  if (!B) return MDSC_OK;
  cudaSetDevice(B->device);
  if (B->st) cudaStreamSynchronize(B->st);
  for (auto& g : B->graph)
    if (g) cudaGraphExecDestroy(g);
  for (auto& g : B->graph_io)
    if (g) cudaGraphExecDestroy(g);
  if (B->arena) cudaFree(B->arena);
  if (B->b.ecand) cudaFree(B->b.ecand);
  if (B->b.ecnt) cudaFree(B->b.ecnt);
  if (B->h_noise) cudaFreeHost(B->h_noise);
  if (B->h_noise2) cudaFreeHost(B->h_noise2);
  for (cudaEvent_t e : B->ev_noise)
    if (e) cudaEventDestroy(e);
  if (B->h_obs) cudaFreeHost(B->h_obs);
  if (B->h_trace) cudaFreeHost(B->h_trace);
  if (B->ev_fork) cudaEventDestroy(B->ev_fork);
  if (B->ev_j2) cudaEventDestroy(B->ev_j2);
  if (B->ev_j3) cudaEventDestroy(B->ev_j3);
  if (B->ev_x) cudaEventDestroy(B->ev_x);
  if (B->ev_f) cudaEventDestroy(B->ev_f);
  if (B->sio) cudaStreamDestroy(B->sio);
  if (B->t_beg) cudaEventDestroy(B->t_beg);
  if (B->t_end) cudaEventDestroy(B->t_end);
  if (B->st) cudaStreamDestroy(B->st);
  if (B->s2) cudaStreamDestroy(B->s2);
  if (B->s3) cudaStreamDestroy(B->s3);
  delete B;
  return MDSC_OK;
}

int mdsc_num_systems(const mdsc_batch* B) { return B ? B->nsys : 0; }
size_t mdsc_device_bytes(const mdsc_batch* B) {
  if (!B) return 0;
  // + the energy criterion's candidate lists, allocated on first use
  const size_t n = (size_t)std::max(B->lo.ntot, 1);
  return B->arena_bytes + (B->b.ecand ? sizeof(int) * n * (kMaxE + 1) : 0);
}
int mdsc_launches_per_step(const mdsc_batch* B) { return B ? B->launches : 0; }
void* mdsc_stream(const mdsc_batch* B) { return B ? (void*)B->st : nullptr; }

mdsc_status mdsc_last_error(const mdsc_batch* B, char* buf, size_t len) {
  if (!B || !buf || !len) return MDSC_ERR_BAD_ARG;
  snprintf(buf, len, "%s", B->err.c_str());
  return MDSC_OK;
}

// The list build's cell grid of a system: cells no smaller than the largest
// reach of a list entry -- the segment-distance radius plus both rods' half
// lengths (at most the longest rod), or the real-space neighbour radius --
// so that every partner of a rod lies in the 27 cells around its own.  At
// most cell_cap cells (dimensions shrunk, largest first); fewer than 3
// cells along an axis, or no capacity: ncell = 0, the all-pairs scan.
static void set_cell_grid(SysDev& P, const double* len) {
  P.ncell = P.cnx = P.cny = P.cnz = 0;
  if (P.cell_cap < 27) return;
  double lmax = 0.0;
  for (int i = 0; i < P.n; ++i) lmax = std::max(lmax, len[i]);
  double side = (P.r_list + lmax) * 1.0001 + 1e-4;
  if (P.rc_real > 0) side = std::max(side, std::sqrt((double)P.rl_r2) * 1.0001 + 1e-4);
  int c[3];
  for (int a = 0; a < 3; ++a) c[a] = (int)std::floor(P.L[a] / side);
  while ((long long)c[0] * c[1] * c[2] > P.cell_cap) {
    int a = 0;
    for (int k = 1; k < 3; ++k)
      if (c[k] > c[a]) a = k;
    --c[a];
  }
  if (c[0] < 3 || c[1] < 3 || c[2] < 3) return;
  P.cnx = c[0];
  P.cny = c[1];
  P.cnz = c[2];
  P.ncell = c[0] * c[1] * c[2];
}

static mdsc_status upload_one(mdsc_batch* B, int s, const mdsc_host_state* h, bool sync) {
  const SysDev& P = B->lo.sys[s];
  const int n = P.n;
  if (!h->r || !h->p || !h->O || !h->l) return fail(B, MDSC_ERR_BAD_ARG, "r, p, O, l are required");
  const bool shapes = h->len && h->dia && h->mass && (P.nd == 0 || h->dip);
  if (!shapes && !B->uploaded[s])
    return fail(B, MDSC_ERR_BAD_ARG, "the first upload of a system needs len, dia, mass and dip");
  Batch& b = B->b;
  const int i0 = P.part_off;
  // cluster labels as given (a restart's conf.dat): they stand until the
  // next clustering step replaces them
  if (h->clust) {
    B->labels[s].assign(h->clust, h->clust + n);
    int mx = -1;
    for (int i = 0; i < n; ++i) mx = std::max(mx, h->clust[i]);
    B->n_clusters[s] = mx + 1;
  }
  auto up = [&](void* dst, const void* src, size_t bytes) -> cudaError_t {
    return bytes ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, B->st) : cudaSuccess;
  };
  CU(up(b.r + 3 * i0, h->r, sizeof(double) * 3 * n));
  CU(up(b.p + 3 * i0, h->p, sizeof(double) * 3 * n));
  CU(up(b.O + 9 * i0, h->O, sizeof(double) * 9 * n));
  CU(up(b.l + 3 * i0, h->l, sizeof(double) * 3 * n));
  if (h->F && h->T) {
    CU(up(b.F + 3 * i0, h->F, sizeof(double) * 3 * n));
    CU(up(b.T + 3 * i0, h->T, sizeof(double) * 3 * n));
  }
  if (shapes) {
    std::vector<double> inert, invm, invI, dpc, dob, dmu;
    std::vector<int> downer;
    double Uself = 0;
    shapes_to_host(B, s, h, inert, invm, invI, dpc, dob, dmu, downer, Uself);
    CU(up(b.len + i0, h->len, sizeof(double) * n));
    CU(up(b.dia + i0, h->dia, sizeof(double) * n));
    CU(up(b.mass + i0, h->mass, sizeof(double) * n));
    CU(up(b.inert + 3 * i0, inert.data(), sizeof(double) * 3 * n));
    CU(up(b.invm + i0, invm.data(), sizeof(double) * n));
    CU(up(b.invI + 3 * i0, invI.data(), sizeof(double) * 3 * n));
    const int g0 = P.dip_off, nd = P.ndip;
    CU(up(b.dpc + g0, dpc.data(), sizeof(double) * nd));
    CU(up(b.dob + 3 * g0, dob.data(), sizeof(double) * 3 * nd));
    CU(up(b.dmu + g0, dmu.data(), sizeof(double) * nd));
    CU(up(b.downer + g0, downer.data(), sizeof(int) * nd));
    // list radius: max(2^(1/6) sigma, sigma + min_s) + skin, skin = 0.9 d_min
    // (the reference's r_list_max - r_list_min, v25/main.cpp:460-463)
    double dmax = 0, dmin = 1e300;
    for (int i = 0; i < n; ++i) {
      dmax = std::max(dmax, h->dia[i]);
      dmin = std::min(dmin, h->dia[i]);
    }
    if (n == 0) dmin = dmax = 1.0;
    SysDev& Pm = B->lo.sys[s];
    Pm.sig_max = dmax;
    Pm.skin = 0.9 * dmin;
    Pm.r_list = std::max(1.122462048309373 * dmax, dmax + B->desc[s].min_s) + Pm.skin;
    if (Pm.rc_real > 0) {
      // real-space neighbours: rods whose centres are within rc + Lh (the
      // last table interval) + the dipoles' offsets + the skin, with room
      // for the FP32 centre distance
      double e = 0;
      for (int g = 0; g < nd; ++g) e = std::max(e, std::fabs(dpc[g]));
      const double rr = (Pm.rc_real + kLh + 2 * e + Pm.skin) * 1.0001 + 1e-4;
      Pm.rl_r2 = (float)(rr * rr);
    }
    set_cell_grid(Pm, h->len);
    Pm.Uself = Uself;
    CU(up((void*)(b.sys + s), &Pm, sizeof(SysDev)));
    if (B->uploaded[s]) {
      // new shapes: the list must be rebuilt
      const int one = 1;
      CU(up((char*)(b.st + s) + offsetof(SysState, force_list), &one, sizeof(int)));
    }
  }
  B->uploaded[s] = 1;
  B->have_forces[s] = (h->F && h->T) ? 1 : 0;
  if (sync) CU(cudaStreamSynchronize(B->st));
  return MDSC_OK;
}

mdsc_status mdsc_upload(mdsc_batch* B, int sys, const mdsc_host_state* h) {
  if (!B || !h || sys < 0 || sys >= B->nsys) return MDSC_ERR_BAD_ARG;
  cudaSetDevice(B->device);
  return upload_one(B, sys, h, true);
}

mdsc_status mdsc_upload_all(mdsc_batch* B, const mdsc_host_state* h) {
  if (!B || !h) return MDSC_ERR_BAD_ARG;
  cudaSetDevice(B->device);
  bool first = false;
  for (int s = 0; s < B->nsys; ++s) first |= !B->uploaded[s];
  const bool shapes = h->len && h->dia && h->mass;
  if (first || shapes) {
    // per system (computes the host-side shape data)
    for (int s = 0; s < B->nsys; ++s) {
      const SysDev& P = B->lo.sys[s];
      mdsc_host_state v = *h;
      v.r = h->r + 3 * (size_t)P.part_off;
      v.p = h->p + 3 * (size_t)P.part_off;
      v.O = h->O + 9 * (size_t)P.part_off;
      v.l = h->l + 3 * (size_t)P.part_off;
      v.F = h->F ? h->F + 3 * (size_t)P.part_off : nullptr;
      v.T = h->T ? h->T + 3 * (size_t)P.part_off : nullptr;
      v.len = h->len ? h->len + P.part_off : nullptr;
      v.dia = h->dia ? h->dia + P.part_off : nullptr;
      v.mass = h->mass ? h->mass + P.part_off : nullptr;
      v.dip = h->dip ? h->dip + 5 * (size_t)P.dip_off : nullptr;
      mdsc_status st = upload_one(B, s, &v, false);
      if (st != MDSC_OK) return st;
    }
    CU(cudaStreamSynchronize(B->st));
    return MDSC_OK;
  }
  // state only: one copy per array for the whole batch, one after another on
  // the main stream.  Each copy runs at the host link's rate (~205 GB/s to
  // the device on this GB300); spreading the arrays over several streams
  // made the copies share the link and the whole no faster (the same e2e
  // within 1%, 175 GB/s for 4 concurrent copies against 207 for one)
  const size_t n = B->lo.ntot;
  Batch& b = B->b;
  const bool forces = h->F && h->T;
  CU(cudaMemcpyAsync(b.O, h->O, sizeof(double) * 9 * n, cudaMemcpyHostToDevice, B->st));
  CU(cudaMemcpyAsync(b.r, h->r, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, B->st));
  CU(cudaMemcpyAsync(b.p, h->p, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, B->st));
  CU(cudaMemcpyAsync(b.l, h->l, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, B->st));
  if (forces) {
    CU(cudaMemcpyAsync(b.F, h->F, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, B->st));
    CU(cudaMemcpyAsync(b.T, h->T, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, B->st));
  }
  for (int s = 0; s < B->nsys; ++s) B->have_forces[s] = forces ? 1 : 0;
  return MDSC_OK;
}

static mdsc_status download_range(mdsc_batch* B, int i0, int n, int s_first, int s_last,
                                  mdsc_host_state* h) {
  Batch& b = B->b;
  // after the main stream's work, one copy per array on that stream (as
  // the uploads: concurrent copies share the host link)
  auto dn = [&](void* dst, const void* src, size_t bytes) -> cudaError_t {
    return (dst && bytes) ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, B->st) : cudaSuccess;
  };
  CU(dn(h->O, b.O + 9 * i0, sizeof(double) * 9 * n));
  CU(dn(h->r, b.r + 3 * i0, sizeof(double) * 3 * n));
  CU(dn(h->p, b.p + 3 * i0, sizeof(double) * 3 * n));
  CU(dn(h->F, b.F + 3 * i0, sizeof(double) * 3 * n));
  CU(dn(h->l, b.l + 3 * i0, sizeof(double) * 3 * n));
  CU(dn(h->T, b.T + 3 * i0, sizeof(double) * 3 * n));
  CU(cudaStreamSynchronize(B->st));
  if (h->clust) {
    int off = 0;
    for (int s = s_first; s <= s_last; ++s) {
      const std::vector<int>& lab = B->labels[s];
      std::copy(lab.begin(), lab.end(), h->clust + off);
      off += (int)lab.size();
    }
  }
  return MDSC_OK;
}

mdsc_status mdsc_download(mdsc_batch* B, int sys, mdsc_host_state* h) {
  if (!B || !h || sys < 0 || sys >= B->nsys) return MDSC_ERR_BAD_ARG;
  cudaSetDevice(B->device);
  const SysDev& P = B->lo.sys[sys];
  return download_range(B, P.part_off, P.n, sys, sys, h);
}

mdsc_status mdsc_download_all(mdsc_batch* B, mdsc_host_state* h) {
  if (!B || !h) return MDSC_ERR_BAD_ARG;
  cudaSetDevice(B->device);
  return download_range(B, 0, B->lo.ntot, 0, B->nsys - 1, h);
}

mdsc_status mdsc_set_thermostat(mdsc_batch* B, int sys, const double xi[2], const double strn[2]) {
  if (!B || sys < 0 || sys >= B->nsys || !xi) return MDSC_ERR_BAD_ARG;
  cudaSetDevice(B->device);
  SysState st;
  CU(cudaMemcpy(&st, B->b.st + sys, sizeof st, cudaMemcpyDeviceToHost));
  st.xi[0] = xi[0];
  st.xi[1] = xi[1];
  if (strn) {
    st.strn[0] = strn[0];
    st.strn[1] = strn[1];
  }
  CU(cudaMemcpy(B->b.st + sys, &st, sizeof st, cudaMemcpyHostToDevice));
  return MDSC_OK;
}

mdsc_status mdsc_get_thermostat(mdsc_batch* B, int sys, double xi[2], double strn[2]) {
  if (!B || sys < 0 || sys >= B->nsys) return MDSC_ERR_BAD_ARG;
  cudaSetDevice(B->device);
  SysState st;
  CU(cudaMemcpy(&st, B->b.st + sys, sizeof st, cudaMemcpyDeviceToHost));
  for (int k = 0; k < 2; ++k) {
    if (xi) xi[k] = st.xi[k];
    if (strn) strn[k] = st.strn[k];
  }
  return MDSC_OK;
}

// ---- function-level entry points --------------------------------------
static mdsc_status need_state(mdsc_batch* B) {
  if (!B) return MDSC_ERR_BAD_ARG;
  cudaSetDevice(B->device);
  for (int s = 0; s < B->nsys; ++s)
    if (!B->uploaded[s]) return fail(B, MDSC_ERR_STATE, "system " + std::to_string(s) + " has no state yet");
  return MDSC_OK;
}

mdsc_status mdsc_zero_forces(mdsc_batch* B) {
  mdsc_status st = need_state(B);
  if (st) return st;
  CU(cudaMemsetAsync(B->b.F, 0, sizeof(double) * 3 * B->lo.ntot, B->st));
  CU(cudaMemsetAsync(B->b.T, 0, sizeof(double) * 3 * B->lo.ntot, B->st));
  CU(cudaStreamSynchronize(B->st));
  return MDSC_OK;
}

mdsc_status mdsc_force_sc(mdsc_batch* B, double* U, double* W, double* PT) {
  mdsc_status st = need_state(B);
  if (st) return st;
  launch_derive(B->b, B->st);
  launch_list_build(B->b, 0, B->st);
  launch_wca(B->b, 0, B->st);
  launch_finalize(B->b, kMaskWca | kFlagAccum, B->st);
  launch_order_terms(B->b, B->st);
  launch_reduce_obs(B->b, kRedEnergies, B->st);
  st = read_obs(B, nullptr);
  for (int s = 0; s < B->nsys; ++s) {
    const SysObs& o = B->h_obs[s];
    if (U) U[s] = o.U_ss;
    if (W) W[s] = o.W_ss;
    if (PT) memcpy(PT + 9 * s, o.PT_ss, sizeof(double) * 9);
  }
  return st;
}

mdsc_status mdsc_force_dipR(mdsc_batch* B, double* U, double* PT) {
  mdsc_status st = need_state(B);
  if (st) return st;
  launch_derive(B->b, B->st);
  if (B->b.any_rc) launch_list_build(B->b, 0, B->st);
  launch_near_pass(B->b, 1, B->st);
  launch_real_pairs(B->b, B->lo.multi, B->st);
  launch_real_sum(B->b, B->st);
  launch_finalize(B->b, kMaskReal | kFlagAccum, B->st);
  launch_order_terms(B->b, B->st);
  launch_reduce_obs(B->b, kRedEnergies, B->st);
  st = read_obs(B, nullptr);
  for (int s = 0; s < B->nsys; ++s) {
    const SysObs& o = B->h_obs[s];
    if (U) U[s] = o.U_dipR;
    if (PT) memcpy(PT + 9 * s, o.PT_dipR, sizeof(double) * 9);
  }
  return st;
}

mdsc_status mdsc_force_dipK(mdsc_batch* B, double* U, double* PT) {
  mdsc_status st = need_state(B);
  if (st) return st;
  launch_derive(B->b, B->st);
  launch_kspace(B->b, B->lo.maxnd, B->kwork, (int)B->lo.kwork.size(), B->kowner, B->b.kE, B->st);
  launch_finalize(B->b, kMaskK | kFlagAccum, B->st);
  launch_order_terms(B->b, B->st);
  launch_reduce_obs(B->b, kRedEnergies, B->st);
  st = read_obs(B, nullptr);
  for (int s = 0; s < B->nsys; ++s) {
    const SysObs& o = B->h_obs[s];
    if (U) U[s] = o.U_dipK;
    if (PT) memcpy(PT + 9 * s, o.PT_dipK, sizeof(double) * 9);
  }
  return st;
}

mdsc_status mdsc_ext_field(mdsc_batch* B, double* U) {
  mdsc_status st = need_state(B);
  if (st) return st;
  launch_derive(B->b, B->st);
  launch_finalize(B->b, kMaskExt | kFlagAccum, B->st);
  launch_order_terms(B->b, B->st);
  launch_reduce_obs(B->b, kRedEnergies, B->st);
  st = read_obs(B, nullptr);
  for (int s = 0; s < B->nsys; ++s)
    if (U) U[s] = B->h_obs[s].U_ext;
  return st;
}

mdsc_status mdsc_self_ener(mdsc_batch* B, double* U) {
  mdsc_status st = need_state(B);
  if (st) return st;
  for (int s = 0; s < B->nsys; ++s)
    if (U) U[s] = B->lo.sys[s].Uself;
  return MDSC_OK;
}

mdsc_status mdsc_moveX(mdsc_batch* B) {
  mdsc_status st = need_state(B);
  if (st) return st;
  launch_movex(B->b, B->st);
  CU(cudaGetLastError());
  CU(cudaStreamSynchronize(B->st));
  return MDSC_OK;
}

mdsc_status mdsc_renorm(mdsc_batch* B) {
  mdsc_status st = need_state(B);
  if (st) return st;
  launch_renorm(B->b, B->st);
  launch_derive(B->b, B->st);
  CU(cudaGetLastError());
  CU(cudaStreamSynchronize(B->st));
  return MDSC_OK;
}

mdsc_status mdsc_moveP(mdsc_batch* B, const double* xi, int last, double* K, double* PT) {
  mdsc_status st = need_state(B);
  if (st) return st;
  if (!xi) return fail(B, MDSC_ERR_BAD_ARG, "xi is required");
  // the noise buffer is free outside mdsc_step: stage xi there
  CU(cudaMemcpyAsync(B->noise[1], xi, sizeof(double) * 2 * B->nsys, cudaMemcpyHostToDevice, B->st));
  launch_movep(B->b, B->noise[1], last, B->st);
  std::vector<double> part(9 * B->b.nblk);
  CU(cudaMemcpyAsync(part.data(), B->b.kin2, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, B->st));
  CU(cudaStreamSynchronize(B->st));
  for (int s = 0; s < B->nsys; ++s) {
    const SysDev& P = B->lo.sys[s];
    double v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int k = 0; k < P.nblk; ++k)
      for (int c = 0; c < 9; ++c) v[c] += part[9 * (P.blk_off + k) + c];
    if (K) {
      K[2 * s] = 0.5 * v[0];
      K[2 * s + 1] = 0.5 * v[1];
    }
    if (PT) {
      const int map[9] = {2, 3, 4, 3, 5, 6, 4, 6, 7};
      for (int c = 0; c < 9; ++c) PT[9 * s + c] = last ? v[map[c]] : 0.0;
    }
  }
  return MDSC_OK;
}

mdsc_status mdsc_neigh_list(mdsc_batch* B) {
  mdsc_status st = need_state(B);
  if (st) return st;
  launch_derive(B->b, B->st);
  launch_list_build(B->b, 1, B->st);
  CU(cudaGetLastError());
  CU(cudaStreamSynchronize(B->st));
  for (int s = 0; s < B->nsys; ++s) B->built[s] = 1;
  return MDSC_OK;
}

mdsc_status mdsc_check_list(mdsc_batch* B, int* rebuild) {
  mdsc_status st = need_state(B);
  if (st) return st;
  launch_derive(B->b, B->st);
  std::vector<double> dm(B->b.nblk);
  CU(cudaMemcpyAsync(dm.data(), B->b.dmax, sizeof(double) * dm.size(), cudaMemcpyDeviceToHost, B->st));
  CU(cudaStreamSynchronize(B->st));
  for (int s = 0; s < B->nsys; ++s) {
    const SysDev& P = B->lo.sys[s];
    double m = 0;
    for (int k = 0; k < P.nblk; ++k) m = std::max(m, dm[P.blk_off + k]);
    if (rebuild) rebuild[s] = (!B->built[s] || 2.0 * m > P.skin) ? 1 : 0;
  }
  return MDSC_OK;
}

mdsc_status mdsc_clust_conf(mdsc_batch* B, int sys, int* labels, int* n_clusters) {
  mdsc_status st = need_state(B);
  if (st) return st;
  if (sys < 0 || sys >= B->nsys) return MDSC_ERR_BAD_ARG;
  launch_derive(B->b, B->st);
  launch_list_build(B->b, 0, B->st);
  st = run_clusters(B, std::vector<int>{sys});
  if (st) return st;
  if (labels) std::copy(B->labels[sys].begin(), B->labels[sys].end(), labels);
  if (n_clusters) *n_clusters = B->n_clusters[sys];
  return MDSC_OK;
}

// the candidate lists of the energy screen, for every particle of the batch,
// allocated when a system of it first takes the energy criterion
static mdsc_status ensure_energy_lists(mdsc_batch* B) {
  if (B->b.ecand && B->b.ecnt) return MDSC_OK;
  const size_t n = (size_t)std::max(B->lo.ntot, 1);
  // both lists or neither: the batch keeps them only once both exist
  int* cand = nullptr;
  int* cnt = nullptr;
  CU(cudaMalloc(&cand, sizeof(int) * n * kMaxE));
  const cudaError_t e = cudaMalloc(&cnt, sizeof(int) * n);
  if (e != cudaSuccess) {
    cudaFree(cand);
    return fail(B, e == cudaErrorMemoryAllocation ? MDSC_ERR_OOM : MDSC_ERR_CUDA,
                std::string("energy candidate counts: ") + cudaGetErrorString(e));
  }
  B->b.ecand = cand;
  B->b.ecnt = cnt;
  CU(cudaMemsetAsync(cnt, 0, sizeof(int) * n, B->st));
  return MDSC_OK;
}

mdsc_status mdsc_set_cluster_energy(mdsc_batch* B, int sys, double u_bond_kT) {
  if (!B || sys < 0 || sys >= B->nsys || !(u_bond_kT >= 0.0)) return MDSC_ERR_BAD_ARG;
  cudaSetDevice(B->device);
  if (u_bond_kT > 0.0) {
    const mdsc_status st = ensure_energy_lists(B);
    if (st) return st;
  }
  SysDev& P = B->lo.sys[sys];
  P.cl_mode = u_bond_kT > 0.0 ? 1 : 0;
  P.cl_ubond = u_bond_kT * B->desc[sys].temp;
  CU(cudaMemcpyAsync((void*)(B->b.sys + sys), &P, sizeof(SysDev), cudaMemcpyHostToDevice, B->st));
  CU(cudaStreamSynchronize(B->st));
  return MDSC_OK;
}

void mdsc_abi_sizes(size_t* desc, size_t* host_state, size_t* observables, size_t* view) {
  if (desc) *desc = sizeof(mdsc_system_desc);
  if (host_state) *host_state = sizeof(mdsc_host_state);
  if (observables) *observables = sizeof(mdsc_observables);
  if (view) *view = sizeof(mdsc_view);
}

// ---- observables outside the step ---------------------------------------
int mdsc_correlation_bins(const mdsc_batch* B, int sys, double bar_w) {
  if (!B || sys < 0 || sys >= B->nsys || !(bar_w > 0.0)) return 0;
  return std::max(0, corr_bins(B->lo.sys[sys], bar_w));
}

mdsc_status mdsc_set_species(mdsc_batch* B, int sys, int nspecies, const int* counts) {
  if (!B || sys < 0 || sys >= B->nsys || nspecies < 1 || nspecies > 255 || !counts) return MDSC_ERR_BAD_ARG;
  long long tot = 0;
  for (int k = 0; k < nspecies; ++k) {
    if (counts[k] < 1) return fail(B, MDSC_ERR_BAD_ARG, "mdsc_set_species: every species needs a particle");
    tot += counts[k];
  }
  if (tot != B->lo.sys[sys].n) return fail(B, MDSC_ERR_BAD_ARG, "mdsc_set_species: counts do not add up to n");
  B->species[sys].assign(counts, counts + nspecies);
  return MDSC_OK;
}

int mdsc_correlation_size(const mdsc_batch* B, int sys, double bar_w) {
  if (!B || sys < 0 || sys >= B->nsys || !(bar_w > 0.0)) return 0;
  const int nc = (int)B->species[sys].size();
  return (nc + nc * (nc - 1) / 2) * 4 * std::max(0, corr_bins(B->lo.sys[sys], bar_w));
}

mdsc_status mdsc_correlations(mdsc_batch* B, double bar_w, double* hist) {
  mdsc_status st = need_state(B);
  if (st) return st;
  if (!(bar_w > 0.0) || !hist) return fail(B, MDSC_ERR_BAD_ARG, "mdsc_correlations: bar_w > 0 and hist required");
  std::vector<CorrSys> cs(B->nsys);
  std::vector<unsigned char> sp(std::max(B->lo.ntot, 1), 0);
  int tot = 0, max_bins = 0;
  for (int s = 0; s < B->nsys; ++s) {
    const int nb = std::max(0, corr_bins(B->lo.sys[s], bar_w));
    const int nc = (int)B->species[s].size();
    const int nblocks = nc + nc * (nc - 1) / 2;
    cs[s] = CorrSys{nb, tot, nc, 0};
    tot += nblocks * 4 * nb;
    max_bins = std::max(max_bins, nblocks * nb);
    int i = B->lo.sys[s].part_off;
    for (int k = 0; k < nc; ++k)
      for (int q = 0; q < B->species[s][k]; ++q) sp[i++] = (unsigned char)k;
  }
  if (tot == 0) return MDSC_OK;
  char* d = nullptr;
  const size_t hbytes = sizeof(unsigned long long) * tot, cbytes = sizeof(CorrSys) * B->nsys;
  CU(cudaMallocAsync((void**)&d, hbytes + cbytes + sp.size(), B->st));
  unsigned long long* dh = reinterpret_cast<unsigned long long*>(d);
  CorrSys* dcs = reinterpret_cast<CorrSys*>(d + hbytes);
  unsigned char* dsp = reinterpret_cast<unsigned char*>(d + hbytes + cbytes);
  std::vector<unsigned long long> h(tot);
  CU(cudaMemcpyAsync(dcs, cs.data(), cbytes, cudaMemcpyHostToDevice, B->st));
  CU(cudaMemcpyAsync(dsp, sp.data(), sp.size(), cudaMemcpyHostToDevice, B->st));
  CU(cudaMemsetAsync(dh, 0, hbytes, B->st));
  launch_derive(B->b, B->st);
  launch_correlations(B->b, dcs, dsp, bar_w, max_bins, dh, B->st);
  CU(cudaGetLastError());
  CU(cudaMemcpyAsync(h.data(), dh, hbytes, cudaMemcpyDeviceToHost, B->st));
  CU(cudaFreeAsync(d, B->st));
  CU(cudaStreamSynchronize(B->st));
  // counts are exact integers; the other three are fixed point in 2^-24 units
  for (int s = 0; s < B->nsys; ++s) {
    const int nb = cs[s].nbins, nc = cs[s].nsp, nblocks = nc + nc * (nc - 1) / 2;
    for (int q = 0; q < nblocks; ++q) {
      const int o = cs[s].off + q * 4 * nb;
      for (int k = 0; k < nb; ++k) hist[o + k] += (double)h[o + k];
      for (int k = nb; k < 4 * nb; ++k) hist[o + k] += std::ldexp((double)(long long)h[o + k], -24);
    }
  }
  return MDSC_OK;
}

mdsc_status mdsc_order_params(mdsc_batch* B, double* G1, double* G2, double* M) {
  mdsc_status st = need_state(B);
  if (st) return st;
  const int nblk = B->b.nblk;
  std::vector<double> part(12 * (size_t)nblk);
  double* d = nullptr;
  CU(cudaMallocAsync((void**)&d, sizeof(double) * part.size(), B->st));
  launch_derive(B->b, B->st);
  launch_order_sums(B->b, d, B->st);
  CU(cudaGetLastError());
  CU(cudaMemcpyAsync(part.data(), d, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, B->st));
  CU(cudaFreeAsync(d, B->st));
  CU(cudaStreamSynchronize(B->st));
  for (int s = 0; s < B->nsys; ++s) {
    const SysDev& P = B->lo.sys[s];
    double v[12] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int k = 0; k < P.nblk; ++k)
      for (int c = 0; c < 12; ++c) v[c] += part[12 * (size_t)(P.blk_off + k) + c];
    order_params(v, P.n, G1 ? &G1[s] : nullptr, G2 ? &G2[s] : nullptr, M ? &M[3 * s] : nullptr);
  }
  return MDSC_OK;
}

// ---- a new configuration ----------------------------------------------------
mdsc_status mdsc_lattice(mdsc_batch* B, int sys, int nspecies, const int* counts, int* n_overlaps) {
  mdsc_status st = need_state(B);
  if (st) return st;
  if (sys < 0 || sys >= B->nsys || nspecies < 1 || !counts) return MDSC_ERR_BAD_ARG;
  const SysDev& P = B->lo.sys[sys];
  long long tot = 0;
  for (int k = 0; k < nspecies; ++k) {
    if (counts[k] < 1) return fail(B, MDSC_ERR_BAD_ARG, "mdsc_lattice: every species needs a particle");
    tot += counts[k];
  }
  if (tot != P.n) return fail(B, MDSC_ERR_BAD_ARG, "mdsc_lattice: counts do not add up to n");
  Batch& b = B->b;
  std::vector<double> len(P.n), dia(P.n);
  CU(cudaMemcpyAsync(len.data(), b.len + P.part_off, sizeof(double) * P.n, cudaMemcpyDeviceToHost, B->st));
  CU(cudaMemcpyAsync(dia.data(), b.dia + P.part_off, sizeof(double) * P.n, cudaMemcpyDeviceToHost, B->st));
  CU(cudaStreamSynchronize(B->st));
  const double sq = std::sqrt(3.) / 2., sqtt = std::sqrt(6.) / 3;
  int first = 0;
  for (int k = 0; k < nspecies; ++k) {
    const double L0 = len[first], D0 = dia[first];
    // sites per row, rows per layer, layers (v25/functions.cpp:507-509)
    const int num1 = (int)std::max(std::floor(P.L[0] / D0), 1.);
    const int num2 = (int)std::max(std::floor(P.L[1] / (D0 * sq)), 1.);
    const int num3 = (int)std::max(std::floor(P.L[2] / (D0 * sqtt + L0)), 1.);
    const long long ns = (long long)num1 * num2 * num3;
    if (ns > (1 << 28)) return fail(B, MDSC_ERR_TOO_LARGE, "mdsc_lattice: too many lattice sites");
    double* d_r = nullptr;
    int* d_ok = nullptr;
    CU(cudaMallocAsync((void**)&d_r, sizeof(double) * 3 * ns, B->st));
    CU(cudaMallocAsync((void**)&d_ok, sizeof(int) * ns, B->st));
    launch_lattice_sites(b, sys, L0, D0, num1, num2, (int)ns, P.part_off, first, d_r, d_ok, B->st);
    CU(cudaGetLastError());
    std::vector<double> hr(3 * ns);
    std::vector<int> ok(ns);
    CU(cudaMemcpyAsync(hr.data(), d_r, sizeof(double) * 3 * ns, cudaMemcpyDeviceToHost, B->st));
    CU(cudaMemcpyAsync(ok.data(), d_ok, sizeof(int) * ns, cudaMemcpyDeviceToHost, B->st));
    CU(cudaFreeAsync(d_r, B->st));
    CU(cudaFreeAsync(d_ok, B->st));
    CU(cudaStreamSynchronize(B->st));
    std::vector<long long> acc;
    for (long long q = 0; q < ns; ++q)
      if (ok[q]) acc.push_back(q);
    if (acc.empty()) return fail(B, MDSC_ERR_OVERLAP, "mdsc_lattice: no free lattice site for a species");
    // the accepted sites in order, from the first again when they run out
    std::vector<double> r(3 * counts[k]), O(9 * counts[k], 0.0);
    for (int q = 0; q < counts[k]; ++q) {
      const long long site = acc[q % acc.size()];
      for (int a = 0; a < 3; ++a) r[3 * q + a] = hr[3 * site + a];
      O[9 * q + 0] = O[9 * q + 4] = O[9 * q + 8] = 1.0;
    }
    CU(cudaMemcpyAsync(b.r + 3 * (P.part_off + first), r.data(), sizeof(double) * r.size(), cudaMemcpyHostToDevice,
                       B->st));
    CU(cudaMemcpyAsync(b.O + 9 * (P.part_off + first), O.data(), sizeof(double) * O.size(), cudaMemcpyHostToDevice,
                       B->st));
    first += counts[k];
  }
  int* d_cnt = nullptr;
  int cnt = 0;
  CU(cudaMallocAsync((void**)&d_cnt, sizeof(int), B->st));
  CU(cudaMemsetAsync(d_cnt, 0, sizeof(int), B->st));
  launch_overlap_count(b, sys, P.n, d_cnt, B->st);
  CU(cudaMemcpyAsync(&cnt, d_cnt, sizeof(int), cudaMemcpyDeviceToHost, B->st));
  CU(cudaFreeAsync(d_cnt, B->st));
  const int one = 1;
  CU(cudaMemcpyAsync((char*)(b.st + sys) + offsetof(SysState, force_list), &one, sizeof(int), cudaMemcpyHostToDevice,
                     B->st));
  CU(cudaStreamSynchronize(B->st));
  B->have_forces[sys] = 0;
  if (n_overlaps) *n_overlaps = cnt;
  return MDSC_OK;
}

mdsc_status mdsc_thermalize(mdsc_batch* B, int sys, double temp, unsigned long long seed) {
  mdsc_status st = need_state(B);
  if (st) return st;
  if (sys < 0 || sys >= B->nsys || !(temp >= 0.0)) return MDSC_ERR_BAD_ARG;
  launch_thermalize(B->b, sys, B->lo.sys[sys].n, temp, seed, B->st);
  CU(cudaGetLastError());
  CU(cudaStreamSynchronize(B->st));
  return MDSC_OK;
}

// ---- picture ---------------------------------------------------------------
mdsc_status mdsc_render(mdsc_batch* B, int sys, const mdsc_view* v, unsigned char* rgb) {
  mdsc_status st = need_state(B);
  if (st) return st;
  if (sys < 0 || sys >= B->nsys || !v || !rgb || v->width <= 0 || v->height <= 0 || v->width > 16384 ||
      v->height > 16384)
    return fail(B, MDSC_ERR_BAD_ARG, "mdsc_render: bad system, view or buffer");
  const SysDev& P = B->lo.sys[sys];
  // the viewer's camera (v25/graphic.cpp:680-692,405-415): gluLookAt from usr
  // to ref, then the scene pushed back |usr| along the view
  const double usr[3] = {v->dist * std::sin(v->theta) * std::cos(v->phi),
                         v->dist * std::sin(v->theta) * std::sin(v->phi), v->dist * std::cos(v->theta)};
  double ref[3], view[3];
  for (int a = 0; a < 3; ++a) ref[a] = v->ref[a];
  for (int a = 0; a < 3; ++a) view[a] = usr[a] - ref[a];
  const double vn = std::sqrt(view[0] * view[0] + view[1] * view[1] + view[2] * view[2]);
  const double un = std::sqrt(usr[0] * usr[0] + usr[1] * usr[1] + usr[2] * usr[2]);
  if (!(vn > 0.0)) return fail(B, MDSC_ERR_BAD_ARG, "mdsc_render: the camera sits on the point it looks at");
  double eye[3], fwd[3], right[3], up[3];
  for (int a = 0; a < 3; ++a) {
    eye[a] = usr[a] + un * view[a] / vn - v->shift[a];  // shifting the scene = shifting the camera back
    fwd[a] = -view[a] / vn;
  }
  const double zup[3] = {0.0, 0.0, 1.0}, yup[3] = {0.0, 1.0, 0.0};
  const double* wu = std::fabs(fwd[2]) > 0.999999 ? yup : zup;
  right[0] = fwd[1] * wu[2] - fwd[2] * wu[1];
  right[1] = fwd[2] * wu[0] - fwd[0] * wu[2];
  right[2] = fwd[0] * wu[1] - fwd[1] * wu[0];
  const double rn = std::sqrt(right[0] * right[0] + right[1] * right[1] + right[2] * right[2]);
  for (int a = 0; a < 3; ++a) right[a] /= rn;
  up[0] = right[1] * fwd[2] - right[2] * fwd[1];
  up[1] = right[2] * fwd[0] - right[0] * fwd[2];
  up[2] = right[0] * fwd[1] - right[1] * fwd[0];
  const double tan_half = std::tan(M_PI / 6.0);
  // a pixel at the distance looked at: the viewer's 2-pixel dipole lines and 1-pixel box edges
  const double pix = 2.0 * (vn + un) * tan_half / v->height;
  float e[3], f[3], r[3], u[3], l[3];
  for (int a = 0; a < 3; ++a) {
    e[a] = (float)eye[a];
    f[a] = (float)fwd[a];
    r[a] = (float)right[a];
    u[a] = (float)up[a];
    l[a] = un > 0.0 ? (float)(usr[a] / un) : (a == 2 ? 1.f : 0.f);
  }
  // species and the cluster filter, per particle
  std::vector<unsigned char> sp(std::max(P.n, 1), 0);
  {
    int i = 0;
    for (size_t k = 0; k < B->species[sys].size(); ++k)
      for (int q = 0; q < B->species[sys][k]; ++q) sp[i++] = (unsigned char)k;
  }
  std::vector<int> keep;
  if (v->cluster >= 0) {
    keep.assign(std::max(P.n, 1), 0);
    for (int i = 0; i < P.n; ++i) keep[i] = B->labels[sys][i] == v->cluster ? 1 : 0;
  }
  const size_t img = (size_t)v->width * v->height * 3;
  const size_t scratch = render_scratch_bytes(P.n, P.nd, v->images);
  char* d = nullptr;
  const size_t spb = (sp.size() + 255) / 256 * 256, kb = (keep.size() * sizeof(int) + 255) / 256 * 256;
  CU(cudaMallocAsync((void**)&d, scratch + spb + kb + img, B->st));
  unsigned char* dsp = reinterpret_cast<unsigned char*>(d + scratch);
  int* dkeep = keep.empty() ? nullptr : reinterpret_cast<int*>(d + scratch + spb);
  unsigned char* dimg = reinterpret_cast<unsigned char*>(d + scratch + spb + kb);
  CU(cudaMemcpyAsync(dsp, sp.data(), sp.size(), cudaMemcpyHostToDevice, B->st));
  if (dkeep) CU(cudaMemcpyAsync(dkeep, keep.data(), sizeof(int) * keep.size(), cudaMemcpyHostToDevice, B->st));
  launch_render(B->b, sys, P.n, dsp, dkeep, v->images, v->dipoles, v->box, (float)pix, (float)(0.5 * pix), e, f, r,
                u, l, (float)tan_half, v->width, v->height, d, dimg, B->st);
  CU(cudaGetLastError());
  CU(cudaMemcpyAsync(rgb, dimg, img, cudaMemcpyDeviceToHost, B->st));
  CU(cudaFreeAsync(d, B->st));
  CU(cudaStreamSynchronize(B->st));
  return MDSC_OK;
}

// ---- moving a system between batches (continuous batching) -------------
mdsc_status mdsc_transfer(mdsc_batch* D, int dsys, mdsc_batch* S, int ssys) {
  if (!D || !S || dsys < 0 || dsys >= D->nsys || ssys < 0 || ssys >= S->nsys) return MDSC_ERR_BAD_ARG;
  mdsc_batch* B = D;
  const SysDev& Ps = S->lo.sys[ssys];
  SysDev& Pd = D->lo.sys[dsys];
  if (Ps.n != Pd.n || Ps.nd != Pd.nd || S->device != D->device)
    return fail(D, MDSC_ERR_BAD_ARG, "mdsc_transfer: systems differ in size or device");
  if (!S->uploaded[ssys]) return fail(D, MDSC_ERR_STATE, "mdsc_transfer: source system has no state");
  cudaSetDevice(D->device);
  CU(cudaStreamSynchronize(S->st));
  const int n = Ps.n, nd = Ps.ndip;
  const int is = Ps.part_off, id = Pd.part_off, gs = Ps.dip_off, gd = Pd.dip_off;
  const Batch& a = S->b;
  const Batch& b = D->b;
  auto cp = [&](void* dst, const void* src, size_t bytes) -> cudaError_t {
    return bytes ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, D->st) : cudaSuccess;
  };
  CU(cp(b.r + 3 * id, a.r + 3 * is, sizeof(double) * 3 * n));
  CU(cp(b.p + 3 * id, a.p + 3 * is, sizeof(double) * 3 * n));
  CU(cp(b.O + 9 * id, a.O + 9 * is, sizeof(double) * 9 * n));
  CU(cp(b.l + 3 * id, a.l + 3 * is, sizeof(double) * 3 * n));
  CU(cp(b.F + 3 * id, a.F + 3 * is, sizeof(double) * 3 * n));
  CU(cp(b.T + 3 * id, a.T + 3 * is, sizeof(double) * 3 * n));
  CU(cp(b.len + id, a.len + is, sizeof(double) * n));
  CU(cp(b.dia + id, a.dia + is, sizeof(double) * n));
  CU(cp(b.mass + id, a.mass + is, sizeof(double) * n));
  CU(cp(b.inert + 3 * id, a.inert + 3 * is, sizeof(double) * 3 * n));
  CU(cp(b.invm + id, a.invm + is, sizeof(double) * n));
  CU(cp(b.invI + 3 * id, a.invI + 3 * is, sizeof(double) * 3 * n));
  CU(cp(b.dpc + gd, a.dpc + gs, sizeof(double) * nd));
  CU(cp(b.dob + 3 * gd, a.dob + 3 * gs, sizeof(double) * 3 * nd));
  CU(cp(b.dmu + gd, a.dmu + gs, sizeof(double) * nd));
  std::vector<int> owner(nd);
  for (int g = 0; g < nd; ++g) owner[g] = id + g / std::max(Ps.nd, 1);
  CU(cudaMemcpyAsync(b.downer + gd, owner.data(), sizeof(int) * nd, cudaMemcpyHostToDevice, D->st));
  // per-system constants set at upload, and the mutable state
  Pd.sig_max = Ps.sig_max;
  Pd.skin = Ps.skin;
  Pd.r_list = Ps.r_list;
  Pd.Uself = Ps.Uself;
  Pd.cl_mode = Ps.cl_mode;
  Pd.rl_r2 = Ps.rl_r2;
  Pd.ncell = Ps.ncell;
  Pd.cnx = Ps.cnx;
  Pd.cny = Ps.cny;
  Pd.cnz = Ps.cnz;
  if (Pd.cl_mode == 1) {
    const mdsc_status est = ensure_energy_lists(D);
    if (est) return est;
  }
  Pd.cl_ubond = Ps.cl_ubond;
  CU(cudaMemcpyAsync((void*)(b.sys + dsys), &Pd, sizeof(SysDev), cudaMemcpyHostToDevice, D->st));
  SysState st;
  CU(cudaMemcpy(&st, a.st + ssys, sizeof st, cudaMemcpyDeviceToHost));
  st.force_list = 1;
  st.rebuild = 0;
  st.iter = 0;
  CU(cudaMemcpyAsync(b.st + dsys, &st, sizeof st, cudaMemcpyHostToDevice, D->st));
  CU(cudaStreamSynchronize(D->st));
  D->thermo_rng[2 * dsys] = S->thermo_rng[2 * ssys];
  D->thermo_rng[2 * dsys + 1] = S->thermo_rng[2 * ssys + 1];
  D->clus_rng[dsys] = S->clus_rng[ssys];
  D->step_h[dsys] = S->step_h[ssys];
  D->stop_h[dsys] = S->stop_h[ssys];
  D->labels[dsys] = S->labels[ssys];
  D->n_clusters[dsys] = S->n_clusters[ssys];
  D->uploaded[dsys] = 1;
  D->built[dsys] = 0;
  D->have_forces[dsys] = S->have_forces[ssys];
  return MDSC_OK;
}

mdsc_status mdsc_transfer_many(mdsc_batch* D, mdsc_batch* S, const int* dsys, const int* ssys, int count) {
  if (!D || !S || count < 0 || (count > 0 && (!dsys || !ssys))) return MDSC_ERR_BAD_ARG;
  mdsc_batch* B = D;
  if (S->device != D->device) return fail(D, MDSC_ERR_BAD_ARG, "mdsc_transfer_many: batches on different devices");
  std::vector<int2> pairs(count);
  bool energy = false;
  for (int k = 0; k < count; ++k) {
    const int d = dsys[k], q = ssys[k];
    if (d < 0 || d >= D->nsys || q < 0 || q >= S->nsys) return MDSC_ERR_BAD_ARG;
    const SysDev& Ps = S->lo.sys[q];
    const SysDev& Pd = D->lo.sys[d];
    if (Ps.n != Pd.n || Ps.nd != Pd.nd)
      return fail(D, MDSC_ERR_BAD_ARG, "mdsc_transfer_many: systems differ in size");
    if (!S->uploaded[q]) return fail(D, MDSC_ERR_STATE, "mdsc_transfer_many: a source system has no state");
    energy |= Ps.cl_mode == 1;
    pairs[k] = make_int2(d, q);
  }
  if (count == 0) return MDSC_OK;
  cudaSetDevice(D->device);
  if (energy) {
    const mdsc_status est = ensure_energy_lists(D);
    if (est) return est;
  }
  // the source's work is done before its state is read
  CU(cudaEventRecord(S->ev_fork, S->st));
  CU(cudaStreamWaitEvent(D->st, S->ev_fork, 0));
  for (const int2& pr : pairs) {
    const SysDev& Ps = S->lo.sys[pr.y];
    SysDev& Pd = D->lo.sys[pr.x];
    Pd.sig_max = Ps.sig_max;
    Pd.skin = Ps.skin;
    Pd.r_list = Ps.r_list;
    Pd.Uself = Ps.Uself;
    Pd.cl_mode = Ps.cl_mode;
    Pd.rl_r2 = Ps.rl_r2;
    Pd.ncell = Ps.ncell;
    Pd.cnx = Ps.cnx;
    Pd.cny = Ps.cny;
    Pd.cnz = Ps.cnz;
    Pd.cl_ubond = Ps.cl_ubond;
  }
  // the whole constant table once (the host copy stays alive with the batch)
  CU(cudaMemcpyAsync((void*)D->b.sys, D->lo.sys.data(), sizeof(SysDev) * D->nsys, cudaMemcpyHostToDevice, D->st));
  CU(launch_transfer(D->b, S->b, pairs, D->st));
  // the source's stream waits for the copies, so destroying the source
  // (which synchronizes its stream before freeing) cannot free what they read
  {
    cudaEvent_t copied = nullptr;
    CU(cudaEventCreateWithFlags(&copied, cudaEventDisableTiming));
    const cudaError_t e1 = cudaEventRecord(copied, D->st);
    const cudaError_t e2 = e1 == cudaSuccess ? cudaStreamWaitEvent(S->st, copied, 0) : e1;
    cudaEventDestroy(copied);
    CU(e2);
  }
  for (const int2& pr : pairs) {
    const int d = pr.x, q = pr.y;
    D->thermo_rng[2 * d] = S->thermo_rng[2 * q];
    D->thermo_rng[2 * d + 1] = S->thermo_rng[2 * q + 1];
    D->clus_rng[d] = S->clus_rng[q];
    D->step_h[d] = S->step_h[q];
    D->stop_h[d] = S->stop_h[q];
    D->labels[d] = S->labels[q];
    D->n_clusters[d] = S->n_clusters[q];
    D->uploaded[d] = 1;
    D->built[d] = 0;
    D->have_forces[d] = S->have_forces[q];
  }
  return MDSC_OK;
}

// ---- the fused step ----------------------------------------------------
// nsteps steps; trace (nsteps x nsys, may be NULL) gets every step's
// observables: a copy of the device observables after each graph launch into
// pinned staging, converted after the chunk
// out (mdsc_step_io): the host state the last step's results go to, the
// positions and orientations while that step's forces are computed
static mdsc_status run_steps(mdsc_batch* B, int nsteps, mdsc_observables* trace,
                             const mdsc_host_state* out = nullptr) {
  mdsc_status st = ensure_forces(B);
  if (st) return st;
  if (!B->tuned && !B->graph[0]) {
    // launch mappings by the autotuner (MDSC_AUTOTUNE=0: keep the defaults)
    const char* env = std::getenv("MDSC_AUTOTUNE");
    if (env && env[0] == '0') {
      B->tuned = 1;
    } else {
      st = autotune(B, 0, 5);
      if (st) return st;
    }
  }
  for (int w = 0; w < 2; ++w)
    if (!B->graph[w]) {
      st = capture_step(B, w);
      if (st) return st;
    }
  for (int w = 0; out && w < 2; ++w)
    if (!B->graph_io[w]) {
      st = capture_step(B, w, true);
      if (st) return st;
    }
  if (trace && !B->h_trace) CU(cudaMallocHost(&B->h_trace, sizeof(SysObs) * kNoiseChunk * B->nsys));
  int which = 0;
  int done = 0;
  double dev_ms = 0.0;
  while (done < nsteps) {
    // steps until the next clustering step of any system (inclusive)
    int chunk = std::min(nsteps - done, kNoiseChunk);
    for (int s = 0; s < B->nsys; ++s) {
      const int fr = B->desc[s].cl_fr;
      if (fr <= 0) continue;
      const long long k0 = B->step_h[s];
      const long long next = ((k0 + fr - 1) / fr) * fr;  // first k >= k0 with k % fr == 0
      chunk = (int)std::min<long long>(chunk, next - k0 + 1);
    }
    // noise for this chunk, into the host buffer of this noise buffer once
    // its last copy has gone (no wait for the GPU's other work: an upload or
    // the last chunk's steps run meanwhile)
    double* hn = which ? B->h_noise2 : B->h_noise;
    CU(cudaEventSynchronize(B->ev_noise[which]));
    draw_noise(B, chunk, hn);
    CU(cudaEventRecord(B->t_beg, B->st));
    CU(cudaMemcpyAsync(B->noise[which], hn, sizeof(double) * chunk * B->nsys * 4, cudaMemcpyHostToDevice, B->st));
    CU(cudaEventRecord(B->ev_noise[which], B->st));
    launch_reset_iter(B->b, B->st);
    for (int k = 0; k < chunk; ++k) {
      const bool io = out && done + k == nsteps - 1;
      CU(cudaGraphLaunch(io ? B->graph_io[which] : B->graph[which], B->st));
      if (io) {
        // r and O are final after the first half-step (moveX; renorm every
        // 100 steps before it): they go home while the forces are computed;
        // p, l, F, T once the force assembly has written them, beside the
        // per-system sums
        const size_t n = B->lo.ntot;
        auto dn = [&](double* dst, const double* src, size_t w) -> cudaError_t {
          return dst ? cudaMemcpyAsync(dst, src, sizeof(double) * w * n, cudaMemcpyDeviceToHost, B->sio) : cudaSuccess;
        };
        CU(cudaStreamWaitEvent(B->sio, B->ev_x, 0));
        CU(dn(out->r, B->b.r, 3));
        CU(dn(out->O, B->b.O, 9));
        CU(cudaStreamWaitEvent(B->sio, B->ev_f, 0));
        CU(dn(out->p, B->b.p, 3));
        CU(dn(out->l, B->b.l, 3));
        CU(dn(out->F, B->b.F, 3));
        CU(dn(out->T, B->b.T, 3));
      }
      if (trace)
        CU(cudaMemcpyAsync(B->h_trace + (size_t)k * B->nsys, B->b.obs, sizeof(SysObs) * B->nsys,
                           cudaMemcpyDeviceToHost, B->st));
    }
    CU(cudaEventRecord(B->t_end, B->st));
    {
      CU(cudaEventSynchronize(B->t_end));
      float t = 0.f;
      CU(cudaEventElapsedTime(&t, B->t_beg, B->t_end));
      dev_ms += t;
    }
    std::vector<int> due;
    for (int s = 0; s < B->nsys; ++s) {
      const int fr = B->desc[s].cl_fr;
      const long long took = std::max(0LL, std::min<long long>(chunk, B->stop_h[s] - B->step_h[s]));
      const long long last = B->step_h[s] + took - 1;
      if (fr > 0 && took == chunk && last % fr == 0) due.push_back(s);
      B->step_h[s] += took;
    }
    if (trace)  // cluster counts as they stood before this chunk's clustering step
      for (int k = 0; k < chunk; ++k)
        for (int s = 0; s < B->nsys; ++s)
          convert_obs(B->h_trace[(size_t)k * B->nsys + s], B->lo.sys[s].n, B->n_clusters[s],
                      trace[(size_t)(done + k) * B->nsys + s]);
    if (!due.empty()) {
      st = run_clusters(B, due);
      if (st) return st;
      if (trace)
        for (int s : due) trace[(size_t)(done + chunk - 1) * B->nsys + s].n_clusters = B->n_clusters[s];
    }
    done += chunk;
    which ^= 1;
  }
  B->last_ms = dev_ms;
  return MDSC_OK;
}

mdsc_status mdsc_step(mdsc_batch* B, int nsteps, mdsc_observables* obs) {
  if (!B || nsteps < 0) return MDSC_ERR_BAD_ARG;
  cudaSetDevice(B->device);
  mdsc_status st = run_steps(B, nsteps, nullptr);
  if (st) return st;
  return read_obs(B, obs);
}

mdsc_status mdsc_step_io(mdsc_batch* B, const mdsc_host_state* in, int nsteps, mdsc_host_state* out,
                         mdsc_observables* obs) {
  if (!B || nsteps < 0) return MDSC_ERR_BAD_ARG;
  cudaSetDevice(B->device);
  mdsc_status st = MDSC_OK;
  if (in) {
    st = mdsc_upload_all(B, in);
    if (st) return st;
  }
  if (nsteps == 0) {
    if (out) st = mdsc_download_all(B, out);
    return st ? st : read_obs(B, obs);
  }
  st = run_steps(B, nsteps, nullptr, out);
  if (st) return st;
  // the observables behind the state on the same stream, one wait for both
  CU(cudaMemcpyAsync(B->h_obs, B->b.obs, sizeof(SysObs) * B->nsys, cudaMemcpyDeviceToHost, B->st));
  CU(cudaStreamSynchronize(B->sio));
  CU(cudaStreamSynchronize(B->st));
  if (out) {
    if (out->clust) {
      int off = 0;
      for (int s = 0; s < B->nsys; ++s) {
        std::copy(B->labels[s].begin(), B->labels[s].end(), out->clust + off);
        off += (int)B->labels[s].size();
      }
    }
  }
  return finish_obs(B, obs);
}

mdsc_status mdsc_step_trace(mdsc_batch* B, int nsteps, mdsc_observables* trace) {
  if (!B || nsteps < 0 || (nsteps > 0 && !trace)) return MDSC_ERR_BAD_ARG;
  cudaSetDevice(B->device);
  mdsc_status st = run_steps(B, nsteps, trace);
  if (st) return st;
  st = read_obs(B, nullptr);  // a system's error bits persist: they show in its last step
  if (st) return st;
  for (size_t k = 0; k < (size_t)nsteps * B->nsys; ++k)
    if (trace[k].status != MDSC_OK) return fail(B, (mdsc_status)trace[k].status, "a system reported an error");
  return MDSC_OK;
}

mdsc_status mdsc_get_rng(const mdsc_batch* B, int sys, int which, uint32_t* mt, int* mti) {
  if (!B || sys < 0 || sys >= B->nsys || which < 0 || which > 2 || !mt || !mti) return MDSC_ERR_BAD_ARG;
  const Mt19937& g = which < 2 ? B->thermo_rng[2 * sys + which] : B->clus_rng[sys];
  g.get_state(mt, mti);
  return MDSC_OK;
}

mdsc_status mdsc_set_rng(mdsc_batch* B, int sys, int which, const uint32_t* mt, int mti) {
  if (!B || sys < 0 || sys >= B->nsys || which < 0 || which > 2 || !mt) return MDSC_ERR_BAD_ARG;
  Mt19937& g = which < 2 ? B->thermo_rng[2 * sys + which] : B->clus_rng[sys];
  if (!g.set_state(mt, mti)) return fail(B, MDSC_ERR_BAD_ARG, "mdsc_set_rng: position outside 0..624");
  return MDSC_OK;
}

double mdsc_last_device_ms(const mdsc_batch* B) { return B ? B->last_ms : 0.0; }

mdsc_status mdsc_autotune(mdsc_batch* B, int force) {
  if (!B) return MDSC_ERR_BAD_ARG;
  cudaSetDevice(B->device);
  const mdsc_status st = autotune(B, force, 5);
  if (st) return st;
  // the step graphs hold the old mappings: capture them again at the next step
  drop_graphs(B);
  return MDSC_OK;
}

mdsc_status mdsc_set_step_limit(mdsc_batch* B, int sys, long long limit) {
  if (!B || sys < 0 || sys >= B->nsys) return MDSC_ERR_BAD_ARG;
  cudaSetDevice(B->device);
  const long long v = limit > 0 ? limit : LLONG_MAX;
  B->stop_h[sys] = v;
  SysState* d = B->b.st + sys;
  CU(cudaMemcpyAsync((char*)d + offsetof(SysState, stop), &v, sizeof v, cudaMemcpyHostToDevice, B->st));
  CU(cudaStreamSynchronize(B->st));
  return MDSC_OK;
}

mdsc_status mdsc_set_list_cells(mdsc_batch* B, int on) {
  if (!B || (on != 0 && on != 1)) return MDSC_ERR_BAD_ARG;
  B->b.cells = on;
  drop_graphs(B);
  return MDSC_OK;
}

mdsc_status mdsc_set_tuning(mdsc_batch* B, const int* values) {
  if (!B || !values) return MDSC_ERR_BAD_ARG;
  const int w = values[0], rt = values[1], wb = values[2], kg = values[3];
  if (!(w == 1 || w == 2 || w == 4) || !(rt == 128 || rt == 256 || rt == 512) || wb < 1 || wb > (1 << 20) ||
      !(kg == 0 || kg == 1))
    return fail(B, MDSC_ERR_BAD_ARG, "mdsc_set_tuning: tiles per block 1/2/4, strip-sum threads 128/256/512, "
                                     "WCA blocks 1..2^20, gather form 0/1");
  B->b.tune.rp_warps = w;
  B->b.tune.rsum_threads = rt;
  B->b.tune.wca_blocks = wb;
  B->b.tune.kg_scalar = kg;
  B->tuned = 1;
  drop_graphs(B);
  return MDSC_OK;
}

mdsc_status mdsc_tuning(const mdsc_batch* B, int* values, char* log, size_t len) {
  if (!B) return MDSC_ERR_BAD_ARG;
  if (values) {
    values[0] = B->b.tune.rp_warps;
    values[1] = B->b.tune.rsum_threads;
    values[2] = B->b.tune.wca_blocks;
    values[3] = B->b.tune.kg_scalar;
    values[4] = B->tuned;
  }
  if (log && len) snprintf(log, len, "%s", B->tune_log.c_str());
  return MDSC_OK;
}

mdsc_status mdsc_observe(mdsc_batch* B, mdsc_observables* obs) {
  if (!B) return MDSC_ERR_BAD_ARG;
  cudaSetDevice(B->device);
  mdsc_status st = ensure_forces(B);
  if (st) return st;
  return read_obs(B, obs);
}

mdsc_status mdsc_profile_steps(mdsc_batch* B, int nsteps, int max_kernels, char* names,
                               size_t name_stride, double* ms, int* n_kernels) {
  if (!B || nsteps <= 0) return MDSC_ERR_BAD_ARG;
  cudaSetDevice(B->device);
  mdsc_status st = ensure_forces(B);
  if (st) return st;
  const char* kn[12] = {"integrate_first", "order_terms", "list_build", "wca", "real_pairs", "real_sum",
                        "near_pass_real", "kspace_sum", "kspace_combine", "kspace_gather", "finalize",
                        "reduce_obs"};
  const int nk = 12;
  std::vector<cudaEvent_t> ev(nk + 1);
  for (auto& e : ev) cudaEventCreate(&e);
  std::vector<double> acc(nk, 0.0);
  CU(cudaEventSynchronize(B->ev_noise[0]));
  draw_noise(B, 1, B->h_noise);
  Batch b = batch_with_noise(B, 0);
  for (int it = 0; it < nsteps; ++it) {
    CU(cudaMemcpyAsync(B->noise[0], B->h_noise, sizeof(double) * B->nsys * 4, cudaMemcpyHostToDevice, B->st));
    launch_reset_iter(b, B->st);
    cudaEventRecord(ev[0], B->st);
    launch_integrate_first(b, B->st);
    cudaEventRecord(ev[1], B->st);
    launch_order_terms(b, B->st);
    cudaEventRecord(ev[2], B->st);
    launch_list_build(b, 0, B->st);
    cudaEventRecord(ev[3], B->st);
    launch_wca(b, 0, B->st);
    cudaEventRecord(ev[4], B->st);
    launch_real_pairs(b, B->lo.multi, B->st);
    cudaEventRecord(ev[5], B->st);
    launch_real_sum(b, B->st);
    cudaEventRecord(ev[6], B->st);
    launch_near_pass(b, 1, B->st);
    cudaEventRecord(ev[7], B->st);
    // the three k-space kernels, timed one by one
    launch_kspace_parts(b, B->lo.maxnd, B->kwork, (int)B->lo.kwork.size(), B->kowner, b.kE, 0, B->st);
    cudaEventRecord(ev[8], B->st);
    launch_kspace_parts(b, B->lo.maxnd, B->kwork, (int)B->lo.kwork.size(), B->kowner, b.kE, 1, B->st);
    cudaEventRecord(ev[9], B->st);
    launch_kspace_parts(b, B->lo.maxnd, B->kwork, (int)B->lo.kwork.size(), B->kowner, b.kE, 2, B->st);
    cudaEventRecord(ev[10], B->st);
    launch_finalize(b, kMaskAll | kFlagMoveP, B->st);
    cudaEventRecord(ev[11], B->st);
    launch_reduce_obs(b, kRedStep, B->st);
    cudaEventRecord(ev[12], B->st);
    CU(cudaStreamSynchronize(B->st));
    for (int k = 0; k < nk; ++k) {
      float t = 0;
      cudaEventElapsedTime(&t, ev[k], ev[k + 1]);
      acc[k] += t;
    }
    for (int s = 0; s < B->nsys; ++s) B->step_h[s] += 1;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  const int m = std::min(nk, max_kernels);
  for (int k = 0; k < m; ++k) {
    if (names) snprintf(names + k * name_stride, name_stride, "%s", kn[k]);
    if (ms) ms[k] = acc[k] / nsteps;
  }
  if (n_kernels) *n_kernels = m;
  CU(cudaGetLastError());
  return MDSC_OK;
}

}  // extern "C"
