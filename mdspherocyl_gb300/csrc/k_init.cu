// A new configuration on the GPU -- the reference's signal-0 start.
//
// Positions: ini_pos's lattice (v25/functions.cpp:491-582).  Species n is put
// on the sites of a lattice of its own diameter and length -- rows dia apart
// in x, staggered rows sqrt(3)/2 dia apart in y, layers dia sqrt(6)/3 + len
// apart in z, all stretched by 1.0001 and wrapped into the box -- in the
// order nz, ny, nx, with every rod along z.  A site of species n > 0 is
// skipped when the rod there would come closer than (dia_n + dia_m)/2 to
// any rod of an earlier species m (the reference's segment distance, in
// its own arithmetic: this file is compiled without FMA contraction).  Each
// site is a thread; the host takes the accepted sites in order, and past
// the last site starts over, as the reference's while loop does.  The
// overlap test ini_pos closes with (:599-665) is a pair kernel.
//
// Momenta: Maxwell-Boltzmann at temperature T with zero total momentum,
// from a counter-based generator (SplitMix64, Steele, Lea & Flood, OOPSLA
// 2014, on (seed, system, particle, component)) and Box-Muller.  This is
// not the reference's ini_mom, which draws from its run generator; the
// reference then also shuffles the lattice with 1000 cluster moves
// (GCAmix, :3328-3409), which are not made here.
#include "mdsc_dev.cuh"
#include "seg_dist.cuh"

namespace mdsc {

struct LatticeSpec {
  double len, dia;   // this species
  int num1, num2;    // sites per row and rows per layer
  int nsites;        // num1 * num2 * num3
  int prev_first, prev_n;  // earlier species: batch particles [prev_first, prev_first + prev_n)
};

__device__ __forceinline__ void lattice_site(const LatticeSpec& S, const SysDev& P, int s, double r[3]) {
  const double sq = sqrt(3.) / 2.;
  const double sqt = 1. / (2 * sqrt(3.));
  const double sqtt = sqrt(6.) / 3;
  const int nx = s % S.num1, ny = (s / S.num1) % S.num2, nz = s / (S.num1 * S.num2);
  const double dia = S.dia;
  if (nz % 2 == 0) {
    r[0] = ny % 2 == 0 ? dia * (double)nx * 1.0001 : dia * ((double)nx + 0.5) * 1.0001;
    r[1] = dia * (double)ny * sq * 1.0001;
  } else {
    r[0] = ny % 2 != 0 ? dia * (double)nx * 1.0001 : dia * ((double)nx + 0.5) * 1.0001;
    r[1] = dia * ((double)ny * sq + sqt) * 1.0001;
  }
  r[2] = (dia * sqtt + S.len) * (double)nz * 1.0001;
  for (int a = 0; a < 3; ++a) r[a] -= P.L[a] * floor(r[a] / P.L[a] + 0.5);
}

// every site of one species: its position, and whether it is free of the
// earlier species
__global__ void lattice_sites_kernel(Batch b, int sys, LatticeSpec S, double* __restrict__ site_r,
                                     int* __restrict__ ok) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= S.nsites) return;
  const SysDev& P = b.sys[sys];
  RodD A;
  lattice_site(S, P, s, A.r);
  A.o[0] = 0.0;
  A.o[1] = 0.0;
  A.o[2] = 1.0;
  A.len = S.len;
  int free = 1;
  for (int j = S.prev_first; j < S.prev_first + S.prev_n && free; ++j) {
    RodD Bj;
    for (int a = 0; a < 3; ++a) {
      Bj.r[a] = b.r[3 * j + a];
      Bj.o[a] = b.O[9 * j + 6 + a];
    }
    Bj.len = b.len[j];
    double rij[3];
    for (int a = 0; a < 3; ++a) rij[a] = dmimg(A.r[a] - Bj.r[a], P.L[a]);
    const double dd = (S.dia + b.dia[j]) / 2;
    // no overlap is possible beyond the half lengths and the contact distance
    const double reach = 0.5 * (S.len + Bj.len) + dd;
    if (rij[0] * rij[0] + rij[1] * rij[1] + rij[2] * rij[2] >= reach * reach * 1.0000001) continue;
    double dAB[3], st[2];
    const double dsq = seg_dist_ref<true>(A, Bj, P.L, rij, dAB, st);
    if (dsq < dd * dd) free = 0;
  }
  for (int a = 0; a < 3; ++a) site_r[3 * s + a] = A.r[a];
  ok[s] = free;
}

// ini_pos's closing test: any two rods of the system closer than their
// mean diameter; counts the overlapping pairs
__global__ void overlap_count_kernel(Batch b, int sys, int* __restrict__ count) {
  const SysDev& P = b.sys[sys];
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= P.n) return;
  const int i = P.part_off + k;
  RodD A;
  for (int a = 0; a < 3; ++a) {
    A.r[a] = b.r[3 * i + a];
    A.o[a] = b.O[9 * i + 6 + a];
  }
  A.len = b.len[i];
  int c = 0;
  for (int j = i + 1; j < P.part_off + P.n; ++j) {
    RodD Bj;
    for (int a = 0; a < 3; ++a) {
      Bj.r[a] = b.r[3 * j + a];
      Bj.o[a] = b.O[9 * j + 6 + a];
    }
    Bj.len = b.len[j];
    double rij[3];
    for (int a = 0; a < 3; ++a) rij[a] = dmimg(A.r[a] - Bj.r[a], P.L[a]);
    const double dd = (b.dia[i] + b.dia[j]) / 2;
    const double reach = 0.5 * (A.len + Bj.len) + dd;
    if (rij[0] * rij[0] + rij[1] * rij[1] + rij[2] * rij[2] >= reach * reach * 1.0000001) continue;
    double dAB[3], st[2];
    if (seg_dist_ref<true>(A, Bj, P.L, rij, dAB, st) < dd * dd) ++c;
  }
  if (c) atomicAdd(count, c);
}

__device__ __forceinline__ unsigned long long splitmix64(unsigned long long x) {
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

// a standard normal deviate from stream (key, k): two uniforms in (0, 1]
// from the 53 high bits of two generator outputs, Box-Muller
__device__ __forceinline__ double normal_of(unsigned long long key, int k) {
  const unsigned long long a = splitmix64(key ^ splitmix64(2ull * k));
  const unsigned long long c = splitmix64(key ^ splitmix64(2ull * k + 1));
  const double u1 = ((double)(a >> 11) + 1.0) * (1.0 / 9007199254740992.0);
  const double u2 = (double)(c >> 11) * (1.0 / 9007199254740992.0);
  return sqrt(-2.0 * log(u1)) * cos(2.0 * M_PI * u2);
}

// momenta and angular momenta at temperature T (body frame sqrt(I T) N(0,1),
// turned to the lab frame by O^T); the total momentum is removed after
__global__ void thermalize_kernel(Batch b, int sys, double temp, unsigned long long seed) {
  const SysDev& P = b.sys[sys];
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= P.n) return;
  const int i = P.part_off + k;
  const unsigned long long key = splitmix64(seed ^ splitmix64(((unsigned long long)sys << 32) | (unsigned)k));
  const double sm = sqrt(b.mass[i] * temp);
  double lb[3];
  for (int a = 0; a < 3; ++a) {
    b.p[3 * i + a] = sm * normal_of(key, a);
    lb[a] = sqrt(b.inert[3 * i + a] * temp) * normal_of(key, 3 + a);
  }
  const double* O = b.O + 9 * i;
  for (int a = 0; a < 3; ++a) b.l[3 * i + a] = O[0 * 3 + a] * lb[0] + O[1 * 3 + a] * lb[1] + O[2 * 3 + a] * lb[2];
}

// one block: the system's mean momentum, in particle order, taken off
__global__ void zero_momentum_kernel(Batch b, int sys) {
  __shared__ double part[3][256];
  const SysDev& P = b.sys[sys];
  double s[3] = {0.0, 0.0, 0.0};
  for (int k = threadIdx.x; k < P.n; k += blockDim.x)
    for (int a = 0; a < 3; ++a) s[a] += b.p[3 * (P.part_off + k) + a];
  for (int a = 0; a < 3; ++a) part[a][threadIdx.x] = s[a];
  __syncthreads();
  __shared__ double mean[3];
  if (threadIdx.x < 3) {
    double t = 0.0;
    for (int q = 0; q < (int)blockDim.x; ++q) t += part[threadIdx.x][q];
    mean[threadIdx.x] = P.n > 0 ? t / P.n : 0.0;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < P.n; k += blockDim.x)
    for (int a = 0; a < 3; ++a) b.p[3 * (P.part_off + k) + a] -= mean[a];
}

void launch_lattice_sites(const Batch& b, int sys, double len, double dia, int num1, int num2, int nsites,
                          int prev_first, int prev_n, double* site_r, int* ok, cudaStream_t s) {
  LatticeSpec S{len, dia, num1, num2, nsites, prev_first, prev_n};
  if (nsites > 0) lattice_sites_kernel<<<cdiv(nsites, 128), 128, 0, s>>>(b, sys, S, site_r, ok);
}
void launch_overlap_count(const Batch& b, int sys, int n, int* count, cudaStream_t s) {
  if (n > 0) overlap_count_kernel<<<cdiv(n, 128), 128, 0, s>>>(b, sys, count);
}
void launch_thermalize(const Batch& b, int sys, int n, double temp, unsigned long long seed, cudaStream_t s) {
  if (n <= 0) return;
  thermalize_kernel<<<cdiv(n, 128), 128, 0, s>>>(b, sys, temp, seed);
  zero_momentum_kernel<<<1, 256, 0, s>>>(b, sys);
}

}  // namespace mdsc
