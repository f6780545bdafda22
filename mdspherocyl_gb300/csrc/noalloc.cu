// Real-space Ewald forces for callers that cannot allocate GPU memory.
//
// Some callers of this library may not call cudaMalloc (or anything that
// allocates) at the point where they need forces: code running inside a
// host that owns a fixed device-memory budget and forbids allocation after
// start-up, a real-time loop where an allocation could stall or fail, or a
// plugin whose host manages every buffer itself.  They hand over inputs and
// outputs that already live on the GPU and need a call that takes no memory
// of its own.  mdsc_force_dipR_noalloc() serves them: it runs the same
// tiled real-space kernel as mdsc_force_dipR(), with its scratch -- the
// per-tile partial sums, the tile list and the single-precision copies of
// the inputs -- in one fixed array of this library's device memory,
// declared below.  That array exists on every GPU that loads the library
// and stays there until the process exits.
//
// Limit: at most kNoAllocMaxDipoles dipoles per call (one dipole per
// particle).  Every call uses the same array and overwrites all of it that
// it reads, so nothing carries over from one call to the next; two calls
// whose work overlaps on the GPU (different streams, or host threads
// calling at once) race on the array and give wrong results.
//
// The array's device address is looked up on a device's first call and
// kept, together with the CUDA context it belongs to.  A later call in
// another context (after cudaDeviceReset, or when the primary context was
// released and created again) looks it up again.  A CUDA error left
// pending by earlier, unrelated work on this thread makes the call return
// MDSC_ERR_CUDA before it launches anything, and the error stays pending
// for its owner to read.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <mutex>

#include "mdsc.h"
#include "mdsc_dev.cuh"

namespace mdsc {
void launch_real_pairs(const Batch& b, bool multi, cudaStream_t s);
}

namespace {

using namespace mdsc;

constexpr int kNoAllocMaxDipoles = 4096;
constexpr int kNoAllocMaxStrips = kNoAllocMaxDipoles / kTile;
constexpr int kNoAllocMaxTiles = kNoAllocMaxStrips * (kNoAllocMaxStrips + 1) / 2;

// byte layout of the scratch array (each part 256-byte aligned)
constexpr size_t al(size_t x) { return (x + 255) / 256 * 256; }
constexpr size_t kOffSys = 0;
constexpr size_t kOffTiles = kOffSys + al(sizeof(SysDev));
constexpr size_t kOffFix = kOffTiles + al(sizeof(int4) * kNoAllocMaxTiles);
constexpr size_t kOffMom = kOffFix + al(sizeof(uint32_t) * 3 * kNoAllocMaxDipoles);
constexpr size_t kOffOwner = kOffMom + al(sizeof(float) * 3 * kNoAllocMaxDipoles);
constexpr size_t kOffPart = kOffOwner + al(sizeof(int) * kNoAllocMaxDipoles);
constexpr size_t kOffTileE = kOffPart + al(sizeof(float) * (size_t)kNoAllocMaxStrips * kNoAllocMaxStrips * 6 * kTile);
constexpr size_t kScratchBytes = kOffTileE + al(sizeof(float) * 10 * kNoAllocMaxTiles);  // ~6.5 MB

// the scratch: file scope, static, fixed size; device code could name it
// directly, host code must ask the runtime for its device address
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr double kLh = 0.5 * (200 * 1.001) / 32768;  // the reference's table spacing

// copies of the inputs the tile kernel reads, its constants and its tile list
__global__ void noalloc_prep_kernel(unsigned char* scr, int ndip, const double* __restrict__ pos,
                                    const double* __restrict__ mom, double bx, double by, double bz,
                                    double alpha) {
  SysDev* P = reinterpret_cast<SysDev*>(scr + kOffSys);
  int4* tiles = reinterpret_cast<int4*>(scr + kOffTiles);
  uint32_t* fx = reinterpret_cast<uint32_t*>(scr + kOffFix);
  float* m = reinterpret_cast<float*>(scr + kOffMom);
  int* own = reinterpret_cast<int*>(scr + kOffOwner);
  const int ns = cdiv(ndip, kTile);
  const int ntile = ns * (ns + 1) / 2;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const double L[3] = {bx, by, bz};
  if (t == 0) {
    SysDev d;
    memset(&d, 0, sizeof d);
    d.n = d.ndip = ndip;
    d.nd = 1;
    d.nstrip = ns;
    d.ntile = ntile;
    for (int a = 0; a < 3; ++a) {
      d.L[a] = L[a];
      d.invL[a] = 1.0 / L[a];
      d.invL32[a] = d.invL[a] * 4294967296.0;
      d.Lfix[a] = (float)(L[a] / 4294967296.0);
      d.Lf[a] = (float)L[a];
    }
    d.alpha = alpha;
    set_real_consts(d, kLh);
    *P = d;
  }
  if (t < ntile) {
    // row-major upper triangle: tile t -> strips (I, J), I <= J
    int I = 0, start = 0;
    while (start + (ns - I) <= t) {
      start += ns - I;
      ++I;
    }
    tiles[t] = make_int4(0, I, I + (t - start), 0);
  }
  if (t < ndip) {
    for (int a = 0; a < 3; ++a) {
      fx[a * ndip + t] = to_fix(pos[3 * t + a], 4294967296.0 / L[a]);
      m[a * ndip + t] = (float)mom[3 * t + a];
    }
    own[t] = t;
  }
}

// per dipole: the tile partials over all partner strips -> F and torque
// (FP64 outputs); one extra block sums the tiles' energy and pressure tensor
__global__ void noalloc_reduce_kernel(const unsigned char* scr, int ndip, double* __restrict__ F,
                                      double* __restrict__ T, double* __restrict__ UPT) {
  const float* part = reinterpret_cast<const float*>(scr + kOffPart);
  const float* tE = reinterpret_cast<const float*>(scr + kOffTileE);
  const int ns = cdiv(ndip, kTile);
  const int nblk_d = cdiv(ndip, blockDim.x);
  if ((int)blockIdx.x < nblk_d) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ndip) return;
    const int X = g / kTile, lx = g % kTile;
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for (int Y = 0; Y < ns; ++Y)
      for (int c = 0; c < 6; ++c) acc[c] += (double)part[((size_t)(X * ns + Y) * 6 + c) * kTile + lx];
    for (int a = 0; a < 3; ++a) {
      F[3 * g + a] = acc[a];
      T[3 * g + a] = acc[3 + a];
    }
    return;
  }
  // energy and pressure tensor: one block, fixed order
  __shared__ double sh[10][256];
  const int ntile = ns * (ns + 1) / 2;
  double v[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int t = threadIdx.x; t < ntile; t += blockDim.x)
    for (int c = 0; c < 10; ++c) v[c] += (double)tE[(size_t)t * 10 + c];
  for (int c = 0; c < 10; ++c) sh[c][threadIdx.x] = v[c];
  __syncthreads();
  if (threadIdx.x < 10) {
    double s = 0.0;
    for (int k = 0; k < (int)blockDim.x; ++k) s += sh[threadIdx.x][k];
    UPT[threadIdx.x] = s;
  }
}

std::mutex g_mu;
void* g_scratch_ptr[64] = {nullptr};  // device address of g_scratch, per device
CUcontext g_scratch_ctx[64] = {nullptr};  // the context that address belongs to

// the calling thread's current context (driver entry point, resolved once)
CUcontext current_context() {
  using Fn = CUresult (*)(CUcontext*);
  static Fn fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return (Fn)f;
  }();
  CUcontext c = nullptr;
  if (!fn || fn(&c) != CUDA_SUCCESS) return nullptr;
  return c;
}

}  // namespace

extern "C" mdsc_status mdsc_force_dipR_noalloc(int ndip, const double* d_pos, const double* d_mom,
                                               const double box[3], double alpha, double* d_F, double* d_T,
                                               double* d_UPT, void* stream) {
  if (ndip < 1 || !d_pos || !d_mom || !box || !d_F || !d_T || !d_UPT) return MDSC_ERR_BAD_ARG;
  if (ndip > kNoAllocMaxDipoles) {
    fprintf(stderr, "mdsc_force_dipR_noalloc: %d dipoles exceed the fixed scratch limit of %d\n", ndip,
            kNoAllocMaxDipoles);
    return MDSC_ERR_TOO_LARGE;
  }
  if (!(box[0] > 0 && box[1] > 0 && box[2] > 0 && alpha > 0)) return MDSC_ERR_BAD_ARG;
  const double hd = 0.5 * std::sqrt(box[0] * box[0] + box[1] * box[1] + box[2] * box[2]);
  if (hd >= 0.5 * 200 * 1.001) return MDSC_ERR_TABLE_RANGE;
  // an error left pending by earlier work stays with its owner
  if (cudaPeekAtLastError() != cudaSuccess) return MDSC_ERR_CUDA;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return MDSC_ERR_NO_DEVICE;
  void* scr = nullptr;
  {
    // set-up, once per device and context, with that device current: the
    // device address of the scratch array
    std::lock_guard<std::mutex> lk(g_mu);
    const CUcontext ctx = current_context();
    if (!g_scratch_ptr[dev] || ctx != g_scratch_ctx[dev]) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || !p) return MDSC_ERR_CUDA;
      g_scratch_ptr[dev] = p;
      g_scratch_ctx[dev] = current_context();
    }
    scr = g_scratch_ptr[dev];
  }
  cudaStream_t st = (cudaStream_t)stream;
  unsigned char* base = (unsigned char*)scr;
  const int ns = cdiv(ndip, kTile);
  const int ntile = ns * (ns + 1) / 2;
  const int nthr = ndip > ntile ? ndip : ntile;
  noalloc_prep_kernel<<<cdiv(nthr, 256), 256, 0, st>>>(base, ndip, d_pos, d_mom, box[0], box[1], box[2],
                                                        alpha);
  if (cudaGetLastError() != cudaSuccess) return MDSC_ERR_CUDA;
  Batch b{};
  b.nsys = 1;
  b.ntot = ndip;
  b.ndtot = ndip;
  b.ntiles = ntile;
  b.sys = reinterpret_cast<const SysDev*>(base + kOffSys);
  b.tiles = reinterpret_cast<int4*>(base + kOffTiles);
  b.dfx = reinterpret_cast<uint32_t*>(base + kOffFix);
  b.dm = reinterpret_cast<float*>(base + kOffMom);
  b.downer = reinterpret_cast<int*>(base + kOffOwner);
  b.rpart = reinterpret_cast<float*>(base + kOffPart);
  b.tileE = reinterpret_cast<float*>(base + kOffTileE);
  launch_real_pairs(b, false, st);
  if (cudaGetLastError() != cudaSuccess) return MDSC_ERR_CUDA;
  noalloc_reduce_kernel<<<cdiv(ndip, 256) + 1, 256, 0, st>>>(base, ndip, d_F, d_T, d_UPT);
  return cudaGetLastError() == cudaSuccess ? MDSC_OK : MDSC_ERR_CUDA;
}
