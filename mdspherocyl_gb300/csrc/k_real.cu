// Real-space Ewald dipolar sum over all minimum-image dipole pairs -- the
// GPU form of force_dipR (v25/functions.cpp:1555-1678).
//
// Work: every unordered pair of dipoles of different particles of a system.
// The pair triangle of each system is cut into 64x64 tiles (I <= J); one
// warp owns one tile, each lane holds two i-dipoles in registers and the
// 64 j-dipoles sit in shared memory.  At step t lane l pairs its i-dipoles
// with j = (l + t) mod 64, so the 32 lanes touch 32 different j's and the
// j-side sums in shared memory need no atomics.  Each pair is evaluated
// once (Newton's third law); the tile writes its i- and j-side sums to
// fixed slots of a partial buffer, which the finalize kernel adds in a
// fixed order -- the result is deterministic.
//
// Arithmetic: FP32.  Pair separations come from 32-bit fixed-point box
// fractions, so the minimum image is an exact integer wrap and the
// separation keeps ~1e-7 relative precision at any box size.  The
// reference does not evaluate erfc directly: it interpolates linearly in a
// 32768-entry FP64 table with spacing Lh = 0.5*200.2/32768
// (v25/functions.cpp:1563,1606-1614,1680-1697), which differs from the
// analytic B(r), C(r) by up to ~5e-5 near contact.  The kernel evaluates the
// analytic terms and adds the table's own interpolation error to second
// and third order, h2 f''(r) + h3 f'''(r) with a = r - r0, b = r1 - r,
// h2 = ab/2, h3 = ab(b - a)/6, using the closed forms (A, B, C as the
// reference's table columns, s = 5B + C)
//   A'' = 4B + C,                A''' = -4s/r - 2a^2 r C
//   B'' = 6s/r^2 + 2a^2 C,       B''' = -42s/r^3 - 12a^2 C/r - 4a^4 r C
//   C'' = 2a^2 C (2a^2 r^2 - 1), C''' = 4a^4 r C (3 - 2a^2 r^2)
// which matches the table to ~2e-9 without reading it.
#include "mdsc_dev.cuh"

namespace mdsc {

struct PairOut {
  float fx, fy, fz;     // force on i (j gets -f)
  float tix, tiy, tiz;  // torque on i without lever arm
  float tjx, tjy, tjz;  // torque on j without lever arm
  float u;              // pair energy
};

// One dipole pair: d = r_i - r_j (minimum image), moment vectors mi, mj.
__device__ __forceinline__ void dip_pair(const SysDev& P, float dx, float dy, float dz, float mix,
                                         float miy, float miz, float mjx, float mjy, float mjz,
                                         PairOut& o) {
  const float r2 = dx * dx + dy * dy + dz * dz;
  const float rinv = rsqrtf(r2);
  const float r = r2 * rinv;
  const float rinv2 = rinv * rinv;
  const float x = P.alphaf * r;
  const float E = erfcf(x);
  const float G = P.gpref * expf(-x * x);
  const float rinv3 = rinv2 * rinv;
  float A = E * rinv3 + G * rinv2;
  float B = (3.f * E * rinv3 + G * (P.alpha2x2 + 3.f * rinv2)) * rinv2;
  float C = P.alpha4x4 * G;
  // the reference table's linear-interpolation error to third order:
  // h2 f'' + h3 f''' with a = r - r0, b = r1 - r, h2 = ab/2, h3 = ab(b - a)/6
  const float uu = r * P.invLh;
  const float fr = uu - floorf(uu);
  const float ab = fr * (1.f - fr);
  const float h2 = P.halfLh2 * ab;
  const float h3 = P.sixthLh3 * ab * (1.f - 2.f * fr);
  const float s5 = 5.f * B + C;
  const float a2 = P.alpha2x2;
  const float a2C = a2 * C;
  const float a2rC = a2C * r;
  const float dA = h2 * (4.f * B + C) - h3 * (4.f * s5 * rinv + a2rC);
  const float dB = h2 * (6.f * s5 * rinv2 + a2C) - h3 * (42.f * s5 * rinv3 + 6.f * a2C * rinv + a2 * a2rC);
  const float dC = h2 * (a2C * (a2 * r2 - 1.f)) + h3 * (a2 * a2rC * (3.f - a2 * r2));
  A += dA;
  B += dB;
  C += dC;

  const float mimj = mix * mjx + miy * mjy + miz * mjz;
  const float mir = mix * dx + miy * dy + miz * dz;
  const float mjr = mjx * dx + mjy * dy + mjz * dz;
  const float pr = mir * mjr;
  o.u = mimj * A - pr * B;
  const float q = pr * rinv2;
  const float fact = (mimj - 5.f * q) * B - q * C;
  o.fx = fact * dx + (mir * mjx + mjr * mix) * B;
  o.fy = fact * dy + (mir * mjy + mjr * miy) * B;
  o.fz = fact * dz + (mir * mjz + mjr * miz) * B;
  // mi x mj scaled by A
  const float wx = A * (miy * mjz - miz * mjy);
  const float wy = A * (miz * mjx - mix * mjz);
  const float wz = A * (mix * mjy - miy * mjx);
  const float bj = mjr * B, bi = mir * B;
  o.tix = bj * (miy * dz - miz * dy) - wx;
  o.tiy = bj * (miz * dx - mix * dz) - wy;
  o.tiz = bj * (mix * dy - miy * dx) - wz;
  o.tjx = bi * (mjy * dz - mjz * dy) + wx;
  o.tjy = bi * (mjz * dx - mjx * dz) + wy;
  o.tjz = bi * (mjx * dy - mjy * dx) + wz;
}

struct IDip {
  uint32_t x, y, z;
  float mx, my, mz;
  int own;
  bool ok;
  float f[3], t[3];
};

template <bool MULTI>
__global__ void __launch_bounds__(32) real_pairs_kernel(Batch b) {
  __shared__ uint32_t sx[kTile], sy[kTile], sz[kTile];
  __shared__ float smx[kTile], smy[kTile], smz[kTile];
  __shared__ int sown[kTile];
  __shared__ float sacc[6][kTile];

  const int4 tl = b.tiles[blockIdx.x];
  const SysDev& P = b.sys[tl.x];
  const int I = tl.y, J = tl.z;
  const bool diag = (I == J);
  const int lane = threadIdx.x;
  const int ndip = P.ndip;
  const int ND = b.ndtot;
  const float sxs = P.Lfix[0], sys_ = P.Lfix[1], szs = P.Lfix[2];

  for (int k = lane; k < kTile; k += 32) {
    const int jj = J * kTile + k;
    const bool v = jj < ndip;
    const int g = P.dip_off + (v ? jj : 0);
    sx[k] = b.dfx[g];
    sy[k] = b.dfx[ND + g];
    sz[k] = b.dfx[2 * ND + g];
    smx[k] = v ? b.dm[g] : 0.f;
    smy[k] = v ? b.dm[ND + g] : 0.f;
    smz[k] = v ? b.dm[2 * ND + g] : 0.f;
    sown[k] = v ? b.downer[g] : -1;
#pragma unroll
    for (int c = 0; c < 6; ++c) sacc[c][k] = 0.f;
  }

  IDip id[2];
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int ii = I * kTile + lane + 32 * h;
    id[h].ok = ii < ndip;
    const int g = P.dip_off + (id[h].ok ? ii : 0);
    id[h].x = b.dfx[g];
    id[h].y = b.dfx[ND + g];
    id[h].z = b.dfx[2 * ND + g];
    id[h].mx = b.dm[g];
    id[h].my = b.dm[ND + g];
    id[h].mz = b.dm[2 * ND + g];
    id[h].own = b.downer[g];
#pragma unroll
    for (int c = 0; c < 3; ++c) id[h].f[c] = id[h].t[c] = 0.f;
  }
  float U = 0.f, Uc = 0.f;  // Kahan-compensated pair-energy sum
  float pt[9];
#pragma unroll
  for (int c = 0; c < 9; ++c) pt[c] = 0.f;
  __syncwarp();

  const int jvalid = min(kTile, ndip - J * kTile);
  for (int t = 0; t < kTile; ++t) {
    const int lj = (lane + t) & (kTile - 1);
    const bool jv = lj < jvalid;
    const uint32_t jx = sx[lj], jy = sy[lj], jz = sz[lj];
    const float mjx = smx[lj], mjy = smy[lj], mjz = smz[lj];
    const int jown = sown[lj];
    float ja[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int li = lane + 32 * h;
      bool act = id[h].ok && jv && (!diag || lj > li);
      if (MULTI) act = act && (id[h].own != jown);
      if (act) {
        const float dx = fix_diff(id[h].x, jx, sxs);
        const float dy = fix_diff(id[h].y, jy, sys_);
        const float dz = fix_diff(id[h].z, jz, szs);
        PairOut o;
        dip_pair(P, dx, dy, dz, id[h].mx, id[h].my, id[h].mz, mjx, mjy, mjz, o);
        id[h].f[0] += o.fx;
        id[h].f[1] += o.fy;
        id[h].f[2] += o.fz;
        id[h].t[0] += o.tix;
        id[h].t[1] += o.tiy;
        id[h].t[2] += o.tiz;
        ja[0] -= o.fx;
        ja[1] -= o.fy;
        ja[2] -= o.fz;
        ja[3] += o.tjx;
        ja[4] += o.tjy;
        ja[5] += o.tjz;
        // Kahan: U += o.u
        const float yk = o.u - Uc;
        const float tk = U + yk;
        Uc = (tk - U) - yk;
        U = tk;
        pt[0] += dx * o.fx; pt[1] += dx * o.fy; pt[2] += dx * o.fz;
        pt[3] += dy * o.fx; pt[4] += dy * o.fy; pt[5] += dy * o.fz;
        pt[6] += dz * o.fx; pt[7] += dz * o.fy; pt[8] += dz * o.fz;
      }
    }
#pragma unroll
    for (int c = 0; c < 6; ++c) sacc[c][lj] += ja[c];
  }
  __syncwarp();

  // partial slots: (strip X, strip Y, component c, local index)
  const int ns = P.nstrip;
  float* base_ij = b.rpart + P.pp_off + ((long long)(I * ns + J) * 6) * kTile;
  float* base_ji = b.rpart + P.pp_off + ((long long)(J * ns + I) * 6) * kTile;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int li = lane + 32 * h;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      float fv = id[h].f[c], tv = id[h].t[c];
      if (diag) {
        fv += sacc[c][li];
        tv += sacc[3 + c][li];
      }
      base_ij[c * kTile + li] = fv;
      base_ij[(3 + c) * kTile + li] = tv;
    }
  }
  if (!diag) {
    for (int k = lane; k < kTile; k += 32) {
#pragma unroll
      for (int c = 0; c < 6; ++c) base_ji[c * kTile + k] = sacc[c][k];
    }
  }
  // tile energy and pressure tensor
  float red[10];
  red[0] = U + (-Uc);
#pragma unroll
  for (int c = 0; c < 9; ++c) red[1 + c] = pt[c];
#pragma unroll
  for (int c = 0; c < 10; ++c) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) red[c] += __shfl_xor_sync(0xffffffffu, red[c], off);
  }
  if (lane == 0) {
#pragma unroll
    for (int c = 0; c < 10; ++c) b.tileE[(long long)blockIdx.x * 10 + c] = red[c];
  }
}

void launch_real_pairs(const Batch& b, bool multi, cudaStream_t s) {
  if (b.ntiles == 0) return;
  if (multi)
    real_pairs_kernel<true><<<b.ntiles, 32, 0, s>>>(b);
  else
    real_pairs_kernel<false><<<b.ntiles, 32, 0, s>>>(b);
}

}  // namespace mdsc
