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
// Packed arithmetic: a lane's two i-dipoles meet the same j at each step,
// so the two pair evaluations run side by side in the two halves of
// float2 values with Blackwell's paired FP32 instructions (__ffma2_rn,
// __fmul2_rn, __fadd2_rn: two FP32 operations per issued instruction).
// Only the special-function steps (rsqrt, exp2, reciprocal, floor) and the
// integer minimum image stay scalar.  Pairs that must be skipped (the lower
// triangle and self pairs of diagonal tiles, ragged strips, dipoles of one
// particle) are zeroed by scaling the i-moment by 0 -- every output is
// linear in it -- so the warp never diverges; tiles with no such pairs run
// a loop without the masks.
//
// Arithmetic: FP32.  Pair separations come from 32-bit fixed-point box
// fractions, so the minimum image is an exact integer wrap and the
// separation keeps ~1e-7 relative precision at any box size.  The
// reference does not evaluate erfc directly: it interpolates linearly in a
// 32768-entry FP64 table with spacing Lh = 0.5*200.2/32768
// (v25/functions.cpp:1563,1606-1614,1680-1697), which differs from the
// analytic B(r), C(r) by up to ~5e-5 near contact.  Two forms reproduce it:
//
// TAB (the neighbour pass of cutoff systems, and the tiles with
// MDSC_REAL_FORM=table): the same interpolation, in the system's own table.
// The host builds it once per system with tabul's expressions in FP64 over
// the distances the box can hold and stores each entry as FP32 A, B, C and
// the differences to the next entry, 32 bytes, read with one 256-bit load
// (one L1 wavefront per lane per lookup).  The lookups are scattered, so
// the kernel leans on the L1 and L2 as well as on the FP32 pipe.
//
// Analytic (the tiles by default, and callers without a table such as
// mdsc_force_dipR_noalloc): the kernel evaluates the analytic terms and
// adds the table's own interpolation error to second order, h2 f''(r) with
// a = r - r0, b = r1 - r, h2 = ab/2, using the closed forms (A, B, C as the
// reference's table columns, s = 5B + C)
//   A'' = 4B + C,   B'' = 6s/r^2 + 2a^2 C,   C'' = 2a^2 C (2a^2 r^2 - 1)
// which matches the table to 2e-7 of each value at r = 0.8 and to 1e-8
// beyond r = 3 (alpha <= 0.55) without reading it; what remains is the
// third-order term h3 f'''(r), h3 = ab(b - a)/6.  The pair step is then
// bound by the FP32 pipe alone.
//
// erfc(x) = exp(-x^2) t Q(t), t = 1/(1 + x/2), with Q a degree-9 polynomial
// fitted to erfcx(x)/t by weighted least squares on Chebyshev nodes over
// 0 <= x <= 9.5 (fit_erfcx.py beside this file; relative error 5e-8 with
// FP32 coefficients).  exp(-x^2) is shared with the Gaussian term.  Beyond
// x = 9.35 exp(-x^2) is below the FP32 range and both terms are 0, as the
// reference's table is there to FP32 precision.
#include "mdsc_dev.cuh"
#include "reduce.cuh"
#include "wca_screen.cuh"

namespace mdsc {

namespace {

using f2 = float2;
__device__ __forceinline__ f2 b2(float a) { return make_float2(a, a); }
__device__ __forceinline__ f2 add2(f2 a, f2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ f2 mul2(f2 a, f2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ f2 neg2(f2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ f2 sub2(f2 a, f2 b) { return __fadd2_rn(a, neg2(b)); }

__device__ __forceinline__ float ex2_approx(float y) {
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(y));
  return r;
}
__device__ __forceinline__ float rcp_approx(float y) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(y));
  return r;
}
__device__ __forceinline__ float rsqrt_approx(float y) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(y));
  return r;
}
// minimum-image separation of two fixed-point coordinates: the integer
// difference times L / 2^32, the scale carried as hi + lo so that its FP32
// rounding does not bias every separation of the system the same way
__device__ __forceinline__ f2 fix_diff2(uint32_t a0, uint32_t a1, uint32_t b0, uint32_t b1, f2 hi, f2 lo) {
  const f2 k = make_float2((float)(int32_t)(a0 - b0), (float)(int32_t)(a1 - b1));
  return fma2(k, hi, mul2(k, lo));
}

// Q(t) coefficients, constant term first (fit_erfcx.py)
constexpr float kQ0 = 2.820587754e-01f, kQ1 = 2.829789221e-01f, kQ2 = 2.375463843e-01f,
                kQ3 = 2.310565114e-01f, kQ4 = -1.153462157e-01f, kQ5 = 4.548966587e-01f,
                kQ6 = -7.125887275e-01f, kQ7 = 4.623427987e-01f, kQ8 = -1.380545348e-01f,
                kQ9 = 1.510943193e-02f;

// one 32-byte table entry in a single 256-bit load through the read-only
// path: the L1 serves a warp's 32 scattered entries in 32 wavefronts, where
// two 128-bit loads would take 64.  Not volatile: the table is constant
// during the kernel, so the compiler may hoist the next step's loads.
__device__ __forceinline__ void ld_entry(const float4* e, float4& p, float4& q) {
  asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=f"(p.x), "=f"(p.y), "=f"(p.z), "=f"(p.w), "=f"(q.x), "=f"(q.y), "=f"(q.z), "=f"(q.w)
               : "l"(e));
}

// 1/Lh of the reference's table spacing Lh = 0.5*200.2/32768, as hi + lo
constexpr double kInvLhD = 32768.0 / (0.5 * (200 * 1.001));
constexpr float kInvLhHi = (float)kInvLhD;
constexpr float kInvLhLo = (float)(kInvLhD - (double)kInvLhHi);

// The analytic form in units of 1/s, s = alpha sqrt(log2 e) (lengths r~ =
// s r, x = alpha r = r~ / sqrt(log2 e)): exp(-x^2) = 2^(-r~^2), and with
// g = 2 / sqrt(pi log2 e) and E = exp(-x^2)
//   A = s^3 (erfc(x)/r~^3 + g E/r~^2),  B = s^5 (3 A~ + (2g/log2 e) E)/r~^2,
//   C = s^5 (4g/log2 e^2) E,  2 alpha^2 = s^2 (2/log2 e)
// so the pair step holds no per-system factor but the length unit; the
// tile's sums go back to length units once, at its end.
constexpr float kHalfX = 0.41627730557884884f;  // 1 / (2 sqrt(log2 e)): x / 2 = kHalfX r~
constexpr float kGq = 0.9394372786996514f;      // g
constexpr float kGB = 1.3023366020871419f;      // 2 g / log2 e
constexpr float kGC = 1.8054218877534436f;      // 4 g / log2 e^2
constexpr float kGC2 = 2.502846182435027f;      // 8 g / log2 e^3
constexpr float kA2 = 1.3862943611198906f;      // 2 / log2 e

// per-system constants, the same value in both halves; lengths in the
// step's unit (1/s for the analytic form, 1 for the table forms)
struct PairConst {
  f2 invLh, halfLh2;                // 1 / Lh and Lh^2 / 2
  f2 Lhx, Lhy, Lhz, Llx, Lly, Llz;  // the fixed-point unit per axis as float-float pairs
  f2 ihh, ihl;                      // 1 / Lh as a float-float pair (table index)
  float rnear;                      // kNearTab
  const float4* tab;                // the system's table entries in global memory (MODE 1)
  const float4* stab;               // its values in shared memory (MODE 2): A, B, C, A' - A per entry
  int tn;                           // its number of entries
};

// how a tile kernel gets the reference's interpolation
enum : int {
  kAnalytic = 0,   // analytic terms plus the table's interpolation error (no table)
  kTabGlobal = 1,  // the system's table in global memory, one 256-bit load per lookup
  kTabShared = 2,  // the system's table staged in shared memory, two 128-bit loads per lookup
};

struct Lane2 {
  uint32_t x0, x1, y0, y1, z0, z1;  // fixed-point positions of the two i-dipoles
  f2 mx, my, mz;                    // their moments (0 for a missing dipole)
  int own0, own1;
  bool ok0, ok1;
  // sums over the lane's pairs: force, the dipolar field of the partners
  // (the torque is mi x field, taken once at the end), pressure tensor and
  // energy (Kahan)
  f2 F[3], E[3], pt[9], U, Uc;
};

// j-side results of one step for the two halves (half 0 pairs i-dipole
// lane with j0, half 1 pairs lane + 32 with j1): the force on i (j gets
// minus it) and the field of i at j
struct JOut {
  f2 fx, fy, fz, ex, ey, ez;
};

// one step of a tile loop: the lane's two i-dipoles against j0 (half 0)
// and j1 (half 1) -- the same j in off-diagonal tiles.  Pairs masked off
// (a0, a1 false) contribute exactly zero: both moments are scaled by 0.
template <bool MASKED, int MODE>
__device__ __forceinline__ void tile_step(const PairConst& K, Lane2& s, const uint4 jp0, const float4 jm0,
                                          const uint4 jp1, const float4 jm1, bool a0, bool a1, JOut& o) {
  f2 mix = s.mx, miy = s.my, miz = s.mz;
  f2 mjx = make_float2(jm0.x, jm1.x), mjy = make_float2(jm0.y, jm1.y), mjz = make_float2(jm0.z, jm1.z);
  if (MASKED) {
    const f2 on = make_float2(a0 ? 1.f : 0.f, a1 ? 1.f : 0.f);
    mix = mul2(mix, on);
    miy = mul2(miy, on);
    miz = mul2(miz, on);
    mjx = mul2(mjx, on);
    mjy = mul2(mjy, on);
    mjz = mul2(mjz, on);
  }
  const f2 dx = fix_diff2(s.x0, s.x1, jp0.x, jp1.x, K.Lhx, K.Llx);
  const f2 dy = fix_diff2(s.y0, s.y1, jp0.y, jp1.y, K.Lhy, K.Lly);
  const f2 dz = fix_diff2(s.z0, s.z1, jp0.z, jp1.z, K.Lhz, K.Llz);
  f2 r2 = fma2(dz, dz, fma2(dy, dy, mul2(dx, dx)));
  if (MASKED) {
    r2.x = a0 ? r2.x : 1.f;
    r2.y = a1 ? r2.y : 1.f;
  }
  const f2 rinv = make_float2(rsqrt_approx(r2.x), rsqrt_approx(r2.y));
  const f2 r = mul2(r2, rinv);
  const f2 rinv2 = mul2(rinv, rinv);

  f2 Ac, Bc, Cc;
  if (MODE == kTabShared) {
    // the same interpolation, entries from the block's shared copy: A and
    // A's difference as stored, B and C's differences from the next entry
    const f2 uu = fma2(r, K.ihh, mul2(r, K.ihl));
    const float fl0 = floorf(uu.x), fl1 = floorf(uu.y);
    const f2 fr = add2(fma2(r, K.ihh, make_float2(-fl0, -fl1)), mul2(r, K.ihl));
    const int e0 = min(max((int)fl0 - 1, 0), K.tn - 1), e1 = min(max((int)fl1 - 1, 0), K.tn - 1);
    const float4 p0 = K.stab[e0], n0 = K.stab[e0 + 1];
    const float4 p1 = K.stab[e1], n1 = K.stab[e1 + 1];
    Ac = fma2(fr, make_float2(p0.w, p1.w), make_float2(p0.x, p1.x));
    Bc = fma2(fr, make_float2(n0.y - p0.y, n1.y - p1.y), make_float2(p0.y, p1.y));
    Cc = fma2(fr, make_float2(n0.z - p0.z, n1.z - p1.z), make_float2(p0.z, p1.z));
  } else if (MODE == kTabGlobal) {
    // the reference's own method: linear interpolation in its table
    // (v25/functions.cpp:1606-1614), entry ri - 1 and ri for ri = floor(r/Lh);
    // r/Lh from a float-float 1/Lh, the fraction by one FMA against the
    // floor so it keeps full precision
    const f2 uu = fma2(r, K.ihh, mul2(r, K.ihl));
    const float fl0 = floorf(uu.x), fl1 = floorf(uu.y);
    const f2 fr = add2(fma2(r, K.ihh, make_float2(-fl0, -fl1)), mul2(r, K.ihl));
    const int e0 = min(max((int)fl0 - 1, 0), K.tn - 1), e1 = min(max((int)fl1 - 1, 0), K.tn - 1);
    float4 p0, q0, p1, q1;
    ld_entry(K.tab + 2 * e0, p0, q0);
    ld_entry(K.tab + 2 * e1, p1, q1);
    Ac = fma2(fr, make_float2(p0.w, p1.w), make_float2(p0.x, p1.x));
    Bc = fma2(fr, make_float2(q0.x, q1.x), make_float2(p0.y, p1.y));
    Cc = fma2(fr, make_float2(q0.y, q1.y), make_float2(p0.z, p1.z));
  } else {
    // exp(-x^2) = 2^(-r~^2) and erfc(x) (lengths in units of 1/s: the
    // exponent is the squared distance itself, with no rounded constant
    // that would shift every far pair's weight alike)
    const f2 ex = make_float2(ex2_approx(-r2.x), ex2_approx(-r2.y));
    const f2 den = fma2(r, b2(kHalfX), b2(1.f));
    const f2 tt = make_float2(rcp_approx(den.x), rcp_approx(den.y));
    f2 q = fma2(b2(kQ9), tt, b2(kQ8));
    q = fma2(q, tt, b2(kQ7));
    q = fma2(q, tt, b2(kQ6));
    q = fma2(q, tt, b2(kQ5));
    q = fma2(q, tt, b2(kQ4));
    q = fma2(q, tt, b2(kQ3));
    q = fma2(q, tt, b2(kQ2));
    q = fma2(q, tt, b2(kQ1));
    q = fma2(q, tt, b2(kQ0));
    // A~ = E (t Q(t) / r~ + g) / r~^2, B~ = (3 A~ + (2g/log2 e) E) / r~^2,
    // C~ = (4g/log2 e^2) E
    const f2 A = mul2(mul2(ex, fma2(mul2(tt, q), rinv, b2(kGq))), rinv2);
    const f2 B = mul2(fma2(b2(3.f), A, mul2(b2(kGB), ex)), rinv2);
    const f2 C = mul2(b2(kGC), ex);

    // the table's linear-interpolation error to second order, (ab/2) f''(r)
    // with a = r - r0, b = r1 - r (the third-order term is below 3e-7 of
    // each value at r >= 0.8 for alpha <= 0.55); in the step's units
    // 2 alpha^2 is kA2 and 2 alpha^2 C is kGC2 E
    const f2 uu = mul2(r, K.invLh);
    const f2 fr = sub2(uu, make_float2(floorf(uu.x), floorf(uu.y)));
    const f2 hh = mul2(fma2(neg2(fr), fr, fr), K.halfLh2);
    const f2 a2C = mul2(b2(kGC2), ex);
    Ac = fma2(hh, fma2(b2(4.f), B, C), A);
    Bc = fma2(hh, fma2(mul2(b2(6.f), fma2(b2(5.f), B, C)), rinv2, a2C), B);
    Cc = fma2(hh, mul2(a2C, fma2(b2(kA2), r2, b2(-1.f))), C);
    // near contact (r < kNearTab) the pair terms are largest, and the
    // rounding of the FP32 erfc chain (a few ulp, against one for a table
    // entry) would dominate the error of energy sums that cancel between
    // pairs: such pairs interpolate in the system's short table, as the
    // reference does.  A warp takes the lookups only when one of its pairs
    // is that close, and only those lanes load.  The short table holds A /
    // s^3, B / s^5, C / s^5 (the step's units); r / Lh is r~ / (s Lh).
    const bool nr0 = a0 && r.x < K.rnear, nr1 = a1 && r.y < K.rnear;
    if (K.tab != nullptr && __any_sync(0xffffffffu, nr0 || nr1)) {
      const f2 ut = fma2(r, K.ihh, mul2(r, K.ihl));
      const float fl0 = floorf(ut.x), fl1 = floorf(ut.y);
      const f2 ft = add2(fma2(r, K.ihh, make_float2(-fl0, -fl1)), mul2(r, K.ihl));
      const int e0 = min(max((int)fl0 - 1, 0), K.tn - 1), e1 = min(max((int)fl1 - 1, 0), K.tn - 1);
      if (nr0) {
        float4 p0, q0;
        ld_entry(K.tab + 2 * e0, p0, q0);
        Ac.x = fmaf(ft.x, p0.w, p0.x);
        Bc.x = fmaf(ft.x, q0.x, p0.y);
        Cc.x = fmaf(ft.x, q0.y, p0.z);
      }
      if (nr1) {
        float4 p1, q1;
        ld_entry(K.tab + 2 * e1, p1, q1);
        Ac.y = fmaf(ft.y, p1.w, p1.x);
        Bc.y = fmaf(ft.y, q1.x, p1.y);
        Cc.y = fmaf(ft.y, q1.y, p1.z);
      }
    }
  }

  // dipole-dipole energy, force on i, and the fields of the pair at each
  // other: the torque on a dipole is its moment crossed with the field
  // (v25/functions.cpp:1640-1661 without lever arms), so the fields are
  // summed and crossed once per tile
  const f2 mimj = fma2(miz, mjz, fma2(miy, mjy, mul2(mix, mjx)));
  const f2 mir = fma2(miz, dz, fma2(miy, dy, mul2(mix, dx)));
  const f2 mjr = fma2(mjz, dz, fma2(mjy, dy, mul2(mjx, dx)));
  const f2 pr = mul2(mir, mjr);
  const f2 u = fma2(neg2(pr), Bc, mul2(mimj, Ac));
  const f2 qq = mul2(pr, rinv2);
  const f2 fact = fma2(neg2(qq), Cc, mul2(fma2(b2(-5.f), qq, mimj), Bc));
  const f2 mirB = mul2(mir, Bc), mjrB = mul2(mjr, Bc);
  const f2 fx = fma2(fact, dx, fma2(mirB, mjx, mul2(mjrB, mix)));
  const f2 fy = fma2(fact, dy, fma2(mirB, mjy, mul2(mjrB, miy)));
  const f2 fz = fma2(fact, dz, fma2(mirB, mjz, mul2(mjrB, miz)));
  // field of j at i, (mj.r) B r - A mj, into the lane's sums; field of i at j
  const f2 nA = neg2(Ac);
  s.E[0] = fma2(nA, mjx, fma2(mjrB, dx, s.E[0]));
  s.E[1] = fma2(nA, mjy, fma2(mjrB, dy, s.E[1]));
  s.E[2] = fma2(nA, mjz, fma2(mjrB, dz, s.E[2]));
  o.ex = fma2(mirB, dx, mul2(nA, mix));
  o.ey = fma2(mirB, dy, mul2(nA, miy));
  o.ez = fma2(mirB, dz, mul2(nA, miz));

  s.F[0] = add2(s.F[0], fx);
  s.F[1] = add2(s.F[1], fy);
  s.F[2] = add2(s.F[2], fz);
  o.fx = fx;
  o.fy = fy;
  o.fz = fz;
  // Kahan: U += u
  const f2 yk = sub2(u, s.Uc);
  const f2 tk = add2(s.U, yk);
  s.Uc = sub2(sub2(tk, s.U), yk);
  s.U = tk;
  s.pt[0] = fma2(dx, fx, s.pt[0]);
  s.pt[1] = fma2(dx, fy, s.pt[1]);
  s.pt[2] = fma2(dx, fz, s.pt[2]);
  s.pt[3] = fma2(dy, fx, s.pt[3]);
  s.pt[4] = fma2(dy, fy, s.pt[4]);
  s.pt[5] = fma2(dy, fz, s.pt[5]);
  s.pt[6] = fma2(dz, fx, s.pt[6]);
  s.pt[7] = fma2(dz, fy, s.pt[7]);
  s.pt[8] = fma2(dz, fz, s.pt[8]);
}

// Off-diagonal tile (strips I < J): 64 steps, at step t lane l pairs both
// its i-dipoles with j = (l + t) mod 64; the two halves' j-side terms are
// added into that j's sums.
template <bool MASKED, bool MULTI, int MODE>
__device__ __forceinline__ void tile_loop(const PairConst& K, Lane2& s, const uint4* sj, const float4* smj,
                                          float4* sa4, float2* sa2, int lane, int jvalid) {
#pragma unroll 2
  for (int t = 0; t < kTile; ++t) {
    const int lj = (lane + t) & (kTile - 1);
    const uint4 jp = sj[lj];
    const float4 jm = smj[lj];
    bool a0 = true, a1 = true;
    if (MASKED) {
      const bool jv = lj < jvalid;
      a0 = s.ok0 && jv;
      a1 = s.ok1 && jv;
      if (MULTI) {
        a0 = a0 && (s.own0 != (int)jp.w);
        a1 = a1 && (s.own1 != (int)jp.w);
      }
    }
    JOut o;
    tile_step<MASKED, MODE>(K, s, jp, jm, jp, jm, a0, a1, o);
    float4 ja4 = sa4[lj];
    float2 ja2 = sa2[lj];
    ja4.x -= o.fx.x + o.fx.y;
    ja4.y -= o.fy.x + o.fy.y;
    ja4.z -= o.fz.x + o.fz.y;
    ja4.w += o.ex.x + o.ex.y;
    ja2.x += o.ey.x + o.ey.y;
    ja2.y += o.ez.x + o.ez.y;
    sa4[lj] = ja4;
    sa2[lj] = ja2;
    __syncwarp();
  }
}

// Diagonal tile (strip I with itself): every unordered pair of its 64
// dipoles once, in 32 steps.  At step t (1..32) i-dipole x = l (half 0) and
// x = l + 32 (half 1) pair with (x + t) mod 64: each pair at cyclic distance
// d < 32 is met once from its lower end, d > 32 once from its upper end,
// and d = 32 from half 0 only.  The 64 j's of a step are distinct.
template <bool MULTI, int MODE>
__device__ __forceinline__ void diag_loop(const PairConst& K, Lane2& s, const uint4* sj, const float4* smj,
                                          float4* sa4, float2* sa2, int lane, int jvalid) {
#pragma unroll 1
  for (int t = 1; t <= kTile / 2; ++t) {
    const int j0 = (lane + t) & (kTile - 1), j1 = (lane + 32 + t) & (kTile - 1);
    const uint4 jp0 = sj[j0], jp1 = sj[j1];
    const float4 jm0 = smj[j0], jm1 = smj[j1];
    bool a0 = s.ok0 && j0 < jvalid;
    bool a1 = s.ok1 && j1 < jvalid && t < kTile / 2;
    if (MULTI) {
      a0 = a0 && (s.own0 != (int)jp0.w);
      a1 = a1 && (s.own1 != (int)jp1.w);
    }
    JOut o;
    tile_step<true, MODE>(K, s, jp0, jm0, jp1, jm1, a0, a1, o);
    float4 ja4 = sa4[j0];
    float2 ja2 = sa2[j0];
    ja4.x -= o.fx.x;
    ja4.y -= o.fy.x;
    ja4.z -= o.fz.x;
    ja4.w += o.ex.x;
    ja2.x += o.ey.x;
    ja2.y += o.ez.x;
    sa4[j0] = ja4;
    sa2[j0] = ja2;
    ja4 = sa4[j1];
    ja2 = sa2[j1];
    ja4.x -= o.fx.y;
    ja4.y -= o.fy.y;
    ja4.z -= o.fz.y;
    ja4.w += o.ex.y;
    ja2.x += o.ey.y;
    ja2.y += o.ez.y;
    sa4[j1] = ja4;
    sa2[j1] = ja2;
    __syncwarp();
  }
}

}  // namespace

// per-system constants of the pair step: lengths in units of 1/s for the
// analytic form, in length units for the table forms
__device__ __forceinline__ PairConst pair_consts(const Batch& b, const SysDev& P, int mode, const float4* stab) {
  PairConst K;
  const bool an = (mode == kAnalytic);
  K.Lhx = b2(an ? P.Shi[0] : P.Lhi[0]);
  K.Llx = b2(an ? P.Slo[0] : P.Llo[0]);
  K.Lhy = b2(an ? P.Shi[1] : P.Lhi[1]);
  K.Lly = b2(an ? P.Slo[1] : P.Llo[1]);
  K.Lhz = b2(an ? P.Shi[2] : P.Lhi[2]);
  K.Llz = b2(an ? P.Slo[2] : P.Llo[2]);
  K.invLh = b2(P.sihh);
  K.halfLh2 = b2(P.shalfLh2);
  K.ihh = b2(an ? P.sihh : kInvLhHi);
  K.ihl = b2(an ? P.sihl : kInvLhLo);
  K.rnear = P.snear;
  K.tab = (mode == kTabGlobal || mode == kAnalytic) && b.rtab != nullptr && P.rt_n > 0
              ? b.rtab + 2 * (long long)P.rt_off
              : nullptr;
  K.stab = stab;
  K.tn = P.rt_n;
  return K;
}

// A tile's sum back to length units: the analytic form's forces by s^4 and
// its fields, torques, energy and pressure tensor by s^3 (float-float
// factors); the table forms' sums are in length units already.
template <int MODE>
__device__ __forceinline__ float to_len(float v, const float* sc) {
  if (MODE != kAnalytic) return v;
  return fmaf(v, sc[0], v * sc[1]);
}

// One tile (strips I <= J of one system) by one warp: the j-strip staged in
// the warp's shared arrays, the i-strip in registers, the pair loop, the
// partial slots and the tile's energy and pressure tensor.
template <bool MULTI, int MODE>
__device__ __forceinline__ void tile_work(const Batch& b, int tile, const PairConst& K, uint4* sj, float4* smj,
                                          float4* sa4, float2* sa2) {
  const int4 tl = b.tiles[tile];
  const SysDev& P = b.sys[tl.x];
  const int I = tl.y, J = tl.z;
  const bool diag = (I == J);
  const int lane = threadIdx.x & 31;
  const int ndip = P.ndip;
  const int ND = b.ndtot;

  for (int k = lane; k < kTile; k += 32) {
    const int jj = J * kTile + k;
    const bool v = jj < ndip;
    const int g = P.dip_off + (v ? jj : 0);
    sj[k] = make_uint4(b.dfx[g], b.dfx[ND + g], b.dfx[2 * ND + g], v ? (uint32_t)b.downer[g] : 0xffffffffu);
    smj[k] = v ? make_float4(b.dm[g], b.dm[ND + g], b.dm[2 * ND + g], 0.f) : make_float4(0.f, 0.f, 0.f, 0.f);
    sa4[k] = make_float4(0.f, 0.f, 0.f, 0.f);
    sa2[k] = make_float2(0.f, 0.f);
  }

  Lane2 s;
  {
    const int i0 = I * kTile + lane, i1 = i0 + 32;
    s.ok0 = i0 < ndip;
    s.ok1 = i1 < ndip;
    const int g0 = P.dip_off + (s.ok0 ? i0 : 0), g1 = P.dip_off + (s.ok1 ? i1 : 0);
    s.x0 = b.dfx[g0];
    s.y0 = b.dfx[ND + g0];
    s.z0 = b.dfx[2 * ND + g0];
    s.x1 = b.dfx[g1];
    s.y1 = b.dfx[ND + g1];
    s.z1 = b.dfx[2 * ND + g1];
    const float z0 = s.ok0 ? 1.f : 0.f, z1 = s.ok1 ? 1.f : 0.f;
    s.mx = make_float2(z0 * b.dm[g0], z1 * b.dm[g1]);
    s.my = make_float2(z0 * b.dm[ND + g0], z1 * b.dm[ND + g1]);
    s.mz = make_float2(z0 * b.dm[2 * ND + g0], z1 * b.dm[2 * ND + g1]);
    s.own0 = b.downer[g0];
    s.own1 = b.downer[g1];
#pragma unroll
    for (int c = 0; c < 3; ++c) s.F[c] = s.E[c] = b2(0.f);
#pragma unroll
    for (int c = 0; c < 9; ++c) s.pt[c] = b2(0.f);
    s.U = s.Uc = b2(0.f);
  }
  __syncwarp();

  const int jvalid = min(kTile, ndip - J * kTile);
  // no pair of this tile is skipped: the fast loop without masks
  const bool full = !MULTI && !diag && jvalid == kTile;
  if (diag)
    diag_loop<MULTI, MODE>(K, s, sj, smj, sa4, sa2, lane, jvalid);
  else if (full)
    tile_loop<false, MULTI, MODE>(K, s, sj, smj, sa4, sa2, lane, jvalid);
  else
    tile_loop<true, MULTI, MODE>(K, s, sj, smj, sa4, sa2, lane, jvalid);
  __syncwarp();
  // partial slots: (strip X, strip Y, component c, local index)
  const int ns = P.nstrip;
  float* base_ij = b.rpart + P.pp_off + ((long long)(I * ns + J) * 6) * kTile;
  float* base_ji = b.rpart + P.pp_off + ((long long)(J * ns + I) * 6) * kTile;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int li = lane + 32 * h;
    float fv[3], ev[3], tv[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      fv[c] = h ? s.F[c].y : s.F[c].x;
      ev[c] = h ? s.E[c].y : s.E[c].x;
    }
    if (diag) {
      const float4 a4 = sa4[li];
      const float2 a2 = sa2[li];
      fv[0] += a4.x;
      fv[1] += a4.y;
      fv[2] += a4.z;
      ev[0] += a4.w;
      ev[1] += a2.x;
      ev[2] += a2.y;
    }
    // torque without lever arm: moment x field
    const float mx = h ? s.mx.y : s.mx.x, my = h ? s.my.y : s.my.x, mz = h ? s.mz.y : s.mz.x;
    tv[0] = my * ev[2] - mz * ev[1];
    tv[1] = mz * ev[0] - mx * ev[2];
    tv[2] = mx * ev[1] - my * ev[0];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      base_ij[c * kTile + li] = to_len<MODE>(fv[c], P.sc4);
      base_ij[(3 + c) * kTile + li] = to_len<MODE>(tv[c], P.sc3);
    }
  }
  if (!diag) {
    for (int k = lane; k < kTile; k += 32) {
      const float4 a4 = sa4[k];
      const float2 a2 = sa2[k];
      const float4 mj = smj[k];
      base_ji[0 * kTile + k] = to_len<MODE>(a4.x, P.sc4);
      base_ji[1 * kTile + k] = to_len<MODE>(a4.y, P.sc4);
      base_ji[2 * kTile + k] = to_len<MODE>(a4.z, P.sc4);
      base_ji[3 * kTile + k] = to_len<MODE>(mj.y * a2.y - mj.z * a2.x, P.sc3);
      base_ji[4 * kTile + k] = to_len<MODE>(mj.z * a4.w - mj.x * a2.y, P.sc3);
      base_ji[5 * kTile + k] = to_len<MODE>(mj.x * a2.x - mj.y * a4.w, P.sc3);
    }
  }
  // tile energy and pressure tensor
  float red[10];
  red[0] = (s.U.x + (-s.Uc.x)) + (s.U.y + (-s.Uc.y));
#pragma unroll
  for (int c = 0; c < 9; ++c) red[1 + c] = s.pt[c].x + s.pt[c].y;
#pragma unroll
  for (int c = 0; c < 10; ++c) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) red[c] += __shfl_xor_sync(0xffffffffu, red[c], off);
  }
  if (lane == 0) {
#pragma unroll
    for (int c = 0; c < 10; ++c) b.tileE[(long long)tile * 10 + c] = to_len<MODE>(red[c], P.sc3);
  }
}

// W warps per block, one tile per warp (tile = W * blockIdx.x + warp, or
// the warp's entry of the list `gtile`): the block size changes how tiles
// are grouped for scheduling, never what a tile computes, so every W gives
// the same bits (the autotuner picks W).  MODE kAnalytic: the analytic
// terms with the table's interpolation error added (the default);
// kTabGlobal: interpolate in the reference's table in global memory.  20
// warps per SM hold the kernel to 96 registers (no spills in the analytic
// form, 12 B in the table form).  Measured on the 256-replica mix (CUDA
// events, one box): analytic 0.436 ms per launch at 20 warps per SM, 0.446
// at 16 (124 registers), 0.453 at 24 (80 registers, 120 B of spills); the
// table form 0.485 ms.
template <bool MULTI, int W, int MODE>
__global__ void __launch_bounds__(32 * W, 20 / W) real_pairs_kernel(Batch b, const int* gtile, int ntile) {
  __shared__ uint4 sj_all[W][kTile];    // fixed-point x, y, z and owner of the j-dipoles
  __shared__ float4 smj_all[W][kTile];  // their moments
  __shared__ float4 sa4_all[W][kTile];  // j-side sums: force x, y, z and field x
  __shared__ float2 sa2_all[W][kTile];  // field y, z
  const int wid = threadIdx.x >> 5;
  const int k = W * blockIdx.x + wid;
  if (k >= ntile) return;
  const int tile = gtile ? gtile[k] : k;
  if (at_limit(b, b.tiles[tile].x)) return;
  const SysDev& P = b.sys[b.tiles[tile].x];
  const PairConst K = pair_consts(b, P, MODE, nullptr);
  tile_work<MULTI, MODE>(b, tile, K, sj_all[wid], smj_all[wid], sa4_all[wid], sa2_all[wid]);
}

// Tiles of systems whose table fits a block's shared memory: a block takes
// a run of one system's tiles (rpwork: system, first tile, tiles), stages
// the system's interpolation table once -- A, B, C and A's difference per
// entry, 16 bytes, plus a copy of the last entry -- and its kSmemWarps
// warps take the run's tiles in turn.  A lookup is two 128-bit shared
// loads (entries k and k + 1, for the differences of B and C) instead of a
// scattered 256-bit global load: the table lookups no longer queue on the
// L1's tag stage behind misses to L2.  One block of kSmemWarps warps per SM.
template <bool MULTI>
__global__ void __launch_bounds__(32 * kSmemWarps, 1) real_pairs_smem_kernel(Batch b) {
  extern __shared__ float4 dyn[];
  const int4 wk = b.rpwork[blockIdx.x];
  if (at_limit(b, wk.x)) return;
  const SysDev& P = b.sys[wk.x];
  const int tn = P.rt_n;
  float4* stab = dyn;
  const float4* g = b.rtab + 2 * (long long)P.rt_off;
  // asynchronous 16-byte copies global -> shared, all in flight at once
  for (int e = threadIdx.x; e <= tn; e += blockDim.x) {
    const unsigned dst = (unsigned)__cvta_generic_to_shared(stab + e);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(g + 2 * min(e, tn - 1)) : "memory");
  }
  asm volatile("cp.async.wait_all;" ::: "memory");
  // per warp: 64 x (uint4 + float4 + float4) + 64 float2, after the table
  const int wid = threadIdx.x >> 5;
  float4* wbase = dyn + (tn + 1) + wid * (3 * kTile + kTile / 2);
  uint4* sj = reinterpret_cast<uint4*>(wbase);
  float4* smj = wbase + kTile;
  float4* sa4 = wbase + 2 * kTile;
  float2* sa2 = reinterpret_cast<float2*>(wbase + 3 * kTile);
  __syncthreads();
  const PairConst K = pair_consts(b, P, kTabShared, stab);
  for (int t = wk.y + wid; t < wk.y + wk.z; t += kSmemWarps)
    tile_work<MULTI, kTabShared>(b, t, K, sj, smj, sa4, sa2);
}

// The neighbour pass of the systems with a real-space cutoff, over the two
// lists one scan of list_build wrote for each rod.
//
// Real space (mode kNearReal): the reference's force_dipR with its table
// zeroed beyond rc_real, where pairs
// beyond rc_real + Lh add nothing, so only the rods on the system's
// real-space list are visited -- those whose centres are within rc_real +
// Lh + the dipoles' offsets + the skin (list_build).  A group of kCutLanes
// lanes per dipole i takes its partner dipoles -- the listed rods' dipoles,
// rods in ascending order -- two at a time through the tiles' pair step
// (both halves holding dipole i), lane j the pair steps j, j + kCutLanes,
// ...; a fixed shuffle tree adds the lanes' sums.  Only i's own force and
// torque are kept, so every pair is met from both ends and the energy and
// pressure tensor take half of each meeting.  No atomics: the same bits
// alone and in any batch.  Writes each dipole's force and torque where
// real_sum writes them, and its block's energy and pressure tensor
// (float-float block sums) for the per-system sum.
//
// WCA screen (mode kNearWca): in the same blocks, the first kPartBlock
// threads, a particle each, screen its Verlet list as the WCA screen kernel
// does for the other systems (wca_screen.cuh), feeding the same FP64
// evaluation.
constexpr int kCutLanes = 4;
enum : int { kNearReal = 1, kNearWca = 2 };

__global__ void __launch_bounds__(kPartBlock * kCutLanes) near_pass_kernel(Batch b, int mode) {
  __shared__ double sh[10 * kPartBlock * kCutLanes / 32];
  const int2 bk = b.blk[blockIdx.x];
  const SysDev& P = b.sys[bk.x];
  if (P.rc_real <= 0.0 || at_limit(b, bk.x)) return;  // the same for the whole block
  if ((mode & kNearWca) && threadIdx.x < kPartBlock) {  // whole warps
    const int i = bk.y + threadIdx.x;
    const bool ok = i < P.part_off + P.n;
    const int nl = ok ? b.nbc[i] : 0;
    const int* lst = b.nb + (long long)(ok ? i : bk.y) * kMaxNb;
    int k = 0;
    wca_screen_one(b, P, bk.x, i, ok, [&]() { return k < nl ? lst[k++] : -1; });
  }
  if (!(mode & kNearReal)) return;
  const int nd = P.nd;
  const int p0 = bk.y - P.part_off;
  const int np = min(kPartBlock, P.n - p0);
  const int ND = b.ndtot;
  const int lane = threadIdx.x % kCutLanes;
  const PairConst K = pair_consts(b, P, kTabGlobal, nullptr);
  FF e[10];
#pragma unroll
  for (int c = 0; c < 10; ++c) e[c] = ff_of(0.f);
  // a warp holds 32 / kCutLanes groups; every lane of a warp takes the same
  // trips (the shuffles need the whole warp), groups past the block's
  // dipoles with no partners
  const int wg = (threadIdx.x % 32) / kCutLanes;
  for (int base = (threadIdx.x / 32) * (32 / kCutLanes); base < np * nd; base += kPartBlock) {
    const bool act = base + wg < np * nd;
    const int loc = act ? base + wg : base;
    const int il = p0 * nd + loc;  // dipole within the system
    const int g = P.dip_off + il;
    const int ip = P.part_off + il / nd;
    Lane2 s;
    s.x0 = s.x1 = b.dfx[g];
    s.y0 = s.y1 = b.dfx[ND + g];
    s.z0 = s.z1 = b.dfx[2 * ND + g];
    s.mx = b2(b.dm[g]);
    s.my = b2(b.dm[ND + g]);
    s.mz = b2(b.dm[2 * ND + g]);
    s.own0 = s.own1 = ip;
    s.ok0 = s.ok1 = true;
#pragma unroll
    for (int c = 0; c < 3; ++c) s.F[c] = s.E[c] = b2(0.f);
#pragma unroll
    for (int c = 0; c < 9; ++c) s.pt[c] = b2(0.f);
    s.U = s.Uc = b2(0.f);
    const int* lst = b.rnb + (long long)ip * kMaxR;
    const int nj = act ? b.rnbc[ip] * nd : 0;
    for (int k = 2 * lane; k < nj; k += 2 * kCutLanes) {
      const bool two = k + 1 < nj;
      const int k1 = two ? k + 1 : k;
      const int ga = P.dip_off + (lst[k / nd] - P.part_off) * nd + k % nd;
      const int gb = P.dip_off + (lst[k1 / nd] - P.part_off) * nd + k1 % nd;
      const uint4 jpa = make_uint4(b.dfx[ga], b.dfx[ND + ga], b.dfx[2 * ND + ga], 0u);
      const uint4 jpb = make_uint4(b.dfx[gb], b.dfx[ND + gb], b.dfx[2 * ND + gb], 0u);
      const float4 jma = make_float4(b.dm[ga], b.dm[ND + ga], b.dm[2 * ND + ga], 0.f);
      const float4 jmb = make_float4(b.dm[gb], b.dm[ND + gb], b.dm[2 * ND + gb], 0.f);
      JOut o;
      tile_step<true, kTabGlobal>(K, s, jpa, jma, jpb, jmb, true, two, o);
    }
    // a lane's sums, then the group's (xor tree over the kCutLanes lanes)
    float v[17];
    {
      // both halves hold dipole i: its field, then the torque mi x field
      float ev[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        v[c] = s.F[c].x + s.F[c].y;
        ev[c] = s.E[c].x + s.E[c].y;
      }
      v[3] = s.my.x * ev[2] - s.mz.x * ev[1];
      v[4] = s.mz.x * ev[0] - s.mx.x * ev[2];
      v[5] = s.mx.x * ev[1] - s.my.x * ev[0];
    }
    v[6] = (s.U.x + (-s.Uc.x)) + (s.U.y + (-s.Uc.y));
#pragma unroll
    for (int c = 0; c < 9; ++c) v[7 + c] = s.pt[c].x + s.pt[c].y;
    float lo[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) lo[c] = 0.f;
#pragma unroll
    for (int off = kCutLanes / 2; off > 0; off >>= 1) {
#pragma unroll
      for (int c = 0; c < 16; ++c) {
        const float w = __shfl_xor_sync(0xffffffffu, v[c], off);
        if (c < 6) {  // forces and torques in float-float (TwoSum)
          const float wl = __shfl_xor_sync(0xffffffffu, lo[c], off);
          const float sum = v[c] + w;
          const float bb = sum - v[c];
          lo[c] += wl + ((v[c] - (sum - bb)) + (w - bb));
          v[c] = sum;
        } else {
          v[c] += w;
        }
      }
    }
    if (act && lane == 0) {
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        const float r = v[c] + lo[c];
        b.rsum[(long long)c * ND + g] = make_float2(r, lo[c] - (r - v[c]));
      }
      e[0] = ff_add(e[0], ff_of(0.5f * v[6]));
#pragma unroll
      for (int c = 0; c < 9; ++c) e[1 + c] = ff_add(e[1 + c], ff_of(0.5f * v[7 + c]));
    }
  }
  double out[10];
  block_sum<10, kPartBlock * kCutLanes>(e, sh, out);
  if (threadIdx.x == 0) {
    double* dst = b.rlE + (long long)blk_slot(P, bk) * 10;
#pragma unroll
    for (int c = 0; c < 10; ++c) dst[c] = out[c];
  }
}

// Each dipole's real-space force and torque: the sum of its tile partials
// over all partner strips, in strip order, in float-float.  One thread per
// (dipole, component) of a particle block, component-major so that a warp
// reads 32 consecutive dipoles of one component (coalesced) and the block
// has six times as many independent load streams as dipoles.
__global__ void __launch_bounds__(512) real_sum_kernel(Batch b) {
  const int2 bk = b.blk[blockIdx.x];
  const SysDev& P = b.sys[bk.x];
  if (P.rc_real > 0.0 || at_limit(b, bk.x)) return;  // cutoff systems: summed by their neighbour pass
  const int nd = P.nd;
  const int p0 = bk.y - P.part_off;
  const int np = min(kPartBlock, P.n - p0);
  const int nloc = np * nd, loc0 = p0 * nd;
  const int ns = P.nstrip;
  const int ND = b.ndtot;
  for (int it = threadIdx.x; it < 6 * nloc; it += blockDim.x) {
    const int c = it / nloc, loc = loc0 + (it - c * nloc);
    const int X = loc / kTile, lx = loc % kTile;
    const float* base = b.rpart + P.pp_off + (long long)X * ns * 6 * kTile + c * kTile + lx;
    float hi = 0.f, lo = 0.f;
#pragma unroll 8
    for (int Y = 0; Y < ns; ++Y) {
      // float-float accumulation (TwoSum)
      const float v = base[(long long)Y * 6 * kTile];
      const float sum = hi + v;
      const float bb = sum - hi;
      lo += (hi - (sum - bb)) + (v - bb);
      hi = sum;
    }
    const float r = hi + lo;
    b.rsum[(long long)c * ND + P.dip_off + loc] = make_float2(r, lo - (r - hi));
  }
}

// Energy rows of the strips of large systems (more than kStripRows strips):
// a warp per strip X sums the tile energies (U, PT) of the tiles (X, J >= X),
// lanes over J (J = X + lane, + 32, ...), float-float, then a shuffle tree
// -- lane 0's sums are in a fixed order.  The per-system sum then adds one
// row per strip instead of one per tile.
__global__ void __launch_bounds__(128) strip_energy_kernel(Batch b) {
  const int w = blockIdx.x * 4 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (w >= b.nbstrips) return;
  const int2 sx = b.bstrips[w];
  if (at_limit(b, sx.x)) return;
  const SysDev& P = b.sys[sx.x];
  const int X = sx.y, ns = P.nstrip;
  const long long t0 = P.tile_off + (long long)X * ns - (long long)X * (X - 1) / 2;
  FF acc[10];
#pragma unroll
  for (int c = 0; c < 10; ++c) acc[c] = ff_of(0.f);
  for (int J = X + lane; J < ns; J += 32) {
    const float* e = b.tileE + (t0 + (J - X)) * 10;
#pragma unroll
    for (int c = 0; c < 10; ++c) acc[c] = ff_add(acc[c], ff_of(e[c]));
  }
#pragma unroll
  for (int c = 0; c < 10; ++c) acc[c] = ff_warp_sum(acc[c]);
  if (lane == 0) {  // hi + lo in FP64 keeps the float-float value; the per-system sum splits it back
    double* out = b.stripE + (long long)(P.strip_off + X) * 10;
#pragma unroll
    for (int c = 0; c < 10; ++c) out[c] = soft_f2d(acc[c].hi) + soft_f2d(acc[c].lo);
  }
}

void launch_near_pass(const Batch& b, int mode, cudaStream_t s) {
  if (b.any_rc && b.nblk && mode) near_pass_kernel<<<b.nblk, kPartBlock * kCutLanes, 0, s>>>(b, mode);
}

void launch_real_sum(const Batch& b, cudaStream_t s) {
  if (b.ntiles == 0 || b.nblk == 0) return;
  real_sum_kernel<<<b.nblk, b.tune.rsum_threads, 0, s>>>(b);
  if (b.nbstrips) strip_energy_kernel<<<cdiv(b.nbstrips, 4), 128, 0, s>>>(b);
}

size_t real_pairs_smem_bytes(int tn) {
  return sizeof(float4) * ((size_t)tn + 1 + (size_t)kSmemWarps * (3 * kTile + kTile / 2));
}

// Once per device, outside any stream capture: the largest dynamic shared
// memory a shared-table tile launch may ask for.
cudaError_t prepare_real_pairs() {
  const int most = (int)real_pairs_smem_bytes(kSmemTableMax);
  cudaError_t e = cudaFuncSetAttribute(real_pairs_smem_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, most);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(real_pairs_smem_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, most);
  return e;
}

// one tile per warp over `list` (all tiles when null), W warps per block
template <int MODE>
void launch_tiles(const Batch& b, bool multi, int W, const int* list, int n, cudaStream_t s) {
  const int grid = cdiv(n, W);
  if (W == 4) {
    if (multi) real_pairs_kernel<true, 4, MODE><<<grid, 128, 0, s>>>(b, list, n);
    else real_pairs_kernel<false, 4, MODE><<<grid, 128, 0, s>>>(b, list, n);
  } else if (W == 2) {
    if (multi) real_pairs_kernel<true, 2, MODE><<<grid, 64, 0, s>>>(b, list, n);
    else real_pairs_kernel<false, 2, MODE><<<grid, 64, 0, s>>>(b, list, n);
  } else {
    if (multi) real_pairs_kernel<true, 1, MODE><<<n, 32, 0, s>>>(b, list, n);
    else real_pairs_kernel<false, 1, MODE><<<n, 32, 0, s>>>(b, list, n);
  }
}

void launch_real_pairs(const Batch& b, bool multi, cudaStream_t s) {
  if (b.ntiles == 0) return;
  if (b.rtab == nullptr) {  // no table (callers without one): the analytic form, one tile per block
    launch_tiles<kAnalytic>(b, multi, 1, nullptr, b.ntiles, s);
    return;
  }
  if (b.nrpwork) {
    const size_t bytes = real_pairs_smem_bytes(b.smem_tn);
    if (multi) real_pairs_smem_kernel<true><<<b.nrpwork, 32 * kSmemWarps, bytes, s>>>(b);
    else real_pairs_smem_kernel<false><<<b.nrpwork, 32 * kSmemWarps, bytes, s>>>(b);
  }
  if (b.ngtile == 0) return;
  if (b.rp_table) launch_tiles<kTabGlobal>(b, multi, b.tune.rp_warps, b.gtile, b.ngtile, s);
  else launch_tiles<kAnalytic>(b, multi, b.tune.rp_warps, b.gtile, b.ngtile, s);
}

}  // namespace mdsc
