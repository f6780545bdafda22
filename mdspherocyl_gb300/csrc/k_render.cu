// Headless picture of a system -- the GPU replacement of the reference's
// SDL/OpenGL viewer (v25/graphic.cpp), which needs a display and a GL stack.
// The scene is the viewer's (v25/graphic.cpp:183-330,612-680):
//   * each rod a spherocylinder of its length and diameter, grey by species
//     (tone_list), with a blue tip on the +axis cap (latitude sin > 0.8) and
//     red and green meridians on the cylinder marking the body x and y axes;
//   * each dipole a pair of segments through its position, blue behind and
//     red ahead, 1.5 radii long each;
//   * the box edges in (0.6, 0.3, 0.3), around [-L/2, L/2]^3;
//   * optionally the 26 periodic images, optionally one cluster only;
//   * white background, the viewer's camera: gluLookAt from
//     usr = dist (sin t cos p, sin t sin p, cos t) to ref with z up, then
//     moved back |usr| along the view (computeLocation, :405-415), a
//     60-degree vertical field; ambient 0.5 plus a directional light of 0.7
//     from usr (:612-624).
// Lines of the viewer (dipoles 2 pixels wide, box edges 1) become capsules
// of that width at the distance looked at.
// It is ray cast instead of rasterised: one thread per pixel, every ray
// tested against every capsule (rods, dipole segments, box edges), the
// capsules staged through shared memory 128 at a time.  Output: 8-bit RGB,
// rows from the top.
#include "mdsc_dev.cuh"

namespace mdsc {

// a capsule of the scene: segment a..b, radius, shading data
struct Capsule {
  float ax, ay, az, bx, by, bz;
  float rad;
  float ex, ey, ez;     // body x axis (rods), for the meridians
  float tone;           // grey of the species (rods); < 0: flat colour r, g, b below
  float cr, cg, cb;     // flat colour (segments)
  int kind;             // 0 rod, 1 segment
};

struct RenderView {
  int width, height;
  float eye[3], fwd[3], right[3], up[3];
  float tan_half;   // tan(fov / 2)
  float light[3];   // unit vector towards the light
};

__constant__ float kTone[5] = {1.f, 0.4f, 0.6f, 0.2f, 0.8f};

// per particle: its rod (and its periodic images) and its dipoles' segments
__global__ void scene_kernel(Batch b, int sys, const unsigned char* __restrict__ species,
                             const int* __restrict__ keep, int images, int dipoles, float seg_rad,
                             Capsule* __restrict__ rods, Capsule* __restrict__ segs, int* __restrict__ counts) {
  const SysDev& P = b.sys[sys];
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= P.n) return;
  if (keep && !keep[k]) return;
  const int i = P.part_off + k;
  const double* O = b.O + 9 * i;
  const double* r = b.r + 3 * i;
  const float h = (float)(0.5 * b.len[i]), rad = (float)(0.5 * b.dia[i]);
  const float u[3] = {(float)O[6], (float)O[7], (float)O[8]};
  const int nimg = images ? 27 : 1;
  const int ri = atomicAdd(&counts[0], nimg);
  const int nd = dipoles ? P.nd : 0;
  const int si = atomicAdd(&counts[1], 2 * nd * nimg);
  for (int m = 0; m < nimg; ++m) {
    const float sh[3] = {images ? (float)(P.L[0] * (m % 3 - 1)) : 0.f,
                         images ? (float)(P.L[1] * ((m / 3) % 3 - 1)) : 0.f,
                         images ? (float)(P.L[2] * (m / 9 - 1)) : 0.f};
    const float c[3] = {(float)r[0] + sh[0], (float)r[1] + sh[1], (float)r[2] + sh[2]};
    Capsule q;
    q.ax = c[0] - h * u[0];
    q.ay = c[1] - h * u[1];
    q.az = c[2] - h * u[2];
    q.bx = c[0] + h * u[0];
    q.by = c[1] + h * u[1];
    q.bz = c[2] + h * u[2];
    q.rad = rad;
    q.ex = (float)O[0];
    q.ey = (float)O[1];
    q.ez = (float)O[2];
    q.tone = kTone[species[k] % 5];
    q.cr = q.cg = q.cb = 0.f;
    q.kind = 0;
    rods[ri + m] = q;
    // dipoles: lab position r + offset * axis, direction O^T o_body
    for (int w = 0; w < nd; ++w) {
      const int g = P.dip_off + k * nd + w;
      if (b.dmu[g] == 0.0) {
        // a padding dipole: an empty segment
        for (int s = 0; s < 2; ++s) {
          Capsule z{};
          z.rad = 0.f;
          z.kind = 1;
          z.tone = -1.f;
          segs[si + 2 * (m * nd + w) + s] = z;
        }
        continue;
      }
      const double pc = b.dpc[g];
      const float p[3] = {c[0] + (float)(pc * O[6]), c[1] + (float)(pc * O[7]), c[2] + (float)(pc * O[8])};
      const double ox = b.dob[3 * g], oy = b.dob[3 * g + 1], oz = b.dob[3 * g + 2];
      const float d[3] = {(float)(O[0] * ox + O[3] * oy + O[6] * oz), (float)(O[1] * ox + O[4] * oy + O[7] * oz),
                          (float)(O[2] * ox + O[5] * oy + O[8] * oz)};
      const float mlt = 1.5f * rad, thick = seg_rad;
      for (int s = 0; s < 2; ++s) {
        Capsule z;
        const float s0 = s == 0 ? -mlt : 0.f, s1 = s == 0 ? 0.f : mlt;
        z.ax = p[0] + s0 * d[0];
        z.ay = p[1] + s0 * d[1];
        z.az = p[2] + s0 * d[2];
        z.bx = p[0] + s1 * d[0];
        z.by = p[1] + s1 * d[1];
        z.bz = p[2] + s1 * d[2];
        z.rad = thick;
        z.ex = z.ey = z.ez = 0.f;
        z.tone = -1.f;
        z.cr = s == 0 ? 0.f : 1.f;
        z.cg = 0.f;
        z.cb = s == 0 ? 1.f : 0.f;
        z.kind = 1;
        segs[si + 2 * (m * nd + w) + s] = z;
      }
    }
  }
}

// distance along the unit ray o + t d to the capsule surface, or -1
__device__ __forceinline__ float hit_capsule(const float o[3], const float d[3], const Capsule& c) {
  if (c.rad <= 0.f) return -1.f;
  const float ba[3] = {c.bx - c.ax, c.by - c.ay, c.bz - c.az};
  const float oa[3] = {o[0] - c.ax, o[1] - c.ay, o[2] - c.az};
  const float baba = ba[0] * ba[0] + ba[1] * ba[1] + ba[2] * ba[2];
  const float bard = ba[0] * d[0] + ba[1] * d[1] + ba[2] * d[2];
  const float baoa = ba[0] * oa[0] + ba[1] * oa[1] + ba[2] * oa[2];
  const float rdoa = d[0] * oa[0] + d[1] * oa[1] + d[2] * oa[2];
  const float oaoa = oa[0] * oa[0] + oa[1] * oa[1] + oa[2] * oa[2];
  const float r2 = c.rad * c.rad;
  // the cylinder: |(oa + t d) - ((oa + t d).ba / baba) ba|^2 = r^2, a quadratic in t
  const float qa = baba - bard * bard;
  const float qb = baba * rdoa - baoa * bard;
  const float qc = baba * oaoa - baoa * baoa - r2 * baba;
  if (qa > 1e-12f * baba) {
    const float disc = qb * qb - qa * qc;
    if (disc >= 0.f) {
      const float t = (-qb - sqrtf(disc)) / qa;
      const float y = baoa + t * bard;  // along the axis, 0..baba on the body
      if (t > 0.f && y > 0.f && y < baba) return t;
    }
  }
  // the end spheres: the nearer of the two intersections
  float best = -1.f;
#pragma unroll
  for (int e = 0; e < 2; ++e) {
    const float oc[3] = {e ? o[0] - c.bx : oa[0], e ? o[1] - c.by : oa[1], e ? o[2] - c.bz : oa[2]};
    const float hb = d[0] * oc[0] + d[1] * oc[1] + d[2] * oc[2];
    const float hc = oc[0] * oc[0] + oc[1] * oc[1] + oc[2] * oc[2] - r2;
    const float disc = hb * hb - hc;
    if (disc >= 0.f) {
      const float t = -hb - sqrtf(disc);
      if (t > 0.f && (best < 0.f || t < best)) best = t;
    }
  }
  return best;
}

constexpr int kRenderTile = 128;

__global__ void __launch_bounds__(kRenderTile) render_kernel(RenderView v, const Capsule* __restrict__ rods,
                                                             const Capsule* __restrict__ segs,
                                                             const int* __restrict__ counts,
                                                             unsigned char* __restrict__ rgb) {
  __shared__ Capsule sc[kRenderTile];
  const int px = blockIdx.x * 16 + (threadIdx.x & 15);
  const int py = blockIdx.y * 8 + (threadIdx.x >> 4);
  const bool on = px < v.width && py < v.height;
  // the ray through the pixel centre
  const float aspect = (float)v.width / (float)v.height;
  const float sx = (2.f * (px + 0.5f) / v.width - 1.f) * v.tan_half * aspect;
  const float sy = (1.f - 2.f * (py + 0.5f) / v.height) * v.tan_half;
  float d[3];
  float nrm = 0.f;
  for (int a = 0; a < 3; ++a) {
    d[a] = v.fwd[a] + sx * v.right[a] + sy * v.up[a];
    nrm += d[a] * d[a];
  }
  nrm = rsqrtf(nrm);
  for (int a = 0; a < 3; ++a) d[a] *= nrm;
  float tmin = 3.0e38f;
  Capsule hit{};
  bool any = false;
  for (int list = 0; list < 2; ++list) {
    const Capsule* src = list ? segs : rods;
    const int n = counts[list];
    for (int c0 = 0; c0 < n; c0 += kRenderTile) {
      __syncthreads();
      if (c0 + (int)threadIdx.x < n) sc[threadIdx.x] = src[c0 + threadIdx.x];
      __syncthreads();
      const int m = min(kRenderTile, n - c0);
      if (!on) continue;
      for (int k = 0; k < m; ++k) {
        const float t = hit_capsule(v.eye, d, sc[k]);
        if (t > 0.f && t < tmin) {
          tmin = t;
          hit = sc[k];
          any = true;
        }
      }
    }
  }
  if (!on) return;
  float col[3] = {1.f, 1.f, 1.f};  // the background
  if (any) {
    const float p[3] = {v.eye[0] + tmin * d[0], v.eye[1] + tmin * d[1], v.eye[2] + tmin * d[2]};
    if (hit.kind == 1) {
      col[0] = hit.cr;
      col[1] = hit.cg;
      col[2] = hit.cb;
    } else {
      // the nearest point of the axis segment gives the normal
      const float ba[3] = {hit.bx - hit.ax, hit.by - hit.ay, hit.bz - hit.az};
      const float len2 = ba[0] * ba[0] + ba[1] * ba[1] + ba[2] * ba[2];
      const float pa[3] = {p[0] - hit.ax, p[1] - hit.ay, p[2] - hit.az};
      float s = len2 > 0.f ? (pa[0] * ba[0] + pa[1] * ba[1] + pa[2] * ba[2]) / len2 : 0.f;
      s = fminf(fmaxf(s, 0.f), 1.f);
      float nv[3];
      for (int a = 0; a < 3; ++a) nv[a] = (pa[a] - s * ba[a]) / hit.rad;
      const float il = len2 > 0.f ? rsqrtf(len2) : 0.f;
      const float u[3] = {ba[0] * il, ba[1] * il, ba[2] * il};
      float base[3] = {hit.tone, hit.tone, hit.tone};
      if (s >= 1.f) {
        // the +axis cap: blue above latitude sin = 0.8
        const float z = nv[0] * u[0] + nv[1] * u[1] + nv[2] * u[2];
        if (z > 0.8f) base[0] = base[1] = 0.f, base[2] = 1.f;
      } else if (s > 0.f) {
        // the cylinder: red and green meridians at the body x and y axes,
        // fading over one facet of the viewer's 12 (30 degrees) on each side
        const float ey[3] = {u[1] * hit.ez - u[2] * hit.ey, u[2] * hit.ex - u[0] * hit.ez,
                             u[0] * hit.ey - u[1] * hit.ex};
        const float cx = nv[0] * hit.ex + nv[1] * hit.ey + nv[2] * hit.ez;
        const float cy = nv[0] * ey[0] + nv[1] * ey[1] + nv[2] * ey[2];
        const float phi = atan2f(cy, cx);
        const float facet = 3.14159265f / 6.f;
        const float wr = fmaxf(0.f, 1.f - fabsf(phi) / facet);
        const float wg = fmaxf(0.f, 1.f - fabsf(phi - 1.57079633f) / facet);
        const float wt = 1.f - wr - wg;
        base[0] = wt * hit.tone + wr;
        base[1] = wt * hit.tone + wg;
        base[2] = wt * hit.tone;
      }
      const float lam = fmaxf(0.f, nv[0] * v.light[0] + nv[1] * v.light[1] + nv[2] * v.light[2]);
      const float shade = 0.5f + 0.7f * lam;
      for (int a = 0; a < 3; ++a) col[a] = fminf(1.f, base[a] * shade);
    }
  }
  const size_t o = 3 * ((size_t)py * v.width + px);
  for (int a = 0; a < 3; ++a) rgb[o + a] = (unsigned char)__float2int_rn(255.f * fminf(fmaxf(col[a], 0.f), 1.f));
}

// the box's 12 edges as flat segments
__global__ void box_kernel(Batch b, int sys, float thick, Capsule* __restrict__ segs, int* __restrict__ counts) {
  const int e = threadIdx.x;
  if (e >= 12) return;
  const SysDev& P = b.sys[sys];
  const float h[3] = {(float)(0.5 * P.L[0]), (float)(0.5 * P.L[1]), (float)(0.5 * P.L[2])};
  const int axis = e / 4, corner = e % 4;
  float a[3], c[3];
  const int o1 = (axis + 1) % 3, o2 = (axis + 2) % 3;
  a[axis] = -h[axis];
  c[axis] = h[axis];
  a[o1] = c[o1] = (corner & 1) ? h[o1] : -h[o1];
  a[o2] = c[o2] = (corner & 2) ? h[o2] : -h[o2];
  const int base = atomicAdd(&counts[1], 0);  // the dipole segments are written first
  Capsule z;
  z.ax = a[0];
  z.ay = a[1];
  z.az = a[2];
  z.bx = c[0];
  z.by = c[1];
  z.bz = c[2];
  z.rad = thick;
  z.ex = z.ey = z.ez = 0.f;
  z.tone = -1.f;
  z.cr = 0.6f;
  z.cg = 0.3f;
  z.cb = 0.3f;
  z.kind = 1;
  segs[base + e] = z;
  __syncthreads();
  if (e == 0) counts[1] = base + 12;
}

size_t render_scratch_bytes(int n, int nd, int images) {
  const size_t nimg = images ? 27 : 1;
  return sizeof(Capsule) * ((size_t)n * nimg + (size_t)2 * n * nd * nimg + 12) + 64;
}

// scratch: render_scratch_bytes(n, nd, images) bytes of device memory;
// eye, fwd, right, up: the camera frame; light: unit vector to the light;
// seg_rad, box_rad: radii of the dipole and box-edge capsules
void launch_render(const Batch& b, int sys, int n, const unsigned char* species, const int* keep, int images,
                   int dipoles, int draw_box, float seg_rad, float box_rad, const float* eye, const float* fwd,
                   const float* right, const float* up, const float* light, float tan_half, int width,
                   int height, void* scratch, unsigned char* rgb, cudaStream_t s) {
  char* base = static_cast<char*>(scratch);
  int* counts = reinterpret_cast<int*>(base);
  Capsule* rods = reinterpret_cast<Capsule*>(base + 64);
  const size_t nimg = images ? 27 : 1;
  Capsule* segs = rods + (size_t)n * nimg;
  cudaMemsetAsync(counts, 0, 64, s);
  if (n > 0)
    scene_kernel<<<cdiv(n, 128), 128, 0, s>>>(b, sys, species, keep, images, dipoles, seg_rad, rods, segs, counts);
  if (draw_box) box_kernel<<<1, 32, 0, s>>>(b, sys, box_rad, segs, counts);
  RenderView v;
  v.width = width;
  v.height = height;
  for (int a = 0; a < 3; ++a) {
    v.eye[a] = eye[a];
    v.fwd[a] = fwd[a];
    v.right[a] = right[a];
    v.up[a] = up[a];
    v.light[a] = light[a];
  }
  v.tan_half = tan_half;
  dim3 grid(cdiv(width, 16), cdiv(height, 8));
  render_kernel<<<grid, kRenderTile, 0, s>>>(v, rods, segs, counts, rgb);
}

}  // namespace mdsc
