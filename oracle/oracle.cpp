// CPU oracle: restatement of the anari-visionaray CPU device's per-pixel hot
// path (raycast + pathtrace renderers, volume marching, delta tracking, frame
// accumulation).
//
// TEST INFRASTRUCTURE ONLY: the checker for the CUDA product path, and the
// timed CPU baseline. The product never links this file.
//
// Citations are file:line in the reference project. Arithmetic follows the
// reference's order; helpers that live in the (un-vendored) Visionaray
// library are restated in oracle_math.h with their conventions named.
#include "vsr_oracle.h"
#include "oracle_math.h"

#include <atomic>
#include <cstring>
#include <memory>
#include <thread>
#include <vector>

using namespace orc;

namespace {

struct Ray {
  f3 ori, dir;
  float tmin, tmax, time;
};

// ---------------------------------------------------------------------------
// Affine transforms (scene/Instance.cpp:92-98: affineInv = inverse(top_left),
// transInv = -translation, normalXfm = transpose(affineInv)).
// ---------------------------------------------------------------------------
struct M3 {
  f3 c0, c1, c2; // columns
  f3 operator*(f3 v) const { return c0 * v.x + c1 * v.y + c2 * v.z; }
};

M3 inverse3(const M3 &m) {
  f3 a = m.c0, b = m.c1, c = m.c2;
  f3 r0 = cross(b, c), r1 = cross(c, a), r2 = cross(a, b);
  float det = dot(a, r0);
  float id = 1.f / det;
  // rows of the inverse are r0/det, r1/det, r2/det
  M3 inv;
  inv.c0 = f3(r0.x, r1.x, r2.x) * id;
  inv.c1 = f3(r0.y, r1.y, r2.y) * id;
  inv.c2 = f3(r0.z, r1.z, r2.z) * id;
  return inv;
}

M3 transpose3(const M3 &m) {
  M3 t;
  t.c0 = f3(m.c0.x, m.c1.x, m.c2.x);
  t.c1 = f3(m.c0.y, m.c1.y, m.c2.y);
  t.c2 = f3(m.c0.z, m.c1.z, m.c2.z);
  return t;
}

struct Inst {
  M3 affineInv, normalXfm;
  f3 transInv;
  int group;
  uint32_t userID;
  Ray toLocal(const Ray &r) const {
    Ray l = r;
    l.ori = affineInv * (r.ori + transInv);
    l.dir = affineInv * r.dir;
    return l;
  }
};

// ---------------------------------------------------------------------------
// Triangles (basic_triangle v1/e1/e2, scene/surface/geometry/Triangle.cpp:76-83)
// and a binned-SAH BVH2 per group. The BVH shape only affects speed: closest
// hits are resolved by (t, instance, triangle) so any valid BVH gives the same
// answer.
// ---------------------------------------------------------------------------
struct Tri { f3 v1, e1, e2; };

struct Box {
  f3 lo{FLT_MAX}, hi{-FLT_MAX};
  void grow(f3 p) { lo = min3(lo, p); hi = max3(hi, p); }
  void grow(const Box &b) { lo = min3(lo, b.lo); hi = max3(hi, b.hi); }
  float area() const {
    f3 d = hi - lo;
    if (d.x < 0) return 0.f;
    return 2.f * (d.x * d.y + d.y * d.z + d.z * d.x);
  }
};

struct BNode {
  Box box;
  int32_t first; // leaf: first index into prim; inner: left child (right = first+1)
  int32_t count; // >0 leaf
};

struct GroupBVH {
  std::vector<BNode> nodes;
  std::vector<int32_t> prim; // global triangle ids
};

void buildBVH(GroupBVH &bvh, const std::vector<Tri> &tris, int begin, int end) {
  int n = end - begin;
  bvh.nodes.clear();
  bvh.prim.resize(n);
  if (n <= 0) return;
  std::vector<Box> pb(n);
  std::vector<f3> pc(n);
  for (int i = 0; i < n; ++i) {
    const Tri &t = tris[begin + i];
    Box b;
    b.grow(t.v1);
    b.grow(t.v1 + t.e1);
    b.grow(t.v1 + t.e2);
    pb[i] = b;
    pc[i] = (b.lo + b.hi) * 0.5f;
    bvh.prim[i] = begin + i;
  }
  std::vector<int32_t> idx(n);
  for (int i = 0; i < n; ++i) idx[i] = i;
  bvh.nodes.reserve(2 * n);
  bvh.nodes.push_back(BNode{});
  struct Task { int node, lo, hi; };
  std::vector<Task> stack{{0, 0, n}};
  const int kBins = 16;
  while (!stack.empty()) {
    Task tk = stack.back();
    stack.pop_back();
    Box nb, cb;
    for (int i = tk.lo; i < tk.hi; ++i) { nb.grow(pb[idx[i]]); cb.grow(pc[idx[i]]); }
    int cnt = tk.hi - tk.lo;
    bvh.nodes[tk.node].box = nb;
    if (cnt <= 4) {
      bvh.nodes[tk.node].first = tk.lo;
      bvh.nodes[tk.node].count = cnt;
      continue;
    }
    int bestAxis = -1, bestSplit = -1;
    float bestCost = FLT_MAX;
    for (int axis = 0; axis < 3; ++axis) {
      float clo = cb.lo[axis], chi = cb.hi[axis];
      if (!(chi > clo)) continue;
      Box bins[kBins];
      int bc[kBins] = {0};
      float scale = kBins / (chi - clo);
      for (int i = tk.lo; i < tk.hi; ++i) {
        int b = std::min(kBins - 1, (int)((pc[idx[i]][axis] - clo) * scale));
        bins[b].grow(pb[idx[i]]);
        bc[b]++;
      }
      Box rb[kBins];
      int rc[kBins];
      Box acc;
      int ac = 0;
      for (int b = kBins - 1; b > 0; --b) {
        acc.grow(bins[b]);
        ac += bc[b];
        rb[b] = acc;
        rc[b] = ac;
      }
      Box lb;
      int lc = 0;
      for (int b = 0; b < kBins - 1; ++b) {
        lb.grow(bins[b]);
        lc += bc[b];
        if (lc == 0 || rc[b + 1] == 0) continue;
        float cost = lb.area() * lc + rb[b + 1].area() * rc[b + 1];
        if (cost < bestCost) { bestCost = cost; bestAxis = axis; bestSplit = b; }
      }
    }
    int mid;
    if (bestAxis < 0) {
      mid = tk.lo + cnt / 2;
    } else {
      float clo = cb.lo[bestAxis], chi = cb.hi[bestAxis];
      float scale = kBins / (chi - clo);
      int *l = &idx[tk.lo], *r = &idx[tk.hi - 1];
      while (l <= r) {
        int b = std::min(kBins - 1, (int)((pc[*l][bestAxis] - clo) * scale));
        if (b <= bestSplit) ++l;
        else { std::swap(*l, *r); --r; }
      }
      mid = (int)(l - &idx[0]);
      if (mid == tk.lo || mid == tk.hi) mid = tk.lo + cnt / 2;
    }
    int left = (int)bvh.nodes.size();
    bvh.nodes.push_back(BNode{});
    bvh.nodes.push_back(BNode{});
    bvh.nodes[tk.node].first = left;
    bvh.nodes[tk.node].count = 0;
    stack.push_back({left, tk.lo, mid});
    stack.push_back({left + 1, mid, tk.hi});
  }
  std::vector<int32_t> p2(n);
  for (int i = 0; i < n; ++i) p2[i] = begin + idx[i];
  bvh.prim.swap(p2);
}

// ---------------------------------------------------------------------------
// Volumes: structuredRegular field + transferFunction1D.
// ---------------------------------------------------------------------------
struct Vol {
  const OrVolume *v;
  Box bounds;           // StructuredRegularField.cpp:90-93
  f3 S, T;              // voxel space: S * (P + T), StructuredRegularField.cpp:37-39
  float cellSize;       // min(spacing), :40
  int gdims[3] = {0, 0, 0};
  std::vector<float> maxOpacity;
  f3 pointToVoxelSpace(f3 p) const { return S * (p + T); }
  f3 vectorToVoxelSpace(f3 d) const { return S * d; }
};

// tex3D with normalized coordinates, linear filter, clamp addressing; texel
// i is centred at (i+0.5)/N (sampleField, DeviceCopyableObjects.h:478-481).
float sampleField(const OrVolume *v, f3 P) {
  const int nx = v->dims[0], ny = v->dims[1], nz = v->dims[2];
  float x = P.x * nx - 0.5f, y = P.y * ny - 0.5f, z = P.z * nz - 0.5f;
  float fx0 = std::floor(x), fy0 = std::floor(y), fz0 = std::floor(z);
  float fx = x - fx0, fy = y - fy0, fz = z - fz0;
  auto cl = [](float f, int n) {
    return f < 0.f ? 0 : (f > (float)(n - 1) ? n - 1 : (int)f);
  };
  int x0 = cl(fx0, nx), x1 = cl(fx0 + 1.f, nx);
  int y0 = cl(fy0, ny), y1 = cl(fy0 + 1.f, ny);
  int z0 = cl(fz0, nz), z1 = cl(fz0 + 1.f, nz);
  const float *d = v->data;
  auto at = [&](int i, int j, int k) { return d[(size_t(k) * ny + j) * nx + i]; };
  float c00 = lerpf(at(x0, y0, z0), at(x1, y0, z0), fx);
  float c10 = lerpf(at(x0, y1, z0), at(x1, y1, z0), fx);
  float c01 = lerpf(at(x0, y0, z1), at(x1, y0, z1), fx);
  float c11 = lerpf(at(x0, y1, z1), at(x1, y1, z1), fx);
  float c0 = lerpf(c00, c10, fy);
  float c1 = lerpf(c01, c11, fy);
  return lerpf(c0, c1, fz);
}

// tex1D over the TF table, normalized coordinates, linear, clamp.
f4 tfTex(const OrVolume *v, float u) {
  const int n = v->tfSize;
  float x = u * n - 0.5f;
  float f0 = std::floor(x);
  float f = x - f0;
  int i0 = f0 < 0.f ? 0 : (f0 > (float)(n - 1) ? n - 1 : (int)f0);
  int i1 = (f0 + 1.f) < 0.f ? 0 : ((f0 + 1.f) > (float)(n - 1) ? n - 1 : (int)(f0 + 1.f));
  const float *a = v->tf + 4 * i0, *b = v->tf + 4 * i1;
  return f4(lerpf(a[0], b[0], f), lerpf(a[1], b[1], f), lerpf(a[2], b[2], f), lerpf(a[3], b[3], f));
}

// postClassify, DeviceCopyableObjects.h:614-619.
f4 postClassify(const OrVolume *v, float val) {
  val = (val - v->valueRange[0]) / (v->valueRange[1] - v->valueRange[0]);
  return tfTex(v, val);
}

// projectOnGrid / linearIndex, GridAccel-common.h:9-25.
void projectOnGrid(f3 V, const int *dims, const Box &wb, int *out) {
  f3 V01 = (V - wb.lo) / (wb.hi - wb.lo);
  for (int a = 0; a < 3; ++a) {
    int c = (int)(V01[a] * (float)dims[a]);
    out[a] = std::min(std::max(c, 0), dims[a] - 1);
  }
}

void buildMajorants(Vol &vol) {
  const OrVolume *v = vol.v;
  if (v->gridMethod == OR_GRID_REFERENCE) {
    // StructuredRegularField::buildGrid (:95-127) + rasterizeBox
    // (GridAccel.h:51-68) + computeMaxOpacities (GridAccel.cpp:69-108).
    for (int a = 0; a < 3; ++a) vol.gdims[a] = v->gridDims[a];
    size_t nc = size_t(vol.gdims[0]) * vol.gdims[1] * vol.gdims[2];
    std::vector<float> vmin(nc, FLT_MAX), vmax(nc, -FLT_MAX);
    f3 org(v->origin[0], v->origin[1], v->origin[2]);
    f3 sp(v->spacing[0], v->spacing[1], v->spacing[2]);
    for (int z = 0; z < v->dims[2]; ++z)
      for (int y = 0; y < v->dims[1]; ++y)
        for (int x = 0; x < v->dims[0]; ++x) {
          f3 xyz((float)x, (float)y, (float)z);
          f3 P = org + xyz * sp;
          float value = sampleField(v, vol.pointToVoxelSpace(P));
          Box cell;
          cell.lo = org + xyz * sp;
          cell.hi = org + (xyz + f3(1.f)) * sp;
          int lo[3], hi[3];
          projectOnGrid(cell.lo, vol.gdims, vol.bounds, lo);
          projectOnGrid(cell.hi, vol.gdims, vol.bounds, hi);
          for (int mz = lo[2]; mz <= hi[2]; ++mz)
            for (int my = lo[1]; my <= hi[1]; ++my)
              for (int mx = lo[0]; mx <= hi[0]; ++mx) {
                size_t id = (size_t(mz) * vol.gdims[1] + my) * vol.gdims[0] + mx;
                vmin[id] = std::min(vmin[id], value);
                vmax[id] = std::max(vmax[id], value);
              }
        }
    vol.maxOpacity.assign(nc, 0.f);
    const int N = v->tfSize;
    for (size_t c = 0; c < nc; ++c) {
      if (vmax[c] < vmin[c]) { vol.maxOpacity[c] = 0.f; continue; }
      float lo = (vmin[c] - v->valueRange[0]) / (v->valueRange[1] - v->valueRange[0]);
      float hi = (vmax[c] - v->valueRange[0]) / (v->valueRange[1] - v->valueRange[0]);
      int ilo = std::min(std::max((int)(lo * (N - 1)), 0), N - 1);
      int ihi = std::min(std::max((int)(hi * (N - 1)) + 1, 0), N - 1);
      float m = 0.f;
      for (int i = ilo; i <= ihi; ++i) m = std::fmax(m, tfTex(v, (i + .5f) / N).w);
      vol.maxOpacity[c] = m;
    }
  } else if (v->gridMethod == OR_GRID_BRICK) {
    // Brick majorants: cell k along an axis covers normalized coordinates
    // [k/G, (k+1)/G]; every trilinear sample there reads texels
    // floor(k*N/G-0.5) .. floor((k+1)*N/G-0.5)+1 (clamped), whose min/max
    // bound the sample; the TF bins touched by [min,max] bound its alpha.
    const int B = v->brickSize;
    for (int a = 0; a < 3; ++a) vol.gdims[a] = (v->dims[a] + B - 1) / B;
    size_t nc = size_t(vol.gdims[0]) * vol.gdims[1] * vol.gdims[2];
    vol.maxOpacity.assign(nc, 0.f);
    const int N = v->tfSize;
    for (int kz = 0; kz < vol.gdims[2]; ++kz)
      for (int ky = 0; ky < vol.gdims[1]; ++ky)
        for (int kx = 0; kx < vol.gdims[0]; ++kx) {
          int k[3] = {kx, ky, kz}, t0[3], t1[3];
          for (int a = 0; a < 3; ++a) {
            int n = v->dims[a], G = vol.gdims[a];
            double lo = std::floor(double(k[a]) * n / G - 0.5);
            double hi = std::floor(double(k[a] + 1) * n / G - 0.5) + 1.0;
            t0[a] = (int)std::min(std::max(lo, 0.0), double(n - 1));
            t1[a] = (int)std::min(std::max(hi, 0.0), double(n - 1));
          }
          float mn = FLT_MAX, mx = -FLT_MAX;
          for (int z = t0[2]; z <= t1[2]; ++z)
            for (int y = t0[1]; y <= t1[1]; ++y)
              for (int x = t0[0]; x <= t1[0]; ++x) {
                float val = v->data[(size_t(z) * v->dims[1] + y) * v->dims[0] + x];
                mn = std::min(mn, val);
                mx = std::max(mx, val);
              }
          float lo = (mn - v->valueRange[0]) / (v->valueRange[1] - v->valueRange[0]);
          float hi = (mx - v->valueRange[0]) / (v->valueRange[1] - v->valueRange[0]);
          int ilo = (int)std::floor(lo * N - 0.5f);
          int ihi = (int)std::floor(hi * N - 0.5f) + 1;
          ilo = std::min(std::max(ilo, 0), N - 1);
          ihi = std::min(std::max(ihi, 0), N - 1);
          float m = 0.f;
          for (int i = ilo; i <= ihi; ++i) m = std::fmax(m, v->tf[4 * i + 3]);
          vol.maxOpacity[(size_t(kz) * vol.gdims[1] + ky) * vol.gdims[0] + kx] = m;
        }
  }
}

// ---------------------------------------------------------------------------
// Committed scene.
// ---------------------------------------------------------------------------
// An HDRI light's tables (scene/light/HDRI.cpp:30-164): the row-wise
// normalised CDFs, the normalised CDF of the row sums, the image frame.
struct Hdri {
  std::vector<float> rows, lastCol;
  float toWorld[9], toLocal[9];
};

struct Scene {
  const OrScene *src;
  std::vector<Hdri> hdri;  // per light (empty tables for other types)
  std::vector<std::vector<uint8_t>> texels;  // per sampler: its image as RGBA8
  std::vector<Tri> tris;
  std::vector<Vol> isoFields;  // the iso-surfaces' fields (bounds and voxel space)
  std::vector<f3> triNormal;   // quads: the shading normal per triangle (empty if none)
  std::vector<char> hasNormal;
  std::vector<GroupBVH> bvh;
  std::vector<Vol> vols;
  std::vector<Inst> insts;
};

struct Counters {
  uint64_t rays = 0, nodes = 0, tris = 0, march = 0, track = 0, cells = 0;
};

// Slab test (Visionaray intersect(ray, aabb)): tnear = max of per-axis
// minima, tfar = min of per-axis maxima, hit = tnear <= tfar.
struct BoxHit { bool hit; float tnear, tfar; };
BoxHit intersectBox(const Ray &r, const Box &b) {
  f3 inv = f3(1.f) / r.dir;
  f3 t1 = (b.lo - r.ori) * inv, t2 = (b.hi - r.ori) * inv;
  float tn = max_element(min3(t1, t2)), tf = min_element(max3(t1, t2));
  return BoxHit{tn <= tf, tn, tf};
}

struct SurfHit {
  bool hit = false;
  float t = FLT_MAX, u = 0, v = 0;
  int inst = -1, tri = -1;  // tri: global triangle index, -1 otherwise
  int prim = -1;            // global sphere / cone / cylinder index, -1 otherwise
  int iso = -1;             // global iso-surface index, -1 otherwise
  int key = -1;             // order within the instance: triangles, then spheres
  f3 isect_pos;             // instance-local hit position
};

// Ray/sphere test as Visionaray's basic_sphere intersection (the reference's
// intersect(ray, bls.asSphere), DeviceCopyableObjects.h:1486-1507): the
// smaller root of |o + t d - c|^2 = r^2 from the cancellation-free
// quadratic formula; -FLT_MAX without real roots.
inline float hitSphere(const Ray &r, const float *sph) {
  f3 oc = r.ori - f3(sph[0], sph[1], sph[2]);
  float A = dot(r.dir, r.dir);
  float B = 2.f * dot(r.dir, oc);
  float C = dot(oc, oc) - sph[3] * sph[3];
  float disc = B * B - 4.f * A * C;
  if (!(disc >= 0.f)) return -FLT_MAX;
  float rd = std::sqrt(disc);
  float q = B < 0.f ? -0.5f * (B - rd) : -0.5f * (B + rd);
  float t1 = q / A, t2 = C / q;
  return t1 > t2 ? t2 : t1;
}

// Capped cone (v1, r1) -> (v2, r2): intersect(Ray, Cone),
// DeviceCopyableObjects.h:933-1007 (Quilez's cone intersector). Caps first
// (the one the origin lies behind), then the body's smaller root; u = 0 / 1
// on the caps and y / |v2-v1|^2 on the body, v = y.
inline float hitCone(const Ray &r, const float *q, float &u, float &v) {
  f3 pa(q[0], q[1], q[2]), pb(q[4], q[5], q[6]);
  float ra = q[3], rb = q[7];
  f3 ba = pb - pa, oa = r.ori - pa, ob = r.ori - pb;
  float m0 = dot(ba, ba), m1 = dot(oa, ba), m2 = dot(r.dir, ba);
  float m3 = dot(r.dir, oa), m5 = dot(oa, oa), m9 = dot(ob, ba);
  if (m1 < 0.f) {
    f3 w = oa * m2 - r.dir * m1;
    if (dot(w, w) < ra * ra * m2 * m2) { u = 0.f; v = 0.f; return -m1 / m2; }
  } else if (m9 > 0.f) {
    float t = -m9 / m2;
    f3 w = ob + r.dir * t;
    if (dot(w, w) < rb * rb) { u = 1.f; v = 0.f; return t; }
  }
  float rr = ra - rb;
  float hy = m0 + rr * rr;
  float k2 = m0 * m0 - m2 * m2 * hy;
  float k1 = m0 * m0 * m3 - m1 * m2 * hy + m0 * ra * (rr * m2 * 1.f);
  float k0 = m0 * m0 * m5 - m1 * m1 * hy + m0 * ra * (rr * m1 * 2.f - m0 * ra);
  float h = k1 * k1 - k2 * k0;
  if (h < 0.f) return -FLT_MAX;
  float t = (-k1 - std::sqrt(h)) / k2;
  float y = m1 + t * m2;
  if (y > 0.f && y < m0) { u = y / m0; v = y; return t; }
  return -FLT_MAX;
}

// Capped cylinder v1 -> v2 of radius r1 (Quilez's published capped-cylinder
// intersector; Visionaray's basic_cylinder test is not part of the
// reference): the body's smaller root, else the cap plane the body root
// falls beyond, accepted inside the radius.
inline float hitCylinder(const Ray &r, const float *q) {
  f3 pa(q[0], q[1], q[2]), pb(q[4], q[5], q[6]);
  float ra = q[3];
  f3 ba = pb - pa, oc = r.ori - pa;
  float baba = dot(ba, ba), bard = dot(ba, r.dir), baoc = dot(ba, oc);
  float k2 = baba - bard * bard;
  float k1 = baba * dot(oc, r.dir) - baoc * bard;
  float k0 = baba * dot(oc, oc) - baoc * baoc - ra * ra * baba;
  float h = k1 * k1 - k2 * k0;
  if (h < 0.f) return -FLT_MAX;
  h = std::sqrt(h);
  float t = (-k1 - h) / k2;
  float y = baoc + t * bard;
  if (y > 0.f && y < baba) return t;
  t = ((y < 0.f ? 0.f : baba) - baoc) / bard;
  if (std::fabs(k1 + k2 * t) < h) return t;
  return -FLT_MAX;
}

// Ray/triangle test in the basic_triangle (Moller-Trumbore) form; u,v are
// the barycentrics of v2 and v3.
inline bool hitTri(const Ray &r, const Tri &T, float tmin, float &t, float &u, float &v) {
  f3 s1 = cross(r.dir, T.e2);
  float div = dot(s1, T.e1);
  if (div == 0.f) return false;
  float inv = 1.f / div;
  f3 d = r.ori - T.v1;
  float b1 = dot(d, s1) * inv;
  if (b1 < 0.f || b1 > 1.f) return false;
  f3 s2 = cross(d, T.e1);
  float b2 = dot(r.dir, s2) * inv;
  if (b2 < 0.f || b1 + b2 > 1.f) return false;
  float tt = dot(T.e2, s2) * inv;
  if (!(tt >= tmin)) return false;
  t = tt; u = b1; v = b2;
  return true;
}

// Iso-surface test, intersect(Ray, ISOSurface), DeviceCopyableObjects.h:
// 825-911, as the reference's CPU device runs it but without its 16^3
// empty-space grid. A known divergence: the reference restarts the march in
// each grid cell whose value range holds an iso value, so a lattice
// interval straddling such a cell and an empty one is not sampled there,
// while this march samples it (a crossing next to an empty cell may come
// out at a slightly different t). Here: in voxel
// space with the direction normalised, samples on the lattice anchored at
// tmin - dt/2 (by repeated addition, dt = (min spacing / 2) |S d|) over
// [tmin, tmax] clipped to the field box; the first lattice interval whose
// values bracket an iso value (inclusive) gives the hit by linear
// interpolation (the smallest over the values bracketed there; an interval
// bracketing one with equal ends stops the march without a hit). Returns
// the object-space t or -FLT_MAX.
float hitIso(const Vol &vol, const OrIso &iso, const Ray &l, float tmax) {
  BoxHit bh = intersectBox(l, vol.bounds);
  if (!bh.hit) return -FLT_MAX;
  const float tmin = std::fmax(l.tmin, bh.tnear);
  tmax = std::fmin(tmax, bh.tfar);
  f3 ov = vol.pointToVoxelSpace(l.ori), dv = vol.vectorToVoxelSpace(l.dir);
  const float scale = length(dv);
  dv = normalize(dv);
  const float t0v = tmin * scale, t1v = tmax * scale;
  const float dt = scale * (0.5f * vol.cellSize);
  if (!(dt > 0.f)) return -FLT_MAX;
  long budget = 1 << 22;
  float t0 = t0v - dt / 2.f, t1 = t0v - dt / 2.f;
  while (t0 < t0v) { t0 += dt; if (--budget <= 0) return -FLT_MAX; }
  while (t1 < t1v) { t1 += dt; if (--budget <= 0) return -FLT_MAX; }
  float v1 = sampleField(vol.v, ov + dv * t0);
  for (float t = t0; t < t1; t += dt) {
    if (--budget <= 0) return -FLT_MAX;
    float v2 = sampleField(vol.v, ov + dv * (t + dt));
    float lo = std::fmin(v1, v2), hi = std::fmax(v1, v2);
    bool hit = false;
    float best = FLT_MAX;
    for (int i = 0; i < iso.numValues; ++i) {
      float x = iso.values[i];
      if (x >= lo && x <= hi) {
        float f = (x - v1) / (v2 - v1);
        float tHit = t + dt * f;
        if (tHit < best) best = tHit;
        hit = true;
      }
    }
    if (hit) return best < FLT_MAX ? best / scale : -FLT_MAX;
    v1 = v2;
  }
  return -FLT_MAX;
}

// Bezier curve (BezierCurve, DeviceCopyableObjects.h:1034-1057): the cubic
// and its derivative as f / dfdt write them; q holds (w0, r, w1, -, w2, -,
// w3, -).
struct CurveR {
  f3 w0, w1, w2, w3;
  float r;
  explicit CurveR(const float *q)
      : w0(q[0], q[1], q[2]), w1(q[4], q[5], q[6]), w2(q[8], q[9], q[10]),
        w3(q[12], q[13], q[14]), r(q[3]) {}
  CurveR() : r(0.f) {}
  f3 f(float t) const {
    const float ti = 1.0f - t;
    return ti * ti * ti * w0 + 3.0f * ti * ti * t * w1 + 3.0f * ti * t * t * w2 + t * t * t * w3;
  }
  f3 dfdt(float t) const {
    const float ti = 1.0f - t;
    return -3.0f * ti * ti * w0 + 3.0f * (3.0f * t * t - 4.0f * t + 1.0f) * w1 +
           3.0f * (2.0f - 3.0f * t) * t * w2 + 3.0f * t * t * w3;
  }
};

// intersect(Ray, BezierCurve), DeviceCopyableObjects.h:1072-1289 (the
// Phantom ray-hair intersector, Reshetov and Luebke 2018): the early-out
// cylinder around the end points (radius from the curve points at t = 1/3
// and 2/3, plus r); the curve in the ray-centric frame (e3 = normalised
// direction, e1, e2 from make_orthonormal_basis, origin at the ray's; the
// frame's inverse applied as its transpose); up to 40 Newton steps of the
// ray / cylinder test (RayConeIntersection with dr = 0) from the end the
// direction points away from, regula falsi on a sign change of the step
// (bisection every 4th), then the other end; converged at |dt| < 5e-5.
// Returns s + c0.z (the distance along the normalised direction) or
// -FLT_MAX, and the curve parameter in u.
float hitCurve(const Ray &r, const float *q, float &uOut) {
  const CurveR c(q);
  auto distToAxis = [&](f3 pt) { return length(cross(pt - c.w0, pt - c.w3)) / length(c.w3 - c.w0); };
  const float rmax = std::fmax(distToAxis(c.f(0.33333f)), distToAxis(c.f(0.66667f))) + c.r;
  const f3 axis = normalize(c.w3 - c.w0);
  const f3 p0 = c.w0 - axis * c.r, p1 = c.w3 + axis * c.r;
  {
    const f3 ba = p1 - p0, oc = r.ori - p0;
    const float baba = dot(ba, ba), bard = dot(ba, r.dir), baoc = dot(ba, oc);
    const float k2 = baba - bard * bard;
    const float k1 = baba * dot(oc, r.dir) - baoc * bard;
    const float k0 = baba * dot(oc, oc) - baoc * baoc - rmax * rmax * baba;
    float h = k1 * k1 - k2 * k0;
    if (h < 0.0f) return -FLT_MAX;
    h = std::sqrt(h);
    float t = (-k1 - h) / k2;
    const float y = baoc + t * bard;
    bool hitCyl = y > 0.0f && y < baba;
    if (!hitCyl) {
      t = ((y < 0.0f ? 0.0f : baba) - baoc) / bard;
      hitCyl = std::fabs(k1 + k2 * t) < h;
    }
    if (!hitCyl) return -FLT_MAX;
  }
  f3 e1, e2;
  const f3 e3 = normalize(r.dir);
  make_orthonormal_basis(e1, e2, e3);
  auto rcc = [&](f3 p) {
    const f3 d = p - r.ori;
    return f3(dot(e1, d), dot(e2, d), dot(e3, d));
  };
  CurveR x;
  x.w0 = rcc(c.w0);
  x.w1 = rcc(c.w1);
  x.w2 = rcc(c.w2);
  x.w3 = rcc(c.w3);
  x.r = c.r;
  float tstart = dot(x.w3 - x.w0, r.dir) > 0.0f ? 0.0f : 1.0f;
  for (int ep = 0; ep < 2; ++ep) {
    float t = tstart, told = 0.f, dt1 = 0.f, dt2 = 0.f;
    for (int i = 0; i < 40; ++i) {
      const f3 c0 = x.f(t), cd = x.dfdt(t);
      const float r2 = c.r * c.r;
      float ddd = cd.x * cd.x + cd.y * cd.y;
      const float dp = c0.x * c0.x + c0.y * c0.y;
      const float cdd = c0.x * cd.x + c0.y * cd.y;
      const float cxd = c0.x * cd.y - c0.y * cd.x;
      const float cc = ddd;
      const float b = cd.z * (0.0f - cdd);
      const float cdz2 = cd.z * cd.z;
      ddd += cdz2;
      const float a = 2.0f * 0.0f * cdd + cxd * cxd - ddd * r2 + dp * cdz2;
      const float discr = b * b - a * cc;
      const float sRoot = (b - (discr > 0.0f ? std::sqrt(discr) : 0.0f)) / cc;
      float dt = (sRoot * cd.z - cdd) / ddd;
      if (discr > 0.0f && std::fabs(dt) < 5e-5f) {
        uOut = t;
        return sRoot + c0.z;
      }
      dt = std::fmin(dt, 0.5f);
      dt = std::fmax(dt, -0.5f);
      dt1 = dt2;
      dt2 = dt;
      if (dt1 * dt2 < 0.0f) {
        const float tnext = (i & 3) == 0 ? 0.5f * (told + t) : (dt2 * told - dt1 * t) / (dt2 - dt1);
        told = t;
        t = tnext;
      } else {
        told = t;
        t += dt;
      }
      if (t < 0.0f || t > 1.0f) break;
    }
    tstart = 1.0f - tstart;
  }
  return -FLT_MAX;
}

// Closest hit over all instances: intersectSurfaces(Ray,TLS) with the
// instance transform of intersect(Ray, Instance), DeviceCopyableObjects.h:
// 1772-1839. Hits are ordered by (t, instance, triangle).
SurfHit traceSurfaces(const Scene &sc, const Ray &ray, Counters &c) {
  SurfHit best;
  best.t = ray.tmax;
  c.rays++;
  for (size_t ii = 0; ii < sc.insts.size(); ++ii) {
    const Inst &inst = sc.insts[ii];
    const GroupBVH &bvh = sc.bvh[inst.group];
    const OrGroup &og = sc.src->groups[inst.group];
    Ray l = inst.toLocal(ray);
    // spheres, cones, cylinders: every one of the group's (no acceleration
    // structure)
    for (int k = og.apBegin; k < og.apEnd; ++k) {
      c.tris++;
      const float *q = sc.src->prims + 16 * (size_t)k;
      float u = 0.f, v = 0.f, t;
      if (sc.src->primKind[k] == 0) {
        t = hitSphere(l, q);
      } else if (sc.src->primKind[k] == 3) {
        t = hitCurve(l, q, u);
      } else {
        // cones and cylinders: the origin moved along the ray to twice the
        // bounding-sphere radius before the point nearest its centre (same
        // roots, no cancellation in the quadratics' terms; an origin outside
        // the bounding sphere keeps the cone's cap selection exact)
        f3 pa(q[0], q[1], q[2]), pb(q[4], q[5], q[6]);
        float R = 0.5f * length(pb - pa) + std::fmax(q[3], q[7]);
        float L2 = dot(l.dir, l.dir);
        float tc = dot(0.5f * (pa + pb) - l.ori, l.dir) / L2;
        float t0 = std::fmax(0.f, tc - 2.f * R / std::sqrt(L2));
        Ray l2 = l;
        l2.ori = l.ori + t0 * l.dir;
        t = sc.src->primKind[k] == 1 ? hitCone(l2, q, u, v) : hitCylinder(l2, q);
        if (t != -FLT_MAX) t = t0 + t;
      }
      if (!(t >= l.tmin)) continue;
      int key = (og.triEnd - og.triBegin) + (k - og.apBegin);
      bool closer = t < best.t ||
                    (t == best.t && best.hit &&
                     ((int)ii < best.inst || ((int)ii == best.inst && key < best.key)));
      if (!closer) continue;
      best.hit = true; best.t = t; best.u = u; best.v = v;
      best.inst = (int)ii; best.tri = -1; best.prim = k; best.iso = -1; best.key = key;
      best.isect_pos = l.ori + t * l.dir;
    }
    // iso-surfaces of the group, after its triangles and analytic primitives
    for (int k = og.isoBegin; k < og.isoEnd; ++k) {
      c.tris++;
      float t = hitIso(sc.isoFields[k], sc.src->isos[k], l, best.t);
      if (!(t >= l.tmin)) continue;
      int key = (og.triEnd - og.triBegin) + (og.apEnd - og.apBegin) + (k - og.isoBegin);
      bool closer = t < best.t ||
                    (t == best.t && best.hit &&
                     ((int)ii < best.inst || ((int)ii == best.inst && key < best.key)));
      if (!closer) continue;
      best.hit = true; best.t = t; best.u = 0.f; best.v = 0.f;
      best.inst = (int)ii; best.tri = -1; best.prim = -1; best.iso = k; best.key = key;
      best.isect_pos = l.ori + t * l.dir;
    }
    if (bvh.nodes.empty()) continue;
    f3 inv = f3(1.f) / l.dir;
    int stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp) {
      const BNode &n = bvh.nodes[stack[--sp]];
      c.nodes++;
      f3 t1 = (n.box.lo - l.ori) * inv, t2 = (n.box.hi - l.ori) * inv;
      float tn = std::fmax(max_element(min3(t1, t2)), l.tmin);
      float tf = std::fmin(min_element(max3(t1, t2)), best.t);
      if (tn > tf) continue;
      if (n.count > 0) {
        for (int k = 0; k < n.count; ++k) {
          int tri = bvh.prim[n.first + k];
          c.tris++;
          float t, u, v;
          if (!hitTri(l, sc.tris[tri], l.tmin, t, u, v)) continue;
          int key = tri - og.triBegin;
          bool closer = t < best.t ||
                        (t == best.t && best.hit &&
                         ((int)ii < best.inst || ((int)ii == best.inst && key < best.key)));
          if (!closer) continue;
          best.hit = true; best.t = t; best.u = u; best.v = v;
          best.inst = (int)ii; best.tri = tri; best.prim = -1; best.iso = -1; best.key = key;
          best.isect_pos = l.ori + t * l.dir;
        }
      } else {
        stack[sp++] = n.first;
        stack[sp++] = n.first + 1;
      }
    }
  }
  if (!best.hit) best.t = FLT_MAX;
  return best;
}

// Surface index and object-space geometric normal of a surface hit at its
// local position P (getNormals, renderer/common.h:241-303): normalize(e1 x
// e2) for a triangle; normalize((P - c) / r) for a sphere; for a cone the
// cap axis (u <= 0, u >= 1) or the body normal from the axis parameter v;
// for a cylinder the cap axis within the radius of an end point, else P
// minus its projection on the axis.
uint32_t hitSurface(const OrScene &S, const SurfHit &h) {
  if (h.iso >= 0) return S.isos[h.iso].surface;
  return h.prim >= 0 ? S.primSurface[h.prim] : S.triSurface[h.tri];
}

f3 fieldGradient(const OrVolume *v, f3 P, f3 delta);
f3 gradientDelta(const Vol &vol);

f3 hitNormal(const Scene &sc, const SurfHit &h) {
  if (h.iso >= 0) {  // the normalised field gradient (NaN for a zero difference)
    const Vol &vol = sc.isoFields[h.iso];
    return fieldGradient(vol.v, vol.pointToVoxelSpace(h.isect_pos), gradientDelta(vol));
  }
  if (h.prim >= 0) {
    const float *q = sc.src->prims + 16 * (size_t)h.prim;
    const f3 P = h.isect_pos, v1(q[0], q[1], q[2]), v2(q[4], q[5], q[6]);
    const int kind = sc.src->primKind[h.prim];
    if (kind == 0) return normalize((P - v1) / q[3]);
    if (kind == 3) return normalize(P - CurveR(q).f(h.u));  // renderer/common.h:304-308
    if (kind == 1) {
      f3 ba = v2 - v1;
      float m0 = dot(ba, ba);
      if (h.u <= 0.f) return -ba * (1.f / std::sqrt(m0));
      if (h.u >= 1.f) return ba * (1.f / std::sqrt(m0));
      float ra = q[3], rr = q[3] - q[7];
      float hy = m0 + rr * rr;
      return normalize(m0 * (m0 * (P - v1) + rr * ba * ra) - ba * hy * h.v);
    }
    f3 axis = normalize(v2 - v1);
    if (length(P - v1) < q[3]) return -axis;
    if (length(P - v2) < q[3]) return axis;
    float s = dot(P - v1, axis);
    return normalize(P - (v1 + s * axis));
  }
  if (!sc.hasNormal.empty() && sc.hasNormal[h.tri]) return sc.triNormal[h.tri];
  const Tri &T = sc.tris[h.tri];
  return normalize(cross(T.e1, T.e2));
}

// ---------------------------------------------------------------------------
// DDA (renderer/DDA.h:12-113) with the callback func(cellID, t0, t1).
// ---------------------------------------------------------------------------
template <typename Func>
void dda3(Ray ray, const int *gridDims, const Box &modelBounds, Func &&func) {
  const float ray_tmin = ray.tmin;
  ray.ori = ray.ori + ray.tmin * ray.dir;
  ray.tmin = 0.f;
  ray.tmax -= ray_tmin;
  const f3 rcp_dir = f3(1.f) / ray.dir;
  const f3 lo = (modelBounds.lo - ray.ori) * rcp_dir;
  const f3 hi = (modelBounds.hi - ray.ori) * rcp_dir;
  f3 tnear = min3(lo, hi);
  const f3 tfar = max3(lo, hi);
  if (ray.dir.x == 0.f) tnear.x = FLT_MAX;
  if (ray.dir.y == 0.f) tnear.y = FLT_MAX;
  if (ray.dir.z == 0.f) tnear.z = FLT_MAX;
  int cell[3];
  projectOnGrid(ray.ori, gridDims, modelBounds, cell);
  f3 gd((float)gridDims[0], (float)gridDims[1], (float)gridDims[2]);
  const f3 dist = max3(f3(0.f), (tfar - tnear) / gd);
  const int step[3] = {ray.dir.x > 0.f ? 1 : -1, ray.dir.y > 0.f ? 1 : -1,
                       ray.dir.z > 0.f ? 1 : -1};
  const int stop[3] = {ray.dir.x > 0.f ? gridDims[0] : -1,
                       ray.dir.y > 0.f ? gridDims[1] : -1,
                       ray.dir.z > 0.f ? gridDims[2] : -1};
  f3 tnext;
  for (int a = 0; a < 3; ++a)
    tnext[a] = ray.dir[a] > 0.f ? tnear[a] + float(cell[a] + 1) * dist[a]
                                : tnear[a] + float(gridDims[a] - cell[a]) * dist[a];
  float t0 = 0.f;
  while (1) {
    const float t1 = std::fmin(min_element(tnext), ray.tmax);
    int id = (cell[2] * gridDims[1] + cell[1]) * gridDims[0] + cell[0];
    if (!func(id, ray_tmin + t0, ray_tmin + t1)) return;
    const float tc = min_element(tnext);
    bool done = false;
    for (int a = 0; a < 3 && !done; ++a) {
      if (tnext[a] == tc) {
        tnext[a] += dist[a];
        cell[a] += step[a];
        if (cell[a] == stop[a]) done = true;
      }
    }
    if (done) break;
    t0 = t1;
  }
}

struct VolHit {
  bool hit = false;
  float t = FLT_MAX;
  f3 albedo;
  float Tr = 1.f;
  int inst = -1, vol = -1;
};

// Delta tracking, intersect(Ray, Volume), DeviceCopyableObjects.h:680-796.
// Returns true with t (object-space ray parameter) on a scattering event.
bool deltaTrack(const Vol &vol, Ray ray, LCG &rnd, float &tHit, f3 &albedo, Counters &c) {
  const OrVolume *v = vol.v;
  BoxHit bh = intersectBox(ray, vol.bounds);
  // The BVH over volumes culls boxes whose [tnear,tfar] misses [tmin,tmax].
  if (!bh.hit || bh.tfar < ray.tmin || bh.tnear > ray.tmax) return false;
  ray.tmin = std::fmax(ray.tmin, bh.tnear);
  ray.tmax = std::fmin(ray.tmax, bh.tfar);
  ray.ori = vol.pointToVoxelSpace(ray.ori);
  ray.dir = vol.vectorToVoxelSpace(ray.dir);
  const float dt_scale = length(ray.dir);
  ray.dir = normalize(ray.dir);
  ray.tmin = ray.tmin * dt_scale;
  ray.tmax = ray.tmax * dt_scale;
  float unitDistance = v->unitDistance * dt_scale;
  float invUnitDistance = 1.f / unitDistance;
  bool hit = false;
  float ht = ray.tmax;
  const bool gridValid = !vol.maxOpacity.empty();
  auto woodcock = [&](int leafID, float t0, float t1) -> bool {
    c.cells++;
    const float majorant = gridValid ? vol.maxOpacity[leafID] : 1.f;
    float t = t0;
    while (1) {
      if (majorant <= 0.f) break;
      t -= (std::log(1.f - rnd()) / (majorant * invUnitDistance));
      if (t >= t1) break;
      c.track++;
      f3 P = ray.ori + ray.dir * t;
      f4 s = postClassify(v, sampleField(v, P));
      float u = rnd();
      if (s.w >= u * majorant) {
        albedo = s.xyz();
        hit = true;
        ht = t;
        return false;
      }
    }
    return true;
  };
  if (gridValid) {
    Box gb;
    gb.lo = f3(0.f);
    gb.hi = f3(1.f);
    dda3(ray, vol.gdims, gb, woodcock);
  } else {
    woodcock(-1, ray.tmin, ray.tmax);
  }
  if (hit) tHit = ht / dt_scale;
  return hit;
}

// intersectVolumes over the world (DeviceCopyableObjects.h:1861-1879).
VolHit traceVolumes(const Scene &sc, const Ray &ray, LCG &rnd, Counters &c) {
  VolHit best;
  for (size_t ii = 0; ii < sc.insts.size(); ++ii) {
    const Inst &inst = sc.insts[ii];
    const OrGroup &g = sc.src->groups[inst.group];
    for (int vi = g.volBegin; vi < g.volEnd; ++vi) {
      Ray l = inst.toLocal(ray);
      float t;
      f3 alb;
      if (deltaTrack(sc.vols[vi], l, rnd, t, alb, c) && t < best.t) {
        best.hit = true;
        best.t = t;
        best.albedo = alb;
        best.Tr = 0.f;
        best.inst = (int)ii;
        best.vol = vi;
      }
    }
  }
  return best;
}

// ---------------------------------------------------------------------------
// Camera (DeviceCopyableObjects.h:2497-2600; camera/Perspective.cpp:33-44).
// Thin-lens convention: u = 2 s.x - 1, v = 2 s.y - 1 with s the image-region
// mapped ((x+.5)/w, (y+.5)/h); dir = normalize(u U + v V + W), |U| =
// tan(fovy/2) aspect, |V| = tan(fovy/2), W = view direction. The lens draws
// two random numbers per ray (used only when apertureRadius > 0); every
// primary ray then draws one for ray.time.
// ---------------------------------------------------------------------------
struct Cam {
  OrCamera c;
  f3 U, V, W, eye;
  float inv[16];
};

void mul44(const float *a, const float *b, float *o) {
  for (int col = 0; col < 4; ++col)
    for (int row = 0; row < 4; ++row) {
      float s = 0.f;
      for (int k = 0; k < 4; ++k) s += a[k * 4 + row] * b[col * 4 + k];
      o[col * 4 + row] = s;
    }
}

bool inv44(const float *m, float *out) {
  double a[4][8];
  for (int r = 0; r < 4; ++r)
    for (int cidx = 0; cidx < 4; ++cidx) {
      a[r][cidx] = m[cidx * 4 + r];
      a[r][cidx + 4] = (r == cidx) ? 1.0 : 0.0;
    }
  for (int cidx = 0; cidx < 4; ++cidx) {
    int p = cidx;
    for (int r = cidx + 1; r < 4; ++r)
      if (std::fabs(a[r][cidx]) > std::fabs(a[p][cidx])) p = r;
    if (a[p][cidx] == 0.0) return false;
    if (p != cidx)
      for (int k = 0; k < 8; ++k) std::swap(a[p][k], a[cidx][k]);
    double d = a[cidx][cidx];
    for (int k = 0; k < 8; ++k) a[cidx][k] /= d;
    for (int r = 0; r < 4; ++r)
      if (r != cidx) {
        double f = a[r][cidx];
        for (int k = 0; k < 8; ++k) a[r][k] -= f * a[cidx][k];
      }
  }
  for (int r = 0; r < 4; ++r)
    for (int cidx = 0; cidx < 4; ++cidx) out[cidx * 4 + r] = (float)a[r][cidx + 4];
  return true;
}

Cam makeCam(const OrCamera &c) {
  Cam k;
  k.c = c;
  f3 dir = normalize(f3(c.direction[0], c.direction[1], c.direction[2]));
  f3 up = normalize(f3(c.up[0], c.up[1], c.up[2]));
  k.eye = f3(c.position[0], c.position[1], c.position[2]);
  if (c.type == OR_CAM_PERSPECTIVE) {
    float th = std::tan(0.5f * c.fovy);
    k.W = dir;
    k.U = normalize(cross(dir, up)) * (th * c.aspect);
    k.V = normalize(cross(k.U, dir)) * th;
  } else if (c.type == OR_CAM_ORTHO) {
    k.U = normalize(cross(dir, up)) * (c.height * c.aspect);
    k.V = normalize(cross(k.U, dir)) * c.height;
    k.W = k.eye - 0.5f * k.U - 0.5f * k.V;
  } else if (c.type == OR_CAM_OMNI) {
    k.U = normalize(cross(dir, up));
    k.V = normalize(cross(k.U, dir));
    k.W = k.eye - 0.5f * k.U - 0.5f * k.V;
  } else if (c.type == OR_CAM_MATRIX) {
    float pv[16];
    mul44(c.proj, c.view, pv);
    inv44(pv, k.inv);
  }
  return k;
}

Ray primaryRay(const Cam &k, LCG *rng, float x, float y, float w, float h) {
  Ray r;
  r.tmin = 0.f;
  r.tmax = FLT_MAX;
  r.time = 0.5f;
  const OrCamera &c = k.c;
  if (c.type == OR_CAM_PERSPECTIVE) {
    float sx = (x + 0.5f) / w, sy = (y + 0.5f) / h;
    sx = (1.f - sx) * c.imageRegion[0] + sx * c.imageRegion[2];
    sy = (1.f - sy) * c.imageRegion[1] + sy * c.imageRegion[3];
    float u = 2.f * sx - 1.f, v = 2.f * sy - 1.f;
    r.ori = k.eye;
    r.dir = normalize(k.U * u + k.V * v + k.W);
    float l1 = 0.f, l2 = 0.f;
    if (rng) { l1 = (*rng)(); l2 = (*rng)(); }
    if (c.apertureRadius > 0.f) {
      f3 focal = r.ori + r.dir * (c.focusDistance / dot(r.dir, k.W));
      // concentric disk (Shirley-Chiu)
      float a = 2.f * l1 - 1.f, b = 2.f * l2 - 1.f, rr, phi;
      if (a == 0.f && b == 0.f) { rr = 0.f; phi = 0.f; }
      else if (std::fabs(a) > std::fabs(b)) { rr = a; phi = (kPi / 4.f) * (b / a); }
      else { rr = b; phi = (kPi / 2.f) - (kPi / 4.f) * (a / b); }
      float dx = rr * std::cos(phi) * c.apertureRadius, dy = rr * std::sin(phi) * c.apertureRadius;
      r.ori = k.eye + normalize(k.U) * dx + normalize(k.V) * dy;
      r.dir = normalize(focal - r.ori);
    }
  } else if (c.type == OR_CAM_MATRIX) {
    float u = 2.f * (x + 0.5f) / w - 1.f, v = 2.f * (y + 0.5f) / h - 1.f;
    auto xf = [&](float z) {
      float p[4] = {u, v, z, 1.f}, o[4];
      for (int row = 0; row < 4; ++row) {
        o[row] = 0.f;
        for (int col = 0; col < 4; ++col) o[row] += k.inv[col * 4 + row] * p[col];
      }
      return f3(o[0] / o[3], o[1] / o[3], o[2] / o[3]);
    };
    f3 p0 = xf(-1.f), p1 = xf(1.f);
    r.ori = p0;
    r.dir = normalize(p1 - p0);
  } else if (c.type == OR_CAM_ORTHO) {
    float sx = (x + 0.5f) / w, sy = (y + 0.5f) / h;
    sx = (1.f - sx) * c.imageRegion[0] + sx * c.imageRegion[2];
    sy = (1.f - sy) * c.imageRegion[1] + sy * c.imageRegion[3];
    r.ori = k.U * sx + k.V * sy + k.W;
    r.dir = normalize(f3(c.direction[0], c.direction[1], c.direction[2]));
  } else if (c.type == OR_CAM_OMNI) {
    float sx = (x + 0.5f) / w, sy = (y + 0.5f) / h;
    float theta = kPi * sy, phi = kTwoPi * sx;
    f3 ld(std::sin(theta) * std::cos(phi), std::cos(theta), std::sin(theta) * std::sin(phi));
    r.ori = k.U * sx + k.V * sy + k.W;
    r.dir = ld * f3(1.f, -1.f, 1.f);
  }
  if (rng) {
    float tr = (*rng)();
    r.time = (1.f - tr) * c.shutter[0] + tr * c.shutter[1];
  }
  return r;
}

// clipRay, renderer/common.h:1469-1482.
Ray clipRay(Ray ray, const OrRenderer &R) {
  for (int i = 0; i < R.numClipPlanes; ++i) {
    const float *p = R.clipPlanes + 4 * i;
    f3 N(p[0], p[1], p[2]);
    float D = p[3];
    float s = dot(N, ray.dir);
    if (s != 0.f) {
      float t = (D - dot(N, ray.ori)) / s;
      if (s < 0.f) ray.tmin = std::fmax(ray.tmin, t);
      else ray.tmax = std::fmin(ray.tmax, t);
    }
  }
  return ray;
}

// ---------------------------------------------------------------------------
// Materials (renderer/common.h:793-1415). Constant parameters only; tangent
// frames are absent, so the anisotropic branches never activate (their
// guard compares a NaN length) and are not restated.
// ---------------------------------------------------------------------------
inline float pow5(float f) { return f * f * f * f * f; }
inline f3 lerpR(f3 a, f3 b, float t) { return a * (1.f - t) + b * t; }
inline float mapRoughness(float r) { return std::fmax(0.045f, r); }

inline float D_GGX(float NdotH, float roughness, float EPS) {
  float alpha = roughness;
  float alpha2 = alpha * alpha;
  float d = (NdotH * alpha2 - NdotH) * NdotH + 1.f;
  float denom = kPi * d * d;
  return alpha2 / std::fmax(EPS, denom);
}

f3 materialColor(const OrMaterial &m) {
  f3 base(m.baseColor[0], m.baseColor[1], m.baseColor[2]);
  if (m.type == OR_PBR) return lerpR(base, f3(0.f), m.metallic); // getColorPBM :708-718
  return base;
}

float materialOpacity(const OrMaterial &m) { // getOpacity :735-760
  float op = m.opacity;
  if (m.alphaMode == OR_ALPHA_OPAQUE) return 1.f;
  if (m.alphaMode == OR_ALPHA_BLEND) return op;
  return op >= m.alphaCutoff ? 1.f : 0.f;
}

// ---------------------------------------------------------------------------
// Attributes and samplers (renderer/common.h:365-640).
// ---------------------------------------------------------------------------
// toRGBA (common.h:265-360): the element's components, the rest of
// (0, 0, 0, 1); unorm as value / (2^bits - 1); past the array: the default.
f4 attrFetch(const OrAttr &a, uint32_t i) {
  float c[4] = {0.f, 0.f, 0.f, 1.f};
  if (i < a.len) {
    for (int k = 0; k < a.comps; ++k) {
      if (a.fixedBits == 8) c[k] = ((const uint8_t *)a.data)[size_t(i) * a.comps + k] / 255.f;
      else if (a.fixedBits == 16) c[k] = ((const uint16_t *)a.data)[size_t(i) * a.comps + k] / 65535.f;
      else c[k] = ((const float *)a.data)[size_t(i) * a.comps + k];
    }
  }
  return f4(c[0], c[1], c[2], c[3]);
}

// lerp_r(a, b, c, u, v) over a triangle: (1 - u - v) a + u b + v c
f4 baryLerp(f4 a, f4 b, f4 c, float u, float v) {
  const float w = 1.f - u - v;
  return f4(w * a.x + u * b.x + v * c.x, w * a.y + u * b.y + v * c.y,
            w * a.z + u * b.z + v * c.z, w * a.w + u * b.w + v * c.w);
}

struct AttrCtx {
  const OrSurfAttr *sa = nullptr;
  const OrInstance *inst = nullptr;
  uint32_t primID = 0;
  float u = 0.f, v = 0.f;
  f3 worldPos, worldNormal, objectPos, objectNormal;
};

// getAttribute (renderer/common.h:365-521): triangles take face-varying,
// else per-vertex values (barycentric), else the primitive's; then the
// geometry's uniform value, then the instance's; else (0, 0, 0, 1).
f4 getAttr(const AttrCtx &c, int id) {
  if (id >= OR_ATTR_WORLD_POS && id <= OR_ATTR_OBJECT_NORMAL) {
    const f3 h = id == OR_ATTR_WORLD_POS ? c.worldPos : id == OR_ATTR_WORLD_NORMAL ? c.worldNormal
               : id == OR_ATTR_OBJECT_POS ? c.objectPos : c.objectNormal;
    return f4(h, 1.f);
  }
  if (id < 0 || id > OR_ATTR_COLOR || !c.sa) return f4(0.f, 0.f, 0.f, 1.f);
  const OrSurfAttr &s = *c.sa;
  if (s.isTriangle) {
    const uint32_t p = c.primID;
    if (s.faceVarying[id].comps)
      return baryLerp(attrFetch(s.faceVarying[id], 3 * p), attrFetch(s.faceVarying[id], 3 * p + 1),
                      attrFetch(s.faceVarying[id], 3 * p + 2), c.u, c.v);
    if (s.vertex[id].comps) {
      uint32_t i0 = 3 * p, i1 = 3 * p + 1, i2 = 3 * p + 2;
      if (s.index) { i0 = s.index[i0]; i1 = s.index[i1]; i2 = s.index[i2]; }
      return baryLerp(attrFetch(s.vertex[id], i0), attrFetch(s.vertex[id], i1),
                      attrFetch(s.vertex[id], i2), c.u, c.v);
    }
    if (s.primitive[id].comps) return attrFetch(s.primitive[id], p);
  }
  if (s.uniformMask & (1u << id))
    return f4(s.uniform[id][0], s.uniform[id][1], s.uniform[id][2], s.uniform[id][3]);
  if (c.inst && (c.inst->attrMask & (1u << id)))
    return f4(c.inst->attr[id][0], c.inst->attr[id][1], c.inst->attr[id][2], c.inst->attr[id][3]);
  return f4(0.f, 0.f, 0.f, 1.f);
}

// getNormals' shading normal (renderer/common.h:241-264): the vertex
// normals interpolated and normalised (with face-varying normals set, the
// reference reads the vertex normals at 3 primID + k), else Ng.
f3 shadingNormal(const OrSurfAttr &s, uint32_t p, float u, float v, f3 Ng) {
  if (!s.isTriangle || !s.vertexNormal) return Ng;
  uint32_t i[3] = {3 * p, 3 * p + 1, 3 * p + 2};
  if (!s.fvNormal && s.index)
    for (int k = 0; k < 3; ++k) i[k] = s.index[i[k]];
  for (int k = 0; k < 3; ++k)
    if (i[k] >= s.numVertexNormals) return Ng;
  const float *N = s.vertexNormal;
  f4 n = baryLerp(f4(N[3 * i[0]], N[3 * i[0] + 1], N[3 * i[0] + 2], 0.f),
                  f4(N[3 * i[1]], N[3 * i[1] + 1], N[3 * i[1] + 2], 0.f),
                  f4(N[3 * i[2]], N[3 * i[2] + 1], N[3 * i[2] + 2], 0.f), u, v);
  return normalize(n.xyz());
}

f4 mat4mul(const float *m, f4 v) {
  return f4(((m[0] * v.x + m[4] * v.y) + m[8] * v.z) + m[12] * v.w,
            ((m[1] * v.x + m[5] * v.y) + m[9] * v.z) + m[13] * v.w,
            ((m[2] * v.x + m[6] * v.y) + m[10] * v.z) + m[14] * v.w,
            ((m[3] * v.x + m[7] * v.y) + m[11] * v.z) + m[15] * v.w);
}

// toAddressMode (scene/surface/common.h:59-72): clampToEdge, repeat,
// mirrorRepeat on texel indices.
int wrapIndex(float fi, int n, int mode) {
  const int i = !(fi > -1e9f && fi < 1e9f) ? 0 : (int)fi;
  if (mode == 1) return ((i % n) + n) % n;
  if (mode == 2) {
    const int m = ((i % (2 * n)) + 2 * n) % (2 * n);
    return m < n ? m : 2 * n - 1 - m;
  }
  return i < 0 ? 0 : (i > n - 1 ? n - 1 : i);
}

// tex1D / tex2D / tex3D on the RGBA8 image: texel centres at (i + 0.5) / n,
// linear (x, then y, then z) or nearest.
f4 imageSample(const OrSampler &s, const std::vector<uint8_t> &tx, f4 tc) {
  const int axes = s.type == OR_SAMP_IMAGE1D ? 1 : (s.type == OR_SAMP_IMAGE2D ? 2 : 3);
  const float c[3] = {tc.x, tc.y, tc.z};
  int i0[3] = {0, 0, 0}, i1[3] = {0, 0, 0};
  float f[3] = {0.f, 0.f, 0.f};
  for (int a = 0; a < axes; ++a) {
    const int n = s.dims[a];
    if (s.linear) {
      const float x = c[a] * n - 0.5f;
      const float fl = std::floor(x);
      f[a] = x - fl;
      i0[a] = wrapIndex(fl, n, s.wrap[a]);
      i1[a] = wrapIndex(fl + 1.f, n, s.wrap[a]);
    } else {
      i0[a] = i1[a] = wrapIndex(std::floor(c[a] * n), n, s.wrap[a]);
    }
  }
  auto at = [&](int i, int j, int k) {
    const uint8_t *t = &tx[4 * ((size_t(k) * s.dims[1] + j) * s.dims[0] + i)];
    return f4(t[0] / 255.f, t[1] / 255.f, t[2] / 255.f, t[3] / 255.f);
  };
  auto lerp4 = [](f4 p, f4 q, float t) {
    return f4(p.x + t * (q.x - p.x), p.y + t * (q.y - p.y), p.z + t * (q.z - p.z), p.w + t * (q.w - p.w));
  };
  const f4 c00 = lerp4(at(i0[0], i0[1], i0[2]), at(i1[0], i0[1], i0[2]), f[0]);
  if (axes == 1) return c00;
  const f4 c10 = lerp4(at(i0[0], i1[1], i0[2]), at(i1[0], i1[1], i0[2]), f[0]);
  const f4 c0 = lerp4(c00, c10, f[1]);
  if (axes == 2) return c0;
  const f4 c01 = lerp4(at(i0[0], i0[1], i1[2]), at(i1[0], i0[1], i1[2]), f[0]);
  const f4 c11 = lerp4(at(i0[0], i1[1], i1[2]), at(i1[0], i1[1], i1[2]), f[0]);
  return lerp4(c0, lerp4(c01, c11, f[1]), f[2]);
}

// getSample (renderer/common.h:546-590).
f4 getSample(const Scene &sc, int k, const AttrCtx &c) {
  const OrSampler &s = sc.src->samplers[k];
  if (s.type == OR_SAMP_PRIMITIVE) return attrFetch(s.prim, c.primID + s.primOffset);
  f4 a = getAttr(c, s.inAttribute);
  auto addv = [](f4 p, const float *o) { return f4(p.x + o[0], p.y + o[1], p.z + o[2], p.w + o[3]); };
  if (s.type == OR_SAMP_TRANSFORM) return addv(mat4mul(s.outXfm, a), s.outOffset);
  a = addv(mat4mul(s.inXfm, a), s.inOffset);
  return addv(mat4mul(s.outXfm, imageSample(s, sc.texels[k], a)), s.outOffset);
}

f4 materialParam(const Scene &sc, int src, f4 value, const AttrCtx &c) {
  if (src < 0) return value;
  if (src >= 16) return getSample(sc, src - 16, c);
  return getAttr(c, src);
}

// The material at a hit with its parameters looked up (getColor, getF,
// getOpacity, renderer/common.h:642-710).
OrMaterial resolveMaterial(const Scene &sc, const OrMaterial &m, const AttrCtx &c) {
  OrMaterial r = m;
  const f4 col = materialParam(sc, m.src[0], f4(m.baseColor[0], m.baseColor[1], m.baseColor[2], 1.f), c);
  r.baseColor[0] = col.x;
  r.baseColor[1] = col.y;
  r.baseColor[2] = col.z;
  r.opacity = col.w * materialParam(sc, m.src[1], f4(m.opacity, 0.f, 0.f, 1.f), c).x;
  if (m.type == OR_PBR) {
    r.metallic = materialParam(sc, m.src[2], f4(m.metallic, 0.f, 0.f, 1.f), c).x;
    r.roughness = materialParam(sc, m.src[3], f4(m.roughness, 0.f, 0.f, 1.f), c).x;
  }
  return r;
}

// The attribute context of a surface hit (hit attributes zero).
AttrCtx hitAttrCtx(const Scene &sc, const SurfHit &h) {
  AttrCtx c;
  const OrScene &S = *sc.src;
  if (S.surfAttr) c.sa = &S.surfAttr[hitSurface(S, h)];
  c.inst = &S.instances[h.inst];
  c.primID = (h.prim < 0 && h.iso < 0) ? S.triPrimID[h.tri] : 0u;
  c.u = h.u;
  c.v = h.v;
  return c;
}

f3 evalPBR(const OrMaterial &m, f3 Ns, f3 viewDir, f3 lightDir) {
  const float metallic = m.metallic, roughness = m.roughness;
  const float clearcoat = m.clearcoat, clearcoatRoughness = m.clearcoatRoughness;
  const float ior = m.ior;
  f3 sheenColor(m.sheenColor[0], m.sheenColor[1], m.sheenColor[2]);
  const float perceptualRoughness = mapRoughness(roughness);
  const float perceptualClearcoatRoughness = mapRoughness(clearcoatRoughness);
  const float perceptualSheenRoughness = mapRoughness(m.sheenRoughness);
  const float alpha = perceptualRoughness * perceptualRoughness;
  const float clearcoatAlpha = perceptualClearcoatRoughness * perceptualClearcoatRoughness;
  const float EPS = 1e-14f;
  const f3 H = normalize(lightDir + viewDir);
  const float NdotV = std::fabs(dot(Ns, viewDir)) + EPS;
  const float NdotH = std::fmax(EPS, dot(Ns, H));
  const float NdotL = std::fmax(EPS, dot(Ns, lightDir));
  const float LdotH = std::fmax(EPS, dot(lightDir, H));
  const float VdotH = std::fmax(EPS, dot(viewDir, H));
  f3 baseColor(m.baseColor[0], m.baseColor[1], m.baseColor[2]);
  f3 diffuseColor = lerpR(baseColor, f3(0.f), metallic);
  float f0s = ((1.f - ior) / (1.f + ior));
  f0s = f0s * f0s;
  f3 f0 = lerpR(f3(f0s), baseColor, metallic);
  f3 F = f0 + (f3(1.f) - f0) * pow5(1.f - VdotH);
  // Fd_Burley
  float f90 = 0.5f + 2.f * alpha * LdotH * LdotH;
  float lightScatter = 1.f + (f90 - 1.f) * pow5(1.f - NdotL);
  float viewScatter = 1.f + (f90 - 1.f) * pow5(1.f - NdotV);
  f3 diffuseBRDF = diffuseColor * (lightScatter * viewScatter * kInvPi);
  float D = D_GGX(NdotH, alpha, EPS);
  // V_SmithGGXCorrelated as written at renderer/common.h:891-899
  float a2 = alpha * alpha;
  float GGXV = NdotL / (NdotV + std::sqrt(a2 + (1.f - a2) * NdotV * NdotV));
  float GGXL = NdotV / (NdotL + std::sqrt(a2 + (1.f - a2) * NdotL * NdotL));
  float V = 0.5f / (GGXV + GGXL);
  f3 specularBRDF = F * (D * V);
  float Dc = D_GGX(NdotH, clearcoatAlpha, EPS);
  float Vc = 0.25f / std::fmax(EPS, LdotH * LdotH);
  float Fc = (0.04f + (1.f - 0.04f) * pow5(1.f - LdotH)) * clearcoat;
  float Frc = (Dc * Vc) * Fc;
  float sheenAlphaInv = 1.f / perceptualSheenRoughness;
  float cos2h = NdotH * NdotH;
  float sin2h = std::fmax(1.f - cos2h, 0.0078125f);
  f3 Ds = sheenColor * ((2.f + sheenAlphaInv) * std::pow(sin2h, sheenAlphaInv * 0.5f) / kTwoPi);
  return ((diffuseBRDF + specularBRDF) * (1.f - Fc) + f3(Frc)) + Ds;
}

f3 evalMaterial(const OrMaterial &m, f3 Ns, f3 viewDir, f3 lightDir) {
  if (m.type == OR_MATTE) return materialColor(m) * kInvPi;
  return evalPBR(m, Ns, viewDir, lightDir);
}

struct BSDFSample { f3 dir, f; float pdf, cosT; };

f3 sampleGGXVNDF(f3 V, float ax, float ay, float U1, float U2) {
  f3 Vh = normalize(V * f3(ax, ay, 1.f));
  float lensq = Vh.x * Vh.x + Vh.y * Vh.y;
  f3 T1 = lensq > 0.f ? f3(-Vh.y, Vh.x, 0.f) / std::sqrt(lensq) : f3(1.f, 0.f, 0.f);
  f3 T2 = cross(Vh, T1);
  float r = std::sqrt(U1);
  float phi = kTwoPi * U2;
  float t1 = r * std::cos(phi);
  float t2 = r * std::sin(phi);
  float s = 0.5f * (1.f + Vh.z);
  t2 = (1.f - s) * std::sqrt(std::fmax(0.f, 1.f - t1 * t1)) + s * t2;
  f3 Nh = t1 * T1 + t2 * T2 + std::sqrt(1.f - t1 * t1 - t2 * t2) * Vh;
  return normalize(f3(Nh.x * ax, Nh.y * ay, std::fmax(0.f, Nh.z)));
}

void pdfGGXVNDF(f3 L, f3 V, float ax, float eta_i, float eta_t, f3 Ns, float &pdfSpec,
                float &pdfTrans) {
  const float EPS = 1e-14f;
  pdfSpec = 0.f;
  pdfTrans = 0.f;
  const float NdotL = dot(Ns, L);
  const float NdotV = std::fmax(EPS, dot(Ns, V));
  if (NdotL > 0.f) {
    f3 H = V + L;
    float lenH = length(H);
    if (lenH > 1e-4f) {
      H /= lenH;
      float NdotH = std::fmax(EPS, dot(Ns, H));
      const float ax2 = ax * ax;
      float D = D_GGX(NdotH, ax, EPS);
      float G1 = 2.f * NdotV / (NdotV + std::sqrt(ax2 + (1.f - ax2) * NdotV * NdotV));
      pdfSpec = (D * G1) / (4.f * NdotV);
    }
  } else if (NdotL < 0.f) {
    f3 H = -(V * eta_i + L * eta_t);
    float lenH = length(H);
    if (lenH > 1e-4f) {
      H /= lenH;
      if (dot(Ns, H) < 0.f) H = -H;
      const float alpha2 = ax * ax;
      float NdotH = std::fmax(EPS, dot(Ns, H));
      float LdotH = std::fabs(dot(L, H));
      float VdotH = std::fabs(dot(V, H));
      if (VdotH > 0.f && LdotH > 0.f) {
        float D = D_GGX(NdotH, ax, EPS);
        float G1 = 2.f * NdotV / (NdotV + std::sqrt(alpha2 + (1.f - alpha2) * NdotV * NdotV));
        float pdfNe = (D * G1 * VdotH) / NdotV;
        float denom = (eta_i * VdotH + eta_t * LdotH);
        float jacobian = (eta_t * eta_t * LdotH) / (denom * denom);
        pdfTrans = pdfNe * jacobian;
      }
    }
  }
}

// sampleMaterial, renderer/common.h:1371-1415 (and :1209-1368 for PBR).
// Two-argument calls such as cosine_sample_hemisphere(rnd(), rnd()) draw
// their arguments left to right.
BSDFSample sampleMaterial(const OrMaterial &m, f3 Ng, f3 Ns, f3 viewDir, LCG &rnd) {
  BSDFSample res;
  f3 w = faceforward(Ns, viewDir, Ng);
  f3 v = std::fabs(w.x) > std::fabs(w.y) ? normalize(f3(-w.z, 0.f, w.x))
                                         : normalize(f3(0.f, w.z, -w.y));
  f3 u = cross(v, w);
  if (m.type == OR_MATTE) {
    float u1 = rnd(), u2 = rnd();
    f3 sp = cosine_sample_hemisphere(u1, u2);
    res.dir = normalize(sp.x * u + sp.y * v + sp.z * w);
    res.pdf = std::fmax(0.f, dot(Ns, res.dir)) * kInvPi;
  } else {
    const float EPS = 1e-14f;
    const float metallic = m.metallic;
    const float alpha = mapRoughness(m.roughness) * mapRoughness(m.roughness);
    const float ccR = mapRoughness(m.clearcoatRoughness);
    const float clearcoatAlpha = ccR * ccR;
    const float transmission = m.transmission, ior = m.ior, clearcoat = m.clearcoat;
    const float NdotV = std::fmax(EPS, dot(Ns, viewDir));
    f3 baseColor(m.baseColor[0], m.baseColor[1], m.baseColor[2]);
    f3 diffuseColor = lerpR(baseColor, f3(0.f), metallic);
    float f0s = ((1.f - ior) / (1.f + ior));
    f0s = f0s * f0s;
    f3 f0 = lerpR(f3(f0s), baseColor, metallic);
    f3 F = f0 + (f3(1.f) - f0) * pow5(1.f - NdotV);
    const float fClear = clearcoat * 0.04f;
    const float baseEnergy = 1.f - fClear;
    const float fSpec = rgb_to_luminance(F);
    const float remainingEnergy = baseEnergy * (1.f - fSpec);
    float wDiff = rgb_to_luminance(diffuseColor) * remainingEnergy * (1.f - transmission);
    float wSpec = baseEnergy * fSpec;
    float wTrans = remainingEnergy * transmission;
    float wClear = fClear;
    float wSum = wDiff + wSpec + wTrans + wClear;
    float pDiff = wSum > 0.f ? wDiff / wSum : 0.0f;
    float pSpec = wSum > 0.f ? wSpec / wSum : 0.333f;
    float pTrans = wSum > 0.f ? wTrans / wSum : 0.667f;
    float pClear = 1.f - pDiff - pSpec - pTrans;
    float lobe = rnd();
    f3 V(dot(u, viewDir), dot(v, viewDir), dot(w, viewDir));
    bool entering = dot(Ns, viewDir) > 0.f;
    float eta_i = entering ? 1.0f : ior;
    float eta_t = entering ? ior : 1.0f;
    auto toWorld = [&](f3 n) { return u * n.x + v * n.y + w * n.z; };
    if (lobe < pDiff) {
      float u1 = rnd(), u2 = rnd();
      f3 sp = cosine_sample_hemisphere(u1, u2);
      res.dir = normalize(sp.x * u + sp.y * v + sp.z * w);
    } else if (lobe < pDiff + pSpec) {
      float u1 = rnd(), u2 = rnd();
      f3 Ne = sampleGGXVNDF(V, alpha, alpha, u1, u2);
      res.dir = reflect(viewDir, toWorld(Ne));
    } else if (lobe < pDiff + pSpec + pTrans) {
      float u1 = rnd(), u2 = rnd();
      f3 Ne = sampleGGXVNDF(V, alpha, alpha, u1, u2);
      if (dot(V, Ne) < 0.f) Ne = -Ne;
      res.dir = refract(viewDir, toWorld(Ne), eta_t / eta_i);
      if (length(res.dir) < 1e-4f) res.dir = reflect(viewDir, toWorld(Ne));
    } else {
      float u1 = rnd(), u2 = rnd();
      f3 Ne = sampleGGXVNDF(V, clearcoatAlpha, clearcoatAlpha, u1, u2);
      res.dir = reflect(viewDir, toWorld(Ne));
    }
    float pdfDiff = std::fmax(0.f, dot(Ns, res.dir)) * kInvPi;
    float pdfSpec = 0.f, pdfTrans = 0.f;
    pdfGGXVNDF(res.dir, viewDir, alpha, eta_i, eta_t, Ns, pdfSpec, pdfTrans);
    float pdfClear = 0.f, dummy = 0.f;
    float ceta_i = entering ? 1.0f : 1.5f;
    float ceta_t = entering ? 1.5f : 1.0f;
    pdfGGXVNDF(res.dir, viewDir, clearcoatAlpha, ceta_i, ceta_t, Ns, pdfClear, dummy);
    res.pdf = pDiff * pdfDiff + pSpec * pdfSpec + pTrans * pdfTrans + pClear * pdfClear;
  }
  res.cosT = std::fmax(0.f, dot(Ns, res.dir));
  res.f = evalMaterial(m, Ns, viewDir, res.dir);
  return res;
}

// ---------------------------------------------------------------------------
// Lights: sampleLight (renderer/common.h:1432-1466) towards reference point
// P. Directional (scene/light/Directional.cpp:30-40): the stored direction
// is -direction; with angularDiameter == 0 no random number is drawn,
// dist = FLT_MAX, pdf = 1, dist2 = 1; a positive angular diameter samples a
// uniform cone (2 draws). Point (scene/light/Point.cpp:28-37, Visionaray's
// point_light with constant attenuation 1) and spot
// (DeviceCopyableObjects.h:2286-2321): dir = position - P, dist = |dir|,
// dist2 = dist^2, pdf = 1, three draws for a light normal that delta lights
// do not use; intensity = color * intensity, for the spot times a
// smoothstep between cos(openingAngle) and cos(openingAngle - 2 falloff)
// (Spot.cpp:34-45).
// ---------------------------------------------------------------------------
struct LightSample { f3 intensity, dir; float pdf = 0.f, dist = 0.f, dist2 = 0.f; };

// Quad light geometry (dco::Quad, DeviceCopyableObjects.h:2187-2257): the
// parallelogram v1 + a e1 + b e2 tessellated as the triangles
// (v1, e1, e1 + e2) and (v1, e1 + e2, e2); each triangle's area is half the
// length of its edges' cross product, the light's normal the first
// triangle's unit normal.
struct QuadGeom { f3 v1, e1, e2, d, n; float A1, A2; };
QuadGeom quadGeom(const OrLight &L) {
  QuadGeom q;
  q.v1 = f3(L.position[0], L.position[1], L.position[2]);
  q.e1 = f3(L.edge1[0], L.edge1[1], L.edge1[2]);
  q.e2 = f3(L.edge2[0], L.edge2[1], L.edge2[2]);
  q.d = q.e1 + q.e2;
  const f3 c1 = cross(q.e1, q.d), c2 = cross(q.d, q.e2);
  const float n1 = length(c1);
  q.A1 = 0.5f * n1;
  q.A2 = 0.5f * length(c2);
  q.n = c1 / n1;
  return q;
}

// upper_bound + sample_cdf (sampleCDF.h:16-55): the first bin whose value
// exceeds x and its probability (0 past the end, where the reference reads
// an unset value).
unsigned cdfBin(const float *d, unsigned n, float x, float &pdf) {
  unsigned first = 0;
  int count = (int)n;
  while (count > 0) {
    const int step = count / 2;
    const unsigned it = first + step;
    if (!(x < d[it])) { first = it + 1; count -= step + 1; }
    else count = step;
  }
  if (first == 0) pdf = d[0];
  else if (first < n) pdf = d[first] - d[first - 1];
  else pdf = 0.f;
  return first;
}

// sampleCDF (sampleCDF.h:84-94) with the light record's tables as
// HDRI.cpp:156-157 stores them: the row from the row sums' CDF, then the
// column from that row's CDF.
void hdriSampleCdf(const OrLight &L, const Hdri &h, float rx, float ry, unsigned &x, unsigned &y,
                   float &pdfx, float &pdfy) {
  const unsigned W = (unsigned)L.hdriW, H = (unsigned)L.hdriH;
  y = cdfBin(h.lastCol.data(), H, ry, pdfy);
  y = std::min(y, H - 1);
  x = cdfBin(h.rows.data() + size_t(y) * W, W, rx, pdfx);
}

// toPolar / toUV (sampleCDF.h:57-82): M_PI makes the angle arithmetic
// double, rounded to float where the reference stores a float.
constexpr double kPiD = 3.14159265358979323846;
f3 hdriToPolar(float u, float v) {
  const float theta = (float)(2.0f * kPiD * (double)u + -kPiD / 2.0f);
  const float phi = (float)(kPiD * (double)v);
  f3 n;
  n.x = std::cos(theta) * std::sin(phi);
  n.z = std::sin(theta) * std::sin(phi);
  n.y = std::cos(phi);
  n.x = -n.x;
  return n;
}
void hdriToUV(f3 n, float &u, float &v) {
  u = std::atan2(n.x, n.z);
  u = (float)(((double)u + kPiD / 2.0f) / (kPiD * 2.0f) + kPiD * (double)(28.670f / 360.0f));
  v = std::fmin(std::fmax((float)((double)std::acos(n.y) / kPiD), .001f), .999f);
}

f3 mat3CM(const float *m, f3 v) {
  return f3((m[0] * v.x + m[3] * v.y) + m[6] * v.z, (m[1] * v.x + m[4] * v.y) + m[7] * v.z,
            (m[2] * v.x + m[5] * v.y) + m[8] * v.z);
}

// tex2D(radiance, uv): texel centres at (i + 0.5) / n, bilinear, clamp
// (HDRI.cpp:129-131), as Visionaray filters on the CPU.
f3 hdriTex(const OrLight &L, float u, float v) {
  const int W = L.hdriW, H = L.hdriH;
  const float x = u * W - 0.5f, y = v * H - 0.5f;
  const float fx0 = std::floor(x), fy0 = std::floor(y);
  const float fx = x - fx0, fy = y - fy0;
  auto cl = [](float f, int n) { return !(f >= 0.f) ? 0 : (f > (float)(n - 1) ? n - 1 : (int)f); };
  const int x0 = cl(fx0, W), x1 = cl(fx0 + 1.f, W), y0 = cl(fy0, H), y1 = cl(fy0 + 1.f, H);
  auto at = [&](int i, int j) {
    const float *c = L.radiance + 3 * (size_t(j) * W + i);
    return f3(c[0], c[1], c[2]);
  };
  const f3 r0 = lerp3(at(x0, y0), at(x1, y0), fx), r1 = lerp3(at(x0, y1), at(x1, y1), fx);
  return lerp3(r0, r1, fy);
}

// intensity(dir) = tex2D(radiance, toUV(toLocal dir)).xyz * scale
// (DeviceCopyableObjects.h:2384-2388).
f3 hdriIntensity(const OrLight &L, const Hdri &h, f3 dir) {
  float u, v;
  hdriToUV(mat3CM(h.toLocal, dir), u, v);
  return hdriTex(L, u, v) * L.scale;
}

// The HDRI density of a direction that hit the light (Pathtrace_impl.cpp:
// 160-172): the CDFs looked up with the direction's (u, v), the bin
// probabilities times W H / (2 pi^2 sin theta); 0 where sin theta is 0.
float hdriHitPdf(const OrLight &L, const Hdri &h, f3 rayDir) {
  const f3 dir = mat3CM(h.toLocal, rayDir);
  float u, v;
  hdriToUV(dir, u, v);
  unsigned x, y;
  float pdfx, pdfy;
  hdriSampleCdf(L, h, u, v, x, y, pdfx, pdfy);
  const float theta = std::acos(std::fmin(std::fmax(dir.y, -1.f), 1.f));
  const float sinTheta = std::sin(theta);
  if (sinTheta == 0.f) return 0.f;
  return (pdfx * pdfy) * (float)((unsigned)L.hdriW * (unsigned)L.hdriH) /
         (2.0f * kPi * kPi * sinTheta);
}

LightSample sampleLight(const Scene &sc, int li, f3 P, LCG &rnd) {
  const OrLight &L = sc.src->lights[li];
  LightSample s;
  s.pdf = 1.f;
  if (L.type == 4) {
    // HDRI (DeviceCopyableObjects.h:2371-2382, renderer/common.h:1459-1461):
    // a texel from the CDFs, the direction of its corner through toPolar
    // and toWorld, pdf = pdfx pdfy W H / (4 pi), dist = FLT_MAX, dist2 = 1.
    // The two draws are arguments of one call; GCC, which builds the
    // reference's CPU device, evaluates them right to left (the row's draw
    // first).
    const Hdri &h = sc.hdri[li];
    const float ry = rnd();
    const float rx = rnd();
    unsigned x, y;
    float pdfx, pdfy;
    hdriSampleCdf(L, h, rx, ry, x, y, pdfx, pdfy);
    const float invJacobian = (float)((unsigned)L.hdriW * (unsigned)L.hdriH) / (float)(4 * kPiD);
    s.dir = mat3CM(h.toWorld, hdriToPolar(x / (float)L.hdriW, y / (float)L.hdriH));
    s.dist = FLT_MAX;
    s.dist2 = 1.f;
    s.pdf = pdfx * pdfy * invJacobian;
    s.intensity = hdriIntensity(L, h, s.dir);
    return s;
  }
  if (L.type == 3) {
    // area_light<float, dco::Quad> (Visionaray, not vendored; conventions
    // restated): sample_surface(Quad) takes the first triangle when
    // A1 / (A1 + A2) < r (DeviceCopyableObjects.h:2258-2271), then the
    // triangle point v1 + sqrt(u1)(1 - u2) e1 + sqrt(u1) u2 e2 of two more
    // draws; intensity = color * intensity; pdf = 1 / (A |cos|) with the
    // cosine between the sample direction and the light's normal, so that
    // intensity / dist^2 / pdf is the area light's estimator as
    // renderer/common.h:1441-1464 and Pathtrace_impl.cpp:343-354 use it.
    const QuadGeom q = quadGeom(L);
    const float r = rnd();
    f3 a = q.d, b = q.e2;
    if (q.A1 / (q.A1 + q.A2) < r) { a = q.e1; b = q.d; }
    const float u1 = rnd(), u2 = rnd();
    const float su = std::sqrt(u1);
    const f3 pos = q.v1 + a * (su * (1.f - u2)) + b * (su * u2);
    s.dir = pos - P;
    s.dist = length(s.dir);
    s.dist2 = s.dist * s.dist;
    const float cosL = std::fabs(dot(s.dir, q.n)) / s.dist;
    s.pdf = 1.f / ((q.A1 + q.A2) * cosL);
    s.intensity = f3(L.color[0], L.color[1], L.color[2]) * L.intensity;
    return s;
  }
  if (L.type == 0) {
    f3 d = -normalize(f3(L.direction[0], L.direction[1], L.direction[2]));
    if (L.angularDiameter > 0.f) {
      float cosMax = std::cos(0.5f * L.angularDiameter);
      float u1 = rnd(), u2 = rnd();
      float cz = 1.f - u1 * (1.f - cosMax);
      float sz = std::sqrt(std::fmax(0.f, 1.f - cz * cz));
      float phi = kTwoPi * u2;
      f3 a, b;
      make_orthonormal_basis(a, b, d);
      d = normalize(a * (sz * std::cos(phi)) + b * (sz * std::sin(phi)) + d * cz);
    }
    s.dir = d;
    s.dist = FLT_MAX;
    s.dist2 = 1.f;
    s.intensity = f3(L.color[0], L.color[1], L.color[2]) * L.irradiance;
    return s;
  }
  s.dir = f3(L.position[0], L.position[1], L.position[2]) - P;
  s.dist = length(s.dir);
  s.dist2 = s.dist * s.dist;
  for (int k = 0; k < 3; ++k) (void)rnd();
  s.intensity = f3(L.color[0], L.color[1], L.color[2]) * L.intensity;
  if (L.type == 2) {
    const float cosOuter = std::cos(L.openingAngle);
    const float cosInner = std::cos(L.openingAngle - 2.f * L.falloffAngle);
    float spot = dot(normalize(f3(L.direction[0], L.direction[1], L.direction[2])),
                     normalize(-s.dir));
    if (spot < cosOuter) {
      s.intensity = f3(0.f);
    } else if (!(spot > cosInner)) {
      spot = (spot - cosOuter) / (cosInner - cosOuter);
      s.intensity = s.intensity * (spot * spot * (3.f - 2.f * spot));
    }
  }
  return s;
}

inline float safe_rcp(float f) { return f > 0.f ? 1.f / f : 0.f; }

// intersectLights (renderer/common.h:1566-1603): each quad light is tested
// as its two triangles with the ray's [tmin, tmax] (intersect(Ray, Quad),
// DeviceCopyableObjects.h:2211-2237, the nearer hit kept; both sides lit,
// Quad.cpp:48-51 fixes the side to Both) and taken when nearer than the hit
// so far (the first on ties); an HDRI light is always met at FLT_MAX and
// taken when nothing was hit yet or, against another light at FLT_MAX,
// when it is visible and that one is not; at bounce 0 invisible lights are
// skipped. Returns the light's index or -1 and its distance in tl.
int intersectLights(const OrScene &S, const Ray &ray, unsigned bounceID, float &tl) {
  auto tri = [&](f3 v1, f3 e1, f3 e2, float &t) {
    f3 s1 = cross(ray.dir, e2);
    float div = dot(s1, e1);
    if (div == 0.f) return false;
    float inv = 1.f / div;
    f3 d = ray.ori - v1;
    float b1 = dot(d, s1) * inv;
    if (b1 < 0.f || b1 > 1.f) return false;
    f3 s2 = cross(d, e1);
    float b2 = dot(ray.dir, s2) * inv;
    if (b2 < 0.f || b1 + b2 > 1.f) return false;
    t = dot(e2, s2) * inv;
    return t >= ray.tmin && t <= ray.tmax;
  };
  int id = -1;
  bool hit = false, vis = false;
  tl = FLT_MAX;
  for (int i = 0; i < S.numLights; ++i) {
    const OrLight &L = S.lights[i];
    if (bounceID == 0 && !L.visible) continue;
    if (L.type == 4) {
      if (!hit || (tl == FLT_MAX && L.visible && !vis)) {
        hit = true; vis = L.visible != 0; tl = FLT_MAX; id = i;
      }
      continue;
    }
    if (L.type != 3) continue;
    const QuadGeom q = quadGeom(L);
    float t1 = FLT_MAX, t2 = FLT_MAX;
    const bool h1 = tri(q.v1, q.e1, q.d, t1);
    const bool h2 = tri(q.v1, q.d, q.e2, t2);
    float t = FLT_MAX;
    if (h1) t = t1;
    if (h2 && t2 < t) t = t2;
    if ((h1 || h2) && t < tl) { hit = true; vis = L.visible != 0; tl = t; id = i; }
  }
  return id;
}

struct PixelSample {
  f4 color;
  float depth = 1e31f;
  f3 Ng, albedo;
  float mvx = 0.f, mvy = 0.f;  // motion vector (TAA), Pathtrace_impl.cpp:290-297
};

// Window position of P under a column-major view-projection matrix
// (Visionaray's project, the gluProject convention; viewport = the frame):
// clip = M (P, 1), ndc = clip / w, win = size (ndc + 1) / 2, each operation
// rounded in this order.
void projectWin(const float *M, f3 P, float W, float H, float &wx, float &wy) {
  auto row = [&](int r) { return ((M[r] * P.x + M[4 + r] * P.y) + M[8 + r] * P.z) + M[12 + r]; };
  const float cx = row(0), cy = row(1), cw = row(3);
  const float nx = cx / cw, ny = cy / cw;
  wx = (W * (nx + 1.f)) * 0.5f;
  wy = (H * (ny + 1.f)) * 0.5f;
}

// The view-projection matrix of a perspective camera as Visionaray's
// pinhole camera sets it up (Perspective.cpp:35-40: perspective(fovy,
// aspect, 0.001, 1000) and a look-at view from eye along dir with up), in
// double from the camera's direction and up as given (normalised here),
// rounded once to float; matrix cameras: proj * view.
void perspectiveViewProj(const float *eye, const float *dir, const float *up, float fovy,
                         float aspect, float *out) {
  const double n = 0.001, f = 1000.0;
  double F[3] = {dir[0], dir[1], dir[2]}, Up[3] = {up[0], up[1], up[2]};
  const double fl = std::sqrt(F[0] * F[0] + F[1] * F[1] + F[2] * F[2]);
  const double ul = std::sqrt(Up[0] * Up[0] + Up[1] * Up[1] + Up[2] * Up[2]);
  for (int k = 0; k < 3; ++k) {
    F[k] /= fl;
    Up[k] /= ul;
  }
  double S[3] = {F[1] * Up[2] - F[2] * Up[1], F[2] * Up[0] - F[0] * Up[2],
                 F[0] * Up[1] - F[1] * Up[0]};
  const double sl = std::sqrt(S[0] * S[0] + S[1] * S[1] + S[2] * S[2]);
  for (double &v : S) v /= sl;
  const double U[3] = {S[1] * F[2] - S[2] * F[1], S[2] * F[0] - S[0] * F[2],
                       S[0] * F[1] - S[1] * F[0]};
  double V[16] = {0};
  for (int k = 0; k < 3; ++k) {
    V[4 * k + 0] = S[k];
    V[4 * k + 1] = U[k];
    V[4 * k + 2] = -F[k];
  }
  V[12] = -(S[0] * eye[0] + S[1] * eye[1] + S[2] * eye[2]);
  V[13] = -(U[0] * eye[0] + U[1] * eye[1] + U[2] * eye[2]);
  V[14] = F[0] * eye[0] + F[1] * eye[1] + F[2] * eye[2];
  V[15] = 1.0;
  const double t = 1.0 / std::tan(0.5 * (double)fovy);
  double P[16] = {0};
  P[0] = t / aspect;
  P[5] = t;
  P[10] = (f + n) / (n - f);
  P[11] = -1.0;
  P[14] = 2.0 * f * n / (n - f);
  for (int col = 0; col < 4; ++col)
    for (int row = 0; row < 4; ++row) {
      double acc = 0.0;
      for (int k = 0; k < 4; ++k) acc += P[4 * k + row] * V[4 * col + k];
      out[4 * col + row] = (float)acc;
    }
}

// Raycast renderSample, renderer/Raycast_impl.cpp:10-243.
// sampleGradient (DeviceCopyableObjects.h:582-597): central differences of
// the field at voxel-space P, one offset of `delta` per axis, normalised as
// the callers do (VolumeIntegration.h:424-425, Pathtrace_impl.cpp:209-210).
// A zero difference normalises to NaN, as there.
f3 fieldGradient(const OrVolume *v, f3 P, f3 delta) {
  f3 g(sampleField(v, P + f3(delta.x, 0.f, 0.f)) - sampleField(v, P - f3(delta.x, 0.f, 0.f)),
       sampleField(v, P + f3(0.f, delta.y, 0.f)) - sampleField(v, P - f3(0.f, delta.y, 0.f)),
       sampleField(v, P + f3(0.f, 0.f, delta.z)) - sampleField(v, P - f3(0.f, 0.f, delta.z)));
  return g / std::sqrt(dot(g, g));
}

// The voxel-space offsets of the gradient: cellSize times the diagonal of
// the voxel-space transform (VolumeIntegration.h:398-401).
f3 gradientDelta(const Vol &vol) { return vol.S * vol.cellSize; }

// rayMarchVolume<1>'s shading of one classified sample
// (VolumeIntegration.h:420-460): a matte surface of the sample's colour
// along the face-forwarded gradient, lit by every light (zero-state
// generator, as for surfaces), plus the ambient term.
f3 gradientShade(const Scene &sc, const OrRenderer &R, const Vol &vol, f3 P, f3 viewDir, f3 rgb) {
  const OrScene &S = *sc.src;
  f3 gn = fieldGradient(vol.v, P, gradientDelta(vol));
  gn = faceforward(gn, viewDir, gn);
  f3 shaded(0.f);
  if (length(gn) > 1e-10f) {
    for (int li = 0; li < S.numLights; ++li) {
      LCG dummy;  // state 0: the reference's raycast stream is never seeded
      LightSample ls = sampleLight(sc, li, P, dummy);
      f3 lightDir = normalize(ls.dir);
      f3 lightIntensity = ls.intensity * safe_rcp(ls.dist2);
      const float NdotL = std::fmax(0.f, dot(gn, lightDir));
      shaded += rgb * kInvPi * lightIntensity * NdotL * safe_rcp(ls.pdf);
    }
  }
  return shaded + rgb * f3(R.ambientColor[0], R.ambientColor[1], R.ambientColor[2]) *
                      R.ambientRadiance;
}

PixelSample raycastSample(const Scene &sc, const OrRenderer &R, Ray ray, Counters &c) {
  PixelSample result;
  f4 bgColor(R.background[0], R.background[1], R.background[2], R.background[3]);
  result.color = bgColor;
  result.depth = 1e31f;
  if (sc.insts.empty()) return result;
  const OrScene &S = *sc.src;
  SurfHit hr = traceSurfaces(sc, ray, c);
  bool hit = false;
  f3 surfaceColor(0.f);
  float surfaceAlpha = 0.f;
  int layers = 0;
  while (true) {
    if (!hr.hit) break;
    if (++layers > (1 << 12)) break;  // same bound as the GPU path (zero epsilon would loop)
    const Inst &inst = sc.insts[hr.inst];
    uint32_t surf = hitSurface(S, hr);
    f3 hitPos = ray.ori + hr.t * ray.dir;
    f3 gn = hitNormal(sc, hr);
    f3 sn = gn;
    OrMaterial mat = S.surfMaterial[surf];
    if (S.surfAttr) {
      // shading normal and attributes (Raycast_impl.cpp:45-60): the
      // "worldNormal" attribute is the object-space normal, the
      // "objectNormal" one the transformed normal, as the reference passes
      AttrCtx ac = hitAttrCtx(sc, hr);
      sn = shadingNormal(*ac.sa, ac.primID, hr.u, hr.v, gn);
      ac.worldPos = hitPos;
      ac.worldNormal = gn;
      ac.objectPos = hr.isect_pos;
      gn = normalize(inst.normalXfm * gn);
      sn = normalize(inst.normalXfm * sn);
      ac.objectNormal = gn;
      mat = resolveMaterial(sc, mat, ac);
    } else {
      gn = normalize(inst.normalXfm * gn);
      sn = normalize(inst.normalXfm * sn);
    }
    f3 color = materialColor(mat);
    f3 shadedColor(0.f);
    f3 viewDir = -ray.dir;
    for (int li = 0; li < S.numLights; ++li) {
      LCG dummy;  // state 0: the reference's raycast stream is never seeded
      LightSample ls = sampleLight(sc, li, hitPos, dummy);
      f3 lightDir = normalize(ls.dir);
      f3 lightIntensity = ls.intensity * safe_rcp(ls.dist2);
      const float NdotL = std::fmax(0.f, dot(sn, lightDir));
      f3 bsdf = evalMaterial(mat, sn, normalize(viewDir), lightDir);
      shadedColor += bsdf * lightIntensity * NdotL * safe_rcp(ls.pdf);
    }
    shadedColor += color * f3(R.ambientColor[0], R.ambientColor[1], R.ambientColor[2]) *
                   R.ambientRadiance;
    float a = materialOpacity(mat);
    surfaceColor += (1.f - surfaceAlpha) * a * shadedColor;
    surfaceAlpha += (1.f - surfaceAlpha) * a;
    if (!hit) {
      result.depth = hr.t;
      result.Ng = gn;
      result.albedo = color;
    }
    hit = true;
    if (surfaceAlpha < 0.999f) {
      const float eps = epsilonFrom(hitPos, ray.dir, hr.t);
      ray.tmin = hr.t + eps;
      hr = traceSurfaces(sc, ray, c);
    } else {
      ray.tmax = hr.t;
      break;
    }
  }
  // behind the surfaces: the quad light the ray meets (its intensity,
  // alpha 1), else the background (Raycast_impl.cpp:158-172)
  f4 back = bgColor;
  {
    float tl;
    const int li = intersectLights(S, ray, 0, tl);
    if (li >= 0) {
      const OrLight &L = S.lights[li];
      back = L.type == 4 ? f4(hdriIntensity(L, sc.hdri[li], ray.dir), 1.f)
                         : f4(f3(L.color[0], L.color[1], L.color[2]) * L.intensity, 1.f);
    }
  }
  result.color = over(f4(surfaceColor, surfaceAlpha), back);

  // intersectVolumeBounds: closest volume box entry.
  int vInst = -1, vIdx = -1;
  float vT = FLT_MAX;
  for (size_t ii = 0; ii < sc.insts.size(); ++ii) {
    const Inst &inst = sc.insts[ii];
    const OrGroup &g = S.groups[inst.group];
    for (int vi = g.volBegin; vi < g.volEnd; ++vi) {
      Ray l = inst.toLocal(ray);
      BoxHit bh = intersectBox(l, sc.vols[vi].bounds);
      bool h = bh.hit && (bh.tfar >= l.tmin) && (bh.tnear <= l.tmax);
      float t = std::fmax(l.tmin, bh.tnear);
      if (h && t < vT) { vT = t; vInst = (int)ii; vIdx = vi; }
    }
  }
  if (vIdx >= 0) {
    const Vol &vol = sc.vols[vIdx];
    Ray l = sc.insts[vInst].toLocal(ray);
    // rayMarchVolume<0>, renderer/VolumeIntegration.h:374-468.
    BoxHit bh = intersectBox(l, vol.bounds);
    l.tmin = std::fmax(l.tmin, bh.tnear);
    l.tmax = std::fmin(l.tmax, bh.tfar);
    l.ori = vol.pointToVoxelSpace(l.ori);
    l.dir = vol.vectorToVoxelSpace(l.dir);
    float dt = vol.cellSize * (R.volumeSamplingRate > 0.f ? 1.f / R.volumeSamplingRate : 0.f);
    f3 color(0.f);
    float alpha = 0.f;
    float t = l.tmin;
    float transmittance = 1.f;
    const float expo = dt / vol.v->unitDistance;
    int steps = 0;
    // bounded like the GPU path: dt <= 0 or dt below the float spacing of t
    // would never end
    for (; t <= l.tmax && alpha < 0.99f && dt > 0.f && steps < (1 << 20); t += dt, ++steps) {
      f3 P = l.ori + l.dir * t;
      c.march++;
      float v = sampleField(vol.v, P);
      f4 s = postClassify(vol.v, v);
      float stepTransmittance = std::pow(1.f - s.w, expo);
      f3 rgb = s.xyz();
      if (R.gradientShading) rgb = gradientShade(sc, R, vol, P, -l.dir, rgb);
      color += transmittance * (1.f - stepTransmittance) * rgb;
      alpha += transmittance * (1.f - stepTransmittance);
      transmittance *= stepTransmittance;
    }
    result.color = over(alpha * f4(color, 1.f), result.color);
    result.Ng = f3(0.f);
    result.albedo = f3(0.f);
  }
  return result;
}

enum RayType { Radiance, Shadow, AO, Miss };

struct HitRec {
  SurfHit surface;
  VolHit volume;
  bool hit = false, volumeHit = false;
  bool lightHit = false;  // a quad light is the nearest hit
  int lightID = -1;
  float lightT = FLT_MAX;
};

// intersectAll (renderer/common.h:1605-1620) with intersectSurfaces<1>
// (:1502-1543): one random number is drawn per surface hit for stochastic
// opacity, then the volumes are tracked with the same generator.
HitRec intersectAll(const Scene &sc, const Ray &ray, LCG &rnd, Counters &c, unsigned bounceID) {
  HitRec h;
  const OrScene &S = *sc.src;
  Ray r = ray;
  SurfHit hr = traceSurfaces(sc, r, c);
  while (hr.hit) {
    // intersectSurfaces<EvalOpacity>: attributes at the hit, hit
    // attributes zero (renderer/common.h:1502-1543)
    const OrMaterial &mat = S.surfMaterial[hitSurface(S, hr)];
    float opacity = S.surfAttr ? materialOpacity(resolveMaterial(sc, mat, hitAttrCtx(sc, hr)))
                               : materialOpacity(mat);
    float u = rnd();
    if (u > opacity) {
      f3 hitPos = r.ori + hr.t * r.dir;
      const float eps = epsilonFrom(hitPos, r.dir, hr.t);
      r.tmin = hr.t + eps;
      hr = traceSurfaces(sc, r, c);
    } else {
      break;
    }
  }
  h.surface = hr;
  h.volume = traceVolumes(sc, ray, rnd, c);
  h.lightID = intersectLights(S, ray, bounceID, h.lightT);
  const bool lh = h.lightID >= 0;
  // a light hit takes precedence over surface and volume hits at equal
  // distance, a volume over a surface only when nearer
  h.hit = h.surface.hit || h.volume.hit || lh;
  h.lightHit = lh && (!h.surface.hit || h.lightT <= h.surface.t) &&
               (!h.volume.hit || h.lightT <= h.volume.t);
  h.volumeHit = h.volume.hit && (!h.surface.hit || h.volume.t < h.surface.t) &&
                (!lh || h.volume.t < h.lightT);
  return h;
}

struct ShadeState {
  f3 baseColor, shadedColor, hitPosOff, sn;
  int aoSamples = 0;
  float aoWeights = 0.f, aoCount = 0.f;
  BSDFSample bsdf{};
  LightSample light{};
  float misWeightNEE = 0.f;
  RayType nextType = Miss;
  Ray nextRay{};
  float visLight = 1.f, visAO = 1.f;
};

// shade(), renderer/Pathtrace_impl.cpp:93-487 (default render mode).
void shade(const Scene &sc, const OrRenderer &R, const OrFrame &F, LCG &rnd, const Ray &ray,
           RayType rayType, const HitRec &hitRec, ShadeState &ss, PixelSample &result,
           unsigned bounceID) {
  const OrScene &S = *sc.src;
  ss.nextType = Miss;
  if (rayType == Radiance) {
    ss.baseColor = f3(0.f);
    ss.visLight = 1.f;
    ss.visAO = 1.f;
    ss.aoSamples = 0;
    ss.aoWeights = 0.f;
    ss.aoCount = 0.f;
    if (!hitRec.hit) {
      ss.shadedColor = f3(0.f);
      ss.nextType = Miss;
      return;
    }
    if (hitRec.lightHit) {
      // a quad light seen by the ray: its intensity, after a bounce weighted
      // by the BSDF sample's MIS weight against the light's solid-angle
      // density (the light pdf over the number of lights); the path ends
      // (Pathtrace_impl.cpp:139-182)
      const OrLight &L = S.lights[hitRec.lightID];
      const bool hdri = L.type == 4;
      ss.shadedColor = hdri ? hdriIntensity(L, sc.hdri[hitRec.lightID], ray.dir)
                            : f3(L.color[0], L.color[1], L.color[2]) * L.intensity;
      ss.misWeightNEE = 1.f;
      if (bounceID > 0) {
        float lightPDF;
        if (hdri) {
          lightPDF = hdriHitPdf(L, sc.hdri[hitRec.lightID], ray.dir);
        } else {
          const QuadGeom q = quadGeom(L);
          const f3 hp = ray.ori + hitRec.lightT * ray.dir;
          const float ld = length(hp - ray.ori);
          const f3 Ld = normalize(hp - ray.ori);
          const float LdotNl = std::fabs(dot(-Ld, q.n));
          const float solidAngle = (LdotNl * (q.A1 + q.A2)) / (ld * ld);
          lightPDF = 1.f / solidAngle;
        }
        ss.shadedColor = ss.shadedColor * power_heuristic(ss.bsdf.pdf, lightPDF / float(S.numLights));
      }
      ss.nextType = Miss;
      return;
    }
    f3 hitPos, gn, sn, color;
    float eps;
    f3 viewDir = -normalize(ray.dir);
    const OrMaterial *mat = nullptr;
    OrMaterial resolved;
    if (hitRec.volumeHit) {
      const VolHit &hv = hitRec.volume;
      const Inst &inst = sc.insts[hv.inst];
      hitPos = ray.ori + hv.t * ray.dir;
      eps = epsilonFrom(hitPos, ray.dir, hv.t);
      gn = f3(0.f);
      if (R.gradientShading) {
        // the gradient at the instance-local hit position in voxel space
        // (Pathtrace_impl.cpp:203-211)
        const Vol &vol = sc.vols[hv.vol];
        Ray l = inst.toLocal(ray);
        gn = fieldGradient(vol.v, vol.pointToVoxelSpace(l.ori + hv.t * l.dir), gradientDelta(vol));
      }
      if (R.ambientSamples > 0 && length(gn) < 1e-3f) {
        float u1 = rnd(), u2 = rnd();
        gn = uniform_sample_sphere(u1, u2);
      }
      sn = gn;
      gn = inst.normalXfm * gn;
      sn = inst.normalXfm * sn;
      sn = faceforward(sn, viewDir, gn);
      gn = faceforward(gn, viewDir, gn);
      color = hv.albedo;
      if (bounceID == 0) result.depth = hv.t;
    } else {
      const SurfHit &hr = hitRec.surface;
      const Inst &inst = sc.insts[hr.inst];
      hitPos = ray.ori + hr.t * ray.dir;
      eps = epsilonFrom(hitPos, ray.dir, hr.t);
      mat = &S.surfMaterial[hitSurface(S, hr)];
      gn = hitNormal(sc, hr);
      sn = gn;
      AttrCtx ac;
      if (S.surfAttr) {
        ac = hitAttrCtx(sc, hr);
        sn = shadingNormal(*ac.sa, ac.primID, hr.u, hr.v, gn);
        ac.worldPos = hitPos;
        ac.worldNormal = gn;
        ac.objectPos = hr.isect_pos;
      }
      gn = normalize(inst.normalXfm * gn);
      sn = normalize(inst.normalXfm * sn);
      sn = faceforward(sn, viewDir, gn);
      gn = faceforward(gn, viewDir, gn);
      if (S.surfAttr) {
        // the material's looked-up parameters (Pathtrace_impl.cpp:255-270)
        ac.objectNormal = gn;
        resolved = resolveMaterial(sc, *mat, ac);
        mat = &resolved;
      }
      color = materialColor(*mat);
      if (bounceID == 0) result.depth = hr.t;
    }
    if (bounceID == 0) {
      result.Ng = gn;
      result.albedo = color;
    }
    ss.sn = sn;
    ss.hitPosOff = hitPos + sn * eps;
    if (R.taa) {
      // every radiance hit overwrites the sample's motion vector
      float px, py, cx, cy;
      projectWin(F.prevMVP, hitPos, (float)F.width, (float)F.height, px, py);
      projectWin(F.currMVP, hitPos, (float)F.width, (float)F.height, cx, cy);
      result.mvx = px - cx;
      result.mvy = py - cy;
    }
    int lightID = -1;
    bool areaSample = false;
    if (S.numLights > 0) {
      float r = rnd();
      lightID = int(r * S.numLights);
      if (lightID == S.numLights) lightID = 0;
      ss.light = sampleLight(sc, lightID, hitPos, rnd);
      areaSample = S.lights[lightID].type == 3 || S.lights[lightID].type == 4;
    }
    f3 lightDir = normalize(ss.light.dir);
    f3 lightIntensity = ss.light.intensity * safe_rcp(ss.light.dist2);
    const float NdotL = std::fmax(0.f, dot(sn, lightDir));
    if (hitRec.volumeHit) {
      const f3 &alb = hitRec.volume.albedo;
      if (R.gradientShading && length(gn) > 1e-10f)  // matte along the gradient, :313-328
        ss.shadedColor = alb * kInvPi * lightIntensity * NdotL * safe_rcp(ss.light.pdf) *
                         float(S.numLights);
      else
        ss.shadedColor = alb * lightIntensity * safe_rcp(ss.light.pdf) * safe_rcp(ss.light.dist2);
      float u1 = rnd(), u2 = rnd();
      ss.bsdf.dir = uniform_sample_sphere(u1, u2);
      ss.bsdf.f = alb;
      ss.bsdf.pdf = 1.f;
      ss.bsdf.cosT = 1.f;
    } else {
      f3 f = evalMaterial(*mat, sn, viewDir, lightDir);
      ss.shadedColor = f * lightIntensity * NdotL * safe_rcp(ss.light.pdf) * float(S.numLights);
      ss.bsdf = sampleMaterial(*mat, gn, sn, viewDir, rnd);
    }
    // Pathtrace_impl.cpp:365-375: the light sample's MIS weight against the
    // BSDF sample for an area light, 1 for a delta light
    ss.misWeightNEE = 0.f;
    if (S.numLights > 0) ss.misWeightNEE = 1.f;
    if (areaSample) ss.misWeightNEE = power_heuristic(ss.light.pdf / float(S.numLights), ss.bsdf.pdf);
    ss.baseColor = color;
  }

  auto prepShadow = [&]() {
    ss.nextType = Shadow;
    ss.nextRay.ori = ss.hitPosOff;
    ss.nextRay.dir = normalize(ss.light.dir);
    ss.nextRay.tmin = 0.f;
    ss.nextRay.tmax = ss.light.dist;
    ss.nextRay.time = ray.time;
  };
  auto prepAO = [&]() {
    f3 u, v, w = ss.sn;
    make_orthonormal_basis(u, v, w);
    float u1 = rnd(), u2 = rnd();
    f3 sp = cosine_sample_hemisphere(u1, u2);
    ss.nextType = AO;
    ss.nextRay.ori = ss.hitPosOff;
    ss.nextRay.dir = normalize(sp.x * u + sp.y * v + sp.z * w);
    ss.nextRay.tmin = 0.f;
    ss.nextRay.tmax = R.occlusionDistance;
    ss.nextRay.time = ray.time;
  };
  auto prepBounce = [&]() {
    ss.nextType = Radiance;
    ss.nextRay.ori = ss.hitPosOff;
    ss.nextRay.dir = normalize(ss.bsdf.dir);
    ss.nextRay.tmin = 0.f;
    ss.nextRay.tmax = 1e31f;
    ss.nextRay.time = ray.time;
  };

  if (rayType == Radiance) {
    if (ss.light.pdf >= 0.f) { prepShadow(); return; }
    if (ss.aoSamples < R.ambientSamples) { prepAO(); return; }
    if (ss.bsdf.pdf >= 0.f) { prepBounce(); return; }
    return;
  } else if (rayType == Shadow) {
    int surfV = hitRec.surface.hit ? 0 : 1;
    int volV = hitRec.volumeHit ? 0 : 1;
    ss.visLight = surfV * volV * hitRec.volume.Tr;
    if (ss.aoSamples < R.ambientSamples) { prepAO(); return; }
    if (ss.bsdf.pdf >= 0.f) { prepBounce(); return; }
    return;
  } else if (rayType == AO) {
    ss.aoSamples++;
    float weight = std::fmax(0.f, dot(ray.dir, ss.sn));
    ss.aoWeights += weight;
    if (weight > 0.f && hitRec.hit) ss.aoCount += weight;
    if (ss.aoSamples < R.ambientSamples) { prepAO(); return; }
    float aoV = 0.f;
    if (ss.aoWeights > 0.f) aoV = 1.f - (ss.aoCount / ss.aoWeights);
    ss.visAO *= aoV;
    if (ss.bsdf.pdf >= 0.f) { prepBounce(); return; }
    return;
  }
}

struct Ctx {
  const Scene *sc;
  Cam cam;
  const OrRenderer *R;
  OrFrame *F;
};

// cvt_uint32 / cvt_uint32_srgb, frame/common.h:31-48: clamp to [0,1],
// scale by 255 and truncate, RGBA in bytes 0..3 (sRGB encodes rgb only).
uint32_t cvtColor(f4 c, bool srgb) {
  auto cv = [](float f) { return (uint32_t)(255.f * std::min(std::max(f, 0.f), 1.f)); };
  if (srgb) c = f4(linear_to_srgb1(c.x), linear_to_srgb1(c.y), linear_to_srgb1(c.z), c.w);
  return cv(c.x) | (cv(c.y) << 8) | (cv(c.z) << 16) | (cv(c.w) << 24);
}

// Per-pixel body of VisionarayRendererPathtrace::renderFrame,
// renderer/Pathtrace_impl.cpp:498-640, followed by dco::Frame::writeSample.
void pathtracePixel(const Ctx &cx, int x, int y, Counters &c) {
  const Scene &sc = *cx.sc;
  const OrRenderer &R = *cx.R;
  OrFrame &F = *cx.F;
  const int W = F.width, H = F.height;
  int pixelID = x + W * y;
  LCG rng((uint32_t)pixelID, (uint32_t)F.accumID);
  LCG rnd = rng; // ScreenSample keeps its own copy (:512-513)
  f4 accumColor(0.f);
  PixelSample closest;
  closest.depth = 1e31f;
  const int spp = R.pixelSamples;
  const f3 ambient = f3(R.ambientColor[0], R.ambientColor[1], R.ambientColor[2]) * R.ambientRadiance;
  for (int sampleID = 0; sampleID < spp; ++sampleID) {
    float xf = (float)x, yf = (float)y;
    float jx = rnd() - .5f;
    float jy = rnd() - .5f;
    xf += jx;
    yf += jy;
    Ray ray = primaryRay(cx.cam, &rnd, xf, yf, (float)W, (float)H);
    PixelSample ps;
    ps.color = f4(R.background[0], R.background[1], R.background[2], R.background[3]);
    ps.depth = 1e31f;
    if (!sc.insts.empty()) {
      bool firstHit = false;
      ShadeState ss;
      RayType rayType = Radiance;
      f3 throughput(1.f), intensity(0.f);
      for (unsigned passID = 0, bounceID = 0; true; ++passID) {
        ray = clipRay(ray, R);
        HitRec hitRec = intersectAll(sc, ray, rnd, c, bounceID);
        shade(sc, R, F, rnd, ray, rayType, hitRec, ss, ps, bounceID);
        if (passID == 0 && bounceID == 0) firstHit = hitRec.hit;
        ray = ss.nextRay;
        rayType = ss.nextType;
        if (rayType == Miss || rayType == Radiance) {
          f3 direct = ss.shadedColor * ss.visLight;
          f3 amb = ss.baseColor * ambient * ss.visAO;
          intensity += throughput * ss.misWeightNEE * direct;
          intensity += throughput * amb;
          throughput *= ss.bsdf.f * ss.bsdf.cosT * safe_rcp(ss.bsdf.pdf);
          bounceID++;
        }
        if (rayType == Miss || bounceID > (unsigned)R.maxBounce) break;
        if (bounceID > 1) {
          float prob = max_element(throughput);
          if (rng.next() > prob) break;
          throughput /= prob;
        }
      }
      if (firstHit) ps.color = f4(intensity, 1.f);
    }
    accumColor += ps.color;
    if (F.sampleSum) {
      double *s = F.sampleSum + 3 * size_t(pixelID);
      double *q = F.sampleSumSq + 3 * size_t(pixelID);
      s[0] += ps.color.x; s[1] += ps.color.y; s[2] += ps.color.z;
      q[0] += double(ps.color.x) * ps.color.x;
      q[1] += double(ps.color.y) * ps.color.y;
      q[2] += double(ps.color.z) * ps.color.z;
    }
    if (ps.depth < closest.depth) closest = ps;
  }
  PixelSample fin = closest;
  fin.color = accumColor * (1.f / spp);
  // writeSample = fillGBuffer + accumSample + toneMap (DeviceCopyableObjects.h:2692-2781)
  size_t idx = size_t(y) * W + x;
  if (R.taa) {
    // fillGBuffer only (Pathtrace_impl.cpp:636-637); the resolve pass blends
    F.motionVec[2 * idx] = fin.mvx;
    F.motionVec[2 * idx + 1] = fin.mvy;
    F.taaCurr[4 * idx] = fin.color.x;
    F.taaCurr[4 * idx + 1] = fin.color.y;
    F.taaCurr[4 * idx + 2] = fin.color.z;
    F.taaCurr[4 * idx + 3] = fin.color.w;
    F.taaCurrAlbedo[3 * idx] = fin.albedo.x;
    F.taaCurrAlbedo[3 * idx + 1] = fin.albedo.y;
    F.taaCurrAlbedo[3 * idx + 2] = fin.albedo.z;
    if (F.depth && !(fin.depth > F.depth[idx])) {
      F.depth[idx] = fin.depth;
      if (F.normal) { F.normal[3 * idx] = fin.Ng.x; F.normal[3 * idx + 1] = fin.Ng.y; F.normal[3 * idx + 2] = fin.Ng.z; }
      if (F.albedo) { F.albedo[3 * idx] = fin.albedo.x; F.albedo[3 * idx + 1] = fin.albedo.y; F.albedo[3 * idx + 2] = fin.albedo.z; }
    }
    return;
  }
  if (F.depth && !(fin.depth > F.depth[idx])) {
    F.depth[idx] = fin.depth;
    if (F.normal) { F.normal[3 * idx] = fin.Ng.x; F.normal[3 * idx + 1] = fin.Ng.y; F.normal[3 * idx + 2] = fin.Ng.z; }
    if (F.albedo) { F.albedo[3 * idx] = fin.albedo.x; F.albedo[3 * idx + 1] = fin.albedo.y; F.albedo[3 * idx + 2] = fin.albedo.z; }
  }
  float a = 1.f / (F.accumID + 1);
  float *acc = F.accum + 4 * idx;
  acc[0] = (1 - a) * acc[0] + a * fin.color.x;
  acc[1] = (1 - a) * acc[1] + a * fin.color.y;
  acc[2] = (1 - a) * acc[2] + a * fin.color.z;
  acc[3] = (1 - a) * acc[3] + a * fin.color.w;
  fin.color = f4(acc[0], acc[1], acc[2], acc[3]);
  if (F.color) {
    if (F.colorType == OR_COLOR_FLOAT4) {
      float *o = (float *)F.color + 4 * idx;
      o[0] = fin.color.x; o[1] = fin.color.y; o[2] = fin.color.z; o[3] = fin.color.w;
    } else {
      ((uint32_t *)F.color)[idx] = cvtColor(fin.color, F.colorType == OR_COLOR_SRGB8);
    }
  }
}

// Per-pixel body of VisionarayRendererRaycast::renderFrame,
// renderer/Raycast_impl.cpp:254-321 (non-stochastic: color written as is).
void raycastPixel(const Ctx &cx, int x, int y, Counters &c) {
  const Scene &sc = *cx.sc;
  const OrRenderer &R = *cx.R;
  OrFrame &F = *cx.F;
  const int W = F.width, H = F.height;
  f4 accumColor(0.f);
  PixelSample first;
  const int spp = R.pixelSamples;
  for (int sampleID = 0; sampleID < spp; ++sampleID) {
    Ray ray = primaryRay(cx.cam, nullptr, (float)x, (float)y, (float)W, (float)H);
    ray = clipRay(ray, R);
    PixelSample ps = raycastSample(sc, R, ray, c);
    accumColor += ps.color;
    if (sampleID == 0) first = ps;
  }
  PixelSample fin = first;
  fin.color = accumColor * (1.f / spp);
  size_t idx = size_t(y) * W + x;
  if (F.sampleSum) {
    double *s = F.sampleSum + 3 * idx;
    double *q = F.sampleSumSq + 3 * idx;
    s[0] += fin.color.x; s[1] += fin.color.y; s[2] += fin.color.z;
    q[0] += double(fin.color.x) * fin.color.x;
    q[1] += double(fin.color.y) * fin.color.y;
    q[2] += double(fin.color.z) * fin.color.z;
  }
  if (F.depth && !(fin.depth > F.depth[idx])) {
    F.depth[idx] = fin.depth;
    if (F.normal) { F.normal[3 * idx] = fin.Ng.x; F.normal[3 * idx + 1] = fin.Ng.y; F.normal[3 * idx + 2] = fin.Ng.z; }
    if (F.albedo) { F.albedo[3 * idx] = fin.albedo.x; F.albedo[3 * idx + 1] = fin.albedo.y; F.albedo[3 * idx + 2] = fin.albedo.z; }
  }
  if (F.color) {
    if (F.colorType == OR_COLOR_FLOAT4) {
      float *o = (float *)F.color + 4 * idx;
      o[0] = fin.color.x; o[1] = fin.color.y; o[2] = fin.color.z; o[3] = fin.color.w;
    } else {
      ((uint32_t *)F.color)[idx] = cvtColor(fin.color, F.colorType == OR_COLOR_SRGB8);
    }
  }
}

// makeCDF (HDRI.cpp:30-68): per texel max(r, g, b); each row's running
// sum in float, the row's total kept, the row divided by its last entry
// unless that is 0; the totals scanned and normalised the same way.
void makeHdriCdf(const OrLight &L, Hdri &h) {
  const int W = L.hdriW, H = L.hdriH;
  h.rows.assign(size_t(W) * H, 0.f);
  h.lastCol.assign(H, 0.f);
  std::vector<float> total(H);
  for (int y = 0; y < H; ++y) {
    float *r = h.rows.data() + size_t(y) * W;
    float acc = 0.f;
    for (int x = 0; x < W; ++x) {
      const float *c = L.radiance + 3 * (size_t(y) * W + x);
      const float lum = std::max(std::max(c[0], c[1]), c[2]);
      acc = x == 0 ? lum : acc + lum;
      r[x] = acc;
    }
    total[y] = r[W - 1];
    const float back = r[W - 1];
    if (back != 0.f)
      for (int x = 0; x < W; ++x) r[x] = r[x] / back;
  }
  float acc = 0.f;
  for (int y = 0; y < H; ++y) {
    acc = y == 0 ? total[0] : acc + total[y];
    h.lastCol[y] = acc;
  }
  const float back = h.lastCol[H - 1];
  if (back != 0.f)
    for (int y = 0; y < H; ++y) h.lastCol[y] = h.lastCol[y] / back;
  // toWorld's columns (HDRI.cpp:146-150): -normalize(up),
  // normalize(cross(col1, direction)), normalize(cross(col0, col1));
  // toLocal its inverse (cofactors over the determinant in double)
  f3 c1 = -normalize(f3(L.up[0], L.up[1], L.up[2]));
  f3 c0 = normalize(cross(c1, f3(L.direction[0], L.direction[1], L.direction[2])));
  f3 c2 = normalize(cross(c0, c1));
  const f3 cols[3] = {c0, c1, c2};
  for (int c = 0; c < 3; ++c)
    for (int k = 0; k < 3; ++k) h.toWorld[3 * c + k] = cols[c][k];
  double a[9];
  for (int i = 0; i < 9; ++i) a[i] = h.toWorld[i];
  const double c00 = a[4] * a[8] - a[7] * a[5], c01 = a[7] * a[2] - a[1] * a[8],
               c02 = a[1] * a[5] - a[4] * a[2];
  const double det = a[0] * c00 + a[3] * c01 + a[6] * c02;
  h.toLocal[0] = (float)(c00 / det);
  h.toLocal[1] = (float)(c01 / det);
  h.toLocal[2] = (float)(c02 / det);
  h.toLocal[3] = (float)((a[6] * a[5] - a[3] * a[8]) / det);
  h.toLocal[4] = (float)((a[0] * a[8] - a[6] * a[2]) / det);
  h.toLocal[5] = (float)((a[3] * a[2] - a[0] * a[5]) / det);
  h.toLocal[6] = (float)((a[3] * a[7] - a[6] * a[4]) / det);
  h.toLocal[7] = (float)((a[6] * a[1] - a[0] * a[7]) / det);
  h.toLocal[8] = (float)((a[0] * a[4] - a[3] * a[1]) / det);
}

// imageSamplerUpdateData (scene/surface/material/sampler/common.h:27-60):
// every image format as RGBA8, missing channels 0 and alpha 1; floats
// clamped to [0, 1], times 255, truncated (as cvt_uint32, frame/common.h:
// 31-48, converts); sRGB texels decoded with the sRGB transfer function.
std::vector<uint8_t> samplerTexels(const OrSampler &sp) {
  const size_t n = size_t(sp.dims[0]) * sp.dims[1] * sp.dims[2];
  std::vector<uint8_t> out(4 * n);
  auto cv = [](float f) { return (uint8_t)(255.f * std::min(std::max(f, 0.f), 1.f)); };
  for (size_t i = 0; i < n; ++i) {
    uint8_t *o = &out[4 * i];
    o[0] = o[1] = o[2] = 0;
    o[3] = 255;
    const int c = sp.imageComps;
    if (sp.imageType == OR_IMG_FLOAT) {
      const float *p = (const float *)sp.image + c * i;
      for (int k = 0; k < c; ++k) o[k] = cv(p[k]);
    } else if (sp.imageType == OR_IMG_UNORM8) {
      const uint8_t *p = (const uint8_t *)sp.image + c * i;
      for (int k = 0; k < c; ++k) o[k] = p[k];
    } else {
      const uint8_t *p = (const uint8_t *)sp.image + 4 * i;
      for (int k = 0; k < 3; ++k) {
        const float x = p[k] / 255.f;
        o[k] = cv(x <= 0.04045f ? x / 12.92f : std::pow((x + 0.055f) / 1.055f, 2.4f));
      }
      o[3] = p[3];
    }
  }
  return out;
}

Scene *commit(const OrScene *s) {
  auto *sc = new Scene;
  sc->src = s;
  sc->texels.resize(s->numSamplers);
  for (int i = 0; i < s->numSamplers; ++i)
    if (s->samplers[i].type <= OR_SAMP_IMAGE3D) sc->texels[i] = samplerTexels(s->samplers[i]);
  sc->hdri.resize(s->numLights);
  for (int i = 0; i < s->numLights; ++i)
    if (s->lights[i].type == 4) makeHdriCdf(s->lights[i], sc->hdri[i]);
  sc->tris.resize(s->numTriangles);
  for (int i = 0; i < s->numTriangles; ++i) {
    const float *p = s->triVerts + 9 * i;
    f3 v1(p[0], p[1], p[2]), v2(p[3], p[4], p[5]), v3(p[6], p[7], p[8]);
    sc->tris[i] = Tri{v1, v2 - v1, v3 - v1};
  }
  // quad geometries (Quad.cpp:69-110 tessellation; getNormals,
  // renderer/common.h:266-267): a quad's triangles are shaded with the normal
  // of the triangle whose position in the geometry's list is the quad's index
  if (s->triNormalFrom) {
    sc->triNormal.resize(s->numTriangles);
    sc->hasNormal.assign(s->numTriangles, 0);
    for (int i = 0; i < s->numTriangles; ++i) {
      const int from = s->triNormalFrom[i];
      if (from < 0) continue;
      const Tri &T = sc->tris[from];
      f3 n = cross(T.e1, T.e2);
      const float l = std::sqrt(n.x * n.x + n.y * n.y + n.z * n.z);
      sc->triNormal[i] = f3(n.x / l, n.y / l, n.z / l);
      sc->hasNormal[i] = 1;
    }
  }
  sc->bvh.resize(s->numGroups);
  for (int g = 0; g < s->numGroups; ++g)
    buildBVH(sc->bvh[g], sc->tris, s->groups[g].triBegin, s->groups[g].triEnd);
  sc->vols.resize(s->numVolumes);
  for (int i = 0; i < s->numVolumes; ++i) {
    Vol &v = sc->vols[i];
    v.v = &s->volumes[i];
    f3 org(v.v->origin[0], v.v->origin[1], v.v->origin[2]);
    f3 sp(v.v->spacing[0], v.v->spacing[1], v.v->spacing[2]);
    f3 dims((float)v.v->dims[0], (float)v.v->dims[1], (float)v.v->dims[2]);
    v.bounds.lo = org;
    v.bounds.hi = org + (dims - f3(1.f)) * sp;
    v.S = f3(1.f) / (v.bounds.hi - v.bounds.lo);
    v.T = -v.bounds.lo;
    v.cellSize = min_element(sp);
    buildMajorants(v);
  }
  sc->isoFields.resize(s->numIsos);
  for (int i = 0; i < s->numIsos; ++i) {
    Vol &v = sc->isoFields[i];
    v.v = &s->isoFields[s->isos[i].field];
    f3 org(v.v->origin[0], v.v->origin[1], v.v->origin[2]);
    f3 sp(v.v->spacing[0], v.v->spacing[1], v.v->spacing[2]);
    f3 dims((float)v.v->dims[0], (float)v.v->dims[1], (float)v.v->dims[2]);
    v.bounds.lo = org;
    v.bounds.hi = org + (dims - f3(1.f)) * sp;
    v.S = f3(1.f) / (v.bounds.hi - v.bounds.lo);
    v.T = -v.bounds.lo;
    v.cellSize = min_element(sp);
  }
  sc->insts.resize(s->numInstances);
  for (int i = 0; i < s->numInstances; ++i) {
    const OrInstance &oi = s->instances[i];
    M3 a;
    a.c0 = f3(oi.xfm[0], oi.xfm[1], oi.xfm[2]);
    a.c1 = f3(oi.xfm[3], oi.xfm[4], oi.xfm[5]);
    a.c2 = f3(oi.xfm[6], oi.xfm[7], oi.xfm[8]);
    Inst &in = sc->insts[i];
    in.affineInv = inverse3(a);
    in.transInv = -f3(oi.xfm[9], oi.xfm[10], oi.xfm[11]);
    in.normalXfm = transpose3(in.affineInv);
    in.group = oi.group;
    in.userID = oi.userID;
  }
  return sc;
}

} // namespace

extern "C" {

void *or_scene_commit(const OrScene *scene) { return commit(scene); }
void or_scene_release(void *h) { delete (Scene *)h; }

void or_frame_reset(OrFrame *F) {
  size_t n = size_t(F->width) * F->height;
  if (F->accum) std::fill(F->accum, F->accum + 4 * n, 0.f);
  if (F->depth) std::fill(F->depth, F->depth + n, 1e31f);
  F->accumID = 0;
}

// The history read of the TAA resolve pass: the previous resolved image at
// normalised (u, v), clamp addressing, cardinal-spline (Catmull-Rom) filter
// over 4x4 texels with texel centres at (i + 0.5) / size (the reference's
// history texture, frame/Frame.cpp:541-545).
void catmullRomWeights(float f, float *w) {
  const float f2 = f * f, f3v = f2 * f;
  w[0] = 0.5f * (-f3v + 2.f * f2 - f);
  w[1] = 0.5f * (3.f * f3v - 5.f * f2 + 2.f);
  w[2] = 0.5f * (-3.f * f3v + 4.f * f2 + f);
  w[3] = 0.5f * (f3v - f2);
}

f4 historyAt(const float *img, int W, int H, float u, float v) {
  const float tx = u * (float)W - 0.5f, ty = v * (float)H - 0.5f;
  const float fx0 = std::floor(tx), fy0 = std::floor(ty);
  float wx[4], wy[4];
  catmullRomWeights(tx - fx0, wx);
  catmullRomWeights(ty - fy0, wy);
  const int x0 = (int)fx0 - 1, y0 = (int)fy0 - 1;
  f4 r(0.f);
  for (int j = 0; j < 4; ++j) {
    const int yy = std::min(std::max(y0 + j, 0), H - 1);
    f4 row(0.f);
    for (int i = 0; i < 4; ++i) {
      const int xx = std::min(std::max(x0 + i, 0), W - 1);
      const float *t = img + 4 * (size_t(yy) * W + xx);
      row.x += wx[i] * t[0]; row.y += wx[i] * t[1]; row.z += wx[i] * t[2]; row.w += wx[i] * t[3];
    }
    r.x += wy[j] * row.x; r.y += wy[j] * row.y; r.z += wy[j] * row.z; r.w += wy[j] * row.w;
  }
  return r;
}

// The TAA resolve pass (frame/Frame.cpp:339-381, dco::Frame::accumSample,
// DeviceCopyableObjects.h:2692-2720) over rows [r0, r1): reproject by the
// motion vector, blend with weight taaAlpha (1 where the albedo moved by
// 1e-2 or more), convert into the colour channel; then the frame becomes
// the next one's history.
void taaResolve(const OrRenderer &R, OrFrame &F, int r0, int r1) {
  const int W = F.width, H = F.height;
  for (int y = r0; y < r1; ++y)
    for (int x = 0; x < W; ++x) {
      const size_t idx = size_t(y) * W + x;
      const float mvx = F.motionVec[2 * idx], mvy = F.motionVec[2 * idx + 1];
      int px = (int)((float)x + mvx), py = (int)((float)y + mvy);
      px = std::min(std::max(px, 0), W - 1);
      py = std::min(std::max(py, 0), H - 1);
      const size_t pidx = size_t(py) * W + px;
      float alpha = R.taaAlpha;
      const float *pa = F.taaPrevAlbedo + 3 * pidx, *ca = F.taaCurrAlbedo + 3 * idx;
      if (!(std::fabs(pa[0] - ca[0]) < 1e-2f && std::fabs(pa[1] - ca[1]) < 1e-2f &&
            std::fabs(pa[2] - ca[2]) < 1e-2f))
        alpha = 1.f;
      const float u = ((float)x + mvx + 0.5f) / (float)W, v = ((float)y + mvy + 0.5f) / (float)H;
      const f4 h = historyAt(F.taaPrev, W, H, u, v);
      float *c = F.taaCurr + 4 * idx;
      const f4 o((1.f - alpha) * h.x + alpha * c[0], (1.f - alpha) * h.y + alpha * c[1],
                 (1.f - alpha) * h.z + alpha * c[2], (1.f - alpha) * h.w + alpha * c[3]);
      c[0] = o.x; c[1] = o.y; c[2] = o.z; c[3] = o.w;
      if (F.color) {
        if (F.colorType == OR_COLOR_FLOAT4) {
          float *d = (float *)F.color + 4 * idx;
          d[0] = o.x; d[1] = o.y; d[2] = o.z; d[3] = o.w;
        } else {
          ((uint32_t *)F.color)[idx] = cvtColor(o, F.colorType == OR_COLOR_SRGB8);
        }
      }
    }
  const size_t n = size_t(W) * H;
  std::copy(F.taaCurr, F.taaCurr + 4 * n, F.taaPrev);
  std::copy(F.taaCurrAlbedo, F.taaCurrAlbedo + 3 * n, F.taaPrevAlbedo);
}

int or_render_frame(void *scene, const OrCamera *cam, const OrRenderer *rend, OrFrame *frame,
                    int numThreads, OrStats *stats) {
  if (rend->type == OR_PATHTRACE) {
    // Frame.cpp:315-334: the current view-projection from a perspective or
    // matrix camera; the previous one is the last frame's
    if (cam->type == OR_CAM_PERSPECTIVE) {
      perspectiveViewProj(cam->position, cam->direction, cam->up, cam->fovy, cam->aspect,
                          frame->currMVP);
    } else if (cam->type == OR_CAM_MATRIX) {
      mul44(cam->proj, cam->view, frame->currMVP);
    }
  }
  if (rend->taa && rend->type == OR_PATHTRACE &&
      (!frame->taaCurr || !frame->taaPrev || !frame->taaCurrAlbedo || !frame->taaPrevAlbedo ||
       !frame->motionVec))
    return 1;
  Ctx cx{(const Scene *)scene, makeCam(*cam), rend, frame};
  const int W = frame->width, H = frame->height;
  int r0 = frame->rowBegin, r1 = frame->rowEnd;
  if (r0 == 0 && r1 == 0) r1 = H;
  // 64x64 tiles on a pool of hardware_concurrency() threads (for_each.h:71-85,
  // SyncContext.cpp:21); tests may ask for smaller tiles.
  const int T = frame->tileSize > 0 ? frame->tileSize : 64;
  const int tx = (W + T - 1) / T, ty = (r1 - r0 + T - 1) / T;
  const int ntiles = tx * ty;
  if (numThreads <= 0) numThreads = (int)std::max(1u, std::thread::hardware_concurrency());
  std::atomic<int> next{0};
  std::vector<Counters> cnt(numThreads);
  auto worker = [&](int tid) {
    Counters &c = cnt[tid];
    for (;;) {
      int t = next.fetch_add(1);
      if (t >= ntiles) break;
      int bx = (t % tx) * T, by = r0 + (t / tx) * T;
      for (int y = by; y < std::min(by + T, r1); ++y)
        for (int x = bx; x < std::min(bx + T, W); ++x) {
          if (rend->type == OR_PATHTRACE) pathtracePixel(cx, x, y, c);
          else raycastPixel(cx, x, y, c);
        }
    }
  };
  std::vector<std::thread> th;
  for (int i = 1; i < numThreads; ++i) th.emplace_back(worker, i);
  worker(0);
  for (auto &t : th) t.join();
  if (stats) {
    for (auto &c : cnt) {
      stats->rays += c.rays; stats->nodeVisits += c.nodes; stats->triTests += c.tris;
      stats->marchSamples += c.march; stats->trackingSamples += c.track; stats->cellsVisited += c.cells;
    }
  }
  if (rend->taa && rend->type == OR_PATHTRACE) taaResolve(*rend, *frame, r0, r1);
  if (rend->type == OR_PATHTRACE) std::copy(frame->currMVP, frame->currMVP + 16, frame->prevMVP);
  frame->accumID++;
  return 0;
}

void or_lcg_sequence(uint32_t v0, uint32_t v1, int n, float *out) {
  LCG r(v0, v1);
  for (int i = 0; i < n; ++i) out[i] = r();
}

float or_sample_field(const OrVolume *vol, float px, float py, float pz) {
  return sampleField(vol, f3(px, py, pz));
}

void or_tf_lookup(const OrVolume *vol, float v, float *rgba) {
  f4 c = postClassify(vol, v);
  rgba[0] = c.x; rgba[1] = c.y; rgba[2] = c.z; rgba[3] = c.w;
}

void or_primary_ray(const OrCamera *cam, float x, float y, float w, float h, uint32_t s0,
                    uint32_t s1, float *ori, float *dir) {
  Cam k = makeCam(*cam);
  LCG r(s0, s1);
  Ray ray = primaryRay(k, &r, x, y, w, h);
  ori[0] = ray.ori.x; ori[1] = ray.ori.y; ori[2] = ray.ori.z;
  dir[0] = ray.dir.x; dir[1] = ray.dir.y; dir[2] = ray.dir.z;
}

void or_eval_material(const OrMaterial *mat, const float *Ng, const float *Ns, const float *vd,
                      const float *ld, float *out) {
  (void)Ng;
  f3 r = evalMaterial(*mat, f3(Ns[0], Ns[1], Ns[2]), f3(vd[0], vd[1], vd[2]), f3(ld[0], ld[1], ld[2]));
  out[0] = r.x; out[1] = r.y; out[2] = r.z;
}

void or_sample_material(const OrMaterial *mat, const float *Ng, const float *Ns, const float *vd,
                        uint32_t s0, uint32_t s1, float *dir, float *f, float *pdf, float *cosT) {
  LCG r(s0, s1);
  BSDFSample b = sampleMaterial(*mat, f3(Ng[0], Ng[1], Ng[2]), f3(Ns[0], Ns[1], Ns[2]),
                                f3(vd[0], vd[1], vd[2]), r);
  dir[0] = b.dir.x; dir[1] = b.dir.y; dir[2] = b.dir.z;
  f[0] = b.f.x; f[1] = b.f.y; f[2] = b.f.z;
  *pdf = b.pdf;
  *cosT = b.cosT;
}

int or_majorants(void *scene, int vol, int32_t *dims, float *out, int maxCells) {
  const Scene *sc = (const Scene *)scene;
  const Vol &v = sc->vols[vol];
  for (int a = 0; a < 3; ++a) dims[a] = v.gdims[a];
  int n = (int)v.maxOpacity.size();
  for (int i = 0; i < n && i < maxCells; ++i) out[i] = v.maxOpacity[i];
  return n;
}

void or_cvt(const float *rgba, int n, int srgb, uint32_t *out) {
  for (int i = 0; i < n; ++i)
    out[i] = cvtColor(f4(rgba[4 * i], rgba[4 * i + 1], rgba[4 * i + 2], rgba[4 * i + 3]), srgb != 0);
}

int or_dda(const float *ori, const float *dir, float tmin, float tmax, const int32_t *dims,
           const float *lo, const float *hi, int32_t *cells, float *t01, int maxCells) {
  Ray r;
  r.ori = f3(ori[0], ori[1], ori[2]);
  r.dir = f3(dir[0], dir[1], dir[2]);
  r.tmin = tmin;
  r.tmax = tmax;
  Box b;
  b.lo = f3(lo[0], lo[1], lo[2]);
  b.hi = f3(hi[0], hi[1], hi[2]);
  int d[3] = {dims[0], dims[1], dims[2]};
  int n = 0;
  dda3(r, d, b, [&](int id, float t0, float t1) {
    if (n < maxCells) { cells[n] = id; t01[2 * n] = t0; t01[2 * n + 1] = t1; }
    ++n;
    return n < 1000000;
  });
  return n;
}

int or_trace(void *scene, const float *ori, const float *dir, float tmin, float tmax, float *t,
             uint32_t *inst, uint32_t *tri, float *uv) {
  const Scene *sc = (const Scene *)scene;
  Ray r;
  r.ori = f3(ori[0], ori[1], ori[2]);
  r.dir = f3(dir[0], dir[1], dir[2]);
  r.tmin = tmin;
  r.tmax = tmax;
  r.time = 0.5f;
  Counters c;
  SurfHit h = traceSurfaces(*sc, r, c);
  *t = h.t;
  *inst = (uint32_t)h.inst;
  *tri = (uint32_t)h.tri;
  uv[0] = h.u;
  uv[1] = h.v;
  return h.hit ? 1 : 0;
}

} // extern "C"
