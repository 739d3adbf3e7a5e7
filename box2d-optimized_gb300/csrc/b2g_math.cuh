// b2g_math.cuh - float arithmetic of the Step path, callable from host and device.
//
// Every routine performs the reference's float operations in the reference's order
// (include/box2d/b2_math.h, src/collision/*, src/dynamics/b2_contact_solver.cpp, joints), so
// that with contraction disabled (nvcc --fmad=false, host -ffp-contract=off) and IEEE division
// and square root, the GPU produces the same bits as a CPU evaluation of the same formulas.
// The only deliberate difference from the reference is b2Rot::Set: sine and cosine come from
// b2g_sincos below, a portable routine that gives identical results on host and device.
#pragma once

#include <stdint.h>

#include "../../include/b2g_capi.h"

#ifdef __CUDACC__
#define B2G_HD __host__ __device__ __forceinline__
#else
#define B2G_HD inline
#include <math.h>
#endif

namespace b2g {

// Tuning constants (include/box2d/b2_common.h:39-41, 110-182)
#define B2G_MAX_FLOAT 3.402823466e+38f
#define B2G_EPSILON 1.192092896e-07f
#define B2G_PI 3.14159265359f
#define B2G_LINEAR_SLOP 0.005f
#define B2G_ANGULAR_SLOP (2.0f / 180.0f * B2G_PI)
#define B2G_POLYGON_RADIUS (2.0f * B2G_LINEAR_SLOP)
#define B2G_MAX_LINEAR_CORRECTION 0.2f
#define B2G_MAX_ANGULAR_CORRECTION (8.0f / 180.0f * B2G_PI)
#define B2G_MAX_TRANSLATION 2.0f
#define B2G_MAX_TRANSLATION_SQ (B2G_MAX_TRANSLATION * B2G_MAX_TRANSLATION)
#define B2G_MAX_ROTATION (0.5f * B2G_PI)
#define B2G_MAX_ROTATION_SQ (B2G_MAX_ROTATION * B2G_MAX_ROTATION)
#define B2G_BAUMGARTE 0.2f

struct V2 {
  float x, y;
};
B2G_HD V2 mk(float x, float y) { V2 r; r.x = x; r.y = y; return r; }
B2G_HD V2 operator+(V2 a, V2 b) { return mk(a.x + b.x, a.y + b.y); }
B2G_HD V2 operator-(V2 a, V2 b) { return mk(a.x - b.x, a.y - b.y); }
B2G_HD V2 operator-(V2 a) { return mk(-a.x, -a.y); }
B2G_HD V2 operator*(float s, V2 a) { return mk(s * a.x, s * a.y); }
B2G_HD void addTo(V2& a, V2 b) { a.x += b.x; a.y += b.y; }
B2G_HD void subFrom(V2& a, V2 b) { a.x -= b.x; a.y -= b.y; }
B2G_HD float dot(V2 a, V2 b) { return a.x * b.x + a.y * b.y; }
B2G_HD float cross(V2 a, V2 b) { return a.x * b.y - a.y * b.x; }
B2G_HD V2 cross(V2 a, float s) { return mk(s * a.y, -s * a.x); }
B2G_HD V2 cross(float s, V2 a) { return mk(-s * a.y, s * a.x); }
B2G_HD float lengthOf(V2 a) { return sqrtf(a.x * a.x + a.y * a.y); }
B2G_HD float lengthSq(V2 a) { return a.x * a.x + a.y * a.y; }
B2G_HD float distSq(V2 a, V2 b) { V2 c = a - b; return c.x * c.x + c.y * c.y; }
// b2Vec2::Normalize (b2_math.h:117-130)
B2G_HD float normalize(V2& a) {
  float length = lengthOf(a);
  if (length < B2G_EPSILON) return 0.0f;
  float inv = 1.0f / length;
  a.x *= inv;
  a.y *= inv;
  return length;
}
B2G_HD float fmin2(float a, float b) { return a < b ? a : b; }
B2G_HD float fmax2(float a, float b) { return a > b ? a : b; }
B2G_HD float fclamp(float a, float lo, float hi) { return fmax2(lo, fmin2(a, hi)); }
B2G_HD float fabs2(float a) { return a > 0.0f ? a : -a; }
B2G_HD int imin2(int a, int b) { return a < b ? a : b; }
B2G_HD V2 vmin(V2 a, V2 b) { return mk(fmin2(a.x, b.x), fmin2(a.y, b.y)); }
B2G_HD V2 vmax(V2 a, V2 b) { return mk(fmax2(a.x, b.x), fmax2(a.y, b.y)); }

struct Rot { float s, c; };
struct Xf { V2 p; Rot q; };
B2G_HD V2 mul(Rot q, V2 v) { return mk(q.c * v.x - q.s * v.y, q.s * v.x + q.c * v.y); }
B2G_HD V2 mulT(Rot q, V2 v) { return mk(q.c * v.x + q.s * v.y, -q.s * v.x + q.c * v.y); }
B2G_HD V2 mul(const Xf& T, V2 v) {
  float x = (T.q.c * v.x - T.q.s * v.y) + T.p.x;
  float y = (T.q.s * v.x + T.q.c * v.y) + T.p.y;
  return mk(x, y);
}
B2G_HD V2 mulT(const Xf& T, V2 v) {
  float px = v.x - T.p.x;
  float py = v.y - T.p.y;
  float x = (T.q.c * px + T.q.s * py);
  float y = (-T.q.s * px + T.q.c * py);
  return mk(x, y);
}
B2G_HD Rot mulT(Rot q, Rot r) {
  Rot o;
  o.s = q.c * r.s - q.s * r.c;
  o.c = q.c * r.c + q.s * r.s;
  return o;
}
B2G_HD Xf mulT(const Xf& A, const Xf& B) {
  Xf C;
  C.q = mulT(A.q, B.q);
  C.p = mulT(A.q, B.p - A.p);
  return C;
}

// b2Mat22 (b2_math.h:184-256)
struct M22 { V2 ex, ey; };
B2G_HD M22 inverse(const M22& m) {
  float a = m.ex.x, b = m.ey.x, c = m.ex.y, d = m.ey.y;
  M22 B;
  float det = a * d - b * c;
  if (det != 0.0f) det = 1.0f / det;
  B.ex.x = det * d;  B.ey.x = -det * b;
  B.ex.y = -det * c; B.ey.y = det * a;
  return B;
}
B2G_HD V2 solve(const M22& m, V2 b) {
  float a11 = m.ex.x, a12 = m.ey.x, a21 = m.ex.y, a22 = m.ey.y;
  float det = a11 * a22 - a12 * a21;
  if (det != 0.0f) det = 1.0f / det;
  V2 x;
  x.x = det * (a22 * b.x - a12 * b.y);
  x.y = det * (a11 * b.y - a21 * b.x);
  return x;
}
B2G_HD V2 mul(const M22& A, V2 v) { return mk(A.ex.x * v.x + A.ey.x * v.y, A.ex.y * v.x + A.ey.y * v.y); }

struct V3 { float x, y, z; };
B2G_HD float dot3(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
B2G_HD V3 cross3(V3 a, V3 b) {
  V3 r; r.x = a.y * b.z - a.z * b.y; r.y = a.z * b.x - a.x * b.z; r.z = a.x * b.y - a.y * b.x; return r;
}
// b2Mat33::Solve33 (src/common/b2_math.cpp:28-40)
B2G_HD V3 solve33(V3 ex, V3 ey, V3 ez, V3 b) {
  float det = dot3(ex, cross3(ey, ez));
  if (det != 0.0f) det = 1.0f / det;
  V3 x;
  x.x = det * dot3(b, cross3(ey, ez));
  x.y = det * dot3(ex, cross3(b, ez));
  x.z = det * dot3(ex, cross3(ey, b));
  return x;
}

// ---- GJK distance for sensors: b2TestOverlap (src/collision/b2_collision.cpp:239-258) over
// b2Distance (src/collision/b2_distance.cpp:432-579) with an empty simplex cache and radii.
struct SimplexVertex { V2 wA, wB, w; float a; int indexA, indexB; };
B2G_HD int proxyCount(const b2g_shape& s) {
  return s.type == B2G_SHAPE_CIRCLE ? 1 : (s.type == B2G_SHAPE_EDGE ? 2 : s.count);
}
B2G_HD V2 proxyVertex(const b2g_shape& s, int i) { return mk(s.vertices[i][0], s.vertices[i][1]); }
// b2DistanceProxy::GetSupport (include/box2d/b2_distance.h:137-152)
B2G_HD int proxySupport(const b2g_shape& s, V2 d) {
  const int n = proxyCount(s);
  int bestIndex = 0;
  float bestValue = dot(proxyVertex(s, 0), d);
  for (int i = 1; i < n; ++i) {
    float value = dot(proxyVertex(s, i), d);
    if (value > bestValue) {
      bestIndex = i;
      bestValue = value;
    }
  }
  return bestIndex;
}
// b2Simplex::Solve2 (b2_distance.cpp:284-321); v holds m_v1, m_v2, m_v3
B2G_HD void simplexSolve2(SimplexVertex* v, int& count) {
  V2 w1 = v[0].w, w2 = v[1].w;
  V2 e12 = w2 - w1;
  float d12_2 = -dot(w1, e12);
  if (d12_2 <= 0.0f) {
    v[0].a = 1.0f;
    count = 1;
    return;
  }
  float d12_1 = dot(w2, e12);
  if (d12_1 <= 0.0f) {
    v[1].a = 1.0f;
    count = 1;
    v[0] = v[1];
    return;
  }
  float inv_d12 = 1.0f / (d12_1 + d12_2);
  v[0].a = d12_1 * inv_d12;
  v[1].a = d12_2 * inv_d12;
  count = 2;
}
// b2Simplex::Solve3 (b2_distance.cpp:323-430)
B2G_HD void simplexSolve3(SimplexVertex* v, int& count) {
  V2 w1 = v[0].w, w2 = v[1].w, w3 = v[2].w;
  V2 e12 = w2 - w1;
  float w1e12 = dot(w1, e12);
  float w2e12 = dot(w2, e12);
  float d12_1 = w2e12;
  float d12_2 = -w1e12;
  V2 e13 = w3 - w1;
  float w1e13 = dot(w1, e13);
  float w3e13 = dot(w3, e13);
  float d13_1 = w3e13;
  float d13_2 = -w1e13;
  V2 e23 = w3 - w2;
  float w2e23 = dot(w2, e23);
  float w3e23 = dot(w3, e23);
  float d23_1 = w3e23;
  float d23_2 = -w2e23;
  float n123 = cross(e12, e13);
  float d123_1 = n123 * cross(w2, w3);
  float d123_2 = n123 * cross(w3, w1);
  float d123_3 = n123 * cross(w1, w2);
  if (d12_2 <= 0.0f && d13_2 <= 0.0f) {
    v[0].a = 1.0f;
    count = 1;
    return;
  }
  if (d12_1 > 0.0f && d12_2 > 0.0f && d123_3 <= 0.0f) {
    float inv_d12 = 1.0f / (d12_1 + d12_2);
    v[0].a = d12_1 * inv_d12;
    v[1].a = d12_2 * inv_d12;
    count = 2;
    return;
  }
  if (d13_1 > 0.0f && d13_2 > 0.0f && d123_2 <= 0.0f) {
    float inv_d13 = 1.0f / (d13_1 + d13_2);
    v[0].a = d13_1 * inv_d13;
    v[2].a = d13_2 * inv_d13;
    count = 2;
    v[1] = v[2];
    return;
  }
  if (d12_1 <= 0.0f && d23_2 <= 0.0f) {
    v[1].a = 1.0f;
    count = 1;
    v[0] = v[1];
    return;
  }
  if (d13_1 <= 0.0f && d23_1 <= 0.0f) {
    v[2].a = 1.0f;
    count = 1;
    v[0] = v[2];
    return;
  }
  if (d23_1 > 0.0f && d23_2 > 0.0f && d123_1 <= 0.0f) {
    float inv_d23 = 1.0f / (d23_1 + d23_2);
    v[1].a = d23_1 * inv_d23;
    v[2].a = d23_2 * inv_d23;
    count = 2;
    v[0] = v[2];
    return;
  }
  float inv_d123 = 1.0f / (d123_1 + d123_2 + d123_3);
  v[0].a = d123_1 * inv_d123;
  v[1].a = d123_2 * inv_d123;
  v[2].a = d123_3 * inv_d123;
  count = 3;
}
// The GJK distance between the shapes' cores (radii applied as b2Distance's useRadii).
B2G_HD float shapeDistance(const b2g_shape& A, const Xf& xfA, const b2g_shape& B, const Xf& xfB) {
  SimplexVertex v[3];
  v[0].indexA = 0;
  v[0].indexB = 0;
  v[0].wA = mul(xfA, proxyVertex(A, 0));
  v[0].wB = mul(xfB, proxyVertex(B, 0));
  v[0].w = v[0].wB - v[0].wA;
  v[0].a = 1.0f;
  int count = 1;
  int saveA[3], saveB[3];
  for (int iter = 0; iter < 20;) {
    const int saveCount = count;
    for (int i = 0; i < saveCount; ++i) {
      saveA[i] = v[i].indexA;
      saveB[i] = v[i].indexB;
    }
    if (count == 2) simplexSolve2(v, count);
    else if (count == 3) simplexSolve3(v, count);
    if (count == 3) break;
    V2 d;
    if (count == 1) {
      d = -v[0].w;
    } else {
      V2 e12 = v[1].w - v[0].w;
      float sgn = cross(e12, -v[0].w);
      d = sgn > 0.0f ? cross(1.0f, e12) : cross(e12, 1.0f);
    }
    if (lengthSq(d) < B2G_EPSILON * B2G_EPSILON) break;
    SimplexVertex& nv = v[count];
    nv.indexA = proxySupport(A, mulT(xfA.q, -d));
    nv.wA = mul(xfA, proxyVertex(A, nv.indexA));
    nv.indexB = proxySupport(B, mulT(xfB.q, d));
    nv.wB = mul(xfB, proxyVertex(B, nv.indexB));
    nv.w = nv.wB - nv.wA;
    ++iter;
    bool duplicate = false;
    for (int i = 0; i < saveCount; ++i) {
      if (nv.indexA == saveA[i] && nv.indexB == saveB[i]) {
        duplicate = true;
        break;
      }
    }
    if (duplicate) break;
    ++count;
  }
  V2 pA, pB;
  if (count == 1) {
    pA = v[0].wA;
    pB = v[0].wB;
  } else if (count == 2) {
    pA = v[0].a * v[0].wA + v[1].a * v[1].wA;
    pB = v[0].a * v[0].wB + v[1].a * v[1].wB;
  } else {
    pA = (v[0].a * v[0].wA + v[1].a * v[1].wA) + v[2].a * v[2].wA;
    pB = pA;
  }
  float distance = lengthOf(pA - pB);
  const float rA = A.radius, rB = B.radius;
  if (distance > rA + rB && distance > B2G_EPSILON) return distance - (rA + rB);
  return 0.0f;
}
B2G_HD bool testOverlap(const b2g_shape& A, const Xf& xfA, const b2g_shape& B, const Xf& xfB) {
  return shapeDistance(A, xfA, B, xfB) < 10.0f * B2G_EPSILON;
}

// ---- portable sine/cosine ------------------------------------------------------------------
// Cody & Waite reduction of x by pi/2 (pi/2 split into two 12-bit parts and a float remainder,
// so k*part is exact for |k| < 4096, i.e. |x| < ~6400 rad) and the Taylor series of sin (to
// x^9) and cos (to x^10) on |r| <= pi/4 by Horner's rule; truncation error < 3e-9 relative.
// Identical operation sequence on host and device: rintf rounds half to even on both.
B2G_HD void sincos_portable(float x, float* s_out, float* c_out) {
  const float kTwoOverPi = 0.636619772367581343f;
  const float kA = 1.5703125f;
  const float kB = 4.8351287841796875e-04f;
  const float kC = 3.13916473e-07f;
  float k = rintf(x * kTwoOverPi);
  float r = x - k * kA;
  r = r - k * kB;
  r = r - k * kC;
  float z = r * r;
  float s = r + (r * z) * (-1.66666667e-01f + z * (8.33333333e-03f + z * (-1.98412698e-04f + z * 2.75573192e-06f)));
  float c = 1.0f + z * (-0.5f + z * (4.16666667e-02f + z * (-1.38888889e-03f + z * (2.48015873e-05f + z * -2.75573192e-07f))));
  long long ki = (long long)k;
  int q = (int)(ki & 3);
  if (q == 0) { *s_out = s; *c_out = c; }
  else if (q == 1) { *s_out = c; *c_out = -s; }
  else if (q == 2) { *s_out = -s; *c_out = -c; }
  else { *s_out = -c; *c_out = s; }
}
B2G_HD Rot rotOf(float angle) {
  Rot q;
  sincos_portable(angle, &q.s, &q.c);
  return q;
}

// ---- shapes --------------------------------------------------------------------------------
B2G_HD V2 sv(const b2g_shape& s, int i) { return mk(s.vertices[i][0], s.vertices[i][1]); }
B2G_HD V2 sn(const b2g_shape& s, int i) { return mk(s.normals[i][0], s.normals[i][1]); }

struct AABB { V2 lo, hi; };

// ComputeAABB: polygon (src/collision/b2_polygon_shape.cpp:373-388), circle
// (b2_circle_shape.cpp:91-96), edge (b2_edge_shape.cpp:156-167).
B2G_HD AABB shapeAABB(const b2g_shape& s, const Xf& xf) {
  AABB bb;
  if (s.type == B2G_SHAPE_CIRCLE) {
    V2 p = xf.p + mul(xf.q, sv(s, 0));
    bb.lo = mk(p.x - s.radius, p.y - s.radius);
    bb.hi = mk(p.x + s.radius, p.y + s.radius);
    return bb;
  }
  if (s.type == B2G_SHAPE_EDGE) {
    V2 a = mul(xf, sv(s, 0));
    V2 b = mul(xf, sv(s, 1));
    V2 r = mk(s.radius, s.radius);
    bb.lo = vmin(a, b) - r;
    bb.hi = vmax(a, b) + r;
    return bb;
  }
  V2 lower = mul(xf, sv(s, 0));
  V2 upper = lower;
  for (int i = 1; i < s.count; ++i) {
    V2 v = mul(xf, sv(s, i));
    lower = vmin(lower, v);
    upper = vmax(upper, v);
  }
  V2 r = mk(s.radius, s.radius);
  bb.lo = lower - r;
  bb.hi = upper + r;
  return bb;
}

// b2TestOverlap(const b2AABB&, const b2AABB&), include/box2d/b2_collision.h:270-276
B2G_HD bool overlap(const AABB& a, const AABB& b) {
  return (a.hi.x >= b.lo.x) & (a.lo.x <= b.hi.x) & (a.hi.y >= b.lo.y) & (a.lo.y <= b.hi.y);
}

// ---- ray casts ---------------------------------------------------------------------------
// b2RayCastOutput: where along p1 -> p2 the ray enters the shape, and the surface normal there.
struct RayHit {
  float fraction;
  V2 normal;
};

// b2PolygonShape::RayCast (src/collision/b2_polygon_shape.cpp:303-364): clip the parametric
// segment against every face's half-space in the polygon's frame; a hit needs an entering face.
B2G_HD bool rayPolygon(const b2g_shape& s, const Xf& xf, V2 P1, V2 P2, float maxFraction, RayHit* out) {
  V2 p1 = mulT(xf.q, P1 - xf.p);
  V2 p2 = mulT(xf.q, P2 - xf.p);
  V2 d = p2 - p1;
  float lower = 0.0f, upper = maxFraction;
  int index = -1;
  for (int i = 0; i < s.count; ++i) {
    float numerator = dot(sn(s, i), sv(s, i) - p1);
    float denominator = dot(sn(s, i), d);
    if (denominator == 0.0f) {
      if (numerator < 0.0f) return false;
    } else if (denominator < 0.0f && numerator < lower * denominator) {
      lower = numerator / denominator;  // the segment enters this half-space
      index = i;
    } else if (denominator > 0.0f && numerator < upper * denominator) {
      upper = numerator / denominator;  // ... and leaves this one
    }
    if (upper < lower) return false;
  }
  if (index < 0) return false;
  out->fraction = lower;
  out->normal = mul(xf.q, sn(s, index));
  return true;
}

// b2CircleShape::RayCast (src/collision/b2_circle_shape.cpp:56-87): the smaller root of
// |p1 + t r - c|^2 = radius^2, accepted on [0, maxFraction].
B2G_HD bool rayCircle(const b2g_shape& s, const Xf& xf, V2 P1, V2 P2, float maxFraction, RayHit* out) {
  V2 position = xf.p + mul(xf.q, sv(s, 0));
  V2 d = P1 - position;
  float b = dot(d, d) - s.radius * s.radius;
  V2 r = P2 - P1;
  float c = dot(d, r);
  float rr = dot(r, r);
  float sigma = c * c - rr * b;
  if (sigma < 0.0f || rr < B2G_EPSILON) return false;
  float a = -(c + sqrtf(sigma));
  if (!(0.0f <= a && a <= maxFraction * rr)) return false;
  a /= rr;
  out->fraction = a;
  V2 n = d + a * r;
  normalize(n);
  out->normal = n;
  return true;
}

// b2EdgeShape::RayCast (src/collision/b2_edge_shape.cpp:89-149): crossing of the edge's line,
// kept when it lies on the segment and the edge; one-sided edges ignore rays from behind.
B2G_HD bool rayEdge(const b2g_shape& s, const Xf& xf, V2 P1, V2 P2, float maxFraction, RayHit* out) {
  V2 p1 = mulT(xf.q, P1 - xf.p);
  V2 p2 = mulT(xf.q, P2 - xf.p);
  V2 d = p2 - p1;
  V2 v1 = sv(s, 0), v2 = sv(s, 1);
  V2 e = v2 - v1;
  V2 normal = mk(e.y, -e.x);  // to the right, looking from v1 at v2
  normalize(normal);
  float numerator = dot(normal, v1 - p1);
  if (s.one_sided && numerator > 0.0f) return false;
  float denominator = dot(normal, d);
  if (denominator == 0.0f) return false;
  float t = numerator / denominator;
  if (t < 0.0f || maxFraction < t) return false;
  V2 q = p1 + t * d;
  V2 r = v2 - v1;
  float rr = dot(r, r);
  if (rr == 0.0f) return false;
  float sc = dot(q - v1, r) / rr;
  if (sc < 0.0f || 1.0f < sc) return false;
  out->fraction = t;
  out->normal = numerator > 0.0f ? -mul(xf.q, normal) : mul(xf.q, normal);
  return true;
}

B2G_HD bool rayShape(const b2g_shape& s, const Xf& xf, V2 p1, V2 p2, float maxFraction, RayHit* out) {
  if (s.type == B2G_SHAPE_CIRCLE) return rayCircle(s, xf, p1, p2, maxFraction, out);
  if (s.type == B2G_SHAPE_EDGE) return rayEdge(s, xf, p1, p2, maxFraction, out);
  return rayPolygon(s, xf, p1, p2, maxFraction, out);
}

// The pruning tests b2BroadPhase::RayCast applies to a tree node's box
// (include/box2d/b2_broad_phase.h:646-710): overlap with the box of the segment so far, then the
// separating axis |dot(v, p1 - c)| > dot(|v|, h), v the segment's unit normal. True = skip.
B2G_HD bool rayPrunes(const AABB& box, const AABB& segment, V2 p1, V2 v, V2 absV) {
  if (!overlap(box, segment)) return true;
  V2 c = 0.5f * (box.lo + box.hi);
  V2 h = 0.5f * (box.hi - box.lo);
  float separation = fabs2(dot(v, p1 - c)) - dot(absV, h);
  return separation > 0.0f;
}

// Box of the segment p1 -> p1 + maxFraction (p2 - p1).
B2G_HD AABB raySegmentBox(V2 p1, V2 p2, float maxFraction) {
  V2 t = p1 + maxFraction * (p2 - p1);
  AABB bb;
  bb.lo = vmin(p1, t);
  bb.hi = vmax(p1, t);
  return bb;
}

// Collider dispatch of b2Contact::InitializeRegisters (src/dynamics/b2_contact.cpp:46-56).
B2G_HD bool hasCollider(int ta, int tb) {
  return (ta == 0 && tb == 0) || (ta == 2 && tb == 0) || (ta == 2 && tb == 2) || (ta == 1 && tb == 0) ||
         (ta == 1 && tb == 2);
}

// ---- narrowphase ---------------------------------------------------------------------------
B2G_HD uint32_t makeId(int indexA, int indexB, int typeA, int typeB) {
  return (uint32_t)(uint8_t)indexA | ((uint32_t)(uint8_t)indexB << 8) | ((uint32_t)(uint8_t)typeA << 16) |
         ((uint32_t)(uint8_t)typeB << 24);
}
B2G_HD uint32_t swapId(uint32_t id) {
  return ((id >> 8) & 0xffu) | ((id & 0xffu) << 8) | (((id >> 24) & 0xffu) << 16) | (((id >> 16) & 0xffu) << 24);
}
#define B2G_FEATURE_VERTEX 0
#define B2G_FEATURE_FACE 1

struct ClipVertex { V2 v; uint32_t id; };

// Manifold in registers; written out as b2g_manifold.
struct Man {
  V2 lp[2];
  uint32_t id[2];
  V2 localNormal, localPoint;
  int type, pointCount;
};

// b2ClipSegmentToLine (src/collision/b2_collision.cpp:205-237)
B2G_HD int clipSegmentToLine(ClipVertex vOut[2], const ClipVertex vIn[2], V2 normal, float offset, int vertexIndexA) {
  int count = 0;
  float distance0 = dot(normal, vIn[0].v) - offset;
  float distance1 = dot(normal, vIn[1].v) - offset;
  if (distance0 <= 0.0f) vOut[count++] = vIn[0];
  if (distance1 <= 0.0f) vOut[count++] = vIn[1];
  if (distance0 * distance1 < 0.0f) {
    float interp = distance0 / (distance0 - distance1);
    vOut[count].v = vIn[0].v + interp * (vIn[1].v - vIn[0].v);
    vOut[count].id = makeId(vertexIndexA, (int)((vIn[0].id >> 8) & 0xff), B2G_FEATURE_VERTEX, B2G_FEATURE_FACE);
    ++count;
  }
  return count;
}

// b2CollideCircles (src/collision/b2_collide_circle.cpp:27-53)
B2G_HD void collideCircles(Man* m, const b2g_shape& A, const Xf& xfA, const b2g_shape& B, const Xf& xfB) {
  m->pointCount = 0;
  V2 pA = mul(xfA, sv(A, 0));
  V2 pB = mul(xfB, sv(B, 0));
  V2 d = pB - pA;
  float distSqr = dot(d, d);
  float radius = A.radius + B.radius;
  if (distSqr > radius * radius) return;
  m->type = B2G_MANIFOLD_CIRCLES;
  m->localPoint = sv(A, 0);
  m->localNormal = mk(0.0f, 0.0f);
  m->pointCount = 1;
  m->lp[0] = sv(B, 0);
  m->id[0] = 0;
}

// b2CollidePolygonAndCircle (src/collision/b2_collide_circle.cpp:55-158)
B2G_HD void collidePolygonAndCircle(Man* m, const b2g_shape& P, const Xf& xfA, const b2g_shape& Cs, const Xf& xfB) {
  m->pointCount = 0;
  V2 c = mul(xfB, sv(Cs, 0));
  V2 cLocal = mulT(xfA, c);
  int normalIndex = 0;
  float separation = -B2G_MAX_FLOAT;
  float radius = P.radius + Cs.radius;
  int vertexCount = P.count;
  for (int i = 0; i < vertexCount; ++i) {
    float s = dot(sn(P, i), cLocal - sv(P, i));
    if (s > radius) return;
    if (s > separation) { separation = s; normalIndex = i; }
  }
  int vertIndex1 = normalIndex;
  int vertIndex2 = vertIndex1 + 1 < vertexCount ? vertIndex1 + 1 : 0;
  V2 v1 = sv(P, vertIndex1);
  V2 v2 = sv(P, vertIndex2);
  if (separation < B2G_EPSILON) {
    m->pointCount = 1;
    m->type = B2G_MANIFOLD_FACE_A;
    m->localNormal = sn(P, normalIndex);
    m->localPoint = 0.5f * (v1 + v2);
    m->lp[0] = sv(Cs, 0);
    m->id[0] = 0;
    return;
  }
  float u1 = dot(cLocal - v1, v2 - v1);
  float u2 = dot(cLocal - v2, v1 - v2);
  if (u1 <= 0.0f) {
    if (distSq(cLocal, v1) > radius * radius) return;
    m->pointCount = 1;
    m->type = B2G_MANIFOLD_FACE_A;
    m->localNormal = cLocal - v1;
    normalize(m->localNormal);
    m->localPoint = v1;
  } else if (u2 <= 0.0f) {
    if (distSq(cLocal, v2) > radius * radius) return;
    m->pointCount = 1;
    m->type = B2G_MANIFOLD_FACE_A;
    m->localNormal = cLocal - v2;
    normalize(m->localNormal);
    m->localPoint = v2;
  } else {
    V2 faceCenter = 0.5f * (v1 + v2);
    float s = dot(cLocal - faceCenter, sn(P, vertIndex1));
    if (s > radius) return;
    m->pointCount = 1;
    m->type = B2G_MANIFOLD_FACE_A;
    m->localNormal = sn(P, vertIndex1);
    m->localPoint = faceCenter;
  }
  m->lp[0] = sv(Cs, 0);
  m->id[0] = 0;
}

// b2FindMaxSeparation (src/collision/b2_collide_polygon.cpp:27-66)
B2G_HD float findMaxSeparation(int* edgeIndex, const b2g_shape& p1, const Xf& xf1, const b2g_shape& p2,
                               const Xf& xf2) {
  int count1 = p1.count;
  int count2 = p2.count;
  Xf xf = mulT(xf2, xf1);
  int bestIndex = 0;
  float maxSeparation = -B2G_MAX_FLOAT;
  for (int i = 0; i < count1; ++i) {
    V2 n = mul(xf.q, sn(p1, i));
    V2 v1 = mul(xf, sv(p1, i));
    float si = B2G_MAX_FLOAT;
    for (int j = 0; j < count2; ++j) {
      float sij = dot(n, sv(p2, j) - v1);
      if (sij < si) si = sij;
    }
    if (si > maxSeparation) { maxSeparation = si; bestIndex = i; }
  }
  *edgeIndex = bestIndex;
  return maxSeparation;
}

// b2FindIncidentEdge (src/collision/b2_collide_polygon.cpp:68-111)
B2G_HD void findIncidentEdge(ClipVertex c[2], const b2g_shape& p1, const Xf& xf1, int edge1, const b2g_shape& p2,
                             const Xf& xf2) {
  V2 normal1 = mulT(xf2.q, mul(xf1.q, sn(p1, edge1)));
  int index = 0;
  float minDot = B2G_MAX_FLOAT;
  for (int i = 0; i < p2.count; ++i) {
    float d = dot(normal1, sn(p2, i));
    if (d < minDot) { minDot = d; index = i; }
  }
  int i1 = index;
  int i2 = i1 + 1 < p2.count ? i1 + 1 : 0;
  c[0].v = mul(xf2, sv(p2, i1));
  c[0].id = makeId(edge1, i1, B2G_FEATURE_FACE, B2G_FEATURE_VERTEX);
  c[1].v = mul(xf2, sv(p2, i2));
  c[1].id = makeId(edge1, i2, B2G_FEATURE_FACE, B2G_FEATURE_VERTEX);
}

// b2CollidePolygons (src/collision/b2_collide_polygon.cpp:120-243)
B2G_HD void collidePolygons(Man* m, const b2g_shape& A, const Xf& xfA, const b2g_shape& B, const Xf& xfB) {
  m->pointCount = 0;
  float totalRadius = A.radius + B.radius;
  int edgeA = 0;
  float separationA = findMaxSeparation(&edgeA, A, xfA, B, xfB);
  if (separationA > totalRadius) return;
  int edgeB = 0;
  float separationB = findMaxSeparation(&edgeB, B, xfB, A, xfA);
  if (separationB > totalRadius) return;
  const float k_tol = 0.1f * B2G_LINEAR_SLOP;
  bool flip = separationB > separationA + k_tol;
  const b2g_shape& poly1 = flip ? B : A;
  const b2g_shape& poly2 = flip ? A : B;
  Xf xf1 = flip ? xfB : xfA;
  Xf xf2 = flip ? xfA : xfB;
  int edge1 = flip ? edgeB : edgeA;
  m->type = flip ? B2G_MANIFOLD_FACE_B : B2G_MANIFOLD_FACE_A;
  ClipVertex incidentEdge[2];
  findIncidentEdge(incidentEdge, poly1, xf1, edge1, poly2, xf2);
  int count1 = poly1.count;
  int iv1 = edge1;
  int iv2 = edge1 + 1 < count1 ? edge1 + 1 : 0;
  V2 v11 = sv(poly1, iv1);
  V2 v12 = sv(poly1, iv2);
  V2 localTangent = v12 - v11;
  normalize(localTangent);
  V2 localNormal = cross(localTangent, 1.0f);
  V2 planePoint = 0.5f * (v11 + v12);
  V2 tangent = mul(xf1.q, localTangent);
  V2 normal = cross(tangent, 1.0f);
  v11 = mul(xf1, v11);
  v12 = mul(xf1, v12);
  float frontOffset = dot(normal, v11);
  float sideOffset1 = -dot(tangent, v11) + totalRadius;
  float sideOffset2 = dot(tangent, v12) + totalRadius;
  ClipVertex clipPoints1[2];
  ClipVertex clipPoints2[2];
  int np = clipSegmentToLine(clipPoints1, incidentEdge, -tangent, sideOffset1, iv1);
  if (np < 2) return;
  np = clipSegmentToLine(clipPoints2, clipPoints1, tangent, sideOffset2, iv2);
  if (np < 2) return;
  m->localNormal = localNormal;
  m->localPoint = planePoint;
  int pointCount = 0;
  for (int i = 0; i < 2; ++i) {
    float separation = dot(normal, clipPoints2[i].v) - frontOffset;
    if (separation <= totalRadius) {
      m->lp[pointCount] = mulT(xf2, clipPoints2[i].v);
      m->id[pointCount] = flip ? swapId(clipPoints2[i].id) : clipPoints2[i].id;
      ++pointCount;
    }
  }
  m->pointCount = pointCount;
}

// b2CollideEdgeAndCircle (src/collision/b2_collide_edge.cpp:31-165)
B2G_HD void collideEdgeAndCircle(Man* m, const b2g_shape& E, const Xf& xfA, const b2g_shape& Cs, const Xf& xfB) {
  m->pointCount = 0;
  V2 Q = mulT(xfA, mul(xfB, sv(Cs, 0)));
  V2 A = sv(E, 0), B = sv(E, 1);
  V2 e = B - A;
  V2 n = mk(e.y, -e.x);
  float offset = dot(n, Q - A);
  bool oneSided = E.one_sided != 0;
  if (oneSided && offset < 0.0f) return;
  float u = dot(e, B - Q);
  float v = dot(e, Q - A);
  float radius = E.radius + Cs.radius;
  if (v <= 0.0f) {
    V2 P = A;
    V2 d = Q - P;
    float dd = dot(d, d);
    if (dd > radius * radius) return;
    if (oneSided) {
      V2 A1 = sv(E, 2);
      V2 B1 = A;
      V2 e1 = B1 - A1;
      float u1 = dot(e1, B1 - Q);
      if (u1 > 0.0f) return;
    }
    m->pointCount = 1;
    m->type = B2G_MANIFOLD_CIRCLES;
    m->localNormal = mk(0.0f, 0.0f);
    m->localPoint = P;
    m->id[0] = makeId(0, 0, B2G_FEATURE_VERTEX, B2G_FEATURE_VERTEX);
    m->lp[0] = sv(Cs, 0);
    return;
  }
  if (u <= 0.0f) {
    V2 P = B;
    V2 d = Q - P;
    float dd = dot(d, d);
    if (dd > radius * radius) return;
    if (oneSided) {
      V2 B2 = sv(E, 3);
      V2 A2 = B;
      V2 e2 = B2 - A2;
      float v2 = dot(e2, Q - A2);
      if (v2 > 0.0f) return;
    }
    m->pointCount = 1;
    m->type = B2G_MANIFOLD_CIRCLES;
    m->localNormal = mk(0.0f, 0.0f);
    m->localPoint = P;
    m->id[0] = makeId(1, 0, B2G_FEATURE_VERTEX, B2G_FEATURE_VERTEX);
    m->lp[0] = sv(Cs, 0);
    return;
  }
  float den = dot(e, e);
  V2 P = (1.0f / den) * (u * A + v * B);
  V2 d = Q - P;
  float dd = dot(d, d);
  if (dd > radius * radius) return;
  if (offset < 0.0f) n = mk(-n.x, -n.y);
  normalize(n);
  m->pointCount = 1;
  m->type = B2G_MANIFOLD_FACE_A;
  m->localNormal = n;
  m->localPoint = A;
  m->id[0] = makeId(0, 0, B2G_FEATURE_FACE, B2G_FEATURE_VERTEX);
  m->lp[0] = sv(Cs, 0);
}

// b2CollideEdgeAndPolygon with b2ComputeEdgeSeparation / b2ComputePolygonSeparation
// (src/collision/b2_collide_edge.cpp:167-524)
struct EPAxis { V2 normal; int type; int index; float separation; };  // type: 0 unknown, 1 edgeA, 2 edgeB

B2G_HD void collideEdgeAndPolygon(Man* m, const b2g_shape& E, const Xf& xfA, const b2g_shape& PB, const Xf& xfB) {
  m->pointCount = 0;
  Xf xf = mulT(xfA, xfB);
  V2 centroidB = mul(xf, mk(PB.centroid[0], PB.centroid[1]));
  V2 v1 = sv(E, 0);
  V2 v2 = sv(E, 1);
  V2 edge1 = v2 - v1;
  normalize(edge1);
  V2 normal1 = mk(edge1.y, -edge1.x);
  float offset1 = dot(normal1, centroidB - v1);
  bool oneSided = E.one_sided != 0;
  if (oneSided && offset1 < 0.0f) return;
  V2 tv[B2G_MAX_POLYGON_VERTICES], tn[B2G_MAX_POLYGON_VERTICES];
  int tcount = PB.count;
  for (int i = 0; i < tcount; ++i) {
    tv[i] = mul(xf, sv(PB, i));
    tn[i] = mul(xf.q, sn(PB, i));
  }
  float radius = PB.radius + E.radius;
  EPAxis edgeAxis;
  {
    edgeAxis.type = 1; edgeAxis.index = -1; edgeAxis.separation = -B2G_MAX_FLOAT; edgeAxis.normal = mk(0.0f, 0.0f);
    V2 axes[2] = {normal1, -normal1};
    for (int j = 0; j < 2; ++j) {
      float sj = B2G_MAX_FLOAT;
      for (int i = 0; i < tcount; ++i) {
        float si = dot(axes[j], tv[i] - v1);
        if (si < sj) sj = si;
      }
      if (sj > edgeAxis.separation) { edgeAxis.index = j; edgeAxis.separation = sj; edgeAxis.normal = axes[j]; }
    }
  }
  if (edgeAxis.separation > radius) return;
  EPAxis polygonAxis;
  {
    polygonAxis.type = 0; polygonAxis.index = -1; polygonAxis.separation = -B2G_MAX_FLOAT;
    polygonAxis.normal = mk(0.0f, 0.0f);
    for (int i = 0; i < tcount; ++i) {
      V2 n = -tn[i];
      float s1 = dot(n, tv[i] - v1);
      float s2 = dot(n, tv[i] - v2);
      float s = fmin2(s1, s2);
      if (s > polygonAxis.separation) {
        polygonAxis.type = 2; polygonAxis.index = i; polygonAxis.separation = s; polygonAxis.normal = n;
      }
    }
  }
  if (polygonAxis.separation > radius) return;
  const float k_relativeTol = 0.98f;
  const float k_absoluteTol = 0.001f;
  EPAxis primaryAxis;
  if (polygonAxis.separation - radius > k_relativeTol * (edgeAxis.separation - radius) + k_absoluteTol)
    primaryAxis = polygonAxis;
  else
    primaryAxis = edgeAxis;
  if (oneSided) {
    V2 edge0 = v1 - sv(E, 2);
    normalize(edge0);
    V2 normal0 = mk(edge0.y, -edge0.x);
    bool convex1 = cross(edge0, edge1) >= 0.0f;
    V2 edge2 = sv(E, 3) - v2;
    normalize(edge2);
    V2 normal2 = mk(edge2.y, -edge2.x);
    bool convex2 = cross(edge1, edge2) >= 0.0f;
    const float sinTol = 0.1f;
    bool side1 = dot(primaryAxis.normal, edge1) <= 0.0f;
    if (side1) {
      if (convex1) {
        if (cross(primaryAxis.normal, normal0) > sinTol) return;
      } else {
        primaryAxis = edgeAxis;
      }
    } else {
      if (convex2) {
        if (cross(normal2, primaryAxis.normal) > sinTol) return;
      } else {
        primaryAxis = edgeAxis;
      }
    }
  }
  ClipVertex clipPoints[2];
  int ri1, ri2;
  V2 rv1, rv2, rnormal, sideNormal1, sideNormal2;
  if (primaryAxis.type == 1) {
    m->type = B2G_MANIFOLD_FACE_A;
    int bestIndex = 0;
    float bestValue = dot(primaryAxis.normal, tn[0]);
    for (int i = 1; i < tcount; ++i) {
      float value = dot(primaryAxis.normal, tn[i]);
      if (value < bestValue) { bestValue = value; bestIndex = i; }
    }
    int i1 = bestIndex;
    int i2 = i1 + 1 < tcount ? i1 + 1 : 0;
    clipPoints[0].v = tv[i1];
    clipPoints[0].id = makeId(0, i1, B2G_FEATURE_FACE, B2G_FEATURE_VERTEX);
    clipPoints[1].v = tv[i2];
    clipPoints[1].id = makeId(0, i2, B2G_FEATURE_FACE, B2G_FEATURE_VERTEX);
    ri1 = 0; ri2 = 1; rv1 = v1; rv2 = v2;
    rnormal = primaryAxis.normal;
    sideNormal1 = -edge1;
    sideNormal2 = edge1;
  } else {
    m->type = B2G_MANIFOLD_FACE_B;
    clipPoints[0].v = v2;
    clipPoints[0].id = makeId(1, primaryAxis.index, B2G_FEATURE_VERTEX, B2G_FEATURE_FACE);
    clipPoints[1].v = v1;
    clipPoints[1].id = makeId(0, primaryAxis.index, B2G_FEATURE_VERTEX, B2G_FEATURE_FACE);
    ri1 = primaryAxis.index;
    ri2 = ri1 + 1 < tcount ? ri1 + 1 : 0;
    rv1 = tv[ri1];
    rv2 = tv[ri2];
    rnormal = tn[ri1];
    sideNormal1 = mk(rnormal.y, -rnormal.x);
    sideNormal2 = -sideNormal1;
  }
  float sideOffset1 = dot(sideNormal1, rv1);
  float sideOffset2 = dot(sideNormal2, rv2);
  ClipVertex clipPoints1[2];
  ClipVertex clipPoints2[2];
  int np = clipSegmentToLine(clipPoints1, clipPoints, sideNormal1, sideOffset1, ri1);
  if (np < 2) return;
  np = clipSegmentToLine(clipPoints2, clipPoints1, sideNormal2, sideOffset2, ri2);
  if (np < 2) return;
  if (primaryAxis.type == 1) {
    m->localNormal = rnormal;
    m->localPoint = rv1;
  } else {
    m->localNormal = sn(PB, ri1);
    m->localPoint = sv(PB, ri1);
  }
  int pointCount = 0;
  for (int i = 0; i < 2; ++i) {
    float separation = dot(rnormal, clipPoints2[i].v - rv1);
    if (separation <= radius) {
      if (primaryAxis.type == 1) {
        m->lp[pointCount] = mulT(xf, clipPoints2[i].v);
        m->id[pointCount] = clipPoints2[i].id;
      } else {
        m->lp[pointCount] = clipPoints2[i].v;
        m->id[pointCount] = swapId(clipPoints2[i].id);
      }
      ++pointCount;
    }
  }
  m->pointCount = pointCount;
}

// b2Contact::Evaluate through the dispatch table (src/dynamics/b2_contact.cpp:40-56).
B2G_HD void evaluate(Man* m, const b2g_shape& A, const Xf& xfA, const b2g_shape& B, const Xf& xfB) {
  m->pointCount = 0;
  m->type = 0;
  m->localNormal = mk(0.0f, 0.0f);
  m->localPoint = mk(0.0f, 0.0f);
  m->lp[0] = mk(0.0f, 0.0f);
  m->lp[1] = mk(0.0f, 0.0f);
  m->id[0] = 0;
  m->id[1] = 0;
  if (A.type == B2G_SHAPE_CIRCLE && B.type == B2G_SHAPE_CIRCLE) collideCircles(m, A, xfA, B, xfB);
  else if (A.type == B2G_SHAPE_POLYGON && B.type == B2G_SHAPE_CIRCLE) collidePolygonAndCircle(m, A, xfA, B, xfB);
  else if (A.type == B2G_SHAPE_POLYGON && B.type == B2G_SHAPE_POLYGON) collidePolygons(m, A, xfA, B, xfB);
  else if (A.type == B2G_SHAPE_EDGE && B.type == B2G_SHAPE_CIRCLE) collideEdgeAndCircle(m, A, xfA, B, xfB);
  else if (A.type == B2G_SHAPE_EDGE && B.type == B2G_SHAPE_POLYGON) collideEdgeAndPolygon(m, A, xfA, B, xfB);
}

// b2WorldManifold::Initialize (src/collision/b2_collision.cpp:26-90)
struct WorldMan { V2 normal; V2 points[2]; float separations[2]; };
B2G_HD void worldManifold(WorldMan* wm, int type, int pointCount, V2 localNormal, V2 localPoint, const V2* lp,
                          const Xf& xfA, float radiusA, const Xf& xfB, float radiusB) {
  if (pointCount == 0) return;
  if (type == B2G_MANIFOLD_CIRCLES) {
    wm->normal = mk(1.0f, 0.0f);
    V2 pointA = mul(xfA, localPoint);
    V2 pointB = mul(xfB, lp[0]);
    if (distSq(pointA, pointB) > B2G_EPSILON * B2G_EPSILON) {
      wm->normal = pointB - pointA;
      normalize(wm->normal);
    }
    V2 cA = pointA + radiusA * wm->normal;
    V2 cB = pointB - radiusB * wm->normal;
    wm->points[0] = 0.5f * (cA + cB);
    wm->separations[0] = dot(cB - cA, wm->normal);
  } else if (type == B2G_MANIFOLD_FACE_A) {
    wm->normal = mul(xfA.q, localNormal);
    V2 planePoint = mul(xfA, localPoint);
    for (int i = 0; i < pointCount; ++i) {
      V2 clipPoint = mul(xfB, lp[i]);
      V2 cA = clipPoint + (radiusA - dot(clipPoint - planePoint, wm->normal)) * wm->normal;
      V2 cB = clipPoint - radiusB * wm->normal;
      wm->points[i] = 0.5f * (cA + cB);
      wm->separations[i] = dot(cB - cA, wm->normal);
    }
  } else {
    wm->normal = mul(xfB.q, localNormal);
    V2 planePoint = mul(xfB, localPoint);
    for (int i = 0; i < pointCount; ++i) {
      V2 clipPoint = mul(xfA, lp[i]);
      V2 cB = clipPoint + (radiusB - dot(clipPoint - planePoint, wm->normal)) * wm->normal;
      V2 cA = clipPoint - radiusA * wm->normal;
      wm->points[i] = 0.5f * (cA + cB);
      wm->separations[i] = dot(cA - cB, wm->normal);
    }
    wm->normal = -wm->normal;
  }
}

// Colouring priority of a contact (hash of its (emitter, partner) fixture pair, world-local
// indices) and of a joint (hash of its creation index); lower colours first.
B2G_HD uint32_t fmix32(uint32_t h) {
  h ^= h >> 16; h *= 0x85ebca6bu; h ^= h >> 13; h *= 0xc2b2ae35u; h ^= h >> 16; return h;
}
B2G_HD uint32_t contactPriority(uint32_t emitterLocal, uint32_t partnerLocal) {
  return fmix32(emitterLocal * 0x9e3779b1u ^ fmix32(partnerLocal + 0x7f4a7c15u));
}
B2G_HD uint32_t jointPriority(uint32_t j) { return fmix32(j * 0x9e3779b1u + 0x632be5abu); }

}  // namespace b2g
