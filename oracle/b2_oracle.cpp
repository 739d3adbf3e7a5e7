// b2_oracle.cpp - CPU ORACLE for the GB300 Step engine. TEST INFRASTRUCTURE ONLY.
//
// A plain, single-threaded restatement of box2d-optimized's per-step hot path
// (b2World::Step, src/dynamics/b2_world.cpp:1108-1171) in the canonical order the GPU engine
// uses, so that the engine's results can be checked against it value for value:
//   * contacts are kept sorted by (emitter fixture, partner fixture) instead of the reference's
//     broadphase traversal order;
//   * Gauss-Seidel constraint order is colour by colour (a greedy colouring in hashed-priority
//     order, identical to the engine's) instead of island DFS order, and the position solver's
//     early exit is per world instead of per island;
//   * sine/cosine come from a portable routine (Cody-Waite reduction + Taylor polynomials) that
//     the engine evaluates identically on the GPU; `orc_set_libm_trig(1)` switches the oracle to
//     libm sinf/cosf like the reference.
// Everything else restates the reference's arithmetic in the reference's operation order; each
// function cites the reference file:line it follows.
//
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load this library; the
// product never links or calls it. Pinned against the reference engine compiled from its own
// sources (oracle/_ref, see Makefile) and against committed golden vectors in tests/golden/.

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "../include/b2g_capi.h"

namespace orc {

// ------------------------------------------------------------------------------------------------
// Constants (include/box2d/b2_common.h:39-41, 110-182; b2_settings.h:45-54)
static const float kMaxFloat = FLT_MAX;
static const float kEpsilon = FLT_EPSILON;
static const float kPi = 3.14159265359f;
static const float kLinearSlop = 0.005f;
static const float kAngularSlop = (2.0f / 180.0f * kPi);
static const float kPolygonRadius = (2.0f * kLinearSlop);
static const float kMaxLinearCorrection = 0.2f;
static const float kMaxAngularCorrection = (8.0f / 180.0f * kPi);
static const float kMaxTranslation = 2.0f;
static const float kMaxTranslationSquared = (kMaxTranslation * kMaxTranslation);
static const float kMaxRotation = (0.5f * kPi);
static const float kMaxRotationSquared = (kMaxRotation * kMaxRotation);
static const float kTimeToSleep = 0.5f;                                  // b2_common.h:176
static const float kLinearSleepTolerance = 0.01f;                        // b2_common.h:179
static const float kAngularSleepTolerance = (2.0f / 180.0f * kPi);       // b2_common.h:182
static const float kBaumgarte = 0.2f;

// ------------------------------------------------------------------------------------------------
// Vector algebra with the reference's expression order (include/box2d/b2_math.h:56-735).
struct V2 {
  float x, y;
};
static inline V2 v2(float x, float y) { V2 r; r.x = x; r.y = y; return r; }
static inline V2 operator+(V2 a, V2 b) { return v2(a.x + b.x, a.y + b.y); }
static inline V2 operator-(V2 a, V2 b) { return v2(a.x - b.x, a.y - b.y); }
static inline V2 operator-(V2 a) { return v2(-a.x, -a.y); }
static inline V2 operator*(float s, V2 a) { return v2(s * a.x, s * a.y); }
static inline void addTo(V2& a, V2 b) { a.x += b.x; a.y += b.y; }
static inline void subFrom(V2& a, V2 b) { a.x -= b.x; a.y -= b.y; }
static inline float dot(V2 a, V2 b) { return a.x * b.x + a.y * b.y; }
static inline float cross(V2 a, V2 b) { return a.x * b.y - a.y * b.x; }
static inline V2 cross(V2 a, float s) { return v2(s * a.y, -s * a.x); }
static inline V2 cross(float s, V2 a) { return v2(-s * a.y, s * a.x); }
static inline float lengthOf(V2 a) { return sqrtf(a.x * a.x + a.y * a.y); }
static inline float lengthSq(V2 a) { return a.x * a.x + a.y * a.y; }
static inline float distSq(V2 a, V2 b) { V2 c = a - b; return c.x * c.x + c.y * c.y; }
// b2Vec2::Normalize, b2_math.h:117-130
static inline float normalize(V2& a) {
  float length = lengthOf(a);
  if (length < kEpsilon) return 0.0f;
  float inv = 1.0f / length;
  a.x *= inv;
  a.y *= inv;
  return length;
}
template <typename T> static inline T bmin(T a, T b) { return a < b ? a : b; }
template <typename T> static inline T bmax(T a, T b) { return a > b ? a : b; }
template <typename T> static inline T bclamp(T a, T lo, T hi) { return bmax(lo, bmin(a, hi)); }
static inline float babs(float a) { return a > 0.0f ? a : -a; }
static inline V2 vmin(V2 a, V2 b) { return v2(bmin(a.x, b.x), bmin(a.y, b.y)); }
static inline V2 vmax(V2 a, V2 b) { return v2(bmax(a.x, b.x), bmax(a.y, b.y)); }

struct Rot { float s, c; };
struct Xf { V2 p; Rot q; };
static inline V2 mul(Rot q, V2 v) { return v2(q.c * v.x - q.s * v.y, q.s * v.x + q.c * v.y); }
static inline V2 mulT(Rot q, V2 v) { return v2(q.c * v.x + q.s * v.y, -q.s * v.x + q.c * v.y); }
static inline V2 mul(const Xf& T, V2 v) {
  float x = (T.q.c * v.x - T.q.s * v.y) + T.p.x;
  float y = (T.q.s * v.x + T.q.c * v.y) + T.p.y;
  return v2(x, y);
}
static inline V2 mulT(const Xf& T, V2 v) {
  float px = v.x - T.p.x;
  float py = v.y - T.p.y;
  float x = (T.q.c * px + T.q.s * py);
  float y = (-T.q.s * px + T.q.c * py);
  return v2(x, y);
}
static inline Rot mulT(Rot q, Rot r) {
  Rot o;
  o.s = q.c * r.s - q.s * r.c;
  o.c = q.c * r.c + q.s * r.s;
  return o;
}
static inline Xf mulT(const Xf& A, const Xf& B) {
  Xf C;
  C.q = mulT(A.q, B.q);
  C.p = mulT(A.q, B.p - A.p);
  return C;
}

// b2Mat22 (b2_math.h:184-256)
struct M22 { V2 ex, ey; };
static inline M22 inverse(const M22& m) {
  float a = m.ex.x, b = m.ey.x, c = m.ex.y, d = m.ey.y;
  M22 B;
  float det = a * d - b * c;
  if (det != 0.0f) det = 1.0f / det;
  B.ex.x = det * d;  B.ey.x = -det * b;
  B.ex.y = -det * c; B.ey.y = det * a;
  return B;
}
static inline V2 solve(const M22& m, V2 b) {
  float a11 = m.ex.x, a12 = m.ey.x, a21 = m.ex.y, a22 = m.ey.y;
  float det = a11 * a22 - a12 * a21;
  if (det != 0.0f) det = 1.0f / det;
  V2 x;
  x.x = det * (a22 * b.x - a12 * b.y);
  x.y = det * (a11 * b.y - a21 * b.x);
  return x;
}
static inline V2 mul(const M22& A, V2 v) { return v2(A.ex.x * v.x + A.ey.x * v.y, A.ex.y * v.x + A.ey.y * v.y); }

// b2Vec3 / b2Mat33::Solve33 (b2_math.h:493-520, src/common/b2_math.cpp:28-40)
struct V3 { float x, y, z; };
static inline float dot3(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline V3 cross3(V3 a, V3 b) {
  V3 r; r.x = a.y * b.z - a.z * b.y; r.y = a.z * b.x - a.x * b.z; r.z = a.x * b.y - a.y * b.x; return r;
}
static inline V3 solve33(V3 ex, V3 ey, V3 ez, V3 b) {
  float det = dot3(ex, cross3(ey, ez));
  if (det != 0.0f) det = 1.0f / det;
  V3 x;
  x.x = det * dot3(b, cross3(ey, ez));
  x.y = det * dot3(ex, cross3(b, ez));
  x.z = det * dot3(ex, cross3(ey, b));
  return x;
}

// ------------------------------------------------------------------------------------------------
// Portable sine/cosine (the engine's trig; libm on request).
// Method: Cody & Waite argument reduction by pi/2 with a three-part split of pi/2 whose two
// leading parts carry 12 significant bits (so k*part is exact for |k| < 4096), followed by the
// Taylor series of sin (to r^9) and cos (to r^10) on |r| <= pi/4, evaluated by Horner's rule.
// Truncation error < 3e-9 relative on that interval, well under float's 6e-8 ulp.
static int g_libm_trig = 0;
static const float kTwoOverPi = 0.636619772367581343f;
static const float kPio2A = 1.5703125f;                 // pi/2 to 12 bits
static const float kPio2B = 4.8351287841796875e-04f;    // next 12 bits of pi/2
static const float kPio2C = 3.13916473e-07f;            // remainder of pi/2 (rounded to float)
static inline void sincos_portable(float x, float* s_out, float* c_out) {
  float k = rintf(x * kTwoOverPi);
  float r = x - k * kPio2A;
  r = r - k * kPio2B;
  r = r - k * kPio2C;
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
static inline Rot rotOf(float angle) {
  Rot q;
  if (g_libm_trig) { q.s = sinf(angle); q.c = cosf(angle); }
  else sincos_portable(angle, &q.s, &q.c);
  return q;
}

// ------------------------------------------------------------------------------------------------
// Shapes (src/collision/b2_polygon_shape.cpp, b2_circle_shape.cpp, b2_edge_shape.cpp)
struct Shape {
  int type;       // 0 circle, 1 edge, 2 polygon
  int count;
  float radius;
  bool oneSided;
  V2 v[8];        // polygon vertices / circle p in v[0] / edge v1, v2, v0, v3
  V2 n[8];
  V2 centroid;
};

static Shape shapeFrom(const b2g_shape& s) {
  Shape o;
  memset(&o, 0, sizeof(o));
  o.type = s.type; o.count = s.count; o.radius = s.radius; o.oneSided = s.one_sided != 0;
  for (int i = 0; i < 8; ++i) {
    o.v[i] = v2(s.vertices[i][0], s.vertices[i][1]);
    o.n[i] = v2(s.normals[i][0], s.normals[i][1]);
  }
  o.centroid = v2(s.centroid[0], s.centroid[1]);
  return o;
}
static void shapeTo(const Shape& o, b2g_shape* s) {
  memset(s, 0, sizeof(*s));
  s->type = o.type; s->count = o.count; s->radius = o.radius; s->one_sided = o.oneSided ? 1 : 0;
  for (int i = 0; i < 8; ++i) {
    s->vertices[i][0] = o.v[i].x; s->vertices[i][1] = o.v[i].y;
    s->normals[i][0] = o.n[i].x; s->normals[i][1] = o.n[i].y;
  }
  s->centroid[0] = o.centroid.x; s->centroid[1] = o.centroid.y;
}

// b2PolygonShape::SetAsBox (b2_polygon_shape.cpp:36-48, 50-75)
static void setAsBox(Shape* p, float hx, float hy, bool oriented, V2 center, float angle) {
  memset(p, 0, sizeof(*p));
  p->type = 2; p->radius = kPolygonRadius; p->count = 4;
  p->v[0] = v2(-hx, -hy); p->v[1] = v2(hx, -hy); p->v[2] = v2(hx, hy); p->v[3] = v2(-hx, hy);
  p->n[0] = v2(0.0f, -1.0f); p->n[1] = v2(1.0f, 0.0f); p->n[2] = v2(0.0f, 1.0f); p->n[3] = v2(-1.0f, 0.0f);
  p->centroid = v2(0.0f, 0.0f);
  if (oriented) {
    p->centroid = center;
    Xf xf;
    xf.p = center;
    xf.q.s = sinf(angle);   // b2Rot::Set on the host uses libm (b2_math.h:313-318)
    xf.q.c = cosf(angle);
    for (int i = 0; i < 4; ++i) {
      p->v[i] = mul(xf, p->v[i]);
      p->n[i] = mul(xf.q, p->n[i]);
    }
  }
}

// ComputeCentroid (b2_polygon_shape.cpp:77-111)
static V2 computeCentroid(const V2* vs, int count) {
  V2 c = v2(0.0f, 0.0f);
  float area = 0.0f;
  V2 s = vs[0];
  const float inv3 = 1.0f / 3.0f;
  for (int i = 0; i < count; ++i) {
    V2 p1 = vs[0] - s;
    V2 p2 = vs[i] - s;
    V2 p3 = i + 1 < count ? vs[i + 1] - s : vs[0] - s;
    V2 e1 = p2 - p1;
    V2 e2 = p3 - p1;
    float D = cross(e1, e2);
    float triangleArea = 0.5f * D;
    area += triangleArea;
    addTo(c, (triangleArea * inv3) * ((p1 + p2) + p3));
  }
  c = (1.0f / area) * c + s;
  return c;
}

// b2PolygonShape::Set (b2_polygon_shape.cpp:113-243): weld, gift-wrap hull, normals, centroid.
static void polygonSet(Shape* p, const V2* vertices, int count) {
  if (count < 3) { setAsBox(p, 1.0f, 1.0f, false, v2(0, 0), 0); return; }
  int n = bmin(count, 8);
  V2 ps[8];
  int tempCount = 0;
  for (int i = 0; i < n; ++i) {
    V2 v = vertices[i];
    bool unique = true;
    for (int j = 0; j < tempCount; ++j) {
      if (distSq(v, ps[j]) < ((0.5f * kLinearSlop) * (0.5f * kLinearSlop))) { unique = false; break; }
    }
    if (unique) ps[tempCount++] = v;
  }
  n = tempCount;
  if (n < 3) { setAsBox(p, 1.0f, 1.0f, false, v2(0, 0), 0); return; }
  int i0 = 0;
  float x0 = ps[0].x;
  for (int i = 1; i < n; ++i) {
    float x = ps[i].x;
    if (x > x0 || (x == x0 && ps[i].y < ps[i0].y)) { i0 = i; x0 = x; }
  }
  int hull[8];
  int m = 0;
  int ih = i0;
  for (;;) {
    if (m >= 8) break;
    hull[m] = ih;
    int ie = 0;
    for (int j = 1; j < n; ++j) {
      if (ie == ih) { ie = j; continue; }
      V2 r = ps[ie] - ps[hull[m]];
      V2 v = ps[j] - ps[hull[m]];
      float c = cross(r, v);
      if (c < 0.0f) ie = j;
      if (c == 0.0f && lengthSq(v) > lengthSq(r)) ie = j;
    }
    ++m;
    ih = ie;
    if (ie == i0) break;
  }
  if (m < 3) { setAsBox(p, 1.0f, 1.0f, false, v2(0, 0), 0); return; }
  memset(p, 0, sizeof(*p));
  p->type = 2; p->radius = kPolygonRadius; p->count = m;
  for (int i = 0; i < m; ++i) p->v[i] = ps[hull[i]];
  for (int i = 0; i < m; ++i) {
    int i1 = i;
    int i2 = i + 1 < m ? i + 1 : 0;
    V2 edge = p->v[i2] - p->v[i1];
    p->n[i] = cross(edge, 1.0f);
    normalize(p->n[i]);
  }
  p->centroid = computeCentroid(p->v, m);
}

struct MassData { float mass; V2 center; float I; };

// ComputeMass for polygon (b2_polygon_shape.cpp:390-464), circle (b2_circle_shape.cpp:98-104),
// edge (b2_edge_shape.cpp:169-176).
static MassData computeMass(const Shape& s, float density) {
  MassData md;
  if (s.type == 0) {
    md.mass = density * kPi * s.radius * s.radius;
    md.center = s.v[0];
    md.I = md.mass * (0.5f * s.radius * s.radius + dot(s.v[0], s.v[0]));
    return md;
  }
  if (s.type == 1) {
    md.mass = 0.0f;
    md.center = 0.5f * (s.v[0] + s.v[1]);
    md.I = 0.0f;
    return md;
  }
  V2 center = v2(0.0f, 0.0f);
  float area = 0.0f;
  float I = 0.0f;
  V2 sref = s.v[0];
  const float k_inv3 = 1.0f / 3.0f;
  for (int i = 0; i < s.count; ++i) {
    V2 e1 = s.v[i] - sref;
    V2 e2 = i + 1 < s.count ? s.v[i + 1] - sref : s.v[0] - sref;
    float D = cross(e1, e2);
    float triangleArea = 0.5f * D;
    area += triangleArea;
    addTo(center, (triangleArea * k_inv3) * (e1 + e2));
    float ex1 = e1.x, ey1 = e1.y;
    float ex2 = e2.x, ey2 = e2.y;
    float intx2 = ex1 * ex1 + ex2 * ex1 + ex2 * ex2;
    float inty2 = ey1 * ey1 + ey2 * ey1 + ey2 * ey2;
    I += (0.25f * k_inv3 * D) * (intx2 + inty2);
  }
  md.mass = density * area;
  float inv = 1.0f / area;
  center.x *= inv;
  center.y *= inv;
  md.center = center + sref;
  md.I = density * I;
  md.I += md.mass * (dot(md.center, md.center) - dot(center, center));
  return md;
}

struct AABB { V2 lo, hi; };

// ComputeAABB: polygon (b2_polygon_shape.cpp:373-388), circle (b2_circle_shape.cpp:91-96),
// edge (b2_edge_shape.cpp:156-167).
static AABB computeAABB(const Shape& s, const Xf& xf) {
  AABB bb;
  if (s.type == 0) {
    V2 p = xf.p + mul(xf.q, s.v[0]);
    bb.lo = v2(p.x - s.radius, p.y - s.radius);
    bb.hi = v2(p.x + s.radius, p.y + s.radius);
    return bb;
  }
  if (s.type == 1) {
    V2 a = mul(xf, s.v[0]);
    V2 b = mul(xf, s.v[1]);
    V2 lower = vmin(a, b);
    V2 upper = vmax(a, b);
    V2 r = v2(s.radius, s.radius);
    bb.lo = lower - r;
    bb.hi = upper + r;
    return bb;
  }
  V2 lower = mul(xf, s.v[0]);
  V2 upper = lower;
  for (int i = 1; i < s.count; ++i) {
    V2 v = mul(xf, s.v[i]);
    lower = vmin(lower, v);
    upper = vmax(upper, v);
  }
  V2 r = v2(s.radius, s.radius);
  bb.lo = lower - r;
  bb.hi = upper + r;
  return bb;
}

// b2TestOverlap(AABB, AABB), include/box2d/b2_collision.h:270-276 (inclusive)
static inline bool overlap(const AABB& a, const AABB& b) {
  return (a.hi.x >= b.lo.x) & (a.lo.x <= b.hi.x) & (a.hi.y >= b.lo.y) & (a.lo.y <= b.hi.y);
}

// ------------------------------------------------------------------------------------------------
// Narrowphase (src/collision/b2_collide_*.cpp, b2_collision.cpp)
struct MPoint { V2 localPoint; float normalImpulse, tangentImpulse; uint32_t id; };
struct Manifold { MPoint points[2]; V2 localNormal; V2 localPoint; int type; int pointCount; };

static inline uint32_t makeId(int indexA, int indexB, int typeA, int typeB) {
  return (uint32_t)(uint8_t)indexA | ((uint32_t)(uint8_t)indexB << 8) |
         ((uint32_t)(uint8_t)typeA << 16) | ((uint32_t)(uint8_t)typeB << 24);
}
static inline int idIndexA(uint32_t id) { return (int)(id & 0xff); }
static inline int idIndexB(uint32_t id) { return (int)((id >> 8) & 0xff); }
static inline int idTypeA(uint32_t id) { return (int)((id >> 16) & 0xff); }
static inline int idTypeB(uint32_t id) { return (int)((id >> 24) & 0xff); }
static inline uint32_t swapId(uint32_t id) {
  return makeId(idIndexB(id), idIndexA(id), idTypeB(id), idTypeA(id));
}
enum { kVertex = 0, kFace = 1 };

struct ClipVertex { V2 v; uint32_t id; };

// b2ClipSegmentToLine (b2_collision.cpp:205-237)
static int clipSegmentToLine(ClipVertex vOut[2], const ClipVertex vIn[2], V2 normal, float offset,
                             int vertexIndexA) {
  int count = 0;
  float distance0 = dot(normal, vIn[0].v) - offset;
  float distance1 = dot(normal, vIn[1].v) - offset;
  if (distance0 <= 0.0f) vOut[count++] = vIn[0];
  if (distance1 <= 0.0f) vOut[count++] = vIn[1];
  if (distance0 * distance1 < 0.0f) {
    float interp = distance0 / (distance0 - distance1);
    vOut[count].v = vIn[0].v + interp * (vIn[1].v - vIn[0].v);
    vOut[count].id = makeId(vertexIndexA, idIndexB(vIn[0].id), kVertex, kFace);
    ++count;
  }
  return count;
}

// b2CollideCircles (b2_collide_circle.cpp:27-53)
static void collideCircles(Manifold* m, const Shape& A, const Xf& xfA, const Shape& B, const Xf& xfB) {
  m->pointCount = 0;
  V2 pA = mul(xfA, A.v[0]);
  V2 pB = mul(xfB, B.v[0]);
  V2 d = pB - pA;
  float distSqr = dot(d, d);
  float rA = A.radius, rB = B.radius;
  float radius = rA + rB;
  if (distSqr > radius * radius) return;
  m->type = 0;
  m->localPoint = A.v[0];
  m->localNormal = v2(0.0f, 0.0f);
  m->pointCount = 1;
  m->points[0].localPoint = B.v[0];
  m->points[0].id = 0;
}

// b2CollidePolygonAndCircle (b2_collide_circle.cpp:55-158)
static void collidePolygonAndCircle(Manifold* m, const Shape& P, const Xf& xfA, const Shape& Cs,
                                    const Xf& xfB) {
  m->pointCount = 0;
  V2 c = mul(xfB, Cs.v[0]);
  V2 cLocal = mulT(xfA, c);
  int normalIndex = 0;
  float separation = -kMaxFloat;
  float radius = P.radius + Cs.radius;
  int vertexCount = P.count;
  for (int i = 0; i < vertexCount; ++i) {
    float s = dot(P.n[i], cLocal - P.v[i]);
    if (s > radius) return;
    if (s > separation) { separation = s; normalIndex = i; }
  }
  int vertIndex1 = normalIndex;
  int vertIndex2 = vertIndex1 + 1 < vertexCount ? vertIndex1 + 1 : 0;
  V2 v1 = P.v[vertIndex1];
  V2 v2_ = P.v[vertIndex2];
  if (separation < kEpsilon) {
    m->pointCount = 1;
    m->type = 1;
    m->localNormal = P.n[normalIndex];
    m->localPoint = 0.5f * (v1 + v2_);
    m->points[0].localPoint = Cs.v[0];
    m->points[0].id = 0;
    return;
  }
  float u1 = dot(cLocal - v1, v2_ - v1);
  float u2 = dot(cLocal - v2_, v1 - v2_);
  if (u1 <= 0.0f) {
    if (distSq(cLocal, v1) > radius * radius) return;
    m->pointCount = 1;
    m->type = 1;
    m->localNormal = cLocal - v1;
    normalize(m->localNormal);
    m->localPoint = v1;
    m->points[0].localPoint = Cs.v[0];
    m->points[0].id = 0;
  } else if (u2 <= 0.0f) {
    if (distSq(cLocal, v2_) > radius * radius) return;
    m->pointCount = 1;
    m->type = 1;
    m->localNormal = cLocal - v2_;
    normalize(m->localNormal);
    m->localPoint = v2_;
    m->points[0].localPoint = Cs.v[0];
    m->points[0].id = 0;
  } else {
    V2 faceCenter = 0.5f * (v1 + v2_);
    float s = dot(cLocal - faceCenter, P.n[vertIndex1]);
    if (s > radius) return;
    m->pointCount = 1;
    m->type = 1;
    m->localNormal = P.n[vertIndex1];
    m->localPoint = faceCenter;
    m->points[0].localPoint = Cs.v[0];
    m->points[0].id = 0;
  }
}

// b2FindMaxSeparation (b2_collide_polygon.cpp:27-66)
static float findMaxSeparation(int* edgeIndex, const Shape& p1, const Xf& xf1, const Shape& p2, const Xf& xf2) {
  int count1 = p1.count;
  int count2 = p2.count;
  Xf xf = mulT(xf2, xf1);
  int bestIndex = 0;
  float maxSeparation = -kMaxFloat;
  for (int i = 0; i < count1; ++i) {
    V2 n = mul(xf.q, p1.n[i]);
    V2 v1 = mul(xf, p1.v[i]);
    float si = kMaxFloat;
    for (int j = 0; j < count2; ++j) {
      float sij = dot(n, p2.v[j] - v1);
      if (sij < si) si = sij;
    }
    if (si > maxSeparation) { maxSeparation = si; bestIndex = i; }
  }
  *edgeIndex = bestIndex;
  return maxSeparation;
}

// b2FindIncidentEdge (b2_collide_polygon.cpp:68-111)
static void findIncidentEdge(ClipVertex c[2], const Shape& p1, const Xf& xf1, int edge1, const Shape& p2,
                             const Xf& xf2) {
  V2 normal1 = mulT(xf2.q, mul(xf1.q, p1.n[edge1]));
  int index = 0;
  float minDot = kMaxFloat;
  for (int i = 0; i < p2.count; ++i) {
    float d = dot(normal1, p2.n[i]);
    if (d < minDot) { minDot = d; index = i; }
  }
  int i1 = index;
  int i2 = i1 + 1 < p2.count ? i1 + 1 : 0;
  c[0].v = mul(xf2, p2.v[i1]);
  c[0].id = makeId(edge1, i1, kFace, kVertex);
  c[1].v = mul(xf2, p2.v[i2]);
  c[1].id = makeId(edge1, i2, kFace, kVertex);
}

// b2CollidePolygons (b2_collide_polygon.cpp:120-243)
static void collidePolygons(Manifold* m, const Shape& A, const Xf& xfA, const Shape& B, const Xf& xfB) {
  m->pointCount = 0;
  float totalRadius = A.radius + B.radius;
  int edgeA = 0;
  float separationA = findMaxSeparation(&edgeA, A, xfA, B, xfB);
  if (separationA > totalRadius) return;
  int edgeB = 0;
  float separationB = findMaxSeparation(&edgeB, B, xfB, A, xfA);
  if (separationB > totalRadius) return;
  const Shape* poly1;
  const Shape* poly2;
  Xf xf1, xf2;
  int edge1;
  int flip;
  const float k_tol = 0.1f * kLinearSlop;
  if (separationB > separationA + k_tol) {
    poly1 = &B; poly2 = &A; xf1 = xfB; xf2 = xfA; edge1 = edgeB; m->type = 2; flip = 1;
  } else {
    poly1 = &A; poly2 = &B; xf1 = xfA; xf2 = xfB; edge1 = edgeA; m->type = 1; flip = 0;
  }
  ClipVertex incidentEdge[2];
  findIncidentEdge(incidentEdge, *poly1, xf1, edge1, *poly2, xf2);
  int count1 = poly1->count;
  int iv1 = edge1;
  int iv2 = edge1 + 1 < count1 ? edge1 + 1 : 0;
  V2 v11 = poly1->v[iv1];
  V2 v12 = poly1->v[iv2];
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
      MPoint* cp = m->points + pointCount;
      cp->localPoint = mulT(xf2, clipPoints2[i].v);
      cp->id = flip ? swapId(clipPoints2[i].id) : clipPoints2[i].id;
      ++pointCount;
    }
  }
  m->pointCount = pointCount;
}

// b2CollideEdgeAndCircle (b2_collide_edge.cpp:31-165)
static void collideEdgeAndCircle(Manifold* m, const Shape& E, const Xf& xfA, const Shape& Cs, const Xf& xfB) {
  m->pointCount = 0;
  V2 Q = mulT(xfA, mul(xfB, Cs.v[0]));
  V2 A = E.v[0], B = E.v[1];
  V2 e = B - A;
  V2 n = v2(e.y, -e.x);
  float offset = dot(n, Q - A);
  bool oneSided = E.oneSided;
  if (oneSided && offset < 0.0f) return;
  float u = dot(e, B - Q);
  float v = dot(e, Q - A);
  float radius = E.radius + Cs.radius;
  if (v <= 0.0f) {
    V2 P = A;
    V2 d = Q - P;
    float dd = dot(d, d);
    if (dd > radius * radius) return;
    if (E.oneSided) {
      V2 A1 = E.v[2];
      V2 B1 = A;
      V2 e1 = B1 - A1;
      float u1 = dot(e1, B1 - Q);
      if (u1 > 0.0f) return;
    }
    m->pointCount = 1;
    m->type = 0;
    m->localNormal = v2(0.0f, 0.0f);
    m->localPoint = P;
    m->points[0].id = makeId(0, 0, kVertex, kVertex);
    m->points[0].localPoint = Cs.v[0];
    return;
  }
  if (u <= 0.0f) {
    V2 P = B;
    V2 d = Q - P;
    float dd = dot(d, d);
    if (dd > radius * radius) return;
    if (E.oneSided) {
      V2 B2 = E.v[3];
      V2 A2 = B;
      V2 e2 = B2 - A2;
      float v2v = dot(e2, Q - A2);
      if (v2v > 0.0f) return;
    }
    m->pointCount = 1;
    m->type = 0;
    m->localNormal = v2(0.0f, 0.0f);
    m->localPoint = P;
    m->points[0].id = makeId(1, 0, kVertex, kVertex);
    m->points[0].localPoint = Cs.v[0];
    return;
  }
  float den = dot(e, e);
  V2 P = (1.0f / den) * (u * A + v * B);
  V2 d = Q - P;
  float dd = dot(d, d);
  if (dd > radius * radius) return;
  if (offset < 0.0f) n = v2(-n.x, -n.y);
  normalize(n);
  m->pointCount = 1;
  m->type = 1;
  m->localNormal = n;
  m->localPoint = A;
  m->points[0].id = makeId(0, 0, kFace, kVertex);
  m->points[0].localPoint = Cs.v[0];
}

// b2EPAxis, b2TempPolygon, b2ReferenceFace and b2CollideEdgeAndPolygon (b2_collide_edge.cpp:167-524)
struct EPAxis { V2 normal; int type; int index; float separation; };  // type 0 unknown 1 edgeA 2 edgeB
struct TempPoly { V2 v[8]; V2 n[8]; int count; };

static EPAxis computeEdgeSeparation(const TempPoly& pb, V2 v1, V2 normal1) {
  EPAxis axis;
  axis.type = 1; axis.index = -1; axis.separation = -FLT_MAX; axis.normal = v2(0.0f, 0.0f);
  V2 axes[2] = {normal1, -normal1};
  for (int j = 0; j < 2; ++j) {
    float sj = FLT_MAX;
    for (int i = 0; i < pb.count; ++i) {
      float si = dot(axes[j], pb.v[i] - v1);
      if (si < sj) sj = si;
    }
    if (sj > axis.separation) { axis.index = j; axis.separation = sj; axis.normal = axes[j]; }
  }
  return axis;
}

static EPAxis computePolygonSeparation(const TempPoly& pb, V2 v1, V2 v2_) {
  EPAxis axis;
  axis.type = 0; axis.index = -1; axis.separation = -FLT_MAX; axis.normal = v2(0.0f, 0.0f);
  for (int i = 0; i < pb.count; ++i) {
    V2 n = -pb.n[i];
    float s1 = dot(n, pb.v[i] - v1);
    float s2 = dot(n, pb.v[i] - v2_);
    float s = bmin(s1, s2);
    if (s > axis.separation) { axis.type = 2; axis.index = i; axis.separation = s; axis.normal = n; }
  }
  return axis;
}

static void collideEdgeAndPolygon(Manifold* m, const Shape& E, const Xf& xfA, const Shape& PB, const Xf& xfB) {
  m->pointCount = 0;
  Xf xf = mulT(xfA, xfB);
  V2 centroidB = mul(xf, PB.centroid);
  V2 v1 = E.v[0];
  V2 v2_ = E.v[1];
  V2 edge1 = v2_ - v1;
  normalize(edge1);
  V2 normal1 = v2(edge1.y, -edge1.x);
  float offset1 = dot(normal1, centroidB - v1);
  bool oneSided = E.oneSided;
  if (oneSided && offset1 < 0.0f) return;
  TempPoly tp;
  tp.count = PB.count;
  for (int i = 0; i < PB.count; ++i) {
    tp.v[i] = mul(xf, PB.v[i]);
    tp.n[i] = mul(xf.q, PB.n[i]);
  }
  float radius = PB.radius + E.radius;
  EPAxis edgeAxis = computeEdgeSeparation(tp, v1, normal1);
  if (edgeAxis.separation > radius) return;
  EPAxis polygonAxis = computePolygonSeparation(tp, v1, v2_);
  if (polygonAxis.separation > radius) return;
  const float k_relativeTol = 0.98f;
  const float k_absoluteTol = 0.001f;
  EPAxis primaryAxis;
  if (polygonAxis.separation - radius > k_relativeTol * (edgeAxis.separation - radius) + k_absoluteTol)
    primaryAxis = polygonAxis;
  else
    primaryAxis = edgeAxis;
  if (oneSided) {
    V2 edge0 = v1 - E.v[2];
    normalize(edge0);
    V2 normal0 = v2(edge0.y, -edge0.x);
    bool convex1 = cross(edge0, edge1) >= 0.0f;
    V2 edge2 = E.v[3] - v2_;
    normalize(edge2);
    V2 normal2 = v2(edge2.y, -edge2.x);
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
    m->type = 1;
    int bestIndex = 0;
    float bestValue = dot(primaryAxis.normal, tp.n[0]);
    for (int i = 1; i < tp.count; ++i) {
      float value = dot(primaryAxis.normal, tp.n[i]);
      if (value < bestValue) { bestValue = value; bestIndex = i; }
    }
    int i1 = bestIndex;
    int i2 = i1 + 1 < tp.count ? i1 + 1 : 0;
    clipPoints[0].v = tp.v[i1];
    clipPoints[0].id = makeId(0, i1, kFace, kVertex);
    clipPoints[1].v = tp.v[i2];
    clipPoints[1].id = makeId(0, i2, kFace, kVertex);
    ri1 = 0; ri2 = 1; rv1 = v1; rv2 = v2_;
    rnormal = primaryAxis.normal;
    sideNormal1 = -edge1;
    sideNormal2 = edge1;
  } else {
    m->type = 2;
    clipPoints[0].v = v2_;
    clipPoints[0].id = makeId(1, primaryAxis.index, kVertex, kFace);
    clipPoints[1].v = v1;
    clipPoints[1].id = makeId(0, primaryAxis.index, kVertex, kFace);
    ri1 = primaryAxis.index;
    ri2 = ri1 + 1 < tp.count ? ri1 + 1 : 0;
    rv1 = tp.v[ri1];
    rv2 = tp.v[ri2];
    rnormal = tp.n[ri1];
    sideNormal1 = v2(rnormal.y, -rnormal.x);
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
    m->localNormal = PB.n[ri1];
    m->localPoint = PB.v[ri1];
  }
  int pointCount = 0;
  for (int i = 0; i < 2; ++i) {
    float separation = dot(rnormal, clipPoints2[i].v - rv1);
    if (separation <= radius) {
      MPoint* cp = m->points + pointCount;
      if (primaryAxis.type == 1) {
        cp->localPoint = mulT(xf, clipPoints2[i].v);
        cp->id = clipPoints2[i].id;
      } else {
        cp->localPoint = clipPoints2[i].v;
        cp->id = swapId(clipPoints2[i].id);
      }
      ++pointCount;
    }
  }
  m->pointCount = pointCount;
}

// Dispatch in b2Contact's table order (src/dynamics/b2_contact.cpp:46-56); A's shape first.
static bool hasCollider(int ta, int tb) {
  return (ta == 0 && tb == 0) || (ta == 2 && tb == 0) || (ta == 2 && tb == 2) || (ta == 1 && tb == 0) ||
         (ta == 1 && tb == 2);
}
static void evaluate(Manifold* m, const Shape& A, const Xf& xfA, const Shape& B, const Xf& xfB) {
  if (A.type == 0 && B.type == 0) collideCircles(m, A, xfA, B, xfB);
  else if (A.type == 2 && B.type == 0) collidePolygonAndCircle(m, A, xfA, B, xfB);
  else if (A.type == 2 && B.type == 2) collidePolygons(m, A, xfA, B, xfB);
  else if (A.type == 1 && B.type == 0) collideEdgeAndCircle(m, A, xfA, B, xfB);
  else if (A.type == 1 && B.type == 2) collideEdgeAndPolygon(m, A, xfA, B, xfB);
  else m->pointCount = 0;
}

// b2WorldManifold::Initialize (b2_collision.cpp:26-90)
struct WorldManifold { V2 normal; V2 points[2]; float separations[2]; };
static void worldManifold(WorldManifold* wm, const Manifold& m, const Xf& xfA, float radiusA, const Xf& xfB,
                          float radiusB) {
  if (m.pointCount == 0) return;
  if (m.type == 0) {
    wm->normal = v2(1.0f, 0.0f);
    V2 pointA = mul(xfA, m.localPoint);
    V2 pointB = mul(xfB, m.points[0].localPoint);
    if (distSq(pointA, pointB) > kEpsilon * kEpsilon) {
      wm->normal = pointB - pointA;
      normalize(wm->normal);
    }
    V2 cA = pointA + radiusA * wm->normal;
    V2 cB = pointB - radiusB * wm->normal;
    wm->points[0] = 0.5f * (cA + cB);
    wm->separations[0] = dot(cB - cA, wm->normal);
  } else if (m.type == 1) {
    wm->normal = mul(xfA.q, m.localNormal);
    V2 planePoint = mul(xfA, m.localPoint);
    for (int i = 0; i < m.pointCount; ++i) {
      V2 clipPoint = mul(xfB, m.points[i].localPoint);
      V2 cA = clipPoint + (radiusA - dot(clipPoint - planePoint, wm->normal)) * wm->normal;
      V2 cB = clipPoint - radiusB * wm->normal;
      wm->points[i] = 0.5f * (cA + cB);
      wm->separations[i] = dot(cB - cA, wm->normal);
    }
  } else {
    wm->normal = mul(xfB.q, m.localNormal);
    V2 planePoint = mul(xfB, m.localPoint);
    for (int i = 0; i < m.pointCount; ++i) {
      V2 clipPoint = mul(xfA, m.points[i].localPoint);
      V2 cB = clipPoint + (radiusB - dot(clipPoint - planePoint, wm->normal)) * wm->normal;
      V2 cA = clipPoint - radiusA * wm->normal;
      wm->points[i] = 0.5f * (cA + cB);
      wm->separations[i] = dot(cA - cB, wm->normal);
    }
    wm->normal = -wm->normal;
  }
}

static Manifold manifoldFrom(const b2g_manifold& s) {
  Manifold m;
  memset(&m, 0, sizeof(m));
  for (int i = 0; i < 2; ++i) {
    m.points[i].localPoint = v2(s.points[i].local_point[0], s.points[i].local_point[1]);
    m.points[i].normalImpulse = s.points[i].normal_impulse;
    m.points[i].tangentImpulse = s.points[i].tangent_impulse;
    m.points[i].id = s.points[i].id;
  }
  m.localNormal = v2(s.local_normal[0], s.local_normal[1]);
  m.localPoint = v2(s.local_point[0], s.local_point[1]);
  m.type = s.type;
  m.pointCount = s.point_count;
  return m;
}
static void manifoldTo(const Manifold& m, b2g_manifold* s) {
  memset(s, 0, sizeof(*s));
  for (int i = 0; i < 2; ++i) {
    s->points[i].local_point[0] = m.points[i].localPoint.x;
    s->points[i].local_point[1] = m.points[i].localPoint.y;
    s->points[i].normal_impulse = m.points[i].normalImpulse;
    s->points[i].tangent_impulse = m.points[i].tangentImpulse;
    s->points[i].id = m.points[i].id;
  }
  s->local_normal[0] = m.localNormal.x; s->local_normal[1] = m.localNormal.y;
  s->local_point[0] = m.localPoint.x; s->local_point[1] = m.localPoint.y;
  s->type = m.type;
  s->point_count = m.pointCount;
}

// ------------------------------------------------------------------------------------------------
// World model
struct Body {
  Xf xf;
  V2 c; float a;
  V2 v; float w;
  V2 localCenter;
  float mass, invMass, I, invI;
  float linearDamping, angularDamping, gravityScale;
  V2 force; float torque;
  int type;
  uint32_t flags;
  float sleepTime = 0.0f;
  V2 c0;                       // b2Sweep::c0, a0, alpha0: the centre and angle at alpha0
  float a0 = 0.0f, alpha0 = 0.0f;
  bool awake() const { return (flags & B2G_BODY_AWAKE) != 0; }
};

struct Fixture {
  Shape shape;
  int body;
  float density, friction, restitution, threshold;
  uint16_t category, mask; int16_t group;
  bool sensor;
};

struct Joint {
  b2g_joint_def d;
  // state (b2RevoluteJoint / b2PrismaticJoint / b2DistanceJoint members)
  V2 impulse2;       // revolute / prismatic m_impulse
  float impulse1;    // distance m_impulse
  float motorImpulse, lowerImpulse, upperImpulse;
  // solver temporaries
  int iA, iB;
  V2 lcA, lcB;
  float mA, mB, invIA, invIB;
  V2 rA, rB;
  M22 K;
  float axialMass, angle;
  V2 localXAxisA, localYAxisA, axis, perp;
  float a1, a2, s1, s2, translation;
  V2 u; float currentLength, mass, softMass, gamma, bias;
  // weld, wheel, motor, friction, mouse, pulley (b2_weld_joint.h:117-125, b2_wheel_joint.h:178-212,
  // b2_motor_joint.h:106-122, b2_friction_joint.h:95-107, b2_mouse_joint.h:110-127,
  // b2_pulley_joint.h:125-148): imp[] holds their accumulated impulses in the b2g_joint.impulse
  // layout; the wheel keeps ax/ay in axis/perp and sAx, sBx, sAy, sBy in a1, a2, s1, s2
  float imp[3];
  float mass3[9];
  float springMass, motorMass;
  V2 err; float angularError;
  V2 uB; float constant;
  // gear (b2_gear_joint.h:52-110): A, B = d.body_a / d.body_b (the coupled joints' bodies B),
  // C, D = their bodies A; geometry from the two joints; m_impulse in imp[0]
  int iC, iD, typeA, typeB;
  V2 gLA, gLB, gLC, gLD, gAxC, gAxD;
  float gRefA, gRefB;
  V2 gLcA, gLcB, gLcC, gLcD;
  float gmA, gmB, gmC, gmD, giA, giB, giC, giD;
  V2 JvAC, JvBD;
  float JwA, JwB, JwC, JwD, gMass;
};

struct Contact {
  uint64_t key;   // emitter << 32 | partner
  int fA, fB;     // oriented per the dispatch table
  uint32_t flags;
  float friction, restitution, threshold, tangentSpeed;
  Manifold m;
};

struct VCPoint { V2 rA, rB; float normalImpulse, tangentImpulse, normalMass, tangentMass, velocityBias; };
struct VC {
  VCPoint points[2];
  V2 normal;
  M22 normalMass, K;
  int indexA, indexB;
  float invMassA, invMassB, invIA, invIB;
  float friction, restitution, threshold, tangentSpeed;
  int pointCount;
  int contact;
};
struct PC {
  V2 localPoints[2];
  V2 localNormal, localPoint;
  int indexA, indexB;
  float invMassA, invMassB;
  V2 localCenterA, localCenterB;
  float invIA, invIB;
  int type;
  float radiusA, radiusB;
  int pointCount;
};

// Hash of a constraint's stable identity, the colouring priority (lower first).
static inline uint32_t fmix32(uint32_t h) {
  h ^= h >> 16; h *= 0x85ebca6bu; h ^= h >> 13; h *= 0xc2b2ae35u; h ^= h >> 16; return h;
}
static inline uint32_t contactPriority(uint64_t key) {
  uint32_t e = (uint32_t)(key >> 32), p = (uint32_t)key;
  return fmix32(e * 0x9e3779b1u ^ fmix32(p + 0x7f4a7c15u));
}
static inline uint32_t jointPriority(uint32_t j) { return fmix32(j * 0x9e3779b1u + 0x632be5abu); }

static const int kColors = 64;          // colours 0..62 regular, 63 = overflow (solved serially)
static const int kOverflow = kColors - 1;

struct World {
  V2 gravity;
  bool allowSleep = false;
  bool sleepers = false;                   // bodies may be asleep although sleeping is not allowed
  bool warmStarting = true;
  bool autoClearForces = true;
  bool newContacts = true;
  float inv_dt0 = 0.0f;
  std::vector<Body> bodies;
  std::vector<Fixture> fixtures;
  std::vector<Joint> joints;
  std::vector<Contact> contacts;           // sorted by key
  bool continuous = false;                 // b2World::SetContinuousPhysics
  std::vector<AABB> aabb;                  // per fixture: its box at the last pair update
  std::vector<uint64_t> noCollide;         // sorted body pairs joined by collideConnected=false joints
  // last step's solver order record
  std::vector<int> contactColor;           // per contact (-1 not solved)
  std::vector<uint32_t> contactPrio;
  std::vector<int> jointColor;
  std::vector<uint32_t> jointPrioV;
  std::vector<int32_t> lastContactOrder;   // (fixture A, fixture B) pairs in solve order
  std::vector<int32_t> lastJointOrder;     // joint indices in solve order
  // last step's islands (sleep mode): per island its root body, whether it is an orphan, its
  // bodies, its contacts as (fixture A, fixture B) in solve order and its joints in solve order
  std::vector<int32_t> islandRoot, islandOrphan, islandBodyOff, islandBodies;
  std::vector<int32_t> islandContactOff, islandContacts, islandJointOff, islandJoints;
  // listener events of the steps since the last read (b2ContactListener, src/dynamics/
  // b2_world_callbacks.h:133-209), when recording is on: Begin / End / PreSolve from the
  // narrowphase (b2Contact::Update), PostSolve from the solver (b2Island::Report), End for the
  // touching contacts the broadphase drops (b2ContactManager::Destroy)
  bool recordEvents = false;
  std::vector<b2g_event> events;
  bool sleepMode() const { return allowSleep || sleepers; }
};

static void recordEvent(World* w, int kind, int fa, int fb, const b2g_manifold* old = nullptr, int pc = 0,
                        const float* ni = nullptr, const float* ti = nullptr) {
  b2g_event e;
  memset(&e, 0, sizeof(e));
  e.kind = kind;
  e.fixture_a = fa;
  e.fixture_b = fb;
  e.point_count = pc;
  for (int k = 0; k < 2; ++k) {
    e.normal_impulses[k] = ni ? ni[k] : 0.0f;
    e.tangent_impulses[k] = ti ? ti[k] : 0.0f;
  }
  if (old) e.old_manifold = *old;
  w->events.push_back(e);
}

// b2Body::SetAwake (include/box2d/b2_body.h:719-740).
static void setAwake(Body& b, bool flag) {
  if (b.type == 0) return;
  if (flag) {
    b.flags |= B2G_BODY_AWAKE;
    b.sleepTime = 0.0f;
  } else {
    b.flags &= ~B2G_BODY_AWAKE;
    b.sleepTime = 0.0f;
    b.v = v2(0.0f, 0.0f);
    b.w = 0.0f;
    b.force = v2(0.0f, 0.0f);
    b.torque = 0.0f;
  }
}

static void rebuildNoCollide(World* w) {
  w->noCollide.clear();
  for (const Joint& j : w->joints) {
    if (j.d.collide_connected) continue;
    uint32_t a = (uint32_t)j.d.body_a, b = (uint32_t)j.d.body_b;
    if (a > b) std::swap(a, b);
    w->noCollide.push_back(((uint64_t)a << 32) | b);
  }
  std::sort(w->noCollide.begin(), w->noCollide.end());
}

// b2Body::ShouldCollide (src/dynamics/b2_body.cpp:459-480) + b2ContactFilter::ShouldCollide
// (src/dynamics/b2_world_callbacks.cpp:28-39).
static bool shouldCollide(const World& w, int fi, int fj) {
  const Fixture& a = w.fixtures[fi];
  const Fixture& b = w.fixtures[fj];
  if (a.body == b.body) return false;
  const Body& ba = w.bodies[a.body];
  const Body& bb = w.bodies[b.body];
  if (ba.type != 2 && bb.type != 2) return false;
  uint32_t x = (uint32_t)a.body, y = (uint32_t)b.body;
  if (x > y) std::swap(x, y);
  if (std::binary_search(w.noCollide.begin(), w.noCollide.end(), ((uint64_t)x << 32) | y)) return false;
  if (a.group == b.group && a.group != 0) return a.group > 0;
  return (a.mask & b.category) != 0 && (a.category & b.mask) != 0;
}

// Broadphase: the set of overlapping fixture AABB pairs (reference pair set:
// include/box2d/b2_broad_phase.h:252-343 reports every overlapping pair, QueryCallback
// src/dynamics/b2_contact_manager.cpp:136-188 filters it) in canonical (emitter, partner) order.
// Emitter: the non-static fixture of a static/non-static pair, else the lower index.
static void findPairs(const World& w, const std::vector<AABB>& bb, std::vector<uint64_t>* out) {
  int n = (int)w.fixtures.size();
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::sort(order.begin(), order.end(), [&](int a, int b) {
    if (bb[a].lo.x != bb[b].lo.x) return bb[a].lo.x < bb[b].lo.x;
    return a < b;
  });
  out->clear();
  for (int oi = 0; oi < n; ++oi) {
    int i = order[oi];
    for (int oj = oi + 1; oj < n; ++oj) {
      int j = order[oj];
      if (bb[j].lo.x > bb[i].hi.x) break;
      if (!overlap(bb[i], bb[j])) continue;
      bool si = w.bodies[w.fixtures[i].body].type == 0;
      bool sj = w.bodies[w.fixtures[j].body].type == 0;
      if (si && sj) continue;
      int e, p;
      if (si) { e = j; p = i; }
      else if (sj) { e = i; p = j; }
      else { e = bmin(i, j); p = bmax(i, j); }
      if (!shouldCollide(w, e, p)) continue;
      if (!hasCollider(w.fixtures[e].shape.type, w.fixtures[p].shape.type) &&
          !hasCollider(w.fixtures[p].shape.type, w.fixtures[e].shape.type))
        continue;
      out->push_back(((uint64_t)(uint32_t)e << 32) | (uint32_t)p);
    }
  }
  std::sort(out->begin(), out->end());
}

// b2Contact::b2Contact (src/dynamics/b2_contact.cpp:96-122) with b2Contact::Create's orientation
// (:58-77); mixing laws include/box2d/b2_contact.h:42-60.
static Contact makeContact(const World& w, uint64_t key) {
  Contact c;
  memset(&c, 0, sizeof(c));
  int e = (int)(key >> 32), p = (int)(uint32_t)key;
  int te = w.fixtures[e].shape.type, tp = w.fixtures[p].shape.type;
  if (hasCollider(te, tp)) { c.fA = e; c.fB = p; }
  else { c.fA = p; c.fB = e; }
  c.key = key;
  c.flags = B2G_CONTACT_ENABLED;
  c.m.pointCount = 0;
  const Fixture& fa = w.fixtures[c.fA];
  const Fixture& fb = w.fixtures[c.fB];
  c.friction = sqrtf(fa.friction * fb.friction);
  c.restitution = fa.restitution > fb.restitution ? fa.restitution : fb.restitution;
  c.threshold = fa.threshold < fb.threshold ? fa.threshold : fb.threshold;
  c.tangentSpeed = 0.0f;
  return c;
}

// FindNewContacts + RemoveDeadContacts (src/dynamics/b2_contact_manager.cpp:118-134): the new
// contact list is the pair list; persisting contacts keep their state.
static void updatePairs(World* w) {
  int nf = (int)w->fixtures.size();
  std::vector<AABB> bb(nf);
  for (int i = 0; i < nf; ++i) bb[i] = computeAABB(w->fixtures[i].shape, w->bodies[w->fixtures[i].body].xf);
  std::vector<uint64_t> pairs;
  findPairs(*w, bb, &pairs);
  w->aabb = bb;
  std::vector<Contact> next;
  next.reserve(pairs.size());
  std::vector<char> kept(w->contacts.size(), 0);
  size_t k = 0;
  for (uint64_t key : pairs) {
    while (k < w->contacts.size() && w->contacts[k].key < key) ++k;
    if (k < w->contacts.size() && w->contacts[k].key == key) {
      next.push_back(w->contacts[k]);
      kept[k] = 1;
    } else {
      next.push_back(makeContact(*w, key));
    }
  }
  // EndContact for the touching contacts dropped (b2ContactManager::Destroy,
  // src/dynamics/b2_contact_manager.cpp:48-61)
  if (w->recordEvents)
    for (size_t i = 0; i < w->contacts.size(); ++i) {
      const Contact& c = w->contacts[i];
      if (!kept[i] && (c.flags & B2G_CONTACT_TOUCHING)) recordEvent(w, B2G_EVENT_END, c.fA, c.fB);
    }
  // b2Contact::Destroy wakes both bodies of a destroyed contact with manifold points
  // (src/dynamics/b2_contact.cpp:80-91)
  if (w->sleepMode())
    for (size_t i = 0; i < w->contacts.size(); ++i) {
      const Contact& c = w->contacts[i];
      if (kept[i] || !(c.flags & B2G_CONTACT_TOUCHING)) continue;
      if (w->fixtures[c.fA].sensor || w->fixtures[c.fB].sensor) continue;
      setAwake(w->bodies[w->fixtures[c.fA].body], true);
      setAwake(w->bodies[w->fixtures[c.fB].body], true);
    }
  w->contacts.swap(next);
}

// ---- GJK distance (src/collision/b2_distance.cpp:31-579) for b2TestOverlap
// (src/collision/b2_collision.cpp:239-258): empty simplex cache, radii applied.
struct SV { V2 wA, wB, w; float a; int iA, iB; };
static int gjkCount(const Shape& s) { return s.type == 0 ? 1 : (s.type == 1 ? 2 : s.count); }
static V2 gjkVertex(const Shape& s, int i) { return s.v[i]; }  // circle p, edge v1 v2, polygon vertices
static int gjkSupport(const Shape& s, V2 d) {
  int best = 0;
  float bestValue = dot(gjkVertex(s, 0), d);
  for (int i = 1; i < gjkCount(s); ++i) {
    float value = dot(gjkVertex(s, i), d);
    if (value > bestValue) { best = i; bestValue = value; }
  }
  return best;
}
static float gjkDistance(const Shape& A, const Xf& xfA, const Shape& B, const Xf& xfB) {
  SV sv[3];
  int n = 1;
  sv[0].iA = 0; sv[0].iB = 0;
  sv[0].wA = mul(xfA, gjkVertex(A, 0));
  sv[0].wB = mul(xfB, gjkVertex(B, 0));
  sv[0].w = sv[0].wB - sv[0].wA;
  sv[0].a = 1.0f;
  int saveA[3], saveB[3];
  int iter = 0;
  while (iter < 20) {
    int saveCount = n;
    for (int i = 0; i < saveCount; ++i) { saveA[i] = sv[i].iA; saveB[i] = sv[i].iB; }
    if (n == 2) {  // b2Simplex::Solve2
      V2 w1 = sv[0].w, w2 = sv[1].w, e12 = w2 - w1;
      float d12_2 = -dot(w1, e12);
      if (d12_2 <= 0.0f) { sv[0].a = 1.0f; n = 1; }
      else {
        float d12_1 = dot(w2, e12);
        if (d12_1 <= 0.0f) { sv[1].a = 1.0f; n = 1; sv[0] = sv[1]; }
        else {
          float inv = 1.0f / (d12_1 + d12_2);
          sv[0].a = d12_1 * inv; sv[1].a = d12_2 * inv; n = 2;
        }
      }
    } else if (n == 3) {  // b2Simplex::Solve3
      V2 w1 = sv[0].w, w2 = sv[1].w, w3 = sv[2].w;
      V2 e12 = w2 - w1;
      float d12_1 = dot(w2, e12), d12_2 = -dot(w1, e12);
      V2 e13 = w3 - w1;
      float d13_1 = dot(w3, e13), d13_2 = -dot(w1, e13);
      V2 e23 = w3 - w2;
      float d23_1 = dot(w3, e23), d23_2 = -dot(w2, e23);
      float n123 = cross(e12, e13);
      float d123_1 = n123 * cross(w2, w3);
      float d123_2 = n123 * cross(w3, w1);
      float d123_3 = n123 * cross(w1, w2);
      if (d12_2 <= 0.0f && d13_2 <= 0.0f) { sv[0].a = 1.0f; n = 1; }
      else if (d12_1 > 0.0f && d12_2 > 0.0f && d123_3 <= 0.0f) {
        float inv = 1.0f / (d12_1 + d12_2);
        sv[0].a = d12_1 * inv; sv[1].a = d12_2 * inv; n = 2;
      } else if (d13_1 > 0.0f && d13_2 > 0.0f && d123_2 <= 0.0f) {
        float inv = 1.0f / (d13_1 + d13_2);
        sv[0].a = d13_1 * inv; sv[2].a = d13_2 * inv; n = 2; sv[1] = sv[2];
      } else if (d12_1 <= 0.0f && d23_2 <= 0.0f) { sv[1].a = 1.0f; n = 1; sv[0] = sv[1]; }
      else if (d13_1 <= 0.0f && d23_1 <= 0.0f) { sv[2].a = 1.0f; n = 1; sv[0] = sv[2]; }
      else if (d23_1 > 0.0f && d23_2 > 0.0f && d123_1 <= 0.0f) {
        float inv = 1.0f / (d23_1 + d23_2);
        sv[1].a = d23_1 * inv; sv[2].a = d23_2 * inv; n = 2; sv[0] = sv[2];
      } else {
        float inv = 1.0f / (d123_1 + d123_2 + d123_3);
        sv[0].a = d123_1 * inv; sv[1].a = d123_2 * inv; sv[2].a = d123_3 * inv; n = 3;
      }
    }
    if (n == 3) break;
    V2 d;
    if (n == 1) d = -sv[0].w;
    else {
      V2 e12 = sv[1].w - sv[0].w;
      float sgn = cross(e12, -sv[0].w);
      d = sgn > 0.0f ? cross(1.0f, e12) : cross(e12, 1.0f);
    }
    if (lengthSq(d) < kEpsilon * kEpsilon) break;
    SV& nv = sv[n];
    nv.iA = gjkSupport(A, mulT(xfA.q, -d));
    nv.wA = mul(xfA, gjkVertex(A, nv.iA));
    nv.iB = gjkSupport(B, mulT(xfB.q, d));
    nv.wB = mul(xfB, gjkVertex(B, nv.iB));
    nv.w = nv.wB - nv.wA;
    ++iter;
    bool duplicate = false;
    for (int i = 0; i < saveCount; ++i)
      if (nv.iA == saveA[i] && nv.iB == saveB[i]) { duplicate = true; break; }
    if (duplicate) break;
    ++n;
  }
  V2 pA, pB;
  if (n == 1) { pA = sv[0].wA; pB = sv[0].wB; }
  else if (n == 2) {
    pA = sv[0].a * sv[0].wA + sv[1].a * sv[1].wA;
    pB = sv[0].a * sv[0].wB + sv[1].a * sv[1].wB;
  } else {
    pA = sv[0].a * sv[0].wA + sv[1].a * sv[1].wA + sv[2].a * sv[2].wA;
    pB = pA;
  }
  float distance = lengthOf(pA - pB);
  float rA = A.radius, rB = B.radius;
  if (distance > rA + rB && distance > kEpsilon) return distance - (rA + rB);
  return 0.0f;
}
static bool testOverlap(const Shape& A, const Xf& xfA, const Shape& B, const Xf& xfB) {
  return gjkDistance(A, xfA, B, xfB) < 10.0f * kEpsilon;
}

// ---- time of impact: b2TimeOfImpact (src/collision/b2_time_of_impact.cpp:258-490) over
// b2Distance with a simplex cache (src/collision/b2_distance.cpp:86-135, 432-579) and the
// separating-axis function b2SeparationFunction (b2_time_of_impact.cpp:35-251).
struct Sweep { V2 localCenter, c0, c; float a0, a, alpha0; };
// b2Sweep::GetTransform / Normalize (include/box2d/b2_math.h:707-733; Advance below on bodies)
static Xf sweepTransform(const Sweep& s, float beta) {
  Xf xf;
  xf.p = (1.0f - beta) * s.c0 + beta * s.c;
  float angle = (1.0f - beta) * s.a0 + beta * s.a;
  xf.q = rotOf(angle);
  subFrom(xf.p, mul(xf.q, s.localCenter));
  return xf;
}
static void sweepNormalize(Sweep& s) {
  float twoPi = 2.0f * kPi;
  float d = twoPi * floorf(s.a0 / twoPi);
  s.a0 -= d;
  s.a -= d;
}

struct SimplexCache { float metric; int count; int iA[3], iB[3]; };

// b2Simplex with its cache round trip; solve2/solve3 as in gjkDistance above.
struct Simplex {
  SV v[3];
  int n;
  float metric() const {
    if (n == 2) { V2 c = v[0].w - v[1].w; return lengthOf(c); }
    if (n == 3) return cross(v[1].w - v[0].w, v[2].w - v[0].w);
    return 0.0f;
  }
  void setVertex(int i, int iA, int iB, const Shape& A, const Xf& xfA, const Shape& B, const Xf& xfB) {
    v[i].iA = iA;
    v[i].iB = iB;
    v[i].wA = mul(xfA, gjkVertex(A, iA));
    v[i].wB = mul(xfB, gjkVertex(B, iB));
    v[i].w = v[i].wB - v[i].wA;
  }
  void readCache(const SimplexCache& c, const Shape& A, const Xf& xfA, const Shape& B, const Xf& xfB) {
    n = c.count;
    for (int i = 0; i < n; ++i) {
      setVertex(i, c.iA[i], c.iB[i], A, xfA, B, xfB);
      v[i].a = 0.0f;
    }
    if (n > 1) {
      float m1 = c.metric, m2 = metric();
      if (m2 < 0.5f * m1 || 2.0f * m1 < m2 || m2 < kEpsilon) n = 0;
    }
    if (n == 0) {
      setVertex(0, 0, 0, A, xfA, B, xfB);
      v[0].a = 1.0f;
      n = 1;
    }
  }
  void writeCache(SimplexCache& c) const {
    c.metric = metric();
    c.count = n;
    for (int i = 0; i < n; ++i) { c.iA[i] = v[i].iA; c.iB[i] = v[i].iB; }
  }
  void solve2() {
    V2 w1 = v[0].w, w2 = v[1].w, e12 = w2 - w1;
    float d12_2 = -dot(w1, e12);
    if (d12_2 <= 0.0f) { v[0].a = 1.0f; n = 1; return; }
    float d12_1 = dot(w2, e12);
    if (d12_1 <= 0.0f) { v[1].a = 1.0f; n = 1; v[0] = v[1]; return; }
    float inv = 1.0f / (d12_1 + d12_2);
    v[0].a = d12_1 * inv; v[1].a = d12_2 * inv; n = 2;
  }
  void solve3() {
    V2 w1 = v[0].w, w2 = v[1].w, w3 = v[2].w;
    V2 e12 = w2 - w1;
    float d12_1 = dot(w2, e12), d12_2 = -dot(w1, e12);
    V2 e13 = w3 - w1;
    float d13_1 = dot(w3, e13), d13_2 = -dot(w1, e13);
    V2 e23 = w3 - w2;
    float d23_1 = dot(w3, e23), d23_2 = -dot(w2, e23);
    float n123 = cross(e12, e13);
    float d123_1 = n123 * cross(w2, w3), d123_2 = n123 * cross(w3, w1), d123_3 = n123 * cross(w1, w2);
    if (d12_2 <= 0.0f && d13_2 <= 0.0f) { v[0].a = 1.0f; n = 1; return; }
    if (d12_1 > 0.0f && d12_2 > 0.0f && d123_3 <= 0.0f) {
      float inv = 1.0f / (d12_1 + d12_2);
      v[0].a = d12_1 * inv; v[1].a = d12_2 * inv; n = 2; return;
    }
    if (d13_1 > 0.0f && d13_2 > 0.0f && d123_2 <= 0.0f) {
      float inv = 1.0f / (d13_1 + d13_2);
      v[0].a = d13_1 * inv; v[2].a = d13_2 * inv; n = 2; v[1] = v[2]; return;
    }
    if (d12_1 <= 0.0f && d23_2 <= 0.0f) { v[1].a = 1.0f; n = 1; v[0] = v[1]; return; }
    if (d13_1 <= 0.0f && d23_1 <= 0.0f) { v[2].a = 1.0f; n = 1; v[0] = v[2]; return; }
    if (d23_1 > 0.0f && d23_2 > 0.0f && d123_1 <= 0.0f) {
      float inv = 1.0f / (d23_1 + d23_2);
      v[1].a = d23_1 * inv; v[2].a = d23_2 * inv; n = 2; v[0] = v[2]; return;
    }
    float inv = 1.0f / (d123_1 + d123_2 + d123_3);
    v[0].a = d123_1 * inv; v[1].a = d123_2 * inv; v[2].a = d123_3 * inv; n = 3;
  }
};

// b2Distance with useRadii = false: the distance between the witness points.
static float gjkCached(const Shape& A, const Xf& xfA, const Shape& B, const Xf& xfB, SimplexCache& cache) {
  Simplex s;
  s.readCache(cache, A, xfA, B, xfB);
  int saveA[3], saveB[3];
  int iter = 0;
  while (iter < 20) {
    int saveCount = s.n;
    for (int i = 0; i < saveCount; ++i) { saveA[i] = s.v[i].iA; saveB[i] = s.v[i].iB; }
    if (s.n == 2) s.solve2();
    else if (s.n == 3) s.solve3();
    if (s.n == 3) break;
    V2 d;
    if (s.n == 1) d = -s.v[0].w;
    else {
      V2 e12 = s.v[1].w - s.v[0].w;
      d = cross(e12, -s.v[0].w) > 0.0f ? cross(1.0f, e12) : cross(e12, 1.0f);
    }
    if (lengthSq(d) < kEpsilon * kEpsilon) break;
    int iA = gjkSupport(A, mulT(xfA.q, -d));
    int iB = gjkSupport(B, mulT(xfB.q, d));
    s.setVertex(s.n, iA, iB, A, xfA, B, xfB);
    ++iter;
    bool duplicate = false;
    for (int i = 0; i < saveCount; ++i)
      if (iA == saveA[i] && iB == saveB[i]) { duplicate = true; break; }
    if (duplicate) break;
    ++s.n;
  }
  V2 pA, pB;
  if (s.n == 1) { pA = s.v[0].wA; pB = s.v[0].wB; }
  else if (s.n == 2) {
    pA = s.v[0].a * s.v[0].wA + s.v[1].a * s.v[1].wA;
    pB = s.v[0].a * s.v[0].wB + s.v[1].a * s.v[1].wB;
  } else {
    pA = s.v[0].a * s.v[0].wA + s.v[1].a * s.v[1].wA + s.v[2].a * s.v[2].wA;
    pB = pA;
  }
  s.writeCache(cache);
  V2 c = pA - pB;
  return lengthOf(c);
}

struct Separation {
  enum Kind { kPoints, kFaceA, kFaceB };
  const Shape *A, *B;
  Sweep sA, sB;
  Kind kind;
  V2 localPoint, axis;

  float init(const SimplexCache& cache, const Shape& pa, const Sweep& wa, const Shape& pb, const Sweep& wb, float t1) {
    A = &pa; B = &pb; sA = wa; sB = wb;
    Xf xfA = sweepTransform(sA, t1), xfB = sweepTransform(sB, t1);
    if (cache.count == 1) {
      kind = kPoints;
      axis = mul(xfB, gjkVertex(*B, cache.iB[0])) - mul(xfA, gjkVertex(*A, cache.iA[0]));
      return normalize(axis);
    }
    const bool faceB = cache.iA[0] == cache.iA[1];
    const Shape& F = faceB ? *B : *A;
    const Shape& P = faceB ? *A : *B;
    const Xf& xfF = faceB ? xfB : xfA;
    const Xf& xfP = faceB ? xfA : xfB;
    const int* fi = faceB ? cache.iB : cache.iA;
    const int pi = faceB ? cache.iA[0] : cache.iB[0];
    kind = faceB ? kFaceB : kFaceA;
    V2 l1 = gjkVertex(F, fi[0]), l2 = gjkVertex(F, fi[1]);
    axis = cross(l2 - l1, 1.0f);
    normalize(axis);
    V2 normal = mul(xfF.q, axis);
    localPoint = 0.5f * (l1 + l2);
    V2 pointF = mul(xfF, localPoint);
    V2 pointP = mul(xfP, gjkVertex(P, pi));
    float s = dot(pointP - pointF, normal);
    if (s < 0.0f) { axis = -axis; s = -s; }
    return s;
  }
  float findMin(int* iA, int* iB, float t) const {
    Xf xfA = sweepTransform(sA, t), xfB = sweepTransform(sB, t);
    if (kind == kPoints) {
      *iA = gjkSupport(*A, mulT(xfA.q, axis));
      *iB = gjkSupport(*B, mulT(xfB.q, -axis));
      return dot(mul(xfB, gjkVertex(*B, *iB)) - mul(xfA, gjkVertex(*A, *iA)), axis);
    }
    if (kind == kFaceA) {
      V2 normal = mul(xfA.q, axis);
      V2 pointA = mul(xfA, localPoint);
      *iA = -1;
      *iB = gjkSupport(*B, mulT(xfB.q, -normal));
      return dot(mul(xfB, gjkVertex(*B, *iB)) - pointA, normal);
    }
    V2 normal = mul(xfB.q, axis);
    V2 pointB = mul(xfB, localPoint);
    *iB = -1;
    *iA = gjkSupport(*A, mulT(xfA.q, -normal));
    return dot(mul(xfA, gjkVertex(*A, *iA)) - pointB, normal);
  }
  float evaluate(int iA, int iB, float t) const {
    Xf xfA = sweepTransform(sA, t), xfB = sweepTransform(sB, t);
    if (kind == kPoints) return dot(mul(xfB, gjkVertex(*B, iB)) - mul(xfA, gjkVertex(*A, iA)), axis);
    if (kind == kFaceA) return dot(mul(xfB, gjkVertex(*B, iB)) - mul(xfA, localPoint), mul(xfA.q, axis));
    return dot(mul(xfA, gjkVertex(*A, iA)) - mul(xfB, localPoint), mul(xfB.q, axis));
  }
};

// b2TimeOfImpact: the state (B2G_TOI_*) and the time in [0, tMax] written to *t.
static int timeOfImpact(const Shape& A, const Shape& B, Sweep sA, Sweep sB, float tMax, float* t) {
  *t = tMax;
  sweepNormalize(sA);
  sweepNormalize(sB);
  const float target = bmax(kLinearSlop, (A.radius + B.radius) - 3.0f * kLinearSlop);
  const float tolerance = 0.25f * kLinearSlop;
  float t1 = 0.0f;
  SimplexCache cache;
  cache.count = 0;
  cache.metric = 0.0f;
  for (int iter = 1;; ++iter) {
    float distance = gjkCached(A, sweepTransform(sA, t1), B, sweepTransform(sB, t1), cache);
    if (distance <= 0.0f) { *t = 0.0f; return B2G_TOI_OVERLAPPED; }
    if (distance < target + tolerance) { *t = t1; return B2G_TOI_TOUCHING; }
    Separation fcn;
    fcn.init(cache, A, sA, B, sB, t1);
    float t2 = tMax;
    for (int push = 1;; ++push) {
      int iA, iB;
      float s2 = fcn.findMin(&iA, &iB, t2);
      if (s2 > target + tolerance) { *t = tMax; return B2G_TOI_SEPARATED; }
      if (s2 > target - tolerance) { t1 = t2; break; }
      float s1 = fcn.evaluate(iA, iB, t1);
      if (s1 < target - tolerance) { *t = t1; return B2G_TOI_FAILED; }
      if (s1 <= target + tolerance) { *t = t1; return B2G_TOI_TOUCHING; }
      float a1 = t1, a2 = t2;
      for (int root = 0; root < 50;) {
        float tm = (root & 1) ? a1 + (target - s1) * (a2 - a1) / (s2 - s1) : 0.5f * (a1 + a2);
        ++root;
        float s = fcn.evaluate(iA, iB, tm);
        if (babs(s - target) < tolerance) { t2 = tm; break; }
        if (s > target) { a1 = tm; s1 = s; }
        else { a2 = tm; s2 = s; }
      }
      if (push == 8) break;  // b2_maxPolygonVertices
    }
    if (iter == 20) { *t = t1; return B2G_TOI_FAILED; }
  }
}

// b2Contact::Update (src/dynamics/b2_contact.cpp:126-210) for one contact; returns whether
// touching changed on a non-sensor contact (which wakes both bodies, :183-188).
static bool updateContact(World* w, Contact& c) {
  Manifold old = c.m;
  const bool wasTouching = (c.flags & B2G_CONTACT_TOUCHING) != 0;
  c.flags |= B2G_CONTACT_ENABLED;
  const Fixture& fa = w->fixtures[c.fA];
  const Fixture& fb = w->fixtures[c.fB];
  bool touching = false;
  if (fa.sensor || fb.sensor) {
    touching = testOverlap(fa.shape, w->bodies[fa.body].xf, fb.shape, w->bodies[fb.body].xf);
    c.m.pointCount = 0;
  } else {
    evaluate(&c.m, fa.shape, w->bodies[fa.body].xf, fb.shape, w->bodies[fb.body].xf);
    touching = c.m.pointCount > 0;
    for (int i = 0; i < c.m.pointCount; ++i) {
      MPoint* mp2 = c.m.points + i;
      mp2->normalImpulse = 0.0f;
      mp2->tangentImpulse = 0.0f;
      for (int j = 0; j < old.pointCount; ++j) {
        if (old.points[j].id == mp2->id) {
          mp2->normalImpulse = old.points[j].normalImpulse;
          mp2->tangentImpulse = old.points[j].tangentImpulse;
          break;
        }
      }
    }
  }
  if (touching) c.flags |= B2G_CONTACT_TOUCHING;
  else c.flags &= ~B2G_CONTACT_TOUCHING;
  if (w->recordEvents) {  // b2_contact.cpp:197-209
    const bool sensor = fa.sensor || fb.sensor;
    if (!wasTouching && touching) recordEvent(w, B2G_EVENT_BEGIN, c.fA, c.fB);
    if (wasTouching && !touching) recordEvent(w, B2G_EVENT_END, c.fA, c.fB);
    if (!sensor && touching) {
      b2g_manifold om;
      manifoldTo(old, &om);
      recordEvent(w, B2G_EVENT_PRESOLVE, c.fA, c.fB, &om);
    }
  }
  return !fa.sensor && !fb.sensor && touching != wasTouching;
}

// b2ContactManager::Collide (src/dynamics/b2_contact_manager.cpp:66-116). Sleep mode: a contact
// is updated when one of its bodies was awake at the start of the pass (static bodies never are),
// or, as a wake closure, once one of its bodies has been woken by another contact's touching
// change in this pass; wakes apply after the pass. The reference's single sequential pass gives
// the same result whenever a waking contact precedes the contacts it wakes (its list keeps the
// newest contacts first); the closure does not depend on the list order.
static void collide(World* w) {
  const bool sleepMode = w->sleepMode();
  const size_t n = w->contacts.size();
  std::vector<char> evaluated(n, 0), wake(w->bodies.size(), 0);
  auto mark = [&](const Contact& c) {
    int a = w->fixtures[c.fA].body, b = w->fixtures[c.fB].body;
    bool fresh = false;
    if (w->bodies[a].type != 0 && !wake[a]) { wake[a] = 1; fresh = true; }
    if (w->bodies[b].type != 0 && !wake[b]) { wake[b] = 1; fresh = true; }
    return fresh;
  };
  for (size_t k = 0; k < n; ++k) {
    Contact& c = w->contacts[k];
    if (sleepMode && !w->bodies[w->fixtures[c.fA].body].awake() && !w->bodies[w->fixtures[c.fB].body].awake())
      continue;
    evaluated[k] = 1;
    if (updateContact(w, c) && sleepMode) mark(c);
  }
  if (!sleepMode) return;
  for (bool changed = true; changed;) {
    changed = false;
    for (size_t k = 0; k < n; ++k) {
      Contact& c = w->contacts[k];
      if (evaluated[k] || (!wake[w->fixtures[c.fA].body] && !wake[w->fixtures[c.fB].body])) continue;
      evaluated[k] = 1;
      if (updateContact(w, c) && mark(c)) changed = true;
    }
  }
  for (size_t b = 0; b < wake.size(); ++b)
    if (wake[b]) setAwake(w->bodies[b], true);
}

// Greedy colouring in priority order: each constraint takes the lowest colour not used by an
// earlier (higher-priority) constraint sharing a non-static body; 63 = overflow (serial).
static void colorConstraints(int n, const int* bodyA, const int* bodyB, const uint32_t* prio,
                             const std::vector<Body>& bodies, std::vector<int>* color) {
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::sort(order.begin(), order.end(), [&](int a, int b) {
    if (prio[a] != prio[b]) return prio[a] < prio[b];
    return a < b;
  });
  std::vector<uint64_t> mask(bodies.size(), 0);
  color->assign(n, -1);
  for (int idx : order) {
    int a = bodyA[idx], b = bodyB[idx];
    if (a < 0) {  // a constraint solved serially (gear joint): the overflow colour
      (*color)[idx] = kOverflow;
      continue;
    }
    bool sa = bodies[a].type == 0, sb = bodies[b].type == 0;
    uint64_t used = (sa ? 0 : mask[a]) | (sb ? 0 : mask[b]);
    uint64_t freeBits = ~used & ((1ull << kOverflow) - 1);
    int col;
    if (freeBits == 0) col = kOverflow;
    else {
      col = __builtin_ctzll(freeBits);
      if (!sa) mask[a] |= 1ull << col;
      if (!sb) mask[b] |= 1ull << col;
    }
    (*color)[idx] = col;
  }
}

// Solve order: colour by colour; within a colour by (priority, index).
static std::vector<int> solveOrder(int n, const std::vector<int>& color, const uint32_t* prio) {
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::sort(order.begin(), order.end(), [&](int a, int b) {
    if (color[a] != color[b]) return color[a] < color[b];
    if (prio[a] != prio[b]) return prio[a] < prio[b];
    return a < b;
  });
  return order;
}

struct SolverBody { V2 c; float a; V2 v; float w; };

// ---- joints (src/dynamics/b2_revolute_joint.cpp, b2_prismatic_joint.cpp, b2_distance_joint.cpp)
struct Step { float dt, inv_dt, dtRatio; int vi, pi; bool warm; };

// b2Mat33 of the weld joint, GetInverse22 / GetSymInverse33 / Solve22 (src/common/b2_math.cpp:42-97),
// stored as ex, ey, ez.
static void weldK(V2 rA, V2 rB, float mA, float mB, float iA, float iB, V3& ex, V3& ey, V3& ez) {
  ex.x = mA + mB + rA.y * rA.y * iA + rB.y * rB.y * iB;
  ey.x = -rA.y * rA.x * iA - rB.y * rB.x * iB;
  ez.x = -rA.y * iA - rB.y * iB;
  ex.y = ey.x;
  ey.y = mA + mB + rA.x * rA.x * iA + rB.x * rB.x * iB;
  ez.y = rA.x * iA + rB.x * iB;
  ex.z = ez.x;
  ey.z = ez.y;
  ez.z = iA + iB;
}
static void inverse22(V3 ex, V3 ey, float* M) {
  float a = ex.x, b = ey.x, c = ex.y, d = ey.y;
  float det = a * d - b * c;
  if (det != 0.0f) det = 1.0f / det;
  M[0] = det * d; M[1] = -det * c; M[2] = 0.0f;
  M[3] = -det * b; M[4] = det * a; M[5] = 0.0f;
  M[6] = M[7] = M[8] = 0.0f;
}
static void symInverse33(V3 ex, V3 ey, V3 ez, float* M) {
  float det = dot3(ex, cross3(ey, ez));
  if (det != 0.0f) det = 1.0f / det;
  float a11 = ex.x, a12 = ey.x, a13 = ez.x, a22 = ey.y, a23 = ez.y, a33 = ez.z;
  M[0] = det * (a22 * a33 - a23 * a23);
  M[1] = det * (a13 * a23 - a12 * a33);
  M[2] = det * (a12 * a23 - a13 * a22);
  M[3] = M[1];
  M[4] = det * (a11 * a33 - a13 * a13);
  M[5] = det * (a13 * a12 - a11 * a23);
  M[6] = M[2];
  M[7] = M[5];
  M[8] = det * (a11 * a22 - a12 * a12);
}
static V2 solve22(V3 ex, V3 ey, V2 b) {
  float a11 = ex.x, a12 = ey.x, a21 = ex.y, a22 = ey.y;
  float det = a11 * a22 - a12 * a21;
  if (det != 0.0f) det = 1.0f / det;
  return v2(det * (a22 * b.x - a12 * b.y), det * (a11 * b.y - a21 * b.x));
}
// Linear mass (inverse of K) and angular mass of the motor and friction joints
// (b2_motor_joint.cpp:91-104, b2_friction_joint.cpp:88-101).
static void linearAngularMass(Joint& J, float mA, float mB, float iA, float iB) {
  M22 K;
  K.ex.x = mA + mB + iA * J.rA.y * J.rA.y + iB * J.rB.y * J.rB.y;
  K.ex.y = -iA * J.rA.x * J.rA.y - iB * J.rB.x * J.rB.y;
  K.ey.x = K.ex.y;
  K.ey.y = mA + mB + iA * J.rA.x * J.rA.x + iB * J.rB.x * J.rB.x;
  J.K = inverse(K);
  J.axialMass = iA + iB;
  if (J.axialMass > 0.0f) J.axialMass = 1.0f / J.axialMass;
}
// Clamped angular then linear impulse of the motor joint (with its position feedback,
// b2_motor_joint.cpp:157-193) and the friction joint (without, b2_friction_joint.cpp:144-180).
static void solveLinearAngular(Joint& J, V2& vA, float& wA, V2& vB, float& wB, float h, bool motor, float inv_h) {
  float mA = J.mA, mB = J.mB, iA = J.invIA, iB = J.invIB;
  {
    float Cdot = motor ? wB - wA + inv_h * J.d.correction_factor * J.angularError : wB - wA;
    float impulse = -J.axialMass * Cdot;
    float oldImpulse = J.imp[2];
    float maxImpulse = h * J.d.max_torque;
    J.imp[2] = bclamp(J.imp[2] + impulse, -maxImpulse, maxImpulse);
    impulse = J.imp[2] - oldImpulse;
    wA -= iA * impulse;
    wB += iB * impulse;
  }
  {
    V2 Cdot = motor ? vB + cross(wB, J.rB) - vA - cross(wA, J.rA) + inv_h * J.d.correction_factor * J.err
                    : vB + cross(wB, J.rB) - vA - cross(wA, J.rA);
    V2 impulse = -mul(J.K, Cdot);
    V2 oldImpulse = v2(J.imp[0], J.imp[1]);
    V2 li = oldImpulse;
    addTo(li, impulse);
    float maxImpulse = h * J.d.max_force;
    if (lengthSq(li) > maxImpulse * maxImpulse) {
      normalize(li);
      li.x *= maxImpulse;
      li.y *= maxImpulse;
    }
    J.imp[0] = li.x; J.imp[1] = li.y;
    impulse = li - oldImpulse;
    subFrom(vA, mA * impulse);
    wA -= iA * cross(J.rA, impulse);
    addTo(vB, mB * impulse);
    wB += iB * cross(J.rB, impulse);
  }
}

// ---- gear joint (src/dynamics/b2_gear_joint.cpp:141-372), four bodies
// Jacobian rows and summed effective mass at rotations qA..qD (:178-216, :290-332).
static float gearRows(Joint& J, Rot qA, Rot qB, Rot qC, Rot qD, V2& JvAC, V2& JvBD, float& JwA, float& JwB,
                      float& JwC, float& JwD) {
  const float ratio = J.d.ratio;
  float mass = 0.0f;
  if (J.typeA == B2G_JOINT_REVOLUTE) {
    JvAC = v2(0.0f, 0.0f);
    JwA = 1.0f;
    JwC = 1.0f;
    mass += J.giA + J.giC;
  } else {
    V2 u = mul(qC, J.gAxC);
    V2 rC = mul(qC, J.gLC - J.gLcC);
    V2 rA = mul(qA, J.gLA - J.gLcA);
    JvAC = u;
    JwC = cross(rC, u);
    JwA = cross(rA, u);
    mass += J.gmC + J.gmA + J.giC * JwC * JwC + J.giA * JwA * JwA;
  }
  if (J.typeB == B2G_JOINT_REVOLUTE) {
    JvBD = v2(0.0f, 0.0f);
    JwB = ratio;
    JwD = ratio;
    mass += ratio * ratio * (J.giB + J.giD);
  } else {
    V2 u = mul(qD, J.gAxD);
    V2 rD = mul(qD, J.gLD - J.gLcD);
    V2 rB = mul(qB, J.gLB - J.gLcB);
    JvBD = ratio * u;
    JwD = ratio * cross(rD, u);
    JwB = ratio * cross(rB, u);
    mass += ratio * ratio * (J.gmD + J.gmB) + J.giD * JwD * JwD + J.giB * JwB * JwB;
  }
  return mass;
}

// impulse along the rows, velocities (pos = false) or positions; bodies written A, B, C, D
static void gearApply(Joint& J, std::vector<SolverBody>& sb, bool pos, float impulse, V2 JvAC, V2 JvBD, float JwA,
                      float JwB, float JwC, float JwD) {
  const int a = J.d.body_a, b = J.d.body_b, c = J.iC, d = J.iD;
  V2 xA = pos ? sb[a].c : sb[a].v, xB = pos ? sb[b].c : sb[b].v, xC = pos ? sb[c].c : sb[c].v, xD = pos ? sb[d].c : sb[d].v;
  float tA = pos ? sb[a].a : sb[a].w, tB = pos ? sb[b].a : sb[b].w, tC = pos ? sb[c].a : sb[c].w, tD = pos ? sb[d].a : sb[d].w;
  addTo(xA, (J.gmA * impulse) * JvAC);
  tA += J.giA * impulse * JwA;
  addTo(xB, (J.gmB * impulse) * JvBD);
  tB += J.giB * impulse * JwB;
  xC = xC - (J.gmC * impulse) * JvAC;
  tC -= J.giC * impulse * JwC;
  xD = xD - (J.gmD * impulse) * JvBD;
  tD -= J.giD * impulse * JwD;
  if (pos) {
    sb[a].c = xA; sb[a].a = tA; sb[b].c = xB; sb[b].a = tB; sb[c].c = xC; sb[c].a = tC; sb[d].c = xD; sb[d].a = tD;
  } else {
    sb[a].v = xA; sb[a].w = tA; sb[b].v = xB; sb[b].w = tB; sb[c].v = xC; sb[c].w = tC; sb[d].v = xD; sb[d].w = tD;
  }
}

static void gearInit(Joint& J, const std::vector<Body>& bodies, std::vector<SolverBody>& sb, const Step& st) {
  const Body& bA = bodies[J.d.body_a];
  const Body& bB = bodies[J.d.body_b];
  const Body& bC = bodies[J.iC];
  const Body& bD = bodies[J.iD];
  J.gLcA = bA.localCenter; J.gLcB = bB.localCenter; J.gLcC = bC.localCenter; J.gLcD = bD.localCenter;
  J.gmA = bA.invMass; J.gmB = bB.invMass; J.gmC = bC.invMass; J.gmD = bD.invMass;
  J.giA = bA.invI; J.giB = bB.invI; J.giC = bC.invI; J.giD = bD.invI;
  Rot qA = rotOf(sb[J.d.body_a].a), qB = rotOf(sb[J.d.body_b].a), qC = rotOf(sb[J.iC].a), qD = rotOf(sb[J.iD].a);
  float mass = gearRows(J, qA, qB, qC, qD, J.JvAC, J.JvBD, J.JwA, J.JwB, J.JwC, J.JwD);
  J.gMass = mass > 0.0f ? 1.0f / mass : 0.0f;
  if (st.warm) gearApply(J, sb, false, J.imp[0], J.JvAC, J.JvBD, J.JwA, J.JwB, J.JwC, J.JwD);
  else J.imp[0] = 0.0f;
}

static void gearSolveVelocity(Joint& J, std::vector<SolverBody>& sb) {
  const SolverBody &A = sb[J.d.body_a], &B = sb[J.d.body_b], &Cb = sb[J.iC], &D = sb[J.iD];
  float Cdot = dot(J.JvAC, A.v - Cb.v) + dot(J.JvBD, B.v - D.v);
  Cdot += (J.JwA * A.w - J.JwC * Cb.w) + (J.JwB * B.w - J.JwD * D.w);
  float impulse = -J.gMass * Cdot;
  J.imp[0] += impulse;
  gearApply(J, sb, false, impulse, J.JvAC, J.JvBD, J.JwA, J.JwB, J.JwC, J.JwD);
}

static bool gearSolvePosition(Joint& J, std::vector<SolverBody>& sb) {
  const V2 cA = sb[J.d.body_a].c, cB = sb[J.d.body_b].c, cC = sb[J.iC].c, cD = sb[J.iD].c;
  const float aA = sb[J.d.body_a].a, aB = sb[J.d.body_b].a, aC = sb[J.iC].a, aD = sb[J.iD].a;
  Rot qA = rotOf(aA), qB = rotOf(aB), qC = rotOf(aC), qD = rotOf(aD);
  V2 JvAC, JvBD;
  float JwA, JwB, JwC, JwD;
  float mass = gearRows(J, qA, qB, qC, qD, JvAC, JvBD, JwA, JwB, JwC, JwD);
  float coordinateA, coordinateB;
  if (J.typeA == B2G_JOINT_REVOLUTE) {
    coordinateA = aA - aC - J.gRefA;
  } else {
    V2 rA = mul(qA, J.gLA - J.gLcA);
    V2 pC = J.gLC - J.gLcC;
    V2 pA = mulT(qC, rA + (cA - cC));
    coordinateA = dot(pA - pC, J.gAxC);
  }
  if (J.typeB == B2G_JOINT_REVOLUTE) {
    coordinateB = aB - aD - J.gRefB;
  } else {
    V2 rB = mul(qB, J.gLB - J.gLcB);
    V2 pD = J.gLD - J.gLcD;
    V2 pB = mulT(qD, rB + (cB - cD));
    coordinateB = dot(pB - pD, J.gAxD);
  }
  float C = (coordinateA + J.d.ratio * coordinateB) - J.d.gear_constant;
  float impulse = 0.0f;
  if (mass > 0.0f) impulse = -C / mass;
  gearApply(J, sb, true, impulse, JvAC, JvBD, JwA, JwB, JwC, JwD);
  return true;  // the reference's linear error is always 0 (b2_gear_joint.cpp:370-371)
}

static void jointInit(Joint& J, const std::vector<Body>& bodies, std::vector<SolverBody>& sb, const Step& st) {
  if (J.d.type == B2G_JOINT_GEAR) {
    gearInit(J, bodies, sb, st);
    return;
  }
  const Body& bA = bodies[J.d.body_a];
  const Body& bB = bodies[J.d.body_b];
  J.iA = J.d.body_a; J.iB = J.d.body_b;
  J.lcA = bA.localCenter; J.lcB = bB.localCenter;
  J.mA = bA.invMass; J.mB = bB.invMass; J.invIA = bA.invI; J.invIB = bB.invI;
  V2 cA = sb[J.iA].c; float aA = sb[J.iA].a; V2 vA = sb[J.iA].v; float wA = sb[J.iA].w;
  V2 cB = sb[J.iB].c; float aB = sb[J.iB].a; V2 vB = sb[J.iB].v; float wB = sb[J.iB].w;
  Rot qA = rotOf(aA), qB = rotOf(aB);
  V2 la = v2(J.d.local_anchor_a[0], J.d.local_anchor_a[1]);
  V2 lb = v2(J.d.local_anchor_b[0], J.d.local_anchor_b[1]);
  float mA = J.mA, mB = J.mB, iA = J.invIA, iB = J.invIB;
  if (J.d.type == B2G_JOINT_REVOLUTE) {
    // b2RevoluteJoint::InitVelocityConstraints (b2_revolute_joint.cpp:73-165)
    J.rA = mul(qA, la - J.lcA);
    J.rB = mul(qB, lb - J.lcB);
    J.K.ex.x = mA + mB + J.rA.y * J.rA.y * iA + J.rB.y * J.rB.y * iB;
    J.K.ey.x = -J.rA.y * J.rA.x * iA - J.rB.y * J.rB.x * iB;
    J.K.ex.y = J.K.ey.x;
    J.K.ey.y = mA + mB + J.rA.x * J.rA.x * iA + J.rB.x * J.rB.x * iB;
    J.axialMass = iA + iB;
    bool fixedRotation;
    if (J.axialMass > 0.0f) { J.axialMass = 1.0f / J.axialMass; fixedRotation = false; }
    else fixedRotation = true;
    J.angle = aB - aA - J.d.reference_angle;
    if (J.d.enable_limit == 0 || fixedRotation) { J.lowerImpulse = 0.0f; J.upperImpulse = 0.0f; }
    if (J.d.enable_motor == 0 || fixedRotation) J.motorImpulse = 0.0f;
    if (st.warm) {
      J.impulse2.x *= st.dtRatio; J.impulse2.y *= st.dtRatio;
      J.motorImpulse *= st.dtRatio; J.lowerImpulse *= st.dtRatio; J.upperImpulse *= st.dtRatio;
      float axialImpulse = J.motorImpulse + J.lowerImpulse - J.upperImpulse;
      V2 P = v2(J.impulse2.x, J.impulse2.y);
      subFrom(vA, mA * P);
      wA -= iA * (cross(J.rA, P) + axialImpulse);
      addTo(vB, mB * P);
      wB += iB * (cross(J.rB, P) + axialImpulse);
    } else {
      J.impulse2 = v2(0.0f, 0.0f); J.motorImpulse = 0.0f; J.lowerImpulse = 0.0f; J.upperImpulse = 0.0f;
    }
  } else if (J.d.type == B2G_JOINT_PRISMATIC) {
    // b2PrismaticJoint::InitVelocityConstraints (b2_prismatic_joint.cpp:114-224)
    V2 rA = mul(qA, la - J.lcA);
    V2 rB = mul(qB, lb - J.lcB);
    V2 d = ((cB - cA) + rB) - rA;
    J.axis = mul(qA, J.localXAxisA);
    J.a1 = cross(d + rA, J.axis);
    J.a2 = cross(rB, J.axis);
    J.axialMass = mA + mB + iA * J.a1 * J.a1 + iB * J.a2 * J.a2;
    if (J.axialMass > 0.0f) J.axialMass = 1.0f / J.axialMass;
    J.perp = mul(qA, J.localYAxisA);
    J.s1 = cross(d + rA, J.perp);
    J.s2 = cross(rB, J.perp);
    float k11 = mA + mB + iA * J.s1 * J.s1 + iB * J.s2 * J.s2;
    float k12 = iA * J.s1 + iB * J.s2;
    float k22 = iA + iB;
    if (k22 == 0.0f) k22 = 1.0f;
    J.K.ex = v2(k11, k12);
    J.K.ey = v2(k12, k22);
    if (J.d.enable_limit) J.translation = dot(J.axis, d);
    else { J.lowerImpulse = 0.0f; J.upperImpulse = 0.0f; }
    if (J.d.enable_motor == 0) J.motorImpulse = 0.0f;
    if (st.warm) {
      J.impulse2.x *= st.dtRatio; J.impulse2.y *= st.dtRatio;
      J.motorImpulse *= st.dtRatio; J.lowerImpulse *= st.dtRatio; J.upperImpulse *= st.dtRatio;
      float axialImpulse = J.motorImpulse + J.lowerImpulse - J.upperImpulse;
      V2 P = J.impulse2.x * J.perp + axialImpulse * J.axis;
      float LA = J.impulse2.x * J.s1 + J.impulse2.y + axialImpulse * J.a1;
      float LB = J.impulse2.x * J.s2 + J.impulse2.y + axialImpulse * J.a2;
      subFrom(vA, mA * P);
      wA -= iA * LA;
      addTo(vB, mB * P);
      wB += iB * LB;
    } else {
      J.impulse2 = v2(0.0f, 0.0f); J.motorImpulse = 0.0f; J.lowerImpulse = 0.0f; J.upperImpulse = 0.0f;
    }
  } else if (J.d.type == B2G_JOINT_DISTANCE) {
    // b2DistanceJoint::InitVelocityConstraints (b2_distance_joint.cpp:76-173)
    J.rA = mul(qA, la - J.lcA);
    J.rB = mul(qB, lb - J.lcB);
    J.u = ((cB + J.rB) - cA) - J.rA;
    J.currentLength = lengthOf(J.u);
    if (J.currentLength > kLinearSlop) {
      J.u = (1.0f / J.currentLength) * J.u;
    } else {
      J.u = v2(0.0f, 0.0f);
      J.mass = 0.0f; J.impulse1 = 0.0f; J.lowerImpulse = 0.0f; J.upperImpulse = 0.0f;
    }
    float crAu = cross(J.rA, J.u);
    float crBu = cross(J.rB, J.u);
    float invMass = J.mA + J.invIA * crAu * crAu + J.mB + J.invIB * crBu * crBu;
    J.mass = invMass != 0.0f ? 1.0f / invMass : 0.0f;
    if (J.d.stiffness > 0.0f && J.d.min_length < J.d.max_length) {
      float C = J.currentLength - J.d.length;
      float d = J.d.damping;
      float k = J.d.stiffness;
      float h = st.dt;
      J.gamma = h * (d + h * k);
      J.gamma = J.gamma != 0.0f ? 1.0f / J.gamma : 0.0f;
      J.bias = C * h * k * J.gamma;
      invMass += J.gamma;
      J.softMass = invMass != 0.0f ? 1.0f / invMass : 0.0f;
    } else {
      J.gamma = 0.0f; J.bias = 0.0f; J.softMass = J.mass;
    }
    if (st.warm) {
      J.impulse1 *= st.dtRatio; J.lowerImpulse *= st.dtRatio; J.upperImpulse *= st.dtRatio;
      V2 P = ((J.impulse1 + J.lowerImpulse) - J.upperImpulse) * J.u;
      subFrom(vA, J.mA * P);
      wA -= J.invIA * cross(J.rA, P);
      addTo(vB, J.mB * P);
      wB += J.invIB * cross(J.rB, P);
    } else {
      J.impulse1 = 0.0f;
    }
  } else if (J.d.type == B2G_JOINT_WELD) {
    // b2WeldJoint::InitVelocityConstraints (b2_weld_joint.cpp:93-187)
    J.rA = mul(qA, la - J.lcA);
    J.rB = mul(qB, lb - J.lcB);
    V3 ex, ey, ez;
    weldK(J.rA, J.rB, mA, mB, iA, iB, ex, ey, ez);
    if (J.d.stiffness > 0.0f) {
      inverse22(ex, ey, J.mass3);
      float invM = iA + iB;
      float C = aB - aA - J.d.reference_angle;
      float d = J.d.damping, k = J.d.stiffness, h = st.dt;
      J.gamma = h * (d + h * k);
      J.gamma = J.gamma != 0.0f ? 1.0f / J.gamma : 0.0f;
      J.bias = C * h * k * J.gamma;
      invM += J.gamma;
      J.mass3[8] = invM != 0.0f ? 1.0f / invM : 0.0f;
    } else if (ez.z == 0.0f) {
      inverse22(ex, ey, J.mass3);
      J.gamma = 0.0f; J.bias = 0.0f;
    } else {
      symInverse33(ex, ey, ez, J.mass3);
      J.gamma = 0.0f; J.bias = 0.0f;
    }
    if (st.warm) {
      for (int k = 0; k < 3; ++k) J.imp[k] *= st.dtRatio;
      V2 P = v2(J.imp[0], J.imp[1]);
      subFrom(vA, mA * P);
      wA -= iA * (cross(J.rA, P) + J.imp[2]);
      addTo(vB, mB * P);
      wB += iB * (cross(J.rB, P) + J.imp[2]);
    } else {
      J.imp[0] = J.imp[1] = J.imp[2] = 0.0f;
    }
  } else if (J.d.type == B2G_JOINT_WHEEL) {
    // b2WheelJoint::InitVelocityConstraints (b2_wheel_joint.cpp:89-211)
    V2 rA = mul(qA, la - J.lcA);
    V2 rB = mul(qB, lb - J.lcB);
    V2 d = cB + rB - cA - rA;
    J.perp = mul(qA, J.localYAxisA);
    J.s1 = cross(d + rA, J.perp);
    J.s2 = cross(rB, J.perp);
    J.mass = mA + mB + iA * J.s1 * J.s1 + iB * J.s2 * J.s2;
    if (J.mass > 0.0f) J.mass = 1.0f / J.mass;
    J.axis = mul(qA, J.localXAxisA);
    J.a1 = cross(d + rA, J.axis);
    J.a2 = cross(rB, J.axis);
    const float invMass = mA + mB + iA * J.a1 * J.a1 + iB * J.a2 * J.a2;
    J.axialMass = invMass > 0.0f ? 1.0f / invMass : 0.0f;
    J.springMass = 0.0f; J.bias = 0.0f; J.gamma = 0.0f;
    if (J.d.stiffness > 0.0f && invMass > 0.0f) {
      J.springMass = 1.0f / invMass;
      float C = dot(d, J.axis);
      float h = st.dt;
      J.gamma = h * (J.d.damping + h * J.d.stiffness);
      if (J.gamma > 0.0f) J.gamma = 1.0f / J.gamma;
      J.bias = C * h * J.d.stiffness * J.gamma;
      J.springMass = invMass + J.gamma;
      if (J.springMass > 0.0f) J.springMass = 1.0f / J.springMass;
    } else {
      J.imp[1] = 0.0f;
    }
    if (J.d.enable_limit) J.translation = dot(J.axis, d);
    else { J.lowerImpulse = 0.0f; J.upperImpulse = 0.0f; }
    if (J.d.enable_motor) {
      J.motorMass = iA + iB;
      if (J.motorMass > 0.0f) J.motorMass = 1.0f / J.motorMass;
    } else {
      J.motorMass = 0.0f; J.motorImpulse = 0.0f;
    }
    if (st.warm) {
      J.imp[0] *= st.dtRatio; J.imp[1] *= st.dtRatio; J.motorImpulse *= st.dtRatio;
      float axialImpulse = J.imp[1] + J.lowerImpulse - J.upperImpulse;
      V2 P = J.imp[0] * J.perp + axialImpulse * J.axis;
      float LA = J.imp[0] * J.s1 + axialImpulse * J.a1 + J.motorImpulse;
      float LB = J.imp[0] * J.s2 + axialImpulse * J.a2 + J.motorImpulse;
      subFrom(vA, mA * P); wA -= iA * LA;
      addTo(vB, mB * P); wB += iB * LB;
    } else {
      J.imp[0] = J.imp[1] = 0.0f; J.motorImpulse = J.lowerImpulse = J.upperImpulse = 0.0f;
    }
  } else if (J.d.type == B2G_JOINT_MOTOR || J.d.type == B2G_JOINT_FRICTION) {
    // b2MotorJoint::InitVelocityConstraints (b2_motor_joint.cpp:58-136) and
    // b2FrictionJoint::InitVelocityConstraints (b2_friction_joint.cpp:60-123)
    if (J.d.type == B2G_JOINT_MOTOR) {
      J.rA = mul(qA, v2(J.d.linear_offset[0], J.d.linear_offset[1]) - J.lcA);
      J.rB = mul(qB, -J.lcB);
    } else {
      J.rA = mul(qA, la - J.lcA);
      J.rB = mul(qB, lb - J.lcB);
    }
    linearAngularMass(J, mA, mB, iA, iB);
    if (J.d.type == B2G_JOINT_MOTOR) {
      J.err = cB + J.rB - cA - J.rA;
      J.angularError = aB - aA - J.d.reference_angle;
    }
    if (st.warm) {
      for (int k = 0; k < 3; ++k) J.imp[k] *= st.dtRatio;
      V2 P = v2(J.imp[0], J.imp[1]);
      subFrom(vA, mA * P);
      wA -= iA * (cross(J.rA, P) + J.imp[2]);
      addTo(vB, mB * P);
      wB += iB * (cross(J.rB, P) + J.imp[2]);
    } else {
      J.imp[0] = J.imp[1] = J.imp[2] = 0.0f;
    }
  } else if (J.d.type == B2G_JOINT_MOUSE) {
    // b2MouseJoint::InitVelocityConstraints (b2_mouse_joint.cpp:75-132): body B only
    float d = J.d.damping, k = J.d.stiffness, h = st.dt;
    J.gamma = h * (d + h * k);
    if (J.gamma != 0.0f) J.gamma = 1.0f / J.gamma;
    J.bias = h * k * J.gamma;
    J.rB = mul(qB, lb - J.lcB);
    M22 K;
    K.ex.x = mB + iB * J.rB.y * J.rB.y + J.gamma;
    K.ex.y = -iB * J.rB.x * J.rB.y;
    K.ey.x = K.ex.y;
    K.ey.y = mB + iB * J.rB.x * J.rB.x + J.gamma;
    J.K = inverse(K);
    J.err = cB + J.rB - v2(J.d.target[0], J.d.target[1]);
    J.err.x *= J.bias;
    J.err.y *= J.bias;
    wB *= 0.98f;
    if (st.warm) {
      J.imp[0] *= st.dtRatio; J.imp[1] *= st.dtRatio;
      V2 P = v2(J.imp[0], J.imp[1]);
      addTo(vB, mB * P);
      wB += iB * cross(J.rB, P);
    } else {
      J.imp[0] = J.imp[1] = 0.0f;
    }
  } else {
    // b2PulleyJoint::InitVelocityConstraints (b2_pulley_joint.cpp:78-157)
    J.rA = mul(qA, la - J.lcA);
    J.rB = mul(qB, lb - J.lcB);
    J.u = cA + J.rA - v2(J.d.ground_anchor_a[0], J.d.ground_anchor_a[1]);
    J.uB = cB + J.rB - v2(J.d.ground_anchor_b[0], J.d.ground_anchor_b[1]);
    float lengthA = lengthOf(J.u), lengthB = lengthOf(J.uB);
    if (lengthA > 10.0f * kLinearSlop) { float s = 1.0f / lengthA; J.u.x *= s; J.u.y *= s; }
    else J.u = v2(0.0f, 0.0f);
    if (lengthB > 10.0f * kLinearSlop) { float s = 1.0f / lengthB; J.uB.x *= s; J.uB.y *= s; }
    else J.uB = v2(0.0f, 0.0f);
    float ruA = cross(J.rA, J.u), ruB = cross(J.rB, J.uB);
    float pmA = mA + iA * ruA * ruA;
    float pmB = mB + iB * ruB * ruB;
    J.mass = pmA + J.d.ratio * J.d.ratio * pmB;
    if (J.mass > 0.0f) J.mass = 1.0f / J.mass;
    if (st.warm) {
      J.imp[0] *= st.dtRatio;
      V2 PA = -(J.imp[0]) * J.u;
      V2 PB = (-J.d.ratio * J.imp[0]) * J.uB;
      addTo(vA, mA * PA); wA += iA * cross(J.rA, PA);
      addTo(vB, mB * PB); wB += iB * cross(J.rB, PB);
    } else {
      J.imp[0] = 0.0f;
    }
  }
  sb[J.iA].v = vA; sb[J.iA].w = wA;
  sb[J.iB].v = vB; sb[J.iB].w = wB;
}

static void jointSolveVelocity(Joint& J, std::vector<SolverBody>& sb, const Step& st) {
  if (J.d.type == B2G_JOINT_GEAR) {
    gearSolveVelocity(J, sb);
    return;
  }
  V2 vA = sb[J.iA].v; float wA = sb[J.iA].w;
  V2 vB = sb[J.iB].v; float wB = sb[J.iB].w;
  float mA = J.mA, mB = J.mB, iA = J.invIA, iB = J.invIB;
  if (J.d.type == B2G_JOINT_REVOLUTE) {
    // b2RevoluteJoint::SolveVelocityConstraints (b2_revolute_joint.cpp:167-243)
    bool fixedRotation = (iA + iB == 0.0f);
    if (J.d.enable_motor && fixedRotation == false) {
      float Cdot = wB - wA - J.d.motor_speed;
      float impulse = -J.axialMass * Cdot;
      float oldImpulse = J.motorImpulse;
      float maxImpulse = st.dt * J.d.max_motor;
      J.motorImpulse = bclamp(J.motorImpulse + impulse, -maxImpulse, maxImpulse);
      impulse = J.motorImpulse - oldImpulse;
      wA -= iA * impulse;
      wB += iB * impulse;
    }
    if (J.d.enable_limit && fixedRotation == false) {
      {
        float C = J.angle - J.d.lower;
        float Cdot = wB - wA;
        float impulse = -J.axialMass * (Cdot + bmax(C, 0.0f) * st.inv_dt);
        float oldImpulse = J.lowerImpulse;
        J.lowerImpulse = bmax(J.lowerImpulse + impulse, 0.0f);
        impulse = J.lowerImpulse - oldImpulse;
        wA -= iA * impulse;
        wB += iB * impulse;
      }
      {
        float C = J.d.upper - J.angle;
        float Cdot = wA - wB;
        float impulse = -J.axialMass * (Cdot + bmax(C, 0.0f) * st.inv_dt);
        float oldImpulse = J.upperImpulse;
        J.upperImpulse = bmax(J.upperImpulse + impulse, 0.0f);
        impulse = J.upperImpulse - oldImpulse;
        wA += iA * impulse;
        wB -= iB * impulse;
      }
    }
    {
      V2 Cdot = ((vB + cross(wB, J.rB)) - vA) - cross(wA, J.rA);
      V2 impulse = solve(J.K, -Cdot);
      J.impulse2.x += impulse.x;
      J.impulse2.y += impulse.y;
      subFrom(vA, mA * impulse);
      wA -= iA * cross(J.rA, impulse);
      addTo(vB, mB * impulse);
      wB += iB * cross(J.rB, impulse);
    }
  } else if (J.d.type == B2G_JOINT_PRISMATIC) {
    // b2PrismaticJoint::SolveVelocityConstraints (b2_prismatic_joint.cpp:226-330)
    if (J.d.enable_motor) {
      float Cdot = (dot(J.axis, vB - vA) + J.a2 * wB) - J.a1 * wA;
      float impulse = J.axialMass * (J.d.motor_speed - Cdot);
      float oldImpulse = J.motorImpulse;
      float maxImpulse = st.dt * J.d.max_motor;
      J.motorImpulse = bclamp(J.motorImpulse + impulse, -maxImpulse, maxImpulse);
      impulse = J.motorImpulse - oldImpulse;
      V2 P = impulse * J.axis;
      float LA = impulse * J.a1;
      float LB = impulse * J.a2;
      subFrom(vA, mA * P); wA -= iA * LA;
      addTo(vB, mB * P); wB += iB * LB;
    }
    if (J.d.enable_limit) {
      {
        float C = J.translation - J.d.lower;
        float Cdot = (dot(J.axis, vB - vA) + J.a2 * wB) - J.a1 * wA;
        float impulse = -J.axialMass * (Cdot + bmax(C, 0.0f) * st.inv_dt);
        float oldImpulse = J.lowerImpulse;
        J.lowerImpulse = bmax(J.lowerImpulse + impulse, 0.0f);
        impulse = J.lowerImpulse - oldImpulse;
        V2 P = impulse * J.axis;
        float LA = impulse * J.a1;
        float LB = impulse * J.a2;
        subFrom(vA, mA * P); wA -= iA * LA;
        addTo(vB, mB * P); wB += iB * LB;
      }
      {
        float C = J.d.upper - J.translation;
        float Cdot = (dot(J.axis, vA - vB) + J.a1 * wA) - J.a2 * wB;
        float impulse = -J.axialMass * (Cdot + bmax(C, 0.0f) * st.inv_dt);
        float oldImpulse = J.upperImpulse;
        J.upperImpulse = bmax(J.upperImpulse + impulse, 0.0f);
        impulse = J.upperImpulse - oldImpulse;
        V2 P = impulse * J.axis;
        float LA = impulse * J.a1;
        float LB = impulse * J.a2;
        addTo(vA, mA * P); wA += iA * LA;
        subFrom(vB, mB * P); wB -= iB * LB;
      }
    }
    {
      V2 Cdot;
      Cdot.x = (dot(J.perp, vB - vA) + J.s2 * wB) - J.s1 * wA;
      Cdot.y = wB - wA;
      V2 df = solve(J.K, -Cdot);
      addTo(J.impulse2, df);
      V2 P = df.x * J.perp;
      float LA = df.x * J.s1 + df.y;
      float LB = df.x * J.s2 + df.y;
      subFrom(vA, mA * P); wA -= iA * LA;
      addTo(vB, mB * P); wB += iB * LB;
    }
  } else if (J.d.type == B2G_JOINT_DISTANCE) {
    // b2DistanceJoint::SolveVelocityConstraints (b2_distance_joint.cpp:175-266)
    if (J.d.min_length < J.d.max_length) {
      if (J.d.stiffness > 0.0f) {
        V2 vpA = vA + cross(wA, J.rA);
        V2 vpB = vB + cross(wB, J.rB);
        float Cdot = dot(J.u, vpB - vpA);
        float impulse = -J.softMass * ((Cdot + J.bias) + J.gamma * J.impulse1);
        J.impulse1 += impulse;
        V2 P = impulse * J.u;
        subFrom(vA, J.mA * P); wA -= J.invIA * cross(J.rA, P);
        addTo(vB, J.mB * P); wB += J.invIB * cross(J.rB, P);
      }
      {
        float C = J.currentLength - J.d.min_length;
        float bias = bmax(0.0f, C) * st.inv_dt;
        V2 vpA = vA + cross(wA, J.rA);
        V2 vpB = vB + cross(wB, J.rB);
        float Cdot = dot(J.u, vpB - vpA);
        float impulse = -J.mass * (Cdot + bias);
        float oldImpulse = J.lowerImpulse;
        J.lowerImpulse = bmax(0.0f, J.lowerImpulse + impulse);
        impulse = J.lowerImpulse - oldImpulse;
        V2 P = impulse * J.u;
        subFrom(vA, J.mA * P); wA -= J.invIA * cross(J.rA, P);
        addTo(vB, J.mB * P); wB += J.invIB * cross(J.rB, P);
      }
      {
        float C = J.d.max_length - J.currentLength;
        float bias = bmax(0.0f, C) * st.inv_dt;
        V2 vpA = vA + cross(wA, J.rA);
        V2 vpB = vB + cross(wB, J.rB);
        float Cdot = dot(J.u, vpA - vpB);
        float impulse = -J.mass * (Cdot + bias);
        float oldImpulse = J.upperImpulse;
        J.upperImpulse = bmax(0.0f, J.upperImpulse + impulse);
        impulse = J.upperImpulse - oldImpulse;
        V2 P = -impulse * J.u;
        subFrom(vA, J.mA * P); wA -= J.invIA * cross(J.rA, P);
        addTo(vB, J.mB * P); wB += J.invIB * cross(J.rB, P);
      }
    } else {
      V2 vpA = vA + cross(wA, J.rA);
      V2 vpB = vB + cross(wB, J.rB);
      float Cdot = dot(J.u, vpB - vpA);
      float impulse = -J.mass * Cdot;
      J.impulse1 += impulse;
      V2 P = impulse * J.u;
      subFrom(vA, J.mA * P); wA -= J.invIA * cross(J.rA, P);
      addTo(vB, J.mB * P); wB += J.invIB * cross(J.rB, P);
    }
  } else if (J.d.type == B2G_JOINT_WELD) {
    // b2WeldJoint::SolveVelocityConstraints (b2_weld_joint.cpp:189-250)
    float mA = J.mA, mB = J.mB, iA = J.invIA, iB = J.invIB;
    const float* M = J.mass3;
    if (J.d.stiffness > 0.0f) {
      float Cdot2 = wB - wA;
      float impulse2 = -M[8] * (Cdot2 + J.bias + J.gamma * J.imp[2]);
      J.imp[2] += impulse2;
      wA -= iA * impulse2;
      wB += iB * impulse2;
      V2 Cdot1 = vB + cross(wB, J.rB) - vA - cross(wA, J.rA);
      V2 impulse1 = -v2(M[0] * Cdot1.x + M[3] * Cdot1.y, M[1] * Cdot1.x + M[4] * Cdot1.y);
      J.imp[0] += impulse1.x;
      J.imp[1] += impulse1.y;
      subFrom(vA, mA * impulse1); wA -= iA * cross(J.rA, impulse1);
      addTo(vB, mB * impulse1); wB += iB * cross(J.rB, impulse1);
    } else {
      V2 Cdot1 = vB + cross(wB, J.rB) - vA - cross(wA, J.rA);
      float Cdot2 = wB - wA;
      // -b2Mul(m_mass, Cdot) = -(Cdot.x ex + Cdot.y ey + Cdot.z ez)
      float ix = -(Cdot1.x * M[0] + Cdot1.y * M[3] + Cdot2 * M[6]);
      float iy = -(Cdot1.x * M[1] + Cdot1.y * M[4] + Cdot2 * M[7]);
      float iz = -(Cdot1.x * M[2] + Cdot1.y * M[5] + Cdot2 * M[8]);
      J.imp[0] += ix; J.imp[1] += iy; J.imp[2] += iz;
      V2 P = v2(ix, iy);
      subFrom(vA, mA * P); wA -= iA * (cross(J.rA, P) + iz);
      addTo(vB, mB * P); wB += iB * (cross(J.rB, P) + iz);
    }
  } else if (J.d.type == B2G_JOINT_WHEEL) {
    // b2WheelJoint::SolveVelocityConstraints (b2_wheel_joint.cpp:213-323)
    float mA = J.mA, mB = J.mB, iA = J.invIA, iB = J.invIB;
    {
      float Cdot = dot(J.axis, vB - vA) + J.a2 * wB - J.a1 * wA;
      float impulse = -J.springMass * (Cdot + J.bias + J.gamma * J.imp[1]);
      J.imp[1] += impulse;
      V2 P = impulse * J.axis;
      float LA = impulse * J.a1, LB = impulse * J.a2;
      subFrom(vA, mA * P); wA -= iA * LA;
      addTo(vB, mB * P); wB += iB * LB;
    }
    {
      float Cdot = wB - wA - J.d.motor_speed;
      float impulse = -J.motorMass * Cdot;
      float oldImpulse = J.motorImpulse;
      float maxImpulse = st.dt * J.d.max_motor;
      J.motorImpulse = bclamp(J.motorImpulse + impulse, -maxImpulse, maxImpulse);
      impulse = J.motorImpulse - oldImpulse;
      wA -= iA * impulse;
      wB += iB * impulse;
    }
    if (J.d.enable_limit) {
      {
        float C = J.translation - J.d.lower;
        float Cdot = dot(J.axis, vB - vA) + J.a2 * wB - J.a1 * wA;
        float impulse = -J.axialMass * (Cdot + bmax(C, 0.0f) * st.inv_dt);
        float oldImpulse = J.lowerImpulse;
        J.lowerImpulse = bmax(J.lowerImpulse + impulse, 0.0f);
        impulse = J.lowerImpulse - oldImpulse;
        V2 P = impulse * J.axis;
        float LA = impulse * J.a1, LB = impulse * J.a2;
        subFrom(vA, mA * P); wA -= iA * LA;
        addTo(vB, mB * P); wB += iB * LB;
      }
      {
        float C = J.d.upper - J.translation;
        float Cdot = dot(J.axis, vA - vB) + J.a1 * wA - J.a2 * wB;
        float impulse = -J.axialMass * (Cdot + bmax(C, 0.0f) * st.inv_dt);
        float oldImpulse = J.upperImpulse;
        J.upperImpulse = bmax(J.upperImpulse + impulse, 0.0f);
        impulse = J.upperImpulse - oldImpulse;
        V2 P = impulse * J.axis;
        float LA = impulse * J.a1, LB = impulse * J.a2;
        addTo(vA, mA * P); wA += iA * LA;
        subFrom(vB, mB * P); wB -= iB * LB;
      }
    }
    {
      float Cdot = dot(J.perp, vB - vA) + J.s2 * wB - J.s1 * wA;
      float impulse = -J.mass * Cdot;
      J.imp[0] += impulse;
      V2 P = impulse * J.perp;
      float LA = impulse * J.s1, LB = impulse * J.s2;
      subFrom(vA, mA * P); wA -= iA * LA;
      addTo(vB, mB * P); wB += iB * LB;
    }
  } else if (J.d.type == B2G_JOINT_MOTOR || J.d.type == B2G_JOINT_FRICTION) {
    // b2MotorJoint / b2FrictionJoint::SolveVelocityConstraints (b2_motor_joint.cpp:138-196,
    // b2_friction_joint.cpp:125-183)
    solveLinearAngular(J, vA, wA, vB, wB, st.dt, J.d.type == B2G_JOINT_MOTOR, st.inv_dt);
  } else if (J.d.type == B2G_JOINT_MOUSE) {
    // b2MouseJoint::SolveVelocityConstraints (b2_mouse_joint.cpp:134-160)
    V2 Cdot = vB + cross(wB, J.rB);
    V2 old = v2(J.imp[0], J.imp[1]);
    V2 impulse = mul(J.K, -(Cdot + J.err + J.gamma * old));
    V2 acc = old;
    addTo(acc, impulse);
    float maxImpulse = st.dt * J.d.max_force;
    if (lengthSq(acc) > maxImpulse * maxImpulse) {
      float s = maxImpulse / lengthOf(acc);
      acc.x *= s;
      acc.y *= s;
    }
    J.imp[0] = acc.x; J.imp[1] = acc.y;
    impulse = acc - old;
    addTo(vB, J.mB * impulse);
    wB += J.invIB * cross(J.rB, impulse);
  } else {
    // b2PulleyJoint::SolveVelocityConstraints (b2_pulley_joint.cpp:159-182)
    V2 vpA = vA + cross(wA, J.rA);
    V2 vpB = vB + cross(wB, J.rB);
    float Cdot = -dot(J.u, vpA) - J.d.ratio * dot(J.uB, vpB);
    float impulse = -J.mass * Cdot;
    J.imp[0] += impulse;
    V2 PA = -impulse * J.u;
    V2 PB = -J.d.ratio * impulse * J.uB;
    addTo(vA, J.mA * PA); wA += J.invIA * cross(J.rA, PA);
    addTo(vB, J.mB * PB); wB += J.invIB * cross(J.rB, PB);
  }
  sb[J.iA].v = vA; sb[J.iA].w = wA;
  sb[J.iB].v = vB; sb[J.iB].w = wB;
}

static bool jointSolvePosition(Joint& J, std::vector<SolverBody>& sb) {
  if (J.d.type == B2G_JOINT_GEAR) return gearSolvePosition(J, sb);
  V2 cA = sb[J.iA].c; float aA = sb[J.iA].a;
  V2 cB = sb[J.iB].c; float aB = sb[J.iB].a;
  Rot qA = rotOf(aA), qB = rotOf(aB);
  V2 la = v2(J.d.local_anchor_a[0], J.d.local_anchor_a[1]);
  V2 lb = v2(J.d.local_anchor_b[0], J.d.local_anchor_b[1]);
  bool ok;
  if (J.d.type == B2G_JOINT_REVOLUTE) {
    // b2RevoluteJoint::SolvePositionConstraints (b2_revolute_joint.cpp:245-321)
    float angularError = 0.0f;
    float positionError = 0.0f;
    bool fixedRotation = (J.invIA + J.invIB == 0.0f);
    if (J.d.enable_limit && fixedRotation == false) {
      float angle = aB - aA - J.d.reference_angle;
      float C = 0.0f;
      if (babs(J.d.upper - J.d.lower) < 2.0f * kAngularSlop)
        C = bclamp(angle - J.d.lower, -kMaxAngularCorrection, kMaxAngularCorrection);
      else if (angle <= J.d.lower)
        C = bclamp(angle - J.d.lower + kAngularSlop, -kMaxAngularCorrection, 0.0f);
      else if (angle >= J.d.upper)
        C = bclamp(angle - J.d.upper - kAngularSlop, 0.0f, kMaxAngularCorrection);
      float limitImpulse = -J.axialMass * C;
      aA -= J.invIA * limitImpulse;
      aB += J.invIB * limitImpulse;
      angularError = babs(C);
    }
    {
      qA = rotOf(aA);
      qB = rotOf(aB);
      V2 rA = mul(qA, la - J.lcA);
      V2 rB = mul(qB, lb - J.lcB);
      V2 C = ((cB + rB) - cA) - rA;
      positionError = lengthOf(C);
      float mA = J.mA, mB = J.mB, iA = J.invIA, iB = J.invIB;
      M22 K;
      K.ex.x = mA + mB + iA * rA.y * rA.y + iB * rB.y * rB.y;
      K.ex.y = -iA * rA.x * rA.y - iB * rB.x * rB.y;
      K.ey.x = K.ex.y;
      K.ey.y = mA + mB + iA * rA.x * rA.x + iB * rB.x * rB.x;
      V2 impulse = -solve(K, C);
      subFrom(cA, mA * impulse);
      aA -= iA * cross(rA, impulse);
      addTo(cB, mB * impulse);
      aB += iB * cross(rB, impulse);
    }
    ok = positionError <= kLinearSlop && angularError <= kAngularSlop;
  } else if (J.d.type == B2G_JOINT_PRISMATIC) {
    // b2PrismaticJoint::SolvePositionConstraints (b2_prismatic_joint.cpp:340-459)
    float mA = J.mA, mB = J.mB, iA = J.invIA, iB = J.invIB;
    V2 rA = mul(qA, la - J.lcA);
    V2 rB = mul(qB, lb - J.lcB);
    V2 d = ((cB + rB) - cA) - rA;
    V2 axis = mul(qA, J.localXAxisA);
    float a1 = cross(d + rA, axis);
    float a2 = cross(rB, axis);
    V2 perp = mul(qA, J.localYAxisA);
    float s1 = cross(d + rA, perp);
    float s2 = cross(rB, perp);
    V3 impulse;
    V2 C1;
    C1.x = dot(perp, d);
    C1.y = aB - aA - J.d.reference_angle;
    float linearError = babs(C1.x);
    float angularError = babs(C1.y);
    bool active = false;
    float C2 = 0.0f;
    if (J.d.enable_limit) {
      float translation = dot(axis, d);
      if (babs(J.d.upper - J.d.lower) < 2.0f * kLinearSlop) {
        C2 = translation;
        linearError = bmax(linearError, babs(translation));
        active = true;
      } else if (translation <= J.d.lower) {
        C2 = bmin(translation - J.d.lower, 0.0f);
        linearError = bmax(linearError, J.d.lower - translation);
        active = true;
      } else if (translation >= J.d.upper) {
        C2 = bmax(translation - J.d.upper, 0.0f);
        linearError = bmax(linearError, translation - J.d.upper);
        active = true;
      }
    }
    if (active) {
      float k11 = mA + mB + iA * s1 * s1 + iB * s2 * s2;
      float k12 = iA * s1 + iB * s2;
      float k13 = iA * s1 * a1 + iB * s2 * a2;
      float k22 = iA + iB;
      if (k22 == 0.0f) k22 = 1.0f;
      float k23 = iA * a1 + iB * a2;
      float k33 = mA + mB + iA * a1 * a1 + iB * a2 * a2;
      V3 ex = {k11, k12, k13}, ey = {k12, k22, k23}, ez = {k13, k23, k33};
      V3 Cn = {-C1.x, -C1.y, -C2};
      impulse = solve33(ex, ey, ez, Cn);
    } else {
      float k11 = mA + mB + iA * s1 * s1 + iB * s2 * s2;
      float k12 = iA * s1 + iB * s2;
      float k22 = iA + iB;
      if (k22 == 0.0f) k22 = 1.0f;
      M22 K;
      K.ex = v2(k11, k12);
      K.ey = v2(k12, k22);
      V2 impulse1 = solve(K, -C1);
      impulse.x = impulse1.x; impulse.y = impulse1.y; impulse.z = 0.0f;
    }
    V2 P = impulse.x * perp + impulse.z * axis;
    float LA = (impulse.x * s1 + impulse.y) + impulse.z * a1;
    float LB = (impulse.x * s2 + impulse.y) + impulse.z * a2;
    subFrom(cA, mA * P); aA -= iA * LA;
    addTo(cB, mB * P); aB += iB * LB;
    ok = linearError <= kLinearSlop && angularError <= kAngularSlop;
  } else if (J.d.type == B2G_JOINT_DISTANCE) {
    // b2DistanceJoint::SolvePositionConstraints (b2_distance_joint.cpp:268-314)
    V2 rA = mul(qA, la - J.lcA);
    V2 rB = mul(qB, lb - J.lcB);
    V2 u = ((cB + rB) - cA) - rA;
    float length = normalize(u);
    float C;
    if (J.d.min_length == J.d.max_length) C = length - J.d.min_length;
    else if (length < J.d.min_length) C = length - J.d.min_length;
    else if (J.d.max_length < length) C = length - J.d.max_length;
    else return true;
    float impulse = -J.mass * C;
    V2 P = impulse * u;
    subFrom(cA, J.mA * P); aA -= J.invIA * cross(rA, P);
    addTo(cB, J.mB * P); aB += J.invIB * cross(rB, P);
    ok = babs(C) < kLinearSlop;
  } else if (J.d.type == B2G_JOINT_WELD) {
    // b2WeldJoint::SolvePositionConstraints (b2_weld_joint.cpp:252-329)
    float mA = J.mA, mB = J.mB, iA = J.invIA, iB = J.invIB;
    V2 rA = mul(qA, la - J.lcA);
    V2 rB = mul(qB, lb - J.lcB);
    float positionError, angularError;
    V3 ex, ey, ez;
    weldK(rA, rB, mA, mB, iA, iB, ex, ey, ez);
    if (J.d.stiffness > 0.0f) {
      V2 C1 = cB + rB - cA - rA;
      positionError = lengthOf(C1);
      angularError = 0.0f;
      V2 P = -solve22(ex, ey, C1);
      subFrom(cA, mA * P); aA -= iA * cross(rA, P);
      addTo(cB, mB * P); aB += iB * cross(rB, P);
    } else {
      V2 C1 = cB + rB - cA - rA;
      float C2 = aB - aA - J.d.reference_angle;
      positionError = lengthOf(C1);
      angularError = babs(C2);
      V3 C = {C1.x, C1.y, C2};
      V3 impulse;
      if (ez.z > 0.0f) {
        V3 x = solve33(ex, ey, ez, C);
        impulse = V3{-x.x, -x.y, -x.z};
      } else {
        V2 impulse2 = -solve22(ex, ey, C1);
        impulse = V3{impulse2.x, impulse2.y, 0.0f};
      }
      V2 P = v2(impulse.x, impulse.y);
      subFrom(cA, mA * P); aA -= iA * (cross(rA, P) + impulse.z);
      addTo(cB, mB * P); aB += iB * (cross(rB, P) + impulse.z);
    }
    ok = positionError <= kLinearSlop && angularError <= kAngularSlop;
  } else if (J.d.type == B2G_JOINT_WHEEL) {
    // b2WheelJoint::SolvePositionConstraints (b2_wheel_joint.cpp:325-420); like the reference,
    // the limit uses the step's m_ax and the point constraint the step's m_sAy, m_sBy
    float linearError = 0.0f;
    if (J.d.enable_limit) {
      V2 rA = mul(qA, la - J.lcA);
      V2 rB = mul(qB, lb - J.lcB);
      V2 d = (cB - cA) + rB - rA;
      V2 ax = mul(qA, J.localXAxisA);
      float sAx = cross(d + rA, J.axis);
      float sBx = cross(rB, J.axis);
      float C = 0.0f;
      float translation = dot(ax, d);
      if (babs(J.d.upper - J.d.lower) < 2.0f * kLinearSlop) C = translation;
      else if (translation <= J.d.lower) C = bmin(translation - J.d.lower, 0.0f);
      else if (translation >= J.d.upper) C = bmax(translation - J.d.upper, 0.0f);
      if (C != 0.0f) {
        float invMass = J.mA + J.mB + J.invIA * sAx * sAx + J.invIB * sBx * sBx;
        float impulse = 0.0f;
        if (invMass != 0.0f) impulse = -C / invMass;
        V2 P = impulse * ax;
        float LA = impulse * sAx, LB = impulse * sBx;
        subFrom(cA, J.mA * P); aA -= J.invIA * LA;
        addTo(cB, J.mB * P); aB += J.invIB * LB;
        linearError = babs(C);
      }
    }
    {
      Rot qA2 = rotOf(aA), qB2 = rotOf(aB);
      V2 rA = mul(qA2, la - J.lcA);
      V2 rB = mul(qB2, lb - J.lcB);
      V2 d = (cB - cA) + rB - rA;
      V2 ay = mul(qA2, J.localYAxisA);
      float sAy = cross(d + rA, ay);
      float sBy = cross(rB, ay);
      float C = dot(d, ay);
      float invMass = J.mA + J.mB + J.invIA * J.s1 * J.s1 + J.invIB * J.s2 * J.s2;
      float impulse = 0.0f;
      if (invMass != 0.0f) impulse = -C / invMass;
      V2 P = impulse * ay;
      float LA = impulse * sAy, LB = impulse * sBy;
      subFrom(cA, J.mA * P); aA -= J.invIA * LA;
      addTo(cB, J.mB * P); aB += J.invIB * LB;
      linearError = bmax(linearError, babs(C));
    }
    ok = linearError <= kLinearSlop;
  } else if (J.d.type == B2G_JOINT_PULLEY) {
    // b2PulleyJoint::SolvePositionConstraints (b2_pulley_joint.cpp:184-256)
    V2 rA = mul(qA, la - J.lcA);
    V2 rB = mul(qB, lb - J.lcB);
    V2 uA = cA + rA - v2(J.d.ground_anchor_a[0], J.d.ground_anchor_a[1]);
    V2 uB = cB + rB - v2(J.d.ground_anchor_b[0], J.d.ground_anchor_b[1]);
    float lengthA = lengthOf(uA), lengthB = lengthOf(uB);
    if (lengthA > 10.0f * kLinearSlop) { float s = 1.0f / lengthA; uA.x *= s; uA.y *= s; }
    else uA = v2(0.0f, 0.0f);
    if (lengthB > 10.0f * kLinearSlop) { float s = 1.0f / lengthB; uB.x *= s; uB.y *= s; }
    else uB = v2(0.0f, 0.0f);
    float ruA = cross(rA, uA), ruB = cross(rB, uB);
    float pmA = J.mA + J.invIA * ruA * ruA;
    float pmB = J.mB + J.invIB * ruB * ruB;
    float mass = pmA + J.d.ratio * J.d.ratio * pmB;
    if (mass > 0.0f) mass = 1.0f / mass;
    float C = J.constant - lengthA - J.d.ratio * lengthB;
    float linearError = babs(C);
    float impulse = -mass * C;
    V2 PA = -impulse * uA;
    V2 PB = -J.d.ratio * impulse * uB;
    addTo(cA, J.mA * PA); aA += J.invIA * cross(rA, PA);
    addTo(cB, J.mB * PB); aB += J.invIB * cross(rB, PB);
    ok = linearError < kLinearSlop;
  } else {
    return true;  // motor, friction and mouse joints have no position constraint
  }
  sb[J.iA].c = cA; sb[J.iA].a = aA;
  sb[J.iB].c = cB; sb[J.iB].a = aB;
  return ok;
}

// Reaction force/torque after the step (GetReactionForce/Torque of each joint type).
static void jointReaction(const Joint& J, float inv_dt, float* F, float* T) {
  if (J.d.type == B2G_JOINT_GEAR) {  // b2_gear_joint.cpp:387-397
    V2 P = J.imp[0] * J.JvAC;
    F[0] = inv_dt * P.x; F[1] = inv_dt * P.y;
    *T = inv_dt * (J.imp[0] * J.JwA);
  } else if (J.d.type == B2G_JOINT_REVOLUTE) {
    F[0] = inv_dt * J.impulse2.x; F[1] = inv_dt * J.impulse2.y;
    *T = inv_dt * ((J.motorImpulse + J.lowerImpulse) - J.upperImpulse);
  } else if (J.d.type == B2G_JOINT_PRISMATIC) {
    V2 f = inv_dt * (J.impulse2.x * J.perp + ((J.motorImpulse + J.lowerImpulse) - J.upperImpulse) * J.axis);
    F[0] = f.x; F[1] = f.y;
    *T = inv_dt * J.impulse2.y;
  } else if (J.d.type == B2G_JOINT_DISTANCE) {
    V2 f = (inv_dt * ((J.impulse1 + J.lowerImpulse) - J.upperImpulse)) * J.u;
    F[0] = f.x; F[1] = f.y;
    *T = 0.0f;
  } else if (J.d.type == B2G_JOINT_WHEEL) {  // b2_wheel_joint.cpp:448-461
    V2 f = inv_dt * (J.imp[0] * J.perp + ((J.imp[1] + J.lowerImpulse) - J.upperImpulse) * J.axis);
    F[0] = f.x; F[1] = f.y;
    *T = inv_dt * J.motorImpulse;
  } else if (J.d.type == B2G_JOINT_PULLEY) {  // b2_pulley_joint.cpp:276-286
    V2 f = inv_dt * (J.imp[0] * J.uB);
    F[0] = f.x; F[1] = f.y;
    *T = 0.0f;
  } else {  // weld, motor, friction, mouse
    F[0] = inv_dt * J.imp[0]; F[1] = inv_dt * J.imp[1];
    *T = J.d.type == B2G_JOINT_MOUSE ? inv_dt * 0.0f : inv_dt * J.imp[2];
  }
}

// ---- the contact solver (src/dynamics/b2_contact_solver.cpp)
static void prepareContacts(World* w, const std::vector<int>& solverContacts, std::vector<SolverBody>& sb,
                            const Step& st, std::vector<VC>& vcs, std::vector<PC>& pcs) {
  int n = (int)solverContacts.size();
  vcs.assign(n, VC());
  pcs.assign(n, PC());
  for (int i = 0; i < n; ++i) {
    // b2ContactSolver::Initialize (:65-152)
    Contact& c = w->contacts[solverContacts[i]];
    const Fixture& fa = w->fixtures[c.fA];
    const Fixture& fb = w->fixtures[c.fB];
    const Body& bA = w->bodies[fa.body];
    const Body& bB = w->bodies[fb.body];
    VC& vc = vcs[i];
    PC& pc = pcs[i];
    memset(&vc, 0, sizeof(vc));
    memset(&pc, 0, sizeof(pc));
    vc.friction = c.friction; vc.restitution = c.restitution; vc.threshold = c.threshold;
    vc.tangentSpeed = c.tangentSpeed;
    vc.indexA = fa.body; vc.indexB = fb.body;
    vc.invMassA = bA.invMass; vc.invMassB = bB.invMass; vc.invIA = bA.invI; vc.invIB = bB.invI;
    vc.contact = solverContacts[i];
    vc.pointCount = c.m.pointCount;
    pc.indexA = fa.body; pc.indexB = fb.body;
    pc.invMassA = bA.invMass; pc.invMassB = bB.invMass;
    pc.localCenterA = bA.localCenter; pc.localCenterB = bB.localCenter;
    pc.invIA = bA.invI; pc.invIB = bB.invI;
    pc.localNormal = c.m.localNormal; pc.localPoint = c.m.localPoint;
    pc.pointCount = c.m.pointCount;
    pc.radiusA = fa.shape.radius; pc.radiusB = fb.shape.radius;
    pc.type = c.m.type;
    for (int j = 0; j < c.m.pointCount; ++j) {
      if (st.warm) {
        vc.points[j].normalImpulse = st.dtRatio * c.m.points[j].normalImpulse;
        vc.points[j].tangentImpulse = st.dtRatio * c.m.points[j].tangentImpulse;
      } else {
        vc.points[j].normalImpulse = 0.0f;
        vc.points[j].tangentImpulse = 0.0f;
      }
      pc.localPoints[j] = c.m.points[j].localPoint;
    }
  }
  for (int i = 0; i < n; ++i) {
    // b2ContactSolver::InitializeVelocityConstraints (:155-258)
    VC& vc = vcs[i];
    PC& pc = pcs[i];
    const Manifold& manifold = w->contacts[vc.contact].m;
    float mA = vc.invMassA, mB = vc.invMassB, iA = vc.invIA, iB = vc.invIB;
    V2 cA = sb[vc.indexA].c; float aA = sb[vc.indexA].a; V2 vA = sb[vc.indexA].v; float wA = sb[vc.indexA].w;
    V2 cB = sb[vc.indexB].c; float aB = sb[vc.indexB].a; V2 vB = sb[vc.indexB].v; float wB = sb[vc.indexB].w;
    Xf xfA, xfB;
    xfA.q = rotOf(aA);
    xfB.q = rotOf(aB);
    xfA.p = cA - mul(xfA.q, pc.localCenterA);
    xfB.p = cB - mul(xfB.q, pc.localCenterB);
    WorldManifold wm;
    memset(&wm, 0, sizeof(wm));
    worldManifold(&wm, manifold, xfA, pc.radiusA, xfB, pc.radiusB);
    vc.normal = wm.normal;
    V2 tangent = cross(vc.normal, 1.0f);
    for (int j = 0; j < vc.pointCount; ++j) {
      VCPoint& vcp = vc.points[j];
      vcp.rA = wm.points[j] - cA;
      vcp.rB = wm.points[j] - cB;
      float rnA = cross(vcp.rA, vc.normal);
      float rnB = cross(vcp.rB, vc.normal);
      float kNormal = mA + mB + iA * rnA * rnA + iB * rnB * rnB;
      vcp.normalMass = kNormal > 0.0f ? 1.0f / kNormal : 0.0f;
      float rtA = cross(vcp.rA, tangent);
      float rtB = cross(vcp.rB, tangent);
      float kTangent = mA + mB + iA * rtA * rtA + iB * rtB * rtB;
      vcp.tangentMass = kTangent > 0.0f ? 1.0f / kTangent : 0.0f;
      vcp.velocityBias = 0.0f;
      float vRel = dot(vc.normal, (vB + cross(wB, vcp.rB)) - (vA + cross(wA, vcp.rA)));
      if (vRel < -vc.threshold) vcp.velocityBias = -vc.restitution * vRel;
    }
    if (vc.pointCount == 2) {
      VCPoint& vcp1 = vc.points[0];
      VCPoint& vcp2 = vc.points[1];
      float rn1A = cross(vcp1.rA, vc.normal);
      float rn1B = cross(vcp1.rB, vc.normal);
      float rn2A = cross(vcp2.rA, vc.normal);
      float rn2B = cross(vcp2.rB, vc.normal);
      float k11 = mA + mB + iA * rn1A * rn1A + iB * rn1B * rn1B;
      float k22 = mA + mB + iA * rn2A * rn2A + iB * rn2B * rn2B;
      float k12 = mA + mB + iA * rn1A * rn2A + iB * rn1B * rn2B;
      const float k_maxConditionNumber = 1000.0f;
      if (k11 * k11 < k_maxConditionNumber * (k11 * k22 - k12 * k12)) {
        vc.K.ex = v2(k11, k12);
        vc.K.ey = v2(k12, k22);
        vc.normalMass = inverse(vc.K);
      } else {
        vc.pointCount = 1;
      }
    }
  }
}

// b2ContactSolver::WarmStart (:260-299) for one constraint.
static void warmStartOne(VC& vc, std::vector<SolverBody>& sb) {
  float mA = vc.invMassA, iA = vc.invIA, mB = vc.invMassB, iB = vc.invIB;
  V2 vA = sb[vc.indexA].v; float wA = sb[vc.indexA].w;
  V2 vB = sb[vc.indexB].v; float wB = sb[vc.indexB].w;
  V2 normal = vc.normal;
  V2 tangent = cross(normal, 1.0f);
  for (int j = 0; j < vc.pointCount; ++j) {
    VCPoint& vcp = vc.points[j];
    V2 P = vcp.normalImpulse * normal + vcp.tangentImpulse * tangent;
    wA -= iA * cross(vcp.rA, P);
    subFrom(vA, mA * P);
    wB += iB * cross(vcp.rB, P);
    addTo(vB, mB * P);
  }
  sb[vc.indexA].v = vA; sb[vc.indexA].w = wA;
  sb[vc.indexB].v = vB; sb[vc.indexB].w = wB;
}

// b2ContactSolver::SolveVelocityConstraints (:301-639) for one constraint.
static void solveVelocityOne(VC& vc, std::vector<SolverBody>& sb) {
  float mA = vc.invMassA, iA = vc.invIA, mB = vc.invMassB, iB = vc.invIB;
  int pointCount = vc.pointCount;
  V2 vA = sb[vc.indexA].v; float wA = sb[vc.indexA].w;
  V2 vB = sb[vc.indexB].v; float wB = sb[vc.indexB].w;
  V2 normal = vc.normal;
  V2 tangent = cross(normal, 1.0f);
  for (int j = 0; j < pointCount; ++j) {
    VCPoint& vcp = vc.points[j];
    V2 dv = (vB + cross(wB, vcp.rB)) - (vA + cross(wA, vcp.rA));
    float vt = dot(dv, tangent) - vc.tangentSpeed;
    float lambda = vcp.tangentMass * (-vt);
    float maxFriction = vc.friction * vcp.normalImpulse;
    float newImpulse = bclamp(vcp.tangentImpulse + lambda, -maxFriction, maxFriction);
    lambda = newImpulse - vcp.tangentImpulse;
    vcp.tangentImpulse = newImpulse;
    V2 P = lambda * tangent;
    subFrom(vA, mA * P);
    wA -= iA * cross(vcp.rA, P);
    addTo(vB, mB * P);
    wB += iB * cross(vcp.rB, P);
  }
  if (pointCount == 1) {
    VCPoint& vcp = vc.points[0];
    V2 dv = (vB + cross(wB, vcp.rB)) - (vA + cross(wA, vcp.rA));
    float vn = dot(dv, normal);
    float lambda = -vcp.normalMass * (vn - vcp.velocityBias);
    float newImpulse = bmax(vcp.normalImpulse + lambda, 0.0f);
    lambda = newImpulse - vcp.normalImpulse;
    vcp.normalImpulse = newImpulse;
    V2 P = lambda * normal;
    subFrom(vA, mA * P);
    wA -= iA * cross(vcp.rA, P);
    addTo(vB, mB * P);
    wB += iB * cross(vcp.rB, P);
  } else {
    VCPoint& cp1 = vc.points[0];
    VCPoint& cp2 = vc.points[1];
    V2 a = v2(cp1.normalImpulse, cp2.normalImpulse);
    V2 dv1 = (vB + cross(wB, cp1.rB)) - (vA + cross(wA, cp1.rA));
    V2 dv2 = (vB + cross(wB, cp2.rB)) - (vA + cross(wA, cp2.rA));
    float vn1 = dot(dv1, normal);
    float vn2 = dot(dv2, normal);
    V2 b;
    b.x = vn1 - cp1.velocityBias;
    b.y = vn2 - cp2.velocityBias;
    subFrom(b, mul(vc.K, a));
    for (;;) {
      V2 x = -mul(vc.normalMass, b);
      if (x.x >= 0.0f && x.y >= 0.0f) {
        V2 d = x - a;
        V2 P1 = d.x * normal;
        V2 P2 = d.y * normal;
        subFrom(vA, mA * (P1 + P2));
        wA -= iA * (cross(cp1.rA, P1) + cross(cp2.rA, P2));
        addTo(vB, mB * (P1 + P2));
        wB += iB * (cross(cp1.rB, P1) + cross(cp2.rB, P2));
        cp1.normalImpulse = x.x;
        cp2.normalImpulse = x.y;
        break;
      }
      x.x = -cp1.normalMass * b.x;
      x.y = 0.0f;
      vn1 = 0.0f;
      vn2 = vc.K.ex.y * x.x + b.y;
      if (x.x >= 0.0f && vn2 >= 0.0f) {
        V2 d = x - a;
        V2 P1 = d.x * normal;
        V2 P2 = d.y * normal;
        subFrom(vA, mA * (P1 + P2));
        wA -= iA * (cross(cp1.rA, P1) + cross(cp2.rA, P2));
        addTo(vB, mB * (P1 + P2));
        wB += iB * (cross(cp1.rB, P1) + cross(cp2.rB, P2));
        cp1.normalImpulse = x.x;
        cp2.normalImpulse = x.y;
        break;
      }
      x.x = 0.0f;
      x.y = -cp2.normalMass * b.y;
      vn1 = vc.K.ey.x * x.y + b.x;
      vn2 = 0.0f;
      if (x.y >= 0.0f && vn1 >= 0.0f) {
        V2 d = x - a;
        V2 P1 = d.x * normal;
        V2 P2 = d.y * normal;
        subFrom(vA, mA * (P1 + P2));
        wA -= iA * (cross(cp1.rA, P1) + cross(cp2.rA, P2));
        addTo(vB, mB * (P1 + P2));
        wB += iB * (cross(cp1.rB, P1) + cross(cp2.rB, P2));
        cp1.normalImpulse = x.x;
        cp2.normalImpulse = x.y;
        break;
      }
      x.x = 0.0f;
      x.y = 0.0f;
      vn1 = b.x;
      vn2 = b.y;
      if (vn1 >= 0.0f && vn2 >= 0.0f) {
        V2 d = x - a;
        V2 P1 = d.x * normal;
        V2 P2 = d.y * normal;
        subFrom(vA, mA * (P1 + P2));
        wA -= iA * (cross(cp1.rA, P1) + cross(cp2.rA, P2));
        addTo(vB, mB * (P1 + P2));
        wB += iB * (cross(cp1.rB, P1) + cross(cp2.rB, P2));
        cp1.normalImpulse = x.x;
        cp2.normalImpulse = x.y;
        break;
      }
      break;
    }
  }
  sb[vc.indexA].v = vA; sb[vc.indexA].w = wA;
  sb[vc.indexB].v = vB; sb[vc.indexB].w = wB;
}

// b2PositionSolverManifold::Initialize (:659-708) + SolvePositionConstraints (:711-787) for one
// constraint; returns this constraint's minimum separation (starting from 0).
static float solvePositionOne(const PC& pc, std::vector<SolverBody>& sb) {
  float minSeparation = 0.0f;
  V2 localCenterA = pc.localCenterA, localCenterB = pc.localCenterB;
  float mA = pc.invMassA, iA = pc.invIA, mB = pc.invMassB, iB = pc.invIB;
  V2 cA = sb[pc.indexA].c; float aA = sb[pc.indexA].a;
  V2 cB = sb[pc.indexB].c; float aB = sb[pc.indexB].a;
  for (int j = 0; j < pc.pointCount; ++j) {
    Xf xfA, xfB;
    xfA.q = rotOf(aA);
    xfB.q = rotOf(aB);
    xfA.p = cA - mul(xfA.q, localCenterA);
    xfB.p = cB - mul(xfB.q, localCenterB);
    V2 normal, point;
    float separation;
    if (pc.type == 0) {
      V2 pointA = mul(xfA, pc.localPoint);
      V2 pointB = mul(xfB, pc.localPoints[0]);
      normal = pointB - pointA;
      normalize(normal);
      point = 0.5f * (pointA + pointB);
      separation = (dot(pointB - pointA, normal) - pc.radiusA) - pc.radiusB;
    } else if (pc.type == 1) {
      normal = mul(xfA.q, pc.localNormal);
      V2 planePoint = mul(xfA, pc.localPoint);
      V2 clipPoint = mul(xfB, pc.localPoints[j]);
      separation = (dot(clipPoint - planePoint, normal) - pc.radiusA) - pc.radiusB;
      point = clipPoint;
    } else {
      normal = mul(xfB.q, pc.localNormal);
      V2 planePoint = mul(xfB, pc.localPoint);
      V2 clipPoint = mul(xfA, pc.localPoints[j]);
      separation = (dot(clipPoint - planePoint, normal) - pc.radiusA) - pc.radiusB;
      point = clipPoint;
      normal = -normal;
    }
    V2 rA = point - cA;
    V2 rB = point - cB;
    minSeparation = bmin(minSeparation, separation);
    float C = bclamp(kBaumgarte * (separation + kLinearSlop), -kMaxLinearCorrection, 0.0f);
    float rnA = cross(rA, normal);
    float rnB = cross(rB, normal);
    float K = mA + mB + iA * rnA * rnA + iB * rnB * rnB;
    float impulse = K > 0.0f ? -C / K : 0.0f;
    V2 P = impulse * normal;
    subFrom(cA, mA * P);
    aA -= iA * cross(rA, P);
    addTo(cB, mB * P);
    aB += iB * cross(rB, P);
  }
  sb[pc.indexA].c = cA; sb[pc.indexA].a = aA;
  sb[pc.indexB].c = cB; sb[pc.indexB].a = aB;
  return minSeparation;
}

// Islands of a sleep-mode world (b2World::Solve's depth-first search, src/dynamics/b2_world.cpp:
// 520-650): connected components over solid contacts and joints between non-static bodies, each
// labelled by its lowest body index (-1 for static bodies). `linked` marks bodies with any contact
// or joint (the others are orphans, solved by b2Island::SolveOrphan).
static int findRoot(std::vector<int>& parent, int x) {
  while (parent[x] != x) x = parent[x];
  return x;
}
static void buildIslands(const World& w, std::vector<int>* label, std::vector<char>* linked) {
  const int nb = (int)w.bodies.size();
  std::vector<int> parent(nb);
  for (int i = 0; i < nb; ++i) parent[i] = w.bodies[i].type == 0 ? -1 : i;
  linked->assign(nb, 0);
  auto unite = [&](int x, int y) {
    if (parent[x] < 0 || parent[y] < 0) return;
    x = findRoot(parent, x);
    y = findRoot(parent, y);
    if (x == y) return;
    if (x < y) std::swap(x, y);
    parent[x] = y;  // the larger root under the smaller: roots are lowest indices
  };
  for (const Contact& c : w.contacts) {
    int a = w.fixtures[c.fA].body, b = w.fixtures[c.fB].body;
    (*linked)[a] = (*linked)[b] = 1;
    if ((c.flags & B2G_CONTACT_TOUCHING) && (c.flags & B2G_CONTACT_ENABLED) && !w.fixtures[c.fA].sensor &&
        !w.fixtures[c.fB].sensor)
      unite(a, b);
  }
  for (const Joint& j : w.joints) {
    (*linked)[j.d.body_a] = (*linked)[j.d.body_b] = 1;
    unite(j.d.body_a, j.d.body_b);
  }
  label->assign(nb, -1);
  for (int i = 0; i < nb; ++i)
    if (parent[i] >= 0) (*label)[i] = findRoot(parent, i);
}

// One b2World::Step (src/dynamics/b2_world.cpp:1108-1171) with CCD off. Sleep-mode worlds
// (sleeping allowed, or sleepers present) solve only islands holding an awake body, iterate
// positions per island with the island's own early exit, and run the island sleep timers.
// ---- continuous collision: b2World::SolveTOI (src/dynamics/b2_world.cpp:859-1106) with the
// min-heap of contact times of impact (b2TOIMinHeap, :671-850), b2Contact::CalculateTOI
// (src/dynamics/b2_contact.cpp:212-280) and b2Island::SolveTOI (src/dynamics/b2_island.cpp:486-619).
// Order: the heap is built over the contacts in list order, and a body's contacts are visited in
// list order. Inside the event loop a moved body's existing contacts are kept or dropped by the
// overlap of their stored boxes (b2BroadPhase::UpdateNoRebuild + Query); pairs that begin to
// overlap there become contacts at the pair update that follows the loop.
static void advanceSweep(Body& b, float alpha) {
  float beta = (alpha - b.alpha0) / (1.0f - b.alpha0);
  addTo(b.c0, beta * (b.c - b.c0));
  b.a0 += beta * (b.a - b.a0);
  b.alpha0 = alpha;
}
// b2Body::Advance (include/box2d/b2_body.h:963-971)
static void advanceBody(Body& b, float alpha) {
  advanceSweep(b, alpha);
  b.c = b.c0;
  b.a = b.a0;
  b.xf.q = rotOf(b.a);
  b.xf.p = b.c - mul(b.xf.q, b.localCenter);
}
static void syncTransform(Body& b) {
  b.xf.q = rotOf(b.a);
  b.xf.p = b.c - mul(b.xf.q, b.localCenter);
}
static Sweep sweepOfBody(const Body& b) {
  Sweep s;
  s.localCenter = b.localCenter; s.c0 = b.c0; s.c = b.c; s.a0 = b.a0; s.a = b.a; s.alpha0 = b.alpha0;
  return s;
}
static bool isBullet(const Body& b) { return (b.flags & B2G_BODY_BULLET) != 0; }

static float calculateTOI(World* w, int ci) {
  Contact& c = w->contacts[ci];
  const Fixture& fa = w->fixtures[c.fA];
  const Fixture& fb = w->fixtures[c.fB];
  if (fa.sensor || fb.sensor || !(c.flags & B2G_CONTACT_ENABLED)) return 1.0f;
  Body& A = w->bodies[fa.body];
  Body& B = w->bodies[fb.body];
  bool active;
  if (w->sleepMode()) active = (A.awake() && A.type != 0) && (B.awake() && B.type != 0);
  else active = A.type != 0 && B.type != 0;
  if (!active) return 1.0f;
  const bool collideA = isBullet(A) || A.type != 2;
  const bool collideB = isBullet(B) || B.type != 2;
  if (!collideA && !collideB) return 1.0f;
  float alpha0 = A.alpha0;
  if (A.alpha0 < B.alpha0) {
    alpha0 = B.alpha0;
    advanceSweep(A, alpha0);
  } else if (B.alpha0 < A.alpha0) {
    alpha0 = A.alpha0;
    advanceSweep(B, alpha0);
  }
  float t;
  int state = timeOfImpact(fa.shape, fb.shape, sweepOfBody(A), sweepOfBody(B), 1.0f, &t);
  return state == B2G_TOI_TOUCHING ? bmin(alpha0 + (1.0f - alpha0) * t, 1.0f) : 1.0f;
}

struct ToiHeap {
  struct Node { float toi; int count; int c; };
  World* w;
  std::vector<Node> h;
  std::vector<int> pos;  // per contact: its node, -1 when not in the heap
  void swapNodes(int i, int j) {
    std::swap(pos[h[i].c], pos[h[j].c]);
    std::swap(h[i], h[j]);
  }
  void down(int i) {
    const int n = (int)h.size();
    for (;;) {
      int m = i, l = 2 * i + 1, r = 2 * i + 2;
      if (l < n && h[l].toi < h[m].toi) m = l;
      if (r < n && h[r].toi < h[m].toi) m = r;
      if (m == i) return;
      swapNodes(i, m);
      i = m;
    }
  }
  void up(int i) {
    while (i > 0 && h[i].toi < h[(i - 1) / 2].toi) {
      swapNodes(i, (i - 1) / 2);
      i = (i - 1) / 2;
    }
  }
  void setKey(int i, float toi) {
    const bool u = toi < h[i].toi, d = toi > h[i].toi;
    h[i].toi = toi;
    if (u) up(i);
    else if (d) down(i);
  }
  void update(int c) {
    const int i = pos[c];
    setKey(i, h[i].count > 8 ? 1.0f : calculateTOI(w, c));  // b2_maxSubSteps
  }
  void insert(int c) {
    float toi = calculateTOI(w, c);
    if (toi < 1.0f) {
      h.push_back({toi, 0, c});
      pos[c] = (int)h.size() - 1;
      up((int)h.size() - 1);
    }
  }
};

// b2ContactSolver::SolveTOIPositionConstraints (src/dynamics/b2_contact_solver.cpp:790-878) for
// one constraint: only the two bodies of the impact move.
static float solveTOIPositionOne(const PC& pc, std::vector<SolverBody>& sb, int toiA, int toiB) {
  float minSeparation = 0.0f;
  float mA = 0.0f, iA = 0.0f, mB = 0.0f, iB = 0.0f;
  if (pc.indexA == toiA || pc.indexA == toiB) { mA = pc.invMassA; iA = pc.invIA; }
  if (pc.indexB == toiA || pc.indexB == toiB) { mB = pc.invMassB; iB = pc.invIB; }
  V2 cA = sb[pc.indexA].c; float aA = sb[pc.indexA].a;
  V2 cB = sb[pc.indexB].c; float aB = sb[pc.indexB].a;
  for (int j = 0; j < pc.pointCount; ++j) {
    Xf xfA, xfB;
    xfA.q = rotOf(aA);
    xfB.q = rotOf(aB);
    xfA.p = cA - mul(xfA.q, pc.localCenterA);
    xfB.p = cB - mul(xfB.q, pc.localCenterB);
    V2 normal, point;
    float separation;
    if (pc.type == 0) {
      V2 pointA = mul(xfA, pc.localPoint);
      V2 pointB = mul(xfB, pc.localPoints[0]);
      normal = pointB - pointA;
      normalize(normal);
      point = 0.5f * (pointA + pointB);
      separation = (dot(pointB - pointA, normal) - pc.radiusA) - pc.radiusB;
    } else if (pc.type == 1) {
      normal = mul(xfA.q, pc.localNormal);
      V2 clipPoint = mul(xfB, pc.localPoints[j]);
      separation = (dot(clipPoint - mul(xfA, pc.localPoint), normal) - pc.radiusA) - pc.radiusB;
      point = clipPoint;
    } else {
      normal = mul(xfB.q, pc.localNormal);
      V2 clipPoint = mul(xfA, pc.localPoints[j]);
      separation = (dot(clipPoint - mul(xfB, pc.localPoint), normal) - pc.radiusA) - pc.radiusB;
      point = clipPoint;
      normal = -normal;
    }
    V2 rA = point - cA, rB = point - cB;
    minSeparation = bmin(minSeparation, separation);
    float C = bclamp(0.75f * (separation + kLinearSlop), -kMaxLinearCorrection, 0.0f);  // b2_toiBaumgarte
    float rnA = cross(rA, normal), rnB = cross(rB, normal);
    float K = mA + mB + iA * rnA * rnA + iB * rnB * rnB;
    float impulse = K > 0.0f ? -C / K : 0.0f;
    V2 P = impulse * normal;
    subFrom(cA, mA * P);
    aA -= iA * cross(rA, P);
    addTo(cB, mB * P);
    aB += iB * cross(rB, P);
  }
  sb[pc.indexA].c = cA; sb[pc.indexA].a = aA;
  sb[pc.indexB].c = cB; sb[pc.indexB].a = aB;
  return minSeparation;
}

static void solveTOI(World* w, const Step& step) {
  const int nc = (int)w->contacts.size();
  if (nc == 0) return;
  const bool sleepMode = w->sleepMode();
  const int nb = (int)w->bodies.size();
  std::vector<char> bodyIsland(nb, 0), contactIsland(nc, 0), persist(nc, 1);
  for (Body& b : w->bodies) b.alpha0 = 0.0f;
  ToiHeap heap;
  heap.w = w;
  heap.pos.assign(nc, -1);
  for (int i = 0; i < nc; ++i) {
    if (!(w->contacts[i].flags & B2G_CONTACT_ENABLED)) continue;
    float toi = calculateTOI(w, i);
    if (toi < 1.0f) heap.h.push_back({toi, 0, i});
  }
  for (int i = (int)heap.h.size() / 2 - 1; i >= 0; --i) heap.down(i);
  for (int i = 0; i < (int)heap.h.size(); ++i) heap.pos[heap.h[i].c] = i;
  auto bodyOf = [&](int ci, int side) { return w->fixtures[side ? w->contacts[ci].fB : w->contacts[ci].fA].body; };
  auto wakeOnChange = [&](int ci) {
    if (updateContact(w, w->contacts[ci]) && sleepMode) {
      setAwake(w->bodies[bodyOf(ci, 0)], true);
      setAwake(w->bodies[bodyOf(ci, 1)], true);
    }
  };
  auto awake = [&](int b) { if (sleepMode) setAwake(w->bodies[b], true); };
  while (!heap.h.empty()) {
    ToiHeap::Node& mn = heap.h[0];
    ++mn.count;
    const int mc = mn.c;
    const float minAlpha = mn.toi;
    if (1.0f - 10.0f * kEpsilon < minAlpha) break;
    const int ia = bodyOf(mc, 0), ib = bodyOf(mc, 1);
    Body& bA = w->bodies[ia];
    Body& bB = w->bodies[ib];
    const Body backA = bA, backB = bB;
    advanceBody(bA, minAlpha);
    advanceBody(bB, minAlpha);
    wakeOnChange(mc);
    heap.update(mc);
    Contact& cm = w->contacts[mc];
    if (!(cm.flags & B2G_CONTACT_ENABLED) || !(cm.flags & B2G_CONTACT_TOUCHING)) {
      cm.flags &= ~B2G_CONTACT_ENABLED;
      bA.c0 = backA.c0; bA.c = backA.c; bA.a0 = backA.a0; bA.a = backA.a; bA.alpha0 = backA.alpha0;
      bB.c0 = backB.c0; bB.c = backB.c; bB.a0 = backB.a0; bB.a = backB.a; bB.alpha0 = backB.alpha0;
      syncTransform(bA);
      syncTransform(bB);
      heap.update(mc);
      continue;
    }
    awake(ia);
    awake(ib);
    std::vector<int> ibodies = {ia, ib}, icontacts = {mc};
    bodyIsland[ia] = bodyIsland[ib] = 1;
    contactIsland[mc] = 1;
    for (int k = 0; k < 2; ++k) {
      const int body = k ? ib : ia;
      if (w->bodies[body].type != 2) continue;
      for (int ci = 0; ci < (int)w->contacts.size(); ++ci) {
        const int ca = bodyOf(ci, 0), cb = bodyOf(ci, 1);
        if (ca != body && cb != body) continue;
        if ((int)ibodies.size() == 64 || (int)icontacts.size() == 32) break;  // 2 * b2_maxTOIContacts
        if (contactIsland[ci] || !persist[ci]) continue;
        const int other = ca == body ? cb : ca;
        Body& ob = w->bodies[other];
        if (ob.type == 2 && !isBullet(w->bodies[body]) && !isBullet(ob)) continue;
        if (w->fixtures[w->contacts[ci].fA].sensor || w->fixtures[w->contacts[ci].fB].sensor) continue;
        const Body backup = ob;
        if (!bodyIsland[other]) advanceBody(ob, minAlpha);
        wakeOnChange(ci);
        const uint32_t fl = w->contacts[ci].flags;
        if (!(fl & B2G_CONTACT_ENABLED) || !(fl & B2G_CONTACT_TOUCHING)) {
          ob.c0 = backup.c0; ob.c = backup.c; ob.a0 = backup.a0; ob.a = backup.a; ob.alpha0 = backup.alpha0;
          syncTransform(ob);
          continue;
        }
        contactIsland[ci] = 1;
        icontacts.push_back(ci);
        if (bodyIsland[other]) continue;
        bodyIsland[other] = 1;
        if (ob.type != 0) awake(other);
        ibodies.push_back(other);
      }
    }
    // b2Island::SolveTOI
    Step sub;
    sub.dt = (1.0f - minAlpha) * step.dt;
    sub.inv_dt = 1.0f / sub.dt;
    sub.dtRatio = 1.0f;
    sub.vi = step.vi;
    sub.pi = 20;
    sub.warm = false;
    std::vector<SolverBody> sb(nb);
    for (int b : ibodies) {
      const Body& bd = w->bodies[b];
      sb[b].c = bd.c; sb[b].a = bd.a; sb[b].v = bd.v; sb[b].w = bd.w;
    }
    std::vector<VC> vcs;
    std::vector<PC> pcs;
    prepareContacts(w, icontacts, sb, sub, vcs, pcs);
    for (int it = 0; it < sub.pi; ++it) {
      float minSep = 0.0f;
      for (const PC& pc : pcs) minSep = bmin(minSep, solveTOIPositionOne(pc, sb, ia, ib));
      if (minSep >= -1.5f * kLinearSlop) break;
    }
    bA.c0 = sb[ia].c; bA.a0 = sb[ia].a;
    bB.c0 = sb[ib].c; bB.a0 = sb[ib].a;
    prepareContacts(w, icontacts, sb, sub, vcs, pcs);  // InitializeVelocityConstraints at the new positions
    for (int it = 0; it < sub.vi; ++it)
      for (VC& vc : vcs) solveVelocityOne(vc, sb);
    const float h = sub.dt;
    for (int b : ibodies) {
      V2 c = sb[b].c; float a = sb[b].a; V2 v = sb[b].v; float wv = sb[b].w;
      V2 translation = h * v;
      if (dot(translation, translation) > kMaxTranslationSquared) {
        float ratio = kMaxTranslation / lengthOf(translation);
        v.x *= ratio; v.y *= ratio;
      }
      float rotation = h * wv;
      if (rotation * rotation > kMaxRotationSquared) {
        float ratio = kMaxRotation / babs(rotation);
        wv *= ratio;
      }
      addTo(c, h * v);
      a += h * wv;
      Body& bd = w->bodies[b];
      bd.c = c; bd.a = a; bd.v = v; bd.w = wv;
      syncTransform(bd);
    }
    if (w->recordEvents)  // b2Island::Report (src/dynamics/b2_island.cpp:621-647)
      for (const VC& vc : vcs) {
        const Contact& c = w->contacts[vc.contact];
        float ni[2] = {vc.points[0].normalImpulse, vc.points[1].normalImpulse};
        float ti[2] = {vc.points[0].tangentImpulse, vc.points[1].tangentImpulse};
        if (vc.pointCount < 2) ni[1] = ti[1] = 0.0f;
        recordEvent(w, B2G_EVENT_POSTSOLVE, c.fA, c.fB, nullptr, vc.pointCount, ni, ti);
      }
    // reset the island flags, move the proxies of the dynamic bodies, refresh their contacts' TOIs
    for (int b : ibodies) {
      bodyIsland[b] = 0;
      if (w->bodies[b].type != 2) continue;
      for (size_t f = 0; f < w->fixtures.size(); ++f)
        if (w->fixtures[f].body == b) w->aabb[f] = computeAABB(w->fixtures[f].shape, w->bodies[b].xf);
      for (int ci = 0; ci < (int)w->contacts.size(); ++ci) {
        if (bodyOf(ci, 0) != b && bodyOf(ci, 1) != b) continue;
        if (persist[ci]) {
          if (heap.pos[ci] == -1) heap.insert(ci);
          else heap.update(ci);
        }
        contactIsland[ci] = 0;
        persist[ci] = 0;
      }
    }
    // b2BroadPhase::Query with each moved fixture's box (b2ContactManager::QueryCallback): the
    // contacts of the overlapping fixtures persist, and overlapping pairs without one get a new
    // contact (a fixture's partners in fixture order)
    for (int b : ibodies) {
      if (w->bodies[b].type != 2) continue;
      const int nf = (int)w->fixtures.size();
      for (int f = 0; f < nf; ++f) {
        if (w->fixtures[f].body != b) continue;
        for (int g = 0; g < nf; ++g) {
          if (w->fixtures[g].body == b || !overlap(w->aabb[f], w->aabb[g])) continue;
          int found = -1;
          for (int ci = 0; ci < (int)w->contacts.size() && found < 0; ++ci) {
            const Contact& c = w->contacts[ci];
            if ((c.fA == f && c.fB == g) || (c.fA == g && c.fB == f)) found = ci;
          }
          if (found >= 0) {
            persist[found] = 1;
            if (heap.pos[found] == -1) heap.insert(found);
            continue;
          }
          const bool sg = w->bodies[w->fixtures[g].body].type == 0;
          const int e = sg ? f : bmin(f, g), pp = sg ? g : bmax(f, g);
          if (!shouldCollide(*w, e, pp)) continue;
          if (!hasCollider(w->fixtures[e].shape.type, w->fixtures[pp].shape.type) &&
              !hasCollider(w->fixtures[pp].shape.type, w->fixtures[e].shape.type))
            continue;
          if ((int)w->contacts.size() - nc == 32) continue;  // at most 32 made in one step
          w->contacts.push_back(makeContact(*w, ((uint64_t)(uint32_t)e << 32) | (uint32_t)pp));
          contactIsland.push_back(0);
          persist.push_back(1);
          heap.pos.push_back(-1);
          heap.insert((int)w->contacts.size() - 1);
        }
      }
    }
  }
  // the contacts made inside the loop are made again, with no touching history, by the pair
  // update that follows (b2World::Step's next FindNewContacts finds the same pairs)
  w->contacts.resize(nc);
}

static void stepWorld(World* w, float dt, int vi, int pi) {
  if (w->newContacts) {
    updatePairs(w);
    w->newContacts = false;
  }
  Step st;
  st.dt = dt;
  st.inv_dt = (dt > 0.0f) ? 1.0f / dt : 0.0f;
  st.dtRatio = w->inv_dt0 * dt;
  st.vi = vi;
  st.pi = pi;
  st.warm = w->warmStarting;
  collide(w);
  const bool sleepMode = w->sleepMode();
  if (dt > 0.0f) {
    int nb = (int)w->bodies.size();
    float h = st.dt;
    std::vector<int> label;
    std::vector<char> linked;
    std::vector<char> islandAwake(nb, 0);
    if (sleepMode) {
      buildIslands(*w, &label, &linked);
      for (int i = 0; i < nb; ++i)
        if (label[i] >= 0 && w->bodies[i].awake()) islandAwake[label[i]] = 1;
      // the search marks every body it reaches awake without resetting its timer
      for (int i = 0; i < nb; ++i)
        if (label[i] >= 0 && islandAwake[label[i]]) w->bodies[i].flags |= B2G_BODY_AWAKE;
    }
    auto solved = [&](int i) { return !sleepMode || w->bodies[i].awake(); };
    auto rootOf = [&](int a, int b) { return label[a] >= 0 ? label[a] : label[b]; };
    auto jointActive = [&](const Joint& J) { return !sleepMode || w->bodies[J.d.body_a].awake() || w->bodies[J.d.body_b].awake(); };
    std::vector<SolverBody> sb(nb);
    // b2Island::Solve velocity integration (src/dynamics/b2_island.cpp:256-293) / SolveOrphan
    for (int i = 0; i < nb; ++i) {
      Body& b = w->bodies[i];
      V2 v = b.v;
      float wv = b.w;
      if (b.type == 2 && solved(i)) {
        addTo(v, (h * b.invMass) * (b.gravityScale * b.mass * w->gravity + b.force));
        wv += h * b.invI * b.torque;
        v.x /= (1.0f + h * b.linearDamping);
        v.y /= (1.0f + h * b.linearDamping);
        wv /= (1.0f + h * b.angularDamping);
      }
      sb[i].c = b.c; sb[i].a = b.a; sb[i].v = v; sb[i].w = wv;
    }
    // solver contact set: touching, enabled, no sensor, enabled bodies (b2_world.cpp:567-599)
    std::vector<int> solverContacts;
    for (int i = 0; i < (int)w->contacts.size(); ++i) {
      const Contact& c = w->contacts[i];
      if ((c.flags & B2G_CONTACT_TOUCHING) == 0 || (c.flags & B2G_CONTACT_ENABLED) == 0) continue;
      if (w->fixtures[c.fA].sensor || w->fixtures[c.fB].sensor) continue;
      if (sleepMode && !islandAwake[rootOf(w->fixtures[c.fA].body, w->fixtures[c.fB].body)]) continue;
      solverContacts.push_back(i);
    }
    int nc = (int)solverContacts.size();
    int nj = (int)w->joints.size();
    std::vector<VC> vcs;
    std::vector<PC> pcs;
    prepareContacts(w, solverContacts, sb, st, vcs, pcs);
    // colouring
    std::vector<int> cA(nc), cB(nc), jA(nj), jB(nj);
    std::vector<uint32_t> cp(nc), jp(nj);
    for (int i = 0; i < nc; ++i) {
      cA[i] = vcs[i].indexA; cB[i] = vcs[i].indexB;
      cp[i] = contactPriority(w->contacts[solverContacts[i]].key);
    }
    for (int j = 0; j < nj; ++j) {
      const bool gear = w->joints[j].d.type == B2G_JOINT_GEAR;
      jA[j] = gear ? -1 : w->joints[j].d.body_a; jB[j] = gear ? -1 : w->joints[j].d.body_b;
      jp[j] = jointPriority((uint32_t)j);
    }
    std::vector<int> ccol, jcol;
    colorConstraints(nc, cA.data(), cB.data(), cp.data(), w->bodies, &ccol);
    colorConstraints(nj, jA.data(), jB.data(), jp.data(), w->bodies, &jcol);
    std::vector<int> corder = solveOrder(nc, ccol, cp.data());
    std::vector<int> jorder = solveOrder(nj, jcol, jp.data());
    w->contactColor.assign(w->contacts.size(), -1);
    w->contactPrio.assign(w->contacts.size(), 0);
    for (int i = 0; i < nc; ++i) {
      w->contactColor[solverContacts[i]] = ccol[i];
      w->contactPrio[solverContacts[i]] = cp[i];
    }
    w->jointColor = jcol;
    w->jointPrioV = jp;
    w->lastContactOrder.clear();
    for (int i : corder) {
      w->lastContactOrder.push_back(w->contacts[solverContacts[i]].fA);
      w->lastContactOrder.push_back(w->contacts[solverContacts[i]].fB);
    }
    w->lastJointOrder.assign(jorder.begin(), jorder.end());
    // warm start (b2_island.cpp:304-325): contacts, then joint init
    if (st.warm)
      for (int i : corder) warmStartOne(vcs[i], sb);
    for (int j : jorder)
      if (jointActive(w->joints[j])) jointInit(w->joints[j], w->bodies, sb, st);
    // velocity iterations (b2_island.cpp:327-346): joints then contacts
    for (int it = 0; it < vi; ++it) {
      for (int j : jorder)
        if (jointActive(w->joints[j])) jointSolveVelocity(w->joints[j], sb, st);
      for (int i : corder) solveVelocityOne(vcs[i], sb);
    }
    // PostSolve with the velocity impulses (b2Island::Report, src/dynamics/b2_island.cpp:621-647),
    // recorded here (their values do not change after the velocity iterations) and delivered
    // after the step like the engine's
    if (w->recordEvents)
      for (int i = 0; i < nc; ++i) {
        const VC& vc = vcs[i];
        const Contact& c = w->contacts[vc.contact];
        float ni[2] = {vc.points[0].normalImpulse, vc.points[1].normalImpulse};
        float ti[2] = {vc.points[0].tangentImpulse, vc.points[1].tangentImpulse};
        if (vc.pointCount < 2) ni[1] = ti[1] = 0.0f;
        recordEvent(w, B2G_EVENT_POSTSOLVE, c.fA, c.fB, nullptr, vc.pointCount, ni, ti);
      }
    // StoreImpulses (b2_contact_solver.cpp:641-657)
    for (int i = 0; i < nc; ++i) {
      Manifold& m = w->contacts[vcs[i].contact].m;
      for (int j = 0; j < vcs[i].pointCount; ++j) {
        m.points[j].normalImpulse = vcs[i].points[j].normalImpulse;
        m.points[j].tangentImpulse = vcs[i].points[j].tangentImpulse;
      }
    }
    // integrate positions (b2_island.cpp:349-385)
    for (int i = 0; i < nb; ++i) {
      // every body's position at the step's start, for continuous collision (b2Island::Solve
      // stores it for the bodies it solves; the others have not moved since)
      w->bodies[i].c0 = sb[i].c;
      w->bodies[i].a0 = sb[i].a;
      if (w->bodies[i].type == 0 || !solved(i)) continue;
      V2 c = sb[i].c; float a = sb[i].a; V2 v = sb[i].v; float wv = sb[i].w;
      V2 translation = h * v;
      if (dot(translation, translation) > kMaxTranslationSquared) {
        float ratio = kMaxTranslation / lengthOf(translation);
        v.x *= ratio; v.y *= ratio;
      }
      float rotation = h * wv;
      if (rotation * rotation > kMaxRotationSquared) {
        float ratio = kMaxRotation / babs(rotation);
        wv *= ratio;
      }
      addTo(c, h * v);
      a += h * wv;
      sb[i].c = c; sb[i].a = a; sb[i].v = v; sb[i].w = wv;
    }
    // position iterations (b2_island.cpp:387-428): contacts then joints, early exit per world;
    // in sleep mode per island (an island okay in an iteration is done, as the reference's loop)
    std::vector<int> badIt(nb, 0);
    std::vector<char> done(nb, 0);
    for (int it = 0; it < pi; ++it) {
      float minSep = 0.0f;
      for (int i : corder) {
        int root = 0;
        if (sleepMode) {
          root = rootOf(pcs[i].indexA, pcs[i].indexB);
          if (done[root]) continue;
        }
        float sep = solvePositionOne(pcs[i], sb);
        minSep = bmin(minSep, sep);
        if (sleepMode && !(sep >= -3.0f * kLinearSlop)) badIt[root] = it + 1;
      }
      bool contactsOkay = minSep >= -3.0f * kLinearSlop;
      bool jointsOkay = true;
      for (int j : jorder) {
        Joint& J = w->joints[j];
        int root = 0;
        if (sleepMode) {
          if (!jointActive(J)) continue;
          root = rootOf(J.d.body_a, J.d.body_b);
          if (done[root]) continue;
        }
        bool ok = jointSolvePosition(J, sb);
        jointsOkay = jointsOkay && ok;
        if (sleepMode && !ok) badIt[root] = it + 1;
      }
      if (sleepMode) {
        bool pending = false;
        for (int i = 0; i < nb; ++i) {
          if (label[i] != i || !islandAwake[i] || done[i]) continue;
          if (badIt[i] == it + 1) pending = true;
          else done[i] = 1;
        }
        if (!pending) break;
      } else if (contactsOkay && jointsOkay) {
        break;
      }
    }
    // write back + SynchronizeTransform (b2_island.cpp:430-438, include/box2d/b2_body.h:957-961)
    for (int i = 0; i < nb; ++i) {
      Body& b = w->bodies[i];
      if (b.type == 0 || !solved(i)) continue;
      b.c = sb[i].c; b.a = sb[i].a; b.v = sb[i].v; b.w = sb[i].w;
      b.xf.q = rotOf(b.a);
      b.xf.p = b.c - mul(b.xf.q, b.localCenter);
    }
    // sleep timers (b2_island.cpp:444-483; orphans b2Island::SolveOrphan :230-249, which the
    // caller marks awake again, b2_world.cpp:545-549)
    if (w->allowSleep) {
      const float linTolSqr = kLinearSleepTolerance * kLinearSleepTolerance;
      const float angTolSqr = kAngularSleepTolerance * kAngularSleepTolerance;
      std::vector<float> minSleep(nb, FLT_MAX);
      for (int i = 0; i < nb; ++i) {
        Body& b = w->bodies[i];
        if (b.type == 0 || !b.awake()) continue;
        float t = 0.0f;
        if ((b.flags & B2G_BODY_AUTO_SLEEP) == 0 || b.w * b.w > angTolSqr || dot(b.v, b.v) > linTolSqr) {
          b.sleepTime = 0.0f;
        } else {
          b.sleepTime += h;
          t = b.sleepTime;
        }
        if (!linked[i]) {
          if (t >= kTimeToSleep) {
            setAwake(b, false);
            b.flags |= B2G_BODY_AWAKE;
          }
        } else {
          minSleep[label[i]] = bmin(minSleep[label[i]], t);
        }
      }
      for (int i = 0; i < nb; ++i) {
        Body& b = w->bodies[i];
        if (b.type == 0 || !b.awake() || !linked[i]) continue;
        if (minSleep[label[i]] >= kTimeToSleep && done[label[i]]) setAwake(b, false);
      }
    }
    // the island structure of this step, for replaying it on the reference
    w->islandRoot.clear(); w->islandOrphan.clear(); w->islandBodies.clear(); w->islandContacts.clear();
    w->islandJoints.clear(); w->islandBodyOff.assign(1, 0); w->islandContactOff.assign(1, 0);
    w->islandJointOff.assign(1, 0);
    if (sleepMode) {
      for (int r = 0; r < nb; ++r) {
        if (label[r] != r || !islandAwake[r]) continue;
        w->islandRoot.push_back(r);
        w->islandOrphan.push_back(linked[r] ? 0 : 1);
        for (int i = r; i < nb; ++i)
          if (label[i] == r) w->islandBodies.push_back(i);
        for (int i : corder) {
          const Contact& c = w->contacts[solverContacts[i]];
          if (rootOf(w->fixtures[c.fA].body, w->fixtures[c.fB].body) != r) continue;
          w->islandContacts.push_back(c.fA);
          w->islandContacts.push_back(c.fB);
        }
        for (int j : jorder)
          if (rootOf(w->joints[j].d.body_a, w->joints[j].d.body_b) == r) w->islandJoints.push_back(j);
        w->islandBodyOff.push_back((int)w->islandBodies.size());
        w->islandContactOff.push_back((int)w->islandContacts.size() / 2);
        w->islandJointOff.push_back((int)w->islandJoints.size());
      }
    }
    // broadphase at the end of Solve (b2_world.cpp:663-669)
    updatePairs(w);
    // b2World::Step's SolveTOI (b2_world.cpp:1152-1156); the pair update after it stands for
    // the proxy moves and dead-contact removal inside SolveTOI
    if (w->continuous) {
      solveTOI(w, st);
      updatePairs(w);
    }
    w->inv_dt0 = st.inv_dt;
    for (Joint& j : w->joints) {
      float F[2], T;
      jointReaction(j, st.inv_dt, F, &T);
      (void)F; (void)T;
    }
  }
  if (w->autoClearForces) {
    for (Body& b : w->bodies) { b.force = v2(0.0f, 0.0f); b.torque = 0.0f; }
  }
}

}  // namespace orc

// ================================================================================================
// C ABI of the oracle (loaded by tests through ctypes)
using namespace orc;

extern "C" {

// Listener-event recording (off by default) and the recorded events of the steps since the last
// call, sorted like the engine's batch delivery (kind, then fixture pair); returns their number
// and clears them when `out` holds them all.
void orc_world_events_enable(void* h, int32_t on) {
  World* w = (World*)h;
  w->recordEvents = on != 0;
  w->events.clear();
}

int32_t orc_world_events(void* h, b2g_event* out, int32_t cap) {
  World* w = (World*)h;
  std::stable_sort(w->events.begin(), w->events.end(), [](const b2g_event& x, const b2g_event& y) {
    if (x.kind != y.kind) return x.kind < y.kind;
    if (x.fixture_a != y.fixture_a) return x.fixture_a < y.fixture_a;
    return x.fixture_b < y.fixture_b;
  });
  const int32_t n = (int32_t)w->events.size();
  if (out && cap >= n) {
    for (int32_t i = 0; i < n; ++i) out[i] = w->events[i];
    w->events.clear();
  }
  return n;
}

void orc_set_libm_trig(int32_t on) { g_libm_trig = on; }

void orc_sincos(float x, float* s, float* c) { sincos_portable(x, s, c); }

int orc_polygon_set(const float* xy, int32_t n, b2g_shape* out) {
  V2 v[8];
  for (int i = 0; i < n && i < 8; ++i) v[i] = v2(xy[2 * i], xy[2 * i + 1]);
  Shape p;
  polygonSet(&p, v, n);
  shapeTo(p, out);
  return 0;
}

int orc_polygon_box(float hx, float hy, float cx, float cy, float angle, int32_t oriented, b2g_shape* out) {
  Shape p;
  setAsBox(&p, hx, hy, oriented != 0, v2(cx, cy), angle);
  shapeTo(p, out);
  return 0;
}

int orc_shape_mass(const b2g_shape* s, float density, float* out4) {
  MassData md = computeMass(shapeFrom(*s), density);
  out4[0] = md.mass; out4[1] = md.center.x; out4[2] = md.center.y; out4[3] = md.I;
  return 0;
}

int orc_shape_aabb(const b2g_shape* s, const float* xf, float* out4) {
  Xf t;
  t.p = v2(xf[0], xf[1]); t.q.s = xf[2]; t.q.c = xf[3];
  AABB bb = computeAABB(shapeFrom(*s), t);
  out4[0] = bb.lo.x; out4[1] = bb.lo.y; out4[2] = bb.hi.x; out4[3] = bb.hi.y;
  return 0;
}

// GJK distance with radii (distance out) and b2TestOverlap (returned) of two shapes.
int orc_test_overlap(const b2g_shape* sa, const float* xfa, const b2g_shape* sb, const float* xfb, float* distance) {
  Shape A = shapeFrom(*sa), B = shapeFrom(*sb);
  Xf ta, tb;
  ta.p = v2(xfa[0], xfa[1]); ta.q.s = xfa[2]; ta.q.c = xfa[3];
  tb.p = v2(xfb[0], xfb[1]); tb.q.s = xfb[2]; tb.q.c = xfb[3];
  *distance = gjkDistance(A, ta, B, tb);
  return testOverlap(A, ta, B, tb) ? 1 : 0;
}

static Sweep sweepFrom(const b2g_sweep& s) {
  Sweep o;
  o.localCenter = v2(s.local_center[0], s.local_center[1]);
  o.c0 = v2(s.c0[0], s.c0[1]);
  o.c = v2(s.c[0], s.c[1]);
  o.a0 = s.a0; o.a = s.a; o.alpha0 = s.alpha0;
  return o;
}

// b2TimeOfImpact for n inputs.
void orc_time_of_impact(const b2g_toi_input* in, int32_t n, b2g_toi_output* out) {
  for (int32_t i = 0; i < n; ++i) {
    Shape A = shapeFrom(in[i].shape_a), B = shapeFrom(in[i].shape_b);
    out[i].state = timeOfImpact(A, B, sweepFrom(in[i].sweep_a), sweepFrom(in[i].sweep_b), in[i].t_max, &out[i].t);
  }
}

int orc_collide(const b2g_shape* sa, const float* xfa, const b2g_shape* sb, const float* xfb, b2g_manifold* out) {
  Shape A = shapeFrom(*sa), B = shapeFrom(*sb);
  Xf ta, tb;
  ta.p = v2(xfa[0], xfa[1]); ta.q.s = xfa[2]; ta.q.c = xfa[3];
  tb.p = v2(xfb[0], xfb[1]); tb.q.s = xfb[2]; tb.q.c = xfb[3];
  Manifold m;
  memset(&m, 0, sizeof(m));
  if (!hasCollider(A.type, B.type)) return 1;
  evaluate(&m, A, ta, B, tb);
  manifoldTo(m, out);
  return 0;
}

int orc_world_manifold(const b2g_manifold* mi, const float* xfa, float ra, const float* xfb, float rb, float* out8) {
  Manifold m = manifoldFrom(*mi);
  Xf ta, tb;
  ta.p = v2(xfa[0], xfa[1]); ta.q.s = xfa[2]; ta.q.c = xfa[3];
  tb.p = v2(xfb[0], xfb[1]); tb.q.s = xfb[2]; tb.q.c = xfb[3];
  WorldManifold wm;
  memset(&wm, 0, sizeof(wm));
  worldManifold(&wm, m, ta, ra, tb, rb);
  out8[0] = wm.normal.x; out8[1] = wm.normal.y;
  out8[2] = wm.points[0].x; out8[3] = wm.points[0].y;
  out8[4] = wm.points[1].x; out8[5] = wm.points[1].y;
  out8[6] = wm.separations[0]; out8[7] = wm.separations[1];
  return 0;
}

// All pairs i < j of n AABBs that overlap (inclusive), sorted, as i << 32 | j.
int64_t orc_pairs(const float* aabbs, int32_t n, uint64_t* out, int64_t cap) {
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  auto lo = [&](int i) { return aabbs[4 * i]; };
  std::sort(order.begin(), order.end(), [&](int a, int b) { return lo(a) != lo(b) ? lo(a) < lo(b) : a < b; });
  std::vector<uint64_t> pairs;
  for (int oi = 0; oi < n; ++oi) {
    int i = order[oi];
    AABB a = {{aabbs[4 * i], aabbs[4 * i + 1]}, {aabbs[4 * i + 2], aabbs[4 * i + 3]}};
    for (int oj = oi + 1; oj < n; ++oj) {
      int j = order[oj];
      if (aabbs[4 * j] > a.hi.x) break;
      AABB b = {{aabbs[4 * j], aabbs[4 * j + 1]}, {aabbs[4 * j + 2], aabbs[4 * j + 3]}};
      if (!overlap(a, b)) continue;
      uint32_t x = (uint32_t)bmin(i, j), y = (uint32_t)bmax(i, j);
      pairs.push_back(((uint64_t)x << 32) | y);
    }
  }
  std::sort(pairs.begin(), pairs.end());
  for (int64_t k = 0; k < (int64_t)pairs.size() && k < cap; ++k) out[k] = pairs[k];
  return (int64_t)pairs.size();
}

void* orc_world_new(float gx, float gy) {
  World* w = new World();
  w->gravity = v2(gx, gy);
  return w;
}

void orc_world_free(void* h) { delete (World*)h; }

// Loads a world from exported records (bodies/fixtures/joints in creation order; contacts with
// their fixture indices, flags and manifolds). With no contacts given, the first step finds them
// (like b2World::Step after CreateFixture, b2_world.cpp:1113-1116).
int orc_world_load(void* h, const b2g_body* bodies, int32_t nb, const b2g_fixture* fixtures, int32_t nf,
                   const b2g_joint* joints, int32_t nj, const b2g_contact* contacts, int32_t nc, float inv_dt0) {
  World* w = (World*)h;
  w->bodies.resize(nb);
  for (int i = 0; i < nb; ++i) {
    const b2g_body& s = bodies[i];
    Body& b = w->bodies[i];
    b.xf.p = v2(s.xf[0], s.xf[1]); b.xf.q.s = s.xf[2]; b.xf.q.c = s.xf[3];
    b.c = v2(s.c[0], s.c[1]); b.a = s.a;
    b.v = v2(s.v[0], s.v[1]); b.w = s.w;
    b.localCenter = v2(s.local_center[0], s.local_center[1]);
    b.mass = s.mass; b.invMass = s.inv_mass; b.I = s.inertia; b.invI = s.inv_inertia;
    b.linearDamping = s.linear_damping; b.angularDamping = s.angular_damping; b.gravityScale = s.gravity_scale;
    b.force = v2(s.force[0], s.force[1]); b.torque = s.torque;
    b.type = s.type; b.flags = s.flags;
    b.sleepTime = 0.0f;
    b.c0 = b.c; b.a0 = b.a; b.alpha0 = 0.0f;
    if (b.type != 0 && !b.awake()) w->sleepers = true;
  }
  w->fixtures.resize(nf);
  for (int i = 0; i < nf; ++i) {
    const b2g_fixture& s = fixtures[i];
    Fixture& f = w->fixtures[i];
    f.shape = shapeFrom(s.shape);
    f.body = s.body;
    if (f.body < 0 || f.body >= nb) return 1;
    f.density = s.density; f.friction = s.friction; f.restitution = s.restitution;
    f.threshold = s.restitution_threshold;
    f.category = s.category_bits; f.mask = s.mask_bits; f.group = s.group_index;
    f.sensor = s.is_sensor != 0;
  }
  w->joints.resize(nj);
  for (int i = 0; i < nj; ++i) {
    Joint& J = w->joints[i];
    memset(&J, 0, sizeof(J));
    J.d = joints[i].def;
    J.impulse2 = v2(joints[i].impulse[0], joints[i].impulse[1]);
    J.impulse1 = joints[i].impulse[0];
    for (int k = 0; k < 3; ++k) J.imp[k] = joints[i].impulse[k];
    J.motorImpulse = joints[i].motor_impulse;
    J.lowerImpulse = joints[i].lower_impulse;
    J.upperImpulse = joints[i].upper_impulse;
    if (J.d.type == B2G_JOINT_PRISMATIC || J.d.type == B2G_JOINT_WHEEL) {
      J.localXAxisA = v2(J.d.local_axis_a[0], J.d.local_axis_a[1]);
      J.localYAxisA = cross(1.0f, J.localXAxisA);
    }
    if (J.d.type == B2G_JOINT_PULLEY) J.constant = J.d.length_a + J.d.ratio * J.d.length_b;
    if (J.d.body_a < 0 || J.d.body_a >= nb || J.d.body_b < 0 || J.d.body_b >= nb) return 1;
    if (J.d.type == B2G_JOINT_GEAR) {  // the two earlier joints it couples
      if (J.d.joint_1 < 0 || J.d.joint_1 >= i || J.d.joint_2 < 0 || J.d.joint_2 >= i) return 1;
      const b2g_joint_def& j1 = joints[J.d.joint_1].def;
      const b2g_joint_def& j2 = joints[J.d.joint_2].def;
      J.iC = j1.body_a; J.iD = j2.body_a;
      J.typeA = j1.type; J.typeB = j2.type;
      J.gLC = v2(j1.local_anchor_a[0], j1.local_anchor_a[1]); J.gLA = v2(j1.local_anchor_b[0], j1.local_anchor_b[1]);
      J.gLD = v2(j2.local_anchor_a[0], j2.local_anchor_a[1]); J.gLB = v2(j2.local_anchor_b[0], j2.local_anchor_b[1]);
      J.gRefA = j1.reference_angle; J.gRefB = j2.reference_angle;
      J.gAxC = j1.type == B2G_JOINT_PRISMATIC ? v2(j1.local_axis_a[0], j1.local_axis_a[1]) : v2(0.0f, 0.0f);
      J.gAxD = j2.type == B2G_JOINT_PRISMATIC ? v2(j2.local_axis_a[0], j2.local_axis_a[1]) : v2(0.0f, 0.0f);
    }
  }
  rebuildNoCollide(w);
  w->contacts.clear();
  for (int i = 0; i < nc; ++i) {
    const b2g_contact& s = contacts[i];
    int a = s.fixture_a, b = s.fixture_b;
    bool sa = w->bodies[w->fixtures[a].body].type == 0;
    bool sbb = w->bodies[w->fixtures[b].body].type == 0;
    int e, p;
    if (sa) { e = b; p = a; } else if (sbb) { e = a; p = b; } else { e = bmin(a, b); p = bmax(a, b); }
    Contact c = makeContact(*w, ((uint64_t)(uint32_t)e << 32) | (uint32_t)p);
    c.fA = a;  // a loaded contact keeps its orientation: its manifold was computed for it
    c.fB = b;
    c.flags = s.flags;
    c.friction = s.friction; c.restitution = s.restitution; c.threshold = s.restitution_threshold;
    c.tangentSpeed = s.tangent_speed;
    c.m = manifoldFrom(s.manifold);
    w->contacts.push_back(c);
  }
  std::sort(w->contacts.begin(), w->contacts.end(), [](const Contact& x, const Contact& y) { return x.key < y.key; });
  w->newContacts = (nc == 0);
  w->inv_dt0 = inv_dt0;
  return 0;
}

// b2World::SetAllowSleeping (src/dynamics/b2_world.cpp:474-488): turning sleep off wakes every body.
// b2World::SetContinuousPhysics
void orc_world_set_continuous(void* h, int32_t on) { ((World*)h)->continuous = on != 0; }

void orc_world_set_sleep(void* h, int32_t allow_sleep) {
  World* w = (World*)h;
  w->allowSleep = allow_sleep != 0;
  if (!w->allowSleep) {
    for (Body& b : w->bodies) setAwake(b, true);
    w->sleepers = false;
  }
}

// Marks the world's contacts for re-finding at the start of the next step (as b2World::Step does
// after bodies were moved or fixtures created, b2_world.cpp:1113-1122).
void orc_world_flag_new_contacts(void* h) { ((World*)h)->newContacts = true; }

void orc_world_sleep_times(void* h, float* out) {
  World* w = (World*)h;
  for (size_t i = 0; i < w->bodies.size(); ++i) out[i] = w->bodies[i].sleepTime;
}

void orc_world_set_sleep_times(void* h, const float* in) {
  World* w = (World*)h;
  for (size_t i = 0; i < w->bodies.size(); ++i) w->bodies[i].sleepTime = in[i];
}

// The last step's islands (sleep-mode worlds): counts[0..3] = islands, bodies, contacts, joints.
// Arrays (each may be null): per island root, orphan flag, body offsets (islands + 1), contact
// offsets (islands + 1, in contacts), joint offsets (islands + 1); then the bodies, the contacts
// as (fixture A, fixture B) pairs in solve order, and the joints in solve order.
void orc_world_last_islands(void* h, int32_t* counts, int32_t* root, int32_t* orphan, int32_t* body_off,
                            int32_t* contact_off, int32_t* joint_off, int32_t* bodies, int32_t* contacts,
                            int32_t* joints) {
  World* w = (World*)h;
  counts[0] = (int32_t)w->islandRoot.size();
  counts[1] = (int32_t)w->islandBodies.size();
  counts[2] = (int32_t)w->islandContacts.size() / 2;
  counts[3] = (int32_t)w->islandJoints.size();
  auto cp = [](int32_t* dst, const std::vector<int32_t>& v) {
    if (dst && !v.empty()) memcpy(dst, v.data(), v.size() * sizeof(int32_t));
  };
  cp(root, w->islandRoot); cp(orphan, w->islandOrphan); cp(body_off, w->islandBodyOff);
  cp(contact_off, w->islandContactOff); cp(joint_off, w->islandJointOff); cp(bodies, w->islandBodies);
  cp(contacts, w->islandContacts); cp(joints, w->islandJoints);
}

double orc_world_step(void* h, float dt, int32_t vi, int32_t pi, int32_t n) {
  World* w = (World*)h;
  auto t0 = std::chrono::steady_clock::now();
  for (int i = 0; i < n; ++i) stepWorld(w, dt, vi, pi);
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

int32_t orc_world_sizes(void* h, int32_t* out4) {
  World* w = (World*)h;
  out4[0] = (int32_t)w->bodies.size();
  out4[1] = (int32_t)w->fixtures.size();
  out4[2] = (int32_t)w->joints.size();
  out4[3] = (int32_t)w->contacts.size();
  return 0;
}

void orc_world_bodies(void* h, b2g_body* out) {
  World* w = (World*)h;
  for (size_t i = 0; i < w->bodies.size(); ++i) {
    const Body& b = w->bodies[i];
    b2g_body& s = out[i];
    memset(&s, 0, sizeof(s));
    s.xf[0] = b.xf.p.x; s.xf[1] = b.xf.p.y; s.xf[2] = b.xf.q.s; s.xf[3] = b.xf.q.c;
    s.c[0] = b.c.x; s.c[1] = b.c.y; s.a = b.a;
    s.v[0] = b.v.x; s.v[1] = b.v.y; s.w = b.w;
    s.local_center[0] = b.localCenter.x; s.local_center[1] = b.localCenter.y;
    s.mass = b.mass; s.inv_mass = b.invMass; s.inertia = b.I; s.inv_inertia = b.invI;
    s.linear_damping = b.linearDamping; s.angular_damping = b.angularDamping; s.gravity_scale = b.gravityScale;
    s.force[0] = b.force.x; s.force[1] = b.force.y; s.torque = b.torque;
    s.type = b.type; s.flags = b.flags;
  }
}

void orc_world_joints(void* h, b2g_joint* out) {
  World* w = (World*)h;
  for (size_t i = 0; i < w->joints.size(); ++i) {
    const Joint& J = w->joints[i];
    b2g_joint& s = out[i];
    memset(&s, 0, sizeof(s));
    s.def = J.d;
    if (J.d.type == B2G_JOINT_DISTANCE) s.impulse[0] = J.impulse1;
    else if (J.d.type != B2G_JOINT_REVOLUTE && J.d.type != B2G_JOINT_PRISMATIC)
      for (int k = 0; k < 3; ++k) s.impulse[k] = J.imp[k];
    else { s.impulse[0] = J.impulse2.x; s.impulse[1] = J.impulse2.y; }
    s.motor_impulse = J.motorImpulse; s.lower_impulse = J.lowerImpulse; s.upper_impulse = J.upperImpulse;
    float F[2], T;
    jointReaction(J, 1.0f, F, &T);
    s.reaction_impulse[0] = F[0]; s.reaction_impulse[1] = F[1]; s.reaction_angular_impulse = T;
  }
}

int32_t orc_world_contacts(void* h, b2g_contact* out, int32_t cap) {
  World* w = (World*)h;
  int32_t n = (int32_t)w->contacts.size();
  for (int32_t i = 0; i < n && i < cap; ++i) {
    const Contact& c = w->contacts[i];
    b2g_contact& s = out[i];
    memset(&s, 0, sizeof(s));
    s.fixture_a = c.fA; s.fixture_b = c.fB; s.flags = c.flags;
    s.friction = c.friction; s.restitution = c.restitution; s.restitution_threshold = c.threshold;
    s.tangent_speed = c.tangentSpeed;
    manifoldTo(c.m, &s.manifold);
  }
  return n;
}

int orc_world_solver_order(void* h, int32_t* ccol, uint32_t* cprio, int32_t nc, int32_t* jcol, uint32_t* jprio,
                           int32_t nj) {
  World* w = (World*)h;
  for (int i = 0; i < nc && i < (int)w->contactColor.size(); ++i) { ccol[i] = w->contactColor[i]; cprio[i] = w->contactPrio[i]; }
  for (int j = 0; j < nj && j < (int)w->jointColor.size(); ++j) { jcol[j] = w->jointColor[j]; jprio[j] = w->jointPrioV[j]; }
  return 0;
}

// ---- world queries (brute force over the world's fixtures) --------------------------------
// b2World::QueryAABB (src/dynamics/b2_world.cpp:1193-1207 over b2BroadPhase::Query,
// include/box2d/b2_broad_phase.h:622-644): fixtures whose AABB overlaps the box, ascending; a
// world of one fixture reports it for any box (the tree's root leaf is reported untested).
int32_t orc_world_query_aabb(void* h, const float* box4, int32_t* out, int32_t cap) {
  World* w = (World*)h;
  AABB q;
  q.lo = v2(box4[0], box4[1]);
  q.hi = v2(box4[2], box4[3]);
  int32_t n = 0;
  for (size_t f = 0; f < w->fixtures.size(); ++f) {
    const Fixture& fx = w->fixtures[f];
    AABB bb = computeAABB(fx.shape, w->bodies[fx.body].xf);
    if (w->fixtures.size() == 1 || overlap(bb, q)) {
      if (n < cap) out[n] = (int32_t)f;
      ++n;
    }
  }
  return n;
}

struct RayOut {
  float fraction;
  V2 normal;
};

// b2PolygonShape::RayCast (src/collision/b2_polygon_shape.cpp:303-364)
static bool rayPolygon(const Shape& s, const Xf& xf, V2 P1, V2 P2, float maxFraction, RayOut* out) {
  V2 p1 = mulT(xf.q, P1 - xf.p), p2 = mulT(xf.q, P2 - xf.p);
  V2 d = p2 - p1;
  float lower = 0.0f, upper = maxFraction;
  int index = -1;
  for (int i = 0; i < s.count; ++i) {
    float num = dot(s.n[i], s.v[i] - p1);
    float den = dot(s.n[i], d);
    if (den == 0.0f) {
      if (num < 0.0f) return false;
    } else if (den < 0.0f && num < lower * den) {
      lower = num / den;
      index = i;
    } else if (den > 0.0f && num < upper * den) {
      upper = num / den;
    }
    if (upper < lower) return false;
  }
  if (index < 0) return false;
  out->fraction = lower;
  out->normal = mul(xf.q, s.n[index]);
  return true;
}

// b2CircleShape::RayCast (src/collision/b2_circle_shape.cpp:56-87)
static bool rayCircle(const Shape& s, const Xf& xf, V2 P1, V2 P2, float maxFraction, RayOut* out) {
  V2 position = xf.p + mul(xf.q, s.v[0]);
  V2 sv = P1 - position;
  float b = dot(sv, sv) - s.radius * s.radius;
  V2 r = P2 - P1;
  float c = dot(sv, r);
  float rr = dot(r, r);
  float sigma = c * c - rr * b;
  if (sigma < 0.0f || rr < 1.192092896e-07f) return false;
  float a = -(c + sqrtf(sigma));
  if (!(0.0f <= a && a <= maxFraction * rr)) return false;
  a /= rr;
  out->fraction = a;
  V2 n = sv + a * r;
  normalize(n);
  out->normal = n;
  return true;
}

// b2EdgeShape::RayCast (src/collision/b2_edge_shape.cpp:89-149)
static bool rayEdge(const Shape& s, const Xf& xf, V2 P1, V2 P2, float maxFraction, RayOut* out) {
  V2 p1 = mulT(xf.q, P1 - xf.p), p2 = mulT(xf.q, P2 - xf.p);
  V2 d = p2 - p1;
  V2 v1 = s.v[0], v2_ = s.v[1];
  V2 e = v2_ - v1;
  V2 normal = v2(e.y, -e.x);
  normalize(normal);
  float num = dot(normal, v1 - p1);
  if (s.oneSided && num > 0.0f) return false;
  float den = dot(normal, d);
  if (den == 0.0f) return false;
  float t = num / den;
  if (t < 0.0f || maxFraction < t) return false;
  V2 q = p1 + t * d;
  V2 r = v2_ - v1;
  float rr = dot(r, r);
  if (rr == 0.0f) return false;
  float sc = dot(q - v1, r) / rr;
  if (sc < 0.0f || 1.0f < sc) return false;
  out->fraction = t;
  out->normal = num > 0.0f ? -mul(xf.q, normal) : mul(xf.q, normal);
  return true;
}

// b2World::RayCast with a closest-hit callback (src/dynamics/b2_world.cpp:1209-1238 over
// b2BroadPhase::RayCast, include/box2d/b2_broad_phase.h:646-710): every fixture whose AABB
// passes the segment-box and separating-axis tests is ray cast against the segment clipped to
// the best fraction so far. Returns the fixture index (-1: no hit); out5 = point, normal,
// fraction. A tie keeps the lower index.
int32_t orc_world_raycast(void* h, const float* ray4, float* out5) {
  World* w = (World*)h;
  V2 p1 = v2(ray4[0], ray4[1]), p2 = v2(ray4[2], ray4[3]);
  V2 r = p2 - p1;
  if (normalize(r) == 0.0f) return -1;
  V2 v = cross(1.0f, r);
  V2 absV = v2(fabsf(v.x), fabsf(v.y));
  float maxFraction = 1.0f;
  int best = -1;
  RayOut bo = {0.0f, v2(0.0f, 0.0f)};
  for (size_t f = 0; f < w->fixtures.size(); ++f) {
    const Fixture& fx = w->fixtures[f];
    const Xf& xf = w->bodies[fx.body].xf;
    AABB bb = computeAABB(fx.shape, xf);
    V2 t = p1 + maxFraction * (p2 - p1);
    AABB seg;
    seg.lo = vmin(p1, t);
    seg.hi = vmax(p1, t);
    if (!overlap(bb, seg)) continue;
    V2 c = 0.5f * (bb.lo + bb.hi);
    V2 hh = 0.5f * (bb.hi - bb.lo);
    float separation = fabsf(dot(v, p1 - c)) - dot(absV, hh);
    if (separation > 0.0f) continue;
    RayOut o;
    bool hit = fx.shape.type == 0 ? rayCircle(fx.shape, xf, p1, p2, maxFraction, &o)
               : fx.shape.type == 1 ? rayEdge(fx.shape, xf, p1, p2, maxFraction, &o)
                                    : rayPolygon(fx.shape, xf, p1, p2, maxFraction, &o);
    if (!hit) continue;
    if (best >= 0 && o.fraction == bo.fraction) continue;  // fixtures are visited in ascending order
    best = (int)f;
    bo = o;
    maxFraction = o.fraction;
  }
  if (best < 0) return -1;
  V2 point = (1.0f - bo.fraction) * p1 + bo.fraction * p2;
  out5[0] = point.x;
  out5[1] = point.y;
  out5[2] = bo.normal.x;
  out5[3] = bo.normal.y;
  out5[4] = bo.fraction;
  return best;
}

// The Gauss-Seidel order of the last step: (fixture A, fixture B) per solved contact and joint
// indices, both in solve order. Returns the number of solved contacts.
int32_t orc_world_last_order(void* h, int32_t* pairs, int32_t cap_pairs, int32_t* joints, int32_t cap_joints,
                             int32_t* n_joints) {
  World* w = (World*)h;
  int32_t nc = (int32_t)(w->lastContactOrder.size() / 2);
  for (int32_t i = 0; i < 2 * nc && i < 2 * cap_pairs; ++i) pairs[i] = w->lastContactOrder[i];
  int32_t nj = (int32_t)w->lastJointOrder.size();
  for (int32_t j = 0; j < nj && j < cap_joints; ++j) joints[j] = w->lastJointOrder[j];
  if (n_joints) *n_joints = nj;
  return nc;
}

// Steps n worlds on `threads` host threads (disjoint subsets); returns wall seconds.
double orc_worlds_step_parallel(void** hs, int32_t n, float dt, int32_t vi, int32_t pi, int32_t nsteps,
                                int32_t threads) {
  auto t0 = std::chrono::steady_clock::now();
  std::vector<std::thread> th;
  for (int t = 0; t < threads; ++t) {
    th.emplace_back([=]() {
      for (int i = t; i < n; i += threads)
        for (int s = 0; s < nsteps; ++s) stepWorld((World*)hs[i], dt, vi, pi);
    });
  }
  for (auto& x : th) x.join();
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // extern "C"
