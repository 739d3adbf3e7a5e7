// shapes.cpp - host-side shape set-up and mass data (run when fixtures are created).
//
// b2PolygonShape::Set / SetAsBox, ComputeMass, b2Body::ResetMassData, with the reference's
// operation order so that the processed shapes and mass data are bit-identical to what the
// reference's CreateFixture produces. Compiled with -ffp-contract=off.
#include <math.h>
#include <string.h>

#include "b2g_math.cuh"
#include "engine.h"

namespace b2g {

// b2PolygonShape::SetAsBox (src/collision/b2_polygon_shape.cpp:36-75); the oriented form uses
// libm sinf/cosf like b2Rot::Set (include/box2d/b2_math.h:313-318).
void polygon_box(b2g_shape* p, float hx, float hy, bool oriented, float cx, float cy, float angle) {
  memset(p, 0, sizeof(*p));
  p->type = B2G_SHAPE_POLYGON;
  p->radius = B2G_POLYGON_RADIUS;
  p->count = 4;
  V2 v[4] = {mk(-hx, -hy), mk(hx, -hy), mk(hx, hy), mk(-hx, hy)};
  V2 n[4] = {mk(0.0f, -1.0f), mk(1.0f, 0.0f), mk(0.0f, 1.0f), mk(-1.0f, 0.0f)};
  V2 centroid = mk(0.0f, 0.0f);
  if (oriented) {
    centroid = mk(cx, cy);
    Xf xf;
    xf.p = centroid;
    xf.q.s = sinf(angle);
    xf.q.c = cosf(angle);
    for (int i = 0; i < 4; ++i) {
      v[i] = mul(xf, v[i]);
      n[i] = mul(xf.q, n[i]);
    }
  }
  for (int i = 0; i < 4; ++i) {
    p->vertices[i][0] = v[i].x; p->vertices[i][1] = v[i].y;
    p->normals[i][0] = n[i].x; p->normals[i][1] = n[i].y;
  }
  p->centroid[0] = centroid.x;
  p->centroid[1] = centroid.y;
}

// ComputeCentroid (src/collision/b2_polygon_shape.cpp:77-111)
static V2 compute_centroid(const V2* vs, int count) {
  V2 c = mk(0.0f, 0.0f);
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
  return (1.0f / area) * c + s;
}

// b2PolygonShape::Set (src/collision/b2_polygon_shape.cpp:113-243): welding, gift-wrapping
// hull from the right-most (then lowest) point, edge normals, centroid. Degenerate input
// falls back to SetAsBox(1, 1) as the reference does.
void polygon_set(b2g_shape* p, const float* xy, int count) {
  if (count < 3) { polygon_box(p, 1.0f, 1.0f, false, 0, 0, 0); return; }
  int n = imin2(count, B2G_MAX_POLYGON_VERTICES);
  V2 ps[B2G_MAX_POLYGON_VERTICES];
  int tempCount = 0;
  for (int i = 0; i < n; ++i) {
    V2 v = mk(xy[2 * i], xy[2 * i + 1]);
    bool unique = true;
    for (int j = 0; j < tempCount; ++j) {
      if (distSq(v, ps[j]) < ((0.5f * B2G_LINEAR_SLOP) * (0.5f * B2G_LINEAR_SLOP))) { unique = false; break; }
    }
    if (unique) ps[tempCount++] = v;
  }
  n = tempCount;
  if (n < 3) { polygon_box(p, 1.0f, 1.0f, false, 0, 0, 0); return; }
  int i0 = 0;
  float x0 = ps[0].x;
  for (int i = 1; i < n; ++i) {
    float x = ps[i].x;
    if (x > x0 || (x == x0 && ps[i].y < ps[i0].y)) { i0 = i; x0 = x; }
  }
  int hull[B2G_MAX_POLYGON_VERTICES];
  int m = 0;
  int ih = i0;
  for (;;) {
    if (m >= B2G_MAX_POLYGON_VERTICES) break;
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
  if (m < 3) { polygon_box(p, 1.0f, 1.0f, false, 0, 0, 0); return; }
  memset(p, 0, sizeof(*p));
  p->type = B2G_SHAPE_POLYGON;
  p->radius = B2G_POLYGON_RADIUS;
  p->count = m;
  V2 vs[B2G_MAX_POLYGON_VERTICES];
  for (int i = 0; i < m; ++i) vs[i] = ps[hull[i]];
  for (int i = 0; i < m; ++i) {
    int i2 = i + 1 < m ? i + 1 : 0;
    V2 edge = vs[i2] - vs[i];
    V2 nn = cross(edge, 1.0f);
    normalize(nn);
    p->vertices[i][0] = vs[i].x; p->vertices[i][1] = vs[i].y;
    p->normals[i][0] = nn.x; p->normals[i][1] = nn.y;
  }
  V2 c = compute_centroid(vs, m);
  p->centroid[0] = c.x;
  p->centroid[1] = c.y;
}

// ComputeMass: polygon (src/collision/b2_polygon_shape.cpp:390-464), circle
// (src/collision/b2_circle_shape.cpp:98-104), edge (src/collision/b2_edge_shape.cpp:169-176).
void shape_mass(const b2g_shape& s, float density, float* mass, float* cx, float* cy, float* I) {
  if (s.type == B2G_SHAPE_CIRCLE) {
    float m = density * B2G_PI * s.radius * s.radius;
    V2 p = sv(s, 0);
    *mass = m; *cx = p.x; *cy = p.y;
    *I = m * (0.5f * s.radius * s.radius + dot(p, p));
    return;
  }
  if (s.type == B2G_SHAPE_EDGE) {
    V2 c = 0.5f * (sv(s, 0) + sv(s, 1));
    *mass = 0.0f; *cx = c.x; *cy = c.y; *I = 0.0f;
    return;
  }
  V2 center = mk(0.0f, 0.0f);
  float area = 0.0f;
  float inertia = 0.0f;
  V2 sref = sv(s, 0);
  const float k_inv3 = 1.0f / 3.0f;
  for (int i = 0; i < s.count; ++i) {
    V2 e1 = sv(s, i) - sref;
    V2 e2 = i + 1 < s.count ? sv(s, i + 1) - sref : sv(s, 0) - sref;
    float D = cross(e1, e2);
    float triangleArea = 0.5f * D;
    area += triangleArea;
    addTo(center, (triangleArea * k_inv3) * (e1 + e2));
    float ex1 = e1.x, ey1 = e1.y;
    float ex2 = e2.x, ey2 = e2.y;
    float intx2 = ex1 * ex1 + ex2 * ex1 + ex2 * ex2;
    float inty2 = ey1 * ey1 + ey2 * ey1 + ey2 * ey2;
    inertia += (0.25f * k_inv3 * D) * (intx2 + inty2);
  }
  float m = density * area;
  float inv = 1.0f / area;
  center.x *= inv;
  center.y *= inv;
  V2 mc = center + sref;
  float Iv = density * inertia;
  Iv += m * (dot(mc, mc) - dot(center, center));
  *mass = m; *cx = mc.x; *cy = mc.y; *I = Iv;
}

// b2Fixture::Create (src/dynamics/b2_fixture.cpp:44-66) with the shape built from the def.
int process_fixture_def(const b2g_fixture_def& d, b2g_fixture* out) {
  memset(out, 0, sizeof(*out));
  b2g_shape& s = out->shape;
  if (d.shape_type == B2G_SHAPE_CIRCLE) {
    if (!(d.radius > 0.0f) || !isfinite(d.center[0]) || !isfinite(d.center[1])) return B2G_E_INVALID_ARG;
    s.type = B2G_SHAPE_CIRCLE;
    s.radius = d.radius;
    s.vertices[0][0] = d.center[0];
    s.vertices[0][1] = d.center[1];
  } else if (d.shape_type == B2G_SHAPE_EDGE) {
    s.type = B2G_SHAPE_EDGE;
    s.radius = B2G_POLYGON_RADIUS;
    for (int i = 0; i < 4; ++i) {
      s.vertices[i][0] = d.verts[i][0];
      s.vertices[i][1] = d.verts[i][1];
      if (!isfinite(d.verts[i][0]) || !isfinite(d.verts[i][1])) return B2G_E_INVALID_ARG;
    }
    s.one_sided = d.one_sided ? 1 : 0;
  } else if (d.shape_type == B2G_SHAPE_POLYGON) {
    if (d.poly_mode == B2G_POLY_HULL) {
      if (d.count < 3 || d.count > B2G_MAX_POLYGON_VERTICES) return B2G_E_INVALID_ARG;
      for (int i = 0; i < d.count; ++i)
        if (!isfinite(d.verts[i][0]) || !isfinite(d.verts[i][1])) return B2G_E_INVALID_ARG;
      polygon_set(&s, &d.verts[0][0], d.count);
    } else if (d.poly_mode == B2G_POLY_BOX || d.poly_mode == B2G_POLY_BOX_ORIENTED) {
      if (!(d.box[0] > 0.0f) || !(d.box[1] > 0.0f)) return B2G_E_INVALID_ARG;
      polygon_box(&s, d.box[0], d.box[1], d.poly_mode == B2G_POLY_BOX_ORIENTED, d.box[2], d.box[3], d.box[4]);
    } else if (d.poly_mode == B2G_POLY_RAW) {
      if (d.shape.type != B2G_SHAPE_POLYGON || d.shape.count < 3 || d.shape.count > B2G_MAX_POLYGON_VERTICES)
        return B2G_E_INVALID_ARG;
      s = d.shape;
    } else {
      return B2G_E_INVALID_ARG;
    }
  } else {
    return B2G_E_INVALID_ARG;
  }
  out->body = d.body;
  out->density = d.density;
  out->friction = d.friction;
  out->restitution = d.restitution;
  out->restitution_threshold = d.restitution_threshold;
  out->category_bits = d.category_bits;
  out->mask_bits = d.mask_bits;
  out->group_index = d.group_index;
  out->is_sensor = d.is_sensor ? 1 : 0;
  return B2G_OK;
}

// b2Body::ResetMassData (src/dynamics/b2_body.cpp:352-416). Fixtures are visited newest first,
// the order of the body's prepended fixture list.
void reset_mass_data(HostWorld& w, int bi) {
  b2g_body& b = w.bodies[bi];
  b.mass = 0.0f; b.inv_mass = 0.0f; b.inertia = 0.0f; b.inv_inertia = 0.0f;
  b.local_center[0] = 0.0f; b.local_center[1] = 0.0f;
  if (b.type == B2G_STATIC || b.type == B2G_KINEMATIC) {
    b.c[0] = b.xf[0];
    b.c[1] = b.xf[1];
    return;
  }
  V2 localCenter = mk(0.0f, 0.0f);
  float mass = 0.0f, I = 0.0f;
  const std::vector<int>& fl = w.body_fixtures[bi];
  for (int k = (int)fl.size() - 1; k >= 0; --k) {
    const b2g_fixture& f = w.fixtures[fl[k]];
    if (f.density == 0.0f) continue;
    float m, cx, cy, fI;
    shape_mass(f.shape, f.density, &m, &cx, &cy, &fI);
    mass += m;
    addTo(localCenter, m * mk(cx, cy));
    I += fI;
  }
  float invMass = 0.0f, invI = 0.0f;
  if (mass > 0.0f) {
    invMass = 1.0f / mass;
    localCenter.x *= invMass;
    localCenter.y *= invMass;
  }
  if (I > 0.0f && (b.flags & B2G_BODY_FIXED_ROTATION) == 0) {
    I -= mass * dot(localCenter, localCenter);
    invI = 1.0f / I;
  } else {
    I = 0.0f;
    invI = 0.0f;
  }
  V2 oldCenter = mk(b.c[0], b.c[1]);
  Xf xf;
  xf.p = mk(b.xf[0], b.xf[1]);
  xf.q.s = b.xf[2];
  xf.q.c = b.xf[3];
  V2 c = mul(xf, localCenter);
  b.mass = mass; b.inv_mass = invMass; b.inertia = I; b.inv_inertia = invI;
  b.local_center[0] = localCenter.x; b.local_center[1] = localCenter.y;
  b.c[0] = c.x; b.c[1] = c.y;
  V2 dv = cross(b.w, c - oldCenter);
  b.v[0] += dv.x;
  b.v[1] += dv.y;
}

}  // namespace b2g
