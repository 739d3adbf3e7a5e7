// ref_shim.cpp - test-only C wrapper around the reference engine compiled from its own sources
// (see Makefile target `ref`). It exists to pin the oracle restatement and to generate golden
// fixtures in a container that has the reference checked out; nothing in the product links it.
//
// It exposes: the reference's shape set-up and collide functions on b2g_* POD records, worlds
// built by the shared scene recipes, state export in b2g_* records, and a "replay" step that runs
// the reference b2Island solver with a caller-given constraint order (src/dynamics/b2_island.cpp:253).

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <new>
#include <random>
#include <unordered_map>
#include <vector>

// The replay harness needs the reference's internal members (island, contact manager, joint
// impulses); the test shim opens them up instead of changing the reference.
#define private public
#define protected public
#include "box2d/box2d.h"
#include "box2d/b2_distance.h"
#include "box2d/b2_time_of_impact.h"
#include "dynamics/b2_contact_solver.h"
#include "dynamics/b2_island.h"
#include "box2d/b2_stack_allocator.h"
#undef private
#undef protected

#include "../include/b2g_capi.h"
#include "scenes/scenes_joints.h"

extern "C" {

// ---------------------------------------------------------------- shapes
static void shape_from_ref(const b2Shape* s, b2g_shape* o) {
  memset(o, 0, sizeof(*o));
  o->type = (int32_t)s->m_type;
  o->radius = s->m_radius;
  if (s->m_type == b2Shape::e_circle) {
    const b2CircleShape* c = (const b2CircleShape*)s;
    o->vertices[0][0] = c->m_p.x;
    o->vertices[0][1] = c->m_p.y;
  } else if (s->m_type == b2Shape::e_edge) {
    const b2EdgeShape* e = (const b2EdgeShape*)s;
    o->vertices[0][0] = e->m_vertex1.x; o->vertices[0][1] = e->m_vertex1.y;
    o->vertices[1][0] = e->m_vertex2.x; o->vertices[1][1] = e->m_vertex2.y;
    o->vertices[2][0] = e->m_vertex0.x; o->vertices[2][1] = e->m_vertex0.y;
    o->vertices[3][0] = e->m_vertex3.x; o->vertices[3][1] = e->m_vertex3.y;
    o->one_sided = e->m_oneSided ? 1 : 0;
  } else if (s->m_type == b2Shape::e_polygon) {
    const b2PolygonShape* p = (const b2PolygonShape*)s;
    o->count = p->m_count;
    for (int i = 0; i < p->m_count; ++i) {
      o->vertices[i][0] = p->m_vertices[i].x; o->vertices[i][1] = p->m_vertices[i].y;
      o->normals[i][0] = p->m_normals[i].x; o->normals[i][1] = p->m_normals[i].y;
    }
    o->centroid[0] = p->m_centroid.x; o->centroid[1] = p->m_centroid.y;
  }
}

struct AnyShape {
  b2CircleShape circle;
  b2EdgeShape edge;
  b2PolygonShape poly;
  const b2Shape* ptr = nullptr;
};

static void shape_to_ref(const b2g_shape* o, AnyShape* a) {
  if (o->type == B2G_SHAPE_CIRCLE) {
    a->circle.m_radius = o->radius;
    a->circle.m_p.Set(o->vertices[0][0], o->vertices[0][1]);
    a->ptr = &a->circle;
  } else if (o->type == B2G_SHAPE_EDGE) {
    a->edge.m_radius = o->radius;
    a->edge.m_vertex1.Set(o->vertices[0][0], o->vertices[0][1]);
    a->edge.m_vertex2.Set(o->vertices[1][0], o->vertices[1][1]);
    a->edge.m_vertex0.Set(o->vertices[2][0], o->vertices[2][1]);
    a->edge.m_vertex3.Set(o->vertices[3][0], o->vertices[3][1]);
    a->edge.m_oneSided = o->one_sided != 0;
    a->ptr = &a->edge;
  } else {
    a->poly.m_radius = o->radius;
    a->poly.m_count = o->count;
    for (int i = 0; i < o->count; ++i) {
      a->poly.m_vertices[i].Set(o->vertices[i][0], o->vertices[i][1]);
      a->poly.m_normals[i].Set(o->normals[i][0], o->normals[i][1]);
    }
    a->poly.m_centroid.Set(o->centroid[0], o->centroid[1]);
    a->ptr = &a->poly;
  }
}

static b2Transform xf_from(const float* x) {
  b2Transform t;
  t.p.Set(x[0], x[1]);
  t.q.s = x[2];
  t.q.c = x[3];
  return t;
}

static void manifold_out(const b2Manifold& m, b2g_manifold* o) {
  memset(o, 0, sizeof(*o));
  for (int i = 0; i < 2; ++i) {
    o->points[i].local_point[0] = m.points[i].localPoint.x;
    o->points[i].local_point[1] = m.points[i].localPoint.y;
    o->points[i].normal_impulse = m.points[i].normalImpulse;
    o->points[i].tangent_impulse = m.points[i].tangentImpulse;
    o->points[i].id = m.points[i].id.key;
  }
  o->local_normal[0] = m.localNormal.x; o->local_normal[1] = m.localNormal.y;
  o->local_point[0] = m.localPoint.x; o->local_point[1] = m.localPoint.y;
  o->type = (int32_t)m.type;
  o->point_count = m.pointCount;
}

static b2Sweep sweep_to_ref(const b2g_sweep& s) {
  b2Sweep o;
  o.localCenter.Set(s.local_center[0], s.local_center[1]);
  o.c0.Set(s.c0[0], s.c0[1]);
  o.c.Set(s.c[0], s.c[1]);
  o.a0 = s.a0;
  o.a = s.a;
  o.alpha0 = s.alpha0;
  return o;
}

// The reference's b2TimeOfImpact (src/collision/b2_time_of_impact.cpp:258) for n inputs.
void ref_time_of_impact(const b2g_toi_input* in, int32_t n, b2g_toi_output* out) {
  for (int32_t i = 0; i < n; ++i) {
    AnyShape a, b;
    shape_to_ref(&in[i].shape_a, &a);
    shape_to_ref(&in[i].shape_b, &b);
    b2TOIInput ti;
    ti.proxyA.Set(a.ptr);
    ti.proxyB.Set(b.ptr);
    ti.sweepA = sweep_to_ref(in[i].sweep_a);
    ti.sweepB = sweep_to_ref(in[i].sweep_b);
    ti.tMax = in[i].t_max;
    b2TOIOutput to;
    b2TimeOfImpact(&to, &ti);
    out[i].state = (int32_t)to.state;
    out[i].t = to.t;
  }
}

int ref_polygon_set(const float* xy, int32_t n, b2g_shape* out) {
  b2Vec2 v[b2_maxPolygonVertices];
  for (int i = 0; i < n && i < b2_maxPolygonVertices; ++i) v[i].Set(xy[2 * i], xy[2 * i + 1]);
  b2PolygonShape p;
  p.Set(v, n);
  shape_from_ref(&p, out);
  return 0;
}

int ref_polygon_box(float hx, float hy, float cx, float cy, float angle, int32_t oriented,
                    b2g_shape* out) {
  b2PolygonShape p;
  if (oriented) p.SetAsBox(hx, hy, b2Vec2(cx, cy), angle);
  else p.SetAsBox(hx, hy);
  shape_from_ref(&p, out);
  return 0;
}

int ref_shape_mass(const b2g_shape* s, float density, float* out4) {
  AnyShape a;
  shape_to_ref(s, &a);
  b2MassData md;
  a.ptr->ComputeMass(&md, density);
  out4[0] = md.mass; out4[1] = md.center.x; out4[2] = md.center.y; out4[3] = md.I;
  return 0;
}

int ref_shape_aabb(const b2g_shape* s, const float* xf, float* out4) {
  AnyShape a;
  shape_to_ref(s, &a);
  b2AABB bb;
  a.ptr->ComputeAABB(&bb, xf_from(xf));
  out4[0] = bb.lowerBound.x; out4[1] = bb.lowerBound.y;
  out4[2] = bb.upperBound.x; out4[3] = bb.upperBound.y;
  return 0;
}

// Manifold of shapes A (type >= B's type) and B with the reference collide function picked by
// b2Contact's dispatch table (src/dynamics/b2_contact.cpp:46-56).
int ref_collide(const b2g_shape* sa, const float* xfa, const b2g_shape* sb, const float* xfb,
                b2g_manifold* out) {
  AnyShape a, b;
  shape_to_ref(sa, &a);
  shape_to_ref(sb, &b);
  b2Transform ta = xf_from(xfa), tb = xf_from(xfb);
  b2Manifold m;
  memset(&m, 0, sizeof(m));
  int ka = sa->type, kb = sb->type;
  if (ka == B2G_SHAPE_CIRCLE && kb == B2G_SHAPE_CIRCLE)
    b2CollideCircles(&m, &a.circle, ta, &b.circle, tb);
  else if (ka == B2G_SHAPE_POLYGON && kb == B2G_SHAPE_CIRCLE)
    b2CollidePolygonAndCircle(&m, &a.poly, ta, &b.circle, tb);
  else if (ka == B2G_SHAPE_POLYGON && kb == B2G_SHAPE_POLYGON)
    b2CollidePolygons(&m, &a.poly, ta, &b.poly, tb);
  else if (ka == B2G_SHAPE_EDGE && kb == B2G_SHAPE_CIRCLE)
    b2CollideEdgeAndCircle(&m, &a.edge, ta, &b.circle, tb);
  else if (ka == B2G_SHAPE_EDGE && kb == B2G_SHAPE_POLYGON)
    b2CollideEdgeAndPolygon(&m, &a.edge, ta, &b.poly, tb);
  else
    return 1;
  manifold_out(m, out);
  return 0;
}

// b2Distance with radii between two shapes (distance out) and b2TestOverlap (returned).
int ref_test_overlap(const b2g_shape* sa, const float* xfa, const b2g_shape* sb, const float* xfb, float* distance) {
  AnyShape a, b;
  shape_to_ref(sa, &a);
  shape_to_ref(sb, &b);
  b2DistanceInput input;
  input.proxyA.Set(a.ptr);
  input.proxyB.Set(b.ptr);
  input.transformA = xf_from(xfa);
  input.transformB = xf_from(xfb);
  input.useRadii = true;
  b2SimplexCache cache;
  cache.count = 0;
  b2DistanceOutput output;
  b2Distance(&output, &cache, &input);
  *distance = output.distance;
  return b2TestOverlap(a.ptr, b.ptr, xf_from(xfa), xf_from(xfb)) ? 1 : 0;
}

// b2WorldManifold::Initialize (src/collision/b2_collision.cpp:26-90): out = normal(2), points(4),
// separations(2).
int ref_world_manifold(const b2g_manifold* mi, const float* xfa, float ra, const float* xfb,
                       float rb, float* out8) {
  b2Manifold m;
  memset(&m, 0, sizeof(m));
  for (int i = 0; i < 2; ++i) {
    m.points[i].localPoint.Set(mi->points[i].local_point[0], mi->points[i].local_point[1]);
    m.points[i].id.key = mi->points[i].id;
  }
  m.localNormal.Set(mi->local_normal[0], mi->local_normal[1]);
  m.localPoint.Set(mi->local_point[0], mi->local_point[1]);
  m.type = (b2Manifold::Type)mi->type;
  m.pointCount = mi->point_count;
  b2WorldManifold wm;
  memset(&wm, 0, sizeof(wm));
  wm.Initialize(&m, xf_from(xfa), ra, xf_from(xfb), rb);
  out8[0] = wm.normal.x; out8[1] = wm.normal.y;
  out8[2] = wm.points[0].x; out8[3] = wm.points[0].y;
  out8[4] = wm.points[1].x; out8[5] = wm.points[1].y;
  out8[6] = wm.separations[0]; out8[7] = wm.separations[1];
  return 0;
}

// ---------------------------------------------------------------- worlds
struct RefWorld;

// A b2ContactListener that records every callback of the reference's own Step as an engine
// event record (fixtures by creation index; PreSolve with the old manifold, PostSolve with the
// b2ContactImpulse entries the solver filled).
struct EventRecorder : public b2ContactListener {
  RefWorld* rw = nullptr;
  std::vector<b2g_event> events;
  void add(int kind, b2Contact* c, const b2Manifold* old, const b2ContactImpulse* imp);
  void BeginContact(b2Contact* c) override { add(B2G_EVENT_BEGIN, c, nullptr, nullptr); }
  void EndContact(b2Contact* c) override { add(B2G_EVENT_END, c, nullptr, nullptr); }
  void PreSolve(b2Contact* c, const b2Manifold* old) override { add(B2G_EVENT_PRESOLVE, c, old, nullptr); }
  void PostSolve(b2Contact* c, const b2ContactImpulse* imp) override { add(B2G_EVENT_POSTSOLVE, c, nullptr, imp); }
};

struct RefWorld {
  b2World* world;
  std::vector<b2Body*> bodies;      // creation order
  std::vector<b2Fixture*> fixtures; // creation order
  std::vector<b2Joint*> joints;     // creation order
  std::unordered_map<const b2Body*, int> body_index;
  std::unordered_map<const b2Fixture*, int> fixture_index;
  std::unordered_map<const b2Joint*, int> joint_index;
  EventRecorder recorder;
};

void EventRecorder::add(int kind, b2Contact* c, const b2Manifold* old, const b2ContactImpulse* imp) {
  b2g_event e;
  memset(&e, 0, sizeof(e));
  e.kind = kind;
  e.fixture_a = rw->fixture_index[c->GetFixtureA()];
  e.fixture_b = rw->fixture_index[c->GetFixtureB()];
  if (old) manifold_out(*old, &e.old_manifold);
  if (imp) {
    e.point_count = imp->count;
    for (int k = 0; k < imp->count && k < 2; ++k) {
      e.normal_impulses[k] = imp->normalImpulses[k];
      e.tangent_impulses[k] = imp->tangentImpulses[k];
    }
  }
  events.push_back(e);
}

static void index_world(RefWorld* rw) {
  rw->bodies.clear(); rw->fixtures.clear(); rw->joints.clear();
  rw->body_index.clear(); rw->fixture_index.clear(); rw->joint_index.clear();
  std::vector<std::pair<uintptr_t, b2Body*>> bs;
  std::vector<std::pair<uintptr_t, b2Fixture*>> fs;
  for (b2Body* b = rw->world->GetBodyList(); b; b = b->GetNext()) {
    bs.push_back({b->GetUserData().pointer, b});
    for (b2Fixture* f = b->GetFixtureList(); f; f = f->GetNext())
      fs.push_back({f->GetUserData().pointer, f});
  }
  std::sort(bs.begin(), bs.end());
  std::sort(fs.begin(), fs.end());
  for (auto& p : bs) { rw->body_index[p.second] = (int)rw->bodies.size(); rw->bodies.push_back(p.second); }
  for (auto& p : fs) { rw->fixture_index[p.second] = (int)rw->fixtures.size(); rw->fixtures.push_back(p.second); }
  std::vector<b2Joint*> js;
  for (b2Joint* j = rw->world->GetJointList(); j; j = j->GetNext()) js.push_back(j);
  std::reverse(js.begin(), js.end());  // the world list is prepended: reverse = creation order
  for (b2Joint* j : js) { rw->joint_index[j] = (int)rw->joints.size(); rw->joints.push_back(j); }
}

// Creates a world with gravity (gx, gy) and builds scene `kind` (the B2G_SCENE_* recipes).
void* ref_scene_world(int32_t kind, uint32_t seed, int32_t n, float p0, float p1, float gx,
                      float gy, int32_t* counts) {
  RefWorld* rw = new RefWorld();
  rw->world = new b2World(b2Vec2(gx, gy));
  b2scenes::ResetTags();
  b2scenes::Counts c;
  if (kind == B2G_SCENE_PYRAMID) c = b2scenes::Pyramid(rw->world, n, p0, p1, true);
  else if (kind == B2G_SCENE_MIXED_DROP) c = b2scenes::MixedDrop(rw->world, n, seed);
  else if (kind == B2G_SCENE_CHAINS) c = b2scenes::ChainsOverPile(rw->world, n, 20, (int)p0, seed);
  else if (kind == B2G_SCENE_BATCH_WORLD) c = b2scenes::BatchWorld(rw->world, seed, n);
  else if (kind == B2G_SCENE_JOINTS) c = b2scenes::JointZoo(rw->world, n, seed);
  else if (kind == B2G_SCENE_SLIDERS) c = b2scenes::SliderRigs(rw->world, n, seed);
  else if (kind == B2G_SCENE_GEARS) c = b2scenes::GearRigs(rw->world, n, seed);
  else if (kind == B2G_SCENE_BULLETS) c = b2scenes::Bullets(rw->world, n, seed, p0 > 0.5f);
  if (counts) { counts[0] = c.bodies; counts[1] = c.fixtures; counts[2] = c.joints; }
  index_world(rw);
  return rw;
}

// Records the reference's listener callbacks (on) or detaches the recorder (off).
void ref_world_events_enable(void* h, int32_t on) {
  RefWorld* rw = (RefWorld*)h;
  rw->recorder.rw = rw;
  rw->recorder.events.clear();
  rw->world->SetContactListener(on ? &rw->recorder : nullptr);
}

// The callbacks recorded since the last call, sorted by (kind, fixture A, fixture B) like the
// engine's batch delivery; returns their number and clears them when `out` holds them all.
int32_t ref_world_events(void* h, b2g_event* out, int32_t cap) {
  RefWorld* rw = (RefWorld*)h;
  std::vector<b2g_event>& ev = rw->recorder.events;
  std::stable_sort(ev.begin(), ev.end(), [](const b2g_event& x, const b2g_event& y) {
    if (x.kind != y.kind) return x.kind < y.kind;
    if (x.fixture_a != y.fixture_a) return x.fixture_a < y.fixture_a;
    return x.fixture_b < y.fixture_b;
  });
  const int32_t n = (int32_t)ev.size();
  if (out && cap >= n) {
    for (int32_t i = 0; i < n; ++i) out[i] = ev[i];
    ev.clear();
  }
  return n;
}

// b2World::Dump of the reference world (writes box2d_dump.inl in the working directory).
void ref_world_dump(void* h) {
  RefWorld* rw = (RefWorld*)h;
  rw->world->Dump();
}

void ref_world_free(void* h) {
  RefWorld* rw = (RefWorld*)h;
  delete rw->world;
  delete rw;
}

void ref_world_set_flags(void* h, int32_t allow_sleep, int32_t warm, int32_t continuous) {
  RefWorld* rw = (RefWorld*)h;
  rw->world->SetAllowSleeping(allow_sleep != 0);
  rw->world->SetWarmStarting(warm != 0);
  rw->world->SetContinuousPhysics(continuous != 0);
}

// Steps the reference world n times; returns the summed wall time in seconds of the Step calls.
double ref_world_step(void* h, float dt, int32_t vi, int32_t pi, int32_t nsteps) {
  RefWorld* rw = (RefWorld*)h;
  b2Timer t;
  for (int i = 0; i < nsteps; ++i) rw->world->Step(dt, vi, pi);
  return t.GetMilliseconds() * 1e-3;
}

int32_t ref_world_sizes(void* h, int32_t* out4) {
  RefWorld* rw = (RefWorld*)h;
  out4[0] = (int32_t)rw->bodies.size();
  out4[1] = (int32_t)rw->fixtures.size();
  out4[2] = (int32_t)rw->joints.size();
  out4[3] = rw->world->GetContactCount();
  return 0;
}

void ref_world_bodies(void* h, b2g_body* out) {
  RefWorld* rw = (RefWorld*)h;
  for (size_t i = 0; i < rw->bodies.size(); ++i) {
    const b2Body* b = rw->bodies[i];
    b2g_body* o = out + i;
    memset(o, 0, sizeof(*o));
    o->xf[0] = b->m_xf.p.x; o->xf[1] = b->m_xf.p.y; o->xf[2] = b->m_xf.q.s; o->xf[3] = b->m_xf.q.c;
    o->c[0] = b->m_sweep.c.x; o->c[1] = b->m_sweep.c.y; o->a = b->m_sweep.a;
    o->v[0] = b->m_linearVelocity.x; o->v[1] = b->m_linearVelocity.y; o->w = b->m_angularVelocity;
    o->local_center[0] = b->m_sweep.localCenter.x; o->local_center[1] = b->m_sweep.localCenter.y;
    o->mass = b->m_mass; o->inv_mass = b->m_invMass; o->inertia = b->m_I; o->inv_inertia = b->m_invI;
    o->linear_damping = b->m_linearDamping; o->angular_damping = b->m_angularDamping;
    o->gravity_scale = b->m_gravityScale;
    o->force[0] = b->m_force.x; o->force[1] = b->m_force.y; o->torque = b->m_torque;
    o->type = (int32_t)b->m_type;
    uint32_t fl = 0;
    if (b->m_flags & b2Body::e_enabledFlag) fl |= B2G_BODY_ENABLED;
    if (b->m_flags & b2Body::e_fixedRotationFlag) fl |= B2G_BODY_FIXED_ROTATION;
    if (b->m_flags & b2Body::e_bulletFlag) fl |= B2G_BODY_BULLET;
    if (b->m_flags & b2Body::e_awakeFlag) fl |= B2G_BODY_AWAKE;
    if (b->m_flags & b2Body::e_autoSleepFlag) fl |= B2G_BODY_AUTO_SLEEP;
    o->flags = fl;
  }
}

void ref_world_fixtures(void* h, b2g_fixture* out) {
  RefWorld* rw = (RefWorld*)h;
  for (size_t i = 0; i < rw->fixtures.size(); ++i) {
    const b2Fixture* f = rw->fixtures[i];
    b2g_fixture* o = out + i;
    memset(o, 0, sizeof(*o));
    shape_from_ref(f->m_shape, &o->shape);
    o->body = rw->body_index[f->m_body];
    o->density = f->m_density; o->friction = f->m_friction; o->restitution = f->m_restitution;
    o->restitution_threshold = f->m_restitutionThreshold;
    o->category_bits = f->m_filter.categoryBits; o->mask_bits = f->m_filter.maskBits;
    o->group_index = f->m_filter.groupIndex; o->is_sensor = f->m_isSensor ? 1 : 0;
  }
}

void ref_world_joints(void* h, b2g_joint* out) {
  RefWorld* rw = (RefWorld*)h;
  for (size_t i = 0; i < rw->joints.size(); ++i) {
    b2Joint* j = rw->joints[i];
    b2g_joint* o = out + i;
    memset(o, 0, sizeof(*o));
    o->def.body_a = rw->body_index[j->m_bodyA];
    o->def.body_b = rw->body_index[j->m_bodyB];
    o->def.collide_connected = j->m_collideConnected ? 1 : 0;
    if (j->m_type == e_revoluteJoint) {
      b2RevoluteJoint* r = (b2RevoluteJoint*)j;
      o->def.type = B2G_JOINT_REVOLUTE;
      o->def.local_anchor_a[0] = r->m_localAnchorA.x; o->def.local_anchor_a[1] = r->m_localAnchorA.y;
      o->def.local_anchor_b[0] = r->m_localAnchorB.x; o->def.local_anchor_b[1] = r->m_localAnchorB.y;
      o->def.reference_angle = r->m_referenceAngle;
      o->def.enable_limit = r->m_enableLimit; o->def.lower = r->m_lowerAngle; o->def.upper = r->m_upperAngle;
      o->def.enable_motor = r->m_enableMotor; o->def.max_motor = r->m_maxMotorTorque;
      o->def.motor_speed = r->m_motorSpeed;
      o->impulse[0] = r->m_impulse.x; o->impulse[1] = r->m_impulse.y;
      o->motor_impulse = r->m_motorImpulse; o->lower_impulse = r->m_lowerImpulse;
      o->upper_impulse = r->m_upperImpulse;
    } else if (j->m_type == e_prismaticJoint) {
      b2PrismaticJoint* p = (b2PrismaticJoint*)j;
      o->def.type = B2G_JOINT_PRISMATIC;
      o->def.local_anchor_a[0] = p->m_localAnchorA.x; o->def.local_anchor_a[1] = p->m_localAnchorA.y;
      o->def.local_anchor_b[0] = p->m_localAnchorB.x; o->def.local_anchor_b[1] = p->m_localAnchorB.y;
      o->def.local_axis_a[0] = p->m_localXAxisA.x; o->def.local_axis_a[1] = p->m_localXAxisA.y;
      o->def.reference_angle = p->m_referenceAngle;
      o->def.enable_limit = p->m_enableLimit; o->def.lower = p->m_lowerTranslation;
      o->def.upper = p->m_upperTranslation; o->def.enable_motor = p->m_enableMotor;
      o->def.max_motor = p->m_maxMotorForce; o->def.motor_speed = p->m_motorSpeed;
      o->impulse[0] = p->m_impulse.x; o->impulse[1] = p->m_impulse.y;
      o->motor_impulse = p->m_motorImpulse; o->lower_impulse = p->m_lowerImpulse;
      o->upper_impulse = p->m_upperImpulse;
    } else if (j->m_type == e_distanceJoint) {
      b2DistanceJoint* d = (b2DistanceJoint*)j;
      o->def.type = B2G_JOINT_DISTANCE;
      o->def.local_anchor_a[0] = d->m_localAnchorA.x; o->def.local_anchor_a[1] = d->m_localAnchorA.y;
      o->def.local_anchor_b[0] = d->m_localAnchorB.x; o->def.local_anchor_b[1] = d->m_localAnchorB.y;
      o->def.length = d->m_length; o->def.min_length = d->m_minLength; o->def.max_length = d->m_maxLength;
      o->def.stiffness = d->m_stiffness; o->def.damping = d->m_damping;
      o->impulse[0] = d->m_impulse;
      o->lower_impulse = d->m_lowerImpulse; o->upper_impulse = d->m_upperImpulse;
    } else if (j->m_type == e_weldJoint) {
      b2WeldJoint* q = (b2WeldJoint*)j;
      o->def.type = B2G_JOINT_WELD;
      o->def.local_anchor_a[0] = q->m_localAnchorA.x; o->def.local_anchor_a[1] = q->m_localAnchorA.y;
      o->def.local_anchor_b[0] = q->m_localAnchorB.x; o->def.local_anchor_b[1] = q->m_localAnchorB.y;
      o->def.reference_angle = q->m_referenceAngle;
      o->def.stiffness = q->m_stiffness; o->def.damping = q->m_damping;
      o->impulse[0] = q->m_impulse.x; o->impulse[1] = q->m_impulse.y; o->impulse[2] = q->m_impulse.z;
    } else if (j->m_type == e_wheelJoint) {
      b2WheelJoint* q = (b2WheelJoint*)j;
      o->def.type = B2G_JOINT_WHEEL;
      o->def.local_anchor_a[0] = q->m_localAnchorA.x; o->def.local_anchor_a[1] = q->m_localAnchorA.y;
      o->def.local_anchor_b[0] = q->m_localAnchorB.x; o->def.local_anchor_b[1] = q->m_localAnchorB.y;
      o->def.local_axis_a[0] = q->m_localXAxisA.x; o->def.local_axis_a[1] = q->m_localXAxisA.y;
      o->def.enable_limit = q->m_enableLimit; o->def.lower = q->m_lowerTranslation;
      o->def.upper = q->m_upperTranslation; o->def.enable_motor = q->m_enableMotor;
      o->def.max_motor = q->m_maxMotorTorque; o->def.motor_speed = q->m_motorSpeed;
      o->def.stiffness = q->m_stiffness; o->def.damping = q->m_damping;
      o->impulse[0] = q->m_impulse; o->impulse[1] = q->m_springImpulse;
      o->motor_impulse = q->m_motorImpulse; o->lower_impulse = q->m_lowerImpulse;
      o->upper_impulse = q->m_upperImpulse;
    } else if (j->m_type == e_motorJoint) {
      b2MotorJoint* q = (b2MotorJoint*)j;
      o->def.type = B2G_JOINT_MOTOR;
      o->def.linear_offset[0] = q->m_linearOffset.x; o->def.linear_offset[1] = q->m_linearOffset.y;
      o->def.reference_angle = q->m_angularOffset;
      o->def.max_force = q->m_maxForce; o->def.max_torque = q->m_maxTorque;
      o->def.correction_factor = q->m_correctionFactor;
      o->impulse[0] = q->m_linearImpulse.x; o->impulse[1] = q->m_linearImpulse.y;
      o->impulse[2] = q->m_angularImpulse;
    } else if (j->m_type == e_frictionJoint) {
      b2FrictionJoint* q = (b2FrictionJoint*)j;
      o->def.type = B2G_JOINT_FRICTION;
      o->def.local_anchor_a[0] = q->m_localAnchorA.x; o->def.local_anchor_a[1] = q->m_localAnchorA.y;
      o->def.local_anchor_b[0] = q->m_localAnchorB.x; o->def.local_anchor_b[1] = q->m_localAnchorB.y;
      o->def.max_force = q->m_maxForce; o->def.max_torque = q->m_maxTorque;
      o->impulse[0] = q->m_linearImpulse.x; o->impulse[1] = q->m_linearImpulse.y;
      o->impulse[2] = q->m_angularImpulse;
    } else if (j->m_type == e_mouseJoint) {
      b2MouseJoint* q = (b2MouseJoint*)j;
      o->def.type = B2G_JOINT_MOUSE;
      o->def.target[0] = q->m_targetA.x; o->def.target[1] = q->m_targetA.y;
      o->def.local_anchor_b[0] = q->m_localAnchorB.x; o->def.local_anchor_b[1] = q->m_localAnchorB.y;
      o->def.max_force = q->m_maxForce; o->def.stiffness = q->m_stiffness; o->def.damping = q->m_damping;
      o->impulse[0] = q->m_impulse.x; o->impulse[1] = q->m_impulse.y;
    } else if (j->m_type == e_pulleyJoint) {
      b2PulleyJoint* q = (b2PulleyJoint*)j;
      o->def.type = B2G_JOINT_PULLEY;
      o->def.ground_anchor_a[0] = q->m_groundAnchorA.x; o->def.ground_anchor_a[1] = q->m_groundAnchorA.y;
      o->def.ground_anchor_b[0] = q->m_groundAnchorB.x; o->def.ground_anchor_b[1] = q->m_groundAnchorB.y;
      o->def.local_anchor_a[0] = q->m_localAnchorA.x; o->def.local_anchor_a[1] = q->m_localAnchorA.y;
      o->def.local_anchor_b[0] = q->m_localAnchorB.x; o->def.local_anchor_b[1] = q->m_localAnchorB.y;
      o->def.length_a = q->m_lengthA; o->def.length_b = q->m_lengthB; o->def.ratio = q->m_ratio;
      o->impulse[0] = q->m_impulse;
    } else if (j->m_type == e_gearJoint) {
      b2GearJoint* q = (b2GearJoint*)j;
      o->def.type = B2G_JOINT_GEAR;
      o->def.local_anchor_a[0] = q->m_localAnchorA.x; o->def.local_anchor_a[1] = q->m_localAnchorA.y;
      o->def.local_anchor_b[0] = q->m_localAnchorB.x; o->def.local_anchor_b[1] = q->m_localAnchorB.y;
      o->def.joint_1 = rw->joint_index[q->m_joint1];
      o->def.joint_2 = rw->joint_index[q->m_joint2];
      o->def.ratio = q->m_ratio;
      o->def.gear_constant = q->m_constant;
      o->impulse[0] = q->m_impulse;
    }
    b2Vec2 F = j->GetReactionForce(1.0f);
    o->reaction_impulse[0] = F.x; o->reaction_impulse[1] = F.y;
    o->reaction_angular_impulse = j->GetReactionTorque(1.0f);
  }
}

// Contacts of the world list (order of the reference list), with fixture creation indices.
int32_t ref_world_contacts(void* h, b2g_contact* out, int32_t cap) {
  RefWorld* rw = (RefWorld*)h;
  int32_t n = 0;
  for (b2Contact* c = rw->world->GetContactListStart(); c != rw->world->GetContactListEnd(); c = c->GetNext()) {
    if (n < cap) {
      b2g_contact* o = out + n;
      memset(o, 0, sizeof(*o));
      o->fixture_a = rw->fixture_index[c->m_fixtureA];
      o->fixture_b = rw->fixture_index[c->m_fixtureB];
      uint32_t fl = 0;
      if (c->m_flags & b2Contact::e_touchingFlag) fl |= B2G_CONTACT_TOUCHING;
      if (c->m_flags & b2Contact::e_enabledFlag) fl |= B2G_CONTACT_ENABLED;
      o->flags = fl;
      o->friction = c->m_friction; o->restitution = c->m_restitution;
      o->restitution_threshold = c->m_restitutionThreshold; o->tangent_speed = c->m_tangentSpeed;
      manifold_out(c->m_manifold, &o->manifold);
    }
    ++n;
  }
  return n;
}

// Overwrites body kinematic state (xf, sweep c/a, velocities) from records in creation order.
void ref_world_set_bodies(void* h, const b2g_body* in) {
  RefWorld* rw = (RefWorld*)h;
  for (size_t i = 0; i < rw->bodies.size(); ++i) {
    b2Body* b = rw->bodies[i];
    const b2g_body* o = in + i;
    b->m_xf.p.Set(o->xf[0], o->xf[1]); b->m_xf.q.s = o->xf[2]; b->m_xf.q.c = o->xf[3];
    b->m_sweep.c.Set(o->c[0], o->c[1]); b->m_sweep.a = o->a;
    b->m_sweep.c0 = b->m_sweep.c; b->m_sweep.a0 = b->m_sweep.a;
    b->m_linearVelocity.Set(o->v[0], o->v[1]); b->m_angularVelocity = o->w;
  }
}

// One b2World::Step in which the solve phase is a single b2Island holding every enabled body,
// the solver contacts in the order given by (fixture_a, fixture_b) pairs, and the joints in the
// given creation-index order; the rest follows b2World::Step (src/dynamics/b2_world.cpp:1108-1171)
// and b2World::Solve (:492-670) with sleeping off. Contacts not listed are not solved.
// b2World::RayCast with a closest-hit callback (ties keep the lower fixture index); returns the
// fixture index or -1, out5 = point, normal, fraction.
struct RefClosestHit : public b2RayCastCallback {
  RefWorld* rw;
  int best = -1;
  b2Vec2 point, normal;
  float fraction = 1.0f;
  float ReportFixture(b2Fixture* fixture, const b2Vec2& p, const b2Vec2& n, float f) override {
    int idx = rw->fixture_index[fixture];
    if (best < 0 || f < fraction || (f == fraction && idx < best)) {
      best = idx;
      point = p;
      normal = n;
      fraction = f;
    }
    return f;
  }
};

int32_t ref_world_raycast(void* h, const float* ray4, float* out5) {
  RefWorld* rw = (RefWorld*)h;
  RefClosestHit cb;
  cb.rw = rw;
  rw->world->RayCast(&cb, b2Vec2(ray4[0], ray4[1]), b2Vec2(ray4[2], ray4[3]));
  if (cb.best < 0) return -1;
  out5[0] = cb.point.x; out5[1] = cb.point.y; out5[2] = cb.normal.x; out5[3] = cb.normal.y; out5[4] = cb.fraction;
  return cb.best;
}

// b2World::QueryAABB: the reported fixtures, ascending; returns their number.
struct RefQuery : public b2QueryCallback {
  RefWorld* rw;
  std::vector<int32_t> found;
  bool ReportFixture(b2Fixture* fixture) override {
    found.push_back(rw->fixture_index[fixture]);
    return true;
  }
};

int32_t ref_world_query_aabb(void* h, const float* box4, int32_t* out, int32_t cap) {
  RefWorld* rw = (RefWorld*)h;
  RefQuery cb;
  cb.rw = rw;
  b2AABB box;
  box.lowerBound = b2Vec2(box4[0], box4[1]);
  box.upperBound = b2Vec2(box4[2], box4[3]);
  rw->world->QueryAABB(&cb, box);
  std::sort(cb.found.begin(), cb.found.end());
  for (size_t i = 0; i < cb.found.size() && (int32_t)i < cap; ++i) out[i] = cb.found[i];
  return (int32_t)cb.found.size();
}

int ref_replay_step(void* h, float dt, int32_t vi, int32_t pi, const int32_t* contact_pairs,
                    int32_t nc, const int32_t* joint_order, int32_t nj) {
  RefWorld* rw = (RefWorld*)h;
  b2World* w = rw->world;
  w->m_locked = true;
  if (w->m_newContacts) w->m_contactManager.FindNewContacts();
  if (w->m_newContacts || w->m_removedBodies) {
    w->RemoveDeadContacts();
    w->m_newContacts = false;
    w->m_removedBodies = false;
  }
  b2TimeStep step;
  step.dt = dt;
  step.inv_dt = (dt > 0.0f) ? 1.0f / dt : 0.0f;
  step.velocityIterations = vi;
  step.positionIterations = pi;
  step.particleIterations = 0;
  step.dtRatio = w->m_inv_dt0 * dt;
  step.warmStarting = w->m_warmStarting;
  w->m_contactManager.Collide();
  if (dt > 0.0f) {
    std::map<std::pair<int, int>, b2Contact*> byPair;
    for (b2Contact* c = w->GetContactListStart(); c != w->GetContactListEnd(); c = c->GetNext())
      byPair[{rw->fixture_index[c->m_fixtureA], rw->fixture_index[c->m_fixtureB]}] = c;
    b2Island island((int32)rw->bodies.size(), nc, nj, &w->m_stackAllocator,
                    w->m_contactManager.m_contactListener);
    for (b2Body* b : rw->bodies) {
      b->m_xf0 = b->m_xf;
      b->m_sweep.c0 = b->m_sweep.c;
      b->m_sweep.a0 = b->m_sweep.a;
      if (b->IsEnabled()) island.Add(b);
    }
    for (int i = 0; i < nc; ++i) {
      auto it = byPair.find({contact_pairs[2 * i], contact_pairs[2 * i + 1]});
      if (it == byPair.end()) return 1;
      island.Add(it->second);
    }
    for (int i = 0; i < nj; ++i) island.Add(rw->joints[joint_order[i]]);
    island.Solve(step, w->m_gravity, false);
    w->m_contactManager.FindNewContacts();
    w->RemoveDeadContacts();
    if (w->m_continuousPhysics) w->SolveTOI(step);  // b2World::Step, src/dynamics/b2_world.cpp:1152-1156
    w->m_inv_dt0 = step.inv_dt;
  }
  if (w->m_clearForces) w->ClearForces();
  w->m_locked = false;
  return 0;
}

// The bodies' sleep timers (b2Body::m_sleepTime), creation order.
void ref_world_sleep_times(void* h, float* out) {
  RefWorld* rw = (RefWorld*)h;
  for (size_t i = 0; i < rw->bodies.size(); ++i) out[i] = rw->bodies[i]->m_sleepTime;
}

// One Step with b2World::Solve's island loop (src/dynamics/b2_world.cpp:492-670) replayed over
// caller-given islands: the reference's own narrowphase (b2ContactManager::Collide, with its
// sleep rules), then per island either b2Island::SolveOrphan (orphan islands, then flagged awake
// as b2World::Solve does) or a b2Island holding the island's bodies (marked awake without a timer
// reset), the static bodies its contacts and joints touch, its contacts and its joints in the
// given order, solved with the world's sleep setting; then the reference's broadphase and dead
// contact removal. Contacts are given as (fixture A, fixture B) pairs. Returns 1 when a listed
// contact does not exist.
int ref_replay_step_islands(void* h, float dt, int32_t vi, int32_t pi, int32_t n_islands, const int32_t* orphan,
                            const int32_t* body_off, const int32_t* contact_off, const int32_t* joint_off,
                            const int32_t* bodies, const int32_t* contact_pairs, const int32_t* joints) {
  RefWorld* rw = (RefWorld*)h;
  b2World* w = rw->world;
  w->m_locked = true;
  if (w->m_newContacts) w->m_contactManager.FindNewContacts();
  if (w->m_newContacts || w->m_removedBodies) {
    w->RemoveDeadContacts();
    w->m_newContacts = false;
    w->m_removedBodies = false;
  }
  b2TimeStep step;
  step.dt = dt;
  step.inv_dt = (dt > 0.0f) ? 1.0f / dt : 0.0f;
  step.velocityIterations = vi;
  step.positionIterations = pi;
  step.particleIterations = 0;
  step.dtRatio = w->m_inv_dt0 * dt;
  step.warmStarting = w->m_warmStarting;
  w->m_contactManager.Collide();
  if (dt > 0.0f) {
    std::map<std::pair<int, int>, b2Contact*> byPair;
    for (b2Contact* c = w->GetContactListStart(); c != w->GetContactListEnd(); c = c->GetNext())
      byPair[{rw->fixture_index[c->m_fixtureA], rw->fixture_index[c->m_fixtureB]}] = c;
    for (b2Body* b : rw->bodies) {
      b->m_xf0 = b->m_xf;
      b->m_sweep.c0 = b->m_sweep.c;
      b->m_sweep.a0 = b->m_sweep.a;
    }
    int maxc = 0, maxj = 0;
    for (int k = 0; k < n_islands; ++k) {
      maxc = std::max(maxc, contact_off[k + 1] - contact_off[k]);
      maxj = std::max(maxj, joint_off[k + 1] - joint_off[k]);
    }
    b2Island island((int32)rw->bodies.size(), std::max(maxc, 1), std::max(maxj, 1), &w->m_stackAllocator,
                    w->m_contactManager.m_contactListener);
    for (int k = 0; k < n_islands; ++k) {
      if (orphan[k]) {
        b2Body* b = rw->bodies[bodies[body_off[k]]];
        island.SolveOrphan(b, step, w->m_gravity, w->m_allowSleep);
        b->m_flags |= (b2Body::e_islandFlag | b2Body::e_awakeFlag);
        continue;
      }
      island.Clear();
      std::vector<b2Body*> statics;
      auto note_static = [&](b2Body* b) {
        if (b->GetType() == b2_staticBody && std::find(statics.begin(), statics.end(), b) == statics.end())
          statics.push_back(b);
      };
      std::vector<b2Contact*> cs;
      for (int i = contact_off[k]; i < contact_off[k + 1]; ++i) {
        auto it = byPair.find({contact_pairs[2 * i], contact_pairs[2 * i + 1]});
        if (it == byPair.end()) {
          w->m_locked = false;
          return 1;
        }
        cs.push_back(it->second);
        note_static(it->second->m_fixtureA->m_body);
        note_static(it->second->m_fixtureB->m_body);
      }
      for (int i = joint_off[k]; i < joint_off[k + 1]; ++i) {
        note_static(rw->joints[joints[i]]->m_bodyA);
        note_static(rw->joints[joints[i]]->m_bodyB);
      }
      for (int i = body_off[k]; i < body_off[k + 1]; ++i) {
        b2Body* b = rw->bodies[bodies[i]];
        b->m_flags |= b2Body::e_awakeFlag;
        island.Add(b);
      }
      for (b2Body* b : statics) island.Add(b);
      for (b2Contact* c : cs) island.Add(c);
      for (int i = joint_off[k]; i < joint_off[k + 1]; ++i) island.Add(rw->joints[joints[i]]);
      island.Solve(step, w->m_gravity, w->m_allowSleep);
    }
    w->m_contactManager.FindNewContacts();
    w->RemoveDeadContacts();
    w->m_inv_dt0 = step.inv_dt;
  }
  if (w->m_clearForces) w->ClearForces();
  w->m_locked = false;
  return 0;
}

// Runs `ref_world_step`-style stepping of a list of worlds on `threads` host threads (each thread
// steps a disjoint subset); returns wall seconds. Used as the multi-core CPU baseline.
double ref_worlds_step_parallel(void** hs, int32_t n, float dt, int32_t vi, int32_t pi,
                                int32_t nsteps, int32_t threads);

}  // extern "C"

#include <thread>
#include <chrono>
extern "C" double ref_worlds_step_parallel(void** hs, int32_t n, float dt, int32_t vi, int32_t pi,
                                           int32_t nsteps, int32_t threads) {
  auto t0 = std::chrono::steady_clock::now();
  std::vector<std::thread> th;
  for (int t = 0; t < threads; ++t) {
    th.emplace_back([=]() {
      for (int i = t; i < n; i += threads) {
        RefWorld* rw = (RefWorld*)hs[i];
        for (int s = 0; s < nsteps; ++s) rw->world->Step(dt, vi, pi);
      }
    });
  }
  for (auto& x : th) x.join();
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}
