// facade.cpp - the b2World / b2Body / b2Fixture / b2Joint / b2Contact facade over the C ABI,
// and the scene builder entry point (b2g_scene_build) that runs the shared scene recipes
// through it.
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <stdexcept>
#include <typeinfo>

#include "../include/box2d/box2d.h"
#include "../scenes/scenes_joints.h"
#include "engine.h"

const b2Vec2 b2Vec2_zero(0.0f, 0.0f);

// ---------------------------------------------------------------- shapes
void b2CircleShape::ComputeAABB(b2AABB* aabb, const b2Transform& xf) const {
  b2Vec2 p = xf.p + b2Mul(xf.q, m_p);
  aabb->lowerBound.Set(p.x - m_radius, p.y - m_radius);
  aabb->upperBound.Set(p.x + m_radius, p.y + m_radius);
}
void b2CircleShape::ComputeMass(b2MassData* md, float density) const {
  b2g_shape s;
  ToRecord(&s);
  b2g::shape_mass(s, density, &md->mass, &md->center.x, &md->center.y, &md->I);
}
void b2CircleShape::ToRecord(b2g_shape* out) const {
  memset(out, 0, sizeof(*out));
  out->type = B2G_SHAPE_CIRCLE;
  out->radius = m_radius;
  out->vertices[0][0] = m_p.x;
  out->vertices[0][1] = m_p.y;
}

void b2EdgeShape::ComputeAABB(b2AABB* aabb, const b2Transform& xf) const {
  b2Vec2 v1 = b2Mul(xf, m_vertex1);
  b2Vec2 v2 = b2Mul(xf, m_vertex2);
  b2Vec2 r(m_radius, m_radius);
  aabb->lowerBound = b2Min(v1, v2) - r;
  aabb->upperBound = b2Max(v1, v2) + r;
}
void b2EdgeShape::ComputeMass(b2MassData* md, float density) const {
  B2_NOT_USED(density);
  md->mass = 0.0f;
  md->center = 0.5f * (m_vertex1 + m_vertex2);
  md->I = 0.0f;
}
void b2EdgeShape::ToRecord(b2g_shape* out) const {
  memset(out, 0, sizeof(*out));
  out->type = B2G_SHAPE_EDGE;
  out->radius = m_radius;
  out->vertices[0][0] = m_vertex1.x; out->vertices[0][1] = m_vertex1.y;
  out->vertices[1][0] = m_vertex2.x; out->vertices[1][1] = m_vertex2.y;
  out->vertices[2][0] = m_vertex0.x; out->vertices[2][1] = m_vertex0.y;
  out->vertices[3][0] = m_vertex3.x; out->vertices[3][1] = m_vertex3.y;
  out->one_sided = m_oneSided ? 1 : 0;
}

static void polygon_from_record(b2PolygonShape* p, const b2g_shape& s) {
  p->m_count = s.count;
  p->m_radius = s.radius;
  for (int i = 0; i < s.count; ++i) {
    p->m_vertices[i].Set(s.vertices[i][0], s.vertices[i][1]);
    p->m_normals[i].Set(s.normals[i][0], s.normals[i][1]);
  }
  p->m_centroid.Set(s.centroid[0], s.centroid[1]);
}

void b2PolygonShape::Set(const b2Vec2* points, int32 count) {
  float xy[2 * b2_maxPolygonVertices];
  int n = count < b2_maxPolygonVertices ? count : b2_maxPolygonVertices;
  for (int i = 0; i < n; ++i) { xy[2 * i] = points[i].x; xy[2 * i + 1] = points[i].y; }
  b2g_shape s;
  b2g::polygon_set(&s, xy, count);
  polygon_from_record(this, s);
}
void b2PolygonShape::SetAsBox(float hx, float hy) {
  b2g_shape s;
  b2g::polygon_box(&s, hx, hy, false, 0.0f, 0.0f, 0.0f);
  polygon_from_record(this, s);
}
void b2PolygonShape::SetAsBox(float hx, float hy, const b2Vec2& center, float angle) {
  b2g_shape s;
  b2g::polygon_box(&s, hx, hy, true, center.x, center.y, angle);
  polygon_from_record(this, s);
}
void b2PolygonShape::ComputeAABB(b2AABB* aabb, const b2Transform& xf) const {
  b2Vec2 lower = b2Mul(xf, m_vertices[0]);
  b2Vec2 upper = lower;
  for (int32 i = 1; i < m_count; ++i) {
    b2Vec2 v = b2Mul(xf, m_vertices[i]);
    lower = b2Min(lower, v);
    upper = b2Max(upper, v);
  }
  b2Vec2 r(m_radius, m_radius);
  aabb->lowerBound = lower - r;
  aabb->upperBound = upper + r;
}
void b2PolygonShape::ComputeMass(b2MassData* md, float density) const {
  b2g_shape s;
  ToRecord(&s);
  b2g::shape_mass(s, density, &md->mass, &md->center.x, &md->center.y, &md->I);
}
void b2PolygonShape::ToRecord(b2g_shape* out) const {
  memset(out, 0, sizeof(*out));
  out->type = B2G_SHAPE_POLYGON;
  out->radius = m_radius;
  out->count = m_count;
  for (int i = 0; i < m_count; ++i) {
    out->vertices[i][0] = m_vertices[i].x; out->vertices[i][1] = m_vertices[i].y;
    out->normals[i][0] = m_normals[i].x; out->normals[i][1] = m_normals[i].y;
  }
  out->centroid[0] = m_centroid.x;
  out->centroid[1] = m_centroid.y;
}

// b2WorldManifold::Initialize (src/collision/b2_collision.cpp:26-90), host evaluation.
void b2WorldManifold::Initialize(const b2Manifold* manifold, const b2Transform& xfA, float radiusA,
                                 const b2Transform& xfB, float radiusB) {
  if (manifold->pointCount == 0) return;
  switch (manifold->type) {
    case b2Manifold::e_circles: {
      normal.Set(1.0f, 0.0f);
      b2Vec2 pointA = b2Mul(xfA, manifold->localPoint);
      b2Vec2 pointB = b2Mul(xfB, manifold->points[0].localPoint);
      if (b2DistanceSquared(pointA, pointB) > b2_epsilon * b2_epsilon) {
        normal = pointB - pointA;
        normal.Normalize();
      }
      b2Vec2 cA = pointA + radiusA * normal;
      b2Vec2 cB = pointB - radiusB * normal;
      points[0] = 0.5f * (cA + cB);
      separations[0] = b2Dot(cB - cA, normal);
    } break;
    case b2Manifold::e_faceA: {
      normal = b2Mul(xfA.q, manifold->localNormal);
      b2Vec2 planePoint = b2Mul(xfA, manifold->localPoint);
      for (int32 i = 0; i < manifold->pointCount; ++i) {
        b2Vec2 clipPoint = b2Mul(xfB, manifold->points[i].localPoint);
        b2Vec2 cA = clipPoint + (radiusA - b2Dot(clipPoint - planePoint, normal)) * normal;
        b2Vec2 cB = clipPoint - radiusB * normal;
        points[i] = 0.5f * (cA + cB);
        separations[i] = b2Dot(cB - cA, normal);
      }
    } break;
    case b2Manifold::e_faceB: {
      normal = b2Mul(xfB.q, manifold->localNormal);
      b2Vec2 planePoint = b2Mul(xfB, manifold->localPoint);
      for (int32 i = 0; i < manifold->pointCount; ++i) {
        b2Vec2 clipPoint = b2Mul(xfA, manifold->points[i].localPoint);
        b2Vec2 cB = clipPoint + (radiusB - b2Dot(clipPoint - planePoint, normal)) * normal;
        b2Vec2 cA = clipPoint - radiusA * normal;
        points[i] = 0.5f * (cA + cB);
        separations[i] = b2Dot(cA - cB, normal);
      }
      normal = -normal;
    } break;
  }
}

bool b2ContactFilter::ShouldCollide(b2Fixture* fixtureA, b2Fixture* fixtureB) {
  const b2Filter& a = fixtureA->GetFilterData();
  const b2Filter& b = fixtureB->GetFilterData();
  if (a.groupIndex == b.groupIndex && a.groupIndex != 0) return a.groupIndex > 0;
  return (a.maskBits & b.categoryBits) != 0 && (a.categoryBits & b.maskBits) != 0;
}

// ---------------------------------------------------------------- fixtures
b2Shape* b2Fixture::GetShape() { return m_shape.get(); }
const b2Shape* b2Fixture::GetShape() const { return m_shape.get(); }
void b2Fixture::GetMassData(b2MassData* massData) const { m_shape->ComputeMass(massData, m_density); }

// ---------------------------------------------------------------- bodies
static b2g_fixture_def fixture_def_record(const b2FixtureDef* def, int body) {
  b2g_fixture_def d;
  memset(&d, 0, sizeof(d));
  d.body = body;
  const b2Shape* s = def->shape;
  d.shape_type = s->GetType();
  if (s->GetType() == b2Shape::e_polygon) {
    d.poly_mode = B2G_POLY_RAW;
    s->ToRecord(&d.shape);
  } else if (s->GetType() == b2Shape::e_circle) {
    const b2CircleShape* c = (const b2CircleShape*)s;
    d.radius = c->m_radius;
    d.center[0] = c->m_p.x;
    d.center[1] = c->m_p.y;
  } else {
    b2g_shape r;
    s->ToRecord(&r);
    for (int i = 0; i < 4; ++i) { d.verts[i][0] = r.vertices[i][0]; d.verts[i][1] = r.vertices[i][1]; }
    d.one_sided = r.one_sided;
  }
  d.friction = def->friction;
  d.restitution = def->restitution;
  d.restitution_threshold = def->restitutionThreshold;
  d.density = def->density;
  d.is_sensor = def->isSensor ? 1 : 0;
  d.category_bits = def->filter.categoryBits;
  d.mask_bits = def->filter.maskBits;
  d.group_index = def->filter.groupIndex;
  d.user_data = def->userData.pointer;
  return d;
}

static b2Shape* clone_shape(const b2Shape* s) {
  if (s->GetType() == b2Shape::e_circle) return new b2CircleShape(*(const b2CircleShape*)s);
  if (s->GetType() == b2Shape::e_edge) return new b2EdgeShape(*(const b2EdgeShape*)s);
  return new b2PolygonShape(*(const b2PolygonShape*)s);
}

b2Fixture* b2Body::CreateFixture(const b2FixtureDef* def) {
  if (!def || !def->shape) return nullptr;
  b2g_fixture_def d = fixture_def_record(def, m_index);
  int32_t id = -1;
  int st = b2g_fixtures_add(m_world->m_batch, m_world->m_index, &d, 1, &id);
  if (st != B2G_OK) return nullptr;
  m_world->m_fixtures.emplace_back();
  b2Fixture* f = &m_world->m_fixtures.back();
  f->m_body = this;
  f->m_index = id;
  f->m_shapeType = def->shape->GetType();
  f->m_shape.reset(clone_shape(def->shape));
  f->m_density = def->density;
  f->m_friction = def->friction;
  f->m_restitution = def->restitution;
  f->m_restitutionThreshold = def->restitutionThreshold;
  f->m_isSensor = def->isSensor;
  f->m_filter = def->filter;
  f->m_userData = def->userData;
  f->m_next = m_fixtureList;
  m_fixtureList = f;
  m_world->m_fixtureIndex.push_back(f);
  m_world->InvalidateCaches();
  return f;
}

b2Fixture* b2Body::CreateFixture(const b2Shape* shape, float density) {
  b2FixtureDef def;
  def.shape = shape;
  def.density = density;
  return CreateFixture(&def);
}

void b2Body::Sync() const {
  if (m_seen == m_world->StateVersion()) return;
  const b2g_body& r = m_world->BodyRecord(m_index);
  m_xf.p.Set(r.xf[0], r.xf[1]);
  m_xf.q.s = r.xf[2];
  m_xf.q.c = r.xf[3];
  m_c.Set(r.c[0], r.c[1]);
  m_a = r.a;
  m_lc.Set(r.local_center[0], r.local_center[1]);
  m_v.Set(r.v[0], r.v[1]);
  m_w = r.w;
  m_seen = m_world->StateVersion();
}

const b2Transform& b2Body::GetTransform() const { Sync(); return m_xf; }
float b2Body::GetAngle() const { Sync(); return m_a; }
const b2Vec2& b2Body::GetWorldCenter() const { Sync(); return m_c; }
const b2Vec2& b2Body::GetLocalCenter() const { Sync(); return m_lc; }
const b2Vec2& b2Body::GetLinearVelocity() const { Sync(); return m_v; }
float b2Body::GetAngularVelocity() const { Sync(); return m_w; }
float b2Body::GetMass() const { return m_world->BodyRecord(m_index).mass; }
float b2Body::GetInertia() const {
  const b2g_body& r = m_world->BodyRecord(m_index);
  return r.inertia + r.mass * (r.local_center[0] * r.local_center[0] + r.local_center[1] * r.local_center[1]);
}
void b2Body::GetMassData(b2MassData* data) const {
  data->mass = GetMass();
  data->I = GetInertia();
  data->center = GetLocalCenter();
}

// b2Body::SetTransform (src/dynamics/b2_body.cpp:482-504)
void b2Body::SetTransform(const b2Vec2& position, float angle) {
  b2g_body r = m_world->BodyRecord(m_index);
  b2Transform xf;
  xf.q.Set(angle);
  xf.p = position;
  b2Vec2 c = b2Mul(xf, b2Vec2(r.local_center[0], r.local_center[1]));
  r.xf[0] = xf.p.x; r.xf[1] = xf.p.y; r.xf[2] = xf.q.s; r.xf[3] = xf.q.c;
  r.c[0] = c.x; r.c[1] = c.y;
  r.a = angle;
  m_world->WriteBody(m_index, r);
}
void b2Body::SetLinearVelocity(const b2Vec2& v) {
  if (m_type == b2_staticBody) return;
  b2g_body r = m_world->BodyRecord(m_index);
  r.v[0] = v.x; r.v[1] = v.y;
  m_world->WriteBody(m_index, r);
}
void b2Body::SetAngularVelocity(float w) {
  if (m_type == b2_staticBody) return;
  b2g_body r = m_world->BodyRecord(m_index);
  r.w = w;
  m_world->WriteBody(m_index, r);
}
// b2Body::ApplyForce and friends (include/box2d/b2_body.h:750-860)
void b2Body::ApplyForce(const b2Vec2& force, const b2Vec2& point, bool wake) {
  B2_NOT_USED(wake);
  if (m_type != b2_dynamicBody) return;
  b2g_body r = m_world->BodyRecord(m_index);
  r.force[0] += force.x; r.force[1] += force.y;
  r.torque += b2Cross(point - b2Vec2(r.c[0], r.c[1]), force);
  m_world->WriteBody(m_index, r);
}
void b2Body::ApplyForceToCenter(const b2Vec2& force, bool wake) {
  B2_NOT_USED(wake);
  if (m_type != b2_dynamicBody) return;
  b2g_body r = m_world->BodyRecord(m_index);
  r.force[0] += force.x; r.force[1] += force.y;
  m_world->WriteBody(m_index, r);
}
void b2Body::ApplyTorque(float torque, bool wake) {
  B2_NOT_USED(wake);
  if (m_type != b2_dynamicBody) return;
  b2g_body r = m_world->BodyRecord(m_index);
  r.torque += torque;
  m_world->WriteBody(m_index, r);
}
void b2Body::ApplyLinearImpulse(const b2Vec2& impulse, const b2Vec2& point, bool wake) {
  B2_NOT_USED(wake);
  if (m_type != b2_dynamicBody) return;
  b2g_body r = m_world->BodyRecord(m_index);
  r.v[0] += r.inv_mass * impulse.x;
  r.v[1] += r.inv_mass * impulse.y;
  r.w += r.inv_inertia * b2Cross(point - b2Vec2(r.c[0], r.c[1]), impulse);
  m_world->WriteBody(m_index, r);
}
void b2Body::ApplyLinearImpulseToCenter(const b2Vec2& impulse, bool wake) {
  B2_NOT_USED(wake);
  if (m_type != b2_dynamicBody) return;
  b2g_body r = m_world->BodyRecord(m_index);
  r.v[0] += r.inv_mass * impulse.x;
  r.v[1] += r.inv_mass * impulse.y;
  m_world->WriteBody(m_index, r);
}
void b2Body::ApplyAngularImpulse(float impulse, bool wake) {
  B2_NOT_USED(wake);
  if (m_type != b2_dynamicBody) return;
  b2g_body r = m_world->BodyRecord(m_index);
  r.w += r.inv_inertia * impulse;
  m_world->WriteBody(m_index, r);
}

// ---------------------------------------------------------------- joint defs
void b2RevoluteJointDef::Initialize(b2Body* bA, b2Body* bB, const b2Vec2& anchor) {
  bodyA = bA;
  bodyB = bB;
  localAnchorA = bodyA->GetLocalPoint(anchor);
  localAnchorB = bodyB->GetLocalPoint(anchor);
  referenceAngle = bodyB->GetAngle() - bodyA->GetAngle();
}
void b2PrismaticJointDef::Initialize(b2Body* bA, b2Body* bB, const b2Vec2& anchor, const b2Vec2& axis) {
  bodyA = bA;
  bodyB = bB;
  localAnchorA = bodyA->GetLocalPoint(anchor);
  localAnchorB = bodyB->GetLocalPoint(anchor);
  localAxisA = bodyA->GetLocalVector(axis);
  referenceAngle = bodyB->GetAngle() - bodyA->GetAngle();
}
// b2WeldJointDef::Initialize (src/dynamics/b2_weld_joint.cpp:39-46)
void b2WeldJointDef::Initialize(b2Body* bA, b2Body* bB, const b2Vec2& anchor) {
  bodyA = bA;
  bodyB = bB;
  localAnchorA = bodyA->GetLocalPoint(anchor);
  localAnchorB = bodyB->GetLocalPoint(anchor);
  referenceAngle = bodyB->GetAngle() - bodyA->GetAngle();
}
// b2WheelJointDef::Initialize (src/dynamics/b2_wheel_joint.cpp:33-40)
void b2WheelJointDef::Initialize(b2Body* bA, b2Body* bB, const b2Vec2& anchor, const b2Vec2& axis) {
  bodyA = bA;
  bodyB = bB;
  localAnchorA = bodyA->GetLocalPoint(anchor);
  localAnchorB = bodyB->GetLocalPoint(anchor);
  localAxisA = bodyA->GetLocalVector(axis);
}
// b2MotorJointDef::Initialize (src/dynamics/b2_motor_joint.cpp:34-44)
void b2MotorJointDef::Initialize(b2Body* bA, b2Body* bB) {
  bodyA = bA;
  bodyB = bB;
  b2Vec2 xB = bodyB->GetPosition();
  linearOffset = bodyA->GetLocalPoint(xB);
  float angleA = bodyA->GetAngle();
  float angleB = bodyB->GetAngle();
  angularOffset = angleB - angleA;
}
// b2FrictionJointDef::Initialize (src/dynamics/b2_friction_joint.cpp:38-44)
void b2FrictionJointDef::Initialize(b2Body* bA, b2Body* bB, const b2Vec2& anchor) {
  bodyA = bA;
  bodyB = bB;
  localAnchorA = bodyA->GetLocalPoint(anchor);
  localAnchorB = bodyB->GetLocalPoint(anchor);
}
// b2PulleyJointDef::Initialize (src/dynamics/b2_pulley_joint.cpp:39-58)
void b2PulleyJointDef::Initialize(b2Body* bA, b2Body* bB, const b2Vec2& groundA, const b2Vec2& groundB,
                                  const b2Vec2& anchorA, const b2Vec2& anchorB, float r) {
  bodyA = bA;
  bodyB = bB;
  groundAnchorA = groundA;
  groundAnchorB = groundB;
  localAnchorA = bodyA->GetLocalPoint(anchorA);
  localAnchorB = bodyB->GetLocalPoint(anchorB);
  b2Vec2 dA = anchorA - groundA;
  lengthA = dA.Length();
  b2Vec2 dB = anchorB - groundB;
  lengthB = dB.Length();
  ratio = r;
}
// Effective mass (or inertia) of the pair: the reduced value when both are positive, else the
// positive one; stiffness = m w^2 and damping = 2 m zeta w with w = 2 pi f, in the reference's
// operation order (src/dynamics/b2_joint.cpp:40-88).
static float pairValue(float a, float b) {
  if (a > 0.0f && b > 0.0f) return a * b / (a + b);
  return a > 0.0f ? a : b;
}
void b2LinearStiffness(float& stiffness, float& damping, float frequencyHertz, float dampingRatio,
                       const b2Body* bodyA, const b2Body* bodyB) {
  float mass = pairValue(bodyA->GetMass(), bodyB->GetMass());
  float omega = 2.0f * b2_pi * frequencyHertz;
  stiffness = mass * omega * omega;
  damping = 2.0f * mass * dampingRatio * omega;
}
void b2AngularStiffness(float& stiffness, float& damping, float frequencyHertz, float dampingRatio,
                        const b2Body* bodyA, const b2Body* bodyB) {
  float inertia = pairValue(bodyA->GetInertia(), bodyB->GetInertia());
  float omega = 2.0f * b2_pi * frequencyHertz;
  stiffness = inertia * omega * omega;
  damping = 2.0f * inertia * dampingRatio * omega;
}
void b2DistanceJointDef::Initialize(b2Body* b1, b2Body* b2, const b2Vec2& anchor1, const b2Vec2& anchor2) {
  bodyA = b1;
  bodyB = b2;
  localAnchorA = bodyA->GetLocalPoint(anchor1);
  localAnchorB = bodyB->GetLocalPoint(anchor2);
  b2Vec2 d = anchor2 - anchor1;
  length = b2Max(d.Length(), b2_linearSlop);
  minLength = length;
  maxLength = length;
}

// GetReactionForce / GetReactionTorque of each joint type (b2_revolute_joint.cpp:333-342,
// b2_prismatic_joint.cpp:461-469, b2_distance_joint.cpp:326-330): inv_dt times the last step's
// constraint impulse.
b2Vec2 b2Joint::GetReactionForce(float inv_dt) const {
  const b2g_joint& r = m_world->JointRecord(m_index);
  return inv_dt * b2Vec2(r.reaction_impulse[0], r.reaction_impulse[1]);
}
float b2Joint::GetReactionTorque(float inv_dt) const {
  const b2g_joint& r = m_world->JointRecord(m_index);
  return inv_dt * r.reaction_angular_impulse;
}

// ---------------------------------------------------------------- contacts
void b2Contact::GetWorldManifold(b2WorldManifold* wm) const {
  const b2Body* bodyA = m_fixtureA->GetBody();
  const b2Body* bodyB = m_fixtureB->GetBody();
  wm->Initialize(&m_manifold, bodyA->GetTransform(), m_fixtureA->GetShape()->m_radius, bodyB->GetTransform(),
                 m_fixtureB->GetShape()->m_radius);
}

static void manifold_from(const b2g_manifold& s, b2Manifold* m) {
  for (int i = 0; i < 2; ++i) {
    m->points[i].localPoint.Set(s.points[i].local_point[0], s.points[i].local_point[1]);
    m->points[i].normalImpulse = s.points[i].normal_impulse;
    m->points[i].tangentImpulse = s.points[i].tangent_impulse;
    m->points[i].id.key = s.points[i].id;
  }
  m->localNormal.Set(s.local_normal[0], s.local_normal[1]);
  m->localPoint.Set(s.local_point[0], s.local_point[1]);
  m->type = (b2Manifold::Type)s.type;
  m->pointCount = s.point_count;
}

// ---------------------------------------------------------------- world
b2World::b2World(const b2Vec2& gravity) : m_gravity(gravity) {
  if (b2g_batch_create(0, 0, &m_batch) != B2G_OK) throw std::runtime_error(b2g_last_error());
  m_ownsBatch = true;
  b2g_world_add(m_batch, gravity.x, gravity.y, &m_index);
  ApplyFlags();
}

b2World::b2World(b2g_batch* batch, const b2Vec2& gravity) : m_gravity(gravity) {
  m_batch = batch;
  m_ownsBatch = false;
  b2g_world_add(m_batch, gravity.x, gravity.y, &m_index);
  ApplyFlags();
}

b2World::b2World(b2g_batch* batch, int32 index, bool attach) {
  B2_NOT_USED(attach);
  m_batch = batch;
  m_ownsBatch = false;
  m_index = index;
  m_gravity.Set(0.0f, -10.0f);
  // an attached world keeps the flags it has
  int32_t sleep = 0, warm = 1, continuous = 0, clear = 1;
  b2g_world_get_flags(m_batch, m_index, &sleep, &warm, &continuous, &clear);
  m_allowSleep = sleep != 0;
  m_warmStarting = warm != 0;
  m_continuous = continuous != 0;
  m_autoClear = clear != 0;
}

b2World::~b2World() {
  if (m_ownsBatch && m_batch) b2g_batch_destroy(m_batch);
}

void b2World::ApplyFlags() { b2g_world_set_flags(m_batch, m_index, m_allowSleep, m_warmStarting, m_continuous, m_autoClear); }

void b2World::SetAllowSleeping(bool flag) { m_allowSleep = flag; ApplyFlags(); }
void b2World::SetWarmStarting(bool flag) { m_warmStarting = flag; ApplyFlags(); }
void b2World::SetContinuousPhysics(bool flag) { m_continuous = flag; ApplyFlags(); }
void b2World::SetAutoClearForces(bool flag) { m_autoClear = flag; ApplyFlags(); }
void b2World::SetGravity(const b2Vec2& g) { m_gravity = g; b2g_world_set_gravity(m_batch, m_index, g.x, g.y); }

void b2World::SetContactListener(b2ContactListener* listener) {
  m_listener = listener;
  b2g_events_enable(m_batch, listener ? 1 : 0);
}

b2Body* b2World::CreateBody(const b2BodyDef* def) {
  b2g_body_def d;
  memset(&d, 0, sizeof(d));
  d.type = def->type;
  d.position[0] = def->position.x; d.position[1] = def->position.y;
  d.angle = def->angle;
  d.linear_velocity[0] = def->linearVelocity.x; d.linear_velocity[1] = def->linearVelocity.y;
  d.angular_velocity = def->angularVelocity;
  d.linear_damping = def->linearDamping;
  d.angular_damping = def->angularDamping;
  d.gravity_scale = def->gravityScale;
  d.allow_sleep = def->allowSleep;
  d.awake = def->awake;
  d.fixed_rotation = def->fixedRotation;
  d.bullet = def->bullet;
  d.enabled = def->enabled;
  d.user_data = def->userData.pointer;
  int32_t id = -1;
  if (b2g_bodies_add(m_batch, m_index, &d, 1, &id) != B2G_OK) return nullptr;
  b2Body* last = m_bodyTail;  // the last live body, which links to the new one
  m_bodies.emplace_back();
  b2Body* b = &m_bodies.back();
  b->m_world = this;
  b->m_index = id;
  b->m_type = def->type;
  b->m_fixedRotation = def->fixedRotation;
  b->m_userData = def->userData;
  if (last) last->m_next = b;
  else m_bodyHead = b;
  m_bodyTail = b;
  ++m_bodyCount;
  InvalidateCaches();
  return b;
}

void b2World::Dump() {
  uint64_t n = 0;
  b2g_world_dump(m_batch, m_index, nullptr, 0, &n);
  std::vector<char> text(n + 1);
  if (b2g_world_dump(m_batch, m_index, text.data(), n + 1, &n) != B2G_OK) return;
  FILE* f = fopen("box2d_dump.inl", "w");
  if (!f) return;
  fwrite(text.data(), 1, n, f);
  fclose(f);
}

void b2World::SetContactFilter(b2ContactFilter* filter) {
  m_filter = filter;
  m_filterUnsupported = filter && typeid(*filter) != typeid(b2ContactFilter);
}

// EndContact for the contacts a removal destroyed (the engine's End records carry the fixture
// indices from before the removal), with the contact as it was.
void b2World::EndContacts(const std::vector<b2g_event>& ended, int32 n, const std::vector<b2Contact>& before) {
  if (!m_listener) return;
  std::map<std::pair<int, int>, const b2Contact*> byPair;
  for (const b2Contact& c : before) byPair[{c.m_fixtureA->m_index, c.m_fixtureB->m_index}] = &c;
  for (int32 i = 0; i < n && i < (int32)ended.size(); ++i) {
    auto it = byPair.find({ended[i].fixture_a, ended[i].fixture_b});
    if (it == byPair.end()) continue;
    b2Contact c = *it->second;
    c.m_next = nullptr;
    m_listener->EndContact(&c);
  }
}

// Indices follow the engine's renumbering: live bodies, fixtures and joints keep their creation
// order and are numbered 0, 1, ... again; the fixture index table is rebuilt.
void b2World::Renumber() {
  int32 k = 0;
  for (b2Body* b = m_bodyHead; b; b = b->m_next) b->m_index = k++;
  m_bodyCount = k;
  std::vector<b2Fixture*> live;
  for (b2Fixture* f : m_fixtureIndex)
    if (f->m_index >= 0) live.push_back(f);
  for (size_t i = 0; i < live.size(); ++i) live[i]->m_index = (int32)i;
  m_fixtureIndex.swap(live);
  for (size_t i = 0; i < m_joints.size(); ++i) {
    m_joints[i]->m_index = (int32)i;
    m_joints[i]->m_next = i + 1 < m_joints.size() ? m_joints[i + 1].get() : nullptr;
  }
  InvalidateCaches();
}

void b2World::DestroyBody(b2Body* body) {
  if (!body || body->m_index < 0 || body->m_world != this) return;
  // the joints it takes along (SayGoodbye first, as the reference does)
  for (auto& j : m_joints)
    if ((j->m_bodyA == body || j->m_bodyB == body) && m_destruction) m_destruction->SayGoodbye(j.get());
  for (b2Fixture* f = body->m_fixtureList; f; f = f->m_next)
    if (m_destruction) m_destruction->SayGoodbye(f);
  std::vector<b2Contact> before;
  if (m_listener) {
    GetContactListStart();
    before = m_contacts;
  }
  std::vector<b2g_event> ended((size_t)std::max(GetContactCount(), 1));
  int32_t ne = 0;
  const int32_t idx = body->m_index;
  m_lastStatus = b2g_bodies_remove(m_batch, m_index, &idx, 1, ended.data(), (int32_t)ended.size(), &ne);
  if (m_lastStatus != B2G_OK) return;
  EndContacts(ended, ne, before);
  // drop the body's joints, fixtures and the body itself from the facade's lists
  for (size_t i = 0; i < m_joints.size();) {
    if (m_joints[i]->m_bodyA == body || m_joints[i]->m_bodyB == body) m_joints.erase(m_joints.begin() + i);
    else ++i;
  }
  EraseOrphanGears();
  for (b2Fixture* f = body->m_fixtureList; f; f = f->m_next) f->m_index = -1;
  b2Body* prev = nullptr;
  for (b2Body* x = m_bodyHead; x && x != body; x = x->m_next) prev = x;
  if (prev) prev->m_next = body->m_next;
  else m_bodyHead = body->m_next;
  if (m_bodyTail == body) m_bodyTail = prev;
  body->m_next = nullptr;
  body->m_fixtureList = nullptr;
  body->m_index = -1;
  Renumber();
}

void b2World::DestroyJoint(b2Joint* joint) {
  if (!joint || joint->m_world != this) return;
  size_t i = 0;
  while (i < m_joints.size() && m_joints[i].get() != joint) ++i;
  if (i == m_joints.size()) return;
  const int32_t idx = joint->m_index;
  m_lastStatus = b2g_joints_remove(m_batch, m_index, &idx, 1);
  if (m_lastStatus != B2G_OK) return;
  m_joints.erase(m_joints.begin() + i);
  EraseOrphanGears();
  Renumber();
}

// The engine removes a gear together with either joint it couples; the facade follows.
void b2World::EraseOrphanGears() {
  for (bool again = true; again;) {
    again = false;
    for (size_t i = 0; i < m_joints.size(); ++i) {
      if (m_joints[i]->m_type != e_gearJoint) continue;
      b2GearJoint* g = (b2GearJoint*)m_joints[i].get();
      bool alive1 = false, alive2 = false;
      for (auto& x : m_joints) {
        alive1 |= x.get() == g->m_joint1;
        alive2 |= x.get() == g->m_joint2;
      }
      if (!alive1 || !alive2) {
        m_joints.erase(m_joints.begin() + i);
        again = true;
        break;
      }
    }
  }
}

void b2Body::DestroyFixture(b2Fixture* fixture) {
  if (!fixture || fixture->m_body != this || fixture->m_index < 0) return;
  b2World* w = m_world;
  std::vector<b2Contact> before;
  if (w->m_listener) {
    w->GetContactListStart();
    before = w->m_contacts;
  }
  std::vector<b2g_event> ended((size_t)std::max(w->GetContactCount(), 1));
  int32_t ne = 0;
  const int32_t idx = fixture->m_index;
  w->m_lastStatus = b2g_fixtures_remove(w->m_batch, w->m_index, &idx, 1, ended.data(), (int32_t)ended.size(), &ne);
  if (w->m_lastStatus != B2G_OK) return;
  w->EndContacts(ended, ne, before);
  b2Fixture** link = &m_fixtureList;
  while (*link && *link != fixture) link = &(*link)->m_next;
  if (*link) *link = fixture->m_next;
  fixture->m_next = nullptr;
  fixture->m_index = -1;
  w->Renumber();
}

void b2Body::SetAwake(bool flag) {
  m_world->m_lastStatus = b2g_body_set_awake(m_world->m_batch, m_world->m_index, m_index, flag ? 1 : 0);
  m_world->InvalidateCaches();
}

bool b2Body::IsAwake() const { return (m_world->BodyRecord(m_index).flags & B2G_BODY_AWAKE) != 0; }

void b2Body::SetBullet(bool flag) {
  m_world->m_lastStatus = b2g_body_set_bullet(m_world->m_batch, m_world->m_index, m_index, flag ? 1 : 0);
  m_world->InvalidateCaches();
}

bool b2Body::IsBullet() const { return (m_world->BodyRecord(m_index).flags & B2G_BODY_BULLET) != 0; }

bool b2Body::IsSleepingAllowed() const { return (m_world->BodyRecord(m_index).flags & B2G_BODY_AUTO_SLEEP) != 0; }

b2Joint* b2World::CreateJoint(const b2JointDef* def) {
  if (!def || !def->bodyA || !def->bodyB) return nullptr;
  b2g_joint_def d;
  memset(&d, 0, sizeof(d));
  d.body_a = def->bodyA->m_index;
  d.body_b = def->bodyB->m_index;
  d.collide_connected = def->collideConnected ? 1 : 0;
  d.user_data = def->userData.pointer;
  std::unique_ptr<b2Joint> j;
  b2Vec2 la(0.0f, 0.0f), lb(0.0f, 0.0f);  // the motor and mouse joints have no local anchor A
  if (def->type == e_revoluteJoint) {
    const b2RevoluteJointDef* r = (const b2RevoluteJointDef*)def;
    d.type = B2G_JOINT_REVOLUTE;
    la = r->localAnchorA; lb = r->localAnchorB;
    d.reference_angle = r->referenceAngle;
    d.enable_limit = r->enableLimit; d.lower = r->lowerAngle; d.upper = r->upperAngle;
    d.enable_motor = r->enableMotor; d.max_motor = r->maxMotorTorque; d.motor_speed = r->motorSpeed;
    j.reset(new b2RevoluteJoint());
  } else if (def->type == e_prismaticJoint) {
    const b2PrismaticJointDef* p = (const b2PrismaticJointDef*)def;
    d.type = B2G_JOINT_PRISMATIC;
    la = p->localAnchorA; lb = p->localAnchorB;
    d.local_axis_a[0] = p->localAxisA.x; d.local_axis_a[1] = p->localAxisA.y;
    d.reference_angle = p->referenceAngle;
    d.enable_limit = p->enableLimit; d.lower = p->lowerTranslation; d.upper = p->upperTranslation;
    d.enable_motor = p->enableMotor; d.max_motor = p->maxMotorForce; d.motor_speed = p->motorSpeed;
    j.reset(new b2PrismaticJoint());
  } else if (def->type == e_distanceJoint) {
    const b2DistanceJointDef* q = (const b2DistanceJointDef*)def;
    d.type = B2G_JOINT_DISTANCE;
    la = q->localAnchorA; lb = q->localAnchorB;
    d.length = q->length; d.min_length = q->minLength; d.max_length = q->maxLength;
    d.stiffness = q->stiffness; d.damping = q->damping;
    j.reset(new b2DistanceJoint());
  } else if (def->type == e_weldJoint) {
    const b2WeldJointDef* q = (const b2WeldJointDef*)def;
    d.type = B2G_JOINT_WELD;
    la = q->localAnchorA; lb = q->localAnchorB;
    d.reference_angle = q->referenceAngle; d.stiffness = q->stiffness; d.damping = q->damping;
    j.reset(new b2WeldJoint());
  } else if (def->type == e_wheelJoint) {
    const b2WheelJointDef* q = (const b2WheelJointDef*)def;
    d.type = B2G_JOINT_WHEEL;
    la = q->localAnchorA; lb = q->localAnchorB;
    d.local_axis_a[0] = q->localAxisA.x; d.local_axis_a[1] = q->localAxisA.y;
    d.enable_limit = q->enableLimit; d.lower = q->lowerTranslation; d.upper = q->upperTranslation;
    d.enable_motor = q->enableMotor; d.max_motor = q->maxMotorTorque; d.motor_speed = q->motorSpeed;
    d.stiffness = q->stiffness; d.damping = q->damping;
    j.reset(new b2WheelJoint());
  } else if (def->type == e_motorJoint) {
    const b2MotorJointDef* q = (const b2MotorJointDef*)def;
    d.type = B2G_JOINT_MOTOR;
    d.linear_offset[0] = q->linearOffset.x; d.linear_offset[1] = q->linearOffset.y;
    d.reference_angle = q->angularOffset;
    d.max_force = q->maxForce; d.max_torque = q->maxTorque; d.correction_factor = q->correctionFactor;
    j.reset(new b2MotorJoint());
  } else if (def->type == e_gearJoint) {
    const b2GearJointDef* q = (const b2GearJointDef*)def;
    if (!q->joint1 || !q->joint2 || q->joint1->m_world != this || q->joint2->m_world != this) return nullptr;
    d.type = B2G_JOINT_GEAR;
    d.joint_1 = q->joint1->m_index;
    d.joint_2 = q->joint2->m_index;
    d.ratio = q->ratio;
    // the gear's bodies and anchors are its joints' bodies B (b2_gear_joint.cpp:62-110)
    la = q->joint1->m_localAnchorB;
    lb = q->joint2->m_localAnchorB;
    b2GearJoint* g = new b2GearJoint();
    g->m_joint1 = q->joint1;
    g->m_joint2 = q->joint2;
    g->m_ratio = q->ratio;
    j.reset(g);
  } else if (def->type == e_frictionJoint) {
    const b2FrictionJointDef* q = (const b2FrictionJointDef*)def;
    d.type = B2G_JOINT_FRICTION;
    la = q->localAnchorA; lb = q->localAnchorB;
    d.max_force = q->maxForce; d.max_torque = q->maxTorque;
    j.reset(new b2FrictionJoint());
  } else if (def->type == e_mouseJoint) {
    const b2MouseJointDef* q = (const b2MouseJointDef*)def;
    d.type = B2G_JOINT_MOUSE;
    d.target[0] = q->target.x; d.target[1] = q->target.y;
    d.max_force = q->maxForce; d.stiffness = q->stiffness; d.damping = q->damping;
    j.reset(new b2MouseJoint());
  } else if (def->type == e_pulleyJoint) {
    const b2PulleyJointDef* q = (const b2PulleyJointDef*)def;
    d.type = B2G_JOINT_PULLEY;
    la = q->localAnchorA; lb = q->localAnchorB;
    d.ground_anchor_a[0] = q->groundAnchorA.x; d.ground_anchor_a[1] = q->groundAnchorA.y;
    d.ground_anchor_b[0] = q->groundAnchorB.x; d.ground_anchor_b[1] = q->groundAnchorB.y;
    d.length_a = q->lengthA; d.length_b = q->lengthB; d.ratio = q->ratio;
    j.reset(new b2PulleyJoint());
  } else {
    return nullptr;
  }
  d.local_anchor_a[0] = la.x; d.local_anchor_a[1] = la.y;
  d.local_anchor_b[0] = lb.x; d.local_anchor_b[1] = lb.y;
  int32_t id = -1;
  if (b2g_joints_add(m_batch, m_index, &d, 1, &id) != B2G_OK) return nullptr;
  if (def->type == e_mouseJoint) {  // the engine computed the anchor on body B from the target
    b2g_joint rec;
    if (b2g_joints_read(m_batch, m_index, id, 1, &rec) == B2G_OK) lb.Set(rec.def.local_anchor_b[0], rec.def.local_anchor_b[1]);
  }
  j->m_world = this;
  j->m_index = id;
  j->m_type = def->type;
  j->m_bodyA = def->bodyA;
  j->m_bodyB = def->bodyB;
  if (def->type == e_gearJoint) {  // b2GearJoint::b2GearJoint replaces the def's bodies
    const b2GearJointDef* q = (const b2GearJointDef*)def;
    j->m_bodyA = q->joint1->m_bodyB;
    j->m_bodyB = q->joint2->m_bodyB;
  }
  j->m_collideConnected = def->collideConnected;
  j->m_localAnchorA = la;
  j->m_localAnchorB = lb;
  j->m_userData = def->userData;
  b2Joint* raw = j.get();
  if (!m_joints.empty()) m_joints.back()->m_next = raw;
  m_joints.push_back(std::move(j));
  InvalidateCaches();
  return raw;
}

const b2g_body& b2World::BodyRecord(int32 index) const {
  if (!m_stateValid) {
    int32_t nb = 0;  // the engine world's bodies (an attached world may hold some made elsewhere)
    b2g_world_sizes(m_batch, m_index, &nb, nullptr, nullptr, nullptr);
    m_state.resize((size_t)nb);
    if (!m_state.empty()) b2g_bodies_read(m_batch, m_index, 0, (int32_t)m_state.size(), m_state.data());
    m_stateValid = true;
  }
  return m_state[index];
}

void b2World::WriteBody(int32 index, const b2g_body& rec) {
  b2g_bodies_write(m_batch, m_index, index, 1, &rec);
  InvalidateCaches();
}

const b2g_joint& b2World::JointRecord(int32 index) const {
  if (!m_jointsValid) {
    int32_t nj = 0;
    b2g_world_sizes(m_batch, m_index, nullptr, nullptr, &nj, nullptr);
    m_jointState.resize((size_t)nj);
    if (!m_jointState.empty()) b2g_joints_read(m_batch, m_index, 0, (int32_t)m_jointState.size(), m_jointState.data());
    m_jointsValid = true;
  }
  return m_jointState[index];
}

void b2World::Step(float dt, int32 vi, int32 pi, int32 particleIterations) {
  B2_NOT_USED(particleIterations);
  if (m_filterUnsupported) {  // a custom b2ContactFilter cannot be run: nothing is stepped
    m_lastStatus = B2G_E_INVALID_ARG;
    return;
  }
  int32_t nw = 0;
  b2g_world_count(m_batch, &nw);
  std::vector<uint8_t> mask(nw, 0);
  mask[m_index] = 1;
  m_lastStatus = b2g_step(m_batch, dt, vi, pi, mask.data());
  InvalidateCaches();
  b2g_profile p;
  if (b2g_profile_get(m_batch, &p) == B2G_OK) {
    m_profile.step = p.step; m_profile.collide = p.collide; m_profile.solve = p.solve;
    m_profile.broadphase = p.broadphase; m_profile.solveTOI = p.solve_toi;
  }
  if (m_listener) Deliver();
}

void b2World::ClearForces() {
  for (b2Body* b = m_bodyHead; b; b = b->m_next) {
    b2g_body r = BodyRecord(b->m_index);
    if (r.force[0] != 0.0f || r.force[1] != 0.0f || r.torque != 0.0f) {
      r.force[0] = r.force[1] = 0.0f;
      r.torque = 0.0f;
      WriteBody(b->m_index, r);
    }
  }
}

b2Contact* b2World::GetContactListStart() {
  if (!m_contactsValid) {
    int32_t n = 0;
    b2g_contacts_read(m_batch, m_index, nullptr, 0, &n);
    std::vector<b2g_contact> recs(n);
    if (n) b2g_contacts_read(m_batch, m_index, recs.data(), n, &n);
    m_contacts.assign(n, b2Contact());
    for (int32_t i = 0; i < n; ++i) {
      b2Contact& c = m_contacts[i];
      c.m_fixtureA = m_fixtureIndex[recs[i].fixture_a];
      c.m_fixtureB = m_fixtureIndex[recs[i].fixture_b];
      c.m_flags = recs[i].flags;
      c.m_friction = recs[i].friction;
      c.m_restitution = recs[i].restitution;
      c.m_restitutionThreshold = recs[i].restitution_threshold;
      c.m_tangentSpeed = recs[i].tangent_speed;
      manifold_from(recs[i].manifold, &c.m_manifold);
    }
    for (int32_t i = 0; i < n; ++i) m_contacts[i].m_next = (i + 1 < n) ? &m_contacts[i + 1] : &m_contactEnd;
    m_contactsValid = true;
  }
  return m_contacts.empty() ? &m_contactEnd : &m_contacts[0];
}

int32 b2World::GetContactCount() const {
  int32_t nc = 0;
  b2g_world_sizes(m_batch, m_index, nullptr, nullptr, nullptr, &nc);
  return nc;
}

// Batched listener delivery after the step: this world's events only (the other worlds of a
// shared batch keep theirs for their own b2World::DeliverEvents).
void b2World::DeliverEvents() {
  if (m_listener) Deliver();
}

void b2World::Deliver() {
  std::vector<b2g_event> ev(1 << 16);
  b2Contact* start = GetContactListStart();
  B2_NOT_USED(start);
  std::map<std::pair<int, int>, b2Contact*> byPair;
  for (b2Contact& c : m_contacts) byPair[{c.m_fixtureA->m_index, c.m_fixtureB->m_index}] = &c;
  for (;;) {
    int32_t n = 0;
    if (b2g_events_drain_world(m_batch, m_index, ev.data(), (int32_t)ev.size(), &n) != B2G_OK || n == 0) break;
    for (int32_t i = 0; i < n; ++i) {
      const b2g_event& e = ev[i];
      b2Contact tmp;
      b2Contact* c = &tmp;
      auto it = byPair.find({e.fixture_a, e.fixture_b});
      if (it != byPair.end()) c = it->second;
      else {
        tmp.m_fixtureA = m_fixtureIndex[e.fixture_a];
        tmp.m_fixtureB = m_fixtureIndex[e.fixture_b];
        tmp.m_manifold.pointCount = 0;
      }
      if (e.kind == B2G_EVENT_BEGIN) m_listener->BeginContact(c);
      else if (e.kind == B2G_EVENT_END) m_listener->EndContact(c);
      else if (e.kind == B2G_EVENT_PRESOLVE) {
        b2Manifold old;
        manifold_from(e.old_manifold, &old);
        m_listener->PreSolve(c, &old);
      } else if (e.kind == B2G_EVENT_POSTSOLVE) {
        b2ContactImpulse imp;
        imp.count = e.point_count;
        for (int k = 0; k < 2; ++k) { imp.normalImpulses[k] = e.normal_impulses[k]; imp.tangentImpulses[k] = e.tangent_impulses[k]; }
        m_listener->PostSolve(c, &imp);
      }
    }
  }
}

// ---------------------------------------------------------------- scenes through the facade
extern "C" B2G_API int b2g_scene_build(b2g_batch* b, int32_t world, int32_t kind, uint32_t seed, int32_t n, float p0,
                                       float p1, int32_t* counts) {
  if (!b || n < 0) return B2G_E_INVALID_ARG;
  int32_t nw = 0;
  b2g_world_count(b, &nw);
  if (world < 0 || world >= nw) return B2G_E_INVALID_ARG;
  b2World w(b, world, true);
  b2scenes::ResetTags();
  b2scenes::Counts c;
  if (kind == B2G_SCENE_PYRAMID) c = b2scenes::Pyramid(&w, n, p0, p1, true);
  else if (kind == B2G_SCENE_MIXED_DROP) c = b2scenes::MixedDrop(&w, n, seed);
  else if (kind == B2G_SCENE_CHAINS) c = b2scenes::ChainsOverPile(&w, n, 20, (int)p0, seed);
  else if (kind == B2G_SCENE_BATCH_WORLD) c = b2scenes::BatchWorld(&w, seed, n);
  else if (kind == B2G_SCENE_JOINTS) c = b2scenes::JointZoo(&w, n, seed);
  else if (kind == B2G_SCENE_SLIDERS) c = b2scenes::SliderRigs(&w, n, seed);
  else if (kind == B2G_SCENE_GEARS) c = b2scenes::GearRigs(&w, n, seed);
  else if (kind == B2G_SCENE_BULLETS) c = b2scenes::Bullets(&w, n, seed, p0 > 0.5f);
  else return B2G_E_INVALID_ARG;
  if (counts) { counts[0] = c.bodies; counts[1] = c.fixtures; counts[2] = c.joints; }
  return B2G_OK;
}

extern "C" B2G_API int b2g_batch_world_params(uint32_t seed, int32_t* n_bodies, float* gx, float* gy) {
  if (n_bodies) *n_bodies = b2scenes::BatchBodyCount(seed);
  b2Vec2 g = b2scenes::BatchGravity(seed);
  if (gx) *gx = g.x;
  if (gy) *gy = g.y;
  return B2G_OK;
}
