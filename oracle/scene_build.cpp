// The oracle's scene builder: runs the batched scene recipes (box2d-optimized_gb300/scenes/
// scenes.h) through the oracle's own scene-building API (scene_api/box2d/box2d.h) and loads the
// resulting records into an oracle world. Test infrastructure only: it lets the CPU baseline and
// the reference arm of the benchmark build their worlds without loading the engine library. The
// records it makes are byte-identical to the engine facade's for the same recipe (checked by the
// CPU tests), which in turn are byte-identical to the reference's own set-up.
#include <string.h>

#include "scene_api/box2d/box2d.h"
#include "../box2d-optimized_gb300/scenes/scenes.h"

extern "C" {
int orc_polygon_set(const float* xy, int32_t n, b2g_shape* out);
int orc_polygon_box(float hx, float hy, float cx, float cy, float angle, int32_t oriented, b2g_shape* out);
int orc_shape_mass(const b2g_shape* s, float density, float* out4);
void* orc_world_new(float gx, float gy);
int orc_world_load(void* h, const b2g_body* bodies, int32_t nb, const b2g_fixture* fixtures, int32_t nf,
                   const b2g_joint* joints, int32_t nj, const b2g_contact* contacts, int32_t nc, float inv_dt0);
}

// ---------------------------------------------------------------- shapes
void b2EdgeShape::SetTwoSided(const b2Vec2& v1, const b2Vec2& v2) {
  // m_vertex1 = v1, m_vertex2 = v2, ghost vertices m_vertex0 = m_vertex3 = 0, two-sided
  memset(&rec, 0, sizeof(rec));
  rec.type = B2G_SHAPE_EDGE;
  rec.radius = b2_polygonRadius;
  rec.vertices[0][0] = v1.x;
  rec.vertices[0][1] = v1.y;
  rec.vertices[1][0] = v2.x;
  rec.vertices[1][1] = v2.y;
  rec.one_sided = 0;
}

void b2PolygonShape::Set(const b2Vec2* points, int32 count) {
  float xy[2 * b2_maxPolygonVertices];
  const int n = count < b2_maxPolygonVertices ? count : b2_maxPolygonVertices;
  for (int i = 0; i < n; ++i) {
    xy[2 * i] = points[i].x;
    xy[2 * i + 1] = points[i].y;
  }
  orc_polygon_set(xy, count, &rec);
}

void b2PolygonShape::SetAsBox(float hx, float hy) { orc_polygon_box(hx, hy, 0.0f, 0.0f, 0.0f, 0, &rec); }

void b2PolygonShape::SetAsBox(float hx, float hy, const b2Vec2& center, float angle) {
  orc_polygon_box(hx, hy, center.x, center.y, angle, 1, &rec);
}

// ---------------------------------------------------------------- bodies
static inline b2Vec2 mulT(const b2g_body& b, const b2Vec2& v) {
  // b2MulT(m_xf, v): the inverse rotation of (v - p)
  const float px = v.x - b.xf[0], py = v.y - b.xf[1];
  return b2Vec2(b.xf[3] * px + b.xf[2] * py, -b.xf[2] * px + b.xf[3] * py);
}

b2Body* b2World::CreateBody(const b2BodyDef* def) {
  b2g_body r;
  memset(&r, 0, sizeof(r));
  r.xf[0] = def->position.x;
  r.xf[1] = def->position.y;
  r.xf[2] = sinf(def->angle);
  r.xf[3] = cosf(def->angle);
  r.c[0] = def->position.x;
  r.c[1] = def->position.y;
  r.a = def->angle;
  r.v[0] = def->linearVelocity.x;
  r.v[1] = def->linearVelocity.y;
  r.w = def->angularVelocity;
  r.linear_damping = def->linearDamping;
  r.angular_damping = def->angularDamping;
  r.gravity_scale = def->gravityScale;
  r.type = (int32_t)def->type;
  uint32_t fl = 0;
  if (def->bullet) fl |= B2G_BODY_BULLET;
  if (def->fixedRotation) fl |= B2G_BODY_FIXED_ROTATION;
  if (def->allowSleep) fl |= B2G_BODY_AUTO_SLEEP;
  if (def->awake && def->type != b2_staticBody) fl |= B2G_BODY_AWAKE;
  if (def->enabled) fl |= B2G_BODY_ENABLED;
  r.flags = fl;
  bodies.push_back(r);
  bodyFixtures.emplace_back();
  b2Body* b = new b2Body();
  b->m_world = this;
  b->m_index = (int)bodies.size() - 1;
  handles.push_back(b);
  return b;
}

b2Vec2 b2Body::GetPosition() const {
  const b2g_body& r = m_world->bodies[m_index];
  return b2Vec2(r.xf[0], r.xf[1]);
}

float b2Body::GetAngle() const { return m_world->bodies[m_index].a; }

b2Vec2 b2Body::GetLocalPoint(const b2Vec2& worldPoint) const { return mulT(m_world->bodies[m_index], worldPoint); }

// b2Body::ResetMassData: mass, centre and rotational inertia from the fixtures, newest first.
static void resetMassData(b2World* w, int bi) {
  b2g_body& b = w->bodies[bi];
  b.mass = 0.0f;
  b.inv_mass = 0.0f;
  b.inertia = 0.0f;
  b.inv_inertia = 0.0f;
  b.local_center[0] = 0.0f;
  b.local_center[1] = 0.0f;
  if (b.type == B2G_STATIC || b.type == B2G_KINEMATIC) {
    b.c[0] = b.xf[0];
    b.c[1] = b.xf[1];
    return;
  }
  float lcx = 0.0f, lcy = 0.0f, mass = 0.0f, I = 0.0f;
  const std::vector<int>& fl = w->bodyFixtures[bi];
  for (int k = (int)fl.size() - 1; k >= 0; --k) {
    const b2g_fixture& f = w->fixtures[fl[k]];
    if (f.density == 0.0f) continue;
    float md[4];  // mass, centre x, centre y, inertia
    orc_shape_mass(&f.shape, f.density, md);
    mass += md[0];
    lcx += md[0] * md[1];
    lcy += md[0] * md[2];
    I += md[3];
  }
  float invMass = 0.0f, invI = 0.0f;
  if (mass > 0.0f) {
    invMass = 1.0f / mass;
    lcx *= invMass;
    lcy *= invMass;
  }
  if (I > 0.0f && (b.flags & B2G_BODY_FIXED_ROTATION) == 0) {
    I -= mass * (lcx * lcx + lcy * lcy);
    invI = 1.0f / I;
  } else {
    I = 0.0f;
    invI = 0.0f;
  }
  const float ocx = b.c[0], ocy = b.c[1];
  // b2Mul(m_xf, localCenter)
  const float cx = (b.xf[3] * lcx - b.xf[2] * lcy) + b.xf[0];
  const float cy = (b.xf[2] * lcx + b.xf[3] * lcy) + b.xf[1];
  b.mass = mass;
  b.inv_mass = invMass;
  b.inertia = I;
  b.inv_inertia = invI;
  b.local_center[0] = lcx;
  b.local_center[1] = lcy;
  b.c[0] = cx;
  b.c[1] = cy;
  // m_linearVelocity += b2Cross(w, c - oldCenter)
  const float dx = cx - ocx, dy = cy - ocy;
  b.v[0] += -b.w * dy;
  b.v[1] += b.w * dx;
}

b2Fixture* b2Body::CreateFixture(const b2FixtureDef* def) {
  if (!def || !def->shape) return nullptr;
  b2g_fixture f;
  memset(&f, 0, sizeof(f));
  f.shape = def->shape->rec;
  if (f.shape.type == B2G_SHAPE_CIRCLE) {
    const b2CircleShape* c = static_cast<const b2CircleShape*>(def->shape);
    memset(&f.shape, 0, sizeof(f.shape));
    f.shape.type = B2G_SHAPE_CIRCLE;
    f.shape.radius = c->m_radius;
    f.shape.vertices[0][0] = c->m_p.x;
    f.shape.vertices[0][1] = c->m_p.y;
  }
  f.body = m_index;
  f.density = def->density;
  f.friction = def->friction;
  f.restitution = def->restitution;
  f.restitution_threshold = def->restitutionThreshold;
  f.category_bits = def->filter.categoryBits;
  f.mask_bits = def->filter.maskBits;
  f.group_index = def->filter.groupIndex;
  f.is_sensor = def->isSensor ? 1 : 0;
  m_world->fixtures.push_back(f);
  m_world->bodyFixtures[m_index].push_back((int)m_world->fixtures.size() - 1);
  if (f.density > 0.0f) resetMassData(m_world, m_index);
  static b2Fixture handle;
  return &handle;
}

b2Fixture* b2Body::CreateFixture(const b2Shape* shape, float density) {
  b2FixtureDef def;
  def.shape = shape;
  def.density = density;
  return CreateFixture(&def);
}

// ---------------------------------------------------------------- joints
void b2RevoluteJointDef::Initialize(b2Body* bA, b2Body* bB, const b2Vec2& anchor) {
  bodyA = bA;
  bodyB = bB;
  localAnchorA = bodyA->GetLocalPoint(anchor);
  localAnchorB = bodyB->GetLocalPoint(anchor);
  referenceAngle = bodyB->GetAngle() - bodyA->GetAngle();
}

b2Joint* b2World::CreateJoint(const b2JointDef* def) {
  if (!def || !def->bodyA || !def->bodyB || def->type != e_revoluteJoint) return nullptr;
  const b2RevoluteJointDef* r = static_cast<const b2RevoluteJointDef*>(def);
  b2g_joint j;
  memset(&j, 0, sizeof(j));
  j.def.type = B2G_JOINT_REVOLUTE;
  j.def.body_a = def->bodyA->m_index;
  j.def.body_b = def->bodyB->m_index;
  j.def.collide_connected = def->collideConnected ? 1 : 0;
  j.def.user_data = def->userData.pointer;
  j.def.local_anchor_a[0] = r->localAnchorA.x;
  j.def.local_anchor_a[1] = r->localAnchorA.y;
  j.def.local_anchor_b[0] = r->localAnchorB.x;
  j.def.local_anchor_b[1] = r->localAnchorB.y;
  j.def.reference_angle = r->referenceAngle;
  j.def.enable_limit = r->enableLimit;
  j.def.lower = r->lowerAngle;
  j.def.upper = r->upperAngle;
  j.def.enable_motor = r->enableMotor;
  j.def.max_motor = r->maxMotorTorque;
  j.def.motor_speed = r->motorSpeed;
  joints.push_back(j);
  static b2Joint handle;
  return &handle;
}

// ---------------------------------------------------------------- exports
// Runs scene recipe `kind` (0 pyramid(rows = n, density p0, friction p1), 1 mixed drop(n), 2 chains
// over a pile(n chains of 20, p0 circles), 3 batch world(n bodies), with `seed`) into `w`.
static bool build_scene(b2World* w, int32_t kind, uint32_t seed, int32_t n, float p0, float p1, int32_t* counts) {
  b2scenes::ResetTags();
  b2scenes::Counts c;
  if (kind == B2G_SCENE_PYRAMID) c = b2scenes::Pyramid(w, n, p0, p1, true);
  else if (kind == B2G_SCENE_MIXED_DROP) c = b2scenes::MixedDrop(w, n, seed);
  else if (kind == B2G_SCENE_CHAINS) c = b2scenes::ChainsOverPile(w, n, 20, (int)p0, seed);
  else if (kind == B2G_SCENE_BATCH_WORLD) c = b2scenes::BatchWorld(w, seed, n);
  else if (kind == B2G_SCENE_BULLETS) c = b2scenes::Bullets(w, n, seed, p0 > 0.5f);
  else return false;
  if (counts) {
    counts[0] = c.bodies;
    counts[1] = c.fixtures;
    counts[2] = c.joints;
  }
  return true;
}

extern "C" {

// Builds scene `kind` into a new oracle world with gravity (gx, gy). counts[3] = dynamic bodies,
// fixtures, joints. Returns the world handle (orc_world_free), or null for an unknown kind.
void* orc_scene_world(int32_t kind, uint32_t seed, int32_t n, float p0, float p1, float gx, float gy,
                      int32_t* counts) {
  b2World w(b2Vec2(gx, gy));
  if (!build_scene(&w, kind, seed, n, p0, p1, counts)) return nullptr;
  void* h = orc_world_new(gx, gy);
  orc_world_load(h, w.bodies.data(), (int32_t)w.bodies.size(), w.fixtures.data(), (int32_t)w.fixtures.size(),
                 w.joints.data(), (int32_t)w.joints.size(), nullptr, 0, 0.0f);
  return h;
}

// The records scene `kind` makes (for comparison with other builders): sizes[3] receives the
// body, fixture and joint counts; each array is filled when its capacity holds them all.
int32_t orc_scene_records(int32_t kind, uint32_t seed, int32_t n, float p0, float p1, int32_t* sizes, b2g_body* bodies,
                          int32_t nb_cap, b2g_fixture* fixtures, int32_t nf_cap, b2g_joint* joints, int32_t nj_cap) {
  b2World w(b2Vec2(0.0f, -10.0f));
  if (!build_scene(&w, kind, seed, n, p0, p1, nullptr)) return 1;
  sizes[0] = (int32_t)w.bodies.size();
  sizes[1] = (int32_t)w.fixtures.size();
  sizes[2] = (int32_t)w.joints.size();
  if (bodies && nb_cap >= sizes[0]) memcpy(bodies, w.bodies.data(), sizeof(b2g_body) * w.bodies.size());
  if (fixtures && nf_cap >= sizes[1]) memcpy(fixtures, w.fixtures.data(), sizeof(b2g_fixture) * w.fixtures.size());
  if (joints && nj_cap >= sizes[2]) memcpy(joints, w.joints.data(), sizeof(b2g_joint) * w.joints.size());
  return 0;
}

// Body count and gravity of world `seed` of the batched workload (scenes.h BatchBodyCount /
// BatchGravity).
int orc_batch_world_params(uint32_t seed, int32_t* n_bodies, float* gx, float* gy) {
  if (n_bodies) *n_bodies = b2scenes::BatchBodyCount(seed);
  const b2Vec2 g = b2scenes::BatchGravity(seed);
  if (gx) *gx = g.x;
  if (gy) *gy = g.y;
  return 0;
}

}  // extern "C"
