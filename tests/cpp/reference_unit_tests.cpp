// Known-answer tests of the reference's unit-test suite (unit-test/hello_world.cpp,
// joint_test.cpp, world_test.cpp, collision_test.cpp, math_test.cpp), restated against this
// library's b2World facade. The same source also compiles against the reference headers.
// Prints one line per check and exits non-zero on any failure.
#include <stdio.h>

#include "box2d/box2d.h"

static int g_fail = 0;
#define CHECK(cond)                                                          \
  do {                                                                       \
    bool ok_ = (cond);                                                       \
    printf("%s %s:%d %s\n", ok_ ? "PASS" : "FAIL", __func__, __LINE__, #cond); \
    if (!ok_) ++g_fail;                                                      \
  } while (0)

// unit-test/hello_world.cpp
static void hello_world() {
  b2Vec2 gravity(0.0f, -10.0f);
  b2World world(gravity);
  b2BodyDef groundBodyDef;
  groundBodyDef.position.Set(0.0f, -10.0f);
  b2Body* groundBody = world.CreateBody(&groundBodyDef);
  b2PolygonShape groundBox;
  groundBox.SetAsBox(50.0f, 10.0f);
  groundBody->CreateFixture(&groundBox, 0.0f);
  b2BodyDef bodyDef;
  bodyDef.type = b2_dynamicBody;
  bodyDef.position.Set(0.0f, 4.0f);
  b2Body* body = world.CreateBody(&bodyDef);
  b2PolygonShape dynamicBox;
  dynamicBox.SetAsBox(1.0f, 1.0f);
  b2FixtureDef fixtureDef;
  fixtureDef.shape = &dynamicBox;
  fixtureDef.density = 1.0f;
  fixtureDef.friction = 0.3f;
  body->CreateFixture(&fixtureDef);
  float timeStep = 1.0f / 60.0f;
  b2Vec2 position = body->GetPosition();
  float angle = body->GetAngle();
  for (int32 i = 0; i < 60; ++i) {
    world.Step(timeStep, 6, 2);
    position = body->GetPosition();
    angle = body->GetAngle();
  }
  printf("hello_world final %4.2f %4.2f %4.2f\n", position.x, position.y, angle);
  CHECK(b2Abs(position.x) < 0.01f);
  CHECK(b2Abs(position.y - 1.01f) < 0.01f);
  CHECK(b2Abs(angle) < 0.01f);
}

// unit-test/joint_test.cpp
static void joint_reactions() {
  b2Vec2 gravity(0, -10.0f);
  b2World world(gravity);
  b2BodyDef bodyDef;
  b2Body* ground = world.CreateBody(&bodyDef);
  b2CircleShape circle;
  circle.m_radius = 1.0f;
  b2FixtureDef fixtureDef;
  fixtureDef.filter.maskBits = 0;
  fixtureDef.density = 1.0f;
  fixtureDef.shape = &circle;
  bodyDef.type = b2_dynamicBody;
  bodyDef.position.Set(-2.0f, 3.0f);
  b2Body* bodyA = world.CreateBody(&bodyDef);
  b2Body* bodyB = world.CreateBody(&bodyDef);
  b2Body* bodyC = world.CreateBody(&bodyDef);
  b2MassData massData;
  circle.ComputeMass(&massData, fixtureDef.density);
  const float mg = massData.mass * gravity.y;
  bodyA->CreateFixture(&fixtureDef);
  bodyB->CreateFixture(&fixtureDef);
  bodyC->CreateFixture(&fixtureDef);
  b2DistanceJointDef distanceJointDef;
  distanceJointDef.Initialize(ground, bodyA, bodyDef.position + b2Vec2(0.0f, 4.0f), bodyDef.position);
  distanceJointDef.minLength = distanceJointDef.length;
  distanceJointDef.maxLength = distanceJointDef.length;
  b2PrismaticJointDef prismaticJointDef;
  prismaticJointDef.Initialize(ground, bodyB, bodyDef.position, b2Vec2(1.0f, 0.0f));
  b2RevoluteJointDef revoluteJointDef;
  revoluteJointDef.Initialize(ground, bodyC, bodyDef.position);
  b2Joint* distanceJoint = world.CreateJoint(&distanceJointDef);
  b2Joint* prismaticJoint = world.CreateJoint(&prismaticJointDef);
  b2Joint* revoluteJoint = world.CreateJoint(&revoluteJointDef);
  const float timeStep = 1.f / 60.f;
  const float invTimeStep = 60.0f;
  world.Step(timeStep, 6, 2);
  const float tol = 1e-5f;
  {
    b2Vec2 F = distanceJoint->GetReactionForce(invTimeStep);
    float T = distanceJoint->GetReactionTorque(invTimeStep);
    CHECK(F.x == 0.0f);
    CHECK(b2Abs(F.y + mg) < tol);
    CHECK(T == 0.0f);
  }
  {
    b2Vec2 F = prismaticJoint->GetReactionForce(invTimeStep);
    float T = prismaticJoint->GetReactionTorque(invTimeStep);
    CHECK(F.x == 0.0f);
    CHECK(b2Abs(F.y + mg) < tol);
    CHECK(T == 0.0f);
  }
  {
    b2Vec2 F = revoluteJoint->GetReactionForce(invTimeStep);
    float T = revoluteJoint->GetReactionTorque(invTimeStep);
    CHECK(F.x == 0.0f);
    CHECK(b2Abs(F.y + mg) < tol);
    CHECK(T == 0.0f);
  }
}

// unit-test/world_test.cpp
static bool begin_contact = false;
class MyContactListener : public b2ContactListener {
 public:
  void BeginContact(b2Contact* contact) override {
    B2_NOT_USED(contact);
    begin_contact = true;
  }
};
static void world_begin_contact() {
  b2World world(b2Vec2(0.0f, -10.0f));
  MyContactListener listener;
  world.SetContactListener(&listener);
  b2CircleShape circle;
  circle.m_radius = 5.f;
  b2BodyDef bodyDef;
  bodyDef.type = b2_dynamicBody;
  b2Body* bodyA = world.CreateBody(&bodyDef);
  b2Body* bodyB = world.CreateBody(&bodyDef);
  bodyA->CreateFixture(&circle, 0.0f);
  bodyB->CreateFixture(&circle, 0.0f);
  bodyA->SetTransform(b2Vec2(0.f, 0.f), 0.f);
  bodyB->SetTransform(b2Vec2(100.f, 0.f), 0.f);
  world.Step(1.f / 60.f, 6, 2);
  CHECK(world.GetContactListStart() == world.GetContactListEnd());
  CHECK(begin_contact == false);
  bodyB->SetTransform(b2Vec2(1.f, 0.f), 0.f);
  world.Step(1.f / 60.f, 6, 2);
  CHECK(world.GetContactListStart() != world.GetContactListEnd());
  CHECK(begin_contact == true);
}

// unit-test/collision_test.cpp
static void polygon_mass_data() {
  const b2Vec2 center(100.0f, -50.0f);
  const float hx = 0.5f, hy = 1.5f;
  const float angle1 = 0.25f;
  b2PolygonShape polygon1;
  polygon1.SetAsBox(hx, hy, center, angle1);
  const float absTol = 2.0f * b2_epsilon;
  const float relTol = 2.0f * b2_epsilon;
  CHECK(b2Abs(polygon1.m_centroid.x - center.x) < absTol + relTol * b2Abs(center.x));
  CHECK(b2Abs(polygon1.m_centroid.y - center.y) < absTol + relTol * b2Abs(center.y));
  b2Vec2 vertices[4];
  vertices[0].Set(center.x - hx, center.y - hy);
  vertices[1].Set(center.x + hx, center.y - hy);
  vertices[2].Set(center.x - hx, center.y + hy);
  vertices[3].Set(center.x + hx, center.y + hy);
  b2PolygonShape polygon2;
  polygon2.Set(vertices, 4);
  CHECK(b2Abs(polygon2.m_centroid.x - center.x) < absTol + relTol * b2Abs(center.x));
  CHECK(b2Abs(polygon2.m_centroid.y - center.y) < absTol + relTol * b2Abs(center.y));
  const float mass = 4.0f * hx * hy;
  const float inertia = (mass / 3.0f) * (hx * hx + hy * hy) + mass * b2Dot(center, center);
  b2MassData massData1;
  polygon1.ComputeMass(&massData1, 1.0f);
  CHECK(b2Abs(massData1.center.x - center.x) < absTol + relTol * b2Abs(center.x));
  CHECK(b2Abs(massData1.center.y - center.y) < absTol + relTol * b2Abs(center.y));
  CHECK(b2Abs(massData1.mass - mass) < 20.0f * (absTol + relTol * mass));
  CHECK(b2Abs(massData1.I - inertia) < 40.0f * (absTol + relTol * inertia));
  b2MassData massData2;
  polygon2.ComputeMass(&massData2, 1.0f);
  CHECK(b2Abs(massData2.center.x - center.x) < absTol + relTol * b2Abs(center.x));
  CHECK(b2Abs(massData2.center.y - center.y) < absTol + relTol * b2Abs(center.y));
  CHECK(b2Abs(massData2.mass - mass) < 20.0f * (absTol + relTol * mass));
  CHECK(b2Abs(massData2.I - inertia) < 40.0f * (absTol + relTol * inertia));
}

// unit-test/math_test.cpp
static void sweep_transform() {
  b2Sweep sweep;
  sweep.localCenter.SetZero();
  sweep.c0.Set(-2.0f, 4.0f);
  sweep.c.Set(3.0f, 8.0f);
  sweep.a0 = 0.5f;
  sweep.a = 5.0f;
  sweep.alpha0 = 0.0f;
  b2Transform transform;
  sweep.GetTransform(&transform, 0.0f);
  CHECK(transform.p.x == sweep.c0.x);
  CHECK(transform.p.y == sweep.c0.y);
  CHECK(transform.q.c == cosf(sweep.a0));
  CHECK(transform.q.s == sinf(sweep.a0));
  sweep.GetTransform(&transform, 1.0f);
  CHECK(transform.p.x == sweep.c.x);
  CHECK(transform.p.y == sweep.c.y);
  CHECK(transform.q.c == cosf(sweep.a));
  CHECK(transform.q.s == sinf(sweep.a));
}

// b2World::DestroyBody / DestroyJoint, b2Body::DestroyFixture with a contact listener and a
// destruction listener (the reference's semantics: src/dynamics/b2_world.cpp:178-410,
// b2_body.cpp:280-350): EndContact for the touching contacts of a destroyed body before the call
// returns, SayGoodbye for the joints and fixtures it takes along, counts and lists updated, the
// world steps on without it.
struct CountingListener : public b2ContactListener {
  int begins = 0, ends = 0;
  void BeginContact(b2Contact* contact) override { B2_NOT_USED(contact); ++begins; }
  void EndContact(b2Contact* contact) override { B2_NOT_USED(contact); ++ends; }
};
struct Goodbyes : public b2DestructionListener {
  int joints = 0, fixtures = 0;
  void SayGoodbye(b2Joint* joint) override { B2_NOT_USED(joint); ++joints; }
  void SayGoodbye(b2Fixture* fixture) override { B2_NOT_USED(fixture); ++fixtures; }
};
static void destroy_calls() {
  b2World world(b2Vec2(0.0f, -10.0f));
  world.SetAllowSleeping(false);
  CountingListener listener;
  Goodbyes goodbyes;
  world.SetContactListener(&listener);
  world.SetDestructionListener(&goodbyes);
  b2BodyDef gd;
  b2Body* ground = world.CreateBody(&gd);
  b2EdgeShape edge;
  edge.SetTwoSided(b2Vec2(-20.0f, 0.0f), b2Vec2(20.0f, 0.0f));
  ground->CreateFixture(&edge, 0.0f);
  b2PolygonShape box;
  box.SetAsBox(0.5f, 0.5f);
  b2Body* stack[3];
  for (int i = 0; i < 3; ++i) {
    b2BodyDef bd;
    bd.type = b2_dynamicBody;
    bd.position.Set(0.0f, 0.5f + 1.0f * (float)i);
    stack[i] = world.CreateBody(&bd);
    stack[i]->CreateFixture(&box, 1.0f);
  }
  b2BodyDef pd;
  pd.type = b2_dynamicBody;
  pd.position.Set(5.0f, 3.0f);
  b2Body* pendulum = world.CreateBody(&pd);
  pendulum->CreateFixture(&box, 1.0f);
  b2RevoluteJointDef jd;
  jd.Initialize(ground, pendulum, b2Vec2(5.0f, 5.0f));
  b2Joint* joint = world.CreateJoint(&jd);
  for (int i = 0; i < 60; ++i) world.Step(1.0f / 60.0f, 8, 3);
  CHECK(listener.begins >= 3);
  const int ends0 = listener.ends;
  const float topY = stack[2]->GetPosition().y;
  world.DestroyBody(stack[0]);  // touching the ground and the middle box
  CHECK(listener.ends - ends0 == 2);
  CHECK(goodbyes.fixtures == 1 && goodbyes.joints == 0);
  CHECK(world.GetBodyCount() == 4);
  int listed = 0;
  for (b2Body* b = world.GetBodyList(); b; b = b->GetNext()) ++listed;
  CHECK(listed == 4);
  for (int i = 0; i < 60; ++i) world.Step(1.0f / 60.0f, 8, 3);
  CHECK(stack[2]->GetPosition().y < topY - 0.9f);  // the two boxes above fell by a box height
  world.DestroyJoint(joint);
  CHECK(world.GetJointCount() == 0);
  for (int i = 0; i < 30; ++i) world.Step(1.0f / 60.0f, 8, 3);
  CHECK(pendulum->GetPosition().y < 3.0f - 0.5f);  // released: it falls
  stack[2]->DestroyFixture(stack[2]->GetFixtureList());
  CHECK(stack[2]->GetFixtureList() == nullptr);
  CHECK(world.GetProxyCount() == 3);
}

#ifdef B2G_API
// This engine's extension: a b2ContactFilter subclass cannot run on the GPU, so Step refuses to
// advance with one set (LastStatus() = B2G_E_INVALID_ARG); the default filter is accepted.
struct NoCollide : public b2ContactFilter {
  bool ShouldCollide(b2Fixture* a, b2Fixture* b) override { B2_NOT_USED(a); B2_NOT_USED(b); return false; }
};
static void custom_filter_refused() {
  b2World world(b2Vec2(0.0f, -10.0f));
  b2BodyDef bd;
  bd.type = b2_dynamicBody;
  bd.position.Set(0.0f, 4.0f);
  b2Body* body = world.CreateBody(&bd);
  b2CircleShape c;
  c.m_radius = 0.5f;
  body->CreateFixture(&c, 1.0f);
  NoCollide filter;
  world.SetContactFilter(&filter);
  world.Step(1.0f / 60.0f, 8, 3);
  CHECK(world.LastStatus() == B2G_E_INVALID_ARG);
  CHECK(body->GetPosition().y == 4.0f);
  b2ContactFilter plain;
  world.SetContactFilter(&plain);
  world.Step(1.0f / 60.0f, 8, 3);
  CHECK(world.LastStatus() == B2G_OK);
  CHECK(body->GetPosition().y < 4.0f);
}
#endif

int main(int argc, char** argv) {
  bool host_only = argc > 1;
  polygon_mass_data();
  sweep_transform();
  if (!host_only) {
    hello_world();
    joint_reactions();
    world_begin_contact();
    destroy_calls();
#ifdef B2G_API
    custom_filter_refused();
#endif
  }
  printf("%s: %d failures\n", g_fail ? "FAILED" : "OK", g_fail);
  return g_fail ? 1 : 0;
}
