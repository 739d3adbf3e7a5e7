// The oracle's scene-building API: the slice of the Box2D C++ API that the batched scene recipes
// (box2d-optimized_gb300/scenes/scenes.h) call, restated over the oracle's own world records, so
// that the CPU oracle builds the benchmark worlds without the engine library. Test
// infrastructure only (the CPU baseline and the reference-arm timing); nothing in the engine uses
// it.
//
// What each call computes follows the reference (and the engine's facade, which is pinned to it
// byte for byte), in the same operation order:
//   b2World::CreateBody        src/dynamics/b2_body.cpp:29-122  (transform from sinf/cosf)
//   b2Body::CreateFixture      src/dynamics/b2_body.cpp:230-269 (shape clone, ResetMassData)
//   b2Body::ResetMassData      src/dynamics/b2_body.cpp:352-416 (fixtures newest first)
//   b2PolygonShape::Set/SetAsBox src/collision/b2_polygon_shape.cpp:36-243
//   b2EdgeShape::SetTwoSided   src/collision/b2_edge_shape.cpp:36-42
//   b2RevoluteJointDef::Initialize src/dynamics/b2_revolute_joint.cpp:38-45
// Polygon hulls and shape mass data come from the oracle's restatements (orc_polygon_set,
// orc_polygon_box, orc_shape_mass), which are pinned to the reference's.
#pragma once

#include <math.h>
#include <stdint.h>

#include <vector>

#include "../../../include/b2g_capi.h"

#define b2_pi 3.14159265359f
#define b2_maxPolygonVertices 8
#define b2_linearSlop 0.005f
#define b2_polygonRadius (2.0f * b2_linearSlop)
typedef int32_t int32;

struct b2Vec2 {
  b2Vec2() : x(0.0f), y(0.0f) {}
  b2Vec2(float xIn, float yIn) : x(xIn), y(yIn) {}
  void Set(float x_, float y_) { x = x_; y = y_; }
  void SetZero() { x = 0.0f; y = 0.0f; }
  void operator+=(const b2Vec2& v) { x += v.x; y += v.y; }
  void operator-=(const b2Vec2& v) { x -= v.x; y -= v.y; }
  void operator*=(float a) { x *= a; y *= a; }
  float x, y;
};
inline b2Vec2 operator+(const b2Vec2& a, const b2Vec2& b) { return b2Vec2(a.x + b.x, a.y + b.y); }
inline b2Vec2 operator-(const b2Vec2& a, const b2Vec2& b) { return b2Vec2(a.x - b.x, a.y - b.y); }
inline b2Vec2 operator*(float s, const b2Vec2& a) { return b2Vec2(s * a.x, s * a.y); }

struct b2BodyUserData {
  uintptr_t pointer = 0;
};
struct b2FixtureUserData {
  uintptr_t pointer = 0;
};
struct b2JointUserData {
  uintptr_t pointer = 0;
};

enum b2BodyType { b2_staticBody = 0, b2_kinematicBody, b2_dynamicBody };

struct b2BodyDef {
  b2BodyType type = b2_staticBody;
  b2Vec2 position;
  float angle = 0.0f;
  b2Vec2 linearVelocity;
  float angularVelocity = 0.0f;
  float linearDamping = 0.0f;
  float angularDamping = 0.0f;
  bool allowSleep = true;
  bool awake = true;
  bool fixedRotation = false;
  bool bullet = false;
  bool enabled = true;
  b2BodyUserData userData;
  float gravityScale = 1.0f;
};

struct b2Filter {
  uint16_t categoryBits = 0x0001;
  uint16_t maskBits = 0xFFFF;
  int16_t groupIndex = 0;
};

// A shape is its engine record (b2g_shape).
class b2Shape {
 public:
  b2g_shape rec = {};
};

class b2CircleShape : public b2Shape {
 public:
  b2CircleShape() { rec.type = B2G_SHAPE_CIRCLE; }
  float m_radius = 0.0f;
  b2Vec2 m_p;
};

class b2EdgeShape : public b2Shape {
 public:
  b2EdgeShape() {
    rec.type = B2G_SHAPE_EDGE;
    rec.radius = b2_polygonRadius;
  }
  void SetTwoSided(const b2Vec2& v1, const b2Vec2& v2);
};

class b2PolygonShape : public b2Shape {
 public:
  b2PolygonShape() {
    rec.type = B2G_SHAPE_POLYGON;
    rec.radius = b2_polygonRadius;
  }
  void Set(const b2Vec2* points, int32 count);
  void SetAsBox(float hx, float hy);
  void SetAsBox(float hx, float hy, const b2Vec2& center, float angle);
};

struct b2FixtureDef {
  const b2Shape* shape = nullptr;
  b2FixtureUserData userData;
  float friction = 0.2f;
  float restitution = 0.0f;
  float restitutionThreshold = 1.0f;
  float density = 0.0f;
  bool isSensor = false;
  b2Filter filter;
};

class b2World;
class b2Fixture {};

class b2Body {
 public:
  b2Fixture* CreateFixture(const b2FixtureDef* def);
  b2Fixture* CreateFixture(const b2Shape* shape, float density);
  b2Vec2 GetPosition() const;
  float GetAngle() const;
  b2Vec2 GetLocalPoint(const b2Vec2& worldPoint) const;

  b2World* m_world = nullptr;
  int m_index = -1;
};

enum b2JointType { e_unknownJoint, e_revoluteJoint };

struct b2JointDef {
  b2JointType type = e_unknownJoint;
  b2JointUserData userData;
  b2Body* bodyA = nullptr;
  b2Body* bodyB = nullptr;
  bool collideConnected = false;
};

struct b2RevoluteJointDef : public b2JointDef {
  b2RevoluteJointDef() { type = e_revoluteJoint; }
  void Initialize(b2Body* bA, b2Body* bB, const b2Vec2& anchor);
  b2Vec2 localAnchorA, localAnchorB;
  float referenceAngle = 0.0f;
  bool enableLimit = false;
  float lowerAngle = 0.0f, upperAngle = 0.0f;
  bool enableMotor = false;
  float motorSpeed = 0.0f;
  float maxMotorTorque = 0.0f;
};

class b2Joint {};

// A world under construction: the engine's body, fixture and joint records in creation order.
class b2World {
 public:
  explicit b2World(const b2Vec2& gravity) : m_gravity(gravity) {}
  b2Body* CreateBody(const b2BodyDef* def);
  b2Joint* CreateJoint(const b2JointDef* def);

  b2Vec2 m_gravity;
  std::vector<b2g_body> bodies;
  std::vector<b2g_fixture> fixtures;
  std::vector<b2g_joint> joints;
  std::vector<std::vector<int>> bodyFixtures;  // per body, fixture indices in creation order
  std::vector<b2Body*> handles;
  ~b2World() {
    for (b2Body* b : handles) delete b;
  }
};
