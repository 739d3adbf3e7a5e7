// box2d/box2d.h - drop-in C++ facade of the GB300 Step engine.
//
// Keeps the reference's public API for the Step path (include/box2d/b2_world.h, b2_body.h,
// b2_fixture.h, b2_joint.h, b2_revolute_joint.h, b2_prismatic_joint.h, b2_distance_joint.h,
// b2_contact.h, b2_world_callbacks.h, b2_collision.h, b2_*_shape.h, b2_math.h): same class names,
// member names and signatures, so code written against box2d-optimized compiles against it.
// Every call goes through the C ABI in include/b2g_capi.h; the simulation runs on the GPU.
//
// Differences from the reference, by design:
//  * Contact listener callbacks are delivered as a batch after each Step, grouped per world and
//    sorted by kind (Begin, End, PreSolve, PostSolve), then fixture pair; the set of callbacks of
//    a step is the reference's. A PreSolve that disables a contact takes effect from the next
//    step. Worlds stepped together through b2g_step deliver with b2World::DeliverEvents.
//  * Custom b2ContactFilter subclasses cannot run on the GPU: SetContactFilter with one makes the
//    next Step fail (LastStatus() = B2G_E_INVALID_ARG, the world does not advance); the default
//    filter (group / category / mask) always applies.
//  * Continuous collision (SolveTOI) runs on the GPU for bullets and kinematic bodies, as in the
//    reference (on by default); contacts it makes inside its loop are remade by the pair update
//    after it. Particle systems are not part of this engine. Sleeping is (the world allows it by
//    default, like the reference).
//  * Sine/cosine inside the step come from a portable routine (identical on host and GPU), so
//    trajectories agree with the reference to rounding, not bit for bit.
#pragma once

#include <float.h>
#include <math.h>
#include <stdint.h>

#include <deque>
#include <memory>
#include <vector>

#include "../../../include/b2g_capi.h"

typedef signed char int8;
typedef signed short int16;
typedef signed int int32;
typedef unsigned char uint8;
typedef unsigned short uint16;
typedef unsigned int uint32;
typedef float float32;

#define b2_maxFloat FLT_MAX
#define b2_epsilon FLT_EPSILON
#define b2_pi 3.14159265359f
#define b2_lengthUnitsPerMeter 1.0f
#define b2_maxPolygonVertices 8
#define b2_maxManifoldPoints 2
#define b2_linearSlop (0.005f * b2_lengthUnitsPerMeter)
#define b2_angularSlop (2.0f / 180.0f * b2_pi)
#define b2_polygonRadius (2.0f * b2_linearSlop)
#define b2Assert(A) ((void)0)
#define B2_NOT_USED(x) ((void)(x))

// ---------------------------------------------------------------- math (include/box2d/b2_math.h)
inline bool b2IsValid(float x) { return isfinite(x); }
#define b2Sqrt(x) sqrtf(x)
#define b2Atan2(y, x) atan2f(y, x)

struct b2Vec2 {
  b2Vec2() {}
  b2Vec2(float xIn, float yIn) : x(xIn), y(yIn) {}
  void SetZero() { x = 0.0f; y = 0.0f; }
  void Set(float x_, float y_) { x = x_; y = y_; }
  b2Vec2 operator-() const { return b2Vec2(-x, -y); }
  float operator()(int32 i) const { return (&x)[i]; }
  float& operator()(int32 i) { return (&x)[i]; }
  void operator+=(const b2Vec2& v) { x += v.x; y += v.y; }
  void operator-=(const b2Vec2& v) { x -= v.x; y -= v.y; }
  void operator*=(float a) { x *= a; y *= a; }
  void operator/=(float a) { x /= a; y /= a; }
  float Length() const { return b2Sqrt(x * x + y * y); }
  float LengthSquared() const { return x * x + y * y; }
  float Normalize() {
    float length = Length();
    if (length < b2_epsilon) return 0.0f;
    float invLength = 1.0f / length;
    x *= invLength;
    y *= invLength;
    return length;
  }
  bool IsValid() const { return b2IsValid(x) && b2IsValid(y); }
  b2Vec2 Skew() const { return b2Vec2(-y, x); }
  float x, y;
};

struct b2Vec3 {
  b2Vec3() {}
  b2Vec3(float xIn, float yIn, float zIn) : x(xIn), y(yIn), z(zIn) {}
  void SetZero() { x = 0.0f; y = 0.0f; z = 0.0f; }
  void Set(float x_, float y_, float z_) { x = x_; y = y_; z = z_; }
  b2Vec3 operator-() const { return b2Vec3(-x, -y, -z); }
  float x, y, z;
};

struct b2Mat22 {
  b2Mat22() {}
  b2Mat22(const b2Vec2& c1, const b2Vec2& c2) : ex(c1), ey(c2) {}
  void Set(const b2Vec2& c1, const b2Vec2& c2) { ex = c1; ey = c2; }
  void SetIdentity() { ex.Set(1.0f, 0.0f); ey.Set(0.0f, 1.0f); }
  void SetZero() { ex.SetZero(); ey.SetZero(); }
  b2Mat22 GetInverse() const {
    float a = ex.x, b = ey.x, c = ex.y, d = ey.y;
    b2Mat22 B;
    float det = a * d - b * c;
    if (det != 0.0f) det = 1.0f / det;
    B.ex.x = det * d; B.ey.x = -det * b;
    B.ex.y = -det * c; B.ey.y = det * a;
    return B;
  }
  b2Vec2 Solve(const b2Vec2& b) const {
    float a11 = ex.x, a12 = ey.x, a21 = ex.y, a22 = ey.y;
    float det = a11 * a22 - a12 * a21;
    if (det != 0.0f) det = 1.0f / det;
    return b2Vec2(det * (a22 * b.x - a12 * b.y), det * (a11 * b.y - a21 * b.x));
  }
  b2Vec2 ex, ey;
};

struct b2Rot {
  b2Rot() {}
  explicit b2Rot(float angle) { s = sinf(angle); c = cosf(angle); }
  void Set(float angle) { s = sinf(angle); c = cosf(angle); }
  void SetIdentity() { s = 0.0f; c = 1.0f; }
  float GetAngle() const { return b2Atan2(s, c); }
  b2Vec2 GetXAxis() const { return b2Vec2(c, s); }
  b2Vec2 GetYAxis() const { return b2Vec2(-s, c); }
  float s, c;
};

struct b2Transform {
  b2Transform() {}
  b2Transform(const b2Vec2& position, const b2Rot& rotation) : p(position), q(rotation) {}
  void SetIdentity() { p.SetZero(); q.SetIdentity(); }
  void Set(const b2Vec2& position, float angle) { p = position; q.Set(angle); }
  b2Vec2 p;
  b2Rot q;
};

struct b2Sweep {
  void GetTransform(b2Transform* xf, float beta) const;
  void Advance(float alpha);
  void Normalize();
  b2Vec2 localCenter;
  b2Vec2 c0, c;
  float a0, a;
  float alpha0;
};

extern const b2Vec2 b2Vec2_zero;

inline float b2Dot(const b2Vec2& a, const b2Vec2& b) { return a.x * b.x + a.y * b.y; }
inline float b2Cross(const b2Vec2& a, const b2Vec2& b) { return a.x * b.y - a.y * b.x; }
inline b2Vec2 b2Cross(const b2Vec2& a, float s) { return b2Vec2(s * a.y, -s * a.x); }
inline b2Vec2 b2Cross(float s, const b2Vec2& a) { return b2Vec2(-s * a.y, s * a.x); }
inline b2Vec2 b2Mul(const b2Mat22& A, const b2Vec2& v) { return b2Vec2(A.ex.x * v.x + A.ey.x * v.y, A.ex.y * v.x + A.ey.y * v.y); }
inline b2Vec2 b2MulT(const b2Mat22& A, const b2Vec2& v) { return b2Vec2(b2Dot(v, A.ex), b2Dot(v, A.ey)); }
inline b2Vec2 operator+(const b2Vec2& a, const b2Vec2& b) { return b2Vec2(a.x + b.x, a.y + b.y); }
inline b2Vec2 operator-(const b2Vec2& a, const b2Vec2& b) { return b2Vec2(a.x - b.x, a.y - b.y); }
inline b2Vec2 operator*(float s, const b2Vec2& a) { return b2Vec2(s * a.x, s * a.y); }
inline b2Vec2 operator/(const b2Vec2& v, float f) { return b2Vec2(v.x / f, v.y / f); }
inline bool operator==(const b2Vec2& a, const b2Vec2& b) { return a.x == b.x && a.y == b.y; }
inline bool operator!=(const b2Vec2& a, const b2Vec2& b) { return a.x != b.x || a.y != b.y; }
inline float b2Distance(const b2Vec2& a, const b2Vec2& b) { return (a - b).Length(); }
inline float b2DistanceSquared(const b2Vec2& a, const b2Vec2& b) { b2Vec2 c = a - b; return b2Dot(c, c); }
inline b2Vec3 operator*(float s, const b2Vec3& a) { return b2Vec3(s * a.x, s * a.y, s * a.z); }
inline b2Vec3 operator+(const b2Vec3& a, const b2Vec3& b) { return b2Vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline b2Vec3 operator-(const b2Vec3& a, const b2Vec3& b) { return b2Vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline float b2Dot(const b2Vec3& a, const b2Vec3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline b2Vec3 b2Cross(const b2Vec3& a, const b2Vec3& b) {
  return b2Vec3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline b2Rot b2Mul(const b2Rot& q, const b2Rot& r) {
  b2Rot qr; qr.s = q.s * r.c + q.c * r.s; qr.c = q.c * r.c - q.s * r.s; return qr;
}
inline b2Rot b2MulT(const b2Rot& q, const b2Rot& r) {
  b2Rot qr; qr.s = q.c * r.s - q.s * r.c; qr.c = q.c * r.c + q.s * r.s; return qr;
}
inline b2Vec2 b2Mul(const b2Rot& q, const b2Vec2& v) { return b2Vec2(q.c * v.x - q.s * v.y, q.s * v.x + q.c * v.y); }
inline b2Vec2 b2MulT(const b2Rot& q, const b2Vec2& v) { return b2Vec2(q.c * v.x + q.s * v.y, -q.s * v.x + q.c * v.y); }
inline b2Vec2 b2Mul(const b2Transform& T, const b2Vec2& v) {
  float x = (T.q.c * v.x - T.q.s * v.y) + T.p.x;
  float y = (T.q.s * v.x + T.q.c * v.y) + T.p.y;
  return b2Vec2(x, y);
}
inline b2Vec2 b2MulT(const b2Transform& T, const b2Vec2& v) {
  float px = v.x - T.p.x, py = v.y - T.p.y;
  return b2Vec2(T.q.c * px + T.q.s * py, -T.q.s * px + T.q.c * py);
}
inline b2Transform b2Mul(const b2Transform& A, const b2Transform& B) {
  b2Transform C; C.q = b2Mul(A.q, B.q); C.p = b2Mul(A.q, B.p) + A.p; return C;
}
inline b2Transform b2MulT(const b2Transform& A, const b2Transform& B) {
  b2Transform C; C.q = b2MulT(A.q, B.q); C.p = b2MulT(A.q, B.p - A.p); return C;
}
template <typename T> inline T b2Abs(T a) { return a > T(0) ? a : -a; }
inline b2Vec2 b2Abs(const b2Vec2& a) { return b2Vec2(b2Abs(a.x), b2Abs(a.y)); }
template <typename T> inline T b2Min(T a, T b) { return a < b ? a : b; }
inline b2Vec2 b2Min(const b2Vec2& a, const b2Vec2& b) { return b2Vec2(b2Min(a.x, b.x), b2Min(a.y, b.y)); }
template <typename T> inline T b2Max(T a, T b) { return a > b ? a : b; }
inline b2Vec2 b2Max(const b2Vec2& a, const b2Vec2& b) { return b2Vec2(b2Max(a.x, b.x), b2Max(a.y, b.y)); }
template <typename T> inline T b2Clamp(T a, T low, T high) { return b2Max(low, b2Min(a, high)); }
template <typename T> inline void b2Swap(T& a, T& b) { T tmp = a; a = b; b = tmp; }

inline void b2Sweep::GetTransform(b2Transform* xf, float beta) const {
  xf->p = (1.0f - beta) * c0 + beta * c;
  float angle = (1.0f - beta) * a0 + beta * a;
  xf->q.Set(angle);
  xf->p -= b2Mul(xf->q, localCenter);
}
inline void b2Sweep::Advance(float alpha) {
  float beta = (alpha - alpha0) / (1.0f - alpha0);
  c0 += beta * (c - c0);
  a0 += beta * (a - a0);
  alpha0 = alpha;
}
inline void b2Sweep::Normalize() {
  float twoPi = 2.0f * b2_pi;
  float d = twoPi * floorf(a0 / twoPi);
  a0 -= d;
  a -= d;
}

// ---------------------------------------------------------------- collision types
struct b2AABB {
  bool IsValid() const { return lowerBound.IsValid() && upperBound.IsValid(); }
  b2Vec2 GetCenter() const { return 0.5f * (lowerBound + upperBound); }
  b2Vec2 GetExtents() const { return 0.5f * (upperBound - lowerBound); }
  void Combine(const b2AABB& a) { lowerBound = b2Min(lowerBound, a.lowerBound); upperBound = b2Max(upperBound, a.upperBound); }
  b2Vec2 lowerBound, upperBound;
};
inline bool b2TestOverlap(const b2AABB& a, const b2AABB& b) {
  return (a.upperBound.x >= b.lowerBound.x) & (a.lowerBound.x <= b.upperBound.x) &
         (a.upperBound.y >= b.lowerBound.y) & (a.lowerBound.y <= b.upperBound.y);
}

struct b2ContactFeature {
  enum Type { e_vertex = 0, e_face = 1 };
  uint8 indexA, indexB, typeA, typeB;
};
union b2ContactID {
  b2ContactFeature cf;
  uint32 key;
};
struct b2ManifoldPoint {
  b2Vec2 localPoint;
  float normalImpulse;
  float tangentImpulse;
  b2ContactID id;
};
struct b2Manifold {
  enum Type { e_circles, e_faceA, e_faceB };
  b2ManifoldPoint points[b2_maxManifoldPoints];
  b2Vec2 localNormal;
  b2Vec2 localPoint;
  Type type;
  int32 pointCount;
};
struct b2WorldManifold {
  void Initialize(const b2Manifold* manifold, const b2Transform& xfA, float radiusA, const b2Transform& xfB,
                  float radiusB);
  b2Vec2 normal;
  b2Vec2 points[b2_maxManifoldPoints];
  float separations[b2_maxManifoldPoints];
};
struct b2MassData {
  float mass;
  b2Vec2 center;
  float I;
};

// ---------------------------------------------------------------- shapes
class b2Shape {
 public:
  enum Type { e_circle = 0, e_edge = 1, e_polygon = 2, e_chain = 3, e_typeCount = 4 };
  virtual ~b2Shape() {}
  Type GetType() const { return m_type; }
  virtual int32 GetChildCount() const { return 1; }
  virtual void ComputeAABB(b2AABB* aabb, const b2Transform& xf) const = 0;
  virtual void ComputeMass(b2MassData* massData, float density) const = 0;
  virtual void ToRecord(b2g_shape* out) const = 0;
  Type m_type;
  float m_radius;
};

class b2CircleShape : public b2Shape {
 public:
  b2CircleShape() { m_type = e_circle; m_radius = 0.0f; m_p.SetZero(); }
  void ComputeAABB(b2AABB* aabb, const b2Transform& xf) const override;
  void ComputeMass(b2MassData* massData, float density) const override;
  void ToRecord(b2g_shape* out) const override;
  b2Vec2 m_p;
};

class b2EdgeShape : public b2Shape {
 public:
  b2EdgeShape() {
    m_type = e_edge; m_radius = b2_polygonRadius;
    m_vertex0.SetZero(); m_vertex1.SetZero(); m_vertex2.SetZero(); m_vertex3.SetZero(); m_oneSided = false;
  }
  void SetOneSided(const b2Vec2& v0, const b2Vec2& v1, const b2Vec2& v2, const b2Vec2& v3) {
    m_vertex0 = v0; m_vertex1 = v1; m_vertex2 = v2; m_vertex3 = v3; m_oneSided = true;
  }
  void SetTwoSided(const b2Vec2& v1, const b2Vec2& v2) { m_vertex1 = v1; m_vertex2 = v2; m_oneSided = false; }
  void ComputeAABB(b2AABB* aabb, const b2Transform& xf) const override;
  void ComputeMass(b2MassData* massData, float density) const override;
  void ToRecord(b2g_shape* out) const override;
  b2Vec2 m_vertex1, m_vertex2;
  b2Vec2 m_vertex0, m_vertex3;
  bool m_oneSided;
};

class b2PolygonShape : public b2Shape {
 public:
  b2PolygonShape() { m_type = e_polygon; m_radius = b2_polygonRadius; m_count = 0; m_centroid.SetZero(); }
  void Set(const b2Vec2* points, int32 count);
  void SetAsBox(float hx, float hy);
  void SetAsBox(float hx, float hy, const b2Vec2& center, float angle);
  bool Validate() const { return m_count >= 3; }
  void ComputeAABB(b2AABB* aabb, const b2Transform& xf) const override;
  void ComputeMass(b2MassData* massData, float density) const override;
  void ToRecord(b2g_shape* out) const override;
  b2Vec2 m_centroid;
  b2Vec2 m_vertices[b2_maxPolygonVertices];
  b2Vec2 m_normals[b2_maxPolygonVertices];
  int32 m_count;
};

// ---------------------------------------------------------------- bodies and fixtures
class b2World;
class b2Body;
class b2Fixture;
class b2Joint;
class b2Contact;

enum b2BodyType { b2_staticBody = 0, b2_kinematicBody, b2_dynamicBody };

struct b2BodyUserData { b2BodyUserData() : pointer(0) {} uintptr_t pointer; };
struct b2FixtureUserData { b2FixtureUserData() : pointer(0) {} uintptr_t pointer; };
struct b2JointUserData { b2JointUserData() : pointer(0) {} uintptr_t pointer; };

struct b2BodyDef {
  b2BodyDef() {
    position.Set(0.0f, 0.0f); angle = 0.0f; linearVelocity.Set(0.0f, 0.0f); angularVelocity = 0.0f;
    linearDamping = 0.0f; angularDamping = 0.0f; allowSleep = true; awake = true; fixedRotation = false;
    bullet = false; type = b2_staticBody; enabled = true; gravityScale = 1.0f;
  }
  b2BodyType type;
  b2Vec2 position;
  float angle;
  b2Vec2 linearVelocity;
  float angularVelocity;
  float linearDamping;
  float angularDamping;
  bool allowSleep;
  bool awake;
  bool fixedRotation;
  bool bullet;
  bool enabled;
  b2BodyUserData userData;
  float gravityScale;
};

struct b2Filter {
  b2Filter() : categoryBits(0x0001), maskBits(0xFFFF), groupIndex(0) {}
  uint16 categoryBits;
  uint16 maskBits;
  int16 groupIndex;
};

struct b2FixtureDef {
  b2FixtureDef() : shape(nullptr), friction(0.2f), restitution(0.0f), restitutionThreshold(1.0f), density(0.0f), isSensor(false) {}
  const b2Shape* shape;
  b2FixtureUserData userData;
  float friction;
  float restitution;
  float restitutionThreshold;
  float density;
  bool isSensor;
  b2Filter filter;
};

class b2Fixture {
 public:
  b2Shape::Type GetType() const { return (b2Shape::Type)m_shapeType; }
  b2Shape* GetShape();
  const b2Shape* GetShape() const;
  bool IsSensor() const { return m_isSensor; }
  const b2Filter& GetFilterData() const { return m_filter; }
  b2Body* GetBody() { return m_body; }
  const b2Body* GetBody() const { return m_body; }
  b2Fixture* GetNext() { return m_next; }
  const b2Fixture* GetNext() const { return m_next; }
  b2FixtureUserData& GetUserData() { return m_userData; }
  float GetDensity() const { return m_density; }
  float GetFriction() const { return m_friction; }
  float GetRestitution() const { return m_restitution; }
  float GetRestitutionThreshold() const { return m_restitutionThreshold; }
  void GetMassData(b2MassData* massData) const;
  int32 GetIndex() const { return m_index; }

  b2Body* m_body = nullptr;
  b2Fixture* m_next = nullptr;
  int32 m_index = 0;
  int32 m_shapeType = 0;
  std::unique_ptr<b2Shape> m_shape;
  float m_density = 0, m_friction = 0, m_restitution = 0, m_restitutionThreshold = 0;
  bool m_isSensor = false;
  b2Filter m_filter;
  b2FixtureUserData m_userData;
};

class b2Body {
 public:
  b2Fixture* CreateFixture(const b2FixtureDef* def);
  b2Fixture* CreateFixture(const b2Shape* shape, float density);
  // b2Body::DestroyFixture (src/dynamics/b2_body.cpp:280-350): its contacts end (EndContact for
  // the touching ones, before this returns) and the body's mass data is reset.
  void DestroyFixture(b2Fixture* fixture);
  void SetTransform(const b2Vec2& position, float angle);
  const b2Transform& GetTransform() const;
  const b2Vec2& GetPosition() const { return GetTransform().p; }
  float GetAngle() const;
  const b2Vec2& GetWorldCenter() const;
  const b2Vec2& GetLocalCenter() const;
  void SetLinearVelocity(const b2Vec2& v);
  const b2Vec2& GetLinearVelocity() const;
  void SetAngularVelocity(float omega);
  float GetAngularVelocity() const;
  void ApplyForce(const b2Vec2& force, const b2Vec2& point, bool wake);
  void ApplyForceToCenter(const b2Vec2& force, bool wake);
  void ApplyTorque(float torque, bool wake);
  void ApplyLinearImpulse(const b2Vec2& impulse, const b2Vec2& point, bool wake);
  void ApplyLinearImpulseToCenter(const b2Vec2& impulse, bool wake);
  void ApplyAngularImpulse(float impulse, bool wake);
  float GetMass() const;
  float GetInertia() const;
  void GetMassData(b2MassData* data) const;
  b2Vec2 GetWorldPoint(const b2Vec2& localPoint) const { return b2Mul(GetTransform(), localPoint); }
  b2Vec2 GetWorldVector(const b2Vec2& localVector) const { return b2Mul(GetTransform().q, localVector); }
  b2Vec2 GetLocalPoint(const b2Vec2& worldPoint) const { return b2MulT(GetTransform(), worldPoint); }
  b2Vec2 GetLocalVector(const b2Vec2& worldVector) const { return b2MulT(GetTransform().q, worldVector); }
  b2Vec2 GetLinearVelocityFromWorldPoint(const b2Vec2& worldPoint) const {
    return GetLinearVelocity() + b2Cross(GetAngularVelocity(), worldPoint - GetWorldCenter());
  }
  b2BodyType GetType() const { return m_type; }
  // b2Body::SetBullet / IsBullet (include/box2d/b2_body.h:701-716): continuous collision with
  // other dynamic bodies
  void SetBullet(bool flag);
  bool IsBullet() const;
  void SetSleepingAllowed(bool flag) { B2_NOT_USED(flag); }
  bool IsSleepingAllowed() const;
  // b2Body::SetAwake / IsAwake (include/box2d/b2_body.h:719-746)
  void SetAwake(bool flag);
  bool IsAwake() const;
  bool IsEnabled() const { return true; }
  bool IsFixedRotation() const { return m_fixedRotation; }
  b2Fixture* GetFixtureList() { return m_fixtureList; }
  const b2Fixture* GetFixtureList() const { return m_fixtureList; }
  b2Body* GetNext() { return m_next; }
  const b2Body* GetNext() const { return m_next; }
  b2BodyUserData& GetUserData() { return m_userData; }
  b2World* GetWorld() { return m_world; }
  const b2World* GetWorld() const { return m_world; }
  int32 GetIndex() const { return m_index; }

  b2World* m_world = nullptr;
  int32 m_index = 0;
  b2BodyType m_type = b2_staticBody;
  bool m_fixedRotation = false;
  b2Body* m_next = nullptr;
  b2Fixture* m_fixtureList = nullptr;
  b2BodyUserData m_userData;

 private:
  void Sync() const;
  mutable uint64_t m_seen = ~0ull;
  mutable b2Transform m_xf;
  mutable b2Vec2 m_c, m_lc, m_v;
  mutable float m_a = 0.0f, m_w = 0.0f;
};

// ---------------------------------------------------------------- joints
enum b2JointType {
  e_unknownJoint, e_revoluteJoint, e_prismaticJoint, e_distanceJoint, e_pulleyJoint, e_mouseJoint, e_gearJoint,
  e_wheelJoint, e_weldJoint, e_frictionJoint, e_ropeJoint, e_motorJoint
};

struct b2JointDef {
  b2JointDef() : type(e_unknownJoint), bodyA(nullptr), bodyB(nullptr), collideConnected(false) {}
  b2JointType type;
  b2JointUserData userData;
  b2Body* bodyA;
  b2Body* bodyB;
  bool collideConnected;
};

struct b2RevoluteJointDef : public b2JointDef {
  b2RevoluteJointDef() {
    type = e_revoluteJoint; localAnchorA.Set(0.0f, 0.0f); localAnchorB.Set(0.0f, 0.0f); referenceAngle = 0.0f;
    lowerAngle = 0.0f; upperAngle = 0.0f; maxMotorTorque = 0.0f; motorSpeed = 0.0f; enableLimit = false;
    enableMotor = false;
  }
  void Initialize(b2Body* bodyA, b2Body* bodyB, const b2Vec2& anchor);
  b2Vec2 localAnchorA, localAnchorB;
  float referenceAngle;
  bool enableLimit;
  float lowerAngle, upperAngle;
  bool enableMotor;
  float motorSpeed;
  float maxMotorTorque;
};

struct b2PrismaticJointDef : public b2JointDef {
  b2PrismaticJointDef() {
    type = e_prismaticJoint; localAnchorA.SetZero(); localAnchorB.SetZero(); localAxisA.Set(1.0f, 0.0f);
    referenceAngle = 0.0f; enableLimit = false; lowerTranslation = 0.0f; upperTranslation = 0.0f;
    enableMotor = false; maxMotorForce = 0.0f; motorSpeed = 0.0f;
  }
  void Initialize(b2Body* bodyA, b2Body* bodyB, const b2Vec2& anchor, const b2Vec2& axis);
  b2Vec2 localAnchorA, localAnchorB, localAxisA;
  float referenceAngle;
  bool enableLimit;
  float lowerTranslation, upperTranslation;
  bool enableMotor;
  float maxMotorForce;
  float motorSpeed;
};

struct b2DistanceJointDef : public b2JointDef {
  b2DistanceJointDef() {
    type = e_distanceJoint; localAnchorA.Set(0.0f, 0.0f); localAnchorB.Set(0.0f, 0.0f); length = 1.0f;
    minLength = 0.0f; maxLength = FLT_MAX; stiffness = 0.0f; damping = 0.0f;
  }
  void Initialize(b2Body* bodyA, b2Body* bodyB, const b2Vec2& anchorA, const b2Vec2& anchorB);
  b2Vec2 localAnchorA, localAnchorB;
  float length, minLength, maxLength, stiffness, damping;
};

// Spring stiffness and damping from a frequency and damping ratio over the bodies' mass or
// inertia (include/box2d/b2_joint.h:97-107).
void b2LinearStiffness(float& stiffness, float& damping, float frequencyHertz, float dampingRatio,
                       const b2Body* bodyA, const b2Body* bodyB);
void b2AngularStiffness(float& stiffness, float& damping, float frequencyHertz, float dampingRatio,
                        const b2Body* bodyA, const b2Body* bodyB);

// b2WeldJointDef (include/box2d/b2_weld_joint.h:31-65)
struct b2WeldJointDef : public b2JointDef {
  b2WeldJointDef() {
    type = e_weldJoint; localAnchorA.Set(0.0f, 0.0f); localAnchorB.Set(0.0f, 0.0f); referenceAngle = 0.0f;
    stiffness = 0.0f; damping = 0.0f;
  }
  void Initialize(b2Body* bodyA, b2Body* bodyB, const b2Vec2& anchor);
  b2Vec2 localAnchorA, localAnchorB;
  float referenceAngle, stiffness, damping;
};

// b2WheelJointDef (include/box2d/b2_wheel_joint.h:34-89)
struct b2WheelJointDef : public b2JointDef {
  b2WheelJointDef() {
    type = e_wheelJoint; localAnchorA.SetZero(); localAnchorB.SetZero(); localAxisA.Set(1.0f, 0.0f);
    enableLimit = false; lowerTranslation = 0.0f; upperTranslation = 0.0f; enableMotor = false;
    maxMotorTorque = 0.0f; motorSpeed = 0.0f; stiffness = 0.0f; damping = 0.0f;
  }
  void Initialize(b2Body* bodyA, b2Body* bodyB, const b2Vec2& anchor, const b2Vec2& axis);
  b2Vec2 localAnchorA, localAnchorB, localAxisA;
  bool enableLimit;
  float lowerTranslation, upperTranslation;
  bool enableMotor;
  float maxMotorTorque, motorSpeed, stiffness, damping;
};

// b2MotorJointDef (include/box2d/b2_motor_joint.h:29-59)
struct b2MotorJointDef : public b2JointDef {
  b2MotorJointDef() {
    type = e_motorJoint; linearOffset.SetZero(); angularOffset = 0.0f; maxForce = 1.0f; maxTorque = 1.0f;
    correctionFactor = 0.3f;
  }
  void Initialize(b2Body* bodyA, b2Body* bodyB);
  b2Vec2 linearOffset;
  float angularOffset, maxForce, maxTorque, correctionFactor;
};

// b2FrictionJointDef (include/box2d/b2_friction_joint.h:29-56)
struct b2FrictionJointDef : public b2JointDef {
  b2FrictionJointDef() {
    type = e_frictionJoint; localAnchorA.SetZero(); localAnchorB.SetZero(); maxForce = 0.0f; maxTorque = 0.0f;
  }
  void Initialize(b2Body* bodyA, b2Body* bodyB, const b2Vec2& anchor);
  b2Vec2 localAnchorA, localAnchorB;
  float maxForce, maxTorque;
};

// b2MouseJointDef (include/box2d/b2_mouse_joint.h:30-56)
struct b2MouseJointDef : public b2JointDef {
  b2MouseJointDef() { type = e_mouseJoint; target.Set(0.0f, 0.0f); maxForce = 0.0f; stiffness = 0.0f; damping = 0.0f; }
  b2Vec2 target;
  float maxForce, stiffness, damping;
};

// b2PulleyJointDef (include/box2d/b2_pulley_joint.h:32-75)
struct b2PulleyJointDef : public b2JointDef {
  b2PulleyJointDef() {
    type = e_pulleyJoint; groundAnchorA.Set(-1.0f, 1.0f); groundAnchorB.Set(1.0f, 1.0f);
    localAnchorA.Set(-1.0f, 0.0f); localAnchorB.Set(1.0f, 0.0f); lengthA = 0.0f; lengthB = 0.0f; ratio = 1.0f;
    collideConnected = true;
  }
  void Initialize(b2Body* bodyA, b2Body* bodyB, const b2Vec2& groundAnchorA, const b2Vec2& groundAnchorB,
                  const b2Vec2& anchorA, const b2Vec2& anchorB, float ratio);
  b2Vec2 groundAnchorA, groundAnchorB, localAnchorA, localAnchorB;
  float lengthA, lengthB, ratio;
};

// b2GearJointDef (include/box2d/b2_gear_joint.h:28-45): couples two revolute or prismatic
// joints: coordinate 1 + ratio * coordinate 2 stays constant.
struct b2GearJointDef : public b2JointDef {
  b2GearJointDef() { type = e_gearJoint; joint1 = nullptr; joint2 = nullptr; ratio = 1.0f; }
  class b2Joint* joint1;
  class b2Joint* joint2;
  float ratio;
};

class b2Joint {
 public:
  virtual ~b2Joint() {}
  b2JointType GetType() const { return m_type; }
  b2Body* GetBodyA() { return m_bodyA; }
  b2Body* GetBodyB() { return m_bodyB; }
  b2Vec2 GetAnchorA() const { return m_bodyA->GetWorldPoint(m_localAnchorA); }
  b2Vec2 GetAnchorB() const { return m_bodyB->GetWorldPoint(m_localAnchorB); }
  // Reaction force / torque of the last step, scaled by inv_dt (b2Joint::GetReactionForce).
  b2Vec2 GetReactionForce(float inv_dt) const;
  float GetReactionTorque(float inv_dt) const;
  b2Joint* GetNext() { return m_next; }
  b2JointUserData& GetUserData() { return m_userData; }
  bool GetCollideConnected() const { return m_collideConnected; }
  int32 GetIndex() const { return m_index; }

  b2World* m_world = nullptr;
  int32 m_index = 0;
  b2JointType m_type = e_unknownJoint;
  b2Body* m_bodyA = nullptr;
  b2Body* m_bodyB = nullptr;
  b2Joint* m_next = nullptr;
  bool m_collideConnected = false;
  b2Vec2 m_localAnchorA, m_localAnchorB;
  b2JointUserData m_userData;
};
class b2RevoluteJoint : public b2Joint {};
class b2PrismaticJoint : public b2Joint {};
class b2DistanceJoint : public b2Joint {};
class b2WeldJoint : public b2Joint {};
class b2WheelJoint : public b2Joint {};
class b2MotorJoint : public b2Joint {};
class b2FrictionJoint : public b2Joint {};
class b2MouseJoint : public b2Joint {};
class b2PulleyJoint : public b2Joint {};
class b2GearJoint : public b2Joint {
 public:
  b2Joint* GetJoint1() { return m_joint1; }
  b2Joint* GetJoint2() { return m_joint2; }
  float GetRatio() const { return m_ratio; }
  b2Joint* m_joint1 = nullptr;
  b2Joint* m_joint2 = nullptr;
  float m_ratio = 1.0f;
};

// ---------------------------------------------------------------- contacts and listeners
class b2Contact {
 public:
  b2Manifold* GetManifold() { return &m_manifold; }
  const b2Manifold* GetManifold() const { return &m_manifold; }
  void GetWorldManifold(b2WorldManifold* worldManifold) const;
  bool IsTouching() const { return (m_flags & B2G_CONTACT_TOUCHING) != 0; }
  void SetEnabled(bool flag) { if (flag) m_flags |= B2G_CONTACT_ENABLED; else m_flags &= ~B2G_CONTACT_ENABLED; }
  bool IsEnabled() const { return (m_flags & B2G_CONTACT_ENABLED) != 0; }
  b2Contact* GetNext() { return m_next; }
  const b2Contact* GetNext() const { return m_next; }
  b2Fixture* GetFixtureA() { return m_fixtureA; }
  const b2Fixture* GetFixtureA() const { return m_fixtureA; }
  b2Fixture* GetFixtureB() { return m_fixtureB; }
  const b2Fixture* GetFixtureB() const { return m_fixtureB; }
  int32 GetChildIndexA() const { return 0; }
  int32 GetChildIndexB() const { return 0; }
  float GetFriction() const { return m_friction; }
  float GetRestitution() const { return m_restitution; }
  float GetRestitutionThreshold() const { return m_restitutionThreshold; }
  float GetTangentSpeed() const { return m_tangentSpeed; }

  b2Fixture* m_fixtureA = nullptr;
  b2Fixture* m_fixtureB = nullptr;
  b2Contact* m_next = nullptr;
  uint32 m_flags = 0;
  float m_friction = 0, m_restitution = 0, m_restitutionThreshold = 0, m_tangentSpeed = 0;
  b2Manifold m_manifold;
};

struct b2ContactImpulse {
  float normalImpulses[b2_maxManifoldPoints];
  float tangentImpulses[b2_maxManifoldPoints];
  int32 count;
};

class b2ContactFilter {
 public:
  virtual ~b2ContactFilter() {}
  virtual bool ShouldCollide(b2Fixture* fixtureA, b2Fixture* fixtureB);
};

class b2ContactListener {
 public:
  virtual ~b2ContactListener() {}
  virtual void BeginContact(b2Contact* contact) { B2_NOT_USED(contact); }
  virtual void EndContact(b2Contact* contact) { B2_NOT_USED(contact); }
  virtual void PreSolve(b2Contact* contact, const b2Manifold* oldManifold) { B2_NOT_USED(contact); B2_NOT_USED(oldManifold); }
  virtual void PostSolve(b2Contact* contact, const b2ContactImpulse* impulse) { B2_NOT_USED(contact); B2_NOT_USED(impulse); }
};

// b2DestructionListener (include/box2d/b2_world_callbacks.h:35-47): called for the joints and
// fixtures a DestroyBody call destroys implicitly.
class b2DestructionListener {
 public:
  virtual ~b2DestructionListener() {}
  virtual void SayGoodbye(b2Joint* joint) = 0;
  virtual void SayGoodbye(b2Fixture* fixture) = 0;
};

struct b2Profile {
  float step, collide, solve, solveInit, solveVelocity, solvePosition, broadphase, solveTOI;
};

// ---------------------------------------------------------------- world
class b2World {
 public:
  explicit b2World(const b2Vec2& gravity);
  // Adds a world to an existing batch (the batch steps all its worlds in one launch sequence).
  b2World(b2g_batch* batch, const b2Vec2& gravity);
  // Wraps world `index` of an existing batch without owning it.
  b2World(b2g_batch* batch, int32 index, bool attach);
  ~b2World();
  b2World(const b2World&) = delete;
  b2World& operator=(const b2World&) = delete;

  void SetDestructionListener(b2DestructionListener* listener) { m_destruction = listener; }
  // A b2ContactFilter subclass cannot run inside the GPU broadphase: with one set, Step returns
  // without stepping and LastStatus() is B2G_E_INVALID_ARG. The base class (the default
  // group / category / mask filter, which the engine applies anyway) and nullptr are accepted.
  void SetContactFilter(b2ContactFilter* filter);
  void SetContactListener(b2ContactListener* listener);
  b2Body* CreateBody(const b2BodyDef* def);
  // b2World::DestroyBody (src/dynamics/b2_world.cpp:178-266): its joints (SayGoodbye), contacts
  // (EndContact for the touching ones, before this returns) and fixtures (SayGoodbye) go with it.
  // Indices (GetIndex) of the bodies, fixtures and joints created after it shift down.
  void DestroyBody(b2Body* body);
  b2Joint* CreateJoint(const b2JointDef* def);
  // b2World::DestroyJoint (src/dynamics/b2_world.cpp:326-410): both bodies wake.
  void DestroyJoint(b2Joint* joint);
  void Step(float timeStep, int32 velocityIterations, int32 positionIterations, int32 particleIterations = 1);
  void ClearForces();
  b2Body* GetBodyList() { return m_bodyHead; }
  b2Joint* GetJointList() { return m_joints.empty() ? nullptr : m_joints.front().get(); }
  b2Contact* GetContactListStart();
  b2Contact* GetContactListEnd() { return &m_contactEnd; }
  void SetAllowSleeping(bool flag);
  bool GetAllowSleeping() const { return m_allowSleep; }
  void SetWarmStarting(bool flag);
  bool GetWarmStarting() const { return m_warmStarting; }
  void SetContinuousPhysics(bool flag);
  bool GetContinuousPhysics() const { return m_continuous; }
  void SetSubStepping(bool flag) { B2_NOT_USED(flag); }
  bool GetSubStepping() const { return false; }
  int32 GetProxyCount() const { return (int32)m_fixtureIndex.size(); }
  int32 GetBodyCount() const { return m_bodyCount; }
  int32 GetJointCount() const { return (int32)m_joints.size(); }
  int32 GetContactCount() const;
  void SetGravity(const b2Vec2& gravity);
  b2Vec2 GetGravity() const { return m_gravity; }
  bool IsLocked() const { return false; }
  void SetAutoClearForces(bool flag);
  bool GetAutoClearForces() const { return m_autoClear; }
  const b2Profile& GetProfile() const { return m_profile; }
  // b2World::Dump (src/dynamics/b2_world.cpp:1469-1531): writes the world as C++ source to
  // box2d_dump.inl in the working directory, in the reference's format.
  void Dump();

  // Extensions of this engine
  // After stepping a shared batch with b2g_step (all its worlds at once), hands this world's
  // listener events of that step to its b2ContactListener. b2World::Step does this itself.
  void DeliverEvents();
  b2g_batch* GetBatch() { return m_batch; }
  int32 GetWorldIndex() const { return m_index; }
  int LastStatus() const { return m_lastStatus; }

  // internal: cached body state of this world (refreshed after a step)
  uint64_t StateVersion() const { return m_version; }
  const b2g_body& BodyRecord(int32 index) const;
  void WriteBody(int32 index, const b2g_body& rec);
  void InvalidateCaches() { m_stateValid = false; m_contactsValid = false; m_jointsValid = false; ++m_version; }
  b2Fixture* FixtureAt(int32 i) { return m_fixtureIndex[i]; }
  const b2g_joint& JointRecord(int32 index) const;

 private:
  void ApplyFlags();
  void Deliver();
  // after a removal: the engine's End callbacks for the destroyed contacts, then renumbering
  void EndContacts(const std::vector<b2g_event>& ended, int32 n, const std::vector<b2Contact>& before);
  void Renumber();
  void EraseOrphanGears();
  b2g_batch* m_batch = nullptr;
  bool m_ownsBatch = false;
  int32 m_index = 0;
  b2Vec2 m_gravity;
  // b2World's defaults (src/dynamics/b2_world.cpp:56-62): sleeping and continuous physics on
  bool m_allowSleep = true, m_warmStarting = true, m_continuous = true, m_autoClear = true;
  b2ContactListener* m_listener = nullptr;
  b2ContactFilter* m_filter = nullptr;
  bool m_filterUnsupported = false;
  b2DestructionListener* m_destruction = nullptr;
  std::deque<b2Body> m_bodies;  // every body created; destroyed ones keep m_index = -1
  b2Body* m_bodyHead = nullptr;  // first live body (creation order)
  b2Body* m_bodyTail = nullptr;  // last live body
  int32 m_bodyCount = 0;
  std::deque<b2Fixture> m_fixtures;
  std::vector<b2Fixture*> m_fixtureIndex;
  std::vector<std::unique_ptr<b2Joint>> m_joints;
  mutable std::vector<b2g_body> m_state;
  mutable bool m_stateValid = false;
  mutable std::vector<b2g_joint> m_jointState;
  mutable bool m_jointsValid = false;
  std::vector<b2Contact> m_contacts;
  bool m_contactsValid = false;
  b2Contact m_contactEnd;
  b2Profile m_profile = {};
  int m_lastStatus = B2G_OK;
  uint64_t m_version = 1;
  friend class b2Body;
};
