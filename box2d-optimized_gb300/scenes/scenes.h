// Seeded scene generators for the benchmark and parity workloads.
//
// Written only against the public Box2D C++ API (b2World, b2BodyDef, b2FixtureDef, b2PolygonShape,
// b2CircleShape, b2EdgeShape, b2RevoluteJointDef), so the same source builds a world for the
// reference engine, for this library's b2World facade and for the CPU oracle's scene builder:
// the worlds are created by the same sequence of calls with the same arguments.
//
// Scene recipes:
//   Pyramid      - testbed/tests/pyramid.cpp:33-70 layout (rows of 0.5 m half-extent boxes on a
//                  two-sided edge ground), with density/friction as parameters.
//   MixedDrop    - dynamic boxes / circles / convex polygons dropped from a jittered grid into a
//                  static U made of three two-sided edges.
//   ChainsOverPile - chains of thin boxes linked by revolute joints (some limited, some motorised),
//                  hung above a pile of circles in the same U container.
//   BatchWorld   - one world of a batched workload: picks one of the above by seed, scaled to a
//                  body count, with gravity and friction jittered by +-10%.
//   Bullets      - bullets fired or thrown at boxes resting on the ground (continuous collision).
//   (scenes_joints.h: JointZoo and SliderRigs, rigs of the other joint types.)
//
// Random numbers come from std::mt19937 (fully specified by the C++ standard) with a portable
// 24-bit float conversion, and every draw is its own statement (argument evaluation order is
// unspecified in C++), so every compiler generates the same sequence of draws.
#pragma once

#include <cmath>
#include <cstdint>
#include <random>
#include <vector>

#include "box2d/box2d.h"

namespace b2scenes {

struct Rng {
  std::mt19937 g;
  explicit Rng(uint32_t seed) : g(seed) {}
  // Uniform in [0, 1) with 24 random bits.
  float u01() { return (float)(g() >> 8) * (1.0f / 16777216.0f); }
  float uni(float lo, float hi) { return lo + (hi - lo) * u01(); }
  int irange(int lo, int hi_inclusive) { return lo + (int)(g() % (uint32_t)(hi_inclusive - lo + 1)); }
};

struct Counts {
  int bodies = 0;     // dynamic bodies created
  int fixtures = 0;   // all fixtures created (including static)
  int joints = 0;
};

// Creation-order tags. Every body and fixture made by these recipes carries its creation index
// (counted per world) in userData.pointer, so a caller can line up bodies and fixtures of two
// engines whose internal lists are ordered differently.
struct Tagger {
  uintptr_t nextBody = 0;
  uintptr_t nextFixture = 0;
};
inline Tagger& Tags() {
  static thread_local Tagger t;
  return t;
}
inline void ResetTags() { Tags() = Tagger(); }
inline b2Body* MakeBody(b2World* world, b2BodyDef* bd) {
  bd->userData.pointer = Tags().nextBody++;
  return world->CreateBody(bd);
}
inline b2Fixture* MakeFixture(b2Body* body, b2FixtureDef* fd) {
  fd->userData.pointer = Tags().nextFixture++;
  return body->CreateFixture(fd);
}
inline b2Fixture* MakeFixture(b2Body* body, const b2Shape* shape, float density) {
  b2FixtureDef fd;
  fd.shape = shape;
  fd.density = density;
  return MakeFixture(body, &fd);
}

// Static two-sided edge from (x1,y1) to (x2,y2) on body `ground`.
inline void AddEdge(b2Body* ground, float x1, float y1, float x2, float y2, Counts* c) {
  b2EdgeShape e;
  e.SetTwoSided(b2Vec2(x1, y1), b2Vec2(x2, y2));
  MakeFixture(ground, &e, 0.0f);
  c->fixtures++;
}

// testbed/tests/pyramid.cpp:33-70 with `rows` rows; box half-extent 0.5, start (-7, 0.75),
// deltaX (0.5625, 1.25), deltaY (1.125, 0); ground edge (-40,0)-(40,0).
inline Counts Pyramid(b2World* world, int rows, float density, float friction, bool ground = true,
                      float x0 = -7.0f) {
  Counts c;
  if (ground) {
    b2BodyDef bd;
    b2Body* g = MakeBody(world, &bd);
    AddEdge(g, -40.0f, 0.0f, 40.0f, 0.0f, &c);
  }
  float a = 0.5f;
  b2PolygonShape shape;
  shape.SetAsBox(a, a);
  b2FixtureDef fd;
  fd.shape = &shape;
  fd.density = density;
  fd.friction = friction;

  b2Vec2 x(x0, 0.75f);
  b2Vec2 y;
  b2Vec2 deltaX(0.5625f, 1.25f);
  b2Vec2 deltaY(1.125f, 0.0f);
  for (int i = 0; i < rows; ++i) {
    y = x;
    for (int j = i; j < rows; ++j) {
      b2BodyDef bd;
      bd.type = b2_dynamicBody;
      bd.position = y;
      b2Body* body = MakeBody(world, &bd);
      MakeFixture(body, &fd);
      c.bodies++;
      c.fixtures++;
      y += deltaY;
    }
    x += deltaX;
  }
  return c;
}

// Static U container: floor y=0 for x in [-halfWidth, halfWidth], walls up to `height`.
inline b2Body* UContainer(b2World* world, float halfWidth, float height, Counts* c) {
  b2BodyDef bd;
  b2Body* g = MakeBody(world, &bd);
  AddEdge(g, -halfWidth, 0.0f, halfWidth, 0.0f, c);
  AddEdge(g, -halfWidth, 0.0f, -halfWidth, height, c);
  AddEdge(g, halfWidth, 0.0f, halfWidth, height, c);
  return g;
}

// One random dynamic shape of the mixed-drop recipe at `pos`.
//   40% boxes (half-extents U[0.1,0.5]), 30% circles (r U[0.1,0.5]), 30% convex polygons with
//   3-8 vertices at angles 2*pi*(k + U[0,0.3])/n on a circle of radius U[0.2,0.6].
inline void MixedBody(b2World* world, Rng& rng, b2Vec2 pos, float friction, Counts* c) {
  b2BodyDef bd;
  bd.type = b2_dynamicBody;
  bd.position = pos;
  bd.angle = rng.uni(-3.14159265f, 3.14159265f);
  b2Body* body = MakeBody(world, &bd);
  b2FixtureDef fd;
  fd.density = rng.uni(0.5f, 2.0f);
  fd.friction = friction;
  float pick = rng.u01();
  if (pick < 0.4f) {
    b2PolygonShape box;
    float hx = rng.uni(0.1f, 0.5f);
    float hy = rng.uni(0.1f, 0.5f);
    box.SetAsBox(hx, hy);
    fd.shape = &box;
    MakeFixture(body, &fd);
  } else if (pick < 0.7f) {
    b2CircleShape circle;
    circle.m_radius = rng.uni(0.1f, 0.5f);
    fd.shape = &circle;
    MakeFixture(body, &fd);
  } else {
    int n = rng.irange(3, 8);
    float r = rng.uni(0.2f, 0.6f);
    b2Vec2 vs[8];
    for (int k = 0; k < n; ++k) {
      float ang = 6.28318531f * ((float)k + rng.uni(0.0f, 0.3f)) / (float)n;
      vs[k].Set(r * std::cos(ang), r * std::sin(ang));
    }
    b2PolygonShape poly;
    poly.Set(vs, n);
    fd.shape = &poly;
    MakeFixture(body, &fd);
  }
  c->bodies++;
  c->fixtures++;
}

// `n` mixed dynamic bodies dropped from a jittered grid (2 m pitch) into a U container whose
// width scales with sqrt(n). With n = 20000 this is a 200 m x 400 m grid over a 220 m U.
inline Counts MixedDrop(b2World* world, int n, uint32_t seed, float friction = 0.6f) {
  Counts c;
  Rng rng(seed);
  int cols = (int)std::ceil(std::sqrt((double)n / 2.0));
  if (cols < 4) cols = 4;
  int rows = (n + cols - 1) / cols;
  float pitch = 2.0f;
  float halfWidth = 0.5f * pitch * (float)cols + 10.0f;
  float height = 10.0f + pitch * (float)rows + 50.0f;
  UContainer(world, halfWidth, height, &c);
  float x0 = -0.5f * pitch * (float)(cols - 1);
  int made = 0;
  for (int r = 0; r < rows && made < n; ++r) {
    for (int k = 0; k < cols && made < n; ++k, ++made) {
      float jx = rng.uni(-0.3f, 0.3f);
      float jy = rng.uni(-0.3f, 0.3f);
      b2Vec2 p(x0 + pitch * (float)k + jx, 10.0f + pitch * (float)r + jy);
      MixedBody(world, rng, p, friction, &c);
    }
  }
  return c;
}

// `nchains` chains of `links` boxes (half-extents 0.05 x 0.25) joined end to end by revolute
// joints and hung from the static container body; half the joints of a chain are limited to
// +-30 deg, every tenth chain is motorised (max torque 50 N.m). Below them `ncircles` circles
// (r U[0.05,0.3]) are dropped from a jittered grid into the U container.
inline Counts ChainsOverPile(b2World* world, int nchains, int links, int ncircles, uint32_t seed,
                             float friction = 0.6f) {
  Counts c;
  Rng rng(seed);
  int perRow = nchains < 1000 ? nchains : 1000;
  int chainRows = (nchains + perRow - 1) / perRow;
  float chainPitch = 0.2f;
  int pileCols = (int)std::ceil(std::sqrt((double)ncircles * 2.0));
  if (pileCols < 4) pileCols = 4;
  float pilePitch = 0.7f;
  float halfWidth = 0.5f * std::fmax(chainPitch * (float)perRow, pilePitch * (float)pileCols) + 5.0f;
  int pileRows = (ncircles + pileCols - 1) / pileCols;
  float pileTop = 2.0f + pilePitch * (float)pileRows;
  float linkLen = 0.5f;
  float firstRowY = pileTop + 5.0f + (float)chainRows * ((float)links * linkLen + 3.0f);
  b2Body* ground = UContainer(world, halfWidth, firstRowY + 20.0f, &c);

  // pile of circles
  {
    float x0 = -0.5f * pilePitch * (float)(pileCols - 1);
    int made = 0;
    for (int r = 0; r < pileRows && made < ncircles; ++r) {
      for (int k = 0; k < pileCols && made < ncircles; ++k, ++made) {
        b2BodyDef bd;
        bd.type = b2_dynamicBody;
        float jx = rng.uni(-0.05f, 0.05f);
        float jy = rng.uni(-0.05f, 0.05f);
        bd.position.Set(x0 + pilePitch * (float)k + jx, 2.0f + pilePitch * (float)r + jy);
        b2Body* b = MakeBody(world, &bd);
        b2CircleShape circle;
        circle.m_radius = rng.uni(0.05f, 0.3f);
        b2FixtureDef fd;
        fd.shape = &circle;
        fd.density = 1.0f;
        fd.friction = friction;
        MakeFixture(b, &fd);
        c.bodies++;
        c.fixtures++;
      }
    }
  }

  // chains
  b2PolygonShape link;
  link.SetAsBox(0.05f, 0.25f);
  b2FixtureDef lfd;
  lfd.shape = &link;
  lfd.density = 1.0f;
  lfd.friction = friction;
  for (int ch = 0; ch < nchains; ++ch) {
    int row = ch / perRow;
    int col = ch % perRow;
    float x = -0.5f * chainPitch * (float)(perRow - 1) + chainPitch * (float)col;
    float yTop = firstRowY - (float)row * ((float)links * linkLen + 3.0f);
    bool motor = (ch % 10) == 0;
    b2Body* prev = ground;
    for (int l = 0; l < links; ++l) {
      b2BodyDef bd;
      bd.type = b2_dynamicBody;
      bd.position.Set(x, yTop - linkLen * ((float)l + 0.5f));
      b2Body* b = MakeBody(world, &bd);
      MakeFixture(b, &lfd);
      c.bodies++;
      c.fixtures++;
      b2RevoluteJointDef jd;
      jd.Initialize(prev, b, b2Vec2(x, yTop - linkLen * (float)l));
      if (l % 2 == 1) {
        jd.enableLimit = true;
        jd.lowerAngle = -0.523598776f;
        jd.upperAngle = 0.523598776f;
      }
      if (motor) {
        jd.enableMotor = true;
        jd.maxMotorTorque = 50.0f;
        jd.motorSpeed = 0.5f;
      }
      world->CreateJoint(&jd);
      c.joints++;
      prev = b;
    }
  }
  return c;
}

// Body count of world `index` of a batched workload: 2^U[4,13] (log-uniform in [16, 8192]).
inline int BatchBodyCount(uint32_t seed, int lo = 16, int hi = 8192) {
  Rng rng(seed * 2654435761u + 12345u);
  float e = rng.uni(std::log2((float)lo), std::log2((float)hi));
  int n = (int)std::lround(std::exp2(e));
  if (n < lo) n = lo;
  if (n > hi) n = hi;
  return n;
}

// Gravity of world `seed` of a batched workload: (0, -10) jittered by U[-10%, +10%].
inline b2Vec2 BatchGravity(uint32_t seed) {
  Rng rng(seed * 747796405u + 2891336453u);
  return b2Vec2(0.0f, -10.0f * (1.0f + rng.uni(-0.1f, 0.1f)));
}

// Fills `world` (created with BatchGravity(seed)) with about `n` dynamic bodies: a pyramid,
// a mixed grid drop or chains over a circle pile, picked by seed; friction 0.6 jittered +-10%.
inline Counts BatchWorld(b2World* world, uint32_t seed, int n) {
  Rng rng(seed * 2246822519u + 374761393u);
  float friction = 0.6f * (1.0f + rng.uni(-0.1f, 0.1f));
  int kind = (int)(rng.g() % 3u);
  if (kind == 0) {
    int rows = (int)std::floor((std::sqrt(8.0 * (double)n + 1.0) - 1.0) / 2.0);
    if (rows < 1) rows = 1;
    Counts c = Pyramid(world, rows, 1.0f, friction, true);
    int rest = n - c.bodies;
    if (rest > 0) {
      // the remainder falls onto the pyramid's right-hand side from a small grid
      for (int i = 0; i < rest; ++i) {
        float jx = rng.uni(-0.2f, 0.2f);
        float jy = rng.uni(-0.2f, 0.2f);
        b2Vec2 p(25.0f + 1.5f * (float)(i % 8) + jx, 2.0f + 1.5f * (float)(i / 8) + jy);
        MixedBody(world, rng, p, friction, &c);
      }
    }
    return c;
  } else if (kind == 1) {
    return MixedDrop(world, n, seed ^ 0x9e3779b9u, friction);
  } else {
    int links = 10;
    int nchains = n / (2 * links);
    if (nchains < 1) nchains = 1;
    int ncircles = n - nchains * links;
    if (ncircles < 0) ncircles = 0;
    return ChainsOverPile(world, nchains, links, ncircles, seed ^ 0x85ebca6bu, friction);
  }
}

// `n` lanes 16 m apart on a static edge ground. In each a dynamic box (half-extent 0.6-1.0 m)
// rests on the ground and a bullet (b2BodyDef::bullet; a circle of radius 0.1-0.25 m in even
// lanes, a square of half-extent 0.1-0.25 m in odd ones, density 3) flies at it: fired
// horizontally at 25-70 m/s from 7 m away, or, in every third lane, thrown down at it at
// 25-70 m/s from 7 m above. With `kinematic`, every fourth lane drives a kinematic bar (0.3 x 1.2 m)
// at its box at 15-40 m/s instead of a bullet. Continuous collision resolves the impacts.
inline Counts Bullets(b2World* world, int n, uint32_t seed, bool kinematic = false) {
  Counts c;
  Rng rng(seed);
  b2BodyDef gd;
  b2Body* ground = MakeBody(world, &gd);
  AddEdge(ground, -20.0f, 0.0f, 16.0f * (float)n + 20.0f, 0.0f, &c);
  for (int i = 0; i < n; ++i) {
    const float x0 = 16.0f * (float)i;
    const float half = rng.uni(0.6f, 1.0f);
    b2BodyDef td;
    td.type = b2_dynamicBody;
    td.position.Set(x0 + 7.0f, half);
    b2Body* target = MakeBody(world, &td);
    b2PolygonShape box;
    box.SetAsBox(half, half);
    b2FixtureDef fd;
    fd.shape = &box;
    fd.density = 1.0f;
    fd.friction = 0.6f;
    MakeFixture(target, &fd);
    c.bodies++;
    c.fixtures++;
    const float speed = rng.uni(25.0f, 70.0f);
    const float lateral = rng.uni(-0.4f, 0.4f);
    const float spin = rng.uni(-5.0f, 5.0f);
    const float size = rng.uni(0.1f, 0.25f);
    if (kinematic && i % 4 == 3) {
      b2BodyDef kd;
      kd.type = b2_kinematicBody;
      kd.position.Set(x0, half + lateral);
      kd.linearVelocity.Set(0.5f * speed + 2.5f, 0.0f);
      kd.angularVelocity = 0.2f * spin;
      b2Body* bar = MakeBody(world, &kd);
      b2PolygonShape shape;
      shape.SetAsBox(0.15f, 0.6f);
      MakeFixture(bar, &shape, 1.0f);
      c.fixtures++;
      continue;
    }
    b2BodyDef bd;
    bd.type = b2_dynamicBody;
    bd.bullet = true;
    if (i % 3 == 2) {
      bd.position.Set(x0 + 7.0f + lateral, 2.0f * half + 7.0f);
      bd.linearVelocity.Set(0.0f, -speed);
    } else {
      bd.position.Set(x0, half + lateral);
      bd.linearVelocity.Set(speed, 0.0f);
    }
    bd.angularVelocity = spin;
    b2Body* bullet = MakeBody(world, &bd);
    b2FixtureDef bf;
    bf.density = 3.0f;
    bf.friction = 0.4f;
    b2CircleShape circle;
    b2PolygonShape square;
    if (i % 2 == 0) {
      circle.m_radius = size;
      bf.shape = &circle;
    } else {
      square.SetAsBox(size, size);
      bf.shape = &square;
    }
    MakeFixture(bullet, &bf);
    c.bodies++;
    c.fixtures++;
  }
  return c;
}

}  // namespace b2scenes
