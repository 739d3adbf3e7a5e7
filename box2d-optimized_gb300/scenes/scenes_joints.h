// Seeded rigs of the joint types beyond the revolute joint, over a ground edge (see scenes.h for
// the random numbers, tags and counts these recipes share):
//   JointZoo     - rigs of the weld, wheel, motor, friction, mouse and pulley joints
//                  (b2WeldJointDef, b2WheelJointDef, b2MotorJointDef, b2FrictionJointDef,
//                  b2MouseJointDef, b2PulleyJointDef).
//   SliderRigs   - rigs of distance joints (rigid rods, springs from b2LinearStiffness, min/max
//                  lengths) and prismatic joints (limits, motors, a piston between two dynamic
//                  bodies), with loose boxes falling onto them.
//   GearRigs     - gear joints (b2GearJointDef) coupling revolute and prismatic joints: a motor
//                  driven wheel pair, a rack and pinion, and a double pendulum whose two hinges
//                  are geared, with boxes falling onto them.
// Written against the public Box2D C++ API like scenes.h, so the same source builds a world for
// the reference engine and for this library's b2World facade.
#pragma once

#include "scenes.h"

namespace b2scenes {

// `rigs` rigs side by side over one ground edge, each: a cantilever of three boxes welded to a
// static post (a rigid weld, then two soft ones); a car whose chassis rides on two sprung wheel
// joints (rear motorised, front with translation limits) driving along the ground and carrying a
// sensor disc; a box that a motor joint drives toward an offset from a static anchor; a sliding
// box held back by a friction joint through a static sensor gate; a box pulled up toward a point
// by a mouse joint; two boxes hanging from a pulley.
inline Counts JointZoo(b2World* world, int rigs, uint32_t seed, float friction = 0.6f) {
  Counts c;
  Rng rng(seed);
  if (rigs < 1) rigs = 1;
  const float pitch = 32.0f;
  const float half = 0.5f * pitch * (float)rigs + 20.0f;
  b2BodyDef gd;
  b2Body* ground = MakeBody(world, &gd);
  AddEdge(ground, -half, 0.0f, half, 0.0f, &c);
  b2PolygonShape box;
  box.SetAsBox(0.5f, 0.25f);
  b2FixtureDef fd;
  fd.shape = &box;
  fd.density = 1.0f;
  fd.friction = friction;
  auto dynamicBox = [&](float x, float y, float angle) {
    b2BodyDef bd;
    bd.type = b2_dynamicBody;
    bd.position.Set(x, y);
    bd.angle = angle;
    b2Body* b = MakeBody(world, &bd);
    MakeFixture(b, &fd);
    c.bodies++;
    c.fixtures++;
    return b;
  };
  auto staticPost = [&](float x, float y) {
    b2BodyDef bd;
    bd.position.Set(x, y);
    b2Body* b = MakeBody(world, &bd);
    b2PolygonShape ps;
    ps.SetAsBox(0.2f, 0.2f);
    MakeFixture(b, &ps, 0.0f);
    c.fixtures++;
    return b;
  };
  for (int r = 0; r < rigs; ++r) {
    const float x0 = -0.5f * pitch * (float)rigs + pitch * (float)r + 2.0f;
    const float jit = rng.uni(-0.1f, 0.1f);
    // welded cantilever
    {
      b2Body* post = staticPost(x0, 6.0f);
      b2Body* prev = post;
      for (int k = 0; k < 3; ++k) {
        float x = x0 + 0.7f + 1.0f * (float)k;
        b2Body* b = dynamicBox(x, 6.0f + jit * (float)k, 0.0f);
        b2WeldJointDef jd;
        jd.Initialize(prev, b, b2Vec2(x - 0.5f, 6.0f));
        if (k > 0) {
          jd.stiffness = 40.0f + 20.0f * (float)k;
          jd.damping = 2.0f;
        }
        world->CreateJoint(&jd);
        c.joints++;
        prev = b;
      }
    }
    // car on two wheel joints
    {
      float cx = x0 + 6.0f;
      b2Body* chassis = dynamicBox(cx, 1.4f, 0.0f);
      b2CircleShape disc;  // a sensor reaching below the chassis: touches the ground edge
      disc.m_radius = 1.3f;
      b2FixtureDef sfd;
      sfd.shape = &disc;
      sfd.isSensor = true;
      sfd.density = 0.0f;
      MakeFixture(chassis, &sfd);
      c.fixtures++;
      b2CircleShape wheel;
      wheel.m_radius = 0.35f;
      b2FixtureDef wfd;
      wfd.shape = &wheel;
      wfd.density = 1.0f;
      wfd.friction = 0.9f;
      for (int k = 0; k < 2; ++k) {
        b2BodyDef bd;
        bd.type = b2_dynamicBody;
        float wx = cx + (k == 0 ? -0.45f : 0.45f);
        bd.position.Set(wx, 0.7f);
        b2Body* w = MakeBody(world, &bd);
        MakeFixture(w, &wfd);
        c.bodies++;
        c.fixtures++;
        b2WheelJointDef jd;
        jd.Initialize(chassis, w, w->GetPosition(), b2Vec2(0.0f, 1.0f));
        jd.stiffness = 30.0f;
        jd.damping = 1.5f;
        if (k == 0) {
          jd.enableMotor = true;
          jd.maxMotorTorque = 8.0f;
          jd.motorSpeed = -4.0f - 2.0f * jit;
        } else {
          jd.enableLimit = true;
          jd.lowerTranslation = -0.25f;
          jd.upperTranslation = 0.1f;
        }
        world->CreateJoint(&jd);
        c.joints++;
      }
    }
    // motor joint driving a box toward an offset from a static anchor
    {
      b2Body* anchor = staticPost(x0 + 12.0f, 3.0f);
      b2Body* b = dynamicBox(x0 + 12.0f, 1.0f, 0.3f);
      b2MotorJointDef jd;
      jd.Initialize(anchor, b);
      jd.linearOffset.Set(1.5f + jit, 2.0f);
      jd.angularOffset = 0.5f;
      jd.maxForce = 60.0f;
      jd.maxTorque = 20.0f;
      world->CreateJoint(&jd);
      c.joints++;
    }
    // friction joint holding back a box thrown along the ground through a sensor gate
    {
      b2Body* gate = staticPost(x0 + 17.5f, 2.0f);
      b2PolygonShape gs;
      gs.SetAsBox(0.4f, 2.0f);
      b2FixtureDef gfd;
      gfd.shape = &gs;
      gfd.isSensor = true;
      MakeFixture(gate, &gfd);
      c.fixtures++;
      b2Body* b = dynamicBox(x0 + 16.0f, 0.25f, 0.0f);
      b->SetLinearVelocity(b2Vec2(6.0f + jit, 0.0f));
      b->SetAngularVelocity(3.0f);
      b2FrictionJointDef jd;
      jd.Initialize(ground, b, b->GetPosition());
      jd.maxForce = 4.0f;
      jd.maxTorque = 2.0f;
      world->CreateJoint(&jd);
      c.joints++;
    }
    // mouse joint pulling a box toward a point
    {
      b2Body* b = dynamicBox(x0 + 20.0f, 0.25f, 0.0f);
      b2MouseJointDef jd;
      jd.bodyA = ground;
      jd.bodyB = b;
      jd.target.Set(x0 + 21.0f, 4.0f + jit);
      jd.maxForce = 30.0f;
      jd.stiffness = 15.0f;
      jd.damping = 0.7f;
      world->CreateJoint(&jd);
      c.joints++;
    }
    // pulley with two boxes of different mass
    {
      float px = x0 + 25.0f;
      b2Body* a = dynamicBox(px - 1.5f, 4.0f, 0.0f);
      b2Body* b = dynamicBox(px + 1.5f, 5.0f, 0.0f);
      b2PolygonShape heavy;
      heavy.SetAsBox(0.3f, 0.3f);
      MakeFixture(b, &heavy, 2.0f);
      c.fixtures++;
      b2PulleyJointDef jd;
      jd.Initialize(a, b, b2Vec2(px - 1.5f, 9.0f), b2Vec2(px + 1.5f, 9.0f), b2Vec2(px - 1.5f, 4.25f),
                    b2Vec2(px + 1.5f, 5.25f), 1.5f);
      world->CreateJoint(&jd);
      c.joints++;
    }
  }
  return c;
}

// `rigs` rigs side by side over one ground edge, each:
//  * a pendulum: a box on a rigid distance rod (stiffness 0) from a static post, swung out;
//  * a spring: a box on a soft distance joint (b2LinearStiffness at 2-3.5 Hz) with a minimum and
//    a maximum length, hanging from a post and started off its rest length;
//  * a rope: four boxes linked by distance joints whose maximum length is the rest length plus
//    slack and whose minimum is zero, one end on a post;
//  * an elevator: a box on a vertical prismatic axis with translation limits and a motor pushing
//    it up against the upper limit;
//  * a slider: a box on a tilted prismatic axis with limits and no motor, which slides down to its
//    lower stop, and a loose box dropped onto it;
//  * a piston: two dynamic boxes on one prismatic axis with a motor pulling them apart and limits,
//    resting on the ground.
inline Counts SliderRigs(b2World* world, int rigs, uint32_t seed, float friction = 0.6f) {
  Counts c;
  Rng rng(seed);
  if (rigs < 1) rigs = 1;
  const float pitch = 24.0f;
  const float half = 0.5f * pitch * (float)rigs + 20.0f;
  b2BodyDef gd;
  b2Body* ground = MakeBody(world, &gd);
  AddEdge(ground, -half, 0.0f, half, 0.0f, &c);
  b2PolygonShape box;
  box.SetAsBox(0.4f, 0.3f);
  b2FixtureDef fd;
  fd.shape = &box;
  fd.density = 1.0f;
  fd.friction = friction;
  auto dynamicBox = [&](float x, float y, float angle) {
    b2BodyDef bd;
    bd.type = b2_dynamicBody;
    bd.position.Set(x, y);
    bd.angle = angle;
    b2Body* b = MakeBody(world, &bd);
    MakeFixture(b, &fd);
    c.bodies++;
    c.fixtures++;
    return b;
  };
  auto staticPost = [&](float x, float y) {
    b2BodyDef bd;
    bd.position.Set(x, y);
    b2Body* b = MakeBody(world, &bd);
    b2PolygonShape ps;
    ps.SetAsBox(0.2f, 0.2f);
    MakeFixture(b, &ps, 0.0f);
    c.fixtures++;
    return b;
  };
  for (int r = 0; r < rigs; ++r) {
    const float x0 = -0.5f * pitch * (float)rigs + pitch * (float)r + 2.0f;
    const float jit = rng.uni(-0.2f, 0.2f);
    const float hz = rng.uni(2.0f, 3.5f);
    // pendulum on a rigid rod
    {
      b2Body* post = staticPost(x0, 8.0f);
      b2Body* b = dynamicBox(x0 + 3.0f + jit, 8.5f, 0.2f);
      b2DistanceJointDef jd;
      jd.Initialize(post, b, post->GetPosition(), b->GetPosition());
      world->CreateJoint(&jd);
      c.joints++;
    }
    // spring with limits, started stretched
    {
      b2Body* post = staticPost(x0 + 5.0f, 9.0f);
      b2Body* b = dynamicBox(x0 + 5.0f + jit, 4.0f, 0.0f);
      b2DistanceJointDef jd;
      jd.Initialize(post, b, post->GetPosition(), b->GetPosition() + b2Vec2(0.0f, 0.3f));
      jd.length = 2.5f;
      jd.minLength = 1.5f;
      jd.maxLength = 5.0f;
      b2LinearStiffness(jd.stiffness, jd.damping, hz, 0.3f, post, b);
      world->CreateJoint(&jd);
      c.joints++;
    }
    // rope of four boxes: slack distance joints (min 0, max = rest + 0.2)
    {
      b2Body* prev = staticPost(x0 + 8.0f, 9.0f);
      for (int k = 0; k < 4; ++k) {
        b2Body* b = dynamicBox(x0 + 9.0f + 1.2f * (float)k, 9.0f + jit * (float)k, 0.0f);
        b2DistanceJointDef jd;
        b2Vec2 pa = prev->GetPosition() + b2Vec2(k == 0 ? 0.0f : 0.4f, 0.0f);
        b2Vec2 pb = b->GetPosition() - b2Vec2(0.4f, 0.0f);
        jd.Initialize(prev, b, pa, pb);
        jd.minLength = 0.0f;
        jd.maxLength = jd.length + 0.2f;
        jd.stiffness = 0.0f;
        world->CreateJoint(&jd);
        c.joints++;
        prev = b;
      }
    }
    // elevator: vertical axis, limits, motor up
    {
      b2Body* b = dynamicBox(x0 + 15.0f, 1.0f, 0.0f);
      b2PrismaticJointDef jd;
      jd.Initialize(ground, b, b->GetPosition(), b2Vec2(0.0f, 1.0f));
      jd.enableLimit = true;
      jd.lowerTranslation = -0.5f;
      jd.upperTranslation = 3.0f + jit;
      jd.enableMotor = true;
      jd.maxMotorForce = 30.0f;
      jd.motorSpeed = 2.0f;
      world->CreateJoint(&jd);
      c.joints++;
      dynamicBox(x0 + 15.0f + 0.1f * jit, 2.5f, 0.0f);  // a passenger
    }
    // slider on a tilted axis with a lower stop, and a box dropped on it
    {
      b2Body* post = staticPost(x0 + 18.0f, 5.0f);
      b2Body* b = dynamicBox(x0 + 18.0f, 6.0f, 0.5f);
      b2PrismaticJointDef jd;
      b2Vec2 axis(0.8f, -0.6f);
      axis.Normalize();
      jd.Initialize(post, b, b->GetPosition(), axis);
      jd.enableLimit = true;
      jd.lowerTranslation = -0.5f;
      jd.upperTranslation = 2.5f + jit;
      world->CreateJoint(&jd);
      c.joints++;
      dynamicBox(x0 + 18.3f, 8.0f, 0.1f);
    }
    // piston between two dynamic boxes on the ground
    {
      b2Body* a = dynamicBox(x0 + 21.0f, 0.3f, 0.0f);
      b2Body* b = dynamicBox(x0 + 22.0f, 0.3f, 0.0f);
      b2PrismaticJointDef jd;
      jd.Initialize(a, b, a->GetPosition(), b2Vec2(1.0f, 0.0f));
      jd.enableLimit = true;
      jd.lowerTranslation = 0.5f;
      jd.upperTranslation = 2.0f;
      jd.enableMotor = true;
      jd.maxMotorForce = 10.0f + 10.0f * jit;
      jd.motorSpeed = 1.0f;
      world->CreateJoint(&jd);
      c.joints++;
    }
  }
  return c;
}

// `rigs` rigs side by side over one ground edge, each:
//  * a wheel pair: a disc (r 1) on a motorised revolute joint to a static post and a disc (r 0.5)
//    on a free one, geared 1 : 2 so that their rims turn together (ratio 2);
//  * a rack and pinion: a disc (r 0.6) on a motorised revolute joint and a bar on a horizontal
//    prismatic joint with limits, geared so that the bar moves with the disc's rim (ratio
//    -1 / 0.6) until it reaches a limit;
//  * a geared double pendulum: an arm hinged to a post and a second arm hinged to the first,
//    the two hinges geared (ratio 1); the second joint's body A is the first arm, so the gear's
//    bodies A and D are one body;
//  * boxes dropped onto the wheels and the bar.
inline Counts GearRigs(b2World* world, int rigs, uint32_t seed, float friction = 0.6f) {
  Counts c;
  Rng rng(seed);
  if (rigs < 1) rigs = 1;
  const float pitch = 18.0f;
  const float half = 0.5f * pitch * (float)rigs + 20.0f;
  b2BodyDef gd;
  b2Body* ground = MakeBody(world, &gd);
  AddEdge(ground, -half, 0.0f, half, 0.0f, &c);
  auto disc = [&](float x, float y, float r) {
    b2BodyDef bd;
    bd.type = b2_dynamicBody;
    bd.position.Set(x, y);
    b2Body* b = MakeBody(world, &bd);
    b2CircleShape cs;
    cs.m_radius = r;
    b2FixtureDef fd;
    fd.shape = &cs;
    fd.density = 1.0f;
    fd.friction = friction;
    MakeFixture(b, &fd);
    c.bodies++;
    c.fixtures++;
    return b;
  };
  auto box = [&](float x, float y, float hx, float hy, float angle) {
    b2BodyDef bd;
    bd.type = b2_dynamicBody;
    bd.position.Set(x, y);
    bd.angle = angle;
    b2Body* b = MakeBody(world, &bd);
    b2PolygonShape ps;
    ps.SetAsBox(hx, hy);
    b2FixtureDef fd;
    fd.shape = &ps;
    fd.density = 1.0f;
    fd.friction = friction;
    MakeFixture(b, &fd);
    c.bodies++;
    c.fixtures++;
    return b;
  };
  auto hinge = [&](b2Body* a, b2Body* b, b2Vec2 at) {
    b2RevoluteJointDef jd;
    jd.Initialize(a, b, at);
    c.joints++;
    return world->CreateJoint(&jd);
  };
  auto gear = [&](b2Joint* j1, b2Joint* j2, float ratio) {
    b2GearJointDef jd;
    jd.bodyA = j1->GetBodyB();
    jd.bodyB = j2->GetBodyB();
    jd.joint1 = j1;
    jd.joint2 = j2;
    jd.ratio = ratio;
    c.joints++;
    return world->CreateJoint(&jd);
  };
  for (int r = 0; r < rigs; ++r) {
    const float x0 = -0.5f * pitch * (float)rigs + pitch * (float)r + 2.0f;
    const float jit = rng.uni(-0.2f, 0.2f);
    // wheel pair
    {
      b2Body* big = disc(x0, 5.0f, 1.0f);
      b2Body* small = disc(x0 + 1.6f, 5.0f, 0.5f);
      b2RevoluteJointDef jd;
      jd.Initialize(ground, big, big->GetPosition());
      jd.enableMotor = true;
      jd.motorSpeed = 1.0f + jit;
      jd.maxMotorTorque = 20.0f;
      b2Joint* j1 = world->CreateJoint(&jd);
      c.joints++;
      b2Joint* j2 = hinge(ground, small, small->GetPosition());
      gear(j1, j2, 2.0f);
      box(x0 + 0.3f + jit, 8.0f, 0.3f, 0.3f, 0.2f);
    }
    // rack and pinion
    {
      b2Body* pinion = disc(x0 + 7.0f, 3.0f, 0.6f);
      b2RevoluteJointDef pj;
      pj.Initialize(ground, pinion, pinion->GetPosition());
      pj.enableMotor = true;
      pj.motorSpeed = -1.5f - jit;
      pj.maxMotorTorque = 15.0f;
      b2Joint* j3 = world->CreateJoint(&pj);
      c.joints++;
      b2Body* bar = box(x0 + 7.0f, 2.2f, 2.0f, 0.2f, 0.0f);
      b2PrismaticJointDef pd;
      pd.Initialize(ground, bar, bar->GetPosition(), b2Vec2(1.0f, 0.0f));
      pd.enableLimit = true;
      pd.lowerTranslation = -3.0f;
      pd.upperTranslation = 3.0f;
      b2Joint* j4 = world->CreateJoint(&pd);
      c.joints++;
      gear(j3, j4, -1.0f / 0.6f);
      box(x0 + 8.5f, 4.0f + jit, 0.3f, 0.3f, 0.0f);
    }
    // geared double pendulum
    {
      b2Body* arm1 = box(x0 + 12.5f, 6.0f, 1.0f, 0.1f, 0.0f);
      b2Body* arm2 = box(x0 + 14.5f, 6.0f, 1.0f, 0.1f, 0.0f);
      b2Joint* j5 = hinge(ground, arm1, b2Vec2(x0 + 11.5f, 6.0f));
      b2Joint* j6 = hinge(arm1, arm2, b2Vec2(x0 + 13.5f, 6.0f));
      gear(j5, j6, 1.0f);
    }
  }
  return c;
}

}  // namespace b2scenes
