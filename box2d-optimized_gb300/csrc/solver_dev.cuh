// solver_dev.cuh - per-constraint device routines of the sequential-impulse solver.
//
// Contact constraints: b2ContactSolver (src/dynamics/b2_contact_solver.cpp) split per
// constraint: prepare (Initialize + InitializeVelocityConstraints, :65-258), warm start
// (:260-299), velocity solve with the 2-point block solver (:301-639), position solve
// (:659-787). Joints: b2RevoluteJoint, b2PrismaticJoint and b2DistanceJoint
// Init/SolveVelocity/SolvePosition. Each routine reads and writes only its two bodies, so
// constraints of one colour run concurrently. Operation order follows the reference.
#pragma once

#include "b2g_math.cuh"
#include "engine.h"

namespace b2g {

struct SBody {
  V2 c; float a; V2 v; float w;
};

B2G_HD V2 ld2(const float* p) { return mk(p[0], p[1]); }
B2G_HD void st2(float* p, V2 v) { p[0] = v.x; p[1] = v.y; }

// Prepare one contact constraint from its manifold and the (velocity-integrated) body state.
B2G_HD void prepareContact(VCDev& vc, const b2g_manifold& m, float4 mat, float radiusA, float radiusB,
                           int ia, int ib, float4 massA, float4 massB, float2 lcA, float2 lcB, float4 posA,
                           float4 velA, float4 posB, float4 velB, float dtRatio, bool warm, int contact) {
  vc.friction = mat.x;
  float restitution = mat.y;
  float threshold = mat.z;
  vc.tangentSpeed = mat.w;
  vc.indexA = ia;
  vc.indexB = ib;
  vc.invMassA = massA.y;
  vc.invMassB = massB.y;
  vc.invIA = massA.w;
  vc.invIB = massB.w;
  vc.pointCount = m.point_count;
  vc.contact = contact;
  vc.localCenterA[0] = lcA.x; vc.localCenterA[1] = lcA.y;
  vc.localCenterB[0] = lcB.x; vc.localCenterB[1] = lcB.y;
  vc.localNormal[0] = m.local_normal[0]; vc.localNormal[1] = m.local_normal[1];
  vc.localPoint[0] = m.local_point[0]; vc.localPoint[1] = m.local_point[1];
  vc.pcPointCount = m.point_count;
  vc.radiusA = radiusA;
  vc.radiusB = radiusB;
  vc.type = m.type;
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    vc.normalImpulse[j] = 0.0f; vc.tangentImpulse[j] = 0.0f;
    vc.normalMass[j] = 0.0f; vc.tangentMass[j] = 0.0f; vc.velocityBias[j] = 0.0f;
    vc.rA[j][0] = vc.rA[j][1] = vc.rB[j][0] = vc.rB[j][1] = 0.0f;
    vc.localPoints[j][0] = m.points[j].local_point[0];
    vc.localPoints[j][1] = m.points[j].local_point[1];
  }
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    if (j >= m.point_count) break;
    if (warm) {
      vc.normalImpulse[j] = dtRatio * m.points[j].normal_impulse;
      vc.tangentImpulse[j] = dtRatio * m.points[j].tangent_impulse;
    }
  }
  // InitializeVelocityConstraints
  float mA = vc.invMassA, mB = vc.invMassB, iA = vc.invIA, iB = vc.invIB;
  V2 cA = mk(posA.x, posA.y); float aA = posA.z; V2 vA = mk(velA.x, velA.y); float wA = velA.z;
  V2 cB = mk(posB.x, posB.y); float aB = posB.z; V2 vB = mk(velB.x, velB.y); float wB = velB.z;
  Xf xfA, xfB;
  xfA.q = rotOf(aA);
  xfB.q = rotOf(aB);
  xfA.p = cA - mul(xfA.q, ld2(vc.localCenterA));
  xfB.p = cB - mul(xfB.q, ld2(vc.localCenterB));
  WorldMan wm;
  V2 lp[2] = {ld2(vc.localPoints[0]), ld2(vc.localPoints[1])};
  wm.normal = mk(0.0f, 0.0f);
  wm.points[0] = wm.points[1] = mk(0.0f, 0.0f);
  worldManifold(&wm, m.type, m.point_count, ld2(vc.localNormal), ld2(vc.localPoint), lp, xfA, radiusA, xfB, radiusB);
  V2 normal = wm.normal;
  st2(vc.normal, normal);
  V2 tangent = cross(normal, 1.0f);
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    if (j >= vc.pointCount) break;
    V2 rA = wm.points[j] - cA;
    V2 rB = wm.points[j] - cB;
    st2(vc.rA[j], rA);
    st2(vc.rB[j], rB);
    float rnA = cross(rA, normal);
    float rnB = cross(rB, normal);
    float kNormal = mA + mB + iA * rnA * rnA + iB * rnB * rnB;
    vc.normalMass[j] = kNormal > 0.0f ? 1.0f / kNormal : 0.0f;
    float rtA = cross(rA, tangent);
    float rtB = cross(rB, tangent);
    float kTangent = mA + mB + iA * rtA * rtA + iB * rtB * rtB;
    vc.tangentMass[j] = kTangent > 0.0f ? 1.0f / kTangent : 0.0f;
    vc.velocityBias[j] = 0.0f;
    float vRel = dot(normal, (vB + cross(wB, rB)) - (vA + cross(wA, rA)));
    if (vRel < -threshold) vc.velocityBias[j] = -restitution * vRel;
  }
  if (vc.pointCount == 2) {
    V2 r1A = ld2(vc.rA[0]), r1B = ld2(vc.rB[0]), r2A = ld2(vc.rA[1]), r2B = ld2(vc.rB[1]);
    float rn1A = cross(r1A, normal);
    float rn1B = cross(r1B, normal);
    float rn2A = cross(r2A, normal);
    float rn2B = cross(r2B, normal);
    float k11 = mA + mB + iA * rn1A * rn1A + iB * rn1B * rn1B;
    float k22 = mA + mB + iA * rn2A * rn2A + iB * rn2B * rn2B;
    float k12 = mA + mB + iA * rn1A * rn2A + iB * rn1B * rn2B;
    const float k_maxConditionNumber = 1000.0f;
    if (k11 * k11 < k_maxConditionNumber * (k11 * k22 - k12 * k12)) {
      M22 K;
      K.ex = mk(k11, k12);
      K.ey = mk(k12, k22);
      M22 NM = inverse(K);
      vc.K[0] = K.ex.x; vc.K[1] = K.ex.y; vc.K[2] = K.ey.x; vc.K[3] = K.ey.y;
      vc.NM[0] = NM.ex.x; vc.NM[1] = NM.ex.y; vc.NM[2] = NM.ey.x; vc.NM[3] = NM.ey.y;
    } else {
      vc.pointCount = 1;
    }
  }
}

B2G_HD void loadVel(const float4* vel, int i, V2& v, float& w) {
  float4 x = vel[i];
  v = mk(x.x, x.y);
  w = x.z;
}
B2G_HD void storeVel(float4* vel, int i, V2 v, float w) { vel[i] = make_float4(v.x, v.y, w, 0.0f); }
// A body with zero inverse mass and inertia (static, or massless) is left untouched: its update
// would be v - 0*P, a no-op, and skipping it keeps constraints of one colour that share such a
// body from writing the same address.
B2G_HD bool moves(float invMass, float invI) { return invMass != 0.0f || invI != 0.0f; }
B2G_HD void loadPos(const float4* pos, int i, V2& c, float& a) {
  float4 x = pos[i];
  c = mk(x.x, x.y);
  a = x.z;
}
B2G_HD void storePos(float4* pos, int i, V2 c, float a) { pos[i] = make_float4(c.x, c.y, a, 0.0f); }

// b2ContactSolver::WarmStart for one constraint.
B2G_HD void warmStartContact(const VCDev& vc, float4* vel) {
  float mA = vc.invMassA, iA = vc.invIA, mB = vc.invMassB, iB = vc.invIB;
  V2 vA, vB; float wA, wB;
  loadVel(vel, vc.indexA, vA, wA);
  loadVel(vel, vc.indexB, vB, wB);
  V2 normal = ld2(vc.normal);
  V2 tangent = cross(normal, 1.0f);
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    if (j >= vc.pointCount) break;
    V2 P = vc.normalImpulse[j] * normal + vc.tangentImpulse[j] * tangent;
    wA -= iA * cross(ld2(vc.rA[j]), P);
    subFrom(vA, mA * P);
    wB += iB * cross(ld2(vc.rB[j]), P);
    addTo(vB, mB * P);
  }
  if (moves(mA, iA)) storeVel(vel, vc.indexA, vA, wA);
  if (moves(mB, iB)) storeVel(vel, vc.indexB, vB, wB);
}

// b2ContactSolver::SolveVelocityConstraints for one constraint (friction, then normal with the
// 2-point block solver's total enumeration of the four LCP cases).
B2G_HD void solveContactVelocity(VCDev& vc, float4* vel) {
  float mA = vc.invMassA, iA = vc.invIA, mB = vc.invMassB, iB = vc.invIB;
  int pointCount = vc.pointCount;
  V2 vA, vB; float wA, wB;
  loadVel(vel, vc.indexA, vA, wA);
  loadVel(vel, vc.indexB, vB, wB);
  V2 normal = ld2(vc.normal);
  V2 tangent = cross(normal, 1.0f);
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    if (j >= pointCount) break;
    V2 rA = ld2(vc.rA[j]), rB = ld2(vc.rB[j]);
    V2 dv = (vB + cross(wB, rB)) - (vA + cross(wA, rA));
    float vt = dot(dv, tangent) - vc.tangentSpeed;
    float lambda = vc.tangentMass[j] * (-vt);
    float maxFriction = vc.friction * vc.normalImpulse[j];
    float newImpulse = fclamp(vc.tangentImpulse[j] + lambda, -maxFriction, maxFriction);
    lambda = newImpulse - vc.tangentImpulse[j];
    vc.tangentImpulse[j] = newImpulse;
    V2 P = lambda * tangent;
    subFrom(vA, mA * P);
    wA -= iA * cross(rA, P);
    addTo(vB, mB * P);
    wB += iB * cross(rB, P);
  }
  if (pointCount == 1) {
    V2 rA = ld2(vc.rA[0]), rB = ld2(vc.rB[0]);
    V2 dv = (vB + cross(wB, rB)) - (vA + cross(wA, rA));
    float vn = dot(dv, normal);
    float lambda = -vc.normalMass[0] * (vn - vc.velocityBias[0]);
    float newImpulse = fmax2(vc.normalImpulse[0] + lambda, 0.0f);
    lambda = newImpulse - vc.normalImpulse[0];
    vc.normalImpulse[0] = newImpulse;
    V2 P = lambda * normal;
    subFrom(vA, mA * P);
    wA -= iA * cross(rA, P);
    addTo(vB, mB * P);
    wB += iB * cross(rB, P);
  } else {
    V2 r1A = ld2(vc.rA[0]), r1B = ld2(vc.rB[0]), r2A = ld2(vc.rA[1]), r2B = ld2(vc.rB[1]);
    M22 K, NM;
    K.ex = mk(vc.K[0], vc.K[1]); K.ey = mk(vc.K[2], vc.K[3]);
    NM.ex = mk(vc.NM[0], vc.NM[1]); NM.ey = mk(vc.NM[2], vc.NM[3]);
    V2 a = mk(vc.normalImpulse[0], vc.normalImpulse[1]);
    V2 dv1 = (vB + cross(wB, r1B)) - (vA + cross(wA, r1A));
    V2 dv2 = (vB + cross(wB, r2B)) - (vA + cross(wA, r2A));
    float vn1 = dot(dv1, normal);
    float vn2 = dot(dv2, normal);
    V2 b;
    b.x = vn1 - vc.velocityBias[0];
    b.y = vn2 - vc.velocityBias[1];
    subFrom(b, mul(K, a));
    V2 x;
    bool solved = false;
    // Case 1: vn = 0
    x = -mul(NM, b);
    if (x.x >= 0.0f && x.y >= 0.0f) {
      solved = true;
    } else {
      // Case 2: vn1 = 0 and x2 = 0
      x.x = -vc.normalMass[0] * b.x;
      x.y = 0.0f;
      vn2 = K.ex.y * x.x + b.y;
      if (x.x >= 0.0f && vn2 >= 0.0f) {
        solved = true;
      } else {
        // Case 3: vn2 = 0 and x1 = 0
        x.x = 0.0f;
        x.y = -vc.normalMass[1] * b.y;
        vn1 = K.ey.x * x.y + b.x;
        if (x.y >= 0.0f && vn1 >= 0.0f) {
          solved = true;
        } else {
          // Case 4: x1 = 0 and x2 = 0
          x.x = 0.0f;
          x.y = 0.0f;
          vn1 = b.x;
          vn2 = b.y;
          if (vn1 >= 0.0f && vn2 >= 0.0f) solved = true;
        }
      }
    }
    if (solved) {
      V2 d = x - a;
      V2 P1 = d.x * normal;
      V2 P2 = d.y * normal;
      subFrom(vA, mA * (P1 + P2));
      wA -= iA * (cross(r1A, P1) + cross(r2A, P2));
      addTo(vB, mB * (P1 + P2));
      wB += iB * (cross(r1B, P1) + cross(r2B, P2));
      vc.normalImpulse[0] = x.x;
      vc.normalImpulse[1] = x.y;
    }
  }
  if (moves(mA, iA)) storeVel(vel, vc.indexA, vA, wA);
  if (moves(mB, iB)) storeVel(vel, vc.indexB, vB, wB);
}

// b2PositionSolverManifold + SolvePositionConstraints for one constraint; returns its minimum
// separation (starting from 0 as the reference's minSeparation does).
B2G_HD float solveContactPosition(const VCDev& vc, float4* pos) {
  float minSeparation = 0.0f;
  V2 localCenterA = ld2(vc.localCenterA), localCenterB = ld2(vc.localCenterB);
  float mA = vc.invMassA, iA = vc.invIA, mB = vc.invMassB, iB = vc.invIB;
  V2 cA, cB; float aA, aB;
  loadPos(pos, vc.indexA, cA, aA);
  loadPos(pos, vc.indexB, cB, aB);
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    if (j >= vc.pcPointCount) break;
    Xf xfA, xfB;
    xfA.q = rotOf(aA);
    xfB.q = rotOf(aB);
    xfA.p = cA - mul(xfA.q, localCenterA);
    xfB.p = cB - mul(xfB.q, localCenterB);
    V2 normal, point;
    float separation;
    if (vc.type == B2G_MANIFOLD_CIRCLES) {
      V2 pointA = mul(xfA, ld2(vc.localPoint));
      V2 pointB = mul(xfB, ld2(vc.localPoints[0]));
      normal = pointB - pointA;
      normalize(normal);
      point = 0.5f * (pointA + pointB);
      separation = (dot(pointB - pointA, normal) - vc.radiusA) - vc.radiusB;
    } else if (vc.type == B2G_MANIFOLD_FACE_A) {
      normal = mul(xfA.q, ld2(vc.localNormal));
      V2 planePoint = mul(xfA, ld2(vc.localPoint));
      V2 clipPoint = mul(xfB, ld2(vc.localPoints[j]));
      separation = (dot(clipPoint - planePoint, normal) - vc.radiusA) - vc.radiusB;
      point = clipPoint;
    } else {
      normal = mul(xfB.q, ld2(vc.localNormal));
      V2 planePoint = mul(xfB, ld2(vc.localPoint));
      V2 clipPoint = mul(xfA, ld2(vc.localPoints[j]));
      separation = (dot(clipPoint - planePoint, normal) - vc.radiusA) - vc.radiusB;
      point = clipPoint;
      normal = -normal;
    }
    V2 rA = point - cA;
    V2 rB = point - cB;
    minSeparation = fmin2(minSeparation, separation);
    float C = fclamp(B2G_BAUMGARTE * (separation + B2G_LINEAR_SLOP), -B2G_MAX_LINEAR_CORRECTION, 0.0f);
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
  if (moves(mA, iA)) storePos(pos, vc.indexA, cA, aA);
  if (moves(mB, iB)) storePos(pos, vc.indexB, cB, aB);
  return minSeparation;
}

// ---- joints -----------------------------------------------------------------------------
B2G_HD M22 ldK(const float* k) { M22 m; m.ex = mk(k[0], k[1]); m.ey = mk(k[2], k[3]); return m; }
B2G_HD void stK(float* k, const M22& m) { k[0] = m.ex.x; k[1] = m.ex.y; k[2] = m.ey.x; k[3] = m.ey.y; }

// b2Mat33 (weld): K from the anchors, and GetInverse22 / GetSymInverse33 (src/common/b2_math.cpp:
// 55-97) into 9 floats (ex, ey, ez).
B2G_HD void weldK(V2 rA, V2 rB, float mA, float mB, float iA, float iB, V3& ex, V3& ey, V3& ez) {
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
B2G_HD void inverse22(V3 ex, V3 ey, float* M) {
  float a = ex.x, b = ey.x, c = ex.y, d = ey.y;
  float det = a * d - b * c;
  if (det != 0.0f) det = 1.0f / det;
  M[0] = det * d;  M[3] = -det * b; M[2] = 0.0f;
  M[1] = -det * c; M[4] = det * a;  M[5] = 0.0f;
  M[6] = 0.0f; M[7] = 0.0f; M[8] = 0.0f;
}
B2G_HD void symInverse33(V3 ex, V3 ey, V3 ez, float* M) {
  float det = dot3(ex, cross3(ey, ez));
  if (det != 0.0f) det = 1.0f / det;
  float a11 = ex.x, a12 = ey.x, a13 = ez.x;
  float a22 = ey.y, a23 = ez.y;
  float a33 = ez.z;
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
// b2Mat33::Solve22 (b2_math.cpp:42-53)
B2G_HD V2 solve22(V3 ex, V3 ey, V2 b) {
  float a11 = ex.x, a12 = ey.x, a21 = ex.y, a22 = ey.y;
  float det = a11 * a22 - a12 * a21;
  if (det != 0.0f) det = 1.0f / det;
  return mk(det * (a22 * b.x - a12 * b.y), det * (a11 * b.y - a21 * b.x));
}
// Linear/angular mass of the motor and friction joints (b2_motor_joint.cpp:91-104,
// b2_friction_joint.cpp:88-101): K in the reference's operand order, inverted.
B2G_HD void linearAngularMass(JointDev& J, V2 rA, V2 rB, float mA, float mB, float iA, float iB) {
  M22 K;
  K.ex.x = mA + mB + iA * rA.y * rA.y + iB * rB.y * rB.y;
  K.ex.y = -iA * rA.x * rA.y - iB * rB.x * rB.y;
  K.ey.x = K.ex.y;
  K.ey.y = mA + mB + iA * rA.x * rA.x + iB * rB.x * rB.x;
  stK(J.K, inverse(K));
  J.axialMass = iA + iB;
  if (J.axialMass > 0.0f) J.axialMass = 1.0f / J.axialMass;
}
// The clamped linear and angular impulses of the motor and friction joints
// (b2_motor_joint.cpp:157-193, b2_friction_joint.cpp:144-180); the motor adds its position-error
// feedback to both velocity errors (friction adds nothing: not even a zero, which could turn the
// sign of a zero velocity error).
B2G_HD void solveLinearAngular(JointDev& J, V2& vA, float& wA, V2& vB, float& wB, float h, bool feedback,
                               float angBias, V2 linBias) {
  float mA = J.mA, mB = J.mB, iA = J.invIA, iB = J.invIB;
  V2 rA = ld2(J.rA), rB = ld2(J.rB);
  {
    float Cdot = wB - wA;
    if (feedback) Cdot = Cdot + angBias;
    float impulse = -J.axialMass * Cdot;
    float oldImpulse = J.impulse[2];
    float maxImpulse = h * J.d.max_torque;
    J.impulse[2] = fclamp(J.impulse[2] + impulse, -maxImpulse, maxImpulse);
    impulse = J.impulse[2] - oldImpulse;
    wA -= iA * impulse;
    wB += iB * impulse;
  }
  {
    V2 Cdot = ((vB + cross(wB, rB)) - vA) - cross(wA, rA);
    if (feedback) Cdot = Cdot + linBias;
    V2 impulse = -mul(ldK(J.K), Cdot);
    V2 oldImpulse = mk(J.impulse[0], J.impulse[1]);
    V2 acc = oldImpulse + impulse;
    float maxImpulse = h * J.d.max_force;
    if (lengthSq(acc) > maxImpulse * maxImpulse) {
      normalize(acc);
      acc.x *= maxImpulse;
      acc.y *= maxImpulse;
    }
    J.impulse[0] = acc.x; J.impulse[1] = acc.y;
    impulse = acc - oldImpulse;
    subFrom(vA, mA * impulse);
    wA -= iA * cross(rA, impulse);
    addTo(vB, mB * impulse);
    wB += iB * cross(rB, impulse);
  }
}

// InitVelocityConstraints (revolute :73-165, prismatic :114-224, distance :76-173).
B2G_HD void jointInit(JointDev& J, const float4* massd, const float2* lc, const float4* pos, float4* vel, float dt,
                      float dtRatio, bool warm) {
  int ia = J.d.body_a, ib = J.d.body_b;
  J.iA = ia; J.iB = ib;
  float2 la2 = lc[ia], lb2 = lc[ib];
  J.lcA[0] = la2.x; J.lcA[1] = la2.y; J.lcB[0] = lb2.x; J.lcB[1] = lb2.y;
  float4 mdA = massd[ia], mdB = massd[ib];
  J.mA = mdA.y; J.mB = mdB.y; J.invIA = mdA.w; J.invIB = mdB.w;
  V2 cA, cB, vA, vB; float aA, aB, wA, wB;
  loadPos(pos, ia, cA, aA); loadVel(vel, ia, vA, wA);
  loadPos(pos, ib, cB, aB); loadVel(vel, ib, vB, wB);
  Rot qA = rotOf(aA), qB = rotOf(aB);
  V2 la = ld2(J.d.local_anchor_a), lb = ld2(J.d.local_anchor_b);
  V2 lcA = ld2(J.lcA), lcB = ld2(J.lcB);
  float mA = J.mA, mB = J.mB, iA = J.invIA, iB = J.invIB;
  if (J.d.type == B2G_JOINT_REVOLUTE) {
    V2 rA = mul(qA, la - lcA);
    V2 rB = mul(qB, lb - lcB);
    st2(J.rA, rA); st2(J.rB, rB);
    M22 K;
    K.ex.x = mA + mB + rA.y * rA.y * iA + rB.y * rB.y * iB;
    K.ey.x = -rA.y * rA.x * iA - rB.y * rB.x * iB;
    K.ex.y = K.ey.x;
    K.ey.y = mA + mB + rA.x * rA.x * iA + rB.x * rB.x * iB;
    stK(J.K, K);
    J.axialMass = iA + iB;
    bool fixedRotation;
    if (J.axialMass > 0.0f) { J.axialMass = 1.0f / J.axialMass; fixedRotation = false; }
    else fixedRotation = true;
    J.angle = aB - aA - J.d.reference_angle;
    if (J.d.enable_limit == 0 || fixedRotation) { J.lowerImpulse = 0.0f; J.upperImpulse = 0.0f; }
    if (J.d.enable_motor == 0 || fixedRotation) J.motorImpulse = 0.0f;
    if (warm) {
      J.impulse[0] *= dtRatio; J.impulse[1] *= dtRatio;
      J.motorImpulse *= dtRatio; J.lowerImpulse *= dtRatio; J.upperImpulse *= dtRatio;
      float axialImpulse = J.motorImpulse + J.lowerImpulse - J.upperImpulse;
      V2 P = mk(J.impulse[0], J.impulse[1]);
      subFrom(vA, mA * P);
      wA -= iA * (cross(rA, P) + axialImpulse);
      addTo(vB, mB * P);
      wB += iB * (cross(rB, P) + axialImpulse);
    } else {
      J.impulse[0] = 0.0f; J.impulse[1] = 0.0f;
      J.motorImpulse = 0.0f; J.lowerImpulse = 0.0f; J.upperImpulse = 0.0f;
    }
  } else if (J.d.type == B2G_JOINT_PRISMATIC) {
    V2 rA = mul(qA, la - lcA);
    V2 rB = mul(qB, lb - lcB);
    V2 d = ((cB - cA) + rB) - rA;
    V2 axis = mul(qA, ld2(J.localXAxisA));
    float a1 = cross(d + rA, axis);
    float a2 = cross(rB, axis);
    st2(J.axis, axis);
    J.a1 = a1; J.a2 = a2;
    J.axialMass = mA + mB + iA * a1 * a1 + iB * a2 * a2;
    if (J.axialMass > 0.0f) J.axialMass = 1.0f / J.axialMass;
    V2 perp = mul(qA, ld2(J.localYAxisA));
    st2(J.perp, perp);
    J.s1 = cross(d + rA, perp);
    J.s2 = cross(rB, perp);
    float k11 = mA + mB + iA * J.s1 * J.s1 + iB * J.s2 * J.s2;
    float k12 = iA * J.s1 + iB * J.s2;
    float k22 = iA + iB;
    if (k22 == 0.0f) k22 = 1.0f;
    M22 K;
    K.ex = mk(k11, k12);
    K.ey = mk(k12, k22);
    stK(J.K, K);
    if (J.d.enable_limit) J.translation = dot(axis, d);
    else { J.lowerImpulse = 0.0f; J.upperImpulse = 0.0f; }
    if (J.d.enable_motor == 0) J.motorImpulse = 0.0f;
    if (warm) {
      J.impulse[0] *= dtRatio; J.impulse[1] *= dtRatio;
      J.motorImpulse *= dtRatio; J.lowerImpulse *= dtRatio; J.upperImpulse *= dtRatio;
      float axialImpulse = J.motorImpulse + J.lowerImpulse - J.upperImpulse;
      V2 P = J.impulse[0] * perp + axialImpulse * axis;
      float LA = J.impulse[0] * J.s1 + J.impulse[1] + axialImpulse * a1;
      float LB = J.impulse[0] * J.s2 + J.impulse[1] + axialImpulse * a2;
      subFrom(vA, mA * P);
      wA -= iA * LA;
      addTo(vB, mB * P);
      wB += iB * LB;
    } else {
      J.impulse[0] = 0.0f; J.impulse[1] = 0.0f;
      J.motorImpulse = 0.0f; J.lowerImpulse = 0.0f; J.upperImpulse = 0.0f;
    }
  } else if (J.d.type == B2G_JOINT_DISTANCE) {
    V2 rA = mul(qA, la - lcA);
    V2 rB = mul(qB, lb - lcB);
    st2(J.rA, rA); st2(J.rB, rB);
    V2 u = ((cB + rB) - cA) - rA;
    J.currentLength = lengthOf(u);
    if (J.currentLength > B2G_LINEAR_SLOP) {
      u = (1.0f / J.currentLength) * u;
    } else {
      u = mk(0.0f, 0.0f);
      J.mass = 0.0f; J.impulse[0] = 0.0f; J.lowerImpulse = 0.0f; J.upperImpulse = 0.0f;
    }
    st2(J.u, u);
    float crAu = cross(rA, u);
    float crBu = cross(rB, u);
    float invMass = J.mA + J.invIA * crAu * crAu + J.mB + J.invIB * crBu * crBu;
    J.mass = invMass != 0.0f ? 1.0f / invMass : 0.0f;
    if (J.d.stiffness > 0.0f && J.d.min_length < J.d.max_length) {
      float C = J.currentLength - J.d.length;
      float dd = J.d.damping;
      float k = J.d.stiffness;
      float h = dt;
      J.gamma = h * (dd + h * k);
      J.gamma = J.gamma != 0.0f ? 1.0f / J.gamma : 0.0f;
      J.bias = C * h * k * J.gamma;
      invMass += J.gamma;
      J.softMass = invMass != 0.0f ? 1.0f / invMass : 0.0f;
    } else {
      J.gamma = 0.0f; J.bias = 0.0f; J.softMass = J.mass;
    }
    if (warm) {
      J.impulse[0] *= dtRatio; J.lowerImpulse *= dtRatio; J.upperImpulse *= dtRatio;
      V2 P = ((J.impulse[0] + J.lowerImpulse) - J.upperImpulse) * u;
      subFrom(vA, J.mA * P);
      wA -= J.invIA * cross(rA, P);
      addTo(vB, J.mB * P);
      wB += J.invIB * cross(rB, P);
    } else {
      J.impulse[0] = 0.0f;
    }
  } else if (J.d.type == B2G_JOINT_WELD) {  // b2_weld_joint.cpp:93-187
    V2 rA = mul(qA, la - lcA);
    V2 rB = mul(qB, lb - lcB);
    st2(J.rA, rA); st2(J.rB, rB);
    V3 ex, ey, ez;
    weldK(rA, rB, mA, mB, iA, iB, ex, ey, ez);
    if (J.d.stiffness > 0.0f) {
      inverse22(ex, ey, J.mass3);
      float invM = iA + iB;
      float C = aB - aA - J.d.reference_angle;
      float d = J.d.damping;
      float k = J.d.stiffness;
      float h = dt;
      J.gamma = h * (d + h * k);
      J.gamma = J.gamma != 0.0f ? 1.0f / J.gamma : 0.0f;
      J.bias = C * h * k * J.gamma;
      invM += J.gamma;
      J.mass3[8] = invM != 0.0f ? 1.0f / invM : 0.0f;
    } else if (ez.z == 0.0f) {
      inverse22(ex, ey, J.mass3);
      J.gamma = 0.0f;
      J.bias = 0.0f;
    } else {
      symInverse33(ex, ey, ez, J.mass3);
      J.gamma = 0.0f;
      J.bias = 0.0f;
    }
    if (warm) {
      J.impulse[0] *= dtRatio; J.impulse[1] *= dtRatio; J.impulse[2] *= dtRatio;
      V2 P = mk(J.impulse[0], J.impulse[1]);
      subFrom(vA, mA * P);
      wA -= iA * (cross(rA, P) + J.impulse[2]);
      addTo(vB, mB * P);
      wB += iB * (cross(rB, P) + J.impulse[2]);
    } else {
      J.impulse[0] = 0.0f; J.impulse[1] = 0.0f; J.impulse[2] = 0.0f;
    }
  } else if (J.d.type == B2G_JOINT_WHEEL) {  // b2_wheel_joint.cpp:89-211
    V2 rA = mul(qA, la - lcA);
    V2 rB = mul(qB, lb - lcB);
    V2 d = ((cB + rB) - cA) - rA;
    V2 ay = mul(qA, ld2(J.localYAxisA));
    J.s1 = cross(d + rA, ay);
    J.s2 = cross(rB, ay);
    st2(J.perp, ay);
    J.mass = mA + mB + iA * J.s1 * J.s1 + iB * J.s2 * J.s2;
    if (J.mass > 0.0f) J.mass = 1.0f / J.mass;
    V2 ax = mul(qA, ld2(J.localXAxisA));
    st2(J.axis, ax);
    J.a1 = cross(d + rA, ax);
    J.a2 = cross(rB, ax);
    const float invMass = mA + mB + iA * J.a1 * J.a1 + iB * J.a2 * J.a2;
    J.axialMass = invMass > 0.0f ? 1.0f / invMass : 0.0f;
    J.springMass = 0.0f;
    J.bias = 0.0f;
    J.gamma = 0.0f;
    if (J.d.stiffness > 0.0f && invMass > 0.0f) {
      J.springMass = 1.0f / invMass;
      float C = dot(d, ax);
      float h = dt;
      J.gamma = h * (J.d.damping + h * J.d.stiffness);
      if (J.gamma > 0.0f) J.gamma = 1.0f / J.gamma;
      J.bias = C * h * J.d.stiffness * J.gamma;
      J.springMass = invMass + J.gamma;
      if (J.springMass > 0.0f) J.springMass = 1.0f / J.springMass;
    } else {
      J.impulse[1] = 0.0f;
    }
    if (J.d.enable_limit) J.translation = dot(ax, d);
    else { J.lowerImpulse = 0.0f; J.upperImpulse = 0.0f; }
    if (J.d.enable_motor) {
      J.motorMass = iA + iB;
      if (J.motorMass > 0.0f) J.motorMass = 1.0f / J.motorMass;
    } else {
      J.motorMass = 0.0f;
      J.motorImpulse = 0.0f;
    }
    if (warm) {
      J.impulse[0] *= dtRatio; J.impulse[1] *= dtRatio; J.motorImpulse *= dtRatio;
      float axialImpulse = J.impulse[1] + J.lowerImpulse - J.upperImpulse;
      V2 P = J.impulse[0] * ay + axialImpulse * ax;
      float LA = J.impulse[0] * J.s1 + axialImpulse * J.a1 + J.motorImpulse;
      float LB = J.impulse[0] * J.s2 + axialImpulse * J.a2 + J.motorImpulse;
      subFrom(vA, mA * P);
      wA -= iA * LA;
      addTo(vB, mB * P);
      wB += iB * LB;
    } else {
      J.impulse[0] = 0.0f; J.impulse[1] = 0.0f; J.motorImpulse = 0.0f;
      J.lowerImpulse = 0.0f; J.upperImpulse = 0.0f;
    }
  } else if (J.d.type == B2G_JOINT_MOTOR) {  // b2_motor_joint.cpp:58-136
    V2 rA = mul(qA, ld2(J.d.linear_offset) - lcA);
    V2 rB = mul(qB, -lcB);
    st2(J.rA, rA); st2(J.rB, rB);
    linearAngularMass(J, rA, rB, mA, mB, iA, iB);
    st2(J.err, ((cB + rB) - cA) - rA);
    J.angularError = aB - aA - J.d.reference_angle;
    if (warm) {
      J.impulse[0] *= dtRatio; J.impulse[1] *= dtRatio; J.impulse[2] *= dtRatio;
      V2 P = mk(J.impulse[0], J.impulse[1]);
      subFrom(vA, mA * P);
      wA -= iA * (cross(rA, P) + J.impulse[2]);
      addTo(vB, mB * P);
      wB += iB * (cross(rB, P) + J.impulse[2]);
    } else {
      J.impulse[0] = 0.0f; J.impulse[1] = 0.0f; J.impulse[2] = 0.0f;
    }
  } else if (J.d.type == B2G_JOINT_FRICTION) {  // b2_friction_joint.cpp:60-123
    V2 rA = mul(qA, la - lcA);
    V2 rB = mul(qB, lb - lcB);
    st2(J.rA, rA); st2(J.rB, rB);
    linearAngularMass(J, rA, rB, mA, mB, iA, iB);
    if (warm) {
      J.impulse[0] *= dtRatio; J.impulse[1] *= dtRatio; J.impulse[2] *= dtRatio;
      V2 P = mk(J.impulse[0], J.impulse[1]);
      subFrom(vA, mA * P);
      wA -= iA * (cross(rA, P) + J.impulse[2]);
      addTo(vB, mB * P);
      wB += iB * (cross(rB, P) + J.impulse[2]);
    } else {
      J.impulse[0] = 0.0f; J.impulse[1] = 0.0f; J.impulse[2] = 0.0f;
    }
  } else if (J.d.type == B2G_JOINT_MOUSE) {  // b2_mouse_joint.cpp:75-132 (body B only)
    float d = J.d.damping;
    float k = J.d.stiffness;
    float h = dt;
    J.gamma = h * (d + h * k);
    if (J.gamma != 0.0f) J.gamma = 1.0f / J.gamma;
    J.bias = h * k * J.gamma;  // beta
    V2 rB = mul(qB, lb - lcB);
    st2(J.rB, rB);
    M22 K;
    K.ex.x = mB + iB * rB.y * rB.y + J.gamma;
    K.ex.y = -iB * rB.x * rB.y;
    K.ey.x = K.ex.y;
    K.ey.y = mB + iB * rB.x * rB.x + J.gamma;
    stK(J.K, inverse(K));
    V2 C = (cB + rB) - ld2(J.d.target);
    C.x *= J.bias;
    C.y *= J.bias;
    st2(J.err, C);
    wB *= 0.98f;
    if (warm) {
      J.impulse[0] *= dtRatio; J.impulse[1] *= dtRatio;
      V2 P = mk(J.impulse[0], J.impulse[1]);
      addTo(vB, mB * P);
      wB += iB * cross(rB, P);
    } else {
      J.impulse[0] = 0.0f; J.impulse[1] = 0.0f;
    }
  } else {  // pulley, b2_pulley_joint.cpp:78-157
    V2 rA = mul(qA, la - lcA);
    V2 rB = mul(qB, lb - lcB);
    st2(J.rA, rA); st2(J.rB, rB);
    V2 uA = (cA + rA) - ld2(J.d.ground_anchor_a);
    V2 uB = (cB + rB) - ld2(J.d.ground_anchor_b);
    float lengthA = lengthOf(uA);
    float lengthB = lengthOf(uB);
    if (lengthA > 10.0f * B2G_LINEAR_SLOP) { float s = 1.0f / lengthA; uA.x *= s; uA.y *= s; }
    else uA = mk(0.0f, 0.0f);
    if (lengthB > 10.0f * B2G_LINEAR_SLOP) { float s = 1.0f / lengthB; uB.x *= s; uB.y *= s; }
    else uB = mk(0.0f, 0.0f);
    st2(J.u, uA); st2(J.uB, uB);
    float ruA = cross(rA, uA);
    float ruB = cross(rB, uB);
    float pmA = mA + iA * ruA * ruA;
    float pmB = mB + iB * ruB * ruB;
    J.mass = pmA + J.d.ratio * J.d.ratio * pmB;
    if (J.mass > 0.0f) J.mass = 1.0f / J.mass;
    if (warm) {
      J.impulse[0] *= dtRatio;
      V2 PA = -(J.impulse[0]) * uA;
      V2 PB = (-J.d.ratio * J.impulse[0]) * uB;
      addTo(vA, mA * PA);
      wA += iA * cross(rA, PA);
      addTo(vB, mB * PB);
      wB += iB * cross(rB, PB);
    } else {
      J.impulse[0] = 0.0f;
    }
  }
  if (moves(mA, iA)) storeVel(vel, ia, vA, wA);
  if (moves(mB, iB)) storeVel(vel, ib, vB, wB);
}

// SolveVelocityConstraints (revolute :167-243, prismatic :226-330, distance :175-266).
B2G_HD void jointSolveVelocity(JointDev& J, float4* vel, float dt, float inv_dt) {
  V2 vA, vB; float wA, wB;
  loadVel(vel, J.iA, vA, wA);
  loadVel(vel, J.iB, vB, wB);
  float mA = J.mA, mB = J.mB, iA = J.invIA, iB = J.invIB;
  if (J.d.type == B2G_JOINT_REVOLUTE) {
    V2 rA = ld2(J.rA), rB = ld2(J.rB);
    bool fixedRotation = (iA + iB == 0.0f);
    if (J.d.enable_motor && fixedRotation == false) {
      float Cdot = wB - wA - J.d.motor_speed;
      float impulse = -J.axialMass * Cdot;
      float oldImpulse = J.motorImpulse;
      float maxImpulse = dt * J.d.max_motor;
      J.motorImpulse = fclamp(J.motorImpulse + impulse, -maxImpulse, maxImpulse);
      impulse = J.motorImpulse - oldImpulse;
      wA -= iA * impulse;
      wB += iB * impulse;
    }
    if (J.d.enable_limit && fixedRotation == false) {
      {
        float C = J.angle - J.d.lower;
        float Cdot = wB - wA;
        float impulse = -J.axialMass * (Cdot + fmax2(C, 0.0f) * inv_dt);
        float oldImpulse = J.lowerImpulse;
        J.lowerImpulse = fmax2(J.lowerImpulse + impulse, 0.0f);
        impulse = J.lowerImpulse - oldImpulse;
        wA -= iA * impulse;
        wB += iB * impulse;
      }
      {
        float C = J.d.upper - J.angle;
        float Cdot = wA - wB;
        float impulse = -J.axialMass * (Cdot + fmax2(C, 0.0f) * inv_dt);
        float oldImpulse = J.upperImpulse;
        J.upperImpulse = fmax2(J.upperImpulse + impulse, 0.0f);
        impulse = J.upperImpulse - oldImpulse;
        wA += iA * impulse;
        wB -= iB * impulse;
      }
    }
    {
      V2 Cdot = ((vB + cross(wB, rB)) - vA) - cross(wA, rA);
      V2 impulse = solve(ldK(J.K), -Cdot);
      J.impulse[0] += impulse.x;
      J.impulse[1] += impulse.y;
      subFrom(vA, mA * impulse);
      wA -= iA * cross(rA, impulse);
      addTo(vB, mB * impulse);
      wB += iB * cross(rB, impulse);
    }
  } else if (J.d.type == B2G_JOINT_PRISMATIC) {
    V2 axis = ld2(J.axis), perp = ld2(J.perp);
    if (J.d.enable_motor) {
      float Cdot = (dot(axis, vB - vA) + J.a2 * wB) - J.a1 * wA;
      float impulse = J.axialMass * (J.d.motor_speed - Cdot);
      float oldImpulse = J.motorImpulse;
      float maxImpulse = dt * J.d.max_motor;
      J.motorImpulse = fclamp(J.motorImpulse + impulse, -maxImpulse, maxImpulse);
      impulse = J.motorImpulse - oldImpulse;
      V2 P = impulse * axis;
      float LA = impulse * J.a1;
      float LB = impulse * J.a2;
      subFrom(vA, mA * P); wA -= iA * LA;
      addTo(vB, mB * P); wB += iB * LB;
    }
    if (J.d.enable_limit) {
      {
        float C = J.translation - J.d.lower;
        float Cdot = (dot(axis, vB - vA) + J.a2 * wB) - J.a1 * wA;
        float impulse = -J.axialMass * (Cdot + fmax2(C, 0.0f) * inv_dt);
        float oldImpulse = J.lowerImpulse;
        J.lowerImpulse = fmax2(J.lowerImpulse + impulse, 0.0f);
        impulse = J.lowerImpulse - oldImpulse;
        V2 P = impulse * axis;
        float LA = impulse * J.a1;
        float LB = impulse * J.a2;
        subFrom(vA, mA * P); wA -= iA * LA;
        addTo(vB, mB * P); wB += iB * LB;
      }
      {
        float C = J.d.upper - J.translation;
        float Cdot = (dot(axis, vA - vB) + J.a1 * wA) - J.a2 * wB;
        float impulse = -J.axialMass * (Cdot + fmax2(C, 0.0f) * inv_dt);
        float oldImpulse = J.upperImpulse;
        J.upperImpulse = fmax2(J.upperImpulse + impulse, 0.0f);
        impulse = J.upperImpulse - oldImpulse;
        V2 P = impulse * axis;
        float LA = impulse * J.a1;
        float LB = impulse * J.a2;
        addTo(vA, mA * P); wA += iA * LA;
        subFrom(vB, mB * P); wB -= iB * LB;
      }
    }
    {
      V2 Cdot;
      Cdot.x = (dot(perp, vB - vA) + J.s2 * wB) - J.s1 * wA;
      Cdot.y = wB - wA;
      V2 df = solve(ldK(J.K), -Cdot);
      J.impulse[0] += df.x;
      J.impulse[1] += df.y;
      V2 P = df.x * perp;
      float LA = df.x * J.s1 + df.y;
      float LB = df.x * J.s2 + df.y;
      subFrom(vA, mA * P); wA -= iA * LA;
      addTo(vB, mB * P); wB += iB * LB;
    }
  } else if (J.d.type == B2G_JOINT_DISTANCE) {
    V2 rA = ld2(J.rA), rB = ld2(J.rB), u = ld2(J.u);
    if (J.d.min_length < J.d.max_length) {
      if (J.d.stiffness > 0.0f) {
        V2 vpA = vA + cross(wA, rA);
        V2 vpB = vB + cross(wB, rB);
        float Cdot = dot(u, vpB - vpA);
        float impulse = -J.softMass * ((Cdot + J.bias) + J.gamma * J.impulse[0]);
        J.impulse[0] += impulse;
        V2 P = impulse * u;
        subFrom(vA, J.mA * P); wA -= J.invIA * cross(rA, P);
        addTo(vB, J.mB * P); wB += J.invIB * cross(rB, P);
      }
      {
        float C = J.currentLength - J.d.min_length;
        float bias = fmax2(0.0f, C) * inv_dt;
        V2 vpA = vA + cross(wA, rA);
        V2 vpB = vB + cross(wB, rB);
        float Cdot = dot(u, vpB - vpA);
        float impulse = -J.mass * (Cdot + bias);
        float oldImpulse = J.lowerImpulse;
        J.lowerImpulse = fmax2(0.0f, J.lowerImpulse + impulse);
        impulse = J.lowerImpulse - oldImpulse;
        V2 P = impulse * u;
        subFrom(vA, J.mA * P); wA -= J.invIA * cross(rA, P);
        addTo(vB, J.mB * P); wB += J.invIB * cross(rB, P);
      }
      {
        float C = J.d.max_length - J.currentLength;
        float bias = fmax2(0.0f, C) * inv_dt;
        V2 vpA = vA + cross(wA, rA);
        V2 vpB = vB + cross(wB, rB);
        float Cdot = dot(u, vpA - vpB);
        float impulse = -J.mass * (Cdot + bias);
        float oldImpulse = J.upperImpulse;
        J.upperImpulse = fmax2(0.0f, J.upperImpulse + impulse);
        impulse = J.upperImpulse - oldImpulse;
        V2 P = -impulse * u;
        subFrom(vA, J.mA * P); wA -= J.invIA * cross(rA, P);
        addTo(vB, J.mB * P); wB += J.invIB * cross(rB, P);
      }
    } else {
      V2 vpA = vA + cross(wA, rA);
      V2 vpB = vB + cross(wB, rB);
      float Cdot = dot(u, vpB - vpA);
      float impulse = -J.mass * Cdot;
      J.impulse[0] += impulse;
      V2 P = impulse * u;
      subFrom(vA, J.mA * P); wA -= J.invIA * cross(rA, P);
      addTo(vB, J.mB * P); wB += J.invIB * cross(rB, P);
    }
  } else if (J.d.type == B2G_JOINT_WELD) {  // b2_weld_joint.cpp:189-250
    V2 rA = ld2(J.rA), rB = ld2(J.rB);
    const float* M = J.mass3;
    if (J.d.stiffness > 0.0f) {
      float Cdot2 = wB - wA;
      float impulse2 = -M[8] * (Cdot2 + J.bias + J.gamma * J.impulse[2]);
      J.impulse[2] += impulse2;
      wA -= iA * impulse2;
      wB += iB * impulse2;
      V2 Cdot1 = ((vB + cross(wB, rB)) - vA) - cross(wA, rA);
      V2 impulse1 = -mk(M[0] * Cdot1.x + M[3] * Cdot1.y, M[1] * Cdot1.x + M[4] * Cdot1.y);
      J.impulse[0] += impulse1.x;
      J.impulse[1] += impulse1.y;
      V2 P = impulse1;
      subFrom(vA, mA * P);
      wA -= iA * cross(rA, P);
      addTo(vB, mB * P);
      wB += iB * cross(rB, P);
    } else {
      V2 Cdot1 = ((vB + cross(wB, rB)) - vA) - cross(wA, rA);
      float Cdot2 = wB - wA;
      V3 impulse;
      impulse.x = -((Cdot1.x * M[0] + Cdot1.y * M[3]) + Cdot2 * M[6]);
      impulse.y = -((Cdot1.x * M[1] + Cdot1.y * M[4]) + Cdot2 * M[7]);
      impulse.z = -((Cdot1.x * M[2] + Cdot1.y * M[5]) + Cdot2 * M[8]);
      J.impulse[0] += impulse.x; J.impulse[1] += impulse.y; J.impulse[2] += impulse.z;
      V2 P = mk(impulse.x, impulse.y);
      subFrom(vA, mA * P);
      wA -= iA * (cross(rA, P) + impulse.z);
      addTo(vB, mB * P);
      wB += iB * (cross(rB, P) + impulse.z);
    }
  } else if (J.d.type == B2G_JOINT_WHEEL) {  // b2_wheel_joint.cpp:213-323
    V2 ax = ld2(J.axis), ay = ld2(J.perp);
    {
      float Cdot = dot(ax, vB - vA) + J.a2 * wB - J.a1 * wA;
      float impulse = -J.springMass * (Cdot + J.bias + J.gamma * J.impulse[1]);
      J.impulse[1] += impulse;
      V2 P = impulse * ax;
      float LA = impulse * J.a1;
      float LB = impulse * J.a2;
      subFrom(vA, mA * P); wA -= iA * LA;
      addTo(vB, mB * P); wB += iB * LB;
    }
    {
      float Cdot = wB - wA - J.d.motor_speed;
      float impulse = -J.motorMass * Cdot;
      float oldImpulse = J.motorImpulse;
      float maxImpulse = dt * J.d.max_motor;
      J.motorImpulse = fclamp(J.motorImpulse + impulse, -maxImpulse, maxImpulse);
      impulse = J.motorImpulse - oldImpulse;
      wA -= iA * impulse;
      wB += iB * impulse;
    }
    if (J.d.enable_limit) {
      {
        float C = J.translation - J.d.lower;
        float Cdot = dot(ax, vB - vA) + J.a2 * wB - J.a1 * wA;
        float impulse = -J.axialMass * (Cdot + fmax2(C, 0.0f) * inv_dt);
        float oldImpulse = J.lowerImpulse;
        J.lowerImpulse = fmax2(J.lowerImpulse + impulse, 0.0f);
        impulse = J.lowerImpulse - oldImpulse;
        V2 P = impulse * ax;
        float LA = impulse * J.a1;
        float LB = impulse * J.a2;
        subFrom(vA, mA * P); wA -= iA * LA;
        addTo(vB, mB * P); wB += iB * LB;
      }
      {
        float C = J.d.upper - J.translation;
        float Cdot = dot(ax, vA - vB) + J.a1 * wA - J.a2 * wB;
        float impulse = -J.axialMass * (Cdot + fmax2(C, 0.0f) * inv_dt);
        float oldImpulse = J.upperImpulse;
        J.upperImpulse = fmax2(J.upperImpulse + impulse, 0.0f);
        impulse = J.upperImpulse - oldImpulse;
        V2 P = impulse * ax;
        float LA = impulse * J.a1;
        float LB = impulse * J.a2;
        addTo(vA, mA * P); wA += iA * LA;
        subFrom(vB, mB * P); wB -= iB * LB;
      }
    }
    {
      float Cdot = dot(ay, vB - vA) + J.s2 * wB - J.s1 * wA;
      float impulse = -J.mass * Cdot;
      J.impulse[0] += impulse;
      V2 P = impulse * ay;
      float LA = impulse * J.s1;
      float LB = impulse * J.s2;
      subFrom(vA, mA * P); wA -= iA * LA;
      addTo(vB, mB * P); wB += iB * LB;
    }
  } else if (J.d.type == B2G_JOINT_MOTOR) {  // b2_motor_joint.cpp:138-196
    float fb = inv_dt * J.d.correction_factor;
    solveLinearAngular(J, vA, wA, vB, wB, dt, true, fb * J.angularError, fb * ld2(J.err));
  } else if (J.d.type == B2G_JOINT_FRICTION) {  // b2_friction_joint.cpp:125-183
    solveLinearAngular(J, vA, wA, vB, wB, dt, false, 0.0f, mk(0.0f, 0.0f));
  } else if (J.d.type == B2G_JOINT_MOUSE) {  // b2_mouse_joint.cpp:134-160
    V2 rB = ld2(J.rB);
    V2 Cdot = vB + cross(wB, rB);
    V2 old = mk(J.impulse[0], J.impulse[1]);
    V2 impulse = mul(ldK(J.K), -((Cdot + ld2(J.err)) + J.gamma * old));
    V2 acc = old + impulse;
    float maxImpulse = dt * J.d.max_force;
    if (lengthSq(acc) > maxImpulse * maxImpulse) {
      float s = maxImpulse / lengthOf(acc);
      acc.x *= s;
      acc.y *= s;
    }
    J.impulse[0] = acc.x; J.impulse[1] = acc.y;
    impulse = acc - old;
    addTo(vB, mB * impulse);
    wB += iB * cross(rB, impulse);
  } else {  // pulley, b2_pulley_joint.cpp:159-182
    V2 rA = ld2(J.rA), rB = ld2(J.rB), uA = ld2(J.u), uB = ld2(J.uB);
    V2 vpA = vA + cross(wA, rA);
    V2 vpB = vB + cross(wB, rB);
    float Cdot = -dot(uA, vpA) - J.d.ratio * dot(uB, vpB);
    float impulse = -J.mass * Cdot;
    J.impulse[0] += impulse;
    V2 PA = -impulse * uA;
    V2 PB = -J.d.ratio * impulse * uB;
    addTo(vA, mA * PA);
    wA += iA * cross(rA, PA);
    addTo(vB, mB * PB);
    wB += iB * cross(rB, PB);
  }
  if (moves(J.mA, J.invIA)) storeVel(vel, J.iA, vA, wA);
  if (moves(J.mB, J.invIB)) storeVel(vel, J.iB, vB, wB);
}

// SolvePositionConstraints (revolute :245-321, prismatic :340-459, distance :268-314).
B2G_HD bool jointSolvePosition(JointDev& J, float4* pos) {
  V2 cA, cB; float aA, aB;
  loadPos(pos, J.iA, cA, aA);
  loadPos(pos, J.iB, cB, aB);
  Rot qA = rotOf(aA), qB = rotOf(aB);
  V2 la = ld2(J.d.local_anchor_a), lb = ld2(J.d.local_anchor_b);
  V2 lcA = ld2(J.lcA), lcB = ld2(J.lcB);
  bool ok;
  if (J.d.type == B2G_JOINT_REVOLUTE) {
    float angularError = 0.0f;
    float positionError = 0.0f;
    bool fixedRotation = (J.invIA + J.invIB == 0.0f);
    if (J.d.enable_limit && fixedRotation == false) {
      float angle = aB - aA - J.d.reference_angle;
      float C = 0.0f;
      if (fabs2(J.d.upper - J.d.lower) < 2.0f * B2G_ANGULAR_SLOP)
        C = fclamp(angle - J.d.lower, -B2G_MAX_ANGULAR_CORRECTION, B2G_MAX_ANGULAR_CORRECTION);
      else if (angle <= J.d.lower)
        C = fclamp(angle - J.d.lower + B2G_ANGULAR_SLOP, -B2G_MAX_ANGULAR_CORRECTION, 0.0f);
      else if (angle >= J.d.upper)
        C = fclamp(angle - J.d.upper - B2G_ANGULAR_SLOP, 0.0f, B2G_MAX_ANGULAR_CORRECTION);
      float limitImpulse = -J.axialMass * C;
      aA -= J.invIA * limitImpulse;
      aB += J.invIB * limitImpulse;
      angularError = fabs2(C);
    }
    {
      qA = rotOf(aA);
      qB = rotOf(aB);
      V2 rA = mul(qA, la - lcA);
      V2 rB = mul(qB, lb - lcB);
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
    ok = positionError <= B2G_LINEAR_SLOP && angularError <= B2G_ANGULAR_SLOP;
  } else if (J.d.type == B2G_JOINT_PRISMATIC) {
    float mA = J.mA, mB = J.mB, iA = J.invIA, iB = J.invIB;
    V2 rA = mul(qA, la - lcA);
    V2 rB = mul(qB, lb - lcB);
    V2 d = ((cB + rB) - cA) - rA;
    V2 axis = mul(qA, ld2(J.localXAxisA));
    float a1 = cross(d + rA, axis);
    float a2 = cross(rB, axis);
    V2 perp = mul(qA, ld2(J.localYAxisA));
    float s1 = cross(d + rA, perp);
    float s2 = cross(rB, perp);
    V3 impulse;
    V2 C1;
    C1.x = dot(perp, d);
    C1.y = aB - aA - J.d.reference_angle;
    float linearError = fabs2(C1.x);
    float angularError = fabs2(C1.y);
    bool active = false;
    float C2 = 0.0f;
    if (J.d.enable_limit) {
      float translation = dot(axis, d);
      if (fabs2(J.d.upper - J.d.lower) < 2.0f * B2G_LINEAR_SLOP) {
        C2 = translation;
        linearError = fmax2(linearError, fabs2(translation));
        active = true;
      } else if (translation <= J.d.lower) {
        C2 = fmin2(translation - J.d.lower, 0.0f);
        linearError = fmax2(linearError, J.d.lower - translation);
        active = true;
      } else if (translation >= J.d.upper) {
        C2 = fmax2(translation - J.d.upper, 0.0f);
        linearError = fmax2(linearError, translation - J.d.upper);
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
      K.ex = mk(k11, k12);
      K.ey = mk(k12, k22);
      V2 impulse1 = solve(K, -C1);
      impulse.x = impulse1.x; impulse.y = impulse1.y; impulse.z = 0.0f;
    }
    V2 P = impulse.x * perp + impulse.z * axis;
    float LA = (impulse.x * s1 + impulse.y) + impulse.z * a1;
    float LB = (impulse.x * s2 + impulse.y) + impulse.z * a2;
    subFrom(cA, mA * P); aA -= iA * LA;
    addTo(cB, mB * P); aB += iB * LB;
    ok = linearError <= B2G_LINEAR_SLOP && angularError <= B2G_ANGULAR_SLOP;
  } else if (J.d.type == B2G_JOINT_DISTANCE) {
    V2 rA = mul(qA, la - lcA);
    V2 rB = mul(qB, lb - lcB);
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
    ok = fabs2(C) < B2G_LINEAR_SLOP;
  } else if (J.d.type == B2G_JOINT_WELD) {  // b2_weld_joint.cpp:252-329
    float mA = J.mA, mB = J.mB, iA = J.invIA, iB = J.invIB;
    V2 rA = mul(qA, la - lcA);
    V2 rB = mul(qB, lb - lcB);
    float positionError, angularError;
    V3 ex, ey, ez;
    weldK(rA, rB, mA, mB, iA, iB, ex, ey, ez);
    if (J.d.stiffness > 0.0f) {
      V2 C1 = ((cB + rB) - cA) - rA;
      positionError = lengthOf(C1);
      angularError = 0.0f;
      V2 P = -solve22(ex, ey, C1);
      subFrom(cA, mA * P);
      aA -= iA * cross(rA, P);
      addTo(cB, mB * P);
      aB += iB * cross(rB, P);
    } else {
      V2 C1 = ((cB + rB) - cA) - rA;
      float C2 = aB - aA - J.d.reference_angle;
      positionError = lengthOf(C1);
      angularError = fabs2(C2);
      V3 C = {C1.x, C1.y, C2};
      V3 impulse;
      if (ez.z > 0.0f) {
        V3 x = solve33(ex, ey, ez, C);
        impulse.x = -x.x; impulse.y = -x.y; impulse.z = -x.z;
      } else {
        V2 impulse2 = -solve22(ex, ey, C1);
        impulse.x = impulse2.x; impulse.y = impulse2.y; impulse.z = 0.0f;
      }
      V2 P = mk(impulse.x, impulse.y);
      subFrom(cA, mA * P);
      aA -= iA * (cross(rA, P) + impulse.z);
      addTo(cB, mB * P);
      aB += iB * (cross(rB, P) + impulse.z);
    }
    ok = positionError <= B2G_LINEAR_SLOP && angularError <= B2G_ANGULAR_SLOP;
  } else if (J.d.type == B2G_JOINT_WHEEL) {  // b2_wheel_joint.cpp:325-420
    // the reference mixes this step's axis and point arms from InitVelocityConstraints (m_ax,
    // m_sAy, m_sBy) into its position pass; kept as it is
    float linearError = 0.0f;
    if (J.d.enable_limit) {
      V2 rA = mul(qA, la - lcA);
      V2 rB = mul(qB, lb - lcB);
      V2 d = ((cB - cA) + rB) - rA;
      V2 ax = mul(qA, ld2(J.localXAxisA));
      float sAx = cross(d + rA, ld2(J.axis));
      float sBx = cross(rB, ld2(J.axis));
      float C = 0.0f;
      float translation = dot(ax, d);
      if (fabs2(J.d.upper - J.d.lower) < 2.0f * B2G_LINEAR_SLOP) C = translation;
      else if (translation <= J.d.lower) C = fmin2(translation - J.d.lower, 0.0f);
      else if (translation >= J.d.upper) C = fmax2(translation - J.d.upper, 0.0f);
      if (C != 0.0f) {
        float invMass = J.mA + J.mB + J.invIA * sAx * sAx + J.invIB * sBx * sBx;
        float impulse = 0.0f;
        if (invMass != 0.0f) impulse = -C / invMass;
        V2 P = impulse * ax;
        float LA = impulse * sAx;
        float LB = impulse * sBx;
        subFrom(cA, J.mA * P); aA -= J.invIA * LA;
        addTo(cB, J.mB * P); aB += J.invIB * LB;
        linearError = fabs2(C);
      }
    }
    {
      Rot qA2 = rotOf(aA), qB2 = rotOf(aB);
      V2 rA = mul(qA2, la - lcA);
      V2 rB = mul(qB2, lb - lcB);
      V2 d = ((cB - cA) + rB) - rA;
      V2 ay = mul(qA2, ld2(J.localYAxisA));
      float sAy = cross(d + rA, ay);
      float sBy = cross(rB, ay);
      float C = dot(d, ay);
      float invMass = J.mA + J.mB + J.invIA * J.s1 * J.s1 + J.invIB * J.s2 * J.s2;
      float impulse = 0.0f;
      if (invMass != 0.0f) impulse = -C / invMass;
      V2 P = impulse * ay;
      float LA = impulse * sAy;
      float LB = impulse * sBy;
      subFrom(cA, J.mA * P); aA -= J.invIA * LA;
      addTo(cB, J.mB * P); aB += J.invIB * LB;
      linearError = fmax2(linearError, fabs2(C));
    }
    ok = linearError <= B2G_LINEAR_SLOP;
  } else if (J.d.type == B2G_JOINT_PULLEY) {  // b2_pulley_joint.cpp:184-256
    V2 rA = mul(qA, la - lcA);
    V2 rB = mul(qB, lb - lcB);
    V2 uA = (cA + rA) - ld2(J.d.ground_anchor_a);
    V2 uB = (cB + rB) - ld2(J.d.ground_anchor_b);
    float lengthA = lengthOf(uA);
    float lengthB = lengthOf(uB);
    if (lengthA > 10.0f * B2G_LINEAR_SLOP) { float s = 1.0f / lengthA; uA.x *= s; uA.y *= s; }
    else uA = mk(0.0f, 0.0f);
    if (lengthB > 10.0f * B2G_LINEAR_SLOP) { float s = 1.0f / lengthB; uB.x *= s; uB.y *= s; }
    else uB = mk(0.0f, 0.0f);
    float ruA = cross(rA, uA);
    float ruB = cross(rB, uB);
    float pmA = J.mA + J.invIA * ruA * ruA;
    float pmB = J.mB + J.invIB * ruB * ruB;
    float mass = pmA + J.d.ratio * J.d.ratio * pmB;
    if (mass > 0.0f) mass = 1.0f / mass;
    float C = J.constant - lengthA - J.d.ratio * lengthB;
    float linearError = fabs2(C);
    float impulse = -mass * C;
    V2 PA = -impulse * uA;
    V2 PB = -J.d.ratio * impulse * uB;
    addTo(cA, J.mA * PA); aA += J.invIA * cross(rA, PA);
    addTo(cB, J.mB * PB); aB += J.invIB * cross(rB, PB);
    ok = linearError < B2G_LINEAR_SLOP;
  } else {  // motor, friction, mouse: no position constraint
    return true;
  }
  if (moves(J.mA, J.invIA)) storePos(pos, J.iA, cA, aA);
  if (moves(J.mB, J.invIB)) storePos(pos, J.iB, cB, aB);
  return ok;
}

#ifdef __CUDACC__
// ---- joint velocity rows. A joint's velocity pass reads a few dozen of its record's fields, spread
// over the record; read from the record in global memory, each field is a separate transaction per
// thread and the pass costs about ten contact solves. The rows hold those fields packed per type
// (B2G_JV_ROWS float4 planes of `stride` slots, one slot per joint in colour order, so a colour's
// threads read consecutive slots), written by the joint's init; the velocity iterations run the
// same jointSolveVelocity on a register copy, and the accumulated impulses go back to the record
// after the last iteration.
//   row 0: iA, iB, type, flags (as int bits)     row 1: mA, mB, invIA, invIB
//   rows 2-6: per type (below; row 4 holds K for the prismatic joint, motorMass, bias and gamma
//             for the wheel joint)               row 7: impulse 0-2, motorImpulse
//   row 8: lowerImpulse, upperImpulse
// The position iterations read rows 0-1 and the position rows 9-12 the same way:
//   row 9: local anchors A, B                     row 10: local centres A, B
//   rows 11-12: per type (jointPackPos)
// The init itself runs on a per-type register copy of the record's fields it reads, so that the
// record is only read during the step and written once, by jointStoreImpulses.
#define B2G_JV_MOTOR 1
#define B2G_JV_LIMIT 2
#define B2G_JV_ASLEEP 4
#define B2G_JV_GEAR 8   // the slot's joint is a gear, solved on its record (serial colour only)

__device__ __forceinline__ void jointPackVel(const JointDev& J, float4* P, int stride, int slot) {
  float4 r[B2G_JV_ROWS];
  for (int k = 0; k < B2G_JV_ROWS; ++k) r[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  const int flags = (J.d.enable_motor ? B2G_JV_MOTOR : 0) | (J.d.enable_limit ? B2G_JV_LIMIT : 0);
  r[0] = make_float4(__int_as_float(J.iA), __int_as_float(J.iB), __int_as_float(J.d.type), __int_as_float(flags));
  r[1] = make_float4(J.mA, J.mB, J.invIA, J.invIB);
  switch (J.d.type) {
    case B2G_JOINT_REVOLUTE:
      r[2] = make_float4(J.rA[0], J.rA[1], J.rB[0], J.rB[1]);
      r[3] = make_float4(J.K[0], J.K[1], J.K[2], J.K[3]);
      r[4] = make_float4(J.axialMass, J.angle, J.d.lower, J.d.upper);
      r[5] = make_float4(J.d.motor_speed, J.d.max_motor, 0.0f, 0.0f);
      break;
    case B2G_JOINT_PRISMATIC:
    case B2G_JOINT_WHEEL:
      r[2] = make_float4(J.axis[0], J.axis[1], J.perp[0], J.perp[1]);
      r[3] = make_float4(J.a1, J.a2, J.s1, J.s2);
      r[4] = make_float4(J.K[0], J.K[1], J.K[2], J.K[3]);
      r[5] = make_float4(J.axialMass, J.translation, J.d.lower, J.d.upper);
      r[6] = make_float4(J.d.motor_speed, J.d.max_motor, J.mass, J.springMass);
      r[4] = J.d.type == B2G_JOINT_WHEEL ? make_float4(J.motorMass, J.bias, J.gamma, 0.0f) : r[4];
      break;
    case B2G_JOINT_DISTANCE:
      r[2] = make_float4(J.rA[0], J.rA[1], J.rB[0], J.rB[1]);
      r[3] = make_float4(J.u[0], J.u[1], J.softMass, J.bias);
      r[4] = make_float4(J.gamma, J.mass, J.currentLength, J.d.min_length);
      r[5] = make_float4(J.d.max_length, J.d.stiffness, 0.0f, 0.0f);
      break;
    case B2G_JOINT_WELD:
      r[2] = make_float4(J.rA[0], J.rA[1], J.rB[0], J.rB[1]);
      r[3] = make_float4(J.mass3[0], J.mass3[1], J.mass3[2], J.mass3[3]);
      r[4] = make_float4(J.mass3[4], J.mass3[5], J.mass3[6], J.mass3[7]);
      r[5] = make_float4(J.mass3[8], J.bias, J.gamma, J.d.stiffness);
      break;
    case B2G_JOINT_MOTOR:
    case B2G_JOINT_FRICTION:
      r[2] = make_float4(J.rA[0], J.rA[1], J.rB[0], J.rB[1]);
      r[3] = make_float4(J.K[0], J.K[1], J.K[2], J.K[3]);
      r[4] = make_float4(J.axialMass, J.d.max_force, J.d.max_torque, J.d.correction_factor);
      r[5] = make_float4(J.angularError, J.err[0], J.err[1], 0.0f);
      break;
    case B2G_JOINT_MOUSE:
      r[2] = make_float4(J.rA[0], J.rA[1], J.rB[0], J.rB[1]);
      r[3] = make_float4(J.K[0], J.K[1], J.K[2], J.K[3]);
      r[4] = make_float4(J.err[0], J.err[1], J.gamma, J.d.max_force);
      break;
    default:  // pulley
      r[2] = make_float4(J.rA[0], J.rA[1], J.rB[0], J.rB[1]);
      r[3] = make_float4(J.u[0], J.u[1], J.uB[0], J.uB[1]);
      r[4] = make_float4(J.mass, J.d.ratio, 0.0f, 0.0f);
      break;
  }
  r[7] = make_float4(J.impulse[0], J.impulse[1], J.impulse[2], J.motorImpulse);
  r[8] = make_float4(J.lowerImpulse, J.upperImpulse, 0.0f, 0.0f);
#pragma unroll
  for (int k = 0; k < B2G_JV_ROWS; ++k) P[(int64_t)k * stride + slot] = r[k];
}

// The position pass's rows of a joint whose init just ran (J holds its step temporaries).
__device__ __forceinline__ void jointPackPos(const JointDev& J, float4* P, int stride, int slot) {
  float4 r11 = make_float4(0.0f, 0.0f, 0.0f, 0.0f), r12 = r11;
  switch (J.d.type) {
    case B2G_JOINT_REVOLUTE:
      r11 = make_float4(J.axialMass, J.d.reference_angle, J.d.lower, J.d.upper);
      break;
    case B2G_JOINT_PRISMATIC:
      r11 = make_float4(J.localXAxisA[0], J.localXAxisA[1], J.localYAxisA[0], J.localYAxisA[1]);
      r12 = make_float4(J.d.reference_angle, J.d.lower, J.d.upper, 0.0f);
      break;
    case B2G_JOINT_DISTANCE:
      r11 = make_float4(J.d.max_length, J.d.min_length, J.mass, 0.0f);
      break;
    case B2G_JOINT_WELD:
      r11 = make_float4(J.d.reference_angle, J.d.stiffness, 0.0f, 0.0f);
      break;
    case B2G_JOINT_WHEEL:
      r11 = make_float4(J.localXAxisA[0], J.localXAxisA[1], J.localYAxisA[0], J.localYAxisA[1]);
      r12 = make_float4(J.d.lower, J.d.upper, J.s1, J.s2);
      break;
    case B2G_JOINT_PULLEY:
      r11 = make_float4(J.d.ground_anchor_a[0], J.d.ground_anchor_a[1], J.d.ground_anchor_b[0], J.d.ground_anchor_b[1]);
      r12 = make_float4(J.constant, J.d.ratio, 0.0f, 0.0f);
      break;
    default:
      break;
  }
  P[(int64_t)9 * stride + slot] = make_float4(J.d.local_anchor_a[0], J.d.local_anchor_a[1], J.d.local_anchor_b[0], J.d.local_anchor_b[1]);
  P[(int64_t)10 * stride + slot] = make_float4(J.lcA[0], J.lcA[1], J.lcB[0], J.lcB[1]);
  P[(int64_t)11 * stride + slot] = r11;
  P[(int64_t)12 * stride + slot] = r12;
}

// InitVelocityConstraints of the joint record G into the rows of `slot`: per type, a register
// copy of the record's fields the init and the rows read, the init on it, the rows packed.
// ---- gear joint (src/dynamics/b2_gear_joint.cpp:141-372). Four bodies: it runs in the serial
// joint colour on its record, one thread. A, B are d.body_a / d.body_b; C, D are g.iC / g.iD.

// The Jacobian rows and effective mass of the gear at rotations qA..qD (InitVelocityConstraints
// :178-216 and SolvePositionConstraints :290-332 compute them alike); returns the summed mass.
B2G_HD float gearJacobian(JointDev::Gear& g, float ratio, Rot qA, Rot qB, Rot qC, Rot qD, V2& JvAC, V2& JvBD,
                          float& JwA, float& JwB, float& JwC, float& JwD) {
  float mass = 0.0f;
  if (g.typeA == B2G_JOINT_REVOLUTE) {
    JvAC = mk(0.0f, 0.0f);
    JwA = 1.0f;
    JwC = 1.0f;
    mass += g.iA + g.iC_;
  } else {
    V2 u = mul(qC, ld2(g.axC));
    V2 rC = mul(qC, ld2(g.lC) - ld2(g.lcC));
    V2 rA = mul(qA, ld2(g.lA) - ld2(g.lcA));
    JvAC = u;
    JwC = cross(rC, u);
    JwA = cross(rA, u);
    mass += g.mC + g.mA + g.iC_ * JwC * JwC + g.iA * JwA * JwA;
  }
  if (g.typeB == B2G_JOINT_REVOLUTE) {
    JvBD = mk(0.0f, 0.0f);
    JwB = ratio;
    JwD = ratio;
    mass += ratio * ratio * (g.iB + g.iD_);
  } else {
    V2 u = mul(qD, ld2(g.axD));
    V2 rD = mul(qD, ld2(g.lD) - ld2(g.lcD));
    V2 rB = mul(qB, ld2(g.lB) - ld2(g.lcB));
    JvBD = ratio * u;
    JwD = ratio * cross(rD, u);
    JwB = ratio * cross(rB, u);
    mass += ratio * ratio * (g.mD + g.mB) + g.iD_ * JwD * JwD + g.iB * JwB * JwB;
  }
  return mass;
}

// Applies `impulse` along the gear's rows to the four bodies (velocities, or positions with
// the angular rows acting on angles).
B2G_HD void gearApply(float4* state, int a, int b, int c, int d, const JointDev::Gear& g, float impulse, V2 JvAC,
                      V2 JvBD, float JwA, float JwB, float JwC, float JwD) {
  V2 xA, xB, xC, xD;
  float tA, tB, tC, tD;
  loadVel(state, a, xA, tA);
  loadVel(state, b, xB, tB);
  loadVel(state, c, xC, tC);
  loadVel(state, d, xD, tD);
  addTo(xA, (g.mA * impulse) * JvAC);
  tA += g.iA * impulse * JwA;
  addTo(xB, (g.mB * impulse) * JvBD);
  tB += g.iB * impulse * JwB;
  subFrom(xC, (g.mC * impulse) * JvAC);
  tC -= g.iC_ * impulse * JwC;
  subFrom(xD, (g.mD * impulse) * JvBD);
  tD -= g.iD_ * impulse * JwD;
  // the reference writes A, B, C, D in this order: a body that appears twice gets its last write
  storeVel(state, a, xA, tA);
  storeVel(state, b, xB, tB);
  storeVel(state, c, xC, tC);
  storeVel(state, d, xD, tD);
}

__device__ __forceinline__ void gearInit(JointDev& J, const float4* massd, const float2* lc, const float4* pos,
                                         float4* vel, bool warm) {
  JointDev::Gear& g = J.g;
  const int a = J.d.body_a, b = J.d.body_b, c = g.iC, d = g.iD;
  const float2 la = lc[a], lb = lc[b], lcc = lc[c], ld = lc[d];
  g.lcA[0] = la.x; g.lcA[1] = la.y; g.lcB[0] = lb.x; g.lcB[1] = lb.y;
  g.lcC[0] = lcc.x; g.lcC[1] = lcc.y; g.lcD[0] = ld.x; g.lcD[1] = ld.y;
  g.mA = massd[a].y; g.mB = massd[b].y; g.mC = massd[c].y; g.mD = massd[d].y;
  g.iA = massd[a].w; g.iB = massd[b].w; g.iC_ = massd[c].w; g.iD_ = massd[d].w;
  const Rot qA = rotOf(pos[a].z), qB = rotOf(pos[b].z), qC = rotOf(pos[c].z), qD = rotOf(pos[d].z);
  V2 JvAC, JvBD;
  float JwA, JwB, JwC, JwD;
  float mass = gearJacobian(g, J.d.ratio, qA, qB, qC, qD, JvAC, JvBD, JwA, JwB, JwC, JwD);
  g.mass = mass > 0.0f ? 1.0f / mass : 0.0f;
  g.JvAC[0] = JvAC.x; g.JvAC[1] = JvAC.y; g.JvBD[0] = JvBD.x; g.JvBD[1] = JvBD.y;
  g.JwA = JwA; g.JwB = JwB; g.JwC = JwC; g.JwD = JwD;
  if (warm) gearApply(vel, a, b, c, d, g, J.impulse[0], JvAC, JvBD, JwA, JwB, JwC, JwD);
  else J.impulse[0] = 0.0f;
}

__device__ __forceinline__ void gearSolveVelocity(JointDev& J, float4* vel) {
  JointDev::Gear& g = J.g;
  const int a = J.d.body_a, b = J.d.body_b, c = g.iC, d = g.iD;
  V2 vA, vB, vC, vD;
  float wA, wB, wC, wD;
  loadVel(vel, a, vA, wA);
  loadVel(vel, b, vB, wB);
  loadVel(vel, c, vC, wC);
  loadVel(vel, d, vD, wD);
  const V2 JvAC = ld2(g.JvAC), JvBD = ld2(g.JvBD);
  float Cdot = dot(JvAC, vA - vC) + dot(JvBD, vB - vD);
  Cdot += (g.JwA * wA - g.JwC * wC) + (g.JwB * wB - g.JwD * wD);
  const float impulse = -g.mass * Cdot;
  J.impulse[0] += impulse;
  gearApply(vel, a, b, c, d, g, impulse, JvAC, JvBD, g.JwA, g.JwB, g.JwC, g.JwD);
}

// The position pass; its linear error is always zero (b2_gear_joint.cpp:370-371), so it is
// always "okay".
__device__ __forceinline__ bool gearSolvePosition(JointDev& J, float4* pos) {
  JointDev::Gear& g = J.g;
  const int a = J.d.body_a, b = J.d.body_b, c = g.iC, d = g.iD;
  V2 cA, cB, cC, cD;
  float aA, aB, aC, aD;
  loadPos(pos, a, cA, aA);
  loadPos(pos, b, cB, aB);
  loadPos(pos, c, cC, aC);
  loadPos(pos, d, cD, aD);
  const Rot qA = rotOf(aA), qB = rotOf(aB), qC = rotOf(aC), qD = rotOf(aD);
  V2 JvAC, JvBD;
  float JwA, JwB, JwC, JwD;
  const float ratio = J.d.ratio;
  float mass = gearJacobian(g, ratio, qA, qB, qC, qD, JvAC, JvBD, JwA, JwB, JwC, JwD);
  float coordinateA, coordinateB;
  if (g.typeA == B2G_JOINT_REVOLUTE) {
    coordinateA = aA - aC - g.refA;
  } else {
    V2 rA = mul(qA, ld2(g.lA) - ld2(g.lcA));
    V2 pC = ld2(g.lC) - ld2(g.lcC);
    V2 pA = mulT(qC, rA + (cA - cC));
    coordinateA = dot(pA - pC, ld2(g.axC));
  }
  if (g.typeB == B2G_JOINT_REVOLUTE) {
    coordinateB = aB - aD - g.refB;
  } else {
    V2 rB = mul(qB, ld2(g.lB) - ld2(g.lcB));
    V2 pD = ld2(g.lD) - ld2(g.lcD);
    V2 pB = mulT(qD, rB + (cB - cD));
    coordinateB = dot(pB - pD, ld2(g.axD));
  }
  const float C = (coordinateA + ratio * coordinateB) - J.d.gear_constant;
  float impulse = 0.0f;
  if (mass > 0.0f) impulse = -C / mass;
  gearApply(pos, a, b, c, d, g, impulse, JvAC, JvBD, JwA, JwB, JwC, JwD);
  return true;
}

__device__ __forceinline__ void jointInitSlot(const JointDev& G, float4* P, int stride, int slot, const float4* massd,
                                              const float2* lc, const float4* pos, float4* vel, float dt, float dtRatio,
                                              bool warm) {
#define B2G_JI_COMMON(TYPE)                                                                      \
  JointDev J;                                                                                    \
  J.d.type = TYPE;                                                                               \
  J.d.body_a = G.d.body_a; J.d.body_b = G.d.body_b;                                              \
  J.d.local_anchor_a[0] = G.d.local_anchor_a[0]; J.d.local_anchor_a[1] = G.d.local_anchor_a[1];  \
  J.d.local_anchor_b[0] = G.d.local_anchor_b[0]; J.d.local_anchor_b[1] = G.d.local_anchor_b[1];  \
  J.d.enable_limit = G.d.enable_limit; J.d.enable_motor = G.d.enable_motor;                      \
  J.impulse[0] = G.impulse[0]; J.impulse[1] = G.impulse[1]; J.impulse[2] = G.impulse[2];         \
  J.motorImpulse = G.motorImpulse; J.lowerImpulse = G.lowerImpulse; J.upperImpulse = G.upperImpulse
#define B2G_JI_AXES                                                                              \
  J.localXAxisA[0] = G.localXAxisA[0]; J.localXAxisA[1] = G.localXAxisA[1];                      \
  J.localYAxisA[0] = G.localYAxisA[0]; J.localYAxisA[1] = G.localYAxisA[1]
#define B2G_JI_FINISH                                                                            \
  jointInit(J, massd, lc, pos, vel, dt, dtRatio, warm);                                          \
  jointPackVel(J, P, stride, slot);                                                              \
  jointPackPos(J, P, stride, slot)
  switch (G.d.type) {
    case B2G_JOINT_REVOLUTE: {
      B2G_JI_COMMON(B2G_JOINT_REVOLUTE);
      J.d.reference_angle = G.d.reference_angle; J.d.lower = G.d.lower; J.d.upper = G.d.upper;
      J.d.motor_speed = G.d.motor_speed; J.d.max_motor = G.d.max_motor;
      B2G_JI_FINISH;
    } break;
    case B2G_JOINT_PRISMATIC: {
      B2G_JI_COMMON(B2G_JOINT_PRISMATIC);
      B2G_JI_AXES;
      J.d.reference_angle = G.d.reference_angle; J.d.lower = G.d.lower; J.d.upper = G.d.upper;
      J.d.motor_speed = G.d.motor_speed; J.d.max_motor = G.d.max_motor;
      B2G_JI_FINISH;
    } break;
    case B2G_JOINT_DISTANCE: {
      B2G_JI_COMMON(B2G_JOINT_DISTANCE);
      J.d.damping = G.d.damping; J.d.length = G.d.length; J.d.min_length = G.d.min_length;
      J.d.max_length = G.d.max_length; J.d.stiffness = G.d.stiffness;
      B2G_JI_FINISH;
    } break;
    case B2G_JOINT_WELD: {
      B2G_JI_COMMON(B2G_JOINT_WELD);
      J.d.damping = G.d.damping; J.d.reference_angle = G.d.reference_angle; J.d.stiffness = G.d.stiffness;
      B2G_JI_FINISH;
    } break;
    case B2G_JOINT_WHEEL: {
      B2G_JI_COMMON(B2G_JOINT_WHEEL);
      B2G_JI_AXES;
      J.d.damping = G.d.damping; J.d.stiffness = G.d.stiffness; J.d.lower = G.d.lower; J.d.upper = G.d.upper;
      J.d.motor_speed = G.d.motor_speed; J.d.max_motor = G.d.max_motor;
      B2G_JI_FINISH;
    } break;
    case B2G_JOINT_MOTOR:
    case B2G_JOINT_FRICTION: {
      B2G_JI_COMMON(G.d.type);
      J.d.linear_offset[0] = G.d.linear_offset[0]; J.d.linear_offset[1] = G.d.linear_offset[1];
      J.d.reference_angle = G.d.reference_angle; J.d.max_force = G.d.max_force; J.d.max_torque = G.d.max_torque;
      J.d.correction_factor = G.d.correction_factor;
      B2G_JI_FINISH;
    } break;
    case B2G_JOINT_MOUSE: {
      B2G_JI_COMMON(B2G_JOINT_MOUSE);
      J.d.damping = G.d.damping; J.d.stiffness = G.d.stiffness;
      J.d.target[0] = G.d.target[0]; J.d.target[1] = G.d.target[1]; J.d.max_force = G.d.max_force;
      B2G_JI_FINISH;
    } break;
    default: {  // pulley
      B2G_JI_COMMON(B2G_JOINT_PULLEY);
      J.d.ground_anchor_a[0] = G.d.ground_anchor_a[0]; J.d.ground_anchor_a[1] = G.d.ground_anchor_a[1];
      J.d.ground_anchor_b[0] = G.d.ground_anchor_b[0]; J.d.ground_anchor_b[1] = G.d.ground_anchor_b[1];
      J.d.ratio = G.d.ratio; J.constant = G.constant;
      B2G_JI_FINISH;
    } break;
  }
#undef B2G_JI_COMMON
#undef B2G_JI_AXES
#undef B2G_JI_FINISH
}

// One position iteration of the joint in `slot` (SolvePositionConstraints) on a per-type register
// copy of its rows; returns the joint's position check. A joint of a sleeping island is not called.
__device__ __forceinline__ bool jointSolvePositionSlot(const float4* P, int stride, int slot, float4* pos) {
  const float4 r0 = P[slot];
  const int type = __float_as_int(r0.z);
  if (type == B2G_JOINT_MOTOR || type == B2G_JOINT_FRICTION || type == B2G_JOINT_MOUSE) return true;
  const float4 r1 = P[(int64_t)stride + slot];
  const float4 r9 = P[(int64_t)9 * stride + slot], r10 = P[(int64_t)10 * stride + slot];
  const float4 r11 = P[(int64_t)11 * stride + slot], r12 = P[(int64_t)12 * stride + slot];
  const int flags = __float_as_int(r0.w);
#define B2G_JP_COMMON(TYPE)                                                                  \
  JointDev J;                                                                                \
  J.iA = __float_as_int(r0.x); J.iB = __float_as_int(r0.y); J.d.type = TYPE;                 \
  J.d.enable_limit = (flags & B2G_JV_LIMIT) ? 1 : 0;                                         \
  J.mA = r1.x; J.mB = r1.y; J.invIA = r1.z; J.invIB = r1.w;                                  \
  J.d.local_anchor_a[0] = r9.x; J.d.local_anchor_a[1] = r9.y;                                \
  J.d.local_anchor_b[0] = r9.z; J.d.local_anchor_b[1] = r9.w;                                \
  J.lcA[0] = r10.x; J.lcA[1] = r10.y; J.lcB[0] = r10.z; J.lcB[1] = r10.w
  bool ok = true;
  switch (type) {
    case B2G_JOINT_REVOLUTE: {
      B2G_JP_COMMON(B2G_JOINT_REVOLUTE);
      J.axialMass = r11.x; J.d.reference_angle = r11.y; J.d.lower = r11.z; J.d.upper = r11.w;
      ok = jointSolvePosition(J, pos);
    } break;
    case B2G_JOINT_PRISMATIC: {
      B2G_JP_COMMON(B2G_JOINT_PRISMATIC);
      J.localXAxisA[0] = r11.x; J.localXAxisA[1] = r11.y; J.localYAxisA[0] = r11.z; J.localYAxisA[1] = r11.w;
      J.d.reference_angle = r12.x; J.d.lower = r12.y; J.d.upper = r12.z;
      ok = jointSolvePosition(J, pos);
    } break;
    case B2G_JOINT_DISTANCE: {
      B2G_JP_COMMON(B2G_JOINT_DISTANCE);
      J.d.max_length = r11.x; J.d.min_length = r11.y; J.mass = r11.z;
      ok = jointSolvePosition(J, pos);
    } break;
    case B2G_JOINT_WELD: {
      B2G_JP_COMMON(B2G_JOINT_WELD);
      J.d.reference_angle = r11.x; J.d.stiffness = r11.y;
      ok = jointSolvePosition(J, pos);
    } break;
    case B2G_JOINT_WHEEL: {
      B2G_JP_COMMON(B2G_JOINT_WHEEL);
      const float4 r2 = P[(int64_t)2 * stride + slot];
      J.axis[0] = r2.x; J.axis[1] = r2.y;
      J.localXAxisA[0] = r11.x; J.localXAxisA[1] = r11.y; J.localYAxisA[0] = r11.z; J.localYAxisA[1] = r11.w;
      J.d.lower = r12.x; J.d.upper = r12.y; J.s1 = r12.z; J.s2 = r12.w;
      ok = jointSolvePosition(J, pos);
    } break;
    default: {  // pulley
      B2G_JP_COMMON(B2G_JOINT_PULLEY);
      J.d.ground_anchor_a[0] = r11.x; J.d.ground_anchor_a[1] = r11.y;
      J.d.ground_anchor_b[0] = r11.z; J.d.ground_anchor_b[1] = r11.w;
      J.constant = r12.x; J.d.ratio = r12.y;
      ok = jointSolvePosition(J, pos);
    } break;
  }
#undef B2G_JP_COMMON
  return ok;
}

// A joint left out of this step (its island sleeps): its velocity iterations skip it.
__device__ __forceinline__ void jointPackAsleep(float4* P, int slot) {
  P[slot] = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(B2G_JV_ASLEEP));
}
__device__ __forceinline__ void jointPackGear(float4* P, int slot, int bodyA, int bodyB) {
  P[slot] = make_float4(__int_as_float(bodyA), __int_as_float(bodyB), 0.0f, __int_as_float(B2G_JV_GEAR));
}
__device__ __forceinline__ bool jointSlotIsGear(const float4* P, int slot) {
  return (__float_as_int(P[slot].w) & B2G_JV_GEAR) != 0;
}

// One velocity iteration of the joint in `slot`: the register copy of its rows through
// jointSolveVelocity, its impulses written back to the rows.
__device__ __forceinline__ void jointSolveVelocitySlot(float4* P, int stride, int slot, float4* vel, float dt,
                                                      float inv_dt) {
  const float4 r0 = P[slot];
  const int flags = __float_as_int(r0.w);
  if (flags & B2G_JV_ASLEEP) return;
  const float4 r1 = P[(int64_t)stride + slot], r2 = P[(int64_t)2 * stride + slot], r3 = P[(int64_t)3 * stride + slot];
  const float4 r4 = P[(int64_t)4 * stride + slot], r5 = P[(int64_t)5 * stride + slot], r6 = P[(int64_t)6 * stride + slot];
  const float4 r7 = P[(int64_t)7 * stride + slot], r8 = P[(int64_t)8 * stride + slot];
  // each type on its own register copy with a constant type, so that only its branch of
  // jointSolveVelocity remains and the copy stays in registers
#define B2G_JV_COMMON(TYPE)                                                                   \
  JointDev J;                                                                                 \
  J.iA = __float_as_int(r0.x); J.iB = __float_as_int(r0.y); J.d.type = TYPE;                  \
  J.d.enable_motor = (flags & B2G_JV_MOTOR) ? 1 : 0;                                          \
  J.d.enable_limit = (flags & B2G_JV_LIMIT) ? 1 : 0;                                          \
  J.mA = r1.x; J.mB = r1.y; J.invIA = r1.z; J.invIB = r1.w;                                   \
  J.impulse[0] = r7.x; J.impulse[1] = r7.y; J.impulse[2] = r7.z; J.motorImpulse = r7.w;       \
  J.lowerImpulse = r8.x; J.upperImpulse = r8.y;                                               \
  J.rA[0] = r2.x; J.rA[1] = r2.y; J.rB[0] = r2.z; J.rB[1] = r2.w
#define B2G_JV_FINISH                                                                         \
  jointSolveVelocity(J, vel, dt, inv_dt);                                                     \
  P[(int64_t)7 * stride + slot] = make_float4(J.impulse[0], J.impulse[1], J.impulse[2], J.motorImpulse); \
  P[(int64_t)8 * stride + slot] = make_float4(J.lowerImpulse, J.upperImpulse, 0.0f, 0.0f)
  switch (__float_as_int(r0.z)) {
    case B2G_JOINT_REVOLUTE: {
      B2G_JV_COMMON(B2G_JOINT_REVOLUTE);
      J.K[0] = r3.x; J.K[1] = r3.y; J.K[2] = r3.z; J.K[3] = r3.w;
      J.axialMass = r4.x; J.angle = r4.y; J.d.lower = r4.z; J.d.upper = r4.w;
      J.d.motor_speed = r5.x; J.d.max_motor = r5.y;
      B2G_JV_FINISH;
    } break;
    case B2G_JOINT_PRISMATIC: {
      B2G_JV_COMMON(B2G_JOINT_PRISMATIC);
      J.axis[0] = r2.x; J.axis[1] = r2.y; J.perp[0] = r2.z; J.perp[1] = r2.w;
      J.a1 = r3.x; J.a2 = r3.y; J.s1 = r3.z; J.s2 = r3.w;
      J.K[0] = r4.x; J.K[1] = r4.y; J.K[2] = r4.z; J.K[3] = r4.w;
      J.axialMass = r5.x; J.translation = r5.y; J.d.lower = r5.z; J.d.upper = r5.w;
      J.d.motor_speed = r6.x; J.d.max_motor = r6.y;
      B2G_JV_FINISH;
    } break;
    case B2G_JOINT_WHEEL: {
      B2G_JV_COMMON(B2G_JOINT_WHEEL);
      J.axis[0] = r2.x; J.axis[1] = r2.y; J.perp[0] = r2.z; J.perp[1] = r2.w;
      J.a1 = r3.x; J.a2 = r3.y; J.s1 = r3.z; J.s2 = r3.w;
      J.motorMass = r4.x; J.bias = r4.y; J.gamma = r4.z;
      J.axialMass = r5.x; J.translation = r5.y; J.d.lower = r5.z; J.d.upper = r5.w;
      J.d.motor_speed = r6.x; J.d.max_motor = r6.y; J.mass = r6.z; J.springMass = r6.w;
      B2G_JV_FINISH;
    } break;
    case B2G_JOINT_DISTANCE: {
      B2G_JV_COMMON(B2G_JOINT_DISTANCE);
      J.u[0] = r3.x; J.u[1] = r3.y; J.softMass = r3.z; J.bias = r3.w;
      J.gamma = r4.x; J.mass = r4.y; J.currentLength = r4.z; J.d.min_length = r4.w;
      J.d.max_length = r5.x; J.d.stiffness = r5.y;
      B2G_JV_FINISH;
    } break;
    case B2G_JOINT_WELD: {
      B2G_JV_COMMON(B2G_JOINT_WELD);
      J.mass3[0] = r3.x; J.mass3[1] = r3.y; J.mass3[2] = r3.z; J.mass3[3] = r3.w;
      J.mass3[4] = r4.x; J.mass3[5] = r4.y; J.mass3[6] = r4.z; J.mass3[7] = r4.w;
      J.mass3[8] = r5.x; J.bias = r5.y; J.gamma = r5.z; J.d.stiffness = r5.w;
      B2G_JV_FINISH;
    } break;
    case B2G_JOINT_MOTOR:
    case B2G_JOINT_FRICTION: {
      B2G_JV_COMMON(__float_as_int(r0.z));
      J.K[0] = r3.x; J.K[1] = r3.y; J.K[2] = r3.z; J.K[3] = r3.w;
      J.axialMass = r4.x; J.d.max_force = r4.y; J.d.max_torque = r4.z; J.d.correction_factor = r4.w;
      J.angularError = r5.x; J.err[0] = r5.y; J.err[1] = r5.z;
      B2G_JV_FINISH;
    } break;
    case B2G_JOINT_MOUSE: {
      B2G_JV_COMMON(B2G_JOINT_MOUSE);
      J.K[0] = r3.x; J.K[1] = r3.y; J.K[2] = r3.z; J.K[3] = r3.w;
      J.err[0] = r4.x; J.err[1] = r4.y; J.gamma = r4.z; J.d.max_force = r4.w;
      B2G_JV_FINISH;
    } break;
    default: {  // pulley
      B2G_JV_COMMON(B2G_JOINT_PULLEY);
      J.u[0] = r3.x; J.u[1] = r3.y; J.uB[0] = r3.z; J.uB[1] = r3.w;
      J.mass = r4.x; J.d.ratio = r4.y;
      B2G_JV_FINISH;
    } break;
  }
#undef B2G_JV_COMMON
#undef B2G_JV_FINISH
}

// The accumulated impulses of the joint in `slot` back into its record, with the step's constraint
// directions its reaction force is read along (prismatic and wheel axes, distance and pulley
// directions).
__device__ __forceinline__ void jointStoreImpulses(const float4* P, int stride, int slot, JointDev& J) {
  const float4 r0 = P[slot];
  if (__float_as_int(r0.w) & B2G_JV_ASLEEP) return;
  const float4 i0 = P[(int64_t)7 * stride + slot], i1 = P[(int64_t)8 * stride + slot];
  J.impulse[0] = i0.x; J.impulse[1] = i0.y; J.impulse[2] = i0.z; J.motorImpulse = i0.w;
  J.lowerImpulse = i1.x; J.upperImpulse = i1.y;
  const int type = __float_as_int(r0.z);
  if (type == B2G_JOINT_PRISMATIC || type == B2G_JOINT_WHEEL) {
    const float4 r2 = P[(int64_t)2 * stride + slot];
    J.axis[0] = r2.x; J.axis[1] = r2.y; J.perp[0] = r2.z; J.perp[1] = r2.w;
  } else if (type == B2G_JOINT_DISTANCE) {
    const float4 r3 = P[(int64_t)3 * stride + slot];
    J.u[0] = r3.x; J.u[1] = r3.y;
  } else if (type == B2G_JOINT_PULLEY) {
    const float4 r3 = P[(int64_t)3 * stride + slot];
    J.u[0] = r3.x; J.u[1] = r3.y; J.uB[0] = r3.z; J.uB[1] = r3.w;
  }
}
#endif

}  // namespace b2g
