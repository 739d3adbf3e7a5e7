// toi.cuh - time of impact of two swept shapes, callable from host and device.
//
// b2TimeOfImpact (src/collision/b2_time_of_impact.cpp:258-490): conservative advancement over
// the GJK distance with a warm-started simplex cache (b2Distance, src/collision/b2_distance.cpp:
// 86-135 ReadCache/WriteCache, 432-579), the separating-axis function of the cached simplex
// (b2SeparationFunction, b2_time_of_impact.cpp:35-251) and a mixed bisection/secant root finder.
// Sweeps follow b2Sweep (include/box2d/b2_math.h:707-733). The float operations are the
// reference's, in its order; rotations come from the portable sine/cosine like every other
// rotation of the engine.
#pragma once

#include "b2g_math.cuh"

namespace b2g {

// b2Sweep: local centre, centre and angle at alpha0 (c0, a0) and at the step's end (c, a).
struct Sweep {
  V2 lc, c0, c;
  float a0, a, alpha0;
};

// b2Sweep::GetTransform (b2_math.h:707-715)
B2G_HD Xf sweepXf(const Sweep& s, float beta) {
  Xf xf;
  xf.p = (1.0f - beta) * s.c0 + beta * s.c;
  float angle = (1.0f - beta) * s.a0 + beta * s.a;
  xf.q = rotOf(angle);
  xf.p = xf.p - mul(xf.q, s.lc);
  return xf;
}
// b2Sweep::Advance (b2_math.h:717-724)
B2G_HD void sweepAdvance(Sweep& s, float alpha) {
  float beta = (alpha - s.alpha0) / (1.0f - s.alpha0);
  s.c0 = s.c0 + beta * (s.c - s.c0);
  s.a0 += beta * (s.a - s.a0);
  s.alpha0 = alpha;
}
// b2Sweep::Normalize (b2_math.h:727-733)
B2G_HD void sweepNormalize(Sweep& s) {
  const float twoPi = 2.0f * B2G_PI;
  float d = twoPi * floorf(s.a0 / twoPi);
  s.a0 -= d;
  s.a -= d;
}

// b2SimplexCache (include/box2d/b2_distance.h:54-61)
struct SimplexCache {
  float metric;
  int count;
  int indexA[3], indexB[3];
};

// b2Simplex::GetMetric (b2_distance.cpp:248-271)
B2G_HD float simplexMetric3(const SimplexVertex& v0, const SimplexVertex& v1, const SimplexVertex& v2, int count) {
  if (count == 2) return lengthOf(v0.w - v1.w);
  if (count == 3) return cross(v1.w - v0.w, v2.w - v0.w);
  return 0.0f;
}

// b2Simplex::Solve2 (b2_distance.cpp:284-321) on named vertices (kept in registers)
B2G_HD void simplexSolve2r(SimplexVertex& v0, SimplexVertex& v1, int& count) {
  V2 w1 = v0.w, w2 = v1.w;
  V2 e12 = w2 - w1;
  float d12_2 = -dot(w1, e12);
  if (d12_2 <= 0.0f) {
    v0.a = 1.0f;
    count = 1;
    return;
  }
  float d12_1 = dot(w2, e12);
  if (d12_1 <= 0.0f) {
    v1.a = 1.0f;
    count = 1;
    v0 = v1;
    return;
  }
  float inv_d12 = 1.0f / (d12_1 + d12_2);
  v0.a = d12_1 * inv_d12;
  v1.a = d12_2 * inv_d12;
  count = 2;
}
// b2Simplex::Solve3 (b2_distance.cpp:323-430) on named vertices
B2G_HD void simplexSolve3r(SimplexVertex& v0, SimplexVertex& v1, SimplexVertex& v2, int& count) {
  V2 w1 = v0.w, w2 = v1.w, w3 = v2.w;
  V2 e12 = w2 - w1;
  float w1e12 = dot(w1, e12);
  float w2e12 = dot(w2, e12);
  float d12_1 = w2e12;
  float d12_2 = -w1e12;
  V2 e13 = w3 - w1;
  float w1e13 = dot(w1, e13);
  float w3e13 = dot(w3, e13);
  float d13_1 = w3e13;
  float d13_2 = -w1e13;
  V2 e23 = w3 - w2;
  float w2e23 = dot(w2, e23);
  float w3e23 = dot(w3, e23);
  float d23_1 = w3e23;
  float d23_2 = -w2e23;
  float n123 = cross(e12, e13);
  float d123_1 = n123 * cross(w2, w3);
  float d123_2 = n123 * cross(w3, w1);
  float d123_3 = n123 * cross(w1, w2);
  if (d12_2 <= 0.0f && d13_2 <= 0.0f) {
    v0.a = 1.0f;
    count = 1;
    return;
  }
  if (d12_1 > 0.0f && d12_2 > 0.0f && d123_3 <= 0.0f) {
    float inv_d12 = 1.0f / (d12_1 + d12_2);
    v0.a = d12_1 * inv_d12;
    v1.a = d12_2 * inv_d12;
    count = 2;
    return;
  }
  if (d13_1 > 0.0f && d13_2 > 0.0f && d123_2 <= 0.0f) {
    float inv_d13 = 1.0f / (d13_1 + d13_2);
    v0.a = d13_1 * inv_d13;
    v2.a = d13_2 * inv_d13;
    count = 2;
    v1 = v2;
    return;
  }
  if (d12_1 <= 0.0f && d23_2 <= 0.0f) {
    v1.a = 1.0f;
    count = 1;
    v0 = v1;
    return;
  }
  if (d13_1 <= 0.0f && d23_1 <= 0.0f) {
    v2.a = 1.0f;
    count = 1;
    v0 = v2;
    return;
  }
  if (d23_1 > 0.0f && d23_2 > 0.0f && d123_1 <= 0.0f) {
    float inv_d23 = 1.0f / (d23_1 + d23_2);
    v1.a = d23_1 * inv_d23;
    v2.a = d23_2 * inv_d23;
    count = 2;
    v0 = v2;
    return;
  }
  float inv_d123 = 1.0f / (d123_1 + d123_2 + d123_3);
  v0.a = d123_1 * inv_d123;
  v1.a = d123_2 * inv_d123;
  v2.a = d123_3 * inv_d123;
  count = 3;
}

B2G_HD void simplexVertexAt(SimplexVertex& v, int iA, int iB, const b2g_shape& A, const Xf& xfA, const b2g_shape& B,
                            const Xf& xfB) {
  v.indexA = iA;
  v.indexB = iB;
  v.wA = mul(xfA, proxyVertex(A, iA));
  v.wB = mul(xfB, proxyVertex(B, iB));
  v.w = v.wB - v.wA;
}

// b2Distance without radii (useRadii = false), warm-started from and written back to `cache`.
// Returns the distance between the witness points. The simplex's three vertices are named
// values, not an indexed array, so that they stay in registers.
B2G_HD float distanceCached(const b2g_shape& A, const Xf& xfA, const b2g_shape& B, const Xf& xfB,
                            SimplexCache& cache, V2* pA_out, V2* pB_out) {
  SimplexVertex v0 = {}, v1 = {}, v2 = {};
  // ReadCache
  int count = cache.count;
  if (count > 0) { simplexVertexAt(v0, cache.indexA[0], cache.indexB[0], A, xfA, B, xfB); v0.a = 0.0f; }
  if (count > 1) { simplexVertexAt(v1, cache.indexA[1], cache.indexB[1], A, xfA, B, xfB); v1.a = 0.0f; }
  if (count > 2) { simplexVertexAt(v2, cache.indexA[2], cache.indexB[2], A, xfA, B, xfB); v2.a = 0.0f; }
  if (count > 1) {
    float metric1 = cache.metric;
    float metric2 = simplexMetric3(v0, v1, v2, count);
    if (metric2 < 0.5f * metric1 || 2.0f * metric1 < metric2 || metric2 < B2G_EPSILON) count = 0;
  }
  if (count == 0) {
    simplexVertexAt(v0, 0, 0, A, xfA, B, xfB);
    v0.a = 1.0f;
    count = 1;
  }
  int sA0 = 0, sB0 = 0, sA1 = 0, sB1 = 0, sA2 = 0, sB2 = 0;
  for (int iter = 0; iter < 20;) {
    const int saveCount = count;
    sA0 = v0.indexA; sB0 = v0.indexB;
    sA1 = v1.indexA; sB1 = v1.indexB;
    sA2 = v2.indexA; sB2 = v2.indexB;
    if (count == 2) simplexSolve2r(v0, v1, count);
    else if (count == 3) simplexSolve3r(v0, v1, v2, count);
    if (count == 3) break;
    V2 d;
    if (count == 1) {
      d = -v0.w;
    } else {
      V2 e12 = v1.w - v0.w;
      float sgn = cross(e12, -v0.w);
      d = sgn > 0.0f ? cross(1.0f, e12) : cross(e12, 1.0f);
    }
    if (lengthSq(d) < B2G_EPSILON * B2G_EPSILON) break;
    const int iA = proxySupport(A, mulT(xfA.q, -d));
    const int iB = proxySupport(B, mulT(xfB.q, d));
    if (count == 1) simplexVertexAt(v1, iA, iB, A, xfA, B, xfB);
    else simplexVertexAt(v2, iA, iB, A, xfA, B, xfB);
    ++iter;
    const bool duplicate = (saveCount > 0 && iA == sA0 && iB == sB0) || (saveCount > 1 && iA == sA1 && iB == sB1) ||
                           (saveCount > 2 && iA == sA2 && iB == sB2);
    if (duplicate) break;
    ++count;
  }
  V2 pA, pB;
  if (count == 1) {
    pA = v0.wA;
    pB = v0.wB;
  } else if (count == 2) {
    pA = v0.a * v0.wA + v1.a * v1.wA;
    pB = v0.a * v0.wB + v1.a * v1.wB;
  } else {
    pA = (v0.a * v0.wA + v1.a * v1.wA) + v2.a * v2.wA;
    pB = pA;
  }
  // WriteCache
  cache.metric = simplexMetric3(v0, v1, v2, count);
  cache.count = count;
  cache.indexA[0] = v0.indexA; cache.indexB[0] = v0.indexB;
  if (count > 1) { cache.indexA[1] = v1.indexA; cache.indexB[1] = v1.indexB; }
  if (count > 2) { cache.indexA[2] = v2.indexA; cache.indexB[2] = v2.indexB; }
  if (pA_out) *pA_out = pA;
  if (pB_out) *pB_out = pB;
  return lengthOf(pA - pB);
}

// b2SeparationFunction: the separating axis of a cached simplex, as points (one vertex on each
// side), face of A or face of B.
struct SepFn {
  const b2g_shape* A;
  const b2g_shape* B;
  Sweep sA, sB;
  int type;  // 0 points, 1 face A, 2 face B
  V2 localPoint, axis;
};

// b2SeparationFunction::Initialize (b2_time_of_impact.cpp:47-125)
B2G_HD float sepInit(SepFn& f, const SimplexCache& cache, const b2g_shape& A, const Sweep& sA,
                     const b2g_shape& B, const Sweep& sB, float t1) {
  f.A = &A;
  f.B = &B;
  f.sA = sA;
  f.sB = sB;
  Xf xfA = sweepXf(sA, t1), xfB = sweepXf(sB, t1);
  if (cache.count == 1) {
    f.type = 0;
    V2 pointA = mul(xfA, proxyVertex(A, cache.indexA[0]));
    V2 pointB = mul(xfB, proxyVertex(B, cache.indexB[0]));
    f.axis = pointB - pointA;
    f.localPoint = mk(0.0f, 0.0f);
    return normalize(f.axis);
  }
  if (cache.indexA[0] == cache.indexA[1]) {
    f.type = 2;
    V2 localPointB1 = proxyVertex(B, cache.indexB[0]);
    V2 localPointB2 = proxyVertex(B, cache.indexB[1]);
    f.axis = cross(localPointB2 - localPointB1, 1.0f);
    normalize(f.axis);
    V2 normal = mul(xfB.q, f.axis);
    f.localPoint = 0.5f * (localPointB1 + localPointB2);
    V2 pointB = mul(xfB, f.localPoint);
    V2 pointA = mul(xfA, proxyVertex(A, cache.indexA[0]));
    float s = dot(pointA - pointB, normal);
    if (s < 0.0f) {
      f.axis = -f.axis;
      s = -s;
    }
    return s;
  }
  f.type = 1;
  V2 localPointA1 = proxyVertex(A, cache.indexA[0]);
  V2 localPointA2 = proxyVertex(A, cache.indexA[1]);
  f.axis = cross(localPointA2 - localPointA1, 1.0f);
  normalize(f.axis);
  V2 normal = mul(xfA.q, f.axis);
  f.localPoint = 0.5f * (localPointA1 + localPointA2);
  V2 pointA = mul(xfA, f.localPoint);
  V2 pointB = mul(xfB, proxyVertex(B, cache.indexB[0]));
  float s = dot(pointB - pointA, normal);
  if (s < 0.0f) {
    f.axis = -f.axis;
    s = -s;
  }
  return s;
}

// b2SeparationFunction::FindMinSeparation (b2_time_of_impact.cpp:128-195)
B2G_HD float sepFindMin(const SepFn& f, int* indexA, int* indexB, float t) {
  Xf xfA = sweepXf(f.sA, t), xfB = sweepXf(f.sB, t);
  if (f.type == 0) {
    V2 axisA = mulT(xfA.q, f.axis);
    V2 axisB = mulT(xfB.q, -f.axis);
    *indexA = proxySupport(*f.A, axisA);
    *indexB = proxySupport(*f.B, axisB);
    V2 pointA = mul(xfA, proxyVertex(*f.A, *indexA));
    V2 pointB = mul(xfB, proxyVertex(*f.B, *indexB));
    return dot(pointB - pointA, f.axis);
  }
  if (f.type == 1) {
    V2 normal = mul(xfA.q, f.axis);
    V2 pointA = mul(xfA, f.localPoint);
    V2 axisB = mulT(xfB.q, -normal);
    *indexA = -1;
    *indexB = proxySupport(*f.B, axisB);
    V2 pointB = mul(xfB, proxyVertex(*f.B, *indexB));
    return dot(pointB - pointA, normal);
  }
  V2 normal = mul(xfB.q, f.axis);
  V2 pointB = mul(xfB, f.localPoint);
  V2 axisA = mulT(xfA.q, -normal);
  *indexB = -1;
  *indexA = proxySupport(*f.A, axisA);
  V2 pointA = mul(xfA, proxyVertex(*f.A, *indexA));
  return dot(pointA - pointB, normal);
}

// b2SeparationFunction::Evaluate (b2_time_of_impact.cpp:198-245)
B2G_HD float sepEval(const SepFn& f, int indexA, int indexB, float t) {
  Xf xfA = sweepXf(f.sA, t), xfB = sweepXf(f.sB, t);
  if (f.type == 0) {
    V2 pointA = mul(xfA, proxyVertex(*f.A, indexA));
    V2 pointB = mul(xfB, proxyVertex(*f.B, indexB));
    return dot(pointB - pointA, f.axis);
  }
  if (f.type == 1) {
    V2 normal = mul(xfA.q, f.axis);
    V2 pointA = mul(xfA, f.localPoint);
    V2 pointB = mul(xfB, proxyVertex(*f.B, indexB));
    return dot(pointB - pointA, normal);
  }
  V2 normal = mul(xfB.q, f.axis);
  V2 pointB = mul(xfB, f.localPoint);
  V2 pointA = mul(xfA, proxyVertex(*f.A, indexA));
  return dot(pointA - pointB, normal);
}

// b2TimeOfImpact (b2_time_of_impact.cpp:258-490). Returns the state (B2G_TOI_*) and writes t.
B2G_HD int timeOfImpact(const b2g_shape& A, const b2g_shape& B, Sweep sweepA, Sweep sweepB, float tMax,
                        float* t_out) {
  int state = B2G_TOI_UNKNOWN;
  float t_res = tMax;
  sweepNormalize(sweepA);
  sweepNormalize(sweepB);
  const float totalRadius = A.radius + B.radius;
  const float target = fmax2(B2G_LINEAR_SLOP, totalRadius - 3.0f * B2G_LINEAR_SLOP);
  const float tolerance = 0.25f * B2G_LINEAR_SLOP;
  float t1 = 0.0f;
  const int kMaxIterations = 20;
  int iter = 0;
  SimplexCache cache;
  cache.count = 0;
  cache.metric = 0.0f;
  for (;;) {
    Xf xfA = sweepXf(sweepA, t1), xfB = sweepXf(sweepB, t1);
    float distance = distanceCached(A, xfA, B, xfB, cache, nullptr, nullptr);
    if (distance <= 0.0f) {
      state = B2G_TOI_OVERLAPPED;
      t_res = 0.0f;
      break;
    }
    if (distance < target + tolerance) {
      state = B2G_TOI_TOUCHING;
      t_res = t1;
      break;
    }
    SepFn fcn;
    sepInit(fcn, cache, A, sweepA, B, sweepB, t1);
    bool done = false;
    float t2 = tMax;
    int pushBackIter = 0;
    for (;;) {
      int indexA, indexB;
      float s2 = sepFindMin(fcn, &indexA, &indexB, t2);
      if (s2 > target + tolerance) {
        state = B2G_TOI_SEPARATED;
        t_res = tMax;
        done = true;
        break;
      }
      if (s2 > target - tolerance) {
        t1 = t2;
        break;
      }
      float s1 = sepEval(fcn, indexA, indexB, t1);
      if (s1 < target - tolerance) {
        state = B2G_TOI_FAILED;
        t_res = t1;
        done = true;
        break;
      }
      if (s1 <= target + tolerance) {
        state = B2G_TOI_TOUCHING;
        t_res = t1;
        done = true;
        break;
      }
      int rootIterCount = 0;
      float a1 = t1, a2 = t2;
      for (;;) {
        float t;
        if (rootIterCount & 1) t = a1 + (target - s1) * (a2 - a1) / (s2 - s1);
        else t = 0.5f * (a1 + a2);
        ++rootIterCount;
        float s = sepEval(fcn, indexA, indexB, t);
        if (fabs2(s - target) < tolerance) {
          t2 = t;
          break;
        }
        if (s > target) {
          a1 = t;
          s1 = s;
        } else {
          a2 = t;
          s2 = s;
        }
        if (rootIterCount == 50) break;
      }
      ++pushBackIter;
      if (pushBackIter == B2G_MAX_POLYGON_VERTICES) break;
    }
    ++iter;
    if (done) break;
    if (iter == kMaxIterations) {
      state = B2G_TOI_FAILED;
      t_res = t1;
      break;
    }
  }
  *t_out = t_res;
  return state;
}

}  // namespace b2g
