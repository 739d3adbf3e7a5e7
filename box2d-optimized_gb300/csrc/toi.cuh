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
B2G_HD float simplexMetric(const SimplexVertex* v, int count) {
  if (count == 2) return lengthOf(v[0].w - v[1].w);
  if (count == 3) return cross(v[1].w - v[0].w, v[2].w - v[0].w);
  return 0.0f;
}

// b2Distance without radii (useRadii = false), warm-started from and written back to `cache`.
// Returns the distance between the witness points pA and pB.
B2G_HD float distanceCached(const b2g_shape& A, const Xf& xfA, const b2g_shape& B, const Xf& xfB,
                            SimplexCache& cache, V2* pA_out, V2* pB_out) {
  SimplexVertex v[3];
  // ReadCache
  int count = cache.count;
  for (int i = 0; i < count; ++i) {
    v[i].indexA = cache.indexA[i];
    v[i].indexB = cache.indexB[i];
    v[i].wA = mul(xfA, proxyVertex(A, v[i].indexA));
    v[i].wB = mul(xfB, proxyVertex(B, v[i].indexB));
    v[i].w = v[i].wB - v[i].wA;
    v[i].a = 0.0f;
  }
  if (count > 1) {
    float metric1 = cache.metric;
    float metric2 = simplexMetric(v, count);
    if (metric2 < 0.5f * metric1 || 2.0f * metric1 < metric2 || metric2 < B2G_EPSILON) count = 0;
  }
  if (count == 0) {
    v[0].indexA = 0;
    v[0].indexB = 0;
    v[0].wA = mul(xfA, proxyVertex(A, 0));
    v[0].wB = mul(xfB, proxyVertex(B, 0));
    v[0].w = v[0].wB - v[0].wA;
    v[0].a = 1.0f;
    count = 1;
  }
  int saveA[3], saveB[3];
  for (int iter = 0; iter < 20;) {
    const int saveCount = count;
    for (int i = 0; i < saveCount; ++i) {
      saveA[i] = v[i].indexA;
      saveB[i] = v[i].indexB;
    }
    if (count == 2) simplexSolve2(v, count);
    else if (count == 3) simplexSolve3(v, count);
    if (count == 3) break;
    V2 d;
    if (count == 1) {
      d = -v[0].w;
    } else {
      V2 e12 = v[1].w - v[0].w;
      float sgn = cross(e12, -v[0].w);
      d = sgn > 0.0f ? cross(1.0f, e12) : cross(e12, 1.0f);
    }
    if (lengthSq(d) < B2G_EPSILON * B2G_EPSILON) break;
    SimplexVertex& nv = v[count];
    nv.indexA = proxySupport(A, mulT(xfA.q, -d));
    nv.wA = mul(xfA, proxyVertex(A, nv.indexA));
    nv.indexB = proxySupport(B, mulT(xfB.q, d));
    nv.wB = mul(xfB, proxyVertex(B, nv.indexB));
    nv.w = nv.wB - nv.wA;
    ++iter;
    bool duplicate = false;
    for (int i = 0; i < saveCount; ++i) {
      if (nv.indexA == saveA[i] && nv.indexB == saveB[i]) {
        duplicate = true;
        break;
      }
    }
    if (duplicate) break;
    ++count;
  }
  V2 pA, pB;
  if (count == 1) {
    pA = v[0].wA;
    pB = v[0].wB;
  } else if (count == 2) {
    pA = v[0].a * v[0].wA + v[1].a * v[1].wA;
    pB = v[0].a * v[0].wB + v[1].a * v[1].wB;
  } else {
    pA = (v[0].a * v[0].wA + v[1].a * v[1].wA) + v[2].a * v[2].wA;
    pB = pA;
  }
  // WriteCache
  cache.metric = simplexMetric(v, count);
  cache.count = count;
  for (int i = 0; i < count; ++i) {
    cache.indexA[i] = v[i].indexA;
    cache.indexB[i] = v[i].indexB;
  }
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
