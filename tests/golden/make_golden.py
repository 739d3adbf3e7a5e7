"""Generates the golden vectors in tests/golden/ from the reference engine.

Run where the reference sources are checked out and oracle/_ref/libb2ref.so is built
(`make -C oracle ref`):

    python tests/golden/make_golden.py

Every vector is an output of the reference's own code (compiled from its sources) on seeded
inputs: polygon hulls and mass data (b2PolygonShape::Set / SetAsBox / ComputeMass), manifolds of
the five collide functions, one replayed solver step (b2Island::Solve in a given constraint
order) on exported world states, the listener callbacks of one replayed step, the final state of
a 256-step reference rollout, the physical measures of 256-step reference rollouts, and
b2TimeOfImpact on swept shape pairs (`python tests/golden/make_golden.py toi` writes those alone).
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
import oracle_bind as ob  # noqa: E402

G = ob.G


def rec_bytes(arr):
    return np.frombuffer(b"".join(bytes(x) for x in arr), dtype=np.uint8)


def shapes(ref, rng):
    n = 400
    counts = rng.integers(3, 9, n)
    verts = rng.uniform(-1, 1, (n, 16)).astype(np.float32)
    hulls, masses = [], []
    for i in range(n):
        s = G.Shape()
        ref.ref_polygon_set(verts[i].ctypes.data_as(C.POINTER(C.c_float)), int(counts[i]), s)
        m = (C.c_float * 4)()
        ref.ref_shape_mass(s, 1.7, m)
        hulls.append(s)
        masses.append(list(m))
    boxes = rng.uniform(0.05, 2.0, (100, 5)).astype(np.float32)
    boxes[:, 2:4] = rng.uniform(-50, 50, (100, 2))
    boxes[:, 4] = rng.uniform(-3, 3, 100)
    box_out = []
    for b in boxes:
        s = G.Shape()
        ref.ref_polygon_box(float(b[0]), float(b[1]), float(b[2]), float(b[3]), float(b[4]), 1, s)
        box_out.append(s)
    np.savez_compressed(HERE / "shapes.npz", counts=counts, verts=verts, hulls=rec_bytes(hulls),
                        masses=np.array(masses, np.float32), boxes=boxes, box_shapes=rec_bytes(box_out))


def rand_shape(ref, rng, kind):
    s = G.Shape()
    if kind == 0:
        s.type = 0
        s.radius = float(rng.uniform(0.1, 0.6))
        s.vertices[0][0] = float(rng.uniform(-0.2, 0.2))
        s.vertices[0][1] = float(rng.uniform(-0.2, 0.2))
    elif kind == 1:
        s.type = 1
        s.radius = 0.01
        for i in range(4):
            s.vertices[i][0] = float(rng.uniform(-2, 2))
            s.vertices[i][1] = float(rng.uniform(-2, 2))
        s.one_sided = int(rng.integers(0, 2))
    else:
        n = int(rng.integers(3, 9))
        xy = rng.uniform(-0.6, 0.6, 2 * n).astype(np.float32)
        if rng.uniform() < 0.3:
            ref.ref_polygon_box(float(rng.uniform(0.1, 0.5)), float(rng.uniform(0.1, 0.5)), 0, 0, 0, 0, s)
        else:
            ref.ref_polygon_set(xy.ctypes.data_as(C.POINTER(C.c_float)), n, s)
    return s


def collide(ref, rng):
    kinds = [(0, 0), (2, 0), (2, 2), (1, 0), (1, 2)]
    n = 1500
    A, B, M = [], [], []
    xa = np.zeros((n, 4), np.float32)
    xb = np.zeros((n, 4), np.float32)
    for i in range(n):
        ka, kb = kinds[i % 5]
        a, b = rand_shape(ref, rng, ka), rand_shape(ref, rng, kb)
        for x in (xa, xb):
            ang = rng.uniform(-3.2, 3.2)
            x[i] = (rng.uniform(-0.7, 0.7), rng.uniform(-0.7, 0.7), np.sin(ang), np.cos(ang))
        m = G.Manifold()
        ref.ref_collide(a, (C.c_float * 4)(*xa[i]), b, (C.c_float * 4)(*xb[i]), m)
        A.append(a)
        B.append(b)
        M.append(m)
    np.savez_compressed(HERE / "collide.npz", a=rec_bytes(A), b=rec_bytes(B), xa=xa, xb=xb, m=rec_bytes(M))


def replay(ref, orc, name, kind, n, seed, p0, warm, vi, pi):
    """World state after `warm` reference steps, and the reference's next step replayed in the
    oracle's constraint order (the oracle runs with libm trig, like the reference)."""
    rw = ob.RefWorld(ref, kind, seed=seed, n=n, p0=p0, p1=0.6)
    rw.step(warm, vi=vi, pi=pi)
    bodies, fixtures, joints, contacts = rw.bodies(), rw.fixtures(), rw.joints(), rw.contacts()
    orc.orc_set_libm_trig(1)
    ow = ob.OracleWorld(orc, (0.0, -10.0), list(bodies), list(fixtures), list(joints), list(contacts), inv_dt0=60.0)
    ow.step(1, 1 / 60, vi, pi)
    orc.orc_set_libm_trig(0)
    pairs, jorder = ow.last_order()
    arr = (C.c_int32 * max(len(pairs), 1))(*pairs)
    jar = (C.c_int32 * max(len(jorder), 1))(*jorder)
    assert ref.ref_replay_step(rw.h, 1 / 60, vi, pi, arr, len(pairs) // 2, jar, len(jorder)) == 0
    after = rw.bodies()
    np.savez_compressed(HERE / f"replay_{name}.npz", bodies=rec_bytes(bodies), fixtures=rec_bytes(fixtures),
                        joints=rec_bytes(joints) if joints else np.zeros(0, np.uint8), contacts=rec_bytes(contacts),
                        order_pairs=np.array(pairs, np.int32), order_joints=np.array(jorder, np.int32),
                        after=rec_bytes(after), vi=vi, pi=pi)


def events(ref, orc, name, kind, n, seed, p0, warm, vi, pi):
    """World state after `warm` reference steps and the reference's listener callbacks during its
    next step, replayed in the oracle's solver order: (kind, fixture A, fixture B, point count,
    old manifold point count, normal impulses, tangent impulses) per callback."""
    rw = ob.RefWorld(ref, kind, seed=seed, n=n, p0=p0, p1=0.6)
    rw.step(warm, vi=vi, pi=pi)
    bodies, fixtures, joints, contacts = rw.bodies(), rw.fixtures(), rw.joints(), rw.contacts()
    orc.orc_set_libm_trig(1)
    ow = ob.OracleWorld(orc, (0.0, -10.0), list(bodies), list(fixtures), list(joints), list(contacts), inv_dt0=60.0)
    ow.step(1, 1 / 60, vi, pi)
    orc.orc_set_libm_trig(0)
    pairs, jorder = ow.last_order()
    arr = (C.c_int32 * max(len(pairs), 1))(*pairs)
    jar = (C.c_int32 * max(len(jorder), 1))(*jorder)
    rw.events_enable(True)
    assert ref.ref_replay_step(rw.h, 1 / 60, vi, pi, arr, len(pairs) // 2, jar, len(jorder)) == 0
    ev = rw.events()
    ints = np.array([(e.kind, e.fixture_a, e.fixture_b, e.point_count, e.old_manifold.point_count) for e in ev],
                    np.int32)
    imps = np.array([tuple(e.normal_impulses) + tuple(e.tangent_impulses) for e in ev], np.float32)
    np.savez_compressed(HERE / f"events_{name}.npz", bodies=rec_bytes(bodies), fixtures=rec_bytes(fixtures),
                        joints=rec_bytes(joints) if joints else np.zeros(0, np.uint8), contacts=rec_bytes(contacts),
                        ints=ints, impulses=imps, vi=vi, pi=pi)


def rollout(ref, name, kind, n, seed, p0, steps, vi, pi):
    rw = ob.RefWorld(ref, kind, seed=seed, n=n, p0=p0, p1=0.6)
    start = rw.bodies()
    rw.step(steps, vi=vi, pi=pi)
    np.savez_compressed(HERE / f"rollout_{name}.npz", start=rec_bytes(start), final=rec_bytes(rw.bodies()),
                        steps=steps, vi=vi, pi=pi)


MEASURE_KEYS = ("linear", "angular", "com_height", "top_height", "penetration")


def measures(ref, orc, name, kind, n, seed, p0, steps, vi, pi, every=32):
    """Physical measures (oracle_bind.rollout_measures) of the reference's own rollout every
    `every` steps: linear momentum (2), angular momentum, centre-of-mass height, top height and
    deepest penetration per row."""
    rw = ob.RefWorld(ref, kind, seed=seed, n=n, p0=p0, p1=0.6)
    rows = []
    for _ in range(steps // every):
        rw.step(every, vi=vi, pi=pi)
        m = ob.rollout_measures(orc, list(rw.bodies()), list(rw.fixtures()), list(rw.contacts()))
        rows.append([m["linear"][0], m["linear"][1], m["angular"], m["com_height"], m["top_height"], m["penetration"]])
    np.savez_compressed(HERE / f"measures_{name}.npz", rows=np.array(rows, np.float64), every=every, steps=steps,
                        vi=vi, pi=pi, kind=kind, n=n, seed=seed, p0=p0)


def toi(ref, rng, n=1500):
    """b2TimeOfImpact on swept shape pairs: random sweeps, and sweeps where A crosses a slowly
    moving B (touching times inside (0, 1), the root finder's work), some with alpha0 > 0 and
    tMax < 1."""
    kinds = [(0, 0), (2, 0), (2, 2), (1, 0), (1, 2), (0, 2), (2, 1)]
    arr = (G.TOIInput * n)()
    for i in range(n):
        ka, kb = kinds[i % len(kinds)]
        q = arr[i]
        q.shape_a = rand_shape(ref, rng, ka)
        q.shape_b = rand_shape(ref, rng, kb)
        cross = i % 2 == 1
        for k, sw in enumerate((q.sweep_a, q.sweep_b)):
            sw.local_center[:] = rng.uniform(-0.2, 0.2, 2)
            if cross and k == 0:
                d = rng.uniform(1.5, 6.0)
                th = rng.uniform(-3.2, 3.2)
                sw.c0[:] = (-d * np.cos(th), -d * np.sin(th))
                sw.c[:] = (d * np.cos(th) + rng.uniform(-0.5, 0.5), d * np.sin(th) + rng.uniform(-0.5, 0.5))
            elif cross:
                c0 = rng.uniform(-0.3, 0.3, 2)
                sw.c0[:] = c0
                sw.c[:] = c0 + rng.uniform(-0.2, 0.2, 2)
            else:
                c0 = rng.uniform(-2, 2, 2)
                sw.c0[:] = c0
                sw.c[:] = c0 + rng.uniform(-3, 3, 2)
            sw.a0 = rng.uniform(-7, 7)
            sw.a = sw.a0 + rng.uniform(-2, 2)
            sw.alpha0 = 0.0 if i % 5 else float(rng.uniform(0.0, 0.6))
        q.t_max = 1.0 if i % 4 else float(rng.uniform(0.3, 1.0))
    out = (G.TOIOutput * n)()
    ref.ref_time_of_impact(arr, n, out)
    np.savez_compressed(HERE / "toi.npz", inputs=rec_bytes(arr), states=np.array([o.state for o in out], np.int32),
                        t=np.array([o.t for o in out], np.float32))


def replay_toi(ref, orc, seed=3, n=12, warm=5, steps=10, vi=8, pi=3):
    """Consecutive steps of the bullets scene with continuous collision, each replayed by the
    reference (b2Island::Solve in the oracle's order, then b2World::SolveTOI) from the state the
    reference reached: per step the state before, the order and the bodies after."""
    rw = ob.RefWorld(ref, G.SCENE_BULLETS, seed=seed, n=n, p0=0.0, p1=0.6, continuous=True)
    rw.step(warm, vi=vi, pi=pi)
    out = {"bodies": [], "contacts": [], "pairs": [], "after": [], "after_pairs": []}
    fixtures = rw.fixtures()
    orc.orc_set_libm_trig(1)
    for _ in range(steps):
        bodies, contacts = rw.bodies(), rw.contacts()
        ow = ob.OracleWorld(orc, (0.0, -10.0), list(bodies), list(fixtures), [], list(contacts), inv_dt0=60.0,
                            continuous=True)
        ow.step(1, 1 / 60, vi, pi)
        pairs, _ = ow.last_order()
        arr = (C.c_int32 * max(len(pairs), 1))(*pairs)
        assert ref.ref_replay_step(rw.h, 1 / 60, vi, pi, arr, len(pairs) // 2, (C.c_int32 * 1)(), 0) == 0
        out["bodies"].append(rec_bytes(bodies))
        out["contacts"].append(rec_bytes(contacts) if len(contacts) else np.zeros(0, np.uint8))
        out["pairs"].append(np.array(pairs, np.int32))
        out["after"].append(rec_bytes(rw.bodies()))
        out["after_pairs"].append(np.array(sorted((min(c.fixture_a, c.fixture_b), max(c.fixture_a, c.fixture_b))
                                                  for c in rw.contacts()), np.int32).reshape(-1))
    orc.orc_set_libm_trig(0)
    flat = {}
    for k, v in out.items():
        flat[k] = np.concatenate(v) if v else np.zeros(0)
        flat[k + "_off"] = np.cumsum([0] + [len(x) for x in v]).astype(np.int64)
    np.savez_compressed(HERE / "replay_bullets.npz", fixtures=rec_bytes(fixtures), vi=vi, pi=pi, **flat)


def main():
    ref = ob.Ref()
    if sys.argv[1:] == ["toi"]:  # the continuous-collision vectors alone
        toi(ref, np.random.default_rng(20261204))
        replay_toi(ref, ob.Oracle())
        return
    orc = ob.Oracle()
    rng = np.random.default_rng(20261203)
    shapes(ref, rng)
    collide(ref, rng)
    replay(ref, orc, "pyramid", G.SCENE_PYRAMID, 20, 1, 1.0, 40, 8, 3)
    replay(ref, orc, "mixed", G.SCENE_MIXED_DROP, 300, 3, 0.0, 150, 8, 3)
    replay(ref, orc, "chains", G.SCENE_CHAINS, 10, 2, 150.0, 100, 10, 4)
    replay(ref, orc, "sliders", G.SCENE_SLIDERS, 3, 9, 0.0, 60, 8, 3)
    replay(ref, orc, "gears", G.SCENE_GEARS, 3, 9, 0.0, 90, 8, 3)
    rollout(ref, "pyramid", G.SCENE_PYRAMID, 20, 1, 1.0, 256, 8, 3)
    events(ref, orc, "mixed", G.SCENE_MIXED_DROP, 400, 5, 0.0, 200, 8, 3)
    events(ref, orc, "chains", G.SCENE_CHAINS, 15, 4, 200.0, 80, 10, 4)
    measures(ref, orc, "pyramid", G.SCENE_PYRAMID, 20, 1, 1.0, 256, 8, 3)
    measures(ref, orc, "mixed", G.SCENE_MIXED_DROP, 300, 3, 0.0, 256, 8, 3)
    measures(ref, orc, "chains", G.SCENE_CHAINS, 10, 2, 150.0, 256, 10, 4)
    toi(ref, np.random.default_rng(20261204))
    replay_toi(ref, orc)
    print("golden vectors written to", HERE)


if __name__ == "__main__":
    main()
