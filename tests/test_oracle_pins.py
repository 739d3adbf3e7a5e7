"""Pins of the CPU oracle (and of the engine's host-side set-up) to the reference.

Two sources of truth:
* tests/golden/*.npz - outputs of the reference's own code on seeded inputs (generator:
  tests/golden/make_golden.py), usable everywhere;
* the reference compiled from its sources (oracle/_ref), where it is present: live comparisons
  on fresh random inputs.
Integer outputs (point counts, feature ids, pair sets) are compared exactly; float outputs of
shapes and collide functions bit for bit; one replayed solver step within 1e-5 relative (bit for
bit where the host's libm matches the reference's); rollouts by physical measures.
"""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

import b2gpu as G
import oracle_bind as ob

GOLD = Path(__file__).resolve().parent / "golden"


def recs(cls, raw):
    raw = bytes(np.asarray(raw, np.uint8))
    n = len(raw) // C.sizeof(cls)
    return list((cls * n).from_buffer_copy(raw)) if n else []


def test_oracle_shapes_vs_golden(orc):
    g = np.load(GOLD / "shapes.npz")
    hulls = recs(G.Shape, g["hulls"])
    for i, (cnt, v) in enumerate(zip(g["counts"], g["verts"])):
        s = G.Shape()
        orc.orc_polygon_set(np.ascontiguousarray(v).ctypes.data_as(C.POINTER(C.c_float)), int(cnt), s)
        assert bytes(s) == bytes(hulls[i]), i
        m = (C.c_float * 4)()
        orc.orc_shape_mass(s, 1.7, m)
        assert np.array_equal(np.array(list(m), np.float32), g["masses"][i]), i
    boxes = recs(G.Shape, g["box_shapes"])
    for b, ref_s in zip(g["boxes"], boxes):
        s = G.Shape()
        orc.orc_polygon_box(*[float(x) for x in b], 1, s)
        # oriented boxes use the host libm sinf/cosf, as b2Rot::Set does: equal up to libm ulps
        np.testing.assert_allclose(np.frombuffer(bytes(s), np.float32)[4:], np.frombuffer(bytes(ref_s), np.float32)[4:],
                                   rtol=2e-6, atol=2e-5)


def test_oracle_collide_vs_golden(orc):
    g = np.load(GOLD / "collide.npz")
    A, B, M = recs(G.Shape, g["a"]), recs(G.Shape, g["b"]), recs(G.Manifold, g["m"])
    touching = 0
    for i in range(len(A)):
        m = G.Manifold()
        orc.orc_collide(A[i], (C.c_float * 4)(*g["xa"][i]), B[i], (C.c_float * 4)(*g["xb"][i]), m)
        r = M[i]
        assert m.point_count == r.point_count, i
        if r.point_count:
            touching += 1
            assert m.type == r.type
            for j in range(r.point_count):
                assert m.points[j].id == r.points[j].id
                assert tuple(m.points[j].local_point) == tuple(r.points[j].local_point)
            assert tuple(m.local_normal) == tuple(r.local_normal)
            assert tuple(m.local_point) == tuple(r.local_point)
    assert touching > 300


def test_oracle_toi_vs_golden(orc):
    """b2TimeOfImpact: the oracle, with libm trig like the reference, gives the reference's states
    and times bit for bit on random and crossing sweeps (alpha0 > 0 and tMax < 1 included)."""
    g = np.load(GOLD / "toi.npz")
    inputs = recs(G.TOIInput, g["inputs"])
    n = len(inputs)
    arr = (G.TOIInput * n)(*inputs)
    out = (G.TOIOutput * n)()
    orc.orc_set_libm_trig(1)
    try:
        orc.orc_time_of_impact(arr, n, out)
    finally:
        orc.orc_set_libm_trig(0)
    states = np.array([o.state for o in out], np.int32)
    t = np.array([o.t for o in out], np.float32)
    assert np.array_equal(states, g["states"])
    assert np.array_equal(t.view(np.uint32), g["t"].view(np.uint32))
    assert (g["states"] == G.TOI_TOUCHING).sum() > 300 and ((g["t"] > 0) & (g["t"] < 1)).sum() > 300


def _split(g, key, i):
    off = g[key + "_off"]
    return g[key][off[i]:off[i + 1]]


def test_oracle_toi_replay_vs_golden(orc):
    """Continuous collision: ten consecutive steps of the bullets scene, each replayed by the
    reference (b2Island::Solve in the oracle's order, then b2World::SolveTOI); the oracle with
    continuous collision reproduces the bodies bit for bit (libm trig like the reference) and the
    contact set exactly, and without it differs (the impacts are resolved by SolveTOI)."""
    g = np.load(GOLD / "replay_bullets.npz")
    fixtures = recs(G.Fixture, g["fixtures"])
    vi, pi = int(g["vi"]), int(g["pi"])
    steps = len(g["bodies_off"]) - 1
    changed = 0
    orc.orc_set_libm_trig(1)
    try:
        for i in range(steps):
            bodies, contacts = recs(G.Body, _split(g, "bodies", i)), recs(G.Contact, _split(g, "contacts", i))
            after = bytes(np.asarray(_split(g, "after", i), np.uint8))
            results = {}
            for cont in (True, False):
                ow = ob.OracleWorld(orc, (0.0, -10.0), bodies, fixtures, [], contacts, inv_dt0=60.0, continuous=cont)
                ow.step(1, 1 / 60, vi, pi)
                results[cont] = ow
            ob_after = b"".join(bytes(b) for b in results[True].bodies())
            assert [ob_after[k * C.sizeof(G.Body):k * C.sizeof(G.Body) + 40] for k in range(len(bodies))] == \
                   [after[k * C.sizeof(G.Body):k * C.sizeof(G.Body) + 40] for k in range(len(bodies))], i
            pairs = sorted((min(c.fixture_a, c.fixture_b), max(c.fixture_a, c.fixture_b)) for c in results[True].contacts())
            assert np.array_equal(np.array(pairs, np.int32).reshape(-1), _split(g, "after_pairs", i)), i
            plain = b"".join(bytes(b)[:40] for b in results[False].bodies())
            changed += plain != b"".join(bytes(b)[:40] for b in results[True].bodies())
    finally:
        orc.orc_set_libm_trig(0)
    assert changed >= 3


@pytest.mark.parametrize("n,seed,p0", [(12, 1, 0.0), (12, 8, 0.0), (30, 4, 0.0), (16, 3, 1.0), (24, 7, 1.0)])
def test_oracle_toi_replay_vs_reference_live(ref, orc, n, seed, p0):
    """b2World::SolveTOI against the oracle's restatement over 40 replayed steps of the bullets
    scene (fired and thrown bullets, circles and squares; with p0 = 1 kinematic bars driven at
    boxes in every fourth lane), contacts exactly. The lanes of circle
    bullets match bit for bit. In the lanes of square bullets a polygon-polygon contact made by
    the pair update just before the impact takes its fixture order (which shape is A) from the
    reference's broadphase tree, where the oracle's is canonical: the manifold's frame differs,
    and those lanes agree to 1e-5."""
    rw = ob.RefWorld(ref, G.SCENE_BULLETS, seed=seed, n=n, p0=p0, p1=0.6, continuous=True)
    fixtures = list(rw.fixtures())
    orc.orc_set_libm_trig(1)
    try:
        for step in range(40):
            ow = ob.OracleWorld(orc, (0.0, -10.0), list(rw.bodies()), fixtures, [], list(rw.contacts()),
                                inv_dt0=60.0 if step else 0.0, continuous=True)
            ow.step(1, 1 / 60, 8, 3)
            pairs, _ = ow.last_order()
            arr = (C.c_int32 * max(len(pairs), 1))(*pairs)
            assert ref.ref_replay_step(rw.h, 1 / 60, 8, 3, arr, len(pairs) // 2, (C.c_int32 * 1)(), 0) == 0
            rset = sorted((min(c.fixture_a, c.fixture_b), max(c.fixture_a, c.fixture_b)) for c in rw.contacts())
            oset = sorted((min(c.fixture_a, c.fixture_b), max(c.fixture_a, c.fixture_b)) for c in ow.contacts())
            assert rset == oset, step
            rb, obs = list(rw.bodies()), list(ow.bodies())
            for k in range(len(rb)):
                circle_lane = k == 0 or ((k - 1) // 2) % 2 == 0
                if circle_lane:
                    assert bytes(rb[k])[:40] == bytes(obs[k])[:40], (step, k)
                else:
                    np.testing.assert_allclose(np.frombuffer(bytes(obs[k])[:40], np.float32),
                                               np.frombuffer(bytes(rb[k])[:40], np.float32), rtol=1e-5, atol=1e-5)
    finally:
        orc.orc_set_libm_trig(0)


@pytest.mark.parametrize("name", ["pyramid", "mixed", "chains", "sliders", "gears"])
def test_oracle_replayed_step_vs_golden(orc, name):
    """One step from an exported reference state; the reference's b2Island solved the constraints
    in the order the oracle chooses, so the two steps differ only by libm rounding."""
    g = np.load(GOLD / f"replay_{name}.npz")
    bodies, fixtures = recs(G.Body, g["bodies"]), recs(G.Fixture, g["fixtures"])
    joints, contacts = recs(G.Joint, g["joints"]), recs(G.Contact, g["contacts"])
    orc.orc_set_libm_trig(1)
    try:
        ow = ob.OracleWorld(orc, (0.0, -10.0), bodies, fixtures, joints, contacts, inv_dt0=60.0)
        ow.step(1, 1 / 60, int(g["vi"]), int(g["pi"]))
        pairs, jorder = ow.last_order()
    finally:
        orc.orc_set_libm_trig(0)
    assert pairs == list(g["order_pairs"]) and jorder == list(g["order_joints"])
    got = G.body_array_to_numpy((G.Body * len(bodies))(*ow.bodies()))
    exp = G.body_array_to_numpy((G.Body * len(bodies))(*recs(G.Body, g["after"])))
    for k in ("c", "a", "v", "w", "xf"):
        np.testing.assert_allclose(got[k], exp[k], rtol=1e-5, atol=1e-5, err_msg=k)


def test_oracle_rollout_vs_reference_golden(orc):
    """256-step pyramid (20 rows, density 1, friction 0.6): the oracle (engine order, portable
    trig) against the reference's own rollout, by physical measures."""
    g = np.load(GOLD / "rollout_pyramid.npz")
    start = recs(G.Body, g["start"])
    host_batch = _host_batch()
    w = host_batch.add_world(0.0, -10.0)
    host_batch.scene(w, G.SCENE_PYRAMID, n=20, p0=1.0, p1=0.6)
    assert b"".join(bytes(b) for b in host_batch.bodies(w)) == b"".join(bytes(b) for b in start)
    ow = ob.OracleWorld(orc, (0.0, -10.0), host_batch.bodies(w), host_batch.fixtures(w), host_batch.joints(w))
    ow.step(int(g["steps"]), 1 / 60, int(g["vi"]), int(g["pi"]))
    got = G.body_array_to_numpy((G.Body * len(start))(*ow.bodies()))
    exp = G.body_array_to_numpy((G.Body * len(start))(*recs(G.Body, g["final"])))
    dyn = exp["type"] == G.DYNAMIC
    assert abs(got["c"][dyn, 1].max() - exp["c"][dyn, 1].max()) < 0.02  # settled stack height
    assert np.abs(got["c"][dyn] - exp["c"][dyn]).max() < 0.1           # every box within a fifth of its size
    assert np.abs(got["v"][dyn]).max() < 0.5 and np.abs(exp["v"][dyn]).max() < 0.5
    host_batch.close()


def _host_batch():
    lib = G.Lib()
    b = G.Batch.__new__(G.Batch)
    b.lib = lib
    h = C.c_void_p()
    lib.check(lib.b2g_batch_create(-1, 0, C.byref(h)), "host batch")
    b.h = h
    return b


# ------------------------------------------------------------------ live, where the reference is built
def test_oracle_vs_reference_live(ref, orc):
    rng = np.random.default_rng(99)
    for _ in range(300):
        n = int(rng.integers(3, 9))
        xy = rng.uniform(-1, 1, 2 * n).astype(np.float32)
        a, b = G.Shape(), G.Shape()
        ref.ref_polygon_set(xy.ctypes.data_as(C.POINTER(C.c_float)), n, a)
        orc.orc_polygon_set(xy.ctypes.data_as(C.POINTER(C.c_float)), n, b)
        assert bytes(a) == bytes(b)


@pytest.mark.parametrize("kind,n,seed,p0,warm,vi,pi", [
    (G.SCENE_PYRAMID, 20, 1, 1.0, 30, 8, 3),
    (G.SCENE_MIXED_DROP, 400, 5, 0.0, 200, 8, 3),
    (G.SCENE_CHAINS, 15, 4, 200.0, 80, 10, 4),
    (G.SCENE_JOINTS, 3, 9, 0.0, 1, 8, 3),
    (G.SCENE_JOINTS, 3, 9, 0.0, 40, 8, 3),
    (G.SCENE_JOINTS, 2, 17, 0.0, 150, 10, 4),
    (G.SCENE_SLIDERS, 3, 9, 0.0, 1, 8, 3),
    (G.SCENE_SLIDERS, 3, 9, 0.0, 40, 8, 3),
    (G.SCENE_SLIDERS, 2, 17, 0.0, 150, 10, 4),
    (G.SCENE_GEARS, 3, 9, 0.0, 1, 8, 3),
    (G.SCENE_GEARS, 3, 9, 0.0, 60, 8, 3),
    (G.SCENE_GEARS, 2, 17, 0.0, 200, 10, 4),
])
def test_oracle_replay_vs_reference_live(ref, orc, kind, n, seed, p0, warm, vi, pi):
    """The reference's b2Island::Solve replaying the oracle's order: bit-exact, 3 steps."""
    rw = ob.RefWorld(ref, kind, seed=seed, n=n, p0=p0, p1=0.6)
    rw.step(warm, vi=vi, pi=pi)
    orc.orc_set_libm_trig(1)
    sensor_touching = 0
    try:
        for _ in range(3):
            ow = ob.OracleWorld(orc, (0.0, -10.0), list(rw.bodies()), list(rw.fixtures()), list(rw.joints()),
                                list(rw.contacts()), inv_dt0=60.0)
            ow.step(1, 1 / 60, vi, pi)
            pairs, jorder = ow.last_order()
            arr = (C.c_int32 * max(len(pairs), 1))(*pairs)
            jar = (C.c_int32 * max(len(jorder), 1))(*jorder)
            assert ref.ref_replay_step(rw.h, 1 / 60, vi, pi, arr, len(pairs) // 2, jar, len(jorder)) == 0
            assert b"".join(bytes(b)[:40] for b in rw.bodies()) == b"".join(bytes(b)[:40] for b in ow.bodies())
            rset = sorted((min(c.fixture_a, c.fixture_b), max(c.fixture_a, c.fixture_b)) for c in rw.contacts())
            oset = sorted((min(c.fixture_a, c.fixture_b), max(c.fixture_a, c.fixture_b)) for c in ow.contacts())
            assert rset == oset
            # sensor contacts: touching is the GJK overlap (b2TestOverlap) on both sides
            sensors = {i for i, f in enumerate(rw.fixtures()) if f.is_sensor}
            key = lambda c: (min(c.fixture_a, c.fixture_b), max(c.fixture_a, c.fixture_b))  # noqa: E731
            rs = {key(c): c.flags & 2 for c in rw.contacts() if {c.fixture_a, c.fixture_b} & sensors}
            os_ = {key(c): c.flags & 2 for c in ow.contacts() if {c.fixture_a, c.fixture_b} & sensors}
            assert rs == os_
            sensor_touching += sum(1 for v in rs.values() if v)
    finally:
        orc.orc_set_libm_trig(0)
    if kind == G.SCENE_JOINTS and warm >= 40:  # the sensors touch once the rigs have moved
        assert sensor_touching > 0


@pytest.mark.parametrize("kind,n,seed,p0", [
    (G.SCENE_PYRAMID, 20, 1, 1.0), (G.SCENE_MIXED_DROP, 500, 3, 0.0), (G.SCENE_CHAINS, 30, 2, 300.0),
    (G.SCENE_BATCH_WORLD, 777, 5, 0.0), (G.SCENE_JOINTS, 3, 9, 0.0), (G.SCENE_SLIDERS, 3, 9, 0.0),
    (G.SCENE_GEARS, 3, 9, 0.0)])
def test_host_scene_setup_vs_reference_live(ref, kind, n, seed, p0):
    """The engine's host-side set-up (facade -> shapes -> mass data -> joint defs) produces the
    reference's body, fixture and joint state byte for byte."""
    hb = _host_batch()
    w = hb.add_world(0.0, -10.0)
    hb.scene(w, kind, seed=seed, n=n, p0=p0, p1=0.6)
    rw = ob.RefWorld(ref, kind, seed=seed, n=n, p0=p0, p1=0.6)
    assert [bytes(x) for x in hb.bodies(w)] == [bytes(x) for x in rw.bodies()]
    assert [bytes(x) for x in hb.fixtures(w)] == [bytes(x) for x in rw.fixtures()]
    assert [_def_bytes(x) for x in hb.joints(w)] == [_def_bytes(x) for x in rw.joints()]
    hb.close()


def _def_bytes(joint):
    """A joint definition's bytes without its user data (the scene recipes tag no joints)."""
    raw = bytearray(bytes(joint.def_))
    off = G.JointDef.user_data.offset
    raw[off:off + 8] = bytes(8)
    return bytes(raw)


def _query_cases(bodies, rng, n_rays=300, n_boxes=120):
    """Seeded rays and boxes over the scene's extent (bodies' centres, padded)."""
    c = np.array([[b.c[0], b.c[1]] for b in bodies], dtype=np.float64)
    lo, hi = c.min(axis=0) - 3.0, c.max(axis=0) + 3.0
    rays = []
    for _ in range(n_rays):
        p1 = rng.uniform(lo, hi)
        p2 = rng.uniform(lo, hi)
        rays.append(tuple(float(np.float32(v)) for v in (*p1, *p2)))
    boxes = []
    for _ in range(n_boxes):
        a = rng.uniform(lo, hi)
        ext = rng.uniform(0.05, 4.0, size=2)
        boxes.append(tuple(float(np.float32(v)) for v in (a[0], a[1], a[0] + ext[0], a[1] + ext[1])))
    return rays, boxes


@pytest.mark.parametrize("kind,n,seed,p0", [
    (G.SCENE_PYRAMID, 20, 1, 1.0), (G.SCENE_MIXED_DROP, 400, 3, 1.0), (G.SCENE_CHAINS, 12, 2, 200.0)])
def test_oracle_queries_vs_reference_live(ref, orc, kind, n, seed, p0):
    """b2World::RayCast (closest hit) and QueryAABB of the reference after 40 steps, against the
    oracle's brute force over the same bodies: identical fixtures, points, normals, fractions."""
    rw = ob.RefWorld(ref, kind, seed=seed, n=n, p0=p0)
    rw.step(40)
    ow = ob.OracleWorld(orc, (0.0, -10.0), rw.bodies(), rw.fixtures(), rw.joints())
    rays, boxes = _query_cases(rw.bodies(), np.random.default_rng(seed))
    hits = 0
    for ray in rays:
        r, o = rw.raycast(ray), ow.raycast(ray)
        assert r == o, (ray, r, o)
        hits += r[0] >= 0
    assert hits > len(rays) // 10
    found = 0
    for box in boxes:
        r, o = rw.query_aabb(box), ow.query_aabb(box)
        assert r == o, box
        found += len(r)
    assert found > 0
    rw.close()
    ow.close()


@pytest.mark.parametrize("kind,n,seed,p0,warm,steps,vi,pi", [
    (G.SCENE_PYRAMID, 10, 1, 1.0, 85, 40, 8, 3),          # the pyramid falls asleep as one island
    (G.SCENE_CHAINS, 6, 4, 100.0, 262, 70, 10, 4),        # chains and a pile: islands fall asleep
    (G.SCENE_CHAINS, 6, 4, 100.0, 468, 15, 10, 4),        # ... and are woken (5 bodies at step 475)
    (G.SCENE_MIXED_DROP, 200, 5, 0.0, 300, 35, 8, 3),     # settled bodies fall asleep
    (G.SCENE_MIXED_DROP, 200, 5, 0.0, 466, 15, 8, 3),     # a late body wakes sleeping ones (step 473)
    (G.SCENE_BATCH_WORLD, 300, 7, 0.0, 450, 35, 8, 3),    # 144 bodies fall asleep
    (G.SCENE_BATCH_WORLD, 200, 11, 0.0, 740, 12, 8, 3),   # 83 bodies woken through their island (748)
])
def test_oracle_sleep_replay_vs_reference_live(ref, orc, kind, n, seed, p0, warm, steps, vi, pi):
    """Sleeping pinned to the reference, step by step: the reference world (sleep allowed) is
    loaded into the oracle, the oracle steps once, and the reference replays that step with its
    own narrowphase (awake rules, wakes on touching changes), its own b2Island::Solve or
    SolveOrphan per island of the oracle's partition and order (sleep timers, per-island position
    exit, SetAwake(false)) and its own broadphase (wakes of destroyed contacts). Body states, awake
    flags and sleep timers must agree bit for bit after every step."""
    rw = ob.RefWorld(ref, kind, seed=seed, n=n, p0=p0, p1=0.6, allow_sleep=True)
    rw.step(warm, vi=vi, pi=pi)
    orc.orc_set_libm_trig(1)
    asleep_seen, transitions, woken = 0, 0, 0
    try:
        prev = None
        for s in range(steps):
            ow = ob.OracleWorld(orc, (0.0, -10.0), list(rw.bodies()), list(rw.fixtures()), list(rw.joints()),
                                list(rw.contacts()), inv_dt0=60.0)
            ow.set_sleep(True)
            ow.set_sleep_times(rw.sleep_times())
            ow.step(1, 1 / 60, vi, pi)
            assert rw.replay_islands(ow.last_islands(), 1 / 60, vi, pi) == 0
            rb, obd = rw.bodies(), ow.bodies()
            for i, (x, y) in enumerate(zip(rb, obd)):
                assert bytes(x)[:40] == bytes(y)[:40] and x.flags == y.flags, f"step {s + 1} body {i}"
            assert rw.sleep_times() == ow.sleep_times(), f"step {s + 1}"
            awake = tuple(b.flags & 8 for b in rb)
            asleep_seen = max(asleep_seen, sum(1 for b in rb if b.type != 0 and not b.flags & 8))
            if prev is not None and awake != prev:
                transitions += 1
                woken += sum(1 for x, y in zip(prev, awake) if y and not x)
            prev = awake
    finally:
        orc.orc_set_libm_trig(0)
    assert asleep_seen > 0 and transitions > 0
    if warm in (468, 466, 740):
        assert woken > 0


def _random_shape(ref, rng, kind):
    s = G.Shape()
    if kind == 0:
        s.type = 0
        s.radius = float(np.float32(rng.uniform(0.05, 1.0)))
        s.vertices[0][0], s.vertices[0][1] = (float(np.float32(v)) for v in rng.uniform(-0.3, 0.3, 2))
    elif kind == 1:
        s.type = 1
        s.radius = 0.01
        a, b = rng.uniform(-1.5, 1.5, 2), rng.uniform(-1.5, 1.5, 2)
        s.vertices[0][0], s.vertices[0][1] = (float(np.float32(v)) for v in a)
        s.vertices[1][0], s.vertices[1][1] = (float(np.float32(v)) for v in b)
    else:
        n = int(rng.integers(3, 9))
        xy = rng.uniform(-1, 1, 2 * n).astype(np.float32)
        ref.ref_polygon_set(xy.ctypes.data_as(C.POINTER(C.c_float)), n, s)
    return s


def test_oracle_overlap_vs_reference_live(ref, orc):
    """b2TestOverlap (GJK b2Distance with radii) of the oracle against the reference on random
    circle / edge / polygon pairs placed from well apart to interpenetrating: identical overlap
    decisions and bit-identical distances."""
    rng = np.random.default_rng(2024)
    overlaps = 0
    for k in range(3000):
        ka, kb = int(rng.integers(0, 3)), int(rng.integers(0, 3))
        a, b = _random_shape(ref, rng, ka), _random_shape(ref, rng, kb)
        xa = (C.c_float * 4)(*[float(np.float32(v)) for v in (0.0, 0.0, 0.0, 1.0)])
        ang = rng.uniform(-3.14, 3.14)
        d = rng.uniform(0.0, 3.0)
        th = rng.uniform(-3.14, 3.14)
        xb = (C.c_float * 4)(*[float(np.float32(v)) for v in (d * np.cos(th), d * np.sin(th), np.sin(ang), np.cos(ang))])
        dr, do = C.c_float(), C.c_float()
        r = ref.ref_test_overlap(a, xa, b, xb, C.byref(dr))
        o = orc.orc_test_overlap(a, xa, b, xb, C.byref(do))
        assert (r, dr.value) == (o, do.value), (k, ka, kb)
        overlaps += r
    assert 300 < overlaps < 2700


@pytest.mark.parametrize("kind,n,seed,p0", [
    (G.SCENE_PYRAMID, 20, 1, 1.0), (G.SCENE_MIXED_DROP, 700, 3, 0.0), (G.SCENE_CHAINS, 30, 2, 300.0),
    (G.SCENE_BATCH_WORLD, 0, 0, 0.0), (G.SCENE_BATCH_WORLD, 0, 1, 0.0), (G.SCENE_BATCH_WORLD, 0, 2, 0.0),
    (G.SCENE_BATCH_WORLD, 0, 40, 0.0), (G.SCENE_BATCH_WORLD, 0, 77, 0.0)])
def test_oracle_scene_builder_matches_engine_setup(orc, kind, n, seed, p0):
    """The oracle's own scene builder (used by the CPU baseline and the reference arm, so that
    neither loads the engine library) makes the engine facade's records byte for byte: bodies
    with mass data, fixtures with hulls, revolute joints with anchors. Batch worlds take the
    workload's body count and gravity for their seed, as the benchmark does."""
    if kind == G.SCENE_BATCH_WORLD:
        n, gx, gy = orc.batch_world_params(seed)
        lib = G.Lib()
        m, hx, hy = C.c_int32(), C.c_float(), C.c_float()
        lib.b2g_batch_world_params(seed, C.byref(m), C.byref(hx), C.byref(hy))
        assert (m.value, hx.value, hy.value) == (n, gx, gy)
    hb = _host_batch()
    w = hb.add_world(0.0, -10.0)
    hb.scene(w, kind, seed=seed, n=n, p0=p0, p1=0.6)
    B, F, J = orc.scene_records(kind, seed=seed, n=n, p0=p0, p1=0.6)
    assert b"".join(bytes(b) for b in hb.bodies(w)) == b"".join(bytes(b) for b in B)
    assert b"".join(bytes(f) for f in hb.fixtures(w)) == b"".join(bytes(f) for f in F)
    assert b"".join(bytes(j) for j in hb.joints(w)) == b"".join(bytes(j) for j in J)
    hb.close()


def event_key(e, impulses=True):
    """The meaningful content of a listener event: kind, fixture pair (either orientation), the
    old manifold's point count (PreSolve), the impulse entries the solver filled (PostSolve)."""
    pc = e.point_count if e.kind == G.EVENT_POSTSOLVE else 0
    imp = ()
    if impulses and e.kind == G.EVENT_POSTSOLVE:
        imp = tuple(e.normal_impulses[:pc]) + tuple(e.tangent_impulses[:pc])
    old = e.old_manifold.point_count if e.kind == G.EVENT_PRESOLVE else 0
    return (e.kind, min(e.fixture_a, e.fixture_b), max(e.fixture_a, e.fixture_b), pc, old, imp)


@pytest.mark.parametrize("kind,n,seed,p0,warm,vi,pi", [
    (G.SCENE_PYRAMID, 20, 1, 1.0, 30, 8, 3),
    (G.SCENE_MIXED_DROP, 400, 5, 0.0, 200, 8, 3),
    (G.SCENE_CHAINS, 15, 4, 200.0, 80, 10, 4),
    (G.SCENE_JOINTS, 3, 9, 0.0, 40, 8, 3),
    (G.SCENE_SLIDERS, 3, 9, 0.0, 40, 8, 3),
])
def test_oracle_events_vs_reference_live(ref, orc, kind, n, seed, p0, warm, vi, pi):
    """Listener events, step by step: the reference's own Step (b2ContactListener callbacks from
    b2Contact::Update, b2Island::Report and b2ContactManager::Destroy, replaying the oracle's
    solver order) and the oracle's recorded events are the same set: kinds, fixture pairs, old
    manifold point counts and PostSolve impulses bit for bit."""
    rw = ob.RefWorld(ref, kind, seed=seed, n=n, p0=p0, p1=0.6)
    rw.step(warm, vi=vi, pi=pi)
    rw.events_enable(True)
    orc.orc_set_libm_trig(1)
    seen = set()
    try:
        for _ in range(4):
            ow = ob.OracleWorld(orc, (0.0, -10.0), list(rw.bodies()), list(rw.fixtures()), list(rw.joints()),
                                list(rw.contacts()), inv_dt0=60.0)
            ow.events_enable(True)
            ow.step(1, 1 / 60, vi, pi)
            pairs, jorder = ow.last_order()
            arr = (C.c_int32 * max(len(pairs), 1))(*pairs)
            jar = (C.c_int32 * max(len(jorder), 1))(*jorder)
            assert ref.ref_replay_step(rw.h, 1 / 60, vi, pi, arr, len(pairs) // 2, jar, len(jorder)) == 0
            got = sorted(event_key(e) for e in ow.events())
            exp = sorted(event_key(e) for e in rw.events())
            assert got == exp
            seen |= {k[0] for k in got}
            ow.close()
    finally:
        orc.orc_set_libm_trig(0)
    assert {G.EVENT_PRESOLVE, G.EVENT_POSTSOLVE} <= seen


@pytest.mark.parametrize("name", ["mixed", "chains"])
def test_oracle_events_vs_golden(orc, name):
    """The listener callbacks of one replayed reference step (golden) equal the oracle's events
    for the same step from the same state: kinds, pairs, point counts, impulses bit for bit."""
    g = np.load(GOLD / f"events_{name}.npz")
    bodies, fixtures = recs(G.Body, g["bodies"]), recs(G.Fixture, g["fixtures"])
    joints, contacts = recs(G.Joint, g["joints"]), recs(G.Contact, g["contacts"])
    orc.orc_set_libm_trig(1)
    try:
        ow = ob.OracleWorld(orc, (0.0, -10.0), bodies, fixtures, joints, contacts, inv_dt0=60.0)
        ow.events_enable(True)
        ow.step(1, 1 / 60, int(g["vi"]), int(g["pi"]))
        got = sorted(event_key(e) for e in ow.events())
    finally:
        orc.orc_set_libm_trig(0)
    exp = []
    for (kind, fa, fb, pc, old), imp in zip(g["ints"].tolist(), g["impulses"]):
        pc = pc if kind == G.EVENT_POSTSOLVE else 0
        im = tuple(float(x) for x in imp[:pc]) + tuple(float(x) for x in imp[2:2 + pc]) if kind == G.EVENT_POSTSOLVE else ()
        exp.append((kind, min(fa, fb), max(fa, fb), pc, old if kind == G.EVENT_PRESOLVE else 0,
                    tuple(np.float32(x) for x in im)))
    assert got == sorted(exp)
    kinds = {k[0] for k in got}
    assert {G.EVENT_BEGIN, G.EVENT_END, G.EVENT_PRESOLVE, G.EVENT_POSTSOLVE} <= kinds


@pytest.mark.parametrize("name", ["pyramid", "mixed", "chains"])
def test_oracle_rollout_measures_vs_reference_golden(orc, name):
    """256-step rollouts of the pyramid (210 boxes), a 300-body mixed drop and 10 chains over 150
    circles: the oracle (the engine's colour order) against the reference's own rollout (its own
    order), by linear and angular momentum, centre-of-mass and top height, and the deepest
    penetration every 32 steps, each within the tolerance ob.ROLLOUT_TOLERANCES states."""
    g = np.load(GOLD / f"measures_{name}.npz")
    kind, n, seed, p0 = int(g["kind"]), int(g["n"]), int(g["seed"]), float(g["p0"])
    every, vi, pi = int(g["every"]), int(g["vi"]), int(g["pi"])
    hb = _host_batch()
    w = hb.add_world(0.0, -10.0)
    hb.scene(w, kind, seed=seed, n=n, p0=p0, p1=0.6)
    fixtures = list(hb.fixtures(w))
    ow = ob.OracleWorld(orc, (0.0, -10.0), hb.bodies(w), fixtures, hb.joints(w))
    rows = []
    for _ in range(len(g["rows"])):
        ow.step(every, 1 / 60, vi, pi)
        rows.append(ob.measure_row(ob.rollout_measures(orc, list(ow.bodies()), fixtures, list(ow.contacts()))))
    ob.check_rollout_measures(name, rows, g["rows"])
    hb.close()


@pytest.mark.parametrize("kind,n,seed,p0", [
    (G.SCENE_PYRAMID, 6, 1, 1.0), (G.SCENE_MIXED_DROP, 60, 3, 0.0), (G.SCENE_CHAINS, 4, 2, 30.0),
    (G.SCENE_JOINTS, 2, 9, 0.0), (G.SCENE_SLIDERS, 2, 9, 0.0), (G.SCENE_GEARS, 2, 9, 0.0)])
def test_world_dump_text_vs_reference_live(ref, kind, n, seed, p0, tmp_path, monkeypatch):
    """b2World::Dump: the engine's text (b2g_world_dump) equals the reference's own Dump of the
    same scene line for line (bodies, fixtures with every shape type, every joint type, gears
    after the other joints)."""
    monkeypatch.chdir(tmp_path)
    rw = ob.RefWorld(ref, kind, seed=seed, n=n, p0=p0, p1=0.6)
    ref.ref_world_dump(rw.h)
    expected = (tmp_path / "box2d_dump.inl").read_text()
    hb = _host_batch()
    w = hb.add_world(0.0, -10.0)
    hb.scene(w, kind, seed=seed, n=n, p0=p0, p1=0.6)
    got = hb.dump(w)
    assert got.splitlines() == expected.splitlines()
    hb.close()
