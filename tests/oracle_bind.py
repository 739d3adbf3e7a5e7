"""ctypes bindings of the oracle libraries (test infrastructure only).

* ``Ref``    - oracle/_ref/libb2ref.so: the reference engine compiled from its own sources plus
               oracle/ref_shim.cpp. It exists only where the reference sources are checked out.
* ``Oracle`` - oracle/_build/libb2oracle.so: the CPU restatement of the Step path that the GPU
               engine is checked against everywhere (it is built from the repository alone).
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "box2d-optimized_gb300"))
import b2gpu as G  # noqa: E402

REF_PATH = ROOT / "oracle" / "_ref" / "libb2ref.so"
ORACLE_PATH = ROOT / "oracle" / "_build" / "libb2oracle.so"

P = C.POINTER
vp, i32, u32, f32 = C.c_void_p, C.c_int32, C.c_uint32, C.c_float


class Ref:
    def __init__(self, path=REF_PATH):
        self.lib = L = C.CDLL(str(path))
        sig = {
            "ref_polygon_set": ([P(f32), i32, P(G.Shape)], C.c_int),
            "ref_polygon_box": ([f32, f32, f32, f32, f32, i32, P(G.Shape)], C.c_int),
            "ref_shape_mass": ([P(G.Shape), f32, P(f32)], C.c_int),
            "ref_shape_aabb": ([P(G.Shape), P(f32), P(f32)], C.c_int),
            "ref_collide": ([P(G.Shape), P(f32), P(G.Shape), P(f32), P(G.Manifold)], C.c_int),
            "ref_test_overlap": ([P(G.Shape), P(f32), P(G.Shape), P(f32), P(f32)], C.c_int),
            "ref_time_of_impact": ([P(G.TOIInput), i32, P(G.TOIOutput)], None),
            "ref_world_manifold": ([P(G.Manifold), P(f32), f32, P(f32), f32, P(f32)], C.c_int),
            "ref_scene_world": ([i32, u32, i32, f32, f32, f32, f32, P(i32)], vp),
            "ref_world_free": ([vp], None),
            "ref_world_set_flags": ([vp, i32, i32, i32], None),
            "ref_world_step": ([vp, f32, i32, i32, i32], C.c_double),
            "ref_world_sizes": ([vp, P(i32)], i32),
            "ref_world_bodies": ([vp, P(G.Body)], None),
            "ref_world_fixtures": ([vp, P(G.Fixture)], None),
            "ref_world_joints": ([vp, P(G.Joint)], None),
            "ref_world_contacts": ([vp, P(G.Contact), i32], i32),
            "ref_world_raycast": ([vp, P(f32), P(f32)], i32),
            "ref_world_query_aabb": ([vp, P(f32), P(i32), i32], i32),
            "ref_world_set_bodies": ([vp, P(G.Body)], None),
            "ref_replay_step": ([vp, f32, i32, i32, P(i32), i32, P(i32), i32], C.c_int),
            "ref_replay_step_islands": ([vp, f32, i32, i32, i32, P(i32), P(i32), P(i32), P(i32), P(i32), P(i32),
                                         P(i32)], C.c_int),
            "ref_world_sleep_times": ([vp, P(f32)], None),
            "ref_worlds_step_parallel": ([P(vp), i32, f32, i32, i32, i32, i32], C.c_double),
            "ref_world_events_enable": ([vp, i32], None),
            "ref_world_events": ([vp, P(G.Event), i32], i32),
            "ref_world_dump": ([vp], None),
        }
        for name, (a, r) in sig.items():
            fn = getattr(L, name)
            fn.argtypes = a
            fn.restype = r

    def __getattr__(self, name):
        return getattr(self.lib, name)


def _raycast(fn, h, ray):
    r = (f32 * 4)(*ray)
    o = (f32 * 5)()
    f = fn(h, r, o)
    return (f, tuple(o[:2]), tuple(o[2:4]), o[4]) if f >= 0 else (-1, None, None, None)


def _query(fn, h, box, cap=4096):
    b = (f32 * 4)(*box)
    out = (i32 * cap)()
    n = fn(h, b, out, cap)
    assert n <= cap
    return list(out[:n])


class RefWorld:
    """A reference b2World built by one of the shared scene recipes."""

    def __init__(self, ref: Ref, kind, seed=1, n=20, p0=1.0, p1=0.6, gravity=(0.0, -10.0),
                 allow_sleep=False, warm=True, continuous=False):
        self.ref = ref
        counts = (i32 * 3)()
        self.h = ref.ref_scene_world(kind, seed, n, p0, p1, gravity[0], gravity[1], counts)
        self.counts = tuple(counts)
        ref.ref_world_set_flags(self.h, int(allow_sleep), int(warm), int(continuous))
        self._raycast_fn, self._query_fn = ref.ref_world_raycast, ref.ref_world_query_aabb

    def close(self):
        if self.h:
            self.ref.ref_world_free(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def sizes(self):
        s = (i32 * 4)()
        self.ref.ref_world_sizes(self.h, s)
        return tuple(s)

    def step(self, n=1, dt=1 / 60, vi=8, pi=3):
        return self.ref.ref_world_step(self.h, dt, vi, pi, n)

    def bodies(self):
        nb = self.sizes()[0]
        arr = (G.Body * nb)()
        self.ref.ref_world_bodies(self.h, arr)
        return arr

    def fixtures(self):
        nf = self.sizes()[1]
        arr = (G.Fixture * nf)()
        self.ref.ref_world_fixtures(self.h, arr)
        return arr

    def joints(self):
        nj = self.sizes()[2]
        arr = (G.Joint * max(nj, 1))()
        self.ref.ref_world_joints(self.h, arr)
        return arr[:nj]

    def raycast(self, ray):
        """Closest hit (fixture, point, normal, fraction) of the segment ray = (x1, y1, x2, y2)."""
        return _raycast(self._raycast_fn, self.h, ray)

    def query_aabb(self, box):
        return _query(self._query_fn, self.h, box)

    def sleep_times(self):
        nb = self.sizes()[0]
        arr = (f32 * max(nb, 1))()
        self.ref.ref_world_sleep_times(self.h, arr)
        return list(arr[:nb])

    def events_enable(self, on=True):
        self.ref.ref_world_events_enable(self.h, int(on))

    def events(self):
        """Listener callbacks since the last call, sorted by (kind, fixture A, fixture B)."""
        n = self.ref.ref_world_events(self.h, None, 0)
        arr = (G.Event * max(n, 1))()
        self.ref.ref_world_events(self.h, arr, n)
        return arr[:n]

    def replay_islands(self, islands, dt=1 / 60, vi=8, pi=3):
        """One Step with the reference's island solver over the oracle's islands (last_islands)."""
        root, orphan, boff, coff, joff, bodies, pairs, joints = islands
        arr = lambda v: (i32 * max(len(v), 1))(*v)  # noqa: E731
        return self.ref.ref_replay_step_islands(self.h, dt, vi, pi, len(root), arr(orphan), arr(boff), arr(coff),
                                                arr(joff), arr(bodies), arr(pairs), arr(joints))

    def contacts(self):
        n = self.ref.ref_world_contacts(self.h, None, 0)
        arr = (G.Contact * max(n, 1))()
        self.ref.ref_world_contacts(self.h, arr, n)
        return arr[:n]


class Oracle:
    def __init__(self, path=ORACLE_PATH):
        self.lib = L = C.CDLL(str(path))
        sig = {
            "orc_polygon_set": ([P(f32), i32, P(G.Shape)], C.c_int),
            "orc_polygon_box": ([f32, f32, f32, f32, f32, i32, P(G.Shape)], C.c_int),
            "orc_shape_mass": ([P(G.Shape), f32, P(f32)], C.c_int),
            "orc_shape_aabb": ([P(G.Shape), P(f32), P(f32)], C.c_int),
            "orc_collide": ([P(G.Shape), P(f32), P(G.Shape), P(f32), P(G.Manifold)], C.c_int),
            "orc_test_overlap": ([P(G.Shape), P(f32), P(G.Shape), P(f32), P(f32)], C.c_int),
            "orc_time_of_impact": ([P(G.TOIInput), i32, P(G.TOIOutput)], None),
            "orc_world_manifold": ([P(G.Manifold), P(f32), f32, P(f32), f32, P(f32)], C.c_int),
            "orc_sincos": ([f32, P(f32), P(f32)], None),
            "orc_world_new": ([f32, f32], vp),
            "orc_world_free": ([vp], None),
            "orc_world_load": ([vp, P(G.Body), i32, P(G.Fixture), i32, P(G.Joint), i32,
                                P(G.Contact), i32, f32], C.c_int),
            "orc_world_step": ([vp, f32, i32, i32, i32], C.c_double),
            "orc_world_sizes": ([vp, P(i32)], i32),
            "orc_world_bodies": ([vp, P(G.Body)], None),
            "orc_world_joints": ([vp, P(G.Joint)], None),
            "orc_world_contacts": ([vp, P(G.Contact), i32], i32),
            "orc_world_solver_order": ([vp, P(i32), P(u32), i32, P(i32), P(u32), i32], C.c_int),
            "orc_world_last_order": ([vp, P(i32), i32, P(i32), i32, P(i32)], i32),
            "orc_world_raycast": ([vp, P(f32), P(f32)], i32),
            "orc_world_query_aabb": ([vp, P(f32), P(i32), i32], i32),
            "orc_world_set_sleep": ([vp, i32], None),
            "orc_world_set_continuous": ([vp, i32], None),
            "orc_world_flag_new_contacts": ([vp], None),
            "orc_world_sleep_times": ([vp, P(f32)], None),
            "orc_world_set_sleep_times": ([vp, P(f32)], None),
            "orc_world_last_islands": ([vp, P(i32), P(i32), P(i32), P(i32), P(i32), P(i32), P(i32), P(i32),
                                        P(i32)], None),
            "orc_set_libm_trig": ([i32], None),
            "orc_pairs": ([P(f32), i32, P(C.c_uint64), C.c_int64], C.c_int64),
            "orc_worlds_step_parallel": ([P(vp), i32, f32, i32, i32, i32, i32], C.c_double),
            "orc_scene_world": ([i32, u32, i32, f32, f32, f32, f32, P(i32)], vp),
            "orc_scene_records": ([i32, u32, i32, f32, f32, P(i32), P(G.Body), i32, P(G.Fixture), i32,
                                   P(G.Joint), i32], i32),
            "orc_batch_world_params": ([u32, P(i32), P(f32), P(f32)], C.c_int),
            "orc_world_events_enable": ([vp, i32], None),
            "orc_world_events": ([vp, P(G.Event), i32], i32),
        }
        for name, (a, r) in sig.items():
            fn = getattr(L, name)
            fn.argtypes = a
            fn.restype = r

    def __getattr__(self, name):
        return getattr(self.lib, name)

    def batch_world_params(self, seed):
        """(bodies, gx, gy) of world `seed` of the batched workload."""
        n, gx, gy = i32(), f32(), f32()
        self.lib.orc_batch_world_params(seed, C.byref(n), C.byref(gx), C.byref(gy))
        return n.value, gx.value, gy.value

    def scene_records(self, kind, seed=1, n=20, p0=1.0, p1=0.6):
        """(bodies, fixtures, joints) records the oracle's scene builder makes for a recipe."""
        sz = (i32 * 3)()
        self.lib.orc_scene_records(kind, seed, n, p0, p1, sz, None, 0, None, 0, None, 0)
        B, F, J = (G.Body * max(sz[0], 1))(), (G.Fixture * max(sz[1], 1))(), (G.Joint * max(sz[2], 1))()
        self.lib.orc_scene_records(kind, seed, n, p0, p1, sz, B, sz[0], F, sz[1], J, sz[2])
        return B[:sz[0]], F[:sz[1]], J[:sz[2]]


class OracleWorld:
    """A world of the CPU restatement loaded from exported records (or, with `scene`, built by
    the oracle's own scene builder: scene = (kind, seed, n, p0, p1))."""

    def __init__(self, orc: Oracle, gravity, bodies=(), fixtures=(), joints=(), contacts=(),
                 inv_dt0=0.0, scene=None, continuous=False):
        self.orc = orc
        self._continuous = continuous
        self._raycast_fn, self._query_fn = orc.orc_world_raycast, orc.orc_world_query_aabb
        if scene is not None:
            kind, seed, n, p0, p1 = scene
            counts = (i32 * 3)()
            self.h = orc.orc_scene_world(kind, seed, n, p0, p1, gravity[0], gravity[1], counts)
            if not self.h:
                raise RuntimeError(f"orc_scene_world: unknown scene kind {kind}")
            self.counts = tuple(counts)
            orc.orc_world_set_continuous(self.h, int(continuous))
            return
        self.h = orc.orc_world_new(gravity[0], gravity[1])
        nb, nf, nj, nc = len(bodies), len(fixtures), len(joints), len(contacts)
        B = (G.Body * max(nb, 1))(*bodies)
        F = (G.Fixture * max(nf, 1))(*fixtures)
        J = (G.Joint * max(nj, 1))(*joints)
        Cc = (G.Contact * max(nc, 1))(*contacts)
        st = orc.orc_world_load(self.h, B, nb, F, nf, J, nj, Cc, nc, inv_dt0)
        if st != 0:
            raise RuntimeError(f"orc_world_load failed: {st}")
        orc.orc_world_set_continuous(self.h, int(continuous))
        self._raycast_fn, self._query_fn = orc.orc_world_raycast, orc.orc_world_query_aabb

    def close(self):
        if self.h:
            self.orc.orc_world_free(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def sizes(self):
        s = (i32 * 4)()
        self.orc.orc_world_sizes(self.h, s)
        return tuple(s)

    def step(self, n=1, dt=1 / 60, vi=8, pi=3, new_contacts=False):
        return self.orc.orc_world_step(self.h, dt, vi, pi, n)

    def bodies(self):
        nb = self.sizes()[0]
        arr = (G.Body * max(nb, 1))()
        self.orc.orc_world_bodies(self.h, arr)
        return arr[:nb]

    def joints(self):
        nj = self.sizes()[2]
        arr = (G.Joint * max(nj, 1))()
        self.orc.orc_world_joints(self.h, arr)
        return arr[:nj]

    def raycast(self, ray):
        """Closest hit (fixture, point, normal, fraction) of the segment ray = (x1, y1, x2, y2)."""
        return _raycast(self._raycast_fn, self.h, ray)

    def query_aabb(self, box):
        return _query(self._query_fn, self.h, box)

    def contacts(self):
        n = self.orc.orc_world_contacts(self.h, None, 0)
        arr = (G.Contact * max(n, 1))()
        self.orc.orc_world_contacts(self.h, arr, n)
        return arr[:n]

    def set_sleep(self, allow):
        self.orc.orc_world_set_sleep(self.h, int(allow))

    def events_enable(self, on=True):
        self.orc.orc_world_events_enable(self.h, int(on))

    def events(self):
        """Listener events of the steps since the last call, sorted like the engine's delivery."""
        n = self.orc.orc_world_events(self.h, None, 0)
        arr = (G.Event * max(n, 1))()
        self.orc.orc_world_events(self.h, arr, n)
        return arr[:n]

    def sleep_times(self):
        nb = self.sizes()[0]
        arr = (f32 * max(nb, 1))()
        self.orc.orc_world_sleep_times(self.h, arr)
        return list(arr[:nb])

    def set_sleep_times(self, times):
        self.orc.orc_world_set_sleep_times(self.h, (f32 * max(len(times), 1))(*times))

    def last_islands(self):
        """The last step's islands: (roots, orphan flags, body offsets, contact offsets, joint
        offsets, bodies, contact fixture pairs, joints)."""
        cnt = (i32 * 4)()
        self.orc.orc_world_last_islands(self.h, cnt, *([None] * 8))
        ni, nb, nc, nj = cnt
        bufs = [(i32 * max(k, 1))() for k in (ni, ni, ni + 1, ni + 1, ni + 1, nb, 2 * nc, nj)]
        self.orc.orc_world_last_islands(self.h, cnt, *bufs)
        sizes = (ni, ni, ni + 1, ni + 1, ni + 1, nb, 2 * nc, nj)
        return tuple(list(b[:k]) for b, k in zip(bufs, sizes))

    def last_order(self):
        nj = C.c_int32()
        nc = self.orc.orc_world_last_order(self.h, None, 0, None, 0, C.byref(nj))
        pairs = (i32 * max(2 * nc, 1))()
        joints = (i32 * max(nj.value, 1))()
        self.orc.orc_world_last_order(self.h, pairs, nc, joints, nj.value, C.byref(nj))
        return list(pairs[:2 * nc]), list(joints[:nj.value])

    def solver_order(self):
        nc = self.sizes()[3]
        nj = self.sizes()[2]
        cc = (i32 * max(nc, 1))()
        cp = (u32 * max(nc, 1))()
        jc = (i32 * max(nj, 1))()
        jp = (u32 * max(nj, 1))()
        self.orc.orc_world_solver_order(self.h, cc, cp, nc, jc, jp, nj)
        return list(cc[:nc]), list(cp[:nc]), list(jc[:nj]), list(jp[:nj])


def rollout_measures(orc, bodies, fixtures, contacts):
    """Physical measures of a world state, for judging rollouts whose Gauss-Seidel orders differ:
    linear momentum per unit mass (m/s, 2-vector), angular momentum about the origin per unit mass
    (m^2/s), height of the centre of mass and of the highest body centre (m) over the dynamic
    bodies, and the deepest penetration (m): minus the smallest world-manifold separation over the
    touching contacts (b2WorldManifold::Initialize, src/collision/b2_collision.cpp:26-90),
    0 when nothing overlaps."""
    import numpy as np  # noqa: PLC0415

    b = G.body_array_to_numpy((G.Body * len(bodies))(*bodies))
    dyn = b["type"] == G.DYNAMIC
    m = b["mass"][dyn].astype(np.float64)
    v = b["v"][dyn].astype(np.float64)
    c = b["c"][dyn].astype(np.float64)
    w = b["w"][dyn].astype(np.float64)
    inertia = b["inertia"][dyn].astype(np.float64)
    total = m.sum()
    lin = (m[:, None] * v).sum(axis=0) / total
    ang = (inertia * w + m * (c[:, 0] * v[:, 1] - c[:, 1] * v[:, 0])).sum() / total
    pen = 0.0
    out = (f32 * 8)()
    for ct in contacts:
        if not ct.flags & 2 or ct.manifold.point_count == 0:
            continue
        fa, fb = fixtures[ct.fixture_a], fixtures[ct.fixture_b]
        xa = (f32 * 4)(*bodies[fa.body].xf)
        xb = (f32 * 4)(*bodies[fb.body].xf)
        orc.orc_world_manifold(ct.manifold, xa, fa.shape.radius, xb, fb.shape.radius, out)
        for j in range(ct.manifold.point_count):
            pen = max(pen, -out[6 + j])
    return {"linear": lin, "angular": ang, "com_height": float((m * c[:, 1]).sum() / total),
            "top_height": float(c[:, 1].max()), "penetration": pen}


# Tolerances of a rollout judged against the reference's own rollout by physical measures (the
# two differ in Gauss-Seidel order, so states agree to rounding at first and then diverge within
# the physics): per measure, the largest difference allowed at any checkpoint (every 32 steps),
# and the largest penetration either may show. Units: m/s, m^2/s, m, m, m.
ROLLOUT_TOLERANCES = {
    # 210 boxes settling into a stack: everything close
    "pyramid": {"linear": 0.05, "angular": 0.3, "com_height": 0.01, "top_height": 0.02, "penetration": 0.01,
                "max_penetration": 0.06},
    # 300 mixed shapes landing in a U: chaotic while they land, settled by step 256
    "mixed": {"linear": 0.75, "angular": 4.0, "com_height": 0.15, "top_height": 0.6, "penetration": 0.15,
              "max_penetration": 0.35},
    # 10 swinging chains over 150 circles: the chains' swing is chaotic
    "chains": {"linear": 0.5, "angular": 5.0, "com_height": 0.1, "top_height": 0.1, "penetration": 0.05,
               "max_penetration": 0.15},
}


def measure_row(m):
    return [m["linear"][0], m["linear"][1], m["angular"], m["com_height"], m["top_height"], m["penetration"]]


def check_rollout_measures(name, rows, golden_rows):
    """Asserts that measure rows (one per checkpoint, as measure_row) stay within the scene's
    tolerances of the reference's rows."""
    import numpy as np  # noqa: PLC0415

    tol = ROLLOUT_TOLERANCES[name]
    got, exp = np.asarray(rows, np.float64), np.asarray(golden_rows, np.float64)
    assert got.shape == exp.shape
    lin = np.hypot(got[:, 0] - exp[:, 0], got[:, 1] - exp[:, 1])
    checks = {"linear": lin, "angular": np.abs(got[:, 2] - exp[:, 2]), "com_height": np.abs(got[:, 3] - exp[:, 3]),
              "top_height": np.abs(got[:, 4] - exp[:, 4]), "penetration": np.abs(got[:, 5] - exp[:, 5])}
    for k, d in checks.items():
        assert d.max() <= tol[k], f"{name}: {k} differs by {d.max():.4f} (> {tol[k]}) at checkpoint {int(d.argmax())}"
    assert got[:, 5].max() <= tol["max_penetration"] and exp[:, 5].max() <= tol["max_penetration"]
