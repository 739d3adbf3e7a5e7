"""World queries on the GPU against the oracle: b2World::RayCast with a closest-hit callback and
b2World::QueryAABB, batched over several worlds, bit for bit (fixture, point, normal, fraction;
ascending fixture sets). The oracle's queries are pinned to the reference's own in
test_oracle_pins.py."""
import ctypes as C

import numpy as np
import pytest

import b2gpu as G
import oracle_bind as ob

pytestmark = pytest.mark.gpu


def _params(lib, seed):
    n, gx, gy = C.c_int32(), C.c_float(), C.c_float()
    lib.b2g_batch_world_params(seed, C.byref(n), C.byref(gx), C.byref(gy))
    return n.value, gx.value, gy.value


def _cases(bodies, rng, n_rays, n_boxes):
    c = np.array([[b.c[0], b.c[1]] for b in bodies], dtype=np.float64)
    lo, hi = c.min(axis=0) - 3.0, c.max(axis=0) + 3.0
    rays = [tuple(float(np.float32(v)) for v in (*rng.uniform(lo, hi), *rng.uniform(lo, hi))) for _ in range(n_rays)]
    boxes = []
    for _ in range(n_boxes):
        a = rng.uniform(lo, hi)
        e = rng.uniform(0.05, 4.0, size=2)
        boxes.append(tuple(float(np.float32(v)) for v in (a[0], a[1], a[0] + e[0], a[1] + e[1])))
    return rays, boxes


def _check(lib, orc, batch, worlds, rng, n_rays=200, n_boxes=60):
    qw, rays, qb, boxes, expect_r, expect_b = [], [], [], [], [], []
    for w in worlds:
        ow = ob.OracleWorld(orc, (0.0, -10.0), batch.bodies(w), batch.fixtures(w))
        r, bx = _cases(batch.bodies(w), rng, n_rays, n_boxes)
        qw += [w] * len(r)
        rays += r
        expect_r += [ow.raycast(x) for x in r]
        qb += [w] * len(bx)
        boxes += bx
        expect_b += [ow.query_aabb(x) for x in bx]
        ow.close()
    # interleave the worlds so that one launch serves them all
    perm = rng.permutation(len(rays))
    got = batch.raycast([qw[i] for i in perm], [rays[i] for i in perm])
    for k, i in enumerate(perm):
        assert got[k] == expect_r[i], (qw[i], rays[i], got[k], expect_r[i])
    permb = rng.permutation(len(boxes))
    gotb = batch.query_aabb([qb[i] for i in permb], [boxes[i] for i in permb])
    for k, i in enumerate(permb):
        assert gotb[k] == expect_b[i], (qb[i], boxes[i])
    return sum(1 for h in got if h[0] >= 0), sum(len(x) for x in gotb)


def test_queries_match_oracle(lib, orc):
    b = G.Batch(lib, device=0)
    ws = []
    for s, n in ((51, 300), (52, 1200), (53, 40), (54, 2500)):
        _, gx, gy = _params(lib, s)
        w = b.add_world(gx, gy)
        b.set_flags(w)
        b.scene(w, G.SCENE_BATCH_WORLD, seed=s, n=n)
        ws.append(w)
    # a world of one fixture: the reference reports it for any query box
    lone = b.add_world(0.0, -10.0)
    b.set_flags(lone)
    b.scene(lone, G.SCENE_PYRAMID, n=0, p0=1.0, p1=0.6)
    for _ in range(40):
        b.step(1 / 60, 8, 3)
    rng = np.random.default_rng(7)
    hits, found = _check(lib, orc, b, ws + [lone], rng)
    assert hits > 100 and found > 50
    assert b.query_aabb([lone], [(1e6, 1e6, 1e6 + 1, 1e6 + 1)]) == [list(range(b.sizes(lone)[1]))] or b.sizes(lone)[1] != 1
    b.close()


def test_queries_after_appending_and_compacting(lib, orc):
    """Trees are rebuilt for queries when the layout changed since the last broadphase."""
    b = G.Batch(lib, device=0)
    ws = []
    for s, n in ((61, 500), (62, 900), (63, 200)):
        _, gx, gy = _params(lib, s)
        w = b.add_world(gx, gy)
        b.set_flags(w)
        b.scene(w, G.SCENE_BATCH_WORLD, seed=s, n=n)
        ws.append(w)
    for _ in range(20):
        b.step(1 / 60, 8, 3)
    rng = np.random.default_rng(11)
    # a world appended after the last step: queried before it is ever stepped
    _, gx, gy = _params(lib, 64)
    late = b.add_world(gx, gy)
    b.set_flags(late)
    b.scene(late, G.SCENE_BATCH_WORLD, seed=64, n=700)
    _check(lib, orc, b, ws + [late], rng, 120, 40)
    lib.check(lib.b2g_world_retire(b.h, ws[1]), "retire")
    nmap = (C.c_int32 * 4)()
    lib.check(lib.b2g_compact(b.h, nmap, 4), "compact")
    _check(lib, orc, b, [0, 1, 2], rng, 120, 40)
    for _ in range(5):
        b.step(1 / 60, 8, 3)
    _check(lib, orc, b, [0, 1, 2], rng, 120, 40)
    b.close()
