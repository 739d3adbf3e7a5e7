"""The C ABI without a GPU: libb2g.so loads, exports every entry point include/*.h declares, the
ctypes binding declares them all, and the record layouts match the header's stated sizes."""
import ctypes as C
import re
from pathlib import Path

import pytest

import b2gpu as G

ROOT = Path(__file__).resolve().parents[1]


def _declared():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        names |= set(re.findall(r"B2G_API\s+[\w\s\*]+?\b(b2g_\w+)\s*\(", text))
    return names


def test_library_exports_every_declared_entry_point():
    names = _declared()
    assert len(names) > 40
    lib = C.CDLL(str(G.LIB_PATH))
    missing = sorted(n for n in names if not hasattr(lib, n))
    assert not missing, missing


def test_binding_declares_every_entry_point():
    assert _declared() == set(G.Lib.SYMBOLS)


def test_record_sizes_match_the_header():
    sizes = {"b2g_shape": G.Shape, "b2g_manifold_point": None, "b2g_manifold": G.Manifold, "b2g_body": G.Body,
             "b2g_ray_hit": G.RayHit}
    stated = {"b2g_shape": 152, "b2g_manifold": 64, "b2g_body": 96, "b2g_ray_hit": 24}
    for name, n in stated.items():
        assert C.sizeof(sizes[name]) == n, name
    for name, n in G.RECORD_SIZES.items():
        if sizes.get(name) is not None:
            assert C.sizeof(sizes[name]) == n, name


def test_host_only_batch_builds_and_reads_back():
    lib = G.Lib()
    b = G.Batch(lib, device=G.HOST_ONLY)
    w = b.add_world(0.0, -10.0)
    b.scene(w, G.SCENE_PYRAMID, n=5, p0=1.0, p1=0.6)
    nb, nf, nj, nc = b.sizes(w)
    assert nb == 16 and nf == 16 and nj == 0
    bodies = b.bodies(w)
    assert bodies[1].mass > 0 and bodies[0].type == 0
    b.close()


def test_bullets_scene_and_set_bullet_on_the_host():
    """The bullets scene on a host-only batch: a box and a bullet (B2G_BODY_BULLET) per lane,
    kinematic bars instead of bullets in every fourth lane with p0 = 1; b2g_body_set_bullet sets
    and clears the flag (b2Body::SetBullet) and rejects bad indices; the world's continuous flag
    reads back as set (b2World::GetContinuousPhysics)."""
    lib = G.Lib()
    b = G.Batch(lib, device=G.HOST_ONLY)
    w = b.add_world(0.0, -10.0)
    b.set_flags(w, continuous=True)
    b.scene(w, G.SCENE_BULLETS, seed=4, n=8, p0=1.0, p1=0.6)
    bodies = b.bodies(w)
    assert len(bodies) == 1 + 2 * 8
    bullets = [i for i, r in enumerate(bodies) if r.flags & G.BODY_BULLET]
    kinematic = [i for i, r in enumerate(bodies) if r.type == 1]
    assert len(bullets) == 6 and len(kinematic) == 2
    b.set_bullet(w, bullets[0], False)
    b.set_bullet(w, 1, True)
    now = b.bodies(w)
    assert not now[bullets[0]].flags & G.BODY_BULLET and now[1].flags & G.BODY_BULLET
    assert lib.lib.b2g_body_set_bullet(b.h, w, len(bodies), 1) == 1  # B2G_E_INVALID_ARG
    flags = [C.c_int32() for _ in range(4)]
    assert lib.lib.b2g_world_get_flags(b.h, w, *[C.byref(x) for x in flags]) == 0
    assert flags[2].value == 1
    b.close()


def test_snapshot_round_trip_on_the_host():
    """A world's snapshot restores into an equal world (host-only batch: no device involved),
    and malformed blobs are rejected with INVALID_ARG."""
    lib = G.Lib()
    b = G.Batch(lib, device=G.HOST_ONLY)
    w = b.add_world(0.5, -9.0)
    b.scene(w, G.SCENE_CHAINS, seed=3, n=6, p0=40.0, p1=0.6)
    blob = b.snapshot(w)
    w2 = b.restore(blob)
    assert b.sizes(w2) == b.sizes(w)
    assert [bytes(x) for x in b.bodies(w2)] == [bytes(x) for x in b.bodies(w)]
    assert [bytes(x) for x in b.joints(w2)] == [bytes(x) for x in b.joints(w)]
    assert b.snapshot(w2) == blob
    bad = bytearray(blob)
    bad[0] ^= 0xFF
    st = lib.lib.b2g_world_restore(b.h, C.create_string_buffer(bytes(bad), len(bad)), len(bad), None)
    assert st == 1
    st = lib.lib.b2g_world_restore(b.h, C.create_string_buffer(blob[:-8], len(blob) - 8), len(blob) - 8, None)
    assert st == 1
    b.close()


def test_server_cancels_queued_requests_without_a_device():
    """Queued requests cancel on the host: they finish with CANCELLED and zero steps; unknown or
    already finished ids are INVALID_ARG."""
    lib = G.Lib()
    srv = G.Server(lib, device=G.HOST_ONLY, budget_bytes=1 << 30, max_worlds=4)
    a = srv.submit(1, 100, 10)
    b = srv.submit(2, 100, 10)
    assert srv.cancel(b) == 0
    assert srv.cancel(b) == 1
    assert srv.cancel(12345) == 1
    res = srv.poll()
    assert [(r.request_id, r.status, r.steps) for r in res] == [(b, 8, 0)]
    assert srv.stats()["queued"] == 1
    assert srv.cancel(a) == 0
    assert srv.stats()["queued"] == 0
    srv.close()


def test_builder_threads_build_admitted_worlds_on_the_host():
    """Admission builds worlds on builder threads (each on a host-only batch) and moves them into
    the served batch; with no device the tick then fails at the step, after admission."""
    lib = G.Lib()
    for builders in (0, 3):
        srv = G.Server(lib, device=G.HOST_ONLY, budget_bytes=1 << 30, max_worlds=8, builders=builders)
        ids = [srv.submit(10 + i, 50 + 30 * i, 5) for i in range(4)]
        with pytest.raises(G.B2GError):
            srv.tick()
        st = srv.stats()
        assert st["queued"] == 0 and st["active"] == 4
        bh = C.c_void_p()
        lib.check(lib.b2g_server_batch(srv.h, C.byref(bh)), "server_batch")
        n = C.c_int32()
        lib.check(lib.b2g_world_count(bh, C.byref(n)), "world_count")
        assert n.value == 4
        assert srv.cancel(ids[1]) == 0
        assert srv.stats()["active"] == 3
        srv.close()


def test_tuning_knobs_and_split_step_on_a_host_only_batch():
    lib = G.Lib()
    b = G.Batch(lib, device=G.HOST_ONLY)
    assert lib.b2g_batch_set_tree_rebuild_period(b.h, 0) == 1   # INVALID_ARG
    assert lib.b2g_batch_set_tree_rebuild_period(b.h, 4) == 0
    assert lib.b2g_batch_set_solver_waves(b.h, -1.0) == 1
    assert lib.b2g_batch_set_solver_waves(b.h, 0.0) == 0
    assert b.step_done()             # nothing in flight
    b.stage()                        # no device: nothing to pack
    assert lib.b2g_step_end(b.h) == 1  # no step in flight
    b.close()


def test_removal_renumbers_host_records():
    """b2g_bodies_remove / b2g_fixtures_remove / b2g_joints_remove on a world not yet on a device:
    a removed body takes its fixtures and joints along, the rest keep their creation order and
    are renumbered (fixture bodies and joint bodies follow), a removed fixture resets its body's
    mass data, and out-of-range indices are refused."""
    lib = G.Lib()
    b = G.Batch(lib, device=G.HOST_ONLY)
    w = b.add_world(0.0, -10.0)
    b.scene(w, G.SCENE_CHAINS, seed=2, n=3, p0=10, p1=0.6)
    bodies, fixtures, joints = b.bodies(w), b.fixtures(w), b.joints(w)
    nb, nf, nj = len(bodies), len(fixtures), len(joints)
    # a chain link: body with one joint to its predecessor and one to its successor
    link = joints[5].def_.body_b
    attached = [j for j in range(nj) if link in (joints[j].def_.body_a, joints[j].def_.body_b)]
    assert len(attached) == 2
    assert b.remove(w, bodies=[link]) == []
    nb2, nf2, nj2, _ = b.sizes(w)
    assert (nb2, nf2, nj2) == (nb - 1, nf - 1, nj - 2)
    shift = lambda i: i - 1 if i > link else i  # noqa: E731
    kept = [j for j in range(nj) if j not in attached]
    after = b.joints(w)
    for k, j in enumerate(kept):
        assert (after[k].def_.body_a, after[k].def_.body_b) == (shift(joints[j].def_.body_a), shift(joints[j].def_.body_b))
    after_f = b.fixtures(w)
    assert [f.body for f in after_f] == [shift(f.body) for f in fixtures if f.body != link]
    assert bytes(b.bodies(w)[link]) == bytes(bodies[link + 1])
    # a second fixture on a body, then its removal restores the one-fixture mass data
    one = b.bodies(w)[1]  # the first pile circle (body 0 is the container)
    fd = G.FixtureDef()
    fd.body = 1
    fd.shape_type = 0
    fd.radius = 0.5
    fd.density = 3.0
    fd.friction = 0.2
    fid = C.c_int32()
    lib.check(lib.b2g_fixtures_add(b.h, w, C.byref(fd), 1, C.byref(fid)), "b2g_fixtures_add")
    assert b.bodies(w)[1].mass > one.mass
    b.remove(w, fixtures=[fid.value])
    assert bytes(b.bodies(w)[1]) == bytes(one)
    bad = (C.c_int32 * 1)(10 ** 6)
    assert lib.b2g_joints_remove(b.h, w, bad, 1) == 1  # INVALID_ARG
    b.close()
