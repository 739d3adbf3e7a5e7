"""GPU parity: the CUDA engine (through the C ABI) against the CPU oracle, bit for bit.

The oracle restates the reference's arithmetic in the engine's canonical order (contacts sorted
by fixture pair, colour-ordered Gauss-Seidel, per-world position early exit, portable sin/cos),
so on identical inputs every float of the body state must match exactly. Integer outputs
(pair sets, manifold point counts, feature ids) are compared exactly as well.
"""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

import b2gpu as G
import oracle_bind as ob

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _dev_bytes(buf: bytes):
    t = torch.frombuffer(bytearray(buf), dtype=torch.uint8).cuda()
    return t


def _state_bytes(records):
    # xf, c, a, v, w: the first 40 bytes of each b2g_body
    return b"".join(bytes(r)[:40] for r in records)


def _first_diff(g, o):
    gn = G.body_array_to_numpy((G.Body * len(g))(*g))
    on = G.body_array_to_numpy((G.Body * len(o))(*o))
    for k in ("xf", "c", "a", "v", "w"):
        d = np.abs(gn[k].astype(np.float64) - on[k].astype(np.float64))
        if d.max() > 0:
            i = int(np.argmax(d.reshape(len(g), -1).max(axis=1)))
            return f"{k} body {i}: gpu {gn[k][i]} oracle {on[k][i]}"
    return "no difference"


def _contact_key(c):
    """The meaningful content of a contact record: slots beyond point_count (and the local
    normal/point of an empty manifold) are left over from earlier steps and never read."""
    m = c.manifold
    pts = tuple((m.points[j].local_point[0], m.points[j].local_point[1], m.points[j].normal_impulse,
                 m.points[j].tangent_impulse, m.points[j].id) for j in range(m.point_count))
    geo = (m.type, tuple(m.local_normal), tuple(m.local_point)) if m.point_count else ()
    return (c.fixture_a, c.fixture_b, c.flags, c.friction, c.restitution, c.restitution_threshold,
            c.tangent_speed, m.point_count, geo, pts)


def _rollout(lib, orc, kind, n, seed=1, p0=1.0, p1=0.6, steps=60, vi=8, pi=3, gravity=(0.0, -10.0),
             continuous=False):
    batch = G.Batch(lib, device=0)
    w = batch.add_world(*gravity)
    batch.set_flags(w, allow_sleep=False, warm_starting=True, continuous=continuous)
    batch.scene(w, kind, seed=seed, n=n, p0=p0, p1=p1)
    ow = ob.OracleWorld(orc, gravity, batch.bodies(w), batch.fixtures(w), batch.joints(w), continuous=continuous)
    for s in range(steps):
        batch.step(1 / 60, vi, pi)
        ow.step(1, 1 / 60, vi, pi)
        g, o = batch.bodies(w), ow.bodies()
        assert _state_bytes(g) == _state_bytes(o), f"step {s + 1}: {_first_diff(g, o)}"
    gc = batch.contacts(w)
    oc = ow.contacts()
    assert len(gc) == len(oc)
    assert [_contact_key(x) for x in gc] == [_contact_key(y) for y in oc], "contact lists differ"
    gj, oj = batch.joints(w), ow.joints()
    for x, y in zip(gj, oj):
        assert list(x.impulse) == list(y.impulse)
        assert (x.motor_impulse, x.lower_impulse, x.upper_impulse) == (y.motor_impulse, y.lower_impulse, y.upper_impulse)
    batch.close()
    return len(gc)


def test_pyramid_rollout_bit_exact(lib, orc):
    # the 20-row pyramid configuration (210 boxes, density 1, friction 0.6), 8/3 iterations,
    # its full 256 steps
    nc = _rollout(lib, orc, G.SCENE_PYRAMID, 20, steps=256)
    assert nc > 300


@pytest.mark.parametrize("n,seed,p0", [(12, 1, 0.0), (40, 4, 0.0), (24, 7, 1.0)])
def test_bullets_rollout_bit_exact(lib, orc, n, seed, p0):
    """Continuous collision (b2World::SolveTOI on the device, one warp per world): bullets fired
    and thrown at boxes (with p0 = 1 also kinematic bars driven through boxes), 120 steps, bodies
    bit for bit every step and contacts at the end; the impacts change the outcome (the same
    rollout without continuous collision differs)."""
    _rollout(lib, orc, G.SCENE_BULLETS, n, seed=seed, p0=p0, steps=120, continuous=True)
    plain = ob.OracleWorld(orc, (0.0, -10.0), scene=(G.SCENE_BULLETS, seed, n, p0, 0.6))
    ccd = ob.OracleWorld(orc, (0.0, -10.0), scene=(G.SCENE_BULLETS, seed, n, p0, 0.6), continuous=True)
    plain.step(120, 1 / 60, 8, 3)
    ccd.step(120, 1 / 60, 8, 3)
    assert _state_bytes(plain.bodies()) != _state_bytes(ccd.bodies())


def test_set_bullet_mid_rollout(lib, orc):
    """b2Body::SetBullet through the C ABI: half the bullets of a bullets world lose the flag
    after 4 steps (their impacts then go through the discrete step only) and the world steps on
    bit for bit like the oracle loaded with the edited state; clearing the rest turns
    SolveTOI off for the world (no bullet or kinematic body left)."""
    batch = G.Batch(lib, device=0)
    w = batch.add_world(0.0, -10.0)
    batch.set_flags(w, allow_sleep=False, warm_starting=True, continuous=True)
    batch.scene(w, G.SCENE_BULLETS, seed=5, n=16, p0=0.0, p1=0.6)
    batch.step_n(4, 1 / 60, 8, 3)
    bullets = [i for i, r in enumerate(batch.bodies(w)) if r.flags & G.BODY_BULLET]
    assert len(bullets) == 16
    for i in bullets[::2]:
        batch.set_bullet(w, i, False)
    assert [bool(batch.bodies(w)[i].flags & G.BODY_BULLET) for i in bullets] == [k % 2 == 1 for k in range(16)]
    ow = ob.OracleWorld(orc, (0.0, -10.0), batch.bodies(w), batch.fixtures(w), batch.joints(w), batch.contacts(w),
                        inv_dt0=60.0, continuous=True)
    for s in range(60):
        batch.step(1 / 60, 8, 3)
        ow.step(1, 1 / 60, 8, 3)
        g, o = batch.bodies(w), ow.bodies()
        assert _state_bytes(g) == _state_bytes(o), f"step {s + 1}: {_first_diff(g, o)}"
    for i in bullets[1::2]:
        batch.set_bullet(w, i, False)
    batch.step(1 / 60, 8, 3)
    assert batch.profile().solve_toi == 0.0
    batch.close()


def test_bullets_batch_sleep_events_step_io(lib, orc):
    """A batch of a bullets world with sleeping allowed, a bullets world without and a pyramid
    without continuous collision, stepped through b2g_step_io (transforms read after SolveTOI)
    with listener events on: every world bit for bit like the oracle every step, awake flags
    included, and the events (those of the sub-step impacts among them) equal per world."""
    from test_oracle_pins import event_key

    batch = G.Batch(lib, device=0)
    specs = [(G.SCENE_BULLETS, 15, 2, True, True), (G.SCENE_BULLETS, 9, 6, False, True),
             (G.SCENE_PYRAMID, 8, 1, False, False)]
    worlds, ows = [], []
    for kind, n, seed, sleep, cont in specs:
        w = batch.add_world(0.0, -10.0)
        batch.set_flags(w, allow_sleep=sleep, warm_starting=True, continuous=cont)
        batch.scene(w, kind, seed=seed, n=n, p0=1.0, p1=0.6)
        ow = ob.OracleWorld(orc, (0.0, -10.0), batch.bodies(w), batch.fixtures(w), batch.joints(w), continuous=cont)
        ow.set_sleep(sleep)
        ow.events_enable(True)
        worlds.append(w)
        ows.append(ow)
    batch.events(enable=True)
    nb = sum(len(batch.bodies(w)) for w in worlds)
    xf = np.zeros((nb, 4), np.float32)
    for s in range(100):
        got_n = batch.step_io(0, 0, xf.ctypes.data, nb, 1 / 60, 8, 3)
        assert got_n == nb
        off = 0
        for w, ow in zip(worlds, ows):
            ow.step(1, 1 / 60, 8, 3)
            g, o = batch.bodies(w), ow.bodies()
            assert _state_bytes(g) == _state_bytes(o), f"world {w} step {s + 1}: {_first_diff(g, o)}"
            assert _awake_flags(g) == _awake_flags(o), (w, s)
            got_xf = xf[off:off + len(g)]
            assert np.array_equal(got_xf, np.array([list(r.xf) for r in g], np.float32)), (w, s)
            off += len(g)
            got = [event_key(e) for e in batch.world_events(w)]
            exp = [event_key(e) for e in ow.events()]
            assert sorted(got) == sorted(exp), f"world {w} step {s + 1}: {len(got)} events against {len(exp)}"
    batch.close()


@pytest.mark.parametrize("n,seed,vi,pi", [(3, 9, 8, 3), (2, 17, 10, 4)])
def test_slider_rigs_rollout_bit_exact(lib, orc, n, seed, vi, pi):
    # distance joints (rigid rods, springs with min/max length, slack ropes) and prismatic joints
    # (limits, motors, a piston between two dynamic bodies): bodies every step, joint impulses
    # (including the limit and motor impulses) and contacts at the end
    _rollout(lib, orc, G.SCENE_SLIDERS, n, seed=seed, steps=240, vi=vi, pi=pi)


@pytest.mark.parametrize("n,seed,vi,pi", [(3, 9, 8, 3), (2, 17, 10, 4)])
def test_gear_rigs_rollout_bit_exact(lib, orc, n, seed, vi, pi):
    # gear joints (revolute-revolute with a motor, rack and pinion with prismatic limits, a double
    # pendulum whose gear moves one body through two of its rows) in the serial joint colour:
    # bodies every step, joint impulses (the gear's included) and contacts at the end
    _rollout(lib, orc, G.SCENE_GEARS, n, seed=seed, steps=240, vi=vi, pi=pi)


def _state_np(records_bytes, n):
    return np.frombuffer(records_bytes, dtype=np.uint8).reshape(n, -1)[:, :40]


def _rollout_large(lib, orc, kind, n, seed, p0, steps, checks, vi, pi):
    """One large world on the GPU and in the oracle, body states compared bit for bit at the
    `checks` steps (the whole record array at once), contact lists and joint impulses at the end."""
    batch = G.Batch(lib, device=0)
    w = batch.add_world(0.0, -10.0)
    batch.set_flags(w, allow_sleep=False, warm_starting=True, continuous=False)
    batch.scene(w, kind, seed=seed, n=n, p0=p0, p1=0.6)
    nb = batch.sizes(w)[0]
    ow = ob.OracleWorld(orc, (0.0, -10.0), batch.bodies(w), batch.fixtures(w), batch.joints(w))
    done = 0
    for at in checks:
        batch.step_n(at - done, 1 / 60, vi, pi, use_graph=True)
        ow.step(at - done, 1 / 60, vi, pi)
        done = at
        g = bytes((G.Body * nb)(*batch.bodies(w)))
        o = bytes((G.Body * nb)(*ow.bodies()))
        if g != o:
            diff = np.nonzero((_state_np(g, nb) != _state_np(o, nb)).any(axis=1))[0]
            raise AssertionError(f"step {at}: {len(diff)} bodies differ, first {diff[0]}: "
                                 f"{_first_diff(batch.bodies(w)[diff[0]:diff[0] + 1], ow.bodies()[diff[0]:diff[0] + 1])}")
    gc, oc = batch.contacts(w), ow.contacts()
    assert [_contact_key(x) for x in gc] == [_contact_key(y) for y in oc], "contact lists differ"
    for x, y in zip(batch.joints(w), ow.joints()):
        assert list(x.impulse) == list(y.impulse)
        assert (x.motor_impulse, x.lower_impulse, x.upper_impulse) == (y.motor_impulse, y.lower_impulse, y.upper_impulse)
    touching = sum(1 for c in gc if c.flags & 2)
    batch.close()
    return touching


def test_config_single_large_world_mixed_drop(lib, orc):
    """The single-large-world configuration at size: 20 000 boxes, circles and 3-8-gons dropped
    from a 200 x 400 m grid into the U container, 8/3 iterations, its full 512 steps (the bottom
    rows have landed and piled up by then)."""
    touching = _rollout_large(lib, orc, G.SCENE_MIXED_DROP, 20000, 1, 0.0, 512, (64, 192, 320, 512), 8, 3)
    assert touching > 5000


def test_config_chains_over_pile(lib, orc):
    """The joints + dense contact configuration at size: 2 000 chains of 20 boxes on revolute
    joints (limits, motors) over 10 000 circles, 10/4 iterations, 256 steps."""
    touching = _rollout_large(lib, orc, G.SCENE_CHAINS, 2000, 1, 10000.0, 256, (64, 128, 256), 10, 4)
    assert touching > 5000


def test_mixed_drop_rollout_bit_exact(lib, orc):
    # boxes, circles and 3-8 gons dropped into a U of two-sided edges
    _rollout(lib, orc, G.SCENE_MIXED_DROP, 600, seed=3, steps=200)


def test_chains_rollout_bit_exact(lib, orc):
    # revolute chains (limits, motors) over a circle pile, 10/4 iterations
    _rollout(lib, orc, G.SCENE_CHAINS, 20, seed=2, p0=300, steps=120, vi=10, pi=4)


@pytest.mark.parametrize("seed", [11, 12, 13])
def test_batch_world_rollout_bit_exact(lib, orc, seed):
    n = 300 + 97 * seed
    _rollout(lib, orc, G.SCENE_BATCH_WORLD, n, seed=seed, steps=80)


@pytest.mark.parametrize("rows", [90, 161])
def test_large_pyramid_rollout_bit_exact(lib, orc, rows):
    # 90 rows (4096 bodies): body state and per-body colouring state in shared memory, the
    # per-contact colouring arrays in global memory; 161 rows (13042 bodies): too large for the
    # CTA's shared memory, every solver array in global memory
    _rollout(lib, orc, G.SCENE_PYRAMID, rows, steps=4)


@pytest.mark.parametrize("kind,n,p0", [(G.SCENE_PYRAMID, 20, 1.0), (G.SCENE_CHAINS, 12, 200.0)])
def test_solver_order_matches_oracle(lib, orc, kind, n, p0):
    """The colour and priority of every solved contact and joint equal the oracle's greedy
    colouring (the Gauss-Seidel order up to the order inside a colour, which does not matter:
    constraints of one colour share no non-static body)."""
    batch = G.Batch(lib, device=0)
    w = batch.add_world(0.0, -10.0)
    batch.set_flags(w, allow_sleep=False, warm_starting=True, continuous=False)
    batch.scene(w, kind, seed=2, n=n, p0=p0, p1=0.6)
    ow = ob.OracleWorld(orc, (0.0, -10.0), batch.bodies(w), batch.fixtures(w), batch.joints(w))
    for _ in range(40):
        batch.step(1 / 60, 8, 3)
        ow.step(1, 1 / 60, 8, 3)
    before = [(c.fixture_a, c.fixture_b) for c in ow.contacts()]
    batch.step(1 / 60, 8, 3)
    ow.step(1, 1 / 60, 8, 3)
    after = [(c.fixture_a, c.fixture_b) for c in ow.contacts()]
    nb, nf, nj, nc = batch.sizes(w)
    gc, gp, gj, gjp = batch.solver_order(w, nc, nj)
    oc, op, oj, ojp = ow.solver_order()
    assert gj == oj and gjp == ojp
    if kind == G.SCENE_PYRAMID:
        # a settled pyramid keeps its contact list, so the oracle's per-contact record (indexed by
        # the list the solve read) lines up with the current list
        assert before == after and len(after) == nc
    if before == after:
        assert gc == oc and gp == op
        assert max(gc) >= 2
    batch.close()


@pytest.mark.parametrize("n,seed,vi,pi", [(4, 9, 8, 3), (2, 17, 10, 4)])
def test_joint_zoo_rollout_bit_exact(lib, orc, n, seed, vi, pi):
    """Weld (rigid and soft), wheel (springs, motor, limits), motor, friction, mouse and pulley
    joints: every body state, joint impulse and contact equals the oracle's after every step."""
    _rollout(lib, orc, G.SCENE_JOINTS, n, seed=seed, p0=0.0, steps=240, vi=vi, pi=pi)


def test_batched_equals_alone(lib):
    """Worlds stepped together in one batch are bit-identical to the same worlds stepped alone."""
    seeds = [21, 22, 23, 24, 25, 26]
    sizes = [40, 700, 16, 1500, 300, 90]
    together = G.Batch(lib, device=0)
    ws = []
    for s, n in zip(seeds, sizes):
        _, gx, gy = _params(lib, s)
        w = together.add_world(gx, gy)
        together.set_flags(w)
        together.scene(w, G.SCENE_BATCH_WORLD, seed=s, n=n)
        ws.append(w)
    for _ in range(40):
        together.step(1 / 60, 8, 3)
    for w, s, n in zip(ws, seeds, sizes):
        _, gx, gy = _params(lib, s)
        alone = G.Batch(lib, device=0)
        a = alone.add_world(gx, gy)
        alone.set_flags(a)
        alone.scene(a, G.SCENE_BATCH_WORLD, seed=s, n=n)
        for _ in range(40):
            alone.step(1 / 60, 8, 3)
        assert _state_bytes(together.bodies(w)) == _state_bytes(alone.bodies(a))
        alone.close()
    together.close()


def _mixed_batch(lib, seeds, sizes):
    b = G.Batch(lib, device=0)
    ws = []
    for s, n in zip(seeds, sizes):
        _, gx, gy = _params(lib, s)
        w = b.add_world(gx, gy)
        b.set_flags(w)
        b.scene(w, G.SCENE_BATCH_WORLD, seed=s, n=n)
        ws.append(w)
    return b, ws


# worlds in each CTA size class of the solver (at most 64, 512, 2048 and 8192 bodies)
CLASS_SEEDS = [31, 32, 33, 34, 35, 36]
CLASS_SIZES = [40, 200, 900, 3000, 5000, 60]


def test_solver_threads_do_not_change_results(lib):
    """Every world of every size class gives the same bits with 64 or 1024 threads per world (and
    the shared-memory allowance that goes with each)."""
    out = []
    for threads in ([64] * 5, [1024] * 5, [128, 256, 512, 1024, 512]):
        b, ws = _mixed_batch(lib, CLASS_SEEDS, CLASS_SIZES)
        assert b.solver_threads(threads) == threads
        for _ in range(30):
            b.step(1 / 60, 8, 3)
        out.append([_state_bytes(b.bodies(w)) for w in ws])
        b.close()
    assert out[0] == out[1] == out[2]


@pytest.mark.parametrize("kind,n,p0,vi,pi", [(G.SCENE_PYRAMID, 161, 1.0, 8, 3),
                                             (G.SCENE_CHAINS, 420, 2000.0, 10, 4)])
def test_cluster_solve_equals_one_cta(lib, kind, n, p0, vi, pi):
    """Worlds above 8192 bodies (a 13 041-box pyramid; 420 revolute chains over 2 000 circles)
    solved by thread-block clusters of 16, 8 and 2 CTAs give the bits of one CTA per world, beside
    a small world in the same batch."""
    out = []
    for ctas in (1, 16, 8, 2):
        b = G.Batch(lib, device=0)
        b.cluster_solve(ctas)
        w = b.add_world(0.0, -10.0)
        b.set_flags(w)
        b.scene(w, kind, seed=3, n=n, p0=p0, p1=0.6)
        small = b.add_world(0.0, -10.0)
        b.set_flags(small)
        b.scene(small, G.SCENE_PYRAMID, n=12, p0=1.0, p1=0.6)
        for _ in range(40):
            b.step(1 / 60, vi, pi)
        b.step_n(20, 1 / 60, vi, pi, use_graph=True)
        out.append((_state_bytes(b.bodies(w)), _state_bytes(b.bodies(small)),
                    [list(j.impulse) for j in b.joints(w)]))
        b.close()
    assert out[0] == out[1] == out[2] == out[3]


def test_cluster_solve_sleep_mode_bit_exact(lib, orc):
    """A 9 000-body batch world (chains over a pile) with sleeping allowed, solved by a cluster:
    the island union-find, the per-island position exit and the sleep timers run across the
    cluster's SMs (device checks verify the labels every step); body states, awake flags and
    sleep timers equal the oracle's at every check."""
    batch = G.Batch(lib, device=0)
    batch.set_debug_checks(True)
    w = _sleep_world(batch, G.SCENE_BATCH_WORLD, 9000, 7, 0.0)
    ow = ob.OracleWorld(orc, (0.0, -10.0), batch.bodies(w), batch.fixtures(w), batch.joints(w))
    ow.set_sleep(True)
    done = 0
    for at in (100, 200, 300, 400):
        batch.step_n(at - done, 1 / 60, 8, 3)
        ow.step(at - done, 1 / 60, 8, 3)
        done = at
        g, o = batch.bodies(w), ow.bodies()
        assert _state_bytes(g) == _state_bytes(o), f"step {at}: {_first_diff(g, o)}"
        assert _awake_flags(g) == _awake_flags(o), f"step {at}: awake flags differ"
        times = batch.sleep_times(w)
        assert times == ow.sleep_times(), f"step {at}: sleep timers differ"
    assert sum(1 for t in times if t > 0.0) > 100  # resting bodies are being timed
    batch.close()


def test_solver_build_and_tree_period_do_not_change_results(lib):
    """The occupancy (64-register) and wide (128-register) builds of the solver, and broadphases
    that rebuild every tree each step or refit kept trees for 16 steps, give the same bits, with
    CUDA graphs and without."""
    out = []
    for waves, period, graphs in ((0.0, 1, False), (1e9, 16, False), (0.0, 16, True), (1e9, 3, True)):
        b, ws = _mixed_batch(lib, CLASS_SEEDS, CLASS_SIZES)
        lib.check(lib.b2g_batch_set_solver_waves(b.h, waves), "waves")
        lib.check(lib.b2g_batch_set_tree_rebuild_period(b.h, period), "period")
        b.set_graphs(graphs)
        for _ in range(40):
            b.step(1 / 60, 8, 3)
        out.append([_state_bytes(b.bodies(w)) for w in ws])
        b.close()
    assert out[0] == out[1] == out[2] == out[3]


def test_autotune_picks_valid_threads_and_keeps_results(lib):
    tuned, ws = _mixed_batch(lib, CLASS_SEEDS, CLASS_SIZES)
    threads, taken = tuned.autotune(steps=2)
    assert all(t in (64, 128, 256, 512, 1024) for t in threads)
    assert tuned.solver_threads() == threads and taken >= 2
    for _ in range(10):
        tuned.step(1 / 60, 8, 3)
    plain, ws2 = _mixed_batch(lib, CLASS_SEEDS, CLASS_SIZES)
    for _ in range(taken + 10):
        plain.step(1 / 60, 8, 3)
    for w, w2 in zip(ws, ws2):
        assert _state_bytes(tuned.bodies(w)) == _state_bytes(plain.bodies(w2))
    tuned.close()
    plain.close()


def test_device_compaction_equals_fresh_batch(lib):
    """Retiring worlds and compacting the batch on the device leaves the kept worlds exactly as a
    batch that never held the others (bodies, contacts and the steps after)."""
    seeds, sizes = CLASS_SEEDS, CLASS_SIZES
    big, ws = _mixed_batch(lib, seeds, sizes)
    for _ in range(20):
        big.step(1 / 60, 8, 3)
    for w in (ws[1], ws[3]):
        lib.check(lib.b2g_world_retire(big.h, w), "retire")
    nmap = (C.c_int32 * len(ws))()
    lib.check(lib.b2g_compact(big.h, nmap, len(ws)), "compact")
    assert list(nmap) == [0, -1, 1, -1, 2, 3]
    for _ in range(20):
        big.step(1 / 60, 8, 3)
    kept = [0, 2, 4, 5]
    small, ws2 = _mixed_batch(lib, [seeds[i] for i in kept], [sizes[i] for i in kept])
    for _ in range(40):
        small.step(1 / 60, 8, 3)
    for new, w2 in enumerate(ws2):
        assert _state_bytes(big.bodies(new)) == _state_bytes(small.bodies(w2))
        assert [_contact_key(x) for x in big.contacts(new)] == [_contact_key(y) for y in small.contacts(w2)]
    big.close()
    small.close()


def test_appended_worlds_match_alone(lib):
    """Worlds appended to a running batch get their first contacts from a broadphase over the
    appended fixtures only; each world ends bit-identical to the same world stepped alone."""
    first, ws = _mixed_batch(lib, [41, 42], [500, 60])
    for _ in range(10):
        first.step(1 / 60, 8, 3)
    late = []
    for s, n in ((43, 800), (44, 3000), (45, 20)):
        _, gx, gy = _params(lib, s)
        w = first.add_world(gx, gy)
        first.set_flags(w)
        first.scene(w, G.SCENE_BATCH_WORLD, seed=s, n=n)
        late.append((w, s, n))
    for _ in range(30):
        first.step(1 / 60, 8, 3)
    for w, s, n, steps in [(ws[0], 41, 500, 40), (ws[1], 42, 60, 40)] + [(w, s, n, 30) for w, s, n in late]:
        alone, wa = _mixed_batch(lib, [s], [n])
        for _ in range(steps):
            alone.step(1 / 60, 8, 3)
        assert _state_bytes(first.bodies(w)) == _state_bytes(alone.bodies(wa[0])), s
        assert [_contact_key(x) for x in first.contacts(w)] == [_contact_key(y) for y in alone.contacts(wa[0])], s
        alone.close()
    first.close()


def test_nonfinite_world_is_frozen_alone(lib):
    """A world driven to a non-finite state (infinite forces: a floating-point fault, nothing on
    the device faults) is frozen and reported; the other worlds step on exactly as if it were
    not in the batch."""
    seeds, sizes = [71, 72, 73], [300, 500, 200]
    b, ws = _mixed_batch(lib, seeds, sizes)
    for _ in range(10):
        b.step(1 / 60, 8, 3)
    counts = [b.sizes(w)[0] for w in ws]
    forces = np.zeros((sum(counts), 4), dtype=np.float32)
    forces[counts[0]:counts[0] + counts[1], 1] = np.inf
    lib.check(lib.b2g_batch_set_forces(b.h, forces.ctypes.data_as(C.POINTER(C.c_float)), len(forces)), "forces")
    b.step(1 / 60, 8, 3)
    assert b.world_status(ws[1]) == 4 and b.world_status(ws[0]) == 0 and b.world_status(ws[2]) == 0
    frozen = _state_bytes(b.bodies(ws[1]))
    assert not np.isfinite(G.body_array_to_numpy((G.Body * counts[1])(*b.bodies(ws[1])))["c"]).all()
    for _ in range(20):
        b.step(1 / 60, 8, 3)
    assert _state_bytes(b.bodies(ws[1])) == frozen
    other, wo = _mixed_batch(lib, [seeds[0], seeds[2]], [sizes[0], sizes[2]])
    for _ in range(31):
        other.step(1 / 60, 8, 3)
    assert _state_bytes(b.bodies(ws[0])) == _state_bytes(other.bodies(wo[0]))
    assert _state_bytes(b.bodies(ws[2])) == _state_bytes(other.bodies(wo[1]))
    b.close()
    other.close()


def test_masked_step_leaves_other_worlds(lib):
    b = G.Batch(lib, device=0)
    w0 = b.add_world(0, -10)
    w1 = b.add_world(0, -10)
    for w in (w0, w1):
        b.set_flags(w)
        b.scene(w, G.SCENE_PYRAMID, n=5, p0=1.0, p1=0.6)
    before = _state_bytes(b.bodies(w1))
    b.step(1 / 60, 8, 3, mask=[1, 0])
    assert _state_bytes(b.bodies(w1)) == before
    assert _state_bytes(b.bodies(w0)) != _state_bytes(b.bodies(w1))
    b.close()


def _params(lib, seed):
    n = C.c_int32()
    gx = C.c_float()
    gy = C.c_float()
    lib.b2g_batch_world_params(seed, C.byref(n), C.byref(gx), C.byref(gy))
    return n.value, gx.value, gy.value


# ---------------------------------------------------------------- standalone kernels
def _rand_shape(rng, kind):
    s = G.Shape()
    if kind == G.SHAPE_CIRCLE:
        s.type = 0
        s.radius = float(rng.uniform(0.1, 0.6))
        s.vertices[0][0] = float(rng.uniform(-0.2, 0.2))
        s.vertices[0][1] = float(rng.uniform(-0.2, 0.2))
    elif kind == G.SHAPE_EDGE:
        s.type = 1
        s.radius = 0.01
        for i in range(4):
            s.vertices[i][0] = float(rng.uniform(-2, 2))
            s.vertices[i][1] = float(rng.uniform(-2, 2))
        s.one_sided = int(rng.integers(0, 2))
    else:
        n = int(rng.integers(3, 9))
        xy = rng.uniform(-0.6, 0.6, 2 * n).astype(np.float32)
        ob_ = ob.Oracle()
        if rng.uniform() < 0.3:
            ob_.orc_polygon_box(float(rng.uniform(0.1, 0.5)), float(rng.uniform(0.1, 0.5)), 0, 0, 0, 0, s)
        else:
            ob_.orc_polygon_set(xy.ctypes.data_as(C.POINTER(C.c_float)), n, s)
    return s


def test_collide_kernel_matches_oracle(lib, orc):
    rng = np.random.default_rng(7)
    kinds = [(0, 0), (2, 0), (2, 2), (1, 0), (1, 2)]
    n = 20000
    A = (G.Shape * n)()
    B = (G.Shape * n)()
    xa = np.zeros((n, 4), np.float32)
    xb = np.zeros((n, 4), np.float32)
    for i in range(n):
        ka, kb = kinds[i % 5]
        A[i] = _rand_shape(rng, ka)
        B[i] = _rand_shape(rng, kb)
        for x in (xa, xb):
            ang = rng.uniform(-3.2, 3.2)
            x[i] = (rng.uniform(-0.7, 0.7), rng.uniform(-0.7, 0.7), np.sin(ang), np.cos(ang))
    dA, dB = _dev_bytes(bytes(A)), _dev_bytes(bytes(B))
    dxa, dxb = torch.from_numpy(xa).cuda(), torch.from_numpy(xb).cuda()
    dout = torch.zeros(n * C.sizeof(G.Manifold), dtype=torch.uint8, device="cuda")
    st = lib.b2g_collide(dA.data_ptr(), dxa.data_ptr(), dB.data_ptr(), dxb.data_ptr(), n, dout.data_ptr(), None)
    assert st == 0
    torch.cuda.synchronize()
    out = (G.Manifold * n).from_buffer(bytearray(dout.cpu().numpy().tobytes()))
    touching = 0
    for i in range(n):
        m = G.Manifold()
        orc.orc_collide(A[i], (C.c_float * 4)(*xa[i]), B[i], (C.c_float * 4)(*xb[i]), m)
        g = out[i]
        assert g.point_count == m.point_count, i
        if m.point_count:
            touching += 1
            assert g.type == m.type
            assert bytes(g) == bytes(m), i
    assert touching > 3000


def test_toi_kernel_matches_oracle(lib, orc):
    """b2g_time_of_impact against the oracle's b2TimeOfImpact, bit for bit: the reference's own
    input set (tests/golden/toi.npz) and 20 000 random sweeps of every shape pairing."""
    g = np.load(Path(__file__).resolve().parent / "golden" / "toi.npz")
    raw = bytes(np.asarray(g["inputs"], np.uint8))
    golden = list((G.TOIInput * (len(raw) // C.sizeof(G.TOIInput))).from_buffer_copy(raw))
    rng = np.random.default_rng(11)
    kinds = [(0, 0), (2, 0), (2, 2), (1, 0), (1, 2), (0, 2), (2, 1)]
    extra = []
    for i in range(20000):
        q = G.TOIInput()
        ka, kb = kinds[i % len(kinds)]
        q.shape_a, q.shape_b = _rand_shape(rng, ka), _rand_shape(rng, kb)
        for k, sw in enumerate((q.sweep_a, q.sweep_b)):
            sw.local_center[:] = rng.uniform(-0.2, 0.2, 2)
            c0 = rng.uniform(-3, 3, 2) if k == 0 else rng.uniform(-0.3, 0.3, 2)
            sw.c0[:] = c0
            sw.c[:] = (-c0 if k == 0 else c0) + rng.uniform(-0.5, 0.5, 2)
            sw.a0 = rng.uniform(-7, 7)
            sw.a = sw.a0 + rng.uniform(-2, 2)
            sw.alpha0 = 0.0 if i % 3 else float(rng.uniform(0, 0.5))
        q.t_max = 1.0
        extra.append(q)
    inputs = golden + extra
    n = len(inputs)
    arr = (G.TOIInput * n)(*inputs)
    din = _dev_bytes(bytes(arr))
    dout = torch.zeros(n * C.sizeof(G.TOIOutput), dtype=torch.uint8, device="cuda")
    assert lib.b2g_time_of_impact(din.data_ptr(), n, dout.data_ptr(), None) == 0
    torch.cuda.synchronize()
    got = (G.TOIOutput * n).from_buffer(bytearray(dout.cpu().numpy().tobytes()))
    want = (G.TOIOutput * n)()
    orc.orc_time_of_impact(arr, n, want)
    assert bytes(got) == bytes(want)
    states = np.array([o.state for o in want])
    assert (states == G.TOI_TOUCHING).sum() > 3000 and (states == G.TOI_SEPARATED).sum() > 1000
    assert lib.b2g_time_of_impact(din.data_ptr(), -1, dout.data_ptr(), None) == 1  # B2G_E_INVALID_ARG


def test_pairs_kernel_matches_oracle(lib, orc):
    rng = np.random.default_rng(3)
    for n in (1, 2, 17, 1000, 20000):
        c = rng.uniform(-50, 50, (n, 2)).astype(np.float32)
        h = rng.uniform(0.05, 1.5, (n, 2)).astype(np.float32)
        aabb = np.concatenate([c - h, c + h], axis=1).astype(np.float32)
        fp = aabb.ctypes.data_as(C.POINTER(C.c_float))
        cap = int(orc.orc_pairs(fp, n, None, 0)) + 16
        ref = np.zeros(cap, np.uint64)
        nref = orc.orc_pairs(fp, n, ref.ctypes.data_as(C.POINTER(C.c_uint64)), cap)
        d_aabb = torch.from_numpy(aabb).cuda()
        d_pairs = torch.zeros(cap, dtype=torch.int64, device="cuda")
        npairs = C.c_int64()
        st = lib.b2g_pairs(d_aabb.data_ptr(), n, d_pairs.data_ptr(), cap, C.byref(npairs), None)
        assert st == 0
        assert npairs.value == nref
        got = d_pairs.cpu().numpy().view(np.uint64)[:nref]
        assert np.array_equal(got, ref[:nref])


def test_pairs_capacity_reported(lib):
    n = 100
    aabb = np.tile(np.array([[0, 0, 1, 1]], np.float32), (n, 1))
    d_aabb = torch.from_numpy(aabb).cuda()
    d_pairs = torch.zeros(10, dtype=torch.int64, device="cuda")
    npairs = C.c_int64()
    st = lib.b2g_pairs(d_aabb.data_ptr(), n, d_pairs.data_ptr(), 10, C.byref(npairs), None)
    assert st == 7  # B2G_E_CAPACITY
    assert npairs.value == n * (n - 1) // 2


# ---------------------------------------------------------------- graphs and capacity recovery
def test_graph_replay_equals_eager(lib):
    """The Step replayed as a captured CUDA graph is bit-identical to the eagerly launched Step."""
    out = []
    for graphs in (0, 1):
        b = G.Batch(lib, device=0)
        for s, n in ((31, 900), (32, 200), (33, 2500)):
            _, gx, gy = _params(lib, s)
            w = b.add_world(gx, gy)
            b.set_flags(w)
            b.scene(w, G.SCENE_BATCH_WORLD, seed=s, n=n)
        lib.b2g_batch_set_graphs(b.h, graphs)
        for _ in range(60):
            b.step(1 / 60, 8, 3)
        out.append([_state_bytes(b.bodies(w)) for w in range(3)])
        b.close()
    assert out[0] == out[1]


@pytest.mark.parametrize("kind,n,every,continuous", [(G.SCENE_PYRAMID, 12, 10, False), (G.SCENE_BULLETS, 20, 3, True)])
def test_pair_overflow_recovery_bit_exact(lib, orc, kind, n, every, continuous):
    """Contact buffers far too small: every overflowing broadphase is redone with larger buffers
    and the rollout still matches the oracle bit for bit. With continuous collision a step has two
    pair updates around SolveTOI: an overflow of the first makes the TOI kernel stand aside and
    the stage rerun after the redone update; an overflow of the second redoes only that one."""
    b = G.Batch(lib, device=0)
    w = b.add_world(0.0, -10.0)
    b.set_flags(w, continuous=continuous)
    b.scene(w, kind, n=n, p0=1.0, p1=0.6)
    ow = ob.OracleWorld(orc, (0.0, -10.0), b.bodies(w), b.fixtures(w), b.joints(w), continuous=continuous)
    for s in range(40):
        if s % every == 0:
            nc = b.sizes(w)[3]
            assert lib.b2g_debug_set_contact_capacity(b.h, max(nc, 1)) == 0
        b.step(1 / 60, 8, 3)
        ow.step(1, 1 / 60, 8, 3)
        assert _state_bytes(b.bodies(w)) == _state_bytes(ow.bodies()), f"step {s + 1}"
    b.close()


def test_snapshot_resumes_bit_identically(lib):
    """Checkpoint a world mid-rollout, keep stepping the original; restoring the checkpoint into a
    fresh batch (and into the same batch, as an appended world) and stepping as far gives the same
    bits, warm starting included."""
    b, ws = _mixed_batch(lib, [81, 82, 83], [400, 1500, 90])
    for _ in range(30):
        b.step(1 / 60, 8, 3)
    blob = b.snapshot(ws[1])
    fresh = G.Batch(lib, device=0)
    wf = fresh.restore(blob)
    for _ in range(25):
        b.step(1 / 60, 8, 3)
        fresh.step(1 / 60, 8, 3)
    assert _state_bytes(fresh.bodies(wf)) == _state_bytes(b.bodies(ws[1]))
    assert [_contact_key(x) for x in fresh.contacts(wf)] == [_contact_key(y) for y in b.contacts(ws[1])]
    again = b.restore(b.snapshot(ws[0]))
    for _ in range(10):
        b.step(1 / 60, 8, 3)
    twin = G.Batch(lib, device=0)
    wt = twin.restore(blob)
    for _ in range(35):
        twin.step(1 / 60, 8, 3)
    assert _state_bytes(twin.bodies(wt)) == _state_bytes(b.bodies(ws[1]))
    assert _state_bytes(b.bodies(again)) == _state_bytes(b.bodies(ws[0]))
    fresh.close()
    twin.close()
    b.close()


def test_colouring_check_passes_and_changes_nothing(lib):
    """With the device colouring check on, every step of worlds in every size class (and worlds
    with joint chains and a dense pyramid) passes it, and the results equal those without it."""
    out = []
    for checks in (True, False):
        b, ws = _mixed_batch(lib, CLASS_SEEDS, CLASS_SIZES)
        for kind, n, p0 in ((G.SCENE_CHAINS, 12, 30.0), (G.SCENE_PYRAMID, 40, 1.0)):
            w = b.add_world(0.0, -10.0)
            b.set_flags(w)
            b.scene(w, kind, seed=5, n=n, p0=p0, p1=0.6)
            ws.append(w)
        b.set_debug_checks(checks)
        for s in range(30):
            b.step(1 / 60, 8, 3)
            if s == 10:
                b.set_graphs(False)
        out.append([_state_bytes(b.bodies(w)) for w in ws])
        b.close()
    assert out[0] == out[1]


def test_budget_exhaustion_fails_cleanly(lib):
    """A batch whose device memory budget cannot hold its worlds fails the step with
    OUT_OF_MEMORY and a message (no partial state is stepped); the batch closes cleanly and a
    batch with room steps the same world to the same bits as one without a budget."""
    _, gx, gy = _params(lib, 41)
    tight = G.Batch(lib, device=0, budget_bytes=2 << 20)
    w = tight.add_world(gx, gy)
    tight.set_flags(w)
    tight.scene(w, G.SCENE_BATCH_WORLD, seed=41, n=6000)
    with pytest.raises(G.B2GError, match="OUT_OF_MEMORY"):
        tight.step(1 / 60, 8, 3)
    assert "budget" in lib.b2g_last_error().decode()
    tight.close()
    out = []
    for budget in (0, 1 << 30):
        b = G.Batch(lib, device=0, budget_bytes=budget)
        w = b.add_world(gx, gy)
        b.set_flags(w)
        b.scene(w, G.SCENE_BATCH_WORLD, seed=41, n=6000)
        for _ in range(10):
            b.step(1 / 60, 8, 3)
        out.append(_state_bytes(b.bodies(w)))
        b.close()
    assert out[0] == out[1]


def _awake_flags(records):
    return [r.flags & 8 for r in records]


def _sleep_world(batch, kind, n, seed, p0):
    w = batch.add_world(0.0, -10.0)
    batch.set_flags(w, allow_sleep=True)
    batch.scene(w, kind, seed=seed, n=n, p0=p0, p1=0.6)
    return w


@pytest.mark.parametrize("kind,n,seed,p0,steps,vi,pi", [
    (G.SCENE_JOINTS, 3, 9, 0.0, 400, 8, 3),
    (G.SCENE_PYRAMID, 10, 1, 1.0, 160, 8, 3),
    (G.SCENE_CHAINS, 6, 4, 100.0, 500, 10, 4),
    (G.SCENE_MIXED_DROP, 200, 5, 0.0, 490, 8, 3),
    (G.SCENE_BATCH_WORLD, 200, 11, 0.0, 760, 8, 3),
])
def test_sleep_rollout_bit_exact(lib, orc, kind, n, seed, p0, steps, vi, pi):
    """Sleeping on: islands fall asleep, are skipped while asleep and are woken by impacts and
    through their islands; body states, awake flags and sleep timers equal the oracle's (whose
    sleep rules are pinned to the reference step by step) after every step."""
    batch = G.Batch(lib, device=0)
    batch.set_debug_checks(True)  # colouring and island labels verified on the device every step
    w = _sleep_world(batch, kind, n, seed, p0)
    ow = ob.OracleWorld(orc, (0.0, -10.0), batch.bodies(w), batch.fixtures(w), batch.joints(w))
    ow.set_sleep(True)
    asleep_max, woken = 0, 0
    prev = _awake_flags(batch.bodies(w))
    for s in range(steps):
        batch.step(1 / 60, vi, pi)
        ow.step(1, 1 / 60, vi, pi)
        g, o = batch.bodies(w), ow.bodies()
        assert _state_bytes(g) == _state_bytes(o), f"step {s + 1}: {_first_diff(g, o)}"
        cur = _awake_flags(g)
        assert cur == _awake_flags(o), f"step {s + 1}: awake flags differ"
        woken += sum(1 for x, y in zip(prev, cur) if y and not x)
        asleep_max = max(asleep_max, sum(1 for r in g if r.type != 0 and not r.flags & 8))
        prev = cur
        if s % 20 == 19 or s == steps - 1:
            assert batch.sleep_times(w) == ow.sleep_times(), f"step {s + 1}: sleep timers differ"
    gc, oc = batch.contacts(w), ow.contacts()
    assert [_contact_key(x) for x in gc] == [_contact_key(y) for y in oc]
    assert asleep_max > 0
    if kind == G.SCENE_CHAINS:
        assert woken > 0
    batch.close()


def test_sleeping_pyramid_woken_by_a_moved_box(lib, orc):
    """A sleeping pyramid whose top box is lifted and thrown down: the lifted box's destroyed
    contacts wake the boxes under it, its impact wakes them again, the pyramid settles and falls
    asleep anew; every step equals the oracle."""
    batch = G.Batch(lib, device=0)
    w = _sleep_world(batch, G.SCENE_PYRAMID, 10, 1, 1.0)
    for _ in range(150):
        batch.step(1 / 60, 8, 3)
    bodies = batch.bodies(w)
    assert all(not r.flags & 8 for r in bodies if r.type != 0)
    top = max(range(len(bodies)), key=lambda i: bodies[i].c[1])
    r = bodies[top]
    r.c[1] += 3.0
    r.xf[1] += 3.0
    r.v[1] = -1.0
    recs = list(bodies)
    recs[top] = r
    batch.write_bodies(w, recs)
    ow = ob.OracleWorld(orc, (0.0, -10.0), batch.bodies(w), batch.fixtures(w), batch.joints(w),
                        batch.contacts(w), inv_dt0=60.0)
    ow.set_sleep(True)
    ow.set_sleep_times(batch.sleep_times(w))
    ow.orc.orc_world_flag_new_contacts(ow.h)
    woken, asleep_end = 0, 0
    prev = _awake_flags(batch.bodies(w))
    for s in range(200):
        batch.step(1 / 60, 8, 3)
        ow.step(1, 1 / 60, 8, 3)
        g, o = batch.bodies(w), ow.bodies()
        assert _state_bytes(g) == _state_bytes(o), f"step {s + 1}: {_first_diff(g, o)}"
        cur = _awake_flags(g)
        assert cur == _awake_flags(o), f"step {s + 1}"
        woken += sum(1 for x, y in zip(prev, cur) if y and not x)
        prev = cur
    assert batch.sleep_times(w) == ow.sleep_times()
    assert woken > 5
    batch.close()


def test_sleep_worlds_batched_with_others_equal_alone(lib):
    """Sleep-mode worlds and ordinary worlds stepped together (graph replay) give each world the
    bits it gets alone; compaction and snapshots carry the sleep state."""
    specs = [(G.SCENE_PYRAMID, 10, 1, 1.0, True), (G.SCENE_BATCH_WORLD, 300, 7, 0.0, False),
             (G.SCENE_BATCH_WORLD, 200, 11, 0.0, True), (G.SCENE_CHAINS, 6, 4, 100.0, True),
             (G.SCENE_MIXED_DROP, 150, 3, 0.0, False)]

    def make(batch, spec):
        kind, n, seed, p0, sleep = spec
        w = batch.add_world(0.0, -10.0)
        batch.set_flags(w, allow_sleep=sleep)
        batch.scene(w, kind, seed=seed, n=n, p0=p0, p1=0.6)
        return w

    together = G.Batch(lib, device=0)
    together.set_debug_checks(True)
    ws = [make(together, sp) for sp in specs]
    for _ in range(300):
        together.step(1 / 60, 8, 3)
    snap = together.snapshot(ws[2])
    # retire the second world and compact: the others keep their sleep state
    lib.check(lib.b2g_world_retire(together.h, ws[1]), "retire")
    nmap = (C.c_int32 * len(ws))()
    lib.check(lib.b2g_compact(together.h, nmap, len(ws)), "compact")
    kept = [nmap[w] for w in ws]
    restored = together.restore(snap)
    for _ in range(200):
        together.step(1 / 60, 8, 3)
    for i, sp in enumerate(specs):
        if i == 1:
            continue
        alone = G.Batch(lib, device=0)
        a = make(alone, sp)
        alone.set_graphs(False)
        for _ in range(500):
            alone.step(1 / 60, 8, 3)
        w = kept[i]
        assert _state_bytes(together.bodies(w)) == _state_bytes(alone.bodies(a)), i
        assert _awake_flags(together.bodies(w)) == _awake_flags(alone.bodies(a)), i
        assert together.sleep_times(w) == alone.sleep_times(a), i
        if i == 2:  # the restored copy went on from step 300 like the original
            assert _state_bytes(together.bodies(restored)) == _state_bytes(alone.bodies(a))
            assert together.sleep_times(restored) == alone.sleep_times(a)
        alone.close()
    together.close()


def test_set_awake_and_disallowing_sleep(lib, orc):
    """b2Body::SetAwake(false) on a falling body freezes it until a contact wakes it, and
    SetAllowSleeping(false) wakes every body: both equal the oracle."""
    batch = G.Batch(lib, device=0)
    w = _sleep_world(batch, G.SCENE_PYRAMID, 10, 1, 1.0)
    for _ in range(150):
        batch.step(1 / 60, 8, 3)
    assert all(not r.flags & 8 for r in batch.bodies(w) if r.type != 0)
    ow = ob.OracleWorld(orc, (0.0, -10.0), batch.bodies(w), batch.fixtures(w), batch.joints(w),
                        batch.contacts(w), inv_dt0=60.0)
    ow.set_sleep(True)
    ow.set_sleep_times(batch.sleep_times(w))
    for _ in range(30):
        batch.step(1 / 60, 8, 3)
        ow.step(1, 1 / 60, 8, 3)
    assert _state_bytes(batch.bodies(w)) == _state_bytes(ow.bodies())
    batch.set_flags(w, allow_sleep=False)
    ow.set_sleep(False)
    assert all(r.flags & 8 for r in batch.bodies(w) if r.type != 0)
    for s in range(30):
        batch.step(1 / 60, 8, 3)
        ow.step(1, 1 / 60, 8, 3)
        assert _state_bytes(batch.bodies(w)) == _state_bytes(ow.bodies()), s
    # a body put to sleep by hand: flags, velocity and force cleared; its island wakes it again
    batch.set_flags(w, allow_sleep=True)
    top = len(batch.bodies(w)) - 1
    batch.set_awake(w, top, False)
    r = batch.bodies(w)[top]
    assert not r.flags & 8 and tuple(r.v) == (0.0, 0.0) and r.w == 0.0 and tuple(r.force) == (0.0, 0.0)
    ow = ob.OracleWorld(orc, (0.0, -10.0), batch.bodies(w), batch.fixtures(w), batch.joints(w),
                        batch.contacts(w), inv_dt0=60.0)
    ow.set_sleep(True)
    ow.set_sleep_times(batch.sleep_times(w))
    for s in range(40):
        batch.step(1 / 60, 8, 3)
        ow.step(1, 1 / 60, 8, 3)
        assert _state_bytes(batch.bodies(w)) == _state_bytes(ow.bodies()), s
        assert _awake_flags(batch.bodies(w)) == _awake_flags(ow.bodies()), s
    batch.close()


def test_destroy_body_fixture_joint(lib, orc):
    """b2World::DestroyBody / b2Body::DestroyFixture / b2World::DestroyJoint through the C ABI on
    a settled pyramid and a chain: the destroyed contacts that were touching end (End events,
    returned at once), the rest of the world keeps its contacts and impulses, and it steps on
    bit for bit like the oracle loaded with the same post-removal state."""
    batch = G.Batch(lib, device=0)
    w = batch.add_world(0.0, -10.0)
    batch.set_flags(w, allow_sleep=False)
    batch.scene(w, G.SCENE_PYRAMID, n=10, p0=1.0, p1=0.6)
    c = batch.add_world(0.0, -10.0)
    batch.set_flags(c, allow_sleep=False)
    batch.scene(c, G.SCENE_CHAINS, seed=2, n=6, p0=60, p1=0.6)
    batch.step_n(90, 1 / 60, 8, 3)
    bodies = batch.bodies(w)
    nb0 = len(bodies)
    # the bottom-row box nearest the pyramid's middle (body 0 is the ground)
    mid = min((i for i in range(1, nb0) if bodies[i].c[1] < 1.0), key=lambda i: abs(bodies[i].c[0]))
    fixtures = batch.fixtures(w)
    fid = [i for i, f in enumerate(fixtures) if f.body == mid][0]
    before = batch.contacts(w)
    touching = {(x.fixture_a, x.fixture_b) for x in before if x.flags & 2 and fid in (x.fixture_a, x.fixture_b)}
    assert len(touching) >= 3
    ended = batch.remove(w, bodies=[mid])
    assert {(e.fixture_a, e.fixture_b) for e in ended} == touching and all(e.kind == G.EVENT_END for e in ended)
    assert len(batch.bodies(w)) == nb0 - 1
    # the other contacts stay, with fixture indices past the removed one shifted down
    down = lambda f: f - 1 if f > fid else f  # noqa: E731
    kept = [(down(x.fixture_a), down(x.fixture_b), x.flags, bytes(x.manifold)) for x in before
            if fid not in (x.fixture_a, x.fixture_b)]
    assert [(x.fixture_a, x.fixture_b, x.flags, bytes(x.manifold)) for x in batch.contacts(w)] == kept
    # a joint and a fixture of the chain world
    nj0 = len(batch.joints(c))
    batch.remove(c, joints=[3])
    assert len(batch.joints(c)) == nj0 - 1
    cf = batch.fixtures(c)
    ended_f = batch.remove(c, fixtures=[len(cf) - 1])
    assert len(batch.fixtures(c)) == len(cf) - 1
    assert all(e.kind == G.EVENT_END for e in ended_f)
    # both worlds step on like the oracle from the post-removal state
    worlds = [(w, (0.0, -10.0), 8, 3), (c, (0.0, -10.0), 8, 3)]
    ows = [ob.OracleWorld(orc, g, batch.bodies(x), batch.fixtures(x), batch.joints(x), batch.contacts(x),
                          inv_dt0=60.0) for x, g, _, _ in worlds]
    for s in range(60):
        batch.step(1 / 60, 8, 3)
        for (x, _, vi, pi), ow in zip(worlds, ows):
            ow.step(1, 1 / 60, vi, pi)
            g, o = batch.bodies(x), ow.bodies()
            assert _state_bytes(g) == _state_bytes(o), f"world {x} step {s + 1}: {_first_diff(g, o)}"
    batch.close()


def test_listener_events_match_oracle(lib, orc):
    """Begin / End / PreSolve / PostSolve events of every step, per world (b2g_events_drain_world)
    for a pyramid and a chains-over-pile world stepped in one batch, equal the oracle's events
    (whose event set is pinned to the reference's listener callbacks): kinds, fixture pairs, old
    manifold point counts, PostSolve impulses bit for bit. Draining one world leaves the
    other's events in place."""
    from test_oracle_pins import event_key

    batch = G.Batch(lib, device=0)
    specs = [(G.SCENE_PYRAMID, 15, 1, 1.0), (G.SCENE_CHAINS, 8, 3, 120.0)]
    worlds, ows = [], []
    for kind, n, seed, p0 in specs:
        w = batch.add_world(0.0, -10.0)
        batch.set_flags(w, allow_sleep=False)
        batch.scene(w, kind, seed=seed, n=n, p0=p0, p1=0.6)
        ow = ob.OracleWorld(orc, (0.0, -10.0), batch.bodies(w), batch.fixtures(w), batch.joints(w))
        ow.events_enable(True)
        worlds.append(w)
        ows.append(ow)
    batch.events(enable=True)
    kinds = set()
    for s in range(150):
        batch.step(1 / 60, 8, 3)
        for w, ow in zip(reversed(worlds), reversed(ows)):  # the second world drained first
            ow.step(1, 1 / 60, 8, 3)
            got = [event_key(e) for e in batch.world_events(w)]
            exp = [event_key(e) for e in ow.events()]
            assert got == exp, f"world {w} step {s + 1}: {len(got)} events against {len(exp)}"
            kinds |= {k[0] for k in got}
        assert batch.events() == []  # nothing left once every world drained its own
    assert kinds == {G.EVENT_BEGIN, G.EVENT_END, G.EVENT_PRESOLVE, G.EVENT_POSTSOLVE}
    batch.close()


@pytest.mark.parametrize("name", ["pyramid", "mixed", "chains"])
def test_rollout_measures_vs_reference_golden(lib, orc, name):
    """The GPU's 256-step rollouts of the pyramid, a mixed drop and chains over a pile against the
    reference's own rollouts, by physical measures every 32 steps (momentum, centre-of-mass and
    top height, deepest penetration), within ob.ROLLOUT_TOLERANCES."""
    from pathlib import Path

    g = np.load(Path(__file__).resolve().parent / "golden" / f"measures_{name}.npz")
    kind, n, seed, p0 = int(g["kind"]), int(g["n"]), int(g["seed"]), float(g["p0"])
    every, vi, pi = int(g["every"]), int(g["vi"]), int(g["pi"])
    batch = G.Batch(lib, device=0)
    w = batch.add_world(0.0, -10.0)
    batch.set_flags(w, allow_sleep=False)
    batch.scene(w, kind, seed=seed, n=n, p0=p0, p1=0.6)
    fixtures = list(batch.fixtures(w))
    rows = []
    for _ in range(len(g["rows"])):
        batch.step_n(every, 1 / 60, vi, pi, use_graph=True)
        rows.append(ob.measure_row(ob.rollout_measures(orc, list(batch.bodies(w)), fixtures, list(batch.contacts(w)))))
    ob.check_rollout_measures(name, rows, g["rows"])
    batch.close()


def test_step_io_equals_separate_calls(lib):
    """b2g_step_io (forces in, transforms out, the copies overlapping the step on a stream of their
    own) gives bit for bit what b2g_batch_set_forces + b2g_step + b2g_batch_read_states give, step
    after step, under graph replay and with forces that change every step."""
    import torch

    a, _ = _mixed_batch(lib, CLASS_SEEDS[:4], CLASS_SIZES[:4])
    b, _ = _mixed_batch(lib, CLASS_SEEDS[:4], CLASS_SIZES[:4])
    a.step(1 / 60, 8, 3)
    b.step(1 / 60, 8, 3)
    nb = a.profile().bodies
    rng = np.random.default_rng(5)
    forces = torch.zeros((nb, 4), dtype=torch.float32).pin_memory()
    xa = torch.empty((nb, 4), dtype=torch.float32).pin_memory()
    xb = torch.empty((nb, 4), dtype=torch.float32).pin_memory()
    n_out = C.c_int64()
    for step in range(24):
        forces.copy_(torch.from_numpy(rng.normal(0.0, 5.0, (nb, 4)).astype(np.float32)))
        assert a.step_io(forces.data_ptr(), nb, xa.data_ptr(), nb) == nb
        lib.check(lib.b2g_batch_set_forces(b.h, forces.data_ptr(), nb), "set_forces")
        b.step(1 / 60, 8, 3)
        lib.check(lib.b2g_batch_read_states(b.h, C.cast(xb.data_ptr(), C.POINTER(C.c_float)), None, nb,
                                            C.byref(n_out)), "read_states")
        assert torch.equal(xa, xb), f"step {step}"
    for w in range(4):
        assert _state_bytes(a.bodies(w)) == _state_bytes(b.bodies(w))
    # without host buffers it is a plain step
    assert a.step_io(0, 0, 0, 0) == nb
    b.step(1 / 60, 8, 3)
    for w in range(4):
        assert _state_bytes(a.bodies(w)) == _state_bytes(b.bodies(w))
    a.close()
    b.close()
