"""Continuous-batching server: a rollout's result does not depend on what else is being served.

Each request (seeded scene + K steps) is run once alone on its own server and once in a mix of
requests arriving at different ticks, with retirements and compactions in between; the final
state summaries must be identical bit for bit (every world is stepped independently, so joining
a batch cannot change its arithmetic). Admission obeys the device memory budget.
"""
import pytest

import b2gpu as G

pytestmark = pytest.mark.gpu

REQS = [(101, 40, 30), (102, 350, 12), (103, 900, 25), (104, 64, 1), (105, 1500, 18), (106, 200, 40),
        (107, 32, 0), (108, 700, 22)]


def _run(lib, reqs, arrivals, builders=None):
    srv = G.Server(lib, device=0, budget_bytes=8 << 30, max_worlds=64, builders=builders)
    ids = {}
    pending = sorted(zip(arrivals, reqs))
    results = {}
    tick = 0
    while pending or srv.stats()["active"] or srv.stats()["queued"]:
        while pending and pending[0][0] <= tick:
            _, (seed, n, k) = pending.pop(0)
            ids[srv.submit(seed, n, k)] = seed
        srv.tick()
        for r in srv.poll():
            results[ids[r.request_id]] = (r.status, r.steps, tuple(r.checksum))
        tick += 1
        assert tick < 1000
    srv.close()
    return results


@pytest.mark.parametrize("builders", [None, 0, 4])
def test_results_same_alone_and_in_mix(lib, builders):
    """Alone vs in a mix, with worlds built on builder threads (default 2, or 4) or by the tick
    itself while the device steps (0)."""
    alone = {}
    for q in REQS:
        alone.update(_run(lib, [q], [0]))
    mixed = _run(lib, REQS, [0, 0, 3, 5, 5, 9, 10, 17], builders)
    assert set(mixed) == {q[0] for q in REQS}
    for seed, n, k in REQS:
        assert alone[seed][0] == 0 and mixed[seed][0] == 0
        assert alone[seed][1] == k == mixed[seed][1]
        assert alone[seed] == mixed[seed], seed


def test_admission_respects_budget_and_rejects_oversize(lib):
    per_body = 2304
    srv = G.Server(lib, device=0, budget_bytes=1000 * per_body, max_worlds=16)
    big = srv.submit(7, 5000, 5)          # larger than the whole budget: rejected
    a = srv.submit(8, 400, 50)
    b = srv.submit(9, 400, 50)
    c = srv.submit(10, 400, 50)           # does not fit next to a and b: waits
    active, _ = srv.tick()
    assert active == 2
    st = srv.stats()
    assert st["queued"] == 1 and st["rejected"] == 1
    rejected = [r for r in srv.poll() if r.request_id == big]
    assert rejected and rejected[0].status == 2  # B2G_E_OUT_OF_MEMORY
    done = set()
    for _ in range(200):
        srv.tick()
        done |= {r.request_id for r in srv.poll()}
        if {a, b, c} <= done:
            break
    assert {a, b, c} <= done
    srv.close()


def test_cancel_mid_rollout_leaves_the_others_unchanged(lib):
    """A running request cancelled mid-rollout finishes with CANCELLED after the steps it took; its
    world's slot and budget are released and the requests served beside it end exactly as alone."""
    alone = {}
    for q in REQS[:3]:
        alone.update(_run(lib, [q], [0]))
    srv = G.Server(lib, device=0, budget_bytes=8 << 30, max_worlds=64)
    ids = {srv.submit(seed, n, k): seed for seed, n, k in REQS[:3]}
    victim = srv.submit(999, 1200, 500)
    late = None
    results, tick = {}, 0
    while srv.stats()["active"] or srv.stats()["queued"]:
        srv.tick()
        tick += 1
        if tick == 3:
            late = srv.submit(998, 2000, 300)  # admitted while tick 4 steps; never stepped
        if tick == 4:
            assert srv.cancel(late) == 0
        if tick == 6:
            assert srv.cancel(victim) == 0
            assert srv.cancel(victim) == 1  # already finished
        for r in srv.poll():
            results[r.request_id] = (r.status, r.steps, tuple(r.checksum))
        assert tick < 1000
    assert results[victim][:2] == (8, 5)  # admitted in tick 1, stepped in ticks 2-6
    assert results[late][:2] == (8, 0)
    for rid, seed in ids.items():
        assert results[rid] == alone[seed], seed
    srv.close()


def _snap(batch, world):
    return bytes(memoryview((G.Body * batch.sizes(world)[0])(*batch.bodies(world))))


def test_split_step_with_staged_admission_matches_plain_step(lib):
    """b2g_step_begin/_end with a world built and staged while the step runs gives the same bytes
    as plain steps with the world built between them; calls that need the device state return
    LOCKED while the step is in flight, and edits of the world not on the device yet are allowed."""
    def make():
        b = G.Batch(lib, 0)
        for seed in (11, 12):
            w = b.add_world()
            b.set_flags(w, warm_starting=True)
            b.scene(w, G.SCENE_BATCH_WORLD, seed=seed, n=300)
        b.step()
        return b

    plain, split = make(), make()
    for _ in range(4):   # the split batch's fourth step is the one with the world built beside it
        plain.step()
    w_plain = plain.add_world()
    plain.scene(w_plain, G.SCENE_JOINTS, seed=5, n=2)
    plain.step(mask=[1, 1, 0])

    for _ in range(3):
        split.step_begin()
        split.step_end()
    split.step_begin()
    with pytest.raises(G.B2GError, match="LOCKED"):
        split.bodies(0)
    w_split = split.add_world()
    split.scene(w_split, G.SCENE_JOINTS, seed=5, n=2)
    split.stage()
    split.step_end()
    assert split.step_done()
    split.step_begin(mask=[1, 1, 0])   # uploads the staged world, leaves it out of the solve
    split.step_end()
    assert w_split == w_plain
    for _ in range(20):
        plain.step()
        split.step_begin()
        split.step_end()
    for w in range(3):
        assert _snap(plain, w) == _snap(split, w), w
    plain.close()
    split.close()
