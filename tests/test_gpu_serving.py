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


def _run(lib, reqs, arrivals):
    srv = G.Server(lib, device=0, budget_bytes=8 << 30, max_worlds=64)
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


def test_results_same_alone_and_in_mix(lib):
    alone = {}
    for q in REQS:
        alone.update(_run(lib, [q], [0]))
    mixed = _run(lib, REQS, [0, 0, 3, 5, 5, 9, 10, 17])
    assert set(mixed) == {q[0] for q in REQS}
    for seed, n, k in REQS:
        assert alone[seed][0] == 0 and mixed[seed][0] == 0
        assert alone[seed][1] == k == mixed[seed][1]
        assert alone[seed] == mixed[seed], seed


def test_admission_respects_budget_and_rejects_oversize(lib):
    per_body = 2048
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
    results, tick = {}, 0
    while srv.stats()["active"] or srv.stats()["queued"]:
        srv.tick()
        tick += 1
        if tick == 6:
            assert srv.cancel(victim) == 0
            assert srv.cancel(victim) == 1  # already finished
        for r in srv.poll():
            results[r.request_id] = (r.status, r.steps, tuple(r.checksum))
        assert tick < 1000
    assert results[victim][:2] == (8, 6)
    for rid, seed in ids.items():
        assert results[rid] == alone[seed], seed
    srv.close()
