"""Benchmark of the batched b2World::Step on one GB300 (and N GPUs as independent shards).

Workload (one "step" = one batched Step of every world): 4096 independent worlds per GPU, body
counts log-uniform in [16, 8192] by seed, each a pyramid, a mixed grid drop or revolute chains
over a circle pile, gravity and friction jittered +-10%, dt 1/60, 8 velocity / 3 position
iterations, sleeping and CCD off. Synthetic scenes from seeded generators; all state stays in
HBM (far larger than the 129 MB L2, so no L2 flush is needed between steps).

Prints one JSON line. `value` is whole-job body-steps/s (bodies x steps / max-over-ranks device
time of the timed steps). `e2e` is the same metric through the public C ABI with host buffers:
every step copies the bodies' forces host->device (pinned) and reads the transforms back, on a
second batch of the same worlds over the same window of steps, through b2g_step_io (one call per
step; its copies overlap the step's kernels); the loop through three separate calls is reported
beside it.
`--impl reference` times the reference algorithm on the host cores instead (the CPU oracle
restatement of the reference's Step, run on all host threads over a bounded sample of worlds).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "box2d-optimized_gb300"))
sys.path.insert(0, str(ROOT / "tests"))

import b2gpu as G  # noqa: E402

METRIC = "batched body-steps/s vs plain GPU b2World::Step; served p50/p99 step latency"
DT, VI, PI = 1.0 / 60.0, 8, 3


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 200 ms while running."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        # nvidia-smi's start-up (NVML initialisation) stalls the driver for a moment: wait for its
        # first sample so that the stall falls before the timed region, not inside it
        t0 = time.time()
        while self.proc and self.proc.poll() is None and time.time() - t0 < 15.0:
            if os.path.getsize(self.path) > 0:
                break
            time.sleep(0.05)
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9 or not f[1].replace(".", "").isdigit():
                    continue
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
                for name, v in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"),
                                   f[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(name)
        except OSError:
            pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def world_params(lib, seed):
    n = C.c_int32()
    gx = C.c_float()
    gy = C.c_float()
    lib.b2g_batch_world_params(seed, C.byref(n), C.byref(gx), C.byref(gy))
    return n.value, gx.value, gy.value


def shard_seeds(rank, world_size, worlds_per_rank, cost=None):
    """World seeds of one rank. The job steps seeds 0 .. world_size * worlds_per_rank - 1 (weak
    scaling: worlds_per_rank per GPU on average), cut into contiguous ranges of about equal total
    cost. cost(seed) is a world's cost; by default each world counts 1 (equal world counts). The
    benchmark passes the world's body count, which its contacts and joints grow with (a world's
    step work is about proportional to bodies + contacts)."""
    total = world_size * worlds_per_rank
    if world_size == 1:
        return list(range(total))
    w = [float(cost(s)) if cost else 1.0 for s in range(total)]
    whole = sum(w)
    acc, cuts = 0.0, [0]
    for s in range(total):
        acc += w[s]
        # a range ends once its running cost passes the next 1/world_size of the whole
        while len(cuts) < world_size and acc >= whole * len(cuts) / world_size:
            cuts.append(s + 1)
    while len(cuts) < world_size:
        cuts.append(total)
    cuts.append(total)
    return list(range(cuts[rank], cuts[rank + 1]))


def reduce_over_ranks(ms_per_step, bodies, device):
    """(max over ranks of the step time, sum over ranks of the bodies) through torch.distributed."""
    import torch  # noqa: PLC0415

    if not torch.distributed.is_initialized() or torch.distributed.get_world_size() == 1:
        return float(ms_per_step), float(bodies)
    t = torch.tensor([float(ms_per_step)], dtype=torch.float64, device=device)
    n = torch.tensor([float(bodies)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    torch.distributed.all_reduce(n, op=torch.distributed.ReduceOp.SUM)
    return float(t.item()), float(n.item())


def serve(lib, dev, seconds, rate, seed0, budget=120 << 30):
    """Poisson stream of rollout requests (32-4096 bodies log-uniform, K ~ U[16, 512]) at `rate`
    requests/s (rate=None: closed loop, the queue is kept full). Returns tick and request
    latencies and the served body-steps/s."""
    import numpy as np  # noqa: PLC0415

    rng = np.random.default_rng(seed0)
    srv = G.Server(lib, device=dev, budget_bytes=budget, max_worlds=4096)
    t0 = time.perf_counter()
    next_arrival = 0.0
    steps_ms, lat, body_steps = [], [], 0
    sizes = {}
    k = 0
    while True:
        now = time.perf_counter() - t0
        if now > seconds:
            break
        if rate is None:
            st = srv.stats()
            while st["queued"] < 8:
                n = int(round(2 ** rng.uniform(5, 12)))
                rid = srv.submit(seed0 + k, n, int(rng.integers(16, 513)))
                sizes[rid] = n
                k += 1
                st["queued"] += 1
        else:
            while next_arrival <= now:
                n = int(round(2 ** rng.uniform(5, 12)))
                rid = srv.submit(seed0 + k, n, int(rng.integers(16, 513)))
                sizes[rid] = n
                k += 1
                next_arrival += rng.exponential(1.0 / rate)
        active, ms = srv.tick()
        if active:
            steps_ms.append(ms)
        for r in srv.poll():
            if r.status == 0:
                lat.append((r.finish_time_s - r.submit_time_s) * 1e3)
                body_steps += r.bodies * r.steps
    elapsed = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    q = lambda a, p: float(np.percentile(a, p)) if len(a) else None  # noqa: E731
    return {"rate_req_s": rate, "seconds": round(elapsed, 1), "completed": st["completed"],
            "throughput_req_s": st["completed"] / elapsed, "body_steps_s": body_steps / elapsed,
            "step_ms_p50": q(steps_ms, 50), "step_ms_p99": q(steps_ms, 99),
            "request_ms_p50": q(lat, 50), "request_ms_p99": q(lat, 99), "ticks": len(steps_ms)}


def query_bench(batch, n_rays):
    """Rays per second (closest hit) and AABB queries per second over all worlds of the batch,
    timed end to end through the C ABI (inputs copied in, results copied out)."""
    import numpy as np  # noqa: PLC0415

    rng = np.random.default_rng(99)
    count = C.c_int32()
    batch.lib.check(batch.lib.b2g_world_count(batch.h, C.byref(count)), "world_count")
    nw = count.value
    worlds = rng.integers(0, nw, size=n_rays).astype(np.int32)
    # rays over a 40 m x 40 m window around each world's origin region (the scenes start near it)
    p1 = rng.uniform([-20.0, -2.0], [20.0, 38.0], size=(n_rays, 2))
    p2 = p1 + rng.uniform(-15.0, 15.0, size=(n_rays, 2))
    rays = np.concatenate([p1, p2], axis=1).astype(np.float32)
    out = (G.RayHit * n_rays)()
    wp = worlds.ctypes.data_as(C.POINTER(C.c_int32))
    rp = rays.ctypes.data_as(C.POINTER(C.c_float))
    batch.lib.check(batch.lib.b2g_raycast_closest(batch.h, wp, rp, n_rays, out), "raycast")  # warm-up
    t0 = time.perf_counter()
    reps = 3
    for _ in range(reps):
        batch.lib.check(batch.lib.b2g_raycast_closest(batch.h, wp, rp, n_rays, out), "raycast")
    ray_s = (time.perf_counter() - t0) / reps
    hit = int((np.frombuffer(out, dtype=np.int32).reshape(n_rays, 6)[:, 0] >= 0).sum())
    nq = n_rays // 4
    lo = rng.uniform([-20.0, -2.0], [20.0, 38.0], size=(nq, 2))
    boxes = np.concatenate([lo, lo + rng.uniform(0.2, 3.0, size=(nq, 2))], axis=1).astype(np.float32)
    qw = worlds[:nq].copy()
    counts = (C.c_int32 * nq)()
    cap = 64 * nq
    found = (C.c_int32 * cap)()
    total = C.c_int64()
    args_q = (batch.h, qw.ctypes.data_as(C.POINTER(C.c_int32)), boxes.ctypes.data_as(C.POINTER(C.c_float)), nq,
              counts, found, cap, C.byref(total))
    batch.lib.check(batch.lib.b2g_query_aabb(*args_q), "query_aabb")
    t0 = time.perf_counter()
    for _ in range(reps):
        batch.lib.check(batch.lib.b2g_query_aabb(*args_q), "query_aabb")
    q_s = (time.perf_counter() - t0) / reps
    return {"rays": n_rays, "raycasts_per_s": n_rays / ray_s, "ray_hit_fraction": hit / n_rays,
            "aabb_queries": nq, "aabb_queries_per_s": nq / q_s, "fixtures_reported_per_query": total.value / nq,
            "timing": "end to end through the C ABI with host buffers, mean of 3 calls after a warm-up call"}


def build_batch(lib, seeds, device, allow_sleep=False):
    batch = G.Batch(lib, device=device)
    nb = 0
    for s in seeds:
        n, gx, gy = world_params(lib, s)
        w = batch.add_world(gx, gy)
        batch.set_flags(w, allow_sleep=allow_sleep, warm_starting=True, continuous=False)
        c = batch.scene(w, G.SCENE_BATCH_WORLD, seed=s, n=n)
        nb += c[0]
    return batch, nb


def sleep_bench(lib, dev, seeds, settle, steps, cpu):
    """Island sleep on: a sample of the same worlds settles for `settle` steps with sleeping
    allowed, then `steps` steps are timed (CUDA events); the same sample with sleeping off is
    timed over the same window, and, with `cpu`, the CPU oracle steps the sample with sleeping
    allowed (the reference's default) over the same window on all host threads."""
    out = {}
    for sleep in (True, False):
        batch, nb = build_batch(lib, seeds, dev, allow_sleep=sleep)
        batch.step_timed(settle, DT, VI, PI)
        ms = batch.step_timed(steps, DT, VI, PI)
        asleep = 0
        for w in range(len(seeds)):
            asleep += sum(1 for r in batch.bodies(w) if r.type != 0 and not r.flags & G.BODY_AWAKE)
        batch.set_graphs(False)
        batch.step(DT, VI, PI)  # one eager step for the per-phase breakdown
        p = batch.profile()
        out["on" if sleep else "off"] = {"value": nb * steps / (ms / 1e3), "ms_per_step": ms / steps,
                                         "asleep_fraction": asleep / nb,
                                         "breakdown_ms": {"collide": p.collide, "solve": p.solve,
                                                          "broadphase": p.broadphase}}
        batch.close()
    res = {"value": out["on"]["value"], "unit": "body-steps/s", "ms_per_step": out["on"]["ms_per_step"],
           "asleep_fraction": out["on"]["asleep_fraction"], "sleep_off_value": out["off"]["value"],
           "breakdown_ms": out["on"]["breakdown_ms"], "sleep_off_breakdown_ms": out["off"]["breakdown_ms"],
           "sample": f"{len(seeds)} of the worlds ({nb} bodies), steps {settle + 1}-{settle + steps}"}
    if cpu:
        import oracle_bind as ob  # noqa: PLC0415 - CPU baseline leg only

        threads = os.cpu_count() or 1
        orc = ob.Oracle()
        worlds, _ = oracle_batch(orc, seeds, sleep=True)
        hs = (C.c_void_p * len(worlds))(*[w.h for w in worlds])
        orc.orc_worlds_step_parallel(hs, len(worlds), DT, VI, PI, settle, threads)
        secs = orc.orc_worlds_step_parallel(hs, len(worlds), DT, VI, PI, steps, threads)
        res["cpu_baseline"] = {"value": nb * steps / secs, "unit": "body-steps/s", "cores": threads, "kind": "port",
                               "sample": "the same worlds and window, sleeping allowed"}
    return res


def ccd_bench(lib, dev, n_worlds, lanes, steps, cpu):
    """Continuous collision (b2World::SolveTOI on the device): `n_worlds` bullets worlds (`lanes`
    bullets fired or thrown at boxes each, seeds 1..n) stepped `steps` steps from the start, when
    the impacts happen, with continuous physics on and, for comparison, off; the TOI stage's share
    of one more step; with `cpu`, the CPU oracle over the same worlds and window on all host
    threads."""
    out = {}
    for cont in (True, False):
        batch = G.Batch(lib, device=dev)
        nb = 0
        for i in range(n_worlds):
            w = batch.add_world(0.0, -10.0)
            batch.set_flags(w, allow_sleep=False, warm_starting=True, continuous=cont)
            nb += batch.scene(w, G.SCENE_BULLETS, seed=i + 1, n=lanes, p0=0.0, p1=0.0)[0]
        batch.step_timed(1, DT, VI, PI)  # upload and first contacts
        ms = batch.step_timed(steps, DT, VI, PI)
        batch.set_graphs(False)
        batch.step(DT, VI, PI)  # one eager step for the TOI kernel's time
        p = batch.profile()
        out[cont] = {"ms": ms / steps, "toi_ms": p.solve_toi, "nb": nb,
                     "breakdown": {"step": p.step, "collide": p.collide, "solve": p.solve,
                                   "pair_updates_and_toi": p.broadphase, "toi_kernel": p.solve_toi}}
        batch.close()
    nb = out[True]["nb"]
    res = {"value": nb * steps / (out[True]["ms"] * steps / 1e3), "unit": "body-steps/s",
           "ms_per_step": out[True]["ms"], "continuous_off_ms_per_step": out[False]["ms"],
           "toi_stage_ms": out[True]["toi_ms"],
           "breakdown_ms": out[True]["breakdown"], "continuous_off_breakdown_ms": out[False]["breakdown"],
           "workload": f"{n_worlds} bullets worlds of {lanes} lanes ({nb} bodies), steps 2-{steps + 1}, "
                       "continuous physics on (the step's graph holds SolveTOI and a second pair update)"}
    if cpu:
        import oracle_bind as ob  # noqa: PLC0415 - CPU baseline leg only

        threads = os.cpu_count() or 1
        orc = ob.Oracle()
        worlds = [ob.OracleWorld(orc, (0.0, -10.0), scene=(G.SCENE_BULLETS, i + 1, lanes, 0.0, 0.0), continuous=True)
                  for i in range(n_worlds)]
        hs = (C.c_void_p * len(worlds))(*[w.h for w in worlds])
        orc.orc_worlds_step_parallel(hs, len(worlds), DT, VI, PI, 1, threads)
        secs = orc.orc_worlds_step_parallel(hs, len(worlds), DT, VI, PI, steps, threads)
        res["cpu_baseline"] = {"value": nb * steps / secs, "unit": "body-steps/s", "cores": threads, "kind": "port",
                               "sample": "the same worlds and window, continuous physics on"}
    return res


# The single-world configurations: (name, scene kind, seed, n, p0, velocity / position
# iterations, steps, workload).
LARGE_CONFIGS = [
    ("pyramid_210", G.SCENE_PYRAMID, 1, 20, 1.0, 8, 3, 256,
     "20-row box pyramid (210 boxes, density 1, friction 0.6) on a 40 m edge, 8/3 iterations, 256 steps"),
    ("mixed_20000", G.SCENE_MIXED_DROP, 1, 20000, 0.0, 8, 3, 512,
     "single large world: 20 000 boxes / circles / 3-8-gons dropped from a 200 x 400 m grid into a U, 8/3, 512 steps"),
    ("chains_2000x20_pile_10000", G.SCENE_CHAINS, 1, 2000, 10000.0, 10, 4, 256,
     "2 000 chains of 20 boxes on revolute joints (limits, motors) over 10 000 circles, 10/4 iterations, 256 steps"),
]


def large_worlds(lib, dev, cpu, cpu_steps=16):
    """Each single-world configuration stepped alone for its full step count (CUDA graphs, device
    time by CUDA events): ms per step over the whole rollout and over its last `cpu_steps`
    steps, with worlds above 8192 bodies solved by a thread-block cluster (the default) and, for
    comparison, by one CTA. With `cpu`, the CPU oracle (restatement of the reference's Step, one
    host thread, like the reference) is loaded with the GPU's state before the last `cpu_steps`
    steps and times those same steps: a bounded sample of the settled workload."""
    out = {}
    for name, kind, seed, n, p0, vi, pi, steps, desc in LARGE_CONFIGS:
        res = {"workload": desc}
        big = None
        for ctas in (-1, 1):
            b = G.Batch(lib, device=dev)
            b.cluster_solve(ctas)
            w = b.add_world(0.0, -10.0)
            b.set_flags(w, allow_sleep=False, warm_starting=True, continuous=False)
            counts = b.scene(w, kind, seed=seed, n=n, p0=p0, p1=0.6)
            big = counts[0] > 8192  # solved by a thread-block cluster by default
            if ctas == 1 and not big:
                b.close()
                break
            head = b.step_timed(steps - cpu_steps, DT, vi, pi)
            if ctas == -1 and cpu:
                import oracle_bind as ob  # noqa: PLC0415 - CPU baseline leg only

                ow = ob.OracleWorld(ob.Oracle(), (0.0, -10.0), b.bodies(w), b.fixtures(w), b.joints(w),
                                    b.contacts(w), inv_dt0=1.0 / DT)
                secs = ow.step(cpu_steps, DT, vi, pi)
                res["cpu_baseline"] = {"value": counts[0] * cpu_steps / secs, "unit": "body-steps/s", "cores": 1,
                                       "kind": "port", "ms_per_step": secs * 1e3 / cpu_steps,
                                       "sample": f"steps {steps - cpu_steps + 1}-{steps} from the GPU's state, one thread"}
                ow.close()
            tail = b.step_timed(cpu_steps, DT, vi, pi)
            b.set_graphs(False)
            b.step(DT, vi, pi)
            p = b.profile()
            key = "cluster" if ctas == -1 else "one_cta"
            res[key] = {"ms_per_step": (head + tail) / steps, "ms_per_step_last": tail / cpu_steps,
                        "body_steps_per_s": counts[0] * steps / ((head + tail) / 1e3),
                        "eager_step_after_ms": {"collide": p.collide, "solve": p.solve, "broadphase": p.broadphase,
                                                "step": p.step},
                        "touching_at_end": p.touching, "joints": p.joints, "colors_max": p.colors_max}
            if ctas == -1:
                res["bodies"] = counts[0]
                res["cluster"]["ctas_per_world"] = b.cluster_ctas() if big else 1
            b.close()
        out[name] = res
    return out


def solve_traffic(sb):
    """DRAM bytes of the solver launches of one step, from the ncu capture of the settled
    384-world case committed in profiles/k_solve_dram.json, scaled to this step by algorithmic
    bytes (traffic grows with the solver's work); None when the capture is absent."""
    try:
        with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "profiles", "k_solve_dram.json")) as f:
            d = json.load(f)
        return d["dram_bytes_per_step"] * sb / d["solve_bytes_per_step"]
    except (OSError, KeyError, ValueError, ZeroDivisionError):
        return None


def step_bytes(nb, nf, np_, nc, nj, vi=VI, pi=PI):
    """Algorithmic bytes of one Step (fixed accounting): bodies 96/body, broadphase 144/fixture +
    8/pair, per touching contact 524 + 192 vi + 144 pi, per joint 160 + 128 vi + 96 pi."""
    return 96 * nb + 144 * nf + 8 * np_ + nc * (524 + 192 * vi + 144 * pi) + nj * (160 + 128 * vi + 96 * pi)


def solve_bytes(nb, nc, nj, vi=VI, pi=PI):
    """Algorithmic bytes of the solver kernel alone: body state read/write (64/body), contact
    prepare 208 + store 16, velocity 192 vi and position 144 pi per touching contact, joints."""
    return 64 * nb + nc * (208 + 16 + 192 * vi + 144 * pi) + nj * (160 + 128 * vi + 96 * pi)


def oracle_batch(orc, seeds, sleep=False):
    """The batched workload's worlds `seeds`, built by the CPU oracle's own scene builder (no
    engine library involved); returns (worlds, bodies)."""
    import oracle_bind as ob  # noqa: PLC0415 - CPU baseline and reference arm only

    worlds, nb = [], 0
    for s in seeds:
        n, gx, gy = orc.batch_world_params(s)
        ow = ob.OracleWorld(orc, (gx, gy), scene=(G.SCENE_BATCH_WORLD, s, n, 0.0, 0.0))
        if sleep:
            ow.set_sleep(True)
        nb += ow.counts[0]  # dynamic bodies, as the GPU arm counts them
        worlds.append(ow)
    return worlds, nb


def cpu_sample(seeds, warmup, steps, threads):
    """Steps the CPU oracle (restatement of the reference Step) over a sample of worlds."""
    import oracle_bind as ob  # noqa: PLC0415 - CPU baseline leg only

    orc = ob.Oracle()
    worlds, nb = oracle_batch(orc, seeds)
    hs = (C.c_void_p * len(worlds))(*[w.h for w in worlds])
    orc.orc_worlds_step_parallel(hs, len(worlds), DT, VI, PI, warmup, threads)  # untimed, like the GPU warm-up
    secs = orc.orc_worlds_step_parallel(hs, len(worlds), DT, VI, PI, steps, threads)
    return nb * steps / secs, nb, secs


def run_reference(args, rank):
    """The reference arm: the reference's Step algorithm (the CPU oracle's restatement, pinned
    to the reference's own code) on all host threads, over the same worlds, warm-up and timed
    steps as the GPU arm. Worlds are built by the oracle's scene builder, so this arm loads no
    engine library."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    import oracle_bind as ob  # noqa: PLC0415 - the reference arm runs the oracle port

    orc = ob.Oracle()
    t0 = time.time()
    worlds, nb = oracle_batch(orc, list(range(args.worlds)))
    build_s = time.time() - t0
    hs = (C.c_void_p * len(worlds))(*[w.h for w in worlds])
    orc.orc_worlds_step_parallel(hs, len(worlds), DT, VI, PI, args.warmup, threads)
    secs = orc.orc_worlds_step_parallel(hs, len(worlds), DT, VI, PI, args.steps, threads)
    value = nb * args.steps / secs
    sample = (f"all {args.worlds} worlds ({nb} bodies), steps {args.warmup + 1}-{args.warmup + args.steps} after "
              f"{args.warmup} untimed, {threads} threads; built in {build_s:.1f} s by the oracle's scene builder")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "body-steps/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": secs * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"batched {args.worlds} worlds per GPU, 16-8192 bodies log-uniform (pyramid / "
                               f"mixed drop / chains), 8/3 iterations, dt 1/60",
                   "worlds": args.worlds, "bodies": nb, "l2": "state larger than L2 (no flush needed)"},
        "cpu_baseline": {"value": value, "unit": "body-steps/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "body-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args, rank, world_size):
    import torch  # noqa: PLC0415 - device selection and pinned host buffers

    lib = G.Lib()
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    seeds = shard_seeds(rank, world_size, args.worlds, cost=lambda s: world_params(lib, s)[0])
    # autotune the solver's threads per world on a settled sample of the same worlds (every 8th);
    # results do not depend on the choice, so the timed batch just takes it
    threads, tune_s = None, 0.0
    if not args.no_autotune:
        t0 = time.time()
        sample, _ = build_batch(lib, seeds[::8], dev)
        sample.step_timed(100, DT, VI, PI)
        threads, _ = sample.autotune(steps=3, dt=DT, vi=VI, pi=PI)
        sample.close()
        tune_s = time.time() - t0
    t0 = time.time()
    batch, nb = build_batch(lib, seeds, dev)
    if threads:
        batch.solver_threads(threads)
    batch_threads = batch.solver_threads()
    build_s = time.time() - t0
    # warm-up (includes the first upload and contact creation)
    batch.step_timed(args.warmup, DT, VI, PI)
    prof_w = batch.profile()
    if world_size > 1:
        torch.distributed.barrier()
    touching0 = batch.profile().touching_total
    with ClockSampler(dev) as clocks:
        ms = batch.step_timed(args.steps, DT, VI, PI)
    prof = batch.profile()
    touching_window = prof.touching_total - touching0
    ms_per_step = ms / args.steps
    ms_per_step_own = ms_per_step
    ms_per_step, nb_all = reduce_over_ranks(ms_per_step_own, nb, f"cuda:{dev}")
    _, touching_all = reduce_over_ranks(ms_per_step_own, touching_window, f"cuda:{dev}")
    value = nb_all / (ms_per_step / 1e3)
    # contact-constraint iterations: solver contacts of every timed step x (velocity + position
    # iterations), per second of the whole job
    contact_iters = touching_all * (VI + PI) / (ms_per_step * args.steps / 1e3)

    # end to end through the C ABI with pinned host buffers: forces in, transforms out, every step,
    # on a second batch of the same worlds over the same window of steps as the timed region (the
    # later steps of a rollout cost more, so a later window would not be the same workload)
    nbody = prof.bodies
    forces = torch.zeros((nbody, 4), dtype=torch.float32).pin_memory()
    xf_out = torch.empty((nbody, 4), dtype=torch.float32).pin_memory()
    n_out = C.c_int64()
    e2e_steps = args.steps
    eb, _ = build_batch(lib, seeds, dev)
    if threads:
        eb.solver_threads(threads)
    eb.step_timed(args.warmup, DT, VI, PI)
    torch.cuda.synchronize()
    # b2g_step_io: the forces' copy overlaps the contact update and the transforms' copy the
    # closing broadphase; the call returns after the step and both copies
    t1 = time.perf_counter()
    for _ in range(e2e_steps):
        lib.check(lib.b2g_step_io(eb.h, DT, VI, PI, C.c_void_p(forces.data_ptr()), nbody,
                                  C.c_void_p(xf_out.data_ptr()), nbody, C.byref(n_out)), "step_io")
    e2e_s = time.perf_counter() - t1
    # the same loop through the three separate calls (b2g_batch_set_forces, b2g_step,
    # b2g_batch_read_states), over the next e2e_steps steps: each copy then runs alone
    phase = [0.0, 0.0, 0.0]  # host time in set_forces, step, read_states
    for _ in range(e2e_steps):
        ta = time.perf_counter()
        lib.check(lib.b2g_batch_set_forces(eb.h, forces.data_ptr(), nbody), "set_forces")
        tb = time.perf_counter()
        lib.check(lib.b2g_step(eb.h, DT, VI, PI, None), "step")
        tc = time.perf_counter()
        lib.check(lib.b2g_batch_read_states(eb.h, C.cast(xf_out.data_ptr(), C.POINTER(C.c_float)), None,
                                            nbody, C.byref(n_out)), "read_states")
        td = time.perf_counter()
        phase[0] += tb - ta
        phase[1] += tc - tb
        phase[2] += td - tc
    eb.close()
    e2e_value = nb * e2e_steps / e2e_s * world_size

    # the same batch after it has settled: ms/step and body-steps/s over `settled_steps` steps
    # starting at step settle_at + 1 (graph replay, CUDA events), with the touching contacts
    # solved per step there (piles have formed; the driver's short window is mostly free fall)
    settled = None
    if args.settled_at > 0:
        batch.step_timed(max(0, args.settled_at - args.warmup - args.steps), DT, VI, PI)
        t0c = batch.profile().touching_total
        sms = batch.step_timed(args.settled_steps, DT, VI, PI)
        tch = (batch.profile().touching_total - t0c) / args.settled_steps
        sms_max, _ = reduce_over_ranks(sms / args.settled_steps, nb, f"cuda:{dev}")
        first = max(args.settled_at, args.warmup + args.steps) + 1
        settled = {"value": nb_all / (sms_max / 1e3), "unit": "body-steps/s", "ms_per_step": sms_max,
                   "steps": f"{first}-{first + args.settled_steps - 1}", "touching_per_step_per_gpu": tch,
                   "contact_constraint_iterations_per_s": tch * (VI + PI) * world_size / (sms_max / 1e3)}

    # world queries on the settled batch: closest-hit ray casts and AABB queries, end to end
    # through the C ABI (host buffers in and out), seeded rays over each world's extent
    queries = None
    if args.rays > 0:
        queries = query_bench(batch, args.rays)

    # island sleep on a sample of the same worlds (settled, then timed), beside sleep off and the CPU
    sleep = None
    if args.sleep_worlds > 0:
        ss = seeds[:: max(1, len(seeds) // args.sleep_worlds)][: args.sleep_worlds]
        sleep = sleep_bench(lib, dev, ss, args.sleep_settle, max(3, args.steps // 2),
                            rank == 0 and world_size == 1 and not args.no_cpu)

    # continuous collision on its own workload (the batched worlds above run without it)
    ccd = None
    if args.ccd_worlds > 0:
        ccd = ccd_bench(lib, dev, args.ccd_worlds, 12, 30, rank == 0 and world_size == 1 and not args.no_cpu)

    # per-phase breakdown: one eager (non-graph) step after the timed region
    lib.b2g_batch_set_graphs(batch.h, 0)
    batch.step(DT, VI, PI)
    lib.b2g_batch_set_graphs(batch.h, 1)
    prof = batch.profile()

    # plain per-world GPU Step: a sample of the same worlds, each stepped alone in its own batch
    # (one world per launch sequence, no graph), over the same rollout window
    plain = None
    if not args.no_plain:
        ps = seeds[:: max(1, len(seeds) // args.plain_worlds)][: args.plain_worlds]
        p_bodies, p_ms = 0, 0.0
        for s in ps:
            one, nb1 = build_batch(lib, [s], dev)
            lib.b2g_batch_set_graphs(one.h, 0)
            one.step_timed(args.warmup, DT, VI, PI)
            p_ms += one.step_timed(args.steps, DT, VI, PI)
            p_bodies += nb1
            one.close()
        pv = p_bodies * args.steps / (p_ms / 1e3)
        plain = {"value": pv, "unit": "body-steps/s", "sample": f"{len(ps)} of the worlds ({p_bodies} bodies), "
                 f"each stepped alone, steps {args.warmup + 1}-{args.warmup + args.steps}",
                 "ms_per_world_step": p_ms / (len(ps) * args.steps)}

    # roofline of the dominant kernel (the per-world solver CTA), from the eager step
    peak, peak_kind = _peaks()
    sb = solve_bytes(prof.bodies, prof.touching, prof.joints)
    achieved = sb / (prof.solve / 1e3) / 1e9 if prof.solve > 0 else None
    step_b = step_bytes(prof.bodies, prof.fixtures, prof.contacts, prof.touching, prof.joints)

    # served: closed-loop saturation, then a Poisson stream at 70% of it
    served = None
    if rank == 0 and not args.no_serve:
        sat = serve(lib, dev, args.serve_seconds, None, 1_000_000)
        rate = 0.7 * sat["throughput_req_s"]
        at70 = serve(lib, dev, args.serve_seconds, rate, 2_000_000)
        served = {"saturation": sat, "at_70pct": at70,
                  "step_ms_p50": at70["step_ms_p50"], "step_ms_p99": at70["step_ms_p99"],
                  "request_ms_p50": at70["request_ms_p50"], "request_ms_p99": at70["request_ms_p99"],
                  "workload": "Poisson rollout requests, 32-4096 bodies log-uniform, K ~ U[16,512] steps, "
                              "120 GB HBM budget; rate = 0.7 x closed-loop saturation throughput"}

    # the single-world configurations (20-row pyramid, 20 000-body drop, 2 000 chains over a pile)
    large = None
    if rank == 0 and not args.no_large:
        large = large_worlds(lib, dev, world_size == 1 and not args.no_cpu)

    line = None
    if rank == 0:
        cpu = None
        if world_size == 1 and not args.no_cpu:
            threads = os.cpu_count() or 1
            cpu_seeds = seeds[:: max(1, len(seeds) // args.cpu_worlds)][: args.cpu_worlds]
            v, cnb, secs = cpu_sample(cpu_seeds, args.warmup, args.steps, threads)
            cpu = {"value": v, "unit": "body-steps/s", "cores": threads, "kind": "port",
                   "sample": f"{len(cpu_seeds)} of the worlds ({cnb} bodies), steps {args.warmup + 1}-"
                             f"{args.warmup + args.steps} of the same rollout, {secs:.1f} s on {threads} threads"}
        # own kernels per step (CUB's sort and scan kernels not counted): collide, the solver's
        # setup and iteration kernels of the four CTA size classes and the cluster kernel of the
        # largest worlds (9), aabb, refit init, lbvh bounds, pair count, world contact ranges, pair
        # emit, diff, commit, clear forces = 19 on a step whose closing broadphase refits the kept
        # trees; a full rebuild (every 32nd broadphase) launches world bounds, morton and lbvh
        # init / internal instead of the refit init (+3)
        kernels_per_step = 19
        full_builds = args.steps // 32
        line = {
            "metric": METRIC, "value": value, "unit": "body-steps/s", "n_gpus": world_size, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"batched {args.worlds} worlds per GPU, 16-8192 bodies log-uniform (pyramid / "
                                   f"mixed drop / chains), 8/3 iterations, dt 1/60",
                       "worlds": args.worlds * world_size, "bodies": int(nb_all), "fixtures_per_gpu": prof.fixtures,
                       "contacts_per_gpu": prof.contacts, "touching_per_gpu": prof.touching,
                       "joints_per_gpu": prof.joints, "l2": "state larger than L2 (no flush needed)",
                       "parallelism": f"{world_size} independent world shards", "build_s": round(build_s, 1),
                       "solver_threads_per_class": batch_threads,
                       "autotune": (f"threads per world for size classes <=64/512/2048/8192/more bodies, tuned on "
                                    f"every 8th world after 100 steps in {tune_s:.1f} s") if threads else "off"},
            "breakdown_ms": {"collide": prof.collide, "solve": prof.solve, "broadphase": prof.broadphase,
                             "step": prof.step},
            "step_bytes": step_b, "step_gbs": step_b / (ms_per_step / 1e3) / 1e9,
            "roofline": {"kernel": "k_solve", "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": (achieved / peak) if achieved else None, "traffic": solve_traffic(sb),
                         "peak_kind": f"{peak_kind} hbm_gbs", "bytes_per_launch": sb},
            "cpu_baseline": cpu,
            "served": served,
            "plain_gpu": plain,
            "batched_over_plain": (value / world_size / plain["value"]) if plain else None,
            "e2e": {"value": e2e_value, "unit": "body-steps/s", "h2d_bytes_per_step": 16 * nbody,
                    "d2h_bytes_per_step": 16 * nbody, "steps": e2e_steps, "call": "b2g_step_io",
                    "separate_calls": {
                        "value": nb * e2e_steps / sum(phase) * world_size,
                        "window": f"the next {e2e_steps} steps",
                        "host_ms_per_step": {k: round(v * 1e3 / e2e_steps, 3)
                                             for k, v in zip(("set_forces", "step", "read_states"), phase)}}},
            "gpu_launches": kernels_per_step * args.steps + 3 * full_builds,
            "contact_constraint_iterations_per_s": contact_iters,
            "settled": settled,
            "large_worlds": large,
            "queries": queries,
            "sleep": sleep,
            "continuous": ccd,
            "clocks": clocks.summary(),
        }
    batch.close()
    if line:
        print(json.dumps(line), flush=True)


def profile_window(args):
    """Profiling case for ncu: builds the batch, settles it for --settle steps (CUDA graphs), then
    runs two eager steps inside the NVTX range "profile" (select them with
    `ncu --nvtx --nvtx-include profile/`). Prints the state sizes; no timing is reported."""
    import torch  # noqa: PLC0415 - NVTX ranges

    lib = G.Lib()
    batch, nb = build_batch(lib, shard_seeds(0, 1, args.worlds), 0)
    batch.step_timed(args.settle, DT, VI, PI)
    lib.b2g_batch_set_graphs(batch.h, 0)
    torch.cuda.nvtx.range_push("profile")
    for _ in range(2):
        batch.step(DT, VI, PI)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    p = batch.profile()
    print(json.dumps({"profile_window": {"worlds": args.worlds, "settle_steps": args.settle, "bodies": nb,
                                         "fixtures": p.fixtures, "contacts": p.contacts, "touching": p.touching,
                                         "joints": p.joints, "colors_max": p.colors_max}}))
    batch.close()


def profile_large(args):
    """Profiling case for ncu on one single-world configuration (--profile-large NAME): steps it
    --settle steps (CUDA graphs), then two eager steps inside the NVTX range "profile"."""
    import torch  # noqa: PLC0415 - NVTX ranges

    cfg = {c[0]: c for c in LARGE_CONFIGS}[args.profile_large]
    _, kind, seed, n, p0, vi, pi, _, _ = cfg
    lib = G.Lib()
    b = G.Batch(lib, device=0)
    w = b.add_world(0.0, -10.0)
    b.set_flags(w, allow_sleep=False, warm_starting=True, continuous=False)
    counts = b.scene(w, kind, seed=seed, n=n, p0=p0, p1=0.6)
    b.step_timed(args.settle, DT, vi, pi)
    b.set_graphs(False)
    torch.cuda.nvtx.range_push("profile")
    for _ in range(2):
        b.step(DT, vi, pi)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    p = b.profile()
    print(json.dumps({"profile_large": {"config": args.profile_large, "settle_steps": args.settle, "bodies": counts[0],
                                        "touching": p.touching, "joints": p.joints, "colors_max": p.colors_max,
                                        "ctas_per_world": b.cluster_ctas()}}))
    b.close()


def serve_ticks(args):
    """Tick-driven served measurement (also the ncu case for served steps): a Poisson number of
    rollout requests (mean --serve-per-tick; 32-4096 bodies log-uniform, K ~ U[16, 512]) arrives
    before each of --serve-ticks ticks, so the load does not depend on the tick's own duration
    (as it would under a profiler). Prints the percentiles of the served step and of the device
    step and its phases over the last two thirds of the ticks."""
    import numpy as np  # noqa: PLC0415

    lib = G.Lib()
    rng = np.random.default_rng(2_000_000)
    srv = G.Server(lib, device=0, budget_bytes=120 << 30, max_worlds=4096)
    bh = C.c_void_p()
    lib.check(lib.b2g_server_batch(srv.h, C.byref(bh)), "b2g_server_batch")
    prof = G.Profile()
    rec, k = [], 0
    for _ in range(args.serve_ticks):
        for _ in range(rng.poisson(args.serve_per_tick)):
            n = int(round(2 ** rng.uniform(5, 12)))
            srv.submit(2_000_000 + k, n, int(rng.integers(16, 513)))
            k += 1
        active, ms = srv.tick()
        lib.b2g_profile_get(bh, C.byref(prof))
        rec.append((ms, active, prof.step, prof.collide, prof.solve, prof.broadphase))
        list(srv.poll())
    srv.close()
    a = np.array(rec[len(rec) // 3:])
    pct = lambda x: [round(float(np.percentile(x, q)), 3) for q in (50, 90, 99)]  # noqa: E731
    print(json.dumps({"serve_ticks": {"per_tick": args.serve_per_tick, "ticks": len(rec),
                                      "active_p50_p90_p99": pct(a[:, 1]), "step_ms": pct(a[:, 0]),
                                      "gpu_step_ms": pct(a[:, 2]), "collide_ms": pct(a[:, 3]),
                                      "solve_ms": pct(a[:, 4]), "broadphase_ms": pct(a[:, 5])}}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=256)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--worlds", type=int, default=4096)
    ap.add_argument("--ref-worlds", type=int, default=128)
    ap.add_argument("--cpu-worlds", type=int, default=128)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--plain-worlds", type=int, default=32)
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--serve-seconds", type=float, default=12.0)
    ap.add_argument("--no-autotune", action="store_true", help="keep the default solver threads per world")
    ap.add_argument("--settled-at", type=int, default=260, help="step after which the settled window starts (0: skip)")
    ap.add_argument("--settled-steps", type=int, default=16)
    ap.add_argument("--no-large", action="store_true", help="skip the single-world configurations")
    ap.add_argument("--rays", type=int, default=1 << 20, help="rays of the world-query measurement (0: skip)")
    ap.add_argument("--sleep-worlds", type=int, default=256, help="worlds of the island-sleep measurement (0: skip)")
    ap.add_argument("--sleep-settle", type=int, default=480, help="steps before the island-sleep window")
    ap.add_argument("--ccd-worlds", type=int, default=4096, help="worlds of the continuous-collision measurement (0: skip)")
    ap.add_argument("--profile-window", action="store_true",
                    help="ncu case: settle --settle steps, then 2 steps inside the NVTX range 'profile'")
    ap.add_argument("--settle", type=int, default=250)
    ap.add_argument("--profile-large", default="", help="ncu case: one single-world configuration by name "
                    "(pyramid_210, mixed_20000, chains_2000x20_pile_10000), settled, 2 steps in NVTX 'profile'")
    ap.add_argument("--serve-ticks", type=int, default=0,
                    help="tick-driven served measurement over this many ticks (see serve_ticks)")
    ap.add_argument("--serve-per-tick", type=float, default=1.77)
    args = ap.parse_args()
    if args.profile_window:
        profile_window(args)
        return
    if args.profile_large:
        profile_large(args)
        return
    if args.serve_ticks > 0:
        serve_ticks(args)
        return
    args.warmup = max(args.warmup, 3)
    rank = int(os.environ.get("RANK", "0"))
    world_size = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        run_reference(args, rank)
        return
    if world_size > 1:
        import torch  # noqa: PLC0415

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        torch.distributed.init_process_group("nccl")
    run_ours(args, rank, world_size)
    if world_size > 1:
        import torch  # noqa: PLC0415

        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
