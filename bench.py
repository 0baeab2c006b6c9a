#!/usr/bin/env python
"""Benchmark of the GPU rigid-body step (JBullet's stepSimulation pipeline) on one GB300.

Workload (default): 100,000 bodies (40% spheres, 40% boxes, 20% capsules) dropped on a static
plane, dt = 1/120, 10 PGS iterations; a "step" is one internal single step of the whole
pipeline (gravity, predict, aabbs, pairs, narrowphase, islands, solver, integrate,
activation) over all bodies.  Metric: body-steps/s.

Every measurement starts from the same point of the drop: the world is stepped --settle
steps from rest (untimed; 300 by default, when most bodies have reached the pile), then W
warm-up steps, then the K timed steps.  The timed window is steps settle+W .. settle+W+K-1.

  value  device-timed throughput: K steps through jbgpu_world_step with the world resident in
         HBM (per-step working set of bodies, pairs, manifolds and solver rows exceeds the
         129 MB L2; no separate flush), timed by CUDA events on the world's stream.  The
         per-phase breakdown comes from a second run of the same steps with phase event marks
         (the marks themselves cost time, so they stay out of the timed run).
  e2e    the same K steps through the reference-facing call jbgpu_world_step_simulation (the
         W warm-up steps also go through it, which primes its time accumulator), each step with
         a host->device upload of per-body forces (RigidBody.applyCentralForce) and a
         device->host read of all body transforms (MotionState synchronisation), both from
         pinned host memory; the steps counted are the executed ones, min(returned, maxSubSteps).
  roofline  the phase with the largest device time (CUDA events on the world's stream),
         algorithmic bytes from the per-step counters / measured phase time vs the measured
         HBM copy bandwidth; traffic = the DRAM bytes of one ncu capture of that kernel,
         scaled to the window's own algorithmic bytes per launch (profiles/traffic.json).
  cpu_baseline  the CPU restatement of the reference (oracle, one core, the reference's island
         solver order) continued for --cpu-window steps from GPU snapshots inside the timed
         window.
  other_workloads  the 1,000-box, 20,000-hull and 4,096-world workloads measured beside the
         headline in the same run (device-timed from a settled point, with their phases).

--impl reference times that CPU restatement on the same window: the GPU steps the world to
the window's first step (untimed set-up), the oracle takes over its state and manifolds and
is timed alone for K steps (within a time budget).
Multi-GPU: one process per GPU (torchrun).  A batched workload (independent worlds) is split
by world across the ranks (jbgpu.shard: greedy by N_w^2, no collective on the data path); a
single-world workload runs an independent replica per rank.  Weak scaling; rank 0 prints the
line.
"""
import argparse
import json
import os
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "libgdx-jbullet_gb300"))

import numpy as np  # noqa: E402

METRIC = "body-steps/s @100k bodies"
UNIT = "body-steps/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=100)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="mixed_100k")
    p.add_argument("--seed", type=int, default=0)
    p.add_argument("--settle", type=int, default=300, help="untimed steps from rest before the warm-up")
    p.add_argument("--shard-cost", default="square", choices=["square", "linear"],
                   help="per-world cost used to split a batched workload across ranks")
    p.add_argument("--cpu-window", type=int, default=10)
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--solver-parts", type=int, default=0, help="jbgpu_config.solver_parts (0: automatic)")
    p.add_argument("--solver-threads", type=int, default=0, help="jbgpu_config.solver_threads (0: 256)")
    p.add_argument("--solver-smem-bodies", type=int, default=0, help="jbgpu_config.solver_smem_bodies (0: 2048)")
    p.add_argument("--autotune", action="store_true", help="choose the solver knobs with jbgpu.autotune first")
    p.add_argument("--rebuild-interval", type=int, default=None, help="jbgpu_config.broadphase_rebuild_interval")
    p.add_argument("--ref-seconds", type=float, default=120.0, help="time budget of the reference arm's timed steps")
    p.add_argument("--no-learned", action="store_true", help="skip the learned-warm-start comparison")
    p.add_argument("--no-others", action="store_true", help="skip the 1k-box, 20k-hull and 4,096-world workloads")
    p.add_argument("--learned-cap", type=int, default=12000, help="iteration cap of the world-residual comparison")
    p.add_argument("--no-rays", action="store_true", help="skip the rayTest batch measurement")
    p.add_argument("--sweeps", type=int, default=4096, help="convexSweepTest sweeps per measured batch (0: skip)")
    p.add_argument("--graph", type=int, default=1, help="1: replay the step as CUDA graphs (jbgpu_world_set_graph), 0: launches")
    p.add_argument("--rays", type=int, default=1 << 20, help="rays per rayTest batch")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Dist:
    def __init__(self):
        self.rank, self.size, self.local = dist_env()
        self.pg = None
        if self.size > 1:
            import torch.distributed as td
            td.init_process_group(backend="gloo")
            self.td = td

    def barrier(self):
        if self.size > 1:
            self.td.barrier()

    def max(self, x):
        if self.size == 1:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x):
        if self.size == 1:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.size > 1:
            self.td.destroy_process_group()


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = os.path.join("/tmp", "jbgpu_clocks_%d_%d.csv" % (os.getpid(), device))

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), float(parts[3]), parts[5:9]))
            except ValueError:
                continue
        if not rows:
            return None
        sm = np.array([r[0] for r in rows])
        pw = np.array([r[2] for r in rows])
        load = sm[pw >= np.median(pw)] if len(rows) > 2 else sm
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i, v in enumerate(r[3]) if v.lower() == "active"})
        return {"sm_mhz": float(np.median(load)), "sm_max_mhz": float(max(r[1] for r in rows)), "reasons": reasons,
                "samples": len(rows), "power_w_max": float(pw.max())}


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return None


# Algorithmic bytes per step of each phase: the per-unit figures of the step's data movement
# (per body: predict 112, aabb 80, morton 40 + radix 64 + tree build/refit 150 + traversal 32,
# integrate 150; per pair: key write 8 + persistence 32; per executed pair: two body states
# 96 + manifold read/write 512; per contact: setup 400, write-back 12; per solver row and
# iteration: 64 B row + 8 B impulse + 2 x 48 B body velocities = 168, three rows per contact).
def phase_bytes(phase, c, bodies, iters):
    rows = c["solver_rows"]
    return {
        "predict": 112 * bodies,
        "aabb": 80 * bodies,
        "pair_count": (40 + 64 + 150 + 32) * bodies,
        "pair_fill": 40 * c["pairs"] + 32 * bodies,
        "narrow_gjk": (96 + 512) * c["pairs"],
        "narrow_epa": (96 + 512) * c["epa_calls"],
        "setup": 400 * rows,
        "pgs": (iters + 1) * 3 * rows * 168 + 12 * rows,
        "integrate": 150 * bodies,
        "activation": 48 * bodies,
    }.get(phase)


def make_scene(name, seed):
    from jbgpu import scenes
    return scenes.SCENES[name](seed=seed)


def rank_scene(args, rank, size):
    """The scene this rank steps: its share of the worlds of a batched workload (split by
    jbgpu.shard, no world on two ranks), else an independent replica (seed + rank)."""
    from jbgpu import shard
    sc = make_scene(args.workload, args.seed)
    if size > 1 and sc.world_of_body is not None:
        mine, parts = shard.shard_scene(sc, rank, size, cost=args.shard_cost)
        return mine, {"mode": "sharded by world", "worlds": len(parts[rank]), "worlds_total": len(parts),
                      "cost": args.shard_cost}
    if size > 1:
        sc = make_scene(args.workload, args.seed + rank)
    return sc, {"mode": "replica" if size > 1 else "single", "worlds": 1 if sc.world_of_body is None
                else int(sc.world_of_body.max()) + 1}


def window(args):
    first = args.settle + args.warmup
    return first, first + args.steps - 1


def bench_config(sc, args, iters):
    """The config keys both arms print (the reference arm's line carries the same ones)."""
    first, last = window(args)
    return {"workload": sc.name, "bodies": sc.n_bodies, "dt": sc.dt, "iterations": iters, "seed": args.seed,
            "settle_steps": args.settle, "warmup_steps": args.warmup,
            "timed_steps": "%d..%d of the drop from rest" % (first, last),
            "l2": "no flush: per-step working set (bodies, two pair/manifold buffers, solver rows) exceeds L2"}


def advance(w, sc, n):
    for _ in range(n):
        w.step(sc.dt)


def pinned(shape):
    try:
        import torch
        if torch.cuda.is_available():
            return torch.empty(shape, dtype=torch.float32, pin_memory=True).numpy()
    except Exception:
        pass
    return np.zeros(shape, np.float32)


def snapshot_to_oracle(g, o):
    """Hands a GPU world's state and manifolds to an oracle world (the CPU side then continues
    from exactly the state the GPU reached)."""
    st = g.get_state()
    o.set_state({k: st[k] for k in ("transform", "linear_velocity", "angular_velocity", "inv_inertia_world",
                                     "total_force", "total_torque", "aabb", "activation_state", "deactivation_time")})
    o.set_manifolds(g.get_manifolds())


def run_cpu_baseline(scene, world_cls, cfg, snap_steps, window_len):
    """Oracle (reference island order, 1 core) continued for `window_len` steps from GPU
    snapshots at the given steps of the trajectory from rest."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    g = world_cls(scene, config=cfg)
    g.set_graph(True)
    done, total_t, total_steps = 0, 0.0, 0
    for s in sorted(set(snap_steps)):
        advance(g, scene, s - done)
        done = s
        o = pyoracle.OracleWorld(scene, order_mode=pyoracle.ORDER_REFERENCE)
        snapshot_to_oracle(g, o)
        t0 = time.perf_counter()
        for _ in range(window_len):
            o.step(scene.dt)
        total_t += time.perf_counter() - t0
        total_steps += window_len
        del o
    g.close()
    value = scene.n_bodies * total_steps / total_t
    return {"value": value, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": "CPU restatement of the reference (oracle, 1 thread, reference island solver order): %d-step windows "
                      "from GPU snapshots at steps %s of the %s trajectory from rest, %.1f s of CPU work" % (
                          window_len, sorted(set(snap_steps)), scene.name, total_t)}


def measure_rays(w, scene, nrays, seed, local):
    """CollisionWorld.rayTest batches on the world as the timed steps left it: nrays rays per
    batch from device buffers (half straight down from above the bodies, half between random
    points of their bounding region), CUDA events on the world's stream around 5 batches after 2
    untimed ones; a 1,024-ray sample compared with the oracle bit for bit and timed on 1 core."""
    import torch
    from jbgpu import _abi
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    st = w.get_state()
    pos = st["transform"][:, 9:]
    fin = np.all(np.abs(pos) < 1e6, axis=1)
    lo, hi = pos[fin].min(0), pos[fin].max(0)
    rng = np.random.Generator(np.random.PCG64(seed))
    a = rng.uniform(lo, hi, (nrays, 3)).astype(np.float32)
    b = rng.uniform(lo, hi, (nrays, 3)).astype(np.float32)
    h = nrays // 2
    a[:h, 1] = hi[1] + 5.0
    b[:h] = a[:h]
    b[:h, 1] = lo[1] - 2.0
    dev = "cuda:%d" % local
    df, dt = torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev)
    dh = torch.empty(nrays * _abi.RAY_HIT_DTYPE.itemsize, dtype=torch.uint8, device=dev)
    for _ in range(2):
        w.ray_test_device(df.data_ptr(), dt.data_ptr(), nrays, dh.data_ptr())
    w.synchronize()
    reps = 5
    w.timer_start()
    for _ in range(reps):
        w.ray_test_device(df.data_ptr(), dt.data_ptr(), nrays, dh.data_ptr())
    ms = w.timer_stop() / reps
    replays = w.counters()["ray_replays"]
    hits = dh.cpu().numpy().view(_abi.RAY_HIT_DTYPE)
    t0 = time.perf_counter()
    hh = w.ray_test(a, b)
    host_ms = (time.perf_counter() - t0) * 1e3
    o = pyoracle.OracleWorld(scene)
    o.set_state({"transform": st["transform"]})
    k = 1024
    t0 = time.perf_counter()
    ho = o.ray_test(a[:k], b[:k])
    cpu_s = time.perf_counter() - t0
    same = bool(np.array_equal(ho.view(np.uint8), hits[:k].view(np.uint8)) and
                np.array_equal(hh.view(np.uint8), hits.view(np.uint8)))
    return {"rays_per_batch": nrays, "ms_per_batch": ms, "rays_per_s": nrays / (ms * 1e-3),
            "hit_fraction": float(np.mean(hits["body"] >= 0)), "replayed_rays": int(replays),
            "host_buffers_ms_per_batch": host_ms,
            "cpu_oracle_rays_per_s": k / cpu_s, "cpu_sample": "%d rays of the batch, oracle (the reference's object "
                                                                 "loop restated), 1 thread" % k,
            "bit_exact_vs_oracle_sample": same,
            "clock": "CUDA events on the world's stream around 5 batches of device buffers"}


def measure_sweeps(w, scene, nsweeps, seed, local):
    """CollisionWorld.convexSweepTest batches on the world as the timed steps left it: nsweeps
    sweeps of the scene's first sphere shape (else its first convex shape) per batch from device
    buffers, each with its own start and end rotation (half straight down from above the bodies,
    half between random points of their bounding region), filter mask without the static group
    (the reference throws on a sweep that reaches its static plane); CUDA events on the world's
    stream around 3 batches after 1 untimed one; a 64-sweep sample compared with the oracle bit for
    bit and timed on 1 core."""
    import torch
    from jbgpu import _abi
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    st = w.get_state()
    pos = st["transform"][:, 9:]
    fin = np.all(np.abs(pos) < 1e6, axis=1)
    lo, hi = pos[fin].min(0), pos[fin].max(0)
    rng = np.random.Generator(np.random.PCG64(seed))
    a = rng.uniform(lo, hi, (nsweeps, 3)).astype(np.float32)
    b = rng.uniform(lo, hi, (nsweeps, 3)).astype(np.float32)
    h = nsweeps // 2
    a[:h, 1] = hi[1] + 5.0
    b[:h] = a[:h]
    b[:h, 1] = lo[1] - 2.0

    def rot(q):
        x, y, z, ww = q / np.linalg.norm(q)
        return np.array([1 - 2 * (y * y + z * z), 2 * (x * y - z * ww), 2 * (x * z + y * ww),
                         2 * (x * y + z * ww), 1 - 2 * (x * x + z * z), 2 * (y * z - x * ww),
                         2 * (x * z - y * ww), 2 * (y * z + x * ww), 1 - 2 * (x * x + y * y)], np.float32)
    fr = np.zeros((nsweeps, 12), np.float32)
    to = np.zeros((nsweeps, 12), np.float32)
    for i in range(nsweeps):
        fr[i, :9], to[i, :9] = rot(rng.normal(size=4)), rot(rng.normal(size=4))
    fr[:, 9:], to[:, 9:] = a, b
    kinds = [s["type"] for s in scene.shapes]
    shape = kinds.index(_abi.SHAPE_SPHERE) if _abi.SHAPE_SPHERE in kinds else \
        next(i for i, k in enumerate(kinds) if k != _abi.SHAPE_STATIC_PLANE)
    mask = ~2 & 0xFFFF
    dev = "cuda:%d" % local
    df, dt = torch.from_numpy(fr).to(dev), torch.from_numpy(to).to(dev)
    dh = torch.empty(nsweeps * _abi.RAY_HIT_DTYPE.itemsize, dtype=torch.uint8, device=dev)
    w.convex_sweep_test_device(shape, df.data_ptr(), dt.data_ptr(), nsweeps, dh.data_ptr(), mask=mask)
    w.synchronize()
    reps = 3
    w.timer_start()
    for _ in range(reps):
        w.convex_sweep_test_device(shape, df.data_ptr(), dt.data_ptr(), nsweeps, dh.data_ptr(), mask=mask)
    ms = w.timer_stop() / reps
    hits = dh.cpu().numpy().view(_abi.RAY_HIT_DTYPE)
    o = pyoracle.OracleWorld(scene)
    o.set_state({"transform": st["transform"]})
    k = 64
    t0 = time.perf_counter()
    ho, _ = o.convex_sweep(shape, fr[:k], to[:k], mask=mask)
    cpu_s = time.perf_counter() - t0
    return {"sweeps_per_batch": nsweeps, "cast_shape": int(kinds[shape]), "ms_per_batch": ms,
            "sweeps_per_s": nsweeps / (ms * 1e-3), "hit_fraction": float(np.mean(hits["body"] >= 0)),
            "cpu_oracle_sweeps_per_s": k / cpu_s,
            "cpu_sample": "%d sweeps of the batch, oracle (the reference's object loop restated), 1 thread" % k,
            "bit_exact_vs_oracle_sample": bool(np.array_equal(ho.view(np.uint8), hits[:k].view(np.uint8))),
            "clock": "CUDA events on the world's stream around 3 batches of device buffers"}


def traffic_for_window(dom, window_bytes, workload):
    """DRAM bytes per launch of the dominant kernel for this window: one ncu capture's
    dram__bytes_read.sum + dram__bytes_write.sum, scaled by the window's algorithmic bytes per
    launch over the capture's (profiles/traffic.json)."""
    tp = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(tp):
        return None, None
    rec = json.load(open(tp)).get(dom)
    if not isinstance(rec, dict) or not rec.get("algorithmic_bytes") or rec.get("workload") != workload:
        return None, None
    scale = window_bytes / rec["algorithmic_bytes"]
    return rec["dram_bytes"] * scale, {"captured": rec.get("captured"), "capture_dram_bytes": rec["dram_bytes"],
                                       "capture_algorithmic_bytes": rec["algorithmic_bytes"], "scale": scale}


# The other workloads of the step, measured beside the headline in the same run: each stepped
# from rest to a settled point (untimed), then timed over `steps` steps by CUDA events on the
# world's stream (CUDA graphs, as the headline); the phases come from a second, event-marked run.
OTHER_WORKLOADS = [("boxes_1k", 100, 100), ("hulls_20k", 300, 20), ("batched_4096", 200, 20), ("terrain_20k", 300, 20)]


def measure_workload(name, settle, steps, seed, local):
    from jbgpu import _abi
    from jbgpu.lib import GpuWorld
    sc = make_scene(name, seed)
    cfg = _abi.default_config(**sc.config)
    cfg.device = local
    w = GpuWorld(sc, config=cfg)
    w.set_graph(True)
    advance(w, sc, settle)
    w.synchronize()
    w.timer_start()
    advance(w, sc, steps)
    ms = w.timer_stop() / steps
    c = w.counters()
    w.close()
    w = GpuWorld(sc, config=cfg)
    advance(w, sc, settle)
    w.set_profiling(steps)
    advance(w, sc, steps)
    w.synchronize()
    ph, k, _ = w.phase_times()
    w.close()
    worlds = 1 if sc.world_of_body is None else int(sc.world_of_body.max()) + 1
    return {"workload": sc.name, "bodies": sc.n_bodies, "worlds": worlds, "dt": sc.dt, "iterations": cfg.num_iterations,
            "timed_steps": "%d..%d from rest" % (settle, settle + steps - 1), "ms_per_step": ms,
            "body_steps_per_s": sc.n_bodies / (ms * 1e-3),
            "phases_ms": {a: round(b / k, 4) for a, b in ph.items() if b > 0},
            "counters": {q: c[q] for q in ("pairs", "contacts", "solver_rows", "colours", "cut_colours", "gjk_calls",
                                           "epa_calls", "status_flags")},
            "clock": "CUDA events on the world's stream, CUDA graphs; phases from a second event-marked run"}


def run_ours(args, dist):
    from jbgpu import _abi, _build, lib
    from jbgpu.lib import GpuWorld
    _build.build()
    sc, split = rank_scene(args, dist.rank, dist.size)
    cfg = _abi.default_config(**sc.config)
    cfg.device = dist.local
    cfg.solver_parts = args.solver_parts
    cfg.solver_threads = args.solver_threads
    cfg.solver_smem_bodies = args.solver_smem_bodies
    if args.rebuild_interval is not None:
        cfg.broadphase_rebuild_interval = args.rebuild_interval
    tuned = None
    if args.autotune:
        from jbgpu import autotune
        tuned = autotune.tune(sc, device=dist.local)
        for k, v in tuned["best"].items():
            setattr(cfg, k, v)
    iters = cfg.num_iterations
    n = sc.n_bodies
    K, W, S = args.steps, args.warmup, args.settle
    first, last = window(args)
    # ---- device-timed run: CUDA events on the world's stream around K steps ----------------
    w = GpuWorld(sc, config=cfg)
    if args.graph:
        w.set_graph(True)
    advance(w, sc, S + W)
    clk = ClockSampler(dist.local)
    clk.start()
    dist.barrier()
    w.synchronize()
    l0 = lib.launch_count()
    t0 = time.perf_counter()
    w.timer_start()
    for _ in range(K):
        w.step(sc.dt)
    device_ms = w.timer_stop()
    t1 = time.perf_counter()
    launches = lib.launch_count() - l0
    dist.barrier()
    clocks = clk.stop()
    final = w.counters()
    graph_info = None
    if args.graph:
        ng, gerr = w.graph_status()
        graph_info = {"graphs_held": ng, "capture_error": gerr or None}
    rays = None
    if dist.rank == 0 and not args.no_rays:
        rays = measure_rays(w, sc, args.rays, args.seed + 20, dist.local)
    sweeps = None
    if dist.rank == 0 and args.sweeps > 0:
        sweeps = measure_sweeps(w, sc, args.sweeps, args.seed + 30, dist.local)
    w.close()
    others = None
    if dist.rank == 0 and dist.size == 1 and not args.no_others:
        others = [measure_workload(nm, st, k, args.seed, dist.local) for nm, st, k in OTHER_WORKLOADS
                  if nm != args.workload]
    wall = t1 - t0
    elapsed = dist.max(device_ms * 1e-3)
    # ---- the same steps again with per-phase event marks (the breakdown and the roofline) ---
    w = GpuWorld(sc, config=cfg)
    if args.graph:
        w.set_graph(True)
    advance(w, sc, S + W)
    w.set_profiling(K)
    advance(w, sc, K)
    w.synchronize()
    phases, nsteps, window_ms = w.phase_times()
    ctrs = w.profile_counters()
    w.close()
    total_body_steps = dist.sum(n * K)
    value = total_body_steps / elapsed
    # ---- roofline of the dominant phase ----------------------------------------------------
    dom = max(phases, key=lambda k: phases[k])
    pk = peaks()
    roof = None
    side = {}
    for ph, ms in phases.items():
        by = [phase_bytes(ph, c, n, iters) for c in ctrs]
        if by and by[0] is not None and ms > 0:
            side[ph] = {"ms_per_step": ms / nsteps, "GB_per_s": sum(by) / (ms * 1e-3) / 1e9}
        else:
            side[ph] = {"ms_per_step": ms / nsteps}
    by = [phase_bytes(dom, c, n, iters) for c in ctrs]
    if by and by[0] is not None:
        achieved = sum(by) / (phases[dom] * 1e-3) / 1e9
        peak = pk["hbm_gbs"] if pk else 6800.0
        per_launch = sum(by) / len(by)
        traffic, traffic_src = traffic_for_window(dom, per_launch, sc.name)
        roof = {"bound": "hbm", "kernel_phase": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic, "traffic_from": traffic_src,
                "peak_source": "of measured (MEASURED_PEAKS.json hbm_gbs)" if pk else "of fallback 6.8 TB/s",
                "algorithmic_bytes_per_launch": per_launch,
                "timing": "CUDA events around the phase on the world's stream, profiled run of the same window"}
    # ---- end to end through the reference-facing call with host buffers --------------------
    e2e = None
    if not args.no_e2e:
        w = GpuWorld(sc, config=cfg)
        if args.graph:
            w.set_graph(True)
        force = pinned((n, 3))
        xout = pinned((n, 12))
        advance(w, sc, S)
        for _ in range(W):
            w.apply_forces(force, None)
            w.step_simulation(sc.dt, 1, sc.dt)
            w.get_transforms(xout)
        dist.barrier()
        w.synchronize()
        ts = time.perf_counter()
        executed = 0
        for _ in range(K):
            w.apply_forces(force, None)
            executed += min(w.step_simulation(sc.dt, 1, sc.dt), 1)
            w.get_transforms(xout)
        te = time.perf_counter()
        dist.barrier()
        w.close()
        e_el = dist.max(te - ts)
        e2e = {"value": dist.sum(n * executed) / e_el, "unit": UNIT, "h2d_bytes_per_step": int(force.nbytes),
               "d2h_bytes_per_step": int(xout.nbytes), "substeps": executed,
               "clock": "host wall clock around the K calls (each ends with its transforms on the host)",
               "call": "jbgpu_world_step_simulation(dt, maxSubSteps 1, fixedTimeStep dt); substeps = executed steps"}
    # ---- CPU baseline (rank 0, N = 1 only): windows inside the timed window -----------------
    cpu = None
    if dist.rank == 0 and dist.size == 1 and not args.no_cpu:
        win = min(args.cpu_window, K)
        snaps = [first, first + (K - win) // 2, first + K - win]
        cpu = run_cpu_baseline(sc, GpuWorld, cfg, snaps, win)
    # ---- learned warm start vs the reference warm start at residual 1e-4 (rank 0) -----------
    learned = None
    if dist.rank == 0 and not args.no_learned:
        from jbgpu import warmstart
        if os.path.exists(warmstart.WEIGHTS):
            m = warmstart.load(device=dist.local)
            # the benchmark's rule: every row of the world to residual 1e-4, with a cap the plain
            # solve does not reach; the per-island rule at the 200 cap beside it
            learned = warmstart.evaluate(m, seed=args.seed + 10, settle=900, steps=4, max_iter=args.learned_cap,
                                         scope=1)
            learned["per_island"] = warmstart.evaluate(m, seed=args.seed + 10, settle=900, steps=10, max_iter=200,
                                                       scope=0)
            learned["weights"] = "jbgpu/warmstart_weights.npz (trained by python -m jbgpu.warmstart train)"
            m.close()
    last_c = ctrs[-1] if ctrs else final
    config = bench_config(sc, args, iters)
    # the workload only, key for key as the reference arm prints it; how each arm runs it is
    # in "execution"
    config["parallelism"] = split["mode"] if dist.size > 1 else "one world"
    config["split"] = split
    last_step_counters = {k: last_c[k] for k in ("pairs", "contacts", "solver_manifolds", "solver_rows", "colours",
                                                 "cut_colours", "cut_manifolds", "islands", "gjk_calls", "epa_calls")}
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.size, "steps": K, "warmup": W,
        "ms_per_step": elapsed * 1e3 / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic: seeded PCG64 scene generator (no dataset exists for this workload)",
        "config": config,
        "execution": "one world per GPU" if dist.size == 1 else "worlds split across the GPUs (config.split)",
        "last_step_counters": last_step_counters,
        "timing": {"value_from": "CUDA events on the world's stream around the K steps (jbgpu_world_timer)",
                   "device_ms": device_ms, "host_wall_ms": wall * 1e3,
                   "phases_from": "a second run of the same steps with per-phase event marks",
                   "profiled_window_ms": window_ms},
        "gpu_launches": int(launches),
        "phases": side,
        "roofline": roof,
        "e2e": e2e,
        "cpu_baseline": cpu,
        "learned_warmstart": learned,
        "ray_test": rays,
        "convex_sweep_test": sweeps,
        "other_workloads": others,
        "step_graphs": graph_info,
        "clocks": clocks,
        "status_flags": final["status_flags"],
        "autotune": tuned,
    }
    return out


def run_reference(args, dist):
    """The reference's CPU path (restated as the oracle, 1 thread) on the same window: the GPU
    world is stepped from rest to the window's first step (untimed set-up), the oracle takes
    over its state and manifolds and alone is timed over the K steps (within --ref-seconds)."""
    if dist.rank != 0:
        return None
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    pyoracle.build()
    from jbgpu import _abi, _build
    from jbgpu.lib import GpuWorld
    _build.build()
    sc = make_scene(args.workload, args.seed)
    cfg = _abi.default_config(**sc.config)
    first, last = window(args)
    g = GpuWorld(sc, config=cfg)
    g.set_graph(True)
    advance(g, sc, first)
    o = pyoracle.OracleWorld(sc, order_mode=pyoracle.ORDER_REFERENCE)
    snapshot_to_oracle(g, o)
    g.close()
    t0 = time.perf_counter()
    done = 0
    while done < args.steps:
        o.step(sc.dt)
        done += 1
        if time.perf_counter() - t0 > args.ref_seconds:
            break
    el = time.perf_counter() - t0
    value = sc.n_bodies * done / el
    config = bench_config(sc, args, cfg.num_iterations)
    config["parallelism"] = "one world"
    config["split"] = {"mode": "single", "worlds": 1 if sc.world_of_body is None else int(sc.world_of_body.max()) + 1}
    sample = ("CPU restatement of the reference (oracle; no JVM on this machine), 1 thread, full workload, steps "
              "%d..%d (%d of the %d asked, %.0f s budget), started from the GPU world's state and manifolds at step %d "
              "(untimed set-up)" % (first, first + done - 1, done, args.steps, args.ref_seconds, first))
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.size, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": el * 1e3 / done, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: seeded PCG64 scene generator (no dataset exists for this workload)",
            "config": config,
            "execution": "one world, one host thread",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    args = parse()
    dist = Dist()
    out = run_reference(args, dist) if args.impl == "reference" else run_ours(args, dist)
    if dist.rank == 0 and out is not None:
        print(json.dumps(out))
    dist.close()


if __name__ == "__main__":
    main()
