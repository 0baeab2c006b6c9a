"""Learned warm start: data collection, training and evaluation on the GPU.

    python -m jbgpu.warmstart train --out weights.npz     # collect, train, save
    python -m jbgpu.warmstart eval --weights weights.npz  # plain vs learned solver time
    python -m jbgpu.warmstart trace                       # residual against iteration, per arm

Protocol.  Scenes are `scenes.learned_warmstart` (100k mixed bodies + pyramids of unit boxes).
A world settles with the reference's fixed 10 iterations, then switches to the residual-
terminated PGS.  The residual is r_k = max|lambda_k - lambda_k-1| / max(max|lambda_k|, 1e-6)
over all rows of the world (solver_residual_scope 1), the stopping rule of the benchmark; the
per-island rule (scope 0: each island stops on its own rows) is reported beside it.
Training samples are the features of every contact point before a solve and its impulses after
the solve has reached the residual over the whole world (all points, the large connected pile
included), from plain-PGS runs on held-out seeds (1000 + k).  Evaluation uses fresh seeds: two
worlds built from the same seed settle identically (the step is deterministic), then one keeps
the reference warm start (0.85 x last impulses) and the other takes the MLP's predictions; both
run the same number of steps to the same residual, and the device time of solver setup
(including the MLP inference) plus PGS, and the iteration counts, are compared."""
import argparse
import json
import os
import sys

import numpy as np

from . import _abi, scenes
from .lib import GpuWorld, Mlp, MLP_INPUTS, MLP_OUTPUTS, MLP_NORM

WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "warmstart_weights.npz")


def make_world(seed, n, pyramids, levels, region, device=0):
    sc = scenes.learned_warmstart(n, seed=seed, pyramids=pyramids, levels=levels, region=region)
    cfg = _abi.default_config(**sc.config)
    cfg.device = device
    return sc, GpuWorld(sc, config=cfg)


def make_world_scoped(seed, n, pyramids, levels, region, scope, device=0):
    sc = scenes.learned_warmstart(n, seed=seed, pyramids=pyramids, levels=levels, region=region)
    cfg = _abi.default_config(**sc.config)
    cfg.device = device
    cfg.solver_residual_scope = scope
    return sc, GpuWorld(sc, config=cfg)


def collect(seeds, n=100_000, pyramids=50, levels=15, region=(200.0, 100.0, 200.0), settle=600, steps=12,
            residual=1e-4, max_iter=200, log=None, scope=0):
    """Samples of plain-PGS solves.  scope 0: points of islands that reached the residual (cap
    max_iter); scope 1: every point, after the solve reached the residual over the whole world."""
    xs, ts = [], []
    for seed in seeds:
        sc, w = make_world_scoped(seed, n, pyramids, levels, region, scope)
        for _ in range(settle):
            w.step(sc.dt)
        w.set_solver_iterations(10, residual, max_iter)
        w.set_sample_logging(True, all_points=scope == 1)
        for s in range(steps):
            w.step(sc.dt)
            x, t = w.get_samples()
            xs.append(x)
            ts.append(t)
            if log:
                log("seed %d step %d: %d samples, %d iterations" % (seed, s, len(x), w.counters()["solver_iterations"]))
        w.close()
    return np.concatenate(xs), np.concatenate(ts)


# features used by the output transform (see jbgpu_world_set_warmstart_mlp)
F_IM0, F_IM1, F_LAST_IMPULSE, F_FRICTION = 10, 11, 18, 21


REL = 0.01   # the network carries relative corrections r as asinh(r / REL)


def relative_targets(x, t, unit, clip=5.0):
    """Converged impulses -> the network's targets asinh(y / REL): with b the last normal
    impulse and u = unit / (invMass0 + invMass1): y0 = (normal - b) / (b + u),
    yk = friction_k / (mu (b + u)), each clipped to [-clip, clip]."""
    b = np.maximum(x[:, F_LAST_IMPULSE], 0.0)
    u = unit / np.maximum(x[:, F_IM0] + x[:, F_IM1], 1e-6)
    s = b + u
    mu = x[:, F_FRICTION]
    y = np.empty_like(t)
    y[:, 0] = (t[:, 0] - b) / s
    fs = mu * s
    for k in (1, 2):
        y[:, k] = np.where(fs > 0, t[:, k] / np.maximum(fs, 1e-30), 0.0)
    return np.arcsinh(np.clip(y, -clip, clip) / REL).astype(np.float32)


def normalisation(x, y, unit):
    """in_mean, in_scale (median and inter-quartile scale; constant features get scale 0),
    out_mean, out_scale (of the relative targets), unit."""
    q1, med, q3 = np.percentile(x, [25, 50, 75], axis=0)
    spread = (q3 - q1) / 1.349
    sd = x.std(0)
    spread = np.where(spread > 1e-9, spread, sd)
    isd = np.where(spread > 1e-9, 1.0 / np.maximum(spread, 1e-9), 0.0)
    om, osd = y.mean(0), np.maximum(y.std(0), 1e-6)
    return np.concatenate([med, isd, om, osd, [unit]]).astype(np.float32)


def fit(x, t, unit, epochs=20, batch=2048, lr=2e-3, seed=0):
    y = relative_targets(x, t, unit)
    m = Mlp(seed=seed)
    m.set_params(norm=normalisation(x, y, unit))
    losses = m.train(x, y, epochs=epochs, batch=batch, lr=lr, seed=seed)
    return m, losses


def save(m, path):
    p, nrm = m.params()
    np.savez(path, params=p, norm=nrm)


def load(path=WEIGHTS, device=0):
    d = np.load(path)
    m = Mlp(device=device, seed=0)
    m.set_params(d["params"], d["norm"])
    return m


def _arm_stats(w, steps, max_iter):
    ph, k, _ = w.phase_times()
    pc = w.profile_counters()
    its = [c["solver_iterations"] for c in pc]
    isl = sum(c["solver_islands"] for c in pc)
    return {"solver_ms_per_step": (ph["setup"] + ph["pgs"]) / k, "pgs_ms_per_step": ph["pgs"] / k,
            "iterations_mean": float(np.mean(its)), "iterations_max": int(np.max(its)),
            "steps_at_cap": int(sum(i >= max_iter for i in its)), "steps": k,
            "island_iterations_mean": sum(c["solver_island_iterations"] for c in pc) / max(isl, 1),
            "islands_converged": sum(c["solver_islands_converged"] for c in pc) / max(isl, 1),
            "islands_per_step": isl / k, "contact_rows": int(w.counters()["solver_rows"])}


def evaluate(mlp, seed, n=100_000, pyramids=50, levels=15, region=(200.0, 100.0, 200.0), settle=600, steps=10,
             residual=1e-4, max_iter=200, scope=0):
    """Plain vs learned warm start from the same settled state: per-arm mean solver device time
    (setup + PGS) per step, mean and max iterations, steps that hit the cap.  scope 1 applies the
    residual to all rows of the world at once (every island iterates until it holds)."""
    out = {}
    sc, plain = make_world_scoped(seed, n, pyramids, levels, region, scope)
    _, learned = make_world_scoped(seed, n, pyramids, levels, region, scope)
    for _ in range(settle):
        plain.step(sc.dt)
        learned.step(sc.dt)
    for name, w in (("plain", plain), ("learned", learned)):
        w.set_solver_iterations(10, residual, max_iter)
        if name == "learned":
            w.set_warmstart_mlp(mlp)
        w.set_profiling(steps)
        for _ in range(steps):
            w.step(sc.dt)
        out[name] = _arm_stats(w, steps, max_iter)
        w.close()
    out["time_saving"] = 1.0 - out["learned"]["solver_ms_per_step"] / out["plain"]["solver_ms_per_step"]
    out["iteration_saving"] = 1.0 - out["learned"]["iterations_mean"] / out["plain"]["iterations_mean"]
    out["island_iteration_saving"] = 1.0 - out["learned"]["island_iterations_mean"] / out["plain"]["island_iterations_mean"]
    out["config"] = {"bodies": int(sc.n_bodies), "pyramids": pyramids, "levels": levels, "residual": residual,
                     "residual_scope": "world" if scope else "island", "max_iterations": max_iter,
                     "settle_steps": settle, "eval_steps": steps, "seed": seed}
    return out


def trace(mlp, seed, n=100_000, pyramids=50, levels=15, region=(200.0, 100.0, 200.0), settle=900, steps=3,
          residual=1e-4, max_iter=12000, marks=(1, 10, 50, 100, 200, 500, 1000, 2000, 3000, 5000)):
    """World residual against iteration for the reference warm start (factor 0.85), factor 1.0
    and the MLP, each from the same settled state: how many iterations the slow modes of a large
    pile need, and whether the warm start changes that."""
    out = {}
    sc = scenes.learned_warmstart(n, seed=seed, pyramids=pyramids, levels=levels, region=region)
    base = GpuWorld(sc, config=_abi.default_config(**sc.config))
    for _ in range(settle):           # one settled state (reference warm start) for every arm
        base.step(sc.dt)
    st = base.get_state()
    mf = base.get_manifolds()
    base.close()
    keep = ("transform", "linear_velocity", "angular_velocity", "inv_inertia_world", "total_force", "total_torque",
            "aabb", "activation_state", "deactivation_time")
    arms = [("reference_0.85", 0.85, None), ("factor_1.0", 1.0, None)] + ([("learned", 0.85, mlp)] if mlp else [])
    for name, factor, m in arms:
        cfg = _abi.default_config(**sc.config)
        cfg.solver_residual_scope = 1
        cfg.warmstarting_factor = factor
        w = GpuWorld(sc, config=cfg)
        w.set_state({k: st[k] for k in keep})
        w.set_manifolds(mf)
        w.set_solver_iterations(10, residual, max_iter)
        if m is not None:
            w.set_warmstart_mlp(m)
        recs = []
        for _ in range(steps):
            w.step(sc.dt)
            tr = w.residual_trace()
            r = tr[:, 0] / np.maximum(tr[:, 1], np.float32(1e-6))
            recs.append({"iterations": int(w.counters()["solver_iterations"]),
                         "residual_at": {int(k): float(r[k - 1]) for k in marks if k < len(r)}})
        out[name] = recs
        w.close()
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("cmd", choices=["train", "eval", "trace"])
    ap.add_argument("--scope", type=int, default=1, help="residual scope: 0 per island, 1 the world's rows")
    ap.add_argument("--max-iter", type=int, default=10000)
    ap.add_argument("--out", default=WEIGHTS)
    ap.add_argument("--weights", default=WEIGHTS)
    ap.add_argument("--bodies", type=int, default=100_000)
    ap.add_argument("--pyramids", type=int, default=50)
    ap.add_argument("--levels", type=int, default=15)
    ap.add_argument("--seeds", type=int, default=2)
    ap.add_argument("--steps", type=int, default=12)
    ap.add_argument("--settle", type=int, default=600)
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--eval-seed", type=int, default=0)
    a = ap.parse_args(argv)
    log = lambda s: print(s, file=sys.stderr, flush=True)
    if a.cmd == "train":
        x, t = collect([1000 + k for k in range(a.seeds)], a.bodies, a.pyramids, a.levels, settle=a.settle,
                       steps=a.steps, log=log, scope=a.scope, max_iter=a.max_iter)
        log("samples: %d" % len(x))
        sc = scenes.learned_warmstart(0, pyramids=1, levels=2)
        unit = float(np.linalg.norm(sc.config["gravity"])) * sc.dt
        m, losses = fit(x, t, unit, epochs=a.epochs)
        log("loss per epoch: " + " ".join("%.4g" % l for l in losses))
        save(m, a.out)
        print(json.dumps({"samples": int(len(x)), "losses": [float(l) for l in losses], "out": a.out}))
    elif a.cmd == "trace":
        m = load(a.weights) if os.path.exists(a.weights) else None
        print(json.dumps(trace(m, a.eval_seed, a.bodies, a.pyramids, a.levels, settle=a.settle, steps=a.steps,
                               max_iter=a.max_iter)))
    else:
        m = load(a.weights)
        print(json.dumps(evaluate(m, a.eval_seed, a.bodies, a.pyramids, a.levels, settle=a.settle, steps=a.steps,
                                  max_iter=a.max_iter, scope=a.scope)))


if __name__ == "__main__":
    main()
