"""Autotuner of the solver's launch shape for a workload.

Sweeps threads per solver block {64, 128, 256} and the largest solver part whose velocities are
staged in shared memory {512, 1024, 2048} bodies (which sets how many blocks fit on an SM and
so how many worlds or parts run at once), timing a few steps of the workload's own world with
device events after a short warm-up, and returns the fastest setting.  The choice changes
only scheduling: every setting gives bit-identical results, which the tuner checks on the
final body state of each candidate."""
import itertools
import json
import os

import numpy as np

from . import _abi
from .lib import GpuWorld

THREADS = (64, 128, 256)
SMEM_BODIES = (512, 1024, 2048)


def tune(scene, device=0, warmup=20, steps=10, threads=THREADS, smem_bodies=SMEM_BODIES, log=None):
    results = []
    ref_state = None
    for t, sm in itertools.product(threads, smem_bodies):
        cfg = _abi.default_config(**scene.config)
        cfg.device = device
        cfg.solver_threads = t
        cfg.solver_smem_bodies = sm
        w = GpuWorld(scene, config=cfg)
        for _ in range(warmup):
            w.step(scene.dt)
        w.set_profiling(steps)
        for _ in range(steps):
            w.step(scene.dt)
        _, k, window = w.phase_times()
        st = w.get_state()["transform"]
        w.close()
        same = ref_state is None or np.array_equal(st.view(np.uint32), ref_state.view(np.uint32))
        if ref_state is None:
            ref_state = st
        results.append({"solver_threads": t, "solver_smem_bodies": sm, "ms_per_step": window / k, "identical": bool(same)})
        if log:
            log(json.dumps(results[-1]))
    best = min(results, key=lambda r: r["ms_per_step"])
    return {"best": {"solver_threads": best["solver_threads"], "solver_smem_bodies": best["solver_smem_bodies"]},
            "candidates": results, "warmup_steps": warmup, "timed_steps": steps,
            "all_identical": all(r["identical"] for r in results)}
