"""The learned warm start end to end on the GPU: samples logged by residual-terminated plain
PGS on a held-out seed, an MLP trained on them with the library's own kernels, then plain and
learned warm starts compared from the same settled state of a fresh seed.

What the test pins: the samples are finite and come only from islands that reached the
residual; training lowers the loss; the learned arm runs the same physics to the same residual
(every island it solves converges as often as plain's do) and needs fewer iterations per island
than the reference warm start (0.85 x last impulses)."""
import numpy as np
import pytest

from jbgpu import warmstart as W

pytestmark = pytest.mark.gpu

SCENE = dict(n=6000, pyramids=8, levels=10, region=(60.0, 30.0, 60.0))


def test_learned_warm_start_gains_over_the_reference_warm_start(gpu_lib):
    x, t = W.collect([1000], settle=500, steps=8, **SCENE)
    assert len(x) > 5000 and np.all(np.isfinite(x)) and np.all(np.isfinite(t))
    assert np.all(t[:, 0] >= 0.0)                     # converged normal impulses
    unit = 9.81 / 120.0
    m, losses = W.fit(x, t, unit, epochs=12, batch=1024, lr=2e-3)
    assert np.all(np.isfinite(losses)) and losses[-1] < 0.8 * losses[0], losses
    r = W.evaluate(m, 7, settle=500, steps=8, **SCENE)
    p, l = r["plain"], r["learned"]
    assert l["islands_converged"] >= p["islands_converged"] - 0.02, r
    assert l["island_iterations_mean"] < p["island_iterations_mean"], r
    m.close()
