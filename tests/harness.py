"""Shared helpers for parity tests: build the oracle and the GPU world from one scene,
copy a snapshot from one to the other, and compare state / manifold snapshots."""
import numpy as np

from jbgpu import _abi

STATE_COPY = ("transform", "linear_velocity", "angular_velocity", "inv_inertia_world", "total_force", "total_torque",
              "aabb", "activation_state", "deactivation_time")


def copy_world(src, dst, manifolds=True):
    st = src.get_state()
    dst.set_state({k: st[k] for k in STATE_COPY})
    if manifolds:
        dst.set_manifolds(src.get_manifolds())


def rel_err(a, b, floor=1e-6):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b) / np.maximum(np.maximum(np.abs(a), np.abs(b)), floor)


def bits_equal(a, b):
    """Element-wise binary32 equality, +0 == -0, NaN == NaN."""
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    return (a == b) | (np.isnan(a) & np.isnan(b))


def compare_state(a, b, fields=STATE_COPY, rtol=0.0):
    """Returns {field: (n_mismatch, max_rel_err)} for fields that differ beyond rtol."""
    bad = {}
    for k in fields:
        x, y = a[k], b[k]
        if x.dtype == np.int32:
            n = int(np.sum(x != y))
            if n:
                bad[k] = (n, None)
            continue
        eq = bits_equal(x, y)
        if rtol > 0:
            eq = eq | (rel_err(x, y) <= rtol)
        n = int(np.sum(~eq))
        if n:
            bad[k] = (n, float(np.max(rel_err(x, y))))
    return bad


# point field slices in the 32-float manifold point layout
PT_FIELDS = {"localA": slice(0, 3), "localB": slice(3, 6), "worldA": slice(6, 9), "worldB": slice(9, 12),
             "normal": slice(12, 15), "distance": slice(15, 16), "friction": slice(16, 17), "restitution": slice(17, 18),
             "impulse": slice(18, 19), "lat1": slice(19, 20), "lat2": slice(20, 21), "latInit": slice(21, 22),
             "life": slice(22, 23), "dir1": slice(23, 26), "dir2": slice(26, 29)}


def compare_manifolds(a, b, rtol=0.0):
    """Compare two manifold snapshots; keys/flags/counts must match exactly."""
    out = {}
    if len(a["keys"]) != len(b["keys"]) or np.any(a["keys"] != b["keys"]):
        out["keys"] = (int(np.sum(~np.isin(a["keys"], b["keys"]))) + int(np.sum(~np.isin(b["keys"], a["keys"]))), None)
        return out
    for k in ("flags", "num_points"):
        n = int(np.sum(a[k] != b[k]))
        if n:
            out[k] = (n, None)
    if out:
        return out
    npts = a["num_points"]
    mask = np.arange(4)[None, :] < npts[:, None]
    pa, pb = a["points"][mask], b["points"][mask]
    lat = pa[:, 21] != 0
    for name, sl in PT_FIELDS.items():
        x, y = pa[:, sl], pb[:, sl]
        if name in ("dir1", "dir2"):
            x, y = x[lat], y[lat]
        eq = bits_equal(x, y)
        if rtol > 0:
            eq = eq | (rel_err(x, y) <= rtol)
        n = int(np.sum(~eq))
        if n:
            out[name] = (n, float(np.max(rel_err(x, y))))
    return out
