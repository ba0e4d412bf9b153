"""Seeded ray sets and comparison helpers for the parity tests."""
import numpy as np

from snkpt import abi


def scene_bounds(scene):
    lo = np.full(3, np.inf)
    hi = np.full(3, -np.inf)
    for inst in scene.instances:
        m = scene.meshes[int(inst["mesh_id"])]
        M = inst["transform"].reshape(3, 4).astype(np.float64)
        p = m.positions.astype(np.float64) @ M[:, :3].T + M[:, 3]
        lo = np.minimum(lo, p.min(0))
        hi = np.maximum(hi, p.max(0))
    return lo, hi


def camera_rays(view, n=None, rng=None, tmin=0.0, tmax=1e4):
    """Primary rays through pixel centres (all pixels, or n random ones)."""
    W, H = int(view["width"]), int(view["height"])
    if n is None:
        ys, xs = np.mgrid[0:H, 0:W]
        xs, ys = xs.reshape(-1), ys.reshape(-1)
    else:
        xs, ys = rng.integers(0, W, n), rng.integers(0, H, n)
    fx = (xs + 0.5) / W * 2 - 1
    fy = 1 - (ys + 0.5) / H * 2
    t = float(view["tan_half_fov_y"])
    d = (view["forward"][None, :] + view["right"][None, :] * (fx * t * float(view["aspect"]))[:, None]
         + view["up"][None, :] * (fy * t)[:, None])
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = np.zeros(len(xs), abi.RAY_DTYPE)
    r["o"] = view["pos"]
    r["d"] = d
    r["tmin"] = tmin
    r["tmax"] = tmax
    return r


def random_rays(scene, n, rng, tmin=0.0, tmax=1e4):
    """Incoherent rays: origins uniform in the scene bounds, directions uniform on the sphere."""
    lo, hi = scene_bounds(scene)
    o = rng.uniform(lo, hi, (n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = np.zeros(n, abi.RAY_DTYPE)
    r["o"], r["d"], r["tmin"], r["tmax"] = o, d, tmin, tmax
    return r


def shadow_rays(scene, n, rng):
    """Segments between two random points of the scene box (tmax = their distance)."""
    lo, hi = scene_bounds(scene)
    a = rng.uniform(lo, hi, (n, 3))
    b = rng.uniform(lo, hi, (n, 3))
    d = b - a
    dist = np.linalg.norm(d, axis=1)
    r = np.zeros(n, abi.RAY_DTYPE)
    r["o"], r["d"], r["tmin"], r["tmax"] = a, d / dist[:, None], 0.001, dist
    return r


def assert_hits_equal(a, b, what=""):
    """Bit-exact comparison of two hit arrays (t, instance, triangle, barycentrics)."""
    a = np.asarray(a, abi.HIT_DTYPE)
    b = np.asarray(b, abi.HIT_DTYPE)
    bad = ((a["t"].view(np.uint32) != b["t"].view(np.uint32)) | (a["inst"] != b["inst"]) | (a["prim"] != b["prim"])
           | (a["u"].view(np.uint32) != b["u"].view(np.uint32)) | (a["v"].view(np.uint32) != b["v"].view(np.uint32))
           | (a["flags"] != b["flags"]))
    nbad = int(bad.sum())
    if nbad:
        i = int(np.flatnonzero(bad)[0])
        raise AssertionError(f"{what}: {nbad}/{len(a)} hits differ; first #{i}: {a[i]} vs {b[i]}")


def max_rel(a, b, floor=1e-6):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float((np.abs(a - b) / np.maximum(np.abs(b), floor)).max()) if a.size else 0.0
