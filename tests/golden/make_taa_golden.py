"""Generate tests/golden/taa.npz: a 3-frame TAA resolve sequence.

An independent vectorised numpy restatement of TAA_Resolve.comp
(Core/res/shaders/TAA_Resolve.comp:12-86) in binary32 (every operation on
float32 arrays, constants rounded to float32 first, as a GLSL compiler folds
them), with the history handling of TAA_ResolvePass
(Core/src/renderpasses/TAA_ResolvePass.cpp:39-56: history = the resolved frame,
previous velocity = this frame's velocity) and the sampler of
Core/src/resources/Images.cpp:16-36 (linear filter, repeat addressing), with
exact bilinear weights.  The first frame takes itself as history.

Inputs are seeded: radiance with negative and large values, motion that pushes
the reprojected coordinate outside [0, 1] (clamp) and across the image edge
(repeat wrap).  Run:  python tests/golden/make_taa_golden.py
"""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
f32 = np.float32


def bilinear_repeat(img, w, h, cu, cv):
    u = cu * f32(w) - f32(0.5)
    v = cv * f32(h) - f32(0.5)
    fu, fv = np.floor(u), np.floor(v)
    a, b = u - fu, v - fv
    i0 = np.mod(fu.astype(np.int64), w); i1 = np.mod(fu.astype(np.int64) + 1, w)
    j0 = np.mod(fv.astype(np.int64), h); j1 = np.mod(fv.astype(np.int64) + 1, h)
    one = f32(1.0)
    w00 = ((one - a) * (one - b))[..., None]
    w10 = (a * (one - b))[..., None]
    w01 = ((one - a) * b)[..., None]
    w11 = (a * b)[..., None]
    t = img.reshape(h, w, -1)
    return ((w00 * t[j0, i0] + w10 * t[j0, i1]) + w01 * t[j1, i0]) + w11 * t[j1, i1]


def taa_resolve(cur, motion, hist, pmot, w, h):
    cur = cur.reshape(h, w, 4).astype(f32)
    mot = motion.reshape(h, w, 2).astype(f32)
    ys, xs = np.meshgrid(np.arange(h), np.arange(w), indexing="ij")
    hx = (xs.astype(f32) + f32(0.5)) / f32(w) + mot[..., 0]
    hy = (ys.astype(f32) + f32(0.5)) / f32(h) + mot[..., 1]
    hx = np.minimum(np.maximum(hx, f32(0)), f32(1))
    hy = np.minimum(np.maximum(hy, f32(0)), f32(1))
    mn = np.full((h, w, 3), f32(9999.0), f32)
    mx = np.full((h, w, 3), f32(-9999.0), f32)
    m = np.zeros((h, w, 3), f32)
    m2 = np.zeros((h, w, 3), f32)
    for ox in (-1, 0, 1):
        for oy in (-1, 0, 1):
            qx = np.clip(xs + ox, 0, w - 1)
            qy = np.clip(ys + oy, 0, h - 1)
            col = np.maximum(cur[qy, qx, :3], f32(0))
            mn = np.minimum(mn, col)
            mx = np.maximum(mx, col)
            m = m + col
            m2 = m2 + col * col
    inv9 = f32(1.0) / f32(9.0)
    gamma, eps = f32(0.55), f32(0.00000001)
    mu = m * inv9
    sigma = np.sqrt(np.abs(m2 * inv9 - mu * mu))
    minc = mu - gamma * sigma
    maxc = mu + gamma * sigma
    p = np.minimum(np.maximum(mu, mn), mx)
    hc = bilinear_repeat(hist.astype(f32), w, h, hx, hy)[..., :3]
    r = np.maximum(hc, f32(0)) - p
    for c in range(3):
        rmax = maxc[..., c] - p[..., c]
        sel = r[..., c] > rmax + eps
        s = np.where(sel, rmax / np.where(sel, r[..., c], f32(1)), f32(1))
        r = np.where(sel[..., None], r * s[..., None], r)
    for c in range(3):
        rmin = minc[..., c] - p[..., c]
        sel = r[..., c] < rmin - eps
        s = np.where(sel, rmin / np.where(sel, r[..., c], f32(1)), f32(1))
        r = np.where(sel[..., None], r * s[..., None], r)
    pv = bilinear_repeat(pmot.astype(f32), w, h, hx, hy)
    vx = pv[..., 0] + mot[..., 0]
    vy = pv[..., 1] + mot[..., 1]
    vlen = np.sqrt(vx * vx + vy * vy)
    dis = np.minimum(np.maximum((vlen - f32(0.001)) * f32(10.0), f32(0)), f32(1))[..., None]
    hcol = p + r
    f = cur[..., :3] * (f32(1.0) - f32(0.9)) + hcol * f32(0.9)
    fin = f * (f32(1.0) - dis) + mu * dis
    out = np.concatenate([fin, np.ones((h, w, 1), f32)], -1)
    return out.reshape(h * w, 4)


def main():
    rng = np.random.default_rng(20240607)
    w, h, frames = 37, 21, 3
    rad, mot, outs = [], [], []
    hist = pmot = None
    for f in range(frames):
        r = rng.lognormal(-0.5, 1.2, (h * w, 4)).astype(f32)
        r[rng.uniform(size=(h * w, 4)) < 0.05] *= -1.0          # negative inputs
        r[:, 3] = 1.0
        mv = rng.normal(0.0, 0.02, (h * w, 2)).astype(f32)
        mv[rng.uniform(size=h * w) < 0.1] *= 30.0                 # far outside [0, 1]: clamp
        mv[rng.uniform(size=h * w) < 0.3] = 0.0                   # static pixels
        if hist is None:
            hist, pmot = r.copy(), mv.copy()
        o = taa_resolve(r, mv, hist, pmot, w, h)
        hist, pmot = o.copy(), mv.copy()
        rad.append(r); mot.append(mv); outs.append(o)
    np.savez_compressed(os.path.join(HERE, "taa.npz"), width=w, height=h, radiance=np.stack(rad),
                        motion=np.stack(mot), resolved=np.stack(outs))


if __name__ == "__main__":
    main()
