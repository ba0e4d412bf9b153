"""Quality guard of the MLP radiance cache: frames over a relMSE budget fall back
to plain path tracing.

Every ``check_every`` frames the guard renders a probe of the frame's view at
1/``probe_scale`` resolution twice with ``probe_spp`` samples per pixel: once
with the cache (no training step, ``cache_lr`` < 0) and once with plain path
tracing, the unbiased estimator the cache stands in for.  Their relative MSE over
``block`` x ``block`` pixel means, mean((cache - plain)^2 / (plain^2 + 0.01)),
measures the cache's bias (block means divide the probes' own noise by the block
area); above ``relmse_budget`` the following frames render plainly
until a later probe passes again.  A plain frame is rendered in cache mode with an
infinite spread threshold: no path ends in the cache, so the image is exactly the
plain tracer's (bit for bit), while the frame's training paths keep training the
network, which returns to service at the next passing probe.
"""
from __future__ import annotations

import numpy as np

from . import abi


def rel_mse(x, ref, eps: float = 1e-2) -> float:
    x = np.asarray(x, np.float64)[:, :3]
    ref = np.asarray(ref, np.float64)[:, :3]
    return float(np.mean((x - ref) ** 2 / (ref ** 2 + eps)))


def block_means(img, w: int, h: int, block: int):
    a = np.asarray(img, np.float64)[:, :3].reshape(h, w, 3)
    bh, bw = h // block, w // block
    a = a[:bh * block, :bw * block].reshape(bh, block, bw, block, 3).mean(axis=(1, 3))
    return a.reshape(-1, 3)


class RadianceCacheGuard:
    def __init__(self, tracer, relmse_budget: float = 0.05, check_every: int = 10, probe_scale: int = 4,
                 probe_spp: int = 16, block: int = 4, device=None):
        self.pt = tracer
        self.budget = float(relmse_budget)
        self.check_every = max(1, int(check_every))
        self.scale = max(1, int(probe_scale))
        self.spp = max(1, int(probe_spp))
        self.block = max(1, int(block))
        self.device = device
        self.frames = 0
        self.fallback = False
        self.last_probe = None
        self.history = []          # (frame, probe relMSE, fallback after the probe)

    def _probe_view(self, view):
        v = np.array(view, copy=True)
        w, h = max(1, int(v["width"]) // self.scale), max(1, int(v["height"]) // self.scale)
        v["width"], v["height"] = w, h
        return v, w, h

    def _render(self, view, settings, w, h):
        from . import alloc_outputs
        out = alloc_outputs(w, h, device=self.device, names=("radiance",))
        self.pt.render([view], settings, [out])
        self.pt.synchronize()
        r = out["radiance"]
        return r.cpu().numpy() if hasattr(r, "cpu") else r

    def probe(self, view, settings) -> float:
        v, w, h = self._probe_view(view)
        base = dict(spp=self.spp, max_depth=int(settings["max_depth"]), rr_depth=int(settings["rr_depth"]),
                    seed=int(settings["seed"]) + 0x5EED, frame_index=int(settings["frame_index"]))
        cached = self._render(v, abi.settings(mode=abi.MODE_PATH_CACHE, cache_lr=-1.0,
                                              cache_spread=float(settings["cache_spread"]), **base), w, h)
        plain = self._render(v, abi.settings(mode=abi.MODE_PATH, **base), w, h)
        b = min(self.block, w, h)
        e = rel_mse(block_means(cached, w, h, b), block_means(plain, w, h, b))
        self.last_probe = e
        return e

    def render(self, view, settings, outputs) -> dict:
        """Renders one frame with the cache, or plainly when the last probe was
        over budget; returns {"mode": ..., "probe_relmse": value or None}."""
        probe = None
        if self.frames % self.check_every == 0 and self.frames > 0:
            probe = self.probe(view, settings)
            self.fallback = probe > self.budget
            self.history.append((self.frames, probe, self.fallback))
        st = np.array(settings, copy=True)
        st["mode"] = abi.MODE_PATH_CACHE
        if self.fallback:
            st["cache_spread"] = 1e30     # no path terminates into the cache: plain image, training continues
        self.pt.render([view], st, [outputs])
        self.frames += 1
        return {"mode": "plain" if self.fallback else "cache", "probe_relmse": probe}
