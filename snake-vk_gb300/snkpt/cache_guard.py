"""Quality guard of the MLP radiance cache: frames over a relMSE budget fall back
to plain path tracing.

The guard lives in the library (snk_pt_cache_set_guard, include/snk_pt.h), so C
callers get the same fallback: every ``check_every`` cache frames it renders a
probe of the frame's view at 1/``probe_scale`` resolution twice with
``probe_spp`` samples per pixel -- once with the cache (no training step) and
once with plain path tracing, the unbiased estimator the cache stands in for --
and compares them by the relative MSE over ``block`` x ``block`` pixel means,
mean((cache - plain)^2 / (plain^2 + 0.01)) (block means divide the probes' own
noise by the block area).  Above ``relmse_budget`` the following frames render
plainly until a later probe passes again: no path ends in the cache, so the image
is exactly the plain tracer's (bit for bit), while the frame's training paths keep
training the network, which returns to service at the next passing probe.

This module is the Python face of that guard (:class:`RadianceCacheGuard`) and a
numpy statement of its error measure (:func:`rel_mse` of :func:`block_means`),
which the tests hold the library's measure (:func:`relmse_library`) to.
"""
from __future__ import annotations

import ctypes as C

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


def relmse_library(cached, plain, w: int, h: int, block: int) -> float:
    """The library's measure (snk_cache_guard_relmse) of two RGBA32F host images."""
    from . import lib, SnkError
    c = np.ascontiguousarray(cached, np.float32).reshape(-1, 4)
    p = np.ascontiguousarray(plain, np.float32).reshape(-1, 4)
    out = C.c_double()
    rc = lib().snk_cache_guard_relmse(c.ctypes.data, p.ctypes.data, w, h, block, C.byref(out))
    if rc:
        raise SnkError(rc, "snk_cache_guard_relmse: bad arguments")
    return out.value


class RadianceCacheGuard:
    """Sets the library's guard on a tracer and renders frames through it."""

    def __init__(self, tracer, relmse_budget: float = 0.05, check_every: int = 10, probe_scale: int = 4,
                 probe_spp: int = 16, block: int = 4, device=None):
        self.pt = tracer
        self.device = device
        tracer.set_cache_guard(relmse_budget=float(relmse_budget), check_every=max(1, int(check_every)),
                               probe_scale=max(1, int(probe_scale)), probe_spp=max(1, int(probe_spp)),
                               block=max(1, int(block)))
        self.history = []          # (frame, probe relMSE, fallback after the probe)

    def render(self, view, settings, outputs) -> dict:
        """Renders one cache frame through the guard; returns {"mode": "cache" or
        "plain", "probe_relmse": the probe made before this frame, or None}."""
        before = self.pt.cache_guard_state()
        st = np.array(settings, copy=True)
        st["mode"] = abi.MODE_PATH_CACHE
        self.pt.render([view], st, [outputs])
        s = self.pt.cache_guard_state()
        probe = s["last_probe_relmse"] if s["probes"] > before["probes"] else None
        if probe is not None:
            self.history.append((before["frames"], probe, s["fallback"]))
        plain = s["fallback_frames"] > before["fallback_frames"]
        return {"mode": "plain" if plain else "cache", "probe_relmse": probe}
