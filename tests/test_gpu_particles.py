"""Particle collision queries (snk_pt_contact_rays / particle_probe /
particle_constrain) against the CPU oracle's restatement of
ParticleUpdate.rgen/.rchit: bit-exact contacts (t, normal, position, velocity)."""
import numpy as np
import pytest

import oracle as O
import snkpt
from helpers import random_rays
from snkpt import abi, scenes

pytestmark = pytest.mark.gpu

DT = 1.0 / 120.0


def moving_scene():
    sc = scenes.config1(width=64, height=36)
    rng = np.random.default_rng(77)
    inst = np.array(sc.instances, copy=True)
    prev = inst["transform"].reshape(-1, 3, 4).copy()
    prev[:, :, 3] -= rng.normal(0.0, 0.05, (len(inst), 3)).astype(np.float32)   # moved since last frame
    inst["prev_transform"] = prev.reshape(inst["prev_transform"].shape)
    sc.instances = inst
    return sc


def particles_near_surfaces(sc, n, rng):
    osc = O.OracleScene(sc)
    rays = random_rays(sc, 4 * n, rng)
    hits = osc.trace(rays)
    ok = np.nonzero(hits["flags"] == 1)[0][:n]
    o = rays["o"][ok] + rays["d"][ok] * (hits["t"][ok, None] - rng.uniform(0.0, 0.6, (len(ok), 1)))
    p = np.zeros(len(ok), abi.PARTICLE_DTYPE)
    p["position_radius"][:, :3] = o
    p["position_radius"][:, 3] = rng.uniform(0.05, 0.5, len(ok))
    v = rng.normal(0.0, 3.0, (len(ok), 3))
    v[rng.uniform(size=len(ok)) < 0.05] = 0.0            # zero speed: no collision rays
    p["velocity"][:, :3] = v
    p["velocity"][:, 3] = (rng.uniform(size=len(ok)) < 0.9).astype(np.float32)   # 10 % asleep
    p["colour"][:] = 1.0
    return p


def same_bits(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint32), np.ascontiguousarray(b).view(np.uint32))


@pytest.fixture(scope="module")
def world(cuda, built_lib):
    sc = moving_scene()
    pt = snkpt.PathTracer(0)
    pt.load_scene(sc)
    return sc, pt, O.OracleScene(sc)


def test_contact_rays_bit_exact(world):
    sc, pt, osc = world
    rng = np.random.default_rng(5)
    rays = random_rays(sc, 200_000, rng)
    rays["tmax"] = rng.uniform(0.5, 60.0, len(rays))
    g, r = pt.contact_rays(rays, DT), osc.contact_rays(rays, DT)
    assert same_bits(g, r), int((g["distance"] != r["distance"]).sum())
    hit = r["distance"] > 0
    assert 0.03 < hit.mean() < 0.95
    assert np.abs(np.linalg.norm(r["normal"][hit], axis=1) - 1.0).max() < 1e-5
    assert np.abs(r["velocity"][hit]).max() > 0.0        # moving instances give contact velocity


def test_particle_probe_bit_exact(world):
    sc, pt, osc = world
    p = particles_near_surfaces(sc, 100_000, np.random.default_rng(6))
    (gc, gg), (rc, rg) = pt.particle_probe(p, DT), osc.particle_probe(p, DT)
    assert same_bits(gc, rc) and same_bits(gg, rg)
    assert (rc["distance"] > 0).mean() > 0.05 and (rg == 0.0).mean() > 0.001
    # device buffers give the same
    import torch
    t = torch.from_numpy(p.view(np.float32).reshape(-1, 12).copy()).cuda()
    dc, dg = pt.particle_probe(t, DT)
    assert same_bits(dc.cpu().numpy(), gc.view(np.float32).reshape(-1, 12)) and same_bits(dg.cpu().numpy(), gg)


def test_particle_constrain_bit_exact(world):
    sc, pt, osc = world
    rng = np.random.default_rng(9)
    p = particles_near_surfaces(sc, 50_000, rng)
    off = rng.normal(0.0, 0.5, (len(p), 3)).astype(np.float32)
    off[rng.uniform(size=len(p)) < 0.05] = 0.0           # below the 1e-5 length cut
    g, r = pt.particle_constrain(p, off, DT), osc.particle_constrain(p, off, DT)
    assert same_bits(g, r)
    assert (np.abs(r - off).max(axis=1) > 0).mean() > 0.05   # some offsets were constrained
