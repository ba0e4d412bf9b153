"""Generate the golden vectors in tests/golden/*.npz.

The reference (Snake-VK) ships no tests and no known-answer vectors, and its
shaders cannot run here (no graphics stack).  These fixtures are an independent
float64 numpy transcription of the reference GLSL, evaluated on seeded inputs:

  LightBuffers.glsl:65-124   FresnelSchlick, DistributionGGX, GeometrySchlickGGX,
                             GeometrySmith, CookTorranceBRDF
  LightBuffers.glsl:126-157  CalcDirectionalLight, CalcPointlight
  RayGen.rgen / Util.glsl    (mix(vec3(0.04), albedo, metallic) for f0, RayGen.rgen:552-553)

The CPU oracle (float32, fixed operation order) must agree with them to float
rounding.  Run:  python tests/golden/make_golden.py
"""
import os

import numpy as np

PI = 3.1415926  # LightBuffers.glsl:29
HERE = os.path.dirname(os.path.abspath(__file__))


def normalize(v):
    return v / np.linalg.norm(v, axis=-1, keepdims=True)


def fresnel_schlick(cos_theta, f0):
    return f0 + (1.0 - f0) * np.clip(1.0 - cos_theta, 0.0, 1.0)[..., None] ** 5.0


def distribution_ggx(h, n, roughness):
    a = roughness * roughness
    a2 = a * a
    ndh = np.maximum(np.sum(n * h, -1), 0.0)
    denom = ndh * ndh * (a2 - 1.0) + 1.0
    return a2 / (PI * denom * denom)


def geometry_schlick_ggx(ndv, roughness):
    r = roughness + 1.0
    k = r * r / 8.0
    return ndv / (ndv * (1.0 - k) + k)


def geometry_smith(v, l, n, roughness):
    ndv = np.maximum(np.sum(n * v, -1), 0.0)
    ndl = np.maximum(np.sum(n * l, -1), 0.0)
    return geometry_schlick_ggx(ndv, roughness) * geometry_schlick_ggx(ndl, roughness)


def brdf_terms(l, v, f0, n, roughness, metallic):
    h = normalize(v + l)
    f = fresnel_schlick(np.maximum(np.sum(h * v, -1), 0.0), f0)
    ndf = distribution_ggx(h, n, roughness)
    g = geometry_smith(v, l, n, roughness)
    ndl = np.maximum(np.sum(n * l, -1), 0.0)
    num = (ndf * g)[..., None] * f
    denom = 4.0 * np.maximum(np.sum(n * v, -1), 0.0) * ndl + 0.0001
    spec = num / denom[..., None]
    kd = (1.0 - f) * (1.0 - metallic)[..., None]
    return kd, spec, ndl


def cook_torrance(l, v, f0, n, roughness, metallic):
    kd, spec, ndl = brdf_terms(l, v, f0, n, roughness, metallic)
    return (kd / PI + spec) * ndl[..., None]


def calc_directional(ldir, colour, v, f0, n, roughness, metallic, albedo):
    kd, spec, ndl = brdf_terms(ldir, v, f0, n, roughness, metallic)
    return (kd * albedo / PI + spec) * ndl[..., None] * colour


def calc_pointlight(lpos, colour, att, world_pos, v, f0, n, roughness, metallic, albedo):
    ftl = lpos - world_pos
    d = np.linalg.norm(ftl, axis=-1)
    atten = att[:, 0] + att[:, 1] * d + att[:, 2] * d ** 2
    brdf = cook_torrance(normalize(ftl), v, f0, n, roughness, metallic)
    return brdf * albedo * colour / atten[..., None]


def f0_of(albedo, metallic):
    return 0.04 * (1.0 - metallic)[..., None] + albedo * metallic[..., None]


def unit(rng, n):
    return normalize(rng.normal(size=(n, 3)))


def main():
    rng = np.random.default_rng(20241203)
    n = 512
    nrm = unit(rng, n)
    # light/view directions in the upper hemisphere of n (plus a few grazing/below)
    l = unit(rng, n)
    l = np.where(np.sum(l * nrm, -1, keepdims=True) < 0, -l, l)
    v = unit(rng, n)
    v = np.where(np.sum(v * nrm, -1, keepdims=True) < 0, -v, v)
    l[:16] = -l[:16]            # light below the surface: n.l clamps to 0
    rough = rng.uniform(0.1, 1.0, n)
    metal = (rng.uniform(size=n) < 0.3).astype(np.float64)
    albedo = rng.uniform(0.2, 0.8, (n, 3))
    f0 = f0_of(albedo, metal)
    # round the inputs to float32 first: both sides consume the same float32 values
    f32 = lambda a: a.astype(np.float32).astype(np.float64)
    nrm, l, v, rough, metal, albedo = map(f32, (nrm, l, v, rough, metal, albedo))
    f0 = f32(f0_of(albedo, metal))
    kd, spec, ndl = brdf_terms(l, v, f0, nrm, rough, metal)
    ct = (kd / PI + spec) * ndl[..., None]
    brdf_in = np.concatenate([l, v, f0, nrm, rough[:, None], metal[:, None]], 1).astype(np.float32)
    brdf_out = np.concatenate([kd, spec, ndl[:, None], ct], 1)

    colour = f32(rng.uniform(0.5, 3.0, (n, 3)))
    dl = calc_directional(l, colour, v, f0, nrm, rough, metal, albedo)
    dir_in = np.concatenate([l, colour, v, nrm, albedo, rough[:, None], metal[:, None]], 1).astype(np.float32)

    wpos = f32(rng.uniform(-10, 10, (n, 3)))
    lpos = f32(wpos + unit(rng, n) * rng.uniform(0.5, 20.0, (n, 1)))
    att = f32(np.tile([0.5, 0.25, 0.05], (n, 1)))
    pl = calc_pointlight(lpos, colour, att, wpos, v, f0_of(albedo, metal), nrm, rough, metal, albedo)
    pl_in = np.concatenate([lpos, colour, att, wpos, v, nrm, albedo, rough[:, None], metal[:, None]], 1).astype(np.float32)

    np.savez_compressed(os.path.join(HERE, "brdf.npz"), brdf_in=brdf_in, brdf_out=brdf_out, dir_in=dir_in, dir_out=dl,
                        pl_in=pl_in, pl_out=pl)
    print("wrote", os.path.join(HERE, "brdf.npz"))


if __name__ == "__main__":
    main()
