"""Seeded synthetic scenes for the five benchmark configurations.

The reference renders whatever the editor scene holds (meshes from
``.meshdata`` assets, ``StaticMeshComponent`` instances, point/spot lights,
one directional light).  There are no test scenes in the reference, so the
workloads are generated here with fixed seeds:

* config 0 -- closed 10x10x10 room, 32x32 floor grid, 5 boxes, 2x2 ceiling light
* config 1 -- 200 icosphere-3 instances over a 256x256 ground grid, 1 directional
  light and 16 sphere lights (two-level BVH)
* config 2 -- config 1 plus 4096 emissive quads (ReSTIR DI stress)
* config 3 -- 64 instances of a 256x256 value-noise terrain tile plus config 1's
  spheres, 8 uneven views
* config 4 -- config 3's geometry, one 1080p view flying a seeded spline

All arrays use the layouts of ``include/snk_pt.h`` (see ``snkpt.abi``): a mesh
is float32 positions/normals (V,3) and uint32 indices (T,3); an instance holds
two row-major 3x4 object-to-world transforms (current and previous frame), a
mesh id and a material id (the reference's ``InstanceData``,
``Core/headers/scene/RaytracingBufferSystem.h:14-28``); a material is the
reference's ``Material`` (``Core/res/shaders/TexMatBuffers.glsl:5-20``) without
texture indices.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import abi

MAT_EMISSIVE = 1


@dataclass
class Mesh:
    positions: np.ndarray  # (V,3) float32
    normals: np.ndarray    # (V,3) float32
    indices: np.ndarray    # (T,3) uint32

    @property
    def num_triangles(self) -> int:
        return int(self.indices.shape[0])


@dataclass
class Scene:
    meshes: list
    instances: np.ndarray      # abi.INSTANCE_DTYPE
    materials: np.ndarray      # abi.MATERIAL_DTYPE
    dir_light: np.ndarray      # abi.DIR_LIGHT_DTYPE (shape ())
    point_lights: np.ndarray   # abi.POINT_LIGHT_DTYPE
    views: list = field(default_factory=list)   # list of abi.VIEW_DTYPE scalars
    name: str = ""

    @property
    def num_instanced_triangles(self) -> int:
        return int(sum(self.meshes[int(m)].num_triangles for m in self.instances["mesh_id"]))


# ----------------------------------------------------------------------------
# meshes
# ----------------------------------------------------------------------------

def grid_mesh(nx: int, nz: int, size_x: float, size_z: float, height=None) -> Mesh:
    """(nx x nz) quads in the xz plane centred at the origin, 2 triangles each.

    ``height`` is an optional (nz+1, nx+1) array of y displacements.  Normals
    come from central differences of the height field (flat +y when absent).
    """
    xs = np.linspace(-0.5 * size_x, 0.5 * size_x, nx + 1)
    zs = np.linspace(-0.5 * size_z, 0.5 * size_z, nz + 1)
    X, Z = np.meshgrid(xs, zs)            # (nz+1, nx+1)
    Y = np.zeros_like(X) if height is None else np.asarray(height, np.float64)
    pos = np.stack([X, Y, Z], -1).reshape(-1, 3)
    if height is None:
        nrm = np.tile([0.0, 1.0, 0.0], (pos.shape[0], 1))
    else:
        dx = size_x / nx
        dz = size_z / nz
        gy = np.gradient(Y, dz, axis=0)
        gx = np.gradient(Y, dx, axis=1)
        n = np.stack([-gx, np.ones_like(Y), -gy], -1).reshape(-1, 3)
        nrm = n / np.linalg.norm(n, axis=1, keepdims=True)
    i = np.arange(nz)[:, None] * (nx + 1) + np.arange(nx)[None, :]
    i = i.reshape(-1)
    a, b, c, d = i, i + 1, i + nx + 1, i + nx + 2
    tris = np.stack([np.stack([a, c, b], 1), np.stack([b, c, d], 1)], 1).reshape(-1, 3)
    return Mesh(pos.astype(np.float32), nrm.astype(np.float32), tris.astype(np.uint32))


def quad_mesh() -> Mesh:
    """Unit quad in the xz plane, normal +y, 2 triangles."""
    pos = np.array([[-0.5, 0, -0.5], [0.5, 0, -0.5], [0.5, 0, 0.5], [-0.5, 0, 0.5]], np.float32)
    nrm = np.tile(np.array([0, 1, 0], np.float32), (4, 1))
    idx = np.array([[0, 2, 1], [0, 3, 2]], np.uint32)
    return Mesh(pos, nrm, idx)


def cube_mesh() -> Mesh:
    """Unit cube centred at the origin, flat normals, 12 triangles."""
    pos, nrm, idx = [], [], []
    for axis in range(3):
        for sign in (-1.0, 1.0):
            n = np.zeros(3)
            n[axis] = sign
            u = np.zeros(3)
            u[(axis + 1) % 3] = 1.0
            v = np.cross(n, u)
            c = 0.5 * n
            base = len(pos)
            for su, sv in ((-1, -1), (1, -1), (1, 1), (-1, 1)):
                pos.append(c + 0.5 * su * u + 0.5 * sv * v)
                nrm.append(n)
            idx += [[base, base + 1, base + 2], [base, base + 2, base + 3]]
    return Mesh(np.array(pos, np.float32), np.array(nrm, np.float32), np.array(idx, np.uint32))


def icosphere(subdiv: int) -> Mesh:
    """Icosahedron subdivided ``subdiv`` times (subdiv 3: 642 vertices, 1280 triangles)."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t),
             (0, -1, -t), (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = [np.array(v, np.float64) / np.linalg.norm(v) for v in verts]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
             (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
             (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(subdiv):
        cache = {}

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    p = np.array(verts, np.float32)
    return Mesh(p, p.copy(), np.array(faces, np.uint32))


def value_noise(n: int, octaves: int, rng: np.random.Generator) -> np.ndarray:
    """(n+1, n+1) fractal value noise in [-1,1]-ish, ``octaves`` octaves, smoothstep interpolation."""
    out = np.zeros((n + 1, n + 1))
    amp, total = 1.0, 0.0
    cells = 4
    coords = np.linspace(0.0, 1.0, n + 1)
    for _ in range(octaves):
        lat = rng.uniform(-1.0, 1.0, (cells + 1, cells + 1))
        f = coords * cells
        i0 = np.minimum(np.floor(f).astype(int), cells - 1)
        tt = f - i0
        s = tt * tt * (3.0 - 2.0 * tt)
        a = lat[np.ix_(i0, i0)]
        b = lat[np.ix_(i0, i0 + 1)]
        c = lat[np.ix_(i0 + 1, i0)]
        d = lat[np.ix_(i0 + 1, i0 + 1)]
        sx = s[None, :]
        sz = s[:, None]
        out += amp * ((a * (1 - sx) + b * sx) * (1 - sz) + (c * (1 - sx) + d * sx) * sz)
        total += amp
        amp *= 0.5
        cells *= 2
    return out / total


# ----------------------------------------------------------------------------
# transforms, materials, cameras
# ----------------------------------------------------------------------------

def rot_x(a):
    c, s = math.cos(a), math.sin(a)
    return np.array([[1, 0, 0], [0, c, -s], [0, s, c]])


def rot_y(a):
    c, s = math.cos(a), math.sin(a)
    return np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]])


def random_rotation(rng) -> np.ndarray:
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def affine(R=None, scale=(1.0, 1.0, 1.0), t=(0.0, 0.0, 0.0)) -> np.ndarray:
    """Row-major 3x4 object-to-world matrix  R @ diag(scale) | t  as float32."""
    R = np.eye(3) if R is None else np.asarray(R, np.float64)
    A = R @ np.diag(np.asarray(scale, np.float64))
    return np.concatenate([A, np.asarray(t, np.float64)[:, None]], 1).astype(np.float32)


def random_material(rng) -> tuple:
    """Lambert+GGX parameters: albedo U[0.2,0.8]^3, roughness U[0.1,1], metallic Bernoulli(0.2)."""
    albedo = rng.uniform(0.2, 0.8, 3)
    rough = rng.uniform(0.1, 1.0)
    metal = 1.0 if rng.uniform() < 0.2 else 0.0
    return albedo, rough, metal


def make_materials(rows) -> np.ndarray:
    m = np.zeros(len(rows), abi.MATERIAL_DTYPE)
    for i, (albedo, rough, metal, flags) in enumerate(rows):
        m[i]["albedo"] = albedo
        m[i]["roughness"] = rough
        m[i]["metallic"] = metal
        m[i]["ao"] = 1.0
        m[i]["flags"] = flags
    return m


def make_instances(rows) -> np.ndarray:
    inst = np.zeros(len(rows), abi.INSTANCE_DTYPE)
    for i, (M, mesh, mat) in enumerate(rows):
        inst[i]["transform"] = np.asarray(M, np.float32).reshape(12)
        inst[i]["prev_transform"] = np.asarray(M, np.float32).reshape(12)
        inst[i]["mesh_id"] = mesh
        inst[i]["material_id"] = mat
    return inst


def look_at_view(pos, target, fov_y_deg, width, height, prev=None) -> np.ndarray:
    """Pinhole view with an orthonormal basis (y up); ``prev`` is the previous frame's view."""
    pos = np.asarray(pos, np.float64)
    fwd = np.asarray(target, np.float64) - pos
    fwd /= np.linalg.norm(fwd)
    right = np.cross(fwd, [0.0, 1.0, 0.0])
    right /= np.linalg.norm(right)
    up = np.cross(right, fwd)
    v = np.zeros((), abi.VIEW_DTYPE)
    v["pos"] = pos
    v["forward"] = fwd
    v["right"] = right
    v["up"] = up
    v["tan_half_fov_y"] = math.tan(math.radians(fov_y_deg) * 0.5)
    v["aspect"] = width / height
    v["width"] = width
    v["height"] = height
    src = v if prev is None else prev
    v["prev_pos"] = src["pos"]
    v["prev_forward"] = src["forward"]
    v["prev_right"] = src["right"]
    v["prev_up"] = src["up"]
    v["prev_tan_half_fov_y"] = src["tan_half_fov_y"]
    v["prev_aspect"] = src["aspect"]
    v["prev_valid"] = 0 if prev is None else 1
    return v


def dir_light(direction, colour) -> np.ndarray:
    d = np.asarray(direction, np.float64)
    d /= np.linalg.norm(d)
    L = np.zeros((), abi.DIR_LIGHT_DTYPE)
    L["dir"] = d
    L["colour"] = colour
    L["enabled"] = 1
    return L


def no_dir_light() -> np.ndarray:
    return np.zeros((), abi.DIR_LIGHT_DTYPE)


def point_lights(rows) -> np.ndarray:
    """rows of (pos, radius, colour); attenuation uses the reference defaults
    c=0.5, l=0.25, e=0.05 (``Core/headers/components/Lights.h:6-10``)."""
    p = np.zeros(len(rows), abi.POINT_LIGHT_DTYPE)
    for i, (pos, radius, colour) in enumerate(rows):
        p[i]["pos"] = pos
        p[i]["radius"] = radius
        p[i]["colour"] = colour
        p[i]["atten_constant"] = 0.5
        p[i]["atten_linear"] = 0.25
        p[i]["atten_exp"] = 0.05
    return p


# ----------------------------------------------------------------------------
# configs
# ----------------------------------------------------------------------------

def config0(seed: int = 1, width: int = 256, height: int = 256) -> Scene:
    rng = np.random.default_rng(1000 + seed)
    meshes = [grid_mesh(32, 32, 10.0, 10.0), quad_mesh(), cube_mesh()]
    mats, inst = [], []
    # floor (32x32 quads, 2048 triangles)
    mats.append((*random_material(rng), 0))
    inst.append((affine(t=(0, 0, 0)), 0, 0))
    # 4 walls + ceiling (unit quad scaled to 10x10, normals inward)
    walls = [
        (rot_x(-math.pi / 2), (0, 5, 5)),   # z=+5, normal -z
        (rot_x(math.pi / 2), (0, 5, -5)),   # z=-5, normal +z
        (rot_y(math.pi / 2) @ rot_x(-math.pi / 2), (5, 5, 0)),
        (rot_y(-math.pi / 2) @ rot_x(-math.pi / 2), (-5, 5, 0)),
        (rot_x(math.pi), (0, 10, 0)),       # ceiling, normal -y
    ]
    for R, t in walls:
        mats.append((*random_material(rng), 0))
        inst.append((affine(R, (10, 1, 10), t), 1, len(mats) - 1))
    # 5 axis-aligned boxes, sizes U[0.5,3], standing on the floor
    for _ in range(5):
        size = rng.uniform(0.5, 3.0, 3)
        cx, cz = rng.uniform(-4.0 + size[0] / 2, 4.0 - size[0] / 2), rng.uniform(-4.0 + size[2] / 2, 4.0 - size[2] / 2)
        mats.append((*random_material(rng), 0))
        inst.append((affine(None, size, (cx, size[1] / 2, cz)), 2, len(mats) - 1))
    # 2x2 area light just below the ceiling, facing down, radiance 15
    mats.append(((15.0, 15.0, 15.0), 1.0, 0.0, MAT_EMISSIVE))
    inst.append((affine(rot_x(math.pi), (2, 1, 2), (0, 9.99, 0)), 1, len(mats) - 1))
    view = look_at_view((0.0, 5.0, -4.8), (0.0, 3.5, 5.0), 60.0, width, height)
    return Scene(meshes, make_instances(inst), make_materials(mats), no_dir_light(),
                 point_lights([]), [view], "config0")


def _sphere_field(rng, meshes, mats, inst, sphere_mesh_id):
    for _ in range(200):
        p = rng.uniform(0.0, 100.0, 3)
        s = rng.uniform(0.5, 4.0)
        R = random_rotation(rng)
        mats.append((*random_material(rng), 0))
        inst.append((affine(R, (s, s, s), p), sphere_mesh_id, len(mats) - 1))


def _config1_lights(rng):
    rows = []
    for _ in range(16):
        pos = rng.uniform(5.0, 50.0, 3)
        intensity = rng.uniform(5.0, 50.0)
        rows.append((pos, 0.5, (intensity, intensity, intensity)))
    return dir_light((0.35, 1.0, 0.25), (2.4, 2.3, 2.1)), point_lights(rows)


def config1(seed: int = 1, width: int = 1920, height: int = 1080) -> Scene:
    rng = np.random.default_rng(2000 + seed)
    meshes = [icosphere(3), grid_mesh(256, 256, 200.0, 200.0)]
    mats, inst = [], []
    _sphere_field(rng, meshes, mats, inst, 0)
    mats.append((*random_material(rng), 0))
    inst.append((affine(t=(50.0, 0.0, 50.0)), 1, len(mats) - 1))
    dl, pl = _config1_lights(rng)
    view = look_at_view((50.0, 45.0, -55.0), (50.0, 15.0, 50.0), 60.0, width, height)
    return Scene(meshes, make_instances(inst), make_materials(mats), dl, pl, [view], "config1")


def config2(seed: int = 1, width: int = 1920, height: int = 1080, frames: int = 16) -> Scene:
    sc = config1(seed, width, height)
    rng = np.random.default_rng(3000 + seed)
    meshes = sc.meshes + [quad_mesh()]
    quad_id = len(meshes) - 1
    mats = [tuple(r) for r in zip(sc.materials["albedo"], sc.materials["roughness"],
                                  sc.materials["metallic"], sc.materials["flags"])]
    rows = [(sc.instances[i]["transform"].reshape(3, 4), int(sc.instances[i]["mesh_id"]),
             int(sc.instances[i]["material_id"])) for i in range(len(sc.instances))]
    for _ in range(4096):
        side = rng.uniform(0.1, 0.5)
        L = rng.uniform(1.0, 20.0, 3)
        p = rng.uniform(0.0, 100.0, 3)
        R = random_rotation(rng)
        mats.append((L, 1.0, 0.0, MAT_EMISSIVE))
        rows.append((affine(R, (side, 1.0, side), p), quad_id, len(mats) - 1))
    views = []
    base = sc.views[0]
    prev = None
    for f in range(frames):
        off = np.array([0.05 * f, 0.0, 0.0])
        v = look_at_view(base["pos"] + off, np.array([50.0, 15.0, 50.0]) + off, 60.0, width, height, prev)
        views.append(v)
        prev = v
    return Scene(meshes, make_instances(rows), make_materials(mats), sc.dir_light, sc.point_lights,
                 views, "config2")


CONFIG3_RESOLUTIONS = [(640, 360), (960, 540), (1280, 720), (1600, 900), (1920, 1080), (1920, 1080),
                       (2560, 1440), (3840, 2160)]


def terrain_tile(rng, n: int = 256, size: float = 32.0, amplitude: float = 5.0) -> Mesh:
    h = value_noise(n, 6, rng) * amplitude
    return grid_mesh(n, n, size, size, h)


def config3(seed: int = 1, resolutions=None) -> Scene:
    rng = np.random.default_rng(4000 + seed)
    resolutions = CONFIG3_RESOLUTIONS if resolutions is None else resolutions
    meshes = [icosphere(3), terrain_tile(rng)]
    mats, inst = [], []
    srng = np.random.default_rng(2000 + seed)
    _sphere_field(srng, meshes, mats, inst, 0)
    for k in range(64):
        gx, gz = k % 8, k // 8
        p = (-60.0 + 32.0 * gx + rng.uniform(-3, 3), rng.uniform(-2.0, 0.0), -60.0 + 32.0 * gz + rng.uniform(-3, 3))
        R = rot_y(rng.uniform(0, 2 * math.pi))
        mats.append((*random_material(rng), 0))
        inst.append((affine(R, (1, 1, 1), p), 1, len(mats) - 1))
    dl, pl = _config1_lights(srng)
    views = []
    for k, (w, h) in enumerate(resolutions):
        a = 2 * math.pi * k / len(resolutions)
        pos = (50 + 90 * math.cos(a), 30 + 5 * k, 50 + 90 * math.sin(a))
        views.append(look_at_view(pos, (50.0, 5.0, 50.0), 60.0, w, h))
    return Scene(meshes, make_instances(inst), make_materials(mats), dl, pl, views, "config3")


def spline_path(seed: int, frames: int):
    """Seeded Catmull-Rom camera path over the config 3/4 terrain."""
    rng = np.random.default_rng(5000 + seed)
    ctrl = np.stack([rng.uniform(-20, 120, 8), rng.uniform(15, 45, 8), rng.uniform(-20, 120, 8)], 1)
    pts = []
    for f in range(frames):
        s = f / max(frames - 1, 1) * (len(ctrl) - 3)
        i = min(int(s), len(ctrl) - 4)
        t = s - i
        p0, p1, p2, p3 = ctrl[i:i + 4]
        pts.append(0.5 * ((2 * p1) + (-p0 + p2) * t + (2 * p0 - 5 * p1 + 4 * p2 - p3) * t * t
                          + (-p0 + 3 * p1 - 3 * p2 + p3) * t ** 3))
    return pts


def config4(seed: int = 1, width: int = 1920, height: int = 1080, frames: int = 120) -> Scene:
    sc = config3(seed, resolutions=[(width, height)])
    path = spline_path(seed, frames + 1)
    views, prev = [], None
    for f in range(frames):
        v = look_at_view(path[f], path[f + 1] + np.array([0.0, -12.0, 0.0]), 60.0, width, height, prev)
        views.append(v)
        prev = v
    sc.views = views
    sc.name = "config4"
    return sc


CONFIGS = {0: config0, 1: config1, 2: config2, 3: config3, 4: config4}


def make(config: int, **kw) -> Scene:
    return CONFIGS[config](**kw)
