"""Snake-VK ``.meshdata`` assets through the library's reader (snk_meshdata_*).

``load`` mirrors AssetLoader::DeserializeMeshData
(Core/src/assets/AssetLoader.cpp:166-211): it returns the asset's uuid, name,
submesh records, vertex arrays and material/texture UUIDs, and ``meshes()``
gives one mesh per submesh, the unit the reference builds a BLAS for
(BLAS::GenerateFromMeshData, Core/src/resources/TLAS.cpp:109-186).  ``write``
produces the byte layout of AssetLoader::SerializeMeshDataBinary (:146-164) for
tools and tests.
"""
from __future__ import annotations

import ctypes as C
import struct
from dataclasses import dataclass, field

import numpy as np

from . import Mesh as _CMesh
from . import SnkError, lib
from .scenes import Mesh

SUBMESH_DTYPE = np.dtype([("num_indices", "<u4"), ("num_vertices", "<u4"), ("base_vertex", "<u4"),
                          ("base_index", "<u4"), ("material_index", "<u4")])


class _Info(C.Structure):
    _fields_ = [("uuid", C.c_uint64), ("name", C.c_void_p), ("name_len", C.c_uint64),
                ("num_submeshes", C.c_uint32), ("num_vertices", C.c_uint32), ("num_indices", C.c_uint32),
                ("num_materials", C.c_uint32), ("num_textures", C.c_uint32), ("pad", C.c_uint32),
                ("submeshes", C.c_void_p), ("positions", C.c_void_p), ("normals", C.c_void_p),
                ("tangents", C.c_void_p), ("tex_coords", C.c_void_p), ("indices", C.c_void_p),
                ("materials", C.c_void_p), ("textures", C.c_void_p)]


def _array(ptr, n, dtype, shape=None):
    if n == 0:
        return np.zeros(shape or (0,), dtype)
    raw = C.string_at(ptr, n * np.dtype(dtype).itemsize)
    a = np.frombuffer(raw, dtype=dtype).copy()
    return a.reshape(shape) if shape else a


@dataclass
class MeshData:
    uuid: int
    name: str
    submeshes: np.ndarray            # SUBMESH_DTYPE
    positions: np.ndarray            # (V, 3) float32
    normals: np.ndarray
    tangents: np.ndarray
    tex_coords: np.ndarray           # (V, 2) float32
    indices: np.ndarray              # (I,) uint32
    materials: np.ndarray            # uint64 UUIDs
    textures: np.ndarray             # uint64 UUIDs
    _submesh_meshes: list = field(default_factory=list, repr=False)

    def meshes(self) -> list:
        """One scenes.Mesh per submesh (local indices, as its BLAS sees them)."""
        return list(self._submesh_meshes)


def load(src) -> MeshData:
    """Parse a .meshdata file (path) or its bytes with the library's reader."""
    data = src if isinstance(src, (bytes, bytearray, memoryview)) else open(src, "rb").read()
    buf = C.create_string_buffer(bytes(data), len(data))
    h = C.c_void_p()
    err = C.create_string_buffer(512)
    rc = lib().snk_meshdata_load(C.cast(buf, C.c_void_p), len(data), C.byref(h), err, 512)
    if rc != 0:
        raise SnkError(rc, err.value.decode(errors="replace"))
    try:
        info = _Info()
        rc = lib().snk_meshdata_get_info(h, C.byref(info))
        if rc != 0:
            raise SnkError(rc, "snk_meshdata_get_info failed")
        nv, ni = info.num_vertices, info.num_indices
        md = MeshData(
            uuid=int(info.uuid),
            name=C.string_at(info.name, info.name_len).decode("utf-8", errors="replace") if info.name_len else "",
            submeshes=_array(info.submeshes, info.num_submeshes, SUBMESH_DTYPE),
            positions=_array(info.positions, 3 * nv, np.float32, (nv, 3)),
            normals=_array(info.normals, 3 * nv, np.float32, (nv, 3)),
            tangents=_array(info.tangents, 3 * nv, np.float32, (nv, 3)),
            tex_coords=_array(info.tex_coords, 2 * nv, np.float32, (nv, 2)),
            indices=_array(info.indices, ni, np.uint32),
            materials=_array(info.materials, info.num_materials, np.uint64),
            textures=_array(info.textures, info.num_textures, np.uint64))
        for k in range(info.num_submeshes):
            m = _CMesh()
            rc = lib().snk_meshdata_submesh(h, k, C.byref(m))
            if rc != 0:
                raise SnkError(rc, f"submesh {k} is out of range of the asset's arrays")
            pos = _array(m.positions, 3 * m.num_vertices, np.float32, (m.num_vertices, 3))
            nrm = _array(m.normals, 3 * m.num_vertices, np.float32, (m.num_vertices, 3))
            idx = _array(m.indices, 3 * m.num_triangles, np.uint32, (m.num_triangles, 3))
            md._submesh_meshes.append(Mesh(pos, nrm, idx))
        return md
    finally:
        lib().snk_meshdata_free(h)


def write(path_or_none, uuid: int, name: str, submeshes, positions, normals, tangents, tex_coords, indices,
          materials=(), textures=()) -> bytes:
    """The byte layout of AssetLoader::SerializeMeshDataBinary; writes it to
    `path_or_none` when given and returns it."""
    def block(b: bytes) -> bytes:
        return struct.pack("<Q", len(b)) + b
    sub = np.asarray(submeshes, SUBMESH_DTYPE) if not isinstance(submeshes, np.ndarray) else \
        submeshes.astype(SUBMESH_DTYPE)
    pos = np.ascontiguousarray(positions, np.float32)
    idx = np.ascontiguousarray(indices, np.uint32).reshape(-1)
    out = b"".join([
        struct.pack("<Q", uuid), block(name.encode("utf-8")), block(sub.tobytes()),
        struct.pack("<II", pos.shape[0], idx.size),
        block(pos.tobytes()), block(np.ascontiguousarray(normals, np.float32).tobytes()),
        block(np.ascontiguousarray(tangents, np.float32).tobytes()),
        block(np.ascontiguousarray(tex_coords, np.float32).tobytes()), block(idx.tobytes()),
        block(np.asarray(materials, np.uint64).tobytes()), block(np.asarray(textures, np.uint64).tobytes())])
    if path_or_none:
        with open(path_or_none, "wb") as f:
            f.write(out)
    return out
