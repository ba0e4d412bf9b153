"""Generate tests/golden/two_submeshes.meshdata, a small asset in the byte layout
of AssetLoader::SerializeMeshDataBinary (Core/src/assets/AssetLoader.cpp:146-164)
written field by field with struct (independently of the library's writer):

  submesh 0: a unit quad in the xz plane (4 vertices, 2 triangles), material 0
  submesh 1: a tetrahedron above it (4 vertices, 4 triangles), material 1

Indices are local to each submesh (the reference's BLAS reads positions from
base_vertex and indices from base_index).  Run:
python tests/golden/make_meshdata_golden.py
"""
import os
import struct

HERE = os.path.dirname(os.path.abspath(__file__))

UUID = 0x1234ABCD5678EF01
NAME = "two_submeshes"
QUAD = [(-1.0, 0.0, -1.0), (1.0, 0.0, -1.0), (1.0, 0.0, 1.0), (-1.0, 0.0, 1.0)]
QUAD_IDX = [0, 2, 1, 0, 3, 2]
TETRA = [(0.0, 0.5, 0.0), (0.5, 0.5, 0.0), (0.0, 1.0, 0.0), (0.0, 0.5, 0.5)]
TETRA_IDX = [0, 1, 2, 0, 2, 3, 0, 3, 1, 1, 3, 2]
MATERIALS = [0xAAAA000000000001, 0xBBBB000000000002]
TEXTURES = [0xCCCC000000000003]


def block(b: bytes) -> bytes:
    return struct.pack("<Q", len(b)) + b


def build() -> bytes:
    pos = QUAD + TETRA
    nrm = [(0.0, 1.0, 0.0)] * 4 + [(0.0, 0.0, 1.0)] * 4
    tan = [(1.0, 0.0, 0.0)] * 8
    uv = [(0.0, 0.0), (1.0, 0.0), (1.0, 1.0), (0.0, 1.0)] * 2
    idx = QUAD_IDX + TETRA_IDX
    sub = struct.pack("<5I", len(QUAD_IDX), 4, 0, 0, 0) + struct.pack("<5I", len(TETRA_IDX), 4, 4, len(QUAD_IDX), 1)
    f3 = lambda rows: b"".join(struct.pack("<3f", *r) for r in rows)
    return b"".join([
        struct.pack("<Q", UUID), block(NAME.encode()), block(sub), struct.pack("<II", len(pos), len(idx)),
        block(f3(pos)), block(f3(nrm)), block(f3(tan)), block(b"".join(struct.pack("<2f", *r) for r in uv)),
        block(struct.pack(f"<{len(idx)}I", *idx)), block(struct.pack(f"<{len(MATERIALS)}Q", *MATERIALS)),
        block(struct.pack(f"<{len(TEXTURES)}Q", *TEXTURES))])


if __name__ == "__main__":
    with open(os.path.join(HERE, "two_submeshes.meshdata"), "wb") as f:
        f.write(build())
