"""The .meshdata reader (snk_meshdata_*, host code) against the oracle's
restatement of the reference's ByteDeserializer reads, on a golden asset written
field by field, on round trips of the writer, and on malformed files."""
import os

import numpy as np
import pytest

import meshdata_ref as R
import snkpt
from snkpt import meshdata as MD

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "two_submeshes.meshdata")


def same_as_reference(md, ref):
    assert md.uuid == ref["uuid"] and md.name == ref["name"]
    assert np.array_equal(md.submeshes, ref["submeshes"])
    for k in ("positions", "normals", "tangents", "tex_coords", "indices", "materials", "textures"):
        assert np.array_equal(getattr(md, k), ref[k]), k


def test_golden_asset(built_lib):
    data = open(GOLDEN, "rb").read()
    md = MD.load(GOLDEN)
    same_as_reference(md, R.parse(data))
    assert md.uuid == 0x1234ABCD5678EF01 and md.name == "two_submeshes"
    assert len(md.submeshes) == 2 and md.positions.shape == (8, 3) and md.indices.size == 18
    assert list(md.materials) == [0xAAAA000000000001, 0xBBBB000000000002]
    quad, tet = md.meshes()
    assert quad.indices.shape == (2, 3) and tet.indices.shape == (4, 3)
    assert tet.indices.max() == 3                       # local to the submesh
    assert np.array_equal(tet.positions, md.positions[4:8])
    assert int(md.submeshes[1]["material_index"]) == 1


def test_writer_round_trip(built_lib):
    rng = np.random.default_rng(3)
    nv = [5, 40, 7]
    ni = [9, 90, 6]
    pos = rng.normal(size=(sum(nv), 3)).astype(np.float32)
    idx = np.concatenate([rng.integers(0, v, n) for v, n in zip(nv, ni)]).astype(np.uint32)
    sub = np.zeros(3, MD.SUBMESH_DTYPE)
    sub["num_vertices"], sub["num_indices"] = nv, ni
    sub["base_vertex"] = np.cumsum([0] + nv[:-1])
    sub["base_index"] = np.cumsum([0] + ni[:-1])
    sub["material_index"] = [2, 0, 1]
    b = MD.write(None, 99, "räume", sub, pos, -pos, pos * 2, pos[:, :2], idx, [1, 2, 3], [])
    md = MD.load(b)
    same_as_reference(md, R.parse(b))
    assert md.name == "räume" and md.textures.size == 0
    for k, m in enumerate(md.meshes()):
        assert np.array_equal(m.positions, pos[sub["base_vertex"][k]:sub["base_vertex"][k] + nv[k]])


REF_GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_serializer.meshdata")


def reference_writer_content():
    """The mesh oracle/ref_serializer/meshdata_writer.cpp serializes (same formulas)."""
    i = np.arange(11, dtype=np.float32)
    pos = np.stack([i * np.float32(0.5) - np.float32(2.0), i * i * np.float32(0.125), np.float32(3.0) - i * np.float32(0.25)], 1)
    nrm = np.stack([np.zeros(11, np.float32), np.where(np.arange(11) % 2 == 1, 1.0, -1.0).astype(np.float32),
                    np.zeros(11, np.float32)], 1)
    tan = np.stack([np.ones(11, np.float32), np.zeros(11, np.float32), i * np.float32(0.0625)], 1)
    uv = np.stack([i * np.float32(0.1), np.float32(1.0) - i * np.float32(0.1)], 1)
    idx = np.concatenate([(np.arange(9) * 2 + 1) % 5, (np.arange(12) * 5 + 2) % 6]).astype(np.uint32)
    sub = np.zeros(2, MD.SUBMESH_DTYPE)
    sub[0] = (9, 5, 0, 0, 1)
    sub[1] = (12, 6, 5, 9, 0)
    return dict(uuid=0x5EED0A55E7000001, name="reference_serializer", submeshes=sub, positions=pos, normals=nrm,
                tangents=tan, tex_coords=uv, indices=idx, materials=[0x0A0A000000000011, 0x0B0B000000000022],
                textures=[0x0C0C000000000033])


def test_asset_written_by_the_reference_serializer(built_lib, tmp_path):
    """A .meshdata written by the reference's own ByteSerializer (compiled from
    Core/headers/util/ByteSerializer.h, driven as AssetLoader::SerializeMeshDataBinary
    drives it): the library's reader and the oracle's restatement both read back
    every field of what was written.  Where the reference's sources are present the
    committed file is also regenerated and must be byte-identical."""
    import build_ref
    data = open(REF_GOLDEN, "rb").read()
    fresh = str(tmp_path / "fresh.meshdata")
    if build_ref.write_meshdata(fresh):
        assert open(fresh, "rb").read() == data
    want = reference_writer_content()
    md = MD.load(data)
    ref = R.parse(data)
    same_as_reference(md, ref)
    assert md.uuid == want["uuid"] and md.name == want["name"]
    assert np.array_equal(md.submeshes, want["submeshes"])
    for k in ("positions", "normals", "tangents", "tex_coords", "indices"):
        assert np.array_equal(getattr(md, k), want[k]), k
    assert list(md.materials) == want["materials"] and list(md.textures) == want["textures"]
    a, b = md.meshes()   # one snk_mesh per submesh, indices local to it
    assert a.indices.shape == (3, 3) and b.indices.shape == (4, 3)
    assert np.array_equal(b.positions, want["positions"][5:11])


def test_truncated_files_are_rejected(built_lib):
    data = open(GOLDEN, "rb").read()
    for cut in range(len(data)):
        with pytest.raises(snkpt.SnkError) as e:
            MD.load(data[:cut])
        assert "truncated" in str(e.value)
        with pytest.raises(R.Truncated):
            R.parse(data[:cut])
    # trailing bytes are ignored, as by the reference
    same_as_reference(MD.load(data + b"\0" * 13), R.parse(data))


def test_inconsistent_counts_and_ranges_are_rejected(built_lib):
    pos = np.zeros((4, 3), np.float32)
    sub = np.zeros(1, MD.SUBMESH_DTYPE)
    sub["num_vertices"], sub["num_indices"] = 4, 3
    # normals shorter than num_vertices
    with pytest.raises(snkpt.SnkError, match="normals"):
        MD.load(MD.write(None, 1, "x", sub, pos, pos[:3], pos, pos[:, :2], [0, 1, 2]))
    # a submesh reaching past the vertex array
    bad = sub.copy()
    bad["base_vertex"] = 2
    with pytest.raises(snkpt.SnkError, match="submesh 0"):
        MD.load(MD.write(None, 1, "x", bad, pos, pos, pos, pos[:, :2], [0, 1, 2]))
    # an index outside its submesh
    with pytest.raises(snkpt.SnkError, match="submesh 0"):
        MD.load(MD.write(None, 1, "x", sub, pos, pos, pos, pos[:, :2], [0, 1, 4]))
    # a byte count that is not a whole number of records
    b = bytearray(MD.write(None, 1, "x", sub, pos, pos, pos, pos[:, :2], [0, 1, 2]))
    off = 8 + 8 + 1          # uuid, name count, name
    b[off:off + 8] = (19).to_bytes(8, "little")
    with pytest.raises(snkpt.SnkError):
        MD.load(bytes(b))
