"""Test infrastructure: a pure-Python restatement of the reference's .meshdata
reader, used only to check the library's reader.

Follows AssetLoader::DeserializeMeshData (Core/src/assets/AssetLoader.cpp:166-211)
and ByteDeserializer (Core/headers/util/ByteSerializer.h:66-112): Value(T) copies
sizeof(T) bytes; Value(T*&, ...) and Container(...) read a size_t byte count
(8 bytes on the reference's 64-bit builds) then that many bytes; every read
asserts it stays inside the buffer.
"""
import struct

import numpy as np

SUBMESH_DTYPE = np.dtype([("num_indices", "<u4"), ("num_vertices", "<u4"), ("base_vertex", "<u4"),
                          ("base_index", "<u4"), ("material_index", "<u4")])


class Truncated(ValueError):
    pass


def parse(data: bytes) -> dict:
    pos = 0

    def value(fmt):
        nonlocal pos
        n = struct.calcsize(fmt)
        if pos + n > len(data):
            raise Truncated(f"value at {pos}")
        v = struct.unpack_from(fmt, data, pos)[0]
        pos += n
        return v

    def blob():
        nonlocal pos
        size = value("<Q")
        if pos + size > len(data):
            raise Truncated(f"block of {size} bytes at {pos}")
        b = data[pos:pos + size]
        pos += size
        return b

    out = {"uuid": value("<Q")}
    out["name"] = blob().decode("utf-8")
    out["submeshes"] = np.frombuffer(blob(), SUBMESH_DTYPE).copy()
    out["num_vertices"] = value("<I")
    out["num_indices"] = value("<I")
    out["positions"] = np.frombuffer(blob(), np.float32).reshape(-1, 3).copy()
    out["normals"] = np.frombuffer(blob(), np.float32).reshape(-1, 3).copy()
    out["tangents"] = np.frombuffer(blob(), np.float32).reshape(-1, 3).copy()
    out["tex_coords"] = np.frombuffer(blob(), np.float32).reshape(-1, 2).copy()
    out["indices"] = np.frombuffer(blob(), np.uint32).copy()
    out["materials"] = np.frombuffer(blob(), np.uint64).copy()
    out["textures"] = np.frombuffer(blob(), np.uint64).copy()
    return out
