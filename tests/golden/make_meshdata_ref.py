"""Writes tests/golden/reference_serializer.meshdata with the reference's own
ByteSerializer (oracle/build_ref.py compiles Core/headers/util/ByteSerializer.h from
the reference's sources into oracle/_ref/meshdata_writer, which serializes a fixed
mesh in the call order of AssetLoader::SerializeMeshDataBinary).  Run where the
reference's sources are present:  python tests/golden/make_meshdata_ref.py"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(HERE)), "oracle"))

import build_ref  # noqa: E402

if __name__ == "__main__":
    out = os.path.join(HERE, "reference_serializer.meshdata")
    if not build_ref.write_meshdata(out):
        sys.exit("the reference's sources are not here")
    print("wrote", out, os.path.getsize(out), "bytes")
