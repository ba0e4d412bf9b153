"""Test infrastructure: builds the parts of the reference that compile here
(oracle/_ref/, kept out of the repository's history).

meshdata_writer: the reference's ByteSerializer (Core/headers/util/ByteSerializer.h)
compiled from the reference's own header, with stand-ins for the two engine
headers it includes (oracle/ref_serializer/util/), driven in the call order of
AssetLoader::SerializeMeshDataBinary.  Needs the reference's sources, which exist
only where the repository is developed; elsewhere build() returns None.
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF_HEADERS = "/root/reference/Core/headers"
OUT = os.path.join(HERE, "_ref")
WRITER = os.path.join(OUT, "meshdata_writer")


def build() -> str | None:
    if not os.path.exists(os.path.join(REF_HEADERS, "util", "ByteSerializer.h")):
        return None
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(HERE, "ref_serializer", "meshdata_writer.cpp")
    # the stand-ins come first, so the reference header's "util/..." includes find them
    subprocess.check_call(["g++", "-std=c++20", "-O1", "-I", os.path.join(HERE, "ref_serializer"), "-I",
                           REF_HEADERS, src, "-o", WRITER + ".tmp"])
    os.replace(WRITER + ".tmp", WRITER)
    return WRITER


def write_meshdata(path: str) -> bool:
    """Writes the reference-serialized asset to path; False when the writer cannot be built."""
    w = build()
    if not w:
        return False
    subprocess.check_call([w, path])
    return True


if __name__ == "__main__":
    print(build())
