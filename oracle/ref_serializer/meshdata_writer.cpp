// Test infrastructure: writes a .meshdata file with the reference's own serializer
// (SNAKE::ByteSerializer, Core/headers/util/ByteSerializer.h:18-65, compiled from
// the reference's header) in the call order of AssetLoader::SerializeMeshDataBinary
// (Core/src/assets/AssetLoader.cpp:146-164).  The mesh content is a fixed formula
// of the vertex / index number that tests/test_meshdata.py computes again, so the
// library's reader and the oracle's restatement can be checked against a file the
// reference's code wrote.  Usage: meshdata_writer <output path>
#include <cstdint>
#include <string>
#include <vector>

#include "util/ByteSerializer.h"

namespace {
struct Submesh {   // Core/headers/assets/MeshData.h:11-17
    unsigned num_indices, num_vertices, base_vertex, base_index, material_index;
};
struct Vec3 { float x, y, z; };   // aiVector3D
struct Vec2 { float x, y; };      // aiVector2D
}  // namespace

int main(int argc, char** argv) {
    if (argc != 2) return 2;
    const uint64_t uuid = 0x5EED0A55E7000001ull;
    std::string name = "reference_serializer";
    // two submeshes: 5 vertices / 9 indices, then 6 vertices / 12 indices
    std::vector<Submesh> submeshes = {{9u, 5u, 0u, 0u, 1u}, {12u, 6u, 5u, 9u, 0u}};
    unsigned num_vertices = 11, num_indices = 21;
    std::vector<Vec3> pos(num_vertices), nrm(num_vertices), tan(num_vertices);
    std::vector<Vec2> uv(num_vertices);
    for (unsigned i = 0; i < num_vertices; i++) {
        const float f = (float)i;
        pos[i] = {f * 0.5f - 2.0f, f * f * 0.125f, 3.0f - f * 0.25f};
        nrm[i] = {0.0f, (i % 2) ? 1.0f : -1.0f, 0.0f};
        tan[i] = {1.0f, 0.0f, f * 0.0625f};
        uv[i] = {f * 0.1f, 1.0f - f * 0.1f};
    }
    std::vector<unsigned> idx(num_indices);
    for (unsigned k = 0; k < 9; k++) idx[k] = (k * 2u + 1u) % 5u;
    for (unsigned k = 0; k < 12; k++) idx[9 + k] = (k * 5u + 2u) % 6u;
    std::vector<uint64_t> materials = {0x0A0A000000000011ull, 0x0B0B000000000022ull};
    std::vector<uint64_t> textures = {0x0C0C000000000033ull};

    SNAKE::ByteSerializer s;
    s.Value(uuid);
    s.Container(name);
    s.Container(submeshes);
    s.Value(num_vertices);
    s.Value(num_indices);
    s.Value(reinterpret_cast<const std::byte*>(pos.data()), num_vertices * sizeof(Vec3));
    s.Value(reinterpret_cast<const std::byte*>(nrm.data()), num_vertices * sizeof(Vec3));
    s.Value(reinterpret_cast<const std::byte*>(tan.data()), num_vertices * sizeof(Vec3));
    s.Value(reinterpret_cast<const std::byte*>(uv.data()), num_vertices * sizeof(Vec2));
    s.Value(reinterpret_cast<const std::byte*>(idx.data()), num_indices * sizeof(unsigned));
    s.Container(materials);
    s.Container(textures);
    s.OutputToFile(argv[1]);
    return 0;
}
