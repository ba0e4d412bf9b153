// meshdata.cpp -- reader of the reference's .meshdata binary mesh assets.
//
// AssetLoader::DeserializeMeshData (Core/src/assets/AssetLoader.cpp:166-211)
// reads, through ByteDeserializer (Core/headers/util/ByteSerializer.h:66-112), the
// sequence SerializeMeshDataBinary (:146-164) wrote: a u64 uuid, the name, the
// submesh records, two u32 counts, five length-prefixed vertex/index arrays and
// the material and texture UUID lists.  Every length prefix is a 64-bit byte
// count.  This reader bounds-checks each field, checks the vertex arrays against
// the counts, and copies the arrays into aligned storage owned by the handle
// (the reference copies them into new[] arrays the same way).
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/snk_pt.h"

struct snk_meshdata {
    uint64_t uuid = 0;
    std::string name;
    std::vector<snk_submesh> submeshes;
    uint32_t num_vertices = 0, num_indices = 0;
    std::vector<float> positions, normals, tangents, tex_coords;
    std::vector<uint32_t> indices;
    std::vector<uint64_t> materials, textures;
};

namespace {

struct Reader {
    const unsigned char* p;
    size_t size, pos = 0;
    std::string err;

    bool take(void* dst, size_t n, const char* what) {
        if (n > size - pos) {
            err = std::string("truncated .meshdata: ") + what + " needs " + std::to_string(n) + " bytes at offset " +
                  std::to_string(pos) + ", " + std::to_string(size - pos) + " left";
            return false;
        }
        if (n) std::memcpy(dst, p + pos, n);
        pos += n;
        return true;
    }
    // a length-prefixed block of whole elements of `elem` bytes
    template <class T>
    bool block(std::vector<T>& out, size_t elem, const char* what) {
        uint64_t bytes = 0;
        if (!take(&bytes, 8, what)) return false;
        if (bytes > size - pos) {
            err = std::string("truncated .meshdata: ") + what + " declares " + std::to_string(bytes) + " bytes, " +
                  std::to_string(size - pos) + " left";
            return false;
        }
        if (bytes % elem) {
            err = std::string(".meshdata: ") + what + " size " + std::to_string(bytes) + " is not a multiple of " +
                  std::to_string(elem);
            return false;
        }
        out.resize(bytes / sizeof(T));
        return take(out.data(), bytes, what);
    }
};

void set_err(char* err, size_t len, const std::string& msg) {
    if (!err || !len) return;
    std::strncpy(err, msg.c_str(), len - 1);
    err[len - 1] = 0;
}

}  // namespace

extern "C" {

int snk_meshdata_load(const void* bytes, size_t size, snk_meshdata** out, char* err, size_t err_len) {
    if (!out || (size && !bytes)) {
        set_err(err, err_len, "meshdata_load: null argument");
        return SNK_ERR_INVALID_ARG;
    }
    *out = nullptr;
    Reader r{static_cast<const unsigned char*>(bytes), size};
    snk_meshdata* md = new snk_meshdata();
    std::vector<char> name;
    std::vector<unsigned char> sub_raw;
    bool ok = r.take(&md->uuid, 8, "uuid") && r.block(name, 1, "name") && r.block(sub_raw, sizeof(snk_submesh), "submeshes") &&
              r.take(&md->num_vertices, 4, "num_vertices") && r.take(&md->num_indices, 4, "num_indices") &&
              r.block(md->positions, 12, "positions") && r.block(md->normals, 12, "normals") &&
              r.block(md->tangents, 12, "tangents") && r.block(md->tex_coords, 8, "tex_coords") &&
              r.block(md->indices, 4, "indices") && r.block(md->materials, 8, "materials") &&
              r.block(md->textures, 8, "textures");
    if (ok) {
        const uint64_t nv = md->num_vertices, ni = md->num_indices;
        const struct { const char* what; size_t have, want; } checks[] = {
            {"positions", md->positions.size(), 3 * nv}, {"normals", md->normals.size(), 3 * nv},
            {"tangents", md->tangents.size(), 3 * nv},   {"tex_coords", md->tex_coords.size(), 2 * nv},
            {"indices", md->indices.size(), ni}};
        for (const auto& c : checks)
            if (c.have != c.want) {
                r.err = std::string(".meshdata: ") + c.what + " holds " + std::to_string(c.have) + " values, the counts need " +
                        std::to_string(c.want);
                ok = false;
                break;
            }
    }
    if (!ok) {
        set_err(err, err_len, r.err);
        delete md;
        return SNK_ERR_INVALID_ARG;
    }
    md->name.assign(name.begin(), name.end());
    md->submeshes.resize(sub_raw.size() / sizeof(snk_submesh));
    if (!sub_raw.empty()) std::memcpy(md->submeshes.data(), sub_raw.data(), sub_raw.size());
    *out = md;
    return SNK_OK;
}

int snk_meshdata_get_info(const snk_meshdata* md, snk_meshdata_info* info) {
    if (!md || !info) return SNK_ERR_INVALID_ARG;
    std::memset(info, 0, sizeof(*info));
    info->uuid = md->uuid;
    info->name = md->name.c_str();
    info->name_len = md->name.size();
    info->num_submeshes = (uint32_t)md->submeshes.size();
    info->num_vertices = md->num_vertices;
    info->num_indices = md->num_indices;
    info->num_materials = (uint32_t)md->materials.size();
    info->num_textures = (uint32_t)md->textures.size();
    info->submeshes = md->submeshes.data();
    info->positions = md->positions.data();
    info->normals = md->normals.data();
    info->tangents = md->tangents.data();
    info->tex_coords = md->tex_coords.data();
    info->indices = md->indices.data();
    info->materials = md->materials.data();
    info->textures = md->textures.data();
    return SNK_OK;
}

int snk_meshdata_submesh(const snk_meshdata* md, uint32_t index, snk_mesh* out) {
    if (!md || !out || index >= md->submeshes.size()) return SNK_ERR_INVALID_ARG;
    const snk_submesh& s = md->submeshes[index];
    if ((uint64_t)s.base_vertex + s.num_vertices > md->num_vertices ||
        (uint64_t)s.base_index + s.num_indices > md->num_indices || s.num_indices % 3 != 0)
        return SNK_ERR_INVALID_ARG;
    for (uint32_t k = 0; k < s.num_indices; k++)
        if (md->indices[(size_t)s.base_index + k] >= s.num_vertices) return SNK_ERR_INVALID_ARG;
    std::memset(out, 0, sizeof(*out));
    out->positions = md->positions.data() + 3ull * s.base_vertex;
    out->normals = md->normals.data() + 3ull * s.base_vertex;
    out->indices = md->indices.data() + s.base_index;
    out->num_vertices = s.num_vertices;
    out->num_triangles = s.num_indices / 3;
    return SNK_OK;
}

int snk_meshdata_free(snk_meshdata* md) {
    delete md;
    return SNK_OK;
}

}  // extern "C"
