// Test infrastructure: stand-in for the reference's Core/headers/util/FileUtil.h,
// declaring only what Core/headers/util/ByteSerializer.h calls (WriteBinaryFile),
// so that the reference's serializer compiles here unchanged from its own header.
#pragma once
#include <cstddef>
#include <cstdio>
#include <string>

namespace SNAKE {
namespace files {
inline bool WriteBinaryFile(const std::string& filepath, void* data, size_t size) {
    std::FILE* f = std::fopen(filepath.c_str(), "wb");
    if (!f) return false;
    const bool ok = std::fwrite(data, 1, size, f) == size;
    return std::fclose(f) == 0 && ok;
}
}  // namespace files
}  // namespace SNAKE
