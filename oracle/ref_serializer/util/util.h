// Test infrastructure: stand-in for the reference's Core/headers/util/util.h with
// what Core/headers/util/ByteSerializer.h uses (SNK_ASSERT; the reference logs and
// exits, this one prints and exits) and the standard headers it relies on.
#pragma once
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#define SNK_ASSERT(x)                                         \
    if (!(x)) {                                               \
        std::fprintf(stderr, "assertion failed: %s\n", #x);   \
        std::exit(1);                                         \
    }
