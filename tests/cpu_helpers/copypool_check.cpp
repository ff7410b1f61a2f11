// Test harness: the library's parallel host copy (csrc/fv2d_hostcopy.h) on sizes around its chunk
// and alignment boundaries, unaligned source and destination, guard bytes untouched.
#include "fv2d_hostcopy.h"
#include <cstdio>
#include <random>
int main() {
    std::mt19937_64 rng(1);
    for (size_t bytes : {size_t(0), size_t(1), size_t(1) << 20, (size_t(1) << 20) + 7, size_t(33) << 20, (size_t(8) << 20) * 3 + 12345, size_t(100000003)}) {
        std::vector<unsigned char> a(bytes + 64), b(bytes + 64, 0xAB);
        for (auto& x : a) x = (unsigned char)rng();
        fv2d::CopyPool::get().copy(b.data() + 3, a.data() + 5, bytes);
        bool ok = std::memcmp(b.data() + 3, a.data() + 5, bytes) == 0 && b[0] == 0xAB && b[bytes + 3] == 0xAB;
        printf("%zu %s\n", bytes, ok ? "ok" : "BAD");
        if (!ok) return 1;
    }
    return 0;
}
