// Checks candidate_mask (start_gb300/csrc/philox.h) against candidate_byte on
// Philox blocks of the collision streams and on blocks with planted zero
// bytes (every pattern of zero bytes, with random and 0x80 / 0x01 neighbours).
// Prints the number of mismatches (0 expected) and exits non-zero on any.
#include <cstdio>
#include <cstdint>
#include <random>

#include "philox.h"

namespace {

long long check(const spg::Philox4 &b) {
    const uint32_t m = spg::candidate_mask(b);
    long long bad = 0;
    for (uint32_t k = 0; k < 16; ++k) {
        const bool want = spg::candidate_byte(b, k) == 0u;
        if (bool((m >> k) & 1u) != want) ++bad;
    }
    if (m >> 16) ++bad;
    return bad;
}

}  // namespace

int main(int argc, char **argv) {
    const long long n = argc > 1 ? std::atoll(argv[1]) : 1000000;
    long long bad = 0, tested = 0;
    for (long long i = 0; i < n; ++i) {
        bad += check(spg::candidate_block(uint64_t(i) * 16u, uint32_t(i * 2654435761u), 0x9abcdef0u, 0x12345678u));
        ++tested;
    }
    std::mt19937_64 g(7);
    const uint32_t fills[] = {0x80u, 0x01u, 0xffu, 0x7fu};
    for (uint32_t pattern = 0; pattern < (1u << 16); ++pattern) {
        for (int rep = 0; rep < 8; ++rep) {
            spg::Philox4 b;
            for (int q = 0; q < 4; ++q) {
                uint32_t w = 0;
                for (int k = 0; k < 4; ++k) {
                    uint32_t byte = rep < 4 ? fills[rep] : uint32_t(g() % 255u) + 1u;
                    if ((pattern >> (4 * q + k)) & 1u) byte = 0u;
                    w |= byte << (8 * k);
                }
                b.v[q] = w;
            }
            bad += check(b);
            ++tested;
        }
    }
    std::printf("checked %lld blocks, mismatches %lld\n", tested, bad);
    return bad == 0 ? 0 : 1;
}
