// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC'11), usable from host and
// device code. The collision streams are keyed by (particle id, seed) and
// counted by (step, draw), so a particle's draws do not depend on how
// particles are ordered, sorted or sharded, and a restored run repeats them.
#pragma once
#include <cstdint>

#if defined(__CUDACC__)
#define SPG_HD __host__ __device__ __forceinline__
#else
#define SPG_HD inline
#endif

namespace spg {

struct Philox4 {
    uint32_t v[4];
};

SPG_HD void philox_mulhilo(uint32_t a, uint32_t b, uint32_t &hi, uint32_t &lo) {
    const uint64_t p = uint64_t(a) * uint64_t(b);
    hi = uint32_t(p >> 32);
    lo = uint32_t(p);
}

SPG_HD Philox4 philox4x32_10(Philox4 c, uint32_t k0, uint32_t k1) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0, lo0, hi1, lo1;
        philox_mulhilo(M0, c.v[0], hi0, lo0);
        philox_mulhilo(M1, c.v[2], hi1, lo1);
        Philox4 o;
        o.v[0] = hi1 ^ c.v[1] ^ k0;
        o.v[1] = lo1;
        o.v[2] = hi0 ^ c.v[3] ^ k1;
        o.v[3] = lo0;
        c = o;
        k0 += W0;
        k1 += W1;
    }
    return c;
}

// 53-bit uniform double in [0, 1) from two 32-bit words.
SPG_HD double u01_from(uint32_t a, uint32_t b) {
    return (double(a >> 5) * 67108864.0 + double(b >> 6)) * (1.0 / 9007199254740992.0);
}

// Draw block `draw` of particle `id` at step `step`: four words.
SPG_HD Philox4 collision_draw(uint64_t step, uint32_t draw, uint32_t id, uint32_t seed_lo, uint32_t seed_hi) {
    Philox4 c;
    c.v[0] = uint32_t(step);
    c.v[1] = draw;
    c.v[2] = uint32_t(step >> 32);
    c.v[3] = seed_hi;
    return philox4x32_10(c, id, seed_lo);
}

// Collision test of step s of a particle whose collision probability is P
// (q = 1/256):
//  * the sixteen candidate bytes of steps 16m .. 16m + 15 are one block
//    (count m, draw 2); step s is a candidate when its byte (s & 15) is zero,
//    probability q;
//  * P <= q: a collision iff s is a candidate and u_acc < P / q = 256 P,
//    u_acc from block (s, draw 3), words 0-1;
//  * P > q: a collision iff s is a candidate or else u_f < (P - q) / (1 - q),
//    u_f from block (s, draw 4), words 0-1;
// so every step collides with probability exactly P, independently of the
// others, and one Philox block serves the tests of sixteen steps. The angle
// draws of a collision are block (s, draw 1): u1 from words 0-1, u2 from
// words 2-3.
constexpr double kCandQ = 1.0 / 256.0;

SPG_HD Philox4 candidate_block(uint64_t step, uint32_t id, uint32_t seed_lo, uint32_t seed_hi) {
    return collision_draw(step >> 4, 2u, id, seed_lo, seed_hi);
}

// The 53-bit uniform of words 0-1 of a block.
SPG_HD double u01_from_block(const Philox4 &r) { return u01_from(r.v[0], r.v[1]); }

SPG_HD uint32_t candidate_byte(const Philox4 &b, uint64_t step) {
    const uint32_t k = uint32_t(step & 15u);
    const uint32_t w = k < 8u ? (k < 4u ? b.v[0] : b.v[1]) : (k < 12u ? b.v[2] : b.v[3]);
    return (w >> (8u * (k & 3u))) & 0xffu;
}

// Bit k (0..15) set iff candidate_byte(b, 16 g + k) == 0: the candidate
// steps of the block's sixteen, so a step's test is one shift and one and.
SPG_HD uint32_t candidate_mask(const Philox4 &b) {
    uint32_t m = 0u;
    for (int q = 0; q < 4; ++q) {
        const uint32_t w = b.v[q];
        // 0x80 in each zero byte of w: (w & 0x7f) + 0x7f <= 0xfe, so no carry
        // crosses a byte, and the sum's top bit or w's is set iff the byte is not zero
        const uint32_t z = ~(((w & 0x7f7f7f7fu) + 0x7f7f7f7fu) | w) & 0x80808080u;
        // the byte flags at bits 0, 8, 16, 24 times 2^24 + 2^17 + 2^10 + 2^3:
        // flag i lands on bit 24 + i, every other partial product on a distinct
        // bit below 24 (no carry) or beyond 31
        m |= ((((z >> 7) * 0x01020408u) >> 24) & 0xfu) << (4 * q);
    }
    return m;
}

}  // namespace spg
