#include "xoshiro.hpp"

#include <mutex>

namespace ft {

static uint64_t splitmix(uint64_t& x)
{
    uint64_t z = (x += 0x9e3779b97f4a7c15ULL);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

xstate seed_state(uint64_t seed)
{
    xstate x;
    for (int i = 0; i < 4; i++) x.s[i] = splitmix(seed);
    return x;
}

uint64_t next(xstate& x)
{
    uint64_t* s = x.s;
    const uint64_t out = s[0] + s[3];
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = (s[3] << 45) | (s[3] >> 19);
    return out;
}

namespace {

void apply(const uint64_t* M, const uint64_t* v, uint64_t* out)
{
    uint64_t r0 = 0, r1 = 0, r2 = 0, r3 = 0;
    for (int w = 0; w < 4; w++) {
        uint64_t bits = v[w];
        while (bits) {
            int b = __builtin_ctzll(bits);
            bits &= bits - 1;
            const uint64_t* col = M + (size_t)(w * 64 + b) * 4;
            r0 ^= col[0];
            r1 ^= col[1];
            r2 ^= col[2];
            r3 ^= col[3];
        }
    }
    out[0] = r0;
    out[1] = r1;
    out[2] = r2;
    out[3] = r3;
}

std::vector<uint64_t> build_powers()
{
    std::vector<uint64_t> P((size_t)64 * 256 * 4);
    // T: one step applied to each basis state
    for (int c = 0; c < 256; c++) {
        xstate x{{0, 0, 0, 0}};
        x.s[c >> 6] = 1ULL << (c & 63);
        next(x);
        for (int w = 0; w < 4; w++) P[(size_t)c * 4 + w] = x.s[w];
    }
    // T^(2^(b+1)) = T^(2^b) T^(2^b)
    for (int b = 0; b < 63; b++) {
        const uint64_t* A = P.data() + (size_t)b * 1024;
        uint64_t* C = P.data() + (size_t)(b + 1) * 1024;
        for (int c = 0; c < 256; c++) apply(A, A + c * 4, C + c * 4);
    }
    return P;
}

}  // namespace

const std::vector<uint64_t>& power_table()
{
    static std::once_flag once;
    static std::vector<uint64_t> table;
    std::call_once(once, [] { table = build_powers(); });
    return table;
}

xstate advance(xstate x, uint64_t steps)
{
    const std::vector<uint64_t>& P = power_table();
    for (int b = 0; b < 64; b++)
        if ((steps >> b) & 1) {
            uint64_t out[4];
            apply(P.data() + (size_t)b * 1024, x.s, out);
            for (int w = 0; w < 4; w++) x.s[w] = out[w];
        }
    return x;
}

}  // namespace ft
