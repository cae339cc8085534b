// Host check of the kernels' invariant division (make_idx_div / idx_div in
// ttv_gb300/csrc/ttv_kernels.cuh, compiled here as host code): n / d for
// every divisor class the launches build (small, powers of two and their
// neighbours, random 32-bit ones) and dividends at the edges of the 32-bit
// range plus random ones, against the plain division.  Prints "PASSED <n>".
#include <cstdint>
#include <cstdio>
#include <vector>

#include "../../ttv_gb300/csrc/ttv_kernels.cuh"

using tlibg::IdxDiv;

static uint64_t rng_state = 0x9E3779B97F4A7C15ull;
static uint32_t next32()
{
    rng_state ^= rng_state << 13;
    rng_state ^= rng_state >> 7;
    rng_state ^= rng_state << 17;
    return (uint32_t)(rng_state >> 16);
}

int main()
{
    std::vector<uint64_t> ds;
    for (uint64_t d = 1; d < 1100; ++d) ds.push_back(d);
    for (int k = 1; k < 32; ++k)
        for (int e = -1; e <= 1; ++e) {
            const int64_t d = (int64_t(1) << k) + e;
            if (d >= 1 && d < (int64_t(1) << 32)) ds.push_back((uint64_t)d);
        }
    for (int i = 0; i < 500; ++i) ds.push_back(1 + next32() % 0xFFFFFFFFu);
    ds.push_back(0xFFFFFFFFull);
    uint64_t checked = 0;
    for (uint64_t d : ds) {
        const IdxDiv v = tlibg::make_idx_div(d, 0xFFFFFFFFull);
        if (!v.fast) {
            std::printf("FAILED: divisor %llu not on the fast path\n", (unsigned long long)d);
            return 1;
        }
        std::vector<uint64_t> ns = {0, 1, d - 1, d, d + 1, 2 * d - 1, 0x7FFFFFFFull, 0x80000000ull, 0xFFFFFFFFull};
        for (int i = 0; i < 60; ++i) ns.push_back(next32());
        for (uint64_t n : ns) {
            if (n > 0xFFFFFFFFull) continue;
            if (tlibg::idx_div(n, v) != n / d) {
                std::printf("FAILED: %llu / %llu\n", (unsigned long long)n, (unsigned long long)d);
                return 1;
            }
            ++checked;
        }
    }
    // a dividend range past 32 bits takes the plain division
    const IdxDiv wide = tlibg::make_idx_div(1000, uint64_t(1) << 40);
    if (wide.fast || tlibg::idx_div((uint64_t(1) << 40) - 1, wide) != ((uint64_t(1) << 40) - 1) / 1000) {
        std::printf("FAILED: wide dividends\n");
        return 1;
    }
    std::printf("PASSED %llu\n", (unsigned long long)checked);
    return 0;
}
