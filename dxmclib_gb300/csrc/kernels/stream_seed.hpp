// Seeding of the per-history random streams and the invariant-divisor division
// the kernels use, usable from host and device code.
//
// Every history draws from its own xoshiro128+ generator (Blackman and Vigna,
// "Scrambled linear pseudorandom number generators", 2021).  Its 128-bit state
// is the next two outputs of SplitMix64 (Steele, Lea and Flood, "Fast
// splittable pseudorandom number generators", OOPSLA 2014), the seeding Vigna
// recommends for the xoshiro family, from a starting counter of the mixed job
// seed XOR the history id.  The counters SplitMix64 visits for two histories
// (start + 1 and 2 Weyl increments) never coincide: starting counters of
// histories below 2^62 differ by less than 2^62, a Weyl increment is larger.
// A history's stream depends on (seed, history) only, so a job can be split,
// batched or resumed at any history id.
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define DXMC_HD __host__ __device__
#else
#define DXMC_HD
#endif

namespace dxmc_gb300 {

constexpr std::uint64_t SPLITMIX_GAMMA = 0x9e3779b97f4a7c15ull; // 2^64 / golden ratio, odd

// One SplitMix64 step: advances x by the Weyl increment and returns the mixed value.
DXMC_HD inline std::uint64_t splitmix64(std::uint64_t& x)
{
    std::uint64_t z = (x += SPLITMIX_GAMMA);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

// The xoshiro128+ state of history `history` of a job seeded with `seed`; the
// all-zero state is excluded by setting the lowest bit of the last word.
DXMC_HD inline void stream_seed(std::uint64_t seed, std::uint64_t history, std::uint32_t out[4])
{
    std::uint64_t k = seed;
    std::uint64_t x = splitmix64(k) ^ history;
    const std::uint64_t a = splitmix64(x);
    const std::uint64_t b = splitmix64(x);
    out[0] = static_cast<std::uint32_t>(a);
    out[1] = static_cast<std::uint32_t>(a >> 32);
    out[2] = static_cast<std::uint32_t>(b);
    out[3] = static_cast<std::uint32_t>(b >> 32) | 1u;
}

DXMC_HD inline std::uint32_t mulhi32(std::uint32_t a, std::uint32_t b)
{
#if defined(__CUDA_ARCH__)
    return __umulhi(a, b);
#else
    return static_cast<std::uint32_t>((static_cast<std::uint64_t>(a) * b) >> 32);
#endif
}

// Unsigned 32-bit division by a divisor fixed for a whole job, as a multiply-high
// and two shifts (Granlund and Montgomery, "Division by invariant integers using
// multiplication", PLDI 1994; the round-up variant for every divisor):
// n / d = (t + ((n - t) >> s1)) >> s2 with t = mulhi(m, n), for all n < 2^32.
// The kernels use it to find a history's exposure.
struct UDivMagic {
    std::uint32_t m;
    std::uint32_t shifts; // s1 | s2 << 8
};

inline UDivMagic udiv_magic(std::uint32_t d)
{
    if (d <= 1)
        return UDivMagic { 0u, 0u }; // n / 1 = n
    int l = 0;
    while ((std::uint64_t { 1 } << l) < d)
        ++l; // l = ceil(log2 d)
    const std::uint64_t m = ((std::uint64_t { 1 } << 32) * ((std::uint64_t { 1 } << l) - d)) / d + 1;
    return UDivMagic { static_cast<std::uint32_t>(m), 1u | (static_cast<std::uint32_t>(l - 1) << 8) };
}

DXMC_HD inline std::uint32_t udiv_apply(std::uint32_t n, std::uint32_t m, std::uint32_t shifts)
{
    const std::uint32_t t = mulhi32(m, n);
    return (t + ((n - t) >> (shifts & 0xffu))) >> (shifts >> 8);
}

} // namespace dxmc_gb300
