// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC'11), usable from host and
// device code.  Ten rounds of the 4x32 Philox S-box with the published
// multipliers and Weyl key increments.
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define DXMC_HD __host__ __device__
#else
#define DXMC_HD
#endif

namespace dxmc_gb300 {

DXMC_HD inline std::uint32_t mulhi32(std::uint32_t a, std::uint32_t b)
{
#if defined(__CUDA_ARCH__)
    return __umulhi(a, b);
#else
    return static_cast<std::uint32_t>((static_cast<std::uint64_t>(a) * b) >> 32);
#endif
}

DXMC_HD inline void philox4x32_10(std::uint32_t& c0, std::uint32_t& c1, std::uint32_t& c2, std::uint32_t& c3, std::uint32_t k0, std::uint32_t k1)
{
    constexpr std::uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    constexpr std::uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#if defined(__CUDACC__)
#pragma unroll
#endif
    for (int r = 0; r < 10; ++r) {
        const std::uint32_t hi0 = mulhi32(M0, c0), lo0 = M0 * c0;
        const std::uint32_t hi1 = mulhi32(M1, c2), lo1 = M1 * c2;
        const std::uint32_t n0 = hi1 ^ c1 ^ k0;
        const std::uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
        k0 += W0;
        k1 += W1;
    }
}

// Unsigned 32-bit division by a divisor fixed for a whole job, as a multiply-high
// and two shifts (Granlund and Montgomery, "Division by invariant integers using
// multiplication", PLDI 1994; the round-up variant for every divisor):
// n / d = (t + ((n - t) >> s1)) >> s2 with t = mulhi(m, n), for all n < 2^32.
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
