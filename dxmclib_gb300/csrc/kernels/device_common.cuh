// Device-side data layouts, counter-based RNG and table lookups shared by the
// transport kernel, the probe kernels and the post-processing kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "stream_seed.hpp"

namespace dxmc_gb300::dev {

// ---------------------------------------------------------------------------
// Layouts in HBM
// ---------------------------------------------------------------------------

// One voxel: density, material index and forced-interaction flag packed into
// one 8-byte word so a Woodcock step needs a single 32-byte-sector gather.
struct alignas(8) Voxel {
    float density;
    std::uint8_t material;
    std::uint8_t measurement;
    std::uint16_t pad;
};
static_assert(sizeof(Voxel) == 8, "voxel must pack into 8 bytes");

// One exposure after Exposure::alignToDirectionCosines (exposure.hpp:268-278).
struct alignas(16) DevExposure {
    float pos[3];
    float weight;
    float cosx[3];
    float mono_energy;
    float cosy[3];
    float pad0;
    float beam[3];
    float pad1;
    float coll[4]; // x0, x1, y0, y1
};
static_assert(sizeof(DevExposure) == 80, "exposure record is 80 bytes");

// Float LUT image: one contiguous buffer so a block can stage it into shared
// memory with a single cooperative copy.  Offsets are in floats.
struct LutMeta {
    int n_materials;
    int R;           // energy nodes / segments
    int linear_index;
    int total_floats;
    float linear_step;
    float inv_linear_step;
    float linear_energy;
    float max_energy;
    int off_x;       // R log10 energies
    int off_coef;    // n_materials * R * 6
    int off_maxcoef; // R * 2
    int off_rita;    // n_materials * 4 * 56 (x, e, a, b)
    int off_spline;  // n_materials * 64 (60 coefficients, start, step, stop, pad)
    int off_shells;  // n_materials * 12 * SHELL_FLOATS
    // inverse-CDF sampling tables, after total_floats (read from global memory,
    // not staged in shared memory): rows of tab_nu + 1 quantiles
    int off_ckn;     // Compton energy fraction, no scatter factor: tab_ne rows
    int off_csf;     // Compton with scatter factor: n_materials * tab_ne rows
    int off_ray;     // Rayleigh q^2 / q_max^2: n_materials * tab_ne rows
    int tab_ne, tab_nu;
    float tab_le0;     // ln of the first table energy
    float tab_inv_dle; // 1 / ln step
    int pad0;
};

// Rows of the sampling tables around energy E: row i and i + 1 with weight f of
// the upper one.  Draws interpolate the two rows' quantiles at the same level
// (quantile interpolation), which follows distributions that stretch with
// energy far more closely than a mixture of the rows would.
__device__ __forceinline__ int table_row(const LutMeta& m, float E, float& f)
{
    const float t = (__logf(E) - m.tab_le0) * m.tab_inv_dle;
    int i = static_cast<int>(floorf(t));
    f = t - static_cast<float>(i);
    if (i < 0) {
        i = 0;
        f = 0.0f;
    } else if (i > m.tab_ne - 2) {
        i = m.tab_ne - 2;
        f = 1.0f;
    }
    return i;
}

// Quantile at level u of the energy rows `row` and `row + 1` (stride nu + 1),
// linear between the stored levels k / nu and between the two rows (weight fe).
__device__ __forceinline__ float table_quantile(const float* row, int nu, float u, float fe)
{
    const float pos = u * static_cast<float>(nu);
    const int j = min(static_cast<int>(pos), nu - 1);
    const float f = pos - static_cast<float>(j);
    const float a0 = __ldg(row + j), b0 = __ldg(row + j + 1);
    const float a1 = __ldg(row + nu + 1 + j), b1 = __ldg(row + nu + 1 + j + 1);
    const float q0 = fmaf(f, b0 - a0, a0);
    const float q1 = fmaf(f, b1 - a1, a1);
    return fmaf(fe, q1 - q0, q0);
}

constexpr int RITA_N = 56;
constexpr int SPLINE_N = 16;
constexpr int SPLINE_FLOATS = 64;
constexpr int SHELL_FLOATS = 12; // binding, nElectrons, J0, photoProb, yield, lineP[3], lineE[3], pad
constexpr int N_SHELLS = 12;

constexpr float KEV_TO_ANGSTROM = 12.398520f;
constexpr float ELECTRON_REST_MASS = 510.9989461f;
constexpr float PI_F = 3.14159265358979f;
constexpr float ENERGY_CUTOFF = 1.0f;           // transport.hpp:827-830
constexpr float ROULETTE_THRESHOLD = 5.0f;      // transport.hpp:823-826
constexpr float ROULETTE_PROBABILITY = 0.8f;    // transport.hpp:819-822
constexpr float N_ERROR = 1.0e-9f;              // transport.hpp:831-834
constexpr int REJECTION_CAP = 4096;             // iteration cap on every sampling loop

// Per-history random stream: xoshiro128+ (Blackman and Vigna, "Scrambled
// linear pseudorandom number generators", 2021), a 32-bit-native generator,
// with its 128-bit state from SplitMix64 of (job seed, history id)
// (stream_seed.hpp).  Every history has its own stream, so a job can be split
// or resumed at any history id and results do not depend on scheduling.
struct Rng {
    uint32_t s0, s1, s2, s3;

    __device__ void init(uint64_t seed, uint64_t history)
    {
        uint32_t st[4];
        stream_seed(seed, history, st);
        s0 = st[0];
        s1 = st[1];
        s2 = st[2];
        s3 = st[3];
    }
    // the sum output of xoshiro128+: its lowest bits are weak, and every use
    // takes the high bits (23-bit float mantissas, multiply-high integers)
    __device__ __forceinline__ uint32_t next()
    {
        const uint32_t result = s0 + s3;
        const uint32_t t = s1 << 9;
        s2 ^= s0;
        s3 ^= s1;
        s1 ^= s2;
        s0 ^= s3;
        s2 ^= t;
        s3 = __funnelshift_l(s3, s3, 11);
        return result;
    }
    // [0, 1) with 23 random bits: the top bits as the mantissa of a float in [1, 2),
    // minus one (no integer-to-float conversion)
    __device__ __forceinline__ float uniform() { return __uint_as_float(0x3f800000u | (next() >> 9)) - 1.0f; }
    // (0, 1] for logarithms: two minus a float in [1, 2)
    __device__ __forceinline__ float uniform_open() { return 2.0f - __uint_as_float(0x3f800000u | (next() >> 9)); }
    // integer in [0, n) by the multiply-high method (Lemire)
    __device__ __forceinline__ uint32_t below(uint32_t n) { return __umulhi(next(), n); }
    // azimuth uniform in [-pi, pi)
    __device__ __forceinline__ float azimuth() { return fmaf(uniform(), 6.28318530717959f, -3.14159265358979f); }
};

// ---------------------------------------------------------------------------
// Math helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ float exp10_fast(float y) { return exp2f(y * 3.32192809488736f); }

// vectormath::rotate (vectormath.hpp:83-99): Rodrigues rotation about a (not
// necessarily unit) axis.
__device__ __forceinline__ void rotate(float& vx, float& vy, float& vz, float ax, float ay, float az, float angle)
{
    float s, c;
    sincosf(angle, &s, &c);
    const float midt = (1.0f - c) * (vx * ax + vy * ay + vz * az);
    const float ox = c * vx + midt * ax + s * (ay * vz - az * vy);
    const float oy = c * vy + midt * ay + s * (-ax * vz + az * vx);
    const float oz = c * vz + midt * az + s * (ax * vy - ay * vx);
    vx = ox;
    vy = oy;
    vz = oz;
}

// vectormath::peturb (vectormath.hpp:197-221), including its quirk: the
// orthogonal axis cross(vec, e_k) is never normalised, so |dir| shrinks after
// every direction change exactly as in the reference (and the angle between the
// old and new direction is not theta).  normalize = true scales the axis to unit
// length first: a unit direction then turns by exactly theta and stays a unit
// vector (the normalised physics mode; it does not match the reference).  Takes
// cos(theta).
__device__ __forceinline__ void peturb(float& vx, float& vy, float& vz, float cos_theta, float phi, bool normalize = false)
{
    const float ax = fabsf(vx), ay = fabsf(vy), az = fabsf(vz);
    const int k = ax <= ay ? (ax <= az ? 0 : 2) : (ay <= az ? 1 : 2);
    // cross(vec, e_k)
    float ux, uy, uz;
    if (k == 0) {
        ux = 0.0f;
        uy = vz;
        uz = -vy;
    } else if (k == 1) {
        ux = -vz;
        uy = 0.0f;
        uz = vx;
    } else {
        ux = vy;
        uy = -vx;
        uz = 0.0f;
    }
    if (normalize) {
        const float inv = rsqrtf(ux * ux + uy * uy + uz * uz);
        ux *= inv;
        uy *= inv;
        uz *= inv;
    }
    rotate(ux, uy, uz, vx, vy, vz, phi);
    const float st = sqrtf(fmaxf(0.0f, 1.0f - cos_theta * cos_theta));
    vx = vx * cos_theta + ux * st;
    vy = vy * cos_theta + uy * st;
    vz = vz * cos_theta + uz * st;
}

// ---------------------------------------------------------------------------
// LUT lookups (attenuationinterpolator.hpp:207-248, attenuationlut.hpp:124-204,
// interpolation.hpp:169-176, dxmcrandom.hpp:483-500)
// ---------------------------------------------------------------------------
__device__ __forceinline__ int upper_bound_f(const float* x, int n, float v)
{
    int lo = 0, count = n;
    while (count > 0) {
        const int step = count >> 1;
        if (!(v < x[lo + step])) {
            lo += step + 1;
            count -= step + 1;
        } else {
            count = step;
        }
    }
    return lo;
}

__device__ __forceinline__ int lut_segment(const float* L, const LutMeta& m, float logE)
{
    if (logE > m.linear_energy) {
        const int idx = static_cast<int>((logE - m.linear_energy) * m.inv_linear_step) + m.linear_index;
        return min(idx, m.R - 1);
    }
    const int pos = upper_bound_f(L + m.off_x, m.R, logE);
    return pos < m.R ? pos : m.R - 1;
}

__device__ __forceinline__ void lut_attenuation(const float* L, const LutMeta& m, int material, float logE, int seg, float& photo, float& compt, float& rayl)
{
    const float2* c = reinterpret_cast<const float2*>(L + m.off_coef + (material * m.R + seg) * 6);
    const float2 p = c[0], q = c[1], r = c[2];
    photo = exp10_fast(fmaf(p.y, logE, p.x));
    compt = exp10_fast(fmaf(q.y, logE, q.x));
    rayl = exp10_fast(fmaf(r.y, logE, r.x));
}

__device__ __forceinline__ float lut_max_inverse(const float* L, const LutMeta& m, float logE, int seg)
{
    const float2 c = reinterpret_cast<const float2*>(L + m.off_maxcoef)[seg];
    return exp10_fast(fmaf(c.y, logE, c.x));
}

} // namespace dxmc_gb300::dev
