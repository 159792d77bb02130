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

__device__ __forceinline__ float exp10_fast(float y) { return exp2f(y * 3.32192809488736f); }

// Arithmetic in the precision a kernel computes in: float (single-precision
// intrinsics; the transport's translation unit is built with fast math) or
// double (the FP64-everywhere precision mode, accurate double functions).
// One source serves both through these overloads.
__device__ __forceinline__ float m_log(float x) { return __logf(x); }
__device__ __forceinline__ double m_log(double x) { return log(x); }
__device__ __forceinline__ float m_log2(float x) { return __log2f(x); }
__device__ __forceinline__ double m_log2(double x) { return log2(x); }
__device__ __forceinline__ float m_log10(float x) { return __log10f(x); }
__device__ __forceinline__ double m_log10(double x) { return log10(x); }
__device__ __forceinline__ float m_exp10(float y) { return exp10_fast(y); }
__device__ __forceinline__ double m_exp10(double y) { return exp10(y); }
__device__ __forceinline__ float m_exp(float y) { return expf(y); }
__device__ __forceinline__ double m_exp(double y) { return exp(y); }
__device__ __forceinline__ void m_sincos(float a, float* s, float* c) { sincosf(a, s, c); }
__device__ __forceinline__ void m_sincos(double a, double* s, double* c) { sincos(a, s, c); }
__device__ __forceinline__ float m_cos(float a) { return cosf(a); }
__device__ __forceinline__ double m_cos(double a) { return cos(a); }
__device__ __forceinline__ float m_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double m_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float m_rsqrt(float x) { return rsqrtf(x); }
__device__ __forceinline__ double m_rsqrt(double x) { return rsqrt(x); }
__device__ __forceinline__ float m_fma(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double m_fma(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float m_min(float a, float b) { return fminf(a, b); }
__device__ __forceinline__ double m_min(double a, double b) { return fmin(a, b); }
__device__ __forceinline__ float m_max(float a, float b) { return fmaxf(a, b); }
__device__ __forceinline__ double m_max(double a, double b) { return fmax(a, b); }
__device__ __forceinline__ float m_abs(float a) { return fabsf(a); }
__device__ __forceinline__ double m_abs(double a) { return fabs(a); }
__device__ __forceinline__ float m_floor(float a) { return floorf(a); }
__device__ __forceinline__ double m_floor(double a) { return floor(a); }
__device__ __forceinline__ int m_floor_int(float a) { return __float2int_rd(a); }
__device__ __forceinline__ int m_floor_int(double a) { return __double2int_rd(a); }

// Rows of the sampling tables around energy E: row i and i + 1 with weight f of
// the upper one.  Draws interpolate the two rows' quantiles at the same level
// (quantile interpolation), which follows distributions that stretch with
// energy far more closely than a mixture of the rows would.
template <class Real>
__device__ __forceinline__ int table_row(const LutMeta& m, Real E, Real& f)
{
    const Real t = (m_log(E) - m.tab_le0) * m.tab_inv_dle;
    int i = static_cast<int>(m_floor(t));
    f = t - static_cast<Real>(i);
    if (i < 0) {
        i = 0;
        f = Real(0);
    } else if (i > m.tab_ne - 2) {
        i = m.tab_ne - 2;
        f = Real(1);
    }
    return i;
}

// Quantile at level u of the energy rows `row` and `row + 1` (stride nu + 1),
// linear between the stored levels k / nu and between the two rows (weight fe).
template <class Real>
__device__ __forceinline__ Real table_quantile(const float* row, int nu, Real u, Real fe)
{
    const Real pos = u * static_cast<Real>(nu);
    const int j = min(static_cast<int>(pos), nu - 1);
    const Real f = pos - static_cast<Real>(j);
    const Real a0 = __ldg(row + j), b0 = __ldg(row + j + 1);
    const Real a1 = __ldg(row + nu + 1 + j), b1 = __ldg(row + nu + 1 + j + 1);
    const Real q0 = m_fma(f, b0 - a0, a0);
    const Real q1 = m_fma(f, b1 - a1, a1);
    return m_fma(fe, q1 - q0, q0);
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
// the same constants in double, for kernels that compute in double (a float
// kernel rounds them to the float values above)
constexpr double PI_D = 3.14159265358979323846;
constexpr double KEV_TO_ANGSTROM_D = 12.398520;
constexpr double ELECTRON_REST_MASS_D = 510.9989461;
constexpr double ENERGY_CUTOFF_D = 1.0;
constexpr double ROULETTE_THRESHOLD_D = 5.0;
constexpr double ROULETTE_PROBABILITY_D = 0.8;
constexpr double N_ERROR_D = 1.0e-9;

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

// azimuth uniform in [-pi, pi) in the kernel's precision, from the same 23-bit draw
template <class Real>
__device__ __forceinline__ Real rng_azimuth(Rng& r)
{
    return m_fma(static_cast<Real>(r.uniform()), Real(2.0 * PI_D), Real(-PI_D));
}

// ---------------------------------------------------------------------------
// Math helpers
// ---------------------------------------------------------------------------

// vectormath::rotate (vectormath.hpp:83-99): Rodrigues rotation about a (not
// necessarily unit) axis.
template <class Real>
__device__ __forceinline__ void rotate(Real& vx, Real& vy, Real& vz, Real ax, Real ay, Real az, Real angle)
{
    Real s, c;
    m_sincos(angle, &s, &c);
    const Real midt = (Real(1) - c) * (vx * ax + vy * ay + vz * az);
    const Real ox = c * vx + midt * ax + s * (ay * vz - az * vy);
    const Real oy = c * vy + midt * ay + s * (-ax * vz + az * vx);
    const Real oz = c * vz + midt * az + s * (ax * vy - ay * vx);
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
template <class Real>
__device__ __forceinline__ void peturb(Real& vx, Real& vy, Real& vz, Real cos_theta, Real phi, bool normalize = false)
{
    const Real ax = m_abs(vx), ay = m_abs(vy), az = m_abs(vz);
    const int k = ax <= ay ? (ax <= az ? 0 : 2) : (ay <= az ? 1 : 2);
    // cross(vec, e_k)
    Real ux, uy, uz;
    if (k == 0) {
        ux = Real(0);
        uy = vz;
        uz = -vy;
    } else if (k == 1) {
        ux = -vz;
        uy = Real(0);
        uz = vx;
    } else {
        ux = vy;
        uy = -vx;
        uz = Real(0);
    }
    if (normalize) {
        const Real inv = m_rsqrt(ux * ux + uy * uy + uz * uz);
        ux *= inv;
        uy *= inv;
        uz *= inv;
    }
    rotate(ux, uy, uz, vx, vy, vz, phi);
    const Real st = m_sqrt(m_max(Real(0), Real(1) - cos_theta * cos_theta));
    vx = vx * cos_theta + ux * st;
    vy = vy * cos_theta + uy * st;
    vz = vz * cos_theta + uz * st;
}

// ---------------------------------------------------------------------------
// LUT lookups (attenuationinterpolator.hpp:207-248, attenuationlut.hpp:124-204,
// interpolation.hpp:169-176, dxmcrandom.hpp:483-500)
// ---------------------------------------------------------------------------
template <class Real>
__device__ __forceinline__ int upper_bound_f(const float* x, int n, Real v)
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

template <class Real>
__device__ __forceinline__ int lut_segment(const float* L, const LutMeta& m, Real logE)
{
    if (logE > m.linear_energy) {
        const int idx = static_cast<int>((logE - m.linear_energy) * m.inv_linear_step) + m.linear_index;
        return min(idx, m.R - 1);
    }
    const int pos = upper_bound_f(L + m.off_x, m.R, logE);
    return pos < m.R ? pos : m.R - 1;
}

template <class Real>
__device__ __forceinline__ void lut_attenuation(const float* L, const LutMeta& m, int material, Real logE, int seg, Real& photo, Real& compt, Real& rayl)
{
    const float2* c = reinterpret_cast<const float2*>(L + m.off_coef + (material * m.R + seg) * 6);
    const float2 p = c[0], q = c[1], r = c[2];
    photo = m_exp10(m_fma(Real(p.y), logE, Real(p.x)));
    compt = m_exp10(m_fma(Real(q.y), logE, Real(q.x)));
    rayl = m_exp10(m_fma(Real(r.y), logE, Real(r.x)));
}

template <class Real>
__device__ __forceinline__ Real lut_max_inverse(const float* L, const LutMeta& m, Real logE, int seg)
{
    const float2 c = reinterpret_cast<const float2*>(L + m.off_maxcoef)[seg];
    return m_exp10(m_fma(Real(c.y), logE, Real(c.x)));
}

} // namespace dxmc_gb300::dev
