// ORACLE TEST INFRASTRUCTURE — CPU restatement of DXMClib's photon transport.
//
// Used only as the checker (tests/, __graft_entry__.smoke) and as the timed
// CPU baseline of bench.py.  It is validated against the reference itself
// through the golden fixtures (tests/test_oracle_port.py) and it travels to
// machines where the reference checkout does not exist.
//
// It follows DXMClib function by function in double precision with the
// reference's PCG32 generator; every function cites the reference lines it
// restates.  It consumes the same host LUT tables as the reference
// (attenuation coefficients, majorant, RITA, spline, shells) in double.
#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <numeric>
#include <thread>
#include <vector>

namespace {

constexpr double PI = 3.14159265358979323846;
constexpr double KEV_TO_ANGSTROM = 12.398520;       // constants.hpp:26-30
constexpr double ELECTRON_REST_MASS = 510.9989461;  // constants.hpp:58-62
constexpr double ENERGY_CUTOFF = 1.0;               // transport.hpp:827-830
constexpr double RR_THRESHOLD = 5.0;                // transport.hpp:823-826
constexpr double RR_PROB = 0.8;                     // transport.hpp:819-822
constexpr double N_ERROR = 1.0e-9;                  // transport.hpp:831-834

// PCG32 XSH-RR (dxmcrandom.hpp:156-165) with uniform = u32 * 2^-32 (:66-73)
struct Pcg32 {
    std::uint64_t s0, s1;
    std::uint32_t next()
    {
        const std::uint64_t old = s0;
        s0 = old * 6364136223846793005ULL + (s1 | 1);
        const std::uint32_t xs = static_cast<std::uint32_t>(((old >> 18u) ^ old) >> 27u);
        const std::uint32_t rot = static_cast<std::uint32_t>(old >> 59u);
        return (xs >> rot) | (xs << ((-rot) & 31));
    }
    double uniform() { return next() * 2.32830643653869628906e-010; }
    // bounded integer by rejection (dxmcrandom.hpp:82-90)
    std::uint32_t below(std::uint32_t max)
    {
        const std::uint32_t threshold = static_cast<std::uint32_t>(-max) % max;
        for (;;) {
            const std::uint32_t r = next();
            if (r >= threshold)
                return r % max;
        }
    }
};

struct Particle {
    double pos[3];
    double dir[3];
    double energy;
    double weight;
};

struct Lut {
    int nm = 0, R = 0;
    std::size_t linear_index = 0;
    double linear_step = 0, linear_energy = 0;
    const double* x = nullptr;
    const double* coef = nullptr;
    const double* maxcoef = nullptr;
    const double* rita = nullptr;   // nm * 4 * 56
    const double* spline = nullptr; // nm * 79
    const double* shells = nullptr; // nm * 12 * 13
};

// vectormath::rotate (vectormath.hpp:83-99)
void rotate(double v[3], const double a[3], double angle)
{
    const double s = std::sin(angle), c = std::cos(angle);
    const double midt = (1 - c) * (v[0] * a[0] + v[1] * a[1] + v[2] * a[2]);
    double o[3];
    o[0] = c * v[0] + midt * a[0] + s * (a[1] * v[2] - a[2] * v[1]);
    o[1] = c * v[1] + midt * a[1] + s * (-a[0] * v[2] + a[2] * v[0]);
    o[2] = c * v[2] + midt * a[2] + s * (a[0] * v[1] - a[1] * v[0]);
    v[0] = o[0];
    v[1] = o[1];
    v[2] = o[2];
}

// Normalised physics mode (no reference counterpart): the orthogonal axis of
// peturb is scaled to unit length, so directions stay unit vectors.  Set for a
// whole run through oracle_port_set_direction.
bool g_normalize_direction = false;

// vectormath::peturb (vectormath.hpp:197-221), orthogonal axis left unnormalised
// (or normalised in the normalised physics mode)
void peturb(double v[3], double theta, double phi)
{
    const double ax = std::abs(v[0]), ay = std::abs(v[1]), az = std::abs(v[2]);
    const int k = ax <= ay ? (ax <= az ? 0 : 2) : (ay <= az ? 1 : 2);
    double e[3] = { 0, 0, 0 };
    e[k] = 1;
    double u[3] = { v[1] * e[2] - v[2] * e[1], v[2] * e[0] - v[0] * e[2], v[0] * e[1] - v[1] * e[0] };
    if (g_normalize_direction) {
        const double inv = 1.0 / std::sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
        for (double& c : u)
            c *= inv;
    }
    rotate(u, v, phi);
    const double ts = std::sin(theta), tc = std::cos(theta);
    for (int i = 0; i < 3; ++i)
        v[i] = v[i] * tc + u[i] * ts;
}

// AttenuationLutInterpolator::operator() (attenuationinterpolator.hpp:207-229)
std::size_t segment(const Lut& L, double logE, bool clamp)
{
    if (logE > L.linear_energy) {
        std::size_t idx = static_cast<std::size_t>((logE - L.linear_energy) / L.linear_step) + L.linear_index;
        if (clamp || idx > static_cast<std::size_t>(L.R - 1))
            idx = std::min(idx, static_cast<std::size_t>(L.R - 1));
        return idx;
    }
    const double* p = std::upper_bound(L.x, L.x + L.R, logE);
    return p != L.x + L.R ? static_cast<std::size_t>(p - L.x) : static_cast<std::size_t>(L.R - 1);
}

std::array<double, 3> attenuation(const Lut& L, int mat, double E)
{
    const double logE = std::log10(E);
    const std::size_t off = static_cast<std::size_t>(mat) * L.R * 6 + segment(L, logE, true) * 6;
    return { std::pow(10.0, L.coef[off] + L.coef[off + 1] * logE), std::pow(10.0, L.coef[off + 2] + L.coef[off + 3] * logE),
        std::pow(10.0, L.coef[off + 4] + L.coef[off + 5] * logE) };
}

// maxAttenuationInverse (attenuationinterpolator.hpp:231-248)
double max_inverse(const Lut& L, double E)
{
    const double logE = std::log10(E);
    const std::size_t i = segment(L, logE, false);
    return std::pow(10.0, L.maxcoef[2 * i] + L.maxcoef[2 * i + 1] * logE);
}

// CubicSplineInterpolator::operator() (interpolation.hpp:169-176)
double scatter_factor(const Lut& L, int mat, double q)
{
    const double* s = L.spline + mat * 79;
    const double start = s[76], step = s[77], stop = s[78];
    const double x = std::clamp(q, start, stop);
    const std::size_t index = x > start ? static_cast<std::size_t>((x - start) / step) : 0;
    const std::size_t off = index < 15 ? index * 4 : 14 * 4;
    return s[off] + s[off + 1] * x + s[off + 2] * x * x + s[off + 3] * x * x * x;
}

// RITA::operator()(state, maxValue) (dxmcrandom.hpp:483-500)
double rita(const Lut& L, int mat, double maxValue, Pcg32& rng)
{
    const double* x = L.rita + mat * 4 * 56;
    const double* e = x + 56;
    const double* a = e + 56;
    const double* b = a + 56;
    const double* ub = std::upper_bound(x, x + 56, maxValue);
    const double modifier = ub != x + 56 ? e[ub - x] : 1.0;
    double res;
    do {
        const double r1 = rng.uniform() * modifier;
        const std::size_t i = static_cast<std::size_t>(std::upper_bound(e, e + 56, r1) - e) - 1;
        const double v = r1 - e[i];
        const double d = e[i + 1] - e[i];
        res = x[i] + (1 + a[i] + b[i]) * d * v / (d * d + a[i] * d * v + b[i] * v * v) * (x[i + 1] - x[i]);
    } while (res > maxValue);
    return res;
}

struct Shell {
    const double* p;
    double binding() const { return p[0]; }
    double electrons() const { return p[1]; }
    double j0() const { return p[2]; }
    double photoProb() const { return p[3]; }
    double yield() const { return p[4]; }
    double lineProb(int k) const { return p[5 + k]; }
    double lineEnergy(int k) const { return p[8 + k]; }
};

struct Job {
    Lut lut;
    const double* density;
    const std::uint8_t* material;
    const std::uint8_t* measurement;
    std::uint64_t dims[3];
    double lo[3], hi[3], spacing[3];
    int model;
    // exposures: n x 19 (pos, cos, beam, coll, weight, nhist, mono)
    const double* exposures;
    std::uint64_t n_exposures;
    // spectrum
    int spec_n;
    const double* spec_e;
    std::vector<double> spec_p;
    std::vector<std::uint64_t> spec_a;
    // heel
    const double* heel_w;
    double heel_e0, heel_es, heel_a0, heel_as;
    int heel_ne, heel_na;
    // bow-tie
    std::vector<std::pair<double, double>> bowtie;
    // output
    double* dose;
    double* var;
    std::uint32_t* nev;
    std::atomic<std::uint64_t> next_exposure { 0 };

    Shell shell(int mat, int s) const { return Shell { lut.shells + (mat * 12 + s) * 13 }; }

    void score(std::size_t idx, double e)
    {
        std::atomic_ref<double>(dose[idx]).fetch_add(e);
        std::atomic_ref<std::uint32_t>(nev[idx]).fetch_add(1u);
        std::atomic_ref<double>(var[idx]).fetch_add(e * e);
    }

    // photoAbsorption (transport.hpp:216-263)
    double photo(Particle& p, int mat, Pcg32& rng)
    {
        const double E = p.energy;
        p.energy = 0;
        if (model < 2)
            return E;
        std::array<double, 12> probs;
        for (int s = 0; s < 12; ++s)
            probs[s] = E > shell(mat, s).binding() ? shell(mat, s).photoProb() : 0;
        std::partial_sum(probs.begin(), probs.end(), probs.begin());
        std::size_t idx = 0;
        const double sample = probs.back() * rng.uniform();
        while (probs[idx] < sample && idx < 11)
            ++idx;
        const Shell sh = shell(mat, static_cast<int>(idx));
        if (sh.binding() > E || sh.binding() < ENERGY_CUTOFF)
            return E;
        if (rng.uniform() <= sh.yield()) {
            int line = 0;
            double r3 = rng.uniform() - sh.lineProb(0);
            while (r3 > 0 && line < 2) {
                ++line;
                r3 -= sh.lineProb(line);
            }
            p.energy = sh.lineEnergy(line);
            const double theta = rng.uniform() * PI;
            const double phi = rng.uniform() * 2 * PI;
            peturb(p.dir, theta, phi);
            return E - p.energy;
        }
        return E;
    }

    // rayleightScatter (transport.hpp:264-298)
    void rayleigh(Particle& p, int mat, Pcg32& rng)
    {
        if (model == 0) {
            double theta;
            bool reject = true;
            while (reject) {
                const double extreme = (4 * std::sqrt(2.0)) / (3 * std::sqrt(3.0));
                const double r1 = rng.uniform() * extreme;
                theta = rng.uniform() * PI;
                const double s = std::sin(theta);
                reject = r1 > ((2 - s * s) * s);
            }
            peturb(p.dir, theta, rng.uniform() * 2 * PI);
        } else {
            const double qmax = p.energy / KEV_TO_ANGSTROM;
            const double qmax2 = qmax * qmax;
            double cosA;
            do {
                const double q2 = rita(lut, mat, qmax2, rng);
                const double invE = KEV_TO_ANGSTROM / p.energy;
                cosA = 1 - 2 * q2 * invE * invE;
            } while ((1 + cosA * cosA) * 0.5 < rng.uniform());
            peturb(p.dir, std::acos(cosA), rng.uniform() * 2 * PI);
        }
    }

    // comptonScatterNRC (transport.hpp:342-483)
    double compton_ia(Particle& p, int mat, Pcg32& rng)
    {
        std::array<double, 12> probs;
        for (int s = 0; s < 12; ++s)
            probs[s] = (shell(mat, s).binding() < p.energy && shell(mat, s).j0() > 0) ? shell(mat, s).electrons() : 0;
        std::partial_sum(probs.begin(), probs.end(), probs.begin());
        int si = 0;
        const double sample = probs.back() * rng.uniform();
        while (probs[si] < sample && si < 11)
            ++si;
        const Shell sh = shell(mat, si);
        const double U = sh.binding() / ELECTRON_REST_MASS;
        const double pp = std::sqrt(2 * U + U * U);
        const double J0 = sh.j0();
        const double k = p.energy / ELECTRON_REST_MASS;
        if (U > k)
            return 0;
        const double emin = 1 / (1 + 2 * k);
        const double gmax_inv = 1 / (1 / emin + emin);
        const double sp2 = std::sqrt(2 * PI);
        const double a1 = 0.34802, a2 = -0.0958798, a3 = 0.7478556;
        const double sqrte = std::sqrt(std::exp(1.0));
        double e, cosA;
        bool rejected;
        do {
            const double r1 = rng.uniform();
            e = r1 + (1 - r1) * emin;
            const double t = (1 - e) / (k * e);
            const double sin2 = t * (2 - t);
            cosA = 1 - t;
            const double g = (1 / e + e - sin2) * gmax_inv;
            rejected = rng.uniform() > g;
            if (!rejected) {
                const double pi = (k * (k - U) * (1 - cosA) - U) / std::sqrt(2 * k * (k - U) * (1 - cosA) + U * U);
                const double kc = k * e;
                const double qc = std::sqrt(k * k + kc * kc - 2 * k * kc * cosA);
                const double alpha = qc * (1 + kc * (kc - k * cosA) / (qc * qc)) / k;
                const double bp = 1 + 2 * J0 * std::abs(pi);
                const double b = (bp * bp + 1) / 2;
                const double expb = std::exp(-b);
                double S;
                const double part1 = alpha * sp2 / (4 * J0);
                const double tp = 1 / (1 + 0.332673 * (1 + 2 * J0 * std::abs(pp)));
                const double tpi = 1 / (1 + 0.332673 * (1 + 2 * J0 * std::abs(pi)));
                const double p2p = sqrte - expb * tp * (a1 + a2 * tp + a3 * tp * tp);
                const double p2pi = sqrte - expb * tpi * (a1 + a2 * tpi + a3 * tpi * tpi);
                if (pi <= -pp)
                    S = (1 - alpha * pp) * expb / 2;
                else if (pi <= 0)
                    S = (1 - alpha * pi) * expb / 2 - part1 * (p2p - p2pi);
                else if (pi < pp)
                    S = 1 - (1 - alpha * pi) * expb / 2 - part1 * (p2p - p2pi);
                else
                    S = 1 - (1 - alpha * pp) * expb / 2;
                rejected = rng.uniform() > S;
                if (!rejected) {
                    const double Fmax = pi <= -pp ? 1 - alpha * pp : (pi >= pp ? 1 + alpha * pp : 1 + alpha * pi);
                    const double rb = 2 * rng.uniform() * expb;
                    double pz;
                    if (rb < 1)
                        pz = (1 - std::sqrt(1 - 2 * std::log(rb))) / (2 * J0) / ELECTRON_REST_MASS;
                    else
                        pz = (std::sqrt(1 - 2 * std::log(2 - rb)) - 1) / (2 * J0) / ELECTRON_REST_MASS;
                    const double Fpz = pz <= -pp ? 1 - alpha * pp : (pz >= pp ? 1 + alpha * pp : 1 + alpha * pz);
                    rejected = rng.uniform() > Fpz / Fmax;
                    if (!rejected) {
                        const double part = std::sqrt(1 - 2 * e * cosA + e * e * (1 - pz * pz * sin2));
                        const double kbar = kc / (1 - pz * pz * e * e) * (1 - pz * pz * e * cosA + pz * part);
                        e = kbar / k;
                    }
                }
            }
        } while (rejected);
        peturb(p.dir, std::acos(cosA), rng.uniform() * 2 * PI);
        const double E = p.energy;
        p.energy *= e;
        return E - p.energy;
    }

    // comptonScatter (transport.hpp:300-340)
    double compton(Particle& p, int mat, Pcg32& rng)
    {
        if (model == 2)
            return compton_ia(p, mat, rng);
        const double E = p.energy;
        const double k = E / ELECTRON_REST_MASS;
        const double emin = 1 / (1 + 2 * k);
        const double gmax_inv = 1 / (1 / emin + emin);
        double e, cosA;
        bool rejected;
        do {
            const double r1 = rng.uniform();
            e = r1 + (1 - r1) * emin;
            const double t = (1 - e) / (k * e);
            const double sin2 = t * (2 - t);
            cosA = 1 - t;
            const double g = (1 / e + e - sin2) * gmax_inv;
            const double r2 = rng.uniform();
            if (model == 1) {
                const double q = E * (1 / KEV_TO_ANGSTROM) * std::sqrt(0.5 - cosA * 0.5);
                rejected = r2 > g * scatter_factor(lut, mat, q);
            } else {
                rejected = r2 > g;
            }
        } while (rejected);
        peturb(p.dir, std::acos(cosA), rng.uniform() * 2 * PI);
        p.energy *= e;
        return E - p.energy;
    }

    bool inside(const double pos[3]) const
    {
        return (pos[0] > lo[0] && pos[0] < hi[0]) && (pos[1] > lo[1] && pos[1] < hi[1]) && (pos[2] > lo[2] && pos[2] < hi[2]);
    }

    // transportParticleToWorld (transport.hpp:702-728)
    bool to_world(Particle& p) const
    {
        if (inside(p.pos))
            return true;
        double amin = std::numeric_limits<double>::lowest(), amax = std::numeric_limits<double>::max();
        for (int i = 0; i < 3; ++i) {
            if (std::abs(p.dir[i]) > N_ERROR) {
                const double a0 = (lo[i] - p.pos[i]) / p.dir[i];
                const double an = (hi[i] - p.pos[i]) / p.dir[i];
                amin = std::max(amin, std::min(a0, an));
                amax = std::min(amax, std::max(a0, an));
            }
        }
        if (amin < amax && amin > 0) {
            for (int i = 0; i < 3; ++i)
                p.pos[i] += amin * p.dir[i];
            return true;
        }
        return false;
    }

    // Exposure::sampleParticle (exposure.hpp:280-304)
    Particle sample(const double* ex, Pcg32& rng) const
    {
        const double theta = ex[12] + rng.uniform() * (ex[13] - ex[12]);
        const double phi = ex[14] + rng.uniform() * (ex[15] - ex[14]);
        Particle p { { ex[0], ex[1], ex[2] }, { ex[9], ex[10], ex[11] }, 0.0, ex[16] };
        rotate(p.dir, ex + 6, theta);
        rotate(p.dir, ex + 3, phi);
        if (spec_n > 0) {
            const double r = rng.uniform();
            const std::uint32_t k = rng.below(static_cast<std::uint32_t>(spec_n));
            const std::uint64_t ind = r < spec_p[k] ? k : spec_a[k];
            p.energy = ind < static_cast<std::uint64_t>(spec_n - 1) ? spec_e[ind] + rng.uniform() * (spec_e[ind + 1] - spec_e[ind]) : spec_e[ind];
        } else {
            p.energy = ex[18];
        }
        if (!bowtie.empty()) {
            // BowTieFilter::sampleIntensityWeight (beamfilters.hpp:150-190)
            const double angle = std::abs(theta);
            std::size_t first = 0, last = bowtie.size() - 1;
            std::size_t it = first + (last - first) / 2;
            while (it != first) {
                if (angle < bowtie[it].first) {
                    last = it;
                    it = first;
                } else {
                    first = it;
                }
                it += (last - first) / 2;
            }
            double w;
            if (angle < bowtie[first].first)
                w = bowtie[0].second;
            else if (angle > bowtie[last].first)
                w = bowtie.back().second;
            else
                w = bowtie[first].second + (angle - bowtie[first].first) * (bowtie[last].second - bowtie[first].second) / (bowtie[last].first - bowtie[first].first);
            p.weight *= w;
        }
        if (heel_w) {
            // HeelFilter::sampleIntensityWeight (beamfilters.hpp:514-538)
            std::size_t ei = static_cast<std::size_t>(std::max(0.0, (p.energy - heel_e0 + 0.5 * heel_es) / heel_es));
            if (ei >= static_cast<std::size_t>(heel_ne))
                ei = heel_ne - 1;
            if (p.energy < heel_e0)
                ei = 0;
            std::size_t ai = static_cast<std::size_t>(std::max(0.0, (phi - heel_a0) / heel_as));
            if (ai >= static_cast<std::size_t>(heel_na))
                ai = heel_na - 1;
            if (phi < heel_a0)
                ai = 0;
            const std::size_t wi = ei * heel_na + ai;
            double w = heel_w[wi];
            if (ai < static_cast<std::size_t>(heel_na - 1)) {
                const double a0 = heel_a0 + heel_as * ai, a1 = heel_a0 + heel_as * (ai + 1);
                w = heel_w[wi] + (heel_w[wi + 1] - heel_w[wi]) * (phi - a0) / (a1 - a0);
            }
            p.weight *= w;
        }
        return p;
    }

    // woodcockParticleTracking (transport.hpp:640-700) with computeInteractions(:583-638)
    // and computeInteractionsForced (:523-581)
    void track(Particle& p, Pcg32& rng, std::uint64_t& steps)
    {
        double maxInv = 0;
        bool update = true;
        bool cont = true;
        while (cont) {
            if (update) {
                maxInv = max_inverse(lut, p.energy);
                update = false;
            }
            const double step = -std::log(rng.uniform()) * maxInv * 10;
            for (int i = 0; i < 3; ++i)
                p.pos[i] += p.dir[i] * step;
            if (!inside(p.pos))
                break;
            const std::size_t ix = static_cast<std::size_t>((p.pos[0] - lo[0]) / spacing[0]);
            const std::size_t iy = static_cast<std::size_t>((p.pos[1] - lo[1]) / spacing[1]);
            const std::size_t iz = static_cast<std::size_t>((p.pos[2] - lo[2]) / spacing[2]);
            const std::size_t idx = iz * dims[0] * dims[1] + iy * dims[0] + ix;
            ++steps;
            const int mat = material[idx];
            const auto att = attenuation(lut, mat, p.energy);
            const double attTot = att[0] + att[1] + att[2];
            const double eventProb = attTot * density[idx] * maxInv;
            if (!measurement || measurement[idx] == 0) {
                if (rng.uniform() < eventProb) {
                    const double r3 = rng.uniform() * attTot;
                    if (r3 < att[0]) {
                        const double e = photo(p, mat, rng);
                        if (p.energy < ENERGY_CUTOFF) {
                            score(idx, (e + p.energy) * p.weight);
                            p.energy = 0;
                            cont = false;
                        } else {
                            score(idx, e * p.weight);
                            update = true;
                        }
                    } else if (r3 < att[0] + att[1]) {
                        const double e = compton(p, mat, rng);
                        if (p.energy < ENERGY_CUTOFF) {
                            score(idx, (e + p.energy) * p.weight);
                            p.energy = 0;
                            cont = false;
                        } else {
                            score(idx, e * p.weight);
                            update = true;
                        }
                    } else {
                        rayleigh(p, mat, rng);
                    }
                }
            } else {
                const double photoProb = att[0] / attTot;
                const double wc = eventProb * photoProb;
                {
                    Particle f = p;
                    const double ef = photo(f, mat, rng);
                    score(idx, (f.energy < ENERGY_CUTOFF ? ef + f.energy : ef) * f.weight * wc);
                }
                if (rng.uniform() < eventProb * (1 - photoProb)) {
                    const double r2 = rng.uniform() * (att[1] + att[2]);
                    if (r2 < att[1]) {
                        const double e = compton(p, mat, rng);
                        if (p.energy < ENERGY_CUTOFF) {
                            score(idx, (e + p.energy) * p.weight);
                            p.energy = 0;
                            cont = false;
                        } else {
                            score(idx, e * p.weight);
                            update = true;
                        }
                    } else {
                        rayleigh(p, mat, rng);
                    }
                }
                if (cont)
                    p.weight *= (1 - wc);
            }
            if (cont && p.energy * p.weight < RR_THRESHOLD) {
                if (rng.uniform() < RR_PROB)
                    cont = false;
                else
                    p.weight *= 1 / (1 - RR_PROB);
            }
        }
    }

    void worker(std::uint64_t seed, std::uint64_t& steps_out)
    {
        // one PCG stream per worker (workerRun, transport.hpp:745-763)
        Pcg32 rng { seed * 0x9E3779B97F4A7C15ULL + 0x1234567ULL, (seed << 1) | 1 };
        for (int i = 0; i < 16; ++i)
            rng.next();
        std::uint64_t steps = 0;
        for (;;) {
            const std::uint64_t e = next_exposure.fetch_add(1);
            if (e >= n_exposures)
                break;
            const double* ex = exposures + e * 19;
            const std::uint64_t n = static_cast<std::uint64_t>(ex[17]);
            for (std::uint64_t h = 0; h < n; ++h) {
                Particle p = sample(ex, rng);
                if (to_world(p))
                    track(p, rng, steps);
            }
        }
        steps_out = steps;
    }
};

// alias table (dxmcrandom.hpp:229-274)
void alias_table(const double* w, int n, std::vector<double>& probs, std::vector<std::uint64_t>& alias)
{
    probs.assign(n, 0);
    alias.assign(n, 0);
    std::vector<double> norm(n);
    std::vector<std::int64_t> small(n), large(n);
    std::int64_t ns = 0, nl = 0;
    const double sum = std::accumulate(w, w + n, 0.0);
    for (int i = 0; i < n; ++i)
        norm[i] = w[i] * (n / sum);
    for (std::int64_t i = n - 1; i >= 0; --i)
        (norm[i] < 1 ? small[ns++] : large[nl++]) = i;
    while (ns && nl) {
        const auto s = small[--ns], l = large[--nl];
        probs[s] = norm[s];
        alias[s] = l;
        norm[l] = norm[l] + norm[s] - 1;
        (norm[l] < 1 ? small[ns++] : large[nl++]) = l;
    }
    while (nl)
        probs[large[--nl]] = 1;
    while (ns)
        probs[small[--ns]] = 1;
}

} // namespace

extern "C" {

struct PortLut {
    int n_materials;
    int n_energy;
    int linear_index;
    int pad;
    double linear_step;
    double linear_energy;
    const double* log_energy;
    const double* coefficients;
    const double* max_coefficients;
    const double* rita;
    const double* spline;
    const double* shells; // n_materials * 12 * 13
};

struct PortWorld {
    std::uint64_t dims[3];
    double spacing[3];
    double origin[3];
    const double* density;
    const std::uint8_t* material;
    const std::uint8_t* measurement;
};

struct PortSource {
    const double* exposures; // n x 19
    std::uint64_t n_exposures;
    int spec_n;
    const double* spec_energies;
    const double* spec_weights;
    int heel_ne, heel_na;
    double heel_e0, heel_es, heel_a0, heel_as;
    const double* heel_weights;
    int bowtie_n;
    const double* bowtie_angles;
    const double* bowtie_weights;
};

// 0: the reference's peturb; 1: the normalised physics mode (for the next runs).
void oracle_port_set_direction(int normalized) { g_normalize_direction = normalized != 0; }

// Runs the transport and writes energy imparted (keV) and its squared sum per
// voxel (raw tallies, the reference's Result before normalizeScoring).
// Returns the wall time in seconds; out_steps receives the Woodcock step count.
double oracle_port_transport(const PortLut* lut, const PortWorld* w, const PortSource* s, int model, int n_threads,
    std::uint64_t seed, double* dose, double* variance, std::uint32_t* n_events, std::uint64_t* out_steps)
{
    Job job;
    job.lut.nm = lut->n_materials;
    job.lut.R = lut->n_energy;
    job.lut.linear_index = static_cast<std::size_t>(lut->linear_index);
    job.lut.linear_step = lut->linear_step;
    job.lut.linear_energy = lut->linear_energy;
    job.lut.x = lut->log_energy;
    job.lut.coef = lut->coefficients;
    job.lut.maxcoef = lut->max_coefficients;
    job.lut.rita = lut->rita;
    job.lut.spline = lut->spline;
    job.lut.shells = lut->shells;
    job.density = w->density;
    job.material = w->material;
    job.measurement = w->measurement;
    for (int i = 0; i < 3; ++i) {
        job.dims[i] = w->dims[i];
        job.spacing[i] = w->spacing[i];
        // World<double>::updateMatrixExtent (world.hpp:55-68)
        const double half = (w->dims[i] * w->spacing[i]) * 0.5;
        const double lower = w->origin[i] - half, upper = w->origin[i] + half;
        job.lo[i] = std::nextafter(lower, upper);
        job.hi[i] = std::nextafter(upper, lower);
    }
    job.model = model;
    job.exposures = s->exposures;
    job.n_exposures = s->n_exposures;
    job.spec_n = s->spec_n;
    job.spec_e = s->spec_energies;
    if (s->spec_n > 0)
        alias_table(s->spec_weights, s->spec_n, job.spec_p, job.spec_a);
    job.heel_w = s->heel_weights;
    job.heel_ne = s->heel_ne;
    job.heel_na = s->heel_na;
    job.heel_e0 = s->heel_e0;
    job.heel_es = s->heel_es;
    job.heel_a0 = s->heel_a0;
    job.heel_as = s->heel_as;
    if (s->bowtie_n > 0) {
        for (int i = 0; i < s->bowtie_n; ++i)
            job.bowtie.emplace_back(std::abs(s->bowtie_angles[i]), s->bowtie_weights[i]);
        std::sort(job.bowtie.begin(), job.bowtie.end());
        double mean = 0;
        for (auto& b : job.bowtie)
            mean += b.second;
        mean /= job.bowtie.size();
        for (auto& b : job.bowtie)
            b.second /= mean;
    }
    job.dose = dose;
    job.var = variance;
    job.nev = n_events;
    const int nt = n_threads > 0 ? n_threads : std::max(1u, std::thread::hardware_concurrency());
    std::vector<std::uint64_t> steps(nt, 0);
    const auto t0 = std::chrono::steady_clock::now();
    std::vector<std::thread> threads;
    for (int t = 1; t < nt; ++t)
        threads.emplace_back([&, t] { job.worker(seed + 7919 * t, steps[t]); });
    job.worker(seed, steps[0]);
    for (auto& th : threads)
        th.join();
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (out_steps)
        *out_steps = std::accumulate(steps.begin(), steps.end(), std::uint64_t { 0 });
    return secs;
}

} // extern "C"
