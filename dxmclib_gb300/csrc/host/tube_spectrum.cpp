// X-ray tube spectra: thick-target semi-relativistic Bethe-Heitler
// bremsstrahlung from tabulated electron fluence in tungsten, tungsten K lines
// and filtration (see tube_spectrum.hpp).  The numerical steps (depth and
// energy-fraction grids, the interpolation of the fluence tables, the line
// model) follow DXMClib's so that the spectra agree with the reference's to
// rounding; the bremsstrahlung integral is organised as a product of a
// per-voltage fluence matrix with per-energy cross sections.
#include "tube_spectrum.hpp"

#include "../physics/physics_model.hpp"

#include <algorithm>
#include <cmath>
#include <mutex>
#include <unordered_map>

namespace dxmc_gb300::host {

namespace {

#include "tungsten_fluence.inc"

namespace phys = dxmc_gb300::physics;

constexpr int TUNGSTEN_Z = 74;
constexpr double ELECTRON_REST_MASS = 510.9989461; // keV (constants.hpp)
constexpr double FINE_STRUCTURE = 7.29735308E-03;
constexpr double ELECTRON_RADIUS = 2.81794092E-15; // m
constexpr double DEPTH_MAX = 14.0;                  // mg/cm2 of the depth integral (at 100 keV)
constexpr double DEPTH_STEP = 0.1;
constexpr double FRACTION_MAX = 1.0;                // electron energy fraction integral
constexpr double FRACTION_STEP = 0.005;
constexpr double FLUENCE_ENERGY = 100.0;            // keV of the tabulated electron transport

// Thomson-Whiddington range of an electron of energy T0 (keV) in tungsten, mg/cm2
// (valid for 50-150 keV)
double tw_range(double T0) { return 0.0119 * std::pow(T0, 1.513); }

// First node >= v, kept at least two nodes from the end (the upper node of the
// pair is the next one): the node choice of the reference's table lookups.
int node_at_or_above(const double* nodes, int n, double v)
{
    const int i = static_cast<int>(std::lower_bound(nodes, nodes + n, v) - nodes);
    const int left = n - i;
    return left < 2 ? n - 3 + left : i;
}

// Fraction of the initial energy squared left at depth x by the Thomson-Whiddington law
double tw_law(double x, double voltage)
{
    const int i = node_at_or_above(TW_VOLTAGE, 5, voltage);
    const double C = TW_CONSTANT[i] + ((TW_CONSTANT[i + 1] - TW_CONSTANT[i]) / (TW_VOLTAGE[i + 1] - TW_VOLTAGE[i])) * (voltage - TW_VOLTAGE[i]);
    const double t = (voltage * voltage - C * x) / (voltage * voltage);
    return t < 0 ? 0 : t;
}

double fraction_f(double x, double voltage) { return std::pow(tw_law(x, voltage), 1.753); }

double fraction_m(double x, double voltage)
{
    constexpr double K = 18.0, Bd = 0.584, B0 = 0.5;
    const double e = 1 - std::exp(-K * x / tw_range(voltage));
    const double F = Bd * e;
    const double B = B0 + (Bd - B0) * e;
    return fraction_f(x, voltage) * B * (F + 1) / (1 - B * F);
}

// Bilinear interpolation of a fluence table (rows FLUENCE_U, columns `depth`) at
// (u, x), both clamped to the table
double fluence(const double* table, const double* depth, double u, double x)
{
    x = std::clamp(x, depth[0], depth[FLUENCE_X_NODES - 1]);
    u = std::clamp(u, FLUENCE_U[0], FLUENCE_U[FLUENCE_U_NODES - 1]);
    const int ix = node_at_or_above(depth, FLUENCE_X_NODES, x);
    const int iu = node_at_or_above(FLUENCE_U, FLUENCE_U_NODES, u);
    const double x1 = depth[ix], x2 = depth[ix + 1];
    const double u1 = FLUENCE_U[iu], u2 = FLUENCE_U[iu + 1];
    const double* lo = table + iu * FLUENCE_X_NODES;
    const double* hi = lo + FLUENCE_X_NODES;
    const double wx1 = (x2 - x) / (x2 - x1), wx2 = (x - x1) / (x2 - x1);
    const double at_u1 = wx1 * lo[ix] + wx2 * lo[ix + 1];
    const double at_u2 = wx1 * hi[ix] + wx2 * hi[ix + 1];
    return ((u2 - u) / (u2 - u1)) * at_u1 + ((u - u1) / (u2 - u1)) * at_u2;
}

// Semi-relativistic Bethe-Heitler cross section (Elwert-corrected) of an
// electron of kinetic energy Ti (keV) emitting a photon hv (keV) in tungsten
double bethe_heitler(double hv, double Ti)
{
    constexpr double m = ELECTRON_REST_MASS;
    constexpr double phi = (TUNGSTEN_Z * TUNGSTEN_Z) * ELECTRON_RADIUS * ELECTRON_RADIUS * FINE_STRUCTURE;
    constexpr double prefactor = (phi * 2) / 3;
    const double Ei = m + Ti;
    const double Ef = Ei - hv;
    const double pi = std::sqrt(Ei * Ei - m * m);
    const double pf2 = Ef * Ef - m * m;
    if (pf2 <= 0)
        return 0;
    const double pf = std::sqrt(pf2);
    const double L = 2 * std::log((Ei * Ef + pi * pf - m * m) / (m * hv));
    const double elwert = pi / pf;
    return prefactor * (4 * Ei * Ef * L - 7 * pi * pf) / (hv * pi * pi) * elwert;
}

double tungsten_attenuation(double hv)
{
    phys::Composition w;
    w.Z = { TUNGSTEN_Z };
    w.massFraction = { 1.0 };
    w.numberFraction = { 1.0 };
    return phys::mass_attenuation_photo(w, hv) + phys::mass_attenuation_compton(w, hv) + phys::mass_attenuation_rayleigh(w, hv);
}

// The integration grids as the reference walks them (accumulated steps)
const std::vector<double>& depth_grid()
{
    static const std::vector<double> g = [] {
        std::vector<double> v;
        for (double x = 0; x <= DEPTH_MAX; x = x + DEPTH_STEP)
            v.push_back(x);
        return v;
    }();
    return g;
}
const std::vector<double>& fraction_grid()
{
    static const std::vector<double> g = [] {
        std::vector<double> v;
        for (double u = FRACTION_STEP; u <= FRACTION_MAX; u = u + FRACTION_STEP)
            v.push_back(u);
        return v;
    }();
    return g;
}

// Electron fluence at every (depth, energy fraction) node for initial energy T0:
// it depends on the voltage only, so it is built once per voltage and reused for
// every photon energy, anode angle and filter.
const std::vector<double>& fluence_matrix(double T0)
{
    static std::mutex m;
    static std::unordered_map<double, std::vector<double>> cache;
    std::lock_guard<std::mutex> lock(m);
    auto it = cache.find(T0);
    if (it != cache.end())
        return it->second;
    const auto& xs = depth_grid();
    const auto& us = fraction_grid();
    const double scale = tw_range(FLUENCE_ENERGY) / tw_range(T0);
    std::vector<double> rho(xs.size() * us.size());
    for (std::size_t j = 0; j < xs.size(); ++j) {
        const double x = xs[j];
        const double nf = fraction_f(x, T0), nm = fraction_m(x, T0);
        for (std::size_t k = 0; k < us.size(); ++k)
            rho[j * us.size() + k] = nf * fluence(FLUENCE_F, FLUENCE_F_DEPTH, us[k], x * scale)
                + nm * fluence(FLUENCE_M, FLUENCE_M_DEPTH, us[k], x * scale);
    }
    return cache.emplace(T0, std::move(rho)).first->second;
}

} // namespace

namespace {

// Photons of energy hv produced per depth node by electrons of initial energy T0
// (the fluence matrix times the cross sections).  It does not depend on the
// take-off angle, so a heel table's spectra at several angles, and every tube
// with the same voltage, share it.
struct DepthKey {
    double T0, hv;
    bool operator==(const DepthKey& o) const { return T0 == o.T0 && hv == o.hv; }
};
struct DepthKeyHash {
    std::size_t operator()(const DepthKey& k) const
    {
        return std::hash<double>()(k.T0) * 1000003u ^ std::hash<double>()(k.hv);
    }
};

const std::vector<double>& production_at_depth(double T0, double hv)
{
    static std::mutex m;
    static std::unordered_map<DepthKey, std::vector<double>, DepthKeyHash> cache;
    std::lock_guard<std::mutex> lock(m);
    const DepthKey key { T0, hv };
    auto it = cache.find(key);
    if (it != cache.end())
        return it->second;
    const auto& xs = depth_grid();
    const auto& us = fraction_grid();
    const auto& rho = fluence_matrix(T0);
    std::vector<double> sigma(us.size());
    for (std::size_t k = 0; k < us.size(); ++k)
        sigma[k] = bethe_heitler(hv, T0 * us[k]);
    std::vector<double> at_depth(xs.size());
    for (std::size_t j = 0; j < xs.size(); ++j) {
        const double* r = rho.data() + j * us.size();
        double a = 0;
        for (std::size_t k = 0; k < us.size(); ++k)
            a = a + sigma[k] * r[k] * FRACTION_STEP;
        at_depth[j] = a;
    }
    return cache.emplace(key, std::move(at_depth)).first->second;
}

} // namespace

double thick_target_bremsstrahlung(double T0, double hv, double takeoff_angle)
{
    if (hv <= 0)
        return 0;
    const double att = tungsten_attenuation(hv);
    const auto& xs = depth_grid();
    const auto& at_depth = production_at_depth(T0, hv);
    const double sin_takeoff = std::sin(takeoff_angle);
    double total = 0;
    for (std::size_t j = 0; j < xs.size(); ++j) {
        // photons produced at depth x leave the anode through x / sin(takeoff) of tungsten
        total = total + at_depth[j] * std::exp(-att * xs[j] * 0.001 / sin_takeoff) * DEPTH_STEP;
    }
    return total;
}

std::vector<double> tube_spectrum(double voltage, double takeoff_angle, double line_takeoff_angle,
    const std::vector<double>& energies, const std::vector<SpectrumFilter>& filters, bool normalize)
{
    std::vector<double> s(energies.size());
    for (std::size_t i = 0; i < energies.size(); ++i)
        s[i] = thick_target_bremsstrahlung(voltage, energies[i], takeoff_angle);
    // tungsten K lines: energy (keV), share, added to the spectrum bin at or above the
    // line when that bin lies within 2 keV of it
    constexpr double line_energy[4] = { 59.3, 58.0, 67.2, 69.1 };
    constexpr double line_share[4] = { 0.505, 0.291, 0.162, 0.042 };
    constexpr double P = 0.33, omega_k = 0.94, rk = 4.4;
    for (int l = 0; l < 4; ++l) {
        const double n = (1 + P) * line_share[l] * rk * omega_k * thick_target_bremsstrahlung(voltage, line_energy[l], line_takeoff_angle);
        const auto it = std::lower_bound(energies.begin(), energies.end(), line_energy[l]);
        if (it != energies.end() && std::abs(line_energy[l] - *it) <= 2.0)
            s[static_cast<std::size_t>(it - energies.begin())] += n;
    }
    for (const auto& f : filters) {
        const double cm = f.mm * 0.1;
        for (std::size_t i = 0; i < energies.size(); ++i)
            s[i] = s[i] * std::exp(-f.total_attenuation(f.user, energies[i]) * f.density * cm);
    }
    if (normalize) {
        double sum = 0;
        for (double v : s)
            sum += v;
        for (double& v : s)
            v = v / sum;
    }
    return s;
}

} // namespace dxmc_gb300::host
