// Closed-form photon-interaction data model; see physics_model.hpp for the
// list of models and their sources.
#include "physics_model.hpp"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <stdexcept>

namespace dxmc_gb300::physics {

namespace {

    constexpr double PI = 3.14159265358979323846;

    struct ElementRecord {
        const char* symbol;
        double weight;
        double density;
    };

    // Standard atomic weights (IUPAC, abridged) and densities at standard
    // conditions (gases at 0 C, 1 atm).
    const ElementRecord ELEMENT_RECORDS[MAX_Z + 1] = {
        { "", 0, 0 },
        { "H", 1.008, 8.99e-5 }, { "He", 4.0026, 1.785e-4 }, { "Li", 6.94, 0.534 },
        { "Be", 9.0122, 1.85 }, { "B", 10.81, 2.34 }, { "C", 12.011, 2.26 },
        { "N", 14.007, 1.251e-3 }, { "O", 15.999, 1.429e-3 }, { "F", 18.998, 1.696e-3 },
        { "Ne", 20.180, 9.0e-4 }, { "Na", 22.990, 0.971 }, { "Mg", 24.305, 1.738 },
        { "Al", 26.982, 2.699 }, { "Si", 28.085, 2.33 }, { "P", 30.974, 1.82 },
        { "S", 32.06, 2.07 }, { "Cl", 35.45, 3.214e-3 }, { "Ar", 39.948, 1.784e-3 },
        { "K", 39.098, 0.862 }, { "Ca", 40.078, 1.55 }, { "Sc", 44.956, 2.99 },
        { "Ti", 47.867, 4.54 }, { "V", 50.942, 6.11 }, { "Cr", 51.996, 7.19 },
        { "Mn", 54.938, 7.33 }, { "Fe", 55.845, 7.874 }, { "Co", 58.933, 8.9 },
        { "Ni", 58.693, 8.902 }, { "Cu", 63.546, 8.96 }, { "Zn", 65.38, 7.133 },
        { "Ga", 69.723, 5.904 }, { "Ge", 72.630, 5.323 }, { "As", 74.922, 5.73 },
        { "Se", 78.971, 4.5 }, { "Br", 79.904, 3.12 }, { "Kr", 83.798, 3.74e-3 },
        { "Rb", 85.468, 1.532 }, { "Sr", 87.62, 2.54 }, { "Y", 88.906, 4.47 },
        { "Zr", 91.224, 6.506 }, { "Nb", 92.906, 8.57 }, { "Mo", 95.95, 10.22 },
        { "Tc", 98.0, 11.5 }, { "Ru", 101.07, 12.41 }, { "Rh", 102.91, 12.41 },
        { "Pd", 106.42, 12.02 }, { "Ag", 107.87, 10.5 }, { "Cd", 112.41, 8.65 },
        { "In", 114.82, 7.31 }, { "Sn", 118.71, 7.31 }, { "Sb", 121.76, 6.691 },
        { "Te", 127.60, 6.24 }, { "I", 126.90, 4.93 }, { "Xe", 131.29, 5.89e-3 },
        { "Cs", 132.91, 1.873 }, { "Ba", 137.33, 3.5 }, { "La", 138.91, 6.154 },
        { "Ce", 140.12, 6.657 }, { "Pr", 140.91, 6.71 }, { "Nd", 144.24, 6.9 },
        { "Pm", 145.0, 7.22 }, { "Sm", 150.36, 7.46 }, { "Eu", 151.96, 5.243 },
        { "Gd", 157.25, 7.9 }, { "Tb", 158.93, 8.229 }, { "Dy", 162.50, 8.55 },
        { "Ho", 164.93, 8.795 }, { "Er", 167.26, 9.066 }, { "Tm", 168.93, 9.321 },
        { "Yb", 173.05, 6.73 }, { "Lu", 174.97, 9.84 }, { "Hf", 178.49, 13.31 },
        { "Ta", 180.95, 16.654 }, { "W", 183.84, 19.3 }, { "Re", 186.21, 21.02 },
        { "Os", 190.23, 22.57 }, { "Ir", 192.22, 22.42 }, { "Pt", 195.08, 21.45 },
        { "Au", 196.97, 19.32 }, { "Hg", 200.59, 13.546 }, { "Tl", 204.38, 11.72 },
        { "Pb", 207.2, 11.35 }, { "Bi", 208.98, 9.747 }, { "Po", 209.0, 9.32 },
        { "At", 210.0, 7.0 }, { "Rn", 222.0, 9.73e-3 }, { "Fr", 223.0, 1.87 },
        { "Ra", 226.0, 5.5 }, { "Ac", 227.0, 10.07 }, { "Th", 232.04, 11.72 },
        { "Pa", 231.04, 15.37 }, { "U", 238.03, 18.95 }
    };

    // Slater effective principal quantum number.
    double slater_nstar(int n)
    {
        static const double table[] = { 0, 1.0, 2.0, 3.0, 3.7, 4.0, 4.2, 4.4 };
        return table[std::clamp(n, 1, 7)];
    }

    // Slater group ordering: (1s)(2s2p)(3s3p)(3d)(4s4p)(4d)(4f)(5s5p)(5d)(5f)(6s6p)(6d)(7s7p).
    int slater_group(int n, int l)
    {
        struct G {
            int n, l; // l = 1 stands for the (ns,np) group
        };
        static const G groups[] = { { 1, 1 }, { 2, 1 }, { 3, 1 }, { 3, 2 }, { 4, 1 }, { 4, 2 }, { 4, 3 },
            { 5, 1 }, { 5, 2 }, { 5, 3 }, { 6, 1 }, { 6, 2 }, { 7, 1 } };
        const int key_l = l <= 1 ? 1 : l;
        for (int g = 0; g < static_cast<int>(sizeof(groups) / sizeof(groups[0])); ++g)
            if (groups[g].n == n && groups[g].l == key_l)
                return g;
        return 12;
    }

    // Spectroscopic subshell index: K, L1, L2, L3, M1..M5, N1..N7, O1..O7, P1..P5, Q1...
    int subshell_index(int n, int l, double j)
    {
        int idx = 0;
        for (int nn = 1; nn <= n; ++nn) {
            const int lmax = std::min(nn - 1, 3);
            for (int ll = 0; ll <= lmax; ++ll) {
                const int nj = ll == 0 ? 1 : 2;
                for (int k = 0; k < nj; ++k) {
                    const double jj = ll == 0 ? 0.5 : (k == 0 ? ll - 0.5 : ll + 0.5);
                    if (nn == n && ll == l && std::abs(jj - j) < 1e-9)
                        return idx;
                    ++idx;
                }
            }
        }
        return idx;
    }

    Element build_element(int Z)
    {
        Element e;
        e.Z = Z;
        e.symbol = ELEMENT_RECORDS[Z].symbol;
        e.atomic_weight = ELEMENT_RECORDS[Z].weight;
        e.density = ELEMENT_RECORDS[Z].density;

        // Madelung (n + l, then n) filling order.
        std::vector<std::pair<int, int>> order;
        for (int s = 1; s <= 8; ++s)
            for (int n = s; n >= 1; --n) {
                const int l = s - n;
                if (l < n && l <= 3)
                    order.emplace_back(n, l);
            }
        int remaining = Z;
        struct Occ {
            int n, l;
            double j;
            int cap;
            int occ;
        };
        std::vector<Occ> occs;
        for (auto [n, l] : order) {
            if (remaining <= 0)
                break;
            if (l == 0) {
                const int o = std::min(remaining, 2);
                occs.push_back({ n, 0, 0.5, 2, o });
                remaining -= o;
            } else {
                const int c1 = 2 * l, c2 = 2 * l + 2;
                const int o1 = std::min(remaining, c1);
                occs.push_back({ n, l, l - 0.5, c1, o1 });
                remaining -= o1;
                if (remaining > 0) {
                    const int o2 = std::min(remaining, c2);
                    occs.push_back({ n, l, l + 0.5, c2, o2 });
                    remaining -= o2;
                }
            }
        }
        // Slater screening for each subshell.
        for (const auto& o : occs) {
            const int g = slater_group(o.n, o.l);
            double S = 0;
            for (const auto& other : occs) {
                const int go = slater_group(other.n, other.l);
                double count = other.occ;
                if (&other == &o)
                    count -= 1; // the electron itself
                if (count <= 0)
                    continue;
                if (go == g) {
                    S += count * (o.n == 1 ? 0.30 : 0.35);
                } else if (go < g) {
                    if (o.l <= 1) {
                        if (other.n == o.n - 1)
                            S += count * 0.85;
                        else if (other.n < o.n - 1)
                            S += count * 1.00;
                        else // same n but lower group cannot happen for s/p
                            S += count * 1.00;
                    } else {
                        S += count * 1.00;
                    }
                }
            }
            Subshell sh;
            sh.n = o.n;
            sh.l = o.l;
            sh.j = o.j;
            sh.occupancy = o.occ;
            sh.nstar = slater_nstar(o.n);
            sh.zeff = std::max(Z - S, 1.0);
            double g_split = 1.0;
            if (o.l == 0 && o.n >= 2)
                g_split = 1.0 + 0.05 / sh.nstar; // s-orbital penetration
            else if (o.l >= 1 && o.j < o.l)
                g_split = 1.0 + (FINE_STRUCTURE * sh.zeff) * (FINE_STRUCTURE * sh.zeff) / (2.0 * sh.nstar); // spin-orbit
            sh.binding = RYDBERG_KEV * (sh.zeff / sh.nstar) * (sh.zeff / sh.nstar) * g_split;
            sh.index = subshell_index(o.n, o.l, o.j);
            e.shells.push_back(sh);
        }
        std::sort(e.shells.begin(), e.shells.end(), [](const auto& a, const auto& b) { return a.index < b.index; });
        return e;
    }

    const std::vector<Element>& element_table()
    {
        static const std::vector<Element> table = [] {
            std::vector<Element> t(MAX_Z + 1);
            for (int Z = 1; Z <= MAX_Z; ++Z)
                t[Z] = build_element(Z);
            return t;
        }();
        return table;
    }

    const Subshell* find_shell(const Element& e, int shellIndex)
    {
        for (const auto& s : e.shells)
            if (s.index == shellIndex)
                return &s;
        return nullptr;
    }

    double shell_form_factor(const Subshell& s, double x)
    {
        const double a = s.nstar * s.nstar * BOHR_RADIUS_ANGSTROM / s.zeff;
        const double t = 2 * PI * x * a;
        const double d = 1 + t * t;
        return 1.0 / (d * d);
    }

    // Gauss-Legendre nodes/weights on [-1, 1] (Newton iteration on P_n).
    struct Gauss {
        std::vector<double> x, w;
        explicit Gauss(int n)
        {
            x.resize(n);
            w.resize(n);
            for (int i = 0; i < n; ++i) {
                double z = std::cos(PI * (i + 0.75) / (n + 0.5));
                for (int it = 0; it < 100; ++it) {
                    double p1 = 1, p2 = 0;
                    for (int k = 1; k <= n; ++k) {
                        const double p3 = p2;
                        p2 = p1;
                        p1 = ((2 * k - 1) * z * p2 - (k - 1) * p3) / k;
                    }
                    const double pp = n * (z * p1 - p2) / (z * z - 1);
                    const double dz = p1 / pp;
                    z -= dz;
                    if (std::abs(dz) < 1e-15) {
                        double q1 = 1, q2 = 0;
                        for (int k = 1; k <= n; ++k) {
                            const double q3 = q2;
                            q2 = q1;
                            q1 = ((2 * k - 1) * z * q2 - (k - 1) * q3) / k;
                        }
                        const double qp = n * (z * q1 - q2) / (z * z - 1);
                        x[i] = z;
                        w[i] = 2 / ((1 - z * z) * qp * qp);
                        break;
                    }
                }
            }
        }
    };

    // Angular integral over the momentum transfer x in [0, 1/lambda] carried out
    // on a log(x) grid, which resolves the narrow forward peak of F^2 at high
    // energies. kind 0: coherent (Thomson x F^2); 1: incoherent (KN x S);
    // 2: incoherent energy-transfer (KN x S x (1 - E'/E)).
    double angular_integral(int Z, double energy, int kind)
    {
        static const Gauss gauss(8);
        const double lambda = KEV_ANGSTROM / energy;
        const double xmax = 1.0 / lambda;
        const double tmin = std::log(1e-6), tmax = std::log(xmax);
        const int nsub = 96;
        const double k = energy / ELECTRON_MASS_KEV;
        double sum = 0;
        for (int s = 0; s < nsub; ++s) {
            const double a = tmin + (tmax - tmin) * s / nsub;
            const double b = tmin + (tmax - tmin) * (s + 1) / nsub;
            for (std::size_t g = 0; g < gauss.x.size(); ++g) {
                const double t = 0.5 * (a + b) + 0.5 * (b - a) * gauss.x[g];
                const double x = std::exp(t);
                // mu = 1 - 2 (lambda x)^2 ; dmu = 4 lambda^2 x dx = 4 lambda^2 x^2 dt
                const double lx = lambda * x;
                const double mu = 1 - 2 * lx * lx;
                const double jac = 4 * lambda * lambda * x * x;
                double f;
                if (kind == 0) {
                    const double F = form_factor(Z, x);
                    f = (1 + mu * mu) * F * F;
                } else {
                    const double ratio = 1 / (1 + k * (1 - mu)); // E'/E
                    const double kn = ratio * ratio * (ratio + 1 / ratio - (1 - mu * mu));
                    f = kn * incoherent_sf(Z, x);
                    if (kind == 2)
                        f *= (1 - ratio);
                }
                sum += 0.5 * (b - a) * gauss.w[g] * f * jac;
            }
        }
        // dsigma/dOmega integrated over phi: 2 pi * (r_e^2 / 2) * integral dmu
        const double cm2 = PI * ELECTRON_RADIUS_CM * ELECTRON_RADIUS_CM * sum;
        return cm2 * 1e24; // barn
    }

    // Per-element cache of the angular integrals on a log-energy grid.
    struct ScatterCache {
        static constexpr int N = 481;
        static constexpr double LOG_EMIN = -1.0; // 0.1 keV
        static constexpr double LOG_EMAX = 3.0;  // 1000 keV
        std::array<double, N> coh {}, inc {}, tr {};
    };

    const ScatterCache& scatter_cache(int Z)
    {
        static std::mutex mtx;
        static std::map<int, std::unique_ptr<ScatterCache>> caches;
        std::lock_guard<std::mutex> lock(mtx);
        auto it = caches.find(Z);
        if (it != caches.end())
            return *it->second;
        auto c = std::make_unique<ScatterCache>();
        for (int i = 0; i < ScatterCache::N; ++i) {
            const double le = ScatterCache::LOG_EMIN + (ScatterCache::LOG_EMAX - ScatterCache::LOG_EMIN) * i / (ScatterCache::N - 1);
            const double e = std::pow(10.0, le);
            c->coh[i] = angular_integral(Z, e, 0);
            c->inc[i] = angular_integral(Z, e, 1);
            c->tr[i] = angular_integral(Z, e, 2);
        }
        auto& ref = *c;
        caches[Z] = std::move(c);
        return ref;
    }

    double cache_interp(const std::array<double, ScatterCache::N>& table, double energy)
    {
        const double le = std::log10(std::clamp(energy, 0.1, 1000.0));
        const double pos = (le - ScatterCache::LOG_EMIN) / (ScatterCache::LOG_EMAX - ScatterCache::LOG_EMIN) * (ScatterCache::N - 1);
        int i = static_cast<int>(pos);
        i = std::clamp(i, 0, ScatterCache::N - 2);
        const double f = pos - i;
        const double y0 = std::log(std::max(table[i], 1e-300));
        const double y1 = std::log(std::max(table[i + 1], 1e-300));
        return std::exp(y0 + (y1 - y0) * f);
    }

    double per_gram(int Z)
    {
        return AVOGADRO / element(Z).atomic_weight * 1e-24;
    }

    void normalise(Composition& c)
    {
        const double ms = std::accumulate(c.massFraction.begin(), c.massFraction.end(), 0.0);
        for (auto& m : c.massFraction)
            m /= ms;
        c.numberFraction.resize(c.Z.size());
        for (std::size_t i = 0; i < c.Z.size(); ++i)
            c.numberFraction[i] = c.massFraction[i] / element(c.Z[i]).atomic_weight;
        const double ns = std::accumulate(c.numberFraction.begin(), c.numberFraction.end(), 0.0);
        for (auto& n : c.numberFraction)
            n /= ns;
    }

    struct NamedMaterial {
        const char* name;
        double density;
        std::vector<std::pair<int, double>> mass; // (Z, mass fraction)
    };

    // Project-defined reference compositions (mass fractions).
    const std::vector<NamedMaterial>& named_materials()
    {
        static const std::vector<NamedMaterial> list = {
            { "Water, Liquid", 1.0, { { 1, 0.111894 }, { 8, 0.888106 } } },
            { "Air, Dry (near sea level)", 0.00120479, { { 6, 0.000124 }, { 7, 0.755268 }, { 8, 0.231781 }, { 18, 0.012827 } } },
            { "Polymethyl Methacralate (Lucite, Perspex)", 1.19, { { 1, 0.080538 }, { 6, 0.599848 }, { 8, 0.319614 } } },
            { "Tissue, Soft (ICRP)", 1.03, { { 1, 0.104472 }, { 6, 0.232190 }, { 7, 0.024880 }, { 8, 0.630238 }, { 11, 0.001130 }, { 12, 0.000130 }, { 15, 0.001330 }, { 16, 0.001990 }, { 17, 0.001340 }, { 19, 0.001990 }, { 20, 0.000230 }, { 26, 0.000050 }, { 30, 0.000030 } } },
            { "Lung Tissue (ICRU-44)", 1.05, { { 1, 0.103 }, { 6, 0.105 }, { 7, 0.031 }, { 8, 0.749 }, { 11, 0.002 }, { 15, 0.002 }, { 16, 0.003 }, { 17, 0.003 }, { 19, 0.002 } } },
            { "Bone, Cortical (ICRP)", 1.92, { { 1, 0.034 }, { 6, 0.155 }, { 7, 0.042 }, { 8, 0.435 }, { 11, 0.001 }, { 12, 0.002 }, { 15, 0.103 }, { 16, 0.003 }, { 20, 0.225 } } },
            { "Adipose Tissue (ICRP)", 0.95, { { 1, 0.114 }, { 6, 0.598 }, { 7, 0.007 }, { 8, 0.278 }, { 11, 0.001 }, { 16, 0.001 }, { 17, 0.001 } } },
        };
        return list;
    }

} // namespace

const Element& element(int Z)
{
    if (Z < 1 || Z > MAX_Z)
        throw std::out_of_range("atomic number out of range");
    return element_table()[Z];
}

int atomic_number_from_symbol(const std::string& symbol)
{
    for (int Z = 1; Z <= MAX_Z; ++Z)
        if (symbol == ELEMENT_RECORDS[Z].symbol)
            return Z;
    return 0;
}

double photo_subshell_barn(int Z, int shellIndex, double energy)
{
    const auto* s = find_shell(element(Z), shellIndex);
    if (!s || energy < s->binding || energy <= 0)
        return 0;
    // Kramers: per electron K0 * Ry * B^2 / (n* E^3), K0 = 64 pi alpha a0^2 / (3 sqrt 3)
    const double a0_cm = BOHR_RADIUS_ANGSTROM * 1e-8;
    const double K0 = 64 * PI * FINE_STRUCTURE * a0_cm * a0_cm / (3 * std::sqrt(3.0));
    const double cm2 = s->occupancy * K0 * RYDBERG_KEV * s->binding * s->binding / (s->nstar * energy * energy * energy);
    return cm2 * 1e24;
}

double photo_barn(int Z, double energy)
{
    double sum = 0;
    for (const auto& s : element(Z).shells)
        sum += photo_subshell_barn(Z, s.index, energy);
    return sum;
}

double incoherent_barn(int Z, double energy) { return cache_interp(scatter_cache(Z).inc, energy); }
double coherent_barn(int Z, double energy) { return cache_interp(scatter_cache(Z).coh, energy); }
double energy_transfer_fraction(int Z, double energy)
{
    const auto& c = scatter_cache(Z);
    return cache_interp(c.tr, energy) / cache_interp(c.inc, energy);
}

double form_factor(int Z, double x)
{
    double F = 0;
    for (const auto& s : element(Z).shells)
        F += s.occupancy * shell_form_factor(s, x);
    return F;
}

double incoherent_sf(int Z, double x)
{
    double S = 0;
    for (const auto& s : element(Z).shells) {
        const double f = shell_form_factor(s, x);
        S += s.occupancy * (1 - f * f);
    }
    return S;
}

double compton_profile_j0(int Z, int shellIndex)
{
    const auto* s = find_shell(element(Z), shellIndex);
    if (!s)
        return 0;
    return 8.0 * s->nstar / (3.0 * PI * s->zeff);
}

double fluorescence_yield(int Z, int shellIndex)
{
    const double z4 = static_cast<double>(Z) * Z * Z * Z;
    if (shellIndex == 0)
        return z4 / (1.12e6 + z4);
    if (shellIndex >= 1 && shellIndex <= 3)
        return z4 / (1.0e8 + z4);
    return 0;
}

int fluorescence_lines(int Z, int shellIndex, double energies[3], double rates[3])
{
    // (target subshell index, relative rate) for the three strongest dipole
    // transitions filling a vacancy in K, L1, L2, L3.
    struct Line {
        int target;
        double rate;
    };
    static const Line K[] = { { 3, 0.58 }, { 2, 0.30 }, { 6, 0.12 } };  // L3, L2, M3
    static const Line L1[] = { { 6, 0.50 }, { 5, 0.30 }, { 11, 0.20 } }; // M3, M2, N3
    static const Line L2[] = { { 7, 0.60 }, { 12, 0.25 }, { 4, 0.15 } }; // M4, N4, M1
    static const Line L3[] = { { 8, 0.60 }, { 13, 0.25 }, { 7, 0.15 } }; // M5, N5, M4
    const Line* lines = nullptr;
    if (shellIndex == 0)
        lines = K;
    else if (shellIndex == 1)
        lines = L1;
    else if (shellIndex == 2)
        lines = L2;
    else if (shellIndex == 3)
        lines = L3;
    const auto& e = element(Z);
    const auto* vac = find_shell(e, shellIndex);
    int count = 0;
    if (lines && vac) {
        for (int i = 0; i < 3; ++i) {
            const auto* t = find_shell(e, lines[i].target);
            if (t && t->occupancy > 0 && t->binding < vac->binding) {
                energies[count] = vac->binding - t->binding;
                rates[count] = lines[i].rate;
                ++count;
            }
        }
    }
    for (int i = count; i < 3; ++i) {
        energies[i] = 0;
        rates[i] = 0;
    }
    return count;
}

bool parse_formula(const std::string& formula, Composition& out)
{
    // Recursive-descent parser: group := (element | '(' group ')') number? ...
    std::size_t pos = 0;
    std::map<int, double> counts;
    bool ok = true;
    auto parse_number = [&](double def) {
        const std::size_t start = pos;
        while (pos < formula.size() && (std::isdigit(static_cast<unsigned char>(formula[pos])) || formula[pos] == '.'))
            ++pos;
        if (pos == start)
            return def;
        return std::stod(formula.substr(start, pos - start));
    };
    std::function<std::map<int, double>()> parse_group = [&]() -> std::map<int, double> {
        std::map<int, double> local;
        while (pos < formula.size() && ok) {
            const char ch = formula[pos];
            if (ch == '(') {
                ++pos;
                auto inner = parse_group();
                if (pos >= formula.size() || formula[pos] != ')') {
                    ok = false;
                    return local;
                }
                ++pos;
                const double mult = parse_number(1.0);
                for (auto& [z, n] : inner)
                    local[z] += n * mult;
            } else if (ch == ')') {
                return local;
            } else if (std::isupper(static_cast<unsigned char>(ch))) {
                std::string sym(1, ch);
                ++pos;
                while (pos < formula.size() && std::islower(static_cast<unsigned char>(formula[pos])))
                    sym.push_back(formula[pos++]);
                const int Z = atomic_number_from_symbol(sym);
                if (Z == 0) {
                    ok = false;
                    return local;
                }
                local[Z] += parse_number(1.0);
            } else {
                ok = false;
                return local;
            }
        }
        return local;
    };
    if (formula.empty())
        return false;
    counts = parse_group();
    if (!ok || pos != formula.size() || counts.empty())
        return false;
    Composition c;
    for (auto& [Z, n] : counts) {
        if (n <= 0)
            return false;
        c.Z.push_back(Z);
        c.massFraction.push_back(n * element(Z).atomic_weight);
    }
    normalise(c);
    out = c;
    return true;
}

bool named_material(const std::string& name, Composition& out, double& density)
{
    for (const auto& m : named_materials()) {
        if (name == m.name) {
            Composition c;
            for (auto [Z, w] : m.mass) {
                c.Z.push_back(Z);
                c.massFraction.push_back(w);
            }
            normalise(c);
            out = c;
            density = m.density;
            return true;
        }
    }
    return false;
}

std::vector<std::string> named_material_list()
{
    std::vector<std::string> names;
    for (const auto& m : named_materials())
        names.emplace_back(m.name);
    return names;
}

double mass_attenuation_photo(const Composition& c, double energy)
{
    double s = 0;
    for (std::size_t i = 0; i < c.Z.size(); ++i)
        s += c.massFraction[i] * photo_barn(c.Z[i], energy) * per_gram(c.Z[i]);
    return s;
}
double mass_attenuation_compton(const Composition& c, double energy)
{
    double s = 0;
    for (std::size_t i = 0; i < c.Z.size(); ++i)
        s += c.massFraction[i] * incoherent_barn(c.Z[i], energy) * per_gram(c.Z[i]);
    return s;
}
double mass_attenuation_rayleigh(const Composition& c, double energy)
{
    double s = 0;
    for (std::size_t i = 0; i < c.Z.size(); ++i)
        s += c.massFraction[i] * coherent_barn(c.Z[i], energy) * per_gram(c.Z[i]);
    return s;
}
double mass_energy_absorption(const Composition& c, double energy)
{
    double s = 0;
    for (std::size_t i = 0; i < c.Z.size(); ++i) {
        const int Z = c.Z[i];
        const double pg = per_gram(Z);
        s += c.massFraction[i] * pg * (photo_barn(Z, energy) + incoherent_barn(Z, energy) * energy_transfer_fraction(Z, energy));
    }
    return s;
}

double form_factor_squared(const Composition& c, double x)
{
    double s = 0;
    for (std::size_t i = 0; i < c.Z.size(); ++i) {
        const double F = form_factor(c.Z[i], x);
        s += c.numberFraction[i] * F * F;
    }
    return s;
}

double normalized_scatter_factor(const Composition& c, double x)
{
    double s = 0;
    for (std::size_t i = 0; i < c.Z.size(); ++i)
        s += c.numberFraction[i] * incoherent_sf(c.Z[i], x) / c.Z[i];
    return s;
}

std::vector<double> binding_energies(const Composition& c, double minEnergy)
{
    std::vector<double> edges;
    for (int Z : c.Z)
        for (const auto& s : element(Z).shells)
            if (s.occupancy > 0 && s.binding > minEnergy)
                edges.push_back(s.binding);
    std::sort(edges.begin(), edges.end(), std::greater<double>());
    return edges;
}

std::array<ShellConfig, 12> electron_configuration(const Composition& c)
{
    std::vector<ShellConfig> all;
    for (std::size_t i = 0; i < c.Z.size(); ++i) {
        const int Z = c.Z[i];
        for (const auto& s : element(Z).shells) {
            ShellConfig sc;
            sc.bindingEnergy = s.binding;
            sc.numberElectrons = c.numberFraction[i] * s.occupancy;
            sc.hartreeFockOrbital_0 = compton_profile_j0(Z, s.index);
            sc.fluorescenceYield = fluorescence_yield(Z, s.index);
            double e[3], r[3];
            fluorescence_lines(Z, s.index, e, r);
            const double rs = r[0] + r[1] + r[2];
            for (int k = 0; k < 3; ++k) {
                sc.fluorLineEnergies[k] = e[k];
                sc.fluorLineProbabilities[k] = rs > 0 ? r[k] / rs : 0.0;
            }
            // Relative photoionisation weight: number fraction x partial cross
            // section summed over 0.5 .. 399.5 keV in 1 keV steps.
            double w = 0;
            for (int k = 0; k < 400; ++k)
                w += photo_subshell_barn(Z, s.index, 0.5 + k);
            sc.photoIonizationProbability = c.numberFraction[i] * w;
            sc.Z = Z;
            sc.shell = s.index;
            all.push_back(sc);
        }
    }
    std::stable_sort(all.begin(), all.end(), [](const auto& a, const auto& b) { return a.bindingEnergy > b.bindingEnergy; });
    std::array<ShellConfig, 12> out {};
    for (auto& o : out) {
        o = ShellConfig {};
    }
    const std::size_t n = std::min<std::size_t>(all.size(), 12);
    for (std::size_t i = 0; i < n; ++i)
        out[i] = all[i];
    double esum = 0, psum = 0;
    for (std::size_t i = 0; i < n; ++i) {
        esum += out[i].numberElectrons;
        psum += out[i].photoIonizationProbability;
    }
    for (std::size_t i = 0; i < n; ++i) {
        if (esum > 0)
            out[i].numberElectrons /= esum;
        if (psum > 0)
            out[i].photoIonizationProbability /= psum;
    }
    return out;
}

} // namespace dxmc_gb300::physics
