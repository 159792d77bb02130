// ORACLE TEST INFRASTRUCTURE — CPU restatement of DXMClib's photon transport.
//
// Used only as the checker (tests/, __graft_entry__.smoke) and as the timed
// CPU baseline of bench.py.  It is validated against the reference itself
// through the golden fixtures (tests/test_oracle_port.py) and it travels to
// machines where the reference checkout does not exist.
//
// It follows DXMClib function by function with the reference's PCG32
// generator, in double or in float precision (Transport<double> and
// Transport<float>): the core (port_core.inc) is compiled once for each.
// Every function cites the reference lines it restates.  It consumes the same
// host LUT tables as the reference (attenuation coefficients, majorant, RITA,
// spline, shells), converted to the precision of the run.
#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <mutex>
#include <utility>
#include <numeric>
#include <thread>
#include <type_traits>
#include <vector>

// the precision-generic core, once per precision
namespace port64 {
using real = double;
#include "port_core.inc"
} // namespace port64
namespace port32 {
using real = float;
#include "port_core.inc"
} // namespace port32

namespace {

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
void oracle_port_set_direction(int normalized)
{
    port64::g_normalize_direction = normalized != 0;
    port32::g_normalize_direction = normalized != 0;
}

} // extern "C"

namespace {

template <class T>
std::vector<T> converted(const double* p, std::size_t n)
{
    return p ? std::vector<T>(p, p + n) : std::vector<T>();
}

// One transport run in the precision of the core namespace NS (real = T).  The
// tables, densities and exposures are converted to T before the timed region;
// the tallies are accumulated in T (as Result<T>) and widened afterwards.
template <class Job, class Lut, class T>
double run_port(const PortLut* lut, const PortWorld* w, const PortSource* s, int model, int n_threads,
    std::uint64_t seed, double* dose, double* variance, std::uint32_t* n_events, std::uint64_t* out_steps)
{
    const std::size_t nm = lut->n_materials, R = lut->n_energy;
    const std::size_t nv = w->dims[0] * w->dims[1] * w->dims[2];
    const auto x = converted<T>(lut->log_energy, R), coef = converted<T>(lut->coefficients, nm * R * 6),
               maxcoef = converted<T>(lut->max_coefficients, R * 2), rita = converted<T>(lut->rita, nm * 4 * 56),
               spline = converted<T>(lut->spline, nm * 79), shells = converted<T>(lut->shells, nm * 12 * 13);
    const auto dens = converted<T>(w->density, nv);
    const auto exposures = converted<T>(s->exposures, s->n_exposures * 19);
    const auto spec_e = converted<T>(s->spec_energies, s->spec_n > 0 ? s->spec_n : 0);
    const auto heel = converted<T>(s->heel_weights, s->heel_weights ? static_cast<std::size_t>(s->heel_ne) * s->heel_na : 0);
    std::vector<T> tally_d, tally_v;
    T* out_d;
    T* out_v;
    if constexpr (std::is_same_v<T, double>) {
        std::fill(dose, dose + nv, 0.0);
        std::fill(variance, variance + nv, 0.0);
        out_d = dose;
        out_v = variance;
    } else {
        tally_d.assign(nv, T(0));
        tally_v.assign(nv, T(0));
        out_d = tally_d.data();
        out_v = tally_v.data();
    }
    std::fill(n_events, n_events + nv, 0u);
    Job job;
    job.lut.nm = lut->n_materials;
    job.lut.R = lut->n_energy;
    job.lut.linear_index = static_cast<std::size_t>(lut->linear_index);
    job.lut.linear_step = lut->linear_step;
    job.lut.linear_energy = lut->linear_energy;
    job.lut.x = x.data();
    job.lut.coef = coef.data();
    job.lut.maxcoef = maxcoef.data();
    job.lut.rita = rita.data();
    job.lut.spline = spline.data();
    job.lut.shells = shells.data();
    job.density = dens.data();
    job.material = w->material;
    job.measurement = w->measurement;
    for (int i = 0; i < 3; ++i) {
        job.dims[i] = w->dims[i];
        job.spacing[i] = static_cast<T>(w->spacing[i]);
        // World<T>::updateMatrixExtent (world.hpp:55-68)
        const T half = (w->dims[i] * static_cast<T>(w->spacing[i])) * T(0.5);
        const T lower = static_cast<T>(w->origin[i]) - half, upper = static_cast<T>(w->origin[i]) + half;
        job.lo[i] = std::nextafter(lower, upper);
        job.hi[i] = std::nextafter(upper, lower);
    }
    job.model = model;
    job.exposures = exposures.data();
    job.n_exposures = s->n_exposures;
    job.spec_n = s->spec_n;
    job.spec_e = spec_e.data();
    if (s->spec_n > 0) {
        std::vector<double> probs;
        alias_table(s->spec_weights, s->spec_n, probs, job.spec_a);
        job.spec_p.assign(probs.begin(), probs.end());
    }
    job.heel_w = s->heel_weights ? heel.data() : nullptr;
    job.heel_ne = s->heel_ne;
    job.heel_na = s->heel_na;
    job.heel_e0 = static_cast<T>(s->heel_e0);
    job.heel_es = static_cast<T>(s->heel_es);
    job.heel_a0 = static_cast<T>(s->heel_a0);
    job.heel_as = static_cast<T>(s->heel_as);
    if (s->bowtie_n > 0) {
        for (int i = 0; i < s->bowtie_n; ++i)
            job.bowtie.emplace_back(static_cast<T>(std::abs(s->bowtie_angles[i])), static_cast<T>(s->bowtie_weights[i]));
        std::sort(job.bowtie.begin(), job.bowtie.end());
        T mean = 0;
        for (auto& b : job.bowtie)
            mean += b.second;
        mean /= job.bowtie.size();
        for (auto& b : job.bowtie)
            b.second /= mean;
    }
    job.dose = out_d;
    job.var = out_v;
    job.nev = n_events;
    const int nt = n_threads > 0 ? n_threads : std::max(1u, std::thread::hardware_concurrency());
    job.make_pool(job.n_exposures, static_cast<std::uint64_t>(nt));
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
    if constexpr (!std::is_same_v<T, double>) {
        for (std::size_t i = 0; i < nv; ++i) {
            dose[i] = static_cast<double>(tally_d[i]);
            variance[i] = static_cast<double>(tally_v[i]);
        }
    }
    return secs;
}

} // namespace

extern "C" {

// Runs the transport in double (precision 0) or float (precision 1) and writes
// energy imparted (keV) and its squared sum per voxel (raw tallies, the
// reference's Result before normalizeScoring).  Returns the wall time of the
// transport in seconds (tables converted beforehand); out_steps receives the
// Woodcock step count.
double oracle_port_transport_ex(const PortLut* lut, const PortWorld* w, const PortSource* s, int model, int n_threads,
    std::uint64_t seed, int precision, double* dose, double* variance, std::uint32_t* n_events, std::uint64_t* out_steps)
{
    if (precision == 1)
        return run_port<port32::Job, port32::Lut, float>(lut, w, s, model, n_threads, seed, dose, variance, n_events, out_steps);
    return run_port<port64::Job, port64::Lut, double>(lut, w, s, model, n_threads, seed, dose, variance, n_events, out_steps);
}

// The double-precision run (Transport<double>).
double oracle_port_transport(const PortLut* lut, const PortWorld* w, const PortSource* s, int model, int n_threads,
    std::uint64_t seed, double* dose, double* variance, std::uint32_t* n_events, std::uint64_t* out_steps)
{
    return oracle_port_transport_ex(lut, w, s, model, n_threads, seed, 0, dose, variance, n_events, out_steps);
}

} // extern "C"
