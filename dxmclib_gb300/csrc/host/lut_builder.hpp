// Host-side attenuation LUT build (DXMClib keeps this on the host too).
//
// Restates, in the project's own code, the table generation of
//   AttenuationLut<T>::generate            attenuationlut.hpp:64-96
//   AttenuationLutInterpolator<T>::generate attenuationinterpolator.hpp:119-205
//   generateMaxAttenuationLut              attenuationinterpolator.hpp:48-84
//   generateFFdata / RITA<T,56>            attenuationlut.hpp:212-233, dxmcrandom.hpp:384-468
//   generateSFdata / CubicSpline<T,16>     attenuationlut.hpp:240-265, interpolation.hpp:127-167
// in double precision, with the same node placement, segment indexing and
// quirks (the uniform fast path reads the segment one to the left of the one
// that contains the energy; the last split of the RITA table keeps stale
// rational coefficients), so the tables agree entry by entry with the
// reference's AttenuationLut<double> given the same material data.
#pragma once

#include "dxmc_gpu.h"

#include <array>
#include <cstdint>
#include <functional>
#include <memory>
#include <mutex>
#include <vector>

struct dxmc_lut_blob {
    int n_materials = 0;
    double min_energy = 1;  // AttenuationLut m_minEnergy
    double max_energy = 150; // AttenuationLut m_maxEnergy
    // interpolator
    std::vector<double> log_energy;   // m_x after the first node is dropped (R entries)
    std::vector<double> coefficients; // [material][segment][type][b, a], R segments
    std::vector<double> max_coefficients; // [segment][b, a]
    std::size_t linear_index = 0;
    double linear_step = 0;
    double linear_energy = 0;
    // form factor RITA tables, per material: x, e, a, b (56 each)
    std::vector<std::array<double, 4 * 56>> rita;
    // Compton scatter factor splines: 60 coefficients, 16 knots, start, step, stop
    std::vector<std::array<double, 79>> spline;
    std::vector<std::array<dxmc_shell_config, 12>> shells;
    std::vector<double> max_density;
    // inverse-CDF sampling tables and the local-majorant ratio bounds, built on
    // first upload and kept with the blob (both under tables_mutex)
    std::shared_ptr<std::mutex> tables_mutex = std::make_shared<std::mutex>();
    mutable std::shared_ptr<const void> tables;
    mutable std::shared_ptr<const void> majorant;

    std::size_t resolution() const { return log_energy.size(); }
};

namespace dxmc_gb300::host {

constexpr int RITA_N = 56;
constexpr int SPLINE_N = 16;
constexpr double KEV_TO_ANGSTROM = 12.398520;
constexpr double ELECTRON_REST_MASS = 510.9989461;

struct MaterialData {
    const dxmc_material_provider* p;
    double photo(double e) const { return p->photoelectric(p->user, e); }
    double compton(double e) const { return p->compton(p->user, e); }
    double rayleigh(double e) const { return p->rayleigh(p->user, e); }
    double ff2(double q) const { return p->form_factor_squared(p->user, q); }
    double sf(double q) const { return p->scatter_factor(p->user, q); }
    std::vector<double> edges(double minEnergy) const;
    std::array<dxmc_shell_config, 12> shells() const;
};

// Builds the full blob; max_density[i] is the largest density of material i in the world.
int build_lut(const std::vector<MaterialData>& materials, const std::vector<double>& max_density,
    double max_energy, dxmc_lut_blob& out);

// Table lookups in double precision following attenuationinterpolator.hpp:207-248
// and interpolation.hpp:169-176.
std::array<double, 3> lut_attenuation(const dxmc_lut_blob& b, int material, double energy);
double lut_max_inverse(const dxmc_lut_blob& b, double energy);
double lut_scatter_factor(const dxmc_lut_blob& b, int material, double q);

// RITA adaptive rational inverse-transform table (Salvat et al., PENELOPE) as
// laid out in dxmcrandom.hpp:384-468: outputs x, e, a, b (N each).
void build_rita(double min, double max, const std::function<double(double)>& pdf, int N, double* x, double* e, double* a, double* b);

// Natural cubic spline on N knots spaced (stop-start)/(N-2), interpolation.hpp:127-167.
void build_spline(double start, double stop, const std::function<double(double)>& f, int N, double* coef, double* knots, double& step, double& stop_out);

// Inverse-CDF tables for divergence-free interaction sampling on the GPU.  For
// ne log-spaced energies between the LUT's minimum and maximum energy, each row
// holds nu + 1 quantiles (levels k / nu) of the density the reference's rejection
// samplers draw from:
//   compton_kn[E]      Compton energy fraction e in [e_min, 1], density
//                      (1/e + e - sin^2) (transport.hpp:300-340, NONE model),
//                      stored as (e - e_min) / (1 - e_min);
//   compton_sf[m][E]   the same times the scatter factor S(q) (LIVERMORE model);
//   rayleigh[m][E]     momentum transfer q^2 from the RITA form-factor table
//                      truncated at q_max^2, times (1 + cos^2) / 2
//                      (transport.hpp:264-298), stored as q^2 / q_max^2.
struct SamplingTables {
    int ne = 0, nu = 0;
    double le0 = 0, dle = 0; // natural log of the first energy, log step
    std::vector<float> compton_kn, compton_sf, rayleigh;
};
void build_sampling_tables(const dxmc_lut_blob& b, int ne, int nu, SamplingTables& out);
// The blob's tables for (ne, nu), built once and shared by every upload of the blob.
std::shared_ptr<const SamplingTables> sampling_tables(const dxmc_lut_blob& b, int ne, int nu);
// RITA inverse transform of xi in [0, 1] for material m (dxmcrandom.hpp:483-500).
double rita_value(const dxmc_lut_blob& b, int material, double xi);

// Alias table by the squaring-the-histogram method, dxmcrandom.hpp:229-274.
void build_alias_table(const std::vector<double>& weights, std::vector<double>& probs, std::vector<std::uint64_t>& alias);

} // namespace dxmc_gb300::host
