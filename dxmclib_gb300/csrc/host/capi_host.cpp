// Host-only entry points of the C ABI (no CUDA calls): project physics
// materials, LUT build and introspection, spectrum alias tables.
#include "dxmc_gpu.h"

#include "../physics/physics_model.hpp"
#include "lut_builder.hpp"
#include "../kernels/stream_seed.hpp"
#include "tube_spectrum.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace phys = dxmc_gb300::physics;
namespace host = dxmc_gb300::host;

namespace {

struct PhysicsMaterial {
    phys::Composition composition;
};

PhysicsMaterial* pm(void* u) { return static_cast<PhysicsMaterial*>(u); }

// A C++ exception must not cross the C ABI: called from the catch clause of the
// entry points that build host tables, host memory exhaustion becomes
// DXMC_ERR_OOM and anything else DXMC_ERR_INVALID.
int exception_status() noexcept
{
    try {
        throw;
    } catch (const std::bad_alloc&) {
        return DXMC_ERR_OOM;
    } catch (const std::length_error&) {
        return DXMC_ERR_OOM;
    } catch (...) {
        return DXMC_ERR_INVALID;
    }
}

double cb_photo(void* u, double e) { return phys::mass_attenuation_photo(pm(u)->composition, e); }
double cb_compton(void* u, double e) { return phys::mass_attenuation_compton(pm(u)->composition, e); }
double cb_rayleigh(void* u, double e) { return phys::mass_attenuation_rayleigh(pm(u)->composition, e); }
double cb_ff2(void* u, double q) { return phys::form_factor_squared(pm(u)->composition, q); }
double cb_sf(void* u, double q) { return phys::normalized_scatter_factor(pm(u)->composition, q); }
int cb_edges(void* u, double minE, double* out, int cap)
{
    const auto e = phys::binding_energies(pm(u)->composition, minE);
    const int n = static_cast<int>(e.size());
    for (int i = 0; i < std::min(n, cap); ++i)
        out[i] = e[i];
    return n;
}
void cb_shells(void* u, dxmc_shell_config out[12])
{
    const auto s = phys::electron_configuration(pm(u)->composition);
    for (int i = 0; i < 12; ++i) {
        out[i].binding_energy = s[i].bindingEnergy;
        out[i].number_electrons = s[i].numberElectrons;
        out[i].hartree_fock_j0 = s[i].hartreeFockOrbital_0;
        out[i].photo_ionization_probability = s[i].photoIonizationProbability;
        out[i].fluorescence_yield = s[i].fluorescenceYield;
        for (int k = 0; k < 3; ++k) {
            out[i].line_probabilities[k] = s[i].fluorLineProbabilities[k];
            out[i].line_energies[k] = s[i].fluorLineEnergies[k];
        }
        out[i].Z = s[i].Z;
        out[i].shell = s[i].shell;
    }
}

void fill_provider(PhysicsMaterial* m, double density, dxmc_material_provider* out)
{
    out->user = m;
    out->standard_density = density;
    out->photoelectric = cb_photo;
    out->compton = cb_compton;
    out->rayleigh = cb_rayleigh;
    out->form_factor_squared = cb_ff2;
    out->scatter_factor = cb_sf;
    out->binding_energies = cb_edges;
    out->shells = cb_shells;
}

bool provider_ok(const dxmc_material_provider& p)
{
    return p.photoelectric && p.compton && p.rayleigh && p.form_factor_squared && p.scatter_factor && p.binding_energies && p.shells;
}

} // namespace

extern "C" {

int dxmc_gpu_abi_version(void) { return DXMC_GPU_ABI_VERSION; }

int dxmc_physics_material(const char* name, double density, dxmc_material_provider* out)
try {
    if (!name || !out)
        return DXMC_ERR_INVALID;
    phys::Composition c;
    double standard = -1;
    const std::string n(name);
    if (!phys::named_material(n, c, standard)) {
        if (!phys::parse_formula(n, c))
            return DXMC_ERR_INVALID;
        if (c.Z.size() == 1)
            standard = phys::element(c.Z[0]).density;
    }
    const double d = density > 0 ? density : standard;
    if (!(d > 0))
        return DXMC_ERR_INVALID; // like Material::isValid without a density (material.hpp:64)
    auto* m = new (std::nothrow) PhysicsMaterial { c };
    if (!m)
        return DXMC_ERR_OOM;
    fill_provider(m, d, out);
    return DXMC_OK;
} catch (...) {
    return exception_status();
}

int dxmc_physics_element_material(int Z, dxmc_material_provider* out)
try {
    if (Z < 1 || Z > phys::MAX_Z || !out)
        return DXMC_ERR_INVALID;
    return dxmc_physics_material(phys::element(Z).symbol.c_str(), -1, out);
} catch (...) {
    return exception_status();
}

int dxmc_physics_mass_energy_absorption(const dxmc_material_provider* provider, double energy, double* out)
try {
    // only providers made by dxmc_physics_material carry a composition
    if (!provider || !out || !provider->user || provider->photoelectric != cb_photo || !(energy > 0))
        return DXMC_ERR_INVALID;
    *out = phys::mass_energy_absorption(pm(provider->user)->composition, energy);
    return DXMC_OK;
} catch (...) {
    return exception_status();
}

void dxmc_physics_material_free(dxmc_material_provider* provider)
{
    if (provider && provider->user) {
        delete pm(provider->user);
        provider->user = nullptr;
    }
}

int dxmc_lut_build_max_density(const dxmc_material_provider* materials, int n_materials,
    const double* max_density, double max_energy, dxmc_lut_blob** out)
try {
    if (!materials || n_materials <= 0 || n_materials > 255 || !max_density || !out)
        return DXMC_ERR_INVALID;
    std::vector<host::MaterialData> mats;
    for (int i = 0; i < n_materials; ++i) {
        if (!provider_ok(materials[i]))
            return DXMC_ERR_INVALID;
        mats.push_back(host::MaterialData { &materials[i] });
    }
    auto* blob = new (std::nothrow) dxmc_lut_blob;
    if (!blob)
        return DXMC_ERR_OOM;
    const std::vector<double> md(max_density, max_density + n_materials);
    const int rc = host::build_lut(mats, md, max_energy, *blob);
    if (rc != DXMC_OK) {
        delete blob;
        return rc;
    }
    *out = blob;
    return DXMC_OK;
} catch (...) {
    return exception_status();
}

int dxmc_lut_build(const dxmc_material_provider* materials, int n_materials,
    const float* density, const uint8_t* material, uint64_t n_voxels,
    double max_energy, dxmc_lut_blob** out)
try {
    if (!density || !material || n_voxels == 0 || n_materials <= 0 || n_materials > 255)
        return DXMC_ERR_INVALID;
    std::vector<double> md(n_materials, 0.0);
    for (uint64_t i = 0; i < n_voxels; ++i) {
        const int m = material[i];
        if (m < n_materials)
            md[m] = std::max(md[m], static_cast<double>(density[i]));
    }
    return dxmc_lut_build_max_density(materials, n_materials, md.data(), max_energy, out);
} catch (...) {
    return exception_status();
}

void dxmc_lut_blob_free(dxmc_lut_blob* blob) { delete blob; }

int dxmc_lut_attenuation(const dxmc_lut_blob* blob, int material, double energy, double out[3])
{
    if (!blob || material < 0 || material >= blob->n_materials || !out)
        return DXMC_ERR_INVALID;
    const auto a = host::lut_attenuation(*blob, material, energy);
    out[0] = a[0];
    out[1] = a[1];
    out[2] = a[2];
    return DXMC_OK;
}

double dxmc_lut_max_attenuation_inverse(const dxmc_lut_blob* blob, double energy)
{
    return blob ? host::lut_max_inverse(*blob, energy) : 0.0;
}

double dxmc_lut_scatter_factor(const dxmc_lut_blob* blob, int material, double q)
{
    if (!blob || material < 0 || material >= blob->n_materials)
        return 0.0;
    return host::lut_scatter_factor(*blob, material, q);
}

int dxmc_lut_get_info(const dxmc_lut_blob* blob, dxmc_lut_info* info)
{
    if (!blob || !info)
        return DXMC_ERR_INVALID;
    std::memset(info, 0, sizeof(*info));
    info->n_materials = blob->n_materials;
    info->n_energy = static_cast<int32_t>(blob->resolution());
    info->linear_index = static_cast<int32_t>(blob->linear_index);
    info->linear_step = blob->linear_step;
    info->linear_energy = blob->linear_energy;
    info->min_energy = blob->min_energy;
    info->max_energy = blob->max_energy;
    info->log_energy = blob->log_energy.data();
    info->coefficients = blob->coefficients.data();
    info->max_coefficients = blob->max_coefficients.data();
    info->rita = blob->rita.empty() ? nullptr : blob->rita[0].data();
    info->spline = blob->spline.empty() ? nullptr : blob->spline[0].data();
    info->shells = blob->shells.empty() ? nullptr : blob->shells[0].data();
    return DXMC_OK;
}

int dxmc_bowtie_table(const double* angles, const double* weights, int n, double* table_angles, double* table_weights)
try {
    if (n <= 0 || n > DXMC_MAX_BOWTIE_POINTS || !angles || !weights || !table_angles || !table_weights)
        return DXMC_ERR_INVALID;
    std::vector<std::pair<double, double>> data(static_cast<size_t>(n));
    for (int i = 0; i < n; ++i)
        data[i] = { std::abs(angles[i]), weights[i] };
    std::sort(data.begin(), data.end());
    double sum = 0.0; // in table order, from zero: the normalisation's sum
    for (const auto& p : data)
        sum += p.second;
    const double mean = sum / n;
    if (!(mean > 0.0) || !std::isfinite(mean))
        return DXMC_ERR_INVALID;
    for (int i = 0; i < n; ++i) {
        table_angles[i] = data[i].first;
        table_weights[i] = data[i].second / mean;
    }
    return DXMC_OK;
} catch (...) {
    return exception_status();
}

int dxmc_udiv_invariant(const uint32_t* n, uint64_t count, uint32_t d, uint32_t* out)
{
    if (!n || !out || d == 0)
        return DXMC_ERR_INVALID;
    const auto q = dxmc_gb300::udiv_magic(d);
    for (uint64_t i = 0; i < count; ++i)
        out[i] = dxmc_gb300::udiv_apply(n[i], q.m, q.shifts);
    return DXMC_OK;
}

namespace {
double provider_total_attenuation(const void* user, double e)
{
    const auto* p = static_cast<const dxmc_material_provider*>(user);
    return p->photoelectric(p->user, e) + p->compton(p->user, e) + p->rayleigh(p->user, e);
}
} // namespace

int dxmc_tube_spectrum(double voltage, double takeoff_angle, double line_takeoff_angle, const double* energies, int n_energies,
    const dxmc_material_provider* filters, const double* filter_mm, int n_filters, int normalize, double* out)
try {
    if (!energies || !out || n_energies <= 0 || !(voltage > 0) || n_filters < 0 || (n_filters > 0 && (!filters || !filter_mm)))
        return DXMC_ERR_INVALID;
    std::vector<dxmc_gb300::host::SpectrumFilter> f;
    for (int i = 0; i < n_filters; ++i) {
        if (!provider_ok(filters[i]) || !(filters[i].standard_density > 0))
            return DXMC_ERR_INVALID;
        f.push_back({ provider_total_attenuation, &filters[i], filters[i].standard_density, std::abs(filter_mm[i]) });
    }
    const std::vector<double> e(energies, energies + n_energies);
    const auto s = dxmc_gb300::host::tube_spectrum(voltage, takeoff_angle, line_takeoff_angle, e, f, normalize != 0);
    std::copy(s.begin(), s.end(), out);
    return DXMC_OK;
} catch (...) {
    return exception_status();
}

int dxmc_stream_seed(uint64_t seed, uint64_t history, uint32_t out[4])
{
    if (!out)
        return DXMC_ERR_INVALID;
    dxmc_gb300::stream_seed(seed, history, out);
    return DXMC_OK;
}

int dxmc_alias_table(const double* weights, int n, double* probs, uint64_t* alias)
try {
    if (!weights || n <= 0 || !probs || !alias)
        return DXMC_ERR_INVALID;
    std::vector<double> w(weights, weights + n), p;
    std::vector<std::uint64_t> a;
    host::build_alias_table(w, p, a);
    for (int i = 0; i < n; ++i) {
        probs[i] = p[i];
        alias[i] = a[i];
    }
    return DXMC_OK;
} catch (...) {
    return exception_status();
}

} // extern "C"
