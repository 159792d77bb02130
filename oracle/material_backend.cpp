// ORACLE TEST INFRASTRUCTURE — not part of the product.
//
// Definitions of the dxmc::Material members that DXMClib declares in
// include/dxmc/material.hpp:60-139 and implements on top of xraylib in
// src/material.cpp:31-377.  xraylib is not available, so this file answers the
// same calls from the project physics model (dxmclib_gb300/csrc/physics),
// which lets the reference headers compile and link unmodified.  Each member
// follows the meaning of the xraylib-backed original:
//   material.cpp:31-34   getPhotoelectricAttenuation  -> cm2/g
//   material.cpp:36-39   getRayleightAttenuation      -> cm2/g
//   material.cpp:41-44   getComptonAttenuation        -> cm2/g
//   material.cpp:46-54   getTotalAttenuation (material / element)
//   material.cpp:56-59   getMassEnergyAbsorbtion
//   material.cpp:133-141 getRayleightFormFactorSquared: sum_i n_i F_i(q)^2
//   material.cpp:274-283 getComptonNormalizedScatterFactor: sum_i n_i S_i(q)/Z_i
//   material.cpp:143-273 getElectronConfiguration: 12 shells sorted by binding energy
//   material.cpp:285-322 getBindingEnergies: edges above minValue, descending
//   material.cpp:324-377 name / compound / atomic-number constructors
#include "dxmc/material.hpp"

#include "../dxmclib_gb300/csrc/physics/physics_model.hpp"

#include <numeric>

namespace phys = dxmc_gb300::physics;

namespace dxmc {

namespace {
    phys::Composition composition_of(const std::vector<int>& Z, const std::vector<double>& numberFraction)
    {
        phys::Composition c;
        c.Z = Z;
        c.numberFraction = numberFraction;
        c.massFraction.resize(Z.size());
        double s = 0;
        for (std::size_t i = 0; i < Z.size(); ++i) {
            c.massFraction[i] = numberFraction[i] * phys::element(Z[i]).atomic_weight;
            s += c.massFraction[i];
        }
        for (auto& m : c.massFraction)
            m /= s;
        return c;
    }
}

#define DXMC_ORACLE_COMPOSITION composition_of(m_elements, m_elementNumberFraction)

double Material::getPhotoelectricAttenuation(double energy) const
{
    return phys::mass_attenuation_photo(DXMC_ORACLE_COMPOSITION, energy);
}

double Material::getRayleightAttenuation(double energy) const
{
    return phys::mass_attenuation_rayleigh(DXMC_ORACLE_COMPOSITION, energy);
}

double Material::getComptonAttenuation(double energy) const
{
    return phys::mass_attenuation_compton(DXMC_ORACLE_COMPOSITION, energy);
}

double Material::getTotalAttenuation(double energy) const
{
    const auto c = DXMC_ORACLE_COMPOSITION;
    return phys::mass_attenuation_photo(c, energy) + phys::mass_attenuation_compton(c, energy) + phys::mass_attenuation_rayleigh(c, energy);
}

double Material::getTotalAttenuation(int atomicNumber, double energy)
{
    phys::Composition c;
    c.Z = { atomicNumber };
    c.massFraction = { 1.0 };
    c.numberFraction = { 1.0 };
    return phys::mass_attenuation_photo(c, energy) + phys::mass_attenuation_compton(c, energy) + phys::mass_attenuation_rayleigh(c, energy);
}

double Material::getMassEnergyAbsorbtion(double energy) const
{
    return phys::mass_energy_absorption(DXMC_ORACLE_COMPOSITION, energy);
}

double Material::getAtomicWeight(int Z)
{
    return phys::element(Z).atomic_weight;
}

std::string Material::getAtomicNumberToSymbol(int Z)
{
    return phys::element(Z).symbol;
}

Material::Material(int atomicNumber)
{
    setByAtomicNumber(atomicNumber);
}

const std::string& Material::prettyName(void) const
{
    if (m_prettyName.empty())
        return m_name;
    return m_prettyName;
}

Material::Material(const std::string& nameOrCompound, const std::string& prettyName, const double density)
{
    setByMaterialName(nameOrCompound);
    if (!m_valid)
        setByCompoundName(nameOrCompound);
    m_prettyName = prettyName.size() > 0 ? prettyName : m_name;
    if (density > 0)
        setStandardDensity(density);
}

void Material::setStandardDensity(double density)
{
    if (density > 0.0) {
        m_density = density;
        m_hasDensity = true;
    }
}

std::vector<std::string> Material::getNISTCompoundNames(void)
{
    return phys::named_material_list();
}

int Material::getAtomicNumberFromSymbol(const std::string& symbol)
{
    return phys::atomic_number_from_symbol(symbol);
}

std::string Material::getSymbolFromAtomicNumber(int Z)
{
    return phys::element(Z).symbol;
}

double Material::getRayleightFormFactorSquared(const double momentumTransfer) const
{
    return phys::form_factor_squared(DXMC_ORACLE_COMPOSITION, momentumTransfer);
}

double Material::getComptonNormalizedScatterFactor(const double momentumTransfer) const
{
    return phys::normalized_scatter_factor(DXMC_ORACLE_COMPOSITION, momentumTransfer);
}

std::array<ElectronShellConfiguration<double>, 12> Material::getElectronConfiguration() const
{
    const auto src = phys::electron_configuration(DXMC_ORACLE_COMPOSITION);
    std::array<ElectronShellConfiguration<double>, 12> out;
    for (std::size_t i = 0; i < 12; ++i) {
        out[i].bindingEnergy = src[i].bindingEnergy;
        out[i].numberElectrons = src[i].numberElectrons;
        out[i].hartreeFockOrbital_0 = src[i].hartreeFockOrbital_0;
        out[i].photoIonizationProbability = src[i].photoIonizationProbability;
        out[i].fluorescenceYield = src[i].fluorescenceYield;
        out[i].fluorLineProbabilities = src[i].fluorLineProbabilities;
        out[i].fluorLineEnergies = src[i].fluorLineEnergies;
        out[i].Z = src[i].Z;
        out[i].shell = src[i].shell;
    }
    return out;
}

std::vector<double> Material::getBindingEnergies(const double minValue) const
{
    return phys::binding_energies(DXMC_ORACLE_COMPOSITION, minValue);
}

void Material::setByAtomicNumber(int atomicNumber)
{
    if (atomicNumber < 1 || atomicNumber > phys::MAX_Z)
        return;
    const auto& e = phys::element(atomicNumber);
    m_name = e.symbol;
    m_density = e.density;
    m_hasDensity = true;
    m_valid = true;
    m_elements = { atomicNumber };
    m_elementNumberFraction = { 1.0 };
}

void Material::setByCompoundName(const std::string& name)
{
    phys::Composition c;
    if (phys::parse_formula(name, c)) {
        m_name = name;
        m_valid = true;
        m_hasDensity = false;
        m_elements = c.Z;
        m_elementNumberFraction = c.numberFraction;
    }
}

void Material::setByMaterialName(const std::string& name)
{
    phys::Composition c;
    double density = 0;
    if (phys::named_material(name, c, density)) {
        m_name = name;
        m_valid = true;
        m_hasDensity = true;
        m_density = density;
        m_elements = c.Z;
        m_elementNumberFraction = c.numberFraction;
    }
}

} // namespace dxmc
