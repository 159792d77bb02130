// Project photon-interaction data model.
//
// DXMClib takes its cross sections, form factors, scatter functions and shell
// data from xraylib (src/material.cpp:31-377 calls CS_*_CP, FF_Rayl, SF_Compt,
// EdgeEnergy, ComptonProfile_Partial, FluorYield, RadRate, LineEnergy,
// CSb_Photo_Partial, CompoundParser).  xraylib is not part of this project, so
// the host side gets its physics data from the closed-form models below.  Every
// number is computed from a named textbook formula; no tabulated xraylib data
// is used.  Both the GPU path and the CPU oracle consume these same values, so
// transport parity is meaningful; absolute agreement with xraylib is not
// claimed.
//
//  * Shell structure: aufbau (Madelung) filling into relativistic subshells
//    (s1/2, p1/2, p3/2, d3/2, d5/2, f5/2, f7/2), ordered K, L1..L3, M1..M5, ...
//  * Binding energies: Slater's screening rules, E = Ry (Z_eff / n*)^2, with a
//    small s-penetration / spin-orbit split so subshell edges are distinct.
//  * Photoionisation: Kramers' semi-classical hydrogenic cross section per
//    electron, sigma = K0 Ry B^2 / (n* E^3) for E >= B.
//  * Atomic form factor: independent hydrogenic 1s-shaped shells,
//    f_s(x) = (1 + (2 pi x a_s)^2)^-2, a_s = n*^2 a0 / Z_eff.
//  * Incoherent scatter function: Waller-Hartree without exchange terms,
//    S(x) = sum_s N_s (1 - f_s(x)^2).
//  * Incoherent cross section: Klein-Nishina x S(x) integrated over angle.
//  * Coherent cross section: Thomson x F(x)^2 integrated over angle.
//  * Fluorescence yield: the Z^4 law omega = Z^4 / (a + Z^4).
//  * Compton profile at p_z = 0: hydrogenic J(0) = 8 n* / (3 pi Z_eff) (a.u.).
#pragma once

#include <array>
#include <cstdint>
#include <string>
#include <vector>

namespace dxmc_gb300::physics {

inline constexpr double RYDBERG_KEV = 0.013605693;     // keV
inline constexpr double BOHR_RADIUS_ANGSTROM = 0.529177; // angstrom
inline constexpr double ELECTRON_RADIUS_CM = 2.8179403e-13;
inline constexpr double AVOGADRO = 6.02214076e23;
inline constexpr double ELECTRON_MASS_KEV = 510.9989461;
inline constexpr double KEV_ANGSTROM = 12.398520; // hc in keV*angstrom
inline constexpr double FINE_STRUCTURE = 7.2973525693e-3;
inline constexpr int MAX_Z = 92;

struct Subshell {
    int index = 0;            // K=0, L1=1, L2=2, L3=3, M1=4, ... (spectroscopic order)
    int n = 0;                // principal quantum number
    int l = 0;                // orbital angular momentum
    double j = 0.5;           // total angular momentum
    double occupancy = 0;     // electrons in the subshell
    double nstar = 1;         // Slater effective principal quantum number
    double zeff = 1;          // Slater effective charge
    double binding = 0;       // keV
};

struct Element {
    int Z = 0;
    std::string symbol;
    double atomic_weight = 0; // g/mol
    double density = 0;       // g/cm3 at standard conditions
    std::vector<Subshell> shells;
};

const Element& element(int Z);
int atomic_number_from_symbol(const std::string& symbol);

// Per-atom cross sections in barn (1e-24 cm2); energy in keV.
double photo_subshell_barn(int Z, int shellIndex, double energy);
double photo_barn(int Z, double energy);
double incoherent_barn(int Z, double energy);
double coherent_barn(int Z, double energy);
double energy_transfer_fraction(int Z, double energy); // Compton energy-transfer fraction

// Momentum transfer x = sin(theta/2) / lambda in 1/angstrom.
double form_factor(int Z, double x);
double incoherent_sf(int Z, double x);

// Per-shell atomic data.
double compton_profile_j0(int Z, int shellIndex);
double fluorescence_yield(int Z, int shellIndex);
// Up to three emission lines for a vacancy in shellIndex: energies (keV) and
// relative rates (not normalised). Returns the number of lines found.
int fluorescence_lines(int Z, int shellIndex, double energies[3], double rates[3]);

struct Composition {
    std::vector<int> Z;
    std::vector<double> massFraction;   // normalised to 1
    std::vector<double> numberFraction; // normalised to 1
};

// Chemical formula such as "H2O", "N0.76O0.23Ar0.01", "Ca5(PO4)3OH".
bool parse_formula(const std::string& formula, Composition& out);
// Named reference materials (project-defined compositions).
bool named_material(const std::string& name, Composition& out, double& density);
std::vector<std::string> named_material_list();

// Material-level quantities (mixture rule over numberFraction / massFraction).
double mass_attenuation_photo(const Composition& c, double energy);    // cm2/g
double mass_attenuation_compton(const Composition& c, double energy);  // cm2/g
double mass_attenuation_rayleigh(const Composition& c, double energy); // cm2/g
double mass_energy_absorption(const Composition& c, double energy);    // cm2/g
double form_factor_squared(const Composition& c, double x);
double normalized_scatter_factor(const Composition& c, double x);
std::vector<double> binding_energies(const Composition& c, double minEnergy); // sorted descending

struct ShellConfig {
    double bindingEnergy = 0;
    double numberElectrons = 0;
    double hartreeFockOrbital_0 = 0;
    double photoIonizationProbability = 1;
    double fluorescenceYield = 0;
    std::array<double, 3> fluorLineProbabilities = { 1, 1, 1 };
    std::array<double, 3> fluorLineEnergies = { 0, 0, 0 };
    int Z = 0;
    int shell = 0;
};
std::array<ShellConfig, 12> electron_configuration(const Composition& c);

} // namespace dxmc_gb300::physics
