// X-ray tube spectra on the host: the thick-target semi-relativistic
// Bethe-Heitler model with tabulated electron fluence in tungsten
// (Poludniowski and Evans, Med. Phys. 34 (2007) 2164 and 2175), tungsten K
// lines and filtration, as DXMClib's Tube<T> computes them (tube.hpp:191-261,
// betheHeitlerCrossSection.hpp:326-407).  Spectrum generation stays on the host.
#pragma once

#include <vector>

namespace dxmc_gb300::host {

// Mass attenuation (cm2/g) callback of a filter material and its density (g/cm3).
struct SpectrumFilter {
    double (*total_attenuation)(const void* user, double energy_kev);
    const void* user;
    double density;
    double mm;
};

// Photon fluence per energy of a tube at `voltage` kV whose photons leave the
// anode at `takeoff_angle` (radians) from its surface, at the given energies
// (keV): bremsstrahlung, plus the tungsten K lines computed at
// `line_takeoff_angle` (DXMClib evaluates the lines at the tube's own anode
// angle, tube.hpp:220-241), attenuated by the filters and, with `normalize`,
// scaled to sum to one (tube.hpp:200-218).
std::vector<double> tube_spectrum(double voltage, double takeoff_angle, double line_takeoff_angle,
    const std::vector<double>& energies, const std::vector<SpectrumFilter>& filters, bool normalize);

// Bremsstrahlung leaving a tungsten anode per unit photon energy at hv (keV) for
// electrons of initial energy T0 (keV) (betheHeitlerSpectra,
// betheHeitlerCrossSection.hpp:367-390).
double thick_target_bremsstrahlung(double T0, double hv, double takeoff_angle);

} // namespace dxmc_gb300::host
