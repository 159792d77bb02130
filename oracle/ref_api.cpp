// ORACLE TEST INFRASTRUCTURE — not part of the product.
//
// A C entry layer around the UNMODIFIED DXMClib headers (compiled from the
// reference checkout by oracle/Makefile, never copied) so that the golden
// fixture generator (tests/golden/make_golden.py) can drive the reference's
// own code through ctypes.  It exposes:
//   * ref_lut_dump         AttenuationLut<double>::generate(world, maxE)
//                          (attenuationlut.hpp:64-96) and its public lookups
//                          (attenuationlut.hpp:105-204), plus the internal
//                          tables read through the standard explicit-
//                          instantiation member-pointer technique, so the
//                          project's own LUT builder can be compared entry
//                          by entry;
//   * ref_source_tables    Source::getExposure(i) + alignToDirectionCosines
//                          (source.hpp, exposure.hpp:268-278), the spectrum
//                          alias table (dxmcrandom.hpp:229-274) and the heel
//                          table (beamfilters.hpp:455-505);
//   * ref_transport        Transport<double>::operator() (transport.hpp:135-202)
//                          in EV_PER_HISTORY mode;
//   * ref_interactions     the protected interaction samplers of Transport
//                          (transport.hpp:216-483) driven through a subclass;
//   * ref_bowtie           BowTieFilter<double> (beamfilters.hpp:65-197): its
//                          normalised table and sampleIntensityWeight.

#include "std_reduce_shim.hpp" // before the reference headers: BowTieFilter compiles with GCC 13

#include "dxmc/attenuationlut.hpp"
#include "dxmc/source.hpp"
#include "dxmc/transport.hpp"
#include "dxmc/world.hpp"

#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <thread>
#include <vector>

using namespace dxmc;

// ---- read access to private members (member-pointer explicit instantiation) --
template <typename Tag, typename Tag::type M>
struct PrivateMember {
    friend typename Tag::type member(Tag) { return M; }
};

using Rita56 = RITA<double, 56>;
using Spline16 = CubicSplineInterpolator<double, 16>;
using Interp = AttenuationLutInterpolator<double>;
using Lut = AttenuationLut<double>;
using Arr56 = std::array<double, 56>;
using Arr60 = std::array<double, 60>;
using Arr16 = std::array<double, 16>;
using VecD = std::vector<double>;
using VecRita = std::vector<Rita56>;
using VecSpline = std::vector<Spline16>;
using Heel = HeelFilter<double>;

#define DXMC_ORACLE_PRIVATE(TagName, Class, Type, Member) \
    struct TagName {                                      \
        using type = Type Class::*;                       \
        friend type member(TagName);                      \
    };                                                    \
    template struct PrivateMember<TagName, &Class::Member>

DXMC_ORACLE_PRIVATE(RitaX, Rita56, Arr56, m_x);
DXMC_ORACLE_PRIVATE(RitaE, Rita56, Arr56, m_e);
DXMC_ORACLE_PRIVATE(RitaA, Rita56, Arr56, m_a);
DXMC_ORACLE_PRIVATE(RitaB, Rita56, Arr56, m_b);
DXMC_ORACLE_PRIVATE(SplineCoef, Spline16, Arr60, m_coefficients);
DXMC_ORACLE_PRIVATE(SplineX, Spline16, Arr16, m_x);
DXMC_ORACLE_PRIVATE(SplineStep, Spline16, double, m_step);
DXMC_ORACLE_PRIVATE(SplineStart, Spline16, double, m_start);
DXMC_ORACLE_PRIVATE(SplineStop, Spline16, double, m_stop);
DXMC_ORACLE_PRIVATE(InterpX, Interp, VecD, m_x);
DXMC_ORACLE_PRIVATE(InterpCoef, Interp, VecD, m_coefficients);
DXMC_ORACLE_PRIVATE(InterpMaxCoef, Interp, VecD, m_maxCoefficients);
DXMC_ORACLE_PRIVATE(InterpResolution, Interp, std::size_t, m_resolution);
DXMC_ORACLE_PRIVATE(InterpLinearIndex, Interp, std::size_t, m_linearIndex);
DXMC_ORACLE_PRIVATE(InterpLinearStep, Interp, double, m_linearStep);
DXMC_ORACLE_PRIVATE(InterpLinearEnergy, Interp, double, m_linearEnergy);
DXMC_ORACLE_PRIVATE(LutFF, Lut, VecRita, m_formFactor);
DXMC_ORACLE_PRIVATE(LutSF, Lut, VecSpline, m_comptonScatterFactor);
DXMC_ORACLE_PRIVATE(LutData, Lut, Interp, m_attenuationData);
DXMC_ORACLE_PRIVATE(LutMinE, Lut, double, m_minEnergy);
DXMC_ORACLE_PRIVATE(LutMaxE, Lut, double, m_maxEnergy);
DXMC_ORACLE_PRIVATE(HeelAngleStart, Heel, double, m_angleStart);
using Expo = Exposure<double>;
using SpecPtr = const SpecterDistribution<double>*;
using HeelPtr = const HeelFilter<double>*;
DXMC_ORACLE_PRIVATE(ExpoSpecter, Expo, SpecPtr, m_specterDistribution);
DXMC_ORACLE_PRIVATE(ExpoHeel, Expo, HeelPtr, m_heelFilter);
DXMC_ORACLE_PRIVATE(HeelAngleStep, Heel, double, m_angleStep);
DXMC_ORACLE_PRIVATE(HeelEnergyStart, Heel, double, m_energyStart);
DXMC_ORACLE_PRIVATE(HeelEnergyStep, Heel, double, m_energyStep);

extern "C" {

struct RefWorldDesc {
    std::uint64_t dims[3];
    double spacing[3]; // mm
    double origin[3];
    double direction_cosines[6];
    const double* density;
    const std::uint8_t* material;
    const std::uint8_t* measurement; // may be null
    int n_materials;
    const char* const* material_names;
    const double* material_densities; // <= 0: standard density
};

// Source types
enum { REF_PENCIL = 0, REF_ISOTROPIC = 1, REF_DX = 2, REF_CTSPIRAL = 3, REF_CTAXIAL = 4, REF_CBCT = 5, REF_ISOTROPIC_CT = 6,
    REF_CT_CALIBRATION = 7, // the axial copy a CT spiral source calibrates with (source.hpp:925-950)
    REF_CTSPIRAL_DUAL = 8, REF_CTAXIAL_DUAL = 9, REF_CTTOPOGRAM = 10 };

struct RefSourceDesc {
    int type;
    int heel;
    double position[3];
    double direction_cosines[6];
    std::uint64_t histories_per_exposure;
    std::uint64_t total_exposures;
    // pencil
    double energy;
    // isotropic
    double collimation[4];
    const double* spec_energies;
    const double* spec_weights;
    int spec_n;
    // tube
    double kvp;
    double anode_angle_deg;
    double al_mm;
    double cu_mm;
    // DX / CBCT
    double field_size[2];
    double sdd;
    double source_angles_deg[2];
    double tube_rotation_deg;
    double span_deg;
    double step_deg;
    // CT
    double ct_collimation;
    double pitch;
    double scan_length;
    double angle_step_deg;
    double start_angle_deg;
    double fov;
    double tilt_deg;
    const double* bowtie_angles;
    const double* bowtie_weights;
    int bowtie_n;
    // CT axial step (<= 0: the collimation, the constructor's); dual sources: tube B
    // and the tube currents (set_b = 0 keeps the CTDualSource constructor's defaults)
    double axial_step;
    int set_b;
    double kvp_b;
    double al_mm_b;
    double cu_mm_b;
    double mas_a;
    double mas_b;
    double sdd_b;
    double fov_b;
    double start_angle_b_deg;
};

} // extern "C"

namespace {

std::vector<Material> make_materials(const RefWorldDesc& w)
{
    std::vector<Material> mats;
    for (int i = 0; i < w.n_materials; ++i) {
        Material m(w.material_names[i]);
        if (w.material_densities && w.material_densities[i] > 0)
            m.setStandardDensity(w.material_densities[i]);
        mats.push_back(m);
    }
    return mats;
}

template <class T>
bool make_world(const RefWorldDesc& d, World<T>& world)
{
    world.setDimensions({ d.dims[0], d.dims[1], d.dims[2] });
    world.setSpacing({ static_cast<T>(d.spacing[0]), static_cast<T>(d.spacing[1]), static_cast<T>(d.spacing[2]) });
    world.setOrigin({ static_cast<T>(d.origin[0]), static_cast<T>(d.origin[1]), static_cast<T>(d.origin[2]) });
    world.setDirectionCosines({ static_cast<T>(d.direction_cosines[0]), static_cast<T>(d.direction_cosines[1]), static_cast<T>(d.direction_cosines[2]), static_cast<T>(d.direction_cosines[3]), static_cast<T>(d.direction_cosines[4]), static_cast<T>(d.direction_cosines[5]) });
    const std::size_t n = d.dims[0] * d.dims[1] * d.dims[2];
    auto dens = std::make_shared<std::vector<T>>(d.density, d.density + n);
    auto mat = std::make_shared<std::vector<std::uint8_t>>(d.material, d.material + n);
    world.setDensityArray(dens);
    world.setMaterialIndexArray(mat);
    if (d.measurement)
        world.setMeasurementMapArray(std::make_shared<std::vector<std::uint8_t>>(d.measurement, d.measurement + n));
    for (const auto& m : make_materials(d))
        world.addMaterialToMap(m);
    world.makeValid();
    return world.isValid();
}

template <class T>
void setup_tube(Tube<T>& tube, const RefSourceDesc& s)
{
    tube.setVoltage(s.kvp);
    if (s.anode_angle_deg > 0)
        tube.setAnodeAngleDeg(s.anode_angle_deg);
    tube.setAlFiltration(s.al_mm);
    if (s.cu_mm > 0)
        tube.setCuFiltration(s.cu_mm);
}

template <class T>
std::unique_ptr<Source<T>> make_source(const RefSourceDesc& s)
{
    const std::array<T, 3> pos { static_cast<T>(s.position[0]), static_cast<T>(s.position[1]), static_cast<T>(s.position[2]) };
    std::array<T, 6> cos {};
    for (int k = 0; k < 6; ++k)
        cos[k] = static_cast<T>(s.direction_cosines[k]);
    switch (s.type) {
    case REF_PENCIL: {
        auto p = std::make_unique<PencilSource<T>>();
        p->setPosition(pos);
        p->setDirectionCosines(cos);
        p->setPhotonEnergy(s.energy);
        p->setHistoriesPerExposure(s.histories_per_exposure);
        p->setTotalExposures(s.total_exposures);
        return p;
    }
    case REF_ISOTROPIC:
    case REF_ISOTROPIC_CT: {
        std::unique_ptr<IsotropicSource<T>> p;
        if (s.type == REF_ISOTROPIC)
            p = std::make_unique<IsotropicSource<T>>();
        else
            p = std::make_unique<IsotropicCTSource<T>>();
        p->setPosition(pos);
        p->setDirectionCosines(cos);
        p->setCollimationAngles(s.collimation[0], s.collimation[1], s.collimation[2], s.collimation[3]);
        std::vector<T> e(s.spec_energies, s.spec_energies + s.spec_n);
        std::vector<T> w(s.spec_weights, s.spec_weights + s.spec_n);
        p->setSpecter(w, e);
        p->setHistoriesPerExposure(s.histories_per_exposure);
        p->setTotalExposures(s.total_exposures);
        return p;
    }
    case REF_DX: {
        auto p = std::make_unique<DXSource<T>>();
        setup_tube(p->tube(), s);
        p->setPosition(pos);
        p->setSourceDetectorDistance(s.sdd);
        p->setFieldSize({ s.field_size[0], s.field_size[1] });
        p->setTubeRotationDeg(s.tube_rotation_deg);
        p->setSourceAnglesDeg(s.source_angles_deg[0], s.source_angles_deg[1]);
        p->setModelHeelEffect(s.heel != 0);
        p->setHistoriesPerExposure(s.histories_per_exposure);
        p->setTotalExposures(s.total_exposures);
        return p;
    }
    case REF_CBCT: {
        auto p = std::make_unique<CBCTSource<T>>();
        setup_tube(p->tube(), s);
        p->setPosition(pos);
        p->setSourceDetectorDistance(s.sdd);
        p->setFieldSize({ s.field_size[0], s.field_size[1] });
        p->setSourceAnglesDeg(s.source_angles_deg[0], s.source_angles_deg[1]);
        p->setSpanAngleDeg(s.span_deg);
        p->setStepAngleDeg(s.step_deg);
        p->setModelHeelEffect(s.heel != 0);
        p->setHistoriesPerExposure(s.histories_per_exposure);
        return p;
    }
    case REF_CT_CALIBRATION: {
        // CTSpiralSource::getCalibrationValue copies the source into a CTAxialSource
        // (source.hpp:1358-1363, 1603-1608); ctCalibration then aligns it with the
        // phantom axis, centres it and scans one collimation (source.hpp:937-942)
        RefSourceDesc sp = s;
        sp.type = REF_CTSPIRAL;
        auto spiral = make_source<T>(sp);
        auto p = std::make_unique<CTAxialSource<T>>(*dynamic_cast<CTSpiralSource<T>*>(spiral.get()));
        p->setDirectionCosines(std::array<T, 6> { -1, 0, 0, 0, 0, 1 });
        p->setPosition(std::array<T, 3> { 0, 0, 0 });
        p->setScanLenght(p->collimation());
        p->setUseXCareFilter(false);
        p->setHistoriesPerExposure(s.histories_per_exposure);
        return p;
    }
    case REF_CTTOPOGRAM: {
        auto p = std::make_unique<CTTopogramSource<T>>();
        setup_tube(p->tube(), s);
        p->setPosition(pos);
        p->setSourceDetectorDistance(s.sdd);
        p->setCollimation(s.ct_collimation);
        p->setFieldOfView(s.fov);
        p->setGantryTiltAngleDeg(s.tilt_deg);
        p->setStartAngleDeg(s.start_angle_deg);
        p->setScanLenght(s.scan_length);
        p->setModelHeelEffect(s.heel != 0);
        p->setHistoriesPerExposure(s.histories_per_exposure);
        return p;
    }
    case REF_CTSPIRAL_DUAL:
    case REF_CTAXIAL_DUAL: {
        std::unique_ptr<CTDualSource<T>> p;
        if (s.type == REF_CTSPIRAL_DUAL) {
            auto sp = std::make_unique<CTSpiralDualSource<T>>();
            sp->setPitch(s.pitch);
            p = std::move(sp);
        } else {
            auto ax = std::make_unique<CTAxialDualSource<T>>();
            if (s.axial_step > 0)
                ax->setStep(s.axial_step);
            p = std::move(ax);
        }
        setup_tube(p->tube(), s);
        if (s.set_b) {
            Tube<T>& b = p->tubeB();
            b.setVoltage(s.kvp_b);
            if (s.anode_angle_deg > 0)
                b.setAnodeAngleDeg(s.anode_angle_deg);
            b.setAlFiltration(s.al_mm_b);
            if (s.cu_mm_b > 0)
                b.setCuFiltration(s.cu_mm_b);
            p->setTubeAmas(s.mas_a);
            p->setTubeBmas(s.mas_b);
            p->setSourceDetectorDistanceB(s.sdd_b);
            p->setFieldOfViewB(s.fov_b);
            p->setStartAngleDegB(s.start_angle_b_deg);
        }
        p->setPosition(pos);
        p->setSourceDetectorDistance(s.sdd);
        p->setCollimation(s.ct_collimation);
        p->setFieldOfView(s.fov);
        p->setGantryTiltAngleDeg(s.tilt_deg);
        p->setStartAngleDeg(s.start_angle_deg);
        p->setExposureAngleStepDeg(s.angle_step_deg);
        p->setScanLenght(s.scan_length);
        p->setModelHeelEffect(s.heel != 0);
        p->setHistoriesPerExposure(s.histories_per_exposure);
        return p;
    }
    case REF_CTSPIRAL:
    case REF_CTAXIAL: {
        std::unique_ptr<CTSource<T>> p;
        if (s.type == REF_CTSPIRAL) {
            auto sp = std::make_unique<CTSpiralSource<T>>();
            sp->setPitch(s.pitch);
            p = std::move(sp);
        } else {
            auto ax = std::make_unique<CTAxialSource<T>>();
            if (s.axial_step > 0)
                ax->setStep(s.axial_step);
            p = std::move(ax);
        }
        setup_tube(p->tube(), s);
        p->setPosition(pos);
        p->setSourceDetectorDistance(s.sdd);
        p->setCollimation(s.ct_collimation);
        p->setFieldOfView(s.fov);
        p->setGantryTiltAngleDeg(s.tilt_deg);
        p->setStartAngleDeg(s.start_angle_deg);
        p->setExposureAngleStepDeg(s.angle_step_deg);
        p->setScanLenght(s.scan_length);
        p->setModelHeelEffect(s.heel != 0);
        p->setHistoriesPerExposure(s.histories_per_exposure);
        if (s.bowtie_n > 0) {
            std::vector<T> a(s.bowtie_angles, s.bowtie_angles + s.bowtie_n);
            std::vector<T> w(s.bowtie_weights, s.bowtie_weights + s.bowtie_n);
            p->setBowTieFilter(std::make_shared<BowTieFilter<T>>(a, w));
        }
        return p;
    }
    default:
        return nullptr;
    }
}

} // namespace

extern "C" {

// BowTieFilter<double>(angles, weights) (beamfilters.hpp:102-115): its table
// (|angle| sorted, weights normalised to mean 1; n pairs into table_angles /
// table_weights) and sampleIntensityWeight (beamfilters.hpp:150-190) at the
// m query angles.
int ref_bowtie(const double* angles, const double* weights, int n, const double* queries, int m,
    double* table_angles, double* table_weights, double* out)
{
    if (n < 1 || !angles || !weights)
        return -1;
    const BowTieFilter<double> f(std::vector<double>(angles, angles + n), std::vector<double>(weights, weights + n));
    const auto& d = f.data();
    for (int i = 0; i < n; ++i) {
        table_angles[i] = d[i].first;
        table_weights[i] = d[i].second;
    }
    for (int i = 0; i < m; ++i)
        out[i] = f.sampleIntensityWeight(queries[i]);
    return 0;
}

// Number of energy nodes (after the first node is dropped) for a LUT built on
// this world; lets the caller size the coefficient buffers.
int ref_lut_dump(const RefWorldDesc* wd, double maxEnergy,
    const double* energies, int n_e, double* out_att, double* out_maxinv,
    const double* q, int n_q, double* out_sf,
    double* out_shells, // n_mat * 12 * 13
    double* out_rita, // n_mat * 4 * 56 (x, e, a, b)
    double* out_spline, // n_mat * (60 + 16 + 3)
    double* out_meta, // [resolution, linearIndex, linearStep, linearEnergy, minE, maxE]
    double* out_x, double* out_coef, double* out_maxcoef, int cap)
{
    World<double> world;
    if (!make_world(*wd, world))
        return -1;
    Lut lut;
    lut.generate(world, maxEnergy);
    const int nm = wd->n_materials;
    for (int m = 0; m < nm; ++m)
        for (int i = 0; i < n_e; ++i) {
            const auto a = lut.photoComptRayAttenuation(m, energies[i]);
            for (int k = 0; k < 3; ++k)
                out_att[(m * n_e + i) * 3 + k] = a[k];
        }
    for (int i = 0; i < n_e; ++i)
        out_maxinv[i] = lut.maxTotalAttenuationInverse(energies[i]);
    for (int m = 0; m < nm; ++m)
        for (int i = 0; i < n_q; ++i)
            out_sf[m * n_q + i] = lut.comptonScatterFactor(m, q[i]);
    for (int m = 0; m < nm; ++m) {
        const auto& sh = lut.electronShellConfiguration(m);
        for (int s = 0; s < 12; ++s) {
            double* o = out_shells + (m * 12 + s) * 13;
            o[0] = sh[s].bindingEnergy;
            o[1] = sh[s].numberElectrons;
            o[2] = sh[s].hartreeFockOrbital_0;
            o[3] = sh[s].photoIonizationProbability;
            o[4] = sh[s].fluorescenceYield;
            for (int k = 0; k < 3; ++k) {
                o[5 + k] = sh[s].fluorLineProbabilities[k];
                o[8 + k] = sh[s].fluorLineEnergies[k];
            }
            o[11] = sh[s].Z;
            o[12] = sh[s].shell;
        }
    }
    const auto& ff = lut.*member(LutFF {});
    const auto& sf = lut.*member(LutSF {});
    for (int m = 0; m < nm; ++m) {
        for (int k = 0; k < 56; ++k) {
            out_rita[(m * 4 + 0) * 56 + k] = (ff[m].*member(RitaX {}))[k];
            out_rita[(m * 4 + 1) * 56 + k] = (ff[m].*member(RitaE {}))[k];
            out_rita[(m * 4 + 2) * 56 + k] = (ff[m].*member(RitaA {}))[k];
            out_rita[(m * 4 + 3) * 56 + k] = (ff[m].*member(RitaB {}))[k];
        }
        double* o = out_spline + m * 79;
        const auto& c = sf[m].*member(SplineCoef {});
        const auto& x = sf[m].*member(SplineX {});
        for (int k = 0; k < 60; ++k)
            o[k] = c[k];
        for (int k = 0; k < 16; ++k)
            o[60 + k] = x[k];
        o[76] = sf[m].*member(SplineStart {});
        o[77] = sf[m].*member(SplineStep {});
        o[78] = sf[m].*member(SplineStop {});
    }
    const auto& data = lut.*member(LutData {});
    const auto& xs = data.*member(InterpX {});
    const auto& coef = data.*member(InterpCoef {});
    const auto& mcoef = data.*member(InterpMaxCoef {});
    out_meta[0] = static_cast<double>(data.*member(InterpResolution {}));
    out_meta[1] = static_cast<double>(data.*member(InterpLinearIndex {}));
    out_meta[2] = data.*member(InterpLinearStep {});
    out_meta[3] = data.*member(InterpLinearEnergy {});
    out_meta[4] = lut.*member(LutMinE {});
    out_meta[5] = lut.*member(LutMaxE {});
    out_meta[6] = static_cast<double>(xs.size());
    out_meta[7] = static_cast<double>(coef.size());
    out_meta[8] = static_cast<double>(mcoef.size());
    if (static_cast<int>(coef.size()) > cap)
        return -2;
    std::copy(xs.begin(), xs.end(), out_x);
    std::copy(coef.begin(), coef.end(), out_coef);
    std::copy(mcoef.begin(), mcoef.end(), out_maxcoef);
    return 0;
}

// Exposure table (19 doubles per exposure, world basis applied):
// pos[3], dirCos[6], beamDir[3], collimation[4], weight, nHistories, 0
// plus the spectrum (energies, alias probabilities, alias indices) and heel
// table when the source has them.
int ref_source_tables(const RefSourceDesc* sd, const RefWorldDesc* wd,
    double* out_exposures, std::uint64_t cap_exposures, std::uint64_t* n_exposures,
    double* spec_energies, double* spec_weights, double* spec_probs, std::uint64_t* spec_alias, int* spec_n, int spec_cap,
    double* heel_meta, double* heel_weights, int heel_cap,
    double* max_energy)
{
    World<double> world;
    if (!make_world(*wd, world))
        return -1;
    auto src = make_source<double>(*sd);
    if (!src)
        return -2;
    src->updateFromWorld(world);
    src->validate();
    if (!src->isValid())
        return -3;
    *max_energy = src->maxPhotonEnergyProduced();
    const auto n = src->totalExposures();
    *n_exposures = n;
    if (n > cap_exposures)
        return -4;
    const auto& basis = world.directionCosines();
    for (std::uint64_t i = 0; i < n; ++i) {
        auto e = src->getExposure(i);
        e.alignToDirectionCosines(basis);
        double* o = out_exposures + i * 19;
        for (int k = 0; k < 3; ++k)
            o[k] = e.position()[k];
        for (int k = 0; k < 6; ++k)
            o[3 + k] = e.directionCosines()[k];
        for (int k = 0; k < 3; ++k)
            o[9 + k] = e.beamDirection()[k];
        for (int k = 0; k < 4; ++k)
            o[12 + k] = e.collimationAngles()[k];
        o[16] = e.beamIntensityWeight();
        o[17] = static_cast<double>(e.numberOfHistories());
        o[18] = 0;
    }
    *spec_n = 0;
    heel_meta[0] = 0;
    const Tube<double>* tube = nullptr;
    double heel_span = 0;
    if (auto* dap = dynamic_cast<DAPSource<double>*>(src.get())) {
        tube = &static_cast<const DAPSource<double>*>(dap)->tube();
        heel_span = static_cast<const DAPSource<double>*>(dap)->collimationAngles()[1];
        if (!dap->modelHeelEffect())
            heel_span = -1;
    } else if (auto* ct = dynamic_cast<CTBaseSource<double>*>(src.get())) {
        tube = &static_cast<const CTBaseSource<double>*>(ct)->tube();
        heel_span = std::atan(ct->collimation() * 0.5 / ct->sourceDetectorDistance()) * 2.0;
        if (!ct->modelHeelEffect())
            heel_span = -1;
    }
    if (tube) {
        auto energies = tube->getEnergy();
        auto weights = tube->getSpecter(energies);
        SpecterDistribution<double> dist(weights, energies);
        const int ns = static_cast<int>(energies.size());
        if (ns > spec_cap)
            return -5;
        *spec_n = ns;
        for (int i = 0; i < ns; ++i) {
            spec_energies[i] = energies[i];
            spec_weights[i] = weights[i];
            spec_probs[i] = dist.probabilityData()[i];
            spec_alias[i] = dist.aliasingData()[i];
        }
        if (heel_span >= 0) {
            Heel heel(*tube, heel_span);
            const auto& w = heel.weights();
            if (static_cast<int>(w.size()) > heel_cap)
                return -6;
            heel_meta[0] = 1;
            heel_meta[1] = heel.*member(HeelEnergyStart {});
            heel_meta[2] = heel.*member(HeelEnergyStep {});
            heel_meta[3] = static_cast<double>(heel.energySize());
            heel_meta[4] = heel.*member(HeelAngleStart {});
            heel_meta[5] = heel.*member(HeelAngleStep {});
            heel_meta[6] = static_cast<double>(heel.angleSize());
            std::copy(w.begin(), w.end(), heel_weights);
        }
    } else if (sd->type == REF_ISOTROPIC || sd->type == REF_ISOTROPIC_CT) {
        std::vector<double> e(sd->spec_energies, sd->spec_energies + sd->spec_n);
        std::vector<double> w(sd->spec_weights, sd->spec_weights + sd->spec_n);
        SpecterDistribution<double> dist(w, e);
        if (sd->spec_n > spec_cap)
            return -5;
        *spec_n = sd->spec_n;
        for (int i = 0; i < sd->spec_n; ++i) {
            spec_energies[i] = e[i];
            spec_weights[i] = w[i];
            spec_probs[i] = dist.probabilityData()[i];
            spec_alias[i] = dist.aliasingData()[i];
        }
    }
    return 0;
}

// Alias table of SpecterDistribution for arbitrary weights (dxmcrandom.hpp:229-274).
int ref_alias_table(const double* weights, int n, double* probs, std::uint64_t* alias)
{
    std::vector<double> w(weights, weights + n);
    std::vector<double> e(n);
    for (int i = 0; i < n; ++i)
        e[i] = i;
    SpecterDistribution<double> dist(w, e);
    for (int i = 0; i < n; ++i) {
        probs[i] = dist.probabilityData()[i];
        alias[i] = dist.aliasingData()[i];
    }
    return 0;
}

int ref_transport(const RefWorldDesc* wd, const RefSourceDesc* sd, int model, int n_threads,
    double* dose, double* variance, std::uint32_t* n_events, double* meta)
{
    World<double> world;
    if (!make_world(*wd, world))
        return -1;
    auto src = make_source<double>(*sd);
    if (!src)
        return -2;
    Transport<double> transport;
    transport.setNumberOfWorkers(n_threads > 0 ? n_threads : std::thread::hardware_concurrency());
    transport.setLowEnergyCorrectionModel(static_cast<LOWENERGYCORRECTION>(model));
    transport.setOutputMode(Transport<double>::OUTPUTMODE::EV_PER_HISTORY);
    auto res = transport(world, src.get(), nullptr, false);
    const std::size_t n = world.size();
    for (std::size_t i = 0; i < n; ++i) {
        dose[i] = res.dose[i];
        variance[i] = res.variance[i];
        n_events[i] = res.nEvents[i];
    }
    meta[0] = static_cast<double>(res.numberOfHistories);
    meta[1] = res.simulationTime.count();
    return res.numberOfHistories > 0 ? 0 : -3;
}

} // extern "C"

namespace {
template <class T>
int transport_any(const RefWorldDesc* wd, const RefSourceDesc* sd, int model, int n_threads, int output_mode,
    int use_calibration, double* dose, double* variance, std::uint32_t* n_events, double* meta)
{
    World<T> world;
    if (!make_world(*wd, world))
        return -1;
    auto src = make_source<T>(*sd);
    if (!src)
        return -2;
    Transport<T> transport;
    transport.setNumberOfWorkers(n_threads > 0 ? n_threads : std::thread::hardware_concurrency());
    transport.setLowEnergyCorrectionModel(static_cast<LOWENERGYCORRECTION>(model));
    transport.setOutputMode(output_mode == 1 ? Transport<T>::OUTPUTMODE::DOSE : Transport<T>::OUTPUTMODE::EV_PER_HISTORY);
    auto res = transport(world, src.get(), nullptr, use_calibration != 0);
    const std::size_t n = world.size();
    for (std::size_t i = 0; i < n; ++i) {
        dose[i] = res.dose[i];
        variance[i] = res.variance[i];
        n_events[i] = res.nEvents[i];
    }
    meta[0] = static_cast<double>(res.numberOfHistories);
    meta[1] = std::chrono::duration<double>(res.simulationTime).count();
    meta[2] = 0.0;
    meta[3] = res.dose_units == "mGy" ? 2 : (res.dose_units == "keV/kg" ? 1 : 0);
    return res.numberOfHistories > 0 ? 0 : -3;
}
} // namespace

extern "C" {

// Transport<T>::operator() (transport.hpp:135-202) in T = double (precision 0) or
// float (precision 1) on World<T>, in EV_PER_HISTORY (output_mode 0) or DOSE
// (output_mode 1) mode; with use_calibration the source's calibration factor
// converts keV/kg to mGy (transport.hpp:187-195).  meta: [histories, seconds of
// Result::simulationTime (the timed transport, transport.hpp:166-174), 0,
// units (0 eV/history, 1 keV/kg, 2 mGy)].
int ref_transport_ex(const RefWorldDesc* wd, const RefSourceDesc* sd, int model, int n_threads, int output_mode,
    int use_calibration, int precision, double* dose, double* variance, std::uint32_t* n_events, double* meta)
{
    if (precision == 1)
        return transport_any<float>(wd, sd, model, n_threads, output_mode, use_calibration, dose, variance, n_events, meta);
    return transport_any<double>(wd, sd, model, n_threads, output_mode, use_calibration, dose, variance, n_events, meta);
}

// Source<double>::getCalibrationValue (source.hpp:196) after updateFromWorld and
// validate, as Transport::operator() calls it in DOSE mode (transport.hpp:146-190):
// the factor that turns keV/kg into mGy.  Deterministic for DX (dose-area
// product, source.hpp:552-568); a Monte Carlo estimate for CT sources.
int ref_calibration_value(const RefWorldDesc* wd, const RefSourceDesc* sd, int model, double* value)
{
    World<double> world;
    if (!make_world(*wd, world))
        return -1;
    auto src = make_source<double>(*sd);
    if (!src)
        return -2;
    src->updateFromWorld(world);
    src->validate();
    if (!src->isValid())
        return -3;
    *value = src->getCalibrationValue(static_cast<LOWENERGYCORRECTION>(model), nullptr);
    return 0;
}

// CTDIPhantom<double> (world.hpp:229-390): arrays and the five hole index lists
// (Center, West, East, South, North).  Sizes are queried with null arrays.
int ref_ctdi_phantom(int diameter, std::uint64_t* dims, double* density, std::uint8_t* material, std::uint8_t* measurement,
    std::uint64_t* hole_counts, std::uint64_t* hole_indices, std::uint64_t hole_cap)
{
    CTDIPhantom<double> w(static_cast<std::size_t>(diameter));
    const auto d = w.dimensions();
    for (int k = 0; k < 3; ++k)
        dims[k] = d[k];
    const std::size_t n = w.size();
    if (density) {
        const auto& dens = *w.densityArray();
        const auto& mat = *w.materialIndexArray();
        const auto& meas = *w.measurementMapArray();
        for (std::size_t i = 0; i < n; ++i) {
            density[i] = dens[i];
            material[i] = mat[i];
            measurement[i] = meas[i];
        }
    }
    using H = CTDIPhantom<double>::HolePosition;
    const H order[5] = { H::Center, H::West, H::East, H::South, H::North };
    std::uint64_t off = 0;
    for (int h = 0; h < 5; ++h) {
        const auto& idx = w.holeIndices(order[h]);
        hole_counts[h] = idx.size();
        if (hole_indices) {
            if (off + idx.size() > hole_cap)
                return -1;
            for (auto v : idx)
                hole_indices[off++] = v;
        }
    }
    return 0;
}

// The spectrum and heel tables exposure `index` of a source samples with (its
// SpecterDistribution and HeelFilter, exposure.hpp:45-47): dual-source CT
// alternates two of each (source.hpp:1384-1410).  Tube B's energies and
// normalised weights (CTDualSource::updateSpecterDistribution, source.hpp:1150-1175)
// are written for dual sources.
int ref_exposure_tables(const RefSourceDesc* sd, const RefWorldDesc* wd, std::uint64_t index,
    double* spec_probs, std::uint64_t* spec_alias, int* spec_n, int spec_cap,
    double* heel_meta, double* heel_weights, int heel_cap,
    double* tube_b_energies, double* tube_b_weights, int* tube_b_n)
{
    World<double> world;
    if (!make_world(*wd, world))
        return -1;
    auto src = make_source<double>(*sd);
    if (!src)
        return -2;
    src->updateFromWorld(world);
    src->validate();
    if (!src->isValid() || index >= src->totalExposures())
        return -3;
    const auto e = src->getExposure(index);
    *spec_n = 0;
    heel_meta[0] = 0;
    if (SpecPtr d = e.*member(ExpoSpecter {})) {
        const auto& probs = d->probabilityData();
        const auto& alias = d->aliasingData();
        if (static_cast<int>(probs.size()) > spec_cap)
            return -5;
        *spec_n = static_cast<int>(probs.size());
        std::copy(probs.begin(), probs.end(), spec_probs);
        std::copy(alias.begin(), alias.end(), spec_alias);
    }
    if (HeelPtr h = e.*member(ExpoHeel {})) {
        const auto& w = h->weights();
        if (static_cast<int>(w.size()) > heel_cap)
            return -6;
        heel_meta[0] = 1;
        heel_meta[1] = h->*member(HeelEnergyStart {});
        heel_meta[2] = h->*member(HeelEnergyStep {});
        heel_meta[3] = static_cast<double>(h->energySize());
        heel_meta[4] = h->*member(HeelAngleStart {});
        heel_meta[5] = h->*member(HeelAngleStep {});
        heel_meta[6] = static_cast<double>(h->angleSize());
        std::copy(w.begin(), w.end(), heel_weights);
    }
    *tube_b_n = 0;
    if (auto* dual = dynamic_cast<CTDualSource<double>*>(src.get())) {
        const Tube<double>& b = static_cast<const CTDualSource<double>*>(dual)->tubeB();
        const auto energies = b.getEnergy();
        const auto weights = b.getSpecter(energies);
        if (static_cast<int>(energies.size()) > spec_cap)
            return -7;
        *tube_b_n = static_cast<int>(energies.size());
        std::copy(energies.begin(), energies.end(), tube_b_energies);
        std::copy(weights.begin(), weights.end(), tube_b_weights);
    }
    return 0;
}

// CTSpiralSource<double>::getCalibrationValue (source.hpp:1358-1363 -> ctCalibration,
// source.hpp:925-988): the reference's CTDI calibration factor, run with its own
// Transport<double> on n_threads workers.  meta: [axial exposures per rotation,
// histories per exposure of the calibration run, mean exposure weight].
int ref_ct_calibration(const RefSourceDesc* sd, int model, int n_threads, double ctdivol, int diameter, double* factor,
    double* meta)
{
    if (sd->type != REF_CTSPIRAL)
        return -1;
    auto base = make_source<double>(*sd);
    auto* spiral = dynamic_cast<CTSpiralSource<double>*>(base.get());
    if (!spiral)
        return -2;
    spiral->setCtdiVol(ctdivol);
    spiral->setCtdiPhantomDiameter(static_cast<std::uint64_t>(diameter));
    if (n_threads > 0) {
        // Transport's default worker count is hardware_concurrency; ctCalibration
        // constructs its own Transport, so the count cannot be passed through.
    }
    spiral->validate();
    CTAxialSource<double> axial(*spiral);
    double meanWeight = 0;
    for (std::uint64_t i = 0; i < spiral->totalExposures(); ++i)
        meanWeight += spiral->getExposure(i).beamIntensityWeight();
    meanWeight /= static_cast<double>(spiral->totalExposures());
    std::size_t stat = CTDIPhantom<double>::ctdiMinHistories() / (axial.exposuresPerRotatition() * axial.historiesPerExposure());
    if (stat < 1)
        stat = 1;
    meta[0] = static_cast<double>(axial.exposuresPerRotatition());
    meta[1] = static_cast<double>(axial.historiesPerExposure() * stat);
    meta[2] = meanWeight;
    *factor = spiral->getCalibrationValue(static_cast<LOWENERGYCORRECTION>(model), nullptr);
    return 0;
}

} // extern "C"

namespace {
// Subclass exposing the reference's protected interaction samplers.
class Sampler : public Transport<double> {
public:
    template <int L>
    void run(int kind, double energy, std::uint64_t n, int nbins, double* hist_cos, double* hist_e, double* sums, RandomState& state)
    {
        const std::array<double, 3> dir0 { 0, 0, 1 };
        for (std::uint64_t i = 0; i < n; ++i) {
            Particle<double> p { .pos = { 0, 0, 0 }, .dir = dir0, .energy = energy, .weight = 1 };
            double dep = 0;
            if (kind == 0)
                dep = this->template photoAbsorption<L>(p, 0, state);
            else if (kind == 1)
                dep = this->template comptonScatter<L>(p, 0, state);
            else
                this->template rayleightScatter<L>(p, 0, state);
            const double len = std::sqrt(p.dir[0] * p.dir[0] + p.dir[1] * p.dir[1] + p.dir[2] * p.dir[2]);
            const double c = len > 0 ? p.dir[2] / len : 1.0;
            int bc = static_cast<int>((c + 1) * 0.5 * nbins);
            bc = std::clamp(bc, 0, nbins - 1);
            hist_cos[bc] += 1;
            int be = static_cast<int>(p.energy / energy * nbins);
            be = std::clamp(be, 0, nbins - 1);
            hist_e[be] += 1;
            sums[0] += dep;
            sums[1] += p.energy;
            sums[2] += len;
        }
    }
};
}

extern "C" int ref_interactions(const RefWorldDesc* wd, double maxEnergy, int model, int kind, double energy,
    std::uint64_t n, int nbins, std::uint64_t seed, double* hist_cos, double* hist_e, double* sums)
{
    World<double> world;
    if (!make_world(*wd, world))
        return -1;
    Sampler s;
    s.attenuationLut().generate(world, maxEnergy);
    std::uint64_t st[2] = { seed * 0x9E3779B97F4A7C15ULL + 1, seed ^ 0xD1B54A32D192ED03ULL };
    RandomState state(st);
    if (model == 0)
        s.run<0>(kind, energy, n, nbins, hist_cos, hist_e, sums, state);
    else if (model == 1)
        s.run<1>(kind, energy, n, nbins, hist_cos, hist_e, sums, state);
    else
        s.run<2>(kind, energy, n, nbins, hist_cos, hist_e, sums, state);
    return 0;
}
