// dxmc_gpu/transport.hpp — drop-in GPU replacement for dxmc::Transport<T>.
//
// Header-only C++20 adapter for code that uses DXMClib: include this header
// after DXMClib's own headers and replace
//
//     dxmc::Transport<T> transport;             // include/dxmc/transport.hpp:114-840
//     auto result = transport(world, &source);
// with
//     dxmc::gpu::Transport<T> transport;
//     auto result = transport(world, &source);
//
// The adapter keeps DXMClib's World / Source / Material / ProgressBar types and
// its Result<T>; it reads them only through their public members, flattens the
// exposures (Source::getExposure + Exposure::alignToDirectionCosines), wraps
// each Material as a dxmc_material_provider for the host LUT build, and runs
// photon generation, Woodcock tracking, interactions and scoring on the GPU
// through the C ABI in dxmc_gpu.h.  Link with libdxmc_gpu.so.
//
// Error behaviour follows the reference (transport.hpp:142-151, 176-185): an
// invalid world or source, a missing GPU, or a cancelled run returns a
// zero-filled Result with numberOfHistories == 0; lastError() explains why.
#pragma once

#include "dxmc_gpu.h"

#include "dxmc/exposure.hpp"
#include "dxmc/lowenergycorrectionmodel.hpp"
#include "dxmc/material.hpp"
#include "dxmc/progressbar.hpp"
#include "dxmc/source.hpp"
#include "dxmc/transport.hpp"
#include "dxmc/world.hpp"

#include <chrono>
#include <cmath>
#include <memory>
#include <string>
#include <vector>

namespace dxmc::gpu {

namespace detail {

    // dxmc::Material -> dxmc_material_provider (material.hpp:60-101)
    inline double photo_cb(void* u, double e) { return static_cast<const Material*>(u)->getPhotoelectricAttenuation(e); }
    inline double compton_cb(void* u, double e) { return static_cast<const Material*>(u)->getComptonAttenuation(e); }
    inline double rayleigh_cb(void* u, double e) { return static_cast<const Material*>(u)->getRayleightAttenuation(e); }
    inline double ff2_cb(void* u, double q) { return static_cast<const Material*>(u)->getRayleightFormFactorSquared(q); }
    inline double sf_cb(void* u, double q) { return static_cast<const Material*>(u)->getComptonNormalizedScatterFactor(q); }
    inline int edges_cb(void* u, double minE, double* out, int cap)
    {
        const auto e = static_cast<const Material*>(u)->getBindingEnergies(minE);
        const int n = static_cast<int>(e.size());
        for (int i = 0; i < n && i < cap; ++i)
            out[i] = e[i];
        return n;
    }
    inline void shells_cb(void* u, dxmc_shell_config out[12])
    {
        const auto c = static_cast<const Material*>(u)->getElectronConfiguration();
        for (int i = 0; i < 12; ++i) {
            out[i].binding_energy = c[i].bindingEnergy;
            out[i].number_electrons = c[i].numberElectrons;
            out[i].hartree_fock_j0 = c[i].hartreeFockOrbital_0;
            out[i].photo_ionization_probability = c[i].photoIonizationProbability;
            out[i].fluorescence_yield = c[i].fluorescenceYield;
            for (int k = 0; k < 3; ++k) {
                out[i].line_probabilities[k] = c[i].fluorLineProbabilities[k];
                out[i].line_energies[k] = c[i].fluorLineEnergies[k];
            }
            out[i].Z = c[i].Z;
            out[i].shell = c[i].shell;
        }
    }

    inline dxmc_material_provider provider(const Material& m)
    {
        dxmc_material_provider p {};
        p.user = const_cast<Material*>(&m);
        p.standard_density = m.standardDensity();
        p.photoelectric = photo_cb;
        p.compton = compton_cb;
        p.rayleigh = rayleigh_cb;
        p.form_factor_squared = ff2_cb;
        p.scatter_factor = sf_cb;
        p.binding_energies = edges_cb;
        p.shells = shells_cb;
        return p;
    }

} // namespace detail

// Host tables of one source, ready for dxmc_gpu_job_submit.
template <Floating T>
struct FlatSource {
    std::vector<dxmc_exposure> exposures;
    std::vector<double> spec_energies, spec_weights;
    std::vector<double> heel_weights;
    dxmc_heel_desc heel {};
    bool has_heel = false;
    std::vector<double> bowtie_angles, bowtie_weights;
    double max_energy = 0;
};

// Spectrum (Tube::getSpecter, normalised) and, for heel_span >= 0, the heel table
// (HeelFilter, beamfilters.hpp:455-505) of one tube.
template <Floating T>
void tube_tables(const Tube<T>& tube, T heel_span, FlatSource<T>& out)
{
    const auto energies = tube.getEnergy();
    const auto weights = tube.getSpecter(energies);
    out.spec_energies.assign(energies.begin(), energies.end());
    out.spec_weights.assign(weights.begin(), weights.end());
    out.heel_weights.clear();
    out.has_heel = false;
    if (heel_span >= 0) {
        HeelFilter<T> heel(tube, heel_span);
        out.heel_weights.assign(heel.weights().begin(), heel.weights().end());
        // grid of HeelFilter::update (beamfilters.hpp:467-483): 10 keV + 2 keV steps,
        // angle bins from -min(anode angle, span/2) to +span/2
        const T span = std::abs(heel_span);
        const T start = tube.anodeAngle() < span / 2 ? -tube.anodeAngle() : -span / 2;
        out.heel.energy_start = 10.0;
        out.heel.energy_step = 2.0;
        out.heel.energy_size = static_cast<int32_t>(heel.energySize());
        out.heel.angle_size = static_cast<int32_t>(heel.angleSize());
        out.heel.angle_start = start;
        out.heel.angle_step = (span / 2 - start) / static_cast<T>(heel.angleSize());
        out.heel.weights = out.heel_weights.data();
        out.has_heel = true;
    }
}

// Flattens Source::getExposure(i) for every exposure (source.hpp), applying the
// world basis like workerRun does (transport.hpp:750-757).  Spectrum, heel and
// bow-tie tables are read through the public API of the sources that own them:
// DAPSource/CBCT and the CT family expose tube() (tube.hpp:165-212) and the CT
// family bowTieFilter(); IsotropicSource keeps its spectrum private, so callers
// pass it in `isotropic_spectrum` (energies, weights).
template <Floating T>
bool flatten(const World<T>& world, Source<T>* source, FlatSource<T>& out,
    const std::pair<std::vector<T>, std::vector<T>>* isotropic_spectrum = nullptr)
{
    const auto n = source->totalExposures();
    out.exposures.resize(n);
    const auto& basis = world.directionCosines();
    for (std::uint64_t i = 0; i < n; ++i) {
        auto e = source->getExposure(i);
        e.alignToDirectionCosines(basis);
        auto& x = out.exposures[i];
        for (int k = 0; k < 3; ++k) {
            x.position[k] = e.position()[k];
            x.beam_direction[k] = e.beamDirection()[k];
        }
        for (int k = 0; k < 6; ++k)
            x.direction_cosines[k] = e.directionCosines()[k];
        for (int k = 0; k < 4; ++k)
            x.collimation[k] = e.collimationAngles()[k];
        x.weight = e.beamIntensityWeight();
        x.n_histories = e.numberOfHistories();
        x.mono_energy = 0;
    }
    out.max_energy = source->maxPhotonEnergyProduced();
    const Tube<T>* tube = nullptr;
    T heel_span = -1;
    if (auto* pencil = dynamic_cast<PencilSource<T>*>(source)) {
        for (auto& x : out.exposures)
            x.mono_energy = pencil->photonEnergy();
    } else if (auto* dap = dynamic_cast<DAPSource<T>*>(source)) {
        const auto* cdap = dap;
        tube = &cdap->tube();
        if (dap->modelHeelEffect())
            heel_span = cdap->collimationAngles()[1]; // DAPSource::updateSpecterDistribution (source.hpp:600-612)
    } else if (auto* ct = dynamic_cast<CTBaseSource<T>*>(source)) {
        const auto* cct = ct;
        tube = &cct->tube();
        if (ct->modelHeelEffect()) // CTBaseSource::updateSpecterDistribution (source.hpp:989-1002)
            heel_span = std::atan(ct->collimation() * T { 0.5 } / ct->sourceDetectorDistance()) * T { 2.0 };
        if (auto bt = cct->bowTieFilter()) {
            for (const auto& [a, w] : bt->data()) {
                out.bowtie_angles.push_back(a);
                out.bowtie_weights.push_back(w);
            }
        }
    } else if (dynamic_cast<IsotropicSource<T>*>(source)) {
        if (!isotropic_spectrum)
            return false;
        out.spec_energies.assign(isotropic_spectrum->first.begin(), isotropic_spectrum->first.end());
        out.spec_weights.assign(isotropic_spectrum->second.begin(), isotropic_spectrum->second.end());
    }
    if (tube)
        tube_tables(*tube, heel_span, out);
    return true;
}

// The beams of a source: groups of its exposures that sample one spectrum, heel
// table and bow-tie filter, each run as a job of its own.  A dual-source CT
// scanner (CTDualSource, source.hpp:1078-1190) alternates tube A (even exposures)
// and tube B (odd ones), each with its own spectrum, heel table (always built,
// with tube A's distance: source.hpp:1170-1172) and bow-tie filter; every other
// source is one beam.
template <Floating T>
bool flatten_beams(const World<T>& world, Source<T>* source, std::vector<FlatSource<T>>& beams,
    const std::pair<std::vector<T>, std::vector<T>>* isotropic_spectrum = nullptr)
{
    beams.assign(1, FlatSource<T> {});
    if (!flatten(world, source, beams[0], isotropic_spectrum))
        return false;
    auto* dual = dynamic_cast<CTDualSource<T>*>(source);
    if (!dual)
        return true;
    const auto* cdual = dual;
    FlatSource<T> all = std::move(beams[0]);
    beams.assign(2, FlatSource<T> {});
    for (std::size_t i = 0; i < all.exposures.size(); ++i)
        beams[i % 2].exposures.push_back(all.exposures[i]);
    const T span = std::atan(cdual->collimation() * T { 0.5 } / cdual->sourceDetectorDistance()) * T { 2.0 };
    tube_tables(cdual->tube(), span, beams[0]);
    tube_tables(cdual->tubeB(), span, beams[1]);
    const std::shared_ptr<BowTieFilter<T>> filters[2] = { cdual->bowTieFilter(), cdual->bowTieFilterB() };
    for (int b = 0; b < 2; ++b) {
        beams[b].max_energy = all.max_energy;
        if (filters[b])
            for (const auto& [a, w] : filters[b]->data()) {
                beams[b].bowtie_angles.push_back(a);
                beams[b].bowtie_weights.push_back(w);
            }
    }
    return true;
}

template <Floating T = double>
class Transport {
public:
    enum class OUTPUTMODE { EV_PER_HISTORY, DOSE };

    Transport() = default;
    ~Transport() { release(); }
    Transport(const Transport&) = delete;
    Transport& operator=(const Transport&) = delete;

    void setNumberOfWorkers(std::uint64_t) { } // the GPU launch replaces worker threads
    std::size_t numberOfWorkers() const { return 1; }
    void setLowEnergyCorrectionModel(LOWENERGYCORRECTION model) { m_model = model; }
    LOWENERGYCORRECTION lowEnergyCorrectionModel() const { return m_model; }
    void setOutputMode(OUTPUTMODE mode) { m_mode = mode; }
    OUTPUTMODE outputMode() const { return m_mode; }
    void setDevice(int device) { m_options.device = device; }
    void setSeed(std::uint64_t seed) { m_seed = seed; }
    void setTallyMode(int mode) { m_options.tally_mode = mode; }
    // GPU-only choices, with the reference's behaviour at REFERENCE direction and
    // either tracking mode (local majorants sample the same process, faster):
    // DXMC_TRACKING_DEFAULT / GLOBAL / LOCAL and DXMC_DIRECTION_REFERENCE / NORMALIZED.
    void setTracking(int tracking) { m_tracking = tracking; }
    int tracking() const { return m_tracking; }
    void setDirectionMode(int direction) { m_direction = direction; }
    int directionMode() const { return m_direction; }
    // DXMC_PRECISION_FP32 (default: FP32 transport, FP64 tallies) or
    // DXMC_PRECISION_FP64 (everything in double, as Transport<double> computes)
    void setTransportPrecision(int precision) { m_precision = precision; }
    int transportPrecision() const { return m_precision; }
    // Spectrum for IsotropicSource, whose spectrum has no public getter.
    void setIsotropicSpectrum(std::vector<T> energies, std::vector<T> weights) { m_iso = { std::move(energies), std::move(weights) }; }
    const std::string& lastError() const { return m_error; }

    template <typename U>
        requires std::is_base_of<World<T>, U>::value
    Result<T> operator()(const U& world, Source<T>* source, ProgressBar<T>* progressbar = nullptr, bool useSourceDoseCalibration = true)
    {
        Result<T> result(world.size());
        m_error.clear();
        if (!world.isValid() || !source) {
            m_error = "invalid world or source";
            return result;
        }
        source->updateFromWorld(world);
        source->validate();
        if (!source->isValid()) {
            m_error = "invalid source";
            return result;
        }
        std::vector<FlatSource<T>> beams;
        if (!flatten_beams(world, source, beams, m_iso.first.empty() ? nullptr : &m_iso)) {
            m_error = "source type needs setIsotropicSpectrum";
            return result;
        }
        if (!ensure_context())
            return result;

        const auto& dims = world.dimensions();
        const std::size_t n = world.size();
        std::vector<float> density(n);
        const auto& dsrc = *world.densityArray();
        for (std::size_t i = 0; i < n; ++i)
            density[i] = static_cast<float>(dsrc[i]);
        dxmc_world_desc wd {};
        for (int i = 0; i < 3; ++i) {
            wd.dims[i] = dims[i];
            wd.spacing[i] = world.spacing()[i];
            wd.origin[i] = world.origin()[i];
        }
        for (int i = 0; i < 6; ++i)
            wd.direction_cosines[i] = world.directionCosines()[i];
        wd.density = density.data();
        wd.material = world.materialIndexArray()->data();
        const auto meas = world.measurementMapArray();
        bool any_meas = false;
        if (meas)
            for (auto v : *meas)
                if (v) {
                    any_meas = true;
                    break;
                }
        wd.measurement = any_meas ? meas->data() : nullptr;
        const auto& materials = world.materialMap();
        wd.n_materials = static_cast<int32_t>(materials.size());

        dxmc_world* dworld = nullptr;
        if (!check(dxmc_gpu_world_upload(m_ctx, &wd, &dworld), "world upload"))
            return result;
        std::vector<double> maxDensity(materials.size());
        std::vector<dxmc_material_provider> providers;
        for (const auto& m : materials)
            providers.push_back(detail::provider(m));
        dxmc_lut_blob* blob = nullptr;
        dxmc_lut* lut = nullptr;
        bool ok = check(dxmc_gpu_world_max_density(dworld, maxDensity.data(), static_cast<int>(maxDensity.size())), "max density")
            && check(dxmc_lut_build_max_density(providers.data(), static_cast<int>(providers.size()), maxDensity.data(), beams[0].max_energy, &blob), "lut build")
            && check(dxmc_gpu_lut_upload(m_ctx, blob, &lut), "lut upload");
        // one job per beam; beam k draws from streams of a seed of its own
        const std::uint64_t seed = m_seed++;
        std::vector<dxmc_job*> jobs(beams.size(), nullptr);
        std::uint64_t histories = 0, total_exposures = 0;
        for (const auto& b : beams) {
            total_exposures += b.exposures.size();
            for (const auto& e : b.exposures)
                histories += e.n_histories;
        }
        const auto start = std::chrono::system_clock::now();
        if (progressbar)
            progressbar->setTotalExposures(total_exposures);
        for (std::size_t k = 0; k < beams.size() && ok; ++k) {
            auto& b = beams[k];
            b.heel.weights = b.heel_weights.data();
            dxmc_spectrum_desc spec { static_cast<int32_t>(b.spec_energies.size()), b.spec_energies.data(), b.spec_weights.data() };
            dxmc_bowtie_desc bowtie { static_cast<int32_t>(b.bowtie_angles.size()), b.bowtie_angles.data(), b.bowtie_weights.data() };
            dxmc_job_desc jd {};
            jd.exposures = b.exposures.data();
            jd.n_exposures = b.exposures.size();
            jd.spectrum = b.spec_energies.empty() ? nullptr : &spec;
            jd.heel = b.has_heel ? &b.heel : nullptr;
            jd.bowtie = b.bowtie_angles.empty() ? nullptr : &bowtie;
            jd.seed = seed + k * 0x9E3779B97F4A7C15ull;
            jd.model = static_cast<int32_t>(m_model);
            jd.tally_mode = -1;
            jd.tracking = m_tracking;
            jd.direction = m_direction;
            jd.precision = m_precision;
            ok = check(dxmc_gpu_job_submit(m_ctx, dworld, lut, &jd, &jobs[k]), "job submit");
        }
        bool cancelled = false;
        std::uint64_t reported = 0; // exposures reported to the progress bar
        std::vector<double> preview, part;
        auto last_preview = std::chrono::steady_clock::now();
        const std::uint64_t per_exposure = std::max<std::uint64_t>(1, beams[0].exposures.empty() ? 1 : beams[0].exposures[0].n_histories);
        for (std::size_t k = 0; k < jobs.size() && ok; ++k) {
            while (ok) {
                const int rc = dxmc_gpu_job_wait(jobs[k], 50);
                if (rc == DXMC_OK)
                    break;
                if (rc != DXMC_ERR_TIMEOUT) {
                    ok = check(rc, "job wait");
                    break;
                }
                if (progressbar && progressbar->cancel() && !cancelled) {
                    for (auto* j : jobs)
                        dxmc_gpu_job_cancel(j);
                    cancelled = true;
                }
                if (progressbar && !cancelled) {
                    // ProgressBar::exposureCompleted per exposure's worth of histories taken, and
                    // a dose preview from the live tallies about once a second (progressbar.hpp:54-101)
                    std::uint64_t started = 0;
                    for (auto* j : jobs) {
                        std::uint64_t s_j = 0;
                        if (dxmc_gpu_job_progress(j, &s_j, nullptr) == DXMC_OK)
                            started += s_j;
                    }
                    const std::uint64_t done = std::min<std::uint64_t>(started / per_exposure, total_exposures);
                    for (; reported < done; ++reported)
                        progressbar->exposureCompleted();
                    const auto now = std::chrono::steady_clock::now();
                    if (now - last_preview > std::chrono::seconds(1)) {
                        last_preview = now;
                        preview.assign(n, 0.0);
                        part.resize(n);
                        bool got = true;
                        for (auto* j : jobs) {
                            got = got && dxmc_gpu_job_preview(j, part.data()) == DXMC_OK;
                            for (std::size_t i = 0; got && i < n; ++i)
                                preview[i] += part[i];
                        }
                        if (got) {
                            for (std::size_t i = 0; i < n; ++i)
                                result.dose[i] = static_cast<T>(preview[i]);
                            progressbar->setDoseData(result.dose.data(), world.dimensions(), world.spacing());
                        }
                    }
                }
            }
        }
        result.simulationTime = std::chrono::system_clock::now() - start;
        if (ok && !cancelled) {
            result.numberOfHistories = histories;
            double cal = 1.0;
            if (m_mode == OUTPUTMODE::DOSE)
                cal = useSourceDoseCalibration ? static_cast<double>(calibrationValue(source, progressbar)) : 1.0;
            if (jobs.size() == 1) {
                std::vector<double> dose(n), var(n);
                const int mode = m_mode == OUTPUTMODE::DOSE ? DXMC_OUTPUT_DOSE : DXMC_OUTPUT_EV_PER_HISTORY;
                ok = check(dxmc_gpu_job_result(jobs[0], mode, cal, dose.data(), var.data(), result.nEvents.data(), nullptr), "job result");
                for (std::size_t i = 0; ok && i < n; ++i) {
                    result.dose[i] = static_cast<T>(dose[i]);
                    result.variance[i] = static_cast<T>(var[i]);
                }
            } else {
                // the beams' raw tallies add; then the reference's normalisation over all
                // histories (normalizeScoring / energyImpartedToDose, transport.hpp:780-816)
                std::vector<double> e(n, 0.0), e2(n, 0.0), de(n), de2(n);
                std::vector<std::uint32_t> ev(n);
                std::fill(result.nEvents.begin(), result.nEvents.end(), 0u);
                for (auto* j : jobs) {
                    ok = ok && check(dxmc_gpu_job_result(j, DXMC_OUTPUT_RAW, 1.0, de.data(), de2.data(), ev.data(), nullptr), "job result");
                    for (std::size_t i = 0; ok && i < n; ++i) {
                        e[i] += de[i];
                        e2[i] += de2[i];
                        result.nEvents[i] += ev[i];
                    }
                }
                if (ok && m_mode == OUTPUTMODE::DOSE) {
                    const auto& sp = world.spacing();
                    const double voxel_volume = sp[0] * sp[1] * sp[2] / 1000.0; // cm3
                    for (std::size_t i = 0; i < n; ++i) {
                        const double d = static_cast<double>(dsrc[i]);
                        const double factor = d > 0.0 ? cal / (d * voxel_volume * 0.001) : 0.0; // per kg
                        result.dose[i] = static_cast<T>(d > 0.0 ? e[i] * factor : 0.0);
                        result.variance[i] = static_cast<T>(d > 0.0 ? e2[i] * factor * factor : 0.0);
                    }
                } else if (ok) {
                    const double h = static_cast<double>(histories);
                    for (std::size_t i = 0; i < n; ++i) {
                        const double d = e[i] * (1e3 / h);
                        result.dose[i] = static_cast<T>(d);
                        result.variance[i] = static_cast<T>((e2[i] * (1e6 / h) - d * d) * (1.0 / (h - 1.0)));
                    }
                }
            }
            if (ok)
                result.dose_units = m_mode == OUTPUTMODE::DOSE ? (useSourceDoseCalibration ? "mGy" : "keV/kg") : "eV/history";
            else
                result.numberOfHistories = 0;
        }
        if (progressbar)
            progressbar->clearDoseData();
        for (auto* j : jobs)
            dxmc_gpu_job_free(j);
        dxmc_gpu_lut_free(lut);
        dxmc_lut_blob_free(blob);
        dxmc_gpu_world_free(dworld);
        if (!ok || cancelled) {
            std::fill(result.dose.begin(), result.dose.end(), T { 0 });
            std::fill(result.variance.begin(), result.variance.end(), T { 0 });
            std::fill(result.nEvents.begin(), result.nEvents.end(), 0u);
            result.numberOfHistories = 0;
            if (cancelled)
                m_error = "cancelled";
        }
        return result;
    }

    // Source::getCalibrationValue, with the CTDI calibration run of the CT sources
    // (CTBaseSource::ctCalibration, source.hpp:925-988) done by this GPU transport
    // instead of a second CPU transport; other sources keep their own (closed-form) value.
    T calibrationValue(Source<T>* source, ProgressBar<T>* progressbar = nullptr)
    {
        if (auto* spiral = dynamic_cast<CTSpiralSource<T>*>(source)) {
            CTAxialSource<T> copy(*spiral); // source.hpp:1358-1363
            return ctCalibration(copy) * spiral->pitch();
        }
        if (auto* axial = dynamic_cast<CTAxialSource<T>*>(source)) {
            CTAxialSource<T> copy(*axial); // source.hpp:1277-1281
            return ctCalibration(copy);
        }
        if (auto* sdual = dynamic_cast<CTSpiralDualSource<T>*>(source)) {
            CTAxialDualSource<T> copy(*sdual); // source.hpp:1576-1581, both tubes in the CTDI run
            return ctCalibration(copy) * sdual->pitch();
        }
        if (auto* adual = dynamic_cast<CTAxialDualSource<T>*>(source)) {
            CTAxialDualSource<T> copy(*adual); // source.hpp:1477-1481
            return ctCalibration(copy);
        }
        if (auto* topo = dynamic_cast<CTTopogramSource<T>*>(source)) {
            // CTTopogramSource::getCalibrationValue (source.hpp:1679-1701): an axial source
            // with the topogram's CT settings, stepping one collimation, CTDIvol scaled by
            // the scan length over the collimation, the angle step matched to the exposures
            CTAxialSource<T> copy;
            static_cast<CTBaseSource<T>&>(copy) = static_cast<const CTBaseSource<T>&>(*topo);
            copy.setCtdiVol(topo->ctdiVol() * topo->scanLenght() / topo->collimation());
            copy.setScanLenght(0);
            copy.setStep(topo->collimation());
            const T max_step = (2 * PI_VAL<T>()) / 72;
            const auto exposures = topo->totalExposures();
            copy.setExposureAngleStep(std::min(2 * PI_VAL<T>() / exposures, max_step));
            const T factor = ctCalibration(copy);
            return factor * exposures / copy.totalExposures();
        }
        return source->getCalibrationValue(m_model, progressbar);
    }

private:
    template <typename Axial>
    T ctCalibration(Axial& copy)
    {
        T meanWeight = 0;
        for (std::uint64_t i = 0; i < copy.totalExposures(); ++i)
            meanWeight += copy.getExposure(i).beamIntensityWeight();
        meanWeight /= copy.totalExposures();
        copy.setDirectionCosines(std::array<T, 6> { -1, 0, 0, 0, 0, 1 });
        copy.setPosition(std::array<T, 3> { 0, 0, 0 });
        copy.setScanLenght(copy.collimation());
        copy.setUseXCareFilter(false);
        std::size_t stat = CTDIPhantom<T>::ctdiMinHistories() / (copy.exposuresPerRotatition() * copy.historiesPerExposure());
        stat = std::max<std::size_t>(stat, 1);
        CTDIPhantom<T> world(copy.ctdiPhantomDiameter());
        copy.updateFromWorld(world);
        copy.setHistoriesPerExposure(copy.historiesPerExposure() * stat);
        copy.validate();
        const OUTPUTMODE mode = m_mode;
        m_mode = OUTPUTMODE::DOSE;
        auto result = (*this)(world, &copy, nullptr, false);
        m_mode = mode;
        if (result.numberOfHistories == 0)
            return T { 0 };
        using H = typename CTDIPhantom<T>::HolePosition;
        const H order[5] = { H::Center, H::West, H::East, H::South, H::North };
        T measured[5] {};
        for (int i = 0; i < 5; ++i) {
            const auto& idx = world.holeIndices(order[i]);
            for (auto v : idx)
                measured[i] += result.dose[v];
            measured[i] /= static_cast<T>(idx.size());
        }
        const T periphery = (measured[1] + measured[2] + measured[3] + measured[4]) / T { 4 };
        const T ctdiw = (measured[0] + 2 * periphery) / 3 * T { 100 } / copy.collimation();
        return copy.ctdiVol() / ctdiw / meanWeight;
    }

    bool ensure_context()
    {
        if (m_ctx)
            return true;
        const int rc = dxmc_gpu_ctx_create(&m_options, &m_ctx);
        if (rc != DXMC_OK) {
            m_ctx = nullptr;
            m_error = rc == DXMC_ERR_NO_DEVICE ? "no CUDA device available" : "context creation failed";
            return false;
        }
        return true;
    }
    bool check(int rc, const char* what)
    {
        if (rc == DXMC_OK)
            return true;
        m_error = std::string(what) + ": " + dxmc_gpu_last_error(m_ctx);
        return false;
    }
    void release()
    {
        if (m_ctx)
            dxmc_gpu_ctx_destroy(m_ctx);
        m_ctx = nullptr;
    }

    dxmc_gpu_ctx* m_ctx = nullptr;
    dxmc_gpu_options m_options {};
    std::uint64_t m_seed = 1;
    int m_tracking = DXMC_TRACKING_DEFAULT;
    int m_direction = DXMC_DIRECTION_REFERENCE;
    int m_precision = DXMC_PRECISION_FP32;
    std::pair<std::vector<T>, std::vector<T>> m_iso;
    std::string m_error;
    OUTPUTMODE m_mode = OUTPUTMODE::DOSE;                             // transport.hpp:838
    LOWENERGYCORRECTION m_model = LOWENERGYCORRECTION::LIVERMORE;     // transport.hpp:839
};

} // namespace dxmc::gpu
