// Compiles DXMClib's unmodified headers together with include/dxmc_gpu/transport.hpp
// and checks the adapter on the host: exposure flattening, the LUT built through
// the Material provider against DXMClib's own AttenuationLut, and the zero-Result
// error convention when no GPU is present.  Prints one line per check.
#include "std_reduce_shim.hpp" // oracle/: lets the reference's BowTieFilter compile with GCC 13

#include "dxmc_gpu/transport.hpp"

#include <cmath>
#include <cstdio>
#include <memory>

using namespace dxmc;

int main()
{
    int failures = 0;
    World<double> world;
    world.setDimensions({ 24, 20, 16 });
    world.setSpacing({ 2.0, 2.0, 2.5 });
    const std::size_t n = world.size();
    auto dens = std::make_shared<std::vector<double>>(n);
    auto mat = std::make_shared<std::vector<std::uint8_t>>(n);
    for (std::size_t i = 0; i < n; ++i) {
        (*mat)[i] = static_cast<std::uint8_t>(i % 3);
        // densities on a 1/64 grid are exact in float, like the f32 density the GPU stores
        (*dens)[i] = (i % 3 == 0) ? 1.0 : ((i % 3 == 1) ? std::round(64 * 1.92 * (0.5 + (i % 7) / 7.0)) / 64 : 0.25);
    }
    world.setDensityArray(dens);
    world.setMaterialIndexArray(mat);
    world.addMaterialToMap(Material("Water, Liquid"));
    world.addMaterialToMap(Material("Bone, Cortical (ICRP)"));
    world.addMaterialToMap(Material("Lung Tissue (ICRU-44)"));
    world.makeValid();
    if (!world.isValid()) {
        std::printf("FAIL world\n");
        return 1;
    }

    // 1) flattening of a CT spiral source matches getExposure + alignToDirectionCosines
    CTSpiralSource<double> ct;
    ct.setCollimation(20);
    ct.setScanLenght(30);
    ct.setPitch(1.2);
    ct.setGantryTiltAngleDeg(5);
    ct.setHistoriesPerExposure(10);
    ct.validate();
    gpu::FlatSource<double> flat;
    if (!gpu::flatten<double>(world, &ct, flat)) {
        std::printf("FAIL flatten\n");
        return 1;
    }
    double maxdiff = 0;
    for (std::uint64_t i = 0; i < ct.totalExposures(); ++i) {
        auto e = ct.getExposure(i);
        e.alignToDirectionCosines(world.directionCosines());
        for (int k = 0; k < 3; ++k)
            maxdiff = std::max(maxdiff, std::abs(e.position()[k] - flat.exposures[i].position[k]));
        for (int k = 0; k < 4; ++k)
            maxdiff = std::max(maxdiff, std::abs(e.collimationAngles()[k] - flat.exposures[i].collimation[k]));
    }
    const bool flat_ok = maxdiff == 0 && flat.exposures.size() == ct.totalExposures() && flat.has_heel && !flat.spec_energies.empty();
    std::printf("%s flatten exposures=%zu maxdiff=%g heel=%d spectrum=%zu\n", flat_ok ? "OK" : "FAIL", flat.exposures.size(), maxdiff,
        flat.has_heel ? 1 : 0, flat.spec_energies.size());
    failures += !flat_ok;

    // 1b) a dual-source scanner flattens into two beams: the even exposures with tube
    // A's spectrum and heel table, the odd ones with tube B's (CTDualSource)
    {
        CTSpiralDualSource<double> dual;
        dual.setCollimation(20);
        dual.setScanLenght(30);
        dual.tubeB().setVoltage(80);
        dual.tubeB().setAlFiltration(6.0);
        dual.setTubeBmas(250);
        dual.setModelHeelEffect(false); // the dual source builds its heel tables regardless
        dual.setHistoriesPerExposure(10);
        dual.validate();
        std::vector<gpu::FlatSource<double>> beams;
        bool dual_ok = gpu::flatten_beams<double>(world, &dual, beams) && beams.size() == 2;
        double dmax = 0;
        for (std::uint64_t i = 0; dual_ok && i < dual.totalExposures(); ++i) {
            auto e = dual.getExposure(i);
            e.alignToDirectionCosines(world.directionCosines());
            const auto& f = beams[i % 2].exposures[i / 2];
            for (int k = 0; k < 3; ++k)
                dmax = std::max(dmax, std::abs(e.position()[k] - f.position[k]));
            dmax = std::max(dmax, std::abs(e.beamIntensityWeight() - f.weight));
        }
        const auto eb = dual.tubeB().getEnergy();
        const auto wb = dual.tubeB().getSpecter(eb);
        dual_ok = dual_ok && dmax == 0 && beams[0].exposures.size() + beams[1].exposures.size() == dual.totalExposures()
            && beams[0].has_heel && beams[1].has_heel && beams[1].spec_energies.size() == eb.size()
            && beams[1].spec_weights == std::vector<double>(wb.begin(), wb.end())
            && beams[0].spec_energies.size() == dual.tube().getEnergy().size()
            && beams[1].heel.energy_size < beams[0].heel.energy_size;
        std::printf("%s dual-source beams=%zu exposures=%zu+%zu maxdiff=%g\n", dual_ok ? "OK" : "FAIL", beams.size(),
            beams.size() > 0 ? beams[0].exposures.size() : 0, beams.size() > 1 ? beams[1].exposures.size() : 0, dmax);
        failures += !dual_ok;
        std::vector<gpu::FlatSource<double>> single;
        const bool single_ok = gpu::flatten_beams<double>(world, &ct, single) && single.size() == 1
            && single[0].exposures.size() == ct.totalExposures();
        std::printf("%s single-source beams=%zu\n", single_ok ? "OK" : "FAIL", single.size());
        failures += !single_ok;
        // a bow-tie filter travels as the filter's own table (BowTieFilter::data(),
        // beamfilters.hpp:196), which the jobs' table build leaves as it is
        const std::vector<double> bta { 0.2, 0.0, -0.06, 0.1, 0.4 }, btw { 0.6, 1.0, 0.95, 0.8, 0.2 };
        ct.setBowTieFilter(std::make_shared<BowTieFilter<double>>(bta, btw));
        std::vector<gpu::FlatSource<double>> with_bt;
        bool bt_ok = gpu::flatten_beams<double>(world, &ct, with_bt) && with_bt.size() == 1;
        const auto& data = ct.bowTieFilter()->data();
        bt_ok = bt_ok && with_bt[0].bowtie_angles.size() == data.size() && with_bt[0].bowtie_weights.size() == data.size();
        double bt_diff = 0;
        if (bt_ok) {
            std::vector<double> ta(data.size()), tw(data.size());
            bt_ok = dxmc_bowtie_table(with_bt[0].bowtie_angles.data(), with_bt[0].bowtie_weights.data(),
                        static_cast<int>(data.size()), ta.data(), tw.data())
                == DXMC_OK;
            for (std::size_t i = 0; i < data.size() && bt_ok; ++i) {
                bt_ok = with_bt[0].bowtie_angles[i] == data[i].first && with_bt[0].bowtie_weights[i] == data[i].second
                    && ta[i] == data[i].first;
                bt_diff = std::max(bt_diff, std::abs(tw[i] - data[i].second));
            }
        }
        bt_ok = bt_ok && bt_diff < 1e-15;
        std::printf("%s bow-tie table n=%zu maxdiff=%g\n", bt_ok ? "OK" : "FAIL", data.size(), bt_diff);
        failures += !bt_ok;
        ct.setBowTieFilter(nullptr);
    }

    // 2) LUT through the provider == DXMClib's AttenuationLut on the same Material objects
    AttenuationLut<double> ref;
    ref.generate(world, 90.0);
    std::vector<dxmc_material_provider> prov;
    for (const auto& m : world.materialMap())
        prov.push_back(gpu::detail::provider(m));
    std::vector<float> fd(dens->begin(), dens->end());
    dxmc_lut_blob* blob = nullptr;
    const int rc = dxmc_lut_build(prov.data(), 3, fd.data(), mat->data(), n, 90.0, &blob);
    double worst = 0;
    for (int m = 0; m < 3 && rc == 0; ++m) {
        for (double e = 1.0; e <= 90.0; e += 0.37) {
            double att[3];
            dxmc_lut_attenuation(blob, m, e, att);
            const auto r = ref.photoComptRayAttenuation(m, e);
            for (int k = 0; k < 3; ++k)
                worst = std::max(worst, std::abs(att[k] / r[k] - 1));
            worst = std::max(worst, std::abs(dxmc_lut_max_attenuation_inverse(blob, e) / ref.maxTotalAttenuationInverse(e) - 1));
        }
        for (double q = 0; q < 8; q += 0.05)
            worst = std::max(worst, std::abs(dxmc_lut_scatter_factor(blob, m, q) - ref.comptonScatterFactor(m, q)));
    }
    const bool lut_ok = rc == 0 && worst < 1e-12;
    std::printf("%s lut rc=%d worst_rel=%g\n", lut_ok ? "OK" : "FAIL", rc, worst);
    failures += !lut_ok;
    dxmc_lut_blob_free(blob);

    // 3) without a GPU the adapter keeps the reference's zero-Result convention
    if (dxmc_gpu_device_count() == 0) {
        gpu::Transport<double> t;
        t.setOutputMode(gpu::Transport<double>::OUTPUTMODE::EV_PER_HISTORY);
        auto res = t(world, &ct);
        double sum = 0;
        for (auto d : res.dose)
            sum += d;
        const bool nogpu_ok = res.numberOfHistories == 0 && sum == 0 && res.dose.size() == n && !t.lastError().empty();
        std::printf("%s no-device result histories=%llu error='%s'\n", nogpu_ok ? "OK" : "FAIL",
            static_cast<unsigned long long>(res.numberOfHistories), t.lastError().c_str());
        failures += !nogpu_ok;
    }
    // 4) the GPU-only choices default to the reference's behaviour and round-trip
    {
        gpu::Transport<double> t;
        bool opt_ok = t.tracking() == DXMC_TRACKING_DEFAULT && t.directionMode() == DXMC_DIRECTION_REFERENCE;
        t.setTracking(DXMC_TRACKING_GLOBAL);
        t.setDirectionMode(DXMC_DIRECTION_NORMALIZED);
        opt_ok = opt_ok && t.tracking() == DXMC_TRACKING_GLOBAL && t.directionMode() == DXMC_DIRECTION_NORMALIZED;
        std::printf("%s options tracking=%d direction=%d\n", opt_ok ? "OK" : "FAIL", t.tracking(), t.directionMode());
        failures += !opt_ok;
    }
    return failures;
}
