// Host-side LUT build; see lut_builder.hpp for the reference functions each
// part restates.
#include "lut_builder.hpp"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <thread>
#include <limits>
#include <numeric>

namespace dxmc_gb300::host {

std::vector<double> MaterialData::edges(double minEnergy) const
{
    std::vector<double> out(64);
    int n = p->binding_energies(p->user, minEnergy, out.data(), static_cast<int>(out.size()));
    if (n > static_cast<int>(out.size())) {
        out.resize(n);
        n = p->binding_energies(p->user, minEnergy, out.data(), n);
    }
    out.resize(std::max(n, 0));
    return out;
}

std::array<dxmc_shell_config, 12> MaterialData::shells() const
{
    std::array<dxmc_shell_config, 12> s {};
    p->shells(p->user, s.data());
    return s;
}

namespace {

    // Composite Simpson rule on 50 intervals (dxmcrandom.hpp:341-350).
    double simpson50(double start, double stop, const std::function<double(double)>& pdf)
    {
        const double h = (stop - start) / 50;
        double result = pdf(start) + pdf(stop);
        for (std::size_t i = 1; i < 50; ++i) {
            const double prod = i % 2 == 0 ? 2 : 4;
            result += prod * pdf(start + h * i);
        }
        return h * result / 3;
    }

    struct RitaNode {
        double x, e, a, b, error;
    };

    // Thomas elimination for the spline system (interpolation.hpp:93-122).
    std::vector<double> thomas(const std::vector<double>& h, std::vector<double> H, std::vector<double> d)
    {
        const std::size_t n = d.size();
        for (std::size_t i = 1; i < n; ++i) {
            const double w = h[i - 1] / H[i - 1];
            H[i] -= w * h[i - 1];
            d[i] -= w * d[i - 1];
        }
        std::vector<double> x(n);
        x[n - 1] = d[n - 1] / H[n - 1];
        for (int i = static_cast<int>(n) - 2; i >= 0; --i)
            x[i] = (d[i] - h[i] * x[i + 1]) / H[i];
        return x;
    }

    double momentum_transfer_max(double energy)
    {
        constexpr double k = 1 / KEV_TO_ANGSTROM;
        return energy * k;
    }

} // namespace

void build_rita(double min, double max, const std::function<double(double)>& pdf, int N, double* xo, double* eo, double* ao, double* bo)
{
    std::size_t n = 10;
    std::vector<RitaNode> v(n);
    v.reserve(N);
    for (std::size_t i = 0; i < n; ++i) {
        v[i].x = min + i * (max - min) / (n - 1);
        v[i].e = 0;
        v[i].a = 0;
        v[i].b = 0;
        v[i].error = -1;
    }
    auto integrate = [&]() {
        for (std::size_t j = 1; j < n; ++j)
            v[j].e = v[j - 1].e + simpson50(v[j - 1].x, v[j].x, pdf);
    };
    integrate();
    const double pdf_scale = v[n - 1].e; // normalisation of the first pass, kept fixed
    for (std::size_t j = 1; j < n; ++j)
        v[j].e = v[j].e / v[n - 1].e;

    while (n != static_cast<std::size_t>(N)) {
        for (std::size_t i = 0; i + 1 < n; ++i) {
            if (v[i].error >= 0)
                continue;
            const double dx = v[i + 1].x - v[i].x;
            const double slope = (v[i + 1].e - v[i].e) / dx;
            const double p0 = pdf(v[i].x) / pdf_scale;
            const double p1 = pdf(v[i + 1].x) / pdf_scale;
            v[i].b = (p0 > 0 && p1 > 0) ? 1 - slope * slope / (p0 * p1) : 0;
            v[i].a = p0 > 0 ? slope / p0 - v[i].b - 1 : 0;
            // L1 distance between the rational approximation and the pdf
            v[i].error = 0;
            const double a = v[i].a, b = v[i].b;
            for (std::size_t j = 1; j < 50; ++j) {
                const double x = v[i].x + j * (v[i + 1].x - v[i].x) / 50;
                const double t = (x - v[i].x) / (v[i + 1].x - v[i].x);
                const double f = (1 + a + b - a * t);
                const double nu = f * (1 - std::sqrt(1 - 4 * b * t * t / (f * f))) / (2 * b * t);
                const double q = (1 + a * nu + b * nu * nu);
                const double approx = q * q * (v[i + 1].e - v[i].e) / ((1 + a + b) * (1 - b * nu * nu) * (v[i + 1].x - v[i].x));
                v[i].error += std::abs(approx - pdf(x)) * (v[i + 1].x - v[i].x) / 50;
            }
        }
        auto worst = std::max_element(v.begin(), v.end(), [](const RitaNode& l, const RitaNode& r) { return l.error < r.error; });
        const double x0 = worst->x;
        worst->error = -1;
        ++worst;
        const double x1 = worst->x;
        v.insert(worst, RitaNode { x0 + (x1 - x0) / 2, 0, 0, 0, -1 });
        ++n;
        integrate();
        for (std::size_t j = 1; j < n; ++j)
            v[j].e = v[j].e / v[n - 1].e;
    }
    for (int i = 0; i < N; ++i) {
        xo[i] = v[i].x;
        eo[i] = v[i].e;
        ao[i] = v[i].a;
        bo[i] = v[i].b;
    }
}

void build_spline(double start, double stop, const std::function<double(double)>& f, int N, double* coef, double* knots, double& step, double& stop_out)
{
    std::vector<double> x(N), y(N);
    step = (stop - start) / (N - 2);
    for (int i = 0; i < N; ++i) {
        x[i] = start + step * i;
        y[i] = f(x[i]);
    }
    stop_out = x.back();
    std::vector<double> h(N, 0.0);
    for (int i = 0; i < N - 1; ++i)
        h[i] = x[i + 1] - x[i];
    std::vector<double> delta(N, 1.0);
    for (int i = 0; i < N - 1; ++i)
        delta[i] = (y[i + 1] - y[i]) / h[i];
    std::vector<double> H(N, 0.0);
    for (int i = 1; i < N; ++i)
        H[i] = 2 * (h[i - 1] + h[i]);
    H[0] = H[1];
    std::vector<double> d(N, 0.0);
    for (int i = 1; i < N; ++i)
        d[i] = 6 * (delta[i] - delta[i - 1]);
    d[N - 1] = 0;
    d[0] = 0;
    const auto s = thomas(h, H, d);
    for (int i = 0; i < N - 1; ++i) {
        double* c = coef + i * 4;
        c[0] = (s[i] * x[i + 1] * x[i + 1] * x[i + 1] - s[i + 1] * x[i] * x[i] * x[i] + 6 * (y[i] * x[i + 1] - y[i + 1] * x[i])) / (6 * h[i]);
        c[0] += h[i] * (s[i + 1] * x[i] - s[i] * x[i + 1]) / 6;
        c[1] = (s[i + 1] * x[i] * x[i] - s[i] * x[i + 1] * x[i + 1] + 2 * (y[i + 1] - y[i])) / (2 * h[i]) + h[i] * (s[i] - s[i + 1]) / 6;
        c[2] = (s[i] * x[i + 1] - s[i + 1] * x[i]) / (2 * h[i]);
        c[3] = (s[i + 1] - s[i]) / (6 * h[i]);
    }
    for (int i = 0; i < N; ++i)
        knots[i] = x[i];
}

void build_alias_table(const std::vector<double>& weights, std::vector<double>& probs, std::vector<std::uint64_t>& alias)
{
    const std::size_t n = weights.size();
    probs.assign(n, 0.0);
    alias.assign(n, 0);
    std::vector<double> scaled(n);
    std::vector<std::int64_t> large(n), small(n);
    std::int64_t ns = 0, nl = 0;
    const double sum = std::accumulate(weights.begin(), weights.end(), 0.0);
    const double scale = n / sum;
    for (std::size_t i = 0; i < n; ++i)
        scaled[i] = weights[i] * scale;
    for (std::int64_t i = static_cast<std::int64_t>(n) - 1; i >= 0; --i) {
        if (scaled[i] < 1.0)
            small[ns++] = i;
        else
            large[nl++] = i;
    }
    while (ns && nl) {
        const auto s = small[--ns];
        const auto l = large[--nl];
        probs[s] = scaled[s];
        alias[s] = static_cast<std::uint64_t>(l);
        scaled[l] = scaled[l] + scaled[s] - 1;
        if (scaled[l] < 1)
            small[ns++] = l;
        else
            large[nl++] = l;
    }
    while (nl)
        probs[large[--nl]] = 1;
    while (ns)
        probs[small[--ns]] = 1;
}

std::array<double, 3> lut_attenuation(const dxmc_lut_blob& b, int material, double energy)
{
    std::array<double, 3> res {};
    const std::size_t R = b.resolution();
    const double logE = std::log10(energy);
    std::size_t index;
    if (logE > b.linear_energy) {
        index = std::min(static_cast<std::size_t>((logE - b.linear_energy) / b.linear_step) + b.linear_index, R - 1);
    } else {
        const auto pos = std::upper_bound(b.log_energy.begin(), b.log_energy.end(), logE);
        index = pos != b.log_energy.end() ? static_cast<std::size_t>(pos - b.log_energy.begin()) : R - 1;
    }
    const std::size_t off = static_cast<std::size_t>(material) * R * 6 + index * 6;
    for (int i = 0; i < 3; ++i)
        res[i] = std::pow(10.0, b.coefficients[off + 2 * i] + b.coefficients[off + 2 * i + 1] * logE);
    return res;
}

double lut_max_inverse(const dxmc_lut_blob& b, double energy)
{
    const std::size_t R = b.resolution();
    const double logE = std::log10(energy);
    std::size_t index;
    if (logE > b.linear_energy) {
        // The reference leaves this index unclamped (attenuationinterpolator.hpp:511);
        // it stays below R for every energy up to the table maximum.
        index = std::min(static_cast<std::size_t>((logE - b.linear_energy) / b.linear_step) + b.linear_index, R - 1);
    } else {
        const auto pos = std::upper_bound(b.log_energy.begin(), b.log_energy.end(), logE);
        index = pos != b.log_energy.end() ? static_cast<std::size_t>(pos - b.log_energy.begin()) : R - 1;
    }
    return std::pow(10.0, b.max_coefficients[2 * index] + b.max_coefficients[2 * index + 1] * logE);
}

double lut_scatter_factor(const dxmc_lut_blob& b, int material, double q)
{
    const auto& sp = b.spline[material];
    const double start = sp[76], step = sp[77], stop = sp[78];
    const double x = std::clamp(q, start, stop);
    const std::size_t index = x > start ? static_cast<std::size_t>((x - start) / step) : 0;
    const std::size_t off = index < SPLINE_N - 1 ? index * 4 : (SPLINE_N - 2) * 4;
    return sp[off] + sp[off + 1] * x + sp[off + 2] * x * x + sp[off + 3] * x * x * x;
}

double rita_value(const dxmc_lut_blob& b, int material, double xi)
{
    const auto& r = b.rita[material];
    const double* x = r.data();
    const double* e = x + RITA_N;
    const double* a = e + RITA_N;
    const double* bb = a + RITA_N;
    int i = static_cast<int>(std::upper_bound(e, e + RITA_N, xi) - e) - 1;
    i = std::clamp(i, 0, RITA_N - 2);
    const double v = xi - e[i];
    const double d = e[i + 1] - e[i];
    return x[i] + (1.0 + a[i] + bb[i]) * d * v / (d * d + a[i] * d * v + bb[i] * v * v) * (x[i + 1] - x[i]);
}

namespace {

// Quantiles at levels k / nu (k = 0..nu) of the density w on [lo, hi] (trapezoid
// cumulative on M intervals, linear inversion); returns them mapped by `store`.
void quantiles(double lo, double hi, const std::function<double(double)>& w, int nu, const std::function<double(double)>& store,
    float* out)
{
    constexpr int M = 2048;
    std::vector<double> G(M + 1, 0.0);
    const double h = (hi - lo) / M;
    double prev = std::max(w(lo), 0.0);
    for (int j = 1; j <= M; ++j) {
        const double cur = std::max(w(lo + j * h), 0.0);
        G[j] = G[j - 1] + 0.5 * (prev + cur) * h;
        prev = cur;
    }
    const double total = G[M];
    int j = 0;
    for (int k = 0; k <= nu; ++k) {
        double x;
        if (!(total > 0)) {
            x = lo + (hi - lo) * k / nu; // flat: uniform
        } else {
            const double target = total * k / nu;
            while (j < M - 1 && G[j + 1] < target)
                ++j;
            const double dg = G[j + 1] - G[j];
            const double f = dg > 0 ? std::clamp((target - G[j]) / dg, 0.0, 1.0) : 0.0;
            x = lo + (j + f) * h;
        }
        out[k] = static_cast<float>(store(std::clamp(x, lo, hi)));
    }
}

} // namespace

void build_sampling_tables(const dxmc_lut_blob& b, int ne, int nu, SamplingTables& out)
{
    const int nm = b.n_materials;
    out.ne = ne;
    out.nu = nu;
    out.le0 = std::log(b.min_energy);
    out.dle = (std::log(b.max_energy) - out.le0) / (ne - 1);
    const size_t row = static_cast<size_t>(nu) + 1;
    out.compton_kn.assign(static_cast<size_t>(ne) * row, 0.0f);
    out.compton_sf.assign(static_cast<size_t>(nm) * ne * row, 0.0f);
    out.rayleigh.assign(static_cast<size_t>(nm) * ne * row, 0.0f);
    // rows are independent: spread the energies over the host cores
    auto build_row = [&](int i) {
        const double E = std::exp(out.le0 + i * out.dle);
        const double k = E / ELECTRON_REST_MASS;
        const double emin = 1.0 / (1.0 + 2.0 * k);
        const double qscale = E / KEV_TO_ANGSTROM; // q = qscale * sqrt((1 - cos) / 2)
        auto kn = [=](double e) {
            const double t = (1.0 - e) / (k * e);
            return 1.0 / e + e - t * (2.0 - t);
        };
        auto q_of = [=](double e) {
            const double cos = 1.0 - (1.0 - e) / (k * e);
            return qscale * std::sqrt(std::max(0.5 - 0.5 * cos, 0.0));
        };
        auto to_x = [=](double e) { return (e - emin) / (1.0 - emin); };
        quantiles(emin, 1.0, kn, nu, to_x, out.compton_kn.data() + i * row);
        const double qmax2 = qscale * qscale;
        for (int m = 0; m < nm; ++m) {
            quantiles(emin, 1.0, [&](double e) { return kn(e) * lut_scatter_factor(b, m, q_of(e)); }, nu, to_x,
                out.compton_sf.data() + (static_cast<size_t>(m) * ne + i) * row);
            // RITA restricted to q^2 <= qmax^2 (rita_sample: the proposal stops at e[ub] and
            // draws above qmax^2 are rejected): find xi* with x(xi*) = qmax^2
            const double* xs = b.rita[m].data();
            const double* es = xs + RITA_N;
            const int ub = static_cast<int>(std::upper_bound(xs, xs + RITA_N, qmax2) - xs);
            double hi = ub < RITA_N ? es[ub] : 1.0;
            if (rita_value(b, m, hi) > qmax2) {
                double lo = 0.0;
                for (int it = 0; it < 80; ++it) {
                    const double mid = 0.5 * (lo + hi);
                    (rita_value(b, m, mid) > qmax2 ? hi : lo) = mid;
                }
                hi = lo;
            }
            auto w = [&](double xi) {
                const double cos = 1.0 - 2.0 * rita_value(b, m, xi) / qmax2;
                return 0.5 * (1.0 + cos * cos);
            };
            auto to_y = [&](double xi) { return std::clamp(rita_value(b, m, xi) / qmax2, 0.0, 1.0); };
            quantiles(0.0, hi, w, nu, to_y, out.rayleigh.data() + (static_cast<size_t>(m) * ne + i) * row);
        }
    };
    const int workers = std::clamp(static_cast<int>(std::thread::hardware_concurrency()), 1, 32);
    std::atomic<int> next { 0 };
    std::vector<std::thread> pool;
    for (int t = 0; t < workers; ++t)
        pool.emplace_back([&] {
            for (int i = next++; i < ne; i = next++)
                build_row(i);
        });
    for (auto& th : pool)
        th.join();
}

std::shared_ptr<const SamplingTables> sampling_tables(const dxmc_lut_blob& b, int ne, int nu)
{
    std::lock_guard<std::mutex> lock(*b.tables_mutex);
    auto cached = std::static_pointer_cast<const SamplingTables>(b.tables);
    if (cached && cached->ne == ne && cached->nu == nu)
        return cached;
    auto t = std::make_shared<SamplingTables>();
    build_sampling_tables(b, ne, nu, *t);
    b.tables = t;
    return t;
}

int build_lut(const std::vector<MaterialData>& materials, const std::vector<double>& max_density, double max_energy, dxmc_lut_blob& out)
{
    const int nm = static_cast<int>(materials.size());
    if (nm <= 0 || static_cast<int>(max_density.size()) != nm || !(max_energy > 0))
        return DXMC_ERR_INVALID;
    dxmc_lut_blob b;
    b.n_materials = nm;
    b.max_density = max_density;
    // AttenuationLut::generate(materials, maxEnergy, minEnergy = 1), attenuationlut.hpp:82-83
    const double minEnergyArg = 1.0;
    b.min_energy = std::max(0.5, std::min(max_energy, minEnergyArg));
    b.max_energy = std::min(2 * ELECTRON_REST_MASS, std::max(max_energy, minEnergyArg));

    // Form-factor RITA tables (attenuationlut.hpp:212-233)
    b.rita.resize(nm);
    {
        const double qmax = momentum_transfer_max(b.max_energy);
        const double qmax_squared = qmax * qmax;
        for (int m = 0; m < nm; ++m) {
            const auto& mat = materials[m];
            double q_app = 1;
            double ff = mat.ff2(q_app);
            while (q_app < qmax_squared && ff > 0.001) {
                if (ff > 0.5)
                    q_app += 0.5;
                else
                    q_app += 0.1;
                ff = mat.ff2(q_app);
            }
            auto& r = b.rita[m];
            build_rita(0, q_app, [&](double q2) { return mat.ff2(std::sqrt(q2)); }, RITA_N, r.data(), r.data() + 56, r.data() + 112, r.data() + 168);
        }
    }
    // Compton scatter-factor splines (attenuationlut.hpp:240-265)
    b.spline.resize(nm);
    {
        const double qmax_energy = momentum_transfer_max(b.max_energy);
        for (int m = 0; m < nm; ++m) {
            const auto& mat = materials[m];
            double q_app = 0.5;
            double sf = mat.sf(q_app);
            while (sf < 0.999 && q_app < qmax_energy) {
                sf = mat.sf(q_app);
                if (sf < 0.5)
                    q_app += 0.5;
                else
                    q_app += 0.1;
            }
            auto& sp = b.spline[m];
            double step = 0, stop = 0;
            build_spline(0, q_app, [&](double q) { return mat.sf(q); }, SPLINE_N, sp.data(), sp.data() + 60, step, stop);
            sp[76] = 0;
            sp[77] = step;
            sp[78] = stop;
        }
    }
    // Electron shells (attenuationlut.hpp:89-92)
    b.shells.resize(nm);
    for (int m = 0; m < nm; ++m)
        b.shells[m] = materials[m].shells();

    // Interpolation tables (attenuationinterpolator.hpp:88-97, 119-205)
    const double minE = std::max(0.1, b.min_energy);
    const double maxE = std::max(b.max_energy, 50.0);
    std::size_t resolution = std::max(static_cast<std::size_t>(maxE - minE), std::size_t { 10 });
    const double logMin = std::log10(minE);
    const double logMax = std::log10(maxE);
    constexpr double shell_offset = 0.001;
    std::vector<double> edges;
    for (const auto& mat : materials)
        for (const double e : mat.edges(minE)) {
            edges.push_back(std::log10(e - shell_offset));
            edges.push_back(std::log10(e));
        }
    std::sort(edges.begin(), edges.end());
    edges.erase(std::unique(edges.begin(), edges.end()), edges.end());
    std::vector<double> x;
    x.reserve(resolution + 1 + edges.size());
    for (std::size_t i = 0; i <= resolution; ++i)
        x.push_back(logMin + (i * (logMax - logMin)) / (resolution));
    for (const double e : edges)
        x.push_back(e);
    std::sort(x.begin(), x.end());
    x.erase(std::unique(x.begin(), x.end()), x.end());

    const std::size_t nseg = x.size() - 1;
    b.coefficients.assign(static_cast<std::size_t>(nm) * nseg * 6, 0.0);
    for (int m = 0; m < nm; ++m) {
        for (int type = 0; type < 3; ++type) {
            std::vector<double> y(x.size());
            for (std::size_t i = 0; i < x.size(); ++i) {
                const double e = std::pow(10.0, x[i]);
                const double mu = type == 0 ? materials[m].photo(e) : (type == 1 ? materials[m].compton(e) : materials[m].rayleigh(e));
                y[i] = std::log10(mu);
            }
            for (std::size_t i = 0; i + 1 < x.size(); ++i) {
                const std::size_t off = m * nseg * 6 + type * 2 + i * 6;
                const double w = (y[i + 1] - y[i]) / (x[i + 1] - x[i]);
                b.coefficients[off] = y[i] - x[i] * w;
                b.coefficients[off + 1] = w;
            }
        }
    }
    const double firstNode = x.front();
    x.erase(x.begin());
    if (!edges.empty()) {
        const auto pos = std::upper_bound(x.begin(), x.end(), edges.back());
        if (pos == x.end()) {
            b.linear_index = x.size();
            b.linear_step = x[x.size() - 1] - x[x.size() - 2];
            b.linear_energy = x.back();
        } else {
            b.linear_index = static_cast<std::size_t>(pos - x.begin());
            // The reference reads x[index + 1] here; at the last node that is past
            // the end, so the previous spacing is used instead.
            b.linear_step = b.linear_index + 1 < x.size() ? x[b.linear_index + 1] - x[b.linear_index] : x[b.linear_index] - x[b.linear_index - 1];
            b.linear_energy = x[b.linear_index];
        }
    } else {
        b.linear_index = 0;
        b.linear_step = x[1] - x[0];
        b.linear_energy = x.front();
    }
    b.log_energy = x;

    // Majorant table (attenuationinterpolator.hpp:48-84)
    std::vector<double> xm = x;
    xm.insert(xm.begin(), firstNode);
    std::vector<double> ym(xm.size());
    for (std::size_t k = 0; k < xm.size(); ++k) {
        double maxVal = 0;
        for (int m = 0; m < nm; ++m) {
            const auto vals = lut_attenuation(b, m, std::pow(10.0, xm[k]));
            const double val = max_density[m] * (0.0 + vals[0] + vals[1] + vals[2]);
            maxVal = std::max(maxVal, val);
        }
        ym[k] = std::log10(1 / maxVal);
    }
    b.max_coefficients.assign(x.size() * 2, 0.0);
    for (std::size_t i = 0; i + 1 < xm.size(); ++i) {
        const double w = (ym[i + 1] - ym[i]) / (xm[i + 1] - xm[i]);
        b.max_coefficients[2 * i] = ym[i] - xm[i] * w;
        b.max_coefficients[2 * i + 1] = w;
    }
    out = std::move(b);
    return DXMC_OK;
}

} // namespace dxmc_gb300::host
