// dxmc_gpu_transport_noalloc: the transport job without any allocation.
//
// Some callers cannot allocate device memory while they run a dose
// calculation: code that runs inside a memory pool or arena handed out by a
// host application (a treatment-planning or imaging pipeline that owns the
// whole device budget), real-time loops that must not hit the allocator, and
// embedding environments that forbid cudaMalloc after start-up.  For them this
// entry point runs the same transport kernel as dxmc_gpu_job_submit, but every
// byte of scratch the job needs (the work-queue head and counters, the packed
// exposure table, the history prefix sums, the spectrum alias table and the
// heel / bow-tie tables) lives in one file-scope __device__ array of fixed
// size.  The caller passes the resident world and LUT (inputs it created
// earlier) and its own device buffers for the tallies (outputs).
//
// Limits: at most NOALLOC_MAX_EXPOSURES exposures, NOALLOC_MAX_SPECTRUM
// spectrum bins, NOALLOC_MAX_HEEL heel weights and NOALLOC_MAX_BOWTIE bow-tie
// points; larger jobs are rejected with DXMC_ERR_INVALID and a message.  The
// array (about 2.2 MB) stays resident on every device that loads the library
// until the process exits.  All calls share it: calls that overlap on the GPU
// race with each other, so issue them one at a time.  dxmc_gpu_ctx_create
// loads this file's module and the transport kernels' modules on its device
// (CUDA loads modules lazily, and loading one allocates device memory) and looks
// up the array's device address (cudaGetSymbolAddress) with that device current,
// so a caller that creates its context before it fills the device meets no
// allocation in its first call; a first call on a device whose context skipped
// that step does the look-up itself and should come before any stream capture.
// Local-majorant
// tracking uses the (world, LUT) grid only if it was built before
// (dxmc_gpu_world_prepare, or an earlier job on the pair); otherwise the call
// tracks with the global majorant.
#include "dxmc_gpu.h"

#include "../kernels/transport.cuh"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

using namespace dxmc_gb300;

namespace {

constexpr uint64_t NOALLOC_MAX_EXPOSURES = 8192;
constexpr int NOALLOC_MAX_SPECTRUM = 2048;
constexpr int NOALLOC_MAX_HEEL = 8192;
constexpr int NOALLOC_MAX_BOWTIE = 1024;
constexpr int NOALLOC_MAX_DEVICES = 64;

constexpr size_t align256(size_t v) { return (v + 255) / 256 * 256; }

// Byte layout of the scratch array.
constexpr size_t OFF_COUNTERS = 0;
constexpr size_t OFF_RAW_EXPOSURES = align256(OFF_COUNTERS + sizeof(dev::JobCounters));
constexpr size_t OFF_EXPOSURES = align256(OFF_RAW_EXPOSURES + NOALLOC_MAX_EXPOSURES * sizeof(dxmc_exposure));
constexpr size_t OFF_OFFSETS = align256(OFF_EXPOSURES + NOALLOC_MAX_EXPOSURES * sizeof(dev::DevExposure));
constexpr size_t OFF_SPEC_RAW = align256(OFF_OFFSETS + (NOALLOC_MAX_EXPOSURES + 1) * sizeof(uint64_t));
constexpr size_t OFF_SPEC_E = align256(OFF_SPEC_RAW + 2 * NOALLOC_MAX_SPECTRUM * sizeof(double));
constexpr size_t OFF_SPEC_P = align256(OFF_SPEC_E + NOALLOC_MAX_SPECTRUM * sizeof(float));
constexpr size_t OFF_SPEC_A = align256(OFF_SPEC_P + NOALLOC_MAX_SPECTRUM * sizeof(float));
constexpr size_t OFF_SPEC_WORK = align256(OFF_SPEC_A + NOALLOC_MAX_SPECTRUM * sizeof(uint32_t));
constexpr size_t OFF_HEEL_RAW = align256(OFF_SPEC_WORK + NOALLOC_MAX_SPECTRUM * (sizeof(double) + 2 * sizeof(int32_t)));
constexpr size_t OFF_HEEL = align256(OFF_HEEL_RAW + NOALLOC_MAX_HEEL * sizeof(double));
constexpr size_t OFF_BOWTIE_RAW = align256(OFF_HEEL + NOALLOC_MAX_HEEL * sizeof(float));
constexpr size_t OFF_BOWTIE_A = align256(OFF_BOWTIE_RAW + 2 * NOALLOC_MAX_BOWTIE * sizeof(double));
constexpr size_t OFF_BOWTIE_W = align256(OFF_BOWTIE_A + NOALLOC_MAX_BOWTIE * sizeof(float));
constexpr size_t NOALLOC_SCRATCH_BYTES = align256(OFF_BOWTIE_W + NOALLOC_MAX_BOWTIE * sizeof(float));

// The scratch array itself.  Host code must not use this name as an address:
// on the host it is only a stand-in; the device address comes from
// cudaGetSymbolAddress in scratch_address().
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

std::mutex g_setup_mutex;
void* g_scratch_address[NOALLOC_MAX_DEVICES] = {};

// Once per device, with that device current: the device address of the array.
cudaError_t scratch_address(int device, unsigned char** out)
{
    if (device < 0 || device >= NOALLOC_MAX_DEVICES)
        return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_address[device]) {
        void* ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess)
            return e;
        g_scratch_address[device] = ptr;
    }
    *out = static_cast<unsigned char*>(g_scratch_address[device]);
    return cudaSuccess;
}

__global__ void noalloc_setup_kernel(unsigned char* s, uint32_t n_exposures, int spec_n, int heel_n, int bowtie_n);

} // namespace

namespace dxmc_gb300::noalloc {
// Called by dxmc_gpu_ctx_create with the context's device current: loads the
// module of the scratch array and of the set-up kernel, and the transport
// kernels' modules, and records the array's device address, so that the first
// dxmc_gpu_transport_noalloc call on the device triggers no lazy module load.
cudaError_t preload(int device)
{
    unsigned char* s = nullptr;
    cudaError_t e = scratch_address(device, &s);
    cudaFuncAttributes attr {};
    if (e == cudaSuccess)
        e = cudaFuncGetAttributes(&attr, noalloc_setup_kernel);
    if (e == cudaSuccess)
        e = dev::preload_transport_kernels();
    return e;
}
} // namespace dxmc_gb300::noalloc

namespace {

// Builds the job tables inside the scratch array from the raw copies of the
// caller's host structures: packed exposures, history prefix sums, the
// spectrum alias table (squaring the histogram, as dxmc_gpu_job_submit builds
// it on the host), float heel weights and the normalised bow-tie table; clears
// the counters.  One block.
__global__ void noalloc_setup_kernel(unsigned char* s, uint32_t n_exposures, int spec_n, int heel_n, int bowtie_n)
{
    const dxmc_exposure* raw = reinterpret_cast<const dxmc_exposure*>(s + OFF_RAW_EXPOSURES);
    dev::DevExposure* ex = reinterpret_cast<dev::DevExposure*>(s + OFF_EXPOSURES);
    for (uint32_t i = threadIdx.x; i < n_exposures; i += blockDim.x) {
        const dxmc_exposure& r = raw[i];
        dev::DevExposure d;
        for (int k = 0; k < 3; ++k) {
            d.pos[k] = static_cast<float>(r.position[k]);
            d.cosx[k] = static_cast<float>(r.direction_cosines[k]);
            d.cosy[k] = static_cast<float>(r.direction_cosines[3 + k]);
            d.beam[k] = static_cast<float>(r.beam_direction[k]);
        }
        for (int k = 0; k < 4; ++k)
            d.coll[k] = static_cast<float>(r.collimation[k]);
        d.weight = static_cast<float>(r.weight);
        d.mono_energy = static_cast<float>(r.mono_energy);
        d.pad0 = 0.0f;
        d.pad1 = 0.0f;
        ex[i] = d;
    }
    float* heel = reinterpret_cast<float*>(s + OFF_HEEL);
    const double* heel_raw = reinterpret_cast<const double*>(s + OFF_HEEL_RAW);
    for (int i = threadIdx.x; i < heel_n; i += blockDim.x)
        heel[i] = static_cast<float>(heel_raw[i]);
    if (threadIdx.x == 0) {
        auto* counters = reinterpret_cast<dev::JobCounters*>(s + OFF_COUNTERS);
        *counters = dev::JobCounters {};
        uint64_t* offsets = reinterpret_cast<uint64_t*>(s + OFF_OFFSETS);
        offsets[0] = 0;
        for (uint32_t i = 0; i < n_exposures; ++i)
            offsets[i + 1] = offsets[i] + raw[i].n_histories;
    }
    if (threadIdx.x == 32 && spec_n > 0) {
        const double* se = reinterpret_cast<const double*>(s + OFF_SPEC_RAW);
        const double* sw = se + NOALLOC_MAX_SPECTRUM;
        float* oe = reinterpret_cast<float*>(s + OFF_SPEC_E);
        float* op = reinterpret_cast<float*>(s + OFF_SPEC_P);
        uint32_t* oa = reinterpret_cast<uint32_t*>(s + OFF_SPEC_A);
        double* scaled = reinterpret_cast<double*>(s + OFF_SPEC_WORK);
        int32_t* small = reinterpret_cast<int32_t*>(scaled + NOALLOC_MAX_SPECTRUM);
        int32_t* large = small + NOALLOC_MAX_SPECTRUM;
        double sum = 0;
        for (int i = 0; i < spec_n; ++i)
            sum += sw[i];
        const double scale = spec_n / sum;
        int ns = 0, nl = 0;
        for (int i = 0; i < spec_n; ++i) {
            scaled[i] = sw[i] * scale;
            oe[i] = static_cast<float>(se[i]);
            op[i] = 0.0f;
            oa[i] = 0u;
        }
        for (int i = spec_n - 1; i >= 0; --i) {
            if (scaled[i] < 1.0)
                small[ns++] = i;
            else
                large[nl++] = i;
        }
        while (ns && nl) {
            const int sm = small[--ns];
            const int lg = large[--nl];
            op[sm] = static_cast<float>(scaled[sm]);
            oa[sm] = static_cast<uint32_t>(lg);
            scaled[lg] = scaled[lg] + scaled[sm] - 1;
            if (scaled[lg] < 1)
                small[ns++] = lg;
            else
                large[nl++] = lg;
        }
        while (nl)
            op[large[--nl]] = 1.0f;
        while (ns)
            op[small[--ns]] = 1.0f;
    }
    if (threadIdx.x == 64 && bowtie_n > 0) {
        double* a = reinterpret_cast<double*>(s + OFF_BOWTIE_RAW);
        double* w = a + NOALLOC_MAX_BOWTIE;
        for (int i = 0; i < bowtie_n; ++i)
            a[i] = fabs(a[i]);
        // insertion sort by (angle, weight), then normalise the weights to mean 1
        for (int i = 1; i < bowtie_n; ++i) {
            const double ka = a[i], kw = w[i];
            int j = i - 1;
            while (j >= 0 && (a[j] > ka || (a[j] == ka && w[j] > kw))) {
                a[j + 1] = a[j];
                w[j + 1] = w[j];
                --j;
            }
            a[j + 1] = ka;
            w[j + 1] = kw;
        }
        double mean = 0;
        for (int i = 0; i < bowtie_n; ++i)
            mean += w[i];
        mean /= bowtie_n;
        float* oa = reinterpret_cast<float*>(s + OFF_BOWTIE_A);
        float* ow = reinterpret_cast<float*>(s + OFF_BOWTIE_W);
        for (int i = 0; i < bowtie_n; ++i) {
            oa[i] = static_cast<float>(a[i]);
            ow[i] = static_cast<float>(w[i] / mean);
        }
    }
}

int reject(dxmc_gpu_ctx* ctx, const std::string& msg);

} // namespace

// Context internals shared with capi_device.cu (same layout, defined there).
struct dxmc_gpu_ctx;
struct dxmc_world;
struct dxmc_lut;
namespace dxmc_gb300::capi {
int ctx_device(const dxmc_gpu_ctx* ctx);
cudaStream_t ctx_stream(const dxmc_gpu_ctx* ctx);
int ctx_sm_count(const dxmc_gpu_ctx* ctx);
size_t ctx_max_smem(const dxmc_gpu_ctx* ctx);
void ctx_set_error(dxmc_gpu_ctx* ctx, const std::string& msg);
int exception_status(dxmc_gpu_ctx* ctx) noexcept; // inside a catch clause: the status of the exception
std::mutex& ctx_mutex(dxmc_gpu_ctx* ctx);
int ctx_regen_threshold(const dxmc_gpu_ctx* ctx, bool local);
int ctx_interact_threshold(const dxmc_gpu_ctx* ctx);
int default_woodcock_burst(bool local);
const dev::WorldParams* world_params(const dxmc_world* w, const dxmc_gpu_ctx** owner, int* n_materials);
const float* lut_image(const dxmc_lut* l, dev::LutMeta* meta, const dxmc_gpu_ctx** owner);
const dev::MajorantGrid* built_majorant(dxmc_gpu_ctx* ctx, dxmc_world* w, const dxmc_lut* l, const dxmc_job_desc* jd);
}

namespace {
int reject(dxmc_gpu_ctx* ctx, const std::string& msg)
{
    capi::ctx_set_error(ctx, msg);
    return DXMC_ERR_INVALID;
}
}

extern "C" int dxmc_gpu_transport_noalloc(dxmc_gpu_ctx* ctx, dxmc_world* world, dxmc_lut* lut, const dxmc_job_desc* jd,
    double* tally, uint32_t* n_events, dxmc_job_stats* stats)
try {
    if (!ctx || !world || !lut || !jd || !tally || !n_events)
        return DXMC_ERR_INVALID;
    std::lock_guard<std::mutex> lock(capi::ctx_mutex(ctx));
    const dxmc_gpu_ctx* world_owner = nullptr;
    const dxmc_gpu_ctx* lut_owner = nullptr;
    int world_materials = 0;
    const dev::WorldParams* wp = capi::world_params(world, &world_owner, &world_materials);
    dev::LutMeta meta {};
    const float* image = capi::lut_image(lut, &meta, &lut_owner);
    if (world_owner != ctx || lut_owner != ctx)
        return reject(ctx, "world or lut belongs to another context");
    if (!jd->exposures || jd->n_exposures == 0)
        return reject(ctx, "job needs at least one exposure");
    if (jd->n_exposures > NOALLOC_MAX_EXPOSURES)
        return reject(ctx, "dxmc_gpu_transport_noalloc: " + std::to_string(jd->n_exposures) + " exposures exceed the maximum of " + std::to_string(NOALLOC_MAX_EXPOSURES));
    const int spec_n = jd->spectrum ? jd->spectrum->n : 0;
    if (jd->spectrum && (spec_n <= 0 || !jd->spectrum->energies || !jd->spectrum->weights))
        return reject(ctx, "invalid spectrum");
    if (spec_n > NOALLOC_MAX_SPECTRUM)
        return reject(ctx, "dxmc_gpu_transport_noalloc: " + std::to_string(spec_n) + " spectrum bins exceed the maximum of " + std::to_string(NOALLOC_MAX_SPECTRUM));
    if (jd->heel && (jd->heel->energy_size <= 0 || jd->heel->angle_size <= 0 || !jd->heel->weights || !(jd->heel->energy_step > 0) || !(jd->heel->angle_step != 0)))
        return reject(ctx, "invalid heel table");
    // the table size in 64 bits, checked before it narrows: a product that wrapped in
    // int could pass the limit while the kernel indexes with the caller's sizes
    const int64_t heel_n64 = jd->heel ? static_cast<int64_t>(jd->heel->energy_size) * jd->heel->angle_size : 0;
    if (heel_n64 > NOALLOC_MAX_HEEL)
        return reject(ctx, "dxmc_gpu_transport_noalloc: " + std::to_string(heel_n64) + " heel weights exceed the maximum of " + std::to_string(NOALLOC_MAX_HEEL));
    const int heel_n = static_cast<int>(heel_n64);
    const int bowtie_n = jd->bowtie ? jd->bowtie->n : 0;
    if (jd->bowtie && (bowtie_n <= 0 || !jd->bowtie->angles || !jd->bowtie->weights))
        return reject(ctx, "invalid bow-tie table");
    if (bowtie_n > NOALLOC_MAX_BOWTIE)
        return reject(ctx, "dxmc_gpu_transport_noalloc: " + std::to_string(bowtie_n) + " bow-tie points exceed the maximum of " + std::to_string(NOALLOC_MAX_BOWTIE));
    if (bowtie_n > 0) {
        // the weights are normalised by their mean on the device: as the job entry
        // point (dxmc_bowtie_table), a mean that is not positive is rejected here
        double sum = 0.0;
        for (int i = 0; i < bowtie_n; ++i)
            sum += jd->bowtie->weights[i];
        if (!(sum > 0.0) || !std::isfinite(sum))
            return reject(ctx, "invalid bow-tie table");
    }
    if (jd->tracking < DXMC_TRACKING_DEFAULT || jd->tracking > DXMC_TRACKING_LOCAL)
        return reject(ctx, "dxmc_gpu_transport_noalloc: unknown tracking mode");
    if (jd->direction != DXMC_DIRECTION_REFERENCE && jd->direction != DXMC_DIRECTION_NORMALIZED)
        return reject(ctx, "dxmc_gpu_transport_noalloc: unknown direction mode");
    if (jd->precision != DXMC_PRECISION_FP32 && jd->precision != DXMC_PRECISION_FP64)
        return reject(ctx, "dxmc_gpu_transport_noalloc: unknown precision");
    if (jd->model < 0 || jd->model > 2)
        return reject(ctx, "unknown low-energy correction model");
    if (meta.n_materials < world_materials)
        return reject(ctx, "lut has fewer materials than the world");
    uint64_t total = 0;
    for (uint64_t i = 0; i < jd->n_exposures; ++i)
        total += jd->exposures[i].n_histories;
    if (total == 0)
        return reject(ctx, "job has no histories");

    const int device = capi::ctx_device(ctx);
    cudaError_t e = cudaSetDevice(device);
    unsigned char* s = nullptr;
    if (e == cudaSuccess)
        e = scratch_address(device, &s);
    cudaStream_t stream = capi::ctx_stream(ctx);
    const uint64_t nv = wp->n_voxels;
    // copy the caller's host tables into the scratch array, clear the outputs
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(s + OFF_RAW_EXPOSURES, jd->exposures, jd->n_exposures * sizeof(dxmc_exposure), cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess && spec_n > 0) {
        e = cudaMemcpyAsync(s + OFF_SPEC_RAW, jd->spectrum->energies, spec_n * sizeof(double), cudaMemcpyHostToDevice, stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(s + OFF_SPEC_RAW + NOALLOC_MAX_SPECTRUM * sizeof(double), jd->spectrum->weights, spec_n * sizeof(double), cudaMemcpyHostToDevice, stream);
    }
    if (e == cudaSuccess && heel_n > 0)
        e = cudaMemcpyAsync(s + OFF_HEEL_RAW, jd->heel->weights, heel_n * sizeof(double), cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess && bowtie_n > 0) {
        e = cudaMemcpyAsync(s + OFF_BOWTIE_RAW, jd->bowtie->angles, bowtie_n * sizeof(double), cudaMemcpyHostToDevice, stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(s + OFF_BOWTIE_RAW + NOALLOC_MAX_BOWTIE * sizeof(double), jd->bowtie->weights, bowtie_n * sizeof(double), cudaMemcpyHostToDevice, stream);
    }
    if (e == cudaSuccess)
        e = cudaMemsetAsync(tally, 0, nv * 2 * sizeof(double), stream);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(n_events, 0, nv * sizeof(uint32_t), stream);
    if (e == cudaSuccess) {
        noalloc_setup_kernel<<<1, 256, 0, stream>>>(s, static_cast<uint32_t>(jd->n_exposures), spec_n, heel_n, bowtie_n);
        e = cudaGetLastError();
    }
    const auto t0 = std::chrono::steady_clock::now();
    if (e == cudaSuccess) {
        dev::TransportParams p {};
        p.world = *wp;
        auto& S = p.source;
        S.exposures = reinterpret_cast<const dev::DevExposure*>(s + OFF_EXPOSURES);
        S.history_offsets = reinterpret_cast<const uint64_t*>(s + OFF_OFFSETS);
        S.n_exposures = static_cast<uint32_t>(jd->n_exposures);
        S.spec_n = spec_n;
        S.spec_energy = reinterpret_cast<const float*>(s + OFF_SPEC_E);
        S.spec_prob = reinterpret_cast<const float*>(s + OFF_SPEC_P);
        S.spec_alias = reinterpret_cast<const uint32_t*>(s + OFF_SPEC_A);
        if (jd->heel) {
            S.heel_weights = reinterpret_cast<const float*>(s + OFF_HEEL);
            S.heel_e_start = static_cast<float>(jd->heel->energy_start);
            S.heel_e_step = static_cast<float>(jd->heel->energy_step);
            S.heel_e_size = jd->heel->energy_size;
            S.heel_a_size = jd->heel->angle_size;
            S.heel_a_start = static_cast<float>(jd->heel->angle_start);
            S.heel_a_step = static_cast<float>(jd->heel->angle_step);
        }
        if (bowtie_n > 0) {
            S.bowtie_angle = reinterpret_cast<const float*>(s + OFF_BOWTIE_A);
            S.bowtie_weight = reinterpret_cast<const float*>(s + OFF_BOWTIE_W);
            S.bowtie_n = bowtie_n;
        }
        p.lut = image;
        p.lut_meta = meta;
        p.tally = tally;
        p.tally_f32 = nullptr;
        p.n_events = n_events;
        p.counters = reinterpret_cast<dev::JobCounters*>(s + OFF_COUNTERS);
        p.cancel = nullptr;
        p.total_histories = total;
        p.seed = jd->seed;
        p.tally_mode = 0; // FP64 atomics
        p.uniform_hpe = 0; // exposure found by binary search over the prefix sums
        // local majorants only from a grid built earlier (dxmc_gpu_world_prepare or a job)
        const dev::MajorantGrid* g = capi::built_majorant(ctx, world, lut, jd);
        if (g)
            p.majorant = *g;
        p.normalize_direction = jd->direction == DXMC_DIRECTION_NORMALIZED ? 1 : 0;
        p.precision = jd->precision;
        p.regen_threshold = capi::ctx_regen_threshold(ctx, g != nullptr);
        p.interact_threshold = capi::ctx_interact_threshold(ctx);
        p.woodcock_burst = jd->woodcock_burst > 0 ? std::min(jd->woodcock_burst, 64) : capi::default_woodcock_burst(g != nullptr);
        const size_t lut_bytes = static_cast<size_t>(meta.total_floats) * sizeof(float);
        const size_t smem_limit = std::min<size_t>(capi::ctx_max_smem(ctx), 96 * 1024);
        p.lut_in_smem = lut_bytes <= smem_limit ? 1 : 0;
        const bool palette = wp->palette_index != nullptr;
        const size_t smem = dev::transport_smem_bytes(lut_bytes, p.lut_in_smem != 0, palette);
        const int block = 256;
        int per_sm = dev::transport_max_blocks_per_sm(jd->model, palette, block, smem, jd->precision);
        if (per_sm <= 0)
            per_sm = 1;
        e = dev::launch_transport(p, jd->model, capi::ctx_sm_count(ctx) * per_sm, block, smem, stream);
    }
    // the counters are read back on every call (into this stack copy, no allocation):
    // a rejection-cap overflow is reported whether or not the caller asked for stats
    dev::JobCounters c {};
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&c, s + OFF_COUNTERS, sizeof(c), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(stream);
    if (e == cudaSuccess && stats) {
        // no CUDA events here (creating one is an allocation): host wall time of the call
        const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        stats->histories = c.histories_done;
        stats->steps = c.steps;
        stats->deposits = c.deposits;
        stats->rejection_overflows = c.overflows;
        stats->kernel_ms = ms;
        stats->job_ms = ms;
    }
    if (e != cudaSuccess) {
        capi::ctx_set_error(ctx, std::string("dxmc_gpu_transport_noalloc: ") + cudaGetErrorString(e));
        return DXMC_ERR_DEVICE;
    }
    if (c.overflows) {
        capi::ctx_set_error(ctx, "sampling loops hit the rejection cap");
        return DXMC_ERR_REJECTION_CAP;
    }
    return DXMC_OK;
} catch (...) {
    return capi::exception_status(ctx);
}
