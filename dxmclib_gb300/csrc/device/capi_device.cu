// Device-side entry points of the C ABI (include/dxmc_gpu.h): context,
// resident worlds and LUTs, job submission on the context stream, result
// post-processing and the component probes.  Every entry point returns an int
// status and records a message retrievable with dxmc_gpu_last_error.
#include "dxmc_gpu.h"

#include "../host/lut_builder.hpp"
#include "../kernels/transport.cuh"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <stdexcept>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

using namespace dxmc_gb300;

namespace dxmc_gb300::noalloc {
cudaError_t preload(int device); // noalloc.cu
}

// Warp scheduling of the transport kernel: refill idle lanes once this many
// are idle; run the per-type interaction passes once this many lanes wait.
constexpr int DEFAULT_REGEN_THRESHOLD = 8;        // photons generated in the transport kernel
constexpr int DEFAULT_INTERACT_THRESHOLD = 8;
constexpr int DEFAULT_QUEUE_REGEN_THRESHOLD = 4;  // photons taken from the pre-generated queue
constexpr int DEFAULT_QUEUE_INTERACT_THRESHOLD = 8;
#ifndef DXMC_DEFAULT_WOODCOCK_BURST
#define DXMC_DEFAULT_WOODCOCK_BURST 8
#endif
constexpr int DEFAULT_WOODCOCK_BURST = DXMC_DEFAULT_WOODCOCK_BURST; // Woodcock steps per loop iteration
// With local majorants a history takes fewer, more varied steps: shorter bursts
// and a later refill keep more lanes of a warp stepping together.
constexpr int DEFAULT_LOCAL_REGEN_THRESHOLD = 10;
constexpr int DEFAULT_LOCAL_WOODCOCK_BURST = 4;
// Local-majorant grid: target cell edge and energy bands (above 15 keV)
#ifndef DXMC_MAJORANT_CELL_MM
#define DXMC_MAJORANT_CELL_MM 6.0
#endif
#ifndef DXMC_MAJORANT_BANDS
#define DXMC_MAJORANT_BANDS 8
#endif
#ifndef DXMC_MAJORANT_BOX
#define DXMC_MAJORANT_BOX 1 // cells outside the box of the denser cells may fly to it
#endif
constexpr double MAJORANT_CELL_MM = DXMC_MAJORANT_CELL_MM; // target cell edge
constexpr int MAJORANT_BANDS = DXMC_MAJORANT_BANDS;         // energy bands above 15 keV
static_assert(MAJORANT_BANDS >= 1 && MAJORANT_BANDS <= dev::MAJORANT_MAX_BANDS, "band count");

// Photons are generated inside the transport kernel unless a job or the context
// asks for a pre-generated queue (2^n photons per generation pass): with the
// Woodcock burst the in-kernel generation is as fast and needs no queue memory.
constexpr int DEFAULT_QUEUE_LOG2 = -1;
// Sampling tables: energies (log-spaced over the LUT range) and quantile levels per row.
constexpr int SAMPLING_ENERGIES = 128;
constexpr int SAMPLING_LEVELS = 512;

struct BatchEngines;

// Page-locked, mapped host blocks that hold a job's cancel flag (byte 0) and the
// host copy of its counters (byte 16).  Freeing page-locked memory waits for all
// work on the device, which would make freeing one job wait for the jobs queued
// after it: the blocks go back to this list and are released with the context.
struct PinnedSlots {
    static constexpr size_t SLOT = 128;
    static constexpr int PER_CHUNK = 64;
    static_assert(16 + sizeof(dev::JobCounters) <= SLOT, "a slot holds the flag and the counters");
    std::vector<void*> chunks;
    std::vector<std::pair<int*, int*>> free_slots; // (host, device) addresses
    cudaError_t take(int** host, int** device)
    {
        if (free_slots.empty()) {
            void* chunk = nullptr;
            cudaError_t e = cudaHostAlloc(&chunk, SLOT * PER_CHUNK, cudaHostAllocMapped);
            if (e != cudaSuccess)
                return e;
            void* dchunk = nullptr;
            e = cudaHostGetDevicePointer(&dchunk, chunk, 0);
            if (e != cudaSuccess) {
                cudaFreeHost(chunk);
                return e;
            }
            chunks.push_back(chunk);
            for (int i = PER_CHUNK - 1; i >= 0; --i)
                free_slots.emplace_back(reinterpret_cast<int*>(static_cast<unsigned char*>(chunk) + i * SLOT),
                    reinterpret_cast<int*>(static_cast<unsigned char*>(dchunk) + i * SLOT));
        }
        *host = free_slots.back().first;
        *device = free_slots.back().second;
        free_slots.pop_back();
        std::memset(*host, 0, SLOT);
        return cudaSuccess;
    }
    void give(int* host, int* device) { free_slots.emplace_back(host, device); }
    void release()
    {
        for (void* c : chunks)
            cudaFreeHost(c);
        chunks.clear();
        free_slots.clear();
    }
};

// Large buffers of finished jobs (tallies, counts, photon queues), kept for the
// next job that needs the same size.  A job hands them back only after its
// kernels and result copies are done, so a kept buffer is idle and serves a job
// at once, without a stream-ordered allocation: that call waited, on the host,
// for an earlier job's result copies before it returned a reused block.
struct JobBufferCache {
    static constexpr size_t MAX_BUFFERS = 8;
    struct Entry {
        void* ptr;
        uint64_t bytes;
    };
    std::vector<Entry> entries; // oldest first
    uint64_t held = 0;
    void* take(uint64_t bytes)
    {
        for (size_t i = entries.size(); i-- > 0;)
            if (entries[i].bytes == bytes) {
                void* p = entries[i].ptr;
                entries.erase(entries.begin() + static_cast<std::ptrdiff_t>(i));
                held -= bytes;
                return p;
            }
        return nullptr;
    }
    // keeps an idle buffer; the oldest one goes back to the pool when the cache is full
    void put(void* p, uint64_t bytes, cudaStream_t s)
    {
        if (entries.size() == MAX_BUFFERS) {
            cudaFreeAsync(entries.front().ptr, s);
            held -= entries.front().bytes;
            entries.erase(entries.begin());
        }
        entries.push_back({ p, bytes });
        held += bytes;
    }
    void release(cudaStream_t s)
    {
        for (const auto& e : entries)
            cudaFreeAsync(e.ptr, s);
        entries.clear();
        held = 0;
    }
};

// Page-locked staging blocks for the host-to-device copy of a job's tables.  A
// copy from pageable memory returns only once the driver has staged it, which
// waited for the copy engine behind other jobs' result copies (tens of
// milliseconds each while serving); from a page-locked block the copy is queued
// at once.  A job holds its block until it is freed; blocks go back to a free
// list per size class and are released with the context.
struct PinnedStaging {
    std::unordered_map<size_t, std::vector<void*>> free_blocks;
    std::vector<void*> blocks;
    static size_t size_class(size_t bytes)
    {
        size_t c = size_t { 64 } << 10;
        while (c < bytes)
            c <<= 1;
        return c;
    }
    cudaError_t take(size_t bytes, void** p, size_t* cls)
    {
        *cls = size_class(bytes);
        auto& l = free_blocks[*cls];
        if (!l.empty()) {
            *p = l.back();
            l.pop_back();
            return cudaSuccess;
        }
        const cudaError_t e = cudaHostAlloc(p, *cls, cudaHostAllocDefault);
        if (e == cudaSuccess)
            blocks.push_back(*p);
        return e;
    }
    void give(void* p, size_t cls) { free_blocks[cls].push_back(p); }
    void release()
    {
        for (void* b : blocks)
            cudaFreeHost(b);
        blocks.clear();
        free_blocks.clear();
    }
};

struct dxmc_gpu_ctx {
    BatchEngines* engines = nullptr; // created by the first batch
    cudaMemPool_t pool = nullptr;    // stream-ordered allocations of this context
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t result_stream = nullptr; // post-processing and result copies
    // world and table uploads: their copies and host waits do not queue behind
    // the jobs on the context stream (uploading the next world overlaps a job)
    cudaStream_t upload_stream = nullptr;
    dxmc_gpu_options options {};
    std::mutex mutex;
    std::string last_error;
    uint64_t budget = 0;
    uint64_t in_use = 0;
    size_t max_smem_optin = 0;
    uint64_t submission = 0; // counts the calls that may build grids (job, batch, world prepare)
    PinnedSlots pinned;      // the jobs' cancel flags and counter copies
    PinnedStaging staging;   // the jobs' tables on their way to the device
    JobBufferCache job_buffers; // idle tally and queue buffers of finished jobs
    // Page-locked, mapped area for the small read-backs a call waits for (palette
    // size and table, a grid's level histogram, per-material maxima).  A kernel
    // writes them there: a copy would queue on the copy engine behind an earlier
    // job's result copies (hundreds of MB) and make the call wait for those.
    unsigned char* readback_host = nullptr;
    unsigned char* readback_dev = nullptr;
};

constexpr size_t READBACK_BYTES = 64 << 10;

// Local-majorant grid of the world for one LUT (built on first use; the least
// recently used one is freed when a world holds too many; see MajorantGrid).
struct MajorantCache {
    uint64_t lut_serial = 0;
    float2* cells = nullptr;
    uint64_t bytes = 0;
    uint64_t last_use = 0;
    uint64_t submission = 0; // the last submission whose jobs read it
    dev::MajorantGrid grid {};
};

// Where in the context's streams an object was last read (see dxmc_world::usage).
struct Usage {
    cudaEvent_t on_stream = nullptr; // after the last single job on the context stream
    cudaEvent_t on_results = nullptr; // after the last result post-processing on the result stream
    bool batched = false;             // read by a batch: wait for all streams
    cudaError_t mark(cudaEvent_t& ev, cudaStream_t s)
    {
        if (!ev) {
            const cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
            if (e != cudaSuccess)
                return e;
        }
        return cudaEventRecord(ev, s);
    }
    void destroy()
    {
        if (on_stream)
            cudaEventDestroy(on_stream);
        if (on_results)
            cudaEventDestroy(on_results);
        on_stream = on_results = nullptr;
    }
};

struct dxmc_world {
    dxmc_gpu_ctx* ctx = nullptr;
    std::vector<MajorantCache> majorants;
    uint64_t majorant_clock = 0;
    dev::Voxel* voxels = nullptr;
    uint8_t* palette_index = nullptr;      // compact layout, null if not used
    dev::PaletteEntry* palette = nullptr;
    std::vector<dev::PaletteEntry> host_palette; // compact layout: the distinct voxels
    uint64_t dims[3] {};
    double spacing[3] {};
    double origin[3] {};
    double cosines[6] {};
    int n_materials = 0;
    bool has_measurement = false;
    uint64_t bytes = 0;
    dev::WorldParams params {};
    // the last use of the world by single jobs on the context stream and by the
    // post-processing of asynchronous results on the result stream: freeing the
    // world waits for these, not for unrelated work; a world used by a batch
    // (chain or engine streams) waits for every stream of the context
    Usage usage;
};

struct dxmc_lut {
    dxmc_gpu_ctx* ctx = nullptr;
    float* image = nullptr;
    dev::LutMeta meta {};
    uint64_t bytes = 0;
    uint64_t serial = 0;              // unique per upload: key of the worlds' majorant grids
    // local-majorant energy bands: r_m of each band (max over the band's energies of
    // mu_m(E) / global majorant, per g/cm3; bands x n_materials), the band edges
    // (keV) and the global majorant (1/mm) at each band's reference energy
    int majorant_bands = 1;
    float band_edge[dev::MAJORANT_MAX_BANDS - 1] {};
    float band_log0 = 1.0f, band_inv_dlog = 0.0f; // log10 of the first edge's base (10 keV) and 1 / log10 step
    std::vector<float> majorant_ratio;
    float mu_ref[dev::MAJORANT_MAX_BANDS] {};
    Usage usage; // as the world's
};

struct dxmc_job {
    dxmc_gpu_ctx* ctx = nullptr;
    dxmc_world* world = nullptr;
    dev::TallyRecord* records = nullptr; // FP64 tallies (modes 0 and 2): one 32-byte record per voxel
    float* tally_f32 = nullptr;          // FP32 tally mode: interleaved (energy, energy^2) ...
    uint32_t* n_events = nullptr;        // ... with the event counts beside it
    dev::JobCounters* counters = nullptr;
    unsigned char* tables = nullptr;
    unsigned char* queue = nullptr; // pre-generated photons (SoA)
    uint64_t tally_bytes = 0, count_bytes = 0, queue_bytes = 0; // sizes of the cached buffers above
    void* staging = nullptr; // page-locked copy of the tables (PinnedStaging)
    size_t staging_class = 0;
    int* cancel_host = nullptr;  // pinned, mapped; the counters' host copy follows at byte 16
    int* cancel_dev = nullptr;
    cudaEvent_t begin = nullptr, start = nullptr, stop = nullptr; // job begin, kernel start, kernel end
    uint64_t histories = 0;
    int tally_mode = 0;
    uint64_t bytes = 0;
    bool cancelled = false;
    bool overflowed = false;
    // an asynchronous result (dxmc_gpu_job_result_async): its completion and the
    // caller's buffers (zeroed by the wait if the job was cancelled)
    cudaEvent_t result_done = nullptr;
    void* result_dose = nullptr;
    void* result_variance = nullptr;
    uint32_t* result_events = nullptr;
    size_t result_elem = 0;
};

namespace {

int fail(dxmc_gpu_ctx* ctx, int code, const std::string& msg)
{
    if (ctx)
        ctx->last_error = msg;
    return code;
}

int cuda_fail(dxmc_gpu_ctx* ctx, cudaError_t e, const char* what)
{
    return fail(ctx, DXMC_ERR_DEVICE, std::string(what) + ": " + cudaGetErrorString(e));
}

// A C++ exception must not cross the C ABI.  The entry points that build host
// tables (sized by the caller's input) call this from their catch clause: host
// memory exhaustion becomes DXMC_ERR_OOM, anything else DXMC_ERR_INVALID, with
// the reason in the context's last error.
int exception_status(dxmc_gpu_ctx* ctx) noexcept
{
    int code = DXMC_ERR_INVALID;
    const char* what = "unexpected exception";
    try {
        throw;
    } catch (const std::bad_alloc&) {
        code = DXMC_ERR_OOM;
        what = "out of host memory";
    } catch (const std::length_error&) {
        code = DXMC_ERR_OOM;
        what = "host table larger than the host can allocate";
    } catch (const std::exception& e) {
        what = e.what();
    } catch (...) {
    }
    if (ctx) {
        try {
            std::lock_guard<std::mutex> lock(ctx->mutex);
            ctx->last_error = what;
        } catch (...) {
        }
    }
    return code;
}

#define DXMC_CUDA(ctx, call)                         \
    do {                                             \
        cudaError_t e_ = (call);                     \
        if (e_ != cudaSuccess)                       \
            return cuda_fail((ctx), e_, #call);      \
    } while (0)

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

} // namespace
extern "C" {
namespace {
void sync_ctx_streams(dxmc_gpu_ctx* ctx); // waits for every stream of the context (defined below)
} // namespace
} // extern "C"
namespace {

// Stream-ordered allocation from the context's own memory pool, which keeps
// freed memory up to the context's budget instead of returning it to the
// driver at every synchronisation: a world, a job's 1 GB of tallies or a grid
// allocated again after a free costs no new mapping.  The pool never makes one
// stream wait for another to reuse a block (a job's tallies would otherwise
// wait for the previous job's result copies, an upload for the running job):
// a block freed on another stream is reused once that free has completed, and
// an allocation that finds no room waits for the context's streams and tries
// again.
template <typename T>
cudaError_t pool_alloc(dxmc_gpu_ctx* ctx, T** ptr, size_t bytes, cudaStream_t stream)
{
    cudaError_t e = cudaMallocFromPoolAsync(reinterpret_cast<void**>(ptr), bytes, ctx->pool, stream);
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        ctx->job_buffers.release(stream);
        sync_ctx_streams(ctx); // every pending free completes
        e = cudaMallocFromPoolAsync(reinterpret_cast<void**>(ptr), bytes, ctx->pool, stream);
    }
    return e;
}

// A job buffer: an idle one of the same size from the cache, else from the pool.
template <typename T>
cudaError_t job_alloc(dxmc_gpu_ctx* ctx, T** ptr, size_t bytes, cudaStream_t stream)
{
    if (void* p = ctx->job_buffers.take(bytes)) {
        *ptr = static_cast<T*>(p);
        return cudaSuccess;
    }
    return pool_alloc(ctx, ptr, bytes, stream);
}

// The device address of a page-locked host buffer (cudaHostAlloc or
// cudaHostRegister), if it is one; false for pageable or device memory.
template <typename T>
bool mapped_host(T* ptr, T*& device_ptr)
{
    cudaPointerAttributes a {};
    if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (a.type != cudaMemoryTypeHost || !a.devicePointer)
        return false;
    device_ptr = static_cast<T*>(a.devicePointer);
    return true;
}

// Local-majorant bounds of a LUT: band edges, per band and material the ratio
// bound, per band the cost model's reference majorant.
struct MajorantRatios {
    int bands = 1;
    float band_edge[dev::MAJORANT_MAX_BANDS - 1] {};
    float band_log0 = 1.0f, band_inv_dlog = 0.0f;
    std::vector<float> ratio; // bands x materials
    float mu_ref[dev::MAJORANT_MAX_BANDS] {};
};

// Per energy band and material m, the largest ratio of m's attenuation (per
// g/cm3) to the global majorant over the band's energies, from the float image
// the kernels read.  Photons are tracked from 1 keV (the transport cutoff) to
// the LUT's maximum energy; above 15 keV that range is cut into MAJORANT_BANDS
// bands with edges log-spaced from 10 keV, since soft tissue's share of a bone-set
// majorant varies five-fold over a diagnostic spectrum.  In each log-log
// segment both attenuations are exponentials of log E, so the ratio of their
// sum to the majorant is convex in log E and peaks at an end of the interval of
// log E that the kernels' segment lookup (lut_segment) maps to that segment.
// Those ends are nodes of the table, steps of its linear part, band edges or
// the range limits: every segment is evaluated at each such point where the
// lookup selects it on either side.  A band's interval is widened by 0.1 % so
// that rounding of the band choice stays covered, and a 0.2 % margin covers the
// device's exponential and the level arithmetic.  mu_ref: the global majorant
// (1/mm) at each band's geometric mid-energy, the cost model's reference.
void compute_majorant_ratios(const std::vector<float>& img, const dev::LutMeta& m, MajorantRatios& lut)
{
    const int R = m.R;
    const float* x = img.data() + m.off_x;
    const float* maxc = img.data() + m.off_maxcoef;
    // the kernels' segment lookup, in the same float arithmetic
    auto segment = [&](float le) {
        if (le > m.linear_energy) {
            const int idx = static_cast<int>((le - m.linear_energy) * m.inv_linear_step) + m.linear_index;
            return std::min(idx, R - 1);
        }
        const int pos = static_cast<int>(std::upper_bound(x, x + R, le) - x);
        return pos < R ? pos : R - 1;
    };
    auto max_inverse = [&](float le) {
        const int seg = segment(le);
        return std::pow(10.0, static_cast<double>(maxc[2 * seg]) + maxc[2 * seg + 1] * static_cast<double>(le));
    };
    const double e_max = std::max(static_cast<double>(m.max_energy), 1.0);
    lut.bands = e_max > 15.0 ? MAJORANT_BANDS : 1;
    const int nb = lut.bands;
    std::vector<double> edges { 1.0 };
    for (int k = 1; k < nb; ++k)
        edges.push_back(10.0 * std::pow(e_max / 10.0, static_cast<double>(k) / nb));
    edges.push_back(e_max);
    for (int k = 0; k < dev::MAJORANT_MAX_BANDS - 1; ++k)
        lut.band_edge[k] = k + 1 < nb ? static_cast<float>(edges[k + 1]) : INFINITY;
    lut.band_log0 = 1.0f;
    lut.band_inv_dlog = nb > 1 ? static_cast<float>(nb / std::log10(e_max / 10.0)) : 0.0f;
    std::vector<float> points;
    for (int k = 0; k < R; ++k)
        points.push_back(x[k]);
    for (int k = 0; k <= R; ++k)
        points.push_back(m.linear_energy + static_cast<float>(k) / m.inv_linear_step);
    lut.ratio.assign(static_cast<size_t>(nb) * m.n_materials, 0.0f);
    for (int b = 0; b < nb; ++b) {
        const float le_lo = static_cast<float>(std::log10(edges[b]) - (b > 0 ? 4.34e-4 : 0.0));
        const float le_hi = static_cast<float>(std::log10(edges[b + 1]) + (b + 1 < nb ? 4.34e-4 : 0.0));
        std::vector<float> pts { le_lo, le_hi };
        for (const float t : points)
            if (t > le_lo && t < le_hi)
                pts.push_back(t);
        for (int mat = 0; mat < m.n_materials; ++mat) {
            double r = 0.0;
            for (const float t : pts) {
                for (const float le : { std::nextafter(t, -1e30f), t, std::nextafter(t, 1e30f) }) {
                    if (!(le >= le_lo && le <= le_hi))
                        continue;
                    const int seg = segment(le);
                    const float* c = img.data() + m.off_coef + (static_cast<size_t>(mat) * R + seg) * 6;
                    double tot = 0.0;
                    for (int k = 0; k < 3; ++k)
                        tot += std::pow(10.0, static_cast<double>(c[2 * k]) + c[2 * k + 1] * static_cast<double>(t));
                    const double inv = std::pow(10.0, static_cast<double>(maxc[2 * seg]) + maxc[2 * seg + 1] * static_cast<double>(t));
                    r = std::max(r, tot * inv);
                }
            }
            lut.ratio[static_cast<size_t>(b) * m.n_materials + mat] = static_cast<float>(r * 1.002);
        }
        const double inv_cm = max_inverse(static_cast<float>(0.5 * (std::log10(edges[b]) + std::log10(edges[b + 1]))));
        lut.mu_ref[b] = static_cast<float>(inv_cm > 0 ? 0.1 / inv_cm : 0.01);
    }
}

// The ratio bounds of a blob, computed at its first upload and kept with it (the
// same blob is often uploaded again, to other contexts or after a free).
std::shared_ptr<const MajorantRatios> majorant_ratios(const dxmc_lut_blob& b, const std::vector<float>& img, const dev::LutMeta& m)
{
    std::lock_guard<std::mutex> lock(*b.tables_mutex);
    if (auto cached = std::static_pointer_cast<const MajorantRatios>(b.majorant))
        return cached;
    auto r = std::make_shared<MajorantRatios>();
    compute_majorant_ratios(img, m, *r);
    b.majorant = r;
    return r;
}

size_t dev_palette_table_bytes();

// Safe extents exactly as World<float>::updateMatrixExtent (world.hpp:55-68).
void world_extents(const uint64_t dims[3], const double spacing[3], const double origin[3], float lo[3], float hi[3])
{
    for (int i = 0; i < 3; ++i) {
        const float sp = static_cast<float>(spacing[i]);
        const float half = (static_cast<float>(dims[i]) * sp) * 0.5f;
        const float o = static_cast<float>(origin[i]);
        const float lower = o - half;
        const float upper = o + half;
        lo[i] = std::nextafter(lower, upper);
        hi[i] = std::nextafter(upper, lower);
    }
}

__global__ void pack_voxels_kernel(const float* __restrict__ density, const uint8_t* __restrict__ material,
    const uint8_t* __restrict__ measurement, uint64_t n, dev::Voxel* __restrict__ out)
{
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n; i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        dev::Voxel v;
        v.density = density[i];
        v.material = material[i];
        v.measurement = measurement ? measurement[i] : 0;
        v.pad = 0;
        out[i] = v;
    }
}

// Sets *bad if any material index is >= n_materials (16 indices per load where
// the array is 16-byte aligned, then the tail).
__global__ void readback_kernel(const unsigned int* __restrict__ src, unsigned int* __restrict__ dst, uint32_t n_words)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_words; i += gridDim.x * blockDim.x)
        dst[i] = src[i];
}

// Enqueues the copy of `bytes` (a multiple of 4) from device memory into the
// context's read-back area at `offset`; the host reads readback_host + offset
// after synchronising the stream.  Caller holds the context mutex.
cudaError_t enqueue_readback(dxmc_gpu_ctx* ctx, const void* src, size_t offset, size_t bytes, cudaStream_t s)
{
    if (offset % 4 || bytes % 4 || offset + bytes > READBACK_BYTES)
        return cudaErrorInvalidValue;
    const uint32_t words = static_cast<uint32_t>(bytes / 4);
    const int blocks = static_cast<int>(std::min<uint32_t>((words + 255) / 256, 32));
    readback_kernel<<<std::max(blocks, 1), 256, 0, s>>>(static_cast<const unsigned int*>(src),
        reinterpret_cast<unsigned int*>(ctx->readback_dev + offset), words);
    return cudaGetLastError();
}

__global__ void check_materials_kernel(const uint8_t* __restrict__ material, uint64_t n, int n_materials, unsigned int* bad)
{
    const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
    const uint64_t t0 = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
    bool found = false;
    uint64_t first_scalar = 0;
    if ((reinterpret_cast<uintptr_t>(material) & 15u) == 0) {
        const uint64_t vecs = n / 16;
        for (uint64_t v = t0; v < vecs; v += stride) {
            const uint4 q = reinterpret_cast<const uint4*>(material)[v];
            const uint32_t words[4] = { q.x, q.y, q.z, q.w };
#pragma unroll
            for (int k = 0; k < 16; ++k)
                found = found || static_cast<int>((words[k >> 2] >> (8 * (k & 3))) & 0xffu) >= n_materials;
        }
        first_scalar = vecs * 16;
    }
    for (uint64_t i = first_scalar + t0; i < n; i += stride)
        found = found || material[i] >= n_materials;
    if (found)
        atomicOr(bad, 1u);
}

// ---- compact palette layout ---------------------------------------------------------
// Distinct (density, material, measurement) triples are collected in an
// open-addressing hash table; with at most PALETTE_MAX of them every voxel is
// stored as a 1-byte palette index (exact: the palette holds the f32 density).
constexpr int PALETTE_TABLE = 4096; // hash slots (power of two)
constexpr int PALETTE_SEEN = 512;   // per-block cache of keys already in the table (power of two)
constexpr uint64_t PALETTE_EMPTY = 0ull;

__device__ __forceinline__ uint64_t palette_key(float density, uint8_t material, uint8_t measurement)
{
    return (1ull << 63) | (static_cast<uint64_t>(__float_as_uint(density)) << 16) | (static_cast<uint64_t>(material) << 8) | measurement;
}

__device__ __forceinline__ uint32_t palette_hash(uint64_t key)
{
    key ^= key >> 33;
    key *= 0xff51afd7ed558ccdull;
    key ^= key >> 33;
    return static_cast<uint32_t>(key) & (PALETTE_TABLE - 1);
}

// The voxels of 4-voxel group g (i = 4g .. 4g + 3) when every array allows vector
// loads; the caller runs the scalar tail.
struct VoxelQuad {
    uint64_t key[4];
};

__device__ __forceinline__ VoxelQuad load_quad(const float* __restrict__ density, const uint8_t* __restrict__ material,
    const uint8_t* __restrict__ measurement, uint64_t g)
{
    const float4 d = reinterpret_cast<const float4*>(density)[g];
    const uchar4 m = reinterpret_cast<const uchar4*>(material)[g];
    const uchar4 f = measurement ? reinterpret_cast<const uchar4*>(measurement)[g] : make_uchar4(0, 0, 0, 0);
    return VoxelQuad { { palette_key(d.x, m.x, f.x), palette_key(d.y, m.y, f.y), palette_key(d.z, m.z, f.z), palette_key(d.w, m.w, f.w) } };
}

__device__ __forceinline__ bool quad_loads(const float* density, const uint8_t* material, const uint8_t* measurement)
{
    return (reinterpret_cast<uintptr_t>(density) & 15u) == 0 && (reinterpret_cast<uintptr_t>(material) & 3u) == 0
        && (reinterpret_cast<uintptr_t>(measurement) & 3u) == 0;
}

// Adds key to the global table unless the block's cache of keys already in the
// table holds it.  The cache is direct-mapped; concurrent writers of one slot
// each store a key that is in the table, so any value read is a valid hit.
__device__ __forceinline__ void palette_insert(uint64_t key, unsigned long long* seen, unsigned long long* table,
    unsigned int* count)
{
    const uint32_t h0 = palette_hash(key);
    unsigned long long* cached = seen + (h0 & (PALETTE_SEEN - 1));
    if (*reinterpret_cast<volatile unsigned long long*>(cached) == key)
        return;
    if (*reinterpret_cast<volatile unsigned int*>(count) > static_cast<unsigned>(dev::PALETTE_MAX))
        return; // already too many distinct voxels: the 8-byte layout will be used
    uint32_t h = h0;
    for (int probe = 0; probe < PALETTE_TABLE; ++probe) {
        const unsigned long long cur = table[h];
        if (cur == key)
            break;
        if (cur == PALETTE_EMPTY) {
            const unsigned long long prev = atomicCAS(table + h, PALETTE_EMPTY, key);
            if (prev == PALETTE_EMPTY) {
                atomicAdd(count, 1u);
                break;
            }
            if (prev == key)
                break;
        }
        h = (h + 1) & (PALETTE_TABLE - 1);
    }
    *reinterpret_cast<volatile unsigned long long*>(cached) = key;
}

__global__ void palette_insert_kernel(const float* __restrict__ density, const uint8_t* __restrict__ material,
    const uint8_t* __restrict__ measurement, uint64_t n, unsigned long long* table, unsigned int* count)
{
    __shared__ unsigned long long seen[PALETTE_SEEN];
    for (int i = threadIdx.x; i < PALETTE_SEEN; i += blockDim.x)
        seen[i] = PALETTE_EMPTY;
    __syncthreads();
    const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
    const uint64_t t0 = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
    uint64_t first_scalar = 0;
    if (quad_loads(density, material, measurement)) {
        const uint64_t quads = n / 4;
        for (uint64_t g = t0; g < quads; g += stride) {
            const VoxelQuad q = load_quad(density, material, measurement, g);
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (k == 0 || q.key[k] != q.key[k - 1])
                    palette_insert(q.key[k], seen, table, count);
        }
        first_scalar = quads * 4;
    }
    for (uint64_t i = first_scalar + t0; i < n; i += stride)
        palette_insert(palette_key(density[i], material[i], measurement ? measurement[i] : 0), seen, table, count);
}

// The palette index of every voxel, probing a copy of the table in shared memory.
__global__ void palette_map_kernel(const float* __restrict__ density, const uint8_t* __restrict__ material,
    const uint8_t* __restrict__ measurement, uint64_t n, const unsigned long long* __restrict__ table,
    const uint8_t* __restrict__ slot_index, uint8_t* __restrict__ out)
{
    __shared__ unsigned long long keys[PALETTE_TABLE];
    __shared__ uint8_t slots[PALETTE_TABLE];
    for (int i = threadIdx.x; i < PALETTE_TABLE; i += blockDim.x) {
        keys[i] = table[i];
        slots[i] = slot_index[i];
    }
    __syncthreads();
    auto lookup = [&](uint64_t key) -> uint8_t {
        uint32_t h = palette_hash(key);
        for (int probe = 0; probe < PALETTE_TABLE; ++probe) {
            if (keys[h] == key)
                return slots[h];
            h = (h + 1) & (PALETTE_TABLE - 1);
        }
        return 0;
    };
    const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
    const uint64_t t0 = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
    uint64_t first_scalar = 0;
    if (quad_loads(density, material, measurement) && (reinterpret_cast<uintptr_t>(out) & 3u) == 0) {
        const uint64_t quads = n / 4;
        for (uint64_t g = t0; g < quads; g += stride) {
            const VoxelQuad q = load_quad(density, material, measurement, g);
            uint8_t idx[4];
#pragma unroll
            for (int k = 0; k < 4; ++k)
                idx[k] = (k > 0 && q.key[k] == q.key[k - 1]) ? idx[k - 1] : lookup(q.key[k]);
            reinterpret_cast<uchar4*>(out)[g] = make_uchar4(idx[0], idx[1], idx[2], idx[3]);
        }
        first_scalar = quads * 4;
    }
    for (uint64_t i = first_scalar + t0; i < n; i += stride)
        out[i] = lookup(palette_key(density[i], material[i], measurement ? measurement[i] : 0));
}

size_t dev_palette_table_bytes() { return PALETTE_TABLE * sizeof(unsigned long long); }

} // namespace

extern "C" {

namespace {
void sync_ctx_streams(dxmc_gpu_ctx* ctx);
void wait_unused(dxmc_gpu_ctx* ctx, const Usage& u);
void release_engines(dxmc_gpu_ctx* ctx);
int wait_event(dxmc_gpu_ctx* ctx, cudaEvent_t ev, int64_t timeout_ms, const char* what);
int world_majorant(dxmc_gpu_ctx* ctx, dxmc_world* w, const dxmc_lut* lut, bool build, const dev::MajorantGrid** out);
} // namespace

int dxmc_gpu_device_count(void)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess)
        return 0;
    return n;
}

int dxmc_gpu_ctx_memory(const dxmc_gpu_ctx* ctx, uint64_t* budget, uint64_t* in_use)
{
    if (!ctx)
        return DXMC_ERR_INVALID;
    std::lock_guard<std::mutex> lock(const_cast<dxmc_gpu_ctx*>(ctx)->mutex);
    if (budget)
        *budget = ctx->budget;
    if (in_use)
        *in_use = ctx->in_use;
    return DXMC_OK;
}

int dxmc_gpu_host_alloc(uint64_t bytes, void** out)
{
    if (!out || bytes == 0)
        return DXMC_ERR_INVALID;
    *out = nullptr;
    return cudaHostAlloc(out, bytes, cudaHostAllocDefault) == cudaSuccess ? DXMC_OK : DXMC_ERR_OOM;
}

void dxmc_gpu_host_free(void* ptr)
{
    if (ptr)
        cudaFreeHost(ptr);
}

int dxmc_gpu_ctx_create(const dxmc_gpu_options* options, dxmc_gpu_ctx** out)
try {
    if (!out)
        return DXMC_ERR_INVALID;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0)
        return DXMC_ERR_NO_DEVICE;
    auto* ctx = new (std::nothrow) dxmc_gpu_ctx;
    if (!ctx)
        return DXMC_ERR_OOM;
    if (options)
        ctx->options = *options;
    ctx->device = ctx->options.device;
    if (ctx->device < 0 || ctx->device >= count || ctx->options.tracking < DXMC_TRACKING_DEFAULT
        || ctx->options.tracking > DXMC_TRACKING_LOCAL) {
        delete ctx;
        return DXMC_ERR_INVALID;
    }
    if (cudaSetDevice(ctx->device) != cudaSuccess) {
        delete ctx;
        return DXMC_ERR_DEVICE;
    }
    cudaDeviceProp prop {};
    cudaGetDeviceProperties(&prop, ctx->device);
    ctx->sm_count = prop.multiProcessorCount;
    ctx->max_smem_optin = prop.sharedMemPerBlockOptin;
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete ctx;
        return DXMC_ERR_DEVICE;
    }
    if (cudaStreamCreateWithFlags(&ctx->result_stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaStreamDestroy(ctx->stream);
        delete ctx;
        return DXMC_ERR_DEVICE;
    }
    // uploads and grid builds at the device's greatest priority: a world's palette
    // kernels and its majorant grid are what the next job waits for, so their blocks
    // take the SMs before an earlier job's post-processing
    int least_priority = 0, greatest_priority = 0;
    cudaDeviceGetStreamPriorityRange(&least_priority, &greatest_priority);
    if (cudaStreamCreateWithPriority(&ctx->upload_stream, cudaStreamNonBlocking, greatest_priority) != cudaSuccess) {
        cudaStreamDestroy(ctx->result_stream);
        cudaStreamDestroy(ctx->stream);
        delete ctx;
        return DXMC_ERR_DEVICE;
    }
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    ctx->budget = ctx->options.memory_budget ? ctx->options.memory_budget : static_cast<uint64_t>(free_b * 0.9);
    cudaMemPoolProps props {};
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = ctx->device;
    uint64_t keep = ctx->budget;
    int no_cross_stream_waits = 0;
    if (cudaMemPoolCreate(&ctx->pool, &props) != cudaSuccess
        || cudaMemPoolSetAttribute(ctx->pool, cudaMemPoolAttrReleaseThreshold, &keep) != cudaSuccess
        || cudaMemPoolSetAttribute(ctx->pool, cudaMemPoolReuseAllowInternalDependencies, &no_cross_stream_waits)
            != cudaSuccess) {
        if (ctx->pool)
            cudaMemPoolDestroy(ctx->pool);
        cudaStreamDestroy(ctx->upload_stream);
        cudaStreamDestroy(ctx->result_stream);
        cudaStreamDestroy(ctx->stream);
        delete ctx;
        return DXMC_ERR_DEVICE;
    }
    void* rb_dev = nullptr;
    if (cudaHostAlloc(reinterpret_cast<void**>(&ctx->readback_host), READBACK_BYTES, cudaHostAllocMapped) != cudaSuccess
        || cudaHostGetDevicePointer(&rb_dev, ctx->readback_host, 0) != cudaSuccess) {
        if (ctx->readback_host)
            cudaFreeHost(ctx->readback_host);
        cudaMemPoolDestroy(ctx->pool);
        cudaStreamDestroy(ctx->upload_stream);
        cudaStreamDestroy(ctx->result_stream);
        cudaStreamDestroy(ctx->stream);
        delete ctx;
        return DXMC_ERR_DEVICE;
    }
    ctx->readback_dev = static_cast<unsigned char*>(rb_dev);
    // the no-allocation entry point must not meet a lazy module load (which
    // allocates) in its first call: load its module and the transport kernels now
    if (noalloc::preload(ctx->device) != cudaSuccess) {
        cudaFreeHost(ctx->readback_host);
        cudaMemPoolDestroy(ctx->pool);
        cudaStreamDestroy(ctx->upload_stream);
        cudaStreamDestroy(ctx->result_stream);
        cudaStreamDestroy(ctx->stream);
        delete ctx;
        return DXMC_ERR_DEVICE;
    }
    *out = ctx;
    return DXMC_OK;
} catch (...) {
    return exception_status(nullptr);
}

void dxmc_gpu_ctx_destroy(dxmc_gpu_ctx* ctx)
{
    if (!ctx)
        return;
    cudaSetDevice(ctx->device);
    sync_ctx_streams(ctx);
    release_engines(ctx);
    ctx->job_buffers.release(ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    ctx->pinned.release();
    ctx->staging.release();
    cudaFreeHost(ctx->readback_host);
    cudaStreamDestroy(ctx->upload_stream);
    cudaStreamDestroy(ctx->result_stream);
    cudaStreamDestroy(ctx->stream);
    cudaMemPoolDestroy(ctx->pool); // memory still held by objects not freed is released with them
    delete ctx;
}

const char* dxmc_gpu_last_error(const dxmc_gpu_ctx* ctx)
{
    return ctx ? ctx->last_error.c_str() : "no context";
}

int dxmc_gpu_world_upload(dxmc_gpu_ctx* ctx, const dxmc_world_desc* d, dxmc_world** out)
try {
    if (!ctx || !d || !out)
        return DXMC_ERR_INVALID;
    std::lock_guard<std::mutex> lock(ctx->mutex);
    *out = nullptr;
    const uint64_t n = d->dims[0] * d->dims[1] * d->dims[2];
    // World::validate (world.hpp:182-227)
    if (n == 0 || !(d->spacing[0] * d->spacing[1] * d->spacing[2] > 0) || !d->density || !d->material || d->n_materials <= 0 || d->n_materials > 255)
        return fail(ctx, DXMC_ERR_INVALID, "invalid world: dimensions, spacing, arrays or material count");
    if (d->dims[0] > 0xffffffffull || d->dims[1] > 0xffffffffull || d->dims[2] > 0xffffffffull)
        return fail(ctx, DXMC_ERR_INVALID, "invalid world: dimension exceeds 2^32");
    {
        const double* c = d->direction_cosines;
        const double n1 = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
        const double n2 = std::sqrt(c[3] * c[3] + c[4] * c[4] + c[5] * c[5]);
        if (!(n1 > 0) || !(n2 > 0))
            return fail(ctx, DXMC_ERR_INVALID, "invalid world: zero direction cosine");
        const double x[3] = { c[0] / n1, c[1] / n1, c[2] / n1 };
        const double y[3] = { c[3] / n2, c[4] / n2, c[5] / n2 };
        const double z[3] = { x[1] * y[2] - x[2] * y[1], x[2] * y[0] - x[0] * y[2], x[0] * y[1] - x[1] * y[0] };
        const double ortho = (z[0] * x[0] + z[1] * x[1] + z[2] * x[2]) + (z[0] * y[0] + z[1] * y[1] + z[2] * y[2]) + (x[0] * y[0] + x[1] * y[1] + x[2] * y[2]);
        if (std::abs(ortho) > 0.001)
            return fail(ctx, DXMC_ERR_INVALID, "invalid world: direction cosines are not orthogonal");
    }
    const uint64_t bytes = n * sizeof(dev::Voxel);
    if (ctx->in_use + bytes > ctx->budget)
        return fail(ctx, DXMC_ERR_OOM, "world exceeds the device memory budget");
    cudaSetDevice(ctx->device);
    auto* w = new (std::nothrow) dxmc_world;
    if (!w)
        return DXMC_ERR_OOM;
    w->ctx = ctx;
    // stage raw arrays, validate and pack on the device
    float* d_density = nullptr;
    uint8_t* d_material = nullptr;
    uint8_t* d_meas = nullptr;
    unsigned int* d_bad = nullptr;
    cudaError_t e = pool_alloc(ctx, &d_density, n * sizeof(float), ctx->upload_stream);
    if (e == cudaSuccess)
        e = pool_alloc(ctx, &d_material, n, ctx->upload_stream);
    if (e == cudaSuccess && d->measurement)
        e = pool_alloc(ctx, &d_meas, n, ctx->upload_stream);
    if (e == cudaSuccess)
        e = pool_alloc(ctx, &d_bad, sizeof(unsigned int), ctx->upload_stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_density, d->density, n * sizeof(float), cudaMemcpyHostToDevice, ctx->upload_stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_material, d->material, n, cudaMemcpyHostToDevice, ctx->upload_stream);
    if (e == cudaSuccess && d_meas)
        e = cudaMemcpyAsync(d_meas, d->measurement, n, cudaMemcpyHostToDevice, ctx->upload_stream);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(d_bad, 0, sizeof(unsigned int), ctx->upload_stream);
    unsigned int bad = 0;
    if (e == cudaSuccess) {
        const int grid = ctx->sm_count * 8;
        check_materials_kernel<<<grid, 256, 0, ctx->upload_stream>>>(d_material, n, d->n_materials, d_bad);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) // read after the upload's last synchronisation
        e = enqueue_readback(ctx, d_bad, 0, sizeof(unsigned int), ctx->upload_stream);
    // compact palette layout when the world has few distinct voxels
    unsigned long long* d_table = nullptr;
    unsigned int* d_count = nullptr;
    unsigned int distinct = 0;
    std::vector<dev::PaletteEntry> palette;
    if (e == cudaSuccess && d->layout == 0 && n <= 0xffffffffull) { // the compact layout indexes voxels in 32 bits
        e = pool_alloc(ctx, &d_table, dev_palette_table_bytes(), ctx->upload_stream);
        if (e == cudaSuccess)
            e = pool_alloc(ctx, &d_count, sizeof(unsigned int), ctx->upload_stream);
        if (e == cudaSuccess)
            e = cudaMemsetAsync(d_table, 0, dev_palette_table_bytes(), ctx->upload_stream);
        if (e == cudaSuccess)
            e = cudaMemsetAsync(d_count, 0, sizeof(unsigned int), ctx->upload_stream);
        if (e == cudaSuccess) {
            palette_insert_kernel<<<ctx->sm_count * 8, 256, 0, ctx->upload_stream>>>(d_density, d_material, d_meas, n, d_table, d_count);
            e = cudaGetLastError();
        }
        // the count and the table in one read-back (the table is only used when the count fits)
        if (e == cudaSuccess)
            e = enqueue_readback(ctx, d_count, 4, sizeof(unsigned int), ctx->upload_stream);
        if (e == cudaSuccess)
            e = enqueue_readback(ctx, d_table, 64, dev_palette_table_bytes(), ctx->upload_stream);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(ctx->upload_stream);
        if (e == cudaSuccess)
            std::memcpy(&distinct, ctx->readback_host + 4, sizeof(unsigned int));
        if (e == cudaSuccess && distinct >= 1 && distinct <= static_cast<unsigned>(dev::PALETTE_MAX)) {
            std::vector<unsigned long long> table(PALETTE_TABLE);
            std::memcpy(table.data(), ctx->readback_host + 64, dev_palette_table_bytes());
            std::vector<uint8_t> slot_index(PALETTE_TABLE, 0);
            for (int slot = 0; slot < PALETTE_TABLE && e == cudaSuccess; ++slot) {
                const unsigned long long key = table[slot];
                if (key == PALETTE_EMPTY)
                    continue;
                dev::PaletteEntry pe;
                const uint32_t bits = static_cast<uint32_t>(key >> 16);
                std::memcpy(&pe.density, &bits, sizeof(float));
                pe.code = static_cast<uint32_t>(key & 0xffffu); // material | measurement << 8
                pe.code = (pe.code >> 8) | ((pe.code & 0xffu) << 8);
                slot_index[slot] = static_cast<uint8_t>(palette.size());
                palette.push_back(pe);
            }
            uint8_t* d_slots = nullptr;
            if (e == cudaSuccess)
                e = pool_alloc(ctx, &d_slots, PALETTE_TABLE, ctx->upload_stream);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(d_slots, slot_index.data(), PALETTE_TABLE, cudaMemcpyHostToDevice, ctx->upload_stream);
            if (e == cudaSuccess)
                e = pool_alloc(ctx, &w->palette_index, n, ctx->upload_stream);
            if (e == cudaSuccess)
                e = pool_alloc(ctx, &w->palette, dev::PALETTE_MAX * sizeof(dev::PaletteEntry), ctx->upload_stream);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(w->palette, palette.data(), palette.size() * sizeof(dev::PaletteEntry), cudaMemcpyHostToDevice, ctx->upload_stream);
            if (e == cudaSuccess) {
                palette_map_kernel<<<ctx->sm_count * 8, 256, 0, ctx->upload_stream>>>(d_density, d_material, d_meas, n, d_table, d_slots, w->palette_index);
                e = cudaGetLastError();
            }
            if (d_slots)
                cudaFreeAsync(d_slots, ctx->upload_stream);
        }
    }
    // the 8-byte layout only when the compact one is not used (too many distinct voxels, or asked for)
    if (e == cudaSuccess && !w->palette_index) {
        palette.clear();
        e = pool_alloc(ctx, &w->voxels, bytes, ctx->upload_stream);
        if (e == cudaSuccess) {
            pack_voxels_kernel<<<ctx->sm_count * 8, 256, 0, ctx->upload_stream>>>(d_density, d_material, d_meas, n, w->voxels);
            e = cudaGetLastError();
        }
    }
    if (d_table)
        cudaFreeAsync(d_table, ctx->upload_stream);
    if (d_count)
        cudaFreeAsync(d_count, ctx->upload_stream);
    if (d_density)
        cudaFreeAsync(d_density, ctx->upload_stream);
    if (d_material)
        cudaFreeAsync(d_material, ctx->upload_stream);
    if (d_meas)
        cudaFreeAsync(d_meas, ctx->upload_stream);
    if (d_bad)
        cudaFreeAsync(d_bad, ctx->upload_stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(ctx->upload_stream);
    if (e == cudaSuccess)
        std::memcpy(&bad, ctx->readback_host, sizeof(unsigned int));
    if (e != cudaSuccess || bad) {
        if (w->voxels)
            cudaFreeAsync(w->voxels, ctx->upload_stream);
        if (w->palette_index)
            cudaFreeAsync(w->palette_index, ctx->upload_stream);
        if (w->palette)
            cudaFreeAsync(w->palette, ctx->upload_stream);
        cudaStreamSynchronize(ctx->upload_stream);
        delete w;
        if (e != cudaSuccess)
            return cuda_fail(ctx, e, "world upload");
        return fail(ctx, DXMC_ERR_INVALID, "invalid world: material index >= n_materials");
    }
    for (int i = 0; i < 3; ++i) {
        w->dims[i] = d->dims[i];
        w->spacing[i] = d->spacing[i];
        w->origin[i] = d->origin[i];
    }
    std::memcpy(w->cosines, d->direction_cosines, sizeof(w->cosines));
    w->n_materials = d->n_materials;
    w->has_measurement = d->measurement != nullptr;
    w->bytes = w->palette_index ? n + dev::PALETTE_MAX * sizeof(dev::PaletteEntry) : bytes;
    w->host_palette = palette;
    ctx->in_use += w->bytes;
    auto& P = w->params;
    P.voxels = w->voxels;
    P.palette_index = w->palette_index;
    P.palette = w->palette;
    P.palette_n = static_cast<int>(palette.size());
    for (int i = 0; i < 3; ++i) {
        P.dims[i] = static_cast<uint32_t>(d->dims[i]);
        P.inv_spacing[i] = static_cast<float>(1.0 / static_cast<double>(static_cast<float>(d->spacing[i])));
        P.spacing[i] = static_cast<float>(d->spacing[i]);
        P.lower[i] = static_cast<float>(d->origin[i] - 0.5 * static_cast<double>(d->dims[i]) * d->spacing[i]);
    }
    world_extents(d->dims, d->spacing, d->origin, P.lo, P.hi);
    for (int i = 0; i < 3; ++i) {
        P.lo_inv[i] = P.lo[i] * P.inv_spacing[i];
        P.dims_f[i] = static_cast<float>(d->dims[i]);
    }
    P.nxy = d->dims[0] * d->dims[1];
    P.n_voxels = n;
    *out = w;
    return DXMC_OK;
} catch (...) {
    return exception_status(ctx);
}

int dxmc_gpu_world_max_density(dxmc_world* w, double* out, int n_materials)
try {
    if (!w || !out || n_materials <= 0)
        return DXMC_ERR_INVALID;
    dxmc_gpu_ctx* ctx = w->ctx;
    std::lock_guard<std::mutex> lock(ctx->mutex);
    if (w->palette_index) {
        // the palette holds every distinct (density, material) pair of the grid
        for (int i = 0; i < n_materials; ++i)
            out[i] = 0.0;
        for (const auto& pe : w->host_palette) {
            const int mat = static_cast<int>(pe.code & 0xffu);
            if (mat < n_materials)
                out[mat] = std::max(out[mat], static_cast<double>(std::max(pe.density, 0.0f)));
        }
        return DXMC_OK;
    }
    cudaSetDevice(ctx->device);
    unsigned int* d_bits = nullptr;
    DXMC_CUDA(ctx, pool_alloc(ctx, &d_bits, n_materials * sizeof(unsigned int), ctx->upload_stream));
    DXMC_CUDA(ctx, cudaMemsetAsync(d_bits, 0, n_materials * sizeof(unsigned int), ctx->upload_stream));
    DXMC_CUDA(ctx, dev::launch_max_density(w->voxels, w->params.n_voxels, d_bits, n_materials, ctx->upload_stream));
    // voxel materials are below 256: the maxima beyond stay zero
    std::vector<unsigned int> bits(n_materials, 0u);
    const int read = std::min(n_materials, 256);
    DXMC_CUDA(ctx, enqueue_readback(ctx, d_bits, 0, read * sizeof(unsigned int), ctx->upload_stream));
    cudaFreeAsync(d_bits, ctx->upload_stream);
    DXMC_CUDA(ctx, cudaStreamSynchronize(ctx->upload_stream));
    std::memcpy(bits.data(), ctx->readback_host, read * sizeof(unsigned int));
    for (int i = 0; i < n_materials; ++i) {
        float f;
        std::memcpy(&f, &bits[i], sizeof(float));
        out[i] = f;
    }
    return DXMC_OK;
} catch (...) {
    return exception_status(w ? w->ctx : nullptr);
}

void dxmc_gpu_world_free(dxmc_world* w)
{
    if (!w)
        return;
    std::lock_guard<std::mutex> lock(w->ctx->mutex);
    cudaSetDevice(w->ctx->device);
    wait_unused(w->ctx, w->usage); // no queued batch, job or result post-processing still reads the grid
    // the voxels go back to the pool in the order of the upload stream (the host
    // has waited for their readers), so the next upload reuses them without
    // waiting for the jobs queued on the context stream; the grids too
    if (w->voxels)
        cudaFreeAsync(w->voxels, w->ctx->upload_stream);
    if (w->palette_index)
        cudaFreeAsync(w->palette_index, w->ctx->upload_stream);
    if (w->palette)
        cudaFreeAsync(w->palette, w->ctx->upload_stream);
    for (auto& m : w->majorants) {
        cudaFreeAsync(m.cells, w->ctx->upload_stream);
        w->ctx->in_use -= m.bytes;
    }
    w->usage.destroy();
    w->ctx->in_use -= w->bytes;
    delete w;
}

int dxmc_gpu_world_prepare(dxmc_gpu_ctx* ctx, dxmc_world* world, const dxmc_lut* lut)
try {
    if (!ctx || !world || !lut)
        return DXMC_ERR_INVALID;
    std::lock_guard<std::mutex> lock(ctx->mutex);
    if (world->ctx != ctx || lut->ctx != ctx)
        return fail(ctx, DXMC_ERR_INVALID, "world or lut belongs to another context");
    cudaSetDevice(ctx->device);
    ++ctx->submission; // no job of this call holds a grid: every grid but the new one may go
    const dev::MajorantGrid* grid = nullptr;
    return world_majorant(ctx, world, lut, true, &grid); // complete when it returns
} catch (...) {
    return exception_status(ctx);
}

int dxmc_gpu_world_majorant(dxmc_gpu_ctx* ctx, dxmc_world* world, const dxmc_lut* lut, uint32_t* cells_per_axis,
    int32_t* shift, int32_t* bands, float* band_edges, float* box, float* cells)
try {
    if (!ctx || !world || !lut || !cells_per_axis || !shift || !bands)
        return DXMC_ERR_INVALID;
    std::lock_guard<std::mutex> lock(ctx->mutex);
    const dev::MajorantGrid* g = nullptr;
    world_majorant(ctx, world, lut, false, &g);
    if (!g)
        return fail(ctx, DXMC_ERR_STATE, "no local-majorant grid for this world and lut");
    for (int a = 0; a < 3; ++a) {
        shift[a] = g->shift[a];
        cells_per_axis[a] = static_cast<uint32_t>((world->dims[a] + (1ull << g->shift[a]) - 1) >> g->shift[a]);
    }
    *bands = g->bands;
    for (int k = 0; band_edges && k + 1 < g->bands; ++k)
        band_edges[k] = g->band_edge[k];
    cudaSetDevice(ctx->device);
    cudaError_t e = cudaSuccess;
    if (box)
        e = cudaMemcpyAsync(box, g->box, 6 * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess && !cells)
        e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "local-majorant grid read");
    if (cells) {
        const uint64_t n = static_cast<uint64_t>(cells_per_axis[0]) * cells_per_axis[1] * cells_per_axis[2] * g->bands;
        e = cudaMemcpyAsync(cells, g->cells, n * sizeof(float2), cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess)
            return cuda_fail(ctx, e, "local-majorant grid read");
    }
    return DXMC_OK;
} catch (...) {
    return exception_status(ctx);
}

int dxmc_gpu_lut_upload(dxmc_gpu_ctx* ctx, const dxmc_lut_blob* b, dxmc_lut** out)
try {
    if (!ctx || !b || !out || b->n_materials <= 0)
        return DXMC_ERR_INVALID;
    std::lock_guard<std::mutex> lock(ctx->mutex);
    *out = nullptr;
    const int nm = b->n_materials;
    const int R = static_cast<int>(b->resolution());
    dev::LutMeta m {};
    m.n_materials = nm;
    m.R = R;
    m.linear_index = static_cast<int>(b->linear_index);
    m.linear_step = static_cast<float>(b->linear_step);
    m.inv_linear_step = static_cast<float>(1.0 / b->linear_step);
    m.linear_energy = static_cast<float>(b->linear_energy);
    m.max_energy = static_cast<float>(b->max_energy);
    size_t off = 0;
    m.off_x = static_cast<int>(off);
    off = align_up(off + R, 4);
    m.off_coef = static_cast<int>(off);
    off = align_up(off + static_cast<size_t>(nm) * R * 6, 4);
    m.off_maxcoef = static_cast<int>(off);
    off = align_up(off + static_cast<size_t>(R) * 2, 4);
    m.off_rita = static_cast<int>(off);
    off = align_up(off + static_cast<size_t>(nm) * 4 * dev::RITA_N, 4);
    m.off_spline = static_cast<int>(off);
    off = align_up(off + static_cast<size_t>(nm) * dev::SPLINE_FLOATS, 4);
    m.off_shells = static_cast<int>(off);
    off = align_up(off + static_cast<size_t>(nm) * dev::N_SHELLS * dev::SHELL_FLOATS, 4);
    m.total_floats = static_cast<int>(off);
    std::vector<float> img(off, 0.0f);
    for (int i = 0; i < R; ++i)
        img[m.off_x + i] = static_cast<float>(b->log_energy[i]);
    for (size_t i = 0; i < static_cast<size_t>(nm) * R * 6; ++i)
        img[m.off_coef + i] = static_cast<float>(b->coefficients[i]);
    for (int i = 0; i < R * 2; ++i)
        img[m.off_maxcoef + i] = static_cast<float>(b->max_coefficients[i]);
    for (int mat = 0; mat < nm; ++mat) {
        for (int k = 0; k < 4 * dev::RITA_N; ++k)
            img[m.off_rita + mat * 4 * dev::RITA_N + k] = static_cast<float>(b->rita[mat][k]);
        float* sp = img.data() + m.off_spline + mat * dev::SPLINE_FLOATS;
        for (int k = 0; k < 60; ++k)
            sp[k] = static_cast<float>(b->spline[mat][k]);
        sp[60] = static_cast<float>(b->spline[mat][76]);
        sp[61] = static_cast<float>(b->spline[mat][77]);
        sp[62] = static_cast<float>(b->spline[mat][78]);
        sp[63] = static_cast<float>(1.0 / b->spline[mat][77]);
        for (int s = 0; s < dev::N_SHELLS; ++s) {
            const auto& c = b->shells[mat][s];
            float* o = img.data() + m.off_shells + (mat * dev::N_SHELLS + s) * dev::SHELL_FLOATS;
            o[0] = static_cast<float>(c.binding_energy);
            o[1] = static_cast<float>(c.number_electrons);
            o[2] = static_cast<float>(c.hartree_fock_j0);
            o[3] = static_cast<float>(c.photo_ionization_probability);
            o[4] = static_cast<float>(c.fluorescence_yield);
            for (int k = 0; k < 3; ++k) {
                o[5 + k] = static_cast<float>(c.line_probabilities[k]);
                o[8 + k] = static_cast<float>(c.line_energies[k]);
            }
        }
    }
    // inverse-CDF sampling tables for the Compton and Rayleigh samplers, after the
    // part of the image that the kernels stage in shared memory
    {
        const auto tp = dxmc_gb300::host::sampling_tables(*b, SAMPLING_ENERGIES, SAMPLING_LEVELS);
        const auto& t = *tp;
        m.tab_ne = t.ne;
        m.tab_nu = t.nu;
        m.tab_le0 = static_cast<float>(t.le0);
        m.tab_inv_dle = static_cast<float>(1.0 / t.dle);
        m.off_ckn = static_cast<int>(img.size());
        m.off_csf = m.off_ckn + static_cast<int>(t.compton_kn.size());
        m.off_ray = m.off_csf + static_cast<int>(t.compton_sf.size());
        img.insert(img.end(), t.compton_kn.begin(), t.compton_kn.end());
        img.insert(img.end(), t.compton_sf.begin(), t.compton_sf.end());
        img.insert(img.end(), t.rayleigh.begin(), t.rayleigh.end());
    }
    cudaSetDevice(ctx->device);
    auto* lut = new (std::nothrow) dxmc_lut;
    if (!lut)
        return DXMC_ERR_OOM;
    lut->ctx = ctx;
    lut->meta = m;
    static std::atomic<uint64_t> lut_serials { 0 };
    lut->serial = ++lut_serials;
    {
        const auto mr = majorant_ratios(*b, img, m);
        lut->majorant_bands = mr->bands;
        std::copy(std::begin(mr->band_edge), std::end(mr->band_edge), lut->band_edge);
        lut->band_log0 = mr->band_log0;
        lut->band_inv_dlog = mr->band_inv_dlog;
        lut->majorant_ratio = mr->ratio;
        std::copy(std::begin(mr->mu_ref), std::end(mr->mu_ref), lut->mu_ref);
    }
    lut->bytes = img.size() * sizeof(float);
    cudaError_t e = pool_alloc(ctx, &lut->image, lut->bytes, ctx->upload_stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(lut->image, img.data(), lut->bytes, cudaMemcpyHostToDevice, ctx->upload_stream);
    const cudaError_t se = cudaStreamSynchronize(ctx->upload_stream); // img is a local buffer
    if (e == cudaSuccess)
        e = se;
    if (e != cudaSuccess) {
        if (lut->image) {
            cudaFreeAsync(lut->image, ctx->upload_stream);
            cudaStreamSynchronize(ctx->upload_stream);
        }
        delete lut;
        return cuda_fail(ctx, e, "lut upload");
    }
    ctx->in_use += lut->bytes;
    *out = lut;
    return DXMC_OK;
} catch (...) {
    return exception_status(ctx);
}

void dxmc_gpu_lut_free(dxmc_lut* lut)
{
    if (!lut)
        return;
    std::lock_guard<std::mutex> lock(lut->ctx->mutex);
    cudaSetDevice(lut->ctx->device);
    wait_unused(lut->ctx, lut->usage); // no queued batch or job still reads the table
    cudaFreeAsync(lut->image, lut->ctx->upload_stream);
    lut->usage.destroy();
    lut->ctx->in_use -= lut->bytes;
    delete lut;
}

namespace {

// Frees a job's device buffers; `idle`: its kernels and copies are known to be
// done, so the large buffers may serve the next job (the cache) at once.
void free_job_device(dxmc_job* j, bool idle)
{
    cudaStream_t s = j->ctx->stream;
    auto give = [&](void* p, uint64_t bytes) {
        if (!p)
            return;
        if (idle)
            j->ctx->job_buffers.put(p, bytes, s);
        else
            cudaFreeAsync(p, s);
    };
    give(j->records, j->tally_bytes);
    give(j->tally_f32, j->tally_bytes);
    give(j->n_events, j->count_bytes);
    give(j->queue, j->queue_bytes);
    if (j->counters)
        cudaFreeAsync(j->counters, s);
    if (j->tables)
        cudaFreeAsync(j->tables, s);
    if (j->staging) {
        if (!idle)
            cudaStreamSynchronize(s); // the tables copy may still be queued
        j->ctx->staging.give(j->staging, j->staging_class);
        j->staging = nullptr;
    }
    j->queue = nullptr;
    j->records = nullptr;
    j->tally_f32 = nullptr;
    j->n_events = nullptr;
    j->counters = nullptr;
    j->tables = nullptr;
}

} // namespace

namespace {

// Validates a job, builds its host tables, allocates and clears its device
// buffers on the context stream and fills its kernel parameters.  Batched jobs
// get no photon queue.  Caller holds the context mutex.
// Photon queue of a job: its own buffer (single jobs), none (photons generated in
// the persistent multi-job kernel) or a buffer shared by the jobs of one batch
// chain, which run one after another on the chain's stream.
// ---- local-majorant grids ------------------------------------------------------------
#ifndef DXMC_MAJORANT_LEVELS_PER_OCTAVE
#define DXMC_MAJORANT_LEVELS_PER_OCTAVE 6
#endif
constexpr int MAJORANT_LEVELS_PER_OCTAVE = DXMC_MAJORANT_LEVELS_PER_OCTAVE;
// the emptiest level (air and empty cells): scale 2^-12, or 2^-10.5 at six levels per octave;
// levels index a 64-bit mask
constexpr int MAJORANT_MAX_LEVEL = MAJORANT_LEVELS_PER_OCTAVE * 12 < 63 ? MAJORANT_LEVELS_PER_OCTAVE * 12 : 63;
constexpr uint64_t MAJORANT_MAX_CELLS_PER_AXIS = 1024;
constexpr size_t MAJORANT_GRIDS_PER_WORLD = 4;    // one per LUT used with the world, least recently used evicted
constexpr int MAJORANT_MAX_CANDIDATES = 12;       // distance transforms per band at most
constexpr size_t MAJORANT_SCRATCH_BYTES = 512ull << 20; // distance-transform scratch of one group of levels
static_assert(MAJORANT_MAX_CANDIDATES * dev::MAJORANT_MAX_BANDS <= dev::MAJORANT_MAX_PAIRS, "pair table too small");

int majorant_level(float m)
{
    if (m >= 1.0f)
        return 0;
    if (!(m > 0.0f))
        return MAJORANT_MAX_LEVEL;
    int lv = std::min(MAJORANT_MAX_LEVEL, static_cast<int>(std::floor(-MAJORANT_LEVELS_PER_OCTAVE * std::log2(m))));
    while (lv > 0 && std::exp2(-static_cast<double>(lv) / MAJORANT_LEVELS_PER_OCTAVE) < m)
        --lv;
    return lv;
}

// The local-majorant grid of (world, lut): found in the world's cache, else (if
// build) built on the context stream and cached.  Caller holds the context mutex.
// A grid that a job of the current submission (ctx->submission) copied into its
// parameters is not evicted before that submission has launched.
int world_majorant(dxmc_gpu_ctx* ctx, dxmc_world* w, const dxmc_lut* lut, bool build, const dev::MajorantGrid** out)
{
    *out = nullptr;
    for (auto& m : w->majorants) {
        if (m.lut_serial == lut->serial) {
            m.last_use = ++w->majorant_clock;
            m.submission = ctx->submission;
            *out = &m.grid;
            return DXMC_OK;
        }
    }
    if (!build)
        return DXMC_OK;
    if (lut->meta.n_materials < w->n_materials)
        return fail(ctx, DXMC_ERR_INVALID, "lut has fewer materials than the world");
    dev::MajorantBuild b {};
    int shift[3];
    for (int a = 0; a < 3; ++a) {
        int sh = static_cast<int>(std::lround(std::log2(std::max(MAJORANT_CELL_MM / w->spacing[a], 1.0))));
        sh = std::min(std::max(sh, 0), 6);
        while (((w->dims[a] + (1ull << sh) - 1) >> sh) > MAJORANT_MAX_CELLS_PER_AXIS)
            ++sh;
        shift[a] = sh;
    }
    auto cells_along = [&](int a) { return (w->dims[a] + (1ull << shift[a]) - 1) >> shift[a]; };
    // the kernels index (cell, band) pairs in 32 bits: coarser cells for huge grids
    while (cells_along(0) * cells_along(1) * cells_along(2) * static_cast<uint64_t>(lut->majorant_bands) >= (1ull << 31)) {
        const int a = cells_along(0) >= cells_along(1) ? (cells_along(0) >= cells_along(2) ? 0 : 2) : (cells_along(1) >= cells_along(2) ? 1 : 2);
        ++shift[a];
    }
    uint64_t ncell = 1;
    for (int a = 0; a < 3; ++a) {
        b.shift[a] = shift[a];
        b.n[a] = static_cast<uint32_t>(cells_along(a));
        b.edge[a] = static_cast<float>(w->spacing[a] * static_cast<double>(1ull << shift[a]));
        ncell *= b.n[a];
    }
    b.levels_per_octave = MAJORANT_LEVELS_PER_OCTAVE;
    b.max_level = MAJORANT_MAX_LEVEL;
    b.bands = lut->majorant_bands;
    // per band, the voxel scales and (compact layout) the palette's own levels
    const int nm = lut->meta.n_materials;
    std::vector<float> scales(static_cast<size_t>(b.bands) * dev::PALETTE_MAX, 0.0f);
    std::vector<uint64_t> levels(b.bands, 0);
    for (int band = 0; band < b.bands; ++band) {
        const float* ratio = lut->majorant_ratio.data() + static_cast<size_t>(band) * nm;
        if (w->palette_index) {
            for (size_t i = 0; i < w->host_palette.size() && i < static_cast<size_t>(dev::PALETTE_MAX); ++i) {
                const auto& pe = w->host_palette[i];
                const int mat = static_cast<int>(pe.code & 0xffu);
                const bool meas = ((pe.code >> 8) & 0xffu) != 0;
                const float sc = meas ? 1.0f : pe.density * ratio[mat];
                scales[static_cast<size_t>(band) * dev::PALETTE_MAX + i] = sc;
                levels[band] |= 1ull << majorant_level(sc);
            }
        } else {
            // the levels come from the device histogram
            for (int m = 0; m < nm && m < dev::PALETTE_MAX; ++m)
                scales[static_cast<size_t>(band) * dev::PALETTE_MAX + m] = ratio[m];
        }
    }
    // each band's emptiest level: the palette's highest level; for the 8-byte layout it
    // comes from the device's level histogram after the first level pass (below)
    std::vector<int> floor_level(b.bands, -1);
    bool use_box = false;
    if (w->palette_index && DXMC_MAJORANT_BOX) {
        for (int band = 0; band < b.bands; ++band) {
            for (int lv = MAJORANT_MAX_LEVEL; lv >= 0; --lv) {
                if (levels[band] >> lv & 1ull) {
                    floor_level[band] = lv;
                    break;
                }
            }
            use_box = use_box || floor_level[band] >= 0;
        }
    }
    const uint64_t cell_bytes = ncell * b.bands * sizeof(float2) + 8 * sizeof(float); // + the box
    if (ctx->in_use + cell_bytes > ctx->budget)
        return fail(ctx, DXMC_ERR_OOM, "local-majorant grid exceeds the device memory budget");
    // least recently used first, never a grid the current submission reads
    // (the cache may then hold more grids until a later submission)
    while (w->majorants.size() >= MAJORANT_GRIDS_PER_WORLD) {
        auto victim = w->majorants.end();
        for (auto it = w->majorants.begin(); it != w->majorants.end(); ++it)
            if (it->submission != ctx->submission && (victim == w->majorants.end() || it->last_use < victim->last_use))
                victim = it;
        if (victim == w->majorants.end())
            break;
        sync_ctx_streams(ctx); // no queued job still reads the grid
        cudaFreeAsync(victim->cells, ctx->upload_stream);
        ctx->in_use -= victim->bytes;
        w->majorants.erase(victim);
    }
    // built on the upload stream (greatest priority) and complete before the call
    // returns, so jobs on any stream read it without a cross-stream wait
    cudaStream_t s = ctx->upload_stream;
    float2* cells = nullptr;
    uint8_t* level = nullptr;
    uint8_t* minlev = nullptr;
    float *d0 = nullptr, *d1 = nullptr, *cost = nullptr, *d_scales = nullptr;
    int* bounds = nullptr;
    unsigned int* d_hist = nullptr;
    cudaError_t e = pool_alloc(ctx, &cells, cell_bytes, s);
    float* box = cells ? reinterpret_cast<float*>(cells + ncell * b.bands) : nullptr;
    if (e == cudaSuccess)
        e = pool_alloc(ctx, &bounds, 6 * sizeof(int), s);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(bounds, 0x7f, 3 * sizeof(int), s); // minima start large
    if (e == cudaSuccess)
        e = cudaMemsetAsync(bounds + 3, 0xff, 3 * sizeof(int), s); // maxima start at -1
    if (e == cudaSuccess)
        e = pool_alloc(ctx, &level, ncell * b.bands, s);
    if (e == cudaSuccess)
        e = pool_alloc(ctx, &minlev, ncell * b.bands, s);
    if (e == cudaSuccess)
        e = pool_alloc(ctx, &cost, ncell * b.bands * sizeof(float), s);
    if (e == cudaSuccess)
        e = pool_alloc(ctx, &d_scales, scales.size() * sizeof(float), s);
    if (e == cudaSuccess) // pageable source: staged before the call returns
        e = cudaMemcpyAsync(d_scales, scales.data(), scales.size() * sizeof(float), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = pool_alloc(ctx, &d_hist, static_cast<size_t>(b.bands) * 64 * sizeof(unsigned int), s);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(d_hist, 0, static_cast<size_t>(b.bands) * 64 * sizeof(unsigned int), s);
    for (int a = 0; a < 3; ++a)
        b.lower[a] = w->params.lower[a];
    for (int band = 0; band < dev::MAJORANT_MAX_BANDS; ++band) {
        b.floor_levels[band] = band < b.bands ? floor_level[band] : -1;
        b.mu_refs[band] = band < b.bands ? lut->mu_ref[band] : 0.0f;
    }
    // the levels of every band in one pass over the voxels, then the distance
    // transforms band by band
    if (e == cudaSuccess)
        e = dev::launch_majorant_levels(w->params, d_scales, b, level, cells, cost, bounds, d_hist, s);
    // the levels worth a distance transform: those the cells actually have, at
    // most MAJORANT_MAX_CANDIDATES per band (the most populated, and the
    // emptiest one for the body box); any subset gives a valid grid
    std::vector<unsigned int> hist(static_cast<size_t>(b.bands) * 64, 0u);
    if (e == cudaSuccess)
        e = enqueue_readback(ctx, d_hist, 0, hist.size() * sizeof(unsigned int), s);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s);
    if (e == cudaSuccess)
        std::memcpy(hist.data(), ctx->readback_host, hist.size() * sizeof(unsigned int));
    // 8-byte layout: the host learns the cells' levels only now.  Each band's emptiest
    // level is the lowest of the run of populated levels that ends at its highest one
    // (air and what is as thin as air; the body lies levels below), and the level pass
    // runs again with those levels to find the box of the cells above them
    if (e == cudaSuccess && !w->palette_index && DXMC_MAJORANT_BOX) {
        for (int band = 0; band < b.bands; ++band) {
            const unsigned int* hb = hist.data() + static_cast<size_t>(band) * 64;
            int top = -1;
            for (int lv = MAJORANT_MAX_LEVEL; lv >= 0 && top < 0; --lv)
                if (hb[lv])
                    top = lv;
            int floor = top;
            while (floor > 1 && hb[floor - 1])
                --floor;
            floor_level[band] = floor >= 1 ? floor : -1;
            b.floor_levels[band] = floor_level[band];
            use_box = use_box || floor_level[band] >= 0;
        }
        if (use_box)
            e = dev::launch_majorant_levels(w->params, d_scales, b, level, cells, cost, bounds, d_hist, s);
    }
    // each cell's lowest level over its neighbourhood: the dilated set of every level
    if (e == cudaSuccess)
        e = dev::launch_majorant_minfilter(b, level, minlev, s);
    std::vector<std::pair<int, int>> pairs; // (band, level), band-major, levels ascending
    for (int band = 0; band < b.bands && e == cudaSuccess; ++band) {
        std::vector<std::pair<unsigned int, int>> present; // (cells, level)
        for (int lv = 1; lv <= MAJORANT_MAX_LEVEL; ++lv)
            if (hist[static_cast<size_t>(band) * 64 + lv])
                present.emplace_back(hist[static_cast<size_t>(band) * 64 + lv], lv);
        std::sort(present.begin(), present.end(), [](const auto& x, const auto& y) { return x.first > y.first; });
        uint64_t chosen = 0;
        if (floor_level[band] >= 1 && hist[static_cast<size_t>(band) * 64 + floor_level[band]])
            chosen |= 1ull << floor_level[band];
        int n_chosen = __builtin_popcountll(chosen);
        for (const auto& pr : present)
            if (n_chosen < MAJORANT_MAX_CANDIDATES && !(chosen >> pr.second & 1ull)) {
                chosen |= 1ull << pr.second;
                ++n_chosen;
            }
        for (int lv = 1; lv <= MAJORANT_MAX_LEVEL; ++lv)
            if (chosen >> lv & 1ull)
                pairs.emplace_back(band, lv);
    }
    // the distance transforms of many pairs run as one launch per pass, in groups
    // whose two scratch grids stay within MAJORANT_SCRATCH_BYTES and what the
    // context's budget leaves beside the grid and the build's other buffers (one
    // pair at a time if it leaves less)
    const uint64_t held = ctx->in_use + cell_bytes + ncell * b.bands * (2 + sizeof(float));
    const uint64_t room = std::min<uint64_t>(MAJORANT_SCRATCH_BYTES, ctx->budget > held ? ctx->budget - held : 0);
    const size_t group = std::clamp<size_t>(room / (2 * ncell * sizeof(float)), 1,
        std::min<size_t>(std::max<size_t>(pairs.size(), 1), dev::MAJORANT_MAX_PAIRS));
    if (e == cudaSuccess && !pairs.empty())
        e = pool_alloc(ctx, &d0, group * ncell * sizeof(float), s);
    if (e == cudaSuccess && !pairs.empty())
        e = pool_alloc(ctx, &d1, group * ncell * sizeof(float), s);
    for (size_t g0 = 0; g0 < pairs.size() && e == cudaSuccess; g0 += group) {
        dev::MajorantPairs pg {};
        pg.count = static_cast<int>(std::min(group, pairs.size() - g0));
        for (int i = 0; i < pg.count; ++i) {
            pg.band[i] = static_cast<uint8_t>(pairs[g0 + i].first);
            pg.level[i] = static_cast<uint8_t>(pairs[g0 + i].second);
        }
        for (int band = 0, i = 0; band <= dev::MAJORANT_MAX_BANDS; ++band) {
            while (i < pg.count && pg.band[i] < band)
                ++i;
            pg.first[band] = i;
        }
        e = dev::launch_majorant_level_passes(b, pg, minlev, d0, d1, cells, cost, s);
    }
    static const float no_box[6] = { INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY };
    if (e == cudaSuccess && use_box)
        e = dev::launch_majorant_box(b, bounds, cells, box, s);
    else if (e == cudaSuccess) // an empty box: no cell is marked, the read-back says so
        e = cudaMemcpyAsync(box, no_box, sizeof(no_box), cudaMemcpyHostToDevice, s);
    for (void* ptr : { static_cast<void*>(level), static_cast<void*>(minlev), static_cast<void*>(d0), static_cast<void*>(d1), static_cast<void*>(cost),
             static_cast<void*>(bounds), static_cast<void*>(d_scales), static_cast<void*>(d_hist) })
        if (ptr)
            cudaFreeAsync(ptr, s);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        if (cells)
            cudaFreeAsync(cells, s);
        cudaStreamSynchronize(s);
        return cuda_fail(ctx, e, "local-majorant grid");
    }
    MajorantCache m;
    m.lut_serial = lut->serial;
    m.cells = cells;
    m.bytes = cell_bytes;
    m.last_use = ++w->majorant_clock;
    m.submission = ctx->submission;
    m.grid.cells = cells;
    m.grid.box = box;
    m.grid.nx = b.n[0];
    m.grid.nxy = b.n[0] * b.n[1];
    for (int a = 0; a < 3; ++a)
        m.grid.shift[a] = b.shift[a];
    m.grid.bands = b.bands;
    for (int k = 0; k < dev::MAJORANT_MAX_BANDS - 1; ++k)
        m.grid.band_edge[k] = lut->band_edge[k];
    m.grid.band_log0 = lut->band_log0;
    m.grid.band_inv_dlog = lut->band_inv_dlog;
    ctx->in_use += cell_bytes;
    w->majorants.push_back(m);
    *out = &w->majorants.back().grid;
    return DXMC_OK;
}

int job_tracking(const dxmc_gpu_ctx* ctx, const dxmc_job_desc* jd)
{
    const int t = jd->tracking != DXMC_TRACKING_DEFAULT ? jd->tracking : ctx->options.tracking;
    return t == DXMC_TRACKING_GLOBAL ? DXMC_TRACKING_GLOBAL : DXMC_TRACKING_LOCAL;
}

enum class QueueMode { own, none, shared };

int prepare_job(dxmc_gpu_ctx* ctx, dxmc_world* world, dxmc_lut* lut, const dxmc_job_desc* jd, QueueMode qmode,
    uint64_t shared_capacity, dxmc_job** out, dev::TransportParams& p, uint64_t& chunk_out)
{
    *out = nullptr;
    if (world->ctx != ctx || lut->ctx != ctx)
        return fail(ctx, DXMC_ERR_INVALID, "world or lut belongs to another context");
    if (!jd->exposures || jd->n_exposures == 0 || jd->n_exposures > 0xffffffffull)
        return fail(ctx, DXMC_ERR_INVALID, "job needs at least one exposure");
    if (jd->model < 0 || jd->model > 2)
        return fail(ctx, DXMC_ERR_INVALID, "unknown low-energy correction model");
    if (lut->meta.n_materials < world->n_materials)
        return fail(ctx, DXMC_ERR_INVALID, "lut has fewer materials than the world");
    const int tally_mode = jd->tally_mode >= 0 ? jd->tally_mode : ctx->options.tally_mode;
    if (tally_mode < 0 || tally_mode > 2)
        return fail(ctx, DXMC_ERR_INVALID, "unknown tally mode");
    if (jd->tracking < DXMC_TRACKING_DEFAULT || jd->tracking > DXMC_TRACKING_LOCAL)
        return fail(ctx, DXMC_ERR_INVALID, "unknown tracking mode");
    if (jd->direction != DXMC_DIRECTION_REFERENCE && jd->direction != DXMC_DIRECTION_NORMALIZED)
        return fail(ctx, DXMC_ERR_INVALID, "unknown direction mode");
    if (jd->precision != DXMC_PRECISION_FP32 && jd->precision != DXMC_PRECISION_FP64)
        return fail(ctx, DXMC_ERR_INVALID, "unknown precision");

    // ---- host-side tables: exposures, prefix offsets, spectrum, heel, bow-tie ----
    const uint64_t ne = jd->n_exposures;
    std::vector<dev::DevExposure> ex(ne);
    std::vector<uint64_t> offsets(ne + 1, 0);
    for (uint64_t i = 0; i < ne; ++i) {
        const dxmc_exposure& s = jd->exposures[i];
        dev::DevExposure& d = ex[i];
        std::memset(&d, 0, sizeof(d));
        for (int k = 0; k < 3; ++k) {
            d.pos[k] = static_cast<float>(s.position[k]);
            d.cosx[k] = static_cast<float>(s.direction_cosines[k]);
            d.cosy[k] = static_cast<float>(s.direction_cosines[3 + k]);
            d.beam[k] = static_cast<float>(s.beam_direction[k]);
        }
        for (int k = 0; k < 4; ++k)
            d.coll[k] = static_cast<float>(s.collimation[k]);
        d.weight = static_cast<float>(s.weight);
        d.mono_energy = static_cast<float>(s.mono_energy);
        offsets[i + 1] = offsets[i] + s.n_histories;
    }
    const uint64_t total = offsets[ne];
    if (total == 0)
        return fail(ctx, DXMC_ERR_INVALID, "job has no histories");
    std::vector<float> spec_e, spec_p;
    std::vector<uint32_t> spec_a;
    if (jd->spectrum) {
        const int n = jd->spectrum->n;
        if (n <= 0 || !jd->spectrum->energies || !jd->spectrum->weights)
            return fail(ctx, DXMC_ERR_INVALID, "invalid spectrum");
        std::vector<double> w(jd->spectrum->weights, jd->spectrum->weights + n), probs;
        std::vector<uint64_t> alias;
        host::build_alias_table(w, probs, alias);
        for (int i = 0; i < n; ++i) {
            spec_e.push_back(static_cast<float>(jd->spectrum->energies[i]));
            spec_p.push_back(static_cast<float>(probs[i]));
            spec_a.push_back(static_cast<uint32_t>(alias[i]));
        }
    }
    std::vector<float> heel;
    if (jd->heel) {
        const auto* h = jd->heel;
        if (h->energy_size <= 0 || h->angle_size <= 0 || !h->weights || !(h->energy_step > 0) || !(h->angle_step != 0))
            return fail(ctx, DXMC_ERR_INVALID, "invalid heel table");
        // the table size in 64 bits: a product that wraps in int would leave the kernel
        // indexing a short table with the caller's (huge) sizes
        const int64_t heel_n = static_cast<int64_t>(h->energy_size) * h->angle_size;
        if (heel_n > DXMC_MAX_HEEL_WEIGHTS)
            return fail(ctx, DXMC_ERR_INVALID, "heel table has " + std::to_string(heel_n) + " weights, more than the maximum of "
                    + std::to_string(DXMC_MAX_HEEL_WEIGHTS));
        heel.assign(h->weights, h->weights + heel_n);
    }
    std::vector<float> bt_a, bt_w;
    if (jd->bowtie) {
        // BowTieFilter constructor: |angle|, sort, normalise to mean 1 (beamfilters.hpp:86-130)
        const int n = jd->bowtie->n;
        if (n > DXMC_MAX_BOWTIE_POINTS)
            return fail(ctx, DXMC_ERR_INVALID, "bow-tie table has " + std::to_string(n) + " points, more than the maximum of "
                    + std::to_string(DXMC_MAX_BOWTIE_POINTS));
        std::vector<double> ta(n > 0 ? n : 0), tw(n > 0 ? n : 0);
        if (dxmc_bowtie_table(jd->bowtie->angles, jd->bowtie->weights, n, ta.data(), tw.data()) != DXMC_OK)
            return fail(ctx, DXMC_ERR_INVALID, "invalid bow-tie table");
        bt_a.assign(ta.begin(), ta.end());
        bt_w.assign(tw.begin(), tw.end());
    }
    // one device buffer for all tables
    size_t off = 0;
    const size_t off_ex = off;
    off = align_up(off + ne * sizeof(dev::DevExposure), 256);
    const size_t off_offsets = off;
    off = align_up(off + (ne + 1) * sizeof(uint64_t), 256);
    const size_t off_se = off;
    off = align_up(off + spec_e.size() * 4, 256);
    const size_t off_sp = off;
    off = align_up(off + spec_p.size() * 4, 256);
    const size_t off_sa = off;
    off = align_up(off + spec_a.size() * 4, 256);
    const size_t off_heel = off;
    off = align_up(off + heel.size() * 4, 256);
    const size_t off_bta = off;
    off = align_up(off + bt_a.size() * 4, 256);
    const size_t off_btw = off;
    off = align_up(off + bt_w.size() * 4, 256);
    const size_t table_bytes = off;
    std::vector<unsigned char> tables(table_bytes, 0);
    std::memcpy(tables.data() + off_ex, ex.data(), ne * sizeof(dev::DevExposure));
    std::memcpy(tables.data() + off_offsets, offsets.data(), (ne + 1) * sizeof(uint64_t));
    std::memcpy(tables.data() + off_se, spec_e.data(), spec_e.size() * 4);
    std::memcpy(tables.data() + off_sp, spec_p.data(), spec_p.size() * 4);
    std::memcpy(tables.data() + off_sa, spec_a.data(), spec_a.size() * 4);
    std::memcpy(tables.data() + off_heel, heel.data(), heel.size() * 4);
    std::memcpy(tables.data() + off_bta, bt_a.data(), bt_a.size() * 4);
    std::memcpy(tables.data() + off_btw, bt_w.data(), bt_w.size() * 4);

    const uint64_t nv = world->params.n_voxels;
    const uint64_t tally_bytes = tally_mode == 1 ? nv * 2 * sizeof(float) : nv * sizeof(dev::TallyRecord);
    const uint64_t count_bytes = tally_mode == 1 ? nv * sizeof(uint32_t) : 0; // records hold their counts
    // photon queue: chunks of 2^k histories, 48 bytes per queued photon
    const int log2_option = jd->queue_log2_chunk != 0 ? jd->queue_log2_chunk : ctx->options.queue_log2_chunk;
    // FP64 jobs generate their photons in the kernel (the queue holds FP32 photons)
    const int log2_chunk = jd->precision == DXMC_PRECISION_FP64 ? -1 : (log2_option == 0 ? DEFAULT_QUEUE_LOG2 : log2_option);
    uint64_t chunk = 0;
    if (log2_chunk >= 0 && qmode == QueueMode::own)
        chunk = std::min<uint64_t>(total, 1ull << std::min(log2_chunk, 34));
    else if (log2_chunk >= 0 && qmode == QueueMode::shared)
        chunk = std::min<uint64_t>({ total, shared_capacity, 1ull << std::min(log2_chunk, 34) });
    const uint64_t queue_bytes = qmode == QueueMode::own ? chunk * 48 : 0;
    const uint64_t job_bytes = tally_bytes + count_bytes + table_bytes + sizeof(dev::JobCounters) + queue_bytes;
    if (ctx->in_use + ctx->job_buffers.held + job_bytes > ctx->budget)
        ctx->job_buffers.release(ctx->stream); // idle buffers give way to the job
    if (ctx->in_use + job_bytes > ctx->budget)
        return fail(ctx, DXMC_ERR_OOM, "job exceeds the device memory budget");

    cudaSetDevice(ctx->device);
    const dev::MajorantGrid* grid = nullptr;
    if (job_tracking(ctx, jd) == DXMC_TRACKING_LOCAL) {
        const int rc = world_majorant(ctx, world, lut, true, &grid);
        if (rc != DXMC_OK)
            return rc;
        if (ctx->in_use + job_bytes > ctx->budget)
            return fail(ctx, DXMC_ERR_OOM, "job exceeds the device memory budget");
    }
    auto* j = new (std::nothrow) dxmc_job;
    if (!j)
        return DXMC_ERR_OOM;
    j->ctx = ctx;
    j->world = world;
    j->histories = total;
    j->tally_mode = tally_mode;
    j->bytes = job_bytes;
    cudaStream_t s = ctx->stream;
    cudaError_t e = cudaSuccess;
    j->tally_bytes = tally_bytes;
    j->count_bytes = count_bytes;
    j->queue_bytes = queue_bytes;
    if (tally_mode == 1) {
        e = job_alloc(ctx, &j->tally_f32, tally_bytes, s);
        if (e == cudaSuccess)
            e = job_alloc(ctx, &j->n_events, count_bytes, s);
    } else {
        e = job_alloc(ctx, &j->records, tally_bytes, s);
    }
    if (e == cudaSuccess)
        e = pool_alloc(ctx, &j->counters, sizeof(dev::JobCounters), s);
    if (e == cudaSuccess)
        e = pool_alloc(ctx, &j->tables, table_bytes, s);
    if (e == cudaSuccess && queue_bytes)
        e = job_alloc(ctx, &j->queue, queue_bytes, s);
    if (e == cudaSuccess)
        e = cudaEventCreate(&j->begin);
    if (e == cudaSuccess)
        e = cudaEventRecord(j->begin, s);
    if (e == cudaSuccess)
        e = ctx->pinned.take(&j->cancel_host, &j->cancel_dev);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(j->records ? static_cast<void*>(j->records) : static_cast<void*>(j->tally_f32), 0, tally_bytes, s);
    if (e == cudaSuccess && j->n_events)
        e = cudaMemsetAsync(j->n_events, 0, count_bytes, s);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(j->counters, 0, sizeof(dev::JobCounters), s);
    if (e == cudaSuccess)
        e = ctx->staging.take(table_bytes, &j->staging, &j->staging_class);
    if (e == cudaSuccess) {
        std::memcpy(j->staging, tables.data(), table_bytes);
        e = cudaMemcpyAsync(j->tables, j->staging, table_bytes, cudaMemcpyHostToDevice, s);
    }
    if (e == cudaSuccess)
        e = cudaEventCreate(&j->start);
    if (e == cudaSuccess)
        e = cudaEventCreate(&j->stop);
    if (e != cudaSuccess) {
        free_job_device(j, false);
        if (j->cancel_host)
            ctx->pinned.give(j->cancel_host, j->cancel_dev);
        delete j;
        return cuda_fail(ctx, e, "job allocation");
    }

    p = dev::TransportParams {};
    p.world = world->params;
    auto& S = p.source;
    S.exposures = reinterpret_cast<const dev::DevExposure*>(j->tables + off_ex);
    S.history_offsets = reinterpret_cast<const uint64_t*>(j->tables + off_offsets);
    S.n_exposures = static_cast<uint32_t>(ne);
    S.spec_n = static_cast<int>(spec_e.size());
    S.spec_energy = reinterpret_cast<const float*>(j->tables + off_se);
    S.spec_prob = reinterpret_cast<const float*>(j->tables + off_sp);
    S.spec_alias = reinterpret_cast<const uint32_t*>(j->tables + off_sa);
    if (jd->heel) {
        S.heel_weights = reinterpret_cast<const float*>(j->tables + off_heel);
        S.heel_e_start = static_cast<float>(jd->heel->energy_start);
        S.heel_e_step = static_cast<float>(jd->heel->energy_step);
        S.heel_e_size = jd->heel->energy_size;
        S.heel_a_size = jd->heel->angle_size;
        S.heel_a_start = static_cast<float>(jd->heel->angle_start);
        S.heel_a_step = static_cast<float>(jd->heel->angle_step);
    }
    if (jd->bowtie) {
        S.bowtie_angle = reinterpret_cast<const float*>(j->tables + off_bta);
        S.bowtie_weight = reinterpret_cast<const float*>(j->tables + off_btw);
        S.bowtie_n = static_cast<int>(bt_a.size());
    }
    p.lut = lut->image;
    p.lut_meta = lut->meta;
    p.records = j->records;
    p.tally = nullptr;
    p.tally_f32 = j->tally_f32;
    p.n_events = j->n_events;
    p.counters = j->counters;
    p.cancel = j->cancel_dev;
    p.total_histories = total;
    p.seed = jd->seed;
    p.tally_mode = tally_mode;
    p.precision = jd->precision;
    p.uniform_hpe = 0;
    {
        bool uniform = true;
        for (uint64_t i = 1; i < ne && uniform; ++i)
            uniform = jd->exposures[i].n_histories == jd->exposures[0].n_histories;
        if (uniform) {
            p.uniform_hpe = jd->exposures[0].n_histories;
            if (p.uniform_hpe <= 0xffffffffull) {
                const auto q = udiv_magic(static_cast<uint32_t>(p.uniform_hpe));
                p.hpe_magic = q.m;
                p.hpe_shifts = q.shifts;
            }
        }
    }
    {
        // job value, else context option, else the default for the generation mode
        const bool queued = chunk > 0;
        const int regen = jd->regen_threshold > 0 ? jd->regen_threshold : ctx->options.regen_threshold;
        const int inter = jd->interact_threshold > 0 ? jd->interact_threshold : ctx->options.interact_threshold;
        const int regen_default = queued ? DEFAULT_QUEUE_REGEN_THRESHOLD : (grid ? DEFAULT_LOCAL_REGEN_THRESHOLD : DEFAULT_REGEN_THRESHOLD);
        p.regen_threshold = regen > 0 ? std::min(regen, 32) : regen_default;
        p.interact_threshold = inter > 0 ? std::min(inter, 32) : (queued ? DEFAULT_QUEUE_INTERACT_THRESHOLD : DEFAULT_INTERACT_THRESHOLD);
        p.woodcock_burst = jd->woodcock_burst > 0 ? std::min(jd->woodcock_burst, 64)
                                                  : (grid ? DEFAULT_LOCAL_WOODCOCK_BURST : DEFAULT_WOODCOCK_BURST);
    }
    if (grid)
        p.majorant = *grid;
    p.normalize_direction = jd->direction == DXMC_DIRECTION_NORMALIZED ? 1 : 0;


    chunk_out = chunk;
    *out = j;
    return DXMC_OK;
}

void discard_job(dxmc_job* j)
{
    free_job_device(j, false);
    if (j->cancel_host)
        j->ctx->pinned.give(j->cancel_host, j->cancel_dev);
    if (j->begin)
        cudaEventDestroy(j->begin);
    if (j->start)
        cudaEventDestroy(j->start);
    if (j->stop)
        cudaEventDestroy(j->stop);
    delete j;
}

struct LaunchPlan {
    int grid = 0, block = 256, gen_grid = 0;
    size_t smem = 0;
};

// Grid, block and shared memory of a job's transport kernel; sets p.lut_in_smem.
LaunchPlan plan_launch(dxmc_gpu_ctx* ctx, const dxmc_world* world, const dxmc_lut* lut, const dxmc_job_desc* jd, dev::TransportParams& p)
{
    const int model = jd->model;
    LaunchPlan L;
    const size_t lut_bytes = static_cast<size_t>(lut->meta.total_floats) * sizeof(float);
    const size_t smem_limit = std::min<size_t>(ctx->max_smem_optin, 96 * 1024);
    p.lut_in_smem = lut_bytes <= smem_limit ? 1 : 0;
    const bool palette = world->palette_index != nullptr;
    L.smem = dev::transport_smem_bytes(lut_bytes, p.lut_in_smem != 0, palette);
    L.block = jd->block_size == 128 || jd->block_size == 256 ? jd->block_size
                                                              : (ctx->options.block_size > 0 ? ctx->options.block_size : 256);
    // also sets the kernel's dynamic shared-memory limit for this launch
    const int occ = dev::transport_max_blocks_per_sm(model, palette, L.block, L.smem, p.precision);
    int per_sm = jd->blocks_per_sm > 0 ? std::min(jd->blocks_per_sm, std::max(occ, 1))
                                        : (ctx->options.blocks_per_sm > 0 ? ctx->options.blocks_per_sm : occ);
    if (per_sm <= 0)
        per_sm = 1;
    L.grid = ctx->sm_count * per_sm;
    L.gen_grid = ctx->sm_count * 8;
    return L;
}

cudaError_t record(cudaEvent_t ev, cudaStream_t s, bool capturing)
{
    return capturing ? cudaEventRecordWithFlags(ev, s, cudaEventRecordExternal) : cudaEventRecord(ev, s);
}

// Queues one job on stream s: the transport kernel alone (photons generated in
// the kernel) or, per chunk of the photon queue, a counter reset, the generation
// pass and the transport kernel.  Records the job's start and stop events.
cudaError_t enqueue_job(dxmc_job* j, dev::TransportParams p, int model, uint64_t chunk, unsigned char* queue,
    const LaunchPlan& L, cudaStream_t s, bool capturing)
{
    cudaError_t e = cudaSuccess;
    if (chunk == 0) {
        e = record(j->start, s, capturing);
        if (e == cudaSuccess)
            e = dev::launch_transport(p, model, L.grid, L.block, L.smem, s);
    } else {
        p.queue.pos_energy = reinterpret_cast<float4*>(queue);
        p.queue.dir_weight = reinterpret_cast<float4*>(queue + chunk * 16);
        p.queue.rng = reinterpret_cast<uint4*>(queue + chunk * 32);
        p.queue.capacity = chunk;
        const uint64_t total = j->histories;
        for (uint64_t first = 0; first < total && e == cudaSuccess; first += chunk) {
            const uint64_t count = std::min(chunk, total - first);
            // queue_count and next_photon restart for every chunk
            e = cudaMemsetAsync(&j->counters->queue_count, 0, 2 * sizeof(unsigned long long), s);
            if (e == cudaSuccess)
                e = dev::launch_generate(p, first, count, L.gen_grid, s);
            if (e == cudaSuccess && first == 0)
                e = record(j->start, s, capturing);
            if (e == cudaSuccess)
                e = dev::launch_transport(p, model, L.grid, L.block, L.smem, s);
        }
    }
    if (e == cudaSuccess)
        e = record(j->stop, s, capturing);
    return e;
}

} // namespace

int dxmc_gpu_job_submit(dxmc_gpu_ctx* ctx, dxmc_world* world, dxmc_lut* lut, const dxmc_job_desc* jd, dxmc_job** out)
try {
    if (!ctx || !world || !lut || !jd || !out)
        return DXMC_ERR_INVALID;
    std::lock_guard<std::mutex> lock(ctx->mutex);
    ++ctx->submission;
    dev::TransportParams p {};
    uint64_t chunk = 0;
    dxmc_job* j = nullptr;
    const int rc = prepare_job(ctx, world, lut, jd, QueueMode::own, 0, &j, p, chunk);
    if (rc != DXMC_OK)
        return rc;
    const LaunchPlan L = plan_launch(ctx, world, lut, jd, p);
    cudaError_t e = enqueue_job(j, p, jd->model, chunk, j->queue, L, ctx->stream, false);
    if (e == cudaSuccess)
        e = world->usage.mark(world->usage.on_stream, ctx->stream);
    if (e == cudaSuccess)
        e = lut->usage.mark(lut->usage.on_stream, ctx->stream);
    if (e != cudaSuccess) {
        cudaStreamSynchronize(ctx->stream);
        discard_job(j);
        return cuda_fail(ctx, e, "transport launch");
    }
    ctx->in_use += j->bytes;
    *out = j;
    return DXMC_OK;
} catch (...) {
    return exception_status(ctx);
}

// ---- batches --------------------------------------------------------------------------
//
// Two ways to run a batch:
//
// * concurrent (default): every job keeps the single-job kernels (parameters in
//   the kernel's constant bank, LUT staged in shared memory, photon queue).  The
//   context owns a few chains (a stream and a photon-queue buffer each); a batch
//   deals its jobs longest-first onto the chains with the least outstanding work,
//   shortest-first within a chain, and launches each chain's share on the chain's
//   stream (a one-off sequence: instantiating it as a graph would cost more than
//   its few launches).  Chains run side by side, so one job's
//   blocks fill the SMs as another chain's job drains, and a batch submitted while
//   others run queues behind them chain by chain (continuous batching); jobs on a
//   chain run one after another, which is what lets them share its queue buffer.
// * persistent: one multi-job kernel per correction model drains work items
//   (job, first history, count) of all jobs from a device-side queue.  Its graph
//   is instantiated once per engine: three host-to-device copies (job parameters,
//   items, control block) and the three kernels as independent nodes; only the
//   copy sizes change between batches.  Two engines are used in turn.
constexpr int MAX_BATCH_JOBS = 4096;
constexpr uint64_t MAX_BATCH_ITEMS = 1ull << 20;
constexpr int MAX_CHAINS = 8;
constexpr int DEFAULT_CHAINS = 2;

struct BatchEngine {
    bool ready = false;
    cudaStream_t stream = nullptr;
    dev::TransportParams* d_params = nullptr;
    dev::BatchItem* d_items = nullptr;
    dev::BatchControl* d_control = nullptr;
    dev::TransportParams* h_params = nullptr; // pinned staging
    dev::BatchItem* h_items = nullptr;
    dev::BatchControl* h_control = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaGraphNode_t copy_params = nullptr, copy_items = nullptr;
    cudaEvent_t done = nullptr; // staging may be rewritten once this has completed
    dev::BatchParams kparams {};
    uint64_t bytes = 0;
};

struct Chain {
    cudaStream_t stream = nullptr;
    unsigned char* queue = nullptr;
    std::vector<std::pair<cudaEvent_t, uint64_t>> pending; // (end of a queued share, its histories)
};

struct BatchEngines {
    BatchEngine e[2];
    int next = 0;
    Chain chain[MAX_CHAINS];
    cudaStream_t collector = nullptr; // records batch completion after all its chains
    uint64_t queue_capacity = 0;      // photons per chain queue buffer
    uint64_t chain_bytes = 0;
    std::vector<cudaEvent_t> spare_events;
};

namespace {

BatchEngines* engines_of(dxmc_gpu_ctx* ctx, bool create)
{
    if (!ctx->engines && create)
        ctx->engines = new (std::nothrow) BatchEngines;
    return ctx->engines;
}

void release_engine(dxmc_gpu_ctx* ctx, BatchEngine& g)
{
    if (g.stream)
        cudaStreamSynchronize(g.stream);
    if (g.exec)
        cudaGraphExecDestroy(g.exec);
    if (g.graph)
        cudaGraphDestroy(g.graph);
    cudaFree(g.d_params);
    cudaFree(g.d_items);
    cudaFree(g.d_control);
    cudaFreeHost(g.h_params);
    cudaFreeHost(g.h_items);
    cudaFreeHost(g.h_control);
    if (g.done)
        cudaEventDestroy(g.done);
    if (g.stream)
        cudaStreamDestroy(g.stream);
    ctx->in_use -= g.bytes;
    g = BatchEngine {};
}

void release_chains(dxmc_gpu_ctx* ctx, BatchEngines& en)
{
    for (auto& c : en.chain) {
        if (c.stream) {
            cudaStreamSynchronize(c.stream);
            cudaStreamDestroy(c.stream);
        }
        cudaFree(c.queue);
        for (auto& pr : c.pending)
            cudaEventDestroy(pr.first);
        c = Chain {};
    }
    if (en.collector) {
        cudaStreamSynchronize(en.collector);
        cudaStreamDestroy(en.collector);
        en.collector = nullptr;
    }
    for (auto ev : en.spare_events)
        cudaEventDestroy(ev);
    en.spare_events.clear();
    ctx->in_use -= en.chain_bytes;
    en.chain_bytes = 0;
    en.queue_capacity = 0;
}

cudaError_t build_engine(dxmc_gpu_ctx* ctx, BatchEngine& g)
{
    cudaError_t e = cudaStreamCreateWithFlags(&g.stream, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = cudaMalloc(&g.d_params, MAX_BATCH_JOBS * sizeof(dev::TransportParams));
    if (e == cudaSuccess)
        e = cudaMalloc(&g.d_items, MAX_BATCH_ITEMS * sizeof(dev::BatchItem));
    if (e == cudaSuccess)
        e = cudaMalloc(&g.d_control, sizeof(dev::BatchControl));
    if (e == cudaSuccess)
        e = cudaHostAlloc(&g.h_params, MAX_BATCH_JOBS * sizeof(dev::TransportParams), cudaHostAllocDefault);
    if (e == cudaSuccess)
        e = cudaHostAlloc(&g.h_items, MAX_BATCH_ITEMS * sizeof(dev::BatchItem), cudaHostAllocDefault);
    if (e == cudaSuccess)
        e = cudaHostAlloc(&g.h_control, sizeof(dev::BatchControl), cudaHostAllocDefault);
    if (e == cudaSuccess)
        e = cudaEventCreateWithFlags(&g.done, cudaEventDisableTiming);
    if (e == cudaSuccess)
        e = cudaGraphCreate(&g.graph, 0);
    if (e != cudaSuccess)
        return e;
    g.bytes = MAX_BATCH_JOBS * sizeof(dev::TransportParams) + MAX_BATCH_ITEMS * sizeof(dev::BatchItem) + sizeof(dev::BatchControl);
    ctx->in_use += g.bytes;
    std::memset(g.h_control, 0, sizeof(dev::BatchControl));
    // copies (sizes are updated per batch; instantiate with one job and one item)
    cudaGraphNode_t copy_control = nullptr;
    e = cudaGraphAddMemcpyNode1D(&g.copy_params, g.graph, nullptr, 0, g.d_params, g.h_params, sizeof(dev::TransportParams), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaGraphAddMemcpyNode1D(&g.copy_items, g.graph, nullptr, 0, g.d_items, g.h_items, sizeof(dev::BatchItem), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaGraphAddMemcpyNode1D(&copy_control, g.graph, nullptr, 0, g.d_control, g.h_control, sizeof(dev::BatchControl), cudaMemcpyHostToDevice);
    if (e != cudaSuccess)
        return e;
    g.kparams = dev::BatchParams { g.d_params, g.d_items, g.d_control };
    const cudaGraphNode_t deps[3] = { g.copy_params, g.copy_items, copy_control };
    for (int model = 0; model < 3 && e == cudaSuccess; ++model) {
        cudaKernelNodeParams kp {};
        kp.func = const_cast<void*>(dev::batch_kernel_function(model));
        kp.gridDim = dim3(ctx->sm_count * std::max(1, dev::batch_max_blocks_per_sm(model)));
        kp.blockDim = dim3(256);
        kp.sharedMemBytes = 0;
        void* args[1] = { &g.kparams };
        kp.kernelParams = args;
        cudaGraphNode_t node;
        e = cudaGraphAddKernelNode(&node, g.graph, deps, 3, &kp);
    }
    if (e == cudaSuccess)
        e = cudaGraphInstantiate(&g.exec, g.graph, 0);
    if (e == cudaSuccess)
        g.ready = true;
    return e;
}

// Streams and photon-queue buffers (`capacity` photons) of the first `chains` chains.
int ensure_chains(dxmc_gpu_ctx* ctx, BatchEngines& en, int chains, uint64_t capacity)
{
    if (!en.collector && cudaStreamCreateWithFlags(&en.collector, cudaStreamNonBlocking) != cudaSuccess)
        return fail(ctx, DXMC_ERR_DEVICE, "batch collector stream");
    if (capacity > en.queue_capacity) {
        // larger buffers: wait for every chain, then drop the old ones
        for (auto& c : en.chain) {
            if (c.stream)
                cudaStreamSynchronize(c.stream);
            if (c.queue) {
                cudaFree(c.queue);
                c.queue = nullptr;
                en.chain_bytes -= en.queue_capacity * 48;
                ctx->in_use -= en.queue_capacity * 48;
            }
        }
        en.queue_capacity = capacity;
    }
    for (int k = 0; k < chains; ++k) {
        Chain& c = en.chain[k];
        if (!c.stream && cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking) != cudaSuccess)
            return fail(ctx, DXMC_ERR_DEVICE, "batch chain stream");
        if (c.queue || capacity == 0)
            continue;
        const uint64_t bytes = en.queue_capacity * 48;
        if (ctx->in_use + bytes > ctx->budget)
            return fail(ctx, DXMC_ERR_OOM, "batch photon queues exceed the device memory budget");
        const cudaError_t e = cudaMalloc(&c.queue, bytes);
        if (e != cudaSuccess)
            return cuda_fail(ctx, e, "batch photon queue");
        en.chain_bytes += bytes;
        ctx->in_use += bytes;
    }
    return DXMC_OK;
}

// Histories still queued or running on a chain (its completed shares are dropped).
uint64_t chain_outstanding(BatchEngines& en, Chain& c)
{
    uint64_t left = 0;
    std::vector<std::pair<cudaEvent_t, uint64_t>> keep;
    for (auto& pr : c.pending) {
        if (cudaEventQuery(pr.first) == cudaSuccess) {
            en.spare_events.push_back(pr.first);
        } else {
            left += pr.second;
            keep.push_back(pr);
        }
    }
    c.pending.swap(keep);
    return left;
}

cudaError_t take_event(BatchEngines& en, cudaEvent_t* ev)
{
    if (!en.spare_events.empty()) {
        *ev = en.spare_events.back();
        en.spare_events.pop_back();
        return cudaSuccess;
    }
    return cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
}

} // namespace

struct dxmc_batch {
    dxmc_gpu_ctx* ctx = nullptr;
    std::vector<dxmc_job*> jobs;
    std::vector<cudaGraphExec_t> execs; // concurrent mode: one graph per chain used
    cudaEvent_t start = nullptr, stop = nullptr;
};

int dxmc_gpu_batch_submit(dxmc_gpu_ctx* ctx, const dxmc_batch_entry* entries, int n, const dxmc_batch_options* opt,
    dxmc_batch** out)
try {
    if (!ctx || !entries || n <= 0 || !out)
        return DXMC_ERR_INVALID;
    *out = nullptr;
    if (n > MAX_BATCH_JOBS)
        return fail(ctx, DXMC_ERR_INVALID, "a batch holds at most " + std::to_string(MAX_BATCH_JOBS) + " jobs");
    const int mode = opt ? opt->mode : DXMC_BATCH_AUTO;
    if (mode < DXMC_BATCH_AUTO || mode > DXMC_BATCH_PERSISTENT)
        return fail(ctx, DXMC_ERR_INVALID, "unknown batch mode");
    const bool persistent = mode == DXMC_BATCH_PERSISTENT;
    if (persistent)
        for (int i = 0; i < n; ++i)
            if (entries[i].job && entries[i].job->precision != DXMC_PRECISION_FP32)
                return fail(ctx, DXMC_ERR_INVALID, "the persistent multi-job kernel computes in FP32: run FP64 jobs in a concurrent batch");
    const int chains = std::clamp(opt && opt->chains > 0 ? opt->chains : DEFAULT_CHAINS, 1, MAX_CHAINS);
    std::lock_guard<std::mutex> lock(ctx->mutex);
    ++ctx->submission; // the grids of every entry stay until the batch has launched
    cudaSetDevice(ctx->device);
    BatchEngines* en = engines_of(ctx, true);
    if (!en)
        return DXMC_ERR_OOM;
    BatchEngine* g = nullptr;
    if (persistent) {
        g = &en->e[en->next];
        if (!g->ready) {
            const cudaError_t e = build_engine(ctx, *g);
            if (e != cudaSuccess) {
                release_engine(ctx, *g);
                return cuda_fail(ctx, e, "batch engine");
            }
        }
        // the engine's staging buffers are free once its previous batch has finished
        if (cudaEventSynchronize(g->done) != cudaSuccess)
            return fail(ctx, DXMC_ERR_DEVICE, "previous batch of the engine failed");
    } else {
        const int log2_chunk = ctx->options.queue_log2_chunk == 0 ? DEFAULT_QUEUE_LOG2 : ctx->options.queue_log2_chunk;
        const int rc = ensure_chains(ctx, *en, chains, log2_chunk >= 0 ? 1ull << std::min(log2_chunk, 34) : 0);
        if (rc != DXMC_OK)
            return rc;
    }
    auto* b = new (std::nothrow) dxmc_batch;
    if (!b)
        return DXMC_ERR_OOM;
    b->ctx = ctx;
    cudaStream_t s = ctx->stream;
    std::vector<int> models(n);
    std::vector<uint64_t> chunks(n, 0);
    std::vector<dev::TransportParams> params(persistent ? 0 : n);
    uint64_t all = 0;
    auto abort = [&](int rc) {
        cudaStreamSynchronize(s);
        for (auto* j : b->jobs) {
            ctx->in_use -= j->bytes;
            discard_job(j);
        }
        for (auto x : b->execs)
            cudaGraphExecDestroy(x);
        if (b->start)
            cudaEventDestroy(b->start);
        if (b->stop)
            cudaEventDestroy(b->stop);
        delete b;
        return rc;
    };
    for (int i = 0; i < n; ++i) {
        const dxmc_batch_entry& entry = entries[i];
        if (!entry.world || !entry.lut || !entry.job)
            return abort(fail(ctx, DXMC_ERR_INVALID, "batch entry " + std::to_string(i) + " is incomplete"));
        entry.world->usage.batched = true;
        entry.lut->usage.batched = true;
        dxmc_job* j = nullptr;
        const int rc = persistent
            ? prepare_job(ctx, entry.world, entry.lut, entry.job, QueueMode::none, 0, &j, g->h_params[i], chunks[i])
            : prepare_job(ctx, entry.world, entry.lut, entry.job, QueueMode::shared, en->queue_capacity, &j, params[i], chunks[i]);
        if (rc != DXMC_OK)
            return abort(rc);
        ctx->in_use += j->bytes; // later entries see the earlier ones in the admission check
        b->jobs.push_back(j);
        models[i] = entry.job->model;
        all += j->histories;
    }
    cudaError_t e = cudaEventCreate(&b->start);
    if (e == cudaSuccess)
        e = cudaEventCreate(&b->stop);
    // job preparation (allocations, clears, source tables) on the context stream comes first
    if (e == cudaSuccess)
        e = cudaEventRecord(b->start, s);
    if (e != cudaSuccess)
        return abort(cuda_fail(ctx, e, "batch setup"));

    const char* step = "batch launch";
    if (persistent) {
        // work items: about four per resident warp, 256 to 8192 histories each unless set
        const int per_sm = std::max(1, dev::batch_max_blocks_per_sm(1));
        const uint64_t warps = static_cast<uint64_t>(ctx->sm_count) * per_sm * 8;
        uint64_t item = opt && opt->item_histories > 0 ? static_cast<uint64_t>(opt->item_histories)
                                                       : std::clamp<uint64_t>(all / (warps * 4), 256, 8192);
        item = std::max<uint64_t>(32, (item + 31) / 32 * 32);
        auto count_items = [&](uint64_t it) {
            uint64_t c = 0;
            for (auto* j : b->jobs)
                c += (j->histories + it - 1) / it;
            return c;
        };
        while (count_items(item) > MAX_BATCH_ITEMS)
            item *= 2;
        if (item > 0xffffffffull)
            return abort(fail(ctx, DXMC_ERR_INVALID, "batch too large"));
        dev::BatchControl& c = *g->h_control;
        std::memset(&c, 0, sizeof(c));
        uint64_t n_items = 0;
        for (int model = 0; model < 3; ++model) {
            c.item_base[model] = n_items;
            for (int i = 0; i < n; ++i) {
                if (models[i] != model)
                    continue;
                const uint64_t total = b->jobs[i]->histories;
                for (uint64_t first = 0; first < total; first += item)
                    g->h_items[n_items++] = dev::BatchItem { static_cast<uint32_t>(i), static_cast<uint32_t>(std::min(item, total - first)), first };
            }
            c.n_items[model] = n_items - c.item_base[model];
        }
        const int regen = opt && opt->regen_threshold > 0 ? opt->regen_threshold
                                                          : (ctx->options.regen_threshold > 0 ? ctx->options.regen_threshold : DEFAULT_REGEN_THRESHOLD);
        const int inter = opt && opt->interact_threshold > 0 ? opt->interact_threshold
                                                             : (ctx->options.interact_threshold > 0 ? ctx->options.interact_threshold : DEFAULT_INTERACT_THRESHOLD);
        c.regen_threshold = std::clamp(regen, 1, 32);
        c.interact_threshold = std::clamp(inter, 1, 32);
        e = cudaGraphExecMemcpyNodeSetParams1D(g->exec, g->copy_params, g->d_params, g->h_params, n * sizeof(dev::TransportParams), cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaGraphExecMemcpyNodeSetParams1D(g->exec, g->copy_items, g->d_items, g->h_items, n_items * sizeof(dev::BatchItem), cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaStreamWaitEvent(g->stream, b->start, 0);
        for (auto* j : b->jobs) // every job's kernel time is the batch's
            if (e == cudaSuccess)
                e = cudaEventRecord(j->start, g->stream);
        if (e == cudaSuccess)
            e = cudaGraphLaunch(g->exec, g->stream);
        for (auto* j : b->jobs)
            if (e == cudaSuccess)
                e = cudaEventRecord(j->stop, g->stream);
        if (e == cudaSuccess)
            e = cudaEventRecord(b->stop, g->stream);
        if (e == cudaSuccess)
            e = cudaEventRecord(g->done, g->stream);
        if (e == cudaSuccess)
            en->next ^= 1;
    } else {
        // longest job first onto the chain with the least outstanding work
        std::vector<uint64_t> load(chains);
        for (int c = 0; c < chains; ++c)
            load[c] = chain_outstanding(*en, en->chain[c]);
        std::vector<int> order(n);
        for (int i = 0; i < n; ++i)
            order[i] = i;
        std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return b->jobs[x]->histories > b->jobs[y]->histories; });
        std::vector<std::vector<int>> lists(chains);
        for (int i : order) {
            const int c = static_cast<int>(std::min_element(load.begin(), load.end()) - load.begin());
            load[c] += b->jobs[i]->histories;
            lists[c].push_back(i);
        }
        std::vector<LaunchPlan> plans(n);
        for (int i = 0; i < n; ++i) // occupancy queries and attributes stay outside the capture
            plans[i] = plan_launch(ctx, entries[i].world, entries[i].lut, entries[i].job, params[i]);
        for (int c = 0; c < chains && e == cudaSuccess; ++c) {
            if (lists[c].empty())
                continue;
            std::reverse(lists[c].begin(), lists[c].end()); // shortest first within the chain
            Chain& ch = en->chain[c];
            e = cudaStreamWaitEvent(ch.stream, b->start, 0);
            uint64_t share = 0;
            // the chain's jobs go straight onto its stream: a batch's launch sequence is
            // used once, and instantiating it as a graph cost milliseconds per chain
            step = "batch launch";
            for (size_t k = 0; k < lists[c].size() && e == cudaSuccess; ++k) {
                const int i = lists[c][k];
                e = enqueue_job(b->jobs[i], params[i], models[i], chunks[i], ch.queue, plans[i], ch.stream, false);
                share += b->jobs[i]->histories;
            }
            cudaEvent_t end = nullptr;
            if (e == cudaSuccess)
                e = take_event(*en, &end);
            if (e == cudaSuccess)
                e = cudaEventRecord(end, ch.stream);
            if (e == cudaSuccess) {
                ch.pending.emplace_back(end, share);
                e = cudaStreamWaitEvent(en->collector, end, 0);
            } else if (end) {
                en->spare_events.push_back(end);
            }
        }
        if (e == cudaSuccess)
            e = cudaEventRecord(b->stop, en->collector);
    }
    if (e != cudaSuccess) {
        if (g)
            cudaStreamSynchronize(g->stream);
        for (int c = 0; c < chains; ++c)
            if (en->chain[c].stream)
                cudaStreamSynchronize(en->chain[c].stream);
        return abort(cuda_fail(ctx, e, step));
    }
    *out = b;
    return DXMC_OK;
} catch (...) {
    return exception_status(ctx);
}

int dxmc_gpu_batch_wait(dxmc_batch* b, int64_t timeout_ms)
{
    if (!b)
        return DXMC_ERR_INVALID;
    return wait_event(b->ctx, b->stop, timeout_ms, "batch wait");
}

int dxmc_gpu_batch_job(dxmc_batch* b, int index, dxmc_job** job)
{
    if (!b || !job || index < 0 || index >= static_cast<int>(b->jobs.size()))
        return DXMC_ERR_INVALID;
    *job = b->jobs[index];
    return DXMC_OK;
}

double dxmc_gpu_batch_kernel_ms(dxmc_batch* b)
{
    if (!b)
        return 0.0;
    float ms = 0;
    if (cudaEventElapsedTime(&ms, b->start, b->stop) != cudaSuccess)
        return 0.0;
    return ms;
}

void dxmc_gpu_batch_free(dxmc_batch* b)
{
    if (!b)
        return;
    cudaSetDevice(b->ctx->device);
    cudaEventSynchronize(b->stop);
    for (auto x : b->execs) // the graphs record the jobs' events: destroy them first
        cudaGraphExecDestroy(x);
    for (auto* j : b->jobs)
        dxmc_gpu_job_free(j);
    cudaEventDestroy(b->start);
    cudaEventDestroy(b->stop);
    delete b;
}

namespace {

// Waits for the batch engines' streams as well as the context stream (before
// freeing resources that a queued batch may still read).
// Waits until no queued work reads an object: its recorded last uses, or every
// stream of the context when a batch read it.  Later work on the streams is not
// waited for, so an object can be freed while the next job runs.
void wait_unused(dxmc_gpu_ctx* ctx, const Usage& u)
{
    if (u.batched) {
        sync_ctx_streams(ctx);
        return;
    }
    if (u.on_stream)
        cudaEventSynchronize(u.on_stream);
    if (u.on_results)
        cudaEventSynchronize(u.on_results);
}

void sync_ctx_streams(dxmc_gpu_ctx* ctx)
{
    cudaStreamSynchronize(ctx->stream);
    cudaStreamSynchronize(ctx->result_stream);
    cudaStreamSynchronize(ctx->upload_stream);
    if (BatchEngines* en = engines_of(ctx, false)) {
        for (auto& g : en->e)
            if (g.stream)
                cudaStreamSynchronize(g.stream);
        for (auto& c : en->chain)
            if (c.stream)
                cudaStreamSynchronize(c.stream);
    }
}

void release_engines(dxmc_gpu_ctx* ctx)
{
    if (!ctx->engines)
        return;
    for (auto& g : ctx->engines->e)
        release_engine(ctx, g);
    release_chains(ctx, *ctx->engines);
    delete ctx->engines;
    ctx->engines = nullptr;
}

} // namespace

namespace {

// Polls an event until it completes or timeout_ms (< 0: no limit) has passed.
int wait_event(dxmc_gpu_ctx* ctx, cudaEvent_t ev, int64_t timeout_ms, const char* what)
{
    cudaSetDevice(ctx->device);
    const auto t0 = std::chrono::steady_clock::now();
    while (true) {
        const cudaError_t e = cudaEventQuery(ev);
        if (e == cudaSuccess)
            return DXMC_OK;
        if (e != cudaErrorNotReady)
            return cuda_fail(ctx, e, what);
        if (timeout_ms >= 0) {
            const auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - t0).count();
            if (ms >= timeout_ms)
                return fail(ctx, DXMC_ERR_TIMEOUT, std::string(what) + " timed out");
        }
        std::this_thread::sleep_for(std::chrono::microseconds(100));
    }
}

} // namespace

int dxmc_gpu_job_wait(dxmc_job* j, int64_t timeout_ms)
{
    if (!j)
        return DXMC_ERR_INVALID;
    return wait_event(j->ctx, j->stop, timeout_ms, "job wait");
}

int dxmc_gpu_job_cancel(dxmc_job* j)
{
    if (!j)
        return DXMC_ERR_INVALID;
    *reinterpret_cast<volatile int*>(j->cancel_host) = 1;
    j->cancelled = true;
    return DXMC_OK;
}

int dxmc_gpu_job_result(dxmc_job* j, int output_mode, double calibration, double* dose, double* variance, uint32_t* n_events, dxmc_job_stats* stats)
try {
    if (!j || output_mode < 0 || output_mode > 2)
        return DXMC_ERR_INVALID;
    dxmc_gpu_ctx* ctx = j->ctx;
    const int wrc = dxmc_gpu_job_wait(j, -1);
    if (wrc != DXMC_OK)
        return wrc;
    const uint64_t nv = j->world->params.n_voxels;
    auto* hc = reinterpret_cast<dev::JobCounters*>(reinterpret_cast<unsigned char*>(j->cancel_host) + 16);
    cudaEvent_t done = nullptr;
    {
        // queue post-processing and copies on the result stream under the lock, wait without it
        std::lock_guard<std::mutex> lock(ctx->mutex);
        cudaSetDevice(ctx->device);
        cudaStream_t s = ctx->result_stream;
        if (!j->records && !j->tally_f32)
            return fail(ctx, DXMC_ERR_STATE, "job results were already released");
        DXMC_CUDA(ctx, cudaMemcpyAsync(hc, j->counters, sizeof(dev::JobCounters), cudaMemcpyDeviceToHost, s));
        // page-locked output buffers are written by the post-processing kernel through
        // their device mapping (one pass over the link, no staging buffer or copies)
        double* m_dose = nullptr;
        double* m_var = nullptr;
        uint32_t* m_events = nullptr;
        const bool mapped = !j->cancelled && (dose || variance || n_events) && (!dose || mapped_host(dose, m_dose))
            && (!variance || mapped_host(variance, m_var)) && (!n_events || mapped_host(n_events, m_events));
        if (mapped) {
            const double vv = j->world->spacing[0] * j->world->spacing[1] * j->world->spacing[2] / 1000.0;
            const cudaError_t e = j->tally_mode == 1
                ? dev::launch_postprocess_f32(j->tally_f32, j->world->params, nv, output_mode, static_cast<double>(j->histories), vv,
                      calibration, m_dose, m_var, j->n_events, m_events, s)
                : dev::launch_postprocess_records(j->records, j->world->params, nv, output_mode, static_cast<double>(j->histories), vv,
                      calibration, m_dose, m_var, m_events, s);
            if (e != cudaSuccess)
                return cuda_fail(ctx, e, "result post-processing");
        }
        // counts of record tallies are unpacked by the post-processing kernel into a staging array
        const bool unpack_counts = n_events && j->records;
        if (!mapped && !j->cancelled && (dose || variance || unpack_counts)) {
            double* d_out = nullptr;
            const uint64_t out_elems = (dose ? nv : 0) + (variance ? nv : 0) + (unpack_counts ? (nv + 1) / 2 : 0);
            DXMC_CUDA(ctx, pool_alloc(ctx, &d_out, out_elems * sizeof(double), s));
            double* d_dose = dose ? d_out : nullptr;
            double* d_var = variance ? d_out + (dose ? nv : 0) : nullptr;
            uint32_t* d_counts = unpack_counts ? reinterpret_cast<uint32_t*>(d_out + (dose ? nv : 0) + (variance ? nv : 0)) : nullptr;
            const double vv = j->world->spacing[0] * j->world->spacing[1] * j->world->spacing[2] / 1000.0;
            cudaError_t e;
            if (j->tally_mode == 1)
                e = dev::launch_postprocess_f32(j->tally_f32, j->world->params, nv, output_mode, static_cast<double>(j->histories), vv, calibration, d_dose, d_var, nullptr, nullptr, s);
            else
                e = dev::launch_postprocess_records(j->records, j->world->params, nv, output_mode, static_cast<double>(j->histories), vv, calibration, d_dose, d_var, d_counts, s);
            if (e == cudaSuccess && dose)
                e = cudaMemcpyAsync(dose, d_dose, nv * sizeof(double), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess && variance)
                e = cudaMemcpyAsync(variance, d_var, nv * sizeof(double), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess && d_counts)
                e = cudaMemcpyAsync(n_events, d_counts, nv * sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
            cudaFreeAsync(d_out, s);
            if (e != cudaSuccess)
                return cuda_fail(ctx, e, "result post-processing");
        }
        if (!mapped && !j->cancelled && n_events && j->n_events)
            DXMC_CUDA(ctx, cudaMemcpyAsync(n_events, j->n_events, nv * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        DXMC_CUDA(ctx, cudaEventCreateWithFlags(&done, cudaEventDisableTiming));
        const cudaError_t e = cudaEventRecord(done, s);
        if (e != cudaSuccess) {
            cudaEventDestroy(done);
            return cuda_fail(ctx, e, "result copy");
        }
    }
    const cudaError_t e = cudaEventSynchronize(done);
    cudaEventDestroy(done);
    std::lock_guard<std::mutex> lock(ctx->mutex);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "result copy");
    const dev::JobCounters c = *hc;
    if (stats) {
        stats->histories = c.histories_done;
        stats->steps = c.steps;
        stats->deposits = c.deposits;
        stats->rejection_overflows = c.overflows;
        float ms = 0, jms = 0;
        cudaEventElapsedTime(&ms, j->start, j->stop);
        cudaEventElapsedTime(&jms, j->begin, j->stop);
        stats->kernel_ms = ms;
        stats->job_ms = jms;
    }
    if (j->cancelled) {
        // transport.hpp:176-185: a cancelled run reports zeros
        if (dose)
            std::memset(dose, 0, nv * sizeof(double));
        if (variance)
            std::memset(variance, 0, nv * sizeof(double));
        if (n_events)
            std::memset(n_events, 0, nv * sizeof(uint32_t));
        return fail(ctx, DXMC_ERR_CANCELLED, "job was cancelled");
    }
    if (c.overflows)
        return fail(ctx, DXMC_ERR_REJECTION_CAP, "sampling loops hit the rejection cap in " + std::to_string(c.overflows) + " events");
    return DXMC_OK;
} catch (...) {
    return exception_status(j ? j->ctx : nullptr);
}

int dxmc_gpu_job_progress(dxmc_job* j, uint64_t* started, uint64_t* total)
{
    if (!j || !started)
        return DXMC_ERR_INVALID;
    dxmc_gpu_ctx* ctx = j->ctx;
    std::lock_guard<std::mutex> lock(ctx->mutex);
    if (!j->counters)
        return fail(ctx, DXMC_ERR_STATE, "job results were already released");
    cudaSetDevice(ctx->device);
    if (total)
        *total = j->histories;
    // before the job's kernel starts, its counters may not be cleared yet (a reused buffer)
    if (cudaEventQuery(j->start) != cudaSuccess) {
        *started = 0;
        return DXMC_OK;
    }
    auto* hc = reinterpret_cast<dev::JobCounters*>(reinterpret_cast<unsigned char*>(j->cancel_host) + 16);
    // a racy snapshot of a counter the kernels only increase
    DXMC_CUDA(ctx, cudaMemcpyAsync(&hc->next_history, &j->counters->next_history, 3 * sizeof(unsigned long long),
        cudaMemcpyDeviceToHost, ctx->result_stream));
    DXMC_CUDA(ctx, cudaStreamSynchronize(ctx->result_stream));
    const bool done = cudaEventQuery(j->stop) == cudaSuccess;
    *started = done ? j->histories : std::min<uint64_t>(std::max(hc->next_history, hc->histories_done), j->histories);
    if (total)
        *total = j->histories;
    return DXMC_OK;
}

int dxmc_gpu_job_preview(dxmc_job* j, double* energy)
try {
    if (!j || !energy)
        return DXMC_ERR_INVALID;
    dxmc_gpu_ctx* ctx = j->ctx;
    std::lock_guard<std::mutex> lock(ctx->mutex);
    if (!j->records)
        return fail(ctx, DXMC_ERR_STATE, j->tally_f32 ? "dose preview needs the FP64 tally" : "job results were already released");
    cudaSetDevice(ctx->device);
    const uint64_t nv = j->world->params.n_voxels;
    // before the job's kernel starts, its tally may not be cleared yet (a reused buffer)
    if (cudaEventQuery(j->start) != cudaSuccess) {
        std::fill(energy, energy + nv, 0.0);
        return DXMC_OK;
    }
    // the energy sum of each 32-byte tally record
    DXMC_CUDA(ctx, cudaMemcpy2DAsync(energy, sizeof(double), j->records, sizeof(dev::TallyRecord), sizeof(double), nv,
        cudaMemcpyDeviceToHost, ctx->result_stream));
    DXMC_CUDA(ctx, cudaStreamSynchronize(ctx->result_stream));
    return DXMC_OK;
} catch (...) {
    return exception_status(j ? j->ctx : nullptr);
}

int dxmc_gpu_job_result_async(dxmc_job* j, int output_mode, double calibration, int result_type, void* dose, void* variance,
    uint32_t* n_events)
try {
    if (!j || output_mode < 0 || output_mode > 2 || (result_type != DXMC_RESULT_F64 && result_type != DXMC_RESULT_F32))
        return DXMC_ERR_INVALID;
    dxmc_gpu_ctx* ctx = j->ctx;
    std::lock_guard<std::mutex> lock(ctx->mutex);
    cudaSetDevice(ctx->device);
    if (!j->records && !j->tally_f32)
        return fail(ctx, DXMC_ERR_STATE, "job results were already released");
    if (j->result_done)
        return fail(ctx, DXMC_ERR_STATE, "the job already has an asynchronous result pending");
    if (result_type == DXMC_RESULT_F32 && !j->records)
        return fail(ctx, DXMC_ERR_INVALID, "float results need an FP64 tally");
    const uint64_t nv = j->world->params.n_voxels;
    const size_t elem = result_type == DXMC_RESULT_F32 ? sizeof(float) : sizeof(double);
    cudaStream_t s = ctx->result_stream;
    auto* hc = reinterpret_cast<dev::JobCounters*>(reinterpret_cast<unsigned char*>(j->cancel_host) + 16);
    // everything below runs on the result stream after the job's kernel: the caller may
    // submit the next job at once, and these copies run on the copy engine beside it
    DXMC_CUDA(ctx, cudaStreamWaitEvent(s, j->stop, 0));
    DXMC_CUDA(ctx, cudaMemcpyAsync(hc, j->counters, sizeof(dev::JobCounters), cudaMemcpyDeviceToHost, s));
    const bool counts_staged = n_events && j->records;
    const size_t bytes = ((dose ? nv : 0) + (variance ? nv : 0)) * elem + (counts_staged ? nv * sizeof(uint32_t) : 0);
    unsigned char* stage = nullptr;
    if (bytes)
        DXMC_CUDA(ctx, pool_alloc(ctx, &stage, bytes, s));
    unsigned char* d_dose = dose ? stage : nullptr;
    unsigned char* d_var = variance ? stage + (dose ? nv * elem : 0) : nullptr;
    uint32_t* d_counts = counts_staged ? reinterpret_cast<uint32_t*>(stage + ((dose ? nv : 0) + (variance ? nv : 0)) * elem) : nullptr;
    const double vv = j->world->spacing[0] * j->world->spacing[1] * j->world->spacing[2] / 1000.0;
    const double hist = static_cast<double>(j->histories);
    cudaError_t e = cudaSuccess;
    if (dose || variance || counts_staged) {
        if (!j->records)
            e = dev::launch_postprocess_f32(j->tally_f32, j->world->params, nv, output_mode, hist, vv, calibration,
                reinterpret_cast<double*>(d_dose), reinterpret_cast<double*>(d_var), nullptr, nullptr, s);
        else if (result_type == DXMC_RESULT_F32)
            e = dev::launch_postprocess_records_f32(j->records, j->world->params, nv, output_mode, hist, vv, calibration,
                reinterpret_cast<float*>(d_dose), reinterpret_cast<float*>(d_var), d_counts, s);
        else
            e = dev::launch_postprocess_records(j->records, j->world->params, nv, output_mode, hist, vv, calibration,
                reinterpret_cast<double*>(d_dose), reinterpret_cast<double*>(d_var), d_counts, s);
    }
    if (e == cudaSuccess && dose)
        e = cudaMemcpyAsync(dose, d_dose, nv * elem, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && variance)
        e = cudaMemcpyAsync(variance, d_var, nv * elem, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && n_events)
        e = cudaMemcpyAsync(n_events, counts_staged ? d_counts : j->n_events, nv * sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
    if (stage)
        cudaFreeAsync(stage, s);
    if (e == cudaSuccess)
        e = cudaEventCreateWithFlags(&j->result_done, cudaEventDisableTiming);
    if (e == cudaSuccess)
        e = cudaEventRecord(j->result_done, s);
    if (e == cudaSuccess) // DOSE post-processing reads the world's densities
        e = j->world->usage.mark(j->world->usage.on_results, s);
    if (e != cudaSuccess) {
        if (j->result_done) {
            cudaEventDestroy(j->result_done);
            j->result_done = nullptr;
        }
        return cuda_fail(ctx, e, "asynchronous result");
    }
    j->result_dose = dose;
    j->result_variance = variance;
    j->result_events = n_events;
    j->result_elem = elem;
    return DXMC_OK;
} catch (...) {
    return exception_status(j ? j->ctx : nullptr);
}

int dxmc_gpu_job_result_wait(dxmc_job* j, dxmc_job_stats* stats)
try {
    if (!j)
        return DXMC_ERR_INVALID;
    dxmc_gpu_ctx* ctx = j->ctx;
    cudaEvent_t done = nullptr;
    {
        std::lock_guard<std::mutex> lock(ctx->mutex);
        done = j->result_done;
        if (!done)
            return fail(ctx, DXMC_ERR_STATE, "the job has no asynchronous result pending");
    }
    const cudaError_t e = cudaEventSynchronize(done);
    std::lock_guard<std::mutex> lock(ctx->mutex);
    cudaEventDestroy(done);
    j->result_done = nullptr;
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "asynchronous result");
    const dev::JobCounters c = *reinterpret_cast<dev::JobCounters*>(reinterpret_cast<unsigned char*>(j->cancel_host) + 16);
    const uint64_t nv = j->world->params.n_voxels;
    if (stats) {
        stats->histories = c.histories_done;
        stats->steps = c.steps;
        stats->deposits = c.deposits;
        stats->rejection_overflows = c.overflows;
        float ms = 0, jms = 0;
        cudaEventElapsedTime(&ms, j->start, j->stop);
        cudaEventElapsedTime(&jms, j->begin, j->stop);
        stats->kernel_ms = ms;
        stats->job_ms = jms;
    }
    if (j->cancelled) {
        // transport.hpp:176-185: a cancelled run reports zeros
        if (j->result_dose)
            std::memset(j->result_dose, 0, nv * j->result_elem);
        if (j->result_variance)
            std::memset(j->result_variance, 0, nv * j->result_elem);
        if (j->result_events)
            std::memset(j->result_events, 0, nv * sizeof(uint32_t));
        return fail(ctx, DXMC_ERR_CANCELLED, "job was cancelled");
    }
    if (c.overflows)
        return fail(ctx, DXMC_ERR_REJECTION_CAP, "sampling loops hit the rejection cap in " + std::to_string(c.overflows) + " events");
    return DXMC_OK;
} catch (...) {
    return exception_status(j ? j->ctx : nullptr);
}

int dxmc_gpu_job_release(dxmc_job* j)
{
    if (!j)
        return DXMC_ERR_INVALID;
    dxmc_gpu_ctx* ctx = j->ctx;
    std::lock_guard<std::mutex> lock(ctx->mutex);
    cudaSetDevice(ctx->device);
    if (j->stop)
        cudaEventSynchronize(j->stop);
    if (j->result_done)
        cudaEventSynchronize(j->result_done); // the asynchronous result still reads the tallies
    free_job_device(j, true);
    ctx->in_use -= j->bytes;
    j->bytes = 0;
    return DXMC_OK;
}

void dxmc_gpu_job_free(dxmc_job* j)
{
    if (!j)
        return;
    dxmc_gpu_ctx* ctx = j->ctx;
    std::lock_guard<std::mutex> lock(ctx->mutex);
    cudaSetDevice(ctx->device);
    if (j->stop)
        cudaEventSynchronize(j->stop); // a batched job runs on its engine's stream
    if (j->result_done) {
        cudaEventSynchronize(j->result_done);
        cudaEventDestroy(j->result_done);
        j->result_done = nullptr;
    }
    // the job's kernels and copies are done: its buffers go back to the pool in the
    // context stream's order, without waiting for later jobs
    free_job_device(j, true);
    if (j->cancel_host)
        ctx->pinned.give(j->cancel_host, j->cancel_dev);
    if (j->begin)
        cudaEventDestroy(j->begin);
    if (j->start)
        cudaEventDestroy(j->start);
    if (j->stop)
        cudaEventDestroy(j->stop);
    ctx->in_use -= j->bytes;
    delete j;
}

int dxmc_gpu_radiological_path(dxmc_gpu_ctx* ctx, dxmc_world* world, dxmc_lut* lut, const float* rays, uint64_t n_rays,
    double* out)
try {
    if (!ctx || !world || !lut || !rays || !out || n_rays == 0)
        return DXMC_ERR_INVALID;
    if (world->ctx != ctx || lut->ctx != ctx)
        return fail(ctx, DXMC_ERR_INVALID, "world or lut belongs to another context");
    if (lut->meta.n_materials < world->n_materials)
        return fail(ctx, DXMC_ERR_INVALID, "lut has fewer materials than the world");
    std::lock_guard<std::mutex> lock(ctx->mutex);
    cudaSetDevice(ctx->device);
    cudaStream_t s = ctx->stream;
    float* d_rays = nullptr;
    double* d_out = nullptr;
    cudaError_t e = pool_alloc(ctx, &d_rays, n_rays * 7 * sizeof(float), s);
    if (e == cudaSuccess)
        e = pool_alloc(ctx, &d_out, n_rays * sizeof(double), s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_rays, rays, n_rays * 7 * sizeof(float), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = dev::launch_radiological_path(world->params, lut->image, lut->meta, d_rays, n_rays, d_out, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out, d_out, n_rays * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (d_rays)
        cudaFreeAsync(d_rays, s);
    if (d_out)
        cudaFreeAsync(d_out, s);
    const cudaError_t se = cudaStreamSynchronize(s);
    if (e == cudaSuccess)
        e = se;
    return e == cudaSuccess ? DXMC_OK : cuda_fail(ctx, e, "radiological path");
} catch (...) {
    return exception_status(ctx);
}

int dxmc_gpu_probe_lut(dxmc_gpu_ctx* ctx, dxmc_lut* lut, int material, const double* energies, int n, double* out_att, double* out_maxinv)
try {
    if (!ctx || !lut || !energies || n <= 0 || !out_att || !out_maxinv || material < 0 || material >= lut->meta.n_materials)
        return DXMC_ERR_INVALID;
    std::lock_guard<std::mutex> lock(ctx->mutex);
    cudaSetDevice(ctx->device);
    cudaStream_t s = ctx->stream;
    double* buf = nullptr;
    DXMC_CUDA(ctx, pool_alloc(ctx, &buf, static_cast<size_t>(n) * 5 * sizeof(double), s));
    DXMC_CUDA(ctx, cudaMemcpyAsync(buf, energies, n * sizeof(double), cudaMemcpyHostToDevice, s));
    DXMC_CUDA(ctx, dev::launch_probe_lut(lut->image, lut->meta, material, buf, n, buf + n, buf + 4 * static_cast<size_t>(n), s));
    DXMC_CUDA(ctx, cudaMemcpyAsync(out_att, buf + n, 3 * static_cast<size_t>(n) * sizeof(double), cudaMemcpyDeviceToHost, s));
    DXMC_CUDA(ctx, cudaMemcpyAsync(out_maxinv, buf + 4 * static_cast<size_t>(n), n * sizeof(double), cudaMemcpyDeviceToHost, s));
    cudaFreeAsync(buf, s);
    DXMC_CUDA(ctx, cudaStreamSynchronize(s));
    return DXMC_OK;
} catch (...) {
    return exception_status(ctx);
}

int dxmc_gpu_probe_interactions(dxmc_gpu_ctx* ctx, dxmc_lut* lut, int material, int model, int kind, double energy, uint64_t n, uint64_t seed,
    float* out_cos, float* out_energy, float* out_dep)
try {
    if (!ctx || !lut || n == 0 || !out_cos || !out_energy || !out_dep || material < 0 || material >= lut->meta.n_materials || model < 0 || model > 2 || kind < 0 || kind > 2 || !(energy > 0))
        return DXMC_ERR_INVALID;
    std::lock_guard<std::mutex> lock(ctx->mutex);
    cudaSetDevice(ctx->device);
    cudaStream_t s = ctx->stream;
    float* buf = nullptr;
    DXMC_CUDA(ctx, pool_alloc(ctx, &buf, n * 3 * sizeof(float), s));
    DXMC_CUDA(ctx, dev::launch_probe_interactions(lut->image, lut->meta, material, model, kind, static_cast<float>(energy), n, seed, buf, buf + n, buf + 2 * n, s));
    DXMC_CUDA(ctx, cudaMemcpyAsync(out_cos, buf, n * sizeof(float), cudaMemcpyDeviceToHost, s));
    DXMC_CUDA(ctx, cudaMemcpyAsync(out_energy, buf + n, n * sizeof(float), cudaMemcpyDeviceToHost, s));
    DXMC_CUDA(ctx, cudaMemcpyAsync(out_dep, buf + 2 * n, n * sizeof(float), cudaMemcpyDeviceToHost, s));
    cudaFreeAsync(buf, s);
    DXMC_CUDA(ctx, cudaStreamSynchronize(s));
    return DXMC_OK;
} catch (...) {
    return exception_status(ctx);
}

int dxmc_gpu_probe_uniform(dxmc_gpu_ctx* ctx, uint64_t seed, uint64_t n_streams, uint32_t draws_per_stream, int kind,
    int32_t n_bins, uint64_t* hist)
try {
    if (!ctx || !hist || n_streams == 0 || draws_per_stream == 0 || kind < 0 || kind > 2 || n_bins < 1 || n_bins > 4096)
        return DXMC_ERR_INVALID;
    std::lock_guard<std::mutex> lock(ctx->mutex);
    cudaSetDevice(ctx->device);
    cudaStream_t s = ctx->stream;
    unsigned long long* buf = nullptr;
    const size_t bytes = (static_cast<size_t>(n_bins) + 1) * sizeof(unsigned long long);
    DXMC_CUDA(ctx, pool_alloc(ctx, &buf, bytes, s));
    DXMC_CUDA(ctx, cudaMemsetAsync(buf, 0, bytes, s));
    DXMC_CUDA(ctx, dev::launch_probe_uniform(seed, n_streams, draws_per_stream, kind, n_bins, buf, ctx->sm_count, s));
    DXMC_CUDA(ctx, cudaMemcpyAsync(hist, buf, bytes, cudaMemcpyDeviceToHost, s));
    cudaFreeAsync(buf, s);
    DXMC_CUDA(ctx, cudaStreamSynchronize(s));
    return DXMC_OK;
} catch (...) {
    return exception_status(ctx);
}

} // extern "C"

// Read-only accessors used by the no-allocation entry point (noalloc.cu).
namespace dxmc_gb300::capi {
int ctx_device(const dxmc_gpu_ctx* ctx) { return ctx->device; }
cudaStream_t ctx_stream(const dxmc_gpu_ctx* ctx) { return ctx->stream; }
int ctx_sm_count(const dxmc_gpu_ctx* ctx) { return ctx->sm_count; }
size_t ctx_max_smem(const dxmc_gpu_ctx* ctx) { return ctx->max_smem_optin; }
void ctx_set_error(dxmc_gpu_ctx* ctx, const std::string& msg) { ctx->last_error = msg; }
int exception_status(dxmc_gpu_ctx* ctx) noexcept { return ::exception_status(ctx); }
std::mutex& ctx_mutex(dxmc_gpu_ctx* ctx) { return ctx->mutex; }
int ctx_regen_threshold(const dxmc_gpu_ctx* ctx, bool local)
{
    return ctx->options.regen_threshold > 0 ? std::min(ctx->options.regen_threshold, 32)
                                            : (local ? DEFAULT_LOCAL_REGEN_THRESHOLD : DEFAULT_REGEN_THRESHOLD);
}
int default_woodcock_burst(bool local) { return local ? DEFAULT_LOCAL_WOODCOCK_BURST : DEFAULT_WOODCOCK_BURST; }

int ctx_interact_threshold(const dxmc_gpu_ctx* ctx)
{
    return ctx->options.interact_threshold > 0 ? std::min(ctx->options.interact_threshold, 32) : DEFAULT_INTERACT_THRESHOLD;
}
const dev::WorldParams* world_params(const dxmc_world* w, const dxmc_gpu_ctx** owner, int* n_materials)
{
    *owner = w->ctx;
    *n_materials = w->n_materials;
    return &w->params;
}
const float* lut_image(const dxmc_lut* l, dev::LutMeta* meta, const dxmc_gpu_ctx** owner)
{
    *owner = l->ctx;
    *meta = l->meta;
    return l->image;
}
// The local-majorant grid of (world, lut) if the job tracks with local majorants
// and the grid was built before (no allocation here); else nullptr.
const dev::MajorantGrid* built_majorant(dxmc_gpu_ctx* ctx, dxmc_world* w, const dxmc_lut* l, const dxmc_job_desc* jd)
{
    const dev::MajorantGrid* g = nullptr;
    if (job_tracking(ctx, jd) == DXMC_TRACKING_LOCAL)
        world_majorant(ctx, w, l, false, &g);
    return g;
}
} // namespace dxmc_gb300::capi
