// Parameters of the photon-transport kernels and the host-side launchers.
#pragma once

#include "device_common.cuh"

namespace dxmc_gb300::dev {

// Palette entry of the compact voxel layout: density and (material | measurement << 8).
struct PaletteEntry {
    float density;
    uint32_t code;
};

constexpr int PALETTE_MAX = 256;

struct WorldParams {
    const Voxel* voxels;            // 8-byte layout, or nullptr when the compact layout is used
    const uint8_t* palette_index;   // 1-byte layout, or nullptr when the world has > 256 distinct voxels
    const PaletteEntry* palette;    // PALETTE_MAX entries
    int palette_n;
    int pad_palette;
    uint32_t dims[3];
    uint32_t pad;
    float lo[3];          // nextafter-safe lower extent (world.hpp:55-68)
    float hi[3];          // nextafter-safe upper extent
    float inv_spacing[3]; // 1 / spacing (mm)
    float lo_inv[3];      // lo * inv_spacing (voxel index as one FMA)
    float dims_f[3];      // dims as floats (grid coordinates are inside in [0, dims))
    float spacing[3];     // voxel size (mm)
    float lower[3];       // lower grid corner (mm), the plane of voxel boundary 0
    uint64_t nxy;
    uint64_t n_voxels;
};

// Local majorants for Woodcock tracking: the voxel grid is cut into cells of
// 2^shift voxels per axis and the photon energies into bands; cell c holds for
// band b the pair cells[c * bands + b] = (1 / s, R): every voxel within the
// distance R (mm) of any point of the cell attenuates less than s times the
// global majorant at every energy of the band.  A flight drawn with the
// majorant s * M(E) stops after R without a collision test and is drawn again
// from there (the exponential distribution has no memory), so the tracking
// stays exact while it takes far fewer steps through air, lung and soft tissue.
// cells == nullptr selects the global majorant of the reference (s = 1, R
// infinite).
// Cells outside the box of all cells above the emptiest level (the body of a CT
// phantom) hold -R: a photon there may also fly straight to that box, since only
// cells of the emptiest level lie before it on its ray.
constexpr int MAJORANT_MAX_BANDS = 8;
struct MajorantGrid {
    const float2* cells;
    const float* box;    // lo[3], hi[3] in mm (grid frame) of the cells above the emptiest level
    uint32_t nx, nxy;    // cells along x, cells per z slab
    int shift[3];        // log2 of the cell size in voxels
    int bands;
    float band_edge[MAJORANT_MAX_BANDS - 1]; // keV, ascending; band = number of edges <= E (unused: infinity)
    // the edges are log-spaced: band = clamp(floor((log10 E - band_log0) * band_inv_dlog), 0, bands - 1)
    float band_log0;
    float band_inv_dlog;
};

struct SourceParams {
    const DevExposure* exposures;
    const uint64_t* history_offsets; // n_exposures + 1 prefix sums
    uint32_t n_exposures;
    int spec_n;                      // 0: monoenergetic
    const float* spec_energy;
    const float* spec_prob;
    const uint32_t* spec_alias;
    const float* heel_weights;       // nullptr: no heel
    float heel_e_start, heel_e_step;
    int heel_e_size, heel_a_size;
    float heel_a_start, heel_a_step;
    const float* bowtie_angle;       // nullptr: no bow-tie
    const float* bowtie_weight;
    int bowtie_n;
    int pad;
};

// Counters shared by all blocks of one job (device scratch).
struct JobCounters {
    unsigned long long next_history;   // work queue head (in-kernel photon generation)
    unsigned long long histories_done;
    unsigned long long steps;          // Woodcock steps inside the grid
    unsigned long long deposits;       // depositing events
    unsigned long long overflows;      // rejection-cap hits
    unsigned long long queue_count;    // photons in the pre-generated queue
    unsigned long long next_photon;    // pre-generated queue head
    unsigned long long pad;
};

// Pre-generated photons (structure of arrays): position + energy, direction +
// weight, and the history's random-stream state after generation.
struct PhotonQueue {
    float4* pos_energy;
    float4* dir_weight;
    uint4* rng;
    uint64_t capacity;
};

// FP64 tally of one voxel in one 32-byte sector (the unit of L2 and DRAM
// transfers): a deposit's three atomic additions touch a single sector.
struct alignas(32) TallyRecord {
    double energy;   // sum of energy imparted x weight (keV)
    double energy2;  // sum of its squares
    uint32_t events; // deposits
    uint32_t pad0;
    uint64_t pad1;
};
static_assert(sizeof(TallyRecord) == 32, "one tally record per 32-byte sector");

struct TransportParams {
    WorldParams world;
    SourceParams source;
    const float* lut;   // global LUT image
    LutMeta lut_meta;
    TallyRecord* records; // FP64 tallies as one record per voxel (jobs); nullptr: the arrays below
    double* tally;      // interleaved (energy, energy^2) per voxel, FP64 (with n_events; the no-allocation path)
    float* tally_f32;   // interleaved, FP32 tally mode
    uint32_t* n_events;
    JobCounters* counters;
    const volatile int* cancel; // host-mapped flag, may be null
    PhotonQueue queue;          // pos_energy == nullptr: photons are generated inside the transport kernel
    uint64_t total_histories;
    uint64_t seed;
    uint64_t uniform_hpe;   // histories per exposure when every exposure has the same count, else 0
    uint32_t hpe_magic;     // history / uniform_hpe as a multiply-high (udiv_magic), jobs below 2^32 histories
    uint32_t hpe_shifts;
    int tally_mode;
    int lut_in_smem;
    int regen_threshold;    // refill finished lanes once at least this many are idle (1..32)
    int interact_threshold; // run the interaction passes once at least this many lanes wait (1..32)
    int woodcock_burst;     // Woodcock steps a lane may take per loop iteration (1..64)
    int normalize_direction; // 1: unit scattering axis in peturb (normalised physics), 0: the reference's
    int precision;          // 0: FP32 transport; 1: FP64 everywhere (position, direction, energy, LUT, sampling)
    int pad_precision;
    MajorantGrid majorant;
};

// Work item of the batched kernel: histories [first, first + count) of job `job`.
struct BatchItem {
    uint32_t job;
    uint32_t count;
    uint64_t first;
};

// Per-batch control block in device memory, written by one host-to-device copy
// before the batch kernels start: the kernels' own arguments never change, so
// one instantiated CUDA graph serves every batch of an engine.
struct BatchControl {
    unsigned long long next_item[4]; // work-queue heads, one per correction model (start at zero)
    uint64_t item_base[4];           // first item of each model in the item array
    uint64_t n_items[4];             // items of each model
    int regen_threshold;
    int interact_threshold;
    int pad[2];
};

struct BatchParams {
    const TransportParams* jobs;
    const BatchItem* items;
    BatchControl* control;
};

// Launchers (defined in transport_kernels.cu).
// Entry function of the batched kernel for a correction model (for graph kernel nodes).
const void* batch_kernel_function(int model);
int batch_max_blocks_per_sm(int model);
// Samples histories [first, first + count) into p.queue (compacted: photons that
// miss the world are counted but not queued).
cudaError_t launch_generate(const TransportParams& p, uint64_t first, uint64_t count, int grid, cudaStream_t stream);
cudaError_t launch_transport(const TransportParams& p, int model, int grid, int block, size_t smem, cudaStream_t stream);
// Loads the modules of every single-job transport kernel on the current device
// (CUDA loads modules lazily, on first use, and a load allocates device memory).
cudaError_t preload_transport_kernels();
// blocks per SM for this configuration; also raises the kernel's dynamic shared-memory limit
int transport_max_blocks_per_sm(int model, bool palette, int block, size_t smem, int precision = 0);
// dynamic shared memory the transport kernel needs for a LUT image of lut_bytes
size_t transport_smem_bytes(size_t lut_bytes, bool lut_in_smem, bool palette);
// Post-processing of the tallies into dose / variance (densities from the world's layout).
// dose, variance and counts_out may be device memory or page-locked host memory
// (written through its device mapping); counts_out, if not null, gets a copy of counts.
cudaError_t launch_postprocess(const double* tally, const WorldParams& w, uint64_t n,
    int mode, double histories, double voxel_volume_cm3, double calibration, double* dose, double* variance,
    const uint32_t* counts, uint32_t* counts_out, cudaStream_t stream);
cudaError_t launch_postprocess_records(const TallyRecord* records, const WorldParams& w, uint64_t n,
    int mode, double histories, double voxel_volume_cm3, double calibration, double* dose, double* variance,
    uint32_t* counts_out, cudaStream_t stream);
// The same with float results (Result<float>: 12 bytes per voxel with the counts).
cudaError_t launch_postprocess_records_f32(const TallyRecord* records, const WorldParams& w, uint64_t n,
    int mode, double histories, double voxel_volume_cm3, double calibration, float* dose, float* variance,
    uint32_t* counts_out, cudaStream_t stream);
cudaError_t launch_postprocess_f32(const float* tally, const WorldParams& w, uint64_t n,
    int mode, double histories, double voxel_volume_cm3, double calibration, double* dose, double* variance,
    const uint32_t* counts, uint32_t* counts_out, cudaStream_t stream);
// Radiological path of n rays (Siddon traversal): rays are 7 floats each
// (origin mm, direction, energy keV); out[i] = sum of mu * density * length (cm).
cudaError_t launch_radiological_path(const WorldParams& w, const float* lut, LutMeta meta, const float* rays, uint64_t n,
    double* out, cudaStream_t stream);
// Local-majorant grid construction (majorant_kernels.cu).  The scale tables hold
// the scale of each palette entry (compact layout) or the ratio r_m of each
// material (8-byte layout: scale = density * r_m, 1 for measurement voxels).
struct MajorantBuild {
    uint32_t n[3];       // cells per axis
    int shift[3];
    float edge[3];       // cell size (mm)
    int levels_per_octave;
    int max_level;
    int bands;           // output pairs at cells[c * bands + band]
    int floor_levels[MAJORANT_MAX_BANDS]; // each band's emptiest level (its cells may be flown through), -1: none
    float mu_refs[MAJORANT_MAX_BANDS];    // global majorant (1/mm) at each band's reference energy (cost model)
    float lower[3];      // grid corner (mm)
};
// Candidate levels whose distance transforms run together: pairs[first[k],
// first[k + 1]) are band k's levels, in ascending order.
constexpr int MAJORANT_MAX_PAIRS = MAJORANT_MAX_BANDS * 16;
struct MajorantPairs {
    int count;
    int first[MAJORANT_MAX_BANDS + 1];
    uint8_t band[MAJORANT_MAX_PAIRS];
    uint8_t level[MAJORANT_MAX_PAIRS];
};
// All bands in one pass: scales is bands x PALETTE_MAX floats in device memory;
// level and cost are bands x ncell; hist (bands x 64, zeroed by the caller)
// counts the cells of each level.
cudaError_t launch_majorant_levels(const WorldParams& w, const float* scales, const MajorantBuild& b,
    uint8_t* level, float2* cells, float* cost, int* bounds, unsigned int* hist, cudaStream_t stream);
// After all bands: writes the box (mm) of the cells that lay above their band's
// emptiest level (bounds: cell index min x, y, z, max x, y, z; set up as empty
// by the caller) and marks every cell outside it by negating its R in all bands.
cudaError_t launch_majorant_box(const MajorantBuild& b, const int* bounds, float2* cells, float* box, cudaStream_t stream);
// minlev (bands x ncell): each cell's lowest level over its 27-neighbourhood.
cudaError_t launch_majorant_minfilter(const MajorantBuild& b, const uint8_t* level, uint8_t* minlev, cudaStream_t stream);
// Adds a group of candidate (band, level) pairs: for each, cells whose
// 27-neighbourhood holds no cell above the level (minlev >= level) get (level
// scale, distance to the nearest such cell) if that lowers the band's expected
// number of steps per mm, a band's levels tried in ascending order.  d0 and d1
// are scratch grids of pairs.count x ncell floats.
cudaError_t launch_majorant_level_passes(const MajorantBuild& b, const MajorantPairs& pairs, const uint8_t* minlev,
    float* d0, float* d1, float2* cells, float* cost, cudaStream_t stream);
cudaError_t launch_max_density(const Voxel* voxels, uint64_t n, unsigned int* out_bits, int n_materials, cudaStream_t stream);
cudaError_t launch_probe_lut(const float* lut, LutMeta meta, int material, const double* energies, int n, double* out_att, double* out_maxinv, cudaStream_t stream);
// Histogram of the per-history random streams' output (see dxmc_gpu_probe_uniform).
cudaError_t launch_probe_uniform(uint64_t seed, uint64_t n_streams, uint32_t draws, int kind, int nbins,
    unsigned long long* hist, int sm_count, cudaStream_t stream);
cudaError_t launch_probe_interactions(const float* lut, LutMeta meta, int material, int model, int kind, float energy,
    uint64_t n, uint64_t seed, float* out_cos, float* out_energy, float* out_dep, cudaStream_t stream);

} // namespace dxmc_gb300::dev
