/*
 * dxmc_gpu.h — C ABI of the GB300 (sm_103a) photon-transport engine.
 *
 * This is the drop-in boundary for DXMClib's photon-transport hot path.  In
 * DXMClib the path sits behind C++ templates (include/dxmc/transport.hpp:
 * Transport<T>::operator()(world, source, progress, useSourceDoseCalibration),
 * lines 135-202).  Everything on the GPU side of that call is reached through
 * the plain-C entry points below: opaque handles, plain pointers and sizes,
 * an int status on every call, no exceptions and no torch types.  The C++
 * adapter include/dxmc_gpu/transport.hpp maps DXMClib's World / Source /
 * Material objects onto these calls; ctypes / cgo / JNI bindings can use them
 * directly.
 *
 * Units follow DXMClib: lengths in mm, energies in keV, densities in g/cm3,
 * mass attenuation in cm2/g, momentum transfer in 1/angstrom.
 */
#ifndef DXMC_GPU_H
#define DXMC_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DXMC_GPU_ABI_VERSION 3

/* ---- status codes ------------------------------------------------------- */
enum {
    DXMC_OK = 0,
    DXMC_ERR_INVALID = -1,      /* invalid argument / invalid world or source */
    DXMC_ERR_OOM = -2,          /* allocation failed or admission budget exceeded */
    DXMC_ERR_DEVICE = -3,       /* CUDA runtime error */
    DXMC_ERR_REJECTION_CAP = -4,/* a sampling loop hit its iteration cap (histories ended early) */
    DXMC_ERR_TIMEOUT = -5,      /* dxmc_gpu_job_wait timed out */
    DXMC_ERR_CANCELLED = -6,    /* job was cancelled; results are zero */
    DXMC_ERR_NO_DEVICE = -7,    /* no CUDA device / extension not usable */
    DXMC_ERR_STATE = -8         /* call not valid in the object's current state */
};

/* Low-energy correction models: include/dxmc/lowenergycorrectionmodel.hpp:22-26 */
enum { DXMC_MODEL_NONE = 0, DXMC_MODEL_LIVERMORE = 1, DXMC_MODEL_IA = 2 };

/* Output modes: Transport<T>::OUTPUTMODE (transport.hpp:117-120) plus the raw tally. */
enum {
    DXMC_OUTPUT_RAW = 0,            /* sum of energy imparted (keV) and sum of its squares */
    DXMC_OUTPUT_EV_PER_HISTORY = 1, /* normalizeScoring, transport.hpp:780-794 */
    DXMC_OUTPUT_DOSE = 2            /* energyImpartedToDose, transport.hpp:796-816 */
};

/* Tally precision modes for the per-voxel accumulators. */
enum {
    DXMC_TALLY_F64 = 0,         /* FP64 atomics for every deposit (reference semantics) */
    DXMC_TALLY_F32 = 1,         /* FP32 atomics only (precision study) */
    DXMC_TALLY_WARP_F64 = 2     /* FP32 warp-aggregated partials flushed to FP64 */
};

/* Woodcock tracking majorant.  GLOBAL is the reference's delta tracking
 * (woodcockParticleTracking, transport.hpp:640-700): every flight is drawn with
 * the largest attenuation in the world.  LOCAL draws each flight with a bound of
 * the photon's neighbourhood from a grid built per (world, LUT) pair, and ends a
 * flight without a collision test where that bound stops holding; both sample
 * the same transport process, LOCAL with fewer virtual collisions. */
enum {
    DXMC_TRACKING_DEFAULT = 0,  /* the context's choice (LOCAL unless set) */
    DXMC_TRACKING_GLOBAL = 1,
    DXMC_TRACKING_LOCAL = 2
};

/* Direction changes.  REFERENCE keeps vectormath::peturb's unnormalised
 * orthogonal axis (vectormath.hpp:197-221): |dir| shrinks after each scatter and
 * the turn is not exactly the sampled angle, as in the reference.  NORMALIZED
 * scales the axis to unit length (directions stay unit vectors and turn by the
 * sampled angle); its results do not match the reference's. */
enum { DXMC_DIRECTION_REFERENCE = 0, DXMC_DIRECTION_NORMALIZED = 1 };

/* ---- physics data for the host LUT build -------------------------------- */
/* One electron shell, mirrors dxmc::ElectronShellConfiguration (material.hpp:29-58). */
typedef struct dxmc_shell_config {
    double binding_energy;
    double number_electrons;
    double hartree_fock_j0;
    double photo_ionization_probability;
    double fluorescence_yield;
    double line_probabilities[3];
    double line_energies[3];
    int32_t Z;
    int32_t shell;
} dxmc_shell_config;

/* Host callbacks answering the dxmc::Material queries that the LUT build makes
 * (material.hpp:60-101; attenuationlut.hpp:212-265; attenuationinterpolator.hpp:
 * 119-205).  A DXMClib user wraps their xraylib-backed Material; the project
 * physics model provides one through dxmc_physics_material(). */
typedef struct dxmc_material_provider {
    void* user;
    double standard_density;
    double (*photoelectric)(void* user, double energy_kev);
    double (*compton)(void* user, double energy_kev);
    double (*rayleigh)(void* user, double energy_kev);
    double (*form_factor_squared)(void* user, double momentum_transfer);
    double (*scatter_factor)(void* user, double momentum_transfer);
    /* binding energies above min_energy, descending; returns the count (may exceed capacity) */
    int (*binding_energies)(void* user, double min_energy, double* out, int capacity);
    void (*shells)(void* user, dxmc_shell_config out[12]);
} dxmc_material_provider;

/* Project physics model (closed-form; replaces xraylib).  name is a named
 * material ("Water, Liquid", ...), a chemical formula ("H2O") or an element
 * symbol; density <= 0 keeps the standard density.  The provider stays valid
 * until dxmc_physics_material_free. */
int dxmc_physics_material(const char* name, double density, dxmc_material_provider* out);
void dxmc_physics_material_free(dxmc_material_provider* provider);
/* Mass energy-absorption coefficient (cm2/g) of a material made by
 * dxmc_physics_material: Material::getMassEnergyAbsorbtion (material.cpp:56-59),
 * which the DX dose-area-product calibration weighs the spectrum with
 * (source.hpp:552-568). */
int dxmc_physics_mass_energy_absorption(const dxmc_material_provider* provider, double energy_kev, double* out);
int dxmc_physics_element_material(int atomic_number, dxmc_material_provider* out);

/* ---- tube spectra (host; Tube<T>::getSpecter, tube.hpp:191-261) ----------- */
/* Photon fluence per energy of an x-ray tube at voltage_kv with a tungsten
 * anode: thick-target semi-relativistic Bethe-Heitler bremsstrahlung from the
 * tabulated electron fluence of Poludniowski and Evans (2007), photons leaving
 * the anode at takeoff_angle (radians), the tungsten K lines computed at
 * line_takeoff_angle (the tube's own anode angle: DXMClib evaluates the lines
 * there even for the heel table's other angles, tube.hpp:220-241), then
 * attenuated by n_filters materials of filter_mm thickness each at their
 * standard density, and with normalize scaled to sum to one.  energies are in
 * keV, ascending (Tube::getEnergy: the resolution, twice it, ... up to the
 * voltage).  Replaces betheHeitlerCrossSection.hpp:326-407 and tube.hpp:191-261. */
int dxmc_tube_spectrum(double voltage_kv, double takeoff_angle, double line_takeoff_angle, const double* energies,
    int n_energies, const dxmc_material_provider* filters, const double* filter_mm, int n_filters, int normalize,
    double* out);

/* ---- bow-tie table (host; BowTieFilter<T>, beamfilters.hpp:65-197) ------- */
/* The table a job samples bow-tie weights from: the n (|angle|, weight) pairs
 * sorted by angle, weights divided by their mean (the BowTieFilter
 * constructors and normalizeData, beamfilters.hpp:88-130).  angles in radians.
 * DXMC_ERR_INVALID for n <= 0, n > DXMC_MAX_BOWTIE_POINTS or a mean weight that
 * is not positive. */
int dxmc_bowtie_table(const double* angles, const double* weights, int n, double* table_angles,
    double* table_weights);

/* ---- host LUT (AttenuationLut<T>::generate, attenuationlut.hpp:64-96) ---- */
typedef struct dxmc_lut_blob dxmc_lut_blob;

/* Builds the attenuation / form-factor / scatter-factor / shell tables for
 * materials [0, n_materials) of a world.  The majorant uses the maximum
 * density of each material over the voxels (attenuationinterpolator.hpp:48-84).
 * max_energy is the source's maximum photon energy (transport.hpp:155-157). */
int dxmc_lut_build(const dxmc_material_provider* materials, int n_materials,
    const float* density, const uint8_t* material, uint64_t n_voxels,
    double max_energy, dxmc_lut_blob** out);
/* Same, with the per-material maximum density supplied by the caller
 * (for example from dxmc_gpu_world_max_density). */
int dxmc_lut_build_max_density(const dxmc_material_provider* materials, int n_materials,
    const double* max_density, double max_energy, dxmc_lut_blob** out);
void dxmc_lut_blob_free(dxmc_lut_blob* blob);
/* Host evaluation of the tables (AttenuationLut public lookups, attenuationlut.hpp:105-153). */
int dxmc_lut_attenuation(const dxmc_lut_blob* blob, int material, double energy, double out_photo_compt_rayl[3]);
double dxmc_lut_max_attenuation_inverse(const dxmc_lut_blob* blob, double energy);
double dxmc_lut_scatter_factor(const dxmc_lut_blob* blob, int material, double momentum_transfer);
/* Introspection for tests: table sizes and raw arrays (double precision). */
typedef struct dxmc_lut_info {
    int32_t n_materials;
    int32_t n_energy;          /* number of energy nodes / segments */
    int32_t linear_index;
    int32_t pad;
    double linear_step;
    double linear_energy;
    double min_energy;
    double max_energy;
    const double* log_energy;  /* n_energy */
    const double* coefficients;/* n_materials * n_energy * 6 : (b, a) for photo, compton, rayleigh */
    const double* max_coefficients; /* n_energy * 2 */
    const double* rita;        /* n_materials * 4 * 56 : x, e, a, b */
    const double* spline;      /* n_materials * 79 : 60 coefficients, 16 knots, start, step, stop */
    const dxmc_shell_config* shells; /* n_materials * 12 */
} dxmc_lut_info;
int dxmc_lut_get_info(const dxmc_lut_blob* blob, dxmc_lut_info* info);

/* ---- sources: per-exposure table (Source::getExposure + alignToDirectionCosines) ---- */
typedef struct dxmc_exposure {
    double position[3];          /* mm, world basis */
    double direction_cosines[6]; /* x then y direction cosine, world basis */
    double beam_direction[3];
    double collimation[4];       /* x0, x1, y0, y1 in radians (exposure.hpp:40) */
    double weight;               /* beam intensity weight */
    uint64_t n_histories;
    double mono_energy;          /* keV, used when the job has no spectrum */
} dxmc_exposure;

/* Spectrum: SpecterDistribution (dxmcrandom.hpp:284-330). The alias table is built
 * on the host from the weights (squaring-the-histogram, dxmcrandom.hpp:229-274). */
typedef struct dxmc_spectrum_desc {
    int32_t n;
    const double* energies;  /* keV, increasing */
    const double* weights;
} dxmc_spectrum_desc;

/* Heel table: HeelFilter (beamfilters.hpp:435-569).  At most
 * DXMC_MAX_HEEL_WEIGHTS weights (energy_size * angle_size, counted in 64 bits);
 * a larger table is rejected with DXMC_ERR_INVALID. */
#define DXMC_MAX_HEEL_WEIGHTS (1 << 24)
typedef struct dxmc_heel_desc {
    double energy_start, energy_step;
    int32_t energy_size;
    int32_t angle_size;
    double angle_start, angle_step;
    const double* weights; /* energy_size * angle_size, angle fastest */
} dxmc_heel_desc;

/* Bow-tie: BowTieFilter (beamfilters.hpp:78-198): angle/weight pairs; the
 * library takes |angle|, sorts and normalises the weights to mean 1.  At most
 * DXMC_MAX_BOWTIE_POINTS pairs; a larger table, or one whose mean weight is not
 * positive, is rejected with DXMC_ERR_INVALID. */
#define DXMC_MAX_BOWTIE_POINTS (1 << 20)
typedef struct dxmc_bowtie_desc {
    int32_t n;
    const double* angles;
    const double* weights;
} dxmc_bowtie_desc;

/* The xoshiro128+ state of the random stream of history `history` of a job
 * seeded with `seed` (SplitMix64 of (seed, history)), as the kernels seed it;
 * exposed for known-answer tests.  Replaces RandomState's seeding from
 * std::random_device (dxmcrandom.hpp:42-48), which is not reproducible. */
int dxmc_stream_seed(uint64_t seed, uint64_t history, uint32_t out[4]);
/* The kernels' division of history ids by the histories per exposure (multiply-high
 * and shifts, magic from the divisor), for host-side checks: out[i] = n[i] / d. */
int dxmc_udiv_invariant(const uint32_t* n, uint64_t count, uint32_t d, uint32_t* out);

/* Alias table of a spectrum (host), exposed for parity tests. */
int dxmc_alias_table(const double* weights, int n, double* probs, uint64_t* alias);

/* ---- device context ------------------------------------------------------ */
typedef struct dxmc_gpu_ctx dxmc_gpu_ctx;
typedef struct dxmc_world dxmc_world;
typedef struct dxmc_lut dxmc_lut;
typedef struct dxmc_job dxmc_job;

typedef struct dxmc_gpu_options {
    int32_t device;          /* CUDA device ordinal */
    int32_t block_size;      /* threads per block, 0 = default (256) */
    int32_t blocks_per_sm;   /* resident blocks per SM, 0 = occupancy-derived */
    int32_t tally_mode;      /* DXMC_TALLY_* */
    uint64_t memory_budget;  /* admission budget in bytes, 0 = 90% of free memory */
    int32_t regen_threshold; /* refill finished lanes of a warp once this many are idle; 0 = default */
    int32_t interact_threshold; /* run the per-type interaction passes once this many lanes wait; 0 = default */
    int32_t queue_log2_chunk;   /* n > 0: photons are pre-generated in chunks of 2^n histories (48 B per
                                   photon); 0 = default (generated inside the transport kernel); -1 = inside */
    int32_t tracking;           /* DXMC_TRACKING_* of jobs that leave theirs at DEFAULT */
} dxmc_gpu_options;

int dxmc_gpu_ctx_create(const dxmc_gpu_options* options, dxmc_gpu_ctx** out);
void dxmc_gpu_ctx_destroy(dxmc_gpu_ctx* ctx);
const char* dxmc_gpu_last_error(const dxmc_gpu_ctx* ctx);
int dxmc_gpu_device_count(void);
int dxmc_gpu_abi_version(void);
/* Device-memory budget of the context and the bytes its worlds, LUTs, jobs and
 * batch buffers hold (the admission check of every upload and submit). */
int dxmc_gpu_ctx_memory(const dxmc_gpu_ctx* ctx, uint64_t* budget, uint64_t* in_use);
/* Page-locked host memory for result buffers (cudaHostAlloc / cudaFreeHost). */
int dxmc_gpu_host_alloc(uint64_t bytes, void** out);
void dxmc_gpu_host_free(void* ptr);

/* ---- world (World<T>, world.hpp:37-227) ---------------------------------- */
typedef struct dxmc_world_desc {
    uint64_t dims[3];
    double spacing[3];            /* mm */
    double origin[3];             /* mm, centre of the grid */
    double direction_cosines[6];
    const float* density;         /* g/cm3, x fastest; host pointer */
    const uint8_t* material;      /* material index, host pointer */
    const uint8_t* measurement;   /* forced-interaction map, may be NULL */
    int32_t n_materials;          /* material indices must be < n_materials */
    int32_t layout;               /* 0: compact 1-byte palette layout when the world has at most 256
                                     distinct (material, density, measurement) voxels, else 8-byte;
                                     1: always the 8-byte layout */
} dxmc_world_desc;

/* Validates like World::validate (world.hpp:182-227) and copies the arrays to
 * the device; the caller keeps ownership of the host arrays. */
int dxmc_gpu_world_upload(dxmc_gpu_ctx* ctx, const dxmc_world_desc* desc, dxmc_world** out);
/* Per-material maximum density of a resident world, computed on the device. */
int dxmc_gpu_world_max_density(dxmc_world* world, double* out, int n_materials);
void dxmc_gpu_world_free(dxmc_world* world);
/* Builds the local-majorant grid of a (world, LUT) pair ahead of its first job
 * (jobs with LOCAL tracking build it on first use; dxmc_gpu_transport_noalloc
 * uses it only if it exists).  A world keeps the grids of its last four LUTs:
 * building a fifth frees the least recently used one (after the jobs queued on
 * the context have finished), never one that an entry of the same batch reads.
 * The grid is built on the context's upload stream and is complete on return. */
int dxmc_gpu_world_prepare(dxmc_gpu_ctx* ctx, dxmc_world* world, const dxmc_lut* lut);
/* Reads back a built local-majorant grid: cells per axis, log2 of the cell size
 * in voxels per axis, the number of energy bands, the band edges (keV, bands - 1
 * values; may be NULL), the box of the cells above their band's emptiest level
 * (lo[3], hi[3] in mm from the grid corner's frame, lo = +inf and hi = -inf
 * where no box is used, as for the 8-byte voxel layout; may be NULL) and, if cells
 * is not NULL, (1 / scale, R mm) per cell and band, band fastest, then x, y, z;
 * R < 0 marks a cell outside that box (safe length |R|, or up to the box along
 * the ray).  DXMC_ERR_STATE if the pair has no grid. */
int dxmc_gpu_world_majorant(dxmc_gpu_ctx* ctx, dxmc_world* world, const dxmc_lut* lut, uint32_t* cells_per_axis,
    int32_t* shift, int32_t* bands, float* band_edges, float* box, float* cells);

/* ---- LUT on the device --------------------------------------------------- */
int dxmc_gpu_lut_upload(dxmc_gpu_ctx* ctx, const dxmc_lut_blob* blob, dxmc_lut** out);
void dxmc_gpu_lut_free(dxmc_lut* lut);

/* ---- jobs ---------------------------------------------------------------- */
typedef struct dxmc_job_desc {
    const dxmc_exposure* exposures;
    uint64_t n_exposures;
    const dxmc_spectrum_desc* spectrum; /* NULL: monoenergetic exposures */
    const dxmc_heel_desc* heel;         /* NULL: no heel effect */
    const dxmc_bowtie_desc* bowtie;     /* NULL: no bow-tie filter */
    uint64_t seed;                      /* counter-based RNG key */
    int32_t model;                      /* DXMC_MODEL_* */
    int32_t tally_mode;                 /* DXMC_TALLY_*; -1 = context default */
    /* launch parameters of this job (0 = the context's; set by an autotuner) */
    int32_t regen_threshold;            /* refill idle lanes once this many are idle (1..32) */
    int32_t interact_threshold;         /* interaction passes once this many lanes wait (1..32) */
    int32_t blocks_per_sm;              /* resident blocks per SM (1..occupancy limit) */
    int32_t queue_log2_chunk;           /* photon queue chunk 2^n; -1 = photons generated in the kernel */
    int32_t woodcock_burst;             /* Woodcock steps a lane may take per loop iteration (1..64) */
    int32_t block_size;                 /* threads per block of the transport kernel: 128 or 256 */
    int32_t tracking;                   /* DXMC_TRACKING_*; 0 = the context's */
    int32_t direction;                  /* DXMC_DIRECTION_* */
    /* DXMC_PRECISION_FP32 (0): FP32 transport with FP64 tallies, the default;
     * DXMC_PRECISION_FP64 (1): FP64 everywhere (position, direction, energy, LUT
     * evaluation and sampling in double, as Transport<double>, transport.hpp:114-840)
     * on the same per-history random streams; photons are generated in the kernel */
    int32_t precision;
} dxmc_job_desc;

#define DXMC_PRECISION_FP32 0
#define DXMC_PRECISION_FP64 1

typedef struct dxmc_job_stats {
    uint64_t histories;        /* histories simulated */
    uint64_t steps;            /* Woodcock steps inside the grid (S) */
    uint64_t deposits;         /* depositing events (D) */
    uint64_t rejection_overflows;
    double kernel_ms;          /* device time of the transport kernel */
    double job_ms;             /* device time from the job's first stream operation to the kernel's end */
} dxmc_job_stats;

/* Non-blocking: enqueues upload + transport on the context's stream. */
int dxmc_gpu_job_submit(dxmc_gpu_ctx* ctx, dxmc_world* world, dxmc_lut* lut,
    const dxmc_job_desc* job, dxmc_job** out);
/* Waits for completion; timeout_ms < 0 waits forever. Returns DXMC_ERR_TIMEOUT on expiry. */
int dxmc_gpu_job_wait(dxmc_job* job, int64_t timeout_ms);
/* Requests cancellation: the kernel stops taking new histories; results read as zero
 * (transport.hpp:176-185). */
int dxmc_gpu_job_cancel(dxmc_job* job);
/* Post-processes on the device (output_mode) and copies to host buffers of
 * world size; any output pointer may be NULL.  calibration multiplies DOSE. */
int dxmc_gpu_job_result(dxmc_job* job, int output_mode, double calibration,
    double* dose, double* variance, uint32_t* n_events, dxmc_job_stats* stats);
/* Live progress of a running job (ProgressBar, progressbar.hpp:42-80): the
 * histories its kernels have taken so far (photons generated in the kernel) or
 * queued (pre-generated photons); reads a device counter, does not wait. */
int dxmc_gpu_job_progress(dxmc_job* job, uint64_t* histories_started, uint64_t* histories_total);
/* Dose preview while the job runs (ProgressBar::setDoseData, progressbar.hpp:94-101):
 * copies the energy imparted scored so far (keV per voxel, FP64 tally mode)
 * into energy[n_voxels]; the values grow until the job ends. */
int dxmc_gpu_job_preview(dxmc_job* job, double* energy);
/* Frees a finished job's device buffers (tallies, tables) and returns them to
 * the memory budget; the handle stays valid for dxmc_gpu_job_free, results are
 * gone.  For batched jobs, whose handles the batch owns. */
int dxmc_gpu_job_release(dxmc_job* job);
void dxmc_gpu_job_free(dxmc_job* job);

/* ---- batches: many jobs in one persistent launch ---------------------------- */
/* No counterpart in the reference (which runs one source at a time).  Every
 * job keeps its own world, LUT, source tables and tallies; the jobs are cut
 * into work items on a device-side queue that one persistent kernel launch
 * (per correction model) drains.  A job's tallies are the same whether it runs
 * alone or in a batch (each history has its own random stream). */
typedef struct dxmc_batch dxmc_batch;
typedef struct dxmc_batch_entry {
    dxmc_world* world;
    dxmc_lut* lut;
    const dxmc_job_desc* job;
} dxmc_batch_entry;
enum {
    DXMC_BATCH_AUTO = 0,       /* currently the concurrent mode */
    DXMC_BATCH_CONCURRENT = 1, /* single-job kernels, jobs dealt onto parallel chains (streams) */
    DXMC_BATCH_PERSISTENT = 2  /* one multi-job kernel per model over a device-side work queue */
};
typedef struct dxmc_batch_options {
    int32_t mode;               /* DXMC_BATCH_* */
    int32_t chains;             /* concurrent mode: parallel chains (1..8); 0: 2 */
    int32_t regen_threshold;    /* persistent mode: refill idle lanes once this many are idle (1..32); 0: default */
    int32_t interact_threshold; /* persistent mode: interaction passes once this many lanes wait (1..32); 0: default */
    int32_t item_histories;     /* persistent mode: histories per work item; 0: automatic (256..8192) */
    int32_t pad;
} dxmc_batch_options;
/* Non-blocking.  At most 4096 jobs per batch; `options` may be NULL.
 * Concurrent mode: the context keeps up to 8 chains (stream + photon-queue buffer
 * of 48 B x 2^queue_log2_chunk each); a batch's jobs queue behind the work
 * already on those chains, so batches can be submitted while others run.
 * Persistent mode: two engines (stream + instantiated graph) are used in turn;
 * a third submit waits until the engine's previous batch has finished. */
int dxmc_gpu_batch_submit(dxmc_gpu_ctx* ctx, const dxmc_batch_entry* entries, int n_entries,
                          const dxmc_batch_options* options, dxmc_batch** out);
int dxmc_gpu_batch_wait(dxmc_batch* batch, int64_t timeout_ms);
/* Job handle of entry `index`, for dxmc_gpu_job_result; owned by the batch. */
int dxmc_gpu_batch_job(dxmc_batch* batch, int index, dxmc_job** job);
/* Device time from the batch's submission being ready to its last job's end (ms). */
double dxmc_gpu_batch_kernel_ms(dxmc_batch* batch);
void dxmc_gpu_batch_free(dxmc_batch* batch);

/* ---- Siddon traversal --------------------------------------------------------- */
/* No counterpart in the reference (which tracks photons with Woodcock steps only;
 * docs/sphinx/physicsmodel.rst:27).  Radiological path of straight rays through
 * the world: `rays` holds n_rays records of 7 floats (origin x, y, z in mm in the
 * world's grid frame, direction x, y, z (normalised here), energy in keV); the
 * part of each ray from its origin onwards is traversed voxel by voxel and
 * out[i] = sum over crossed voxels of mu_total(E, material) / rho * density *
 * length (cm), so exp(-out[i]) is the primary transmission.  Host buffers; blocks. */
int dxmc_gpu_radiological_path(dxmc_gpu_ctx* ctx, dxmc_world* world, dxmc_lut* lut, const float* rays, uint64_t n_rays,
                               double* out);

/* ---- transport without allocation ------------------------------------------ */
/* No counterpart in the reference.  Runs the same transport as
 * dxmc_gpu_job_submit + dxmc_gpu_job_result(DXMC_OUTPUT_RAW) for callers that
 * cannot allocate device memory once they are running (an application that
 * hands the library a fixed arena, a real-time loop that must not reach the
 * allocator): every piece of scratch the job needs lives in one fixed-size
 * static device array inside the library (about 2.2 MB per device, held until
 * the process exits), and the call makes no cudaMalloc / cudaFree or other
 * allocating call.  The caller passes the resident world and LUT and its own
 * device outputs: tally[2 * n_voxels] (voxel i: energy imparted sum at 2i,
 * sum of squares at 2i + 1, keV) and n_events[n_voxels]; both are cleared by
 * the call.  Limits: 8192 exposures, 2048 spectrum bins, 8192 heel weights,
 * 1024 bow-tie points; larger jobs return DXMC_ERR_INVALID with a message.
 * FP64 tallies only (job->tally_mode is ignored).  The call blocks until the
 * transport has finished; stats may be NULL (its times are host wall time).
 * All calls share the static array, so calls that overlap on the GPU race:
 * issue them one at a time.  The first call on a device looks the array up on
 * that device; make it before any stream capture. */
int dxmc_gpu_transport_noalloc(dxmc_gpu_ctx* ctx, dxmc_world* world, dxmc_lut* lut, const dxmc_job_desc* job,
    double* tally, uint32_t* n_events, dxmc_job_stats* stats);

/* Asynchronous results.  dxmc_gpu_job_result_async queues the post-processing
 * (output_mode and calibration as dxmc_gpu_job_result) and the copies into the
 * caller's buffers on the context's result stream, ordered after the job's
 * kernel, and returns at once: the caller may submit the next job meanwhile and
 * the copies run on the copy engine beside its transport.  result_type
 * DXMC_RESULT_F64 writes double dose / variance (Result<double>, 20 bytes per
 * voxel with the counts), DXMC_RESULT_F32 float ones (Result<float>, 12 bytes;
 * needs an FP64 tally).  Any of dose, variance, n_events may be NULL; page-locked
 * buffers make the copies asynchronous.  The buffers must stay valid until
 * dxmc_gpu_job_result_wait returns, which waits, fills stats and returns the
 * job's status as dxmc_gpu_job_result does (zeroed buffers and
 * DXMC_ERR_CANCELLED for a cancelled job).  One asynchronous result per job at
 * a time.  Together they replace the result hand-back of Transport<T>::operator()
 * (transport.hpp:176-201) for callers that overlap jobs. */
#define DXMC_RESULT_F64 0
#define DXMC_RESULT_F32 1
int dxmc_gpu_job_result_async(dxmc_job* job, int output_mode, double calibration, int result_type, void* dose,
    void* variance, uint32_t* n_events);
int dxmc_gpu_job_result_wait(dxmc_job* job, dxmc_job_stats* stats);

/* ---- device probes for component parity tests ----------------------------- */
/* Runs the device LUT lookup on energies[n]: out_att[n*3], out_maxinv[n]. */
int dxmc_gpu_probe_lut(dxmc_gpu_ctx* ctx, dxmc_lut* lut, int material, const double* energies, int n,
    double* out_att, double* out_maxinv);
/* Runs n independent interaction samples of one kind (0 photo, 1 Compton,
 * 2 Rayleigh) at a fixed energy in one material on the device, starting from
 * direction +z; writes cos(theta) of the new direction, the outgoing energy
 * and the energy imparted for each sample. */
int dxmc_gpu_probe_interactions(dxmc_gpu_ctx* ctx, dxmc_lut* lut, int material, int model, int kind,
    double energy, uint64_t n, uint64_t seed, float* out_cos, float* out_energy, float* out_deposit);

/* Histogram of the per-history random streams every device sampler draws
 * from (xoshiro128+ seeded by SplitMix64 of (seed, stream)): n_streams
 * streams of draws_per_stream values.  kind 0: uniform in [0, 1); kind 1: the
 * open-at-zero uniform in (0, 1] used for logarithms, binned as 1 - u; kind 2:
 * an integer below n_bins.  hist gets n_bins + 1 counts, the last one of the
 * values outside their range.  Replaces RandomState's generator
 * (dxmcrandom.hpp:37-167) and carries the reference's uniformity check
 * (tests/testrandom.cpp:21-58) over to the device generator. */
int dxmc_gpu_probe_uniform(dxmc_gpu_ctx* ctx, uint64_t seed, uint64_t n_streams, uint32_t draws_per_stream, int kind,
    int32_t n_bins, uint64_t* hist);

#ifdef __cplusplus
}
#endif

#endif /* DXMC_GPU_H */
