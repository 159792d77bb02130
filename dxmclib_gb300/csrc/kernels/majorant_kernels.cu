// Construction of the local-majorant grid of a (world, LUT) pair.
//
// The reference tracks every photon with one global majorant: the largest
// attenuation of any material at its largest density (woodcockParticleTracking,
// transport.hpp:640-700, with AttenuationLut::maxMassTotalAttenuation).  In a CT
// body phantom that bound is set by cortical bone, so in air, lung and soft
// tissue nearly every Woodcock step is a virtual collision.  The grid built here
// lets the transport kernel use a smaller majorant where the neighbourhood of a
// photon allows it (see MajorantGrid in transport.cuh):
//
//   1. per energy band, every voxel gets a scale s_v = density * r_m, with r_m
//      the largest ratio of material m's attenuation to the global majorant
//      over the band's energies (1 for voxels of forced-interaction scoring,
//      which keep the reference's majorant); each cell takes the maximum over
//      its voxels, rounded up to a level 2^(-level / levels_per_octave) (one
//      pass over the voxels for all bands, with a histogram of the levels);
//   2. for each level the cells have (the host picks at most a dozen per band
//      from the histogram), the cells above it are dilated by one cell (one
//      min-filter of the levels over the 27-neighbourhood serves every level)
//      and a Euclidean distance transform (three separable passes over the
//      cell grid, cell sizes in mm: warp scans along x rows, scans along y and
//      z) gives every
//      other cell the distance R to the nearest point of a cell above the
//      level: a flight of length at most R from anywhere in the cell stays
//      where the level's scale bounds the attenuation.  All (band, level)
//      pairs of a group run in one launch per pass (blockIdx.y = pair);
//   3. each cell keeps the (level, R) of smallest expected steps per mm,
//      mu / (1 - exp(-mu R)) with mu = scale * global majorant at the band's
//      reference energy, or the global majorant itself (R infinite); one
//      thread per cell and band tries the band's levels in ascending order,
//      so the grid does not depend on the grouping.
// Last, the cells outside the box of all cells above their band's emptiest
// level get -R: there a flight may also run to that box (MajorantGrid).
#include <algorithm>
#include <cmath>

#include "transport.cuh"

namespace dxmc_gb300::dev {

namespace {

__device__ __forceinline__ void cell_coords(uint64_t c, const MajorantBuild& b, uint32_t& cx, uint32_t& cy, uint32_t& cz)
{
    cx = static_cast<uint32_t>(c % b.n[0]);
    const uint64_t t = c / b.n[0];
    cy = static_cast<uint32_t>(t % b.n[1]);
    cz = static_cast<uint32_t>(t / b.n[1]);
}

__device__ __forceinline__ float level_scale(int level, int per_octave)
{
    return exp2f(-static_cast<float>(level) / static_cast<float>(per_octave));
}

// Cell levels of every band in one pass over the voxels: scales holds bands x 256
// scales (per palette entry, or r_m per material for the 8-byte layout); level
// and cost are bands x ncell, cells ncell x bands.
__global__ void majorant_level_kernel(WorldParams w, const float* __restrict__ scales, MajorantBuild b,
    uint8_t* __restrict__ level, float2* __restrict__ cells, float* __restrict__ cost, int* __restrict__ bounds,
    unsigned int* __restrict__ hist)
{
    __shared__ float scale_table[MAJORANT_MAX_BANDS * PALETTE_MAX];
    __shared__ unsigned int shist[MAJORANT_MAX_BANDS * 64];
    for (int i = threadIdx.x; i < b.bands * PALETTE_MAX; i += blockDim.x)
        scale_table[i] = scales[i];
    for (int i = threadIdx.x; i < MAJORANT_MAX_BANDS * 64; i += blockDim.x)
        shist[i] = 0u;
    __syncthreads();
    const uint64_t ncell = static_cast<uint64_t>(b.n[0]) * b.n[1] * b.n[2];
    for (uint64_t c = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; c < ncell;
         c += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        uint32_t cx, cy, cz;
        cell_coords(c, b, cx, cy, cz);
        const uint32_t x0 = cx << b.shift[0], x1 = min(w.dims[0], (cx + 1) << b.shift[0]);
        const uint32_t y0 = cy << b.shift[1], y1 = min(w.dims[1], (cy + 1) << b.shift[1]);
        const uint32_t z0 = cz << b.shift[2], z1 = min(w.dims[2], (cz + 1) << b.shift[2]);
        float m[MAJORANT_MAX_BANDS];
#pragma unroll
        for (int k = 0; k < MAJORANT_MAX_BANDS; ++k)
            m[k] = 0.0f;
        int last_idx = -1; // a voxel equal to the one before adds nothing to the maxima
        float last_dens = 0.0f;
        bool last_forced = false;
        for (uint32_t z = z0; z < z1; ++z) {
            for (uint32_t y = y0; y < y1; ++y) {
                const uint64_t row = static_cast<uint64_t>(z) * w.nxy + static_cast<uint64_t>(y) * w.dims[0];
                for (uint32_t x = x0; x < x1; ++x) {
                    int idx;
                    float dens = 1.0f;
                    bool forced = false;
                    if (w.palette_index) {
                        idx = w.palette_index[row + x];
                    } else {
                        const Voxel v = w.voxels[row + x];
                        idx = v.material;
                        dens = v.density;
                        forced = v.measurement != 0;
                    }
                    if (idx == last_idx && dens == last_dens && forced == last_forced)
                        continue;
                    last_idx = idx;
                    last_dens = dens;
                    last_forced = forced;
#pragma unroll
                    for (int k = 0; k < MAJORANT_MAX_BANDS; ++k)
                        if (k < b.bands)
                            m[k] = fmaxf(m[k], forced ? 1.0f : dens * scale_table[k * PALETTE_MAX + idx]);
                }
            }
        }
        bool above = false;
#pragma unroll
        for (int k = 0; k < MAJORANT_MAX_BANDS; ++k) {
            if (k >= b.bands)
                break;
            int lv = b.max_level;
            if (m[k] >= 1.0f) {
                lv = 0;
            } else if (m[k] > 0.0f) {
                lv = min(b.max_level, static_cast<int>(floorf(-static_cast<float>(b.levels_per_octave) * log2f(m[k]))));
                // the level's scale must not fall below the cell's maximum, whatever the rounding of log2f
                while (lv > 0 && level_scale(lv, b.levels_per_octave) < m[k])
                    --lv;
            }
            level[k * ncell + c] = static_cast<uint8_t>(lv);
            atomicAdd(&shist[k * 64 + lv], 1u);
            cells[c * b.bands + k] = make_float2(1.0f, INFINITY); // the global majorant until a level does better
            cost[k * ncell + c] = b.mu_refs[k];
            above = above || (b.floor_levels[k] >= 0 && lv < b.floor_levels[k]);
        }
        // cells above their band's emptiest level widen the box (warp-reduced atomics)
        const unsigned mask = __ballot_sync(__activemask(), above);
        if (mask) {
            const unsigned active = __activemask();
            const int big = 0x7fffffff;
            const int lo[3] = { above ? static_cast<int>(cx) : big, above ? static_cast<int>(cy) : big, above ? static_cast<int>(cz) : big };
            const int hi[3] = { above ? static_cast<int>(cx) : -1, above ? static_cast<int>(cy) : -1, above ? static_cast<int>(cz) : -1 };
            const bool leader = (threadIdx.x & 31) == __ffs(active) - 1;
            for (int a = 0; a < 3; ++a) {
                const int mn = __reduce_min_sync(active, lo[a]);
                const int mx = __reduce_max_sync(active, hi[a]);
                if (leader) {
                    atomicMin(bounds + a, mn);
                    atomicMax(bounds + 3 + a, mx);
                }
            }
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < b.bands * 64; i += blockDim.x)
        if (shist[i])
            atomicAdd(hist + i, shist[i]);
}

__global__ void majorant_box_kernel(const __grid_constant__ MajorantBuild b, const int* __restrict__ bounds, float2* __restrict__ cells, float* __restrict__ box)
{
    int lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
        lo[a] = bounds[a];
        hi[a] = bounds[3 + a];
    }
    const bool empty = lo[0] > hi[0];
    if (blockIdx.x == 0 && threadIdx.x < 3) {
        const int a = threadIdx.x;
        box[a] = empty ? INFINITY : b.lower[a] + static_cast<float>(lo[a]) * b.edge[a];
        box[3 + a] = empty ? -INFINITY : b.lower[a] + static_cast<float>(hi[a] + 1) * b.edge[a];
    }
    const uint64_t ncell = static_cast<uint64_t>(b.n[0]) * b.n[1] * b.n[2];
    for (uint64_t c = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; c < ncell;
         c += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        uint32_t q[3];
        cell_coords(c, b, q[0], q[1], q[2]);
        bool outside = empty;
        for (int a = 0; a < 3; ++a)
            outside = outside || static_cast<int>(q[a]) < lo[a] || static_cast<int>(q[a]) > hi[a];
        if (!outside)
            continue;
        for (int k = 0; k < b.bands; ++k) {
            // every cell outside the box lies at or below the band's emptiest level (the
            // box holds every cell above it), so a flight drawn with that level's scale
            // may run to the box: a cell whose own scale is smaller takes the level's
            // (a larger majorant bounds everything its own did, within its R as well)
            const int fl = b.floor_levels[k];
            float2& cell = cells[c * b.bands + k];
            if (fl >= 0) {
                cell.x = fminf(cell.x, 1.0f / level_scale(fl, b.levels_per_octave));
                cell.y = -cell.y;
            }
        }
    }
}

// minlev[k][c] = the lowest level (largest scale) of band k in the 27-neighbourhood
// of cell c (blockIdx.y = band): cell c lies in the dilated set of level lv, the
// cells above lv grown by one cell, exactly when minlev < lv.
__global__ void majorant_minfilter_kernel(MajorantBuild b, const uint8_t* __restrict__ level, uint8_t* __restrict__ minlev)
{
    const uint64_t ncell = static_cast<uint64_t>(b.n[0]) * b.n[1] * b.n[2];
    const uint64_t off = static_cast<uint64_t>(blockIdx.y) * ncell;
    const uint8_t* __restrict__ lvl = level + off;
    for (uint64_t c = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; c < ncell;
         c += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        uint32_t cx, cy, cz;
        cell_coords(c, b, cx, cy, cz);
        int lo = 255;
        for (int dz = -1; dz <= 1; ++dz) {
            const int z = static_cast<int>(cz) + dz;
            if (z < 0 || z >= static_cast<int>(b.n[2]))
                continue;
            for (int dy = -1; dy <= 1; ++dy) {
                const int y = static_cast<int>(cy) + dy;
                if (y < 0 || y >= static_cast<int>(b.n[1]))
                    continue;
                const uint64_t row = (static_cast<uint64_t>(z) * b.n[1] + y) * b.n[0];
                for (int dx = -1; dx <= 1; ++dx) {
                    const int x = static_cast<int>(cx) + dx;
                    if (x >= 0 && x < static_cast<int>(b.n[0]))
                        lo = min(lo, static_cast<int>(lvl[row + x]));
                }
            }
        }
        minlev[off + c] = static_cast<uint8_t>(lo);
    }
}

// One step of the separable squared distance transform at position pos of a
// line of n cells of size e: min over t of get(t) + ((pos - t) * e)^2, scanned
// outward from pos until the distance alone exceeds the best value.
template <typename Get>
__device__ __forceinline__ float line_min(Get get, int n, int pos, float e)
{
    float best = get(pos);
    for (int k = 1; k < n; ++k) {
        const float dk = static_cast<float>(k) * e;
        const float d2 = dk * dk;
        if (d2 >= best)
            break;
        const bool lo = pos - k >= 0, hi = pos + k < n;
        if (!lo && !hi)
            break;
        if (lo)
            best = fminf(best, get(pos - k) + d2);
        if (hi)
            best = fminf(best, get(pos + k) + d2);
    }
    return best;
}

// line_min along AXIS through cell c, reading the grid in global memory
template <int AXIS>
__device__ __forceinline__ float axis_min(const MajorantBuild& b, const float* __restrict__ in, uint64_t c, int pos)
{
    const uint64_t stride = AXIS == 0 ? 1 : (AXIS == 1 ? b.n[0] : static_cast<uint64_t>(b.n[0]) * b.n[1]);
    const uint64_t base = c - static_cast<uint64_t>(pos) * stride;
    return line_min([&](int t) { return in[base + static_cast<uint64_t>(t) * stride]; }, static_cast<int>(b.n[AXIS]), pos,
        b.edge[AXIS]);
}

// Shared-memory tiles for the y and z passes: the lines of 32 adjacent x cells,
// tile[t * 32 + lane] = the line of x0 + lane at position t (infinity past the
// grid), so a warp scanning its 32 lines reads 32 consecutive banks.
constexpr int TILE_W = 32;
constexpr size_t TILE_SMEM_MAX = 48 * 1024;

__device__ __forceinline__ void load_tile(float* tile, const float* __restrict__ src, uint32_t x0, uint32_t n0, int n,
    uint64_t base, uint64_t stride)
{
    for (uint32_t i = threadIdx.x; i < static_cast<uint32_t>(n) * TILE_W; i += blockDim.x) {
        const uint32_t t = i / TILE_W, x = x0 + i % TILE_W;
        tile[i] = x < n0 ? src[base + t * stride + x] : INFINITY;
    }
}

// A middle pass of the distance transform for every pair (blockIdx.y = pair).
template <int AXIS>
__global__ void majorant_axis_kernel(MajorantBuild b, const float* __restrict__ in, float* __restrict__ out)
{
    const uint64_t ncell = static_cast<uint64_t>(b.n[0]) * b.n[1] * b.n[2];
    const uint64_t off = static_cast<uint64_t>(blockIdx.y) * ncell;
    for (uint64_t c = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; c < ncell;
         c += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        uint32_t coord[3];
        cell_coords(c, b, coord[0], coord[1], coord[2]);
        out[off + c] = axis_min<AXIS>(b, in + off, c, static_cast<int>(coord[AXIS]));
    }
}

// The last (z) pass of every pair, then the choice (blockIdx.y = band): each
// cell keeps the best of its current (scale, R) and its band's levels of the
// group, in ascending order; R is the distance less a small margin that keeps
// rounding of the photon's position on the safe side.
__global__ void majorant_choose_kernel(const __grid_constant__ MajorantBuild b, const __grid_constant__ MajorantPairs pairs,
    const float* __restrict__ d, float2* __restrict__ cells, float* __restrict__ cost)
{
    const int band = blockIdx.y;
    const int p0 = pairs.first[band], p1 = pairs.first[band + 1];
    if (p0 == p1)
        return;
    const uint64_t ncell = static_cast<uint64_t>(b.n[0]) * b.n[1] * b.n[2];
    const float mu_ref = b.mu_refs[band];
    for (uint64_t c = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; c < ncell;
         c += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        uint32_t cx, cy, cz;
        cell_coords(c, b, cx, cy, cz);
        float best_cost = cost[static_cast<uint64_t>(band) * ncell + c];
        float2 choice = make_float2(0.0f, 0.0f);
        bool changed = false;
        for (int p = p0; p < p1; ++p) {
            const float best = axis_min<2>(b, d + static_cast<uint64_t>(p) * ncell, c, static_cast<int>(cz));
            if (best <= 0.0f)
                continue; // the cell itself lies in the dilated set
            const float R = fmaf(sqrtf(best), 0.999f, -1.0e-3f);
            if (!(R > 0.0f))
                continue;
            const float s = level_scale(pairs.level[p], b.levels_per_octave);
            const float mu = mu_ref * s;
            const float c_new = mu / (1.0f - expf(-mu * R)); // R infinite: mu
            if (c_new < best_cost) {
                best_cost = c_new;
                choice = make_float2(1.0f / s, R);
                changed = true;
            }
        }
        if (changed) {
            cost[static_cast<uint64_t>(band) * ncell + c] = best_cost;
            cells[c * b.bands + band] = choice;
        }
    }
}

// The y (AXIS 1) or z (AXIS 2) pass with tiles in shared memory (blockIdx.y =
// pair): one tile per x group of 32 cells and the other axis' position, the
// block's warps taking the cells of the lines in turn.
template <int AXIS>
__global__ void majorant_axis_tiled_kernel(MajorantBuild b, const float* __restrict__ in, float* __restrict__ out)
{
    extern __shared__ float tile[];
    const uint32_t n0 = b.n[0], n1 = b.n[1], n2 = b.n[2];
    const uint64_t ncell = static_cast<uint64_t>(n0) * n1 * n2;
    const uint64_t off = static_cast<uint64_t>(blockIdx.y) * ncell;
    const uint32_t n = AXIS == 1 ? n1 : n2;      // cells along the lines
    const uint32_t other = AXIS == 1 ? n2 : n1;  // positions of the tiles across them
    const uint64_t stride = AXIS == 1 ? n0 : static_cast<uint64_t>(n0) * n1;
    const uint64_t other_stride = AXIS == 1 ? static_cast<uint64_t>(n0) * n1 : n0;
    const uint32_t xtiles = (n0 + TILE_W - 1) / TILE_W;
    const uint64_t tiles = static_cast<uint64_t>(xtiles) * other;
    const uint32_t lane = threadIdx.x % TILE_W, warps = blockDim.x / TILE_W;
    for (uint64_t ti = blockIdx.x; ti < tiles; ti += gridDim.x) {
        const uint32_t o = static_cast<uint32_t>(ti / xtiles), x0 = static_cast<uint32_t>(ti % xtiles) * TILE_W;
        const uint64_t base = off + o * other_stride;
        __syncthreads(); // the previous tile is no longer read
        load_tile(tile, in, x0, n0, static_cast<int>(n), base, stride);
        __syncthreads();
        const uint32_t x = x0 + lane;
        for (uint32_t t = threadIdx.x / TILE_W; t < n; t += warps) {
            const float best = line_min([&](int k) { return tile[k * TILE_W + lane]; }, static_cast<int>(n),
                static_cast<int>(t), b.edge[AXIS]);
            if (x < n0)
                out[base + t * stride + x] = best;
        }
    }
}

// The choice after a tiled z pass (blockIdx.y = band): d holds each pair's
// squared distances; the arithmetic of majorant_choose_kernel.
__global__ void majorant_choose_final_kernel(const __grid_constant__ MajorantBuild b, const __grid_constant__ MajorantPairs pairs,
    const float* __restrict__ d, float2* __restrict__ cells, float* __restrict__ cost)
{
    const int band = blockIdx.y;
    const int p0 = pairs.first[band], p1 = pairs.first[band + 1];
    if (p0 == p1)
        return;
    const uint64_t ncell = static_cast<uint64_t>(b.n[0]) * b.n[1] * b.n[2];
    const float mu_ref = b.mu_refs[band];
    for (uint64_t c = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; c < ncell;
         c += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        float best_cost = cost[static_cast<uint64_t>(band) * ncell + c];
        float2 choice = make_float2(0.0f, 0.0f);
        bool changed = false;
        for (int p = p0; p < p1; ++p) {
            const float best = d[static_cast<uint64_t>(p) * ncell + c];
            if (best <= 0.0f)
                continue; // the cell itself lies in the dilated set
            const float R = fmaf(sqrtf(best), 0.999f, -1.0e-3f);
            if (!(R > 0.0f))
                continue;
            const float s = level_scale(pairs.level[p], b.levels_per_octave);
            const float mu = mu_ref * s;
            const float c_new = mu / (1.0f - expf(-mu * R)); // R infinite: mu
            if (c_new < best_cost) {
                best_cost = c_new;
                choice = make_float2(1.0f / s, R);
                changed = true;
            }
        }
        if (changed) {
            cost[static_cast<uint64_t>(band) * ncell + c] = best_cost;
            cells[c * b.bands + band] = choice;
        }
    }
}

// The first (x) pass of the distance transform on the dilated set of pair p
// (blockIdx.y = p; minlev < the pair's level): one warp per grid row finds each
// cell's nearest set cell before and after it on the row with a max- and a
// min-scan over 32-cell chunks, carried from chunk to chunk, and writes the
// squared distance (cell sizes in mm) to out.
__global__ void majorant_sweep_x_kernel(MajorantBuild b, const __grid_constant__ MajorantPairs pairs,
    const uint8_t* __restrict__ minlev, float* __restrict__ out)
{
    const uint64_t rows = static_cast<uint64_t>(b.n[1]) * b.n[2];
    const int n = static_cast<int>(b.n[0]);
    const float e = b.edge[0];
    const int p = blockIdx.y;
    const int lv = pairs.level[p];
    const uint64_t ncell = rows * n;
    const uint8_t* __restrict__ in = minlev + static_cast<uint64_t>(pairs.band[p]) * ncell;
    float* __restrict__ dst = out + static_cast<uint64_t>(p) * ncell;
    const int lane = threadIdx.x & 31;
    const uint64_t warps = static_cast<uint64_t>(gridDim.x) * (blockDim.x >> 5);
    for (uint64_t r = blockIdx.x * static_cast<uint64_t>(blockDim.x >> 5) + (threadIdx.x >> 5); r < rows; r += warps) {
        const uint8_t* row_in = in + r * n;
        float* row_out = dst + r * n;
        int last = -1; // the nearest set cell at or before the chunk's cells
        for (int x0 = 0; x0 < n; x0 += 32) {
            const int x = x0 + lane;
            int v = (x < n && row_in[x] < lv) ? x : -1;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, v, o);
                if (lane >= o)
                    v = max(v, t);
            }
            v = max(v, last);
            if (x < n)
                row_out[x] = v >= 0 ? static_cast<float>(x - v) : INFINITY;
            last = __shfl_sync(0xffffffffu, v, 31);
        }
        constexpr int none = 0x7fffffff;
        int next = none; // the nearest set cell at or after the chunk's cells
        for (int x0 = ((n - 1) / 32) * 32; x0 >= 0; x0 -= 32) {
            const int x = x0 + lane;
            int v = (x < n && row_in[x] < lv) ? x : none;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_down_sync(0xffffffffu, v, o);
                if (lane + o < 32)
                    v = min(v, t);
            }
            v = min(v, next);
            if (x < n) {
                const float k = fminf(row_out[x], v != none ? static_cast<float>(v - x) : INFINITY);
                const float d = k * e;
                row_out[x] = d * d;
            }
            next = __shfl_sync(0xffffffffu, v, 0);
        }
    }
}

int grid_for(uint64_t n)
{
    const uint64_t blocks = (n + 255) / 256;
    return static_cast<int>(blocks < 4096 ? (blocks > 0 ? blocks : 1) : 4096);
}

} // namespace

cudaError_t launch_majorant_levels(const WorldParams& w, const float* scales, const MajorantBuild& b,
    uint8_t* level, float2* cells, float* cost, int* bounds, unsigned int* hist, cudaStream_t stream)
{
    const uint64_t ncell = static_cast<uint64_t>(b.n[0]) * b.n[1] * b.n[2];
    majorant_level_kernel<<<grid_for(ncell), 256, 0, stream>>>(w, scales, b, level, cells, cost, bounds, hist);
    return cudaGetLastError();
}

cudaError_t launch_majorant_box(const MajorantBuild& b, const int* bounds, float2* cells, float* box, cudaStream_t stream)
{
    const uint64_t ncell = static_cast<uint64_t>(b.n[0]) * b.n[1] * b.n[2];
    majorant_box_kernel<<<grid_for(ncell), 256, 0, stream>>>(b, bounds, cells, box);
    return cudaGetLastError();
}

cudaError_t launch_majorant_minfilter(const MajorantBuild& b, const uint8_t* level, uint8_t* minlev, cudaStream_t stream)
{
    const uint64_t ncell = static_cast<uint64_t>(b.n[0]) * b.n[1] * b.n[2];
    majorant_minfilter_kernel<<<dim3(grid_for(ncell), b.bands), 256, 0, stream>>>(b, level, minlev);
    return cudaGetLastError();
}

cudaError_t launch_majorant_level_passes(const MajorantBuild& b, const MajorantPairs& pairs, const uint8_t* minlev,
    float* d0, float* d1, float2* cells, float* cost, cudaStream_t stream)
{
    if (pairs.count <= 0)
        return cudaSuccess;
    const uint64_t ncell = static_cast<uint64_t>(b.n[0]) * b.n[1] * b.n[2];
    const uint64_t rows = static_cast<uint64_t>(b.n[1]) * b.n[2];
    majorant_sweep_x_kernel<<<dim3(static_cast<unsigned>(std::min<uint64_t>((rows + 7) / 8, 4096)), pairs.count), 256, 0, stream>>>(
        b, pairs, minlev, d1);
    // the y and z passes from shared-memory tiles where a tile's lines fit (the
    // same arithmetic in the same order as the global-memory kernels), the
    // choice then one thread per cell and band; otherwise the z pass runs inside
    // the choice from global memory
    const size_t smem_y = static_cast<size_t>(b.n[1]) * TILE_W * sizeof(float);
    const size_t smem_z = static_cast<size_t>(b.n[2]) * TILE_W * sizeof(float);
    const uint64_t xtiles = (b.n[0] + TILE_W - 1) / TILE_W;
    if (smem_y <= TILE_SMEM_MAX)
        majorant_axis_tiled_kernel<1><<<dim3(static_cast<unsigned>(std::min<uint64_t>(xtiles * b.n[2], 4096)), pairs.count), 256, smem_y,
            stream>>>(b, d1, d0);
    else
        majorant_axis_kernel<1><<<dim3(grid_for(ncell), pairs.count), 256, 0, stream>>>(b, d1, d0);
    if (smem_z <= TILE_SMEM_MAX) {
        majorant_axis_tiled_kernel<2><<<dim3(static_cast<unsigned>(std::min<uint64_t>(xtiles * b.n[1], 4096)), pairs.count), 256, smem_z,
            stream>>>(b, d0, d1);
        majorant_choose_final_kernel<<<dim3(grid_for(ncell), b.bands), 256, 0, stream>>>(b, pairs, d1, cells, cost);
    } else {
        majorant_choose_kernel<<<dim3(grid_for(ncell), b.bands), 256, 0, stream>>>(b, pairs, d0, cells, cost);
    }
    return cudaGetLastError();
}

} // namespace dxmc_gb300::dev
