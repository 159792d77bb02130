// Siddon traversal: the radiological path of straight rays through the voxel
// grid.  DXMClib has no counterpart (it tracks photons with Woodcock steps only);
// the kernel serves primary-transmission and projection computations on the
// same resident world and LUT as the transport.
//
// One thread per ray, incremental form (Jacobs et al., Int. J. Imaging Syst.
// Technol. 1998): after the slab intersection with the grid box, the ray moves
// from one voxel boundary plane to the next, taking the nearest of the three
// next crossings, and adds mu / rho (LUT, recomputed only when the material
// changes) x density x segment length.
#include "transport.cuh"

namespace dxmc_gb300::dev {
namespace {

    template <bool PALETTE>
    __device__ __forceinline__ void voxel_at(const WorldParams& w, uint64_t idx, float& density, int& mat)
    {
        if constexpr (PALETTE) {
            const PaletteEntry e = w.palette[__ldg(w.palette_index + idx)];
            density = e.density;
            mat = static_cast<int>(e.code & 0xffu);
        } else {
            const uint2 raw = __ldg(reinterpret_cast<const uint2*>(w.voxels) + idx);
            density = __uint_as_float(raw.x);
            mat = static_cast<int>(raw.y & 0xffu);
        }
    }

    template <bool PALETTE>
    __global__ void __launch_bounds__(256) radiological_path_kernel(const __grid_constant__ WorldParams w, const float* __restrict__ L,
        const __grid_constant__ LutMeta m, const float* __restrict__ rays, uint64_t n, double* __restrict__ out)
    {
        for (uint64_t r = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; r < n; r += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
            const float* ray = rays + 7 * r;
            float o[3] = { ray[0], ray[1], ray[2] };
            float d[3] = { ray[3], ray[4], ray[5] };
            const float energy = ray[6];
            const float norm = sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            double result = 0.0;
            if (norm > 0.0f && energy > 0.0f) {
                for (int k = 0; k < 3; ++k)
                    d[k] /= norm;
                // slab intersection with the grid box, forward part of the ray only
                float tmin = 0.0f, tmax = INFINITY;
                bool hit = true;
                for (int k = 0; k < 3; ++k) {
                    const float lo = w.lower[k];
                    const float hi = w.lower[k] + w.spacing[k] * static_cast<float>(w.dims[k]);
                    if (d[k] != 0.0f) {
                        const float t1 = (lo - o[k]) / d[k];
                        const float t2 = (hi - o[k]) / d[k];
                        tmin = fmaxf(tmin, fminf(t1, t2));
                        tmax = fminf(tmax, fmaxf(t1, t2));
                    } else if (o[k] < lo || o[k] >= hi) {
                        hit = false;
                    }
                }
                if (hit && tmax > tmin) {
                    int idx[3], step[3];
                    float tnext[3], dt[3];
                    for (int k = 0; k < 3; ++k) {
                        // voxel of the first segment's midpoint-side: entry point nudged along the ray
                        const float p = o[k] + d[k] * tmin;
                        int i = static_cast<int>(floorf((p - w.lower[k]) / w.spacing[k]));
                        if (d[k] < 0.0f && p - w.lower[k] == static_cast<float>(i) * w.spacing[k])
                            --i; // on a boundary plane moving down: the voxel below
                        i = min(max(i, 0), static_cast<int>(w.dims[k]) - 1);
                        idx[k] = i;
                        if (d[k] > 0.0f) {
                            step[k] = 1;
                            tnext[k] = (w.lower[k] + static_cast<float>(i + 1) * w.spacing[k] - o[k]) / d[k];
                            dt[k] = w.spacing[k] / d[k];
                        } else if (d[k] < 0.0f) {
                            step[k] = -1;
                            tnext[k] = (w.lower[k] + static_cast<float>(i) * w.spacing[k] - o[k]) / d[k];
                            dt[k] = -w.spacing[k] / d[k];
                        } else {
                            step[k] = 0;
                            tnext[k] = INFINITY;
                            dt[k] = INFINITY;
                        }
                    }
                    const float logE = log10f(energy);
                    const int seg = lut_segment(L, m, logE);
                    int cached = -1;
                    float mu_rho = 0.0f;
                    float t = tmin;
                    float acc = 0.0f, comp = 0.0f; // compensated sum of mu * length (mm)
                    const int max_iter = static_cast<int>(w.dims[0] + w.dims[1] + w.dims[2]) + 3;
                    for (int it = 0; it < max_iter; ++it) {
                        const int k = tnext[0] <= tnext[1] ? (tnext[0] <= tnext[2] ? 0 : 2) : (tnext[1] <= tnext[2] ? 1 : 2);
                        const float tn = fminf(tnext[k], tmax);
                        if (tn > t) {
                            float density;
                            int mat;
                            voxel_at<PALETTE>(w, static_cast<uint64_t>(idx[2]) * w.nxy + static_cast<uint64_t>(idx[1]) * w.dims[0] + idx[0], density, mat);
                            if (mat != cached) {
                                float a0, a1, a2;
                                lut_attenuation(L, m, mat, logE, seg, a0, a1, a2);
                                mu_rho = a0 + a1 + a2;
                                cached = mat;
                            }
                            const float y = mu_rho * density * (tn - t) - comp;
                            const float s = acc + y;
                            comp = (s - acc) - y;
                            acc = s;
                            t = tn;
                        }
                        if (tnext[k] >= tmax)
                            break;
                        idx[k] += step[k];
                        if (idx[k] < 0 || idx[k] >= static_cast<int>(w.dims[k]))
                            break;
                        tnext[k] += dt[k];
                    }
                    result = 0.1 * static_cast<double>(acc); // mm -> cm
                }
            }
            out[r] = result;
        }
    }

} // namespace

cudaError_t launch_radiological_path(const WorldParams& w, const float* lut, LutMeta meta, const float* rays, uint64_t n,
    double* out, cudaStream_t stream)
{
    const int block = 256;
    const int grid = static_cast<int>(std::min<uint64_t>((n + block - 1) / block, 152ull * 32));
    if (w.palette_index)
        radiological_path_kernel<true><<<grid, block, 0, stream>>>(w, lut, meta, rays, n, out);
    else
        radiological_path_kernel<false><<<grid, block, 0, stream>>>(w, lut, meta, rays, n, out);
    return cudaGetLastError();
}

} // namespace dxmc_gb300::dev
