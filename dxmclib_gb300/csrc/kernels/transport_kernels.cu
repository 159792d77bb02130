// Photon-transport kernels for sm_103a.
//
// One persistent launch per job: every lane owns one photon history at a
// time and, inside a warp-synchronous loop, takes a burst of Woodcock steps per
// iteration.  Lanes whose history ended take the next history id from a
// warp-local pool that one lane refills from a global work queue, so warps
// stay full until the job runs dry.  Physics follows DXMClib's
// Transport<T> (include/dxmc/transport.hpp) function by function; each
// device function names the reference lines it restates.
#include "transport.cuh"

#include <mutex>

#include <algorithm>

namespace dxmc_gb300::dev {

namespace {

    constexpr unsigned FULL_MASK = 0xffffffffu;
    constexpr int WARP_POOL_CHUNK = 256; // histories fetched per queue access
    constexpr uint32_t MAX_STEPS_PER_HISTORY = 1u << 20; // guard against unbounded histories

    template <class Real>
    struct PhotonT {
        Real px, py, pz;
        Real dx, dy, dz;
        Real energy;
        Real weight;
    };

    // ---- scoring (transport.hpp:208-214, 598-609) ------------------------------
    // Atomic additions to the tally with an L2 evict-first policy: the tally is
    // read-modify-written at random voxels and would otherwise push the voxel and
    // majorant grids (gathered on every flight) out of L2.
    __device__ __forceinline__ void red_add_evict_first(double* a, double v)
    {
#ifdef DXMC_TALLY_NO_HINT
        atomicAdd(a, v);
        return;
#endif
        asm volatile("{\n\t.reg .b64 pol;\n\tcreatepolicy.fractional.L2::evict_first.b64 pol, 1.0;\n\t"
                     "red.global.add.L2::cache_hint.f64 [%0], %1, pol;\n\t}" ::"l"(a), "d"(v) : "memory");
    }
    __device__ __forceinline__ void red_add_evict_first(uint32_t* a, uint32_t v)
    {
#ifdef DXMC_TALLY_NO_HINT
        atomicAdd(a, v);
        return;
#endif
        asm volatile("{\n\t.reg .b64 pol;\n\tcreatepolicy.fractional.L2::evict_first.b64 pol, 1.0;\n\t"
                     "red.global.add.L2::cache_hint.u32 [%0], %1, pol;\n\t}" ::"l"(a), "r"(v) : "memory");
    }
    __device__ __forceinline__ void score_record(TallyRecord* r, double e, double e2, uint32_t n)
    {
        red_add_evict_first(&r->energy, e);
        red_add_evict_first(&r->energy2, e2);
        red_add_evict_first(&r->events, n);
    }

    template <class Real>
    __device__ __forceinline__ void score(const TransportParams& p, uint64_t idx, Real e)
    {
        if (p.records) {
            const double ed = static_cast<double>(e);
            score_record(p.records + idx, ed, ed * ed, 1u);
            return;
        }
        if (p.tally_mode == 1) {
            float* t = p.tally_f32 + 2 * idx;
            atomicAdd(t, e);
            atomicAdd(t + 1, e * e);
        } else {
            double* t = p.tally + 2 * idx;
            const double ed = static_cast<double>(e);
            atomicAdd(t, ed);
            atomicAdd(t + 1, ed * ed);
        }
        atomicAdd(p.n_events + idx, 1u);
    }

    // Warp-aggregated scoring: lanes depositing into the same voxel in the same
    // iteration are combined by __match_any_sync and one leader issues the
    // atomics (FP32 partial sums flushed to the FP64 accumulators).
    template <class Real>
    __device__ __forceinline__ void score_aggregated(const TransportParams& p, unsigned active, uint64_t idx, Real e)
    {
        const unsigned peers = __match_any_sync(active, idx);
        const int leader = __ffs(peers) - 1;
        const int lane = threadIdx.x & 31;
        Real sum = Real(0.0), sum2 = Real(0.0);
        unsigned count = 0;
        // each peer group reduces over its members (group sizes are small)
        for (unsigned m = peers; m; m &= m - 1) {
            const int src = __ffs(m) - 1;
            const Real v = __shfl_sync(peers, e, src);
            sum += v;
            sum2 += v * v;
            ++count;
        }
        if (lane == leader) {
            if (p.records) {
                score_record(p.records + idx, static_cast<double>(sum), static_cast<double>(sum2), count);
            } else {
                double* t = p.tally + 2 * idx;
                atomicAdd(t, static_cast<double>(sum));
                atomicAdd(t + 1, static_cast<double>(sum2));
                atomicAdd(p.n_events + idx, count);
            }
        }
    }

    // ---- photoelectric (transport.hpp:216-263) ---------------------------------
    template <int MODEL, class Real>
    __device__ __forceinline__ Real photo_absorption(const float* L, const LutMeta& m, PhotonT<Real>& ph, int material, Rng& rng, bool norm = false)
    {
        const Real E = ph.energy;
        ph.energy = Real(0.0);
        if constexpr (MODEL < 2) {
            return E;
        } else {
            const float* shells = L + m.off_shells + material * N_SHELLS * SHELL_FLOATS;
            Real total = Real(0.0);
#pragma unroll
            for (int s = 0; s < N_SHELLS; ++s)
                total += E > shells[s * SHELL_FLOATS] ? shells[s * SHELL_FLOATS + 3] : Real(0.0);
            const Real sample = total * static_cast<Real>(rng.uniform());
            Real cum = Real(0.0);
            int idx = 0;
            for (int s = 0; s < N_SHELLS; ++s) {
                cum += E > shells[s * SHELL_FLOATS] ? shells[s * SHELL_FLOATS + 3] : Real(0.0);
                idx = s;
                if (!(cum < sample) || s == N_SHELLS - 1)
                    break;
            }
            const float* sh = shells + idx * SHELL_FLOATS;
            const Real binding = sh[0];
            if (binding > E || binding < Real(ENERGY_CUTOFF_D))
                return E;
            const Real r1 = static_cast<Real>(rng.uniform());
            if (r1 <= sh[4]) {
                int line = 0;
                Real r3 = static_cast<Real>(rng.uniform()) - sh[5];
                while (r3 > Real(0.0) && line < 2) {
                    ++line;
                    r3 -= sh[5 + line];
                }
                ph.energy = sh[8 + line];
                const Real theta = static_cast<Real>(rng.uniform()) * Real(PI_D);
                const Real phi = rng_azimuth<Real>(rng);
                peturb(ph.dx, ph.dy, ph.dz, m_cos(theta), phi, norm);
                return E - ph.energy;
            }
            return E;
        }
    }

    // ---- Rayleigh (transport.hpp:264-298) ---------------------------------------
    template <int MODEL, class Real>
    __device__ __forceinline__ bool rayleigh_scatter(const float* L, const float* G, const LutMeta& m, PhotonT<Real>& ph, int material, Rng& rng, bool norm = false)
    {
        if constexpr (MODEL == 0) {
            constexpr Real extreme = Real(1.08866210790363); // 4 sqrt(2) / (3 sqrt(3))
            for (int it = 0; it < REJECTION_CAP; ++it) {
                const Real r1 = static_cast<Real>(rng.uniform()) * extreme;
                const Real theta = static_cast<Real>(rng.uniform()) * Real(PI_D);
                Real s, c;
                m_sincos(theta, &s, &c);
                if (!(r1 > (Real(2.0) - s * s) * s)) {
                    const Real phi = rng_azimuth<Real>(rng);
                    peturb(ph.dx, ph.dy, ph.dz, c, phi, norm);
                    return true;
                }
            }
            return false;
        } else {
            // the density of the reference's RITA draw of q^2 <= q_max^2 followed by the
            // (1 + cos^2) / 2 rejection, drawn by inverse CDF: no loop, no divergence
            Real fe;
            const int row = table_row(m, ph.energy, fe);
            const Real y = table_quantile(G + m.off_ray + (material * m.tab_ne + row) * (m.tab_nu + 1), m.tab_nu, static_cast<Real>(rng.uniform()), fe);
            const Real cosA = Real(1.0) - Real(2.0) * y; // q^2 / q_max^2 = (1 - cos) / 2
            const Real phi = rng_azimuth<Real>(rng);
            peturb(ph.dx, ph.dy, ph.dz, cosA, phi, norm);
            return true;
        }
    }

    // ---- Compton, impulse approximation (transport.hpp:342-483) -----------------
    template <class Real>
    __device__ __forceinline__ bool compton_ia(const float* L, const LutMeta& m, PhotonT<Real>& ph, int material, Rng& rng, Real& deposit, bool norm = false)
    {
        const float* shells = L + m.off_shells + material * N_SHELLS * SHELL_FLOATS;
        Real total = Real(0.0);
#pragma unroll
        for (int s = 0; s < N_SHELLS; ++s)
            total += (shells[s * SHELL_FLOATS] < ph.energy && shells[s * SHELL_FLOATS + 2] > Real(0.0)) ? shells[s * SHELL_FLOATS + 1] : Real(0.0);
        const Real sample = total * static_cast<Real>(rng.uniform());
        Real cum = Real(0.0);
        int shell = 0;
        for (int s = 0; s < N_SHELLS; ++s) {
            cum += (shells[s * SHELL_FLOATS] < ph.energy && shells[s * SHELL_FLOATS + 2] > Real(0.0)) ? shells[s * SHELL_FLOATS + 1] : Real(0.0);
            shell = s;
            if (!(cum < sample) || s == N_SHELLS - 1)
                break;
        }
        if (!(total > Real(0.0))) {
            deposit = Real(0.0); // no shell can take part: the interaction is rejected
            return true;
        }
        const float* sh = shells + shell * SHELL_FLOATS;
        const Real U = sh[0] / Real(ELECTRON_REST_MASS_D);
        const Real pU = m_sqrt(Real(2.0) * U + U * U);
        const Real J0 = sh[2];
        const Real k = ph.energy / Real(ELECTRON_REST_MASS_D);
        if (U > k) {
            deposit = Real(0.0); // interaction rejected (corrects the cross section)
            return true;
        }
        const Real emin = Real(1.0) / (Real(1.0) + Real(2.0) * k);
        const Real gmax_inv = Real(1.0) / (Real(1.0) / emin + emin);
        constexpr Real sp2 = Real(2.50662827463100); // 1 / (1/sqrt(pi) / sqrt(2)) = sqrt(2 pi)
        constexpr Real a1 = Real(0.34802), a2 = -Real(0.0958798), a3 = Real(0.7478556);
        const Real sqrte = Real(1.64872127070013);
        Real e = Real(1.0), cosA = Real(1.0);
        bool accepted = false;
        for (int it = 0; it < REJECTION_CAP && !accepted; ++it) {
            const Real r1 = static_cast<Real>(rng.uniform());
            // e = r1 + (1 - r1) emin, with 1 - e = (1 - r1)(1 - emin) formed directly so
            // that t stays positive when e rounds to 1 in single precision
            const Real one_minus_e = (Real(1.0) - r1) * (Real(1.0) - emin);
            e = Real(1.0) - one_minus_e;
            const Real t = one_minus_e / (k * e);
            const Real sin2 = t * (Real(2.0) - t);
            cosA = Real(1.0) - t;
            const Real g = (Real(1.0) / e + e - sin2) * gmax_inv;
            const Real r2 = static_cast<Real>(rng.uniform());
            if (r2 > g)
                continue;
            const Real pi = (k * (k - U) * t - U) / m_sqrt(m_max(Real(2.0) * k * (k - U) * t + U * U, Real(1e-30)));
            const Real kc = k * e;
            const Real qc = m_sqrt(m_max(k * k + kc * kc - Real(2.0) * k * kc * cosA, Real(1e-30)));
            const Real alpha = qc * (Real(1.0) + kc * (kc - k * cosA) / (qc * qc)) / k;
            const Real b_part = Real(1.0) + Real(2.0) * J0 * m_abs(pi);
            const Real b = (b_part * b_part + Real(1.0)) * Real(0.5);
            const Real expb = m_exp(-b);
            Real S;
            if (pi <= -pU) {
                S = (Real(1.0) - alpha * pU) * expb * Real(0.5);
            } else if (pi < pU) {
                const Real part1 = alpha * sp2 / (Real(4.0) * J0);
                const Real tp = Real(1.0) / (Real(1.0) + Real(0.332673) * (Real(1.0) + Real(2.0) * J0 * m_abs(pU)));
                const Real tpi = Real(1.0) / (Real(1.0) + Real(0.332673) * (Real(1.0) + Real(2.0) * J0 * m_abs(pi)));
                const Real part2p = sqrte - expb * tp * (a1 + a2 * tp + a3 * tp * tp);
                const Real part2pi = sqrte - expb * tpi * (a1 + a2 * tpi + a3 * tpi * tpi);
                if (pi <= Real(0.0))
                    S = (Real(1.0) - alpha * pi) * expb * Real(0.5) - part1 * (part2p - part2pi);
                else
                    S = Real(1.0) - (Real(1.0) - alpha * pi) * expb * Real(0.5) - part1 * (part2p - part2pi);
            } else {
                S = Real(1.0) - (Real(1.0) - alpha * pU) * expb * Real(0.5);
            }
            const Real r3 = static_cast<Real>(rng.uniform());
            if (r3 > S)
                continue;
            Real Fmax;
            if (pi <= -pU)
                Fmax = Real(1.0) - alpha * pU;
            else if (pi >= pU)
                Fmax = Real(1.0) + alpha * pU;
            else
                Fmax = Real(1.0) + alpha * pi;
            const Real r4 = static_cast<Real>(rng.uniform_open()); // log(rbar2) below needs rbar2 > 0
            const Real rbar2 = Real(2.0) * r4 * expb;
            Real pz;
            if (rbar2 < Real(1.0)) {
                const Real part = m_sqrt(Real(1.0) - Real(2.0) * m_log(rbar2));
                pz = (Real(1.0) - part) / (Real(2.0) * J0) / Real(ELECTRON_REST_MASS_D);
            } else {
                const Real part = m_sqrt(Real(1.0) - Real(2.0) * m_log(Real(2.0) - rbar2));
                pz = (part - Real(1.0)) / (Real(2.0) * J0) / Real(ELECTRON_REST_MASS_D);
            }
            Real Fpz;
            if (pz <= -pU)
                Fpz = Real(1.0) - alpha * pU;
            else if (pz >= pU)
                Fpz = Real(1.0) + alpha * pU;
            else
                Fpz = Real(1.0) + alpha * pz;
            const Real r5 = static_cast<Real>(rng.uniform());
            if (r5 > Fpz / Fmax)
                continue;
            const Real part = m_sqrt(m_max(Real(1.0) - Real(2.0) * e * cosA + e * e * (Real(1.0) - pz * pz * sin2), Real(0.0)));
            const Real kbar = kc / (Real(1.0) - pz * pz * e * e) * (Real(1.0) - pz * pz * e * cosA + pz * part);
            e = kbar / k;
            accepted = true;
        }
        if (!accepted)
            return false;
        const Real phi = rng_azimuth<Real>(rng);
        peturb(ph.dx, ph.dy, ph.dz, cosA, phi, norm);
        const Real E = ph.energy;
        ph.energy *= e;
        deposit = E - ph.energy;
        return true;
    }

    // ---- Compton, Klein-Nishina with optional scatter factor (transport.hpp:300-340)
    template <int MODEL, class Real>
    __device__ __forceinline__ bool compton_scatter(const float* L, const float* G, const LutMeta& m, PhotonT<Real>& ph, int material, Rng& rng, Real& deposit, bool norm = false)
    {
        if constexpr (MODEL == 2) {
            return compton_ia(L, m, ph, material, rng, deposit, norm);
        } else {
            // the density of the reference's Klein-Nishina rejection (times the scatter
            // factor S(q) for LIVERMORE), drawn by inverse CDF: no loop, no divergence
            const Real E = ph.energy;
            const Real k = E / Real(ELECTRON_REST_MASS_D);
            const Real emin = Real(1.0) / (Real(1.0) + Real(2.0) * k);
            Real fe;
            const int row = table_row(m, E, fe);
            const float* tab = MODEL == 1 ? G + m.off_csf + (material * m.tab_ne + row) * (m.tab_nu + 1)
                                          : G + m.off_ckn + row * (m.tab_nu + 1);
            const Real x = table_quantile(tab, m.tab_nu, static_cast<Real>(rng.uniform()), fe); // (e - e_min) / (1 - e_min)
            const Real one_minus_e = (Real(1.0) - x) * (Real(1.0) - emin);
            const Real e = Real(1.0) - one_minus_e;
            const Real cosA = Real(1.0) - one_minus_e / (k * e);
            const Real phi = rng_azimuth<Real>(rng);
            peturb(ph.dx, ph.dy, ph.dz, m_max(cosA, -Real(1.0)), phi, norm);
            ph.energy = E * e;
            deposit = E - ph.energy;
            return true;
        }
    }

    // ---- photon generation: Exposure::sampleParticle (exposure.hpp:280-304) -----
    template <class Real>
    __device__ __forceinline__ void sample_particle(const SourceParams& s, const DevExposure& ex, Rng& rng, PhotonT<Real>& ph)
    {
        const Real theta = ex.coll[0] + static_cast<Real>(rng.uniform()) * (ex.coll[1] - ex.coll[0]);
        const Real phi = ex.coll[2] + static_cast<Real>(rng.uniform()) * (ex.coll[3] - ex.coll[2]);
        ph.px = ex.pos[0];
        ph.py = ex.pos[1];
        ph.pz = ex.pos[2];
        ph.dx = ex.beam[0];
        ph.dy = ex.beam[1];
        ph.dz = ex.beam[2];
        ph.weight = ex.weight;
        rotate(ph.dx, ph.dy, ph.dz, Real(ex.cosy[0]), Real(ex.cosy[1]), Real(ex.cosy[2]), theta);
        rotate(ph.dx, ph.dy, ph.dz, Real(ex.cosx[0]), Real(ex.cosx[1]), Real(ex.cosx[2]), phi);
        if (s.spec_n > 0) {
            // SpecterDistribution::sampleValue (dxmcrandom.hpp:322-326)
            const Real r = static_cast<Real>(rng.uniform());
            const uint32_t k = rng.below(static_cast<uint32_t>(s.spec_n));
            const uint32_t idx = r < __ldg(s.spec_prob + k) ? k : __ldg(s.spec_alias + k);
            if (idx + 1 < static_cast<uint32_t>(s.spec_n)) {
                const Real e0 = __ldg(s.spec_energy + idx), e1 = __ldg(s.spec_energy + idx + 1);
                ph.energy = e0 + static_cast<Real>(rng.uniform()) * (e1 - e0);
            } else {
                ph.energy = __ldg(s.spec_energy + idx);
            }
        } else {
            ph.energy = ex.mono_energy;
        }
        if (s.bowtie_angle) {
            // BowTieFilter::sampleIntensityWeight (beamfilters.hpp:150-190)
            const Real angle = m_abs(theta);
            int first = 0, last = s.bowtie_n - 1;
            int it = first + (last - first) / 2;
            while (it != first) {
                if (angle < __ldg(s.bowtie_angle + it)) {
                    last = it;
                    it = first;
                } else {
                    first = it;
                }
                it += (last - first) / 2;
            }
            Real w;
            if (angle < __ldg(s.bowtie_angle + first))
                w = __ldg(s.bowtie_weight);
            else if (angle > __ldg(s.bowtie_angle + last))
                w = __ldg(s.bowtie_weight + s.bowtie_n - 1);
            else {
                const Real x0 = __ldg(s.bowtie_angle + first), x1 = __ldg(s.bowtie_angle + last);
                const Real y0 = __ldg(s.bowtie_weight + first), y1 = __ldg(s.bowtie_weight + last);
                w = y0 + (angle - x0) * (y1 - y0) / (x1 - x0);
            }
            ph.weight *= w;
        }
        if (s.heel_weights) {
            // HeelFilter::sampleIntensityWeight (beamfilters.hpp:514-538)
            const Real energy = ph.energy;
            int e_index = static_cast<int>((energy - s.heel_e_start + Real(0.5) * s.heel_e_step) / s.heel_e_step);
            if (e_index >= s.heel_e_size || e_index < 0)
                e_index = e_index < 0 ? 0 : s.heel_e_size - 1;
            if (energy < s.heel_e_start)
                e_index = 0;
            int a_index = static_cast<int>((phi - s.heel_a_start) / s.heel_a_step);
            if (a_index >= s.heel_a_size || a_index < 0)
                a_index = a_index < 0 ? 0 : s.heel_a_size - 1;
            if (phi < s.heel_a_start)
                a_index = 0;
            const int w_index = e_index * s.heel_a_size + a_index;
            Real w;
            if (a_index < s.heel_a_size - 1) {
                const Real a0 = s.heel_a_start + s.heel_a_step * a_index;
                const Real a1 = s.heel_a_start + s.heel_a_step * (a_index + 1);
                const Real w0 = __ldg(s.heel_weights + w_index), w1 = __ldg(s.heel_weights + w_index + 1);
                w = w0 + (w1 - w0) * (phi - a0) / (a1 - a0);
            } else {
                w = __ldg(s.heel_weights + w_index);
            }
            ph.weight *= w;
        }
    }

    template <class Real>
    __device__ __forceinline__ bool inside(const WorldParams& w, Real x, Real y, Real z)
    {
        return (x > w.lo[0] && x < w.hi[0]) && (y > w.lo[1] && y < w.hi[1]) && (z > w.lo[2] && z < w.hi[2]);
    }

    // transportParticleToWorld (transport.hpp:702-728)
    template <class Real>
    __device__ __forceinline__ bool transport_to_world(const WorldParams& w, PhotonT<Real>& ph)
    {
        if (inside(w, ph.px, ph.py, ph.pz))
            return true;
        Real amin = -Real(3.402823466e38), amax = Real(3.402823466e38);
        const Real pos[3] = { ph.px, ph.py, ph.pz };
        const Real dir[3] = { ph.dx, ph.dy, ph.dz };
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            if (m_abs(dir[i]) > Real(N_ERROR_D)) {
                const Real inv = Real(1.0) / dir[i];
                const Real a0 = (w.lo[i] - pos[i]) * inv;
                const Real an = (w.hi[i] - pos[i]) * inv;
                amin = m_max(amin, m_min(a0, an));
                amax = m_min(amax, m_max(a0, an));
            }
        }
        if (amin < amax && amin > Real(0.0)) {
            ph.px += amin * ph.dx;
            ph.py += amin * ph.dy;
            ph.pz += amin * ph.dz;
            return true;
        }
        return false;
    }

    __device__ __forceinline__ uint32_t find_exposure(const SourceParams& s, uint64_t h)
    {
        // last exposure whose offset <= h
        uint32_t lo = 0, hi = s.n_exposures;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (__ldg(s.history_offsets + mid) <= h)
                lo = mid;
            else
                hi = mid;
        }
        return lo;
    }

    __device__ __forceinline__ void load_exposure(const DevExposure* ptr, DevExposure& ex)
    {
        const float4* src = reinterpret_cast<const float4*>(ptr);
        float4* dst = reinterpret_cast<float4*>(&ex);
#pragma unroll
        for (int i = 0; i < 5; ++i)
            dst[i] = __ldg(src + i);
    }

    // ---- the transport kernel ----------------------------------------------------
    //
    // Warp-synchronous loop.  Each iteration every lane with a live photon and no
    // pending interaction takes up to woodcock_burst Woodcock steps; a real event
    // only records its type (photoelectric / Compton / Rayleigh) and ends the lane's
    // burst.  The interactions are then run in
    // one converged pass per type once enough lanes wait, and finished lanes are
    // refilled together once enough are idle, so the expensive branches run with
    // many lanes active instead of one or two.
    enum : int { EV_NONE = 0, EV_PHOTO = 1, EV_COMPTON = 2, EV_RAYLEIGH = 3 };

    // A voxel as read from the grid: its palette index (compact layout) or its
    // 8-byte record; decode_voxel turns it into density, material and the
    // measurement flag.
    template <bool PALETTE>
    struct VoxelRaw {
        uint2 v;
    };
    template <>
    struct VoxelRaw<true> {
        uint32_t index;
    };

    template <bool PALETTE>
    __device__ __forceinline__ VoxelRaw<PALETTE> load_voxel(const WorldParams& w, uint64_t vidx)
    {
        if constexpr (PALETTE)
            return VoxelRaw<true> { __ldg(w.palette_index + vidx) };
        else
            return VoxelRaw<false> { __ldg(reinterpret_cast<const uint2*>(w.voxels) + vidx) };
    }

    template <bool PALETTE, class Real>
    __device__ __forceinline__ void decode_voxel(const VoxelRaw<PALETTE>& raw, const PaletteEntry* pal, Real& density, int& mat, bool& measured)
    {
        if constexpr (PALETTE) {
            const PaletteEntry e = pal[raw.index];
            density = e.density;
            mat = static_cast<int>(e.code & 0xffu);
            measured = (e.code >> 8) != 0u;
        } else {
            density = __uint_as_float(raw.v.x);
            mat = static_cast<int>(raw.v.y & 0xffu);
            measured = ((raw.v.y >> 8) & 0xffu) != 0u;
        }
    }

#ifndef DXMC_RAYLEIGH_THRESHOLD
#define DXMC_RAYLEIGH_THRESHOLD 2 // lanes waiting for a Rayleigh event before its pass runs alone
#endif
    constexpr int RAYLEIGH_THRESHOLD = DXMC_RAYLEIGH_THRESHOLD;

#ifndef DXMC_MIN_BLOCKS_PER_SM
#define DXMC_MIN_BLOCKS_PER_SM 4 // resident 256-thread blocks per SM the register budget must allow (64 registers)
#endif

    // State of one lane: its photon, random stream, cached lookups and counters.
    // Per-warp counters of a job in shared memory (lane 0 adds warp totals; rare
    // events use shared atomics), flushed to the job's counters: they cost the
    // lanes no registers.
    struct WarpTally {
        unsigned long long steps, deposits, overflows, histories;
    };

    template <class Real>
    struct LaneT {
        PhotonT<Real> ph;
        Rng rng;
        bool alive;
        int pending;
        Real stepK, logE; // Woodcock step = -log2(u) * stepK (mm): 10 * ln 2 / majorant
        int seg;
        bool updateMax;
        int cached_mat;
        uint32_t hist_steps;
        Real probInv;  // attenuation of the current material / majorant (event probability per unit density)
        Real p0, p01;  // photoelectric and photoelectric + Compton shares of the attenuation
        uint64_t vidx;
        Real forced_wc; // weight correction waiting for a forced-voxel interaction pass
        bool armed;      // energy x weight is below the Russian-roulette threshold
        Real cinv, cR;  // local majorant: 1 / scale and the flight length it holds for (MajorantGrid)
        int band;        // energy band of the local-majorant grid

        __device__ void start_photon()
        {
            pending = EV_NONE;
            updateMax = true;
            cached_mat = -1;
            hist_steps = 0;
            forced_wc = Real(0.0);
            cinv = Real(1.0); // the first flight from the grid boundary uses the global majorant
            cR = INFINITY;
            arm();
        }
        // energy and weight change only at interactions and roulette: the roulette
        // test of a virtual step reads this flag
        __device__ void arm() { armed = ph.energy * ph.weight < Real(ROULETTE_THRESHOLD_D); }
    };

    // Local majorant of the photon's cell for its energy band, after the energy
    // changed (a new photon, or an interaction): the flight drawn next must be
    // bounded for the new energy.  A new photon sits on the grid boundary, so the
    // coordinates are clamped onto the grid.
    template <class Real>
    __device__ __forceinline__ void fetch_cell(LaneT<Real>& s, const TransportParams& p)
    {
        const MajorantGrid& g = p.majorant;
        const WorldParams& w = p.world;
        // s.logE = log10 E was just computed; the band intervals of the bounds are
        // widened by 0.1 % on the host, which covers the rounding here
        s.band = min(max(m_floor_int((s.logE - g.band_log0) * g.band_inv_dlog), 0), g.bands - 1);
        const Real fx = m_min(m_max(m_fma(s.ph.px, w.inv_spacing[0], -w.lo_inv[0]), Real(0.0)), w.dims_f[0] - Real(1.0));
        const Real fy = m_min(m_max(m_fma(s.ph.py, w.inv_spacing[1], -w.lo_inv[1]), Real(0.0)), w.dims_f[1] - Real(1.0));
        const Real fz = m_min(m_max(m_fma(s.ph.pz, w.inv_spacing[2], -w.lo_inv[2]), Real(0.0)), w.dims_f[2] - Real(1.0));
        const uint32_t ix = static_cast<uint32_t>(fx), iy = static_cast<uint32_t>(fy), iz = static_cast<uint32_t>(fz);
        const uint32_t c = (iz >> g.shift[2]) * g.nxy + (iy >> g.shift[1]) * g.nx + (ix >> g.shift[0]);
        const float2 cell = __ldg(g.cells + (c * g.bands + s.band));
        s.cinv = cell.x;
        s.cR = cell.y;
    }

    // Safe flight length in a cell outside the box of the denser cells (the cell
    // holds -R): the ball of radius R, or the ray up to where it enters the box
    // (slab test in flight-parameter units, as the position update), whichever
    // reaches further.  A ray that misses the box may fly to the grid boundary.
    template <class Real>
    __device__ __forceinline__ Real reach_to_box(const PhotonT<Real>& ph, const MajorantGrid& g, Real R)
    {
        const Real p[3] = { ph.px, ph.py, ph.pz };
        const Real d[3] = { ph.dx, ph.dy, ph.dz };
        Real tmin = Real(0.0), tmax = INFINITY;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const Real inv = Real(1.0) / d[a];
            const Real t0 = (__ldg(g.box + a) - p[a]) * inv;
            const Real t1 = (__ldg(g.box + 3 + a) - p[a]) * inv;
            tmin = m_max(tmin, m_min(t0, t1));
            tmax = m_min(tmax, m_max(t0, t1));
        }
        return m_max(R, tmin <= tmax ? tmin : INFINITY);
    }

    // Loads photon + stream state from the pre-generated queue.
    template <class Real>
    __device__ __forceinline__ void take_queued(LaneT<Real>& s, const PhotonQueue& q, uint64_t i)
    {
        const float4 pe = __ldg(q.pos_energy + i);
        const float4 dw = __ldg(q.dir_weight + i);
        const uint4 rs = __ldg(q.rng + i);
        s.ph = PhotonT<Real> { pe.x, pe.y, pe.z, dw.x, dw.y, dw.z, pe.w, dw.w };
        s.rng.s0 = rs.x;
        s.rng.s1 = rs.y;
        s.rng.s2 = rs.z;
        s.rng.s3 = rs.w;
        s.alive = true;
        s.start_photon();
    }

    // Samples history h of the job in place (Exposure::sampleParticle + transportParticleToWorld).
    template <class Real>
    __device__ __forceinline__ void take_history(LaneT<Real>& s, const TransportParams& p, uint64_t h)
    {
        s.rng.init(p.seed, h);
        uint32_t ei;
        if (p.uniform_hpe && p.total_histories <= 0xffffffffull)
            ei = udiv_apply(static_cast<uint32_t>(h), p.hpe_magic, p.hpe_shifts);
        else
            ei = p.uniform_hpe ? static_cast<uint32_t>(h / p.uniform_hpe) : find_exposure(p.source, h);
        DevExposure ex;
        load_exposure(p.source.exposures + ei, ex);
        sample_particle(p.source, ex, s.rng, s.ph);
        s.alive = transport_to_world(p.world, s.ph);
        s.start_photon();
    }

    // One iteration of the warp-synchronous loop for every lane of the warp: a
    // Woodcock step for lanes without a pending interaction (transport.hpp:650-699),
    // the per-type interaction passes once enough lanes wait (transport.hpp:523-638),
    // Russian roulette and scoring.  Must be called by all 32 lanes.  LEAN (the
    // persistent multi-job kernel, which holds more state per lane) keeps the voxel
    // read after the truncation test and one interaction pass per event type: the
    // overlapped reads and the merged pass cost that kernel more spills than they save.
    template <int MODEL, bool PALETTE, bool LEAN = false, class Real>
    __device__ __forceinline__ void advance(LaneT<Real>& s, WarpTally& wt, const TransportParams& p, const float* L, const PaletteEntry* pal,
        bool drain, int interact_t)
    {
        const LutMeta& m = p.lut_meta;
        const WorldParams& w = p.world;
        bool do_score = false;
        Real deposit = Real(0.0); // energy imparted x weight to score
        bool check_roulette = false;

        if (s.alive && s.pending == EV_NONE) {
            if (s.updateMax) {
                s.logE = m_log10(s.ph.energy);
                s.seg = lut_segment(L, m, s.logE);
                s.stepK = lut_max_inverse(L, m, s.logE, s.seg) * (Real(10.0) * Real(0.693147180559945)); // cm -> mm, log2 -> ln
                s.updateMax = false;
                s.cached_mat = -1;
                if (p.majorant.cells)
                    fetch_cell(s, p);
            }
            // Up to p.woodcock_burst Woodcock steps per iteration: a lane keeps stepping
            // through virtual collisions and stops at a real event, the grid boundary or a
            // forced-scoring voxel.  Each lane draws its own stream in the reference's
            // order, so the burst length changes the schedule, not the histories.
            const int burst = max(p.woodcock_burst, 1); // at least one step: every iteration makes progress
            if (s.hist_steps > MAX_STEPS_PER_HISTORY) {
                // bounded work per history (checked per burst: at most burst - 1 steps over)
                atomicAdd(&wt.overflows, 1ull);
                s.alive = false;
            }
            for (int k = 0; k < burst && s.alive; ++k) {
                // a flight drawn with the local majorant ends without a collision test
                // where that majorant stops holding (truncated: drawn again from there)
                Real R = s.cR;
                if (R < Real(0.0))
                    R = reach_to_box(s.ph, p.majorant, -R);
                const Real flight = -m_log2(static_cast<Real>(s.rng.uniform_open())) * (s.stepK * s.cinv);
                const bool truncated = flight > R;
                const Real step = m_min(flight, R);
                s.ph.px = m_fma(s.ph.dx, step, s.ph.px);
                s.ph.py = m_fma(s.ph.dy, step, s.ph.py);
                s.ph.pz = m_fma(s.ph.dz, step, s.ph.pz);
                // grid coordinates (p - lo) / spacing as one FMA each, rounded down; the photon
                // is inside while all three lie in [0, dims) (one unsigned compare each: a
                // negative or saturated conversion falls outside), which bounds the voxel index
                const int jx = m_floor_int(m_fma(s.ph.px, w.inv_spacing[0], -w.lo_inv[0]));
                const int jy = m_floor_int(m_fma(s.ph.py, w.inv_spacing[1], -w.lo_inv[1]));
                const int jz = m_floor_int(m_fma(s.ph.pz, w.inv_spacing[2], -w.lo_inv[2]));
                if (!(static_cast<uint32_t>(jx) < w.dims[0] && static_cast<uint32_t>(jy) < w.dims[1]
                        && static_cast<uint32_t>(jz) < w.dims[2])) {
                    s.alive = false;
                    break;
                }
                ++s.hist_steps;
                const uint32_t ix = static_cast<uint32_t>(jx);
                const uint32_t iy = static_cast<uint32_t>(jy);
                const uint32_t iz = static_cast<uint32_t>(jz);
                const Real cinv = s.cinv; // the majorant this flight was drawn with
                // the voxel is read before the majorant cell, so that the two L2 reads
                // overlap (a truncated flight does not use the voxel)
                VoxelRaw<PALETTE> raw {};
                if constexpr (!LEAN) {
                    if constexpr (PALETTE) // compact worlds have fewer than 2^32 voxels (world upload)
                        s.vidx = iz * static_cast<uint32_t>(w.nxy) + (iy * w.dims[0] + ix);
                    else
                        s.vidx = static_cast<uint64_t>(iz) * w.nxy + static_cast<uint64_t>(iy) * w.dims[0] + ix;
                    raw = load_voxel<PALETTE>(w, s.vidx);
                }
                if (p.majorant.cells) {
                    const MajorantGrid& g = p.majorant;
                    const uint32_t c = (iz >> g.shift[2]) * g.nxy + (iy >> g.shift[1]) * g.nx + (ix >> g.shift[0]);
                    const float2 cell = __ldg(g.cells + (c * g.bands + s.band));
                    s.cinv = cell.x;
                    s.cR = cell.y;
                }
                if (truncated)
                    continue;
                if constexpr (LEAN) {
                    if constexpr (PALETTE)
                        s.vidx = iz * static_cast<uint32_t>(w.nxy) + (iy * w.dims[0] + ix);
                    else
                        s.vidx = static_cast<uint64_t>(iz) * w.nxy + static_cast<uint64_t>(iy) * w.dims[0] + ix;
                    raw = load_voxel<PALETTE>(w, s.vidx);
                }
                Real density;
                int mat;
                bool measured;
                decode_voxel<PALETTE>(raw, pal, density, mat, measured);
                if (mat != s.cached_mat) {
                    Real a0, a1, a2;
                    lut_attenuation(L, m, mat, s.logE, s.seg, a0, a1, a2);
                    const Real attTot = a0 + a1 + a2;
                    const Real inv = Real(1.0) / attTot;
                    s.probInv = attTot * s.stepK * (Real(1.0) / (Real(10.0) * Real(0.693147180559945)));
                    s.p0 = a0 * inv;
                    s.p01 = (a0 + a1) * inv;
                    s.cached_mat = mat;
                }
                const Real eventProb = s.probInv * density * cinv;
                if (!measured) {
                    // naive sampling (computeInteractions): decide the event type now,
                    // run it in the interaction pass
                    if (static_cast<Real>(s.rng.uniform()) < eventProb) {
                        const Real r3 = static_cast<Real>(s.rng.uniform());
                        s.pending = r3 < s.p0 ? EV_PHOTO : (r3 < s.p01 ? EV_COMPTON : EV_RAYLEIGH);
                        break;
                    }
                    // virtual collision: Russian roulette (transport.hpp:684-694)
                    if (s.armed) {
                        if (static_cast<Real>(s.rng.uniform()) < Real(ROULETTE_PROBABILITY_D)) {
                            s.alive = false;
                            break;
                        }
                        s.ph.weight *= Real(1.0) / (Real(1.0) - Real(ROULETTE_PROBABILITY_D));
                        s.arm();
                    }
                } else {
                    // forced photoelectric scoring (computeInteractionsForced): score the forced
                    // photoelectric share now; a real Compton or Rayleigh event goes through the
                    // interaction passes and the weight correction (1 - wc) is applied after it
                    const Real photoProb = s.p0;
                    s.forced_wc = eventProb * photoProb;
                    {
                        PhotonT<Real> forced = s.ph;
                        const Real ef = photo_absorption<MODEL>(L, m, forced, mat, s.rng, p.normalize_direction);
                        deposit = (forced.energy < Real(ENERGY_CUTOFF_D) ? (ef + forced.energy) : ef) * forced.weight * s.forced_wc;
                        do_score = true;
                    }
                    if (static_cast<Real>(s.rng.uniform()) < eventProb * (Real(1.0) - photoProb)) {
                        s.pending = static_cast<Real>(s.rng.uniform()) * (Real(1.0) - s.p0) < s.p01 - s.p0 ? EV_COMPTON : EV_RAYLEIGH;
                    } else {
                        s.ph.weight *= (Real(1.0) - s.forced_wc);
                        s.forced_wc = Real(0.0);
                        check_roulette = true;
                    }
                    break; // the forced deposit is scored before the next step
                }
            }
        }
        if (do_score) {
            // the forced photoelectric deposit is scored before this lane's
            // interaction pass can add a second deposit in the same iteration
            if (isfinite(deposit)) {
                score(p, s.vidx, deposit);
                atomicAdd(&wt.deposits, 1ull);
            } else {
                atomicAdd(&wt.overflows, 1ull);
                s.alive = false;
                s.pending = EV_NONE;
            }
            do_score = false;
        }

        // ---- interaction passes, one converged pass per event type ---------------------
        if constexpr (MODEL == 1 && !LEAN) {
            // LIVERMORE: Compton and Rayleigh both draw one quantile from an energy-row
            // table and rotate the direction, and photoabsorption only ends the photon,
            // so every waiting lane runs in one pass (Rayleigh lanes ride along instead
            // of waiting for a pass of their own).  Each lane draws from its stream in
            // the order of compton_scatter<1> / rayleigh_scatter<1>.
            const unsigned waiting = __ballot_sync(FULL_MASK, s.pending != EV_NONE);
            const unsigned can_step = __ballot_sync(FULL_MASK, s.alive && s.pending == EV_NONE);
            if (waiting && (__popc(waiting) >= interact_t || can_step == 0u || drain) && s.pending != EV_NONE) {
                const Real E = s.ph.energy;
                if (s.pending == EV_PHOTO) {
                    // photo_absorption<1>: the photon ends and deposits its energy
                    deposit = E * s.ph.weight;
                    s.ph.energy = Real(0.0);
                    s.alive = false;
                } else {
                    const bool compton = s.pending == EV_COMPTON;
                    Real fe;
                    const int row = table_row(m, E, fe);
                    const float* tab = p.lut + (compton ? m.off_csf : m.off_ray) + (s.cached_mat * m.tab_ne + row) * (m.tab_nu + 1);
                    const Real x = table_quantile(tab, m.tab_nu, static_cast<Real>(s.rng.uniform()), fe);
                    Real cosA, e = Real(1.0);
                    if (compton) {
                        // (e - e_min) / (1 - e_min) = x
                        const Real k = E / Real(ELECTRON_REST_MASS_D);
                        const Real emin = Real(1.0) / (Real(1.0) + Real(2.0) * k);
                        const Real one_minus_e = (Real(1.0) - x) * (Real(1.0) - emin);
                        e = Real(1.0) - one_minus_e;
                        cosA = m_max(Real(1.0) - one_minus_e / (k * e), -Real(1.0));
                    } else {
                        cosA = Real(1.0) - Real(2.0) * x; // q^2 / q_max^2 = (1 - cos) / 2
                    }
                    const Real phi = rng_azimuth<Real>(s.rng);
                    peturb(s.ph.dx, s.ph.dy, s.ph.dz, cosA, phi, p.normalize_direction);
                    if (compton) {
                        s.ph.energy = E * e;
                        if (s.ph.energy < Real(ENERGY_CUTOFF_D)) {
                            deposit = ((E - s.ph.energy) + s.ph.energy) * s.ph.weight;
                            s.ph.energy = Real(0.0);
                            s.alive = false;
                        } else {
                            deposit = (E - s.ph.energy) * s.ph.weight;
                            s.updateMax = true;
                        }
                    }
                }
                do_score = s.pending != EV_RAYLEIGH;
                if (s.alive && s.forced_wc != Real(0.0))
                    s.ph.weight *= (Real(1.0) - s.forced_wc);
                s.forced_wc = Real(0.0);
                check_roulette = s.alive;
                s.pending = EV_NONE;
            }
        } else {
            // Rayleigh events are rare (about one in ten interactions here), so their pass
            // waits until RAYLEIGH_THRESHOLD lanes have one, or until nothing else can run
            const unsigned ray = __ballot_sync(FULL_MASK, s.pending == EV_RAYLEIGH);
            const unsigned waiting = __ballot_sync(FULL_MASK, s.pending != EV_NONE);
            const unsigned can_step = __ballot_sync(FULL_MASK, s.alive && s.pending == EV_NONE);
            const unsigned waiting_other = waiting & ~ray;
            const bool stuck = can_step == 0u || drain;
            const bool run_ray = ray && (__popc(ray) >= RAYLEIGH_THRESHOLD || stuck);
            if ((waiting_other && (__popc(waiting_other) >= interact_t || stuck)) || run_ray) {
                const int mat = s.cached_mat;
                if (__any_sync(FULL_MASK, s.pending == EV_PHOTO) && s.pending == EV_PHOTO) {
                    const Real e = photo_absorption<MODEL>(L, m, s.ph, mat, s.rng, p.normalize_direction);
                    do_score = true;
                    if (s.ph.energy < Real(ENERGY_CUTOFF_D)) {
                        deposit = (e + s.ph.energy) * s.ph.weight;
                        s.ph.energy = Real(0.0);
                        s.alive = false;
                    } else {
                        deposit = e * s.ph.weight;
                        s.updateMax = true;
                    }
                }
                if (__any_sync(FULL_MASK, s.pending == EV_COMPTON) && s.pending == EV_COMPTON) {
                    Real e = Real(0.0);
                    if (!compton_scatter<MODEL>(L, p.lut, m, s.ph, mat, s.rng, e, p.normalize_direction)) {
                        atomicAdd(&wt.overflows, 1ull);
                        s.alive = false;
                    } else {
                        do_score = true;
                        if (s.ph.energy < Real(ENERGY_CUTOFF_D)) {
                            deposit = (e + s.ph.energy) * s.ph.weight;
                            s.ph.energy = Real(0.0);
                            s.alive = false;
                        } else {
                            deposit = e * s.ph.weight;
                            s.updateMax = true;
                        }
                    }
                }
                if (run_ray && s.pending == EV_RAYLEIGH) {
                    if (!rayleigh_scatter<MODEL>(L, p.lut, m, s.ph, mat, s.rng, p.normalize_direction)) {
                        atomicAdd(&wt.overflows, 1ull);
                        s.alive = false;
                    }
                }
                if (s.pending != EV_NONE && (s.pending != EV_RAYLEIGH || run_ray)) {
                    if (s.alive && s.forced_wc != Real(0.0))
                        s.ph.weight *= (Real(1.0) - s.forced_wc);
                    s.forced_wc = Real(0.0);
                    check_roulette = s.alive;
                    s.pending = EV_NONE;
                }
            }
        }
        if (check_roulette) {
            // Russian roulette (transport.hpp:684-694) after an interaction or a forced step
            if (s.ph.energy * s.ph.weight < Real(ROULETTE_THRESHOLD_D)) {
                if (static_cast<Real>(s.rng.uniform()) < Real(ROULETTE_PROBABILITY_D))
                    s.alive = false;
                else
                    s.ph.weight *= Real(1.0) / (Real(1.0) - Real(ROULETTE_PROBABILITY_D));
            }
            s.arm();
        }
        if (do_score && !isfinite(deposit)) {
            // never let a non-finite value into the FP64 accumulators: end the
            // history and report it through the overflow counter
            do_score = false;
            s.alive = false;
            atomicAdd(&wt.overflows, 1ull);
        }
        // ---- scoring; the warp is converged here ----------------------------------------
        const unsigned scoring = __ballot_sync(FULL_MASK, do_score);
        if (p.tally_mode == 2) {
            if (do_score)
                score_aggregated(p, scoring, s.vidx, deposit);
        } else if (do_score) {
            score(p, s.vidx, deposit);
        }
        if ((threadIdx.x & 31) == 0)
            wt.deposits += __popc(scoring);
    }

    // Counts the steps of the photons a warp's lanes finished (before they are
    // refilled or at a flush).  Called by all 32 lanes.
    template <class Real>
    __device__ __forceinline__ void count_steps(LaneT<Real>& s, WarpTally& wt, bool finished)
    {
        const unsigned n = __reduce_add_sync(FULL_MASK, finished ? s.hist_steps : 0u);
        if ((threadIdx.x & 31) == 0)
            wt.steps += n;
        if (finished)
            s.hist_steps = 0;
    }

    // Adds the warp's counters to a job's counters and clears them.  Called by all 32 lanes.
    template <class Real>
    __device__ __forceinline__ void flush_counters(LaneT<Real>& s, WarpTally& wt, JobCounters* c)
    {
        count_steps(s, wt, true); // counted once: the photons' steps so far
        __syncwarp();
        if ((threadIdx.x & 31) == 0) {
            if (wt.steps)
                atomicAdd(&c->steps, wt.steps);
            if (wt.deposits)
                atomicAdd(&c->deposits, wt.deposits);
            if (wt.overflows)
                atomicAdd(&c->overflows, wt.overflows);
            if (wt.histories)
                atomicAdd(&c->histories_done, wt.histories);
            wt = WarpTally {};
        }
        __syncwarp();
    }

    // ---- single-job transport kernel ----------------------------------------------------
    //
    // Warp-synchronous loop.  Each iteration every lane with a live photon and no
    // pending interaction takes up to woodcock_burst Woodcock steps; a real event
    // only records its type (photoelectric / Compton / Rayleigh) and ends the lane's
    // burst.  The interactions are then run in
    // one converged pass per type once enough lanes wait, and finished lanes are
    // refilled together once enough are idle, so the expensive branches run with
    // many lanes active instead of one or two.
    // the FP64-everywhere instantiation needs about twice the registers: two blocks per SM
    template <class Real, int MODEL, bool PALETTE>
    __global__ void __launch_bounds__(256, sizeof(Real) == 4 ? DXMC_MIN_BLOCKS_PER_SM : 2) transport_kernel(const __grid_constant__ TransportParams p)
    {
        extern __shared__ float4 smem_f4[];
        const float* L = p.lut;
        size_t smem_off = 0;
        if (p.lut_in_smem) {
            float4* dst = smem_f4;
            const float4* src = reinterpret_cast<const float4*>(p.lut);
            const int n4 = (p.lut_meta.total_floats + 3) / 4;
            for (int i = threadIdx.x; i < n4; i += blockDim.x)
                dst[i] = __ldg(src + i);
            L = reinterpret_cast<const float*>(smem_f4);
            smem_off = static_cast<size_t>(n4);
        }
        const PaletteEntry* pal = nullptr;
        if constexpr (PALETTE) {
            PaletteEntry* spal = reinterpret_cast<PaletteEntry*>(smem_f4 + smem_off);
            for (int i = threadIdx.x; i < PALETTE_MAX; i += blockDim.x)
                spal[i] = i < p.world.palette_n ? p.world.palette[i] : PaletteEntry { Real(0.0), 0u };
            pal = spal;
        }
        __syncthreads();
        const int lane = threadIdx.x & 31;
        const unsigned lanemask_lt = (1u << lane) - 1u;
        const int regen_t = p.regen_threshold;
        const int interact_t = p.interact_threshold;
        const bool use_queue = p.queue.pos_energy != nullptr;
        const unsigned long long source_total = use_queue ? p.counters->queue_count : p.total_histories;
        unsigned long long* source_head = use_queue ? &p.counters->next_photon : &p.counters->next_history;

        __shared__ WarpTally tallies[1024 / 32];
        WarpTally& wt = tallies[threadIdx.x >> 5];
        if (lane == 0)
            wt = WarpTally {};
        __syncwarp();
        LaneT<Real> s {};
        s.alive = false;
        // warp-uniform pool of ids (queue slots or history ids) [pool_next, pool_end)
        uint64_t pool_next = 0, pool_end = 0;
        bool exhausted = false;

        while (true) {
            // ---- refill idle lanes together ------------------------------------------------
            unsigned need = __ballot_sync(FULL_MASK, !s.alive && !exhausted);
            const unsigned live = __ballot_sync(FULL_MASK, s.alive);
            if (need && (__popc(need) >= regen_t || live == 0u)) {
                while (need && !exhausted) {
                    if (pool_next >= pool_end) {
                        unsigned long long base = 0;
                        if (lane == 0) {
                            const bool cancelled = p.cancel && *p.cancel;
                            base = cancelled ? source_total : atomicAdd(source_head, (unsigned long long)WARP_POOL_CHUNK);
                        }
                        base = __shfl_sync(FULL_MASK, base, 0);
                        if (base >= source_total) {
                            exhausted = true;
                            break;
                        }
                        pool_next = base;
                        pool_end = min(static_cast<uint64_t>(base + WARP_POOL_CHUNK), static_cast<uint64_t>(source_total));
                    }
                    const uint64_t avail = pool_end - pool_next;
                    const unsigned rank = __popc(need & lanemask_lt);
                    const bool mine = ((need >> lane) & 1u) && rank < avail;
                    const unsigned taken = __ballot_sync(FULL_MASK, mine);
                    count_steps(s, wt, mine);
                    if (lane == 0 && !use_queue)
                        wt.histories += __popc(taken);
                    if (mine) {
                        if (use_queue) {
                            take_queued(s, p.queue, pool_next + rank);
                        } else
                            take_history(s, p, pool_next + rank);
                    }
                    pool_next += __popc(taken);
                    need &= ~taken;
                }
            }
            if (exhausted && __ballot_sync(FULL_MASK, s.alive) == 0u)
                break;
            advance<MODEL, PALETTE>(s, wt, p, L, pal, exhausted, interact_t);
        }
        flush_counters(s, wt, p.counters);
    }

    // ---- batched transport kernel ------------------------------------------------------
    //
    // Many jobs (worlds, LUTs, sources, tallies of their own) in one persistent launch.
    // Work items (job, first history, count) are taken from a device-side queue by whole
    // warps; a warp keeps its current job's parameters in shared memory and switches to
    // another job only once all its lanes have finished, so every lane of a warp always
    // works on the same job.  LUTs and palettes are read through the L1 (__ldg) since the
    // warps of one block may serve different jobs.  Each history keeps its own random
    // stream, so a job's tallies do not depend on what else runs in the batch.
    constexpr int BATCH_WARPS = 8; // 256-thread blocks

    template <int MODEL>
    __global__ void __launch_bounds__(256, DXMC_MIN_BLOCKS_PER_SM) batch_transport_kernel(const __grid_constant__ BatchParams b)
    {
        __shared__ TransportParams sjob[BATCH_WARPS];
        __shared__ PaletteEntry spal[BATCH_WARPS][PALETTE_MAX];
        const int lane = threadIdx.x & 31;
        const int warp = threadIdx.x >> 5;
        const unsigned lanemask_lt = (1u << lane) - 1u;
        TransportParams& p = sjob[warp];
        PaletteEntry* pal = spal[warp];
        BatchControl* ctl = b.control;
        const BatchItem* items = b.items + ctl->item_base[MODEL];
        const uint64_t n_items = ctl->n_items[MODEL];
        unsigned long long* next_item = &ctl->next_item[MODEL];
        const int regen_t = ctl->regen_threshold;
        const int interact_t = ctl->interact_threshold;

        __shared__ WarpTally tallies[BATCH_WARPS];
        WarpTally& wt = tallies[warp];
        if (lane == 0)
            wt = WarpTally {};
        __syncwarp();
        LaneT<float> s {};
        s.alive = false;
        int job = -1;
        uint64_t pool_next = 0, pool_end = 0;
        BatchItem next {};
        bool have_next = false;
        bool exhausted = false;

        while (true) {
            unsigned need = __ballot_sync(FULL_MASK, !s.alive && !exhausted);
            const unsigned live = __ballot_sync(FULL_MASK, s.alive);
            if (need && (__popc(need) >= regen_t || live == 0u)) {
                while (need && !exhausted) {
                    if (pool_next >= pool_end) {
                        if (!have_next) {
                            unsigned long long it = 0;
                            if (lane == 0)
                                it = atomicAdd(next_item, 1ull);
                            it = __shfl_sync(FULL_MASK, it, 0);
                            if (it >= n_items) {
                                exhausted = true;
                                break;
                            }
                            next = items[it];
                            have_next = true;
                        }
                        if (static_cast<int>(next.job) != job) {
                            // switch jobs only when every lane is idle
                            if (__ballot_sync(FULL_MASK, s.alive) != 0u)
                                break;
                            if (job >= 0)
                                flush_counters(s, wt, p.counters);
                            job = static_cast<int>(next.job);
                            __syncwarp();
                            const int* src = reinterpret_cast<const int*>(b.jobs + job);
                            int* dst = reinterpret_cast<int*>(&p);
                            for (int k = lane; k < static_cast<int>(sizeof(TransportParams) / sizeof(int)); k += 32)
                                dst[k] = __ldg(src + k);
                            __syncwarp();
                            const int np = p.world.palette_index ? p.world.palette_n : 0;
                            for (int k = lane; k < PALETTE_MAX; k += 32)
                                pal[k] = k < np ? p.world.palette[k] : PaletteEntry { 0.0f, 0u };
                            __syncwarp();
                        }
                        pool_next = next.first;
                        pool_end = next.first + next.count;
                        have_next = false;
                    }
                    const uint64_t avail = pool_end - pool_next;
                    const unsigned rank = __popc(need & lanemask_lt);
                    const bool mine = ((need >> lane) & 1u) && rank < avail;
                    const unsigned taken = __ballot_sync(FULL_MASK, mine);
                    count_steps(s, wt, mine);
                    if (lane == 0)
                        wt.histories += __popc(taken);
                    if (mine)
                        take_history(s, p, pool_next + rank);
                    pool_next += __popc(taken);
                    need &= ~taken;
                }
            }
            const unsigned live2 = __ballot_sync(FULL_MASK, s.alive);
            if (exhausted && live2 == 0u)
                break;
            if (live2 == 0u)
                continue; // waiting to switch jobs with nothing in flight: refill again
            if (p.world.palette_index)
                advance<MODEL, true, true>(s, wt, p, p.lut, pal, exhausted || have_next, interact_t);
            else
                advance<MODEL, false, true>(s, wt, p, p.lut, pal, exhausted || have_next, interact_t);
        }
        if (job >= 0)
            flush_counters(s, wt, p.counters);
    }

    // ---- photon generation pass ---------------------------------------------------------
    // One thread per history: Exposure::sampleParticle + transportParticleToWorld with
    // every lane of the warp busy; photons inside the world are appended to the queue
    // together with the state of their random stream.
    __global__ void __launch_bounds__(256) generate_kernel(const __grid_constant__ TransportParams p, uint64_t first, uint64_t count)
    {
        const int lane = threadIdx.x & 31;
        unsigned long long generated = 0;
        for (uint64_t base = blockIdx.x * static_cast<uint64_t>(blockDim.x); base < count; base += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
            const uint64_t i = base + threadIdx.x;
            bool inworld = false;
            PhotonT<float> ph {};
            Rng rng;
            if (i < count) {
                const uint64_t h = first + i;
                rng.init(p.seed, h);
                uint32_t ei;
                if (p.uniform_hpe && p.total_histories <= 0xffffffffull)
                    ei = udiv_apply(static_cast<uint32_t>(h), p.hpe_magic, p.hpe_shifts);
                else
                    ei = p.uniform_hpe ? static_cast<uint32_t>(h / p.uniform_hpe) : find_exposure(p.source, h);
                DevExposure ex;
                load_exposure(p.source.exposures + ei, ex);
                sample_particle(p.source, ex, rng, ph);
                inworld = transport_to_world(p.world, ph);
                ++generated;
            }
            const unsigned mask = __ballot_sync(FULL_MASK, inworld);
            unsigned long long slot0 = 0;
            if (lane == 0 && mask)
                slot0 = atomicAdd(&p.counters->queue_count, static_cast<unsigned long long>(__popc(mask)));
            slot0 = __shfl_sync(FULL_MASK, slot0, 0);
            if (inworld) {
                const uint64_t q = slot0 + __popc(mask & ((1u << lane) - 1u));
                p.queue.pos_energy[q] = make_float4(ph.px, ph.py, ph.pz, ph.energy);
                p.queue.dir_weight[q] = make_float4(ph.dx, ph.dy, ph.dz, ph.weight);
                p.queue.rng[q] = make_uint4(rng.s0, rng.s1, rng.s2, rng.s3);
            }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1)
            generated += __shfl_down_sync(FULL_MASK, generated, off);
        if (lane == 0 && generated)
            atomicAdd(&p.counters->histories_done, generated);
    }

    // ---- post-processing (transport.hpp:780-816) -------------------------------------
    template <typename TallyT>
    __global__ void postprocess_kernel(const TallyT* __restrict__ tally, const Voxel* __restrict__ voxels,
        const uint8_t* __restrict__ palette_index, const PaletteEntry* __restrict__ palette, uint64_t n, int mode,
        double histories, double voxel_volume_cm3, double calibration, double* __restrict__ dose, double* __restrict__ variance,
        const uint32_t* __restrict__ counts, uint32_t* __restrict__ counts_out)
    {
        const double h_inv = 1.0 / (histories - 1.0);
        const double h_d = 1.0e3 / histories;
        const double h_v = 1.0e6 / histories;
        for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n; i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
            const double e = static_cast<double>(tally[2 * i]);
            const double ee = static_cast<double>(tally[2 * i + 1]);
            double d = e, v = ee;
            if (mode == 1) { // EV_PER_HISTORY: normalizeScoring
                d = e * h_d;
                v = (ee * h_v - d * d) * h_inv;
            } else if (mode == 2) { // DOSE: energyImpartedToDose
                const double de = static_cast<double>(voxels ? voxels[i].density : palette[palette_index[i]].density);
                const double mass = de * voxel_volume_cm3 * 0.001;
                const double f = calibration / mass;
                d = de > 0.0 ? e * f : 0.0;
                v = de > 0.0 ? ee * f * f : 0.0;
            }
            if (dose)
                dose[i] = d;
            if (variance)
                variance[i] = v;
            if (counts_out)
                counts_out[i] = __ldg(counts + i);
        }
    }

    // Post-processing from tally records: one 32-byte record read per voxel; the
    // results in double (Result<double>) or float (Result<float>), computed in double.
    template <typename OutT>
    __global__ void postprocess_records_kernel(const TallyRecord* __restrict__ rec, const Voxel* __restrict__ voxels,
        const uint8_t* __restrict__ palette_index, const PaletteEntry* __restrict__ palette, uint64_t n, int mode,
        double histories, double voxel_volume_cm3, double calibration, OutT* __restrict__ dose, OutT* __restrict__ variance,
        uint32_t* __restrict__ counts_out)
    {
        const double h_inv = 1.0 / (histories - 1.0);
        const double h_d = 1.0e3 / histories;
        const double h_v = 1.0e6 / histories;
        for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n; i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
            const double2 ee2 = __ldcs(reinterpret_cast<const double2*>(rec + i));
            const double e = ee2.x, ee = ee2.y;
            double d = e, v = ee;
            if (mode == 1) { // EV_PER_HISTORY: normalizeScoring
                d = e * h_d;
                v = (ee * h_v - d * d) * h_inv;
            } else if (mode == 2) { // DOSE: energyImpartedToDose
                const double de = static_cast<double>(voxels ? voxels[i].density : palette[palette_index[i]].density);
                const double mass = de * voxel_volume_cm3 * 0.001;
                const double f = calibration / mass;
                d = de > 0.0 ? e * f : 0.0;
                v = de > 0.0 ? ee * f * f : 0.0;
            }
            if (dose)
                dose[i] = static_cast<OutT>(d);
            if (variance)
                variance[i] = static_cast<OutT>(v);
            if (counts_out)
                counts_out[i] = __ldcs(&rec[i].events);
        }
    }

    // ---- per-material maximum density (attenuationinterpolator.hpp:48-60) ------------
    __global__ void max_density_kernel(const Voxel* __restrict__ voxels, uint64_t n, unsigned int* out_bits, int n_materials)
    {
        extern __shared__ unsigned int sbits[];
        for (int i = threadIdx.x; i < n_materials; i += blockDim.x)
            sbits[i] = 0u;
        __syncthreads();
        for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n; i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
            const uint2 raw = __ldg(reinterpret_cast<const uint2*>(voxels) + i);
            const int mat = raw.y & 0xffu;
            const float d = __uint_as_float(raw.x);
            if (mat < n_materials && d > 0.0f)
                atomicMax(&sbits[mat], raw.x); // non-negative floats order like their bits
        }
        __syncthreads();
        for (int i = threadIdx.x; i < n_materials; i += blockDim.x)
            if (sbits[i])
                atomicMax(out_bits + i, sbits[i]);
    }

    // ---- probes ------------------------------------------------------------------------
    __global__ void probe_lut_kernel(const float* L, LutMeta m, int material, const double* energies, int n, double* out_att, double* out_maxinv)
    {
        const int i = blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= n)
            return;
        const float E = static_cast<float>(energies[i]);
        const float logE = __log10f(E);
        const int seg = lut_segment(L, m, logE);
        float a, b, c;
        lut_attenuation(L, m, material, logE, seg, a, b, c);
        out_att[3 * i] = a;
        out_att[3 * i + 1] = b;
        out_att[3 * i + 2] = c;
        out_maxinv[i] = lut_max_inverse(L, m, logE, seg);
    }

    template <int MODEL>
    __global__ void probe_interactions_kernel(const float* L, LutMeta m, int material, int kind, float energy, uint64_t n, uint64_t seed,
        float* out_cos, float* out_energy, float* out_dep)
    {
        for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n; i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
            Rng rng;
            rng.init(seed, i);
            PhotonT<float> ph { 0, 0, 0, 0, 0, 1, energy, 1 };
            float dep = 0.0f;
            bool ok = true;
            if (kind == 0)
                dep = photo_absorption<MODEL>(L, m, ph, material, rng);
            else if (kind == 1)
                ok = compton_scatter<MODEL>(L, L, m, ph, material, rng, dep);
            else
                ok = rayleigh_scatter<MODEL>(L, L, m, ph, material, rng);
            const float len = sqrtf(ph.dx * ph.dx + ph.dy * ph.dy + ph.dz * ph.dz);
            out_cos[i] = ok ? (len > 0 ? ph.dz / len : 1.0f) : 2.0f;
            out_energy[i] = ph.energy;
            out_dep[i] = dep;
        }
    }

    // Histogram of the per-history streams' output (the generator every sampler
    // draws from): n_streams streams of `draws` values each.  kind 0: uniform()
    // in [0, 1); kind 1: uniform_open() in (0, 1], binned as 1 - u; kind 2:
    // below(nbins).  hist[nbins] counts values outside their stated range.
    __global__ void probe_uniform_kernel(uint64_t seed, uint64_t n_streams, uint32_t draws, int kind, int nbins,
        unsigned long long* hist)
    {
        extern __shared__ unsigned int sbins[];
        for (int i = threadIdx.x; i <= nbins; i += blockDim.x)
            sbins[i] = 0u;
        __syncthreads();
        for (uint64_t h = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; h < n_streams;
             h += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
            Rng rng;
            rng.init(seed, h);
            for (uint32_t k = 0; k < draws; ++k) {
                int b;
                if (kind == 0) {
                    const float u = rng.uniform();
                    b = (u >= 0.0f && u < 1.0f) ? min(static_cast<int>(u * nbins), nbins - 1) : nbins;
                } else if (kind == 1) {
                    const float u = rng.uniform_open();
                    b = (u > 0.0f && u <= 1.0f) ? min(static_cast<int>((1.0f - u) * nbins), nbins - 1) : nbins;
                } else {
                    const uint32_t v = rng.below(static_cast<uint32_t>(nbins));
                    b = v < static_cast<uint32_t>(nbins) ? static_cast<int>(v) : nbins;
                }
                atomicAdd(&sbins[b], 1u);
            }
        }
        __syncthreads();
        for (int i = threadIdx.x; i <= nbins; i += blockDim.x)
            if (sbins[i])
                atomicAdd(hist + i, static_cast<unsigned long long>(sbins[i]));
    }

} // namespace

template <class Real, int MODEL, bool PALETTE>
static void* transport_entry() { return reinterpret_cast<void*>(&transport_kernel<Real, MODEL, PALETTE>); }

template <class Real>
static void* transport_function_as(int model, bool palette)
{
    if (palette)
        return model == 0 ? transport_entry<Real, 0, true>() : (model == 1 ? transport_entry<Real, 1, true>() : transport_entry<Real, 2, true>());
    return model == 0 ? transport_entry<Real, 0, false>() : (model == 1 ? transport_entry<Real, 1, false>() : transport_entry<Real, 2, false>());
}

// precision 0: FP32 transport (the fast path); 1: FP64 everywhere (the precision study)
static void* transport_function(int model, bool palette, int precision)
{
    return precision == 1 ? transport_function_as<double>(model, palette) : transport_function_as<float>(model, palette);
}

const void* batch_kernel_function(int model)
{
    if (model == 0)
        return reinterpret_cast<const void*>(&batch_transport_kernel<0>);
    if (model == 1)
        return reinterpret_cast<const void*>(&batch_transport_kernel<1>);
    return reinterpret_cast<const void*>(&batch_transport_kernel<2>);
}

int batch_max_blocks_per_sm(int model)
{
    int n = 0;
    cudaError_t e;
    if (model == 0)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_transport_kernel<0>, 256, 0);
    else if (model == 1)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_transport_kernel<1>, 256, 0);
    else
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_transport_kernel<2>, 256, 0);
    return e == cudaSuccess ? n : 0;
}

cudaError_t launch_generate(const TransportParams& p, uint64_t first, uint64_t count, int grid, cudaStream_t stream)
{
    generate_kernel<<<grid, 256, 0, stream>>>(p, first, count);
    return cudaGetLastError();
}

size_t transport_smem_bytes(size_t lut_bytes, bool lut_in_smem, bool palette)
{
    size_t b = lut_in_smem ? (lut_bytes + 15) / 16 * 16 : 0;
    if (palette)
        b += PALETTE_MAX * sizeof(PaletteEntry);
    return b;
}

cudaError_t launch_transport(const TransportParams& p, int model, int grid, int block, size_t smem, cudaStream_t stream)
{
    const bool palette = p.world.palette_index != nullptr;
    void* fn = transport_function(model, palette, p.precision);
    void* args[] = { const_cast<TransportParams*>(&p) };
    return cudaLaunchKernel(fn, dim3(grid), dim3(block), args, smem, stream);
}

cudaError_t preload_transport_kernels()
{
    for (int precision = 0; precision < 2; ++precision)
        for (int model = 0; model < 3; ++model)
            for (int palette = 0; palette < 2; ++palette) {
                cudaFuncAttributes attr {};
                const cudaError_t e = cudaFuncGetAttributes(&attr, transport_function(model, palette != 0, precision));
                if (e != cudaSuccess)
                    return e;
            }
    return cudaSuccess;
}

int transport_max_blocks_per_sm(int model, bool palette, int block, size_t smem, int precision)
{
    void* fn = transport_function(model, palette, precision);
    // The dynamic shared-memory limit is a property of the function, read when a
    // launch (or a graph holding it) is made: it only ever grows, so launches
    // queued or captured earlier with larger LUTs stay valid.
    static std::mutex m;
    static int limit[12] = {};
    {
        std::lock_guard<std::mutex> lock(m);
        int& cur = limit[(precision == 1 ? 6 : 0) + model * 2 + (palette ? 1 : 0)];
        if (static_cast<int>(smem) > cur) {
            if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)) == cudaSuccess)
                cur = static_cast<int>(smem);
        }
    }
    int n = 0;
    const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, block, smem);
    return e == cudaSuccess ? n : 0;
}

cudaError_t launch_postprocess(const double* tally, const WorldParams& w, uint64_t n, int mode, double histories,
    double voxel_volume_cm3, double calibration, double* dose, double* variance, const uint32_t* counts, uint32_t* counts_out,
    cudaStream_t stream)
{
    const int block = 256;
    const int grid = static_cast<int>(std::min<uint64_t>((n + block - 1) / block, 152ull * 16));
    postprocess_kernel<double><<<grid, block, 0, stream>>>(tally, w.palette_index ? nullptr : w.voxels, w.palette_index, w.palette, n, mode,
        histories, voxel_volume_cm3, calibration, dose, variance, counts, counts_out);
    return cudaGetLastError();
}

cudaError_t launch_postprocess_records(const TallyRecord* records, const WorldParams& w, uint64_t n, int mode,
    double histories, double voxel_volume_cm3, double calibration, double* dose, double* variance, uint32_t* counts_out,
    cudaStream_t stream)
{
    const int block = 256;
    const int grid = static_cast<int>(std::min<uint64_t>((n + block - 1) / block, 152ull * 16));
    postprocess_records_kernel<double><<<grid, block, 0, stream>>>(records, w.palette_index ? nullptr : w.voxels, w.palette_index,
        w.palette, n, mode, histories, voxel_volume_cm3, calibration, dose, variance, counts_out);
    return cudaGetLastError();
}

cudaError_t launch_postprocess_records_f32(const TallyRecord* records, const WorldParams& w, uint64_t n, int mode,
    double histories, double voxel_volume_cm3, double calibration, float* dose, float* variance, uint32_t* counts_out,
    cudaStream_t stream)
{
    const int block = 256;
    const int grid = static_cast<int>(std::min<uint64_t>((n + block - 1) / block, 152ull * 16));
    postprocess_records_kernel<float><<<grid, block, 0, stream>>>(records, w.palette_index ? nullptr : w.voxels, w.palette_index,
        w.palette, n, mode, histories, voxel_volume_cm3, calibration, dose, variance, counts_out);
    return cudaGetLastError();
}

cudaError_t launch_postprocess_f32(const float* tally, const WorldParams& w, uint64_t n, int mode, double histories,
    double voxel_volume_cm3, double calibration, double* dose, double* variance, const uint32_t* counts, uint32_t* counts_out,
    cudaStream_t stream)
{
    const int block = 256;
    const int grid = static_cast<int>(std::min<uint64_t>((n + block - 1) / block, 152ull * 16));
    postprocess_kernel<float><<<grid, block, 0, stream>>>(tally, w.palette_index ? nullptr : w.voxels, w.palette_index, w.palette, n, mode,
        histories, voxel_volume_cm3, calibration, dose, variance, counts, counts_out);
    return cudaGetLastError();
}

cudaError_t launch_max_density(const Voxel* voxels, uint64_t n, unsigned int* out_bits, int n_materials, cudaStream_t stream)
{
    const int block = 256;
    const int grid = static_cast<int>(std::min<uint64_t>((n + block - 1) / block, 152ull * 8));
    max_density_kernel<<<grid, block, n_materials * sizeof(unsigned int), stream>>>(voxels, n, out_bits, n_materials);
    return cudaGetLastError();
}

cudaError_t launch_probe_lut(const float* lut, LutMeta meta, int material, const double* energies, int n, double* out_att, double* out_maxinv, cudaStream_t stream)
{
    probe_lut_kernel<<<(n + 127) / 128, 128, 0, stream>>>(lut, meta, material, energies, n, out_att, out_maxinv);
    return cudaGetLastError();
}

cudaError_t launch_probe_interactions(const float* lut, LutMeta meta, int material, int model, int kind, float energy,
    uint64_t n, uint64_t seed, float* out_cos, float* out_energy, float* out_dep, cudaStream_t stream)
{
    const int block = 256;
    const int grid = static_cast<int>(std::min<uint64_t>((n + block - 1) / block, 152ull * 8));
    if (model == 0)
        probe_interactions_kernel<0><<<grid, block, 0, stream>>>(lut, meta, material, kind, energy, n, seed, out_cos, out_energy, out_dep);
    else if (model == 1)
        probe_interactions_kernel<1><<<grid, block, 0, stream>>>(lut, meta, material, kind, energy, n, seed, out_cos, out_energy, out_dep);
    else
        probe_interactions_kernel<2><<<grid, block, 0, stream>>>(lut, meta, material, kind, energy, n, seed, out_cos, out_energy, out_dep);
    return cudaGetLastError();
}

cudaError_t launch_probe_uniform(uint64_t seed, uint64_t n_streams, uint32_t draws, int kind, int nbins,
    unsigned long long* hist, int sm_count, cudaStream_t stream)
{
    const int block = 256;
    const int grid = static_cast<int>(std::min<uint64_t>((n_streams + block - 1) / block, static_cast<uint64_t>(sm_count) * 8));
    probe_uniform_kernel<<<grid, block, (nbins + 1) * sizeof(unsigned int), stream>>>(seed, n_streams, draws, kind, nbins, hist);
    return cudaGetLastError();
}

} // namespace dxmc_gb300::dev
