// Device kernels of the MD step: cell keys, gather into cell order, Verlet-list build, the fused
// LJ force + integer leapfrog, the cell-list force, kicks/observables and reversal.
//
// Reference counterparts (crates/md/shaders): md.wgsl:26-33 / md3.wgsl:208-215 (cells),
// reorder.wgsl:17-70 (reorder), neighbors.wgsl:27-64 / md3.wgsl:443-483 (build_list),
// neighbors.wgsl:67-100 / md3.wgsl:486-518 (force_list, integrate_list), md.wgsl:39-76 /
// md3.wgsl:272-303 (cell-list force, integrate), md.wgsl:169-179 (reverse). The CPU definitions
// they must reproduce bit for bit: md-ref int_engine.rs:130-344 and int_engine3.rs:48-184.
#pragma once

#include "common.cuh"

namespace gbmd {

template <int D> using PosRec = typename PosT<D>::T;

// Position and species of slot i. In 3D the species rides in the record's fourth word; in 2D it
// is read from `species` when the system has more than one.
template <int D, bool MULTI>
__device__ __forceinline__ uint32_t load_particle(const PosRec<D>* pos, const uint32_t* species, uint32_t i, int64_t* x) {
    if constexpr (D == 2) {
        longlong2 v = __ldg(pos + i);
        x[0] = v.x;
        x[1] = v.y;
        return MULTI ? __ldg(species + i) : 0u;
    } else {
        const longlong2* q = reinterpret_cast<const longlong2*>(pos + i);
        longlong2 a = __ldg(q), b = __ldg(q + 1);
        x[0] = a.x;
        x[1] = a.y;
        x[2] = b.x;
        return MULTI ? (uint32_t)b.y : 0u;
    }
}

// Row-major cell key (md-ref cells.rs:10-15; int_engine3.rs:53-57) with f64 cell_of per axis.
template <int D> __device__ __forceinline__ uint32_t cell_key(const Params& P, const int64_t* x, uint32_t* c) {
    c[0] = cell_of(x[0], P.box_f[0], P.nc[0]);
    c[1] = cell_of(x[1], P.box_f[1], P.nc[1]);
    if constexpr (D == 2) {
        c[2] = 0;
        return c[1] * P.nc[0] + c[0];
    } else {
        c[2] = cell_of(x[2], P.box_f[2], P.nc[2]);
        return (c[2] * P.nc[1] + c[1]) * P.nc[0] + c[0];
    }
}

template <int D> __global__ void k_keys(Params P, const PosRec<D>* pos, uint32_t* keys, uint32_t* vals) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    int64_t x[3];
    load_particle<D, false>(pos, nullptr, i, x);
    uint32_t c[3];
    keys[i] = cell_key<D>(P, x, c);
    vals[i] = i;
}

// Storage permutation into cell order (one fused gather; reorder.wgsl's gathers + copy-backs).
template <int D>
__global__ void k_gather(uint32_t n, uint32_t dim, const uint32_t* items, const PosRec<D>* pos, const int32_t* vel, const uint32_t* species,
                         const uint32_t* ids, PosRec<D>* pos_o, int32_t* vel_o, uint32_t* species_o, uint32_t* ids_o) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    uint32_t o = items[s];
    pos_o[s] = pos[o];
    for (uint32_t a = 0; a < D; a++) vel_o[D * s + a] = vel[D * o + a];
    species_o[s] = species[o];
    ids_o[s] = ids[o];
}

__device__ __forceinline__ int32_t wadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }

// One directed pair (i from j): adds the integer kick rint(a * f) per axis, exactly
// IntEngine::forces' `(a * fx).round_even().to_i32()` summed with wrapping adds.
template <int D>
__device__ __forceinline__ bool pair_kick(const Params& P, const PairC& pc, float cs, const int64_t* xi, const int64_t* xj, int32_t* k,
                                          float& fr_s, float& s6, float& r2) {
    bool ok = true;
    float f[D];
#pragma unroll
    for (int a = 0; a < D; a++) f[a] = sep_s(min_image(xj[a] - xi[a], P.box[a], P.half[a]), ok);
    if (!ok) return false;
    if (!pair_fr<D>(pc, f, fr_s, s6, r2)) return false;
    float am = __fmul_rn(-fr_s, cs);
#pragma unroll
    for (int a = 0; a < D; a++) k[a] = wadd(k[a], rni_f32(__fmul_rn(am, f[a])));
    return true;
}

// Leapfrog of one particle (int_engine.rs:265-339 / int_engine3.rs:147-179, periodic):
// v += kick + g (wrapping i32), x += v (exact i64), wrap into [0, L).
template <int D>
__device__ __forceinline__ void leapfrog(const Params& P, uint32_t si, const int32_t* k, int32_t* v, int64_t* x) {
    bool pinned = (P.pinned >> si) & 1u;
#pragma unroll
    for (int a = 0; a < D; a++) {
        v[a] = wadd(wadd(v[a], k[a]), pinned ? 0 : P.gravity[a]);
        x[a] = wrap(x[a] + (int64_t)v[a], P.box[a]);
    }
}

// The displacement trigger of integrate_list (neighbors.wgsl:90-100): has the particle moved
// half the skin since the list was built? (f32 separations; beyond 8 sigma counts as moved.)
template <int D> __device__ __forceinline__ bool moved_half_skin(const Params& P, const int64_t* ref, const int64_t* x) {
    bool ok = true;
    float f[D];
#pragma unroll
    for (int a = 0; a < D; a++) f[a] = sep_s(min_image(x[a] - ref[a], P.box[a], P.half[a]), ok);
    if (!ok) return true;
    float r2 = __fadd_rn(__fmul_rn(f[0], f[0]), __fmul_rn(f[1], f[1]));
    if (D == 3) r2 = __fadd_rn(r2, __fmul_rn(f[2], f[2]));
    return !(r2 < P.half_skin2s);
}

// Visit the 3^D cells around cell c (cells.rs:36-48 order), calling f(cell).
template <int D, typename Fn> __device__ __forceinline__ void for_cells(const Params& P, const uint32_t* c, Fn&& f) {
    const uint32_t nx = P.nc[0], ny = P.nc[1], nz = P.nc[2];
    for (int oz = 0; oz < (D == 3 ? 3 : 1); oz++) {
        uint32_t z = D == 3 ? (c[2] + nz + (uint32_t)oz - 1) % nz : 0;
        for (int oy = 0; oy < 3; oy++) {
            uint32_t y = (c[1] + ny + (uint32_t)oy - 1) % ny;
            for (int ox = 0; ox < 3; ox++) {
                uint32_t x = (c[0] + nx + (uint32_t)ox - 1) % nx;
                f((z * ny + y) * nx + x);
            }
        }
    }
}

__device__ __forceinline__ void cell_coords(const Params& P, uint32_t key, uint32_t* c) {
    c[0] = key % P.nc[0];
    c[1] = (key / P.nc[0]) % P.nc[1];
    c[2] = key / (P.nc[0] * P.nc[1]);
}

// Verlet-list build over the cell-sorted scratch state (neighbors.wgsl:27-64 with the exact f32
// test of engine.rs:302-313 / 184-186): lists are column-major, nbr[k * n + i]; a particle with
// more than `cap` neighbours sets ctl[1] (overflow). Also copies the sorted state back into the
// engine's arrays and records each particle's reference position for the trigger.
template <int D, bool MULTI>
__global__ void __launch_bounds__(128) k_build_list(Params P, const PosRec<D>* __restrict__ pos_s, const int32_t* __restrict__ vel_s,
                                                    const uint32_t* __restrict__ species_s, const uint32_t* __restrict__ ids_s,
                                                    const uint32_t* __restrict__ keys, const uint32_t* __restrict__ start,
                                                    PosRec<D>* __restrict__ pos_o, int32_t* __restrict__ vel_o,
                                                    uint32_t* __restrict__ species_o, uint32_t* __restrict__ ids_o,
                                                    PosRec<D>* __restrict__ ref_pos, uint32_t* __restrict__ nbr,
                                                    uint32_t* __restrict__ nbr_count, uint32_t* __restrict__ ctl) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    int64_t xi[3];
    uint32_t si = load_particle<D, MULTI>(pos_s, species_s, i, xi);
    uint32_t c[3];
    cell_coords(P, keys[i], c);
    uint32_t count = 0;
    const uint32_t n = P.n, cap = P.cap;
    for_cells<D>(P, c, [&](uint32_t cell) {
        uint32_t j0 = __ldg(start + cell), j1 = __ldg(start + cell + 1);
        for (uint32_t j = j0; j < j1; j++) {
            if (j == i) continue;
            int64_t xj[3];
            uint32_t sj = load_particle<D, MULTI>(pos_s, species_s, j, xj);
            bool ok = true;
            float f[D];
#pragma unroll
            for (int a = 0; a < D; a++) f[a] = sep_s(min_image(xj[a] - xi[a], P.box[a], P.half[a]), ok);
            if (!ok) continue;
            float r2 = __fadd_rn(__fmul_rn(f[0], f[0]), __fmul_rn(f[1], f[1]));
            if (D == 3) r2 = __fadd_rn(r2, __fmul_rn(f[2], f[2]));
            if (r2 < P.pc[si * P.ns + sj].list2s) {
                if (count < cap) nbr[(size_t)count * n + i] = j;
                count++;
            }
        }
    });
    if (count > cap) {
        ctl[1] = 1;
        count = cap;
    }
    nbr_count[i] = count;
    pos_o[i] = pos_s[i];
    ref_pos[i] = pos_s[i];
#pragma unroll
    for (int a = 0; a < D; a++) vel_o[D * i + a] = vel_s[D * i + a];
    species_o[i] = species_s[i];
    ids_o[i] = ids_s[i];
}

// The hot kernel: LJ pair kicks over the Verlet list fused with the integer leapfrog and the
// rebuild trigger. Reads positions from pos_in and writes the moved ones to pos_out (the engine
// ping-pongs the two), so every kick sees positions of the same time step.
template <int D, bool MULTI>
__global__ void __launch_bounds__(128) k_force_list(Params P, const PosRec<D>* __restrict__ pos_in, PosRec<D>* __restrict__ pos_out,
                                                    int32_t* __restrict__ vel, const uint32_t* __restrict__ species,
                                                    const uint32_t* __restrict__ nbr, const uint32_t* __restrict__ nbr_count,
                                                    const PosRec<D>* __restrict__ ref_pos, uint32_t* __restrict__ ctl) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    int64_t xi[3];
    uint32_t si = load_particle<D, MULTI>(pos_in, species, i, xi);
    const float cs = P.kick_cs[si];
    int32_t k[3] = {0, 0, 0};
    const uint32_t m = __ldg(nbr_count + i), n = P.n;
    const PairC pc0 = P.pc[0];
    for (uint32_t q = 0; q < m; q++) {
        uint32_t j = __ldg(nbr + (size_t)q * n + i);
        int64_t xj[3];
        uint32_t sj = load_particle<D, MULTI>(pos_in, species, j, xj);
        float fr, s6, r2;
        pair_kick<D>(P, MULTI ? P.pc[si * P.ns + sj] : pc0, cs, xi, xj, k, fr, s6, r2);
    }
    int32_t v[3];
#pragma unroll
    for (int a = 0; a < D; a++) v[a] = vel[D * i + a];
    leapfrog<D>(P, si, k, v, xi);
#pragma unroll
    for (int a = 0; a < D; a++) vel[D * i + a] = v[a];
    store_pos<D>(pos_out, i, xi, si);
    int64_t xr[3];
    load_particle<D, false>(ref_pos, nullptr, i, xr);
    if (moved_half_skin<D>(P, xr, xi)) ctl[0] = 1;
}

// Cell-list force + leapfrog (ForceMode::CellList; md.wgsl:39-76): scans the 3^D cells of the
// sorted scratch state and writes the moved state back into the engine's arrays.
template <int D, bool MULTI>
__global__ void __launch_bounds__(128) k_force_cells(Params P, const PosRec<D>* __restrict__ pos_s, const int32_t* __restrict__ vel_s,
                                                     const uint32_t* __restrict__ species_s, const uint32_t* __restrict__ ids_s,
                                                     const uint32_t* __restrict__ keys, const uint32_t* __restrict__ start,
                                                     PosRec<D>* __restrict__ pos_o, int32_t* __restrict__ vel_o,
                                                     uint32_t* __restrict__ species_o, uint32_t* __restrict__ ids_o) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    int64_t xi[3];
    uint32_t si = load_particle<D, MULTI>(pos_s, species_s, i, xi);
    const float cs = P.kick_cs[si];
    int32_t k[3] = {0, 0, 0};
    uint32_t c[3];
    cell_coords(P, keys[i], c);
    for_cells<D>(P, c, [&](uint32_t cell) {
        uint32_t j0 = __ldg(start + cell), j1 = __ldg(start + cell + 1);
        for (uint32_t j = j0; j < j1; j++) {
            if (j == i) continue;
            int64_t xj[3];
            uint32_t sj = load_particle<D, MULTI>(pos_s, species_s, j, xj);
            float fr, s6, r2;
            pair_kick<D>(P, P.pc[si * P.ns + sj], cs, xi, xj, k, fr, s6, r2);
        }
    });
    int32_t v[3];
#pragma unroll
    for (int a = 0; a < D; a++) v[a] = vel_s[D * i + a];
    leapfrog<D>(P, si, k, v, xi);
#pragma unroll
    for (int a = 0; a < D; a++) vel_o[D * i + a] = v[a];
    store_pos<D>(pos_o, i, xi, si);
    species_o[i] = species_s[i];
    ids_o[i] = ids_s[i];
}

// Kicks at the current positions (no move), optionally with the f64 per-particle observables
// reduced per block: partial[4 b + 0] potential (1/2 sum of f32 u), [1] virial (1/2 sum of the
// f32 fr r^2), [2] on-step kinetic energy (int_engine.rs:417-446). `list` selects the Verlet
// list (nbr != nullptr) or the 3^D cell scan over `start`/`keys`. With `reverse` set the
// velocities become -(v + kick + g) (int_engine.rs:396-413).
template <int D, bool MULTI>
__global__ void __launch_bounds__(128) k_kicks(Params P, const PosRec<D>* __restrict__ pos, const uint32_t* __restrict__ species,
                                               const uint32_t* __restrict__ nbr, const uint32_t* __restrict__ nbr_count,
                                               const uint32_t* __restrict__ keys, const uint32_t* __restrict__ start,
                                               int32_t* __restrict__ vel, int32_t* __restrict__ kicks, double* __restrict__ partial,
                                               int reverse) {
    __shared__ double sh[3][4];
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    double pe = 0.0, w = 0.0, ke = 0.0;
    if (i < P.n) {
        int64_t xi[3];
        uint32_t si = load_particle<D, MULTI>(pos, species, i, xi);
        const float cs = P.kick_cs[si];
        int32_t k[3] = {0, 0, 0};
        auto visit = [&](uint32_t j) {
            int64_t xj[3];
            uint32_t sj = load_particle<D, MULTI>(pos, species, j, xj);
            const PairC& pc = P.pc[si * P.ns + sj];
            float fr, s6, r2;
            if (pair_kick<D>(P, pc, cs, xi, xj, k, fr, s6, r2)) {
                pe += (double)pair_u(pc, s6);
                w += (double)__fmul_rn(fr, r2);
            }
        };
        if (nbr) {
            uint32_t m = nbr_count[i];
            for (uint32_t q = 0; q < m; q++) visit(nbr[(size_t)q * P.n + i]);
        } else {
            uint32_t c[3];
            cell_coords(P, keys[i], c);
            for_cells<D>(P, c, [&](uint32_t cell) {
                for (uint32_t j = start[cell]; j < start[cell + 1]; j++)
                    if (j != i) visit(j);
            });
        }
        pe *= 0.5;
        w *= 0.5;
        double m = P.masses[si];
        for (int a = 0; a < D; a++) {
            int32_t v0 = vel[D * i + a];
            int32_t next = wadd(wadd(v0, k[a]), P.gravity[a]);
            // 0.5 (velocity(v) + velocity(next)), velocity(v) = v UNIT / dt (system.rs:423-425)
            double vh = __dmul_rn(0.5, __dadd_rn(__ddiv_rn(__dmul_rn((double)v0, 1.0 / 4294967296.0), P.dt),
                                                 __ddiv_rn(__dmul_rn((double)next, 1.0 / 4294967296.0), P.dt)));
            ke += 0.5 * m * vh * vh;
            if (kicks) kicks[D * i + a] = k[a];
            if (reverse) {
                bool pinned = (P.pinned >> si) & 1u;
                vel[D * i + a] = (int32_t)(0u - (uint32_t)wadd(wadd(v0, k[a]), pinned ? 0 : P.gravity[a]));
            }
        }
    }
    if (!partial) return;
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double vals[3] = {pe, w, ke};
    for (int q = 0; q < 3; q++) {
        double x = vals[q];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) sh[q][warp] = x;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double s = 0.0;
        for (int wq = 0; wq < (int)(blockDim.x >> 5); wq++) s += sh[threadIdx.x][wq];
        partial[4 * blockIdx.x + threadIdx.x] = s;
    }
}

} // namespace gbmd
