// Batched replicas: many independent periodic systems of uneven size stepped together.
//
// The reference batches only equal compartments of one box separated by walls
// (crates/md-core/src/system.rs:41-48, 219-256; init.rs:126-149). Here every system keeps its
// own box, species table and seed, and all of them share one set of launches:
//   - a segmented cell-key space: system k's cells are numbered from cell_base[k] (the cells of
//     the systems before it), so one stable radix sort bins every system at once and leaves each
//     system's particles contiguous and in cell order;
//   - a per-particle system index selects the system's parameter block (box, pair constants,
//     kick coefficients) from a device table;
//   - the force kernel is persistent (a grid-stride loop over all particles of all systems on a
//     grid sized to the GPU), and 100-step blocks are captured as CUDA graphs with the list
//     rebuild in a conditional node, as in the single-system engine.
// A system's trajectory does not depend on when lists are rebuilt (integer kicks are summed
// order-independently), so each replica's state equals its plain single-system run bit for bit.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"
#include "engine.cuh"
#include "kernels.cuh"
#include "sort.cuh"

using namespace gbmd;

namespace {

// Geometry of one system held in registers by a thread.
struct Geom {
    int64_t box[3], half[3];
    int32_t gravity[3];
    uint32_t pinned, periodic;
    float half_skin2s;
};
__device__ __forceinline__ Geom geom_of(const Params& P) {
    Geom g;
    for (int a = 0; a < 3; a++) {
        g.box[a] = P.box[a];
        g.half[a] = P.half[a];
        g.gravity[a] = P.gravity[a];
    }
    g.pinned = P.pinned;
    g.periodic = P.periodic;
    g.half_skin2s = P.half_skin2s;
    return g;
}

template <int D>
__global__ void k_bkeys(uint32_t N, const Params* __restrict__ tab, const uint32_t* __restrict__ sysidx, const PosRec<D>* pos,
                        uint32_t* keys, uint32_t* vals) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const Params& P = tab[sysidx[i]];
    int64_t x[3];
    load_particle<D, false>(pos, nullptr, i, x);
#pragma unroll
    for (int a = 0; a < D; a++) x[a] = wrap(x[a], P.box[a]); // positions drift out between list builds
    uint32_t c[3];
    keys[i] = P.cell_base + cell_key<D>(P, x, c);
    vals[i] = i;
}

template <int D>
__global__ void k_bgather(uint32_t N, const Params* __restrict__ tab, const uint32_t* items, const uint32_t* keys, const PosRec<D>* pos,
                          const int32_t* vel, const uint32_t* species, const uint32_t* ids, const uint32_t* sysidx, PosRec<D>* pos_o,
                          int32_t* vel_o, uint32_t* species_o, uint32_t* ids_o, uint32_t* sysidx_o, float4* relf) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= N) return;
    uint32_t o = items[s];
    PosRec<D> r = pos[o];
    const Params& P = tab[sysidx[o]];
    long long* x = reinterpret_cast<long long*>(&r);
#pragma unroll
    for (int a = 0; a < D; a++) x[a] = wrap(x[a], P.box[a]);
    pos_o[s] = r;
    // the position relative to its cell's origin in its own system, f32 sigma (as k_gather)
    uint32_t c[3];
    cell_coords(P, keys[s] - P.cell_base, c);
    float4 f;
    f.x = off_f32(x[0] - (int64_t)c[0] * P.cell_w[0]);
    f.y = off_f32(x[1] - (int64_t)c[1] * P.cell_w[1]);
    f.z = D == 3 ? off_f32(x[2] - (int64_t)c[2] * P.cell_w[2]) : 0.0f;
    f.w = __uint_as_float(species[o]);
    relf[s] = f;
    for (int a = 0; a < D; a++) vel_o[D * s + a] = vel[D * o + a];
    species_o[s] = species[o];
    ids_o[s] = ids[o];
    sysidx_o[s] = sysidx[o];
}

// The list build of k_build_list, each particle in its own system's cells and geometry: the f32
// prefilter over cell-relative records (relf), branch-free appends, and the exact test only for
// the candidates in the prefilter's band, in a second walk of the cells that have one.
template <int D, bool MULTI>
__global__ void __launch_bounds__(128) k_bbuild_list(uint32_t N, uint32_t cap, const Params* __restrict__ tab,
                                                     const uint32_t* __restrict__ sysidx_s, const PosRec<D>* __restrict__ pos_s,
                                                     const int32_t* __restrict__ vel_s, const uint32_t* __restrict__ species_s,
                                                     const uint32_t* __restrict__ ids_s, const uint32_t* __restrict__ keys,
                                                     const uint32_t* __restrict__ start, const float4* __restrict__ relf,
                                                     PosRec<D>* __restrict__ pos_o, int32_t* __restrict__ vel_o,
                                                     uint32_t* __restrict__ species_o, uint32_t* __restrict__ ids_o,
                                                     uint32_t* __restrict__ sysidx_o, PosRec<D>* __restrict__ ref_pos,
                                                     uint32_t* __restrict__ nbr, uint32_t* __restrict__ nbr_count, uint32_t* __restrict__ ctl,
                                                     uint4* __restrict__ qpos_o) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    uint32_t sys = sysidx_s[i];
    const Params& P = tab[sys];
    const uint32_t base = P.cell_base, ns = P.ns, cap4 = (cap + 3u) & ~3u;
    int64_t xi[3];
    uint32_t si = load_particle<D, MULTI>(pos_s, species_s, i, xi);
    uint32_t c[3];
    cell_coords(P, keys[i] - base, c);
    uint32_t count = 0;
    const size_t lbase = list_slot(i, 0, cap4);
    const bool unchecked = P.sep_unchecked;
    int64_t reli[3];
#pragma unroll
    for (int a = 0; a < 3; a++) reli[a] = a < D ? xi[a] - (int64_t)c[a] * P.cell_w[a] : 0;
    auto exact = [&](uint32_t j, const int64_t* xs, uint32_t sj) -> bool {
        int64_t xj[3];
        load_particle<D, false>(pos_s, nullptr, j, xj);
        float f[D];
        bool ok = true;
        if (unchecked) {
#pragma unroll
            for (int a = 0; a < D; a++) f[a] = sep_near(xj[a] - xs[a]);
        } else {
#pragma unroll
            for (int a = 0; a < D; a++) f[a] = sep_s(xj[a] - xs[a], ok);
        }
        float r2 = __fadd_rn(__fmul_rn(f[0], f[0]), __fmul_rn(f[1], f[1]));
        if (D == 3) r2 = __fadd_rn(r2, __fmul_rn(f[2], f[2]));
        return ok && r2 < P.pc[si * ns + sj].list2s;
    };
    const float lo0 = P.pc[si * ns].list2lo, hi0 = P.pc[si * ns].list2hi;
    const uint32_t nx = P.nc[0], ny = P.nc[1], nz = P.nc[2];
    // each neighbour cell at the periodic image that places it next to this one: the list entry
    // carries that image, so the force kernel needs no minimum image (as k_build_list)
    for (int oz = 0; oz < (D == 3 ? 3 : 1); oz++) {
        const int tz = (int)c[2] + oz - 1;
        const uint32_t z = D == 3 ? (tz < 0 ? nz - 1 : (tz >= (int)nz ? 0 : (uint32_t)tz)) : 0;
        const int64_t sz = D == 3 ? (tz < 0 ? -P.box[2] : (tz >= (int)nz ? P.box[2] : 0)) : 0;
        for (int oy = 0; oy < 3; oy++) {
            const int ty = (int)c[1] + oy - 1;
            const uint32_t y = ty < 0 ? ny - 1 : (ty >= (int)ny ? 0 : (uint32_t)ty);
            const int64_t sy = ty < 0 ? -P.box[1] : (ty >= (int)ny ? P.box[1] : 0);
            for (int ox = 0; ox < 3; ox++) {
                const int tx = (int)c[0] + ox - 1;
                const uint32_t x = tx < 0 ? nx - 1 : (tx >= (int)nx ? 0 : (uint32_t)tx);
                const int64_t sx = tx < 0 ? -P.box[0] : (tx >= (int)nx ? P.box[0] : 0);
                const uint32_t cell = (z * ny + y) * nx + x;
                const int64_t xs[3] = {xi[0] - sx, xi[1] - sy, D == 3 ? xi[2] - sz : 0};
                const uint32_t code = image_code(sx, sy, sz);
                const float b0 = off_f32(((int64_t)x - (int64_t)c[0]) * P.cell_w[0] + sx - reli[0]);
                const float b1 = off_f32(((int64_t)y - (int64_t)c[1]) * P.cell_w[1] + sy - reli[1]);
                const float b2 = D == 3 ? off_f32(((int64_t)z - (int64_t)c[2]) * P.cell_w[2] + sz - reli[2]) : 0.0f;
                const uint32_t j0 = __ldg(start + base + cell), j1 = __ldg(start + base + cell + 1);
                auto r2_of = [&](const float4& r) {
                    const float dx = r.x + b0, dy = r.y + b1, dz = D == 3 ? r.z + b2 : 0.0f;
                    return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
                };
                bool band = false;
#pragma unroll 4
                for (uint32_t j = j0; j < j1; j++) {
                    const float4 r = __ldg(relf + j);
                    const float r2a = r2_of(r);
                    const uint32_t sj = MULTI ? __float_as_uint(r.w) : 0u;
                    const float lo = MULTI ? P.pc[si * ns + sj].list2lo : lo0, hi = MULTI ? P.pc[si * ns + sj].list2hi : hi0;
                    const bool in = r2a < lo && j != i;
                    band |= r2a >= lo && r2a <= hi;
                    const size_t at = lbase + ((size_t)(count & ~3u) << 5) + (count & 3u);
                    if (in && count < cap) nbr[at] = j | code;
                    count += in ? 1u : 0u;
                }
                if (band)
                    for (uint32_t j = j0; j < j1; j++) {
                        const float4 r = __ldg(relf + j);
                        const float r2a = r2_of(r);
                        const uint32_t sj = MULTI ? __float_as_uint(r.w) : 0u;
                        const float lo = MULTI ? P.pc[si * ns + sj].list2lo : lo0, hi = MULTI ? P.pc[si * ns + sj].list2hi : hi0;
                        if (r2a >= lo && r2a <= hi && j != i && exact(j, xs, sj)) {
                            if (count < cap) nbr[lbase + ((size_t)(count & ~3u) << 5) + (count & 3u)] = j | code;
                            count++;
                        }
                    }
            }
        }
    }
    if (count > cap) {
        ctl[1] = 1;
        count = cap;
    }
    nbr_count[i] = count;
    pos_o[i] = pos_s[i];
    ref_pos[i] = pos_s[i];
    uint4 q = quot_record<D>(xi, si);
    if (D == 2) q.z = 1u; // the path since this build: 0 (force_list_one's path bound)
    qpos_o[i] = q;
    for (int a = 0; a < D; a++) vel_o[D * i + a] = vel_s[D * i + a];
    species_o[i] = species_s[i];
    ids_o[i] = ids_s[i];
    sysidx_o[i] = sys;
}

// Persistent fused force + leapfrog over every particle of every system: the single-system
// engine's step (force_list_one: warp-tiled lists with periodic-image codes, 16-byte quotient
// records, positions left unwrapped between list builds), each lane with the parameter block of
// its own system. Warps step through the particles 32 / S at a time, S lanes per particle (each
// takes every S-th group of the particle's list; the kicks are summed across its lanes).
template <int D, bool MULTI, bool SIG1, int S>
__global__ void __launch_bounds__(128, 10) k_bforce_list(uint32_t N, const Params* __restrict__ tab, const uint32_t* __restrict__ sysidx,
                                                         const PosRec<D>* __restrict__ pos_in, PosRec<D>* __restrict__ pos_out,
                                                         const uint4* __restrict__ qpos_in, uint4* __restrict__ qpos_out,
                                                         int32_t* __restrict__ vel, const uint32_t* __restrict__ species,
                                                         const uint32_t* __restrict__ nbr, const uint32_t* __restrict__ nbr_count,
                                                         const PosRec<D>* __restrict__ ref_pos, uint32_t* __restrict__ ctl) {
    constexpr uint32_t PER = 32u / S; // particles per warp
    const uint32_t lane = threadIdx.x & 31u, nwarps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w * PER < N; w += nwarps) { // (warp-uniform)
        const uint32_t i = w * PER + lane / S;
        if (S == 1 && i >= N) continue;
        const uint32_t iv = i < N ? i : N - 1; // (S > 1: every lane of the warp takes part in the sums)
        if (force_list_one<D, MULTI, false, SIG1 && !MULTI, S, false>(tab[sysidx[iv]], N, w * 32u + lane, pos_in, pos_out, qpos_in, qpos_out,
                                                                        vel, species, nbr, nbr_count, ref_pos))
            ctl[0] = 1;
    }
}

// The Andersen bath of each system that has one, after the batch's force step: the single-system
// pass (k_bath) with the system's own parameters, its particles' ids counted from the system's
// first, the batch's step clock (every system of a batch has taken the same steps), and the
// system's own ledger slot.
template <int D>
__global__ void k_bbath(uint32_t N, const Params* __restrict__ tab, const uint32_t* __restrict__ sysidx, PosRec<D>* __restrict__ pos,
                        uint4* __restrict__ qpos, int32_t* __restrict__ vel, const uint32_t* __restrict__ species,
                        const uint32_t* __restrict__ ids, const PosRec<D>* __restrict__ ref_pos, uint32_t* __restrict__ ctl,
                        unsigned long long* __restrict__ ledger) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const uint32_t k = sysidx[i];
    const Params& P = tab[k];
    if (!P.bath) return;
    const uint32_t si = species[i];
    if (((P.pinned >> si) & 1u) || !((P.bath_species >> si) & 1u)) return;
    int64_t x[3];
    load_particle<D, false>(pos, nullptr, i, x);
    int32_t v[3] = {0, 0, 0};
#pragma unroll
    for (int a = 0; a < D; a++) v[a] = vel[D * i + a];
    if (D == 2) {
        const uint32_t ax = P.bath_axis;
        const int64_t p = wrap(x[ax] - (int64_t)v[ax], P.box[ax]);
        if (!(p >= P.bath_region[0] && p < P.bath_region[1])) return;
    }
    const BathDraw o = bath_draw<D>(ids[i] - P.id_base, ctl[CTL_CLOCK] + P.clock_base, P.bath_key[0], P.bath_key[1], P.bath_rate_dt, P.bath_sd[si],
                                    P.masses[si], P.dt, P.bath_drift, 0, v[0], v[1], v[2], ledger + 2 * k);
    if (!o.hit) return;
#pragma unroll
    for (int a = 0; a < D; a++) {
        x[a] += (int64_t)o.v[a] - (int64_t)v[a];
        vel[D * i + a] = o.v[a];
    }
    store_pos<D>(pos, i, x, si);
    qpos[i] = quot_record<D>(x, si);
    int64_t xr[3];
    load_particle<D, false>(ref_pos, nullptr, i, xr);
    if (moved_half_skin<D>(geom_of(P), xr, x)) ctl[0] = 1;
}
__global__ void k_bclock_tick(uint32_t* ctl) { ctl[CTL_CLOCK] += 1u; }

template <int D>
__global__ void k_bfrom_host(uint32_t N, const int64_t* ipos, const int32_t* ivel, const uint32_t* ispecies, const uint32_t* isys,
                             PosRec<D>* pos, int32_t* vel, uint32_t* species, uint32_t* ids, uint32_t* sysidx) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= N) return;
    int64_t x[3];
    for (int a = 0; a < D; a++) {
        x[a] = ipos[(size_t)D * s + a];
        vel[D * s + a] = ivel[(size_t)D * s + a];
    }
    store_pos<D>(pos, s, x, ispecies[s]);
    species[s] = ispecies[s];
    ids[s] = s;
    sysidx[s] = isys[s];
}

template <int D>
__global__ void k_bto_ids(uint32_t N, const Params* __restrict__ tab, const uint32_t* sysidx, const PosRec<D>* pos, const int32_t* vel,
                          const uint32_t* species, const uint32_t* ids, int64_t* opos, int32_t* ovel, uint32_t* ospecies) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= N) return;
    uint32_t id = ids[s];
    int64_t x[3];
    load_particle<D, false>(pos, nullptr, s, x);
    const Params& P = tab[sysidx[s]];
    for (int a = 0; a < D; a++) {
        opos[(size_t)D * id + a] = wrap(x[a], P.box[a]); // positions drift out between list builds
        ovel[(size_t)D * id + a] = vel[D * s + a];
    }
    ospecies[id] = species[s];
}

__global__ void k_brebuild_done(uint32_t* ctl) {
    ctl[0] = 0;
    ctl[2] += 1;
}
__global__ void k_bset_cond(cudaGraphConditionalHandle h, const uint32_t* ctl) { cudaGraphSetConditional(h, ctl[0] ? 1u : 0u); }

uint32_t nblocks(uint64_t n, uint32_t t) { return (uint32_t)((n + t - 1) / t); }

} // namespace

struct gbmd_batch {
    uint32_t K = 0, N = 0;
    int D = 2;
    bool multi = false;
    bool sig1 = false; // every pair type sigma = 1 (and one species): the packed force path
    std::vector<gbmd_system> sys;
    std::vector<uint32_t> offsets;
    std::vector<Params> P;
    Params* tab = nullptr;
    uint32_t cap = 0, ncell = 0, bits = 1, grid = 1;
    size_t rec = 16;
    cudaStream_t st = nullptr, st_body = nullptr;
    void *pos[2] = {nullptr, nullptr}, *pos_scr = nullptr, *ref_pos = nullptr;
    int32_t *vel = nullptr, *vel_scr = nullptr;
    uint32_t *species = nullptr, *species_scr = nullptr, *ids = nullptr, *ids_scr = nullptr, *sysidx = nullptr, *sysidx_scr = nullptr;
    uint32_t *keys[2] = {nullptr, nullptr}, *vals[2] = {nullptr, nullptr}, *hist = nullptr, *scan_tmp = nullptr, *start = nullptr;
    uint32_t *nbr = nullptr, *nbr_count = nullptr, *ctl = nullptr;
    uint4* qpos[2] = {nullptr, nullptr}; // quotient records of the positions (ping-pong)
    float4* relf = nullptr;              // cell-relative f32 coordinates of the sorted scratch state
    void* staging = nullptr;
    int32_t* staging_v = nullptr;
    uint32_t* staging_s = nullptr;
    int cur = 0, sorted = 0;
    uint32_t block_steps = 100;
    double skin = 0.4;
    bool bath = false;                   // some system has an Andersen bath
    unsigned long long* ledger = nullptr; // per system: [2k] bath energy (2^-24 epsilon), [2k + 1] redraws
    cudaGraphExec_t exec[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    uint64_t exec_launches[2][2] = {{0, 0}, {0, 0}};
    uint64_t body_launches = 0, launches = 0;
    bool failed = false;
    uint64_t steps = 0;
    uint32_t S = 1; // force lanes per particle
    // frames (gbmd_batch_observe_*): a rebuild when the trigger is set, then per-tile partial sums
    // (a tile: up to 128 slots of one system, whose slots are contiguous) and per-system RDF bins
    cudaGraphExec_t exec_prep[2] = {nullptr, nullptr};
    uint64_t exec_prep_launches[2] = {0, 0};
    std::vector<uint4> tiles_h; // (system, first slot, slots, 0)
    uint4* tiles = nullptr;
    uint32_t* reach = nullptr; // per system: the RDF walk's cell reach per axis (8 bits each)
    double reach_for = -1.0;   // the rmax `reach` was computed for
    double* part = nullptr;
    unsigned long long* obs_bins = nullptr;
    size_t obs_bins_cap = 0;
    double* part_h = nullptr;
    size_t part_h_cap = 0;
    unsigned long long* bins_h = nullptr;
    size_t bins_h_cap = 0;
    bool obs_pending = false;
    uint32_t obs_nbins = 0;
};

namespace {

// Stream-ordered device memory (cudaFree would synchronise the whole device, stalling every other
// engine and batch of a server each time one is retired).
template <typename T> int balloc(T** p, size_t count, cudaStream_t s) {
    cudaError_t e = cudaMallocAsync((void**)p, std::max<size_t>(count, 1) * sizeof(T), s);
    if (e != cudaSuccess) return fail(e == cudaErrorMemoryAllocation ? GBMD_E_NOMEM : GBMD_E_CUDA, std::string("cudaMallocAsync: ") + cudaGetErrorString(e));
    return GBMD_OK;
}

void bfree(gbmd_batch* b) {
    for (int p = 0; p < 2; p++) {
        for (int k = 0; k < 2; k++)
            if (b->exec[p][k]) cudaGraphExecDestroy(b->exec[p][k]);
        if (b->exec_prep[p]) cudaGraphExecDestroy(b->exec_prep[p]);
    }
    void* ptrs[] = {b->tab, b->pos[0], b->pos[1], b->pos_scr, b->ref_pos, b->vel, b->vel_scr, b->species, b->species_scr, b->ids, b->ids_scr,
                    b->sysidx, b->sysidx_scr, b->keys[0], b->keys[1], b->vals[0], b->vals[1], b->hist, b->scan_tmp, b->start, b->nbr,
                    b->nbr_count, b->ctl, b->staging, b->staging_v, b->staging_s, b->qpos[0], b->qpos[1], b->relf, b->ledger,
                    b->tiles, b->part, b->obs_bins, b->reach};
    if (b->st)
        for (void* p : ptrs)
            if (p) cudaFreeAsync(p, b->st);
    pinned_release(b->part_h, b->part_h_cap);
    pinned_release(b->bins_h, b->bins_h_cap);
    if (b->st) cudaStreamDestroy(b->st);
    if (b->st_body) cudaStreamDestroy(b->st_body);
}

template <int D, bool MULTI> void benqueue_rebuild_t(gbmd_batch* b, cudaStream_t s) {
    uint32_t N = b->N;
    k_bkeys<D><<<nblocks(N, 256), 256, 0, s>>>(N, b->tab, b->sysidx, (const PosRec<D>*)b->pos[b->cur], b->keys[0], b->vals[0]);
    b->sorted = radix_sort_pairs(b->keys[0], b->vals[0], b->keys[1], b->vals[1], N, (int)b->bits, b->hist, b->scan_tmp, s);
    cell_starts(b->keys[b->sorted], N, b->ncell, b->start, s);
    k_bgather<D><<<nblocks(N, 256), 256, 0, s>>>(N, b->tab, b->vals[b->sorted], b->keys[b->sorted], (const PosRec<D>*)b->pos[b->cur],
                                                b->vel, b->species, b->ids, b->sysidx, (PosRec<D>*)b->pos_scr, b->vel_scr, b->species_scr,
                                                b->ids_scr, b->sysidx_scr, b->relf);
    k_bbuild_list<D, MULTI><<<nblocks(N, 128), 128, 0, s>>>(N, b->cap, b->tab, b->sysidx_scr, (const PosRec<D>*)b->pos_scr, b->vel_scr,
                                                           b->species_scr, b->ids_scr, b->keys[b->sorted], b->start, b->relf,
                                                           (PosRec<D>*)b->pos[b->cur], b->vel, b->species, b->ids, b->sysidx,
                                                           (PosRec<D>*)b->ref_pos, b->nbr, b->nbr_count, b->ctl, b->qpos[b->cur]);
    k_brebuild_done<<<1, 1, 0, s>>>(b->ctl);
    note_launch(6 + 3 * (uint64_t)radix_passes((int)b->bits));
}
void benqueue_rebuild(gbmd_batch* b, cudaStream_t s) {
    if (b->D == 2) b->multi ? benqueue_rebuild_t<2, true>(b, s) : benqueue_rebuild_t<2, false>(b, s);
    else b->multi ? benqueue_rebuild_t<3, true>(b, s) : benqueue_rebuild_t<3, false>(b, s);
}
// The force kernel variant of a batch: its dimension, species, sigma = 1 and lanes per particle.
template <int D, bool MULTI> const void* bforce_kernel(bool sig1, uint32_t S) {
    if (sig1 && !MULTI)
        return S == 4 ? (const void*)k_bforce_list<D, MULTI, true, 4> : S == 2 ? (const void*)k_bforce_list<D, MULTI, true, 2>
                                                                        : (const void*)k_bforce_list<D, MULTI, true, 1>;
    return S == 4 ? (const void*)k_bforce_list<D, MULTI, false, 4> : S == 2 ? (const void*)k_bforce_list<D, MULTI, false, 2>
                                                                     : (const void*)k_bforce_list<D, MULTI, false, 1>;
}
const void* bforce_kernel_of(int D, bool multi, bool sig1, uint32_t S) {
    if (D == 2) return multi ? bforce_kernel<2, true>(sig1, S) : bforce_kernel<2, false>(sig1, S);
    return multi ? bforce_kernel<3, true>(sig1, S) : bforce_kernel<3, false>(sig1, S);
}
template <int D, bool MULTI> void benqueue_force_t(gbmd_batch* b, cudaStream_t s) {
    const PosRec<D>* pin = (const PosRec<D>*)b->pos[b->cur];
    PosRec<D>* pout = (PosRec<D>*)b->pos[b->cur ^ 1];
    const uint4* qin = b->qpos[b->cur];
    uint4* qout = b->qpos[b->cur ^ 1];
    const PosRec<D>* ref = (const PosRec<D>*)b->ref_pos;
    void* args[] = {(void*)&b->N, (void*)&b->tab, (void*)&b->sysidx, (void*)&pin, (void*)&pout, (void*)&qin, (void*)&qout, (void*)&b->vel,
                    (void*)&b->species, (void*)&b->nbr, (void*)&b->nbr_count, (void*)&ref, (void*)&b->ctl};
    cudaLaunchKernel(bforce_kernel<D, MULTI>(b->sig1, b->S), dim3(b->grid), dim3(128), args, 0, s);
    note_launch();
    b->cur ^= 1;
    if (b->bath) {
        k_bbath<D><<<nblocks(b->N, 256), 256, 0, s>>>(b->N, b->tab, b->sysidx, (PosRec<D>*)b->pos[b->cur], b->qpos[b->cur], b->vel, b->species,
                                                      b->ids, (const PosRec<D>*)b->ref_pos, b->ctl, b->ledger);
        k_bclock_tick<<<1, 1, 0, s>>>(b->ctl);
        note_launch(2);
    }
}
void benqueue_force(gbmd_batch* b, cudaStream_t s) {
    if (b->D == 2) b->multi ? benqueue_force_t<2, true>(b, s) : benqueue_force_t<2, false>(b, s);
    else b->multi ? benqueue_force_t<3, true>(b, s) : benqueue_force_t<3, false>(b, s);
}

// `count` steps (a conditional rebuild, then the force step, each); with `force` false a single
// conditional rebuild (before a frame).
int bcapture(gbmd_batch* b, int parity, uint32_t count, cudaGraphExec_t* out, uint64_t* launches, bool force = true) {
    int saved = b->cur;
    b->cur = parity;
    uint64_t l0 = launch_total();
    cudaStream_t s = b->st;
    GBMD_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    for (uint32_t k = 0; k < count; k++) {
        cudaStreamCaptureStatus status;
        cudaGraph_t g;
        const cudaGraphNode_t* deps;
        const cudaGraphEdgeData* edges;
        size_t ndeps;
        GBMD_CUDA_TRY(cudaStreamGetCaptureInfo(s, &status, nullptr, &g, &deps, &edges, &ndeps));
        cudaGraphConditionalHandle h;
        GBMD_CUDA_TRY(cudaGraphConditionalHandleCreate(&h, g, 0, 0));
        k_bset_cond<<<1, 1, 0, s>>>(h, b->ctl);
        note_launch();
        GBMD_CUDA_TRY(cudaStreamGetCaptureInfo(s, &status, nullptr, &g, &deps, &edges, &ndeps));
        cudaGraphNodeParams cp{};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeIf;
        cp.conditional.size = 1;
        cudaGraphNode_t node;
        GBMD_CUDA_TRY(cudaGraphAddNode(&node, g, deps, edges, ndeps, &cp));
        GBMD_CUDA_TRY(cudaStreamBeginCaptureToGraph(b->st_body, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                                    cudaStreamCaptureModeThreadLocal));
        uint64_t b0 = launch_total();
        benqueue_rebuild(b, b->st_body);
        b->body_launches = launch_total() - b0;
        note_launch(0);
        cudaGraph_t tmp;
        GBMD_CUDA_TRY(cudaStreamEndCapture(b->st_body, &tmp));
        GBMD_CUDA_TRY(cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
        if (force) benqueue_force(b, s);
    }
    cudaGraph_t graph;
    cudaError_t err = cudaStreamEndCapture(s, &graph);
    b->cur = saved;
    if (err != cudaSuccess) return fail(GBMD_E_CUDA, std::string("graph capture: ") + cudaGetErrorString(err));
    err = cudaGraphInstantiate(out, graph, 0);
    cudaGraphDestroy(graph);
    if (err != cudaSuccess) return fail(GBMD_E_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(err));
    *launches = launch_total() - l0 - count * b->body_launches;
    note_launch(0);
    return GBMD_OK;
}

int brun(gbmd_batch* b, int which) {
    int parity = b->cur;
    uint32_t count = which ? b->block_steps : 1;
    if (!b->exec[parity][which]) GBMD_TRY(bcapture(b, parity, count, &b->exec[parity][which], &b->exec_launches[parity][which]));
    GBMD_CUDA_TRY(cudaGraphLaunch(b->exec[parity][which], b->st));
    b->launches += b->exec_launches[parity][which];
    if (count & 1) b->cur ^= 1;
    return GBMD_OK;
}

// The per-system observables of gbmd_observe over the batch's Verlet lists (IntEngine::energy's
// on-step kinetic energy, the pair potential and virial): the list path of k_kicks with the
// system's own parameter block. Each block takes one tile of one system's slots and writes its
// partial sums (potential, virial, kinetic), which the host adds per system in tile order.
template <int D, bool MULTI>
__global__ void __launch_bounds__(128) k_bframe(const Params* __restrict__ tab, const uint4* __restrict__ tiles, const PosRec<D>* __restrict__ pos,
                                                const uint32_t* __restrict__ species, const uint32_t* __restrict__ nbr,
                                                const uint32_t* __restrict__ nbr_count, const int32_t* __restrict__ vel,
                                                double* __restrict__ partial) {
    __shared__ double sh[4][4];
    const uint4 t = tiles[blockIdx.x];
    const Params& P = tab[t.x];
    double pe = 0.0, w = 0.0, ke = 0.0, gpe = 0.0;
    if (threadIdx.x < t.z) {
        const uint32_t i = t.y + threadIdx.x;
        int64_t xi[3];
        const uint32_t si = load_particle<D, MULTI>(pos, species, i, xi);
        const float cs = P.kick_cs[si];
        int32_t k[3] = {0, 0, 0};
        F32Sum pe32, w32;
        const uint32_t m = nbr_count[i], cap4 = (P.cap + 3u) & ~3u;
        for (uint32_t q = 0; q < m; q++) {
            const uint32_t j = nbr[list_slot(i, q, cap4)] & LIST_MASK;
            int64_t xj[3];
            const uint32_t sj = load_particle<D, MULTI>(pos, species, j, xj);
            const PairC& pc = P.pc[si * P.ns + sj];
            float fr, s6, r2;
            if (pair_kick<D>(P, pc, cs, xi, xj, k, fr, s6, r2)) {
                pe32.add(pair_u(pc, s6));
                w32.add(__fmul_rn(fr, r2));
            }
        }
        pe = 0.5 * pe32.value();
        w = 0.5 * w32.value();
        // the kinetic energy as k_kicks sums it (m (v + next)^2, scaled on the host), and gravity's
        // potential in its own partial
        const double m_i = P.masses[si];
        const bool counted = !(D == 3 && ((P.pinned >> si) & 1u));
        for (int a = 0; a < D; a++) {
            const int32_t v0 = vel[D * i + a];
            const int32_t next = wadd(wadd(v0, k[a]), P.gravity[a]);
            const double sv = (double)((int64_t)v0 + (int64_t)next);
            if (counted) {
                ke = __fma_rn(__dmul_rn(m_i, sv), sv, ke);
                if (P.grav_f[a] != 0.0) gpe = __fma_rn(-__dmul_rn(m_i, P.grav_f[a]), to_f64(wrap(xi[a], P.box[a])), gpe);
            }
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double vals[4] = {pe, w, ke, gpe};
    for (int q = 0; q < 4; q++) {
        double x = vals[q];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) sh[q][warp] = x;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double s = 0.0;
        for (int wq = 0; wq < (int)(blockDim.x >> 5); wq++) s += sh[threadIdx.x][wq];
        partial[4 * blockIdx.x + threadIdx.x] = s;
    }
}

// Per-system RDF counts (unordered pairs, each once: slot j > slot i; floor(r bins / rmax) of
// the exact minimum-image separation, rdf_bin) over the cells of the last list build. Every
// particle is within half the skin of the position it was binned at, so a pair within rmax has
// binned positions within rmax + skin: its cells differ by at most R = ceil((rmax + skin) nc / L)
// per axis (every cell of an axis with 2R + 1 >= nc, each once); `reach` holds R per system (8
// bits per axis; 255 stands for any reach of 255 or more, and walks every cell). Each block counts one tile of one system; each warp into its own shared
// histogram when `bins` allows (`per_warp`), then the block adds its counts to that system's bins.
template <int D>
__global__ void __launch_bounds__(128) k_brdf(const Params* __restrict__ tab, const uint4* __restrict__ tiles, const PosRec<D>* __restrict__ pos,
                                              const uint32_t* __restrict__ keys, const uint32_t* __restrict__ start,
                                              const uint32_t* __restrict__ reach, uint32_t bins, bool per_warp, double scale, float scalef,
                                              float lim2f, float margin, unsigned long long* __restrict__ out) {
    extern __shared__ uint32_t h[];
    const uint32_t nh = per_warp ? (blockDim.x >> 5) : 1u;
    for (uint32_t b = threadIdx.x; b < bins * nh; b += blockDim.x) h[b] = 0;
    __syncthreads();
    uint32_t* hw = per_warp ? h + (threadIdx.x >> 5) * bins : h;
    const uint4 t = tiles[blockIdx.x];
    const Params& P = tab[t.x];
    if (threadIdx.x < t.z) {
        const uint32_t i = t.y + threadIdx.x;
        int64_t xi[3] = {0, 0, 0};
        load_particle<D, false>(pos, nullptr, i, xi);
#pragma unroll
        for (int a = 0; a < D; a++) xi[a] = wrap(xi[a], P.box[a]);
        uint32_t c[3] = {0, 0, 0}, lo[3] = {0, 0, 0}, span[3] = {1, 1, 1};
        cell_coords(P, keys[i] - P.cell_base, c);
        const uint32_t rr = reach[t.x];
#pragma unroll
        for (int a = 0; a < D; a++) {
            const uint32_t nc = P.nc[a], R = (rr >> (8 * a)) & 255u;
            if (R == 255u || 2 * R + 1 >= nc) { // (255: a reach beyond 8 bits, every cell)
                lo[a] = 0;
                span[a] = nc;
            } else {
                lo[a] = c[a] + nc - R;
                span[a] = 2 * R + 1;
            }
        }
        for (uint32_t oz = 0; oz < span[2]; oz++) {
            const uint32_t z = D == 3 ? (lo[2] + oz) % P.nc[2] : 0u;
            for (uint32_t oy = 0; oy < span[1]; oy++) {
                const uint32_t y = (lo[1] + oy) % P.nc[1];
                for (uint32_t ox = 0; ox < span[0]; ox++) {
                    const uint32_t x = (lo[0] + ox) % P.nc[0];
                    const uint32_t cell = P.cell_base + (z * P.nc[1] + y) * P.nc[0] + x;
                    const uint32_t j1 = start[cell + 1];
                    for (uint32_t j = max(start[cell], i + 1); j < j1; j++) {
                        int64_t xj[3] = {0, 0, 0}, d[3] = {0, 0, 0};
                        load_particle<D, false>(pos, nullptr, j, xj);
#pragma unroll
                        for (int a = 0; a < D; a++) d[a] = min_image(wrap(xj[a], P.box[a]) - xi[a], P.box[a], P.half[a]);
                        const int k = rdf_bin<D>(d, bins, scale, scalef, lim2f, margin);
                        if (k >= 0) atomicAdd(&hw[k], 1u);
                    }
                }
            }
        }
    }
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < bins; b += blockDim.x) {
        uint32_t v = 0;
        for (uint32_t q = 0; q < nh; q++) v += h[q * bins + b];
        if (v) atomicAdd(out + (size_t)t.x * bins + b, (unsigned long long)v);
    }
}

int bcheck(gbmd_batch* b) {
    uint32_t c[3];
    GBMD_CUDA_TRY(cudaMemcpyAsync(c, b->ctl, 12, cudaMemcpyDeviceToHost, b->st));
    GBMD_CUDA_TRY(cudaStreamSynchronize(b->st));
    if (c[1]) {
        b->failed = true;
        return fail(GBMD_E_OVERFLOW, "a Verlet list of the batch overflowed its capacity");
    }
    return GBMD_OK;
}

} // namespace

extern "C" int gbmd_batch_create(const gbmd_system* systems, uint32_t count, const uint32_t* offsets, const int64_t* pos,
                                 const int32_t* vel, const uint32_t* species, const gbmd_options* opts, gbmd_batch** out);

namespace {

// One autotuner trial: a batch with options t from the caller's state, timed with CUDA events
// over its second block of steps (the first captures the graphs and warms up).
int time_trial(const gbmd_system* systems, uint32_t count, const uint32_t* offsets, const int64_t* pos, const int32_t* vel,
               const uint32_t* species, const gbmd_options& t, float* ms) {
    gbmd_batch* tb = nullptr;
    int r = gbmd_batch_create(systems, count, offsets, pos, vel, species, &t, &tb);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (r == GBMD_OK) r = gbmd_batch_step(tb, t.block_steps);
    if (r == GBMD_OK) r = gbmd_batch_sync(tb);
    if (r == GBMD_OK && (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)) r = fail(GBMD_E_CUDA, "cudaEventCreate");
    if (r == GBMD_OK && cudaEventRecord(e0, tb->st) != cudaSuccess) r = fail(GBMD_E_CUDA, "cudaEventRecord");
    if (r == GBMD_OK) r = gbmd_batch_step(tb, t.block_steps);
    if (r == GBMD_OK && cudaEventRecord(e1, tb->st) != cudaSuccess) r = fail(GBMD_E_CUDA, "cudaEventRecord");
    if (r == GBMD_OK) r = gbmd_batch_sync(tb);
    if (r == GBMD_OK && cudaEventElapsedTime(ms, e0, e1) != cudaSuccess) r = fail(GBMD_E_CUDA, "cudaEventElapsedTime");
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (tb) gbmd_batch_destroy(tb);
    return r;
}

// The autotuner: the rebuild cadence (the skin, one trial per candidate with one force lane per
// particle), then the neighbours per warp (1, 2 or 4 lanes per particle at that skin). A
// candidate whose lists overflow a fixed capacity, or that does not fit in memory, drops out.
// Sets o.skin and o's force lanes to the fastest and clears the flag.
int tune_skin(const gbmd_system* systems, uint32_t count, const uint32_t* offsets, const int64_t* pos, const int32_t* vel,
              const uint32_t* species, gbmd_options& o) {
    static const double cand[] = {0.3, 0.4, 0.5, 0.6, 0.7};
    o.flags &= ~GBMD_FLAG_TUNE_SKIN;
    gbmd_options t = o;
    t.block_steps = std::min<uint32_t>(o.block_steps ? o.block_steps : 100, 100);
    double best = 0.0;
    float best_ms = 0.0f;
    int last = GBMD_OK;
    std::string last_msg;
    t.flags = (o.flags & ~(31u << 8)) | GBMD_FLAG_FORCE_LANES(1);
    for (double sk : cand) {
        t.skin = sk;
        float ms = 0.0f;
        int r = time_trial(systems, count, offsets, pos, vel, species, t, &ms);
        if (r == GBMD_OK && (best == 0.0 || ms < best_ms)) best = sk, best_ms = ms;
        if (r != GBMD_OK) {
            if (r != GBMD_E_OVERFLOW && r != GBMD_E_NOMEM) return r;
            last = r;
            last_msg = gbmd_last_error();
        }
    }
    if (best == 0.0) return fail(last, "skin tuning: no candidate ran (" + last_msg + ")");
    // then the force lanes per particle (neighbours per warp) at that skin
    uint32_t best_s = 1;
    for (uint32_t S : {2u, 4u}) {
        t.skin = best;
        t.flags = (o.flags & ~(31u << 8)) | GBMD_FLAG_FORCE_LANES(S);
        float ms = 0.0f;
        int r = time_trial(systems, count, offsets, pos, vel, species, t, &ms);
        if (r == GBMD_OK && ms < best_ms) best_s = S, best_ms = ms;
        if (r != GBMD_OK && r != GBMD_E_OVERFLOW && r != GBMD_E_NOMEM) return r;
    }
    o.skin = best;
    o.flags = (o.flags & ~(31u << 8)) | GBMD_FLAG_FORCE_LANES(best_s);
    return GBMD_OK;
}

} // namespace

extern "C" {

int gbmd_batch_create(const gbmd_system* systems, uint32_t count, const uint32_t* offsets, const int64_t* pos, const int32_t* vel,
                      const uint32_t* species, const gbmd_options* opts, gbmd_batch** out) {
    if (!systems || !offsets || !pos || !vel || !species || !out || count == 0) return fail(GBMD_E_INVALID, "null argument");
    *out = nullptr;
    gbmd_options o{};
    if (opts) o = *opts;
    if (o.arith != GBMD_ARITH_F32) return fail(GBMD_E_UNSUPPORTED, "batches run f32 pair forces");
    if (o.mode == GBMD_MODE_CELLS) return fail(GBMD_E_UNSUPPORTED, "batches run Verlet lists");
    uint32_t D = systems[0].dim;
    for (uint32_t k = 0; k < count; k++) {
        GBMD_TRY(validate_system(systems[k], offsets[k + 1] - offsets[k]));
        if ((systems[k].periodic & ((1u << systems[k].dim) - 1u)) != ((1u << systems[k].dim) - 1u))
            return fail(GBMD_E_UNSUPPORTED, "batches hold periodic systems only (walls run on a plain engine)");
        if (systems[k].dim != D) return fail(GBMD_E_INVALID, "a batch holds systems of one dimension");
        if (offsets[k + 1] <= offsets[k]) return fail(GBMD_E_INVALID, "every system needs at least one particle");
    }
    if (offsets[0] != 0) return fail(GBMD_E_INVALID, "offsets[0] must be 0");
    if (o.flags & GBMD_FLAG_TUNE_SKIN) GBMD_TRY(tune_skin(systems, count, offsets, pos, vel, species, o));
    auto* b = new gbmd_batch;
    b->K = count;
    b->N = offsets[count];
    b->D = (int)D;
    b->rec = D == 2 ? 16 : 32;
    b->sys.assign(systems, systems + count);
    b->offsets.assign(offsets, offsets + count + 1);
    b->block_steps = o.block_steps ? o.block_steps : 100;
    double skin = o.skin > 0 ? o.skin : 0.4;
    b->skin = skin;
    b->P.resize(count);
    uint64_t cell_base = 0;
    for (uint32_t k = 0; k < count; k++) {
        const gbmd_system& s = systems[k];
        if (s.nspecies > 1) b->multi = true;
        uint32_t nk = offsets[k + 1] - offsets[k];
        uint32_t nc[3];
        int r = cells_for(s, rc_max(s) + skin, nc);
        if (r != GBMD_OK) {
            delete b;
            return r;
        }
        double vol = 1.0, rr = rc_max(s) + skin;
        for (uint32_t a = 0; a < D; a++) vol *= (double)s.box_len[a] * (1.0 / 4294967296.0);
        double sphere = D == 2 ? M_PI * rr * rr : 4.0 / 3.0 * M_PI * rr * rr * rr;
        uint32_t cap = o.cap ? o.cap : (uint32_t)std::ceil(sphere * std::max(2.0 * nk / vol, 1.2)) + 8;
        b->cap = std::max(b->cap, cap);
        fill_params(b->P[k], s, nk, skin, cap, nc);
        b->P[k].cell_base = (uint32_t)cell_base;
        b->P[k].id_base = offsets[k];
        if (s.bath) b->bath = true;
        cell_base += b->P[k].ncell;
        if (cell_base >= UINT32_MAX) {
            delete b;
            return fail(GBMD_E_INVALID, "too many cells in the batch");
        }
    }
    for (uint32_t k = 0; k < count; k++) b->P[k].cap = b->cap;
    b->ncell = (uint32_t)cell_base;
    b->bits = (uint32_t)key_bits(b->ncell);
    int dev_sms = 0;
    int r = GBMD_OK;
    auto step = [&](int rc) {
        if (r == GBMD_OK) r = rc;
    };
    step(cudaSetDevice(o.device) == cudaSuccess ? GBMD_OK : fail(GBMD_E_CUDA, "cudaSetDevice"));
    cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, o.device);
    int occ = 0;
    // every pair type of every system with sigma = 1: the packed chain with sigma compiled in
    b->sig1 = !b->multi;
    for (uint32_t k = 0; k < count; k++)
        for (uint32_t q = 0; q < b->P[k].ns * b->P[k].ns; q++) b->sig1 = b->sig1 && b->P[k].pc[q].sigma2s == 0x1p56f;
    // lanes per particle of the force step (1, 2 or 4; the autotuner's or the caller's choice)
    {
        const uint32_t fl = (o.flags >> 8) & 31u;
        b->S = fl == 2u || fl == 4u ? fl : 1u;
    }
    // the persistent grid: as many blocks as stay resident for the variant that will run
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, bforce_kernel_of((int)D, b->multi, b->sig1, b->S), 128, 0);
    b->grid = std::max<uint32_t>(1, std::min<uint32_t>(nblocks(b->N, 128), (uint32_t)std::max(dev_sms, 1) * (uint32_t)std::max(occ, 1)));
    if (r == GBMD_OK && cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) != cudaSuccess) r = fail(GBMD_E_CUDA, "stream");
    if (r == GBMD_OK && cudaStreamCreateWithFlags(&b->st_body, cudaStreamNonBlocking) != cudaSuccess) r = fail(GBMD_E_CUDA, "stream");
    size_t N = b->N;
    step(balloc(&b->tab, count, b->st));
    step(balloc((char**)&b->pos[0], N * b->rec, b->st));
    step(balloc((char**)&b->pos[1], N * b->rec, b->st));
    step(balloc((char**)&b->pos_scr, N * b->rec, b->st));
    step(balloc((char**)&b->ref_pos, N * b->rec, b->st));
    step(balloc(&b->vel, N * D, b->st));
    step(balloc(&b->vel_scr, N * D, b->st));
    step(balloc(&b->species, N, b->st));
    step(balloc(&b->species_scr, N, b->st));
    step(balloc(&b->ids, N, b->st));
    step(balloc(&b->ids_scr, N, b->st));
    step(balloc(&b->sysidx, N, b->st));
    step(balloc(&b->sysidx_scr, N, b->st));
    for (int k = 0; k < 2; k++) {
        step(balloc(&b->keys[k], N, b->st));
        step(balloc(&b->vals[k], N, b->st));
    }
    size_t hist_n = radix_hist_elems(N);
    step(balloc(&b->hist, hist_n, b->st));
    step(balloc(&b->scan_tmp, std::max(scan_tmp_elems(hist_n), scan_tmp_elems(N)), b->st));
    step(balloc(&b->start, (size_t)b->ncell + 1, b->st));
    step(balloc(&b->nbr, (N + 31) / 32 * 32 * (((size_t)b->cap + 3) & ~(size_t)3), b->st)); // warp-tiled (list_slot)
    step(balloc(&b->qpos[0], N, b->st));
    step(balloc(&b->relf, N, b->st));
    step(balloc(&b->qpos[1], N, b->st));
    step(balloc(&b->nbr_count, N, b->st));
    step(balloc(&b->ctl, 16, b->st));
    step(balloc(&b->ledger, 2 * (size_t)count, b->st));
    for (uint32_t k = 0; k < count; k++) // frame tiles: up to 128 slots of one system each
        for (uint32_t s0 = offsets[k]; s0 < offsets[k + 1]; s0 += 128)
            b->tiles_h.push_back(make_uint4(k, s0, std::min<uint32_t>(128u, offsets[k + 1] - s0), 0u));
    step(balloc(&b->tiles, b->tiles_h.size(), b->st));
    step(balloc(&b->part, 4 * b->tiles_h.size(), b->st));
    step(balloc(&b->reach, count, b->st));
    if (r == GBMD_OK)
        cudaMemcpyAsync(b->tiles, b->tiles_h.data(), b->tiles_h.size() * sizeof(uint4), cudaMemcpyHostToDevice, b->st);
    if (r == GBMD_OK) cudaMemsetAsync(b->ledger, 0, 16 * (size_t)count, b->st);
    step(balloc((char**)&b->staging, N * D * 8, b->st));
    step(balloc(&b->staging_v, N * D, b->st));
    step(balloc(&b->staging_s, N, b->st));
    if (r == GBMD_OK) {
        std::vector<uint32_t> sysi(N);
        for (uint32_t k = 0; k < count; k++)
            for (uint32_t i = offsets[k]; i < offsets[k + 1]; i++) sysi[i] = k;
        for (size_t i = 0; i < N; i++) {
            uint32_t k = sysi[i];
            if (species[i] >= systems[k].nspecies) r = fail(GBMD_E_INVALID, "species index out of range");
            for (uint32_t a = 0; a < D; a++)
                if (pos[D * i + a] < 0 || pos[D * i + a] >= systems[k].box_len[a]) r = fail(GBMD_E_INVALID, "positions must lie in [0, L)");
        }
        uint32_t* dsys = nullptr;
        if (r == GBMD_OK) step(balloc(&dsys, N, b->st));
        if (r == GBMD_OK) {
            cudaMemcpyAsync(b->tab, b->P.data(), count * sizeof(Params), cudaMemcpyHostToDevice, b->st);
            cudaMemcpyAsync(b->staging, pos, N * D * 8, cudaMemcpyHostToDevice, b->st);
            cudaMemcpyAsync(b->staging_v, vel, N * D * 4, cudaMemcpyHostToDevice, b->st);
            cudaMemcpyAsync(b->staging_s, species, N * 4, cudaMemcpyHostToDevice, b->st);
            cudaMemcpyAsync(dsys, sysi.data(), N * 4, cudaMemcpyHostToDevice, b->st);
            if (D == 2)
                k_bfrom_host<2><<<nblocks(N, 256), 256, 0, b->st>>>((uint32_t)N, (const int64_t*)b->staging, b->staging_v, b->staging_s, dsys,
                                                                   (PosRec<2>*)b->pos[0], b->vel, b->species, b->ids, b->sysidx);
            else
                k_bfrom_host<3><<<nblocks(N, 256), 256, 0, b->st>>>((uint32_t)N, (const int64_t*)b->staging, b->staging_v, b->staging_s, dsys,
                                                                   (PosRec<3>*)b->pos[0], b->vel, b->species, b->ids, b->sysidx);
            note_launch();
            cudaMemsetAsync(b->ctl, 0, 64, b->st);
            uint32_t one = 1;
            cudaMemcpyAsync(b->ctl, &one, 4, cudaMemcpyHostToDevice, b->st);
            cudaError_t e = cudaStreamSynchronize(b->st);
            if (e != cudaSuccess) r = fail(GBMD_E_CUDA, cudaGetErrorString(e));
        }
        if (dsys) cudaFreeAsync(dsys, b->st);
    }
    if (r != GBMD_OK) {
        std::string msg = gbmd_last_error();
        bfree(b);
        delete b;
        return fail(r, msg);
    }
    *out = b;
    return GBMD_OK;
}

int gbmd_batch_step(gbmd_batch* b, uint64_t steps) {
    if (!b) return fail(GBMD_E_INVALID, "null batch");
    if (b->failed) return fail(GBMD_E_OVERFLOW, "the batch is in a failed state (a list overflowed)");
    if (b->obs_pending) return fail(GBMD_E_INVALID, "a frame is in flight (gbmd_batch_observe_end first)");
    b->steps += steps;
    uint64_t left = steps;
    while (left >= b->block_steps) {
        GBMD_TRY(brun(b, 1));
        left -= b->block_steps;
    }
    while (left--) GBMD_TRY(brun(b, 0));
    GBMD_CUDA_TRY(cudaGetLastError());
    return GBMD_OK;
}

int gbmd_batch_time_phases(gbmd_batch* b, uint32_t steps, double* force_ms, double* rebuild_ms, uint32_t* rebuilds) {
    if (!b) return fail(GBMD_E_INVALID, "null batch");
    if (b->failed) return fail(GBMD_E_OVERFLOW, "the batch is in a failed state (a list overflowed)");
    GBMD_CUDA_TRY(cudaStreamSynchronize(b->st));
    cudaEvent_t e0, e1, e2;
    GBMD_CUDA_TRY(cudaEventCreate(&e0));
    GBMD_CUDA_TRY(cudaEventCreate(&e1));
    GBMD_CUDA_TRY(cudaEventCreate(&e2));
    double tf = 0.0, tr = 0.0;
    uint32_t nr = 0;
    const uint64_t l0 = launch_total();
    for (uint32_t k = 0; k < steps; k++) {
        uint32_t flag = 0;
        GBMD_CUDA_TRY(cudaMemcpyAsync(&flag, b->ctl, 4, cudaMemcpyDeviceToHost, b->st));
        GBMD_CUDA_TRY(cudaStreamSynchronize(b->st));
        GBMD_CUDA_TRY(cudaEventRecord(e0, b->st));
        if (flag) {
            benqueue_rebuild(b, b->st);
            nr++;
        }
        GBMD_CUDA_TRY(cudaEventRecord(e1, b->st));
        benqueue_force(b, b->st);
        GBMD_CUDA_TRY(cudaEventRecord(e2, b->st));
        GBMD_CUDA_TRY(cudaEventSynchronize(e2));
        float m1 = 0.f, m2 = 0.f;
        cudaEventElapsedTime(&m1, e0, e1);
        cudaEventElapsedTime(&m2, e1, e2);
        if (flag) tr += m1;
        tf += m2;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaEventDestroy(e2);
    // (gbmd_batch_stats counts each rebuild's kernels from the device's rebuild count)
    b->launches += launch_total() - l0 - (uint64_t)nr * b->body_launches;
    if (force_ms) *force_ms = steps ? tf / steps : 0.0;
    if (rebuild_ms) *rebuild_ms = nr ? tr / nr : 0.0;
    if (rebuilds) *rebuilds = nr;
    GBMD_CUDA_TRY(cudaGetLastError());
    return bcheck(b);
}

int gbmd_batch_observe_begin(gbmd_batch* b, uint32_t rdf_bins, double rdf_rmax) {
    if (!b) return fail(GBMD_E_INVALID, "null batch");
    if (b->obs_pending) return fail(GBMD_E_INVALID, "a frame is already in flight (gbmd_batch_observe_end first)");
    if (rdf_bins && (rdf_bins > 8192 || !(rdf_rmax > 0.0))) return fail(GBMD_E_INVALID, "bad RDF arguments");
    const int parity = b->cur;
    if (!b->exec_prep[parity]) GBMD_TRY(bcapture(b, parity, 1, &b->exec_prep[parity], &b->exec_prep_launches[parity], false));
    GBMD_CUDA_TRY(cudaGraphLaunch(b->exec_prep[parity], b->st)); // the lists and cells, rebuilt if the trigger is set
    b->launches += b->exec_prep_launches[parity];
    const uint32_t nt = (uint32_t)b->tiles_h.size();
    if (b->D == 2) {
        if (b->multi)
            k_bframe<2, true><<<nt, 128, 0, b->st>>>(b->tab, b->tiles, (const PosRec<2>*)b->pos[b->cur], b->species, b->nbr, b->nbr_count, b->vel, b->part);
        else
            k_bframe<2, false><<<nt, 128, 0, b->st>>>(b->tab, b->tiles, (const PosRec<2>*)b->pos[b->cur], b->species, b->nbr, b->nbr_count, b->vel, b->part);
    } else {
        if (b->multi)
            k_bframe<3, true><<<nt, 128, 0, b->st>>>(b->tab, b->tiles, (const PosRec<3>*)b->pos[b->cur], b->species, b->nbr, b->nbr_count, b->vel, b->part);
        else
            k_bframe<3, false><<<nt, 128, 0, b->st>>>(b->tab, b->tiles, (const PosRec<3>*)b->pos[b->cur], b->species, b->nbr, b->nbr_count, b->vel, b->part);
    }
    note_launch();
    if (!b->part_h) {
        b->part_h = (double*)pinned_alloc(4 * (size_t)nt * 8, &b->part_h_cap);
        if (!b->part_h) return fail(GBMD_E_NOMEM, "pinned frame buffer");
    }
    GBMD_CUDA_TRY(cudaMemcpyAsync(b->part_h, b->part, 4 * (size_t)nt * 8, cudaMemcpyDeviceToHost, b->st));
    if (rdf_bins) {
        const size_t nbins = (size_t)rdf_bins * b->K;
        if (nbins > b->obs_bins_cap) {
            if (b->obs_bins) GBMD_CUDA_TRY(cudaFreeAsync(b->obs_bins, b->st));
            b->obs_bins = nullptr;
            b->obs_bins_cap = 0;
            GBMD_TRY(balloc(&b->obs_bins, nbins, b->st));
            b->obs_bins_cap = nbins;
        }
        if (nbins * 8 > b->bins_h_cap) {
            pinned_release(b->bins_h, b->bins_h_cap);
            b->bins_h = (unsigned long long*)pinned_alloc(nbins * 8, &b->bins_h_cap);
            if (!b->bins_h) return fail(GBMD_E_NOMEM, "pinned RDF buffer");
        }
        GBMD_CUDA_TRY(cudaMemsetAsync(b->obs_bins, 0, nbins * 8, b->st));
        if (b->reach_for != rdf_rmax) { // R = ceil((rmax + skin) nc / L) per system and axis
            std::vector<uint32_t> rr(b->K, 0);
            for (uint32_t k = 0; k < b->K; k++)
                for (int a = 0; a < b->D; a++) {
                    const double L = (double)b->sys[k].box_len[a] * (1.0 / 4294967296.0);
                    const double R = std::ceil((rdf_rmax + b->skin) * b->P[k].nc[a] / L + 1e-9);
                    rr[k] |= (uint32_t)std::min(R, 255.0) << (8 * a);
                }
            GBMD_CUDA_TRY(cudaMemcpyAsync(b->reach, rr.data(), b->K * 4, cudaMemcpyHostToDevice, b->st));
            GBMD_CUDA_TRY(cudaStreamSynchronize(b->st)); // (rr leaves scope)
            b->reach_for = rdf_rmax;
        }
        const double scale = (double)rdf_bins / rdf_rmax;
        const float scalef = (float)scale, lim2f = (float)(rdf_rmax * rdf_rmax * (1.0 + 1e-4));
        const float margin = (float)(1e-6 * rdf_bins + 1e-5);
        const bool per_warp = rdf_bins <= 2048; // four histograms of 8 KB at most
        const size_t shm = (size_t)rdf_bins * 4 * (per_warp ? 4 : 1);
        if (b->D == 2)
            k_brdf<2><<<nt, 128, shm, b->st>>>(b->tab, b->tiles, (const PosRec<2>*)b->pos[b->cur], b->keys[b->sorted], b->start, b->reach,
                                               rdf_bins, per_warp, scale, scalef, lim2f, margin, b->obs_bins);
        else
            k_brdf<3><<<nt, 128, shm, b->st>>>(b->tab, b->tiles, (const PosRec<3>*)b->pos[b->cur], b->keys[b->sorted], b->start, b->reach,
                                               rdf_bins, per_warp, scale, scalef, lim2f, margin, b->obs_bins);
        note_launch();
        GBMD_CUDA_TRY(cudaMemcpyAsync(b->bins_h, b->obs_bins, nbins * 8, cudaMemcpyDeviceToHost, b->st));
    }
    GBMD_CUDA_TRY(cudaGetLastError());
    b->obs_pending = true;
    b->obs_nbins = rdf_bins;
    return GBMD_OK;
}

int gbmd_batch_observe_end(gbmd_batch* b, gbmd_frame* frames, uint64_t* rdf) {
    if (!b) return fail(GBMD_E_INVALID, "null batch");
    if (!b->obs_pending) return fail(GBMD_E_INVALID, "no frame in flight (gbmd_batch_observe_begin first)");
    b->obs_pending = false;
    GBMD_TRY(gbmd_batch_sync(b)); // returns at once when the frame's work is done
    if (rdf && b->obs_nbins) std::memcpy(rdf, b->bins_h, (size_t)b->obs_nbins * b->K * 8);
    if (!frames) return GBMD_OK;
    std::vector<double> pe(b->K, 0.0), w(b->K, 0.0), ke(b->K, 0.0), gpe(b->K, 0.0);
    for (size_t t = 0; t < b->tiles_h.size(); t++) { // per system, in tile order
        const uint32_t k = b->tiles_h[t].x;
        pe[k] += b->part_h[4 * t];
        w[k] += b->part_h[4 * t + 1];
        ke[k] += b->part_h[4 * t + 2];
        gpe[k] += b->part_h[4 * t + 3];
    }
    for (uint32_t k = 0; k < b->K; k++) { // as gbmd_observe_end
        ke[k] *= 0x1p-64 / (8.0 * b->sys[k].dt * b->sys[k].dt);
        pe[k] += gpe[k];
    }
    bool finite = true;
    for (uint32_t k = 0; k < b->K; k++) { // as gbmd_observe_end
        const gbmd_system& s = b->sys[k];
        const uint32_t n = b->offsets[k + 1] - b->offsets[k];
        double vol = 1.0;
        for (int a = 0; a < b->D; a++) vol *= (double)s.box_len[a] * (1.0 / 4294967296.0);
        const double dof = 0.5 * b->D * std::max((double)n - 1.0, 1.0);
        gbmd_frame& f = frames[k];
        f.step = b->steps;
        f.kinetic = ke[k];
        f.potential = pe[k];
        f.virial = w[k];
        f.temperature = ke[k] / dof;
        f.pressure = (double)n / vol * f.temperature + w[k] / (b->D * vol);
        f.volume = vol;
        f.n = n;
        f.dim = (uint32_t)b->D;
        finite = finite && std::isfinite(ke[k]) && std::isfinite(pe[k]) && std::isfinite(w[k]);
    }
    if (!finite) return fail(GBMD_E_NONFINITE, "a non-finite energy or virial (the frames are filled in)");
    return GBMD_OK;
}

int gbmd_batch_observe(gbmd_batch* b, gbmd_frame* frames, uint64_t* rdf, uint32_t rdf_bins, double rdf_rmax) {
    GBMD_TRY(gbmd_batch_observe_begin(b, rdf_bins, rdf_rmax));
    return gbmd_batch_observe_end(b, frames, rdf);
}

int gbmd_batch_set_clocks(gbmd_batch* b, const uint32_t* clocks) {
    if (!b || !clocks) return fail(GBMD_E_INVALID, "null argument");
    if (b->obs_pending) return fail(GBMD_E_INVALID, "a frame is in flight (gbmd_batch_observe_end first)");
    uint32_t c = 0;
    GBMD_CUDA_TRY(cudaMemcpyAsync(&c, b->ctl + CTL_CLOCK, 4, cudaMemcpyDeviceToHost, b->st));
    GBMD_CUDA_TRY(cudaStreamSynchronize(b->st));
    for (uint32_t k = 0; k < b->K; k++) b->P[k].clock_base = clocks[k] - c; // (wrapping, as the clock)
    GBMD_CUDA_TRY(cudaMemcpyAsync(b->tab, b->P.data(), b->K * sizeof(Params), cudaMemcpyHostToDevice, b->st));
    return gbmd_batch_sync(b);
}

int gbmd_batch_read_all(gbmd_batch* b, int64_t* pos, int32_t* vel, uint32_t* species) {
    if (!b) return fail(GBMD_E_INVALID, "null batch");
    size_t N = b->N, D = b->D;
    if (D == 2)
        k_bto_ids<2><<<nblocks(N, 256), 256, 0, b->st>>>((uint32_t)N, b->tab, b->sysidx, (const PosRec<2>*)b->pos[b->cur], b->vel,
                                                        b->species, b->ids, (int64_t*)b->staging, b->staging_v, b->staging_s);
    else
        k_bto_ids<3><<<nblocks(N, 256), 256, 0, b->st>>>((uint32_t)N, b->tab, b->sysidx, (const PosRec<3>*)b->pos[b->cur], b->vel,
                                                        b->species, b->ids, (int64_t*)b->staging, b->staging_v, b->staging_s);
    note_launch();
    if (pos) GBMD_CUDA_TRY(cudaMemcpyAsync(pos, b->staging, N * D * 8, cudaMemcpyDeviceToHost, b->st));
    if (vel) GBMD_CUDA_TRY(cudaMemcpyAsync(vel, b->staging_v, N * D * 4, cudaMemcpyDeviceToHost, b->st));
    if (species) GBMD_CUDA_TRY(cudaMemcpyAsync(species, b->staging_s, N * 4, cudaMemcpyDeviceToHost, b->st));
    return gbmd_batch_sync(b);
}

int gbmd_batch_sync(gbmd_batch* b) {
    if (!b) return fail(GBMD_E_INVALID, "null batch");
    GBMD_CUDA_TRY(cudaStreamSynchronize(b->st));
    return bcheck(b);
}

int gbmd_batch_read_system(gbmd_batch* b, uint32_t k, int64_t* pos, int32_t* vel, uint32_t* species) {
    if (!b || k >= b->K) return fail(GBMD_E_INVALID, "bad batch or system index");
    size_t N = b->N, D = b->D;
    if (D == 2)
        k_bto_ids<2><<<nblocks(N, 256), 256, 0, b->st>>>((uint32_t)N, b->tab, b->sysidx, (const PosRec<2>*)b->pos[b->cur], b->vel,
                                                        b->species, b->ids, (int64_t*)b->staging, b->staging_v, b->staging_s);
    else
        k_bto_ids<3><<<nblocks(N, 256), 256, 0, b->st>>>((uint32_t)N, b->tab, b->sysidx, (const PosRec<3>*)b->pos[b->cur], b->vel,
                                                        b->species, b->ids, (int64_t*)b->staging, b->staging_v, b->staging_s);
    note_launch();
    size_t o = b->offsets[k], n = b->offsets[k + 1] - o;
    if (pos) GBMD_CUDA_TRY(cudaMemcpyAsync(pos, (int64_t*)b->staging + o * D, n * D * 8, cudaMemcpyDeviceToHost, b->st));
    if (vel) GBMD_CUDA_TRY(cudaMemcpyAsync(vel, b->staging_v + o * D, n * D * 4, cudaMemcpyDeviceToHost, b->st));
    if (species) GBMD_CUDA_TRY(cudaMemcpyAsync(species, b->staging_s + o, n * 4, cudaMemcpyDeviceToHost, b->st));
    return gbmd_batch_sync(b);
}

int gbmd_batch_stream(gbmd_batch* b, void** stream) {
    if (!b || !stream) return fail(GBMD_E_INVALID, "null argument");
    *stream = (void*)b->st;
    return GBMD_OK;
}

int gbmd_batch_stats(gbmd_batch* b, uint64_t* launches, uint32_t* rebuilds) {
    if (!b) return fail(GBMD_E_INVALID, "null batch");
    uint32_t c[3];
    GBMD_CUDA_TRY(cudaMemcpyAsync(c, b->ctl, 12, cudaMemcpyDeviceToHost, b->st));
    GBMD_CUDA_TRY(cudaStreamSynchronize(b->st));
    if (rebuilds) *rebuilds = c[2];
    if (launches) *launches = b->launches + (uint64_t)c[2] * b->body_launches;
    return GBMD_OK;
}

int gbmd_batch_read_ledger(gbmd_batch* b, uint32_t k, double* energy, double* impulse, uint64_t* hits) {
    if (!b || k >= b->K) return fail(GBMD_E_INVALID, "bad batch or system index");
    unsigned long long l[2];
    GBMD_CUDA_TRY(cudaMemcpyAsync(l, b->ledger + 2 * (size_t)k, 16, cudaMemcpyDeviceToHost, b->st));
    GBMD_CUDA_TRY(cudaStreamSynchronize(b->st));
    for (int w = 0; w < GBMD_LEDGER_SLOTS; w++) {
        if (energy) energy[w] = w == GBMD_LEDGER_BATH ? (double)(long long)l[0] * (1.0 / 16777216.0) : 0.0;
        if (impulse) impulse[w] = 0.0;
        if (hits) hits[w] = w == GBMD_LEDGER_BATH ? (uint64_t)l[1] : 0;
    }
    return GBMD_OK;
}

int gbmd_batch_skin(gbmd_batch* b, double* skin) {
    if (!b || !skin) return fail(GBMD_E_INVALID, "null argument");
    *skin = b->skin;
    return GBMD_OK;
}

int gbmd_batch_force_lanes(gbmd_batch* b, uint32_t* lanes) {
    if (!b || !lanes) return fail(GBMD_E_INVALID, "null argument");
    *lanes = b->S;
    return GBMD_OK;
}

int gbmd_batch_destroy(gbmd_batch* b) {
    if (!b) return GBMD_OK;
    cudaStreamSynchronize(b->st);
    bfree(b);
    delete b;
    return GBMD_OK;
}

} // extern "C"
