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
#include "fdlibm.cuh"
#include "sort.cuh"

namespace gbmd {

template <int D> using PosRec = typename PosT<D>::T;

// Position and species of slot i. In 3D the species rides in the record's fourth word; in 2D it
// is read from `species` when the system has more than one.
// CG: load through L2 only (ld.global.cg), for arrays that other blocks write during the same
// launch (the persistent step loop); otherwise through the read-only path.
template <bool CG, class T> __device__ __forceinline__ T ld_in(const T* p) {
    if constexpr (CG) return __ldcg(p);
    else return __ldg(p);
}
template <int D, bool MULTI, bool CG = false>
__device__ __forceinline__ uint32_t load_particle(const PosRec<D>* pos, const uint32_t* species, uint32_t i, int64_t* x) {
    if constexpr (D == 2) {
        longlong2 v = ld_in<CG>(pos + i);
        x[0] = v.x;
        x[1] = v.y;
        return MULTI ? __ldg(species + i) : 0u;
    } else {
        const longlong2* q = reinterpret_cast<const longlong2*>(pos + i);
        longlong2 a = ld_in<CG>(q), b = ld_in<CG>(q + 1);
        x[0] = a.x;
        x[1] = a.y;
        x[2] = b.x;
        return MULTI ? (uint32_t)b.y : 0u;
    }
}

// Row-major cell key (md-ref cells.rs:10-15; int_engine3.rs:53-57) with f64 cell_of per axis.
template <int D> __device__ __forceinline__ uint32_t cell_key(const Params& P, const int64_t* x, uint32_t* c) {
    c[0] = cell_of_fast(x[0], P.box_f[0], P.nc[0], P.cell_scale_f[0], P.cell_delta[0]);
    c[1] = cell_of_fast(x[1], P.box_f[1], P.nc[1], P.cell_scale_f[1], P.cell_delta[1]);
    if constexpr (D == 2) {
        c[2] = 0;
        return c[1] * P.nc[0] + c[0];
    } else {
        c[2] = cell_of_fast(x[2], P.box_f[2], P.nc[2], P.cell_scale_f[2], P.cell_delta[2]);
        return (c[2] * P.nc[1] + c[1]) * P.nc[0] + c[0];
    }
}

// Slab of a particle's last coordinate inside its cell: floor(2^key_shift z_rel / cell_w) in f32,
// z_rel the offset from the cell's origin, clamped to [0, 2^key_shift). The list build relies on
// one property only: the slab does not decrease as z_rel grows.
__device__ __forceinline__ uint32_t sub_bucket(const Params& P, int64_t zrel) {
    const int b = __float2int_rd(__fmul_rn(__int2float_rn((int32_t)(zrel >> 8)), P.sub_scale));
    const int top = (1 << P.key_shift) - 1;
    return (uint32_t)(b < 0 ? 0 : (b > top ? top : b));
}

// Cell key of particle i; with key_shift > 0 (list builds) the key is cell << key_shift | slab.
template <int D> __device__ __forceinline__ uint32_t particle_key(const Params& P, const PosRec<D>* pos, uint32_t i) {
    int64_t x[3];
    load_particle<D, false>(pos, nullptr, i, x);
#pragma unroll
    for (int a = 0; a < D; a++) x[a] = wrap(x[a], P.box[a]);
    uint32_t c[3];
    uint32_t key = cell_key<D>(P, x, c);
    if (P.key_shift) key = (key << P.key_shift) | sub_bucket(P, x[D - 1] - (int64_t)c[D - 1] * P.cell_w[D - 1]);
    return key;
}
template <int D> __global__ void k_keys(Params P, const PosRec<D>* pos, uint32_t* keys, uint32_t* vals) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    keys[i] = particle_key<D>(P, pos, i);
    vals[i] = i;
}
// The keys fused with the first radix pass's histogram: block b keys the RADIX_TILE particles of
// tile b (rounds of 256) and counts their low 8 bits into hist[d tiles + b], the layout of the
// sort's own histogram kernel, which the sort then skips for that pass.
template <int D>
__global__ void __launch_bounds__(256) k_keys_hist(Params P, const PosRec<D>* pos, uint32_t* keys, uint32_t* vals, uint32_t* hist, uint32_t tiles) {
    __shared__ uint32_t cnt[256];
    cnt[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t base = blockIdx.x * RADIX_TILE;
    for (uint32_t r = 0; r < RADIX_TILE / 256; r++) {
        const uint32_t i = base + r * 256 + threadIdx.x;
        if (i < P.n) {
            const uint32_t key = particle_key<D>(P, pos, i);
            keys[i] = key;
            vals[i] = i;
            atomicAdd(&cnt[key & 255u], 1u);
        }
    }
    __syncthreads();
    hist[(size_t)threadIdx.x * tiles + blockIdx.x] = cnt[threadIdx.x];
}

__device__ __forceinline__ void cell_coords(const Params& P, uint32_t key, uint32_t* c);

// A small fixed-point offset (a few cells, |v| < 2^37) as f32 sigma for the list build's
// prefilter, through a 32-bit conversion of v >> 8 (2^-24 sigma units): the 64-bit conversion
// runs on the slow FP64 pipe. The error, ~1e-6 sigma, is far inside the prefilter's 1e-4 band.
__device__ __forceinline__ float off_f32(int64_t v) { return __fmul_rn(__int2float_rn((int32_t)(v >> 8)), 1.0f / 16777216.0f); }

// Storage permutation into cell order (one fused gather; reorder.wgsl's gathers + copy-backs).
// Also records each particle's position relative to its cell's origin (c * cell_w, an exact
// integer) as f32 sigma, with its species in the fourth word, for the list build's prefilter.
// With `start` given, also the cell starts of the sorted keys (as cell_starts: start[c] = first
// slot with key >= c, c in [0, nkeys]).
template <int D>
__global__ void k_gather(Params P, const uint32_t* items, const uint32_t* keys, const PosRec<D>* pos, const int32_t* vel,
                         const uint32_t* species, const uint32_t* ids, PosRec<D>* pos_o, int32_t* vel_o, uint32_t* species_o,
                         uint32_t* ids_o, float4* relf, uint32_t* start = nullptr, uint32_t nkeys = 0) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= P.n) return;
    if (start) {
        const uint32_t cur = keys[s];
        for (int64_t c = s == 0 ? 0 : (int64_t)keys[s - 1] + 1; c <= (int64_t)cur; c++) start[c] = s;
        if (s == P.n - 1)
            for (uint64_t c = (uint64_t)cur + 1; c <= nkeys; c++) start[c] = P.n;
    }
    uint32_t o = items[s];
    PosRec<D> r = pos[o];
    {
        long long* x = reinterpret_cast<long long*>(&r);
#pragma unroll
        for (int a = 0; a < D; a++) x[a] = wrap(x[a], P.box[a]);
    }
    pos_o[s] = r;
    for (uint32_t a = 0; a < D; a++) vel_o[D * s + a] = vel[D * o + a];
    uint32_t sp = species[o];
    species_o[s] = sp;
    ids_o[s] = ids[o];
    if (relf) {
        uint32_t c[3];
        cell_coords(P, keys[s] >> P.key_shift, c);
        const long long* x = reinterpret_cast<const long long*>(&r);
        float4 f;
        f.x = off_f32(x[0] - (int64_t)c[0] * P.cell_w[0]);
        f.y = off_f32(x[1] - (int64_t)c[1] * P.cell_w[1]);
        // (2D: the cell's x index, exact in f32, for the list build's row walk)
        f.z = D == 3 ? off_f32(x[2] - (int64_t)c[2] * P.cell_w[2]) : (float)c[0];
        f.w = __uint_as_float(sp);
        relf[s] = f;
    }
}

__device__ __forceinline__ int32_t wadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }

// ---------------------------------------------------------------- f32 sums with f64 accuracy
// An unevaluated sum hi + lo of two f32 (Knuth's TwoSum adds each term exactly): sums of f32 pair
// energies to about 2^-48 relative without f64 arithmetic, which runs at a small fraction of the
// f32 rate on this GPU. Every operation is an explicit round-to-nearest add (no fusion).
struct F32Sum {
    float hi = 0.0f, lo = 0.0f;
    __device__ __forceinline__ void add(float x) {
        const float s = __fadd_rn(hi, x), bb = __fsub_rn(s, hi);
        const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(x, bb));
        hi = s;
        lo = __fadd_rn(lo, err);
    }
    __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

// ---------------------------------------------------------------- all-integer table forces
// IntTables::kick (table.rs:76-105): d rounded to 2^-20 sigma per axis, r2 to 2^-24 sigma^2, the
// table's kick coefficient interpolated linearly between entries 2^12 apart in r2, and each
// axis's kick -t q >> 22 with the sign taken apart (the product fits 54 bits). Pure integer
// arithmetic: bit-identical on every device. Adds to k and returns true inside the cutoff.
template <int D>
__device__ __forceinline__ bool int_kick(const Params& P, uint32_t pair, const int64_t* d, int32_t* k) {
    const int64_t limit = (int64_t)8 << 32;
    int64_t q[3] = {0, 0, 0};
#pragma unroll
    for (int a = 0; a < D; a++)
        if (!(d[a] >= -limit && d[a] < limit)) return false;
    uint64_t sq = 0;
#pragma unroll
    for (int a = 0; a < D; a++) {
        const uint64_t ax = d[a] < 0 ? (uint64_t)0 - (uint64_t)d[a] : (uint64_t)d[a];
        const int64_t m = (int64_t)((ax + (1ull << 11)) >> 12);
        q[a] = d[a] < 0 ? -m : m;
        sq += (uint64_t)(q[a] * q[a]);
    }
    const uint32_t r2 = (uint32_t)((sq + (1ull << 15)) >> 16);
    if (r2 >= P.irc2[pair]) return false;
    const int32_t* tab = P.itab + (size_t)pair * P.itab_len;
    const int64_t t0 = __ldg(tab + (r2 >> 12)), t1 = __ldg(tab + (r2 >> 12) + 1);
    const int64_t t = t0 + (((t1 - t0) * (int64_t)(r2 & 4095u)) >> 12);
    const uint64_t at = t < 0 ? (uint64_t)0 - (uint64_t)t : (uint64_t)t;
#pragma unroll
    for (int a = 0; a < D; a++) {
        const uint64_t aq = q[a] < 0 ? (uint64_t)0 - (uint64_t)q[a] : (uint64_t)q[a];
        const int64_t m = (int64_t)((at * aq) >> 22);
        const bool neg = (t < 0) != (q[a] < 0);
        k[a] = (int32_t)((uint32_t)k[a] + (uint32_t)(neg ? m : -m));
    }
    return true;
}
// Pair::energy and f_over_r (pair.rs:36-51) in f64 at r2 in sigma^2: the instruments of the
// integer path (IntEngine::forces sums Pair::energy of the exact separations).
__device__ __forceinline__ void pair_f64(const double* c, double r2, double& u, double& fr) {
    const double eps = c[0], sigma = c[1], rc = c[2], shift = c[3];
    u = 0.0;
    fr = 0.0;
    if (r2 >= __dmul_rn(rc, rc)) return;
    const double y = __ddiv_rn(__dmul_rn(sigma, sigma), r2);
    const double s6 = __dmul_rn(y, __dmul_rn(y, y));
    u = __dsub_rn(__dmul_rn(__dmul_rn(__dmul_rn(4.0, eps), s6), __dsub_rn(s6, 1.0)), shift);
    fr = __ddiv_rn(__dmul_rn(__dmul_rn(__dmul_rn(24.0, eps), s6), __dsub_rn(__dmul_rn(2.0, s6), 1.0)), r2);
}

// Two directed pairs of one particle (single species, sigma = 1) in packed f32x2 arithmetic:
// the same roundings as two pair_fr + kick calls. A pair that is not valid (a slot past the list
// end) or beyond the cutoff gets a zero coefficient, and rint(0 f) adds nothing; a pack holding
// an in-range pair closer than sigma / 8 takes the scalar chain (pair_fr) for both.
template <int D>
__device__ __forceinline__ void pair_kicks2_sig1(const PairC& pc, float cs, const float* fa, const float* fb, bool va, bool vb, int32_t* k) {
    // r2 as sums of products: scalar (a packed mul feeding a packed add would be fused)
    float r2a = __fadd_rn(__fmul_rn(fa[0], fa[0]), __fmul_rn(fa[1], fa[1]));
    float r2b = __fadd_rn(__fmul_rn(fb[0], fb[0]), __fmul_rn(fb[1], fb[1]));
    if (D == 3) {
        r2a = __fadd_rn(r2a, __fmul_rn(fa[2], fa[2]));
        r2b = __fadd_rn(r2b, __fmul_rn(fb[2], fb[2]));
    }
    // (no early exit when both are beyond the cutoff: the warp runs the chain for its other lanes
    // anyway, and the branch cost 1.9%; such pairs get a zero coefficient below)
    const bool ina = va && r2a < pc.rc2s, inb = vb && r2b < pc.rc2s;
    if ((ina && !(r2a >= pc.fast_lo)) || (inb && !(r2b >= pc.fast_lo))) {
        const float* fs[2] = {fa, fb};
        const bool ins[2] = {ina, inb};
#pragma unroll
        for (int q = 0; q < 2; q++) {
            float fr, s6, rr;
            if (ins[q] && pair_fr<D, true>(pc, fs[q], fr, s6, rr)) {
                const float am = __fmul_rn(-fr, cs);
#pragma unroll
                for (int a = 0; a < D; a++) k[a] = wadd(k[a], rni_f32(__fmul_rn(am, fs[q][a])));
            }
        }
        return;
    }
    const f32x2 r2 = f2_pack(r2a, r2b), nr2 = f2_pack(-r2a, -r2b);
    const f32x2 y = rcp_cr2(r2, nr2);
    const f32x2 s2 = f2_mul(y, f2_pack(0x1p56f, 0x1p56f));
    const f32x2 s6 = f2_mul(f2_mul(s2, s2), s2);
    // 2 s6 - 1 as (s6 + s6) + (-1): s6 + s6 = 2 s6 exactly, and no mul feeds the add
    const f32x2 t = f2_mul(f2_mul(f2_pack(pc.c6, pc.c6), s6), f2_add(f2_add(s6, s6), f2_pack(-1.0f, -1.0f)));
    const f32x2 fr = div_cr2(t, nr2, y);
    float ama, amb;
    f2_unpack(f2_mul(fr, f2_pack(-cs, -cs)), ama, amb);
    const f32x2 am = f2_pack(ina ? ama : 0.0f, inb ? amb : 0.0f);
#pragma unroll
    for (int a = 0; a < D; a++) {
        float ka, kb;
        f2_unpack(f2_mul(am, f2_pack(fa[a], fb[a])), ka, kb);
        k[a] = wadd(k[a], wadd(rni_f32(ka), rni_f32(kb)));
    }
}

// One directed pair (i from j): adds the integer kick rint(a * f) per axis, exactly
// IntEngine::forces' `(a * fx).round_even().to_i32()` summed with wrapping adds.
template <int D, class G>
__device__ __forceinline__ bool pair_kick(const G& P, const PairC& pc, float cs, const int64_t* xi, const int64_t* xj, int32_t* k,
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
// With WRAP false the position is left unwrapped (the Verlet-list engine wraps at each list
// build and on read-back: wrap(wrap(x) + v) = wrap(x + v) while x stays within a box length).
template <int D, class G, bool WRAP = true>
__device__ __forceinline__ void leapfrog(const G& P, uint32_t si, const int32_t* k, int32_t* v, int64_t* x) {
    bool pinned = (P.pinned >> si) & 1u;
#pragma unroll
    for (int a = 0; a < D; a++) {
        v[a] = wadd(wadd(v[a], k[a]), pinned ? 0 : P.gravity[a]);
        // (a walled axis is not wrapped: a particle that left the box is mirrored after the step)
        x[a] = (WRAP && ((P.periodic >> a) & 1u)) ? wrap(x[a] + (int64_t)v[a], P.box[a]) : x[a] + (int64_t)v[a];
    }
}

// ---------------------------------------------------------------- the Andersen bath
// walls::andersen (walls.rs:113-133) with IntEngine's use of it (int_engine.rs:275-293) in 2D,
// three::andersen (three.rs:247-265) with int_engine3.rs:155-160 in 3D: Threefry on (id, clock)
// under the thermostat key decides, with probability rate dt, to replace the kicked velocity by a
// Maxwell draw at the bath's temperature (fdlibm ln, cos, sin in IEEE double, the reference's
// operation order), each component rounded by to_step_displacement; 2D adds the fan's drift to
// x and flow1 to y (the affine flow under a driven piston, int_engine.rs:282-286). The energy change 0.5 m (|v'|^2 - |v|^2), in the reference's f64 order, is booked on the
// ledger rounded half away from zero to 2^-24 epsilon, so the total does not depend on the order
// in which the GPU books events.
struct BathDraw {
    int32_t v[3];
    int hit;
};
template <int D>
__device__ __forceinline__ BathDraw bath_draw(uint32_t id, uint32_t clock, uint32_t k0, uint32_t k1, double rate_dt, double sd, double m,
                                           double dt, int32_t drift, int32_t flow1, int32_t v0, int32_t v1, int32_t v2,
                                           unsigned long long* ledger) {
    BathDraw o{{v0, v1, v2}, 0};
    uint32_t r0, r1;
    threefry2x32(id, clock, k0, k1, r0, r1);
    if (!(to_unit_f64(r0, 0u) < rate_dt)) return o;
    uint32_t q0, q1;
    threefry2x32(id, clock, k0, k1 ^ 1u, q0, q1);
    const double tau = 6.28318530717958647692;
    double u[3];
    {
        const double rad = __dsqrt_rn(__dmul_rn(-2.0, dev_log(__dsub_rn(1.0, to_unit_f64(r1, 0u)))));
        const double a = __dmul_rn(tau, to_unit_f64(q0, 0u));
        const double sr = __dmul_rn(sd, rad);
        u[0] = __dmul_rn(sr, dev_cos(a));
        u[1] = __dmul_rn(sr, dev_sin(a));
        u[2] = 0.0;
    }
    if (D == 3) {
        uint32_t w0, w1;
        threefry2x32(id, clock, k0, k1 ^ 2u, w0, w1);
        const double rad3 = __dsqrt_rn(__dmul_rn(-2.0, dev_log(__dsub_rn(1.0, to_unit_f64(w0, 0u)))));
        const double a3 = __dmul_rn(tau, to_unit_f64(w1, 0u));
        u[2] = __dmul_rn(__dmul_rn(sd, rad3), dev_cos(a3));
    }
    auto vel = [&](int32_t x) { return __ddiv_rn(__dmul_rn((double)x, 1.0 / 4294967296.0), dt); };
    auto step = [&](double x) { return sat_i32_f64(round_away(__dmul_rn(__dmul_rn(x, dt), 4294967296.0))); };
    const int32_t vin[3] = {v0, v1, v2};
    double de;
    if (D == 2) {
        const double b0 = vel(v0), b1 = vel(v1);
        o.v[0] = wadd(step(u[0]), drift);
        o.v[1] = wadd(step(u[1]), flow1);
        const double a0 = vel(o.v[0]), a1 = vel(o.v[1]);
        // 0.5 m (a0 a0 + a1 a1 - b0 b0 - b1 b1), left to right
        const double s = __dsub_rn(__dsub_rn(__dadd_rn(__dmul_rn(a0, a0), __dmul_rn(a1, a1)), __dmul_rn(b0, b0)), __dmul_rn(b1, b1));
        de = __dmul_rn(__dmul_rn(0.5, m), s);
    } else {
        double before = 0.0, after = 0.0;
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const double b = vel(vin[a]);
            before = __dadd_rn(before, __dmul_rn(b, b));
            o.v[a] = step(u[a]);
            const double c = vel(o.v[a]);
            after = __dadd_rn(after, __dmul_rn(c, c));
        }
        de = __dmul_rn(__dmul_rn(0.5, m), __dsub_rn(after, before));
    }
    atomicAdd(ledger, (unsigned long long)sat_i64_f64(round_away(__dmul_rn(de, 16777216.0))));
    atomicAdd(ledger + 1, 1ull);
    o.hit = 1;
    return o;
}

// The displacement trigger of integrate_list (neighbors.wgsl:90-100): has the particle moved
// half the skin since the list was built? (f32 separations; beyond 8 sigma counts as moved.)
template <int D, class G> __device__ __forceinline__ bool moved_half_skin(const G& P, const int64_t* ref, const int64_t* x) {
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

// A list entry is the neighbour's slot in its low LIST_BITS bits and, above, the periodic
// image the pair was found at (2 bits per axis: 1 for +L, 2 for -L), so that with positions left
// unwrapped between list builds the separation is xj + image - xi exactly, with no minimum image.
constexpr uint32_t LIST_BITS = 26;
constexpr uint32_t LIST_MASK = (1u << LIST_BITS) - 1u;
__device__ __forceinline__ uint32_t image_code(int64_t sx, int64_t sy, int64_t sz) {
    uint32_t c = (sx > 0 ? 1u : sx < 0 ? 2u : 0u) | (sy > 0 ? 4u : sy < 0 ? 8u : 0u) | (sz > 0 ? 16u : sz < 0 ? 32u : 0u);
    return c << LIST_BITS;
}

// Verlet lists are warp-tiled: the 32 particles of a warp (consecutive slots) store their
// neighbours in groups of four, group g of lane l at ((w cap4 + 4 g) 32 + 4 l), so one 16-byte
// load gives a thread four neighbours and a warp's load is 512 contiguous bytes. cap4 is the
// capacity rounded up to a multiple of 4.
__device__ __forceinline__ size_t list_slot(uint32_t i, uint32_t k, uint32_t cap4) {
    return ((size_t)(i >> 5) * cap4 + (k & ~3u)) * 32 + ((i & 31u) << 2) + (k & 3u);
}

// The quotient record of a position: the low 32 bits of x >> 4 per axis and the remainders
// x & 15 in bytes of the fourth word (species in its top byte). For two particles whose true
// separation d = xj - xi needs no periodic image and is below 8 sigma, D = Xj - Xi in wrapping
// 32-bit arithmetic is exact and d = 16 D + (Rj - Ri).
template <int D> __device__ __forceinline__ uint4 quot_record(const int64_t* x, uint32_t species) {
    uint4 r;
    r.x = (uint32_t)(x[0] >> 4);
    r.y = (uint32_t)(x[1] >> 4);
    r.z = D == 3 ? (uint32_t)(x[2] >> 4) : 0u;
    uint32_t w = (uint32_t)(x[0] & 15) | ((uint32_t)(x[1] & 15) << 8) | (species << 24);
    if (D == 3) w |= (uint32_t)(x[2] & 15) << 16;
    r.w = w;
    return r;
}
// sep_near from quotient records: trunc(d / 16) with d = 16 D + (rj - ri), 0 <= r < 16:
// floor(d / 16) = D - (rj < ri), and trunc adds one back when d < 0 and rj != ri.
// Shift a quotient record (X, R) by +L (c = 1) or -L (c = 2): x + L = 16 (X + (L >> 4)) + (R + (L & 15)),
// carrying a sixteen out of R; x - L borrowing likewise.
__device__ __forceinline__ void quot_shift(uint32_t c, int64_t L, uint32_t& X, uint32_t& R) {
    const uint32_t XL = (uint32_t)(L >> 4), RL = (uint32_t)(L & 15);
    if (c == 1u) {
        uint32_t t = R + RL;
        X += XL + (t >> 4);
        R = t & 15u;
    } else if (c == 2u) {
        uint32_t t = R + 16u - RL;
        X -= XL + (t < 16u ? 1u : 0u);
        R = t & 15u;
    }
}
__device__ __forceinline__ float quot_sep(uint32_t Xj, uint32_t rj, uint32_t Xi, uint32_t ri) {
    int32_t f = (int32_t)(Xj - Xi) - (rj < ri ? 1 : 0);
    int32_t q = f + ((f < 0 && rj != ri) ? 1 : 0);
    return __int2float_rn(q);
}
// The same with Xj - Xi formed as an integer multiply-add Xj * one + nXi (one = 1 from the
// parameter block, nXi = -Xi), which issues on the FMA pipe instead of the integer ALU pipe that
// bounds the force kernel.
__device__ __forceinline__ float quot_sep_mad(uint32_t Xj, uint32_t rj, uint32_t nXi, uint32_t ri, uint32_t one) {
    uint32_t d;
    asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(Xj), "r"(one), "r"(nXi));
    int32_t f = (int32_t)d - (rj < ri ? 1 : 0);
    int32_t q = f + ((f < 0 && rj != ri) ? 1 : 0);
    return __int2float_rn(q);
}

// Verlet-list build over the cell-sorted scratch state (neighbors.wgsl:27-64 with the exact f32
// test of engine.rs:302-313 / 184-186): lists are warp-tiled (list_slot); a particle with
// more than `cap` neighbours sets ctl[1] (overflow). Also copies the sorted state back into the
// engine's arrays and records each particle's reference position for the trigger.
// With slab keys (key_shift > 0) a cell one layer up along the last axis is scanned only over its
// slabs up to the particle's own (of its offset + sub_delta), a cell one layer down only from the
// particle's own slab (of its offset - sub_delta): a pair the exact test accepts lies within the
// list radius on that axis, and a cell is at least that wide, so no neighbour is skipped.
// S lanes per particle (small systems, whose one-lane build is a single long dependent walk):
// lane s takes candidates s, s + S, ... of each cell and the segment's ballot orders the appends,
// so the list is the one-lane list entry for entry.
template <int D, bool MULTI, int S = 1>
__global__ void __launch_bounds__(128) k_build_list(Params P, const PosRec<D>* __restrict__ pos_s, const int32_t* __restrict__ vel_s,
                                                    const uint32_t* __restrict__ species_s, const uint32_t* __restrict__ ids_s,
                                                    const uint32_t* __restrict__ keys, const uint32_t* __restrict__ start,
                                                    const float4* __restrict__ relf, PosRec<D>* __restrict__ pos_o,
                                                    int32_t* __restrict__ vel_o, uint32_t* __restrict__ species_o,
                                                    uint32_t* __restrict__ ids_o, PosRec<D>* __restrict__ ref_pos,
                                                    uint32_t* __restrict__ nbr, uint32_t* __restrict__ nbr_count,
                                                    uint32_t* __restrict__ ctl, uint4* __restrict__ qpos_o) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t i = t / S, seg = t % S;
    if (t == 0) {
        ctl[0] = 0; // the rebuild is done: clear the trigger, count it
        ctl[2] += 1;
    }
    if (S == 1 && i >= P.n) return;
    const bool valid = i < P.n; // (S > 1: every lane of the warp takes part in its ballots)
    const uint32_t iv = valid ? i : P.n - 1;
    int64_t xi[3];
    uint32_t si = load_particle<D, MULTI>(pos_s, species_s, iv, xi);
    uint32_t c[3];
    const uint32_t sh = S > 1 ? P.key_shift : 0u; // (slab keys come only with several lanes)
    cell_coords(P, keys[iv] >> sh, c);
    uint32_t count = 0;
    const uint32_t cap = P.cap, cap4 = (P.cap + 3u) & ~3u;
    const size_t lbase = list_slot(iv, 0, cap4); // entry k at lbase + (k & ~3) 32 + (k & 3)
    const bool unchecked = P.sep_unchecked;
    // Candidate j of a neighbour cell cj sits at d = relf[j] + base: base = (cj - c) cell_w + shift
    // - (xi - c cell_w), an exact integer converted once per cell. Outside [lo, hi] the f32
    // distance decides (its error is far below the 1e-4 margin); inside, the exact test does.
    int64_t reli[3];
#pragma unroll
    for (int a = 0; a < 3; a++) reli[a] = a < D ? xi[a] - (int64_t)c[a] * P.cell_w[a] : 0;
    // slabs [0, up] of the cells a layer up, [dn, top] of those a layer down (all: no slab keys)
    const uint32_t up = (S > 1 && sh) ? sub_bucket(P, reli[D - 1] + P.sub_delta) : 0u;
    const uint32_t dn = (S > 1 && sh) ? sub_bucket(P, reli[D - 1] - P.sub_delta) : 0u;
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
        return ok && r2 < P.pc[si * P.ns + sj].list2s;
    };
    const float lo0 = P.pc[si * P.ns].list2lo, hi0 = P.pc[si * P.ns].list2hi;
    const uint32_t nx = P.nc[0], ny = P.nc[1], nz = P.nc[2];
    for (int oz = 0; oz < (D == 3 ? 3 : 1); oz++) {
        int tz = (int)c[2] + oz - 1;
        uint32_t z = D == 3 ? (tz < 0 ? nz - 1 : (tz >= (int)nz ? 0 : (uint32_t)tz)) : 0;
        int64_t sz = D == 3 ? image_shift(P, 2, tz < 0 ? -P.box[2] : (tz >= (int)nz ? P.box[2] : 0)) : 0;
        for (int oy = 0; oy < 3; oy++) {
            int ty = (int)c[1] + oy - 1;
            uint32_t y = ty < 0 ? ny - 1 : (ty >= (int)ny ? 0 : (uint32_t)ty);
            int64_t sy = image_shift(P, 1, ty < 0 ? -P.box[1] : (ty >= (int)ny ? P.box[1] : 0));
            const int layer = D == 3 ? oz : oy; // along the last axis: 0 down, 1 same, 2 up
            const uint32_t slab0 = layer == 0 ? dn : 0u, slab1 = layer == 2 ? up + 1u : (1u << sh);
            if constexpr (D == 2 && S == 1) {
                // 2D, away from the x edges: the row's three cells are consecutive keys, one range
                // with no x image; a candidate's offset from this particle's cell is its cell's x
                // index (the record's third word) minus this one's, in cell widths.
                if (c[0] >= 1u && c[0] + 1u < nx) {
                    const uint32_t row0 = y * nx + c[0] - 1u;
                    const uint32_t j0 = __ldg(start + row0), j1 = __ldg(start + row0 + 3u);
                    const int64_t xs[3] = {xi[0], xi[1] - sy, 0};
                    const uint32_t code = image_code(0, sy, 0);
                    const float b0 = off_f32(-reli[0]), wf = off_f32(P.cell_w[0]), cxf = (float)c[0];
                    const float b1 = off_f32(((int64_t)y - (int64_t)c[1]) * P.cell_w[1] + sy - reli[1]);
                    auto r2_of = [&](const float4& r) {
                        const float dx = __fmaf_rn(__fsub_rn(r.z, cxf), wf, __fadd_rn(r.x, b0)), dy = r.y + b1;
                        return __fmaf_rn(dy, dy, __fmul_rn(dx, dx));
                    };
                    bool band = false; // (the band as in the cell walk below)
#pragma unroll 4
                    for (uint32_t j = j0; j < j1; j++) {
                        const float4 r = __ldg(relf + j);
                        const float r2a = r2_of(r);
                        const uint32_t sj = MULTI ? __float_as_uint(r.w) : 0u;
                        const float lo = MULTI ? P.pc[si * P.ns + sj].list2lo : lo0, hi = MULTI ? P.pc[si * P.ns + sj].list2hi : hi0;
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
                            const float lo = MULTI ? P.pc[si * P.ns + sj].list2lo : lo0, hi = MULTI ? P.pc[si * P.ns + sj].list2hi : hi0;
                            if (r2a >= lo && r2a <= hi && j != i && exact(j, xs, sj)) {
                                if (count < cap) nbr[lbase + ((size_t)(count & ~3u) << 5) + (count & 3u)] = j | code;
                                count++;
                            }
                        }
                    continue;
                }
            }
            for (int ox = 0; ox < 3; ox++) {
                int tx = (int)c[0] + ox - 1;
                uint32_t x = tx < 0 ? nx - 1 : (tx >= (int)nx ? 0 : (uint32_t)tx);
                int64_t sx = image_shift(P, 0, tx < 0 ? -P.box[0] : (tx >= (int)nx ? P.box[0] : 0));
                uint32_t cell = (z * ny + y) * nx + x;
                const int64_t xs[3] = {xi[0] - sx, xi[1] - sy, D == 3 ? xi[2] - sz : 0};
                const uint32_t code = image_code(sx, sy, sz);
                const float b0 = off_f32(((int64_t)x - (int64_t)c[0]) * P.cell_w[0] + sx - reli[0]);
                const float b1 = off_f32(((int64_t)y - (int64_t)c[1]) * P.cell_w[1] + sy - reli[1]);
                const float b2 = D == 3 ? off_f32(((int64_t)z - (int64_t)c[2]) * P.cell_w[2] + sz - reli[2]) : 0.0f;
                const uint32_t j0 = __ldg(start + ((cell << sh) | slab0)), j1 = __ldg(start + (cell << sh) + slab1);
                auto test = [&](uint32_t j) -> bool {
                    float4 r = __ldg(relf + j);
                    float dx = r.x + b0, dy = r.y + b1, dz = D == 3 ? r.z + b2 : 0.0f;
                    // approximate (fused) distance: its error is far inside the 1e-4 band
                    float r2a = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
                    uint32_t sj = MULTI ? __float_as_uint(r.w) : 0u;
                    float lo = MULTI ? P.pc[si * P.ns + sj].list2lo : lo0, hi = MULTI ? P.pc[si * P.ns + sj].list2hi : hi0;
                    return (r2a < lo || (r2a <= hi && exact(j, xs, sj))) && j != i;
                };
                if constexpr (S == 1) {
                    // Branch-free walk: candidates inside the band's lower edge are appended by a
                    // predicated store and count += accepted; a candidate inside the band only
                    // marks the cell, which a second walk then settles with the exact test (rare:
                    // ~0.02 band candidates per particle). 6% and 7% faster than branching around
                    // the append and around the exact test (most warps took them for a few lanes).
                    bool band = false;
#pragma unroll 4
                    for (uint32_t j = j0; j < j1; j++) {
                        const float4 r = __ldg(relf + j);
                        const float dx = r.x + b0, dy = r.y + b1, dz = D == 3 ? r.z + b2 : 0.0f;
                        const float r2a = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
                        const uint32_t sj = MULTI ? __float_as_uint(r.w) : 0u;
                        const float lo = MULTI ? P.pc[si * P.ns + sj].list2lo : lo0, hi = MULTI ? P.pc[si * P.ns + sj].list2hi : hi0;
                        const bool in = r2a < lo && j != i;
                        band |= r2a >= lo && r2a <= hi;
                        const size_t at = lbase + ((size_t)(count & ~3u) << 5) + (count & 3u);
                        if (in && count < cap) nbr[at] = j | code;
                        count += in ? 1u : 0u;
                    }
                    if (band)
                        for (uint32_t j = j0; j < j1; j++) {
                            const float4 r = __ldg(relf + j);
                            const float dx = r.x + b0, dy = r.y + b1, dz = D == 3 ? r.z + b2 : 0.0f;
                            const float r2a = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
                            const uint32_t sj = MULTI ? __float_as_uint(r.w) : 0u;
                            const float lo = MULTI ? P.pc[si * P.ns + sj].list2lo : lo0, hi = MULTI ? P.pc[si * P.ns + sj].list2hi : hi0;
                            if (r2a >= lo && r2a <= hi && j != i && exact(j, xs, sj)) {
                                if (count < cap) nbr[lbase + ((size_t)(count & ~3u) << 5) + (count & 3u)] = j | code;
                                count++;
                            }
                        }
                } else {
                    // the warp walks the longest of its particles' ranges, so every ballot is whole
                    const uint32_t lane = threadIdx.x & 31u;
                    const uint32_t segmask = ((1u << S) - 1u) << (lane & ~(uint32_t)(S - 1));
                    const uint32_t below = ((1u << lane) - 1u) & segmask;
                    const uint32_t je = valid ? j1 : j0;
                    const uint32_t trips = __reduce_max_sync(0xffffffffu, (je - j0 + 4 * S - 1) / (4 * S));
                    for (uint32_t r = 0; r < trips; r++) {
                        const uint32_t jb = j0 + r * 4 * S;
                        bool in[4];
#pragma unroll
                        for (int u = 0; u < 4; u++) {
                            const uint32_t j = jb + u * S + seg;
                            in[u] = j < je && test(j);
                        }
#pragma unroll
                        for (int u = 0; u < 4; u++) {
                            const uint32_t m = __ballot_sync(0xffffffffu, in[u]) & segmask;
                            const uint32_t k = count + __popc(m & below);
                            if (in[u] && k < cap) nbr[lbase + ((size_t)(k & ~3u) << 5) + (k & 3u)] = (jb + u * S + seg) | code;
                            count += __popc(m);
                        }
                    }
                }
            }
        }
    }
    if (!valid || (S > 1 && seg != 0)) return;
    if (count > cap) {
        ctl[1] = 1;
        count = cap;
    }
    nbr_count[i] = count;
    pos_o[i] = pos_s[i];
    ref_pos[i] = pos_s[i];
    if (qpos_o) {
        uint4 q = quot_record<D>(xi, si);
        if (D == 2) q.z = 1u; // the path since this build: 0 (the unused z word, as U + 1)
        qpos_o[i] = q;
    }
#pragma unroll
    for (int a = 0; a < D; a++) vel_o[D * i + a] = vel_s[D * i + a];
    species_o[i] = species_s[i];
    ids_o[i] = ids_s[i];
}

// The scenario epilogue's pieces (defined with the bonds and walls below).
template <int D>
__device__ __forceinline__ float bond_kicks(const Params& P, uint32_t id, const int64_t* xi, const PosRec<D>* pos, float c, int32_t* k);
template <int D>
__device__ __forceinline__ void wall_kicks(const Params& P, const int64_t* xo, float c, int32_t* k, unsigned long long* ledger);
template <int D>
__device__ __forceinline__ bool wall_post(const Params& P, uint32_t si, uint32_t id, uint32_t clock, int64_t* x, int32_t* v,
                                          unsigned long long* ledger, bool wrap_periodic);

// The hot kernel: LJ pair kicks over the Verlet list fused with the integer leapfrog and the
// rebuild trigger. Reads positions from pos_in and writes the moved ones to pos_out (the engine
// ping-pongs the two), so every kick sees positions of the same time step.
// Ten blocks of 128 per SM (48 registers, a 16-byte spill outside the pair loop): measured 2.4%
// faster than the unconstrained 62 registers at eight blocks.
// S lanes per particle (1; up to 16 for small systems, which would otherwise leave the GPU with
// too few threads to hide the latency of ~20 groups walked one after another): lane s of a
// particle takes its groups s, s + S, ... and the integer kicks are summed across the S lanes
// (wrapping integer sums: the result does not depend on the split). CG: positions and records
// are read through L2 only (the persistent step loop, where other blocks rewrite them).
// `n`: the particles of the arrays (a batch passes all of its systems' particles, with P the
// parameter block of the system that lane t's particle belongs to).
template <int D, bool MULTI, bool INT, bool SIG1, int S, bool CG, bool EXT = false>
__device__ __forceinline__ bool force_list_one(const Params& P, uint32_t n, uint32_t t, const PosRec<D>* __restrict__ pos_in,
                                               PosRec<D>* __restrict__ pos_out, const uint4* __restrict__ qpos_in, uint4* __restrict__ qpos_out,
                                               int32_t* __restrict__ vel, const uint32_t* __restrict__ species, const uint32_t* __restrict__ nbr,
                                               const uint32_t* __restrict__ nbr_count, const PosRec<D>* __restrict__ ref_pos) {
    const uint32_t i = S == 1 ? t : (t >> 5) * (32u / S) + (t & 31u) / S, seg = S == 1 ? 0u : (t & 31u) % S;
    if (S == 1 && i >= n) return false;
    const bool valid = i < n; // (S > 1: every lane takes part in the kick sum)
    const uint32_t iv = valid ? i : n - 1;
    int64_t xi[3];
    uint32_t si = load_particle<D, MULTI, CG>(pos_in, species, iv, xi);
    const float cs = P.kick_cs[si];
    int32_t k[3] = {0, 0, 0};
    const uint32_t m = valid ? __ldg(nbr_count + i) : 0u, cap4 = (P.cap + 3u) & ~3u;
    const PairC pc0 = P.pc[0];
    uint32_t path = 0; // 2D: the quotient record's z word, the path since the list build + 1 (0: unknown)
    const uint4* groups = reinterpret_cast<const uint4*>(nbr + list_slot(iv, 0, cap4)); // group g at groups[32 g]
    // Every listed neighbour is within 8 sigma of xi at its recorded image (list radius + skin),
    // so neither a minimum image nor a range check is needed.
    auto add_kick = [&](const float* f, const PairC& pc) {
        float fr, s6, r2;
        if (pair_fr<D, SIG1>(pc, f, fr, s6, r2)) {
            float am = __fmul_rn(-fr, cs);
#pragma unroll
            for (int a = 0; a < D; a++) k[a] = wadd(k[a], rni_f32(__fmul_rn(am, f[a])));
        }
    };
    const uint32_t ngroups = (m + 3u) >> 2;
    {
        // Neighbours come from the 16-byte quotient records (one gather each) and the separation
        // is formed with 32-bit integers (quot_sep); a neighbour listed at a periodic image has
        // its quotient record shifted by that image exactly (quot_shift). 2D and 3D alike.
        const uint4 qi = ld_in<CG>(qpos_in + iv);
        const uint32_t Xi[3] = {qi.x, qi.y, qi.z};
        if (D == 2) path = qi.z;
        for (uint32_t g = seg; g < ngroups; g += S) {
            // (the prefetch index clamped to the last group rather than guarded: no branch)
            asm volatile("prefetch.global.L2 [%0];" ::"l"(groups + 32 * min(g + 2 * S, ngroups - 1u)));
            const uint4 jv = __ldg(groups + 32 * g);
            const uint32_t jj[4] = {jv.x, jv.y, jv.z, jv.w};
            const uint32_t left = m - 4 * g;
            uint4 r[4];
#pragma unroll
            for (int u = 0; u < 4; u++) r[u] = ld_in<CG>(qpos_in + ((uint32_t)u < left ? (jj[u] & LIST_MASK) : iv));
            if constexpr (!INT && !MULTI && SIG1) {
                // Four neighbours as two packed pairs: integer separations per neighbour, then the
                // f32 chain of both pairs of a pack in f32x2 instructions. Slots past the list end
                // and pairs beyond the cutoff get a zero coefficient (rint(0 f) = 0 adds nothing);
                // a pack holding a pair closer than sigma / 8 goes through the scalar chain.
                float f[4][3];
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    uint32_t Xj[3] = {r[u].x, r[u].y, r[u].z};
                    // the remainders are whole bytes of the fourth word: one byte select each
                    uint32_t Rj[3] = {__byte_perm(r[u].w, 0u, 0x4440u), __byte_perm(r[u].w, 0u, 0x4441u), __byte_perm(r[u].w, 0u, 0x4442u)};
                    const uint32_t code = jj[u] >> LIST_BITS;
                    // (a slot past the list's end holds a stale word; shifting this particle's own
                    // record for it is harmless, its pair gets a zero coefficient)
                    if (code) {
#pragma unroll
                        for (int a = 0; a < D; a++) quot_shift((code >> (2 * a)) & 3u, P.box[a], Xj[a], Rj[a]);
                    }
#pragma unroll
                    for (int a = 0; a < D; a++) f[u][a] = quot_sep_mad(Xj[a], Rj[a], 0u - Xi[a], (qi.w >> (8 * a)) & 15u, P.one);
                    if (D == 2) f[u][2] = 0.0f;
                }
#pragma unroll
                for (int h = 0; h < 2; h++) pair_kicks2_sig1<D>(pc0, cs, f[2 * h], f[2 * h + 1], (uint32_t)(2 * h) < left, (uint32_t)(2 * h + 1) < left, k);
            } else {
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    if ((uint32_t)u >= left) break;
                    uint32_t Xj[3] = {r[u].x, r[u].y, r[u].z};
                    uint32_t Rj[3] = {r[u].w & 15u, (r[u].w >> 8) & 15u, (r[u].w >> 16) & 15u};
                    const uint32_t code = jj[u] >> LIST_BITS;
                    if (code) {
#pragma unroll
                        for (int a = 0; a < D; a++) quot_shift((code >> (2 * a)) & 3u, P.box[a], Xj[a], Rj[a]);
                    }
                    if constexpr (INT) {
                        // the exact separation from the records: d = 16 (Xj - Xi) + (rj - ri)
                        int64_t d[3] = {0, 0, 0};
#pragma unroll
                        for (int a = 0; a < D; a++)
                            d[a] = (int64_t)(int32_t)(Xj[a] - Xi[a]) * 16 + ((int64_t)Rj[a] - (int64_t)((qi.w >> (8 * a)) & 15u));
                        int_kick<D>(P, MULTI ? si * P.ns + (r[u].w >> 24) : 0u, d, k);
                    } else {
                        float f[D];
#pragma unroll
                        for (int a = 0; a < D; a++) f[a] = quot_sep(Xj[a], Rj[a], Xi[a], (qi.w >> (8 * a)) & 15u);
                        add_kick(f, MULTI ? P.pc[si * P.ns + (r[u].w >> 24)] : pc0);
                    }
                }
            }
        }
    }
    if constexpr (S > 1) {
#pragma unroll
        for (int o = 1; o < S; o <<= 1)
#pragma unroll
            for (int a = 0; a < D; a++) k[a] = wadd(k[a], __shfl_xor_sync(0xffffffffu, k[a], o));
        if (!valid || seg != 0) return false;
    }
    if constexpr (EXT) {
        // the scenario's other kicks, from the step's start positions, as IntEngine::forces sums
        // them with the pair kicks (int_engine.rs:185-246): bonds (partners read from pos_in
        // through the id -> slot map of the last list build), soft walls and the piston
        const float c = __fmul_rn(cs, 1.0f / 268435456.0f);
        if (D == 2 && P.bonds) bond_kicks<D>(P, P.ids_list[i], xi, pos_in, c, k);
        if (P.walls) wall_kicks<D>(P, xi, c, k, P.ledger);
    }
    int32_t v[3];
#pragma unroll
    for (int a = 0; a < D; a++) v[a] = vel[D * i + a];
    leapfrog<D, Params, false>(P, si, k, v, xi);
    if constexpr (EXT) {
        // then the bath, the membrane, the walls' mirrors and collisions, the piston's mirror
        if (P.walls || P.bath) wall_post<D>(P, si, P.ids_list[i], *P.clock_word, xi, v, P.ledger, false);
    }
#pragma unroll
    for (int a = 0; a < D; a++) vel[D * i + a] = v[a];
    store_pos<D>(pos_out, i, xi, si);
    uint4 qo = quot_record<D>(xi, si);
    if constexpr (D == 2 && !EXT) {
        // Positions move by exactly v each step between list builds (no wrap), so |x - ref| is at
        // most the path U = sum of |vx| + |vy|. While U stays below ub_thr the trigger cannot fire
        // and the reference record need not be read. Any other writer of the record leaves z = 0,
        // and the test then runs until the next build.
        if (path != 0u && P.ub_thr != 0u) {
            const uint64_t U = (uint64_t)(path - 1u) + (uint64_t)uabs32(v[0]) + (uint64_t)uabs32(v[1]);
            if (U < P.ub_thr) {
                qo.z = (uint32_t)U + 1u;
                qpos_out[i] = qo;
                return false;
            }
        }
    }
    qpos_out[i] = qo;
    int64_t xr[3];
    load_particle<D, false>(ref_pos, nullptr, i, xr);
    return moved_half_skin<D>(P, xr, xi);
}

// EXT: the scenario variant (bonds, walls, the piston, the bath), which takes those in its own
// epilogue instead of separate passes over the state.
template <int D, bool MULTI, bool INT = false, bool SIG1 = false, int S = 1, bool EXT = false>
__global__ void __launch_bounds__(128, 10) k_force_list(Params P, const PosRec<D>* __restrict__ pos_in, PosRec<D>* __restrict__ pos_out,
                                                    const uint4* __restrict__ qpos_in, uint4* __restrict__ qpos_out,
                                                    int32_t* __restrict__ vel, const uint32_t* __restrict__ species,
                                                    const uint32_t* __restrict__ nbr, const uint32_t* __restrict__ nbr_count,
                                                    const PosRec<D>* __restrict__ ref_pos, uint32_t* __restrict__ ctl) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (force_list_one<D, MULTI, INT, SIG1, S, false, EXT>(P, P.n, t, pos_in, pos_out, qpos_in, qpos_out, vel, species, nbr, nbr_count,
                                                           ref_pos))
        ctl[0] = 1;
}

// ---------------------------------------------------------------- the persistent step loop
// Words of the engine's control block used by the loop (0: trigger, 1: overflow, 2: rebuilds).
constexpr uint32_t CTL_CLOCK = 14;      // the Andersen bath's step clock (IntEngine::clock)
constexpr uint32_t CTL_LOOP_DONE = 4;   // steps the loop has taken in the current graph block
constexpr uint32_t CTL_BAR_GEN = 6;     // grid barrier: barriers released (low 31 bits) | stop (bit 31)
constexpr uint32_t CTL_LOOP_ERR = 8;    // a barrier wait ran out (the loop stopped; an error status)
constexpr uint32_t CTL_LOOP_ITERS = 9;  // loop launches so far (launch accounting)
constexpr uint32_t CTL_BAR_ARRIVE = 12; // grid barrier, words 12-13 as one 64-bit counter: arrivals in
                                        // this launch | blocks that saw the trigger << 32
constexpr uint32_t BARRIER_SPINS = 1u << 20; // polls of 0.1-0.5 us: well under a second

__device__ __forceinline__ uint32_t ld_acquire_gpu(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_gpu(uint32_t* p, uint32_t v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Grid-wide barrier of a cooperative launch, carrying one bit: whether any block's particles
// moved half the skin in this step. Thread 0 of each block arrives with one 64-bit atomic add
// (one arrival, plus one in the high word if the block saw the trigger). The block whose add
// completes the k-th barrier of the launch (k x blocks arrivals) publishes generation base + k
// with the stop bit by a release store; the others poll for it with acquire loads. No word is
// reset between barriers, so an arrival costs one atomic round trip and a release one store.
// A poll is bounded: after BARRIER_SPINS the block records CTL_LOOP_ERR and returns "stop", so a
// grid that is somehow not co-resident ends with an error status instead of a hang. The arrival
// counter is cleared by block 0 after the launch's last barrier (every block has arrived then).
struct GridBarrier {
    uint32_t* ctl;
    uint32_t base;  // generation when the launch began (read by every block before any release)
    uint32_t k = 0; // barriers of this launch so far
    __device__ static uint32_t begin(uint32_t* ctl) {
        __shared__ uint32_t s_base;
        if (threadIdx.x == 0) s_base = ld_acquire_gpu(ctl + CTL_BAR_GEN) & 0x7fffffffu;
        __syncthreads();
        return s_base;
    }
    __device__ bool wait(bool moved) {
        __shared__ uint32_t s_res;
        const int any = __syncthreads_or(moved ? 1 : 0);
        k++;
        if (threadIdx.x == 0) {
            const uint32_t want = (base + k) & 0x7fffffffu;
            __threadfence(); // the block's stores (seen through the CTA barrier) before its arrival
            const unsigned long long old = atomicAdd(reinterpret_cast<unsigned long long*>(ctl + CTL_BAR_ARRIVE), any ? 0x100000001ull : 1ull);
            const uint32_t arrived = (uint32_t)old + 1u, saw = (uint32_t)(old >> 32) + (any ? 1u : 0u);
            uint32_t res;
            if (arrived == k * gridDim.x) {
                res = want | (saw ? 0x80000000u : 0u);
                st_release_gpu(ctl + CTL_BAR_GEN, res);
            } else {
                uint32_t spins = 0;
                while (((res = ld_acquire_gpu(ctl + CTL_BAR_GEN)) & 0x7fffffffu) != want) {
                    if (++spins > BARRIER_SPINS) {
                        atomicExch(ctl + CTL_LOOP_ERR, 1u);
                        res = 0x80000000u;
                        break;
                    }
                    __nanosleep(32);
                }
            }
            __threadfence();
            s_res = res;
        }
        __syncthreads();
        return (s_res & 0x80000000u) != 0u;
    }
    // after the launch's last barrier: block 0 clears the arrival counter for the next launch
    __device__ void end() const {
        if (blockIdx.x == 0 && threadIdx.x == 0) *reinterpret_cast<unsigned long long*>(ctl + CTL_BAR_ARRIVE) = 0ull;
    }
};

// The barrier with block `absent` never arriving: the others' waits run out (CTL_LOOP_ERR).
static __global__ void k_barrier_absent(uint32_t* ctl, uint32_t absent) {
    GridBarrier bar{ctl, GridBarrier::begin(ctl)};
    if (blockIdx.x == absent) return;
    bar.wait(false);
}

// Steps of the Verlet-list engine in one cooperative launch (small systems, one species, sigma
// = 1, f32 chain): force + leapfrog + trigger per step as k_force_list, a grid barrier between
// steps, and out as soon as a particle has moved half the skin (the list must be rebuilt before
// the next step) or the block of `target` steps is done. Positions ping-pong between pos0 and
// pos1 inside the launch and end in pos0 (copied back after an odd number of steps), so the
// graph around it sees one fixed buffer. Positions and records written during the launch are
// read through L2 only (ld_in<true>).
template <int D, int S>
__global__ void __launch_bounds__(128, 10) k_force_loop(Params P, PosRec<D>* __restrict__ pos0, PosRec<D>* __restrict__ pos1,
                                                    uint4* __restrict__ q0, uint4* __restrict__ q1, int32_t* __restrict__ vel,
                                                    const uint32_t* __restrict__ nbr, const uint32_t* __restrict__ nbr_count,
                                                    const PosRec<D>* __restrict__ ref_pos, uint32_t* __restrict__ ctl, uint32_t target) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    // Words no block writes before every block has read them: the steps done (written at the
    // end, after the last barrier) and the error word (written only by a barrier that ran out).
    // (The trigger is not read here: a block that started late could see this launch's own.)
    const uint32_t done = *(volatile uint32_t*)(ctl + CTL_LOOP_DONE);
    bool stop = done >= target || *(volatile uint32_t*)(ctl + CTL_LOOP_ERR) != 0u;
    GridBarrier bar{ctl, GridBarrier::begin(ctl)};
    uint32_t k = 0;
    while (!stop) {
        const bool odd = k & 1u;
        const bool moved = force_list_one<D, false, false, true, S, true>(P, P.n, t, odd ? pos1 : pos0, odd ? pos0 : pos1, odd ? q1 : q0,
                                                                          odd ? q0 : q1, vel, nullptr, nbr, nbr_count, ref_pos);
        if (moved) ctl[0] = 1;
        k++;
        stop = bar.wait(moved) || done + k >= target;
    }
    bar.end();
    const uint32_t i = t / S;
    if ((k & 1u) && t % S == 0 && i < P.n) {
        // the record as 16-byte halves (a 3D record is two of them)
        constexpr int H = sizeof(PosRec<D>) / sizeof(longlong2);
        const longlong2* src = reinterpret_cast<const longlong2*>(pos1 + i);
        longlong2* dst = reinterpret_cast<longlong2*>(pos0 + i);
#pragma unroll
        for (int h = 0; h < H; h++) dst[h] = __ldcg(src + h);
        q0[i] = __ldcg(q1 + i);
    }
    if (t == 0) {
        ctl[CTL_LOOP_DONE] = done + k;
        ctl[CTL_LOOP_ITERS] += 1u;
    }
}

// The bath as a pass after the force step, so that the force kernels carry none of it: the step
// left x' = x + v with v the kicked velocity; a redrawn particle gets v' and x' + (v' - v) =
// x + v', exact in integers (wrapped again in cell mode, where positions stay in the box). The
// region test uses the position before the drift, x' - v, as the reference does. With Verlet
// lists the quotient record is rewritten and the displacement trigger re-tested at the new
// position (a trigger the force step already set stays set: an extra rebuild changes nothing).
// The draw is keyed on the clock word, which the next launch in the stream advances.
// The velocity a drawn particle at height y (position units, before the move) takes from a
// driven piston's affine flow: round(piston_v clamp(y / piston_w, 0, 1)) (int_engine.rs:282-286).
__device__ __forceinline__ int32_t piston_flow(const Params& P, int64_t y) {
    double f = __ddiv_rn(to_f64(y), to_f64(P.piston->w));
    f = f < 0.0 ? 0.0 : (f > 1.0 ? 1.0 : f); // (NaN stays NaN and converts to 0)
    return sat_i32_f64(round_away(__dmul_rn((double)P.piston->v, f)));
}
// The bath on one particle's moved state (x, v as the step left them): returns whether it drew.
template <int D>
__device__ __forceinline__ bool bath_one(const Params& P, uint32_t si, uint32_t id, uint32_t clock, int64_t* x, int32_t* v,
                                         unsigned long long* ledger) {
    if (((P.pinned >> si) & 1u) || !((P.bath_species >> si) & 1u)) return false;
    if (D == 2) {
        const uint32_t ax = P.bath_axis;
        const int64_t p = wrap(x[ax] - (int64_t)v[ax], P.box[ax]);
        if (!(p >= P.bath_region[0] && p < P.bath_region[1])) return false;
    }
    const int32_t flow1 = (D == 2 && P.piston_drive == 1) ? piston_flow(P, x[1] - (int64_t)v[1]) : 0;
    const BathDraw o = bath_draw<D>(id, clock, P.bath_key[0], P.bath_key[1], P.bath_rate_dt, P.bath_sd[si], P.masses[si], P.dt, P.bath_drift,
                                    flow1, v[0], v[1], v[2], ledger);
    if (!o.hit) return false;
#pragma unroll
    for (int a = 0; a < D; a++) {
        x[a] += (int64_t)o.v[a] - (int64_t)v[a];
        v[a] = o.v[a];
    }
    return true;
}

template <int D, bool LIST>
__global__ void k_bath(Params P, PosRec<D>* __restrict__ pos, uint4* __restrict__ qpos, int32_t* __restrict__ vel,
                       const uint32_t* __restrict__ species, const uint32_t* __restrict__ ids, const PosRec<D>* __restrict__ ref_pos,
                       uint32_t* __restrict__ ctl, unsigned long long* __restrict__ ledger) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const uint32_t si = species[i];
    if (((P.pinned >> si) & 1u) || !((P.bath_species >> si) & 1u)) return;
    int64_t x[3];
    load_particle<D, false>(pos, nullptr, i, x);
    int32_t v[3] = {0, 0, 0};
#pragma unroll
    for (int a = 0; a < D; a++) v[a] = vel[D * i + a];
    if (!bath_one<D>(P, si, ids[i], ctl[CTL_CLOCK], x, v, ledger)) return;
#pragma unroll
    for (int a = 0; a < D; a++) {
        if (!LIST) x[a] = wrap(x[a], P.box[a]);
        vel[D * i + a] = v[a];
    }
    store_pos<D>(pos, i, x, si);
    if (LIST) {
        qpos[i] = quot_record<D>(x, si);
        int64_t xr[3];
        load_particle<D, false>(ref_pos, nullptr, i, xr);
        if (moved_half_skin<D>(P, xr, x)) ctl[0] = 1;
    }
}

// Insulating compartments with Verlet lists: the build lists every pair within the list radius;
// this pass drops, in place, the pairs whose particles are in different boxes (they never interact,
// int_engine.rs:161-163, and a particle never leaves its box, so the list stays right until the
// next build). The compartment axes are walled: no periodic image enters.
static __global__ void k_filter_compartments(Params P, const PosRec<2>* __restrict__ pos, uint32_t* __restrict__ nbr,
                                      uint32_t* __restrict__ nbr_count) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    int64_t xi[3];
    load_particle<2, false>(pos, nullptr, i, xi);
    const uint32_t m = nbr_count[i], cap4 = (P.cap + 3u) & ~3u;
    uint32_t kept = 0;
    for (uint32_t q = 0; q < m; q++) {
        const uint32_t e = nbr[list_slot(i, q, cap4)];
        int64_t xj[3];
        load_particle<2, false>(pos, nullptr, e & LIST_MASK, xj);
        if (!same_compartment(P.comp_shift, xi, xj)) continue;
        nbr[list_slot(i, kept, cap4)] = e;
        kept++;
    }
    nbr_count[i] = kept;
}

// ---------------------------------------------------------------- bonds (2D)
// fixed.rs:63-72 sep_long_f32: sep_f32 within 8 sigma (in sigma units); beyond, the magnitude's
// whole sigma plus its fraction in f32, then the sign.
__device__ __forceinline__ float sep_long_f32(int64_t d) {
    bool ok = true;
    const float s = __fmul_rn(sep_s(d, ok), 1.0f / 268435456.0f);
    if (ok) return s;
    const uint64_t m = d < 0 ? (uint64_t)0 - (uint64_t)d : (uint64_t)d;
    const float mag = __fadd_rn(__uint2float_rn((uint32_t)(m >> 32)), __fmul_rn(__uint2float_rn((uint32_t)m), 1.0f / 4294967296.0f));
    return d < 0 ? -mag : mag;
}
// BondConsts::eval (real.rs:175-196) in f32: -U'(r)/r and U at r2 (sigma^2), the reference's
// operation order, the FENE logarithm in IEEE double (fdlibm).
__device__ __forceinline__ void bond_eval(const Params& P, uint32_t t, float r2, float& fr, float& u) {
    const float k = P.bond_k[t], r0 = P.bond_r0[t];
    if (P.bond_fene[t]) {
        float x = __fdiv_rn(r2, __fmul_rn(r0, r0));
        if (x > 0.999999f) x = 0.999999f;
        const float om = __fsub_rn(1.0f, x);
        u = __fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(-0.5f, k), r0), r0), (float)dev_log((double)om));
        fr = __fdiv_rn(-k, om);
    } else if (r0 == 0.0f) { // a zero-length spring (tethers): -k exactly
        fr = -k;
        u = __fmul_rn(__fmul_rn(0.5f, k), r2);
    } else {
        const float r = __fsqrt_rn(r2), dr = __fsub_rn(r, r0);
        fr = __fdiv_rn(__fmul_rn(-k, dr), r);
        u = __fmul_rn(__fmul_rn(__fmul_rn(0.5f, k), dr), dr);
    }
}
// IntEngine::forces' bond kicks on a particle (int_engine.rs:185-202): each bond rounded on its
// own like a pair, from the positions `pos` (partners found through P.slot_of), c the particle's
// kick coefficient in f32; adds to k and returns the bonds' f32 energy sum.
template <int D>
__device__ __forceinline__ float bond_kicks(const Params& P, uint32_t id, const int64_t* xi, const PosRec<D>* pos, float c, int32_t* k) {
    float pe = 0.0f;
    for (uint32_t q = 0; q < 4; q++) {
        const uint32_t jid = P.bond_tab[8 * (size_t)id + 2 * q];
        if (jid == 0xffffffffu) break;
        const uint32_t t = P.bond_tab[8 * (size_t)id + 2 * q + 1] & 3u;
        int64_t xj[3];
        load_particle<D, false>(pos, nullptr, P.slot_of[jid], xj);
        float f[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int a = 0; a < D; a++) f[a] = sep_long_f32(min_image(xj[a] - xi[a], P.box[a], P.half[a]));
        float r2 = __fadd_rn(__fmul_rn(f[0], f[0]), __fmul_rn(f[1], f[1]));
        if (D == 3) r2 = __fadd_rn(r2, __fmul_rn(f[2], f[2]));
        float fr, u;
        bond_eval(P, t, r2, fr, u);
        const float aa = __fmul_rn(-fr, c);
#pragma unroll
        for (int a = 0; a < D; a++) k[a] = wadd(k[a], rni_f32(__fmul_rn(aa, f[a])));
        pe = __fadd_rn(pe, u);
    }
    return pe;
}
// The storage slot of each particle id, for the bond pass.
static __global__ void k_slot_of(uint32_t n, const uint32_t* __restrict__ ids, uint32_t* __restrict__ slot_of) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n) slot_of[ids[s]] = s;
}
// After the force step of a bonded system: each particle's bond kicks from the step's start
// positions `x0` (read only here, so no particle sees another's update) are added to its velocity
// and to its moved position, exactly as if the force step had summed them with the pair kicks.
template <int D, bool LIST>
__global__ void k_bonds(Params P, const PosRec<D>* __restrict__ x0, PosRec<D>* __restrict__ pos, uint4* __restrict__ qpos,
                        int32_t* __restrict__ vel, const uint32_t* __restrict__ species, const uint32_t* __restrict__ ids,
                        const PosRec<D>* __restrict__ ref_pos, uint32_t* __restrict__ ctl) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const uint32_t si = species[i];
    int64_t xs[3];
    load_particle<D, false>(x0, nullptr, i, xs);
    int32_t kb[3] = {0, 0, 0};
    bond_kicks<D>(P, ids[i], xs, x0, __fmul_rn(P.kick_cs[si], 1.0f / 268435456.0f), kb);
    if (!(kb[0] | kb[1] | (D == 3 ? kb[2] : 0))) return;
    int64_t x[3];
#pragma unroll
    for (int a = 0; a < D; a++) { // the move from the start with the wrapped velocity sum (x += v)
        const int32_t v = wadd(vel[D * i + a], kb[a]);
        vel[D * i + a] = v;
        x[a] = xs[a] + (int64_t)v;
        if (!LIST && ((P.periodic >> a) & 1u)) x[a] = wrap(x[a], P.box[a]);
    }
    store_pos<D>(pos, i, x, si);
    if (LIST) {
        qpos[i] = quot_record<D>(x, si);
        int64_t xr[3];
        load_particle<D, false>(ref_pos, nullptr, i, xr);
        if (moved_half_skin<D>(P, xr, x)) ctl[0] = 1;
    }
}

// ---------------------------------------------------------------- walls
// md_core::walls (walls.rs) as IntEngine runs them (int_engine.rs:203-227 and 256-263, the soft
// walls' kicks and impulses; 316-330, the mirror; 363-390, collide; int_engine3.rs:107-126,
// 140-145 and 186-205 in 3D). Ledger slots 2 axis + side, three words each: the energy given
// (2^-24 epsilon), the hits, the normal momentum given to the wall (2^-24); each event's f64
// value is rounded half away from zero before it is added, so the totals do not depend on the
// order in which the GPU books events.
constexpr float SOFT_WALL_RC = 1.12246204830937298f; // walls.rs:104, 2^(1/6) (f32 of the f64 constant)
__device__ __forceinline__ unsigned long long ledger_fixed(double x) {
    return (unsigned long long)sat_i64_f64(round_away(__dmul_rn(x, 16777216.0)));
}
// The soft wall's WCA force at distance dw from the wall, in f32 (Real<f32>, no contraction):
// s2 = 1 / (d d), s6 = s2 s2 s2, f = 24 s6 (2 s6 - 1) / d; false beyond its range.
__device__ __forceinline__ bool soft_wall_force(int64_t dw, float& f, float& s6_out) {
    bool ok = true;
    const float d = __fmul_rn(sep_s(dw, ok), 1.0f / 268435456.0f); // sep_f32: 2^-28 sigma units
    if (!ok || !(d < SOFT_WALL_RC)) return false;
    const float s2 = __fdiv_rn(1.0f, __fmul_rn(d, d));
    const float s6 = __fmul_rn(__fmul_rn(s2, s2), s2);
    f = __fdiv_rn(__fmul_rn(__fmul_rn(24.0f, s6), __fsub_rn(__fmul_rn(2.0f, s6), 1.0f)), d);
    s6_out = s6;
    return true;
}
// walls::thermal_velocity (walls.rs:89-101) / three::thermal_velocity (three.rs:222-243): the
// normal component (into the box) and the tangential ones of a Maxwell-flux draw at kT = t.
template <int D>
__device__ __forceinline__ void thermal_velocity(const Params& P, uint32_t id, uint32_t clock, double t, double m, double inward,
                                                 double& vn, double* vt) {
    uint32_t r0, r1, q0, q1;
    threefry2x32(id, clock, P.wall_key[0], P.wall_key[1], r0, r1);
    threefry2x32(id, clock, P.wall_key[0], P.wall_key[1] ^ 1u, q0, q1);
    const double u1 = __dsub_rn(1.0, to_unit_f64(r0, r1));
    const double u2 = __dsub_rn(1.0, to_unit_f64(q0, 0u)), u3 = to_unit_f64(q1, 0u);
    const double tau = 6.28318530717958647692;
    const double sd = __dsqrt_rn(__ddiv_rn(t, m));
    vn = __dmul_rn(__dmul_rn(inward, sd), __dsqrt_rn(__dmul_rn(-2.0, dev_log(u1))));
    if (D == 2) {
        vt[0] = __dmul_rn(__dmul_rn(sd, __dsqrt_rn(__dmul_rn(-2.0, dev_log(u2)))), dev_cos(__dmul_rn(tau, u3)));
    } else {
        const double rad = __dmul_rn(sd, __dsqrt_rn(__dmul_rn(-2.0, dev_log(u2))));
        const double a = __dmul_rn(tau, u3);
        vt[0] = __dmul_rn(rad, dev_cos(a));
        vt[1] = __dmul_rn(rad, dev_sin(a));
    }
}
// The ledger entry of slot w for a particle at x: its compartment along the wall, i.e. along the
// other axis (IntEngine::ledger_compartment, int_engine.rs:392-394; 0 without compartments, in 3D
// and for the bath).
template <int D>
__device__ __forceinline__ unsigned long long* ledger_at(const Params& P, unsigned long long* ledger, int w, int axis, const int64_t* x) {
    uint32_t c = 0;
    if (D == 2 && axis < 2) {
        const uint32_t o = 1 - axis, sh = P.comp_shift[o];
        if (sh) c = (uint32_t)(x[o] >> sh);
    }
    return ledger + 3 * ((size_t)w * P.ledger_per_wall + c);
}
// The walls' kicks on one particle at its step-start position xo (int_engine.rs:203-246): each
// soft wall's WCA kick (its impulse booked on the ledger) and the piston's (its force summed in
// 2^-16 eps/sigma units), added to k like the pair kicks; c is the particle's kick coefficient.
template <int D>
__device__ __forceinline__ void wall_kicks(const Params& P, const int64_t* xo, float c, int32_t* k, unsigned long long* ledger) {
#pragma unroll
    for (int a = 0; a < D; a++) {
        if ((P.periodic >> a) & 1u) continue;
#pragma unroll
        for (int side = 0; side < 2; side++) {
            if (P.wall_kind[a][side] != GBMD_WALL_SOFT) continue;
            float f, s6;
            if (!soft_wall_force(side == 0 ? xo[a] : P.box[a] - xo[a], f, s6)) continue;
            const int32_t kw = rni_f32(__fmul_rn(f, c));
            k[a] = wadd(k[a], side == 0 ? kw : (int32_t)(0u - (uint32_t)kw));
            atomicAdd(ledger_at<D>(P, ledger, 2 * a + side, a, xo) + 2, ledger_fixed(__dmul_rn((double)f, P.dt)));
        }
    }
    if (D == 2 && P.piston_drive) {
        // the piston (int_engine.rs:230-246): a soft wall at the step's piston height pushing down
        float f, s6;
        if (soft_wall_force(P.piston->w - xo[1], f, s6)) {
            k[1] = wadd(k[1], (int32_t)(0u - (uint32_t)rni_f32(__fmul_rn(f, c))));
            atomicAdd(&P.piston->force_fixed, (unsigned long long)sat_i64_f64(round_away(__dmul_rn((double)f, 65536.0))));
        }
    }
}

// One particle's step after its move (x = x_start + v, v = v_start + k + g with every kick): the
// heat bath if there is one, a blocked species' membrane crossing, a wall on a walled axis that
// it passed (mirrored back in and collided: hard and soft walls reverse the normal component, a
// thermal wall draws a new velocity on (id, step clock)), a crossing into another compartment,
// and the piston (int_engine.rs:265-336, int_engine3.rs:147-179, in that order). Returns whether
// it changed x or v. Periodic axes are wrapped only with `wrap_periodic` (cell lists).
template <int D>
__device__ __forceinline__ bool wall_post(const Params& P, uint32_t si, uint32_t id, uint32_t clock, int64_t* x, int32_t* v,
                                          unsigned long long* ledger, bool wrap_periodic) {
    bool changed = false;
    if (P.bath && bath_one<D>(P, si, id, clock, x, v, ledger + 3 * (size_t)GBMD_LEDGER_BATH * P.ledger_per_wall)) changed = true;
    const double m = P.masses[si];
    int64_t old[3];
#pragma unroll
    for (int a = 0; a < D; a++) old[a] = x[a] - (int64_t)v[a]; // the position before the move
    if (D == 2 && P.membrane && ((P.membrane_blocks >> si) & 1u)) {
        // the membrane (int_engine.rs:296-313, walls::cross_membrane walls.rs:18-25): a blocked
        // species that crossed it outside a pore is mirrored about position - 1/2
        const uint32_t a = P.membrane_axis;
        // (the other axis may be periodic and, with Verlet lists, left unwrapped between builds)
        const int64_t w = P.membrane_position, along = ((P.periodic >> (1 - a)) & 1u) ? wrap(old[1 - a], P.box[1 - a]) : old[1 - a];
        const bool pore = P.membrane_pore_shift != 0 && (along & (((int64_t)1 << P.membrane_pore_shift) - 1)) < P.membrane_pore_width;
        if (!pore && (old[a] < w) != (x[a] < w)) {
            const int face = old[a] < w ? 4 : 5; // walls::MEMBRANE faces (walls.rs:7-14)
            x[a] = 2 * w - 1 - x[a];
            const double vel_a = __ddiv_rn(__dmul_rn((double)v[a], 1.0 / 4294967296.0), P.dt);
            const double dp = __dmul_rn(__dmul_rn(2.0, m), fabs(vel_a));
            v[a] = (int32_t)(0u - (uint32_t)v[a]);
            unsigned long long* l = ledger_at<D>(P, ledger, face, (int)a, old);
            atomicAdd(l + 1, 1ull);
            atomicAdd(l + 2, ledger_fixed(dp));
            changed = true;
        }
    }
#pragma unroll
    for (int a = 0; a < D; a++) {
        if ((P.periodic >> a) & 1u) {
            if (wrap_periodic) x[a] = wrap(x[a], P.box[a]);
            continue;
        }
        int side = -1;
        if (x[a] < 0) {
            x[a] = -1 - x[a];
            side = 0;
        } else if (x[a] >= P.box[a]) {
            x[a] = 2 * P.box[a] - 1 - x[a];
            side = 1;
        }
        if (side < 0) {
            if (D == 2 && a < 2 && P.comp_shift[a]) {
                // a particle that crossed into another compartment is mirrored back into its home
                // one (int_engine.rs:324-330, walls::mirror_compartment walls.rs:72-78)
                const uint32_t sh = P.comp_shift[a];
                const int64_t home = old[a] >> sh;
                if ((x[a] >> sh) != home) {
                    const int64_t lo = home << sh, hi = (home + 1) << sh;
                    x[a] = x[a] < lo ? 2 * lo - 1 - x[a] : (x[a] >= hi ? 2 * hi - 1 - x[a] : x[a]);
                    v[a] = (int32_t)(0u - (uint32_t)v[a]);
                    changed = true;
                }
            }
            continue;
        }
        changed = true;
        double before[3], after[3];
        auto vel_of = [&](int32_t q) { return __ddiv_rn(__dmul_rn((double)q, 1.0 / 4294967296.0), P.dt); };
        auto step_of = [&](double q) { return sat_i32_f64(round_away(__dmul_rn(__dmul_rn(q, P.dt), 4294967296.0))); };
#pragma unroll
        for (int b = 0; b < D; b++) before[b] = vel_of(v[b]);
        if (P.wall_kind[a][side] == GBMD_WALL_THERMAL) {
            double vn, vt[2];
            thermal_velocity<D>(P, id, clock, P.wall_t[a][side], m, side == 0 ? 1.0 : -1.0, vn, vt);
            v[a] = step_of(vn);
            if (D == 2) {
                v[1 - a] = step_of(vt[0]);
            } else {
                v[(a + 1) % 3] = step_of(vt[0]);
                v[(a + 2) % 3] = step_of(vt[1]);
            }
        } else {
            v[a] = (int32_t)(0u - (uint32_t)v[a]);
        }
#pragma unroll
        for (int b = 0; b < D; b++) after[b] = vel_of(v[b]);
        auto ke = [&](const double* u) {
            double q = __dadd_rn(__dmul_rn(u[0], u[0]), __dmul_rn(u[1], u[1]));
            if (D == 3) q = __dadd_rn(q, __dmul_rn(u[2], u[2]));
            return __dmul_rn(__dmul_rn(0.5, m), q);
        };
        const double de = __dsub_rn(ke(after), ke(before));
        const double imp = fabs(__dmul_rn(m, __dsub_rn(before[a], after[a])));
        unsigned long long* l = ledger_at<D>(P, ledger, 2 * a + side, a, old);
        atomicAdd(l, ledger_fixed(de));
        atomicAdd(l + 1, 1ull);
        atomicAdd(l + 2, ledger_fixed(imp));
    }
    if (D == 2 && P.piston_drive) {
        const int64_t pw = P.piston->w; // mirrored below the piston (int_engine.rs:333-336)
        if (x[1] >= pw) {
            x[1] = 2 * pw - 1 - x[1];
            v[1] = (int32_t)(0u - (uint32_t)v[1]);
            changed = true;
        }
    }
    return changed;
}

// After the force step on a system with walls (when the force kernel did not take them itself):
// the step left v' = v + k + g and x' = x + v' with k the pair (and bond) kicks. This pass adds
// the walls' kicks, from the position at the step's start x' - v' (exact in integers), to v' and
// moves the particle from there again (the reference's x += v with the wrapped velocity sum), then
// runs wall_post.
template <int D, bool LIST>
__global__ void k_walls(Params P, PosRec<D>* __restrict__ pos, uint4* __restrict__ qpos, int32_t* __restrict__ vel,
                        const uint32_t* __restrict__ species, const uint32_t* __restrict__ ids, const PosRec<D>* __restrict__ ref_pos,
                        uint32_t* __restrict__ ctl, unsigned long long* __restrict__ ledger) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const uint32_t si = species[i], id = ids[i], clock = ctl[CTL_CLOCK];
    int64_t x[3] = {0, 0, 0};
    load_particle<D, false>(pos, nullptr, i, x);
    int32_t v[3] = {0, 0, 0};
#pragma unroll
    for (int a = 0; a < D; a++) v[a] = vel[D * i + a];
    int64_t xo[3] = {0, 0, 0};
#pragma unroll
    for (int a = 0; a < D; a++) xo[a] = x[a] - (int64_t)v[a];
    int32_t kw[3] = {0, 0, 0};
    wall_kicks<D>(P, xo, __fmul_rn(P.kick_cs[si], 1.0f / 268435456.0f), kw, ledger); // kick_coeff in f32
    bool changed = false;
#pragma unroll
    for (int a = 0; a < D; a++)
        if (kw[a]) {
            v[a] = wadd(v[a], kw[a]);
            x[a] = xo[a] + (int64_t)v[a];
            changed = true;
        }
    if (wall_post<D>(P, si, id, clock, x, v, ledger, !LIST)) changed = true;
    if (!changed) return;
#pragma unroll
    for (int a = 0; a < D; a++) vel[D * i + a] = v[a];
    store_pos<D>(pos, i, x, si);
    if (LIST) {
        qpos[i] = quot_record<D>(x, si);
        int64_t xr[3];
        load_particle<D, false>(ref_pos, nullptr, i, xr);
        if (moved_half_skin<D>(P, xr, x)) ctl[0] = 1;
    }
}

// walls::piston_kick (walls.rs:143-146): F dt^2 / M in position units, rounded half away from
// zero, in the reference's f64 order.
__device__ __forceinline__ int32_t piston_kick(const Params& P, double net) {
    return sat_i32_f64(round_away(__dmul_rn(__ddiv_rn(__dmul_rn(__dmul_rn(net, P.dt), P.dt), P.piston_mass), 4294967296.0)));
}
// After the walls pass: IntEngine::move_piston (int_engine.rs:346-361) on the step's force sum
// (a free piston's kick, the drift, the stops, the work), then the step clock advances.
static __global__ void k_piston_tick(Params P, uint32_t* ctl) {
    PistonState& ps = *P.piston;
    const double gas = __dmul_rn(__ll2double_rn((long long)ps.force_fixed), 1.0 / 65536.0);
    ps.force_fixed = 0ull;
    ps.gas = gas;
    if (P.piston_drive == 2) ps.v = wadd(ps.v, piston_kick(P, __dsub_rn(gas, P.piston_ext)));
    const int64_t old = ps.w;
    int64_t w = old + (int64_t)ps.v;
    if (w < P.piston_lo || w > P.piston_hi) {
        w = w < P.piston_lo ? P.piston_lo : P.piston_hi;
        ps.v = 0;
    }
    ps.w = w;
    ps.work = __dadd_rn(ps.work, __dmul_rn(gas, to_f64(w - old)));
    ctl[CTL_CLOCK] += 1u;
}
// Reversal's piston step (int_engine.rs:404-410): v <- -(v + kick), a free piston's kick from the
// force the reversing kicks pass summed.
static __global__ void k_piston_reverse(Params P) {
    PistonState& ps = *P.piston;
    const double gas = __dmul_rn(__ll2double_rn((long long)ps.force_fixed), 1.0 / 65536.0);
    ps.force_fixed = 0ull;
    const int32_t kick = P.piston_drive == 2 ? piston_kick(P, __dsub_rn(gas, P.piston_ext)) : 0;
    ps.v = (int32_t)(0u - (uint32_t)wadd(ps.v, kick));
}

// Cell-list force + leapfrog (ForceMode::CellList; md.wgsl:39-76): scans the 3^D cells of the
// sorted scratch state and writes the moved state back into the engine's arrays.
template <int D, bool MULTI, bool INT = false>
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
            if (D == 2 && P.comp_filter && !same_compartment(P.comp_shift, xi, xj)) continue; // int_engine.rs:161-163
            if constexpr (INT) {
                int64_t d[3] = {0, 0, 0};
#pragma unroll
                for (int a = 0; a < D; a++) d[a] = min_image(xj[a] - xi[a], P.box[a], P.half[a]);
                int_kick<D>(P, si * P.ns + sj, d, k);
            } else {
                float fr, s6, r2;
                pair_kick<D>(P, P.pc[si * P.ns + sj], cs, xi, xj, k, fr, s6, r2);
            }
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
template <int D, bool MULTI, bool INT = false>
__global__ void __launch_bounds__(128) k_kicks(Params P, const PosRec<D>* __restrict__ pos, const uint32_t* __restrict__ species,
                                               const uint32_t* __restrict__ ids,
                                               const uint32_t* __restrict__ nbr, const uint32_t* __restrict__ nbr_count,
                                               const uint32_t* __restrict__ keys, const uint32_t* __restrict__ start,
                                               int32_t* __restrict__ vel, int32_t* __restrict__ kicks, double* __restrict__ partial,
                                               int reverse) {
    __shared__ double sh[4][4];
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    double pe = 0.0, w = 0.0, ke = 0.0, gpe = 0.0;
    F32Sum pe32, w32; // the f32 chain's pair terms, summed without f64 arithmetic
    if (i < P.n) {
        int64_t xi[3];
        uint32_t si = load_particle<D, MULTI>(pos, species, i, xi);
        const float cs = P.kick_cs[si];
        int32_t k[3] = {0, 0, 0};
        auto visit = [&](uint32_t j) {
            int64_t xj[3];
            uint32_t sj = load_particle<D, MULTI>(pos, species, j, xj);
            if (D == 2 && P.comp_filter && !same_compartment(P.comp_shift, xi, xj)) return; // int_engine.rs:161-163
            if constexpr (INT) {
                int64_t d[3] = {0, 0, 0};
#pragma unroll
                for (int a = 0; a < D; a++) d[a] = min_image(xj[a] - xi[a], P.box[a], P.half[a]);
                if (int_kick<D>(P, si * P.ns + sj, d, k)) {
                    double r2 = 0.0;
#pragma unroll
                    for (int a = 0; a < D; a++) {
                        const double x = __dmul_rn((double)d[a], 1.0 / 4294967296.0);
                        r2 = __dadd_rn(r2, __dmul_rn(x, x));
                    }
                    double u, fr;
                    pair_f64(P.ipair + 4 * (si * P.ns + sj), r2, u, fr);
                    pe += u;
                    w += __dmul_rn(fr, r2);
                }
            } else {
                const PairC& pc = P.pc[si * P.ns + sj];
                float fr, s6, r2;
                if (pair_kick<D>(P, pc, cs, xi, xj, k, fr, s6, r2)) {
                    pe32.add(pair_u(pc, s6));
                    w32.add(__fmul_rn(fr, r2));
                }
            }
        };
        if (nbr) {
            uint32_t m = nbr_count[i];
            const uint32_t cap4 = (P.cap + 3u) & ~3u;
            for (uint32_t q = 0; q < m; q++) visit(nbr[list_slot(i, q, cap4)] & LIST_MASK);
        } else {
            uint32_t c[3];
            cell_coords(P, keys[i], c);
            for_cells<D>(P, c, [&](uint32_t cell) {
                for (uint32_t j = start[cell]; j < start[cell + 1]; j++)
                    if (j != i) visit(j);
            });
        }
        if constexpr (!INT) {
            pe = pe32.value();
            w = w32.value();
        }
        pe *= 0.5;
        w *= 0.5;
        if (P.bonds) // (slot_of holds this array's slots)
            pe += 0.5 * (double)bond_kicks<D>(P, ids[i], xi, pos, __fmul_rn(cs, 1.0f / 268435456.0f), k);
        if (P.walls) {
            // the soft walls' kicks and potential (int_engine.rs:203-227, int_engine3.rs:107-126)
            const float c = __fmul_rn(cs, 1.0f / 268435456.0f);
#pragma unroll
            for (int a = 0; a < D; a++) {
                if ((P.periodic >> a) & 1u) continue;
#pragma unroll
                for (int side = 0; side < 2; side++) {
                    float f, s6;
                    if (P.wall_kind[a][side] != GBMD_WALL_SOFT || !soft_wall_force(side == 0 ? xi[a] : P.box[a] - xi[a], f, s6)) continue;
                    const int32_t kw = rni_f32(__fmul_rn(f, c));
                    k[a] = wadd(k[a], side == 0 ? kw : (int32_t)(0u - (uint32_t)kw));
                    pe += (double)__fadd_rn(__fmul_rn(__fmul_rn(4.0f, s6), __fsub_rn(s6, 1.0f)), 1.0f);
                }
            }
            float f, s6; // the piston (int_engine.rs:230-246); reversing sums its force for its own kick
            if (D == 2 && P.piston_drive && soft_wall_force(P.piston->w - xi[1], f, s6)) {
                k[1] = wadd(k[1], (int32_t)(0u - (uint32_t)rni_f32(__fmul_rn(f, c))));
                pe += (double)__fadd_rn(__fmul_rn(__fmul_rn(4.0f, s6), __fsub_rn(s6, 1.0f)), 1.0f);
                if (reverse) atomicAdd(&P.piston->force_fixed, (unsigned long long)sat_i64_f64(round_away(__dmul_rn((double)f, 65536.0))));
            }
        }
        // IntEngine::energy / IntEngine3::energy (int_engine.rs:433-446, int_engine3.rs:222-239):
        // the on-step velocity 0.5 (velocity(v) + velocity(next)), velocity(v) = v UNIT / dt, so
        // 0.5 m vh^2 = m (v + next)^2 UNIT^2 / (8 dt^2); the sum of m (v + next)^2 (exact integers
        // squared in f64) is scaled by UNIT^2 / (8 dt^2) on the host (no f64 division per particle:
        // f64 runs at a small fraction of the f32 rate on this GPU). 3D leaves pinned species out.
        // The gravity potential -m g . x goes to its own partial (the kicks' potential has none).
        const double m = P.masses[si];
        const bool counted = !(D == 3 && ((P.pinned >> si) & 1u));
        for (int a = 0; a < D; a++) {
            int32_t v0 = vel[D * i + a];
            int32_t next = wadd(wadd(v0, k[a]), P.gravity[a]);
            const double sv = (double)((int64_t)v0 + (int64_t)next);
            if (counted) {
                ke = __fma_rn(__dmul_rn(m, sv), sv, ke);
                if (P.grav_f[a] != 0.0) {
                    const int64_t xa = ((P.periodic >> a) & 1u) ? wrap(xi[a], P.box[a]) : xi[a];
                    gpe = __fma_rn(-__dmul_rn(m, P.grav_f[a]), to_f64(xa), gpe);
                }
            }
            if (kicks) kicks[D * i + a] = k[a];
            if (reverse) {
                bool pinned = (P.pinned >> si) & 1u;
                vel[D * i + a] = (int32_t)(0u - (uint32_t)wadd(wadd(v0, k[a]), pinned ? 0 : P.gravity[a]));
            }
        }
    }
    if (!partial) return;
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
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

// ---------------------------------------------------------------- FP64 reference kicks
// The pair constants of IntEngine<f64> (real.rs:105-157 with F = f64): rounded from the f64
// pair parameters, not through f32.
struct PairsF64 {
    double rc2[GBMD_MAX_SPECIES * GBMD_MAX_SPECIES], eps4[GBMD_MAX_SPECIES * GBMD_MAX_SPECIES];
    double sigma2[GBMD_MAX_SPECIES * GBMD_MAX_SPECIES], shift[GBMD_MAX_SPECIES * GBMD_MAX_SPECIES];
    double six_eps4[GBMD_MAX_SPECIES * GBMD_MAX_SPECIES];
    double kick_c[GBMD_MAX_SPECIES]; // kick_coeff (system.rs:415-420), unscaled
};
// Per-particle kicks of IntEngine<f64>::forces (int_engine.rs:130-251): separations to_f64
// (dropped beyond 8 sigma), PairConsts::eval in f64 left to right without fusion, each pair's
// kick rint(-fr c d) saturated to i32 and summed with wrapping adds; pe += u in list order.
// Walks the Verlet list (a superset of the f64 cutoff sphere) or the 3^D cells.
template <int D, bool MULTI>
__global__ void __launch_bounds__(128) k_kicks_f64(Params P, PairsF64 Q, const PosRec<D>* __restrict__ pos, const uint32_t* __restrict__ species,
                                                   const uint32_t* __restrict__ nbr, const uint32_t* __restrict__ nbr_count,
                                                   const uint32_t* __restrict__ keys, const uint32_t* __restrict__ start,
                                                   int32_t* __restrict__ kicks, double* __restrict__ pe_out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    int64_t xi[3];
    uint32_t si = load_particle<D, MULTI>(pos, species, i, xi);
    const double c = Q.kick_c[si];
    int32_t k[3] = {0, 0, 0};
    double pe = 0.0;
    auto visit = [&](uint32_t j) {
        int64_t xj[3];
        uint32_t sj = load_particle<D, MULTI>(pos, species, j, xj);
        double f[3];
#pragma unroll
        for (int a = 0; a < D; a++) {
            int64_t d = min_image(xj[a] - xi[a], P.box[a], P.half[a]);
            if (!(d >= -((int64_t)8 << 32) && d < ((int64_t)8 << 32))) return;
            f[a] = __dmul_rn((double)d, 1.0 / 4294967296.0);
        }
        const uint32_t q = si * P.ns + sj;
        double r2 = __dadd_rn(__dmul_rn(f[0], f[0]), __dmul_rn(f[1], f[1]));
        if (D == 3) r2 = __dadd_rn(r2, __dmul_rn(f[2], f[2]));
        if (!(r2 < Q.rc2[q])) return;
        double s2 = __ddiv_rn(Q.sigma2[q], r2);
        double s6 = __dmul_rn(__dmul_rn(s2, s2), s2);
        double fr = __ddiv_rn(__dmul_rn(__dmul_rn(Q.six_eps4[q], s6), __dsub_rn(__dmul_rn(2.0, s6), 1.0)), r2);
        double u = __dsub_rn(__dmul_rn(__dmul_rn(Q.eps4[q], s6), __dsub_rn(s6, 1.0)), Q.shift[q]);
        double am = __dmul_rn(-fr, c);
#pragma unroll
        for (int a = 0; a < D; a++) k[a] = wadd(k[a], sat_i32_f64(rint(__dmul_rn(am, f[a]))));
        pe = __dadd_rn(pe, u);
    };
    if (nbr) {
        uint32_t m = nbr_count[i];
        const uint32_t cap4 = (P.cap + 3u) & ~3u;
        for (uint32_t q = 0; q < m; q++) visit(nbr[list_slot(i, q, cap4)] & LIST_MASK);
    } else {
        uint32_t cc[3];
        cell_coords(P, keys[i], cc);
        for_cells<D>(P, cc, [&](uint32_t cell) {
            for (uint32_t j = start[cell]; j < start[cell + 1]; j++)
                if (j != i) visit(j);
        });
    }
#pragma unroll
    for (int a = 0; a < D; a++) kicks[D * i + a] = k[a];
    pe_out[i] = 0.5 * pe;
}

// ---------------------------------------------------------------- velocity-rescale thermostat
// The half-step kinetic energy summed exactly: per block and species, the 128-bit sum of v^2 over
// the moving particles' velocity components (part[8 b + 2 s + {0: low, 1: high}]).
template <int D>
__global__ void k_ke_exact(uint32_t n, const int32_t* __restrict__ vel, const uint32_t* __restrict__ species, uint32_t pinned,
                           unsigned long long* __restrict__ part) {
    __shared__ unsigned long long lo[GBMD_MAX_SPECIES][256], hi[GBMD_MAX_SPECIES][256];
    unsigned __int128 acc[GBMD_MAX_SPECIES] = {0, 0, 0, 0};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t s = species[i];
        if ((pinned >> s) & 1u) continue;
        for (int a = 0; a < D; a++) {
            long long v = vel[D * i + a];
            acc[s & 3] += (unsigned __int128)(unsigned long long)(v * v);
        }
    }
    for (int s = 0; s < GBMD_MAX_SPECIES; s++) {
        lo[s][threadIdx.x] = (unsigned long long)acc[s];
        hi[s][threadIdx.x] = (unsigned long long)(acc[s] >> 64);
    }
    __syncthreads();
    if (threadIdx.x < GBMD_MAX_SPECIES) {
        unsigned __int128 t = 0;
        for (uint32_t k = 0; k < blockDim.x; k++) t += ((unsigned __int128)hi[threadIdx.x][k] << 64) | lo[threadIdx.x][k];
        part[8 * blockIdx.x + 2 * threadIdx.x] = (unsigned long long)t;
        part[8 * blockIdx.x + 2 * threadIdx.x + 1] = (unsigned long long)(t >> 64);
    }
}

struct ThermoP {
    uint32_t nblocks, ns;
    double masses[GBMD_MAX_SPECIES];
    double dt, dof, t;
};
// fac[0] = sqrt(t / now) with now = KE / dof, KE = sum_s 1/2 m_s S_s (UNIT / dt)^2 in f64 in
// species order; fac[1] = 1 when now <= 0 (set_temperature then leaves the state alone).
// One block of 256 threads: the per-block integer sums added in 128 bits (exact, so in any
// order), then one thread's f64 arithmetic.
static __global__ void k_thermo_factor(ThermoP T, const unsigned long long* __restrict__ part, double* __restrict__ fac) {
    __shared__ unsigned long long lo[GBMD_MAX_SPECIES][256], hi[GBMD_MAX_SPECIES][256];
    for (uint32_t s = 0; s < T.ns; s++) {
        unsigned __int128 S = 0;
        for (uint32_t b = threadIdx.x; b < T.nblocks; b += blockDim.x) S += ((unsigned __int128)part[8 * b + 2 * s + 1] << 64) | part[8 * b + 2 * s];
        lo[s][threadIdx.x] = (unsigned long long)S;
        hi[s][threadIdx.x] = (unsigned long long)(S >> 64);
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    double ke = 0.0;
    double u = __ddiv_rn(1.0 / 4294967296.0, T.dt);
    for (uint32_t s = 0; s < T.ns; s++) {
        unsigned __int128 S = 0;
        for (uint32_t k = 0; k < blockDim.x; k++) S += ((unsigned __int128)hi[s][k] << 64) | lo[s][k];
        double sum = __dadd_rn(__dmul_rn(__ull2double_rn((unsigned long long)(S >> 64)), 18446744073709551616.0),
                               __ull2double_rn((unsigned long long)S));
        ke = __dadd_rn(ke, __dmul_rn(__dmul_rn(__dmul_rn(0.5, T.masses[s]), sum), __dmul_rn(u, u)));
    }
    double now = __ddiv_rn(ke, T.dof);
    bool skip = !(now > 0.0);
    fac[0] = skip ? 1.0 : __dsqrt_rn(__ddiv_rn(T.t, now));
    fac[1] = skip ? 1.0 : 0.0;
}

// (v as f64 * f).round() as i32 (init.rs:99-101: the velocity rescale) in integer arithmetic,
// for f = m 2^e with m the 53-bit significand of a normal positive f64: the exact product |v| m
// (at most 85 bits, in two 64-bit words) rounded to nearest-even at 53 significant bits, which is
// the f64 multiply's rounding, then half away from zero to an integer, saturating as Rust's `as`
// conversion does. The same value as sat_i32_f64(round(__dmul_rn((double)v, f))), without the
// FP64 pipe, which runs at a small fraction of the integer rate on this GPU.
__device__ __forceinline__ int32_t rescale_i32(int32_t v, uint64_t m, int e) {
    if (v == 0) return 0;
    const uint64_t a = v < 0 ? (uint64_t)0 - (uint64_t)(int64_t)v : (uint64_t)v; // |v| <= 2^31
    const uint64_t lo = a * m, hi = __umul64hi(a, m);
    const int L = hi ? 128 - __clzll((long long)hi) : 64 - __clzll((long long)lo); // bits of |v| m
    int s = L - 53;
    uint64_t q = lo;
    if (s > 0) { // (s <= 32: |v| m < 2^85)
        q = (lo >> s) | (hi << (64 - s));
        const uint64_t rem = lo & ((1ull << s) - 1), half = 1ull << (s - 1);
        if (rem > half || (rem == half && (q & 1ull))) {
            q += 1;
            if (q == (1ull << 53)) {
                q >>= 1;
                s += 1;
            }
        }
    } else {
        s = 0;
    }
    const int t = e + s; // |v f| rounded to f64 is q 2^t, q < 2^53
    uint64_t r;
    if (t >= 0) r = ~0ull; // at least 2^52: saturates
    else if (-t >= 54) r = 0; // below one half
    else r = (q + (1ull << (-t - 1))) >> (-t); // half away from zero, on the magnitude
    if (v > 0) return r > 2147483647ull ? INT32_MAX : (int32_t)r;
    return r > 2147483648ull ? INT32_MIN : (int32_t)(0u - (uint32_t)r);
}

// The velocity sums of the moving particles: the per-block partials vpart[3 b + a] added by one
// block of 256 threads (integers: exact in any order) into tot[a].
static __global__ void k_vsum(const long long* __restrict__ vpart, uint32_t nblocks, long long* __restrict__ tot) {
    __shared__ long long sh[3][256];
    for (int a = 0; a < 3; a++) {
        long long t = 0;
        for (uint32_t b = threadIdx.x; b < nblocks; b += blockDim.x) t += vpart[3 * b + a];
        sh[a][threadIdx.x] = t;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        long long t = 0;
        for (uint32_t k = 0; k < blockDim.x; k++) t += sh[threadIdx.x][k];
        tot[threadIdx.x] = t;
    }
}

// v <- round(v f) as i32 for moving particles (init.rs:99-101), then per-block sums of the new
// velocities of moving particles (vpart[3 b + a]).
template <int D>
__global__ void k_rescale(uint32_t n, int32_t* __restrict__ vel, const uint32_t* __restrict__ species, uint32_t pinned,
                          const double* __restrict__ fac, long long* __restrict__ vpart) {
    __shared__ long long sh[3][32];
    const double f = fac[0];
    const bool skip = fac[1] != 0.0;
    // f = m 2^e; a zero, subnormal or non-finite f takes the f64 path
    const uint64_t fb = (uint64_t)__double_as_longlong(f);
    const uint32_t fe = (uint32_t)(fb >> 52) & 0x7ffu;
    const bool ints = !(fb >> 63) && fe != 0u && fe != 0x7ffu;
    const uint64_t m = (fb & ((1ull << 52) - 1)) | (1ull << 52);
    const int e = (int)fe - 1075;
    long long acc[3] = {0, 0, 0};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if ((pinned >> species[i]) & 1u) continue;
        for (int a = 0; a < D; a++) {
            int32_t v = vel[D * i + a];
            if (!skip) {
                v = ints ? rescale_i32(v, m, e) : sat_i32_f64(round(__dmul_rn((double)v, f)));
                vel[D * i + a] = v;
            }
            acc[a] += v;
        }
    }
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int a = 0; a < 3; a++) {
        long long v = acc[a];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) sh[a][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        long long t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sh[threadIdx.x][w];
        vpart[3 * blockIdx.x + threadIdx.x] = t;
    }
}

// zero_velocity_sum over the moving particles in id order (init.rs:76-89 / three.rs:376-389):
// the k-th moving particle loses q + (k < r), q = div_euclid(sum, m), r = rem_euclid(sum, m);
// mrank[id] is k.
template <int D>
__global__ void k_zero_apply(uint32_t n, int32_t* __restrict__ vel, const uint32_t* __restrict__ species, const uint32_t* __restrict__ ids,
                             const uint32_t* __restrict__ mrank, uint32_t pinned, uint32_t moving, const long long* __restrict__ tot,
                             const double* __restrict__ fac) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || fac[1] != 0.0 || moving == 0 || ((pinned >> species[i]) & 1u)) return;
    long long m = moving, k = mrank[ids[i]];
    for (int a = 0; a < D; a++) {
        long long q = tot[a] / m, r = tot[a] % m;
        if (r < 0) {
            q -= 1;
            r += m;
        }
        vel[D * i + a] = (int32_t)((uint32_t)vel[D * i + a] - (uint32_t)(q + (k < r ? 1 : 0)));
    }
}

// ---------------------------------------------------------------- RDF bins
// The exact bin of a pair whose f32 estimate was too close to a bin edge or to rmax.
template <int D> __device__ __forceinline__ int rdf_bin_exact(const int64_t* d, uint32_t bins, double scale) {
    double r2 = 0.0;
#pragma unroll
    for (int a = 0; a < D; a++) {
        const double x = to_f64(d[a]);
        r2 = __dadd_rn(r2, __dmul_rn(x, x));
    }
    const double r = __dmul_rn(__dsqrt_rn(r2), scale);
    return r < (double)bins ? (int)(uint32_t)r : -1;
}

// The RDF bin of a pair at minimum-image separation d: k = floor(sqrt(r2) bins / rmax) with r2
// the f64 square of the exact separation, or -1 beyond rmax. Decided in f32 when that is safe:
// the f32 estimate of r bins / rmax is within 3.3e-7 of it relatively plus 2^-24 sqrt(D) sigma
// (separations truncated to 2^-24 sigma and rounded to f32 through a 32-bit conversion, a fused
// sum of squares, a square root, one product), so a pair farther than `margin` bins from a bin
// edge, or clearly beyond rmax (r2 above lim2f), is binned without f64 arithmetic, which runs at
// a small fraction of the f32 rate on this GPU (so does a 64-bit integer conversion); the rest
// takes the f64 definition, as does any pair 64 sigma or more apart on an axis.
template <int D>
__device__ __forceinline__ int rdf_bin(const int64_t* d, uint32_t bins, double scale, float scalef, float lim2f, float margin) {
    float r2f = 0.0f;
#pragma unroll
    for (int a = 0; a < D; a++) {
        if (d[a] >= ((int64_t)1 << 38) || d[a] <= -((int64_t)1 << 38)) return rdf_bin_exact<D>(d, bins, scale);
        const float x = __fmul_rn(__int2float_rn((int32_t)(d[a] >> 8)), 0x1p-24f);
        r2f = __fmaf_rn(x, x, r2f);
    }
    if (r2f > lim2f) return -1;
    const float rf = __fmul_rn(__fsqrt_rn(r2f), scalef);
    const float fl = floorf(rf), fr = rf - fl;
    if (fr > margin && fr < 1.0f - margin && rf < (float)bins - margin) return (int)fl;
    return rdf_bin_exact<D>(d, bins, scale);
}

} // namespace gbmd
