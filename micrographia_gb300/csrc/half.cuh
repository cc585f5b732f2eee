// The half-shell force path of 3D single-species systems (GBMD_FLAG_HALF_LISTS): each unordered
// pair within the list radius is listed, and its pair chain evaluated, once. It is exact but not
// the default: on GB300 at 3D N = 2^20 the step's forces take 0.34 ms this way against 0.245 ms
// with full lists. Per listed pair it costs ~110 thread instructions against ~75 (the window
// lookup, the j-end's shared-memory atomics, the saturation check), the halved lists are twice as
// uneven in length within a warp (lane efficiency ~0.8 against ~0.94), and the leapfrog needs a
// pass of its own. Its list build is cheaper (0.75 against 0.85 ms).
//
// md-ref evaluates a pair once in its fast path too (crates/md-ref/src/fast.rs:83-222, the half
// shell), rounding each end's kick on its own: kick_i = rint(a f) and kick_j = rint(a (-f))
// (fast.rs:240-246). With one species a_i = a_j, and since the separation is antisymmetric
// (sep(-d) = -sep(d) exactly, fixed.rs:90-98) and rint is odd, kick_j is the negation of kick_i
// except where the conversion saturated (kick_mirror). Kicks are summed as wrapping 32-bit
// integers, so the order in which a particle's kicks arrive does not change its sum: the
// trajectory equals the full-list engine's and md-ref's bit for bit.
//
// Ownership: a half space per particle. Particle i owns its pair with j when the separation
// d = xj - xi (at the list build, the exact integer one at the pair's periodic image) is positive
// in its last nonzero coordinate taken in the order z, y, x; when d = 0, the lower slot owns it if
// the two slots' sum is odd, the higher if even. d is antisymmetric, so exactly one end owns each
// pair, and every particle owns about half of its neighbours whatever its place in its cell (a
// rule by cells alone gives a particle near the top of its cell far more pairs than one near the
// bottom, and the warps' lanes would wait on the longest). The list build decides by the f32
// offsets it already has, and by the exact integers when |dz| is within 1e-5 sigma.
//
// Cells are stored row-major (x fastest), so the particles of one x-row of cells (y, z) are one
// contiguous storage range. A particle's owned neighbours lie in the cells of its own layer and
// the layer above: six rows, windows w = 3 dz + dy + 1 for dz in {0, 1}, dy in {-1, 0, 1}
// (periodic; the row itself is window 1). The force step runs one block per row; the kicks of the
// j-ends of its pairs are summed in shared memory per window slot with 32-bit atomics, then each
// window is added to the global per-particle accumulators with coalesced reductions. Each row is
// window w of exactly one block for each w. A list entry names its neighbour by window and offset
// in that window's row, so the kernel needs no search. A separate pass applies the leapfrog and
// the rebuild trigger, and clears the accumulators for the next step.
#pragma once

#include "kernels.cuh"

namespace gbmd {

constexpr uint32_t HALF_OFF_BITS = 16;                       // offset of the neighbour in its row
constexpr uint32_t HALF_OFF_MASK = (1u << HALF_OFF_BITS) - 1u;
constexpr uint32_t HALF_WIN_SHIFT = HALF_OFF_BITS;            // then 4 bits of window index
constexpr uint32_t HALF_WINDOWS = 6;                          // three rows of the layer, three of the next
constexpr uint32_t HALF_OWN_WINDOW = 1;                       // the row itself
constexpr uint32_t HALF_THREADS = 256;
constexpr uint32_t HALF_NO_SLOT = 0xffffffffu;                // a window kept in global memory

// rint(a (-f)) from k = rint(a f): the negation, except where the conversion saturated. f32 values
// of magnitude near 2^31 are multiples of 128, so INT32_MAX only comes from a f >= 2^31 (then
// -a f <= -2^31 gives INT32_MIN) and INT32_MIN from a f <= -2^31 (then INT32_MAX).
__device__ __forceinline__ int32_t kick_mirror(int32_t k) {
    return (k == INT32_MIN || k == INT32_MAX) ? ~k : (int32_t)(0u - (uint32_t)k);
}

// Does particle i own its pair with cell-mate j? Lower slot when i + j is odd, higher when even.
__device__ __forceinline__ bool owns_in_cell(uint32_t i, uint32_t j) { return ((i ^ j) & 1u) ? (j > i) : (j < i); }

// The row key of window w = 3 dz + dy + 1 of row (y, z).
__host__ __device__ __forceinline__ uint32_t half_window_row(uint32_t ny, uint32_t nz, uint32_t y, uint32_t z, uint32_t w) {
    const uint32_t dz = w / 3u, dy1 = w % 3u; // dy + 1
    return ((z + dz) % nz) * ny + (y + ny + dy1 - 1u) % ny;
}

// The half list of each particle (3D, one species, one lane per particle): the list definition of
// k_build_list (md3.wgsl:443-483 with the exact f32 test) restricted to the pairs the particle
// owns (the half space above). An entry is the neighbour's offset in its row (16 bits), its window (bits 16-19) and the
// periodic image (bits 26-31, as in full lists). A row of more than 65,536 particles cannot be
// addressed: the build then reports an overflow.
__global__ void __launch_bounds__(128) k_build_half(Params P, const PosRec<3>* __restrict__ pos_s, const int32_t* __restrict__ vel_s,
                                                    const uint32_t* __restrict__ species_s, const uint32_t* __restrict__ ids_s,
                                                    const uint32_t* __restrict__ keys, const uint32_t* __restrict__ start,
                                                    const float4* __restrict__ relf, PosRec<3>* __restrict__ pos_o,
                                                    int32_t* __restrict__ vel_o, uint32_t* __restrict__ species_o,
                                                    uint32_t* __restrict__ ids_o, PosRec<3>* __restrict__ ref_pos,
                                                    uint32_t* __restrict__ nbr, uint32_t* __restrict__ nbr_count,
                                                    uint32_t* __restrict__ ctl, uint4* __restrict__ qpos_o) {
    constexpr int D = 3;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {
        ctl[0] = 0; // the rebuild is done: clear the trigger, count it
        ctl[2] += 1;
    }
    if (i >= P.n) return;
    int64_t xi[3];
    load_particle<D, false>(pos_s, species_s, i, xi);
    uint32_t c[3];
    cell_coords(P, keys[i], c);
    uint32_t count = 0;
    bool far = false; // a neighbour more than 65,536 slots into its row
    const uint32_t cap = P.cap, cap4 = (P.cap + 3u) & ~3u;
    const size_t lbase = list_slot(i, 0, cap4);
    const bool unchecked = P.sep_unchecked;
    int64_t reli[3];
#pragma unroll
    for (int a = 0; a < 3; a++) reli[a] = xi[a] - (int64_t)c[a] * P.cell_w[a];
    auto exact = [&](uint32_t j, const int64_t* xs) -> bool {
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
        r2 = __fadd_rn(r2, __fmul_rn(f[2], f[2]));
        return ok && r2 < P.pc[0].list2s;
    };
    // the exact half-space test on the integer separation at the candidate's image
    auto owns_exact = [&](uint32_t j, const int64_t* xs) -> bool {
        int64_t xj[3];
        load_particle<D, false>(pos_s, nullptr, j, xj);
#pragma unroll
        for (int a = 2; a >= 0; a--) {
            const int64_t d = xj[a] - xs[a];
            if (d != 0) return d > 0;
        }
        return owns_in_cell(i, j);
    };
    constexpr float EPS = 1e-5f; // sigma: far above the f32 offsets' error
    const float lo = P.pc[0].list2lo, hi = P.pc[0].list2hi;
    const uint32_t nx = P.nc[0], ny = P.nc[1], nz = P.nc[2];
    for (int oz = 1; oz < 3; oz++) { // (the layer below holds no owned neighbour)
        int tz = (int)c[2] + oz - 1;
        uint32_t z = tz < 0 ? nz - 1 : (tz >= (int)nz ? 0 : (uint32_t)tz);
        int64_t sz = tz < 0 ? -P.box[2] : (tz >= (int)nz ? P.box[2] : 0);
        const bool same_layer = oz == 1;
        for (int oy = 0; oy < 3; oy++) {
            const uint32_t w = 3u * (uint32_t)(oz - 1) + (uint32_t)oy;
            int ty = (int)c[1] + oy - 1;
            uint32_t y = ty < 0 ? ny - 1 : (ty >= (int)ny ? 0 : (uint32_t)ty);
            int64_t sy = ty < 0 ? -P.box[1] : (ty >= (int)ny ? P.box[1] : 0);
            const uint32_t r2k = z * ny + y;
            const uint32_t row0 = __ldg(start + (size_t)r2k * nx);
            for (int ox = 0; ox < 3; ox++) {
                int tx = (int)c[0] + ox - 1;
                uint32_t x = tx < 0 ? nx - 1 : (tx >= (int)nx ? 0 : (uint32_t)tx);
                int64_t sx = tx < 0 ? -P.box[0] : (tx >= (int)nx ? P.box[0] : 0);
                uint32_t cell = r2k * nx + x;
                const int64_t xs[3] = {xi[0] - sx, xi[1] - sy, xi[2] - sz};
                const uint32_t tag = ((uint32_t)w << HALF_WIN_SHIFT) | image_code(sx, sy, sz);
                const float b0 = off_f32(((int64_t)x - (int64_t)c[0]) * P.cell_w[0] + sx - reli[0]);
                const float b1 = off_f32(((int64_t)y - (int64_t)c[1]) * P.cell_w[1] + sy - reli[1]);
                const float b2 = off_f32(((int64_t)z - (int64_t)c[2]) * P.cell_w[2] + sz - reli[2]);
                const uint32_t j0 = __ldg(start + cell), j1 = __ldg(start + cell + 1);
                far |= j1 > row0 + HALF_OFF_MASK + 1u;
                // the one-lane walk of k_build_list: appends below the band's lower edge, marks a
                // band candidate for a second, exact walk
                bool band = false;
#pragma unroll 4
                for (uint32_t j = j0; j < j1; j++) {
                    const float4 r = __ldg(relf + j);
                    const float dx = r.x + b0, dy = r.y + b1, dz = r.z + b2;
                    const float r2a = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
                    // (in the layer above every candidate is owned; |dz| within EPS: the exact test)
                    const bool near = same_layer && fabsf(dz) <= EPS && r2a <= hi && j != i;
                    const bool mine = !same_layer || dz > EPS || (near && owns_exact(j, xs));
                    const bool in = r2a < lo && j != i && mine;
                    band |= r2a >= lo && r2a <= hi && mine;
                    const size_t at = lbase + ((size_t)(count & ~3u) << 5) + (count & 3u);
                    if (in && count < cap) nbr[at] = ((j - row0) & HALF_OFF_MASK) | tag;
                    count += in ? 1u : 0u;
                }
                if (band)
                    for (uint32_t j = j0; j < j1; j++) {
                        const float4 r = __ldg(relf + j);
                        const float dx = r.x + b0, dy = r.y + b1, dz = r.z + b2;
                        const float r2a = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
                        const bool near = same_layer && fabsf(dz) <= EPS && j != i;
                        const bool mine = !same_layer || dz > EPS || (near && owns_exact(j, xs));
                        if (r2a >= lo && r2a <= hi && j != i && mine && exact(j, xs)) {
                            if (count < cap) nbr[lbase + ((size_t)(count & ~3u) << 5) + (count & 3u)] = ((j - row0) & HALF_OFF_MASK) | tag;
                            count++;
                        }
                    }
            }
        }
    }
    if (count > cap || far) {
        ctl[1] = 1;
        count = count > cap ? cap : count;
    }
    nbr_count[i] = count;
    pos_o[i] = pos_s[i];
    ref_pos[i] = pos_s[i];
    if (qpos_o) qpos_o[i] = quot_record<D>(xi, 0u);
#pragma unroll
    for (int a = 0; a < D; a++) vel_o[D * i + a] = vel_s[D * i + a];
    species_o[i] = species_s[i];
    ids_o[i] = ids_s[i];
}

// Two pairs of one particle in packed f32x2 arithmetic, as pair_kicks2_sig1, returning each pair's
// kick, whether the pair is within the cutoff (a pair beyond it, or a slot past the list end,
// gets zero kicks) and whether its kick may have saturated (a^2 r^2 >= 2^60, or the slow chain).
__device__ __forceinline__ void pair_kicks2_sig1_ext(const PairC& pc, float cs, const float* fa, const float* fb, bool va, bool vb,
                                                     int32_t* ka, int32_t* kb, bool& ina, bool& inb, bool& exa, bool& exb) {
    float r2a = __fadd_rn(__fmul_rn(fa[0], fa[0]), __fmul_rn(fa[1], fa[1]));
    float r2b = __fadd_rn(__fmul_rn(fb[0], fb[0]), __fmul_rn(fb[1], fb[1]));
    r2a = __fadd_rn(r2a, __fmul_rn(fa[2], fa[2]));
    r2b = __fadd_rn(r2b, __fmul_rn(fb[2], fb[2]));
    ina = va && r2a < pc.rc2s;
    inb = vb && r2b < pc.rc2s;
    if ((ina && !(r2a >= pc.fast_lo)) || (inb && !(r2b >= pc.fast_lo))) {
        exa = exb = true;
        const float* fs[2] = {fa, fb};
        const bool ins[2] = {ina, inb};
        int32_t* ks[2] = {ka, kb};
#pragma unroll
        for (int q = 0; q < 2; q++) {
            float fr, s6, rr;
#pragma unroll
            for (int a = 0; a < 3; a++) ks[q][a] = 0;
            if (ins[q] && pair_fr<3, true>(pc, fs[q], fr, s6, rr)) {
                const float am = __fmul_rn(-fr, cs);
#pragma unroll
                for (int a = 0; a < 3; a++) ks[q][a] = rni_f32(__fmul_rn(am, fs[q][a]));
            }
        }
        return;
    }
    const f32x2 r2 = f2_pack(r2a, r2b), nr2 = f2_pack(-r2a, -r2b);
    const f32x2 y = rcp_cr2(r2, nr2);
    const f32x2 s2 = f2_mul(y, f2_pack(0x1p56f, 0x1p56f));
    const f32x2 s6 = f2_mul(f2_mul(s2, s2), s2);
    const f32x2 t = f2_mul(f2_mul(f2_pack(pc.c6, pc.c6), s6), f2_add(f2_add(s6, s6), f2_pack(-1.0f, -1.0f)));
    const f32x2 fr = div_cr2(t, nr2, y);
    float ama, amb;
    f2_unpack(f2_mul(fr, f2_pack(-cs, -cs)), ama, amb);
    const f32x2 am = f2_pack(ina ? ama : 0.0f, inb ? amb : 0.0f);
    float ea, eb;
    f2_unpack(f2_mul(f2_mul(am, am), r2), ea, eb);
    exa = !(ea < 0x1p60f);
    exb = !(eb < 0x1p60f);
#pragma unroll
    for (int a = 0; a < 3; a++) {
        float x, z;
        f2_unpack(f2_mul(am, f2_pack(fa[a], fb[a])), x, z);
        ka[a] = rni_f32(x);
        kb[a] = rni_f32(z);
    }
}

// The walk of one block's particles over their half lists. SMEM: the j-ends' kicks go to the
// shared-memory window slots (negated sums: the pair's own kick, plus one where the conversion
// saturated, -mirror(k) = k + 1 there); otherwise (some window did not fit) to `acc` directly,
// mirrored. Warps take the row's particles 32 at a time from a shared counter, so a warp whose
// particles have short lists takes more of them.
template <bool SIG1, bool SMEM>
__device__ __forceinline__ void half_walk(const Params& P, const uint4* __restrict__ qpos, const uint32_t* __restrict__ nbr,
                                          const uint32_t* __restrict__ nbr_count, int32_t* __restrict__ acc, int32_t* sacc,
                                          const uint2* win, uint32_t r0, uint32_t cnt0, uint32_t so0, uint32_t* next) {
    const float cs = P.kick_cs[0];
    const PairC pc0 = P.pc[0];
    const uint32_t cap4 = (P.cap + 3u) & ~3u, last_slot = P.win_cap - 1u, last_i = P.n - 1u, lane = threadIdx.x & 31u;
    for (;;) {
        uint32_t a0 = 0;
        if (lane == 0) a0 = atomicAdd(next, 32u);
        a0 = __shfl_sync(0xffffffffu, a0, 0);
        if (a0 >= cnt0) break; // (the same for the whole warp)
        const uint32_t a = a0 + lane;
        if (a >= cnt0) continue; // (the next chunk starts past the end: the warp leaves together)
        const uint32_t i = r0 + a;
        const uint4 qi = __ldg(qpos + i);
        const uint32_t Xi[3] = {qi.x, qi.y, qi.z};
        int32_t k[3] = {0, 0, 0};
        const uint32_t m = __ldg(nbr_count + i);
        const uint4* groups = reinterpret_cast<const uint4*>(nbr + list_slot(i, 0, cap4));
        const uint32_t ngroups = (m + 3u) >> 2;
        for (uint32_t g = 0; g < ngroups; g++) {
            asm volatile("prefetch.global.L2 [%0];" ::"l"(groups + 32 * min(g + 2, ngroups - 1u)));
            const uint4 jv = __ldg(groups + 32 * g);
            const uint32_t jj[4] = {jv.x, jv.y, jv.z, jv.w};
            const uint32_t left = m - 4 * g;
            uint32_t jx[4], sl[4];
            uint4 r[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                // (a slot past the list's end holds a stale word: its pair is not used; indices are
                // clamped into their arrays whatever the word holds)
                const uint2 wi = win[(jj[u] >> HALF_WIN_SHIFT) & 7u];
                const uint32_t off = jj[u] & HALF_OFF_MASK;
                jx[u] = (uint32_t)u < left ? min(wi.x + off, last_i) : i;
                sl[u] = min(wi.y + off, last_slot);
                r[u] = __ldg(qpos + jx[u]);
            }
            float f[4][3];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                uint32_t Xj[3] = {r[u].x, r[u].y, r[u].z};
                uint32_t Rj[3] = {__byte_perm(r[u].w, 0u, 0x4440u), __byte_perm(r[u].w, 0u, 0x4441u), __byte_perm(r[u].w, 0u, 0x4442u)};
                const uint32_t code = jj[u] >> LIST_BITS;
                if (code && (uint32_t)u < left) {
#pragma unroll
                    for (int b = 0; b < 3; b++) quot_shift((code >> (2 * b)) & 3u, P.box[b], Xj[b], Rj[b]);
                }
#pragma unroll
                for (int b = 0; b < 3; b++) f[u][b] = quot_sep_mad(Xj[b], Rj[b], 0u - Xi[b], (qi.w >> (8 * b)) & 15u, P.one);
            }
            int32_t kk[4][3];
            bool in[4], ext[4];
            if constexpr (SIG1) {
#pragma unroll
                for (int h = 0; h < 2; h++)
                    pair_kicks2_sig1_ext(pc0, cs, f[2 * h], f[2 * h + 1], (uint32_t)(2 * h) < left, (uint32_t)(2 * h + 1) < left,
                                         kk[2 * h], kk[2 * h + 1], in[2 * h], in[2 * h + 1], ext[2 * h], ext[2 * h + 1]);
            } else {
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    float fr, s6, r2 = 0.0f;
                    in[u] = (uint32_t)u < left && pair_fr<3, false>(pc0, f[u], fr, s6, r2);
                    const float am = in[u] ? __fmul_rn(-fr, cs) : 0.0f;
                    ext[u] = in[u] && !(__fmul_rn(__fmul_rn(am, am), r2) < 0x1p60f);
#pragma unroll
                    for (int b = 0; b < 3; b++) kk[u][b] = rni_f32(__fmul_rn(am, f[u][b]));
                }
            }
#pragma unroll
            for (int u = 0; u < 4; u++) {
#pragma unroll
                for (int b = 0; b < 3; b++) k[b] = wadd(k[b], kk[u][b]);
                if constexpr (SMEM) {
                    if (in[u]) {
                        int32_t* sp = sacc + 3u * sl[u];
#pragma unroll
                        for (int b = 0; b < 3; b++) atomicAdd(sp + b, kk[u][b]);
                    }
                } else {
                    if (in[u]) {
                        int32_t* gp = acc + 4u * (size_t)jx[u];
#pragma unroll
                        for (int b = 0; b < 3; b++) atomicAdd(gp + b, kick_mirror(kk[u][b]));
                    }
                }
            }
            if constexpr (SMEM) {
                // (rare: a kick that may have saturated, whose mirror is not its negation)
                if (ext[0] || ext[1] || ext[2] || ext[3]) {
#pragma unroll
                    for (int u = 0; u < 4; u++)
                        if (in[u] && ext[u]) {
#pragma unroll
                            for (int b = 0; b < 3; b++)
                                if ((uint32_t)kk[u][b] + 0x80000001u < 2u) atomicAdd(sacc + 3u * sl[u] + b, 1);
                        }
                }
            }
        }
        // this particle's own sum: slot a of its own row's window (negated, as the slots are)
        if constexpr (SMEM) {
#pragma unroll
            for (int b = 0; b < 3; b++) atomicAdd(sacc + 3u * (so0 + a) + b, (int32_t)(0u - (uint32_t)k[b]));
        } else {
#pragma unroll
            for (int b = 0; b < 3; b++) atomicAdd(acc + 4u * (size_t)i + b, k[b]);
        }
    }
}

// One block per row (blockIdx.x = z ny + y): the row's particles walk their half lists. Each pair's
// kick is added to the particle's own sum in registers and, mirrored, to the neighbour's slot in
// the block's shared-memory windows; the windows are then added into the global accumulators
// `acc` (4 x int32 per particle, the fourth unused; zero before the step). The shared slots hold
// the negated sums: a mirrored kick is then the pair's own kick, except where the conversion
// saturated. A pair may saturate only if |a f| reaches 2^31 on some axis, so only if a^2 r^2 >=
// 2^62; pairs with a^2 r^2 >= 2^60 in f32 (a factor of four for the roundings; inf and NaN
// included) are checked for it. When the six windows do not fit in the shared memory given
// (win_cap slots) the block accumulates in global memory directly. SIG1: sigma = 1 compiled in
// (the packed chain).
template <bool SIG1>
__global__ void __launch_bounds__(HALF_THREADS, 4) k_force_half(Params P, const uint4* __restrict__ qpos, const uint32_t* __restrict__ nbr,
                                                                const uint32_t* __restrict__ nbr_count, const uint32_t* __restrict__ start,
                                                                int32_t* __restrict__ acc) {
    extern __shared__ int32_t sacc[];
    __shared__ uint2 win[8]; // per window: first storage index of its row, first slot
    __shared__ uint32_t wcnt[8], s_total, s_next;
    const uint32_t nx = P.nc[0], ny = P.nc[1], nz = P.nc[2];
    if (threadIdx.x < 8) {
        const uint32_t w = threadIdx.x;
        uint32_t rs = 0, cnt = 0;
        if (w < HALF_WINDOWS) {
            const uint32_t row = half_window_row(ny, nz, blockIdx.x % ny, blockIdx.x / ny, w);
            rs = __ldg(start + (size_t)row * nx);
            cnt = __ldg(start + (size_t)row * nx + nx) - rs;
        }
        uint32_t before = cnt;
#pragma unroll
        for (int o = 1; o < 8; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffu, before, o, 8);
            if ((int)w >= o) before += t;
        }
        if (w == 7) s_total = before; // all six windows' slots
        before -= cnt;
        win[w] = make_uint2(rs, before);
        wcnt[w] = cnt;
        if (w == 0) s_next = 0;
    }
    __syncthreads();
    const uint32_t total = s_total;
    const bool fits = total <= P.win_cap;
    if (fits)
        for (uint32_t q = threadIdx.x; q < 3u * total; q += blockDim.x) sacc[q] = 0;
    __syncthreads();
    const uint32_t r0 = win[HALF_OWN_WINDOW].x, cnt0 = wcnt[HALF_OWN_WINDOW], so0 = win[HALF_OWN_WINDOW].y;
    if (fits) half_walk<SIG1, true>(P, qpos, nbr, nbr_count, acc, sacc, win, r0, cnt0, so0, &s_next);
    else half_walk<SIG1, false>(P, qpos, nbr, nbr_count, acc, sacc, win, r0, cnt0, so0, &s_next);
    if (!fits) return;
    __syncthreads();
    // the windows into the global accumulators (negating the slots back)
#pragma unroll 1
    for (uint32_t w = 0; w < HALF_WINDOWS; w++) {
        const uint2 wi = win[w];
        const uint32_t words = 3u * wcnt[w];
        int32_t* g = acc + 4u * (size_t)wi.x;
        const int32_t* sp = sacc + 3u * wi.y;
        for (uint32_t q = threadIdx.x; q < words; q += blockDim.x) {
            const int32_t v = sp[q];
            const uint32_t s3 = q / 3u;
            if (v) atomicAdd(g + 4u * s3 + (q - 3u * s3), (int32_t)(0u - (uint32_t)v));
        }
    }
}

// The step after the half-shell forces: v += kick + g (wrapping), x += v (left unwrapped, as the
// full-list step does), the quotient record rewritten, the displacement trigger tested; the
// accumulator cleared for the next step.
__global__ void __launch_bounds__(256) k_leap_half(Params P, const PosRec<3>* __restrict__ pos_in, PosRec<3>* __restrict__ pos_out,
                                                   uint4* __restrict__ qpos_out, int32_t* __restrict__ vel, int4* __restrict__ acc,
                                                   const PosRec<3>* __restrict__ ref_pos, uint32_t* __restrict__ ctl) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    int64_t x[3];
    load_particle<3, false>(pos_in, nullptr, i, x);
    const int4 kv = acc[i];
    acc[i] = make_int4(0, 0, 0, 0);
    const int32_t k[3] = {kv.x, kv.y, kv.z};
    int32_t v[3];
#pragma unroll
    for (int a = 0; a < 3; a++) v[a] = vel[3 * (size_t)i + a];
    leapfrog<3, Params, false>(P, 0u, k, v, x);
#pragma unroll
    for (int a = 0; a < 3; a++) vel[3 * (size_t)i + a] = v[a];
    store_pos<3>(pos_out, i, x, 0u);
    qpos_out[i] = quot_record<3>(x, 0u);
    int64_t xr[3];
    load_particle<3, false>(ref_pos, nullptr, i, xr);
    if (moved_half_skin<3>(P, xr, x)) ctl[0] = 1;
}

} // namespace gbmd
