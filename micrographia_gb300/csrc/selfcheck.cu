// Self-check of the pair chain's own correctly rounded reciprocal and division (rcp_cr, div_cr)
// against the CUDA library's __frcp_rn / __fdiv_rn: every f32 of the reciprocal's range, every
// f32 r2 of each pair type's fast range through the whole chain, and seeded random quotients.
#include <cstring>

#include "common.cuh"
#include "engine.cuh"
#include "kernels.cuh"

using namespace gbmd;

namespace {

__device__ unsigned long long g_bad;

__device__ __forceinline__ void note_bad(bool bad) {
    unsigned b = __ballot_sync(0xffffffffu, bad);
    if ((threadIdx.x & 31u) == 0 && b) atomicAdd(&g_bad, (unsigned long long)__popc(b));
}

// bits in [lo, lo + count): rcp_cr(b) == __frcp_rn(b) bit for bit
__global__ void k_check_rcp(uint32_t lo, uint32_t count) {
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k - (k & 31u) < count; k += gridDim.x * blockDim.x) {
        bool bad = false;
        if (k < count) {
            float b = __uint_as_float(lo + k);
            bad = __float_as_uint(rcp_cr(b)) != __float_as_uint(__frcp_rn(b));
        }
        note_bad(bad);
    }
}

// bits in [lo, lo + count): pair_chain == pair_fr_library (fr and s6) bit for bit
__global__ void k_check_chain(PairC p, uint32_t lo, uint32_t count) {
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k - (k & 31u) < count; k += gridDim.x * blockDim.x) {
        bool bad = false;
        if (k < count) {
            float r2 = __uint_as_float(lo + k);
            float fa, sa, fb, sb;
            pair_chain(p, r2, fa, sa);
            pair_fr_library(p, r2, fb, sb);
            bad = __float_as_uint(fa) != __float_as_uint(fb) || __float_as_uint(sa) != __float_as_uint(sb);
        }
        note_bad(bad);
    }
}

// Seeded random a in +-[2^-100, 2^100), b in [2^-30, 2^62) with a / b within [2^-120, 2^120]:
// div_cr(a, b, rcp_cr(b)) == __fdiv_rn(a, b).
__global__ void k_check_div(uint64_t count, uint32_t seed) {
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k - (k & 31u) < count; k += (uint64_t)gridDim.x * blockDim.x) {
        bool bad = false;
        if (k < count) {
            uint32_t r0, r1, r2, r3;
            threefry2x32((uint32_t)k, (uint32_t)(k >> 32), seed, 0x5eedu, r0, r1);
            threefry2x32((uint32_t)k, (uint32_t)(k >> 32), seed, 0xd1cu, r2, r3);
            float a = __uint_as_float(((27u + r2 % 200u) << 23) | (r0 & 0x7fffffu) | (r3 & 0x80000000u));
            float b = __uint_as_float(((97u + r3 % 92u) << 23) | (r1 & 0x7fffffu));
            float q = __fdiv_rn(a, b), aq = fabsf(q);
            if (aq >= 0x1p-120f && aq <= 0x1p120f) bad = __float_as_uint(div_cr(a, b, rcp_cr(b))) != __float_as_uint(q);
        }
        note_bad(bad);
    }
}

// Seeded random separations (|f| < 3 sigma per axis, in the f32 units of 2^-28 sigma): the
// packed two-pair kicks of the force kernel (pair_kicks2_sig1) equal two scalar pair kicks.
template <int D>
__global__ void k_check_kicks2(PairC p, float cs, uint64_t count, uint32_t seed) {
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k - (k & 31u) < count; k += (uint64_t)gridDim.x * blockDim.x) {
        bool bad = false;
        if (k < count) {
            float f[6];
#pragma unroll
            for (int q = 0; q < 3; q++) {
                uint32_t r0, r1;
                threefry2x32((uint32_t)k, (uint32_t)(k >> 32) * 8u + (uint32_t)q, seed, 0xf2u, r0, r1);
                f[2 * q] = (float)((int32_t)(r0 % (6u << 28)) - (int32_t)(3u << 28));
                f[2 * q + 1] = (float)((int32_t)(r1 % (6u << 28)) - (int32_t)(3u << 28));
            }
            if (D == 2) f[2] = f[5] = 0.0f;
            int32_t k1[3] = {0, 0, 0}, k2[3] = {0, 0, 0};
            pair_kicks2_sig1<D>(p, cs, f, f + 3, true, true, k1);
#pragma unroll
            for (int q = 0; q < 2; q++) {
                float fr, s6, rr;
                if (pair_fr<D, true>(p, f + 3 * q, fr, s6, rr)) {
                    const float am = __fmul_rn(-fr, cs);
#pragma unroll
                    for (int a = 0; a < D; a++) k2[a] = wadd(k2[a], rni_f32(__fmul_rn(am, f[3 * q + a])));
                }
            }
            bad = k1[0] != k2[0] || k1[1] != k2[1] || k1[2] != k2[2];
        }
        note_bad(bad);
    }
}

} // namespace

namespace {
// Seeded random (v, f): v over the whole int32 range (with 0, +-1 and the extremes), f with a
// random 53-bit significand and an exponent of 2^-40 .. 2^40, or within 2^-20 of 1 (a thermostat's
// factors), or an integer plus one half over 2^k (ties after the product): rescale_i32 equals the
// f64 path, sat_i32_f64(round(v f)), bit for bit.
__global__ void k_check_rescale(uint64_t count, uint32_t seed) {
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k - (k & 31u) < count; k += (uint64_t)gridDim.x * blockDim.x) {
        bool bad = false;
        if (k < count) {
            uint32_t r0, r1, r2, r3;
            threefry2x32((uint32_t)k, (uint32_t)(k >> 32), seed, 0x7e5c41eu, r0, r1);
            threefry2x32((uint32_t)k, (uint32_t)(k >> 32), seed, 0x5ca1eu, r2, r3);
            int32_t v = (int32_t)r0;
            const uint32_t pick = r3 & 7u;
            if (pick == 0) v = (int32_t)(r0 % 5u) - 2;                       // 0, +-1, +-2
            else if (pick == 1) v = (r0 & 1u) ? INT32_MAX : INT32_MIN;        // the extremes
            else if (pick == 2) v = (int32_t)(r0 >> (r2 % 31u)) * ((r0 & 2u) ? 1 : -1);
            uint64_t fb;
            const uint32_t kind = (r3 >> 3) % 3u;
            if (kind == 0) fb = ((uint64_t)(1023u - 40u + (r2 % 81u)) << 52) | ((((uint64_t)r1 << 32) | r2) & ((1ull << 52) - 1));
            else if (kind == 1) fb = ((uint64_t)(1022u + (r2 & 1u)) << 52) | (((uint64_t)r1 << 32 | r2) & ((1ull << 52) - 1) & (r2 & 1u ? 0xfffffull : ~0ull));
            else fb = (uint64_t)__double_as_longlong(__dmul_rn((double)((r1 & 0xfffffu) * 2u + 1u), ldexp(1.0, -(int)(1u + r2 % 40u))));
            const double f = __longlong_as_double((long long)fb);
            const uint32_t fe = (uint32_t)(fb >> 52) & 0x7ffu;
            if (fe != 0u && fe != 0x7ffu && !(fb >> 63)) {
                const int32_t want = sat_i32_f64(round(__dmul_rn((double)v, f)));
                const int32_t got = rescale_i32(v, (fb & ((1ull << 52) - 1)) | (1ull << 52), (int)fe - 1075);
                bad = got != want;
            }
        }
        note_bad(bad);
    }
}
} // namespace

// The velocity rescale's integer arithmetic (rescale_i32) against the f64 product and rounding
// it replaces, on `count` seeded random cases.
extern "C" int gbmd_check_rescale(uint64_t count, int32_t device, uint64_t* checked, uint64_t* mismatched) {
    if (!checked || !mismatched) return fail(GBMD_E_INVALID, "null argument");
    GBMD_CUDA_TRY(cudaSetDevice(device));
    cudaStream_t s;
    GBMD_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    unsigned long long zero = 0, bad = 0;
    int rc = GBMD_OK;
    if (cudaMemcpyToSymbolAsync(g_bad, &zero, 8, 0, cudaMemcpyHostToDevice, s) != cudaSuccess) rc = fail(GBMD_E_CUDA, "self-check counter");
    if (rc == GBMD_OK && count) {
        k_check_rescale<<<152 * 8, 256, 0, s>>>(count, 0x2e5ca1eu);
        note_launch();
    }
    if (rc == GBMD_OK && cudaMemcpyFromSymbolAsync(&bad, g_bad, 8, 0, cudaMemcpyDeviceToHost, s) != cudaSuccess) rc = fail(GBMD_E_CUDA, "self-check counter");
    if (rc == GBMD_OK) {
        const cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) rc = fail(GBMD_E_CUDA, cudaGetErrorString(e));
    }
    cudaStreamDestroy(s);
    *checked = count;
    *mismatched = bad;
    return rc;
}

extern "C" int gbmd_check_pair_math(const gbmd_system* sys, uint64_t random_quotients, int32_t device, uint64_t* checked,
                                    uint64_t* mismatched) {
    if (!sys || !checked || !mismatched) return fail(GBMD_E_INVALID, "null argument");
    GBMD_TRY(validate_system(*sys, 1));
    GBMD_CUDA_TRY(cudaSetDevice(device));
    Params P;
    std::memset(&P, 0, sizeof(P));
    uint32_t nc[3] = {3, 3, 3};
    fill_params(P, *sys, 1, 0.3, 1, nc);
    cudaStream_t s;
    GBMD_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    unsigned long long zero = 0;
    int rc = GBMD_OK;
    uint64_t total = 0;
    if (cudaMemcpyToSymbolAsync(g_bad, &zero, 8, 0, cudaMemcpyHostToDevice, s) != cudaSuccess) rc = fail(GBMD_E_CUDA, "self-check counter");
    const int grid = 152 * 8, block = 256;
    // the reciprocal over [2^50, 2^63)
    if (rc == GBMD_OK) {
        uint32_t lo = (127u + 50u) << 23, hi = (127u + 63u) << 23;
        k_check_rcp<<<grid, block, 0, s>>>(lo, hi - lo);
        note_launch();
        total += hi - lo;
    }
    // the whole chain over [fast_lo, rc2s) of each pair type that uses the fast path
    for (uint32_t k = 0; rc == GBMD_OK && k < sys->nspecies * sys->nspecies; k++) {
        const PairC& c = P.pc[k];
        if (!(c.fast_lo < c.rc2s)) continue;
        uint32_t lo, hi;
        std::memcpy(&lo, &c.fast_lo, 4);
        std::memcpy(&hi, &c.rc2s, 4);
        k_check_chain<<<grid, block, 0, s>>>(c, lo, hi - lo);
        note_launch();
        total += hi - lo;
    }
    if (rc == GBMD_OK && random_quotients) {
        k_check_div<<<grid, block, 0, s>>>(random_quotients, 20260u);
        note_launch();
        total += random_quotients;
    }
    // the packed two-pair kicks, for a single species with sigma = 1 (where the force kernel uses them)
    if (rc == GBMD_OK && random_quotients && sys->nspecies == 1 && P.pc[0].sigma2s == 0x1p56f) {
        k_check_kicks2<3><<<grid, block, 0, s>>>(P.pc[0], P.kick_cs[0], random_quotients, 7u);
        k_check_kicks2<2><<<grid, block, 0, s>>>(P.pc[0], P.kick_cs[0], random_quotients, 8u);
        note_launch(2);
        total += 2 * random_quotients;
    }
    unsigned long long bad = 0;
    if (rc == GBMD_OK && cudaMemcpyFromSymbolAsync(&bad, g_bad, 8, 0, cudaMemcpyDeviceToHost, s) != cudaSuccess)
        rc = fail(GBMD_E_CUDA, "self-check counter");
    cudaError_t err = cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    if (rc != GBMD_OK) return rc;
    if (err != cudaSuccess) return fail(GBMD_E_CUDA, cudaGetErrorString(err));
    *checked = total;
    *mismatched = bad;
    return GBMD_OK;
}
