// Scan, stable radix sort and cell starts (see sort.cuh).
#include <algorithm>
#include <utility>

#include "common.cuh"
#include "sort.cuh"

namespace gbmd {

namespace {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_PER_THREAD = SCAN_ITEMS / SCAN_THREADS; // 8
constexpr int RADIX_THREADS = 256;
constexpr int RADIX_WARPS = RADIX_THREADS / 32;
constexpr int RADIX_ROUNDS = RADIX_TILE / RADIX_THREADS; // 8

// Block-wide exclusive scan of one value per thread; returns the block total in *total.
__device__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total) {
    __shared__ uint32_t warp_sums[SCAN_THREADS / 32];
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < SCAN_THREADS / 32 ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < SCAN_THREADS / 32) warp_sums[lane] = w;
    }
    __syncthreads();
    uint32_t before = warp > 0 ? warp_sums[warp - 1] : 0;
    *total = warp_sums[SCAN_THREADS / 32 - 1];
    __syncthreads();
    return before + x - v;
}

// Each block scans SCAN_ITEMS consecutive elements (blocked: thread t owns [8t, 8t + 8)) and
// writes its total to sums[block].
__global__ void k_scan_blocks(const uint32_t* in, uint32_t* out, size_t n, uint32_t* sums) {
    size_t base = (size_t)blockIdx.x * SCAN_ITEMS + (size_t)threadIdx.x * SCAN_PER_THREAD;
    uint32_t v[SCAN_PER_THREAD];
    uint32_t local = 0;
#pragma unroll
    for (int k = 0; k < SCAN_PER_THREAD; k++) {
        v[k] = base + k < n ? in[base + k] : 0;
        local += v[k];
    }
    uint32_t total;
    uint32_t off = block_exclusive_scan(local, &total);
#pragma unroll
    for (int k = 0; k < SCAN_PER_THREAD; k++) {
        if (base + k < n) out[base + k] = off;
        off += v[k];
    }
    if (threadIdx.x == 0 && sums) sums[blockIdx.x] = total;
}

__global__ void k_scan_add(uint32_t* out, size_t n, const uint32_t* offs) {
    size_t base = (size_t)blockIdx.x * SCAN_ITEMS;
    uint32_t add = offs[blockIdx.x];
    for (int k = threadIdx.x; k < (int)SCAN_ITEMS; k += SCAN_THREADS)
        if (base + k < n) out[base + k] += add;
}

// Per-tile histogram of one 8-bit digit: hist[d * tiles + tile].
__global__ void k_radix_hist(const uint32_t* keys, uint32_t n, int shift, uint32_t* hist, uint32_t tiles) {
    __shared__ uint32_t cnt[256];
    cnt[threadIdx.x] = 0;
    __syncthreads();
    size_t base = (size_t)blockIdx.x * RADIX_TILE;
    for (int r = 0; r < RADIX_ROUNDS; r++) {
        size_t i = base + (size_t)r * RADIX_THREADS + threadIdx.x;
        if (i < n) atomicAdd(&cnt[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[(size_t)threadIdx.x * tiles + blockIdx.x] = cnt[threadIdx.x];
}

// Stable scatter of one tile: items are ranked in index order, warp by warp within a round of
// 256, round by round; offs[d * tiles + tile] is the tile's first slot for digit d. LOCAL: offs
// is the histogram itself (few tiles), and each block forms its own offsets from it (the digits
// before d over all tiles, plus digit d over the tiles before this one), with no scan launches.
template <bool LOCAL>
__global__ void k_radix_scatter(const uint32_t* kin, const uint32_t* vin, uint32_t* kout, uint32_t* vout, uint32_t n, int shift,
                                const uint32_t* offs, uint32_t tiles) {
    __shared__ uint32_t base[256];
    __shared__ uint32_t wcnt[RADIX_WARPS][257];
    int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    if constexpr (LOCAL) {
        uint32_t own = 0, tot = 0;
        for (uint32_t j = 0; j < tiles; j++) {
            const uint32_t c = offs[(size_t)t * tiles + j];
            tot += c;
            own += j < blockIdx.x ? c : 0u;
        }
        uint32_t all;
        base[t] = block_exclusive_scan(tot, &all) + own;
    } else {
        base[t] = offs[(size_t)t * tiles + blockIdx.x];
    }
#pragma unroll
    for (int w = 0; w < RADIX_WARPS; w++) wcnt[w][t] = 0;
    __syncthreads();
    const uint32_t lt = (1u << lane) - 1u;
    size_t tile0 = (size_t)blockIdx.x * RADIX_TILE;
    for (int r = 0; r < RADIX_ROUNDS; r++) {
        size_t i = tile0 + (size_t)r * RADIX_THREADS + t;
        bool valid = i < n;
        uint32_t key = valid ? kin[i] : 0u, val = valid ? vin[i] : 0u;
        uint32_t d = valid ? (key >> shift) & 255u : 256u;
        uint32_t peers = __match_any_sync(0xffffffffu, d);
        uint32_t below = peers & lt;
        if (below == 0) wcnt[warp][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            uint32_t p = base[d] + __popc(below);
            for (int w = 0; w < warp; w++) p += wcnt[w][d];
            kout[p] = key;
            vout[p] = val;
        }
        __syncthreads();
        uint32_t s = 0;
#pragma unroll
        for (int w = 0; w < RADIX_WARPS; w++) {
            s += wcnt[w][t];
            wcnt[w][t] = 0;
        }
        base[t] += s;
        __syncthreads();
    }
}

__global__ void k_cell_starts(const uint32_t* keys, uint32_t n, uint32_t ncell, uint32_t* start) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i > n) return;
    int64_t prev = i == 0 ? -1 : (int64_t)keys[i - 1];
    int64_t cur = i == n ? (int64_t)ncell : (int64_t)keys[i];
    for (int64_t c = prev + 1; c <= cur; c++) start[c] = (uint32_t)i;
}

__global__ void k_iota(uint32_t* v, uint32_t n) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = (uint32_t)i;
}

size_t blocks_of(size_t n, size_t per) { return (n + per - 1) / per; }

} // namespace

size_t scan_tmp_elems(size_t n) {
    size_t total = 0;
    size_t m = blocks_of(n, SCAN_ITEMS);
    while (m > 1) {
        total += m;
        m = blocks_of(m, SCAN_ITEMS);
    }
    return total + 1;
}

size_t radix_hist_elems(size_t n) { return 256 * std::max<size_t>(blocks_of(n, RADIX_TILE), 1); }

void scan_exclusive(const uint32_t* in, uint32_t* out, size_t n, uint32_t* tmp, cudaStream_t s) {
    if (n == 0) return;
    size_t nb = blocks_of(n, SCAN_ITEMS);
    if (nb == 1) {
        k_scan_blocks<<<1, SCAN_THREADS, 0, s>>>(in, out, n, nullptr);
        return;
    }
    uint32_t* sums = tmp;
    k_scan_blocks<<<(unsigned)nb, SCAN_THREADS, 0, s>>>(in, out, n, sums);
    scan_exclusive(sums, sums, nb, tmp + nb, s);
    k_scan_add<<<(unsigned)nb, SCAN_THREADS, 0, s>>>(out, n, sums);
}

int radix_passes(int bits) { return bits <= 0 ? 1 : (bits + 7) / 8; }

// Kernels scan_exclusive launches for n elements.
static uint32_t scan_launches(size_t n) {
    if (n == 0) return 0;
    size_t nb = blocks_of(n, SCAN_ITEMS);
    return nb == 1 ? 1u : 2u + scan_launches(nb);
}

int radix_sort_pairs(uint32_t* k0, uint32_t* v0, uint32_t* k1, uint32_t* v1, uint32_t n, int bits, uint32_t* hist, uint32_t* tmp,
                     cudaStream_t s, bool first_hist_done, uint32_t* launches) {
    if (n == 0) return 0;
    uint32_t tiles = (uint32_t)blocks_of(n, RADIX_TILE);
    int passes = radix_passes(bits);
    const bool local = tiles <= RADIX_LOCAL_TILES;
    uint32_t *ki = k0, *vi = v0, *ko = k1, *vo = v1;
    uint32_t count = 0;
    for (int p = 0; p < passes; p++) {
        int shift = 8 * p;
        if (p > 0 || !first_hist_done) {
            k_radix_hist<<<tiles, RADIX_THREADS, 0, s>>>(ki, n, shift, hist, tiles);
            count++;
        }
        if (local) {
            k_radix_scatter<true><<<tiles, RADIX_THREADS, 0, s>>>(ki, vi, ko, vo, n, shift, hist, tiles);
        } else {
            count += scan_launches((size_t)256 * tiles);
            scan_exclusive(hist, hist, (size_t)256 * tiles, tmp, s);
            k_radix_scatter<false><<<tiles, RADIX_THREADS, 0, s>>>(ki, vi, ko, vo, n, shift, hist, tiles);
        }
        count++;
        std::swap(ki, ko);
        std::swap(vi, vo);
    }
    if (launches) *launches = count;
    return passes & 1;
}

void cell_starts(const uint32_t* keys, uint32_t n, uint32_t ncell, uint32_t* start, cudaStream_t s) {
    k_cell_starts<<<(unsigned)blocks_of((size_t)n + 1, 256), 256, 0, s>>>(keys, n, ncell, start);
}

void iota(uint32_t* vals, uint32_t n, cudaStream_t s) {
    if (n) k_iota<<<(unsigned)blocks_of(n, 256), 256, 0, s>>>(vals, n);
}

} // namespace gbmd
