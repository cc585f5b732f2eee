// Cell binning that allocates no device memory.
//
// The engine's binning (keys -> stable radix sort -> cell starts) needs scratch buffers: a second
// key/value pair of arrays to ping-pong between, the per-tile digit histograms and the scan's
// block sums. The engine allocates them with cudaMalloc when it is created. Some callers of this
// library cannot do that: a host that hands the library a fixed device-memory arena at start-up
// and forbids any later allocation (an embedding runtime such as a Rust host that owns every
// device buffer of its `State`), and callers on a stream-ordered hot path, where cudaMalloc and
// cudaFree would synchronise the device and stall the stream. This entry point serves them: the
// caller passes device pointers for the input positions and the three outputs, and all scratch
// lives in one file-scope __device__ array of fixed size, set aside once per device when the
// library is loaded and held until the process exits.
#include <mutex>

#include "common.cuh"
#include "engine.cuh"
#include "sort.cuh"

namespace gbmd {
namespace {

// Largest n the static scratch holds, and its layout in 32-bit words: keys A, values A, keys B,
// values B (n each), the radix histograms (256 per tile of RADIX_TILE keys) and the scan's block
// sums (well under 64 words for these sizes).
constexpr uint32_t MAX_N = GBMD_BIN_STATIC_MAX_N;
constexpr size_t HIST_WORDS = 256 * ((MAX_N + RADIX_TILE - 1) / RADIX_TILE);
constexpr size_t TMP_WORDS = 64;
constexpr size_t SCRATCH_WORDS = 4 * (size_t)MAX_N + HIST_WORDS + TMP_WORDS;

__device__ __align__(256) uint32_t g_bin_scratch[SCRATCH_WORDS];

// Device address of g_bin_scratch per device ordinal, looked up once per device. (A
// cudaDeviceReset of that device in this process would leave the cached address stale: callers
// that reset a device do not use this entry point afterwards.)
constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
uint32_t* g_addr[MAX_DEVICES] = {};

int scratch_address(uint32_t** out) {
    int dev = 0;
    GBMD_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= MAX_DEVICES) return fail(GBMD_E_INVALID, "device ordinal out of range for the static scratch table");
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_bin_scratch);
        if (e != cudaSuccess) return fail(GBMD_E_CUDA, std::string("cudaGetSymbolAddress(g_bin_scratch): ") + cudaGetErrorString(e));
        g_addr[dev] = (uint32_t*)p;
    }
    *out = g_addr[dev];
    return GBMD_OK;
}

struct BinP {
    uint32_t n, dim, nc[3];
    double box_f[3];
};

// Row-major cell key of each particle from id-ordered interleaved int64 positions (the same
// f64 cell_of as the engine, md-ref cells.rs:53-55); values are the particle indices.
__global__ void k_keys_interleaved(BinP B, const int64_t* pos, uint32_t* keys_out, uint32_t* keys, uint32_t* vals) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B.n) return;
    uint32_t c[3] = {0, 0, 0};
    for (uint32_t a = 0; a < B.dim; a++) c[a] = cell_of(pos[(size_t)B.dim * i + a], B.box_f[a], B.nc[a]);
    uint32_t k = B.dim == 2 ? c[1] * B.nc[0] + c[0] : (c[2] * B.nc[1] + c[1]) * B.nc[0] + c[0];
    keys_out[i] = k;
    keys[i] = k;
    vals[i] = i;
}

} // namespace
} // namespace gbmd

using namespace gbmd;

extern "C" int gbmd_bin_cells_static(const gbmd_system* sys, const int64_t* pos, uint32_t n, const uint32_t* cells, uint32_t* keys,
                                     uint32_t* start, uint32_t* items, void* stream) {
    if (!sys || !cells || (n && (!pos || !keys || !items)) || !start) return fail(GBMD_E_INVALID, "null argument");
    if (sys->dim != 2 && sys->dim != 3) return fail(GBMD_E_INVALID, "dim must be 2 or 3");
    if (n > MAX_N)
        return fail(GBMD_E_INVALID, "gbmd_bin_cells_static holds at most GBMD_BIN_STATIC_MAX_N (262144) particles; use an engine for more");
    uint64_t ncell = 1;
    BinP B{};
    B.n = n;
    B.dim = sys->dim;
    for (uint32_t a = 0; a < 3; a++) {
        B.nc[a] = a < sys->dim ? cells[a] : 1;
        if (B.nc[a] == 0) return fail(GBMD_E_INVALID, "cells must be positive");
        if (a < sys->dim && sys->box_len[a] <= 0) return fail(GBMD_E_INVALID, "box lengths must be positive");
        // (checked after every factor, so that the product cannot wrap past the bound)
        ncell *= B.nc[a];
        if (ncell >= UINT32_MAX) return fail(GBMD_E_INVALID, "too many cells");
        B.box_f[a] = a < sys->dim ? (double)sys->box_len[a] * (1.0 / 4294967296.0) : 1.0;
    }
    uint32_t* scratch = nullptr;
    GBMD_TRY(scratch_address(&scratch));
    cudaStream_t s = (cudaStream_t)stream;
    uint32_t *ka = scratch, *va = scratch + MAX_N, *kb = scratch + 2 * (size_t)MAX_N, *vb = scratch + 3 * (size_t)MAX_N;
    uint32_t* hist = scratch + 4 * (size_t)MAX_N;
    uint32_t* tmp = hist + HIST_WORDS;
    if (n) {
        k_keys_interleaved<<<(n + 255) / 256, 256, 0, s>>>(B, pos, keys, ka, va);
        int bits = 1;
        while (bits < 32 && ((uint32_t)(ncell - 1) >> bits)) bits++;
        int res = radix_sort_pairs(ka, va, kb, vb, n, bits, hist, tmp, s);
        cell_starts(res ? kb : ka, n, (uint32_t)ncell, start, s);
        GBMD_CUDA_TRY(cudaMemcpyAsync(items, res ? vb : va, (size_t)n * 4, cudaMemcpyDeviceToDevice, s));
    } else {
        GBMD_CUDA_TRY(cudaMemsetAsync(start, 0, (size_t)(ncell + 1) * 4, s));
    }
    GBMD_CUDA_TRY(cudaGetLastError());
    return GBMD_OK;
}
