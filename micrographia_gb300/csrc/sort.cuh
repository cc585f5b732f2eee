// Device primitives of the cell binning: exclusive scan, stable LSD radix sort of (key, value)
// pairs, and cell starts from sorted keys. They replace gpu-prims' reduce-then-scan
// (crates/gpu-prims/src/prims.rs:157-196, shaders/scan.wgsl) and its unstable counting sort
// (prims.rs:198-248, bin_count.wgsl, bin_scatter.wgsl): the sort here is stable, so the
// permutation is exactly md_ref::CellList::build's (crates/md-ref/src/cells.rs:10-32).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace gbmd {

constexpr uint32_t SCAN_ITEMS = 2048;  // elements per block of the scan (256 threads x 8)
constexpr uint32_t RADIX_TILE = 2048;  // keys per block of a radix pass (8 rounds of 256)
constexpr uint32_t RADIX_THREADS_PER_TILE = 256;
constexpr uint32_t RADIX_LOCAL_TILES = 64; // up to this many tiles, scatter blocks form their own offsets

// Scratch sizes (in uint32 elements).
size_t scan_tmp_elems(size_t n);
size_t radix_hist_elems(size_t n);

// out[i] = sum of in[0..i) (in may equal out). `tmp` holds scan_tmp_elems(n) elements.
void scan_exclusive(const uint32_t* in, uint32_t* out, size_t n, uint32_t* tmp, cudaStream_t s);

// Stable sort of n (key, value) pairs by the low `bits` bits of the key, 8 bits per pass,
// ping-ponging between (k0, v0) and (k1, v1). Returns 0 if the result is in (k0, v0), 1 if in
// (k1, v1). `hist` holds radix_hist_elems(n) elements, `tmp` scan_tmp_elems(radix_hist_elems(n)).
// With few tiles (RADIX_LOCAL_TILES or fewer) each scatter block forms its offsets from the
// histogram itself: two launches per pass. `first_hist_done`: the caller's key kernel has already
// written the first pass's histogram (k_keys_hist). `launches`, if given, receives the count of
// kernels launched.
int radix_sort_pairs(uint32_t* k0, uint32_t* v0, uint32_t* k1, uint32_t* v1, uint32_t n, int bits, uint32_t* hist, uint32_t* tmp,
                     cudaStream_t s, bool first_hist_done = false, uint32_t* launches = nullptr);
int radix_passes(int bits);

// start[c] = first index of sorted `keys` with key >= c, for c in [0, ncell]; start[ncell] = n.
void cell_starts(const uint32_t* keys, uint32_t n, uint32_t ncell, uint32_t* start, cudaStream_t s);

// vals[i] = i.
void iota(uint32_t* vals, uint32_t n, cudaStream_t s);

} // namespace gbmd
