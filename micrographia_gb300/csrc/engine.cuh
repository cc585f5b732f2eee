// Declarations shared by the engine's translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/gbmd.h"

namespace gbmd {

// Kernel-launch accounting: every launch site adds to a process-wide counter, so an engine can
// report how many of its kernels ran (graph replays included).
void note_launch(uint64_t k = 1);
uint64_t launch_total();

// Generate the id-ordered initial state of `spec` into device buffers: positions in the
// engine's record layout (2D: int64 x, y; 3D: int64 x, y, z, species), velocities interleaved
// int32, species uint32 (all zero).
int init_state_device(const gbmd_system& sys, const gbmd_init& spec, void* pos_dev, int32_t* vel_dev, uint32_t* species_dev,
                      cudaStream_t s);

// init::maxwell (init.rs:42-57) / three::maxwell for the given device species: Maxwell draws at
// kT = t, then the exact zero velocity sum over the moving particles; with `fixed_speed`,
// init::fixed_speed's draws (init.rs:61-74, 2D) instead of Maxwell's.
int maxwell_state_device(const gbmd_system& sys, uint32_t n, double t, uint64_t seed, const uint32_t* species_dev, int32_t* vel_dev,
                         cudaStream_t s, bool fixed_speed = false);

// Validate a system for this engine (periodic LJ subset); GBMD_OK or an error (message set).
int validate_system(const gbmd_system& sys, uint32_t n);

struct Params;
// Host-side System maths shared by the engines.
double rc_max(const gbmd_system& s);
int cells_for(const gbmd_system& s, double r, uint32_t* c);                 // System::cells_for
void fill_params(Params& P, const gbmd_system& s, uint32_t n, double skin, uint32_t cap, const uint32_t* nc);
int key_bits(uint32_t ncell);
// Pinned host memory from a process-wide pool that is never freed (freeing pinned memory
// synchronises the device): at least `bytes`, its block size in *cap (0 on failure).
void* pinned_alloc(size_t bytes, size_t* cap);
void pinned_release(void* p, size_t cap);
void set_cells(Params& P, const uint32_t* nc, uint32_t dim);

} // namespace gbmd
