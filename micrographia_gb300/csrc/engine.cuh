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

// Validate a system for this engine (periodic LJ subset); GBMD_OK or an error (message set).
int validate_system(const gbmd_system& sys, uint32_t n);

} // namespace gbmd
