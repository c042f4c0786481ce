// cp_kernels.h -- launch entry points of the step kernels (cp_step.cu),
// called by the host runtime (cp_host.cpp).
#pragma once
#include <cuda_runtime.h>

#include "cp_types.h"

// kernel variants (threads per block, min blocks per SM) the autotuner picks from
int cpk_num_variants();
int cpk_variant_threads(int variant);
int cpk_max_resident_blocks(int variant);
// One World.step for each of the n worlds ids[0..n) of the world table, by a
// persistent grid of `grid` blocks pulling worlds from *d_queue.
cudaError_t cpk_launch_step(const DWorld* d_worlds, const int* d_ids, int n, double dt, int* d_queue, int grid,
                            cudaStream_t stream, int variant);
// status, stepnumber and counts of the listed worlds, gathered into out[4*i..]
cudaError_t cpk_gather_status(const DWorld* d_worlds, const int* d_ids, int n, long long* d_out, cudaStream_t stream);
// clear the status of the listed worlds
cudaError_t cpk_clear_status(const DWorld* d_worlds, const int* d_ids, int n, cudaStream_t stream);
// scatter 6 floats per body into Body.force/torque, gather 13 pose floats per body;
// d_first[i] = index of world ids[i]'s first body in the packed buffer
cudaError_t cpk_scatter_forces(const DWorld* d_worlds, const int* d_ids, const long long* d_first, int n, const float* d_in,
                               cudaStream_t stream);
cudaError_t cpk_gather_poses(const DWorld* d_worlds, const int* d_ids, const long long* d_first, int n, float* d_out,
                             cudaStream_t stream);
// per-phase cycles summed over blocks: prepare, broadphase, narrowphase,
// rows+wake+solve prep, row assembly, levels, GS sweeps, apply+integrate
cudaError_t cpk_phase_cycles(unsigned long long* out, bool reset);
