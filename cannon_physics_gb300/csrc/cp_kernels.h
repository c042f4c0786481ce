// cp_kernels.h -- launch entry points of the step kernels (cp_step.cu),
// called by the host runtime (cp_host.cpp).
#pragma once
#include <cuda_runtime.h>

#include "cp_types.h"

#define CP_GROUP_MAX_WORLDS 8
// kernel variants (threads per block, min blocks per SM) the autotuner picks from
// (pre-solve kernel, solve kernel) variant pairs, numbered 0 .. cpk_num_variants()-1
int cpk_num_variants();
int cpk_num_pre_variants();
int cpk_num_solve_variants();
int cpk_variant_threads(int variant);
// threads per block of the solve kernel of a variant
int cpk_solve_threads(int variant);
// bodies per world group of a variant's solve kernel for the configured group size
int cpk_solve_group_limit(int variant, int group_bodies);
void cpk_max_resident_blocks(int variant, int* pre, int* solve);
// One World.step for the n worlds ids[0..n): the pre-solve kernel (one world
// per block, grid_pre persistent blocks) then the solve kernel (groups of
// worlds ids[gstart[g] .. gstart[g+1]), grid_solve persistent blocks); two
// queue counters at d_queue.
// max_nb: the most bodies of any world in the launch (sizes the pre kernel's
// shared level table)
cudaError_t cpk_launch_step(const DWorld* d_worlds, const int* d_ids, const int* d_gstart, int ngroups, double dt, int* d_queue,
                            int grid_pre, int grid_solve, cudaStream_t stream, int variant, int n, int max_nb);
// resident blocks per SM of a variant's pre kernel for that largest world
int cpk_pre_blocks_per_sm(int variant, int max_nb);
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
// CP_PROFILE_SLOTS counters: per-phase cycles summed over blocks (prepare,
// broadphase, narrowphase, rows+wake+solve prep, row assembly, levels, GS
// sweeps, apply+integrate), then 16 per-resolver thread-cycle sums and 16
// per-resolver call counts (slots 10..12: pairs settled by a binary32
// no-contact certificate for sphere-plane, plane-hull, sphere-box)
cudaError_t cpk_phase_cycles(unsigned long long* out, bool reset);
cudaError_t cpk_set_resolver_profile(int on);
// Address and size of the static step scratch on `device`, which must be the
// current device; the first call per device looks the address up.
#define CP_MAX_DEVICES 64
cudaError_t cpk_static_scratch(int device, void** ptr, size_t* bytes);
// First failed index check of the solve kernel since the last read, as
// {code, world id, index, bound} (code 0: none); clears it once read.
cudaError_t cpk_read_check(int out[4]);
