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
// time_inc: added to each world's time per step (dt for World.step, 0 for
// World.internalStep, which leaves the clock to its caller)
cudaError_t cpk_launch_step(const DWorld* d_worlds, const int* d_ids, const int* d_gstart, int ngroups, double dt, double time_inc,
                            int* d_queue, int grid_pre, int grid_solve, cudaStream_t stream, int variant, int n, int max_nb);
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
// World.step's interpolation of one world (world_class.dart:420-428) at
// t = accumulator / dt: interpolated pose, then previousQuaternion.normalize()
cudaError_t cpk_interpolate(const DWorld* d_world, int nb, double t, cudaStream_t stream);
// the per-step body fields of one world to (to_device = 1) or from the
// packed records d_buf
cudaError_t cpk_states(const DWorld* d_world, int nb, cp_body_state* d_buf, int to_device, cudaStream_t stream);
// One large world over the whole GPU (cp_wide.cu): the sizes and settings
// the host knows, and the most bodies whose sweep velocities fit in one
// block's shared memory.
struct WideShape {
  int nb, nbins, broadphase, n_nocollide;
  int pairs_cap, contacts_cap, rows_cap, bins_cap;
  int smem_vel;  // the sweeps keep vlambda / wlambda in shared memory
  int compound, jobs_cap;  // shape-pair jobs of compound bodies, their capacity
};
int cpk_wide_smem_vel_max();
// nsteps steps of the world whose device descriptor is dw (hw: its host
// copy); each step is a sequence of grid-wide kernels on `stream`; the
// world's step status and counts end up in its parameters as with
// cpk_launch_step.  *launches grows by the kernels launched.
cudaError_t cpk_launch_wide_steps(const DWorld* dw, const DWorld& hw, const WideShape& ws, double dt, double time_inc,
                                  int nsteps, cudaStream_t stream, long long* launches);
// the wide sweep kernel's first failed index check {code, index, bound, 0}
// (code 0: none); clears it once read
cudaError_t cpk_wide_check(const DWorld& hw, int out[4], cudaStream_t stream);
// Filter check switch and counters {pairs checked, disagreements} of the
// one-block kernels (cp_step.cu) and of the wide kernels (cp_wide.cu); the
// device must be current
cudaError_t cpk_filter_check(int on);
cudaError_t cpk_filter_counts(unsigned long long out[2], bool reset);
cudaError_t cpk_wide_filter_check(int on);
cudaError_t cpk_wide_filter_counts(unsigned long long out[2], bool reset);
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
// the same record copied on `stream` into `out` (pinned host memory), without
// clearing it; cpk_read_check reads and clears it once a copy showed a failure
cudaError_t cpk_read_check_async(int* out, cudaStream_t stream);
// World.raycastClosest / Any / All over one world (cp_ray.cu): refresh the
// AABBs that need it (and re-sort a SAP axis list), then one ray per thread
cudaError_t cpk_raycast(const DWorld* d_world, const cp_ray* d_rays, int n, int mode, cp_ray_hit* d_hits, int max_hits,
                        int* d_counts, cudaStream_t stream);
