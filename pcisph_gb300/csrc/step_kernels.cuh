// step_kernels.cuh -- launchers of the PCISPH step kernels (step_kernels.cu).
//
// Layout in HBM: particle vectors are float4 (xyz + a packed scalar where one is
// useful), scalars are float, the cell table is uint2 per bucket, all in the
// step's sorted order. The packed operands avoid separate gathers of a scalar
// per neighbour:
//   pr4[i]  = (x_i, rho_i)            read by the normal and force sweeps
//   pf4[i]  = (x_i, p_i / rho_i^2)    read by the pressure-force sweep
//   bpf[b]  = (x_b, p_b / rho0^2)     boundary operand of the pressure-force sweep
#pragma once
#include <cuda_runtime.h>

#include "common.cuh"

namespace pcisph {

struct StepBuffers {
    // fluid
    float4 *state_pos, *state_vel;   // particle state (integrated), input of the next sort
    float4 *pos, *vel;               // this step's sorted inputs
    float4 *pr4, *normal, *f_other, *f_press, *pred, *pf4;
    float *rho, *press, *err;
    uint32_t *keys, *ids;            // sorted keys and source indices
    uint2* cells;                    // fluid cell table [bucket_count]
    uint32_t* codes;                 // packed cell of each sorted particle (sweep.cuh cell_code)
    uint32_t* groups;                // start of every bucket run (count in ctl->n_groups)
    float* state_skin;               // per-particle skins: each particle's half skin, in the state's order
    float* disp_max;                 // per-particle skins: this step's largest predicted displacement
    uint32_t* nbr;                   // neighbour lists, list_cap entries per particle (kernel_variant 2)
    uint32_t* nbr_count;             // entries per particle; > list_cap means "walk the buckets"
    uint32_t* near;                  // within-h lists, near_cap entries per particle
    uint32_t* near_count;            // entries per particle; > near_cap means "walk the buckets"
    unsigned char* bucket_fast;      // per bucket: holds a particle predicted to move > skin / 2 (this step)
    unsigned char* b_near;           // per particle (B > 0): a boundary particle within the list radius
    uint32_t* bnbr;                  // per particle (B > 0): boundary particles within the list radius
    uint32_t* bnbr_count;            // entries per particle; > bnd_cap means "walk the boundary buckets"
    uint32_t* bfl;                   // per boundary particle: fluid particles within the list radius
    uint32_t* bfl_count;             // entries per boundary particle; > bfl_cap means "walk"
    uint32_t* fast_list;             // partner marks: the round's fast predictions (mark_cap entries)
    uint32_t* walk_stamp;            // partner marks: per particle, the last round that stamped it to walk
    // boundary
    float4 *b_pos, *bpf;
    float *b_press, *b_init;
    uint2* b_cells;                  // boundary cell table [bucket_count]
    uint32_t* b_codes;
    Control* ctl;
};

// Kernels launched per call are reported through the return value (count), errors via cudaGetLastError.
void launch_hash(const float* pos, bool packed, uint32_t n, const DevParams& P, uint32_t* keys, uint32_t* ids,
                 cudaStream_t s);
// Also writes cell codes (if codes) and appends bucket-run starts to groups (if groups).
void launch_reorder(const uint32_t* keys, const uint32_t* ids, const float4* in_pos, const float4* in_vel,
                    uint32_t n, float4* out_pos, float4* out_vel, uint2* cells, uint32_t* codes, uint32_t* groups,
                    const DevParams& P, Control* ctl, cudaStream_t s, const float* in_skin = nullptr);
void launch_begin(Control* ctl, cudaStream_t s);
void launch_density(const DevParams& P, const StepBuffers& b, cudaStream_t s);
void launch_normal(const DevParams& P, const StepBuffers& b, cudaStream_t s);
void launch_force(const DevParams& P, const StepBuffers& b, cudaStream_t s);
void launch_boundary_self_density(const DevParams& P, const StepBuffers& b, cudaStream_t s);
// cells: the fluid cell table in the order b.pred is stored in (sorted or working order)
void launch_boundary_pressure(const DevParams& P, const StepBuffers& b, const uint2* cells, cudaStream_t s);
void launch_pressure(const DevParams& P, const StepBuffers& b, cudaStream_t s);
// mode 0: the loop decision in ctl picks predict or integrate; 1: predict; 2: integrate.
// With use_cond, thread 0 also sets the graph's while-loop condition (continue unless done or max_iters).
void launch_pressure_force(const DevParams& P, const StepBuffers& b, int mode, cudaGraphConditionalHandle cond,
                           bool use_cond, cudaStream_t s);
void launch_pack(const DevParams& P, const StepBuffers& b, cudaStream_t s);
// Warp-per-bucket sweeps (sweep_kernels.cu)
struct SweepGrid {
    int blocks[5];  // resident blocks (SMs x occupancy) of density, normal, force, pressure, pressure force
    int warps[5];
};
cudaError_t sweep_configure(SweepGrid* g);
struct SweepArgs;
void launch_density_sweep(const DevParams& P, const StepBuffers& b, const SweepArgs& A, const SweepGrid& g,
                          cudaStream_t s);
void launch_normal_sweep(const DevParams& P, const StepBuffers& b, const SweepArgs& A, const SweepGrid& g,
                         cudaStream_t s);
void launch_force_sweep(const DevParams& P, const StepBuffers& b, const SweepArgs& A, const SweepGrid& g,
                        cudaStream_t s);
void launch_pressure_sweep(const DevParams& P, const StepBuffers& b, const SweepArgs& A, const SweepGrid& g,
                           cudaStream_t s);
void launch_pressure_force_sweep(const DevParams& P, const StepBuffers& b, const SweepArgs& A, const SweepGrid& g,
                                 int mode, cudaGraphConditionalHandle cond, bool use_cond, cudaStream_t s);

void launch_pack3_to4(const float* in3, float4* out, uint32_t n, cudaStream_t s);
void launch_unpack4_to3(const float4* in, float* out3, uint32_t n, cudaStream_t s);

}  // namespace pcisph
