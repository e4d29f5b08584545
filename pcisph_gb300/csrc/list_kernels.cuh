// list_kernels.cuh -- neighbour-list sweeps for one scene or a batch of scenes (list_kernels.cu).
#pragma once
#include <cuda_runtime.h>

#include "common.cuh"

namespace pcisph {

// Arrays the list sweeps read and write (sorted order; a batch concatenates its scenes).
struct ListBuffers {
    const float4 *pos, *vel;
    float4 *pr4, *normal, *f_other, *f_press, *pred, *pf4, *state_pos, *state_vel;
    float *rho, *press, *err;
    const uint2* cells;
    const uint2* b_cells;
    const float4 *b_pos, *bpf;
    uint32_t* nbr;               // the skin list, list_cap entries per particle in chunks of 8: entries
                                 // 8c..8c+7 of particle i at nbr[8 (c * nbr_stride + i)] (32 bytes)
    uint32_t* nbr_count;         // entries per particle; > list_cap: walk the buckets
    uint32_t* near;              // the within-h list (pairs within h at the current positions), near_cap
                                 // entries per particle, laid out like nbr
    uint32_t* near_count;        // entries per particle; > near_cap: walk the buckets
    unsigned char* bucket_fast;  // per bucket of the cell table: holds a fast particle this step
    uint32_t nbr_stride;         // particles in the arrays (>= every index i)
    const uint32_t* out_index;   // integration writes particle i's state at out_index[i] (null: at i)
    float* disp_max;             // per-particle skins: particle i's largest predicted displacement this step
    float* state_skin;           // per-particle skins: the next step's half skin, stored beside the state
    const float* b_init;         // boundary initial (self) densities and pressures (single scene, B > 0)
    float* b_press;
    unsigned char* b_near;       // per fluid particle (B > 0): a boundary particle within r_list of x at the
                                 // step's start; 0: the boundary terms of the step's sweeps are all zero
    uint32_t* bnbr;              // per fluid particle (B > 0, or null): the boundary particles within r_list
                                 // of x in walk order, bnd_cap entries laid out like nbr
    uint32_t* bnbr_count;        // entries per particle; > bnd_cap: walk the boundary buckets
    uint32_t* bfl;               // per boundary particle (B > 0, or null): the fluid particles within r_list
                                 // of it at the step's start, walk order, bfl_cap entries chunked over the
                                 // boundary particles (stride boundary_count)
    uint32_t* bfl_count;         // entries per boundary particle; > bfl_cap: walk the fluid buckets
    // B > 0 (or null): one byte per cell of the box zone_org + [0, zone_dim): 1 where a boundary particle's
    // cell is within two cells on every axis; a fluid particle whose cell is 0 or outside the box has no
    // boundary particle within 2h (its boundary terms are zero, none is within r_list)
    const unsigned char* b_zone;
    int zone_org[3];
    uint32_t zone_dim[3];
    // partner marks (one scene, or null): the fast predictions of the round (DevParams::mark_cap entries), and
    // per particle the last round in which the marking kernel stamped it to walk. walk_stamp is null in the
    // launches that do not follow a marking kernel (the stage runner, the persistent loop).
    uint32_t* fast_list;
    uint32_t* walk_stamp;
};

// Is the cell in the boundary zone (ListBuffers::b_zone)? Cells are the signed integers the reference's
// floor gives (grid_utils.cl:9-11), held as uint32; the offsets wrap modulo 2^32, which leaves every cell
// of the box at its offset (a cell far outside may wrap into the box: it then walks, which is exact).
__device__ __forceinline__ bool in_boundary_zone(const ListBuffers& b, const Cell& c) {
    const uint32_t ix = c.x - (uint32_t)b.zone_org[0], iy = c.y - (uint32_t)b.zone_org[1],
                   iz = c.z - (uint32_t)b.zone_org[2];
    if (ix >= b.zone_dim[0] || iy >= b.zone_dim[1] || iz >= b.zone_dim[2]) return false;
    return b.b_zone[((size_t)iz * b.zone_dim[1] + iy) * b.zone_dim[0] + ix] != 0;
}

// One scene: parameters by value; the pressure kernel's last block decides the loop.
struct OneScene {
    DevParams P;
    Control* ctl;
    static constexpr bool kBatched = false;
    __device__ uint32_t count() const { return P.fluid_count; }
    __device__ const DevParams& params(uint32_t) const { return P; }
    __device__ Control* control(uint32_t) const { return ctl; }
    __device__ bool skip_pressure(uint32_t) const { return false; }
    __device__ bool skip_force(uint32_t) const { return false; }
};

// A batch: particle i belongs to scene scene_of[i]; per-scene parameters and control in device tables.
struct SceneTable {
    const DevParams* table;
    Control* ctls;
    const uint16_t* scene_of;
    uint32_t n;          // particles of all scenes
    uint32_t n_scenes;
    static constexpr bool kBatched = true;
    __device__ uint32_t count() const { return n; }
    __device__ const DevParams& params(uint32_t i) const { return table[scene_of[i]]; }
    __device__ Control* control(uint32_t i) const { return &ctls[scene_of[i]]; }
    // the scene was decided done in an earlier iteration: no more pressure updates
    __device__ bool skip_pressure(uint32_t i) const { return ctls[scene_of[i]].done != 0u; }
    // the scene was integrated in an earlier iteration
    __device__ bool skip_force(uint32_t i) const { return ctls[scene_of[i]].finished != 0u; }
};

void launch_density_list(const DevParams& P, Control* ctl, const ListBuffers& b, cudaStream_t s);
// Boundary particles (B > 0): their fluid lists at the step's start, and their pressure update per
// iteration from those lists (walking the fluid buckets when a fast fluid particle is near or a list
// overflowed). One scene.
void launch_boundary_fluid_list(const DevParams& P, const ListBuffers& b, cudaStream_t s);
// The boundary particles' cell bounds (bounds = {min x, y, z, max x, y, z}, preset to INT_MAX / INT_MIN), and
// the zone map over org + [0, dim) (zeroed by the caller).
void launch_boundary_cell_bounds(const DevParams& P, const float4* b_pos, int* bounds, cudaStream_t s);
void launch_boundary_zone(const DevParams& P, const float4* b_pos, const int* org, const uint32_t* dim,
                          unsigned char* zone, cudaStream_t s);
void launch_boundary_pressure_list(const DevParams& P, Control* ctl, const ListBuffers& b, cudaStream_t s);
void launch_normal_list(const DevParams& P, Control* ctl, const ListBuffers& b, cudaStream_t s);
void launch_force_list(const DevParams& P, Control* ctl, const ListBuffers& b, cudaStream_t s);
// Partner marks of the prediction round just completed (DevParams::mark_cap; b.fast_list and b.walk_stamp
// set): the particles whose next pressure sweep must walk. That sweep (launched with b.walk_stamp) closes
// the round.
void launch_mark_partners(const DevParams& P, Control* ctl, const ListBuffers& b, cudaStream_t s);
// block: threads per block of the two corrective-loop sweeps (128, 256 or 512)
void launch_pressure_list(const DevParams& P, Control* ctl, const ListBuffers& b, int block, cudaStream_t s);
// mode 0: the loop decision picks predict or integrate; 1: predict; 2: integrate
void launch_pressure_force_list(const DevParams& P, Control* ctl, const ListBuffers& b, int mode,
                                cudaGraphConditionalHandle cond, bool use_cond, int block, cudaStream_t s);

void launch_batch_begin(DevParams* table, Control* ctls, uint32_t n_scenes, Control* batch, cudaStream_t s);
void launch_scene_of(const uint32_t* offsets, uint32_t n_scenes, uint32_t n, uint16_t* scene_of, cudaStream_t s);
void launch_hash_scenes(const SceneTable& t, const float4* pos, uint32_t* keys, cudaStream_t s);
void launch_density_scenes(const SceneTable& t, const ListBuffers& b, cudaStream_t s);
void launch_normal_scenes(const SceneTable& t, const ListBuffers& b, cudaStream_t s);
void launch_force_scenes(const SceneTable& t, const ListBuffers& b, cudaStream_t s);
void launch_pressure_scenes(const SceneTable& t, const ListBuffers& b, cudaStream_t s);
void launch_pressure_force_scenes(const SceneTable& t, const ListBuffers& b, cudaStream_t s);
// The whole corrective loop of a step in one cooperative launch (loop_mode 2); errors if the device cannot
// run it (cooperative launch unsupported).
cudaError_t launch_corrective_loop(const DevParams& P, Control* ctl, const ListBuffers& b, cudaStream_t s);
cudaError_t launch_corrective_loop_scenes(const SceneTable& t, const ListBuffers& b, Control* batch, int max_iters,
                                          cudaStream_t s);
// per-scene loop decision; sets the while-loop condition (continue while a scene iterates)
void launch_batch_decide(const SceneTable& t, Control* batch, int max_iters, cudaGraphConditionalHandle cond,
                         bool use_cond, cudaStream_t s);

}  // namespace pcisph
