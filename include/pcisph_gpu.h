/*
 * pcisph_gpu.h -- C ABI of the GB300 (sm_103a) PCISPH time step.
 *
 * Drop-in for the reference's simulation step, class sim::Fluid
 * (PCISPH/src/sim/Fluid.h:13-102, Fluid.cpp:32-466), and for the clogs radix
 * sort it calls (libs/clogs/include/clogs/radixsort.h:55-211). Plain C types
 * only: pointers, sizes, status codes. All device memory of a context is owned
 * by the context; callers pass host or device pointers to import and export
 * state. Calls on one context are not thread-safe; use one context per thread.
 * Every call returns PCISPH_OK or an error code; pcisph_last_error() gives the
 * message of the last failing call on the calling thread. Nothing throws
 * across this boundary and no kernel traps: device-side failures are status
 * bits read by pcisph_last_stats().
 *
 * Host-side C++ mirror: include/pcisph_fluid.hpp (class pcisph::Fluid).
 */
#ifndef PCISPH_GPU_H
#define PCISPH_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PCISPH_ABI_VERSION 1

#if defined(__GNUC__)
#define PCISPH_API __attribute__((visibility("default")))
#else
#define PCISPH_API
#endif

/* ------------------------------------------------------------ status codes */
enum pcisph_status {
    PCISPH_OK = 0,
    PCISPH_ERR_INVALID_ARG = 1,   /* bad pointer, size, layout or enum value */
    PCISPH_ERR_OOM = 2,           /* device allocation failed */
    PCISPH_ERR_CUDA = 3,          /* a CUDA runtime call failed (message has the CUDA error) */
    PCISPH_ERR_INCONSISTENT = 4,  /* state size does not match the counts (Fluid.cpp:90-106) */
    PCISPH_ERR_NOT_READY = 5,     /* state not set yet */
    PCISPH_ERR_TIMEOUT = 6        /* a bounded device wait gave up */
};

/* Step status bits, written on the device, read through pcisph_last_stats(). */
enum pcisph_step_status {
    PCISPH_STEP_NOT_CONVERGED = 1u, /* max iterations reached with max error >= threshold */
    PCISPH_STEP_NONFINITE = 2u,     /* a predicted density was NaN or infinite */
    PCISPH_STEP_BAD_INDEX = 4u      /* a sorted key or source index was out of range (reorder skipped it) */
};

/* --------------------------------------------------------------- params */
/* Mirror of Simulation_Params (PCISPH/data/kernels/Simulation_Params.h:18-44): 20 x 4 B, packed. */
typedef struct pcisph_sim_params {
    float particle_radius;
    float particle_mass;
    float rest_density;
    uint32_t boundary_count;
    uint32_t fluid_count;
    float kernel_radius;
    float kernel_radius2;
    uint32_t bucket_count;
    float cell_size;
    float poly6_normalization;
    float poly6_d1_normalization;
    float viscosity_d2_normalization;
    float spiky_d1_normalization;
    float surface_tension_coefficient;
    float surface_tension_term;
    float surface_tension_normalization;
    float viscosity_constant;
    float gravity;
    float delta_t;
    float density_variation_scaling_factor;
} pcisph_sim_params;

/* Step options. The reference fixes these in code; defaults reproduce it. */
typedef struct pcisph_options {
    int32_t min_iterations;        /* default 3: the reference tests convergence from i >= 2 (Fluid.cpp:250, :284) */
    int32_t max_iterations;        /* default 7 (Fluid.cpp:251) */
    int32_t walls;                 /* default 0 (reference: none); 1: reflecting box after integration */
    float box_lo[3];
    float box_hi[3];
    float restitution;             /* wall restitution (velocity scale on reflection) */
    int32_t boundary_self_density; /* default 0: boundary-boundary predicted density stays zero, as the
                                      reference never launches that kernel (Fluid.cpp:167-171); 1: computed */
    int32_t loop_mode;             /* default 0: the corrective loop is decided on the device (CUDA graph with
                                      a conditional while node); 1: host reads the decision each iteration,
                                      like the reference (Fluid.cpp:300-306); 2: the whole loop in one
                                      persistent cooperative kernel (grid barriers between the sweeps) */
    int32_t kernel_variant;        /* neighbour sweeps. default 2: per-particle neighbour lists built by the
                                      density sweep (27-bucket walk), reused by the later sweeps of the step;
                                      0: one warp per bucket run with shared-memory staging; 1: one thread per
                                      particle walking the 27 buckets in every sweep */
    float list_skin;               /* variant 2: list radius = kernel_radius * (1 + list_skin), default 0.25 */
    int32_t spatial_order;         /* variant 2: 1, the sweeps run in a working order that places whole
                                      buckets in Morton order of their cells (every sum unchanged; state and
                                      exported fields stay in the reference's sorted order); 0: sorted order;
                                      2 (default): 1 from 131,072 particles, else 0 */
    int32_t sweep_block;           /* variant 2: threads per block of the pressure and pressure-force sweeps
                                      (the corrective loop's kernels): 128, 256 (default) or 512 */
    int32_t particle_skin;         /* variant 2, per-particle skins. 1: particle i's fluid list takes the radius
                                      h + s_i + list_skin h / 2 and its boundary list h + s_i, s_i its own half
                                      skin (twice its largest predicted displacement of the previous step,
                                      within [0.02 h, list_skin h / 2]); a prediction past s_i makes that
                                      particle walk. 0: s_i = list_skin h / 2 for every particle. 2 (default):
                                      1 for scenes with boundary particles (their boundary lists shrink; the
                                      boundary workload runs 6% faster), else 0 (fluid-only lists gain nothing
                                      measurable). Results are the same bits in every mode */
} pcisph_options;

typedef struct pcisph_step_stats {
    int32_t iterations;          /* corrective iterations of the last step */
    float max_density_error;     /* max density variation / rest density, last iteration of the last step */
    uint32_t status;             /* pcisph_step_status bits of the last step */
    uint32_t status_all;         /* OR of the status bits of every step since the last reset */
    uint64_t steps;              /* steps done by this context */
    uint64_t total_iterations;   /* corrective iterations summed over those steps */
    uint64_t list_fallbacks;     /* variant 2: pressure sweeps in which some predicted displacement exceeded
                                    half the list skin (that particle, and the particles its prediction
                                    reached that their lists lacked, walked the buckets) */
    uint64_t fast_particles;     /* variant 2: predictions that moved more than half the list skin */
    float list_skin;             /* variant 2: the list skin of the last step, units of h */
    float max_density_error_max; /* largest end-of-step max_density_error of the steps since the last reset */
    uint64_t unconverged_steps;  /* steps since the last reset that ended at max_iterations with the density
                                    variation still above the threshold (status bit 0) */
} pcisph_step_stats;

/* ----------------------------------------------------------- enums */
enum pcisph_layout {
    PCISPH_LAYOUT_PACKED3 = 0,  /* n x 3 floats (the reference's vload3/vstore3 layout) */
    PCISPH_LAYOUT_FLOAT4 = 1,   /* n x 4 floats, w ignored on input, 0 on output */
    PCISPH_LAYOUT_SCALAR = 2    /* n floats or n uint32 */
};
enum pcisph_memory { PCISPH_MEM_HOST = 0, PCISPH_MEM_DEVICE = 1 };

enum pcisph_field {
    PCISPH_FIELD_POSITION = 0,            /* particle state: after the last step, in its sorted order */
    PCISPH_FIELD_VELOCITY = 1,
    PCISPH_FIELD_NORMAL = 2,              /* Fluid.h:44 fluid_normals */
    PCISPH_FIELD_PREDICTED_POSITION = 3,  /* fluid_predicted_positions */
    PCISPH_FIELD_DENSITY = 4,             /* fluid_densities */
    PCISPH_FIELD_OTHER_FORCE = 5,         /* fluid_other_forces */
    PCISPH_FIELD_PRESSURE = 6,            /* fluid_pressures */
    PCISPH_FIELD_PRESSURE_FORCE = 7,      /* fluid_pressure_forces */
    PCISPH_FIELD_DENSITY_VARIATION = 8,   /* fluid_density_variations (internal, Fluid.h:99) */
    PCISPH_FIELD_SORTED_POSITION = 9,     /* the step's positions after reorder */
    PCISPH_FIELD_SORTED_VELOCITY = 10,
    PCISPH_FIELD_KEYS = 11,               /* fluid_keys, sorted (uint32) */
    PCISPH_FIELD_SRC = 12,                /* fluid_src_locations (uint32) */
    PCISPH_FIELD_CELL_OFFSETS = 13,       /* fluid_cell_offsets, 2 x bucket_count uint32 */
    PCISPH_FIELD_BOUNDARY_POSITION = 14,  /* boundary_positions, sorted once sorted */
    PCISPH_FIELD_BOUNDARY_PRESSURE = 15,
    PCISPH_FIELD_BOUNDARY_INIT_DENSITY = 16,
    PCISPH_FIELD_BOUNDARY_KEYS = 17,
    PCISPH_FIELD_BOUNDARY_SRC = 18,
    PCISPH_FIELD_BOUNDARY_CELL_OFFSETS = 19,
    PCISPH_FIELD_COUNT_ = 20
};

/* Single stages of the step, for parity testing of each kernel on given inputs. */
enum pcisph_stage {
    PCISPH_STAGE_SORT = 0,               /* boundary sort if pending, hash, radix sort, reorder + cell ranges */
    PCISPH_STAGE_DENSITY = 1,            /* pcisph.cl:65-92 */
    PCISPH_STAGE_NORMAL = 2,             /* pcisph.cl:94-112 */
    PCISPH_STAGE_FORCE = 3,              /* pcisph.cl:121-173, then the first predict (pcisph.cl:175-193) */
    PCISPH_STAGE_BOUNDARY_PRESSURE = 4,  /* pcisph.cl:212-263, boundary_update = 1 */
    PCISPH_STAGE_PRESSURE = 5,           /* pcisph.cl:212-263, boundary_update = 0, + max reduction */
    PCISPH_STAGE_PRESSURE_FORCE = 6,     /* pcisph.cl:265-300 then predict (arg 0) or integrate (arg 1) */
    PCISPH_STAGE_PACK = 7,               /* rebuild packed operands from DENSITY, PRESSURE and
                                            BOUNDARY_PRESSURE after set_field */
    PCISPH_STAGE_BOUNDARY_PRESSURE_RESET = 8 /* pcisph.cl:114-119 */
};

typedef struct pcisph_ctx pcisph_ctx;

/* ------------------------------------------------------------- general */
PCISPH_API int pcisph_abi_version(void);
PCISPH_API const char* pcisph_last_error(void);
/* Setters + Fluid::update_deduced_attributes (Fluid.cpp:333-443) as a pure host function. */
PCISPH_API int pcisph_derive_params(float particle_radius, float rest_density, uint32_t fluid_count, uint32_t boundary_count,
                         float delta_t, float gravity, float viscosity, float surface_tension,
                         pcisph_sim_params* out);
/* Fluid.cpp:125-133 */
PCISPH_API uint32_t pcisph_sort_bit_count(uint32_t elements);
PCISPH_API int pcisph_default_options(pcisph_options* out);

/* ------------------------------------------------------------ context */
/* sim::Fluid::Fluid(ctx, device, queue) (Fluid.cpp:32-88). stream: cudaStream_t or NULL (legacy). */
PCISPH_API int pcisph_create(int device, void* stream, pcisph_ctx** out);
PCISPH_API void pcisph_destroy(pcisph_ctx* ctx);
PCISPH_API int pcisph_set_stream(pcisph_ctx* ctx, void* stream);

/* Setters, Fluid.h:21-29 (Fluid.cpp:333-375): each marks the parameters changed; the next update()
 * re-derives them, reallocates and zeroes the velocities, like update_deduced_attributes. */
PCISPH_API int pcisph_set_boundary_count(pcisph_ctx* ctx, uint32_t boundary_count);
PCISPH_API int pcisph_set_fluid_count(pcisph_ctx* ctx, uint32_t fluid_count);
PCISPH_API int pcisph_set_delta_t(pcisph_ctx* ctx, float delta_t);
PCISPH_API int pcisph_set_rest_density(pcisph_ctx* ctx, float rest_density);
PCISPH_API int pcisph_set_particle_radius(pcisph_ctx* ctx, float particle_radius);
PCISPH_API int pcisph_set_gravity(pcisph_ctx* ctx, float gravity);
PCISPH_API int pcisph_set_viscosity(pcisph_ctx* ctx, float viscosity);
PCISPH_API int pcisph_set_surface_tension(pcisph_ctx* ctx, float surface_tension_coefficient);
PCISPH_API int pcisph_set_density_variation_threshold(pcisph_ctx* ctx, float threshold);
PCISPH_API int pcisph_set_options(pcisph_ctx* ctx, const pcisph_options* options);
PCISPH_API int pcisph_get_options(const pcisph_ctx* ctx, pcisph_options* out);
/* Fluid::get_params (Fluid.cpp:329-331): the current struct, derived fields as of the last derivation. */
PCISPH_API int pcisph_get_params(const pcisph_ctx* ctx, pcisph_sim_params* out);
/* Derive now if parameters changed (zeroing velocities), so that state set afterwards survives. */
PCISPH_API int pcisph_prepare(pcisph_ctx* ctx);

/* State import, replacing the caller-assigned cl::Buffers (scenes.cpp:191-208). count must equal the
 * configured count (checked at update(), Fluid.cpp:90-106). vel may be NULL (zero). Stream-ordered. */
PCISPH_API int pcisph_set_fluid_state(pcisph_ctx* ctx, const float* pos, const float* vel, uint32_t count, int layout,
                           int memory);
PCISPH_API int pcisph_set_boundary_state(pcisph_ctx* ctx, const float* pos, uint32_t count, int layout, int memory);
/* Fluid::checkBuffersConsistent (Fluid.cpp:90-106) */
PCISPH_API int pcisph_check_buffers_consistent(const pcisph_ctx* ctx);

/* Fluid::update (Fluid.cpp:108-327): one time step, stream-ordered, no host synchronisation in
 * loop_mode 0. */
PCISPH_API int pcisph_update(pcisph_ctx* ctx);
PCISPH_API int pcisph_step(pcisph_ctx* ctx, uint32_t steps);
PCISPH_API int pcisph_sync(pcisph_ctx* ctx);
/* Bounded wait: PCISPH_ERR_TIMEOUT if the queued work is still running after timeout_ms (0: query once).
 * Nothing is cancelled; a later sync picks the work up. For callers that must not block (a serving loop
 * watching for stalled steps). */
PCISPH_API int pcisph_sync_for(pcisph_ctx* ctx, int64_t timeout_ms);
/* Synchronises, then reports the last step. */
PCISPH_API int pcisph_last_stats(pcisph_ctx* ctx, pcisph_step_stats* out);
PCISPH_API int pcisph_reset_stats(pcisph_ctx* ctx);

/* Export. dst_bytes must cover count x layout; HOST copies synchronise. */
PCISPH_API int pcisph_get_field(pcisph_ctx* ctx, int field, void* dst, size_t dst_bytes, int layout, int memory);
/* The counterpart of pcisph_set_fluid_state: positions and velocities (either may be NULL) in one call with
 * one synchronisation. Pinned host buffers (cudaHostAlloc / cudaHostRegister) are written by the layout
 * conversion kernel directly, as pinned sources are read by pcisph_set_fluid_state; other host memory goes
 * through a device staging buffer. */
PCISPH_API int pcisph_get_fluid_state(pcisph_ctx* ctx, float* pos, float* vel, uint32_t count, int layout, int memory);
/* Overwrite one field (parity tests feed identical inputs to a stage). */
PCISPH_API int pcisph_set_field(pcisph_ctx* ctx, int field, const void* src, size_t src_bytes, int layout, int memory);
/* Zero-copy view (replaces the CL-GL shared buffers): device pointer, element count, native layout. */
PCISPH_API int pcisph_field_device_ptr(pcisph_ctx* ctx, int field, void** ptr, size_t* count, int* layout);
PCISPH_API int pcisph_run_stage(pcisph_ctx* ctx, int stage, int arg);

/* Kernels launched by this context since creation (for launch accounting). */
PCISPH_API uint64_t pcisph_kernel_launches(const pcisph_ctx* ctx);

/* Autotuning. Times `steps` steps (after one warm-up step) of every candidate of variant 2's knobs --
 * list skin 0.15, 0.2, 0.25, 0.3; working order on or off; radix digit width 6 or 8 bits -- from the
 * current state, restores the state and the statistics after each, and keeps the fastest. Every candidate
 * computes the same bits (the knobs change memory layout and list length, never a sum), so tuning leaves
 * the simulation unchanged. Synchronises. No counterpart in the reference. */
typedef struct pcisph_tune_result {
    float list_skin;
    int32_t spatial_order;
    int32_t digit_bits;
    int32_t sweep_block;
    float ms_per_step;          /* the chosen candidate */
    float ms_per_step_before;   /* the settings on entry */
    int32_t candidates;
} pcisph_tune_result;
PCISPH_API int pcisph_autotune(pcisph_ctx* ctx, uint32_t steps, pcisph_tune_result* out);

/* Checkpoints. A snapshot is a self-describing host buffer: a header (magic "PCSN", format version, the
 * sizes of the parameter and option records, particle counts, threshold, steps taken), the parameter
 * setters' values, the options, then the fluid positions and velocities (float4 per particle, sorted
 * order of the last step) and the boundary positions as set (float4). pcisph_snapshot synchronises the
 * context's stream. pcisph_restore sets the parameters and options, re-derives them and loads the state,
 * so the next update continues exactly where the snapshot was taken; the step counter of pcisph_last_stats
 * continues from the snapshot's, the other statistics start over. No counterpart in the reference. */
PCISPH_API int pcisph_snapshot_size(pcisph_ctx* ctx, size_t* bytes);
PCISPH_API int pcisph_snapshot(pcisph_ctx* ctx, void* dst, size_t dst_bytes);
PCISPH_API int pcisph_restore(pcisph_ctx* ctx, const void* src, size_t src_bytes);

/* Per-kernel CUDA-event timing of the host-driven path (loop_mode 1 timing is used while enabled). */
typedef struct pcisph_kernel_time {
    char name[32];
    uint64_t launches;
    double total_ms;
} pcisph_kernel_time;
PCISPH_API int pcisph_profile_enable(pcisph_ctx* ctx, int enable);
PCISPH_API int pcisph_profile_read(pcisph_ctx* ctx, pcisph_kernel_time* out, int max_entries, int* n_entries);

/* ------------------------------------------------------- batched scenes */
/* Many independent scenes advanced together: one launch per kernel per step for all of them. Each scene
 * keeps its own parameters, bucket count and convergence: a scene stops iterating when its own max
 * density error is below its threshold, while the others continue. Scene ids sit in the high part of one
 * shared key space (each scene owns a range of buckets), so one stable sort orders all scenes and each
 * scene's sorted order is the one it would have alone. Scenes have no boundary particles. No counterpart
 * in the reference, which runs one scene per sim::Fluid. */
typedef struct pcisph_batch pcisph_batch;

typedef struct pcisph_scene_desc {
    uint32_t fluid_count;
    float particle_radius;               /* the reference's setters (Fluid.h:21-29) */
    float rest_density;
    float delta_t;
    float gravity;
    float viscosity;                     /* the reference's viscosity_constant */
    float surface_tension;
    float density_variation_threshold;
    int32_t min_iterations;
    int32_t max_iterations;
    int32_t walls;
    float box_lo[3];
    float box_hi[3];
    float restitution;
} pcisph_scene_desc;

/* max_particles and max_scenes size the device pool (all of it is allocated here). */
PCISPH_API int pcisph_batch_create(int device, void* stream, uint32_t max_particles, uint32_t max_scenes,
                                   pcisph_batch** out);
PCISPH_API void pcisph_batch_destroy(pcisph_batch* batch);
/* Bytes of device memory per particle and per scene in a pool (for admission against a budget). */
PCISPH_API int pcisph_batch_memory_model(uint64_t* bytes_per_particle, uint64_t* bytes_per_scene);
/* Adds a scene with its initial state (vel may be NULL: zero); *scene_id is a handle valid until removal.
 * The scene tables and the step's graph are rebuilt once, at the next step, for all additions and
 * removals since the last step. */
PCISPH_API int pcisph_batch_add_scene(pcisph_batch* batch, const pcisph_scene_desc* desc, const float* pos,
                                      const float* vel, int layout, int memory, int32_t* scene_id);
/* Removes a scene: its id is invalid at once; its particles leave the pool at the next step, which compacts
 * the pool once for all removals (stream-ordered device copies). */
PCISPH_API int pcisph_batch_remove_scene(pcisph_batch* batch, int32_t scene_id);
/* Autotuning of a batch on its current scenes: times `steps` batched steps (after a warm-up step) for each
 * list skin (adaptive, 0.25, 0.35, 0.5) x loop mode 0, 2 x radix digit width 8, 10, 6, restoring the
 * pool's state and statistics after each, and keeps the fastest. Every candidate computes the same bits.
 * Synchronises. list_skin = PCISPH_LIST_SKIN_ADAPTIVE when the adaptive skin won. */
typedef struct pcisph_batch_tune_result {
    float list_skin;
    int32_t loop_mode;
    int32_t digit_bits;
    float ms_per_step;
    float ms_per_step_before;
    int32_t candidates;
} pcisph_batch_tune_result;
PCISPH_API int pcisph_batch_autotune(pcisph_batch* batch, uint32_t steps, pcisph_batch_tune_result* out);
/* 0 (default): the corrective loop is a conditional WHILE node of the step's graph; 2: one persistent
 * cooperative kernel runs it with per-scene convergence flags. Same results either way. */
PCISPH_API int pcisph_batch_set_loop_mode(pcisph_batch* batch, int loop_mode);
/* Neighbour-list skin of every scene, in units of h, in [0, 2] (pcisph_options.list_skin of a single
 * context), or PCISPH_LIST_SKIN_ADAPTIVE (the default): before each step every scene takes the smallest of
 * the skins 0.25, 0.35, 0.5 that at most 1 in 500 of its previous step's predictions outran (the largest
 * if none), on the device. Results do not depend on the skin. */
#define PCISPH_LIST_SKIN_ADAPTIVE (-1.0f)
PCISPH_API int pcisph_batch_set_list_skin(pcisph_batch* batch, float skin);
PCISPH_API int pcisph_batch_info(const pcisph_batch* batch, uint32_t* scenes, uint32_t* particles,
                                 uint32_t* free_particles);
/* steps time steps of every scene (one CUDA graph launch each; no host synchronisation). */
PCISPH_API int pcisph_batch_step(pcisph_batch* batch, uint32_t steps);
PCISPH_API int pcisph_batch_sync(pcisph_batch* batch);
/* Per-kernel timing of a batch, as pcisph_profile_enable / _read: while enabled, steps run host-driven (the
 * same kernels as the step graph, the loop's continuation read back each iteration), every launch timed. */
PCISPH_API int pcisph_batch_profile_enable(pcisph_batch* batch, int enable);
PCISPH_API int pcisph_batch_profile_read(pcisph_batch* batch, pcisph_kernel_time* out, int max_entries, int* n_entries);
/* pcisph_sync_for for a batch's stream. */
PCISPH_API int pcisph_batch_sync_for(pcisph_batch* batch, int64_t timeout_ms);
/* Synchronises, then reports the scene's last step (and totals since it was added). */
PCISPH_API int pcisph_batch_scene_stats(pcisph_batch* batch, int32_t scene_id, pcisph_step_stats* out);
/* Replaces a scene's positions (and velocities; NULL: zero), as pcisph_set_fluid_state; count must be the
 * scene's particle count. The scene keeps its parameters, statistics and place in the pool. */
PCISPH_API int pcisph_batch_set_state(pcisph_batch* batch, int32_t scene_id, const float* pos, const float* vel,
                                      uint32_t count, int layout, int memory);
/* A field of one scene (its particles in its own sorted order), as pcisph_get_field. */
PCISPH_API int pcisph_batch_get_field(pcisph_batch* batch, int32_t scene_id, int field, void* dst,
                                      size_t dst_bytes, int layout, int memory);
PCISPH_API uint64_t pcisph_batch_kernel_launches(const pcisph_batch* batch);
/* Step graphs instantiated, and updated in place after a change of composition, since creation. */
PCISPH_API int pcisph_batch_graph_stats(const pcisph_batch* batch, uint64_t* instantiations, uint64_t* updates);

/* ------------------------------------------------------------ rendering */
/* Headless replacement of the reference's OpenGL particle rendering (vis/fluid_rendering.cpp:65-103 with
 * data/shaders/simple_particle.vert and .frag): spheres of the particle radius coloured by density
 * (blue at 0.95 rho0, purple at rho0, orange at 1.05 rho0), lit from +y with 0.2 ambient, darkened with
 * view depth from 5 to 20. The reference's camera is eye = d (sin a, 0.2, cos a), target 0, up +y, 60
 * degrees horizontal field of view (main.cpp:174-179). Output: RGB8, row 0 at the top. */
typedef struct pcisph_camera {
    float eye[3];
    float target[3];
    float up[3];
    float fov_x_degrees;
} pcisph_camera;
/* Device pointers: pos4 (n float4), density (n floats, or NULL: all at rest density), zbuffer (width *
 * height * 8 bytes of scratch), rgb (width * height * 3 bytes). Stream-ordered on `stream`. */
PCISPH_API int pcisph_render(const float* pos4, const float* density, uint32_t n, float particle_radius,
                             float rest_density, const pcisph_camera* cam, int width, int height, void* zbuffer,
                             size_t zbuffer_bytes, uint8_t* rgb, void* stream);
/* The context's fluid (positions and densities of the last step) into a host RGB8 image of width * height
 * * 3 bytes (synchronises). */
PCISPH_API int pcisph_render_fluid(pcisph_ctx* ctx, const pcisph_camera* cam, int width, int height, uint8_t* rgb,
                                   size_t rgb_bytes);

/* --------------------------------------------------- standalone kernels */
/* sort_utils.cl:12-23: key = hash(floor(pos / cell_size)) % bucket_count, id = index. Device pointers. */
PCISPH_API int pcisph_hash_keys(const pcisph_sim_params* params, const float* pos, int layout, uint32_t count, uint32_t* keys,
                     uint32_t* ids, void* stream);

/* Replacement for clogs::Radixsort (radixsort.h:55-211): stable LSD radix sort of uint32 keys carrying
 * uint32 values, on device pointers. max_bits 0 means 32; all keys must be < 2^max_bits. */
typedef struct pcisph_radixsort pcisph_radixsort;
PCISPH_API int pcisph_radixsort_create(int device, pcisph_radixsort** out);
PCISPH_API void pcisph_radixsort_destroy(pcisph_radixsort* sorter);
/* radixsort.h:186-191 */
PCISPH_API int pcisph_radixsort_enqueue(pcisph_radixsort* sorter, uint32_t* keys, uint32_t* values, size_t elements,
                             unsigned int max_bits, void* stream);
/* Digit width in bits (4..11); 0 selects the tuned default. */
PCISPH_API int pcisph_radixsort_set_digit_bits(pcisph_radixsort* sorter, int bits);

/* The same stable sort for callers that must not allocate device memory when they sort (a pool allocator
 * owns the device's memory, or an allocation would stall a latency-critical loop). No counterpart in the
 * reference. Its scratch is a fixed device array inside this library, reserved on every device that loads
 * the library until the process exits; sorts of more than PCISPH_NOALLOC_SORT_MAX_ELEMENTS keys are
 * rejected with PCISPH_ERR_INVALID_ARG. Every call looks up that array's address in the current context
 * (nothing is cached, so a re-created context is safe); the first call on a device may load the library's
 * GPU code there, so make it before any stream capture. All calls share the array: calls that overlap on
 * the GPU race, so order them on one stream. Keys, values, max_bits and stream as in pcisph_radixsort_enqueue, on the current
 * device. */
#define PCISPH_NOALLOC_SORT_MAX_ELEMENTS (1u << 20)
PCISPH_API int pcisph_radixsort_enqueue_noalloc(uint32_t* keys, uint32_t* values, size_t elements,
                                                unsigned int max_bits, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* PCISPH_GPU_H */
