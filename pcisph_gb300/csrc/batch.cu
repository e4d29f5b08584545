// batch.cu -- many independent scenes advanced by one set of launches (C ABI in include/pcisph_gpu.h).
//
// Layout. The scenes share one particle pool: scene k occupies [offset_k, offset_k + N_k) of every
// per-particle array, scenes packed in insertion order, compacted on removal. Scene k owns the bucket
// range [bucket_base_k, bucket_base_k + bucket_count_k) of one cell table, and its key for a particle is
// bucket_base_k + the reference key (grid_utils.cl:12-19 with the scene's own bucket_count). The keys of
// scene k are therefore all below those of scene k+1: one stable radix sort of the whole pool leaves
// every scene in its own range, ordered as a sort of that scene alone would order it.
//
// Step. One CUDA graph per batch composition: begin, clear tables, hash, sort, reorder, then the list
// sweeps of list_kernels.cu with per-particle parameters from the scene table, and a conditional WHILE
// node over {pressure, per-scene decision, pressure force}. A scene's decision follows the reference
// (Fluid.cpp:284-306) with its own threshold and limits; a converged scene integrates and then idles
// (its particles skip the sweeps) while the others keep iterating; the loop ends when every scene is done.
#include <cuda_runtime.h>

#include <cstring>
#include <vector>

#include "host_util.h"
#include "list_kernels.cuh"
#include "radix_sort.cuh"
#include "step_kernels.cuh"

using namespace pcisph;
using namespace pcisph::host;

namespace {

#define BTRY(call)                                                                                             \
    do {                                                                                                       \
        cudaError_t e_ = (call);                                                                               \
        if (e_ != cudaSuccess) return report_error(PCISPH_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

struct SceneSlot {
    int32_t id;
    pcisph_scene_desc desc;
    pcisph_sim_params params;
    uint32_t offset, count, bucket_base;
    bool removed;  // dropped at the next compaction
};

constexpr size_t kParticleBytes = 11 * 16 + 3 * 4 + 4 * 4 + 2 + (kListCapWide + kNearCap) * 4;  // allocate()'s arrays
constexpr size_t kBucketBytesPerParticle = 5;  // (8 B table + 1 B flag) per bucket, ~N/2 buckets

}  // namespace

struct pcisph_batch {
    int device = 0;
    cudaStream_t user_stream = nullptr, own_stream = nullptr, capture_stream = nullptr;
    uint32_t max_particles = 0, max_scenes = 0, max_buckets = 0;
    DeviceBlock pool, tables;
    float4 *state_pos, *state_vel, *pos, *vel, *pr4, *normal, *f_other, *f_press, *pred, *pf4, *staging;
    float *rho, *press, *err;
    uint32_t *keys, *ids, *nbr, *nbr_count, *near, *near_count;
    uint16_t* scene_of;
    uint2* cells;
    unsigned char* bucket_fast;
    DevParams* d_table;
    Control* d_ctls;
    uint32_t* d_offsets;
    Control* d_batch;
    Control* h_ctls = nullptr;  // pinned
    RadixSorter sorter;
    DeviceBlock sort_block;
    std::vector<SceneSlot> scenes;
    int32_t next_id = 1;
    uint32_t n_particles = 0, n_buckets = 0;
    int max_iters = 1;
    int loop_mode = 0;   // 0: conditional WHILE node; 2: one persistent cooperative kernel
    float list_skin = 0.25f;   // the skin of every scene when adaptive_skin is off
    bool adaptive_skin = true;  // each scene picks its skin every step (k_batch_begin)
    bool dirty = false;  // scenes were added or removed since the tables were built
    cudaGraphExec_t graph_exec = nullptr;
    bool graph_valid = false;
    uint64_t graph_instantiations = 0, graph_updates = 0;
    uint64_t host_launches = 0;
    int prefix_launches = 0, iter_launches = 3;
    uint32_t *sorted_keys = nullptr, *sorted_ids = nullptr;
    bool profiling = false;   // steps run host-driven, every launch timed
    host::KernelTimer timer;

    cudaStream_t stream() const { return user_stream; }

    template <class F>
    void timed(const char* name, cudaStream_t s, F&& f) {
        if (profiling) timer.timed(name, s, f);
        else f();
    }

    ~pcisph_batch() {
        DeviceGuard g(device);
        if (user_stream) cudaStreamSynchronize(user_stream);
        timer.release();
        if (graph_exec) cudaGraphExecDestroy(graph_exec);
        pool.release();
        tables.release();
        sort_block.release();
        if (h_ctls) cudaFreeHost(h_ctls);
        if (own_stream) cudaStreamDestroy(own_stream);
        if (capture_stream) cudaStreamDestroy(capture_stream);
    }

    int allocate() {
        const size_t n = max_particles, nb = max_buckets, ns = max_scenes;
        const size_t bytes = 11 * align256(n * 16) + 3 * align256(n * 4) + 4 * align256(n * 4) + align256(n * 2) +
                             align256(n * kListCapWide * 4) + align256(n * kNearCap * 4) + align256(nb * 8) +
                             align256(nb);
        if (pool.ensure(bytes) != cudaSuccess)
            return report_error(PCISPH_ERR_OOM, "device allocation of the batch pool failed (" + std::to_string(bytes) + " bytes)");
        Carver c{static_cast<unsigned char*>(pool.p)};
        state_pos = c.take<float4>(n);
        state_vel = c.take<float4>(n);
        pos = c.take<float4>(n);
        vel = c.take<float4>(n);
        pr4 = c.take<float4>(n);
        normal = c.take<float4>(n);
        f_other = c.take<float4>(n);
        f_press = c.take<float4>(n);
        pred = c.take<float4>(n);
        pf4 = c.take<float4>(n);
        staging = c.take<float4>(n);
        rho = c.take<float>(n);
        press = c.take<float>(n);
        err = c.take<float>(n);
        keys = c.take<uint32_t>(n);
        ids = c.take<uint32_t>(n);
        nbr_count = c.take<uint32_t>(n);
        near_count = c.take<uint32_t>(n);
        scene_of = c.take<uint16_t>(n);
        nbr = c.take<uint32_t>(n * kListCapWide);
        near = c.take<uint32_t>(n * kNearCap);
        cells = c.take<uint2>(nb);
        bucket_fast = c.take<unsigned char>(nb);
        const size_t tbytes = align256(ns * sizeof(DevParams)) + align256(ns * sizeof(Control)) +
                              align256((ns + 1) * 4) + align256(sizeof(Control));
        if (tables.ensure(tbytes) != cudaSuccess) return report_error(PCISPH_ERR_OOM, "device allocation of the scene tables failed");
        Carver t{static_cast<unsigned char*>(tables.p)};
        d_table = t.take<DevParams>(ns);
        d_ctls = t.take<Control>(ns);
        d_offsets = t.take<uint32_t>(ns + 1);
        d_batch = t.take<Control>(1);
        BTRY(cudaMemset(tables.p, 0, tbytes));
        const size_t sbytes = RadixSorter::scratch_bytes(n, sorter.digit_bits());
        if (sort_block.ensure(sbytes) != cudaSuccess) return report_error(PCISPH_ERR_OOM, "device allocation of the sort scratch failed");
        sorter.set_scratch(sort_block.p, sort_block.cap);
        BTRY(cudaMallocHost(&h_ctls, ns * sizeof(Control)));
        return PCISPH_OK;
    }

    SceneTable scene_table() const {
        return SceneTable{d_table, d_ctls, scene_of, n_particles, (uint32_t)scenes.size()};
    }
    ListBuffers list_buffers() const {
        return ListBuffers{pos, vel, pr4, normal, f_other, f_press, pred, pf4, state_pos, state_vel, rho, press, err,
                           cells, cells, nullptr, nullptr, nbr, nbr_count, near, near_count, bucket_fast,
                           n_particles, /*out_index*/ nullptr, /*disp_max*/ nullptr, /*state_skin*/ nullptr};
    }

    uint32_t pool_end() const { return scenes.empty() ? 0u : scenes.back().offset + scenes.back().count; }
    uint32_t live_scenes() const {
        uint32_t n = 0;
        for (const SceneSlot& sl : scenes) n += sl.removed ? 0u : 1u;
        return n;
    }
    uint32_t live_particles() const {
        uint32_t n = 0;
        for (const SceneSlot& sl : scenes) n += sl.removed ? 0u : sl.count;
        return n;
    }

    // Drops the removed scenes: the later scenes move down (through the sorted-order arrays, which are free
    // between steps) and their control records with them. Then the scene tables are rebuilt.
    int compact() {
        cudaStream_t st = stream();
        size_t first = scenes.size();
        for (size_t k = 0; k < scenes.size(); ++k)
            if (scenes[k].removed) {
                first = k;
                break;
            }
        if (first < scenes.size()) {
            std::vector<SceneSlot> kept(scenes.begin(), scenes.begin() + first);
            std::vector<size_t> ctl_src;
            const uint32_t from = scenes[first].offset;
            uint32_t off = from;
            for (size_t k = first; k < scenes.size(); ++k) {
                const SceneSlot& sl = scenes[k];
                if (sl.removed) continue;
                BTRY(cudaMemcpyAsync(pos + off, state_pos + sl.offset, (size_t)sl.count * 16, cudaMemcpyDeviceToDevice, st));
                BTRY(cudaMemcpyAsync(vel + off, state_vel + sl.offset, (size_t)sl.count * 16, cudaMemcpyDeviceToDevice, st));
                ctl_src.push_back(k);
                kept.push_back(sl);
                off += sl.count;
            }
            if (off > from) {
                BTRY(cudaMemcpyAsync(state_pos + from, pos + from, (size_t)(off - from) * 16, cudaMemcpyDeviceToDevice, st));
                BTRY(cudaMemcpyAsync(state_vel + from, vel + from, (size_t)(off - from) * 16, cudaMemcpyDeviceToDevice, st));
            }
            if (!ctl_src.empty()) {  // per-scene statistics move with their scenes
                BTRY(cudaMemcpyAsync(h_ctls, d_ctls, scenes.size() * sizeof(Control), cudaMemcpyDeviceToHost, st));
                BTRY(cudaStreamSynchronize(st));
                for (size_t j = 0; j < ctl_src.size(); ++j) h_ctls[first + j] = h_ctls[ctl_src[j]];  // src >= dst
                BTRY(cudaMemcpyAsync(d_ctls + first, h_ctls + first, ctl_src.size() * sizeof(Control),
                                     cudaMemcpyHostToDevice, st));
            }
            scenes.swap(kept);
        }
        return rebuild();
    }

    // Scene tables after a change of composition (scenes packed from offset 0): bucket ranges, parameters,
    // offsets, particle -> scene.
    int rebuild() {
        std::vector<DevParams> table(scenes.size());
        std::vector<uint32_t> offsets(scenes.size() + 1);
        uint32_t base = 0, off = 0;
        max_iters = 1;
        for (size_t k = 0; k < scenes.size(); ++k) {
            SceneSlot& s = scenes[k];
            s.offset = off;
            s.bucket_base = base;
            const pcisph_scene_desc& d = s.desc;
            make_devparams(s.params, d.min_iterations, d.max_iterations, d.walls, d.box_lo, d.box_hi, d.restitution,
                           d.density_variation_threshold, adaptive_skin ? skin_level_value(0) : list_skin, base,
                           &table[k], kListCapWide, adaptive_skin ? 1 : 0);
            offsets[k] = off;
            off += s.count;
            base += s.params.bucket_count;
            max_iters = std::max(max_iters, d.max_iterations);
        }
        offsets[scenes.size()] = off;
        n_particles = off;
        n_buckets = base;
        cudaStream_t st = stream();
        if (!scenes.empty()) {
            BTRY(cudaMemcpyAsync(d_table, table.data(), table.size() * sizeof(DevParams), cudaMemcpyHostToDevice, st));
            BTRY(cudaMemcpyAsync(d_offsets, offsets.data(), offsets.size() * 4, cudaMemcpyHostToDevice, st));
            launch_scene_of(d_offsets, (uint32_t)scenes.size(), n_particles, scene_of, st);
            ++host_launches;
            BTRY(cudaGetLastError());
        }
        BTRY(cudaStreamSynchronize(st));  // the host vectors above go out of scope
        graph_valid = false;
        dirty = false;
        return PCISPH_OK;
    }

    int record_prefix(cudaStream_t s) {
        const SceneTable t = scene_table();
        int nl = 0;
        launch_batch_begin(d_table, d_ctls, t.n_scenes, d_batch, s);
        ++nl;
        if (cudaMemsetAsync(cells, 0, (size_t)n_buckets * 8, s) != cudaSuccess) return -1;
        if (cudaMemsetAsync(bucket_fast, 0, n_buckets, s) != cudaSuccess) return -1;
        timed("hash", s, [&] { launch_hash_scenes(t, state_pos, keys, s); });
        ++nl;
        uint32_t *sk = nullptr, *sv = nullptr;
        cudaError_t se = cudaSuccess;
        timed("radix_sort", s, [&] { se = sorter.sort(keys, ids, n_particles, key_bits(n_buckets), true, s, &sk, &sv); });
        if (se != cudaSuccess) return -1;
        nl += sorter.last_launches();
        sorted_keys = sk;
        sorted_ids = sv;
        DevParams R{};
        R.bucket_count = n_buckets;
        timed("reorder", s, [&] {
            launch_reorder(sk, sv, state_pos, state_vel, n_particles, pos, vel, cells, nullptr, nullptr, R, d_batch, s);
        });
        const ListBuffers b = list_buffers();
        timed("density", s, [&] { launch_density_scenes(t, b, s); });
        timed("normal", s, [&] { launch_normal_scenes(t, b, s); });
        timed("force", s, [&] { launch_force_scenes(t, b, s); });
        nl += 4;
        return cudaGetLastError() == cudaSuccess ? nl : -1;
    }

    // Capture the step into a new graph. An existing executable graph is updated in place when only kernel
    // parameters changed (a change of composition: particle and scene counts, table contents) -- far
    // cheaper than instantiating again; otherwise it is replaced.
    int capture(cudaGraph_t* out) {
        cudaStream_t s = capture_stream;
        cudaGraph_t graph = nullptr;
        BTRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        const int nl = record_prefix(s);
        if (loop_mode == 2) {  // the corrective loop as one cooperative kernel after the prefix
            const cudaError_t le = nl < 0 ? cudaSuccess
                                          : launch_corrective_loop_scenes(scene_table(), list_buffers(), d_batch,
                                                                          max_iters, s);
            const cudaError_t ee = cudaStreamEndCapture(s, &graph);
            if (nl < 0 || le != cudaSuccess || ee != cudaSuccess) {
                if (graph) cudaGraphDestroy(graph);
                return report_error(PCISPH_ERR_CUDA, std::string("graph capture of the persistent batch step failed: ") +
                                                         cudaGetErrorString(le != cudaSuccess ? le : ee));
            }
            prefix_launches = nl + 1;
            iter_launches = 0;
            *out = graph;
            return PCISPH_OK;
        }
        cudaStreamCaptureStatus st;
        const cudaGraphNode_t* deps = nullptr;
        size_t ndeps = 0;
        cudaError_t e = cudaStreamGetCaptureInfo(s, &st, nullptr, nullptr, &deps, nullptr, &ndeps);
        std::vector<cudaGraphNode_t> leaves(deps, deps + (e == cudaSuccess ? ndeps : 0));
        cudaError_t e2 = cudaStreamEndCapture(s, &graph);
        if (nl < 0 || e != cudaSuccess || e2 != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            return report_error(PCISPH_ERR_CUDA, std::string("graph capture of the batch step failed: ") +
                                                     cudaGetErrorString(e != cudaSuccess ? e : e2));
        }
        prefix_launches = nl;
        iter_launches = 3;
        cudaGraphConditionalHandle handle;
        cudaGraphNodeParams cp{};
        cudaGraphNode_t loop_node;
        e = cudaGraphConditionalHandleCreate(&handle, graph, 1, cudaGraphCondAssignDefault);
        if (e == cudaSuccess) {
            cp.type = cudaGraphNodeTypeConditional;
            cp.conditional.handle = handle;
            cp.conditional.type = cudaGraphCondTypeWhile;
            cp.conditional.size = 1;
            e = cudaGraphAddNode(&loop_node, graph, leaves.data(), nullptr, leaves.size(), &cp);
        }
        if (e == cudaSuccess)
            e = cudaStreamBeginCaptureToGraph(s, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                              cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) {
            cudaGraphDestroy(graph);
            return report_error(PCISPH_ERR_CUDA, std::string("graph loop node: ") + cudaGetErrorString(e));
        }
        const SceneTable t = scene_table();
        const ListBuffers b = list_buffers();
        launch_pressure_scenes(t, b, s);
        launch_batch_decide(t, d_batch, max_iters, handle, true, s);
        launch_pressure_force_scenes(t, b, s);
        cudaGraph_t body = nullptr;
        e = cudaStreamEndCapture(s, &body);
        if (e != cudaSuccess) {
            cudaGraphDestroy(graph);
            return report_error(PCISPH_ERR_CUDA, std::string("graph loop body: ") + cudaGetErrorString(e));
        }
        *out = graph;
        return PCISPH_OK;
    }

    int build_graph() {
        cudaGraph_t graph = nullptr;
        int rc = capture(&graph);
        if (rc) return rc;
        if (graph_exec) {
            cudaGraphExecUpdateResultInfo info{};
            if (cudaGraphExecUpdate(graph_exec, graph, &info) == cudaSuccess) {
                cudaGraphDestroy(graph);
                graph_valid = true;
                ++graph_updates;
                return PCISPH_OK;
            }
            (void)cudaGetLastError();  // the update was refused: instantiate instead
            cudaGraphExecDestroy(graph_exec);
            graph_exec = nullptr;
        }
        const cudaError_t e = cudaGraphInstantiate(&graph_exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return report_error(PCISPH_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
        ++graph_instantiations;
        graph_valid = true;
        return PCISPH_OK;
    }

    int step(uint32_t steps) {
        if (dirty) {
            int rc = compact();
            if (rc) return rc;
        }
        if (scenes.empty()) return PCISPH_OK;
        if (!graph_valid) {
            int rc = build_graph();
            if (rc) return rc;
        }
        if (profiling) {
            for (uint32_t k = 0; k < steps; ++k) {
                int rc = step_profiled();
                if (rc) return rc;
            }
            return PCISPH_OK;
        }
        for (uint32_t k = 0; k < steps; ++k) {
            BTRY(cudaGraphLaunch(graph_exec, stream()));
            host_launches += prefix_launches;
        }
        return PCISPH_OK;
    }

    // One step launched from the host with every launch timed: the same kernels as the graph, and the
    // loop's continuation read back after each iteration (as the graph's WHILE node reads it on the device).
    int step_profiled() {
        cudaStream_t s = stream();
        const int nl = record_prefix(s);
        if (nl < 0) return report_error(PCISPH_ERR_CUDA, std::string("batch step: ") + cudaGetErrorString(cudaGetLastError()));
        host_launches += nl;
        const SceneTable t = scene_table();
        const ListBuffers b = list_buffers();
        iter_launches = loop_mode == 2 ? 0 : 3;  // counted on the device per iteration (total_iters)
        if (loop_mode == 2) {
            cudaError_t le = cudaSuccess;
            timed("corrective_loop", s, [&] { le = launch_corrective_loop_scenes(t, b, d_batch, max_iters, s); });
            if (le != cudaSuccess) return report_error(PCISPH_ERR_CUDA, std::string("persistent loop: ") + cudaGetErrorString(le));
            ++host_launches;
        } else {
            for (int it = 0; it < max_iters; ++it) {
                timed("pressure", s, [&] { launch_pressure_scenes(t, b, s); });
                timed("decide", s, [&] { launch_batch_decide(t, d_batch, max_iters, 0, false, s); });
                timed("pressure_force", s, [&] { launch_pressure_force_scenes(t, b, s); });
                unsigned running = 0;
                BTRY(cudaMemcpyAsync(&running, &d_batch->any_running, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
                BTRY(cudaStreamSynchronize(s));
                if (!running) break;
            }
        }
        BTRY(cudaGetLastError());
        timer.collect(s);
        return PCISPH_OK;
    }

    int find(int32_t id) const {
        for (size_t k = 0; k < scenes.size(); ++k)
            if (scenes[k].id == id && !scenes[k].removed) return (int)k;
        return -1;
    }

    int copy_in(float4* dst, const float* src, uint32_t n, int layout, int memory) {
        if (!n) return PCISPH_OK;
        cudaStream_t s = stream();
        const cudaMemcpyKind kind = memory == PCISPH_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
        if (layout == PCISPH_LAYOUT_FLOAT4) {
            BTRY(cudaMemcpyAsync(dst, src, (size_t)n * 16, kind, s));
        } else {
            const float* d = src;
            if (memory == PCISPH_MEM_HOST) {
                BTRY(cudaMemcpyAsync(staging, src, (size_t)n * 12, kind, s));
                d = reinterpret_cast<const float*>(staging);
            }
            launch_pack3_to4(d, dst, n, s);
            ++host_launches;
            BTRY(cudaGetLastError());
            if (memory == PCISPH_MEM_HOST) BTRY(cudaStreamSynchronize(s));  // staging is reused
        }
        return PCISPH_OK;
    }
};

extern "C" {

int pcisph_batch_memory_model(uint64_t* bytes_per_particle, uint64_t* bytes_per_scene) {
    if (bytes_per_particle) *bytes_per_particle = kParticleBytes + kBucketBytesPerParticle + 12;  // + sort scratch
    if (bytes_per_scene) *bytes_per_scene = sizeof(DevParams) + sizeof(Control) + 4 + 64 * 9;
    return PCISPH_OK;
}

int pcisph_batch_create(int device, void* stream, uint32_t max_particles, uint32_t max_scenes, pcisph_batch** out) {
    if (!out) return report_error(PCISPH_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    if (max_particles == 0 || max_particles >= (1u << 31) || max_scenes == 0 || max_scenes > 65535)
        return report_error(PCISPH_ERR_INVALID_ARG, "max_particles must be in 1..2^31-1 and max_scenes in 1..65535");
    int ndev = 0;
    BTRY(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return report_error(PCISPH_ERR_INVALID_ARG, "no CUDA device " + std::to_string(device));
    DeviceGuard g(device);
    BTRY(cudaFree(nullptr));
    BTRY(radix_configure_kernels());
    pcisph_batch* b = new pcisph_batch();
    b->device = device;
    b->max_particles = max_particles;
    b->max_scenes = max_scenes;
    b->max_buckets = max_particles / 2 + 64u * max_scenes;
    cudaError_t e = cudaStreamCreateWithFlags(&b->capture_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete b;
        return report_error(PCISPH_ERR_CUDA, std::string("stream creation: ") + cudaGetErrorString(e));
    }
    b->user_stream = stream ? static_cast<cudaStream_t>(stream) : b->own_stream;
    int rc = b->allocate();
    if (rc) {
        delete b;
        return rc;
    }
    *out = b;
    return PCISPH_OK;
}

void pcisph_batch_destroy(pcisph_batch* b) { delete b; }

int pcisph_batch_add_scene(pcisph_batch* b, const pcisph_scene_desc* d, const float* pos, const float* vel,
                           int layout, int memory, int32_t* scene_id) {
    if (!b || !d || !scene_id) return report_error(PCISPH_ERR_INVALID_ARG, "NULL argument");
    if (d->fluid_count == 0 || !pos) return report_error(PCISPH_ERR_INVALID_ARG, "a scene needs particles");
    if (layout != PCISPH_LAYOUT_PACKED3 && layout != PCISPH_LAYOUT_FLOAT4)
        return report_error(PCISPH_ERR_INVALID_ARG, "positions take PACKED3 or FLOAT4");
    if (d->min_iterations < 1 || d->max_iterations < 1 || d->max_iterations > 10000)
        return report_error(PCISPH_ERR_INVALID_ARG, "iteration limits must be in 1..10000");
    if (b->live_scenes() >= b->max_scenes) return report_error(PCISPH_ERR_OOM, "batch is full (max_scenes)");
    if ((uint64_t)b->live_particles() + d->fluid_count > b->max_particles)
        return report_error(PCISPH_ERR_OOM, "batch is full (max_particles)");
    DeviceGuard g(b->device);
    if (b->scenes.size() >= b->max_scenes || (uint64_t)b->pool_end() + d->fluid_count > b->max_particles) {
        int rc = b->compact();  // make room: drop the removed scenes now
        if (rc) return rc;
    }
    SceneSlot s{};
    s.id = b->next_id++;
    s.desc = *d;
    s.count = d->fluid_count;
    pcisph_derive_params(d->particle_radius, d->rest_density, d->fluid_count, 0, d->delta_t, d->gravity, d->viscosity,
                         d->surface_tension, &s.params);
    uint64_t buckets = s.params.bucket_count;
    for (const SceneSlot& sl : b->scenes) buckets += sl.removed ? 0u : sl.params.bucket_count;
    if (buckets > b->max_buckets) return report_error(PCISPH_ERR_OOM, "batch is full (buckets)");
    const uint32_t off = b->pool_end();
    s.offset = off;
    int rc = b->copy_in(b->state_pos + off, pos, s.count, layout, memory);
    if (!rc && vel) rc = b->copy_in(b->state_vel + off, vel, s.count, layout, memory);
    else if (!rc) BTRY(cudaMemsetAsync(b->state_vel + off, 0, (size_t)s.count * 16, b->stream()));
    if (rc) return rc;
    const size_t k = b->scenes.size();
    BTRY(cudaMemsetAsync(b->d_ctls + k, 0, sizeof(Control), b->stream()));
    b->scenes.push_back(s);
    b->dirty = true;  // tables and graph are rebuilt by the next step
    *scene_id = s.id;
    return PCISPH_OK;
}

int pcisph_batch_set_state(pcisph_batch* b, int32_t id, const float* pos, const float* vel, uint32_t count,
                           int layout, int memory) {
    if (!b || !pos) return report_error(PCISPH_ERR_INVALID_ARG, "NULL argument");
    if (layout != PCISPH_LAYOUT_PACKED3 && layout != PCISPH_LAYOUT_FLOAT4)
        return report_error(PCISPH_ERR_INVALID_ARG, "positions take PACKED3 or FLOAT4");
    const int k = b->find(id);
    if (k < 0) return report_error(PCISPH_ERR_INVALID_ARG, "unknown scene id " + std::to_string(id));
    const SceneSlot& s = b->scenes[k];
    if (count != s.count)
        return report_error(PCISPH_ERR_INCONSISTENT, "scene " + std::to_string(id) + " has " + std::to_string(s.count) +
                                                         " particles, not " + std::to_string(count));
    DeviceGuard g(b->device);
    int rc = b->copy_in(b->state_pos + s.offset, pos, s.count, layout, memory);
    if (!rc && vel) rc = b->copy_in(b->state_vel + s.offset, vel, s.count, layout, memory);
    else if (!rc) BTRY(cudaMemsetAsync(b->state_vel + s.offset, 0, (size_t)s.count * 16, b->stream()));
    return rc;
}

int pcisph_batch_remove_scene(pcisph_batch* b, int32_t id) {
    if (!b) return report_error(PCISPH_ERR_INVALID_ARG, "batch is NULL");
    const int k = b->find(id);
    if (k < 0) return report_error(PCISPH_ERR_INVALID_ARG, "unknown scene id " + std::to_string(id));
    b->scenes[k].removed = true;  // compacted with every other removal at the next step
    b->dirty = true;
    return PCISPH_OK;
}

int pcisph_batch_autotune(pcisph_batch* b, uint32_t steps, pcisph_batch_tune_result* out) {
    if (!b || !out) return report_error(PCISPH_ERR_INVALID_ARG, "NULL argument");
    if (steps == 0 || steps > 1000) return report_error(PCISPH_ERR_INVALID_ARG, "steps must be in 1..1000");
    DeviceGuard g(b->device);
    if (b->dirty) {
        int rc = b->compact();
        if (rc) return rc;
    }
    const uint32_t n = b->n_particles, ns = (uint32_t)b->scenes.size();
    if (n == 0) return report_error(PCISPH_ERR_NOT_READY, "no scenes to tune on");
    cudaStream_t s = b->stream();
    DeviceBlock saved;
    if (saved.ensure((size_t)n * 32 + (size_t)ns * sizeof(Control) + sizeof(Control)) != cudaSuccess)
        return report_error(PCISPH_ERR_OOM, "device allocation for autotuning failed");
    float4* sp = static_cast<float4*>(saved.p);
    Control* sc = reinterpret_cast<Control*>(sp + 2 * (size_t)n);
    BTRY(cudaMemcpyAsync(sp, b->state_pos, (size_t)n * 16, cudaMemcpyDeviceToDevice, s));
    BTRY(cudaMemcpyAsync(sp + n, b->state_vel, (size_t)n * 16, cudaMemcpyDeviceToDevice, s));
    BTRY(cudaMemcpyAsync(sc, b->d_ctls, (size_t)ns * sizeof(Control), cudaMemcpyDeviceToDevice, s));
    BTRY(cudaMemcpyAsync(sc + ns, b->d_batch, sizeof(Control), cudaMemcpyDeviceToDevice, s));
    const uint64_t launches0 = b->host_launches;
    const float entry_skin = b->adaptive_skin ? PCISPH_LIST_SKIN_ADAPTIVE : b->list_skin;
    const int entry_mode = b->loop_mode, entry_bits = b->sorter.digit_bits();
    auto restore = [&]() -> int {
        BTRY(cudaMemcpyAsync(b->state_pos, sp, (size_t)n * 16, cudaMemcpyDeviceToDevice, s));
        BTRY(cudaMemcpyAsync(b->state_vel, sp + n, (size_t)n * 16, cudaMemcpyDeviceToDevice, s));
        BTRY(cudaMemcpyAsync(b->d_ctls, sc, (size_t)ns * sizeof(Control), cudaMemcpyDeviceToDevice, s));
        BTRY(cudaMemcpyAsync(b->d_batch, sc + ns, sizeof(Control), cudaMemcpyDeviceToDevice, s));
        BTRY(cudaStreamSynchronize(s));
        return PCISPH_OK;
    };
    auto apply = [&](float skin, int mode, int bits) -> int {
        b->adaptive_skin = skin == PCISPH_LIST_SKIN_ADAPTIVE;
        if (!b->adaptive_skin) b->list_skin = skin;
        b->loop_mode = mode;
        b->sorter.set_digit_bits(bits);
        b->sort_block.release();
        const size_t sbytes = RadixSorter::scratch_bytes(b->max_particles, bits);
        if (b->sort_block.ensure(sbytes) != cudaSuccess)
            return report_error(PCISPH_ERR_OOM, "device allocation of the sort scratch failed");
        b->sorter.set_scratch(b->sort_block.p, b->sort_block.cap);
        b->graph_valid = false;
        return b->rebuild();  // scene tables with the new skin
    };
    cudaEvent_t e0, e1;
    BTRY(cudaEventCreate(&e0));
    BTRY(cudaEventCreate(&e1));
    auto time_it = [&](float* ms) -> int {
        int r = restore();
        if (!r) r = b->step(1);  // warm-up: builds the graph
        if (!r) r = restore();
        if (r) return r;
        BTRY(cudaEventRecord(e0, s));
        r = b->step(steps);
        BTRY(cudaEventRecord(e1, s));
        BTRY(cudaEventSynchronize(e1));
        if (r) return r;
        BTRY(cudaEventElapsedTime(ms, e0, e1));
        *ms /= (float)steps;
        return PCISPH_OK;
    };
    float before = 0.f;
    int rc = apply(entry_skin, entry_mode, entry_bits);
    if (!rc) rc = time_it(&before);
    float best_ms = before, best_skin = entry_skin;
    int best_mode = entry_mode, best_bits = entry_bits, cands = 1;
    const float skins[] = {PCISPH_LIST_SKIN_ADAPTIVE, 0.25f, 0.35f, 0.5f};
    const int modes[] = {0, 2};
    const int bits[] = {8, 10, 6};
    for (float sk : skins)
        for (int md : modes)
            for (int bt : bits) {
                if (rc) break;
                if (sk == entry_skin && md == entry_mode && bt == entry_bits) continue;
                float ms = 0.f;
                rc = apply(sk, md, bt);
                if (!rc) rc = time_it(&ms);
                ++cands;
                if (!rc && ms < best_ms) {
                    best_ms = ms;
                    best_skin = sk;
                    best_mode = md;
                    best_bits = bt;
                }
            }
    if (!rc) rc = apply(best_skin, best_mode, best_bits);
    const int rc2 = restore();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    saved.release();
    b->host_launches = launches0;
    if (rc) return rc;
    if (rc2) return rc2;
    out->list_skin = best_skin;
    out->loop_mode = best_mode;
    out->digit_bits = best_bits;
    out->ms_per_step = best_ms;
    out->ms_per_step_before = before;
    out->candidates = cands;
    return PCISPH_OK;
}

int pcisph_batch_set_loop_mode(pcisph_batch* b, int loop_mode) {
    if (!b) return report_error(PCISPH_ERR_INVALID_ARG, "batch is NULL");
    if (loop_mode != 0 && loop_mode != 2) return report_error(PCISPH_ERR_INVALID_ARG, "batch loop_mode must be 0 or 2");
    if (loop_mode != b->loop_mode) {
        b->loop_mode = loop_mode;
        b->graph_valid = false;
    }
    return PCISPH_OK;
}

int pcisph_batch_set_list_skin(pcisph_batch* b, float skin) {
    if (!b) return report_error(PCISPH_ERR_INVALID_ARG, "batch is NULL");
    if (!(skin == PCISPH_LIST_SKIN_ADAPTIVE || (skin >= 0.f && skin <= 2.f)))
        return report_error(PCISPH_ERR_INVALID_ARG, "list_skin must be in [0, 2], or PCISPH_LIST_SKIN_ADAPTIVE");
    const bool adaptive = skin == PCISPH_LIST_SKIN_ADAPTIVE;
    if (adaptive == b->adaptive_skin && (adaptive || skin == b->list_skin)) return PCISPH_OK;
    DeviceGuard g(b->device);
    b->adaptive_skin = adaptive;
    if (!adaptive) b->list_skin = skin;
    return b->rebuild();  // scene tables with the new list radius
}

int pcisph_batch_info(const pcisph_batch* b, uint32_t* scenes, uint32_t* particles, uint32_t* free_particles) {
    if (!b) return report_error(PCISPH_ERR_INVALID_ARG, "batch is NULL");
    const uint32_t live = b->live_particles();
    if (scenes) *scenes = b->live_scenes();
    if (particles) *particles = live;
    if (free_particles) *free_particles = b->max_particles - live;
    return PCISPH_OK;
}

int pcisph_batch_step(pcisph_batch* b, uint32_t steps) {
    if (!b) return report_error(PCISPH_ERR_INVALID_ARG, "batch is NULL");
    DeviceGuard g(b->device);
    return b->step(steps);
}

int pcisph_batch_sync(pcisph_batch* b) {
    if (!b) return report_error(PCISPH_ERR_INVALID_ARG, "batch is NULL");
    DeviceGuard g(b->device);
    BTRY(cudaStreamSynchronize(b->stream()));
    return PCISPH_OK;
}

int pcisph_batch_sync_for(pcisph_batch* b, int64_t timeout_ms) {
    if (!b) return report_error(PCISPH_ERR_INVALID_ARG, "batch is NULL");
    if (timeout_ms < 0) return report_error(PCISPH_ERR_INVALID_ARG, "timeout_ms must be >= 0");
    DeviceGuard g(b->device);
    bool done = false;
    BTRY(host::wait_stream_for(b->stream(), timeout_ms, &done));
    if (!done)
        return report_error(PCISPH_ERR_TIMEOUT, "queued steps still running after " + std::to_string(timeout_ms) + " ms");
    return PCISPH_OK;
}

int pcisph_batch_scene_stats(pcisph_batch* b, int32_t id, pcisph_step_stats* out) {
    if (!b || !out) return report_error(PCISPH_ERR_INVALID_ARG, "NULL argument");
    const int k = b->find(id);
    if (k < 0) return report_error(PCISPH_ERR_INVALID_ARG, "unknown scene id " + std::to_string(id));
    DeviceGuard g(b->device);
    BTRY(cudaStreamSynchronize(b->stream()));
    Control c{}, all{};
    BTRY(cudaMemcpy(&c, b->d_ctls + k, sizeof(Control), cudaMemcpyDeviceToHost));
    BTRY(cudaMemcpy(&all, b->d_batch, sizeof(Control), cudaMemcpyDeviceToHost));
    c.status |= all.status & 4u;  // a broken sort concerns every scene of the step
    c.status_all |= c.status;
    out->iterations = c.iterations_last;
    out->max_density_error = c.max_err_last;
    out->status = c.status;
    out->status_all = c.status_all;
    out->steps = c.steps;
    out->total_iterations = c.total_iters;
    out->list_fallbacks = c.list_fallbacks;
    out->fast_particles = c.fast_particles;
    out->list_skin = b->adaptive_skin ? skin_level_value((int)c.skin_level) : b->list_skin;
    out->max_density_error_max = host::float_from_bits(c.max_err_max_bits);
    out->unconverged_steps = c.unconverged_steps;
    return PCISPH_OK;
}

int pcisph_batch_get_field(pcisph_batch* b, int32_t id, int field, void* dst, size_t dst_bytes, int layout,
                           int memory) {
    if (!b) return report_error(PCISPH_ERR_INVALID_ARG, "batch is NULL");
    const int k = b->find(id);
    if (k < 0) return report_error(PCISPH_ERR_INVALID_ARG, "unknown scene id " + std::to_string(id));
    const SceneSlot& s = b->scenes[k];
    const void* src = nullptr;
    bool vec = true;
    switch (field) {
        case PCISPH_FIELD_POSITION: src = b->state_pos + s.offset; break;
        case PCISPH_FIELD_VELOCITY: src = b->state_vel + s.offset; break;
        case PCISPH_FIELD_NORMAL: src = b->normal + s.offset; break;
        case PCISPH_FIELD_PREDICTED_POSITION: src = b->pred + s.offset; break;
        case PCISPH_FIELD_OTHER_FORCE: src = b->f_other + s.offset; break;
        case PCISPH_FIELD_PRESSURE_FORCE: src = b->f_press + s.offset; break;
        case PCISPH_FIELD_SORTED_POSITION: src = b->pos + s.offset; break;
        case PCISPH_FIELD_DENSITY: src = b->rho + s.offset; vec = false; break;
        case PCISPH_FIELD_PRESSURE: src = b->press + s.offset; vec = false; break;
        case PCISPH_FIELD_DENSITY_VARIATION: src = b->err + s.offset; vec = false; break;
        default: return report_error(PCISPH_ERR_INVALID_ARG, "field not available for batched scenes");
    }
    if (vec && layout == PCISPH_LAYOUT_SCALAR) return report_error(PCISPH_ERR_INVALID_ARG, "vector field: use PACKED3 or FLOAT4");
    if (!vec && layout != PCISPH_LAYOUT_SCALAR) return report_error(PCISPH_ERR_INVALID_ARG, "scalar field: use SCALAR");
    const size_t need = (size_t)s.count * (layout == PCISPH_LAYOUT_PACKED3 ? 12 : layout == PCISPH_LAYOUT_FLOAT4 ? 16 : 4);
    if (!dst || dst_bytes < need) return report_error(PCISPH_ERR_INVALID_ARG, "destination too small");
    DeviceGuard g(b->device);
    cudaStream_t st = b->stream();
    const cudaMemcpyKind kind = memory == PCISPH_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    if (layout == PCISPH_LAYOUT_PACKED3) {
        float* o = memory == PCISPH_MEM_HOST ? reinterpret_cast<float*>(b->staging) : static_cast<float*>(dst);
        launch_unpack4_to3(static_cast<const float4*>(src), o, s.count, st);
        ++b->host_launches;
        BTRY(cudaGetLastError());
        if (memory == PCISPH_MEM_HOST) BTRY(cudaMemcpyAsync(dst, o, need, kind, st));
    } else {
        BTRY(cudaMemcpyAsync(dst, src, need, kind, st));
    }
    if (memory == PCISPH_MEM_HOST) BTRY(cudaStreamSynchronize(st));
    return PCISPH_OK;
}

int pcisph_batch_graph_stats(const pcisph_batch* b, uint64_t* instantiations, uint64_t* updates) {
    if (!b) return report_error(PCISPH_ERR_INVALID_ARG, "batch is NULL");
    if (instantiations) *instantiations = b->graph_instantiations;
    if (updates) *updates = b->graph_updates;
    return PCISPH_OK;
}

int pcisph_batch_profile_enable(pcisph_batch* b, int enable) {
    if (!b) return report_error(PCISPH_ERR_INVALID_ARG, "batch is NULL");
    b->profiling = enable != 0;
    if (enable) b->timer.clear();
    return PCISPH_OK;
}

int pcisph_batch_profile_read(pcisph_batch* b, pcisph_kernel_time* out, int max_entries, int* n_entries) {
    if (!b) return report_error(PCISPH_ERR_INVALID_ARG, "batch is NULL");
    DeviceGuard g(b->device);
    b->timer.collect(b->stream());
    const int n = b->timer.read(out, max_entries);
    if (n_entries) *n_entries = n;
    return PCISPH_OK;
}

uint64_t pcisph_batch_kernel_launches(const pcisph_batch* b) {
    if (!b) return 0;
    DeviceGuard g(b->device);
    cudaStreamSynchronize(b->user_stream);
    Control c{};
    cudaMemcpy(&c, b->d_batch, sizeof(Control), cudaMemcpyDeviceToHost);
    return b->host_launches + c.total_iters * (uint64_t)b->iter_launches;
}

}  // extern "C"
