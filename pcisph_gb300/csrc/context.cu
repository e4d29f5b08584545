// context.cu -- host driver of the PCISPH step and its C ABI (include/pcisph_gpu.h).
//
// pcisph_ctx plays the role of sim::Fluid (PCISPH/src/sim/Fluid.h:13-102):
// parameter setters with lazy derivation (Fluid.cpp:333-443), a consistency
// check (Fluid.cpp:90-106) and update() (Fluid.cpp:108-327). What differs is how
// the step is scheduled on the GPU:
//   - device memory lives in per-context arenas sized by the particle counts;
//   - the fluid sort is the in-house radix sort (radix_sort.cu), keys bounded
//     by bucket_count;
//   - the corrective loop is decided on the device; by default the whole step is
//     one CUDA graph whose loop is a conditional WHILE node, so a step costs one
//     graph launch and no host synchronisation (loop_mode 0). loop_mode 2 puts the
//     whole loop in one persistent cooperative kernel (list_kernels.cu) instead of
//     the WHILE node. loop_mode 1 reads the decision back every iteration, as the
//     reference does (Fluid.cpp:300-306).
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstddef>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/pcisph_gpu.h"
#include "common.cuh"
#include "radix_sort.cuh"
#include "host_util.h"
#include "list_kernels.cuh"
#include "spatial_order.cuh"
#include "step_kernels.cuh"
#include "sweep.cuh"

using namespace pcisph;
using namespace pcisph::host;

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

#define CUDA_TRY(call)                                                                                \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess) return fail(PCISPH_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

size_t fluid_arena_bytes(uint32_t n, uint32_t bk) {
    return 10 * align256((size_t)n * 16) + 3 * align256((size_t)n * 4) + 4 * align256((size_t)n * 4) +
           2 * align256((size_t)n * 4) + align256((size_t)bk * 8);
}
size_t boundary_arena_bytes(uint32_t n, uint32_t bk) {
    return 3 * align256((size_t)n * 16) + 5 * align256((size_t)n * 4) + align256((size_t)bk * 8);
}

}  // namespace

struct pcisph_ctx {
    int device = 0;
    cudaStream_t user_stream = nullptr;  // launches go here (may be the legacy stream)
    cudaStream_t capture_stream = nullptr;
    pcisph_sim_params params{};
    pcisph_options opts{};
    float threshold = 0.01f;
    bool params_changed = true;
    bool boundary_updated = true;
    uint32_t fluid_loaded = 0xFFFFFFFFu, boundary_loaded = 0xFFFFFFFFu;
    uint32_t fluid_cap_n = 0, fluid_cap_bk = 0, boundary_cap_n = 0, boundary_cap_bk = 0;

    DeviceBlock fluid_block, boundary_block, misc_block, sort_block, staging_block, list_block, order_block,
        bucket_sort_block;
    // the boundary zone (list sweeps, B > 0): cell bounds scratch, then one byte per cell of the boundary's
    // cell box widened by two; zone_map null when the box has more than kZoneMaxCells cells
    static constexpr uint64_t kZoneMaxCells = 1ull << 26;
    DeviceBlock zone_block;
    unsigned char* zone_map = nullptr;
    int zone_org[3] = {0, 0, 0};
    uint32_t zone_dim[3] = {0, 0, 0};
    // working order (variant 2 with spatial_order): bucket ranges in working order, bucket Morton codes,
    // the two index maps, scan scratch, and a transfer buffer for fields exported or imported in sorted order
    uint2* cells_w = nullptr;
    uint32_t *bucket_codes = nullptr, *bucket_ids = nullptr, *d_of_w = nullptr, *w_of_d = nullptr;
    uint32_t* range_scratch = nullptr;
    float4* xfer = nullptr;
    RadixSorter bucket_sorter;
    size_t order_n = 0, order_bk = 0;
    std::map<int, DeviceBlock> exports;  // sorted-order copies handed out by pcisph_field_device_ptr
    DeviceBlock render_block;            // depth buffer and image of pcisph_render_fluid
    StepBuffers b{};
    float4* b_pos_in = nullptr;
    uint32_t *f_keys = nullptr, *f_ids = nullptr, *b_keys = nullptr, *b_ids = nullptr;
    uint32_t *sorted_keys = nullptr, *sorted_ids = nullptr;
    Control* ctl = nullptr;
    Control* host_ctl = nullptr;  // pinned
    RadixSorter sorter;
    DevParams P{};
    SweepGrid sweep_grid{};
    size_t list_n = 0;
    size_t list_b_n = 0;  // boundary particles the list block holds lists for

    SweepArgs sweep_args() const {
        return SweepArgs{b.groups, &b.ctl->n_groups, sorted_keys, b.cells, b.b_cells, b.codes, b.b_codes};
    }
    bool warp_sweeps() const { return opts.kernel_variant == 0; }
    bool list_sweeps() const { return opts.kernel_variant == 2; }
    // spatial_order 1: on; 2 (default): on from 131,072 particles, where its cost (~100 us of sorting and
    // scanning per step) is below what it saves in the sweeps
    bool working_order() const {
        return list_sweeps() && (opts.spatial_order == 1 || (opts.spatial_order == 2 && params.fluid_count >= (1u << 17)));
    }
    // marks: the launch follows the partner-marking kernel of its round (the graph's and the host-driven
    // loop's pressure sweeps, and that kernel itself): the pressure sweep may read the stamps
    ListBuffers list_buffers(bool marks = false) const {
        const bool w = working_order();
        const bool m = P.mark_cap != 0;
        return ListBuffers{b.pos, b.vel, b.pr4, b.normal, b.f_other, b.f_press, b.pred, b.pf4, b.state_pos,
                           b.state_vel, b.rho, b.press, b.err, w ? cells_w : b.cells, b.b_cells, b.b_pos, b.bpf,
                           b.nbr, b.nbr_count, b.near, b.near_count, b.bucket_fast, P.fluid_count,
                           w ? d_of_w : nullptr, b.disp_max, b.state_skin, b.b_init, b.b_press, b.b_near, b.bnbr,
                           b.bnbr_count, b.bfl,
                           b.bfl_count, zone_map, {zone_org[0], zone_org[1], zone_org[2]},
                           {zone_dim[0], zone_dim[1], zone_dim[2]}, m ? b.fast_list : nullptr,
                           m && marks ? b.walk_stamp : nullptr};
    }
    // the partner-marking kernel runs after each prediction round of the graph and the host-driven loop
    bool partner_marks() const { return list_sweeps() && P.mark_cap != 0 && opts.loop_mode != 2; }

    // Working-order buffers for n particles and bk buckets; the index maps start as the identity.
    int ensure_order() {
        if (!working_order()) return PCISPH_OK;
        const size_t n = params.fluid_count, bk = params.bucket_count;
        if (order_block.p && order_n == n && order_bk == bk) return PCISPH_OK;
        CUDA_TRY(cudaStreamSynchronize(stream()));
        const size_t bytes = align256(bk * 8) + 2 * align256(bk * 4) + 2 * align256(n * 4) +
                             align256(working_ranges_scratch((uint32_t)bk) * 4) + align256(n * 16);
        if (order_block.ensure(bytes) != cudaSuccess)
            return fail(PCISPH_ERR_OOM, "device allocation of the working-order buffers failed");
        Carver c{static_cast<unsigned char*>(order_block.p)};
        cells_w = c.take<uint2>(bk);
        bucket_codes = c.take<uint32_t>(bk);
        bucket_ids = c.take<uint32_t>(bk);
        d_of_w = c.take<uint32_t>(n);
        w_of_d = c.take<uint32_t>(n);
        range_scratch = c.take<uint32_t>(working_ranges_scratch((uint32_t)bk));
        xfer = c.take<float4>(n);
        bucket_sorter.set_digit_bits(8);
        const size_t sbytes = RadixSorter::scratch_bytes(bk, 8);
        if (bucket_sort_block.ensure(sbytes) != cudaSuccess)
            return fail(PCISPH_ERR_OOM, "device allocation of the bucket-sort scratch failed");
        bucket_sorter.set_scratch(bucket_sort_block.p, bucket_sort_block.cap);
        launch_iota(d_of_w, (uint32_t)n, stream());
        launch_iota(w_of_d, (uint32_t)n, stream());
        host_launches += 2;
        CUDA_TRY(cudaGetLastError());
        order_n = n;
        order_bk = bk;
        graph_valid = false;
        order_age = kNoOrder;
        return PCISPH_OK;
    }

    // After the hash sort (sorted keys sk, ids sv): the reference's cell table, then the working order and
    // the particles gathered into it. Returns the launches issued, or -1.
    int record_working_order(const uint32_t* sk, const uint32_t* sv, cudaStream_t s) {
        const uint32_t N = params.fluid_count, BK = params.bucket_count;
        const bool reuse = reuse_order_now && bucket_order;
        if (!reuse && cudaMemsetAsync(bucket_codes, 0xFF, (size_t)BK * 4, s) != cudaSuccess) return -1;
        int nl = 0;
        timed("reorder", s, [&] { launch_bucket_codes(sk, sv, b.state_pos, N, P, b.cells, bucket_codes, b.ctl, s); });
        ++nl;
        if (!reuse) {
            uint32_t *ok = nullptr, *order = nullptr;
            cudaError_t e = cudaSuccess;
            timed("bucket_sort", s, [&] {
                e = bucket_sorter.sort(bucket_codes, bucket_ids, BK, 24, true, s, &ok, &order);
                nl += bucket_sorter.last_launches();
            });
            if (e != cudaSuccess) return -1;
            bucket_order = order;
        }
        const uint32_t* order = bucket_order;
        timed("working_ranges", s, [&] { launch_working_ranges(order, BK, b.cells, cells_w, range_scratch, N, s); });
        timed("permute", s, [&] {
            launch_permute(sk, sv, b.state_pos, b.state_vel, N, BK, b.cells, cells_w, b.pos, b.vel, d_of_w, w_of_d,
                           b.ctl, s, P.particle_skin ? b.state_skin : nullptr);
        });
        nl += 4;
        return cudaGetLastError() == cudaSuccess ? nl : -1;
    }

    // Fields stored in working order while the working order is on (the state arrays are in sorted order).
    bool in_working_order(int field) const {
        if (!working_order() || !w_of_d) return false;
        switch (field) {
            case PCISPH_FIELD_NORMAL: case PCISPH_FIELD_PREDICTED_POSITION: case PCISPH_FIELD_DENSITY:
            case PCISPH_FIELD_OTHER_FORCE: case PCISPH_FIELD_PRESSURE: case PCISPH_FIELD_PRESSURE_FORCE:
            case PCISPH_FIELD_DENSITY_VARIATION: case PCISPH_FIELD_SORTED_POSITION:
            case PCISPH_FIELD_SORTED_VELOCITY:
                return true;
            default:
                return false;
        }
    }

    int ensure_lists() {
        if (!list_sweeps()) return PCISPH_OK;
        const size_t n = params.fluid_count;
        if (n >= (1u << 31)) return fail(PCISPH_ERR_INVALID_ARG, "kernel variant 2 takes fewer than 2^31 particles");
        const size_t nb = params.boundary_count;
        const bool bnd = nb > 0;
        const size_t bytes = align256(n * P.list_cap * 4) + align256(n * 4) + align256(n * P.near_cap * 4) +
                             align256(n * 4) + align256(params.bucket_count) + align256(n) +
                             align256((size_t)kMarkCap * 4) + align256(n * 4) +
                             (bnd ? align256(n * P.bnd_cap * 4) + align256(n * 4) + align256(nb * P.bfl_cap * 4) +
                                        align256(nb * 4)
                                  : 0);
        if (list_block.p && list_block.cap >= bytes && list_n == n && list_b_n == nb) return PCISPH_OK;
        CUDA_TRY(cudaStreamSynchronize(stream()));
        if (list_block.ensure(bytes) != cudaSuccess)
            return fail(PCISPH_ERR_OOM, "device allocation of the neighbour lists failed");
        Carver c{static_cast<unsigned char*>(list_block.p)};
        b.nbr = c.take<uint32_t>(n * P.list_cap);
        b.nbr_count = c.take<uint32_t>(n);
        b.near = c.take<uint32_t>(n * P.near_cap);
        b.near_count = c.take<uint32_t>(n);
        b.bucket_fast = c.take<unsigned char>(params.bucket_count);
        b.b_near = c.take<unsigned char>(n);
        b.fast_list = c.take<uint32_t>(kMarkCap);
        b.walk_stamp = c.take<uint32_t>(n);
        CUDA_TRY(cudaMemsetAsync(b.walk_stamp, 0, n * 4, stream()));  // round numbers start at 1
        b.bnbr = bnd ? c.take<uint32_t>(n * P.bnd_cap) : nullptr;
        b.bnbr_count = bnd ? c.take<uint32_t>(n) : nullptr;
        b.bfl = bnd ? c.take<uint32_t>(nb * P.bfl_cap) : nullptr;
        b.bfl_count = bnd ? c.take<uint32_t>(nb) : nullptr;
        list_n = n;
        list_b_n = nb;
        graph_valid = false;
        order_age = kNoOrder;
        return PCISPH_OK;
    }


    cudaGraphExec_t graph_exec = nullptr;        // the step, bucket sort included
    cudaGraphExec_t graph_exec_reuse = nullptr;  // the step reusing the last bucket order (working order on)
    bool graph_valid = false;
    // The working order's bucket placement (the bucket sort's output) is refreshed every kOrderRefresh steps
    // and reused in between: any placement of whole buckets keeps every sum, only locality ages as
    // particles change cells. order_age: steps since the last bucket sort ran, kNoOrder when none ran for
    // the current buffers and graphs.
    static constexpr uint32_t kOrderRefresh = 8;
    static constexpr uint32_t kNoOrder = 0xFFFFFFFFu;
    uint32_t order_age = kNoOrder;
    bool reuse_order_now = false;   // record_working_order: keep bucket_order instead of sorting
    const uint32_t* bucket_order = nullptr;  // bucket ids in Morton order of their cells (the last bucket sort)
    int prefix_launches_reuse = 0;
    uint64_t host_launches = 0;
    uint64_t host_mode_iters = 0;  // corrective iterations run by the host-driven loop
    cudaStream_t own_stream = nullptr;
    uint64_t steps_launched = 0;
    int prefix_launches = 0;
    int iter_launches = 0;

    bool profiling = false;
    host::KernelTimer timer;  // per-kernel times of the profiled (host-driven) steps

    cudaStream_t stream() const { return user_stream; }

    // ------------------------------------------------------------ memory
    int ensure_fluid(uint32_t n, uint32_t bk) {
        if (n == fluid_cap_n && bk == fluid_cap_bk && fluid_block.p) return PCISPH_OK;
        CUDA_TRY(cudaStreamSynchronize(stream()));
        if (fluid_block.ensure(fluid_arena_bytes(n, bk)) != cudaSuccess)
            return fail(PCISPH_ERR_OOM, "device allocation of the fluid arena failed (" + std::to_string(n) +
                                            " particles)");
        Carver c{static_cast<unsigned char*>(fluid_block.p)};
        b.state_pos = c.take<float4>(n);
        b.state_vel = c.take<float4>(n);
        b.pos = c.take<float4>(n);
        b.vel = c.take<float4>(n);
        b.pr4 = c.take<float4>(n);
        b.normal = c.take<float4>(n);
        b.f_other = c.take<float4>(n);
        b.f_press = c.take<float4>(n);
        b.pred = c.take<float4>(n);
        b.pf4 = c.take<float4>(n);
        b.rho = c.take<float>(n);
        b.press = c.take<float>(n);
        b.err = c.take<float>(n);
        f_keys = c.take<uint32_t>(n);
        f_ids = c.take<uint32_t>(n);
        b.codes = c.take<uint32_t>(n);
        b.groups = c.take<uint32_t>(n);
        b.state_skin = c.take<float>(n);  // zero: "no skin yet", read as the largest
        b.disp_max = c.take<float>(n);
        b.cells = c.take<uint2>(bk);
        CUDA_TRY(cudaMemsetAsync(fluid_block.p, 0, fluid_arena_bytes(n, bk), stream()));
        fluid_cap_n = n;
        fluid_cap_bk = bk;
        sorted_keys = f_keys;
        sorted_ids = f_ids;
        graph_valid = false;
        order_age = kNoOrder;
        return ensure_shared(std::max(n, boundary_cap_n));
    }

    int ensure_boundary(uint32_t n, uint32_t bk) {
        if (n == boundary_cap_n && bk == boundary_cap_bk && boundary_block.p) return PCISPH_OK;
        CUDA_TRY(cudaStreamSynchronize(stream()));
        if (boundary_block.ensure(boundary_arena_bytes(n, bk)) != cudaSuccess)
            return fail(PCISPH_ERR_OOM, "device allocation of the boundary arena failed");
        Carver c{static_cast<unsigned char*>(boundary_block.p)};
        b_pos_in = c.take<float4>(n);
        b.b_pos = c.take<float4>(n);
        b.bpf = c.take<float4>(n);
        b.b_press = c.take<float>(n);
        b.b_init = c.take<float>(n);
        b_keys = c.take<uint32_t>(n);
        b_ids = c.take<uint32_t>(n);
        b.b_codes = c.take<uint32_t>(n);
        b.b_cells = c.take<uint2>(bk);
        CUDA_TRY(cudaMemsetAsync(boundary_block.p, 0, boundary_arena_bytes(n, bk), stream()));
        boundary_cap_n = n;
        boundary_cap_bk = bk;
        graph_valid = false;
        order_age = kNoOrder;
        return ensure_shared(std::max(n, fluid_cap_n));
    }

    int ensure_shared(uint32_t n) {
        const size_t sort_bytes = RadixSorter::scratch_bytes(std::max<uint32_t>(n, 1), sorter.digit_bits());
        if (sort_block.cap < sort_bytes) {
            if (sort_block.ensure(sort_bytes) != cudaSuccess)
                return fail(PCISPH_ERR_OOM, "device allocation of the sort scratch failed");
            sorter.set_scratch(sort_block.p, sort_block.cap);
            graph_valid = false;
            order_age = kNoOrder;
        }
        if (staging_block.ensure((size_t)std::max<uint32_t>(n, 1) * 16) != cudaSuccess)
            return fail(PCISPH_ERR_OOM, "device allocation of the staging buffer failed");
        return PCISPH_OK;
    }

    // -------------------------------------------------------- parameters
    void build_devparams() {
        make_devparams(params, opts.min_iterations, opts.max_iterations, opts.walls, opts.box_lo, opts.box_hi,
                       opts.restitution, threshold, opts.list_skin, 0, &P);
        const bool skins = opts.particle_skin == 1 || (opts.particle_skin == 2 && params.boundary_count > 0);
        P.particle_skin = skins && list_sweeps() ? 1 : 0;
        P.skin_min_half = std::min(kSkinMinHalf * P.h, P.skin_max_half);
        P.skin_factor = kSkinFactor;
        // partner marks scan the 5 x 5 x 5 cells around a fast prediction: a particle that did not outrun its
        // skin lies within h + skin_max_half of a prediction within h of its own, which must stay below two
        // cells (with a margin for the divisions of cell_of)
        P.mark_cap = list_sweeps() && P.h + P.skin_max_half <= 1.9f * P.cell_size ? kMarkCap : 0u;
        graph_valid = false;
        order_age = kNoOrder;
    }

    // update_deduced_attributes: derive, (re)allocate, zero velocities, mark the boundary for sorting.
    int derive_now() {
        derive(&params);
        // keys of 17-20 bits (131K-1M buckets) sort in two passes of 10-bit digits instead of three of 8
        // (70.6 -> 60.5 us at 1M); other widths keep 8-bit digits. The autotuner may choose again.
        const int kb = key_bits(params.bucket_count);
        sorter.set_digit_bits(kb > 16 && kb <= 20 ? 10 : 8);
        int rc = ensure_fluid(params.fluid_count, params.bucket_count);
        if (rc) return rc;
        rc = ensure_boundary(params.boundary_count, params.bucket_count);
        if (!rc) rc = ensure_shared(std::max(fluid_cap_n, boundary_cap_n));  // scratch for the digit width
        if (rc) return rc;
        if (params.fluid_count) CUDA_TRY(cudaMemsetAsync(b.state_vel, 0, (size_t)params.fluid_count * 16, stream()));
        build_devparams();
        boundary_updated = true;
        params_changed = false;
        return PCISPH_OK;
    }

    // -------------------------------------------------------------- timing
    template <class F>
    void timed(const char* name, cudaStream_t s, F&& f) {
        if (profiling) timer.timed(name, s, f);
        else f();
    }
    void collect_timings() { timer.collect(stream()); }

    // ---------------------------------------------------------------- sort
    int sort_set(const float4* pos_in, uint32_t n, uint32_t* keys, uint32_t* ids, uint32_t** sk, uint32_t** sv,
                 cudaStream_t s) {
        timed("hash", s, [&] { launch_hash(reinterpret_cast<const float*>(pos_in), false, n, P, keys, nullptr, s); });
        int nl = 0;
        cudaError_t e = cudaSuccess;
        timed("radix_sort", s, [&] {
            e = sorter.sort(keys, ids, n, key_bits(params.bucket_count), true, s, sk, sv);
            nl = sorter.last_launches();
        });
        if (e != cudaSuccess) {
            fail(PCISPH_ERR_CUDA, std::string("radix sort: ") + cudaGetErrorString(e));
            return -1;
        }
        return 1 + nl;
    }

    int boundary_sort(cudaStream_t s) {
        const uint32_t B = params.boundary_count;
        CUDA_TRY(cudaMemsetAsync(b.b_cells, 0, (size_t)params.bucket_count * 8, s));
        uint32_t *sk = nullptr, *sv = nullptr;
        int nl = sort_set(b_pos_in, B, b_keys, b_ids, &sk, &sv, s);
        if (nl < 0) return PCISPH_ERR_CUDA;
        if (sk != b_keys) {
            CUDA_TRY(cudaMemcpyAsync(b_keys, sk, (size_t)B * 4, cudaMemcpyDeviceToDevice, s));
            CUDA_TRY(cudaMemcpyAsync(b_ids, sv, (size_t)B * 4, cudaMemcpyDeviceToDevice, s));
        }
        timed("reorder_boundary", s,
              [&] { launch_reorder(b_keys, b_ids, b_pos_in, nullptr, B, b.b_pos, nullptr, b.b_cells, b.b_codes, nullptr, P, b.ctl, s); });
        if (opts.boundary_self_density) timed("boundary_self_density", s, [&] { launch_boundary_self_density(P, b, s); });
        else CUDA_TRY(cudaMemsetAsync(b.b_init, 0, (size_t)B * 4, s));
        host_launches += nl + 1 + (opts.boundary_self_density ? 1 : 0);
        CUDA_TRY(cudaGetLastError());
        int rc = build_boundary_zone(s);
        if (rc) return rc;
        boundary_updated = false;
        return PCISPH_OK;
    }

    // The boundary zone over the sorted boundary positions (list sweeps only; once per boundary change,
    // synchronising for the cell bounds). Kernel arguments change, so the step graphs are rebuilt.
    int build_boundary_zone(cudaStream_t s) {
        zone_map = nullptr;
        graph_valid = false;
        const uint32_t B = params.boundary_count;
        if (!list_sweeps() || B == 0) return PCISPH_OK;
        if (zone_block.ensure(256) != cudaSuccess) return fail(PCISPH_ERR_OOM, "device allocation of the boundary zone failed");
        int* bounds = static_cast<int*>(zone_block.p);
        int h[6] = {INT_MAX, INT_MAX, INT_MAX, INT_MIN, INT_MIN, INT_MIN};
        CUDA_TRY(cudaMemcpyAsync(bounds, h, sizeof(h), cudaMemcpyHostToDevice, s));
        launch_boundary_cell_bounds(P, b.b_pos, bounds, s);
        CUDA_TRY(cudaMemcpyAsync(h, bounds, sizeof(h), cudaMemcpyDeviceToHost, s));
        CUDA_TRY(cudaStreamSynchronize(s));
        host_launches += 1;
        int64_t dim[3];
        uint64_t cells = 1;
        for (int a = 0; a < 3; ++a) {
            if (h[a] < INT_MIN + 2 || h[3 + a] > INT_MAX - 2) return PCISPH_OK;  // saturated cells: no zone
            dim[a] = (int64_t)h[3 + a] - (int64_t)h[a] + 5;
            if (dim[a] <= 0 || dim[a] > (int64_t)kZoneMaxCells) return PCISPH_OK;  // no zone: every particle walks
            cells *= (uint64_t)dim[a];
            if (cells > kZoneMaxCells) return PCISPH_OK;
        }
        if (zone_block.ensure(256 + cells) != cudaSuccess)
            return fail(PCISPH_ERR_OOM, "device allocation of the boundary zone failed");
        unsigned char* map = static_cast<unsigned char*>(zone_block.p) + 256;
        for (int a = 0; a < 3; ++a) {
            zone_org[a] = (int)((int64_t)h[a] - 2);
            zone_dim[a] = (uint32_t)dim[a];
        }
        CUDA_TRY(cudaMemsetAsync(map, 0, cells, s));
        launch_boundary_zone(P, b.b_pos, zone_org, zone_dim, map, s);
        host_launches += 1;
        CUDA_TRY(cudaGetLastError());
        zone_map = map;
        return PCISPH_OK;
    }

    // ---------------------------------------------------------------- step
    // Everything before the corrective loop. Returns the number of kernels, or -1 on error.
    int record_prefix(cudaStream_t s) {
        const uint32_t N = params.fluid_count, B = params.boundary_count;
        int nl = 0;
        launch_begin(b.ctl, s);
        ++nl;
        if (cudaMemsetAsync(b.cells, 0, (size_t)params.bucket_count * 8, s) != cudaSuccess) return -1;
        if (list_sweeps() && cudaMemsetAsync(b.bucket_fast, 0, params.bucket_count, s) != cudaSuccess) return -1;
        uint32_t *sk = nullptr, *sv = nullptr;
        int r = sort_set(b.state_pos, N, f_keys, f_ids, &sk, &sv, s);
        if (r < 0) return -1;
        nl += r;
        sorted_keys = sk;
        sorted_ids = sv;
        if (working_order()) {
            const int r2 = record_working_order(sk, sv, s);
            if (r2 < 0) return -1;
            nl += r2 - 1;  // the reorder launch is counted below
        } else {
            timed("reorder", s, [&] {
                launch_reorder(sk, sv, b.state_pos, b.state_vel, N, b.pos, b.vel, b.cells, b.codes, b.groups, P, b.ctl,
                               s, P.particle_skin ? b.state_skin : nullptr);
            });
        }
        const SweepArgs A = sweep_args();
        if (list_sweeps()) {
            timed("density", s, [&] { launch_density_list(P, b.ctl, list_buffers(), s); });
            timed("normal", s, [&] { launch_normal_list(P, b.ctl, list_buffers(), s); });
            if (B) {
                timed("boundary_list", s, [&] { launch_boundary_fluid_list(P, list_buffers(), s); });
                ++nl;
            }
        } else if (warp_sweeps()) {
            timed("density", s, [&] { launch_density_sweep(P, b, A, sweep_grid, s); });
            timed("normal", s, [&] { launch_normal_sweep(P, b, A, sweep_grid, s); });
        } else {
            timed("density", s, [&] { launch_density(P, b, s); });
            timed("normal", s, [&] { launch_normal(P, b, s); });
        }
        if (B && cudaMemsetAsync(b.b_press, 0, (size_t)B * 4, s) != cudaSuccess) return -1;
        if (list_sweeps()) timed("force", s, [&] { launch_force_list(P, b.ctl, list_buffers(), s); });
        else if (warp_sweeps()) timed("force", s, [&] { launch_force_sweep(P, b, A, sweep_grid, s); });
        else timed("force", s, [&] { launch_force(P, b, s); });
        nl += 4;
        if (partner_marks()) {
            timed("mark", s, [&] { launch_mark_partners(P, b.ctl, list_buffers(true), s); });
            ++nl;
        }
        if (cudaGetLastError() != cudaSuccess) return -1;
        return nl;
    }

    int record_iteration(cudaStream_t s, cudaGraphConditionalHandle cond, bool use_cond) {
        int nl = 0;
        if (params.boundary_count) {
            if (list_sweeps())
                timed("boundary_pressure", s, [&] { launch_boundary_pressure_list(P, b.ctl, list_buffers(), s); });
            else
                timed("boundary_pressure", s, [&] { launch_boundary_pressure(P, b, working_order() ? cells_w : b.cells, s); });
            ++nl;
        }
        if (list_sweeps()) {
            const bool marks = partner_marks();
            timed("pressure", s, [&] { launch_pressure_list(P, b.ctl, list_buffers(marks), opts.sweep_block, s); });
            timed("pressure_force", s, [&] {
                launch_pressure_force_list(P, b.ctl, list_buffers(), 0, cond, use_cond, opts.sweep_block, s);
            });
            if (marks) {
                timed("mark", s, [&] { launch_mark_partners(P, b.ctl, list_buffers(true), s); });
                ++nl;
            }
        } else if (warp_sweeps()) {
            const SweepArgs A = sweep_args();
            timed("pressure", s, [&] { launch_pressure_sweep(P, b, A, sweep_grid, s); });
            timed("pressure_force", s, [&] { launch_pressure_force_sweep(P, b, A, sweep_grid, 0, cond, use_cond, s); });
        } else {
            timed("pressure", s, [&] { launch_pressure(P, b, s); });
            timed("pressure_force", s, [&] { launch_pressure_force(P, b, 0, cond, use_cond, s); });
        }
        nl += 2;
        return nl;
    }

    int build_graph() {
        for (cudaGraphExec_t* g : {&graph_exec, &graph_exec_reuse})
            if (*g) {
                cudaGraphExecDestroy(*g);
                *g = nullptr;
            }
        reuse_order_now = false;
        int rc = capture_graph(&graph_exec, &prefix_launches);
        if (rc) return rc;
        if (working_order()) {  // the same step without the bucket sort
            reuse_order_now = true;
            rc = capture_graph(&graph_exec_reuse, &prefix_launches_reuse);
            reuse_order_now = false;
            if (rc) return rc;
        }
        order_age = kNoOrder;  // the first launch sorts the buckets
        graph_valid = true;
        return PCISPH_OK;
    }

    int capture_graph(cudaGraphExec_t* exec, int* prefix_nl) {
        const bool prof = profiling;
        profiling = false;
        cudaStream_t s = capture_stream;
        cudaGraph_t graph = nullptr;
        CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        int nl = record_prefix(s);
        if (opts.loop_mode == 2) {  // persistent loop: prefix + one cooperative kernel, no conditional node
            cudaError_t le = nl < 0 ? cudaSuccess : launch_corrective_loop(P, b.ctl, list_buffers(), s);
            cudaError_t ee = cudaStreamEndCapture(s, &graph);
            profiling = prof;
            if (nl < 0 || le != cudaSuccess || ee != cudaSuccess) {
                if (graph) cudaGraphDestroy(graph);
                return fail(PCISPH_ERR_CUDA, std::string("graph capture of the persistent step failed: ") +
                                                 cudaGetErrorString(le != cudaSuccess ? le : ee));
            }
            *prefix_nl = nl + 1;
            iter_launches = 0;
            cudaError_t ie = cudaGraphInstantiate(exec, graph, 0);
            cudaGraphDestroy(graph);
            if (ie != cudaSuccess) return fail(PCISPH_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ie));
            return PCISPH_OK;
        }
        cudaStreamCaptureStatus st;
        const cudaGraphNode_t* deps = nullptr;
        size_t ndeps = 0;
        cudaError_t e = cudaStreamGetCaptureInfo(s, &st, nullptr, nullptr, &deps, nullptr, &ndeps);
        std::vector<cudaGraphNode_t> leaves(deps, deps + (e == cudaSuccess ? ndeps : 0));
        cudaError_t e2 = cudaStreamEndCapture(s, &graph);
        profiling = prof;
        if (nl < 0 || e != cudaSuccess || e2 != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            return fail(PCISPH_ERR_CUDA, std::string("graph capture of the step failed: ") +
                                             cudaGetErrorString(e != cudaSuccess ? e : e2));
        }
        *prefix_nl = nl;
        cudaGraphConditionalHandle handle;
        CUDA_TRY(cudaGraphConditionalHandleCreate(&handle, graph, 1, cudaGraphCondAssignDefault));
        cudaGraphNodeParams cp{};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = handle;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t loop_node;
        CUDA_TRY(cudaGraphAddNode(&loop_node, graph, leaves.data(), nullptr, leaves.size(), &cp));
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        CUDA_TRY(cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        profiling = false;
        iter_launches = record_iteration(s, handle, true);
        profiling = prof;
        cudaGraph_t body_out = nullptr;
        CUDA_TRY(cudaStreamEndCapture(s, &body_out));
        e = cudaGraphInstantiate(exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return fail(PCISPH_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
        return PCISPH_OK;
    }

    int check_consistent() const {
        if (params.fluid_count == 0) return PCISPH_OK;
        auto msg = [&](const char* name, uint32_t got) {
            return std::string("Inconsistent ") + name + " (" + std::to_string(got) + ") for " +
                   std::to_string(params.fluid_count) + " particles";
        };
        if (fluid_loaded != params.fluid_count)
            return fail(PCISPH_ERR_INCONSISTENT, msg("positions_size", fluid_loaded == 0xFFFFFFFFu ? 0 : fluid_loaded));
        if (params.boundary_count && boundary_loaded != params.boundary_count)
            return fail(PCISPH_ERR_INCONSISTENT, "Inconsistent boundary_positions (" +
                                                     std::to_string(boundary_loaded == 0xFFFFFFFFu ? 0 : boundary_loaded) +
                                                     ") for " + std::to_string(params.boundary_count) + " particles");
        return PCISPH_OK;
    }

    int update() {
        if (params_changed) {
            int rc = derive_now();
            if (rc) return rc;
        }
        int rc = check_consistent();
        if (rc) return rc;
        if (params.fluid_count == 0) return PCISPH_OK;  // Fluid.cpp:117-118
        rc = ensure_lists();
        if (!rc) rc = ensure_order();
        if (rc) return rc;
        cudaStream_t s = stream();
        if (boundary_updated && params.boundary_count > 0) {
            rc = boundary_sort(s);
            if (rc) return rc;
        }
        if (opts.loop_mode != 1 && !profiling) {
            if (!graph_valid) {
                rc = build_graph();
                if (rc) return rc;
            }
            const bool full = !graph_exec_reuse || order_age >= kOrderRefresh;
            CUDA_TRY(cudaGraphLaunch(full ? graph_exec : graph_exec_reuse, s));
            host_launches += full ? prefix_launches : prefix_launches_reuse;
            order_age = full ? 1u : order_age + 1u;
            ++steps_launched;
            return PCISPH_OK;
        }
        // host-driven loop (Fluid.cpp:250-307), on the same bucket-order schedule as the graphs
        const bool full = !working_order() || order_age >= kOrderRefresh;
        reuse_order_now = !full;
        int nl = record_prefix(s);
        reuse_order_now = false;
        order_age = full ? 1u : order_age + 1u;
        if (nl < 0) return fail(PCISPH_ERR_CUDA, std::string("step launch failed: ") + cudaGetErrorString(cudaGetLastError()));
        host_launches += nl;
        ++steps_launched;
        if (opts.loop_mode == 2) {  // profiled persistent loop
            cudaError_t le = cudaSuccess;
            timed("corrective_loop", s, [&] { le = launch_corrective_loop(P, b.ctl, list_buffers(), s); });
            if (le != cudaSuccess) return fail(PCISPH_ERR_CUDA, std::string("persistent loop: ") + cudaGetErrorString(le));
            ++host_launches;
            collect_timings();
            return PCISPH_OK;
        }
        const int lim = std::max(1, opts.max_iterations);
        for (int i = 0; i < lim; ++i) {
            host_launches += record_iteration(s, 0, false);
            ++host_mode_iters;
            CUDA_TRY(cudaGetLastError());
            if (i + 1 >= std::min(opts.min_iterations, lim)) {
                CUDA_TRY(cudaMemcpyAsync(&host_ctl->done, &b.ctl->done, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
                CUDA_TRY(cudaStreamSynchronize(s));
                if (host_ctl->done) break;
            }
        }
        collect_timings();
        return PCISPH_OK;
    }

    int run_stage(int stage, int arg) {
        if (params_changed) {
            int rc = derive_now();
            if (rc) return rc;
        }
        int rc = check_consistent();
        if (rc) return rc;
        rc = ensure_lists();
        if (!rc) rc = ensure_order();
        if (rc) return rc;
        cudaStream_t s = stream();
        const uint32_t N = params.fluid_count;
        switch (stage) {
            case PCISPH_STAGE_SORT: {
                if (boundary_updated && params.boundary_count > 0) {
                    rc = boundary_sort(s);
                    if (rc) return rc;
                }
                launch_begin(b.ctl, s);
                CUDA_TRY(cudaMemsetAsync(b.cells, 0, (size_t)params.bucket_count * 8, s));
                if (list_sweeps()) CUDA_TRY(cudaMemsetAsync(b.bucket_fast, 0, params.bucket_count, s));
                uint32_t *sk = nullptr, *sv = nullptr;
                int nl = sort_set(b.state_pos, N, f_keys, f_ids, &sk, &sv, s);
                if (nl < 0) return PCISPH_ERR_CUDA;
                sorted_keys = sk;
                sorted_ids = sv;
                if (working_order()) {
                    const int r2 = record_working_order(sk, sv, s);
                    if (r2 < 0) return fail(PCISPH_ERR_CUDA, "working order of the sort stage failed");
                    host_launches += nl + 1 + r2;
                } else {
                    launch_reorder(sk, sv, b.state_pos, b.state_vel, N, b.pos, b.vel, b.cells, b.codes, b.groups, P,
                                   b.ctl, s, P.particle_skin ? b.state_skin : nullptr);
                    host_launches += nl + 2;
                }
                break;
            }
            case PCISPH_STAGE_DENSITY:
                if (list_sweeps()) launch_density_list(P, b.ctl, list_buffers(), s);
                else if (warp_sweeps()) launch_density_sweep(P, b, sweep_args(), sweep_grid, s);
                else launch_density(P, b, s);
                ++host_launches;
                break;
            case PCISPH_STAGE_NORMAL:
                if (list_sweeps()) launch_normal_list(P, b.ctl, list_buffers(), s);
                else if (warp_sweeps()) launch_normal_sweep(P, b, sweep_args(), sweep_grid, s);
                else launch_normal(P, b, s);
                ++host_launches;
                break;
            case PCISPH_STAGE_FORCE:
                if (list_sweeps()) launch_force_list(P, b.ctl, list_buffers(), s);
                else if (warp_sweeps()) launch_force_sweep(P, b, sweep_args(), sweep_grid, s);
                else launch_force(P, b, s);
                ++host_launches;
                break;
            case PCISPH_STAGE_BOUNDARY_PRESSURE: launch_boundary_pressure(P, b, working_order() ? cells_w : b.cells, s); ++host_launches; break;
            case PCISPH_STAGE_PRESSURE:
                if (list_sweeps()) launch_pressure_list(P, b.ctl, list_buffers(), opts.sweep_block, s);
                else if (warp_sweeps()) launch_pressure_sweep(P, b, sweep_args(), sweep_grid, s);
                else launch_pressure(P, b, s);
                ++host_launches;
                break;
            case PCISPH_STAGE_PRESSURE_FORCE:
                if (list_sweeps())
                    launch_pressure_force_list(P, b.ctl, list_buffers(), arg ? 2 : 1, 0, false, opts.sweep_block, s);
                else if (warp_sweeps()) launch_pressure_force_sweep(P, b, sweep_args(), sweep_grid, arg ? 2 : 1, 0, false, s);
                else launch_pressure_force(P, b, arg ? 2 : 1, 0, false, s);
                ++host_launches;
                break;
            case PCISPH_STAGE_PACK: launch_pack(P, b, s); ++host_launches; break;
            case PCISPH_STAGE_BOUNDARY_PRESSURE_RESET:
                if (params.boundary_count) CUDA_TRY(cudaMemsetAsync(b.b_press, 0, (size_t)params.boundary_count * 4, s));
                break;
            default: return fail(PCISPH_ERR_INVALID_ARG, "unknown stage " + std::to_string(stage));
        }
        CUDA_TRY(cudaGetLastError());
        return PCISPH_OK;
    }

    // ---------------------------------------------------------------- fields
    struct FieldView {
        void* ptr;
        size_t count;      // elements (particles, or uint32 entries for tables)
        int layout;        // native: FLOAT4 or SCALAR
    };
    bool field_view(int field, FieldView* v) {
        const size_t N = params.fluid_count, B = params.boundary_count, BK = params.bucket_count;
        switch (field) {
            case PCISPH_FIELD_POSITION: *v = {b.state_pos, N, PCISPH_LAYOUT_FLOAT4}; return true;
            case PCISPH_FIELD_VELOCITY: *v = {b.state_vel, N, PCISPH_LAYOUT_FLOAT4}; return true;
            case PCISPH_FIELD_NORMAL: *v = {b.normal, N, PCISPH_LAYOUT_FLOAT4}; return true;
            case PCISPH_FIELD_PREDICTED_POSITION: *v = {b.pred, N, PCISPH_LAYOUT_FLOAT4}; return true;
            case PCISPH_FIELD_DENSITY: *v = {b.rho, N, PCISPH_LAYOUT_SCALAR}; return true;
            case PCISPH_FIELD_OTHER_FORCE: *v = {b.f_other, N, PCISPH_LAYOUT_FLOAT4}; return true;
            case PCISPH_FIELD_PRESSURE: *v = {b.press, N, PCISPH_LAYOUT_SCALAR}; return true;
            case PCISPH_FIELD_PRESSURE_FORCE: *v = {b.f_press, N, PCISPH_LAYOUT_FLOAT4}; return true;
            case PCISPH_FIELD_DENSITY_VARIATION: *v = {b.err, N, PCISPH_LAYOUT_SCALAR}; return true;
            case PCISPH_FIELD_SORTED_POSITION: *v = {b.pos, N, PCISPH_LAYOUT_FLOAT4}; return true;
            case PCISPH_FIELD_SORTED_VELOCITY: *v = {b.vel, N, PCISPH_LAYOUT_FLOAT4}; return true;
            case PCISPH_FIELD_KEYS: *v = {sorted_keys, N, PCISPH_LAYOUT_SCALAR}; return true;
            case PCISPH_FIELD_SRC: *v = {sorted_ids, N, PCISPH_LAYOUT_SCALAR}; return true;
            case PCISPH_FIELD_CELL_OFFSETS: *v = {b.cells, 2 * BK, PCISPH_LAYOUT_SCALAR}; return true;
            case PCISPH_FIELD_BOUNDARY_POSITION: *v = {b.b_pos, B, PCISPH_LAYOUT_FLOAT4}; return true;
            case PCISPH_FIELD_BOUNDARY_PRESSURE: *v = {b.b_press, B, PCISPH_LAYOUT_SCALAR}; return true;
            case PCISPH_FIELD_BOUNDARY_INIT_DENSITY: *v = {b.b_init, B, PCISPH_LAYOUT_SCALAR}; return true;
            case PCISPH_FIELD_BOUNDARY_KEYS: *v = {b_keys, B, PCISPH_LAYOUT_SCALAR}; return true;
            case PCISPH_FIELD_BOUNDARY_SRC: *v = {b_ids, B, PCISPH_LAYOUT_SCALAR}; return true;
            case PCISPH_FIELD_BOUNDARY_CELL_OFFSETS: *v = {b.b_cells, 2 * BK, PCISPH_LAYOUT_SCALAR}; return true;
            default: return false;
        }
    }

    static size_t layout_bytes(size_t count, int layout) {
        return count * (layout == PCISPH_LAYOUT_PACKED3 ? 12 : layout == PCISPH_LAYOUT_FLOAT4 ? 16 : 4);
    }

    int copy_vectors_in(float4* dst, const float* src, size_t n, int layout, int memory) {
        cudaStream_t s = stream();
        if (n == 0) return PCISPH_OK;
        if (layout == PCISPH_LAYOUT_FLOAT4) {
            CUDA_TRY(cudaMemcpyAsync(dst, src, n * 16,
                                     memory == PCISPH_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, s));
        } else if (layout == PCISPH_LAYOUT_PACKED3) {
            const float* dsrc = src;
            if (memory == PCISPH_MEM_HOST) {
                if (const void* dv = host::pinned_device_view(src)) {
                    dsrc = static_cast<const float*>(dv);  // the conversion reads the pinned buffer itself
                } else {
                    CUDA_TRY(cudaMemcpyAsync(staging_block.p, src, n * 12, cudaMemcpyHostToDevice, s));
                    dsrc = static_cast<const float*>(staging_block.p);
                }
            }
            launch_pack3_to4(dsrc, dst, (uint32_t)n, s);
            ++host_launches;
            CUDA_TRY(cudaGetLastError());
        } else {
            return fail(PCISPH_ERR_INVALID_ARG, "vector fields take PACKED3 or FLOAT4");
        }
        return PCISPH_OK;
    }

    // sync = false: a HOST copy is left queued (the caller synchronises)
    int get_field(int field, void* dst, size_t dst_bytes, int layout, int memory, bool sync = true) {
        FieldView v;
        if (!field_view(field, &v)) return fail(PCISPH_ERR_INVALID_ARG, "unknown field " + std::to_string(field));
        if (!v.ptr) return fail(PCISPH_ERR_NOT_READY, "field not allocated yet (set the state or call update first)");
        if (v.layout == PCISPH_LAYOUT_SCALAR && layout != PCISPH_LAYOUT_SCALAR)
            return fail(PCISPH_ERR_INVALID_ARG, "scalar field: use PCISPH_LAYOUT_SCALAR");
        if (v.layout == PCISPH_LAYOUT_FLOAT4 && layout == PCISPH_LAYOUT_SCALAR)
            return fail(PCISPH_ERR_INVALID_ARG, "vector field: use PACKED3 or FLOAT4");
        const size_t need = layout_bytes(v.count, layout);
        if (dst_bytes < need || (!dst && need))
            return fail(PCISPH_ERR_INVALID_ARG, "destination too small: need " + std::to_string(need) + " bytes");
        if (need == 0) return PCISPH_OK;
        cudaStream_t s = stream();
        const cudaMemcpyKind kind = memory == PCISPH_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
        if (in_working_order(field)) {  // back to sorted order: out[d] = field[w_of_d[d]]
            if (v.layout == PCISPH_LAYOUT_FLOAT4)
                launch_gather4(static_cast<const float4*>(v.ptr), w_of_d, xfer, (uint32_t)v.count, s);
            else
                launch_gather1(static_cast<const float*>(v.ptr), w_of_d, reinterpret_cast<float*>(xfer), (uint32_t)v.count, s);
            ++host_launches;
            CUDA_TRY(cudaGetLastError());
            v.ptr = xfer;
        }
        if (field == PCISPH_FIELD_SORTED_POSITION && layout == PCISPH_LAYOUT_FLOAT4 && P.particle_skin) {
            // w of the step's positions holds each particle's half skin: export 0 there
            float4* tmp = v.ptr == xfer ? xfer : static_cast<float4*>(staging_block.p);
            launch_xyz0(static_cast<const float4*>(v.ptr), tmp, (uint32_t)v.count, s);
            ++host_launches;
            CUDA_TRY(cudaGetLastError());
            v.ptr = tmp;
        }
        if (layout == PCISPH_LAYOUT_PACKED3) {
            void* pinned = memory == PCISPH_MEM_HOST ? host::pinned_device_view(dst) : nullptr;
            float* out = memory == PCISPH_MEM_HOST ? static_cast<float*>(pinned ? pinned : staging_block.p)
                                                   : static_cast<float*>(dst);
            launch_unpack4_to3(static_cast<const float4*>(v.ptr), out, (uint32_t)v.count, s);
            ++host_launches;
            CUDA_TRY(cudaGetLastError());
            if (memory == PCISPH_MEM_HOST && !pinned) CUDA_TRY(cudaMemcpyAsync(dst, out, need, kind, s));
        } else {
            CUDA_TRY(cudaMemcpyAsync(dst, v.ptr, need, kind, s));
        }
        if (memory == PCISPH_MEM_HOST && sync) CUDA_TRY(cudaStreamSynchronize(s));
        return PCISPH_OK;
    }

    int set_field(int field, const void* src, size_t src_bytes, int layout, int memory) {
        FieldView v;
        if (!field_view(field, &v)) return fail(PCISPH_ERR_INVALID_ARG, "unknown field " + std::to_string(field));
        if (!v.ptr) return fail(PCISPH_ERR_NOT_READY, "field not allocated yet");
        const size_t need = layout_bytes(v.count, layout);
        if (src_bytes < need || (!src && need)) return fail(PCISPH_ERR_INVALID_ARG, "source too small");
        if (in_working_order(field) && v.count) {  // sorted order in, working order stored: f[w_of_d[d]] = in[d]
            cudaStream_t s = stream();
            if (v.layout == PCISPH_LAYOUT_FLOAT4) {
                int rc = copy_vectors_in(xfer, static_cast<const float*>(src), v.count, layout, memory);
                if (rc) return rc;
                launch_scatter4(xfer, w_of_d, static_cast<float4*>(v.ptr), (uint32_t)v.count, s);
            } else {
                if (layout != PCISPH_LAYOUT_SCALAR) return fail(PCISPH_ERR_INVALID_ARG, "scalar field: use PCISPH_LAYOUT_SCALAR");
                CUDA_TRY(cudaMemcpyAsync(xfer, src, need,
                                         memory == PCISPH_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, s));
                launch_scatter1(reinterpret_cast<const float*>(xfer), w_of_d, static_cast<float*>(v.ptr), (uint32_t)v.count, s);
            }
            ++host_launches;
            CUDA_TRY(cudaGetLastError());
            if (memory == PCISPH_MEM_HOST) CUDA_TRY(cudaStreamSynchronize(s));
            return PCISPH_OK;
        }
        if (v.layout == PCISPH_LAYOUT_FLOAT4)
            return copy_vectors_in(static_cast<float4*>(v.ptr), static_cast<const float*>(src), v.count, layout, memory);
        if (layout != PCISPH_LAYOUT_SCALAR) return fail(PCISPH_ERR_INVALID_ARG, "scalar field: use PCISPH_LAYOUT_SCALAR");
        CUDA_TRY(cudaMemcpyAsync(v.ptr, src, need,
                                 memory == PCISPH_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice,
                                 stream()));
        if (memory == PCISPH_MEM_HOST) CUDA_TRY(cudaStreamSynchronize(stream()));
        return PCISPH_OK;
    }

    int stats(pcisph_step_stats* out) {
        CUDA_TRY(cudaStreamSynchronize(stream()));
        CUDA_TRY(cudaMemcpy(host_ctl, b.ctl, sizeof(Control), cudaMemcpyDeviceToHost));
        out->iterations = host_ctl->iterations_last;
        out->max_density_error = host_ctl->max_err_last;
        out->status = host_ctl->status;
        out->status_all = host_ctl->status_all;
        out->steps = host_ctl->steps;
        out->total_iterations = host_ctl->total_iters;
        out->list_fallbacks = host_ctl->list_fallbacks;
        out->fast_particles = host_ctl->fast_particles;
        out->list_skin = opts.list_skin;
        out->max_density_error_max = host::float_from_bits(host_ctl->max_err_max_bits);
        out->unconverged_steps = host_ctl->unconverged_steps;
        return PCISPH_OK;
    }

    ~pcisph_ctx() {
        DeviceGuard g(device);
        if (user_stream) cudaStreamSynchronize(user_stream);
        if (graph_exec) cudaGraphExecDestroy(graph_exec);
        if (graph_exec_reuse) cudaGraphExecDestroy(graph_exec_reuse);
        timer.release();
        fluid_block.release();
        boundary_block.release();
        misc_block.release();
        sort_block.release();
        staging_block.release();
        list_block.release();
        zone_block.release();
        order_block.release();
        bucket_sort_block.release();
        for (auto& kv : exports) kv.second.release();
        render_block.release();
        if (host_ctl) cudaFreeHost(host_ctl);
        if (capture_stream) cudaStreamDestroy(capture_stream);
        if (own_stream) cudaStreamDestroy(own_stream);
    }
};

namespace pcisph {
int report_error(int code, const std::string& msg) { return fail(code, msg); }
}  // namespace pcisph

// ====================================================================== C ABI
extern "C" {

int pcisph_abi_version(void) { return PCISPH_ABI_VERSION; }

const char* pcisph_last_error(void) { return g_last_error.c_str(); }

uint32_t pcisph_sort_bit_count(uint32_t elements) { return sort_bit_count_ref(elements); }

int pcisph_derive_params(float particle_radius, float rest_density, uint32_t fluid_count, uint32_t boundary_count,
                         float delta_t, float gravity, float viscosity, float surface_tension,
                         pcisph_sim_params* out) {
    if (!out) return fail(PCISPH_ERR_INVALID_ARG, "out is NULL");
    std::memset(out, 0, sizeof(*out));
    out->particle_radius = particle_radius;
    out->rest_density = rest_density;
    out->fluid_count = fluid_count;
    out->boundary_count = boundary_count;
    out->delta_t = delta_t;
    out->gravity = gravity;
    out->viscosity_constant = viscosity;
    out->surface_tension_coefficient = surface_tension;
    derive(out);
    return PCISPH_OK;
}

int pcisph_default_options(pcisph_options* o) {
    if (!o) return fail(PCISPH_ERR_INVALID_ARG, "out is NULL");
    std::memset(o, 0, sizeof(*o));
    o->min_iterations = 3;
    o->max_iterations = 7;
    o->walls = 0;
    o->restitution = 0.5f;
    o->boundary_self_density = 0;
    o->loop_mode = 0;
    o->kernel_variant = 2;
    o->list_skin = 0.25f;
    o->spatial_order = 2;
    o->sweep_block = 256;
    o->particle_skin = 2;
    return PCISPH_OK;
}

int pcisph_create(int device, void* stream, pcisph_ctx** out) {
    if (!out) return fail(PCISPH_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    int ndev = 0;
    CUDA_TRY(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return fail(PCISPH_ERR_INVALID_ARG, "no CUDA device " + std::to_string(device));
    DeviceGuard g(device);
    CUDA_TRY(cudaFree(nullptr));  // create the primary context
    CUDA_TRY(radix_configure_kernels());
    SweepGrid sg{};
    CUDA_TRY(sweep_configure(&sg));
    pcisph_ctx* c = new pcisph_ctx();
    c->device = device;
    c->sweep_grid = sg;
    pcisph_default_options(&c->opts);
    c->params.rest_density = 1000.f;
    cudaError_t e = cudaStreamCreateWithFlags(&c->capture_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMallocHost(&c->host_ctl, sizeof(Control));
    if (e == cudaSuccess) e = c->misc_block.ensure(sizeof(Control));
    if (e == cudaSuccess) e = cudaMemset(c->misc_block.p, 0, sizeof(Control));
    if (e != cudaSuccess) {
        delete c;
        return fail(PCISPH_ERR_CUDA, std::string("context setup: ") + cudaGetErrorString(e));
    }
    c->user_stream = stream ? static_cast<cudaStream_t>(stream) : c->own_stream;
    c->b.ctl = c->ctl = static_cast<Control*>(c->misc_block.p);
    std::memset(c->host_ctl, 0, sizeof(Control));
    *out = c;
    return PCISPH_OK;
}

void pcisph_destroy(pcisph_ctx* ctx) { delete ctx; }

int pcisph_set_stream(pcisph_ctx* ctx, void* stream) {
    if (!ctx) return fail(PCISPH_ERR_INVALID_ARG, "ctx is NULL");
    DeviceGuard g(ctx->device);
    cudaStreamSynchronize(ctx->user_stream);
    ctx->user_stream = stream ? static_cast<cudaStream_t>(stream) : ctx->own_stream;
    return PCISPH_OK;
}

#define CTX_SETTER(name, field, type)                                   \
    int name(pcisph_ctx* ctx, type v) {                                 \
        if (!ctx) return fail(PCISPH_ERR_INVALID_ARG, "ctx is NULL");   \
        ctx->params.field = v;                                          \
        ctx->params_changed = true;                                     \
        return PCISPH_OK;                                               \
    }
CTX_SETTER(pcisph_set_boundary_count, boundary_count, uint32_t)
CTX_SETTER(pcisph_set_fluid_count, fluid_count, uint32_t)
CTX_SETTER(pcisph_set_delta_t, delta_t, float)
CTX_SETTER(pcisph_set_rest_density, rest_density, float)
CTX_SETTER(pcisph_set_particle_radius, particle_radius, float)
CTX_SETTER(pcisph_set_gravity, gravity, float)
CTX_SETTER(pcisph_set_viscosity, viscosity_constant, float)
CTX_SETTER(pcisph_set_surface_tension, surface_tension_coefficient, float)

int pcisph_set_density_variation_threshold(pcisph_ctx* ctx, float t) {  // Fluid.cpp:373-375: no re-derivation
    if (!ctx) return fail(PCISPH_ERR_INVALID_ARG, "ctx is NULL");
    ctx->threshold = t;
    ctx->P.threshold = t;
    ctx->graph_valid = false;
    ctx->order_age = pcisph_ctx::kNoOrder;
    return PCISPH_OK;
}

int pcisph_set_options(pcisph_ctx* ctx, const pcisph_options* o) {
    if (!ctx || !o) return fail(PCISPH_ERR_INVALID_ARG, "NULL argument");
    if (o->max_iterations < 1 || o->min_iterations < 1 || o->max_iterations > 10000)
        return fail(PCISPH_ERR_INVALID_ARG, "iteration limits must be in 1..10000");
    if (o->loop_mode < 0 || o->loop_mode > 2) return fail(PCISPH_ERR_INVALID_ARG, "loop_mode must be 0, 1 or 2");
    if (o->loop_mode == 2 && o->kernel_variant != 2)
        return fail(PCISPH_ERR_INVALID_ARG, "loop_mode 2 (persistent loop) runs the list sweeps: kernel_variant 2");
    if (o->kernel_variant < 0 || o->kernel_variant > 2)
        return fail(PCISPH_ERR_INVALID_ARG, "kernel_variant must be 0, 1 or 2");
    if (!(o->list_skin >= 0.f && o->list_skin <= 2.f))
        return fail(PCISPH_ERR_INVALID_ARG, "list_skin must be in [0, 2]");
    if (o->sweep_block != 128 && o->sweep_block != 256 && o->sweep_block != 512)
        return fail(PCISPH_ERR_INVALID_ARG, "sweep_block must be 128, 256 or 512");
    if (o->particle_skin < 0 || o->particle_skin > 2) return fail(PCISPH_ERR_INVALID_ARG, "particle_skin must be 0, 1 or 2");
    const bool bsd_changed = o->boundary_self_density != ctx->opts.boundary_self_density;
    ctx->opts = *o;
    if (bsd_changed) ctx->boundary_updated = true;
    if (!ctx->params_changed) ctx->build_devparams();
    return PCISPH_OK;
}

int pcisph_get_options(const pcisph_ctx* ctx, pcisph_options* out) {
    if (!ctx || !out) return fail(PCISPH_ERR_INVALID_ARG, "NULL argument");
    *out = ctx->opts;
    return PCISPH_OK;
}

int pcisph_get_params(const pcisph_ctx* ctx, pcisph_sim_params* out) {
    if (!ctx || !out) return fail(PCISPH_ERR_INVALID_ARG, "NULL argument");
    *out = ctx->params;
    return PCISPH_OK;
}

int pcisph_prepare(pcisph_ctx* ctx) {
    if (!ctx) return fail(PCISPH_ERR_INVALID_ARG, "ctx is NULL");
    DeviceGuard g(ctx->device);
    return ctx->params_changed ? ctx->derive_now() : PCISPH_OK;
}

int pcisph_get_fluid_state(pcisph_ctx* ctx, float* pos, float* vel, uint32_t count, int layout, int memory) {
    if (!ctx) return fail(PCISPH_ERR_INVALID_ARG, "ctx is NULL");
    if (count && !pos && !vel) return fail(PCISPH_ERR_INVALID_ARG, "pos and vel are NULL");
    if (layout != PCISPH_LAYOUT_PACKED3 && layout != PCISPH_LAYOUT_FLOAT4)
        return fail(PCISPH_ERR_INVALID_ARG, "positions take PACKED3 or FLOAT4");
    if (memory != PCISPH_MEM_HOST && memory != PCISPH_MEM_DEVICE) return fail(PCISPH_ERR_INVALID_ARG, "bad memory kind");
    if (count != ctx->params.fluid_count)
        return fail(PCISPH_ERR_INCONSISTENT, "Inconsistent positions_size (" + std::to_string(count) + ") for " +
                                                 std::to_string(ctx->params.fluid_count) + " particles");
    DeviceGuard g(ctx->device);
    const size_t bytes = (size_t)count * (layout == PCISPH_LAYOUT_PACKED3 ? 12 : 16);
    int rc = PCISPH_OK;
    if (pos) rc = ctx->get_field(PCISPH_FIELD_POSITION, pos, bytes, layout, memory, false);
    if (!rc && vel) rc = ctx->get_field(PCISPH_FIELD_VELOCITY, vel, bytes, layout, memory, false);
    if (rc) return rc;
    if (memory == PCISPH_MEM_HOST) CUDA_TRY(cudaStreamSynchronize(ctx->stream()));
    return PCISPH_OK;
}

int pcisph_set_fluid_state(pcisph_ctx* ctx, const float* pos, const float* vel, uint32_t count, int layout,
                           int memory) {
    if (!ctx) return fail(PCISPH_ERR_INVALID_ARG, "ctx is NULL");
    if (count && !pos) return fail(PCISPH_ERR_INVALID_ARG, "pos is NULL");
    if (layout != PCISPH_LAYOUT_PACKED3 && layout != PCISPH_LAYOUT_FLOAT4)
        return fail(PCISPH_ERR_INVALID_ARG, "positions take PACKED3 or FLOAT4");
    if (memory != PCISPH_MEM_HOST && memory != PCISPH_MEM_DEVICE) return fail(PCISPH_ERR_INVALID_ARG, "bad memory kind");
    if (count != ctx->params.fluid_count)
        return fail(PCISPH_ERR_INCONSISTENT, "Inconsistent positions_size (" + std::to_string(count) + ") for " +
                                                 std::to_string(ctx->params.fluid_count) + " particles");
    DeviceGuard g(ctx->device);
    uint32_t bk = ctx->params.fluid_count / 2;
    bk -= bk % 64;
    bk = std::max(64u, bk);
    int rc = ctx->ensure_fluid(count, bk);
    if (rc) return rc;
    rc = ctx->copy_vectors_in(ctx->b.state_pos, pos, count, layout, memory);
    if (rc) return rc;
    if (vel) rc = ctx->copy_vectors_in(ctx->b.state_vel, vel, count, layout, memory);
    else if (count) CUDA_TRY(cudaMemsetAsync(ctx->b.state_vel, 0, (size_t)count * 16, ctx->stream()));
    if (rc) return rc;
    if (memory == PCISPH_MEM_HOST) CUDA_TRY(cudaStreamSynchronize(ctx->stream()));
    ctx->fluid_loaded = count;
    return PCISPH_OK;
}

int pcisph_set_boundary_state(pcisph_ctx* ctx, const float* pos, uint32_t count, int layout, int memory) {
    if (!ctx) return fail(PCISPH_ERR_INVALID_ARG, "ctx is NULL");
    if (count && !pos) return fail(PCISPH_ERR_INVALID_ARG, "pos is NULL");
    if (layout != PCISPH_LAYOUT_PACKED3 && layout != PCISPH_LAYOUT_FLOAT4)
        return fail(PCISPH_ERR_INVALID_ARG, "positions take PACKED3 or FLOAT4");
    if (count != ctx->params.boundary_count)
        return fail(PCISPH_ERR_INCONSISTENT, "Inconsistent boundary_positions (" + std::to_string(count) + ") for " +
                                                 std::to_string(ctx->params.boundary_count) + " particles");
    DeviceGuard g(ctx->device);
    uint32_t bk = ctx->params.fluid_count / 2;
    bk -= bk % 64;
    bk = std::max(64u, bk);
    int rc = ctx->ensure_boundary(count, bk);
    if (rc) return rc;
    rc = ctx->copy_vectors_in(ctx->b_pos_in, pos, count, layout, memory);
    if (rc) return rc;
    if (memory == PCISPH_MEM_HOST) CUDA_TRY(cudaStreamSynchronize(ctx->stream()));
    ctx->boundary_loaded = count;
    ctx->boundary_updated = true;
    return PCISPH_OK;
}

int pcisph_check_buffers_consistent(const pcisph_ctx* ctx) {
    if (!ctx) return fail(PCISPH_ERR_INVALID_ARG, "ctx is NULL");
    return ctx->check_consistent();
}

int pcisph_update(pcisph_ctx* ctx) {
    if (!ctx) return fail(PCISPH_ERR_INVALID_ARG, "ctx is NULL");
    DeviceGuard g(ctx->device);
    return ctx->update();
}

int pcisph_step(pcisph_ctx* ctx, uint32_t steps) {
    if (!ctx) return fail(PCISPH_ERR_INVALID_ARG, "ctx is NULL");
    DeviceGuard g(ctx->device);
    for (uint32_t i = 0; i < steps; ++i) {
        int rc = ctx->update();
        if (rc) return rc;
    }
    return PCISPH_OK;
}

int pcisph_sync(pcisph_ctx* ctx) {
    if (!ctx) return fail(PCISPH_ERR_INVALID_ARG, "ctx is NULL");
    DeviceGuard g(ctx->device);
    CUDA_TRY(cudaStreamSynchronize(ctx->stream()));
    return PCISPH_OK;
}

int pcisph_sync_for(pcisph_ctx* ctx, int64_t timeout_ms) {
    if (!ctx) return fail(PCISPH_ERR_INVALID_ARG, "ctx is NULL");
    if (timeout_ms < 0) return fail(PCISPH_ERR_INVALID_ARG, "timeout_ms must be >= 0");
    DeviceGuard g(ctx->device);
    bool done = false;
    CUDA_TRY(host::wait_stream_for(ctx->stream(), timeout_ms, &done));
    if (!done) return fail(PCISPH_ERR_TIMEOUT, "queued steps still running after " + std::to_string(timeout_ms) + " ms");
    return PCISPH_OK;
}

int pcisph_last_stats(pcisph_ctx* ctx, pcisph_step_stats* out) {
    if (!ctx || !out) return fail(PCISPH_ERR_INVALID_ARG, "NULL argument");
    DeviceGuard g(ctx->device);
    return ctx->stats(out);
}

int pcisph_reset_stats(pcisph_ctx* ctx) {
    if (!ctx) return fail(PCISPH_ERR_INVALID_ARG, "ctx is NULL");
    DeviceGuard g(ctx->device);
    CUDA_TRY(cudaStreamSynchronize(ctx->stream()));
    Control h{};
    CUDA_TRY(cudaMemcpy(&h, ctx->ctl, sizeof(Control), cudaMemcpyDeviceToHost));
    // keep the launch count: fold the device-decided loop launches into the host count
    const uint64_t graph_iters = h.total_iters > ctx->host_mode_iters ? h.total_iters - ctx->host_mode_iters : 0;
    ctx->host_launches += graph_iters * (uint64_t)ctx->iter_launches;
    ctx->host_mode_iters = 0;
    Control zero{};
    CUDA_TRY(cudaMemcpy(ctx->ctl, &zero, sizeof(Control), cudaMemcpyHostToDevice));
    return PCISPH_OK;
}

int pcisph_get_field(pcisph_ctx* ctx, int field, void* dst, size_t dst_bytes, int layout, int memory) {
    if (!ctx) return fail(PCISPH_ERR_INVALID_ARG, "ctx is NULL");
    DeviceGuard g(ctx->device);
    return ctx->get_field(field, dst, dst_bytes, layout, memory);
}

int pcisph_set_field(pcisph_ctx* ctx, int field, const void* src, size_t src_bytes, int layout, int memory) {
    if (!ctx) return fail(PCISPH_ERR_INVALID_ARG, "ctx is NULL");
    DeviceGuard g(ctx->device);
    return ctx->set_field(field, src, src_bytes, layout, memory);
}

int pcisph_field_device_ptr(pcisph_ctx* ctx, int field, void** ptr, size_t* count, int* layout) {
    if (!ctx || !ptr) return fail(PCISPH_ERR_INVALID_ARG, "NULL argument");
    pcisph_ctx::FieldView v;
    if (!ctx->field_view(field, &v)) return fail(PCISPH_ERR_INVALID_ARG, "unknown field");
    if (ctx->in_working_order(field) && v.ptr && v.count) {  // a sorted-order copy, made now (stream-ordered)
        DeviceGuard g(ctx->device);
        const size_t esz = v.layout == PCISPH_LAYOUT_FLOAT4 ? 16 : 4;
        DeviceBlock& e = ctx->exports[field];
        if (e.ensure(v.count * esz) != cudaSuccess) return fail(PCISPH_ERR_OOM, "device allocation of a field copy failed");
        if (esz == 16) launch_gather4(static_cast<const float4*>(v.ptr), ctx->w_of_d, static_cast<float4*>(e.p), (uint32_t)v.count, ctx->stream());
        else launch_gather1(static_cast<const float*>(v.ptr), ctx->w_of_d, static_cast<float*>(e.p), (uint32_t)v.count, ctx->stream());
        ++ctx->host_launches;
        CUDA_TRY(cudaGetLastError());
        v.ptr = e.p;
    }
    if (field == PCISPH_FIELD_SORTED_POSITION && ctx->P.particle_skin && v.ptr && v.count) {
        // w of the step's positions holds each particle's half skin: hand out a copy with 0 there
        DeviceGuard g(ctx->device);
        DeviceBlock& e = ctx->exports[field];
        if (e.ensure(v.count * 16) != cudaSuccess) return fail(PCISPH_ERR_OOM, "device allocation of a field copy failed");
        launch_xyz0(static_cast<const float4*>(v.ptr), static_cast<float4*>(e.p), (uint32_t)v.count, ctx->stream());
        ++ctx->host_launches;
        CUDA_TRY(cudaGetLastError());
        v.ptr = e.p;
    }
    *ptr = v.ptr;
    if (count) *count = v.count;
    if (layout) *layout = v.layout;
    return PCISPH_OK;
}

namespace {
struct SnapshotHeader {
    char magic[4];           // "PCSN"
    uint32_t version;        // 1
    uint32_t params_bytes;   // sizeof(pcisph_sim_params)
    uint32_t options_bytes;  // sizeof(pcisph_options)
    uint32_t fluid_count, boundary_count;
    float threshold;
    uint32_t reserved;
    uint64_t steps;
};
size_t snapshot_bytes(uint32_t n, uint32_t b) {
    return sizeof(SnapshotHeader) + sizeof(pcisph_sim_params) + sizeof(pcisph_options) + (size_t)n * 32 +
           (size_t)b * 16;
}
}  // namespace

int pcisph_snapshot_size(pcisph_ctx* ctx, size_t* bytes) {
    if (!ctx || !bytes) return fail(PCISPH_ERR_INVALID_ARG, "NULL argument");
    *bytes = snapshot_bytes(ctx->params.fluid_count, ctx->params.boundary_count);
    return PCISPH_OK;
}

int pcisph_snapshot(pcisph_ctx* ctx, void* dst, size_t dst_bytes) {
    if (!ctx || !dst) return fail(PCISPH_ERR_INVALID_ARG, "NULL argument");
    const uint32_t N = ctx->params.fluid_count, B = ctx->params.boundary_count;
    const size_t need = snapshot_bytes(N, B);
    if (dst_bytes < need) return fail(PCISPH_ERR_INVALID_ARG, "snapshot buffer too small: need " + std::to_string(need));
    if (ctx->fluid_loaded != N || (B && ctx->boundary_loaded != B))
        return fail(PCISPH_ERR_NOT_READY, "no state to snapshot (set the fluid and boundary state first)");
    DeviceGuard g(ctx->device);
    CUDA_TRY(cudaStreamSynchronize(ctx->stream()));
    Control c{};
    CUDA_TRY(cudaMemcpy(&c, ctx->ctl, sizeof(Control), cudaMemcpyDeviceToHost));
    unsigned char* p = static_cast<unsigned char*>(dst);
    SnapshotHeader h{{'P', 'C', 'S', 'N'}, 1u, (uint32_t)sizeof(pcisph_sim_params), (uint32_t)sizeof(pcisph_options),
                     N, B, ctx->threshold, 0u, c.steps};
    std::memcpy(p, &h, sizeof h);
    p += sizeof h;
    std::memcpy(p, &ctx->params, sizeof(pcisph_sim_params));
    p += sizeof(pcisph_sim_params);
    std::memcpy(p, &ctx->opts, sizeof(pcisph_options));
    p += sizeof(pcisph_options);
    if (N) {
        CUDA_TRY(cudaMemcpy(p, ctx->b.state_pos, (size_t)N * 16, cudaMemcpyDeviceToHost));
        CUDA_TRY(cudaMemcpy(p + (size_t)N * 16, ctx->b.state_vel, (size_t)N * 16, cudaMemcpyDeviceToHost));
        p += (size_t)N * 32;
    }
    if (B) CUDA_TRY(cudaMemcpy(p, ctx->b_pos_in, (size_t)B * 16, cudaMemcpyDeviceToHost));
    return PCISPH_OK;
}

int pcisph_restore(pcisph_ctx* ctx, const void* src, size_t src_bytes) {
    if (!ctx || !src) return fail(PCISPH_ERR_INVALID_ARG, "NULL argument");
    SnapshotHeader h;
    if (src_bytes < sizeof h) return fail(PCISPH_ERR_INVALID_ARG, "snapshot truncated");
    std::memcpy(&h, src, sizeof h);
    if (std::memcmp(h.magic, "PCSN", 4) != 0 || h.version != 1u || h.params_bytes != sizeof(pcisph_sim_params) ||
        h.options_bytes != sizeof(pcisph_options))
        return fail(PCISPH_ERR_INVALID_ARG, "not a snapshot of this library version");
    if (src_bytes < snapshot_bytes(h.fluid_count, h.boundary_count))
        return fail(PCISPH_ERR_INVALID_ARG, "snapshot truncated");
    const unsigned char* p = static_cast<const unsigned char*>(src) + sizeof h;
    pcisph_sim_params sp;
    pcisph_options o;
    std::memcpy(&sp, p, sizeof sp);
    p += sizeof sp;
    std::memcpy(&o, p, sizeof o);
    p += sizeof o;
    if (sp.fluid_count != h.fluid_count || sp.boundary_count != h.boundary_count)
        return fail(PCISPH_ERR_INVALID_ARG, "snapshot counts disagree with its parameters");
    int rc = pcisph_set_options(ctx, &o);
    if (rc) return rc;
    // the nine setters (Fluid.h:21-29), then the derivation (which zeroes velocities), then the state
    ctx->params.fluid_count = sp.fluid_count;
    ctx->params.boundary_count = sp.boundary_count;
    ctx->params.delta_t = sp.delta_t;
    ctx->params.rest_density = sp.rest_density;
    ctx->params.particle_radius = sp.particle_radius;
    ctx->params.gravity = sp.gravity;
    ctx->params.viscosity_constant = sp.viscosity_constant;
    ctx->params.surface_tension_coefficient = sp.surface_tension_coefficient;
    ctx->params_changed = true;
    rc = pcisph_set_density_variation_threshold(ctx, h.threshold);
    if (!rc) rc = pcisph_prepare(ctx);
    if (rc) return rc;
    const float* f = reinterpret_cast<const float*>(p);
    rc = pcisph_set_fluid_state(ctx, f, f + (size_t)h.fluid_count * 4, h.fluid_count, PCISPH_LAYOUT_FLOAT4,
                                PCISPH_MEM_HOST);
    if (rc) return rc;
    if (h.boundary_count)
        rc = pcisph_set_boundary_state(ctx, f + (size_t)h.fluid_count * 8, h.boundary_count, PCISPH_LAYOUT_FLOAT4,
                                       PCISPH_MEM_HOST);
    if (rc) return rc;
    // the step counter continues from the checkpoint's (the other statistics start over)
    DeviceGuard g(ctx->device);
    CUDA_TRY(cudaStreamSynchronize(ctx->stream()));
    const unsigned long long steps = h.steps;
    CUDA_TRY(cudaMemcpy(reinterpret_cast<unsigned char*>(ctx->ctl) + offsetof(Control, steps), &steps, sizeof steps,
                        cudaMemcpyHostToDevice));
    return PCISPH_OK;
}

int pcisph_autotune(pcisph_ctx* ctx, uint32_t steps, pcisph_tune_result* out) {
    if (!ctx || !out) return fail(PCISPH_ERR_INVALID_ARG, "NULL argument");
    if (steps == 0 || steps > 1000) return fail(PCISPH_ERR_INVALID_ARG, "steps must be in 1..1000");
    if (ctx->opts.kernel_variant != 2) return fail(PCISPH_ERR_INVALID_ARG, "autotuning covers kernel variant 2");
    if (ctx->params_changed) {
        int rc = ctx->derive_now();
        if (rc) return rc;
    }
    int rc = ctx->check_consistent();
    if (rc) return rc;
    const uint32_t N = ctx->params.fluid_count;
    if (N == 0) return fail(PCISPH_ERR_NOT_READY, "no particles to tune on");
    DeviceGuard g(ctx->device);
    cudaStream_t s = ctx->stream();
    DeviceBlock saved;
    if (saved.ensure((size_t)N * 32) != cudaSuccess) return fail(PCISPH_ERR_OOM, "device allocation for autotuning failed");
    float4* sp = static_cast<float4*>(saved.p);
    CUDA_TRY(cudaMemcpyAsync(sp, ctx->b.state_pos, (size_t)N * 16, cudaMemcpyDeviceToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(sp + N, ctx->b.state_vel, (size_t)N * 16, cudaMemcpyDeviceToDevice, s));
    Control ctl0{};
    CUDA_TRY(cudaStreamSynchronize(s));
    CUDA_TRY(cudaMemcpy(&ctl0, ctx->ctl, sizeof(Control), cudaMemcpyDeviceToHost));
    const uint64_t launches0 = ctx->host_launches, steps0 = ctx->steps_launched, iters0 = ctx->host_mode_iters;
    const pcisph_options entry = ctx->opts;
    const int entry_bits = ctx->sorter.digit_bits();
    const int entry_order = ctx->working_order() ? 1 : 0;  // "auto" as it resolves for this scene
    cudaEvent_t e0, e1;
    CUDA_TRY(cudaEventCreate(&e0));
    CUDA_TRY(cudaEventCreate(&e1));
    auto restore = [&]() -> int {
        CUDA_TRY(cudaMemcpyAsync(ctx->b.state_pos, sp, (size_t)N * 16, cudaMemcpyDeviceToDevice, s));
        CUDA_TRY(cudaMemcpyAsync(ctx->b.state_vel, sp + N, (size_t)N * 16, cudaMemcpyDeviceToDevice, s));
        CUDA_TRY(cudaMemcpyAsync(ctx->ctl, &ctl0, sizeof(Control), cudaMemcpyHostToDevice, s));
        CUDA_TRY(cudaStreamSynchronize(s));
        return PCISPH_OK;
    };
    auto apply = [&](float skin, int order, int bits, int block) -> int {
        pcisph_options o = ctx->opts;
        o.list_skin = skin;
        o.spatial_order = order;
        o.sweep_block = block;
        int r = pcisph_set_options(ctx, &o);
        if (r) return r;
        ctx->sorter.set_digit_bits(bits);
        ctx->sort_block.release();  // scratch size depends on the digit width
        ctx->sorted_keys = ctx->f_keys;  // no view into the released scratch survives
        ctx->sorted_ids = ctx->f_ids;
        ctx->graph_valid = false;
        ctx->order_age = pcisph_ctx::kNoOrder;
        return ctx->ensure_shared(std::max(N, ctx->boundary_cap_n));
    };
    auto time_it = [&](float* ms) -> int {
        int r = restore();
        if (!r) r = ctx->update();  // warm-up: builds the graph
        if (!r) r = restore();
        if (r) return r;
        CUDA_TRY(cudaEventRecord(e0, s));
        for (uint32_t k = 0; k < steps && !r; ++k) r = ctx->update();
        CUDA_TRY(cudaEventRecord(e1, s));
        CUDA_TRY(cudaEventSynchronize(e1));
        if (r) return r;
        CUDA_TRY(cudaEventElapsedTime(ms, e0, e1));
        *ms /= (float)steps;
        return PCISPH_OK;
    };
    float before = 0.f;
    rc = apply(entry.list_skin, entry_order, entry_bits, entry.sweep_block);
    if (!rc) rc = time_it(&before);
    float best_ms = before, best_skin = entry.list_skin;
    int best_order = entry_order, best_bits = entry_bits, n = 1;
    const float skins[] = {0.15f, 0.2f, 0.25f, 0.3f};
    const int orders[] = {1, 0};
    const int bits[] = {8, 10, 6};
    for (float sk : skins)
        for (int od : orders)
            for (int bt : bits) {
                if (rc) break;
                if (sk == entry.list_skin && od == entry_order && bt == entry_bits) continue;
                float ms = 0.f;
                rc = apply(sk, od, bt, entry.sweep_block);
                if (!rc) rc = time_it(&ms);
                ++n;
                if (!rc && ms < best_ms) {
                    best_ms = ms;
                    best_skin = sk;
                    best_order = od;
                    best_bits = bt;
                }
            }
    // then the block size of the corrective-loop sweeps, on the best of the above
    int best_block = entry.sweep_block;
    for (int bl : {128, 256, 512}) {
        if (rc || bl == entry.sweep_block) continue;
        float ms = 0.f;
        rc = apply(best_skin, best_order, best_bits, bl);
        if (!rc) rc = time_it(&ms);
        ++n;
        if (!rc && ms < best_ms) {
            best_ms = ms;
            best_block = bl;
        }
    }
    if (!rc) rc = apply(best_skin, best_order, best_bits, best_block);
    const int rc2 = restore();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    saved.release();
    ctx->host_launches = launches0;
    ctx->steps_launched = steps0;
    ctx->host_mode_iters = iters0;
    if (rc) return rc;
    if (rc2) return rc2;
    out->list_skin = best_skin;
    out->spatial_order = best_order;
    out->digit_bits = best_bits;
    out->sweep_block = best_block;
    out->ms_per_step = best_ms;
    out->ms_per_step_before = before;
    out->candidates = n;
    return PCISPH_OK;
}

int pcisph_render_fluid(pcisph_ctx* ctx, const pcisph_camera* cam, int width, int height, uint8_t* rgb,
                        size_t rgb_bytes) {
    if (!ctx || !cam || !rgb) return fail(PCISPH_ERR_INVALID_ARG, "NULL argument");
    if (width <= 0 || height <= 0 || width > 16384 || height > 16384)
        return fail(PCISPH_ERR_INVALID_ARG, "image size must be in 1..16384");
    const size_t pixels = (size_t)width * height;
    if (rgb_bytes < pixels * 3) return fail(PCISPH_ERR_INVALID_ARG, "rgb buffer needs width * height * 3 bytes");
    const uint32_t N = ctx->params.fluid_count;
    if (N && ctx->fluid_loaded != N) return fail(PCISPH_ERR_NOT_READY, "no fluid state to render");
    DeviceGuard g(ctx->device);
    void* density = nullptr;
    if (N && ctx->b.rho && ctx->steps_launched) {  // densities of the last step, in the state's order
        size_t cnt = 0;
        int rc = pcisph_field_device_ptr(ctx, PCISPH_FIELD_DENSITY, &density, &cnt, nullptr);
        if (rc) return rc;
    }
    DeviceBlock& img = ctx->render_block;
    const size_t zbytes = align256(pixels * 8);
    if (img.ensure(zbytes + pixels * 3) != cudaSuccess) return fail(PCISPH_ERR_OOM, "device allocation of the image failed");
    uint8_t* d_rgb = static_cast<uint8_t*>(img.p) + zbytes;
    int rc = pcisph_render(reinterpret_cast<const float*>(ctx->b.state_pos), static_cast<const float*>(density), N,
                           ctx->params.particle_radius, ctx->params.rest_density, cam, width, height, img.p, zbytes,
                           d_rgb, ctx->stream());
    if (rc) return rc;
    ctx->host_launches += 2;
    CUDA_TRY(cudaMemcpyAsync(rgb, d_rgb, pixels * 3, cudaMemcpyDeviceToHost, ctx->stream()));
    CUDA_TRY(cudaStreamSynchronize(ctx->stream()));
    return PCISPH_OK;
}

int pcisph_run_stage(pcisph_ctx* ctx, int stage, int arg) {
    if (!ctx) return fail(PCISPH_ERR_INVALID_ARG, "ctx is NULL");
    DeviceGuard g(ctx->device);
    return ctx->run_stage(stage, arg);
}

uint64_t pcisph_kernel_launches(const pcisph_ctx* ctx) {
    if (!ctx) return 0;
    // host-counted launches plus the corrective-loop kernels the device decided to run
    DeviceGuard g(ctx->device);
    cudaStreamSynchronize(ctx->stream());
    Control h{};
    cudaMemcpy(&h, ctx->ctl, sizeof(Control), cudaMemcpyDeviceToHost);
    const uint64_t graph_iters = h.total_iters > ctx->host_mode_iters ? h.total_iters - ctx->host_mode_iters : 0;
    return ctx->host_launches + graph_iters * (uint64_t)ctx->iter_launches;
}

int pcisph_profile_enable(pcisph_ctx* ctx, int enable) {
    if (!ctx) return fail(PCISPH_ERR_INVALID_ARG, "ctx is NULL");
    ctx->profiling = enable != 0;
    if (enable) ctx->timer.clear();
    return PCISPH_OK;
}

int pcisph_profile_read(pcisph_ctx* ctx, pcisph_kernel_time* out, int max_entries, int* n_entries) {
    if (!ctx) return fail(PCISPH_ERR_INVALID_ARG, "ctx is NULL");
    DeviceGuard g(ctx->device);
    ctx->collect_timings();
    const int n = ctx->timer.read(out, max_entries);
    if (n_entries) *n_entries = n;
    return PCISPH_OK;
}

int pcisph_hash_keys(const pcisph_sim_params* params, const float* pos, int layout, uint32_t count, uint32_t* keys,
                     uint32_t* ids, void* stream) {
    if (!params || (count && (!pos || !keys))) return fail(PCISPH_ERR_INVALID_ARG, "NULL argument");
    if (params->bucket_count < 2) return fail(PCISPH_ERR_INVALID_ARG, "bucket_count must be >= 2");
    if (layout != PCISPH_LAYOUT_PACKED3 && layout != PCISPH_LAYOUT_FLOAT4)
        return fail(PCISPH_ERR_INVALID_ARG, "positions take PACKED3 or FLOAT4");
    DevParams P{};
    P.cell_size = params->cell_size;
    P.bucket_count = params->bucket_count;
    magic_for(params->bucket_count, &P.bk_magic, &P.bk_shift);
    launch_hash(pos, layout == PCISPH_LAYOUT_PACKED3, count, P, keys, ids, static_cast<cudaStream_t>(stream));
    CUDA_TRY(cudaGetLastError());
    return PCISPH_OK;
}

struct pcisph_radixsort {
    int device;
    RadixSorter sorter;
};

int pcisph_radixsort_create(int device, pcisph_radixsort** out) {
    if (!out) return fail(PCISPH_ERR_INVALID_ARG, "out is NULL");
    DeviceGuard g(device);
    CUDA_TRY(cudaFree(nullptr));
    CUDA_TRY(radix_configure_kernels());
    *out = new pcisph_radixsort{device, {}};
    return PCISPH_OK;
}

void pcisph_radixsort_destroy(pcisph_radixsort* s) {
    if (!s) return;
    DeviceGuard g(s->device);
    delete s;
}

int pcisph_radixsort_set_digit_bits(pcisph_radixsort* s, int bits) {
    if (!s) return fail(PCISPH_ERR_INVALID_ARG, "sorter is NULL");
    if (bits == 0) bits = 8;
    if (bits < 4 || bits > 11) return fail(PCISPH_ERR_INVALID_ARG, "digit bits must be in 4..11");
    s->sorter.set_digit_bits(bits);
    return PCISPH_OK;
}

int pcisph_radixsort_enqueue(pcisph_radixsort* s, uint32_t* keys, uint32_t* values, size_t elements,
                             unsigned int max_bits, void* stream) {
    if (!s) return fail(PCISPH_ERR_INVALID_ARG, "sorter is NULL");
    if (elements && (!keys || !values)) return fail(PCISPH_ERR_INVALID_ARG, "keys/values are NULL");
    if (max_bits > 32) return fail(PCISPH_ERR_INVALID_ARG, "max_bits > 32");
    DeviceGuard g(s->device);
    cudaError_t e = s->sorter.sort(keys, values, elements, max_bits == 0 ? 32 : (int)max_bits, false,
                                   static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(PCISPH_ERR_CUDA, std::string("radix sort: ") + cudaGetErrorString(e));
    return PCISPH_OK;
}

}  // extern "C"
