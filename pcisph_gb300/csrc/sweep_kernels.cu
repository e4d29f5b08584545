// sweep_kernels.cu -- the fluid neighbour sweeps of the step on the warp-per-bucket
// machinery of sweep.cuh. Pair terms and epilogues are those of the per-particle
// kernels in step_kernels.cu (PCISPH/data/kernels/pcisph.cl expressions); only the
// mapping of work to threads differs.
#include <algorithm>

#include "pair_terms.cuh"
#include "step_kernels.cuh"
#include "sweep.cuh"

namespace pcisph {
namespace {

__device__ __forceinline__ float4 shfl4(const float4& v, int src) {
    return make_float4(__shfl_sync(kFull, v.x, src), __shfl_sync(kFull, v.y, src), __shfl_sync(kFull, v.z, src),
                       __shfl_sync(kFull, v.w, src));
}
__device__ __forceinline__ float3 shfl3(const float3& v, int src) {
    return make_float3(__shfl_sync(kFull, v.x, src), __shfl_sync(kFull, v.y, src), __shfl_sync(kFull, v.z, src));
}
__device__ __forceinline__ float3 shfl3_down(const float3& v, int off) {
    return make_float3(__shfl_down_sync(kFull, v.x, off), __shfl_down_sync(kFull, v.y, off),
                       __shfl_down_sync(kFull, v.z, off));
}

struct NoResult {};

// ------------------------------------------------------------------ density (pcisph.cl:65-92)
struct OpDensity {
    using Cand = float4;
    using Self = float4;
    using Acc = float;
    using Result = NoResult;
    const float4* pos;
    const float4* b_pos;
    float* rho;
    float4* pr4;
    __device__ static Self empty_self() { return make_float4(0.f, 0.f, 0.f, 0.f); }
    __device__ static Result no_result() { return {}; }
    __device__ static void combine(Result&, const Result&) {}
    __device__ Self load_self(uint32_t i) const { return pos[i]; }
    __device__ static float3 cell_pos(const Self& s) { return make_float3(s.x, s.y, s.z); }
    __device__ Cand load_fluid(uint32_t j) const { return __ldg(&pos[j]); }
    __device__ Cand load_boundary(uint32_t j) const { return __ldg(&b_pos[j]); }
    __device__ static Self shfl(const Self& s, int src) { return shfl4(s, src); }
    __device__ static Acc shfl(const Acc& a, int src) { return __shfl_sync(kFull, a, src); }
    __device__ static Acc shfl_down(const Acc& a, int off) { return __shfl_down_sync(kFull, a, off); }
    __device__ static void zero(Acc& a) { a = 0.f; }
    __device__ static void add(Acc& a, const Acc& b) { a += b; }
    __device__ void begin(const DevParams&) const {}
    __device__ void end(const DevParams&, const Result&) const {}
    __device__ __forceinline__ void pair(const DevParams& P, const Self& s, const Cand& o, Acc& a) const {
        const float dx = s.x - o.x, dy = s.y - o.y, dz = s.z - o.z;
        a += poly6(dist2(dx, dy, dz), P.h2);
    }
    __device__ Result finish(const DevParams& P, uint32_t i, const Self& s, const Acc& a) const {
        const float r = a * (P.particle_mass * P.poly6_norm);
        rho[i] = r;
        pr4[i] = make_float4(s.x, s.y, s.z, r);
        return {};
    }
};

// ------------------------------------------------------------------- normal (pcisph.cl:94-112)
struct OpNormal {
    using Cand = float4;
    using Self = float4;
    using Acc = float3;
    using Result = NoResult;
    const float4* pr4;
    float4* normal;
    __device__ static Self empty_self() { return make_float4(0.f, 0.f, 0.f, 0.f); }
    __device__ static Result no_result() { return {}; }
    __device__ static void combine(Result&, const Result&) {}
    __device__ Self load_self(uint32_t i) const { return pr4[i]; }
    __device__ static float3 cell_pos(const Self& s) { return make_float3(s.x, s.y, s.z); }
    __device__ Cand load_fluid(uint32_t j) const { return __ldg(&pr4[j]); }
    __device__ Cand load_boundary(uint32_t) const { return make_float4(1e30f, 1e30f, 1e30f, 1.f); }
    __device__ static Self shfl(const Self& s, int src) { return shfl4(s, src); }
    __device__ static Acc shfl(const Acc& a, int src) { return shfl3(a, src); }
    __device__ static Acc shfl_down(const Acc& a, int off) { return shfl3_down(a, off); }
    __device__ static void zero(Acc& a) { a = make_float3(0.f, 0.f, 0.f); }
    __device__ static void add(Acc& a, const Acc& b) { a = a + b; }
    __device__ void begin(const DevParams&) const {}
    __device__ void end(const DevParams&, const Result&) const {}
    __device__ __forceinline__ void pair(const DevParams& P, const Self& s, const Cand& o, Acc& a) const {
        normal_term(s.x, s.y, s.z, o, P.h2, a);
    }
    __device__ Result finish(const DevParams& P, uint32_t i, const Self&, const Acc& a) const {
        const float scale = P.h * P.particle_mass * P.poly6_d1_norm;
        normal[i] = make_float4(a.x * scale, a.y * scale, a.z * scale, 0.f);
        return {};
    }
};

// -------------------------------------------------------- force (pcisph.cl:121-173) + first predict
struct ForceCand {
    float4 xr;   // x, rho
    float4 v;    // velocity
    float4 n;    // normal
};
struct ForceSelf {
    float4 xr;
    float3 v, n;
};
using ForceAcc = ForceAccum;
struct OpForce {
    using Cand = ForceCand;
    using Self = ForceSelf;
    using Acc = ForceAcc;
    using Result = NoResult;
    const float4* pr4;
    const float4* vel;
    const float4* normal;
    float4* f_other;
    float* press;
    float4* pred;
    __device__ static Self empty_self() { return Self{make_float4(0.f, 0.f, 0.f, 1.f), make_float3(0.f, 0.f, 0.f), make_float3(0.f, 0.f, 0.f)}; }
    __device__ static Result no_result() { return {}; }
    __device__ static void combine(Result&, const Result&) {}
    __device__ Self load_self(uint32_t i) const { return Self{pr4[i], f3(vel[i]), f3(normal[i])}; }
    __device__ static float3 cell_pos(const Self& s) { return make_float3(s.xr.x, s.xr.y, s.xr.z); }
    __device__ Cand load_fluid(uint32_t j) const { return Cand{__ldg(&pr4[j]), __ldg(&vel[j]), __ldg(&normal[j])}; }
    __device__ Cand load_boundary(uint32_t) const { return Cand{make_float4(1e30f, 1e30f, 1e30f, 1.f), make_float4(0.f, 0.f, 0.f, 0.f), make_float4(0.f, 0.f, 0.f, 0.f)}; }
    __device__ static Self shfl(const Self& s, int src) { return Self{shfl4(s.xr, src), shfl3(s.v, src), shfl3(s.n, src)}; }
    __device__ static Acc shfl(const Acc& a, int src) { return Acc{shfl3(a.visc, src), shfl3(a.coh, src), shfl3(a.curv, src)}; }
    __device__ static Acc shfl_down(const Acc& a, int off) { return Acc{shfl3_down(a.visc, off), shfl3_down(a.coh, off), shfl3_down(a.curv, off)}; }
    __device__ static void zero(Acc& a) { a.visc = a.coh = a.curv = make_float3(0.f, 0.f, 0.f); }
    __device__ static void add(Acc& a, const Acc& b) { a.visc = a.visc + b.visc; a.coh = a.coh + b.coh; a.curv = a.curv + b.curv; }
    __device__ void begin(const DevParams&) const {}
    __device__ void end(const DevParams&, const Result&) const {}
    __device__ __forceinline__ void pair(const DevParams& P, const Self& s, const Cand& o, Acc& a) const {
        force_term(s.xr, s.v, s.n, o.xr, f3(o.v), f3(o.n), P, a);
    }
    __device__ Result finish(const DevParams& P, uint32_t i, const Self& s, const Acc& a) const {
        const float m = P.particle_mass;
        const float3 fo = other_force(m, P.gravity, a.visc, P.viscosity * m * P.visc_d2_norm, a.coh,
                                      -P.st_coeff * m * m * P.st_norm, a.curv, -P.st_coeff * m);
        f_other[i] = f4(fo, 0.f);
        press[i] = 0.f;
        const float3 v = s.v + (fo / m) * P.dt;
        const float3 x = make_float3(s.xr.x, s.xr.y, s.xr.z) + v * P.dt;
        pred[i] = f4(x, 0.f);
        return {};
    }
};

// ------------------------------------------- pressure (pcisph.cl:212-263) + stop decision
struct PressSelf {
    float4 x;    // current position: selects the cells (pcisph.cl:238, :246)
    float4 xp;   // predicted position: distances (pcisph.cl:240, :248)
};
struct OpPressure {
    using Cand = float4;
    using Self = PressSelf;
    using Acc = float;
    using Result = float;  // density variation, for the max
    const float4* pos;
    const float4* pred;
    const float4* b_pos;
    const float* rho;
    float* press;
    float* err;
    float4* pf4;
    Control* ctl;
    __device__ static Self empty_self() { return Self{make_float4(0.f, 0.f, 0.f, 0.f), make_float4(0.f, 0.f, 0.f, 0.f)}; }
    __device__ static Result no_result() { return 0.f; }
    __device__ static void combine(Result& a, const Result& b) { a = fmaxf(a, b); }
    __device__ Self load_self(uint32_t i) const { return Self{pos[i], pred[i]}; }
    __device__ static float3 cell_pos(const Self& s) { return make_float3(s.x.x, s.x.y, s.x.z); }
    __device__ Cand load_fluid(uint32_t j) const { return __ldg(&pred[j]); }
    __device__ Cand load_boundary(uint32_t j) const { return __ldg(&b_pos[j]); }
    __device__ static Self shfl(const Self& s, int src) { return Self{shfl4(s.x, src), shfl4(s.xp, src)}; }
    __device__ static Acc shfl(const Acc& a, int src) { return __shfl_sync(kFull, a, src); }
    __device__ static Acc shfl_down(const Acc& a, int off) { return __shfl_down_sync(kFull, a, off); }
    __device__ static void zero(Acc& a) { a = 0.f; }
    __device__ static void add(Acc& a, const Acc& b) { a += b; }
    __device__ void begin(const DevParams&) const {}
    __device__ __forceinline__ void pair(const DevParams& P, const Self& s, const Cand& o, Acc& a) const {
        const float dx = s.xp.x - o.x, dy = s.xp.y - o.y, dz = s.xp.z - o.z;
        a += poly6(dist2(dx, dy, dz), P.h2);
    }
    __device__ Result finish(const DevParams& P, uint32_t i, const Self& s, const Acc& a) const {
        const float rs = a * (P.particle_mass * P.poly6_norm);
        if (!isfinite(rs)) atomicOr(&ctl->status, 2u);
        float dv = rs - P.rest_density;
        dv = 0.f < dv ? dv : 0.f;
        err[i] = dv;
        float p = press[i];
        if (dv != 0.f) {
            p += dv * P.delta;
            press[i] = p;
        }
        const float r = rho[i];
        pf4[i] = make_float4(s.x.x, s.x.y, s.x.z, p / (r * r));
        return dv;
    }
    // block max + last-block decision, as k_pressure in step_kernels.cu
    __device__ void end(const DevParams& P, const Result& dv) const {
        unsigned bits = __reduce_max_sync(kFull, __float_as_uint(dv));
        __shared__ unsigned warp_max[32];
        __shared__ bool is_last;
        const int nwarps = blockDim.x >> 5;
        if ((threadIdx.x & 31) == 0) warp_max[threadIdx.x >> 5] = bits;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned m = 0;
            for (int w = 0; w < nwarps; ++w) m = max(m, warp_max[w]);
            atomicMax(&ctl->max_err_bits, m);
            __threadfence();
            is_last = atomicAdd(&ctl->blocks_done, 1u) == gridDim.x - 1;
        }
        __syncthreads();
        if (is_last && threadIdx.x == 0) {
            __threadfence();
            const float mx = __uint_as_float(atomicAdd(&ctl->max_err_bits, 0u));
            const unsigned it = ctl->iter + 1;
            const float rel = mx / P.rest_density;
            const bool converged = rel < P.threshold;
            const bool done = it >= (unsigned)P.max_iters || (it >= (unsigned)P.min_iters && converged);
            ctl->iter = it;
            ctl->done = done ? 1u : 0u;
            ctl->max_err_bits = 0;
            ctl->blocks_done = 0;
            if (done) close_step(ctl, it, rel, converged);
        }
    }
};

// ------------------------------------- pressure force (pcisph.cl:265-300) + predict / integrate
struct OpPressureForce {
    using Cand = float4;
    using Self = float4;
    using Acc = float3;
    using Result = NoResult;
    const float4* pf4;
    const float4* bpf;
    const float4* vel;
    const float4* f_other;
    float4* f_press;
    float4* pred;
    float4* state_pos;
    float4* state_vel;
    Control* ctl;
    int mode;
    cudaGraphConditionalHandle cond;
    int use_cond;
    __device__ static Self empty_self() { return make_float4(0.f, 0.f, 0.f, 0.f); }
    __device__ static Result no_result() { return {}; }
    __device__ static void combine(Result&, const Result&) {}
    __device__ Self load_self(uint32_t i) const { return pf4[i]; }
    __device__ static float3 cell_pos(const Self& s) { return make_float3(s.x, s.y, s.z); }
    __device__ Cand load_fluid(uint32_t j) const { return __ldg(&pf4[j]); }
    __device__ Cand load_boundary(uint32_t j) const { return __ldg(&bpf[j]); }
    __device__ static Self shfl(const Self& s, int src) { return shfl4(s, src); }
    __device__ static Acc shfl(const Acc& a, int src) { return shfl3(a, src); }
    __device__ static Acc shfl_down(const Acc& a, int off) { return shfl3_down(a, off); }
    __device__ static void zero(Acc& a) { a = make_float3(0.f, 0.f, 0.f); }
    __device__ static void add(Acc& a, const Acc& b) { a = a + b; }
    __device__ void begin(const DevParams& P) const {
        if (use_cond && blockIdx.x == 0 && threadIdx.x == 0) {
            // continue the graph's while loop unless the step is done; the counter bounds it on its own
            const unsigned g = ++ctl->guard_iters;
            const bool stop = ctl->done != 0u || g >= (unsigned)P.max_iters;
            cudaGraphSetConditional(cond, stop ? 0u : 1u);
        }
    }
    __device__ void end(const DevParams&, const Result&) const {}
    __device__ __forceinline__ void pair(const DevParams& P, const Self& s, const Cand& o, Acc& a) const {
        pressure_force_term(s, o, P.h, P.h2, a);
    }
    __device__ Result finish(const DevParams& P, uint32_t i, const Self& s, const Acc& a) const {
        const float m = P.particle_mass;
        const float scale = -P.spiky_d1_norm * m * m;
        const float3 fp = make_float3(a.x * scale, a.y * scale, a.z * scale);
        f_press[i] = f4(fp, 0.f);
        const bool integrate = mode == 0 ? (ctl->done != 0u) : mode == 2;
        const float3 acc = (f3(f_other[i]) + fp) / m;
        float3 v = f3(vel[i]) + acc * P.dt;
        float3 x = make_float3(s.x, s.y, s.z) + v * P.dt;
        if (!integrate) {
            pred[i] = f4(x, 0.f);
            return {};
        }
        if (P.walls) {
            float* xs[3] = {&x.x, &x.y, &x.z};
            float* vs[3] = {&v.x, &v.y, &v.z};
#pragma unroll
            for (int ax = 0; ax < 3; ++ax) {
                if (*xs[ax] < P.box_lo[ax]) {
                    *xs[ax] = P.box_lo[ax];
                    if (*vs[ax] < 0.f) *vs[ax] = -P.restitution * *vs[ax];
                } else if (*xs[ax] > P.box_hi[ax]) {
                    *xs[ax] = P.box_hi[ax];
                    if (*vs[ax] > 0.f) *vs[ax] = -P.restitution * *vs[ax];
                }
            }
        }
        state_pos[i] = f4(x, 0.f);
        state_vel[i] = f4(v, 0.f);
        return {};
    }
};

// 16-byte candidates: 8 warps, 256 staged per warp; force candidates: 4 warps, 160 staged.
constexpr int kW16 = 8, kC16 = 256, kWF = 4, kCF = 160;

template <class Op, int W, int CAPC>
void launch_sweep(const DevParams& P, const Op& op, const SweepArgs& A, int grid, cudaStream_t s) {
    k_sweep<Op, W, CAPC><<<grid, W * 32, sweep_smem_bytes<Op, W, CAPC>(), s>>>(P, op, A);
}

template <class Op, int W, int CAPC>
cudaError_t configure_sweep(int* blocks_per_sm) {
    const size_t smem = sweep_smem_bytes<Op, W, CAPC>();
    cudaError_t e = cudaSuccess;
    if (smem > 48 * 1024)
        e = cudaFuncSetAttribute(k_sweep<Op, W, CAPC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_sweep<Op, W, CAPC>, W * 32, smem);
}

}  // namespace

cudaError_t sweep_configure(SweepGrid* g) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    int occ[5] = {0, 0, 0, 0, 0};
    if ((e = configure_sweep<OpDensity, kW16, kC16>(&occ[0])) != cudaSuccess) return e;
    if ((e = configure_sweep<OpNormal, kW16, kC16>(&occ[1])) != cudaSuccess) return e;
    if ((e = configure_sweep<OpForce, kWF, kCF>(&occ[2])) != cudaSuccess) return e;
    if ((e = configure_sweep<OpPressure, kW16, kC16>(&occ[3])) != cudaSuccess) return e;
    if ((e = configure_sweep<OpPressureForce, kW16, kC16>(&occ[4])) != cudaSuccess) return e;
    for (int k = 0; k < 5; ++k) g->blocks[k] = sms * (occ[k] > 0 ? occ[k] : 1);
    g->warps[0] = g->warps[1] = g->warps[3] = g->warps[4] = kW16;
    g->warps[2] = kWF;
    return cudaSuccess;
}

static inline int sweep_grid(const SweepGrid& g, int k, uint32_t max_groups) {
    const uint32_t need = (max_groups + g.warps[k] - 1) / g.warps[k];
    return (int)std::max<uint32_t>(1u, std::min<uint32_t>(need, (uint32_t)g.blocks[k]));
}

void launch_density_sweep(const DevParams& P, const StepBuffers& b, const SweepArgs& A, const SweepGrid& g,
                          cudaStream_t s) {
    launch_sweep<OpDensity, kW16, kC16>(P, OpDensity{b.pos, b.b_pos, b.rho, b.pr4}, A, sweep_grid(g, 0, P.fluid_count), s);
}

void launch_normal_sweep(const DevParams& P, const StepBuffers& b, const SweepArgs& A, const SweepGrid& g,
                         cudaStream_t s) {
    SweepArgs a = A;
    a.b_cells = A.cells;  // the normal sums fluid only: give the boundary side empty ranges
    DevParams Q = P;
    Q.boundary_count = 0;
    launch_sweep<OpNormal, kW16, kC16>(Q, OpNormal{b.pr4, b.normal}, a, sweep_grid(g, 1, P.fluid_count), s);
}

void launch_force_sweep(const DevParams& P, const StepBuffers& b, const SweepArgs& A, const SweepGrid& g,
                        cudaStream_t s) {
    DevParams Q = P;
    Q.boundary_count = 0;  // the force sums fluid only (pcisph.cl:137)
    launch_sweep<OpForce, kWF, kCF>(Q, OpForce{b.pr4, b.vel, b.normal, b.f_other, b.press, b.pred}, A,
                                    sweep_grid(g, 2, P.fluid_count), s);
}

void launch_pressure_sweep(const DevParams& P, const StepBuffers& b, const SweepArgs& A, const SweepGrid& g,
                           cudaStream_t s) {
    launch_sweep<OpPressure, kW16, kC16>(P, OpPressure{b.pos, b.pred, b.b_pos, b.rho, b.press, b.err, b.pf4, b.ctl},
                                         A, sweep_grid(g, 3, P.fluid_count), s);
}

void launch_pressure_force_sweep(const DevParams& P, const StepBuffers& b, const SweepArgs& A, const SweepGrid& g,
                                 int mode, cudaGraphConditionalHandle cond, bool use_cond, cudaStream_t s) {
    launch_sweep<OpPressureForce, kW16, kC16>(
        P, OpPressureForce{b.pf4, b.bpf, b.vel, b.f_other, b.f_press, b.pred, b.state_pos, b.state_vel, b.ctl, mode, cond,
                           use_cond ? 1 : 0},
        A, sweep_grid(g, 4, P.fluid_count), s);
}

}  // namespace pcisph
