// render.cu -- headless particle rendering into an RGB8 image on the device (C ABI in pcisph_gpu.h).
//
// Replaces the reference's OpenGL render_fluid_simple (PCISPH/src/vis/fluid_rendering.cpp:65-103 with
// data/shaders/simple_particle.vert and .frag): every fluid particle is a sphere of the particle radius,
// coloured by its density (blue at 0.95 rho0, purple at rho0, orange at 1.05 rho0, linear in between,
// simple_particle.vert:19-32), lit by max(0, n . y) plus 0.2 ambient and darkened with view depth between
// 5 and 20 (simple_particle.frag). The camera is the reference's: horizontal field of view, eye looking at
// the origin (main.cpp:174-179). Spheres are drawn as ray-cast impostors: pass 1 writes the nearest
// (depth, particle) per pixel with a 64-bit atomicMin, pass 2 shades each covered pixel from that
// particle's sphere.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <string>

#include "../../include/pcisph_gpu.h"
#include "host_util.h"

namespace pcisph {
namespace {

constexpr int kBlock = 256;

struct Camera {
    float3 eye, right, up, fwd;  // orthonormal basis; fwd points from the eye into the scene
    float tan_half_x, tan_half_y;
    float radius, rho_min, rho_neutral, rho_max;
    int width, height;
};

__device__ __forceinline__ float dot3f(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// view coordinates (x right, y up, z depth along fwd) of p
__device__ __forceinline__ float3 to_view(const Camera& c, float3 p) {
    const float3 d = make_float3(p.x - c.eye.x, p.y - c.eye.y, p.z - c.eye.z);
    return make_float3(dot3f(d, c.right), dot3f(d, c.up), dot3f(d, c.fwd));
}

// pixel coordinates of a view-space point (z > 0)
__device__ __forceinline__ float2 to_pixel(const Camera& c, float3 v) {
    const float nx = v.x / (v.z * c.tan_half_x), ny = v.y / (v.z * c.tan_half_y);
    return make_float2((nx + 1.f) * 0.5f * c.width, (1.f - ny) * 0.5f * c.height);
}

// ray from the eye through the centre of pixel (px, py), in view space (z = 1)
__device__ __forceinline__ float3 pixel_ray(const Camera& c, int px, int py) {
    const float nx = ((px + 0.5f) / c.width) * 2.f - 1.f, ny = 1.f - ((py + 0.5f) / c.height) * 2.f;
    return make_float3(nx * c.tan_half_x, ny * c.tan_half_y, 1.f);
}

// distance t along ray r (from the origin) to the sphere of radius R at s, or -1
__device__ __forceinline__ float hit(float3 r, float3 s, float R) {
    const float rr = dot3f(r, r), rs = dot3f(r, s), ss = dot3f(s, s);
    const float disc = rs * rs - rr * (ss - R * R);
    if (disc < 0.f) return -1.f;
    return (rs - sqrtf(disc)) / rr;
}

__global__ void __launch_bounds__(kBlock) k_splat(const float4* __restrict__ pos, uint32_t n, Camera c,
                                                  unsigned long long* __restrict__ zbuf) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= n) return;
    const float4 p = pos[i];
    const float3 v = to_view(c, make_float3(p.x, p.y, p.z));
    if (!(v.z > c.radius)) return;  // behind the eye (or not finite)
    const float2 q = to_pixel(c, v);
    const float rpx = c.radius / (v.z * c.tan_half_x) * 0.5f * c.width + 1.f;
    const int x0 = max(0, (int)floorf(q.x - rpx)), x1 = min(c.width - 1, (int)ceilf(q.x + rpx));
    const int y0 = max(0, (int)floorf(q.y - rpx)), y1 = min(c.height - 1, (int)ceilf(q.y + rpx));
    if (x0 > x1 || y0 > y1 || (x1 - x0) > 256 || (y1 - y0) > 256) return;  // off screen, or too close
    for (int py = y0; py <= y1; ++py)
        for (int px = x0; px <= x1; ++px) {
            const float3 r = pixel_ray(c, px, py);
            const float t = hit(r, v, c.radius);
            if (t <= 0.f) continue;
            const float depth = t * r.z;  // view depth of the hit point
            const unsigned long long key = ((unsigned long long)__float_as_uint(depth) << 32) | i;
            atomicMin(&zbuf[(size_t)py * c.width + px], key);
        }
}

__device__ __forceinline__ float3 mix3(float3 a, float3 b, float f) {
    return make_float3(a.x + (b.x - a.x) * f, a.y + (b.y - a.y) * f, a.z + (b.z - a.z) * f);
}

__global__ void __launch_bounds__(kBlock) k_shade(const float4* __restrict__ pos, const float* __restrict__ density,
                                                  uint32_t n, Camera c, const unsigned long long* __restrict__ zbuf,
                                                  uint8_t* __restrict__ rgb) {
    const uint32_t pix = blockIdx.x * kBlock + threadIdx.x;
    if (pix >= (uint32_t)(c.width * c.height)) return;
    const unsigned long long key = zbuf[pix];
    float3 color = make_float3(0.f, 0.f, 0.f);
    const uint32_t i = (uint32_t)(key & 0xFFFFFFFFull);
    if (key != ~0ull && i < n) {
        const int px = pix % c.width, py = pix / c.width;
        const float4 p = pos[i];
        const float3 v = to_view(c, make_float3(p.x, p.y, p.z));
        const float3 r = pixel_ray(c, px, py);
        const float t = fmaxf(hit(r, v, c.radius), 0.f);
        const float3 h = make_float3(r.x * t - v.x, r.y * t - v.y, r.z * t - v.z);  // hit - centre, view space
        const float inv = 1.f / c.radius;
        // world-space normal: view x, y, z map to right, up, fwd
        const float3 nrm = make_float3((h.x * c.right.x + h.y * c.up.x + h.z * c.fwd.x) * inv,
                                       (h.x * c.right.y + h.y * c.up.y + h.z * c.fwd.y) * inv,
                                       (h.x * c.right.z + h.y * c.up.z + h.z * c.fwd.z) * inv);
        const float rho = density ? density[i] : c.rho_neutral;
        const float3 cmax = make_float3(1.f, 0.3f, 0.f), cneu = make_float3(0.5f, 0.3f, 0.5f),
                     cmin = make_float3(0.f, 0.3f, 1.f);
        float3 diffuse;
        if (rho > c.rho_neutral)
            diffuse = mix3(cneu, cmax, fminf(fmaxf((rho - c.rho_neutral) / (c.rho_max - c.rho_neutral), 0.f), 1.f));
        else
            diffuse = mix3(cmin, cneu, fminf(fmaxf((rho - c.rho_min) / (c.rho_neutral - c.rho_min), 0.f), 1.f));
        const float light = fmaxf(0.f, nrm.y);
        const float depth = t * r.z;
        const float falloff = 1.f - (depth - 5.f) / (20.f - 5.f);
        color = make_float3((light * diffuse.x + 0.2f) * falloff, (light * diffuse.y + 0.2f) * falloff,
                            (light * diffuse.z + 0.2f) * falloff);
    }
    const auto to8 = [](float x) { return (uint8_t)(fminf(fmaxf(x, 0.f), 1.f) * 255.f + 0.5f); };
    rgb[3 * (size_t)pix + 0] = to8(color.x);
    rgb[3 * (size_t)pix + 1] = to8(color.y);
    rgb[3 * (size_t)pix + 2] = to8(color.z);
}

}  // namespace
}  // namespace pcisph

using namespace pcisph;

extern "C" int pcisph_render(const float* pos4, const float* density, uint32_t n, float particle_radius,
                             float rest_density, const pcisph_camera* cam, int width, int height,
                             void* zbuffer, size_t zbuffer_bytes, uint8_t* rgb, void* stream) {
    if (!cam || !rgb || !zbuffer || (n && !pos4)) return report_error(PCISPH_ERR_INVALID_ARG, "NULL argument");
    if (width <= 0 || height <= 0 || width > 16384 || height > 16384)
        return report_error(PCISPH_ERR_INVALID_ARG, "image size must be in 1..16384");
    if (zbuffer_bytes < (size_t)width * height * 8)
        return report_error(PCISPH_ERR_INVALID_ARG, "zbuffer needs width * height * 8 bytes");
    if (!(cam->fov_x_degrees > 0.f && cam->fov_x_degrees < 179.f))
        return report_error(PCISPH_ERR_INVALID_ARG, "fov_x_degrees must be in (0, 179)");
    Camera c{};
    const float3 eye = make_float3(cam->eye[0], cam->eye[1], cam->eye[2]);
    float3 f = make_float3(cam->target[0] - eye.x, cam->target[1] - eye.y, cam->target[2] - eye.z);
    const float fl = std::sqrt(f.x * f.x + f.y * f.y + f.z * f.z);
    if (!(fl > 0.f)) return report_error(PCISPH_ERR_INVALID_ARG, "eye and target coincide");
    f = make_float3(f.x / fl, f.y / fl, f.z / fl);
    const float3 up0 = make_float3(cam->up[0], cam->up[1], cam->up[2]);
    float3 r = make_float3(f.y * up0.z - f.z * up0.y, f.z * up0.x - f.x * up0.z, f.x * up0.y - f.y * up0.x);
    const float rl = std::sqrt(r.x * r.x + r.y * r.y + r.z * r.z);
    if (!(rl > 0.f)) return report_error(PCISPH_ERR_INVALID_ARG, "up is parallel to the view direction");
    r = make_float3(r.x / rl, r.y / rl, r.z / rl);
    const float3 u = make_float3(r.y * f.z - r.z * f.y, r.z * f.x - r.x * f.z, r.x * f.y - r.y * f.x);
    c.eye = eye;
    c.right = r;
    c.up = u;
    c.fwd = f;
    c.tan_half_x = std::tan(0.5f * cam->fov_x_degrees * host::kPi / 180.f);
    c.tan_half_y = c.tan_half_x * (float)height / (float)width;
    c.radius = particle_radius;
    c.rho_min = 0.95f * rest_density;
    c.rho_neutral = rest_density;
    c.rho_max = 1.05f * rest_density;
    c.width = width;
    c.height = height;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaMemsetAsync(zbuffer, 0xFF, (size_t)width * height * 8, s);
    if (e != cudaSuccess) return report_error(PCISPH_ERR_CUDA, std::string("render: ") + cudaGetErrorString(e));
    auto* z = static_cast<unsigned long long*>(zbuffer);
    if (n) k_splat<<<(n + kBlock - 1) / kBlock, kBlock, 0, s>>>(reinterpret_cast<const float4*>(pos4), n, c, z);
    const uint32_t pixels = (uint32_t)width * (uint32_t)height;
    k_shade<<<(pixels + kBlock - 1) / kBlock, kBlock, 0, s>>>(reinterpret_cast<const float4*>(pos4), density, n, c,
                                                             z, rgb);
    e = cudaGetLastError();
    if (e != cudaSuccess) return report_error(PCISPH_ERR_CUDA, std::string("render: ") + cudaGetErrorString(e));
    return PCISPH_OK;
}
