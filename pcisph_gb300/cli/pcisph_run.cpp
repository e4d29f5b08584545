// pcisph_run -- headless runner: the reference's main loop (PCISPH/src/main.cpp:138-228) without a window.
//
// Loads a reference .xraw scene with the reference's settings (scene::load, scenes.cpp:217-245), steps it
// through pcisph::Fluid (include/pcisph_fluid.hpp, the C ABI) and prints, per step, the corrective
// iterations and the max density error. Optional: frames rendered by the library's headless renderer every
// --every seconds of simulated time (PPM, as main.cpp:204-220 records PNG frames), and a dump of the final
// state (float32 x y z per particle, the sorted order of the last step).
//
//   pcisph_run -i scene.xraw [--name dambreak] [--ppd N] [--steps K] [--max-iters M] [--frames DIR]
//              [--every S] [--size WxH] [--dump FILE] [--device D]
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <chrono>
#include <fstream>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/pcisph_fluid.hpp"

namespace {

// .xraw: 24-byte header ("XRAW", 4 format bytes, volume size x/y/z and palette size as uint32), then one
// byte per voxel, x fastest; 1/2 boundary (visible/invisible), 3 blocker, 4 fluid (scenes.cpp:13-72).
struct Voxels {
    uint32_t sx = 0, sy = 0, sz = 0;
    std::vector<uint8_t> v;
    uint8_t at(int64_t x, int64_t y, int64_t z) const {
        if (x < 0 || y < 0 || z < 0 || x >= sx || y >= sy || z >= sz) return 0;
        return v[(size_t)x + (size_t)y * sx + (size_t)z * sx * sy];
    }
};

Voxels read_xraw(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("File not found: " + path);
    std::vector<char> raw((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    if (raw.size() < 24 || std::memcmp(raw.data(), "XRAW", 4) != 0) throw std::runtime_error("not an XRAW file: " + path);
    Voxels g;
    std::memcpy(&g.sx, raw.data() + 8, 4);
    std::memcpy(&g.sy, raw.data() + 12, 4);
    std::memcpy(&g.sz, raw.data() + 16, 4);
    const size_t n = (size_t)g.sx * g.sy * g.sz;
    if (raw.size() < 24 + n) throw std::runtime_error("XRAW file shorter than its volume: " + path);
    g.v.assign(raw.begin() + 24, raw.begin() + 24 + n);
    return g;
}

// scenes.cpp:76-149: a fluid voxel becomes a ppd^3 block of fluid particles, a boundary voxel a block of
// boundary particles, cut to 3 particle layers next to a blocker; positions (x, z, y), scaled and centred.
void load_scene(const Voxels& g, uint32_t ppd, float scaling, std::vector<float>& fluid, std::vector<float>& boundary) {
    const float ps = scaling / (float)ppd;
    const float off[3] = {-0.5f * scaling * (float)g.sx, -0.5f * scaling * (float)g.sz, -0.5f * scaling * (float)g.sy};
    for (uint32_t z = 0; z < g.sz; ++z)
        for (uint32_t y = 0; y < g.sy; ++y)
            for (uint32_t x = 0; x < g.sx; ++x) {
                const uint8_t t = g.at(x, y, z);
                if (t != 1 && t != 2 && t != 4) continue;
                int64_t lo[3] = {(int64_t)x * ppd, (int64_t)y * ppd, (int64_t)z * ppd};
                int64_t hi[3] = {lo[0] + ppd - 1, lo[1] + ppd - 1, lo[2] + ppd - 1};
                const int64_t c[3] = {x, y, z};
                for (int a = 0; a < 3; ++a) {
                    int64_t p[3] = {x, y, z}, m[3] = {x, y, z};
                    p[a] += 1;
                    m[a] -= 1;
                    if (g.at(p[0], p[1], p[2]) == 3) hi[a] = c[a] * ppd + 2;
                    if (g.at(m[0], m[1], m[2]) == 3) lo[a] = (c[a] + 1) * ppd - 3;
                }
                std::vector<float>& out = t == 4 ? fluid : boundary;
                for (int64_t k = lo[2]; k <= hi[2]; ++k)
                    for (int64_t j = lo[1]; j <= hi[1]; ++j)
                        for (int64_t i = lo[0]; i <= hi[0]; ++i) {
                            out.push_back((float)i * ps + off[0]);
                            out.push_back((float)k * ps + off[1]);
                            out.push_back((float)j * ps + off[2]);
                        }
            }
}

void write_ppm(const std::string& path, int w, int h, const std::vector<uint8_t>& rgb) {
    std::ofstream f(path, std::ios::binary);
    f << "P6\n" << w << " " << h << "\n255\n";
    f.write(reinterpret_cast<const char*>(rgb.data()), (std::streamsize)rgb.size());
}

int usage() {
    std::cout << "pcisph_run -i scene.xraw [--name dambreak|cube_splash|simple_drop] [--ppd N] [--steps K]\n"
                 "           [--max-iters M] [--frames DIR] [--every SECONDS] [--size WxH] [--dump FILE]\n"
                 "           [--device D]\n";
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    std::string path, name, frames, dump;
    uint32_t ppd = 0, steps = 100;
    int max_iters = 7, device = 0, width = 640, height = 480;
    double every = 0.0;
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        auto next = [&]() -> std::string {
            if (i + 1 >= argc) throw std::runtime_error("missing value after " + a);
            return argv[++i];
        };
        if (a == "-h" || a == "--help") return usage();
        else if (a == "-i") path = next();
        else if (a == "--name") name = next();
        else if (a == "--ppd") ppd = (uint32_t)std::stoul(next());
        else if (a == "--steps") steps = (uint32_t)std::stoul(next());
        else if (a == "--max-iters") max_iters = std::stoi(next());
        else if (a == "--frames") frames = next();
        else if (a == "--every") every = std::stod(next());
        else if (a == "--dump") dump = next();
        else if (a == "--device") device = std::stoi(next());
        else if (a == "--size") {
            const std::string v = next();
            if (std::sscanf(v.c_str(), "%dx%d", &width, &height) != 2) throw std::runtime_error("--size WxH");
        } else {
            std::cerr << "unknown argument " << a << "\n";
            return 2;
        }
    }
    if (path.empty()) {
        std::cerr << "-i <scene.xraw> is required\n";
        return 2;
    }
    try {
        if (name.empty()) {  // the file's stem names the scene (scenes.cpp:229-236)
            const size_t s = path.find_last_of('/') + 1, e = path.rfind(".xraw");
            name = path.substr(s, e == std::string::npos ? std::string::npos : e - s);
        }
        // scene::load defaults (scenes.cpp:219-227) and per-scene settings (scenes.cpp:229-236)
        float gravity = -9.81f;
        uint32_t scene_ppd = 3;
        if (name == "simple_drop") {
            scene_ppd = 30;
            gravity = 0.f;
        } else if (name == "cube_splash") {
            scene_ppd = 19;
        } else if (name == "dambreak") {
            scene_ppd = 18;
        }
        if (ppd) scene_ppd = ppd;
        const float scaling = 0.7f;
        std::vector<float> fluid_pos, boundary_pos;
        load_scene(read_xraw(path), scene_ppd, scaling, fluid_pos, boundary_pos);

        pcisph::Fluid fluid(device);
        fluid.set_delta_t(0.002f);
        fluid.set_rest_density(999.972f);
        fluid.set_viscosity(0.00008f);
        fluid.set_surface_tension(1.0f);
        fluid.set_gravity(gravity);
        fluid.set_density_variation_threshold(0.01f);
        fluid.set_particle_radius(0.5f * scaling / (float)scene_ppd);
        fluid.set_fluid_count((unsigned)(fluid_pos.size() / 3));
        fluid.set_boundary_count((unsigned)(boundary_pos.size() / 3));
        pcisph_options o = fluid.options();
        o.max_iterations = max_iters;
        fluid.set_options(o);
        fluid.prepare();
        fluid.set_fluid_state(fluid_pos, {});
        if (!boundary_pos.empty()) fluid.set_boundary_state(boundary_pos);
        std::cout << "Scene loaded!\n-> Fluid-Particles: " << fluid_pos.size() / 3
                  << "\n-> Boundary-Particles: " << boundary_pos.size() / 3 << "\n";

        const float dt = fluid.get_params().delta_t;
        double t = 0.0, last_frame = 0.0;
        int frame = 0;
        std::vector<uint8_t> rgb;
        const auto t0 = std::chrono::steady_clock::now();
        uint64_t iterations = 0;
        for (uint32_t k = 0; k < steps; ++k) {
            fluid.update();
            t += dt;
            const pcisph_step_stats st = fluid.stats();
            iterations += (uint64_t)st.iterations;
            std::printf("step %u iterations %d max_density_error %.5f status %u\n", k, st.iterations,
                        st.max_density_error, st.status);
            if (!frames.empty() && every > 0.0 && t - last_frame >= every) {
                const float a = 0.f, d = 9.f;  // the reference camera (main.cpp:174-179) at angle 0
                pcisph_camera cam = {{d * std::sin(a), d * 0.2f, d * std::cos(a)}, {0.f, 0.f, 0.f}, {0.f, 1.f, 0.f}, 60.f};
                rgb.resize((size_t)width * height * 3);
                pcisph::check(pcisph_render_fluid(fluid.handle(), &cam, width, height, rgb.data(), rgb.size()));
                write_ppm(frames + "/frame_" + std::to_string(frame++) + ".ppm", width, height, rgb);
                last_frame = t;
            }
        }
        fluid.sync();
        const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        std::printf("%u steps, %.2f corrective iterations per step, %.3e particle-steps/s (host-synchronised)\n",
                    steps, steps ? (double)iterations / steps : 0.0, (double)(fluid_pos.size() / 3) * steps / secs);
        if (!dump.empty()) {
            const std::vector<float> pos = fluid.field(PCISPH_FIELD_POSITION);
            std::ofstream f(dump, std::ios::binary);
            f.write(reinterpret_cast<const char*>(pos.data()), (std::streamsize)(pos.size() * sizeof(float)));
        }
    } catch (const std::exception& e) {
        std::cerr << e.what() << "\n";
        return 1;
    }
    return 0;
}
