// C entry point of the reference scene loader (test infrastructure, see scene_shim.cpp).
extern "C" int ref_load_xraw(const char* path, unsigned particles_per_dimension, float scaling, float** fluid,
                             unsigned long* n_fluid, float** boundary, unsigned long* n_boundary, float** cubes,
                             unsigned long* n_cubes) {
    std::vector<float> f, b, c;
    try {
        scene::load_xraw_host(path, particles_per_dimension, scaling, f, b, c);
    } catch (const std::exception&) {
        return -1;
    }
    auto out = [](const std::vector<float>& v, float** p, unsigned long* n) {
        *n = v.size() / 3;
        *p = static_cast<float*>(std::malloc(v.size() * sizeof(float) + 4));
        if (!v.empty()) std::memcpy(*p, v.data(), v.size() * sizeof(float));
    };
    out(f, fluid, n_fluid);
    out(b, boundary, n_boundary);
    out(c, cubes, n_cubes);
    return 0;
}
extern "C" void ref_free(void* p) { std::free(p); }
