// wc_params.cpp — host-only parts of the C ABI: parameter presets and derivation (the
// reference's Fluid constructor and Fluid::setup, src/core/Fluid.cpp:9-27 and :203-216),
// initial-state generators (Fluid::generateInitialParticles, :104-134), error strings.
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>

#include "wc_internal.h"
#include "wc_util.h"

namespace wc {

namespace {
thread_local std::string g_last_error;

inline uint64_t splitmix64(uint64_t& state) {
    uint64_t z = (state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
inline float unit24(uint64_t& state) { return (float)(splitmix64(state) >> 40) * (1.0f / 16777216.0f); }
}  // namespace

wc_status fail(wc_status s, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return s;
}

void clear_error() { g_last_error.clear(); }
const char* last_error() { return g_last_error.c_str(); }

namespace {
std::atomic<long long> g_allocs_left{-1};  // -1: off; n >= 0: allocations that still succeed
}

wc_status device_alloc(void** p, size_t bytes) {
    *p = nullptr;
    if (!bytes) return WC_OK;
    long long left = g_allocs_left.load();
    while (left >= 0) {
        if (left == 0) return fail(WC_ERR_OOM, "device allocation of %zu bytes refused by the test hook", bytes);
        if (g_allocs_left.compare_exchange_weak(left, left - 1)) break;
    }
    const cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        *p = nullptr;
        return fail(e == cudaErrorMemoryAllocation ? WC_ERR_OOM : WC_ERR_CUDA, "cudaMalloc(%zu): %s", bytes,
                    cudaGetErrorString(e));
    }
    return WC_OK;
}

}  // namespace wc

extern "C" WC_API void wc_debug_fail_allocations(long long after) { wc::g_allocs_left.store(after < 0 ? -1 : after); }

namespace wc {

SceneConsts make_scene_consts(const wc_params& p) {
    SceneConsts c;
    std::memset(&c, 0, sizeof c);
    c.size = p.size;
    c.bin = p.bin_size;
    c.h = p.kernel_radius;
    c.h2 = p.kernel_radius * p.kernel_radius;
    c.cull = wc_cull_threshold(p.kernel_radius);
    c.m = p.particle_mass;
    c.rho0 = p.rest_density;
    c.p0 = p.rest_pressure;
    c.k = p.stiffness;
    c.mu = p.viscosity;
    c.c6 = p.poly6_const;
    c.cs = p.spiky_const;
    c.cv = p.visc_const;
    c.max_speed = p.max_speed;
    c.damping = p.wall_damping;
    c.border = p.wall_border;
    for (int a = 0; a < 3; ++a) {
        c.g[a] = p.gravity[a];
        c.mouse_o[a] = p.mouse_origin[a];
        c.mouse_d[a] = p.mouse_dir[a];
    }
    c.R = (int32_t)p.grid_res;
    c.R_magic = r_magic(p.grid_res);
    c.eos = p.eos;
    c.flags = p.flags;
    return c;
}

StepInputs make_step_inputs(const wc_params& p, float dt) {
    StepInputs s{};
    s.dt = dt;
    for (int a = 0; a < 3; ++a) {
        s.g[a] = p.gravity[a];
        s.mouse_o[a] = p.mouse_origin[a];
        s.mouse_d[a] = p.mouse_dir[a];
    }
    return s;
}

}  // namespace wc

using namespace wc;

extern "C" {

WC_API void wc_params_reference_defaults(wc_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof *p);
    p->num_particles = 80000;
    p->grid_res = 21;
    p->size = 1.0f;
    p->particle_radius = 0.01f;
    p->rest_density = 500.0f;
    p->rest_pressure = 0.0f;
    p->stiffness = 100.0f;
    p->viscosity = 200.0f;
    p->gravity[0] = 0.0f;
    p->gravity[1] = -900.0f;  // gravity_direction_ (0,-1,0) * gravity_strength_ 900
    p->gravity[2] = 0.0f;
    p->time_scale = 0.012f;
    p->eos = WC_EOS_DESBRUN_CUBIC;
    p->flags = WC_FLAGS_REFERENCE;
    p->max_speed = 50.0f;
    p->wall_damping = 0.3f;
    p->wall_border = 0.001f;
    // The app's camera (-1, 1/3, 2) seen from the fluid's frame (position_ = -size/2), looking
    // straight up: the ray misses the box, so the mouse force is zero (update.comp:119-121).
    p->mouse_origin[0] = -0.5f;
    p->mouse_origin[1] = 1.0f / 3.0f + 0.5f;
    p->mouse_origin[2] = 2.5f;
    p->mouse_dir[0] = 0.0f;
    p->mouse_dir[1] = 1.0f;
    p->mouse_dir[2] = 0.0f;
}

WC_API void wc_params_dam_break(wc_params* p, uint32_t num_particles) {
    if (!p) return;
    std::memset(p, 0, sizeof *p);
    const double h = 0.0457 * std::cbrt(16384.0 / (double)(num_particles ? num_particles : 1));
    const double s = 0.5 * h;
    p->num_particles = num_particles;
    p->grid_res = 0;  // floor(size / h)
    p->size = 1.0f;
    p->kernel_radius = (float)h;
    p->particle_radius = (float)(h / 4.0);
    p->particle_mass = (float)(1000.0 * s * s * s);
    p->rest_density = 1000.0f;
    p->rest_pressure = 0.0f;
    p->stiffness = 3.0f;
    p->viscosity = 3.5f;
    p->gravity[1] = -9.81f;
    p->time_scale = 1.0f;
    p->eos = WC_EOS_LINEAR;
    p->flags = 0;
    p->max_speed = 50.0f;
    p->wall_damping = 0.5f;  // restitution
    p->wall_border = 0.001f;
    p->mouse_dir[1] = 1.0f;
    p->mouse_origin[1] = 2.0f;
}

WC_API wc_status wc_params_finalize(wc_params* p) {
    clear_error();
    if (!p) return fail(WC_ERR_INVALID_ARG, "wc_params_finalize: null params");
    if (p->num_particles >= (1u << 31)) return fail(WC_ERR_INVALID_ARG, "num_particles must be < 2^31");
    if (!(p->size > 0.0f) || !std::isfinite(p->size)) return fail(WC_ERR_INVALID_ARG, "size must be > 0");
    if (p->kernel_radius == 0.0f) p->kernel_radius = p->particle_radius * 4.0f;  // Fluid.cpp:209
    if (p->particle_mass == 0.0f) p->particle_mass = p->particle_radius * 8.0f;  // Fluid.cpp:210
    if (!(p->kernel_radius > 0.0f) || !std::isfinite(p->kernel_radius))
        return fail(WC_ERR_INVALID_ARG, "kernel radius must be > 0 (set kernel_radius or particle_radius)");
    if (!(p->particle_mass > 0.0f) || !std::isfinite(p->particle_mass))
        return fail(WC_ERR_INVALID_ARG, "particle mass must be > 0");
    if (p->grid_res == 0) {
        const float r = std::floor(p->size / p->kernel_radius);
        p->grid_res = r < 1.0f ? 1u : (uint32_t)r;
    }
    if (p->grid_res > 1024) return fail(WC_ERR_INVALID_ARG, "grid_res %u exceeds 1024", p->grid_res);
    if (p->eos != WC_EOS_DESBRUN_CUBIC && p->eos != WC_EOS_LINEAR)
        return fail(WC_ERR_INVALID_ARG, "unknown eos %u", p->eos);
    if (!(p->rest_density > 0.0f)) return fail(WC_ERR_INVALID_ARG, "rest density must be > 0");
    if (p->bin_size == 0.0f) p->bin_size = p->size / (float)p->grid_res;  // Fluid.cpp:208
    const double h = p->kernel_radius;
    const double pi = 3.14159265358979323846;
    if (p->poly6_const == 0.0f) p->poly6_const = (float)(315.0 / (64.0 * pi * std::pow(h, 9)));
    if (p->spiky_const == 0.0f) p->spiky_const = (float)(-45.0 / (pi * std::pow(h, 6)));
    if (p->visc_const == 0.0f) p->visc_const = (float)(45.0 / (pi * std::pow(h, 6)));
    if (!std::isfinite(p->poly6_const) || !std::isfinite(p->spiky_const))
        return fail(WC_ERR_INVALID_ARG, "kernel constants overflow for h = %g", h);
    return WC_OK;
}

WC_API float wc_cull_threshold(float h) {
    // |r| < h is evaluated as sqrtf(d2) < h; sqrtf is monotonic, so the accepted d2 form a
    // prefix of the floats. Step to its last element.
    float x = h * h;
    while (x > 0.0f && !(std::sqrt(x) < h)) x = std::nextafter(x, 0.0f);
    while (std::sqrt(std::nextafter(x, INFINITY)) < h) x = std::nextafter(x, INFINITY);
    return x;
}

WC_API wc_status wc_generate_dam_break(const wc_params* p, uint64_t seed, wc_particle* out, uint32_t n) {
    clear_error();
    if (!p || (!out && n)) return fail(WC_ERR_INVALID_ARG, "wc_generate_dam_break: null pointer");
    if (!(p->kernel_radius > 0.0f)) return fail(WC_ERR_INVALID_ARG, "finalize params first (kernel_radius is 0)");
    uint32_t a = 1;
    while (2ull * (a + 1) * (a + 1) * (a + 1) <= n) ++a;
    const uint32_t nx = a, nz = a;
    const float h = p->kernel_radius;
    const float s = h * 0.5f;
    const float js = 0.01f * h;
    uint64_t st = seed;
    for (uint32_t q = 0; q < n; ++q) {
        const uint32_t i = q % nx, k = (q / nx) % nz, j = q / (nx * nz);
        const float lat[3] = {((float)i + 0.5f) * s, ((float)j + 0.5f) * s, ((float)k + 0.5f) * s};
        wc_particle& o = out[q];
        for (int c = 0; c < 3; ++c) {
            const float u = unit24(st);
            o.position[c] = lat[c] + (2.0f * u - 1.0f) * js;
            o.velocity[c] = 0.0f;
        }
        o.density = 0.0f;
        o.pressure = 0.0f;
    }
    return WC_OK;
}

WC_API wc_status wc_generate_reference_lattice(const wc_params* p, uint64_t seed, wc_particle* out, uint32_t n) {
    clear_error();
    if (!p || (!out && n)) return fail(WC_ERR_INVALID_ARG, "wc_generate_reference_lattice: null pointer");
    uint32_t d = 1;
    while ((uint64_t)d * d * d < n) ++d;
    const float distance = p->particle_radius * 1.75f;
    const float jitter = distance * 0.5f;
    uint64_t st = seed;
    for (uint32_t q = 0; q < n; ++q) {
        const uint32_t x = q % d, y = (q / d) % d, z = q / (d * d);
        const float lat[3] = {(float)x * distance, (float)y * distance, (float)z * distance};
        wc_particle& o = out[q];
        for (int c = 0; c < 3; ++c) {
            const float u = unit24(st);
            o.position[c] = lat[c] + (u * jitter - jitter / 2.0f);
            o.velocity[c] = 0.0f;
        }
        o.density = 0.0f;
        o.pressure = 0.0f;
    }
    return WC_OK;
}

WC_API const char* wc_last_error(void) { return last_error(); }

WC_API const char* wc_status_string(wc_status s) {
    switch (s) {
        case WC_OK: return "ok";
        case WC_ERR_INVALID_ARG: return "invalid argument";
        case WC_ERR_OOM: return "out of memory";
        case WC_ERR_CUDA: return "CUDA error";
        case WC_ERR_TIMEOUT: return "device wait timed out";
        case WC_ERR_NUMERIC: return "non-finite particle state";
        case WC_ERR_STATE: return "call out of order";
        case WC_ERR_UNSUPPORTED: return "unsupported";
    }
    return "unknown status";
}

WC_API const char* wc_build_info(void) { return "watercube " "1" " sm_103a"; }

}  // extern "C"
