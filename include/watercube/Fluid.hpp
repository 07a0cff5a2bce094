// Fluid.hpp — header-only C++ drop-in for WaterCube's core::Fluid (src/core/Fluid.h:32-141)
// over the C ABI in watercube.h. Call sites written against the reference compile unchanged:
//
//     core::FluidRef fluid = core::Fluid::create("fluid");
//     fluid->numParticles(80000)->gridRes(21);
//     fluid->setup();
//     fluid->update(frameSeconds);        // Scene::update -> Fluid::update
//
// Differences from the reference class, each deliberate:
//   * setters change this object and return it (the reference returns a fresh copy,
//     Fluid.h:85, so an un-chained setter call is lost);
//   * the solver is headless: draw() does nothing and the render setters only store values;
//   * errors throw core::FluidError carrying the library's message (the reference asserts);
//   * particle and sort buffers are readable (particles(), uints(), deviceBuffers()).
// Create instances with Fluid::create (the fluent setters return shared_from_this()).
#ifndef WATERCUBE_FLUID_HPP
#define WATERCUBE_FLUID_HPP

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../watercube.h"

namespace core {

// The reference uses glm::vec3; applications that include glm may define WC_VEC3 to it.
#ifndef WC_VEC3
struct Vec3 {
    float x, y, z;
};
#define WC_VEC3 ::core::Vec3
#endif
typedef WC_VEC3 FluidVec3;

class FluidError : public std::runtime_error {
public:
    FluidError(wc_status s, const std::string& what) : std::runtime_error(what), status(s) {}
    wc_status status;
};

inline void check(wc_status s, const char* what) {
    if (s != WC_OK) throw FluidError(s, std::string(what) + ": " + wc_last_error());
}

class Fluid;
typedef std::shared_ptr<Fluid> FluidRef;

class Fluid : public std::enable_shared_from_this<Fluid> {
public:
    explicit Fluid(const std::string& name) : name_(name) {
        wc_params_reference_defaults(&params_);
        gravity_strength_ = -params_.gravity[1];
    }
    ~Fluid() {
        if (handle_) wc_fluid_destroy(handle_);
    }
    Fluid(const Fluid&) = delete;
    Fluid& operator=(const Fluid&) = delete;

    static FluidRef create(const std::string& name) { return std::make_shared<Fluid>(name); }

    // ---- Fluid.h:37-48 -------------------------------------------------------------------
    int numParticles() const { return (int)params_.num_particles; }
    FluidRef numParticles(int n) { return set(params_.num_particles, (uint32_t)n); }
    FluidRef gridRes(int r) { return set(params_.grid_res, (uint32_t)r); }
    FluidRef size(float s) { return set(params_.size, s); }
    FluidRef particleRadius(float r) { return set(params_.particle_radius, r); }
    FluidRef viscosityCoefficient(float c) { return set(params_.viscosity, c); }
    FluidRef stiffness(float s) { return set(params_.stiffness, s); }
    FluidRef restDensity(float d) { return set(params_.rest_density, d); }
    FluidRef restPressure(float p) { return set(params_.rest_pressure, p); }
    FluidRef position(FluidVec3 p) {
        position_ = p;
        return shared_from_this();
    }
    FluidRef gravityStrength(float g) {
        gravity_strength_ = g;
        applyGravity();
        return shared_from_this();
    }
    FluidRef renderMode(int m) {
        render_mode_ = m;
        return shared_from_this();
    }

    // ---- Fluid.h:50-52 ---------------------------------------------------------------------
    void setCameraPosition(FluidVec3 p) { camera_position_ = p; }
    void setLightPosition(FluidVec3 p) { light_position_ = p; }
    // The mouse ray in the fluid's frame (the reference's getRelativeMouseRay, Fluid.cpp:252-257).
    void setMouseRay(FluidVec3 origin, FluidVec3 direction) {
        const float o[3] = {origin.x, origin.y, origin.z}, d[3] = {direction.x, direction.y, direction.z};
        for (int a = 0; a < 3; ++a) {
            params_.mouse_origin[a] = o[a];
            params_.mouse_dir[a] = d[a];
        }
        if (handle_) check(wc_fluid_set_mouse_ray(handle_, o, d), "setMouseRay");
    }
    // gravity_direction_ (Fluid::updateGravity rotates it when the GUI asks).
    void setGravityDirection(FluidVec3 dir) {
        gravity_dir_ = dir;
        applyGravity();
    }

    // ---- Fluid.h:54-57 ---------------------------------------------------------------------
    // Derive the constants, allocate the device buffers and upload the reference's initial
    // lattice (or `initial`, num_particles entries).
    FluidRef setup(const std::vector<wc_particle>* initial = nullptr, uint64_t seed = 0) {
        wc_params p = params_;
        check(wc_params_finalize(&p), "setup");
        std::vector<wc_particle> lattice;
        if (!initial) {
            lattice.resize(p.num_particles);
            check(wc_generate_reference_lattice(&p, seed, lattice.data(), p.num_particles), "setup");
            initial = &lattice;
        }
        if (!handle_) check(wc_fluid_create(&p, &handle_), "setup");
        check(wc_fluid_setup(handle_, initial->data(), (uint32_t)initial->size()), "setup");
        params_ = p;
        return shared_from_this();
    }
    // One step of dt = float(time) * time scale, enqueued on the fluid's stream.
    void update(double time) { check(wc_fluid_update(require(), time), "update"); }
    // update(time) with host buffers (wc_fluid_update_host): uploads `in` first when it is not
    // null, and returns with the stepped state in `out` (num_particles entries), read back while
    // the step's force pass runs.
    void updateHost(double time, const wc_particle* in, wc_particle* out) {
        check(wc_fluid_update_host(require(), time, in, out, params_.num_particles), "updateHost");
    }
    void draw() {}
    void reset() {}

    // ---- buffer access (util::getParticles / util::getUints, util.cpp:42-72) -----------------
    std::vector<wc_particle> particles(int buffer = WC_BUFFER_STATE) {
        std::vector<wc_particle> out(params_.num_particles);
        check(wc_fluid_get_particles(require(), buffer, out.data(), (uint32_t)out.size()), "particles");
        return out;
    }
    std::vector<uint32_t> uints(int which) {
        const bool cells = which == WC_UINTS_CELL_COUNTS || which == WC_UINTS_CELL_OFFSETS;
        const size_t n = cells ? (size_t)params_.grid_res * params_.grid_res * params_.grid_res
                               : (size_t)params_.num_particles;
        std::vector<uint32_t> out(n);
        check(wc_fluid_get_uints(require(), which, out.data(), n), "uints");
        return out;
    }
    wc_device_buffers deviceBuffers() {
        wc_device_buffers b;
        check(wc_fluid_get_device_buffers(require(), &b), "deviceBuffers");
        return b;
    }
    void synchronize() { check(wc_fluid_synchronize(require()), "synchronize"); }

    const std::string& name() const { return name_; }
    const wc_params& params() const { return params_; }
    wc_fluid* handle() { return handle_; }

private:
    template <class T, class V>
    FluidRef set(T& field, V value) {
        if (handle_) throw FluidError(WC_ERR_STATE, "fluid parameters are fixed after setup()");
        field = (T)value;
        return shared_from_this();
    }
    void applyGravity() {
        params_.gravity[0] = gravity_dir_.x * gravity_strength_;
        params_.gravity[1] = gravity_dir_.y * gravity_strength_;
        params_.gravity[2] = gravity_dir_.z * gravity_strength_;
        if (handle_) check(wc_fluid_set_gravity(handle_, params_.gravity), "gravity");
    }
    wc_fluid* require() {
        if (!handle_) throw FluidError(WC_ERR_STATE, "setup() has not been called");
        return handle_;
    }

    std::string name_;
    wc_params params_{};
    wc_fluid* handle_ = nullptr;
    float gravity_strength_ = 900.0f;
    FluidVec3 gravity_dir_{0.0f, -1.0f, 0.0f};
    FluidVec3 position_{-0.5f, -0.5f, -0.5f};
    FluidVec3 camera_position_{0.0f, 0.0f, 0.0f};
    FluidVec3 light_position_{0.0f, 0.0f, 0.0f};
    int render_mode_ = 0;
};

}  // namespace core

#endif
