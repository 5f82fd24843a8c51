/*
 * sph_fluid.hpp -- C++ host mirror of the reference's solver interface over the C ABI of
 * sph_capi.h (header only, C++17).
 *
 * The reference's application code talks to its solvers through
 *   class FluidSimulation            (fluid/simulation/fluidsimulation.h:23-92)
 *   FluidSimulationFactory           (fluid/simulation/fluidsimulationfactory.h:13-40)
 *   PhysicsSettings / SimulationSettings (settings/physicssettings.h, simulationsettings.h)
 *   FluidVolume / BoxVolume          (fluid/simulation/fluidvolume.h, boxvolume.cpp:11-40)
 *   RigidBody + surface sampling     (scene/rigidbody.h, scene/fishtank.cpp, scene/cube.cpp)
 *   Settings::load key=value files   (settings/settings.cpp:14-59, settings/fileparser.cpp)
 * This header keeps those names, method signatures and semantics so the calling code stays
 * a drop-in.  What changes: OpenCL float4 becomes sph_gb300::Float4, the GL vertex buffer the
 * reference renders from becomes a device pointer (device_positions()), Bullet rigid bodies
 * become a plain pose + surface sampling, and errors, reported by the reference as CLError
 * (a std::runtime_error, clerror.cpp:15-19), are thrown as sph_gb300::Error with the C
 * ABI's status code.
 */
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "sph_capi.h"

namespace sph_gb300 {

struct Float4 {
    float x, y, z, w;
};

/* A failed C-ABI call: status (SPH_E_*) and the context's message. */
class Error : public std::runtime_error {
   public:
    Error(int status, const std::string& msg) : std::runtime_error(msg), status_(status) {}
    int status() const { return status_; }

   private:
    int status_;
};

inline void check(int rc, const sph_ctx* ctx) {
    if (rc != SPH_OK) throw Error(rc, sph_last_error(ctx));
}

/* Fluid physical properties; field names and defaults of settings/physicssettings.h. */
struct PhysicsSettings {
    float rest_density = 998.29f;
    float k_viscosity = 0.0035105f;
    float gravity = 9.8f;
    float gas_stiffness = 3.0f;
    float surface_tension = 0.0728f;
};

/* Simulation parameters; field names and defaults of settings/simulationsettings.h. */
struct SimulationSettings {
    enum Method { WCSPH, PCISPH };
    float time_step = 0.01f;
    float max_vel = 50.0f;
    float fluid_particle_radius = 0.008f;
    float fluid_support_radius = 0.032f;
    int pcisph_max_iterations = 7;
    float pcisph_error_ratio = 0.01f;
    Method sim_method = WCSPH;
};

/* Options of the GB300 build with no counterpart in the reference's settings. */
struct DeviceOptions {
    int mode = SPH_MODE_PHYSICS;          /* SPH_MODE_COMPAT reproduces the kernel text */
    int neighbor_mode = SPH_NEIGH_LIST;
    int use_graph = 1;
    void* cuda_stream = nullptr;          /* null: the context creates its own */
};

/* GraphicsSettings (settings/graphicssettings.h): the render method of the config file. */
struct GraphicsSettings {
    enum RenderMethod { PARTICLES, SCREEN_SPACE } render_method = PARTICLES;
};

/* Settings::load (settings/settings.cpp:14-59) over FileParser's key=value format
 * (settings/fileparser.cpp:7-27): '#' starts a comment, every key of the simulation and
 * physics settings is required, method is wcsph or pcisph. */
inline void load_settings(const std::string& path, PhysicsSettings& phys, SimulationSettings& sim) {
    std::ifstream in(path);
    if (!in) throw Error(SPH_E_INVALID, "cannot open settings file '" + path + "'");
    std::map<std::string, std::string> kv;
    std::string line;
    while (std::getline(in, line)) {
        const size_t hash = line.find('#');
        if (hash != std::string::npos) line.resize(hash);
        const size_t eq = line.find('=');
        if (eq == std::string::npos) continue;
        auto trim = [](std::string s) {
            const char* ws = " \t\r\n";
            s.erase(0, s.find_first_not_of(ws));
            s.erase(s.find_last_not_of(ws) + 1);
            return s;
        };
        kv[trim(line.substr(0, eq))] = trim(line.substr(eq + 1));
    }
    auto opt = [&](const char* k) -> const std::string& {
        auto it = kv.find(k);
        if (it == kv.end()) throw Error(SPH_E_INVALID, std::string("settings file lacks '") + k + "'");
        return it->second;
    };
    sim.time_step = (float)std::atof(opt("time_step").c_str());
    sim.max_vel = (float)std::atof(opt("max_vel").c_str());
    sim.fluid_particle_radius = (float)std::atof(opt("fluid_particle_radius").c_str());
    sim.fluid_support_radius = (float)std::atof(opt("fluid_support_radius").c_str());
    sim.pcisph_max_iterations = std::atoi(opt("pcisph_max_iterations").c_str());
    sim.pcisph_error_ratio = (float)std::atof(opt("pcisph_error_ratio").c_str());
    const std::string& m = opt("method");
    if (m == "wcsph") sim.sim_method = SimulationSettings::WCSPH;
    else if (m == "pcisph") sim.sim_method = SimulationSettings::PCISPH;
    else throw Error(SPH_E_INVALID, "Unknown simulation method '" + m + "'!");
    phys.rest_density = (float)std::atof(opt("rest_density").c_str());
    phys.k_viscosity = (float)std::atof(opt("k_viscosity").c_str());
    phys.gravity = (float)std::atof(opt("gravity").c_str());
    phys.gas_stiffness = (float)std::atof(opt("gas_stiffness").c_str());
    phys.surface_tension = (float)std::atof(opt("surface_tension").c_str());
}

/* The graphics part of the same file: render_method = particles | screenspace (absent:
 * particles; the headless tools need no window to read it). */
inline GraphicsSettings load_graphics_settings(const std::string& path) {
    GraphicsSettings g;
    std::ifstream in(path);
    if (!in) throw Error(SPH_E_INVALID, "cannot open settings file '" + path + "'");
    std::string line;
    while (std::getline(in, line)) {
        const size_t hash = line.find('#');
        if (hash != std::string::npos) line.resize(hash);
        const size_t eq = line.find('=');
        if (eq == std::string::npos) continue;
        std::istringstream k(line.substr(0, eq)), v(line.substr(eq + 1));
        std::string key, val;
        k >> key;
        v >> val;
        if (key != "render_method") continue;
        if (val == "particles") g.render_method = GraphicsSettings::PARTICLES;
        else if (val == "screenspace") g.render_method = GraphicsSettings::SCREEN_SPACE;
        else throw Error(SPH_E_INVALID, "Unknown rendering method '" + val + "'!");
    }
    return g;
}

/* FluidVolume (fluid/simulation/fluidvolume.h): a block of fluid sampled at a radius. */
class FluidVolume {
   public:
    virtual ~FluidVolume() = default;
    virtual std::vector<Float4> particles(float particle_radius) = 0;
};

/* BoxVolume (fluid/simulation/boxvolume.cpp:11-40) through sph_scene_box_volume. */
class BoxVolume : public FluidVolume {
   public:
    BoxVolume(float w, float h, float d, float cx, float cy, float cz) : size_{w, h, d}, center_{cx, cy, cz} {}
    std::vector<Float4> particles(float particle_radius) override {
        const int n = sph_scene_box_volume(size_, center_, particle_radius, nullptr, 0);
        std::vector<Float4> out((size_t)(n > 0 ? n : 0));
        if (n > 0) sph_scene_box_volume(size_, center_, particle_radius, &out[0].x, n);
        return out;
    }

   private:
    float size_[3], center_[3];
};

/* A volume given as explicit particle positions (jittered lattices, loaded states). */
class PointVolume : public FluidVolume {
   public:
    explicit PointVolume(std::vector<Float4> pts) : pts_(std::move(pts)) {}
    std::vector<Float4> particles(float) override { return pts_; }

   private:
    std::vector<Float4> pts_;
};

/* RigidBody without a physics engine: a pose (row-major 3x4 rotation | translation, linear
 * and angular velocity) and a surface sampling in body coordinates.  Mass > 0 makes the
 * solver report fluid forces and torques on it (boundaryhandler.cpp:296-349). */
class RigidBody {
   public:
    virtual ~RigidBody() = default;
    virtual std::vector<Float4> surface_sampling(float spacing) const = 0;
    /* Inverse principal moments of inertia in body coordinates and the distance from the
     * centre kept to the container walls; used when the body has mass and can move. */
    virtual void inverse_inertia(float out[3]) const { out[0] = out[1] = out[2] = 0.f; }
    virtual float bounding_radius() const { return 0.f; }
    /* true when surface_sampling runs on the GPU */
    virtual bool samples_on_device() const { return false; }
    float mass = 0.f;
    float rot3x4[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
    float linear_velocity[4] = {0, 0, 0, 0};
    float angular_velocity[4] = {0, 0, 0, 0};
};

/* FishTank (scene/fishtank.cpp:108-141): base and four walls, open top. */
class FishTank : public RigidBody {
   public:
    FishTank(float w, float h, float d) : w_(w), h_(h), d_(d) {}
    std::vector<Float4> surface_sampling(float spacing) const override {
        const int n = sph_scene_fishtank(w_, h_, d_, spacing, nullptr, 0);
        std::vector<Float4> out((size_t)(n > 0 ? n : 0));
        if (n > 0) sph_scene_fishtank(w_, h_, d_, spacing, &out[0].x, n);
        return out;
    }

   private:
    float w_, h_, d_;
};

/* Cube (scene/cube.cpp:136-171): hollow shell of the given side. */
class Cube : public RigidBody {
   public:
    explicit Cube(float side) : side_(side) {}
    /* solid cube: I = m s^2 / 6 about every principal axis */
    void inverse_inertia(float out[3]) const override {
        const float v = mass > 0.f ? 6.0f / (mass * side_ * side_) : 0.f;
        out[0] = out[1] = out[2] = v;
    }
    float bounding_radius() const override { return 0.5f * side_; }
    std::vector<Float4> surface_sampling(float spacing) const override {
        const int n = sph_scene_cube(side_, spacing, nullptr, 0);
        std::vector<Float4> out((size_t)(n > 0 ? n : 0));
        if (n > 0) sph_scene_cube(side_, spacing, &out[0].x, n);
        return out;
    }

   private:
    float side_;
};

/* Sphere (scene/sphere.cpp:8-13,135-171): level-3 icosphere sampling; inertia of a solid
 * sphere, 0.4 m r^2 (btSphereShape). */
class Sphere : public RigidBody {
   public:
    explicit Sphere(float radius) : r_(radius) {}
    void inverse_inertia(float out[3]) const override {
        const float v = mass > 0.f ? 1.0f / (0.4f * mass * r_ * r_) : 0.f;
        out[0] = out[1] = out[2] = v;
    }
    float bounding_radius() const override { return r_; }
    std::vector<Float4> surface_sampling(float spacing) const override {
        const int n = sph_scene_sphere(r_, spacing, nullptr, 0);
        std::vector<Float4> out((size_t)(n > 0 ? n : 0));
        if (n > 0) sph_scene_sphere(r_, spacing, &out[0].x, n);
        return out;
    }

   private:
    float r_;
};

/* Wall (scene/wall.cpp:9-152): a plane sampled at z = 0; inertia of a thin plate,
 * m / 12 (h^2, w^2, w^2 + h^2) (Bullet's btBox2dShape without its margin). */
class Wall : public RigidBody {
   public:
    Wall(float width, float height) : w_(width), h_(height) {}
    void inverse_inertia(float out[3]) const override {
        const float I[3] = {mass / 12.f * (h_ * h_), mass / 12.f * (w_ * w_), mass / 12.f * (w_ * w_ + h_ * h_)};
        for (int a = 0; a < 3; ++a) out[a] = I[a] > 0.f ? 1.0f / I[a] : 0.f;
    }
    float bounding_radius() const override { return 0.5f * std::sqrt(w_ * w_ + h_ * h_); }
    std::vector<Float4> surface_sampling(float spacing) const override {
        const int n = sph_scene_wall(w_, h_, spacing, nullptr, 0);
        std::vector<Float4> out((size_t)(n > 0 ? n : 0));
        if (n > 0) sph_scene_wall(w_, h_, spacing, &out[0].x, n);
        return out;
    }

   private:
    float w_, h_;
};

/* Model (scene/model.cpp:11-214): an OBJ mesh read as ModelMesh does, sampled by voxelizing
 * it on the GPU (voxel size = spacing, precision = spacing / 10).  Inertia: the box of the
 * mesh's bounding box, I = m / 12 (ly^2 + lz^2, lx^2 + lz^2, lx^2 + ly^2) -- Bullet's
 * approximation for convex hulls (btPolyhedralConvexShape) without its collision margin. */
class Model : public RigidBody {
   public:
    explicit Model(const std::string& obj_filename) {
        int nv = 0, ni = 0;
        int rc = sph_scene_load_obj(obj_filename.c_str(), nullptr, 0, nullptr, 0, &nv, &ni);
        if (rc == SPH_OK) {
            v_.resize(3 * (size_t)nv);
            ix_.resize((size_t)ni);
            rc = sph_scene_load_obj(obj_filename.c_str(), v_.data(), nv, ix_.data(), ni, &nv, &ni);
        }
        if (rc != SPH_OK) throw Error(rc, "could not load model: " + obj_filename);
    }
    int vertex_count() const { return (int)(v_.size() / 3); }
    int triangle_count() const { return (int)(ix_.size() / 3); }
    void inverse_inertia(float out[3]) const override {
        float lo[3] = {0.f, 0.f, 0.f}, hi[3] = {0.f, 0.f, 0.f};
        for (size_t i = 0; i < v_.size(); ++i) {
            const int a = (int)(i % 3);
            if (i < 3 || v_[i] < lo[a]) lo[a] = v_[i];
            if (i < 3 || v_[i] > hi[a]) hi[a] = v_[i];
        }
        const float l2[3] = {(hi[0] - lo[0]) * (hi[0] - lo[0]), (hi[1] - lo[1]) * (hi[1] - lo[1]),
                             (hi[2] - lo[2]) * (hi[2] - lo[2])};
        const float I[3] = {mass / 12.f * (l2[1] + l2[2]), mass / 12.f * (l2[0] + l2[2]),
                            mass / 12.f * (l2[0] + l2[1])};
        for (int a = 0; a < 3; ++a) out[a] = I[a] > 0.f ? 1.0f / I[a] : 0.f;
    }
    float bounding_radius() const override {
        float r2 = 0.f;
        for (size_t i = 0; i + 2 < v_.size(); i += 3)
            r2 = std::max(r2, v_[i] * v_[i] + v_[i + 1] * v_[i + 1] + v_[i + 2] * v_[i + 2]);
        return std::sqrt(r2);
    }
    bool samples_on_device() const override { return true; }
    std::vector<Float4> surface_sampling(float spacing) const override {
        const float precision = spacing / 10;
        const int n = sph_scene_voxelize(v_.data(), vertex_count(), ix_.data(), (int)ix_.size(), spacing, precision,
                                         nullptr, 0);
        if (n < 0) throw Error(-n, "model voxelization failed");
        std::vector<Float4> out((size_t)n);
        if (n > 0) {
            const int m = sph_scene_voxelize(v_.data(), vertex_count(), ix_.data(), (int)ix_.size(), spacing,
                                             precision, &out[0].x, n);
            if (m != n) throw Error(m < 0 ? -m : SPH_E_CUDA, "model voxelization failed");
        }
        return out;
    }

   private:
    std::vector<float> v_;
    std::vector<uint32_t> ix_;
};

/* FluidSimulation (fluid/simulation/fluidsimulation.h:23-92): same methods. */
class FluidSimulation {
   public:
    virtual ~FluidSimulation() = default;
    virtual void simulate() = 0;
    virtual void reset(const PhysicsSettings& fluid_settings, const SimulationSettings& sim_settings) = 0;
    virtual int particle_count() const = 0;
    virtual void add_boundary(const std::shared_ptr<RigidBody> boundary, const std::string& boundary_id,
                              bool can_move = false) = 0;
    virtual void set_rect_limits(float width, float height, float depth) = 0;
    virtual int boundary_particle_count() const = 0;
    virtual void add_volume(const std::shared_ptr<FluidVolume> volume) = 0;
};

inline sph_params to_params(const PhysicsSettings& ph, const SimulationSettings& si, const DeviceOptions& o) {
    sph_params p;
    const int method = si.sim_method == SimulationSettings::PCISPH ? SPH_PCISPH : SPH_WCSPH;
    sph_default_params(method, &p);
    p.mode = o.mode;
    p.time_step = si.time_step;
    p.max_vel = si.max_vel;
    p.particle_radius = si.fluid_particle_radius;
    p.support_radius = si.fluid_support_radius;
    p.pcisph_max_iterations = si.pcisph_max_iterations;
    p.pcisph_error_ratio = si.pcisph_error_ratio;
    p.rest_density = ph.rest_density;
    p.k_viscosity = ph.k_viscosity;
    p.gravity = ph.gravity;
    p.gas_stiffness = ph.gas_stiffness;
    p.surface_tension = ph.surface_tension;
    p.neighbor_mode = o.neighbor_mode;
    p.use_graph = o.use_graph;
    return p;
}

/* The CUDA solver behind FluidSimulation: WCSPHSimulation (wcsphsimluation.cpp) or
 * PCISPHSimulation (pcisphsimluation.cpp) depending on SimulationSettings::sim_method. */
class CudaFluidSimulation : public FluidSimulation {
   public:
    CudaFluidSimulation(const PhysicsSettings& ph, const SimulationSettings& si, const DeviceOptions& opt = {})
        : opt_(opt) {
        params_ = to_params(ph, si, opt);
        check(sph_create(&params_, &ctx_), nullptr);
        if (opt_.cuda_stream) check(sph_set_stream(ctx_, opt_.cuda_stream), ctx_);
    }
    ~CudaFluidSimulation() override {
        if (ctx_) sph_destroy(ctx_);
    }
    CudaFluidSimulation(const CudaFluidSimulation&) = delete;
    CudaFluidSimulation& operator=(const CudaFluidSimulation&) = delete;

    void simulate() override { check(sph_simulate(ctx_, 1), ctx_); }
    /* n steps in one call (one graph replay each, no host round trip in between) */
    void simulate(int steps) { check(sph_simulate(ctx_, steps), ctx_); }
    /* steps with the state in host buffers (4 floats per particle each, updated in place;
     * vhalf4 may be null for PCISPH), the copies beside the step's work; waits for them */
    void simulate_host(float* pos4, float* vel4, float* vhalf4, int steps = 1) {
        check(sph_simulate_host(ctx_, pos4, vel4, vhalf4, steps), ctx_);
        check(sph_synchronize(ctx_), ctx_);
    }
    void reset(const PhysicsSettings& ph, const SimulationSettings& si) override {
        params_ = to_params(ph, si, opt_);
        check(sph_reset(ctx_, &params_), ctx_);
    }
    int particle_count() const override { return sph_particle_count(ctx_); }
    void add_boundary(const std::shared_ptr<RigidBody> body, const std::string& boundary_id,
                      bool can_move = false) override {
        const std::vector<Float4> pts = body->surface_sampling(2.0f * params_.particle_radius);
        if (pts.empty()) return;
        check(sph_add_boundary(ctx_, &pts[0].x, (int)pts.size(), can_move ? 1 : 0, body->rot3x4,
                               body->linear_velocity, body->angular_velocity, body->mass),
              ctx_);
        body_ids_.push_back(boundary_id);
        bodies_.push_back(body);
        if (can_move && body->mass > 0.f) {
            /* the reference hands movable bodies with mass to Bullet (scene.cpp:471); here the
             * solver integrates them itself */
            float ii[3];
            body->inverse_inertia(ii);
            check(sph_set_body_dynamics(ctx_, (int)body_ids_.size() - 1, 1, ii, body->bounding_radius()), ctx_);
        }
    }
    void set_rect_limits(float w, float h, float d) override { check(sph_set_rect_limits(ctx_, w, h, d), ctx_); }
    int boundary_particle_count() const override { return sph_boundary_particle_count(ctx_); }
    void add_volume(const std::shared_ptr<FluidVolume> volume) override {
        const std::vector<Float4> pts = volume->particles(params_.particle_radius);
        if (pts.empty()) return;
        check(sph_add_volume(ctx_, &pts[0].x, nullptr, (int)pts.size()), ctx_);
    }
    /* A volume with initial velocities (float4 per particle). */
    void add_volume(const std::vector<Float4>& pos, const std::vector<Float4>& vel) {
        if (pos.empty()) return;
        check(sph_add_volume(ctx_, &pos[0].x, vel.empty() ? nullptr : &vel[0].x, (int)pos.size()), ctx_);
    }

    /* Moves a movable body (the pose RigidBody::update hands to the solver each frame). */
    void set_body_transform(const std::string& boundary_id, const float rot3x4[12], const float lin[4],
                            const float ang[4]) {
        for (size_t b = 0; b < body_ids_.size(); ++b)
            if (body_ids_[b] == boundary_id) {
                check(sph_set_body_transform(ctx_, (int)b, rot3x4, lin, ang), ctx_);
                return;
            }
        throw Error(SPH_E_INVALID, "unknown boundary id '" + boundary_id + "'");
    }
    /* Current pose of a body: rot3x4 (rotation | centre), linear and angular velocity. */
    void body_pose(const std::string& boundary_id, float rot3x4[12], float lin[4], float ang[4]) {
        for (size_t b = 0; b < body_ids_.size(); ++b)
            if (body_ids_[b] == boundary_id) {
                check(sph_get_body_state(ctx_, (int)b, rot3x4, lin, ang), ctx_);
                return;
            }
        throw Error(SPH_E_INVALID, "unknown boundary id '" + boundary_id + "'");
    }
    /* Fluid force and torque on every body (zero for bodies of zero mass). */
    void body_forces(std::vector<Float4>& force, std::vector<Float4>& torque) {
        force.assign(body_ids_.size(), Float4{0, 0, 0, 0});
        torque.assign(body_ids_.size(), Float4{0, 0, 0, 0});
        if (body_ids_.empty()) return;
        check(sph_body_forces(ctx_, &force[0].x, &torque[0].x, (int)body_ids_.size()), ctx_);
    }

    /* Host copies of the state, in the solver's current particle order (ids() gives each
     * particle's id = its index in the order the volumes were added). */
    std::vector<Float4> positions() { return get4(SPH_F_POS); }
    std::vector<Float4> velocities() { return get4(SPH_F_VEL); }
    std::vector<int32_t> ids() {
        std::vector<int32_t> out((size_t)particle_count());
        if (!out.empty()) check(sph_get_field(ctx_, SPH_F_ID, out.data(), out.size() * 4), ctx_);
        return out;
    }
    /* The positions buffer on the device: what the reference shares with OpenGL as a VBO. */
    const void* device_positions() {
        void* p = nullptr;
        check(sph_field_device_ptr(ctx_, SPH_F_POS, &p), ctx_);
        return p;
    }
    /* mean compression, mean |density error|, max density error, kinetic and potential
     * energy, centre of mass (x, y, z) */
    std::vector<double> stats() {
        std::vector<double> out(8);
        check(sph_stats(ctx_, out.data()), ctx_);
        return out;
    }
    unsigned device_flags(bool clear = false) {
        unsigned f = 0;
        check(sph_device_flags(ctx_, &f, clear ? 1 : 0), ctx_);
        return f;
    }
    void synchronize() { check(sph_synchronize(ctx_), ctx_); }
    /* checkpoint / resume (sph_save_state / sph_load_state) */
    void save_state(const std::string& path) { check(sph_save_state(ctx_, path.c_str()), ctx_); }
    /* a headless frame of the particles (sph_render_frame): screen-space surface or lit
     * particle sprites */
    std::vector<float> render_frame(const sph_view& view, int method, int filter_iterations,
                                    const std::vector<sph_light>& lights) {
        std::vector<float> rgba(4 * (size_t)view.width * view.height);
        check(sph_render_frame(ctx_, &view, method, filter_iterations, lights.empty() ? nullptr : lights.data(),
                               (int)lights.size(), rgba.data()),
              ctx_);
        return rgba;
    }
    void load_state(const std::string& path) { check(sph_load_state(ctx_, path.c_str()), ctx_); }
    sph_ctx* handle() { return ctx_; }

   private:
    std::vector<Float4> get4(int field) {
        std::vector<Float4> out((size_t)particle_count());
        if (!out.empty()) check(sph_get_field(ctx_, field, &out[0].x, out.size() * sizeof(Float4)), ctx_);
        return out;
    }
    sph_params params_{};
    DeviceOptions opt_;
    sph_ctx* ctx_ = nullptr;
    std::vector<std::string> body_ids_;
    std::vector<std::shared_ptr<RigidBody>> bodies_;
};

/* FluidSimulationFactory::build_simulation (fluidsimulationfactory.h:13-40) without the GL
 * buffer argument. */
struct FluidSimulationFactory {
    static std::unique_ptr<CudaFluidSimulation> build_simulation(const PhysicsSettings& ph,
                                                                 const SimulationSettings& si,
                                                                 const DeviceOptions& opt = {}) {
        return std::unique_ptr<CudaFluidSimulation>(new CudaFluidSimulation(ph, si, opt));
    }
};

}  // namespace sph_gb300
