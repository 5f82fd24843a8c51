/*
 * sph_driver.cpp -- headless driver: runs a reference scene file with a reference settings
 * file on the GPU solver through the FluidSimulation mirror (include/sph_fluid.hpp).
 *
 * Replaces the reference's Scene + Fluid objects (scene/scene.cpp:322-476, scene/fluid.cpp)
 * without rendering: the settings come from a key=value file (settings/settings.cpp:14-59),
 * the scene from the reference's JSON format -- "container" {width, height, depth} becomes the
 * rectangular limits, "fluid_volumes" of type "box" {size, center} become BoxVolumes, and
 * "rigid_bodies" of type "cube" {size, center, rotation (x, y, z, w quaternion), mass},
 * "sphere" {size (the radius), center, mass}, "model" {obj_filename, center, rotation, mass}
 * and "wall" become boundary bodies (movable when mass > 0, as scene.cpp:471 passes them, and then
 * moved by the solver's own rigid-body step under the fluid's force and torque and gravity;
 * bodies do not collide with each other).  A model's OBJ path is taken as written when it
 * exists, else under --data-root, else under the directory two levels above the scene file
 * (the reference's data/scenes/ layout); "wall" {size [width, height], center, rotation, mass}
 * is a sampled plane.  Options:
 *
 *   sph_driver --config FILE --scene FILE [--steps N] [--every K] [--mode physics|compat]
 *              [--container-boundary] [--jitter SEED] [--dump FILE] [--dry-run]
 *              [--data-root DIR] [--save FILE] [--resume FILE] [--performance_output FILE]
 *
 * -c / -s / -o are the reference's own short forms of --config / --scene /
 * --performance_output (main.cpp:15-19); the last writes one frames-per-second value per
 * line, each the average of 6 steps (gui/glwidget.cpp:62-73, gui/mainwindow.cpp:99-101),
 * a frame here being one solver step.
 *
 * --frames DIR writes frames of the config's render_method (sph_render_frame: "screenspace"
 * = depth sprites, two blur iterations, normals, final shading over black; "particles", the
 * default as in the reference = lit sphere sprites with the scene's lights) as
 * DIR/frame_NNNNN.ppm every
 * --frame-every K steps (default 10) at --frame-size WxH (default 1280x720), seen by the
 * reference's default camera (fov 45, near 0.5, far 30; translate(0, 0, -4) . rotate 45
 * degrees about x; scene/camera.cpp:4-21, gui/glwidget.cpp:82-88) with its sprite radius
 * 0.0625 (fluid/render/sspacefluidrenderer.cpp:365-366).
 *
 * Prints one JSON line per K steps with the solver statistics and a final line with the
 * wall-clock throughput.  --dump writes the final positions ordered by particle id (float32
 * x, y, z, w per particle).  --save writes a checkpoint after the last step; --resume loads
 * one (written from the same scene and settings) before the first, so a run of A steps then
 * B resumed steps ends bit-identical to A + B steps.  --dry-run parses and samples the scene without touching a GPU
 * (models are read but not voxelized: their particle counts are not included).
 */
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "sph_fluid.hpp"

using namespace sph_gb300;

namespace {

/* ---- a minimal JSON reader (objects, arrays, numbers, strings, true/false/null) ---------- */
struct Json {
    enum Kind { NUL, NUM, STR, BOOL, ARR, OBJ } kind = NUL;
    double num = 0.0;
    bool b = false;
    std::string str;
    std::vector<Json> arr;
    std::map<std::string, Json> obj;
    const Json& operator[](const std::string& k) const {
        static const Json none;
        auto it = obj.find(k);
        return it == obj.end() ? none : it->second;
    }
    const Json& operator[](size_t i) const {
        static const Json none;
        return i < arr.size() ? arr[i] : none;
    }
    double number(double def = 0.0) const { return kind == NUM ? num : def; }
};

struct Parser {
    const char* p;
    const char* end;
    void ws() {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) ++p;
    }
    [[noreturn]] void fail(const char* what) { throw Error(SPH_E_INVALID, std::string("scene JSON: ") + what); }
    Json value() {
        ws();
        if (p >= end) fail("unexpected end");
        Json v;
        if (*p == '{') {
            v.kind = Json::OBJ;
            ++p;
            ws();
            if (p < end && *p == '}') { ++p; return v; }
            for (;;) {
                ws();
                Json k = value();
                if (k.kind != Json::STR) fail("object key is not a string");
                ws();
                if (p >= end || *p != ':') fail("expected ':'");
                ++p;
                v.obj[k.str] = value();
                ws();
                if (p < end && *p == ',') { ++p; continue; }
                if (p < end && *p == '}') { ++p; return v; }
                fail("expected ',' or '}'");
            }
        }
        if (*p == '[') {
            v.kind = Json::ARR;
            ++p;
            ws();
            if (p < end && *p == ']') { ++p; return v; }
            for (;;) {
                v.arr.push_back(value());
                ws();
                if (p < end && *p == ',') { ++p; continue; }
                if (p < end && *p == ']') { ++p; return v; }
                fail("expected ',' or ']'");
            }
        }
        if (*p == '"') {
            v.kind = Json::STR;
            ++p;
            while (p < end && *p != '"') {
                if (*p == '\\' && p + 1 < end) ++p;
                v.str.push_back(*p++);
            }
            if (p >= end) fail("unterminated string");
            ++p;
            return v;
        }
        if (!strncmp(p, "true", 4)) { v.kind = Json::BOOL; v.b = true; p += 4; return v; }
        if (!strncmp(p, "false", 5)) { v.kind = Json::BOOL; p += 5; return v; }
        if (!strncmp(p, "null", 4)) { p += 4; return v; }
        char* e = nullptr;
        v.num = std::strtod(p, &e);
        if (e == p) fail("bad value");
        v.kind = Json::NUM;
        p = e;
        return v;
    }
};

Json parse_file(const std::string& path) {
    std::ifstream in(path);
    if (!in) throw Error(SPH_E_INVALID, "cannot open scene file '" + path + "'");
    std::stringstream ss;
    ss << in.rdbuf();
    const std::string s = ss.str();
    Parser ps{s.data(), s.data() + s.size()};
    return ps.value();
}

/* rotation matrix (row-major 3x4 with translation c) of a unit quaternion (x, y, z, w) */
void pose(const double q[4], const double c[3], float out[12]) {
    const double x = q[0], y = q[1], z = q[2], w = q[3];
    const double n = std::sqrt(x * x + y * y + z * z + w * w);
    const double a = x / n, b = y / n, cc = z / n, d = w / n;
    const double m[9] = {1 - 2 * (b * b + cc * cc), 2 * (a * b - cc * d),     2 * (a * cc + b * d),
                         2 * (a * b + cc * d),     1 - 2 * (a * a + cc * cc), 2 * (b * cc - a * d),
                         2 * (a * cc - b * d),     2 * (b * cc + a * d),     1 - 2 * (a * a + b * b)};
    for (int r = 0; r < 3; ++r) {
        for (int k = 0; k < 3; ++k) out[4 * r + k] = (float)m[3 * r + k];
        out[4 * r + 3] = (float)c[r];
    }
}

struct Scene {
    float container[3] = {0, 0, 0};
    std::vector<sph_light> lights;   /* "lights": direction, diffuse_color / 255 */
    std::vector<std::shared_ptr<FluidVolume>> volumes;
    std::vector<std::pair<std::string, std::shared_ptr<RigidBody>>> bodies;
};

bool file_exists(const std::string& p) {
    std::ifstream f(p);
    return f.good();
}

std::string parent_dir(const std::string& p) {
    const size_t k = p.find_last_of('/');
    return k == std::string::npos ? std::string(".") : (k == 0 ? std::string("/") : p.substr(0, k));
}

std::string resolve_model(const std::string& obj, const std::string& scene_path, const std::string& data_root) {
    if (obj.empty() || obj[0] == '/' || file_exists(obj)) return obj;
    if (!data_root.empty() && file_exists(data_root + "/" + obj)) return data_root + "/" + obj;
    const std::string up2 = parent_dir(parent_dir(scene_path));
    if (file_exists(up2 + "/" + obj)) return up2 + "/" + obj;
    return obj;
}

Scene load_scene(const std::string& path, bool container_boundary, const std::string& data_root) {
    const Json j = parse_file(path);
    Scene sc;
    for (const Json& l : j["lights"].arr) {
        if (sc.lights.size() == 8) break;   /* MAX_DIR_LIGHTS of particles.frag */
        sph_light li{};
        for (int k = 0; k < 3; ++k) li.direction[k] = (float)l["direction"][k].number();
        for (int k = 0; k < 3; ++k) li.diffuse[k] = (float)(l["diffuse_color"][k].number() / 255.0);
        li.diffuse[3] = 1.0f;
        sc.lights.push_back(li);
    }
    const Json& c = j["container"];
    sc.container[0] = (float)c["width"].number();
    sc.container[1] = (float)c["height"].number();
    sc.container[2] = (float)c["depth"].number();
    if (container_boundary)
        sc.bodies.emplace_back("container",
                               std::make_shared<FishTank>(sc.container[0], sc.container[1], sc.container[2]));
    for (const Json& v : j["fluid_volumes"].arr) {
        if (v["type"].str != "box") {
            std::fprintf(stderr, "skipping fluid volume of type '%s'\n", v["type"].str.c_str());
            continue;
        }
        sc.volumes.push_back(std::make_shared<BoxVolume>(
            (float)v["size"][0].number(), (float)v["size"][1].number(), (float)v["size"][2].number(),
            (float)v["center"][0].number(), (float)v["center"][1].number(), (float)v["center"][2].number()));
    }
    for (const Json& r : j["rigid_bodies"].arr) {
        const std::string type = r["type"].str;
        std::shared_ptr<RigidBody> body;
        if (type == "cube") body = std::make_shared<Cube>((float)r["size"].number());
        else if (type == "sphere") body = std::make_shared<Sphere>((float)r["size"].number());
        else if (type == "model")
            body = std::make_shared<Model>(resolve_model(r["obj_filename"].str, path, data_root));
        else if (type == "wall")
            body = std::make_shared<Wall>((float)r["size"][0].number(), (float)r["size"][1].number());
        if (!body) {
            std::fprintf(stderr, "skipping rigid body '%s' of type '%s'\n", r["name"].str.c_str(), type.c_str());
            continue;
        }
        /* a sphere has no rotation in the scene format (identity, scene.cpp:418-426) */
        const bool rot = type != "sphere";
        const double q[4] = {rot ? r["rotation"][0].number(0) : 0.0, rot ? r["rotation"][1].number(0) : 0.0,
                             rot ? r["rotation"][2].number(0) : 0.0, rot ? r["rotation"][3].number(1) : 1.0};
        const double ctr[3] = {r["center"][0].number(), r["center"][1].number(), r["center"][2].number()};
        pose(q, ctr, body->rot3x4);
        body->mass = (float)r["mass"].number();
        sc.bodies.emplace_back(r["name"].str, body);
    }
    return sc;
}

/* A volume whose particles are jittered (splitmix64 stream, amplitude 1e-4 m). */
class Jittered : public FluidVolume {
   public:
    Jittered(std::shared_ptr<FluidVolume> v, uint64_t seed) : v_(std::move(v)), seed_(seed) {}
    std::vector<Float4> particles(float r) override {
        std::vector<Float4> p = v_->particles(r);
        if (!p.empty()) sph_jitter(&p[0].x, (int)p.size(), 1e-4f, seed_);
        return p;
    }

   private:
    std::shared_ptr<FluidVolume> v_;
    uint64_t seed_;
};

/* The reference's default camera as an sph_view (column-major matrices). */
sph_view default_view(int w, int h) {
    sph_view v{};
    const double fov = 45.0, n = 0.5, f = 30.0, aspect = (double)w / (h ? h : 1);
    const double ct = 1.0 / std::tan(fov * 3.14159265358979323846 / 360.0);
    double pr[16] = {0};
    pr[0] = ct / aspect;
    pr[5] = ct;
    pr[10] = -(f + n) / (f - n);
    pr[11] = -1.0;
    pr[14] = -2.0 * f * n / (f - n);
    const double c = std::cos(3.14159265358979323846 / 4), s = std::sin(3.14159265358979323846 / 4);
    /* translate(0, 0, -4) . rotate(45 deg about x) */
    const double mv[16] = {1, 0, 0, 0, 0, c, s, 0, 0, -s, c, 0, 0, 0, -4, 1};
    for (int k = 0; k < 16; ++k) {
        v.projection[k] = (float)pr[k];
        v.modelview[k] = (float)mv[k];
    }
    v.point_radius = 0.0625f;
    v.point_scale = (float)(w * std::tan(fov * 3.14159265358979323846 / 360.0));
    v.width = w;
    v.height = h;
    return v;
}

std::string pad5(int k) {
    char b[16];
    std::snprintf(b, sizeof b, "%05d", k);
    return b;
}

/* 8-bit binary PPM, top row first (the image's row 0 is the bottom) */
void write_ppm(const std::string& path, const std::vector<float>& rgba, int w, int h) {
    std::ofstream out(path, std::ios::binary);
    if (!out) throw Error(SPH_E_INVALID, "cannot write " + path);
    out << "P6\n" << w << " " << h << "\n255\n";
    std::vector<unsigned char> row(3 * (size_t)w);
    for (int y = h - 1; y >= 0; --y) {
        for (int x = 0; x < w; ++x)
            for (int c = 0; c < 3; ++c) {
                const float v = rgba[4 * ((size_t)y * w + x) + c];
                row[3 * (size_t)x + c] = (unsigned char)(v <= 0.f ? 0 : (v >= 1.f ? 255 : (int)(v * 255.f + 0.5f)));
            }
        out.write(reinterpret_cast<const char*>(row.data()), (std::streamsize)row.size());
    }
}

int usage() {
    std::fprintf(stderr,
                 "usage: sph_driver --config FILE --scene FILE [--steps N] [--every K] [--mode physics|compat]\n"
                 "                  [--container-boundary] [--jitter SEED] [--dump FILE] [--dry-run]\n"
                 "                  [--data-root DIR] [--save FILE] [--resume FILE] [-o FILE]\n"
                 "                  [--frames DIR] [--frame-every K] [--frame-size WxH]\n");
    return 2;
}

}  // namespace

int main(int argc, char** argv) {
    std::string config, scene_file, dump, mode = "physics", data_root, save, resume, fps_out, frames;
    int frame_every = 10, frame_w = 1280, frame_h = 720;
    int steps = 100, every = 0;
    bool dry = false, container_boundary = false;
    long long jitter = -1;
    for (int a = 1; a < argc; ++a) {
        const std::string k = argv[a];
        auto next = [&]() -> std::string {
            if (a + 1 >= argc) throw Error(SPH_E_INVALID, "missing value after " + k);
            return argv[++a];
        };
        try {
            if (k == "--config" || k == "-c") config = next();
            else if (k == "--scene" || k == "-s") scene_file = next();
            else if (k == "--performance_output" || k == "-o") fps_out = next();
            else if (k == "--steps") steps = std::atoi(next().c_str());
            else if (k == "--every") every = std::atoi(next().c_str());
            else if (k == "--mode") mode = next();
            else if (k == "--dump") dump = next();
            else if (k == "--jitter") jitter = std::atoll(next().c_str());
            else if (k == "--container-boundary") container_boundary = true;
            else if (k == "--dry-run") dry = true;
            else if (k == "--data-root") data_root = next();
            else if (k == "--save") save = next();
            else if (k == "--frames") frames = next();
            else if (k == "--frame-every") frame_every = std::atoi(next().c_str());
            else if (k == "--frame-size") {
                const std::string v = next();
                if (std::sscanf(v.c_str(), "%dx%d", &frame_w, &frame_h) != 2) throw Error(SPH_E_INVALID, "--frame-size WxH");
            }
            else if (k == "--resume") resume = next();
            else return usage();
        } catch (const Error& e) {
            std::fprintf(stderr, "%s\n", e.what());
            return usage();
        }
    }
    if (config.empty() || scene_file.empty()) return usage();
    try {
        PhysicsSettings phys;
        SimulationSettings sim;
        load_settings(config, phys, sim);
        const GraphicsSettings gfx = load_graphics_settings(config);   /* validated as the reference does */
        Scene sc = load_scene(scene_file, container_boundary, data_root);
        if (jitter >= 0)
            for (size_t v = 0; v < sc.volumes.size(); ++v)
                sc.volumes[v] = std::make_shared<Jittered>(sc.volumes[v], (uint64_t)jitter + v);
        if (dry) {
            size_t nf = 0, nb = 0, ndev = 0;
            for (auto& v : sc.volumes) nf += v->particles(sim.fluid_particle_radius).size();
            for (auto& b : sc.bodies) {
                if (b.second->samples_on_device()) ++ndev;
                else nb += b.second->surface_sampling(2.0f * sim.fluid_particle_radius).size();
            }
            std::printf("{\"method\": \"%s\", \"time_step\": %g, \"particles\": %zu, \"boundary_particles\": %zu, "
                        "\"volumes\": %zu, \"bodies\": %zu, \"device_sampled_bodies\": %zu, "
                        "\"container\": [%g, %g, %g]}\n",
                        sim.sim_method == SimulationSettings::PCISPH ? "pcisph" : "wcsph", sim.time_step, nf, nb,
                        sc.volumes.size(), sc.bodies.size(), ndev, sc.container[0], sc.container[1], sc.container[2]);
            return 0;
        }
        DeviceOptions opt;
        opt.mode = mode == "compat" ? SPH_MODE_COMPAT : SPH_MODE_PHYSICS;
        auto fluid = FluidSimulationFactory::build_simulation(phys, sim, opt);
        fluid->set_rect_limits(sc.container[0], sc.container[1], sc.container[2]);
        for (auto& b : sc.bodies) fluid->add_boundary(b.second, b.first, b.second->mass > 0.0f);
        for (auto& v : sc.volumes) fluid->add_volume(v);
        if (!resume.empty()) fluid->load_state(resume);
        const char* names[8] = {"mean_compression", "mean_abs_density_error", "max_density_error", "kinetic",
                                "potential", "com_x", "com_y", "com_z"};
        fluid->synchronize();
        std::ofstream fps;
        if (!fps_out.empty()) {
            fps.open(fps_out);
            if (!fps.good()) throw Error(SPH_E_INVALID, "cannot write " + fps_out);
        }
        const auto t0 = std::chrono::steady_clock::now();
        auto tf = t0;
        const sph_view view = default_view(frame_w, frame_h);
        int frame_no = 0;
        for (int s = 1; s <= steps; ++s) {
            fluid->simulate();
            if (!frames.empty() && frame_every > 0 && s % frame_every == 0)
                write_ppm(frames + "/frame_" + pad5(frame_no++) + ".ppm", fluid->render_frame(view, gfx.render_method == GraphicsSettings::PARTICLES ? SPH_RENDER_PARTICLES
                                                                                                 : SPH_RENDER_SCREEN_SPACE,
                                                      2, sc.lights), frame_w,
                          frame_h);
            if (fps.is_open() && s % 6 == 0) {   /* frames per second over the last 6 steps */
                fluid->synchronize();
                const auto now = std::chrono::steady_clock::now();
                const double ms = std::chrono::duration<double, std::milli>(now - tf).count();
                tf = now;
                fps << (ms > 0 ? 1000.0 / (ms / 6.0) : 0.0) << "\n";
            }
            if (every > 0 && s % every == 0) {
                const std::vector<double> st = fluid->stats();
                std::printf("{\"step\": %d", s);
                for (int k = 0; k < 8; ++k) std::printf(", \"%s\": %.9g", names[k], st[k]);
                std::printf(", \"bodies\": {");
                bool first = true;
                for (auto& b : sc.bodies) {
                    if (!(b.second->mass > 0.f)) continue;
                    float rot[12], lin[4], ang[4];
                    fluid->body_pose(b.first, rot, lin, ang);
                    std::printf("%s\"%s\": [%.7g, %.7g, %.7g]", first ? "" : ", ", b.first.c_str(), rot[3], rot[7],
                                rot[11]);
                    first = false;
                }
                std::printf("}, \"flags\": %u}\n", fluid->device_flags());
                std::fflush(stdout);
            }
        }
        fluid->synchronize();
        const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (!save.empty()) fluid->save_state(save);
        const int n = fluid->particle_count();
        std::printf("{\"done\": %d, \"particles\": %d, \"boundary_particles\": %d, \"seconds\": %.6f, "
                    "\"particle_updates_per_s\": %.6g, \"flags\": %u}\n",
                    steps, n, fluid->boundary_particle_count(), sec, sec > 0 ? (double)n * steps / sec : 0.0,
                    fluid->device_flags());
        if (!dump.empty()) {
            std::vector<Float4> pos = fluid->positions();
            std::vector<int32_t> ids = fluid->ids();
            std::vector<Float4> by_id(pos.size());
            for (size_t i = 0; i < pos.size(); ++i) by_id[(size_t)ids[i]] = pos[i];
            std::ofstream out(dump, std::ios::binary);
            out.write(reinterpret_cast<const char*>(by_id.data()), (std::streamsize)(by_id.size() * sizeof(Float4)));
        }
    } catch (const Error& e) {
        std::fprintf(stderr, "error (status %d): %s\n", e.status(), e.what());
        return 1;
    }
    return 0;
}
