/*
 * ref_scene.cpp -- the reference's host scene samplers, compiled for the oracle from the
 * reference's own source text: BoxVolume::particles (fluid/simulation/boxvolume.cpp:11-40),
 * FishTank::surface_sampling (scene/fishtank.cpp:108-141) and Cube::surface_sampling
 * (scene/cube.cpp:136-171).  TEST INFRASTRUCTURE: built only by oracle/build_ref.sh into
 * oracle/_ref/, used to pin the library's sph_scene_* samplers and to build the reference
 * arm's scene.
 *
 * Those files also hold the classes' OpenGL, Qt and Bullet code, which does not build here,
 * so build_ref.sh copies each sampler's function text (from its signature line to its
 * closing brace) into oracle/_ref/src/*.inc unchanged, and this file compiles it against
 * minimal stand-ins of the members the samplers read: the box's size and centre, the tank's
 * width, height, depth and body transform, the cube's side.  The samplers run in body
 * coordinates (identity transform), as the library's samplers do; the pose is applied by the
 * solver.  Built with -ffp-contract=off like the library's samplers.
 */
#include <cmath>
#include <vector>

#include "LinearMath/btVector3.h"

using namespace std;

struct cl_float4 {
    float s[4];
};

/* The body transform a sampler applies to its points: the identity (body coordinates). */
struct IdentityTransform {
    btVector3 operator()(const btVector3& v) const { return v; }
};

class BoxVolume {
   public:
    BoxVolume(const btVector3& size, const btVector3& center) : _size(size), _center(center) {}
    vector<cl_float4> particles(float particle_radius);

   private:
    btVector3 _size, _center;
};

class FishTank {
   public:
    FishTank(float w, float h, float d) : _width(w), _height(h), _depth(d) {}
    vector<btVector3> surface_sampling(float particle_spacing) const;

   private:
    float _width, _height, _depth;
    IdentityTransform _transform;
};

class Cube {
   public:
    explicit Cube(float side) : _side(side) {}
    vector<btVector3> surface_sampling(float particle_spacing) const;

   private:
    float _side;
};

#include "boxvolume_particles.inc"
#include "fishtank_surface_sampling.inc"
#include "cube_surface_sampling.inc"

namespace {
int copy_out(const vector<btVector3>& v, float* out4, int cap) {
    const int n = (int)v.size();
    for (int i = 0; out4 && i < n && i < cap; ++i) {
        out4[4 * i + 0] = v[i].x();
        out4[4 * i + 1] = v[i].y();
        out4[4 * i + 2] = v[i].z();
        out4[4 * i + 3] = 1.0f;
    }
    return n;
}
}  // namespace

/* Same arguments and return as the library's sph_scene_box_volume / _fishtank / _cube: the
 * particle count, with up to cap particles written to out4 (x, y, z, 1). */
extern "C" int ref_scene_box_volume(const float* size3, const float* center3, float particle_radius, float* out4,
                                    int cap) {
    BoxVolume b(btVector3(size3[0], size3[1], size3[2]), btVector3(center3[0], center3[1], center3[2]));
    const vector<cl_float4> p = b.particles(particle_radius);
    const int n = (int)p.size();
    for (int i = 0; out4 && i < n && i < cap; ++i)
        for (int k = 0; k < 4; ++k) out4[4 * i + k] = p[i].s[k];
    return n;
}

extern "C" int ref_scene_fishtank(float width, float height, float depth, float spacing, float* out4, int cap) {
    return copy_out(FishTank(width, height, depth).surface_sampling(spacing), out4, cap);
}

extern "C" int ref_scene_cube(float side, float spacing, float* out4, int cap) {
    return copy_out(Cube(side).surface_sampling(spacing), out4, cap);
}
