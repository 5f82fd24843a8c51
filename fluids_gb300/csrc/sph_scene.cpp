/*
 * sph_scene.cpp -- host-side scene builders used by the headless driver and the tests.
 * They restate the reference's particle samplers with its float/double arithmetic, so
 * particle counts and positions equal what the reference's scene loader produces:
 *   BoxVolume::particles          fluid/simulation/boxvolume.cpp:11-40
 *   FishTank::surface_sampling    scene/fishtank.cpp:108-141 (identity body transform)
 *   Cube::surface_sampling        scene/cube.cpp:136-171 (body coordinates)
 * plus a seeded jitter (splitmix64, Steele/Lea/Flood 2014) used by the benchmark scenes.
 */
#include <cmath>
#include <cstdint>

#include "sph_capi.h"

namespace {
struct Out {
    float* p;
    int cap, n;
    void push(float x, float y, float z) {
        if (p && n < cap) {
            p[4 * n] = x; p[4 * n + 1] = y; p[4 * n + 2] = z; p[4 * n + 3] = 1.f;
        }
        ++n;
    }
};
}  // namespace

extern "C" {

int sph_scene_box_volume(const float size3[3], const float center3[3], float particle_radius, float* out4,
                         int cap) {
    if (!size3 || !center3 || !(particle_radius > 0.f)) return -1;
    Out o{out4, cap, 0};
    const float spacing = 2 * particle_radius;
    const float ex = size3[0], ey = size3[1], ez = size3[2];
    const int nx = (int)std::ceil(ex / spacing), ny = (int)std::ceil(ey / spacing), nz = (int)std::ceil(ez / spacing);
    const float dx = ex / nx, dy = ey / ny, dz = ez / nz;
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i)
            for (int k = 0; k < nz; ++k) {
                const float px = (float)((double)(i * dx + center3[0]) - size3[0] / 2.0);
                const float py = (float)((double)(j * dy + center3[1]) - size3[1] / 2.0);
                const float pz = (float)((double)(k * dz + center3[2]) - size3[2] / 2.0);
                o.push(px, py, pz);
            }
    return o.n;
}

int sph_scene_fishtank(float width, float height, float depth, float spacing, float* out4, int cap) {
    if (!(spacing > 0.f)) return -1;
    Out o{out4, cap, 0};
    for (float x = -width / 2; x <= width / 2; x += spacing)
        for (float z = -depth / 2; z <= depth / 2; z += spacing) o.push(x, -height / 2, z);
    const float y0 = -height / 2 + spacing;
    for (float y = y0; y <= height / 2; y += spacing) {
        for (float x = -width / 2; x <= width / 2; x += spacing) {
            o.push(x, y, -depth / 2);
            o.push(x, y, depth / 2);
        }
        for (float z = -depth / 2; z <= depth / 2; z += spacing) {
            o.push(width / 2, y, z);
            o.push(-width / 2, y, z);
        }
    }
    return o.n;
}

int sph_scene_cube(float side, float spacing, float* out4, int cap) {
    if (!(spacing > 0.f)) return -1;
    Out o{out4, cap, 0};
    const float width = side - spacing, height = side - spacing, depth = side - spacing;
    for (float x = -width / 2; x <= width / 2; x += spacing)
        for (float z = -depth / 2; z <= depth / 2; z += spacing) {
            o.push(x, -height / 2, z);
            o.push(x, height / 2, z);
        }
    const float y0 = -height / 2 + spacing;
    for (float y = y0; y <= height / 2; y += spacing) {
        for (float x = -width / 2; x <= width / 2; x += spacing) {
            o.push(x, y, -depth / 2);
            o.push(x, y, depth / 2);
        }
        for (float z = -depth / 2; z <= depth / 2; z += spacing) {
            o.push(width / 2, y, z);
            o.push(-width / 2, y, z);
        }
    }
    return o.n;
}

void sph_jitter(float* pos4, int n, float amp, uint64_t seed) {
    if (!pos4 || n <= 0) return;
    uint64_t s = seed;
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) {
            uint64_t z = (s += 0x9E3779B97F4A7C15ull);
            z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
            z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
            z ^= z >> 31;
            const float u = (float)(z >> 40) * (1.0f / 16777216.0f);
            pos4[4 * (size_t)i + k] += (2.0f * u - 1.0f) * amp;
        }
}

}  // extern "C"
