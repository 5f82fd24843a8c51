/*
 * sph_scene.cpp -- host-side scene builders used by the headless driver and the tests.
 * They restate the reference's particle samplers with its float/double arithmetic, so
 * particle counts and positions equal what the reference's scene loader produces:
 *   BoxVolume::particles          fluid/simulation/boxvolume.cpp:11-40
 *   FishTank::surface_sampling    scene/fishtank.cpp:108-141 (identity body transform)
 *   Cube::surface_sampling        scene/cube.cpp:136-171 (body coordinates)
 *   ModelMesh (OBJ reading)       mesh/modelmesh.cpp:16-88 with the vendored tinyobj's
 *                                 parsing rules (external/tinyobj/tiny_obj_loader.h)
 *   IcoSphereMesh                 mesh/icospheremesh.cpp:10-124
 *   Sphere::surface_sampling      scene/sphere.cpp:135-171 (body coordinates)
 *   Wall::surface_sampling        scene/wall.cpp:142-152 (body coordinates)
 * plus a seeded jitter (splitmix64, Steele/Lea/Flood 2014) used by the benchmark scenes.
 * Built without floating-point contraction, so the samplers give the same bits on every
 * host.
 */
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <random>
#include <string>
#include <utility>
#include <vector>

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

/* OBJ reading with tinyobj's rules: "v x y z [w]" and "vn x y z" records, "f" records of
 * v, v/t, v//n or v/t/n references (1-based; negative = relative to the records read so
 * far), polygons split into the fan (0, k-1, k).  Faces keep file order across groups. */
struct ObjRef {
    int v, n;
};

bool parse_ref(const char* tok, int nv, int nn, ObjRef& r) {
    char* end = nullptr;
    const long v = std::strtol(tok, &end, 10);
    if (end == tok) return false;
    auto fix = [](long i, int n) { return (int)(i > 0 ? i - 1 : (i == 0 ? 0 : n + i)); };
    r.v = fix(v, nv);
    r.n = -1;
    if (*end == '/') {
        const char* q = end + 1;
        if (*q != '/') {   /* texture index: unused */
            std::strtol(q, &end, 10);
            q = end;
        }
        if (*q == '/') {
            const long n = std::strtol(q + 1, &end, 10);
            if (end != q + 1) r.n = fix(n, nn);
        }
    }
    return true;
}

struct ObjMesh {
    std::vector<float> vertices;      /* ModelMesh vertices: one per distinct (v, n) pair */
    std::vector<uint32_t> indices;    /* 16-bit values, as mesh_index stores them */
};

int load_obj(const char* path, ObjMesh& m) {
    std::ifstream in(path, std::ios::binary);
    if (!in) return -1;
    std::vector<float> pos, nrm;
    std::map<std::pair<int, int>, int> seen;
    std::string line;
    std::vector<ObjRef> face;
    while (std::getline(in, line)) {
        const char* p = line.c_str();
        while (*p == ' ' || *p == '\t') ++p;
        if (p[0] == 'v' && (p[1] == ' ' || p[1] == '\t')) {
            char* e = const_cast<char*>(p + 1);
            for (int k = 0; k < 3; ++k) pos.push_back((float)std::strtod(e, &e));
        } else if (p[0] == 'v' && p[1] == 'n' && (p[2] == ' ' || p[2] == '\t')) {
            char* e = const_cast<char*>(p + 2);
            for (int k = 0; k < 3; ++k) nrm.push_back((float)std::strtod(e, &e));
        } else if (p[0] == 'f' && (p[1] == ' ' || p[1] == '\t')) {
            face.clear();
            const char* q = p + 1;
            for (;;) {   /* whitespace-separated references */
                while (*q == ' ' || *q == '\t' || *q == '\r') ++q;
                if (!*q) break;
                ObjRef r;
                if (!parse_ref(q, (int)(pos.size() / 3), (int)(nrm.size() / 3), r)) break;
                face.push_back(r);
                while (*q && *q != ' ' && *q != '\t' && *q != '\r') ++q;
            }
            for (size_t k = 2; k < face.size(); ++k) {
                const ObjRef tri[3] = {face[0], face[k - 1], face[k]};
                for (const ObjRef& r : tri) {
                    if (r.v < 0 || 3 * (size_t)r.v + 2 >= pos.size()) return -2;
                    const auto key = std::make_pair(r.v, r.n);
                    auto it = seen.find(key);
                    if (it != seen.end()) {
                        m.indices.push_back((uint16_t)it->second);
                        continue;
                    }
                    const int id = (int)(m.vertices.size() / 3);
                    for (int c = 0; c < 3; ++c) m.vertices.push_back(pos[3 * (size_t)r.v + c]);
                    m.indices.push_back((uint16_t)id);
                    seen[key] = id;
                }
            }
        }
    }
    return 0;
}

/* Bullet's scalar vector arithmetic on float triples (LinearMath/btVector3.h). */
struct V3 {
    float x, y, z;
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(float s, V3 a) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 unit(V3 a) {
    const float inv = 1.0f / std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
    return inv * a;
}

/* IcoSphereMesh(radius, level): the icosahedron refined level times, every face split into
 * four with three new (unshared) midpoint vertices, then every vertex projected to the
 * sphere.  The 20 starting faces are the reference's table. */
void icosphere(float radius, unsigned level, std::vector<float>& verts, std::vector<uint32_t>& idx) {
    const float t = (float)((1.0 + std::sqrt(5.0)) * 0.5);
    std::vector<V3> v = {{-1, t, 0}, {1, t, 0}, {-1, -t, 0}, {1, -t, 0}, {0, -1, t}, {0, 1, t},
                         {0, -1, -t}, {0, 1, -t}, {t, 0, -1}, {t, 0, 1}, {-t, 0, -1}, {-t, 0, 1}};
    static const uint8_t kFaces[60] = {0, 11, 5, 0, 5, 1, 0, 1, 7, 0, 7, 10, 0, 10, 11, 1, 5, 9, 5, 11,
                                       4, 11, 10, 2, 10, 7, 6, 7, 1, 8, 3, 9, 4, 3, 4, 2, 3, 2, 6, 3,
                                       6, 8, 3, 8, 9, 4, 9, 5, 2, 4, 11, 6, 2, 10, 8, 6, 7, 9, 8, 1};
    std::vector<uint32_t> f(kFaces, kFaces + 60);
    for (unsigned l = 0; l < level; ++l) {
        std::vector<uint32_t> nf;
        std::vector<V3> nv = v;
        for (size_t k = 0; k < f.size(); k += 3) {
            const uint32_t a = f[k], b = f[k + 1], c = f[k + 2];
            const uint32_t ab = (uint32_t)nv.size(), bc = ab + 1, ca = ab + 2;
            nv.push_back(0.5f * (v[a] + v[b]));
            nv.push_back(0.5f * (v[b] + v[c]));
            nv.push_back(0.5f * (v[c] + v[a]));
            const uint32_t sub[12] = {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca};
            nf.insert(nf.end(), sub, sub + 12);
        }
        f.swap(nf);
        v.swap(nv);
    }
    verts.clear();
    for (const V3& p : v) {
        const V3 q = radius * unit(p);
        verts.push_back(q.x);
        verts.push_back(q.y);
        verts.push_back(q.z);
    }
    idx.clear();
    for (uint32_t i : f) idx.push_back((uint16_t)i);
}
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

int sph_scene_load_obj(const char* path, float* vertices3, int vcap, uint32_t* indices, int icap, int* nvertices,
                       int* nindices) {
    if (!path || !nvertices || !nindices) return SPH_E_INVALID;
    ObjMesh m;
    const int rc = load_obj(path, m);
    if (rc != 0) return SPH_E_INVALID;   /* unreadable file or a face referencing no vertex */
    const size_t nv = m.vertices.size() / 3, ni = m.indices.size();
    if (nv > (size_t)INT32_MAX || ni > (size_t)INT32_MAX) return SPH_E_OVERFLOW;
    *nvertices = (int)nv;
    *nindices = (int)ni;
    if (vertices3 && vcap >= (int)nv && nv) std::memcpy(vertices3, m.vertices.data(), 12 * nv);
    if (indices && icap >= (int)ni && ni) std::memcpy(indices, m.indices.data(), 4 * ni);
    return SPH_OK;
}

int sph_scene_icosphere(float radius, int level, float* vertices3, int vcap, uint32_t* indices, int icap,
                        int* nvertices, int* nindices) {
    if (!nvertices || !nindices || level < 0 || level > 4) return SPH_E_INVALID;
    std::vector<float> v;
    std::vector<uint32_t> ix;
    icosphere(radius, (unsigned)level, v, ix);
    *nvertices = (int)(v.size() / 3);
    *nindices = (int)ix.size();
    if (vertices3 && vcap >= *nvertices) std::memcpy(vertices3, v.data(), 4 * v.size());
    if (indices && icap >= *nindices) std::memcpy(indices, ix.data(), 4 * ix.size());
    return SPH_OK;
}

int sph_scene_sphere(float radius, float spacing, float* out4, int cap) {
    if (!(spacing > 0.f) || !(radius > 0.f)) return -1;
    std::vector<float> v;
    std::vector<uint32_t> ix;
    icosphere(radius, 3, v, ix);
    Out o{out4, cap, 0};
    /* the sampler reads each corner at float offset (index, index + 1, index + 2) of the
       flat vertex array, not at 3 * index: kept, since it decides the particles */
    auto corner = [&](uint32_t i) { return V3{v[i], v[i + 1], v[i + 2]}; };
    const float area_particle = (float)(M_PI * std::pow(spacing, 2));
    for (size_t k = 0; k + 2 < ix.size(); k += 3) {
        const V3 a = corner(ix[k]), b = corner(ix[k + 1]), c = corner(ix[k + 2]);
        const V3 ab = a - b, ac = a - c;
        /* the third cross-product term is written as ab.x*ac.y - ab.x*ac.y (zero) */
        const double t0 = std::pow(ab.y * ac.z - ab.z * ac.y, 2), t1 = std::pow(ab.z * ac.x - ab.x * ac.z, 2),
                     t2 = std::pow(ab.x * ac.y - ab.x * ac.y, 2);
        const float area = (float)(0.5f * std::sqrt(t0 + t1 + t2));
        const int n = (int)(2 * std::ceil(area / area_particle));
        /* a fresh default-seeded engine per triangle: every triangle draws the same stream */
        std::default_random_engine gen;
        std::uniform_real_distribution<float> uni(0, 1);
        for (int s = 0; s < n; ++s) {
            const float r1 = std::sqrt(uni(gen));
            const float r2 = uni(gen);
            const V3 p = ((1.0f - r1) * a + (r1 * (1.0f - r2)) * b) + (r2 * r1) * c;
            o.push(p.x, p.y, p.z);
        }
    }
    for (size_t i = 0; i + 2 < v.size(); i += 3) o.push(v[i], v[i + 1], v[i + 2]);
    return o.n;
}

int sph_scene_wall(float width, float height, float spacing, float* out4, int cap) {
    if (!(spacing > 0.f) || !(width >= 0.f) || !(height >= 0.f)) return -1;
    if ((double)width / spacing > 1e6 || (double)height / spacing > 1e6) return -1;
    Out o{out4, cap, 0};
    /* a plane at z = 0: x outer, y inner, float-accumulated steps */
    for (float x = -width / 2; x <= width / 2; x += spacing)
        for (float y = -height / 2; y <= height / 2; y += spacing) o.push(x, y, 0.f);
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
