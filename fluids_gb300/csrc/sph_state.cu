/*
 * sph_state.cu -- checkpoint and resume of a solver context (sph_save_state /
 * sph_load_state).  The reference has none: reset() rebuilds the simulation from the scene
 * (pcisphsimluation.cpp:257-266).  A file holds what the next step reads and no step
 * recomputes: the fluid's positions, velocities and half-step velocities and the particle
 * ids in the context's current order, and every body's transform, velocities and dynamics
 * -- with the parameters, container and counts they belong to, and a checksum.
 *
 * Layout (native little-endian; the loader checks each part):
 *   "SPHSTAT1"  u32 version (1)  u32 sizeof(sph_params)  sph_params  f32 container[3]
 *   i32 n_fluid  i32 n_boundary  i32 n_bodies
 *   per body: i32 count, can_move, dynamic;  f32 mass, xf[20], inv_inertia[3], radius
 *   f32 pos[4n]  f32 vel[4n]  f32 vel_half[4n]  i32 id[n]
 *   u64 FNV-1a of every byte before it
 */
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "sph_ctx.cuh"

namespace {

constexpr char kMagic[8] = {'S', 'P', 'H', 'S', 'T', 'A', 'T', '1'};
constexpr uint32_t kVersion = 1;

struct Writer {
    std::vector<unsigned char> buf;
    void put(const void* p, size_t n) {
        const unsigned char* c = static_cast<const unsigned char*>(p);
        buf.insert(buf.end(), c, c + n);
    }
    template <class T>
    void val(const T& v) {
        put(&v, sizeof v);
    }
};

struct Reader {
    const std::vector<unsigned char>& buf;
    size_t at = 0;
    bool get(void* p, size_t n) {
        if (at + n > buf.size()) return false;
        std::memcpy(p, buf.data() + at, n);
        at += n;
        return true;
    }
    template <class T>
    bool val(T& v) {
        return get(&v, sizeof v);
    }
};

uint64_t fnv1a(const unsigned char* p, size_t n) {
    uint64_t h = 1469598103934665603ull;
    for (size_t i = 0; i < n; ++i) {
        h ^= p[i];
        h *= 1099511628211ull;
    }
    return h;
}

/* the parameters a step's arithmetic depends on (launch shape and graph use do not) */
bool same_physics(sph_params a, sph_params b) {
    a.block_size = b.block_size = 0;
    a.use_graph = b.use_graph = 0;
    return std::memcmp(&a, &b, sizeof a) == 0;
}

const int kStateFields[3] = {SPH_F_POS, SPH_F_VEL, SPH_F_VEL_HALF};

}  // namespace

extern "C" {

int sph_save_state(sph_ctx* x, const char* path) {
    if (!x || !path) return SPH_E_INVALID;
    if (!x->has_state) return sph_ctx_fail(x, SPH_E_STATE, "save_state: no particles added");
    if (!x->scene_in.empty()) return sph_ctx_fail(x, SPH_E_STATE, "save_state: batched contexts are not saved");
    Writer w;
    w.put(kMagic, sizeof kMagic);
    w.val(kVersion);
    w.val((uint32_t)sizeof(sph_params));
    w.val(x->p);
    w.put(x->lim, sizeof x->lim);
    w.val((int32_t)x->N);
    w.val((int32_t)x->NB);
    w.val((int32_t)x->bodies.size());
    for (int bi = 0; bi < (int)x->bodies.size(); ++bi) {
        const SphBody& bd = x->bodies[bi];
        float xf[20];   /* the device copy: a dynamic body's pose changes there */
        const int rc = sph_get_body_state(x, bi, xf, xf + 12, xf + 16);
        if (rc != SPH_OK) return rc;
        w.val((int32_t)bd.count);
        w.val((int32_t)bd.can_move);
        w.val((int32_t)bd.dynamic);
        w.val(bd.mass);
        w.put(xf, sizeof xf);
        w.put(bd.inv_inertia, sizeof bd.inv_inertia);
        w.val(bd.radius);
    }
    std::vector<float> f4(4 * (size_t)x->N);
    for (int f : kStateFields) {
        const int rc = sph_get_field(x, f, f4.data(), 4 * f4.size());
        if (rc != SPH_OK) return rc;
        w.put(f4.data(), 4 * f4.size());
    }
    std::vector<int32_t> ids((size_t)x->N);
    int rc = sph_get_field(x, SPH_F_ID, ids.data(), 4 * ids.size());
    if (rc != SPH_OK) return rc;
    w.put(ids.data(), 4 * ids.size());
    const uint64_t sum = fnv1a(w.buf.data(), w.buf.size());
    w.val(sum);
    const std::string tmp = std::string(path) + ".tmp";
    FILE* fp = std::fopen(tmp.c_str(), "wb");
    if (!fp) return sph_ctx_fail(x, SPH_E_INVALID, std::string("save_state: cannot write ") + path);
    const bool ok = std::fwrite(w.buf.data(), 1, w.buf.size(), fp) == w.buf.size();
    if (std::fclose(fp) != 0 || !ok || std::rename(tmp.c_str(), path) != 0) {
        std::remove(tmp.c_str());
        return sph_ctx_fail(x, SPH_E_INVALID, std::string("save_state: cannot write ") + path);
    }
    return SPH_OK;
}

int sph_load_state(sph_ctx* x, const char* path) {
    if (!x || !path) return SPH_E_INVALID;
    if (!x->has_state) return sph_ctx_fail(x, SPH_E_STATE, "load_state: build the scene first");
    if (!x->scene_in.empty()) return sph_ctx_fail(x, SPH_E_STATE, "load_state: batched contexts are not saved");
    std::vector<unsigned char> buf;
    {
        FILE* fp = std::fopen(path, "rb");
        if (!fp) return sph_ctx_fail(x, SPH_E_INVALID, std::string("load_state: cannot read ") + path);
        unsigned char chunk[1 << 16];
        size_t n;
        while ((n = std::fread(chunk, 1, sizeof chunk, fp)) > 0) buf.insert(buf.end(), chunk, chunk + n);
        std::fclose(fp);
    }
    auto bad = [&](const char* why) { return sph_ctx_fail(x, SPH_E_INVALID, std::string("load_state: ") + why); };
    if (buf.size() < sizeof(kMagic) + 8 + 8) return bad("file too short");
    uint64_t sum;
    std::memcpy(&sum, buf.data() + buf.size() - 8, 8);
    if (fnv1a(buf.data(), buf.size() - 8) != sum) return bad("checksum mismatch");
    Reader r{buf};
    char magic[8];
    uint32_t version = 0, psize = 0;
    sph_params p;
    float lim[3];
    int32_t n = 0, nb = 0, nbodies = 0;
    if (!r.get(magic, 8) || std::memcmp(magic, kMagic, 8) != 0) return bad("not a state file");
    if (!r.val(version) || version != kVersion) return bad("unsupported version");
    if (!r.val(psize) || psize != sizeof(sph_params)) return bad("parameter block of another size");
    if (!r.val(p) || !same_physics(p, x->p)) return bad("parameters differ from the context's");
    if (!r.get(lim, sizeof lim) || std::memcmp(lim, x->lim, sizeof lim) != 0) return bad("container differs");
    if (!r.val(n) || !r.val(nb) || !r.val(nbodies)) return bad("truncated header");
    if (n != x->N || nb != x->NB || nbodies != (int)x->bodies.size()) return bad("particle or body counts differ");
    struct BodyRec {
        int32_t count, can_move, dynamic;
        float mass, xf[20], inv_inertia[3], radius;
    };
    std::vector<BodyRec> recs((size_t)nbodies);
    for (int bi = 0; bi < nbodies; ++bi) {
        BodyRec& b = recs[bi];
        if (!r.val(b.count) || !r.val(b.can_move) || !r.val(b.dynamic) || !r.val(b.mass) ||
            !r.get(b.xf, sizeof b.xf) || !r.get(b.inv_inertia, sizeof b.inv_inertia) || !r.val(b.radius))
            return bad("truncated body records");
        const SphBody& bd = x->bodies[bi];
        if (b.count != bd.count || b.can_move != bd.can_move || b.mass != bd.mass) return bad("bodies differ");
    }
    const size_t nf4 = 4 * (size_t)n;
    if (buf.size() - 8 - r.at != 3 * 4 * nf4 + 4 * (size_t)n) return bad("particle arrays of another size");
    const float* arrays = reinterpret_cast<const float*>(buf.data() + r.at);
    for (int k = 0; k < 3; ++k) {
        const int rc = sph_set_field(x, kStateFields[k], arrays + k * nf4, 4 * nf4);
        if (rc != SPH_OK) return rc;
    }
    int rc = sph_set_field(x, SPH_F_ID, arrays + 3 * nf4, 4 * (size_t)n);
    if (rc != SPH_OK) return rc;
    for (int bi = 0; bi < nbodies; ++bi) {
        const BodyRec& b = recs[bi];
        rc = sph_set_body_dynamics(x, bi, 0, nullptr, 0.f);   /* so the pose below is not read back */
        if (rc == SPH_OK) rc = sph_set_body_transform(x, bi, b.xf, b.xf + 12, b.xf + 16);
        if (rc == SPH_OK && b.dynamic) rc = sph_set_body_dynamics(x, bi, 1, b.inv_inertia, b.radius);
        if (rc != SPH_OK) return rc;
    }
    return SPH_OK;
}

}  // extern "C"
