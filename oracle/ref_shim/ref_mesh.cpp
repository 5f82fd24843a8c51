/*
 * ref_mesh.cpp -- C entry points over the reference's mesh code for the oracle:
 * ModelMesh (mesh/modelmesh.cpp, tinyobj), the vendored voxelizer
 * (external/voxelizer/voxelizer.h) called as Model::surface_sampling does
 * (scene/model.cpp:170-214: voxel size = particle spacing, precision = spacing / 10), and
 * IcoSphereMesh (mesh/icospheremesh.cpp, through the btVector3 stand-in).
 * TEST INFRASTRUCTURE (oracle/_ref only): pins the library's OBJ loader, CUDA voxelizer and
 * icosphere, and generates the voxelizer's golden vectors.
 */
#include <cstring>
#include <vector>

#define VOXELIZER_IMPLEMENTATION
#include "external/voxelizer/voxelizer.h"
#include "mesh/icospheremesh.h"
#include "mesh/modelmesh.h"

extern "C" {

/* Vertices (3 floats each) and 16-bit indices of ModelMesh(path); returns 0, or -1 when
 * the file does not load.  The caller passes capacities; counts are always written. */
int ref_load_obj(const char* path, float* vertices3, int vcap, unsigned* indices, int icap, int* nv, int* ni) {
    try {
        ModelMesh m(path);
        *nv = (int)m.vertices_count();
        *ni = (int)m.indices_count();
        if (vertices3 && vcap >= *nv) std::memcpy(vertices3, m.vertices(), 12 * (size_t)*nv);
        if (indices && icap >= *ni)
            for (int i = 0; i < *ni; ++i) indices[i] = m.mesh_indices()[i];
        return 0;
    } catch (...) {
        return -1;
    }
}

/* vx_voxelize(mesh, s, s, s, precision): the output vertices (8 per voxel, the library's
 * bucket order) as float4 (w = 1).  Returns the vertex count; writes when cap suffices. */
int ref_voxelize(const float* vertices3, int nv, const unsigned* indices, int ni, float spacing, float precision,
                 float* out4, int cap) {
    vx_mesh_t* in = vx_mesh_alloc(nv, ni);
    for (int i = 0; i < nv; ++i) {
        in->vertices[i].x = vertices3[3 * i + 0];
        in->vertices[i].y = vertices3[3 * i + 1];
        in->vertices[i].z = vertices3[3 * i + 2];
    }
    for (int i = 0; i < ni; ++i) in->indices[i] = indices[i];
    vx_mesh_t* vox = vx_voxelize(in, spacing, spacing, spacing, precision);
    const int n = (int)vox->nvertices;
    if (out4 && cap >= n)
        for (int i = 0; i < n; ++i) {
            out4[4 * i + 0] = vox->vertices[i].x;
            out4[4 * i + 1] = vox->vertices[i].y;
            out4[4 * i + 2] = vox->vertices[i].z;
            out4[4 * i + 3] = 1.0f;
        }
    vx_mesh_free(in);
    vx_mesh_free(vox);
    return n;
}

/* IcoSphereMesh(radius, level): vertices and indices. */
int ref_icosphere(float radius, unsigned level, float* vertices3, int vcap, unsigned* indices, int icap, int* nv,
                  int* ni) {
    IcoSphereMesh m(radius, level);
    *nv = (int)m.vertices_count();
    *ni = (int)m.indices_count();
    if (vertices3 && vcap >= *nv) std::memcpy(vertices3, m.vertices(), 12 * (size_t)*nv);
    if (indices && icap >= *ni)
        for (int i = 0; i < *ni; ++i) indices[i] = m.mesh_indices()[i];
    return 0;
}

}  // extern "C"
