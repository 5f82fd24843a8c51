/*
 * ref_grid.cpp -- C entry points running the reference's kernels/grid.cl on the CPU.
 * TEST INFRASTRUCTURE (oracle/_ref only).  Launch shapes follow fluid/simulation/grid.cpp:
 * compute_hashes and compute_cell_intervals with local size 32 (grid.cpp:32,53).
 */
#include "clshim.hpp"

#include <algorithm>
#include <cstring>

#include "clshim_kernel_begin.hpp"
namespace ref_grid {
#include "grid.cl"
}
#include "clshim_kernel_end.hpp"

using namespace clshim;

static ref_grid::GridInfo make_info(float size, float cell_size, int cps) {
    ref_grid::GridInfo gi;
    gi.size = size;
    gi.cell_size = cell_size;
    gi.cells_per_side = cps;
    gi.cells_count = cps * cps * cps;
    return gi;
}

extern "C" {

void ref_compute_hashes(const float* pos4, int n, float size, float cell_size, int cps,
                        uint32_t* hashes, int32_t* mask) {
    ref_grid::GridInfo gi = make_info(size, cell_size, cps);
    run_ndrange((size_t)n, 32, false, [&] {
        ref_grid::compute_hashes(reinterpret_cast<const float4*>(pos4), hashes, mask, gi, n);
    });
}

/* CLAllocator::fill_buffer of the cell table with zeros (grid.cpp:41) on the host's threads:
 * n ints in chunks of 65,536 as independent work-groups. */
void ref_fill_zero(int32_t* p, long long n) {
    const size_t chunk = 65536;
    const size_t groups = (size_t)((n + (long long)chunk - 1) / (long long)chunk);
    run_ndrange(groups, 1, false, [&] {
        const size_t g = get_global_id(0);
        const size_t a = g * chunk, b = std::min((size_t)n, a + chunk);
        std::memset(p + a, 0, 4 * (b - a));
    });
}

/* intervals: 2 * cps^3 ints, zero-filled by the caller (grid.cpp:41). */
void ref_compute_cell_intervals(const float* spos4, const uint32_t* hashes, int n, float size,
                                float cell_size, int cps, int32_t* intervals) {
    ref_grid::GridInfo gi = make_info(size, cell_size, cps);
    const size_t local = 32;
    run_ndrange((size_t)n, local, true, [&] {
        ref_grid::compute_cell_intervals(reinterpret_cast<const float4*>(spos4), hashes, intervals,
                                         static_cast<float4*>(group_local(0, sizeof(float4) * local)), static_cast<uint*>(group_local(1, sizeof(uint) * local)), gi, n);
    });
}

/* cell_size_define: the CELL_SIZE -D constant (6-decimal rounding) used by SQR_SUPPORT_RADIUS. */
void ref_compute_neigh_list(const float* ref_pos4, int nref, const float* neigh_pos4,
                            const int32_t* intervals, float size, float cell_size,
                            float cell_size_define, int cps, int32_t* list, int32_t* len) {
    ref_grid::GridInfo gi = make_info(size, cell_size, cps);
    g_cell_size = cell_size_define;
    image1d_buffer_t im{neigh_pos4, 4};
    run_ndrange((size_t)nref, 64, false, [&] {
        ref_grid::compute_neigh_list(reinterpret_cast<const float4*>(ref_pos4), im,
                                     reinterpret_cast<const int2*>(intervals), list, len, gi, nref);
    });
}

}  // extern "C"
