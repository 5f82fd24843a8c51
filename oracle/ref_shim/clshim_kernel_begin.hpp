/*
 * clshim_kernel_begin.hpp -- OpenCL qualifiers and -D program constants, defined only
 * around the #include of a reference .cl file (TEST INFRASTRUCTURE, oracle/_ref only).
 * clshim_kernel_end.hpp undefines the qualifiers again.
 */
/* OpenCL address-space and access qualifiers */
#define kernel
#define __kernel
#define global
#define __global
#define local
#define __local
#define constant static const
#define read_only
#define write_only
#define __read_only
#define __write_only
#define __constant static const

/* -D program constants (opencl/clcompiler.cpp:38-54) as runtime values */
#define PARTICLE_COUNT (::clshim::g_particle_count)
#define BOUNDARY_PARTICLE_COUNT (::clshim::g_boundary_particle_count)
#define SUPPORT_RADIUS (::clshim::g_support_radius)
#define PARTICLE_MASS (::clshim::g_particle_mass)
#define REST_DENSITY (::clshim::g_rest_density)
#define CELL_SIZE (::clshim::g_cell_size)
#define GRID_SIZE (::clshim::g_grid_size)
#define CELLS_PER_SIDE (::clshim::g_cells_per_side)
/* the program's kernel family: Mueller unless this unit is the Monaghan build (the reference
 * always defines it: wcsphsimluation.cpp:370, pcisphsimluation.cpp:505,
 * boundaryhandler.cpp:413; kernels/kernels.h selects the Monaghan kernels otherwise) */
#ifndef CLSHIM_MONAGHAN
#define USE_MULLER_KERNELS 1
#endif
#define USE_MORTON_ENCODING 1
#define COMPUTE_BOUNDARY 1

