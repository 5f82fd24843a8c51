/*
 * clshim_kernel_end.hpp -- undefines the OpenCL qualifiers of clshim_kernel_begin.hpp
 * (TEST INFRASTRUCTURE, oracle/_ref only).
 */
#undef kernel
#undef __kernel
#undef global
#undef __global
#undef local
#undef __local
#undef constant
#undef read_only
#undef write_only
#undef __read_only
#undef __write_only
#undef __constant
