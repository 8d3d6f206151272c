/*
 * ref_shim.h - lets the reference's kernel bodies compile as host C++.
 *
 * TEST INFRASTRUCTURE ONLY.  Force-included (-include) when oracle/Makefile
 * compiles line ranges of the reference sources (read in place from the
 * reference tree) into oracle/_ref/libmtref.so.  CUDA qualifiers become
 * empty, the fast-math intrinsics become libm calls, and the launch indices
 * become thread-local variables that ref_harness.cpp sets per bead.
 */
#pragma once
#include <cmath>
#include <cstdlib>
#include <climits>
#include <vector_types.h>
#include <vector_functions.h>
#undef __global__
#undef __device__
#undef __constant__
#undef __host__
#undef __forceinline__
#define __global__
#define __device__
#define __constant__
#define __host__
#define __forceinline__ inline
#define __sinf sinf
#define __cosf cosf
using std::isnan;
struct shim_dim3 {
    unsigned x, y, z;
};
extern thread_local shim_dim3 blockIdx, threadIdx, blockDim;
