/*
 * ref_shim.h -- force-included (g++ -include) when oracle/build_ref.sh compiles the
 * reference's own sources (core.cu, preprocess.cu, mathfunc.cu, variables.cu, io.cu,
 * bb_core.cu, bb_utils.cu of dilharaj/ACUM3_periodic) as host C++.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product links this.
 *
 * What the shim does, and why each item is needed:
 *  - __global__/__device__ expand to nothing and __syncthreads() to a no-op, so the
 *    tonal kernel findPressureTimeHistory (core.cu:18) becomes a host function.
 *  - threadIdx/blockIdx are 0 and blockDim/gridDim are 1: every loop of the kernel is
 *    grid-stride (core.cu:40,46,58,239,247,253), so one "thread" walks all of
 *    (step, observer, surface, element) in order, deterministically.
 *  - atomicAdd becomes a plain read-add-write (serial execution).
 *  - With ACUM_REF_F64, `float` is redefined to `double` AFTER all system headers, which
 *    yields the FP64 build of the reference source.  Its fscanf calls use "%f"/"%e"
 *    into what are now double*, so fscanf is routed through acum_ref_fscanf, which
 *    widens those conversions to "%lf"/"%le" and leaves every other conversion alone.
 *  - malloc() is routed through acum_ref_malloc, which never hands out fewer than
 *    4096 bytes.  io.cu:478-507 accumulates a per-section debug sum into two
 *    20-entry arrays and writes past them whenever a BB surface has more than 20
 *    sections; over-allocating small blocks keeps that out-of-bounds write inside the
 *    block without changing any computed value.
 */
#ifndef ACUM_REF_SHIM_H
#define ACUM_REF_SHIM_H

#include <stdio.h>
#include <stdlib.h>
#include <stdarg.h>
#include <string.h>
#include <math.h>
#include <time.h>
#include <cmath>
#include <fstream>
#include <string>

#define __global__
#define __device__
#define __host__
#define __syncthreads() ((void)0)

struct acum_ref_dim3 { unsigned x, y, z; };
static const acum_ref_dim3 threadIdx = {0u, 0u, 0u};
static const acum_ref_dim3 blockIdx = {0u, 0u, 0u};
static const acum_ref_dim3 blockDim = {1u, 1u, 1u};
static const acum_ref_dim3 gridDim = {1u, 1u, 1u};

template <class T>
static inline T atomicAdd(T* p, T v) { T old = *p; *p = old + v; return old; }

void* acum_ref_malloc(size_t n);
#define malloc(n) acum_ref_malloc(n)

#ifdef ACUM_REF_F64
int acum_ref_fscanf(FILE* f, const char* fmt, ...);
#define fscanf acum_ref_fscanf
#define float double
#endif

#endif
