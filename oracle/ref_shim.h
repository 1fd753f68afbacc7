/* Test infrastructure only (oracle/_ref build).
 *
 * Shim that lets the reference's own SW2D kernels and host helpers
 * (SW2D-EFDC.cu, from `init_inf` up to `lake_catchment_smooth`) compile
 * unmodified as plain C++ on the CPU.  The extracted range is written by
 * oracle/build.py into oracle/_ref/ and is never committed.
 *
 * Every CUDA kernel in that range is a 1-D grid-stride loop
 *   id = blockDim.x*blockIdx.x + threadIdx.x; while (id < N) { ...; id += gridDim.x*blockDim.x; }
 * so running it with blockDim.x = 1, threadIdx.x = 0, gridDim.x = T and one
 * host thread per blockIdx.x in [0, T) visits every id exactly once.
 */
#pragma once
#include <iostream>
#include <stdlib.h>
#include <string>
#include <stdio.h>
#include <math.h>
#include <cmath>
#include <ctime>
#include <chrono>
#include <sstream>
#include <omp.h>
#include <string.h>

struct ref_dim3 {
    unsigned x, y, z;
};

extern thread_local ref_dim3 threadIdx;
extern thread_local ref_dim3 blockIdx;
extern ref_dim3 blockDim;
extern ref_dim3 gridDim;

#define __global__
#define __host__
#define __device__
