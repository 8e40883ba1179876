// ---------------------------------------------------------------------------
// CPU execution of the reference's own CUDA kernel source — test
// infrastructure only.
//
// oracle/build_ref.py compiles a few __global__ / __host__ __device__
// functions of ParallelFDTD's src/kernels/kernels3d.cu and
// src/kernels/cudaMesh.cu, taken unchanged from where the reference lies, as
// plain C++ for the host.  This prelude gives that source what it needs
// outside CUDA: the built-in index variables (one set per host thread, so a
// launch can be split over OpenMP threads), the CUDA function-space
// qualifiers as no-ops, and atomicAdd as a locked add.  A "launch" is a loop
// over every (block, thread) pair that calls the kernel function once per
// pair (oracle/ref_cpu_launch.inc).
//
// The kernels emulated this way use no __syncthreads() and no shared memory
// beyond per-block scalars that every thread writes with the same value, so
// running the threads of a block one after another gives the result of any
// parallel schedule.  The reference's fdtd3dSliced kernel, which does rely
// on shared memory between threads, is never compiled here.
//
// Floating point: compiled with -ffp-contract=off, so every product is
// rounded before it is summed, exactly as the source is written.
// ---------------------------------------------------------------------------
#ifndef PFDTD_REF_CPU_EMUL_H
#define PFDTD_REF_CPU_EMUL_H

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

struct ref_dim3 {
  unsigned int x, y, z;
};

static thread_local ref_dim3 blockIdx;
static thread_local ref_dim3 threadIdx;
static thread_local ref_dim3 blockDim;
static thread_local ref_dim3 gridDim;

#define __global__
#define __device__
#define __host__
#define __shared__
#define __forceinline__ inline

// The overload set of CUDA's integer atomicAdd, so that calls with an int
// literal convert the way they do under nvcc.
static inline unsigned int atomicAdd(unsigned int* addr, unsigned int v) {
  unsigned int old;
#pragma omp critical(ref_cpu_atomic)
  {
    old = *addr;
    *addr = old + v;
  }
  return old;
}

static inline int atomicAdd(int* addr, int v) {
  int old;
#pragma omp critical(ref_cpu_atomic)
  {
    old = *addr;
    *addr = old + v;
  }
  return old;
}

#endif
