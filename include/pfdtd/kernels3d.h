// Step launchers with the reference's signatures
// (ParallelFDTD src/kernels/kernels3d.h:36-90).
#ifndef PFDTD_KERNELS3D_H
#define PFDTD_KERNELS3D_H

#include "SimulationParameters.h"
#include "cudaMesh.h"

#define PROGRESS_MOD 100

// Run sp->getNumSteps() single-precision steps; receiver samples go to
// h_return_ptr[rec * num_steps + step].  Returns seconds per step (wall time).
float launchFDTD3d(CudaMesh* d_mesh, SimulationParameters* sp, float* h_return_ptr,
                   bool (*interruptCallback)(void), void (*progressCallback)(int, int, float));

// Double-precision variant.
float launchFDTD3dDouble(CudaMesh* d_mesh, SimulationParameters* sp, double* h_return_ptr,
                         bool (*interruptCallback)(void),
                         void (*progressCallback)(int, int, float));

// One single-precision step in capture mode; step_direction -1 reverses time.
void launchFDTD3dStep(CudaMesh* d_mesh, SimulationParameters* sp, float* h_return_ptr,
                      unsigned int step, int step_direction,
                      void (*progressCallback)(int, int, float));

#endif
