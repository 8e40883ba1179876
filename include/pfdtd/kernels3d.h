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

// All sp->getNumSteps() single-precision steps in one queued run, with the
// slice captures (step, orientation, slice) gathered on the device and copied
// into the caller's pinned buffers p_out[i] / pos_out[i] when their step is
// reached (no counterpart in the reference, whose capture loop steps and
// copies synchronously: App.cpp:407-436).
void launchFDTD3dCaptures(CudaMesh* d_mesh, SimulationParameters* sp, float* h_return_ptr,
                          int n_capture, const int64_t* capture_step,
                          const int32_t* capture_orientation, const int64_t* capture_slice,
                          float* const* p_out, uint8_t* const* pos_out);

#endif
