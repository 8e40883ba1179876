/*
 * pfdtd_app.h — C ABI over FDTD::App for language bindings.
 *
 * One function per method of the reference's Python module libPyFDTD
 * (ParallelFDTD src/AppPy.cpp:96-133), with plain pointers and sizes in
 * place of boost::python lists, plus initializeVoxels (voxelized geometry)
 * and setReferenceQuirks.  Every function returns PFDTD_OK or a negative
 * status; a C++ exception inside App (the reference throws int -1 on CUDA
 * errors, std::out_of_range on bad indices) becomes PFDTD_ERR_CUDA or
 * PFDTD_ERR_ARG with the message in pfdtd_last_error().
 */
#ifndef PFDTD_APP_H_C
#define PFDTD_APP_H_C

#include <stdint.h>

#include "pfdtd.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pfdtd_app pfdtd_app;

int pfdtd_app_create(pfdtd_app** out);
int pfdtd_app_destroy(pfdtd_app* app);
/* App::initializeDevices (AppPy.cpp:107) */
int pfdtd_app_initialize_devices(pfdtd_app* app);
/* App::initializeGeometryPy (AppPy.cpp:29-42, :109) */
int pfdtd_app_initialize_geometry(pfdtd_app* app, const uint32_t* indices, int64_t n_indices,
                                  const float* vertices, int64_t n_vertices);
/* Voxelized geometry: boundary ids 0..27 and material bytes, x fastest. */
int pfdtd_app_initialize_voxels(pfdtd_app* app, const uint8_t* ids, const uint8_t* mats,
                                const uint32_t dims[3]);
/* App::addSource (AppPy.cpp:111) */
int pfdtd_app_add_source(pfdtd_app* app, float x, float y, float z, int type, int signal,
                         int input_signal_idx);
/* App::addSourceDataFloat / Double (AppPy.cpp:68-92, :112-113) */
int pfdtd_app_add_source_data_float(pfdtd_app* app, const float* data, int num_steps,
                                    int num_sources);
int pfdtd_app_add_source_data_double(pfdtd_app* app, const double* data, int num_steps,
                                     int num_sources);
/* App::addReceiver (AppPy.cpp:114) */
int pfdtd_app_add_receiver(pfdtd_app* app, float x, float y, float z);
/* App::addSurfaceMaterials (AppPy.cpp:54-66, :115) */
int pfdtd_app_add_surface_materials(pfdtd_app* app, const float* coefs,
                                    unsigned int number_of_surfaces,
                                    unsigned int number_of_coefficients);
/* App::setSpatialFs, setNumSteps, setUpdateType, setUniformMaterial (AppPy.cpp:116-119) */
int pfdtd_app_set_spatial_fs(pfdtd_app* app, unsigned int fs);
int pfdtd_app_set_num_steps(pfdtd_app* app, unsigned int n);
int pfdtd_app_set_update_type(pfdtd_app* app, int update_type);
int pfdtd_app_set_uniform_material(pfdtd_app* app, float reflection);
/* App::runSimulation / runCapture / runVisualization (AppPy.cpp:120-122) */
int pfdtd_app_run_simulation(pfdtd_app* app);
int pfdtd_app_run_capture(pfdtd_app* app);
int pfdtd_app_run_visualization(pfdtd_app* app);
/* App::getResponse / getResponseDouble (AppPy.cpp:124-125): n values copied. */
int pfdtd_app_get_response(pfdtd_app* app, unsigned int rec, float* out, int64_t n);
int pfdtd_app_get_response_double(pfdtd_app* app, unsigned int rec, double* out, int64_t n);
/* forcePartitionTo, addSliceToCapture, setDouble, setCapturedB, close, getMvox,
 * getNumElems (AppPy.cpp:126-132) */
int pfdtd_app_force_partition_to(pfdtd_app* app, int n);
int pfdtd_app_add_slice_to_capture(pfdtd_app* app, unsigned int slice, unsigned int step,
                                   unsigned int orientation);
int pfdtd_app_add_mesh_to_capture(pfdtd_app* app, unsigned int step);
int pfdtd_app_set_double(pfdtd_app* app, int set_to);
int pfdtd_app_set_captured_b(pfdtd_app* app, float db);
int pfdtd_app_close(pfdtd_app* app);
int pfdtd_app_get_mvox(pfdtd_app* app, float* out);
int pfdtd_app_get_num_elems(pfdtd_app* app, unsigned int* out);
/* Extras used by the bindings. */
int pfdtd_app_get_num_steps(pfdtd_app* app, unsigned int* out);
int pfdtd_app_get_time_per_step(pfdtd_app* app, float* out);
int pfdtd_app_set_octave(pfdtd_app* app, unsigned int octave);
int pfdtd_app_set_reference_quirks(pfdtd_app* app, int quirks);
int pfdtd_app_get_mesh_dims(pfdtd_app* app, uint32_t dims[3]);
int pfdtd_app_get_dx(pfdtd_app* app, float* out);

#ifdef __cplusplus
}
#endif

#endif
