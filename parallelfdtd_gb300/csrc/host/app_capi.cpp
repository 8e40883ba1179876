// C ABI over FDTD::App (declared in include/pfdtd_app.h).
#include "pfdtd_app.h"

#include <stdexcept>
#include <string>

#include "App.h"

namespace pfdtd {
int fail(int code, const std::string& msg);
}

struct pfdtd_app {
  FDTD::App app;
};

namespace {

template <typename F>
int guarded(pfdtd_app* a, F&& f) {
  if (!a) return pfdtd::fail(PFDTD_ERR_ARG, "null app");
  try {
    f(a->app);
    return PFDTD_OK;
  } catch (const std::out_of_range& e) {
    return pfdtd::fail(PFDTD_ERR_ARG, e.what());
  } catch (int) {
    const std::string m = pfdtd_last_error();
    return pfdtd::fail(PFDTD_ERR_CUDA, m.empty() ? "App call failed" : m);
  } catch (const std::exception& e) {
    return pfdtd::fail(PFDTD_ERR_CUDA, e.what());
  }
}

}  // namespace

extern "C" {

int pfdtd_app_create(pfdtd_app** out) {
  if (!out) return pfdtd::fail(PFDTD_ERR_ARG, "null output");
  *out = new pfdtd_app();
  return PFDTD_OK;
}

int pfdtd_app_destroy(pfdtd_app* app) {
  delete app;
  return PFDTD_OK;
}

int pfdtd_app_initialize_devices(pfdtd_app* a) {
  return guarded(a, [](FDTD::App& app) { app.initializeDevices(); });
}

int pfdtd_app_initialize_geometry(pfdtd_app* a, const uint32_t* indices, int64_t n_indices,
                                  const float* vertices, int64_t n_vertices) {
  return guarded(a, [&](FDTD::App& app) {
    app.initializeGeometry((unsigned int*)indices, (float*)vertices, (unsigned)n_indices,
                           (unsigned)n_vertices);
  });
}

int pfdtd_app_initialize_voxels(pfdtd_app* a, const uint8_t* ids, const uint8_t* mats,
                                const uint32_t dims[3]) {
  if (!ids || !mats || !dims) return pfdtd::fail(PFDTD_ERR_ARG, "null voxel arrays");
  return guarded(a, [&](FDTD::App& app) {
    app.initializeVoxels(ids, mats, make_uint3(dims[0], dims[1], dims[2]));
  });
}

int pfdtd_app_add_source(pfdtd_app* a, float x, float y, float z, int type, int signal,
                         int input_signal_idx) {
  return guarded(a, [&](FDTD::App& app) { app.addSource(x, y, z, type, signal, input_signal_idx); });
}

int pfdtd_app_add_source_data_float(pfdtd_app* a, const float* data, int num_steps, int num_sources) {
  return guarded(a, [&](FDTD::App& app) { app.addSourceDataFloat(data, num_steps, num_sources); });
}

int pfdtd_app_add_source_data_double(pfdtd_app* a, const double* data, int num_steps, int num_sources) {
  return guarded(a, [&](FDTD::App& app) { app.addSourceDataDouble(data, num_steps, num_sources); });
}

int pfdtd_app_add_receiver(pfdtd_app* a, float x, float y, float z) {
  return guarded(a, [&](FDTD::App& app) { app.addReceiver(x, y, z); });
}

int pfdtd_app_add_surface_materials(pfdtd_app* a, const float* coefs, unsigned int n_surf,
                                    unsigned int n_coef) {
  return guarded(a, [&](FDTD::App& app) { app.addSurfaceMaterials(coefs, n_surf, n_coef); });
}

int pfdtd_app_set_spatial_fs(pfdtd_app* a, unsigned int fs) {
  return guarded(a, [&](FDTD::App& app) { app.setSpatialFs(fs); });
}

int pfdtd_app_set_num_steps(pfdtd_app* a, unsigned int n) {
  return guarded(a, [&](FDTD::App& app) { app.setNumSteps(n); });
}

int pfdtd_app_set_update_type(pfdtd_app* a, int t) {
  return guarded(a, [&](FDTD::App& app) { app.setUpdateType(t); });
}

int pfdtd_app_set_uniform_material(pfdtd_app* a, float r) {
  return guarded(a, [&](FDTD::App& app) { app.setUniformMaterial(r); });
}

int pfdtd_app_run_simulation(pfdtd_app* a) {
  return guarded(a, [](FDTD::App& app) { app.runSimulation(); });
}

int pfdtd_app_run_capture(pfdtd_app* a) {
  return guarded(a, [](FDTD::App& app) { app.runCapture(); });
}

int pfdtd_app_run_visualization(pfdtd_app* a) {
  return guarded(a, [](FDTD::App& app) { app.runVisualization(); });
}

int pfdtd_app_get_response(pfdtd_app* a, unsigned int rec, float* out, int64_t n) {
  return guarded(a, [&](FDTD::App& app) {
    std::vector<float> r = app.getResponse(rec);
    for (int64_t i = 0; i < n && i < (int64_t)r.size(); ++i) out[i] = r[i];
  });
}

int pfdtd_app_get_response_double(pfdtd_app* a, unsigned int rec, double* out, int64_t n) {
  return guarded(a, [&](FDTD::App& app) {
    std::vector<double> r = app.getResponseDouble(rec);
    for (int64_t i = 0; i < n && i < (int64_t)r.size(); ++i) out[i] = r[i];
  });
}

int pfdtd_app_force_partition_to(pfdtd_app* a, int n) {
  return guarded(a, [&](FDTD::App& app) { app.setForcePartitionTo(n); });
}

int pfdtd_app_add_slice_to_capture(pfdtd_app* a, unsigned int slice, unsigned int step,
                                   unsigned int orientation) {
  return guarded(a, [&](FDTD::App& app) { app.addSliceToCapture(slice, step, orientation); });
}

int pfdtd_app_add_mesh_to_capture(pfdtd_app* a, unsigned int step) {
  return guarded(a, [&](FDTD::App& app) { app.addMeshToCapture(step); });
}

int pfdtd_app_set_double(pfdtd_app* a, int set_to) {
  return guarded(a, [&](FDTD::App& app) { app.setDouble(set_to != 0); });
}

int pfdtd_app_set_captured_b(pfdtd_app* a, float db) {
  return guarded(a, [&](FDTD::App& app) { app.setCapturedB(db); });
}

int pfdtd_app_close(pfdtd_app* a) {
  return guarded(a, [](FDTD::App& app) { app.close(); });
}

int pfdtd_app_get_mvox(pfdtd_app* a, float* out) {
  return guarded(a, [&](FDTD::App& app) { *out = app.getMvoxPerSec(); });
}

int pfdtd_app_get_num_elems(pfdtd_app* a, unsigned int* out) {
  return guarded(a, [&](FDTD::App& app) { *out = app.getNumElements(); });
}

int pfdtd_app_get_num_steps(pfdtd_app* a, unsigned int* out) {
  return guarded(a, [&](FDTD::App& app) { *out = app.m_parameters.getNumSteps(); });
}

int pfdtd_app_get_time_per_step(pfdtd_app* a, float* out) {
  return guarded(a, [&](FDTD::App& app) { *out = app.getTimePerStep(); });
}

int pfdtd_app_set_octave(pfdtd_app* a, unsigned int octave) {
  return guarded(a, [&](FDTD::App& app) { app.m_parameters.setOctave(octave); });
}

int pfdtd_app_set_reference_quirks(pfdtd_app* a, int quirks) {
  return guarded(a, [&](FDTD::App& app) { app.setReferenceQuirks(quirks); });
}

int pfdtd_app_get_mesh_dims(pfdtd_app* a, uint32_t dims[3]) {
  return guarded(a, [&](FDTD::App& app) {
    dims[0] = app.m_mesh.getDimX();
    dims[1] = app.m_mesh.getDimY();
    dims[2] = app.m_mesh.getDimZ();
  });
}

int pfdtd_app_get_dx(pfdtd_app* a, float* out) {
  return guarded(a, [&](FDTD::App& app) { *out = app.m_parameters.getDx(); });
}

}  // extern "C"
