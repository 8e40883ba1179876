// ---------------------------------------------------------------------------
// C interface to the reference's own host classes — test infrastructure only.
//
// oracle/build_ref.py compiles ParallelFDTD's src/base/SimulationParameters.cpp,
// MaterialHandler.cpp and SrcRec.cpp unchanged and links them with this file
// into oracle/_ref/libref_cpu.so.  The functions below only forward to those
// classes so that Python can drive them: source samples, element coordinates,
// the parameter vector and the material table then come from the reference's
// own code when golden vectors are made.
//
// The reference logs through c_log_msg, defined in src/kernels/cudaUtils.cu,
// which is not compiled here; a silent stand-in is given instead.  Its C++
// logger (src/logger.h) appends to solver_log.txt in the working directory,
// so callers run these functions from a scratch directory.
// ---------------------------------------------------------------------------
#include <cstdarg>
#include <cstring>
#include <exception>
#include <string>
#include <vector>

#include "base/MaterialHandler.h"
#include "base/SimulationParameters.h"

extern "C" {

void c_log_msg(log_level, const char*, ...) {}

void* refh_sp_new() { return new SimulationParameters(); }
void refh_sp_free(void* h) { delete static_cast<SimulationParameters*>(h); }

// update_type: 0 SRL_FORWARD, 1 SHARED, 2 SRL (SimulationParameters.h:39)
int refh_sp_config(void* h, int update_type, double lambda, unsigned octave, unsigned steps,
                   unsigned fs, float c) {
  auto* sp = static_cast<SimulationParameters*>(h);
  try {
    sp->setUpdateType(static_cast<UpdateType>(update_type));
    if (lambda > 0) sp->setLambda(lambda);  // setUpdateType sets λ = 1/√3 first
    sp->setOctave(octave);
    sp->setNumSteps(steps);
    sp->setSpatialFs(fs);
    sp->setC(c);
  } catch (...) {
    return -1;
  }
  return 0;
}

double refh_sp_lambda(void* h) { return static_cast<SimulationParameters*>(h)->getLambda(); }
float refh_sp_dx(void* h) { return static_cast<SimulationParameters*>(h)->getDx(); }

void refh_sp_add_source(void* h, float x, float y, float z, int src_type, int input_type,
                        unsigned data_idx) {
  static_cast<SimulationParameters*>(h)->addSource(
      Source(x, y, z, static_cast<SrcType>(src_type), static_cast<InputType>(input_type),
             data_idx));
}

void refh_sp_add_receiver(void* h, float x, float y, float z) {
  static_cast<SimulationParameters*>(h)->addReceiver(x, y, z);
}

void refh_sp_add_input_f32(void* h, const float* data, unsigned n) {
  static_cast<SimulationParameters*>(h)->addInputData(std::vector<float>(data, data + n));
}

void refh_sp_add_input_f64(void* h, const double* data, unsigned n) {
  static_cast<SimulationParameters*>(h)->addInputDataDouble(std::vector<double>(data, data + n));
}

int refh_sp_read_grid_ir(void* h, const char* path) {
  try {
    static_cast<SimulationParameters*>(h)->readGridIr(std::string(path));
  } catch (...) {
    return -1;
  }
  return 0;
}

int refh_sp_source_coords(void* h, unsigned i, int* xyz) {
  try {
    nv::Vec3i v = static_cast<SimulationParameters*>(h)->getSourceElementCoordinates(i);
    xyz[0] = v.x;
    xyz[1] = v.y;
    xyz[2] = v.z;
  } catch (...) {
    return -1;
  }
  return 0;
}

int refh_sp_receiver_coords(void* h, unsigned i, int* xyz) {
  try {
    nv::Vec3i v = static_cast<SimulationParameters*>(h)->getReceiverElementCoordinates(i);
    xyz[0] = v.x;
    xyz[1] = v.y;
    xyz[2] = v.z;
  } catch (...) {
    return -1;
  }
  return 0;
}

// Samples of source i for steps [0, n): float and double paths
// (SimulationParameters.cpp:139-159).  Returns -1 if the reference throws.
int refh_sp_source_vector_f32(void* h, unsigned i, unsigned n, float* out) {
  auto* sp = static_cast<SimulationParameters*>(h);
  try {
    for (unsigned s = 0; s < n; ++s) out[s] = sp->getSourceSample(i, s);
  } catch (...) {
    return -1;
  }
  return 0;
}

int refh_sp_source_vector_f64(void* h, unsigned i, unsigned n, double* out) {
  auto* sp = static_cast<SimulationParameters*>(h);
  try {
    for (unsigned s = 0; s < n; ++s) out[s] = sp->getSourceSampleDouble(i, s);
  } catch (...) {
    return -1;
  }
  return 0;
}

void refh_sp_params_f32(void* h, float* out4) {
  std::memcpy(out4, static_cast<SimulationParameters*>(h)->getParameterPtr(), 4 * sizeof(float));
}

void refh_sp_params_f64(void* h, double* out4) {
  std::memcpy(out4, static_cast<SimulationParameters*>(h)->getParameterPtrDouble(),
              4 * sizeof(double));
}

void* refh_mh_new(int reflectances) {
  auto* m = new MaterialHandler();
  if (reflectances) m->coefsAreReflectances();
  return m;
}
void refh_mh_free(void* h) { delete static_cast<MaterialHandler*>(h); }

int refh_mh_add_materials(void* h, const float* coefs, unsigned n_surfaces, unsigned n_coef) {
  try {
    static_cast<MaterialHandler*>(h)->addMaterials(const_cast<float*>(coefs), n_surfaces, n_coef);
  } catch (...) {
    return -1;
  }
  return 0;
}

unsigned refh_mh_unique(void* h) {
  return static_cast<MaterialHandler*>(h)->getNumberOfUniqueMaterials();
}

// The device material table, [unique × 20] (MaterialHandler.cpp:100-164).
void refh_mh_table_f32(void* h, float* out) {
  auto* m = static_cast<MaterialHandler*>(h);
  std::memcpy(out, m->getMaterialCoefficientPtr(),
              sizeof(float) * m->getNumberOfUniqueMaterials() * MATERIAL_COEF_NUM);
}

void refh_mh_table_f64(void* h, double* out) {
  auto* m = static_cast<MaterialHandler*>(h);
  std::memcpy(out, m->getMaterialCoefficientPtrDouble(),
              sizeof(double) * m->getNumberOfUniqueMaterials() * MATERIAL_COEF_NUM);
}

void refh_mh_indices(void* h, unsigned char* out) {
  auto* m = static_cast<MaterialHandler*>(h);
  for (unsigned i = 0; i < m->getNumberOfSurfaces(); ++i) out[i] = (unsigned char)m->getMaterialIdxAt(i);
}

}  // extern "C"
