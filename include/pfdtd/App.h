// FDTD::App: the reference's orchestration class (ParallelFDTD src/App.h:50-396)
// over the single-GPU domain.  Same members and methods, minus the OpenGL
// window (there is no graphics stack here; runVisualization logs and throws).
//
// Geometry: the reference voxelizes triangles with an external GPU voxelizer
// that is not part of this library.  initializeVoxels() (an addition) takes
// already-voxelized boundary ids and materials; initializeMesh() uses them.
#ifndef PFDTD_APP_H
#define PFDTD_APP_H

#include <string>
#include <vector>

#include "MaterialHandler.h"
#include "SimulationParameters.h"
#include "cudaMesh.h"

typedef bool (*InterruptCallback)(void);
typedef void (*ProgressCallback)(int, int, float);

namespace FDTD {

class App {
 public:
  App()
      : m_parameters(SimulationParameters()),
        m_materials(MaterialHandler()),
        number_of_devices_(0),
        best_device_(0),
        force_partition_to_(-1),
        capture_db_(60),
        interrupt_(false),
        time_per_step_(0.f),
        num_elements_(0),
        current_step_(0),
        step_direction_(1) {
    loggerInit();
    setupDefaultCallbacks();
  }
  ~App();

  SimulationParameters m_parameters;
  MaterialHandler m_materials;
  CudaMesh m_mesh;
  InterruptCallback m_interrupt;
  ProgressCallback m_progress;

  void queryDevices();
  void resetDevices();
  void initializeDevices();
  void initializeGeometry(unsigned int* indices, float* vertices, unsigned int number_of_indices,
                          unsigned int number_of_vertices);
  // Voxelized geometry: boundary ids 0..27 and material bytes, x fastest,
  // dims.x * dims.y * dims.z each (the voxelizer's output format).
  void initializeVoxels(const unsigned char* boundary_ids, const unsigned char* materials,
                        uint3 dims);
  void setupDefaultCallbacks();
  void initializeMesh(unsigned int number_of_partitions);
  void runSimulation();
  void runVisualization();
  void runCapture();
  void close();
  void setCapturedB(float db) { capture_db_ = db; }
  void executeStep();
  void resetPressureMesh();
  void invertTime();
  float getTimePerStep() { return time_per_step_; }
  unsigned int getNumElements() { return num_elements_; }
  unsigned int getResponseSize() {
    return m_mesh.isDouble() ? (unsigned int)responses_double_.size()
                             : (unsigned int)responses_.size();
  }
  float getMvoxPerSec() {
    return (float)((1.f / time_per_step_ * m_mesh.getNumberOfElements()) / 1e6);
  }
  float* getResponsePointer() { return &(responses_[0]); }
  float getResponseSampleAt(unsigned int step, unsigned int rec) {
    return responses_.at(m_parameters.getNumSteps() * rec + step);
  }
  double getResponseDoubleSampleAt(unsigned int step, unsigned int rec) {
    return responses_double_.at(m_parameters.getNumSteps() * rec + step);
  }
  float* getMeshCaptureAt(unsigned int i) { return mesh_captures_.at(i); }
  unsigned int getNumberOfMeshCaptures() { return (unsigned int)mesh_captures_.size(); }
  void addSliceToCapture(unsigned int slice, unsigned int step, unsigned int orientation) {
    step_to_capture_.push_back(step);
    slice_to_capture_.push_back(slice);
    slice_orientation_.push_back(orientation);
  }
  void addMeshToCapture(unsigned int step) { mesh_to_capture_.push_back(step); }
  void saveBitmap(float* data, unsigned char* position_data, unsigned int dim_x,
                  unsigned int dim_y, unsigned int slice, unsigned int orientation,
                  unsigned int step);
  float getVolume();
  float getTotalAborptionArea(unsigned int octave);
  float getSabine(unsigned int octave);
  float getEyring(unsigned int octave);

  unsigned int current_step_;
  int step_direction_;

  void addSource(float x, float y, float z, int type, int signal, int input_signal_idx) {
    m_parameters.addSource(Source(x, y, z, (enum SrcType)type, (enum InputType)signal,
                                  input_signal_idx));
  }
  void addReceiver(float x, float y, float z) { m_parameters.addReceiver(x, y, z); }
  void setSpatialFs(unsigned int fs) { m_parameters.setSpatialFs(fs); }
  void setNumSteps(unsigned int num) { m_parameters.setNumSteps(num); }
  void setUpdateType(int i) { m_parameters.setUpdateType((enum UpdateType)i); }
  void setUniformMaterial(float R);
  std::vector<float> getResponse(unsigned int rec);
  std::vector<double> getResponseDouble(unsigned int rec);
  void setDouble(bool set_to) { m_mesh.setDouble(set_to); }
  void setForcePartitionTo(int num_partitions) { force_partition_to_ = num_partitions; }
  void addSurfaceMaterials(const float* material_coefficients, unsigned int number_of_surfaces,
                           unsigned int number_of_coefficients);
  int addMaterialToMaterialList(const std::vector<float>& coeffs);
  void addSourceDataFloat(const float* src_data, int num_steps, int num_sources);
  void addSourceDataDouble(const double* src_data, int num_steps, int num_sources);
  // Reference-behaviour switches (PFDTD_QUIRK_* bits of pfdtd.h).
  void setReferenceQuirks(int quirks) { quirks_ = quirks; }

 private:
  std::vector<unsigned int> step_to_capture_;
  std::vector<unsigned int> slice_to_capture_;
  std::vector<unsigned int> slice_orientation_;
  std::vector<unsigned int> mesh_to_capture_;
  int number_of_devices_;
  int best_device_;
  std::vector<int> device_mem_sizes_;
  int force_partition_to_;
  float capture_db_;
  bool interrupt_;
  std::vector<float> responses_;
  std::vector<double> responses_double_;
  std::vector<float*> mesh_captures_;
  float time_per_step_;
  unsigned int num_elements_;
  // geometry
  unsigned int number_of_triangles_ = 0;
  std::vector<float> mesh_vertices_;        // triangle mesh for the voxelizer
  std::vector<unsigned int> mesh_indices_;
  std::vector<unsigned char> voxel_ids_;
  std::vector<unsigned char> voxel_mats_;
  uint3 voxel_dims_ = {0, 0, 0};
  int quirks_ = 0;
};

}  // namespace FDTD

#endif
