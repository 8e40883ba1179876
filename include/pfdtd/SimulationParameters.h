// Simulation parameters, sources and receivers: the reference's class with
// the same members and behaviour (ParallelFDTD src/base/SimulationParameters.h:39-177).
#ifndef PFDTD_SIMULATIONPARAMETERS_H
#define PFDTD_SIMULATIONPARAMETERS_H

#include <cmath>
#include <string>
#include <vector>

#include "SrcRec.h"
#include "geomMath.h"

enum UpdateType { SRL_FORWARD, SHARED, SRL };

class SimulationParameters {
 public:
  SimulationParameters()
      : update_type_(SRL_FORWARD),
        c_(344.f),
        lambda_(((double)1 / std::sqrt((double)3))),
        octave_(0),
        num_steps_(1),
        spatial_fs_(7000),
        bounding_box_min_(nv::Vec3f(0.f, 0.f, 0.f)),
        bounding_box_max_(nv::Vec3f(0.f, 0.f, 0.f)),
        add_padding_to_element_idx_(true),
        version_(nextVersion()) {}
  ~SimulationParameters() {}

  void readGridIr(std::string ir_fp);
  void setUpdateType(enum UpdateType update_type);
  void setC(float c) { c_ = c; version_ = nextVersion(); }
  void setLambda(double lambda) { lambda_ = lambda; version_ = nextVersion(); }
  void setOctave(unsigned int octave) { octave_ = octave; version_ = nextVersion(); }
  void setNumSteps(unsigned int num_steps) { num_steps_ = num_steps; version_ = nextVersion(); }
  void setSpatialFs(unsigned int spatial_fs) { spatial_fs_ = spatial_fs; version_ = nextVersion(); }
  void setBoundingBox(nv::Vec3f bounding_box_min, nv::Vec3f bounding_box_max) {
    bounding_box_min_ = bounding_box_min;
    bounding_box_max_ = bounding_box_max;
  }
  void setAddPaddingToElementIdx(bool add_padding_to_element_idx) {
    add_padding_to_element_idx_ = add_padding_to_element_idx;
    version_ = nextVersion();
  }

  enum UpdateType getUpdateType() const { return update_type_; }
  float getC() const { return c_; }
  double getLambda() const { return lambda_; }
  float getDx() const;
  unsigned int getOctave() const { return octave_; }
  unsigned int getNumSteps() const { return num_steps_; }
  unsigned int getSpatialFs() const { return spatial_fs_; }
  unsigned int getStepAtTime(float t) { return (unsigned int)(spatial_fs_ * t); }

  void addSource(float x, float y, float z);
  void addSource(Source src);
  void addReceiver(float x, float y, float z) { receivers_.push_back(Receiver(x, y, z)); version_ = nextVersion(); }
  void addReceiver(Receiver rec) { receivers_.push_back(rec); version_ = nextVersion(); }
  void addSourceDData(float* d_vector);
  void removeSource(unsigned int i);
  void removeReceiver(unsigned int i);
  void updateSourceAt(unsigned int i, Source src);
  void updateReceiverAt(unsigned int i, Receiver rec);
  void resetSourcesAndReceivers();

  void addInputData(float* data, unsigned int number_of_samples);
  void addInputData(std::vector<float> data) { source_input_data_.push_back(data); version_ = nextVersion(); }
  void addInputDataDouble(std::vector<double> data) {
    source_input_data_double_.push_back(data);
    version_ = nextVersion();
  }

  float getSourceSample(unsigned int source_idx, unsigned int step);
  double getSourceSampleDouble(unsigned int source_idx, unsigned int step);
  float* getSourceDData(unsigned int source_idx) { return d_source_output_data_.at(source_idx); }
  float getInputDataSample(unsigned int idx, unsigned int sample);
  double getInputDataSampleDouble(unsigned int idx, unsigned int sample);
  float getGridIrDataSample(unsigned int sample);

  nv::Vec3i getSourceElementCoordinates(unsigned int source_idx);
  nv::Vec3i getReceiverElementCoordinates(unsigned int receiver_idx);
  unsigned int getSourceElementIdx(unsigned int source_idx, unsigned int dim_x, unsigned int dim_y);
  unsigned int getReceiverElementIdx(unsigned int receiver_idx, unsigned int dim_x, unsigned int dim_y);

  unsigned int getNumSources() const { return (unsigned int)sources_.size(); }
  unsigned int getNumReceivers() const { return (unsigned int)receivers_.size(); }
  float* getSourceVectorAt(unsigned int source_idx);

  Source getSource(unsigned int i) const { return sources_.at(i); }
  Receiver getReceiver(unsigned int i) const { return receivers_.at(i); }

  float* getParameterPtr();
  double* getParameterPtrDouble();

  // Process-wide unique stamp renewed by every change that can alter source
  // samples or element coordinates; lets callers cache precomputed tables.
  unsigned long long getVersion() const { return version_; }
  static unsigned long long nextVersion();

 private:
  float getRegularSourceSample(unsigned int source_idx, unsigned int step);
  double getRegularSourceSampleDouble(unsigned int source_idx, unsigned int step);
  float getTransparentSourceSample(unsigned int source_idx, unsigned int step);
  double getTransparentSourceSampleDouble(unsigned int source_idx, unsigned int step);

  UpdateType update_type_;
  float c_;
  double lambda_;
  unsigned int octave_;
  unsigned int num_steps_;
  unsigned int spatial_fs_;
  nv::Vec3f bounding_box_min_;
  nv::Vec3f bounding_box_max_;
  bool add_padding_to_element_idx_;
  std::vector<Source> sources_;
  std::vector<Receiver> receivers_;
  std::vector<std::vector<float> > source_input_data_;
  std::vector<std::vector<double> > source_input_data_double_;
  std::vector<std::vector<float> > source_output_data_;
  std::vector<float*> d_source_output_data_;
  std::vector<float> parameter_vec_;
  std::vector<double> parameter_vec_double_;
  std::vector<float> grid_ir_;
  unsigned long long version_;
};

#endif
