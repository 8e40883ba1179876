// Simulation parameters and source signals with the behaviour of
// ParallelFDTD src/base/SimulationParameters.cpp.
#include "SimulationParameters.h"

#include <cmath>
#include <fstream>
#include <stdexcept>

#include <atomic>

#include "logger.h"
#include "pfdtd.h"

#include <cuda_runtime.h>

unsigned long long SimulationParameters::nextVersion() {
  static std::atomic<unsigned long long> counter{0};
  return ++counter;
}

// Whitespace-separated floats; like FileReader::readFloat
// (src/io/FileReader.cpp:106-127) a value is kept only while the stream
// stays good after reading it.
void SimulationParameters::readGridIr(std::string ir_fp) {
  grid_ir_.clear();
  std::ifstream in(ir_fp.c_str());
  if (!in.good()) {
    c_log_msg(LOG_DEBUG, "grid impulse response file %s could not be read", ir_fp.c_str());
    version_ = nextVersion();
    return;
  }
  float v;
  while (true) {
    in >> v;
    if (!in.good()) break;
    grid_ir_.push_back(v);
  }
  version_ = nextVersion();
}

void SimulationParameters::addSource(float x, float y, float z) {
  sources_.push_back(Source(x, y, z));
  version_ = nextVersion();
}

void SimulationParameters::addSource(Source src) {
  sources_.push_back(src);
  version_ = nextVersion();
}

void SimulationParameters::updateSourceAt(unsigned int i, Source src) {
  if (i >= sources_.size())
    c_log_msg(LOG_ERROR, "no source %u to update", i);
  sources_.at(i) = src;
  version_ = nextVersion();
}

// The reference checks the index against the source count here
// (SimulationParameters.cpp:63) but stores into the receiver list.
void SimulationParameters::updateReceiverAt(unsigned int i, Receiver rec) {
  if (i >= sources_.size())
    c_log_msg(LOG_ERROR, "no receiver %u to update", i);
  receivers_.at(i) = rec;
  version_ = nextVersion();
}

void SimulationParameters::removeSource(unsigned int i) {
  if (i >= sources_.size()) {
    c_log_msg(LOG_ERROR, "no source %u to remove", i);
    throw std::out_of_range("SimulationParameters::removeSource: idx out of range");
  }
  sources_.erase(sources_.begin() + i);
  version_ = nextVersion();
}

void SimulationParameters::removeReceiver(unsigned int i) {
  if (i >= receivers_.size()) {
    c_log_msg(LOG_ERROR, "no receiver %u to remove", i);
    throw std::out_of_range("SimulationParameters::removeReceiver: idx out of range");
  }
  receivers_.erase(receivers_.begin() + i);
  version_ = nextVersion();
}

void SimulationParameters::resetSourcesAndReceivers() {
  receivers_.clear();
  sources_.clear();
  version_ = nextVersion();
}

void SimulationParameters::addInputData(float* data, unsigned int number_of_samples) {
  if (!data) c_log_msg(LOG_WARNING, "input data pointer is null; nothing added");
  std::vector<float> v(number_of_samples, 0.f);
  if (data)
    for (unsigned int i = 0; i < number_of_samples; ++i) v[i] = data[i];
  source_input_data_.push_back(v);
  version_ = nextVersion();
}

void SimulationParameters::addSourceDData(float* d_vector) {
  if (d_source_output_data_.size() < getNumSources()) d_source_output_data_.push_back(d_vector);
}

// Every scheme of the reference runs at lambda = 1/sqrt(3)
// (SimulationParameters.cpp:123-137).
void SimulationParameters::setUpdateType(enum UpdateType update_type) {
  update_type_ = update_type;
  if (update_type == SRL || update_type == SRL_FORWARD || update_type == SHARED)
    lambda_ = std::sqrt((double)1 / 3);
  version_ = nextVersion();
}

float SimulationParameters::getSourceSample(unsigned int source_idx, unsigned int step) {
  float sample = 0.f;
  if (getSource(source_idx).getSourceType() == SRC_TRANSPARENT)
    sample += getTransparentSourceSample(source_idx, step);
  else
    sample += getRegularSourceSample(source_idx, step);
  return sample;
}

double SimulationParameters::getSourceSampleDouble(unsigned int source_idx, unsigned int step) {
  double sample = 0.0;
  if (getSource(source_idx).getSourceType() == SRC_TRANSPARENT)
    sample += getTransparentSourceSampleDouble(source_idx, step);
  else
    sample += getRegularSourceSampleDouble(source_idx, step);
  return sample;
}

// Out-of-range data vector index throws std::out_of_range (the reference's
// vector::at, SimulationParameters.cpp:161-174); past the end gives 0.
float SimulationParameters::getInputDataSample(unsigned int idx, unsigned int sample) {
  if (idx >= source_input_data_.size())
    c_log_msg(LOG_ERROR, "no input data vector %u", idx);
  const std::vector<float>& v = source_input_data_.at(idx);
  if (sample >= v.size()) return 0.f;
  return v.at(sample);
}

double SimulationParameters::getInputDataSampleDouble(unsigned int idx, unsigned int sample) {
  if (idx >= source_input_data_double_.size())
    c_log_msg(LOG_ERROR, "no input data vector %u (double)", idx);
  const std::vector<double>& v = source_input_data_double_.at(idx);
  if (sample >= v.size()) return 0.0;
  return v.at(sample);
}

float SimulationParameters::getGridIrDataSample(unsigned int sample) {
  if (sample >= grid_ir_.size()) return 0.f;
  return grid_ir_.at(sample);
}

nv::Vec3i SimulationParameters::getSourceElementCoordinates(unsigned int source_idx) {
  nv::Vec3i r = getSource(source_idx).getElementIdx(getSpatialFs(), getC(), (float)getLambda());
  if (add_padding_to_element_idx_) { r.x += 1; r.y += 1; r.z += 1; }
  return r;
}

nv::Vec3i SimulationParameters::getReceiverElementCoordinates(unsigned int receiver_idx) {
  nv::Vec3i r = getReceiver(receiver_idx).getElementIdx(getSpatialFs(), getC(), (float)getLambda());
  if (add_padding_to_element_idx_) { r.x += 1; r.y += 1; r.z += 1; }
  return r;
}

// The reference adds the padding increment a second time here
// (SimulationParameters.cpp:226-241).
unsigned int SimulationParameters::getSourceElementIdx(unsigned int source_idx, unsigned int dim_x,
                                                       unsigned int dim_y) {
  nv::Vec3i p = getSourceElementCoordinates(source_idx);
  const unsigned inc = add_padding_to_element_idx_ ? 1u : 0u;
  p.x += inc; p.y += inc; p.z += inc;
  return p.z * dim_x * dim_y + p.y * dim_x + p.x;
}

unsigned int SimulationParameters::getReceiverElementIdx(unsigned int receiver_idx,
                                                         unsigned int dim_x, unsigned int dim_y) {
  nv::Vec3i p = getReceiver(receiver_idx).getElementIdx(getSpatialFs(), getC(), (float)getLambda());
  const unsigned inc = add_padding_to_element_idx_ ? 1u : 0u;
  p.x += inc; p.y += inc; p.z += inc;
  return p.z * dim_x * dim_y + p.y * dim_x + p.x;
}

// IMPULSE: 1 at step 1; GAUSSIAN: t0 = 40, width 4 (in steps); SINE: 120 Hz;
// DATA: the source's input vector (SimulationParameters.cpp:262-298).
float SimulationParameters::getRegularSourceSample(unsigned int source_idx, unsigned int step) {
  float sample = 0.f;
  switch (sources_.at(source_idx).getInputType()) {
    case IMPULSE:
      sample += (step == 1) ? 1.f : 0.f;
      break;
    case GAUSSIAN: {
      float t0 = 40, width = 4;
      float e = ((float)(step - t0) / width);
      sample += expf(-0.5f * (e * e));
      break;
    }
    case DATA:
      sample += getInputDataSample(sources_.at(source_idx).getInputDataIdx(), step);
      break;
    case SINE: {
      float freq = 120;
      float t = (float)step / (float)getSpatialFs();
      sample += sinf(2.f * (float)PI * freq * t);
    }
  }
  return sample;
}

// s(n) - sum_{i<n} h_grid[n-i] s(i) (SimulationParameters.cpp:300-310).
float SimulationParameters::getTransparentSourceSample(unsigned int source_idx, unsigned int step) {
  float acc = 0.f;
  for (unsigned int i = 0; i < step; ++i)
    acc += getGridIrDataSample(step - i) * getRegularSourceSample(source_idx, i);
  return getRegularSourceSample(source_idx, step) - acc;
}

double SimulationParameters::getRegularSourceSampleDouble(unsigned int source_idx, unsigned int step) {
  double sample = 0.0;
  switch (sources_.at(source_idx).getInputType()) {
    case IMPULSE:
      sample += (step == 1) ? 1.0 : 0.0;
      break;
    case GAUSSIAN: {
      double t0 = 40, width = 4;
      double e = ((float)(step - t0) / width);
      sample += exp(-0.5f * (e * e));
      break;
    }
    case DATA:
      sample += getInputDataSampleDouble(sources_.at(source_idx).getInputDataIdx(), step);
      break;
    case SINE: {
      double freq = 120;
      double t = (double)step / (double)getSpatialFs();
      sample += sin(2.f * (double)PI * freq * t);
    }
  }
  return sample;
}

double SimulationParameters::getTransparentSourceSampleDouble(unsigned int source_idx,
                                                              unsigned int step) {
  double acc = 0.0;
  for (unsigned int i = 0; i < step; ++i)
    acc += getGridIrDataSample(step - i) * getRegularSourceSampleDouble(source_idx, i);
  return getRegularSourceSampleDouble(source_idx, step) - acc;
}

// dx = c / (fs * lambda) (SimulationParameters.cpp:362-364).
float SimulationParameters::getDx() const {
  return (float)((double)getC() / ((double)getSpatialFs() * getLambda()));
}

float* SimulationParameters::getSourceVectorAt(unsigned int source_idx) {
  std::vector<float> v(getNumSteps(), 0.f);
  source_output_data_.resize(getNumSources());
  int n_dev = 0;
  if (getSource(source_idx).getSourceType() == SRC_TRANSPARENT && getNumSteps() > 0 &&
      pfdtd_device_count(&n_dev) == PFDTD_OK && n_dev > 0) {
    // The whole transparent vector on the device: O(steps * IR length) in
    // parallel instead of the per-step host sum.
    std::vector<float> regular(getNumSteps());
    for (unsigned int i = 0; i < getNumSteps(); ++i)
      regular[i] = getRegularSourceSample(source_idx, i);
    int dev = 0;
    cudaGetDevice(&dev);
    if (pfdtd_transparent_source(regular.data(), (int64_t)regular.size(),
                                 grid_ir_.empty() ? nullptr : grid_ir_.data(),
                                 (int64_t)grid_ir_.size(), v.data(), dev) != PFDTD_OK) {
      c_log_msg(LOG_ERROR, "transparent source vector: %s", pfdtd_last_error());
      throw(-1);
    }
    source_output_data_.at(source_idx) = v;
    return &(source_output_data_.at(source_idx)[0]);
  }
  for (unsigned int i = 0; i < getNumSteps(); ++i) v[i] = getSourceSample(source_idx, i);
  source_output_data_.at(source_idx) = v;
  return &(source_output_data_.at(source_idx)[0]);
}

// [lambda, lambda^2, 1/3, octave] (SimulationParameters.cpp:379-396).
float* SimulationParameters::getParameterPtr() {
  parameter_vec_.assign(4, 0.f);
  parameter_vec_[0] = (float)getLambda();
  parameter_vec_[1] = (float)(getLambda() * getLambda());
  parameter_vec_[2] = 1.f / 3.f;
  parameter_vec_[3] = (float)getOctave();
  return &parameter_vec_[0];
}

double* SimulationParameters::getParameterPtrDouble() {
  parameter_vec_double_.assign(4, 0.0);
  parameter_vec_double_[0] = getLambda();
  parameter_vec_double_[1] = getLambda() * getLambda();
  parameter_vec_double_[2] = (double)1 / (double)3;
  parameter_vec_double_[3] = (double)getOctave();
  return &parameter_vec_double_[0];
}
