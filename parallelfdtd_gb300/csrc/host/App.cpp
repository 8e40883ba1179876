// FDTD::App over the single-GPU domain, with the behaviour of
// ParallelFDTD src/App.cpp minus the OpenGL window and the external
// triangle voxelizer.
#include "App.h"

#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>

#include "global_includes.h"
#include "kernels3d.h"

namespace {

FDTD::App* g_current_app = nullptr;
volatile bool g_interrupt = false;

bool default_interrupt() { return g_interrupt; }

void default_progress(int step, int max_step, float t_per_step) {
  const float estimate = t_per_step * (float)(max_step - step);
  std::printf("Step %d/%d, time per step %f, estimated time left %f s \n", step, max_step,
              t_per_step, estimate);
}

void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    c_log_msg(LOG_ERROR, "%s: %s", what, cudaGetErrorString(e));
    throw(-1);
  }
}

// Uncompressed 32-bit BGRA TGA, pixel (row i, column j) at width*i + j, as
// the reference's TGAImage (src/io/Image.cpp:44-82).
void write_tga(const std::string& path, const std::vector<unsigned char>& rgba, int w, int h) {
  std::ofstream o(path.c_str(), std::ios::out | std::ios::binary);
  const unsigned char hdr[18] = {0, 0, 2, 0, 0, 0, 0, 0, 0, 0, 0, 0,
                                 (unsigned char)(w & 0xFF), (unsigned char)((w & 0xFF00) / 256),
                                 (unsigned char)(h & 0xFF), (unsigned char)((h & 0xFF00) / 256),
                                 32, 0};
  o.write((const char*)hdr, 18);
  for (int i = 0; i < w * h; ++i) {
    o.put(rgba[4 * i + 2]);
    o.put(rgba[4 * i + 1]);
    o.put(rgba[4 * i + 0]);
    o.put(rgba[4 * i + 3]);
  }
}

}  // namespace

namespace FDTD {

App::~App() {
  for (float* p : mesh_captures_) std::free(p);
  m_mesh.destroyPartitions();
}

void App::setupDefaultCallbacks() {
  m_interrupt = default_interrupt;
  m_progress = default_progress;
}

void App::queryDevices() {
  int n = 0;
  pfdtd_device_count(&n);
  number_of_devices_ = n;
  best_device_ = 0;
  device_mem_sizes_.clear();
  for (int i = 0; i < n; ++i) {
    cudaSetDevice(i);
    size_t free_mem = 0, total_mem = 0;
    cuda_check(cudaMemGetInfo(&free_mem, &total_mem), "App::queryDevices - cudaMemGetInfo");
    device_mem_sizes_.push_back((int)(free_mem / 1e6f));
  }
  if (n > 0) cudaSetDevice(best_device_);
}

// The reference resets every device here (App.cpp:114-120); resetting would
// destroy other users' state in this process's context, so only the
// domain is released.
void App::resetDevices() { m_mesh.destroyPartitions(); }

void App::initializeDevices() {
  queryDevices();
  g_current_app = this;
}

// The triangle mesh (App.cpp:141-145); voxelized on the device by
// initializeMesh unless voxels were given with initializeVoxels.
void App::initializeGeometry(unsigned int* indices, float* vertices,
                             unsigned int number_of_indices, unsigned int number_of_vertices) {
  number_of_triangles_ = indices ? number_of_indices / 3 : 0;
  mesh_indices_.assign(indices, indices + (indices ? number_of_indices : 0));
  // number_of_vertices counts floats, as GeometryHandler::initialize
  // (GeometryHandler.cpp:87-100)
  mesh_vertices_.assign(vertices, vertices + (vertices ? (size_t)number_of_vertices : 0));
  voxel_ids_.clear();
  voxel_mats_.clear();
}

void App::initializeVoxels(const unsigned char* ids, const unsigned char* mats, uint3 dims) {
  const size_t n = (size_t)dims.x * dims.y * dims.z;
  voxel_ids_.assign(ids, ids + n);
  voxel_mats_.assign(mats, mats + n);
  voxel_dims_ = dims;
}

void App::setUniformMaterial(float R) {
  m_materials.setGlobalMaterial(number_of_triangles_, reflection2Admitance(R));
}

// Voxel upload, mesh set-up and the reference's partition decision
// (App.cpp:147-234); every partition count maps to one domain.
void App::initializeMesh(unsigned int number_of_partitions) {
  if (voxel_ids_.empty() && !mesh_indices_.empty()) {
    // voxelizeGeometry (App.cpp:181-191): voxel edge = dx, one material byte
    // per triangle from the material handler
    uint32_t dims[3];
    double origin[3];
    const unsigned char* tri_mat = m_materials.getMaterialIdxPtr();
    std::vector<unsigned char> zeros;
    if (!tri_mat || m_materials.getNumberOfSurfaces() < number_of_triangles_) {
      zeros.assign(number_of_triangles_, 0);
      tri_mat = zeros.data();
    }
    int dev = 0;
    cudaGetDevice(&dev);
    const int64_t nv = (int64_t)mesh_vertices_.size() / 3, nt = (int64_t)number_of_triangles_;
    const double dx = (double)m_parameters.getDx();
    if (pfdtd_voxelize(mesh_vertices_.data(), nv, mesh_indices_.data(), nt, tri_mat, dx, dev,
                       dims, origin, nullptr, nullptr) != PFDTD_OK) {
      c_log_msg(LOG_ERROR, "App::initializeMesh - voxelization: %s", pfdtd_last_error());
      throw(-1);
    }
    const size_t n = (size_t)dims[0] * dims[1] * dims[2];
    voxel_ids_.assign(n, 0);
    voxel_mats_.assign(n, 0);
    if (pfdtd_voxelize(mesh_vertices_.data(), nv, mesh_indices_.data(), nt, tri_mat, dx, dev,
                       dims, origin, voxel_ids_.data(), voxel_mats_.data()) != PFDTD_OK) {
      c_log_msg(LOG_ERROR, "App::initializeMesh - voxelization: %s", pfdtd_last_error());
      throw(-1);
    }
    voxel_dims_ = make_uint3(dims[0], dims[1], dims[2]);
  }
  if (voxel_ids_.empty()) {
    c_log_msg(LOG_ERROR,
              "App::initializeMesh - no geometry: call initializeGeometry (triangle mesh) or "
              "initializeVoxels first");
    throw(-1);
  }
  if (m_materials.getNumberOfUniqueMaterials() == 0) {
    c_log_msg(LOG_ERROR, "App::initializeMesh - no materials assigned");
    throw(-1);
  }
  const bool dbl = m_mesh.isDouble();
  m_mesh.destroyPartitions();
  m_mesh = CudaMesh();
  m_mesh.setDouble(dbl);
  const size_t n = voxel_ids_.size();
  unsigned char *d_pos = NULL, *d_mat = NULL;
  cuda_check(cudaMalloc((void**)&d_pos, n + 1 + voxel_dims_.x), "App::initializeMesh - alloc");
  cuda_check(cudaMalloc((void**)&d_mat, n + 1 + voxel_dims_.x), "App::initializeMesh - alloc");
  cuda_check(cudaMemset(d_pos, 0, n + 1 + voxel_dims_.x), "App::initializeMesh - clear");
  cuda_check(cudaMemset(d_mat, 0, n + 1 + voxel_dims_.x), "App::initializeMesh - clear");
  cuda_check(cudaMemcpy(d_pos, voxel_ids_.data(), n, cudaMemcpyHostToDevice), "App::initializeMesh - upload");
  cuda_check(cudaMemcpy(d_mat, voxel_mats_.data(), n, cudaMemcpyHostToDevice), "App::initializeMesh - upload");
  uint3 block_size = make_uint3(32, 4, 1);
  if (dbl)
    m_mesh.setupMeshDouble(d_pos, d_mat, m_materials.getNumberOfUniqueMaterials(),
                           m_materials.getMaterialCoefficientPtrDouble(),
                           m_parameters.getParameterPtrDouble(), voxel_dims_, block_size,
                           (unsigned int)m_parameters.getUpdateType());
  else
    m_mesh.setupMesh(d_pos, d_mat, m_materials.getNumberOfUniqueMaterials(),
                     m_materials.getMaterialCoefficientPtr(), m_parameters.getParameterPtr(),
                     voxel_dims_, block_size, (unsigned int)m_parameters.getUpdateType());
  num_elements_ = m_mesh.getNumberOfElements();
  unsigned int element_limit = (unsigned int)90e6;
  if (dbl) element_limit /= 2;
  if (force_partition_to_ != -1 && force_partition_to_ <= number_of_devices_)
    m_mesh.makePartition((unsigned)force_partition_to_);
  else if (num_elements_ < element_limit)
    m_mesh.makePartition(1);
  else
    m_mesh.makePartition(number_of_partitions);
  if (quirks_) pfdtd_set_quirks(m_mesh.getDomain(), quirks_);
}

void App::runSimulation() {
  initializeMesh(2);
  if (m_mesh.isDouble()) {
    responses_double_.assign((size_t)m_parameters.getNumSteps() * m_parameters.getNumReceivers(), 0.0);
    time_per_step_ = launchFDTD3dDouble(&m_mesh, &m_parameters, responses_double_.data(),
                                        m_interrupt, m_progress);
  } else {
    responses_.assign((size_t)m_parameters.getNumSteps() * m_parameters.getNumReceivers(), 0.f);
    time_per_step_ = launchFDTD3d(&m_mesh, &m_parameters, responses_.data(), m_interrupt,
                                  m_progress);
  }
  c_log_msg(LOG_INFO, "App::runSimulation - Performance Mvox/sec: %f", getMvoxPerSec());
}

void App::runVisualization() {
  c_log_msg(LOG_ERROR, "App::runVisualization - no OpenGL window in this build; use runCapture");
  throw(-1);
}

// App.cpp:385-405: the reference steps one at a time, capturing the
// scheduled slices and meshes after each step.  Forward runs from step 0
// with slice captures only take the asynchronous captured run instead (one
// run, graph-replayed chunks, device gathers and asynchronous copies; the
// interrupt callback is polled once, before the run); the bitmaps are the
// same.
void App::runCapture() {
  m_mesh.setDouble(false);
  initializeMesh(2);
  const unsigned steps = m_parameters.getNumSteps();
  responses_.assign((size_t)steps * m_parameters.getNumReceivers(), 0.f);
  if (step_direction_ == 1 && current_step_ == 0 && mesh_to_capture_.empty()) {
    if (m_interrupt && m_interrupt()) return;
    std::vector<int64_t> cs, sl;
    std::vector<int32_t> co;
    std::vector<unsigned> w, h;
    for (size_t i = 0; i < step_to_capture_.size(); ++i) {
      const unsigned st = step_to_capture_[i], slice = slice_to_capture_[i];
      const unsigned o = slice_orientation_[i];
      const unsigned lim = o == 0 ? m_mesh.getDimZ() : (o == 1 ? m_mesh.getDimY() : m_mesh.getDimX());
      if (st < 1 || st > steps || o > 2) continue;  // never reached by the stepping loop
      if (slice >= lim) {
        c_log_msg(LOG_INFO, "captureSliceFast - slice %u out of bounds, no capture made", slice);
        continue;
      }
      cs.push_back(st);
      co.push_back((int32_t)o);
      sl.push_back(slice);
      w.push_back(o == 2 ? m_mesh.getDimY() : m_mesh.getDimX());
      h.push_back(o == 0 ? m_mesh.getDimY() : m_mesh.getDimZ());
    }
    const size_t n = cs.size();
    std::vector<float*> pp(n, nullptr);
    std::vector<uint8_t*> qq(n, nullptr);
    int rc = PFDTD_OK;
    for (size_t i = 0; i < n && rc == PFDTD_OK; ++i) {
      rc = pfdtd_host_alloc((size_t)w[i] * h[i] * sizeof(float), (void**)&pp[i]);
      if (rc == PFDTD_OK) rc = pfdtd_host_alloc((size_t)w[i] * h[i], (void**)&qq[i]);
    }
    auto free_all = [&]() {
      for (size_t i = 0; i < n; ++i) {
        pfdtd_host_free(pp[i]);
        pfdtd_host_free(qq[i]);
      }
    };
    if (rc != PFDTD_OK) {
      free_all();
      c_log_msg(LOG_ERROR, "App::runCapture - %s", pfdtd_last_error());
      throw(-1);
    }
    try {
      launchFDTD3dCaptures(&m_mesh, &m_parameters, responses_.empty() ? nullptr : responses_.data(),
                           (int)n, cs.data(), co.data(), sl.data(), pp.data(), qq.data());
    } catch (...) {
      free_all();
      throw;
    }
    for (size_t i = 0; i < n; ++i)
      saveBitmap(pp[i], qq[i], w[i], h[i], (unsigned)sl[i], (unsigned)co[i], (unsigned)cs[i]);
    free_all();
    current_step_ = steps;
    return;
  }
  for (unsigned i = 0; i < steps; ++i) {
    executeStep();
    if (m_interrupt && m_interrupt()) break;
  }
}

void App::resetPressureMesh() {
  m_mesh.resetPressures();
  current_step_ = 0;
}

void App::invertTime() { step_direction_ *= -1; }

// One step, then the slice and mesh captures scheduled at the new step index
// (App.cpp:407-436, visualizationUtils.cu:111-254).
void App::executeStep() {
  launchFDTD3dStep(&m_mesh, &m_parameters, responses_.empty() ? NULL : &responses_[0],
                   current_step_, step_direction_, m_progress);
  current_step_ += step_direction_;
  pfdtd_domain* d = m_mesh.getDomain();
  for (size_t i = 0; i < step_to_capture_.size(); ++i) {
    if (current_step_ != step_to_capture_[i]) continue;
    const unsigned slice = slice_to_capture_[i], orient = slice_orientation_[i];
    const unsigned w = orient == 2 ? m_mesh.getDimY() : m_mesh.getDimX();
    const unsigned h = orient == 0 ? m_mesh.getDimY() : m_mesh.getDimZ();
    std::vector<float> p((size_t)w * h);
    std::vector<unsigned char> q((size_t)w * h);
    if (pfdtd_capture_slice(d, (int)orient, slice, p.data(), q.data()) != PFDTD_OK) {
      c_log_msg(LOG_INFO, "captureSliceFast - slice %u out of bounds, no capture made", slice);
      return;
    }
    saveBitmap(p.data(), q.data(), w, h, slice, orient, current_step_);
  }
  for (size_t i = 0; i < mesh_to_capture_.size(); ++i) {
    if (current_step_ != mesh_to_capture_[i]) continue;
    if (m_mesh.isDouble()) continue;  // single-precision captures only, as the reference
    const size_t n = m_mesh.getNumberOfElements();
    float* data = (float*)std::malloc(n * sizeof(float));
    if (pfdtd_download_field(d, PFDTD_FIELD_CURRENT, data) != PFDTD_OK) {
      std::free(data);
      throw(-1);
    }
    mesh_captures_.push_back(data);
  }
}

void App::close() {
  m_mesh.destroyPartitions();
}

float App::getVolume() {
  const float n = (float)m_mesh.getNumberOfAirElements() + (float)m_mesh.getNumberOfBoundaryElements();
  const float dx = m_parameters.getDx();
  return dx * dx * dx * n;
}

float App::getTotalAborptionArea(unsigned int octave) {
  (void)octave;
  return 0.f;  // needs triangle areas (geometry handling is not part of this library)
}

float App::getSabine(unsigned int octave) {
  const float a = getTotalAborptionArea(octave);
  return a > 0.f ? 0.1611f * getVolume() / a : 0.f;
}

float App::getEyring(unsigned int octave) {
  (void)octave;
  return 0.f;
}

// dB-scaled pressure image, white for boundary nodes (App.cpp:492-567).
void App::saveBitmap(float* data, unsigned char* position_data, unsigned int dim_x,
                     unsigned int dim_y, unsigned int slice, unsigned int orientation,
                     unsigned int step) {
  std::vector<unsigned char> px((size_t)dim_x * dim_y * 4, 0);
  const float dB = capture_db_ / 10.f;
  for (unsigned i = 0; i < dim_y; ++i)
    for (unsigned j = 0; j < dim_x; ++j) {
      const size_t k = (size_t)i * dim_x + j;
      unsigned char* o = &px[4 * k];
      const unsigned char cp = position_data[k];
      o[3] = 255;
      if ((cp >> 7) == 0x01 && (cp & 0x7F) != 0x06) {
        o[0] = o[1] = o[2] = 255;
        continue;
      }
      float c = data[k];
      const float sign = c > 0.f ? 1.f : -1.f;
      c = ((std::log10(c * c) + dB) / dB);
      c = c > 0 ? c : 0.f;
      const float cp_ = sign >= 0 ? c : 0.f, cn = sign < 0 ? c : 0.f;
      o[0] = 0;
      o[1] = (unsigned char)(cp_ * 255);
      o[2] = (unsigned char)(cn * 255);
    }
  std::stringstream ss;
  ss << "capture_" << orientation << "_" << step << "_" << slice << ".tga";
  write_tga(ss.str(), px, (int)dim_x, (int)dim_y);
}

std::vector<float> App::getResponse(unsigned int rec) {
  std::vector<float> r(m_parameters.getNumSteps(), 0.f);
  for (unsigned i = 0; i < m_parameters.getNumSteps(); ++i) r[i] = getResponseSampleAt(i, rec);
  return r;
}

std::vector<double> App::getResponseDouble(unsigned int rec) {
  std::vector<double> r(m_parameters.getNumSteps(), 0.0);
  for (unsigned i = 0; i < m_parameters.getNumSteps(); ++i) r[i] = getResponseDoubleSampleAt(i, rec);
  return r;
}

void App::addSurfaceMaterials(const float* coefs, unsigned int number_of_surfaces,
                              unsigned int number_of_coefficients) {
  std::vector<float> v(coefs, coefs + (size_t)number_of_surfaces * number_of_coefficients);
  m_materials.addMaterials(v.data(), number_of_surfaces, number_of_coefficients);
}

int App::addMaterialToMaterialList(const std::vector<float>& coeffs) {
  return (int)m_materials.addSurfaceMaterial(coeffs);
}

void App::addSourceDataFloat(const float* src_data, int num_steps, int num_sources) {
  std::vector<float> v(src_data, src_data + (size_t)num_steps * num_sources);
  m_parameters.addInputData(v);
}

void App::addSourceDataDouble(const double* src_data, int num_steps, int num_sources) {
  std::vector<double> v(src_data, src_data + (size_t)num_steps * num_sources);
  m_parameters.addInputDataDouble(v);
}

}  // namespace FDTD
