// CudaMesh over one pfdtd_domain (see cudaMesh.h for the partition views).
#include "cudaMesh.h"

#include <cuda_runtime.h>

#include <cstdlib>
#include <cstring>

namespace {

void check(int rc, const char* what) {
  if (rc != PFDTD_OK) {
    c_log_msg(LOG_ERROR, "%s: %s", what, pfdtd_last_error());
    throw(-1);
  }
}

void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    c_log_msg(LOG_ERROR, "%s: %s", what, cudaGetErrorString(e));
    throw(-1);
  }
}

int current_device() {
  int d = 0;
  cudaGetDevice(&d);
  return d;
}

// Pad one byte mesh into a fresh allocation and free the old one, as the
// reference's padWithZeros does (cudaMesh.cu:253-304).
void pad_one(unsigned char** mesh, uint3 dims, unsigned bx, unsigned by, unsigned bz,
             uint3* out_dims) {
  uint32_t in[3] = {dims.x, dims.y, dims.z}, out[3];
  check(pfdtd_pad_mesh(NULL, 0, in, bx, by, bz, NULL, out, current_device()), "padWithZeros");
  unsigned char* fresh = NULL;
  const size_t n = (size_t)out[0] * out[1] * out[2];
  cuda_check(cudaMalloc((void**)&fresh, n + 1 + out[0]), "padWithZeros - allocation");
  cuda_check(cudaMemset(fresh, 0, n + 1 + out[0]), "padWithZeros - clear");
  check(pfdtd_pad_mesh(*mesh, (int64_t)dims.x * dims.y * dims.z, in, bx, by, bz, fresh, out,
                       current_device()),
        "padWithZeros");
  cudaFree(*mesh);
  *mesh = fresh;
  *out_dims = make_uint3(out[0], out[1], out[2]);
}

}  // namespace

void padWithZeros(unsigned char** d_mesh, uint3* dim, unsigned int bx, unsigned int by,
                  unsigned int bz) {
  uint3 out;
  pad_one(d_mesh, *dim, bx, by, bz, &out);
  *dim = out;
}

void padWithZeros(unsigned char** d_position_ptr, unsigned char** d_material_ptr, uint3* dim,
                  unsigned int bx, unsigned int by, unsigned int bz) {
  uint3 out;
  pad_one(d_position_ptr, *dim, bx, by, bz, &out);
  pad_one(d_material_ptr, *dim, bx, by, bz, &out);
  *dim = out;
}

void CudaMesh::setupCommon(unsigned char* d_position_ptr, unsigned char* d_material_ptr,
                           uint3 voxelization_dim, uint3 block_size, bool centred) {
  padWithZeros(&d_position_ptr, &d_material_ptr, &voxelization_dim, block_size.x, block_size.y,
               block_size.z);
  num_elements_ = voxelization_dim.x * voxelization_dim.y * voxelization_dim.z;
  dim_x_ = voxelization_dim.x;
  dim_y_ = voxelization_dim.y;
  dim_z_ = voxelization_dim.z;
  dim_xy_ = voxelization_dim.x * voxelization_dim.y;
  position_idx_ptr_.push_back(d_position_ptr);
  material_idx_ptr_.push_back(d_material_ptr);
  // Scheme translation and air/boundary counts (cudaMesh.cu:155-251).
  const int dev = current_device();
  check(pfdtd_encode_nodes(centred ? 1 : 0, d_position_ptr, d_material_ptr, num_elements_, dev),
        "CudaMesh::setupMesh - scheme translation");
  uint32_t air = 0, boundary = 0;
  check(pfdtd_count_boundaries(d_position_ptr, num_elements_, centred ? 0x80 : 0x86, 0, dev,
                               &air, &boundary),
        "CudaMesh::setupMesh - boundary count");
  num_air_elements_total_ = air;
  num_boundary_elements_total_ = boundary;
  c_log_msg(LOG_INFO, "mesh %u x %u x %u: %u air nodes, %u boundary nodes", dim_x_,
            dim_y_, dim_z_, air, boundary);
}

// element_type 0, 1, 3 -> forward encoding, else centred (cudaMesh.cu:70-73).
void CudaMesh::setupMesh(unsigned char* d_position_ptr, unsigned char* d_material_ptr,
                         unsigned int number_of_unique_materials, float* material_coefficients,
                         float* parameter_ptr, uint3 voxelization_dim, uint3 block_size,
                         unsigned int element_type) {
  block_size_x_ = block_size.x;
  block_size_y_ = block_size.y;
  block_size_z_ = block_size.z;
  h_material_coef_ptr_ = material_coefficients;
  h_parameter_ptr_ = parameter_ptr;
  number_of_unique_materials_ = number_of_unique_materials;
  element_type_ = element_type;
  const bool centred = !(element_type == 0 || element_type == 1 || element_type == 3);
  setupCommon(d_position_ptr, d_material_ptr, voxelization_dim, block_size, centred);
}

// The double set-up pads y to a multiple of block.x and sends element type 3
// to the centred encoding (cudaMesh.cu:106-111, :134-137).
void CudaMesh::setupMeshDouble(unsigned char* d_position_ptr, unsigned char* d_material_ptr,
                               unsigned int number_of_unique_materials,
                               double* material_coefficients, double* parameter_ptr,
                               uint3 voxelization_dim, uint3 block_size,
                               unsigned int element_type) {
  block_size_x_ = block_size.x;
  block_size_y_ = block_size.y;
  block_size_z_ = block_size.z;
  h_material_coef_ptr_double_ = material_coefficients;
  h_parameter_ptr_double_ = parameter_ptr;
  number_of_unique_materials_ = number_of_unique_materials;
  element_type_ = element_type;
  const bool centred = !(element_type == 0 || element_type == 1);
  uint3 b = make_uint3(block_size.x, block_size.x, block_size.z);
  setupCommon(d_position_ptr, d_material_ptr, voxelization_dim, b, centred);
}

std::vector<std::vector<unsigned int> > CudaMesh::getPartitionIndexing(int num_parts, int dim) {
  const int part_size = dim / num_parts;
  std::vector<std::vector<unsigned int> > ret;
  for (int i = 0; i < num_parts; ++i) {
    const int s_inc = (i == 0) ? 0 : 1;
    const int e_inc = (i == num_parts - 1) ? 0 : 1;
    int size = part_size + s_inc + e_inc;
    if (i != 0 && i == num_parts - 1) size += dim - (i + 1) * part_size;
    std::vector<unsigned int> slices(size, 0);
    for (int j = 0; j < size; ++j) slices[j] = (unsigned)(i * part_size - s_inc + j);
    ret.push_back(slices);
  }
  return ret;
}

void CudaMesh::getElementIdxAndDevice(unsigned int x, unsigned int y, unsigned int z, int* dev_i,
                                      int* elem) {
  *dev_i = -1;
  *elem = -1;
  for (int i = 0; i < (int)partition_indexing_.size(); ++i) {
    if (z > partition_indexing_[i].back()) continue;
    if (z < partition_indexing_[i].front()) break;
    *elem = getElementIndex(x, y, z - partition_indexing_[i].front());
    *dev_i = i;
    break;
  }
}

int CudaMesh::getDeviceOfElement(unsigned int x, unsigned int y, unsigned int z) {
  int ret = -1;
  for (int i = 0; i < (int)partition_indexing_.size(); ++i) {
    if (z > partition_indexing_[i].back()) continue;
    if (z < partition_indexing_[i].front()) break;
    ret = (int)device_list_.at(i);
  }
  return ret;
}

void CudaMesh::makePartition(unsigned int number_of_partitions,
                             std::vector<unsigned int> device_list) {
  if (number_of_partitions == 0) number_of_partitions = 1;
  if (device_list.empty())
    for (unsigned i = 0; i < number_of_partitions; ++i) device_list.push_back(i);
  device_list_ = device_list;
  partition_indexing_ = getPartitionIndexing((int)number_of_partitions, (int)dim_z_);
  memory_splits_.clear();
  for (const std::vector<unsigned int>& part : partition_indexing_)
    memory_splits_.push_back(part.empty() ? 0u : part.front());
  number_of_partitions_ = number_of_partitions;
  partition_size_ = (unsigned)partition_indexing_.at(0).size();
  if (domain_) {
    pfdtd_destroy(domain_);
    domain_ = NULL;
  }
  const int dev = (int)device_list_.at(0);
  check(pfdtd_create(dim_x_, dim_y_, dim_z_, isDouble() ? PFDTD_F64 : PFDTD_F32, dev, &domain_),
        "CudaMesh::makePartition");
  unsigned char* pos = position_idx_ptr_.at(0);
  unsigned char* mat = material_idx_ptr_.at(0);
  check(pfdtd_set_nodes(domain_, pos, mat, 1), "CudaMesh::makePartition - node bytes");
  cudaFree(pos);
  cudaFree(mat);
  // Host tables are borrowed, as in the reference (cudaMesh.h:133-139).
  const unsigned n_coef = 20;
  const unsigned n_tab = number_of_unique_materials_ * n_coef;
  std::vector<double> tab(n_tab, 0.0), prm(4, 0.0);
  for (unsigned i = 0; i < n_tab; ++i)
    tab[i] = isDouble() ? h_material_coef_ptr_double_[i] : (double)h_material_coef_ptr_[i];
  for (unsigned i = 0; i < 4; ++i)
    prm[i] = isDouble() ? h_parameter_ptr_double_[i] : (double)h_parameter_ptr_[i];
  if (n_tab > 0)
    check(pfdtd_set_materials(domain_, tab.data(), (int)number_of_unique_materials_, (int)n_coef),
          "CudaMesh::makePartition - materials");
  check(pfdtd_set_params(domain_, prm.data()), "CudaMesh::makePartition - parameters");
  // Device copies behind getMaterialPtrAt / getParameterPtrAt.
  int prev = current_device();
  cudaSetDevice(dev);
  const size_t es = isDouble() ? sizeof(double) : sizeof(float);
  void* d_tab = NULL;
  void* d_prm = NULL;
  cuda_check(cudaMalloc(&d_tab, es * (n_tab > 0 ? n_tab : 1)), "makePartition - material copy");
  cuda_check(cudaMalloc(&d_prm, es * 4), "makePartition - parameter copy");
  if (n_tab > 0)
    cuda_check(cudaMemcpy(d_tab, isDouble() ? (void*)h_material_coef_ptr_double_
                                            : (void*)h_material_coef_ptr_,
                          es * n_tab, cudaMemcpyHostToDevice),
               "makePartition - material copy");
  cuda_check(cudaMemcpy(d_prm, isDouble() ? (void*)h_parameter_ptr_double_ : (void*)h_parameter_ptr_,
                        es * 4, cudaMemcpyHostToDevice),
             "makePartition - parameter copy");
  cudaSetDevice(prev);
  small_allocs_.push_back(d_tab);
  small_allocs_.push_back(d_prm);
  materials_.clear();
  parameters_.clear();
  materials_double_.clear();
  parameters_double_.clear();
  for (unsigned i = 0; i < number_of_partitions; ++i) {
    if (isDouble()) {
      materials_double_.push_back((double*)d_tab);
      parameters_double_.push_back((double*)d_prm);
    } else {
      materials_.push_back((float*)d_tab);
      parameters_.push_back((float*)d_prm);
    }
  }
  refreshViews();
}

// Per-partition pointers into the single domain at each slab's first plane.
void CudaMesh::refreshViews() {
  const size_t np = partition_indexing_.size();
  position_idx_ptr_.assign(np, NULL);
  material_idx_ptr_.assign(np, NULL);
  pressures_.clear();
  pressures_past_.clear();
  pressures_double_.clear();
  pressures_past_double_.clear();
  if (!domain_) return;
  uint8_t *pos = NULL, *mat = NULL;
  pfdtd_get_node_ptrs(domain_, &pos, &mat);
  void *cur = NULL, *past = NULL;
  pfdtd_get_field_ptr(domain_, PFDTD_FIELD_CURRENT, &cur);
  pfdtd_get_field_ptr(domain_, PFDTD_FIELD_PAST, &past);
  for (size_t p = 0; p < np; ++p) {
    const size_t off = (size_t)partition_indexing_[p].front() * dim_xy_;
    position_idx_ptr_[p] = pos + off;
    material_idx_ptr_[p] = mat + off;
    if (isDouble()) {
      pressures_double_.push_back((double*)cur + off);
      pressures_past_double_.push_back((double*)past + off);
    } else {
      pressures_.push_back((float*)cur + off);
      pressures_past_.push_back((float*)past + off);
    }
  }
}

void CudaMesh::destroyPartitions() {
  if (domain_) pfdtd_destroy(domain_);
  domain_ = NULL;
  for (void* p : small_allocs_) cudaFree(p);
  small_allocs_.clear();
  for (unsigned char* p : position_idx_ptr_) (void)p;
  position_idx_ptr_.clear();
  material_idx_ptr_.clear();
  memory_splits_.clear();
  pressures_.clear();
  pressures_past_.clear();
  pressures_double_.clear();
  pressures_past_double_.clear();
  materials_.clear();
  parameters_.clear();
  materials_double_.clear();
  parameters_double_.clear();
}

void CudaMesh::flipPressurePointers() {
  if (!domain_) return;
  pfdtd_flip(domain_);
  refreshViews();
}

void CudaMesh::resetPressures() {
  if (!domain_) return;
  check(pfdtd_reset_fields(domain_), "CudaMesh::resetPressures");
}

// setSample / addSample write the node once; the reference writes every
// partition holding the slice, which in one domain is the same node
// (cudaMesh.h:322-369).  addSample adds unless the soft-source quirk is on.
void CudaMesh::setSampleValue(double v, unsigned int x, unsigned int y, unsigned int z, bool add) {
  int dev = -1, elem = -1;
  getElementIdxAndDevice(x, y, z, &dev, &elem);
  if (dev < 0 || !domain_) return;
  if (add)
    check(pfdtd_add_sample(domain_, x, y, z, v), "CudaMesh::addSample");
  else
    check(pfdtd_set_sample(domain_, x, y, z, v), "CudaMesh::setSample");
}

void CudaMesh::setSampleAtValue(double v, unsigned int x, unsigned int y, unsigned int z,
                                unsigned int p) {
  const unsigned zg = partition_indexing_.at(p).front() + z;
  check(pfdtd_set_sample(domain_, x, y, zg, v), "CudaMesh::setSampleAt");
}

double CudaMesh::getSampleValue(unsigned int x, unsigned int y, unsigned int z) {
  int dev = -1, elem = -1;
  getElementIdxAndDevice(x, y, z, &dev, &elem);
  if (dev < 0 || !domain_) return 0.0;
  double v = 0.0;
  check(pfdtd_get_sample(domain_, x, y, z, &v), "CudaMesh::getSample");
  return v;
}

double CudaMesh::getSampleAtValue(unsigned int x, unsigned int y, unsigned int z, unsigned int p) {
  if (z > partition_indexing_.at(p).size()) {
    c_log_msg(LOG_WARNING, "slice %u is outside the partition (%u slices); sample read as 0", z,
              (unsigned)partition_indexing_.at(p).size());
    return 0.0;
  }
  const unsigned zg = partition_indexing_.at(p).front() + z;
  double v = 0.0;
  check(pfdtd_get_sample(domain_, x, y, zg, &v), "CudaMesh::getSampleAt");
  return v;
}

void* CudaMesh::elementPtrAt(unsigned int x, unsigned int y, unsigned int z, unsigned int p) {
  const size_t es = isDouble() ? 8 : 4;
  void* cur = NULL;
  pfdtd_get_field_ptr(domain_, PFDTD_FIELD_CURRENT, &cur);
  const size_t off = (size_t)partition_indexing_.at(p).front() * dim_xy_ + (size_t)getElementIndex(x, y, z);
  return (char*)cur + off * es;
}

void* CudaMesh::elementPtr(unsigned int x, unsigned int y, unsigned int z, unsigned int* halo) {
  int dev = -1, elem = -1;
  getElementIdxAndDevice(x, y, z, &dev, &elem);
  if (dev < 0) return NULL;
  if (halo) *halo = (unsigned)dev;
  return elementPtrAt(x, y, z - partition_indexing_.at(dev).front(), (unsigned)dev);
}

unsigned char CudaMesh::getPositionSample(unsigned int x, unsigned int y, unsigned int z) {
  int dev = -1, elem = -1;
  getElementIdxAndDevice(x, y, z, &dev, &elem);
  if (dev < 0 || !domain_) return 0;
  uint8_t* pos = NULL;
  pfdtd_get_node_ptrs(domain_, &pos, NULL);
  unsigned char v = 0;
  cuda_check(cudaMemcpy(&v, pos + (size_t)z * dim_xy_ + (size_t)y * dim_x_ + x, 1,
                        cudaMemcpyDeviceToHost),
             "CudaMesh::getPositionSample");
  return v;
}

void* CudaMesh::sliceCopy(unsigned int slice, unsigned int orientation, size_t esize) {
  if (orientation != 0 || !domain_ || slice >= dim_z_) return NULL;
  void* cur = NULL;
  pfdtd_get_field_ptr(domain_, PFDTD_FIELD_CURRENT, &cur);
  const size_t fs = isDouble() ? 8 : 4;
  void* out = std::calloc(dim_xy_, esize);
  const size_t n = (size_t)dim_xy_ * (esize < fs ? esize : fs);
  cuda_check(cudaMemcpy(out, (char*)cur + (size_t)slice * dim_xy_ * fs, n, cudaMemcpyDeviceToHost),
             "CudaMesh::getSlice");
  return out;
}

unsigned char* CudaMesh::getPositionSlice(unsigned int slice, unsigned int orientation) {
  if (orientation != 0 || !domain_ || slice >= dim_z_) return NULL;
  uint8_t* pos = NULL;
  pfdtd_get_node_ptrs(domain_, &pos, NULL);
  unsigned char* out = (unsigned char*)std::malloc(dim_xy_);
  cuda_check(cudaMemcpy(out, pos + (size_t)slice * dim_xy_, dim_xy_, cudaMemcpyDeviceToHost),
             "CudaMesh::getPositionSlice");
  return out;
}
