// CudaMesh: the simulation domain on the device, with the reference's public
// interface (ParallelFDTD src/kernels/cudaMesh.h:62-840).
//
// The reference splits the grid into z-slabs on several GPUs and exchanges a
// halo plane between them every step.  Here one whole domain lives on one
// GPU (a pfdtd_domain from pfdtd.h); makePartition still computes the
// reference's slab indexing, and every per-partition pointer or index is a
// view into the single domain at that slab's first plane, so per-partition
// addressing keeps working while halos are always consistent and
// switchHalos has nothing to do.
#ifndef PFDTD_CUDAMESH_H
#define PFDTD_CUDAMESH_H

#include <vector_functions.h>
#include <vector_types.h>

#include <cstdlib>
#include <vector>

#include "logger.h"
#include "pfdtd.h"

#define INSIDE_SWITCH 7
#define FORWARD_POSITION_MASK 0X7F
#define CENTERED_MASK 0x80
#define DIR_X 0x01
#define DIR_Y 0x02
#define DIR_Z 0x04
#define SIGN_X 0x10
#define SIGN_Y 0x20
#define SIGN_Z 0x40

class CudaMesh {
 public:
  CudaMesh()
      : double_(false), dif_order_(0), number_of_partitions_(0), partition_size_(0),
        h_material_coef_ptr_(NULL), h_material_coef_ptr_double_(NULL),
        number_of_unique_materials_(0), h_parameter_ptr_(NULL), h_parameter_ptr_double_(NULL),
        num_elements_(0), num_air_elements_total_(0), num_boundary_elements_total_(0),
        dim_x_(0), dim_y_(0), dim_z_(0), dim_xy_(0), dx_(0), block_size_x_(0),
        block_size_y_(0), block_size_z_(0), element_type_(0), domain_(NULL) {}
  ~CudaMesh() {}

  bool double_;
  unsigned int dif_order_;
  std::vector<unsigned char*> position_idx_ptr_;
  std::vector<unsigned char*> material_idx_ptr_;
  std::vector<float*> pressures_;
  std::vector<float*> pressures_past_;
  std::vector<float*> parameters_;
  std::vector<float*> materials_;
  std::vector<double*> pressures_double_;
  std::vector<double*> pressures_past_double_;
  std::vector<double*> parameters_double_;
  std::vector<double*> materials_double_;
  std::vector<unsigned int> device_list_;
  std::vector<std::vector<unsigned int> > partition_indexing_;
  std::vector<unsigned int> memory_splits_;
  unsigned int number_of_partitions_;
  unsigned int partition_size_;
  float* h_material_coef_ptr_;
  double* h_material_coef_ptr_double_;
  unsigned int number_of_unique_materials_;
  float* h_parameter_ptr_;
  double* h_parameter_ptr_double_;
  unsigned int num_elements_;
  unsigned int num_air_elements_total_;
  unsigned int num_boundary_elements_total_;
  unsigned int dim_x_, dim_y_, dim_z_, dim_xy_;
  float dx_;
  unsigned int block_size_x_, block_size_y_, block_size_z_;
  unsigned int element_type_;

  void destroyPartitions();

  float* getPressurePtrAt(unsigned int p) { return pressures_.at(p); }
  float* getPastPressurePtrAt(unsigned int p) { return pressures_past_.at(p); }
  float* getMaterialPtrAt(unsigned int p) { return materials_.at(p); }
  float* getParameterPtrAt(unsigned int p) { return parameters_.at(p); }
  double* getMaterialPtrDoubleAt(unsigned int p) { return materials_double_.at(p); }
  double* getParameterPtrDoubleAt(unsigned int p) { return parameters_double_.at(p); }
  double* getPressureDoublePtrAt(unsigned int p) { return pressures_double_.at(p); }
  double* getPastPressureDoublePtrAt(unsigned int p) { return pressures_past_double_.at(p); }
  unsigned char* getPositionIdxPtrAt(unsigned int p) { return position_idx_ptr_.at(p); }
  unsigned char* getMaterialIdxPtrAt(unsigned int p) { return material_idx_ptr_.at(p); }
  // cudaMesh.h:214-215.  The reference declares this getter but never fills
  // the list behind it (its call throws std::out_of_range); here the list
  // holds each partition's first global z-slice, where the mesh memory is
  // split, and is filled by makePartition.  Out-of-range partitions throw
  // std::out_of_range as before.
  unsigned int getMemorySplitAt(unsigned int p) { return memory_splits_.at(p); }
  unsigned int getNumberOfElementsAt(unsigned int p) {
    return (unsigned int)partition_indexing_.at(p).size() * getDimXY();
  }
  unsigned int getNumberOfPartitions() { return (unsigned int)partition_indexing_.size(); }
  unsigned int getPartitionSize() { return (unsigned int)partition_indexing_.at(0).size(); }
  unsigned int getPartitionSize(int partition) {
    unsigned int np = getNumberOfPartitions();
    return partition < (int)np ? (unsigned int)partition_indexing_.at(partition).size() : 0u;
  }
  unsigned int getFirstSliceIdx(int partition) { return partition_indexing_.at(partition).at(0); }
  unsigned int getDeviceAt(int i) { return device_list_.at(i); }
  unsigned int getBlockX() { return block_size_x_; }
  unsigned int getBlockY() { return block_size_y_; }
  unsigned int getBlockZ() { return block_size_z_; }
  unsigned int getDimX() { return dim_x_; }
  unsigned int getDimY() { return dim_y_; }
  unsigned int getDimZ() { return dim_z_; }
  unsigned int getDimXY() { return dim_xy_; }
  unsigned int getGridDimX() { return dim_x_ / block_size_x_; }
  unsigned int getGridDimY() { return dim_y_ / block_size_y_; }
  unsigned int getGridDimZ() { return dim_z_ / block_size_z_; }
  unsigned int getNumberOfElements() { return num_elements_; }
  unsigned int getNumberOfAirElements() { return num_air_elements_total_; }
  unsigned int getNumberOfBoundaryElements() { return num_boundary_elements_total_; }
  bool isDouble() const { return double_; }
  void setDouble(bool is_double) { double_ = is_double; }

  inline int getElementIndex(int x, int y, int z) {
    return (int)(getDimXY() * z + getDimX() * y + x);
  }
  // Partition holding global slice z and the partition-local element index
  // (cudaMesh.h:251-266); -1/-1 when z lies outside every partition.
  void getElementIdxAndDevice(unsigned int x, unsigned int y, unsigned int z, int* dev_i, int* elem);
  int getDeviceOfElement(unsigned int x, unsigned int y, unsigned int z);
  // z-slab indexing with one overlapping slice (cudaMesh.h:280-307).
  std::vector<std::vector<unsigned int> > getPartitionIndexing(int num_parts, int dim);

  // Host buffers for per-partition data (cudaMesh.h:309-318): one zeroed
  // block of slice_dim * (slices in the partition) elements of T per
  // partition, from calloc; the caller frees each with free().
  template <typename T>
  std::vector<T*> splitPartitions(std::vector<std::vector<unsigned int> >& slices, int slice_dim) {
    std::vector<T*> out;
    out.reserve(slices.size());
    for (const std::vector<unsigned int>& part : slices)
      out.push_back(static_cast<T*>(std::calloc((size_t)slice_dim * part.size(), sizeof(T))));
    return out;
  }

  template <typename T>
  void setSample(T sample, unsigned int x, unsigned int y, unsigned int z) {
    setSampleValue((double)sample, x, y, z, false);
  }
  template <typename T>
  void addSample(T sample, unsigned int x, unsigned int y, unsigned int z) {
    setSampleValue((double)sample, x, y, z, true);
  }
  template <typename T>
  void setSampleAt(T sample, unsigned int x, unsigned int y, unsigned int z, unsigned int partition) {
    setSampleAtValue((double)sample, x, y, z, partition);
  }
  template <typename T>
  T getSample(unsigned int x, unsigned int y, unsigned int z) {
    return (T)getSampleValue(x, y, z);
  }
  template <typename T>
  T getSampleAt(unsigned int x, unsigned int y, unsigned int z, unsigned int partition) {
    return (T)getSampleAtValue(x, y, z, partition);
  }
  template <typename T>
  T* getElementAt(unsigned int x, unsigned int y, unsigned int z, unsigned int partition) {
    return (T*)elementPtrAt(x, y, z, partition);
  }
  template <typename T>
  T* getElement(unsigned int x, unsigned int y, unsigned int z, unsigned int* halo) {
    return (T*)elementPtr(x, y, z, halo);
  }
  unsigned char getPositionSample(unsigned int x, unsigned int y, unsigned int z);

  // xy slice of the current pressure / node bytes, host memory from malloc
  // (caller frees), as cudaMesh.h:600-646; orientation 0 only, as there.
  template <typename T>
  T* getSlice(unsigned int slice, unsigned int orientation) {
    return (T*)sliceCopy(slice, orientation, sizeof(T));
  }
  unsigned char* getPositionSlice(unsigned int slice, unsigned int orientation);

  void makePartition(unsigned int number_of_partitions,
                     std::vector<unsigned int> device_list = std::vector<unsigned int>());
  void switchHalos() {}
  void flipPressurePointers();
  void resetPressures();

  void setupMesh(unsigned char* d_position_ptr, unsigned char* d_material_ptr,
                 unsigned int number_of_unique_materials, float* material_coefficients,
                 float* parameter_ptr, uint3 voxelization_dim, uint3 block_size,
                 unsigned int element_type);
  void setupMeshDouble(unsigned char* d_position_ptr, unsigned char* d_material_ptr,
                       unsigned int number_of_unique_materials, double* material_coefficients,
                       double* parameter_ptr, uint3 voxelization_dim, uint3 block_size,
                       unsigned int element_type);

  // The single GPU domain behind the partitions (NULL before makePartition).
  pfdtd_domain* getDomain() { return domain_; }
  // Re-point the per-partition views after the domain swapped its fields.
  void syncViews() { refreshViews(); }

 private:
  void setupCommon(unsigned char* d_position_ptr, unsigned char* d_material_ptr,
                   uint3 voxelization_dim, uint3 block_size, bool centred);
  void refreshViews();
  void setSampleValue(double v, unsigned int x, unsigned int y, unsigned int z, bool add);
  void setSampleAtValue(double v, unsigned int x, unsigned int y, unsigned int z, unsigned int p);
  double getSampleValue(unsigned int x, unsigned int y, unsigned int z);
  double getSampleAtValue(unsigned int x, unsigned int y, unsigned int z, unsigned int p);
  void* elementPtrAt(unsigned int x, unsigned int y, unsigned int z, unsigned int p);
  void* elementPtr(unsigned int x, unsigned int y, unsigned int z, unsigned int* halo);
  void* sliceCopy(unsigned int slice, unsigned int orientation, size_t esize);

  pfdtd_domain* domain_;
  std::vector<void*> small_allocs_;
};

// Pad a device byte mesh to multiples of the block size, replacing *d_mesh
// (cudaMesh.cu:253-326).
void padWithZeros(unsigned char** d_mesh, uint3* dim, unsigned int block_size_x,
                  unsigned int block_size_y, unsigned int block_size_z);
void padWithZeros(unsigned char** d_position_ptr, unsigned char** d_material_ptr, uint3* dim,
                  unsigned int block_size_x, unsigned int block_size_y, unsigned int block_size_z);

#endif
