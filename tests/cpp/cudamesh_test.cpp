// GPU tests of the C++ API with the reference's names, restating
// ParallelFDTD tests/CudaMeshTest.cpp: element indexing, per-partition
// get/set and halo semantics, and bit-identical receiver traces for 1, 2 and
// 5 partitions in float and double (:472-575).  The reference reads its
// geometry from Data/hytti.vtk (not in the repository); a procedural
// 128 x 96 x 49 room of the same size stands in for it.
#include <cuda_runtime.h>

#include <cstring>
#include <stdexcept>
#include <vector>

#include "App.h"
#include "check.h"
#include "cudaMesh.h"
#include "kernels3d.h"

static const unsigned char kBidLut[64] = {
    27, 24, 25, 0, 22, 20, 19, 0, 23, 18, 17, 0, 0, 0, 0, 0, 26, 16, 15, 0, 14, 8,
    7,  0,  13, 6, 5,  0,  0,  0, 0,  0, 21, 12, 11, 0, 10, 4, 3, 0, 9, 2, 1, 0, 0,
    0,  0,  0,  0, 0,  0,  0,  0, 0,  0,  0,  0,  0,  0,  0, 0, 0, 0, 0};

// Shoebox with a solid shell and one solid pillar; ids as the voxelizer.
static void room(unsigned X, unsigned Y, unsigned Z, std::vector<unsigned char>& bid,
                 std::vector<unsigned char>& mat) {
  std::vector<char> solid((size_t)X * Y * Z, 0);
  for (unsigned z = 0; z < Z; ++z)
    for (unsigned y = 0; y < Y; ++y)
      for (unsigned x = 0; x < X; ++x) {
        bool s = x == 0 || y == 0 || z == 0 || x == X - 1 || y == Y - 1 || z == Z - 1;
        s = s || (x >= 40 && x < 52 && y >= 30 && y < 44 && z >= 1 && z < 30);
        solid[(size_t)z * X * Y + y * X + x] = s;
      }
  bid.assign(solid.size(), 0);
  mat.assign(solid.size(), 0);
  for (unsigned z = 1; z + 1 < Z; ++z)
    for (unsigned y = 1; y + 1 < Y; ++y)
      for (unsigned x = 1; x + 1 < X; ++x) {
        const size_t i = (size_t)z * X * Y + y * X + x;
        if (solid[i]) continue;
        unsigned m = 0;
        m |= solid[i - 1] ? 1 : 0;
        m |= solid[i + 1] ? 2 : 0;
        m |= solid[i - X] ? 4 : 0;
        m |= solid[i + X] ? 8 : 0;
        m |= solid[i - (size_t)X * Y] ? 16 : 0;
        m |= solid[i + (size_t)X * Y] ? 32 : 0;
        bid[i] = kBidLut[m];
        mat[i] = (unsigned char)(m ? (x < 40 ? 0 : 1) : 0);
      }
}

static SimulationParameters g_params;
static MaterialHandler g_materials;

static bool no_interrupt() { return false; }
static void quiet_progress(int, int, float) {}

static unsigned char* to_device(const std::vector<unsigned char>& v) {
  unsigned char* d = NULL;
  cudaMalloc((void**)&d, v.size() + 256);
  cudaMemset(d, 0, v.size() + 256);
  cudaMemcpy(d, v.data(), v.size(), cudaMemcpyHostToDevice);
  return d;
}

static CudaMesh* test_mesh(unsigned partitions, bool dbl) {
  std::vector<unsigned char> bid, mat;
  room(128, 96, 49, bid, mat);
  g_params = SimulationParameters();
  g_materials = MaterialHandler();
  std::vector<float> m0(20, 0.2f), m1(20, 0.05f);
  g_materials.addSurfaceMaterial(m0);
  g_materials.addSurfaceMaterial(m1);
  g_params.setSpatialFs(10000);
  g_params.setNumSteps(400);
  const float dx = g_params.getDx();
  // three sources and receivers: bottom, halo and top slabs (CudaMeshTest.cpp:66-77)
  g_params.addSource(Source(20 * dx, 20 * dx, 3.f * dx, SRC_HARD));
  g_params.addSource(Source(60 * dx, 20 * dx, 23.f * dx, SRC_SOFT, GAUSSIAN, 0));
  g_params.addSource(Source(90 * dx, 70 * dx, 40.f * dx, SRC_HARD));
  g_params.addReceiver(Receiver(30 * dx, 20 * dx, 5.f * dx));
  g_params.addReceiver(Receiver(70 * dx, 60 * dx, 24.f * dx));
  g_params.addReceiver(Receiver(100 * dx, 80 * dx, 42.f * dx));
  g_params.setUpdateType(SRL_FORWARD);
  CudaMesh* mesh = new CudaMesh();
  mesh->setDouble(dbl);
  uint3 dim = make_uint3(128, 96, 49);
  uint3 block = make_uint3(32, 4, 1);
  if (dbl)
    mesh->setupMeshDouble(to_device(bid), to_device(mat), g_materials.getNumberOfUniqueMaterials(),
                          g_materials.getMaterialCoefficientPtrDouble(),
                          g_params.getParameterPtrDouble(), dim, block,
                          (unsigned)g_params.getUpdateType());
  else
    mesh->setupMesh(to_device(bid), to_device(mat), g_materials.getNumberOfUniqueMaterials(),
                    g_materials.getMaterialCoefficientPtr(), g_params.getParameterPtr(), dim,
                    block, (unsigned)g_params.getUpdateType());
  std::vector<unsigned int> devices(partitions, 0);
  mesh->makePartition(partitions, devices);
  return mesh;
}

static void set_get_utils() {  // CudaMeshTest.cpp:220-258
  CudaMesh mesh;
  std::vector<float> coefs(20, 0.f), params(10, 0.f);
  unsigned char *p = NULL, *m = NULL;
  cudaMalloc((void**)&p, 8000);
  cudaMalloc((void**)&m, 8000);
  cudaMemset(p, 0, 8000);
  cudaMemset(m, 0, 8000);
  mesh.setupMesh(p, m, 1, &coefs[0], &params[0], make_uint3(20, 20, 20), make_uint3(32, 4, 2), 0);
  mesh.makePartition(1, std::vector<unsigned int>(1, 0));
  CHECK_EQUAL(mesh.pressures_.size(), (size_t)1);
  int dev = 0, elem = 0;
  mesh.getElementIdxAndDevice(10, 10, 10, &dev, &elem);
  CHECK_EQUAL(dev, 0);
  CHECK_EQUAL(elem, 10 * 20 * 32 + 10 * 32 + 10);
  mesh.getElementIdxAndDevice(40, 10, 50, &dev, &elem);
  CHECK_EQUAL(elem, -1);
  CHECK_EQUAL(dev, -1);
  mesh.destroyPartitions();
}

static void get_set_multi() {  // CudaMeshTest.cpp:260-303
  CudaMesh mesh;
  const int dim = 50;
  std::vector<float> coefs(20, 0.f), params(10, 0.f);
  unsigned char *p = NULL, *m = NULL;
  cudaMalloc((void**)&p, dim * dim * dim);
  cudaMalloc((void**)&m, dim * dim * dim);
  cudaMemset(p, 0, dim * dim * dim);
  cudaMemset(m, 0, dim * dim * dim);
  mesh.setupMesh(p, m, 1, &coefs[0], &params[0], make_uint3(dim, dim, dim), make_uint3(1, 1, 1), 0);
  CHECK_EQUAL(mesh.getDimX(), (unsigned)dim);
  CHECK_EQUAL(mesh.getDimZ(), (unsigned)dim);
  std::vector<unsigned int> devices(5, 0);
  mesh.makePartition(5, devices);
  CHECK_EQUAL(mesh.pressures_.size(), (size_t)5);
  // each partition's first global slice (partitions overlap by one slice)
  for (unsigned i = 0; i < 5; ++i)
    CHECK_EQUAL(mesh.getMemorySplitAt(i), mesh.getFirstSliceIdx((int)i));
  CHECK_EQUAL(mesh.getMemorySplitAt(1), 9u);
  CHECK_THROW(mesh.getMemorySplitAt(5), std::out_of_range);
  int dev = 0, elem = 0;
  mesh.getElementIdxAndDevice(10, 10, 11, &dev, &elem);
  CHECK_EQUAL(dev, 1);
  CHECK_EQUAL(elem, 2 * dim * dim + 10 * dim + 10);
  mesh.destroyPartitions();
}

static void one_partition() {  // CudaMeshTest.cpp:306-323
  CudaMesh* mesh = test_mesh(1, false);
  mesh->setSample(3.0, 0, 0, 0);
  CHECK_EQUAL(mesh->getSample<float>(0, 0, 0), 3.f);
  mesh->addSample(3.f, 0, 0, 0);
  CHECK_EQUAL(mesh->getSample<float>(0, 0, 0), 6.f);
  mesh->setSample(1.f, 27, 27, 27);
  CHECK_EQUAL(mesh->getSample<float>(27, 27, 27), 1.f);
  mesh->destroyPartitions();
  delete mesh;
}

template <typename T>
static void two_partitions(bool dbl) {  // CudaMeshTest.cpp:326-469
  CudaMesh* mesh = test_mesh(2, dbl);
  CHECK_EQUAL(mesh->getNumberOfPartitions(), 2u);
  mesh->setSample<T>(3, 0, 0, 0);
  CHECK_EQUAL(mesh->getSample<T>(0, 0, 0), (T)3);
  mesh->addSample<T>(3, 0, 0, 0);
  CHECK_EQUAL(mesh->getSample<T>(0, 0, 0), (T)6);
  mesh->setSample<T>(1, 2, 0, 23);
  mesh->setSample<T>(89, 6, 0, 24);
  CHECK_EQUAL(mesh->getSampleAt<T>(2, 0, 23, 0), (T)1);
  CHECK_EQUAL(mesh->getSampleAt<T>(6, 0, 24, 0), (T)89);
  CHECK_EQUAL(mesh->getSampleAt<T>(2, 0, 0, 1), (T)1);
  CHECK_EQUAL(mesh->getSampleAt<T>(6, 0, 1, 1), (T)89);
  mesh->setSampleAt<T>(8, 2, 0, 1, 1);
  mesh->setSampleAt<T>(45, 3, 0, 23, 0);
  mesh->switchHalos();
  CHECK_EQUAL(mesh->getSampleAt<T>(2, 0, 24, 0), (T)8);
  CHECK_EQUAL(mesh->getSampleAt<T>(3, 0, 0, 1), (T)45);
  mesh->destroyPartitions();
  delete mesh;
}

template <typename T>
static void run_partitions(bool dbl) {  // CudaMeshTest.cpp:472-575
  std::vector<std::vector<T> > rets;
  for (unsigned np : {1u, 2u, 5u}) {
    CudaMesh* mesh = test_mesh(np, dbl);
    std::vector<T> ret((size_t)g_params.getNumSteps() * g_params.getNumReceivers(), (T)0);
    if (dbl)
      launchFDTD3dDouble(mesh, &g_params, (double*)ret.data(), no_interrupt, quiet_progress);
    else
      launchFDTD3d(mesh, &g_params, (float*)ret.data(), no_interrupt, quiet_progress);
    mesh->destroyPartitions();
    delete mesh;
    rets.push_back(ret);
  }
  bool same = true, nonzero = false;
  for (size_t i = 0; i < rets[0].size(); ++i) {
    same = same && rets[0][i] == rets[1][i] && rets[0][i] == rets[2][i];
    nonzero = nonzero || rets[0][i] != 0;
  }
  CHECK_EQUAL(same, true);
  CHECK_EQUAL(nonzero, true);
}

static void app_voxel_run() {
  std::vector<unsigned char> bid, mat;
  room(64, 48, 40, bid, mat);
  FDTD::App app;
  app.initializeDevices();
  app.initializeVoxels(bid.data(), mat.data(), make_uint3(64, 48, 40));
  std::vector<float> m0(20, 0.2f), m1(20, 0.05f);
  app.addMaterialToMaterialList(m0);
  app.addMaterialToMaterialList(m1);
  app.setSpatialFs(10000);
  app.setNumSteps(200);
  const float dx = app.m_parameters.getDx();
  app.addSource(20 * dx, 20 * dx, 20 * dx, SRC_SOFT, GAUSSIAN, 0);
  app.addReceiver(10 * dx, 12 * dx, 14 * dx);
  app.m_interrupt = no_interrupt;
  app.m_progress = quiet_progress;
  app.runSimulation();
  std::vector<float> r = app.getResponse(0);
  float peak = 0;
  for (float v : r) peak = v > peak ? v : (-v > peak ? -v : peak);
  CHECK_EQUAL(r.size(), (size_t)200);
  CHECK_EQUAL(peak > 1e-4f, true);
  CHECK_EQUAL(app.getNumElements(), 64u * 48u * 40u);
  app.close();
}

int main() {
  set_get_utils();
  get_set_multi();
  one_partition();
  two_partitions<float>(false);
  two_partitions<double>(true);
  run_partitions<float>(false);
  run_partitions<double>(true);
  app_voxel_run();
  TEST_MAIN_END();
}
