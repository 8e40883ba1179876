// Host-side API tests that need no GPU, restating the reference's unit tests
// (ParallelFDTD tests/SimulationParametersTest.cpp, tests/MaterialHandlerTest.cpp,
// tests/CudaMeshTest.cpp:182-218) against this library's C++ classes.
#include <cmath>
#include <stdexcept>
#include <vector>

#include "App.h"
#include "MaterialHandler.h"
#include "SimulationParameters.h"
#include "check.h"
#include "cudaMesh.h"
#include "kernels3d.h"

static void parameter_vector() {  // SimulationParametersTest.cpp:80-97
  SimulationParameters sp;
  float* params = sp.getParameterPtr();
  double* params_d = sp.getParameterPtrDouble();
  const double lambda = 1 / std::sqrt(double(3));
  CHECK_EQUAL(params[0], (float)lambda);
  CHECK_EQUAL(params[1], (float)(lambda * lambda));
  CHECK_EQUAL(params[2], 1.f / 3.f);
  CHECK_EQUAL(params[3], (float)sp.getOctave());
  CHECK_EQUAL(params_d[0], lambda);
  CHECK_EQUAL(params_d[1], lambda * lambda);
  CHECK_EQUAL(params_d[2], (double)1 / (double)3);
  CHECK_EQUAL(params_d[3], (double)sp.getOctave());
}

static void sources_receivers() {  // SimulationParametersTest.cpp:40-78 (add/remove)
  SimulationParameters sp;
  sp.addSource(Source(1.f, 1.f, 1.f));
  sp.addSource(Source(2.f, 1.f, 1.f));
  sp.addReceiver(1.f, 1.f, 1.f);
  sp.addReceiver(1.f, 2.f, 1.f);
  CHECK_EQUAL(sp.getNumSources(), 2u);
  CHECK_THROW(sp.removeSource(2), std::out_of_range);
  CHECK_NO_THROW(sp.removeSource(1));
  CHECK_EQUAL(sp.getNumSources(), 1u);
  CHECK_THROW(sp.removeReceiver(2), std::out_of_range);
  CHECK_NO_THROW(sp.removeReceiver(1));
  CHECK_EQUAL(sp.getNumReceivers(), 1u);
}

static void input_data() {  // SimulationParametersTest.cpp:99-124
  SimulationParameters sp;
  sp.setNumSteps(1000);
  std::vector<float> d1(100), d2(200);
  for (unsigned i = 0; i < 200; ++i) {
    if (i < 100) d1[i] = (float)i;
    d2[i] = -1.f * (float)i;
  }
  sp.addInputData(d1.data(), 100);
  sp.addInputData(d2.data(), 200);
  CHECK_EQUAL(sp.getInputDataSample(0, 0), 0);
  CHECK_EQUAL(sp.getInputDataSample(1, 20), -20);
  CHECK_EQUAL(sp.getInputDataSample(0, 99), 99);
  CHECK_EQUAL(sp.getInputDataSample(0, 1000), 0);
  CHECK_THROW(sp.getInputDataSample(2, 1000), std::out_of_range);
}

static void source_samples() {  // SimulationParametersTest.cpp:126-185
  SimulationParameters sp;
  sp.setNumSteps(200);
  sp.addSource(Source(1.f, 1.f, 1.f, SRC_HARD, IMPULSE, 0));
  sp.addSource(Source(1.f, 1.f, 1.f, SRC_HARD, DATA, 0));
  std::vector<float> in;
  for (unsigned i = 0; i < 200; ++i) in.push_back((float)i);
  sp.addInputData(&in[0], (unsigned)(in.size() - 1));
  CHECK_EQUAL(sp.getSourceSample(0, 0), 0.f);
  CHECK_EQUAL(sp.getSourceSample(0, 1), 1.f);
  CHECK_EQUAL(sp.getSourceSample(0, 2), 0.f);
  CHECK_EQUAL(sp.getSourceSample(1, 0), 0.f);
  CHECK_EQUAL(sp.getSourceSample(1, 1), 1.f);
  CHECK_EQUAL(sp.getSourceSample(1, 100), 100.f);
  CHECK_EQUAL(sp.getSourceSample(1, 300), 0.f);
  CHECK_THROW(sp.getSourceSample(2, 1000), std::out_of_range);
  float* s1 = sp.getSourceVectorAt(0);
  float* s2 = sp.getSourceVectorAt(1);
  bool same = true;
  for (unsigned i = 0; i < sp.getNumSteps(); ++i)
    same = same && s1[i] == sp.getSourceSample(0, i) && s2[i] == sp.getSourceSample(1, i);
  CHECK_EQUAL(same, true);
}

static void transparent_source(const char* ir_path) {  // SimulationParametersTest.cpp:187-207
  SimulationParameters sp;
  sp.readGridIr(ir_path);
  CHECK_EQUAL(sp.getGridIrDataSample(0), 0.f);
  CHECK_EQUAL(sp.getGridIrDataSample(2), -0.333333343f);
  sp.addSource(Source(1.f, 1.f, 1.f, SRC_TRANSPARENT, IMPULSE, 0));
  sp.setNumSteps(100);
  CHECK_EQUAL(sp.getSourceSample(0, 0), 0.f);
  CHECK_EQUAL(sp.getSourceSample(0, 1), 1.f);
  CHECK_EQUAL(sp.getSourceSample(0, 3), 1.f / 3.f);
}

static void element_coordinates() {  // SrcRec.cpp:26-34, SimulationParameters.cpp:200-224
  SimulationParameters sp;
  sp.setSpatialFs(10000);
  const float dx = sp.getDx();
  sp.addSource(Source(2.f, 1.f, 3.f * dx, SRC_HARD));
  nv::Vec3i e = sp.getSourceElementCoordinates(0);
  CHECK_EQUAL(e.z, 4);  // round(3) + 1 padding node
  CHECK_EQUAL(e.x, (int)nv::ROUND(2.f / (344.f / (10000.f * (float)sp.getLambda()))) + 1);
  sp.setAddPaddingToElementIdx(false);
  CHECK_EQUAL(sp.getSourceElementCoordinates(0).z, 3);
}

static void materials_unique() {  // MaterialHandlerTest.cpp:70-107
  MaterialHandler mh;
  const unsigned n_surf = 10, n_coef = 20;
  std::vector<float> m(n_surf * n_coef, 0.f);
  for (unsigned s = 0; s < n_surf; ++s)
    for (unsigned c = 0; c < n_coef; ++c) m[s * n_coef + c] = (float)((s % 5) * 10 + c);
  mh.addMaterials(m.data(), n_surf, n_coef);
  CHECK_EQUAL(mh.getNumberOfUniqueMaterials(), 5u);
  CHECK_EQUAL(mh.getUniqueCoefAt(1, 0), 10.f);
  CHECK_EQUAL(mh.getUniqueCoefAt(4, 9), 49.f);
  CHECK_EQUAL(mh.getMaterialIdxAt(7), 2u);
  CHECK_THROW(mh.getUniqueCoefAt(0, 20), std::out_of_range);
}

static void materials_pointer() {  // MaterialHandlerTest.cpp:109-143
  MaterialHandler mh;
  std::vector<float> temp;
  for (unsigned i = 0; i < 10; ++i) temp.push_back(((float)i) / 10.f);
  mh.addSurfaceMaterial(temp);
  temp.at(0) = 0.7f;
  mh.addSurfaceMaterial(temp);
  float* m = mh.getMaterialCoefficientPtr();
  double* md = mh.getMaterialCoefficientPtrDouble();
  CHECK_EQUAL(20u, mh.getNumberOfCoefficients());
  CHECK_EQUAL(2u, mh.getNumberOfUniqueMaterials());
  CHECK_EQUAL(m[0], 0.f);
  CHECK_EQUAL(m[19], 0.f);
  CHECK_EQUAL(m[9], 0.9f);
  CHECK_EQUAL(m[20], 0.7f);
  CHECK_EQUAL(md[0], (double)0.0f);
  CHECK_EQUAL(md[9], (double)0.9f);
  CHECK_EQUAL(md[20], (double)0.7f);
}

static void materials_index() {  // MaterialHandlerTest.cpp:145-159
  MaterialHandler mh;
  mh.setGlobalMaterial(10, 10.f);
  CHECK_EQUAL(mh.getMaterialIdxAt(3), 0u);
  mh.setMaterialIndexAt(3, 3);
  CHECK_EQUAL(mh.getMaterialIdxAt(3), 3u);
  CHECK_NO_THROW(mh.setMaterialIndexAt(12, 3));
}

static void reflectances() {  // global_includes.h:30-33
  MaterialHandler mh;
  mh.coefsAreReflectances();
  mh.setGlobalMaterial(2, 0.5f);
  float* m = mh.getMaterialCoefficientPtr();
  CHECK_EQUAL(m[0], (1.f - 0.5f) / (1.f + 0.5f));
}

static void partition_indexing() {  // CudaMeshTest.cpp:182-218
  CudaMesh mesh;
  const int dim_z = 100, np = 13, ps = dim_z / np;
  std::vector<std::vector<unsigned> > parts = mesh.getPartitionIndexing(np, dim_z);
  std::vector<std::vector<unsigned> > one = mesh.getPartitionIndexing(1, dim_z);
  CHECK_EQUAL((int)parts.size(), np);
  for (int i = 0; i < np; ++i) {
    int end_inc = 0, start_inc = 0;
    if (i == 0) end_inc = 1;
    if (i == np - 1) start_inc = 1;
    if (i != 0 && i != np - 1) { start_inc = 1; end_inc = 1; }
    if (i == np - 1 && np > 1) end_inc = dim_z - (i + 1) * ps;
    CHECK_EQUAL((int)parts[i].size(), dim_z / np + end_inc + start_inc);
    for (size_t j = 0; j < parts[i].size(); ++j)
      CHECK_EQUAL(parts[i][j], (unsigned)(i * ps - start_inc + (int)j));
  }
  CHECK_EQUAL(one.size(), (size_t)1);
  for (size_t j = 0; j < one[0].size(); ++j) CHECK_EQUAL(one[0][j], (unsigned)j);
}

static void split_partitions() {  // cudaMesh.h:309-318
  CudaMesh mesh;
  std::vector<std::vector<unsigned> > parts = mesh.getPartitionIndexing(4, 30);
  std::vector<double*> bufs = mesh.splitPartitions<double>(parts, 12);
  CHECK_EQUAL(bufs.size(), parts.size());
  for (size_t i = 0; i < bufs.size(); ++i) {
    bool zero = bufs[i] != NULL;
    for (size_t k = 0; zero && k < 12 * parts[i].size(); ++k) zero = bufs[i][k] == 0.0;
    CHECK_EQUAL(zero, true);
    free(bufs[i]);
  }
  CHECK_THROW(mesh.getMemorySplitAt(0), std::out_of_range);  // no partitions made yet
}

int main(int argc, char** argv) {
  parameter_vector();
  sources_receivers();
  input_data();
  source_samples();
  if (argc > 1) transparent_source(argv[1]);
  element_coordinates();
  materials_unique();
  materials_pointer();
  materials_index();
  reflectances();
  partition_indexing();
  split_partitions();
  TEST_MAIN_END();
}
