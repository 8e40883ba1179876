// Material de-duplication and coefficient tables with the behaviour of
// ParallelFDTD src/base/MaterialHandler.cpp.
#include "MaterialHandler.h"

#include <stdexcept>

#include "global_includes.h"

void MaterialHandler::addMaterials(float* material_ptr, unsigned int number_of_surfaces,
                                   unsigned int number_of_coefficients) {
  std::vector<float> temp(MATERIAL_COEF_NUM, 0.f);
  for (unsigned int i = 0; i < number_of_surfaces; ++i) {
    for (unsigned int j = 0; j < number_of_coefficients; ++j)
      temp.at(j) = material_ptr[i * number_of_coefficients + j];
    addSurfaceMaterial(temp);
  }
}

// Pads to MATERIAL_COEF_NUM coefficients, reuses an identical unique
// material or appends a new one (MaterialHandler.cpp:47-65, :186-204).
unsigned int MaterialHandler::addSurfaceMaterial(std::vector<float> coefs) {
  if (number_of_coefficients_ != coefs.size())
    c_log_msg(LOG_ERROR, "material rows carry %u coefficients; this handler expects %u",
              (unsigned)coefs.size(), (unsigned)MATERIAL_COEF_NUM);
  while (coefs.size() <= MATERIAL_COEF_NUM) coefs.push_back(0.f);
  const unsigned int idx = checkIfUnique(coefs);
  material_indices_.push_back((unsigned char)idx);
  ++number_of_surfaces_;
  return idx;
}

float MaterialHandler::getUniqueCoefAt(unsigned int material, unsigned int coef_idx) {
  if (coef_idx >= (unsigned)MATERIAL_COEF_NUM) {
    c_log_msg(LOG_ERROR, "coefficient index %u is past the 20 per material", coef_idx);
    throw std::out_of_range("Coef idx out of range");
  }
  return unique_coefficients_.at(material).coefs[coef_idx];
}

float MaterialHandler::getSurfaceCoefAt(unsigned int surface, unsigned int coef_idx) {
  if (coef_idx >= (unsigned)MATERIAL_COEF_NUM) {
    c_log_msg(LOG_ERROR, "coefficient index %u is past the 20 per surface", coef_idx);
    throw std::out_of_range("Coef idx out of range");
  }
  return getUniqueCoefAt(material_indices_.at(surface), coef_idx);
}

unsigned char* MaterialHandler::getMaterialIdxPtr() {
  if (material_indices_.empty()) return (unsigned char*)NULL;
  return &material_indices_[0];
}

// [unique materials x coefficients], reflections converted to admittances
// in single precision (MaterialHandler.cpp:100-130).
float* MaterialHandler::getMaterialCoefficientPtr() {
  coefficient_vector_.clear();
  const unsigned coefs = getNumberOfCoefficients(), n = getNumberOfUniqueMaterials();
  coefficient_vector_.assign(coefs * n, 0.f);
  for (unsigned i = 0; i < n; ++i)
    for (unsigned j = 0; j < coefs; ++j) {
      float c = getUniqueCoefAt(i, j);
      if (!admitance_) c = reflection2Admitance(c);
      coefficient_vector_.at(i * coefs + j) = c;
    }
  if (coefficient_vector_.empty()) return NULL;
  return &coefficient_vector_[0];
}

// Double table; conversions still happen in single precision, as the
// reference's reflection2Admitance takes a float (MaterialHandler.cpp:132-164).
double* MaterialHandler::getMaterialCoefficientPtrDouble() {
  const unsigned coefs = getNumberOfCoefficients(), n = getNumberOfUniqueMaterials();
  coefficient_vector_double_.assign(coefs * n, 0.0);
  for (unsigned i = 0; i < n; ++i)
    for (unsigned j = 0; j < coefs; ++j) {
      double c = (double)getUniqueCoefAt(i, j);
      if (!admitance_) c = (double)reflection2Admitance((float)c);
      coefficient_vector_double_.at(i * coefs + j) = c;
    }
  if (coefficient_vector_double_.empty()) return NULL;
  return &coefficient_vector_double_[0];
}

float MaterialHandler::getMeanAbsorption(unsigned int octave) {
  float mean = 0.f;
  for (unsigned i = 0; i < number_of_surfaces_; ++i) {
    float c = admitance2Reflection(getSurfaceCoefAt(i, octave));
    mean += 1 - c * c;
  }
  return mean / number_of_surfaces_;
}

unsigned int MaterialHandler::checkIfUnique(std::vector<float> coefs) {
  unsigned int idx = 0;
  for (const material_t& m : unique_coefficients_) {
    bool same = true;
    for (unsigned i = 0; i < MATERIAL_COEF_NUM; ++i)
      if (coefs.at(i) != m.coefs[i]) same = false;
    if (same) return idx;
    ++idx;
  }
  material_t n;
  for (unsigned i = 0; i < MATERIAL_COEF_NUM; ++i) n.coefs[i] = coefs.at(i);
  ++number_of_unique_materials_;
  unique_coefficients_.push_back(n);
  return idx;
}

void MaterialHandler::setGlobalMaterial(unsigned int number_of_surfaces, float coef) {
  std::vector<float> mat(MATERIAL_COEF_NUM, coef);
  for (unsigned i = 0; i < number_of_surfaces; ++i) addSurfaceMaterial(mat);
}

void MaterialHandler::setMaterialIndexAt(unsigned int surface_idx, unsigned char material_idx) {
  if (surface_idx >= number_of_surfaces_) {
    c_log_msg(LOG_INFO, "no surface %u (there are %u); material index left unchanged",
              surface_idx, number_of_surfaces_);
    return;
  }
  material_indices_.at(surface_idx) = material_idx;
}
