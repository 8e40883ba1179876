// Minimal vector types with the names the reference's host API uses
// (nv::Vec3f, nv::Vec3i, nv::ROUND; ParallelFDTD src/math/geomMath.h:118-128).
#ifndef PFDTD_GEOMMATH_H
#define PFDTD_GEOMMATH_H

#include <cmath>

namespace nv {

template <typename T>
struct vec3 {
  T x, y, z;
  vec3() : x(T(0)), y(T(0)), z(T(0)) {}
  vec3(T x_, T y_, T z_) : x(x_), y(y_), z(z_) {}
  void set(T x_, T y_, T z_) { x = x_; y = y_; z = z_; }
  bool operator==(const vec3& o) const { return x == o.x && y == o.y && z == o.z; }
};

typedef vec3<float> Vec3f;
typedef vec3<int> Vec3i;
typedef vec3<unsigned int> Vec3ui;

// Round half up in single precision, as geomMath.h:126-128.
inline float ROUND(float num) { return float(std::floor(num + 0.5f)); }

}  // namespace nv

#ifndef PI
#define PI 3.14159265358979323846
#endif

#endif
