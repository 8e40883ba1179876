// Position -> element index (ParallelFDTD src/base/SrcRec.cpp:26-34).
#include "SrcRec.h"

nv::Vec3i Position::getElementIdx(unsigned fs, float c, float lambda) {
  nv::Vec3i ret;
  const float dx = c / ((float)fs * lambda);
  ret.set((int)nv::ROUND(p_.x / dx), (int)nv::ROUND(p_.y / dx), (int)nv::ROUND(p_.z / dx));
  return ret;
}
