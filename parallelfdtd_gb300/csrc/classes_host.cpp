// Per-class update coefficients, evaluated on the host.
//
// Forward classes in the difference form (PFDTD_FORM_DIFFERENCE) hold
// a = s/(1+beta), b = K, c = 1 - beta and the float bits of 1 + beta in the
// pos word, for P+ = a (((1+beta) P + c (P - P-)) + l2 (S - b P)).
//
// A class is one (position byte, material byte) pair present in the grid.
// The terms of the reference kernels that depend only on that pair are
// computed here in the kernel's arithmetic type, with the reference's own
// expressions and association order, so that the device kernels only add the
// neighbour-dependent part.  This file is compiled with -ffp-contract=off:
// every product is rounded before it is summed, as the source is written.
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "pfdtd.h"

namespace pfdtd {
int fail(int code, const std::string& msg);

namespace {

template <typename A>
int eval(int scheme, int form, int quirks, const double* params,
         const std::vector<double>& materials, int n_mat, int n_coef,
         const std::vector<uint16_t>& keys, std::vector<uint8_t>& out) {
  const size_t n = keys.size();
  std::vector<A> ca(n), cb(n), cc(n);
  std::vector<uint32_t> cpos(n);
  const A l = (A)params[0];
  const A l2 = (A)params[1];
  const A octave = (A)params[3];
  const unsigned n_entries = (unsigned)n_mat * (unsigned)n_coef;
  for (size_t i = 0; i < n; ++i) {
    const unsigned pos = keys[i] >> 8;
    const unsigned m = keys[i] & 0xFFu;
    // Material index: forward kernel as written m*20*octave
    // (kernels3d.cu:513, reproduced under PFDTD_QUIRK_MATIDX), otherwise
    // m*20 + octave as the centred kernel computes it (kernels3d.cu:639).
    unsigned mi;
    if (scheme == PFDTD_SRL_FORWARD && (quirks & PFDTD_QUIRK_MATIDX))
      mi = (unsigned)((A)(m * 20u) * octave);
    else
      mi = (unsigned)((A)(m * 20u) + octave);
    if (mi >= n_entries)
      return fail(PFDTD_ERR_MATERIAL,
                  "material index " + std::to_string(mi) + " of node class (pos " +
                      std::to_string(pos) + ", mat " + std::to_string(m) +
                      ") lies outside the material table of " + std::to_string(n_entries) +
                      " entries");
    const A Y = (A)materials[mi];
    const A sw = (A)(pos >> 7);
    if (scheme == PFDTD_IWB) {
      // IWB (finite-volume closure): pos is the geometry code 1 + W16 +
      // 64 * face of an inside node (0 outside); wall nodes (face = 1) lose
      // beta = lambda * Y * W16/16, nodes closed only diagonally none.
      const A swi = (A)(pos != 0);
      const A W = pos >= 65 ? (A)(int)(pos - 65) * (A)0.0625 : (A)0;
      const A beta = Y * l * W;
      ca[i] = swi * ((A)1 / ((A)1 + beta));
      cb[i] = (A)2 - (A)3.5 * l2;  // d4 = 2 - 7/2 lambda^2 (-3/2 at lambda = 1)
      cc[i] = (A)1 - beta;
      // bit 30: an inside node with a closed neighbour (code >= 2), updated
      // by the closure pass on the TMA path
      cpos[i] = pos | (pos >= 2 ? 0x40000000u : 0u);
      continue;
    } else if (scheme != PFDTD_SRL && form == PFDTD_FORM_DIFFERENCE && sizeof(A) == 4) {
      // difference form: a = s/(1+beta), b = K, c = 1 - beta and, in the
      // pos word, the bits of the float 1 + beta
      const A position = (A)(pos & 0x7Fu);
      const A beta = (A)0.5 * (Y * ((A)6 - position) * l);
      const A onep = (A)1 + beta;
      ca[i] = sw * ((A)1 / onep);
      cb[i] = position;
      cc[i] = (A)1 - beta;
      const float e = (float)onep;
      uint32_t bits;
      std::memcpy(&bits, &e, 4);
      cpos[i] = bits;
      continue;
    } else if (scheme != PFDTD_SRL) {
      // kernels3d.cu:509-526
      const A position = (A)(pos & 0x7Fu);
      const A beta = (A)0.5 * (Y * ((A)6 - position) * l);
      ca[i] = sw * ((A)1 / ((A)1 + beta));
      cb[i] = (A)2 - position * l2;
      cc[i] = (A)1 - beta;
    } else {
      // kernels3d.cu:634-663
      const A dx = (A)(pos & 0x01u), dy = (A)((pos & 0x02u) >> 1), dz = (A)((pos & 0x04u) >> 2);
      const A beta = Y * l * (dx + dy + dz);
      ca[i] = sw * ((A)1 / ((A)1 + beta));
      cb[i] = (A)2 - (A)6 * l2;
      cc[i] = beta - (A)1;
    }
    cpos[i] = pos;
  }
  out.resize(n * (3 * sizeof(A) + sizeof(uint32_t)));
  uint8_t* p = out.data();
  std::memcpy(p, ca.data(), n * sizeof(A));
  std::memcpy(p + n * sizeof(A), cb.data(), n * sizeof(A));
  std::memcpy(p + 2 * n * sizeof(A), cc.data(), n * sizeof(A));
  std::memcpy(p + 3 * n * sizeof(A), cpos.data(), n * sizeof(uint32_t));
  return PFDTD_OK;
}

}  // namespace

int eval_class_coefs(int precision, int scheme, int form, int quirks, const double* params,
                     const std::vector<double>& materials, int n_mat, int n_coef,
                     const std::vector<uint16_t>& keys, std::vector<uint8_t>& out_tab) {
  if (precision == PFDTD_F64)
    return eval<double>(scheme, form, quirks, params, materials, n_mat, n_coef, keys, out_tab);
  return eval<float>(scheme, form, quirks, params, materials, n_mat, n_coef, keys, out_tab);
}

}  // namespace pfdtd
