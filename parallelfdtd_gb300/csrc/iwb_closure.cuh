// IWB closure nodes (no counterpart in the reference): the inside nodes with
// a closed neighbour, whose update substitutes the node's own value for every
// closed neighbour.  The streaming TMA update leaves them alone and the
// sparse pass k_iwb_closure (dif.cu) updates them with iwb_closure_apply.
#pragma once

#include "common.cuh"

namespace pfdtd {

// One closure node, records in ascending flat-index order.  cls is the
// node's class (an index into the class table).
struct ClosureRec {
  int64_t idx;
  uint32_t mask;
  uint32_t cls;
};

// Per DIF class: a, b, c, g2 and the filter b0..b3, a1..a3 (11 values).
constexpr int kDifClassVals = 11;

// Update of closure node i from its 3 x 3 x 3 neighbourhood m (raw values,
// centre included) and P^{n-1} pp: closed neighbours (mask bits in the
// canonical order of iwb_bit) take the centre's value, the canonical sums
// give sw, then either the frequency-independent rule of class c or, for a
// node with a DIF state slot, the DIF update (operation for operation as
// k_dif_update), and the result is stored to Pp[i].  A DIF node without a
// slot stores its sw to iwb_sw for the separate DIF pass.
template <typename S>
__device__ __forceinline__ void iwb_closure_apply(float (&m)[3][3][3], uint32_t mask, unsigned c,
                                                  float pp, ClassTab<float> tab, float l2,
                                                  int32_t slot, const float* __restrict__ dtab,
                                                  float* __restrict__ dstate,
                                                  float* __restrict__ iwb_sw, int64_t i,
                                                  S* __restrict__ Pp) {
  using R = Rn<float>;
  using Sto = Store<S>;
  const float p = m[1][1][1];
  int kk = 0;
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b)
#pragma unroll
      for (int e = 0; e < 3; ++e) {
        if (a == 1 && b == 1 && e == 1) continue;
        m[a][b][e] = ((mask >> kk) & 1u) ? p : m[a][b][e];
        ++kk;
      }
  float s1, s2, s3;
  iwb_sums(m, s1, s2, s3);
  const float sw = R::mul(l2, R::add(R::add(R::mul(s1, 0.25f), R::mul(s2, 0.125f)),
                                     R::mul(s3, 0.0625f)));
  if (slot >= 0) {
    const float* t = dtab + (int64_t)kDifClassVals * c;
    float* st = dstate + 4 * (int64_t)slot;
    const float s1d = st[0], ppd = st[3];
    const float num = R::sub(R::sub(R::add(sw, R::mul(t[1], p)), R::mul(t[2], ppd)),
                             R::mul(t[3], s1d));
    const float out = R::mul(t[0], num);
    const float xx = R::mul(R::sub(out, ppd), 0.5f);
    const float yy = R::add(R::mul(t[4], xx), s1d);
    st[0] = R::add(R::sub(R::mul(t[5], xx), R::mul(t[8], yy)), st[1]);
    st[1] = R::add(R::sub(R::mul(t[6], xx), R::mul(t[9], yy)), st[2]);
    st[2] = R::sub(R::mul(t[7], xx), R::mul(t[10], yy));
    st[3] = p;
    Pp[i] = Sto::store(out);
    return;
  }
  if (iwb_sw != nullptr && (__ldg(tab.pos + c) >> 31)) iwb_sw[i] = sw;
  const float out = R::mul(__ldg(tab.a + c), R::sub(R::add(sw, R::mul(__ldg(tab.b + c), p)),
                                                    R::mul(__ldg(tab.c + c), pp)));
  Pp[i] = Sto::store(out);
}

}  // namespace pfdtd
