// ---------------------------------------------------------------------------
// CPU ORACLE — test infrastructure only.
//
// This file restates, in plain C++, the arithmetic of ParallelFDTD's
// time-stepping hot path so that the CUDA implementation can be checked
// against it.  Only the tests, the smoke check and the CPU-baseline leg of
// the benchmark load it; nothing in the product links or calls it.
//
// Parity pin: the reference's own update, padding and node-translation
// kernels and its host classes, compiled unchanged (oracle/build_ref.py),
// produced the golden vectors in tests/golden/ref_fields.npz and
// ref_host_golden.txt (tests/golden/make_ref_golden.py); this restatement
// reproduces every one of them bit for bit (tests/test_ref_golden_cpu.py).
// It is also pinned against the known-answer values the reference's unit
// tests hold (tests/SimulationParametersTest.cpp, MaterialHandlerTest.cpp,
// CudaMeshTest.cpp) and its partition-invariance property.  The IWB scheme,
// the DIF walls, 16-bit storage and the difference form have no counterpart
// in the reference and follow this library's written specification.
//
// Every function cites the reference file:line it follows.  Build with
// -ffp-contract=off so that every product is rounded before it is summed,
// exactly as written in the reference source.
// ---------------------------------------------------------------------------
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cstdlib>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// cudaMesh.h:35-44 — node byte bit masks.
constexpr unsigned kInsideSwitch = 7;
constexpr unsigned kForwardMask = 0x7F;
constexpr unsigned kCenteredMask = 0x80;
constexpr unsigned kDirX = 0x01, kDirY = 0x02, kDirZ = 0x04;
constexpr unsigned kSignX = 0x10, kSignY = 0x20, kSignZ = 0x40;

// cudaMesh.cu:328-361 (toBilbao): voxelizer boundary id 0..27 -> forward K.
void to_bilbao(uint8_t* pos, uint8_t* mat) {
  unsigned k = *pos;
  if (k == 0) { *pos = 0; *mat = 0; return; }
  if (k <= 8) { *pos = 3 | 0x80; return; }
  if (k <= 20) { *pos = 4 | 0x80; return; }
  if (k <= 26) { *pos = 5 | 0x80; return; }
  if (k == 27) { *pos = 6 | 0x80; return; }
  // k > 27: left unchanged, as in the reference.
}

// cudaMesh.cu:363-480 (toKowalczyk): boundary id -> centred DIR/SIGN bits.
// The table lists, per id, the bits the reference assigns.
const uint8_t kKowalczykTable[28] = {
    0,
    kSignZ | kDirX | kDirY | kDirZ | kCenteredMask,                  // 1
    kSignZ | kSignX | kDirX | kDirY | kDirZ | kCenteredMask,         // 2
    kSignZ | kSignY | kDirX | kDirY | kDirZ | kCenteredMask,         // 3
    kSignZ | kSignY | kSignX | kDirX | kDirY | kDirZ | kCenteredMask, // 4
    kDirX | kDirY | kDirZ | kCenteredMask,                           // 5
    kSignX | kDirX | kDirY | kDirZ | kCenteredMask,                  // 6
    kSignY | kDirX | kDirY | kDirZ | kCenteredMask,                  // 7
    kSignY | kSignX | kDirX | kDirY | kDirZ | kCenteredMask,         // 8
    kDirY | kDirZ | kSignZ | kCenteredMask,                          // 9
    kDirY | kDirZ | kSignZ | kSignY | kCenteredMask,                 // 10
    kDirX | kDirZ | kSignZ | kCenteredMask,                          // 11
    kDirX | kDirZ | kSignZ | kSignX | kCenteredMask,                 // 12
    kDirY | kDirZ | kCenteredMask,                                   // 13
    kDirY | kDirZ | kSignY | kCenteredMask,                          // 14
    kDirX | kDirZ | kCenteredMask,                                   // 15
    kDirX | kDirZ | kSignX | kCenteredMask,                          // 16
    kDirY | kDirX | kCenteredMask,                                   // 17
    kDirX | kDirY | kSignX | kCenteredMask,                          // 18
    kDirX | kDirY | kSignY | kCenteredMask,                          // 19
    kDirY | kDirX | kSignY | kSignX | kCenteredMask,                 // 20
    kDirZ | kSignZ | kCenteredMask,                                  // 21
    kDirY | kSignY | kCenteredMask,                                  // 22
    kDirY | kCenteredMask,                                           // 23
    kDirX | kSignX | kCenteredMask,                                  // 24
    kDirX | kCenteredMask,                                           // 25
    kDirZ | kCenteredMask,                                           // 26
    kCenteredMask,                                                   // 27
};

void to_kowalczyk(uint8_t* pos, uint8_t* mat) {
  unsigned k = *pos;
  if (k == 0) { *pos = 0; *mat = 0; return; }
  if (k <= 27) { *pos = kKowalczykTable[k]; return; }
}

// Material-table index of a node.  Forward kernel (kernels3d.cu:513) parses
// `m*20*+octave` as m*20*octave (ref_quirk bit 0); the intended rule, and the
// centred kernel's (kernels3d.cu:639), is m*20+octave.
template <typename T>
bool material_index(unsigned m, T octave, bool quirk_mat, unsigned n_entries,
                    unsigned* out) {
  unsigned idx;
  if (quirk_mat)
    idx = (unsigned)((T)(m * 20u) * octave);
  else
    idx = (unsigned)((T)(m * 20u) + octave);
  if (idx >= n_entries) return false;
  *out = idx;
  return true;
}

// Field storage types.  FP16 uses the compiler's IEEE binary16 type (round to
// nearest even on conversion); BF16 keeps the top 16 bits of a float, rounded
// to nearest even.  Arithmetic happens in float for both.
struct BF16 {
  uint16_t v;
};
inline float to_float(float x) { return x; }
inline double to_float(double x) { return x; }
inline float to_float(_Float16 x) { return (float)x; }
inline float to_float(BF16 x) {
  uint32_t u = (uint32_t)x.v << 16;
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}
template <typename S> inline S from_float(float f);
template <> inline float from_float<float>(float f) { return f; }
template <> inline _Float16 from_float<_Float16>(float f) { return (_Float16)f; }
template <> inline BF16 from_float<BF16>(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  if ((u & 0x7F800000u) == 0x7F800000u && (u & 0x7FFFFFu)) return BF16{(uint16_t)((u >> 16) | 0x40)};
  u += 0x7FFFu + ((u >> 16) & 1u);
  return BF16{(uint16_t)(u >> 16)};
}
template <typename S> struct Arith { typedef float type; };
template <> struct Arith<double> { typedef double type; };
template <typename S> inline S from_arith(typename Arith<S>::type v) { return from_float<S>(v); }
template <> inline double from_arith<double>(double v) { return v; }

struct RunDesc {
  int scheme;   // 0 forward (Bilbao), 1 centred (Kowalczyk), 3 IWB (centred encoding)
  int quirks;   // bit0: forward material index m*20*octave; bit1: soft source overwrites;
                // bit8: forward update in the difference form (the library's
                // PFDTD_FORM_DIFFERENCE, no counterpart in the reference)
  int64_t X, Y, Z;
  const uint8_t* pos;
  const uint8_t* mat;
  const void* table;  // [n_mat*20] of T
  int n_mat;
  const void* params; // [4] of T: lambda, lambda^2, 1/3, octave
  int n_src;
  const int64_t* src_idx;  // flat index, -1 = not in the domain
  const int32_t* src_type; // 0 hard, 1 soft, 2 transparent (added like soft)
  const void* src_samples; // [n_src * steps] of T
  int n_rec;
  const int64_t* rec_idx;
  int64_t steps;
  int threads;
  // Frequency-dependent boundaries: per material a flag and the filter
  // b0..b3, a1..a3 (order <= 3, unused coefficients 0).
  const int32_t* dif_flag;   // [n_mat] or null
  const void* dif_coef;      // [n_mat * 7] of T
  // IWB only, derived by run(): per node the closed-neighbour mask and the
  // class code (see iwb_geometry).
  const uint32_t* iwb_mask = nullptr;
  const uint8_t* iwb_code = nullptr;
};

// IWB geometry of one node: bit k of the mask is set when the k-th of the 26
// neighbours (offsets visited for dz, dy, dx in -1, 0, 1, skipping the
// centre) is closed, i.e. outside the grid or without the inside bit.  The
// class code is 0 for a node without the inside bit, else
// 1 + W16 + 64 * face, with W16 = 4 (closed faces) + 2 (closed edges) +
// (closed corners) and face = 1 when a face neighbour is closed.
void iwb_geometry(const uint8_t* pos, int64_t N, int64_t X, int64_t XY, int64_t c,
                  uint32_t* mask, uint8_t* code) {
  uint32_t m = 0;
  int w16 = 0, face = 0, k = 0;
  for (int dz = -1; dz <= 1; ++dz)
    for (int dy = -1; dy <= 1; ++dy)
      for (int dx = -1; dx <= 1; ++dx) {
        const int n = (dx != 0) + (dy != 0) + (dz != 0);
        if (n == 0) continue;
        const int64_t i = c + dz * XY + dy * X + dx;
        const bool open = i >= 0 && i < N && (pos[i] >> 7);
        if (!open) {
          m |= 1u << k;
          w16 += n == 1 ? 4 : (n == 2 ? 2 : 1);
          face |= n == 1;
        }
        ++k;
      }
  *mask = m;
  *code = (pos[c] >> 7) ? (uint8_t)(1 + w16 + 64 * face) : 0;
}

// Geometric factor G of a boundary node: the loss term of the FI update is
// beta (p+ - p-) = 2 G Y x with x = (p+ - p-)/2 (forward: beta = 0.5 Y (6-K)
// lambda, kernels3d.cu:514; centred: beta = lambda Y axes; IWB: pos is the
// class code, beta = lambda Y W16/16 when a face neighbour is closed).
template <typename T>
T geometric_factor(int scheme, unsigned pos, T lambda) {
  if (scheme == 0) return (T)0.5 * (((T)6 - (T)(pos & kForwardMask)) * lambda);
  if (scheme == 3) {
    if (pos < 65) return (T)0;  // outside, or closed diagonally only
    return lambda * ((T)(int)(pos - 65) * (T)0.0625);
  }
  const T ndirs = (T)((pos & 1u) + ((pos >> 1) & 1u) + ((pos >> 2) & 1u));
  return lambda * ndirs;
}

// IWB 27-point compact scheme (no counterpart in the reference; the
// reference's UpdateType has SRL schemes only, SimulationParameters.h:39).
//
// Interior: p+ = d1*S1 + d2*S2 + d3*S3 + d4*p - p-, with S1/S2/S3 the sums of
// the 6 face, 12 edge and 8 corner neighbours and (a, b) = (1/4, 1/16):
// d1 = l2/4, d2 = l2/8, d3 = l2/16, d4 = 2 - 7/2 l2 (l2 = lambda^2; at the
// scheme's stability limit lambda = 1: 1/4, 1/8, 1/16, -3/2; Kowalczyk & van
// Walstijn, IEEE TASLP 19(1), 2011), evaluated as
// l2 * ((S1/4 + S2/8) + S3/16) + d4 * p.
// Boundary (finite-volume closure on the voxel grid): a closed neighbour
// (see iwb_geometry) contributes the node's own value p, so no flux crosses
// the closed faces, edges and corners of the node's cell.  The update is then
// a weighted graph Laplacian over the open nodes, whose spectrum lies inside
// the full lattice's, so the scheme is energy-stable for lambda <= 1 on any
// voxel geometry.  A node with a closed face neighbour (a wall node, carrying
// its wall's material) adds the locally reacting loss
// beta = lambda * Y * W, W = W16/16 the summed weight of its closed
// neighbours:
//   p+ = s * (d1*S1' + d2*S2' + d3*S3' + d4*p - (1 - beta)*p-) / (1 + beta).
// Canonical evaluation order (shared with the CUDA kernels), built from
// in-plane sums so that a z-marching kernel can compute each plane's sums
// once and use them for the three planes next to it.  With m(dz, dy, dx) the
// neighbour values after the closure substitution and, per plane dz,
//   c0(dz) = m(dz, 0, 0)
//   c1(dz) = ((m(dz,-1,0) + m(dz,0,-1)) + m(dz,0,1)) + m(dz,1,0)
//   c2(dz) = ((m(dz,-1,-1) + m(dz,-1,1)) + m(dz,1,-1)) + m(dz,1,1),
// S1 = (c1(0) + c0(-1)) + c0(1), S2 = (c2(0) + c1(-1)) + c1(1),
// S3 = c2(-1) + c2(1); then ((l2 * ((S1/4 + S2/8) + S3/16) + d4*p) - c*p-) * a.
// The closed mask's bit k is the k-th offset in (dz, dy, dx) row-major order
// with the centre left out.
template <typename T, typename St>
T iwb_node(const St* P, int64_t N, int64_t c, int64_t X, int64_t XY, uint32_t mask, T pp, T a,
           T cc, T l2) {
  const T p = (T)to_float(P[c]);
  T m[3][3][3];
  int k = 0;
  for (int dz = -1; dz <= 1; ++dz)
    for (int dy = -1; dy <= 1; ++dy)
      for (int dx = -1; dx <= 1; ++dx) {
        T v = p;
        if (dx != 0 || dy != 0 || dz != 0) {
          const int64_t i = c + dz * XY + dy * X + dx;
          if (!((mask >> k) & 1u)) v = (T)to_float(P[i]);
          ++k;
        }
        m[dz + 1][dy + 1][dx + 1] = v;
      }
  auto c1 = [&](int z) { return ((m[z][0][1] + m[z][1][0]) + m[z][1][2]) + m[z][2][1]; };
  auto c2 = [&](int z) { return ((m[z][0][0] + m[z][0][2]) + m[z][2][0]) + m[z][2][2]; };
  const T s1 = (c1(1) + m[0][1][1]) + m[2][1][1];
  const T s2 = (c2(1) + c1(0)) + c1(2);
  const T s3 = c2(0) + c2(2);
  const T sw = l2 * (s1 * (T)0.25 + s2 * (T)0.125 + s3 * (T)0.0625);
  const T d4 = (T)2 - (T)3.5 * l2;
  return a * ((sw + d4 * p) - cc * pp);
}

// One leapfrog update over z in [1, Z-2] writing into Pp.
// Forward rule: kernels3d.cu:485-529.  Centred rule: kernels3d.cu:608-665.
// A frequency-dependent boundary node (material with a filter, inside,
// G > 0) replaces the FI loss by the filter output y = b0 x + s1
// (transposed direct form II, x = (p+ - p-)/2):
//   p+ = s/(1+G b0) * ((L - (1 - G b0) p-) - 2 G s1)      forward, IWB
//   p+ = s/(1+G b0) * ((L + (G b0 - 1) p-) - 2 G s1)      centred SRL
// with L the lossless part of the scheme's update, then
//   s1 = (b1 x - a1 y) + s2,  s2 = (b2 x - a2 y) + s3,  s3 = b3 x - a3 y.
template <typename T>
struct DifState {
  std::vector<int64_t> slot;  // per node: state slot or -1
  std::vector<T> s;           // [n_slots * 3]
};

template <typename T, typename St>
int update(const RunDesc& d, const St* P, St* Pp, const std::vector<T>& beta_tab,
           const std::vector<uint8_t>& valid, DifState<T>* dif = nullptr) {
  const T* prm = (const T*)d.params;
  const T l = prm[0], l2 = prm[1];
  const int64_t X = d.X, XY = d.X * d.Y, Z = d.Z;
  const T* dcoef = (const T*)d.dif_coef;
  (void)l;
#pragma omp parallel for schedule(static) num_threads(d.threads)
  for (int64_t z = 1; z < Z - 1; ++z) {
    for (int64_t c = z * XY; c < (z + 1) * XY; ++c) {
      const unsigned pos = d.scheme == 3 ? d.iwb_code[c] : d.pos[c];
      const unsigned key = (pos << 8) | d.mat[c];
      T beta = beta_tab[key];
      const T p = to_float(P[c]);
      const T pp = to_float(Pp[c]);
      const int64_t slot = dif ? dif->slot[c] : -1;
      T g2 = 0, s1 = 0;
      const T* f = nullptr;
      if (slot >= 0) {
        // DIF boundary node: beta from b0, explicit filter state.
        const unsigned mi_f = d.mat[c];
        f = dcoef + 7 * mi_f;
        const T G = geometric_factor<T>(d.scheme, pos, l);
        beta = G * f[0];
        g2 = (T)2 * G;
        s1 = dif->s[3 * slot];
      }
      T ret;
      if (d.scheme == 3) {
        const T sw = (T)(pos != 0);
        const uint32_t mask = d.iwb_mask[c];
        if (slot >= 0) {
          const T lossless = iwb_node<T, St>(P, XY * Z, c, X, XY, mask, (T)0, (T)1, (T)0, l2);
          ret = sw * ((T)1 / ((T)1 + beta)) * ((lossless - ((T)1 - beta) * pp) - g2 * s1);
        } else {
          ret = iwb_node<T, St>(P, XY * Z, c, X, XY, mask, pp, sw * ((T)1 / ((T)1 + beta)),
                                (T)1 - beta, l2);
        }
        // A node without the inside bit holds +0: its update is 0 times a
        // finite value, whose sign would depend on neighbours that no inside
        // node ever reads (the closure substitutes them); +0 fixes its bits.
        if (pos == 0) ret = (T)0;
      } else if (d.scheme == 0 && slot >= 0) {
        const T position = (T)(pos & kForwardMask);
        const T sw = (T)(pos >> kInsideSwitch);
        const T S = (T)to_float(P[c + XY]) + (T)to_float(P[c - XY]) + (T)to_float(P[c + X]) +
                    (T)to_float(P[c - X]) + (T)to_float(P[c + 1]) + (T)to_float(P[c - 1]);
        ret = sw * ((T)1 / ((T)1 + beta)) *
              ((((T)2 - position * l2) * p + l2 * S - ((T)1 - beta) * pp) - g2 * s1);
      } else if (d.scheme == 0 && (d.quirks & 0x100)) {
        // Difference form of the same update (equal in exact arithmetic):
        // s/(1+b) (((1+b) p + (1-b)(p - pp)) + l2 (S - K p)).
        const T position = (T)(pos & kForwardMask);
        const T sw = (T)(pos >> kInsideSwitch);
        const T S = (T)to_float(P[c + XY]) + (T)to_float(P[c - XY]) + (T)to_float(P[c + X]) +
                    (T)to_float(P[c - X]) + (T)to_float(P[c + 1]) + (T)to_float(P[c - 1]);
        ret = sw * ((T)1 / ((T)1 + beta)) *
              ((((T)1 + beta) * p + ((T)1 - beta) * (p - pp)) + l2 * (S - position * p));
      } else if (d.scheme == 0) {
        const T position = (T)(pos & kForwardMask);
        const T sw = (T)(pos >> kInsideSwitch);
        const T S = (T)to_float(P[c + XY]) + (T)to_float(P[c - XY]) + (T)to_float(P[c + X]) +
                    (T)to_float(P[c - X]) + (T)to_float(P[c + 1]) + (T)to_float(P[c - 1]);
        ret = sw * ((T)1 / ((T)1 + beta)) *
              (((T)2 - position * l2) * p + l2 * S - ((T)1 - beta) * pp);
      } else {
        const T sw = (T)(pos >> kInsideSwitch);
        const T dx = (T)(pos & kDirX), dy = (T)((pos & kDirY) >> 1),
                dz = (T)((pos & kDirZ) >> 2);
        T pz[2], py[2], px[2];
        pz[1] = to_float(P[c - XY]);
        pz[0] = to_float(P[c + XY]);
        py[0] = to_float(P[c - X]);
        py[1] = to_float(P[c + X]);
        px[0] = to_float(P[c - 1]);
        px[1] = to_float(P[c + 1]);
        const int sx = (pos & kSignX) >> 4, sy = (pos & kSignY) >> 5,
                  sz = (pos & kSignZ) >> 6;
        const T Sb = px[sx] * dx + py[sy] * dy + pz[sz] * dz;
        const T S = (px[0] + px[1] + py[0] + py[1] + pz[0] + pz[1] + Sb) * l2;
        if (slot >= 0)
          ret = sw * ((T)1 / ((T)1 + beta)) *
                (((S - ((T)2 - (T)6 * l2) * p) + (beta - (T)1) * pp) - g2 * s1);
        else
          ret = (S - ((T)2 - (T)6 * l2) * p + (beta - (T)1) * pp) * sw *
                ((T)1 / ((T)1 + beta));
      }
      if (slot >= 0) {
        T* st = &dif->s[3 * slot];
        const T x = (ret - pp) * (T)0.5;
        const T y = f[0] * x + st[0];
        st[0] = (f[1] * x - f[4] * y) + st[1];
        st[1] = (f[2] * x - f[5] * y) + st[2];
        st[2] = f[3] * x - f[6] * y;
      }
      Pp[c] = from_arith<St>(ret);
    }
  }
  return 0;
}

// Per-(pos, mat) beta, computed with the reference's expressions
// (forward kernels3d.cu:514, centred kernels3d.cu:640).
template <typename T>
int beta_table(const RunDesc& d, std::vector<T>& beta, std::vector<uint8_t>& valid) {
  const T* prm = (const T*)d.params;
  const T* tab = (const T*)d.table;
  const unsigned n_entries = (unsigned)d.n_mat * 20u;
  beta.assign(65536, (T)0);
  valid.assign(65536, 0);
  // Presence scan: only keys present in the grid must have a valid index.
  std::vector<uint8_t> present(65536, 0);
  const int64_t N = d.X * d.Y * d.Z;
  for (int64_t i = d.X * d.Y; i < N - d.X * d.Y; ++i)
    present[((unsigned)(d.scheme == 3 ? d.iwb_code[i] : d.pos[i]) << 8) | d.mat[i]] = 1;
  for (unsigned key = 0; key < 65536; ++key) {
    if (!present[key]) continue;
    const unsigned pos = key >> 8, m = key & 0xFF;
    unsigned mi;
    const bool quirk = (d.scheme == 0) && (d.quirks & 1);
    if (!material_index<T>(m, prm[3], quirk, n_entries, &mi)) return -3;
    const T Y = tab[mi];
    if (d.scheme == 0) {
      const T position = (T)(pos & kForwardMask);
      beta[key] = (T)0.5 * (Y * ((T)6 - position) * prm[0]);
    } else if (d.scheme == 3) {
      // pos is the class code: 1 + W16 + 64 * face for inside nodes
      const T W = pos >= 65 ? (T)(int)(pos - 65) * (T)0.0625 : (T)0;
      beta[key] = Y * prm[0] * W;
    } else {
      const T dx = (T)(pos & kDirX), dy = (T)((pos & kDirY) >> 1),
              dz = (T)((pos & kDirZ) >> 2);
      beta[key] = Y * prm[0] * (dx + dy + dz);
    }
    valid[key] = 1;
  }
  return 0;
}

// Step loop of launchFDTD3d / launchFDTD3dDouble (kernels3d.cu:83-181):
// inject sources into P (:93-104), update (:109-153), swap (:160),
// record receivers from the new P (:164-173).
template <typename T, typename S>
int run(const RunDesc& d0, S* P, S* Pp, T* out) {
  if (d0.X < 1 || d0.Y < 1 || d0.Z < 3) return -1;
  RunDesc d = d0;
  std::vector<uint32_t> iwb_mask;
  std::vector<uint8_t> iwb_code;
  if (d.scheme == 3) {
    const int64_t N = d.X * d.Y * d.Z;
    iwb_mask.assign(N, 0);
    iwb_code.assign(N, 0);
    for (int64_t c = 0; c < N; ++c)
      iwb_geometry(d.pos, N, d.X, d.X * d.Y, c, &iwb_mask[c], &iwb_code[c]);
    d.iwb_mask = iwb_mask.data();
    d.iwb_code = iwb_code.data();
  }
  std::vector<T> beta;
  std::vector<uint8_t> valid;
  int rc = beta_table<T>(d, beta, valid);
  if (rc) return rc;
  const T* samples = (const T*)d.src_samples;
  const int64_t N = d.X * d.Y * d.Z;
  DifState<T> dif;
  bool any_dif = false;
  if (d.dif_flag) {
    const T l = ((const T*)d.params)[0];
    dif.slot.assign(N, -1);
    int64_t n_slots = 0;
    for (int64_t i = d.X * d.Y; i < N - d.X * d.Y; ++i) {
      const unsigned pos = d.scheme == 3 ? d.iwb_code[i] : d.pos[i];
      const bool inside = d.scheme == 3 ? pos != 0 : (pos >> kInsideSwitch) != 0;
      if (!inside || d.mat[i] >= (unsigned)d.n_mat || !d.dif_flag[d.mat[i]]) continue;
      if (geometric_factor<T>(d.scheme, pos, l) <= (T)0) continue;
      dif.slot[i] = n_slots++;
    }
    dif.s.assign(3 * n_slots, (T)0);
    any_dif = n_slots > 0;
  }
  for (int64_t step = 0; step < d.steps; ++step) {
    for (int i = 0; i < d.n_src; ++i) {
      const int64_t idx = d.src_idx[i];
      if (idx < 0 || idx >= N) continue;
      const T v = samples[(int64_t)i * d.steps + step];
      if (d.src_type[i] == 0 || (d.quirks & 2))
        P[idx] = from_arith<S>(v);  // setSample, cudaMesh.h:322-338 (and Q4 addSample)
      else
        P[idx] = from_arith<S>((T)to_float(P[idx]) + v);  // addSample, cudaMesh.h:349-369
    }
    update<T, S>(d, P, Pp, beta, valid, any_dif ? &dif : nullptr);
    S* t = P; P = Pp; Pp = t;
    for (int r = 0; r < d.n_rec; ++r) {
      const int64_t idx = d.rec_idx[r];
      if (idx < 0 || idx >= N) continue;
      out[(int64_t)r * d.steps + step] = to_float(P[idx]);
    }
  }
  // Leave the caller's first buffer holding the current field: after an odd
  // number of swaps the roles of the two buffers are exchanged.
  if ((d.steps & 1) != 0) {
    std::vector<S> cur_copy(P, P + N);      // P is the caller's second buffer
    std::memcpy(P, Pp, sizeof(S) * N);
    std::memcpy(Pp, cur_copy.data(), sizeof(S) * N);
  }
  return 0;
}

// SimulationParameters.cpp:262-298 (getRegularSourceSample) in float.
float regular_sample_f(int input_type, uint32_t step, uint32_t fs, const float* data,
                       uint32_t data_len) {
  float sample = 0.f;
  switch (input_type) {
    case 0:  // IMPULSE
      sample += (step == 1) ? 1.f : 0.f;
      break;
    case 1: {  // GAUSSIAN, t0 = 40, width = 4
      float t0 = 40, width = 4;
      float e = ((float)(step - t0) / width);
      sample += expf(-0.5f * (e * e));
      break;
    }
    case 3:  // DATA
      sample += (step < data_len) ? data[step] : 0.f;
      break;
    case 2: {  // SINE, 120 Hz
      float freq = 120;
      float t = (float)step / (float)fs;
      sample += sinf(2.f * (float)3.14159265358979323846 * freq * t);
      break;
    }
  }
  return sample;
}

// SimulationParameters.cpp:312-348 (getRegularSourceSampleDouble).
double regular_sample_d(int input_type, uint32_t step, uint32_t fs, const double* data,
                        uint32_t data_len) {
  double sample = 0.0;
  switch (input_type) {
    case 0:
      sample += (step == 1) ? 1.0 : 0.0;
      break;
    case 1: {
      double t0 = 40, width = 4;
      double e = ((float)(step - t0) / width);
      sample += exp(-0.5f * (e * e));
      break;
    }
    case 3:
      sample += (step < data_len) ? data[step] : 0.0;
      break;
    case 2: {
      double freq = 120;
      double t = (double)step / (double)fs;
      sample += sin(2.f * (double)3.14159265358979323846 * freq * t);
      break;
    }
  }
  return sample;
}

}  // namespace

extern "C" {

// cudaMesh.cu:155-251 scheme translation, element_type dispatch as in
// cudaMesh.cu:70-73 is done by the caller.
void oracle_encode_nodes(int centred, uint8_t* pos, uint8_t* mat, int64_t n) {
  for (int64_t i = 0; i < n; ++i) {
    if (centred) to_kowalczyk(pos + i, mat + i);
    else to_bilbao(pos + i, mat + i);
  }
}

// cudaMesh.cu:500-514 (calcBoundaries).
void oracle_count_boundaries(const uint8_t* pos, int64_t n, uint8_t air_value,
                             uint8_t outside_value, uint32_t* air, uint32_t* boundary) {
  uint32_t a = 0, b = 0;
  for (int64_t i = 0; i < n; ++i) {
    if (pos[i] == air_value) ++a;
    if (pos[i] != outside_value && pos[i] != air_value) ++b;
  }
  *air = a;
  *boundary = b;
}

// cudaMesh.cu:253-304 (padWithZeros for one byte mesh).  `in_len` is the
// number of readable input bytes; reads past it (which the reference performs
// when a dimension is padded) yield 0.
void oracle_pad(const uint8_t* in, int64_t in_len, const uint32_t dims[3],
                uint32_t bx, uint32_t by, uint32_t bz, uint8_t* out,
                uint32_t out_dims[3]) {
  uint32_t dx = dims[0], dy = dims[1], dz = dims[2];
  uint32_t padX = 0, padY = 0, padZ = 0;
  if (dx % bx) padX = bx - dx % bx;
  if (dy % by) padY = by - dy % by;
  if (dz % bz) padZ = bz - dz % bz;
  const uint64_t nx = dx + padX, ny = dy + padY, nz = dz + padZ;
  if (out) {
    std::memset(out, 0, nx * ny * nz);
    for (uint64_t z = 0; z < dz; ++z)
      for (uint64_t y = 0; y < ny; ++y)
        for (uint64_t x = 0; x < nx; ++x) {
          if (x < (uint64_t)dx + 1 && x > 0 && y < (uint64_t)dy + 1 && y > 0 && z > 0) {
            uint64_t old_idx = z * dx * dy + y * dx + x;
            uint64_t new_idx = z * (dx + padX) * (dy + padY) + y * (dx + padX) + x;
            out[new_idx] = (old_idx < (uint64_t)in_len) ? in[old_idx] : 0;
          }
        }
  }
  out_dims[0] = (uint32_t)nx;
  out_dims[1] = (uint32_t)ny;
  out_dims[2] = (uint32_t)nz;
}

// SimulationParameters.cpp:139-148 / :300-310: one source sample (float).
// src_type 2 = transparent: s(n) - sum_{i<n} h[n-i] s(i).
float oracle_source_sample_f32(int src_type, int input_type, uint32_t step, uint32_t fs,
                               const float* data, uint32_t data_len, const float* grid_ir,
                               uint32_t ir_len) {
  float sample = 0.f;
  if (src_type == 2) {
    float acc = 0.f;
    for (uint32_t i = 0; i < step; ++i) {
      float h = (step - i < ir_len) ? grid_ir[step - i] : 0.f;
      acc += h * regular_sample_f(input_type, i, fs, data, data_len);
    }
    sample += regular_sample_f(input_type, step, fs, data, data_len) - acc;
  } else {
    sample += regular_sample_f(input_type, step, fs, data, data_len);
  }
  return sample;
}

// SimulationParameters.cpp:150-159 / :350-360 (double).
double oracle_source_sample_f64(int src_type, int input_type, uint32_t step, uint32_t fs,
                                const double* data, uint32_t data_len, const float* grid_ir,
                                uint32_t ir_len) {
  double sample = 0.0;
  if (src_type == 2) {
    double acc = 0.0;
    for (uint32_t i = 0; i < step; ++i) {
      float h = (step - i < ir_len) ? grid_ir[step - i] : 0.f;
      acc += h * regular_sample_d(input_type, i, fs, data, data_len);
    }
    sample += regular_sample_d(input_type, step, fs, data, data_len) - acc;
  } else {
    sample += regular_sample_d(input_type, step, fs, data, data_len);
  }
  return sample;
}

// Full run (kernels3d.cu:31-203 float, :205-374 double; precision 2 and 3
// store the fields in FP16 / BF16 with float arithmetic; dif_flag/dif_coef
// optionally give materials frequency-dependent admittance filters).
// store the fields in FP16 / BF16 with float arithmetic).  P and Pp hold the
// initial (current, past) fields and receive the final ones; out receives
// [n_rec * steps] receiver samples, row per receiver (kernels3d.cu:183-191).
// Returns 0, or -1 bad dims, -3 material index out of the table.
int oracle_run(int precision, int scheme, int quirks, int64_t X, int64_t Y, int64_t Z,
               const uint8_t* pos, const uint8_t* mat, const void* table, int n_mat,
               const void* params, int n_src, const int64_t* src_idx,
               const int32_t* src_type, const void* src_samples, int n_rec,
               const int64_t* rec_idx, int64_t steps, void* P, void* Pp, void* out,
               int threads, const int32_t* dif_flag, const void* dif_coef) {
  RunDesc d{scheme, quirks, X, Y, Z, pos, mat, table, n_mat, params, n_src, src_idx,
            src_type, src_samples, n_rec, rec_idx, steps, threads > 0 ? threads : 1,
            dif_flag, dif_coef};
  switch (precision) {
    case 1: return run<double, double>(d, (double*)P, (double*)Pp, (double*)out);
    case 2: return run<float, _Float16>(d, (_Float16*)P, (_Float16*)Pp, (float*)out);
    case 3: return run<float, BF16>(d, (BF16*)P, (BF16*)Pp, (float*)out);
  }
  return run<float, float>(d, (float*)P, (float*)Pp, (float*)out);
}

int oracle_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
