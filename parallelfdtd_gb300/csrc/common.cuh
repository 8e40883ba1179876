// Internal declarations shared by the CUDA translation units of libpfdtd.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include <stdint.h>

#include <atomic>
#include <cmath>
#include <string>
#include <vector>

#include "pfdtd.h"

namespace pfdtd {

// ---------------------------------------------------------------------------
// Error reporting: one message per host thread, read by pfdtd_last_error().
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what, const char* file, int line);

#define PFDTD_CK(call)                                                       \
  do {                                                                       \
    cudaError_t e_ = (call);                                                 \
    if (e_ != cudaSuccess) return ::pfdtd::cuda_fail(e_, #call, __FILE__, __LINE__); \
  } while (0)

// GB300's SM count: the grid-stride kernels launch at most a small multiple
// of it (any grid size is correct; this one keeps every SM busy without
// oversubscribing).
constexpr int kGridSMs = 152;

extern std::atomic<int64_t> g_launches;
inline void count_launch(int64_t n = 1) { g_launches.fetch_add(n, std::memory_order_relaxed); }

// ---------------------------------------------------------------------------
// Arithmetic with explicit rounding.  Every product and sum is rounded on its
// own (no fused multiply-add), in the order the reference source writes it,
// so that the device results equal a -ffp-contract=off CPU evaluation.
template <typename T> struct Rn;
template <> struct Rn<float> {
  static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
  static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
  static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
};
template <> struct Rn<double> {
  static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
  static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
};

// Packed pairs of floats (two fields of one node) and the sm_100-family
// f32x2 operations on them.  Each lane of add/sub/mul.rn.f32x2 rounds as the
// scalar __fadd_rn/__fsub_rn/__fmul_rn.  ptxas may contract a packed multiply
// into a following packed add even with .rn, so kernels that must not fuse
// form products as fma2(x, y, nz) with nz = (-0, -0) taken from a kernel
// argument: one rounding of the exact product, and an addend the compiler
// cannot fold away.
namespace px {
typedef unsigned long long f2;  // the lower field in the low word
__device__ __forceinline__ f2 add2(f2 a, f2 b) {
  f2 d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2 sub2(f2 a, f2 b) {
  f2 d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2 mul2(f2 a, f2 b) {
  f2 d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) {
  f2 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ f2 pk2(float lo, float hi) {
  f2 d;
  asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "f"(lo), "f"(hi));
  return d;
}
__device__ __forceinline__ void up2(f2 v, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
}  // namespace px

// IWB 27-point sums of one node from its 3 x 3 x 3 neighbourhood
// m[dz+1][dy+1][dx+1] after the closure substitution (centre unused), in the
// scheme's canonical order, built from in-plane sums so that a z-march can
// share them between planes:
//   c1(dz) = ((m(dz,-1,0) + m(dz,0,-1)) + m(dz,0,1)) + m(dz,1,0)
//   c2(dz) = ((m(dz,-1,-1) + m(dz,-1,1)) + m(dz,1,-1)) + m(dz,1,1)
//   S1 = (c1(0) + m(-1,0,0)) + m(1,0,0),  S2 = (c2(0) + c1(-1)) + c1(1),
//   S3 = c2(-1) + c2(1).
template <typename A>
__device__ __forceinline__ A iwb_c1(const A (&q)[3][3]) {
  using R = Rn<A>;
  return R::add(R::add(R::add(q[0][1], q[1][0]), q[1][2]), q[2][1]);
}
template <typename A>
__device__ __forceinline__ A iwb_c2(const A (&q)[3][3]) {
  using R = Rn<A>;
  return R::add(R::add(R::add(q[0][0], q[0][2]), q[2][0]), q[2][2]);
}
template <typename A>
__device__ __forceinline__ void iwb_sums(const A (&m)[3][3][3], A& s1, A& s2, A& s3) {
  using R = Rn<A>;
  s1 = R::add(R::add(iwb_c1(m[1]), m[0][1][1]), m[2][1][1]);
  s2 = R::add(R::add(iwb_c2(m[1]), iwb_c1(m[0])), iwb_c1(m[2]));
  s3 = R::add(iwb_c2(m[0]), iwb_c2(m[2]));
}

// Storage type -> arithmetic type.
template <typename S> struct Store;
template <> struct Store<float> {
  using A = float;
  static __device__ __forceinline__ float load(float v) { return v; }
  static __device__ __forceinline__ float store(float v) { return v; }
};
template <> struct Store<double> {
  using A = double;
  static __device__ __forceinline__ double load(double v) { return v; }
  static __device__ __forceinline__ double store(double v) { return v; }
};
template <> struct Store<__half> {
  using A = float;
  static __device__ __forceinline__ float load(__half v) { return __half2float(v); }
  static __device__ __forceinline__ __half store(float v) { return __float2half_rn(v); }
};
template <> struct Store<__nv_bfloat16> {
  using A = float;
  static __device__ __forceinline__ float load(__nv_bfloat16 v) { return __bfloat162float(v); }
  static __device__ __forceinline__ __nv_bfloat16 store(float v) { return __float2bfloat16_rn(v); }
};

// ---------------------------------------------------------------------------
// Per-class coefficient table on the device.  A class is one distinct
// (position byte, material byte) pair present in the grid; the kernels read a
// class id per node instead of the two bytes.
//   forward: out = a * ((b*p + l2*S) - c*pp)
//   centred: out = a * ((l2*(S6 + Sb) - b*p) + c*pp),  pos = DIR/SIGN bits
template <typename A>
struct ClassTab {
  const A* a;
  const A* b;
  const A* c;
  const uint32_t* pos;
  int n;
};

// Tensor maps of the TMA update kernel (stencil_tma.cu): each field buffer
// (two, or four with temporal blocking) viewed as X-wide rows with and
// without the halo box, and the class ids.
struct TmaState {
  CUtensorMap halo[4];
  CUtensorMap tile[4];
  CUtensorMap cls;
  CUtensorMap mask;  // IWB closed-neighbour masks (4 bytes per node)
  int64_t key[7] = {0, 0, 0, 0, 0, 0, 0};
  bool ready = false;
  bool attr_set[2][2][2] = {{{false, false}, {false, false}}, {{false, false}, {false, false}}};
};

// Update kernel variants.
#define PFDTD_KERNEL_AUTO 0
#define PFDTD_KERNEL_ZMARCH 1
#define PFDTD_KERNEL_TMA 2
#define PFDTD_KERNEL_TB 3

struct GraphCache {
  cudaGraphExec_t exec = nullptr;
  int64_t key[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  int64_t launches = 0;  // kernels in one replay (counted while capturing)
};

}  // namespace pfdtd

// The opaque domain handle.
struct pfdtd_domain {
  int device = 0;
  int64_t serial = 0;        // unique per created domain (never reused)
  int sm_count = 152;
  int precision = PFDTD_F32;
  int scheme = PFDTD_SRL_FORWARD;
  int quirks = 0;
  int64_t X = 0, Y = 0, Z = 0, XY = 0, N = 0;
  // Batched fields: K independent fields per node sharing the geometry,
  // interleaved node-major (element = node * K + field); K a power of two.
  int K = 1, kshift = 0;
  int64_t NE = 0;            // field elements, N * K
  size_t esize = 4;          // storage bytes per field element
  int64_t margin = 0;        // elements before node 0 / after node N-1
  // Field buffers: two for the plain leapfrog (P^{n+1} written over P^{n-1}),
  // two more allocated for the temporally blocked update, which writes its
  // two output levels out of place.
  void* field_base[4] = {nullptr, nullptr, nullptr, nullptr};
  int cur = 0;               // index of the current field P^n
  int prev = 1;              // index of the past field P^{n-1}
  uint8_t* d_pos = nullptr;
  uint8_t* d_mat = nullptr;
  bool nodes_set = false;

  // material table and parameters (host copies, arithmetic type widened to double)
  std::vector<double> materials;
  int n_mat = 0, n_coef = 20;
  // lambda = sqrt(1/3) as SimulationParameters::setUpdateType sets it
  double params[4] = {std::sqrt(1.0 / 3.0), 1.0 / 3.0, 1.0 / 3.0, 0.0};
  // PFDTD_FORM_*: arithmetic form of the forward update
  int update_form = 0;

  // class table
  bool classes_dirty = true;
  int class_scheme = -1;
  int class_form = 0;        // update form the class table was built for
  int n_classes = 0;
  int cls_bytes = 1;
  void* d_cls = nullptr;     // per node class id (uint8 or uint16)
  // The class ids with every row padded to a multiple of 16 bytes, for the
  // TMA kernels' tensor map when X * cls_bytes is not (cls_pitch: row length
  // in ids; 0 when the TMA kernels read d_cls itself)
  void* d_cls_tma = nullptr;
  size_t cls_tma_bytes = 0;
  int64_t cls_pitch = 0;
  void* d_ctab = nullptr;    // coefficient arrays (a|b|c in arithmetic type, then pos u32)
  // IWB: per node the closed-neighbour mask (26 bits) and the class code
  // that stands for the position byte in the IWB class key (stencil.cu)
  uint32_t* d_iwb_mask = nullptr;
  uint8_t* d_iwb_code = nullptr;
  // IWB with DIF walls on the TMA path: the weighted neighbour sum sw of each
  // DIF node (classes flagged by bit 31 of their pos word), written by the
  // update kernel and read by the DIF pass instead of a second 27-point gather
  float* d_iwb_sw = nullptr;
  // IWB on the TMA path: the closure nodes (inside, with a closed neighbour;
  // classes flagged by bit 30 of their pos word) as flat-index order records
  // {index, closed mask, class} (dif.cu).  The TMA update leaves P^{n-1} at
  // these nodes and k_iwb_closure updates them.
  void* d_iwb_closure = nullptr;
  int64_t n_iwb_closure = 0;
  // per closure record: its DIF node slot (position in the DIF list), -1 for
  // a node without a filter; set when every DIF node has a record, and then
  // the closure pass also applies the DIF update (no separate DIF pass)
  int32_t* d_iwb_closure_dif = nullptr;
  bool iwb_closure_ready = false;
  int64_t class_version = 0;

  // sources / receivers
  int n_src = 0;
  int64_t n_samples = 0;
  int64_t* d_src_idx = nullptr;
  int32_t* d_src_mode = nullptr;   // 0 overwrite, 1 add
  void* d_src_samples = nullptr;   // [n_src * n_samples], arithmetic type
  std::vector<int64_t> src_idx_h;
  std::vector<int32_t> src_type_h;
  std::vector<uint8_t> src_samples_h;
  int n_rec = 0;
  int64_t* d_rec_idx = nullptr;
  std::vector<int64_t> rec_idx_h;
  int64_t io_version = 0;

  // run scratch
  int64_t* d_step = nullptr;
  void* d_rec_out = nullptr;
  size_t rec_out_bytes = 0;
  cudaStream_t stream = nullptr;
  pfdtd::GraphCache graph;
  int past_step_direction = 1;

  // frequency-dependent boundaries (dif.cu)
  std::vector<int32_t> dif_flags;   // per material: has a filter
  std::vector<double> dif_coefs;    // per material: b0..b3, a1..a3
  int64_t n_dif = 0;
  int64_t* d_dif_list = nullptr;    // ordered flat indices of DIF nodes
  void* d_dif_tab = nullptr;        // per class: a, b, c, 2G, filter (11 values)
  void* d_dif_state = nullptr;      // per DIF node: s1, s2, s3, previous p

  // update kernel selection and the pipeline error flag
  int kernel_variant = PFDTD_KERNEL_AUTO;
  int tma_tile = -1;         // tile shape of the TMA kernel, -1 automatic (stencil_tma.cu)
  int* d_err = nullptr;
  // bound of each pipeline wait of the TMA update kernels (ns); the drain of
  // loads in flight always keeps its own 2 s bound
  uint64_t wait_ns = 2000000000ull;
  pfdtd::TmaState tma;

  // temporal blocking (stencil_tb.cu): requested depth (0 off) and the
  // geometry check it depends on, cached per class build
  int tb_depth = 0;
  int tb_faces_ok = 0;       // every x/y face node of planes 1..Z-2 is outside
  int tb_shape = -1;         // tile shape index, -1 automatic
  int64_t async_steps = 0;   // steps of the last pfdtd_run_async

  size_t arith_size() const { return precision == PFDTD_F64 ? 8 : 4; }
  void* field(int which) const {
    return (char*)field_base[which] + (size_t)margin * esize;
  }
  void* cur_field() const { return field(cur); }
  void* past_field() const { return field(prev); }
  void swap_fields() { const int t = cur; cur = prev; prev = t; }
  // Device buffers of the domain come from the stream-ordered allocator on
  // its own stream: neither allocation nor release waits for other domains'
  // work (cudaFree would synchronise the whole device).
  cudaError_t alloc(void** p, size_t bytes) { return cudaMallocAsync(p, bytes, stream); }
  void release(void* p) {
    if (p) cudaFreeAsync(p, stream);
  }
};

namespace pfdtd {
// Implemented in stencil.cu
int launch_update(pfdtd_domain* d, const void* cur, void* past, cudaStream_t s);
int launch_io(pfdtd_domain* d, void* cur, void* rec_out, int64_t rec_ld, int64_t inject_end,
              cudaStream_t s, int advance = 1);
int build_classes(pfdtd_domain* d);
// noalloc.cu: puts the no-allocation capture's scratch on `device` (current).
int noalloc_prepare(int device);
// Implemented in stencil_tma.cu
bool tma_supported(const pfdtd_domain* d);
// Implemented in dif.cu
int build_dif(pfdtd_domain* d, const std::vector<uint16_t>& keys,
              const std::vector<uint8_t>& main_tab);
int launch_dif(pfdtd_domain* d, const void* cur, void* past, cudaStream_t s);
int launch_dif_init(pfdtd_domain* d, cudaStream_t s);
int build_iwb_closure(pfdtd_domain* d, const std::vector<uint16_t>& keys);
int launch_iwb_closure(pfdtd_domain* d, const void* cur, void* past, cudaStream_t s);
// Implemented in stencil_tma.cu: whether the next update runs the IWB
// closure pass with the DIF update fused into it
bool iwb_closure_fuses_dif(const pfdtd_domain* d);
// Implemented in setup.cu
int launch_slice_gather(pfdtd_domain* d, int orientation, int64_t slice, float* dp, uint8_t* dq,
                        cudaStream_t s);
int tma_tile_count();
int launch_update_tma(pfdtd_domain* d, const void* cur, void* past, cudaStream_t s);
int launch_iwb_tma(pfdtd_domain* d, const void* cur, void* past, cudaStream_t s);
bool uses_tma(const pfdtd_domain* d);
// Implemented in stencil_tb.cu
int tb_usable(const pfdtd_domain* d, std::string* why);
int launch_tb(pfdtd_domain* d, void* rec_out, int64_t rec_ld, int64_t inject_end, cudaStream_t s);
int check_tb_faces(pfdtd_domain* d);
bool tb_shape_valid(const pfdtd_domain* d, int shape);
}  // namespace pfdtd
