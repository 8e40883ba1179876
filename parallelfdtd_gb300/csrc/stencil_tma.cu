// TMA-pipelined z-marching update (sm_103a).
//
// Same update rules and rounding as k_update_zmarch (stencil.cu), with the
// planes staged through shared memory by the Tensor Memory Accelerator:
//
//  * one producer warp issues 2-D cp.async.bulk.tensor loads into a ring of
//    kStages shared-memory stages; stage k holds the P^n plane z0-1+k of the
//    CTA's tile with a one-row / 16-byte halo, and the P^{n-1} plane and class
//    ids of plane z0+k-2 (the plane computed once P^n plane z+1 has arrived);
//  * the consumer warps compute plane z from stages z-1, z, z+1 and store
//    P^{n+1} straight to global memory; after a step the stage holding plane
//    z-1 is released to the producer through an mbarrier;
//  * the forward update of the 7-point scheme runs as packed f32x2 pairs
//    (two fields of a node, or two adjacent x nodes) with every product an
//    fma(x, y, -0) that the compiler cannot contract, so each element keeps
//    the scalar operation order and rounding;
//  * the tensor maps view each field as rows of the flat array (X wide,
//    Y*Z rows), so the row above the last row of a plane is the first row of
//    the next plane, exactly the flat +-X neighbour the reference reads; the
//    x-halo outside the grid is zero-filled by the TMA, and the two nodes per
//    row that need the flat +-1 wrap (x = 0 and x = X-1) read it from global.
//
// Every mbarrier wait is bounded: on expiry the kernel raises the domain's
// error flag, stops issuing loads, waits (bounded) for the loads already in
// flight and returns.
#include "common.cuh"

#include <cuda.h>

#include <algorithm>
#include <atomic>
#include <cstring>
#include <mutex>
#include <type_traits>

namespace pfdtd {
namespace {

constexpr int kVec = 4;             // consecutive x elements per consumer thread (default)
constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s per wait, far above any real wait


// Per-class coefficients packed for one 16-byte (float) or 32-byte (double)
// shared-memory load per node.
template <typename A> struct alignas(4 * sizeof(A)) PackedCoef { A a, b, c; uint32_t pos; };

__host__ __device__ constexpr int round128(int b) { return (b + 127) / 128 * 128; }

// Tile shape: TX nodes along x (box inner extent TX + 2H <= 256), TY rows,
// NS pipeline stages; MASK: each stage also carries the plane's IWB
// closed-neighbour masks (4 bytes per node); MINB: CTAs per SM the register
// allocation must allow; VEC: consecutive x elements per consumer thread (4,
// or 8 for 16-bit fields: one 16-byte shared-memory load per row vector, and
// the per-thread index and barrier work spread over twice the updates); ZC:
// the 7-point consumer keeps planes z-1 and z in registers along the z-march.
template <typename S, typename C, int TX_, int TY_, int NS_, bool XHALO_ = true, bool MASK_ = false,
          int MINB_ = 1, int VEC_ = kVec, bool ZC_ = false>
struct Layout {
  static constexpr int TX = TX_, TY = TY_, NS = NS_, MINB = MINB_, VEC = VEC_;
  static constexpr bool ZC = ZC_;
  static_assert(VEC == 4 || (VEC == 8 && sizeof(S) == 2), "8-element vectors: 16-bit fields");
  // With XHALO the box carries a 16-byte x halo on both sides; without it the
  // box is exactly TX wide (up to 256) and the threads at the tile's x edges
  // read their outside neighbour from global memory (an L2 hit: the
  // neighbouring tile loads it).
  static constexpr bool XHALO = XHALO_;
  static constexpr int H = XHALO ? 16 / (int)sizeof(S) : 0;
  static constexpr int PW = TX + 2 * H;                      // plane row width with halo
  static constexpr int P_BYTES = PW * (TY + 2) * (int)sizeof(S);
  static constexpr int PP_BYTES = TX * TY * (int)sizeof(S);
  static constexpr int CL_BYTES = TX * TY * (int)sizeof(C);
  static constexpr int P_OFF = 0;
  static constexpr int PP_OFF = round128(P_BYTES);
  static constexpr int CL_OFF = PP_OFF + round128(PP_BYTES);
  static constexpr bool MASK = MASK_;
  static constexpr int MK_BYTES = MASK ? TX * TY * 4 : 0;
  static constexpr int MK_OFF = CL_OFF + round128(CL_BYTES);
  static constexpr int STAGE = MK_OFF + round128(MK_BYTES);
  static constexpr int BAR_OFF = STAGE * NS;
  // full + empty barriers + abort flag, plus 128 B to align the dynamic base
  static constexpr int SMEM = BAR_OFF + 2 * NS * 8 + 16 + 128;
  static constexpr int ROW_THREADS = TX / VEC;                 // threads per tile row
  static constexpr int CONSUMER_WARPS = TX * TY / VEC / 32;
  static constexpr int THREADS = (CONSUMER_WARPS + 1) * 32;
  static_assert(CONSUMER_WARPS * 32 * VEC == TX * TY, "consumer mapping");
  static_assert(PW <= 256 && (PW * (int)sizeof(S)) % 16 == 0, "TMA box row");
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Non-blocking test of the phase with the given parity.
__device__ __forceinline__ bool mbar_test(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}

// The waiting part of mbar_wait.  A bound under 1 ms (a watchdog set short)
// polls without blocking and reads the clock at every poll, since a blocking
// try_wait may itself sleep longer than such a bound; a longer bound blocks
// in try_wait and reads the clock every 256 polls.
__device__ __forceinline__ bool mbar_wait_slow(uint32_t bar, uint32_t parity, uint64_t limit_ns) {
  const uint64_t t0 = global_ns();
  if (limit_ns < 1000000ull) {
    while (!mbar_test(bar, parity))
      if (global_ns() - t0 > limit_ns) return false;
    return true;
  }
  for (uint32_t i = 1;; ++i) {
    if (mbar_try(bar, parity)) return true;
    if ((i & 255) == 0 && global_ns() - t0 > limit_ns) return false;
  }
}

// Wait for the phase with the given parity, for at most limit_ns; false on
// expiry.  The common case in a streaming consumer, a phase already complete,
// costs one non-blocking test.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity,
                                          uint64_t limit_ns = kWaitLimitNs) {
  if (mbar_test(bar, parity)) return true;
  return mbar_wait_slow(bar, parity, limit_ns);
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"((uint64_t)map), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

// N consecutive elements of a shared-memory row (16-byte aligned for a
// 16-byte vector).
template <typename S, int N> struct Vn { S v[N]; };
template <typename S> using V4 = Vn<S, 4>;
__device__ __forceinline__ V4<float> lds4(const float* p) {
  const float4 t = *reinterpret_cast<const float4*>(p);
  return V4<float>{{t.x, t.y, t.z, t.w}};
}
__device__ __forceinline__ V4<double> lds4(const double* p) {
  const double2 a = reinterpret_cast<const double2*>(p)[0];
  const double2 b = reinterpret_cast<const double2*>(p)[1];
  return V4<double>{{a.x, a.y, b.x, b.y}};
}
template <typename H2, typename S>
__device__ __forceinline__ V4<S> lds4_16(const S* p) {
  const uint2 t = *reinterpret_cast<const uint2*>(p);
  H2 a, b;
  memcpy(&a, &t.x, 4);
  memcpy(&b, &t.y, 4);
  return V4<S>{{a.x, a.y, b.x, b.y}};
}
__device__ __forceinline__ V4<__half> lds4(const __half* p) { return lds4_16<__half2>(p); }
__device__ __forceinline__ V4<__nv_bfloat16> lds4(const __nv_bfloat16* p) {
  return lds4_16<__nv_bfloat162>(p);
}
__device__ __forceinline__ V4<float> ldg4(const float* p) {
  const float4 t = __ldg(reinterpret_cast<const float4*>(p));
  return V4<float>{{t.x, t.y, t.z, t.w}};
}
__device__ __forceinline__ V4<double> ldg4(const double* p) {
  const double2 a = __ldg(reinterpret_cast<const double2*>(p));
  const double2 b = __ldg(reinterpret_cast<const double2*>(p) + 1);
  return V4<double>{{a.x, a.y, b.x, b.y}};
}
template <typename H2, typename S>
__device__ __forceinline__ V4<S> ldg4_16(const S* p) {
  const uint2 t = __ldg(reinterpret_cast<const uint2*>(p));
  H2 a, b;
  memcpy(&a, &t.x, 4);
  memcpy(&b, &t.y, 4);
  return V4<S>{{a.x, a.y, b.x, b.y}};
}
__device__ __forceinline__ V4<__half> ldg4(const __half* p) { return ldg4_16<__half2>(p); }
__device__ __forceinline__ V4<__nv_bfloat16> ldg4(const __nv_bfloat16* p) {
  return ldg4_16<__nv_bfloat162>(p);
}

template <typename S>
__device__ __forceinline__ void stg4_16(S* p, const S (&v)[4]) {
  uint16_t u[4];
  memcpy(u, v, 8);
  *reinterpret_cast<uint2*>(p) = make_uint2(u[0] | ((uint32_t)u[1] << 16), u[2] | ((uint32_t)u[3] << 16));
}
__device__ __forceinline__ void stg4(__half* p, const __half (&v)[4]) { stg4_16(p, v); }
__device__ __forceinline__ void stg4(__nv_bfloat16* p, const __nv_bfloat16 (&v)[4]) { stg4_16(p, v); }
__device__ __forceinline__ void stg4(float* p, const float (&v)[4]) {
  *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ void stg4(double* p, const double (&v)[4]) {
  reinterpret_cast<double2*>(p)[0] = make_double2(v[0], v[1]);
  reinterpret_cast<double2*>(p)[1] = make_double2(v[2], v[3]);
}

// Eight consecutive 16-bit elements: one 16-byte load or store.
template <typename H2, typename S>
__device__ __forceinline__ Vn<S, 8> unpack8_16(const uint4 t) {
  H2 a, b, c, e;
  memcpy(&a, &t.x, 4);
  memcpy(&b, &t.y, 4);
  memcpy(&c, &t.z, 4);
  memcpy(&e, &t.w, 4);
  return Vn<S, 8>{{a.x, a.y, b.x, b.y, c.x, c.y, e.x, e.y}};
}
template <typename S> struct Half2Of;
template <> struct Half2Of<__half> { using T = __half2; };
template <> struct Half2Of<__nv_bfloat16> { using T = __nv_bfloat162; };

// Vector loads and stores of N = 4 or 8 elements (8: 16-bit types only).
template <int N, typename S>
__device__ __forceinline__ Vn<S, N> ldsv(const S* p) {
  if constexpr (N == 4) {
    return lds4(p);
  } else {
    static_assert(N == 8 && sizeof(S) == 2, "8-element vectors are 16-bit");
    return unpack8_16<typename Half2Of<S>::T, S>(*reinterpret_cast<const uint4*>(p));
  }
}
template <int N, typename S>
__device__ __forceinline__ Vn<S, N> ldgv(const S* p) {
  if constexpr (N == 4) {
    return ldg4(p);
  } else {
    static_assert(N == 8 && sizeof(S) == 2, "8-element vectors are 16-bit");
    return unpack8_16<typename Half2Of<S>::T, S>(__ldg(reinterpret_cast<const uint4*>(p)));
  }
}
template <int N, typename S>
__device__ __forceinline__ void stgv(S* p, const S (&v)[N]) {
  if constexpr (N == 4) {
    stg4(p, v);
  } else {
    static_assert(N == 8 && sizeof(S) == 2, "8-element vectors are 16-bit");
    uint16_t u[8];
    memcpy(u, v, 16);
    *reinterpret_cast<uint4*>(p) =
        make_uint4(u[0] | ((uint32_t)u[1] << 16), u[2] | ((uint32_t)u[3] << 16),
                   u[4] | ((uint32_t)u[5] << 16), u[6] | ((uint32_t)u[7] << 16));
  }
}

// IWB 27-point update (no counterpart in the reference), a consumer thread's
// 4 consecutive x nodes per plane.  The rows around the nodes come from the
// stage ring: the box's 16-byte x halo and one-row y halo hold every edge and
// corner neighbour.  The scheme's canonical sums (iwb_sums) are built from
// in-plane sums, so a thread computes the raw sums of each new plane z+1 once
// and combines them with those of planes z-1 and z carried in registers.
// With the closed-neighbour masks in the stage (tile shapes 0..5), a node
// with a closed neighbour recomputes its three planes with the closure
// substitution; without them (shapes 6..8, the default), such a node keeps
// P^{n-1} here and the closure pass k_iwb_closure (dif.cu) updates it.
// Closure, order and rounding follow k_update_iwb (stencil.cu) operation for
// operation.
// Canonical index (0..25) of neighbour (dz, dy, dx) = (a-1, b-1, c-1) in the
// closed-neighbour mask: (a, b, c) in row-major order with the centre left out.
__host__ __device__ constexpr int iwb_bit(int a, int b, int c) {
  return a * 9 + b * 3 + c - (a * 9 + b * 3 + c > 13 ? 1 : 0);
}

// In-plane sums of one plane (dz = a-1) for a thread's 4 nodes: the centre
// c0, the 4 face-adjacent in-plane neighbours c1 and the 4 in-plane diagonals
// c2, in the order of iwb_c1 / iwb_c2.  The plane's rows y-1, y, y+1, x-1 ..
// x+4, come from the stage (pl, si) and, at the grid's x edges, from global
// memory at their flat index (g: the flat index of (plane, y, x)), so the wrap
// across rows matches k_update_iwb.  SUBST: neighbours whose bit is set in the
// node's closed mask contribute the node's own value p[e].
template <bool SUBST, int a, typename S, typename Lay>
__device__ __forceinline__ void iwb_plane_sums(const S* pl, int si, const S* __restrict__ P,
                                               int64_t g, int x, int X,
                                               const uint32_t (&mk)[kVec],
                                               const float (&p)[kVec], float (&c0)[kVec],
                                               float (&c1)[kVec], float (&c2)[kVec]) {
  using St = Store<S>;
  constexpr int PW = Lay::PW;
  float w[3][6];
#pragma unroll
  for (int b = 0; b < 3; ++b) {
    const S* row = pl + si + (b - 1) * PW;
    const V4<S> mid = lds4(row);
#pragma unroll
    for (int e = 0; e < 4; ++e) w[b][e + 1] = St::load(mid.v[e]);
    w[b][0] = St::load(row[-1]);
    w[b][5] = St::load(row[kVec]);
  }
  if (x == 0 || x + kVec == X) {  // grid x edge: the flat neighbour wraps to the next row
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      const int64_t gr = g + (int64_t)(b - 1) * X;
      if (x == 0) w[b][0] = St::load(P[gr - 1]);
      if (x + kVec == X) w[b][5] = St::load(P[gr + kVec]);
    }
  }
#pragma unroll
  for (int e = 0; e < kVec; ++e) {
    float q[3][3];
#pragma unroll
    for (int b = 0; b < 3; ++b)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        q[b][c] = w[b][e + c];
        if (SUBST && !(a == 1 && b == 1 && c == 1) && ((mk[e] >> iwb_bit(a, b, c)) & 1u))
          q[b][c] = p[e];
      }
    c0[e] = q[1][1];
    c1[e] = iwb_c1(q);
    c2[e] = iwb_c2(q);
  }
}

// Producer of the stage ring (one thread): stage k receives the P^n plane
// z0-1+k of the tile with its halo and, from k = 2 on, the P^{n-1} plane and
// the class ids of plane z0+k-2.  Every wait is bounded (wait_ns for a free
// stage); on expiry it raises the error flag and the abort flag, then waits
// for the loads it already issued, with the full kWaitLimitNs whatever
// wait_ns is, so that no bulk copy is in flight when the CTA exits.
template <typename Lay>
__device__ __forceinline__ void tma_producer(const CUtensorMap* map_cur,
                                             const CUtensorMap* map_past,
                                             const CUtensorMap* map_cls,
                                             const CUtensorMap* map_mask, unsigned char* smem,
                                             uint32_t bar_full, uint32_t bar_empty,
                                             volatile int* abort_flag, int x0, int y0, int z0,
                                             int Y, int K, int kshift, int* err,
                                             uint64_t wait_ns) {
  constexpr int NS = Lay::NS, H = Lay::H;
  int issued = 0;
  for (int k = 0; k < K; ++k) {
    const int slot = k % NS;
    if (k >= NS) {
      if (!mbar_wait(bar_empty + 8 * slot, (uint32_t)((k / NS - 1) & 1), wait_ns)) {
        atomicExch(err, 1);
        *abort_flag = 1;
        break;
      }
    }
    if (*abort_flag) break;
    unsigned char* st = smem + slot * Lay::STAGE;
    const uint32_t bar = bar_full + 8 * slot;
    const int zp = z0 - 1 + k;
    uint32_t bytes = Lay::P_BYTES;
    if (k >= 2) bytes += Lay::PP_BYTES + (Lay::CL_BYTES >> kshift) + Lay::MK_BYTES;
    mbar_expect_tx(bar, bytes);
    tma_load_2d(smem_u32(st + Lay::P_OFF), map_cur, x0 - H, zp * Y + y0 - 1, bar);
    if (k >= 2) {
      const int zc_ = z0 + k - 2;
      tma_load_2d(smem_u32(st + Lay::PP_OFF), map_past, x0, zc_ * Y + y0, bar);
      tma_load_2d(smem_u32(st + Lay::CL_OFF), map_cls, x0 >> kshift, zc_ * Y + y0, bar);
      if constexpr (Lay::MASK)
        tma_load_2d(smem_u32(st + Lay::MK_OFF), map_mask, x0, zc_ * Y + y0, bar);
    }
    issued = k + 1;
  }
  // Wait (bounded) for every load still in flight before the CTA may exit.
  for (int k = max(0, issued - NS); k < issued; ++k)
    mbar_wait(bar_full + 8 * (k % NS), (uint32_t)((k / NS) & 1));
}

// BATCHED: the field holds K = 1 << kshift interleaved fields per node (K a
// multiple of 4): X and XY count elements, a consumer thread's 4 elements are
// 4 fields of one node, the x neighbours are K elements away and the class
// ids (one per node) come in a box K times narrower.
template <typename S, typename C, int SCHEME, typename Lay, bool BATCHED = false>
__global__ void __launch_bounds__(Lay::THREADS, Lay::MINB)
k_update_tma(const __grid_constant__ CUtensorMap map_cur, const __grid_constant__ CUtensorMap map_past,
             const __grid_constant__ CUtensorMap map_cls,
             const __grid_constant__ CUtensorMap map_mask, const S* __restrict__ P,
             S* __restrict__ Pp, ClassTab<typename Store<S>::A> tab, int X, int Y, int64_t XY,
             int z_last, int zc, typename Store<S>::A l2, int* __restrict__ err, int kshift = 0,
             float* __restrict__ iwb_sw = nullptr, float nzf = -0.0f,
             uint64_t wait_ns = kWaitLimitNs) {
  using A = typename Store<S>::A;
  using R = Rn<A>;
  using St = Store<S>;
  constexpr int kTX = Lay::TX, TY = Lay::TY, H = Lay::H, NS = Lay::NS, PW = Lay::PW;
  constexpr int kThreadsPerRow = Lay::ROW_THREADS;
  constexpr int kConsumerWarps = Lay::CONSUMER_WARPS, kThreads = Lay::THREADS;
  constexpr bool kSmemTab = (sizeof(C) == 1);
  extern __shared__ __align__(128) unsigned char smem_raw[];
  // TMA destinations: 128-byte aligned stage buffers.
  // 128-byte aligned base, derived within the shared window (an integer
  // round trip would make every access through it a generic one)
  unsigned char* smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
  __shared__ PackedCoef<A> stab[kSmemTab ? 256 : 1];

  // A launch after one whose pipeline failed does nothing: the run is
  // already invalid and the host reports it.
  if (*(volatile int*)err) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int x0 = blockIdx.x * kTX, y0 = blockIdx.y * TY;
  const int z0 = 1 + blockIdx.z * zc;
  const int z1 = min(z0 + zc, z_last);
  const int nplanes = z1 - z0;
  const uint32_t bar_full = smem_u32(smem + Lay::BAR_OFF);
  const uint32_t bar_empty = bar_full + NS * 8;
  volatile int* abort_flag = (volatile int*)(smem + Lay::BAR_OFF + 2 * NS * 8);

  if (threadIdx.x == 0) {
    for (int s = 0; s < NS; ++s) {
      mbar_init(bar_full + 8 * s, 1);
      mbar_init(bar_empty + 8 * s, kConsumerWarps);
    }
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (kSmemTab) {
    for (int i = threadIdx.x; i < tab.n; i += kThreads)
      stab[i] = PackedCoef<A>{tab.a[i], tab.b[i], tab.c[i], tab.pos[i]};
  }
  __syncthreads();
  if (nplanes <= 0) return;
  const int K = nplanes + 2;  // loads: planes z0-1 .. z1 of P^n

  if (warp == kConsumerWarps) {
    if (lane == 0)
      tma_producer<Lay>(&map_cur, &map_past, &map_cls, &map_mask, smem, bar_full, bar_empty,
                        abort_flag, x0, y0, z0, Y, K, kshift, err, wait_ns);
    return;
  }

  // ---------------- consumers ----------------
  // Thread -> VEC consecutive x elements of one tile row (TX / VEC threads
  // per row).
  constexpr int VEC = Lay::VEC;
  static_assert(SCHEME != 3 || VEC == kVec, "the IWB consumer works on 4-node vectors");
  const int t = threadIdx.x;
  const int lx = (t % kThreadsPerRow) * VEC;
  const int ly = t / kThreadsPerRow;
  const int x = x0 + lx;
  const int y = y0 + ly;
  const bool active = (x < X) && (y < Y);  // X is a multiple of VEC: all VEC or none
  const int si = (ly + 1) * PW + lx + H;   // centre of the thread's first node
  bool ok = mbar_wait(bar_full, 0, wait_ns) && mbar_wait(bar_full + 8, 0, wait_ns);
  // IWB: raw in-plane sums of planes z-1 (m) and z (c) carried along the
  // z-march; each plane's sums are computed once and used for three planes.
  float cm0[kVec], cm1[kVec], cm2[kVec], cc0[kVec], cc1[kVec], cc2[kVec];
  if constexpr (SCHEME == 3) {
    if (ok && active) {
      const uint32_t no_mask[kVec] = {0u, 0u, 0u, 0u};
      const int64_t g0 = (int64_t)(z0 - 1) * XY + (int64_t)y * X + x;
      iwb_plane_sums<false, 0, S, Lay>((const S*)(smem + Lay::P_OFF), si, P, g0, x, X, no_mask,
                                       cm0, cm0, cm1, cm2);
      iwb_plane_sums<false, 0, S, Lay>((const S*)(smem + Lay::STAGE + Lay::P_OFF), si, P,
                                       g0 + XY, x, X, no_mask, cc0, cc0, cc1, cc2);
    }
  }
  // The 7-point update of the thread's VEC elements of plane z = z0 + j from
  // the values of planes z-1 (fm), z (fc) and z+1 (fn) and the stage of
  // plane z (rows y -+ 1, the x neighbours, P^{n-1}, class ids).
  using Vec = Vn<S, VEC>;
  auto srl_update = [&](int j, const A (&fm)[VEC], const A (&fc)[VEC], const A (&fn)[VEC]) {
      const int sc_ = (j + 1) % NS, sp_ = (j + 2) % NS;
      const S* Pc = (const S*)(smem + sc_ * Lay::STAGE + Lay::P_OFF);
      const S* Pq = (const S*)(smem + sp_ * Lay::STAGE + Lay::PP_OFF);
      const C* Cl = (const C*)(smem + sp_ * Lay::STAGE + Lay::CL_OFF);
      const int z = z0 + j;
      const int64_t idx = (int64_t)z * XY + (int64_t)y * X + x;
      const Vec vym = ldsv<VEC>(Pc + si - PW);
      const Vec vyp = ldsv<VEC>(Pc + si + PW);
      const Vec vpp = ldsv<VEC>(Pq + ly * kTX + lx);
      A left = (A)0, right = (A)0;
      Vec vxm, vxp;
      unsigned cid[VEC];
      if (BATCHED) {
        const int kk = 1 << kshift;
        vxm = lx >= kk ? ldsv<VEC>(Pc + si - kk) : ldgv<VEC>(P + idx - kk);
        // the last node of a row reads its flat-index neighbour (the next
        // row's first node) from global memory, also in a partly filled tile
        vxp = (lx + kk < kTX && x + kk < X) ? ldsv<VEC>(Pc + si + kk) : ldgv<VEC>(P + idx + kk);
        const unsigned c = Cl[ly * (kTX >> kshift) + (lx >> kshift)];
#pragma unroll
        for (int e = 0; e < VEC; ++e) cid[e] = c;
      } else {
        if (x == 0 || (!Lay::XHALO && lx == 0)) left = St::load(P[idx - 1]);
        else left = St::load(Pc[si - 1]);
        if (x + VEC == X || (!Lay::XHALO && lx + VEC == kTX)) right = St::load(P[idx + VEC]);
        else right = St::load(Pc[si + VEC]);
      }
      if (BATCHED) {
      } else if (sizeof(C) * VEC == 4) {
        const uint32_t w = *reinterpret_cast<const uint32_t*>(Cl + ly * kTX + lx);
#pragma unroll
        for (int e = 0; e < 4; ++e) cid[e] = (w >> (8 * e)) & 0xFFu;
      } else if (sizeof(C) * VEC == 8) {
        const uint2 w = *reinterpret_cast<const uint2*>(Cl + ly * kTX + lx);
        const uint32_t ws[2] = {w.x, w.y};
#pragma unroll
        for (int e = 0; e < VEC; ++e)
          cid[e] = sizeof(C) == 1 ? (ws[e >> 2] >> (8 * (e & 3))) & 0xFFu
                                  : (ws[e >> 1] >> (16 * (e & 1))) & 0xFFFFu;
      } else {
        const uint4 w = *reinterpret_cast<const uint4*>(Cl + ly * kTX + lx);
        const uint32_t ws[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
        for (int e = 0; e < VEC; ++e) cid[e] = (ws[e >> 1] >> (16 * (e & 1))) & 0xFFFFu;
      }
      if constexpr ((SCHEME == 0 || SCHEME == 4 || (SCHEME == 1 && sizeof(S) == 4)) &&
                    sizeof(A) == 4) {
        // Forward and (FP32 fields) centred updates of the thread's elements
        // as packed pairs: the same operations and rounding as the scalar
        // loop below, with every product formed as fma(x, y, -0) so that
        // none is contracted.  Batched: the pairs are fields of one node (one
        // class); otherwise adjacent x nodes (a class each).  (The centred
        // update of 16-bit fields stays scalar: packed, its 8-element tiles
        // spill under their register cap.)
        using namespace px;
        constexpr int NP = VEC / 2;
        auto coef = [&](int e) -> PackedCoef<A> {
          if (kSmemTab) return stab[cid[e]];
          return PackedCoef<A>{__ldg(tab.a + cid[e]), __ldg(tab.b + cid[e]),
                               __ldg(tab.c + cid[e]), __ldg(tab.pos + cid[e])};
        };
        const f2 l22 = pk2(l2, l2), nz = pk2(nzf, nzf);
        auto pr = [](const Vec& v, int h) -> f2 {
          return pk2(St::load(v.v[2 * h]), St::load(v.v[2 * h + 1]));
        };
        f2 aa[NP], bb[NP], cc[NP], ee[NP], xm2[NP], xp2[NP];
        uint32_t kp[VEC];  // class position words (centred: boundary directions)
        if constexpr (BATCHED) {
          const PackedCoef<A> k = coef(0);
#pragma unroll
          for (int e = 0; e < VEC; ++e) kp[e] = k.pos;
#pragma unroll
          for (int h = 0; h < NP; ++h) {
            aa[h] = pk2(k.a, k.a);
            bb[h] = pk2(k.b, k.b);
            cc[h] = pk2(k.c, k.c);
            ee[h] = pk2(__uint_as_float(k.pos), __uint_as_float(k.pos));
            xm2[h] = pr(vxm, h);
            xp2[h] = pr(vxp, h);
          }
        } else {
#pragma unroll
          for (int h = 0; h < NP; ++h) {
            const PackedCoef<A> k0 = coef(2 * h), k1 = coef(2 * h + 1);
            kp[2 * h] = k0.pos;
            kp[2 * h + 1] = k1.pos;
            aa[h] = pk2(k0.a, k1.a);
            bb[h] = pk2(k0.b, k1.b);
            cc[h] = pk2(k0.c, k1.c);
            ee[h] = pk2(__uint_as_float(k0.pos), __uint_as_float(k1.pos));
            // node e reads x[e-1] and x[e+1]; x[-1] = left, x[VEC] = right
            xm2[h] = pk2(h == 0 ? left : fc[2 * h - 1], fc[2 * h]);
            xp2[h] = pk2(fc[2 * h + 1], h == NP - 1 ? right : fc[2 * h + 2]);
          }
        }
        S res[VEC];
#pragma unroll
        for (int h = 0; h < NP; ++h) {
          const f2 pc2 = pk2(fc[2 * h], fc[2 * h + 1]);
          const f2 pn2 = pk2(fn[2 * h], fn[2 * h + 1]), pm2 = pk2(fm[2 * h], fm[2 * h + 1]);
          f2 o;
          if constexpr (SCHEME == 1) {
            // centred: s7 = ((((((xm + xp) + ym) + yp) + pn) + pm) + sb6, sb6
            // = (bx dx + by dy) + bz dz with each node's boundary neighbours
            // and directions taken from its class position word
            float bx[2], by[2], bz[2], dx[2], dy[2], dz[2];
#pragma unroll
            for (int q = 0; q < 2; ++q) {
              const int e = 2 * h + q;
              const uint32_t cp = kp[e];
              float xm, xp;
              if constexpr (BATCHED) {
                xm = St::load(vxm.v[e]);
                xp = St::load(vxp.v[e]);
              } else {
                xm = e == 0 ? left : fc[e - 1];
                xp = e == VEC - 1 ? right : fc[e + 1];
              }
              bx[q] = (cp & 0x10u) ? xp : xm;
              by[q] = (cp & 0x20u) ? St::load(vyp.v[e]) : St::load(vym.v[e]);
              bz[q] = (cp & 0x40u) ? fm[e] : fn[e];
              dx[q] = (float)(cp & 1u);
              dy[q] = (float)((cp >> 1) & 1u);
              dz[q] = (float)((cp >> 2) & 1u);
            }
            const f2 sb6 = add2(add2(fma2(pk2(bx[0], bx[1]), pk2(dx[0], dx[1]), nz),
                                     fma2(pk2(by[0], by[1]), pk2(dy[0], dy[1]), nz)),
                                fma2(pk2(bz[0], bz[1]), pk2(dz[0], dz[1]), nz));
            const f2 s7 = add2(add2(add2(add2(add2(add2(xm2[h], xp2[h]), pr(vym, h)), pr(vyp, h)),
                                              pn2),
                                         pm2),
                               sb6);
            o = mul2(aa[h], add2(sub2(fma2(s7, l22, nz), fma2(bb[h], pc2, nz)),
                                 fma2(cc[h], pr(vpp, h), nz)));
          } else {
          const f2 s6 = add2(add2(add2(add2(add2(pn2, pm2), pr(vyp, h)), pr(vym, h)), xp2[h]),
                             xm2[h]);
          if constexpr (SCHEME == 4) {
            // difference form: a (((1+beta) p + (1-beta)(p - pp)) + l2 (S - K p))
            o = mul2(aa[h], add2(add2(fma2(ee[h], pc2, nz), fma2(cc[h], sub2(pc2, pr(vpp, h)), nz)),
                                 fma2(l22, sub2(s6, fma2(bb[h], pc2, nz)), nz)));
          } else {
            o = mul2(aa[h], sub2(add2(fma2(bb[h], pc2, nz), fma2(l22, s6, nz)),
                                 fma2(cc[h], pr(vpp, h), nz)));
          }
          }
          float lo, hi;
          up2(o, lo, hi);
          if constexpr (sizeof(S) == 4) {
            res[2 * h] = lo;
            res[2 * h + 1] = hi;
          } else if constexpr (std::is_same<S, __half>::value) {
            const __half2 t = __floats2half2_rn(lo, hi);  // each half rounded to nearest even
            res[2 * h] = __low2half(t);
            res[2 * h + 1] = __high2half(t);
          } else {
            const __nv_bfloat162 t = __floats2bfloat162_rn(lo, hi);
            res[2 * h] = __low2bfloat16(t);
            res[2 * h + 1] = __high2bfloat16(t);
          }
        }
        stgv<VEC>(Pp + idx, res);
      } else {
      S res[VEC];
#pragma unroll
      for (int e = 0; e < VEC; ++e) {
        const A pc = fc[e];
        A xm, xp;
        if (BATCHED) {
          xm = St::load(vxm.v[e]);
          xp = St::load(vxp.v[e]);
        } else {
          xm = e == 0 ? left : fc[e - 1];
          xp = e == VEC - 1 ? right : fc[e + 1];
        }
        const A ym = St::load(vym.v[e]), yp = St::load(vyp.v[e]);
        const A pm = fm[e], pn = fn[e];
        const A pp = St::load(vpp.v[e]);
        PackedCoef<A> k;
        if (kSmemTab) {
          k = stab[cid[e]];
        } else {
          k = PackedCoef<A>{__ldg(tab.a + cid[e]), __ldg(tab.b + cid[e]), __ldg(tab.c + cid[e]),
                            __ldg(tab.pos + cid[e])};
        }
        A out;
        if (SCHEME == 0 || SCHEME == 4) {
          const A s6 = R::add(R::add(R::add(R::add(R::add(pn, pm), yp), ym), xp), xm);
          if (SCHEME == 4 && sizeof(A) == 4) {
            const A e = (A)__uint_as_float(k.pos);
            out = R::mul(k.a, R::add(R::add(R::mul(e, pc), R::mul(k.c, R::sub(pc, pp))),
                                     R::mul(l2, R::sub(s6, R::mul(k.b, pc)))));
          } else {
            out = R::mul(k.a, R::sub(R::add(R::mul(k.b, pc), R::mul(l2, s6)), R::mul(k.c, pp)));
          }
        } else {
          const uint32_t cp = k.pos;
          const A dx = (A)(cp & 1u), dy = (A)((cp >> 1) & 1u), dz = (A)((cp >> 2) & 1u);
          const A bx = (cp & 0x10u) ? xp : xm;
          const A by = (cp & 0x20u) ? yp : ym;
          const A bz = (cp & 0x40u) ? pm : pn;
          const A sb6 = R::add(R::add(R::mul(bx, dx), R::mul(by, dy)), R::mul(bz, dz));
          const A s7 = R::add(R::add(R::add(R::add(R::add(R::add(xm, xp), ym), yp), pn), pm), sb6);
          out = R::mul(k.a, R::add(R::sub(R::mul(s7, l2), R::mul(k.b, pc)), R::mul(k.c, pp)));
        }
        res[e] = St::store(out);
      }
      stgv<VEC>(Pp + idx, res);
      }
  };
  // One plane's elements of the thread, from stage st.
  auto load_plane = [&](int st, A (&f)[VEC]) {
    const Vec v = ldsv<VEC>((const S*)(smem + st * Lay::STAGE + Lay::P_OFF) + si);
#pragma unroll
    for (int e = 0; e < VEC; ++e) f[e] = St::load(v.v[e]);
  };
  if constexpr (Lay::ZC) {
    // The 7-point update with the thread's values of planes z-1 and z kept
    // in registers from the two planes before: each plane is loaded and
    // converted once, for three updates.  Three planes per trip, the arrays'
    // roles rotating, so that no value is copied.
    static_assert(SCHEME != 3, "the IWB consumer carries its own sums");
    A F0[VEC], F1[VEC], F2[VEC];
    if (ok && active) {
      load_plane(0, F0);
      load_plane(1, F1);
    }
    auto step = [&](int j, A (&fm)[VEC], A (&fc)[VEC], A (&fn)[VEC]) -> bool {
      const int sm = j % NS, sp_ = (j + 2) % NS;
      if (!mbar_wait(bar_full + 8 * sp_, (uint32_t)(((j + 2) / NS) & 1), wait_ns)) return false;
      if (active) {
        load_plane(sp_, fn);
        srl_update(j, fm, fc, fn);
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(bar_empty + 8 * sm);
      return true;
    };
    for (int j = 0; j < nplanes && ok; j += 3) {
      ok = step(j, F0, F1, F2);
      if (!ok || j + 1 >= nplanes) break;
      ok = step(j + 1, F1, F2, F0);
      if (!ok || j + 2 >= nplanes) break;
      ok = step(j + 2, F2, F0, F1);
    }
  }
  for (int j = 0; j < nplanes && ok && !Lay::ZC; ++j) {
    const int sm = j % NS, sc_ = (j + 1) % NS, sp_ = (j + 2) % NS;
    if (!mbar_wait(bar_full + 8 * sp_, (uint32_t)(((j + 2) / NS) & 1), wait_ns)) {
      ok = false;
      break;
    }
    if constexpr (SCHEME == 3) {
      // MASK: the stage carries the closed-neighbour masks and a node next to
      // a closed neighbour is updated here with the closure substitution.
      // Without: every node takes the open sums, and a closure node (class
      // flag bit 30) keeps P^{n-1} for the closure pass (k_iwb_closure) that
      // follows, which also serves the DIF nodes' sw.
      if (active) {
        using R = Rn<float>;
        using St = Store<S>;
        const int ci = ly * kTX + lx;
        const int64_t idx = (int64_t)(z0 + j) * XY + (int64_t)y * X + x;
        const S* Pn = (const S*)(smem + sp_ * Lay::STAGE + Lay::P_OFF);
        const uint32_t no_mask[kVec] = {0u, 0u, 0u, 0u};
        // raw sums of plane z+1
        float n0[kVec], n1[kVec], n2[kVec];
        iwb_plane_sums<false, 2, S, Lay>(Pn, si, P, idx + XY, x, X, no_mask, cc0, n0, n1, n2);
        // the closed-neighbour masks of the thread's 4 nodes (stage of plane z)
        uint4 mk4 = make_uint4(0u, 0u, 0u, 0u);
        if constexpr (Lay::MASK)
          mk4 = *reinterpret_cast<const uint4*>(smem + sp_ * Lay::STAGE + Lay::MK_OFF + 4 * ci);
        float s1[kVec], s2[kVec], s3[kVec];
        if (Lay::MASK && (mk4.x | mk4.y | mk4.z | mk4.w) != 0u) {
          // next to a closed neighbour (walls, obstacle surfaces): the sums of
          // this node's substituted neighbourhood, plane by plane
          const uint32_t mk[kVec] = {mk4.x, mk4.y, mk4.z, mk4.w};
          const S* Pm = (const S*)(smem + sm * Lay::STAGE + Lay::P_OFF);
          const S* Pc = (const S*)(smem + sc_ * Lay::STAGE + Lay::P_OFF);
          float a0[kVec], a1[kVec], a2[kVec], b0[kVec], b1[kVec], b2[kVec];
          iwb_plane_sums<true, 0, S, Lay>(Pm, si, P, idx - XY, x, X, mk, cc0, a0, a1, a2);
          iwb_plane_sums<true, 1, S, Lay>(Pc, si, P, idx, x, X, mk, cc0, b0, b1, b2);
#pragma unroll
          for (int e = 0; e < kVec; ++e) {
            s1[e] = R::add(b1[e], a0[e]);
            s2[e] = R::add(b2[e], a1[e]);
            s3[e] = a2[e];
          }
          iwb_plane_sums<true, 2, S, Lay>(Pn, si, P, idx + XY, x, X, mk, cc0, a0, a1, a2);
#pragma unroll
          for (int e = 0; e < kVec; ++e) {
            s1[e] = R::add(s1[e], a0[e]);
            s2[e] = R::add(s2[e], a1[e]);
            s3[e] = R::add(s3[e], a2[e]);
          }
        } else {
#pragma unroll
          for (int e = 0; e < kVec; ++e) {
            s1[e] = R::add(R::add(cc1[e], cm0[e]), n0[e]);
            s2[e] = R::add(R::add(cc2[e], cm1[e]), n1[e]);
            s3[e] = R::add(cm2[e], n2[e]);
          }
        }
        const C* Cl = (const C*)(smem + sp_ * Lay::STAGE + Lay::CL_OFF);
        unsigned cid[kVec];
        if (sizeof(C) == 1) {
          const uint32_t w = *reinterpret_cast<const uint32_t*>(Cl + ci);
#pragma unroll
          for (int e = 0; e < kVec; ++e) cid[e] = (w >> (8 * e)) & 0xFFu;
        } else {
          const uint2 w = *reinterpret_cast<const uint2*>(Cl + ci);
          cid[0] = w.x & 0xFFFFu; cid[1] = w.x >> 16; cid[2] = w.y & 0xFFFFu; cid[3] = w.y >> 16;
        }
        const V4<S> vpp = lds4((const S*)(smem + sp_ * Lay::STAGE + Lay::PP_OFF) + ci);
        S res[kVec];
#pragma unroll
        for (int e = 0; e < kVec; ++e) {
          PackedCoef<A> k;
          if (kSmemTab) k = stab[cid[e]];
          else
            k = PackedCoef<A>{__ldg(tab.a + cid[e]), __ldg(tab.b + cid[e]),
                              __ldg(tab.c + cid[e]), __ldg(tab.pos + cid[e])};
          const float sw = R::mul((float)l2, R::add(R::add(R::mul(s1[e], 0.25f),
                                                           R::mul(s2[e], 0.125f)),
                                                    R::mul(s3[e], 0.0625f)));
          if (Lay::MASK && iwb_sw != nullptr && (k.pos >> 31)) iwb_sw[idx + e] = sw;  // a DIF node
          const float out = R::mul(k.a, R::sub(R::add(sw, R::mul(k.b, cc0[e])),
                                               R::mul(k.c, St::load(vpp.v[e]))));
          // a closure node (maskless tiles) keeps P^{n-1} for the closure
          // pass; a node outside the room (a = 0) holds +0
          res[e] = (!Lay::MASK && ((k.pos >> 30) & 1u)) ? vpp.v[e]
                                                         : St::store(k.a == 0.f ? 0.f : out);
        }
        stg4(Pp + idx, res);
#pragma unroll
        for (int e = 0; e < kVec; ++e) {
          cm0[e] = cc0[e]; cm1[e] = cc1[e]; cm2[e] = cc2[e];
          cc0[e] = n0[e]; cc1[e] = n1[e]; cc2[e] = n2[e];
        }
      }
    } else if (active) {
      A fm[VEC], fc[VEC], fn[VEC];
      load_plane(sm, fm);
      load_plane(sc_, fc);
      load_plane(sp_, fn);
      srl_update(j, fm, fc, fn);
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(bar_empty + 8 * sm);
  }
  if (!ok) {
    atomicExch(err, 1);
    *abort_flag = 1;
  }
}

template <typename S> struct TmaType;
template <> struct TmaType<float> { static constexpr CUtensorMapDataType value = CU_TENSOR_MAP_DATA_TYPE_FLOAT32; };
template <> struct TmaType<double> { static constexpr CUtensorMapDataType value = CU_TENSOR_MAP_DATA_TYPE_FLOAT64; };
template <> struct TmaType<__half> { static constexpr CUtensorMapDataType value = CU_TENSOR_MAP_DATA_TYPE_FLOAT16; };
template <> struct TmaType<__nv_bfloat16> { static constexpr CUtensorMapDataType value = CU_TENSOR_MAP_DATA_TYPE_BFLOAT16; };

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// Looked up once per process (a function-local static: thread-safe, since
// domains may be set up from several threads at once).
EncodeTiledFn encode_fn() {
  static const EncodeTiledFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      return (EncodeTiledFn)p;
    cudaGetLastError();
    return (EncodeTiledFn) nullptr;
  }();
  return fn;
}

// 2-D map over the flat array viewed as X-wide rows (Y*Z rows), each row
// `pitch` elements apart (X when 0).
bool make_map(CUtensorMap* m, CUtensorMapDataType dt, size_t esize, void* base, int64_t X,
              int64_t rows, int box_x, int box_y, int64_t pitch = 0) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return false;
  cuuint64_t dims[2] = {(cuuint64_t)X, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)((pitch > 0 ? pitch : X) * (int64_t)esize)};
  cuuint32_t box[2] = {(cuuint32_t)box_x, (cuuint32_t)box_y};
  cuuint32_t es[2] = {1, 1};
  return fn(m, dt, 2, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <typename S, typename C, int SCHEME, typename Lay, bool BATCHED = false>
int launch_tma_t(pfdtd_domain* d, const void* cur, void* past, cudaStream_t s) {
  using A = typename Store<S>::A;
  constexpr int kTX = Lay::TX;
  const int64_t XE = d->X * d->K;  // row length in elements
  const int64_t nz = d->Z - 2;
  if (nz <= 0) return PFDTD_OK;
  TmaState& ts = d->tma;
  int cur_i = -1, past_i = -1;
  for (int f = 0; f < 4; ++f) {
    if (d->field_base[f] && cur == d->field(f)) cur_i = f;
    if (d->field_base[f] && past == d->field(f)) past_i = f;
  }
  if (cur_i < 0 || past_i < 0) return fail(PFDTD_ERR_ARG, "update fields are not domain buffers");
  // class ids: the padded copy when their rows are not 16-byte aligned
  void* cls_base = d->cls_pitch > 0 ? d->d_cls_tma : d->d_cls;
  const int64_t key[7] = {(int64_t)(intptr_t)cls_base, d->cls_bytes, d->precision * 100 + d->K,
                          (int64_t)Lay::TX * 10000 + Lay::TY * 10 + (Lay::XHALO ? 1 : 0),
                          (int64_t)(intptr_t)d->field_base[2],
                          Lay::MASK ? (int64_t)(intptr_t)d->d_iwb_mask : 0, d->cls_pitch};
  if (!ts.ready || std::memcmp(key, ts.key, sizeof(key)) != 0) {
    const CUtensorMapDataType dt = TmaType<S>::value;
    const CUtensorMapDataType ct =
        sizeof(C) == 1 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_UINT16;
    const int64_t rows = d->Y * d->Z;
    bool ok = true;
    for (int f = 0; f < 4; ++f) {
      if (!d->field_base[f]) continue;
      ok = ok && make_map(&ts.halo[f], dt, sizeof(S), d->field(f), XE, rows, Lay::PW, Lay::TY + 2);
      ok = ok && make_map(&ts.tile[f], dt, sizeof(S), d->field(f), XE, rows, kTX, Lay::TY);
    }
    ok = ok && make_map(&ts.cls, ct, sizeof(C), cls_base, d->X, rows, kTX >> d->kshift, Lay::TY,
                        d->cls_pitch);
    if (Lay::MASK) {
      if (!d->d_iwb_mask) return fail(PFDTD_ERR_STATE, "IWB masks not built");
      ok = ok && make_map(&ts.mask, CU_TENSOR_MAP_DATA_TYPE_UINT32, 4, d->d_iwb_mask, d->X, rows,
                          kTX, Lay::TY);
    }
    if (!ok) return fail(PFDTD_ERR_UNSUPPORTED, "tensor map encoding failed");
    std::memcpy(ts.key, key, sizeof(key));
    ts.ready = true;
  }
  // the shared-memory opt-in, once per instantiation and device
  // (IWB: and its resident CTAs per SM, which registers limit as well);
  // several threads may launch at once (a request loop sets up its domains
  // concurrently), so the first one does it under a lock
  static std::atomic<bool> attr_done[64];
  static std::atomic<int> occupancy[64];
  static std::mutex attr_mu;
  if (d->device >= 64) return fail(PFDTD_ERR_UNSUPPORTED, "device index above 63");
  if (!attr_done[d->device].load(std::memory_order_acquire)) {
    std::lock_guard<std::mutex> lock(attr_mu);
    if (!attr_done[d->device].load(std::memory_order_relaxed)) {
      PFDTD_CK(cudaFuncSetAttribute(k_update_tma<S, C, SCHEME, Lay, BATCHED>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, Lay::SMEM));
      int occ = 0;
      if (SCHEME == 3)
        PFDTD_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &occ, k_update_tma<S, C, SCHEME, Lay, BATCHED>, Lay::THREADS, Lay::SMEM));
      occupancy[d->device].store(occ, std::memory_order_relaxed);
      attr_done[d->device].store(true, std::memory_order_release);
    }
  }
  const int occ = occupancy[d->device].load(std::memory_order_relaxed);
  const int gx = (int)((XE + kTX - 1) / kTX);
  const int gy = (int)((d->Y + Lay::TY - 1) / Lay::TY);
  // z-chunks: several per tile so that the grid fills the machine in whole
  // waves of (SMs x resident CTAs), each chunk at least 16 planes long.
  const int64_t per_sm =
      occ > 0
          ? occ
          : std::max<int64_t>(1, (228 * 1024) / (Lay::SMEM + 1024 + 8192));
  const int64_t resident = (int64_t)d->sm_count * per_sm;
  const int64_t tiles = (int64_t)gx * gy;
  int64_t best_c = 1;
  double best = 1e30;
  for (int64_t c = 1; c <= std::max<int64_t>(1, nz / 16); ++c) {
    const int64_t ctas = tiles * c;
    const int64_t waves = (ctas + resident - 1) / resident;
    const double eff = (double)ctas / (double)(waves * resident);  // wave fill
    const double zlen = (double)nz / (double)c;
    const double cost = 1.0 / eff * (1.0 + 2.0 / zlen);
    if (cost < best - 1e-9) { best = cost; best_c = c; }
  }
  const int64_t zc = (nz + best_c - 1) / best_c;
  const int gz = (int)((nz + zc - 1) / zc);
  const size_t as = sizeof(A);
  const char* tb = (const char*)d->d_ctab;
  ClassTab<A> tab{(const A*)tb, (const A*)(tb + as * d->n_classes),
                  (const A*)(tb + 2 * as * d->n_classes),
                  (const uint32_t*)(tb + 3 * as * d->n_classes), d->n_classes};
  k_update_tma<S, C, SCHEME, Lay, BATCHED><<<dim3(gx, gy, gz), Lay::THREADS, Lay::SMEM, s>>>(
      ts.halo[cur_i], ts.tile[past_i], ts.cls, Lay::MASK ? ts.mask : ts.cls, (const S*)cur,
      (S*)past, tab, (int)XE, (int)d->Y, d->XY * d->K, (int)(d->Z - 1), (int)zc,
      (A)d->params[1], d->d_err, d->kshift, SCHEME == 3 ? d->d_iwb_sw : nullptr, -0.0f,
      d->wait_ns);
  count_launch();
  PFDTD_CK(cudaGetLastError());
  return PFDTD_OK;
}

template <typename S, typename Lay8, typename Lay16>
int launch_tma_batched(pfdtd_domain* d, const void* cur, void* past, cudaStream_t s) {
  const bool centred = (d->class_scheme == PFDTD_SRL);
  if constexpr (std::is_same<S, float>::value) {  // the difference form (FP32 fields)
    if (d->class_form == PFDTD_FORM_DIFFERENCE)
      return d->cls_bytes == 1 ? launch_tma_t<S, uint8_t, 4, Lay8, true>(d, cur, past, s)
                               : launch_tma_t<S, uint16_t, 4, Lay16, true>(d, cur, past, s);
  }
  if (d->cls_bytes == 1)
    return centred ? launch_tma_t<S, uint8_t, 1, Lay8, true>(d, cur, past, s)
                   : launch_tma_t<S, uint8_t, 0, Lay8, true>(d, cur, past, s);
  return centred ? launch_tma_t<S, uint16_t, 1, Lay16, true>(d, cur, past, s)
                 : launch_tma_t<S, uint16_t, 0, Lay16, true>(d, cur, past, s);
}

template <typename S, typename Lay8, typename Lay16>
int launch_tma_l(pfdtd_domain* d, const void* cur, void* past, cudaStream_t s) {
  const bool centred = (d->class_scheme == PFDTD_SRL);
  if constexpr (std::is_same<S, float>::value) {  // the difference form (FP32 fields)
    if (d->class_form == PFDTD_FORM_DIFFERENCE)
      return d->cls_bytes == 1 ? launch_tma_t<S, uint8_t, 4, Lay8>(d, cur, past, s)
                               : launch_tma_t<S, uint16_t, 4, Lay16>(d, cur, past, s);
  }
  if (d->cls_bytes == 1)
    return centred ? launch_tma_t<S, uint8_t, 1, Lay8>(d, cur, past, s)
                   : launch_tma_t<S, uint8_t, 0, Lay8>(d, cur, past, s);
  return centred ? launch_tma_t<S, uint16_t, 1, Lay16>(d, cur, past, s)
                 : launch_tma_t<S, uint16_t, 0, Lay16>(d, cur, past, s);
}

// Tile shapes built for FP32 (index = tile id): TX x TY nodes, stages, x halo
// in the TMA box or read from global at the tile's x edges.
#define PFDTD_F32_TILES(X)                                                             \
  X(0, 64, 16, 8, true) X(1, 128, 8, 8, true) X(2, 32, 32, 8, true) X(3, 128, 16, 6, true)   \
  X(4, 128, 4, 12, true) X(5, 128, 8, 8, false) X(6, 256, 4, 8, false)                        \
  X(7, 256, 8, 6, false) X(8, 256, 2, 16, false)

template <typename S>
int launch_tma_s(pfdtd_domain* d, const void* cur, void* past, cudaStream_t s);

// Whether tiles w nodes wide cover a row with at most 1/16 of the tiles'
// width left empty in the row's last, partly filled tile.
bool tile_fits(const pfdtd_domain* d, int64_t w) {
  const int64_t covered = (d->X + w - 1) / w * w;
  return (covered - d->X) * 16 <= covered;
}

// Automatic tile: the widest x extent (256, 128 or 64 nodes) whose partly
// filled last tile wastes little, so that TMA rows are as long as possible
// (measured on the 512 x 384 x 256 room: 256 x 4 streams at 98% of the copy
// bandwidth, 64 x 16 with an in-box halo at 74%; on 500 x 384 x 256, 64 x 16
// 378 G node-updates/s).
int auto_tile(const pfdtd_domain* d) {
  if (tile_fits(d, 256)) return 6;
  if (tile_fits(d, 128)) return 5;
  return 0;
}

template <>
int launch_tma_s<float>(pfdtd_domain* d, const void* cur, void* past, cudaStream_t s) {
  if (d->K > 1)  // 256 elements (256/K nodes) x 4 rows
    return launch_tma_batched<float, Layout<float, uint8_t, 256, 4, 8, false>,
                              Layout<float, uint16_t, 256, 4, 8, false>>(d, cur, past, s);
  // ids 9 and 10 name IWB-only shapes: the 7-point update takes its
  // automatic tile for them
  switch (d->tma_tile < 0 || d->tma_tile > 8 ? auto_tile(d) : d->tma_tile) {
#define PFDTD_CASE(id, tx, ty, ns, xh)                                                    \
  case id:                                                                                \
    return launch_tma_l<float, Layout<float, uint8_t, tx, ty, ns, xh>,                     \
                        Layout<float, uint16_t, tx, ty, ns, xh>>(d, cur, past, s);
    PFDTD_F32_TILES(PFDTD_CASE)
#undef PFDTD_CASE
  }
  return fail(PFDTD_ERR_ARG, "unknown TMA tile shape");
}

// 16-bit storage tiles (id, TX, TY, stages, x halo in the box, CTAs per SM,
// elements per thread): 0 64x16 (halo in box), 1 128x8, 2 256x8, 3 256x4, with
// 4 elements per thread; 4 256x8, 5 256x8 (6 stages, three CTAs per SM),
// 6 256x4 (four CTAs), 7 128x8 with 8 elements per thread; 8 256x8,
// 9 256x4 (four CTAs) and 10 128x8 with 8 elements per thread and planes
// z-1, z carried in registers.  Measured on the 512 x 384 x 256 room, FP16
// (node-updates/s): 2 655 G, 4 753 G, 5 720 G, 6 677 G, 7 699 G, 8 808 G,
// 9 703 G; BF16: 2 626 G, 4 744 G, 8 777 G, 9 683 G.
#define PFDTD_F16_TILES(X)                                                                    \
  X(0, 64, 16, 8, true, 2, 4, false) X(1, 128, 8, 8, false, 2, 4, false)                       \
  X(2, 256, 8, 8, false, 2, 4, false) X(3, 256, 4, 8, false, 2, 4, false)                      \
  X(4, 256, 8, 8, false, 2, 8, false) X(5, 256, 8, 6, false, 3, 8, false)                      \
  X(6, 256, 4, 8, false, 4, 8, false) X(7, 128, 8, 8, false, 2, 8, false)                      \
  X(8, 256, 8, 8, false, 2, 8, true) X(9, 256, 4, 8, false, 4, 8, true)                       \
  X(10, 128, 8, 8, false, 2, 8, true)

int auto_tile16(const pfdtd_domain* d) {
  if (tile_fits(d, 256)) return 8;
  if (tile_fits(d, 128)) return 10;
  return 0;
}

template <typename S>
int launch_tma_16(pfdtd_domain* d, const void* cur, void* past, cudaStream_t s) {
  // Two CTAs per SM (registers capped to allow it): a 256 x 8 tile of 16-bit
  // fields holds half the bytes of the FP32 tile, and one CTA per SM leaves
  // too few loads in flight to stream at HBM speed.
  if (d->K > 1) {
    // batched tiles: 0 (K not a multiple of 8: the default) 256 x 8
    // elements, 8 stages, two CTAs per SM; 1 = 256 x 4, 8 stages, four CTAs;
    // 2 = 256 x 8, 6 stages, two CTAs; with 8 elements (fields of one node)
    // per thread, for K a multiple of 8: 3 = 256 x 8, 8 stages, two CTAs;
    // 4 = 256 x 4, 8 stages, four CTAs; 5 (the default) = as 3 with planes
    // z-1, z carried in registers; 6 = as 4 with planes carried.  Measured on
    // the 384 x 320 x 256 room, K = 16, FP16 (field-updates/s): 0 710 G,
    // 3 896 G, 4 900 G, 5 928 G, 6 934 G (BF16: 5 908 G, 6 913 G).
    const int tile = d->tma_tile < 0 || d->tma_tile > 6 ? 5 : d->tma_tile;
    if (d->K % 8 == 0 && tile == 6)
      return launch_tma_batched<S, Layout<S, uint8_t, 256, 4, 8, false, false, 4, 8, true>,
                                Layout<S, uint16_t, 256, 4, 8, false, false, 4, 8, true>>(d, cur, past, s);
    if (d->K % 8 == 0 && tile == 5)
      return launch_tma_batched<S, Layout<S, uint8_t, 256, 8, 8, false, false, 2, 8, true>,
                                Layout<S, uint16_t, 256, 8, 8, false, false, 2, 8, true>>(d, cur, past, s);
    if (d->K % 8 == 0 && tile == 3)
      return launch_tma_batched<S, Layout<S, uint8_t, 256, 8, 8, false, false, 2, 8>,
                                Layout<S, uint16_t, 256, 8, 8, false, false, 2, 8>>(d, cur, past, s);
    if (d->K % 8 == 0 && tile == 4)
      return launch_tma_batched<S, Layout<S, uint8_t, 256, 4, 8, false, false, 4, 8>,
                                Layout<S, uint16_t, 256, 4, 8, false, false, 4, 8>>(d, cur, past, s);
    if (tile == 1)
      return launch_tma_batched<S, Layout<S, uint8_t, 256, 4, 8, false, false, 4>,
                                Layout<S, uint16_t, 256, 4, 8, false, false, 4>>(d, cur, past, s);
    if (tile == 2)
      return launch_tma_batched<S, Layout<S, uint8_t, 256, 8, 6, false, false, 2>,
                                Layout<S, uint16_t, 256, 8, 6, false, false, 2>>(d, cur, past, s);
    return launch_tma_batched<S, Layout<S, uint8_t, 256, 8, 8, false, false, 2>,
                              Layout<S, uint16_t, 256, 8, 8, false, false, 2>>(d, cur, past, s);
  }
  switch (d->tma_tile < 0 || d->tma_tile > 10 ? auto_tile16(d) : d->tma_tile) {
#define PFDTD_CASE16(id, tx, ty, ns, xh, minb, vec, zc)                                   \
  case id:                                                                                \
    return launch_tma_l<S, Layout<S, uint8_t, tx, ty, ns, xh, false, minb, vec, zc>,       \
                        Layout<S, uint16_t, tx, ty, ns, xh, false, minb, vec, zc>>(d, cur, past, s);
    PFDTD_F16_TILES(PFDTD_CASE16)
#undef PFDTD_CASE16
  }
  return fail(PFDTD_ERR_ARG, "unknown TMA tile shape for 16-bit fields (0..10)");
}

template <>
int launch_tma_s<__half>(pfdtd_domain* d, const void* cur, void* past, cudaStream_t s) {
  return launch_tma_16<__half>(d, cur, past, s);
}

template <>
int launch_tma_s<__nv_bfloat16>(pfdtd_domain* d, const void* cur, void* past, cudaStream_t s) {
  return launch_tma_16<__nv_bfloat16>(d, cur, past, s);
}

template <>
int launch_tma_s<double>(pfdtd_domain* d, const void* cur, void* past, cudaStream_t s) {
  if (d->K > 1)
    return launch_tma_batched<double, Layout<double, uint8_t, 128, 4, 6, false>,
                              Layout<double, uint16_t, 128, 4, 6, false>>(d, cur, past, s);
  return launch_tma_l<double, Layout<double, uint8_t, 64, 8, 6>, Layout<double, uint16_t, 64, 8, 6>>(
      d, cur, past, s);
}

// IWB on the stage ring: FP32, FP16 and BF16 storage, one field per node,
// tiles with the x halo in the box.  Shapes (d->tma_tile for IWB, -1 auto):
// with the closed-neighbour masks in every stage and the closure computed in
// the kernel: 0 = 64 x 16 and 1 = 128 x 8 (288 threads, 8 stages), 2 = 128 x
// 4 (5 stages), and 160-thread 64 x 8 tiles: 3 = 8 stages, three CTAs per
// SM, 4 = 6 stages, four CTAs, 5 = 5 stages, five CTAs (registers capped to
// fit).  Without masks, every node takes the open sums in the kernel and the
// closure nodes are updated by the sparse closure pass after it: 6 = 128 x 8
// (288 threads), 6 stages, three CTAs per SM (the default), 7 = 128 x 4 (160
// threads), 8 stages, four CTAs, 8 = 128 x 8, 8 stages, two CTAs, 9 = 128 x 8,
// 5 stages, four CTAs, 10 = 128 x 4, 6 stages, six CTAs.  With masks a warp that holds one closure
// node runs the substitution for all its lanes, and in the tiles along the x
// walls that is every warp; the split keeps the streaming kernel on the open
// path and leaves the ~2 % closure nodes to the gather pass.  Measured on the
// 512 x 384 x 256 room, FP32 with third-order DIF walls (C3): shape 3 208 G,
// 6 267 G, 7 249 G, 8 249 G node-updates/s (64 x 8 without masks, four CTAs:
// 235 G).
template <typename S, typename C, int TX, int TY, int NS, int MINB = 1, bool MASK = true>
int launch_iwb_l(pfdtd_domain* d, const void* cur, void* past, cudaStream_t s) {
  if constexpr (MASK) {
    return launch_tma_t<S, C, 3, Layout<S, C, TX, TY, NS, true, true, MINB>>(d, cur, past, s);
  } else {
    if (!d->iwb_closure_ready) return fail(PFDTD_ERR_STATE, "IWB closure list not built");
    if (int rc = launch_tma_t<S, C, 3, Layout<S, C, TX, TY, NS, true, false, MINB>>(d, cur, past, s))
      return rc;
    return launch_iwb_closure(d, cur, past, s);
  }
}

template <typename S, typename C>
int launch_iwb_c(pfdtd_domain* d, const void* cur, void* past, cudaStream_t s) {
  int tile = d->tma_tile;
  if (tile < 0 || tile > 10) tile = 6;
  switch (tile) {
    case 9: return launch_iwb_l<S, C, 128, 8, 5, 4, false>(d, cur, past, s);
    case 10: return launch_iwb_l<S, C, 128, 4, 6, 6, false>(d, cur, past, s);
    case 0: return launch_iwb_l<S, C, 64, 16, 8>(d, cur, past, s);
    case 1: return launch_iwb_l<S, C, 128, 8, 8>(d, cur, past, s);
    case 2: return launch_iwb_l<S, C, 128, 4, 5>(d, cur, past, s);
    case 3: return launch_iwb_l<S, C, 64, 8, 8, 3>(d, cur, past, s);
    case 4: return launch_iwb_l<S, C, 64, 8, 6, 4>(d, cur, past, s);
    case 5: return launch_iwb_l<S, C, 64, 8, 5, 5>(d, cur, past, s);
    case 7: return launch_iwb_l<S, C, 128, 4, 8, 4, false>(d, cur, past, s);
    case 8: return launch_iwb_l<S, C, 128, 8, 8, 2, false>(d, cur, past, s);
    default: return launch_iwb_l<S, C, 128, 8, 6, 3, false>(d, cur, past, s);
  }
}

template <typename S>
int launch_iwb_tma_s(pfdtd_domain* d, const void* cur, void* past, cudaStream_t s) {
  return d->cls_bytes == 1 ? launch_iwb_c<S, uint8_t>(d, cur, past, s)
                           : launch_iwb_c<S, uint16_t>(d, cur, past, s);
}

}  // namespace

int launch_iwb_tma(pfdtd_domain* d, const void* cur, void* past, cudaStream_t s) {
  switch (d->precision) {
    case PFDTD_F32: return launch_iwb_tma_s<float>(d, cur, past, s);
    case PFDTD_F16: return launch_iwb_tma_s<__half>(d, cur, past, s);
    case PFDTD_BF16: return launch_iwb_tma_s<__nv_bfloat16>(d, cur, past, s);
  }
  return fail(PFDTD_ERR_UNSUPPORTED, "IWB on the TMA path needs FP32, FP16 or BF16 fields");
}

bool iwb_closure_fuses_dif(const pfdtd_domain* d) {
  // tile shapes 0..5 run the closure inside the streaming kernel
  return d->class_scheme == PFDTD_IWB && d->n_dif > 0 && d->iwb_closure_ready &&
         d->d_iwb_closure_dif != nullptr && uses_tma(d) && !(d->tma_tile >= 0 && d->tma_tile <= 5);
}

// Whether the next update runs a TMA kernel (7-point or IWB).
bool uses_tma(const pfdtd_domain* d) {
  if (d->kernel_variant == PFDTD_KERNEL_ZMARCH || !tma_supported(d)) return false;
  if (d->class_scheme == PFDTD_IWB) return d->K == 1 && d->precision != PFDTD_F64;
  return true;
}

// The TMA path needs 16-byte aligned field rows (the class ids are padded).
int tma_tile_count() { return 11; }

bool tma_supported(const pfdtd_domain* d) {
  // Batched fields: a thread's 4 elements must be 4 fields of one node, and
  // the class box (tile elements / K, at least 16 bytes) must stay valid.
  // A row that ends inside a tile is handled (TMA fills past the row end with
  // zeros, stores stop at the row end, and the row's last node reads its
  // flat-index neighbour from global memory).
  if (d->K > 1) {
    const int tile = d->precision == PFDTD_F64 ? 128 : 256;
    if (d->K % 4 != 0 || (tile / d->K) * d->cls_bytes < 16) return false;
  }
  // (rows of class ids that are not 16-byte aligned are read from a padded
  // copy, d_cls_tma)
  if ((d->X * (int64_t)d->esize) % 16 != 0) return false;
  if (d->Y * d->Z >= ((int64_t)1 << 31)) return false;
  return encode_fn() != nullptr;
}

int launch_update_tma(pfdtd_domain* d, const void* cur, void* past, cudaStream_t s) {
  switch (d->precision) {
    case PFDTD_F32: return launch_tma_s<float>(d, cur, past, s);
    case PFDTD_F64: return launch_tma_s<double>(d, cur, past, s);
    case PFDTD_F16: return launch_tma_s<__half>(d, cur, past, s);
    case PFDTD_BF16: return launch_tma_s<__nv_bfloat16>(d, cur, past, s);
  }
  return fail(PFDTD_ERR_UNSUPPORTED, "unknown precision");
}

}  // namespace pfdtd
