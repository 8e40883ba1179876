// Temporally blocked leapfrog update kernel and its launcher (templates);
// instantiated per storage type by stencil_tb_f32.cu, stencil_tb_f16.cu and
// stencil_tb_bf16.cu, and dispatched from stencil_tb.cu.
//
// The plain kernels read P^n and P^{n-1} and write P^{n+1} once per step,
// so every step moves the whole field through HBM.  This kernel advances T
// steps per pass over the grid:
//
//  * a CTA owns a core tile of (x, y) nodes and a range of z planes, and
//    computes on an extended tile with a halo of T nodes (4 nodes for the
//    4-node vectors of an unbatched field) so that level t = 1..T of the
//    step sequence is exact on a region that shrinks by one node per level;
//  * it marches z: iteration zl loads P^n plane zl, P^{n-1} plane zl-1 and
//    the class ids of plane zl-1 with cp.async into a ring of kNS stages,
//    then computes level t at plane zl-t for t = 1..T.  Each thread keeps
//    its own column's last three planes of every level in registers; the
//    x/y neighbours come from one shared-memory plane per level (double
//    buffered), so an iteration needs one __syncthreads();
//  * level T-1 and level T of the core are written to two further buffers
//    (the P^{n+T-1} and P^{n+T} of the step sequence), never over the input,
//    because neighbouring CTAs still read the input halo;
//  * the steps in between keep the plain path's per-step order: the value
//    of level t at a receiver is recorded as the receivers of step n+t (before
//    injection), then the sources of step n+t are injected into level t in
//    source order (ParallelFDTD src/kernels/kernels3d.cu:93-104, :164-173).
//    The io kernel before the launch has already recorded level 0 and
//    injected step n, and advanced the step counter by T.
//
// Arithmetic, association order and rounding of every node update are those
// of k_update_zmarch (stencil.cu): levels are rounded to the storage type
// before they are used, so the fields equal T plain steps.  Two conditions
// make the tile halo exact, and the host only enables the kernel when they
// hold: every node on the x and y faces of planes 1..Z-2 is outside
// (position bit 7 clear, so its update is 0 times a finite value whatever
// neighbour the reference's flat-index wrap would read), and no source or
// receiver lies on plane 0 or Z-1 (those planes are never updated, so their
// level t equals level t-2).  A zero produced on a face can differ from the
// plain path's in sign only; every non-zero value is identical.
//
// There are no spin waits: the only synchronisation is __syncthreads() and
// cp.async.wait_group.
#pragma once
#include "common.cuh"

#include <algorithm>
#include <cstring>
#include <mutex>
#include <type_traits>

namespace pfdtd {
namespace tb {

constexpr int kNS = 4;        // cp.async stages (loads run two iterations ahead)
constexpr int kMaxSrc = 64;   // sources per domain the kernel's lists can hold
constexpr int kMaxRec = 256;  // receivers per domain

__host__ __device__ constexpr int r16(int b) { return (b + 15) / 16 * 16; }

// Tile shape.  VW vectors per tile row, TR thread rows of R tile rows each
// (HR = TR * R rows), one 4-element vector per thread and tile row.
// Unbatched: a vector is 4 consecutive x nodes; batched: the 4 fields
// f0..f0+3 of one node (the K fields are split over CTAs in groups of 4,
// which keeps the x halo at T nodes).
template <typename S, int VW_, int TR_, int R_, int T_, bool BATCHED_, int MINB_ = 1>
struct TbShape {
  static constexpr int VW = VW_, TR = TR_, R = R_, T = T_, MINB = MINB_;
  static constexpr int HR = TR * R;
  static constexpr bool BATCHED = BATCHED_;
  static constexpr int THREADS = VW * TR;
  static constexpr int RE = VW * 4;                  // elements per tile row
  static constexpr int NODES = BATCHED ? VW : 4 * VW;  // nodes per tile row
  static constexpr int XH = BATCHED ? T : 4;          // halo nodes left and right
  static constexpr int CXN = NODES - 2 * XH;          // core nodes per row
  static constexpr int CYR = HR - 2 * T;              // core rows
  // class bytes of a tile row: unbatched 4 per vector; batched the row's
  // bytes from the 4-byte boundary at or below the first node
  static constexpr int CL_ROW = BATCHED ? (NODES + 4 + 3) / 4 * 4 : 4 * VW;
  static constexpr int PS = RE * HR * (int)sizeof(S);
  static constexpr int B_OFF = 0;
  static constexpr int A_OFF = r16(PS);
  static constexpr int CL_OFF = A_OFF + r16(PS);
  static constexpr int STAGE = r16(CL_OFF + CL_ROW * HR);
  static constexpr int LEV_PLANE = RE * HR * 4;
  static constexpr int LEV_OFF = STAGE * kNS;
  static constexpr int LIST_OFF = LEV_OFF + (T - 1) * 2 * LEV_PLANE;
  static constexpr int SMEM = LIST_OFF + (kMaxSrc + kMaxRec) * 16 + 16;
  static_assert(CXN > 0 && CYR > 0, "tile smaller than its halo");
  static_assert(SMEM + 128 + 256 * 16 + 128 <= 227 * 1024, "shared memory per CTA");
  static_assert(T >= 2 && T <= 4, "depth");
  static_assert(BATCHED || VW == 16, "unbatched x neighbours are exchanged within half warps");
  static_assert(!BATCHED || VW == 32, "batched rows are one warp wide");
};

template <typename A> struct alignas(4 * sizeof(A)) PackedCoef { A a, b, c; uint32_t pos; };

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// cp.async with zero fill when `ok` is false (src-size 0: nothing is read).
__device__ __forceinline__ void cp16(uint32_t dst, const void* src, bool ok) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src),
               "r"(ok ? 16 : 0)
               : "memory");
}
__device__ __forceinline__ void cp8(uint32_t dst, const void* src, bool ok) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(dst), "l"(src),
               "r"(ok ? 8 : 0)
               : "memory");
}
__device__ __forceinline__ void cp4(uint32_t dst, const void* src, bool ok) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(dst), "l"(src),
               "r"(ok ? 4 : 0)
               : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

template <typename S>
__device__ __forceinline__ void cp_vec(uint32_t dst, const S* src, bool ok) {
  if (sizeof(S) == 4) cp16(dst, src, ok);
  else cp8(dst, src, ok);
}

// 4 storage elements from shared memory, widened to float.
__device__ __forceinline__ void ld4f(const float* p, float (&v)[4]) {
  const float4 t = *reinterpret_cast<const float4*>(p);
  v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
}
__device__ __forceinline__ void ld4f(const __half* p, float (&v)[4]) {
  const uint2 t = *reinterpret_cast<const uint2*>(p);
  __half2 a, b;
  memcpy(&a, &t.x, 4);
  memcpy(&b, &t.y, 4);
  const float2 fa = __half22float2(a), fb = __half22float2(b);
  v[0] = fa.x; v[1] = fa.y; v[2] = fb.x; v[3] = fb.y;
}
__device__ __forceinline__ void ld4f(const __nv_bfloat16* p, float (&v)[4]) {
  const uint2 t = *reinterpret_cast<const uint2*>(p);
  v[0] = __uint_as_float(t.x << 16);
  v[1] = __uint_as_float(t.x & 0xFFFF0000u);
  v[2] = __uint_as_float(t.y << 16);
  v[3] = __uint_as_float(t.y & 0xFFFF0000u);
}
__device__ __forceinline__ float ld1f(const float* p) { return *p; }
__device__ __forceinline__ float ld1f(const __half* p) { return __half2float(*p); }
__device__ __forceinline__ float ld1f(const __nv_bfloat16* p) { return __bfloat162float(*p); }

// 4 values to global storage.
__device__ __forceinline__ void st4(float* p, const float (&v)[4]) {
  *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
template <typename S>
__device__ __forceinline__ void st4_16(S* p, const float (&v)[4]) {
  S h[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) h[e] = Store<S>::store(v[e]);
  uint16_t u[4];
  memcpy(u, h, 8);
  *reinterpret_cast<uint2*>(p) =
      make_uint2(u[0] | ((uint32_t)u[1] << 16), u[2] | ((uint32_t)u[3] << 16));
}
__device__ __forceinline__ void st4(__half* p, const float (&v)[4]) { st4_16(p, v); }
__device__ __forceinline__ void st4(__nv_bfloat16* p, const float (&v)[4]) { st4_16(p, v); }

// Value rounded to the storage type, as the plain path stores and reloads it.
template <typename S>
__device__ __forceinline__ float rnd(float v) {
  return Store<S>::load(Store<S>::store(v));
}

struct ListEntry { int plane, vec, lane, id; };

template <int N>
__device__ __forceinline__ void zero4(float (&v)[N]) {
#pragma unroll
  for (int e = 0; e < N; ++e) v[e] = 0.f;
}

template <typename S, int SCHEME, typename Sh>
__global__ void __launch_bounds__(Sh::THREADS, Sh::MINB)
k_update_tb(const S* __restrict__ Pa, const S* __restrict__ Pb, S* __restrict__ Oc,
            S* __restrict__ Od, const uint8_t* __restrict__ cls, ClassTab<float> tab, float l2,
            int X, int Y, int Z, int kshift, int zc, int groups,
            const int64_t* __restrict__ d_step, int n_src, const int64_t* __restrict__ src_idx,
            const int32_t* __restrict__ src_mode, const float* __restrict__ samples,
            int64_t n_samples, int64_t inject_end, int n_rec, const int64_t* __restrict__ rec_idx,
            float* __restrict__ rec_out, int64_t rec_ld) {
  constexpr int T = Sh::T, VW = Sh::VW, HR = Sh::HR, R = Sh::R;
  constexpr bool BATCHED = Sh::BATCHED;
  using Rf = Rn<float>;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  // 128-byte aligned base, derived within the shared window (an integer
  // round trip would make every access through it a generic one)
  unsigned char* smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
  __shared__ PackedCoef<float> stab[256];
  __shared__ int s_nsrc, s_nrec;
  ListEntry* src_list = (ListEntry*)(smem + Sh::LIST_OFF);
  ListEntry* rec_list = src_list + kMaxSrc;

  const int tid = threadIdx.x;
  const int vx = tid % VW, ry0 = (tid / VW) * R;  // first tile row of this thread
  int bx = blockIdx.x, f0 = 0;
  if (BATCHED) {
    bx = blockIdx.x / groups;
    f0 = 4 * (blockIdx.x % groups);
  }
  const int ex0 = bx * Sh::CXN - Sh::XH;       // first node of the extended tile row
  const int ey0 = blockIdx.y * Sh::CYR - T;    // first row of the extended tile
  const int x = BATCHED ? ex0 + vx : ex0 + 4 * vx;
  const bool xin = x >= 0 && x < X;
  const bool xcore = BATCHED ? (vx >= T && vx < T + Sh::CXN) : (vx >= 1 && vx < VW - 1);
  const int z0 = 1 + blockIdx.z * zc;
  const int z1 = min(z0 + zc, Z - 1);
  if (z0 >= z1) return;
  // output planes: the chunk, widened to the never-updated planes 0 / Z-1
  const int zlo = z0 == 1 ? 0 : z0;
  const int zhi = z1 == Z - 1 ? Z - 1 : z1 - 1;
  const int64_t XY = (int64_t)X * Y;
  const int64_t pstride = XY << kshift;  // field elements per plane
  const int64_t n0 = *d_step - T;        // step number of level 0

  bool rin[R], rcore[R];
  int64_t ebase[R], cbase[R];  // plane-0 element and node offsets of each row's vector
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int y = ey0 + ry0 + r;
    rin[r] = xin && y >= 0 && y < Y;
    rcore[r] = rin[r] && xcore && ry0 + r >= T && ry0 + r < HR - T;
    const int64_t node = rin[r] ? (int64_t)y * X + x : 0;
    cbase[r] = node;
    ebase[r] = BATCHED ? (node << kshift) + f0 : node;
  }

  for (int i = tid; i < tab.n && i < 256; i += Sh::THREADS)
    stab[i] = PackedCoef<float>{tab.a[i], tab.b[i], tab.c[i], tab.pos[i]};

  // Sources and receivers inside this CTA's extended tile, in list order
  // (one warp, ballot + prefix count keeps the order of the global lists).
  if (tid < 32) {
    const int lane = tid;
    for (int pass = 0; pass < 2; ++pass) {
      const int n = pass == 0 ? n_src : n_rec;
      const int64_t* idx = pass == 0 ? src_idx : rec_idx;
      ListEntry* out = pass == 0 ? src_list : rec_list;
      int cnt = 0;
      for (int b = 0; b < n; b += 32) {
        const int k = b + lane;
        bool hit = false;
        ListEntry en{0, 0, 0, k};
        if (k < n) {
          const int64_t e = idx[k];
          if (e >= 0) {
            const int64_t node = e >> kshift;
            const int f = (int)(e & ((1 << kshift) - 1));
            const int nz = (int)(node / XY);
            const int64_t rr = node - (int64_t)nz * XY;
            const int ny = (int)(rr / X), nx = (int)(rr - (int64_t)ny * X);
            const int lx = nx - ex0, ly = ny - ey0;
            bool in = lx >= 0 && lx < Sh::NODES && ly >= 0 && ly < HR &&
                      (!BATCHED || (f >= f0 && f < f0 + 4));
            if (pass == 1) {
              // a receiver is written by the CTA whose core holds it
              const bool cx = BATCHED ? (lx >= T && lx < T + Sh::CXN)
                                      : (lx >= 4 && lx < 4 + Sh::CXN);
              in = in && cx && ly >= T && ly < HR - T && nz >= zlo && nz <= zhi;
            }
            if (in) {
              hit = true;
              const int v = BATCHED ? lx : (lx >> 2);
              en = ListEntry{nz, ly * VW + v, BATCHED ? f - f0 : (lx & 3), k};
            }
          }
        }
        const unsigned m = __ballot_sync(0xffffffffu, hit);
        if (hit) out[cnt + __popc(m & ((1u << lane) - 1u))] = en;
        cnt += __popc(m);
      }
      if (lane == 0) {
        if (pass == 0) s_nsrc = cnt;
        else s_nrec = cnt;
      }
    }
  }
  __syncthreads();
  // whether any source or receiver falls on one of this thread's vectors
  bool has_io = false;
  for (int i = 0; i < s_nsrc + s_nrec; ++i) {
    const int v = (i < s_nsrc ? src_list[i] : rec_list[i - s_nsrc]).vec;
#pragma unroll
    for (int r = 0; r < R; ++r) has_io |= v == (ry0 + r) * VW + vx;
  }

  const int zs = max(0, zlo - T);
  const int n_it = zhi + T - zs + 1;
  auto vec_off = [&](int r) { return ((ry0 + r) * VW + vx) * 4; };  // element offset in a plane

  auto issue = [&](int j) {
    const int zl = zs + j;
    unsigned char* st = smem + (j % kNS) * Sh::STAGE;
    if (j < n_it) {
      if (zl < Z) {
#pragma unroll
        for (int r = 0; r < R; ++r)
          cp_vec<S>(smem_u32(st + Sh::B_OFF) + vec_off(r) * (int)sizeof(S),
                    rin[r] ? Pb + ebase[r] + zl * pstride : Pb, rin[r]);
      }
      const int za = zl - 1;
      if (za >= 0 && za < Z) {
#pragma unroll
        for (int r = 0; r < R; ++r)
          cp_vec<S>(smem_u32(st + Sh::A_OFF) + vec_off(r) * (int)sizeof(S),
                    rin[r] ? Pa + ebase[r] + za * pstride : Pa, rin[r]);
        if (!BATCHED) {
#pragma unroll
          for (int r = 0; r < R; ++r)
            cp4(smem_u32(st + Sh::CL_OFF) + vec_off(r), rin[r] ? cls + cbase[r] + za * XY : cls,
                rin[r]);
        } else {
          constexpr int CPR = Sh::CL_ROW / 4;
          const int cb0 = ex0 & ~3;
          for (int i = tid; i < HR * CPR; i += Sh::THREADS) {
            const int r = i / CPR, c = i - r * CPR;
            const int gy = ey0 + r, gx = cb0 + 4 * c;
            const bool ok = gy >= 0 && gy < Y && gx >= 0 && gx + 4 <= X;
            const int64_t nb = ok ? ((int64_t)za * Y + gy) * X + gx : 0;
            cp4(smem_u32(st + Sh::CL_OFF) + r * Sh::CL_ROW + 4 * c, cls + nb, ok);
          }
        }
      }
    }
    cp_commit();
  };

#pragma unroll
  for (int j = 0; j < kNS - 2; ++j) issue(j);

  // Register columns: level t at planes zl-t-1 (cv) and zl-t-2 (mv) from the
  // previous iterations, fr = this iteration's value of each level.
  float cv[T][R][4], mv[T][R][4], fr[T + 1][R][4];
  uint32_t creg[T][R];
#pragma unroll
  for (int t = 0; t < T; ++t)
#pragma unroll
    for (int r = 0; r < R; ++r) {
      creg[t][r] = 0;
      zero4(cv[t][r]);
      zero4(mv[t][r]);
    }

  for (int it = 0; it < n_it; ++it) {
    const int zl = zs + it;
    cp_wait<kNS - 3>();
    __syncthreads();
    const unsigned char* st = smem + (it % kNS) * Sh::STAGE;
    const unsigned char* stp = smem + ((it + kNS - 1) % kNS) * Sh::STAGE;
#pragma unroll
    for (int r = 0; r < R; ++r) ld4f((const S*)(st + Sh::B_OFF) + vec_off(r), fr[0][r]);
    // class ids of plane zl-1 enter the ring; creg[t] holds plane zl-1-t
#pragma unroll
    for (int t = T - 1; t > 0; --t)
#pragma unroll
      for (int r = 0; r < R; ++r) creg[t][r] = creg[t - 1][r];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      if (!BATCHED)
        creg[0][r] = *(const uint32_t*)(st + Sh::CL_OFF + vec_off(r));
      else
        creg[0][r] = st[Sh::CL_OFF + (ry0 + r) * Sh::CL_ROW + (ex0 - (ex0 & ~3)) + vx];
    }

#pragma unroll
    for (int t = 0; t < T; ++t) {
      const int lev = t + 1;
      const int q = zl - lev;  // level lev is computed at plane q
      const int lo = max(0, zlo - (T - lev)), hi = min(Z - 1, zhi + (T - lev));
      if (q >= lo && q <= hi) {  // uniform over the CTA
        // level t at plane q: shared-memory plane (stage for level 0)
        const float* plf =
            (const float*)(smem + Sh::LEV_OFF + ((t - 1) * 2 + ((it + 1) & 1)) * Sh::LEV_PLANE);
        const S* pls = (const S*)(stp + Sh::B_OFF);
        auto ldp = [&](int off, float (&v)[4]) {
          if (t == 0) ld4f(pls + off, v);
          else ld4f(plf + off, v);
        };
        // x neighbours: unbatched, the scalars next to the vector from the
        // lanes either side (the lanes at the tile's x edges are halo); batched,
        // the neighbouring nodes' vectors
        float xl[R], xr[R];
        if (!BATCHED) {
#pragma unroll
          for (int r = 0; r < R; ++r) {
            xl[r] = __shfl_up_sync(0xffffffffu, cv[t][r][3], 1);
            xr[r] = __shfl_down_sync(0xffffffffu, cv[t][r][0], 1);
          }
        }
        float top[4], bot[4];
        if (ry0 > 0) ldp(vec_off(0) - Sh::RE, top);
        else zero4(top);
        if (ry0 + R < HR) ldp(vec_off(R - 1) + Sh::RE, bot);
        else zero4(bot);
#pragma unroll
        for (int r = 0; r < R; ++r) {
          float out[4], past[4];
          if (t == 0) ld4f((const S*)(st + Sh::A_OFF) + vec_off(r), past);
          else {
#pragma unroll
            for (int e = 0; e < 4; ++e) past[e] = mv[t - 1][r][e];
          }
          if (q == 0 || q == Z - 1) {
#pragma unroll
            for (int e = 0; e < 4; ++e) out[e] = past[e];
          } else {
            float ym[4], yp[4], xm[4], xp[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              ym[e] = r > 0 ? cv[t][r - 1][e] : top[e];
              yp[e] = r < R - 1 ? cv[t][r + 1][e] : bot[e];
            }
            if (BATCHED) {
              if (vx > 0) ldp(vec_off(r) - 4, xm);
              else zero4(xm);
              if (vx < VW - 1) ldp(vec_off(r) + 4, xp);
              else zero4(xp);
            } else {
              xm[0] = xl[r]; xm[1] = cv[t][r][0]; xm[2] = cv[t][r][1]; xm[3] = cv[t][r][2];
              xp[0] = cv[t][r][1]; xp[1] = cv[t][r][2]; xp[2] = cv[t][r][3]; xp[3] = xr[r];
            }
            const uint32_t cw = creg[t][r];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              const unsigned c = BATCHED ? cw : ((cw >> (8 * e)) & 0xFFu);
              const PackedCoef<float> k = stab[c];
              const float pc = cv[t][r][e], pm = mv[t][r][e], pn = fr[t][r][e];
              float o;
              if (SCHEME == 0) {
                const float s6 = Rf::add(
                    Rf::add(Rf::add(Rf::add(Rf::add(pn, pm), yp[e]), ym[e]), xp[e]), xm[e]);
                o = Rf::mul(k.a, Rf::sub(Rf::add(Rf::mul(k.b, pc), Rf::mul(l2, s6)),
                                         Rf::mul(k.c, past[e])));
              } else {
                const uint32_t cp = k.pos;
                const float dx = (float)(cp & 1u), dy = (float)((cp >> 1) & 1u),
                            dz = (float)((cp >> 2) & 1u);
                const float bx_ = (cp & 0x10u) ? xp[e] : xm[e];
                const float by_ = (cp & 0x20u) ? yp[e] : ym[e];
                const float bz_ = (cp & 0x40u) ? pm : pn;
                const float sb6 =
                    Rf::add(Rf::add(Rf::mul(bx_, dx), Rf::mul(by_, dy)), Rf::mul(bz_, dz));
                const float s7 = Rf::add(
                    Rf::add(Rf::add(Rf::add(Rf::add(Rf::add(xm[e], xp[e]), ym[e]), yp[e]), pn),
                            pm),
                    sb6);
                o = Rf::mul(k.a, Rf::add(Rf::sub(Rf::mul(s7, l2), Rf::mul(k.b, pc)),
                                         Rf::mul(k.c, past[e])));
              }
              out[e] = rnd<S>(o);
            }
          }
          if (!rin[r]) zero4(out);
          if (lev < T && has_io) {
            const int vec = (ry0 + r) * VW + vx;
            const int64_t step = n0 + lev;
            // receivers of step n0+lev: the value before this step's injection
            if (rec_out != nullptr && step - 1 < rec_ld) {
              for (int i = 0; i < s_nrec; ++i) {
                const ListEntry en = rec_list[i];
                if (en.plane == q && en.vec == vec) {
                  float v = out[0];
#pragma unroll
                  for (int e = 1; e < 4; ++e) v = en.lane == e ? out[e] : v;
                  rec_out[(int64_t)en.id * rec_ld + step - 1] = v;
                }
              }
            }
            if (step < inject_end && step < n_samples) {
              for (int i = 0; i < s_nsrc; ++i) {
                const ListEntry en = src_list[i];
                if (en.plane == q && en.vec == vec) {
                  const float v = samples[(int64_t)en.id * n_samples + step];
                  const bool add = src_mode[en.id] != 0;
#pragma unroll
                  for (int e = 0; e < 4; ++e)
                    if (en.lane == e) out[e] = rnd<S>(add ? Rf::add(out[e], v) : v);
                }
              }
            }
          }
#pragma unroll
          for (int e = 0; e < 4; ++e) fr[lev][r][e] = out[e];
          if (lev < T) {
            float* pl = (float*)(smem + Sh::LEV_OFF + (t * 2 + (it & 1)) * Sh::LEV_PLANE);
            *reinterpret_cast<float4*>(pl + vec_off(r)) =
                make_float4(out[0], out[1], out[2], out[3]);
          }
          if (rcore[r] && q >= zlo && q <= zhi) {
            if (lev == T - 1) st4(Oc + ebase[r] + q * pstride, out);
            else if (lev == T) st4(Od + ebase[r] + q * pstride, out);
          }
        }
      } else {
#pragma unroll
        for (int r = 0; r < R; ++r) zero4(fr[lev][r]);
      }
    }
#pragma unroll
    for (int t = 0; t < T; ++t)
#pragma unroll
      for (int r = 0; r < R; ++r)
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          mv[t][r][e] = cv[t][r][e];
          cv[t][r][e] = fr[t][r][e];
        }
    issue(it + kNS - 2);
  }
  cp_wait<0>();
}

// ---------------------------------------------------------------------------
// host side

template <typename S, int SCHEME, typename Sh>
int launch_tb_t(pfdtd_domain* d, void* rec_out, int64_t rec_ld, int64_t inject_end,
                cudaStream_t s) {
  const int64_t nz = d->Z - 2;
  const int groups = Sh::BATCHED ? d->K / 4 : 1;
  const int gx = (int)((d->X + Sh::CXN - 1) / Sh::CXN) * groups;
  const int gy = (int)((d->Y + Sh::CYR - 1) / Sh::CYR);
  // shared-memory opt-in and occupancy, once per device and instantiation
  constexpr int kMaxDev = 64;
  static int slots_per_sm[kMaxDev] = {};
  static std::mutex mu;
  if (d->device >= kMaxDev) return fail(PFDTD_ERR_UNSUPPORTED, "device index above 63");
  int slots_sm = 0;
  {
    std::lock_guard<std::mutex> g(mu);
    if (slots_per_sm[d->device] == 0) {
      PFDTD_CK(cudaFuncSetAttribute(k_update_tb<S, SCHEME, Sh>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, Sh::SMEM + 128));
      int n = 0;
      PFDTD_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_update_tb<S, SCHEME, Sh>,
                                                             Sh::THREADS, Sh::SMEM + 128));
      if (n < 1) return fail(PFDTD_ERR_UNSUPPORTED, "blocked kernel does not fit on an SM");
      slots_per_sm[d->device] = n;
    }
    slots_sm = slots_per_sm[d->device];
  }
  // z chunks: fill the waves, each chunk paying ~T planes of extra halo work
  const int64_t slots = (int64_t)d->sm_count * slots_sm;
  const int64_t tiles = (int64_t)gx * gy;
  int64_t best_zc = nz;
  double best = 1e300;
  for (int64_t gz = 1; gz <= nz; ++gz) {
    const int64_t zc = (nz + gz - 1) / gz;
    const int64_t gzr = (nz + zc - 1) / zc;
    const double waves = (double)((tiles * gzr + slots - 1) / slots);
    const double cost = waves * (double)(zc + 2 * Sh::T);
    if (cost < best - 1e-9) {
      best = cost;
      best_zc = zc;
    }
  }
  const int zc = (int)best_zc;
  const int gz = (int)((nz + zc - 1) / zc);
  const int a_size = 4;
  const uint8_t* ctab = (const uint8_t*)d->d_ctab;
  const int nc = d->n_classes;
  ClassTab<float> tab{(const float*)ctab, (const float*)(ctab + (size_t)nc * a_size),
                      (const float*)(ctab + 2 * (size_t)nc * a_size),
                      (const uint32_t*)(ctab + 3 * (size_t)nc * a_size), nc};
  // The four buffers form the pairs {0, 1} and {2, 3}; current and past are
  // always one pair (plain steps swap within it).  A blocked launch writes
  // the other pair slot for slot, so two launches restore the roles and a
  // captured chunk of an even number of launches can be replayed.
  const int o1 = d->prev ^ 2;
  const int o2 = d->cur ^ 2;
  S* Oc = (S*)d->field(o1);
  S* Od = (S*)d->field(o2);
  dim3 grid(gx, gy, gz);
  k_update_tb<S, SCHEME, Sh><<<grid, Sh::THREADS, Sh::SMEM + 128, s>>>(
      (const S*)d->past_field(), (const S*)d->cur_field(), Oc, Od, (const uint8_t*)d->d_cls,
      tab, (float)d->params[1], (int)d->X, (int)d->Y, (int)d->Z, d->kshift, zc, groups,
      d->d_step, d->n_src, d->d_src_idx, d->d_src_mode, (const float*)d->d_src_samples,
      d->n_samples, inject_end, d->n_rec, d->d_rec_idx, (float*)rec_out, rec_ld);
  count_launch();
  PFDTD_CK(cudaGetLastError());
  d->prev = o1;
  d->cur = o2;
  return PFDTD_OK;
}

#include "stencil_tb_packed.cuh"

// Tile shapes (x nodes x rows), selected by index (d->tb_shape, -1 = 0):
//  unbatched  0: 64 x 32 from 256 threads of two rows
//             1: 64 x 32 from 512 threads of one row
//             2: 64 x 64 from 512 threads of two rows (depth 2, 3)
//  batched    0: 32 x 32 nodes of 4 fields from 512 threads of two rows
//             1: 32 x 32 (FP32 depth 4: 32 x 24) from one row per thread
//             2: 32 x 32 nodes of 4 fields, packed pair arithmetic, two rows
//                per thread (stencil_tb_packed.cuh; forward scheme, depth 2, 3)
//             3: as 2 with one row per thread (1024 threads)
// Depth 4 has only shape 1; other combinations report PFDTD_ERR_ARG.
template <typename S, int SCHEME, int T>
int launch_tb_d(pfdtd_domain* d, void* rec_out, int64_t rec_ld, int64_t inject_end,
                cudaStream_t s) {
  const int shape = d->tb_shape < 0 ? (T == 4 ? 1 : 0) : d->tb_shape;
  if (d->K == 1) {
    if constexpr (T == 4) {
      if (shape == 1)
        return launch_tb_t<S, SCHEME, TbShape<S, 16, 32, 1, T, false>>(d, rec_out, rec_ld,
                                                                       inject_end, s);
    } else {
      if (shape == 0)
        return launch_tb_t<S, SCHEME, TbShape<S, 16, 16, 2, T, false>>(d, rec_out, rec_ld,
                                                                       inject_end, s);
      if (shape == 1)
        return launch_tb_t<S, SCHEME, TbShape<S, 16, 32, 1, T, false, 2>>(d, rec_out, rec_ld,
                                                                          inject_end, s);
      if (shape == 2)
        return launch_tb_t<S, SCHEME, TbShape<S, 16, 32, 2, T, false>>(d, rec_out, rec_ld,
                                                                       inject_end, s);
    }
  } else {
    if constexpr (T == 4) {
      constexpr int kRows = sizeof(S) == 4 ? 24 : 32;
      if (shape == 1)
        return launch_tb_t<S, SCHEME, TbShape<S, 32, kRows, 1, T, true>>(d, rec_out, rec_ld,
                                                                         inject_end, s);
    } else {
      if (shape == 0)
        return launch_tb_t<S, SCHEME, TbShape<S, 32, 16, 2, T, true>>(d, rec_out, rec_ld,
                                                                      inject_end, s);
      if (shape == 1)
        return launch_tb_t<S, SCHEME, TbShape<S, 32, 32, 1, T, true>>(d, rec_out, rec_ld,
                                                                      inject_end, s);
      if constexpr (SCHEME == 0) {
        if (shape == 2) return launch_tb_packed<S, T, 2>(d, rec_out, rec_ld, inject_end, s);
        if (shape == 3) return launch_tb_packed<S, T, 1>(d, rec_out, rec_ld, inject_end, s);
      }
    }
  }
  return fail(PFDTD_ERR_ARG, "blocked tile shape not available for this depth and batching");
}

template <typename S, int SCHEME>
int launch_tb_s(pfdtd_domain* d, void* rec_out, int64_t rec_ld, int64_t inject_end,
                cudaStream_t s) {
  switch (d->tb_depth) {
    case 2: return launch_tb_d<S, SCHEME, 2>(d, rec_out, rec_ld, inject_end, s);
    case 3: return launch_tb_d<S, SCHEME, 3>(d, rec_out, rec_ld, inject_end, s);
    case 4: return launch_tb_d<S, SCHEME, 4>(d, rec_out, rec_ld, inject_end, s);
  }
  return fail(PFDTD_ERR_ARG, "temporal block depth must be 2, 3 or 4");
}

template <typename S>
int launch_tb_p(pfdtd_domain* d, void* rec_out, int64_t rec_ld, int64_t inject_end,
                cudaStream_t s) {
  return d->class_scheme == PFDTD_SRL ? launch_tb_s<S, 1>(d, rec_out, rec_ld, inject_end, s)
                                      : launch_tb_s<S, 0>(d, rec_out, rec_ld, inject_end, s);
}

}  // namespace tb
}  // namespace pfdtd
