// Temporally blocked update for batched fields with packed FP32 pair
// arithmetic (SRL forward scheme).  Included by stencil_tb.cuh inside
// namespace pfdtd::tb; it uses that file's cp.async helpers, ListEntry and
// the list capacities.
//
// Same schedule as k_update_tb (a CTA owns a core tile of (x, y) nodes and a
// z range, marches z and computes level t at plane zl - t for t = 1..T on an
// extended tile with a T-node halo, writing levels T-1 and T out of place),
// re-laid out for instruction count, which is what bounds the blocked update
// on GB300 while the per-step update is bound by HBM:
//
//  * the fields of a node are adjacent in memory (element = node * K + field),
//    so a thread holds 4 fields of its node as two 64-bit pairs and every
//    add, subtract and multiply of the update runs as one add.rn.f32x2 /
//    sub.rn.f32x2 / mul.rn.f32x2 (sm_100 family) on two fields: each lane of
//    a packed operation rounds exactly as the scalar __fadd_rn / __fsub_rn /
//    __fmul_rn, so the order and rounding of every update are unchanged;
//  * products are fma.rn.f32x2(x, y, -0) with the -0 from a kernel argument:
//    rounded once like mul.rn, and opaque to the compiler, which otherwise
//    contracts packed multiplies into the following packed add (measured on
//    GB300 with ptxas 13.0 even with .rn), which would change the rounding;
//  * the z-march is unrolled by three, the length of the register ring that
//    holds planes q-1, q, q+1 of every level, so the ring rotates by renaming
//    instead of register moves, and iterations whose levels are all interior
//    planes of the CTA's range run without plane checks;
//  * nodes outside the grid take an all-zero coefficient class appended to
//    the table (index n_classes), so they stay 0 at every level without a
//    per-level select;
//  * coefficients are kept in shared memory as duplicated pairs (a, a),
//    (b, b), (c, c), read with one 128-bit and one 64-bit load.
//
// Tile: 32 nodes (one warp, one node per lane) x 32 rows, R = 1 or 2 rows
// per thread (1024 or 512 threads), 4 fields per CTA; the K fields are split
// over K / 4 CTAs that share the tile.  Depth T = 2 or 3.
#pragma once

namespace pktb {

using px::add2;
using px::f2;
using px::fma2;
using px::mul2;
using px::pk2;
using px::sub2;
using px::up2;

// Fields f0..f0+3 of one node: a = (f0, f0+1), b = (f0+2, f0+3).
struct V4 {
  f2 a, b;
};

__device__ __forceinline__ V4 zero_v4() { return V4{0ull, 0ull}; }

// 4 stored elements from shared memory as float pairs.
__device__ __forceinline__ V4 lds_v4(const float* p) {
  const ulonglong2 t = *reinterpret_cast<const ulonglong2*>(p);
  return V4{t.x, t.y};
}
__device__ __forceinline__ V4 lds_v4(const __half* p) {
  const uint2 t = *reinterpret_cast<const uint2*>(p);
  __half2 h0, h1;
  memcpy(&h0, &t.x, 4);
  memcpy(&h1, &t.y, 4);
  const float2 a = __half22float2(h0), b = __half22float2(h1);
  return V4{pk2(a.x, a.y), pk2(b.x, b.y)};
}
__device__ __forceinline__ V4 lds_v4(const __nv_bfloat16* p) {
  const uint2 t = *reinterpret_cast<const uint2*>(p);
  return V4{pk2(__uint_as_float(t.x << 16), __uint_as_float(t.x & 0xFFFF0000u)),
            pk2(__uint_as_float(t.y << 16), __uint_as_float(t.y & 0xFFFF0000u))};
}
__device__ __forceinline__ void sts_v4(float* p, const V4& v) {
  *reinterpret_cast<ulonglong2*>(p) = make_ulonglong2(v.a, v.b);
}

// Values rounded to the storage type, as the per-step path stores them.
template <typename S>
__device__ __forceinline__ V4 rnd_v4(const V4& v) {
  if constexpr (sizeof(S) == 4) {
    return v;
  } else {
    float x0, x1, x2, x3;
    up2(v.a, x0, x1);
    up2(v.b, x2, x3);
    return V4{pk2(rnd<S>(x0), rnd<S>(x1)), pk2(rnd<S>(x2), rnd<S>(x3))};
  }
}

// 4 values to global storage (16-byte or 8-byte aligned).
__device__ __forceinline__ void stg_v4(float* p, const V4& v) {
  *reinterpret_cast<ulonglong2*>(p) = make_ulonglong2(v.a, v.b);
}
template <typename S>
__device__ __forceinline__ void stg_v4(S* p, const V4& v) {
  float x[4];
  up2(v.a, x[0], x[1]);
  up2(v.b, x[2], x[3]);
  st4(p, x);
}

__device__ __forceinline__ float get_lane(const V4& v, int e) {
  float x0, x1, x2, x3;
  up2(v.a, x0, x1);
  up2(v.b, x2, x3);
  return e == 0 ? x0 : e == 1 ? x1 : e == 2 ? x2 : x3;
}
__device__ __forceinline__ void set_lane(V4& v, int e, float val) {
  float x0, x1, x2, x3;
  up2(v.a, x0, x1);
  up2(v.b, x2, x3);
  x0 = e == 0 ? val : x0;
  x1 = e == 1 ? val : x1;
  x2 = e == 2 ? val : x2;
  x3 = e == 3 ? val : x3;
  v.a = pk2(x0, x1);
  v.b = pk2(x2, x3);
}

struct __align__(32) Coef2 {
  f2 aa, bb, cc, pad;
};

}  // namespace pktb

template <typename S, int T_, int R_>
struct PackedShape {
  static constexpr int T = T_;
  static constexpr int NX = 32, NY = 32, R = R_;
  static constexpr int THREADS = NX * NY / R;           // 1024 or 512
  static constexpr int CXN = NX - 2 * T, CYR = NY - 2 * T;
  static constexpr int PS = NX * NY * 4 * (int)sizeof(S);  // stage plane bytes (4 fields)
  static constexpr int CL_ROW = (NX + 4 + 3) / 4 * 4;     // class bytes per row from x0 & ~3
  static constexpr int B_OFF = 0;
  static constexpr int A_OFF = r16(PS);
  static constexpr int CL_OFF = A_OFF + r16(PS);
  static constexpr int STAGE = r16(CL_OFF + CL_ROW * NY);
  static constexpr int LEV_PLANE = NX * NY * 16;           // FP32 level plane bytes
  static constexpr int LEV_OFF = STAGE * kNS;
  static constexpr int LIST_OFF = LEV_OFF + (T - 1) * 2 * LEV_PLANE;
  static constexpr int SMEM = LIST_OFF + (kMaxSrc + kMaxRec) * 16 + 16;
  static_assert(T == 2 || T == 3, "packed blocked kernel depth");
  static_assert(R == 1 || R == 2, "rows per thread");
  static_assert(SMEM + 128 + 256 * 32 + 64 <= 227 * 1024, "shared memory per CTA");
};

template <typename S, int T, int R>
__global__ void __launch_bounds__(32 * 32 / R, 1)
k_update_tb_packed(const S* __restrict__ Pa, const S* __restrict__ Pb, S* __restrict__ Oc,
                   S* __restrict__ Od, const uint8_t* __restrict__ cls, ClassTab<float> tab,
                   float l2f, float nzf, int X, int Y, int Z, int kshift, int zc, int groups,
                   const int64_t* __restrict__ d_step, int n_src,
                   const int64_t* __restrict__ src_idx, const int32_t* __restrict__ src_mode,
                   const float* __restrict__ samples, int64_t n_samples, int64_t inject_end,
                   int n_rec, const int64_t* __restrict__ rec_idx, float* __restrict__ rec_out,
                   int64_t rec_ld) {
  using namespace pktb;
  using Sh = PackedShape<S, T, R>;
  constexpr int NX = Sh::NX, NY = Sh::NY;
  using Rf = Rn<float>;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  // 128-byte aligned base, kept in the shared window (no integer round trip)
  unsigned char* smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
  __shared__ Coef2 ktab[256];
  __shared__ int s_nsrc, s_nrec;
  ListEntry* src_list = (ListEntry*)(smem + Sh::LIST_OFF);
  ListEntry* rec_list = src_list + kMaxSrc;

  const int tid = threadIdx.x;
  const int lane = tid & 31, y0 = (tid >> 5) * R;  // node column and first row of the thread
  const int bx = blockIdx.x / groups, f0 = 4 * (blockIdx.x % groups);
  const int ex0 = bx * Sh::CXN - T;           // first node of the extended tile row
  const int ey0 = blockIdx.y * Sh::CYR - T;   // first row of the extended tile
  const int x = ex0 + lane;
  const bool xin = x >= 0 && x < X;
  const bool xcore = lane >= T && lane < T + Sh::CXN;
  const int z0 = 1 + blockIdx.z * zc;
  const int z1 = min(z0 + zc, Z - 1);
  if (z0 >= z1) return;
  const int zlo = z0 == 1 ? 0 : z0;
  const int zhi = z1 == Z - 1 ? Z - 1 : z1 - 1;
  const int64_t XY = (int64_t)X * Y;
  const int64_t pstride = XY << kshift;

  bool rin[R], rcore[R];
  int64_t ebase[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int y = ey0 + y0 + r;
    rin[r] = xin && y >= 0 && y < Y;
    rcore[r] = rin[r] && xcore && y0 + r >= T && y0 + r < NY - T;
    const int64_t node = rin[r] ? (int64_t)y * X + x : 0;
    ebase[r] = (node << kshift) + f0;
  }

  const int zs = max(0, zlo - T);
  const int n_it = zhi + T - zs + 1;
  // element offsets (4 per node) in a tile plane: own node per row and the
  // neighbours; neighbours past the tile edge are clamped to an in-tile node
  // (only halo nodes read them, whose values are never used)
  const int own0 = (y0 * NX + lane) * 4;
  auto own = [&](int r) { return own0 + r * NX * 4; };
  const int xm0 = own0 - (lane > 0 ? 4 : 0), xp0 = own0 + (lane < NX - 1 ? 4 : 0);
  const int ym0 = y0 > 0 ? own0 - NX * 4 : own0;                        // row y0 - 1
  const int ypR = y0 + R < NY ? own0 + R * NX * 4 : own0 + (R - 1) * NX * 4;  // row y0 + R
  const int cl_col = (ex0 & 3) + lane;

  auto issue = [&](int j) {
    const int zl = zs + j;
    unsigned char* st = smem + (j % kNS) * Sh::STAGE;
    if (j < n_it) {
      if (zl < Z) {
#pragma unroll
        for (int r = 0; r < R; ++r)
          cp_vec<S>(smem_u32(st + Sh::B_OFF) + own(r) * (int)sizeof(S),
                    rin[r] ? Pb + ebase[r] + zl * pstride : Pb, rin[r]);
      }
      const int za = zl - 1;
      if (za >= 0 && za < Z) {
#pragma unroll
        for (int r = 0; r < R; ++r)
          cp_vec<S>(smem_u32(st + Sh::A_OFF) + own(r) * (int)sizeof(S),
                    rin[r] ? Pa + ebase[r] + za * pstride : Pa, rin[r]);
        constexpr int CPR = Sh::CL_ROW / 4;
        const int cb0 = ex0 & ~3;
        if (tid < NY * CPR) {
          const int r = tid / CPR, c = tid - r * CPR;
          const int gy = ey0 + r, gx = cb0 + 4 * c;
          const bool ok = gy >= 0 && gy < Y && gx >= 0 && gx + 4 <= X;
          const int64_t nb = ok ? ((int64_t)za * Y + gy) * X + gx : 0;
          cp4(smem_u32(st + Sh::CL_OFF) + r * Sh::CL_ROW + 4 * c, cls + nb, ok);
        }
      }
    }
    cp_commit();
  };

  // the first planes load while the tables and lists are built
#pragma unroll
  for (int j = 0; j < kNS - 2; ++j) issue(j);

  const int64_t n0 = *d_step - T;  // step number of level 0
  // coefficient pairs; index tab.n is the zero class of nodes outside the grid
  const unsigned zcls = (unsigned)tab.n;
  for (int i = tid; i <= tab.n && i < 256; i += Sh::THREADS) {
    const float a = i < tab.n ? tab.a[i] : 0.f, b = i < tab.n ? tab.b[i] : 0.f,
                c = i < tab.n ? tab.c[i] : 0.f;
    ktab[i] = Coef2{pk2(a, a), pk2(b, b), pk2(c, c), 0ull};
  }

  // Sources and receivers inside the extended tile and the planes this CTA
  // computes, in list order.
  if (tid < 32) {
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
            bool in = lx >= 0 && lx < NX && ly >= 0 && ly < NY && f >= f0 && f < f0 + 4 &&
                      nz >= zlo - T && nz <= zhi + T;
            if (pass == 1)  // a receiver is written by the CTA whose core holds it
              in = in && lx >= T && lx < T + Sh::CXN && ly >= T && ly < NY - T && nz >= zlo &&
                   nz <= zhi;
            if (in) {
              hit = true;
              en = ListEntry{nz, ly * NX + lx, f - f0, k};
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
  bool has_io = false;
  for (int i = 0; i < s_nsrc + s_nrec; ++i) {
    const int v = (i < s_nsrc ? src_list[i] : rec_list[i - s_nsrc]).vec;
#pragma unroll
    for (int r = 0; r < R; ++r) has_io |= v == (y0 + r) * NX + lane;
  }
  const bool warp_io = __any_sync(0xffffffffu, has_io);

  // lv[t][s][r]: level t of the thread's node in row r at the plane whose
  // ring slot is s (plane p has slot (p - zs) mod 3).
  V4 lv[T][3][R];
#pragma unroll
  for (int t = 0; t < T; ++t)
#pragma unroll
    for (int s = 0; s < 3; ++s)
#pragma unroll
      for (int r = 0; r < R; ++r) lv[t][s][r] = zero_v4();
  // class ids: byte t-1 of creg[r] is the class of plane zl - t
  uint32_t creg[R];
#pragma unroll
  for (int r = 0; r < R; ++r) creg[r] = 0u;
  const f2 l2 = pk2(l2f, l2f);
  // Products are formed as fma(x, y, -0): one rounding, the value of the
  // product, and an addend the compiler cannot see as zero, so no product
  // is contracted into the sums that follow.
  const f2 nz = pk2(nzf, nzf);

  // Sources and receivers of step n0 + L at plane q on this thread's node of
  // row r: record the value before injection, then inject in list order.
  auto apply_io = [&](V4& out, int L, int r, int q) {
    const int vec = (y0 + r) * NX + lane;
    const int64_t step = n0 + L;
    if (rec_out != nullptr && step - 1 < rec_ld) {
      for (int i = 0; i < s_nrec; ++i) {
        const ListEntry en = rec_list[i];
        if (en.plane == q && en.vec == vec)
          rec_out[(int64_t)en.id * rec_ld + step - 1] = get_lane(out, en.lane);
      }
    }
    if (step < inject_end && step < n_samples) {
      for (int i = 0; i < s_nsrc; ++i) {
        const ListEntry en = src_list[i];
        if (en.plane == q && en.vec == vec) {
          const float v = samples[(int64_t)en.id * n_samples + step];
          const float o = get_lane(out, en.lane);
          set_lane(out, en.lane, rnd<S>(src_mode[en.id] != 0 ? Rf::add(o, v) : v));
        }
      }
    }
  };

  // One z iteration.  CHK: the planes of some level leave the range this CTA
  // computes or touch plane 0 / Z-1 (prologue and epilogue); otherwise every
  // level is an interior update and no plane check is made.
  auto iter = [&](auto PHc, auto CHKc, int it) {
    constexpr int PH = decltype(PHc)::value;
    constexpr bool CHK = decltype(CHKc)::value;
    const int zl = zs + it;
    cp_wait<kNS - 3>();
    __syncthreads();
    const unsigned char* st = smem + (it & (kNS - 1)) * Sh::STAGE;
    const unsigned char* stp = smem + ((it + kNS - 1) & (kNS - 1)) * Sh::STAGE;
#pragma unroll
    for (int r = 0; r < R; ++r) lv[0][PH][r] = lds_v4((const S*)(st + Sh::B_OFF) + own(r));
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const unsigned b = st[Sh::CL_OFF + (y0 + r) * Sh::CL_ROW + cl_col];
      creg[r] = (creg[r] << 8) | (rin[r] ? b : zcls);
    }
#pragma unroll
    for (int L = 1; L <= T; ++L) {
      const int q = zl - L;
      const int sc = (PH - L + 6) % 3;      // slot of plane q
      const int sm = (PH - L - 1 + 6) % 3;  // plane q - 1
      const int sn = (PH - L + 1 + 6) % 3;  // plane q + 1
      bool run = true;
      if constexpr (CHK) {
        const int lo = max(0, zlo - (T - L)), hi = min(Z - 1, zhi + (T - L));
        run = q >= lo && q <= hi;
      }
      if (run) {  // uniform over the CTA
        // level L-1 at plane q: the stage of plane zl-1 for level 0, else the
        // level plane written in the previous iteration
        const float* plf = (const float*)(smem + Sh::LEV_OFF +
                                          ((L >= 2 ? (L - 2) * 2 : 0) + ((it + 1) & 1)) *
                                              Sh::LEV_PLANE);
        const S* pls = (const S*)(stp + Sh::B_OFF);
        auto ldn = [&](int off) -> V4 {
          if (L == 1) return lds_v4(pls + off);
          return lds_v4(plf + off);
        };
        const bool edge = CHK && (q == 0 || q == Z - 1);
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const V4 pc = lv[L - 1][sc][r];
          V4 past;
          if (L == 1) past = lds_v4((const S*)(st + Sh::A_OFF) + own(r));
          else past = lv[L - 2][sc][r];
          V4 out;
          if (edge) {
            out = past;  // planes 0 and Z-1 are never updated
          } else {
            const V4 pm = lv[L - 1][sm][r], pn = lv[L - 1][sn][r];
            const V4 xm = ldn(xm0 + r * NX * 4);
            const V4 xp = ldn(xp0 + r * NX * 4);
            const V4 ym = r > 0 ? lv[L - 1][sc][r > 0 ? r - 1 : 0] : ldn(ym0);
            const V4 yp = r < R - 1 ? lv[L - 1][sc][r < R - 1 ? r + 1 : 0] : ldn(ypR);
            const unsigned c = (creg[r] >> (8 * (L - 1))) & 0xFFu;
            const Coef2 k = ktab[c];
            const f2 s6a = add2(add2(add2(add2(add2(pn.a, pm.a), yp.a), ym.a), xp.a), xm.a);
            const f2 s6b = add2(add2(add2(add2(add2(pn.b, pm.b), yp.b), ym.b), xp.b), xm.b);
            out.a = mul2(k.aa, sub2(add2(fma2(k.bb, pc.a, nz), fma2(l2, s6a, nz)),
                                    fma2(k.cc, past.a, nz)));
            out.b = mul2(k.aa, sub2(add2(fma2(k.bb, pc.b, nz), fma2(l2, s6b, nz)),
                                    fma2(k.cc, past.b, nz)));
            out = rnd_v4<S>(out);
          }
          if (L < T && warp_io) apply_io(out, L, r, q);
          if (L < T) {
            lv[L][sc][r] = out;
            float* pl = (float*)(smem + Sh::LEV_OFF + ((L - 1) * 2 + (it & 1)) * Sh::LEV_PLANE);
            sts_v4(pl + own(r), out);
          }
          if (L >= T - 1 && rcore[r]) {
            const bool in_z = !CHK || (q >= zlo && q <= zhi);
            if (in_z) stg_v4((L == T ? Od : Oc) + ebase[r] + q * pstride, out);
          }
        }
      }
    }
    issue(it + kNS - 2);
  };

  // steady iterations: every level interior and inside the CTA's planes
  const int zq0 = max(T + 1, zlo + T), zq1 = min(Z - 1, zhi + T - 1);
  auto one = [&](auto PHc, int it) {
    if (it < n_it) {
      const int zl = zs + it;
      if (zl >= zq0 && zl <= zq1) iter(PHc, std::false_type{}, it);
      else iter(PHc, std::true_type{}, it);
    }
  };
#pragma unroll 1
  for (int itb = 0; itb < n_it; itb += 3) {
    one(std::integral_constant<int, 0>{}, itb);
    one(std::integral_constant<int, 1>{}, itb + 1);
    one(std::integral_constant<int, 2>{}, itb + 2);
  }
  cp_wait<0>();
}

template <typename S, int T, int R>
int launch_tb_packed(pfdtd_domain* d, void* rec_out, int64_t rec_ld, int64_t inject_end,
                     cudaStream_t s) {
  using Sh = PackedShape<S, T, R>;
  if (d->K < 4 || d->K % 4 != 0)
    return fail(PFDTD_ERR_ARG, "the packed blocked kernel needs batched fields (K a multiple of 4)");
  if (d->n_classes >= 256)
    return fail(PFDTD_ERR_ARG, "the packed blocked kernel needs fewer than 256 node classes");
  const int64_t nz = d->Z - 2;
  const int groups = d->K / 4;
  const int gx = (int)((d->X + Sh::CXN - 1) / Sh::CXN) * groups;
  const int gy = (int)((d->Y + Sh::CYR - 1) / Sh::CYR);
  constexpr int kMaxDev = 64;
  static int slots_per_sm[kMaxDev] = {};
  static std::mutex mu;
  if (d->device >= kMaxDev) return fail(PFDTD_ERR_UNSUPPORTED, "device index above 63");
  int slots_sm = 0;
  {
    std::lock_guard<std::mutex> g(mu);
    if (slots_per_sm[d->device] == 0) {
      PFDTD_CK(cudaFuncSetAttribute(k_update_tb_packed<S, T, R>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, Sh::SMEM + 128));
      int n = 0;
      PFDTD_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_update_tb_packed<S, T, R>,
                                                             Sh::THREADS, Sh::SMEM + 128));
      if (n < 1) return fail(PFDTD_ERR_UNSUPPORTED, "packed blocked kernel does not fit on an SM");
      slots_per_sm[d->device] = n;
    }
    slots_sm = slots_per_sm[d->device];
  }
  const int64_t slots = (int64_t)d->sm_count * slots_sm;
  const int64_t tiles = (int64_t)gx * gy;
  int64_t best_zc = nz;
  double best = 1e300;
  for (int64_t gz = 1; gz <= nz; ++gz) {
    const int64_t zc = (nz + gz - 1) / gz;
    const int64_t gzr = (nz + zc - 1) / zc;
    const double waves = (double)((tiles * gzr + slots - 1) / slots);
    const double cost = waves * (double)(zc + 2 * T);
    if (cost < best - 1e-9) {
      best = cost;
      best_zc = zc;
    }
  }
  const int zc = (int)best_zc;
  const int gz = (int)((nz + zc - 1) / zc);
  const uint8_t* ctab = (const uint8_t*)d->d_ctab;
  const int nc = d->n_classes;
  ClassTab<float> tab{(const float*)ctab, (const float*)(ctab + (size_t)nc * 4),
                      (const float*)(ctab + 2 * (size_t)nc * 4),
                      (const uint32_t*)(ctab + 3 * (size_t)nc * 4), nc};
  const int o1 = d->prev ^ 2;
  const int o2 = d->cur ^ 2;
  S* Oc = (S*)d->field(o1);
  S* Od = (S*)d->field(o2);
  dim3 grid(gx, gy, gz);
  k_update_tb_packed<S, T, R><<<grid, Sh::THREADS, Sh::SMEM + 128, s>>>(
      (const S*)d->past_field(), (const S*)d->cur_field(), Oc, Od, (const uint8_t*)d->d_cls,
      tab, (float)d->params[1], -0.0f, (int)d->X, (int)d->Y, (int)d->Z, d->kshift, zc, groups,
      d->d_step, d->n_src, d->d_src_idx, d->d_src_mode, (const float*)d->d_src_samples,
      d->n_samples, inject_end, d->n_rec, d->d_rec_idx, (float*)rec_out, rec_ld);
  count_launch();
  PFDTD_CK(cudaGetLastError());
  d->prev = o1;
  d->cur = o2;
  return PFDTD_OK;
}
