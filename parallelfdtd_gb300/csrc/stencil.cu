// Leapfrog pressure update kernels (SRL forward and centred, frequency-
// independent boundaries) and the per-step source/receiver kernel.
//
// Update rules follow ParallelFDTD src/kernels/kernels3d.cu:485-529
// (forward / Bilbao) and :608-665 (centred / Kowalczyk) operation for
// operation; the coefficients that depend only on the node's (position,
// material) pair are evaluated once per class on the host with the same
// expressions (classes_host.cpp), and every remaining product and sum is
// issued with an explicitly rounded intrinsic so nothing is contracted.
#include "common.cuh"

#include <algorithm>
#include <type_traits>
#include <cstring>

namespace pfdtd {

namespace {

constexpr int kBX = 32;   // threads along x (one warp = one row segment)
constexpr int kBY = 8;    // rows per block

// z-marching update.  One thread owns the column (x, y) for z in [z0, z1):
// P at z-1, z, z+1 stays in registers while the x/y neighbours at plane z are
// read through the read-only cache (they are other threads' centre values).
// Neighbour addressing is by flat offsets (+-1, +-X, +-X*Y) exactly as the
// reference indexes, so a node on an outer x or y face sees the same wrapped
// neighbour the reference kernel reads.
template <typename S, typename C, int SCHEME>
__global__ void __launch_bounds__(kBX * kBY)
k_update_zmarch(const C* __restrict__ cls, const S* __restrict__ P, S* __restrict__ Pp,
                ClassTab<typename Store<S>::A> tab, int X, int Y, int64_t XY, int z_last,
                int zc, typename Store<S>::A l2, int ks, int kshift) {
  using A = typename Store<S>::A;
  using R = Rn<A>;
  using St = Store<S>;
  constexpr bool kSmemTab = (sizeof(C) == 1);
  __shared__ A sa[kSmemTab ? 256 : 1], sb[kSmemTab ? 256 : 1], sc[kSmemTab ? 256 : 1];
  __shared__ uint32_t sp[kSmemTab ? 256 : 1];
  if (kSmemTab) {
    const int t = threadIdx.y * kBX + threadIdx.x;
    for (int i = t; i < tab.n; i += kBX * kBY) {
      sa[i] = tab.a[i];
      sb[i] = tab.b[i];
      sc[i] = tab.c[i];
      sp[i] = tab.pos[i];
    }
    __syncthreads();
  }
  // X and XY count field elements (nodes times ks fields); ks is the element
  // distance of the x neighbour.
  const int x = blockIdx.x * kBX + threadIdx.x;
  const int y = blockIdx.y * kBY + threadIdx.y;
  const int z0 = 1 + blockIdx.z * zc;
  const int z1 = min(z0 + zc, z_last);
  if (x >= X || y >= Y || z0 >= z1) return;
  int64_t idx = (int64_t)z0 * XY + (int64_t)y * X + x;
  A pm = St::load(P[idx - XY]);
  A pc = St::load(P[idx]);
  for (int z = z0; z < z1; ++z, idx += XY) {
    const A pn = St::load(P[idx + XY]);
    const A xm = St::load(P[idx - ks]);
    const A xp = St::load(P[idx + ks]);
    const A ym = St::load(P[idx - X]);
    const A yp = St::load(P[idx + X]);
    const unsigned c = cls[idx >> kshift];
    const A pp = St::load(Pp[idx]);
    A ca, cb, cc;
    uint32_t cp;
    if (kSmemTab) {
      ca = sa[c]; cb = sb[c]; cc = sc[c]; cp = sp[c];
    } else {
      ca = __ldg(tab.a + c); cb = __ldg(tab.b + c); cc = __ldg(tab.c + c); cp = __ldg(tab.pos + c);
    }
    A out;
    if (SCHEME == 0 || SCHEME == 4) {
      // S = P[z+1] + P[z-1] + P[y+1] + P[y-1] + P[x+1] + P[x-1]  (kernels3d.cu:525)
      const A s6 = R::add(R::add(R::add(R::add(R::add(pn, pm), yp), ym), xp), xm);
      if (SCHEME == 4) {
        // difference form: a (((1+beta) p + (1-beta)(p - pp)) + l2 (S - K p)),
        // cb = K and the pos word holds the float 1 + beta
        const A e = (A)__uint_as_float(cp);
        out = R::mul(ca, R::add(R::add(R::mul(e, pc), R::mul(cc, R::sub(pc, pp))),
                                R::mul(l2, R::sub(s6, R::mul(cb, pc)))));
      } else {
        // sw/(1+beta) * ((2 - K l2) p + l2 S - (1 - beta) pp)   (kernels3d.cu:526)
        out = R::mul(ca, R::sub(R::add(R::mul(cb, pc), R::mul(l2, s6)), R::mul(cc, pp)));
      }
    } else {
      // Mirrored boundary neighbour per axis (kernels3d.cu:642-659).
      const A dx = (A)(cp & 1u), dy = (A)((cp >> 1) & 1u), dz = (A)((cp >> 2) & 1u);
      const A bx = (cp & 0x10u) ? xp : xm;
      const A by = (cp & 0x20u) ? yp : ym;
      const A bz = (cp & 0x40u) ? pm : pn;
      const A sb6 = R::add(R::add(R::mul(bx, dx), R::mul(by, dy)), R::mul(bz, dz));
      const A s7 = R::add(R::add(R::add(R::add(R::add(R::add(xm, xp), ym), yp), pn), pm), sb6);
      const A s = R::mul(s7, l2);
      // (S - (2 - 6 l2) p + (beta - 1) pp) * sw / (1 + beta)  (kernels3d.cu:663)
      out = R::mul(ca, R::add(R::sub(s, R::mul(cb, pc)), R::mul(cc, pp)));
    }
    Pp[idx] = St::store(out);
    pm = pc;
    pc = pn;
  }
}

// IWB 27-point update (no counterpart in the reference).  One thread per
// (x, y) column marching z; the 3 x 3 neighbourhood of planes z-1, z and z+1
// stays in registers and each step reads the 3 x 3 block of plane z+1 through
// the read-only cache.  Boundary closure (finite volume on the voxel grid): a
// neighbour whose bit is set in the node's closed mask (k_iwb_geometry)
// contributes the node's own value.  Sums follow the canonical order of the
// oracle (iwb_sums: in-plane sums of each plane, then combined).
template <typename S, typename C>
__global__ void __launch_bounds__(kBX * kBY)
k_update_iwb(const C* __restrict__ cls, const uint32_t* __restrict__ mask,
             const S* __restrict__ P, S* __restrict__ Pp, ClassTab<typename Store<S>::A> tab,
             int X, int Y, int64_t XY, int z_last, int zc, int ks, int kshift,
             typename Store<S>::A l2) {
  using A = typename Store<S>::A;
  using R = Rn<A>;
  using St = Store<S>;
  const int x = blockIdx.x * kBX + threadIdx.x;
  const int y = blockIdx.y * kBY + threadIdx.y;
  const int z0 = 1 + blockIdx.z * zc;
  const int z1 = min(z0 + zc, z_last);
  if (x >= X || y >= Y || z0 >= z1) return;
  // v[plane][dy+1][dx+1]: plane 0 = z-1, 1 = z, 2 = z+1
  A v[3][3][3];
  auto load_plane = [&](int slot, int64_t base) {
#pragma unroll
    for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
      for (int dx = -1; dx <= 1; ++dx)
        v[slot][dy + 1][dx + 1] = St::load(__ldg(P + base + (int64_t)dy * X + dx * ks));
  };
  int64_t idx = (int64_t)z0 * XY + (int64_t)y * X + x;
  load_plane(0, idx - XY);
  load_plane(1, idx);
  for (int z = z0; z < z1; ++z, idx += XY) {
    load_plane(2, idx + XY);
    const unsigned c = cls[idx >> kshift];
    const uint32_t mk = __ldg(mask + (idx >> kshift));
    const A pp = St::load(Pp[idx]);
    const A ca = __ldg(tab.a + c), cb = __ldg(tab.b + c), cc = __ldg(tab.c + c);
    A m[3][3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b)
#pragma unroll
        for (int e = 0; e < 3; ++e) m[a][b][e] = v[a][b][e];
    if (mk) {
      int k = 0;
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b)
#pragma unroll
          for (int e = 0; e < 3; ++e) {
            if (a == 1 && b == 1 && e == 1) continue;
            if ((mk >> k) & 1u) m[a][b][e] = v[1][1][1];
            ++k;
          }
    }
    A s1, s2, s3;
    iwb_sums(m, s1, s2, s3);
    const A sw = R::mul(l2, R::add(R::add(R::mul(s1, (A)0.25), R::mul(s2, (A)0.125)),
                                   R::mul(s3, (A)0.0625)));
    const A out = R::mul(ca, R::sub(R::add(sw, R::mul(cb, v[1][1][1])), R::mul(cc, pp)));
    Pp[idx] = St::store(ca == (A)0 ? (A)0 : out);  // a node outside the room holds +0
#pragma unroll
    for (int b = 0; b < 3; ++b)
#pragma unroll
      for (int e = 0; e < 3; ++e) {
        v[0][b][e] = v[1][b][e];
        v[1][b][e] = v[2][b][e];
      }
  }
}

// IWB geometry per node: bit k of the mask is set when the k-th of the 26
// neighbours (flat offsets dz*XY + dy*X + dx for dz, dy, dx in -1, 0, 1,
// skipping the centre) is closed: outside the grid or without the inside
// bit.  The code is 0 for a node without the inside bit, else
// 1 + W16 + 64 * face, W16 = 4 (closed faces) + 2 (closed edges) + (closed
// corners), face = 1 when a face neighbour is closed; it replaces the
// position byte in the IWB class key.
__global__ void k_iwb_geometry(const uint8_t* __restrict__ pos, int64_t N, int64_t X,
                               int64_t XY, uint32_t* __restrict__ mask,
                               uint8_t* __restrict__ code) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < N;
       c += (int64_t)gridDim.x * blockDim.x) {
    uint32_t m = 0;
    int w16 = 0, face = 0, k = 0;
#pragma unroll
    for (int dz = -1; dz <= 1; ++dz)
#pragma unroll
      for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
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
    mask[c] = m;
    code[c] = (pos[c] >> 7) ? (uint8_t)(1 + w16 + 64 * face) : 0;
  }
}

// Between two updates: record receivers from the current field for the step
// just finished (kernels3d.cu:164-173), then inject this step's source
// samples into the current field in source order (kernels3d.cu:93-104).
template <typename S>
__global__ void k_step_io(S* __restrict__ cur, int64_t* __restrict__ d_step, int n_rec,
                          const int64_t* __restrict__ rec_idx,
                          typename Store<S>::A* __restrict__ rec_out,
                          int64_t rec_ld, int n_src, const int64_t* __restrict__ src_idx,
                          const int32_t* __restrict__ src_mode,
                          const typename Store<S>::A* __restrict__ samples, int64_t n_samples,
                          int64_t inject_end, int advance) {
  using A = typename Store<S>::A;
  using St = Store<S>;
  const int64_t n = *d_step;
  if (n > 0 && rec_out != nullptr) {
    for (int r = threadIdx.x; r < n_rec; r += blockDim.x) {
      const int64_t i = rec_idx[r];
      if (i >= 0 && n - 1 < rec_ld) rec_out[(int64_t)r * rec_ld + (n - 1)] = St::load(cur[i]);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (n < inject_end && n < n_samples) {
      for (int k = 0; k < n_src; ++k) {
        const int64_t i = src_idx[k];
        if (i < 0) continue;
        const A v = samples[(int64_t)k * n_samples + n];
        if (src_mode[k] == 0)
          cur[i] = St::store(v);
        else
          cur[i] = St::store(Rn<A>::add(St::load(cur[i]), v));
      }
    }
    // A temporally blocked update that follows advances by its depth.
    *d_step = n + advance;
  }
}

// Presence of (pos, mat) keys over the updated planes z = 1..Z-2.
__global__ void k_key_presence(const uint8_t* __restrict__ pos, const uint8_t* __restrict__ mat,
                               int64_t begin, int64_t end, uint8_t* __restrict__ present) {
  for (int64_t i = begin + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < end;
       i += (int64_t)gridDim.x * blockDim.x)
    present[((unsigned)pos[i] << 8) | mat[i]] = 1;
}

template <typename C>
__global__ void k_map_classes(const uint8_t* __restrict__ pos, const uint8_t* __restrict__ mat,
                              int64_t n, const uint16_t* __restrict__ lut, C* __restrict__ cls) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    cls[i] = (C)lut[((unsigned)pos[i] << 8) | mat[i]];
}

template <typename S, typename C, int SCHEME>
int launch_update_t(pfdtd_domain* d, const void* cur, void* past, cudaStream_t s) {
  using A = typename Store<S>::A;
  const int64_t nz = d->Z - 2;
  if (nz <= 0) return PFDTD_OK;
  const int64_t XE = d->X * d->K;
  const int gx = (int)((XE + kBX - 1) / kBX);
  const int gy = (int)((d->Y + kBY - 1) / kBY);
  // Enough z-chunks for several waves of 8 resident blocks on each SM.
  const int64_t target = (int64_t)d->sm_count * 8 * 4;
  int64_t zc = std::max<int64_t>(8, (nz * (int64_t)gx * gy + target - 1) / target);
  zc = std::min<int64_t>(zc, nz);
  const int gz = (int)((nz + zc - 1) / zc);
  const size_t as = sizeof(A);
  const char* tb = (const char*)d->d_ctab;
  ClassTab<A> tab{(const A*)tb, (const A*)(tb + as * d->n_classes),
                  (const A*)(tb + 2 * as * d->n_classes),
                  (const uint32_t*)(tb + 3 * as * d->n_classes), d->n_classes};
  k_update_zmarch<S, C, SCHEME><<<dim3(gx, gy, gz), dim3(kBX, kBY), 0, s>>>(
      (const C*)d->d_cls, (const S*)cur, (S*)past, tab, (int)XE, (int)d->Y, d->XY * d->K,
      (int)(d->Z - 1), (int)zc, (A)d->params[1], d->K, d->kshift);
  count_launch();
  PFDTD_CK(cudaGetLastError());
  return PFDTD_OK;
}

template <typename S, typename C>
int launch_iwb_t(pfdtd_domain* d, const void* cur, void* past, cudaStream_t s) {
  using A = typename Store<S>::A;
  const int64_t nz = d->Z - 2;
  if (nz <= 0) return PFDTD_OK;
  const int64_t XE = d->X * d->K;
  const int gx = (int)((XE + kBX - 1) / kBX);
  const int gy = (int)((d->Y + kBY - 1) / kBY);
  const int64_t target = (int64_t)d->sm_count * 8 * 4;
  int64_t zc = std::max<int64_t>(8, (nz * (int64_t)gx * gy + target - 1) / target);
  zc = std::min<int64_t>(zc, nz);
  const int gz = (int)((nz + zc - 1) / zc);
  const size_t as = sizeof(A);
  const char* tb = (const char*)d->d_ctab;
  ClassTab<A> tab{(const A*)tb, (const A*)(tb + as * d->n_classes),
                  (const A*)(tb + 2 * as * d->n_classes),
                  (const uint32_t*)(tb + 3 * as * d->n_classes), d->n_classes};
  k_update_iwb<S, C><<<dim3(gx, gy, gz), dim3(kBX, kBY), 0, s>>>(
      (const C*)d->d_cls, d->d_iwb_mask, (const S*)cur, (S*)past, tab, (int)XE, (int)d->Y,
      d->XY * d->K, (int)(d->Z - 1), (int)zc, d->K, d->kshift, (A)d->params[1]);
  count_launch();
  PFDTD_CK(cudaGetLastError());
  return PFDTD_OK;
}

template <typename S>
int launch_update_s(pfdtd_domain* d, const void* cur, void* past, cudaStream_t s) {
  if (d->class_scheme == PFDTD_IWB)
    return d->cls_bytes == 1 ? launch_iwb_t<S, uint8_t>(d, cur, past, s)
                             : launch_iwb_t<S, uint16_t>(d, cur, past, s);
  const bool centred = (d->class_scheme == PFDTD_SRL);
  if constexpr (std::is_same<S, float>::value) {  // the difference form (FP32 fields)
    if (d->class_form == PFDTD_FORM_DIFFERENCE)
      return d->cls_bytes == 1 ? launch_update_t<S, uint8_t, 4>(d, cur, past, s)
                               : launch_update_t<S, uint16_t, 4>(d, cur, past, s);
  }
  if (d->cls_bytes == 1)
    return centred ? launch_update_t<S, uint8_t, 1>(d, cur, past, s)
                   : launch_update_t<S, uint8_t, 0>(d, cur, past, s);
  return centred ? launch_update_t<S, uint16_t, 1>(d, cur, past, s)
                 : launch_update_t<S, uint16_t, 0>(d, cur, past, s);
}

template <typename S>
int launch_io_t(pfdtd_domain* d, void* cur, void* rec_out, int64_t rec_ld, int64_t inject_end,
                cudaStream_t s, int advance) {
  using A = typename Store<S>::A;
  const int threads = std::max(32, std::min(1024, ((d->n_rec + 31) / 32) * 32));
  k_step_io<S><<<1, threads, 0, s>>>((S*)cur, d->d_step, d->n_rec, d->d_rec_idx, (A*)rec_out,
                                    rec_ld, d->n_src, d->d_src_idx, d->d_src_mode,
                                    (const A*)d->d_src_samples, d->n_samples, inject_end,
                                    advance);
  count_launch();
  PFDTD_CK(cudaGetLastError());
  return PFDTD_OK;
}

}  // namespace

// Host-side class coefficient evaluation (classes_host.cpp).
int eval_class_coefs(int precision, int scheme, int form, int quirks, const double* params,
                     const std::vector<double>& materials, int n_mat, int n_coef,
                     const std::vector<uint16_t>& keys, std::vector<uint8_t>& out_tab);

int launch_update(pfdtd_domain* d, const void* cur, void* past, cudaStream_t s) {
  if (uses_tma(d))
    return d->class_scheme == PFDTD_IWB ? launch_iwb_tma(d, cur, past, s)
                                        : launch_update_tma(d, cur, past, s);
  switch (d->precision) {
    case PFDTD_F32: return launch_update_s<float>(d, cur, past, s);
    case PFDTD_F64: return launch_update_s<double>(d, cur, past, s);
    case PFDTD_F16: return launch_update_s<__half>(d, cur, past, s);
    case PFDTD_BF16: return launch_update_s<__nv_bfloat16>(d, cur, past, s);
  }
  return fail(PFDTD_ERR_UNSUPPORTED, "unknown precision");
}

int launch_io(pfdtd_domain* d, void* cur, void* rec_out, int64_t rec_ld, int64_t inject_end,
              cudaStream_t s, int advance) {
  switch (d->precision) {
    case PFDTD_F32: return launch_io_t<float>(d, cur, rec_out, rec_ld, inject_end, s, advance);
    case PFDTD_F64: return launch_io_t<double>(d, cur, rec_out, rec_ld, inject_end, s, advance);
    case PFDTD_F16: return launch_io_t<__half>(d, cur, rec_out, rec_ld, inject_end, s, advance);
    case PFDTD_BF16:
      return launch_io_t<__nv_bfloat16>(d, cur, rec_out, rec_ld, inject_end, s, advance);
  }
  return fail(PFDTD_ERR_UNSUPPORTED, "unknown precision");
}

// Build the class ids and the coefficient table for the domain's current
// scheme, quirks, parameters and materials.
int build_classes(pfdtd_domain* d) {
  const int scheme = (d->scheme == PFDTD_SRL || d->scheme == PFDTD_IWB) ? d->scheme
                                                                       : PFDTD_SRL_FORWARD;
  const int form = scheme == PFDTD_SRL_FORWARD ? d->update_form : PFDTD_FORM_REFERENCE;
  if (!d->classes_dirty && d->class_scheme == scheme && d->class_form == form) return PFDTD_OK;
  if (!d->nodes_set) return fail(PFDTD_ERR_STATE, "node bytes not set");
  if (d->n_mat <= 0) return fail(PFDTD_ERR_STATE, "material table not set");
  if (form != PFDTD_FORM_REFERENCE) {
    for (int32_t f : d->dif_flags)
      if (f)
        return fail(PFDTD_ERR_UNSUPPORTED,
                    "the difference form is not built for frequency-dependent boundaries");
    if (d->precision != PFDTD_F32)
      return fail(PFDTD_ERR_UNSUPPORTED, "the difference form is built for FP32 fields");
  }
  cudaStream_t s = d->stream;
  uint8_t* d_present = nullptr;
  PFDTD_CK(cudaMallocAsync((void**)&d_present, 65536, s));
  PFDTD_CK(cudaMemsetAsync(d_present, 0, 65536, s));
  // IWB classes are keyed by the geometry code instead of the position byte.
  const uint8_t* key_bytes = d->d_pos;
  if (scheme == PFDTD_IWB) {
    if (!d->d_iwb_mask) {
      if (d->alloc((void**)&d->d_iwb_mask, (size_t)d->N * sizeof(uint32_t)) != cudaSuccess ||
          d->alloc((void**)&d->d_iwb_code, (size_t)d->N) != cudaSuccess)
        return fail(PFDTD_ERR_NOMEM, "IWB geometry allocation failed");
    }
    const int64_t gb = std::min<int64_t>((d->N + 255) / 256, kGridSMs * 32);
    k_iwb_geometry<<<(int)gb, 256, 0, s>>>(d->d_pos, d->N, d->X, d->XY, d->d_iwb_mask,
                                           d->d_iwb_code);
    count_launch();
    PFDTD_CK(cudaGetLastError());
    key_bytes = d->d_iwb_code;
  }
  const int64_t begin = d->XY, end = d->N - d->XY;
  if (end > begin) {
    const int64_t blocks = std::min<int64_t>((end - begin + 255) / 256, kGridSMs * 32);
    k_key_presence<<<(int)blocks, 256, 0, s>>>(key_bytes, d->d_mat, begin, end, d_present);
    count_launch();
    PFDTD_CK(cudaGetLastError());
  }
  std::vector<uint8_t> present(65536);
  PFDTD_CK(cudaMemcpyAsync(present.data(), d_present, 65536, cudaMemcpyDeviceToHost, s));
  PFDTD_CK(cudaStreamSynchronize(s));
  PFDTD_CK(cudaFreeAsync(d_present, s));
  std::vector<uint16_t> keys;
  std::vector<uint16_t> lut(65536, 0);
  for (int k = 0; k < 65536; ++k)
    if (present[k]) {
      lut[k] = (uint16_t)keys.size();
      keys.push_back((uint16_t)k);
    }
  if (keys.empty()) keys.push_back(0);  // grid without updated planes
  std::vector<uint8_t> tab;
  int rc = eval_class_coefs(d->precision, scheme, form, d->quirks, d->params, d->materials,
                            d->n_mat, d->n_coef, keys, tab);
  if (rc != PFDTD_OK) return rc;
  const int n_classes = (int)keys.size();
  const int cls_bytes = n_classes <= 256 ? 1 : 2;
  if (d->d_cls == nullptr || cls_bytes > d->cls_bytes) {
    d->release(d->d_cls);
    d->d_cls = nullptr;
    if (d->alloc(&d->d_cls, (size_t)d->N * cls_bytes + 64) != cudaSuccess)
      return fail(PFDTD_ERR_NOMEM, "class id allocation failed");
  }
  d->cls_bytes = cls_bytes;
  d->release(d->d_ctab);
  d->d_ctab = nullptr;
  PFDTD_CK(d->alloc(&d->d_ctab, tab.size()));
  PFDTD_CK(cudaMemcpyAsync(d->d_ctab, tab.data(), tab.size(), cudaMemcpyHostToDevice, s));
  uint16_t* d_lut = nullptr;
  PFDTD_CK(cudaMallocAsync((void**)&d_lut, 65536 * sizeof(uint16_t), s));
  PFDTD_CK(cudaMemcpyAsync(d_lut, lut.data(), 65536 * sizeof(uint16_t), cudaMemcpyHostToDevice, s));
  const int64_t blocks = std::min<int64_t>((d->N + 255) / 256, kGridSMs * 32);
  if (cls_bytes == 1)
    k_map_classes<uint8_t><<<(int)blocks, 256, 0, s>>>(key_bytes, d->d_mat, d->N, d_lut,
                                                        (uint8_t*)d->d_cls);
  else
    k_map_classes<uint16_t><<<(int)blocks, 256, 0, s>>>(key_bytes, d->d_mat, d->N, d_lut,
                                                         (uint16_t*)d->d_cls);
  count_launch();
  PFDTD_CK(cudaGetLastError());
  PFDTD_CK(cudaFreeAsync(d_lut, s));
  // The TMA kernels read the class ids through a 2-D tensor map whose row
  // stride must be a multiple of 16 bytes.  Where the field rows are 16-byte
  // aligned but the class-id rows (X ids) are not, they read a copy with each
  // row padded to 16 bytes.
  const int64_t cls_row = d->X * cls_bytes;
  if (cls_row % 16 != 0 && (d->X * d->K * (int64_t)d->esize) % 16 == 0) {
    const int64_t pitch = (cls_row + 15) / 16 * 16;
    const size_t need = (size_t)(pitch * d->Y * d->Z);
    if (!d->d_cls_tma || d->cls_tma_bytes < need) {
      d->release(d->d_cls_tma);
      d->d_cls_tma = nullptr;
      d->cls_tma_bytes = 0;
      if (d->alloc(&d->d_cls_tma, need) != cudaSuccess)
        return fail(PFDTD_ERR_NOMEM, "padded class-id allocation failed");
      d->cls_tma_bytes = need;
    }
    PFDTD_CK(cudaMemcpy2DAsync(d->d_cls_tma, (size_t)pitch, d->d_cls, (size_t)cls_row,
                               (size_t)cls_row, (size_t)(d->Y * d->Z), cudaMemcpyDeviceToDevice, s));
    d->cls_pitch = pitch / cls_bytes;
  } else {
    d->cls_pitch = 0;
  }
  PFDTD_CK(cudaStreamSynchronize(s));
  d->n_classes = n_classes;
  d->class_scheme = scheme;
  d->class_form = form;
  rc = build_dif(d, keys, tab);
  if (rc != PFDTD_OK) return rc;
  rc = build_iwb_closure(d, keys);
  if (rc != PFDTD_OK) return rc;
  rc = check_tb_faces(d);
  if (rc != PFDTD_OK) return rc;
  d->classes_dirty = false;
  d->class_version++;
  return PFDTD_OK;
}

}  // namespace pfdtd
