// Frequency-dependent (IIR admittance) boundary nodes.
//
// The reference only reserves room for digital impedance filters
// (src/kernels/cudaMesh.h:88, :122-123).  Here a material may carry
// Y(z) = (b0 + b1 z^-1 + b2 z^-2 + b3 z^-3) / (1 + a1 z^-1 + a2 z^-2 + a3 z^-3).
// At such a boundary node the loss term of the frequency-independent update,
// beta (p+ - p-) = 2 G Y x with x = (p+ - p-)/2 and G the node's geometric
// factor, becomes 2 G y with y = b0 x + s1 the filter output (transposed
// direct form II): the b0 part stays implicit (beta = G b0) and the state s1
// enters explicitly.
//
// The main update kernels treat every node with the FI rule; afterwards
// k_dif_update recomputes the DIF nodes (a sparse, ordered list) from the same
// P^n and overwrites them.  Because the main kernel has by then overwritten
// P^{n-1} at those nodes, each DIF node keeps its own previous value in its
// state (re-read from the past field at the start of every run or step).
// For IWB on the TMA path the closure pass (k_iwb_closure, which updates every
// node with a closed neighbour after the streaming update) stores each DIF
// node's weighted neighbour sum sw (d_iwb_sw), so this pass reads one value
// per node instead of gathering the 26 neighbours again.
#include "common.cuh"
#include "iwb_closure.cuh"

#include <cstdlib>

#include <algorithm>
#include <cstring>
#include <vector>

namespace pfdtd {
namespace {

constexpr int kChunkNodes = 4096;  // nodes per block when listing DIF nodes
constexpr int kListThreads = 256;


__global__ void k_dif_count(const void* __restrict__ cls, int cls_bytes,
                            const uint8_t* __restrict__ is_dif, int64_t begin, int64_t end,
                            int* __restrict__ counts) {
  const int64_t start = begin + (int64_t)blockIdx.x * kChunkNodes;
  int n = 0;
  for (int i = threadIdx.x; i < kChunkNodes; i += blockDim.x) {
    const int64_t j = start + i;
    if (j >= end) break;
    const unsigned c = cls_bytes == 1 ? ((const uint8_t*)cls)[j] : ((const uint16_t*)cls)[j];
    n += is_dif[c];
  }
  for (int o = 16; o > 0; o >>= 1) n += __shfl_down_sync(0xffffffffu, n, o);
  __shared__ int sn[kListThreads / 32];
  if ((threadIdx.x & 31) == 0) sn[threadIdx.x >> 5] = n;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < kListThreads / 32; ++w) t += sn[w];
    counts[blockIdx.x] = t;
  }
}

// Ordered write: thread t owns nodes [start + 16 t, start + 16 t + 16).
__global__ void k_dif_list(const void* __restrict__ cls, int cls_bytes,
                           const uint8_t* __restrict__ is_dif, int64_t begin, int64_t end,
                           const int* __restrict__ offsets, int64_t* __restrict__ list) {
  constexpr int per = kChunkNodes / kListThreads;
  const int64_t start = begin + (int64_t)blockIdx.x * kChunkNodes + (int64_t)threadIdx.x * per;
  int n = 0;
  for (int i = 0; i < per; ++i) {
    const int64_t j = start + i;
    if (j >= end) break;
    const unsigned c = cls_bytes == 1 ? ((const uint8_t*)cls)[j] : ((const uint16_t*)cls)[j];
    n += is_dif[c];
  }
  __shared__ int scan[kListThreads];
  scan[threadIdx.x] = n;
  __syncthreads();
  for (int o = 1; o < kListThreads; o <<= 1) {
    const int v = threadIdx.x >= o ? scan[threadIdx.x - o] : 0;
    __syncthreads();
    scan[threadIdx.x] += v;
    __syncthreads();
  }
  int k = offsets[blockIdx.x] + scan[threadIdx.x] - n;
  for (int i = 0; i < per; ++i) {
    const int64_t j = start + i;
    if (j >= end) break;
    const unsigned c = cls_bytes == 1 ? ((const uint8_t*)cls)[j] : ((const uint16_t*)cls)[j];
    if (is_dif[c]) list[k++] = j;
  }
}

// prev <- P^{n-1} at each DIF node (start of a run or step).
// (n counts DIF nodes times fields; entry k is field k & (K-1) of DIF node
// k >> kshift.)
template <typename S>
__global__ void k_dif_init_prev(const int64_t* __restrict__ list, int64_t n, int kshift,
                                const S* __restrict__ past, typename Store<S>::A* __restrict__ st) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = (list[k >> kshift] << kshift) + (k & ((1 << kshift) - 1));
    st[4 * k + 3] = Store<S>::load(past[e]);
  }
}

template <typename S, int SCHEME>
__global__ void k_dif_update(const int64_t* __restrict__ list, int64_t n, int kshift,
                             const void* __restrict__ cls, int cls_bytes,
                             const typename Store<S>::A* __restrict__ dtab, const S* __restrict__ P,
                             S* __restrict__ Pp, typename Store<S>::A* __restrict__ st, int64_t X,
                             int64_t XY, typename Store<S>::A l2, const uint32_t* __restrict__ cpos,
                             const uint32_t* __restrict__ iwb_mask,
                             const float* __restrict__ iwb_sw) {
  using A = typename Store<S>::A;
  using R = Rn<A>;
  using Sto = Store<S>;
  // X, XY count field elements; the x neighbour is K elements away.
  const int64_t ks = (int64_t)1 << kshift;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t node = list[k >> kshift];
    const int64_t i = (node << kshift) + (k & (ks - 1));
    const unsigned c = cls_bytes == 1 ? ((const uint8_t*)cls)[node] : ((const uint16_t*)cls)[node];
    const A* t = dtab + (int64_t)kDifClassVals * c;
    const A a = t[0], b = t[1], cc = t[2], g2 = t[3];
    A* s = st + 4 * k;
    const A pp = s[3];
    const A s1 = s[0];
    const A p = Sto::load(P[i]);
    A num;
    if (SCHEME == 0) {
      const A s6 = R::add(R::add(R::add(R::add(R::add(Sto::load(P[i + XY]), Sto::load(P[i - XY])),
                                                  Sto::load(P[i + X])), Sto::load(P[i - X])),
                                  Sto::load(P[i + ks])), Sto::load(P[i - ks]));
      num = R::sub(R::sub(R::add(R::mul(b, p), R::mul(l2, s6)), R::mul(cc, pp)), R::mul(g2, s1));
    } else if (SCHEME == 1) {
      const uint32_t cp = cpos[c];
      const A xm = Sto::load(P[i - ks]), xp = Sto::load(P[i + ks]);
      const A ym = Sto::load(P[i - X]), yp = Sto::load(P[i + X]);
      const A zm = Sto::load(P[i - XY]), zp = Sto::load(P[i + XY]);
      const A dx = (A)(cp & 1u), dy = (A)((cp >> 1) & 1u), dz = (A)((cp >> 2) & 1u);
      const A bx = (cp & 0x10u) ? xp : xm;
      const A by = (cp & 0x20u) ? yp : ym;
      const A bz = (cp & 0x40u) ? zm : zp;
      const A sb6 = R::add(R::add(R::mul(bx, dx), R::mul(by, dy)), R::mul(bz, dz));
      const A s7 = R::add(R::add(R::add(R::add(R::add(R::add(xm, xp), ym), yp), zp), zm), sb6);
      num = R::sub(R::add(R::sub(R::mul(s7, l2), R::mul(b, p)), R::mul(cc, pp)), R::mul(g2, s1));
    } else {
      // IWB: closed neighbours (mask bits, canonical order) contribute p.
      // The TMA update kernel has already formed sw for this node (same
      // sums, same rounding) when iwb_sw is given.
      A sw;
      if (iwb_sw != nullptr) {
        sw = (A)iwb_sw[node];
      } else {
        const uint32_t mk = iwb_mask[node];
        A m[3][3][3];
        int kk = 0;
        for (int dz = -1; dz <= 1; ++dz)
          for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
              A v = p;
              if (dx != 0 || dy != 0 || dz != 0) {
                if (!((mk >> kk) & 1u)) v = Sto::load(P[i + dz * XY + dy * X + dx * ks]);
                ++kk;
              }
              m[dz + 1][dy + 1][dx + 1] = v;
            }
        A f1, f2, f3;
        iwb_sums(m, f1, f2, f3);
        sw = R::mul(l2, R::add(R::add(R::mul(f1, (A)0.25), R::mul(f2, (A)0.125)),
                               R::mul(f3, (A)0.0625)));
      }
      num = R::sub(R::sub(R::add(sw, R::mul(b, p)), R::mul(cc, pp)), R::mul(g2, s1));
    }
    const A out = R::mul(a, num);
    // Filter state update (transposed direct form II).
    const A x = R::mul(R::sub(out, pp), (A)0.5);
    const A y = R::add(R::mul(t[4], x), s1);
    s[0] = R::add(R::sub(R::mul(t[5], x), R::mul(t[8], y)), s[1]);
    s[1] = R::add(R::sub(R::mul(t[6], x), R::mul(t[9], y)), s[2]);
    s[2] = R::sub(R::mul(t[7], x), R::mul(t[10], y));
    s[3] = p;
    Pp[i] = Sto::store(out);
  }
}

// IWB closure nodes on the TMA path (no counterpart in the reference): the
// update kernel has left P^{n-1} at every node whose class has a closed
// neighbour (bit 30 of the pos word); this pass updates them with the
// finite-volume closure, operation for operation as k_update_iwb and the
// oracle's iwb_node: a closed neighbour (bit k of the node's mask, canonical
// order) contributes the node's own value, the sums follow iwb_sums, and the
// neighbours are read at their flat offsets.  For a DIF node (bit 31) it
// also stores sw for the DIF pass that follows.
//
// One record per node (index, mask and class read together).  All 26
// neighbours are loaded before the substitution so that a thread has them
// in flight at once: the flat offsets of a node of planes 1..Z-2 stay within
// the field's margins (at least X + 64 elements each side), and a closed
// neighbour's value (outside the grid or in a margin) is replaced by a
// select, never used in arithmetic.

__global__ void k_closure_records(const int64_t* __restrict__ list, int64_t n,
                                  const void* __restrict__ cls, int cls_bytes,
                                  const uint32_t* __restrict__ mask, ClosureRec* __restrict__ rec) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = list[k];
    const unsigned c = cls_bytes == 1 ? ((const uint8_t*)cls)[i] : ((const uint16_t*)cls)[i];
    rec[k] = ClosureRec{i, mask[i], c};
  }
}

// dif_slot (optional): per record the node's position in the DIF list, -1
// for a node without a filter.  A DIF node then takes the DIF update here,
// operation for operation as k_dif_update with the same sw (and its filter
// state at dstate + 4 * slot), instead of the FI rule and the separate pass.
// For each DIF node (flat index order), the record holding it: a binary
// search in the records' ascending indices.  A DIF node without a record
// (none is expected: a DIF node has a closed face neighbour) is counted.
__global__ void k_closure_dif_slots(const int64_t* __restrict__ dif_list, int64_t n_dif,
                                    const ClosureRec* __restrict__ recs, int64_t n_rec,
                                    int32_t* __restrict__ slot, unsigned* __restrict__ missing) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n_dif;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t node = dif_list[k];
    int64_t lo = 0, hi = n_rec;
    while (lo < hi) {
      const int64_t mid = lo + (hi - lo) / 2;
      if (recs[mid].idx < node) lo = mid + 1;
      else hi = mid;
    }
    if (lo < n_rec && recs[lo].idx == node) slot[lo] = (int32_t)k;
    else atomicAdd(missing, 1u);
  }
}

template <typename S>
__global__ void __launch_bounds__(256)
k_iwb_closure(const ClosureRec* __restrict__ recs, int64_t n, ClassTab<float> tab,
              const S* __restrict__ P, S* __restrict__ Pp, int64_t X, int64_t XY, float l2,
              float* __restrict__ iwb_sw, const int32_t* __restrict__ dif_slot,
              const float* __restrict__ dtab, float* __restrict__ dstate) {
  using Sto = Store<S>;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    const ClosureRec r = recs[k];
    const int64_t i = r.idx;
    float m[3][3][3];
#pragma unroll
    for (int dz = -1; dz <= 1; ++dz)
#pragma unroll
      for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
        for (int dx = -1; dx <= 1; ++dx)
          m[dz + 1][dy + 1][dx + 1] = Sto::load(__ldg(P + i + dz * XY + dy * X + dx));
    const float pp = Sto::load(Pp[i]);
    const int32_t slot = dif_slot != nullptr ? dif_slot[k] : -1;
    iwb_closure_apply<S>(m, r.mask, r.cls, pp, tab, l2, slot, dtab, dstate, iwb_sw, i, Pp);
  }
}

// Ordered list of the nodes of planes 1..Z-2 whose class is flagged; *list
// is allocated (stream-ordered) when there is at least one.
int build_flagged_list(pfdtd_domain* d, const std::vector<uint8_t>& flag, int64_t** list,
                       int64_t* count) {
  *list = nullptr;
  *count = 0;
  if (std::find(flag.begin(), flag.end(), 1) == flag.end()) return PFDTD_OK;
  cudaStream_t s = d->stream;
  const int64_t begin = d->XY, end = d->N - d->XY;
  if (end <= begin) return PFDTD_OK;
  const int64_t blocks = (end - begin + kChunkNodes - 1) / kChunkNodes;
  uint8_t* d_is = nullptr;
  int* d_counts = nullptr;
  PFDTD_CK(d->alloc((void**)&d_is, flag.size()));
  PFDTD_CK(d->alloc((void**)&d_counts, sizeof(int) * (blocks + 1)));
  PFDTD_CK(cudaMemcpyAsync(d_is, flag.data(), flag.size(), cudaMemcpyHostToDevice, s));
  k_dif_count<<<(int)blocks, kListThreads, 0, s>>>(d->d_cls, d->cls_bytes, d_is, begin, end,
                                                  d_counts);
  count_launch();
  std::vector<int> counts(blocks);
  PFDTD_CK(cudaMemcpyAsync(counts.data(), d_counts, sizeof(int) * blocks, cudaMemcpyDeviceToHost, s));
  PFDTD_CK(cudaStreamSynchronize(s));
  std::vector<int> offsets(blocks);
  int64_t total = 0;
  for (int64_t b = 0; b < blocks; ++b) {
    offsets[b] = (int)total;
    total += counts[b];
  }
  if (total > 0) {
    PFDTD_CK(cudaMemcpyAsync(d_counts, offsets.data(), sizeof(int) * blocks, cudaMemcpyHostToDevice, s));
    PFDTD_CK(d->alloc((void**)list, sizeof(int64_t) * total));
    k_dif_list<<<(int)blocks, kListThreads, 0, s>>>(d->d_cls, d->cls_bytes, d_is, begin, end,
                                                   d_counts, *list);
    count_launch();
    PFDTD_CK(cudaGetLastError());
  }
  PFDTD_CK(cudaStreamSynchronize(s));
  d->release(d_is);
  d->release(d_counts);
  *count = total;
  return PFDTD_OK;
}

int grid_for(int64_t n) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, kGridSMs * 16));
}

template <typename A>
void eval_dif_classes(const pfdtd_domain* d, int scheme, const std::vector<uint16_t>& keys,
                      const std::vector<uint8_t>& main_tab, std::vector<uint8_t>& is_dif,
                      std::vector<A>& dtab) {
  const size_t n = keys.size();
  const A* mb = (const A*)(main_tab.data() + n * sizeof(A));  // b coefficients
  const A l = (A)d->params[0];
  is_dif.assign(n, 0);
  dtab.assign(n * kDifClassVals, (A)0);
  for (size_t i = 0; i < n; ++i) {
    const unsigned pos = keys[i] >> 8, m = keys[i] & 0xFFu;
    const bool inside = scheme == PFDTD_IWB ? pos != 0 : (pos >> 7) != 0;
    if (!inside || m >= d->dif_flags.size() || !d->dif_flags[m]) continue;
    A G;
    if (scheme == PFDTD_SRL_FORWARD)
      G = (A)0.5 * (((A)6 - (A)(pos & 0x7Fu)) * l);
    else if (scheme == PFDTD_IWB)  // pos is the geometry code
      G = pos >= 65 ? l * ((A)(int)(pos - 65) * (A)0.0625) : (A)0;
    else
      G = l * (A)((pos & 1u) + ((pos >> 1) & 1u) + ((pos >> 2) & 1u));
    if (!(G > (A)0)) continue;
    const double* f = &d->dif_coefs[7 * m];
    const A b0 = (A)f[0];
    const A beta = G * b0;
    A* t = &dtab[i * kDifClassVals];
    t[0] = (A)1 * ((A)1 / ((A)1 + beta));  // inside switch is 1 for DIF nodes
    t[1] = mb[i];
    t[2] = (scheme == PFDTD_SRL) ? beta - (A)1 : (A)1 - beta;
    t[3] = (A)2 * G;
    for (int j = 0; j < 7; ++j) t[4 + j] = (A)f[j];
    is_dif[i] = 1;
  }
}

template <typename S>
int launch_dif_t(pfdtd_domain* d, const void* cur, void* past, cudaStream_t s) {
  using A = typename Store<S>::A;
  const size_t as = sizeof(A);
  const uint32_t* cpos = (const uint32_t*)((const char*)d->d_ctab + 3 * as * d->n_classes);
  const A l2 = (A)d->params[1];
  const int64_t n = d->n_dif * d->K;
  const int64_t XE = d->X * d->K, XYE = d->XY * d->K;
  const int g = grid_for(n);
  const float* iwb_sw =
      (d->class_scheme == PFDTD_IWB && d->d_iwb_sw && uses_tma(d)) ? d->d_iwb_sw : nullptr;
  switch (d->class_scheme) {
    case PFDTD_SRL:
      k_dif_update<S, 1><<<g, 256, 0, s>>>(d->d_dif_list, n, d->kshift, d->d_cls, d->cls_bytes,
                                           (const A*)d->d_dif_tab, (const S*)cur, (S*)past,
                                           (A*)d->d_dif_state, XE, XYE, l2, cpos,
                                           d->d_iwb_mask, iwb_sw);
      break;
    case PFDTD_IWB:
      k_dif_update<S, 2><<<g, 256, 0, s>>>(d->d_dif_list, n, d->kshift, d->d_cls, d->cls_bytes,
                                           (const A*)d->d_dif_tab, (const S*)cur, (S*)past,
                                           (A*)d->d_dif_state, XE, XYE, l2, cpos,
                                           d->d_iwb_mask, iwb_sw);
      break;
    default:
      k_dif_update<S, 0><<<g, 256, 0, s>>>(d->d_dif_list, n, d->kshift, d->d_cls, d->cls_bytes,
                                           (const A*)d->d_dif_tab, (const S*)cur, (S*)past,
                                           (A*)d->d_dif_state, XE, XYE, l2, cpos,
                                           d->d_iwb_mask, iwb_sw);
  }
  count_launch();
  PFDTD_CK(cudaGetLastError());
  return PFDTD_OK;
}

template <typename S>
int launch_init_t(pfdtd_domain* d, cudaStream_t s) {
  using A = typename Store<S>::A;
  const int64_t n = d->n_dif * d->K;
  k_dif_init_prev<S><<<grid_for(n), 256, 0, s>>>(d->d_dif_list, n, d->kshift,
                                                 (const S*)d->past_field(), (A*)d->d_dif_state);
  count_launch();
  PFDTD_CK(cudaGetLastError());
  return PFDTD_OK;
}

}  // namespace

// Build the DIF class table and the ordered DIF node list after the classes
// were (re)built.  keys/main_tab: the class keys and coefficient table.
int build_dif(pfdtd_domain* d, const std::vector<uint16_t>& keys,
              const std::vector<uint8_t>& main_tab) {
  for (void** p : {(void**)&d->d_dif_list, &d->d_dif_tab, &d->d_dif_state})
    if (*p) {
      d->release(*p);
      *p = nullptr;
    }
  d->n_dif = 0;
  if (d->dif_flags.empty()) return PFDTD_OK;
  std::vector<uint8_t> is_dif;
  std::vector<uint8_t> tab_bytes;
  if (d->precision == PFDTD_F64) {
    std::vector<double> t;
    eval_dif_classes<double>(d, d->class_scheme, keys, main_tab, is_dif, t);
    tab_bytes.assign((uint8_t*)t.data(), (uint8_t*)(t.data() + t.size()));
  } else {
    std::vector<float> t;
    eval_dif_classes<float>(d, d->class_scheme, keys, main_tab, is_dif, t);
    tab_bytes.assign((uint8_t*)t.data(), (uint8_t*)(t.data() + t.size()));
  }
  cudaStream_t s = d->stream;
  int64_t total = 0;
  if (int rc = build_flagged_list(d, is_dif, &d->d_dif_list, &total)) return rc;
  if (total > 0) {
    PFDTD_CK(d->alloc(&d->d_dif_tab, tab_bytes.size()));
    PFDTD_CK(cudaMemcpyAsync(d->d_dif_tab, tab_bytes.data(), tab_bytes.size(),
                             cudaMemcpyHostToDevice, s));
    const size_t sbytes = (size_t)total * d->K * 4 * d->arith_size();
    PFDTD_CK(d->alloc(&d->d_dif_state, sbytes));
    PFDTD_CK(cudaMemsetAsync(d->d_dif_state, 0, sbytes, s));
    if (d->class_scheme == PFDTD_IWB && d->K == 1 && d->precision != PFDTD_F64) {
      // flag the DIF classes (bit 31 of the pos word, unused by the IWB
      // kernels) so that the TMA update or the closure pass stores their sw
      // for the DIF pass
      const size_t n = keys.size(), as = d->arith_size();
      std::vector<uint32_t> pos(n);
      std::memcpy(pos.data(), main_tab.data() + 3 * n * as, n * sizeof(uint32_t));
      for (size_t i = 0; i < n; ++i)
        if (is_dif[i]) pos[i] |= 0x80000000u;
      PFDTD_CK(cudaMemcpyAsync((char*)d->d_ctab + 3 * n * as, pos.data(), n * sizeof(uint32_t),
                               cudaMemcpyHostToDevice, s));
      if (!d->d_iwb_sw) PFDTD_CK(d->alloc((void**)&d->d_iwb_sw, (size_t)d->N * sizeof(float)));
    }
    PFDTD_CK(cudaStreamSynchronize(s));
  }
  d->n_dif = total;
  return PFDTD_OK;
}

// The DIF slot of every closure record, so that the closure pass applies the
// DIF update itself.  Only an optimisation: returns nullptr (and the separate
// DIF pass stays in use) if any DIF node has no record or anything fails, with
// every temporary released and the CUDA error cleared.
static int32_t* closure_dif_slots(pfdtd_domain* d, int64_t n) {
  cudaStream_t s = d->stream;
  int32_t* slot = nullptr;
  unsigned* d_missing = nullptr;
  unsigned missing = 1;
  cudaError_t e = d->alloc((void**)&slot, sizeof(int32_t) * (size_t)n);
  if (e == cudaSuccess) e = d->alloc((void**)&d_missing, sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMemsetAsync(slot, 0xFF, sizeof(int32_t) * (size_t)n, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_missing, 0, sizeof(unsigned), s);
  if (e == cudaSuccess) {
    k_closure_dif_slots<<<grid_for(d->n_dif), 256, 0, s>>>(
        d->d_dif_list, d->n_dif, (const ClosureRec*)d->d_iwb_closure, n, slot, d_missing);
    count_launch();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&missing, d_missing, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (d_missing) d->release(d_missing);
  if (e != cudaSuccess || missing != 0) {
    if (e != cudaSuccess) cudaGetLastError();
    if (slot) d->release(slot);
    return nullptr;
  }
  return slot;
}

// The closure-node list of an IWB domain on the TMA path (one field per
// node, FP32/FP16/BF16 storage): classes whose geometry code is >= 2.
int build_iwb_closure(pfdtd_domain* d, const std::vector<uint16_t>& keys) {
  if (d->d_iwb_closure) d->release(d->d_iwb_closure);
  d->d_iwb_closure = nullptr;
  if (d->d_iwb_closure_dif) d->release(d->d_iwb_closure_dif);
  d->d_iwb_closure_dif = nullptr;
  d->n_iwb_closure = 0;
  d->iwb_closure_ready = false;
  if (d->class_scheme != PFDTD_IWB || d->K != 1 || d->precision == PFDTD_F64) return PFDTD_OK;
  std::vector<uint8_t> flag(keys.size());
  for (size_t i = 0; i < keys.size(); ++i) flag[i] = (keys[i] >> 8) >= 2 ? 1 : 0;
  int64_t* list = nullptr;
  int64_t n = 0;
  if (int rc = build_flagged_list(d, flag, &list, &n)) return rc;
  if (n > 0) {
    cudaStream_t s = d->stream;
    cudaError_t e = d->alloc(&d->d_iwb_closure, sizeof(ClosureRec) * (size_t)n);
    if (e != cudaSuccess) {
      d->release(list);
      d->d_iwb_closure = nullptr;
      return cuda_fail(e, "IWB closure records", __FILE__, __LINE__);
    }
    k_closure_records<<<grid_for(n), 256, 0, s>>>(list, n, d->d_cls, d->cls_bytes, d->d_iwb_mask,
                                                  (ClosureRec*)d->d_iwb_closure);
    count_launch();
    e = cudaGetLastError();
    d->release(list);
    if (e != cudaSuccess) return cuda_fail(e, "k_closure_records", __FILE__, __LINE__);
    // PFDTD_IWB_DIF_UNFUSED=1 keeps the DIF update in its own pass (a test
    // hook: both paths give the same result bit for bit).
    const char* unfused = std::getenv("PFDTD_IWB_DIF_UNFUSED");
    if (d->n_dif > 0 && d->n_dif < ((int64_t)1 << 31) && d->d_dif_list &&
        !(unfused && unfused[0] == '1'))
      d->d_iwb_closure_dif = closure_dif_slots(d, n);
  }
  d->n_iwb_closure = n;
  d->iwb_closure_ready = true;
  return PFDTD_OK;
}

template <typename S>
int launch_closure_t(pfdtd_domain* d, const void* cur, void* past, cudaStream_t s) {
  const int64_t n = d->n_iwb_closure;
  const uint8_t* ctab = (const uint8_t*)d->d_ctab;
  const int nc = d->n_classes;
  ClassTab<float> tab{(const float*)ctab, (const float*)(ctab + (size_t)nc * 4),
                      (const float*)(ctab + 2 * (size_t)nc * 4),
                      (const uint32_t*)(ctab + 3 * (size_t)nc * 4), nc};
  const bool fuse = iwb_closure_fuses_dif(d);
  k_iwb_closure<S><<<grid_for(n), 256, 0, s>>>(
      (const ClosureRec*)d->d_iwb_closure, n, tab, (const S*)cur, (S*)past, d->X, d->XY,
      (float)d->params[1], (d->n_dif > 0 && !fuse) ? d->d_iwb_sw : nullptr,
      fuse ? d->d_iwb_closure_dif : nullptr, fuse ? (const float*)d->d_dif_tab : nullptr,
      fuse ? (float*)d->d_dif_state : nullptr);
  count_launch();
  PFDTD_CK(cudaGetLastError());
  return PFDTD_OK;
}

int launch_iwb_closure(pfdtd_domain* d, const void* cur, void* past, cudaStream_t s) {
  if (!d->iwb_closure_ready) return fail(PFDTD_ERR_STATE, "IWB closure list not built");
  if (d->n_iwb_closure <= 0) return PFDTD_OK;
  switch (d->precision) {
    case PFDTD_F32: return launch_closure_t<float>(d, cur, past, s);
    case PFDTD_F16: return launch_closure_t<__half>(d, cur, past, s);
    case PFDTD_BF16: return launch_closure_t<__nv_bfloat16>(d, cur, past, s);
  }
  return fail(PFDTD_ERR_UNSUPPORTED, "IWB closure pass needs FP32, FP16 or BF16 fields");
}

int launch_dif(pfdtd_domain* d, const void* cur, void* past, cudaStream_t s) {
  if (d->n_dif <= 0) return PFDTD_OK;
  if (iwb_closure_fuses_dif(d)) return PFDTD_OK;  // the closure pass applied it
  switch (d->precision) {
    case PFDTD_F32: return launch_dif_t<float>(d, cur, past, s);
    case PFDTD_F64: return launch_dif_t<double>(d, cur, past, s);
    case PFDTD_F16: return launch_dif_t<__half>(d, cur, past, s);
    case PFDTD_BF16: return launch_dif_t<__nv_bfloat16>(d, cur, past, s);
  }
  return fail(PFDTD_ERR_UNSUPPORTED, "unknown precision");
}

int launch_dif_init(pfdtd_domain* d, cudaStream_t s) {
  if (d->n_dif <= 0) return PFDTD_OK;
  switch (d->precision) {
    case PFDTD_F32: return launch_init_t<float>(d, s);
    case PFDTD_F64: return launch_init_t<double>(d, s);
    case PFDTD_F16: return launch_init_t<__half>(d, s);
    case PFDTD_BF16: return launch_init_t<__nv_bfloat16>(d, s);
  }
  return fail(PFDTD_ERR_UNSUPPORTED, "unknown precision");
}

}  // namespace pfdtd
