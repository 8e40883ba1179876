// Device-side mesh set-up and capture: scheme translation of voxelizer ids,
// air/boundary counts, block padding and slice gathers.
#include "common.cuh"

#include <algorithm>

namespace pfdtd {
namespace {

// Voxelizer id 0..27 -> centred DIR/SIGN byte, the values of
// src/kernels/cudaMesh.cu:363-480 in table form.
#define PFDTD_KOWALCZYK_BYTES                                                                 \
  {0x00, 0xC7, 0xD7, 0xE7, 0xF7, 0x87, 0x97, 0xA7, 0xB7, 0xC6, 0xE6, 0xC5, 0xD5, 0x86,           \
   0xA6, 0x85, 0x95, 0x83, 0x93, 0xA3, 0xB3, 0xC4, 0xA2, 0x82, 0x91, 0x81, 0x84, 0x80}
__constant__ uint8_t c_kowalczyk[28] = PFDTD_KOWALCZYK_BYTES;
const uint8_t h_kowalczyk[28] = PFDTD_KOWALCZYK_BYTES;

// toBilbao / toKowalczyk applied per node (cudaMesh.cu:482-498).
__global__ void k_encode(int centred, uint8_t* __restrict__ pos, uint8_t* __restrict__ mat,
                         int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const unsigned k = pos[i];
    if (k == 0) {
      pos[i] = 0;
      mat[i] = 0;
    } else if (k <= 27) {
      if (centred) {
        pos[i] = c_kowalczyk[k];
      } else {
        const unsigned kk = k <= 8 ? 3u : (k <= 20 ? 4u : (k <= 26 ? 5u : 6u));
        pos[i] = (uint8_t)(kk | 0x80u);
      }
    }
  }
}

// calcBoundaries (cudaMesh.cu:500-514) with a block reduction.
__global__ void k_count(const uint8_t* __restrict__ pos, int64_t n, uint8_t air_value,
                        uint8_t outside_value, unsigned long long* __restrict__ counts) {
  unsigned long long a = 0, b = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const uint8_t p = pos[i];
    a += (p == air_value);
    b += (p != outside_value && p != air_value);
  }
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  __shared__ unsigned long long sa[32], sb[32];
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) { sa[w] = a; sb[w] = b; }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long ta = 0, tb = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) { ta += sa[i]; tb += sb[i]; }
    atomicAdd(&counts[0], ta);
    atomicAdd(&counts[1], tb);
  }
}

// padWithZerosKernel (cudaMesh.cu:516-534): new[z][y][x] = old[flat old
// index] for 0 < x <= dim_x, 0 < y <= dim_y, 0 < z, inside the new grid.
// Reads past the old buffer's readable length yield 0.
__global__ void k_pad(const uint8_t* __restrict__ in, int64_t in_len, uint32_t dx, uint32_t dy,
                      uint32_t dz, uint32_t px, uint32_t py, uint8_t* __restrict__ out) {
  const uint64_t nx = dx + px, ny = dy + py;
  const uint64_t total = nx * ny * (uint64_t)dz;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t x = i % nx, y = (i / nx) % ny, z = i / (nx * ny);
    if (x < (uint64_t)dx + 1 && x > 0 && y < (uint64_t)dy + 1 && y > 0 && z > 0) {
      const uint64_t old_idx = z * dx * dy + y * dx + x;
      const uint64_t new_idx = z * nx * ny + y * nx + x;
      out[new_idx] = old_idx < (uint64_t)in_len ? in[old_idx] : 0;
    }
  }
}

// Slice gather as captureSliceKernel (visualizationUtils.cu:500-527): for
// xz and yz the reference's limit (dim * (partition size - 1)) leaves the
// last z row uncaptured; that row is left 0 here too.
template <typename S>
__global__ void k_slice(const S* __restrict__ P, const uint8_t* __restrict__ pos, int X, int Y,
                        int Z, int orientation, int64_t slice, float* __restrict__ p_out,
                        uint8_t* __restrict__ pos_out, int K) {
  const int64_t w = orientation == 0 ? X : (orientation == 1 ? X : Y);
  const int64_t h = orientation == 0 ? Y : Z;
  const int64_t XY = (int64_t)X * Y;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < w * h;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t u = i % w, v = i / w;
    int64_t src;
    if (orientation == 0) src = slice * XY + v * X + u;
    else if (orientation == 1) src = v * XY + slice * X + u;
    else src = v * XY + u * X + slice;
    const bool keep = orientation == 0 || v < Z - 1;
    if (p_out) p_out[i] = keep ? (float)Store<S>::load(P[src * K]) : 0.f;
    if (pos_out) pos_out[i] = keep ? pos[src] : 0;
  }
}

int grid_for(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, kGridSMs * 16)); }

struct DevGuard {
  int prev = -1;
  explicit DevGuard(int dev) { cudaGetDevice(&prev); if (prev != dev) cudaSetDevice(dev); }
  ~DevGuard() { if (prev >= 0) cudaSetDevice(prev); }
};

}  // namespace

// Slice gather of the domain's current field into device buffers (either may
// be null), queued on stream s; no allocation, no synchronisation.
int launch_slice_gather(pfdtd_domain* d, int orientation, int64_t slice, float* dp, uint8_t* dq,
                        cudaStream_t s) {
  const int64_t w = orientation == 2 ? d->Y : d->X;
  const int64_t h = orientation == 0 ? d->Y : d->Z;
  const int64_t n = w * h;
  const void* cur = d->cur_field();
  switch (d->precision) {
    case PFDTD_F32: k_slice<float><<<grid_for(n), 256, 0, s>>>((const float*)cur, d->d_pos, (int)d->X, (int)d->Y, (int)d->Z, orientation, slice, dp, dq, d->K); break;
    case PFDTD_F64: k_slice<double><<<grid_for(n), 256, 0, s>>>((const double*)cur, d->d_pos, (int)d->X, (int)d->Y, (int)d->Z, orientation, slice, dp, dq, d->K); break;
    case PFDTD_F16: k_slice<__half><<<grid_for(n), 256, 0, s>>>((const __half*)cur, d->d_pos, (int)d->X, (int)d->Y, (int)d->Z, orientation, slice, dp, dq, d->K); break;
    default: k_slice<__nv_bfloat16><<<grid_for(n), 256, 0, s>>>((const __nv_bfloat16*)cur, d->d_pos, (int)d->X, (int)d->Y, (int)d->Z, orientation, slice, dp, dq, d->K); break;
  }
  count_launch();
  PFDTD_CK(cudaGetLastError());
  return PFDTD_OK;
}

}  // namespace pfdtd

using namespace pfdtd;

extern "C" {

int pfdtd_encode_nodes_host(int centred, uint8_t* pos, uint8_t* mat, int64_t n) {
  if ((!pos || !mat) && n > 0) return fail(PFDTD_ERR_ARG, "invalid node arrays");
  for (int64_t i = 0; i < n; ++i) {
    const unsigned k = pos[i];
    if (k == 0) {
      mat[i] = 0;
    } else if (k <= 27) {
      if (centred) pos[i] = h_kowalczyk[k];
      else pos[i] = (uint8_t)((k <= 8 ? 3u : (k <= 20 ? 4u : (k <= 26 ? 5u : 6u))) | 0x80u);
    }
  }
  return PFDTD_OK;
}

int pfdtd_encode_nodes(int centred, uint8_t* d_pos, uint8_t* d_mat, int64_t n, int device) {
  if (!d_pos || !d_mat || n < 0) return fail(PFDTD_ERR_ARG, "invalid node arrays");
  if (n == 0) return PFDTD_OK;
  DevGuard g(device);
  k_encode<<<grid_for(n), 256>>>(centred, d_pos, d_mat, n);
  count_launch();
  PFDTD_CK(cudaGetLastError());
  PFDTD_CK(cudaDeviceSynchronize());
  return PFDTD_OK;
}

int pfdtd_count_boundaries(const uint8_t* d_pos, int64_t n, uint8_t air_value,
                           uint8_t outside_value, int device, uint32_t* air,
                           uint32_t* boundary) {
  if (!d_pos || n < 0 || !air || !boundary) return fail(PFDTD_ERR_ARG, "invalid arguments");
  DevGuard g(device);
  unsigned long long* d_counts = nullptr;
  // stream-ordered scratch on the legacy stream: no device-wide synchronisation
  PFDTD_CK(cudaMallocAsync((void**)&d_counts, 2 * sizeof(unsigned long long), 0));
  PFDTD_CK(cudaMemsetAsync(d_counts, 0, 2 * sizeof(unsigned long long), 0));
  if (n > 0) {
    k_count<<<grid_for(n), 256>>>(d_pos, n, air_value, outside_value, d_counts);
    count_launch();
  }
  cudaError_t e = cudaGetLastError();
  unsigned long long h[2] = {0, 0};
  if (e == cudaSuccess) e = cudaMemcpy(h, d_counts, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFreeAsync(d_counts, 0);
  if (e != cudaSuccess) return cuda_fail(e, "boundary count", __FILE__, __LINE__);
  *air = (uint32_t)h[0];
  *boundary = (uint32_t)h[1];
  return PFDTD_OK;
}

int pfdtd_pad_mesh(const uint8_t* d_in, int64_t in_len, const uint32_t dims[3], uint32_t bx,
                   uint32_t by, uint32_t bz, uint8_t* d_out, uint32_t out_dims[3], int device) {
  if (!dims || !out_dims || bx == 0 || by == 0 || bz == 0)
    return fail(PFDTD_ERR_ARG, "invalid padding arguments");
  const uint32_t dx = dims[0], dy = dims[1], dz = dims[2];
  const uint32_t px = dx % bx ? bx - dx % bx : 0;
  const uint32_t py = dy % by ? by - dy % by : 0;
  const uint32_t pz = dz % bz ? bz - dz % bz : 0;
  out_dims[0] = dx + px;
  out_dims[1] = dy + py;
  out_dims[2] = dz + pz;
  if (!d_out) return PFDTD_OK;
  if (!d_in) return fail(PFDTD_ERR_ARG, "null input mesh");
  DevGuard g(device);
  const uint64_t total = (uint64_t)out_dims[0] * out_dims[1] * out_dims[2];
  PFDTD_CK(cudaMemset(d_out, 0, total));
  k_pad<<<grid_for((int64_t)total), 256>>>(d_in, in_len, dx, dy, dz, px, py, d_out);
  count_launch();
  PFDTD_CK(cudaGetLastError());
  PFDTD_CK(cudaDeviceSynchronize());
  return PFDTD_OK;
}

int pfdtd_capture_slice(pfdtd_domain* d, int orientation, int64_t slice, float* p_out,
                        uint8_t* pos_out) {
  if (!d) return fail(PFDTD_ERR_ARG, "null domain");
  if (orientation < 0 || orientation > 2) return fail(PFDTD_ERR_ARG, "orientation must be 0, 1 or 2");
  const int64_t lim = orientation == 0 ? d->Z : (orientation == 1 ? d->Y : d->X);
  if (slice < 0 || slice >= lim) return fail(PFDTD_ERR_ARG, "slice outside the grid, no capture made");
  const int64_t w = orientation == 2 ? d->Y : d->X;
  const int64_t h = orientation == 0 ? d->Y : d->Z;
  const int64_t n = w * h;
  DevGuard g(d->device);
  cudaStream_t s = d->stream;
  float* dp = nullptr;
  uint8_t* dq = nullptr;
  PFDTD_CK(cudaMallocAsync((void**)&dp, n * sizeof(float), s));
  PFDTD_CK(cudaMallocAsync((void**)&dq, n, s));
  const void* cur = d->cur_field();
  switch (d->precision) {
    case PFDTD_F32: k_slice<float><<<grid_for(n), 256, 0, s>>>((const float*)cur, d->d_pos, (int)d->X, (int)d->Y, (int)d->Z, orientation, slice, dp, dq, d->K); break;
    case PFDTD_F64: k_slice<double><<<grid_for(n), 256, 0, s>>>((const double*)cur, d->d_pos, (int)d->X, (int)d->Y, (int)d->Z, orientation, slice, dp, dq, d->K); break;
    case PFDTD_F16: k_slice<__half><<<grid_for(n), 256, 0, s>>>((const __half*)cur, d->d_pos, (int)d->X, (int)d->Y, (int)d->Z, orientation, slice, dp, dq, d->K); break;
    default: k_slice<__nv_bfloat16><<<grid_for(n), 256, 0, s>>>((const __nv_bfloat16*)cur, d->d_pos, (int)d->X, (int)d->Y, (int)d->Z, orientation, slice, dp, dq, d->K); break;
  }
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && p_out) e = cudaMemcpyAsync(p_out, dp, n * sizeof(float), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && pos_out) e = cudaMemcpyAsync(pos_out, dq, n, cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(dp, s);
  cudaFreeAsync(dq, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "slice capture", __FILE__, __LINE__);
  return PFDTD_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Transparent source (SimulationParameters.cpp:300-310): out[n] = s[n] -
// sum_{i<n} h[n-i] * s[i] in float, every product and sum rounded on its own,
// terms added in ascending i as the reference's loop.  The terms with
// n - i >= n_ir (h = 0 there) are skipped, which can change the sign of a zero
// result only.  One thread per output sample.
namespace pfdtd {
namespace {
__global__ void k_transparent(const float* __restrict__ s, const float* __restrict__ h,
                              int64_t n_ir, int64_t steps, float* __restrict__ out) {
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < steps;
       n += (int64_t)gridDim.x * blockDim.x) {
    float acc = 0.f;
    const int64_t i0 = n_ir > 0 ? (n - (n_ir - 1) > 0 ? n - (n_ir - 1) : 0) : n;
    for (int64_t i = i0; i < n; ++i) acc = __fadd_rn(acc, __fmul_rn(h[n - i], s[i]));
    out[n] = __fsub_rn(s[n], acc);
  }
}
}  // namespace
}  // namespace pfdtd

extern "C" int pfdtd_transparent_source(const float* samples, int64_t steps, const float* grid_ir,
                                        int64_t n_ir, float* out, int device) {
  using namespace pfdtd;
  if (steps < 0 || n_ir < 0 || (steps > 0 && (!samples || !out)) || (n_ir > 0 && !grid_ir))
    return fail(PFDTD_ERR_ARG, "invalid transparent source arrays");
  if (steps == 0) return PFDTD_OK;
  DevGuard g(device);
  cudaStream_t s = nullptr;
  PFDTD_CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  float *d_s = nullptr, *d_h = nullptr, *d_o = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&d_s, steps * sizeof(float), s);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&d_o, steps * sizeof(float), s);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&d_h, std::max<int64_t>(n_ir, 1) * sizeof(float), s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_s, samples, steps * sizeof(float), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && n_ir > 0)
    e = cudaMemcpyAsync(d_h, grid_ir, n_ir * sizeof(float), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    k_transparent<<<grid_for(steps), 256, 0, s>>>(d_s, d_h, n_ir, steps, d_o);
    count_launch();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, d_o, steps * sizeof(float), cudaMemcpyDeviceToHost, s);
  if (d_s) cudaFreeAsync(d_s, s);
  if (d_o) cudaFreeAsync(d_o, s);
  if (d_h) cudaFreeAsync(d_h, s);
  const cudaError_t e2 = cudaStreamSynchronize(s);
  cudaStreamDestroy(s);
  if (e == cudaSuccess) e = e2;
  if (e != cudaSuccess) return cuda_fail(e, "transparent source", __FILE__, __LINE__);
  return PFDTD_OK;
}
