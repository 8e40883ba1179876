// Post-processing of receiver traces (python/FDTDfilter.py:13-19,
// matlab/functions/FDTDpostFilter.m:1-31, matlab/testBench.m:203-204): a
// causal FIR low-pass, an optional DC blocker y[n] = x[n] - x[n-1] + a y[n-1],
// and a polyphase rational resampler, over many channels.  Arithmetic in
// double; float or double input and output.
#include "common.cuh"

#include <algorithm>

namespace pfdtd {
namespace {

// y[c][n] = sum_{k <= min(n, nb-1)} b[k] x[c][n-k]; one thread per output.
template <typename T>
__global__ void k_fir(const T* __restrict__ x, int64_t n_ch, int64_t n, const double* __restrict__ b,
                      int nb, T* __restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_ch * n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = i / n, t = i - c * n;
    const T* xc = x + c * n;
    double acc = 0.0;
    const int kmax = t < (int64_t)(nb - 1) ? (int)t : nb - 1;
    for (int k = 0; k <= kmax; ++k) acc += b[k] * (double)xc[t - k];
    y[i] = (T)acc;
  }
}

// DC blocker in place, one thread per channel (the recursion is sequential).
template <typename T>
__global__ void k_dc_block(T* __restrict__ y, int64_t n_ch, int64_t n, double a) {
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= n_ch) return;
  T* yc = y + c * n;
  double xp = 0.0, yp = 0.0;
  for (int64_t t = 0; t < n; ++t) {
    const double xv = (double)yc[t];
    const double v = xv - xp + a * yp;
    xp = xv;
    yp = v;
    yc[t] = (T)v;
  }
}

// Polyphase resampler: y[c][j] = sum_i h[(j + offset) * down - i * up] x[c][i]
// over the i with the tap index in [0, nh) (zero-stuffing by `up`, FIR `h`,
// keeping every `down`-th sample from `offset` on); one thread per output.
template <typename T>
__global__ void k_resample(const T* __restrict__ x, int64_t n_ch, int64_t n_in,
                           const double* __restrict__ h, int nh, int up, int down, int64_t offset,
                           int64_t n_out, T* __restrict__ y) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n_ch * n_out;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = k / n_out, j = k - c * n_out;
    const int64_t t = (j + offset) * down;  // position on the up-sampled axis
    int64_t i_hi = t / up;                  // largest i with t - i*up >= 0
    const int64_t lo_num = t - (nh - 1);    // smallest i with t - i*up <= nh - 1
    int64_t i_lo = lo_num <= 0 ? 0 : (lo_num + up - 1) / up;
    if (i_hi > n_in - 1) i_hi = n_in - 1;
    const T* xc = x + c * n_in;
    double acc = 0.0;
    for (int64_t i = i_lo; i <= i_hi; ++i) acc += h[t - i * up] * (double)xc[i];
    y[k] = (T)acc;
  }
}

template <typename T>
int resample_t(const T* x, int64_t n_ch, int64_t n_in, const double* h, int nh, int up, int down,
               int64_t offset, int64_t n_out, T* out, int device) {
  int prev = -1;
  cudaGetDevice(&prev);
  if (prev != device) cudaSetDevice(device);
  struct Restore {
    int p;
    ~Restore() { if (p >= 0) cudaSetDevice(p); }
  } restore{prev};
  cudaStream_t s = nullptr;
  PFDTD_CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  const size_t in_bytes = (size_t)n_ch * (size_t)n_in * sizeof(T);
  const size_t out_bytes = (size_t)n_ch * (size_t)n_out * sizeof(T);
  T *dx = nullptr, *dy = nullptr;
  double* dh = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&dx, in_bytes, s);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&dy, out_bytes, s);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&dh, sizeof(double) * nh, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dx, x, in_bytes, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dh, h, sizeof(double) * nh, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    const int64_t tot = n_ch * n_out;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((tot + 255) / 256, kGridSMs * 32));
    k_resample<T><<<grid, 256, 0, s>>>(dx, n_ch, n_in, dh, nh, up, down, offset, n_out, dy);
    count_launch();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, dy, out_bytes, cudaMemcpyDeviceToHost, s);
  for (void* p : {(void*)dx, (void*)dy, (void*)dh})
    if (p) cudaFreeAsync(p, s);
  const cudaError_t e2 = cudaStreamSynchronize(s);
  cudaStreamDestroy(s);
  if (e == cudaSuccess) e = e2;
  if (e != cudaSuccess) return cuda_fail(e, "resample", __FILE__, __LINE__);
  return PFDTD_OK;
}

template <typename T>
int post_filter_t(const T* x, int64_t n_ch, int64_t n, const double* b, int nb, int dc, double a,
                  T* out, int device) {
  int prev = -1;
  cudaGetDevice(&prev);
  if (prev != device) cudaSetDevice(device);
  struct Restore {
    int p;
    ~Restore() { if (p >= 0) cudaSetDevice(p); }
  } restore{prev};
  cudaStream_t s = nullptr;
  PFDTD_CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  const size_t bytes = (size_t)n_ch * (size_t)n * sizeof(T);
  T *dx = nullptr, *dy = nullptr;
  double* db = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&dx, bytes, s);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&dy, bytes, s);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&db, sizeof(double) * nb, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dx, x, bytes, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(db, b, sizeof(double) * nb, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    const int64_t tot = n_ch * n;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((tot + 255) / 256, kGridSMs * 32));
    k_fir<T><<<grid, 256, 0, s>>>(dx, n_ch, n, db, nb, dy);
    count_launch();
    if (dc) {
      k_dc_block<T><<<(int)((n_ch + 127) / 128), 128, 0, s>>>(dy, n_ch, n, a);
      count_launch();
    }
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, dy, bytes, cudaMemcpyDeviceToHost, s);
  for (void* p : {(void*)dx, (void*)dy, (void*)db})
    if (p) cudaFreeAsync(p, s);
  const cudaError_t e2 = cudaStreamSynchronize(s);
  cudaStreamDestroy(s);
  if (e == cudaSuccess) e = e2;
  if (e != cudaSuccess) return cuda_fail(e, "post filter", __FILE__, __LINE__);
  return PFDTD_OK;
}

}  // namespace
}  // namespace pfdtd

using namespace pfdtd;

extern "C" int pfdtd_resample(const void* x, int64_t n_channels, int64_t n_in, int is_double,
                              const double* taps, int n_taps, int up, int down, int64_t offset,
                              int64_t n_out, void* out, int device) {
  if (n_channels < 0 || n_in < 1 || n_out < 0 || n_taps < 1 || !taps || up < 1 || down < 1 ||
      offset < 0 || (n_channels * n_out > 0 && (!x || !out)))
    return fail(PFDTD_ERR_ARG, "invalid resampling arguments");
  if (n_channels * n_out == 0) return PFDTD_OK;
  return is_double ? resample_t<double>((const double*)x, n_channels, n_in, taps, n_taps, up, down,
                                        offset, n_out, (double*)out, device)
                   : resample_t<float>((const float*)x, n_channels, n_in, taps, n_taps, up, down,
                                       offset, n_out, (float*)out, device);
}

extern "C" int pfdtd_post_filter(const void* x, int64_t n_channels, int64_t n_samples,
                                 int is_double, const double* taps, int n_taps, int dc_block,
                                 double dc_coef, void* out, int device) {
  if (n_channels < 0 || n_samples < 0 || n_taps < 1 || !taps ||
      (n_channels * n_samples > 0 && (!x || !out)))
    return fail(PFDTD_ERR_ARG, "invalid filter arguments");
  if (n_channels * n_samples == 0) return PFDTD_OK;
  return is_double ? post_filter_t<double>((const double*)x, n_channels, n_samples, taps, n_taps,
                                           dc_block, dc_coef, (double*)out, device)
                   : post_filter_t<float>((const float*)x, n_channels, n_samples, taps, n_taps,
                                          dc_block, dc_coef, (float*)out, device);
}
