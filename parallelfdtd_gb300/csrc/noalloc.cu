// Slice capture that allocates nothing.
//
// pfdtd_capture_slice gathers the slice into device temporaries it allocates
// and frees on every call.  Some callers cannot afford that: a serving loop
// that has committed the whole HBM budget to resident domains (one more
// allocation may fail mid-run), and per-step capture or visualization loops
// that must not stall, since cudaFree synchronizes the whole device.  This
// variant gathers into one fixed scratch array compiled into the library
// instead, and copies from there into the caller's host buffers.
#include "common.cuh"

#include <algorithm>
#include <mutex>
#include <string>

namespace pfdtd {
namespace {

// Largest slice (nodes) the scratch holds: 1,048,576 nodes, e.g. 1024 x 1024.
constexpr int64_t kNoAllocMaxSliceNodes = (int64_t)1 << 20;
// 4 bytes of pressure (float) plus 1 node byte per slice node: 5 MiB.  CUDA
// loads a module's __device__ arrays onto a GPU lazily, the first time the
// module is used there; domain creation resolves the scratch's address
// (noalloc_prepare), so every GPU that has had a domain holds these 5 MiB,
// taken before the domain's own buffers, until the process exits.
constexpr size_t kNoAllocScratchBytes = (size_t)kNoAllocMaxSliceNodes * 5;

static __device__ __align__(256) unsigned char g_slice_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
void* g_scratch_addr[kMaxDevices] = {nullptr};

// Device address of the scratch on the current device, looked up once per
// device.  In host code the array's name only stands in for the symbol; the
// kernel must be given this address.
int scratch_address(int device, void** out) {
  if (device < 0 || device >= kMaxDevices) return fail(PFDTD_ERR_ARG, "device index out of range");
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_addr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_slice_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(slice scratch)", __FILE__, __LINE__);
    g_scratch_addr[device] = p;
  }
  *out = g_scratch_addr[device];
  return PFDTD_OK;
}

// Same gather as the allocating capture: every element of the w x h slice is
// written (the uncaptured last z row of xz/yz slices as 0), so nothing left
// in the scratch by an earlier call reaches the result.
template <typename S>
__global__ void k_slice_into(const S* __restrict__ P, const uint8_t* __restrict__ pos, int X,
                             int Y, int Z, int orientation, int64_t slice,
                             float* __restrict__ p_out, uint8_t* __restrict__ pos_out, int K) {
  const int64_t w = orientation == 2 ? Y : X;
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
    p_out[i] = keep ? (float)Store<S>::load(P[src * K]) : 0.f;
    pos_out[i] = keep ? pos[src] : 0;
  }
}

}  // namespace

// Places the scratch on `device` (the current device) and caches its address.
// Called at domain creation so that the 5 MiB are taken before the caller
// commits the device's memory; a failure here is cleared and the first
// no-allocation capture on the device tries again.
int noalloc_prepare(int device) {
  void* p = nullptr;
  int rc = scratch_address(device, &p);
  if (rc != PFDTD_OK) cudaGetLastError();
  return rc;
}

}  // namespace pfdtd

using namespace pfdtd;

extern "C" int pfdtd_capture_slice_noalloc(pfdtd_domain* d, int orientation, int64_t slice,
                                           float* p_out, uint8_t* pos_out) {
  if (!d) return fail(PFDTD_ERR_ARG, "null domain");
  if (orientation < 0 || orientation > 2) return fail(PFDTD_ERR_ARG, "orientation must be 0, 1 or 2");
  const int64_t lim = orientation == 0 ? d->Z : (orientation == 1 ? d->Y : d->X);
  if (slice < 0 || slice >= lim) return fail(PFDTD_ERR_ARG, "slice outside the grid, no capture made");
  const int64_t w = orientation == 2 ? d->Y : d->X;
  const int64_t h = orientation == 0 ? d->Y : d->Z;
  const int64_t n = w * h;
  if (n > kNoAllocMaxSliceNodes)
    return fail(PFDTD_ERR_ARG, "slice of " + std::to_string(n) + " nodes exceeds the " +
                                   std::to_string(kNoAllocMaxSliceNodes) +
                                   "-node scratch of pfdtd_capture_slice_noalloc; use "
                                   "pfdtd_capture_slice");
  int prev = -1;
  cudaGetDevice(&prev);
  if (prev != d->device) {
    cudaError_t e = cudaSetDevice(d->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice", __FILE__, __LINE__);
  }
  void* scratch = nullptr;
  int rc = scratch_address(d->device, &scratch);
  if (rc == PFDTD_OK) {
    float* dp = (float*)scratch;
    uint8_t* dq = (uint8_t*)scratch + (size_t)kNoAllocMaxSliceNodes * sizeof(float);
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, kGridSMs * 16));
    cudaStream_t s = d->stream;
    const void* cur = d->cur_field();
    const int X = (int)d->X, Y = (int)d->Y, Z = (int)d->Z;
    switch (d->precision) {
      case PFDTD_F32: k_slice_into<float><<<grid, 256, 0, s>>>((const float*)cur, d->d_pos, X, Y, Z, orientation, slice, dp, dq, d->K); break;
      case PFDTD_F64: k_slice_into<double><<<grid, 256, 0, s>>>((const double*)cur, d->d_pos, X, Y, Z, orientation, slice, dp, dq, d->K); break;
      case PFDTD_F16: k_slice_into<__half><<<grid, 256, 0, s>>>((const __half*)cur, d->d_pos, X, Y, Z, orientation, slice, dp, dq, d->K); break;
      default: k_slice_into<__nv_bfloat16><<<grid, 256, 0, s>>>((const __nv_bfloat16*)cur, d->d_pos, X, Y, Z, orientation, slice, dp, dq, d->K); break;
    }
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && p_out)
      e = cudaMemcpyAsync(p_out, dp, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && pos_out)
      e = cudaMemcpyAsync(pos_out, dq, (size_t)n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) rc = cuda_fail(e, "no-allocation slice capture", __FILE__, __LINE__);
  }
  if (prev >= 0 && prev != d->device) cudaSetDevice(prev);
  return rc;
}
