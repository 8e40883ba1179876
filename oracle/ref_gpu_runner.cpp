// ---------------------------------------------------------------------------
// Runs the reference's own CUDA kernels on the GPU — test infrastructure only.
//
// oracle/build_ref.py compiles ParallelFDTD's src/kernels/kernels3d.cu and
// src/kernels/cudaMesh.cu unchanged into sm_103a cubins (one with nvcc's
// default contraction, one with -fmad=false).  This file loads them through
// the CUDA driver API and drives them with the reference's host sequence:
//
//   set-up (CudaMesh::setupMesh, cudaMesh.cu:25-58): padWithZerosKernel on
//     the position and material bytes (cudaMesh.cu:253-304), then
//     toBilbaoKernel or toKowalczykKernel and calcBoundaries on a square grid
//     of 512-thread blocks (cudaMesh.cu:150-248);
//   step loop (launchFDTD3d, kernels3d.cu:86-175): write each source sample
//     into the current field with a one-element host-to-device copy (a hard
//     source sets, a soft one — as the reference runs it, cudaMesh.h:349-369
//     — also writes the sample alone), launch fdtd3dStdMaterials or
//     fdtd3dStdKowalczykMaterials over grid (X/bx, Y/by, Z-2) with block
//     (bx, by, 1) and every pointer advanced by one xy-plane, swap the two
//     fields, copy each receiver's element into its device trace.
//
// Before any launch the host checks that the padded dims are multiples of the
// block and that every buffer holds what the reference kernels index (the
// stencil stays inside [0, X*Y*Z); the padding kernel reads up to X*Y + X
// bytes past the unpadded mesh when a dimension is padded, so that input is
// allocated with that much zeroed slack).  The reference's fdtd3dSliced
// kernel is never launched.
// ---------------------------------------------------------------------------
#include <cuda.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

struct Modules {
  CUcontext ctx = nullptr;
  CUmodule kernels = nullptr;
  CUmodule mesh = nullptr;
  CUfunction fwd_f = nullptr, fwd_d = nullptr, cen_f = nullptr, cen_d = nullptr;
  CUfunction pad = nullptr, to_bilbao = nullptr, to_kowalczyk = nullptr, count = nullptr;
};

Modules g_mod;
char g_err[512];

int fail(const char* what, CUresult r) {
  const char* s = nullptr;
  cuGetErrorString(r, &s);
  snprintf(g_err, sizeof(g_err), "%s: %s", what, s ? s : "unknown CUDA error");
  return -1;
}

#define CK(call)                                  \
  do {                                            \
    CUresult _r = (call);                         \
    if (_r != CUDA_SUCCESS) return fail(#call, _r); \
  } while (0)

// Finds a kernel whose (mangled) name holds every fragment in `parts`.
CUfunction find(CUmodule m, std::initializer_list<const char*> parts) {
  unsigned n = 0;
  if (cuModuleGetFunctionCount(&n, m) != CUDA_SUCCESS || n == 0) return nullptr;
  std::vector<CUfunction> fs(n);
  if (cuModuleEnumerateFunctions(fs.data(), n, m) != CUDA_SUCCESS) return nullptr;
  for (CUfunction f : fs) {
    const char* name = nullptr;
    if (cuFuncGetName(&name, f) != CUDA_SUCCESS || !name) continue;
    std::string s(name);
    bool ok = true;
    for (const char* p : parts) ok = ok && s.find(p) != std::string::npos;
    if (ok) return f;
  }
  return nullptr;
}

struct DevBuf {
  CUdeviceptr p = 0;
  ~DevBuf() {
    if (p) cuMemFree(p);
  }
};

}  // namespace

extern "C" {

const char* refgpu_error() { return g_err; }

// Loads the two cubins on device 0 (its primary context).  Returns 0 or -1.
int refgpu_load(const char* kernels_cubin, const char* mesh_cubin) {
  CK(cuInit(0));
  CUdevice dev;
  CK(cuDeviceGet(&dev, 0));
  if (!g_mod.ctx) CK(cuDevicePrimaryCtxRetain(&g_mod.ctx, dev));
  CK(cuCtxSetCurrent(g_mod.ctx));
  if (g_mod.kernels) {
    cuModuleUnload(g_mod.kernels);
    g_mod.kernels = nullptr;
  }
  if (g_mod.mesh) {
    cuModuleUnload(g_mod.mesh);
    g_mod.mesh = nullptr;
  }
  CK(cuModuleLoad(&g_mod.kernels, kernels_cubin));
  CK(cuModuleLoad(&g_mod.mesh, mesh_cubin));
  // Itanium names: fdtd3dStdMaterials<float> -> ...fdtd3dStdMaterialsIf..., <double> -> ...Id...
  g_mod.fwd_f = find(g_mod.kernels, {"18fdtd3dStdMaterialsIf"});
  g_mod.fwd_d = find(g_mod.kernels, {"18fdtd3dStdMaterialsId"});
  g_mod.cen_f = find(g_mod.kernels, {"27fdtd3dStdKowalczykMaterialsIf"});
  g_mod.cen_d = find(g_mod.kernels, {"27fdtd3dStdKowalczykMaterialsId"});
  g_mod.pad = find(g_mod.mesh, {"18padWithZerosKernel"});
  g_mod.to_bilbao = find(g_mod.mesh, {"14toBilbaoKernel"});
  g_mod.to_kowalczyk = find(g_mod.mesh, {"17toKowalczykKernel"});
  g_mod.count = find(g_mod.mesh, {"14calcBoundaries"});
  if (!g_mod.fwd_f || !g_mod.fwd_d || !g_mod.cen_f || !g_mod.cen_d || !g_mod.pad ||
      !g_mod.to_bilbao || !g_mod.to_kowalczyk || !g_mod.count) {
    snprintf(g_err, sizeof(g_err), "a reference kernel was not found in the cubins");
    return -1;
  }
  return 0;
}

// One reference run.  precision 0 = float (launchFDTD3d), 1 = double
// (launchFDTD3dDouble); scheme 0 = forward, 1 = centred.  bid/mat: voxelizer
// ids and materials, X*Y*Z bytes (unpadded dims X, Y, Z).  params: 4 values,
// table: n_mat*20 values, samples: n_src*steps values, all of the run's type.
// src_idx/rec_idx: element indices in the padded mesh.  Outputs: receivers
// [n_rec*steps], final current and past fields (padded size, may be NULL),
// counts[2] = air and boundary nodes, kernel_ms = summed event time of the
// update launches.  Returns 0, or -1 with refgpu_error() set.
int refgpu_run(int precision, int scheme, const uint8_t* bid, const uint8_t* mat, unsigned X,
               unsigned Y, unsigned Z, unsigned bx, unsigned by, const void* params,
               const void* table, unsigned n_mat, int n_src, const int64_t* src_idx,
               const int* src_hard, const void* samples, int n_rec, const int64_t* rec_idx,
               int steps, void* rec_out, void* p_out, void* pp_out, unsigned* counts,
               float* kernel_ms) {
  if (!g_mod.kernels) {
    snprintf(g_err, sizeof(g_err), "refgpu_load was not called");
    return -1;
  }
  CK(cuCtxSetCurrent(g_mod.ctx));
  const size_t es = precision ? sizeof(double) : sizeof(float);
  // padded dims (padWithZeros, cudaMesh.cu:262-269), block z = 1
  unsigned padX = (X % bx) ? bx - X % bx : 0, padY = (Y % by) ? by - Y % by : 0;
  const unsigned PX = X + padX, PY = Y + padY, PZ = Z;
  if (PX % bx || PY % by || PZ < 3 || bx * by > 1024 || bx == 0 || by == 0) {
    snprintf(g_err, sizeof(g_err), "invalid dims or block");
    return -1;
  }
  const size_t n_old = (size_t)X * Y * Z;
  const size_t n = (size_t)PX * PY * PZ;
  if (n >= (1ull << 31)) {
    snprintf(g_err, sizeof(g_err), "mesh too large for the reference's int indexing");
    return -1;
  }
  for (int i = 0; i < n_src; ++i)
    if (src_idx[i] < 0 || (size_t)src_idx[i] >= n) {
      snprintf(g_err, sizeof(g_err), "source %d outside the mesh", i);
      return -1;
    }
  for (int i = 0; i < n_rec; ++i)
    if (rec_idx[i] < 0 || (size_t)rec_idx[i] >= n) {
      snprintf(g_err, sizeof(g_err), "receiver %d outside the mesh", i);
      return -1;
    }
  const size_t slack = (size_t)X * Y + X + 1;
  DevBuf d_bid_old, d_mat_old, d_pos, d_mat, d_P, d_Pp, d_par, d_tab, d_rec, d_cnt;
  CK(cuMemAlloc(&d_bid_old.p, n_old + slack));
  CK(cuMemAlloc(&d_mat_old.p, n_old + slack));
  CK(cuMemsetD8(d_bid_old.p, 0, n_old + slack));
  CK(cuMemsetD8(d_mat_old.p, 0, n_old + slack));
  CK(cuMemcpyHtoD(d_bid_old.p, bid, n_old));
  CK(cuMemcpyHtoD(d_mat_old.p, mat, n_old));
  CK(cuMemAlloc(&d_pos.p, n));
  CK(cuMemAlloc(&d_mat.p, n));
  CK(cuMemsetD8(d_pos.p, 0, n));
  CK(cuMemsetD8(d_mat.p, 0, n));
  {
    // padWithZerosKernel grid (ceil(X'/bx), ceil(Y'/by), Z), block (bx, by, 1)
    unsigned gx = (unsigned)std::ceil((float)PX / (float)bx);
    unsigned gy = (unsigned)std::ceil((float)PY / (float)by);
    unsigned zero = 0, pz = 0;
    CUdeviceptr dst = d_pos.p, src = d_bid_old.p;
    void* a1[] = {&dst, &src, &X, &Y, &Z, &padX, &padY, &pz, &zero};
    CK(cuLaunchKernel(g_mod.pad, gx, gy, Z, bx, by, 1, 0, 0, a1, nullptr));
    CUdeviceptr dst2 = d_mat.p, src2 = d_mat_old.p;
    void* a2[] = {&dst2, &src2, &X, &Y, &Z, &padX, &padY, &pz, &zero};
    CK(cuLaunchKernel(g_mod.pad, gx, gy, Z, bx, by, 1, 0, 0, a2, nullptr));
  }
  {
    unsigned num = (unsigned)n;
    int blocks = (int)((num + 511) / 512);
    unsigned side = (unsigned)std::ceil(std::sqrt((double)blocks));
    CUdeviceptr p = d_pos.p, m = d_mat.p;
    void* a[] = {&p, &m, &num};
    CK(cuLaunchKernel(scheme ? g_mod.to_kowalczyk : g_mod.to_bilbao, side, side, 1, 512, 1, 1, 0,
                      0, a, nullptr));
    CK(cuMemAlloc(&d_cnt.p, 2 * sizeof(unsigned)));
    CK(cuMemsetD32(d_cnt.p, 0, 2));
    CUdeviceptr air = d_cnt.p, bnd = d_cnt.p + sizeof(unsigned);
    unsigned char air_value = scheme ? 0x80 : 0x86, outside = 0;
    void* c[] = {&p, &air, &bnd, &air_value, &outside, &num};
    CK(cuLaunchKernel(g_mod.count, side, side, 1, 512, 1, 1, 0, 0, c, nullptr));
    unsigned h[2];
    CK(cuMemcpyDtoH(h, d_cnt.p, sizeof(h)));
    if (counts) {
      counts[0] = h[0];
      counts[1] = h[1];
    }
  }
  // fields: size + 1 + X elements, zeroed (cudaMesh.h:683, :717)
  const size_t nf = n + 1 + PX;
  CK(cuMemAlloc(&d_P.p, nf * es));
  CK(cuMemAlloc(&d_Pp.p, nf * es));
  CK(cuMemsetD8(d_P.p, 0, nf * es));
  CK(cuMemsetD8(d_Pp.p, 0, nf * es));
  CK(cuMemAlloc(&d_par.p, 4 * es));
  CK(cuMemcpyHtoD(d_par.p, params, 4 * es));
  CK(cuMemAlloc(&d_tab.p, (size_t)n_mat * 20 * es + es));
  CK(cuMemcpyHtoD(d_tab.p, table, (size_t)n_mat * 20 * es));
  if (n_rec > 0) {
    CK(cuMemAlloc(&d_rec.p, (size_t)n_rec * steps * es));
    CK(cuMemsetD8(d_rec.p, 0, (size_t)n_rec * steps * es));
  }
  CK(cuCtxSynchronize());

  CUfunction k = scheme ? (precision ? g_mod.cen_d : g_mod.cen_f)
                        : (precision ? g_mod.fwd_d : g_mod.fwd_f);
  CUevent e0, e1;
  CK(cuEventCreate(&e0, CU_EVENT_DEFAULT));
  CK(cuEventCreate(&e1, CU_EVENT_DEFAULT));
  float total_ms = 0.f;
  const int xy = (int)(PX * PY), dx = (int)PX;
  CUdeviceptr P = d_P.p, Pp = d_Pp.p;
  const uint8_t* smp = static_cast<const uint8_t*>(samples);
  int rc = 0;
  for (int step = 0; step < steps && rc == 0; ++step) {
    for (int i = 0; i < n_src; ++i) {
      // hard: setSample; soft: addSample as run, which writes the sample alone
      CUresult r = cuMemcpyHtoD(P + (size_t)src_idx[i] * es, smp + ((size_t)i * steps + step) * es,
                                es);
      if (r != CUDA_SUCCESS) {
        rc = fail("source copy", r);
        break;
      }
      (void)src_hard;
    }
    if (rc) break;
    CUdeviceptr a0 = d_pos.p + xy, a1 = d_mat.p + xy, a2 = P + (size_t)xy * es,
                a3 = Pp + (size_t)xy * es, a4 = d_par.p, a5 = d_tab.p;
    int a6 = xy, a7 = dx;
    void* args[] = {&a0, &a1, &a2, &a3, &a4, &a5, &a6, &a7};
    cuEventRecord(e0, 0);
    CUresult r = cuLaunchKernel(k, PX / bx, PY / by, PZ - 2, bx, by, 1, 0, 0, args, nullptr);
    cuEventRecord(e1, 0);
    if (r == CUDA_SUCCESS) r = cuEventSynchronize(e1);
    if (r != CUDA_SUCCESS) {
      rc = fail("update launch", r);
      break;
    }
    float ms = 0.f;
    cuEventElapsedTime(&ms, e0, e1);
    total_ms += ms;
    CUdeviceptr t = P;  // flipPressurePointers
    P = Pp;
    Pp = t;
    for (int i = 0; i < n_rec; ++i) {
      r = cuMemcpyDtoD(d_rec.p + ((size_t)i * steps + step) * es, P + (size_t)rec_idx[i] * es, es);
      if (r != CUDA_SUCCESS) {
        rc = fail("receiver copy", r);
        break;
      }
    }
  }
  cuEventDestroy(e0);
  cuEventDestroy(e1);
  if (rc) return rc;
  CK(cuCtxSynchronize());
  if (n_rec > 0 && rec_out) CK(cuMemcpyDtoH(rec_out, d_rec.p, (size_t)n_rec * steps * es));
  if (p_out) CK(cuMemcpyDtoH(p_out, P, n * es));
  if (pp_out) CK(cuMemcpyDtoH(pp_out, Pp, n * es));
  if (kernel_ms) *kernel_ms = total_ms;
  return 0;
}

}  // extern "C"
