// C ABI of libpfdtd: domain lifecycle, node/material/parameter set-up,
// sources and receivers, the step loop and field access.
//
// The step loop of launchFDTD3d (ParallelFDTD src/kernels/kernels3d.cu:83-181)
// runs here entirely on the device: source samples and receiver buffers live
// in HBM, one small kernel per step records the receivers and injects the
// sources, one update kernel advances the field, and the pointer swap is a
// change of kernel arguments.  Chunks of kChunk steps are captured once into
// a CUDA graph and replayed; the host only polls the interrupt callback and
// reports progress between chunks.
#include "common.cuh"

#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <mutex>

namespace pfdtd {

static thread_local std::string t_error;
std::atomic<int64_t> g_launches{0};
static std::atomic<int64_t> g_serial{0};

void set_error(const std::string& msg) { t_error = msg; }
int fail(int code, const std::string& msg) {
  t_error = msg;
  return code;
}
int cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
  t_error = std::string(what) + " failed: " + cudaGetErrorString(e) + " (" + file + ":" +
            std::to_string(line) + ")";
  return e == cudaErrorMemoryAllocation ? PFDTD_ERR_NOMEM : PFDTD_ERR_CUDA;
}

namespace {

constexpr int64_t kChunk = 50;  // steps per captured graph (even: parity preserved)

size_t storage_size(int precision) {
  switch (precision) {
    case PFDTD_F32: return 4;
    case PFDTD_F64: return 8;
    case PFDTD_F16: return 2;
    case PFDTD_BF16: return 2;
  }
  return 0;
}

// Flat index of element (x, y, z) with the reference's arithmetic
// (cudaMesh.h:247-249); -1 when z lies outside the grid (the reference then
// finds no partition and skips the node, cudaMesh.h:251-266) or the flat
// index falls outside the allocation.
int64_t flat_index(const pfdtd_domain* d, int64_t x, int64_t y, int64_t z) {
  if (z < 0 || z >= d->Z) return -1;
  const int64_t i = z * d->XY + y * d->X + x;
  if (i < 0 || i >= d->N) return -1;
  return i;
}

// Field element of node (x, y, z) and field f, or -1 (see flat_index).
int64_t element_index(const pfdtd_domain* d, int64_t x, int64_t y, int64_t z, int64_t f) {
  if (f < 0 || f >= d->K) return -1;
  const int64_t i = flat_index(d, x, y, z);
  return i < 0 ? -1 : i * d->K + f;
}

int check_domain(const pfdtd_domain* d) {
  if (!d) return fail(PFDTD_ERR_ARG, "null domain");
  return PFDTD_OK;
}

// Convert a host double to the storage type.
void to_storage(int precision, double v, void* out) {
  switch (precision) {
    case PFDTD_F32: { float f = (float)v; std::memcpy(out, &f, 4); break; }
    case PFDTD_F64: std::memcpy(out, &v, 8); break;
    case PFDTD_F16: { __half h = __float2half_rn((float)v); std::memcpy(out, &h, 2); break; }
    case PFDTD_BF16: { __nv_bfloat16 h = __float2bfloat16_rn((float)v); std::memcpy(out, &h, 2); break; }
  }
}

double from_storage(int precision, const void* in) {
  switch (precision) {
    case PFDTD_F32: { float f; std::memcpy(&f, in, 4); return f; }
    case PFDTD_F64: { double v; std::memcpy(&v, in, 8); return v; }
    case PFDTD_F16: { __half h; std::memcpy(&h, in, 2); return __half2float(h); }
    case PFDTD_BF16: { __nv_bfloat16 h; std::memcpy(&h, in, 2); return __bfloat162float(h); }
  }
  return 0.0;
}

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    int now = -1;
    cudaGetDevice(&now);
    if (prev >= 0 && now != prev) cudaSetDevice(prev);
  }
};

int ensure_rec_out(pfdtd_domain* d, int64_t steps) {
  const size_t need = (size_t)std::max(d->n_rec, 1) * (size_t)std::max<int64_t>(steps, 1) *
                      d->arith_size();
  if (need <= d->rec_out_bytes) return PFDTD_OK;
  d->release(d->d_rec_out);
  d->d_rec_out = nullptr;
  d->rec_out_bytes = 0;
  if (d->alloc(&d->d_rec_out, need) != cudaSuccess)
    return fail(PFDTD_ERR_NOMEM, "receiver buffer allocation failed");
  d->rec_out_bytes = need;
  return PFDTD_OK;
}

// One step on the device: io (record previous, inject this) + update + swap.
int enqueue_step(pfdtd_domain* d, void* rec_out, int64_t rec_ld, int64_t inject_end,
                 cudaStream_t s) {
  int rc = launch_io(d, d->cur_field(), rec_out, rec_ld, inject_end, s);
  if (rc) return rc;
  rc = launch_update(d, d->cur_field(), d->past_field(), s);
  if (rc) return rc;
  rc = launch_dif(d, d->cur_field(), d->past_field(), s);
  if (rc) return rc;
  d->swap_fields();
  return PFDTD_OK;
}

// Steps per captured graph with temporal blocking: a multiple of 2T for
// T = 2, 3, 4, so the four buffers return to their roles after a chunk.
constexpr int64_t kChunkTb = 48;

bool tb_active(const pfdtd_domain* d) { return tb_usable(d, nullptr) != 0; }

// A graph of kChunk steps (kChunkTb when blocked) starting from the
// domain's current fields.
int get_chunk_graph(pfdtd_domain* d, void* rec_out, int64_t rec_ld, int64_t inject_end,
                    cudaGraphExec_t* exec) {
  const int tb = tb_active(d) ? d->tb_depth : 0;
  const int64_t chunk = tb ? kChunkTb : kChunk;
  // the kernels a chunk launches depend on the variant and the tile shape
  // too (an IWB shape decides whether a DIF pass follows the update)
  const int64_t cfg = chunk | ((int64_t)(d->tma_tile + 1) << 8) |
                      ((int64_t)d->kernel_variant << 16) | ((int64_t)(d->tb_shape + 1) << 24);
  const int64_t key[8] = {d->cur * 16 + d->prev * 4 + tb, cfg, d->class_version, d->io_version,
                          (int64_t)(intptr_t)rec_out, rec_ld, inject_end,
                          (int64_t)(intptr_t)d->d_cls};
  if (d->graph.exec && std::memcmp(key, d->graph.key, sizeof(key)) == 0) {
    *exec = d->graph.exec;
    return PFDTD_OK;
  }
  if (d->graph.exec) {
    cudaGraphExecDestroy(d->graph.exec);
    d->graph.exec = nullptr;
  }
  cudaStream_t s = d->stream;
  PFDTD_CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  const int cur0 = d->cur, prev0 = d->prev;
  const int64_t before = g_launches.load();
  int rc = PFDTD_OK;
  if (tb) {
    for (int64_t i = 0; i < chunk && rc == PFDTD_OK; i += tb)
      rc = launch_tb(d, rec_out, rec_ld, inject_end, s);
  } else {
    for (int64_t i = 0; i < chunk && rc == PFDTD_OK; ++i)
      rc = enqueue_step(d, rec_out, rec_ld, inject_end, s);
  }
  const int64_t captured = g_launches.load() - before;
  g_launches.store(before);  // captured, not launched
  d->cur = cur0;
  d->prev = prev0;
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamEndCapture(s, &graph);
  if (rc != PFDTD_OK) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture", __FILE__, __LINE__);
  e = cudaGraphInstantiate(&d->graph.exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate", __FILE__, __LINE__);
  std::memcpy(d->graph.key, key, sizeof(key));
  d->graph.launches = captured;
  *exec = d->graph.exec;
  return PFDTD_OK;
}

// Read and clear the pipeline error flag (set by a kernel whose bounded wait
// expired); the stream must be synchronised.
int check_pipeline(pfdtd_domain* d) {
  int e = 0;
  PFDTD_CK(cudaMemcpy(&e, d->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (e) {
    PFDTD_CK(cudaMemset(d->d_err, 0, sizeof(int)));
    return fail(PFDTD_ERR_CUDA, "an update kernel's pipeline wait timed out; results are invalid");
  }
  return PFDTD_OK;
}

int prepare_run(pfdtd_domain* d) {
  if (!d->nodes_set) return fail(PFDTD_ERR_STATE, "node bytes not set");
  if (d->n_mat <= 0) return fail(PFDTD_ERR_STATE, "material table not set");
  int rc = build_classes(d);
  if (rc) return rc;
  // the temporally blocked update writes out of place: two more fields
  if (d->tb_depth >= 2 && !d->field_base[2]) {
    const size_t fbytes = (size_t)(d->NE + 2 * d->margin) * d->esize;
    for (int i = 2; i < 4; ++i) {
      if (d->alloc(&d->field_base[i], fbytes) != cudaSuccess) {
        cudaGetLastError();
        d->release(d->field_base[2]);
        d->field_base[2] = nullptr;
        return fail(PFDTD_ERR_NOMEM, "allocation of the temporal blocking fields failed");
      }
      PFDTD_CK(cudaMemsetAsync(d->field_base[i], 0, fbytes, d->stream));
    }
  }
  return PFDTD_OK;
}

// Queue `steps` steps recording into rec_out (device, [n_rec * steps]).
// Between chunks `between(k_done)` may be called after waiting for chunk
// completion; it returns non-zero to stop.
template <typename F>
int enqueue_run(pfdtd_domain* d, int64_t steps, void* rec_out, F&& between, bool* stopped,
                int64_t* steps_queued, bool poll = true) {
  cudaStream_t s = d->stream;
  PFDTD_CK(cudaMemsetAsync(d->d_step, 0, sizeof(int64_t), s));
  if (int rc0 = launch_dif_init(d, s)) return rc0;
  const int tb = tb_active(d) ? d->tb_depth : 0;
  const int64_t chunk = tb ? kChunkTb : kChunk;
  const int64_t chunks = steps / chunk;
  const int64_t rem = steps - chunks * chunk;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  PFDTD_CK(cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming));
  PFDTD_CK(cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming));
  int rc = PFDTD_OK;
  int64_t queued = 0;
  *stopped = false;
  for (int64_t k = 0; k < chunks; ++k) {
    if (poll && k >= 2) {
      cudaError_t e = cudaEventSynchronize(ev[k % 2]);
      if (e != cudaSuccess) { rc = cuda_fail(e, "cudaEventSynchronize", __FILE__, __LINE__); break; }
      int perr = 0;
      e = cudaMemcpy(&perr, d->d_err, sizeof(int), cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) { rc = cuda_fail(e, "error flag read", __FILE__, __LINE__); break; }
      if (perr) { *stopped = true; break; }  // reported by check_pipeline after the sync
      if (between((k - 1) * chunk)) { *stopped = true; break; }
    }
    cudaGraphExec_t exec = nullptr;
    rc = get_chunk_graph(d, rec_out, steps, steps, &exec);
    if (rc) break;
    cudaError_t e = cudaGraphLaunch(exec, s);
    if (e != cudaSuccess) { rc = cuda_fail(e, "cudaGraphLaunch", __FILE__, __LINE__); break; }
    count_launch(d->graph.launches);
    e = cudaEventRecord(ev[k % 2], s);
    if (e != cudaSuccess) { rc = cuda_fail(e, "cudaEventRecord", __FILE__, __LINE__); break; }
    queued += chunk;
  }
  if (rc == PFDTD_OK && !*stopped) {
    int64_t i = 0;
    for (; tb && i + tb <= rem && rc == PFDTD_OK; i += tb) {
      rc = launch_tb(d, rec_out, steps, steps, s);
      if (rc == PFDTD_OK) queued += tb;
    }
    for (; i < rem && rc == PFDTD_OK; ++i) {
      rc = enqueue_step(d, rec_out, steps, steps, s);
      if (rc == PFDTD_OK) ++queued;
    }
  }
  // Record the receivers of the last step done; never inject.
  if (rc == PFDTD_OK) rc = launch_io(d, d->cur_field(), rec_out, steps, 0, s);
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
  *steps_queued = queued;
  return rc;
}

// Queue `n` steps continuing from the device step counter, without host
// waits: chunk graphs for whole chunks, then blocked launches and single
// steps.  rec_ld / inject_end as in enqueue_run (the run's step count).
int enqueue_steps(pfdtd_domain* d, int64_t n, void* rec_out, int64_t rec_ld, int64_t inject_end) {
  cudaStream_t s = d->stream;
  const int tb = tb_active(d) ? d->tb_depth : 0;
  const int64_t chunk = tb ? kChunkTb : kChunk;
  int64_t done = 0;
  for (; done + chunk <= n; done += chunk) {
    cudaGraphExec_t exec = nullptr;
    if (int rc = get_chunk_graph(d, rec_out, rec_ld, inject_end, &exec)) return rc;
    PFDTD_CK(cudaGraphLaunch(exec, s));
    count_launch(d->graph.launches);
  }
  for (; tb && done + tb <= n; done += tb)
    if (int rc = launch_tb(d, rec_out, rec_ld, inject_end, s)) return rc;
  for (; done < n; ++done)
    if (int rc = enqueue_step(d, rec_out, rec_ld, inject_end, s)) return rc;
  return PFDTD_OK;
}

}  // namespace
}  // namespace pfdtd

using namespace pfdtd;

extern "C" {

const char* pfdtd_last_error(void) { return t_error.c_str(); }

const char* pfdtd_version(void) { return "pfdtd-gb300 0.1 (sm_103a)"; }

int64_t pfdtd_kernel_launches(void) { return g_launches.load(); }

int pfdtd_device_count(int* count) {
  if (!count) return fail(PFDTD_ERR_ARG, "null count");
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess) {
    cudaGetLastError();
    n = 0;
  }
  *count = n;
  return PFDTD_OK;
}

int pfdtd_create(int64_t dim_x, int64_t dim_y, int64_t dim_z, int precision, int device,
                 pfdtd_domain** out) {
  return pfdtd_create_batched(dim_x, dim_y, dim_z, 1, precision, device, out);
}

int pfdtd_create_batched(int64_t dim_x, int64_t dim_y, int64_t dim_z, int fields, int precision,
                         int device, pfdtd_domain** out) {
  if (!out) return fail(PFDTD_ERR_ARG, "null output handle");
  *out = nullptr;
  if (fields < 1 || fields > 64 || (fields & (fields - 1)) != 0)
    return fail(PFDTD_ERR_ARG, "fields per node must be a power of two in 1..64");
  if (dim_x < 1 || dim_y < 1 || dim_z < 3)
    return fail(PFDTD_ERR_ARG, "grid must be at least 1 x 1 x 3 nodes");
  if (dim_x > (1 << 30) || dim_y > (1 << 30) || dim_z > (1 << 30) ||
      dim_x * dim_y > (int64_t)1 << 31)
    return fail(PFDTD_ERR_ARG, "grid dimension too large");
  const size_t es = storage_size(precision);
  if (es == 0) return fail(PFDTD_ERR_ARG, "unknown precision");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return fail(PFDTD_ERR_CUDA, "no CUDA device available");
  }
  if (device < 0 || device >= ndev) return fail(PFDTD_ERR_ARG, "device index out of range");
  DeviceGuard g(device);
  // The no-allocation slice capture's fixed scratch is placed on the device
  // now, before this domain's buffers take the memory it could need.
  noalloc_prepare(device);
  pfdtd_domain* d = new pfdtd_domain();
  d->device = device;
  d->serial = ++g_serial;
  cudaDeviceGetAttribute(&d->sm_count, cudaDevAttrMultiProcessorCount, device);
  d->precision = precision;
  d->X = dim_x;
  d->Y = dim_y;
  d->Z = dim_z;
  d->XY = dim_x * dim_y;
  d->N = d->XY * dim_z;
  d->K = fields;
  d->kshift = 0;
  while ((1 << d->kshift) < fields) ++d->kshift;
  d->NE = d->N * fields;
  d->esize = es;
  // Margins of one row plus a 256-byte-aligned pad on both sides of each
  // field keep every row-wise access of a tile with halo inside the
  // allocation; the reference allocates N + 1 + X (cudaMesh.h:717-718).
  const int64_t align = 256 / (int64_t)es;
  d->margin = (((dim_x + 64) * fields + align - 1) / align) * align;
  const size_t fbytes = (size_t)(d->NE + 2 * d->margin) * es;
  auto cleanup = [&](int code, const char* msg) {
    pfdtd_destroy(d);
    return fail(code, msg);
  };
  if (cudaStreamCreateWithFlags(&d->stream, cudaStreamNonBlocking) != cudaSuccess)
    return cleanup(PFDTD_ERR_CUDA, "stream creation failed");
  for (int i = 0; i < 2; ++i) {
    if (d->alloc(&d->field_base[i], fbytes) != cudaSuccess) {
      cudaGetLastError();
      return cleanup(PFDTD_ERR_NOMEM, "field allocation failed");
    }
    if (cudaMemsetAsync(d->field_base[i], 0, fbytes, d->stream) != cudaSuccess)
      return cleanup(PFDTD_ERR_CUDA, "field clear failed");
  }
  if (d->alloc((void**)&d->d_pos, (size_t)d->N + 1 + dim_x) != cudaSuccess ||
      d->alloc((void**)&d->d_mat, (size_t)d->N + 1 + dim_x) != cudaSuccess) {
    cudaGetLastError();
    return cleanup(PFDTD_ERR_NOMEM, "node byte allocation failed");
  }
  cudaMemsetAsync(d->d_pos, 0, (size_t)d->N + 1 + dim_x, d->stream);
  cudaMemsetAsync(d->d_mat, 0, (size_t)d->N + 1 + dim_x, d->stream);
  if (d->alloc((void**)&d->d_step, sizeof(int64_t)) != cudaSuccess ||
      d->alloc((void**)&d->d_err, sizeof(int)) != cudaSuccess)
    return cleanup(PFDTD_ERR_NOMEM, "step counter allocation failed");
  cudaMemsetAsync(d->d_err, 0, sizeof(int), d->stream);
  if (const char* tv = std::getenv("PFDTD_TMA_TILE")) d->tma_tile = std::atoi(tv);
  if (const char* sv = std::getenv("PFDTD_TB_SHAPE")) d->tb_shape = std::atoi(sv);
  if (const char* kv = std::getenv("PFDTD_KERNEL")) {
    if (std::strcmp(kv, "zmarch") == 0) d->kernel_variant = PFDTD_KERNEL_ZMARCH;
    if (std::strcmp(kv, "tma") == 0) d->kernel_variant = PFDTD_KERNEL_TMA;
  }
  if (cudaStreamSynchronize(d->stream) != cudaSuccess)
    return cleanup(PFDTD_ERR_CUDA, "domain initialisation failed");
  *out = d;
  return PFDTD_OK;
}

int pfdtd_destroy(pfdtd_domain* d) {
  if (!d) return PFDTD_OK;
  DeviceGuard g(d->device);
  if (d->stream) cudaStreamSynchronize(d->stream);
  if (d->graph.exec) cudaGraphExecDestroy(d->graph.exec);
  void* ptrs[] = {d->field_base[0], d->field_base[1], d->field_base[2], d->field_base[3], d->d_pos, d->d_mat, d->d_cls,
                  d->d_ctab, d->d_src_idx, d->d_src_mode, d->d_src_samples, d->d_rec_idx,
                  d->d_step, d->d_rec_out, d->d_err, d->d_dif_list, d->d_dif_tab,
                  d->d_dif_state, d->d_iwb_mask, d->d_iwb_code, d->d_iwb_sw,
                  d->d_iwb_closure, d->d_iwb_closure_dif, d->d_cls_tma};
  for (void* p : ptrs)
    d->release(p);
  if (d->stream) cudaStreamDestroy(d->stream);
  delete d;
  return PFDTD_OK;
}

int pfdtd_get_fields(const pfdtd_domain* d, int* fields) {
  if (int rc = check_domain(d)) return rc;
  if (!fields) return fail(PFDTD_ERR_ARG, "null output");
  *fields = d->K;
  return PFDTD_OK;
}

int pfdtd_get_dims(const pfdtd_domain* d, int64_t dims[3]) {
  if (int rc = check_domain(d)) return rc;
  dims[0] = d->X;
  dims[1] = d->Y;
  dims[2] = d->Z;
  return PFDTD_OK;
}

int pfdtd_get_serial(const pfdtd_domain* d, int64_t* serial) {
  if (int rc = check_domain(d)) return rc;
  if (!serial) return fail(PFDTD_ERR_ARG, "null serial pointer");
  *serial = d->serial;
  return PFDTD_OK;
}

int pfdtd_get_precision(const pfdtd_domain* d, int* precision) {
  if (int rc = check_domain(d)) return rc;
  *precision = d->precision;
  return PFDTD_OK;
}

int pfdtd_set_quirks(pfdtd_domain* d, int quirks) {
  if (int rc = check_domain(d)) return rc;
  if (quirks & ~(PFDTD_QUIRK_MATIDX | PFDTD_QUIRK_SOFTSRC))
    return fail(PFDTD_ERR_ARG, "unknown quirk bits");
  if ((quirks ^ d->quirks) & PFDTD_QUIRK_MATIDX) d->classes_dirty = true;
  if ((quirks ^ d->quirks) & PFDTD_QUIRK_SOFTSRC) {
    d->quirks = quirks;
    // Re-derive source modes.
    if (d->n_src > 0) {
      std::vector<int32_t> mode(d->n_src);
      for (int i = 0; i < d->n_src; ++i)
        mode[i] = (d->src_type_h[i] == PFDTD_SRC_HARD || (quirks & PFDTD_QUIRK_SOFTSRC)) ? 0 : 1;
      DeviceGuard g(d->device);
      PFDTD_CK(cudaMemcpy(d->d_src_mode, mode.data(), mode.size() * 4, cudaMemcpyHostToDevice));
      d->io_version++;
    }
  }
  d->quirks = quirks;
  return PFDTD_OK;
}

int pfdtd_set_wait_limit(pfdtd_domain* d, uint64_t ns) {
  if (int rc = check_domain(d)) return rc;
  d->wait_ns = ns == 0 ? 2000000000ull : ns;
  if (d->graph.exec) {  // the limit is a kernel argument baked into the graph
    cudaGraphExecDestroy(d->graph.exec);
    d->graph.exec = nullptr;
  }
  return PFDTD_OK;
}

int pfdtd_set_update_form(pfdtd_domain* d, int form) {
  if (int rc = check_domain(d)) return rc;
  if (form != PFDTD_FORM_REFERENCE && form != PFDTD_FORM_DIFFERENCE)
    return fail(PFDTD_ERR_ARG, "unknown update form");
  if (form != PFDTD_FORM_REFERENCE && d->precision != PFDTD_F32)
    return fail(PFDTD_ERR_UNSUPPORTED, "the difference form is built for FP32 fields");
  if (form != d->update_form) {
    d->update_form = form;
    d->classes_dirty = true;
    if (d->graph.exec) {
      cudaGraphExecDestroy(d->graph.exec);
      d->graph.exec = nullptr;
    }
  }
  return PFDTD_OK;
}

int pfdtd_set_scheme(pfdtd_domain* d, int scheme) {
  if (int rc = check_domain(d)) return rc;
  if (scheme != PFDTD_SRL_FORWARD && scheme != PFDTD_SHARED && scheme != PFDTD_SRL &&
      scheme != PFDTD_IWB)
    return fail(PFDTD_ERR_UNSUPPORTED, "unknown update scheme");
  auto eff = [](int sc) { return sc == PFDTD_SHARED ? PFDTD_SRL_FORWARD : sc; };
  const int eff_old = eff(d->scheme);
  const int eff_new = eff(scheme);
  if (eff_old != eff_new) d->classes_dirty = true;
  d->scheme = scheme;
  return PFDTD_OK;
}

int pfdtd_set_nodes(pfdtd_domain* d, const uint8_t* pos, const uint8_t* mat, int on_device) {
  if (int rc = check_domain(d)) return rc;
  if (!pos || !mat) return fail(PFDTD_ERR_ARG, "null node pointer");
  DeviceGuard g(d->device);
  const cudaMemcpyKind k = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  PFDTD_CK(cudaMemcpyAsync(d->d_pos, pos, (size_t)d->N, k, d->stream));
  PFDTD_CK(cudaMemcpyAsync(d->d_mat, mat, (size_t)d->N, k, d->stream));
  PFDTD_CK(cudaStreamSynchronize(d->stream));
  d->nodes_set = true;
  d->classes_dirty = true;
  return PFDTD_OK;
}

int pfdtd_get_node_ptrs(pfdtd_domain* d, uint8_t** d_pos, uint8_t** d_mat) {
  if (int rc = check_domain(d)) return rc;
  if (d_pos) *d_pos = d->d_pos;
  if (d_mat) *d_mat = d->d_mat;
  return PFDTD_OK;
}

int pfdtd_get_nodes(pfdtd_domain* d, uint8_t* pos, uint8_t* mat) {
  if (int rc = check_domain(d)) return rc;
  DeviceGuard g(d->device);
  PFDTD_CK(cudaStreamSynchronize(d->stream));
  if (pos) PFDTD_CK(cudaMemcpy(pos, d->d_pos, (size_t)d->N, cudaMemcpyDeviceToHost));
  if (mat) PFDTD_CK(cudaMemcpy(mat, d->d_mat, (size_t)d->N, cudaMemcpyDeviceToHost));
  return PFDTD_OK;
}

int pfdtd_nodes_changed(pfdtd_domain* d) {
  if (int rc = check_domain(d)) return rc;
  d->nodes_set = true;
  d->classes_dirty = true;
  return PFDTD_OK;
}

int pfdtd_set_materials(pfdtd_domain* d, const double* table, int n_mat, int n_coef) {
  if (int rc = check_domain(d)) return rc;
  if (!table || n_mat <= 0 || n_coef <= 0) return fail(PFDTD_ERR_ARG, "empty material table");
  d->materials.assign(table, table + (size_t)n_mat * n_coef);
  d->n_mat = n_mat;
  d->n_coef = n_coef;
  d->classes_dirty = true;
  return PFDTD_OK;
}

int pfdtd_set_params(pfdtd_domain* d, const double params[4]) {
  if (int rc = check_domain(d)) return rc;
  if (!params) return fail(PFDTD_ERR_ARG, "null parameter vector");
  for (int i = 0; i < 4; ++i) d->params[i] = params[i];
  d->classes_dirty = true;
  return PFDTD_OK;
}

int pfdtd_set_sources(pfdtd_domain* d, int n, const int64_t* xyz, const int32_t* type,
                      const void* samples, int64_t n_samples) {
  return pfdtd_set_sources_batched(d, n, xyz, nullptr, type, samples, n_samples);
}

int pfdtd_set_sources_batched(pfdtd_domain* d, int n, const int64_t* xyz, const int32_t* field,
                              const int32_t* type, const void* samples, int64_t n_samples) {
  if (int rc = check_domain(d)) return rc;
  if (n < 0 || (n > 0 && (!xyz || !type || (!samples && n_samples > 0))) || n_samples < 0)
    return fail(PFDTD_ERR_ARG, "invalid source arrays");
  DeviceGuard g(d->device);
  for (void** p : {(void**)&d->d_src_idx, (void**)&d->d_src_mode, &d->d_src_samples})
    if (*p) {
      d->release(*p);
      *p = nullptr;
    }
  d->n_src = n;
  d->n_samples = n_samples;
  d->src_idx_h.assign(n, -1);
  d->src_type_h.assign(type, type + n);
  std::vector<int32_t> mode(n);
  for (int i = 0; i < n; ++i) {
    d->src_idx_h[i] = element_index(d, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2],
                                    field ? field[i] : 0);
    if (type[i] < 0 || type[i] > 2) return fail(PFDTD_ERR_ARG, "unknown source type");
    mode[i] = (type[i] == PFDTD_SRC_HARD || (d->quirks & PFDTD_QUIRK_SOFTSRC)) ? 0 : 1;
  }
  const size_t sbytes = (size_t)n * (size_t)n_samples * d->arith_size();
  d->src_samples_h.assign((const uint8_t*)samples, (const uint8_t*)samples + sbytes);
  const size_t n1 = std::max(n, 1);
  PFDTD_CK(d->alloc((void**)&d->d_src_idx, n1 * sizeof(int64_t)));
  PFDTD_CK(d->alloc((void**)&d->d_src_mode, n1 * sizeof(int32_t)));
  PFDTD_CK(d->alloc(&d->d_src_samples, std::max<size_t>(sbytes, 16)));
  cudaStream_t s = d->stream;
  if (n > 0) {
    PFDTD_CK(cudaMemcpyAsync(d->d_src_idx, d->src_idx_h.data(), n * sizeof(int64_t),
                             cudaMemcpyHostToDevice, s));
    PFDTD_CK(cudaMemcpyAsync(d->d_src_mode, mode.data(), n * sizeof(int32_t),
                             cudaMemcpyHostToDevice, s));
    if (sbytes)
      PFDTD_CK(cudaMemcpyAsync(d->d_src_samples, samples, sbytes, cudaMemcpyHostToDevice, s));
  }
  PFDTD_CK(cudaStreamSynchronize(s));
  d->io_version++;
  return PFDTD_OK;
}

int pfdtd_set_receivers(pfdtd_domain* d, int n, const int64_t* xyz) {
  return pfdtd_set_receivers_batched(d, n, xyz, nullptr);
}

int pfdtd_set_receivers_batched(pfdtd_domain* d, int n, const int64_t* xyz, const int32_t* field) {
  if (int rc = check_domain(d)) return rc;
  if (n < 0 || (n > 0 && !xyz)) return fail(PFDTD_ERR_ARG, "invalid receiver array");
  DeviceGuard g(d->device);
  if (d->d_rec_idx) {
    d->release(d->d_rec_idx);
    d->d_rec_idx = nullptr;
  }
  d->n_rec = n;
  d->rec_idx_h.assign(n, -1);
  for (int i = 0; i < n; ++i)
    d->rec_idx_h[i] = element_index(d, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2],
                                    field ? field[i] : 0);
  PFDTD_CK(d->alloc((void**)&d->d_rec_idx, std::max(n, 1) * sizeof(int64_t)));
  if (n > 0)
    PFDTD_CK(cudaMemcpyAsync(d->d_rec_idx, d->rec_idx_h.data(), n * sizeof(int64_t),
                             cudaMemcpyHostToDevice, d->stream));
  PFDTD_CK(cudaStreamSynchronize(d->stream));
  d->io_version++;
  return PFDTD_OK;
}

int pfdtd_run(pfdtd_domain* d, int64_t steps, void* out, pfdtd_interrupt_fn interrupt_cb,
              pfdtd_progress_fn progress_cb, double* seconds_per_step) {
  if (int rc = check_domain(d)) return rc;
  if (steps < 0) return fail(PFDTD_ERR_ARG, "negative step count");
  if (d->n_rec > 0 && !out && steps > 0) return fail(PFDTD_ERR_ARG, "null output buffer");
  DeviceGuard g(d->device);
  const auto t0 = std::chrono::steady_clock::now();
  int rc = prepare_run(d);
  if (rc) return rc;
  if (steps == 0) {
    if (seconds_per_step) *seconds_per_step = 0.0;
    return PFDTD_OK;
  }
  if (interrupt_cb && interrupt_cb()) {
    if (seconds_per_step) *seconds_per_step = 0.0;
    return PFDTD_INTERRUPTED;
  }
  rc = ensure_rec_out(d, steps);
  if (rc) return rc;
  const size_t rec_bytes = (size_t)d->n_rec * (size_t)steps * d->arith_size();
  if (rec_bytes) PFDTD_CK(cudaMemsetAsync(d->d_rec_out, 0, rec_bytes, d->stream));
  // Progress is reported for every step index that is a multiple of 100
  // (PROGRESS_MOD, kernels3d.h:36) once the chunk holding it has finished.
  int64_t next_progress = 0;
  auto between = [&](int64_t done) -> int {
    if (progress_cb) {
      const double el =
          std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      for (; next_progress < done; next_progress += 100)
        progress_cb((int)next_progress, (int)steps, (float)(el / (double)done));
    }
    return (interrupt_cb && interrupt_cb()) ? 1 : 0;
  };
  bool stopped = false;
  int64_t queued = 0;
  rc = enqueue_run(d, steps, d->d_rec_out, between, &stopped, &queued);
  if (rc) return rc;
  // Rows of receivers outside the grid are left untouched (kernels3d.cu:184-191).
  const size_t row = (size_t)steps * d->arith_size();
  for (int r = 0; r < d->n_rec; ++r)
    if (d->rec_idx_h[r] >= 0)
      PFDTD_CK(cudaMemcpyAsync((char*)out + r * row, (char*)d->d_rec_out + r * row, row,
                               cudaMemcpyDeviceToHost, d->stream));
  PFDTD_CK(cudaStreamSynchronize(d->stream));
  if (int e = check_pipeline(d)) return e;
  const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (progress_cb && !stopped) between(queued);
  if (seconds_per_step) *seconds_per_step = queued > 0 ? el / (double)queued : 0.0;
  return stopped ? PFDTD_INTERRUPTED : PFDTD_OK;
}

int pfdtd_run_device(pfdtd_domain* d, int64_t steps, void* d_out) {
  if (int rc = check_domain(d)) return rc;
  if (steps < 0) return fail(PFDTD_ERR_ARG, "negative step count");
  if (d->n_rec > 0 && !d_out && steps > 0) return fail(PFDTD_ERR_ARG, "null output buffer");
  DeviceGuard g(d->device);
  int rc = prepare_run(d);
  if (rc || steps == 0) return rc;
  bool stopped = false;
  int64_t queued = 0;
  return enqueue_run(d, steps, d_out, [](int64_t) { return 0; }, &stopped, &queued);
}

int pfdtd_run_async(pfdtd_domain* d, int64_t steps) {
  if (int rc = check_domain(d)) return rc;
  if (steps < 0) return fail(PFDTD_ERR_ARG, "negative step count");
  DeviceGuard g(d->device);
  int rc = prepare_run(d);
  if (rc || steps == 0) return rc;
  rc = ensure_rec_out(d, steps);
  if (rc) return rc;
  const size_t rec_bytes = (size_t)d->n_rec * (size_t)steps * d->arith_size();
  if (rec_bytes) PFDTD_CK(cudaMemsetAsync(d->d_rec_out, 0, rec_bytes, d->stream));
  bool stopped = false;
  int64_t queued = 0;
  rc = enqueue_run(d, steps, d->d_rec_out, [](int64_t) { return 0; }, &stopped, &queued, false);
  if (rc == PFDTD_OK) d->async_steps = steps;
  return rc;
}

int pfdtd_run_captures(pfdtd_domain* d, int64_t steps, void* out, int n_cap,
                       const int64_t* cap_step, const int32_t* cap_orientation,
                       const int64_t* cap_slice, float* const* p_out, uint8_t* const* pos_out) {
  if (int rc = check_domain(d)) return rc;
  if (steps < 0 || n_cap < 0) return fail(PFDTD_ERR_ARG, "negative count");
  if (n_cap > 0 && (!cap_step || !cap_orientation || !cap_slice || (!p_out && !pos_out)))
    return fail(PFDTD_ERR_ARG, "invalid capture schedule");
  if (d->n_rec > 0 && !out && steps > 0) return fail(PFDTD_ERR_ARG, "null output buffer");
  std::vector<int> order(n_cap);
  std::vector<int64_t> size(n_cap), offset(n_cap + 1, 0);
  for (int i = 0; i < n_cap; ++i) {
    const int o = cap_orientation[i];
    if (o < 0 || o > 2) return fail(PFDTD_ERR_ARG, "orientation must be 0, 1 or 2");
    const int64_t lim = o == 0 ? d->Z : (o == 1 ? d->Y : d->X);
    if (cap_slice[i] < 0 || cap_slice[i] >= lim) return fail(PFDTD_ERR_ARG, "slice outside the grid");
    if (cap_step[i] < 0 || cap_step[i] > steps) return fail(PFDTD_ERR_ARG, "capture step outside the run");
    size[i] = (o == 2 ? d->Y : d->X) * (o == 0 ? d->Y : d->Z);
    offset[i + 1] = offset[i] + size[i];
    order[i] = i;
  }
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return cap_step[a] < cap_step[b]; });
  DeviceGuard g(d->device);
  int rc = prepare_run(d);
  if (rc) return rc;
  rc = ensure_rec_out(d, std::max<int64_t>(steps, 1));
  if (rc) return rc;
  cudaStream_t s = d->stream;
  const size_t rec_bytes = (size_t)d->n_rec * (size_t)steps * d->arith_size();
  if (rec_bytes) PFDTD_CK(cudaMemsetAsync(d->d_rec_out, 0, rec_bytes, s));
  // device staging for every capture: floats, then node bytes
  void* stage = nullptr;
  const int64_t total = offset[n_cap];
  if (total > 0 && d->alloc(&stage, (size_t)total * 5) != cudaSuccess)
    return fail(PFDTD_ERR_NOMEM, "capture staging allocation failed");
  float* sp = (float*)stage;
  uint8_t* sq = (uint8_t*)stage + (size_t)total * 4;
  PFDTD_CK(cudaMemsetAsync(d->d_step, 0, sizeof(int64_t), s));
  rc = launch_dif_init(d, s);
  int64_t at = 0;
  for (int k = 0; k < n_cap && rc == PFDTD_OK; ++k) {
    const int i = order[k];
    rc = enqueue_steps(d, cap_step[i] - at, d->d_rec_out, steps, steps);
    at = cap_step[i];
    if (rc) break;
    float* dp = p_out && p_out[i] ? sp + offset[i] : nullptr;
    uint8_t* dq = pos_out && pos_out[i] ? sq + offset[i] : nullptr;
    rc = launch_slice_gather(d, cap_orientation[i], cap_slice[i], dp, dq, s);
    if (rc) break;
    cudaError_t e = cudaSuccess;
    if (dp) e = cudaMemcpyAsync(p_out[i], dp, size[i] * sizeof(float), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && dq) e = cudaMemcpyAsync(pos_out[i], dq, size[i], cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) rc = cuda_fail(e, "capture copy", __FILE__, __LINE__);
  }
  if (rc == PFDTD_OK) rc = enqueue_steps(d, steps - at, d->d_rec_out, steps, steps);
  // record the receivers of the last step; never inject
  if (rc == PFDTD_OK && steps > 0) rc = launch_io(d, d->cur_field(), d->d_rec_out, steps, 0, s);
  if (rc == PFDTD_OK) {
    const size_t row = (size_t)steps * d->arith_size();
    for (int r = 0; r < d->n_rec && rc == PFDTD_OK && steps > 0; ++r)
      if (d->rec_idx_h[r] >= 0) {
        cudaError_t e = cudaMemcpyAsync((char*)out + r * row, (char*)d->d_rec_out + r * row, row,
                                        cudaMemcpyDeviceToHost, s);
        if (e != cudaSuccess) rc = cuda_fail(e, "receiver copy", __FILE__, __LINE__);
      }
  }
  d->release(stage);
  const cudaError_t e = cudaStreamSynchronize(s);
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_fail(e, "captured run", __FILE__, __LINE__);
  return check_pipeline(d);
}

int pfdtd_host_alloc(size_t bytes, void** ptr) {
  if (!ptr) return fail(PFDTD_ERR_ARG, "null output");
  *ptr = nullptr;
  if (bytes == 0) return PFDTD_OK;
  cudaError_t e = cudaHostAlloc(ptr, bytes, cudaHostAllocDefault);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *ptr = nullptr;
    return fail(PFDTD_ERR_NOMEM, "pinned host allocation failed");
  }
  return PFDTD_OK;
}

int pfdtd_host_free(void* ptr) {
  if (ptr) PFDTD_CK(cudaFreeHost(ptr));
  return PFDTD_OK;
}

int pfdtd_query(pfdtd_domain* d, int* done) {
  if (int rc = check_domain(d)) return rc;
  if (!done) return fail(PFDTD_ERR_ARG, "null output");
  DeviceGuard g(d->device);
  const cudaError_t e = cudaStreamQuery(d->stream);
  if (e == cudaSuccess) {
    *done = 1;
    return PFDTD_OK;
  }
  if (e == cudaErrorNotReady) {
    cudaGetLastError();
    *done = 0;
    return PFDTD_OK;
  }
  return cuda_fail(e, "stream query", __FILE__, __LINE__);
}

int pfdtd_fetch_receivers(pfdtd_domain* d, void* out) {
  if (int rc = check_domain(d)) return rc;
  if (!out && d->n_rec > 0) return fail(PFDTD_ERR_ARG, "null output buffer");
  DeviceGuard g(d->device);
  PFDTD_CK(cudaStreamSynchronize(d->stream));
  if (int e = check_pipeline(d)) return e;
  const int64_t steps = d->async_steps;
  const size_t row = (size_t)steps * d->arith_size();
  for (int r = 0; r < d->n_rec && steps > 0; ++r)
    if (d->rec_idx_h[r] >= 0)
      PFDTD_CK(cudaMemcpyAsync((char*)out + r * row, (char*)d->d_rec_out + r * row, row,
                               cudaMemcpyDeviceToHost, d->stream));
  PFDTD_CK(cudaStreamSynchronize(d->stream));
  return PFDTD_OK;
}

int pfdtd_profile_update(pfdtd_domain* d, int iters) {
  if (int rc = check_domain(d)) return rc;
  if (iters < 0) return fail(PFDTD_ERR_ARG, "negative iteration count");
  DeviceGuard g(d->device);
  int rc = prepare_run(d);
  if (rc) return rc;
  if (tb_active(d)) {
    // one blocked launch (and its io kernel) per iteration: depth steps,
    // no sources or receivers
    PFDTD_CK(cudaMemsetAsync(d->d_step, 0, sizeof(int64_t), d->stream));
    for (int i = 0; i < iters && rc == PFDTD_OK; ++i)
      rc = launch_tb(d, nullptr, 0, 0, d->stream);
    return rc;
  }
  for (int i = 0; i < iters && rc == PFDTD_OK; ++i) {
    rc = launch_update(d, d->cur_field(), d->past_field(), d->stream);
    d->swap_fields();
  }
  return rc;
}

int pfdtd_step(pfdtd_domain* d, int64_t step, int step_direction, void* out, int64_t num_steps) {
  if (int rc = check_domain(d)) return rc;
  if (step < 0) return fail(PFDTD_ERR_ARG, "negative step index");
  DeviceGuard g(d->device);
  int rc = prepare_run(d);
  if (rc) return rc;
  cudaStream_t s = d->stream;
  // Inject samples[step] (no receiver record), then update.
  PFDTD_CK(cudaMemcpyAsync(d->d_step, &step, sizeof(int64_t), cudaMemcpyHostToDevice, s));
  rc = launch_io(d, d->cur_field(), nullptr, 0, INT64_MAX, s);
  if (rc) return rc;
  rc = launch_dif_init(d, s);
  if (rc) return rc;
  rc = launch_update(d, d->cur_field(), d->past_field(), s);
  if (rc) return rc;
  rc = launch_dif(d, d->cur_field(), d->past_field(), s);
  if (rc) return rc;
  // kernels3d.cu:462-465: swap only while the direction is unchanged.
  if (d->past_step_direction == step_direction) d->swap_fields();
  d->past_step_direction = step_direction;
  PFDTD_CK(cudaStreamSynchronize(s));
  if (int e = check_pipeline(d)) return e;
  if (out && d->n_rec > 0 && step < num_steps) {
    std::vector<uint8_t> v(d->esize);
    for (int r = 0; r < d->n_rec; ++r) {
      const int64_t i = d->rec_idx_h[r];
      if (i < 0) continue;
      PFDTD_CK(cudaMemcpy(v.data(), (char*)d->cur_field() + (size_t)i * d->esize, d->esize,
                          cudaMemcpyDeviceToHost));
      const double val = from_storage(d->precision, v.data());
      if (d->precision == PFDTD_F64)
        ((double*)out)[(int64_t)r * num_steps + step] = val;
      else
        ((float*)out)[(int64_t)r * num_steps + step] = (float)val;
    }
  }
  return PFDTD_OK;
}

static int sample_ptr(pfdtd_domain* d, int64_t x, int64_t y, int64_t z, char** p) {
  const int64_t i = element_index(d, x, y, z, 0);
  if (i < 0) return fail(PFDTD_ERR_ARG, "element outside the grid");
  *p = (char*)d->cur_field() + (size_t)i * d->esize;
  return PFDTD_OK;
}

int pfdtd_set_sample(pfdtd_domain* d, int64_t x, int64_t y, int64_t z, double value) {
  if (int rc = check_domain(d)) return rc;
  DeviceGuard g(d->device);
  char* p;
  if (int rc = sample_ptr(d, x, y, z, &p)) return rc;
  uint8_t v[8];
  to_storage(d->precision, value, v);
  PFDTD_CK(cudaStreamSynchronize(d->stream));
  PFDTD_CK(cudaMemcpy(p, v, d->esize, cudaMemcpyHostToDevice));
  return PFDTD_OK;
}

int pfdtd_add_sample(pfdtd_domain* d, int64_t x, int64_t y, int64_t z, double value) {
  if (int rc = check_domain(d)) return rc;
  DeviceGuard g(d->device);
  char* p;
  if (int rc = sample_ptr(d, x, y, z, &p)) return rc;
  uint8_t v[8];
  PFDTD_CK(cudaStreamSynchronize(d->stream));
  PFDTD_CK(cudaMemcpy(v, p, d->esize, cudaMemcpyDeviceToHost));
  // Sum in the arithmetic type of the domain.
  double cur = from_storage(d->precision, v);
  double sum;
  if (d->precision == PFDTD_F64) sum = cur + value;
  else sum = (double)((float)cur + (float)value);
  to_storage(d->precision, sum, v);
  PFDTD_CK(cudaMemcpy(p, v, d->esize, cudaMemcpyHostToDevice));
  return PFDTD_OK;
}

int pfdtd_get_sample(pfdtd_domain* d, int64_t x, int64_t y, int64_t z, double* value) {
  if (int rc = check_domain(d)) return rc;
  if (!value) return fail(PFDTD_ERR_ARG, "null value pointer");
  DeviceGuard g(d->device);
  char* p;
  if (int rc = sample_ptr(d, x, y, z, &p)) return rc;
  uint8_t v[8];
  PFDTD_CK(cudaStreamSynchronize(d->stream));
  PFDTD_CK(cudaMemcpy(v, p, d->esize, cudaMemcpyDeviceToHost));
  *value = from_storage(d->precision, v);
  return PFDTD_OK;
}

int pfdtd_flip(pfdtd_domain* d) {
  if (int rc = check_domain(d)) return rc;
  d->swap_fields();
  return PFDTD_OK;
}

int pfdtd_reset_fields(pfdtd_domain* d) {
  if (int rc = check_domain(d)) return rc;
  DeviceGuard g(d->device);
  const size_t fbytes = (size_t)(d->NE + 2 * d->margin) * d->esize;
  for (int i = 0; i < 4; ++i)
    if (d->field_base[i]) PFDTD_CK(cudaMemsetAsync(d->field_base[i], 0, fbytes, d->stream));
  if (d->n_dif > 0)
    PFDTD_CK(cudaMemsetAsync(d->d_dif_state, 0, (size_t)d->n_dif * d->K * 4 * d->arith_size(),
                             d->stream));
  PFDTD_CK(cudaStreamSynchronize(d->stream));
  return PFDTD_OK;
}

int pfdtd_set_dif_filters(pfdtd_domain* d, int n_mat, const int32_t* flags, const double* coefs) {
  if (int rc = check_domain(d)) return rc;
  if (n_mat < 0 || (n_mat > 0 && (!flags || !coefs)))
    return fail(PFDTD_ERR_ARG, "invalid filter tables");
  d->dif_flags.assign(flags, flags + n_mat);
  d->dif_coefs.assign(coefs, coefs + (size_t)n_mat * 7);
  for (int m = 0; m < n_mat; ++m) {
    if (!flags[m]) continue;
    const double* f = coefs + 7 * m;
    for (int j = 0; j < 7; ++j)
      if (!(f[j] == f[j])) return fail(PFDTD_ERR_ARG, "filter coefficient is NaN");
  }
  d->classes_dirty = true;
  return PFDTD_OK;
}

int pfdtd_get_dif_count(pfdtd_domain* d, int64_t* n) {
  if (int rc = check_domain(d)) return rc;
  if (!n) return fail(PFDTD_ERR_ARG, "null output");
  DeviceGuard g(d->device);
  int rc = prepare_run(d);
  if (rc) return rc;
  *n = d->n_dif;
  return PFDTD_OK;
}

int pfdtd_get_field_ptr(pfdtd_domain* d, int which, void** d_ptr) {
  if (int rc = check_domain(d)) return rc;
  if (!d_ptr || (which != 0 && which != 1)) return fail(PFDTD_ERR_ARG, "invalid field selector");
  *d_ptr = which == PFDTD_FIELD_CURRENT ? d->cur_field() : d->past_field();
  return PFDTD_OK;
}

int pfdtd_download_field(pfdtd_domain* d, int which, void* host) {
  void* p = nullptr;
  if (int rc = pfdtd_get_field_ptr(d, which, &p)) return rc;
  if (!host) return fail(PFDTD_ERR_ARG, "null host buffer");
  DeviceGuard g(d->device);
  PFDTD_CK(cudaStreamSynchronize(d->stream));
  PFDTD_CK(cudaMemcpy(host, p, (size_t)d->NE * d->esize, cudaMemcpyDeviceToHost));
  return PFDTD_OK;
}

int pfdtd_upload_field(pfdtd_domain* d, int which, const void* host) {
  void* p = nullptr;
  if (int rc = pfdtd_get_field_ptr(d, which, &p)) return rc;
  if (!host) return fail(PFDTD_ERR_ARG, "null host buffer");
  DeviceGuard g(d->device);
  PFDTD_CK(cudaStreamSynchronize(d->stream));
  PFDTD_CK(cudaMemcpy(p, host, (size_t)d->NE * d->esize, cudaMemcpyHostToDevice));
  return PFDTD_OK;
}

int pfdtd_set_kernel(pfdtd_domain* d, int variant) {
  if (int rc = check_domain(d)) return rc;
  if (variant < PFDTD_KERNEL_AUTO || variant > PFDTD_KERNEL_TMA)
    return fail(PFDTD_ERR_ARG, "unknown kernel variant");
  if (variant == PFDTD_KERNEL_TMA && d->nodes_set && !d->classes_dirty && !tma_supported(d))
    return fail(PFDTD_ERR_UNSUPPORTED, "TMA update needs 16-byte aligned rows (X a multiple of 16)");
  d->kernel_variant = variant;
  if (d->graph.exec) {
    cudaGraphExecDestroy(d->graph.exec);
    d->graph.exec = nullptr;
  }
  return PFDTD_OK;
}

int pfdtd_set_tile(pfdtd_domain* d, int tile) {
  if (int rc = check_domain(d)) return rc;
  if (tile < -1 || tile >= tma_tile_count()) return fail(PFDTD_ERR_ARG, "unknown tile shape");
  d->tma_tile = tile;
  if (d->graph.exec) {
    cudaGraphExecDestroy(d->graph.exec);
    d->graph.exec = nullptr;
  }
  return PFDTD_OK;
}

int pfdtd_get_kernel(pfdtd_domain* d, int* variant) {
  if (int rc = check_domain(d)) return rc;
  if (!variant) return fail(PFDTD_ERR_ARG, "null output");
  *variant = uses_tma(d) ? PFDTD_KERNEL_TMA : PFDTD_KERNEL_ZMARCH;
  if (d->tb_depth >= 2 && tb_active(d)) *variant = PFDTD_KERNEL_TB;
  return PFDTD_OK;
}

int pfdtd_set_temporal_block(pfdtd_domain* d, int depth) {
  if (int rc = check_domain(d)) return rc;
  if (depth != 0 && (depth < 2 || depth > 4))
    return fail(PFDTD_ERR_ARG, "temporal block depth must be 0 (off), 2, 3 or 4");
  d->tb_depth = depth;
  if (d->graph.exec) {
    cudaGraphExecDestroy(d->graph.exec);
    d->graph.exec = nullptr;
  }
  return PFDTD_OK;
}

int pfdtd_get_temporal_block(pfdtd_domain* d, int* depth, int* active, char* why,
                             size_t why_len) {
  if (int rc = check_domain(d)) return rc;
  DeviceGuard g(d->device);
  if (d->tb_depth >= 2 && d->nodes_set && d->n_mat > 0) {
    if (int rc = prepare_run(d)) return rc;
  }
  std::string w = "active";
  const int a = tb_usable(d, &w);
  if (depth) *depth = d->tb_depth;
  if (active) *active = a;
  if (why && why_len > 0) {
    std::strncpy(why, w.c_str(), why_len - 1);
    why[why_len - 1] = 0;
  }
  return PFDTD_OK;
}

int pfdtd_set_tb_shape(pfdtd_domain* d, int shape) {
  if (int rc = check_domain(d)) return rc;
  if (shape < -1 || shape > 3) return fail(PFDTD_ERR_ARG, "blocked tile shape must be -1..3");
  d->tb_shape = shape;
  if (d->graph.exec) {
    cudaGraphExecDestroy(d->graph.exec);
    d->graph.exec = nullptr;
  }
  return PFDTD_OK;
}

// Time one update configuration: `iters` launches after one warm-up launch,
// returned as milliseconds per step.
static int time_config(pfdtd_domain* d, int iters, double* ms_per_step) {
  cudaStream_t s = d->stream;
  const bool tb = d->tb_depth >= 2 && tb_active(d);
  auto launch = [&]() -> int {
    if (tb) return launch_tb(d, nullptr, 0, 0, s);
    int rc = launch_update(d, d->cur_field(), d->past_field(), s);
    d->swap_fields();
    return rc;
  };
  PFDTD_CK(cudaMemsetAsync(d->d_step, 0, sizeof(int64_t), s));
  if (int rc = launch()) return rc;
  cudaEvent_t e0, e1;
  PFDTD_CK(cudaEventCreate(&e0));
  PFDTD_CK(cudaEventCreate(&e1));
  int rc = PFDTD_OK;
  cudaEventRecord(e0, s);
  for (int i = 0; i < iters && rc == PFDTD_OK; ++i) rc = launch();
  cudaEventRecord(e1, s);
  cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_fail(e, "autotune timing", __FILE__, __LINE__);
  *ms_per_step = (double)ms / ((double)iters * (tb ? d->tb_depth : 1));
  return PFDTD_OK;
}

int pfdtd_autotune(pfdtd_domain* d, int max_depth, int iters, int* best_depth, int* best_shape,
                   double* best_ms_per_step) {
  if (int rc = check_domain(d)) return rc;
  if (max_depth != 0 && (max_depth < 2 || max_depth > 4))
    return fail(PFDTD_ERR_ARG, "maximum depth must be 0, 2, 3 or 4");
  if (iters < 1) return fail(PFDTD_ERR_ARG, "iteration count must be positive");
  DeviceGuard g(d->device);
  const int depth0 = d->tb_depth, shape0 = d->tb_shape;
  d->tb_depth = max_depth >= 2 ? 2 : 0;  // allocate the blocking buffers if needed
  int rc = prepare_run(d);
  if (rc) {
    d->tb_depth = depth0;
    return rc;
  }
  // The timing launches advance the fields: keep a copy and put it back.
  cudaStream_t s = d->stream;
  const size_t fbytes = (size_t)(d->NE + 2 * d->margin) * d->esize;
  void* keep[2] = {nullptr, nullptr};
  for (int i = 0; i < 2; ++i) {
    if (cudaMallocAsync(&keep[i], fbytes, s) != cudaSuccess) {
      cudaGetLastError();
      if (keep[0]) cudaFreeAsync(keep[0], s);
      d->tb_depth = depth0;
      return fail(PFDTD_ERR_NOMEM, "autotune field snapshot allocation failed");
    }
  }
  // the IWB closure pass also advances the DIF filter states: keep them too
  void* keep_dif = nullptr;
  const size_t dbytes = d->n_dif > 0 ? (size_t)d->n_dif * d->K * 4 * d->arith_size() : 0;
  {
    cudaError_t e = cudaMemcpyAsync(keep[0], d->field_base[d->cur], fbytes,
                                    cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(keep[1], d->field_base[d->prev], fbytes, cudaMemcpyDeviceToDevice, s);
    int code = PFDTD_ERR_CUDA;
    if (e == cudaSuccess && dbytes) {
      e = cudaMallocAsync(&keep_dif, dbytes, s);
      if (e != cudaSuccess) {
        keep_dif = nullptr;
        code = PFDTD_ERR_NOMEM;
      } else {
        e = cudaMemcpyAsync(keep_dif, d->d_dif_state, dbytes, cudaMemcpyDeviceToDevice, s);
      }
    }
    if (e != cudaSuccess) {
      cudaGetLastError();
      cudaFreeAsync(keep[0], s);
      cudaFreeAsync(keep[1], s);
      if (keep_dif) cudaFreeAsync(keep_dif, s);
      d->tb_depth = depth0;
      return code == PFDTD_ERR_NOMEM
                 ? fail(code, "autotune filter-state snapshot allocation failed")
                 : cuda_fail(e, "autotune snapshot", __FILE__, __LINE__);
    }
  }
  double best = 1e300;
  int bd = 0, bs = -1;
  struct Cand { int depth, shape; };
  std::vector<Cand> cands{{0, -1}};
  for (int depth = 2; depth <= max_depth; ++depth)
    for (int shape = 0; shape < 4; ++shape) cands.push_back({depth, shape});
  for (const Cand& c : cands) {
    d->tb_depth = c.depth;
    d->tb_shape = c.shape;
    if (c.depth >= 2 && (!tb_active(d) || !tb_shape_valid(d, c.shape))) continue;
    double ms = 0;
    rc = time_config(d, iters, &ms);
    if (rc == PFDTD_ERR_ARG || rc == PFDTD_ERR_UNSUPPORTED) {  // shape not built here
      rc = PFDTD_OK;
      continue;
    }
    if (rc) break;
    if (ms < best) {
      best = ms;
      bd = c.depth;
      bs = c.shape;
    }
  }
  if (rc == PFDTD_OK) {
    cudaError_t e = cudaMemcpyAsync(d->field_base[d->cur], keep[0], fbytes,
                                    cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d->field_base[d->prev], keep[1], fbytes, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess && keep_dif)
      e = cudaMemcpyAsync(d->d_dif_state, keep_dif, dbytes, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) rc = cuda_fail(e, "autotune field restore", __FILE__, __LINE__);
  }
  cudaFreeAsync(keep[0], s);
  cudaFreeAsync(keep[1], s);
  if (keep_dif) cudaFreeAsync(keep_dif, s);
  cudaError_t e = cudaStreamSynchronize(s);
  if (rc == PFDTD_OK && e != cudaSuccess) rc = cuda_fail(e, "autotune", __FILE__, __LINE__);
  if (d->graph.exec) {
    cudaGraphExecDestroy(d->graph.exec);
    d->graph.exec = nullptr;
  }
  if (rc) {
    d->tb_depth = depth0;
    d->tb_shape = shape0;
    return rc;
  }
  d->tb_depth = bd;
  d->tb_shape = bs;
  if (best_depth) *best_depth = bd;
  if (best_shape) *best_shape = bs;
  if (best_ms_per_step) *best_ms_per_step = best;
  return PFDTD_OK;
}

int pfdtd_synchronize(pfdtd_domain* d) {
  if (int rc = check_domain(d)) return rc;
  DeviceGuard g(d->device);
  PFDTD_CK(cudaStreamSynchronize(d->stream));
  return check_pipeline(d);
}

int pfdtd_get_stream(pfdtd_domain* d, void** stream) {
  if (int rc = check_domain(d)) return rc;
  if (!stream) return fail(PFDTD_ERR_ARG, "null stream pointer");
  *stream = (void*)d->stream;
  return PFDTD_OK;
}

}  // extern "C"
