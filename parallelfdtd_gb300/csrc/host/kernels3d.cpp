// launchFDTD3d / launchFDTD3dDouble / launchFDTD3dStep with the reference's
// signatures (ParallelFDTD src/kernels/kernels3d.h:49-90) over the C ABI.
//
// Source samples are evaluated on the host with the reference's
// SimulationParameters::getSourceSample(Double) for every step up front and
// handed to the device as a table; receivers and sources are addressed by
// the element coordinates the reference computes
// (SimulationParameters::getSource/ReceiverElementCoordinates).
#include "kernels3d.h"

#include <vector>

namespace {

thread_local bool (*t_interrupt)(void) = nullptr;
int interrupt_trampoline(void) { return (t_interrupt && t_interrupt()) ? 1 : 0; }

void check(int rc, const char* what) {
  if (rc != PFDTD_OK && rc != PFDTD_INTERRUPTED) {
    c_log_msg(LOG_ERROR, "%s: %s", what, pfdtd_last_error());
    throw(-1);
  }
}

struct IoCache {
  int64_t serial = -1;
  const SimulationParameters* sp = nullptr;
  unsigned long long version = ~0ull;
  bool dbl = false;
};
thread_local IoCache t_io;

// Upload scheme, source table and receiver positions unless unchanged.
void configure(CudaMesh* m, SimulationParameters* sp, bool dbl) {
  pfdtd_domain* d = m->getDomain();
  if (!d) {
    c_log_msg(LOG_ERROR, "launchFDTD3d - mesh has no partition (call makePartition)");
    throw(-1);
  }
  check(pfdtd_set_scheme(d, (int)sp->getUpdateType()), "launchFDTD3d - update type");
  int64_t serial = -1;
  pfdtd_get_serial(d, &serial);
  if (t_io.serial == serial && t_io.sp == sp && t_io.version == sp->getVersion() &&
      t_io.dbl == dbl)
    return;
  const unsigned n_src = sp->getNumSources(), steps = sp->getNumSteps();
  std::vector<int64_t> xyz(3 * (size_t)n_src);
  std::vector<int32_t> type(n_src);
  std::vector<float> sf;
  std::vector<double> sd;
  if (dbl) sd.assign((size_t)n_src * steps, 0.0);
  else sf.assign((size_t)n_src * steps, 0.f);
  for (unsigned i = 0; i < n_src; ++i) {
    nv::Vec3i p = sp->getSourceElementCoordinates(i);
    xyz[3 * i] = p.x;
    xyz[3 * i + 1] = p.y;
    xyz[3 * i + 2] = p.z;
    type[i] = (int32_t)sp->getSource(i).getSourceType();
    for (unsigned s = 0; s < steps; ++s) {
      if (dbl) sd[(size_t)i * steps + s] = sp->getSourceSampleDouble(i, s);
      else sf[(size_t)i * steps + s] = sp->getSourceSample(i, s);
    }
  }
  check(pfdtd_set_sources(d, (int)n_src, xyz.data(), type.data(),
                          dbl ? (const void*)sd.data() : (const void*)sf.data(), steps),
        "launchFDTD3d - sources");
  const unsigned n_rec = sp->getNumReceivers();
  std::vector<int64_t> rxyz(3 * (size_t)n_rec);
  for (unsigned i = 0; i < n_rec; ++i) {
    nv::Vec3i p = sp->getReceiverElementCoordinates(i);
    rxyz[3 * i] = p.x;
    rxyz[3 * i + 1] = p.y;
    rxyz[3 * i + 2] = p.z;
  }
  check(pfdtd_set_receivers(d, (int)n_rec, rxyz.data()), "launchFDTD3d - receivers");
  t_io.serial = serial;
  t_io.sp = sp;
  t_io.version = sp->getVersion();
  t_io.dbl = dbl;
}

float run(CudaMesh* m, SimulationParameters* sp, void* out, bool (*interrupt)(void),
          void (*progress)(int, int, float), bool dbl) {
  configure(m, sp, dbl);
  t_interrupt = interrupt;
  double sec = 0.0;
  const int rc = pfdtd_run(m->getDomain(), sp->getNumSteps(), out,
                           interrupt ? interrupt_trampoline : nullptr, progress, &sec);
  t_interrupt = nullptr;
  check(rc, dbl ? "launchFDTD3dDouble" : "launchFDTD3d");
  if (rc == PFDTD_INTERRUPTED) c_log_msg(LOG_INFO, "launchFDTD3d interrupted");
  m->syncViews();
  return (float)sec;
}

}  // namespace

float launchFDTD3d(CudaMesh* d_mesh, SimulationParameters* sp, float* h_return_ptr,
                   bool (*interruptCallback)(void), void (*progressCallback)(int, int, float)) {
  return run(d_mesh, sp, h_return_ptr, interruptCallback, progressCallback, false);
}

float launchFDTD3dDouble(CudaMesh* d_mesh, SimulationParameters* sp, double* h_return_ptr,
                         bool (*interruptCallback)(void),
                         void (*progressCallback)(int, int, float)) {
  return run(d_mesh, sp, h_return_ptr, interruptCallback, progressCallback, true);
}

void launchFDTD3dCaptures(CudaMesh* d_mesh, SimulationParameters* sp, float* h_return_ptr,
                          int n_capture, const int64_t* capture_step,
                          const int32_t* capture_orientation, const int64_t* capture_slice,
                          float* const* p_out, uint8_t* const* pos_out) {
  configure(d_mesh, sp, false);
  check(pfdtd_run_captures(d_mesh->getDomain(), sp->getNumSteps(), h_return_ptr, n_capture,
                           capture_step, capture_orientation, capture_slice, p_out, pos_out),
        "launchFDTD3dCaptures");
  d_mesh->syncViews();
}

void launchFDTD3dStep(CudaMesh* d_mesh, SimulationParameters* sp, float* h_return_ptr,
                      unsigned int step, int step_direction,
                      void (*progressCallback)(int, int, float)) {
  configure(d_mesh, sp, false);
  check(pfdtd_step(d_mesh->getDomain(), step, step_direction, h_return_ptr, sp->getNumSteps()),
        "launchFDTD3dStep");
  d_mesh->syncViews();
  if (progressCallback && (step % PROGRESS_MOD) == 0)
    progressCallback((int)step, (int)sp->getNumSteps(), 0.f);
}
