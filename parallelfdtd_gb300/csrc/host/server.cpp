// Request loop with continuous batching over the C ABI (pfdtd_server.h).
//
// One scheduler thread per server and a few set-up workers.  The scheduler
// keeps a FIFO of submitted requests and a set of running ones.  Each pass it
// (1) retires running requests whose domain stream has drained: receivers to
// the host, domain destroyed, memory back to the budget; (2) admits queued
// requests in arrival order while a slot is free and the head request's
// estimated bytes fit beside the running and admitted ones: it reserves the
// bytes and the slot and hands the request to a set-up worker, which creates
// the domain on its own stream, uploads the room, builds the node classes and
// queues the whole run with pfdtd_run_async, then makes the request running.
// Set-up is host work (node bytes re-laid, class tables, graph capture) of up
// to seconds for the largest rooms; on the workers it overlaps the running
// requests, the retirements and the other set-ups.  Nothing waits on the
// device as a whole: queries and synchronisations are per stream and
// allocations are stream-ordered.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "pfdtd.h"
#include "pfdtd_server.h"

namespace pfdtd {
int fail(int code, const std::string& msg);
}
using pfdtd::fail;

struct pfdtd_request {
  int64_t X = 0, Y = 0, Z = 0;
  int fields = 1, precision = PFDTD_F32, scheme = PFDTD_SRL_FORWARD;
  int64_t steps = 0;
  std::vector<uint8_t> pos, mat;
  bool nodes_set = false;
  int64_t n_boundary = 0;  // nodes with a boundary update (for the filter-state estimate)
  std::vector<double> materials;
  int n_mat = 0, n_coef = 20;
  std::vector<int32_t> dif_flags;
  std::vector<double> dif_coefs;
  // lambda = sqrt(1/3), as SimulationParameters::setUpdateType sets it
  double params[4] = {std::sqrt(1.0 / 3.0), 1.0 / 3.0, 1.0 / 3.0, 0.0};
  int n_src = 0;
  int64_t n_samples = 0;
  std::vector<int64_t> src_xyz;
  std::vector<int32_t> src_field, src_type;
  std::vector<double> samples;
  int n_rec = 0;
  std::vector<int64_t> rec_xyz;
  std::vector<int32_t> rec_field;
  int tb_depth = 0;
};

namespace {

using Clock = std::chrono::steady_clock;

// Requests set up at once (each on its own worker thread).
constexpr int kSetupWorkers = 4;

size_t storage_size(int precision) {
  return precision == PFDTD_F64 ? 8 : (precision == PFDTD_F32 ? 4 : 2);
}
size_t arith_size(int precision) { return precision == PFDTD_F64 ? 8 : 4; }

// Fields that carry a source: the work a request asks for.  A batched request
// rounds its field count up to a power of two; the padding fields are
// computed but are not counted as node-updates.
int source_fields(const pfdtd_request* r) {
  if (r->n_src <= 0) return r->fields;
  std::vector<bool> seen((size_t)r->fields, false);
  int n = 0;
  for (int32_t f : r->src_field)
    if (f >= 0 && f < r->fields && !seen[(size_t)f]) {
      seen[(size_t)f] = true;
      ++n;
    }
  return n > 0 ? n : r->fields;
}

struct Job {
  pfdtd_request* req = nullptr;
  int state = PFDTD_REQ_QUEUED;
  // The request's domain: one with all its fields (part_field {-1}), or (an
  // IWB request with several fields, see split_fields) one single-field
  // domain that runs the fields carrying a source one after another,
  // part_field listing them and phase the one running.
  pfdtd_domain* dom = nullptr;
  std::vector<int> part_field;
  size_t phase = 0;
  uint64_t bytes = 0;
  Clock::time_point t_submit, t_admit, t_done;
  std::vector<uint8_t> result;
  std::string error;
};

}  // namespace

struct pfdtd_server {
  int device = 0;
  uint64_t budget = 0;
  int max_active = 1;
  std::mutex mu;
  std::condition_variable cv_sched, cv_done;
  std::deque<int64_t> queue;
  std::vector<int64_t> active;
  std::map<int64_t, Job> jobs;
  int64_t next_ticket = 1;
  bool stop = false;
  int in_transit = 0;  // requests being retired with the lock released
  int admitting = 0;   // requests handed to a set-up worker and not yet running
  std::deque<int64_t> to_admit;
  std::condition_variable cv_work;
  bool workers_stop = false;
  std::thread thread;
  std::vector<std::thread> workers;
  pfdtd_server_stats st{};
};

namespace {

// x extent of the domain a request runs on.  The TMA update kernels need
// 16-byte aligned field rows (X * fields * element size a multiple of 16);
// other rooms run the slower z-march kernel.  A request whose rows are not
// aligned, whose x = X-1 face holds no inside node, and whose sources and
// receivers lie below X, runs on a domain padded with outside nodes up to the
// next multiple of 16, as the reference pads its meshes to the block size
// (cudaMesh.cu:253-304).  No inside node then reads a different neighbour
// (the padding and the x = X-1 face are outside and stay 0), so the
// receivers are those of the unpadded room.
bool split_fields(const pfdtd_request* r);
int64_t domain_x(const pfdtd_request* r) {
  const int64_t X = r->X, Xp = (X + 15) / 16 * 16;
  const int64_t K = split_fields(r) ? 1 : r->fields;
  if (Xp == X || (X * K * (int64_t)storage_size(r->precision)) % 16 == 0 || !r->nodes_set)
    return X;
  for (int i = 0; i < r->n_src; ++i)
    if (r->src_xyz[3 * (size_t)i] >= X) return X;
  for (int i = 0; i < r->n_rec; ++i)
    if (r->rec_xyz[3 * (size_t)i] >= X) return X;
  for (int64_t row = 0; row < r->Y * r->Z; ++row)
    if (r->pos[(size_t)(row * X + X - 1)] & 0x80u) return X;
  return Xp;
}

// A request with several fields runs its fields that carry a source one
// after another on one single-field domain (fields zeroed between them) when
// a batched domain would not stream them at the single-field rate: IWB (its
// streaming TMA kernel and closure pass are single-field; batched IWB fields
// take the column z-march), a field count that the batched TMA kernel does
// not take (not a multiple of 4), or fields without a source (computed in a
// batched domain, skipped here: the batched kernel streams a field at most
// ~1.1x the single-field rate, so every unused field costs more than it
// saves).  Every field of a batched domain is bit-identical to the same field
// run alone, so the receivers do not change.  The domain is set up once.
bool split_fields(const pfdtd_request* r) {
  if (r->fields <= 1) return false;
  return r->scheme == PFDTD_IWB || r->fields % 4 != 0 || source_fields(r) < r->fields;
}

uint64_t estimate_domain_bytes(const pfdtd_request* r, uint64_t K, int n_src, int n_rec) {
  const uint64_t es = storage_size(r->precision), as = arith_size(r->precision);
  const uint64_t DX = (uint64_t)domain_x(r);
  const uint64_t N = (uint64_t)(DX * r->Y * r->Z);
  const uint64_t align = 256 / es;
  const uint64_t margin = ((DX + 64) * K + align - 1) / align * align;
  const uint64_t nfields = r->tb_depth >= 2 ? 4 : 2;
  uint64_t b = nfields * (N * K + 2 * margin) * es;
  b += 2 * (N + 1 + DX) + N + 64;                              // node bytes, class ids
  if (DX % 16 != 0 && (DX * K * es) % 16 == 0) b += 2 * N;  // class ids, 16-byte rows (TMA)
  b += (uint64_t)n_rec * (uint64_t)r->steps * as;            // receiver buffer
  b += (uint64_t)n_src * (uint64_t)r->n_samples * as + 4096;  // sources
  bool dif = false;
  for (int32_t f : r->dif_flags) dif |= f != 0;
  if (dif) b += (uint64_t)r->n_boundary * (K * 4 * as + 8);   // filter states + node list
  if (r->scheme == PFDTD_IWB) {
    b += 5 * N;  // closed-neighbour masks and geometry codes
    if (K == 1 && r->precision != PFDTD_F64) {
      // closure-node records (16 B; nodes closed only diagonally come on top
      // of the face-boundary count, bounded here by the same number again)
      b += 2 * (uint64_t)r->n_boundary * 16;
      if (dif) b += 4 * N;  // the DIF nodes' neighbour sums, one float per node
    }
  }
  return b + (4u << 20);                                     // tables, graphs, scratch
}

uint64_t estimate_bytes(const pfdtd_request* r) {
  return estimate_domain_bytes(r, split_fields(r) ? 1 : (uint64_t)r->fields, r->n_src, r->n_rec);
}

// The request's sources and receivers on field f (all of them for f < 0).
void part_ids(const pfdtd_request* r, int f, std::vector<int>& src_ids, std::vector<int>& rec_ids) {
  src_ids.clear();
  rec_ids.clear();
  for (int i = 0; i < r->n_src; ++i)
    if (f < 0 || r->src_field[(size_t)i] == f) src_ids.push_back(i);
  for (int i = 0; i < r->n_rec; ++i)
    if (f < 0 || r->rec_field[(size_t)i] == f) rec_ids.push_back(i);
}

// Give domain d the sources and receivers of part_field (moved to field 0;
// -1: every field as the request numbers them).
int set_part_io(pfdtd_domain* d, const pfdtd_request* r, int part_field) {
  std::vector<int> src_ids, rec_ids;
  part_ids(r, part_field, src_ids, rec_ids);
  const size_t as = arith_size(r->precision);
  const size_t ns = (size_t)r->n_samples;
  std::vector<uint8_t> samples(src_ids.size() * ns * as);
  std::vector<int64_t> sxyz, rxyz;
  std::vector<int32_t> sfield, stype, rfield;
  for (size_t k = 0; k < src_ids.size(); ++k) {
    const int i = src_ids[k];
    for (int c = 0; c < 3; ++c) sxyz.push_back(r->src_xyz[3 * (size_t)i + c]);
    sfield.push_back(part_field < 0 ? r->src_field[(size_t)i] : 0);
    stype.push_back(r->src_type[(size_t)i]);
    const double* v = r->samples.data() + (size_t)i * ns;
    for (size_t t = 0; t < ns; ++t) {
      if (as == 8) {
        std::memcpy(samples.data() + (k * ns + t) * 8, v + t, 8);
      } else {
        const float f = (float)v[t];
        std::memcpy(samples.data() + (k * ns + t) * 4, &f, 4);
      }
    }
  }
  for (int i : rec_ids) {
    for (int c = 0; c < 3; ++c) rxyz.push_back(r->rec_xyz[3 * (size_t)i + c]);
    rfield.push_back(part_field < 0 ? r->rec_field[(size_t)i] : 0);
  }
  int rc = pfdtd_set_sources_batched(d, (int)src_ids.size(), sxyz.data(), sfield.data(),
                                     stype.data(), samples.data(), r->n_samples);
  if (!rc) rc = pfdtd_set_receivers_batched(d, (int)rec_ids.size(), rxyz.data(), rfield.data());
  return rc;
}

// Create and set up the request's domain and queue the run of its first
// part.  Returns the status; on failure the domain is destroyed and the
// message kept.
int admit(pfdtd_server* s, Job& j) {
  pfdtd_request* r = j.req;
  const int64_t DX = domain_x(r);
  std::vector<uint8_t> ppos, pmat;  // node bytes re-laid on the padded rows
  if (DX != r->X) {
    ppos.assign((size_t)(DX * r->Y * r->Z), 0);
    pmat.assign(ppos.size(), 0);
    for (int64_t row = 0; row < r->Y * r->Z; ++row) {
      std::memcpy(&ppos[(size_t)(row * DX)], &r->pos[(size_t)(row * r->X)], (size_t)r->X);
      std::memcpy(&pmat[(size_t)(row * DX)], &r->mat[(size_t)(row * r->X)], (size_t)r->X);
    }
  }
  j.part_field.clear();
  j.phase = 0;
  if (split_fields(r)) {
    std::vector<bool> seen((size_t)r->fields, false);
    for (int i = 0; i < r->n_src; ++i) {
      const int f = r->src_field[(size_t)i];
      if (f >= 0 && f < r->fields && !seen[(size_t)f]) {
        seen[(size_t)f] = true;
        j.part_field.push_back(f);
      }
    }
    std::sort(j.part_field.begin(), j.part_field.end());
  }
  if (j.part_field.empty()) j.part_field.push_back(-1);
  j.result.assign((size_t)r->n_rec * (size_t)r->steps * arith_size(r->precision), 0);
  const int K = j.part_field[0] < 0 ? r->fields : 1;
  pfdtd_domain* d = nullptr;
  int rc = pfdtd_create_batched(DX, r->Y, r->Z, K, r->precision, s->device, &d);
  if (rc) {
    j.error = pfdtd_last_error();
    return rc;
  }
  rc = DX != r->X ? pfdtd_set_nodes(d, ppos.data(), pmat.data(), 0)
                  : pfdtd_set_nodes(d, r->pos.data(), r->mat.data(), 0);
  if (!rc) rc = pfdtd_set_scheme(d, r->scheme);
  if (!rc) rc = pfdtd_set_materials(d, r->materials.data(), r->n_mat, r->n_coef);
  if (!rc && !r->dif_flags.empty())
    rc = pfdtd_set_dif_filters(d, (int)r->dif_flags.size(), r->dif_flags.data(),
                               r->dif_coefs.data());
  if (!rc) rc = pfdtd_set_params(d, r->params);
  if (!rc) rc = set_part_io(d, r, j.part_field[0]);
  if (!rc) rc = pfdtd_set_temporal_block(d, r->tb_depth);
  if (!rc) rc = pfdtd_run_async(d, r->steps);
  if (rc) {
    j.error = pfdtd_last_error();
    pfdtd_destroy(d);
    return rc;
  }
  j.dom = d;
  return PFDTD_OK;
}

// Receivers of the finished part `phase` into the request's receiver order
// (receivers on fields without a source stay 0, as in a batched run).
int collect_part(Job& j) {
  const pfdtd_request* r = j.req;
  const int f = j.part_field[j.phase];
  if (f < 0) return pfdtd_fetch_receivers(j.dom, j.result.data());
  std::vector<int> src_ids, rec_ids;
  part_ids(r, f, src_ids, rec_ids);
  if (rec_ids.empty()) return PFDTD_OK;
  const size_t row = (size_t)r->steps * arith_size(r->precision);
  std::vector<uint8_t> part(rec_ids.size() * row);
  if (int rc = pfdtd_fetch_receivers(j.dom, part.data())) return rc;
  for (size_t k = 0; k < rec_ids.size(); ++k)
    std::memcpy(j.result.data() + (size_t)rec_ids[k] * row, part.data() + k * row, row);
  return PFDTD_OK;
}

// A part has finished and another follows: its receivers out, fields (and
// filter states) zeroed, the next part's sources and receivers set, its run
// queued.  On failure the domain is destroyed and the message kept.
int advance(Job& j) {
  int rc = collect_part(j);
  if (!rc) {
    j.phase++;
    rc = pfdtd_reset_fields(j.dom);
  }
  if (!rc) rc = set_part_io(j.dom, j.req, j.part_field[j.phase]);
  if (!rc) rc = pfdtd_run_async(j.dom, j.req->steps);
  if (rc) {
    j.error = pfdtd_last_error();
    pfdtd_destroy(j.dom);
    j.dom = nullptr;
  }
  return rc;
}

// Receivers of the last part to the host and the domain destroyed.
int retire(Job& j) {
  int rc = collect_part(j);
  if (rc) j.error = pfdtd_last_error();
  pfdtd_destroy(j.dom);
  j.dom = nullptr;
  return rc;
}

// Set-up worker: takes admitted requests (no domain yet: set up) and
// requests between two parts (advance) in order, does that with the lock
// released, then makes the request running (or failed).
void setup_worker(pfdtd_server* s) {
  std::unique_lock<std::mutex> lk(s->mu);
  for (;;) {
    s->cv_work.wait(lk, [&] { return !s->to_admit.empty() || s->workers_stop; });
    if (s->to_admit.empty()) break;
    const int64_t t = s->to_admit.front();
    s->to_admit.pop_front();
    Job& j = s->jobs[t];  // std::map: the reference stays valid while unlocked
    const bool first = j.dom == nullptr;
    lk.unlock();
    const Clock::time_point t0 = Clock::now();
    const int rc = first ? admit(s, j) : advance(j);
    const double dt = std::chrono::duration<double>(Clock::now() - t0).count();
    lk.lock();
    s->admitting--;
    s->st.setup_seconds += dt;
    if (rc) {
      j.state = PFDTD_REQ_FAILED;
      j.t_done = Clock::now();
      s->st.bytes_in_use -= j.bytes;
      s->st.failed++;
      s->cv_done.notify_all();
    } else {
      s->active.push_back(t);
      if (first) s->st.admitted++;
      s->st.running = (int64_t)s->active.size();
      s->st.max_running = std::max<int>(s->st.max_running, (int)s->active.size());
    }
    s->cv_sched.notify_one();
  }
}

void scheduler(pfdtd_server* s) {
  std::unique_lock<std::mutex> lk(s->mu);
  for (;;) {
    bool progress = false;
    // retire finished requests
    for (size_t i = 0; i < s->active.size();) {
      Job& j = s->jobs[s->active[i]];
      int done = 0;
      const int q = pfdtd_query(j.dom, &done);
      if (q == PFDTD_OK && !done) {
        ++i;
        continue;
      }
      const int64_t ticket = s->active[i];
      s->active.erase(s->active.begin() + (ptrdiff_t)i);
      if (q == PFDTD_OK && j.phase + 1 < j.part_field.size()) {
        // another part follows: a set-up worker queues it; the request keeps
        // its slot and its memory
        s->admitting++;
        s->to_admit.push_back(ticket);
        s->cv_work.notify_one();
        s->st.running = (int64_t)s->active.size();
        progress = true;
        continue;
      }
      s->in_transit++;
      lk.unlock();
      const Clock::time_point t0 = Clock::now();
      const int rc = retire(j);
      const double dt = std::chrono::duration<double>(Clock::now() - t0).count();
      lk.lock();
      s->in_transit--;
      s->st.retire_seconds += dt;
      j.t_done = Clock::now();
      j.state = rc == PFDTD_OK && q == PFDTD_OK ? PFDTD_REQ_DONE : PFDTD_REQ_FAILED;
      s->st.bytes_in_use -= j.bytes;
      s->st.running = (int64_t)s->active.size();
      if (j.state == PFDTD_REQ_DONE) {
        s->st.completed++;
        const pfdtd_request* r = j.req;
        s->st.node_updates += (double)r->X * (double)r->Y * (double)(r->Z - 2) *
                              (double)r->steps * (double)source_fields(r);
      } else {
        s->st.failed++;
      }
      progress = true;
      s->cv_done.notify_all();
    }
    // admit in arrival order while a slot and the memory are free: reserve
    // both and hand the request to a set-up worker
    while (!s->stop && !s->queue.empty() &&
           (int)s->active.size() + s->admitting < s->max_active) {
      const int64_t t = s->queue.front();
      Job& j = s->jobs[t];
      if (s->st.bytes_in_use + j.bytes > s->budget) break;
      s->queue.pop_front();
      s->st.queued = (int64_t)s->queue.size();
      s->st.bytes_in_use += j.bytes;
      s->st.bytes_peak = std::max(s->st.bytes_peak, s->st.bytes_in_use);
      j.state = PFDTD_REQ_RUNNING;
      j.t_admit = Clock::now();
      s->admitting++;
      s->to_admit.push_back(t);
      s->cv_work.notify_one();
      progress = true;
    }
    if (s->stop && s->active.empty() && s->admitting == 0) break;
    if (!progress) s->cv_sched.wait_for(lk, std::chrono::microseconds(200));
  }
  // queued requests left at shutdown fail
  for (int64_t t : s->queue) {
    Job& j = s->jobs[t];
    j.state = PFDTD_REQ_FAILED;
    j.error = "server stopped before admission";
    s->st.failed++;
  }
  s->queue.clear();
  s->cv_done.notify_all();
}

int check_req(const pfdtd_request* r) {
  return r ? PFDTD_OK : fail(PFDTD_ERR_ARG, "null request");
}

}  // namespace

extern "C" {

int pfdtd_request_create(int64_t dim_x, int64_t dim_y, int64_t dim_z, int fields, int precision,
                         int scheme, int64_t steps, pfdtd_request** out) {
  if (!out) return fail(PFDTD_ERR_ARG, "null output");
  if (dim_x <= 0 || dim_y <= 0 || dim_z < 3 || steps < 0)
    return fail(PFDTD_ERR_ARG, "invalid dimensions or step count");
  if (fields < 1 || fields > 64 || (fields & (fields - 1)))
    return fail(PFDTD_ERR_ARG, "fields must be a power of two in 1..64");
  if (precision < PFDTD_F32 || precision > PFDTD_BF16) return fail(PFDTD_ERR_ARG, "precision");
  if (scheme < PFDTD_SRL_FORWARD || scheme > PFDTD_IWB) return fail(PFDTD_ERR_ARG, "scheme");
  pfdtd_request* r = new pfdtd_request();
  r->X = dim_x;
  r->Y = dim_y;
  r->Z = dim_z;
  r->fields = fields;
  r->precision = precision;
  r->scheme = scheme;
  r->steps = steps;
  *out = r;
  return PFDTD_OK;
}

int pfdtd_request_set_nodes(pfdtd_request* r, const uint8_t* pos, const uint8_t* mat) {
  if (int rc = check_req(r)) return rc;
  if (!pos || !mat) return fail(PFDTD_ERR_ARG, "null node arrays");
  const size_t n = (size_t)(r->X * r->Y * r->Z);
  r->pos.assign(pos, pos + n);
  r->mat.assign(mat, mat + n);
  int64_t nb = 0;
  for (size_t i = 0; i < n; ++i) {
    const uint8_t p = r->pos[i];
    const bool inside = p & 0x80u;
    const bool boundary = r->scheme == PFDTD_SRL_FORWARD || r->scheme == PFDTD_SHARED
                              ? (p & 0x7Fu) != 6
                              : (p & 0x07u) != 0;
    nb += inside && boundary;
  }
  r->n_boundary = nb;
  r->nodes_set = true;
  return PFDTD_OK;
}

int pfdtd_request_set_voxels(pfdtd_request* r, const uint8_t* bid, const uint8_t* mat) {
  if (int rc = check_req(r)) return rc;
  if (!bid || !mat) return fail(PFDTD_ERR_ARG, "null voxel arrays");
  const size_t n = (size_t)(r->X * r->Y * r->Z);
  std::vector<uint8_t> p(bid, bid + n), m(mat, mat + n);
  const int centred = r->scheme == PFDTD_SRL || r->scheme == PFDTD_IWB;
  if (int rc = pfdtd_encode_nodes_host(centred, p.data(), m.data(), (int64_t)n)) return rc;
  return pfdtd_request_set_nodes(r, p.data(), m.data());
}

int pfdtd_request_set_materials(pfdtd_request* r, const double* table, int n_mat, int n_coef) {
  if (int rc = check_req(r)) return rc;
  if (!table || n_mat <= 0 || n_coef <= 0) return fail(PFDTD_ERR_ARG, "invalid material table");
  r->materials.assign(table, table + (size_t)n_mat * n_coef);
  r->n_mat = n_mat;
  r->n_coef = n_coef;
  return PFDTD_OK;
}

int pfdtd_request_set_dif_filters(pfdtd_request* r, int n_mat, const int32_t* flags,
                                  const double* coefs) {
  if (int rc = check_req(r)) return rc;
  if (n_mat < 0 || (n_mat > 0 && (!flags || !coefs))) return fail(PFDTD_ERR_ARG, "filters");
  r->dif_flags.assign(flags, flags + n_mat);
  r->dif_coefs.assign(coefs, coefs + (size_t)n_mat * 7);
  return PFDTD_OK;
}

int pfdtd_request_set_params(pfdtd_request* r, const double params[4]) {
  if (int rc = check_req(r)) return rc;
  if (!params) return fail(PFDTD_ERR_ARG, "null parameters");
  std::memcpy(r->params, params, sizeof(r->params));
  return PFDTD_OK;
}

int pfdtd_request_set_sources(pfdtd_request* r, int n, const int64_t* xyz, const int32_t* field,
                              const int32_t* type, const double* samples, int64_t n_samples) {
  if (int rc = check_req(r)) return rc;
  if (n < 0 || n_samples < 0 || (n > 0 && (!xyz || !type || (n_samples > 0 && !samples))))
    return fail(PFDTD_ERR_ARG, "invalid source arrays");
  if (field)
    for (int i = 0; i < n; ++i)
      if (field[i] < 0 || field[i] >= r->fields) return fail(PFDTD_ERR_ARG, "source field out of range");
  r->n_src = n;
  r->n_samples = n_samples;
  r->src_xyz.assign(xyz, xyz + 3 * (size_t)n);
  if (field) r->src_field.assign(field, field + n);
  else r->src_field.assign(n, 0);
  r->src_type.assign(type, type + n);
  r->samples.assign(samples, samples + (size_t)n * (size_t)n_samples);
  return PFDTD_OK;
}

int pfdtd_request_set_receivers(pfdtd_request* r, int n, const int64_t* xyz,
                                const int32_t* field) {
  if (int rc = check_req(r)) return rc;
  if (n < 0 || (n > 0 && !xyz)) return fail(PFDTD_ERR_ARG, "invalid receiver array");
  if (field)
    for (int i = 0; i < n; ++i)
      if (field[i] < 0 || field[i] >= r->fields)
        return fail(PFDTD_ERR_ARG, "receiver field out of range");
  r->n_rec = n;
  r->rec_xyz.assign(xyz, xyz + 3 * (size_t)n);
  if (field) r->rec_field.assign(field, field + n);
  else r->rec_field.assign(n, 0);
  return PFDTD_OK;
}

int pfdtd_request_set_temporal_block(pfdtd_request* r, int depth) {
  if (int rc = check_req(r)) return rc;
  if (depth != 0 && (depth < 2 || depth > 4)) return fail(PFDTD_ERR_ARG, "depth 0, 2, 3 or 4");
  r->tb_depth = depth;
  return PFDTD_OK;
}

int pfdtd_request_bytes(const pfdtd_request* r, uint64_t* bytes) {
  if (int rc = check_req(r)) return rc;
  if (!bytes) return fail(PFDTD_ERR_ARG, "null output");
  *bytes = estimate_bytes(r);
  return PFDTD_OK;
}

int pfdtd_request_destroy(pfdtd_request* r) {
  delete r;
  return PFDTD_OK;
}

int pfdtd_server_create(int device, uint64_t hbm_budget, int max_active, pfdtd_server** out) {
  if (!out) return fail(PFDTD_ERR_ARG, "null output");
  if (hbm_budget == 0 || max_active < 1) return fail(PFDTD_ERR_ARG, "budget and slots");
  int n = 0;
  if (int rc = pfdtd_device_count(&n)) return rc;
  if (device < 0 || device >= n) return fail(PFDTD_ERR_ARG, "device index out of range");
  pfdtd_server* s = new pfdtd_server();
  s->device = device;
  s->budget = hbm_budget;
  s->max_active = max_active;
  for (int i = 0; i < std::min(max_active, kSetupWorkers); ++i)
    s->workers.emplace_back(setup_worker, s);
  s->thread = std::thread(scheduler, s);
  *out = s;
  return PFDTD_OK;
}

int pfdtd_server_submit(pfdtd_server* s, pfdtd_request* r, int64_t* ticket) {
  if (!s || !r || !ticket) return fail(PFDTD_ERR_ARG, "null argument");
  if (!r->nodes_set || r->n_mat <= 0) return fail(PFDTD_ERR_STATE, "request without room or materials");
  const uint64_t bytes = estimate_bytes(r);
  std::lock_guard<std::mutex> g(s->mu);
  if (s->stop) return fail(PFDTD_ERR_STATE, "server stopping");
  const int64_t t = s->next_ticket++;
  Job& j = s->jobs[t];
  j.req = r;
  j.bytes = bytes;
  j.t_submit = Clock::now();
  s->st.submitted++;
  if (bytes > s->budget) {
    j.state = PFDTD_REQ_FAILED;
    j.error = "request larger than the server's memory budget";
    j.t_admit = j.t_done = j.t_submit;
    s->st.failed++;
    *ticket = t;
    return fail(PFDTD_ERR_NOMEM, j.error);
  }
  s->queue.push_back(t);
  s->st.queued = (int64_t)s->queue.size();
  *ticket = t;
  s->cv_sched.notify_one();
  return PFDTD_OK;
}

int pfdtd_server_wait(pfdtd_server* s, int64_t ticket, double timeout_s, int* state) {
  if (!s) return fail(PFDTD_ERR_ARG, "null server");
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->jobs.find(ticket);
  if (it == s->jobs.end()) return fail(PFDTD_ERR_ARG, "unknown ticket");
  auto finished = [&] {
    return it->second.state == PFDTD_REQ_DONE || it->second.state == PFDTD_REQ_FAILED;
  };
  if (timeout_s < 0) s->cv_done.wait(lk, finished);
  else s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), finished);
  if (state) *state = it->second.state;
  return PFDTD_OK;
}

int pfdtd_server_result(pfdtd_server* s, int64_t ticket, void* out, double times[3]) {
  if (!s) return fail(PFDTD_ERR_ARG, "null server");
  std::lock_guard<std::mutex> g(s->mu);
  auto it = s->jobs.find(ticket);
  if (it == s->jobs.end()) return fail(PFDTD_ERR_ARG, "unknown ticket");
  const Job& j = it->second;
  if (j.state == PFDTD_REQ_FAILED) return fail(PFDTD_ERR_STATE, "request failed: " + j.error);
  if (j.state != PFDTD_REQ_DONE) return fail(PFDTD_ERR_STATE, "request not finished");
  if (out && !j.result.empty()) std::memcpy(out, j.result.data(), j.result.size());
  if (times) {
    times[0] = std::chrono::duration<double>(j.t_admit - j.t_submit).count();
    times[1] = std::chrono::duration<double>(j.t_done - j.t_admit).count();
    times[2] = std::chrono::duration<double>(j.t_done - j.t_submit).count();
  }
  return PFDTD_OK;
}

const char* pfdtd_server_request_error(pfdtd_server* s, int64_t ticket) {
  static thread_local std::string msg;
  msg.clear();
  if (!s) return msg.c_str();
  std::lock_guard<std::mutex> g(s->mu);
  auto it = s->jobs.find(ticket);
  if (it != s->jobs.end()) msg = it->second.error;
  return msg.c_str();
}

int pfdtd_server_release(pfdtd_server* s, int64_t ticket) {
  if (!s) return fail(PFDTD_ERR_ARG, "null server");
  std::lock_guard<std::mutex> g(s->mu);
  auto it = s->jobs.find(ticket);
  if (it == s->jobs.end()) return fail(PFDTD_ERR_ARG, "unknown ticket");
  if (it->second.state != PFDTD_REQ_DONE && it->second.state != PFDTD_REQ_FAILED)
    return fail(PFDTD_ERR_STATE, "request not finished");
  delete it->second.req;
  s->jobs.erase(it);
  return PFDTD_OK;
}

int pfdtd_server_stats_get(pfdtd_server* s, pfdtd_server_stats* st) {
  if (!s || !st) return fail(PFDTD_ERR_ARG, "null argument");
  std::lock_guard<std::mutex> g(s->mu);
  *st = s->st;
  return PFDTD_OK;
}

int pfdtd_server_drain(pfdtd_server* s, double timeout_s) {
  if (!s) return fail(PFDTD_ERR_ARG, "null server");
  std::unique_lock<std::mutex> lk(s->mu);
  auto idle = [&] {
    return s->queue.empty() && s->active.empty() && s->in_transit == 0 && s->admitting == 0;
  };
  if (timeout_s < 0) s->cv_done.wait(lk, idle);
  else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), idle))
    return fail(PFDTD_ERR_STATE, "requests still pending after the timeout");
  return PFDTD_OK;
}

int pfdtd_server_destroy(pfdtd_server* s) {
  if (!s) return PFDTD_OK;
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->stop = true;
    s->cv_sched.notify_all();
  }
  if (s->thread.joinable()) s->thread.join();
  {
    // the scheduler has ended with no request left to set up
    std::lock_guard<std::mutex> g(s->mu);
    s->workers_stop = true;
    s->cv_work.notify_all();
  }
  for (std::thread& w : s->workers) w.join();
  for (auto& kv : s->jobs) delete kv.second.req;
  delete s;
  return PFDTD_OK;
}

}  // extern "C"
