/*
 * pfdtd_server.h — request loop over the C ABI (no counterpart in the
 * reference, whose App runs one simulation at a time: src/App.cpp:323-340).
 *
 * A server owns one GPU.  Requests (a room, its materials, sources,
 * receivers and step count) are submitted from any host thread and queued
 * in arrival order.  A scheduler thread admits the request at the head of
 * the queue as soon as an active slot is free and the request's estimated
 * device footprint fits the HBM budget next to the requests already running
 * (continuous batching): it reserves the slot and the bytes and hands the
 * request to one of up to four set-up threads, which creates the request's
 * domain on its own stream and queues the whole run there without waiting
 * (pfdtd_run_async); the scheduler goes on admitting meanwhile.  Admitted
 * requests therefore run concurrently on the device, and the host set-up of
 * one overlaps the others' runs.  An IWB request with several fields runs
 * the fields that carry a source one after another on one single-field
 * domain (the IWB update's pipelined kernels are single-field), with the
 * same receivers as a batched run.
 * When a request's stream has drained, its receivers are copied to the host,
 * its domain is destroyed (stream-ordered frees, no device-wide
 * synchronisation) and its memory returns to the budget.
 *
 * A request's result does not depend on what else runs: each domain has its
 * own fields, filter states and receiver buffers, and every kernel is
 * deterministic, so results equal a standalone pfdtd_run of the same set-up.
 *
 * Request states: PFDTD_REQ_QUEUED, _RUNNING, _DONE, _FAILED.
 */
#ifndef PFDTD_SERVER_H
#define PFDTD_SERVER_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PFDTD_REQ_QUEUED 0
#define PFDTD_REQ_RUNNING 1
#define PFDTD_REQ_DONE 2
#define PFDTD_REQ_FAILED 3

typedef struct pfdtd_request pfdtd_request;
typedef struct pfdtd_server pfdtd_server;

/* A request for `steps` steps of a dim_x*dim_y*dim_z room with `fields`
 * batched fields (power of two), storage precision and update scheme as in
 * pfdtd.h.  Setters copy their inputs. */
int pfdtd_request_create(int64_t dim_x, int64_t dim_y, int64_t dim_z, int fields, int precision,
                         int scheme, int64_t steps, pfdtd_request** out);
/* Voxelizer boundary ids 0..27 (encoded for the scheme on the device at
 * admission, as pfdtd_encode_nodes) or already encoded node bytes. */
int pfdtd_request_set_voxels(pfdtd_request* r, const uint8_t* bid, const uint8_t* mat);
int pfdtd_request_set_nodes(pfdtd_request* r, const uint8_t* pos, const uint8_t* mat);
int pfdtd_request_set_materials(pfdtd_request* r, const double* table, int n_mat, int n_coef);
int pfdtd_request_set_dif_filters(pfdtd_request* r, int n_mat, const int32_t* flags,
                                  const double* coefs);
int pfdtd_request_set_params(pfdtd_request* r, const double params[4]);
/* samples [n * n_samples] as double; rounded to the arithmetic type. */
int pfdtd_request_set_sources(pfdtd_request* r, int n, const int64_t* xyz, const int32_t* field,
                              const int32_t* type, const double* samples, int64_t n_samples);
int pfdtd_request_set_receivers(pfdtd_request* r, int n, const int64_t* xyz,
                                const int32_t* field);
int pfdtd_request_set_temporal_block(pfdtd_request* r, int depth);
/* Estimated device bytes of the request's domain (fields, node bytes and
 * classes, source and receiver buffers, filter states). */
int pfdtd_request_bytes(const pfdtd_request* r, uint64_t* bytes);
int pfdtd_request_destroy(pfdtd_request* r);

/* Server on `device` admitting requests while their summed estimated bytes
 * stay within hbm_budget and at most max_active run at once. */
int pfdtd_server_create(int device, uint64_t hbm_budget, int max_active, pfdtd_server** out);
/* Queue a request; the server takes ownership of it (do not destroy it).
 * A request larger than the whole budget fails at once (PFDTD_ERR_NOMEM). */
int pfdtd_server_submit(pfdtd_server* s, pfdtd_request* r, int64_t* ticket);
/* Wait up to timeout_s seconds (negative: no limit) for the request to
 * finish; *state receives its state either way. */
int pfdtd_server_wait(pfdtd_server* s, int64_t ticket, double timeout_s, int* state);
/* Receivers of a finished request ([n_rec * steps], float, or double for
 * FP64) and its times in seconds: queued (submit to admission), service
 * (admission to completion), total.  Either pointer may be null. */
int pfdtd_server_result(pfdtd_server* s, int64_t ticket, void* out, double times[3]);
/* Error message of a failed request (empty otherwise). */
const char* pfdtd_server_request_error(pfdtd_server* s, int64_t ticket);
/* Forget a finished request and its stored result. */
int pfdtd_server_release(pfdtd_server* s, int64_t ticket);

typedef struct {
  int64_t submitted, admitted, completed, failed;
  int64_t queued, running;
  uint64_t bytes_in_use, bytes_peak;
  int max_running;       /* most requests running at once so far */
  double node_updates;   /* interior node-updates x fields of completed requests */
  double setup_seconds;  /* host time spent setting requests up, summed over the workers */
  double retire_seconds; /* host time spent retiring requests (receivers out, domain freed) */
} pfdtd_server_stats;
int pfdtd_server_stats_get(pfdtd_server* s, pfdtd_server_stats* st);
/* Wait until no request is queued or running (timeout_s < 0: no limit). */
int pfdtd_server_drain(pfdtd_server* s, double timeout_s);
/* Stop the scheduler after the running requests finish; queued requests
 * fail.  Frees the server. */
int pfdtd_server_destroy(pfdtd_server* s);

#ifdef __cplusplus
}
#endif

#endif /* PFDTD_SERVER_H */
