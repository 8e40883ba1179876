/*
 * pfdtd.h — C ABI of the GB300 FDTD time-stepping library (libpfdtd.so).
 *
 * One opaque domain handle holds one whole simulation grid on one GPU: the
 * node bytes, two pressure fields (current and past), the material table,
 * the simulation parameters, the sources and the receivers.  Every function
 * returns an int status (PFDTD_OK = 0) and never throws; the message of the
 * last failure on the calling thread is available from pfdtd_last_error().
 * Pointers are plain host pointers unless a function says otherwise.
 *
 * Grid layout is the reference's: flat arrays, x fastest,
 * index = z*X*Y + y*X + x (ParallelFDTD src/kernels/cudaMesh.h:247-249).
 * Node bytes are the scheme-encoded "position" bytes and material bytes the
 * reference keeps on the device (src/kernels/cudaMesh.h:90-91):
 *   forward scheme (SRL_FORWARD): bit7 = inside switch, bits0-6 = K, the
 *     number of air neighbours (src/kernels/cudaMesh.cu:328-361);
 *   centred scheme (SRL): bit7 = inside, DIR_X/Y/Z = 0x01/0x02/0x04,
 *     SIGN_X/Y/Z = 0x10/0x20/0x40 (src/kernels/cudaMesh.h:35-44).
 *
 * The entry points below replace, for a non-C++ caller, the path
 * CudaMesh::setupMesh -> CudaMesh::makePartition -> launchFDTD3d /
 * launchFDTD3dDouble / launchFDTD3dStep (src/kernels/cudaMesh.h:648-838,
 * src/kernels/kernels3d.h:49-90).  The C++ classes with the reference's own
 * names and signatures sit on top of these (include/pfdtd/).
 */
#ifndef PFDTD_H
#define PFDTD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define PFDTD_OK 0
#define PFDTD_INTERRUPTED 1        /* run stopped by the interrupt callback */
#define PFDTD_ERR_ARG (-1)         /* invalid argument or size */
#define PFDTD_ERR_CUDA (-2)        /* a CUDA runtime call failed */
#define PFDTD_ERR_MATERIAL (-3)    /* a node's material index lies outside the table */
#define PFDTD_ERR_NOMEM (-4)       /* device allocation failed */
#define PFDTD_ERR_STATE (-5)       /* call out of order (e.g. run before geometry) */
#define PFDTD_ERR_UNSUPPORTED (-6) /* combination not built (e.g. scheme x precision) */

/* Field storage precision. */
#define PFDTD_F32 0
#define PFDTD_F64 1
#define PFDTD_F16 2  /* fp16 storage, fp32 arithmetic */
#define PFDTD_BF16 3 /* bf16 storage, fp32 arithmetic */

/* Update schemes, numbered as the reference's UpdateType
 * (src/base/SimulationParameters.h:39).  SHARED runs the forward rule: the
 * reference's shared-memory variant reads and rewrites its shared tile
 * without a barrier in between (src/kernels/kernels3d.cu:572-603). */
#define PFDTD_SRL_FORWARD 0
#define PFDTD_SHARED 1
#define PFDTD_SRL 2
/* IWB 27-point compact scheme at lambda = 1, (a, b) = (1/4, 1/16); no
 * counterpart in the reference.  Uses the centred node encoding; boundary
 * nodes reflect their outward neighbours and lose beta = lambda * Y * (number
 * of boundary axes).  Needs the parameter vector [1, 1, 1/3, octave]. */
#define PFDTD_IWB 3

/* Source types (src/base/SrcRec.h:33). */
#define PFDTD_SRC_HARD 0
#define PFDTD_SRC_SOFT 1
#define PFDTD_SRC_TRANSPARENT 2

/* Reference-behaviour switches (bit flags for pfdtd_set_quirks). */
#define PFDTD_QUIRK_MATIDX 1 /* forward kernel material index m*20*octave (kernels3d.cu:513) */
#define PFDTD_QUIRK_SOFTSRC 2 /* soft source overwrites instead of adding (cudaMesh.h:366) */

/* Field selectors. */
#define PFDTD_FIELD_CURRENT 0
#define PFDTD_FIELD_PAST 1

typedef struct pfdtd_domain pfdtd_domain;

/* Callbacks with the reference's signatures (src/App.h:33-34). */
typedef int (*pfdtd_interrupt_fn)(void);
typedef void (*pfdtd_progress_fn)(int step, int max_step, float seconds_per_step);

/* Message of the last failing call on this thread ("" if none). */
const char* pfdtd_last_error(void);

/* Library version string. */
const char* pfdtd_version(void);

/* Number of visible CUDA devices (0 if none), as App::queryDevices
 * (src/App.cpp:91-112). */
int pfdtd_device_count(int* count);

/* Create a domain of dim_x * dim_y * dim_z nodes on `device` and allocate
 * its fields (zeroed) and node bytes (zeroed = all solid).  Replaces
 * CudaMesh::makePartition (src/kernels/cudaMesh.h:648-751) with one whole
 * domain.  dim_z >= 3. */
int pfdtd_create(int64_t dim_x, int64_t dim_y, int64_t dim_z, int precision, int device,
                 pfdtd_domain** out);
/* Batched domain: `fields` (a power of two, 1..64) independent pressure
 * fields per node sharing the node bytes, materials and parameters — e.g. one
 * field per source position of a multi-source study.  Fields are interleaved
 * node-major (element = node * fields + field), so one class byte is read per
 * `fields` node-updates.  pfdtd_create is pfdtd_create_batched with 1 field.
 * Single-node access, slices and the unbatched source/receiver calls use
 * field 0. */
int pfdtd_create_batched(int64_t dim_x, int64_t dim_y, int64_t dim_z, int fields, int precision,
                         int device, pfdtd_domain** out);
int pfdtd_get_fields(const pfdtd_domain* d, int* fields);
int pfdtd_destroy(pfdtd_domain* d);
int pfdtd_get_dims(const pfdtd_domain* d, int64_t dims[3]);
int pfdtd_get_precision(const pfdtd_domain* d, int* precision);
/* Number unique to this domain among all domains created in the process. */
int pfdtd_get_serial(const pfdtd_domain* d, int64_t* serial);

/* Reference-behaviour switches, PFDTD_QUIRK_* bits; default 0. */
int pfdtd_set_quirks(pfdtd_domain* d, int quirks);

/* Copy scheme-encoded node bytes (pos) and material bytes (mat), N each.
 * on_device != 0: the pointers are device pointers on the domain's device. */
int pfdtd_set_nodes(pfdtd_domain* d, const uint8_t* pos, const uint8_t* mat, int on_device);

/* Device pointers of the domain's node bytes (N each, owned by the domain). */
int pfdtd_get_node_ptrs(pfdtd_domain* d, uint8_t** d_pos, uint8_t** d_mat);
/* Copy the node bytes to the host (N each; either pointer may be null). */
int pfdtd_get_nodes(pfdtd_domain* d, uint8_t* pos, uint8_t* mat);
/* Declare that node bytes were written through those pointers. */
int pfdtd_nodes_changed(pfdtd_domain* d);

/* Material table [n_mat * n_coef] (admittances), row per unique material,
 * as MaterialHandler::getMaterialCoefficientPtr(Double)
 * (src/base/MaterialHandler.cpp:100-164).  Values are double on the ABI and
 * rounded to the domain's arithmetic type (float for every precision but
 * PFDTD_F64) exactly as the reference would hold them. */
int pfdtd_set_materials(pfdtd_domain* d, const double* table, int n_mat, int n_coef);

/* Frequency-dependent boundary admittance (no counterpart in the reference,
 * which only reserves fields for it, src/kernels/cudaMesh.h:88, :122-123).
 * flags[m] != 0 gives material m the filter
 *   Y(z) = (b0 + b1 z^-1 + b2 z^-2 + b3 z^-3) / (1 + a1 z^-1 + a2 z^-2 + a3 z^-3),
 * coefs [n_mat * 7] = b0, b1, b2, b3, a1, a2, a3 per material (orders below 3
 * pad with zeros).  Inside boundary nodes of such materials replace the
 * frequency-independent loss by the filter: with G the node's geometric
 * factor (forward: 0.5 (6-K) lambda; centred and IWB: lambda * axes) and
 * x = (p+ - p-)/2, the loss term 2 G Y x becomes 2 G (b0 x + s1), the filter
 * state (transposed direct form II) kept per node.  n_mat = 0 removes all
 * filters.  States persist across runs and are zeroed by pfdtd_reset_fields. */
int pfdtd_set_dif_filters(pfdtd_domain* d, int n_mat, const int32_t* flags, const double* coefs);
/* Number of frequency-dependent boundary nodes (builds the tables if needed). */
int pfdtd_get_dif_count(pfdtd_domain* d, int64_t* n);

/* Parameter vector [lambda, lambda^2, 1/3, octave] as
 * SimulationParameters::getParameterPtr(Double) (SimulationParameters.cpp:379-396). */
int pfdtd_set_params(pfdtd_domain* d, const double params[4]);

/* Sources: n positions (x,y,z triples, element coordinates), type per source
 * (PFDTD_SRC_*), and a sample table [n * n_samples] (row per source) in the
 * domain's arithmetic type (float, or double for PFDTD_F64).  Sources whose z
 * lies outside the grid are skipped, as CudaMesh::setSample does
 * (cudaMesh.h:322-338). */
int pfdtd_set_sources(pfdtd_domain* d, int n, const int64_t* xyz, const int32_t* type,
                      const void* samples, int64_t n_samples);

/* Sources of a batched domain: field[i] is the field source i drives. */
int pfdtd_set_sources_batched(pfdtd_domain* d, int n, const int64_t* xyz, const int32_t* field,
                              const int32_t* type, const void* samples, int64_t n_samples);

/* Receivers: n positions (x,y,z triples).  A receiver whose z lies outside
 * the grid is skipped and its output row left untouched
 * (kernels3d.cu:66-78, :164-173). */
int pfdtd_set_receivers(pfdtd_domain* d, int n, const int64_t* xyz);

/* Receivers of a batched domain: field[i] is the field receiver i records. */
int pfdtd_set_receivers_batched(pfdtd_domain* d, int n, const int64_t* xyz, const int32_t* field);

/* Update scheme used by the next run/step (PFDTD_SRL_FORWARD, _SHARED, _SRL, _IWB). */
int pfdtd_set_scheme(pfdtd_domain* d, int scheme);

/* Arithmetic form of the forward (SRL_FORWARD / SHARED) update.  No
 * counterpart in the reference.
 * PFDTD_FORM_REFERENCE (default): the reference's expression
 *   P+ = s/(1+b) * ((2 - K l2) P + l2 S - (1 - b) P-)   (kernels3d.cu:526),
 *   bit for bit.
 * PFDTD_FORM_DIFFERENCE: the same update, equal in exact arithmetic,
 *   P+ = s/(1+b) * (((1+b) P + (1-b) (P - P-)) + l2 (S - K P)).
 *   In float, the reference form rounds 6 l2 to 2 + 6e-8, which makes the
 *   uniform (pressure offset) mode of a closed room grow step by step; the
 *   difference form has no such term (S - K P is exactly 0 on a uniform
 *   field), and its receiver error against an FP64 run drops by about two
 *   orders of magnitude at the same memory traffic.  FP32 fields only (with
 *   16-bit storage the storage rounding dominates and the form gains
 *   nothing); no frequency-dependent boundaries and no temporal blocking
 *   (PFDTD_ERR_UNSUPPORTED at the next run).  */
/* Bound, in nanoseconds, of each pipeline wait inside the TMA update kernels
 * (no counterpart in the reference; default 2 s, 0 restores it).  A wait that
 * runs out raises the domain's error flag; the kernel stops issuing loads,
 * waits for the loads already in flight (always with the 2 s bound) and
 * returns, later launches of the run do nothing, and the run returns
 * PFDTD_ERR_CUDA with the flag cleared, the context still usable.  A watchdog
 * for stalled pipelines; tests set it very low to exercise that path. */
int pfdtd_set_wait_limit(pfdtd_domain* d, uint64_t ns);

#define PFDTD_FORM_REFERENCE 0
#define PFDTD_FORM_DIFFERENCE 1
int pfdtd_set_update_form(pfdtd_domain* d, int form);

/* Run `steps` leapfrog steps from step index 0 (launchFDTD3d,
 * src/kernels/kernels3d.cu:31-203): per step inject sources into the current
 * field, update z = 1..Z-2 into the past field, swap, record receivers.
 * out: host buffer [n_rec * steps] in the arithmetic type, row per receiver.
 * The interrupt callback is polled and the progress callback called every
 * 100 steps.  seconds_per_step (optional) receives wall time / steps.
 * Returns PFDTD_INTERRUPTED if stopped early (rows hold the steps done). */
int pfdtd_run(pfdtd_domain* d, int64_t steps, void* out, pfdtd_interrupt_fn interrupt_cb,
              pfdtd_progress_fn progress_cb, double* seconds_per_step);

/* Same as pfdtd_run but with the output left on the device: d_out is a device
 * buffer [n_rec * steps] in the arithmetic type.  No host synchronisation
 * inside; the work is queued on the domain's stream (pfdtd_get_stream). */
int pfdtd_run_device(pfdtd_domain* d, int64_t steps, void* d_out);

/* Queue `iters` update-kernel launches alone (no sources, no receivers),
 * swapping the fields after each, on the domain's stream; no synchronisation.
 * Used to time the update kernel with events recorded around it.  The fields
 * advance (for IWB with frequency-dependent walls on the TMA path, so do the
 * filter states, which the closure pass updates); pfdtd_reset_fields gives a
 * clean start again. */
int pfdtd_profile_update(pfdtd_domain* d, int iters);

/* One step in capture mode (launchFDTD3dStep, kernels3d.cu:376-482): inject
 * samples[step], update, swap unless the step direction changed, then write
 * receiver values to out[r*num_steps + step] (host) when out is non-null. */
int pfdtd_step(pfdtd_domain* d, int64_t step, int step_direction, void* out, int64_t num_steps);

/* Single-node access (CudaMesh::setSample/addSample/getSample,
 * cudaMesh.h:320-404, :497-565), element coordinates, current field. */
int pfdtd_set_sample(pfdtd_domain* d, int64_t x, int64_t y, int64_t z, double value);
int pfdtd_add_sample(pfdtd_domain* d, int64_t x, int64_t y, int64_t z, double value);
int pfdtd_get_sample(pfdtd_domain* d, int64_t x, int64_t y, int64_t z, double* value);

/* Swap current and past fields (CudaMesh::flipPressurePointers, cudaMesh.h:766-779). */
int pfdtd_flip(pfdtd_domain* d);
/* Zero both fields (CudaMesh::resetPressures, cudaMesh.h:782-791). */
int pfdtd_reset_fields(pfdtd_domain* d);
/* Device pointer of a field (PFDTD_FIELD_*); element 0 is node (0,0,0). */
int pfdtd_get_field_ptr(pfdtd_domain* d, int which, void** d_ptr);
/* Copy a whole field to / from the host (N * fields elements of the storage type). */
int pfdtd_download_field(pfdtd_domain* d, int which, void* host);
int pfdtd_upload_field(pfdtd_domain* d, int which, const void* host);

/* Slice capture (captureSliceFast / captureSliceKernel,
 * src/kernels/visualizationUtils.cu:130-254, :500-527): orientation 0 = xy
 * (slice = z), 1 = xz (slice = y), 2 = yz (slice = x).  p_out receives the
 * current pressure as float and pos_out the node bytes (either may be null);
 * sizes X*Y, X*Z and Y*Z respectively.  A slice past the grid returns
 * PFDTD_ERR_ARG and writes nothing, as the reference skips the capture. */
int pfdtd_capture_slice(pfdtd_domain* d, int orientation, int64_t slice, float* p_out,
                        uint8_t* pos_out);

/* Slice capture that allocates no device memory.  No counterpart in the
 * reference: it is the same capture as pfdtd_capture_slice (same arguments,
 * same output), for callers that cannot allocate while a simulation runs —
 * a serving loop that has given the whole HBM budget to resident domains, or
 * a per-step capture loop that must not stall on cudaFree, which synchronizes
 * the device.  The slice is gathered into a fixed 5 MiB scratch array
 * compiled into the library, so a slice may hold at most 1,048,576 nodes
 * (e.g. 1024 x 1024); larger slices return PFDTD_ERR_ARG and write nothing.
 * CUDA places such an array on a GPU only when its code is first used there;
 * pfdtd_create / pfdtd_create_batched do that on their device (looking up
 * the scratch's address with cudaGetSymbolAddress), so the 5 MiB are taken
 * before the domain's buffers and stay on every GPU that has had a domain
 * until the process exits.  Create the domain before committing the rest of
 * the device's memory and before any stream capture.
 * Every call shares the one scratch array: calls that overlap on the GPU
 * (several host threads, or several domains on one device) race.  Each call
 * writes every element of its slice, so no earlier call's data leaks into
 * the result. */
int pfdtd_capture_slice_noalloc(pfdtd_domain* d, int orientation, int64_t slice, float* p_out,
                                uint8_t* pos_out);

/* Asynchronous run (no counterpart in the reference): queue `steps` steps
 * from step 0 on the domain's stream and return without waiting; receivers
 * are recorded on the device.  pfdtd_query reports whether the domain's queued
 * work has finished; pfdtd_fetch_receivers waits for it, reports a failed
 * kernel pipeline and copies the receivers ([n_rec * steps], arithmetic type)
 * of the last asynchronous run to the host.  No call waits for other
 * domains' work. */
int pfdtd_run_async(pfdtd_domain* d, int64_t steps);
/* Run `steps` steps from step 0 and capture slices on the way
 * (App::runCapture / captureSliceFast, App.cpp:407-436 and
 * visualizationUtils.cu:130-254, which step one at a time and gather and
 * copy each slice synchronously): capture i is the slice cap_slice[i] of
 * orientation cap_orientation[i] (0 xy, 1 xz, 2 yz, as pfdtd_capture_slice)
 * of the field after cap_step[i] steps (0 <= cap_step[i] <= steps).  The
 * run is split at the capture steps, whole chunks still replay their CUDA
 * graphs, and each capture is a gather kernel and an asynchronous copy into
 * p_out[i] (floats) and pos_out[i] (node bytes) on the domain's stream
 * (either array, or one of its entries, may be null).  Pinned host buffers
 * (pfdtd_host_alloc) keep the copies asynchronous.  Receivers as pfdtd_run. */
int pfdtd_run_captures(pfdtd_domain* d, int64_t steps, void* out, int n_cap,
                       const int64_t* cap_step, const int32_t* cap_orientation,
                       const int64_t* cap_slice, float* const* p_out, uint8_t* const* pos_out);
/* Page-locked host memory for asynchronous copies. */
int pfdtd_host_alloc(size_t bytes, void** ptr);
int pfdtd_host_free(void* ptr);
int pfdtd_query(pfdtd_domain* d, int* done);
int pfdtd_fetch_receivers(pfdtd_domain* d, void* out);

/* Update kernel variant: 0 automatic (the TMA-pipelined kernel when the
 * field rows are 16-byte aligned: X * fields * element size a multiple of 16;
 * class-id rows that are not are read from a padded copy), 1 the
 * register z-marching kernel, 2 the TMA kernel.  pfdtd_get_kernel reports the
 * variant the next launch will use (1 or 2, or 3 when the temporally blocked
 * kernel of pfdtd_set_temporal_block will run). */
#define PFDTD_KERNEL_AUTO 0
#define PFDTD_KERNEL_ZMARCH 1
#define PFDTD_KERNEL_TMA 2
#define PFDTD_KERNEL_TB 3 /* reported only: temporal blocking active */
int pfdtd_set_kernel(pfdtd_domain* d, int variant);
/* Tile shape of the TMA kernel for FP32 fields: 0 64x16, 1 128x8, 2 32x32,
 * 3 128x16, 4 128x4 (x halo in the TMA box); 5 128x8, 6 256x4, 7 256x8,
 * 8 256x2 (x halo read from global); -1 (default) picks the widest of
 * 256/128/64 whose partly filled last tile leaves at most 1/16 of the row's
 * tiles empty.  FP64 always uses 64x8.  FP16/BF16 fields: 0 64x16, 1 128x8,
 * 2 256x8, 3 256x4 with 4 nodes per thread; 4 256x8, 5 256x8 (three CTAs per
 * SM), 6 256x4, 7 128x8 with 8 nodes per thread; 8 256x8 (default), 9 256x4,
 * 10 128x8 with 8 nodes per thread and planes z-1, z kept in registers.
 * Batched 16-bit fields: 0 256x8, 1 256x4, 2 256x8 with 6 stages (4 fields
 * per thread); for K a multiple of 8, 3 256x8, 4 256x4 (8 fields per
 * thread), 5 256x8 with planes kept in registers (default), 6 256x4 with
 * planes kept in registers.  For the IWB
 * scheme the same index picks the IWB shape: 0..5 carry the closed-neighbour
 * masks and compute the closure in the kernel (0 64x16, 1 128x8, 2 128x4,
 * 3..5 64x8 with 3, 4, 5 CTAs per SM); 6..10 run the open sums in the kernel
 * and a sparse pass for the nodes with a closed neighbour (6 128x8 with 3
 * CTAs per SM, the default; 7 128x4 with 4; 8 128x8 with 2; 9 128x8 with 4;
 * 10 128x4 with 6).  Every shape gives bit-identical results. */
int pfdtd_set_tile(pfdtd_domain* d, int tile);
int pfdtd_get_kernel(pfdtd_domain* d, int* variant);

/* Temporal blocking (no counterpart in the reference, whose launchFDTD3d
 * loop at kernels3d.cu:86-175 runs one kernel per step).  depth 0 (default)
 * runs one update per step; 2, 3 or 4 runs pfdtd_run / pfdtd_run_device
 * with one kernel per `depth` steps that keeps the intermediate steps on
 * chip, records the receivers of and injects the sources into every
 * intermediate step, and writes two fields out of place (two more field
 * buffers are allocated on the next run).  Results equal the per-step path
 * (a zero on an x/y face node may differ in sign).  The blocked kernel is
 * used only when: FP32, FP16 or BF16 storage; the SRL forward or centred
 * scheme; no frequency-dependent boundary; at most 256 node classes; X a
 * multiple of 4; K = 1 or a multiple of 4 fields; every node on the x and y
 * faces of planes 1..Z-2 outside (position bit 7 clear); at most 64 sources
 * and 256 receivers, none on plane 0 or Z-1.  Otherwise the run falls back
 * to the per-step path.  pfdtd_get_temporal_block reports the depth, whether
 * the next run will block (after building the node classes) and, in `why`,
 * the first condition that fails. */
int pfdtd_set_temporal_block(pfdtd_domain* d, int depth);
int pfdtd_get_temporal_block(pfdtd_domain* d, int* depth, int* active, char* why,
                             size_t why_len);
/* Tile shape of the blocked kernel, -1 (default) or 0..3:
 *   one field per node: 0 = 64 x 32 nodes, 256 threads of two rows;
 *     1 = 64 x 32, 512 threads of one row; 2 = 64 x 64, 512 threads of two
 *     rows (depths 2, 3); depth 4 has only shape 1;
 *   batched fields: 0 = 32 x 32 nodes of 4 fields, 512 threads of two rows;
 *     1 = one row per thread (FP32 depth 4: 32 x 24); depth 4 only shape 1;
 *     2 and 3 = 32 x 32 nodes of 4 fields with packed two-field arithmetic,
 *     512 threads of two rows (2) or 1024 threads of one row (3); SRL
 *     forward scheme, depths 2 and 3, fewer than 256 node classes.
 * A shape that does not exist for the depth makes the next run fail with
 * PFDTD_ERR_ARG. */
int pfdtd_set_tb_shape(pfdtd_domain* d, int shape);
/* Autotuner (no counterpart in the reference): times the per-step update and
 * every available (depth <= max_depth, shape) of the blocked update on this
 * domain, `iters` launches each after one warm-up launch, keeps the fastest
 * per step on the domain and reports it.  The fields are copied before and
 * restored after the timing launches; node classes are built first.
 * max_depth 0 times the per-step update only. */
int pfdtd_autotune(pfdtd_domain* d, int max_depth, int iters, int* best_depth, int* best_shape,
                   double* best_ms_per_step);

/* Wait for the domain's queued work and report a kernel pipeline failure
 * (a bounded wait that expired) as PFDTD_ERR_CUDA. */
int pfdtd_synchronize(pfdtd_domain* d);

/* CUDA stream (cudaStream_t) the domain queues its work on. */
int pfdtd_get_stream(pfdtd_domain* d, void** stream);

/* Launches of library kernels since load (for accounting in benchmarks). */
int64_t pfdtd_kernel_launches(void);

/* ---- Device-side mesh set-up (the reference runs these on the GPU) ---- */

/* Translate voxelizer boundary ids (0..27) in place into scheme bytes:
 * forward (toBilbao, cudaMesh.cu:328-361) when centred == 0, else centred
 * (toKowalczyk, :363-480).  d_pos, d_mat: device pointers, n nodes. */
int pfdtd_encode_nodes(int centred, uint8_t* d_pos, uint8_t* d_mat, int64_t n, int device);
/* The same translation on host arrays (no device work). */
int pfdtd_encode_nodes_host(int centred, uint8_t* pos, uint8_t* mat, int64_t n);

/* Solid voxelization of a closed triangle mesh (the room's boundary, closed
 * obstacles inside) into the voxelizer's node bytes: boundary id 0..27 and
 * material byte per node, flat x-fastest (replaces the external voxelizer
 * the reference calls from voxelizationUtils.cu:55-136; that library is not
 * vendored, so its exact output is not pinned).  vertices [n_vertices * 3],
 * indices [n_triangles * 3], tri_materials [n_triangles] (null: 0).  Node i
 * at bbox_min + (i - 1) * voxel_edge (the reference's element coordinates,
 * ROUND(p/dx) + 1), one outside layer on every side; dims and origin (the
 * position of node 0) are returned; with both
 * output arrays null only dims/origin are computed, else both must hold
 * dims[0]*dims[1]*dims[2] bytes.  Inside = odd number of crossings of a +z
 * ray; a solid node next to air takes the material of the triangle between
 * it and its first air neighbour (-x,+x,-y,+y,-z,+z); a boundary node the
 * material of its first solid neighbour; air nodes with solid on both sides
 * of an axis are closed first.  At most 64 crossings per column. */
int pfdtd_voxelize(const float* vertices, int64_t n_vertices, const uint32_t* indices,
                   int64_t n_triangles, const uint8_t* tri_materials, double voxel_edge,
                   int device, uint32_t dims[3], double origin[3], uint8_t* bid_out,
                   uint8_t* mat_out);

/* Receiver post-processing (python/FDTDfilter.py:13-19,
 * matlab/functions/FDTDpostFilter.m:1-31) on the device: each of n_channels
 * traces of n_samples (row-major, float or double) is convolved with the
 * causal FIR `taps` (lfilter(taps, 1, x)), then, with dc_block != 0, passed
 * through y[n] = x[n] - x[n-1] + dc_coef * y[n-1].  Arithmetic in double.
 * Host arrays. */
int pfdtd_post_filter(const void* x, int64_t n_channels, int64_t n_samples, int is_double,
                      const double* taps, int n_taps, int dc_block, double dc_coef, void* out,
                      int device);

/* Rational resampling of n_channels traces of n_in samples (row-major, float
 * or double) on the device (the resample step of matlab/testBench.m:204):
 * out[c][j] = sum_i taps[(j + offset) * down - i * up] * x[c][i], j < n_out,
 * over the i whose tap index lies in [0, n_taps).  The caller designs the
 * anti-aliasing taps (scaled by up) and the delay offset.  Host arrays. */
int pfdtd_resample(const void* x, int64_t n_channels, int64_t n_in, int is_double,
                   const double* taps, int n_taps, int up, int down, int64_t offset,
                   int64_t n_out, void* out, int device);

/* Transparent source vector on the device (SimulationParameters.cpp:300-310,
 * which evaluates it per step on the host, O(steps^2) for a whole run):
 * out[n] = samples[n] - sum_{i<n} grid_ir[n-i] * samples[i] in float, in the
 * reference's order (ascending i), grid_ir[k] = 0 for k >= n_ir.  Host arrays
 * of `steps` floats; out may alias nothing. */
int pfdtd_transparent_source(const float* samples, int64_t steps, const float* grid_ir,
                             int64_t n_ir, float* out, int device);

/* Count air and boundary nodes (calcBoundaries, cudaMesh.cu:500-514). */
int pfdtd_count_boundaries(const uint8_t* d_pos, int64_t n, uint8_t air_value,
                           uint8_t outside_value, int device, uint32_t* air,
                           uint32_t* boundary);

/* Pad a byte mesh to multiples of the block size (padWithZeros,
 * cudaMesh.cu:253-304).  d_in holds in_len readable bytes; d_out must hold
 * the padded size, returned in out_dims. Pass d_out = NULL to query dims. */
int pfdtd_pad_mesh(const uint8_t* d_in, int64_t in_len, const uint32_t dims[3], uint32_t bx,
                   uint32_t by, uint32_t bz, uint8_t* d_out, uint32_t out_dims[3], int device);

#ifdef __cplusplus
}
#endif

#endif /* PFDTD_H */
