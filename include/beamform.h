/*
 * beamform.h -- C ABI of the GB300 (sm_103a) CHORD beamformer.
 *
 * Computes, for every beam b, frequency f, polarization p and time t,
 *
 *   J[b][f][p][t] = ucomplex4(clamp(int(lrint(G[f][b] * float(re))), -7, 7),
 *                             clamp(int(lrint(G[f][b] * float(im))), -7, 7))
 *   re + i*im    = sum_d A[f][b][d] * E[t][f][d][p]        (exact integers)
 *
 * over 4-bit complex data stored as ucomplex4 bytes (real part in the high
 * nibble, imaginary part in the low nibble, each stored as value + 8).  The
 * result is bit-identical to the reference CPU implementation
 * (eschnett/beamforming cpu.cxx:15-46).
 *
 * As in cpu.cxx:38, lrint's 64-bit result is narrowed to int before the
 * clamp: a product with 2^31 <= |G * raw| < 2^63 keeps its low 32 bits (so it
 * clamps to 0, +7 or -7 by those bits), and a NaN, infinite or |G * raw| >= 2^63
 * product gives 0 (what the reference's x86-64 build returns).  Any float G is
 * accepted.
 *
 * Array layouts (all byte arrays, C order) follow the reference accessors:
 *   E[t][f][d][p]   Elinear   arraysizes.hxx:80
 *   A[f][b][d]      Alinear   arraysizes.hxx:115
 *   G[f][b] float   Glinear   arraysizes.hxx:136
 *   J[b][f][p][t]   Jlinear   arraysizes.hxx:92
 *
 * Every entry point except form_beams() returns a bf_status; none of them
 * exits the process.
 */
#ifndef BEAMFORM_H
#define BEAMFORM_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define BF_API __attribute__((visibility("default")))
#else
#define BF_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* Problem shape: the reference's compile-time sizes (arraysizes.hxx:22-27)
 * made run-time values. */
typedef struct bf_dims {
  int64_t ntimes;
  int64_t nfrequencies;
  int64_t ndishes;
  int64_t npolarizations;
  int64_t nbeams;
} bf_dims;

/* A CUDA stream (cudaStream_t); NULL means the legacy default stream. */
typedef void *bf_stream_t;

typedef enum bf_status {
  BF_OK = 0,
  BF_ERR_INVALID_ARGUMENT = 1, /* null pointer, negative size, bad enum */
  BF_ERR_UNSUPPORTED = 2,      /* shape or alignment no kernel handles */
  BF_ERR_NO_DEVICE = 3,        /* no CUDA device, or not a compute-capability 10.3 part */
  BF_ERR_CUDA = 4,             /* a CUDA runtime call failed */
  BF_ERR_OUT_OF_MEMORY = 5,    /* device or pinned-host allocation failed */
  BF_ERR_DEVICE_TIMEOUT = 6,   /* a kernel's bounded wait expired; the result is invalid */
  BF_ERR_NOT_CONFIGURED = 7,   /* form_beams() called before bf_set_dims() */
  BF_ERR_SIZE_MISMATCH = 8,    /* resident weights built for another shape */
  BF_ERR_TOO_LARGE = 9         /* problem exceeds bf_form_beams_noalloc()'s fixed scratch */
} bf_status;

/* Where the array arguments live. */
typedef enum bf_ptr_kind { BF_PTR_HOST = 0, BF_PTR_DEVICE = 1 } bf_ptr_kind;

/* Which kernel family runs the beam sums. */
typedef enum bf_kernel {
  BF_KERNEL_AUTO = 0,   /* tensor-core kernel where the shape allows, else SIMT */
  BF_KERNEL_TENSOR = 1, /* tcgen05 tensor-core kernel (fails if the shape does not fit) */
  BF_KERNEL_SIMT = 2,   /* exact integer dp4a kernel, any shape (Gauss 3-multiply form) */
  BF_KERNEL_SIMT4 = 3   /* the same with the reference's 4-multiply form (cpu.cxx:33-34) */
} bf_kernel;

/* ------------------------------------------------------------------ drop-in */

/* Sets the sizes form_beams() uses.  Replaces the constexpr globals of
 * arraysizes.hxx:22-27. */
BF_API int bf_set_dims(const bf_dims *dims);

/* Drop-in for the reference's
 *   void form_beams(ucomplex4 *J, const ucomplex4 *E, const ucomplex4 *A, const float *G)
 * (cpu.cxx:15-16): host pointers, sizes from bf_set_dims(), synchronous, no
 * return value.  J must hold Jsize/2 bytes.  The status of the last call is
 * available from bf_last_status(). */
BF_API void form_beams(uint8_t *J, const uint8_t *E, const uint8_t *A, const float *G);

/* Status of the most recent form_beams() call on this thread. */
BF_API int bf_last_status(void);

/* Human-readable text for a status code (static storage). */
BF_API const char *bf_status_string(int status);

/* -------------------------------------------------------------- explicit API */

/* One beamforming pass with explicit sizes.  ptr_kind says whether E, A, G and
 * J are host or device pointers.  Device pointers: asynchronous on `stream`;
 * call bf_stream_status() (or synchronize) before reading J.  Host pointers:
 * synchronous (copies in, computes, copies out). */
BF_API int bf_form_beams_ex(const bf_dims *dims, uint8_t *J, const uint8_t *E, const uint8_t *A, const float *G,
                     int ptr_kind, bf_stream_t stream);

/* Synchronizes `stream` and reports any CUDA error or expired device wait
 * recorded by kernels launched by this library since the last call. */
BF_API int bf_stream_status(bf_stream_t stream);

/* Chooses the kernel family for later calls (testing and benchmarking). */
BF_API int bf_set_kernel(int kernel);

/* Test hook for the failure path: while `on` is nonzero, tensor-core launches
 * issue no input copies, so their bounded device waits expire (after about
 * 1.5 s) and the call reports BF_ERR_DEVICE_TIMEOUT.  No memory is touched
 * out of bounds and the CUDA context stays usable. */
BF_API int bf_set_test_stall(int on);

/* Name of the kernel family the last launch on this thread used:
 * "tensor", "simt" or "none". */
BF_API const char *bf_last_kernel(void);

/* --------------------------------------------------------- resident weights */

/* Beam weights kept on the device in the tensor-core operand format, so a
 * stream of voltage chunks for the same frequencies does not re-prepare A. */
typedef struct bf_weights bf_weights;

/* Allocates device storage for the weights of nfrequencies x nbeams x ndishes
 * (2 polarizations) and fills it from A and G (ptr_kind as above). */
BF_API int bf_weights_create(bf_weights **out, int64_t nfrequencies, int64_t nbeams, int64_t ndishes, const uint8_t *A,
                      const float *G, int ptr_kind, bf_stream_t stream);

/* Replaces the weights in place (same sizes): weight refresh. */
BF_API int bf_weights_update(bf_weights *w, const uint8_t *A, const float *G, int ptr_kind, bf_stream_t stream);

BF_API int bf_weights_destroy(bf_weights *w);

/* Beamforms ntimes samples of device-resident E into device J with resident
 * weights; asynchronous on `stream`. */
BF_API int bf_form_beams_resident(const bf_weights *w, int64_t ntimes, uint8_t *J, const uint8_t *E, bf_stream_t stream);

/* ---------------------------------------------------------------- batches */

/* A fixed set of beamforming problems run as one persistent launch.  No
 * counterpart in the reference, which runs one compile-time shape per program;
 * this is the grouped form of bf_form_beams_resident(). */
typedef struct bf_batch bf_batch;

/* One problem of a batch: ntimes samples of device E[t][f][d][p] beamformed
 * with resident weights into device J[b][f][p][t].  ntimes, frequencies and
 * beams may differ between problems; ndishes must be the same for all. */
typedef struct bf_problem {
  const bf_weights *weights;
  int64_t ntimes;
  const uint8_t *E;
  uint8_t *J;
} bf_problem;

/* Builds a batch: times a few launch schedules on the given buffers (tile
 * shape x tile order x shared-memory ring plan), keeps the fastest and
 * captures it in a CUDA graph.  The tile shape groups the problems by beam
 * pass width into one to three persistent launches: passes wider than 64
 * beams; at most 64 (smaller accumulators leave tensor memory for four or
 * more unpacked stages and two unpack warp groups); at most 16 (two CTAs per
 * SM).  Classes share a launch unless timing says to split them.  The
 * buffers must stay allocated while the batch exists; their contents may
 * change between runs.  Each problem needs the tensor-core shape rules
 * (ntimes % 16 == 0, ndishes % 8 == 0, ndishes <= 2048, 16-byte aligned E and
 * J).  BF_ERR_DEVICE_TIMEOUT if a bounded device wait gave up while tuning. */
BF_API int bf_batch_create(bf_batch **out, const bf_problem *problems, int nproblems, bf_stream_t stream);

/* Runs every problem of the batch once (graph replay); asynchronous on
 * `stream`.  bf_stream_status(stream) reports a device wait that gave up. */
BF_API int bf_batch_run(bf_batch *batch, bf_stream_t stream);

/* The schedule the autotuner chose: tiles, tile order (0 as given, 1 largest
 * problem first), ring plan (0 = default) and the tuned time of one run. */
BF_API int bf_batch_info(const bf_batch *batch, int *ntiles, int *order, int *wslots, int *raw, float *tuned_ms);

/* The tile shape the autotuner chose: the number of launches (1 to 3) and,
 * per launch (arrays of at least 3 entries, any of them may be NULL), its
 * problems, tiles, widest beam pass, unpacked stages in tensor memory, unpack
 * warp groups and CTAs per SM (2 when no pass is wider than 16 beams).  No
 * counterpart in the reference. */
BF_API int bf_batch_shape(const bf_batch *batch, int *nlaunches, int *nproblems, int *ntiles, int *max_nb_pass,
                          int *stages, int *unpack_groups, int *ctas_per_sm);

BF_API int bf_batch_destroy(bf_batch *batch);

/* The ring layout the tensor-core kernel plans for a launch over ndishes
 * dishes whose widest beam pass has max_nb_pass beams, with wslots W slots
 * and raw raw-E slots asked for (0: the planner's choice).  out[0..11] =
 * unpacked stages in tensor memory, W slots, raw E slots, unpack warp
 * groups, CTAs per SM, K stages per tile, dynamic shared memory bytes per
 * CTA, tensor-memory columns allocated per CTA, columns of each accumulator,
 * column of the second accumulator, stages beside each accumulator, one past
 * the last column a stage uses.  Host only: needs no GPU.
 * BF_ERR_INVALID_ARGUMENT where no layout fits.  No counterpart in the
 * reference. */
BF_API int bf_plan_rings(int64_t ndishes, int max_nb_pass, int wslots, int raw, int *out);

/* Array layouts (for bf_form_beams_layout).  BF_A_LINEAR / BF_J_LINEAR are the
 * reference's A[f][b][d] and J[b][f][p][t] (Alinear, Jlinear; arraysizes.hxx:92,
 * 115) used everywhere else in this API.  BF_A_A2 is the lossy kernel family's
 * A2[f][b][c][d']: per (f, b) the real parts then the imaginary parts of all
 * dishes as 4-bit nibbles, two per byte (even d' in the low nibble), in the dish
 * order d' = bits 8 | 5..0 | 7..6 of d (A2linear, arraysizes.hxx:125;
 * cuda4.cu:1468-1494); defined for ndishes 256 and 512.  BF_J_J2 is
 * J2[b][f][t][p] (J2linear, arraysizes.hxx:103). */
typedef enum bf_a_layout { BF_A_LINEAR = 0, BF_A_A2 = 1 } bf_a_layout;
typedef enum bf_j_layout { BF_J_LINEAR = 0, BF_J_J2 = 1 } bf_j_layout;

/* bf_form_beams_ex with A read in a_layout and J written in j_layout; the
 * values are identical (J2 holds J's bytes permuted).  BF_ERR_UNSUPPORTED for
 * BF_A_A2 with ndishes other than 256 or 512. */
BF_API int bf_form_beams_layout(const bf_dims *dims, uint8_t *J, const uint8_t *E, const uint8_t *A, const float *G,
                                int a_layout, int j_layout, int ptr_kind, bf_stream_t stream);

/* bf_form_beams_layout that also returns in *adler the adler32 (adler32.c:7-20)
 * of the whole J it wrote, jsize bytes in j_layout: the checksum the
 * reference's main() computes after form_beams (arraysizes.cxx:79), without a
 * second pass over J.  The tensor-core kernel sums the bytes it stores (two
 * dp4a per 4 bytes, positions mod 65521) and a host step finishes
 * a = 1 + sum d_i, b = n + n sum d_i - sum i d_i; when the dp4a kernel runs
 * instead, J is checksummed by bf_adler32_device's pass.  Synchronous for
 * both pointer kinds: *adler is set when it returns BF_OK. */
BF_API int bf_form_beams_adler(const bf_dims *dims, uint8_t *J, const uint8_t *E, const uint8_t *A, const float *G,
                               int a_layout, int j_layout, int ptr_kind, uint32_t *adler, bf_stream_t stream);

/* Measures the dense E4M3 tensor-core rate of the current device, in
 * TFLOP/s (two flops per multiply-add): every SM issues back-to-back
 * tcgen05 MMAs of the kind the beamformer uses (M=128, N=256, K=32, A operand
 * in tensor memory), timed with CUDA events at the run's own clocks.  It is
 * the tensor roofline the benchmarks report fractions of; takes ~15 ms. */
BF_API int bf_tensor_peak(double *tflops, bf_stream_t stream);

/* Measures the CUDA-core dp4a rate of the current device, in dp4a lane
 * operations per second (four int8 multiply-adds each): every SM runs
 * independent dp4a chains, timed with CUDA events.  The roofline of the exact
 * dp4a kernel; takes a few ms. */
BF_API int bf_dp4a_peak(double *dp4a_per_s, bf_stream_t stream);

/* ---------------------------------------------------------------- serving */

/* A served stream of voltage chunks with continuous batching.  No
 * counterpart in the reference.  A server thread admits submitted chunks while
 * a fixed HBM pool has room for their buffers, packs them into one grouped
 * tensor-core launch, and keeps up to max_inflight launches in flight, so
 * chunks that arrive while others run are admitted as memory and launch slots
 * free up.  The caller's resident weights must not be updated while chunks
 * are in flight (drain first); bf_server_update_weights refreshes the
 * server's weights without a drain. */
typedef struct bf_server bf_server;

typedef struct bf_server_config {
  int64_t hbm_budget_bytes; /* device pool for chunk buffers; 0: half of the free HBM */
  int max_batch;            /* chunks per grouped launch; 0: 64 (1: plain per-chunk launches) */
  int max_inflight;         /* launches in flight; 0: 3 */
  int spin_wait;            /* 1: the server thread polls launches instead of sleeping until a host
                               callback wakes it (lower latency; keeps one host core busy) */
  int64_t staging_bytes;    /* pinned host ring for chunks whose host buffers are pageable: the
                               submitting thread copies E into it, the server copies J out of it
                               when the chunk lands, so the device copies stay asynchronous;
                               0: 256 MiB, < 0: none (pageable buffers are copied directly) */
} bf_server_config;

typedef struct bf_server_stats {
  int64_t submitted, completed;
  int64_t batches, chunks_launched, max_batch_seen;
  int64_t pool_bytes, pool_peak_bytes;
  int64_t weight_updates;
  int64_t staged;           /* chunks whose E or J went through the pinned staging ring */
} bf_server_stats;

/* Creates a server over resident weights (all channels = the weights' frequencies). */
BF_API int bf_server_create(bf_server **out, const bf_weights *weights, const bf_server_config *config);

/* Submits one chunk: channels [channel, channel + nchannels) of ntimes samples,
 * E[t][c][d][p] and J[b][c][p][t] in host memory or device memory
 * (e_on_device / j_on_device).  Pinned host buffers are copied directly;
 * pageable ones go through the server's pinned staging ring, so this call
 * copies E into the ring first (waiting for room if landed chunks have not
 * freed enough yet).  Returns with a ticket; the arrival time is the moment
 * of the call.  Needs ntimes % 16 == 0. */
BF_API int bf_server_submit(bf_server *server, int channel, int nchannels, int64_t ntimes, const uint8_t *E,
                            int e_on_device, uint8_t *J, int j_on_device, int64_t *ticket);

/* Refreshes the weights (A[f][b][d], G[f][b] for all of the server's channels,
 * host or device memory per ptr_kind) without draining: chunks submitted
 * after this call use the new weights, chunks submitted before it keep the
 * weights they were submitted under.  The server keeps up to three refreshed
 * versions besides the caller's own weights (which it never writes); the call
 * waits only while every version still has chunks on it.  A and G may be
 * reused when it returns. */
BF_API int bf_server_update_weights(bf_server *server, const uint8_t *A, const float *G, int ptr_kind);

/* Blocks until the ticket's chunk is complete (J written); returns its latency
 * (submission to completion) in seconds. */
BF_API int bf_server_wait(bf_server *server, int64_t ticket, double *latency_s);

/* Blocks until every submitted chunk is complete. */
BF_API int bf_server_drain(bf_server *server);

BF_API int bf_server_stats_get(bf_server *server, bf_server_stats *stats);

/* A load generator for measuring a server without an interpreter in the
 * loop.  Chunk i (one channel channel[i], ntimes[i] samples, input E[i]) is
 * submitted by the calling thread arrival_s[i] seconds after the call (all 0:
 * back to back) into J slot i % nslots (J_slots[k], j_bytes[i] bytes used);
 * a native thread waits for the chunks in order and stores each latency
 * (submission to completion) in latency_s[i], and check_threads native threads
 * (0: none) store the adler32 of each landed J in adler_out[i] before its slot
 * is given to a later chunk (a submission waits for that: *slot_stalls counts
 * the waits).  late_s[i] (may be NULL) is how late chunk i was submitted.
 * Returns when every chunk is complete and checked, with the time from the
 * call to the last completion in *wall_s.  Checking needs J in host memory.
 * On an error (a failed submission or wait) it returns that status without
 * submitting more; chunks already submitted may still be landing in their J
 * slots, so keep E and the J slots alive until bf_server_destroy, which waits
 * for them.  No counterpart in the reference. */
BF_API int bf_server_replay(bf_server *server, int n, const int *channel, const int64_t *ntimes,
                            const uint8_t *const *E, int e_on_device, uint8_t *const *J_slots, int nslots,
                            const int64_t *j_bytes, int j_on_device, const double *arrival_s, int check_threads,
                            double *latency_s, double *late_s, uint32_t *adler_out, double *wall_s,
                            int64_t *slot_stalls);

BF_API int bf_server_destroy(bf_server *server);

/* ------------------------------------------------------- no allocation */

/* No counterpart in the reference.  For callers that cannot allocate device
 * memory -- e.g. a real-time pipeline that sizes all device memory once at
 * start-up and must not allocate mid-stream, or a host framework that owns
 * the memory pool: the tensor-core pass of bf_form_beams_ex(..., BF_PTR_DEVICE,
 * ...) with its scratch (prepared weight operand, row-sum digits, error word) in one
 * fixed 4 MiB device array that every GPU loading the library holds until the
 * process exits.  It calls no cudaMalloc, cudaFree or other allocating routine.
 *
 * E, A, G and J are device pointers.  Limits: the tensor-core shape rules
 * (npolarizations == 2, ndishes % 8 == 0, ntimes % 16 == 0, E and J 16-byte
 * aligned, ndishes <= 2048; else BF_ERR_UNSUPPORTED) and
 *   256 + roundup256(68 * F * npass * nb + 4 * F) + F * 2 * roundup(B, 8) * 2 * D <= 4 MiB
 * (npass = ceil(roundup(B, 8) / 96), nb = roundup(ceil(roundup(B, 8) / npass), 8); else
 * BF_ERR_TOO_LARGE) -- e.g. f=16, b=96, d=512 fits, f=84 does not.
 * Synchronous: returns once the pass on `stream` has finished, with its status.
 * The first call on a device looks up the array's device address; make that
 * first call before any stream capture.  All calls on a device share the one
 * array and each call overwrites it: calls that overlap on the GPU (e.g. from
 * two host threads at once) race and must be serialised by the caller. */
BF_API int bf_form_beams_noalloc(const bf_dims *dims, uint8_t *J, const uint8_t *E, const uint8_t *A,
                                 const float *G, bf_stream_t stream);

/* ---------------------------------------------------------------- checksum */

/* adler32 (adler32.c:7-20) of `len` bytes of device memory; the result is
 * written to *out (host).  Synchronous on `stream`. */
BF_API int bf_adler32_device(const uint8_t *data, size_t len, uint32_t *out, bf_stream_t stream);

/* adler32 of `len` bytes of host memory on the calling thread; needs no device. */
BF_API int bf_adler32_host(const uint8_t *data, size_t len, uint32_t *out);

/* ------------------------------------------------------- workload generator */

/* Seeded uniform bytes (each ucomplex4 nibble uniform on [-8,7]) into device
 * memory: byte i is byte (i % 8), little-endian, of
 *   mix64(key + (i/8 + 1) * 0x9E3779B97F4A7C15),  key = mix64(seed * 2 + stream_id + 1),
 * mix64 the SplitMix64 finaliser.  stream_id 0 is used for E, 1 for A. */
BF_API int bf_fill_random_device(uint8_t *dst, size_t n, uint64_t seed, uint64_t stream_id, bf_stream_t stream);

/* The same bytes into host memory (multi-threaded). */
BF_API int bf_fill_random_host(uint8_t *dst, size_t n, uint64_t seed, uint64_t stream_id);

/* setup()'s gain formula (arraysizes.cxx:31-32) for a shape, into host memory. */
BF_API int bf_gains_host(const bf_dims *dims, float *G);

#ifdef __cplusplus
}
#endif

#endif /* BEAMFORM_H */
