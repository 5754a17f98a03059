// bf_internal.h -- declarations shared by the host API (bf_api.cu) and the
// kernel translation units.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <cstdint>

#include "../../include/beamform.h"

namespace bf {

// Exact integer SIMT kernel (dp4a); any shape with npolarizations <= 2.  J
// rows (b, f, p) are `jpitch` bytes apart (0: ntimes).
cudaError_t launch_simt(const bf_dims &d, uint8_t *J, const uint8_t *E, const uint8_t *A, const float *G,
                        cudaStream_t s, int64_t jpitch = 0);

// Tensor-core path ------------------------------------------------------------

// Layout of the resident operand built from A: for each frequency, nw rows of
// 2*D bytes (E4M3 values), and per row a 32-byte row of E4M3 digits of the
// offset correction sum_k W[n][k] (the operand of one extra MMA per tile).
constexpr int kDigitRow = 32;  // bytes per digit row
struct TcWeights {
  int64_t F = 0, B = 0, D = 0;
  int nb_pass = 0;   // beams per tensor-core pass (multiple of 8, <= 128)
  int npass = 0;     // passes over the beams
  int nw = 0;        // W rows per frequency holding data: 2 * roundup(B, 8)
  int nw_pad = 0;    // digit rows per frequency: npass * 2 * nb_pass
  uint8_t *W = nullptr;      // [F][nw][2D]
  uint8_t *dig = nullptr;    // [F][nw_pad][kDigitRow]
  const float *G = nullptr;  // [F][B] (device)
};

// True when the tensor-core kernel handles this shape.
bool tc_supported(const bf_dims &d);

// Beams per pass and number of passes for B beams.
void tc_plan_beams(int64_t B, int *nb_pass, int *npass);

// Fills w.W and w.dig from device A (w's sizes and buffers already set).
cudaError_t launch_prep_weights(const TcWeights &w, const uint8_t *A, cudaStream_t s);

// Beamforms T times of device E into device J with prepared weights.  `err`
// is a device int that receives a nonzero DeviceError on an expired wait.
// J rows (b, f, p) are `jpitch` bytes apart (0: T), so a time chunk of a longer
// pass can be written in place: E and J point at the chunk's first time.
cudaError_t launch_tc(const TcWeights &w, int64_t T, uint8_t *J, const uint8_t *E, int *err, cudaStream_t s,
                      int64_t jpitch = 0);

// One beamforming problem of a tensor-core launch: operand descriptors,
// pointers, shape.  A plain launch carries one inline; a grouped launch reads
// an array of them from device memory, ordered by tile_begin.
struct TcProblem {  // 128-byte aligned through its tensor maps
  CUtensorMap tm_e;  // E[t][f][d*p] bytes: dims {2D, F, T}, box {128, 1, 64}, 128B swizzle
  CUtensorMap tm_w;  // W[f][n][k] bytes: dims {2D, nw, F}, box {128, 2*nb_pass, 1}, 128B swizzle
  CUtensorMap tm_d;  // digits[f][n][32] bytes: dims {32, nw_pad, F}, box {32, 2*nb_pass, 1}, 32B swizzle
  uint8_t *J;
  const float *G;
  int64_t jpitch;    // bytes between consecutive (b, f, p) rows of J
  int T, F, B;
  int nb_pass;       // beams per pass
  int npass;
  int ntt;           // time tiles per frequency
  int nw_pad;        // digit rows per frequency
  int tile_begin;    // first tile of this problem in the launch
};

// Shared-memory ring depths of a launch (0: planner default).
struct TcRingPlan {
  int wslots = 0;
  int raw = 0;
};

// Fills a problem record (tile_begin left 0) for T times of E with weights w.
cudaError_t tc_make_problem(TcProblem &P, const TcWeights &w, int64_t T, uint8_t *J, const uint8_t *E,
                            int64_t jpitch);
// Tiles of a problem, and K stages per tile for D dishes.
int64_t tc_problem_tiles(const TcProblem &P);
int tc_stages_per_tile(int64_t D);

// One persistent launch over nprob problems (records in device memory; all
// with D dishes).  max_nb_pass = the largest nb_pass among them.
cudaError_t launch_tc_grouped(const TcProblem *table, int nprob, int ntiles, int64_t D, int max_nb_pass,
                              const TcRingPlan &plan, int *err, cudaStream_t s);

// Failure-path test hook: nonzero makes the producer of later tensor-core
// launches issue nothing, so the kernel's bounded waits expire.
void tc_set_test_stall(int on);

// Shared-memory ring depths of the tensor-core kernel (0 = planner default):
// W slots and raw E slots.
void tc_set_ring_plan(int wslots, int raw);

// Checksum ----------------------------------------------------------------------
// Partial adler sums over chunks; `partials` holds 2 * nchunks uint32.
int adler_nchunks(size_t len);
cudaError_t launch_adler_partials(const uint8_t *data, size_t len, uint32_t *partials, cudaStream_t s);
// Combines the partials into one adler32 value in *out (device).
cudaError_t launch_adler_combine(const uint32_t *partials, size_t len, uint32_t *out, cudaStream_t s);

// Workload generator.
cudaError_t launch_fill_random(uint8_t *dst, size_t n, uint64_t seed, uint64_t stream_id, cudaStream_t s);

}  // namespace bf

// Device-resident beam weights behind the C ABI's opaque bf_weights handle.
struct bf_weights {
  int device = 0;
  bf::TcWeights tc;
  uint8_t *A = nullptr;  // raw A kept for the SIMT path
  float *G = nullptr;
};

namespace bf {
// The calling thread's device error word (allocated on first use).
int device_error_word(int **out);
}  // namespace bf
