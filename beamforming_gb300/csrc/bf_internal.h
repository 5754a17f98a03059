// bf_internal.h -- declarations shared by the host API (bf_api.cu) and the
// kernel translation units.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#include "../../include/beamform.h"

namespace bf {

// Exact integer SIMT kernel (dp4a); any shape with npolarizations <= 2.  J
// rows (b, f, p) are `jpitch` bytes apart (0: ntimes).
cudaError_t launch_simt(const bf_dims &d, uint8_t *J, const uint8_t *E, const uint8_t *A, const float *G,
                        cudaStream_t s, int64_t jpitch = 0);

// Tensor-core path ------------------------------------------------------------

// Layout of the resident operand built from A: for each frequency, nw_pad
// rows of 2*D bytes (E4M3 values), and a float bias per row.
struct TcWeights {
  int64_t F = 0, B = 0, D = 0;
  int nb_pass = 0;   // beams per tensor-core pass (multiple of 8, <= 128)
  int npass = 0;     // passes over the beams
  int nw = 0;        // W rows per frequency holding data: 2 * roundup(B, 8)
  int nw_pad = 0;    // bias rows per frequency: npass * 2 * nb_pass
  uint8_t *W = nullptr;      // [F][nw][2D]
  float *bias = nullptr;     // [F][nw_pad]
  const float *G = nullptr;  // [F][B] (device)
};

// True when the tensor-core kernel handles this shape.
bool tc_supported(const bf_dims &d);

// Beams per pass and number of passes for B beams.
void tc_plan_beams(int64_t B, int *nb_pass, int *npass);

// Fills w.W and w.bias from device A (w's sizes and buffers already set).
cudaError_t launch_prep_weights(const TcWeights &w, const uint8_t *A, cudaStream_t s);

// Beamforms T times of device E into device J with prepared weights.  `err`
// is a device int that receives a nonzero DeviceError on an expired wait.
// J rows (b, f, p) are `jpitch` bytes apart (0: T), so a time chunk of a longer
// pass can be written in place: E and J point at the chunk's first time.
cudaError_t launch_tc(const TcWeights &w, int64_t T, uint8_t *J, const uint8_t *E, int *err, cudaStream_t s,
                      int64_t jpitch = 0);

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
