// bf_internal.h -- declarations shared by the host API (bf_api.cu) and the
// kernel translation units.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <cstdint>

#include "../../include/beamform.h"

namespace bf {

// Array layouts besides the reference's Alinear / Jlinear (arraysizes.hxx:92,
// 115): the lossy kernel family's A2[f][b][c][d'] (A2linear, arraysizes.hxx:125,
// dish order d' of cuda4.cu:1468-1494, two dishes' nibbles per byte) and
// J2[b][f][t][p] (J2linear, arraysizes.hxx:103).
enum ALayout : int { kALinear = 0, kA2 = 1 };
enum JLayout : int { kJLinear = 0, kJ2 = 1 };

// A2 is defined for ndishes 256 and 512 (its dish permutation is a bijection there).
inline bool a2_supported(int64_t ndishes) { return ndishes == 256 || ndishes == 512; }

// Position d' of dish d in A2 (cuda4.cu:1472-1476): bits 8 | 5..0 | 7..6.
__host__ __device__ __forceinline__ int64_t a2_dish(int64_t d) {
  return (d & 0x100) | ((d & 0x3F) << 2) | ((d >> 6) & 3);
}

#ifdef __CUDACC__
// Signed 4-bit value of nibble i of a ucomplex4 array: odd i the high (real)
// nibble of byte i / 2, even i the low (imaginary) one (icomplex4.hxx:33-38).
__device__ __forceinline__ int a2_nibble(const uint8_t *A, int64_t i) {
  const uint32_t x = static_cast<uint32_t>(A[i >> 1]) ^ 0x88u;
  return (i & 1) ? static_cast<int>(static_cast<int8_t>(x)) >> 4
                 : static_cast<int>(static_cast<int8_t>(static_cast<uint8_t>(x << 4))) >> 4;
}

// max(-7, min(7, int(lrint(x)))) of cpu.cxx:38-39 for any float x.  lrint
// rounds half to even to a 64-bit long and the int(...) narrowing comes before
// the clamp, so 2^31 <= |x| < 2^63 keeps the low 32 bits of the rounded value
// (two's complement); NaN, infinities and |x| >= 2^63 give 0, the x86-64
// lrint result LONG_MIN narrowed (the reference's own build, checked against
// it on huge gains).
__device__ __forceinline__ int requant_narrow(float x) {
  if (!(fabsf(x) < 9.223372036854775808e18f)) return 0;  // 2^63
  const int v = static_cast<int>(static_cast<unsigned>(static_cast<unsigned long long>(__float2ll_rn(x))));
  return max(-7, min(7, v));
}

// Real and imaginary part of the weight of dish d, beam b, frequency f.
__device__ __forceinline__ void load_a(const uint8_t *A, int a_layout, int64_t f, int64_t b, int64_t d, int64_t B,
                                       int64_t D, int &re, int &im) {
  if (a_layout == kALinear) {  // A[f][b][d] (Alinear, arraysizes.hxx:115)
    const uint32_t a = static_cast<uint32_t>(A[(f * B + b) * D + d]) ^ 0x88u;
    re = static_cast<int>(static_cast<int8_t>(a)) >> 4;
    im = static_cast<int>(static_cast<int8_t>(static_cast<uint8_t>(a << 4))) >> 4;
  } else {  // A2linear(f, b, c, d') = d' + D (c + 2 (b + B f)) nibbles (arraysizes.hxx:125)
    const int64_t base = (f * B + b) * 2 * D + a2_dish(d);
    re = a2_nibble(A, base);
    im = a2_nibble(A, base + D);
  }
}
#endif

// True while bf_set_kernel(BF_KERNEL_SIMT4) selects the 4-multiply SIMT
// kernel; otherwise launch_simt runs the Gauss 3-multiply kernel.
bool simt_four_multiply();

// Exact integer SIMT kernel (dp4a); any shape with npolarizations <= 2.  J
// rows (b, f, p) -- (b, f) for J2 -- are `jpitch` (2 * jpitch for J2) bytes
// apart (0: ntimes).
cudaError_t launch_simt(const bf_dims &d, uint8_t *J, const uint8_t *E, const uint8_t *A, const float *G,
                        cudaStream_t s, int64_t jpitch = 0, int a_layout = kALinear, int j_layout = kJLinear);

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
  float *gs = nullptr;       // [F][nw_pad / 2]: 512 * G, zero past B (the epilogue's gains)
  int *gwide = nullptr;      // [F]: nonzero when a gain of the frequency can take |G * raw| to 2^31
  const float *G = nullptr;  // [F][B] (device; read by the weight preparation)
};

// The digit rows, the scaled gains and the wide-gain flags share one
// allocation: digit rows first (F * nw_pad * 32 bytes, a multiple of 32), then
// the gains (F * nw_pad / 2 floats), then one int per frequency.
inline size_t tc_extra_bytes(const TcWeights &w) {
  return static_cast<size_t>(w.F) * w.nw_pad * (kDigitRow + sizeof(float) / 2) + static_cast<size_t>(w.F) * sizeof(int);
}
inline void tc_set_extra(TcWeights &w, uint8_t *p) {
  w.dig = p;
  w.gs = reinterpret_cast<float *>(p + static_cast<size_t>(w.F) * w.nw_pad * kDigitRow);
  w.gwide = reinterpret_cast<int *>(w.gs + static_cast<size_t>(w.F) * w.nw_pad / 2);
}

// True when the tensor-core kernel handles this shape.
bool tc_supported(const bf_dims &d);

// Beams per pass and number of passes for B beams.
void tc_plan_beams(int64_t B, int *nb_pass, int *npass);

// Fills w.W, w.dig and w.gs from device A and w.G (w's sizes and buffers already set).
cudaError_t launch_prep_weights(const TcWeights &w, const uint8_t *A, cudaStream_t s, int a_layout = kALinear);

// Beamforms T times of device E into device J with prepared weights.  `err`
// is a device int that receives a nonzero DeviceError on an expired wait.
// J rows (b, f, p) are `jpitch` bytes apart (0: T), so a time chunk of a longer
// pass can be written in place: E and J point at the chunk's first time.
// With `adler` set, the epilogue also adds every J byte it stores into the
// adler32 sums adler[0] += d_i, adler[1] += i * d_i (i = byte position from
// jbase, taken mod 65521); the caller zeroes them first and finishes the
// checksum with adler_finish().
cudaError_t launch_tc(const TcWeights &w, int64_t T, uint8_t *J, const uint8_t *E, int *err, cudaStream_t s,
                      int64_t jpitch = 0, int j_layout = kJLinear, unsigned long long *adler = nullptr,
                      const uint8_t *jbase = nullptr);
constexpr uint32_t kAdlerMod = 65521;
// adler32 of n bytes from S1 = sum d_i and S2 = sum i d_i (i from 0, both taken
// mod 65521 or not): a = 1 + S1, b = n + n S1 - S2 (adler32.c:7-20 unrolled).
inline uint32_t adler_finish(unsigned long long s1, unsigned long long s2, unsigned long long n) {
  const unsigned long long m = kAdlerMod;
  const unsigned long long a = (1 + s1 % m) % m;
  const unsigned long long b = (n % m + (n % m) * (s1 % m) % m + m - s2 % m) % m;
  return static_cast<uint32_t>((b << 16) | a);
}

// One beamforming problem of a tensor-core launch: operand descriptors,
// pointers, shape.  A plain launch carries one inline; a grouped launch reads
// an array of them from device memory, ordered by tile_begin.
struct TcProblem {  // 128-byte aligned through its tensor maps
  CUtensorMap tm_e;  // E[t][f][d*p] bytes: dims {2D, F, T}, box {128, 1, 64}, 128B swizzle
  CUtensorMap tm_w;  // W[f][n][k] bytes: dims {2D, nw, F}, box {128, 2*nb_pass, 1}, 128B swizzle
  CUtensorMap tm_d;  // digits[f][n][32] bytes: dims {32, nw_pad, F}, box {32, 2*nb_pass, 1}, 32B swizzle
  uint8_t *J;
  const uint8_t *jbase;        // start of the whole J buffer: byte positions of the fused adler32
  unsigned long long *adler;   // null, or the fused adler32 sums {sum d_i, sum i * d_i} (device)
  const float *gs;   // scaled gains [F][npass * nb_pass]
  const int *gwide;  // [F]: the frequency needs the narrowing requantisation (huge or non-finite gains)
  int64_t jpitch;    // bytes between consecutive (b, f, p) rows of J (J2: (b, f) rows are 2 * jpitch apart)
  int jlayout;       // JLayout
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
                            int64_t jpitch, int j_layout = kJLinear);
// Tiles of a problem, and K stages per tile for D dishes.
int64_t tc_problem_tiles(const TcProblem &P);
int tc_stages_per_tile(int64_t D);

// One persistent launch over nprob problems (records in device memory; all
// with D dishes).  max_nb_pass = the largest nb_pass among them.
cudaError_t launch_tc_grouped(const TcProblem *table, int nprob, int ntiles, int64_t D, int max_nb_pass,
                              const TcRingPlan &plan, int *err, cudaStream_t s);

// The whole ring layout of a launch with these sizes: out[0..11] = stages,
// W slots, raw E slots, unpack groups, CTAs per SM, K stages per tile,
// dynamic shared memory bytes, TMEM columns allocated, accumulator columns,
// column of the second accumulator, stages beside each accumulator, one past
// the last TMEM column a stage uses.
cudaError_t tc_plan_rings(int64_t D, int max_nb_pass, const TcRingPlan &plan, int *out);

// TMEM stages, unpack groups and CTAs per SM of a grouped launch with these sizes.
cudaError_t tc_launch_shape(int64_t D, int max_nb_pass, const TcRingPlan &plan, int *stages, int *groups,
                            int *ctas_per_sm);

// Beam passes of at most kNarrowPass beams leave room for four or more
// unpacked stages in TMEM, and so for two unpack groups.  Passes of at most
// kHalfPass beams fit a CTA with half the SM's TMEM and shared memory, so two
// CTAs share each SM (measured 1.3x on b = 16 passes; at b = 32 the two TMEM
// stages a half CTA keeps lose 5% against six stages and two unpack groups).
constexpr int kNarrowPass = 64;
constexpr int kHalfPass = 16;

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
// adler32 of n bytes of host memory (adler32.c:7-20).
uint32_t adler32_host(const uint8_t *p, size_t n);

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
