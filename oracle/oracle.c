/*
 * oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the reference beamformer (eschnett/beamforming, cpu.cxx)
 * with run-time sizes.  It is the checker for the CUDA path and the timed CPU
 * baseline; nothing in the product path calls it.  Its results are pinned to
 * the reference by the golden checksums of arraysizes.cxx:54-57 and by
 * byte-for-byte comparison with the reference's own cpu.cxx compiled from its
 * sources (oracle/build_ref.sh).
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ucomplex4(real, imag) constructor: icomplex4.hxx:33.  The real part sits in
 * the high nibble, the imaginary part in the low nibble, and the byte is
 * xor'ed with 0x88 (offset-binary storage, x stored as x + 8). */
uint8_t bfo_encode(int re, int im) { return (uint8_t)((((unsigned)(re & 0x0f) << 4) | (unsigned)(im & 0x0f)) ^ 0x88u); }

/* ucomplex4::real(): icomplex4.hxx:37 (arithmetic shift of the de-biased byte). */
int bfo_decode_re(uint8_t data) { return (int)(int8_t)(uint8_t)(data ^ 0x88u) >> 4; }

/* ucomplex4::imag(): icomplex4.hxx:38. */
int bfo_decode_im(uint8_t data) { return (int)(int8_t)(uint8_t)((uint8_t)(data ^ 0x88u) << 4) >> 4; }

/* Requantisation of one accumulator: cpu.cxx:37-39.
 *   max(-7, min(7, int(lrint(G * float(raw)))))
 * G * float(raw) is one IEEE single-precision multiply; lrint rounds half to
 * even in the default rounding mode and returns a 64-bit long.  The int(...)
 * narrowing comes BEFORE the clamp, so a product with 2^31 <= |x| < 2^63 keeps
 * only its low 32 bits (two's complement, as GCC defines the conversion): the
 * clamp then gives 0, +7 or -7 from those bits, not the sign of x.  For NaN,
 * infinities and |x| >= 2^63 lrint has no long to return; the reference's
 * x86-64 build returns LONG_MIN (the "integer indefinite" of cvtss2si), whose
 * low 32 bits are 0.  Both rules are written out here instead of relying on
 * the host's lrintf, so the oracle gives the same bytes on every host. */
static inline int requant(float g, int32_t raw) {
  const float x = g * (float)raw;
  if (!(fabsf(x) < 0x1p63f)) return 0; /* NaN, +-inf, |x| >= 2^63 */
  const uint32_t lo = (uint32_t)(uint64_t)(int64_t)lrintf(x); /* exact below 2^63 */
  const int32_t v = lo >= 0x80000000u ? -(int32_t)(0xFFFFFFFFu - lo) - 1 : (int32_t)lo;
  return v > 7 ? 7 : (v < -7 ? -7 : (int)v);
}

#define T_BLOCK 64

/* form_beams: cpu.cxx:15-46.
 *
 * The reference loops b (OpenMP) -> f -> p -> t -> d.  The integer sums are
 * exact, so the loop order does not change any result; this restatement
 * decodes one (f, 64-time) block of E and one frequency of A into int8 planes
 * and forms the same sums
 *   rawJre = sum_d Are*Ere - Aim*Eim,   rawJim = sum_d Are*Eim + Aim*Ere
 * (cpu.cxx:26-35), then requantises and stores ucomplex4(Jre, Jim) at
 * Jlinear(b,f,p,t) (cpu.cxx:37-41). */
void bfo_form_beams(const bfo_dims *dm, uint8_t *J, const uint8_t *E, const uint8_t *A, const float *G, int nthreads) {
  const int64_t T = dm->ntimes, F = dm->nfrequencies, D = dm->ndishes, P = dm->npolarizations, B = dm->nbeams;
  if (T <= 0 || F <= 0 || D <= 0 || P <= 0 || B <= 0) return;
  const int64_t ntb = (T + T_BLOCK - 1) / T_BLOCK;
  const int64_t njobs = F * ntb;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
  (void)nthreads;
#endif

#pragma omp parallel num_threads(nthreads)
  {
    int8_t *ar = (int8_t *)malloc((size_t)(B * D));
    int8_t *ai = (int8_t *)malloc((size_t)(B * D));
    int8_t *er = (int8_t *)malloc((size_t)(P * T_BLOCK * D));
    int8_t *ei = (int8_t *)malloc((size_t)(P * T_BLOCK * D));
    int64_t cur_f = -1;

#pragma omp for schedule(dynamic, 1)
    for (int64_t job = 0; job < njobs; ++job) {
      const int64_t f = job / ntb;
      const int64_t t0 = (job % ntb) * T_BLOCK;
      const int64_t tn = (T - t0) < T_BLOCK ? (T - t0) : T_BLOCK;

      if (f != cur_f) {
        /* A[f][b][d] (Alinear, arraysizes.hxx:115) */
        for (int64_t b = 0; b < B; ++b)
          for (int64_t d = 0; d < D; ++d) {
            const uint8_t a = A[(f * B + b) * D + d];
            ar[b * D + d] = (int8_t)bfo_decode_re(a);
            ai[b * D + d] = (int8_t)bfo_decode_im(a);
          }
        cur_f = f;
      }
      /* E[t][f][d][p] (Elinear, arraysizes.hxx:80) */
      for (int64_t tt = 0; tt < tn; ++tt) {
        const uint8_t *row = E + ((t0 + tt) * F + f) * D * P;
        for (int64_t d = 0; d < D; ++d)
          for (int64_t p = 0; p < P; ++p) {
            const uint8_t e = row[d * P + p];
            er[(p * T_BLOCK + tt) * D + d] = (int8_t)bfo_decode_re(e);
            ei[(p * T_BLOCK + tt) * D + d] = (int8_t)bfo_decode_im(e);
          }
      }

      for (int64_t b = 0; b < B; ++b) {
        const int8_t *arb = ar + b * D;
        const int8_t *aib = ai + b * D;
        const float g = G[f * B + b]; /* Glinear, arraysizes.hxx:136 */
        for (int64_t p = 0; p < P; ++p) {
          uint8_t *jrow = J + ((b * F + f) * P + p) * T; /* Jlinear, arraysizes.hxx:92 */
          for (int64_t tt = 0; tt < tn; ++tt) {
            const int8_t *erp = er + (p * T_BLOCK + tt) * D;
            const int8_t *eip = ei + (p * T_BLOCK + tt) * D;
            int32_t re = 0, im = 0;
            for (int64_t d = 0; d < D; ++d) {
              re += (int32_t)arb[d] * erp[d] - (int32_t)aib[d] * eip[d];
              im += (int32_t)arb[d] * eip[d] + (int32_t)aib[d] * erp[d];
            }
            jrow[t0 + tt] = bfo_encode(requant(g, re), requant(g, im));
          }
        }
      }
    }
    free(ar);
    free(ai);
    free(er);
    free(ei);
  }
}

/* The two int accumulators of cpu.cxx:24-35 for one output element. */
void bfo_raw_sum(const bfo_dims *dm, const uint8_t *E, const uint8_t *A, int64_t b, int64_t f, int64_t p, int64_t t,
                 int32_t *re, int32_t *im) {
  const int64_t F = dm->nfrequencies, D = dm->ndishes, P = dm->npolarizations, B = dm->nbeams;
  int32_t sre = 0, sim = 0;
  for (int64_t d = 0; d < D; ++d) {
    const uint8_t a = A[(f * B + b) * D + d];
    const uint8_t e = E[((t * F + f) * D + d) * P + p];
    const int are = bfo_decode_re(a), aim = bfo_decode_im(a);
    const int ere = bfo_decode_re(e), eim = bfo_decode_im(e);
    sre += are * ere - aim * eim;
    sim += are * eim + aim * ere;
  }
  *re = sre;
  *im = sim;
}

/* A[f][b][d] -> A2[f][b][c][d'] (A2linear, arraysizes.hxx:125-133): component c
 * of dish d as the nibble at A2linear(f, b, c, d'), two per ucomplex4 byte (even
 * d' in the imaginary slot, odd d' in the real slot), d' the dish order of
 * cuda4.cu:1468-1494 (bits 8 | 5..0 | 7..6 of d; a permutation for D = 256, 512). */
void bfo_A_to_A2(const bfo_dims *dm, uint8_t *A2, const uint8_t *A) {
  const int64_t F = dm->nfrequencies, B = dm->nbeams, D = dm->ndishes;
  for (int64_t f = 0; f < F; ++f)
    for (int64_t b = 0; b < B; ++b)
      for (int64_t c = 0; c < 2; ++c)
        for (int64_t d = 0; d < D; ++d) {
          const int64_t dp = (d & 0x100) | ((d & 63) << 2) | ((d >> 6) & 3);
          const int64_t i = dp + D * (c + 2 * (b + B * f));
          const int v = c == 0 ? bfo_decode_re(A[(f * B + b) * D + d]) : bfo_decode_im(A[(f * B + b) * D + d]);
          uint8_t *byte = &A2[i / 2];
          const int re = (dp % 2 == 0) ? bfo_decode_re(*byte) : v;
          const int im = (dp % 2 == 0) ? v : bfo_decode_im(*byte);
          *byte = bfo_encode(re, im);
        }
}

/* J[b][f][p][t] -> J2[b][f][t][p] (J2linear, arraysizes.hxx:103-112). */
void bfo_J_to_J2(const bfo_dims *dm, uint8_t *J2, const uint8_t *J) {
  const int64_t T = dm->ntimes, F = dm->nfrequencies, P = dm->npolarizations, B = dm->nbeams;
  for (int64_t b = 0; b < B; ++b)
    for (int64_t f = 0; f < F; ++f)
      for (int64_t p = 0; p < P; ++p)
        for (int64_t t = 0; t < T; ++t) J2[((b * F + f) * T + t) * P + p] = J[((b * F + f) * P + p) * T + t];
}

/* adler32: adler32.c:7-20 (byte-serial, modulo 65521 after every byte). */
uint32_t bfo_adler32(const uint8_t *data, size_t len) {
  const uint32_t MOD = 65521u;
  uint32_t a = 1, b = 0;
  for (size_t i = 0; i < len; ++i) {
    a = (a + data[i]) % MOD;
    b = (b + a) % MOD;
  }
  return (b << 16) | a;
}

/* Gain formula of setup(): arraysizes.cxx:31-32,
 *   G[n] = float(n) / Gsize / ndishes * (15 + n % 15) / 30
 * evaluated left to right in single precision, as the C++ source does. */
void bfo_gains(const bfo_dims *dm, float *G) {
  const int64_t gsize = dm->nfrequencies * dm->nbeams;
  const float fg = (float)(uint64_t)gsize;
  const float fd = (float)(uint64_t)dm->ndishes;
  for (int64_t n = 0; n < gsize; ++n) {
    float g = (float)(uint64_t)n;
    g = g / fg;
    g = g / fd;
    g = g * (float)(uint64_t)(15 + n % 15);
    g = g / 30.0f;
    G[n] = g;
  }
}

/* setup(): arraysizes.cxx:16-17 (E), 23-24 (A), 31-32 (G).
 *   E[n] = ucomplex4(n % 15 - 7, (n + 1) % 15 - 7), likewise A. */
void bfo_setup_pattern(const bfo_dims *dm, uint8_t *E, uint8_t *A, float *G) {
  const int64_t esize = dm->ntimes * dm->nfrequencies * dm->ndishes * dm->npolarizations;
  const int64_t asize = dm->nfrequencies * dm->nbeams * dm->ndishes;
  for (int64_t n = 0; n < esize; ++n) E[n] = bfo_encode((int)(n % 15) - 7, (int)((n + 1) % 15) - 7);
  for (int64_t n = 0; n < asize; ++n) A[n] = bfo_encode((int)(n % 15) - 7, (int)((n + 1) % 15) - 7);
  bfo_gains(dm, G);
}

/* SplitMix64 finaliser (Steele, Lea & Flood, OOPSLA 2014). */
static inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

void bfo_fill_random(uint8_t *dst, size_t n, uint64_t seed, uint64_t stream) {
  const uint64_t key = mix64(seed * 2u + stream + 1u);
  const size_t nwords = n / 8;
#pragma omp parallel for schedule(static)
  for (size_t j = 0; j < nwords; ++j) {
    const uint64_t w = mix64(key + (uint64_t)(j + 1) * 0x9E3779B97F4A7C15ull);
    for (int k = 0; k < 8; ++k) dst[8 * j + k] = (uint8_t)(w >> (8 * k));
  }
  if (n % 8) {
    const uint64_t w = mix64(key + (uint64_t)(nwords + 1) * 0x9E3779B97F4A7C15ull);
    for (size_t k = 0; k < n % 8; ++k) dst[8 * nwords + k] = (uint8_t)(w >> (8 * k));
  }
}
