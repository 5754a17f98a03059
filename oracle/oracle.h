/*
 * oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the reference beamformer (eschnett/beamforming) used as
 * the checker for the CUDA path.  Only the test suite, the smoke check and the
 * CPU-baseline leg of the benchmark may load this library; the product path
 * never calls into it.
 *
 * Every function cites the reference file:line it restates.
 */
#ifndef BF_ORACLE_H
#define BF_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Problem shape.  The reference fixes these as compile-time constants
 * (arraysizes.hxx:22-27: ntimes, nfrequencies, ndishes, npolarizations,
 * nbeams); the restatement takes them at run time. */
typedef struct bfo_dims {
  int64_t ntimes;
  int64_t nfrequencies;
  int64_t ndishes;
  int64_t npolarizations;
  int64_t nbeams;
} bfo_dims;

/* ucomplex4 encode/decode (icomplex4.hxx:33,37,38). */
uint8_t bfo_encode(int re, int im);
int bfo_decode_re(uint8_t data);
int bfo_decode_im(uint8_t data);

/* form_beams (cpu.cxx:15-46).  Byte arrays in the reference layouts:
 *   E[t][f][d][p]  (Elinear, arraysizes.hxx:80)
 *   A[f][b][d]     (Alinear, arraysizes.hxx:115)
 *   G[f][b]        (Glinear, arraysizes.hxx:136)
 *   J[b][f][p][t]  (Jlinear, arraysizes.hxx:92)
 * nthreads <= 0 uses every OpenMP thread. */
void bfo_form_beams(const bfo_dims *dims, uint8_t *J, const uint8_t *E, const uint8_t *A, const float *G, int nthreads);

/* Raw (pre-requantisation) sums for one (b,f,p,t): the int accumulators of
 * cpu.cxx:24-35.  Used by tests that look at the integer stage directly. */
void bfo_raw_sum(const bfo_dims *dims, const uint8_t *E, const uint8_t *A, int64_t b, int64_t f, int64_t p, int64_t t,
                 int32_t *re, int32_t *im);

/* J2[b][f][t][p] layout of the lossy kernel family (J2linear, arraysizes.hxx:103). */
void bfo_J_to_J2(const bfo_dims *dims, uint8_t *J2, const uint8_t *J);

/* A2[f][b][c][d'] layout of the lossy kernel family (A2linear, arraysizes.hxx:125;
 * dish order of cuda4.cu:1468-1494); ndishes 256 or 512. */
void bfo_A_to_A2(const bfo_dims *dims, uint8_t *A2, const uint8_t *A);

/* adler32 (adler32.c:7-20). */
uint32_t bfo_adler32(const uint8_t *data, size_t len);

/* setup() pattern (arraysizes.cxx:16-17, 23-24, 31-32). */
void bfo_setup_pattern(const bfo_dims *dims, uint8_t *E, uint8_t *A, float *G);
/* Only the gain formula of setup() (arraysizes.cxx:31-32). */
void bfo_gains(const bfo_dims *dims, float *G);

/* Seeded input bytes: the counter-based generator shared by the CUDA path's
 * workload generator.  Byte i is byte (i % 8) (little-endian) of
 *   mix64(key + (i/8 + 1) * 0x9E3779B97F4A7C15),  key = mix64(seed * 2 + stream + 1),
 * with mix64 the SplitMix64 finaliser.  stream 0 = E, stream 1 = A. */
void bfo_fill_random(uint8_t *dst, size_t n, uint64_t seed, uint64_t stream);

#ifdef __cplusplus
}
#endif

#endif
