// bf_simt.cu -- exact integer beamformer on the CUDA cores (dp4a).
//
// Handles every shape (any ntimes, ndishes, nbeams; 1 or 2 polarizations).
// It is the fallback for shapes the tensor-core kernel does not take and an
// independent second GPU implementation for the parity tests.  Same
// arithmetic as cpu.cxx:24-41: int32 sums of 4-bit products, then
// clamp(lrint(G * float(raw)), -7, 7).
//
// Two kernels form the same integer sums:
//  * bf_form_beams_gauss (the default): the Gauss 3-multiply form,
//      k1 = sum Ar (Er + Ei),  k2 = sum (Ar + Ai) Ei,  k3 = sum (Ai - Ar) Er,
//      rawJre = k1 - k2,  rawJim = k1 + k3,
//    which equals cpu.cxx:33-34 term by term in integers (every factor is in
//    [-16, 15], so int8; |product| <= 128, so int32 sums are exact for any
//    D below 2^24).  Register tiles of 2 (p, t) rows x 4 beams per thread
//    and 16-byte shared-memory loads keep it on the dp4a pipe.
//  * bf_form_beams_simt (BF_KERNEL_SIMT4): the reference's 4-multiply form,
//    one (p, t) row x 8 beams per thread with 4-byte shared loads.
#include "bf_internal.h"

namespace bf {
namespace {

constexpr int kTT = 32;   // times per block
constexpr int kBB = 32;   // beams per block
constexpr int kDC = 64;   // dishes per chunk
constexpr int kDQ = kDC / 4;
constexpr int kThreads = 256;

__device__ __forceinline__ int dec_re(uint32_t byte) { return static_cast<int>(static_cast<int8_t>(byte ^ 0x88u)) >> 4; }
__device__ __forceinline__ int dec_im(uint32_t byte) {
  return static_cast<int>(static_cast<int8_t>(static_cast<uint8_t>((byte ^ 0x88u) << 4))) >> 4;
}
__device__ __forceinline__ uint32_t pack4(int a, int b, int c, int d) {
  return (static_cast<uint32_t>(a) & 0xFFu) | ((static_cast<uint32_t>(b) & 0xFFu) << 8) |
         ((static_cast<uint32_t>(c) & 0xFFu) << 16) | ((static_cast<uint32_t>(d) & 0xFFu) << 24);
}
// clamp(int(lrint(G * float(raw))), -7, 7): cpu.cxx:37-39.  __fmul_rn is one
// IEEE single multiply (never fused); requant_narrow rounds and narrows like
// int(lrint(x)).
__device__ __forceinline__ int requant(float g, int raw) {
  return requant_narrow(__fmul_rn(g, __int2float_rn(raw)));
}

__global__ void __launch_bounds__(kThreads) bf_form_beams_simt(uint8_t *__restrict__ J, const uint8_t *__restrict__ E,
                                                               const uint8_t *__restrict__ A,
                                                               const float *__restrict__ G, int64_t T, int64_t F,
                                                               int64_t D, int64_t P, int64_t B, int64_t jpitch,
                                                               int a_layout, int j_layout) {
  __shared__ int32_t s_er[2][kTT][kDQ + 1];
  __shared__ int32_t s_ei[2][kTT][kDQ + 1];
  __shared__ int32_t s_ar[kBB][kDQ];
  __shared__ int32_t s_ai[kBB][kDQ];
  __shared__ int32_t s_nai[kBB][kDQ];

  const int64_t t0 = static_cast<int64_t>(blockIdx.x) * kTT;
  const int64_t f = blockIdx.y;
  const int64_t b0 = static_cast<int64_t>(blockIdx.z) * kBB;
  const int tid = threadIdx.x;
  const int rows = static_cast<int>(P) * kTT;  // (p, t) rows, <= 64
  const int row = tid % 64;
  const int bsub = tid / 64;  // beams bsub, bsub + 4, ...
  const int p = row / kTT;
  const int tl = row % kTT;

  int acc_re[8], acc_im[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) acc_re[k] = acc_im[k] = 0;

  for (int64_t d0 = 0; d0 < D; d0 += kDC) {
    __syncthreads();
    // E[t][f][d][p] -> packed int8 planes (Elinear, arraysizes.hxx:80).
    for (int idx = tid; idx < rows * kDQ; idx += kThreads) {
      const int pp = idx / (kTT * kDQ);
      const int rem = idx % (kTT * kDQ);
      const int tt = rem / kDQ, dq = rem % kDQ;
      const int64_t t = t0 + tt;
      int re[4] = {0, 0, 0, 0}, im[4] = {0, 0, 0, 0};
      if (t < T) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int64_t d = d0 + 4 * dq + i;
          if (d < D) {
            const uint32_t e = E[((t * F + f) * D + d) * P + pp];
            re[i] = dec_re(e);
            im[i] = dec_im(e);
          }
        }
      }
      s_er[pp][tt][dq] = static_cast<int32_t>(pack4(re[0], re[1], re[2], re[3]));
      s_ei[pp][tt][dq] = static_cast<int32_t>(pack4(im[0], im[1], im[2], im[3]));
    }
    // A[f][b][d] (Alinear, arraysizes.hxx:115) or A2 (arraysizes.hxx:125).
    for (int idx = tid; idx < kBB * kDQ; idx += kThreads) {
      const int bl = idx / kDQ, dq = idx % kDQ;
      const int64_t b = b0 + bl;
      int re[4] = {0, 0, 0, 0}, im[4] = {0, 0, 0, 0};
      if (b < B) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int64_t d = d0 + 4 * dq + i;
          if (d < D) load_a(A, a_layout, f, b, d, B, D, re[i], im[i]);
        }
      }
      s_ar[bl][dq] = static_cast<int32_t>(pack4(re[0], re[1], re[2], re[3]));
      s_ai[bl][dq] = static_cast<int32_t>(pack4(im[0], im[1], im[2], im[3]));
      s_nai[bl][dq] = static_cast<int32_t>(pack4(-im[0], -im[1], -im[2], -im[3]));
    }
    __syncthreads();
    if (row < rows) {
#pragma unroll 4
      for (int dq = 0; dq < kDQ; ++dq) {
        const int er = s_er[p][tl][dq];
        const int ei = s_ei[p][tl][dq];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          const int bl = bsub + 4 * k;
          const int ar = s_ar[bl][dq], ai = s_ai[bl][dq], nai = s_nai[bl][dq];
          // rawJre += Are*Ere - Aim*Eim ; rawJim += Are*Eim + Aim*Ere  (cpu.cxx:33-34)
          acc_re[k] = __dp4a(ar, er, acc_re[k]);
          acc_re[k] = __dp4a(nai, ei, acc_re[k]);
          acc_im[k] = __dp4a(ar, ei, acc_im[k]);
          acc_im[k] = __dp4a(ai, er, acc_im[k]);
        }
      }
    }
  }

  const int64_t t = t0 + tl;
  if (row < rows && t < T) {
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const int64_t b = b0 + bsub + 4 * k;
      if (b < B) {
        const float g = G[f * B + b];  // Glinear, arraysizes.hxx:136
        const int jre = requant(g, acc_re[k]);
        const int jim = requant(g, acc_im[k]);
        // ucomplex4(Jre, Jim) at Jlinear(b,f,p,t) (cpu.cxx:40-41, icomplex4.hxx:33) or J2linear(b,f,t,p)
        const int64_t at = j_layout == kJ2 ? ((b * F + f) * jpitch + t) * P + p : ((b * F + f) * P + p) * jpitch + t;
        J[at] = static_cast<uint8_t>((((static_cast<uint32_t>(jre) & 15u) << 4) | (static_cast<uint32_t>(jim) & 15u)) ^
                                     0x88u);
      }
    }
  }
}

// ---------------------------------------------------------------- Gauss form
constexpr int kGRows = 64;                 // (p, t) rows per block: 64 / P times
constexpr int kGBeams = 32;                // beams per block
constexpr int kGDC = 128;                  // dishes per shared-memory chunk
constexpr int kGDQ = kGDC / 4;             // packed words per row and chunk
constexpr int kGPitch = kGDQ + 4;          // row pitch in words: 16-byte rows, and
                                           // 8 consecutive rows cover all 32 banks
constexpr int kGRowLanes = 32;             // a warp's lanes take 32 consecutive rows
constexpr int kGRowsPerThread = kGRows / kGRowLanes;           // 2
constexpr int kGBeamLanes = kThreads / kGRowLanes;             // 8 warps
constexpr int kGBeamsPerThread = kGBeams / kGBeamLanes;        // 4
static_assert(kGRowsPerThread * kGRowLanes == kGRows && kGBeamsPerThread * kGBeamLanes == kGBeams, "tile");
static_assert((kGPitch * 4) % 16 == 0 && kGDQ % 4 == 0, "16-byte shared rows");

__device__ __forceinline__ void dp4a_x4(int &acc, const int4 &a, const int4 &b) {
  acc = __dp4a(a.x, b.x, acc);
  acc = __dp4a(a.y, b.y, acc);
  acc = __dp4a(a.z, b.z, acc);
  acc = __dp4a(a.w, b.w, acc);
}

// Four stored ucomplex4 bytes at once (SWAR).  A stored nibble u holds the
// value u - 8 (the byte is the two's-complement nibbles xor 0x88,
// icomplex4.hxx), so the planes are byte-wise differences.  Each byte lane
// works with a bias of 128: for v in [0, 127] and s in [0, 128],
// (v + 128 - s) never borrows from the next lane, and xor 128 turns it into
// the two's-complement byte of v - s.
__device__ __forceinline__ uint32_t lanes_sub(uint32_t v, uint32_t s) {
  return ((v | 0x80808080u) - s) ^ 0x80808080u;
}
struct Planes {
  uint32_t re, im, sum, diff;  // u_hi - 8, u_lo - 8, their sum, im - re
};
__device__ __forceinline__ Planes planes_of(uint32_t w) {
  const uint32_t hi = (w >> 4) & 0x0F0F0F0Fu, lo = w & 0x0F0F0F0Fu;
  return {lanes_sub(hi, 0x08080808u), lanes_sub(lo, 0x08080808u), lanes_sub(hi + lo, 0x10101010u),
          lanes_sub(lo, hi)};
}

__global__ void __launch_bounds__(kThreads) bf_form_beams_gauss(uint8_t *__restrict__ J, const uint8_t *__restrict__ E,
                                                                const uint8_t *__restrict__ A,
                                                                const float *__restrict__ G, int64_t T, int64_t F,
                                                                int64_t D, int64_t P, int64_t B, int64_t jpitch,
                                                                int a_layout, int j_layout) {
  // E planes Er, Ei, Er + Ei and A planes Ar, Ar + Ai, Ai - Ar, packed int8 x 4
  __shared__ __align__(16) int32_t s_e[3][kGRows][kGPitch];
  __shared__ __align__(16) int32_t s_a[3][kGBeams][kGPitch];

  const int TT = kGRows / static_cast<int>(P);  // times per block
  const int64_t t0 = static_cast<int64_t>(blockIdx.x) * TT;
  const int64_t f = blockIdx.y;
  const int64_t b0 = static_cast<int64_t>(blockIdx.z) * kGBeams;
  const int tid = threadIdx.x;
  const int rl = tid % kGRowLanes;  // rows rl, rl + 32
  const int bl = tid / kGRowLanes;  // beams bl, bl + 8, bl + 16, bl + 24

  int k1[kGRowsPerThread][kGBeamsPerThread], k2[kGRowsPerThread][kGBeamsPerThread],
      k3[kGRowsPerThread][kGBeamsPerThread];
#pragma unroll
  for (int i = 0; i < kGRowsPerThread; ++i)
#pragma unroll
    for (int j = 0; j < kGBeamsPerThread; ++j) k1[i][j] = k2[i][j] = k3[i][j] = 0;

  // 4-byte loads of whole dish quads where every quad is aligned and complete
  const bool e_words = D % 4 == 0 && (reinterpret_cast<uintptr_t>(E) & 3u) == 0;
  const bool a_words = a_layout == kALinear && D % 4 == 0 && (reinterpret_cast<uintptr_t>(A) & 3u) == 0;

  for (int64_t d0 = 0; d0 < D; d0 += kGDC) {
    __syncthreads();
    // E[t][f][d][p] (Elinear, arraysizes.hxx:80) -> the three E planes; rows
    // past T and dishes past D are zero, so they add nothing.
    if (e_words) {
      // one time and dish quad: P words, split into polarizations by a byte permute
      for (int idx = tid; idx < TT * kGDQ; idx += kThreads) {
        const int tl = idx / kGDQ, dq = idx % kGDQ;
        const int64_t t = t0 + tl;
        const int64_t d = d0 + 4 * dq;
        const bool in = t < T && d < D;
        uint32_t w0 = 0, w1 = 0;
        if (in) {
          const uint32_t *src = reinterpret_cast<const uint32_t *>(E + ((t * F + f) * D + d) * P);
          w0 = __ldg(src);
          if (P == 2) w1 = __ldg(src + 1);
        }
        for (int pp = 0; pp < P; ++pp) {
          const uint32_t x = P == 2 ? __byte_perm(w0, w1, pp ? 0x7531u : 0x6420u) : w0;
          const int row = pp * TT + tl;
          const Planes pl = planes_of(x);
          s_e[0][row][dq] = in ? static_cast<int32_t>(pl.re) : 0;
          s_e[1][row][dq] = in ? static_cast<int32_t>(pl.im) : 0;
          s_e[2][row][dq] = in ? static_cast<int32_t>(pl.sum) : 0;
        }
      }
    } else {
      for (int idx = tid; idx < kGRows * kGDQ; idx += kThreads) {
        const int row = idx / kGDQ, dq = idx % kGDQ;
        const int pp = row / TT;
        const int64_t t = t0 + row % TT;
        int re[4] = {0, 0, 0, 0}, im[4] = {0, 0, 0, 0};
        if (t < T) {
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const int64_t d = d0 + 4 * dq + i;
            if (d < D) {
              const uint32_t e = E[((t * F + f) * D + d) * P + pp];
              re[i] = dec_re(e);
              im[i] = dec_im(e);
            }
          }
        }
        s_e[0][row][dq] = static_cast<int32_t>(pack4(re[0], re[1], re[2], re[3]));
        s_e[1][row][dq] = static_cast<int32_t>(pack4(im[0], im[1], im[2], im[3]));
        s_e[2][row][dq] = static_cast<int32_t>(pack4(re[0] + im[0], re[1] + im[1], re[2] + im[2], re[3] + im[3]));
      }
    }
    // A[f][b][d] (Alinear, arraysizes.hxx:115) or A2 (arraysizes.hxx:125) -> the three A planes
    if (a_words) {
      for (int idx = tid; idx < kGBeams * kGDQ; idx += kThreads) {
        const int bb = idx / kGDQ, dq = idx % kGDQ;
        const int64_t b = b0 + bb;
        const int64_t d = d0 + 4 * dq;
        const bool in = b < B && d < D;
        const Planes pl = planes_of(in ? __ldg(reinterpret_cast<const uint32_t *>(A + (f * B + b) * D + d)) : 0u);
        s_a[0][bb][dq] = in ? static_cast<int32_t>(pl.re) : 0;
        s_a[1][bb][dq] = in ? static_cast<int32_t>(pl.sum) : 0;
        s_a[2][bb][dq] = in ? static_cast<int32_t>(pl.diff) : 0;
      }
    } else {
      for (int idx = tid; idx < kGBeams * kGDQ; idx += kThreads) {
        const int bb = idx / kGDQ, dq = idx % kGDQ;
        const int64_t b = b0 + bb;
        int re[4] = {0, 0, 0, 0}, im[4] = {0, 0, 0, 0};
        if (b < B) {
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const int64_t d = d0 + 4 * dq + i;
            if (d < D) load_a(A, a_layout, f, b, d, B, D, re[i], im[i]);
          }
        }
        s_a[0][bb][dq] = static_cast<int32_t>(pack4(re[0], re[1], re[2], re[3]));
        s_a[1][bb][dq] = static_cast<int32_t>(pack4(re[0] + im[0], re[1] + im[1], re[2] + im[2], re[3] + im[3]));
        s_a[2][bb][dq] = static_cast<int32_t>(pack4(im[0] - re[0], im[1] - re[1], im[2] - re[2], im[3] - re[3]));
      }
    }
    __syncthreads();
#pragma unroll 2
    for (int q = 0; q < kGDQ; q += 4) {
      int4 er[kGRowsPerThread], ei[kGRowsPerThread], es[kGRowsPerThread];
#pragma unroll
      for (int i = 0; i < kGRowsPerThread; ++i) {
        const int row = rl + kGRowLanes * i;
        er[i] = *reinterpret_cast<const int4 *>(&s_e[0][row][q]);
        ei[i] = *reinterpret_cast<const int4 *>(&s_e[1][row][q]);
        es[i] = *reinterpret_cast<const int4 *>(&s_e[2][row][q]);
      }
#pragma unroll
      for (int j = 0; j < kGBeamsPerThread; ++j) {
        const int bb = bl + kGBeamLanes * j;  // the same beam for the whole warp: broadcast loads
        const int4 ar = *reinterpret_cast<const int4 *>(&s_a[0][bb][q]);
        const int4 ap = *reinterpret_cast<const int4 *>(&s_a[1][bb][q]);
        const int4 am = *reinterpret_cast<const int4 *>(&s_a[2][bb][q]);
#pragma unroll
        for (int i = 0; i < kGRowsPerThread; ++i) {
          dp4a_x4(k1[i][j], ar, es[i]);  // Ar (Er + Ei)
          dp4a_x4(k2[i][j], ap, ei[i]);  // (Ar + Ai) Ei
          dp4a_x4(k3[i][j], am, er[i]);  // (Ai - Ar) Er
        }
      }
    }
  }

#pragma unroll
  for (int i = 0; i < kGRowsPerThread; ++i) {
    const int row = rl + kGRowLanes * i;
    const int64_t p = row / TT;
    const int64_t t = t0 + row % TT;
    if (t >= T) continue;
#pragma unroll
    for (int j = 0; j < kGBeamsPerThread; ++j) {
      const int64_t b = b0 + bl + kGBeamLanes * j;
      if (b >= B) continue;
      const float g = G[f * B + b];  // Glinear, arraysizes.hxx:136
      const int jre = requant(g, k1[i][j] - k2[i][j]);
      const int jim = requant(g, k1[i][j] + k3[i][j]);
      // ucomplex4(Jre, Jim) at Jlinear(b,f,p,t) (cpu.cxx:40-41, icomplex4.hxx:33) or J2linear(b,f,t,p);
      // a warp's lanes store 32 consecutive times of one beam
      const int64_t at = j_layout == kJ2 ? ((b * F + f) * jpitch + t) * P + p : ((b * F + f) * P + p) * jpitch + t;
      J[at] =
          static_cast<uint8_t>((((static_cast<uint32_t>(jre) & 15u) << 4) | (static_cast<uint32_t>(jim) & 15u)) ^ 0x88u);
    }
  }
}

}  // namespace

cudaError_t launch_simt(const bf_dims &d, uint8_t *J, const uint8_t *E, const uint8_t *A, const float *G,
                        cudaStream_t s, int64_t jpitch, int a_layout, int j_layout) {
  if (jpitch <= 0) jpitch = d.ntimes;
  if (d.npolarizations < 1 || d.npolarizations > 2) return cudaErrorInvalidValue;
  if (simt_four_multiply()) {
    const int64_t gx = (d.ntimes + kTT - 1) / kTT;
    const int64_t gz = (d.nbeams + kBB - 1) / kBB;
    if (gx > 0x7FFFFFFF || d.nfrequencies > 65535 || gz > 65535) return cudaErrorInvalidConfiguration;
    const dim3 grid(static_cast<unsigned>(gx), static_cast<unsigned>(d.nfrequencies), static_cast<unsigned>(gz));
    bf_form_beams_simt<<<grid, kThreads, 0, s>>>(J, E, A, G, d.ntimes, d.nfrequencies, d.ndishes, d.npolarizations,
                                                 d.nbeams, jpitch, a_layout, j_layout);
    return cudaGetLastError();
  }
  const int64_t tt = kGRows / d.npolarizations;
  const int64_t gx = (d.ntimes + tt - 1) / tt;
  const int64_t gz = (d.nbeams + kGBeams - 1) / kGBeams;
  if (gx > 0x7FFFFFFF || d.nfrequencies > 65535 || gz > 65535) return cudaErrorInvalidConfiguration;
  const dim3 grid(static_cast<unsigned>(gx), static_cast<unsigned>(d.nfrequencies), static_cast<unsigned>(gz));
  bf_form_beams_gauss<<<grid, kThreads, 0, s>>>(J, E, A, G, d.ntimes, d.nfrequencies, d.ndishes, d.npolarizations,
                                                d.nbeams, jpitch, a_layout, j_layout);
  return cudaGetLastError();
}

}  // namespace bf
