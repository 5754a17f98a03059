// bf_simt.cu -- exact integer beamformer on the CUDA cores (dp4a).
//
// Handles every shape (any ntimes, ndishes, nbeams; 1 or 2 polarizations).
// It is the fallback for shapes the tensor-core kernel does not take and an
// independent second GPU implementation for the parity tests.  Same
// arithmetic as cpu.cxx:24-41: int32 sums of 4-bit products, then
// clamp(lrint(G * float(raw)), -7, 7).
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

}  // namespace

cudaError_t launch_simt(const bf_dims &d, uint8_t *J, const uint8_t *E, const uint8_t *A, const float *G,
                        cudaStream_t s, int64_t jpitch, int a_layout, int j_layout) {
  if (jpitch <= 0) jpitch = d.ntimes;
  if (d.npolarizations < 1 || d.npolarizations > 2) return cudaErrorInvalidValue;
  const int64_t gx = (d.ntimes + kTT - 1) / kTT;
  const int64_t gz = (d.nbeams + kBB - 1) / kBB;
  if (gx > 0x7FFFFFFF || d.nfrequencies > 65535 || gz > 65535) return cudaErrorInvalidConfiguration;
  const dim3 grid(static_cast<unsigned>(gx), static_cast<unsigned>(d.nfrequencies), static_cast<unsigned>(gz));
  bf_form_beams_simt<<<grid, kThreads, 0, s>>>(J, E, A, G, d.ntimes, d.nfrequencies, d.ndishes, d.npolarizations,
                                               d.nbeams, jpitch, a_layout, j_layout);
  return cudaGetLastError();
}

}  // namespace bf
