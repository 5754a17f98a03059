// bf_adler.cu -- adler32 on the GPU, and the seeded workload generator.
//
// adler32 (adler32.c:7-20) over n bytes x_0..x_{n-1} is
//   a = 1 + sum_i x_i               (mod 65521)
//   b = n + sum_i (n - i) * x_i     (mod 65521)
// which is linear in the bytes, so each chunk c = [s, s+L) contributes
//   S1_c = sum x_i  and  (n - s) * S1_c - sum (i - s) * x_i
// to a and b.  A first kernel reduces every 64 KiB chunk to (S1, sum (i-s) x_i)
// mod 65521; a one-block kernel combines them.
#include "bf_internal.h"

#include <algorithm>

namespace bf {
namespace {

constexpr uint32_t kMod = 65521u;
constexpr int kChunk = 65536;
constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads) adler_partials(const uint8_t *__restrict__ data, size_t len,
                                                           uint32_t *__restrict__ partials) {
  const size_t s = static_cast<size_t>(blockIdx.x) * kChunk;
  const size_t L = min(static_cast<size_t>(kChunk), len - s);
  uint64_t s1 = 0, sw = 0;
  const bool aligned = (reinterpret_cast<uintptr_t>(data) & 15u) == 0;
  if (aligned && L == kChunk) {
    const uint4 *v = reinterpret_cast<const uint4 *>(data + s);
#pragma unroll 4
    for (int k = 0; k < kChunk / 16 / kThreads; ++k) {
      const int vi = threadIdx.x + k * kThreads;
      const uint4 q = __ldcs(v + vi);
      const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const uint32_t pos = static_cast<uint32_t>(16 * vi + 4 * j);
        const uint32_t sum = __dp4a(w[j], 0x01010101u, 0u);   // x0 + x1 + x2 + x3
        const uint32_t wsum = __dp4a(w[j], 0x03020100u, 0u);  // 0*x0 + 1*x1 + 2*x2 + 3*x3
        s1 += sum;
        sw += static_cast<uint64_t>(pos) * sum + wsum;
      }
    }
  } else {
    for (size_t i = threadIdx.x; i < L; i += kThreads) {
      const uint32_t x = data[s + i];
      s1 += x;
      sw += static_cast<uint64_t>(i) * x;
    }
  }
  // block reduction
  __shared__ uint64_t r1[kThreads / 32], rw[kThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    s1 += __shfl_down_sync(0xffffffffu, s1, o);
    sw += __shfl_down_sync(0xffffffffu, sw, o);
  }
  if ((threadIdx.x & 31) == 0) {
    r1[threadIdx.x / 32] = s1;
    rw[threadIdx.x / 32] = sw;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint64_t a = 0, b = 0;
    for (int i = 0; i < kThreads / 32; ++i) {
      a += r1[i];
      b += rw[i];
    }
    partials[2 * blockIdx.x] = static_cast<uint32_t>(a % kMod);
    partials[2 * blockIdx.x + 1] = static_cast<uint32_t>(b % kMod);
  }
}

__global__ void __launch_bounds__(1024) adler_combine(const uint32_t *__restrict__ partials, size_t len, int nchunks,
                                                      uint32_t *__restrict__ out) {
  uint64_t a = 0, b = 0;
  for (int c = threadIdx.x; c < nchunks; c += blockDim.x) {
    const uint64_t s1 = partials[2 * c], sw = partials[2 * c + 1];
    const uint64_t rest = (len - static_cast<size_t>(c) * kChunk) % kMod;  // (n - s) mod M
    a += s1;
    b += (rest * s1 + (kMod - sw)) % kMod;
  }
  a %= kMod;
  b %= kMod;
  __shared__ uint64_t ra[32], rb[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  if ((threadIdx.x & 31) == 0) {
    ra[threadIdx.x / 32] = a;
    rb[threadIdx.x / 32] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint64_t A = 1, Bv = len % kMod;
    for (int i = 0; i < static_cast<int>(blockDim.x / 32); ++i) {
      A += ra[i];
      Bv += rb[i];
    }
    A %= kMod;
    Bv %= kMod;
    *out = static_cast<uint32_t>((Bv << 16) | A);
  }
}

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__global__ void fill_random_kernel(uint8_t *__restrict__ dst, size_t n, uint64_t key) {
  const size_t nwords = (n + 7) / 8;
  const bool aligned = (reinterpret_cast<uintptr_t>(dst) & 7u) == 0;
  for (size_t j = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; j < nwords;
       j += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const uint64_t w = mix64(key + static_cast<uint64_t>(j + 1) * 0x9E3779B97F4A7C15ull);
    if (aligned && 8 * j + 8 <= n) {
      reinterpret_cast<uint64_t *>(dst)[j] = w;
    } else {
      for (size_t k = 0; k < 8 && 8 * j + k < n; ++k) dst[8 * j + k] = static_cast<uint8_t>(w >> (8 * k));
    }
  }
}

}  // namespace

int adler_nchunks(size_t len) { return static_cast<int>((len + kChunk - 1) / kChunk); }

cudaError_t launch_adler_partials(const uint8_t *data, size_t len, uint32_t *partials, cudaStream_t s) {
  const int n = adler_nchunks(len);
  if (n == 0) return cudaSuccess;
  adler_partials<<<n, kThreads, 0, s>>>(data, len, partials);
  return cudaGetLastError();
}

cudaError_t launch_adler_combine(const uint32_t *partials, size_t len, uint32_t *out, cudaStream_t s) {
  adler_combine<<<1, 1024, 0, s>>>(partials, len, adler_nchunks(len), out);
  return cudaGetLastError();
}

cudaError_t launch_fill_random(uint8_t *dst, size_t n, uint64_t seed, uint64_t stream_id, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  uint64_t z = seed * 2u + stream_id + 1u;  // key = mix64(seed * 2 + stream + 1), computed on the host
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  const uint64_t key = z ^ (z >> 31);
  const size_t nwords = (n + 7) / 8;
  const int blocks = static_cast<int>(std::min<size_t>((nwords + 255) / 256, 152 * 16));
  fill_random_kernel<<<blocks, 256, 0, s>>>(dst, n, key);
  return cudaGetLastError();
}

uint32_t adler32_host(const uint8_t *p, size_t n) {
  uint32_t a = 1, b = 0;
  while (n > 0) {
    // 5552 bytes is the longest run whose sums cannot overflow 32 bits
    // before the reduction (255 n (n + 1) / 2 + (n + 1) (65521 - 1) < 2^32)
    size_t k = n < 5552 ? n : 5552;
    n -= k;
    for (; k >= 8; k -= 8, p += 8) {
      a += p[0]; b += a; a += p[1]; b += a; a += p[2]; b += a; a += p[3]; b += a;
      a += p[4]; b += a; a += p[5]; b += a; a += p[6]; b += a; a += p[7]; b += a;
    }
    for (; k > 0; --k) {
      a += *p++;
      b += a;
    }
    a %= kAdlerMod;
    b %= kAdlerMod;
  }
  return (b << 16) | a;
}

}  // namespace bf

extern "C" int bf_adler32_host(const uint8_t *data, size_t len, uint32_t *out) {
  if (!out || (len && !data)) return BF_ERR_INVALID_ARGUMENT;
  *out = bf::adler32_host(data, len);
  return BF_OK;
}
