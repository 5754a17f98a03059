// bf_peak.cu -- the dense E4M3 tensor-core rate and the CUDA-core dp4a rate
// of this GPU, measured.
//
// The roofline of the beamformer's tensor-core kernel is the rate at which
// the SMs retire `tcgen05.mma.kind::f8f6f4` with the A operand in tensor
// memory -- the instruction the kernel issues.  This stream keeps every SM's
// tensor core busy with back-to-back M=128 N=256 K=32 MMAs (one elected
// thread per CTA, one CTA per SM) and is timed with CUDA events, so the
// figure holds at the clocks of the run that measures it.
#include "bf_internal.h"
#include "bf_ptx.cuh"

namespace bf {
namespace {

constexpr int kPeakM = 128, kPeakN = 256, kPeakK = 32;
// B tile (256 rows x 128 B, 128B swizzle) + alignment + barrier; sized above
// half the SM's shared memory so that no two CTAs share an SM (and its TMEM)
constexpr int kPeakSmem = 128 * 1024;

__global__ void __launch_bounds__(128, 1) bf_tensor_peak_kernel(int reps, int *err) {
  extern __shared__ uint8_t smem_dyn[];
  uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_dyn) + 1023) & ~uintptr_t(1023));
  uint8_t *sB = smem;
  const uint32_t bar = smem_u32(smem + kPeakN * 128);
  uint32_t *holder = reinterpret_cast<uint32_t *>(smem + kPeakN * 128 + 8);
  // operand values do not change the rate; any finite E4M3 bytes do
  for (int i = threadIdx.x; i < kPeakN * 128 / 4; i += blockDim.x) reinterpret_cast<uint32_t *>(sB)[i] = 0x38383838u;
  fence_proxy_async_smem();
  const int warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    fence_barrier_init();
  }
  if (warp == 0) {
    tmem_alloc(smem_u32(holder), 512);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *holder;
  {
    uint32_t r[32];
#pragma unroll
    for (int i = 0; i < 32; ++i) r[i] = 0x0C0C0C0Cu;
    tmem_st_32x32b_x32(tmem + ((32u * warp) << 16) + 256, r);  // A operand: columns 256..287
    tmem_st_wait();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (threadIdx.x == 0) {
    const uint32_t idesc = idesc_e4m3_f32(kPeakM, kPeakN);
    const uint64_t b0 = smem_desc_sw128(smem_u32(sB));
    for (int i = 0; i < reps; ++i) {
      const uint32_t kk = static_cast<uint32_t>(i) & 3u;
      mma_f8f6f4_ts(tmem, tmem + 256 + 8 * kk, b0 + ((32u * kk) >> 4), idesc, i != 0 ? 1u : 0u);
    }
    mma_commit(bar);
    mbar_wait(bar, 0, err, kDevTimeoutAccFull);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, 512);
  }
}

// The CUDA-core dp4a rate, the instruction of the exact kernel: every thread
// runs kDpChains independent dp4a chains (enough to cover the pipe latency)
// with per-chain operands that change every step, and stores one word so
// that nothing is eliminated.
constexpr int kDpChains = 16;  // loop overhead about 1 instruction in 16
constexpr int kDpThreads = 256;
constexpr int kDpBlocksPerSm = 8;

__global__ void __launch_bounds__(kDpThreads) bf_dp4a_peak_kernel(int reps, uint32_t *out) {
  int a[kDpChains], acc[kDpChains];
#pragma unroll
  for (int j = 0; j < kDpChains; ++j) {
    a[j] = static_cast<int>((0x01020304u ^ threadIdx.x) + 0x01010101u * j);
    acc[j] = j;
  }
  int b = static_cast<int>(0x05060708u + blockIdx.x);
  for (int i = 0; i < reps; ++i) {
#pragma unroll
    for (int j = 0; j < kDpChains; ++j) acc[j] = __dp4a(a[j], b, acc[j]);
    b ^= i;
  }
  uint32_t x = 0;
#pragma unroll
  for (int j = 0; j < kDpChains; ++j) x ^= static_cast<uint32_t>(acc[j]);
  out[static_cast<size_t>(blockIdx.x) * kDpThreads + threadIdx.x] = x;
}

}  // namespace
}  // namespace bf

using namespace bf;

extern "C" int bf_dp4a_peak(double *dp4a_per_s, bf_stream_t stream) {
  if (!dp4a_per_s) return BF_ERR_INVALID_ARGUMENT;
  *dp4a_per_s = 0.0;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
    return BF_ERR_NO_DEVICE;
  const int blocks = sms * kDpBlocksPerSm;
  uint32_t *out = nullptr;
  if (cudaMalloc(&out, sizeof(uint32_t) * static_cast<size_t>(blocks) * kDpThreads) != cudaSuccess)
    return BF_ERR_OUT_OF_MEMORY;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int reps = 1 << 13;  // about 1-2 ms per launch
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int st = BF_OK;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) st = BF_ERR_CUDA;
  float best = -1.0f;
  for (int rep = 0; rep < 6 && st == BF_OK; ++rep) {
    cudaEventRecord(e0, s);
    bf_dp4a_peak_kernel<<<blocks, kDpThreads, 0, s>>>(reps, out);
    cudaEventRecord(e1, s);
    if (cudaGetLastError() != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) {
      st = BF_ERR_CUDA;
      break;
    }
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && (best < 0.0f || ms < best)) best = ms;  // the first launch warms up
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(out);
  if (st != BF_OK) return st;
  *dp4a_per_s = static_cast<double>(blocks) * kDpThreads * reps * kDpChains / (best * 1e-3);
  return BF_OK;
}

extern "C" int bf_tensor_peak(double *tflops, bf_stream_t stream) {
  if (!tflops) return BF_ERR_INVALID_ARGUMENT;
  *tflops = 0.0;
  int *err = nullptr;
  int st = device_error_word(&err);
  if (st != BF_OK) return st;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return BF_ERR_NO_DEVICE;
  if (cudaFuncSetAttribute(bf_tensor_peak_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kPeakSmem) !=
      cudaSuccess)
    return BF_ERR_CUDA;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int reps = 1 << 15;  // about 2 ms per launch
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) return BF_ERR_CUDA;
  float best = -1.0f;
  for (int rep = 0; rep < 6 && st == BF_OK; ++rep) {
    cudaEventRecord(e0, s);
    bf_tensor_peak_kernel<<<sms, 128, kPeakSmem, s>>>(reps, err);
    cudaEventRecord(e1, s);
    if (cudaGetLastError() != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) {
      st = BF_ERR_CUDA;
      break;
    }
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && (best < 0.0f || ms < best)) best = ms;  // the first launch warms up
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st != BF_OK) return st;
  int h = 0;
  if (cudaMemcpy(&h, err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return BF_ERR_CUDA;
  if (h != 0) {
    cudaMemset(err, 0, sizeof(int));
    return BF_ERR_DEVICE_TIMEOUT;
  }
  const double flops = 2.0 * kPeakM * kPeakN * kPeakK * static_cast<double>(reps) * sms;
  *tflops = flops / (best * 1e-3) / 1e12;
  return BF_OK;
}
