// bf_noalloc.cu -- bf_form_beams_noalloc(): the tensor-core beamformer for
// callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc: a real-time correlator/beamformer
// pipeline that sizes all of its device memory once at start-up and must not
// allocate afterwards (an allocation can block or fail mid-stream), or a host
// framework that owns the device memory pool and forbids other allocators.
// The regular entry points keep their scratch (the prepared E4M3 operand W,
// the digit rows of its row sums and the device error word) in buffers the library allocates on
// first use.  This entry point keeps that scratch in one fixed array in
// device memory instead, reserved when the library is loaded:
//
//   g_noalloc_scratch   kNoAllocScratchBytes = 4 MiB, 256-byte aligned
//     [0, 256)                    device error word (cleared every call)
//     [256, 256 + extra bytes)    dig[f][n][32] E4M3, F * npass * 2 * nb_pass * 32, then
//                                 512 * G[f][b] floats, F * npass * nb_pass, then
//                                 one wide-gain flag (int) per frequency
//     [.., .. + W bytes)          W[f][n][k]   E4M3,  F * 2 * roundup(B, 8) * 2 * D
//
// Every GPU that loads the library holds these 4 MiB until the process exits.
// The caller passes E, A, G and J in device memory, as for
// bf_form_beams_ex(..., BF_PTR_DEVICE, ...).  No cudaMalloc, cudaFree or other
// allocating call is made.
#include "bf_internal.h"

#include <mutex>

namespace bf {
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(4) << 20;
constexpr size_t kErrBytes = 256;

// Scratch for bf_form_beams_noalloc.  In host code this name is only a
// host-side stand-in for the device array, never a device address: the
// address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) uint8_t g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
void *g_scratch_addr[kMaxDevices] = {};

// Set-up, once per device, with that device current: the device address of
// the scratch array.
cudaError_t scratch_address(int dev, void **out) {
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (!g_scratch_addr[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return cudaSuccess;
}

size_t round256(size_t n) { return (n + 255) / 256 * 256; }

int status_of(cudaError_t e) {
  if (e == cudaSuccess) return BF_OK;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return BF_ERR_NO_DEVICE;
  return BF_ERR_CUDA;
}

}  // namespace
}  // namespace bf

using namespace bf;

extern "C" int bf_form_beams_noalloc(const bf_dims *dims, uint8_t *J, const uint8_t *E, const uint8_t *A,
                                     const float *G, bf_stream_t stream) {
  if (!dims || dims->ntimes < 0 || dims->nfrequencies < 0 || dims->ndishes < 0 || dims->npolarizations < 0 ||
      dims->nbeams < 0)
    return BF_ERR_INVALID_ARGUMENT;
  const bf_dims d = *dims;
  if (d.ntimes == 0 || d.nfrequencies == 0 || d.nbeams == 0 || d.npolarizations == 0) return BF_OK;
  if (!J || !E || !A || !G) return BF_ERR_INVALID_ARGUMENT;
  if (!tc_supported(d) || ((reinterpret_cast<uintptr_t>(E) | reinterpret_cast<uintptr_t>(J)) & 15u))
    return BF_ERR_UNSUPPORTED;

  // Operand layout and the bytes it needs; reject what does not fit the array.
  TcWeights w;
  w.F = d.nfrequencies;
  w.B = d.nbeams;
  w.D = d.ndishes;
  tc_plan_beams(d.nbeams, &w.nb_pass, &w.npass);
  w.nw = static_cast<int>((d.nbeams + 7) / 8 * 8 * 2);
  w.nw_pad = w.npass * 2 * w.nb_pass;
  const size_t dig_bytes = tc_extra_bytes(w);
  const size_t w_bytes = static_cast<size_t>(w.F) * w.nw * 2 * w.D;
  if (kErrBytes + round256(dig_bytes) + w_bytes > kNoAllocScratchBytes) return BF_ERR_TOO_LARGE;

  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return status_of(e);
  if (dev < 0 || dev >= kMaxDevices) return BF_ERR_NO_DEVICE;
  void *base = nullptr;
  e = scratch_address(dev, &base);
  if (e != cudaSuccess) return status_of(e);
  uint8_t *scratch = static_cast<uint8_t *>(base);
  int *err = reinterpret_cast<int *>(scratch);
  tc_set_extra(w, scratch + kErrBytes);
  w.W = scratch + kErrBytes + round256(dig_bytes);
  w.G = G;

  // The array keeps the previous call's contents: the error word must start at
  // zero; W and the digit rows are rewritten in full below.
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  e = cudaMemsetAsync(err, 0, sizeof(int), s);
  if (e == cudaSuccess) e = launch_prep_weights(w, A, s);
  if (e == cudaSuccess) e = launch_tc(w, d.ntimes, J, E, err, s);
  int h = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return status_of(e);
  return h != 0 ? BF_ERR_DEVICE_TIMEOUT : BF_OK;
}
