// bf_api.cu -- host side of the C ABI declared in include/beamform.h.
//
// Owns the per-device state (error word, staging and operand scratch), picks
// the kernel family, and implements the drop-in form_beams() of cpu.cxx:15-16
// on top of the explicit entry points.  No entry point exits the process or
// falls back to the CPU: a shape no GPU kernel takes returns
// BF_ERR_UNSUPPORTED.
#include "bf_internal.h"

#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

namespace bf {
namespace {

int to_status(cudaError_t e) {
  if (e == cudaSuccess) return BF_OK;
  if (e == cudaErrorMemoryAllocation) return BF_ERR_OUT_OF_MEMORY;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return BF_ERR_NO_DEVICE;
  return BF_ERR_CUDA;
}

#define BF_TRY(expr)                          \
  do {                                        \
    const cudaError_t e_ = (expr);            \
    if (e_ != cudaSuccess) return to_status(e_); \
  } while (0)

// Growable device buffer.
struct DevBuf {
  void *p = nullptr;
  size_t cap = 0;
  cudaError_t reserve(size_t n) {
    if (n <= cap) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    const cudaError_t e = cudaMalloc(&p, std::max<size_t>(n, 256));
    if (e == cudaSuccess) cap = std::max<size_t>(n, 256);
    return e;
  }
  template <class T>
  T *as() const {
    return static_cast<T *>(p);
  }
};

// One pipeline lane of the host-pointer path: a stream and the E chunk in flight on it.
struct Lane {
  cudaStream_t s = nullptr;
  cudaEvent_t done = nullptr;
  DevBuf E;
};

constexpr int kLanes = 3;

struct DeviceCtx {
  std::mutex mu;
  bool ready = false;
  bool lanes_ready = false;
  Lane lanes[kLanes];
  int *err = nullptr;       // device error word written by kernels
  uint32_t *adler = nullptr;  // device adler32 result
  DevBuf E, A, G, J;        // staging for host-pointer calls
  DevBuf W, dig;            // tensor-core operand for non-resident calls
  DevBuf partials;          // adler32 partial sums
  DevBuf adl;               // fused adler32 sums {sum d_i, sum i d_i} of the last checked call
};

constexpr int kMaxDevices = 64;
DeviceCtx g_ctx[kMaxDevices];

int current_ctx(DeviceCtx **out) {
  int dev = -1;
  const cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return to_status(e);
  if (dev < 0 || dev >= kMaxDevices) return BF_ERR_NO_DEVICE;
  DeviceCtx &c = g_ctx[dev];
  if (!c.ready) {
    std::lock_guard<std::mutex> lk(c.mu);
    if (!c.ready) {
      BF_TRY(cudaMalloc(&c.err, sizeof(int)));
      BF_TRY(cudaMemset(c.err, 0, sizeof(int)));
      BF_TRY(cudaMalloc(&c.adler, sizeof(uint32_t)));
      c.ready = true;
    }
  }
  *out = &c;
  return BF_OK;
}

std::mutex g_dims_mu;
bool g_dims_set = false;
bf_dims g_dims{};
std::atomic<int> g_kernel{BF_KERNEL_AUTO};
thread_local int t_last_status = BF_OK;
thread_local const char *t_last_kernel = "none";

const char *simt_name() { return g_kernel.load() == BF_KERNEL_SIMT4 ? "simt4" : "simt"; }

bool dims_valid(const bf_dims *d) {
  return d && d->ntimes >= 0 && d->nfrequencies >= 0 && d->ndishes >= 0 && d->npolarizations >= 0 &&
         d->nbeams >= 0;
}

size_t esize(const bf_dims &d) {
  return static_cast<size_t>(d.ntimes) * d.nfrequencies * d.ndishes * d.npolarizations;
}
size_t asize(const bf_dims &d) { return static_cast<size_t>(d.nfrequencies) * d.nbeams * d.ndishes; }
size_t gsize(const bf_dims &d) { return static_cast<size_t>(d.nfrequencies) * d.nbeams; }
size_t jsize(const bf_dims &d) {
  return static_cast<size_t>(d.nbeams) * d.nfrequencies * d.npolarizations * d.ntimes;
}

// Sizes the operand layout for F x B x D weights.
void plan_weights(TcWeights &w, int64_t F, int64_t B, int64_t D) {
  w.F = F;
  w.B = B;
  w.D = D;
  tc_plan_beams(B, &w.nb_pass, &w.npass);
  w.nw = static_cast<int>((B + 7) / 8 * 8 * 2);
  w.nw_pad = w.npass * 2 * w.nb_pass;
}

size_t weights_bytes(const TcWeights &w) { return static_cast<size_t>(w.F) * w.nw * 2 * w.D; }


int choose_tensor(const bf_dims &d, bool *use_tc) {
  const int k = g_kernel.load();
  const bool ok = tc_supported(d);
  if (k == BF_KERNEL_TENSOR && !ok) return BF_ERR_UNSUPPORTED;
  if ((k == BF_KERNEL_SIMT || k == BF_KERNEL_SIMT4) && (d.npolarizations < 1 || d.npolarizations > 2))
    return BF_ERR_UNSUPPORTED;
  if (k == BF_KERNEL_AUTO && !ok && (d.npolarizations < 1 || d.npolarizations > 2)) return BF_ERR_UNSUPPORTED;
  *use_tc = (k == BF_KERNEL_TENSOR) || (k == BF_KERNEL_AUTO && ok);
  return BF_OK;
}

// All four arrays on the device; the tensor-core operand goes to W / dig.
// With `adl` set (zeroed here), a tensor-core launch also sums J for its
// adler32 and *fused reports that it did; the SIMT kernel does not.
int run_device_bufs(const bf_dims &d, uint8_t *J, const uint8_t *E, const uint8_t *A, const float *G, DevBuf &W,
                    DevBuf &dig, int *err, cudaStream_t s, int a_layout = kALinear, int j_layout = kJLinear,
                    unsigned long long *adl = nullptr, bool *fused = nullptr);

// All four arrays on the device.  Operand scratch comes from ctx (caller holds ctx.mu).
int run_device(DeviceCtx &c, const bf_dims &d, uint8_t *J, const uint8_t *E, const uint8_t *A, const float *G,
               cudaStream_t s, int a_layout = kALinear, int j_layout = kJLinear, unsigned long long *adl = nullptr,
               bool *fused = nullptr) {
  return run_device_bufs(d, J, E, A, G, c.W, c.dig, c.err, s, a_layout, j_layout, adl, fused);
}

int run_device_bufs(const bf_dims &d, uint8_t *J, const uint8_t *E, const uint8_t *A, const float *G, DevBuf &Wb,
                    DevBuf &digb, int *err, cudaStream_t s, int a_layout, int j_layout, unsigned long long *adl,
                    bool *fused) {
  if (fused) *fused = false;
  if (jsize(d) == 0) return BF_OK;
  bool use_tc = false;
  const int st = choose_tensor(d, &use_tc);
  if (st != BF_OK) return st;
  if (use_tc && ((reinterpret_cast<uintptr_t>(E) | reinterpret_cast<uintptr_t>(J)) & 15u)) {
    if (g_kernel.load() == BF_KERNEL_TENSOR) return BF_ERR_UNSUPPORTED;
    use_tc = false;
  }
  if (!use_tc) {
    t_last_kernel = simt_name();
    return to_status(launch_simt(d, J, E, A, G, s, 0, a_layout, j_layout));
  }
  TcWeights w;
  plan_weights(w, d.nfrequencies, d.nbeams, d.ndishes);
  BF_TRY(Wb.reserve(weights_bytes(w)));
  BF_TRY(digb.reserve(tc_extra_bytes(w)));
  w.W = Wb.as<uint8_t>();
  tc_set_extra(w, digb.as<uint8_t>());
  w.G = G;
  BF_TRY(launch_prep_weights(w, A, s, a_layout));
  t_last_kernel = "tensor";
  if (adl) {
    BF_TRY(cudaMemsetAsync(adl, 0, 2 * sizeof(unsigned long long), s));
    if (fused) *fused = true;
  }
  return to_status(launch_tc(w, d.ntimes, J, E, err, s, 0, j_layout, adl, J));
}

int read_and_clear_err(DeviceCtx &c, cudaStream_t s) {
  int h = 0;
  BF_TRY(cudaMemcpyAsync(&h, c.err, sizeof(int), cudaMemcpyDeviceToHost, s));
  BF_TRY(cudaStreamSynchronize(s));
  if (h != 0) {
    BF_TRY(cudaMemsetAsync(c.err, 0, sizeof(int), s));
    BF_TRY(cudaStreamSynchronize(s));
    return BF_ERR_DEVICE_TIMEOUT;
  }
  return BF_OK;
}

// Times per pipeline chunk of the host-pointer path: about 256 MB of E per
// chunk (a multiple of 64 times), or all of T when that is one chunk anyway.
// BF_HOST_CHUNK_BYTES overrides the chunk size (tuning and tests).
int64_t chunk_times(const bf_dims &d) {
  const int64_t per_t = std::max<int64_t>(1, d.nfrequencies * d.ndishes * d.npolarizations);
  int64_t bytes = int64_t(256) << 20;
  if (const char *env = std::getenv("BF_HOST_CHUNK_BYTES")) bytes = std::max<int64_t>(1, std::atoll(env));
  int64_t tc = std::max<int64_t>(64, (bytes / per_t) / 64 * 64);
  return tc * 3 / 2 >= d.ntimes ? d.ntimes : tc;
}

int num_sms_api() {
  static const int n = [] {
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      v = 1;
    return v > 0 ? v : 1;
  }();
  return n;
}

// Copies bytes [off, off + len) of each of `rows` rows (`pitch` bytes apart)
// from the device J to the caller's J in pinned host memory (its device
// mapping): one 16-byte load and streaming store per step, so a warp writes
// whole 64-byte lines across the host link.  off, len, pitch and both base
// addresses are multiples of 16.
__global__ void __launch_bounds__(256) drain_rows(const uint8_t *__restrict__ src, uint8_t *__restrict__ dst,
                                                  int64_t rows, int64_t pitch, int64_t off, int64_t len) {
  const int64_t per_row = len / 16;
  const int64_t total = rows * per_row;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t r = i / per_row;
    const int64_t o = r * pitch + off + 16 * (i - r * per_row);
    __stcs(reinterpret_cast<uint4 *>(dst + o), __ldcs(reinterpret_cast<const uint4 *>(src + o)));
  }
}

// Device address of the caller's J when it is pinned host memory that the
// drain can write directly (16-byte aligned, rows a multiple of 16 bytes);
// null otherwise (pageable memory: one copy at the end instead).
uint8_t *mapped_host_j(uint8_t *J, const bf_dims &d, int j_layout) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, J) != cudaSuccess) {
    (void)cudaGetLastError();
    return nullptr;
  }
  const int64_t pitch = j_layout == kJ2 ? d.ntimes * d.npolarizations : d.ntimes;
  if (at.type != cudaMemoryTypeHost || !at.devicePointer || (pitch & 15) ||
      (reinterpret_cast<uintptr_t>(at.devicePointer) & 15))
    return nullptr;
  return static_cast<uint8_t *>(at.devicePointer);
}

// Host-pointer pass pipelined over time chunks: E[t0..t1][f][d][p] is
// contiguous, so each chunk goes in with one copy on one of kLanes streams and
// is beamformed while the next chunk copies; every chunk writes its times of J
// (rows of ntimes bytes) in a device buffer.  When the caller's J is pinned,
// a drain kernel behind each chunk writes the chunk's row segments straight
// into it, so J leaves over the link while later chunks of E arrive;
// otherwise J is copied out once at the end.
// A, G and the tensor-core operand are uploaded / prepared once.  Synchronous;
// the caller holds c.mu.
int run_host_pipelined(DeviceCtx &c, const bf_dims &d, uint8_t *J, const uint8_t *E, const uint8_t *A,
                       const float *G, cudaStream_t caller, int a_layout, int j_layout,
                       unsigned long long *adl = nullptr, bool *fused = nullptr) {
  if (fused) *fused = false;
  if (!c.lanes_ready) {
    for (Lane &l : c.lanes) {
      BF_TRY(cudaStreamCreateWithFlags(&l.s, cudaStreamNonBlocking));
      BF_TRY(cudaEventCreateWithFlags(&l.done, cudaEventDisableTiming));
    }
    c.lanes_ready = true;
  }
  bool use_tc = false;
  int st = choose_tensor(d, &use_tc);
  if (st != BF_OK) return st;
  const int64_t T = d.ntimes, per_t = d.nfrequencies * d.ndishes * d.npolarizations;
  const int64_t tc = chunk_times(d);
  BF_TRY(c.A.reserve(asize(d)));
  BF_TRY(c.G.reserve(gsize(d) * sizeof(float)));
  BF_TRY(c.J.reserve(jsize(d)));
  Lane &l0 = c.lanes[0];
  // work already queued on the caller's stream comes first
  BF_TRY(cudaEventRecord(l0.done, caller));
  BF_TRY(cudaStreamWaitEvent(l0.s, l0.done, 0));
  BF_TRY(cudaMemcpyAsync(c.A.p, A, asize(d), cudaMemcpyHostToDevice, l0.s));
  BF_TRY(cudaMemcpyAsync(c.G.p, G, gsize(d) * sizeof(float), cudaMemcpyHostToDevice, l0.s));
  TcWeights w;
  if (use_tc) {
    plan_weights(w, d.nfrequencies, d.nbeams, d.ndishes);
    BF_TRY(c.W.reserve(weights_bytes(w)));
    BF_TRY(c.dig.reserve(tc_extra_bytes(w)));
    w.W = c.W.as<uint8_t>();
    tc_set_extra(w, c.dig.as<uint8_t>());
    w.G = c.G.as<float>();
    BF_TRY(launch_prep_weights(w, c.A.as<uint8_t>(), l0.s, a_layout));
    if (adl) {  // every chunk's launch adds into the same sums, positions from the start of J
      BF_TRY(cudaMemsetAsync(adl, 0, 2 * sizeof(unsigned long long), l0.s));
      if (fused) *fused = true;
    }
  }
  BF_TRY(cudaEventRecord(l0.done, l0.s));
  for (int i = 1; i < kLanes; ++i) BF_TRY(cudaStreamWaitEvent(c.lanes[i].s, l0.done, 0));
  t_last_kernel = use_tc ? "tensor" : simt_name();
  uint8_t *jmap = mapped_host_j(J, d, j_layout);
  const int64_t P = d.npolarizations;
  const int64_t jrows = j_layout == kJ2 ? d.nbeams * d.nfrequencies : d.nbeams * d.nfrequencies * P;
  const int64_t jpitch = j_layout == kJ2 ? T * P : T;
  const int64_t jscale = j_layout == kJ2 ? P : 1;  // bytes per time in a row
  for (int64_t t0 = 0, k = 0; t0 < T; t0 += tc, ++k) {
    Lane &l = c.lanes[k % kLanes];
    const int64_t nt = std::min(tc, T - t0);
    BF_TRY(l.E.reserve(static_cast<size_t>(nt * per_t)));
    BF_TRY(cudaMemcpyAsync(l.E.p, E + t0 * per_t, static_cast<size_t>(nt * per_t), cudaMemcpyHostToDevice, l.s));
    // the chunk's first time: byte t0 of each J row, byte t0 * P of each J2 row
    uint8_t *Jc = c.J.as<uint8_t>() + (j_layout == kJ2 ? t0 * d.npolarizations : t0);
    if (use_tc) {
      BF_TRY(launch_tc(w, nt, Jc, l.E.as<uint8_t>(), c.err, l.s, T, j_layout, adl, c.J.as<uint8_t>()));
    } else {
      const bf_dims dc{nt, d.nfrequencies, d.ndishes, d.npolarizations, d.nbeams};
      BF_TRY(launch_simt(dc, Jc, l.E.as<uint8_t>(), c.A.as<uint8_t>(), c.G.as<float>(), l.s, T, a_layout, j_layout));
    }
    if (jmap) {
      const int grid = 2 * std::max(1, num_sms_api());
      drain_rows<<<grid, 256, 0, l.s>>>(c.J.as<uint8_t>(), jmap, jrows, jpitch, t0 * jscale, nt * jscale);
      BF_TRY(cudaGetLastError());
    }
  }
  for (int i = 1; i < kLanes; ++i) {
    BF_TRY(cudaEventRecord(c.lanes[i].done, c.lanes[i].s));
    BF_TRY(cudaStreamWaitEvent(l0.s, c.lanes[i].done, 0));
  }
  if (!jmap) BF_TRY(cudaMemcpyAsync(J, c.J.p, jsize(d), cudaMemcpyDeviceToHost, l0.s));
  BF_TRY(cudaStreamSynchronize(l0.s));
  return read_and_clear_err(c, caller);
}

}  // namespace

bool simt_four_multiply() { return g_kernel.load() == BF_KERNEL_SIMT4; }

int device_error_word(int **out) {
  DeviceCtx *c = nullptr;
  const int st = current_ctx(&c);
  if (st != BF_OK) return st;
  *out = c->err;
  return BF_OK;
}

}  // namespace bf

using namespace bf;

// form_beams over any pointer kind and layout; with adler_out set, also the
// adler32 of the J it wrote (synchronous then).
static int form_beams_impl(const bf_dims *dims, uint8_t *J, const uint8_t *E, const uint8_t *A, const float *G,
                           int a_layout, int j_layout, int ptr_kind, bf_stream_t stream, uint32_t *adler_out);

extern "C" {

int bf_set_dims(const bf_dims *dims) {
  if (!dims_valid(dims)) return BF_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(g_dims_mu);
  g_dims = *dims;
  g_dims_set = true;
  return BF_OK;
}

int bf_last_status(void) { return t_last_status; }

const char *bf_last_kernel(void) { return t_last_kernel; }

const char *bf_status_string(int status) {
  switch (status) {
    case BF_OK: return "ok";
    case BF_ERR_INVALID_ARGUMENT: return "invalid argument";
    case BF_ERR_UNSUPPORTED: return "shape or alignment not supported by any GPU kernel";
    case BF_ERR_NO_DEVICE: return "no usable CUDA device";
    case BF_ERR_CUDA: return "CUDA runtime error";
    case BF_ERR_OUT_OF_MEMORY: return "out of memory";
    case BF_ERR_DEVICE_TIMEOUT: return "a device-side wait expired; results are invalid";
    case BF_ERR_NOT_CONFIGURED: return "form_beams() called before bf_set_dims()";
    case BF_ERR_SIZE_MISMATCH: return "weights were built for a different shape";
    case BF_ERR_TOO_LARGE: return "problem exceeds the fixed scratch of bf_form_beams_noalloc";
    default: return "unknown status";
  }
}

int bf_set_kernel(int kernel) {
  if (kernel < BF_KERNEL_AUTO || kernel > BF_KERNEL_SIMT4) return BF_ERR_INVALID_ARGUMENT;
  g_kernel.store(kernel);
  return BF_OK;
}

int bf_set_test_stall(int on) {
  tc_set_test_stall(on);
  return BF_OK;
}

int bf_form_beams_ex(const bf_dims *dims, uint8_t *J, const uint8_t *E, const uint8_t *A, const float *G,
                     int ptr_kind, bf_stream_t stream) {
  return bf_form_beams_layout(dims, J, E, A, G, BF_A_LINEAR, BF_J_LINEAR, ptr_kind, stream);
}

int bf_form_beams_layout(const bf_dims *dims, uint8_t *J, const uint8_t *E, const uint8_t *A, const float *G,
                         int a_layout, int j_layout, int ptr_kind, bf_stream_t stream) {
  return form_beams_impl(dims, J, E, A, G, a_layout, j_layout, ptr_kind, stream, nullptr);
}

int bf_form_beams_adler(const bf_dims *dims, uint8_t *J, const uint8_t *E, const uint8_t *A, const float *G,
                        int a_layout, int j_layout, int ptr_kind, uint32_t *adler, bf_stream_t stream) {
  if (!adler) return BF_ERR_INVALID_ARGUMENT;
  return form_beams_impl(dims, J, E, A, G, a_layout, j_layout, ptr_kind, stream, adler);
}

}  // extern "C"

namespace bf {
namespace {

// The adler32 of the n bytes of device J after a checked call: from the fused
// sums when the tensor-core kernel ran, else by the separate two-kernel pass.
// Synchronises the stream.
int finish_adler(DeviceCtx &c, bool fused, const uint8_t *Jdev, size_t n, cudaStream_t s, uint32_t *out) {
  if (n == 0) {
    *out = 1u;
    return BF_OK;
  }
  if (fused) {
    unsigned long long h[2] = {0, 0};
    BF_TRY(cudaMemcpyAsync(h, c.adl.p, sizeof(h), cudaMemcpyDeviceToHost, s));
    BF_TRY(cudaStreamSynchronize(s));
    *out = adler_finish(h[0], h[1], n);
    return BF_OK;
  }
  BF_TRY(c.partials.reserve(static_cast<size_t>(adler_nchunks(n)) * 2 * sizeof(uint32_t)));
  BF_TRY(launch_adler_partials(Jdev, n, c.partials.as<uint32_t>(), s));
  BF_TRY(launch_adler_combine(c.partials.as<uint32_t>(), n, c.adler, s));
  uint32_t h = 0;
  BF_TRY(cudaMemcpyAsync(&h, c.adler, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  BF_TRY(cudaStreamSynchronize(s));
  *out = h;
  return BF_OK;
}

// After a failed synchronous host-pointer call: wait for what it had already
// queued (copies from the caller's E, drains into the caller's J) so that
// nothing touches the caller's buffers once the call has returned.
void settle_after_error(DeviceCtx &c, cudaStream_t s) {
  (void)cudaStreamSynchronize(s);
  if (c.lanes_ready)
    for (Lane &l : c.lanes) (void)cudaStreamSynchronize(l.s);
  (void)cudaGetLastError();
}

}  // namespace
}  // namespace bf

static int form_beams_impl(const bf_dims *dims, uint8_t *J, const uint8_t *E, const uint8_t *A, const float *G,
                           int a_layout, int j_layout, int ptr_kind, bf_stream_t stream, uint32_t *adler_out) {
  if (!dims_valid(dims)) return BF_ERR_INVALID_ARGUMENT;
  if ((a_layout != BF_A_LINEAR && a_layout != BF_A_A2) || (j_layout != BF_J_LINEAR && j_layout != BF_J_J2))
    return BF_ERR_INVALID_ARGUMENT;
  if (a_layout == BF_A_A2 && !a2_supported(dims->ndishes)) return BF_ERR_UNSUPPORTED;
  if (ptr_kind != BF_PTR_HOST && ptr_kind != BF_PTR_DEVICE) return BF_ERR_INVALID_ARGUMENT;
  const bf_dims d = *dims;
  if (jsize(d) == 0) {
    if (adler_out) *adler_out = 1u;  // adler32 of no bytes
    return BF_OK;
  }
  if (!J || (esize(d) && !E) || (asize(d) && !A) || !G) return BF_ERR_INVALID_ARGUMENT;
  DeviceCtx *c = nullptr;
  int st = current_ctx(&c);
  if (st != BF_OK) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  std::lock_guard<std::mutex> lk(c->mu);
  unsigned long long *adl = nullptr;
  if (adler_out) {
    BF_TRY(c->adl.reserve(2 * sizeof(unsigned long long)));
    adl = c->adl.as<unsigned long long>();
  }
  bool fused = false;
  if (ptr_kind == BF_PTR_DEVICE) {
    st = run_device(*c, d, J, E, A, G, s, a_layout, j_layout, adl, &fused);
    if (st != BF_OK || !adler_out) return st;
    st = finish_adler(*c, fused, J, jsize(d), s, adler_out);
    if (st != BF_OK) return st;
    return read_and_clear_err(*c, s);
  }

  // Host pointers: stage in, compute, stage out, synchronously (cuda.cu:274-314 does the same around its
  // kernel), pipelined over time chunks when there is more than one.
  const int hs = [&]() -> int {
    if (chunk_times(d) < d.ntimes) {
      const int ps = run_host_pipelined(*c, d, J, E, A, G, s, a_layout, j_layout, adl, &fused);
      if (ps != BF_OK || !adler_out) return ps;
      return finish_adler(*c, fused, c->J.as<uint8_t>(), jsize(d), s, adler_out);
    }
    BF_TRY(c->E.reserve(esize(d)));
    BF_TRY(c->A.reserve(asize(d)));
    BF_TRY(c->G.reserve(gsize(d) * sizeof(float)));
    BF_TRY(c->J.reserve(jsize(d)));
    BF_TRY(cudaMemcpyAsync(c->E.p, E, esize(d), cudaMemcpyHostToDevice, s));
    BF_TRY(cudaMemcpyAsync(c->A.p, A, asize(d), cudaMemcpyHostToDevice, s));
    BF_TRY(cudaMemcpyAsync(c->G.p, G, gsize(d) * sizeof(float), cudaMemcpyHostToDevice, s));
    const int rs = run_device(*c, d, c->J.as<uint8_t>(), c->E.as<uint8_t>(), c->A.as<uint8_t>(), c->G.as<float>(),
                              s, a_layout, j_layout, adl, &fused);
    if (rs != BF_OK) return rs;
    BF_TRY(cudaMemcpyAsync(J, c->J.p, jsize(d), cudaMemcpyDeviceToHost, s));
    if (adler_out) {
      const int as = finish_adler(*c, fused, c->J.as<uint8_t>(), jsize(d), s, adler_out);
      if (as != BF_OK) return as;
    }
    return read_and_clear_err(*c, s);
  }();
  if (hs != BF_OK) settle_after_error(*c, s);
  return hs;
}

extern "C" {

void form_beams(uint8_t *J, const uint8_t *E, const uint8_t *A, const float *G) {
  bf_dims d;
  {
    std::lock_guard<std::mutex> lk(g_dims_mu);
    if (!g_dims_set) {
      t_last_status = BF_ERR_NOT_CONFIGURED;
      return;
    }
    d = g_dims;
  }
  t_last_status = bf_form_beams_ex(&d, J, E, A, G, BF_PTR_HOST, nullptr);
}

int bf_stream_status(bf_stream_t stream) {
  DeviceCtx *c = nullptr;
  const int st = current_ctx(&c);
  if (st != BF_OK) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return to_status(e);
  return read_and_clear_err(*c, s);
}

int bf_weights_create(bf_weights **out, int64_t nfrequencies, int64_t nbeams, int64_t ndishes, const uint8_t *A,
                      const float *G, int ptr_kind, bf_stream_t stream) {
  if (!out || nfrequencies <= 0 || nbeams <= 0 || ndishes <= 0 || !A || !G) return BF_ERR_INVALID_ARGUMENT;
  if (ptr_kind != BF_PTR_HOST && ptr_kind != BF_PTR_DEVICE) return BF_ERR_INVALID_ARGUMENT;
  DeviceCtx *c = nullptr;
  int st = current_ctx(&c);
  if (st != BF_OK) return st;
  bf_weights *w = new bf_weights();
  cudaGetDevice(&w->device);
  plan_weights(w->tc, nfrequencies, nbeams, ndishes);
  const size_t na = static_cast<size_t>(nfrequencies) * nbeams * ndishes;
  const size_t ng = static_cast<size_t>(nfrequencies) * nbeams;
  cudaError_t e = cudaMalloc(&w->A, na);
  if (e == cudaSuccess) e = cudaMalloc(&w->G, ng * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&w->tc.W, weights_bytes(w->tc));
  uint8_t *extra = nullptr;
  if (e == cudaSuccess) e = cudaMalloc(&extra, tc_extra_bytes(w->tc));
  if (e == cudaSuccess) tc_set_extra(w->tc, extra);
  if (e != cudaSuccess) {
    bf_weights_destroy(w);
    return to_status(e);
  }
  w->tc.G = w->G;
  st = bf_weights_update(w, A, G, ptr_kind, stream);
  if (st != BF_OK) {
    bf_weights_destroy(w);
    return st;
  }
  *out = w;
  return BF_OK;
}

int bf_weights_update(bf_weights *w, const uint8_t *A, const float *G, int ptr_kind, bf_stream_t stream) {
  if (!w || !A || !G) return BF_ERR_INVALID_ARGUMENT;
  if (ptr_kind != BF_PTR_HOST && ptr_kind != BF_PTR_DEVICE) return BF_ERR_INVALID_ARGUMENT;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t na = static_cast<size_t>(w->tc.F) * w->tc.B * w->tc.D;
  const size_t ng = static_cast<size_t>(w->tc.F) * w->tc.B;
  const cudaMemcpyKind k = ptr_kind == BF_PTR_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
  BF_TRY(cudaMemcpyAsync(w->A, A, na, k, s));
  BF_TRY(cudaMemcpyAsync(w->G, G, ng * sizeof(float), k, s));
  BF_TRY(launch_prep_weights(w->tc, w->A, s));
  if (ptr_kind == BF_PTR_HOST) BF_TRY(cudaStreamSynchronize(s));
  return BF_OK;
}

int bf_weights_destroy(bf_weights *w) {
  if (!w) return BF_OK;
  if (w->A) cudaFree(w->A);
  if (w->G) cudaFree(w->G);
  if (w->tc.W) cudaFree(w->tc.W);
  if (w->tc.dig) cudaFree(w->tc.dig);
  delete w;
  return BF_OK;
}

int bf_form_beams_resident(const bf_weights *w, int64_t ntimes, uint8_t *J, const uint8_t *E, bf_stream_t stream) {
  if (!w || ntimes < 0 || (ntimes > 0 && (!J || !E))) return BF_ERR_INVALID_ARGUMENT;
  if (ntimes == 0) return BF_OK;
  DeviceCtx *c = nullptr;
  const int st = current_ctx(&c);
  if (st != BF_OK) return st;
  const bf_dims d{ntimes, w->tc.F, w->tc.D, 2, w->tc.B};
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  bool use_tc = false;
  const int cs = choose_tensor(d, &use_tc);
  if (cs != BF_OK) return cs;
  if (use_tc && ((reinterpret_cast<uintptr_t>(E) | reinterpret_cast<uintptr_t>(J)) & 15u)) {
    if (g_kernel.load() == BF_KERNEL_TENSOR) return BF_ERR_UNSUPPORTED;
    use_tc = false;
  }
  if (use_tc) {
    t_last_kernel = "tensor";
    return to_status(launch_tc(w->tc, ntimes, J, E, c->err, s));
  }
  t_last_kernel = simt_name();
  return to_status(launch_simt(d, J, E, w->A, w->G, s));
}

int bf_adler32_device(const uint8_t *data, size_t len, uint32_t *out, bf_stream_t stream) {
  if (!out || (len && !data)) return BF_ERR_INVALID_ARGUMENT;
  if (len == 0) {
    *out = 1u;
    return BF_OK;
  }
  DeviceCtx *c = nullptr;
  const int st = current_ctx(&c);
  if (st != BF_OK) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  std::lock_guard<std::mutex> lk(c->mu);
  BF_TRY(c->partials.reserve(static_cast<size_t>(adler_nchunks(len)) * 2 * sizeof(uint32_t)));
  BF_TRY(launch_adler_partials(data, len, c->partials.as<uint32_t>(), s));
  BF_TRY(launch_adler_combine(c->partials.as<uint32_t>(), len, c->adler, s));
  uint32_t h = 0;
  BF_TRY(cudaMemcpyAsync(&h, c->adler, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  BF_TRY(cudaStreamSynchronize(s));
  *out = h;
  return BF_OK;
}

int bf_fill_random_device(uint8_t *dst, size_t n, uint64_t seed, uint64_t stream_id, bf_stream_t stream) {
  if (n && !dst) return BF_ERR_INVALID_ARGUMENT;
  return to_status(launch_fill_random(dst, n, seed, stream_id, static_cast<cudaStream_t>(stream)));
}

int bf_fill_random_host(uint8_t *dst, size_t n, uint64_t seed, uint64_t stream_id) {
  if (n && !dst) return BF_ERR_INVALID_ARGUMENT;
  auto mix64 = [](uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  };
  const uint64_t key = mix64(seed * 2u + stream_id + 1u);
  const size_t nwords = (n + 7) / 8;
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const size_t per = (nwords + hw - 1) / hw;
  std::vector<std::thread> th;
  for (unsigned i = 0; i < hw; ++i) {
    const size_t j0 = i * per, j1 = std::min(nwords, j0 + per);
    if (j0 >= j1) break;
    th.emplace_back([=]() {
      for (size_t j = j0; j < j1; ++j) {
        const uint64_t w = mix64(key + static_cast<uint64_t>(j + 1) * 0x9E3779B97F4A7C15ull);
        if (8 * j + 8 <= n) {
          uint8_t b[8];
          for (int k = 0; k < 8; ++k) b[k] = static_cast<uint8_t>(w >> (8 * k));
          std::memcpy(dst + 8 * j, b, 8);
        } else {
          for (size_t k = 0; 8 * j + k < n; ++k) dst[8 * j + k] = static_cast<uint8_t>(w >> (8 * k));
        }
      }
    });
  }
  for (auto &t : th) t.join();
  return BF_OK;
}

int bf_gains_host(const bf_dims *dims, float *G) {
  if (!dims_valid(dims) || !G) return BF_ERR_INVALID_ARGUMENT;
  // arraysizes.cxx:31-32: float(n) / Gsize / ndishes * (15 + n % 15) / 30, left to right in float
  const int64_t gs = dims->nfrequencies * dims->nbeams;
  const float fg = static_cast<float>(static_cast<uint64_t>(gs));
  const float fd = static_cast<float>(static_cast<uint64_t>(dims->ndishes));
  for (int64_t n = 0; n < gs; ++n) {
    float g = static_cast<float>(static_cast<uint64_t>(n));
    g = g / fg;
    g = g / fd;
    g = g * static_cast<float>(static_cast<uint64_t>(15 + n % 15));
    g = g / 30.0f;
    G[n] = g;
  }
  return BF_OK;
}

}  // extern "C"
