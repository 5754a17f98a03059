// bf_server.cu -- a served stream of voltage chunks with continuous batching.
//
// Clients submit chunks (a range of channels of the resident weights, ntimes,
// E and J buffers) as they arrive.  A server thread admits queued chunks while
// the device pool (a fixed HBM budget) has room for their E and J, packs the
// admitted chunks into one grouped tensor-core launch, and keeps up to
// max_inflight such launches in flight on separate streams, so chunks that
// arrive while others are on the GPU are admitted as memory and launch slots
// free up and their work overlaps on the device.  Each chunk's latency runs
// from submission to the moment its J has landed (input copy, beamforming and
// output copy included); a host function queued behind each launch's output
// copies stamps that moment and wakes the server thread.  max_batch = 1 with
// max_inflight = 1 is the plain per-chunk loop the server is compared against.
// Pageable host buffers go through a pinned staging ring: the submitting
// thread copies E in, the server copies J out when the chunk lands, so the
// device copies of every chunk are asynchronous.
#include "bf_internal.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

namespace {

using namespace bf;
using Clock = std::chrono::steady_clock;

// First-fit allocator over one arena (offsets aligned to 256 bytes): device
// memory for chunk buffers, or pinned host memory for the staging ring.
class Pool {
 public:
  bool init(size_t bytes, bool host = false) {
    host_ = host;
    void *p = nullptr;
    if ((host ? cudaMallocHost(&p, bytes) : cudaMalloc(&p, bytes)) != cudaSuccess) return false;
    base_ = static_cast<uint8_t *>(p);
    size_ = bytes;
    free_[0] = bytes;
    return true;
  }
  ~Pool() {
    if (base_) (void)(host_ ? cudaFreeHost(base_) : cudaFree(base_));
  }
  uint8_t *alloc(size_t n) {
    n = (n + 255) / 256 * 256;
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= n) {
        const size_t off = it->first, rest = it->second - n;
        free_.erase(it);
        if (rest) free_[off + n] = rest;
        used_ += n;
        return base_ + off;
      }
    }
    return nullptr;
  }
  void release(uint8_t *p, size_t n) {
    n = (n + 255) / 256 * 256;
    size_t off = static_cast<size_t>(p - base_);
    used_ -= n;
    auto next = free_.lower_bound(off);
    if (next != free_.end() && off + n == next->first) {  // merge with the following block
      n += next->second;
      next = free_.erase(next);
    }
    if (next != free_.begin()) {  // merge with the preceding block
      auto prev = std::prev(next);
      if (prev->first + prev->second == off) {
        prev->second += n;
        return;
      }
    }
    free_[off] = n;
  }
  size_t size() const { return size_; }
  size_t used() const { return used_; }

 private:
  uint8_t *base_ = nullptr;
  bool host_ = false;
  size_t size_ = 0, used_ = 0;
  std::map<size_t, size_t> free_;
};

// Host memory the copy engines read and write asynchronously (pinned or
// registered); pageable memory answers cudaMemoryTypeUnregistered.  Both the
// first and the last byte of the buffer are checked, so a buffer registered
// only in part goes through the staging ring (a buffer registered in several
// pieces must have no pageable gap between them).
bool pinned_byte(const void *p) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    (void)cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeHost;
}
bool pinned_host(const void *p, size_t bytes) {
  return pinned_byte(p) && (bytes <= 1 || pinned_byte(static_cast<const uint8_t *>(p) + (bytes - 1)));
}

struct Request {
  int64_t ticket;
  int version;  // weight version the chunk was submitted under
  int channel, nchannels;
  int64_t ntimes;
  const uint8_t *E;
  uint8_t *J;
  bool e_on_device, j_on_device;
  Clock::time_point arrival;
  // set on admission
  uint8_t *dE = nullptr, *dJ = nullptr;
  size_t e_bytes = 0, j_bytes = 0;
  // pinned staging of pageable host buffers: E was copied into sE at submit
  // (E then points there); J lands in sJ and is copied to J_user on landing
  uint8_t *sE = nullptr, *sJ = nullptr, *J_user = nullptr;
};

// One launch slot: a stream, its problem table and the chunks it carries.
struct Flight {
  bf_server *owner = nullptr;
  cudaStream_t s = nullptr;
  cudaEvent_t done = nullptr;
  TcProblem *table_host = nullptr;  // pinned
  TcProblem *table_dev = nullptr;
  int *err_dev = nullptr;   // this flight's kernel error word
  int *err_host = nullptr;  // pinned copy, read when the launch has landed
  std::vector<Request> reqs;
  bool busy = false;    // guarded by the server mutex
  bool landed = false;  // set by the host function behind the output copies
  bool failed = false;  // its launch failed part-way: retired without completing its chunks
  Clock::time_point landed_at;
};

// A weight version: version 0 is the caller's resident weights (never
// written); later versions are server-owned copies refreshed in turn.  A
// version is rewritten only when no queued or in-flight chunk refers to it.
constexpr int kMaxVersions = 4;
struct Version {
  const bf_weights *w = nullptr;
  bf_weights *owned = nullptr;
  int64_t refs = 0;              // chunks submitted under this version and not yet landed
  cudaEvent_t ready = nullptr;   // recorded behind the refresh on the update stream
};

}  // namespace

struct bf_server {
  int device = 0;
  const bf_weights *weights = nullptr;
  bf_server_config cfg{};
  Pool pool;
  Pool staging;  // pinned host ring for pageable chunk buffers (may be empty)
  std::vector<std::unique_ptr<Flight>> flights;
  Version ver[kMaxVersions];
  int cur = 0;                      // version new chunks are submitted under
  cudaStream_t upd_stream = nullptr;
  std::mutex upd_mu;                // one refresh at a time

  std::mutex mu;  // guards everything below, the pool and the flights' busy/landed/reqs
  std::condition_variable cv_work, cv_done;
  std::deque<Request> queue;                          // submitted, not admitted
  std::unordered_map<int64_t, double> done_latency;  // ticket -> seconds (until waited for)
  int64_t next_ticket = 0;
  int64_t completed = 0;
  int64_t submitted = 0;
  int status = BF_OK;  // first error seen
  bf_server_stats stats{};
  std::atomic<bool> stop{false};
  std::atomic<int64_t> nqueued{0};  // queue length, readable without the mutex
  std::thread worker;

  void run();
  bool launch(Flight &fl, const std::vector<Request> &reqs, int *ntiles);
  void retire_locked(Flight &fl, std::vector<Request> &staged);
  void hand_out(std::unique_lock<std::mutex> &lk, std::vector<Request> &staged);
};

namespace {

// Weights of channels [c0, c0 + n) as a weights view (the operand rows of
// those frequencies are contiguous).
TcWeights channel_view(const TcWeights &w, int c0, int n) {
  TcWeights v = w;
  v.F = n;
  v.W = w.W + static_cast<int64_t>(c0) * w.nw * 2 * w.D;
  v.dig = w.dig + static_cast<int64_t>(c0) * w.nw_pad * kDigitRow;
  v.gs = w.gs + static_cast<int64_t>(c0) * (w.nw_pad / 2);
  v.gwide = w.gwide + c0;
  v.G = w.G + static_cast<int64_t>(c0) * w.B;
  return v;
}

void CUDART_CB flight_landed(void *arg) {
  Flight *fl = static_cast<Flight *>(arg);
  bf_server *s = fl->owner;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    fl->landed = true;
    fl->landed_at = Clock::now();
  }
  s->cv_work.notify_one();
}

}  // namespace

// Queues one grouped launch for `reqs` on the flight's stream: input copies,
// the problem table, the kernel, the error word, output copies, then the
// host function that marks the flight landed.  Runs without the mutex.
bool bf_server::launch(Flight &fl, const std::vector<Request> &reqs, int *ntiles) {
  const TcWeights &w = weights->tc;
  int64_t begin = 0;
  unsigned waited = 0;  // versions whose refresh this stream already waits for
  for (size_t i = 0; i < reqs.size(); ++i) {
    const Request &r = reqs[i];
    const Version &vr = ver[r.version];  // stable: the chunk holds a reference
    if (vr.ready && !(waited & (1u << r.version))) {
      if (cudaStreamWaitEvent(fl.s, vr.ready, 0) != cudaSuccess) return false;
      waited |= 1u << r.version;
    }
    if (!r.e_on_device && cudaMemcpyAsync(r.dE, r.E, r.e_bytes, cudaMemcpyHostToDevice, fl.s) != cudaSuccess)
      return false;
    const TcWeights v = channel_view(vr.w->tc, r.channel, r.nchannels);
    TcProblem &P = fl.table_host[i];
    if (tc_make_problem(P, v, r.ntimes, r.dJ, r.e_on_device ? r.E : r.dE, 0) != cudaSuccess) return false;
    P.tile_begin = static_cast<int>(begin);
    begin += tc_problem_tiles(P);
  }
  const int n = static_cast<int>(reqs.size());
  if (cudaMemcpyAsync(fl.table_dev, fl.table_host, sizeof(TcProblem) * n, cudaMemcpyHostToDevice, fl.s) !=
      cudaSuccess)
    return false;
  if (launch_tc_grouped(fl.table_dev, n, static_cast<int>(begin), w.D, w.nb_pass, TcRingPlan{}, fl.err_dev,
                        fl.s) != cudaSuccess)
    return false;
  if (cudaMemcpyAsync(fl.err_host, fl.err_dev, sizeof(int), cudaMemcpyDeviceToHost, fl.s) != cudaSuccess)
    return false;
  for (const Request &r : reqs)
    if (!r.j_on_device && cudaMemcpyAsync(r.J, r.dJ, r.j_bytes, cudaMemcpyDeviceToHost, fl.s) != cudaSuccess)
      return false;
  if (cudaEventRecord(fl.done, fl.s) != cudaSuccess) return false;
  // polling mode watches the event instead (a host function of an earlier
  // launch could otherwise mark a later launch on the same stream landed)
  if (!cfg.spin_wait && cudaLaunchHostFunc(fl.s, flight_landed, &fl) != cudaSuccess) return false;
  *ntiles = static_cast<int>(begin);
  return true;
}

// Retires a landed launch (mutex held): frees its pool memory, its slot and
// its weight-version references, and completes its chunks.  A chunk whose J
// still sits in the staging ring is moved to `staged` instead and completes
// in hand_out(), which copies it to the caller without the mutex.
void bf_server::retire_locked(Flight &fl, std::vector<Request> &staged) {
  if (!fl.failed && *fl.err_host != 0 && status == BF_OK) status = BF_ERR_DEVICE_TIMEOUT;  // a kernel wait gave up
  for (Request &r : fl.reqs) {
    --ver[r.version].refs;
    if (!r.e_on_device) pool.release(r.dE, r.e_bytes);
    if (!r.j_on_device) pool.release(r.dJ, r.j_bytes);
    if (r.sE) staging.release(r.sE, r.e_bytes);
    r.sE = nullptr;
    if (fl.failed) {  // never completed: waits for it return the server's error status
      if (r.sJ) staging.release(r.sJ, r.j_bytes);
      continue;
    }
    if (r.sJ) {
      staged.push_back(r);
      continue;
    }
    done_latency[r.ticket] = std::chrono::duration<double>(fl.landed_at - r.arrival).count();
    ++completed;
  }
  fl.reqs.clear();
  fl.busy = false;
  fl.landed = false;
  fl.failed = false;
  cv_done.notify_all();
}

// Copies the J of staged chunks from the ring into the callers' buffers with
// the mutex released (a chunk's J can be hundreds of MB), then frees their
// ring room and completes them.  Called with `lk` held; returns with it held.
void bf_server::hand_out(std::unique_lock<std::mutex> &lk, std::vector<Request> &staged) {
  if (staged.empty()) return;
  lk.unlock();
  std::vector<Clock::time_point> done(staged.size());
  for (size_t i = 0; i < staged.size(); ++i) {
    std::memcpy(staged[i].J_user, staged[i].sJ, staged[i].j_bytes);
    done[i] = Clock::now();
  }
  lk.lock();
  for (size_t i = 0; i < staged.size(); ++i) {
    const Request &r = staged[i];
    staging.release(r.sJ, r.j_bytes);
    done_latency[r.ticket] = std::chrono::duration<double>(done[i] - r.arrival).count();
    ++completed;
  }
  staged.clear();
  cv_done.notify_all();
}

void bf_server::run() {
  cudaSetDevice(device);
  std::unique_lock<std::mutex> lk(mu, std::defer_lock);
  for (;;) {
    if (cfg.spin_wait) {
      // Polling mode: a launch has landed when its event has completed.  Only
      // this thread touches the flights in this mode, so the polling runs
      // without the mutex, which is taken only when there is work to do.
      bool work = stop.load(std::memory_order_relaxed);
      bool free_slot = false;
      for (auto &fp : flights) {
        if (!fp->busy) {
          free_slot = true;
          continue;
        }
        if (fp->landed) {
          work = true;
          continue;
        }
        const cudaError_t q = cudaEventQuery(fp->done);
        if (q == cudaSuccess) {
          fp->landed = true;
          fp->landed_at = Clock::now();
          work = true;
        } else if (q != cudaErrorNotReady) {
          work = true;  // reported below
        }
      }
      if (free_slot && nqueued.load(std::memory_order_acquire) > 0) work = true;
      if (!work) {
        std::this_thread::yield();
        continue;
      }
    }
    lk.lock();
    // retire landed launches: their pool memory and slot become free; J that
    // waits in the staging ring is handed out after the next launch is queued
    std::vector<Request> staged;
    for (auto &fp : flights)
      if (fp->busy && fp->landed) retire_locked(*fp, staged);
    // admit queued chunks into a free slot while the pool has room for them
    Flight *slot = nullptr;
    for (auto &fp : flights)
      if (!fp->busy) {
        slot = fp.get();
        break;
      }
    if (slot && status == BF_OK) {
      std::vector<Request> batch;
      while (!queue.empty() && static_cast<int>(batch.size()) < cfg.max_batch) {
        Request &r = queue.front();
        uint8_t *dE = r.e_on_device ? const_cast<uint8_t *>(r.E) : pool.alloc(r.e_bytes);
        uint8_t *dJ = r.j_on_device ? r.J : (dE ? pool.alloc(r.j_bytes) : nullptr);
        if (!dE || !dJ) {  // not enough free HBM: wait for a launch to land
          if (dE && !r.e_on_device) pool.release(dE, r.e_bytes);
          break;
        }
        r.dE = dE;
        r.dJ = dJ;
        batch.push_back(r);
        queue.pop_front();
        nqueued.fetch_sub(1, std::memory_order_relaxed);
      }
      if (!batch.empty()) {
        stats.pool_peak_bytes = std::max<int64_t>(stats.pool_peak_bytes, static_cast<int64_t>(pool.used()));
        slot->busy = true;
        slot->landed = false;
        lk.unlock();
        int ntiles = 0;
        const bool ok = launch(*slot, batch, &ntiles);
        // A launch that failed part-way records no event of its own (the
        // flight's event still holds an earlier launch) and no host function:
        // let what it did queue finish, then retire it as failed, so that its
        // memory is freed and none of its chunks is reported complete.
        if (!ok) (void)cudaStreamSynchronize(slot->s);
        lk.lock();
        slot->reqs = std::move(batch);
        const int n = static_cast<int>(slot->reqs.size());
        stats.batches += 1;
        stats.chunks_launched += n;
        stats.max_batch_seen = std::max<int64_t>(stats.max_batch_seen, n);
        if (!ok) {
          if (status == BF_OK) status = BF_ERR_CUDA;
          slot->failed = true;
          slot->landed = true;
          slot->landed_at = Clock::now();
          cv_done.notify_all();
        }
        hand_out(lk, staged);
        lk.unlock();
        continue;
      }
    }
    hand_out(lk, staged);
    bool inflight = false;
    for (auto &fp : flights) inflight |= fp->busy;
    if (stop.load() && ((queue.empty() && !inflight) || status != BF_OK)) break;
    if (inflight) {  // a launch that failed never lands: look for errors now and then
      for (auto &fp : flights) {
        if (!fp->busy || fp->landed) continue;
        const cudaError_t q = cudaEventQuery(fp->done);
        if (q != cudaSuccess && q != cudaErrorNotReady && status == BF_OK) status = BF_ERR_CUDA;
      }
      if (status != BF_OK) cv_done.notify_all();
    }
    if (!cfg.spin_wait) cv_work.wait_for(lk, std::chrono::milliseconds(inflight ? 2 : 50));
    lk.unlock();
  }
}

extern "C" {

int bf_server_create(bf_server **out, const bf_weights *weights, const bf_server_config *cfg) {
  if (!out || !weights) return BF_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  const bf_dims d{16, weights->tc.F, weights->tc.D, 2, weights->tc.B};
  if (!tc_supported(d)) return BF_ERR_UNSUPPORTED;
  bf_server *s = new bf_server();
  cudaGetDevice(&s->device);
  s->weights = weights;
  s->ver[0].w = weights;
  if (cfg) s->cfg = *cfg;
  if (s->cfg.max_batch <= 0) s->cfg.max_batch = 64;
  if (s->cfg.max_inflight <= 0) s->cfg.max_inflight = 3;
  size_t free_b = 0, total_b = 0;
  int st = cudaMemGetInfo(&free_b, &total_b) == cudaSuccess ? BF_OK : BF_ERR_NO_DEVICE;
  size_t budget = s->cfg.hbm_budget_bytes > 0 ? static_cast<size_t>(s->cfg.hbm_budget_bytes) : free_b / 2;
  budget = std::min(budget, free_b * 9 / 10);
  s->cfg.hbm_budget_bytes = static_cast<int64_t>(budget);
  if (st == BF_OK && !s->pool.init(budget)) st = BF_ERR_OUT_OF_MEMORY;
  if (s->cfg.staging_bytes == 0) s->cfg.staging_bytes = int64_t(256) << 20;
  if (st == BF_OK && s->cfg.staging_bytes > 0 && !s->staging.init(static_cast<size_t>(s->cfg.staging_bytes), true))
    st = BF_ERR_OUT_OF_MEMORY;
  if (st == BF_OK && cudaStreamCreateWithFlags(&s->upd_stream, cudaStreamNonBlocking) != cudaSuccess)
    st = BF_ERR_CUDA;
  for (int i = 0; st == BF_OK && i < s->cfg.max_inflight; ++i) {
    s->flights.push_back(std::make_unique<Flight>());
    Flight &fl = *s->flights.back();
    fl.owner = s;
    if (cudaStreamCreateWithFlags(&fl.s, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&fl.done, cudaEventDisableTiming) != cudaSuccess ||
        cudaMallocHost(&fl.table_host, sizeof(TcProblem) * s->cfg.max_batch) != cudaSuccess ||
        cudaMalloc(&fl.table_dev, sizeof(TcProblem) * s->cfg.max_batch) != cudaSuccess ||
        cudaMalloc(&fl.err_dev, sizeof(int)) != cudaSuccess ||
        cudaMallocHost(&fl.err_host, sizeof(int)) != cudaSuccess ||
        cudaMemset(fl.err_dev, 0, sizeof(int)) != cudaSuccess)
      st = BF_ERR_OUT_OF_MEMORY;
  }
  if (st != BF_OK) {
    bf_server_destroy(s);
    return st;
  }
  s->worker = std::thread([s]() { s->run(); });
  *out = s;
  return BF_OK;
}

int bf_server_submit(bf_server *s, int channel, int nchannels, int64_t ntimes, const uint8_t *E, int e_on_device,
                     uint8_t *J, int j_on_device, int64_t *ticket) {
  if (!s || !E || !J || !ticket || ntimes <= 0 || nchannels <= 0 || channel < 0 ||
      channel + nchannels > s->weights->tc.F)
    return BF_ERR_INVALID_ARGUMENT;
  const bf_dims d{ntimes, nchannels, s->weights->tc.D, 2, s->weights->tc.B};
  if (!tc_supported(d)) return BF_ERR_UNSUPPORTED;
  if ((e_on_device && (reinterpret_cast<uintptr_t>(E) & 15u)) ||
      (j_on_device && (reinterpret_cast<uintptr_t>(J) & 15u)))
    return BF_ERR_UNSUPPORTED;
  Request r;
  r.channel = channel;
  r.nchannels = nchannels;
  r.ntimes = ntimes;
  r.E = E;
  r.J = J;
  r.e_on_device = e_on_device != 0;
  r.j_on_device = j_on_device != 0;
  r.e_bytes = static_cast<size_t>(ntimes) * nchannels * s->weights->tc.D * 2;
  r.j_bytes = static_cast<size_t>(s->weights->tc.B) * nchannels * 2 * ntimes;
  // a chunk whose buffers can never fit the pool is refused instead of waiting forever
  if ((r.e_on_device ? 0 : r.e_bytes + 256) + (r.j_on_device ? 0 : r.j_bytes + 256) > s->pool.size())
    return BF_ERR_OUT_OF_MEMORY;
  r.arrival = Clock::now();  // latency includes waiting for ring room and the staging copy
  // pageable host buffers go through the pinned ring (when they fit in it):
  // room is taken here, waiting for landed chunks to free it if need be, and
  // E is copied in by this thread, so the server's device copies stay
  // asynchronous; J is copied out of the ring when the chunk lands
  const bool stage_e = !r.e_on_device && !pinned_host(E, r.e_bytes);
  const bool stage_j = !r.j_on_device && !pinned_host(J, r.j_bytes);
  const size_t need = (stage_e ? r.e_bytes + 256 : 0) + (stage_j ? r.j_bytes + 256 : 0);
  if (need > 0 && need <= s->staging.size()) {
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
      if (s->status != BF_OK) return s->status;
      r.sE = stage_e ? s->staging.alloc(r.e_bytes) : nullptr;
      r.sJ = stage_j && (r.sE || !stage_e) ? s->staging.alloc(r.j_bytes) : nullptr;
      if ((r.sE || !stage_e) && (r.sJ || !stage_j)) break;
      if (r.sE) s->staging.release(r.sE, r.e_bytes);  // not both: give back and wait for a landing
      r.sE = r.sJ = nullptr;
      s->cv_done.wait_for(lk, std::chrono::milliseconds(50));
    }
    ++s->stats.staged;
  }
  if (r.sE) {
    std::memcpy(r.sE, E, r.e_bytes);
    r.E = r.sE;
  }
  if (r.sJ) {
    r.J_user = J;
    r.J = r.sJ;
  }
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->status != BF_OK) {
      if (r.sE) s->staging.release(r.sE, r.e_bytes);
      if (r.sJ) s->staging.release(r.sJ, r.j_bytes);
      return s->status;
    }
    r.ticket = s->next_ticket++;
    r.version = s->cur;
    ++s->ver[s->cur].refs;
    ++s->submitted;
    s->queue.push_back(r);
    s->nqueued.fetch_add(1, std::memory_order_release);
  }
  s->cv_work.notify_one();
  *ticket = r.ticket;
  return BF_OK;
}

int bf_server_update_weights(bf_server *s, const uint8_t *A, const float *G, int ptr_kind) {
  if (!s || !A || !G || (ptr_kind != BF_PTR_HOST && ptr_kind != BF_PTR_DEVICE)) return BF_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> one(s->upd_mu);
  // a version slot other than the caller's weights and the current one, with no chunk on it
  int slot = -1;
  {
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
      if (s->status != BF_OK) return s->status;
      for (int i = 1; i < kMaxVersions && slot < 0; ++i)
        if (i != s->cur && s->ver[i].refs == 0) slot = i;
      if (slot >= 0) break;
      s->cv_done.wait_for(lk, std::chrono::milliseconds(50));  // every version busy: wait for chunks to land
    }
  }
  Version &v = s->ver[slot];
  const TcWeights &w = s->weights->tc;
  int st = BF_OK;
  if (!v.owned) {
    st = bf_weights_create(&v.owned, w.F, w.B, w.D, A, G, ptr_kind, s->upd_stream);
    if (st == BF_OK && cudaEventCreateWithFlags(&v.ready, cudaEventDisableTiming) != cudaSuccess) st = BF_ERR_CUDA;
  } else {
    st = bf_weights_update(v.owned, A, G, ptr_kind, s->upd_stream);
  }
  if (st != BF_OK) return st;
  if (cudaEventRecord(v.ready, s->upd_stream) != cudaSuccess) return BF_ERR_CUDA;
  // the caller may reuse or free A and G once this returns
  if (cudaStreamSynchronize(s->upd_stream) != cudaSuccess) return BF_ERR_CUDA;
  std::lock_guard<std::mutex> lk(s->mu);
  v.w = v.owned;
  s->cur = slot;
  ++s->stats.weight_updates;
  return BF_OK;
}

int bf_server_wait(bf_server *s, int64_t ticket, double *latency_s) {
  if (!s || ticket < 0) return BF_ERR_INVALID_ARGUMENT;
  std::unique_lock<std::mutex> lk(s->mu);
  if (ticket >= s->next_ticket) return BF_ERR_INVALID_ARGUMENT;
  for (;;) {
    auto it = s->done_latency.find(ticket);
    if (it != s->done_latency.end()) {
      if (latency_s) *latency_s = it->second;
      s->done_latency.erase(it);
      return BF_OK;
    }
    if (s->status != BF_OK) return s->status;
    s->cv_done.wait_for(lk, std::chrono::milliseconds(50));
  }
}

int bf_server_drain(bf_server *s) {
  if (!s) return BF_ERR_INVALID_ARGUMENT;
  std::unique_lock<std::mutex> lk(s->mu);
  while (s->completed < s->submitted && s->status == BF_OK) s->cv_done.wait_for(lk, std::chrono::milliseconds(50));
  return s->status;
}

int bf_server_replay(bf_server *s, int n, const int *channel, const int64_t *ntimes, const uint8_t *const *E,
                     int e_on_device, uint8_t *const *J_slots, int nslots, const int64_t *j_bytes, int j_on_device,
                     const double *arrival_s, int check_threads, double *latency_s, double *late_s,
                     uint32_t *adler_out, double *wall_s, int64_t *slot_stalls) {
  if (!s || n < 0 || check_threads < 0 || !wall_s) return BF_ERR_INVALID_ARGUMENT;
  if (n > 0 && (!channel || !ntimes || !E || !J_slots || nslots <= 0 || !j_bytes || !arrival_s || !latency_s))
    return BF_ERR_INVALID_ARGUMENT;
  if (check_threads > 0 && (j_on_device || !adler_out)) return BF_ERR_INVALID_ARGUMENT;
  *wall_s = 0.0;
  if (slot_stalls) *slot_stalls = 0;
  if (n == 0) return BF_OK;

  std::vector<int64_t> tickets(static_cast<size_t>(n), -1);
  // slot k may take chunk i once chunk i - nslots, its previous user, is done
  // (landed, and checked when checking); done_upto[k] is the last such chunk
  std::vector<int64_t> done_upto(static_cast<size_t>(nslots), -1);
  std::mutex m;
  std::condition_variable cv_pub, cv_check, cv_free;
  int published = 0;        // chunks submitted (their tickets are valid)
  bool waiter_done = false;
  std::deque<int> to_check;
  std::atomic<int> status{BF_OK};
  const auto t0 = Clock::now();
  Clock::time_point t_last = t0;

  auto release_slot = [&](int i) {
    std::lock_guard<std::mutex> lk(m);
    int64_t &d = done_upto[static_cast<size_t>(i % nslots)];
    d = std::max<int64_t>(d, i);
    cv_free.notify_all();
  };
  std::thread waiter([&] {
    for (int i = 0; i < n; ++i) {
      {
        std::unique_lock<std::mutex> lk(m);
        cv_pub.wait(lk, [&] { return published > i || status.load() != BF_OK; });
        if (published <= i) break;  // the submitter stopped
      }
      double lat = 0.0;
      const int st = bf_server_wait(s, tickets[static_cast<size_t>(i)], &lat);
      if (st != BF_OK) {
        status.store(st);
        break;
      }
      latency_s[i] = lat;
      t_last = Clock::now();
      if (check_threads > 0) {
        std::lock_guard<std::mutex> lk(m);
        to_check.push_back(i);
        cv_check.notify_one();
      } else {
        release_slot(i);
      }
    }
    std::lock_guard<std::mutex> lk(m);
    waiter_done = true;
    cv_check.notify_all();
    cv_free.notify_all();
  });
  std::vector<std::thread> checkers;
  for (int c = 0; c < check_threads; ++c)
    checkers.emplace_back([&] {
      for (;;) {
        int i;
        {
          std::unique_lock<std::mutex> lk(m);
          cv_check.wait(lk, [&] { return !to_check.empty() || waiter_done; });
          if (to_check.empty()) return;
          i = to_check.front();
          to_check.pop_front();
        }
        adler_out[i] = adler32_host(J_slots[i % nslots], static_cast<size_t>(j_bytes[i]));
        release_slot(i);
      }
    });

  int64_t stalls = 0;
  for (int i = 0; i < n && status.load() == BF_OK; ++i) {
    const int k = i % nslots;
    {
      std::unique_lock<std::mutex> lk(m);
      if (done_upto[static_cast<size_t>(k)] < i - nslots) {
        ++stalls;
        cv_free.wait(lk, [&] {
          return done_upto[static_cast<size_t>(k)] >= i - nslots || status.load() != BF_OK || waiter_done;
        });
        if (done_upto[static_cast<size_t>(k)] < i - nslots) break;
      }
    }
    // sleep to just before the arrival time, then spin to it
    const auto due = t0 + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(arrival_s[i]));
    const auto ahead = due - Clock::now();
    if (ahead > std::chrono::microseconds(300)) std::this_thread::sleep_for(ahead - std::chrono::microseconds(200));
    while (Clock::now() < due) {
    }
    int64_t tk = -1;
    const int st = bf_server_submit(s, channel[i], 1, ntimes[i], E[i], e_on_device, J_slots[k], j_on_device, &tk);
    if (late_s) late_s[i] = std::chrono::duration<double>(Clock::now() - due).count();
    if (st != BF_OK) {
      status.store(st);
      break;
    }
    std::lock_guard<std::mutex> lk(m);
    tickets[static_cast<size_t>(i)] = tk;
    published = i + 1;
    cv_pub.notify_one();
  }
  {
    std::lock_guard<std::mutex> lk(m);
    cv_pub.notify_all();  // a failed submission ends the waiter too
  }
  waiter.join();
  for (auto &t : checkers) t.join();
  *wall_s = std::chrono::duration<double>(t_last - t0).count();
  if (slot_stalls) *slot_stalls = stalls;
  return status.load();
}

int bf_server_stats_get(bf_server *s, bf_server_stats *out) {
  if (!s || !out) return BF_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(s->mu);
  *out = s->stats;
  out->pool_bytes = s->cfg.hbm_budget_bytes;
  out->submitted = s->submitted;
  out->completed = s->completed;
  return s->status;
}

int bf_server_destroy(bf_server *s) {
  if (!s) return BF_OK;
  if (s->worker.joinable()) {
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->stop.store(true);
    }
    s->cv_work.notify_all();
    s->worker.join();
  }
  for (auto &fp : s->flights) {
    Flight &fl = *fp;
    if (fl.s) cudaStreamSynchronize(fl.s);  // host functions behind the copies have run after this
    if (fl.s) cudaStreamDestroy(fl.s);
    if (fl.done) cudaEventDestroy(fl.done);
    if (fl.table_host) cudaFreeHost(fl.table_host);
    if (fl.table_dev) cudaFree(fl.table_dev);
    if (fl.err_dev) cudaFree(fl.err_dev);
    if (fl.err_host) cudaFreeHost(fl.err_host);
  }
  for (Version &v : s->ver) {
    if (v.owned) bf_weights_destroy(v.owned);
    if (v.ready) cudaEventDestroy(v.ready);
  }
  if (s->upd_stream) cudaStreamDestroy(s->upd_stream);
  delete s;
  return BF_OK;
}

}  // extern "C"
