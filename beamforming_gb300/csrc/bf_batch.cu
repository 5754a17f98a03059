// bf_batch.cu -- many uneven beamforming problems in one persistent launch.
//
// A batch is a fixed set of problems (each: resident weights for some
// frequencies, a number of times, device E and J).  Every problem keeps its own
// shape -- ntimes and nbeams may all differ; ndishes is shared -- and the
// tensor-core kernel walks one tile list that spans all of them.  At creation
// an autotuner times a few schedules on the real buffers and keeps the
// fastest: the tile shape, the tile order and the shared-memory ring plan.
// The tile shape groups the problems by beam-pass width into up to three
// launches: wide passes (more than 64 beams), narrow ones (at most 64: four or
// more unpacked stages fit in tensor memory beside the narrower accumulators,
// and two unpack groups keep the tensor core fed) and the narrowest (at most
// 16: two CTAs share each SM).  A launch takes the layout of its widest pass,
// so each cut between classes is kept only when timing says so.  The chosen
// launches are captured in a CUDA graph, and bf_batch_run() replays it.
#include "bf_internal.h"

#include <algorithm>
#include <numeric>
#include <vector>

namespace {
// One grouped launch of a batch: a range of the device problem table.
struct BatchLaunch {
  int first = 0, nprob = 0, ntiles = 0, max_nb_pass = 0, stages = 0, groups = 0, ctas_per_sm = 0;
};
constexpr int kMaxLaunches = 3;  // one per pass-width class
}  // namespace

struct bf_batch {
  int device = 0;
  int nprob = 0;
  int ntiles = 0;
  int64_t D = 0;
  int *err = nullptr;
  bf::TcProblem *table = nullptr;  // device copy, launch order
  bf::TcRingPlan plan;
  int order = 0;                   // chosen tile order (0: as given, 1: largest problem first)
  int cuts = 0;                    // chosen tile shape: bit c set = classes c and c + 1 in separate launches
  int nlaunch = 0;
  BatchLaunch launches[kMaxLaunches];
  float tuned_ms = 0.0f;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace {

using namespace bf;

int status_of(cudaError_t e) {
  if (e == cudaSuccess) return BF_OK;
  if (e == cudaErrorMemoryAllocation) return BF_ERR_OUT_OF_MEMORY;
  return BF_ERR_CUDA;
}

#define BF_TRY(expr)                               \
  do {                                             \
    const cudaError_t e_ = (expr);                 \
    if (e_ != cudaSuccess) return status_of(e_);   \
  } while (0)

// A schedule: the problem table in launch order (tile_begin counted from the
// start of each launch) and its launches.
struct Schedule {
  std::vector<TcProblem> table;
  int nlaunch = 0;
  BatchLaunch launches[kMaxLaunches];
};

// Pass-width class of a problem: 0 wide, 1 narrow (<= kNarrowPass beams),
// 2 narrowest (<= kHalfPass beams).
int class_of(const TcProblem &P) { return P.nb_pass <= kHalfPass ? 2 : P.nb_pass <= kNarrowPass ? 1 : 0; }

// Launch of class c under `cuts`: the number of cuts below it.
int launch_of(int cls, int cuts) { return (cls >= 1 && (cuts & 1)) + (cls >= 2 && (cuts & 2)); }

// Problems in `order`, one launch per group of classes that `cuts` keeps
// together (wider classes first); empty launches are dropped.
Schedule schedule_of(const std::vector<TcProblem> &probs, const std::vector<int> &order, int cuts) {
  Schedule sc;
  for (int l = 0; l < kMaxLaunches; ++l) {
    BatchLaunch L;
    L.first = static_cast<int>(sc.table.size());
    int64_t begin = 0;
    for (int i : order) {
      if (launch_of(class_of(probs[i]), cuts) != l) continue;
      TcProblem P = probs[i];
      P.tile_begin = static_cast<int>(begin);
      begin += tc_problem_tiles(P);
      L.max_nb_pass = std::max(L.max_nb_pass, P.nb_pass);
      sc.table.push_back(P);
    }
    L.nprob = static_cast<int>(sc.table.size()) - L.first;
    L.ntiles = static_cast<int>(begin);
    if (L.nprob > 0) sc.launches[sc.nlaunch++] = L;
  }
  return sc;
}

// The device error word after the tuning launches: a bounded wait that gave
// up in any candidate voids the timings and the outputs (the word is cleared).
int take_device_error(int *err, cudaStream_t s) {
  int h = 0;
  BF_TRY(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  BF_TRY(cudaStreamSynchronize(s));
  if (h == 0) return BF_OK;
  BF_TRY(cudaMemsetAsync(err, 0, sizeof(int), s));
  BF_TRY(cudaStreamSynchronize(s));
  return BF_ERR_DEVICE_TIMEOUT;
}

cudaError_t launch_schedule(const bf_batch *b, const BatchLaunch *ls, int n, const TcRingPlan &plan,
                            cudaStream_t s) {
  for (int i = 0; i < n; ++i) {
    const cudaError_t e =
        launch_tc_grouped(b->table + ls[i].first, ls[i].nprob, ls[i].ntiles, b->D, ls[i].max_nb_pass, plan, b->err, s);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace

extern "C" {

int bf_batch_create(bf_batch **out, const bf_problem *problems, int nproblems, bf_stream_t stream) {
  if (!out || !problems || nproblems <= 0) return BF_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int64_t D = -1;
  std::vector<TcProblem> probs(static_cast<size_t>(nproblems));
  bool present[3] = {false, false, false};
  for (int i = 0; i < nproblems; ++i) {
    const bf_problem &q = problems[i];
    if (!q.weights || !q.E || !q.J || q.ntimes <= 0) return BF_ERR_INVALID_ARGUMENT;
    const TcWeights &w = q.weights->tc;
    if (D < 0) D = w.D;
    const bf_dims d{q.ntimes, w.F, w.D, 2, w.B};
    if (w.D != D || !tc_supported(d)) return BF_ERR_UNSUPPORTED;
    if ((reinterpret_cast<uintptr_t>(q.E) | reinterpret_cast<uintptr_t>(q.J)) & 15u) return BF_ERR_UNSUPPORTED;
    BF_TRY(tc_make_problem(probs[i], w, q.ntimes, q.J, q.E, 0));
    present[class_of(probs[i])] = true;
  }
  int *err = nullptr;
  int st = device_error_word(&err);
  if (st != BF_OK) return st;

  bf_batch *b = new bf_batch();
  cudaGetDevice(&b->device);
  b->nprob = nproblems;
  b->D = D;
  b->err = err;
  if (cudaMalloc(&b->table, sizeof(TcProblem) * nproblems) != cudaSuccess) {
    delete b;
    return BF_ERR_OUT_OF_MEMORY;
  }

  // Autotune: tile shape x tile order x ring plan, each timed on the real
  // buffers (every candidate writes the same J, so the outputs are valid
  // afterwards).  A cut is tried only where classes sit on both sides of it.
  std::vector<int> given(static_cast<size_t>(nproblems));
  std::iota(given.begin(), given.end(), 0);
  std::vector<int> largest = given;
  std::stable_sort(largest.begin(), largest.end(), [&](int x, int y) {
    return tc_problem_tiles(probs[x]) > tc_problem_tiles(probs[y]);
  });
  const std::vector<int> *orders[2] = {&given, &largest};
  const bool cut_ok[2] = {present[0] && (present[1] || present[2]), present[2] && (present[0] || present[1])};
  TcRingPlan plans[3];
  plans[1].wslots = 4;
  plans[1].raw = 8;
  plans[2].wslots = 2;
  plans[2].raw = 12;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = -1.0f;
  st = BF_OK;
  for (int cuts = 0; cuts < 4 && st == BF_OK; ++cuts) {
    if (((cuts & 1) && !cut_ok[0]) || ((cuts & 2) && !cut_ok[1])) continue;
    for (int o = 0; o < 2 && st == BF_OK; ++o) {
      const Schedule sc = schedule_of(probs, *orders[o], cuts);
      cudaError_t e = cudaMemcpyAsync(b->table, sc.table.data(), sizeof(TcProblem) * sc.table.size(),
                                      cudaMemcpyHostToDevice, s);
      for (int pl = 0; pl < 3 && e == cudaSuccess; ++pl) {
        e = launch_schedule(b, sc.launches, sc.nlaunch, plans[pl], s);  // warm-up
        if (e != cudaSuccess) break;
        cudaEventRecord(e0, s);
        for (int rep = 0; rep < 3 && e == cudaSuccess; ++rep) e = launch_schedule(b, sc.launches, sc.nlaunch, plans[pl], s);
        cudaEventRecord(e1, s);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float ms = 0.0f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e == cudaSuccess && (best < 0.0f || ms < best)) {
          best = ms;
          b->cuts = cuts;
          b->order = o;
          b->plan = plans[pl];
        }
      }
      if (e != cudaSuccess) st = status_of(e);
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st == BF_OK) st = take_device_error(err, s);
  if (st == BF_OK) {
    const Schedule sc = schedule_of(probs, *orders[b->order], b->cuts);
    b->tuned_ms = best / 3.0f;
    b->nlaunch = sc.nlaunch;
    b->ntiles = 0;
    for (int i = 0; i < sc.nlaunch; ++i) {
      b->launches[i] = sc.launches[i];
      b->ntiles += sc.launches[i].ntiles;
      BatchLaunch &L = b->launches[i];
      if (tc_launch_shape(D, L.max_nb_pass, b->plan, &L.stages, &L.groups, &L.ctas_per_sm) != cudaSuccess)
        st = BF_ERR_UNSUPPORTED;
    }
    cudaError_t e = cudaMemcpyAsync(b->table, sc.table.data(), sizeof(TcProblem) * sc.table.size(),
                                    cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    // capture the chosen launches in a graph
    cudaStream_t cap = nullptr;
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      const cudaError_t le = launch_schedule(b, b->launches, b->nlaunch, b->plan, cap);
      e = cudaStreamEndCapture(cap, &b->graph);
      if (le != cudaSuccess) e = le;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, b->graph, 0);
    if (cap) cudaStreamDestroy(cap);
    if (e != cudaSuccess && st == BF_OK) st = status_of(e);
  }
  if (st != BF_OK) {
    bf_batch_destroy(b);
    return st;
  }
  *out = b;
  return BF_OK;
}

int bf_batch_run(bf_batch *b, bf_stream_t stream) {
  if (!b || !b->exec) return BF_ERR_INVALID_ARGUMENT;
  return status_of(cudaGraphLaunch(b->exec, static_cast<cudaStream_t>(stream)));
}

int bf_batch_info(const bf_batch *b, int *ntiles, int *order, int *wslots, int *raw, float *tuned_ms) {
  if (!b) return BF_ERR_INVALID_ARGUMENT;
  if (ntiles) *ntiles = b->ntiles;
  if (order) *order = b->order;
  if (wslots) *wslots = b->plan.wslots;
  if (raw) *raw = b->plan.raw;
  if (tuned_ms) *tuned_ms = b->tuned_ms;
  return BF_OK;
}

int bf_plan_rings(int64_t ndishes, int max_nb_pass, int wslots, int raw, int *out) {
  if (!out || ndishes <= 0 || ndishes > 2048 || max_nb_pass <= 0 || max_nb_pass > 128 || wslots < 0 || raw < 0)
    return BF_ERR_INVALID_ARGUMENT;
  bf::TcRingPlan plan;
  plan.wslots = wslots;
  plan.raw = raw;
  return bf::tc_plan_rings(ndishes, max_nb_pass, plan, out) == cudaSuccess ? BF_OK : BF_ERR_INVALID_ARGUMENT;
}

int bf_batch_shape(const bf_batch *b, int *nlaunches, int *nproblems, int *ntiles, int *max_nb_pass, int *stages,
                   int *unpack_groups, int *ctas_per_sm) {
  if (!b || !nlaunches) return BF_ERR_INVALID_ARGUMENT;
  *nlaunches = b->nlaunch;
  for (int i = 0; i < b->nlaunch; ++i) {
    const BatchLaunch &L = b->launches[i];
    if (nproblems) nproblems[i] = L.nprob;
    if (ntiles) ntiles[i] = L.ntiles;
    if (max_nb_pass) max_nb_pass[i] = L.max_nb_pass;
    if (stages) stages[i] = L.stages;
    if (unpack_groups) unpack_groups[i] = L.groups;
    if (ctas_per_sm) ctas_per_sm[i] = L.ctas_per_sm;
  }
  return BF_OK;
}

int bf_batch_destroy(bf_batch *b) {
  if (!b) return BF_OK;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  if (b->table) cudaFree(b->table);
  delete b;
  return BF_OK;
}

}  // extern "C"
