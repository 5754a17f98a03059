// bf_tc.cu -- the beamformer on the 5th-generation tensor cores (tcgen05).
//
// The complex sum of cpu.cxx:26-35 becomes one real GEMM per frequency:
//
//   rows    m = (t, p)      128 per tile: 64 times x 2 polarizations
//   columns n = (b, re|im)  2 * beams (<= 192 per pass)
//   depth   k = (d, re|im)  2 * dishes
//
//   [Jre]   [ Ar  -Ai ] [Ere]
//   [Jim] = [ Ai   Ar ] [Eim]      summed over d
//
// Operands are 8-bit floats (E4M3).  A byte holding an unsigned nibble u in
// [0, 15] is, read as E4M3, exactly u * 2^-9 (exponent field 0 or 1: the
// subnormal and the first normal binade share the step 2^-9).  So the raw
// ucomplex4 nibbles (value x stored as u = x + 8) become tensor-core operands
// with one AND per 4 values.  The offset goes into the accumulator's start
// value, set by one extra MMA that opens every tile (digit rows of the row
// sums times a constant tile, see kDigitScaleLo):
//
//   acc[n] = -8 * sum_k W[n][k] / 512 + sum_k u_k W[n][k] / 512
//          = sum_k (u_k - 8) W[n][k] / 512 = raw / 512
//
// W holds the integers Ar, -Ai, Ai in [-8, 8], exact in E4M3; the start value
// and every partial sum are integer multiples of 2^-9 below 2^10 in magnitude
// (at most 19 significant bits), exact in the f32 accumulator.  The
// requantisation clamp(lrint(G * float(raw)), -7, 7) of cpu.cxx:37-39 is one
// IEEE multiply by 512 G (exactly G * raw) and a round-half-even conversion.
//
// Warp roles (one CTA per SM, persistent over tiles; warp numbers for the
// layout of 8 epilogue warps, 480 threads; with 12 epilogue warps, 608
// threads, the roles after the epilogue move up by four):
//   warps 0-7    epilogue: TMEM accumulator -> registers -> requantise (multiply,
//                clamp, convert, saturating nibble pack) -> 4x4 byte transpose
//                across lanes -> 32-bit stores of 4 consecutive times of one beam
//   warp  8      E producer: TMA of raw E boxes into a deep ring released by the unpack
//   warp  9      TMEM allocator and single-thread MMA issuer (A operand from TMEM)
//   warp  10     W producer: TMA of each tile's digit rows and of the W slice of
//                each K stage, released by the MMA
//   warps 11-14  unpack (groups of four take K stages in turn): raw E bytes ->
//                de-interleaved E4M3 operand rows written straight into tensor
//                memory (tcgen05.st); no shared-memory operand
//
// Launches with four or more unpacked stages in TMEM (beam passes of at most
// 64 beams) run two unpack groups, which take the stages in turn, and one more
// warp, the W forwarder: it arrives on a stage's a_full once that stage's W slot
// has landed, so the unpack warps carry no W hand-over, and the W producer
// reuses a slot as soon as the tensor core has finished the stage that used it.
//
// GEMM row r of a tile (TMEM lane r) is (t, p) = (r / 2, r % 2) for the 64 times
// of the tile.  TMEM columns: accumulators at [0, N) and [256, 256 + N), unpacked
// E stages (64 columns = 256 K bytes each) in the remaining columns.
#include "bf_internal.h"
#include "bf_ptx.cuh"

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <cudaTypedefs.h>

namespace bf {
namespace {

// Warp layout: kEpiWarps epilogue warps, the three single-thread roles, then
// kUnpackGroups groups of four unpack warps.  A warp reaches TMEM lanes
// 32 * (warp % 4) .. + 31 only, so every role that touches TMEM rows comes in
// fours covering the four lane quarters.  Twelve epilogue warps suit short K
// (ndishes <= 512: the epilogue paces the tiles), eight suit long K (the
// unpack does, and more epilogue warps take its issue slots).
template <int kEpiWarps_, int kUnpackGroups_>
struct Roles {
  static constexpr int kEpiWarps = kEpiWarps_;
  static constexpr int kUnpackGroups = kUnpackGroups_;
  static constexpr bool kForwarder = kUnpackGroups > 1;  // W-landed forwarder warp
  static constexpr int kEpiThreads = 32 * kEpiWarps;
  static constexpr int kEpiParts = kEpiWarps / 4;  // column parts: each read by four warps (one per lane quarter)
  static constexpr int kEProdWarp = kEpiWarps;
  static constexpr int kMmaWarp = kEpiWarps + 1;
  static constexpr int kWProdWarp = kEpiWarps + 2;
  static constexpr int kUnpackWarp0 = kEpiWarps + 3;
  static constexpr int kFwdWarp = kUnpackWarp0 + 4 * kUnpackGroups;
  static constexpr int kThreads = 32 * (kFwdWarp + (kForwarder ? 1 : 0));
};
constexpr int kTT = 64;                 // times per tile
constexpr int kBM = 128;                // GEMM rows per tile
constexpr int kKC = 128;                // K bytes per TMA box / swizzle atom (64 dishes x re/im)
constexpr int kSub = 2;                 // boxes per pipeline stage
constexpr int kStageK = kSub * kKC;     // K bytes per stage (128 dishes x re/im): 8 MMAs
static_assert(kSub == 2, "mma_ts_stage8 issues the eight MMAs of two W boxes");
constexpr int kRawBox = kTT * kKC;      // raw E per box: 64 times x 64 dishes x 2 pol
constexpr int kRawBytes = kSub * kRawBox;
constexpr int kAccCols = 256;           // TMEM column offset of the second accumulator
// Beam passes of at most kHalfPass beams run the half-SM layout: 4 epilogue
// warps, 256 TMEM columns (second accumulator at column 128) and at most
// kSmemLimitHalf bytes of shared memory, so that two CTAs share each SM and
// each SM has two MMA issuers, two unpack chains and two epilogues.
constexpr int kAccColsHalf = 128;
constexpr int kSmemLimitHalf = 115712;  // half of the SM's 228 KiB less the 1 KiB each block reserves
constexpr int kStageCols = kStageK / 4;  // TMEM columns per unpacked stage
constexpr int kSmemLimit = 232448;      // 227 KiB opt-in per block
constexpr int kMaxStages = 8;
constexpr int kDigSlots = 2;            // digit-row slots (one per tile in flight)
// Offset correction: one extra MMA per tile, issued first (it also clears the
// accumulator), multiplies a constant A tile by the tile's digit rows.  The
// constant row holds -2^-6, -2^-2, -4, -64, -256 at K = 0..4 (again at 16..20,
// so the 32-byte swizzle cannot move them), the digit row of n holds d0..d3 and
// 4 d4 with sum_k W[n][k] = d0 + 16 d1 + 256 d2 + 4096 d3 + 65536 d4, so the
// accumulator starts at -sum_k W[n][k] / 64 = -8 sum_k W[n][k] / 512 exactly.
constexpr uint32_t kDigitScaleLo = 0xE8C8A888u;  // E4M3 -2^-6, -2^-2, -4, -64
constexpr uint32_t kDigitScaleHi = 0x000000F8u;  // E4M3 -256
constexpr int kConstABytes = kBM * kDigitRow;
constexpr int kMaxWSlots = 6;
constexpr int kMinRaw = 4;
constexpr int kMaxRaw = 16;


struct TcParams {
  TcProblem one;            // the problem of a plain launch
  const TcProblem *table;   // grouped launch: nprob problems in device memory, by tile_begin
  int nprob;
  int ntiles;
  int nk;                   // K stages per tile (every problem has the same dishes)
  int max_nb_pass;          // sizes the W slots, gain buffers and TMEM layout
  int stages;               // unpacked-operand stages in TMEM
  int wslots;               // W slots in smem
  int raw;                  // raw E slots in smem
  int test_stall;           // nonzero: the producers issue nothing (failure-path test)
  int groups;               // unpack groups (2: with the W forwarder; needs stages >= 4)
  int half;                 // nonzero: the half-SM layout (two CTAs per SM)
  int *err;
};

// Tiles of a CTA.  A plain launch strides them over the grid.  A grouped
// launch gives each CTA a contiguous range, so that it stays with one problem
// for many tiles: every change of problem costs each role a tensor-map
// acquire and a cold descriptor, and with strided tiles almost every tile of
// a large batch belongs to another problem.
struct TileRange {
  int first, end, step;
  template <bool kGrouped>
  __device__ __forceinline__ static TileRange of(const TcParams &p) {
    if constexpr (kGrouped) {
      const int64_t n = p.ntiles, g = gridDim.x, b = blockIdx.x;
      return {static_cast<int>(b * n / g), static_cast<int>((b + 1) * n / g), 1};
    } else {
      return {static_cast<int>(blockIdx.x), p.ntiles, static_cast<int>(gridDim.x)};
    }
  }
  __device__ __forceinline__ uint32_t count() const {
    return first < end ? static_cast<uint32_t>((end - 1 - first) / step + 1) : 0u;
  }
};

// Problem of a tile and the tile's index inside it; a CTA's tiles only grow,
// so a grouped launch walks the table forward from the last problem seen.
template <bool kGrouped>
struct ProblemCursor {
  int idx = -1;
  __device__ __forceinline__ const TcProblem &at(const TcParams &p, int tile, int &lt) {
    if constexpr (!kGrouped) {
      lt = tile;
      return p.one;
    } else {
      if (idx < 0) {  // first tile: binary search
        int lo = 0, hi = p.nprob - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (p.table[mid].tile_begin <= tile) lo = mid; else hi = mid - 1;
        }
        idx = lo;
      }
      while (idx + 1 < p.nprob && p.table[idx + 1].tile_begin <= tile) ++idx;
      lt = tile - p.table[idx].tile_begin;
      return p.table[idx];
    }
  }
};

// Coordinates (beam pass, 64-time block, frequency) of a CTA's tiles.  A plain
// launch visits tiles blockIdx.x, + gridDim.x, ...: the cursor adds the grid
// size in the same mixed radix (npass, ntt, F) instead of dividing by the
// run-time sizes for every tile (two divisions cost ~40 instructions, and
// every role of the CTA pays them).  A grouped launch may change problem from
// one tile to the next, so it divides.
struct TileCursor {
  int pass = 0, tt = 0, f = 0;  // current tile (plain launches)
  int dp = 0, dt = 0, df = 0;   // gridDim.x in the same radix
  template <bool kGrouped>
  __device__ __forceinline__ void start(const TcParams &p) {
    if constexpr (!kGrouped) {
      const int np = p.one.npass, nt = p.one.ntt;
      const int b = static_cast<int>(blockIdx.x), g = static_cast<int>(gridDim.x);
      pass = b % np;
      tt = (b / np) % nt;
      f = b / (np * nt);
      dp = g % np;
      dt = (g / np) % nt;
      df = g / (np * nt);
    }
  }
  // Coordinates of tile lt of problem P; then steps to the CTA's next tile.
  template <bool kGrouped>
  __device__ __forceinline__ void take(const TcProblem &P, int lt, int &pass_, int &tt_, int &f_) {
    if constexpr (kGrouped) {
      pass_ = lt % P.npass;
      tt_ = (lt / P.npass) % P.ntt;
      f_ = lt / (P.npass * P.ntt);
    } else {
      pass_ = pass;
      tt_ = tt;
      f_ = f;
      pass += dp;
      int c = pass >= P.npass;
      pass -= c ? P.npass : 0;
      tt += dt + c;
      c = tt >= P.ntt;
      tt -= c ? P.ntt : 0;
      f += df + c;
    }
  }
};

struct SmemPlan {
  int wbox, wbytes, dbytes;
  int off_w, off_a, off_d, off_r, off_bar, nbar, total;
};

__host__ __device__ inline SmemPlan smem_plan(int stages, int wslots, int raw, int nb_pass) {
  SmemPlan s{};
  s.wbox = 2 * nb_pass * kKC;
  s.wbytes = kSub * s.wbox;
  s.dbytes = (2 * nb_pass * kDigitRow + 1023) / 1024 * 1024;
  s.off_w = 0;
  s.off_a = s.off_w + wslots * s.wbytes;  // constant A tile of the offset MMA
  s.off_d = s.off_a + kConstABytes;       // digit-row slots
  s.off_r = s.off_d + kDigSlots * s.dbytes;
  s.off_bar = s.off_r + raw * kRawBytes;
  // raw_full[R], raw_empty[R], w_full[SW], w_empty[SW], a_full[S], empty[S], accfull[2], accempty[2],
  // d_full[2], d_empty[2]
  s.nbar = 2 * raw + 2 * wslots + 2 * stages + 4 + 2 * kDigSlots;
  s.total = s.off_bar + 8 * s.nbar + 16;
  return s;
}

// TMEM column of unpacked stage i: the columns left over after the two accumulators.
__host__ __device__ inline uint32_t stage_col(int i, int ncols, int per_half, int acc_cols) {
  return i < per_half ? static_cast<uint32_t>(ncols + kStageCols * i)
                      : static_cast<uint32_t>(acc_cols + ncols + kStageCols * (i - per_half));
}

// Position in a ring of n slots: slot index and the parity of the pass over the ring.
struct Ring {
  uint32_t idx = 0, phase = 0, n;
  __device__ explicit Ring(int n_) : n(static_cast<uint32_t>(n_)) {}
  __device__ __forceinline__ void advance() {
    if (++idx == n) {
      idx = 0;
      phase ^= 1u;
    }
  }
};

__device__ __forceinline__ uint32_t prmt(uint32_t a, uint32_t b, uint32_t sel) {
  uint32_t r;
  asm("prmt.b32 %0, %1, %2, %3;" : "=r"(r) : "r"(a), "r"(b), "r"(sel));
  return r;
}

// (c << 8) | (sat4(re) << 4) | sat4(im): two integers saturated to [-8, 7] and
// packed as the nibbles of one byte below the bytes of c.
__device__ __forceinline__ uint32_t pack_s4x2(int re, int im, uint32_t c) {
  uint32_t r;
  asm("cvt.pack.sat.s4.s32.b32 %0, %1, %2, %3;" : "=r"(r) : "r"(re), "r"(im), "r"(c));
  return r;
}

// Byte offset of 16-byte chunk j of row r in a 128B-swizzled tile (TMA layout).
__device__ __forceinline__ uint32_t sw128_offset(uint32_t r, uint32_t j) {
  return (r >> 3) * 1024u + (r & 7u) * 128u + ((j ^ (r & 7u)) << 4);
}

template <bool kGrouped, bool kJ2, int kEpiW, bool kAdler, int kGroups, bool kHalf>
__global__ void __launch_bounds__(Roles<kEpiW, kGroups>::kThreads, kHalf ? 2 : 1)
    bf_form_beams_tc(const __grid_constant__ TcParams p) {
  using RL = Roles<kEpiW, kGroups>;
  constexpr int kAcc = kHalf ? kAccColsHalf : kAccCols;  // TMEM column of the second accumulator
  constexpr int kEpiThreads = RL::kEpiThreads, kEpiParts = RL::kEpiParts, kEProdWarp = RL::kEProdWarp;
  constexpr int kMmaWarp = RL::kMmaWarp, kWProdWarp = RL::kWProdWarp, kUnpackWarp0 = RL::kUnpackWarp0;
  constexpr int kUnpackGroups = RL::kUnpackGroups;
  extern __shared__ uint8_t smem_dyn[];
  uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_dyn) + 1023) & ~uintptr_t(1023));
  const int S = p.stages, SW = p.wslots, R = p.raw;
  const SmemPlan sp = smem_plan(S, SW, R, p.max_nb_pass);
  uint8_t *sW = smem + sp.off_w;
  uint8_t *sA = smem + sp.off_a;
  uint8_t *sD = smem + sp.off_d;
  uint8_t *sR = smem + sp.off_r;
  const uint32_t bar0 = smem_u32(smem + sp.off_bar);
  auto raw_full = [&](int r) { return bar0 + 8u * r; };
  auto raw_empty = [&](int r) { return bar0 + 8u * (R + r); };
  auto w_full = [&](int s) { return bar0 + 8u * (2 * R + s); };
  auto w_empty = [&](int s) { return bar0 + 8u * (2 * R + SW + s); };
  auto a_full = [&](int s) { return bar0 + 8u * (2 * R + 2 * SW + s); };
  auto empty = [&](int s) { return bar0 + 8u * (2 * R + 2 * SW + S + s); };
  auto accfull = [&](int i) { return bar0 + 8u * (2 * R + 2 * SW + 2 * S + i); };
  auto accempty = [&](int i) { return bar0 + 8u * (2 * R + 2 * SW + 2 * S + 2 + i); };
  auto d_full = [&](int i) { return bar0 + 8u * (2 * R + 2 * SW + 2 * S + 4 + i); };
  auto d_empty = [&](int i) { return bar0 + 8u * (2 * R + 2 * SW + 2 * S + 4 + kDigSlots + i); };
  uint32_t *tmem_holder = reinterpret_cast<uint32_t *>(smem + sp.off_bar + 8 * sp.nbar);

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int ncols = 2 * p.max_nb_pass;                 // accumulator columns reserved (largest GEMM N)
  const int per_half = (kAcc - ncols) / kStageCols;  // unpacked stages beside each accumulator

  if (threadIdx.x == 0) {
    for (int r = 0; r < R; ++r) {
      mbar_init(raw_full(r), 1);
      mbar_init(raw_empty(r), 128);
    }
    for (int s = 0; s < SW; ++s) {
      mbar_init(w_full(s), 1);
      mbar_init(w_empty(s), 1);
    }
    for (int s = 0; s < S; ++s) {
      mbar_init(a_full(s), 128 + (RL::kForwarder ? 1 : 0));  // one unpack group (+ the W forwarder)
      mbar_init(empty(s), 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(accfull(i), 1);
      mbar_init(accempty(i), kEpiThreads);
    }
    for (int i = 0; i < kDigSlots; ++i) {
      mbar_init(d_full(i), 1);
      mbar_init(d_empty(i), 1);
    }
    fence_barrier_init();
  }
  // constant A tile of the offset MMA: every row the same, so the 32-byte
  // swizzle leaves it unchanged
  for (int i = threadIdx.x; i < kConstABytes / 4; i += blockDim.x) {
    const int w = i & 7;
    reinterpret_cast<uint32_t *>(sA)[i] = (w == 0 || w == 4) ? kDigitScaleLo : (w == 1 || w == 5) ? kDigitScaleHi : 0u;
  }
  fence_proxy_async_smem();
  if (warp == kMmaWarp) {
    tmem_alloc(smem_u32(tmem_holder), 2 * kAcc);
    tmem_relinquish();
  }
  if (!kGrouped && warp == kEProdWarp && lane == 0) {
    tma_prefetch_desc(&p.one.tm_e);
    tma_prefetch_desc(&p.one.tm_w);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = *tmem_holder;
  int *err = p.err;

  if (warp == kEProdWarp) {
    // ------------------------------------------------------------ E producer
    if (lane == 0 && !p.test_stall) {
      const uint64_t pol_e = policy_evict_first();
      Ring rr(R);
      uint32_t issued = 0;
      bool ok = true;
      const TcProblem *seen = nullptr;
      TileCursor cur;
      cur.start<kGrouped>(p);
      const TileRange tr = TileRange::of<kGrouped>(p);
      ProblemCursor<kGrouped> pc;
      for (int tile = tr.first; ok && tile < tr.end; tile += tr.step) {
        int lt;
        const TcProblem &P = pc.at(p, tile, lt);
        if (kGrouped && &P != seen) {  // a table entry the host rewrites between launches
          tensormap_acquire(&P.tm_e);
          seen = &P;
        }
        int pass, tt, f;
        cur.take<kGrouped>(P, lt, pass, tt, f);
        (void)pass;
        for (int ks = 0; ks < p.nk; ++ks, rr.advance(), ++issued) {
          const int r = static_cast<int>(rr.idx);
          if (!mbar_wait(raw_empty(r), rr.phase ^ 1u, err, kDevTimeoutEmpty)) {
            ok = false;
            break;
          }
          mbar_arrive_expect_tx(raw_full(r), kRawBytes);
#pragma unroll
          for (int h = 0; h < kSub; ++h)
            tma_load_3d(smem_u32(sR + r * kRawBytes + h * kRawBox), &P.tm_e, raw_full(r), (ks * kSub + h) * kKC, f,
                        tt * kTT, pol_e);
        }
      }
      // Let the copies already issued land before the CTA exits.  Also when
      // this thread saw no error: another role's error can end the consumers
      // before they waited for the last copies.  On a clean run these waits
      // return at once.
      for (uint32_t k = (issued >= static_cast<uint32_t>(R) ? issued - R : 0); k < issued; ++k)
        mbar_wait_drain(raw_full(static_cast<int>(k % R)), (k / R) & 1u);
    }
  } else if (warp == kWProdWarp) {
    // ------------------------------------------------------------ W producer
    if (lane == 0 && !p.test_stall) {
      const uint64_t pol_w = policy_evict_last();
      Ring wr(SW), dr(kDigSlots);
      uint32_t it = 0, dit = 0;
      bool ok = true;
      const TcProblem *seen = nullptr;
      TileCursor cur;
      cur.start<kGrouped>(p);
      const TileRange tr = TileRange::of<kGrouped>(p);
      ProblemCursor<kGrouped> pc;
      for (int tile = tr.first; ok && tile < tr.end; tile += tr.step) {
        int lt;
        const TcProblem &P = pc.at(p, tile, lt);
        if (kGrouped && &P != seen) {  // a table entry the host rewrites between launches
          tensormap_acquire(&P.tm_w);
          tensormap_acquire(&P.tm_d);
          seen = &P;
        }
        int pass, tt, f;
        cur.take<kGrouped>(P, lt, pass, tt, f);
        (void)tt;
        const int wbox = 2 * P.nb_pass * kKC;
        {  // the tile's digit rows, for the offset MMA
          const int ds = static_cast<int>(dr.idx);
          if (!mbar_wait(d_empty(ds), dr.phase ^ 1u, err, kDevTimeoutEmpty)) {
            ok = false;
            break;
          }
          mbar_arrive_expect_tx(d_full(ds), 2 * P.nb_pass * kDigitRow);
          tma_load_3d(smem_u32(sD + ds * sp.dbytes), &P.tm_d, d_full(ds), 0, pass * 2 * P.nb_pass, f, pol_w);
          dr.advance();
          ++dit;
        }
        for (int ks = 0; ks < p.nk; ++ks, ++it, wr.advance()) {
          const int s = static_cast<int>(wr.idx);
          if constexpr (RL::kForwarder) {
            // the slot held sequence it - SW: free once the tensor core finished
            // that stage (its commit on empty).  SW <= S, so the stage's next use
            // (sequence it - SW + S) is not loaded yet and the barrier cannot be a
            // phase past the one waited for.
            if (it >= static_cast<uint32_t>(SW)) {
              const uint32_t j = it - static_cast<uint32_t>(SW);
              if (!mbar_wait(empty(static_cast<int>(j % static_cast<uint32_t>(S))), (j / static_cast<uint32_t>(S)) & 1u,
                             err, kDevTimeoutEmpty)) {
                ok = false;
                break;
              }
            }
          } else if (!mbar_wait(w_empty(s), wr.phase ^ 1u, err, kDevTimeoutEmpty)) {
            ok = false;
            break;
          }
          mbar_arrive_expect_tx(w_full(s), kSub * wbox);
#pragma unroll
          for (int h = 0; h < kSub; ++h)
            tma_load_3d(smem_u32(sW + s * sp.wbytes + h * wbox), &P.tm_w, w_full(s), (ks * kSub + h) * kKC,
                        pass * 2 * P.nb_pass, f, pol_w);
        }
      }
      // as in the E producer: drain on every exit, not only after an own error
      for (uint32_t k = (it >= static_cast<uint32_t>(SW) ? it - SW : 0); k < it; ++k)
        mbar_wait_drain(w_full(static_cast<int>(k % SW)), (k / SW) & 1u);
      for (uint32_t k = (dit >= static_cast<uint32_t>(kDigSlots) ? dit - kDigSlots : 0); k < dit; ++k)
        mbar_wait_drain(d_full(static_cast<int>(k % kDigSlots)), (k / kDigSlots) & 1u);
    }
  } else if (warp == kMmaWarp) {
    // ------------------------------------------------------------ MMA issuer
    if (lane == 0) {
      Ring ar(S), wr(SW), dr(kDigSlots);
      const uint64_t a_const = smem_desc_sw32(smem_u32(sA));
      const uint64_t w_desc0 = smem_desc_sw128(smem_u32(sW));
      uint32_t local = 0;
      uint32_t nstage = 0, ndig = 0, nacc = 0;  // commits issued on empty, d_empty, accfull
      bool ok = true;
      const TileRange tr = TileRange::of<kGrouped>(p);
      ProblemCursor<kGrouped> pc;
      for (int tile = tr.first; ok && tile < tr.end; tile += tr.step, ++local) {
        int lt;
        const TcProblem &P = pc.at(p, tile, lt);
        const uint32_t idesc = idesc_e4m3_f32(kBM, 2 * P.nb_pass);
        const int wbox = 2 * P.nb_pass * kKC;
        const uint32_t ab = local & 1u;
        const uint32_t aph = (local >> 1) & 1u;
        if (!mbar_wait(accempty(ab), aph ^ 1u, err, kDevTimeoutAccEmpty)) break;
        const int ds = static_cast<int>(dr.idx);
        if (!mbar_wait(d_full(ds), dr.phase, err, kDevTimeoutFull)) break;
        tc_fence_after();
        const uint32_t d_tmem = tmem_base + ab * kAcc;
        // the offset MMA starts the accumulator at -8 sum_k W[n][k] / 512
        mma_f8f6f4(d_tmem, a_const, smem_desc_sw32(smem_u32(sD + ds * sp.dbytes)), idesc, 0u);
        mma_commit(d_empty(ds));
        ++ndig;
        dr.advance();
        for (int ks = 0; ks < p.nk; ++ks, ar.advance(), wr.advance()) {
          const int s = static_cast<int>(ar.idx);
          const int sw = static_cast<int>(wr.idx);
          // the unpack arrives on a_full only once this stage's W slot has landed too
          if (!mbar_wait(a_full(s), ar.phase, err, kDevTimeoutUnpacked)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t a_tmem = tmem_base + stage_col(s, ncols, per_half, kAcc);
          const uint64_t b_desc = w_desc0 + static_cast<uint64_t>((sw * sp.wbytes) >> 4);
          mma_ts_stage8(d_tmem, a_tmem, b_desc, b_desc + static_cast<uint64_t>(wbox >> 4), idesc);
          mma_commit(empty(s));  // also frees the W slot: the unpack passes it on
          ++nstage;
        }
        if (!ok) break;
        mma_commit(accfull(ab));
        ++nacc;
      }
      // A commit's arrival is an asynchronous write into this CTA's shared
      // memory, and nothing waits for the last ones on each stage and digit
      // slot: wait for the last phase committed on every barrier (bounded)
      // before the CTA can exit.  On the error path this also lets the MMAs
      // already issued finish before the tensor memory is freed.
      const uint32_t uS = static_cast<uint32_t>(S), uD = static_cast<uint32_t>(kDigSlots);
      for (uint32_t k = nstage > uS ? nstage - uS : 0; k < nstage; ++k)
        mbar_wait_drain(empty(static_cast<int>(k % uS)), (k / uS) & 1u);
      for (uint32_t k = ndig > uD ? ndig - uD : 0; k < ndig; ++k)
        mbar_wait_drain(d_empty(static_cast<int>(k % uD)), (k / uD) & 1u);
      for (uint32_t k = nacc > 2u ? nacc - 2u : 0u; k < nacc; ++k)
        mbar_wait_drain(accfull(static_cast<int>(k & 1u)), (k >> 1) & 1u);
    }
  } else if (RL::kForwarder && warp == RL::kFwdWarp) {
    // ------------------------------------------------------------ W forwarder
    // Sequence it's a_full gets one arrival from here once its W slot has
    // landed, after the previous use of that a_full slot (it - S) completed.
    if (lane == 0 && !p.test_stall) {
      const uint32_t total = TileRange::of<kGrouped>(p).count() * static_cast<uint32_t>(p.nk);
      const uint32_t uS = static_cast<uint32_t>(S), uSW = static_cast<uint32_t>(SW);
      for (uint32_t it = 0; it < total; ++it) {
        if (!mbar_wait(w_full(static_cast<int>(it % uSW)), (it / uSW) & 1u, err, kDevTimeoutFull)) break;
        if (it >= uS &&
            !mbar_wait(a_full(static_cast<int>((it - uS) % uS)), ((it - uS) / uS) & 1u, err, kDevTimeoutUnpacked))
          break;
        mbar_arrive(a_full(static_cast<int>(it % uS)));
      }
    }
  } else if (warp >= kUnpackWarp0) {
    // ------------------------------------------------------------ unpack
    // Group g takes the K stages with it % kUnpackGroups == g.  Lane pair
    // (2u, 2u+1) of quarter q holds rows (t, p=0) and (t, p=1) of time
    // t = 16q + u: both lanes read the raw row and keep their polarization.
    const int group = (warp - kUnpackWarp0) >> 2;
    const int q = warp & 3;
    const uint32_t pp = lane & 1u;
    const uint32_t tl = 16u * q + (lane >> 1);
    const uint32_t lane_addr = static_cast<uint32_t>(32 * q) << 16;
    const uint32_t sel = pp ? 0x7531u : 0x6420u;  // odd or even bytes: polarization 1 or 0
    // this CTA's K stages: its tiles (TileRange) times nk
    const uint32_t my_tiles = TileRange::of<kGrouped>(p).count();
    const uint32_t total = my_tiles * static_cast<uint32_t>(p.nk);
    // W slots: the tensor core's release of an operand stage (empty) also ends
    // its use of that stage's W slot, so the lead lane of the group handling
    // sequence it frees the W slot of sequence it - S when it sees the stage
    // free, and waits for the W slot of sequence it before its a_full arrival.
    // With SW >= S (the planner's rule) the releases of each slot come in
    // order for any number of groups: the release of sequence j precedes the
    // a_full arrival of j + S, and the next use of its slot, j + SW, is
    // released only after the tensor core consumed j + SW >= j + S.
    const bool wlead = warp == kUnpackWarp0 + 4 * group && lane == 0;
    Ring rr(R), ar(S), wr(SW);
    int relslot = ((group - S) % SW + SW) % SW;  // W slot of sequence it - S
    for (int g = 0; g < group; ++g) {
      rr.advance();
      ar.advance();
      wr.advance();
    }
    bool ok = true;
    for (uint32_t it = group; ok && it < total; it += kUnpackGroups) {
      {
        const int r = static_cast<int>(rr.idx);
        const int s = static_cast<int>(ar.idx);
        if (!__all_sync(0xffffffffu, mbar_wait(raw_full(r), rr.phase, err, kDevTimeoutFull))) {
          ok = false;  // the warp leaves together
          break;
        }
        const uint32_t col = tmem_base + lane_addr + stage_col(s, ncols, per_half, kAcc);
        // the whole stage goes to registers first, so that only the tensor-memory
        // stores wait for the tensor core to release the stage
        uint32_t out[kSub][32];
#pragma unroll
        for (int h = 0; h < kSub; ++h) {
          const uint8_t *raw = sR + r * kRawBytes + h * kRawBox;
          uint32_t e[16];  // this lane's polarization, dishes 4m..4m+3 of the box in word m
#pragma unroll
          for (uint32_t j = 0; j < 8; ++j) {
            // 16-byte chunk j: dishes 8j..8j+7, bytes [d0p0 d0p1 d1p0 d1p1 ...]
            const uint4 w = *reinterpret_cast<const uint4 *>(raw + sw128_offset(tl, j));
            e[2 * j] = prmt(w.x, w.y, sel);
            e[2 * j + 1] = prmt(w.z, w.w, sel);
          }
          const uint32_t msk = 0x0F0F0F0Fu;
#pragma unroll
          for (int m = 0; m < 16; ++m) {
            out[h][2 * m] = (e[m] >> 4) & msk;  // real nibbles u (E4M3 bytes = u * 2^-9)
            out[h][2 * m + 1] = e[m] & msk;     // imaginary nibbles
          }
        }
        // the raw slot is in registers now; the next TMA into it is an async-proxy
        // write after these generic reads, so order them across proxies first
        fence_proxy_async_smem();
        mbar_arrive(raw_empty(r));
        if (!__all_sync(0xffffffffu, mbar_wait(empty(s), ar.phase ^ 1u, err, kDevTimeoutEmpty))) {
          ok = false;
          break;
        }
        // the stores first: the W-slot hand-over runs while they drain
#pragma unroll
        for (int h = 0; h < kSub; ++h) tmem_st_32x32b_x32(col + 32 * h, out[h]);
        if constexpr (!RL::kForwarder) {
          if (it >= static_cast<uint32_t>(S) && wlead) mbar_arrive(w_empty(relslot));  // sequence it - S is done
          if (wlead && !mbar_wait(w_full(static_cast<int>(wr.idx)), wr.phase, err, kDevTimeoutFull)) ok = false;
        }
        tmem_st_wait();
        if (!__all_sync(0xffffffffu, ok)) break;
        tc_fence_before();
        mbar_arrive(a_full(s));
      }
#pragma unroll
      for (int g = 0; g < kUnpackGroups; ++g) {
        rr.advance();
        ar.advance();
        wr.advance();
        relslot = relslot + 1 == SW ? 0 : relslot + 1;
      }
    }
  } else {
    // ------------------------------------------------------------ epilogue
    // Warp w reads TMEM lane quarter w % 4 (times 16q..16q+15, both
    // polarizations interleaved by lane) and column part w / 4.
    const int q = warp & 3;
    const int part = warp >> 2;
    const uint32_t pol = lane & 1u;
    const uint32_t lane_addr = static_cast<uint32_t>(32 * q) << 16;

    // The warps of the epilogue share no barrier: each reads its chunks' gains
    // straight from the scaled-gain rows gs = 512 * G (L1-resident) and waits for
    // the accumulator on its own, so a slow warp does not hold up the others.
    uint32_t local = 0;
    // fused adler32 (kAdler): this lane's sums of the J bytes it stores,
    // sum d_i and sum i d_i with the byte position i taken mod 65521
    unsigned long long ad_s1 = 0, ad_s2 = 0;
    TileCursor cur;
    cur.start<kGrouped>(p);
    const TileRange tr = TileRange::of<kGrouped>(p);
    ProblemCursor<kGrouped> pc;
    for (int tile = tr.first; tile < tr.end; tile += tr.step, ++local) {
      int lt;
      const TcProblem &P = pc.at(p, tile, lt);
      int pass, tt, f;
      cur.take<kGrouped>(P, lt, pass, tt, f);
      const int nchunk = P.nb_pass / 8;
      const int c_begin = part * nchunk / kEpiParts, c_end = (part + 1) * nchunk / kEpiParts;
      const uint32_t ab = local & 1u;
      const uint32_t aph = (local >> 1) & 1u;
      const int b0 = pass * P.nb_pass;
      // 512 * G[f][b0 ..] (zero beyond B): the accumulator ends at raw / 512
      // exactly and the power-of-two scaling is exact, so (512 G) * (raw / 512)
      // rounds like G * raw (cpu.cxx:37)
      const float *gcur = P.gs + static_cast<int64_t>(f) * P.npass * P.nb_pass + b0;
      // huge or non-finite gains of this frequency: requantise with the
      // narrowing of cpu.cxx:38 (tile-uniform branch, normally not taken)
      const bool wide = __ldg(P.gwide + f) != 0;
      if (!__all_sync(0xffffffffu, mbar_wait(accfull(ab), aph, err, kDevTimeoutAccFull))) break;
      tc_fence_after();
      const uint32_t acc_addr = tmem_base + ab * kAcc + lane_addr;
      // A 4x4 byte transpose among 4 lanes turns "4 beams of one row" into "4
      // rows of one beam" in each lane.  Jlinear (arraysizes.hxx:92): the 4 lanes
      // of equal polarization and consecutive times (lane bits 1 and 2) exchange,
      // and a lane stores J[b][f][p][t..t+3].  J2linear (arraysizes.hxx:103): 4
      // consecutive rows (t, p), (t, p+1), (t+1, p), (t+1, p+1) (lane bits 0 and
      // 1) exchange, and a lane stores those 4 bytes of J2[b][f][t][p].
      constexpr bool j2 = kJ2;
      const uint32_t j4 = j2 ? (lane & 3u) : ((lane >> 1) & 3u);  // place among the 4 = beam offset after
      const int xd1 = j2 ? 1 : 2, xd2 = j2 ? 2 : 4;
      const uint32_t sel1 = (j4 & 1) ? 0x3715u : 0x6240u;
      const uint32_t sel2 = (j4 & 2) ? 0x3276u : 0x5410u;
      const int64_t bj = static_cast<int64_t>(b0 + static_cast<int>(j4)) * P.F + f;  // beam row b0 + j4
      int64_t t;      // first time of the lane's 4 bytes
      uint8_t *jrow;  // the lane's bytes for beam b0 + j4
      if (!j2) {
        t = static_cast<int64_t>(tt) * kTT + 16 * q + 4 * (lane >> 3);
        jrow = P.J + (bj * 2 + pol) * P.jpitch + t;
      } else {
        const int r0 = 32 * q + static_cast<int>(lane & ~3u);  // first of the 4 rows in the tile
        t = static_cast<int64_t>(tt) * kTT + r0 / 2;
        jrow = P.J + bj * 2 * P.jpitch + 2 * static_cast<int64_t>(tt) * kTT + r0;
      }
      const bool t_ok = t < P.T;
      const int64_t bstride = static_cast<int64_t>(P.F) * 2 * P.jpitch;  // bytes between beams, both layouts
      const int blim = P.B - b0 - static_cast<int>(j4);  // beam offsets below this exist
      uint8_t *dst = jrow + static_cast<int64_t>(8 * c_begin) * bstride;  // beam 8 c + j4 of the lane's chunk c
      // fused adler32: word h of the lane's chunk c_begin + cc sits at byte
      // position base + cc * step + h * half (mod 65521), so the tile needs only
      // a0 = sum of its bytes, a1 = sum cc * (bytes of chunk cc), a2 = sum of the
      // second words' bytes, a3 = sum k * byte_k within words; then
      // sum i d_i = base a0 + step a1 + half a2 + a3 (32-bit sums per tile:
      // bytes <= 255, at most 16 words; the products are taken in 64 bits)
      uint32_t ad_a0 = 0, ad_a1 = 0, ad_a2 = 0, ad_a3 = 0;

      auto process = [&](int c, const uint32_t (&r)[16]) {
        const float4 ga = __ldg(reinterpret_cast<const float4 *>(gcur + 8 * c));
        const float4 gb = __ldg(reinterpret_cast<const float4 *>(gcur + 8 * c + 4));
        const float gv[8] = {ga.x, ga.y, ga.z, ga.w, gb.x, gb.y, gb.z, gb.w};
        // clamp(lrint(G * raw), -7, 7) with acc = raw / 512 exactly: one IEEE
        // multiply, the lower clamp (to -7.25: same result after rounding), a
        // round-half-even conversion, and the upper clamp by the saturating pack
        int qre[8], qim[8];
        if (!wide) {
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            qre[i] = __float2int_rn(fmaxf(__fmul_rn(gv[i], __uint_as_float(r[i])), -7.25f));
            qim[i] = __float2int_rn(fmaxf(__fmul_rn(gv[i], __uint_as_float(r[8 + i])), -7.25f));
          }
        } else {
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            qre[i] = requant_narrow(__fmul_rn(gv[i], __uint_as_float(r[i])));
            qim[i] = requant_narrow(__fmul_rn(gv[i], __uint_as_float(r[8 + i])));
          }
        }
        // ucomplex4 bytes of beams 0-3 and 4-7 for this lane's time
        uint32_t w[2];
#pragma unroll
        for (int h2 = 0; h2 < 2; ++h2) {
          uint32_t x = 0;
#pragma unroll
          for (int j = 3; j >= 0; --j) x = pack_s4x2(qre[4 * h2 + j], qim[4 * h2 + j], x);
          x ^= 0x88888888u;  // byte j = ucomplex4 of beam 4 * h2 + j (icomplex4.hxx:33)
          const uint32_t x1 = prmt(x, __shfl_xor_sync(0xffffffffu, x, xd1), sel1);
          w[h2] = prmt(x1, __shfl_xor_sync(0xffffffffu, x1, xd2), sel2);  // beam 4*h2 + j4, the 4 rows
        }
        if (t_ok) {
          if (8 * c < blim) __stcs(reinterpret_cast<uint32_t *>(dst), w[0]);
          if (8 * c + 4 < blim) __stcs(reinterpret_cast<uint32_t *>(dst + 4 * bstride), w[1]);
        }
        if constexpr (kAdler) {  // only the bytes stored count
          const uint32_t w0 = (t_ok && 8 * c < blim) ? w[0] : 0u;
          const uint32_t w1 = (t_ok && 8 * c + 4 < blim) ? w[1] : 0u;
          const uint32_t s1 = __dp4a(w1, 0x01010101u, 0u);
          const uint32_t s01 = __dp4a(w0, 0x01010101u, s1);
          ad_a0 += s01;
          ad_a1 += static_cast<uint32_t>(c - c_begin) * s01;
          ad_a2 += s1;
          ad_a3 = __dp4a(w1, 0x03020100u, __dp4a(w0, 0x03020100u, ad_a3));
        }
        dst += 8 * bstride;
      };

      // accumulator columns in chunks of 16, the next chunk's TMEM load in flight
      uint32_t ra[16], rb[16];
      if (c_begin < c_end) {
        tmem_ld_32x32b_x16(acc_addr + 16u * c_begin, ra);
        tmem_ld_wait(ra);
      }
      for (int c = c_begin; c < c_end; c += 2) {
        const bool has1 = c + 1 < c_end, has2 = c + 2 < c_end;
        if (has1) tmem_ld_32x32b_x16(acc_addr + 16u * (c + 1), rb);
        process(c, ra);
        if (has1) {
          tmem_ld_wait(rb);
          if (has2) tmem_ld_32x32b_x16(acc_addr + 16u * (c + 2), ra);
          process(c + 1, rb);
          if (has2) tmem_ld_wait(ra);
        }
      }
      tc_fence_before();
      mbar_arrive(accempty(ab));
      if constexpr (kAdler) {
        const uint64_t off = static_cast<uint64_t>((jrow + static_cast<int64_t>(8 * c_begin) * bstride) - P.jbase);
        const uint32_t base = static_cast<uint32_t>(off % kAdlerMod);
        const uint32_t half = static_cast<uint32_t>(static_cast<uint64_t>(4 * bstride) % kAdlerMod);
        const uint32_t step = static_cast<uint32_t>(static_cast<uint64_t>(8 * bstride) % kAdlerMod);
        ad_s1 += ad_a0;
        ad_s2 += static_cast<unsigned long long>(base) * ad_a0 + static_cast<unsigned long long>(step) * ad_a1 +
                 static_cast<unsigned long long>(half) * ad_a2 + ad_a3;
      }
    }
    if constexpr (kAdler) {  // one pair of atomics per warp
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        ad_s1 += __shfl_xor_sync(0xffffffffu, ad_s1, o);
        ad_s2 += __shfl_xor_sync(0xffffffffu, ad_s2, o);
      }
      if (lane == 0) {
        const TcProblem &P0 = p.one;
        atomicAdd(P0.adler, ad_s1);
        atomicAdd(P0.adler + 1, ad_s2);
      }
    }
  }

  tc_fence_before();
  __syncthreads();
  if (warp == kMmaWarp) {
    tc_fence_after();
    tmem_dealloc(tmem_base, 2 * kAcc);
  }
}

// Builds the E4M3 operand W[f][n][k] and the digit rows of the row sums
// sum_k W[f][n][k] from A[f][b][d]; one warp per row n, four k per lane-step.
//   n = 16*(b/8) + 8*cj + b%8      (cj: 0 = real output, 1 = imaginary output)
//   k = 8*(d/4)  + 4*c  + d%4      (c:  0 = real input,  1 = imaginary input)
// W = Ar, -Ai for the real output and Ai, Ar for the imaginary output.
constexpr int kPrepRows = 8;  // rows per 256-thread block
__global__ void __launch_bounds__(32 * kPrepRows) bf_prep_weights(const uint8_t *__restrict__ A,
                                                                   uint8_t *__restrict__ W,
                                                                   uint8_t *__restrict__ dig,
                                                                   const float *__restrict__ G, float *__restrict__ gs,
                                                                   int *__restrict__ gwide, int B, int D, int nw,
                                                                   int nw_pad, int a_layout) {
  // E4M3 codes of the integers 0..8
  const uint8_t e4m3_pos[9] = {0x00, 0x38, 0x40, 0x44, 0x48, 0x4A, 0x4C, 0x4E, 0x50};
  const int rblocks = (nw_pad + kPrepRows - 1) / kPrepRows;  // blocks per frequency
  const int f = static_cast<int>(blockIdx.x) / rblocks;
  const int n = (static_cast<int>(blockIdx.x) % rblocks) * kPrepRows + static_cast<int>(threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (static_cast<int>(blockIdx.x) % rblocks == 0) {  // the frequency's scaled gains: 512 G, zero past B
    const int ng = nw_pad / 2;
    // |raw| <= 128 D, so with |G| * 128 D < 2^30 every product G * raw stays
    // below 2^31 and the plain requantisation is exact; otherwise (or for a
    // non-finite gain) the frequency takes the narrowing one of cpu.cxx:38
    const float wide_at = 1073741824.0f / (128.0f * static_cast<float>(D));
    int wide = 0;
    for (int i = threadIdx.x; i < ng; i += blockDim.x) {
      const float g = i < B ? G[static_cast<int64_t>(f) * B + i] : 0.0f;
      gs[static_cast<int64_t>(f) * ng + i] = 512.0f * g;
      wide |= !(fabsf(g) < wide_at);
    }
    wide = __syncthreads_or(wide);
    if (threadIdx.x == 0) gwide[f] = wide;
  }
  if (n >= nw_pad) return;  // the whole warp
  int sum = 0;
  if (n < nw) {
    const int b = 8 * (n / 16) + (n % 8);
    const int cj = (n / 8) & 1;
    // rows of 2D bytes, D % 8 == 0: 4-byte aligned words
    uint32_t *wrow = reinterpret_cast<uint32_t *>(W + (static_cast<int64_t>(f) * nw + n) * (2 * D));
    for (int k4 = lane; k4 < D / 2; k4 += 32) {  // k = 4 k4 .. 4 k4 + 3: dishes d0 .. d0 + 3, input part c
      const int c = k4 & 1;
      const int d0 = 4 * (k4 >> 1);
      uint32_t word = 0;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        int v = 0;
        if (b < B) {
          int ar, ai;
          load_a(A, a_layout, f, b, d0 + j, B, D, ar, ai);
          v = cj == 0 ? (c == 0 ? ar : -ai) : (c == 0 ? ai : ar);
        }
        const int av = v < 0 ? -v : v;
        word |= static_cast<uint32_t>(e4m3_pos[av] | (v < 0 ? 0x80 : 0x00)) << (8 * j);
        sum += v;
      }
      wrow[k4] = word;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if (lane == 0) {
    // s = sum_k W[n][k], |s| <= 16 D <= 2^15, in balanced base-16 digits
    // d0..d3 in [-8, 7] and d4 in {-1, 0, 1}; the digit row holds the E4M3
    // codes of d0, d1, d2, d3, 4 d4 (see kDigitScaleLo)
    uint32_t w0 = 0, w1 = 0;
    int rest = sum;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int r = rest & 15;
      const int dj = r >= 8 ? r - 16 : r;
      rest = (rest - dj) >> 4;
      const int av = dj < 0 ? -dj : dj;
      w0 |= static_cast<uint32_t>(e4m3_pos[av] | (dj < 0 ? 0x80 : 0x00)) << (8 * j);
    }
    w1 = rest == 0 ? 0u : (rest > 0 ? 0x48u : 0xC8u);  // 4 * d4: +-4 or 0
    uint32_t *row = reinterpret_cast<uint32_t *>(dig + (static_cast<int64_t>(f) * nw_pad + n) * kDigitRow);
    row[0] = w0;
    row[1] = w1;
#pragma unroll
    for (int j = 2; j < kDigitRow / 4; ++j) row[j] = 0u;
  }
}

PFN_cuTensorMapEncodeTiled_v12000 get_encode_fn() {
  // initialised once, thread-safely (the server thread encodes maps too)
  static const PFN_cuTensorMapEncodeTiled_v12000 fn = []() -> PFN_cuTensorMapEncodeTiled_v12000 {
    void *ptr = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(ptr);
    return nullptr;
  }();
  return fn;
}

bool make_map(CUtensorMap *m, const void *base, int rank, const cuuint64_t *dims, const cuuint64_t *strides,
              const cuuint32_t *box, CUtensorMapSwizzle swz) {
  auto fn = get_encode_fn();
  if (!fn) return false;
  cuuint32_t estr[5] = {1, 1, 1, 1, 1};
  const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_UINT8, rank, const_cast<void *>(base), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, swz, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

int g_test_stall = 0;
int g_plan_wslots = 0;  // nonzero: W slots to use (tuning)
int g_plan_raw = 0;     // nonzero: raw E slots to use (tuning)

int num_sms() {
  static const int n = []() {
    int dev = 0, k = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&k, cudaDevAttrMultiProcessorCount, dev);
    return k > 0 ? k : 1;
  }();
  return n;
}

}  // namespace

void tc_set_test_stall(int on) { g_test_stall = on; }

void tc_set_ring_plan(int wslots, int raw) {
  g_plan_wslots = wslots;
  g_plan_raw = raw;
}

void tc_plan_beams(int64_t B, int *nb_pass, int *npass) {
  // at most 96 beams (192 accumulator columns) per pass, so that two
  // accumulators and at least four unpacked stages fit the 512 TMEM columns;
  // passes are balanced
  const int64_t b8 = (B + 7) / 8 * 8;
  const int64_t np = (b8 + 95) / 96;
  const int64_t nbp = ((b8 + np - 1) / np + 7) / 8 * 8;
  *nb_pass = static_cast<int>(nbp);
  *npass = static_cast<int>((b8 + nbp - 1) / nbp);
}

bool tc_supported(const bf_dims &d) {
  if (d.npolarizations != 2) return false;
  if (d.ndishes <= 0 || d.ndishes % 8 != 0) return false;  // TMA row strides: 2*D multiple of 16 bytes
  if (d.ntimes <= 0 || d.ntimes % 16 != 0) return false;   // TMA store row strides: T multiple of 16 bytes
  if (d.nbeams <= 0 || d.nfrequencies <= 0) return false;
  // ndishes <= 2048 keeps |sum_k W[n][k]| <= 2^15, the range of the offset-correction digits
  if (d.ntimes > (1ll << 31) || d.nfrequencies > (1 << 20) || d.nbeams > (1 << 16) || d.ndishes > 2048)
    return false;
  return true;
}

cudaError_t launch_prep_weights(const TcWeights &w, const uint8_t *A, cudaStream_t s, int a_layout) {
  const int64_t blocks = static_cast<int64_t>((w.nw_pad + kPrepRows - 1) / kPrepRows) * w.F;
  if (blocks > 0x7FFFFFFF) return cudaErrorInvalidValue;
  bf_prep_weights<<<static_cast<unsigned>(blocks), 32 * kPrepRows, 0, s>>>(
      A, w.W, w.dig, w.G, w.gs, w.gwide, static_cast<int>(w.B), static_cast<int>(w.D), w.nw, w.nw_pad, a_layout);
  return cudaGetLastError();
}

// Fills a problem record: shape, pointers and the two tensor maps.
static cudaError_t make_problem(TcProblem &P, const TcWeights &w, int64_t T, uint8_t *J, const uint8_t *E,
                                int64_t jpitch, int j_layout) {
  const int64_t F = w.F, D = w.D;
  if ((reinterpret_cast<uintptr_t>(E) & 15u) || (reinterpret_cast<uintptr_t>(J) & 15u)) return cudaErrorMisalignedAddress;
  std::memset(&P, 0, sizeof(P));
  P.T = static_cast<int>(T);
  P.F = static_cast<int>(F);
  P.B = static_cast<int>(w.B);
  P.J = J;
  P.jbase = J;
  P.adler = nullptr;
  P.jpitch = jpitch > 0 ? jpitch : T;
  if (P.jpitch < T || (P.jpitch & 3)) return cudaErrorInvalidValue;
  if (j_layout != kJLinear && j_layout != kJ2) return cudaErrorInvalidValue;
  P.jlayout = j_layout;
  P.nb_pass = w.nb_pass;
  P.npass = w.npass;
  P.ntt = static_cast<int>((T + kTT - 1) / kTT);
  P.nw_pad = w.nw_pad;
  P.gs = w.gs;
  P.gwide = w.gwide;
  {  // E[t][f][d*p] bytes: dims {2D, F, T}
    const cuuint64_t dims[3] = {static_cast<cuuint64_t>(2 * D), static_cast<cuuint64_t>(F),
                                static_cast<cuuint64_t>(T)};
    const cuuint64_t str[2] = {static_cast<cuuint64_t>(2 * D), static_cast<cuuint64_t>(2 * D * F)};
    const cuuint32_t box[3] = {static_cast<cuuint32_t>(kKC), 1, static_cast<cuuint32_t>(kTT)};
    if (!make_map(&P.tm_e, E, 3, dims, str, box, CU_TENSOR_MAP_SWIZZLE_128B)) return cudaErrorInvalidValue;
  }
  {  // W[f][n][k] bytes: dims {2D, nw, F}
    const cuuint64_t dims[3] = {static_cast<cuuint64_t>(2 * D), static_cast<cuuint64_t>(w.nw),
                                static_cast<cuuint64_t>(F)};
    const cuuint64_t str[2] = {static_cast<cuuint64_t>(2 * D), static_cast<cuuint64_t>(2 * D * w.nw)};
    const cuuint32_t box[3] = {static_cast<cuuint32_t>(kKC), static_cast<cuuint32_t>(2 * w.nb_pass), 1};
    if (!make_map(&P.tm_w, w.W, 3, dims, str, box, CU_TENSOR_MAP_SWIZZLE_128B)) return cudaErrorInvalidValue;
  }
  {  // digit rows dig[f][n][32] bytes: dims {32, nw_pad, F}
    const cuuint64_t dims[3] = {static_cast<cuuint64_t>(kDigitRow), static_cast<cuuint64_t>(w.nw_pad),
                                static_cast<cuuint64_t>(F)};
    const cuuint64_t str[2] = {static_cast<cuuint64_t>(kDigitRow), static_cast<cuuint64_t>(kDigitRow) * w.nw_pad};
    const cuuint32_t box[3] = {static_cast<cuuint32_t>(kDigitRow), static_cast<cuuint32_t>(2 * w.nb_pass), 1};
    if (!make_map(&P.tm_d, w.dig, 3, dims, str, box, CU_TENSOR_MAP_SWIZZLE_32B)) return cudaErrorInvalidValue;
  }
  return cudaSuccess;
}

// Ring depths and shared memory for a launch whose largest pass has max_nb_pass beams.
static cudaError_t plan_launch(TcParams &p, int max_nb_pass, const TcRingPlan &plan, int *smem_bytes) {
  // unpacked stages live in the TMEM columns beside the two accumulators; raw E
  // slots take the shared memory the W slots leave
  const bool half = max_nb_pass <= kHalfPass;
  const int acc_cols = half ? kAccColsHalf : kAccCols;
  const int smem_limit = half ? kSmemLimitHalf : kSmemLimit;
  const int per_half = (acc_cols - 2 * max_nb_pass) / kStageCols;
  const int stages = std::min(kMaxStages, 2 * per_half);
  if (stages < 2) return cudaErrorInvalidValue;
  // Four or more unpacked stages: two unpack groups and the W forwarder.  Its
  // W producer reuses the slot of sequence it - SW once the tensor core's
  // commit of that sequence's stage arrives on `empty`, a parity wait that
  // must not find the stage's next use (sequence it - SW + S) committed too,
  // so SW <= S.  Otherwise one group, which hands W slots back S stages late,
  // so at least S slots keep it moving.
  const int groups = stages >= 4 && !half ? 2 : 1;  // the half-SM layout has one group
  // shared memory: W slots first (their loads gate the MMA), then raw E slots
  const int want_w = plan.wslots > 0 ? plan.wslots : g_plan_wslots;
  const int want_r = plan.raw > 0 ? plan.raw : g_plan_raw;
  int wslots = want_w > 0 ? want_w : kMaxWSlots;
  if (groups == 2) wslots = std::min(wslots, stages);
  int raw = want_r > 0 ? want_r : kMinRaw;
  while (wslots > 2 && smem_plan(stages, wslots, raw, max_nb_pass).total + 1024 > smem_limit) --wslots;
  while (raw < kMaxRaw && smem_plan(stages, wslots, raw + 1, max_nb_pass).total + 1024 <= smem_limit && want_r <= 0)
    ++raw;
  while (raw > 2 && smem_plan(stages, wslots, raw, max_nb_pass).total + 1024 > smem_limit) --raw;
  // Two groups take alternate sequences, and raw slot k % R serves sequences
  // k and k - R: an odd R gives them to different groups, and the group with
  // k can reach its raw_full parity wait while k - R's copy has not landed,
  // when the wait (one phase early) returns at once.  An even R keeps every
  // raw slot with one group, which takes its sequences in order.
  if (groups == 2 && raw % 2 == 1) --raw;
  const int st = groups == 2 ? stages : std::min(stages, wslots);
  // The same holds for the TMEM stage ring: stage slot k % S serves k and
  // k + S, so two groups need an even S (here always 2 x stages per accumulator).
  if (groups == 2 && (wslots > st || raw < 2 || st % 2 == 1)) return cudaErrorInvalidValue;
  p.max_nb_pass = max_nb_pass;
  p.stages = st;
  p.wslots = wslots;
  p.raw = raw;
  p.groups = groups;
  p.half = half ? 1 : 0;
  p.test_stall = g_test_stall;
  *smem_bytes = smem_plan(st, wslots, raw, max_nb_pass).total + 1024;
  return *smem_bytes > smem_limit ? cudaErrorInvalidValue : cudaSuccess;
}

template <bool kGrouped, bool kJ2, int kEpiW, bool kAdler, int kGroups, bool kHalf>
static cudaError_t launch_inst(const TcParams &p, int smem_bytes, cudaStream_t s) {
  auto kern = bf_form_beams_tc<kGrouped, kJ2, kEpiW, kAdler, kGroups, kHalf>;
  static std::atomic<bool> attr_set{false};
  if (!attr_set.load()) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         kHalf ? kSmemLimitHalf : kSmemLimit);
    // two half-SM blocks per SM need the whole shared-memory carveout
    if (e == cudaSuccess && kHalf)
      e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return e;
    attr_set.store(true);
  }
  const int grid = std::min(p.ntiles, (kHalf ? 2 : 1) * num_sms());
  if (grid <= 0) return cudaSuccess;
  kern<<<grid, Roles<kEpiW, kGroups>::kThreads, smem_bytes, s>>>(p);
  return cudaGetLastError();
}

// Warp layout of a launch: passes of at most kHalfPass beams run two CTAs per
// SM of four epilogue warps and one unpack group each; otherwise two unpack
// groups (with the forwarder) beside eight epilogue warps; one group beside
// twelve epilogue warps up to 4 K stages per tile (the epilogue paces short
// tiles) or eight for deeper tiles.
template <bool kGrouped, bool kJ2, bool kAdler>
static cudaError_t launch_layout(const TcParams &p, int smem_bytes, cudaStream_t s) {
  if (p.half) return launch_inst<kGrouped, kJ2, 4, kAdler, 1, true>(p, smem_bytes, s);
  if (p.groups == 2) return launch_inst<kGrouped, kJ2, 8, kAdler, 2, false>(p, smem_bytes, s);
  return p.nk <= 4 ? launch_inst<kGrouped, kJ2, 12, kAdler, 1, false>(p, smem_bytes, s)
                   : launch_inst<kGrouped, kJ2, 8, kAdler, 1, false>(p, smem_bytes, s);
}

template <bool kJ2, bool kAdler>
static cudaError_t launch_plain(const TcParams &p, int smem_bytes, cudaStream_t s) {
  return launch_layout<false, kJ2, kAdler>(p, smem_bytes, s);
}

// Instantiation for a launch: J2 output and the fused adler32 only in plain
// launches.
template <bool kGrouped>
static cudaError_t launch_kernel(const TcParams &p, int smem_bytes, cudaStream_t s) {
  if constexpr (kGrouped) {
    return launch_layout<true, false, false>(p, smem_bytes, s);
  } else {
    const bool j2 = p.one.jlayout == kJ2, adler = p.one.adler != nullptr;
    if (j2) return adler ? launch_plain<true, true>(p, smem_bytes, s) : launch_plain<true, false>(p, smem_bytes, s);
    return adler ? launch_plain<false, true>(p, smem_bytes, s) : launch_plain<false, false>(p, smem_bytes, s);
  }
}

cudaError_t tc_make_problem(TcProblem &P, const TcWeights &w, int64_t T, uint8_t *J, const uint8_t *E,
                            int64_t jpitch, int j_layout) {
  return make_problem(P, w, T, J, E, jpitch, j_layout);
}

int64_t tc_problem_tiles(const TcProblem &P) { return static_cast<int64_t>(P.ntt) * P.F * P.npass; }

int tc_stages_per_tile(int64_t D) { return static_cast<int>((D + kStageK / 2 - 1) / (kStageK / 2)); }

cudaError_t tc_plan_rings(int64_t D, int max_nb_pass, const TcRingPlan &plan, int *out) {
  TcParams p{};
  p.nk = tc_stages_per_tile(D);
  int smem_bytes = 0;
  const cudaError_t e = plan_launch(p, max_nb_pass, plan, &smem_bytes);
  if (e != cudaSuccess) return e;
  const int acc = p.half ? kAccColsHalf : kAccCols;  // the kernel's kAcc
  const int ncols = 2 * max_nb_pass;
  const int per_half = (acc - ncols) / kStageCols;
  int last_col = 0;  // one past the highest TMEM column an unpacked stage uses
  for (int i = 0; i < p.stages; ++i)
    last_col = std::max(last_col, static_cast<int>(stage_col(i, ncols, per_half, acc)) + kStageCols);
  out[0] = p.stages;
  out[1] = p.wslots;
  out[2] = p.raw;
  out[3] = p.groups;
  out[4] = p.half ? 2 : 1;
  out[5] = p.nk;
  out[6] = smem_bytes;
  out[7] = 2 * acc;  // TMEM columns allocated
  out[8] = ncols;    // columns of each accumulator (at 0 and at acc)
  out[9] = acc;
  out[10] = per_half;
  out[11] = last_col;
  return cudaSuccess;
}

cudaError_t tc_launch_shape(int64_t D, int max_nb_pass, const TcRingPlan &plan, int *stages, int *groups,
                            int *ctas_per_sm) {
  TcParams p{};
  p.nk = tc_stages_per_tile(D);
  int smem_bytes = 0;
  const cudaError_t e = plan_launch(p, max_nb_pass, plan, &smem_bytes);
  if (e != cudaSuccess) return e;
  *stages = p.stages;
  *groups = p.groups;
  *ctas_per_sm = p.half ? 2 : 1;
  return cudaSuccess;
}

cudaError_t launch_tc_grouped(const TcProblem *table, int nprob, int ntiles, int64_t D, int max_nb_pass,
                              const TcRingPlan &plan, int *err, cudaStream_t s) {
  TcParams p{};
  p.table = table;
  p.nprob = nprob;
  p.ntiles = ntiles;
  p.nk = tc_stages_per_tile(D);
  p.err = err;
  int smem_bytes = 0;
  const cudaError_t e = plan_launch(p, max_nb_pass, plan, &smem_bytes);
  if (e != cudaSuccess) return e;
  return launch_kernel<true>(p, smem_bytes, s);
}

cudaError_t launch_tc(const TcWeights &w, int64_t T, uint8_t *J, const uint8_t *E, int *err, cudaStream_t s,
                      int64_t jpitch, int j_layout, unsigned long long *adler, const uint8_t *jbase) {
  TcParams p{};
  cudaError_t e = make_problem(p.one, w, T, J, E, jpitch, j_layout);
  if (e != cudaSuccess) return e;
  p.one.adler = adler;
  if (jbase) p.one.jbase = jbase;
  if (adler && (p.one.jbase > J)) return cudaErrorInvalidValue;
  const int64_t ntiles = static_cast<int64_t>(p.one.ntt) * w.F * w.npass;
  if (ntiles > 0x7FFFFFFF) return cudaErrorInvalidValue;
  p.ntiles = static_cast<int>(ntiles);
  p.nprob = 1;
  p.nk = tc_stages_per_tile(w.D);
  p.err = err;
  int smem_bytes = 0;
  e = plan_launch(p, w.nb_pass, TcRingPlan{}, &smem_bytes);
  if (e != cudaSuccess) return e;
  return launch_kernel<false>(p, smem_bytes, s);
}

}  // namespace bf
