// bf_tc.cu -- the beamformer on the 5th-generation tensor cores (tcgen05).
//
// The complex sum of cpu.cxx:26-35 becomes one real GEMM per frequency:
//
//   rows    m = (p, t)      128 per tile: 64 times x 2 polarizations
//   columns n = (b, re|im)  2 * beams (<= 256 per pass)
//   depth   k = (d, re|im)  2 * dishes
//
//   [Jre]   [ Ar  -Ai ] [Ere]
//   [Jim] = [ Ai   Ar ] [Eim]      summed over d
//
// Operands are 8-bit floats (E4M3).  A byte holding an unsigned nibble u in
// [0, 15] is, read as E4M3, exactly u * 2^-9 (exponent field 0 or 1: the
// subnormal and the first normal binade share the step 2^-9).  So the raw
// ucomplex4 nibbles (value x stored as u = x + 8) become tensor-core operands
// with one AND per 4 values; the offset is removed in the epilogue:
//
//   sum_k (u_k - 8) W[n][k] = 512 * acc[n] - 8 * sum_k W[n][k]
//
// W holds the integers Ar, -Ai, Ai in [-8, 8], exact in E4M3; every product
// and every partial sum is an integer multiple of 2^-9 below 2^8 in
// magnitude (17 significant bits), exact in the f32 accumulator.  The
// requantisation clamp(lrint(G * float(raw)), -7, 7) of cpu.cxx:37-39 runs in
// the epilogue with one IEEE multiply and a round-half-even conversion.
//
// Warp roles (one CTA per SM, persistent over tiles):
//   warps 0-3  epilogue: TMEM -> registers -> requantise -> J tile in smem -> TMA store
//   warp  4    TMA producer: raw E tile and the W slice of each K stage
//   warp  5    TMEM allocator and single-thread MMA issuer
//   warps 6-9  unpack: raw E bytes -> de-interleaved E4M3 operand (128B-swizzled)
#include "bf_internal.h"
#include "bf_ptx.cuh"

#include <algorithm>
#include <cstdio>
#include <cudaTypedefs.h>

namespace bf {
namespace {

constexpr int kThreads = 320;
constexpr int kTmaWarp = 4;
constexpr int kMmaWarp = 5;
constexpr int kUnpackWarp0 = 6;
constexpr int kTT = 64;                 // times per tile
constexpr int kBM = 128;                // GEMM rows per tile
constexpr int kKC = 128;                // K bytes per stage (64 dishes x re/im)
constexpr int kRawBytes = kTT * kKC;    // raw E per stage: 64 times x 64 dishes x 2 pol
constexpr int kABytes = kBM * kKC;      // unpacked operand per stage
constexpr int kAccCols = 256;           // TMEM columns per accumulator buffer
constexpr int kSmemLimit = 232448;      // 227 KiB opt-in per block
constexpr int kMaxStages = 6;

struct TcParams {
  int T, F, D, B;
  int nb_pass;  // beams per pass
  int npass;
  int ntt;      // time tiles per frequency
  int nk;       // K stages per tile
  int ntiles;
  int stages;
  int nw_pad;
  int test_stall;  // nonzero: the producer issues nothing (failure-path test)
  const float *G;
  const float *bias;
  int *err;
};

struct SmemPlan {
  int stages, wbytes, jbytes;
  int off_a, off_w, off_r, off_j, off_bar, total;
};

__host__ __device__ inline SmemPlan smem_plan(int stages, int nb_pass) {
  SmemPlan s{};
  s.stages = stages;
  s.wbytes = 2 * nb_pass * kKC;
  s.jbytes = nb_pass * 2 * kTT;
  s.off_a = 0;
  s.off_w = s.off_a + stages * kABytes;
  s.off_r = s.off_w + stages * s.wbytes;
  s.off_j = s.off_r + stages * kRawBytes;
  s.off_bar = s.off_j + 2 * s.jbytes;
  // full[S], afull[S], empty[S], accfull[2], accempty[2], tmem address
  s.total = s.off_bar + 8 * (3 * stages + 4) + 16;
  return s;
}

__device__ __forceinline__ uint32_t prmt(uint32_t a, uint32_t b, uint32_t sel) {
  uint32_t r;
  asm("prmt.b32 %0, %1, %2, %3;" : "=r"(r) : "r"(a), "r"(b), "r"(sel));
  return r;
}

// Byte offset of 16-byte chunk j of row r in a 128B-swizzled K-major tile.
__device__ __forceinline__ uint32_t sw128_offset(uint32_t r, uint32_t j) {
  return (r >> 3) * 1024u + (r & 7u) * 128u + ((j ^ (r & 7u)) << 4);
}

__global__ void __launch_bounds__(kThreads, 1)
    bf_form_beams_tc(const __grid_constant__ CUtensorMap tm_e, const __grid_constant__ CUtensorMap tm_w,
                     const __grid_constant__ CUtensorMap tm_j, const TcParams p) {
  extern __shared__ uint8_t smem_dyn[];
  uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_dyn) + 1023) & ~uintptr_t(1023));
  const SmemPlan sp = smem_plan(p.stages, p.nb_pass);
  const int S = p.stages;
  uint8_t *sA = smem + sp.off_a;
  uint8_t *sW = smem + sp.off_w;
  uint8_t *sR = smem + sp.off_r;
  uint8_t *sJ = smem + sp.off_j;
  const uint32_t bar0 = smem_u32(smem + sp.off_bar);
  auto full = [&](int s) { return bar0 + 8u * s; };
  auto afull = [&](int s) { return bar0 + 8u * (S + s); };
  auto empty = [&](int s) { return bar0 + 8u * (2 * S + s); };
  auto accfull = [&](int i) { return bar0 + 8u * (3 * S + i); };
  auto accempty = [&](int i) { return bar0 + 8u * (3 * S + 2 + i); };
  uint32_t *tmem_holder = reinterpret_cast<uint32_t *>(smem + sp.off_bar + 8 * (3 * S + 4));

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(full(s), 1);
      mbar_init(afull(s), 128);
      mbar_init(empty(s), 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(accfull(i), 1);
      mbar_init(accempty(i), 128);
    }
    fence_barrier_init();
  }
  if (warp == kMmaWarp) {
    tmem_alloc(smem_u32(tmem_holder), 2 * kAccCols);
    tmem_relinquish();
  }
  if (warp == kTmaWarp && lane == 0) {
    tma_prefetch_desc(&tm_e);
    tma_prefetch_desc(&tm_w);
    tma_prefetch_desc(&tm_j);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = *tmem_holder;
  int *err = p.err;

  if (warp == kTmaWarp) {
    // ------------------------------------------------------------ producer
    if (lane == 0 && !p.test_stall) {
      const uint64_t pol_e = policy_evict_first();
      const uint64_t pol_w = policy_evict_last();
      const uint32_t tx = kRawBytes + sp.wbytes;
      uint32_t it = 0;
      bool ok = true;
      for (int tile = blockIdx.x; ok && tile < p.ntiles; tile += gridDim.x) {
        const int pass = tile % p.npass;
        const int tt = (tile / p.npass) % p.ntt;
        const int f = tile / (p.npass * p.ntt);
        for (int ks = 0; ks < p.nk; ++ks, ++it) {
          const int s = static_cast<int>(it % S);
          const uint32_t ph = (it / S) & 1u;
          if (!mbar_wait(empty(s), ph ^ 1u, err, kDevTimeoutEmpty)) {
            ok = false;
            break;
          }
          mbar_arrive_expect_tx(full(s), tx);
          tma_load_3d(smem_u32(sR + s * kRawBytes), &tm_e, full(s), ks * kKC, f, tt * kTT, pol_e);
          tma_load_3d(smem_u32(sW + s * sp.wbytes), &tm_w, full(s), ks * kKC, pass * 2 * p.nb_pass, f, pol_w);
        }
      }
      // On failure, let copies already issued land before the CTA exits.
      if (!ok) {
        for (uint32_t k = (it >= static_cast<uint32_t>(S) ? it - S : 0); k < it; ++k)
          mbar_wait(full(static_cast<int>(k % S)), (k / S) & 1u, err, kDevTimeoutFull);
      }
    }
  } else if (warp == kMmaWarp) {
    // ------------------------------------------------------------ MMA issuer
    if (lane == 0) {
      const uint32_t idesc = idesc_e4m3_f32(kBM, 2 * p.nb_pass);
      uint32_t it = 0, local = 0;
      bool ok = true;
      for (int tile = blockIdx.x; ok && tile < p.ntiles; tile += gridDim.x, ++local) {
        const uint32_t ab = local & 1u;
        const uint32_t aph = (local >> 1) & 1u;
        if (!mbar_wait(accempty(ab), aph ^ 1u, err, kDevTimeoutAccEmpty)) break;
        tc_fence_after();
        const uint32_t d_tmem = tmem_base + ab * kAccCols;
        for (int ks = 0; ks < p.nk; ++ks, ++it) {
          const int s = static_cast<int>(it % S);
          const uint32_t ph = (it / S) & 1u;
          if (!mbar_wait(afull(s), ph, err, kDevTimeoutUnpacked) || !mbar_wait(full(s), ph, err, kDevTimeoutFull)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t a_base = smem_u32(sA + s * kABytes);
          const uint32_t b_base = smem_u32(sW + s * sp.wbytes);
#pragma unroll
          for (int kk = 0; kk < kKC / 32; ++kk) {
            mma_f8f6f4(d_tmem, smem_desc_sw128(a_base + 32 * kk), smem_desc_sw128(b_base + 32 * kk), idesc,
                       (ks | kk) != 0 ? 1u : 0u);
          }
          mma_commit(empty(s));
        }
        if (!ok) break;
        mma_commit(accfull(ab));
      }
    }
  } else if (warp >= kUnpackWarp0) {
    // ------------------------------------------------------------ unpack
    const int uw = warp - kUnpackWarp0;
    const uint32_t tl = 32u * (uw & 1) + lane;   // time within the tile
    const uint32_t jbase = 4u * (uw >> 1);       // 16-byte chunks jbase..jbase+3
    const uint32_t row0 = tl, row1 = 64u + tl;  // GEMM rows (p=0, t) and (p=1, t)
    uint32_t it = 0;
    bool ok = true;
    for (int tile = blockIdx.x; ok && tile < p.ntiles; tile += gridDim.x) {
      for (int ks = 0; ks < p.nk; ++ks, ++it) {
        const int s = static_cast<int>(it % S);
        const uint32_t ph = (it / S) & 1u;
        if (!mbar_wait(full(s), ph, err, kDevTimeoutFull)) {
          ok = false;
          break;
        }
        const uint8_t *raw = sR + s * kRawBytes;
        uint8_t *a = sA + s * kABytes;
#pragma unroll
        for (uint32_t jj = 0; jj < 4; ++jj) {
          const uint32_t j = jbase + jj;
          // 8 dishes x 2 polarizations: bytes [d0p0 d0p1 d1p0 d1p1 ... d7p1]
          const uint4 w = *reinterpret_cast<const uint4 *>(raw + sw128_offset(tl, j));
          const uint32_t x0 = prmt(w.x, w.y, 0x6420u), y0 = prmt(w.x, w.y, 0x7531u);  // d0-3, p0 / p1
          const uint32_t x1 = prmt(w.z, w.w, 0x6420u), y1 = prmt(w.z, w.w, 0x7531u);  // d4-7, p0 / p1
          const uint32_t m = 0x0F0F0F0Fu;
          // k order inside the chunk: re(d0-3) im(d0-3) re(d4-7) im(d4-7)
          const uint4 o0 = make_uint4((x0 >> 4) & m, x0 & m, (x1 >> 4) & m, x1 & m);
          const uint4 o1 = make_uint4((y0 >> 4) & m, y0 & m, (y1 >> 4) & m, y1 & m);
          *reinterpret_cast<uint4 *>(a + sw128_offset(row0, j)) = o0;
          *reinterpret_cast<uint4 *>(a + sw128_offset(row1, j)) = o1;
        }
        fence_proxy_async_smem();
        mbar_arrive(afull(s));
      }
    }
  } else {
    // ------------------------------------------------------------ epilogue
    const int q = warp;                       // TMEM lane quarter
    const uint32_t pol = static_cast<uint32_t>(q) >> 1;
    const uint32_t tl = 32u * (q & 1) + lane;
    const uint32_t lane_addr = static_cast<uint32_t>(32 * q) << 16;
    uint32_t local = 0;
    for (int tile = blockIdx.x; tile < p.ntiles; tile += gridDim.x, ++local) {
      const int pass = tile % p.npass;
      const int tt = (tile / p.npass) % p.ntt;
      const int f = tile / (p.npass * p.ntt);
      const uint32_t ab = local & 1u;
      const uint32_t aph = (local >> 1) & 1u;
      uint8_t *js = sJ + ab * sp.jbytes;
      if (threadIdx.x == 0) bulk_wait_group_read<1>();  // the store that used this buffer has read it
      named_bar_sync(1, 128);
      const bool got = mbar_wait(accfull(ab), aph, err, kDevTimeoutAccFull);
      if (!named_bar_and(2, 128, got)) break;  // all four warps leave together
      tc_fence_after();
      const int b0 = pass * p.nb_pass;
      const float *g = p.G + static_cast<int64_t>(f) * p.B;
      const float *bias = p.bias + static_cast<int64_t>(f) * p.nw_pad + 2 * b0;
      for (int c = 0; c < p.nb_pass / 8; ++c) {
        uint32_t r[16];
        tmem_ld_32x32b_x16(tmem_base + ab * kAccCols + lane_addr + 16u * c, r);
        tmem_ld_wait();
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const int bl = 8 * c + i;
          const int b = b0 + bl;
          const float gb = b < p.B ? __ldg(g + b) : 0.0f;
          // exact integer sums: 512 * acc - 8 * sum(W), both below 2^24
          const float raw_re = fmaf(__uint_as_float(r[i]), 512.0f, -__ldg(bias + 16 * c + i));
          const float raw_im = fmaf(__uint_as_float(r[8 + i]), 512.0f, -__ldg(bias + 16 * c + 8 + i));
          const int jre = max(-7, min(7, __float2int_rn(__fmul_rn(gb, raw_re))));
          const int jim = max(-7, min(7, __float2int_rn(__fmul_rn(gb, raw_im))));
          js[(bl * 2 + pol) * kTT + tl] = static_cast<uint8_t>(((jre + 8) << 4) | (jim + 8));
        }
      }
      tc_fence_before();
      mbar_arrive(accempty(ab));
      fence_proxy_async_smem();
      named_bar_sync(1, 128);
      if (threadIdx.x == 0) {
        tma_store_4d(&tm_j, smem_u32(js), tt * kTT, 0, f, b0);
        bulk_commit_group();
      }
    }
    if (threadIdx.x == 0) bulk_wait_group<0>();
  }

  tc_fence_before();
  __syncthreads();
  if (warp == kMmaWarp) {
    tc_fence_after();
    tmem_dealloc(tmem_base, 2 * kAccCols);
  }
}

// Builds the E4M3 operand W[f][n][k] and the per-row offset correction
// bias[f][n] = 8 * sum_k W[f][n][k] from A[f][b][d].
//   n = 16*(b/8) + 8*cj + b%8      (cj: 0 = real output, 1 = imaginary output)
//   k = 8*(d/4)  + 4*c  + d%4      (c:  0 = real input,  1 = imaginary input)
// W = Ar, -Ai for the real output and Ai, Ar for the imaginary output.
__global__ void bf_prep_weights(const uint8_t *__restrict__ A, uint8_t *__restrict__ W, float *__restrict__ bias,
                                int B, int D, int nw, int nw_pad) {
  // E4M3 codes of the integers 0..8
  const uint8_t e4m3_pos[9] = {0x00, 0x38, 0x40, 0x44, 0x48, 0x4A, 0x4C, 0x4E, 0x50};
  const int f = blockIdx.y;
  const int n = blockIdx.x;
  int sum = 0;
  if (n < nw) {
    const int b = 8 * (n / 16) + (n % 8);
    const int cj = (n / 8) & 1;
    uint8_t *wrow = W + (static_cast<int64_t>(f) * nw + n) * (2 * D);
    for (int k = threadIdx.x; k < 2 * D; k += blockDim.x) {
      const int d = 4 * (k / 8) + (k % 4);
      const int c = (k / 4) & 1;
      int v = 0;
      if (b < B) {
        const uint32_t a = A[(static_cast<int64_t>(f) * B + b) * D + d] ^ 0x88u;
        const int ar = static_cast<int>(static_cast<int8_t>(a)) >> 4;
        const int ai = static_cast<int>(static_cast<int8_t>(static_cast<uint8_t>(a << 4))) >> 4;
        v = cj == 0 ? (c == 0 ? ar : -ai) : (c == 0 ? ai : ar);
      }
      const int av = v < 0 ? -v : v;
      wrow[k] = static_cast<uint8_t>(e4m3_pos[av] | (v < 0 ? 0x80 : 0x00));
      sum += v;
    }
  }
  __shared__ int red[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x / 32] = sum;
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int i = 0; i < static_cast<int>(blockDim.x / 32); ++i) s += red[i];
    bias[static_cast<int64_t>(f) * nw_pad + n] = 8.0f * static_cast<float>(s);
  }
}

PFN_cuTensorMapEncodeTiled_v12000 get_encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void *ptr = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(ptr);
  }
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

int num_sms() {
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 1;
  }
  return n;
}

}  // namespace

void tc_set_test_stall(int on) { g_test_stall = on; }

void tc_plan_beams(int64_t B, int *nb_pass, int *npass) {
  const int64_t b8 = (B + 7) / 8 * 8;
  const int64_t nbp = std::min<int64_t>(b8, 128);
  *nb_pass = static_cast<int>(nbp);
  *npass = static_cast<int>((b8 + nbp - 1) / nbp);
}

bool tc_supported(const bf_dims &d) {
  if (d.npolarizations != 2) return false;
  if (d.ndishes <= 0 || d.ndishes % 8 != 0) return false;  // TMA row strides: 2*D multiple of 16 bytes
  if (d.ntimes <= 0 || d.ntimes % 16 != 0) return false;   // TMA store row strides: T multiple of 16 bytes
  if (d.nbeams <= 0 || d.nfrequencies <= 0) return false;
  if (d.ntimes > (1ll << 31) || d.nfrequencies > (1 << 20) || d.nbeams > (1 << 16) || d.ndishes > (1 << 16))
    return false;
  return true;
}

cudaError_t launch_prep_weights(const TcWeights &w, const uint8_t *A, cudaStream_t s) {
  const dim3 grid(static_cast<unsigned>(w.nw_pad), static_cast<unsigned>(w.F));
  bf_prep_weights<<<grid, 256, 0, s>>>(A, w.W, w.bias, static_cast<int>(w.B), static_cast<int>(w.D), w.nw,
                                       w.nw_pad);
  return cudaGetLastError();
}

cudaError_t launch_tc(const TcWeights &w, int64_t T, uint8_t *J, const uint8_t *E, int *err, cudaStream_t s) {
  const int64_t F = w.F, D = w.D, B = w.B;
  if ((reinterpret_cast<uintptr_t>(E) & 15u) || (reinterpret_cast<uintptr_t>(J) & 15u)) return cudaErrorMisalignedAddress;
  TcParams p{};
  p.T = static_cast<int>(T);
  p.F = static_cast<int>(F);
  p.D = static_cast<int>(D);
  p.B = static_cast<int>(B);
  p.nb_pass = w.nb_pass;
  p.npass = w.npass;
  p.ntt = static_cast<int>((T + kTT - 1) / kTT);
  p.nk = static_cast<int>((D + 63) / 64);
  const int64_t ntiles = static_cast<int64_t>(p.ntt) * F * p.npass;
  if (ntiles > 0x7FFFFFFF) return cudaErrorInvalidValue;
  p.ntiles = static_cast<int>(ntiles);
  p.nw_pad = w.nw_pad;
  p.G = w.G;
  p.bias = w.bias;
  p.err = err;
  p.test_stall = g_test_stall;
  int stages = kMaxStages;
  while (stages > 2 && smem_plan(stages, w.nb_pass).total + 1024 > kSmemLimit) --stages;
  p.stages = stages;
  const int smem_bytes = smem_plan(stages, w.nb_pass).total + 1024;
  if (smem_bytes > kSmemLimit) return cudaErrorInvalidValue;

  CUtensorMap tm_e, tm_w, tm_j;
  {  // E[t][f][d*p] bytes: dims {2D, F, T}
    const cuuint64_t dims[3] = {static_cast<cuuint64_t>(2 * D), static_cast<cuuint64_t>(F),
                                static_cast<cuuint64_t>(T)};
    const cuuint64_t str[2] = {static_cast<cuuint64_t>(2 * D), static_cast<cuuint64_t>(2 * D * F)};
    const cuuint32_t box[3] = {static_cast<cuuint32_t>(kKC), 1, static_cast<cuuint32_t>(kTT)};
    if (!make_map(&tm_e, E, 3, dims, str, box, CU_TENSOR_MAP_SWIZZLE_128B)) return cudaErrorInvalidValue;
  }
  {  // W[f][n][k] bytes: dims {2D, nw, F}
    const cuuint64_t dims[3] = {static_cast<cuuint64_t>(2 * D), static_cast<cuuint64_t>(w.nw),
                                static_cast<cuuint64_t>(F)};
    const cuuint64_t str[2] = {static_cast<cuuint64_t>(2 * D), static_cast<cuuint64_t>(2 * D * w.nw)};
    const cuuint32_t box[3] = {static_cast<cuuint32_t>(kKC), static_cast<cuuint32_t>(2 * w.nb_pass), 1};
    if (!make_map(&tm_w, w.W, 3, dims, str, box, CU_TENSOR_MAP_SWIZZLE_128B)) return cudaErrorInvalidValue;
  }
  {  // J[b][f][p][t] bytes: dims {T, 2, F, B}
    const cuuint64_t dims[4] = {static_cast<cuuint64_t>(T), 2, static_cast<cuuint64_t>(F),
                                static_cast<cuuint64_t>(B)};
    const cuuint64_t str[3] = {static_cast<cuuint64_t>(T), static_cast<cuuint64_t>(2 * T),
                               static_cast<cuuint64_t>(2 * T * F)};
    const cuuint32_t box[4] = {static_cast<cuuint32_t>(kTT), 2, 1, static_cast<cuuint32_t>(w.nb_pass)};
    if (!make_map(&tm_j, J, 4, dims, str, box, CU_TENSOR_MAP_SWIZZLE_NONE)) return cudaErrorInvalidValue;
  }

  static bool attr_set = false;
  if (!attr_set) {
    const cudaError_t e =
        cudaFuncSetAttribute(bf_form_beams_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemLimit);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  const int grid = static_cast<int>(std::min<int64_t>(ntiles, num_sms()));
  if (grid <= 0) return cudaSuccess;
  bf_form_beams_tc<<<grid, kThreads, smem_bytes, s>>>(tm_e, tm_w, tm_j, p);
  return cudaGetLastError();
}

}  // namespace bf
