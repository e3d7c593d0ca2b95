// Tensor-core GEMM for the FP32-class contractions (np.tensordot in
// tncontract/tensor.py:735 and the sweep's absorption products) on GB300's
// 5th-generation tensor cores, exact up to the rounding of the FP32 inputs'
// third 8-bit digit and free of accumulation bias.
//
// Why not a TF32 hi/lo split: the tensor cores accumulate in FP32 with
// truncation toward zero, so a long accumulation in tensor memory shrinks every
// product's magnitude by ~1e-8 x K (measured: the norm of a chi = 256 sweep fell
// by 1.6e-3 over its 190 products while the fidelity stayed 1e-9).
//
// Error-free split (after Ozaki's scheme): every row of op(A) and every column
// of op(B) is scaled by a power of two to |x| < 1 and cut into three signed
// 8-bit digits, x = 2^e 2^-8 (d0 + d1 2^-8 + d2 2^-16) (d0 in [-256, 256],
// d1, d2 in [-128, 128], the last rounded to nearest), each digit an exact
// BF16 value.  Digit products are integers below 2^16, so a 64-deep K chunk of
// the products of one level (i + j = 0, 1, 2) sums to an integer below 2^24:
// the FP32 accumulation in tensor memory is exact and its truncation never
// acts.  After each chunk the three level accumulators are read with
// tcgen05.ld and added into registers as L0 + 2^-8 L1 + 2^-16 L2 with
// round-to-nearest FP32 adds.  Levels 3 and 4 are dropped (relative weight
// 2^-24), so the result is FP32-accurate normwise and unbiased.
//
// Complex products run as real ones in the real-block form: row r of op(A)
// becomes rows 2r = [Re, -Im] and 2r+1 = [Im, Re] of A' (K' = 2K), column c of
// op(B) the row [Re, Im] of B'; rows 2r / 2r+1 of the result are the real and
// imaginary parts of C's row r.
//
// Data path: a split kernel (one warp per row) writes the three BF16 digit
// planes of A' (M' x K') and B' (N x K'), K-contiguous and zero-padded to the
// tile grid, and the power-of-two scales.  The GEMM kernel (one CTA per
// 128 x 128 tile of A' B'^T, 4 warps) has thread 0 stream 64-deep K slices of
// the six planes into shared memory with TMA (cp.async.bulk.tensor, 128-byte
// swizzle, completion on an mbarrier), two stages, and issue the six
// tcgen05.mma (kind::f16, BF16 inputs, FP32 accumulators, M = 128, N = 128,
// K = 16) of every K step into three TMEM accumulators; after each slice all
// four warps read their lanes (warp w: tile rows 32w..32w+31) and accumulate.
//
// Every mbarrier wait is bounded; a wait that gives up records an error
// (tnc_gemm_tc_error), waits (bounded) for the copies and MMAs it issued and
// frees its tensor memory before returning.
#include "tnc_common.cuh"

#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <atomic>
#include <mutex>

namespace tnc {

constexpr int kTcBM = 128;  // tile rows of A' (UMMA M)
constexpr int kTcBN = 128;  // tile rows of B' (UMMA N)
constexpr int kTcBK = 64;   // K elements per stage = one 128-byte swizzle atom of BF16
constexpr int kTcNP = 3;    // digit planes
// mbarrier polls before giving up: twice the library's wait limit
// (tnc_set_spin_limit), a try_wait poll being shorter than a sleeping one
static __device__ long long g_tc_spin = 2 * kSpinLimitDefault;

__device__ int g_tc_error = 0;

int spin_limit_set_tc(long long polls) {
  const long long v = 2 * polls;
  return cudaMemcpyToSymbol(g_tc_spin, &v, sizeof(v)) == cudaSuccess ? TNC_OK : TNC_ERR_CUDA;
}

// ------------------------------------------------------------------ PTX wrappers
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n"
      " .reg .pred p;\n"
      " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  long long spins = 0;
  const long long limit = *(volatile long long*)&g_tc_spin;
  while (!mbar_try_wait(bar, parity)) {
    if (++spins > limit) {
      atomicExch(&g_tc_error, 1);
      return false;
    }
  }
  return true;
}
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::
          "r"(smem_u32(dst)),
      "l"(map), "r"(smem_u32(bar)), "r"(x), "r"(y)
      : "memory");
}
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
// 32 consecutive FP32 columns of this warp's 32 TMEM lanes
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// Shared-memory matrix descriptor: K-major operand in the canonical 128-byte
// swizzled layout TMA writes (8-row x 128-byte atoms, 1024 B apart).
__device__ __forceinline__ uint64_t sw128_kmajor_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);  // start address (16-byte units)
  d |= (uint64_t)1u << 16;                   // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024u >> 4) << 32;         // stride byte offset: next 8-row atom
  d |= (uint64_t)1u << 46;                   // descriptor version
  d |= (uint64_t)2u << 61;                   // 128-byte swizzle
  return d;
}

// Instruction descriptor, kind::f16: D = F32, A = B = BF16, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n"
      " .reg .pred p;\n"
      " setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
      "}\n" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// ------------------------------------------------------------------ split kernel
// One warp per source row r of X (X = op(A), rows x K, or X = op(B)^T): the
// row's largest component fixes the power-of-two scale (|x| 2^-e < 1, scale
// 2^e stored), then its digits go to the three planes
// dst[batch][plane][rowsOutPad][Kpad].  Real: output row r, K' = K.  Complex
// A: output rows 2r = [Re, -Im], 2r + 1 = [Im, Re]; complex B: output row r =
// [Re, Im] (K' = 2K).  Rows and columns beyond the data are written as zeros.
template <bool CPLX>
__global__ void tc_split_kernel(const float* __restrict__ src, int op, int isB, int64_t rows, int64_t K, int64_t ld,
                                int64_t sbatch, int64_t batch, int64_t rowsSrcPad, int64_t rowsOutPad, int64_t Kpad,
                                __nv_bfloat16* __restrict__ dst, float* __restrict__ scale) {
  const int lane = threadIdx.x & 31;
  const bool trans = (op == TNC_OP_T || op == TNC_OP_C);
  const bool cj = (op == TNC_OP_C || op == TNC_OP_R);
  const bool rowmajor_rk = isB ? trans : !trans;
  const bool pairA = CPLX && !isB;  // two output rows per source row
  const int64_t plane = rowsOutPad * Kpad;
  const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < batch * rowsSrcPad; w += nw) {
    const int64_t b = w / rowsSrcPad, r = w - b * rowsSrcPad;
    const bool real_row = r < rows;
    const float* sb = src + b * sbatch * (CPLX ? 2 : 1);
    auto load = [&](int64_t k, float& re, float& im) {
      const int64_t off = rowmajor_rk ? (r * ld + k) : (k * ld + r);
      if (CPLX) {
        const float2 v = reinterpret_cast<const float2*>(sb)[off];
        re = v.x;
        im = cj ? -v.y : v.y;
      } else {
        re = sb[off];
        im = 0.f;
      }
    };
    float mx = 0.f;
    if (real_row)
      for (int64_t k = lane; k < K; k += 32) {
        float re, im;
        load(k, re, im);
        mx = fmaxf(mx, fmaxf(fabsf(re), fabsf(im)));
      }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    int e = 0;
    if (mx > 0.f && isfinite(mx)) frexpf(mx, &e);  // mx = f 2^e, f in [0.5, 1)
    if (e > 127) e = 127;
    const int64_t outRows = pairA ? 2 : 1;
    const int64_t o0 = pairA ? 2 * r : r;
    if (lane == 0) {
      scale[b * rowsOutPad + o0] = ldexpf(1.f, e);
      if (pairA) scale[b * rowsOutPad + o0 + 1] = ldexpf(1.f, e);
    }
    __nv_bfloat16* base = dst + b * kTcNP * plane;
    auto put = [&](int64_t orow, int64_t kk, float x) {
      // x 2^-e in (-1, 1): three digits, the last rounded to nearest
      const float y = ldexpf(x, 8 - e);
      const float d0 = rintf(y);
      const float r1 = (y - d0) * 256.f;
      const float d1 = rintf(r1);
      const float d2 = rintf((r1 - d1) * 256.f);
      __nv_bfloat16* q = base + orow * Kpad + kk;
      q[0] = __float2bfloat16_rn(d0);
      q[plane] = __float2bfloat16_rn(d1);
      q[2 * plane] = __float2bfloat16_rn(d2);
    };
    const int64_t Kp = CPLX ? 2 * K : K;
    for (int64_t k = lane; k < Kpad; k += 32) {
      if (CPLX) {
        // k indexes the K' axis: [0, K) real parts, [K, 2K) imaginary parts
        float re = 0.f, im = 0.f;
        const int64_t ks = k < K ? k : k - K;
        if (real_row && k < Kp) load(ks, re, im);
        if (pairA) {
          put(o0, k, k < K ? re : -im);      // row 2r:   [Re, -Im] . [Re', Im']
          put(o0 + 1, k, k < K ? im : re);   // row 2r+1: [Im,  Re]
        } else {
          put(o0, k, k < K ? re : im);       // B: [Re, Im]
        }
      } else {
        float re = 0.f, im;
        if (real_row && k < K) load(k, re, im);
        put(o0, k, re);
      }
    }
    (void)outRows;
  }
}

// ------------------------------------------------------------------ GEMM kernel
struct TcCfg {
  static constexpr uint32_t A_TILE = kTcBM * 128;  // bytes: 128 rows x 64 BF16
  static constexpr uint32_t B_TILE = kTcBN * 128;
  static constexpr uint32_t STAGE = kTcNP * (A_TILE + B_TILE);
  static constexpr int STAGES = 2;
  static constexpr uint32_t SMEM = STAGES * STAGE + 1024;  // + alignment slack
  static constexpr uint32_t TMEM_COLS = 512;               // three 128-column level accumulators
};

template <bool CPLX>
__global__ void __launch_bounds__(128, 1)
gemm_tc_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, int64_t M,
               int64_t N, int64_t Kpad, int64_t rowsA, int64_t rowsB, const float* __restrict__ scaleA,
               const float* __restrict__ scaleB, float ar, float ai, float br, float bi, float* __restrict__ C,
               int64_t ldc, int64_t sC) {
  typedef TcCfg Cfg;
  constexpr int STAGES = Cfg::STAGES;
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t full_bar[STAGES];
  __shared__ uint64_t done_bar;
  __shared__ uint32_t tmem_base;
  __shared__ float sbc[kTcBN];
  __shared__ int ok_s;
  uint8_t* smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t b = blockIdx.z;
  const int64_t m0 = (int64_t)blockIdx.y * kTcBM, n0 = (int64_t)blockIdx.x * kTcBN;
  const int nk = (int)(Kpad / kTcBK);

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) mbar_init(&full_bar[s], 1);
    mbar_init(&done_bar, 1);
    mbar_fence_init();
    ok_s = 1;
  }
  sbc[threadIdx.x] = scaleB[b * rowsB + n0 + threadIdx.x];
  if (warp == 0) {
    tmem_alloc(&tmem_base, Cfg::TMEM_COLS);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base;

  int issued[STAGES] = {0, 0}, consumed[STAGES] = {0, 0};
  auto load_stage = [&](int kt, int s) {
    uint8_t* st = smem + (size_t)s * Cfg::STAGE;
    mbar_expect_tx(&full_bar[s], Cfg::STAGE);
    for (int p = 0; p < kTcNP; ++p)
      tma_load_2d(st + p * Cfg::A_TILE, &mapA, &full_bar[s], kt * kTcBK, (int)((b * kTcNP + p) * rowsA + m0));
    for (int p = 0; p < kTcNP; ++p)
      tma_load_2d(st + kTcNP * Cfg::A_TILE + p * Cfg::B_TILE, &mapB, &full_bar[s], kt * kTcBK,
                  (int)((b * kTcNP + p) * rowsB + n0));
    issued[s]++;
  };
  if (threadIdx.x == 0)
    for (int s = 0; s < STAGES && s < nk; ++s) load_stage(s, s);

  float acc[kTcBN];
#pragma unroll
  for (int j = 0; j < kTcBN; ++j) acc[j] = 0.f;
  constexpr uint32_t ID = idesc_bf16(kTcBM, kTcBN);
  const uint32_t L0 = tmem, L1 = tmem + kTcBN, L2 = tmem + 2 * kTcBN;
  const uint32_t lanes = (uint32_t)(warp * 32) << 16;
  bool ok = true;
  for (int kt = 0; kt < nk; ++kt) {
    const int s = kt % STAGES;
    if (threadIdx.x == 0) {
      if (ok && mbar_wait(&full_bar[s], (uint32_t)((kt / STAGES) & 1))) {
        consumed[s]++;
        tc_fence_after();
        const uint32_t st = smem_u32(smem + (size_t)s * Cfg::STAGE);
#pragma unroll
        for (int kk = 0; kk < kTcBK / 16; ++kk) {
          const uint32_t koff = (uint32_t)kk * 32u;  // 16 BF16 = 32 bytes along K
          uint64_t ad[kTcNP], bd[kTcNP];
#pragma unroll
          for (int p = 0; p < kTcNP; ++p) {
            ad[p] = sw128_kmajor_desc(st + p * Cfg::A_TILE + koff);
            bd[p] = sw128_kmajor_desc(st + kTcNP * Cfg::A_TILE + p * Cfg::B_TILE + koff);
          }
          const uint32_t acc0 = kk == 0 ? 0u : 1u;  // every slice starts the level sums afresh
          umma_bf16(L0, ad[0], bd[0], ID, acc0);
          umma_bf16(L1, ad[0], bd[1], ID, acc0);
          umma_bf16(L1, ad[1], bd[0], ID, 1u);
          umma_bf16(L2, ad[0], bd[2], ID, acc0);
          umma_bf16(L2, ad[1], bd[1], ID, 1u);
          umma_bf16(L2, ad[2], bd[0], ID, 1u);
        }
      } else {
        ok = false;
        ok_s = 0;
      }
      umma_commit(&done_bar);  // arrives when this slice's MMAs (if any) are complete
    }
    const bool done = mbar_wait(&done_bar, (uint32_t)(kt & 1));
    tc_fence_after();
#pragma unroll
    for (int c0 = 0; c0 < kTcBN; c0 += 32) {
      float v0[32], v1[32], v2[32];
      tmem_ld32(L0 + lanes + (uint32_t)c0, v0);
      tmem_ld32(L1 + lanes + (uint32_t)c0, v1);
      tmem_ld32(L2 + lanes + (uint32_t)c0, v2);
      if (done) {
#pragma unroll
        for (int j = 0; j < 32; ++j) acc[c0 + j] += fmaf(v2[j], 0x1p-16f, v1[j] * 0x1p-8f) + v0[j];
      }
    }
    tc_fence_before();
    __syncthreads();
    if (!done || !ok_s) { ok = false; break; }
    if (threadIdx.x == 0 && kt + STAGES < nk) load_stage(kt + STAGES, s);
  }
  if (threadIdx.x == 0 && !ok) {
    // drain: copies issued but not consumed must land before the CTA exits
    for (int s = 0; s < STAGES; ++s)
      while (consumed[s] < issued[s]) {
        if (!mbar_wait(&full_bar[s], (uint32_t)(consumed[s] & 1))) break;
        consumed[s]++;
      }
  }
  if (ok) {
    const int64_t row = m0 + warp * 32 + lane;  // row of A'
    const float sa = scaleA[b * rowsA + row] * 0x1p-16f;
    float* Cb = C + b * sC * (CPLX ? 2 : 1);
#pragma unroll
    for (int j = 0; j < kTcBN; ++j) {
      const int64_t gn = n0 + j;
      const float v = acc[j] * sa * sbc[j];
      if (CPLX) {
        // rows 2r (real part) and 2r + 1 (imaginary part) sit in neighbouring lanes
        const float vi = __shfl_xor_sync(0xffffffffu, v, 1);
        const int64_t gm = row >> 1;
        if ((lane & 1) == 0 && gm < M && gn < N) {
          float2* cp = reinterpret_cast<float2*>(Cb) + gm * ldc + gn;
          float xr = ar * v - ai * vi;
          float xi = ar * vi + ai * v;
          if (br != 0.f || bi != 0.f) {
            const float2 o = *cp;
            xr += br * o.x - bi * o.y;
            xi += br * o.y + bi * o.x;
          }
          *cp = make_float2(xr, xi);
        }
      } else if (row < M && gn < N) {
        float* cp = Cb + row * ldc + gn;
        float x = ar * v;
        if (br != 0.f) x += br * *cp;
        *cp = x;
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, Cfg::TMEM_COLS);
}

// ------------------------------------------------------------------ host side
static size_t align256(size_t x) { return (x + 255) & ~size_t(255); }
static int64_t round_up(int64_t x, int64_t m) { return (x + m - 1) / m * m; }

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static std::once_flag once;
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// 2-D map over BF16 digit rows (inner = Kpad elements), boxes of 64 x box_rows
static int make_map(CUtensorMap* map, void* base, uint64_t inner, uint64_t outer, uint32_t box_rows) {
  PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
  if (!fn) return TNC_ERR_CUDA;
  cuuint64_t dims[2] = {inner, outer};
  cuuint64_t strides[1] = {inner * sizeof(__nv_bfloat16)};
  cuuint32_t box[2] = {(cuuint32_t)kTcBK, box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims, strides, box, es,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? TNC_OK : TNC_ERR_CUDA;
}

struct TcLayout {
  int64_t MoPad, NPad, Kpad, MsPad;  // rows of A' (padded), of B', K' padded, source rows of A (padded)
  size_t a_off, b_off, sa_off, sb_off, total;
};
static TcLayout tc_layout(bool cplx, int64_t m, int64_t n, int64_t k, int64_t batch) {
  TcLayout L;
  L.MoPad = round_up(cplx ? 2 * m : m, kTcBM);
  L.MsPad = cplx ? L.MoPad / 2 : L.MoPad;
  L.NPad = round_up(n, kTcBN);
  L.Kpad = round_up(cplx ? 2 * k : k, kTcBK);
  const size_t a = (size_t)batch * kTcNP * L.MoPad * L.Kpad * sizeof(__nv_bfloat16);
  const size_t bb = (size_t)batch * kTcNP * L.NPad * L.Kpad * sizeof(__nv_bfloat16);
  L.a_off = 0;
  L.b_off = align256(a);
  L.sa_off = L.b_off + align256(bb);
  L.sb_off = L.sa_off + align256((size_t)batch * L.MoPad * sizeof(float));
  L.total = L.sb_off + align256((size_t)batch * L.NPad * sizeof(float));
  return L;
}

template <bool CPLX>
static int ensure_tc_attr() {
  static std::atomic<unsigned long long> mask{0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return TNC_ERR_CUDA;
  const unsigned long long bit = 1ull << (dev & 63);
  if (mask.load() & bit) return TNC_OK;
  if (cudaFuncSetAttribute((const void*)gemm_tc_kernel<CPLX>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)TcCfg::SMEM) != cudaSuccess)
    return TNC_ERR_CUDA;
  mask.fetch_or(bit);
  return TNC_OK;
}

template <bool CPLX>
static int gemm_tc_impl(int opA, int opB, int64_t m, int64_t n, int64_t k, const double* alpha, const float* A,
                        int64_t lda, int64_t sA, const float* B, int64_t ldb, int64_t sB, const double* beta, float* C,
                        int64_t ldc, int64_t sC, int64_t batch, void* work, size_t wb, cudaStream_t st) {
  if (m <= 0 || n <= 0 || k <= 0 || batch <= 0 || batch > 65535 || !A || !B || !C || !work || !alpha || !beta)
    return TNC_ERR_ARG;
  if (opA < 0 || opA > 3 || opB < 0 || opB > 3 || ldc < n) return TNC_ERR_ARG;
  TcLayout L = tc_layout(CPLX, m, n, k, batch);
  if (wb < L.total) return TNC_ERR_WORKSPACE;
  if ((uint64_t)batch * kTcNP * (L.MoPad > L.NPad ? L.MoPad : L.NPad) >= (1ull << 31)) return TNC_ERR_ARG;
  char* w = (char*)work;
  __nv_bfloat16* wA = reinterpret_cast<__nv_bfloat16*>(w + L.a_off);
  __nv_bfloat16* wB = reinterpret_cast<__nv_bfloat16*>(w + L.b_off);
  float* sa = reinterpret_cast<float*>(w + L.sa_off);
  float* sbv = reinterpret_cast<float*>(w + L.sb_off);
  tc_split_kernel<CPLX><<<grid1d(batch * L.MsPad * 32, 256), 256, 0, st>>>(A, opA, 0, m, k, lda, sA, batch, L.MsPad,
                                                                         L.MoPad, L.Kpad, wA, sa);
  tc_split_kernel<CPLX><<<grid1d(batch * L.NPad * 32, 256), 256, 0, st>>>(B, opB, 1, n, k, ldb, sB, batch, L.NPad,
                                                                        L.NPad, L.Kpad, wB, sbv);
  CUtensorMap mapA, mapB;
  if (make_map(&mapA, wA, (uint64_t)L.Kpad, (uint64_t)(batch * kTcNP * L.MoPad), kTcBM)) return TNC_ERR_CUDA;
  if (make_map(&mapB, wB, (uint64_t)L.Kpad, (uint64_t)(batch * kTcNP * L.NPad), kTcBN)) return TNC_ERR_CUDA;
  if (int rc = ensure_tc_attr<CPLX>()) return rc;
  dim3 grid((unsigned)(L.NPad / kTcBN), (unsigned)(L.MoPad / kTcBM), (unsigned)batch);
  gemm_tc_kernel<CPLX><<<grid, 128, TcCfg::SMEM, st>>>(mapA, mapB, m, n, L.Kpad, L.MoPad, L.NPad, sa, sbv,
                                                       (float)alpha[0], (float)alpha[1], (float)beta[0],
                                                       (float)beta[1], C, ldc, sC);
  return launch_status(3);
}

}  // namespace tnc

using namespace tnc;

extern "C" int tnc_gemm_tc_workspace_size(int dtype, int64_t m, int64_t n, int64_t k, int64_t batch, size_t* bytes) {
  if ((dtype != TNC_F32 && dtype != TNC_C64) || m <= 0 || n <= 0 || k <= 0 || batch <= 0 || !bytes) return TNC_ERR_ARG;
  *bytes = tc_layout(dtype == TNC_C64, m, n, k, batch).total;
  return TNC_OK;
}

extern "C" int tnc_gemm_tc(int dtype, int opA, int opB, int64_t m, int64_t n, int64_t k, const double* alpha,
                           const void* A, int64_t lda, int64_t strideA, const void* B, int64_t ldb, int64_t strideB,
                           const double* beta, void* C, int64_t ldc, int64_t strideC, int64_t batch, void* work,
                           size_t work_bytes, void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == TNC_C64)
    return gemm_tc_impl<true>(opA, opB, m, n, k, alpha, (const float*)A, lda, strideA, (const float*)B, ldb, strideB,
                              beta, (float*)C, ldc, strideC, batch, work, work_bytes, st);
  if (dtype == TNC_F32)
    return gemm_tc_impl<false>(opA, opB, m, n, k, alpha, (const float*)A, lda, strideA, (const float*)B, ldb, strideB,
                               beta, (float*)C, ldc, strideC, batch, work, work_bytes, st);
  return TNC_ERR_ARG;
}

extern "C" int tnc_gemm_tc_error(void) {
  int h = 0, z = 0;
  if (cudaMemcpyFromSymbol(&h, g_tc_error, sizeof(int)) != cudaSuccess) return -1;
  if (h) cudaMemcpyToSymbol(g_tc_error, &z, sizeof(int));
  return h;
}
