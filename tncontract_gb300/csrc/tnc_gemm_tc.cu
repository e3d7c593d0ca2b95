// Tensor-core GEMM for the FP32-class contractions (np.tensordot in
// tncontract/tensor.py:735 and the sweep's absorption products) on GB300's
// 5th-generation tensor cores.
//
// Precision: operands are split into a TF32 "hi" part (round to nearest) and
// the FP32 remainder "lo"; each product is hi*hi + hi*lo + lo*hi accumulated
// in FP32 in tensor memory (the lo*lo term is below FP32 resolution), which
// recovers FP32-class accuracy from TF32 MMAs.  Complex products use four
// real products per split term, the negative one through the MMA's negate-A
// bit.
//
// Data path: a split kernel writes op(A) (M x K) and op(B)^T (N x K) as
// planar, K-contiguous FP32 planes ((hi, lo) or (re_hi, re_lo, im_hi, im_lo)),
// zero-padded to the tile grid.  The GEMM kernel (one CTA per 128 x BN
// output tile, 4 warps) has thread 0 stream 32-deep K slices of every plane
// into shared memory with TMA (cp.async.bulk.tensor, 128-byte swizzle,
// completion on an mbarrier) in a multi-stage ring, and issue tcgen05.mma
// (kind::tf32, M=128, K=8 per instruction) from shared-memory descriptors
// into a TMEM accumulator; tcgen05.commit releases each stage.  The four
// warps then read the accumulator with tcgen05.ld (warp w owns TMEM lanes
// 32w..32w+31 = tile rows) and write C = alpha*acc + beta*C.
//
// Every mbarrier wait is bounded; a wait that gives up records an error
// (tnc_gemm_tc_error), waits (bounded) for the copies and MMAs it issued and
// frees its tensor memory before returning.
#include "tnc_common.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>

#include <atomic>
#include <mutex>

namespace tnc {

constexpr int kTcBM = 128;                 // tile rows (UMMA M)
constexpr int kTcBK = 32;                  // K elements per stage = one 128-byte swizzle atom of FP32
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

__device__ __forceinline__ void umma_tf32(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n"
      " .reg .pred p;\n"
      " setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n"
      "}\n" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}
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

// Instruction descriptor, kind::tf32: D = F32, A = B = TF32, both K-major.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N, bool negA) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((negA ? 1u : 0u) << 13) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ float tf32_rn(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// ------------------------------------------------------------------ split kernel
// dst planes [batch][plane][rowsPad][Kpad]; real planes (hi, lo), complex planes
// (re_hi, re_lo, im_hi, im_lo).  Logical operand X (rows x K): for A, X = op(A);
// for B, X = op(B)^T.
template <bool CPLX>
__global__ void tc_split_kernel(const float* __restrict__ src, int op, int isB, int64_t rows, int64_t K, int64_t ld,
                                int64_t sbatch, int64_t batch, int64_t rowsPad, int64_t Kpad, float* __restrict__ dst) {
  constexpr int NP = CPLX ? 4 : 2;
  const bool trans = (op == TNC_OP_T || op == TNC_OP_C);
  const bool cj = (op == TNC_OP_C || op == TNC_OP_R);
  const int64_t plane = rowsPad * Kpad;
  const int64_t total = batch * plane;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / plane;
    const int64_t rem = e - b * plane;
    const int64_t r = rem / Kpad, k = rem - r * Kpad;
    float re = 0.f, im = 0.f;
    if (r < rows && k < K) {
      // A: element (r, k) of op(A) = A[r][k] (N/R) or A[k][r] (T/C)
      // B: element (r, k) of op(B)^T = op(B)[k][r] = B[k][r] (N/R) or B[r][k] (T/C)
      const bool rowmajor_rk = isB ? trans : !trans;
      const int64_t off = b * sbatch + (rowmajor_rk ? (r * ld + k) : (k * ld + r));
      if (CPLX) {
        const float2 v = reinterpret_cast<const float2*>(src)[off];
        re = v.x;
        im = cj ? -v.y : v.y;
      } else {
        re = src[off];
      }
    }
    float* base = dst + b * NP * plane + rem;
    const float hr = tf32_rn(re);
    base[0] = hr;
    base[plane] = re - hr;
    if (CPLX) {
      const float hi = tf32_rn(im);
      base[2 * plane] = hi;
      base[3 * plane] = im - hi;
    }
  }
}

// ------------------------------------------------------------------ GEMM kernel
template <bool CPLX, int BN, int STAGES>
struct TcCfg {
  static constexpr int NP = CPLX ? 4 : 2;
  static constexpr uint32_t A_TILE = kTcBM * 128;  // bytes: 128 rows x 32 FP32
  static constexpr uint32_t B_TILE = BN * 128;
  static constexpr uint32_t STAGE = NP * (A_TILE + B_TILE);
  static constexpr uint32_t SMEM = STAGES * STAGE + 1024;  // + alignment slack
  static constexpr uint32_t TMEM_COLS = CPLX ? 2 * BN : BN;
};

template <bool CPLX, int BN, int STAGES>
__global__ void __launch_bounds__(128, 1)
gemm_tc_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, int64_t M,
               int64_t N, int64_t Kpad, int64_t rowsA, int64_t rowsB, float ar, float ai, float br, float bi,
               float* __restrict__ C, int64_t ldc, int64_t sC) {
  typedef TcCfg<CPLX, BN, STAGES> Cfg;
  constexpr int NP = Cfg::NP;
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t full_bar[STAGES];
  __shared__ uint64_t mma_bar[STAGES];
  __shared__ uint64_t done_bar;
  __shared__ uint32_t tmem_base;
  uint8_t* smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t b = blockIdx.z;
  const int64_t m0 = (int64_t)blockIdx.y * kTcBM, n0 = (int64_t)blockIdx.x * BN;
  const int nk = (int)(Kpad / kTcBK);

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&mma_bar[s], 1);
    }
    mbar_init(&done_bar, 1);
    mbar_fence_init();
  }
  if (warp == 0) {
    tmem_alloc(&tmem_base, Cfg::TMEM_COLS);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base;

  if (threadIdx.x == 0) {
    int issued[STAGES];
    int consumed[STAGES];
    for (int s = 0; s < STAGES; ++s) issued[s] = consumed[s] = 0;
    auto load_stage = [&](int kt, int s) {
      uint8_t* st = smem + (size_t)s * Cfg::STAGE;
      mbar_expect_tx(&full_bar[s], Cfg::STAGE);
      for (int p = 0; p < NP; ++p)
        tma_load_2d(st + p * Cfg::A_TILE, &mapA, &full_bar[s], kt * kTcBK, (int)((b * NP + p) * rowsA + m0));
      for (int p = 0; p < NP; ++p)
        tma_load_2d(st + NP * Cfg::A_TILE + p * Cfg::B_TILE, &mapB, &full_bar[s], kt * kTcBK,
                    (int)((b * NP + p) * rowsB + n0));
      issued[s]++;
    };
    for (int s = 0; s < STAGES && s < nk; ++s) load_stage(s, s);
    constexpr uint32_t ID = idesc_tf32(kTcBM, BN, false);
    constexpr uint32_t IDN = idesc_tf32(kTcBM, BN, true);
    bool ok = true;
    int kt = 0;
    for (; kt < nk; ++kt) {
      const int s = kt % STAGES;
      const uint32_t ph = (uint32_t)((kt / STAGES) & 1);
      if (!mbar_wait(&full_bar[s], ph)) { ok = false; break; }
      consumed[s]++;
      tc_fence_after();
      const uint32_t st = smem_u32(smem + (size_t)s * Cfg::STAGE);
#pragma unroll
      for (int kk = 0; kk < kTcBK / 8; ++kk) {
        const uint32_t koff = (uint32_t)kk * 32u;  // 8 TF32 = 32 bytes along K
        uint64_t ad[NP], bd[NP];
#pragma unroll
        for (int p = 0; p < NP; ++p) {
          ad[p] = sw128_kmajor_desc(st + p * Cfg::A_TILE + koff);
          bd[p] = sw128_kmajor_desc(st + NP * Cfg::A_TILE + p * Cfg::B_TILE + koff);
        }
        const uint32_t first = (kt == 0 && kk == 0) ? 0u : 1u;
        if (!CPLX) {
          umma_tf32(tmem, ad[0], bd[0], ID, first);  // hi*hi
          umma_tf32(tmem, ad[0], bd[1], ID, 1u);     // hi*lo
          umma_tf32(tmem, ad[1], bd[0], ID, 1u);     // lo*hi
        } else {
          const uint32_t cr = tmem, ci = tmem + BN;
          // planes: 0 re_hi, 1 re_lo, 2 im_hi, 3 im_lo
#pragma unroll
          for (int t = 0; t < 3; ++t) {
            const int ah = (t == 2) ? 1 : 0;  // a: hi, hi, lo
            const int bh = (t == 1) ? 1 : 0;  // b: hi, lo, hi
            const uint32_t acc = (t == 0) ? first : 1u;
            umma_tf32(cr, ad[0 + ah], bd[0 + bh], ID, acc);   // + Ar Br
            umma_tf32(cr, ad[2 + ah], bd[2 + bh], IDN, 1u);   // - Ai Bi
            umma_tf32(ci, ad[0 + ah], bd[2 + bh], ID, acc);   // + Ar Bi
            umma_tf32(ci, ad[2 + ah], bd[0 + bh], ID, 1u);    // + Ai Br
          }
        }
      }
      umma_commit(&mma_bar[s]);
      if (kt + STAGES < nk) {
        if (!mbar_wait(&mma_bar[s], ph)) { ok = false; break; }
        load_stage(kt + STAGES, s);
      }
    }
    umma_commit(&done_bar);
    if (!ok) {
      // drain: copies issued but not consumed must land before the CTA exits
      for (int s = 0; s < STAGES; ++s)
        while (consumed[s] < issued[s]) {
          const uint32_t ph = (uint32_t)(consumed[s] & 1);
          if (!mbar_wait(&full_bar[s], ph)) break;
          consumed[s]++;
        }
    }
  }
  __syncthreads();
  const bool done = mbar_wait(&done_bar, 0);
  tc_fence_after();
  const int row = warp * 32 + lane;
  const int64_t gm = m0 + row;
  float* Cb = C + b * sC * (CPLX ? 2 : 1);
#pragma unroll 1
  for (int c0 = 0; c0 < BN; c0 += 32) {
    float vr[32], vi[32];
    tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, vr);
    if (CPLX) tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(BN + c0), vi);
    if (done && gm < M) {
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const int64_t gn = n0 + c0 + j;
        if (gn < N) {
          if (CPLX) {
            float2* cp = reinterpret_cast<float2*>(Cb) + gm * ldc + gn;
            float xr = ar * vr[j] - ai * vi[j];
            float xi = ar * vi[j] + ai * vr[j];
            if (br != 0.f || bi != 0.f) {
              const float2 o = *cp;
              xr += br * o.x - bi * o.y;
              xi += br * o.y + bi * o.x;
            }
            *cp = make_float2(xr, xi);
          } else {
            float* cp = Cb + gm * ldc + gn;
            float x = ar * vr[j];
            if (br != 0.f) x += br * *cp;
            *cp = x;
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (!done && threadIdx.x == 0) mbar_wait(&done_bar, 0);  // one more bounded wait for our own MMAs
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

// 2-D map over planar FP32 rows (inner = Kpad elements), boxes of 32 x box_rows
static int make_map(CUtensorMap* map, float* base, uint64_t inner, uint64_t outer, uint32_t box_rows) {
  PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
  if (!fn) return TNC_ERR_CUDA;
  cuuint64_t dims[2] = {inner, outer};
  cuuint64_t strides[1] = {inner * sizeof(float)};
  cuuint32_t box[2] = {(cuuint32_t)kTcBK, box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? TNC_OK : TNC_ERR_CUDA;
}

struct TcLayout {
  int64_t Mpad, Npad, Kpad;
  size_t a_off, b_off, total;
  int np, bn;
};
static TcLayout tc_layout(bool cplx, int64_t m, int64_t n, int64_t k, int64_t batch) {
  TcLayout L;
  L.np = cplx ? 4 : 2;
  L.bn = cplx ? 64 : 128;
  L.Mpad = round_up(m, kTcBM);
  L.Npad = round_up(n, L.bn);
  L.Kpad = round_up(k, kTcBK);
  const size_t a = (size_t)batch * L.np * L.Mpad * L.Kpad * sizeof(float);
  const size_t b = (size_t)batch * L.np * L.Npad * L.Kpad * sizeof(float);
  L.a_off = 0;
  L.b_off = align256(a);
  L.total = L.b_off + align256(b);
  return L;
}

template <bool CPLX, int BN, int STAGES>
static int ensure_tc_attr() {
  static std::atomic<unsigned long long> mask{0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return TNC_ERR_CUDA;
  const unsigned long long bit = 1ull << (dev & 63);
  if (mask.load() & bit) return TNC_OK;
  if (cudaFuncSetAttribute((const void*)gemm_tc_kernel<CPLX, BN, STAGES>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TcCfg<CPLX, BN, STAGES>::SMEM) !=
      cudaSuccess)
    return TNC_ERR_CUDA;
  mask.fetch_or(bit);
  return TNC_OK;
}

template <bool CPLX>
static int gemm_tc_impl(int opA, int opB, int64_t m, int64_t n, int64_t k, const double* alpha, const float* A,
                        int64_t lda, int64_t sA, const float* B, int64_t ldb, int64_t sB, const double* beta, float* C,
                        int64_t ldc, int64_t sC, int64_t batch, void* work, size_t wb, cudaStream_t st) {
  constexpr int BN = CPLX ? 64 : 128;
  constexpr int STAGES = CPLX ? 2 : 3;
  if (m <= 0 || n <= 0 || k <= 0 || batch <= 0 || batch > 65535 || !A || !B || !C || !work || !alpha || !beta)
    return TNC_ERR_ARG;
  if (opA < 0 || opA > 3 || opB < 0 || opB > 3 || ldc < n) return TNC_ERR_ARG;
  TcLayout L = tc_layout(CPLX, m, n, k, batch);
  if (wb < L.total) return TNC_ERR_WORKSPACE;
  if ((uint64_t)batch * L.np * (L.Mpad > L.Npad ? L.Mpad : L.Npad) >= (1ull << 31)) return TNC_ERR_ARG;
  float* wA = reinterpret_cast<float*>((char*)work + L.a_off);
  float* wB = reinterpret_cast<float*>((char*)work + L.b_off);
  tc_split_kernel<CPLX><<<grid1d(batch * L.Mpad * L.Kpad, 256), 256, 0, st>>>(A, opA, 0, m, k, lda, sA, batch,
                                                                              L.Mpad, L.Kpad, wA);
  tc_split_kernel<CPLX><<<grid1d(batch * L.Npad * L.Kpad, 256), 256, 0, st>>>(B, opB, 1, n, k, ldb, sB, batch,
                                                                              L.Npad, L.Kpad, wB);
  CUtensorMap mapA, mapB;
  if (make_map(&mapA, wA, (uint64_t)L.Kpad, (uint64_t)(batch * L.np * L.Mpad), kTcBM)) return TNC_ERR_CUDA;
  if (make_map(&mapB, wB, (uint64_t)L.Kpad, (uint64_t)(batch * L.np * L.Npad), BN)) return TNC_ERR_CUDA;
  if (int rc = ensure_tc_attr<CPLX, BN, STAGES>()) return rc;
  dim3 grid((unsigned)(L.Npad / BN), (unsigned)(L.Mpad / kTcBM), (unsigned)batch);
  gemm_tc_kernel<CPLX, BN, STAGES><<<grid, 128, TcCfg<CPLX, BN, STAGES>::SMEM, st>>>(
      mapA, mapB, m, n, L.Kpad, L.Mpad, L.Npad, (float)alpha[0], (float)alpha[1], (float)beta[0], (float)beta[1], C,
      ldc, sC);
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
