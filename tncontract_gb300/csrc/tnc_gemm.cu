// Batched GEMM on row-major operands with transpose / conjugate options
// (the product inside np.tensordot, tncontract/tensor.py:735).
//
// CUDA-core tiled kernel: a 64x64 output tile per 256-thread CTA, 4x4
// register micro-tile per thread, K in slices of BK staged in shared memory
// k-major (so a thread reads its 4 consecutive values of each operand with
// 16-byte loads).  Two shared-memory buffers: the next slice is fetched into
// registers while the current one is multiplied, then stored to the other
// buffer -- one CTA barrier per slice and the global-load latency hidden
// behind the FMAs.  Whether an operand's contiguous axis is K (A: N/R,
// B: T/C) or M/N (A: T/C, B: N/R) is a template parameter, so each tile load
// is a coalesced, branch-free pattern.  This is the FP64 / complex128 path
// (GB300 runs FP64 on the CUDA cores), the FP32-accurate path of the blocked
// QR's products, and the general path for small or odd shapes; FP32-class
// products that tolerate TF32-split accuracy can use the tcgen05 kernel.
#include "tnc_common.cuh"

namespace tnc {

template <typename T>
__device__ __forceinline__ T maybe_conj(T v, bool c) { return c ? conj_(v) : v; }

// four consecutive elements of a 16-byte-aligned shared-memory row
__device__ __forceinline__ void lds4(const float* p, float (&v)[4]) {
  const float4 q = *reinterpret_cast<const float4*>(p);
  v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
}
__device__ __forceinline__ void lds4(const double* p, double (&v)[4]) {
  const double2 q0 = reinterpret_cast<const double2*>(p)[0], q1 = reinterpret_cast<const double2*>(p)[1];
  v[0] = q0.x; v[1] = q0.y; v[2] = q1.x; v[3] = q1.y;
}
__device__ __forceinline__ void lds4(const c64* p, c64 (&v)[4]) {
  const float4 q0 = reinterpret_cast<const float4*>(p)[0], q1 = reinterpret_cast<const float4*>(p)[1];
  v[0] = c64(q0.x, q0.y); v[1] = c64(q0.z, q0.w); v[2] = c64(q1.x, q1.y); v[3] = c64(q1.z, q1.w);
}
__device__ __forceinline__ void lds4(const c128* p, c128 (&v)[4]) {
#pragma unroll
  for (int i = 0; i < 4; ++i) v[i] = p[i];
}

template <typename T>
struct GemmTile {
  static constexpr int BM = 64, BN = 64;
  static constexpr int BK = sizeof(T) >= 16 ? 8 : 16;
  static constexpr int PAD = sizeof(T) >= 16 ? 1 : 16 / (int)sizeof(T);  // rows stay 16-byte aligned
  static constexpr int LD = BM + PAD;
  static constexpr int PER = BM * BK / 256;  // tile elements each thread moves
};

// Fetch the BK-slice at k0 of a 64-row operand tile into registers.
// KMAJOR: element (r, k) at X[r * ld + k] (lanes run along k);
// else:   element (r, k) at X[k * ld + r] (lanes run along r).
template <typename T, bool KMAJOR>
__device__ __forceinline__ void tile_fetch(const T* __restrict__ X, int64_t ld, int64_t r0, int64_t R, int64_t k0,
                                           int64_t K, T (&v)[GemmTile<T>::PER]) {
  constexpr int BK = GemmTile<T>::BK;
  const int t = threadIdx.x;
#pragma unroll
  for (int j = 0; j < GemmTile<T>::PER; ++j) {
    int r, k;
    if (KMAJOR) { k = t % BK; r = t / BK + (256 / BK) * j; }
    else { r = t & 63; k = (t >> 6) + 4 * j; }
    const int64_t gr = r0 + r, gk = k0 + k;
    v[j] = (gr < R && gk < K) ? (KMAJOR ? X[gr * ld + gk] : X[gk * ld + gr]) : zero_<T>();
  }
}

template <typename T, bool KMAJOR>
__device__ __forceinline__ void tile_store(T* s, const T (&v)[GemmTile<T>::PER], bool cj) {
  constexpr int BK = GemmTile<T>::BK, LD = GemmTile<T>::LD;
  const int t = threadIdx.x;
#pragma unroll
  for (int j = 0; j < GemmTile<T>::PER; ++j) {
    int r, k;
    if (KMAJOR) { k = t % BK; r = t / BK + (256 / BK) * j; }
    else { r = t & 63; k = (t >> 6) + 4 * j; }
    s[k * LD + r] = maybe_conj(v[j], cj);
  }
}

// One 64 x 64 output tile (rows m0.., columns n0..) of C = alpha op(A) op(B) + beta C.
template <typename T, bool AK, bool BKM>
__device__ __forceinline__ void gemm_tile(int64_t M, int64_t N, int64_t K, bool aC, bool bC, T alpha,
                                          const T* __restrict__ Ab, int64_t lda, const T* __restrict__ Bb,
                                          int64_t ldb, T beta, T* __restrict__ Cb, int64_t ldc, int64_t m0,
                                          int64_t n0, T (*As)[GemmTile<T>::BK * GemmTile<T>::LD],
                                          T (*Bs)[GemmTile<T>::BK * GemmTile<T>::LD]) {
  typedef GemmTile<T> G;
  constexpr int TM = 4, TN = 4;
  const int tid = threadIdx.x;
  const int tx = tid % (G::BN / TN), ty = tid / (G::BN / TN);
  const bool beta_zero = (abs2_(beta) == 0);
  T acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = zero_<T>();

  T va[G::PER], vb[G::PER];
  tile_fetch<T, AK>(Ab, lda, m0, M, 0, K, va);
  tile_fetch<T, BKM>(Bb, ldb, n0, N, 0, K, vb);
  tile_store<T, AK>(As[0], va, aC);
  tile_store<T, BKM>(Bs[0], vb, bC);
  __syncthreads();
  int buf = 0;
  for (int64_t k0 = 0; k0 < K; k0 += G::BK) {
    const bool more = k0 + G::BK < K;
    if (more) {
      tile_fetch<T, AK>(Ab, lda, m0, M, k0 + G::BK, K, va);
      tile_fetch<T, BKM>(Bb, ldb, n0, N, k0 + G::BK, K, vb);
    }
    const T* as = As[buf];
    const T* bs = Bs[buf];
#pragma unroll
    for (int kk = 0; kk < G::BK; ++kk) {
      T a[TM], b[TN];
      lds4(as + kk * G::LD + ty * TM, a);
      lds4(bs + kk * G::LD + tx * TN, b);
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) fma_(acc[i][j], a[i], b[j]);
    }
    if (more) {
      tile_store<T, AK>(As[buf ^ 1], va, aC);
      tile_store<T, BKM>(Bs[buf ^ 1], vb, bC);
    }
    __syncthreads();
    buf ^= 1;
  }
#pragma unroll
  for (int i = 0; i < TM; ++i) {
    const int64_t gm = m0 + ty * TM + i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const int64_t gn = n0 + tx * TN + j;
      if (gn >= N) continue;
      T v = alpha * acc[i][j];
      if (!beta_zero) v += beta * Cb[gm * ldc + gn];
      Cb[gm * ldc + gn] = v;
    }
  }
}

template <typename T, bool AK, bool BKM>
__global__ void __launch_bounds__(256)
gemm_simt_kernel(int64_t M, int64_t N, int64_t K, bool aC, bool bC, T alpha, const T* __restrict__ A, int64_t lda,
                 int64_t sA, const T* __restrict__ B, int64_t ldb, int64_t sB, T beta, T* __restrict__ C,
                 int64_t ldc, int64_t sC, int64_t batch) {
  typedef GemmTile<T> G;
  __shared__ __align__(16) T As[2][G::BK * G::LD];
  __shared__ __align__(16) T Bs[2][G::BK * G::LD];
  const int64_t m0 = (int64_t)blockIdx.y * G::BM, n0 = (int64_t)blockIdx.x * G::BN;
  for (int64_t bz = blockIdx.z; bz < batch; bz += gridDim.z) {
    gemm_tile<T, AK, BKM>(M, N, K, aC, bC, alpha, A + bz * sA, lda, B + bz * sB, ldb, beta, C + bz * sC, ldc, m0,
                          n0, As, Bs);
    __syncthreads();  // the next batch entry reuses the shared tiles
  }
}

// Independent products of different shapes in one launch: the CTAs of the
// grid are dealt out to the problems' output tiles (problem q owns tiles
// [tile0_q, tile0_{q+1})), each problem with its own operand layouts.
struct GroupProblem {
  int64_t m, n, k, lda, ldb, ldc, tile0, tiles_n;
  const void* A;
  const void* B;
  void* C;
  double alpha[2], beta[2];
  int opA, opB;
};
constexpr int kGroupMax = 16;
struct GemmGroup {
  int count;
  GroupProblem p[kGroupMax];
};

template <typename T>
__global__ void __launch_bounds__(256) gemm_grouped_kernel(const __grid_constant__ GemmGroup g) {
  typedef GemmTile<T> G;
  __shared__ __align__(16) T As[2][G::BK * G::LD];
  __shared__ __align__(16) T Bs[2][G::BK * G::LD];
  int q = 0;
  while (q + 1 < g.count && (int64_t)blockIdx.x >= g.p[q + 1].tile0) ++q;
  const GroupProblem& P = g.p[q];
  const int64_t t = (int64_t)blockIdx.x - P.tile0;
  const int64_t m0 = (t / P.tiles_n) * G::BM, n0 = (t % P.tiles_n) * G::BN;
  const T alpha = from_pair<T>(P.alpha), beta = from_pair<T>(P.beta);
  const bool aK = (P.opA == TNC_OP_N || P.opA == TNC_OP_R), bK = (P.opB == TNC_OP_T || P.opB == TNC_OP_C);
  const bool aC = (P.opA == TNC_OP_C || P.opA == TNC_OP_R), bC = (P.opB == TNC_OP_C || P.opB == TNC_OP_R);
  const T* A = (const T*)P.A;
  const T* B = (const T*)P.B;
  T* C = (T*)P.C;
  if (aK && bK) gemm_tile<T, true, true>(P.m, P.n, P.k, aC, bC, alpha, A, P.lda, B, P.ldb, beta, C, P.ldc, m0, n0, As, Bs);
  else if (aK) gemm_tile<T, true, false>(P.m, P.n, P.k, aC, bC, alpha, A, P.lda, B, P.ldb, beta, C, P.ldc, m0, n0, As, Bs);
  else if (bK) gemm_tile<T, false, true>(P.m, P.n, P.k, aC, bC, alpha, A, P.lda, B, P.ldb, beta, C, P.ldc, m0, n0, As, Bs);
  else gemm_tile<T, false, false>(P.m, P.n, P.k, aC, bC, alpha, A, P.lda, B, P.ldb, beta, C, P.ldc, m0, n0, As, Bs);
}

template <typename T>
int gemm_grouped_launch(int count, const tnc_gemm_problem* probs, cudaStream_t st) {
  if (count <= 0 || count > kGroupMax || !probs) return TNC_ERR_ARG;
  GemmGroup g;
  g.count = 0;
  int64_t tiles = 0;
  for (int i = 0; i < count; ++i) {
    const tnc_gemm_problem& p = probs[i];
    if (p.m < 0 || p.n < 0 || p.k <= 0 || p.opA < 0 || p.opA > 3 || p.opB < 0 || p.opB > 3 || p.ldc < p.n)
      return TNC_ERR_ARG;
    if (p.m == 0 || p.n == 0) continue;
    if (!p.A || !p.B || !p.C) return TNC_ERR_ARG;
    GroupProblem& q = g.p[g.count++];
    q.m = p.m; q.n = p.n; q.k = p.k; q.lda = p.lda; q.ldb = p.ldb; q.ldc = p.ldc;
    q.A = p.A; q.B = p.B; q.C = p.C; q.opA = p.opA; q.opB = p.opB;
    q.alpha[0] = p.alpha[0]; q.alpha[1] = p.alpha[1]; q.beta[0] = p.beta[0]; q.beta[1] = p.beta[1];
    q.tiles_n = (p.n + GemmTile<T>::BN - 1) / GemmTile<T>::BN;
    q.tile0 = tiles;
    tiles += q.tiles_n * ((p.m + GemmTile<T>::BM - 1) / GemmTile<T>::BM);
  }
  if (g.count == 0) return TNC_OK;
  if (tiles > 0x7fffffff) return TNC_ERR_ARG;
  gemm_grouped_kernel<T><<<(unsigned)tiles, 256, 0, st>>>(g);
  return launch_status();
}

// C = beta*C when K == 0 (np.tensordot over no axes still has the outer
// product shape; with K == 0 the product is zero)
template <typename T>
__global__ void gemm_scale_c(int64_t M, int64_t N, T beta, T* C, int64_t ldc, int64_t sC, int64_t batch) {
  const int64_t total = M * N * batch;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t b = e / (M * N), r = e - b * M * N;
    int64_t i = r / N, j = r - i * N;
    T* c = C + b * sC + i * ldc + j;
    *c = (abs2_(beta) == 0) ? zero_<T>() : beta * *c;
  }
}

template <typename T>
int gemm_launch(int opA, int opB, int64_t m, int64_t n, int64_t k, T alpha, const T* A, int64_t lda,
                int64_t sA, const T* B, int64_t ldb, int64_t sB, T beta, T* C, int64_t ldc, int64_t sC,
                int64_t batch, cudaStream_t st) {
  if (m < 0 || n < 0 || k < 0 || batch < 0 || opA < 0 || opA > 3 || opB < 0 || opB > 3) return TNC_ERR_ARG;
  if (m == 0 || n == 0 || batch == 0) return TNC_OK;
  if (ldc < n) return TNC_ERR_ARG;
  if (k == 0) {
    gemm_scale_c<T><<<grid1d(m * n * batch, 256), 256, 0, st>>>(m, n, beta, C, ldc, sC, batch);
    return launch_status();
  }
  constexpr int BM = GemmTile<T>::BM, BN = GemmTile<T>::BN;
  int64_t gy = (m + BM - 1) / BM, gx = (n + BN - 1) / BN;
  if (gy > 65535) return TNC_ERR_ARG;
  if (gx > 0x7fffffff) return TNC_ERR_ARG;
  unsigned gz = (unsigned)(batch < 65535 ? batch : 65535);
  dim3 grid((unsigned)gx, (unsigned)gy, gz);
  // A is K-contiguous for N / R, B for T / C
  const bool aK = (opA == TNC_OP_N || opA == TNC_OP_R), bK = (opB == TNC_OP_T || opB == TNC_OP_C);
  const bool aC = (opA == TNC_OP_C || opA == TNC_OP_R), bC = (opB == TNC_OP_C || opB == TNC_OP_R);
#define TNC_GEMM_LAUNCH(AKV, BKV)                                                                              \
  gemm_simt_kernel<T, AKV, BKV><<<grid, 256, 0, st>>>(m, n, k, aC, bC, alpha, A, lda, sA, B, ldb, sB, beta, C, \
                                                      ldc, sC, batch)
  if (aK && bK) TNC_GEMM_LAUNCH(true, true);
  else if (aK) TNC_GEMM_LAUNCH(true, false);
  else if (bK) TNC_GEMM_LAUNCH(false, true);
  else TNC_GEMM_LAUNCH(false, false);
#undef TNC_GEMM_LAUNCH
  return launch_status();
}

template int gemm_launch<float>(int, int, int64_t, int64_t, int64_t, float, const float*, int64_t, int64_t,
                                const float*, int64_t, int64_t, float, float*, int64_t, int64_t, int64_t,
                                cudaStream_t);
template int gemm_launch<double>(int, int, int64_t, int64_t, int64_t, double, const double*, int64_t, int64_t,
                                 const double*, int64_t, int64_t, double, double*, int64_t, int64_t, int64_t,
                                 cudaStream_t);
template int gemm_launch<c64>(int, int, int64_t, int64_t, int64_t, c64, const c64*, int64_t, int64_t, const c64*,
                              int64_t, int64_t, c64, c64*, int64_t, int64_t, int64_t, cudaStream_t);
template int gemm_launch<c128>(int, int, int64_t, int64_t, int64_t, c128, const c128*, int64_t, int64_t,
                               const c128*, int64_t, int64_t, c128, c128*, int64_t, int64_t, int64_t,
                               cudaStream_t);

}  // namespace tnc

using namespace tnc;

extern "C" int tnc_gemm(int dtype, int opA, int opB, int64_t m, int64_t n, int64_t k, const double* alpha,
                        const void* A, int64_t lda, int64_t strideA, const void* B, int64_t ldb,
                        int64_t strideB, const double* beta, void* C, int64_t ldc, int64_t strideC,
                        int64_t batch, void* stream) {
  if (!alpha || !beta) return TNC_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  TNC_DISPATCH(dtype, T,
               return gemm_launch<T>(opA, opB, m, n, k, from_pair<T>(alpha), (const T*)A, lda, strideA,
                                     (const T*)B, ldb, strideB, from_pair<T>(beta), (T*)C, ldc, strideC, batch,
                                     st));
  return TNC_ERR_ARG;
}

extern "C" int tnc_gemm_grouped(int dtype, int count, const tnc_gemm_problem* problems, void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  TNC_DISPATCH(dtype, T, return gemm_grouped_launch<T>(count, problems, st));
  return TNC_ERR_ARG;
}
