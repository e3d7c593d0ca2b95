// Batched GEMM on row-major operands with transpose / conjugate options
// (the product inside np.tensordot, tncontract/tensor.py:735).
//
// CUDA-core tiled kernel: a 64x64 output tile per 256-thread CTA, 16-deep
// K slices staged in shared memory (k-major so the inner loop reads 4
// consecutive values of each operand), 4x4 register micro-tile per thread.
// Tile loads are coalesced along whichever axis is contiguous in memory for
// the requested op.  This is the FP64 / complex128 path (GB300 runs FP64 on
// the CUDA cores) and the general fallback for small or odd shapes; FP32
// class products large enough for the tensor cores go to the tcgen05 kernel.
#include "tnc_common.cuh"

namespace tnc {

template <typename T>
__device__ __forceinline__ T maybe_conj(T v, bool c) { return c ? conj_(v) : v; }

template <typename T, int BM, int BN, int BK>
__global__ void __launch_bounds__(256)
gemm_simt_kernel(int opA, int opB, int64_t M, int64_t N, int64_t K, T alpha, const T* __restrict__ A,
                 int64_t lda, int64_t sA, const T* __restrict__ B, int64_t ldb, int64_t sB, T beta,
                 T* __restrict__ C, int64_t ldc, int64_t sC, int64_t batch) {
  constexpr int TM = 4, TN = 4;
  constexpr int NT = 256;
  __shared__ T As[BK][BM + 1];
  __shared__ T Bs[BK][BN + 1];
  const int tid = threadIdx.x;
  const int tx = tid % (BN / TN), ty = tid / (BN / TN);
  const int64_t m0 = (int64_t)blockIdx.y * BM, n0 = (int64_t)blockIdx.x * BN;
  const bool aT = (opA == TNC_OP_T || opA == TNC_OP_C), aC = (opA == TNC_OP_C || opA == TNC_OP_R);
  const bool bT = (opB == TNC_OP_T || opB == TNC_OP_C), bC = (opB == TNC_OP_C || opB == TNC_OP_R);

  for (int64_t bz = blockIdx.z; bz < batch; bz += gridDim.z) {
    const T* Ab = A + bz * sA;
    const T* Bb = B + bz * sB;
    T* Cb = C + bz * sC;
    T acc[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
      for (int j = 0; j < TN; ++j) acc[i][j] = zero_<T>();

    for (int64_t k0 = 0; k0 < K; k0 += BK) {
#pragma unroll
      for (int e = tid; e < BM * BK; e += NT) {
        int m, k;
        if (aT) { m = e % BM; k = e / BM; } else { k = e % BK; m = e / BK; }
        int64_t gm = m0 + m, gk = k0 + k;
        T v = zero_<T>();
        if (gm < M && gk < K) v = aT ? Ab[gk * lda + gm] : Ab[gm * lda + gk];
        As[k][m] = maybe_conj(v, aC);
      }
#pragma unroll
      for (int e = tid; e < BN * BK; e += NT) {
        int n, k;
        if (bT) { k = e % BK; n = e / BK; } else { n = e % BN; k = e / BN; }
        int64_t gn = n0 + n, gk = k0 + k;
        T v = zero_<T>();
        if (gn < N && gk < K) v = bT ? Bb[gn * ldb + gk] : Bb[gk * ldb + gn];
        Bs[k][n] = maybe_conj(v, bC);
      }
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < BK; ++kk) {
        T a[TM], b[TN];
#pragma unroll
        for (int i = 0; i < TM; ++i) a[i] = As[kk][ty * TM + i];
#pragma unroll
        for (int j = 0; j < TN; ++j) b[j] = Bs[kk][tx * TN + j];
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
          for (int j = 0; j < TN; ++j) fma_(acc[i][j], a[i], b[j]);
      }
      __syncthreads();
    }
    const bool beta_zero = (abs2_(beta) == 0);
#pragma unroll
    for (int i = 0; i < TM; ++i) {
      int64_t gm = m0 + ty * TM + i;
      if (gm >= M) continue;
#pragma unroll
      for (int j = 0; j < TN; ++j) {
        int64_t gn = n0 + tx * TN + j;
        if (gn >= N) continue;
        T v = alpha * acc[i][j];
        if (!beta_zero) v += beta * Cb[gm * ldc + gn];
        Cb[gm * ldc + gn] = v;
      }
    }
  }
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
  constexpr int BM = 64, BN = 64, BK = (sizeof(T) >= 16 ? 8 : 16);
  int64_t gy = (m + BM - 1) / BM, gx = (n + BN - 1) / BN;
  if (gy > 65535) return TNC_ERR_ARG;
  if (gx > 0x7fffffff) return TNC_ERR_ARG;
  unsigned gz = (unsigned)(batch < 65535 ? batch : 65535);
  dim3 grid((unsigned)gx, (unsigned)gy, gz);
  gemm_simt_kernel<T, BM, BN, BK><<<grid, 256, 0, st>>>(opA, opB, m, n, k, alpha, A, lda, sA, B, ldb, sB, beta, C,
                                                       ldc, sC, batch);
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
