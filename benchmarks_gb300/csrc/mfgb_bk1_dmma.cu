// CEED BK1 (mass) E-vector operator on the FP64 tensor cores.  The reference's
// BwdTransHexKernel_mma (sum_factorization/include/kernels/BK1/
// templated_cuda_mma_kernels.cuh:123-240) runs the direction-1 and -2
// contractions of both passes as mma.sync m8n8k4 f64 tiles (the instruction at
// cuda_mma_kernels.cuh:94-100) and direction 0 on the FMA pipe; here all six
// contractions are tiles.
//
//   out_e = B^T (JxW_e o (B x B x B) in_e),  B[q*NM + i] (NQ x NM), JxW[e][NQ^3],
//   in/out[e][NM^3], indices with direction 0 slowest (the serial kernel's order,
//   CEED_BK/include/kernels/BK1/serial_kernels.hpp:20-121).
//
// One warp per element.  Each of the six 1D contractions is a small GEMM
//   Y[m][n] = sum_k A[m][k] X[k][n]   (A = B or B^T, X the element's tensor with
// the contracted index as k and the other two flattened into n),
// cut into 8 x 8 x 4 tiles: M and K padded to 8, N to a multiple of 8.  The
// fragments follow the PTX layout of mma.m8n8k4 .f64: A[row = lane/4][col =
// lane%4], B[row = lane%4][col = lane/4], C/D[row = lane/4][cols 2(lane%4),
// 2(lane%4)+1].  Padded entries are loaded as zeros.  FP64 throughout: the
// result is the FP64 result (1e-12 bar), and the time is what the FP64 tensor
// pipe (1.10 TFLOP/s measured, the DFMA rate) allows.
#include <algorithm>

#include "mfgb_internal.h"
#include "mfgb_launch.cuh"

namespace mfgb {
namespace {

constexpr int kWarps = 4;  // elements (warps) per CTA

__device__ __forceinline__ void dmma(double &c0, double &c1, double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
               : "+d"(c0), "+d"(c1)
               : "d"(a), "d"(b));
}

// Y = A X for one warp: A (M x K) from am(m, k), X (K x N) from xm(k, n),
// result handed to ym(m, n, value); M, K <= 8.
template <int M, int K, int N, class AF, class XF, class YF>
__device__ __forceinline__ void warp_gemm(AF am, XF xm, YF ym) {
  const int lane = threadIdx.x & 31;
  const int ar = lane >> 2, ac = lane & 3;   // A fragment (row, col)
  const int br = lane & 3, bc = lane >> 2;   // B fragment (row, col)
  const int cr = lane >> 2, cc = 2 * (lane & 3);
  constexpr int KT = (K + 3) / 4, NT = (N + 7) / 8;
  double a[KT];
#pragma unroll
  for (int t = 0; t < KT; ++t) {
    const int k = t * 4 + ac;
    a[t] = (ar < M && k < K) ? am(ar, k) : 0.0;
  }
#pragma unroll
  for (int nt = 0; nt < NT; ++nt) {
    double c0 = 0.0, c1 = 0.0;
#pragma unroll
    for (int t = 0; t < KT; ++t) {
      const int k = t * 4 + br, n = nt * 8 + bc;
      const double b = (k < K && n < N) ? xm(k, n) : 0.0;
      dmma(c0, c1, a[t], b);
    }
    const int n0 = nt * 8 + cc;
    if (cr < M) {
      if (n0 < N) ym(cr, n0, c0);
      if (n0 + 1 < N) ym(cr, n0 + 1, c1);
    }
  }
}

template <int NM, int NQ>
__global__ void __launch_bounds__(32 * kWarps)
    bk1_dmma_kernel(const int64_t nelmt, const double *__restrict__ basis,
                    const double *__restrict__ JxW, const double *__restrict__ in,
                    double *__restrict__ out) {
  static_assert(NM <= 8 && NQ <= 8, "one 8-row tile per contraction");
  constexpr int M3 = NM * NM * NM, Q3 = NQ * NQ * NQ;
  __shared__ double sB[NQ * NM];
  __shared__ double s0[kWarps][Q3], s1[kWarps][Q3];
  for (int t = threadIdx.x; t < NQ * NM; t += blockDim.x) sB[t] = basis[t];
  __syncthreads();
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double *x = s0[w], *y = s1[w];
  auto Bf = [&](int q, int i) { return sB[q * NM + i]; };   // B[q][i]
  auto Bt = [&](int i, int q) { return sB[q * NM + i]; };   // B^T[i][q]
  for (int64_t e = (int64_t)blockIdx.x * kWarps + w; e < nelmt; e += (int64_t)gridDim.x * kWarps) {
    for (int t = lane; t < M3; t += 32) x[t] = in[e * M3 + t];
    __syncwarp();
    // t1[q0][j][k] = sum_i B[q0][i] in[i][j][k]          (n = j NM + k)
    warp_gemm<NQ, NM, NM * NM>(Bf, [&](int k, int n) { return x[k * NM * NM + n]; },
                               [&](int m, int n, double v) { y[m * NM * NM + n] = v; });
    __syncwarp();
    // t2[q0][q1][k] = sum_j B[q1][j] t1[q0][j][k]        (n = q0 NM + k)
    warp_gemm<NQ, NM, NQ * NM>(
        Bf, [&](int k, int n) { return y[(n / NM) * NM * NM + k * NM + n % NM]; },
        [&](int m, int n, double v) { x[(n / NM) * NQ * NM + m * NM + n % NM] = v; });
    __syncwarp();
    // t3[q0][q1][q2] = JxW sum_k B[q2][k] t2[q0][q1][k]  (n = q0 NQ + q1)
    warp_gemm<NQ, NM, NQ * NQ>(
        Bf, [&](int k, int n) { return x[n * NM + k]; },
        [&](int m, int n, double v) { y[n * NQ + m] = v * JxW[e * Q3 + n * NQ + m]; });
    __syncwarp();
    // s1[i][q1][q2] = sum_q0 B[q0][i] w[q0][q1][q2]      (n = q1 NQ + q2)
    warp_gemm<NM, NQ, NQ * NQ>(Bt, [&](int k, int n) { return y[k * NQ * NQ + n]; },
                               [&](int m, int n, double v) { x[m * NQ * NQ + n] = v; });
    __syncwarp();
    // s2[i][j][q2] = sum_q1 B[q1][j] s1[i][q1][q2]       (n = i NQ + q2)
    warp_gemm<NM, NQ, NM * NQ>(
        Bt, [&](int k, int n) { return x[(n / NQ) * NQ * NQ + k * NQ + n % NQ]; },
        [&](int m, int n, double v) { y[(n / NQ) * NM * NQ + m * NQ + n % NQ] = v; });
    __syncwarp();
    // out[i][j][k] = sum_q2 B[q2][k] s2[i][j][q2]        (n = i NM + j)
    warp_gemm<NM, NQ, NM * NM>(Bt, [&](int k, int n) { return y[n * NQ + k]; },
                               [&](int m, int n, double v) { out[e * M3 + n * NM + m] = v; });
    __syncwarp();
  }
}

template <int NM, int NQ>
cudaError_t bk1_dmma_launch(int64_t nelmt, const double *basis, const double *JxW,
                            const double *in, double *out, cudaStream_t s) {
  static int per_sm = -1;
  if (per_sm < 0) per_sm = std::max(1, ctas_per_sm(bk1_dmma_kernel<NM, NQ>, 32 * kWarps, 0));
  const int64_t blocks = (nelmt + kWarps - 1) / kWarps;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(blocks, (int64_t)per_sm * num_sms()));
  bk1_dmma_kernel<NM, NQ><<<grid, 32 * kWarps, 0, s>>>(nelmt, basis, JxW, in, out);
  return cudaGetLastError();
}

}  // namespace

// degree 1..6 (NQ = p + 2 <= 8: one tile row per contraction)
cudaError_t bk1_dmma(int degree, int64_t nelmt, const double *basis, const double *JxW,
                     const double *in, double *out, cudaStream_t s) {
  if (nelmt <= 0) return cudaSuccess;
  switch (degree) {
    case 1: return bk1_dmma_launch<2, 3>(nelmt, basis, JxW, in, out, s);
    case 2: return bk1_dmma_launch<3, 4>(nelmt, basis, JxW, in, out, s);
    case 3: return bk1_dmma_launch<4, 5>(nelmt, basis, JxW, in, out, s);
    case 4: return bk1_dmma_launch<5, 6>(nelmt, basis, JxW, in, out, s);
    case 5: return bk1_dmma_launch<6, 7>(nelmt, basis, JxW, in, out, s);
    case 6: return bk1_dmma_launch<7, 8>(nelmt, basis, JxW, in, out, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace mfgb
