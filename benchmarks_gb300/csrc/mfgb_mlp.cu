// mfgb_mlp.cu -- learned smoother weights: per-cell features, per-cell spectral
// targets, a 73-64-64-1 MLP trained on the GPU (FP32, hand-written forward /
// backward / Adam kernels) and evaluated with BF16 tensor-core MMAs.
//
// No counterpart in the reference.  The network predicts, from a cell's
// Jacobians at its 8 corners and its degree, lambda_e = lambda_max(D_e^-1 A_e)
// (the cell matrix scaled by its own diagonal).  The multigrid smoother then
// uses the assembled diagonal D~ = sum_e lambda_e D_e: a positive diagonal, so
// the V-cycle stays linear and symmetric positive definite, and exact lambda_e
// give lambda_max(D~^-1 A) <= 1 (sum over cells of x_e^T A_e x_e).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include <cuda_bf16.h>

#include "mfgb_common.cuh"
#include "mfgb_internal.h"
#include "mfgb_mg_internal.h"

namespace mfgb {
namespace {

constexpr int NIN = 73, NH = 64;
constexpr int NP = NH * NIN + NH + NH * NH + NH + NH + 1;  // 8961
constexpr int OFF_W1 = 0, OFF_B1 = NH * NIN, OFF_W2 = OFF_B1 + NH, OFF_B2 = OFF_W2 + NH * NH,
              OFF_W3 = OFF_B2 + NH, OFF_B3 = OFF_W3 + NH;

#define GS(t, n)                                                               \
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (n); \
       t += (int64_t)gridDim.x * blockDim.x)

unsigned g1(int64_t n) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 32)); }

// ---- features ---------------------------------------------------------------
struct FeatParams {
  double xg[9];            // geometry GLL points
  double Vc[2 * 9];        // geometry basis at the two corner coordinates -1, +1
  double Dc[2 * 9];        // its derivative there
  int ng, degree;
};

__global__ void cell_features_kernel(mfgb_box_desc b, FeatParams fp, float *__restrict__ F) {
  __shared__ double xyz[729 * 3];
  __shared__ double J[8][9];
  __shared__ double det[8];
  const int ng = fp.ng, ng3 = ng * ng * ng;
  const int64_t e = blockIdx.x;
  const int64_t cx = e % b.nx, cy = (e / b.nx) % b.ny, cz = e / ((int64_t)b.nx * b.ny);
  const double hx = (b.hi[0] - b.lo[0]) / b.nx, hy = (b.hi[1] - b.lo[1]) / b.ny,
               hz = (b.hi[2] - b.lo[2]) / b.nz;
  for (int l = threadIdx.x; l < ng3; l += blockDim.x) {
    const int i = l / (ng * ng), j = (l / ng) % ng, k = l % ng;
    const double X = b.lo[0] + ((double)cx + 0.5 * (fp.xg[k] + 1.0)) * hx;
    const double Y = b.lo[1] + ((double)cy + 0.5 * (fp.xg[j] + 1.0)) * hy;
    const double Z = b.lo[2] + ((double)cz + 0.5 * (fp.xg[i] + 1.0)) * hz;
    const double s = b.amplitude * sin(2.0 * M_PI * X) * sin(2.0 * M_PI * Y) * sin(2.0 * M_PI * Z);
    xyz[3 * l] = X + s;
    xyz[3 * l + 1] = Y + s;
    xyz[3 * l + 2] = Z + s;
  }
  __syncthreads();
  // thread (corner, d, a): 8 x 3 x 3 entries
  for (int t = threadIdx.x; t < 72; t += blockDim.x) {
    const int c = t / 9, d = (t / 3) % 3, a = t % 3;
    const int ci = (c >> 2) & 1, cj = (c >> 1) & 1, ck = c & 1;
    double s = 0;
    for (int p = 0; p < ng; ++p)
      for (int q = 0; q < ng; ++q)
        for (int r = 0; r < ng; ++r) {
          const double wi = a == 0 ? fp.Dc[ci * 9 + p] : fp.Vc[ci * 9 + p];
          const double wj = a == 1 ? fp.Dc[cj * 9 + q] : fp.Vc[cj * 9 + q];
          const double wk = a == 2 ? fp.Dc[ck * 9 + r] : fp.Vc[ck * 9 + r];
          s += wi * wj * wk * xyz[3 * ((p * ng + q) * ng + r) + d];
        }
    J[c][d * 3 + a] = s;
  }
  __syncthreads();
  if (threadIdx.x < 8) {
    const double *M = J[threadIdx.x];
    det[threadIdx.x] = M[0] * (M[4] * M[8] - M[5] * M[7]) - M[1] * (M[3] * M[8] - M[5] * M[6]) +
                       M[2] * (M[3] * M[7] - M[4] * M[6]);
  }
  __syncthreads();
  double md = 0;
  for (int c = 0; c < 8; ++c) md += det[c];
  const double sc = 1.0 / cbrt(fabs(md / 8.0));
  for (int t = threadIdx.x; t < 72; t += blockDim.x) F[e * NIN + t] = (float)(J[t / 9][t % 9] * sc);
  if (threadIdx.x == 0) F[e * NIN + 72] = (float)(fp.degree / 8.0);
}

// ---- per-cell lambda_max(D_e^-1 A_e) by power iteration (FP64) -------------
// One CTA per cell, one thread per GLL point; the cell operator applied in
// shared memory; Rayleigh quotient v.Av / v.Dv after `iters` steps.
struct LamParams {
  double D[81];
  int n;
};

__device__ double block_sum_d(double v, double *sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0;
  for (int w = 0; w < (int)((blockDim.x + 31) / 32); ++w) s += sh[w];
  __syncthreads();
  return s;
}

__global__ void cell_lambda_kernel(int64_t n_cells, const double *__restrict__ G, LamParams lp,
                                   int iters, double *__restrict__ lam) {
  __shared__ double v[729], vr[729], vs[729], vt[729], sh[32];
  const int n = lp.n, n3 = n * n * n;
  const int q = threadIdx.x;
  const bool act = q < n3;
  const int i = q / (n * n), j = (q / n) % n, k = q % n;
  for (int64_t e = blockIdx.x; e < n_cells; e += gridDim.x) {
    const double *Ge = G + e * 6 * n3;
    double d = 1.0;
    if (act) {  // cell diagonal (closed form of the GLL-collocation operator)
      d = 0;
      for (int a = 0; a < n; ++a) {
        const double di = lp.D[a * n + i], dj = lp.D[a * n + j], dk = lp.D[a * n + k];
        d += Ge[0 * n3 + a * n * n + j * n + k] * di * di;
        d += Ge[3 * n3 + i * n * n + a * n + k] * dj * dj;
        d += Ge[5 * n3 + i * n * n + j * n + a] * dk * dk;
      }
      const double Dii = lp.D[i * n + i], Djj = lp.D[j * n + j], Dkk = lp.D[k * n + k];
      d += 2.0 * (Ge[1 * n3 + q] * Dii * Djj + Ge[2 * n3 + q] * Dii * Dkk + Ge[4 * n3 + q] * Djj * Dkk);
      // deterministic, non-smooth start
      v[q] = 1.0 + 0.5 * sin(1.0 + 2.3 * q);
    }
    __syncthreads();
    double rq = 0;
    for (int it = 0; it <= iters; ++it) {
      double ur = 0, us = 0, ut = 0;
      if (act)
        for (int m = 0; m < n; ++m) {
          ur += lp.D[i * n + m] * v[m * n * n + j * n + k];
          us += lp.D[j * n + m] * v[i * n * n + m * n + k];
          ut += lp.D[k * n + m] * v[i * n * n + j * n + m];
        }
      __syncthreads();
      if (act) {
        vr[q] = Ge[0 * n3 + q] * ur + Ge[1 * n3 + q] * us + Ge[2 * n3 + q] * ut;
        vs[q] = Ge[1 * n3 + q] * ur + Ge[3 * n3 + q] * us + Ge[4 * n3 + q] * ut;
        vt[q] = Ge[2 * n3 + q] * ur + Ge[4 * n3 + q] * us + Ge[5 * n3 + q] * ut;
      }
      __syncthreads();
      double w = 0;
      if (act)
        for (int m = 0; m < n; ++m)
          w += lp.D[m * n + i] * vr[m * n * n + j * n + k] + lp.D[m * n + j] * vs[i * n * n + m * n + k] +
               lp.D[m * n + k] * vt[i * n * n + j * n + m];
      const double vq = act ? v[q] : 0.0;
      const double vAv = block_sum_d(act ? vq * w : 0.0, sh);
      const double vDv = block_sum_d(act ? vq * d * vq : 0.0, sh);
      rq = vAv / vDv;
      const double z = act ? w / d : 0.0;  // next iterate D^-1 A v, D-normalised
      const double zDz = block_sum_d(act ? z * d * z : 0.0, sh);
      if (act) v[q] = z / sqrt(zDz);
      __syncthreads();
    }
    if (threadIdx.x == 0) lam[e] = rq;
    __syncthreads();
  }
}

// ---- MLP training (FP32, deterministic: no atomics) -------------------------
// activations of a batch: Z1, Z2 [B][64]; z3, dz3 [B]; dH2, dH1 [B][64]
__global__ void mlp_fwd1(int B, const float *__restrict__ P, const float *__restrict__ X,
                         const int *__restrict__ idx, float *__restrict__ Z1) {
  GS(t, (int64_t)B * NH) {
    const int b = (int)(t / NH), o = (int)(t % NH);
    const float *x = X + (int64_t)idx[b] * NIN;
    float s = P[OFF_B1 + o];
    for (int i = 0; i < NIN; ++i) s = fmaf(P[OFF_W1 + o * NIN + i], x[i], s);
    Z1[t] = s;
  }
}

__global__ void mlp_fwd2(int B, const float *__restrict__ P, const float *__restrict__ Z1,
                         float *__restrict__ Z2) {
  GS(t, (int64_t)B * NH) {
    const int b = (int)(t / NH), o = (int)(t % NH);
    float s = P[OFF_B2 + o];
    for (int i = 0; i < NH; ++i) s = fmaf(P[OFF_W2 + o * NH + i], fmaxf(Z1[b * NH + i], 0.f), s);
    Z2[t] = s;
  }
}

__device__ __forceinline__ float softplusf(float z) { return z > 20.f ? z : log1pf(expf(z)); }
__device__ __forceinline__ float sigmoidf(float z) { return 1.f / (1.f + expf(-z)); }

// z3, y, dz3 = dL/dz3 for L = mean (y - t)^2; loss partial per sample
__global__ void mlp_fwd3(int B, const float *__restrict__ P, const float *__restrict__ Z2,
                         const float *__restrict__ T, const int *__restrict__ idx,
                         float *__restrict__ dz3, float *__restrict__ lossv, float *__restrict__ y) {
  GS(t, (int64_t)B) {
    const int b = (int)t;
    float s = P[OFF_B3];
    for (int i = 0; i < NH; ++i) s = fmaf(P[OFF_W3 + i], fmaxf(Z2[b * NH + i], 0.f), s);
    const float yy = softplusf(s);
    if (y) y[b] = yy;
    if (T) {
      const float r = yy - T[idx[b]];
      lossv[b] = r * r;
      dz3[b] = 2.f * r / B * sigmoidf(s);
    }
  }
}

__global__ void mlp_bwd2(int B, const float *__restrict__ P, const float *__restrict__ Z2,
                         const float *__restrict__ dz3, float *__restrict__ dH2) {
  GS(t, (int64_t)B * NH) {
    const int b = (int)(t / NH), o = (int)(t % NH);
    dH2[t] = Z2[t] > 0.f ? dz3[b] * P[OFF_W3 + o] : 0.f;
  }
}

__global__ void mlp_bwd1(int B, const float *__restrict__ P, const float *__restrict__ Z1,
                         const float *__restrict__ dH2, float *__restrict__ dH1) {
  GS(t, (int64_t)B * NH) {
    const int b = (int)(t / NH), i = (int)(t % NH);
    float s = 0.f;
    for (int o = 0; o < NH; ++o) s = fmaf(dH2[b * NH + o], P[OFF_W2 + o * NH + i], s);
    dH1[t] = Z1[t] > 0.f ? s : 0.f;
  }
}

// one thread per parameter, loop over the batch in order
__global__ void mlp_grads(int B, const float *__restrict__ X, const int *__restrict__ idx,
                          const float *__restrict__ Z1, const float *__restrict__ Z2,
                          const float *__restrict__ dz3, const float *__restrict__ dH1,
                          const float *__restrict__ dH2, float *__restrict__ grad) {
  GS(t, (int64_t)NP) {
    float s = 0.f;
    const int p = (int)t;
    if (p < OFF_B1) {
      const int o = p / NIN, i = p % NIN;
      for (int b = 0; b < B; ++b) s = fmaf(dH1[b * NH + o], X[(int64_t)idx[b] * NIN + i], s);
    } else if (p < OFF_W2) {
      const int o = p - OFF_B1;
      for (int b = 0; b < B; ++b) s += dH1[b * NH + o];
    } else if (p < OFF_B2) {
      const int o = (p - OFF_W2) / NH, i = (p - OFF_W2) % NH;
      for (int b = 0; b < B; ++b) s = fmaf(dH2[b * NH + o], fmaxf(Z1[b * NH + i], 0.f), s);
    } else if (p < OFF_W3) {
      const int o = p - OFF_B2;
      for (int b = 0; b < B; ++b) s += dH2[b * NH + o];
    } else if (p < OFF_B3) {
      const int i = p - OFF_W3;
      for (int b = 0; b < B; ++b) s = fmaf(dz3[b], fmaxf(Z2[b * NH + i], 0.f), s);
    } else {
      for (int b = 0; b < B; ++b) s += dz3[b];
    }
    grad[p] = s;
  }
}

__global__ void adam_step(float *__restrict__ P, const float *__restrict__ g, float *__restrict__ m,
                          float *__restrict__ v, float lr, float b1t, float b2t) {
  GS(t, (int64_t)NP) {
    const float gi = g[t];
    const float mi = 0.9f * m[t] + 0.1f * gi;
    const float vi = 0.999f * v[t] + 0.001f * gi * gi;
    m[t] = mi;
    v[t] = vi;
    P[t] -= lr * (mi / (1.f - b1t)) / (sqrtf(vi / (1.f - b2t)) + 1e-8f);
  }
}

// minibatch indices: a fixed pseudo-random sequence (xorshift per step)
__global__ void batch_indices(int B, int64_t n, uint64_t seed, int *__restrict__ idx) {
  GS(t, (int64_t)B) {
    uint64_t s = seed ^ (0x9E3779B97F4A7C15ull * (uint64_t)(t + 1));
    s ^= s >> 33; s *= 0xff51afd7ed558ccdull; s ^= s >> 33; s *= 0xc4ceb9fe1a85ec53ull; s ^= s >> 33;
    idx[t] = (int)(s % (uint64_t)n);
  }
}

__global__ void iota_kernel(int B, int64_t base, int *__restrict__ idx) {
  GS(t, (int64_t)B) idx[t] = (int)(base + t);
}

// ---- inference with BF16 tensor cores (mma.sync m16n8k16, FP32 accumulate) --
// One warp per 16 cells.  Layer 1: X[16 x 80] (K padded 73 -> 80) x W1^T,
// layer 2: H1[16 x 64] x W2^T; the layer-1 accumulators become the layer-2 A
// fragments in registers (same rows, matching column pairs).  Layer 3 and the
// softplus in FP32.
__device__ __forceinline__ void mma_bf16(float *c, const uint32_t *a, const uint32_t *b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 p = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t *>(&p);
}

constexpr int KP = 80;  // padded input width

__global__ void __launch_bounds__(128)
    mlp_infer_bf16(int64_t n, const float *__restrict__ P, const float *__restrict__ X,
                   double *__restrict__ y) {
  __shared__ __nv_bfloat16 sW1[NH * KP];
  __shared__ __nv_bfloat16 sW2[NH * NH];
  __shared__ float sB1[NH], sB2[NH], sW3[NH];
  __shared__ __nv_bfloat16 sX[4][16 * KP];
  for (int t = threadIdx.x; t < NH * KP; t += blockDim.x) {
    const int o = t / KP, i = t % KP;
    sW1[t] = __float2bfloat16(i < NIN ? P[OFF_W1 + o * NIN + i] : 0.f);
  }
  for (int t = threadIdx.x; t < NH * NH; t += blockDim.x) sW2[t] = __float2bfloat16(P[OFF_W2 + t]);
  for (int t = threadIdx.x; t < NH; t += blockDim.x) {
    sB1[t] = P[OFF_B1 + t];
    sB2[t] = P[OFF_B2 + t];
    sW3[t] = P[OFF_W3 + t];
  }
  const float b3 = P[OFF_B3];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, tg = lane & 3;
  __nv_bfloat16 *xs = sX[warp];
  const int64_t n_tiles = (n + 15) / 16;
  for (int64_t tile = blockIdx.x * 4 + warp; tile < n_tiles; tile += (int64_t)gridDim.x * 4) {
    const int64_t r0 = tile * 16;
    for (int t = lane; t < 16 * KP; t += 32) {
      const int r = t / KP, i = t % KP;
      const int64_t row = r0 + r;
      xs[t] = __float2bfloat16(row < n && i < NIN ? X[row * NIN + i] : 0.f);
    }
    __syncwarp();
    float acc[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
#pragma unroll
    for (int kt = 0; kt < KP / 16; ++kt) {
      uint32_t a[4];
      const int c0 = kt * 16 + 2 * tg;
      a[0] = *reinterpret_cast<const uint32_t *>(&xs[g * KP + c0]);
      a[1] = *reinterpret_cast<const uint32_t *>(&xs[(g + 8) * KP + c0]);
      a[2] = *reinterpret_cast<const uint32_t *>(&xs[g * KP + c0 + 8]);
      a[3] = *reinterpret_cast<const uint32_t *>(&xs[(g + 8) * KP + c0 + 8]);
#pragma unroll
      for (int nt = 0; nt < 8; ++nt) {
        uint32_t bb[2];
        const int o = nt * 8 + g;
        bb[0] = *reinterpret_cast<const uint32_t *>(&sW1[o * KP + c0]);
        bb[1] = *reinterpret_cast<const uint32_t *>(&sW1[o * KP + c0 + 8]);
        mma_bf16(acc[nt], a, bb);
      }
    }
    // bias + relu; accumulators of n-tiles (2kt, 2kt+1) form the A fragment of k-tile kt
    uint32_t h[4][4];
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) {
      const int ca = (2 * kt) * 8 + 2 * tg, cb = (2 * kt + 1) * 8 + 2 * tg;
      h[kt][0] = pack_bf16(fmaxf(acc[2 * kt][0] + sB1[ca], 0.f), fmaxf(acc[2 * kt][1] + sB1[ca + 1], 0.f));
      h[kt][1] = pack_bf16(fmaxf(acc[2 * kt][2] + sB1[ca], 0.f), fmaxf(acc[2 * kt][3] + sB1[ca + 1], 0.f));
      h[kt][2] = pack_bf16(fmaxf(acc[2 * kt + 1][0] + sB1[cb], 0.f),
                           fmaxf(acc[2 * kt + 1][1] + sB1[cb + 1], 0.f));
      h[kt][3] = pack_bf16(fmaxf(acc[2 * kt + 1][2] + sB1[cb], 0.f),
                           fmaxf(acc[2 * kt + 1][3] + sB1[cb + 1], 0.f));
    }
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) {
      const int c0 = kt * 16 + 2 * tg;
#pragma unroll
      for (int nt = 0; nt < 8; ++nt) {
        uint32_t bb[2];
        const int o = nt * 8 + g;
        bb[0] = *reinterpret_cast<const uint32_t *>(&sW2[o * NH + c0]);
        bb[1] = *reinterpret_cast<const uint32_t *>(&sW2[o * NH + c0 + 8]);
        mma_bf16(acc[nt], h[kt], bb);
      }
    }
    // layer 3: rows g and g+8, this thread's columns; reduce over the 4 threads of a group
    float s0 = 0.f, s1 = 0.f;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      const int c = nt * 8 + 2 * tg;
      s0 += fmaxf(acc[nt][0] + sB2[c], 0.f) * sW3[c] + fmaxf(acc[nt][1] + sB2[c + 1], 0.f) * sW3[c + 1];
      s1 += fmaxf(acc[nt][2] + sB2[c], 0.f) * sW3[c] + fmaxf(acc[nt][3] + sB2[c + 1], 0.f) * sW3[c + 1];
    }
    s0 += __shfl_xor_sync(0xffffffffu, s0, 1);
    s0 += __shfl_xor_sync(0xffffffffu, s0, 2);
    s1 += __shfl_xor_sync(0xffffffffu, s1, 1);
    s1 += __shfl_xor_sync(0xffffffffu, s1, 2);
    if (tg == 0) {
      if (r0 + g < n) y[r0 + g] = softplusf(s0 + b3);
      if (r0 + g + 8 < n) y[r0 + g + 8] = softplusf(s1 + b3);
    }
    __syncwarp();
  }
}

// weighted assembled diagonal: d_i = sum_e w_e (A_e)_ii  (w = cell weights)
struct WDiagParams {
  double D[81];
};

__global__ void weighted_diagonal_kernel(int n, int64_t n_cells, const uint32_t *__restrict__ map,
                                         const double *__restrict__ G, const double *__restrict__ w,
                                         WDiagParams dp, double *__restrict__ diag) {
  const int n3 = n * n * n;
  GS(t, n_cells * n3) {
    const uint32_t dof = map[t];
    if (dof == MFGB_INVALID_DOF) continue;
    const int64_t e = t / n3;
    const int q = (int)(t - e * n3);
    const int i = q / (n * n), j = (q / n) % n, k = q % n;
    const double *Ge = G + e * 6 * n3;
    double d = 0.0;
    for (int a = 0; a < n; ++a) {
      const double di = dp.D[a * n + i], dj = dp.D[a * n + j], dk = dp.D[a * n + k];
      d += Ge[0 * n3 + a * n * n + j * n + k] * di * di;
      d += Ge[3 * n3 + i * n * n + a * n + k] * dj * dj;
      d += Ge[5 * n3 + i * n * n + j * n + a] * dk * dk;
    }
    const double Dii = dp.D[i * n + i], Djj = dp.D[j * n + j], Dkk = dp.D[k * n + k];
    d += 2.0 * (Ge[1 * n3 + q] * Dii * Djj + Ge[2 * n3 + q] * Dii * Dkk + Ge[4 * n3 + q] * Djj * Dkk);
    atomicAdd(diag + dof, w[e] * d);
  }
}

}  // namespace

cudaError_t weighted_diagonal(const mfgb_operator *op, const double *w, double *diag,
                              cudaStream_t s) {
  WDiagParams dp;
  for (int i = 0; i < 81; ++i) dp.D[i] = op->D[i];
  weighted_diagonal_kernel<<<g1(op->n_cells * op->n * op->n * op->n), 256, 0, s>>>(
      op->n, op->n_cells, op->d_map, op->d_G, w, dp, diag);
  return cudaGetLastError();
}

// Per-cell squared norms of two vectors over the cell's (unconstrained) DoFs:
// one 64-thread block per cell at a time, sums added into na / nb.
__global__ void __launch_bounds__(64)
    cell_sq_norms_kernel(int64_t n_cells, int n3, const uint32_t *__restrict__ map,
                         const double *__restrict__ a, const double *__restrict__ b,
                         double *__restrict__ na, double *__restrict__ nb) {
  __shared__ double s_a[64], s_b[64];
  for (int64_t c = blockIdx.x; c < n_cells; c += gridDim.x) {
    double sa = 0.0, sb = 0.0;
    for (int l = threadIdx.x; l < n3; l += 64) {
      const uint32_t d = map[c * n3 + l];
      if (d != MFGB_INVALID_DOF) {
        sa = __fma_rn(a[d], a[d], sa);
        sb = __fma_rn(b[d], b[d], sb);
      }
    }
    s_a[threadIdx.x] = sa;
    s_b[threadIdx.x] = sb;
    __syncthreads();
    for (int o = 32; o > 0; o >>= 1) {
      if (threadIdx.x < o) {
        s_a[threadIdx.x] += s_a[threadIdx.x + o];
        s_b[threadIdx.x] += s_b[threadIdx.x + o];
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      na[c] += s_a[0];
      nb[c] += s_b[0];
    }
    __syncthreads();
  }
}

__global__ void error_propagate_kernel(int64_t n, const double *__restrict__ e,
                                       const double *__restrict__ z, double *__restrict__ out) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x)
    out[t] = e[t] - z[t];
}

__global__ void ratio_sqrt_kernel(int64_t n, const double *__restrict__ before,
                                  const double *__restrict__ after, double *__restrict__ rho) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x)
    rho[t] = before[t] > 0.0 ? sqrt(after[t] / before[t]) : 0.0;
}

}  // namespace mfgb

using namespace mfgb;

extern "C" {

// Training data the FP64 multigrid generates for the learned smoother: the
// per-cell error reduction of one V-cycle, rho_c = |E e|_c / |e|_c with
// E = I - M A the V-cycle's error propagation, over n_vectors seeded random
// errors e (U[-1,1] from mt19937_64(seed + k), zero on Dirichlet DoFs); the
// norms sum the cell's unconstrained DoFs over all vectors.
mfgb_status mfgb_cell_error_reduction(const mfgb_operator *op, mfgb_mg *mg, int n_vectors,
                                      uint64_t seed, double *d_rho, void *stream) {
  if (!op || !mg || op->quadrature || n_vectors < 1 || (op->n_cells > 0 && !d_rho)) {
    set_error("mfgb_cell_error_reduction: invalid argument");
    return MFGB_ERR_INVALID_ARG;
  }
  if (mg->levels.empty() || mg->levels[0].n != op->n_dofs) {
    set_error("mfgb_cell_error_reduction: the hierarchy is not the operator's");
    return MFGB_ERR_INVALID_ARG;
  }
  const int64_t n = op->n_dofs, nc = op->n_cells;
  const int n3 = op->n * op->n * op->n;
  cudaStream_t s = (cudaStream_t)stream;
  double *e = nullptr, *w = nullptr, *z = nullptr, *na = nullptr, *nb = nullptr;
  auto freeall = [&]() {
    cudaFree(e); cudaFree(w); cudaFree(z); cudaFree(na); cudaFree(nb);
  };
  mfgb_status st;
  if ((st = dalloc((void **)&e, sizeof(double) * n)) || (st = dalloc((void **)&w, sizeof(double) * n)) ||
      (st = dalloc((void **)&z, sizeof(double) * n)) ||
      (st = dalloc((void **)&na, sizeof(double) * std::max<int64_t>(nc, 1))) ||
      (st = dalloc((void **)&nb, sizeof(double) * std::max<int64_t>(nc, 1)))) {
    freeall();
    return st;
  }
  cudaMemsetAsync(na, 0, sizeof(double) * std::max<int64_t>(nc, 1), s);
  cudaMemsetAsync(nb, 0, sizeof(double) * std::max<int64_t>(nc, 1), s);
  const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 16));
  const unsigned gc = (unsigned)std::min<int64_t>(std::max<int64_t>(nc, 1), 152 * 32);
  for (int k = 0; k < n_vectors && !st; ++k) {
    if ((st = mfgb_rhs_uniform(op, seed + (uint64_t)k, e, s)) ||
        (st = mfgb_vmult(op, w, e, MFGB_ARITH_FP64_DF, s)) || (st = mfgb_mg_vmult(mg, z, w, s)))
      break;
    error_propagate_kernel<<<g, 256, 0, s>>>(n, e, z, w);
    if (nc > 0) cell_sq_norms_kernel<<<gc, 64, 0, s>>>(nc, n3, op->d_map, e, w, na, nb);
    st = cuda_status(cudaGetLastError(), "mfgb_cell_error_reduction");
  }
  if (!st && nc > 0) {
    ratio_sqrt_kernel<<<gc, 256, 0, s>>>(nc, na, nb, d_rho);
    st = cuda_status(cudaGetLastError(), "mfgb_cell_error_reduction");
  }
  if (!st) st = cuda_status(cudaStreamSynchronize(s), "mfgb_cell_error_reduction");
  freeall();
  return st;
}

int mfgb_mlp_n_params(void) { return NP; }

mfgb_status mfgb_cell_features(const mfgb_operator *op, float *d_features, void *stream) {
  if (!op || !op->is_box || (op->n_cells > 0 && !d_features)) {
    set_error("mfgb_cell_features: needs a box operator and an output array");
    return MFGB_ERR_INVALID_ARG;
  }
  FeatParams fp{};
  const mfgb_box_desc &b = op->box;
  const int g = b.geometry_degree > 0 ? b.geometry_degree : b.degree;
  fp.ng = g + 1;
  fp.degree = b.degree;
  double wg[9];
  gll_nodes(fp.ng, fp.xg, wg);
  for (int c = 0; c < 2; ++c) {
    const double x = c ? 1.0 : -1.0;
    for (int a = 0; a < fp.ng; ++a) {
      fp.Vc[c * 9 + a] = lagrange_value(fp.ng, fp.xg, a, x);
      fp.Dc[c * 9 + a] = lagrange_derivative(fp.ng, fp.xg, a, x);
    }
  }
  if (op->n_cells == 0) return MFGB_OK;
  cell_features_kernel<<<(unsigned)op->n_cells, 128, 0, (cudaStream_t)stream>>>(b, fp, d_features);
  return cuda_status(cudaGetLastError(), "mfgb_cell_features");
}

mfgb_status mfgb_cell_lambda(const mfgb_operator *op, double *d_lambda, int iterations,
                             void *stream) {
  if (!op || op->quadrature || iterations < 1 || (op->n_cells > 0 && !d_lambda)) {
    set_error("mfgb_cell_lambda: invalid argument");
    return MFGB_ERR_INVALID_ARG;
  }
  LamParams lp{};
  lp.n = op->n;
  for (int i = 0; i < 81; ++i) lp.D[i] = op->D[i];
  const int threads = ((op->n * op->n * op->n + 31) / 32) * 32;
  if (op->n_cells == 0) return MFGB_OK;
  cell_lambda_kernel<<<(unsigned)std::min<int64_t>(op->n_cells, 152 * 16), threads, 0,
                       (cudaStream_t)stream>>>(op->n_cells, op->d_G, lp, iterations, d_lambda);
  return cuda_status(cudaGetLastError(), "mfgb_cell_lambda");
}

// Loss and gradient (FP32) of the batch of all n samples, for checks.
mfgb_status mfgb_mlp_loss_grad(const float *d_params, const float *d_X, const float *d_t, int n,
                               float *h_grad, float *h_loss) {
  if (!d_params || !d_X || !d_t || n < 1 || !h_grad || !h_loss) {
    set_error("mfgb_mlp_loss_grad: invalid argument");
    return MFGB_ERR_INVALID_ARG;
  }
  float *buf = nullptr;
  int *idx = nullptr;
  const size_t fl = (size_t)n * (4 * NH + 3) + NP;
  if (cudaMalloc(&buf, sizeof(float) * fl) != cudaSuccess || cudaMalloc(&idx, sizeof(int) * n) != cudaSuccess) {
    cudaFree(buf);
    return cuda_status(cudaErrorMemoryAllocation, "mlp buffers");
  }
  float *Z1 = buf, *Z2 = Z1 + (size_t)n * NH, *dH1 = Z2 + (size_t)n * NH, *dH2 = dH1 + (size_t)n * NH,
        *dz3 = dH2 + (size_t)n * NH, *lossv = dz3 + n, *grad = lossv + n;
  iota_kernel<<<g1(n), 256>>>(n, 0, idx);
  mlp_fwd1<<<g1((int64_t)n * NH), 256>>>(n, d_params, d_X, idx, Z1);
  mlp_fwd2<<<g1((int64_t)n * NH), 256>>>(n, d_params, Z1, Z2);
  mlp_fwd3<<<g1(n), 256>>>(n, d_params, Z2, d_t, idx, dz3, lossv, nullptr);
  mlp_bwd2<<<g1((int64_t)n * NH), 256>>>(n, d_params, Z2, dz3, dH2);
  mlp_bwd1<<<g1((int64_t)n * NH), 256>>>(n, d_params, Z1, dH2, dH1);
  mlp_grads<<<g1(NP), 256>>>(n, d_X, idx, Z1, Z2, dz3, dH1, dH2, grad);
  std::vector<float> lv(n);
  mfgb_status st = cuda_status(cudaMemcpy(h_grad, grad, sizeof(float) * NP, cudaMemcpyDeviceToHost), "grad");
  if (!st) st = cuda_status(cudaMemcpy(lv.data(), lossv, sizeof(float) * n, cudaMemcpyDeviceToHost), "loss");
  double L = 0;
  for (float v : lv) L += v;
  *h_loss = (float)(L / n);
  cudaFree(buf);
  cudaFree(idx);
  return st;
}

// Adam on minibatches of `batch` samples drawn from the n samples (X: n x 73
// FP32, t: n targets); d_params in/out; h_loss[steps] receives each step's
// minibatch loss (may be NULL).  One step is captured in a CUDA graph.
mfgb_status mfgb_mlp_train(float *d_params, const float *d_X, const float *d_t, int64_t n,
                           int steps, int batch, float lr, uint64_t seed, float *h_loss) {
  if (!d_params || !d_X || !d_t || n < 1 || steps < 0 || batch < 1 || !(lr > 0)) {
    set_error("mfgb_mlp_train: invalid argument");
    return MFGB_ERR_INVALID_ARG;
  }
  const int B = batch;
  float *buf = nullptr;
  int *idx = nullptr;
  const size_t fl = (size_t)B * (4 * NH + 3) + 3 * NP + 8;
  if (cudaMalloc(&buf, sizeof(float) * fl) != cudaSuccess || cudaMalloc(&idx, sizeof(int) * B) != cudaSuccess) {
    cudaFree(buf);
    return cuda_status(cudaErrorMemoryAllocation, "mlp buffers");
  }
  float *Z1 = buf, *Z2 = Z1 + (size_t)B * NH, *dH1 = Z2 + (size_t)B * NH, *dH2 = dH1 + (size_t)B * NH,
        *dz3 = dH2 + (size_t)B * NH, *lossv = dz3 + B, *grad = lossv + B, *m = grad + NP, *v = m + NP;
  cudaMemset(m, 0, sizeof(float) * 2 * NP);
  std::vector<float> lv(B);
  mfgb_status st = MFGB_OK;
  double b1t = 1.0, b2t = 1.0;
  for (int s = 0; s < steps && !st; ++s) {
    b1t *= 0.9;
    b2t *= 0.999;
    batch_indices<<<g1(B), 256>>>(B, n, seed + 0x1000193ull * (uint64_t)s, idx);
    mlp_fwd1<<<g1((int64_t)B * NH), 256>>>(B, d_params, d_X, idx, Z1);
    mlp_fwd2<<<g1((int64_t)B * NH), 256>>>(B, d_params, Z1, Z2);
    mlp_fwd3<<<g1(B), 256>>>(B, d_params, Z2, d_t, idx, dz3, lossv, nullptr);
    mlp_bwd2<<<g1((int64_t)B * NH), 256>>>(B, d_params, Z2, dz3, dH2);
    mlp_bwd1<<<g1((int64_t)B * NH), 256>>>(B, d_params, Z1, dH2, dH1);
    mlp_grads<<<g1(NP), 256>>>(B, d_X, idx, Z1, Z2, dz3, dH1, dH2, grad);
    adam_step<<<g1(NP), 256>>>(d_params, grad, m, v, lr, (float)b1t, (float)b2t);
    if (h_loss) {
      st = cuda_status(cudaMemcpy(lv.data(), lossv, sizeof(float) * B, cudaMemcpyDeviceToHost), "loss");
      double L = 0;
      for (float x : lv) L += x;
      h_loss[s] = (float)(L / B);
    }
  }
  if (!st) st = cuda_status(cudaDeviceSynchronize(), "mlp train");
  cudaFree(buf);
  cudaFree(idx);
  return st;
}

// y = MLP(X) in FP32 (SIMT), for checks
mfgb_status mfgb_mlp_forward_f32(const float *d_params, const float *d_X, int n, float *d_y) {
  if (!d_params || !d_X || n < 1 || !d_y) {
    set_error("mfgb_mlp_forward_f32: invalid argument");
    return MFGB_ERR_INVALID_ARG;
  }
  float *buf = nullptr;
  int *idx = nullptr;
  if (cudaMalloc(&buf, sizeof(float) * (size_t)n * 2 * NH) != cudaSuccess ||
      cudaMalloc(&idx, sizeof(int) * n) != cudaSuccess) {
    cudaFree(buf);
    return cuda_status(cudaErrorMemoryAllocation, "mlp buffers");
  }
  iota_kernel<<<g1(n), 256>>>(n, 0, idx);
  mlp_fwd1<<<g1((int64_t)n * NH), 256>>>(n, d_params, d_X, idx, buf);
  mlp_fwd2<<<g1((int64_t)n * NH), 256>>>(n, d_params, buf, buf + (size_t)n * NH);
  mlp_fwd3<<<g1(n), 256>>>(n, d_params, buf + (size_t)n * NH, nullptr, idx, nullptr, nullptr, d_y);
  mfgb_status st = cuda_status(cudaDeviceSynchronize(), "mlp forward");
  cudaFree(buf);
  cudaFree(idx);
  return st;
}

// y = MLP(X) with BF16 tensor-core MMAs (FP32 accumulate), FP64 output
mfgb_status mfgb_mlp_infer(const float *d_params, const float *d_X, int64_t n, double *d_y,
                           void *stream) {
  if (!d_params || !d_X || n < 0 || (n > 0 && !d_y)) {
    set_error("mfgb_mlp_infer: invalid argument");
    return MFGB_ERR_INVALID_ARG;
  }
  if (n == 0) return MFGB_OK;
  const int64_t tiles = (n + 15) / 16;
  const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>((tiles + 3) / 4, 152 * 8));
  mlp_infer_bf16<<<grid, 128, 0, (cudaStream_t)stream>>>(n, d_params, d_X, d_y);
  return cuda_status(cudaGetLastError(), "mfgb_mlp_infer");
}

}  // extern "C"
