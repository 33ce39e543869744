// mfgb_rates.cu -- arithmetic-pipe and host-link throughput on the running GPU,
// the numbers the
// operator kernels' choice of arithmetic rests on: FP64 FMA (DFMA), FP32 FMA,
// FP64 tensor-core MMA (mma.sync m8n8k4 f64, the instruction of the reference's
// sum_factorization/include/kernels/BK1/cuda_mma_kernels.cuh:94-100) and the
// legacy BF16 tensor-core MMA (mma.sync m16n8k16, FP32 accumulation).
//
// Every kernel runs independent dependency chains in registers (no memory
// traffic but one store per thread, which keeps the work alive) on a grid of
// 8 CTAs x 256 threads per SM.  mfgb_pipe_rate returns operations per second
// (FLOP/s counting an FMA as 2) from CUDA-event timing of `reps` launches.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>

#include "mfgb.h"
#include "mfgb_internal.h"

namespace mfgb {
namespace {

constexpr int kChains = 8;

__global__ void __launch_bounds__(256) dfma_kernel(int iters, double *out) {
  double a[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) a[c] = 1.0 + 1e-3 * (threadIdx.x + c);
  const double x = 0.999999, y = 1e-7;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) a[c] = __fma_rn(a[c], x, y);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += a[c];
  out[blockIdx.x * (int64_t)blockDim.x + threadIdx.x] = s;
}

__global__ void __launch_bounds__(256) ffma_kernel(int iters, double *out) {
  float a[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) a[c] = 1.f + 1e-3f * (threadIdx.x + c);
  const float x = 0.9999f, y = 1e-7f;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) a[c] = __fmaf_rn(a[c], x, y);
  }
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += a[c];
  out[blockIdx.x * (int64_t)blockDim.x + threadIdx.x] = s;
}

// packed dual FP32 FMA (fma.rn.f32x2, __ffma2_rn): two FMAs per instruction
__global__ void __launch_bounds__(256) ffma2_kernel(int iters, double *out) {
  float2 a[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c)
    a[c] = make_float2(1.f + 1e-3f * (threadIdx.x + c), 1.f - 1e-3f * (threadIdx.x + c));
  const float2 x = make_float2(0.9999f, 0.9998f), y = make_float2(1e-7f, 2e-7f);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) a[c] = __ffma2_rn(a[c], x, y);
  }
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += a[c].x + a[c].y;
  out[blockIdx.x * (int64_t)blockDim.x + threadIdx.x] = s;
}

// FP32 FMAs interleaved with one integer logic instruction (lop3) per chain
// step: PAIRED = false issues two scalar FMAs per step, PAIRED = true one
// packed FMA.  Against pipes 1 / 4 this shows whether the integer work finds
// issue slots that the FMAs leave free.
template <bool PAIRED>
__global__ void __launch_bounds__(256) fma_alu_kernel(int iters, double *out) {
  float2 a[kChains];
  uint32_t h[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) {
    a[c] = make_float2(1.f + 1e-3f * (threadIdx.x + c), 1.f - 1e-3f * (threadIdx.x + c));
    h[c] = threadIdx.x * 2654435761u + c;
  }
  const float2 x = make_float2(0.9999f, 0.9998f), y = make_float2(1e-7f, 2e-7f);
  const uint32_t m1 = threadIdx.x | 1u, m2 = threadIdx.x * 7u;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) {
      if (PAIRED) {
        a[c] = __ffma2_rn(a[c], x, y);
      } else {
        a[c].x = __fmaf_rn(a[c].x, x.x, y.x);
        a[c].y = __fmaf_rn(a[c].y, x.y, y.y);
      }
      asm volatile("lop3.b32 %0, %0, %1, %2, 0x96;" : "+r"(h[c]) : "r"(m1), "r"(m2));
    }
  }
  float s = 0.f;
  uint32_t t = 0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += a[c].x + a[c].y, t ^= h[c];
  out[blockIdx.x * (int64_t)blockDim.x + threadIdx.x] = s + (double)(t & 1u);
}

// D(8x8) += A(8x4) B(4x8) in FP64: per thread one A and one B element, two
// accumulator elements; 4 independent accumulators per warp
__global__ void __launch_bounds__(256) dmma_kernel(int iters, double *out) {
  double acc[4][2];
#pragma unroll
  for (int c = 0; c < 4; ++c) acc[c][0] = acc[c][1] = 0.0;
  const double a = 1.0 + 1e-3 * threadIdx.x, b = 0.5 - 1e-4 * threadIdx.x;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < 4; ++c)
      asm volatile(
          "mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
          : "+d"(acc[c][0]), "+d"(acc[c][1])
          : "d"(a), "d"(b));
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < 4; ++c) s += acc[c][0] + acc[c][1];
  out[blockIdx.x * (int64_t)blockDim.x + threadIdx.x] = s;
}

// D(16x8) += A(16x16) B(16x8), BF16 inputs, FP32 accumulation
__global__ void __launch_bounds__(256) hmma_kernel(int iters, double *out) {
  float acc[4][4];
#pragma unroll
  for (int c = 0; c < 4; ++c)
#pragma unroll
    for (int r = 0; r < 4; ++r) acc[c][r] = 0.f;
  const uint32_t a0 = 0x3F803F80u + threadIdx.x, b0 = 0x3F003F00u + threadIdx.x;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < 4; ++c)
      asm volatile(
          "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, "
          "{%8, %9}, {%0, %1, %2, %3};"
          : "+f"(acc[c][0]), "+f"(acc[c][1]), "+f"(acc[c][2]), "+f"(acc[c][3])
          : "r"(a0), "r"(a0), "r"(a0), "r"(a0), "r"(b0), "r"(b0));
  }
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < 4; ++c) s += acc[c][0] + acc[c][1] + acc[c][2] + acc[c][3];
  out[blockIdx.x * (int64_t)blockDim.x + threadIdx.x] = s;
}

// 16-byte copy by the SMs (host memory read or written through its device
// mapping), four independent loads in flight per thread
__global__ void __launch_bounds__(512) link_copy_kernel(const int4 *__restrict__ s,
                                                        int4 *__restrict__ d, size_t n) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t st = (size_t)gridDim.x * blockDim.x;
  for (; i + 3 * st < n; i += 4 * st) {
    const int4 a = s[i], b = s[i + st], c = s[i + 2 * st], e = s[i + 3 * st];
    d[i] = a, d[i + st] = b, d[i + 2 * st] = c, d[i + 3 * st] = e;
  }
  for (; i < n; i += st) d[i] = s[i];
}

}  // namespace
}  // namespace mfgb

using namespace mfgb;

// Host link throughput with pinned host buffers of `bytes` (a multiple of 16):
// mode 0 host->device, 1 device->host, 2 both directions at once, by the copy
// engines (cudaMemcpyAsync); modes 3 / 4 / 5 the same by an SM copy kernel (64
// CTAs per direction).  *bytes_per_s = bytes moved (both directions summed) per
// second, best of `reps`.
extern "C" mfgb_status mfgb_link_rate(int mode, int64_t bytes, int reps, double *bytes_per_s) {
  if (mode < 0 || mode > 5 || bytes < 16 || bytes % 16 || reps < 1 || !bytes_per_s) {
    set_error("mfgb_link_rate: invalid argument");
    return MFGB_ERR_INVALID_ARG;
  }
  void *h_a = nullptr, *h_b = nullptr, *d_a = nullptr, *d_b = nullptr;
  cudaStream_t s0 = nullptr, s1 = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr, ej = nullptr;
  mfgb_status st = MFGB_OK;
  if ((st = cuda_status(cudaHostAlloc(&h_a, bytes, cudaHostAllocDefault), "link host buffer")) ||
      (st = cuda_status(cudaHostAlloc(&h_b, bytes, cudaHostAllocDefault), "link host buffer")) ||
      (st = cuda_status(cudaMalloc(&d_a, bytes), "link device buffer")) ||
      (st = cuda_status(cudaMalloc(&d_b, bytes), "link device buffer")) ||
      (st = cuda_status(cudaStreamCreateWithFlags(&s0, cudaStreamNonBlocking), "link stream")) ||
      (st = cuda_status(cudaStreamCreateWithFlags(&s1, cudaStreamNonBlocking), "link stream")) ||
      (st = cuda_status(cudaEventCreate(&e0), "link event")) ||
      (st = cuda_status(cudaEventCreate(&e1), "link event")) ||
      (st = cuda_status(cudaEventCreateWithFlags(&ej, cudaEventDisableTiming), "link event"))) {
  } else {
    memset(h_a, 0, bytes);
    const size_t n16 = (size_t)bytes / 16;
    const bool up = mode == 0 || mode == 2 || mode == 3 || mode == 5;
    const bool down = mode == 1 || mode == 2 || mode == 4 || mode == 5;
    const bool sm = mode >= 3;
    auto once = [&]() {
      cudaEventRecord(e0, s0);
      cudaStreamWaitEvent(s1, e0, 0);
      if (up) {
        if (sm)
          link_copy_kernel<<<64, 512, 0, s0>>>((const int4 *)h_a, (int4 *)d_a, n16);
        else
          cudaMemcpyAsync(d_a, h_a, bytes, cudaMemcpyHostToDevice, s0);
      }
      if (down) {
        if (sm)
          link_copy_kernel<<<64, 512, 0, s1>>>((const int4 *)d_b, (int4 *)h_b, n16);
        else
          cudaMemcpyAsync(h_b, d_b, bytes, cudaMemcpyDeviceToHost, s1);
      }
      cudaEventRecord(ej, s1);
      cudaStreamWaitEvent(s0, ej, 0);
      cudaEventRecord(e1, s0);
      return cudaEventSynchronize(e1);
    };
    float best = 0.f;
    for (int r = -1; r < reps && !st; ++r) {  // one warm-up
      float ms = 0.f;
      cudaError_t e = once();
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
      st = cuda_status(e, "mfgb_link_rate");
      if (!st && r >= 0 && (best == 0.f || ms < best)) best = ms;
    }
    if (!st) *bytes_per_s = (double)bytes * ((up ? 1 : 0) + (down ? 1 : 0)) / (best * 1e-3);
  }
  if (ej) cudaEventDestroy(ej);
  if (e1) cudaEventDestroy(e1);
  if (e0) cudaEventDestroy(e0);
  if (s1) cudaStreamDestroy(s1);
  if (s0) cudaStreamDestroy(s0);
  cudaFree(d_b);
  cudaFree(d_a);
  cudaFreeHost(h_b);
  cudaFreeHost(h_a);
  return st;
}

// pipe: 0 DFMA, 1 FFMA, 2 DMMA m8n8k4 f64, 3 BF16 mma.sync m16n8k16,
// 4 packed FFMA2, 5 FFMA + lop3, 6 FFMA2 + lop3.
// *ops_per_s = floating-point operations per second (FMA = 2, MMA = 2 m n k;
// the lop3 of pipes 5 / 6 counts nothing).
extern "C" mfgb_status mfgb_pipe_rate(int pipe, int iters, int reps, double *ops_per_s) {
  if (pipe < 0 || pipe > 6 || iters < 1 || reps < 1 || !ops_per_s) {
    set_error("mfgb_pipe_rate: invalid argument");
    return MFGB_ERR_INVALID_ARG;
  }
  int dev = 0, sms = 0;
  mfgb_status st;
  if ((st = cuda_status(cudaGetDevice(&dev), "cudaGetDevice")) ||
      (st = cuda_status(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev),
                        "SM count")))
    return st;
  const int blocks = 8 * sms, threads = 256;
  double *out = nullptr;
  if ((st = cuda_status(cudaMalloc(&out, sizeof(double) * blocks * threads), "rates buffer")))
    return st;
  auto launch = [&]() {
    switch (pipe) {
      case 0: dfma_kernel<<<blocks, threads>>>(iters, out); break;
      case 1: ffma_kernel<<<blocks, threads>>>(iters, out); break;
      case 2: dmma_kernel<<<blocks, threads>>>(iters, out); break;
      case 3: hmma_kernel<<<blocks, threads>>>(iters, out); break;
      case 4: ffma2_kernel<<<blocks, threads>>>(iters, out); break;
      case 5: fma_alu_kernel<false><<<blocks, threads>>>(iters, out); break;
      default: fma_alu_kernel<true><<<blocks, threads>>>(iters, out); break;
    }
  };
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  launch();  // warm-up
  cudaEventRecord(e0);
  for (int r = 0; r < reps; ++r) launch();
  cudaEventRecord(e1);
  cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if ((st = cuda_status(e, "mfgb_pipe_rate"))) return st;
  const double threads_total = (double)blocks * threads;
  double flops_per_iter;  // per thread
  switch (pipe) {
    case 0:
    case 1: flops_per_iter = 2.0 * kChains; break;
    case 2: flops_per_iter = 4.0 * 2.0 * 8 * 8 * 4 / 32.0; break;   // 4 MMAs per warp
    case 3: flops_per_iter = 4.0 * 2.0 * 16 * 8 * 16 / 32.0; break;
    default: flops_per_iter = 4.0 * kChains; break;                  // two FMAs per chain
  }
  *ops_per_s = threads_total * flops_per_iter * iters * reps / (ms * 1e-3);
  return MFGB_OK;
}
