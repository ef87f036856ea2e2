// FP64 throughput microbenchmarks: the compute roofline of the assembly
// kernels on this GPU.  Each thread runs 8 independent FMA chains (FP64 pipe)
// or 4 independent mma.sync.m8n8k4 f64 accumulations (FP64 tensor pipe), or
// (kind 2) the even warps of every block the FMA chains and the odd warps
// the MMA accumulations, which shows whether the two share issue resources;
// the result is written out so nothing is optimised away.  Grids are sized
// to the SM count; every index stays within the output buffer.
#include <cuda_runtime.h>

#include <string>

#include "../../include/gfgpu.h"

namespace gfgpu {
void set_last_error(const std::string &s);
}

namespace {

__global__ void fma_chains(double *out, int iters, double a, double b) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5,
         x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

__global__ void dmma_chains(double *out, int iters) {
  double a = 1.0 + threadIdx.x * 1e-3, b = 0.5;
  double c[4][2] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}};
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 4; ++k)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                   : "+d"(c[k][0]), "+d"(c[k][1])
                   : "d"(a), "d"(b));
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = c[0][0] + c[0][1] + c[1][0] + c[1][1] + c[2][0] +
                                               c[2][1] + c[3][0] + c[3][1];
}

// even warps: the FMA chains of fma_chains; odd warps: the MMA
// accumulations of dmma_chains
__global__ void mixed_chains(double *out, int fma_iters, int mma_iters, double a, double b) {
  double r = 0.0;
  if (((threadIdx.x >> 5) & 1) == 0) {
    double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5,
           x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < fma_iters; ++i) {
      x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
      x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    r = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  } else {
    double ma = 1.0 + threadIdx.x * 1e-3, mb = 0.5;
    double c[4][2] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}};
    for (int i = 0; i < mma_iters; ++i) {
#pragma unroll
      for (int k = 0; k < 4; ++k)
        asm volatile(
            "mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
            : "+d"(c[k][0]), "+d"(c[k][1])
            : "d"(ma), "d"(mb));
    }
    r = c[0][0] + c[0][1] + c[1][0] + c[1][1] + c[2][0] + c[2][1] + c[3][0] + c[3][1];
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = r;
}

}  // namespace

extern "C" int gfgpu_fp64_peak(int32_t kind, double *tflops) {
  if (!tflops || kind < 0 || kind > 2) return GFGPU_E_INVALID;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    gfgpu::set_last_error("no CUDA device");
    return GFGPU_E_CUDA;
  }
  const int threads = 256, blocks = sms * 8;
  double *out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * threads * blocks) != cudaSuccess) return GFGPU_E_NOMEM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int iters = kind == 0 ? 4096 : 2048;
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(e0);
    if (kind == 0) fma_chains<<<blocks, threads>>>(out, iters, 1.0000001, 1e-9);
    else if (kind == 1) dmma_chains<<<blocks, threads>>>(out, iters);
    else mixed_chains<<<blocks, threads>>>(out, 4096, 2048, 1.0000001, 1e-9);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  cudaError_t ce = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (ce != cudaSuccess) {
    gfgpu::set_last_error(cudaGetErrorString(ce));
    return GFGPU_E_CUDA;
  }
  const double fma_flops = 2.0 * 8 * 4096 * double(blocks) * threads;
  const double mma_flops = 4.0 * 2048 * double(blocks) * (threads / 32) * 512.0;
  const double flops = kind == 0 ? fma_flops : kind == 1 ? mma_flops : 0.5 * (fma_flops + mma_flops);
  *tflops = flops / (best * 1e-3) / 1e12;
  return GFGPU_OK;
}
