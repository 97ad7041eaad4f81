// agx_probe.cu -- FP64 throughput probe: the compute ceiling of the plain
// FP64 path (GB300 executes FP64 at a small fraction of its FP32 rate).
//
// Each thread runs 8 independent dependent chains of one operation, so the
// pipe is kept busy while each chain waits on its own latency; the grid is
// 8 blocks of 256 threads per SM.  Operations per second = threads x chains x
// iterations / kernel time (CUDA events).
#include "agx_internal.cuh"
#include "soft64.cuh"
#include <cuda_runtime.h>

namespace {

constexpr int PROBE_CHAINS = 8;

template <int OP>
__global__ void k_fp64_probe(double* out, int iters, double seed) {
  double a[PROBE_CHAINS];
#pragma unroll
  for (int j = 0; j < PROBE_CHAINS; ++j) a[j] = seed + threadIdx.x * 1.0e-9 + j * 1.0e-7;
#pragma unroll 1
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < PROBE_CHAINS; ++j) {
      if (OP == 0) a[j] = fma(a[j], 1.0000001, 1.0e-9);
      if (OP == 1) a[j] = 1.5 / a[j];
      if (OP == 2) a[j] = sqrt(a[j]);
      // the FP64 pipe's add and multiply, the same four on the integer pipes
      // (soft64.cuh), and half of the chains on each (both pipes at once)
      if (OP == 3) a[j] = a[j] + 1.0e-9;
      if (OP == 4) a[j] = a[j] * 1.0000001;
      if (OP == 5) a[j] = soft64::add(a[j], 1.0e-9);
      if (OP == 6) a[j] = soft64::mul(a[j], 1.0000001);
      if (OP == 7) a[j] = soft64::div(1.5, a[j]);
      if (OP == 8) a[j] = soft64::sqrt(a[j]);
      if (OP == 9) a[j] = j & 1 ? soft64::div(1.5, a[j]) : 1.5 / a[j];
      if (OP == 10) a[j] = j & 1 ? soft64::mul(a[j], 1.0000001) : a[j] * 1.0000001;
    }
  }
  double s = 0.0;
#pragma unroll
  for (int j = 0; j < PROBE_CHAINS; ++j) s += a[j];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;    // keeps the chains live
}

template <int OP>
cudaError_t time_probe(double* out, int blocks, int iters, double* gops) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float ms = 0.0f;
  cudaError_t e = cudaSuccess;
  for (int r = 0; r < 2 && e == cudaSuccess; r++) {        // first pass warms up
    cudaEventRecord(e0);
    k_fp64_probe<OP><<<blocks, 256>>>(out, iters, 1.25);
    cudaEventRecord(e1);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  }
  agx::count_launch(2);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *gops = (double)blocks * 256.0 * PROBE_CHAINS * iters / (ms * 1.0e-3) / 1.0e9;
  return e;
}

}  // namespace

extern "C" agx_status agx_fp64_throughput(double* dfma_gops, double* ddiv_gops, double* dsqrt_gops) {
  if (!dfma_gops || !ddiv_gops || !dsqrt_gops) return AGX_E_INVALID;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return AGX_E_CUDA;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return AGX_E_CUDA;
  const int blocks = 8 * sms;
  double* out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * blocks * 256) != cudaSuccess) return AGX_E_NOMEM;
  cudaError_t e = time_probe<0>(out, blocks, 512, dfma_gops);
  if (e == cudaSuccess) e = time_probe<1>(out, blocks, 64, ddiv_gops);
  if (e == cudaSuccess) e = time_probe<2>(out, blocks, 64, dsqrt_gops);
  cudaFree(out);
  return e == cudaSuccess ? AGX_OK : AGX_E_CUDA;
}

// Throughput of binary64 add, multiply, divide and square root on the FP64
// pipe (out[0..3]) and carried out with integer instructions by soft64.cuh
// (out[4..7]), and with half of the work on each (divide out[8], multiply
// out[9]), in G operations per second over the whole device.
extern "C" agx_status agx_soft64_throughput(double* out8) {
  if (!out8) return AGX_E_INVALID;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return AGX_E_CUDA;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return AGX_E_CUDA;
  const int blocks = 8 * sms;
  double* out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * blocks * 256) != cudaSuccess) return AGX_E_NOMEM;
  cudaError_t e = time_probe<3>(out, blocks, 512, out8 + 0);
  if (e == cudaSuccess) e = time_probe<4>(out, blocks, 512, out8 + 1);
  if (e == cudaSuccess) e = time_probe<1>(out, blocks, 64, out8 + 2);
  if (e == cudaSuccess) e = time_probe<2>(out, blocks, 64, out8 + 3);
  if (e == cudaSuccess) e = time_probe<5>(out, blocks, 128, out8 + 4);
  if (e == cudaSuccess) e = time_probe<6>(out, blocks, 128, out8 + 5);
  if (e == cudaSuccess) e = time_probe<7>(out, blocks, 64, out8 + 6);
  if (e == cudaSuccess) e = time_probe<8>(out, blocks, 64, out8 + 7);
  if (e == cudaSuccess) e = time_probe<9>(out, blocks, 64, out8 + 8);
  if (e == cudaSuccess) e = time_probe<10>(out, blocks, 256, out8 + 9);
  cudaFree(out);
  return e == cudaSuccess ? AGX_OK : AGX_E_CUDA;
}
