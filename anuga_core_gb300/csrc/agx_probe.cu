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

// ---- device self-check of soft64.cuh against the FP64 pipe ----------------
__device__ __forceinline__ uint64_t mix64(uint64_t x) {     // splitmix64 finaliser
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

__device__ __forceinline__ bool same_result(double ref, double got) {
  const uint64_t r = soft64::bits(ref), g = soft64::bits(got);
  const bool rn = (r & ~soft64::SIGN) > soft64::EXP_MASK, gn = (g & ~soft64::SIGN) > soft64::EXP_MASK;
  return rn ? gn : r == g;                    // a NaN only has to be a NaN
}

// Case i draws a pair (a, b) of one of four classes: any bit pattern; b with
// an exponent within 35 of a's (cancellation and carries in add/sub); a and
// b moderate integers times powers of two (exact and tie quotients and
// products); results near and below the normal range.  mism[0..4] count the
// add, sub, mul, div and sqrt results that differ from the FP64 pipe's.
__global__ void k_soft64_check(long long n, uint64_t seed, unsigned long long* mism) {
  unsigned long long m[5] = {0, 0, 0, 0, 0};
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const uint64_t h0 = mix64(seed ^ (uint64_t)i), h1 = mix64(h0), h2 = mix64(h1), h3 = mix64(h2);
    uint64_t ab = h0, bb = h1;
    switch (h2 & 3) {
      case 0:
        break;
      case 1: {
        const int de = (int)(h3 % 71) - 35;
        bb = (h1 & 0x800fffffffffffffull) | ((((ab >> 52) & 0x7ff) + de) & 0x7ff) << 52;
        break;
      }
      case 2: {
        const double a = (double)(int64_t)(h0 >> (h3 & 63)) * ldexp(1.0, (int)(h2 >> 8 & 127) - 64);
        const double b = (double)(int64_t)((h1 >> (h3 >> 6 & 63)) | 1) * ldexp(1.0, (int)(h2 >> 16 & 127) - 64);
        ab = soft64::bits(a);
        bb = soft64::bits(b);
        break;
      }
      default:
        ab = (h0 & 0x800fffffffffffffull) | (uint64_t)(h3 % 64) << 52;           // tiny exponents
        bb = (h1 & 0x800fffffffffffffull) | (uint64_t)(1023 - (h3 >> 8) % 64) << 52;
        break;
    }
    const double a = soft64::from_bits(ab), b = soft64::from_bits(bb);
    m[0] += !same_result(__dadd_rn(a, b), soft64::add(a, b));
    m[1] += !same_result(__dsub_rn(a, b), soft64::sub(a, b));
    m[2] += !same_result(__dmul_rn(a, b), soft64::mul(a, b));
    m[3] += !same_result(__ddiv_rn(a, b), soft64::div(a, b));
    m[4] += !same_result(__dsqrt_rn(a), soft64::sqrt(a));
  }
  for (int j = 0; j < 5; j++)
    if (m[j]) atomicAdd(mism + j, m[j]);
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

// Runs n cases of each soft64.cuh operation on the device against the FP64
// pipe's IEEE operations; writes the mismatch count of add, sub, mul, div and
// sqrt to mism5.
extern "C" agx_status agx_soft64_check(long long n, unsigned long long seed, unsigned long long* mism5) {
  if (!mism5 || n < 0) return AGX_E_INVALID;
  unsigned long long* d = nullptr;
  if (cudaMalloc(&d, 5 * sizeof(unsigned long long)) != cudaSuccess) return AGX_E_NOMEM;
  cudaError_t e = cudaMemset(d, 0, 5 * sizeof(unsigned long long));
  int dev = 0, sms = 0;
  if (e == cudaSuccess) e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) {
    k_soft64_check<<<4 * sms, 256>>>(n, seed, d);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(mism5, d, 5 * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
  cudaFree(d);
  return e == cudaSuccess ? AGX_OK : AGX_E_CUDA;
}
