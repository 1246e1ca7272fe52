// peaks.cu -- throughput microbenchmarks that give the roofline denominators
// a copy-bandwidth and GEMM measurement does not: FP64 and FP32 arithmetic
// issue rates and the L2 read bandwidth of this GPU.  Built as its own library
// (libxdgpeaks.so), separate from the engine's C ABI; bench.py runs it on the
// same GPU in the same process as the kernels whose fractions it reports.
//
// Each rate kernel runs 8 independent dependency chains per thread over a
// grid of (SM count x 2048 / block) blocks, so every SM has enough warps in
// flight to hide the pipe latency and the measured figure is the issue rate.
// Every operation is an explicit intrinsic (__dadd_rn, __dmul_rn, __fma_rn,
// __fmaf_rn), so the instruction mix does not depend on -fmad.  Counted in
// thread-operations per second: one DADD, DMUL or DFMA is one operation.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <vector>

namespace {

constexpr int kBlock = 256;
constexpr int kChains = 8;

template <int KIND>
__global__ void __launch_bounds__(kBlock) k_rate64(double* out, int64_t iters, double a, double b) {
  const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) x[c] = 1.0 + 1e-3 * (double)((g + c) & 1023);
  for (int64_t i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) {
      if (KIND == 0) x[c] = __dadd_rn(x[c], b);
      if (KIND == 1) x[c] = __dmul_rn(x[c], a);
      if (KIND == 2) x[c] = __fma_rn(x[c], a, b);
    }
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += x[c];
  out[g] = s;
}

__global__ void __launch_bounds__(kBlock) k_rate32(float* out, int64_t iters, float a, float b) {
  const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  float x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) x[c] = 1.0f + 1e-3f * (float)((g + c) & 1023);
  for (int64_t i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = __fmaf_rn(x[c], a, b);
  }
  float s = 0.0f;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += x[c];
  out[g] = s;
}

// Reads `n4` float4 of `buf` `passes` times (L1 bypassed), grid-stride.
__global__ void __launch_bounds__(kBlock) k_l2_read(const float4* __restrict__ buf, int64_t n4,
                                                   int passes, float* out) {
  const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  float s = 0.0f;
  for (int p = 0; p < passes; ++p) {
    for (int64_t i = g; i < n4; i += stride) {
      const float4 v = __ldcg(&buf[i]);
      s += v.x + v.y + v.z + v.w;
    }
  }
  out[g] = s;
}

float median(std::vector<float> v) {
  std::sort(v.begin(), v.end());
  return v[v.size() / 2];
}

}  // namespace

extern "C" {

// kind: 0 FP64 add, 1 FP64 multiply, 2 FP64 fused multiply-add, 3 FP32 fused
// multiply-add (thread-operations per second), 4 L2 read bandwidth (bytes
// per second over a 32 MiB buffer, well inside the 129 MB L2).  `reps` timed
// launches after two warm-up launches; the median launch is reported.
// Returns 0, or the CUDA error code.
int xdgpk_measure(int device, int kind, int reps, double* per_second, double* ms_median) {
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return (int)e;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const int blocks = sms * (2048 / kBlock);
  const int64_t threads = (int64_t)blocks * kBlock;
  void* out = nullptr;
  float4* buf = nullptr;
  const int64_t n4 = (32ll << 20) / 16;
  const int passes = 2048;
  e = cudaMalloc(&out, threads * sizeof(double));
  if (e == cudaSuccess && kind == 4) {
    e = cudaMalloc(&buf, n4 * 16);
    if (e == cudaSuccess) e = cudaMemset(buf, 0, n4 * 16);
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  // iterations per thread: about 20-60 ms per launch at the expected rates
  const int64_t iters = kind <= 2 ? 4096 : 262144;
  auto launch = [&]() {
    switch (kind) {
      case 0: k_rate64<0><<<blocks, kBlock>>>((double*)out, iters, 1.0000001, 1e-9); break;
      case 1: k_rate64<1><<<blocks, kBlock>>>((double*)out, iters, 1.0000001, 1e-9); break;
      case 2: k_rate64<2><<<blocks, kBlock>>>((double*)out, iters, 0.9999999, 1e-9); break;
      case 3: k_rate32<<<blocks, kBlock>>>((float*)out, iters, 0.9999f, 1e-4f); break;
      default: k_l2_read<<<blocks, kBlock>>>(buf, n4, passes, (float*)out); break;
    }
  };
  std::vector<float> t;
  if (e == cudaSuccess && (kind < 0 || kind > 4)) e = cudaErrorInvalidValue;
  for (int r = 0; e == cudaSuccess && r < reps + 2; ++r) {
    cudaEventRecord(e0);
    launch();
    cudaEventRecord(e1);
    e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaGetLastError();
    float ms = 0.0f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e == cudaSuccess && r >= 2) t.push_back(ms);
  }
  if (e == cudaSuccess && !t.empty()) {
    const double ms = median(t);
    const double work = kind == 4 ? (double)n4 * 16.0 * passes : (double)threads * iters * kChains;
    *per_second = work / (ms * 1e-3);
    *ms_median = ms;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (out) cudaFree(out);
  if (buf) cudaFree(buf);
  return (int)e;
}

}  // extern "C"
