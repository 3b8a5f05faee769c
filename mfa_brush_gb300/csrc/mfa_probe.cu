// mfa_probe.cu -- FP32 FMA throughput of the device: the roof of the FP32-issue-bound kernels
// (pair forces, k-space).  Every thread runs eight independent FMA chains, so one warp per SM
// sub-partition could keep the FMA pipe busy; the grid holds eight warps per sub-partition.
#include <cuda_runtime.h>

#include <algorithm>

#include "mfa_gpu.h"

namespace {

constexpr int PROBE_CHAINS = 8;
constexpr int PROBE_THREADS = 256;

__global__ void __launch_bounds__(PROBE_THREADS) k_fma_probe(float* out, int iters, float a, float b) {
  float x[PROBE_CHAINS];
#pragma unroll
  for (int i = 0; i < PROBE_CHAINS; ++i) x[i] = 1e-3f * (float)threadIdx.x + (float)i;
#pragma unroll 16
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < PROBE_CHAINS; ++i) x[i] = fmaf(x[i], a, b);
  }
  float s = 0.f;
#pragma unroll
  for (int i = 0; i < PROBE_CHAINS; ++i) s += x[i];
  if (s == -1.f) out[blockIdx.x] = s;  // never true (a, b > 0): keeps every chain live
}

}  // namespace

extern "C" int mfa_fp32_fma_peak(int32_t device, double* tflops) {
  if (!tflops) return MFA_ERR_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return MFA_ERR_NO_DEVICE;
  if (device < 0 || device >= ndev) return MFA_ERR_ARG;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(device);
  cudaDeviceProp pr;
  cudaGetDeviceProperties(&pr, device);
  const int blocks = pr.multiProcessorCount * 4;  // 4 x 256 threads: 8 warps per sub-partition
  const int iters = 4096;
  float* out = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = MFA_OK;
  if (cudaMalloc(&out, sizeof(float) * blocks) != cudaSuccess || cudaStreamCreate(&st) != cudaSuccess ||
      cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    rc = MFA_ERR_CUDA;
  } else {
    float best = 1e30f;
    for (int rep = 0; rep < 12; ++rep) {
      cudaEventRecord(e0, st);
      k_fma_probe<<<blocks, PROBE_THREADS, 0, st>>>(out, iters, 0.999f, 1e-3f);
      cudaEventRecord(e1, st);
      if (cudaEventSynchronize(e1) != cudaSuccess) {
        rc = MFA_ERR_CUDA;
        break;
      }
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep >= 2) best = std::min(best, ms);  // two warm-up launches
    }
    if (rc == MFA_OK) {
      const double flop = 2.0 * PROBE_CHAINS * (double)iters * blocks * PROBE_THREADS;
      *tflops = flop / (best * 1e-3) / 1e12;
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  if (out) cudaFree(out);
  cudaSetDevice(prev);
  return rc;
}
