// Integer-pipe peak of this GPU, measured: the rate of 3-input logic ops
// (lop3) and of 32-bit funnel shifts (shf), the two instruction kinds a
// Keccak-f[1600] permutation on 32-bit halves is made of (XOR / AND-NOT
// combinations and 64-bit rotations). The ceiling of a Keccak kernel follows
// from these rates and the permutation's op count.
//
// Each thread runs 8 independent dependency chains of one op kind in inline
// PTX (so nothing is folded), every SM holds 8 blocks of 256 threads, and the
// time of the whole grid is taken with CUDA events (median of 5 after 2
// warm-ups).
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/gmc.h"
#include "engine_internal.h"
#include "kernels.h"

using namespace gmc;

namespace {

constexpr int kChains = 8;
constexpr int kPeakThreads = 256;

template <bool SHF>
__global__ void __launch_bounds__(kPeakThreads) int_peak_kernel(uint32_t *out, int iters, uint32_t salt) {
  uint32_t a[kChains];
#pragma unroll
  for (int u = 0; u < kChains; u++) a[u] = (threadIdx.x + 977u * u) ^ salt;
  const uint32_t b = blockIdx.x * 2654435761u ^ salt, c = 0x5bd1e995u;
#pragma unroll 1
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int r = 0; r < 8; r++)
#pragma unroll
      for (int u = 0; u < kChains; u++) {
        if (SHF)
          asm volatile("shf.l.wrap.b32 %0, %0, %1, 7;" : "+r"(a[u]) : "r"(b));
        else
          asm volatile("lop3.b32 %0, %0, %1, %2, 0x96;" : "+r"(a[u]) : "r"(b), "r"(c));
      }
  }
  uint32_t x = 0;
#pragma unroll
  for (int u = 0; u < kChains; u++) x ^= a[u];
  if (x == 0x9e3779b9u) out[0] = x;  // keeps the chains live; practically never stored
}

template <bool SHF>
cudaError_t time_kernel(int blocks, int iters, uint32_t *out, cudaStream_t st, double *ops_per_s) {
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  std::vector<float> ms;
  for (int rep = 0; rep < 7 && e == cudaSuccess; rep++) {
    cudaEventRecord(e0, st);
    int_peak_kernel<SHF><<<blocks, kPeakThreads, 0, st>>>(out, iters, 0x1234567u + rep);
    cudaEventRecord(e1, st);
    e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaGetLastError();
    float t = 0;
    cudaEventElapsedTime(&t, e0, e1);
    if (rep >= 2) ms.push_back(t);
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (e != cudaSuccess) return e;
  std::sort(ms.begin(), ms.end());
  const double ops = (double)blocks * kPeakThreads * iters * 8.0 * kChains;
  *ops_per_s = ops / (ms[ms.size() / 2] * 1e-3);
  return cudaSuccess;
}

}  // namespace

// Tensor-pipe peak for the GF(2) GEMM engine: the measured rate of its own
// tcgen05.mma (kind::f8f6f4, E4M3, M = 128, N = 256, K = 32) with the operands
// resident in shared memory, in multiply-accumulates per second.
extern "C" int gmc_tc_f8_peak(double *mac_per_s) {
  if (!mac_per_s) {
    set_last_error("gmc_tc_f8_peak: null output");
    return GMC_EINVAL;
  }
  int *err = nullptr;
  cudaStream_t st = nullptr;
  cudaError_t e = cudaMalloc(&err, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(err, 0, sizeof(int));
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = time_tc_f8_peak(mac_per_s, err, st);
  int h = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&h, err, sizeof(int), cudaMemcpyDeviceToHost);
  if (st) cudaStreamDestroy(st);
  if (err) cudaFree(err);
  if (e != cudaSuccess) {
    set_last_error((std::string("gmc_tc_f8_peak: ") + cudaGetErrorString(e)).c_str());
    return GMC_ECUDA;
  }
  if (h) {
    set_last_error("gmc_tc_f8_peak: a bounded wait expired");
    return GMC_ECUDA;
  }
  return GMC_OK;
}

// The legacy 1-bit tensor path's rate: mma.sync m8n8k128 .b1 AND.POPC with
// register operands, in bit multiply-accumulates per second.
extern "C" int gmc_b1mma_peak(double *mac_per_s) {
  if (!mac_per_s) {
    set_last_error("gmc_b1mma_peak: null output");
    return GMC_EINVAL;
  }
  int *out = nullptr;
  cudaStream_t st = nullptr;
  cudaError_t e = cudaMalloc(&out, sizeof(int));
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = time_b1_peak(mac_per_s, out, st);
  if (st) cudaStreamDestroy(st);
  if (out) cudaFree(out);
  if (e != cudaSuccess) {
    set_last_error((std::string("gmc_b1mma_peak: ") + cudaGetErrorString(e)).c_str());
    return GMC_ECUDA;
  }
  return GMC_OK;
}

extern "C" int gmc_int32_peak(double *lop3_per_s, double *shf_per_s) {
  if (!lop3_per_s || !shf_per_s) {
    set_last_error("gmc_int32_peak: null output");
    return GMC_EINVAL;
  }
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  uint32_t *out = nullptr;
  cudaStream_t st = nullptr;
  if (e == cudaSuccess) e = cudaMalloc(&out, sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  const int blocks = sms * 8, iters = 2048;  // ~1.3e10 lane-ops per launch
  if (e == cudaSuccess) e = time_kernel<false>(blocks, iters, out, st, lop3_per_s);
  if (e == cudaSuccess) e = time_kernel<true>(blocks, iters, out, st, shf_per_s);
  if (st) cudaStreamDestroy(st);
  if (out) cudaFree(out);
  if (e != cudaSuccess) {
    set_last_error((std::string("gmc_int32_peak: ") + cudaGetErrorString(e)).c_str());
    return GMC_ECUDA;
  }
  return GMC_OK;
}
