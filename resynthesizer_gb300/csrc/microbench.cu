// microbench.cu -- peaks of the two on-chip resources that bound the
// synthesis kernels, measured on the GPU at hand: shared-memory load
// bandwidth and 32-bit integer ALU throughput.  bench.py divides the wave
// kernel's algorithmic bytes and integer ops by these (its roofline), since
// the corpus and the metric tables live in shared memory and DRAM is not what
// binds those kernels.  No counterpart in the reference.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/resynthesizer.h"

#define RS_EXPORT extern "C" __attribute__((visibility("default")))

extern "C" int rs_fail(int code, const char* msg);

namespace {

constexpr int kSmemWords4 = 2048;   // 32 KB of uint4 per CTA (a power of two: the index wraps with a mask)
constexpr int kUnroll = 8;

// Every warp reads 32 consecutive 16-byte words per load (512 B, no bank
// conflicts); the address moves with the iteration so no load can be hoisted.
__global__ void __launch_bounds__(512) k_smem_read(unsigned* sink, int iters) {
  __shared__ uint4 buf[kSmemWords4];
  for (int i = threadIdx.x; i < kSmemWords4; i += blockDim.x)
    buf[i] = make_uint4(i, i * 3u + 1u, i * 5u + 2u, i * 7u + 3u);
  __syncthreads();
  uint4 acc = make_uint4(0, 0, 0, 0);
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  for (int it = 0; it < iters; it++) {
    const unsigned base = (unsigned)it * (kUnroll * 32u) + warp * 32u + lane;
#pragma unroll
    for (int k = 0; k < kUnroll; k++) {
      const uint4 v = buf[(base + k * 32u) & (kSmemWords4 - 1)];
      acc.x ^= v.x;
      acc.y += v.y;
      acc.z ^= v.z;
      acc.w += v.w;
    }
  }
  if ((acc.x ^ acc.y ^ acc.z ^ acc.w) == 0x9E3779B9u) sink[blockIdx.x] = acc.x;
}

// Eight independent chains of x = (x + b) ^ c: two dependent 32-bit ALU ops
// per step that no compiler can fold into fewer instructions.
__global__ void __launch_bounds__(512) k_int_alu(unsigned* sink, int iters, unsigned seed) {
  unsigned a[8];
#pragma unroll
  for (int j = 0; j < 8; j++) a[j] = (threadIdx.x + blockIdx.x * 977u) * (2u * j + 1u) ^ seed;
  const unsigned b = seed * 0x9E3779B9u + threadIdx.x, c = seed ^ 0x85EBCA6Bu ^ blockIdx.x;
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int k = 0; k < 16; k++) {
#pragma unroll
      for (int j = 0; j < 8; j++) a[j] = (a[j] + b) ^ c;
    }
  }
  unsigned x = 0;
#pragma unroll
  for (int j = 0; j < 8; j++) x ^= a[j];
  if (x == 0x12345678u) sink[blockIdx.x] = x;
}

int sms() {
  int dev = 0, n = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  return n > 0 ? n : 1;
}

}  // namespace

// No counterpart in the reference.  Declared in include/resynthesizer.h.
RS_EXPORT int resynthMicrobench(int which, double* value, double* ms) {
  if (!value || (which != 0 && which != 1)) return rs_fail(RESYNTH_ERROR_ARGUMENT, "resynthMicrobench: bad argument");
  const int grid = sms() * 4, threads = 512;
  const int iters = which == 0 ? 2048 : 4096;
  unsigned* sink = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaMalloc(&sink, grid * sizeof(unsigned));
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 8 && e == cudaSuccess; rep++) {
    cudaEventRecord(e0);
    if (which == 0)
      k_smem_read<<<grid, threads>>>(sink, iters);
    else
      k_int_alu<<<grid, threads>>>(sink, iters, 0x2545F491u + rep);
    cudaEventRecord(e1);
    e = cudaEventSynchronize(e1);
    float t = 0;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
    if (rep >= 3 && t < best) best = t;   // three warm-up launches, then the best of five
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  if (sink) cudaFree(sink);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (e != cudaSuccess) return rs_fail(RESYNTH_ERROR_DEVICE, cudaGetErrorString(e));
  const double threadsTotal = (double)grid * threads;
  if (which == 0)
    *value = threadsTotal * iters * kUnroll * 16.0 / (best * 1e-3) / 1e9;   // GB/s
  else
    *value = threadsTotal * iters * 16.0 * 8.0 * 2.0 / (best * 1e-3) / 1e9;   // Gop/s
  if (ms) *ms = best;
  return 0;
}
