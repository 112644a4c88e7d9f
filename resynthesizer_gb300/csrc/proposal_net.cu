// proposal_net.cu -- the learned proposal network on the tensor cores.
//
// This part has no counterpart in the reference: it proposes candidate
// sources for the synthesis search (the reference draws them uniformly at
// random, lib/synthesize.h:583-603).  Every proposal is scored by the exact
// integer patch metric, so the plain search stays both fallback and judge.
//
// This file holds the tensor-core GEMM launcher (tc_gemm.cuh) and a test
// entry that multiplies host matrices with it.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/resynthesizer.h"
#include "synth_internal.h"
#include "tc_gemm.cuh"

#define RS_EXPORT extern "C" __attribute__((visibility("default")))

extern "C" int rs_fail(int code, const char* msg);

namespace rs {
namespace tc {

// Round to nearest even bf16 (finite inputs).
uint16_t f2bf(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  u += 0x7FFFu + ((u >> 16) & 1u);
  return (uint16_t)(u >> 16);
}

float bf2f(uint16_t h) {
  const uint32_t u = (uint32_t)h << 16;
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}

// Largest shared-memory byte the CTA's descriptors can reach for chunk size K
// and tile N, were the two byte offsets exchanged.  Allocating this much keeps
// every tensor-core read inside the CTA's own allocation whatever the layout.
static size_t guarded_smem(int NT, int K) {
  const size_t lboA = (kTileM / 8) * 128, lboB = (size_t)(NT / 8) * 128;
  const size_t steps = (size_t)K / 16;
  const size_t aExt = lboA * (2 * steps - 2 + kTileM / 8) + 256;
  const size_t bExt = (size_t)kTileM * K * 2 + lboB * (2 * steps - 2 + NT / 8) + 256;
  return std::max(gemm_smem_bytes(NT, K), std::max(aExt, bExt));
}

template <int NT>
static cudaError_t launch_gemm_t(const GemmArgs& g, int tilesM, int tilesN, int chunks, cudaStream_t s) {
  static std::mutex mu;
  static int configured[4] = {-1, -1, -1, -1};
  const size_t smem = guarded_smem(NT, g.K);
  int dev = 0;
  cudaGetDevice(&dev);
  {
    std::lock_guard<std::mutex> lk(mu);
    if (dev < 4 && configured[dev] < (int)smem) {
      cudaError_t e = cudaFuncSetAttribute(k_gemm<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      configured[dev] = (int)smem;
    }
  }
  k_gemm<NT><<<dim3(tilesM, tilesN, chunks), 128, smem, s>>>(g);
  return cudaGetLastError();
}

// D = A . B^T over `chunks` K chunks; NT is 32 or 96.
cudaError_t launch_gemm(int NT, const GemmArgs& g, int tilesM, int tilesN, int chunks, cudaStream_t s) {
  if (g.K % 16 || g.K < 16 || g.K > kMaxK) return cudaErrorInvalidValue;
  if (NT == 32) return launch_gemm_t<32>(g, tilesM, tilesN, chunks, s);
  if (NT == 96) return launch_gemm_t<96>(g, tilesM, tilesN, chunks, s);
  return cudaErrorInvalidValue;
}

// Host packing of a row-major fp32 matrix [R x K] into blocked bf16 tiles of
// Rt rows and Kc columns, tile (t, c) at ((c * nTiles) + t) * Rt * Kc.
static void pack_blocked(const float* src, int R, int K, int Rt, int Kc, int nTiles, int nChunks,
                         std::vector<uint16_t>& out) {
  out.assign((size_t)nTiles * nChunks * Rt * Kc, 0);
  for (int r = 0; r < R; r++)
    for (int k = 0; k < K; k++) {
      const int t = r / Rt, c = k / Kc;
      out[((size_t)c * nTiles + t) * Rt * Kc + blocked_offset(r % Rt, k % Kc, Rt)] = f2bf(src[(size_t)r * K + k]);
    }
}

}  // namespace tc
}  // namespace rs

using namespace rs::tc;

// Test entry: D[M x N] = bf16(A)[M x K] . bf16(B)[N x K]^T with fp32
// accumulation on the tensor cores; host row-major buffers.  K is split into
// chunks of at most 256 that accumulate atomically when there is more than one.
RS_EXPORT int resynthTcGemm(const float* A, const float* B, int M, int N, int K, float* D) {
  if (!A || !B || !D || M <= 0 || N <= 0 || K <= 0 || N % 32) return rs_fail(RESYNTH_ERROR_ARGUMENT, "tc gemm: bad shape");
  const int NT = N % 96 == 0 ? 96 : 32;
  const int K16 = (K + 15) / 16 * 16;
  const int Kc = K16 <= 256 ? K16 : 256;
  const int chunks = (K16 + Kc - 1) / Kc;
  const int tilesM = (M + kTileM - 1) / kTileM, tilesN = N / NT;
  std::vector<uint16_t> hA, hB;
  pack_blocked(A, M, K, kTileM, Kc, tilesM, chunks, hA);
  pack_blocked(B, N, K, NT, Kc, tilesN, chunks, hB);
  uint16_t *dA = nullptr, *dB = nullptr;
  float* dD = nullptr;
  unsigned* dErr = nullptr;
  auto cleanup = [&]() {
    cudaFree(dA);
    cudaFree(dB);
    cudaFree(dD);
    cudaFree(dErr);
  };
  cudaError_t e = cudaMalloc(&dA, hA.size() * 2);
  if (e == cudaSuccess) e = cudaMalloc(&dB, hB.size() * 2);
  if (e == cudaSuccess) e = cudaMalloc(&dD, (size_t)M * N * 4);
  if (e == cudaSuccess) e = cudaMalloc(&dErr, 4);
  if (e == cudaSuccess) e = cudaMemcpy(dA, hA.data(), hA.size() * 2, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dB, hB.data(), hB.size() * 2, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(dD, 0, (size_t)M * N * 4);
  if (e == cudaSuccess) e = cudaMemset(dErr, 0, 4);
  if (e == cudaSuccess) {
    GemmArgs g{};
    g.A = dA;
    g.B = dB;
    g.aTile = (long long)kTileM * Kc;
    g.aChunk = (long long)tilesM * kTileM * Kc;
    g.bTile = (long long)NT * Kc;
    g.bChunk = (long long)tilesN * NT * Kc;
    g.M = M;
    g.N = N;
    g.K = Kc;
    g.accumulate = chunks > 1;
    g.outF = dD;
    g.ldo = N;
    g.err = dErr;
    e = launch_gemm(NT, g, tilesM, tilesN, chunks, 0);
  }
  unsigned herr = 0;
  if (e == cudaSuccess) e = cudaMemcpy(D, dD, (size_t)M * N * 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(&herr, dErr, 4, cudaMemcpyDeviceToHost);
  cleanup();
  if (e != cudaSuccess) return rs_fail(RESYNTH_ERROR_DEVICE, cudaGetErrorString(e));
  if (herr) return rs_fail(RESYNTH_ERROR_DEVICE, "tc gemm: a tensor-core wait ran out");
  return 0;
}
