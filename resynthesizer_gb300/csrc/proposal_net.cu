// proposal_net.cu -- the learned proposal network on the tensor cores.
//
// This part has no counterpart in the reference: it proposes candidate
// sources for the synthesis search, whose only other candidates are the
// neighbours' continuations and uniform random draws (lib/synthesize.h:
// 536-604).  Every proposal is scored by the exact integer patch metric, so
// the plain search stays both the fallback and the arbiter.
//
// Network: an 11 x 11 x 16 context (colour, has-value, map) around a target
// pixel; four 3x3 convolutions of 32 channels with ReLU (11 -> 9 -> 7 -> 5 ->
// 3) and a 3x3 convolution head to 16 (dx, dy) offsets in units of 64 px.
// BF16 operands, fp32 accumulation on the tcgen05 tensor cores.
//
// Two forward implementations share the weights:
//   k_net_infer  -- fused, persistent: a CTA takes 12 contexts at a time and
//                   runs all five layers out of shared memory as implicit
//                   GEMMs (each 3x3 tap is a row-shifted view of the
//                   activation slabs), TMEM accumulators, proposals written
//                   straight for the synthesis kernel;
//   training     -- explicit im2col into blocked tiles + k_gemm per layer,
//                   keeping every activation for the backward pass, which is
//                   also k_gemm (dW = col^T dY, dcol = dY W) plus col2im.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
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

template <int NT>
static cudaError_t launch_gemm_t(const GemmArgs& g, int tilesM, int tilesN, int chunks, cudaStream_t s) {
  static std::mutex mu;
  static int configured[8] = {-1, -1, -1, -1, -1, -1, -1, -1};
  const size_t smem = gemm_smem_bytes(NT, g.K);
  int dev = 0;
  cudaGetDevice(&dev);
  {
    std::lock_guard<std::mutex> lk(mu);
    if (dev >= 8 || configured[dev] < (int)smem) {
      cudaError_t e = cudaFuncSetAttribute(k_gemm<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      if (dev < 8) configured[dev] = (int)smem;
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

namespace net {

using tc::blocked_offset;

constexpr int kLayers = 5, kCtx = 11, kCin0 = 16, kCout = 32, kOffsets = 16;
constexpr float kEps = 0.05f, kLabelScale = 64.f, kLabelClip = 16.f;
__host__ __device__ constexpr int cin_of(int l) { return l == 0 ? kCin0 : kCout; }
__host__ __device__ constexpr int win_of(int l) { return kCtx - 2 * l; }
__host__ __device__ constexpr int k_of(int l) { return 9 * cin_of(l); }
// flat parameter layout: per layer W [32 x K] then b [32]
__host__ __device__ constexpr int w_off(int l) { return l == 0 ? 0 : (32 * 144 + 32) + (l - 1) * (32 * 288 + 32); }
__host__ __device__ constexpr int b_off(int l) { return w_off(l) + 32 * k_of(l); }
constexpr int kParams = w_off(kLayers);
// blocked bf16 weights, B operand of the forward GEMMs: [32 x K] tiles of 32 rows
__host__ __device__ constexpr int wblk_off(int l) { return l == 0 ? 0 : 32 * 144 + (l - 1) * 32 * 288; }
constexpr int kWblk = wblk_off(kLayers);
// blocked bf16 transposed weights, B operand of dcol: [288 x 32] in 96-row tiles, layers 1..4
__host__ __device__ constexpr int wt_off(int l) { return (l - 1) * 288 * 32; }
constexpr int kWt = 4 * 288 * 32;
constexpr int kCtxElems = kCtx * kCtx * kCin0;   // bf16 per context

// ------------------------------------------------------------- contexts

__device__ __forceinline__ uint32_t bf2(float lo, float hi) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&h);
}

// Channels 0-7 of one context pixel: colour 0-2 (grey repeated) as v/255 -
// 0.5 where the pixel has a value, has-value, map 0 as m/255 - 0.5.  Pixels
// outside the target image are zero.  Channels 8-15 are always zero.
// The pixel's words, loaded without waiting on one another.
struct CtxWords {
  uint32_t px, map;
  bool in, valued;
};

__device__ __forceinline__ CtxWords ctx_load(const Problem& pb, int qx, int qy, int visCur) {
  CtxWords w{0u, 0u, false, false};
  if ((unsigned)qx >= (unsigned)pb.tw || (unsigned)qy >= (unsigned)pb.th) return w;
  const int qi = qy * pb.tw + qx;
  w.in = true;
  w.valued = pb.vis ? __ldg(pb.vis + qi) < visCur : __ldg(pb.has + qi) != 0;
  w.px = __ldg(pb.tpx + qi);
  w.map = (pb.nm > 0 && pb.tmap) ? __ldg(pb.tmap + qi) : 0u;
  return w;
}

__device__ __forceinline__ uint4 ctx_encode(const Problem& pb, const CtxWords& w) {
  if (!w.in) return make_uint4(0, 0, 0, 0);
  float c0 = 0.f, c1 = 0.f, c2 = 0.f, h = 0.f, m = 0.f;
  if (w.valued) {
    const int n1 = min(1, pb.nc - 1), n2 = min(2, pb.nc - 1);
    c0 = (float)((w.px >> 8) & 0xFFu) / 255.f - 0.5f;
    c1 = (float)((w.px >> (8 + 8 * n1)) & 0xFFu) / 255.f - 0.5f;
    c2 = (float)((w.px >> (8 + 8 * n2)) & 0xFFu) / 255.f - 0.5f;
    h = 1.f;
  }
  if (pb.nm > 0 && pb.tmap) m = (float)(w.map & 0xFFu) / 255.f - 0.5f;
  return make_uint4(bf2(c0, c1), bf2(c2, h), bf2(m, 0.f), 0u);
}

__device__ __forceinline__ uint4 ctx_pixel(const Problem& pb, int qx, int qy, int visCur) {
  return ctx_encode(pb, ctx_load(pb, qx, qy, visCur));
}

// --------------------------------------------------- fused inference kernel

constexpr int kS = 12;   // contexts per CTA iteration
__host__ __device__ constexpr int in_rows(int l) { return kS * win_of(l) * win_of(l); }
__host__ __device__ constexpr int tiles_of(int l) { return (in_rows(l) + 127) / 128; }
// rows of one input slab: every tile's rows plus the largest tap shift
__host__ __device__ constexpr int pad_of(int l) { return (tiles_of(l) * 128 + 2 * win_of(l) + 2 + 7) / 8 * 8; }
__host__ __device__ constexpr int slab_bytes(int l) { return (cin_of(l) / 8) * pad_of(l) * 16; }
constexpr int cmax(int a, int b) { return a > b ? a : b; }
constexpr int kBuf0 = cmax(slab_bytes(0), cmax(slab_bytes(2), slab_bytes(4)));
constexpr int kBuf1 = cmax(slab_bytes(1), slab_bytes(3));
constexpr int kWBytes = kWblk * 2;
constexpr int kBiasBytes = kLayers * 32 * 4;
constexpr int kInferSmem = kWBytes + kBiasBytes + kBuf0 + kBuf1;
constexpr int kTmemCols = 512;
static_assert(tiles_of(0) * 32 <= kTmemCols, "TMEM columns");
static_assert(kInferSmem + 64 <= 232448, "shared memory");

struct InferArgs {
  const uint16_t* wblk;
  const float* params;
  const uint16_t* x0;      // contexts [n x 121 x 16] (test path) or null
  int n;
  Problem pb;              // synthesis path: contexts built from the live state
  const int2* targets;
  const int* batchStart;
  int batch0, batch1;      // targets [batchStart[batch0], batchStart[batch1])
  int visCur;
  float* out;              // [n x 32] or null
  int2* props;             // [n x 16] proposed sources, or null
  unsigned* err;           // bit 3: a wait ran out
};

// One layer of the fused forward for the kS contexts of a group: one thread
// issues the layer's MMAs (tiles x 9 taps x K steps, descriptors advanced by
// plain adds: the start-address field is byte address / 16), all threads
// read their TMEM lane and write bias + ReLU (bf16) into the next layer's
// slabs, or decode the head.  False when the MMA wait ran out.
template <int L, bool FROM_PROBLEM>
__device__ __forceinline__ bool infer_layer(const InferArgs& a, unsigned char* in, unsigned char* outb,
                                            const uint16_t* sW, const float* sBias, uint32_t tmem,
                                            uint64_t* barMma, uint32_t& phase, int g, int sv, int n0) {
  constexpr int win = win_of(L), wout = win - 2, cin = cin_of(L), kst = cin / 16, tiles = tiles_of(L);
  constexpr int inPad = pad_of(L);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    constexpr uint32_t idesc = tc::instr_desc(128, 32);
    const uint64_t aBase = tc::smem_desc(tc::saddr(in), inPad * 16, 128);
    const uint64_t bBase = tc::smem_desc(tc::saddr(sW + wblk_off(L)), 512, 128);
#pragma unroll 1
    for (int t = 0; t < tiles; t++) {
#pragma unroll
      for (int tap = 0; tap < 9; tap++) {
        const int shift = (tap / 3) * win + tap % 3;
#pragma unroll
        for (int ks = 0; ks < kst; ks++) {
          const uint64_t da = aBase + (uint64_t)(2 * ks * inPad + t * 128 + shift);
          const uint64_t db = bBase + (uint64_t)(((tap * cin + 16 * ks) / 8) * 32);
          tc::mma_bf16(tmem + t * 32, da, db, idesc, (tap | ks) ? 1u : 0u);
        }
      }
    }
    tc::mma_commit(barMma);
  }
  bool done = tc::mbar_wait(barMma, phase, 1 << 20);
  phase ^= 1u;
  done = __syncthreads_and(done) != 0;
  if (!done) return false;
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll 1
  for (int t = 0; t < tiles; t++) {
    uint32_t v[32];
    tc::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(t * 32), v);
    const int r = t * 128 + warp * 32 + lane;
    const int b = r / (win * win), yx = r - b * win * win, y = yx / win, x = yx - y * win;
    if (b >= sv || y >= wout || x >= wout) continue;
    if (L < kLayers - 1) {
      constexpr int outPad = L < kLayers - 1 ? pad_of(L + 1) : 0;
      const int ro = (b * wout + y) * wout + x;
      const float* bias = sBias + L * 32;
#pragma unroll
      for (int q = 0; q < 4; q++) {
        uint32_t w[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const int c = q * 8 + 2 * j;
          w[j] = bf2(fmaxf(__uint_as_float(v[c]) + bias[c], 0.f), fmaxf(__uint_as_float(v[c + 1]) + bias[c + 1], 0.f));
        }
        *reinterpret_cast<uint4*>(outb + q * outPad * 16 + ro * 16) = make_uint4(w[0], w[1], w[2], w[3]);
      }
    } else {
      const int s = g + b;
      const float* bias = sBias + 4 * 32;
      if (a.out) {
#pragma unroll
        for (int j = 0; j < 32; j++) a.out[(size_t)s * 32 + j] = __uint_as_float(v[j]) + bias[j];
      }
      if (a.props) {
        const int2 pos = FROM_PROBLEM ? a.targets[n0 + s] : make_int2(0, 0);
#pragma unroll
        for (int k = 0; k < kOffsets; k++) {
          const float dx = (__uint_as_float(v[2 * k]) + bias[2 * k]) * kLabelScale;
          const float dy = (__uint_as_float(v[2 * k + 1]) + bias[2 * k + 1]) * kLabelScale;
          a.props[(size_t)s * kOffsets + k] = make_int2(pos.x + (int)fmaxf(fminf(rintf(dx), 1e8f), -1e8f),
                                                        pos.y + (int)fmaxf(fminf(rintf(dy), 1e8f), -1e8f));
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  __syncthreads();
  return true;
}

// Activation slab layout: for each 8-channel block q, `pad` rows of 16 bytes;
// row = (sample, y, x) on the layer's own grid.  Row-major in one block makes
// a 3x3 tap a uniform row shift (ky * width + kx) of a 128-row window, so a
// tcgen05 descriptor at the shifted row is the tap's im2col tile.
template <bool FROM_PROBLEM>
__global__ void __launch_bounds__(128, 1) k_net_infer(InferArgs a) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ __align__(8) uint64_t barW, barMma;
  __shared__ uint32_t tmemBase;
  const int n0 = FROM_PROBLEM ? a.batchStart[a.batch0] : 0;
  const int count = FROM_PROBLEM ? a.batchStart[a.batch1] - n0 : a.n;
  if ((int)blockIdx.x * kS >= count) return;
  uint16_t* sW = reinterpret_cast<uint16_t*>(sm);
  float* sBias = reinterpret_cast<float*>(sm + kWBytes);
  unsigned char* buf0 = sm + kWBytes + kBiasBytes;
  unsigned char* buf1 = buf0 + kBuf0;
  const int tid = threadIdx.x, warp = tid >> 5;
  if (tid == 0) {
    tc::mbar_init1(&barW);
    tc::mbar_init1(&barMma);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int i = tid; i < kLayers * 32; i += 128) sBias[i] = a.params[b_off(i / 32) + (i & 31)];
  if (warp == 0) tc::tmem_alloc<kTmemCols>(&tmemBase);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmemBase;
  if (tid == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tc::saddr(&barW)), "r"(kWBytes)
                 : "memory");
    for (int l = 0; l < kLayers; l++)
      tc::bulk_g2s(sW + wblk_off(l), a.wblk + wblk_off(l), 32u * k_of(l) * 2u, &barW);
  }
  bool ok = tc::mbar_wait(&barW, 0, 1 << 20);
  ok = __syncthreads_and(ok) != 0;
  if (!ok && tid == 0) atomicOr(a.err, 8u);
  uint32_t phase = 0;
  for (int g = blockIdx.x * kS; ok && g < count; g += gridDim.x * kS) {
    const int sv = min(kS, count - g);
    // layer-0 input: contexts of samples g .. g + sv.  Channels 8-15 (slab
    // 1) are zero for contexts built here.  Rows go four at a time so that
    // their loads are in flight together.
    constexpr int kRows = kS * 121, kUnroll = 4;
#pragma unroll 1
    for (int base = 0; base < kRows; base += 128 * kUnroll) {
      if (FROM_PROBLEM) {
        CtxWords w[kUnroll];
#pragma unroll
        for (int u = 0; u < kUnroll; u++) {
          const int r = base + u * 128 + tid, b = r / 121, yx = r - b * 121;
          w[u] = CtxWords{0u, 0u, false, false};
          if (r < kRows && b < sv) {
            const int2 pos = a.targets[n0 + g + b];
            const int y = yx / 11, x = yx - y * 11;
            w[u] = ctx_load(a.pb, pos.x + x - 5, pos.y + y - 5, a.visCur);
          }
        }
#pragma unroll
        for (int u = 0; u < kUnroll; u++) {
          const int r = base + u * 128 + tid;
          if (r < kRows) {
            *reinterpret_cast<uint4*>(buf0 + r * 16) = ctx_encode(a.pb, w[u]);
            *reinterpret_cast<uint4*>(buf0 + pad_of(0) * 16 + r * 16) = make_uint4(0, 0, 0, 0);
          }
        }
      } else {
#pragma unroll
        for (int u = 0; u < kUnroll; u++) {
          const int r = base + u * 128 + tid, b = r / 121, yx = r - b * 121;
          if (r >= kRows) continue;
          uint4 lo = make_uint4(0, 0, 0, 0), hi = make_uint4(0, 0, 0, 0);
          if (b < sv) {
            const uint4* src = reinterpret_cast<const uint4*>(a.x0 + ((size_t)(g + b) * 121 + yx) * 16);
            lo = src[0];
            hi = src[1];
          }
          *reinterpret_cast<uint4*>(buf0 + r * 16) = lo;
          *reinterpret_cast<uint4*>(buf0 + pad_of(0) * 16 + r * 16) = hi;
        }
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    ok = infer_layer<0, FROM_PROBLEM>(a, buf0, buf1, sW, sBias, tmem, &barMma, phase, g, sv, n0) &&
         infer_layer<1, FROM_PROBLEM>(a, buf1, buf0, sW, sBias, tmem, &barMma, phase, g, sv, n0) &&
         infer_layer<2, FROM_PROBLEM>(a, buf0, buf1, sW, sBias, tmem, &barMma, phase, g, sv, n0) &&
         infer_layer<3, FROM_PROBLEM>(a, buf1, buf0, sW, sBias, tmem, &barMma, phase, g, sv, n0) &&
         infer_layer<4, FROM_PROBLEM>(a, buf0, buf1, sW, sBias, tmem, &barMma, phase, g, sv, n0);
    if (!ok && tid == 0) atomicOr(a.err, 8u);
  }
  // A failed weight wait may leave the copies in flight: wait once more.
  if (!ok) tc::mbar_wait(&barW, 0, 1 << 20);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) tc::tmem_free<kTmemCols>(tmem);
}

static int g_smCount[8];

template <bool FP>
static cudaError_t launch_infer(const InferArgs& a, int count, cudaStream_t s) {
  static std::mutex mu;
  static bool configured[8];
  int dev = 0;
  cudaGetDevice(&dev);
  {
    std::lock_guard<std::mutex> lk(mu);
    if (dev >= 8 || !configured[dev]) {
      cudaError_t e = cudaFuncSetAttribute(k_net_infer<FP>, cudaFuncAttributeMaxDynamicSharedMemorySize, kInferSmem);
      if (e != cudaSuccess) return e;
      if (dev < 8) {
        configured[dev] = true;
        cudaDeviceGetAttribute(&g_smCount[dev], cudaDevAttrMultiProcessorCount, dev);
      }
    }
  }
  const int sms = dev < 8 && g_smCount[dev] > 0 ? g_smCount[dev] : 148;
  const int grid = std::max(1, std::min(sms, (count + kS - 1) / kS));
  k_net_infer<FP><<<grid, 128, kInferSmem, s>>>(a);
  return cudaGetLastError();
}

// ------------------------------------------------------- training kernels

__global__ void k_im2col(const uint16_t* __restrict__ act, int n, int l, uint16_t* __restrict__ col) {
  const int cin = cin_of(l), win = win_of(l), wo = win - 2, K = k_of(l), kg = K / 8;
  const int rows = n * wo * wo, rowsPad = (rows + 127) / 128 * 128;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < (long long)rowsPad * kg;
       idx += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(idx / kg), q = (int)(idx - (long long)r * kg);
    const int k0 = q * 8, tap = k0 / cin, c0 = k0 - tap * cin;
    uint4 v = make_uint4(0, 0, 0, 0);
    if (r < rows) {
      const int b = r / (wo * wo), yx = r - b * wo * wo, oy = yx / wo, ox = yx - oy * wo;
      const int y = oy + tap / 3, x = ox + tap % 3;
      v = *reinterpret_cast<const uint4*>(act + (((size_t)b * win + y) * win + x) * cin + c0);
    }
    *reinterpret_cast<uint4*>(col + (size_t)(r / 128) * 128 * K + blocked_offset(r % 128, k0, 128)) = v;
  }
}

// Transposed im2col for dW: rows = the K features (tiles of 128), columns =
// sample rows in chunks of 256; tile (t, c) at (c * nFT + t) * 128 * 256.
__global__ void k_im2col_t(const uint16_t* __restrict__ act, int n, int l, int nFT, int chunks,
                           uint16_t* __restrict__ colT) {
  const int cin = cin_of(l), win = win_of(l), wo = win - 2, K = k_of(l);
  const int rows = n * wo * wo, mg = chunks * 32;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < (long long)nFT * 128 * mg;
       idx += (long long)gridDim.x * blockDim.x) {
    const int f = (int)(idx / mg), m0 = (int)(idx - (long long)f * mg) * 8;
    uint16_t v[8];
    const int tap = f / cin, c = f - tap * cin, ky = tap / 3, kx = tap % 3;
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const int m = m0 + j;
      v[j] = 0;
      if (f < K && m < rows) {
        const int b = m / (wo * wo), yx = m - b * wo * wo, oy = yx / wo, ox = yx - oy * wo;
        v[j] = act[(((size_t)b * win + oy + ky) * win + ox + kx) * cin + c];
      }
    }
    uint4 w;
    w.x = v[0] | (uint32_t)v[1] << 16;
    w.y = v[2] | (uint32_t)v[3] << 16;
    w.z = v[4] | (uint32_t)v[5] << 16;
    w.w = v[6] | (uint32_t)v[7] << 16;
    const int ch = m0 / 256, t = f / 128;
    *reinterpret_cast<uint4*>(colT + ((size_t)ch * nFT + t) * 128 * 256 + blocked_offset(f % 128, m0 % 256, 128)) = w;
  }
}

// Relaxed multiple-choice loss: dY = d loss / d out, loss summed into *loss.
__global__ void k_mcl(const float* __restrict__ out, const float* __restrict__ labels, int n, float* __restrict__ dy,
                      float* loss) {
  __shared__ float red[8];
  float part = 0.f;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n) {
    const float ly = fminf(fmaxf(labels[2 * s], -kLabelClip), kLabelClip);
    const float ly1 = fminf(fmaxf(labels[2 * s + 1], -kLabelClip), kLabelClip);
    float d[kOffsets];
    int win = 0;
#pragma unroll
    for (int k = 0; k < kOffsets; k++) {
      const float ex = out[(size_t)s * 32 + 2 * k] - ly, ey = out[(size_t)s * 32 + 2 * k + 1] - ly1;
      d[k] = ex * ex + ey * ey;
      if (d[k] < d[win]) win = k;
    }
    const float wo = kEps / (kOffsets - 1), scale = 2.f / (float)n;
#pragma unroll
    for (int k = 0; k < kOffsets; k++) {
      const float w = k == win ? 1.f - kEps : wo;
      part += w * d[k];
      dy[(size_t)s * 32 + 2 * k] = scale * w * (out[(size_t)s * 32 + 2 * k] - ly);
      dy[(size_t)s * 32 + 2 * k + 1] = scale * w * (out[(size_t)s * 32 + 2 * k + 1] - ly1);
    }
    part /= (float)n;
  }
  for (int o = 16; o; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = part;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
    atomicAdd(loss, t);
  }
}

// dY (fp32 [rows x 32]) -> bf16 blocked A operand [rows x 32] (128-row tiles).
__global__ void k_gpack(const float* __restrict__ dy, int rows, uint16_t* __restrict__ g) {
  const int rowsPad = (rows + 127) / 128 * 128;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < rowsPad * 4; idx += gridDim.x * blockDim.x) {
    const int r = idx >> 2, q = idx & 3;
    uint4 w = make_uint4(0, 0, 0, 0);
    if (r < rows) {
      const float* p = dy + (size_t)r * 32 + q * 8;
      w = make_uint4(bf2(p[0], p[1]), bf2(p[2], p[3]), bf2(p[4], p[5]), bf2(p[6], p[7]));
    }
    *reinterpret_cast<uint4*>(g + (size_t)(r / 128) * 128 * 32 + blocked_offset(r % 128, q * 8, 128)) = w;
  }
}

// dY -> bf16 blocked B operand of dW: [32 x rows], chunks of 256 rows.
__global__ void k_gpack_t(const float* __restrict__ dy, int rows, int chunks, uint16_t* __restrict__ gT) {
  const int mg = chunks * 32;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < 32 * mg; idx += gridDim.x * blockDim.x) {
    const int o = idx / mg, m0 = (idx - o * mg) * 8;
    float v[8];
#pragma unroll
    for (int j = 0; j < 8; j++) v[j] = m0 + j < rows ? dy[(size_t)(m0 + j) * 32 + o] : 0.f;
    const uint4 w = make_uint4(bf2(v[0], v[1]), bf2(v[2], v[3]), bf2(v[4], v[5]), bf2(v[6], v[7]));
    *reinterpret_cast<uint4*>(gT + (size_t)(m0 / 256) * 32 * 256 + blocked_offset(o, m0 % 256, 32)) = w;
  }
}

// Per-block column sums of dY (part[block][32]); k_sum_parts adds the
// blocks in order, so the bias gradient does not depend on block timing.
__global__ void k_bias_grad(const float* __restrict__ dy, int rows, float* __restrict__ part) {
  __shared__ float red[8][32];
  const int c = threadIdx.x & 31, rl = threadIdx.x >> 5;
  float acc = 0.f;
  for (int r = blockIdx.x * 8 + rl; r < rows; r += gridDim.x * 8) acc += dy[(size_t)r * 32 + c];
  red[rl][c] = acc;
  __syncthreads();
  if (rl == 0) {
    float t = 0.f;
    for (int i = 0; i < 8; i++) t += red[i][c];
    part[(size_t)blockIdx.x * 32 + c] = t;
  }
}

// out[i] = sum over z = 0 .. parts-1 of part[z * stride + i], in that order.
__global__ void k_sum_parts(const float* __restrict__ part, int parts, long long stride, int n,
                            float* __restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float t = 0.f;
    for (int z = 0; z < parts; z++) t += part[z * stride + i];
    out[i] = t;
  }
}

// dX of layer l's input = col2im(dcol), masked by ReLU of that input.
__global__ void k_col2im(const float* __restrict__ dcol, int n, int l, const uint16_t* __restrict__ actIn,
                         float* __restrict__ dx) {
  const int win = win_of(l), wo = win - 2, K = k_of(l);
  const long long total = (long long)n * win * win * 32;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(idx & 31);
    const long long p = idx >> 5;
    const int b = (int)(p / (win * win)), yx = (int)(p - (long long)b * win * win), y = yx / win, x = yx - y * win;
    float s = 0.f;
    for (int ky = 0; ky < 3; ky++) {
      const int oy = y - ky;
      if (oy < 0 || oy >= wo) continue;
      for (int kx = 0; kx < 3; kx++) {
        const int ox = x - kx;
        if (ox < 0 || ox >= wo) continue;
        s += dcol[((size_t)(b * wo + oy) * wo + ox) * K + (ky * 3 + kx) * 32 + c];
      }
    }
    dx[idx] = actIn[idx] != 0 && !(actIn[idx] & 0x8000u) ? s : 0.f;
  }
}

// grad[W_l[o][k]] = dWT_l[k][o], summed over the K chunks' partial products
// (chunk z at dwt + z * stride) in chunk order: the gradient is the same
// every run.
__global__ void k_gather_wgrad(const float* __restrict__ dwt, int chunks, long long stride, int l,
                               float* __restrict__ grad) {
  const int K = k_of(l);
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < 32 * K; idx += gridDim.x * blockDim.x) {
    const int o = idx / K, k = idx - o * K;
    float t = 0.f;
    for (int z = 0; z < chunks; z++) t += dwt[z * stride + (size_t)k * 32 + o];
    grad[w_off(l) + idx] = t;
  }
}

__global__ void k_adam(float* __restrict__ p, float* __restrict__ m, float* __restrict__ v,
                       const float* __restrict__ g, int n, float lr, float bc1, float bc2) {
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
  }
}

// fp32 parameters -> blocked bf16 operands of the forward and dcol GEMMs.
__global__ void k_relayout(const float* __restrict__ p, uint16_t* __restrict__ wblk, uint16_t* __restrict__ wt) {
  for (int l = 0; l < kLayers; l++) {
    const int K = k_of(l);
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < 32 * K; idx += gridDim.x * blockDim.x) {
      const int o = idx / K, k = idx - o * K;
      const uint16_t h = __bfloat16_as_ushort(__float2bfloat16_rn(p[w_off(l) + idx]));
      wblk[wblk_off(l) + blocked_offset(o, k, 32)] = h;
      if (l > 0) wt[wt_off(l) + (k / 96) * 96 * 32 + blocked_offset(k % 96, o, 96)] = h;
    }
  }
}

__device__ __forceinline__ uint32_t mix(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

// Minibatch: n pairs drawn uniformly (with replacement) from the store.
__global__ void k_gather_batch(const uint16_t* __restrict__ px0, const float* __restrict__ plab, unsigned count,
                               int n, uint32_t seed, uint16_t* __restrict__ x0, float* __restrict__ lab) {
  constexpr int kVec = kCtxElems / 8;   // uint4 per context
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < (long long)n * kVec;
       idx += (long long)gridDim.x * blockDim.x) {
    const int s = (int)(idx / kVec), j = (int)(idx - (long long)s * kVec);
    const unsigned src = (unsigned)(((unsigned long long)mix(seed ^ mix((uint32_t)s * 0x9E3779B9u)) * count) >> 32);
    reinterpret_cast<uint4*>(x0)[idx] = reinterpret_cast<const uint4*>(px0)[(size_t)src * kVec + j];
    if (j == 0) {
      lab[2 * s] = plab[2 * (size_t)src];
      lab[2 * s + 1] = plab[2 * (size_t)src + 1];
    }
  }
}

// Training pairs from a finished wavefront run: every stride-th target of the
// list; even pairs see the context as it was at the target's pass-0 visit
// (pixels stamped earlier), odd pairs the final, complete context.  Label =
// (final source - target) / 64.
__global__ void k_dump(Problem pb, const int2* __restrict__ targets, int npairs, int stride,
                       uint16_t* __restrict__ x0, float* __restrict__ lab) {
  const int lane = threadIdx.x & 31;
  for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < npairs; i += (gridDim.x * blockDim.x) >> 5) {
    const int2 pos = targets[(size_t)i * stride];
    const int pi = pos.y * pb.tw + pos.x;
    const int visCur = (i & 1) ? INT_MAX - 1 : pb.vis[pi];
    for (int r = lane; r < 121; r += 32) {
      const int y = r / 11, x = r - y * 11;
      uint4* d = reinterpret_cast<uint4*>(x0 + ((size_t)i * 121 + r) * 16);
      d[0] = ctx_pixel(pb, pos.x + x - 5, pos.y + y - 5, visCur);
      d[1] = make_uint4(0, 0, 0, 0);
    }
    if (lane == 0) {
      const int2 s = pb.src[pi];
      lab[2 * i] = (float)(s.x - pos.x) / kLabelScale;
      lab[2 * i + 1] = (float)(s.y - pos.y) / kLabelScale;
    }
  }
}

// Blocks of the bias-gradient reduction (partial sums per block).
constexpr int kBiasBlocks = 512;

static int blocks_for(long long n, int threads, int cap = 4096) {
  return (int)std::max(1LL, std::min<long long>((n + threads - 1) / threads, cap));
}

}  // namespace net
}  // namespace rs

// ----------------------------------------------------------- host objects

using namespace rs;
using namespace rs::net;

struct TResynthPairs {
  int dev = 0;
  unsigned cap = 0, count = 0;
  uint16_t* x0 = nullptr;
  float* labels = nullptr;
  std::mutex mu;
};

struct TResynthNet {
  int dev = 0;
  float* params = nullptr;   // fp32 master parameters
  float* adamM = nullptr;
  float* adamV = nullptr;
  float* grad = nullptr;
  uint16_t* wblk = nullptr;
  uint16_t* wt = nullptr;
  unsigned* err = nullptr;
  float* loss = nullptr;     // per training step
  long long step = 0;
  // training work buffers for `cap` samples
  int cap = 0;
  uint16_t* x0 = nullptr;
  float* labels = nullptr;
  uint16_t* col[kLayers] = {};
  uint16_t* colT[kLayers] = {};
  uint16_t* act[kLayers - 1] = {};
  float* out = nullptr;
  float* dy[2] = {};
  uint16_t* g = nullptr;
  uint16_t* gT = nullptr;
  float* dcol = nullptr;
  float* dwt[kLayers] = {};    // per K chunk: partial dW^T of layer l
  float* biasPart = nullptr;   // per block: partial bias gradients
  std::vector<void*> work;
  cudaStream_t stream = nullptr;
  std::mutex mu;
};

namespace {

struct NetError {
  cudaError_t e;
};
#define NK(call)                                   \
  do {                                             \
    cudaError_t e_ = (call);                       \
    if (e_ != cudaSuccess) throw NetError{e_};     \
  } while (0)

int device_fail(cudaError_t e) { return rs_fail(RESYNTH_ERROR_DEVICE, cudaGetErrorString(e)); }

int rows_of(int n, int l) { return n * (win_of(l) - 2) * (win_of(l) - 2); }
int tiles_rows(int rows) { return (rows + 127) / 128; }
int chunks_rows(int rows) { return (rows + 255) / 256; }
int feat_tiles(int l) { return (k_of(l) + 127) / 128; }

void free_work(TResynthNet* net) {
  for (void* p : net->work) cudaFree(p);
  net->work.clear();
  net->cap = 0;
}

template <typename T>
T* walloc(TResynthNet* net, size_t count) {
  void* p = nullptr;
  NK(cudaMalloc(&p, count * sizeof(T)));
  net->work.push_back(p);
  return static_cast<T*>(p);
}

void ensure_work(TResynthNet* net, int n) {
  if (net->cap >= n) return;
  free_work(net);
  net->x0 = walloc<uint16_t>(net, (size_t)n * kCtxElems);
  net->labels = walloc<float>(net, (size_t)n * 2);
  size_t maxRows = 0;
  for (int l = 0; l < kLayers; l++) {
    const int rows = rows_of(n, l);
    maxRows = std::max(maxRows, (size_t)tiles_rows(rows) * 128);
    net->col[l] = walloc<uint16_t>(net, (size_t)tiles_rows(rows) * 128 * k_of(l));
    net->colT[l] = walloc<uint16_t>(net, (size_t)feat_tiles(l) * 128 * chunks_rows(rows) * 256);
    if (l < kLayers - 1) net->act[l] = walloc<uint16_t>(net, (size_t)rows * 32);
    net->dwt[l] = walloc<float>(net, (size_t)chunks_rows(rows) * feat_tiles(l) * 128 * 32);
  }
  // dY of layer l has rows_of(l) rows; dX of layer l's input has n * win^2 rows
  const size_t dyRows = std::max(maxRows, (size_t)n * 121);
  net->out = walloc<float>(net, (size_t)n * 32);
  net->dy[0] = walloc<float>(net, dyRows * 32);
  net->dy[1] = walloc<float>(net, dyRows * 32);
  net->g = walloc<uint16_t>(net, maxRows * 32);
  net->gT = walloc<uint16_t>(net, (size_t)32 * chunks_rows((int)maxRows) * 256);
  net->dcol = walloc<float>(net, maxRows * 288);
  net->biasPart = walloc<float>(net, (size_t)kBiasBlocks * 32);
  net->cap = n;
}

// Forward through the training kernels: x0 (n contexts) in net->x0.
void train_forward(TResynthNet* net, int n, cudaStream_t s) {
  const uint16_t* in = net->x0;
  for (int l = 0; l < kLayers; l++) {
    const int rows = rows_of(n, l), tiles = tiles_rows(rows), K = k_of(l);
    k_im2col<<<blocks_for((long long)tiles * 128 * (K / 8), 256), 256, 0, s>>>(in, n, l, net->col[l]);
    NK(cudaGetLastError());
    tc::GemmArgs g{};
    g.A = net->col[l];
    g.B = net->wblk + wblk_off(l);
    g.aTile = 128LL * K;
    g.M = rows;
    g.N = 32;
    g.K = K;
    g.bias = net->params + b_off(l);
    g.relu = l < kLayers - 1;
    g.outH = l < kLayers - 1 ? net->act[l] : nullptr;
    g.outF = l == kLayers - 1 ? net->out : nullptr;
    g.ldo = 32;
    g.err = net->err;
    NK(tc::launch_gemm(32, g, tiles, 1, 1, s));
    if (l < kLayers - 1) in = net->act[l];
  }
}

// Loss and gradients (into net->grad) for the n samples in net->x0 / labels.
void train_backward(TResynthNet* net, int n, float* lossSlot, cudaStream_t s) {
  NK(cudaMemsetAsync(net->grad, 0, kParams * sizeof(float), s));
  k_mcl<<<(n + 255) / 256, 256, 0, s>>>(net->out, net->labels, n, net->dy[0], lossSlot);
  NK(cudaGetLastError());
  int cur = 0;
  for (int l = kLayers - 1; l >= 0; l--) {
    const int rows = rows_of(n, l), tiles = tiles_rows(rows), chunks = chunks_rows(rows), K = k_of(l);
    const float* dy = net->dy[cur];
    k_gpack<<<blocks_for((long long)tiles * 128 * 4, 256), 256, 0, s>>>(dy, rows, net->g);
    k_gpack_t<<<blocks_for(32LL * chunks * 32, 256), 256, 0, s>>>(dy, rows, chunks, net->gT);
    const int bb = blocks_for(rows, 8, kBiasBlocks);
    k_bias_grad<<<bb, 256, 0, s>>>(dy, rows, net->biasPart);
    k_sum_parts<<<1, 32, 0, s>>>(net->biasPart, bb, 32, 32, net->grad + b_off(l));
    k_im2col_t<<<blocks_for((long long)feat_tiles(l) * 128 * chunks * 32, 256), 256, 0, s>>>(
        l == 0 ? net->x0 : net->act[l - 1], n, l, feat_tiles(l), chunks, net->colT[l]);
    NK(cudaGetLastError());
    tc::GemmArgs gw{};
    gw.A = net->colT[l];
    gw.B = net->gT;
    gw.aTile = 128LL * 256;
    gw.aChunk = (long long)feat_tiles(l) * 128 * 256;
    gw.bChunk = 32LL * 256;
    gw.M = K;
    gw.N = 32;
    gw.K = 256;
    gw.outF = net->dwt[l];
    gw.outChunk = (long long)feat_tiles(l) * 128 * 32;
    gw.ldo = 32;
    gw.err = net->err;
    NK(tc::launch_gemm(32, gw, feat_tiles(l), 1, chunks, s));
    k_gather_wgrad<<<blocks_for(32LL * K, 256), 256, 0, s>>>(net->dwt[l], chunks, gw.outChunk, l, net->grad);
    NK(cudaGetLastError());
    if (l == 0) break;
    tc::GemmArgs gd{};
    gd.A = net->g;
    gd.B = net->wt + wt_off(l);
    gd.aTile = 128LL * 32;
    gd.bTile = 96LL * 32;
    gd.M = rows;
    gd.N = K;
    gd.K = 32;
    gd.outF = net->dcol;
    gd.ldo = K;
    gd.err = net->err;
    NK(tc::launch_gemm(96, gd, tiles, K / 96, 1, s));
    const long long nx = (long long)n * win_of(l) * win_of(l) * 32;
    k_col2im<<<blocks_for(nx, 256), 256, 0, s>>>(net->dcol, n, l, net->act[l - 1], net->dy[cur ^ 1]);
    NK(cudaGetLastError());
    cur ^= 1;
  }
}

void check_err(TResynthNet* net, cudaStream_t s) {
  unsigned h = 0;
  NK(cudaMemcpyAsync(&h, net->err, 4, cudaMemcpyDeviceToHost, s));
  NK(cudaStreamSynchronize(s));
  if (h) throw NetError{cudaErrorLaunchTimeout};
}

// He-normal weights from a SplitMix64 stream (Box-Muller), zero biases.
std::vector<float> init_params(unsigned seed) {
  std::vector<float> p(kParams, 0.f);
  uint64_t st = 0x9E3779B97F4A7C15ull ^ seed;
  auto next = [&]() {
    uint64_t z = (st += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  };
  auto uni = [&]() { return ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); };
  for (int l = 0; l < kLayers; l++) {
    const double sd = std::sqrt(2.0 / k_of(l));
    for (int i = 0; i < 32 * k_of(l); i++) {
      const double u1 = uni(), u2 = uni();
      p[w_off(l) + i] = (float)(sd * std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2));
    }
  }
  return p;
}

}  // namespace

// ----------------------------------------------------------- internal API

// Proposals of the net for the targets of batches [batch0, batch1) of a
// wavefront pass (count of them known to the caller), context = pixels with
// visit stamp < visCur.  props[i * 16 + k] for the i-th target of the range.
extern "C" cudaError_t rs_net_propose(const TResynthNet* net, const Problem& pb, const int2* targets,
                                      const int* batchStart, int batch0, int batch1, int count, int visCur,
                                      int2* props, unsigned* err, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  InferArgs a{};
  a.wblk = net->wblk;
  a.params = net->params;
  a.pb = pb;
  a.targets = targets;
  a.batchStart = batchStart;
  a.batch0 = batch0;
  a.batch1 = batch1;
  a.visCur = visCur;
  a.props = props;
  a.err = err;
  return launch_infer<true>(a, count, s);
}

// Appends pairs from a finished wavefront run (vis stamps still in pb.vis).
extern "C" cudaError_t rs_net_dump(TResynthPairs* pairs, const Problem& pb, const int2* targets, int ntargets,
                                   unsigned stride, cudaStream_t s) {
  if (!pairs || !pb.vis) return cudaSuccess;
  std::lock_guard<std::mutex> lk(pairs->mu);
  stride = stride ? stride : 16u;
  const unsigned want = (unsigned)((ntargets + stride - 1) / stride);
  const unsigned room = pairs->cap - pairs->count;
  const unsigned np = std::min(want, room);
  if (!np) return cudaSuccess;
  k_dump<<<blocks_for((long long)np * 32, 256), 256, 0, s>>>(
      pb, targets, (int)np, (int)stride, pairs->x0 + (size_t)pairs->count * kCtxElems, pairs->labels + 2 * (size_t)pairs->count);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) pairs->count += np;
  return e;
}

// ------------------------------------------------------------------ C ABI

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
  cudaFree(dA);
  cudaFree(dB);
  cudaFree(dD);
  cudaFree(dErr);
  if (e != cudaSuccess) return rs_fail(RESYNTH_ERROR_DEVICE, cudaGetErrorString(e));
  if (herr) return rs_fail(RESYNTH_ERROR_DEVICE, "tc gemm: a tensor-core wait ran out");
  return 0;
}

// Test entry of the bounded waits: one GEMM tile whose load barrier expects
// 16 bytes more than its bulk copies bring, so the wait runs out (after 2^16
// polls); the kernel sets its error flag, frees its tensor memory and returns.
RS_EXPORT int resynthTcWaitTimeout(void) {
  uint16_t *dA = nullptr, *dB = nullptr;
  float* dD = nullptr;
  unsigned* dErr = nullptr;
  cudaError_t e = cudaMalloc(&dA, (size_t)kTileM * 16 * 2);
  if (e == cudaSuccess) e = cudaMalloc(&dB, (size_t)32 * 16 * 2);
  if (e == cudaSuccess) e = cudaMalloc(&dD, (size_t)kTileM * 32 * 4);
  if (e == cudaSuccess) e = cudaMalloc(&dErr, 4);
  if (e == cudaSuccess) e = cudaMemset(dA, 0, (size_t)kTileM * 16 * 2);
  if (e == cudaSuccess) e = cudaMemset(dB, 0, (size_t)32 * 16 * 2);
  if (e == cudaSuccess) e = cudaMemset(dErr, 0, 4);
  if (e == cudaSuccess) {
    GemmArgs g{};
    g.A = dA;
    g.B = dB;
    g.M = kTileM;
    g.N = 32;
    g.K = 16;
    g.outF = dD;
    g.ldo = 32;
    g.err = dErr;
    g.extraTx = 16;
    g.waitLimit = 1 << 16;
    e = launch_gemm(32, g, 1, 1, 1, 0);
  }
  unsigned herr = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&herr, dErr, 4, cudaMemcpyDeviceToHost);
  cudaFree(dA);
  cudaFree(dB);
  cudaFree(dD);
  cudaFree(dErr);
  if (e != cudaSuccess) return rs_fail(RESYNTH_ERROR_DEVICE, cudaGetErrorString(e));
  if (herr) return rs_fail(RESYNTH_ERROR_DEVICE, "tc gemm: a tensor-core wait ran out");
  return 0;
}

RS_EXPORT unsigned int resynthNetParamCount(void) { return (unsigned)kParams; }

RS_EXPORT void resynthNetDestroy(TResynthNet* net) {
  if (!net) return;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(net->dev);
  if (net->stream) cudaStreamSynchronize(net->stream);
  free_work(net);
  for (void* p : {(void*)net->params, (void*)net->adamM, (void*)net->adamV, (void*)net->grad, (void*)net->wblk,
                  (void*)net->wt, (void*)net->err, (void*)net->loss})
    cudaFree(p);
  if (net->stream) cudaStreamDestroy(net->stream);
  cudaSetDevice(prev);
  delete net;
}

static int upload_params(TResynthNet* net, const float* host) {
  try {
    NK(cudaMemcpyAsync(net->params, host, kParams * sizeof(float), cudaMemcpyHostToDevice, net->stream));
    NK(cudaMemsetAsync(net->adamM, 0, kParams * sizeof(float), net->stream));
    NK(cudaMemsetAsync(net->adamV, 0, kParams * sizeof(float), net->stream));
    k_relayout<<<64, 256, 0, net->stream>>>(net->params, net->wblk, net->wt);
    NK(cudaGetLastError());
    NK(cudaStreamSynchronize(net->stream));
    net->step = 0;
  } catch (const NetError& x) {
    return device_fail(x.e);
  }
  return 0;
}

RS_EXPORT TResynthNet* resynthNetCreate(unsigned int seed) {
  auto* net = new TResynthNet();
  cudaGetDevice(&net->dev);
  cudaError_t e = cudaStreamCreateWithFlags(&net->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&net->params, kParams * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&net->adamM, kParams * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&net->adamV, kParams * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&net->grad, kParams * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&net->wblk, kWblk * sizeof(uint16_t));
  if (e == cudaSuccess) e = cudaMalloc(&net->wt, kWt * sizeof(uint16_t));
  if (e == cudaSuccess) e = cudaMalloc(&net->err, 4);
  if (e == cudaSuccess) e = cudaMemset(net->err, 0, 4);
  if (e == cudaSuccess) e = cudaMemset(net->wt, 0, kWt * sizeof(uint16_t));
  if (e != cudaSuccess) {
    device_fail(e);
    resynthNetDestroy(net);
    return nullptr;
  }
  const std::vector<float> p = init_params(seed);
  if (upload_params(net, p.data())) {
    resynthNetDestroy(net);
    return nullptr;
  }
  return net;
}

RS_EXPORT int resynthNetSetParams(TResynthNet* net, const float* params) {
  if (!net || !params) return rs_fail(RESYNTH_ERROR_ARGUMENT, "net: NULL argument");
  std::lock_guard<std::mutex> lk(net->mu);
  return upload_params(net, params);
}

RS_EXPORT int resynthNetGetParams(TResynthNet* net, float* params) {
  if (!net || !params) return rs_fail(RESYNTH_ERROR_ARGUMENT, "net: NULL argument");
  std::lock_guard<std::mutex> lk(net->mu);
  cudaError_t e = cudaMemcpyAsync(params, net->params, kParams * sizeof(float), cudaMemcpyDeviceToHost, net->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(net->stream);
  return e == cudaSuccess ? 0 : device_fail(e);
}

RS_EXPORT int resynthNetForward(TResynthNet* net, const unsigned short* contexts, unsigned int n, float* out,
                                int path) {
  if (!net || !contexts || !out || !n) return rs_fail(RESYNTH_ERROR_ARGUMENT, "net: NULL argument");
  std::lock_guard<std::mutex> lk(net->mu);
  cudaStream_t s = net->stream;
  try {
    ensure_work(net, (int)n);
    NK(cudaMemsetAsync(net->err, 0, 4, s));
    NK(cudaMemcpyAsync(net->x0, contexts, (size_t)n * kCtxElems * 2, cudaMemcpyHostToDevice, s));
    if (path == 0) {
      InferArgs a{};
      a.wblk = net->wblk;
      a.params = net->params;
      a.x0 = net->x0;
      a.n = (int)n;
      a.out = net->out;
      a.err = net->err;
      NK(launch_infer<false>(a, (int)n, s));
    } else {
      train_forward(net, (int)n, s);
    }
    NK(cudaMemcpyAsync(out, net->out, (size_t)n * 32 * sizeof(float), cudaMemcpyDeviceToHost, s));
    check_err(net, s);
  } catch (const NetError& x) {
    return device_fail(x.e);
  }
  return 0;
}

RS_EXPORT int resynthNetGradients(TResynthNet* net, const unsigned short* contexts, const float* labels,
                                  unsigned int n, float* gradient, float* loss) {
  if (!net || !contexts || !labels || !n) return rs_fail(RESYNTH_ERROR_ARGUMENT, "net: NULL argument");
  std::lock_guard<std::mutex> lk(net->mu);
  cudaStream_t s = net->stream;
  try {
    ensure_work(net, (int)n);
    NK(cudaMemsetAsync(net->err, 0, 4, s));
    NK(cudaMemcpyAsync(net->x0, contexts, (size_t)n * kCtxElems * 2, cudaMemcpyHostToDevice, s));
    NK(cudaMemcpyAsync(net->labels, labels, (size_t)n * 2 * sizeof(float), cudaMemcpyHostToDevice, s));
    float* lossDev = nullptr;
    NK(cudaMallocAsync(&lossDev, sizeof(float), s));
    NK(cudaMemsetAsync(lossDev, 0, sizeof(float), s));
    train_forward(net, (int)n, s);
    train_backward(net, (int)n, lossDev, s);
    float hl = 0.f;
    NK(cudaMemcpyAsync(&hl, lossDev, sizeof(float), cudaMemcpyDeviceToHost, s));
    if (gradient) NK(cudaMemcpyAsync(gradient, net->grad, kParams * sizeof(float), cudaMemcpyDeviceToHost, s));
    NK(cudaFreeAsync(lossDev, s));
    check_err(net, s);
    if (loss) *loss = hl;
  } catch (const NetError& x) {
    return device_fail(x.e);
  }
  return 0;
}

RS_EXPORT int resynthNetTrain(TResynthNet* net, TResynthPairs* pairs, const TResynthTrainOptions* options,
                              float* lossOut) {
  if (!net || !pairs) return rs_fail(RESYNTH_ERROR_ARGUMENT, "net: NULL argument");
  if (!pairs->count) return rs_fail(RESYNTH_ERROR_ARGUMENT, "net: no training pairs");
  TResynthTrainOptions o{};
  if (options) o = *options;
  const unsigned steps = o.steps ? o.steps : 2000u;
  const int n = (int)(o.batch ? o.batch : 512u);
  const float lr = o.learningRate > 0.f ? o.learningRate : 1e-3f;
  std::lock_guard<std::mutex> lk(net->mu);
  std::lock_guard<std::mutex> lp(pairs->mu);
  cudaStream_t s = net->stream;
  try {
    ensure_work(net, n);
    float* losses = nullptr;
    NK(cudaMallocAsync(&losses, steps * sizeof(float), s));
    NK(cudaMemsetAsync(losses, 0, steps * sizeof(float), s));
    NK(cudaMemsetAsync(net->err, 0, 4, s));
    for (unsigned i = 0; i < steps; i++) {
      const uint32_t seed = (o.seed * 0x9E3779B9u) ^ (uint32_t)(net->step * 0x85EBCA6Bu) ^ 0x2545F491u;
      k_gather_batch<<<blocks_for((long long)n * (kCtxElems / 8), 256), 256, 0, s>>>(pairs->x0, pairs->labels,
                                                                                     pairs->count, n, seed, net->x0,
                                                                                     net->labels);
      NK(cudaGetLastError());
      train_forward(net, n, s);
      train_backward(net, n, losses + i, s);
      net->step++;
      const float bc1 = 1.f - std::pow(0.9f, (float)net->step), bc2 = 1.f - std::pow(0.999f, (float)net->step);
      k_adam<<<blocks_for(kParams, 256), 256, 0, s>>>(net->params, net->adamM, net->adamV, net->grad, kParams, lr, bc1,
                                                      bc2);
      k_relayout<<<64, 256, 0, s>>>(net->params, net->wblk, net->wt);
      NK(cudaGetLastError());
    }
    std::vector<float> hl(steps);
    NK(cudaMemcpyAsync(hl.data(), losses, steps * sizeof(float), cudaMemcpyDeviceToHost, s));
    NK(cudaFreeAsync(losses, s));
    check_err(net, s);
    if (lossOut) {
      const unsigned tail = std::max(1u, steps / 10);
      double acc = 0;
      for (unsigned i = steps - tail; i < steps; i++) acc += hl[i];
      *lossOut = (float)(acc / tail);
    }
  } catch (const NetError& x) {
    return device_fail(x.e);
  }
  return 0;
}

RS_EXPORT TResynthPairs* resynthPairsCreate(unsigned int capacity) {
  if (!capacity) {
    rs_fail(RESYNTH_ERROR_ARGUMENT, "pairs: zero capacity");
    return nullptr;
  }
  auto* p = new TResynthPairs();
  cudaGetDevice(&p->dev);
  cudaError_t e = cudaMalloc(&p->x0, (size_t)capacity * kCtxElems * 2);
  if (e == cudaSuccess) e = cudaMalloc(&p->labels, (size_t)capacity * 2 * sizeof(float));
  if (e != cudaSuccess) {
    device_fail(e);
    cudaFree(p->x0);
    cudaFree(p->labels);
    delete p;
    return nullptr;
  }
  p->cap = capacity;
  return p;
}

RS_EXPORT void resynthPairsDestroy(TResynthPairs* pairs) {
  if (!pairs) return;
  cudaDeviceSynchronize();
  cudaFree(pairs->x0);
  cudaFree(pairs->labels);
  delete pairs;
}

RS_EXPORT unsigned int resynthPairsCount(const TResynthPairs* pairs) { return pairs ? pairs->count : 0u; }

RS_EXPORT unsigned int resynthPairsAdd(TResynthPairs* pairs, const unsigned short* contexts, const float* labels,
                                       unsigned int n) {
  if (!pairs || !contexts || !labels) return 0;
  std::lock_guard<std::mutex> lk(pairs->mu);
  const unsigned k = std::min(n, pairs->cap - pairs->count);
  if (!k) return 0;
  cudaError_t e = cudaMemcpy(pairs->x0 + (size_t)pairs->count * kCtxElems, contexts, (size_t)k * kCtxElems * 2,
                             cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(pairs->labels + 2 * (size_t)pairs->count, labels, (size_t)k * 2 * sizeof(float),
                   cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    device_fail(e);
    return 0;
  }
  pairs->count += k;
  return k;
}

RS_EXPORT int resynthPairsRead(const TResynthPairs* pairs, unsigned int first, unsigned int n,
                               unsigned short* contexts, float* labels) {
  if (!pairs) return rs_fail(RESYNTH_ERROR_ARGUMENT, "pairs: NULL argument");
  if ((unsigned long long)first + n > pairs->count) return rs_fail(RESYNTH_ERROR_ARGUMENT, "pairs: range");
  cudaDeviceSynchronize();
  cudaError_t e = cudaSuccess;
  if (contexts)
    e = cudaMemcpy(contexts, pairs->x0 + (size_t)first * kCtxElems, (size_t)n * kCtxElems * 2, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && labels)
    e = cudaMemcpy(labels, pairs->labels + 2 * (size_t)first, (size_t)n * 2 * sizeof(float), cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? 0 : device_fail(e);
}
