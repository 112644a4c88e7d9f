// synth_prep.cu -- device-side preparation for the wavefront mode.
//
// The reference prepares on the host (lib/engine.c:338-431): the selected
// target points in row-major order with their initial hasValue, and the
// corpus points (mask == 0xFF and not transparent).  Here the same lists are
// built by deterministic stream compaction, and each pass's targets are
// bucketed by (band, colour phase) with a counting sort so that batch b is
// targets[batchStart[b] .. batchStart[b+1]).
#include <algorithm>
#include <climits>
#include <cstdint>

#include "synth_internal.h"

namespace rs {
namespace {

constexpr int kThreads = 256;
constexpr int kItems = 16;
constexpr int kChunk = kThreads * kItems;   // pixels per block in the compactions

__device__ __forceinline__ uint32_t mix32p(uint32_t x) {
  x ^= x >> 16;
  x *= 0x85ebca6bu;
  x ^= x >> 13;
  x *= 0xc2b2ae35u;
  x ^= x >> 16;
  return x;
}

// Predicates on the interleaved pixmap.
struct PixPred {
  const uint8_t* raw;
  int bpp, alpha, hasAlpha;
  int mode;   // 0: target selected (mask != 0), 1: corpus point (mask == 0xFF and opaque)
  __device__ bool operator()(int i) const {
    const uint8_t* q = raw + (size_t)i * bpp;
    if (mode == 0) return q[0] != 0;
    return q[0] == 0xFF && (!hasAlpha || q[alpha] != 0);
  }
};

// Block-wide exclusive scan of one count per thread (kThreads threads).
__device__ int block_exclusive(int v, int* warpSums, int& total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warpSums[warp] = x;
  __syncthreads();
  int before = 0;
  total = 0;
  for (int w = 0; w < kThreads / 32; w++) {
    if (w < warp) before += warpSums[w];
    total += warpSums[w];
  }
  __syncthreads();
  return before + x - v;
}

// Target init: hasValue = useContext && !selected && opaque (lib/engine.c:366-384),
// sourceOf = (-1, -1); per-block counts of selected pixels; flags whether any
// pixel has a value (context).
__global__ void k_init_target(const uint8_t* raw, int npx, int bpp, int alpha, int hasAlpha, int useContext,
                              uint8_t* has, int2* src, int* blockCounts, int* anyContext) {
  const int base = blockIdx.x * kChunk;
  int cnt = 0, ctx = 0;
  for (int k = 0; k < kItems; k++) {
    const int i = base + k * kThreads + threadIdx.x;
    if (i < npx) {
      const uint8_t* q = raw + (size_t)i * bpp;
      const bool sel = q[0] != 0;
      const bool opaque = !hasAlpha || q[alpha] != 0;
      const uint8_t hv = (useContext && !sel && opaque) ? 1 : 0;
      has[i] = hv;
      src[i] = make_int2(-1, -1);
      cnt += sel;
      ctx |= hv;
    }
  }
  cnt = __reduce_add_sync(0xffffffffu, cnt);
  ctx = __reduce_or_sync(0xffffffffu, ctx);
  __shared__ int s[kThreads / 32];
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = cnt;
  if ((threadIdx.x & 31) == 0 && ctx) atomicOr(anyContext, 1);
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < kThreads / 32; w++) t += s[w];
    blockCounts[blockIdx.x] = t;
  }
}

__global__ void k_count(PixPred pred, int npx, int* blockCounts) {
  const int base = blockIdx.x * kChunk;
  int cnt = 0;
  for (int k = 0; k < kItems; k++) {
    const int i = base + k * kThreads + threadIdx.x;
    if (i < npx && pred(i)) cnt++;
  }
  cnt = __reduce_add_sync(0xffffffffu, cnt);
  __shared__ int s[kThreads / 32];
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < kThreads / 32; w++) t += s[w];
    blockCounts[blockIdx.x] = t;
  }
}

// Exclusive scan of n counts by one block; offsets[n] = total.
__global__ void k_scan(const int* counts, int n, int* offsets) {
  __shared__ int warpSums[kThreads / 32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int b = 0; b < n; b += kThreads) {
    const int i = b + threadIdx.x;
    const int v = i < n ? counts[i] : 0;
    int total;
    const int ex = block_exclusive(v, warpSums, total);
    if (i < n) offsets[i] = carry + ex;
    __syncthreads();
    if (threadIdx.x == 0) carry += total;
    __syncthreads();
  }
  if (threadIdx.x == 0) offsets[n] = carry;
}

// Writes the (x, y) of every pixel satisfying pred, in row-major order.
__global__ void k_compact(PixPred pred, int npx, int w, const int* blockOffsets, int2* out) {
  __shared__ int warpSums[kThreads / 32];
  int pos = blockOffsets[blockIdx.x];
  const int base = blockIdx.x * kChunk;
  for (int k = 0; k < kItems; k++) {
    const int i = base + k * kThreads + threadIdx.x;
    const bool f = i < npx && pred(i);
    int total;
    const int ex = block_exclusive(f ? 1 : 0, warpSums, total);
    if (f) out[pos + ex] = make_int2(i % w, i / w);
    pos += total;
  }
}

// Targets per bucketing chunk: one CTA each, so the result does not depend
// on the grid.
constexpr int kBucketChunk = 8192;

// Batch keys of one pass.  rank = position in the visit order: given (the
// host order) or drawn from a hash of the pixel (random orders).  Targets of
// rank >= endRank are not visited this pass.  key = band * K + phase.  Each
// CTA counts its chunk's keys; counts are stored key-major, [key][chunk], so
// one exclusive scan gives every (key, chunk) its output position.
__device__ void batch_keys_chunk(int chunk, const int2* targets, int n, int tw, int endRank, int randomOrder,
                                 uint32_t seed, const int* bandEnds, const int* bandPhased, int nbands, int k,
                                 int* keys, int* counts, int nchunks, int* vis, int* hist) {
  const int nkeys = nbands * k * k;
  for (int i = threadIdx.x; i < nkeys; i += blockDim.x) hist[i] = 0;
  __syncthreads();
  for (int i = threadIdx.x; i < kBucketChunk; i += blockDim.x) {
    const int t = chunk * kBucketChunk + i;
    if (t >= n) break;
    const int2 p = targets[t];
    const int rank = randomOrder ? (int)__umulhi(mix32p((uint32_t)(p.y * tw + p.x) * 0x9E3779B1u ^ seed),
                                                 (uint32_t)n)
                                 : t;
    int key = -1;
    if (rank < endRank) {
      int band = 0;
      while (band < nbands - 1 && rank >= bandEnds[band]) band++;
      key = band * k * k + (bandPhased[band] ? (p.y % k) * k + (p.x % k) : 0);
      atomicAdd(&hist[key], 1);
    }
    keys[t] = key;
    // pass 0: the pixel gets its value in batch `key`
    if (vis && key >= 0) vis[p.y * tw + p.x] = key;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nkeys; i += blockDim.x) counts[(size_t)i * nchunks + chunk] = hist[i];
}

__global__ void k_batch_keys(const int2* targets, int n, int tw, int endRank, int randomOrder, uint32_t seed,
                             const int* bandEnds, const int* bandPhased, int nbands, int k, int* keys, int* counts,
                             int nchunks, int* vis) {
  extern __shared__ int hist[];
  batch_keys_chunk(blockIdx.x, targets, n, tw, endRank, randomOrder, seed, bandEnds, bandPhased, nbands, k, keys,
                   counts, nchunks, vis, hist);
}

// Exclusive scan of n ints by one CTA of 1024 threads, 8 consecutive
// elements per thread per round; offsets[n] = the total.
__device__ void scan_wide(const int* counts, int n, int* offsets) {
  __shared__ int warpSums[32];
  __shared__ int carry;
  constexpr int kPer = 8;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < n; base += 1024 * kPer) {
    const int i0 = base + threadIdx.x * kPer;
    int v[kPer], sum = 0;
#pragma unroll
    for (int j = 0; j < kPer; j++) {
      v[j] = i0 + j < n ? counts[i0 + j] : 0;
      sum += v[j];
    }
    int x = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warpSums[warp] = x;
    __syncthreads();
    if (warp == 0) {
      int w = warpSums[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += y;
      }
      warpSums[lane] = w;   // inclusive
    }
    __syncthreads();
    int run = carry + (warp ? warpSums[warp - 1] : 0) + x - sum;
#pragma unroll
    for (int j = 0; j < kPer; j++) {
      if (i0 + j < n) offsets[i0 + j] = run;
      run += v[j];
    }
    __syncthreads();
    if (threadIdx.x == 0) carry += warpSums[31];
    __syncthreads();
  }
  if (threadIdx.x == 0) offsets[n] = carry;
}

__global__ void __launch_bounds__(1024) k_scan_wide(const int* counts, int n, int* offsets) {
  scan_wide(counts, n, offsets);
}

// batchStart[key] = the scanned offset of (key, chunk 0).
__global__ void k_batch_starts(const int* offsets, int nkeys, int nchunks, int* batchStart) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= nkeys; i += gridDim.x * blockDim.x)
    batchStart[i] = offsets[(size_t)i * nchunks];
}

// Stable scatter: within a batch, targets keep their order in the target
// list.  Each CTA places its chunk; a lane's position is its (key, chunk)
// offset + the same-key count of earlier warps (taken warp by warp) + its
// rank among the same-key lanes of its warp.
__device__ void scatter_chunk(int chunk, const int2* targets, int n, const int* keys, const int* offsets, int nkeys,
                              int nchunks, int2* out, int* cnt) {
  for (int i = threadIdx.x; i < nkeys; i += blockDim.x) cnt[i] = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  unsigned lt;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
  for (int base = 0; base < kBucketChunk; base += blockDim.x) {
    const int t = chunk * kBucketChunk + base + threadIdx.x;
    const int key = t < n ? keys[t] : -1;
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    const int leader = __ffs(peers) - 1;
    int before = 0;
    for (int w = 0; w < nwarps; w++) {
      if (warp == w) {
        if (key >= 0) before = cnt[key];
        __syncwarp();
        if (lane == leader && key >= 0) cnt[key] = before + __popc(peers);
      }
      __syncthreads();
    }
    if (key >= 0) out[offsets[(size_t)key * nchunks + chunk] + before + __popc(peers & lt)] = targets[t];
  }
}

__global__ void k_scatter(const int2* targets, int n, const int* keys, const int* offsets, int nkeys, int nchunks,
                          int2* out) {
  extern __shared__ int cnt[];
  scatter_chunk(blockIdx.x, targets, n, keys, offsets, nkeys, nchunks, out, cnt);
}

// The same bucketing for many requests at once: one launch per stage, each
// request's chunks (or, for the scans, one CTA) found from its entry.
__device__ __forceinline__ int job_of_chunk(const int* chunk0, int njobs, int c) {
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (chunk0[mid] <= c) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__global__ void k_batch_keys_multi(const PrepJob* jobs, const int* chunk0, int njobs) {
  extern __shared__ int hist[];
  const int j = job_of_chunk(chunk0, njobs, blockIdx.x);
  const PrepJob& J = jobs[j];
  batch_keys_chunk(blockIdx.x - chunk0[j], J.targets, J.n, J.tw, J.endRank, J.randomOrder, J.seed, J.bandEnds,
                   J.bandPhased, J.nbands, J.k, J.keys, J.counts, J.nchunks, J.vis, hist);
}

__global__ void __launch_bounds__(1024) k_scan_wide_multi(const PrepJob* jobs) {
  const PrepJob& J = jobs[blockIdx.x];
  scan_wide(J.counts, J.nbands * J.k * J.k * J.nchunks, J.offsets);
}

__global__ void k_batch_starts_multi(const PrepJob* jobs) {
  const PrepJob& J = jobs[blockIdx.x];
  const int nkeys = J.nbands * J.k * J.k;
  for (int i = threadIdx.x; i <= nkeys; i += blockDim.x) J.batchStart[i] = J.offsets[(size_t)i * J.nchunks];
}

__global__ void k_scatter_multi(const PrepJob* jobs, const int* chunk0, int njobs) {
  extern __shared__ int cnt[];
  const int j = job_of_chunk(chunk0, njobs, blockIdx.x);
  const PrepJob& J = jobs[j];
  scatter_chunk(blockIdx.x - chunk0[j], J.targets, J.n, J.keys, J.offsets, J.nbands * J.k * J.k, J.nchunks, J.out,
                cnt);
}

int blocks_for(int n, int per) { return (n + per - 1) / per; }

}  // namespace
}  // namespace rs

using namespace rs;

extern "C" cudaError_t rs_prep_target(const uint8_t* raw, int w, int h, int bpp, int alpha, int hasAlpha,
                                      int useContext, uint8_t* has, int2* src, int* scratch, int2* targets,
                                      int* counts, cudaStream_t s) {
  // scratch: 2 * nblocks + 1 ints; counts[0] = number of targets, counts[1] = any context
  const int npx = w * h, nb = blocks_for(npx, kChunk);
  int* blockCounts = scratch;
  int* offsets = scratch + nb;
  cudaMemsetAsync(counts + 1, 0, sizeof(int), s);
  k_init_target<<<nb, kThreads, 0, s>>>(raw, npx, bpp, alpha, hasAlpha, useContext, has, src, blockCounts, counts + 1);
  k_scan<<<1, kThreads, 0, s>>>(blockCounts, nb, offsets);
  PixPred pred{raw, bpp, alpha, hasAlpha, 0};
  k_compact<<<nb, kThreads, 0, s>>>(pred, npx, w, offsets, targets);
  cudaMemcpyAsync(counts, offsets + nb, sizeof(int), cudaMemcpyDeviceToDevice, s);
  return cudaGetLastError();
}

extern "C" cudaError_t rs_prep_corpus(const uint8_t* raw, int w, int h, int bpp, int alpha, int hasAlpha,
                                      int* scratch, int2* points, int* count, cudaStream_t s) {
  const int npx = w * h, nb = blocks_for(npx, kChunk);
  int* blockCounts = scratch;
  int* offsets = scratch + nb;
  PixPred pred{raw, bpp, alpha, hasAlpha, 1};
  k_count<<<nb, kThreads, 0, s>>>(pred, npx, blockCounts);
  k_scan<<<1, kThreads, 0, s>>>(blockCounts, nb, offsets);
  k_compact<<<nb, kThreads, 0, s>>>(pred, npx, w, offsets, points);
  cudaMemcpyAsync(count, offsets + nb, sizeof(int), cudaMemcpyDeviceToDevice, s);
  return cudaGetLastError();
}

extern "C" int rs_prep_scratch_ints(int w, int h) { return 2 * blocks_for(w * h, kChunk) + 1; }

// Buckets the targets of one pass into batches: out[batchStart[b] ..
// batchStart[b+1]) are the targets of batch b = band * k * k + phase, in the
// order of the target list.  work: rs_prep_batches_ints(n, nkeys) ints.
extern "C" cudaError_t rs_prep_batches(const int2* targets, int n, int tw, int endRank, int randomOrder,
                                       uint32_t seed, const int* dBandEnds, const int* dBandPhased, int nbands,
                                       int k, int* work, int* batchStart, int2* out, int* vis, cudaStream_t s) {
  const int nkeys = nbands * k * k;
  const int nchunks = std::max(1, blocks_for(n, kBucketChunk));
  const size_t cells = (size_t)nkeys * nchunks;
  int* counts = work;
  int* offsets = work + cells;
  int* keys = work + 2 * cells + 1;
  const size_t smem = (size_t)nkeys * sizeof(int);
  k_batch_keys<<<nchunks, 256, smem, s>>>(targets, n, tw, endRank, randomOrder, seed, dBandEnds, dBandPhased, nbands,
                                          k, keys, counts, nchunks, vis);
  k_scan_wide<<<1, 1024, 0, s>>>(counts, (int)cells, offsets);
  k_batch_starts<<<blocks_for(nkeys + 1, 256), 256, 0, s>>>(offsets, nkeys, nchunks, batchStart);
  k_scatter<<<nchunks, 256, smem, s>>>(targets, n, keys, offsets, nkeys, nchunks, out);
  return cudaGetLastError();
}

extern "C" size_t rs_prep_batches_ints(int n, int nkeys) {
  const size_t nchunks = (size_t)std::max(1, blocks_for(n, kBucketChunk));
  return 2 * (size_t)nkeys * nchunks + 1 + (size_t)n;
}

namespace rs {
namespace {
// Visit stamps before pass 0: -1 for pixels that have a value from the start
// (context), INT_MAX for the rest; targets get their batch index in pass 0.
__global__ void k_vis_init(const uint8_t* has, int npx, int* vis) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < npx; i += gridDim.x * blockDim.x)
    vis[i] = has[i] ? -1 : 0x7fffffff;
}
__global__ void k_vis_to_has(const int* vis, int npx, uint8_t* has) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < npx; i += gridDim.x * blockDim.x)
    has[i] = vis[i] != 0x7fffffff ? 1 : 0;
}
// Least visit stamp of each kCell x kCell cell: a pixel of the cell can have
// a value during batch b only if the cell's minimum is below b.
__device__ void cell_min(const int* vis, int tw, int th, int* cellMin, int first, int step) {
  const int cw = (tw + kCell - 1) >> kCellShift, ch = (th + kCell - 1) >> kCellShift;
  const int lane = threadIdx.x & 31;
  for (int c = first; c < cw * ch; c += step) {
    const int x0 = (c % cw) << kCellShift, y0 = (c / cw) << kCellShift;
    int m = 0x7fffffff;
    for (int i = lane; i < kCell * kCell; i += 32) {
      const int x = x0 + (i & (kCell - 1)), y = y0 + (i >> kCellShift);
      if (x < tw && y < th) m = min(m, vis[y * tw + x]);
    }
    for (int o = 16; o; o >>= 1) m = min(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0) cellMin[c] = m;
  }
}

__global__ void k_cell_min(const int* vis, int tw, int th, int* cellMin) {
  cell_min(vis, tw, th, cellMin, (blockIdx.x * blockDim.x + threadIdx.x) >> 5, (gridDim.x * blockDim.x) >> 5);
}

// Cell minima of many requests: blockIdx.y is the request (those without a
// cell grid have cellMin == null).
__global__ void k_cell_min_multi(const PrepJob* jobs) {
  const PrepJob& J = jobs[blockIdx.y];
  if (!J.cellMin) return;
  cell_min(J.vis, J.tw, J.th, J.cellMin, (blockIdx.x * blockDim.x + threadIdx.x) >> 5,
           (gridDim.x * blockDim.x) >> 5);
}
}  // namespace
}  // namespace rs

extern "C" cudaError_t rs_cell_min(const int* vis, int tw, int th, int* cellMin, cudaStream_t s) {
  const int cells = ((tw + kCell - 1) >> kCellShift) * ((th + kCell - 1) >> kCellShift);
  k_cell_min<<<std::min(blocks_for(cells * 32, 256), 4096), 256, 0, s>>>(vis, tw, th, cellMin);
  return cudaGetLastError();
}

extern "C" cudaError_t rs_vis_init(const uint8_t* has, int npx, int* vis, cudaStream_t s) {
  k_vis_init<<<std::min(blocks_for(npx, 256), 2048), 256, 0, s>>>(has, npx, vis);
  return cudaGetLastError();
}

extern "C" cudaError_t rs_vis_to_has(const int* vis, int npx, uint8_t* has, cudaStream_t s) {
  k_vis_to_has<<<std::min(blocks_for(npx, 256), 2048), 256, 0, s>>>(vis, npx, has);
  return cudaGetLastError();
}

// ---------------------------------------------------------- simple-API adapters
// adaptSimpleAPI / adaptSimpleAPI2 (lib/adaptSimple.h:260-354) on the device:
// the caller's row-padded image and mask(s) become the interleaved target
// pixmap [mask][pixelels] and corpus pixmap [~mask or mask2][pixelels].
namespace rs {
namespace {
__global__ void k_adapt(const uint8_t* img, size_t imgRow, const uint8_t* mask, size_t maskRow, const uint8_t* mask2,
                        size_t mask2Row, int w, int h, int bpp, uint8_t* target, uint8_t* corpus) {
  const int d = bpp + 1;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w * h; i += gridDim.x * blockDim.x) {
    const int x = i % w, y = i / w;
    const uint8_t* s = img + (size_t)y * imgRow + (size_t)x * bpp;
    uint8_t* t = target + (size_t)i * d;
    uint8_t* c = corpus + (size_t)i * d;
    const uint8_t m = mask[(size_t)y * maskRow + x];
    t[0] = m;
    c[0] = mask2 ? mask2[(size_t)y * mask2Row + x] : (uint8_t)~m;
    for (int k = 0; k < bpp; k++) t[1 + k] = c[1 + k] = s[k];
  }
}
// antiAdaptImage (lib/adaptSimple.h:110-168): every pixel's pixelels back
// into the row-padded image (only target colours can have changed).
__global__ void k_unadapt(const uint8_t* target, int w, int h, int bpp, uint8_t* img, size_t imgRow) {
  const int d = bpp + 1;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w * h; i += gridDim.x * blockDim.x) {
    const int x = i % w, y = i / w;
    uint8_t* o = img + (size_t)y * imgRow + (size_t)x * bpp;
    const uint8_t* t = target + (size_t)i * d;
    for (int k = 0; k < bpp; k++) o[k] = t[1 + k];
  }
}
}  // namespace
}  // namespace rs

extern "C" cudaError_t rs_adapt(const uint8_t* img, size_t imgRow, const uint8_t* mask, size_t maskRow,
                                const uint8_t* mask2, size_t mask2Row, int w, int h, int bpp, uint8_t* target,
                                uint8_t* corpus, cudaStream_t s) {
  k_adapt<<<std::min(blocks_for(w * h, 256), 4096), 256, 0, s>>>(img, imgRow, mask, maskRow, mask2, mask2Row, w, h,
                                                                   bpp, target, corpus);
  return cudaGetLastError();
}

extern "C" cudaError_t rs_unadapt(const uint8_t* target, int w, int h, int bpp, uint8_t* img, size_t imgRow,
                                  cudaStream_t s) {
  k_unadapt<<<std::min(blocks_for(w * h, 256), 4096), 256, 0, s>>>(target, w, h, bpp, img, imgRow);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Directional and brushfire visit orders on the device (lib/orderTarget.h:
// 154-343, lib/brushfire.h:62-163).  The reference sorts the target points
// with libc qsort (glibc: a merge sort) and comparators that never return 0:
// the "more" comparators keep equal keys in input order, the "less" ones
// reverse them.  Both are a stable sort of 32-bit keys -- over the input
// reversed for the "less" comparators -- done here as an LSD radix sort of
// four 8-bit digits.  Keys: |dx| or |dy| from the bounding-box centre for the
// directional types (ordering by dx^2 is ordering by |dx|); for brushfire,
// the float |p|^2 / (largest |q|^2 on p's ray), whose bit pattern orders like
// the value for the non-negative floats it takes.  The banded shuffle that
// follows the sort (lib/orderTarget.h:58-79) is a fixed permutation of
// positions given by the host.
namespace rs {
namespace {

constexpr int kOrderChunk = 8192;
constexpr int kRays = 401;

// work layout (ints): [0..4) bounding box (minx, miny, maxx, maxy),
// [4] NaN flag, [8 .. 8 + kRays) largest |q|^2 per ray, then n rays, keys A,
// keys B, values A, values B, and the digit counts and their offsets.
struct OrderWork {
  int* box;
  int* nan;
  unsigned* maxr;
  int* rays;
  unsigned *keysA, *keysB;
  int *valsA, *valsB;
  int *counts, *offsets;
  int nchunks;
  __host__ __device__ OrderWork(int* w, int n) {
    nchunks = n > 0 ? (n + kOrderChunk - 1) / kOrderChunk : 1;
    box = w;
    nan = w + 4;
    maxr = reinterpret_cast<unsigned*>(w + 8);
    rays = w + 8 + kRays;
    keysA = reinterpret_cast<unsigned*>(rays + n);
    keysB = keysA + n;
    valsA = reinterpret_cast<int*>(keysB + n);
    valsB = valsA + n;
    counts = valsB + n;
    offsets = counts + 256 * nchunks;
  }
  static size_t ints(int n) {
    const size_t nchunks = n > 0 ? ((size_t)n + kOrderChunk - 1) / kOrderChunk : 1;
    return 8 + kRays + 5 * (size_t)n + 2 * 256 * nchunks + 1;
  }
};

__global__ void k_order_init(int* w, int n) {
  OrderWork W(w, n);
  for (int i = threadIdx.x; i < kRays; i += blockDim.x) W.maxr[i] = 0;
  if (threadIdx.x == 0) {
    W.box[0] = W.box[1] = INT_MAX;   // lib/engineTypes.h:187-226 starts from these
    W.box[2] = W.box[3] = 0;
    *W.nan = 0;
  }
}

__global__ void k_order_bbox(const int2* t, int n, int* w) {
  OrderWork W(w, n);
  int x0 = INT_MAX, y0 = INT_MAX, x1 = 0, y1 = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int2 p = t[i];
    x0 = min(x0, p.x);
    y0 = min(y0, p.y);
    x1 = max(x1, p.x);
    y1 = max(y1, p.y);
  }
  x0 = __reduce_min_sync(0xffffffffu, x0);
  y0 = __reduce_min_sync(0xffffffffu, y0);
  x1 = __reduce_max_sync(0xffffffffu, x1);
  y1 = __reduce_max_sync(0xffffffffu, y1);
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&W.box[0], x0);
    atomicMin(&W.box[1], y0);
    atomicMax(&W.box[2], x1);
    atomicMax(&W.box[3], y1);
  }
}

__device__ __forceinline__ int2 rel(const OrderWork& W, int2 p) {
  const int cx = (W.box[2] - W.box[0]) / 2 + W.box[0], cy = (W.box[3] - W.box[1]) / 2 + W.box[1];
  return make_int2(p.x - cx, p.y - cy);
}

// Brushfire rays: (unsigned)(atan2(y, x) * 200 / pi + 200) in double, as the
// reference computes it.  The device atan2 may differ from the host libm's
// in the last bits, which can only matter where the value lies next to a
// whole number (the axes and diagonals): those targets are listed for the
// host to recompute, as (index, dx, dy).
__global__ void k_order_rays(const int2* t, int n, int* w, int* flagCount, int* flags, int cap) {
  OrderWork W(w, n);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int2 p = rel(W, t[i]);
    const double v = atan2((double)(float)p.y, (double)(float)p.x) * 200 / 3.1415926535897932384626433832795 + 200;
    W.rays[i] = (int)(unsigned)v;
    if (fabs(v - rint(v)) < 1e-9) {
      const int k = atomicAdd(flagCount, 1);
      if (k < cap) {
        flags[3 * k] = i;
        flags[3 * k + 1] = p.x;
        flags[3 * k + 2] = p.y;
      }
    }
  }
}

__global__ void k_order_fix_rays(const int* fix, int nfix, int* w, int n) {
  OrderWork W(w, n);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nfix; i += gridDim.x * blockDim.x)
    W.rays[fix[2 * i]] = fix[2 * i + 1];
}

__global__ void k_order_maxr(const int2* t, int n, int* w) {
  OrderWork W(w, n);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int2 p = rel(W, t[i]);
    atomicMax(&W.maxr[W.rays[i]], (unsigned)(p.x * p.x + p.y * p.y));
  }
}

// 0 / 0: the centre is a target and alone on its ray.  The comparators then
// meet a NaN, which orders like no key; the host makes that order.
__global__ void k_order_nan(const int2* t, int n, int* w) {
  OrderWork W(w, n);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int2 p = rel(W, t[i]);
    if (p.x == 0 && p.y == 0 && W.maxr[W.rays[i]] == 0) *W.nan = 1;
  }
}

__global__ void k_order_keys(int type, const int2* t, int n, int* w) {
  OrderWork W(w, n);
  const bool reverse = type == 5 || type == 6 || type == 7;   // the "less" comparators
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int src = reverse ? n - 1 - i : i;
    const int2 p = rel(W, t[src]);
    unsigned key;
    if (type == 3 || type == 6 || type == 4 || type == 7) {
      const unsigned a = (unsigned)abs(type == 3 || type == 6 ? p.x : p.y);
      key = type == 3 || type == 4 ? ~a : a;   // 3, 4: descending; 6, 7: ascending
    } else {
      const float prop = __fdiv_rn((float)(p.y * p.y + p.x * p.x), __uint2float_rn(W.maxr[W.rays[src]]));
      const unsigned b = __float_as_uint(prop);
      key = type == 5 ? b : ~b;                 // 2, 8: descending; 5: ascending
    }
    W.keysA[i] = key;
    W.valsA[i] = src;
  }
}

// One 8-bit digit pass of the radix sort: per chunk, the count of each digit
// value, stored digit-major ([digit][chunk]) for one exclusive scan.
__global__ void k_order_hist(const unsigned* keys, int n, int shift, int* counts, int nchunks) {
  __shared__ int hist[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) hist[i] = 0;
  __syncthreads();
  for (int i = threadIdx.x; i < kOrderChunk; i += blockDim.x) {
    const int j = blockIdx.x * kOrderChunk + i;
    if (j >= n) break;
    atomicAdd(&hist[(keys[j] >> shift) & 0xFFu], 1);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 256; i += blockDim.x) counts[(size_t)i * nchunks + blockIdx.x] = hist[i];
}

// Stable scatter of one digit pass (as k_scatter: warps of a chunk in order,
// lanes of a warp by rank among same-digit lanes).
__global__ void k_order_scatter(const unsigned* keys, const int* vals, int n, int shift, const int* offsets,
                                int nchunks, unsigned* keysOut, int* valsOut) {
  __shared__ int cnt[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) cnt[i] = 0;
  __syncthreads();
  const int chunk = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  unsigned lt;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
  for (int base = 0; base < kOrderChunk; base += blockDim.x) {
    const int j = chunk * kOrderChunk + base + threadIdx.x;
    const int d = j < n ? (int)((keys[j] >> shift) & 0xFFu) : -1;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int leader = __ffs(peers) - 1;
    int before = 0;
    for (int w = 0; w < nwarps; w++) {
      if (warp == w) {
        if (d >= 0) before = cnt[d];
        __syncwarp();
        if (lane == leader && d >= 0) cnt[d] = before + __popc(peers);
      }
      __syncthreads();
    }
    if (d >= 0) {
      const int pos = offsets[(size_t)d * nchunks + chunk] + before + __popc(peers & lt);
      keysOut[pos] = keys[j];
      valsOut[pos] = vals[j];
    }
  }
}

// out[i] = the target at sorted position perm[i] (the banded shuffle).
__global__ void k_order_gather(const int2* t, const int* sorted, const int* perm, int n, int2* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    out[i] = t[sorted[perm[i]]];
}

int grid_of(int n) { return std::max(1, std::min(blocks_for(n, 256), 2048)); }

}  // namespace
}  // namespace rs

extern "C" size_t rs_order_ints(int n) { return OrderWork::ints(n); }

extern "C" cudaError_t rs_order_begin(int type, const int2* targets, int n, int* work, int* flagCount, int* flags,
                                      int cap, cudaStream_t s) {
  k_order_init<<<1, 512, 0, s>>>(work, n);
  k_order_bbox<<<grid_of(n), 256, 0, s>>>(targets, n, work);
  if (type == 2 || type == 5 || type == 8) {
    cudaMemsetAsync(flagCount, 0, sizeof(int), s);
    k_order_rays<<<grid_of(n), 256, 0, s>>>(targets, n, work, flagCount, flags, cap);
  }
  return cudaGetLastError();
}

extern "C" cudaError_t rs_order_rays(const int2* targets, int n, int* work, const int* fix, int nfix,
                                     cudaStream_t s) {
  if (nfix) k_order_fix_rays<<<grid_of(nfix), 256, 0, s>>>(fix, nfix, work, n);
  k_order_maxr<<<grid_of(n), 256, 0, s>>>(targets, n, work);
  k_order_nan<<<grid_of(n), 256, 0, s>>>(targets, n, work);
  return cudaGetLastError();
}

extern "C" int* rs_order_nan_flag(int* work, int n) { return OrderWork(work, n).nan; }

extern "C" cudaError_t rs_order_finish(int type, const int2* targets, int n, int* work, const int* perm, int2* out,
                                       cudaStream_t s) {
  OrderWork W(work, n);
  k_order_keys<<<grid_of(n), 256, 0, s>>>(type, targets, n, work);
  unsigned *ka = W.keysA, *kb = W.keysB;
  int *va = W.valsA, *vb = W.valsB;
  for (int shift = 0; shift < 32; shift += 8) {
    k_order_hist<<<W.nchunks, 256, 0, s>>>(ka, n, shift, W.counts, W.nchunks);
    k_scan_wide<<<1, 1024, 0, s>>>(W.counts, 256 * W.nchunks, W.offsets);
    k_order_scatter<<<W.nchunks, 256, 0, s>>>(ka, va, n, shift, W.offsets, W.nchunks, kb, vb);
    std::swap(ka, kb);
    std::swap(va, vb);
  }
  k_order_gather<<<grid_of(n), 256, 0, s>>>(targets, va, perm, n, out);
  return cudaGetLastError();
}

extern "C" cudaError_t rs_prep_batches_multi(const PrepJob* dJobs, const int* dChunk0, int njobs, int totalChunks,
                                             int maxKeys, int cellBlocks, cudaStream_t s) {
  if (njobs < 1) return cudaSuccess;
  const size_t smem = (size_t)maxKeys * sizeof(int);
  k_batch_keys_multi<<<totalChunks, 256, smem, s>>>(dJobs, dChunk0, njobs);
  k_scan_wide_multi<<<njobs, 1024, 0, s>>>(dJobs);
  k_batch_starts_multi<<<njobs, 256, 0, s>>>(dJobs);
  k_scatter_multi<<<totalChunks, 256, smem, s>>>(dJobs, dChunk0, njobs);
  if (cellBlocks > 0) k_cell_min_multi<<<dim3(cellBlocks, njobs), 256, 0, s>>>(dJobs);
  return cudaGetLastError();
}

extern "C" int rs_prep_chunks(int n) { return std::max(1, blocks_for(n, kBucketChunk)); }

// ---------------------------------------------------------------------------
// The many-request path's set-up and write-back: the same work as rs_adapt,
// the packing, rs_prep_target, rs_prep_corpus and rs_vis_init, then
// rs_unadapt, but for every request of a call in a handful of launches
// (blockIdx.y, or the compaction chunk, says which request).
namespace rs {
namespace {

__device__ __forceinline__ int job_of(const int* chunk0, int njobs, int c) { return job_of_chunk(chunk0, njobs, c); }

// Adaption (lib/adaptSimple.h:260-354), packed words, padded corpus, initial
// hasValue / sourceOf (lib/engine.c:338-391) and visit stamps.
__global__ void k_setup_pixels(const SetupJob* jobs, int* counts) {
  const SetupJob& J = jobs[blockIdx.y];
  const int npx = J.w * J.h, d = J.bpp + 1;
  int ctx = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < npx; i += gridDim.x * blockDim.x) {
    const int x = i % J.w, y = i / J.w;
    const uint8_t* src = J.img + (size_t)y * J.imgRow + (size_t)x * J.bpp;
    const uint8_t m = J.mask[(size_t)y * J.maskRow + x];
    const uint8_t cm = J.mask2 ? J.mask2[(size_t)y * J.mask2Row + x] : (uint8_t)~m;
    uint8_t* t = J.target + (size_t)i * d;
    uint8_t* c = J.corpus + (size_t)i * d;
    t[0] = m;
    c[0] = cm;
    uint32_t tw = m, cw = cm;
    for (int k = 0; k < J.bpp; k++) {
      const uint8_t v = src[k];
      t[1 + k] = c[1 + k] = v;
      if (k < J.nc) {
        tw |= (uint32_t)v << (8 * (k + 1));
        cw |= (uint32_t)v << (8 * (k + 1));
      }
    }
    J.tpx[i] = tw;
    J.cpx[i] = cw;
    const bool opaque = !J.alphaT || src[J.alpha - 1] != 0;
    const uint8_t hv = (J.useContext && m == 0 && opaque) ? 1 : 0;
    J.has[i] = hv;
    J.src[i] = make_int2(-1, -1);
    J.vis[i] = hv ? -1 : 0x7fffffff;
    ctx |= hv;
  }
  // the corpus with a kPad-wide border of masked (zero) words
  const int pw = J.w + 2 * kPad, ph = J.h + 2 * kPad;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < pw * ph; i += gridDim.x * blockDim.x) {
    const int x = i % pw - kPad, y = i / pw - kPad;
    uint32_t word = 0;
    if (x >= 0 && x < J.w && y >= 0 && y < J.h) {
      const uint8_t* src = J.img + (size_t)y * J.imgRow + (size_t)x * J.bpp;
      word = J.mask2 ? J.mask2[(size_t)y * J.mask2Row + x] : (uint8_t)~J.mask[(size_t)y * J.maskRow + x];
      for (int k = 0; k < J.nc; k++) word |= (uint32_t)src[k] << (8 * (k + 1));
    }
    J.cpxPad[i] = word;
  }
  ctx = __reduce_or_sync(0xffffffffu, ctx);
  if ((threadIdx.x & 31) == 0 && ctx) atomicOr(&counts[4 * blockIdx.y + 1], 1);
}

__device__ __forceinline__ bool setup_target(const SetupJob& J, int i) { return J.target[(size_t)i * (J.bpp + 1)] != 0; }
__device__ __forceinline__ bool setup_corpus(const SetupJob& J, int i) {
  const uint8_t* q = J.corpus + (size_t)i * (J.bpp + 1);
  return q[0] == 0xFF && (!J.alphaS || q[J.alpha] != 0);
}

// Per compaction chunk: how many targets and corpus points it holds.
__global__ void k_setup_count(const SetupJob* jobs, const int* chunk0, int njobs, int* cntT, int* cntC) {
  const int j = job_of(chunk0, njobs, blockIdx.x);
  const SetupJob& J = jobs[j];
  const int npx = J.w * J.h, base = (blockIdx.x - chunk0[j]) * kChunk;
  int a = 0, b = 0;
  for (int k = 0; k < kItems; k++) {
    const int i = base + k * kThreads + threadIdx.x;
    if (i < npx) {
      a += setup_target(J, i);
      b += setup_corpus(J, i);
    }
  }
  a = __reduce_add_sync(0xffffffffu, a);
  b = __reduce_add_sync(0xffffffffu, b);
  __shared__ int sa[kThreads / 32], sb[kThreads / 32];
  if ((threadIdx.x & 31) == 0) {
    sa[threadIdx.x >> 5] = a;
    sb[threadIdx.x >> 5] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int ta = 0, tb = 0;
    for (int w = 0; w < kThreads / 32; w++) {
      ta += sa[w];
      tb += sb[w];
    }
    cntT[blockIdx.x] = ta;
    cntC[blockIdx.x] = tb;
  }
}

// One CTA per request: the exclusive scans of its chunks' counts and the totals.
__global__ void k_setup_scan(const int* chunk0, const int* cntT, const int* cntC, int* offT, int* offC, int* counts) {
  __shared__ int warpSums[kThreads / 32];
  const int j = blockIdx.x, c0 = chunk0[j], nb = chunk0[j + 1] - c0;
  for (int which = 0; which < 2; which++) {
    const int* cnt = which ? cntC : cntT;
    int* off = which ? offC : offT;
    int carry = 0;
    for (int b = 0; b < nb; b += kThreads) {
      const int i = b + threadIdx.x;
      const int v = i < nb ? cnt[c0 + i] : 0;
      int total;
      const int ex = block_exclusive(v, warpSums, total);
      if (i < nb) off[c0 + i] = carry + ex;
      carry += total;
    }
    if (threadIdx.x == 0) counts[4 * j + (which ? 2 : 0)] = carry;
    __syncthreads();
  }
}

__global__ void k_setup_compact(const SetupJob* jobs, const int* chunk0, int njobs, const int* offT,
                                const int* offC) {
  __shared__ int warpSums[kThreads / 32];
  const int j = job_of(chunk0, njobs, blockIdx.x);
  const SetupJob& J = jobs[j];
  const int npx = J.w * J.h, base = (blockIdx.x - chunk0[j]) * kChunk;
  int pt = offT[blockIdx.x], pc = offC[blockIdx.x];
  for (int k = 0; k < kItems; k++) {
    const int i = base + k * kThreads + threadIdx.x;
    const bool ft = i < npx && setup_target(J, i);
    const bool fc = i < npx && setup_corpus(J, i);
    int tt, tc;
    const int et = block_exclusive(ft ? 1 : 0, warpSums, tt);
    const int ec = block_exclusive(fc ? 1 : 0, warpSums, tc);
    if (ft) J.targets[pt + et] = make_int2(i % J.w, i / J.w);
    if (fc) J.cpts[pc + ec] = make_int2(i % J.w, i / J.w);
    pt += tt;
    pc += tc;
  }
}

// antiAdaptImage (lib/adaptSimple.h:110-168) for every finished request: the
// synthesized colours into its uploaded image (the other bytes never change).
__global__ void k_writeback(const SetupJob* jobs) {
  const SetupJob& J = jobs[blockIdx.y];
  if (!J.writeBack) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < J.w * J.h; i += gridDim.x * blockDim.x) {
    const int x = i % J.w, y = i / J.w;
    uint8_t* o = const_cast<uint8_t*>(J.img) + (size_t)y * J.imgRow + (size_t)x * J.bpp;
    const uint32_t w = J.tpx[i];
    for (int k = 0; k < J.nc; k++) o[k] = (uint8_t)(w >> (8 * (k + 1)));
  }
}

}  // namespace
}  // namespace rs

extern "C" int rs_setup_chunks(int npx) { return std::max(1, blocks_for(npx, kChunk)); }
extern "C" size_t rs_setup_work_ints(int totalChunks, int njobs) { return 4 * (size_t)totalChunks + 2 * (size_t)njobs; }

extern "C" cudaError_t rs_setup_multi(const SetupJob* dJobs, const int* dChunk0, int njobs, int totalChunks, int maxPx,
                                      int* counts, int* work, cudaStream_t s) {
  if (njobs < 1) return cudaSuccess;
  int* cntT = work;
  int* cntC = work + totalChunks;
  int* offT = work + 2 * (size_t)totalChunks;
  int* offC = work + 3 * (size_t)totalChunks + njobs;
  cudaMemsetAsync(counts, 0, 4 * (size_t)njobs * sizeof(int), s);
  const int bx = std::max(1, std::min(blocks_for(maxPx, 256), 256));
  k_setup_pixels<<<dim3(bx, njobs), 256, 0, s>>>(dJobs, counts);
  k_setup_count<<<totalChunks, kThreads, 0, s>>>(dJobs, dChunk0, njobs, cntT, cntC);
  k_setup_scan<<<njobs, kThreads, 0, s>>>(dChunk0, cntT, cntC, offT, offC, counts);
  k_setup_compact<<<totalChunks, kThreads, 0, s>>>(dJobs, dChunk0, njobs, offT, offC);
  return cudaGetLastError();
}

extern "C" cudaError_t rs_writeback_multi(const SetupJob* dJobs, int njobs, int maxPx, cudaStream_t s) {
  if (njobs < 1) return cudaSuccess;
  const int bx = std::max(1, std::min(blocks_for(maxPx, 256), 256));
  k_writeback<<<dim3(bx, njobs), 256, 0, s>>>(dJobs);
  return cudaGetLastError();
}
