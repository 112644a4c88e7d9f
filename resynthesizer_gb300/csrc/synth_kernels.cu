// synth_kernels.cu -- sm_103a kernels of the synthesis engine.
//
// Building blocks (each restating a reference routine):
//   build_patch_*    prepare_neighbors, lib/synthesize.h:189-241
//   term_cost        one neighbour term of computeBestFit, lib/synthesize.h:289-356
//   score_warp       computeBestFit over an ordered candidate list with the
//                    reference's result rule (strict-less update from UINT_MAX,
//                    lib/synthesize.h:382-399), as a lexicographic minimum of
//                    (patch sum, candidate index) -- early-out is exact because
//                    every term is non-negative.
// Kernels:
//   k_replay   one CTA visiting targets in the reference order (bit-exact
//              sequential replay of lib/synthesize.h:426-642)
//   k_wave     one wavefront batch: a warp (or a team of warps) per target
//   k_wave_multi  step b of many requests at once (batch b of every request)
//   k_commit   applies a batch's staged results when they cannot be stored in
//              place (refinement passes, tiled targets)
//   k_frozen   frozen-state best fit over explicit candidate lists
//   k_energy   full-patch metric at each target's source
#include <climits>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <map>
#include <mutex>

#include "../../include/resynthesizer.h"
#include "synth_internal.h"

extern "C" int rs_fail(int code, const char* msg);

namespace rs {
namespace {

constexpr unsigned kFull = 0xffffffffu;

// One patch (TNeighbor[], lib/synthesize.h:120-125) as structure of arrays:
// lanes that sit at different neighbours read different banks.
struct Patch {
  int off[kMaxNeighbors];        // (dy << 16) | (dx & 0xffff)
  uint32_t px[kMaxNeighbors];    // target pixel word
  uint32_t map[kMaxNeighbors];   // target map word
  int2 src[kMaxNeighbors];       // sourceOf of the neighbour
  int doff[kMaxNeighbors];       // dy * row stride + dx in the padded corpus (wavefront kernel)
};
// The fast scoring path reads four consecutive px / map / doff entries at once.
static_assert(offsetof(Patch, px) % 16 == 0 && offsetof(Patch, map) % 16 == 0 && offsetof(Patch, doff) % 16 == 0,
              "16-byte patch rows");

// A corpus copy in memory: pixel (x, y) is element y * stride + x + origin.
// CorpusView keeps corpus words and map words in separate arrays (the plain
// corpus; the padded corpus of problems without maps); PairView holds the
// padded corpus of problems with maps as (corpus word, map word) pairs, so a
// term is one 8-byte load.
struct CorpusView {
  const uint32_t* px;
  const uint32_t* map;
  int stride, origin;
};
struct PairView {
  const uint2* pm;
  int stride, origin;
};

template <bool MAP>
__device__ __forceinline__ void view_load(const CorpusView& v, int qi, uint32_t& s, uint32_t& m) {
  s = v.px[qi];
  m = MAP ? v.map[qi] : 0u;
}
template <bool MAP>
__device__ __forceinline__ void view_load(const PairView& v, int qi, uint32_t& s, uint32_t& m) {
  const uint2 w = v.pm[qi];
  s = w.x;
  m = w.y;
}
__device__ __forceinline__ uint32_t view_px(const CorpusView& v, int qi) { return v.px[qi]; }
__device__ __forceinline__ uint32_t view_px(const PairView& v, int qi) { return v.pm[qi].x; }

__device__ __forceinline__ int pack_off(int dx, int dy) { return (int)((unsigned)dy << 16 | ((unsigned)dx & 0xffffu)); }
__device__ __forceinline__ int off_dx(int o) { return (int)(short)(o & 0xffff); }
__device__ __forceinline__ int off_dy(int o) { return o >> 16; }

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long w = __shfl_xor_sync(kFull, v, o);
    v = w < v ? w : v;
  }
  return v;
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

// lib/synthesize.h:81-113: wrap into the target when tiling, else clip.
__device__ __forceinline__ bool wrap_or_clip(const Problem& pb, int& x, int& y) {
  if (x < 0 || x >= pb.tw) {
    if (!pb.tileH) return false;
    x %= pb.tw;
    if (x < 0) x += pb.tw;
  }
  if (y < 0 || y >= pb.th) {
    if (!pb.tileV) return false;
    y %= pb.th;
    if (y < 0) y += pb.th;
  }
  return true;
}

__device__ __forceinline__ void load_nb(const Problem& pb, Patch& P, int slot, int off, int qi) {
  P.off[slot] = off;
  P.src[slot] = pb.src[qi];
  P.px[slot] = pb.tpx[qi];
  P.map[slot] = pb.tmap ? pb.tmap[qi] : 0u;
}

// prepare_neighbors for one target with one warp: the target itself first,
// then the nearest sorted offsets whose point lies in (or wraps into) the
// target image and has a value, until the patch limit.  Returns the count.
// At most maxOffsets entries of the offset list are examined.
__device__ int build_patch_warp(const Problem& pb, int px, int py, Patch& P, int lane, int visCur = 0,
                                int maxOffsets = INT_MAX) {
  if (lane == 0) load_nb(pb, P, 0, 0, py * pb.tw + px);
  int count = 1;
  const int limit = pb.patchLimit;
  const int noffs = min(pb.noffs, maxOffsets);
  for (int base = 1; base < noffs && count < limit; base += 32) {
    const int j = base + lane;
    bool ok = false;
    int qi = 0;
    int2 o = make_int2(0, 0);
    if (j < noffs) {
      o = __ldg(&pb.offs[j]);
      int qx = px + o.x, qy = py + o.y;
      // the shared wavefront list spans every box: keep this box's offsets
      if (abs(o.x) < pb.boxW && abs(o.y) < pb.boxH && wrap_or_clip(pb, qx, qy)) {
        qi = qy * pb.tw + qx;
        ok = pb.vis ? pb.vis[qi] < visCur : pb.has[qi] != 0;
      }
    }
    const unsigned m = __ballot_sync(kFull, ok);
    const int slot = count + __popc(m & lanemask_lt());
    if (ok && slot < limit) load_nb(pb, P, slot, pack_off(o.x, o.y), qi);
    count = min(limit, count + __popc(m));
  }
  __syncwarp();
  return count;
}

// The lim (<= 64) smallest keys a warp has seen, ascending, in registers:
// lane i holds entries i (lo) and 32 + i (hi), entries from cnt on are
// kNoKey; thr is the lim-th smallest once the list is full (else kNoKey).
// An insertion is a few shuffles and two votes, with no shared-memory round
// trip.
constexpr uint32_t kNoKey = 0xFFFFFFFFu;
struct WarpTopK {
  uint32_t lo = kNoKey, hi = kNoKey, thr = kNoKey;
  int cnt = 0;
  // Inserts the key each lane holds (kNoKey: none).
  __device__ __forceinline__ void insert(uint32_t key, int lim, int lane) {
    unsigned m = __ballot_sync(kFull, key < thr);
    while (m) {
      const int srcLane = __ffs(m) - 1;
      m &= m - 1;
      const uint32_t k = __shfl_sync(kFull, key, srcLane);
      if (k >= thr) continue;
      const uint32_t loUp = __shfl_up_sync(kFull, lo, 1), hiUp = __shfl_up_sync(kFull, hi, 1);
      const uint32_t lo31 = __shfl_sync(kFull, lo, 31);
      const int pos = __popc(__ballot_sync(kFull, lo < k)) + __popc(__ballot_sync(kFull, hi < k));
      // entry e moves to e + 1 from pos on; k takes entry pos; entries past lim drop
      if (lane > pos) lo = loUp;
      else if (lane == pos) lo = k;
      if (32 + lane > pos) hi = lane == 0 ? lo31 : hiUp;
      else if (32 + lane == pos) hi = k;
      if (lane >= lim) lo = kNoKey;
      if (32 + lane >= lim) hi = kNoKey;
      cnt = min(cnt + 1, lim);
      if (cnt == lim) thr = __shfl_sync(kFull, lim <= 32 ? lo : hi, (lim - 1) & 31);
    }
  }
  // Writes the list to best[0 .. cnt).
  __device__ __forceinline__ void store(uint32_t* best, int lane) const {
    if (lane < cnt) best[lane] = lo;
    if (32 + lane < cnt) best[32 + lane] = hi;
  }
};

// Sorts four or eight keys of one lane ascending (comparator networks).
__device__ __forceinline__ void cmp_swap(uint32_t& a, uint32_t& b) {
  const uint32_t l = min(a, b);
  b = max(a, b);
  a = l;
}
__device__ __forceinline__ void sort4(uint32_t* v) {
  cmp_swap(v[0], v[1]);
  cmp_swap(v[2], v[3]);
  cmp_swap(v[0], v[2]);
  cmp_swap(v[1], v[3]);
  cmp_swap(v[1], v[2]);
}
__device__ __forceinline__ void sort8(uint32_t* v) {
  cmp_swap(v[0], v[2]);
  cmp_swap(v[1], v[3]);
  cmp_swap(v[4], v[6]);
  cmp_swap(v[5], v[7]);
  cmp_swap(v[0], v[4]);
  cmp_swap(v[1], v[5]);
  cmp_swap(v[2], v[6]);
  cmp_swap(v[3], v[7]);
  cmp_swap(v[0], v[1]);
  cmp_swap(v[2], v[3]);
  cmp_swap(v[4], v[5]);
  cmp_swap(v[6], v[7]);
  cmp_swap(v[2], v[4]);
  cmp_swap(v[3], v[5]);
  cmp_swap(v[1], v[4]);
  cmp_swap(v[3], v[6]);
  cmp_swap(v[1], v[2]);
  cmp_swap(v[3], v[4]);
  cmp_swap(v[5], v[6]);
}


// Sort key of neighbour offset (dx, dy) with d2 = dx^2 + dy^2 <= 256^2 (the
// wavefront offset radius): the sorted offset list's order -- ascending d2,
// ties by descending position in the offset box, i.e. larger dy first, then
// larger dx -- packed as d2 (17 bits), 256 - dy (10 bits: 0 .. 512), dx < 0 (1 bit).
// On one circle and row the two points differ in the sign of dx, so the key
// decodes back to (dx, dy).
__device__ __forceinline__ uint32_t offset_key(int dx, int dy, int d2) {
  return ((uint32_t)d2 << 11) | ((uint32_t)(256 - dy) << 1) | (dx < 0 ? 1u : 0u);
}
__device__ __forceinline__ int2 key_offset(uint32_t key) {
  const int d2 = (int)(key >> 11), dy = 256 - (int)((key >> 1) & 0x3FFu), a2 = d2 - dy * dy;
  int a = (int)sqrtf((float)a2);   // a2 <= 2^16 converts exactly; the root is corrected to the integer one
  if (a * a > a2) a--;
  else if ((a + 1) * (a + 1) <= a2) a++;
  return make_int2((key & 1u) ? -a : a, dy);
}

// The patch from a finished register list: self, then the listed neighbours.
__device__ int patch_from_topk(const Problem& pb, int px, int py, Patch& P, const WarpTopK& tk, int lane) {
  if (lane == 0) load_nb(pb, P, 0, 0, py * pb.tw + px);
#pragma unroll
  for (int h = 0; h < 2; h++) {
    const int i = 32 * h + lane;
    if (i < tk.cnt) {
      const int2 o = key_offset(h ? tk.hi : tk.lo);
      load_nb(pb, P, 1 + i, pack_off(o.x, o.y), (py + o.y) * pb.tw + (px + o.x));
    }
  }
  __syncwarp();
  return 1 + tk.cnt;
}

// Number of keys below k in the ascending list a[0 .. n).
__device__ __forceinline__ int keys_below(const uint32_t* a, int n, uint32_t k) {
  int lo = 0, hi = n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (a[mid] < k) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// Patch neighbours when the valued pixels are exactly list[0 .. V) and nothing
// wraps: the lim nearest in sorted-offset order, by a warp-wide insertion into
// a sorted key list instead of walking the offset list.  Part `part` of
// `parts` warps takes every parts-th run of 32 list entries; merging the
// parts' lists gives the whole list's lim smallest keys.
__device__ void sparse_keys(const Problem& pb, int px, int py, WarpTopK& tk, const int2* list, int V, int lane,
                            int part, int parts) {
  constexpr int kU = 4;   // list loads per lane in flight
  const int lim = pb.patchLimit - 1;
  const int bw = pb.boxW, bh = pb.boxH;
  for (int base = part * 32; base < V; base += 32 * parts * kU) {
    uint32_t key[kU];
#pragma unroll
    for (int u = 0; u < kU; u++) {
      const int j = base + 32 * parts * u + lane;
      key[u] = kNoKey;
      if (j < V) {
        const int2 q = list[j];
        const int dx = q.x - px, dy = q.y - py;
        if (dx > -bw && dx < bw && dy > -bh && dy < bh) {
          const long long d2 = (long long)dx * dx + (long long)dy * dy;
          if (d2 <= pb.maxD2) key[u] = offset_key(dx, dy, (int)d2);
        }
      }
    }
    // each lane's keys in ascending order: the first insertions fill the
    // list with small keys, so later ones are mostly turned away by thr
    static_assert(kU == 4, "four keys per lane");
    sort4(key);
#pragma unroll
    for (int u = 0; u < kU; u++) tk.insert(key[u], lim, lane);
  }
}

// Patch neighbours of a pass-0 target from the cell grid (no wrapping): the
// pixels with a value in sorted-offset order, found by visiting the kCell x
// kCell cells in rings of growing distance, skipping cells where no pixel
// has a value yet (least visit stamp) or that lie beyond the list's current
// last entry.  Same neighbours as walking the offset list; cheap when the
// nearest values are far away (deep inside a hole).
__device__ void grid_keys(const Problem& pb, int px, int py, WarpTopK& tk, int lane, int visCur) {
  const int lim = pb.patchLimit - 1;
  const int bw = pb.boxW, bh = pb.boxH;
  const int cx = px >> kCellShift, cy = py >> kCellShift;
  const int rmax = max(max(cx, pb.cellsW - 1 - cx), max(cy, pb.cellsH - 1 - cy));
  for (int R = 0; R <= rmax; R++) {
    if (R >= 1) {
      // every pixel of ring R is at least (R - 1) * kCell + 1 away on one axis
      const long long dmin = (long long)(R - 1) * kCell + 1;
      if (dmin * dmin > pb.maxD2 || (dmin >= bw && dmin >= bh)) break;
      if (tk.cnt == lim && dmin * dmin > (long long)(tk.thr >> 11)) break;
    }
    const int ncell = R == 0 ? 1 : 8 * R;
    for (int c0 = 0; c0 < ncell; c0 += 32) {
      const int ci = c0 + lane;
      bool want = false;
      int qcx = cx, qcy = cy;
      if (ci < ncell) {
        if (R > 0) {
          const int side = ci / (2 * R), o = ci - side * 2 * R;
          if (side == 0) {
            qcx = cx - R + o;
            qcy = cy - R;
          } else if (side == 1) {
            qcx = cx + R;
            qcy = cy - R + o;
          } else if (side == 2) {
            qcx = cx + R - o;
            qcy = cy + R;
          } else {
            qcx = cx - R;
            qcy = cy + R - o;
          }
        }
        if (qcx >= 0 && qcy >= 0 && qcx < pb.cellsW && qcy < pb.cellsH &&
            pb.cellMin[qcy * pb.cellsW + qcx] < visCur) {
          const int x0 = qcx << kCellShift, y0 = qcy << kCellShift;
          const int ddx = max(0, max(x0 - px, px - (x0 + kCell - 1)));
          const int ddy = max(0, max(y0 - py, py - (y0 + kCell - 1)));
          const long long d2 = (long long)ddx * ddx + (long long)ddy * ddy;
          want = d2 <= pb.maxD2 && ddx < bw && ddy < bh && (tk.cnt < lim || d2 <= (long long)(tk.thr >> 11));
        }
      }
      unsigned wm = __ballot_sync(kFull, want);
      // Four wanted cells per warp pass: lanes 8g .. 8g+7 read the eight rows
      // of cell g, eight pixels each, all loads in flight at once.
      static_assert(kCell == 8, "8 x 8 cells");
      const int g = lane >> 3, row = lane & 7;
      while (wm) {
        int src = -1;
#pragma unroll
        for (int t = 0; t < 4; t++) {
          if (wm) {
            if (t == g) src = __ffs(wm) - 1;
            wm &= wm - 1;
          }
        }
        const int scx = __shfl_sync(kFull, qcx, src < 0 ? 0 : src), scy = __shfl_sync(kFull, qcy, src < 0 ? 0 : src);
        const int qy = (scy << kCellShift) + row, dy = qy - py;
        uint32_t key[kCell];
#pragma unroll
        for (int j = 0; j < kCell; j++) {
          const int qx = (scx << kCellShift) + j, dx = qx - px;
          key[j] = kNoKey;
          if (src >= 0 && qx < pb.tw && qy < pb.th && dx > -bw && dx < bw && dy > -bh && dy < bh) {
            const long long d2 = (long long)dx * dx + (long long)dy * dy;
            if (d2 <= pb.maxD2 && pb.vis[qy * pb.tw + qx] < visCur) key[j] = offset_key(dx, dy, (int)d2);
          }
        }
        // each lane's row in ascending key order (see sparse_keys)
        sort8(key);
#pragma unroll
        for (int j = 0; j < kCell; j++) tk.insert(key[j], lim, lane);
      }
    }
  }
}

// One warp: the whole grid search.
__device__ int build_patch_grid(const Problem& pb, int px, int py, Patch& P, int lane, int visCur) {
  WarpTopK tk;
  grid_keys(pb, px, py, tk, lane, visCur);
  return patch_from_topk(pb, px, py, P, tk, lane);
}

// Offsets walked before a pass-0 patch falls back to the cell grid.
constexpr int kScanCap = 512;


// One neighbour term of computeBestFit for candidate (cx, cy): the clip/mask
// penalty, or the colour terms (skipped for the target itself) plus the map
// terms.  Branch-free: an out-of-range point reads word 0 and is discarded.
// The metric tables are symmetric (they are functions of d * d, and negation
// is exact), so ct/mt here are their upper halves, indexed by |t - s|: one
// SIMD absolute difference gives every channel's index at once.
template <int NC, bool MAP, class V>
__device__ __forceinline__ uint32_t term_at(const V& cv, const uint32_t* ct, const uint32_t* mt, int qi,
                                            bool inb, uint32_t t, uint32_t tm, int nm, uint32_t clip, bool self) {
  uint32_t s, sm;
  view_load<MAP>(cv, qi, s, sm);
  const uint32_t ad = __vabsdiffu4(t, s);
  uint32_t sum = ct[(ad >> 8) & 0xFFu];
  if (NC >= 2) sum += ct[(ad >> 16) & 0xFFu];
  if (NC >= 3) sum += ct[ad >> 24];
  if (self) sum = 0;
  if (MAP) {
    const uint32_t am = __vabsdiffu4(tm, sm);
    for (int c = 0; c < nm; c++) sum += mt[(am >> (8 * c)) & 0xFFu];
  }
  return (inb && (s & 0xFFu) == 0xFFu) ? sum : clip;
}

template <int NC, bool MAP, class V>
__device__ __forceinline__ uint32_t term_cost(const Problem& pb, const V& cv, const uint32_t* ct,
                                              const uint32_t* mt, int cx, int cy, int off, uint32_t t, uint32_t tm,
                                              bool self) {
  const int qx = cx + off_dx(off), qy = cy + off_dy(off);
  const bool inb = (unsigned)qx < (unsigned)pb.cw && (unsigned)qy < (unsigned)pb.ch;
  const int qi = inb ? qy * cv.stride + qx + cv.origin : cv.origin;
  return term_at<NC, MAP>(cv, ct, mt, qi, inb, t, tm, pb.nm, pb.clipCost, self);
}

// Loads the upper halves (|d| = 0..255) of the metric tables into shared memory.
__device__ __forceinline__ void load_half_tables(const Problem& pb, uint32_t* ct, uint32_t* mt) {
  for (int i = threadIdx.x; i < 256; i += blockDim.x) {
    ct[i] = pb.ctab[256 + i];
    mt[i] = pb.mtab[256 + i];
  }
}

__device__ __forceinline__ CorpusView plain_view(const Problem& pb) { return CorpusView{pb.cpx, pb.cmap, pb.cw, 0}; }

// Full patch metric, one thread, stopping once the sum reaches stopAt.  The
// check comes after every G terms, whose loads then overlap (a ragged last
// group recomputes the final term and adds zero for it): a sum that would have
// stopped earlier only grows by non-negative terms, so it still reaches
// stopAt, and a complete sum is the same -- the caller's decision (sum < best,
// sum == 0) does not change.
template <int NC, bool MAP, int G = 8>
__device__ uint32_t patch_sum(const Problem& pb, const CorpusView& cv, const uint32_t* ct, const uint32_t* mt,
                              int cx, int cy, const Patch& P, int n, uint32_t stopAt, unsigned& terms) {
  uint32_t sum = 0;
  for (int i = 0; i < n; i += G) {
    uint32_t g = 0;
#pragma unroll
    for (int u = 0; u < G; u++) {
      const int k = min(i + u, n - 1);
      const uint32_t v =
          term_cost<NC, MAP>(pb, cv, ct, mt, cx, cy, P.off[k], P.px[k], MAP ? P.map[k] : 0u, i + u == 0);
      g += i + u < n ? v : 0u;
    }
    sum += g;
    terms += (unsigned)min(G, n - i);
    if (sum >= stopAt) break;
  }
  return sum;
}

// Scores candidates 0..ncand-1 (get(k) -> corpus point) against the patch
// P[0..n) with one warp.  Each lane owns one candidate at a time and takes a
// new one as soon as its current candidate is finished or can no longer win;
// the result is the lexicographic minimum of (sum, k), i.e. the first strict
// minimum in list order, exactly what a sequential computeBestFit loop keeps.
// bestIdx == INT_MAX when ncand == 0.  Warp-uniform outputs.
// FAST: every candidate is a corpus point and every patch offset lies within
// kPad, so with the padded view each term is one load at a precomputed
// linear offset (the masked border supplies the clip penalty).
template <int NC, bool MAP, bool FAST, class V, class Get>
__device__ void score_warp(const Problem& pb, const V& cv, const uint32_t* ct, const uint32_t* mt,
                           const Patch& P, int n, int ncand, Get get, int lane, uint32_t& bestVal, int& bestIdx,
                           unsigned& terms, unsigned& evals) {
  bestVal = 0xFFFFFFFFu;
  bestIdx = INT_MAX;
  int k = lane;
  int2 c = make_int2(0, 0);
  int cb = 0;
  if (k < ncand) {
    c = get(k);
    cb = c.y * cv.stride + c.x + cv.origin;
    evals++;
  }
  auto term = [&](int ii) -> uint32_t {
    if (FAST) return term_at<NC, MAP>(cv, ct, mt, cb + P.doff[ii], true, P.px[ii], MAP ? P.map[ii] : 0u, pb.nm,
                                      pb.clipCost, ii == 0);
    return term_cost<NC, MAP>(pb, cv, ct, mt, c.x, c.y, P.off[ii], P.px[ii], MAP ? P.map[ii] : 0u, ii == 0);
  };
  uint32_t sum = 0;
  int i = 0;
  int next = 32;
  while (__any_sync(kFull, k < ncand)) {
    const bool active = k < ncand;
    if (active) {
      uint32_t add = 0;
      if (FAST && i + 4 <= n) {
        // i is a multiple of 4 here: the patch entries of four terms come
        // in one 16-byte load per array
        const int4 d4 = *reinterpret_cast<const int4*>(&P.doff[i]);
        const uint4 p4 = *reinterpret_cast<const uint4*>(&P.px[i]);
        uint4 m4 = make_uint4(0, 0, 0, 0);
        if (MAP) m4 = *reinterpret_cast<const uint4*>(&P.map[i]);
        add = term_at<NC, MAP>(cv, ct, mt, cb + d4.x, true, p4.x, m4.x, pb.nm, pb.clipCost, i == 0) +
              term_at<NC, MAP>(cv, ct, mt, cb + d4.y, true, p4.y, m4.y, pb.nm, pb.clipCost, false) +
              term_at<NC, MAP>(cv, ct, mt, cb + d4.z, true, p4.z, m4.z, pb.nm, pb.clipCost, false) +
              term_at<NC, MAP>(cv, ct, mt, cb + d4.w, true, p4.w, m4.w, pb.nm, pb.clipCost, false);
      } else if (i + 4 <= n) {
#pragma unroll
        for (int u = 0; u < 4; u++) add += term(i + u);
      } else {
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const uint32_t v = term(min(i + u, n - 1));
          add += (i + u < n) ? v : 0u;
        }
      }
      sum += add;
      i += min(4, n - i);
    }
    // (sum, k) against the best (value, index) so far, as one 64-bit key
    const unsigned long long mine = ((unsigned long long)sum << 32) | (unsigned)k;
    const bool done = active && i >= n;
    const bool fin = done && mine < (((unsigned long long)bestVal << 32) | (unsigned)bestIdx);
    if (__ballot_sync(kFull, fin)) {
      // every finished key is below the best, so their minimum replaces it
      const unsigned long long key = warp_min_u64(fin ? mine : ~0ull);
      bestVal = (uint32_t)(key >> 32);
      bestIdx = (int)(key & 0xffffffffu);
    }
    // A lane stops when finished or when its partial sum can no longer win
    // (sums only grow; a tie wins only with the lower index).
    const bool lost = active && !done && mine > (((unsigned long long)bestVal << 32) | (unsigned)bestIdx);
    const bool need = done || lost;
    const unsigned nm = __ballot_sync(kFull, need);
    if (need) {
      terms += (unsigned)i;
      k = next + __popc(nm & lanemask_lt());
      // After a perfect match no later candidate can win.
      if (bestVal == 0u) k = INT_MAX;
      sum = 0;
      i = 0;
      if (k < ncand) {
        c = get(k);
        cb = c.y * cv.stride + c.x + cv.origin;
        evals++;
      }
    }
    next += __popc(nm);
  }
}

__device__ __forceinline__ uint32_t mix32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x85ebca6bu;
  x ^= x >> 13;
  x *= 0xc2b2ae35u;
  x ^= x >> 16;
  return x;
}

// Counter-based probe draws: a base key per (seed, pass, target pixel), one
// hash per probe.  A uniform corpus point comes straight from the corpus
// rectangle when every pixel is a corpus point (x from the hash's high half,
// y from its low half rotated up), else through the corpus point list.
__device__ __forceinline__ uint32_t probe_base(uint32_t seed, uint32_t pass, uint32_t pix) {
  return mix32(seed ^ mix32(pass * 0x9E3779B9u + 0x7f4a7c15u) ^ (pix * 0x85EBCA77u));
}
__device__ __forceinline__ int2 probe_point(const Problem& pb, uint32_t base, uint32_t j) {
  const uint32_t h = mix32(base + j * 0x9E3779B9u);
  if (pb.fullCorpus)
    return make_int2((int)__umulhi(h, (uint32_t)pb.cw), (int)__umulhi(__funnelshift_l(h, h, 16), (uint32_t)pb.ch));
  return __ldg(&pb.cpts[__umulhi(h, (uint32_t)pb.ncorpus)]);
}

template <class V>
__device__ __forceinline__ bool corpus_ok(const Problem& pb, const V& cv, int2 c) {
  return (unsigned)c.x < (unsigned)pb.cw && (unsigned)c.y < (unsigned)pb.ch &&
         (view_px(cv, c.y * cv.stride + c.x + cv.origin) & 0xFFu) == 0xFFu;
}

// The padded corpus view of a problem (kPad-wide masked border).
template <bool MAP>
__device__ __forceinline__ auto padded_view(const Problem& pb) {
  if constexpr (MAP) return PairView{pb.cpmPad, pb.padW, kPad * pb.padW + kPad};
  else return CorpusView{pb.cpxPad, nullptr, pb.padW, kPad * pb.padW + kPad};
}

// ----------------------------------------------------------- shared memory

__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

// Bulk (TMA) copy global -> shared, completion counted on an mbarrier.
__device__ __forceinline__ void mbar_init(uint64_t* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)));
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned phase) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(phase)
      : "memory");
  return ok != 0;
}

// Stages `words` 32-bit words (a multiple of 4, 16-byte aligned source) into
// shared memory with bulk copies.  Returns false if the wait ran out.
__device__ bool stage_words(uint32_t* dst, const uint32_t* src, unsigned words, uint64_t* bar) {
  if (threadIdx.x == 0) {
    mbar_init(bar);
    mbar_expect_tx(bar, words * 4u);
    const unsigned chunk = 16384;  // words per copy (64 KB)
    for (unsigned w = 0; w < words; w += chunk) {
      const unsigned cnt = min(chunk, words - w);
      bulk_g2s(dst + w, src + w, cnt * 4u, bar);
    }
  }
  __syncthreads();
  bool ok = false;
  for (int it = 0; it < (1 << 22); it++) {
    if (mbar_try_wait(bar, 0)) {
      ok = true;
      break;
    }
    __nanosleep(64);
  }
  // Every thread's wait is bounded; the CTA acts on one shared verdict.
  return __syncthreads_and(ok) != 0;
}

// ------------------------------------------------------------------ frozen

template <int NC, bool MAP>
__global__ void __launch_bounds__(256) k_frozen(ScoreArgs a) {
  __shared__ uint32_t ct[kTable], mt[kTable];
  __shared__ Patch patches[8];
  load_half_tables(a.pb, ct, mt);
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = gridDim.x * (blockDim.x >> 5);
  Patch& P = patches[warp];
  for (int t = blockIdx.x * (blockDim.x >> 5) + warp; t < a.n; t += nw) {
    const int2 pos = a.targets[t];
    const int n = build_patch_warp(a.pb, pos.x, pos.y, P, lane);
    const unsigned c0 = a.candStart[t];
    const int ncand = (int)(a.candStart[t + 1] - c0);
    uint32_t bv;
    int bi;
    unsigned terms = 0, evals = 0;
    score_warp<NC, MAP, false>(a.pb, plain_view(a.pb), ct, mt, P, n, ncand,
                               [&](int k) { return a.cands[c0 + k]; }, lane, bv, bi, terms, evals);
    if (lane == 0) {
      a.outSum[t] = bv;
      a.outPt[t] = bi == INT_MAX ? make_int2(-1, -1) : a.cands[c0 + bi];
      a.outCount[t] = (unsigned)n;
    }
    __syncwarp();
  }
}

// ------------------------------------------------------------------ energy

template <int NC, bool MAP>
__global__ void __launch_bounds__(256) k_energy(ScoreArgs a) {
  __shared__ uint32_t ct[kTable], mt[kTable];
  __shared__ Patch patches[8];
  load_half_tables(a.pb, ct, mt);
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = gridDim.x * (blockDim.x >> 5);
  Patch& P = patches[warp];
  unsigned long long acc = 0;
  for (int t = blockIdx.x * (blockDim.x >> 5) + warp; t < a.n; t += nw) {
    const int2 pos = a.targets[t];
    const int n = build_patch_warp(a.pb, pos.x, pos.y, P, lane);
    const int2 s = a.pb.src[pos.y * a.pb.tw + pos.x];
    unsigned long long v = 0;
    for (int i = lane; i < n; i += 32)
      v += term_cost<NC, MAP>(a.pb, plain_view(a.pb), ct, mt, s.x, s.y, P.off[i], P.px[i], MAP ? P.map[i] : 0u,
                              i == 0);
    v = warp_sum_u64(v);
    if (lane == 0) {
      if (a.outSum) a.outSum[t] = (uint32_t)v;
      acc += v;
    }
    __syncwarp();
  }
  if (lane == 0 && acc) atomicAdd(a.energy, acc);
}

// ------------------------------------------------------------------ replay

__device__ __forceinline__ unsigned long long block_min_u64(unsigned long long v, unsigned long long* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  v = warp_min_u64(v);
  if (lane == 0) red[warp] = v;
  __syncthreads();
  unsigned long long r = lane < nw ? red[lane] : ~0ull;
  r = warp_min_u64(r);
  __syncthreads();
  return r;
}

// Visits targets[t0 .. t1) one after another, exactly as the single-threaded
// reference (lib/synthesize.h:472-641), with the whole CTA working on each
// visit: the patch scan, heuristic-1 candidates (continuations of the
// neighbours' sources, minus those this target already probed, recorded in
// recentProber), the random probes drawn from the reference's PRNG stream,
// and the store.
template <int NC, bool MAP>
__global__ void __launch_bounds__(256, 1) k_replay(ReplayArgs a, int t0, int t1) {
  __shared__ uint32_t ct[kTable], mt[kTable];
  __shared__ Patch P;
  __shared__ int2 hl[kMaxNeighbors];
  __shared__ int2 rpt[256];
  __shared__ unsigned long long red[8];
  __shared__ int wcnt[8];
  __shared__ int s_nh;
  __shared__ unsigned s_cursor;
  const Problem& pb = a.pb;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  load_half_tables(pb, ct, mt);
  if (tid == 0) s_cursor = a.ctr->cursor;
  __syncthreads();
  unsigned cursor = s_cursor;
  unsigned betters = 0, terms = 0;
  unsigned long long refEvals = 0, evals = 0;
  const unsigned div = 2147483647u / (unsigned)pb.ncorpus + 1u;   // lib/glibProxy.c:48

  for (int t = t0; t < t1; t++) {
    const int2 pos = a.targets[t];
    const int pi = pos.y * pb.tw + pos.x;
    // 1. patch (prepare_neighbors) with the whole block scanning offsets.
    if (tid == 0) load_nb(pb, P, 0, 0, pi);
    int count = 1;
    for (int base = 1; base < pb.noffs && count < pb.patchLimit; base += blockDim.x) {
      const int j = base + tid;
      bool ok = false;
      int qi = 0;
      int2 o = make_int2(0, 0);
      if (j < pb.noffs) {
        o = pb.offs[j];
        int qx = pos.x + o.x, qy = pos.y + o.y;
        if (wrap_or_clip(pb, qx, qy)) {
          qi = qy * pb.tw + qx;
          ok = pb.has[qi] != 0;
        }
      }
      const unsigned m = __ballot_sync(kFull, ok);
      if (lane == 0) wcnt[warp] = __popc(m);
      __syncthreads();
      int before = 0, total = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
        total += wcnt[w];
        if (w < warp) before += wcnt[w];
      }
      const int slot = count + before + __popc(m & lanemask_lt());
      if (ok && slot < pb.patchLimit) load_nb(pb, P, slot, pack_off(o.x, o.y), qi);
      count = min(pb.patchLimit, count + total);
      __syncthreads();
    }
    __syncthreads();
    // 2. heuristic-1 list (warp 0): first occurrences, in neighbour order, of
    //    in-corpus continuations not already probed by this target index.
    if (warp == 0) {
      int nh = 0;
      for (int r = 0; r < count; r += 32) {
        const int k = r + lane;
        bool valid = false;
        int2 c = make_int2(0, 0);
        if (k < count && P.src[k].x != -1) {
          c = make_int2(P.src[k].x - off_dx(P.off[k]), P.src[k].y - off_dy(P.off[k]));
          // corpus mask and recentProber are loaded together (no short circuit)
          const bool inb = (unsigned)c.x < (unsigned)pb.cw && (unsigned)c.y < (unsigned)pb.ch;
          const int ci = inb ? c.y * pb.cw + c.x : 0;
          const uint32_t cpx = pb.cpx[ci];
          const unsigned prober = a.recentProber[ci];
          valid = inb && (cpx & 0xFFu) == 0xFFu && prober != (unsigned)t;
        }
        const unsigned long long key =
            valid ? ((unsigned long long)(unsigned)c.y << 32 | (unsigned)c.x) : (~0ull - (unsigned)lane);
        const unsigned peers = __match_any_sync(kFull, key);
        bool keep = valid && (peers & lanemask_lt()) == 0u;
        for (int e = 0; e < nh && keep; e++)
          if (hl[e].x == c.x && hl[e].y == c.y) keep = false;
        const unsigned km = __ballot_sync(kFull, keep);
        if (keep) hl[nh + __popc(km & lanemask_lt())] = c;
        nh += __popc(km);
        __syncwarp();
      }
      if (lane == 0) s_nh = nh;
    }
    __syncthreads();
    const int nh = s_nh;
    // 3. score heuristic-1 candidates (full sums) -> first strict minimum.
    unsigned long long key = ~0ull;
    if (tid < nh) {
      const uint32_t s = patch_sum<NC, MAP>(pb, plain_view(pb), ct, mt, hl[tid].x, hl[tid].y, P, count,
                                            0xFFFFFFFFu, terms);
      key = ((unsigned long long)s << 32) | (unsigned)tid;
    }
    key = block_min_u64(key, red);
    uint32_t bestVal = (uint32_t)(key >> 32);
    int bestIdx = nh > 0 ? (int)(key & 0xffffffffu) : -1;
    int2 bestPt = nh > 0 ? hl[bestIdx] : make_int2(0, 0);
    const bool perfectH = nh > 0 && bestVal == 0u;
    // recentProber is written for every evaluated candidate before a perfect one.
    const int evaluatedH = perfectH ? bestIdx + 1 : nh;
    if (tid < (perfectH ? bestIdx : nh)) a.recentProber[hl[tid].y * pb.cw + hl[tid].x] = (unsigned)t;
    refEvals += (unsigned)evaluatedH;
    evals += (unsigned)nh;
    if (nh == 0) bestVal = 0xFFFFFFFFu;
    // 4. random probes from the reference PRNG stream.
    unsigned draws = 0;
    if (!perfectH) {
      for (unsigned j0 = 0; j0 < a.trys; j0 += blockDim.x) {
        const unsigned j = j0 + tid;
        unsigned long long rk = ~0ull;
        if (j < a.trys) {
          const unsigned pos_ = cursor + j;
          const int r = pos_ < a.randCount ? a.randStream[pos_] : 0;
          if (pos_ >= a.randCount) atomicOr(&a.ctr->error, 2u);
          const int2 c = pb.cpts[(unsigned)r / div];
          rpt[tid] = c;
          const uint32_t s = patch_sum<NC, MAP>(pb, plain_view(pb), ct, mt, c.x, c.y, P, count, bestVal, terms);
          evals++;
          if (s < bestVal) rk = ((unsigned long long)s << 32) | j;
        }
        rk = block_min_u64(rk, red);
        const unsigned chunkN = min((unsigned)blockDim.x, a.trys - j0);
        if (rk != ~0ull) {
          bestVal = (uint32_t)(rk >> 32);
          bestPt = rpt[(unsigned)(rk & 0xffffffffu) - j0];
          bestIdx = 1;
        }
        __syncthreads();  // rpt reuse
        if (rk != ~0ull && bestVal == 0u) {
          draws += (unsigned)(rk & 0xffffffffu) - j0 + 1u;
          break;
        }
        draws += chunkN;
      }
    }
    cursor += draws;
    refEvals += draws;
    // 5. store (only a better, different source), then setHasValue.
    if (tid == 0) {
      const bool bettered = nh > 0 || draws > 0;
      const int2 cur = pb.src[pi];
      if (bettered && (cur.x != bestPt.x || cur.y != bestPt.y)) {
        betters++;
        const uint32_t s = pb.cpx[bestPt.y * pb.cw + bestPt.x];
        pb.tpx[pi] = (pb.tpx[pi] & 0xFFu) | (s & 0xFFFFFF00u);
        pb.src[pi] = bestPt;
      }
      pb.has[pi] = 1;
    }
    __syncthreads();
  }
  // statistics
  unsigned long long tsum = warp_sum_u64(terms);
  if (lane == 0) atomicAdd(&a.ctr->terms, tsum);
  if (tid == 0) {
    a.ctr->cursor = cursor;
    a.ctr->betters += betters;
    a.ctr->refEvals += refEvals;
    a.ctr->evals += evals;
  }
}

// --------------------------------------------------------------- wavefront

// Per-warp shared memory of k_wave: the patch, then one 512-byte area that
// holds the sparse top list while the patch is built and the continuation
// candidates afterwards.
struct WaveSmem {
  static constexpr int kPerWarp = (int)sizeof(Patch) + kMaxNeighbors * (int)sizeof(unsigned long long);
  static constexpr int kHead = 2 * 256 * 4 + 16;   // half tables + two mbarriers
};
static_assert(WaveSmem::kHead % 16 == 0 && WaveSmem::kPerWarp % 16 == 0, "16-byte aligned warp regions");

// Shared memory and team layout of one CTA of the wavefront kernels: warps
// form teams of G (a power of two); a team's patch and candidate list live in
// its first warp's region.
struct WaveTeam {
  int G, team, tw, lead, lane, warp;
  unsigned char* regions;        // per-warp regions (WaveSmem::kPerWarp each)
  unsigned long long* sKey;      // [16]
  int *sN, *sNp, *sFast, *sGather;   // [16] each
  __device__ __forceinline__ void sync() const {
    if (G == 1) __syncwarp();
    else asm volatile("bar.sync %0, %1;" ::"r"(1 + team), "r"(G * 32) : "memory");
  }
  __device__ __forceinline__ unsigned char* region(int w) const { return regions + w * WaveSmem::kPerWarp; }
};

// One target of a wavefront batch (slot `slot` of the batch starting at b0 in
// a.targets), synthesized by one team.  Candidates are the deduplicated
// in-corpus continuations of the patch's sources, then (with a proposal
// network) the network's proposals, then `trys` counter-based random probes;
// the best (first strict minimum) different source is stored in place, or
// staged for k_commit.  Returns 1 if the target's source changed (in place).
template <int NC, bool MAP, class V>
__device__ __forceinline__ unsigned wave_target(const WaveArgs& a, const Problem& pb, const V& cv,
                                                const uint32_t* ct, const uint32_t* mt, int batch, int visCur,
                                                int b0, int slot, bool sparse, const WaveTeam& T, unsigned& terms,
                                                unsigned& evals) {
  const int G = T.G, tw = T.tw, lead = T.lead, lane = T.lane, warp = T.warp;
  unsigned char* wbase = T.region(lead);
  Patch& P = *reinterpret_cast<Patch*>(wbase);
  int2* prop = reinterpret_cast<int2*>(wbase + sizeof(Patch));   // continuation candidates
  const int t = b0 + slot;
  const int2 pos = a.targets[t];
  const int pi = pos.y * pb.tw + pos.x;
  // The patch.  While the valued pixels are a short list, every warp of the
  // team collects the nearest keys of its share of the list and the lead
  // merges them; otherwise the lead walks the offset list, falling back to
  // the cell grid when the nearest values lie beyond the walk's reach.
  int nPatch = 0;
  if (sparse) {
    WarpTopK tk;
    sparse_keys(pb, pos.x, pos.y, tk, a.targets, b0, lane, tw, G);
    if (G > 1) {
      // Every warp's list goes to its top-list area.  A key's rank in the
      // union is its index in its own list plus the keys below it in the
      // others (keys are distinct, one per pixel); the keys of rank below
      // lim land in the second warp's patch area (unused by the team).
      const int lim = pb.patchLimit - 1;
      auto list = [&](int w) { return reinterpret_cast<const uint32_t*>(T.region(lead + w) + sizeof(Patch)); };
      uint32_t* merged = reinterpret_cast<uint32_t*>(T.region(lead + 1));
      tk.store(reinterpret_cast<uint32_t*>(T.region(warp) + sizeof(Patch)), lane);
      if (lane == 0) T.sGather[warp] = tk.cnt;
      T.sync();
      int total = 0;
      for (int w = 0; w < G; w++) total += T.sGather[lead + w];
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int i = 32 * h + lane;
        if (i < tk.cnt) {
          const uint32_t k = h ? tk.hi : tk.lo;
          int rank = i;
          for (int w = 0; w < G; w++)
            if (w != tw) rank += keys_below(list(w), T.sGather[lead + w], k);
          if (rank < lim) merged[rank] = k;
        }
      }
      T.sync();
      if (tw == 0) {
        tk.cnt = min(total, lim);
        tk.lo = lane < tk.cnt ? merged[lane] : kNoKey;
        tk.hi = 32 + lane < tk.cnt ? merged[32 + lane] : kNoKey;
      }
    }
    if (tw == 0) nPatch = patch_from_topk(pb, pos.x, pos.y, P, tk, lane);
  } else if (tw == 0) {
    nPatch = build_patch_warp(pb, pos.x, pos.y, P, lane, visCur, pb.cellMin ? kScanCap : INT_MAX);
    if (pb.cellMin && nPatch < pb.patchLimit && kScanCap < pb.noffs)
      nPatch = build_patch_grid(pb, pos.x, pos.y, P, lane, visCur);
  }
  if (tw == 0) {
    const int n = nPatch;
    // linear offsets into the padded corpus; the fast path needs all within kPad
    int far = 0;
    for (int i = lane; i < n; i += 32) {
      const int dx = off_dx(P.off[i]), dy = off_dy(P.off[i]);
      P.doff[i] = dy * pb.padW + dx;
      far |= (abs(dx) > kPad) | (abs(dy) > kPad);
    }
    far = __any_sync(kFull, far);
    // continuation candidates, deduplicated, in neighbour order
    int np = 0;
    for (int r = 0; r < n; r += 32) {
      const int k = r + lane;
      bool valid = false;
      int2 c = make_int2(0, 0);
      if (k < n && P.src[k].x >= 0) {
        c = make_int2(P.src[k].x - off_dx(P.off[k]), P.src[k].y - off_dy(P.off[k]));
        valid = corpus_ok(pb, cv, c);
      }
      const unsigned long long key =
          valid ? ((unsigned long long)(unsigned)c.y << 32 | (unsigned)c.x) : (~0ull - (unsigned)lane);
      const unsigned peers = __match_any_sync(kFull, key);
      bool keep = valid && (peers & lanemask_lt()) == 0u;
      for (int e = 0; e < np && keep; e++)
        if (prop[e].x == c.x && prop[e].y == c.y) keep = false;
      const unsigned km = __ballot_sync(kFull, keep);
      if (keep) prop[np + __popc(km & lanemask_lt())] = c;
      np += __popc(km);
      __syncwarp();
    }
    if (lane == 0) {
      T.sN[lead] = n;
      T.sNp[lead] = np;
      T.sFast[lead] = !far;
    }
  }
  T.sync();
  const int n = T.sN[lead], np = T.sNp[lead];
  const bool fast = T.sFast[lead] != 0;
  // Candidates: continuations, then the network's proposals (an invalid
  // one is replaced by an extra probe), then the random probes.
  const int nprop = a.props ? a.nprop : 0;
  const int ncand = np + nprop + (int)a.trys;
  // Probe keys: per target pixel, or shared by 16 consecutive slots of the
  // batch (neighbours in the target list, which the batches keep in order):
  // the warps of a CTA then read the same random corpus windows, which stay
  // in L1/L2 when the corpus itself is too large to.
  const uint32_t pbase = a.probeShare
                             ? probe_base(a.seed ^ 0x6A09E667u, a.pass, (uint32_t)batch * 0x01000193u + ((uint32_t)slot >> 4))
                             : probe_base(a.seed, a.pass, (uint32_t)pi);
  const int2* myProps = nprop ? a.props + (size_t)(t - a.batchStart[a.propBatch0]) * 16 : nullptr;
  auto cand = [&](int k) -> int2 {
    if (k < np) return prop[k];
    if (k < np + nprop) {
      const int2 c = myProps[k - np];
      return corpus_ok(pb, cv, c) ? c : probe_point(pb, pbase, a.trys + (uint32_t)(k - np));
    }
    return probe_point(pb, pbase, (uint32_t)(k - np - nprop));
  };
  // Warp tw of the team scores candidates tw, tw + G, tw + 2G, ...
  const int nloc = ncand > tw ? (ncand - tw + G - 1) / G : 0;
  uint32_t bv;
  int bi;
  auto get = [&](int j) { return cand(tw + j * G); };
  if (fast)
    score_warp<NC, MAP, true>(pb, cv, ct, mt, P, n, nloc, get, lane, bv, bi, terms, evals);
  else
    score_warp<NC, MAP, false>(pb, cv, ct, mt, P, n, nloc, get, lane, bv, bi, terms, evals);
  if (lane == 0) T.sKey[warp] = bi == INT_MAX ? ~0ull : ((unsigned long long)bv << 32) | (unsigned)(tw + bi * G);
  T.sync();
  unsigned better = 0;
  if (tw == 0 && lane == 0) {
    unsigned long long best = ~0ull;
    for (int w = 0; w < G; w++) best = min(best, T.sKey[lead + w]);
    int2 out = make_int2(-2, -2);
    if (best != ~0ull) {
      const int k = (int)(best & 0xffffffffu);
      const int2 pt = cand(k);
      const int2 cur = pb.src[pi];
      if (cur.x != pt.x || cur.y != pt.y) out = pt;
    }
    if (a.inPlace) {
      // No target of this batch reads another's state (visit stamps, colour
      // phases), so the store (setColor + setSourceOf) happens right here.
      if (out.x != -2) {
        const uint32_t c = pb.cpx[out.y * pb.cw + out.x];
        pb.tpx[pi] = (pb.tpx[pi] & 0xFFu) | (c & 0xFFFFFF00u);
        pb.src[pi] = out;
        better = 1;
      }
    } else {
      a.stageSrc[slot] = out;
    }
  }
  T.sync();
  return better;
}

// Team size: when the step has fewer targets than the grid has warps, G warps
// (a power of two, at most the CTA) share one target's candidates.  The result
// does not depend on G: every team reduces to the same (sum, candidate index)
// minimum.
__device__ __forceinline__ int team_size(int nslots) {
  const int wpb = blockDim.x >> 5;
  int G = 1;
  while (G < wpb && (long long)nslots * (G * 2) <= (long long)gridDim.x * wpb) G *= 2;
  return G;
}

// One wavefront batch of one problem: a team of warps per target.
template <int NC, bool MAP, bool SMEMC>
__global__ void __launch_bounds__(512, 2) k_wave(WaveArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int b0 = a.batchStart[a.batch], b1 = a.batchStart[a.batch + 1];
  const int nslots = b1 - b0;
  const int wpb = blockDim.x >> 5;
  const int G = team_size(nslots);
  const int teamsPerBlock = wpb / G;
  // CTAs beyond this batch's size leave before staging anything.
  if ((int)(blockIdx.x * teamsPerBlock) >= nslots) return;
  uint32_t* ct = reinterpret_cast<uint32_t*>(smem);
  uint32_t* mt = ct + 256;
  uint64_t* bar = reinterpret_cast<uint64_t*>(mt + 256);
  unsigned char* p = smem + WaveSmem::kHead;
  const Problem& pb = a.pb;
  // The padded corpus: staged into shared memory when it fits.
  const int padH = pb.ch + 2 * kPad;
  auto cv = padded_view<MAP>(pb);
  const unsigned cwords = ((unsigned)(pb.padW * padH) + 3u) & ~3u;
  if (SMEMC) {
    bool ok;
    if constexpr (MAP) {
      uint2* scpm = reinterpret_cast<uint2*>(p);
      p += cwords * 8;
      ok = stage_words(reinterpret_cast<uint32_t*>(scpm), reinterpret_cast<const uint32_t*>(pb.cpmPad), cwords * 2,
                       bar);
      cv.pm = scpm;
    } else {
      uint32_t* scpx = reinterpret_cast<uint32_t*>(p);
      p += cwords * 4;
      ok = stage_words(scpx, pb.cpxPad, cwords, bar);
      cv.px = scpx;
    }
    if (!ok) {
      if (threadIdx.x == 0) atomicOr(&a.ctr->error, 1u);
      return;
    }
  }
  __shared__ int s_abort;
  load_half_tables(pb, ct, mt);
  // One read of the host-mapped flag per CTA, so the whole CTA agrees.
  if (threadIdx.x == 0) s_abort = *a.abortFlag;
  __syncthreads();
  if (s_abort) return;
  __shared__ unsigned long long s_key[16];
  __shared__ int s_n[16], s_np[16], s_fast[16], s_gather[16];
  __shared__ unsigned s_better;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int team = warp / G;
  const WaveTeam T{G, team, warp % G, team * G, lane, warp, p, s_key, s_n, s_np, s_fast, s_gather};
  if (threadIdx.x == 0) s_better = 0;
  __syncthreads();
  const bool sparse = a.sparse && (long long)b0 * b0 < a.sparseLimit2;
  unsigned terms = 0, evals = 0;
  for (int slot = blockIdx.x * teamsPerBlock + team; slot < nslots; slot += gridDim.x * teamsPerBlock) {
    const unsigned better =
        wave_target<NC, MAP>(a, pb, cv, ct, mt, a.batch, a.visCur, b0, slot, sparse, T, terms, evals);
    if (better) atomicAdd(&s_better, 1u);
  }
  __syncthreads();
  if (threadIdx.x == 0 && s_better) atomicAdd(&a.ctr->betters, s_better);
  unsigned long long tv = warp_sum_u64(terms), ev = warp_sum_u64(evals);
  if (lane == 0) {
    atomicAdd(&a.ctr->terms, tv);
    atomicAdd(&a.ctr->evals, ev);
  }
}

// ------------------------------------------------ persistent wavefront pass

// A poll that neither caches the line in L1 nor invalidates L1 (an acquire
// load would, on every poll, taking the L1 away from a working CTA on the
// same SM); the acquire fence comes once, after the value changed.
__device__ __forceinline__ unsigned ld_relaxed_gpu(const unsigned* p) {
  unsigned v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void fence_acq_rel_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Barrier across every CTA of a cooperative launch, on a counter that only
// grows: thread 0 of each CTA publishes the CTA's writes (fence), adds its
// arrival without waiting for the result, and polls until the count reaches
// k * CTAs for the CTA's k-th barrier -- no CTA has to act for the others, so
// the release is one L2 round trip after the last arrival.  A CTA that must
// stop the run (the host's cancel flag, a failed copy) asks, between two
// barriers, for everyone to leave at the next one (request_stop): all CTAs
// then leave at the same barrier.  A wait gives up after timeoutNs of global
// time: the CTA records kErrBarrier and leaves, so a CTA that never arrives
// makes every other CTA leave at its next barrier instead of spinning
// forever.  nbar counts the CTA's barriers.  Returns true when the CTA must
// leave.
__device__ __forceinline__ void request_stop(GridBar* gb, unsigned nbar) {
  atomicMax(&gb->stopInv, ~(nbar + 1u));
}

__device__ bool grid_barrier(GridBar* gb, unsigned& nbar, unsigned* err, long long timeoutNs) {
  __shared__ unsigned s_stop;
  __syncthreads();
  const unsigned k = ++nbar;
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(&gb->count, 1u);
    const unsigned target = k * gridDim.x;
    const unsigned long long t0 = global_ns();
    bool late = false;
    unsigned nap = 32;
    while ((int)(ld_relaxed_gpu(&gb->count) - target) < 0) {
      if ((long long)(global_ns() - t0) > timeoutNs) {
        late = true;
        break;
      }
      __nanosleep(nap);
      if (nap < 256) nap <<= 1;
    }
    fence_acq_rel_gpu();
    unsigned stop = 1u;
    if (late) {
      atomicOr(err, kErrBarrier);
    } else {
      const unsigned inv = *(volatile unsigned*)&gb->stopInv;
      stop = (inv != 0u && ~inv <= k) ? 1u : 0u;
    }
    s_stop = stop;
  }
  __syncthreads();
  return s_stop != 0u;
}

// Applies the staged results of batch `batch` (grid-stride over its slots);
// returns how many of this thread's slots changed source.
__device__ __forceinline__ unsigned commit_batch(const WaveArgs& a, int batch) {
  const Problem& pb = a.pb;
  const int b0 = a.batchStart[batch];
  const int nslots = a.batchStart[batch + 1] - b0;
  unsigned better = 0;
  for (int slot = blockIdx.x * blockDim.x + threadIdx.x; slot < nslots; slot += gridDim.x * blockDim.x) {
    const int2 pos = a.targets[b0 + slot];
    const int pi = pos.y * pb.tw + pos.x;
    const int2 s = a.stageSrc[slot];
    if (s.x != -2) {
      const uint32_t c = pb.cpx[s.y * pb.cw + s.x];
      pb.tpx[pi] = (pb.tpx[pi] & 0xFFu) | (c & 0xFFFFFF00u);
      pb.src[pi] = s;
      better++;
    }
    if (!pb.vis) pb.has[pi] = 1;
  }
  return better;
}

// Batches a.batch .. a.batchEnd - 1 of one pass in one launch: the corpus is
// staged into shared memory once, each batch runs as in k_wave (a team of
// warps per target, sized to the batch), then every CTA meets at a grid
// barrier before the next batch reads the state; staged passes apply their
// results between two barriers.  The outputs are those of one k_wave (+
// k_commit) launch per batch: the same targets, in the same batches, see the
// same state.  Needs a cooperative launch (every CTA resident).
template <int NC, bool MAP, bool SMEMC>
__global__ void __launch_bounds__(512, 2) k_wave_persistent(WaveArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  uint32_t* ct = reinterpret_cast<uint32_t*>(smem);
  uint32_t* mt = ct + 256;
  uint64_t* bar = reinterpret_cast<uint64_t*>(mt + 256);
  unsigned char* p = smem + WaveSmem::kHead;
  const Problem& pb = a.pb;
  const int padH = pb.ch + 2 * kPad;
  auto cv = padded_view<MAP>(pb);
  const unsigned cwords = ((unsigned)(pb.padW * padH) + 3u) & ~3u;
  bool ok = true;
  if (SMEMC) {
    if constexpr (MAP) {
      uint2* scpm = reinterpret_cast<uint2*>(p);
      p += cwords * 8;
      ok = stage_words(reinterpret_cast<uint32_t*>(scpm), reinterpret_cast<const uint32_t*>(pb.cpmPad), cwords * 2,
                       bar);
      cv.pm = scpm;
    } else {
      uint32_t* scpx = reinterpret_cast<uint32_t*>(p);
      p += cwords * 4;
      ok = stage_words(scpx, pb.cpxPad, cwords, bar);
      cv.px = scpx;
    }
    // A CTA whose copy failed does no work but still meets the first barrier,
    // where every CTA leaves.
    if (!ok && threadIdx.x == 0) {
      atomicOr(&a.ctr->error, kErrStage);
      request_stop(a.gbar, 0);
    }
  }
  load_half_tables(pb, ct, mt);
  __shared__ unsigned long long s_key[16];
  __shared__ int s_n[16], s_np[16], s_fast[16], s_gather[16], s_item[16];
  __shared__ unsigned s_better;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  if (threadIdx.x == 0) s_better = 0;
  __syncthreads();
  unsigned terms = 0, evals = 0, committed = 0, nbar = 0;
  for (int b = a.batch; b < a.batchEnd; b++) {
    const int b0 = a.batchStart[b];
    const int nslots = a.batchStart[b + 1] - b0;
    // An empty batch changes nothing: every CTA reads the same boundaries, so
    // all of them skip its barriers together.
    if (nslots == 0) continue;
    // The host's cancel flag (host memory, slow to read) is read by one
    // thread while the batch runs; it stops the run at the batch's end.
    if (blockIdx.x == 0 && threadIdx.x == 0 && *a.abortFlag) request_stop(a.gbar, nbar);
    if (ok) {
      const int G = team_size(nslots);
      const int teamsPerBlock = wpb / G;
      const int team = warp / G;
      const WaveTeam T{G, team, warp % G, team * G, lane, warp, p, s_key, s_n, s_np, s_fast, s_gather};
      const bool sparse = a.sparse && (long long)b0 * b0 < a.sparseLimit2;
      const int visCur = a.pass == 0 ? b : 0x7ffffffe;
      // Part of the batch in fixed shares -- the teams of a CTA take
      // neighbouring slots, whose patches overlap in L1 and, with probes
      // shared by groups of 16 slots, whose probes read the same corpus
      // windows -- then the rest handed out one slot at a time from the
      // batch's queue, so that the batch ends when its last target does
      // rather than when the team with the slowest share does.  Measured
      // (CUDA events): with shared probes three quarters fixed (heal4096
      // 22.8 -> 21.9 ms, mapstyle2048 95.0 -> 86.3 ms against fixed shares
      // only; half fixed 22.3 and 87.9 ms), with a staged corpus half fixed
      // (render1024 9.29 -> 8.96 ms against three quarters; a quarter or
      // three eighths the same, seven eighths 9.68 ms).  One call site of
      // wave_target: the kernel's code stays the size of one target's work.
      const int stride = gridDim.x * teamsPerBlock;
      const int fixedEnd = a.queue ? (a.probeShare ? nslots * 3 / 4 : nslots / 2) / stride * stride : nslots;
      int slot = blockIdx.x * teamsPerBlock + team;
      bool fixed = slot < fixedEnd;
      if (!fixed && fixedEnd < nslots) {
        if (T.tw == 0 && lane == 0) s_item[team] = fixedEnd + (int)atomicAdd(&a.queue[b], 1u);
        T.sync();
        slot = s_item[team];
      }
      while (slot < nslots) {
        const unsigned better = wave_target<NC, MAP>(a, pb, cv, ct, mt, b, visCur, b0, slot, sparse, T, terms, evals);
        if (better) atomicAdd(&s_better, 1u);
        if (fixed) {
          slot += stride;
          fixed = slot < fixedEnd;
          if (fixed || fixedEnd >= nslots) continue;
        }
        if (T.tw == 0 && lane == 0) s_item[team] = fixedEnd + (int)atomicAdd(&a.queue[b], 1u);
        T.sync();
        slot = s_item[team];
      }
    }
    if (!a.inPlace) {
      if (grid_barrier(a.gbar, nbar, &a.ctr->error, a.barTimeoutNs)) break;
      committed += commit_batch(a, b);
    }
    if (grid_barrier(a.gbar, nbar, &a.ctr->error, a.barTimeoutNs)) break;
  }
  for (int o = 16; o > 0; o >>= 1) committed += __shfl_xor_sync(kFull, committed, o);
  if (lane == 0 && committed) atomicAdd(&s_better, committed);
  __syncthreads();
  if (threadIdx.x == 0 && s_better) atomicAdd(&a.ctr->betters, s_better);
  const unsigned long long tv = warp_sum_u64(terms), ev = warp_sum_u64(evals);
  if (lane == 0) {
    atomicAdd(&a.ctr->terms, tv);
    atomicAdd(&a.ctr->evals, ev);
  }
}

// Test kernel of the grid barrier: every CTA but CTA `absent` meets `rounds`
// barriers; CTA `absent` (when in range) leaves at once, so the others' waits
// must run out.
__global__ void k_barrier_probe(GridBar* gb, unsigned* err, int rounds, int absent, long long timeoutNs,
                                unsigned* passed) {
  if ((int)blockIdx.x == absent) return;
  unsigned nbar = 0;
  for (int r = 0; r < rounds; r++) {
    if (grid_barrier(gb, nbar, err, timeoutNs)) return;
    if (threadIdx.x == 0) atomicAdd(passed, 1u);
  }
}

// The request of global slot gs: prefix[r] <= gs < prefix[r + 1].
__device__ __forceinline__ int multi_request(const int* prefix, int nreq, int gs) {
  int lo = 0, hi = nreq - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (prefix[mid] <= gs) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Step `step` of a pass for many problems at once: batch `step` of every
// request with that many batches, the requests' slots concatenated through
// `prefix` (exclusive, prefix[nreq] = total).  Corpora and tables are read
// from global memory; per-request counters take the sums.
template <int NC, bool MAP>
__global__ void __launch_bounds__(512, 2) k_wave_multi(const WaveArgs* jobs, int nreq, const int* prefix, int step,
                                                       int visCur, const volatile int* abortFlag) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int total = prefix[nreq];
  const int wpb = blockDim.x >> 5;
  const int G = team_size(total);
  const int teamsPerBlock = wpb / G;
  if ((int)(blockIdx.x * teamsPerBlock) >= total) return;
  __shared__ int s_abort;
  if (threadIdx.x == 0) s_abort = *abortFlag;
  __shared__ unsigned long long s_key[16];
  __shared__ int s_n[16], s_np[16], s_fast[16], s_gather[16];
  __syncthreads();
  if (s_abort) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int team = warp / G;
  const WaveTeam T{G, team, warp % G, team * G, lane, warp, smem + WaveSmem::kHead, s_key, s_n, s_np, s_fast,
                   s_gather};
  for (int gs = blockIdx.x * teamsPerBlock + team; gs < total; gs += gridDim.x * teamsPerBlock) {
    const int r = multi_request(prefix, nreq, gs);
    const WaveArgs& a = jobs[r];
    const Problem& pb = a.pb;
    const auto cv = padded_view<MAP>(pb);
    const int b0 = a.batchStart[step];
    const bool sparse = a.sparse && (long long)b0 * b0 < a.sparseLimit2;
    unsigned terms = 0, evals = 0;
    const unsigned better = wave_target<NC, MAP>(a, pb, cv, pb.ctab + 256, pb.mtab + 256, step, visCur, b0,
                                                 gs - prefix[r], sparse, T, terms, evals);
    if (better) atomicAdd(&a.ctr->betters, 1u);
    const unsigned long long tv = warp_sum_u64(terms), ev = warp_sum_u64(evals);
    if (lane == 0) {
      atomicAdd(&a.ctr->terms, tv);
      atomicAdd(&a.ctr->evals, ev);
    }
  }
}

// A pass of many problems in one launch: steps 0 .. steps - 1, step b being
// batch b of every request that has one.  prefix[b * (nreq + 1) + r] is the
// first slot of request r in step b (prefix[... + nreq] = the step's total).
// Work per step: three quarters of the step's slots in fixed shares (a CTA's
// teams on neighbouring slots, mostly of one request, whose patches and
// shared probes meet in L1), then the rest through a queue per step
// (queue[b], zeroed by the host): a team takes the next slot as soon as it
// finishes one, so requests of uneven cost share the GPU evenly and the step
// ends with its last target.  A grid barrier closes each step (and,
// when some request stages its results, a commit phase between two
// barriers).  Results equal one k_wave_multi (+ k_commit_multi) launch per
// step.  Needs a cooperative launch.
template <int NC, bool MAP>
__global__ void __launch_bounds__(512, 2) k_wave_multi_persistent(const WaveArgs* jobs, int nreq, int steps,
                                                                  const int* prefix, unsigned* queue, int pass,
                                                                  int staged, GridBar* gb,
                                                                  const volatile int* abortFlag, unsigned* err,
                                                                  long long timeoutNs) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int wpb = blockDim.x >> 5;
  int* sPrefix = reinterpret_cast<int*>(smem + WaveSmem::kHead + wpb * WaveSmem::kPerWarp);
  __shared__ unsigned long long s_key[16];
  __shared__ int s_n[16], s_np[16], s_fast[16], s_gather[16], s_item[16];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned nbar = 0;
  for (int b = 0; b < steps; b++) {
    const int* pre = prefix + (size_t)b * (nreq + 1);
    const int total = pre[nreq];
    if (total == 0) continue;   // the same for every CTA: no barrier needed
    if (blockIdx.x == 0 && threadIdx.x == 0 && *abortFlag) request_stop(gb, nbar);
    for (int r = threadIdx.x; r <= nreq; r += blockDim.x) sPrefix[r] = pre[r];
    __syncthreads();
    const int G = team_size(total);
    const int team = warp / G;
    const WaveTeam T{G, team, warp % G, team * G, lane, warp, smem + WaveSmem::kHead, s_key, s_n, s_np, s_fast,
                     s_gather};
    const int visCur = pass == 0 ? b : 0x7ffffffe;
    const int stride = gridDim.x * (wpb / G);
    const int fixedEnd = (total * 3 / 4) / stride * stride;
    int gs = blockIdx.x * (wpb / G) + team;
    if (gs >= fixedEnd) {
      if (T.tw == 0 && lane == 0) s_item[team] = fixedEnd + (int)atomicAdd(&queue[b], 1u);
      T.sync();
      gs = s_item[team];
    }
    while (gs < total) {
      const bool fixedNext = gs + stride < fixedEnd;
      int nxt = 0;
      if (!fixedNext && T.tw == 0 && lane == 0)
        nxt = fixedEnd + (int)atomicAdd(&queue[b], 1u);   // in flight while this slot runs
      const int r = multi_request(sPrefix, nreq, gs);
      const WaveArgs& a = jobs[r];
      const Problem& pb = a.pb;
      const auto cv = padded_view<MAP>(pb);
      const int b0 = a.batchStart[b];
      const bool sparse = a.sparse && (long long)b0 * b0 < a.sparseLimit2;
      unsigned terms = 0, evals = 0;
      const unsigned better = wave_target<NC, MAP>(a, pb, cv, pb.ctab + 256, pb.mtab + 256, b, visCur, b0,
                                                   gs - sPrefix[r], sparse, T, terms, evals);
      if (better) atomicAdd(&a.ctr->betters, 1u);
      const unsigned long long tv = warp_sum_u64(terms), ev = warp_sum_u64(evals);
      if (lane == 0) {
        atomicAdd(&a.ctr->terms, tv);
        atomicAdd(&a.ctr->evals, ev);
      }
      if (fixedNext) {
        gs += stride;
        continue;
      }
      if (T.tw == 0 && lane == 0) s_item[team] = nxt;
      T.sync();
      gs = s_item[team];
    }
    if (staged) {
      if (grid_barrier(gb, nbar, err, timeoutNs)) return;
      for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
        const int r = multi_request(sPrefix, nreq, g);
        const WaveArgs& a = jobs[r];
        if (a.inPlace) continue;
        const Problem& pb = a.pb;
        const int slot = g - sPrefix[r];
        const int2 pos = a.targets[a.batchStart[b] + slot];
        const int pi = pos.y * pb.tw + pos.x;
        const int2 s = a.stageSrc[slot];
        if (s.x != -2) {
          const uint32_t c = pb.cpx[s.y * pb.cw + s.x];
          pb.tpx[pi] = (pb.tpx[pi] & 0xFFu) | (c & 0xFFFFFF00u);
          pb.src[pi] = s;
          atomicAdd(&a.ctr->betters, 1u);
        }
      }
    }
    if (grid_barrier(gb, nbar, err, timeoutNs)) return;
  }
}

// Every step's exclusive slot prefix over the requests: one CTA per step.
__global__ void __launch_bounds__(1024) k_multi_prefix_all(const WaveArgs* jobs, int nreq, int* prefix) {
  __shared__ int warpSums[32];
  __shared__ int carry;
  const int step = blockIdx.x;
  int* out = prefix + (size_t)step * (nreq + 1);
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int base = 0; base < nreq; base += 1024) {
    const int r = base + threadIdx.x;
    int v = 0;
    if (r < nreq && step < jobs[r].nbatches) v = jobs[r].batchStart[step + 1] - jobs[r].batchStart[step];
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warpSums[warp] = x;
    __syncthreads();
    if (warp == 0) {
      int w = warpSums[lane];
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += y;
      }
      warpSums[lane] = w;
    }
    __syncthreads();
    if (r < nreq) out[r] = carry + (warp ? warpSums[warp - 1] : 0) + x - v;
    __syncthreads();
    if (threadIdx.x == 0) carry += warpSums[31];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[nreq] = carry;
}

// Slot counts of step `step` for every request (0 past its last batch or when
// inactive) and their exclusive prefix; one CTA of 1024 threads.
__global__ void __launch_bounds__(1024) k_multi_prefix(const WaveArgs* jobs, int nreq, int step, int* prefix) {
  __shared__ int warpSums[32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int base = 0; base < nreq; base += 1024) {
    const int r = base + threadIdx.x;
    int v = 0;
    if (r < nreq && step < jobs[r].nbatches) v = jobs[r].batchStart[step + 1] - jobs[r].batchStart[step];
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warpSums[warp] = x;
    __syncthreads();
    if (warp == 0) {
      int w = warpSums[lane];
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += y;
      }
      warpSums[lane] = w;
    }
    __syncthreads();
    if (r < nreq) prefix[r] = carry + (warp ? warpSums[warp - 1] : 0) + x - v;
    __syncthreads();
    if (threadIdx.x == 0) carry += warpSums[31];
    __syncthreads();
  }
  if (threadIdx.x == 0) prefix[nreq] = carry;
}

// Staged results of step `step` for many problems.
__global__ void k_commit_multi(const WaveArgs* jobs, int nreq, const int* prefix, int step) {
  const int total = prefix[nreq];
  for (int gs = blockIdx.x * blockDim.x + threadIdx.x; gs < total; gs += gridDim.x * blockDim.x) {
    const int r = multi_request(prefix, nreq, gs);
    const WaveArgs& a = jobs[r];
    if (a.inPlace) continue;
    const Problem& pb = a.pb;
    const int slot = gs - prefix[r];
    const int2 pos = a.targets[a.batchStart[step] + slot];
    const int pi = pos.y * pb.tw + pos.x;
    const int2 s = a.stageSrc[slot];
    if (s.x != -2) {
      const uint32_t c = pb.cpx[s.y * pb.cw + s.x];
      pb.tpx[pi] = (pb.tpx[pi] & 0xFFu) | (c & 0xFFFFFF00u);
      pb.src[pi] = s;
      atomicAdd(&a.ctr->betters, 1u);
    }
  }
}

__global__ void k_commit(WaveArgs a) {
  const Problem& pb = a.pb;
  // An aborted batch may be partly staged: apply none of it (one read per CTA).
  __shared__ int s_abort;
  if (threadIdx.x == 0) s_abort = *a.abortFlag;
  __syncthreads();
  const int b0 = a.batchStart[a.batch];
  const int nslots = s_abort ? 0 : a.batchStart[a.batch + 1] - b0;
  unsigned better = 0;
  for (int slot = blockIdx.x * blockDim.x + threadIdx.x; slot < nslots; slot += gridDim.x * blockDim.x) {
    const int2 pos = a.targets[b0 + slot];
    const int pi = pos.y * pb.tw + pos.x;
    const int2 s = a.stageSrc[slot];
    if (s.x != -2) {
      const uint32_t c = pb.cpx[s.y * pb.cw + s.x];
      pb.tpx[pi] = (pb.tpx[pi] & 0xFFu) | (c & 0xFFFFFF00u);
      pb.src[pi] = s;
      better++;
    }
    if (!pb.vis) pb.has[pi] = 1;
  }
  for (int o = 16; o > 0; o >>= 1) better += __shfl_xor_sync(kFull, better, o);
  if ((threadIdx.x & 31) == 0 && better) atomicAdd(&a.ctr->betters, better);
}

// ---------------------------------------------------------- pack / unpack

__global__ void k_pack(const uint8_t* raw, int npx, int bpp, int colorStart, int nc, int mapStart, int nm,
                       uint32_t* px, uint32_t* map) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < npx; i += gridDim.x * blockDim.x) {
    const uint8_t* q = raw + (size_t)i * bpp;
    uint32_t w = q[0];
    for (int c = 0; c < nc; c++) w |= (uint32_t)q[colorStart + c] << (8 * (c + 1));
    px[i] = w;
    if (map) {
      uint32_t m = 0;
      for (int c = 0; c < nm; c++) m |= (uint32_t)q[mapStart + c] << (8 * c);
      map[i] = m;
    }
  }
}

// The corpus with a kPad-wide border of zero (masked) words.
__global__ void k_pack_padded(const uint8_t* raw, int w, int h, int bpp, int nc, int mapStart, int nm,
                              uint32_t* px, uint2* pm) {
  const int pw = w + 2 * kPad, ph = h + 2 * kPad;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < pw * ph; i += gridDim.x * blockDim.x) {
    const int x = i % pw - kPad, y = i / pw - kPad;
    uint32_t word = 0, m = 0;
    if (x >= 0 && x < w && y >= 0 && y < h) {
      const uint8_t* q = raw + ((size_t)y * w + x) * bpp;
      word = q[0];
      for (int c = 0; c < nc; c++) word |= (uint32_t)q[1 + c] << (8 * (c + 1));
      for (int c = 0; c < nm; c++) m |= (uint32_t)q[mapStart + c] << (8 * c);
    }
    px[i] = word;
    if (pm) pm[i] = make_uint2(word, m);
  }
}

__global__ void k_unpack_colors(uint8_t* raw, int npx, int bpp, int nc, const uint32_t* px) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < npx; i += gridDim.x * blockDim.x) {
    uint8_t* q = raw + (size_t)i * bpp;
    const uint32_t w = px[i];
    for (int c = 0; c < nc; c++) q[1 + c] = (uint8_t)(w >> (8 * (c + 1)));
  }
}

int grid_for(int n, int perBlock, int maxBlocks) {
  int g = (n + perBlock - 1) / perBlock;
  return g < 1 ? 1 : (g > maxBlocks ? maxBlocks : g);
}

int sm_count() {
  static const int n = [] {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    return v > 0 ? v : 1;
  }();
  return n;
}

}  // namespace
}  // namespace rs

using namespace rs;

#define RS_DISPATCH(NCV, MAPV, CALL)                                       \
  do {                                                                     \
    if ((NCV) == 1) {                                                      \
      if (MAPV) { constexpr int NC = 1; constexpr bool MAP = true; CALL; } \
      else { constexpr int NC = 1; constexpr bool MAP = false; CALL; }     \
    } else if ((NCV) == 2) {                                               \
      if (MAPV) { constexpr int NC = 2; constexpr bool MAP = true; CALL; } \
      else { constexpr int NC = 2; constexpr bool MAP = false; CALL; }     \
    } else {                                                               \
      if (MAPV) { constexpr int NC = 3; constexpr bool MAP = true; CALL; } \
      else { constexpr int NC = 3; constexpr bool MAP = false; CALL; }     \
    }                                                                      \
  } while (0)

extern "C" cudaError_t rs_launch_pack(const uint8_t* raw, int w, int h, int bpp, int colorStart, int nc,
                                      int mapStart, int nm, uint32_t* px, uint32_t* map, cudaStream_t s) {
  const int n = w * h;
  k_pack<<<grid_for(n, 256, sm_count() * 8), 256, 0, s>>>(raw, n, bpp, colorStart, nc, mapStart, nm, px, map);
  return cudaGetLastError();
}

extern "C" cudaError_t rs_launch_pack_padded(const uint8_t* raw, int w, int h, int bpp, int nc, int mapStart,
                                             int nm, uint32_t* px, uint2* pm, cudaStream_t s) {
  const int n = (w + 2 * kPad) * (h + 2 * kPad);
  k_pack_padded<<<grid_for(n, 256, sm_count() * 8), 256, 0, s>>>(raw, w, h, bpp, nc, mapStart, nm, px, pm);
  return cudaGetLastError();
}

extern "C" cudaError_t rs_launch_unpack_colors(uint8_t* raw, int w, int h, int bpp, int nc, const uint32_t* px,
                                               cudaStream_t s) {
  const int n = w * h;
  k_unpack_colors<<<grid_for(n, 256, sm_count() * 8), 256, 0, s>>>(raw, n, bpp, nc, px);
  return cudaGetLastError();
}

extern "C" cudaError_t rs_launch_replay(const ReplayArgs& a, int t0, int t1, cudaStream_t s) {
  RS_DISPATCH(a.pb.nc, a.pb.nm > 0, (k_replay<NC, MAP><<<1, 256, 0, s>>>(a, t0, t1)));
  return cudaGetLastError();
}

extern "C" cudaError_t rs_launch_frozen(const ScoreArgs& a, cudaStream_t s) {
  RS_DISPATCH(a.pb.nc, a.pb.nm > 0, (k_frozen<NC, MAP><<<grid_for(a.n, 8, sm_count() * 8), 256, 0, s>>>(a)));
  return cudaGetLastError();
}

extern "C" cudaError_t rs_launch_energy(const ScoreArgs& a, cudaStream_t s) {
  RS_DISPATCH(a.pb.nc, a.pb.nm > 0, (k_energy<NC, MAP><<<grid_for(a.n, 8, sm_count() * 8), 256, 0, s>>>(a)));
  return cudaGetLastError();
}

// The pass-0 patch of each listed target (pixels with vis < visCur have a
// value) by the offset-list walk or by the cell grid: neighbour offsets in
// patch order, self excluded.  Checks that both builders agree.
__global__ void __launch_bounds__(256) k_patches(Problem pb, const int2* targets, int n, int visCur, int useGrid,
                                                 int* outOff, int* outCount) {
  __shared__ Patch sp[8];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int t = blockIdx.x * 8 + w; t < n; t += gridDim.x * 8) {
    const int2 pos = targets[t];
    const int cnt = useGrid ? build_patch_grid(pb, pos.x, pos.y, sp[w], lane, visCur)
                            : build_patch_warp(pb, pos.x, pos.y, sp[w], lane, visCur);
    for (int i = 1 + lane; i < cnt; i += 32) outOff[(size_t)t * kMaxNeighbors + i - 1] = sp[w].off[i];
    if (lane == 0) outCount[t] = cnt - 1;
    __syncwarp();
  }
}

extern "C" cudaError_t rs_launch_patches(const Problem& pb, const int2* targets, int n, int visCur, int useGrid,
                                         int* outOff, int* outCount, cudaStream_t s) {
  k_patches<<<grid_for(n, 8, sm_count() * 8), 256, 0, s>>>(pb, targets, n, visCur, useGrid, outOff, outCount);
  return cudaGetLastError();
}

namespace {
// Kernels that read the corpus through L1: ask for the smallest shared-memory
// carveout that keeps their occupancy, so that L1 gets the rest (heal4096 and
// mapstyle2048 about 2 % faster than with the driver's default split).  The
// hint is per kernel, so it only grows (pct: the largest asked so far, -1
// once given up): a later, smaller configuration cannot squeeze an earlier
// one.  Falls back to the default when the hint would cost a CTA per SM.
template <class K>
void prefer_l1(K kern, int threads, size_t smem, int perSm, int& pct) {
  if (pct < 0) return;
  int dev = 0, smPerSm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&smPerSm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess || smPerSm <= 0)
    return;
  const size_t need = (size_t)perSm * (smem + 2048);   // + static shared memory and the per-CTA reserve
  const int want = std::max(pct, (int)std::min<size_t>(100, (need * 100 + smPerSm - 1) / smPerSm));
  int after = 0;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, want) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&after, kern, threads, smem) != cudaSuccess || after < perSm) {
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, -1);
    pct = -1;
    return;
  }
  pct = want;
}

size_t wave_smem(const Problem& pb, bool smemc, int warps) {
  size_t b = WaveSmem::kHead;
  if (smemc) {
    const size_t cwords = ((size_t)pb.padW * (pb.ch + 2 * kPad) + 3) & ~(size_t)3;
    b += cwords * 4 * (pb.nm > 0 ? 2 : 1);
  }
  return b + (size_t)warps * WaveSmem::kPerWarp;
}

template <int NC, bool MAP, bool SMEMC>
cudaError_t launch_wave_t(const WaveArgs& a, int warps, int maxCtas, size_t smem, cudaStream_t s) {
  auto kern = k_wave<NC, MAP, SMEMC>;
  // Per-instantiation launch configuration, shared by all host threads.
  static std::mutex mu;
  static size_t configured = 0;
  static std::map<std::pair<size_t, int>, int> perSmCache;
  static int carvePct = 0;
  int perSm = 0;
  {
    std::lock_guard<std::mutex> lock(mu);
    if (smem > configured) {
      const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      configured = smem;
    }
    auto it = perSmCache.find({smem, warps});
    if (it == perSmCache.end()) {
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kern, warps * 32, smem);
      if (!SMEMC && perSm > 0) prefer_l1(kern, warps * 32, smem, perSm, carvePct);
      perSmCache[{smem, warps}] = perSm;
    } else {
      perSm = it->second;
    }
  }
  if (perSm < 1) return cudaErrorInvalidConfiguration;
  // Persistent grid (the batch size is only known on the device), capped by
  // the caller's estimate for small batches so that idle CTAs are not launched.
  int grid = sm_count() * perSm;
  if (maxCtas > 0) grid = std::min(grid, maxCtas);
  kern<<<grid, warps * 32, smem, s>>>(a);
  return cudaGetLastError();
}
}  // namespace

extern "C" cudaError_t rs_launch_wave(const WaveArgs& a, int warps, int maxCtas, cudaStream_t s) {
  if (warps < 1) warps = 16;
  if (warps > 16) warps = 16;
  const size_t smemCorpus = wave_smem(a.pb, true, warps);
  const bool smemc = smemCorpus <= 112 * 1024;   // two CTAs per SM
  const size_t smem = smemc ? smemCorpus : wave_smem(a.pb, false, warps);
  cudaError_t e = cudaSuccess;
  if (smemc) {
    RS_DISPATCH(a.pb.nc, a.pb.nm > 0, (e = launch_wave_t<NC, MAP, true>(a, warps, maxCtas, smem, s)));
  } else {
    RS_DISPATCH(a.pb.nc, a.pb.nm > 0, (e = launch_wave_t<NC, MAP, false>(a, warps, maxCtas, smem, s)));
  }
  return e;
}

namespace {
template <int NC, bool MAP, bool SMEMC>
cudaError_t launch_wave_persistent_t(const WaveArgs& a, int warps, int maxCtas, size_t smem, cudaStream_t s) {
  auto kern = k_wave_persistent<NC, MAP, SMEMC>;
  static std::mutex mu;
  static size_t configured = 0;
  static std::map<std::pair<size_t, int>, int> perSmCache;
  static int carvePct = 0;
  int perSm = 0;
  {
    std::lock_guard<std::mutex> lock(mu);
    if (smem > configured) {
      const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      configured = smem;
    }
    auto it = perSmCache.find({smem, warps});
    if (it == perSmCache.end()) {
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kern, warps * 32, smem);
      if (!SMEMC && perSm > 0) prefer_l1(kern, warps * 32, smem, perSm, carvePct);
      // the occupancy after the carveout hint is what a cooperative launch is checked against
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kern, warps * 32, smem);
      perSmCache[{smem, warps}] = perSm;
    } else {
      perSm = it->second;
    }
  }
  if (perSm < 1) return cudaErrorInvalidConfiguration;
  // One CTA per resident slot: every CTA is on the GPU at once, which the grid
  // barrier needs (the cooperative launch refuses a grid that could not be).
  WaveArgs args = a;
  void* params[] = {&args};
  int grid = sm_count() * perSm;
  if (maxCtas > 0) grid = std::min(grid, maxCtas);
  return cudaLaunchCooperativeKernel((const void*)kern, dim3(grid), dim3(warps * 32), params, smem, s);
}
}  // namespace

extern "C" cudaError_t rs_launch_wave_persistent(const WaveArgs& a, int warps, int maxCtas, cudaStream_t s) {
  if (warps < 1) warps = 16;
  if (warps > 16) warps = 16;
  const size_t smemCorpus = wave_smem(a.pb, true, warps);
  const bool smemc = smemCorpus <= 112 * 1024;   // two CTAs per SM
  const size_t smem = smemc ? smemCorpus : wave_smem(a.pb, false, warps);
  cudaError_t e = cudaSuccess;
  if (smemc) {
    RS_DISPATCH(a.pb.nc, a.pb.nm > 0, (e = launch_wave_persistent_t<NC, MAP, true>(a, warps, maxCtas, smem, s)));
  } else {
    RS_DISPATCH(a.pb.nc, a.pb.nm > 0, (e = launch_wave_persistent_t<NC, MAP, false>(a, warps, maxCtas, smem, s)));
  }
  return e;
}

extern "C" int rs_persistent_supported() {
  static const int v = [] {
    int dev = 0, c = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&c, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess) return 0;
    return c;
  }();
  return v;
}

// No counterpart in the reference.  Test entry of the grid barrier of the
// persistent kernel (declared in include/resynthesizer.h).
extern "C" __attribute__((visibility("default"))) int resynthGridBarrierProbe(int rounds, int absentCta,
                                                                               long long timeoutNs,
                                                                               unsigned* passed, unsigned* error) {
  if (!passed || !error || rounds < 0) return rs_fail(RESYNTH_ERROR_ARGUMENT, "resynthGridBarrierProbe: bad argument");
  if (!rs_persistent_supported()) return rs_fail(RESYNTH_ERROR_DEVICE, "cooperative launches not supported");
  struct Dev {
    GridBar gb;
    unsigned err, passed;
  };
  Dev* d = nullptr;
  cudaError_t e = cudaMalloc(&d, sizeof(Dev));
  if (e == cudaSuccess) e = cudaMemset(d, 0, sizeof(Dev));
  const int grid = sm_count() * 2;
  if (e == cudaSuccess) {
    GridBar* gb = &d->gb;
    unsigned* err = &d->err;
    unsigned* pass = &d->passed;
    void* params[] = {&gb, &err, &rounds, &absentCta, &timeoutNs, &pass};
    e = cudaLaunchCooperativeKernel((const void*)k_barrier_probe, dim3(grid), dim3(256), params, 0, nullptr);
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  Dev h{};
  if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(Dev), cudaMemcpyDeviceToHost);
  if (d) cudaFree(d);
  if (e != cudaSuccess) return rs_fail(RESYNTH_ERROR_DEVICE, cudaGetErrorString(e));
  *passed = h.passed;
  *error = h.err;
  return 0;
}

namespace {
template <int NC, bool MAP>
cudaError_t launch_wave_multi_t(const WaveArgs* jobs, int nreq, const int* prefix, int step, int visCur, int maxCtas,
                                const volatile int* abortFlag, cudaStream_t s) {
  auto kern = k_wave_multi<NC, MAP>;
  constexpr int warps = 16;
  const size_t smem = WaveSmem::kHead + (size_t)warps * WaveSmem::kPerWarp;
  static std::mutex mu;
  static int perSm = 0;
  {
    std::lock_guard<std::mutex> lock(mu);
    if (!perSm) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kern, warps * 32, smem);
      if (e != cudaSuccess) return e;
      int carvePct = 0;
      if (perSm > 0) prefer_l1(kern, warps * 32, smem, perSm, carvePct);
    }
  }
  if (perSm < 1) return cudaErrorInvalidConfiguration;
  int grid = sm_count() * perSm;
  if (maxCtas > 0) grid = std::min(grid, maxCtas);
  kern<<<grid, warps * 32, smem, s>>>(jobs, nreq, prefix, step, visCur, abortFlag);
  return cudaGetLastError();
}
}  // namespace

namespace {
template <int NC, bool MAP>
cudaError_t launch_wave_multi_persistent_t(const WaveArgs* jobs, int nreq, int steps, const int* prefix,
                                           unsigned* queue, int pass, int staged, GridBar* gb,
                                           const volatile int* abortFlag, long long timeoutNs, cudaStream_t s) {
  auto kern = k_wave_multi_persistent<NC, MAP>;
  constexpr int warps = 16;
  const size_t smem = WaveSmem::kHead + (size_t)warps * WaveSmem::kPerWarp + ((((size_t)nreq + 1) * 4 + 15) & ~(size_t)15);
  static std::mutex mu;
  static size_t configured = 0;
  static std::map<size_t, int> perSmCache;
  static int carvePct = 0;
  int perSm = 0;
  {
    std::lock_guard<std::mutex> lock(mu);
    if (smem > configured) {
      const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      configured = smem;
    }
    auto it = perSmCache.find(smem);
    if (it == perSmCache.end()) {
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kern, warps * 32, smem);
      if (perSm > 0) prefer_l1(kern, warps * 32, smem, perSm, carvePct);
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kern, warps * 32, smem);
      perSmCache[smem] = perSm;
    } else {
      perSm = it->second;
    }
  }
  if (perSm < 1) return cudaErrorInvalidConfiguration;
  unsigned* err = &gb->error;
  void* params[] = {(void*)&jobs, &nreq, &steps, (void*)&prefix, &queue, &pass, &staged, &gb, (void*)&abortFlag,
                    &err, &timeoutNs};
  return cudaLaunchCooperativeKernel((const void*)kern, dim3(sm_count() * perSm), dim3(warps * 32), params, smem, s);
}
}  // namespace

extern "C" cudaError_t rs_launch_wave_multi_persistent(const WaveArgs* jobs, int nreq, int steps, const int* prefix,
                                                       unsigned* queue, int pass, int staged, GridBar* gb,
                                                       const volatile int* abortFlag, int nc, int map,
                                                       long long timeoutNs, cudaStream_t s) {
  if (nreq < 1 || nreq > kMultiPersistentMaxRequests) return cudaErrorInvalidValue;
  cudaError_t e = cudaSuccess;
  RS_DISPATCH(nc, map != 0, (e = launch_wave_multi_persistent_t<NC, MAP>(jobs, nreq, steps, prefix, queue, pass,
                                                                         staged, gb, abortFlag, timeoutNs, s)));
  return e;
}

extern "C" cudaError_t rs_launch_multi_prefix_all(const WaveArgs* jobs, int nreq, int steps, int* prefix,
                                                  cudaStream_t s) {
  if (steps < 1) return cudaSuccess;
  k_multi_prefix_all<<<steps, 1024, 0, s>>>(jobs, nreq, prefix);
  return cudaGetLastError();
}

// Step `step` of many problems of one pixel layout (nc colour channels, maps or not).
extern "C" cudaError_t rs_launch_wave_multi(const WaveArgs* jobs, int nreq, const int* prefix, int step, int visCur,
                                            int nc, int map, int maxCtas, const volatile int* abortFlag,
                                            cudaStream_t s) {
  cudaError_t e = cudaSuccess;
  RS_DISPATCH(nc, map != 0, (e = launch_wave_multi_t<NC, MAP>(jobs, nreq, prefix, step, visCur, maxCtas, abortFlag, s)));
  return e;
}

extern "C" cudaError_t rs_launch_multi_prefix(const WaveArgs* jobs, int nreq, int step, int* prefix, cudaStream_t s) {
  k_multi_prefix<<<1, 1024, 0, s>>>(jobs, nreq, step, prefix);
  return cudaGetLastError();
}

extern "C" cudaError_t rs_launch_commit_multi(const WaveArgs* jobs, int nreq, const int* prefix, int step, int maxCtas,
                                              cudaStream_t s) {
  int grid = sm_count() * 2;
  if (maxCtas > 0) grid = std::min(grid, maxCtas);
  k_commit_multi<<<grid, 256, 0, s>>>(jobs, nreq, prefix, step);
  return cudaGetLastError();
}

extern "C" int rs_wave_corpus_staged(const Problem& pb, int warps) {
  if (warps < 1 || warps > 16) warps = 16;
  return wave_smem(pb, true, warps) <= 112 * 1024 ? 1 : 0;
}

extern "C" cudaError_t rs_launch_commit(const WaveArgs& a, int maxCtas, cudaStream_t s) {
  int grid = sm_count() * 2;
  if (maxCtas > 0) grid = std::min(grid, maxCtas);
  k_commit<<<grid, 256, 0, s>>>(a);
  return cudaGetLastError();
}

// ====================================================================
// Frozen-state best fit without device allocation.
//
// Some callers cannot let a library call cudaMalloc: a host application that
// reserves the GPU's memory up front and hands out every buffer from its own
// pool, or a latency-critical loop that cannot afford cudaMalloc's implicit
// device-wide synchronisation.  resynthFrozenBestFitNoAlloc serves them: the
// caller passes device buffers for every input and output, and the working
// memory (packed pixel words and metric tables) lives in the file-scope
// array below, which every GPU that loads this library holds until exit.
// Patches are built by scanning square rings of offsets around the target
// instead of walking a sorted offset list, so no list has to be stored.
// ====================================================================

extern "C" void rs_metric_tables(double sensitivity, double mapWeight, uint32_t* ct, uint32_t* mt);

namespace rs {
namespace {

// One metric table as a kernel argument (2 KiB of parameter space): the
// launch carries the values, which a captured graph keeps with the node.
struct TableArg {
  uint32_t v[kTable];
};
__global__ void __launch_bounds__(256) k_store_table(TableArg t, uint32_t* dst) {
  for (int i = threadIdx.x; i < kTable; i += blockDim.x) dst[i] = t.v[i];
}

constexpr size_t kNoAllocScratchBytes = 8u << 20;   // 8 MiB
constexpr size_t kNoAllocTableBytes = 2 * kTable * sizeof(uint32_t);
static __device__ __align__(256) unsigned char g_noAllocScratch[kNoAllocScratchBytes];

// Ring keys: (dx^2 + dy^2) << kRingIdxBits | (kRingIdxMask - box position).
// An accepted problem holds its target and corpus words in the working array,
// so the offset box (the smaller of the two images on each axis) has at most
// kMaxBoxPx pixels: its (2bw - 1)(2bh - 1) positions fit in kRingIdxBits and
// dx^2 + dy^2 < kMaxBoxPx^2 < 2^40, so the key fits 64 bits.
constexpr size_t kMaxBoxPx = (kNoAllocScratchBytes - kNoAllocTableBytes) / 4 / 2;
constexpr int kRingIdxBits = 23;
constexpr unsigned kRingIdxMask = (1u << kRingIdxBits) - 1u;
static_assert(4 * kMaxBoxPx <= (size_t)kRingIdxMask + 1, "box positions must fit the key's low bits");
static_assert(kMaxBoxPx < (1u << 20), "dx^2 + dy^2 must fit the key's high 41 bits");

// The square ring at Chebyshev distance r >= 1, clipped to the box
// |dx| < bw, |dy| < bh, as four runs: top (dy = -r, dx rising from -r), right
// (dx = r, dy rising from -r), bottom (dy = r, dx falling from r) and left
// (dx = -r, dy falling from r); each corner belongs to one run.
struct RingRuns {
  int lo[4], len[4];
};

__device__ __forceinline__ RingRuns ring_runs(int r, int bw, int bh) {
  RingRuns R;
  const bool rows = r < bh, cols = r < bw;
  // top: dx in [max(-r, 1-bw), min(r-1, bw-1)]
  R.lo[0] = max(-r, 1 - bw);
  R.len[0] = rows ? max(0, min(r - 1, bw - 1) - R.lo[0] + 1) : 0;
  // right: dy in [max(-r, 1-bh), min(r-1, bh-1)]
  R.lo[1] = max(-r, 1 - bh);
  R.len[1] = cols ? max(0, min(r - 1, bh - 1) - R.lo[1] + 1) : 0;
  // bottom: dx falling from min(r, bw-1) to max(1-r, 1-bw)
  R.lo[2] = min(r, bw - 1);
  R.len[2] = rows ? max(0, R.lo[2] - max(1 - r, 1 - bw) + 1) : 0;
  // left: dy falling from min(r, bh-1) to max(1-r, 1-bh)
  R.lo[3] = min(r, bh - 1);
  R.len[3] = cols ? max(0, R.lo[3] - max(1 - r, 1 - bh) + 1) : 0;
  return R;
}

__device__ __forceinline__ int ring_count(int r, int bw, int bh) {
  const RingRuns R = ring_runs(r, bw, bh);
  return R.len[0] + R.len[1] + R.len[2] + R.len[3];
}

// Point k (0 <= k < ring_count) of the clipped ring r.
__device__ __forceinline__ void ring_point(int r, int k, int bw, int bh, int& dx, int& dy) {
  const RingRuns R = ring_runs(r, bw, bh);
  if (k < R.len[0]) { dx = R.lo[0] + k; dy = -r; return; }
  k -= R.len[0];
  if (k < R.len[1]) { dx = r; dy = R.lo[1] + k; return; }
  k -= R.len[1];
  if (k < R.len[2]) { dx = R.lo[2] - k; dy = r; return; }
  k -= R.len[2];
  dx = -r;
  dy = R.lo[3] - k;
}

// prepare_neighbors by rings: every offset of the box, ring by ring, goes
// through the same sorted insertion as build_patch_sparse (key: dx^2 + dy^2,
// then descending box position -- the sorted offset list's order).  Only the
// parts of a ring inside the box are visited, and a warp pass covers the
// points of up to 32 consecutive rings (a thin box has two points per ring),
// so the work per target is O(box pixels / 32) warp passes at worst.  The
// scan stops once the patch is full and the next ring lies wholly beyond its
// last entry.
__device__ int build_patch_rings(const Problem& pb, int px, int py, Patch& P, unsigned long long* best, int lane) {
  if (lane == 0) load_nb(pb, P, 0, 0, py * pb.tw + px);
  const int lim = pb.patchLimit - 1;
  const int bw = pb.boxW, bh = pb.boxH;
  const unsigned W2 = 2u * bw - 1u;
  const int rmax = max(bw, bh) - 1;
  int cnt = 0;
  unsigned long long thr = ~0ull;
  bool done = false;
  for (int r0 = 1; r0 <= rmax && !done; r0 += 32) {
    // rings r0 .. r0 + 31: lane j counts ring r0 + j, an inclusive scan gives
    // where each ring's points start in this group
    const int myR = r0 + lane;
    const int myC = myR <= rmax ? ring_count(myR, bw, bh) : 0;
    int incl = myC;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(kFull, incl, o);
      if (lane >= o) incl += y;
    }
    const int total = __shfl_sync(kFull, incl, 31);
    for (int base = 0; base < total; base += 32) {
      // the ring of this pass's first point: every later point is as far
      const int g0 = base;
      int j0 = 0;
      for (int s = 16; s >= 1; s >>= 1)
        if (__shfl_sync(kFull, incl, j0 + s - 1) <= g0) j0 += s;
      const int rFirst = r0 + j0;
      if (cnt == lim && (unsigned long long)rFirst * rFirst > (thr >> kRingIdxBits)) {
        done = true;
        break;
      }
      const int g = base + lane;
      int j = 0;
      for (int s = 16; s >= 1; s >>= 1)
        if (__shfl_sync(kFull, incl, j + s - 1) <= g) j += s;
      j = min(j, 31);
      const int inclJ = __shfl_sync(kFull, incl, j), cJ = __shfl_sync(kFull, myC, j);
      unsigned long long key = ~0ull;
      if (g < total) {
        int dx, dy;
        ring_point(r0 + j, g - (inclJ - cJ), bw, bh, dx, dy);
        int qx = px + dx, qy = py + dy;
        if (wrap_or_clip(pb, qx, qy) && pb.has[(size_t)qy * pb.tw + qx]) {
          const unsigned idx = (unsigned)(dy + bh - 1) * W2 + (unsigned)(dx + bw - 1);
          const unsigned long long d2 = (unsigned long long)((long long)dx * dx + (long long)dy * dy);
          key = (d2 << kRingIdxBits) | (unsigned long long)(kRingIdxMask - idx);
        }
      }
      unsigned m = __ballot_sync(kFull, key < thr);
      while (m) {
        const int srcLane = __ffs(m) - 1;
        m &= m - 1;
        const unsigned long long kk = __shfl_sync(kFull, key, srcLane);
        if (kk >= thr) continue;
        const unsigned long long e0 = lane < cnt ? best[lane] : ~0ull;
        const unsigned long long e1 = lane + 32 < cnt ? best[lane + 32] : ~0ull;
        const int pos = __popc(__ballot_sync(kFull, e0 < kk)) + __popc(__ballot_sync(kFull, e1 < kk));
        __syncwarp();
        if (lane >= pos && lane < cnt && lane + 1 < lim) best[lane + 1] = e0;
        if (lane + 32 >= pos && lane + 32 < cnt && lane + 33 < lim) best[lane + 33] = e1;
        __syncwarp();
        if (lane == 0) best[pos] = kk;
        __syncwarp();
        cnt = min(cnt + 1, lim);
        thr = cnt == lim ? best[lim - 1] : ~0ull;
      }
    }
  }
  for (int i = lane; i < cnt; i += 32) {
    const unsigned idx = kRingIdxMask - (unsigned)(best[i] & kRingIdxMask);
    const int dx = (int)(idx % W2) - (bw - 1), dy = (int)(idx / W2) - (bh - 1);
    int qx = px + dx, qy = py + dy;
    wrap_or_clip(pb, qx, qy);
    load_nb(pb, P, 1 + i, pack_off(dx, dy), qy * pb.tw + qx);
  }
  __syncwarp();
  return 1 + cnt;
}

template <int NC, bool MAP>
__global__ void __launch_bounds__(256) k_frozen_noalloc(ScoreArgs a) {
  __shared__ uint32_t ct[kTable], mt[kTable];
  __shared__ Patch patches[8];
  __shared__ unsigned long long tops[8][kMaxNeighbors];
  load_half_tables(a.pb, ct, mt);
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = gridDim.x * (blockDim.x >> 5);
  Patch& P = patches[warp];
  for (int t = blockIdx.x * (blockDim.x >> 5) + warp; t < a.n; t += nw) {
    const int2 pos = a.targets[t];
    const int n = build_patch_rings(a.pb, pos.x, pos.y, P, tops[warp], lane);
    const unsigned c0 = a.candStart[t];
    const int ncand = (int)(a.candStart[t + 1] - c0);
    uint32_t bv;
    int bi;
    unsigned terms = 0, evals = 0;
    score_warp<NC, MAP, false>(a.pb, plain_view(a.pb), ct, mt, P, n, ncand,
                               [&](int k) { return a.cands[c0 + k]; }, lane, bv, bi, terms, evals);
    if (lane == 0) {
      a.outSum[t] = bv;
      a.outPt[t] = bi == INT_MAX ? make_int2(-1, -1) : a.cands[c0 + bi];
      a.outCount[t] = (unsigned)n;
    }
    __syncwarp();
  }
}

// The device address of g_noAllocScratch, looked up once per device with that
// device current (in host code the array's name is only a host-side stand-in).
unsigned char* noalloc_scratch(int dev, cudaError_t& err) {
  constexpr int kMaxDevices = 64;
  static std::mutex mu;
  static unsigned char* ptrs[kMaxDevices] = {};
  err = cudaSuccess;
  if (dev < 0 || dev >= kMaxDevices) {
    err = cudaErrorInvalidDevice;
    return nullptr;
  }
  std::lock_guard<std::mutex> lock(mu);
  if (!ptrs[dev]) {
    void* p = nullptr;
    err = cudaGetSymbolAddress(&p, g_noAllocScratch);
    if (err != cudaSuccess) return nullptr;
    ptrs[dev] = static_cast<unsigned char*>(p);
  }
  return ptrs[dev];
}

}  // namespace
}  // namespace rs

// Frozen-state best fit on caller-owned device buffers; allocates nothing.
// Declared in include/resynthesizer.h, which states its contract.
extern "C" __attribute__((visibility("default"))) int resynthFrozenBestFitNoAlloc(
    const TImageSynthParameters* p, const TFormatIndices* f, const unsigned char* dTarget, unsigned int tw,
    unsigned int th, const unsigned char* dCorpus, unsigned int cw, unsigned int ch, const unsigned char* dHasValue,
    const Coordinates* dSourceOf, const Coordinates* dTargets, unsigned int n, const unsigned int* dCandStart,
    const Coordinates* dCands, unsigned int* dBestSum, Coordinates* dBestPoint, unsigned int* dPatchCount,
    void* stream) {
  if (!p || !f || !dTarget || !dCorpus || !dHasValue || !dSourceOf || !dCandStart || !dBestSum || !dBestPoint ||
      !dPatchCount || (n && (!dTargets || !dCands)))
    return rs_fail(RESYNTH_ERROR_ARGUMENT, "resynthFrozenBestFitNoAlloc: NULL argument");
  if (p->patchSize > (unsigned)kMaxNeighbors) return IMAGE_SYNTH_ERROR_PATCH_SIZE_EXCEEDED;
  // Every byte the packing kernel reads (colours at 1 .. colorEndBip - 1, map
  // channels at map_start_bip ..) must lie inside the caller's pixel.
  if (f->img_match_bpp < 1 || f->img_match_bpp > 3 || f->map_match_bpp > 3 || f->total_bpp > 8 ||
      f->colorEndBip != 1 + f->img_match_bpp || f->colorEndBip > f->total_bpp ||
      (f->map_match_bpp && f->map_start_bip + f->map_match_bpp > f->total_bpp) || !tw || !th || !cw || !ch)
    return rs_fail(RESYNTH_ERROR_UNSUPPORTED, "resynthFrozenBestFitNoAlloc: pixel layout not supported");
  const bool maps = f->map_match_bpp > 0;
  const size_t tWords = (size_t)tw * th, cWords = (((size_t)cw * ch) + 3) & ~(size_t)3;
  const size_t need = kNoAllocTableBytes + 4 * (tWords + cWords) * (maps ? 2 : 1);
  if (need > kNoAllocScratchBytes)
    return rs_fail(RESYNTH_ERROR_UNSUPPORTED,
                   "resynthFrozenBestFitNoAlloc: images too large for the 8 MiB working array "
                   "(needs 4 KiB + 4 * (target pixels + corpus pixels) * (2 with map channels, else 1) bytes)");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  unsigned char* base = e == cudaSuccess ? noalloc_scratch(dev, e) : nullptr;
  if (!base) return rs_fail(RESYNTH_ERROR_DEVICE, cudaGetErrorString(e));
  // Working array layout: tables | target words | [target maps] | corpus words | [corpus maps]
  uint32_t tables[2 * kTable];
  rs_metric_tables(p->sensitivityToOutliers, p->mapWeight, tables, tables + kTable);
  uint32_t* dTables = reinterpret_cast<uint32_t*>(base);
  uint32_t* tpx = reinterpret_cast<uint32_t*>(base + kNoAllocTableBytes);
  uint32_t* tmap = maps ? tpx + tWords : nullptr;
  uint32_t* cpx = tpx + tWords * (maps ? 2 : 1);
  uint32_t* cmap = maps ? cpx + cWords : nullptr;
  // the tables travel as kernel arguments: no host copy is enqueued, so a
  // call after the first on a device can be captured into a CUDA graph
  for (int t = 0; t < 2; t++) {
    TableArg arg;
    memcpy(arg.v, tables + t * kTable, sizeof arg.v);
    k_store_table<<<1, 256, 0, s>>>(arg, dTables + t * kTable);
  }
  e = cudaGetLastError();
  if (e == cudaSuccess)
    e = rs_launch_pack(dTarget, (int)tw, (int)th, f->total_bpp, 1, f->img_match_bpp, f->map_start_bip,
                       f->map_match_bpp, tpx, tmap, s);
  if (e == cudaSuccess)
    e = rs_launch_pack(dCorpus, (int)cw, (int)ch, f->total_bpp, 1, f->img_match_bpp, f->map_start_bip,
                       f->map_match_bpp, cpx, cmap, s);
  if (e != cudaSuccess) return rs_fail(RESYNTH_ERROR_DEVICE, cudaGetErrorString(e));
  if (!n) return 0;
  ScoreArgs a{};
  Problem& pb = a.pb;
  pb.tw = (int)tw;
  pb.th = (int)th;
  pb.cw = (int)cw;
  pb.ch = (int)ch;
  pb.nc = f->img_match_bpp;
  pb.nm = f->map_match_bpp;
  pb.tpx = tpx;
  pb.tmap = tmap;
  pb.has = const_cast<uint8_t*>(dHasValue);
  pb.src = const_cast<int2*>(reinterpret_cast<const int2*>(dSourceOf));
  pb.cpx = cpx;
  pb.cmap = cmap;
  pb.patchLimit = (int)(p->patchSize > 2u ? p->patchSize : 2u);
  pb.tileH = p->isMakeSeamlesslyTileableHorizontally ? 1 : 0;
  pb.tileV = p->isMakeSeamlesslyTileableVertically ? 1 : 0;
  pb.boxW = (int)(tw < cw ? tw : cw);
  pb.boxH = (int)(th < ch ? th : ch);
  pb.clipCost = 65535u * f->img_match_bpp + tables[kTable] * f->map_match_bpp;
  pb.ctab = dTables;
  pb.mtab = dTables + kTable;
  a.targets = reinterpret_cast<const int2*>(dTargets);
  a.n = (int)n;
  a.candStart = dCandStart;
  a.cands = reinterpret_cast<const int2*>(dCands);
  a.outSum = dBestSum;
  a.outPt = reinterpret_cast<int2*>(dBestPoint);
  a.outCount = dPatchCount;
  RS_DISPATCH(pb.nc, maps,
              (k_frozen_noalloc<NC, MAP><<<grid_for((int)n, 8, sm_count() * 8), 256, 0, s>>>(a)));
  e = cudaGetLastError();
  return e == cudaSuccess ? 0 : rs_fail(RESYNTH_ERROR_DEVICE, cudaGetErrorString(e));
}
