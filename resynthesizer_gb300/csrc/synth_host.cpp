// synth_host.cpp -- the C ABI of libresynthesizer.so: the reference-compatible
// entry points (imageSynth, imageSynth2, engine, map and format helpers) and
// the extensions declared in include/resynthesizer.h.
//
// Host work mirrors the reference's preparation (lib/engine.c:338-497,
// 539-690): target/corpus point lists, hasValue, sourceOf, sorted offsets,
// metric tables and the target order with the reference's PRNG stream.  The
// passes run on the GPU (synth_kernels.cu) in one of two modes:
//   replay     -- one CTA visits targets in the reference order, consuming the
//                 same PRNG stream: output identical to the reference's
//                 single-threaded engine;
//   wavefront  -- each pass runs as batches of targets synthesized in parallel.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <atomic>
#include <thread>
#include <vector>

#include "../../include/resynthesizer.h"
#include "synth_internal.h"

#define RS_EXPORT extern "C" __attribute__((visibility("default")))

namespace {

// ------------------------------------------------------------------ errors

// Fixed buffer: reporting an error never allocates.
thread_local char g_lastError[512];

int fail(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_lastError, sizeof g_lastError, fmt, ap);
  va_end(ap);
  if (code == RESYNTH_ERROR_DEVICE) fprintf(stderr, "resynthesizer: %s\n", g_lastError);
  return code;
}

struct CudaError {
  cudaError_t e;
  const char* what;
};

#define CK(call)                                              \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) throw CudaError{e_, #call};        \
  } while (0)

// -------------------------------------------------------- reference PRNG

// The PRNG of the reference's standalone build is libc srand/rand
// (lib/glibProxy.c:29-49).  This is glibc's TYPE_3 additive feedback
// generator, restated so the stream can be produced without touching the
// process-wide rand() state: r[0] = seed, r[i] = 16807 r[i-1] mod (2^31 - 1)
// for i < 31, r[i] = r[i-31] for i in 31..33, then r[i] = r[i-3] + r[i-31]
// (mod 2^32); the k-th output is r[k + 344] >> 1.
class GlibcRand {
 public:
  explicit GlibcRand(unsigned seed) {
    int32_t r[34];
    r[0] = seed ? (int32_t)seed : 1;
    for (int i = 1; i < 31; i++) {
      const int64_t v = (16807LL * r[i - 1]) % 2147483647LL;
      r[i] = (int32_t)(v < 0 ? v + 2147483647LL : v);
    }
    for (int i = 31; i < 34; i++) r[i] = r[i - 31];
    for (int i = 0; i < 34; i++) ring_[i] = (uint32_t)r[i];
    pos_ = 34;
    for (int i = 34; i < 344; i++) step();
  }
  int next() { return (int)(step() >> 1); }
  // lib/glibProxy.c:36-49 (no draw when the bound is below 1)
  unsigned range(unsigned lo, unsigned hiExcl) {
    if (hiExcl < 1) return 0;
    const unsigned hi = hiExcl - 1;
    return lo + (unsigned)next() / (2147483647u / (hi - lo + 1) + 1);
  }

 private:
  uint32_t step() {
    const uint32_t v = ring_[(pos_ - 31) % 34] + ring_[(pos_ - 3) % 34];
    ring_[pos_ % 34] = v;
    pos_++;
    return v;
  }
  uint32_t ring_[34];
  uint64_t pos_;
};

// --------------------------------------------------------------- formats

void format_indices(TFormatIndices* f, unsigned colors, unsigned mapColors, int alphaT, int alphaS,
                    int isMap) {
  // lib/imageFormat.c:116-207
  f->img_match_bpp = (TPixelelIndex)colors;
  f->colorEndBip = (TPixelelIndex)(1 + colors);
  if (alphaT || alphaS) {
    f->alpha_bip = f->colorEndBip;
    f->map_start_bip = (TPixelelIndex)(f->colorEndBip + 1);
  } else {
    f->map_start_bip = f->colorEndBip;
  }
  f->map_match_bpp = (TPixelelIndex)(isMap ? mapColors : 0);
  f->map_end_bip = (TPixelelIndex)(f->map_start_bip + f->map_match_bpp);
  f->total_bpp = f->map_end_bip;
  f->isAlphaTarget = alphaT;
  f->isAlphaSource = alphaS;
}

// ------------------------------------------------------------- host prep

struct Pt {
  int x, y;
};

// Comparators of the reference (lib/engineTypes.h:51-149): they never return
// 0, so the tie order is libc qsort's -- the reason ordering calls qsort.
int cmp_more_horizontal(const void* va, const void* vb) {
  const Pt *a = (const Pt*)va, *b = (const Pt*)vb;
  return (a->x * a->x < b->x * b->x) ? 1 : -1;
}
int cmp_less_horizontal(const void* va, const void* vb) {
  const Pt *a = (const Pt*)va, *b = (const Pt*)vb;
  return (a->x * a->x < b->x * b->x) ? -1 : 1;
}
int cmp_more_vertical(const void* va, const void* vb) {
  const Pt *a = (const Pt*)va, *b = (const Pt*)vb;
  return (a->y * a->y < b->y * b->y) ? 1 : -1;
}
int cmp_less_vertical(const void* va, const void* vb) {
  const Pt *a = (const Pt*)va, *b = (const Pt*)vb;
  return (a->y * a->y < b->y * b->y) ? -1 : 1;
}
struct SortElem {
  Pt p;
  float prop;
};
int cmp_less_inward(const void* va, const void* vb) {
  return (((const SortElem*)va)->prop < ((const SortElem*)vb)->prop) ? -1 : 1;
}
int cmp_more_inward(const void* va, const void* vb) { return cmp_less_inward(va, vb) == 1 ? -1 : 1; }

// Sorted offsets (lib/engine.c:465-497): all offsets of the (2w-1) x (2h-1)
// box, w/h the smaller of target and corpus, ascending in x^2 + y^2.  The
// reference sorts with libc qsort and a comparator that never returns 0; with
// glibc's merge sort that leaves equal distances in reverse generation order,
// i.e. descending y, then descending x.  Generated directly in that order
// (checked against libc qsort by the tests), optionally truncated to radius^2.
std::vector<int2> sorted_offsets(int w, int h, long long maxD2) {
  std::vector<uint64_t> keys;
  const int W = 2 * w - 1;
  keys.reserve((size_t)W * (2 * h - 1));
  for (int y = -h + 1; y < h; y++)
    for (int x = -w + 1; x < w; x++) {
      const long long d2 = (long long)x * x + (long long)y * y;
      if (d2 > maxD2) continue;
      const uint32_t idx = (uint32_t)((y + h - 1) * W + (x + w - 1));
      keys.push_back(((uint64_t)d2 << 32) | (uint32_t)~idx);
    }
  std::sort(keys.begin(), keys.end());
  std::vector<int2> out(keys.size());
  for (size_t i = 0; i < keys.size(); i++) {
    const uint32_t idx = ~(uint32_t)(keys[i] & 0xffffffffu);
    out[i] = make_int2((int)(idx % W) - (w - 1), (int)(idx / W) - (h - 1));
  }
  return out;
}

// Metric tables (lib/matchWeighting.h:49-60, 142-178): float parameters,
// double arithmetic, truncating casts -- computed on the host with libm.
void metric_tables(double sensitivity, double mapWeight, uint32_t* ct, uint32_t* mt) {
  const float c = (float)sensitivity, w = (float)mapWeight;
  auto nlc = [c](double x) { return std::log((x / (c * 256)) * (x / (c * 256)) + 1.0); };
  for (int i = -256; i < 256; i++) {
    const double v = nlc(i) / nlc(256) * (float)65535;
    ct[256 + i] = (unsigned short)v;
    mt[256 + i] = (unsigned int)(i * i * w * 4.0);
  }
}

Pt bbox_center(const std::vector<Pt>& v) {  // lib/engineTypes.h:187-226
  int ulx = INT_MAX, uly = INT_MAX, lrx = 0, lry = 0;
  for (const Pt& p : v) {
    ulx = std::min(ulx, p.x);
    uly = std::min(uly, p.y);
    lrx = std::max(lrx, p.x);
    lry = std::max(lry, p.y);
  }
  return Pt{(lrx - ulx) / 2 + ulx, (lry - uly) / 2 + uly};
}

unsigned ray_of(Pt a) {  // lib/brushfire.h:62-67
  return (unsigned)(std::atan2((double)(float)a.y, (double)(float)a.x) * 200 /
                        3.1415926535897932384626433832795028841971693993751 +
                    200);
}

// The target order of lib/orderTarget.h:268-343, consuming `rng` exactly as
// the reference does.  Returns 0 or MATCH_CONTEXT_TYPE_RANGE.
int order_targets(int type, std::vector<Pt>& v, GlibcRand& rng) {
  const unsigned n = (unsigned)v.size();
  if (type == 0 || type == 1) {
    for (unsigned i = 0; i < n; i++) std::swap(v[i], v[rng.range(0, n)]);
    return 0;
  }
  if (type < 0 || type > 8) return IMAGE_SYNTH_ERROR_MATCH_CONTEXT_TYPE_RANGE;
  const Pt c = bbox_center(v);
  for (Pt& p : v) p = Pt{p.x - c.x, p.y - c.y};
  if (type == 2 || type == 5 || type == 8) {
    // Brushfire key: |p|^2 over the largest |q|^2 on the same one of 401 rays
    // (lib/brushfire.h:73-148).  The squeeze order (type 8) writes its sorted
    // array straight back, so it equals the inward order (lib/orderTarget.h:209-262).
    unsigned maxr[401] = {0};
    for (const Pt& p : v) {
      const unsigned d = (unsigned)(p.x * p.x + p.y * p.y), r = ray_of(p);
      if (d > maxr[r]) maxr[r] = d;
    }
    std::vector<SortElem> s(n);
    for (unsigned i = 0; i < n; i++)
      s[i] = SortElem{v[i], (float)(v[i].y * v[i].y + v[i].x * v[i].x) / maxr[ray_of(v[i])]};
    std::qsort(s.data(), n, sizeof(SortElem), type == 5 ? cmp_less_inward : cmp_more_inward);
    for (unsigned i = 0; i < n; i++) v[i] = s[i].p;
  } else {
    auto cmp = type == 3 ? cmp_more_horizontal : type == 4 ? cmp_more_vertical
             : type == 6 ? cmp_less_horizontal : cmp_less_vertical;
    std::qsort(v.data(), n, sizeof(Pt), cmp);
  }
  for (Pt& p : v) p = Pt{p.x + c.x, p.y + c.y};
  // banded shuffle, lib/orderTarget.h:58-79
  const int last = (int)n - 1, half = (int)(n * 0.1);
  for (int i = 0; i <= last; i++) {
    const int lo = std::max(i - half, 0), hi = std::min(i + half, last);
    std::swap(v[i], v[lo + (int)rng.range(0, (unsigned)(hi - lo))]);
  }
  return 0;
}

// The banded shuffle of lib/orderTarget.h:58-79 as a permutation of positions:
// after it, position i holds what the sorted order had at perm[i].  It
// depends only on the count and on the PRNG stream (which the directional
// orders draw from for this shuffle alone), so the device can sort and the
// host shuffle indices at the same time.
std::vector<int> band_shuffle_perm(unsigned n) {
  GlibcRand rng(1198472u);   // lib/engine.c:643
  std::vector<int> idx(n);
  for (unsigned i = 0; i < n; i++) idx[i] = (int)i;
  const int last = (int)n - 1, half = (int)(n * 0.1);
  for (int i = 0; i <= last; i++) {
    const int lo = std::max(i - half, 0), hi = std::min(i + half, last);
    std::swap(idx[i], idx[lo + (int)rng.range(0, (unsigned)(hi - lo))]);
  }
  return idx;
}

// ------------------------------------------------------------ the problem

struct HostPrep {
  std::vector<Pt> targets;         // in visit order
  std::vector<Pt> corpusPts;       // row-major
  std::vector<uint8_t> hasValue;   // initial, target-sized
  uint32_t ct[512], mt[512];
  unsigned ends[rs::kPasses];
  unsigned estimated;
  GlibcRand rng{1198472u};         // engine.c:643, consumed by ordering first
};

// Pass lengths (lib/passes.h:67-93): all n targets twice, then prefixes of
// 3/4 of the previous length; `estimated` is their sum (lib/passes.h:55-63).
void pass_schedule(unsigned n, unsigned ends[rs::kPasses], unsigned& estimated) {
  ends[0] = n;
  estimated = n;
  for (int i = 1; i < rs::kPasses; i++) {
    ends[i] = n;
    estimated += n;
    n = n * 3 / 4;
  }
}

// Engine preparation (lib/engine.c:585-645).  Returns 0 or an engine error.
int prepare(const TImageSynthParameters& p, const TFormatIndices& f, const uint8_t* target, unsigned tw,
            unsigned th, const uint8_t* corpus, unsigned cw, unsigned ch, HostPrep& hp) {
  if (p.patchSize > (unsigned)rs::kMaxNeighbors) return IMAGE_SYNTH_ERROR_PATCH_SIZE_EXCEEDED;
  const size_t tn = (size_t)tw * th, cn = (size_t)cw * ch;
  hp.hasValue.assign(tn, 0);
  hp.targets.clear();
  const int bpp = f.total_bpp;
  for (unsigned y = 0; y < th; y++)
    for (unsigned x = 0; x < tw; x++) {
      const uint8_t* px = target + ((size_t)y * tw + x) * bpp;
      const bool selected = px[0] != 0;
      const bool opaque = f.isAlphaTarget ? px[f.alpha_bip] != 0 : true;
      hp.hasValue[(size_t)y * tw + x] = (p.matchContextType && !selected && opaque) ? 1 : 0;
      if (selected) hp.targets.push_back(Pt{(int)x, (int)y});
    }
  if (hp.targets.empty()) return IMAGE_SYNTH_ERROR_EMPTY_TARGET;
  hp.corpusPts.clear();
  hp.corpusPts.reserve(cn / 2);
  for (unsigned y = 0; y < ch; y++)
    for (unsigned x = 0; x < cw; x++) {
      const uint8_t* px = corpus + ((size_t)y * cw + x) * bpp;
      if (px[0] == 0xFF && (f.isAlphaSource ? px[f.alpha_bip] != 0 : true)) hp.corpusPts.push_back(Pt{(int)x, (int)y});
    }
  if (hp.corpusPts.empty()) return IMAGE_SYNTH_ERROR_EMPTY_CORPUS;
  metric_tables(p.sensitivityToOutliers, p.mapWeight, hp.ct, hp.mt);
  hp.rng = GlibcRand(1198472u);
  const int rc = order_targets(p.matchContextType, hp.targets, hp.rng);
  if (rc) return rc;
  pass_schedule((unsigned)hp.targets.size(), hp.ends, hp.estimated);
  return 0;
}

// Progress emulation: lib/progress.c:53-65 called at every target index that
// is a multiple of 4096 (lib/synthesize.h:493), before that index is visited.
struct Progress {
  unsigned estimated = 1, completed = 0, prior = 0;
  void (*cb)(int, void*) = nullptr;
  void* ctx = nullptr;
  void tick() {
    completed += 4095u;
    const unsigned pct = (unsigned)(((float)completed / estimated) * 100);
    if (pct > prior) {
      if (cb) cb((int)pct, ctx);
      prior = pct;
    }
  }
};

// ----------------------------------------------------------- device state

struct Stream {
  cudaStream_t s = nullptr;
  volatile int* abortHost = nullptr;
  int* abortDev = nullptr;
  rs::Counters* hostCtr = nullptr;   // pinned: counter read-backs stay asynchronous
  int* hostInts = nullptr;           // pinned: small read-backs
  // Side streams for the many-request path: the per-request preparation
  // kernels (small, independent) run on them side by side, forked from and
  // joined back into s with events.
  int* hostBands = nullptr;          // pinned: per-pass band boundaries of every request of a batch
  size_t hostBandsCap = 0;
  int* host_bands(size_t n) {
    if (n > hostBandsCap) {
      if (hostBands) CK(cudaFreeHost(hostBands));
      hostBands = nullptr;
      CK(cudaHostAlloc((void**)&hostBands, n * sizeof(int), cudaHostAllocDefault));
      hostBandsCap = n;
    }
    return hostBands;
  }
  static constexpr int kSide = 8;
  cudaStream_t side[kSide] = {};
  cudaEvent_t fork = nullptr, join[kSide] = {};
  void ensure_side() {
    if (fork) return;
    for (int i = 0; i < kSide; i++) {
      CK(cudaStreamCreateWithFlags(&side[i], cudaStreamNonBlocking));
      CK(cudaEventCreateWithFlags(&join[i], cudaEventDisableTiming));
    }
    CK(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
  }
  // Side streams wait for everything queued on s so far.
  void fork_side() {
    ensure_side();
    CK(cudaEventRecord(fork, s));
    for (int i = 0; i < kSide; i++) CK(cudaStreamWaitEvent(side[i], fork, 0));
  }
  // s waits for everything queued on the side streams.
  void join_side() {
    for (int i = 0; i < kSide; i++) {
      CK(cudaEventRecord(join[i], side[i]));
      CK(cudaStreamWaitEvent(s, join[i], 0));
    }
  }
  // A thread's stream lives as long as the thread (host workers come and go
  // with every many-request call): everything is released at thread exit.
  // Errors are ignored (at process exit the runtime may already be gone).
  ~Stream() {
    for (int i = 0; i < kSide; i++) {
      if (side[i]) cudaStreamDestroy(side[i]);
      if (join[i]) cudaEventDestroy(join[i]);
    }
    if (fork) cudaEventDestroy(fork);
    if (s) cudaStreamDestroy(s);
    if (hostBands) cudaFreeHost(hostBands);
    if (hostInts) cudaFreeHost(hostInts);
    if (hostCtr) cudaFreeHost(hostCtr);
    if (abortHost) cudaFreeHost((void*)abortHost);
  }
  Stream(const Stream&) = delete;
  Stream& operator=(const Stream&) = delete;
  Stream() {
    CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    CK(cudaHostAlloc((void**)&abortHost, sizeof(int), cudaHostAllocMapped));
    *abortHost = 0;
    CK(cudaHostGetDevicePointer((void**)&abortDev, (void*)abortHost, 0));
    CK(cudaHostAlloc((void**)&hostCtr, sizeof(rs::Counters), cudaHostAllocDefault));
    CK(cudaHostAlloc((void**)&hostInts, 16 * sizeof(int), cudaHostAllocDefault));
  }
};

Stream& thread_stream() {
  thread_local std::unique_ptr<Stream> st;
  if (!st) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) throw CudaError{cudaErrorNoDevice, "no CUDA device"};
    static std::once_flag poolOnce;
    std::call_once(poolOnce, [] {
      int dev = 0;
      cudaGetDevice(&dev);
      cudaMemPool_t pool;
      if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        uint64_t thr = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
      }
    });
    st.reset(new Stream());
  }
  return *st;
}

// Stream-ordered device allocations released at scope exit.
// With a chunk size, allocations are carved out of large chunks so that the
// buffers of many small problems sit close together in the address space
// (fewer address-translation misses when one kernel touches all of them).
class Arena {
 public:
  // Allocations are ordered on s; frees on freeStream (default s), which must
  // by then be ordered after every use.
  explicit Arena(cudaStream_t s, size_t chunk = 0, cudaStream_t freeStream = nullptr)
      : s_(s), free_(freeStream ? freeStream : s), chunk_(chunk) {}
  ~Arena() {
    for (void* p : ptrs_) cudaFreeAsync(p, free_);
  }
  template <class T>
  T* alloc(size_t n) {
    const size_t bytes = std::max<size_t>(n, 1) * sizeof(T) + 16;
    if (chunk_ && bytes <= chunk_ / 4) {
      const size_t need = (bytes + 255) & ~(size_t)255;
      if (!cur_ || used_ + need > chunk_) {
        CK(cudaMallocAsync(&cur_, chunk_, s_));
        ptrs_.push_back(cur_);
        used_ = 0;
      }
      void* p = static_cast<char*>(cur_) + used_;
      used_ += need;
      return static_cast<T*>(p);
    }
    void* p = nullptr;
    CK(cudaMallocAsync(&p, bytes, s_));
    ptrs_.push_back(p);
    return static_cast<T*>(p);
  }
  template <class T>
  T* upload(const T* h, size_t n, unsigned long long& bytes) {
    T* d = alloc<T>(n);
    if (n) CK(cudaMemcpyAsync(d, h, n * sizeof(T), cudaMemcpyHostToDevice, s_));
    bytes += n * sizeof(T);
    return d;
  }

 private:
  cudaStream_t s_, free_;
  size_t chunk_ = 0, used_ = 0;
  void* cur_ = nullptr;
  std::vector<void*> ptrs_;
};

// Cached sorted-offset lists (they depend only on the box and the radius).
// Shared ownership: a caller keeps its list alive while other threads evict.
std::shared_ptr<const std::vector<int2>> cached_offsets(int w, int h, long long maxD2) {
  static std::mutex mu;
  static std::map<std::tuple<int, int, long long>, std::shared_ptr<const std::vector<int2>>> cache;
  const auto key = std::make_tuple(w, h, maxD2);
  {
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
  }
  auto list = std::make_shared<const std::vector<int2>>(sorted_offsets(w, h, maxD2));
  std::lock_guard<std::mutex> lock(mu);
  if (cache.size() > 16) cache.clear();
  cache.emplace(key, list);
  return list;
}

// The wavefront offset list: every offset within 256 px, in the sorted
// offset list's order (ascending dx^2 + dy^2, ties by descending dy, then
// descending dx).  That order does not depend on the box, so the wavefront
// list of any image (radius min(box diagonal, 256)) is this one restricted to
// |dx| < box width, |dy| < box height -- the kernels apply that restriction --
// and one list, uploaded once per device, serves every image size.
const std::vector<int2>& wave_offsets_host() {
  static const std::vector<int2> list = sorted_offsets(257, 257, 256LL * 256LL);
  return list;
}

const int2* wave_offsets_device(int& n) {
  static std::mutex mu;
  static std::map<int, int2*> perDevice;
  const std::vector<int2>& host = wave_offsets_host();
  n = (int)host.size();
  int dev = 0;
  CK(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  auto it = perDevice.find(dev);
  if (it != perDevice.end()) return it->second;
  int2* d = nullptr;
  CK(cudaMalloc(&d, host.size() * sizeof(int2)));
  CK(cudaMemcpy(d, host.data(), host.size() * sizeof(int2), cudaMemcpyHostToDevice));
  perDevice[dev] = d;
  return d;
}

// k of the colour phases: the reach of a dense patch (its last offset) + 1.
int phase_side_box(const std::vector<int2>& offs, int patchLimit, int w, int h) {
  int taken = 0;
  int2 last = make_int2(0, 0);
  for (const int2& o : offs) {
    if (std::abs(o.x) >= w || std::abs(o.y) >= h) continue;
    last = o;
    if (++taken == patchLimit) break;
  }
  const double r = std::sqrt((double)last.x * last.x + (double)last.y * last.y);
  return std::max(1, std::min(8, (int)std::floor(r) + 1));
}

struct RecordedState {
  std::vector<int2> src;
  std::vector<uint8_t> has;
  unsigned w = 0, h = 0;
};
thread_local RecordedState g_state;

int g_defaultMode = -1;

int default_mode() {
  if (g_defaultMode < 0) {
    const char* e = getenv("RESYNTH_MODE");
    g_defaultMode = (e && !strcmp(e, "replay")) ? RESYNTH_MODE_REPLAY : RESYNTH_MODE_WAVEFRONT;
  }
  return g_defaultMode;
}

// Layouts the kernels handle, with every byte they read (colours, map
// channels, alpha) inside the pixel: a TFormatIndices that points past
// total_bpp would make the device read past the end of the caller's buffers.
bool supported_format(const TFormatIndices& f) {
  return f.img_match_bpp >= 1 && f.img_match_bpp <= 3 && f.map_match_bpp <= 3 && f.total_bpp <= 8 &&
         f.colorEndBip == 1 + f.img_match_bpp && f.colorEndBip <= f.total_bpp &&
         (!f.map_match_bpp || f.map_start_bip + f.map_match_bpp <= f.total_bpp) &&
         ((!f.isAlphaTarget && !f.isAlphaSource) || f.alpha_bip < f.total_bpp);
}

// Device problem built from device pixmaps.
struct DeviceProblem {
  rs::Problem pb{};
  uint32_t* tpx = nullptr;
  uint32_t* tmap = nullptr;
};

DeviceProblem make_problem(Arena& ar, cudaStream_t s, const TImageSynthParameters& p, const TFormatIndices& f,
                           const uint8_t* dT, unsigned tw, unsigned th, const uint8_t* dC, unsigned cw, unsigned ch,
                           const uint8_t* hasInit, const int2* srcInit,
                           const std::vector<int2>& offs, long long maxD2, unsigned long long& h2d,
                           unsigned& launches, const int2* dOffs = nullptr, int nOffs = 0) {
  DeviceProblem d;
  rs::Problem& pb = d.pb;
  pb.tw = (int)tw;
  pb.th = (int)th;
  pb.cw = (int)cw;
  pb.ch = (int)ch;
  pb.nc = f.img_match_bpp;
  pb.nm = f.map_match_bpp;
  const size_t tn = (size_t)tw * th, cn = (size_t)cw * ch, cnPad = (cn + 3) & ~(size_t)3;
  d.tpx = ar.alloc<uint32_t>(tn);
  d.tmap = pb.nm ? ar.alloc<uint32_t>(tn) : nullptr;
  uint32_t* cpx = ar.alloc<uint32_t>(cnPad);
  uint32_t* cmap = pb.nm ? ar.alloc<uint32_t>(cnPad) : nullptr;
  CK(rs_launch_pack(dT, (int)tw, (int)th, f.total_bpp, 1, pb.nc, f.map_start_bip, pb.nm, d.tpx, d.tmap, s));
  CK(rs_launch_pack(dC, (int)cw, (int)ch, f.total_bpp, 1, pb.nc, f.map_start_bip, pb.nm, cpx, cmap, s));
  // padded copy for the wavefront kernel
  pb.padW = (int)cw + 2 * rs::kPad;
  const size_t padWords = (((size_t)pb.padW * (ch + 2 * rs::kPad)) + 3) & ~(size_t)3;
  uint32_t* cpxPad = ar.alloc<uint32_t>(padWords);
  uint2* cpmPad = pb.nm ? ar.alloc<uint2>(padWords) : nullptr;
  CK(rs_launch_pack_padded(dC, (int)cw, (int)ch, f.total_bpp, pb.nc, f.map_start_bip, pb.nm, cpxPad, cpmPad, s));
  pb.cpxPad = cpxPad;
  pb.cpmPad = cpmPad;
  launches += 3;
  pb.tpx = d.tpx;
  pb.tmap = d.tmap;
  pb.cpx = cpx;
  pb.cmap = cmap;
  if (hasInit) {
    pb.has = ar.upload(hasInit, tn, h2d);
  } else {
    pb.has = ar.alloc<uint8_t>(tn);
  }
  int2* src = ar.alloc<int2>(tn);
  if (srcInit) {
    CK(cudaMemcpyAsync(src, srcInit, tn * sizeof(int2), cudaMemcpyHostToDevice, s));
    h2d += tn * sizeof(int2);
  } else {
    CK(cudaMemsetAsync(src, 0xFF, tn * sizeof(int2), s));   // (-1, -1)
  }
  pb.src = src;
  pb.boxW = (int)std::min(tw, cw);
  pb.boxH = (int)std::min(th, ch);
  pb.maxD2 = maxD2;
  if (dOffs) {
    pb.offs = dOffs;
    pb.noffs = nOffs;
  } else {
    pb.offs = ar.upload(offs.data(), offs.size(), h2d);
    pb.noffs = (int)offs.size();
  }
  pb.patchLimit = (int)std::max(p.patchSize, 2u);
  pb.tileH = p.isMakeSeamlesslyTileableHorizontally ? 1 : 0;
  pb.tileV = p.isMakeSeamlesslyTileableVertically ? 1 : 0;
  uint32_t ct[512], mt[512];
  metric_tables(p.sensitivityToOutliers, p.mapWeight, ct, mt);
  pb.clipCost = 65535u * f.img_match_bpp + mt[0] * f.map_match_bpp;
  pb.ctab = ar.upload(ct, 512, h2d);
  pb.mtab = ar.upload(mt, 512, h2d);
  return d;
}

// Growth of the large pass-0 bands (percent): once a band holds 1/64 of the
// pass, bands grow more slowly, so that fewer targets share a batch when the
// neighbourhoods are dense (energy); the small bands before are latency-bound
// and keep doubling.
constexpr unsigned kDefaultGrowthLarge = 200;

// A grid-barrier wait of the persistent wavefront kernel longer than this
// gives up: far beyond the longest batch (milliseconds), short enough that a
// CTA that never arrives ends the call with an error instead of holding the GPU.
constexpr long long kBarrierTimeoutNs = 10LL * 1000 * 1000 * 1000;

// First pass-0 band of a random order: 16 targets, or for a heal (targets
// with context around them) one 1024th of the targets when that is more.  A
// heal's first targets find context close by, so tiny first bands buy no
// patch energy there (on the CPU restatement of heal4096, over six seeds,
// targets / 1024 ends at 0.989x the energy of 16 with a spread of 0.9 %)
// while each of their batches costs a latency-bound step; texture synthesis
// from nothing keeps 16 (its energy grows with the first band).
unsigned wave_first_band(unsigned ntargets, bool noContext) {
  return noContext ? 16u : std::max(16u, ntargets / 1024u);
}

// Pass-0 band growth in percent of a random order: bands double, or
// quadruple for map-guided problems, whose metric the map term dominates so
// that the schedule matters little for the energy (a 1024^2 map-guided run on
// the CPU restatement, three seeds: +0.1 % energy with 151 batches instead of
// 273).
unsigned wave_band_growth(int mapChannels) { return mapChannels ? 400u : 200u; }

// Passes the wavefront runs at least.  Texture synthesis from nothing (no
// context, no map channels) ends its second pass with a patch energy about
// 1.5 % above the reference's threaded engine (the targets of a batch do not
// see each other); a third pass brings it under 1 % (render1024: 1.0148 ->
// 1.0066 of the threaded mean, 4 seeds against 8 runs).  Heals and map-guided
// runs meet the energy of the reference with its own stop rule.
int wave_min_passes(const TResynthOptions& opt, bool noContext, int mapChannels) {
  if (opt.minPasses) return (int)opt.minPasses;
  return noContext && mapChannels == 0 ? 3 : 0;
}

unsigned ilog2(uint64_t v) {
  unsigned r = 0;
  while (v >>= 1) r++;
  return r;
}

// Autotuned warps per CTA by problem class (0 = not tuned yet).
std::mutex g_tuneMu;
std::map<uint64_t, int> g_tunedWarps;

int tuned_warps(uint64_t key) {
  std::lock_guard<std::mutex> lock(g_tuneMu);
  auto it = g_tunedWarps.find(key);
  return it == g_tunedWarps.end() ? 0 : it->second;
}

void set_tuned_warps(uint64_t key, int warps) {
  std::lock_guard<std::mutex> lock(g_tuneMu);
  g_tunedWarps[key] = warps;
}

// How a problem class's passes are launched, tuned across calls: the first
// six calls of a class (colour and map channels, patch size, corpus and
// target sizes) run, twice in turn, the persistent pass with 16 warps per
// CTA, with 8, and one launch per batch; each records the synthesis's device
// time, and later calls use the configuration with the least of its two times
// (the first use of a configuration in a process also pays for loading its
// kernels, which the second does not).  The persistent pass saves a launch per batch but
// pays a grid barrier per batch, and with fewer warps per CTA more CTAs meet
// at each barrier, so which wins depends on the problem (texture synthesis
// with many small batches gains most from it).  The output does not depend on
// the choice.
enum LaunchConfig { kPersistent16 = 0, kPersistent8 = 1, kPerBatch = 2, kLaunchConfigs = 3 };
constexpr int kLaunchSamples = 2;
struct LaunchTune {
  int trials = 0, best = -1;
  double ms[kLaunchConfigs] = {1e30, 1e30, 1e30};
};
std::map<uint64_t, LaunchTune> g_launchTune;

// The configuration of this call; `trial` when its time is to be recorded
// (the value returned is then the trial number, config = trial % 3).
int launch_config(uint64_t key, bool& trial) {
  std::lock_guard<std::mutex> lock(g_tuneMu);
  LaunchTune& t = g_launchTune[key];
  trial = t.best < 0;
  return trial ? t.trials : t.best;
}

void launch_result(uint64_t key, int trialNo, double ms) {
  std::lock_guard<std::mutex> lock(g_tuneMu);
  LaunchTune& t = g_launchTune[key];
  if (t.best >= 0 || trialNo != t.trials) return;   // another call of the class got there first
  double& m = t.ms[trialNo % kLaunchConfigs];
  m = std::min(m, ms);
  if (++t.trials == kLaunchConfigs * kLaunchSamples) {
    t.best = 0;
    for (int c = 1; c < kLaunchConfigs; c++)
      if (t.ms[c] < t.ms[t.best]) t.best = c;
  }
}

// Radius (squared) of the offset list used by the wavefront mode: enough for
// any dense patch; sparse early batches look this far for context.
long long wave_radius2(int w, int h) {
  const long long full = (long long)(w - 1) * (w - 1) + (long long)(h - 1) * (h - 1);
  return std::min<long long>(full, 256LL * 256LL);
}

// CUDA-event timing of individual kernel launches on their own stream.
class LaunchTimer {
 public:
  ~LaunchTimer() {
    for (auto& p : ev_) {
      cudaEventDestroy(p.first);
      cudaEventDestroy(p.second);
    }
  }
  void begin(cudaStream_t s) {
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    ev_.emplace_back(a, b);
    CK(cudaEventRecord(a, s));
  }
  void end(cudaStream_t s) { CK(cudaEventRecord(ev_.back().second, s)); }
  double total() const {
    double t = 0;
    for (auto& p : ev_) {
      float ms = 0;
      if (cudaEventElapsedTime(&ms, p.first, p.second) == cudaSuccess) t += ms;
    }
    return t;
  }
  unsigned count() const { return (unsigned)ev_.size(); }

 private:
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_;
};

// Side k of the colour phases: one more than the radius of a dense patch
// (the distance of its last offset), so two targets of one phase are never
// inside each other's dense patch.
void wait_stream(Stream& st, cudaEvent_t ev, int* cancel) {
  while (true) {
    const cudaError_t q = cudaEventQuery(ev);
    if (q == cudaSuccess) return;
    if (q != cudaErrorNotReady) throw CudaError{q, "cudaEventQuery"};
    if (cancel && *cancel) *st.abortHost = 1;
    std::this_thread::sleep_for(std::chrono::microseconds(20));
  }
}

// The visit order of a directional or brushfire type (matchContextType 2..8,
// lib/orderTarget.h:268-343) of the n row-major targets in dTargets, made on
// the device into dOut; the banded shuffle's permutation is computed on the
// host meanwhile.  Brushfire needs two short round trips: the rays of the few
// targets next to a ray boundary come from the host's libm (as the
// reference's do), and a NaN key -- the bounding-box centre is a target alone
// on its ray -- sends the whole order to the host's qsort, whose treatment of
// it no key sort reproduces.
void order_directional(int type, const int2* dTargets, int n, int2* dOut, Arena& ar, Stream& st, cudaStream_t s,
                       unsigned long long& h2d, unsigned long long& d2h, unsigned& launches) {
  int* work = ar.alloc<int>(rs_order_ints(n));
  const bool brush = type == 2 || type == 5 || type == 8;
  int* dFlags = brush ? ar.alloc<int>(1 + 3 * (size_t)n) : nullptr;
  CK(rs_order_begin(type, dTargets, n, work, dFlags, dFlags ? dFlags + 1 : nullptr, n, s));
  launches += brush ? 3 : 2;
  if (brush) CK(cudaMemcpyAsync(st.hostInts + 4, dFlags, sizeof(int), cudaMemcpyDeviceToHost, s));
  const std::vector<int> perm = band_shuffle_perm((unsigned)n);   // host work while the device runs
  if (brush) {
    CK(cudaStreamSynchronize(s));
    const int nflag = std::min(st.hostInts[4], n);
    std::vector<int> flags(3 * (size_t)nflag), fix(2 * (size_t)nflag);
    if (nflag) CK(cudaMemcpy(flags.data(), dFlags + 1, flags.size() * sizeof(int), cudaMemcpyDeviceToHost));
    d2h += 4 + flags.size() * sizeof(int);
    for (int i = 0; i < nflag; i++) {
      fix[2 * i] = flags[3 * i];
      fix[2 * i + 1] = (int)ray_of(Pt{flags[3 * i + 1], flags[3 * i + 2]});
    }
    const int* dFix = nflag ? ar.upload(fix.data(), fix.size(), h2d) : nullptr;
    CK(rs_order_rays(dTargets, n, work, dFix, nflag, s));
    launches += nflag ? 3 : 2;
    CK(cudaMemcpyAsync(st.hostInts + 5, rs_order_nan_flag(work, n), sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    d2h += 4;
    if (st.hostInts[5]) {
      std::vector<Pt> v((size_t)n);
      CK(cudaMemcpy(v.data(), dTargets, (size_t)n * sizeof(int2), cudaMemcpyDeviceToHost));
      d2h += (size_t)n * sizeof(int2);
      GlibcRand rng(1198472u);
      order_targets(type, v, rng);
      CK(cudaMemcpyAsync(dOut, v.data(), (size_t)n * sizeof(int2), cudaMemcpyHostToDevice, s));
      CK(cudaStreamSynchronize(s));   // v is pageable and about to go
      h2d += (size_t)n * sizeof(int2);
      return;
    }
  }
  const int* dPerm = ar.upload(perm.data(), perm.size(), h2d);
  CK(rs_order_finish(type, dTargets, n, work, dPerm, dOut, s));
  launches += 14;
}

// The pass loop on device pixmaps.  dT is updated in place.  `prepared` is
// the host preparation when the caller already made it (engine() on host maps).
int run_engine_device(const TImageSynthParameters& p, const TFormatIndices& f, uint8_t* dT, unsigned tw,
                      unsigned th, const uint8_t* dC, unsigned cw, unsigned ch, HostPrep* prepared,
                      cudaStream_t userStream, void (*progressCb)(int, void*), void* ctx,
                      int* cancel, const TResynthOptions& opt, TResynthStats& stats) {
  Stream& st = thread_stream();
  cudaStream_t s = userStream ? userStream : st.s;
  *st.abortHost = 0;
  int zero = 0;
  if (!cancel) cancel = &zero;
  const bool replay = opt.mode == RESYNTH_MODE_REPLAY;
  int launchCfg = -100;      // >= 0: this call tries that launch configuration (launch_config)
  uint64_t launchKey = 0;
  stats.launchMode = -1;
  const bool randomOrder = p.matchContextType == 0 || p.matchContextType == 1;
  // Wavefront runs prepare on the device (the directional orders too, in the
  // reference's exact order); replay uses the host preparation.
  const bool devicePrep = !replay && p.matchContextType >= 0 && p.matchContextType <= 8;
  HostPrep local;
  if (!devicePrep && !prepared) {
    std::vector<uint8_t> tHost((size_t)tw * th * f.total_bpp), cHost((size_t)cw * ch * f.total_bpp);
    CK(cudaMemcpyAsync(tHost.data(), dT, tHost.size(), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(cHost.data(), dC, cHost.size(), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    stats.d2hBytes += tHost.size() + cHost.size();
    const int rc = prepare(p, f, tHost.data(), tw, th, cHost.data(), cw, ch, local);
    if (rc) return rc;
    prepared = &local;
  }
  const int mw = (int)std::min(tw, cw), mh = (int)std::min(th, ch);
  const long long maxD2 = replay ? LLONG_MAX : wave_radius2(mw, mh);
  // Replay walks the reference's full list of this box; the wavefront walks
  // the shared device list restricted to the box.
  const std::vector<int2> noList;
  std::shared_ptr<const std::vector<int2>> offsHeld;
  int nWave = 0;
  const int2* dWave = replay ? nullptr : wave_offsets_device(nWave);
  if (dWave) {
    // only the prefix within this problem's radius (the list is sorted by d^2)
    const std::vector<int2>& wl = wave_offsets_host();
    nWave = (int)(std::partition_point(wl.begin(), wl.end(), [&](const int2& o) {
                    return (long long)o.x * o.x + (long long)o.y * o.y <= maxD2;
                  }) - wl.begin());
  }
  if (replay) offsHeld = cached_offsets(mw, mh, maxD2);
  const std::vector<int2>& offs = replay ? *offsHeld : noList;

  Arena ar(s);
  unsigned long long h2d = 0;
  unsigned launches = 0;
  cudaEvent_t e0, e1, epass;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(cudaEventCreateWithFlags(&epass, cudaEventDisableTiming));
  CK(cudaEventRecord(e0, s));
  DeviceProblem dp = make_problem(ar, s, p, f, dT, tw, th, dC, cw, ch, devicePrep ? nullptr : prepared->hasValue.data(),
                                  nullptr, offs, maxD2, h2d, launches, dWave, nWave);
  int2* dTargets = nullptr;
  unsigned ntargets = 0, ends[rs::kPasses], estimated = 0;
  bool noContext = true;
  if (devicePrep) {
    const size_t tn = (size_t)tw * th, cn = (size_t)cw * ch;
    int* scratch = ar.alloc<int>((size_t)std::max(rs_prep_scratch_ints((int)tw, (int)th), rs_prep_scratch_ints((int)cw, (int)ch)));
    int* dCounts = ar.alloc<int>(4);
    dTargets = ar.alloc<int2>(tn);
    int2* cpts = ar.alloc<int2>(cn);
    CK(rs_prep_target(dT, (int)tw, (int)th, f.total_bpp, f.alpha_bip, f.isAlphaTarget ? 1 : 0,
                      p.matchContextType ? 1 : 0, dp.pb.has, dp.pb.src, scratch, dTargets, dCounts, s));
    CK(rs_prep_corpus(dC, (int)cw, (int)ch, f.total_bpp, f.alpha_bip, f.isAlphaSource ? 1 : 0, scratch, cpts,
                      dCounts + 2, s));
    launches += 6;
    CK(cudaMemcpyAsync(st.hostInts, dCounts, 3 * sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    ntargets = (unsigned)st.hostInts[0];
    noContext = st.hostInts[1] == 0;
    const int ncorpus = st.hostInts[2];
    // lib/engine.c:605-627
    if (!ntargets) return IMAGE_SYNTH_ERROR_EMPTY_TARGET;
    if (!ncorpus) return IMAGE_SYNTH_ERROR_EMPTY_CORPUS;
    dp.pb.cpts = cpts;
    dp.pb.ncorpus = ncorpus;
    dp.pb.fullCorpus = (size_t)ncorpus == cn ? 1 : 0;
    pass_schedule(ntargets, ends, estimated);
    if (!randomOrder) {
      int2* ordered = ar.alloc<int2>(ntargets);
      unsigned long long d2h = 0;
      order_directional(p.matchContextType, dTargets, (int)ntargets, ordered, ar, st, s, h2d, d2h, launches);
      stats.d2hBytes += d2h;
      dTargets = ordered;
    }
  } else {
    HostPrep& hp = *prepared;
    ntargets = (unsigned)hp.targets.size();
    dTargets = ar.upload(reinterpret_cast<const int2*>(hp.targets.data()), hp.targets.size(), h2d);
    dp.pb.cpts = ar.upload(reinterpret_cast<const int2*>(hp.corpusPts.data()), hp.corpusPts.size(), h2d);
    dp.pb.ncorpus = (int)hp.corpusPts.size();
    dp.pb.fullCorpus = (size_t)dp.pb.ncorpus == (size_t)cw * ch ? 1 : 0;
    noContext = std::find(hp.hasValue.begin(), hp.hasValue.end(), 1) == hp.hasValue.end();
    std::copy(hp.ends, hp.ends + rs::kPasses, ends);
    estimated = hp.estimated;
  }
  rs::Counters* ctr = ar.alloc<rs::Counters>(1);
  CK(cudaMemsetAsync(ctr, 0, sizeof(rs::Counters), s));

  Progress prog;
  prog.estimated = estimated;
  prog.cb = progressCb;
  prog.ctx = ctx;
  unsigned bettersTotal = 0;

  if (replay) {
    HostPrep& hp = *prepared;
    // PRNG stream after the ordering draws; each visit draws at most trys.
    unsigned long long visitsMax = 0;
    for (int i = 0; i < rs::kPasses; i++) visitsMax += ends[i];
    const unsigned long long need = visitsMax * p.maxProbeCount + 1;
    if (need > (1ull << 30)) return fail(RESYNTH_ERROR_UNSUPPORTED, "replay mode: PRNG stream too long (%llu)", need);
    std::vector<int> stream(need);
    for (auto& v : stream) v = hp.rng.next();
    rs::ReplayArgs ra{};
    ra.pb = dp.pb;
    ra.targets = dTargets;
    ra.recentProber = ar.alloc<unsigned>((size_t)cw * ch);
    CK(cudaMemsetAsync(ra.recentProber, 0xFF, (size_t)cw * ch * sizeof(unsigned), s));
    ra.randStream = ar.upload(stream.data(), stream.size(), h2d);
    ra.randCount = (unsigned)stream.size();
    ra.trys = p.maxProbeCount;
    ra.ctr = ctr;
    rs::Counters& hc = *st.hostCtr;
    memset(&hc, 0, sizeof hc);
    for (int pass = 0; pass < rs::kPasses; pass++) {
      const unsigned end = ends[pass];
      const unsigned bettersBefore = hc.betters;
      for (unsigned t0 = 0; t0 < end; t0 += 4096u) {
        prog.tick();
        if (*cancel) break;
        const unsigned t1 = std::min(end, t0 + 4096u);
        CK(rs_launch_replay(ra, (int)t0, (int)t1, s));
        launches++;
        CK(cudaEventRecord(epass, s));
        wait_stream(st, epass, nullptr);
      }
      CK(cudaMemcpyAsync(&hc, ctr, sizeof hc, cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      if (hc.error) return fail(RESYNTH_ERROR_DEVICE, "replay kernel reported error %u", hc.error);
      const unsigned betters = hc.betters - bettersBefore;
      stats.passes = pass + 1;
      stats.passLength[pass] = end;
      stats.betters[pass] = betters;
      bettersTotal += betters;
      if ((float)betters / ntargets < 0.1) break;   // lib/refiner.h:111
    }
    stats.visits = 0;
    for (unsigned i = 0; i < stats.passes; i++) stats.visits += stats.passLength[i];
    stats.evals = hc.refEvals;
    stats.terms = hc.terms;
  } else {
    rs::WaveArgs wa{};
    wa.pb = dp.pb;
    wa.trys = p.maxProbeCount;
    wa.seed = opt.seed ? opt.seed : 1198472u;
    wa.ctr = ctr;
    wa.abortFlag = st.abortDev;
    // Schedule defaults chosen by energy sweeps (random orders: a tiny first
    // band of 16 pure-probe targets, bands growing 2x; directional orders:
    // bands of at least 1024 in visit order).
    const unsigned first = opt.firstBatch ? opt.firstBatch : (randomOrder ? wave_first_band(ntargets, noContext) : 1024u);
    const unsigned refine = opt.refineBatches ? opt.refineBatches : 1u;
    const double growth = (opt.bandGrowth ? opt.bandGrowth : wave_band_growth(dp.pb.nm)) / 100.0;
    const double growthLarge =
        (opt.bandGrowthLarge ? opt.bandGrowthLarge : dp.pb.nm ? wave_band_growth(dp.pb.nm) : kDefaultGrowthLarge) / 100.0;
    const int minPasses = wave_min_passes(opt, noContext, dp.pb.nm);
    const int k = opt.phaseSide ? (int)opt.phaseSide : phase_side_box(wave_offsets_host(), dp.pb.patchLimit, mw, mh);
    constexpr int kMaxBands = 64;
    // While no pixel outside the current pass has a value, a batch's patches
    // can come from the list of already-synthesized targets (cheap when short).
    wa.sparseLimit2 = 4LL * dp.pb.patchLimit * (long long)ntargets;
    const bool sparseOk = noContext && !dp.pb.tileH && !dp.pb.tileV;
    wa.stageSrc = ar.alloc<int2>(ntargets);
    rs::GridBar* gbar = ar.alloc<rs::GridBar>(1);
    unsigned* dQueue = ar.alloc<unsigned>((size_t)kMaxBands * k * k);
    int2* dPass = ar.alloc<int2>(ntargets);
    int* dBandEnds = ar.alloc<int>(kMaxBands);
    int* dBandPhased = ar.alloc<int>(kMaxBands);
    // Visit stamps replace hasValue writes: a pixel has a value for batch b of
    // pass 0 iff its stamp < b, and every target has one in later passes.
    int* vis = ar.alloc<int>((size_t)tw * th);
    CK(rs_vis_init(dp.pb.has, (int)(tw * th), vis, s));
    launches++;
    wa.pb.vis = vis;
    const bool tiled = dp.pb.tileH || dp.pb.tileV;
    const int cellsW = ((int)tw + rs::kCell - 1) >> rs::kCellShift, cellsH = ((int)th + rs::kCell - 1) >> rs::kCellShift;
    int* cellMin = tiled ? nullptr : ar.alloc<int>((size_t)cellsW * cellsH);
    int* batchStart = ar.alloc<int>((size_t)kMaxBands * k * k + 1);
    int* work = ar.alloc<int>(rs_prep_batches_ints((int)ntargets, kMaxBands * k * k));
    wa.targets = dPass;
    wa.batchStart = batchStart;
    // Proposal network: run once per band over the band's targets, with the
    // context the band starts from; its offsets join every visit's candidates.
    const TResynthNet* net = opt.net && opt.proposals ? opt.net : nullptr;
    int2* props = nullptr;
    if (net) {
      props = ar.alloc<int2>((size_t)ntargets * 16);
      wa.nprop = (int)std::min(16u, opt.proposals);
    }
    rs::Counters& hc = *st.hostCtr;
    LaunchTimer prof;
    // Warps per CTA: the caller's choice, or autotuned per problem class
    // (colour and map channels, patch size, corpus and target sizes): the
    // first refinement pass of a class times its first three batches with
    // 16, 8 and 4 warps and the fastest serves every later launch of the
    // class.  The result does not depend on the choice (exact minimum).
    const uint64_t tuneKey = (uint64_t)dp.pb.nc | (uint64_t)(dp.pb.nm > 0) << 2 | (uint64_t)dp.pb.patchLimit << 4 |
                             (uint64_t)ilog2((uint64_t)cw * ch) << 12 | (uint64_t)ilog2(ntargets) << 18;
    // The persistent pass (one cooperative launch per pass and grid class,
    // grid barriers between batches) or one launch per batch: chosen per
    // problem class across calls (launch_config), unless the caller fixes
    // it; the proposal network and graph capture keep one launch per batch.
    bool persistentRun = opt.batchLaunches != 1 && !net && !opt.graphs && rs_persistent_supported();
    int warps = 0;
    launchKey = tuneKey;
    if (persistentRun && !opt.warpsPerBlock && opt.batchLaunches == 0) {
      bool trial = false;
      launchCfg = launch_config(tuneKey, trial);
      if (!trial) launchCfg = -1 - launchCfg;   // settled: nothing to record
      const int c = (launchCfg >= 0 ? launchCfg : -1 - launchCfg) % kLaunchConfigs;
      persistentRun = c != kPerBatch;
      warps = c == kPersistent16 ? 16 : c == kPersistent8 ? 8 : tuned_warps(tuneKey);
    } else {
      warps = opt.warpsPerBlock ? (int)opt.warpsPerBlock : persistentRun ? 16 : tuned_warps(tuneKey);
    }
    stats.launchMode = !persistentRun ? kPerBatch : warps == 16 ? kPersistent16 : warps == 8 ? kPersistent8 : 3;
    // Problems whose corpus is read from global memory share their random
    // probes within groups of 16 consecutive batch slots: a CTA's warps then
    // read the same corpus windows (cache reuse; heal4096 18 % faster).  On
    // the CPU restatement the energy with sharing over without is 0.97-1.00
    // (heal 512^2 and 1024^2, render 256^2 and 512^2, map-guided 512^2; four
    // seeds each).  Problems whose corpus sits in shared memory keep
    // per-pixel probes.
    wa.probeShare = opt.probeShare == 1 ? 1 : opt.probeShare == 2 ? 0 : rs_wave_corpus_staged(dp.pb, 16) ? 0 : 1;
    const bool autoWarps = opt.warpsPerBlock == 0 && warps == 0;
    if (!warps) warps = 16;
    static const int kTryWarps[3] = {16, 8, 4};
    cudaEvent_t tev[4] = {};
    for (int pass = 0; pass < rs::kPasses; pass++) {
      const unsigned end = ends[pass];
      // Bands of the visit order (rank thresholds): pass 0 grows
      // geometrically for random orders and is cut into equal widths for the
      // directional orders; refinement passes split their prefix evenly.
      std::vector<int> bandEnds;
      if (pass == 0) {
        double size = randomOrder ? first : std::max<double>(first, std::ceil((double)end / kMaxBands));
        double b = 0;
        while (b < end && (int)bandEnds.size() < kMaxBands - 1) {
          b = std::min<double>(end, b + std::max(1.0, size));
          bandEnds.push_back((int)b);
          if (randomOrder) size *= size * 64 < end ? growth : growthLarge;
        }
        if (bandEnds.back() < (int)end) bandEnds.push_back((int)end);
      } else {
        for (unsigned r = 1; r <= refine; r++) bandEnds.push_back((int)((unsigned long long)end * r / refine));
      }
      const int nb = (int)bandEnds.size();
      // Every band is split into colour phases.  (Leaving sparse pass-0 bands
      // whole saves batches but costs energy: same-band targets then miss each
      // other inside their wide sparse patches.)
      std::vector<int> phased(nb, 1);
      CK(cudaMemcpyAsync(dBandEnds, bandEnds.data(), nb * sizeof(int), cudaMemcpyHostToDevice, s));
      CK(cudaMemcpyAsync(dBandPhased, phased.data(), nb * sizeof(int), cudaMemcpyHostToDevice, s));
      h2d += 2 * nb * sizeof(int);
      // With graphs, the pass's launches (bucketing, cell minima, proposals,
      // the batches) are captured and launched as one CUDA graph; timing and
      // tuning passes use plain launches.
      const bool tuningPass = autoWarps && pass == 1;
      const bool graphPass = opt.graphs && !opt.profile && !tuningPass;
      if (graphPass) CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      // Bucket this pass's targets by (band, colour phase): targets of one
      // phase are at least k apart, farther than a dense patch reaches, so
      // the targets of one batch never read each other.
      CK(rs_prep_batches(dTargets, (int)ntargets, (int)tw, (int)end, randomOrder ? 1 : 0, wa.seed ^ 0x5bd1e995u,
                         dBandEnds, dBandPhased, nb, k, work, batchStart, dPass, pass == 0 ? vis : nullptr, s));
      launches += 4;
      // Pass 0: the least visit stamp per cell lets far-reaching patches skip
      // the empty parts of the image (no wrapping: tiled targets walk the list).
      // Pass-0 stores go straight into the state: no target of a batch reads
      // another (visit stamps).  Later passes read every neighbour, and near
      // the image border a patch reaches past the colour-phase spacing, so
      // their results are staged and applied after each batch; so are those
      // of wrapping (tiled) targets, whose phases can meet across the seam.
      wa.inPlace = (tiled || pass > 0) ? 0 : 1;
      wa.pb.cellMin = nullptr;
      if (pass == 0 && cellMin) {
        CK(rs_cell_min(vis, (int)tw, (int)th, cellMin, s));
        launches++;
        wa.pb.cellMin = cellMin;
        wa.pb.cellsW = cellsW;
        wa.pb.cellsH = cellsH;
      }
      const int nbatches = nb * k * k;
      // the network's proposals in every pass, or in the first proposalPasses
      const bool netPass = net && (!opt.proposalPasses || pass < (int)opt.proposalPasses);
      if (!netPass) wa.props = nullptr;
      wa.pass = (unsigned)pass;
      wa.sparse = (pass == 0 && sparseOk) ? 1 : 0;
      const bool tuning = autoWarps && pass == 1 && nbatches >= 3;
      if (tuning)
        for (auto& e : tev) CK(cudaEventCreate(&e));
      int maxCtas = 0, maxCommit = 0;
      // Persistent pass: the batches run in one cooperative launch with a grid
      // barrier between them (a tuning pass first times its first three
      // batches as single launches).  The proposal network runs between the
      // bands, and graph capture records per-batch launches, so those passes
      // keep one launch per batch.
      const bool persistent = persistentRun;
      const int singleEnd = persistent ? (tuning ? std::min(3, nbatches) : 0) : nbatches;
      for (int b = 0; b < singleEnd; b++) {
        if (!phased[b / (k * k)] && b % (k * k)) continue;   // empty by construction
        if (b % (k * k) == 0) {
          // Grid cap from the band's expected batch size (its targets spread
          // over k * k phases; twice that for the spread): small batches get
          // one CTA per target instead of a persistent grid of idle CTAs.
          const int band = b / (k * k);
          const long long count = bandEnds[band] - (band ? bandEnds[band - 1] : 0);
          const long long expect = 2 * ((count + k * k - 1) / (k * k)) + 4;
          maxCtas = expect < 1 << 20 ? (int)expect : 0;
          maxCommit = (int)std::min<long long>(1 << 20, expect / 256 + 1);
        }
        if (netPass && b % (k * k) == 0) {
          const int band = b / (k * k);
          const int count = bandEnds[band] - (band ? bandEnds[band - 1] : 0);
          CK(rs_net_propose(net, wa.pb, dPass, batchStart, b, b + k * k, count, pass == 0 ? b : 0x7ffffffe, props,
                            &ctr->error, s));
          launches++;
          wa.props = props;
          wa.propBatch0 = b;
        }
        wa.batch = b;
        wa.visCur = pass == 0 ? b : 0x7ffffffe;
        const int w = tuning && b < 3 ? kTryWarps[b] : warps;
        if (tuning && b < 3) CK(cudaEventRecord(tev[b], s));
        if (opt.profile) prof.begin(s);
        CK(rs_launch_wave(wa, w, maxCtas, s));
        if (opt.profile) prof.end(s);
        launches++;
        if (!wa.inPlace) {
          CK(rs_launch_commit(wa, maxCommit, s));
          launches++;
        }
        if (tuning && b == 2) CK(cudaEventRecord(tev[3], s));
      }
      // The rest of the pass, after the single launches it depends on.  A
      // launch's grid fits its bands: a band's batches want about twice their
      // expected size in CTAs (one team per target, with slack for the
      // spread), so runs of consecutive bands are grouped into grid classes
      // of at most 32 CTAs, at most 128, and the whole GPU.  Small pass-0
      // bands then meet at barriers of few CTAs; large ones use every SM.
      if (persistent && singleEnd < nbatches) {
        auto gridClass = [&](int b) {
          const int band = b / (k * k);
          const long long count = bandEnds[band] - (band ? bandEnds[band - 1] : 0);
          const long long want = 2 * ((count + k * k - 1) / (k * k)) + 4;
          return want <= 32 ? 32 : want <= 128 ? 128 : 0;
        };
        wa.gbar = gbar;
        wa.barTimeoutNs = kBarrierTimeoutNs;
        for (int b = singleEnd; b < nbatches;) {
          const int cls = gridClass(b);
          int e = b + 1;
          while (e < nbatches && gridClass(e) == cls) e++;
          wa.batch = b;
          wa.batchEnd = e;
          wa.queue = dQueue;
          CK(cudaMemsetAsync(gbar, 0, sizeof(rs::GridBar), s));
          CK(cudaMemsetAsync(dQueue + b, 0, (size_t)(e - b) * sizeof(unsigned), s));
          if (opt.profile) prof.begin(s);
          CK(rs_launch_wave_persistent(wa, warps, cls, s));
          if (opt.profile) prof.end(s);
          launches++;
          b = e;
        }
      }
      cudaGraphExec_t passExec = nullptr;
      if (graphPass) {
        cudaGraph_t graph = nullptr;
        CK(cudaStreamEndCapture(s, &graph));
        const cudaError_t ie = cudaGraphInstantiate(&passExec, graph, 0);
        cudaGraphDestroy(graph);
        CK(ie);
        CK(cudaGraphLaunch(passExec, s));
      }
      CK(cudaMemcpyAsync(&hc, ctr, sizeof hc, cudaMemcpyDeviceToHost, s));
      CK(cudaMemcpyAsync(st.hostInts + 3, batchStart + nbatches, sizeof(int), cudaMemcpyDeviceToHost, s));
      CK(cudaEventRecord(epass, s));
      wait_stream(st, epass, cancel);
      if (passExec) cudaGraphExecDestroy(passExec);
      if (hc.error) return fail(RESYNTH_ERROR_DEVICE, "wavefront kernel reported error %u", hc.error);
      if (tuning) {
        float t[3];
        for (int i = 0; i < 3; i++) CK(cudaEventElapsedTime(&t[i], tev[i], tev[i + 1]));
        int best = 0;
        for (int i = 1; i < 3; i++)
          if (t[i] < 0.97f * t[best]) best = i;
        set_tuned_warps(tuneKey, kTryWarps[best]);
        warps = kTryWarps[best];
        for (auto& e : tev) cudaEventDestroy(e);
      }
      const unsigned visited = (unsigned)st.hostInts[3];
      // callbacks the reference makes during this pass (lib/synthesize.h:493)
      for (unsigned t = 0; t < end; t += 4096u) prog.tick();
      const unsigned betters = hc.betters - bettersTotal;
      bettersTotal = hc.betters;
      stats.passes = pass + 1;
      stats.passLength[pass] = visited;
      stats.betters[pass] = betters;
      if (*cancel || *st.abortHost) break;
      if ((float)betters / ntargets < 0.1 && pass + 1 >= minPasses) break;   // lib/refiner.h:111
    }
    stats.visits = 0;
    for (unsigned i = 0; i < stats.passes; i++) stats.visits += stats.passLength[i];
    stats.evals = hc.evals;
    stats.terms = hc.terms;
    if (opt.dumpPairs) {
      CK(rs_net_dump(opt.dumpPairs, wa.pb, dTargets, (int)ntargets, opt.dumpStride, s));
      launches++;
    }
    CK(rs_vis_to_has(vis, (int)(tw * th), dp.pb.has, s));
    launches++;
    if (opt.profile) {
      CK(cudaStreamSynchronize(s));
      stats.waveMs = prof.total();
      stats.waveLaunches = prof.count();
      stats.waveTerms = hc.terms;
    }
  }
  CK(rs_launch_unpack_colors(dT, (int)tw, (int)th, f.total_bpp, f.img_match_bpp, dp.tpx, s));
  launches++;
  CK(cudaEventRecord(e1, s));
  if (opt.recordState) {
    g_state.w = tw;
    g_state.h = th;
    g_state.src.resize((size_t)tw * th);
    g_state.has.resize((size_t)tw * th);
    CK(cudaMemcpyAsync(g_state.src.data(), dp.pb.src, g_state.src.size() * sizeof(int2), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(g_state.has.data(), dp.pb.has, g_state.has.size(), cudaMemcpyDeviceToHost, s));
  }
  CK(cudaStreamSynchronize(s));
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, e0, e1));
  stats.deviceMs = ms;
  if (launchCfg >= 0 && !*cancel && !*st.abortHost) launch_result(launchKey, launchCfg, ms);
  stats.launches += launches;
  stats.h2dBytes += h2d;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaEventDestroy(epass);
  return 0;
}

// ------------------------------------------------- many requests at once
// imageSynthBatch's wavefront path for requests with a random order: every
// request is set up on one stream (device adaption, packing, device
// preparation), then each pass buckets every request and runs step b -- batch
// b of every request still active -- as one launch per pixel layout, the
// requests' slots concatenated.  The per-request results equal single calls
// (same batches, probes and patches; the minimum does not depend on the team
// layout).

struct BatchJob {
  TResynthRequest* req = nullptr;
  TImageSynthParameters p{};
  TFormatIndices f{};
  unsigned w = 0, h = 0, bpp = 0;
  size_t imgBytes = 0;
  uint8_t* dImg = nullptr;
  uint8_t* dT = nullptr;
  DeviceProblem dp;
  int2* dTargets = nullptr;
  int2* cpts = nullptr;
  unsigned ntargets = 0, ends[rs::kPasses] = {}, estimated = 0;
  bool noContext = true, tiled = false, active = false;
  int k = 1, cellsW = 0, cellsH = 0;
  int* vis = nullptr;
  int* cellMin = nullptr;
  int* batchStart = nullptr;
  int* work = nullptr;
  int2* dPass = nullptr;
  int* dBandEnds = nullptr;
  int* dBandPhased = nullptr;
  std::vector<int> bandEnds;
  rs::WaveArgs wa{};
  unsigned bettersTotal = 0, passes = 0;
  int setupIdx = -1;             // entry in the call's set-up list (-1: failed a host check)
};

bool batch_eligible(const TResynthRequest& r, const TResynthOptions& opt) {
  if (opt.mode == RESYNTH_MODE_REPLAY || opt.net || opt.dumpPairs || opt.recordState || opt.profile) return false;
  if (!r.image || !r.mask) return false;
  const int ctx = r.parameters ? r.parameters->matchContextType : 1;
  return ctx == 0 || ctx == 1;
}

int run_batch_wave(std::vector<TResynthRequest*>& reqs, const TResynthOptions& opt, TResynthStats& stats) {
  Stream& st = thread_stream();
  cudaStream_t s = st.s;
  Arena ar(s, (size_t)256 << 20);
  constexpr int kMaxBands = 64;
  std::vector<BatchJob> jobs(reqs.size());
  unsigned long long h2d = 0, d2h = 0;
  unsigned launches = 0;
  cudaEvent_t e0, e1, epass;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(cudaEventCreateWithFlags(&epass, cudaEventDisableTiming));
  CK(cudaEventRecord(e0, s));
  *st.abortHost = 0;
  // Requests' uploads and preparation run on the side streams, each with its
  // own arena; on every way out, s first waits for the side streams, then the
  // side arenas free on s.
  struct SideArenas {
    Stream& st;
    std::vector<std::unique_ptr<Arena>> a;
    ~SideArenas() {
      try {
        st.join_side();
      } catch (...) {
      }
    }
  } side{st, {}};
  st.fork_side();
  for (int q = 0; q < Stream::kSide; q++) side.a.emplace_back(new Arena(st.side[q], (size_t)64 << 20, s));
  int nextSide = 0;
  std::vector<rs::SetupJob> setup;
  std::vector<int> setupChunk0;
  int setupChunks = 0, maxPx = 1;
  std::map<std::pair<double, double>, const uint32_t*> tables;   // metric tables by (sensitivity, mapWeight)
  // 1. host checks (the reference's order), upload
  for (size_t i = 0; i < reqs.size(); i++) {
    BatchJob& J = jobs[i];
    TResynthRequest& R = *reqs[i];
    J.req = &R;
    R.result = 0;
    if (R.image->width != R.mask->width || R.image->height != R.mask->height) {
      R.result = IMAGE_SYNTH_ERROR_IMAGE_MASK_MISMATCH;
      continue;
    }
    if (R.parameters) J.p = *R.parameters;
    else setDefaultParams(&J.p);
    if ((R.result = prepareImageFormatIndicesFromFormatType(&J.f, R.format))) continue;
    if (J.p.patchSize > (unsigned)rs::kMaxNeighbors) {
      R.result = IMAGE_SYNTH_ERROR_PATCH_SIZE_EXCEEDED;
      continue;
    }
    J.bpp = countPixelelsPerPixelForFormat(R.format);
    J.w = R.image->width;
    J.h = R.image->height;
    const unsigned w = J.w, h = J.h, d = J.bpp + 1;
    ImageBuffer* img = R.image;
    ImageBuffer* cm = R.mask2 ? R.mask2 : R.mask;
    bool anyTarget = false, anyCorpus = false;
    for (unsigned y = 0; y < h && !anyTarget; y++)
      for (unsigned x = 0; x < w && !anyTarget; x++) anyTarget = R.mask->data[y * R.mask->rowBytes + x] != 0;
    if (!anyTarget) {
      R.result = IMAGE_SYNTH_ERROR_EMPTY_TARGET;
      continue;
    }
    for (unsigned y = 0; y < h && !anyCorpus; y++)
      for (unsigned x = 0; x < w && !anyCorpus; x++) {
        const uint8_t m = cm->data[y * cm->rowBytes + x];
        const uint8_t cmask = R.mask2 ? m : (uint8_t)~m;
        anyCorpus = cmask == 0xFF &&
                    (!J.f.isAlphaSource || img->data[y * img->rowBytes + (size_t)x * J.bpp + J.f.alpha_bip - 1] != 0);
      }
    if (!anyCorpus) {
      R.result = IMAGE_SYNTH_ERROR_EMPTY_CORPUS;
      continue;
    }
    // Buffers from the side arenas, the caller's buffers uploaded as they are
    // (row padding included) on the side streams; the set-up kernels below
    // serve every request at once.
    const int sq = nextSide++ % Stream::kSide;
    const cudaStream_t q = st.side[sq];
    Arena& qa = *side.a[sq];
    J.imgBytes = img->rowBytes * (h - 1) + (size_t)w * J.bpp;
    const size_t mBytes = R.mask->rowBytes * (h - 1) + w;
    J.dImg = qa.alloc<uint8_t>(img->rowBytes * h);
    uint8_t* dMask = qa.alloc<uint8_t>(R.mask->rowBytes * h);
    uint8_t* dMask2 = R.mask2 ? qa.alloc<uint8_t>(R.mask2->rowBytes * h) : nullptr;
    CK(cudaMemcpyAsync(J.dImg, img->data, J.imgBytes, cudaMemcpyHostToDevice, q));
    CK(cudaMemcpyAsync(dMask, R.mask->data, mBytes, cudaMemcpyHostToDevice, q));
    h2d += J.imgBytes + mBytes;
    if (R.mask2) {
      const size_t m2Bytes = R.mask2->rowBytes * (h - 1) + w;
      CK(cudaMemcpyAsync(dMask2, R.mask2->data, m2Bytes, cudaMemcpyHostToDevice, q));
      h2d += m2Bytes;
    }
    const size_t tn = (size_t)w * h, tnPad = (tn + 3) & ~(size_t)3;
    J.dT = qa.alloc<uint8_t>(tn * d);
    uint8_t* dC = qa.alloc<uint8_t>(tn * d);
    rs::Problem& pb = J.dp.pb;
    pb.tw = pb.cw = (int)w;
    pb.th = pb.ch = (int)h;
    pb.nc = J.f.img_match_bpp;
    pb.nm = 0;
    J.dp.tpx = qa.alloc<uint32_t>(tn);
    pb.tpx = J.dp.tpx;
    pb.cpx = qa.alloc<uint32_t>(tnPad);
    pb.padW = (int)w + 2 * rs::kPad;
    pb.cpxPad = qa.alloc<uint32_t>((((size_t)pb.padW * (h + 2 * rs::kPad)) + 3) & ~(size_t)3);
    pb.has = qa.alloc<uint8_t>(tn);
    pb.src = qa.alloc<int2>(tn);
    J.vis = qa.alloc<int>(tn);
    pb.vis = J.vis;
    J.dTargets = qa.alloc<int2>(tn);
    J.cpts = qa.alloc<int2>(tn);
    const long long maxD2 = wave_radius2((int)w, (int)h);
    int nWave = 0;
    pb.offs = wave_offsets_device(nWave);
    const std::vector<int2>& wl = wave_offsets_host();
    pb.noffs = (int)(std::partition_point(wl.begin(), wl.end(), [&](const int2& o) {
                       return (long long)o.x * o.x + (long long)o.y * o.y <= maxD2;
                     }) - wl.begin());
    pb.boxW = (int)w;
    pb.boxH = (int)h;
    pb.maxD2 = maxD2;
    pb.patchLimit = (int)std::max(J.p.patchSize, 2u);
    pb.tileH = J.p.isMakeSeamlesslyTileableHorizontally ? 1 : 0;
    pb.tileV = J.p.isMakeSeamlesslyTileableVertically ? 1 : 0;
    uint32_t ct[512], mt[512];
    metric_tables(J.p.sensitivityToOutliers, J.p.mapWeight, ct, mt);
    pb.clipCost = 65535u * J.f.img_match_bpp;
    const auto key = std::make_pair(J.p.sensitivityToOutliers, J.p.mapWeight);
    auto tab = tables.find(key);
    if (tab == tables.end()) {
      uint32_t both[1024];
      std::copy(ct, ct + 512, both);
      std::copy(mt, mt + 512, both + 512);
      const uint32_t* dTab = qa.upload(both, 1024, h2d);
      tab = tables.emplace(key, dTab).first;
    }
    pb.ctab = tab->second;
    pb.mtab = tab->second + 512;
    rs::SetupJob S{};
    S.img = J.dImg;
    S.imgRow = img->rowBytes;
    S.mask = dMask;
    S.maskRow = R.mask->rowBytes;
    S.mask2 = dMask2;
    S.mask2Row = R.mask2 ? R.mask2->rowBytes : 0;
    S.w = (int)w;
    S.h = (int)h;
    S.bpp = (int)J.bpp;
    S.nc = J.f.img_match_bpp;
    S.alpha = J.f.alpha_bip;
    S.alphaT = J.f.isAlphaTarget ? 1 : 0;
    S.alphaS = J.f.isAlphaSource ? 1 : 0;
    S.useContext = J.p.matchContextType ? 1 : 0;
    S.target = J.dT;
    S.corpus = dC;
    S.tpx = pb.tpx;
    S.cpx = const_cast<uint32_t*>(pb.cpx);
    S.cpxPad = const_cast<uint32_t*>(pb.cpxPad);
    S.padW = pb.padW;
    S.has = pb.has;
    S.src = pb.src;
    S.vis = J.vis;
    S.targets = J.dTargets;
    S.cpts = J.cpts;
    S.chunk0 = setupChunks;
    J.setupIdx = (int)setup.size();
    setup.push_back(S);
    setupChunk0.push_back(setupChunks);
    setupChunks += rs_setup_chunks((int)tn);
    maxPx = std::max(maxPx, (int)std::max(tn, (size_t)pb.padW * (h + 2 * rs::kPad)));
  }
  st.join_side();
  // 2. every request's adaption, packing, initial state and compaction in
  // four launches; their target and corpus counts in one read-back
  setupChunk0.push_back(setupChunks);
  rs::SetupJob* dSetup = setup.empty() ? nullptr : ar.upload(setup.data(), setup.size(), h2d);
  const int* dSetupChunk0 = setup.empty() ? nullptr : ar.upload(setupChunk0.data(), setupChunk0.size(), h2d);
  int* dCountsAll = ar.alloc<int>(4 * std::max<size_t>(1, setup.size()));
  int* setupWork = ar.alloc<int>(rs_setup_work_ints(setupChunks, (int)setup.size()) + 1);
  CK(rs_setup_multi(dSetup, dSetupChunk0, (int)setup.size(), setupChunks, maxPx, dCountsAll, setupWork, s));
  launches += setup.empty() ? 0 : 4;
  std::vector<int> countsAll(4 * setup.size(), 0);
  if (!setup.empty())
    CK(cudaMemcpyAsync(countsAll.data(), dCountsAll, countsAll.size() * sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  d2h += countsAll.size() * sizeof(int);
  rs::Counters* ctrs = ar.alloc<rs::Counters>(jobs.size());
  CK(cudaMemsetAsync(ctrs, 0, jobs.size() * sizeof(rs::Counters), s));
  // every request's band boundaries and phase flags, uploaded once per pass
  int* dBands = ar.alloc<int>(jobs.size() * 2 * kMaxBands);
  for (size_t i = 0; i < jobs.size(); i++) {
    BatchJob& J = jobs[i];
    if (J.setupIdx < 0) continue;
    const int* c = &countsAll[4 * (size_t)J.setupIdx];
    J.ntargets = (unsigned)c[0];
    J.noContext = c[1] == 0;
    const int ncorpus = c[2];
    if (!J.ntargets) {   // lib/engine.c:605-627
      J.req->result = IMAGE_SYNTH_ERROR_EMPTY_TARGET;
      continue;
    }
    if (!ncorpus) {
      J.req->result = IMAGE_SYNTH_ERROR_EMPTY_CORPUS;
      continue;
    }
    rs::Problem& pb = J.dp.pb;
    pb.cpts = J.cpts;
    pb.ncorpus = ncorpus;
    pb.fullCorpus = (size_t)ncorpus == (size_t)J.w * J.h ? 1 : 0;
    pass_schedule(J.ntargets, J.ends, J.estimated);
    J.k = opt.phaseSide ? (int)opt.phaseSide : phase_side_box(wave_offsets_host(), pb.patchLimit, (int)J.w, (int)J.h);
    J.tiled = pb.tileH || pb.tileV;
    J.cellsW = ((int)J.w + rs::kCell - 1) >> rs::kCellShift;
    J.cellsH = ((int)J.h + rs::kCell - 1) >> rs::kCellShift;
    J.cellMin = J.tiled ? nullptr : ar.alloc<int>((size_t)J.cellsW * J.cellsH);
    J.batchStart = ar.alloc<int>((size_t)kMaxBands * J.k * J.k + 1);
    J.work = ar.alloc<int>(rs_prep_batches_ints((int)J.ntargets, kMaxBands * J.k * J.k));
    J.dPass = ar.alloc<int2>(J.ntargets);
    J.dBandEnds = dBands + i * 2 * kMaxBands;
    J.dBandPhased = J.dBandEnds + kMaxBands;
    rs::WaveArgs& wa = J.wa;
    wa.pb = pb;
    wa.trys = J.p.maxProbeCount;
    wa.seed = opt.seed ? opt.seed : 1198472u;
    wa.ctr = ctrs + i;
    wa.abortFlag = st.abortDev;
    wa.sparseLimit2 = 4LL * pb.patchLimit * (long long)J.ntargets;
    wa.stageSrc = ar.alloc<int2>(J.ntargets);
    wa.targets = J.dPass;
    wa.batchStart = J.batchStart;
    wa.probeShare = opt.probeShare == 1 ? 1 : opt.probeShare == 2 ? 0 : rs_wave_corpus_staged(pb, 16) ? 0 : 1;
    J.active = true;
  }
  // 3. passes
  std::vector<rs::Counters> hostCtr(jobs.size());
  std::vector<int> visited(jobs.size(), 0);
  rs::WaveArgs* dJobs = ar.alloc<rs::WaveArgs>(jobs.size());
  int* dPrefix = ar.alloc<int>(jobs.size() + 1);
  std::vector<rs::WaveArgs> hJobs;
  // Persistent passes (one cooperative launch per pixel layout and pass), or
  // one launch per step with options->batchLaunches.
  const bool persistent = opt.batchLaunches != 1 && rs_persistent_supported();
  rs::GridBar* gbar = ar.alloc<rs::GridBar>(1);
  CK(cudaMemsetAsync(gbar, 0, sizeof(rs::GridBar), s));
  unsigned* barErr = reinterpret_cast<unsigned*>(st.hostInts + 8);   // pinned: read back with the counters
  *barErr = 0;
  for (int pass = 0; pass < rs::kPasses; pass++) {
    std::vector<size_t> act;
    for (size_t i = 0; i < jobs.size(); i++)
      if (jobs[i].active) act.push_back(i);
    if (act.empty()) break;
    // Band boundaries of the pass for every active request, one upload.
    int* hb = st.host_bands(jobs.size() * 2 * kMaxBands);
    for (size_t i : act) {
      BatchJob& J = jobs[i];
      const unsigned end = J.ends[pass];
      // pass-0 bands grow 2x from 16 (random orders); later passes one band
      J.bandEnds.clear();
      if (pass == 0) {
        double size = opt.firstBatch ? opt.firstBatch : wave_first_band(J.ntargets, J.noContext), b = 0;
        const double growth = (opt.bandGrowth ? opt.bandGrowth : wave_band_growth(J.dp.pb.nm)) / 100.0;
        const double growthLarge = (opt.bandGrowthLarge ? opt.bandGrowthLarge
                                    : J.dp.pb.nm ? wave_band_growth(J.dp.pb.nm) : kDefaultGrowthLarge) / 100.0;
        while (b < end && (int)J.bandEnds.size() < kMaxBands - 1) {
          b = std::min<double>(end, b + std::max(1.0, size));
          J.bandEnds.push_back((int)b);
          size *= size * 64 < end ? growth : growthLarge;
        }
        if (J.bandEnds.back() < (int)end) J.bandEnds.push_back((int)end);
      } else {
        const unsigned refine = opt.refineBatches ? opt.refineBatches : 1u;
        for (unsigned r = 1; r <= refine; r++) J.bandEnds.push_back((int)((unsigned long long)end * r / refine));
      }
      int* h = hb + i * 2 * kMaxBands;
      std::copy(J.bandEnds.begin(), J.bandEnds.end(), h);
      std::fill(h + kMaxBands, h + kMaxBands + J.bandEnds.size(), 1);
    }
    CK(cudaMemcpyAsync(dBands, hb, jobs.size() * 2 * kMaxBands * sizeof(int), cudaMemcpyHostToDevice, s));
    h2d += jobs.size() * 2 * kMaxBands * sizeof(int);
    // Every active request's bucketing of the pass (and its pass-0 cell
    // minima) in five launches: the requests' entries go up in one copy.
    std::vector<rs::PrepJob> pj;
    std::vector<int> chunk0;
    int totalChunks = 0, maxKeys = 1, maxCells = 0;
    pj.reserve(act.size());
    for (size_t i : act) {
      BatchJob& J = jobs[i];
      const int k = J.k;
      const int nb = (int)J.bandEnds.size();
      const int nkeys = nb * k * k, nchunks = rs_prep_chunks((int)J.ntargets);
      const size_t cells = (size_t)nkeys * nchunks;
      rs::PrepJob P{};
      P.targets = J.dTargets;
      P.n = (int)J.ntargets;
      P.tw = (int)J.w;
      P.th = (int)J.h;
      P.endRank = (int)J.ends[pass];
      P.randomOrder = 1;
      P.seed = J.wa.seed ^ 0x5bd1e995u;
      P.bandEnds = J.dBandEnds;
      P.bandPhased = J.dBandPhased;
      P.nbands = nb;
      P.k = k;
      P.counts = J.work;
      P.offsets = J.work + cells;
      P.keys = J.work + 2 * cells + 1;
      P.nchunks = nchunks;
      P.batchStart = J.batchStart;
      P.out = J.dPass;
      P.vis = pass == 0 ? J.vis : nullptr;
      P.cellMin = pass == 0 ? J.cellMin : nullptr;
      chunk0.push_back(totalChunks);
      totalChunks += nchunks;
      maxKeys = std::max(maxKeys, nkeys);
      if (P.cellMin) maxCells = std::max(maxCells, J.cellsW * J.cellsH);
      pj.push_back(P);
      J.wa.inPlace = (J.tiled || pass > 0) ? 0 : 1;
      J.wa.pb.cellMin = P.cellMin;
      if (P.cellMin) {
        J.wa.pb.cellsW = J.cellsW;
        J.wa.pb.cellsH = J.cellsH;
      }
      J.wa.pass = (unsigned)pass;
      J.wa.sparse = (pass == 0 && J.noContext && !J.tiled) ? 1 : 0;
      J.wa.nbatches = nkeys;
    }
    chunk0.push_back(totalChunks);
    const rs::PrepJob* dPJ = ar.upload(pj.data(), pj.size(), h2d);
    const int* dChunk0 = ar.upload(chunk0.data(), chunk0.size(), h2d);
    const int cellBlocks = maxCells ? std::min(64, (maxCells + 7) / 8) : 0;
    CK(rs_prep_batches_multi(dPJ, dChunk0, (int)pj.size(), totalChunks, maxKeys, cellBlocks, s));
    launches += cellBlocks ? 5 : 4;
    // requests grouped by pixel layout, one launch per group per step
    std::map<std::pair<int, int>, std::vector<size_t>> groups;
    for (size_t i : act) groups[{jobs[i].dp.pb.nc, jobs[i].dp.pb.nm > 0 ? 1 : 0}].push_back(i);
    for (auto& g : groups) {
      const std::vector<size_t>& idx = g.second;
      hJobs.clear();
      int steps = 0;
      bool staged = false;
      for (size_t i : idx) {
        hJobs.push_back(jobs[i].wa);
        steps = std::max(steps, jobs[i].wa.nbatches);
        staged |= !jobs[i].wa.inPlace;
      }
      CK(cudaMemcpyAsync(dJobs, hJobs.data(), hJobs.size() * sizeof(rs::WaveArgs), cudaMemcpyHostToDevice, s));
      h2d += hJobs.size() * sizeof(rs::WaveArgs);
      const int n = (int)idx.size();
      if (persistent) {
        // The whole pass of this layout's requests in one cooperative launch
        // per chunk of requests: every step's slot prefix first, then the
        // steps with a work queue each and a grid barrier between them.
        for (int c0 = 0; c0 < n; c0 += rs::kMultiPersistentMaxRequests) {
          const int cn = std::min(n - c0, rs::kMultiPersistentMaxRequests);
          int* dPrefixAll = ar.alloc<int>((size_t)steps * (cn + 1));
          unsigned* dQueue = ar.alloc<unsigned>((size_t)steps);
          CK(rs_launch_multi_prefix_all(dJobs + c0, cn, steps, dPrefixAll, s));
          CK(cudaMemsetAsync(dQueue, 0, (size_t)steps * sizeof(unsigned), s));
          // count, generation and stop word; the error word collects the whole call
          CK(cudaMemsetAsync(gbar, 0, offsetof(rs::GridBar, error), s));
          CK(rs_launch_wave_multi_persistent(dJobs + c0, cn, steps, dPrefixAll, dQueue, pass, staged ? 1 : 0, gbar,
                                             st.abortDev, g.first.first, g.first.second, kBarrierTimeoutNs, s));
          launches += 2;
        }
        continue;
      }
      for (int b = 0; b < steps; b++) {
        // grid cap from the expected step size: each request's band spread
        // over its k * k phases, twice that for the spread
        long long expect = 4;
        for (size_t i : idx) {
          const BatchJob& J = jobs[i];
          if (b >= J.wa.nbatches) continue;
          const int band = b / (J.k * J.k);
          const long long c = J.bandEnds[band] - (band ? J.bandEnds[band - 1] : 0);
          expect += 2 * ((c + J.k * J.k - 1) / (J.k * J.k));
        }
        const int maxCtas = expect < (1 << 20) ? (int)expect : 0;
        CK(rs_launch_multi_prefix(dJobs, n, b, dPrefix, s));
        CK(rs_launch_wave_multi(dJobs, n, dPrefix, b, pass == 0 ? b : 0x7ffffffe, g.first.first, g.first.second,
                                maxCtas, st.abortDev, s));
        launches += 2;
        if (staged) {
          CK(rs_launch_commit_multi(dJobs, n, dPrefix, b, (int)std::min<long long>(1 << 20, expect / 256 + 1), s));
          launches++;
        }
      }
    }
    CK(cudaMemcpyAsync(hostCtr.data(), ctrs, jobs.size() * sizeof(rs::Counters), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(barErr, &gbar->error, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    for (size_t i : act)
      CK(cudaMemcpyAsync(&visited[i], jobs[i].batchStart + jobs[i].wa.nbatches, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaEventRecord(epass, s));
    wait_stream(st, epass, nullptr);
    if (*barErr) return fail(RESYNTH_ERROR_DEVICE, "many-request wavefront kernel reported error %u", *barErr);
    for (size_t i : act) {
      BatchJob& J = jobs[i];
      const rs::Counters& c = hostCtr[i];
      if (c.error) return fail(RESYNTH_ERROR_DEVICE, "wavefront kernel reported error %u", c.error);
      const unsigned betters = c.betters - J.bettersTotal;
      J.bettersTotal = c.betters;
      J.passes = pass + 1;
      stats.visits += (unsigned)visited[i];
      if ((float)betters / J.ntargets < 0.1 && pass + 1 >= wave_min_passes(opt, J.noContext, J.dp.pb.nm))
        J.active = false;   // lib/refiner.h:111
    }
  }
  // 4. results: the colours of every finished request back into its uploaded
  // image in one launch, then one copy per request into the caller's buffer
  bool anyBack = false;
  for (BatchJob& J : jobs) {
    const bool back = J.setupIdx >= 0 && !J.req->result;
    if (J.setupIdx >= 0) setup[J.setupIdx].writeBack = back ? 1 : 0;
    anyBack |= back;
  }
  if (anyBack) {
    CK(cudaMemcpyAsync(dSetup, setup.data(), setup.size() * sizeof(rs::SetupJob), cudaMemcpyHostToDevice, s));
    CK(rs_writeback_multi(dSetup, (int)setup.size(), maxPx, s));
    launches++;
  }
  for (BatchJob& J : jobs) {
    if (J.setupIdx < 0 || J.req->result) continue;
    CK(cudaMemcpyAsync(J.req->image->data, J.dImg, J.imgBytes, cudaMemcpyDeviceToHost, s));
    d2h += J.imgBytes;
    stats.passes = std::max(stats.passes, J.passes);
  }
  CK(cudaEventRecord(e1, s));
  CK(cudaStreamSynchronize(s));
  for (size_t i = 0; i < jobs.size(); i++)
    if (jobs[i].setupIdx >= 0) {
      stats.evals += hostCtr[i].evals;
      stats.terms += hostCtr[i].terms;
    }
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, e0, e1));
  stats.deviceMs += ms;
  stats.launches += launches;
  stats.h2dBytes += h2d;
  stats.d2hBytes += d2h;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaEventDestroy(epass);
  return 0;
}

// engine() core on host pixmaps.
int run_engine_host(const TImageSynthParameters& p, const TFormatIndices& f, uint8_t* target, unsigned tw,
                    unsigned th, const uint8_t* corpus, unsigned cw, unsigned ch, void (*cb)(int, void*), void* ctx,
                    int* cancel, const TResynthOptions& opt, TResynthStats& stats) {
  if (!supported_format(f)) return fail(RESYNTH_ERROR_UNSUPPORTED, "pixel layout not supported");
  // All argument and data checks of the reference come before any device work
  // (lib/engine.c:591-646), in the reference's order.
  if (p.patchSize > (unsigned)rs::kMaxNeighbors) return IMAGE_SYNTH_ERROR_PATCH_SIZE_EXCEEDED;
  const bool devicePrep = opt.mode != RESYNTH_MODE_REPLAY && p.matchContextType >= 0 && p.matchContextType <= 8;
  HostPrep hp;
  if (devicePrep) {
    const size_t tn = (size_t)tw * th, cn = (size_t)cw * ch;
    const int bpp = f.total_bpp;
    bool anyTarget = false, anyCorpus = false;
    for (size_t i = 0; i < tn && !anyTarget; i++) anyTarget = target[i * bpp] != 0;
    if (!anyTarget) return IMAGE_SYNTH_ERROR_EMPTY_TARGET;
    for (size_t i = 0; i < cn && !anyCorpus; i++)
      anyCorpus = corpus[i * bpp] == 0xFF && (!f.isAlphaSource || corpus[i * bpp + f.alpha_bip] != 0);
    if (!anyCorpus) return IMAGE_SYNTH_ERROR_EMPTY_CORPUS;
  } else {
    const int prc = prepare(p, f, target, tw, th, corpus, cw, ch, hp);
    if (prc) return prc;
  }
  Stream& st = thread_stream();
  cudaStream_t s = st.s;
  const size_t tb = (size_t)tw * th * f.total_bpp, cb_ = (size_t)cw * ch * f.total_bpp;
  Arena ar(s);
  uint8_t* dT = ar.alloc<uint8_t>(tb);
  uint8_t* dC = ar.alloc<uint8_t>(cb_);
  CK(cudaMemcpyAsync(dT, target, tb, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(dC, corpus, cb_, cudaMemcpyHostToDevice, s));
  stats.h2dBytes += tb + cb_;
  const int rc = run_engine_device(p, f, dT, tw, th, dC, cw, ch, devicePrep ? nullptr : &hp, s, cb, ctx, cancel, opt,
                                   stats);
  if (rc) return rc;
  CK(cudaMemcpyAsync(target, dT, tb, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  stats.d2hBytes += tb;
  return 0;
}

int guarded(const char* what, const std::function<int()>& fn) {
  try {
    g_lastError[0] = 0;
    return fn();
  } catch (const CudaError& e) {
    return fail(RESYNTH_ERROR_DEVICE, "%s: %s (%s)", what, cudaGetErrorString(e.e), e.what);
  } catch (const std::bad_alloc&) {
    return fail(RESYNTH_ERROR_DEVICE, "%s: host out of memory", what);
  }
}

TResynthOptions options_or_default(const TResynthOptions* o) {
  TResynthOptions d;
  resynthDefaultOptions(&d);
  return o ? *o : d;
}

// Simple API adaption (lib/adaptSimple.h:47-354) and write-back.
int image_synth_impl(ImageBuffer* img, ImageBuffer* mask, ImageBuffer* mask2, TImageFormat fmt,
                     TImageSynthParameters* params, void (*cb)(int, void*), void* ctx, int* cancel,
                     const TResynthOptions& opt, TResynthStats& stats) {
  if (img->width != mask->width || img->height != mask->height) return IMAGE_SYNTH_ERROR_IMAGE_MASK_MISMATCH;
  TImageSynthParameters defaults;
  if (!params) {
    setDefaultParams(&defaults);
    params = &defaults;
  }
  TFormatIndices f;
  const int rc0 = prepareImageFormatIndicesFromFormatType(&f, fmt);
  if (rc0) return rc0;
  const unsigned bpp = countPixelelsPerPixelForFormat(fmt), w = img->width, h = img->height;
  const unsigned d = bpp + 1;
  int zero0 = 0;
  if (!cancel) cancel = &zero0;
  if (opt.mode != RESYNTH_MODE_REPLAY && params->matchContextType >= 0 && params->matchContextType <= 8) {
    // Device path (wavefront mode, every visit order): the adaption runs on
    // the GPU from one upload of the caller's buffers; only the reference's
    // up-front checks use the host.
    if (params->patchSize > (unsigned)rs::kMaxNeighbors) return IMAGE_SYNTH_ERROR_PATCH_SIZE_EXCEEDED;
    ImageBuffer* cm = mask2 ? mask2 : mask;
    bool anyTarget = false, anyCorpus = false;
    for (unsigned y = 0; y < h && !anyTarget; y++)
      for (unsigned x = 0; x < w && !anyTarget; x++) anyTarget = mask->data[y * mask->rowBytes + x] != 0;
    if (!anyTarget) return IMAGE_SYNTH_ERROR_EMPTY_TARGET;
    for (unsigned y = 0; y < h && !anyCorpus; y++)
      for (unsigned x = 0; x < w && !anyCorpus; x++) {
        const uint8_t m = cm->data[y * cm->rowBytes + x];
        const uint8_t cmask = mask2 ? m : (uint8_t)~m;
        anyCorpus = cmask == 0xFF && (!f.isAlphaSource || img->data[y * img->rowBytes + (size_t)x * bpp + f.alpha_bip - 1] != 0);
      }
    if (!anyCorpus) return IMAGE_SYNTH_ERROR_EMPTY_CORPUS;
    Stream& st = thread_stream();
    cudaStream_t s = st.s;
    Arena ar(s);
    const size_t imgBytes = img->rowBytes * (h - 1) + (size_t)w * bpp;
    const size_t mBytes = mask->rowBytes * (h - 1) + w;
    uint8_t* dImg = ar.alloc<uint8_t>(img->rowBytes * h);
    uint8_t* dMask = ar.alloc<uint8_t>(mask->rowBytes * h);
    uint8_t* dMask2 = mask2 ? ar.alloc<uint8_t>(mask2->rowBytes * h) : nullptr;
    CK(cudaMemcpyAsync(dImg, img->data, imgBytes, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dMask, mask->data, mBytes, cudaMemcpyHostToDevice, s));
    stats.h2dBytes += imgBytes + mBytes;
    if (mask2) {
      const size_t m2Bytes = mask2->rowBytes * (h - 1) + w;
      CK(cudaMemcpyAsync(dMask2, mask2->data, m2Bytes, cudaMemcpyHostToDevice, s));
      stats.h2dBytes += m2Bytes;
    }
    uint8_t* dT = ar.alloc<uint8_t>((size_t)w * h * d);
    uint8_t* dC = ar.alloc<uint8_t>((size_t)w * h * d);
    CK(rs_adapt(dImg, img->rowBytes, dMask, mask->rowBytes, dMask2, mask2 ? mask2->rowBytes : 0, (int)w, (int)h,
                (int)bpp, dT, dC, s));
    const int rc = run_engine_device(*params, f, dT, w, h, dC, w, h, nullptr, s, cb, ctx, cancel, opt, stats);
    stats.launches += 1;
    if (rc) return rc;
    if (!*cancel) {
      CK(rs_unadapt(dT, (int)w, (int)h, (int)bpp, dImg, img->rowBytes, s));
      CK(cudaMemcpyAsync(img->data, dImg, imgBytes, cudaMemcpyDeviceToHost, s));
      stats.d2hBytes += imgBytes;
      stats.launches += 1;
    }
    CK(cudaStreamSynchronize(s));
    return 0;
  }
  std::vector<uint8_t> tgt((size_t)w * h * d), cor((size_t)w * h * d);
  ImageBuffer* cm = mask2 ? mask2 : mask;
  for (unsigned y = 0; y < h; y++) {
    const uint8_t* srow = img->data + y * img->rowBytes;
    const uint8_t* mrow = mask->data + y * mask->rowBytes;
    const uint8_t* crow = cm->data + y * cm->rowBytes;
    for (unsigned x = 0; x < w; x++) {
      uint8_t* t = &tgt[((size_t)y * w + x) * d];
      uint8_t* c = &cor[((size_t)y * w + x) * d];
      t[0] = mrow[x];
      c[0] = mask2 ? crow[x] : (uint8_t)~crow[x];
      memcpy(t + 1, srow + (size_t)x * bpp, bpp);
      memcpy(c + 1, srow + (size_t)x * bpp, bpp);
    }
  }
  const int rc = run_engine_host(*params, f, tgt.data(), w, h, cor.data(), w, h, cb, ctx, cancel, opt, stats);
  if (!rc && !*cancel) {
    for (unsigned y = 0; y < h; y++) {
      uint8_t* drow = img->data + y * img->rowBytes;
      for (unsigned x = 0; x < w; x++) memcpy(drow + (size_t)x * bpp, &tgt[((size_t)y * w + x) * d + 1], bpp);
    }
  }
  return rc;
}

// Frozen-state scoring / energy on host buffers.
int score_host(bool energyMode, const TImageSynthParameters* p, const TFormatIndices* f, const uint8_t* target,
               unsigned tw, unsigned th, const uint8_t* corpus, unsigned cw, unsigned ch, const uint8_t* hasValue,
               const Coordinates* sourceOf, const Coordinates* targets, unsigned n, const unsigned* candStart,
               const Coordinates* cands, unsigned* outSum, Coordinates* outPt, unsigned* outCount,
               unsigned long long* energy) {
  if (!p || !f || !target || !corpus || !hasValue || !sourceOf || (!targets && n))
    return fail(RESYNTH_ERROR_ARGUMENT, "NULL argument");
  if (p->patchSize > (unsigned)rs::kMaxNeighbors) return IMAGE_SYNTH_ERROR_PATCH_SIZE_EXCEEDED;
  if (!supported_format(*f)) return fail(RESYNTH_ERROR_UNSUPPORTED, "pixel layout not supported");
  Stream& st = thread_stream();
  cudaStream_t s = st.s;
  Arena ar(s);
  unsigned long long h2d = 0;
  unsigned launches = 0;
  const size_t tb = (size_t)tw * th * f->total_bpp, cbytes = (size_t)cw * ch * f->total_bpp;
  const uint8_t* dT = ar.upload(target, tb, h2d);
  const uint8_t* dC = ar.upload(corpus, cbytes, h2d);
  const int mw = (int)std::min(tw, cw), mh = (int)std::min(th, ch);
  const auto offsHeld = cached_offsets(mw, mh, LLONG_MAX);
  const std::vector<int2>& offs = *offsHeld;
  DeviceProblem dp = make_problem(ar, s, *p, *f, dT, tw, th, dC, cw, ch, hasValue,
                                  reinterpret_cast<const int2*>(sourceOf), offs, LLONG_MAX, h2d, launches);
  rs::ScoreArgs sa{};
  sa.pb = dp.pb;
  sa.n = (int)n;
  sa.targets = ar.upload(reinterpret_cast<const int2*>(targets), n, h2d);
  sa.outSum = ar.alloc<unsigned>(n);
  if (energyMode) {
    sa.energy = ar.alloc<unsigned long long>(1);
    CK(cudaMemsetAsync(sa.energy, 0, sizeof(unsigned long long), s));
    CK(rs_launch_energy(sa, s));
    unsigned long long e = 0;
    CK(cudaMemcpyAsync(&e, sa.energy, sizeof e, cudaMemcpyDeviceToHost, s));
    if (outSum) CK(cudaMemcpyAsync(outSum, sa.outSum, n * sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    *energy = e;
    return 0;
  }
  if (!candStart || !outSum || !outPt) return fail(RESYNTH_ERROR_ARGUMENT, "NULL argument");
  const unsigned ncand = n ? candStart[n] : 0;
  sa.candStart = ar.upload(candStart, (size_t)n + 1, h2d);
  sa.cands = ar.upload(reinterpret_cast<const int2*>(cands), ncand, h2d);
  sa.outPt = ar.alloc<int2>(n);
  sa.outCount = ar.alloc<unsigned>(n);
  if (n) CK(rs_launch_frozen(sa, s));
  CK(cudaMemcpyAsync(outSum, sa.outSum, n * sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(outPt, sa.outPt, n * sizeof(int2), cudaMemcpyDeviceToHost, s));
  if (outCount) CK(cudaMemcpyAsync(outCount, sa.outCount, n * sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return 0;
}

}  // namespace

// ====================================================== reference entry points

RS_EXPORT void setDefaultParams(TImageSynthParameters* param) {
  // lib/engineParams.c:8-19
  param->isMakeSeamlesslyTileableHorizontally = 0;
  param->isMakeSeamlesslyTileableVertically = 0;
  param->matchContextType = 1;
  param->mapWeight = 0.5;
  param->sensitivityToOutliers = 0.117;
  param->patchSize = 30;
  param->maxProbeCount = 200;
}

RS_EXPORT unsigned int countPixelelsPerPixelForFormat(TImageFormat format) {
  switch (format) {  // lib/imageFormat.c:39-56
    case T_RGB: return 3;
    case T_RGBA: return 4;
    case T_Gray: return 1;
    case T_GrayA: return 2;
    default: return 0;
  }
}

RS_EXPORT void prepareImageFormatIndices(TFormatIndices* indices, unsigned int colors, unsigned int mapColors,
                                         int alphaT, int alphaS, int isMap) {
  format_indices(indices, colors, mapColors, alphaT, alphaS, isMap);
}

RS_EXPORT int prepareImageFormatIndicesFromFormatType(TFormatIndices* indices, TImageFormat format) {
  switch (format) {  // lib/imageFormat.c:65-113
    case T_RGB: format_indices(indices, 3, 0, 0, 0, 0); return 0;
    case T_RGBA: format_indices(indices, 3, 0, 1, 1, 0); return 0;
    case T_Gray: format_indices(indices, 1, 0, 0, 0, 0); return 0;
    case T_GrayA: format_indices(indices, 1, 0, 1, 1, 0); return 0;
    default: return IMAGE_SYNTH_ERROR_INVALID_IMAGE_FORMAT;
  }
}

RS_EXPORT void prepareDefaultFormatIndices(TFormatIndices* f) {
  // lib/imageFormat.c:213-241: RGBA, internal pixel MRGBA
  f->img_match_bpp = 3;
  f->colorEndBip = 4;
  f->alpha_bip = 4;
  f->map_match_bpp = 0;
  f->map_start_bip = 5;
  f->map_end_bip = 5;
  f->total_bpp = 5;
  f->isAlphaTarget = 1;
  f->isAlphaSource = 1;
}

// Maps: a GArray header followed by its storage (lib/mapOps.h:35-107).
namespace {
void map_alloc(Map* m, unsigned w, unsigned h, unsigned depth, size_t eltSize) {
  m->width = w;
  m->height = h;
  m->depth = depth;
  GArray* a = (GArray*)calloc(1, sizeof(GArray));
  a->data = (char*)calloc(std::max<size_t>((size_t)w * h, 1), eltSize);
  a->len = 0;
  m->data = a;
}
}  // namespace

RS_EXPORT void free_map(Map* map) {
  if (map->data) {
    free(map->data->data);
    free(map->data);
  }
  map->data = nullptr;
}
RS_EXPORT void new_pixmap(Map* map, unsigned int w, unsigned int h, unsigned int depth) {
  map_alloc(map, w, h, depth, depth);
}
RS_EXPORT void new_bytemap(Map* map, unsigned int w, unsigned int h) { map_alloc(map, w, h, 1, 1); }
RS_EXPORT void new_intmap(Map* map, unsigned int w, unsigned int h) {
  map_alloc(map, w, h, sizeof(unsigned int), sizeof(unsigned int));
}
RS_EXPORT void new_coordmap(Map* map, unsigned int w, unsigned int h) {
  map_alloc(map, w, h, sizeof(Coordinates), sizeof(Coordinates));
}
RS_EXPORT void set_bytemap(Map* map, unsigned char value) {
  memset(map->data->data, value, (size_t)map->width * map->height);
}
RS_EXPORT void invert_bytemap(Map* map) {
  unsigned char* d = (unsigned char*)map->data->data;
  for (size_t i = 0, n = (size_t)map->width * map->height; i < n; i++) d[i] = (unsigned char)~d[i];
}
RS_EXPORT void interleave_mask(Map* pixmap, Map* mask) {
  // lib/mapOps.h:153-168
  const size_t n = (size_t)pixmap->width * pixmap->height;
  unsigned char* p = (unsigned char*)pixmap->data->data;
  const unsigned char* m = (const unsigned char*)mask->data->data;
  for (size_t i = 0; i < n; i++) p[i * pixmap->depth] = m[i * mask->depth];
}

RS_EXPORT void resynthDefaultOptions(TResynthOptions* o) {
  memset(o, 0, sizeof *o);
  o->mode = default_mode();
}

RS_EXPORT int resynthSetMode(int mode) {
  if (mode != RESYNTH_MODE_WAVEFRONT && mode != RESYNTH_MODE_REPLAY) return -1;
  const int prev = default_mode();
  g_defaultMode = mode;
  return prev;
}

RS_EXPORT const char* resynthLastError(void) { return g_lastError; }

// Internal helpers for the other translation units.
extern "C" int rs_fail(int code, const char* msg) { return fail(code, "%s", msg); }
extern "C" void rs_metric_tables(double sensitivity, double mapWeight, uint32_t* ct, uint32_t* mt) {
  metric_tables(sensitivity, mapWeight, ct, mt);
}

RS_EXPORT int engineEx(const TImageSynthParameters* parameters, const TFormatIndices* indices, Map* targetMap,
                       Map* corpusMap, void (*cb)(int, void*), void* ctx, int* cancel,
                       const TResynthOptions* options, TResynthStats* stats) {
  if (!parameters || !indices || !targetMap || !corpusMap || !targetMap->data || !corpusMap->data)
    return fail(RESYNTH_ERROR_ARGUMENT, "NULL argument");
  TResynthStats local{};
  TResynthStats& st = stats ? *stats : local;
  memset(&st, 0, sizeof st);
  const auto t0 = std::chrono::steady_clock::now();
  const TResynthOptions opt = options_or_default(options);
  int zero = 0;
  const int rc = guarded("engine", [&] {
    return run_engine_host(*parameters, *indices, (uint8_t*)targetMap->data->data, targetMap->width,
                           targetMap->height, (const uint8_t*)corpusMap->data->data, corpusMap->width,
                           corpusMap->height, cb, ctx, cancel ? cancel : &zero, opt, st);
  });
  st.totalMs = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return rc;
}

RS_EXPORT int engine(TImageSynthParameters parameters, TFormatIndices* indices, Map* targetMap, Map* corpusMap,
                     void (*cb)(int, void*), void* ctx, int* cancel) {
  return engineEx(&parameters, indices, targetMap, corpusMap, cb, ctx, cancel, nullptr, nullptr);
}

RS_EXPORT int imageSynthEx(ImageBuffer* img, ImageBuffer* mask, ImageBuffer* mask2, TImageFormat fmt,
                           TImageSynthParameters* params, void (*cb)(int, void*), void* ctx, int* cancel,
                           const TResynthOptions* options, TResynthStats* stats) {
  if (!img || !mask) return fail(RESYNTH_ERROR_ARGUMENT, "NULL argument");
  TResynthStats local{};
  TResynthStats& st = stats ? *stats : local;
  memset(&st, 0, sizeof st);
  const auto t0 = std::chrono::steady_clock::now();
  const TResynthOptions opt = options_or_default(options);
  const int rc = guarded("imageSynth", [&] {
    return image_synth_impl(img, mask, mask2, fmt, params, cb, ctx, cancel, opt, st);
  });
  st.totalMs = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return rc;
}

RS_EXPORT int imageSynth(ImageBuffer* img, ImageBuffer* mask, TImageFormat fmt, TImageSynthParameters* params,
                         void (*cb)(int, void*), void* ctx, int* cancel) {
  return imageSynthEx(img, mask, nullptr, fmt, params, cb, ctx, cancel, nullptr, nullptr);
}

RS_EXPORT int imageSynth2(ImageBuffer* img, ImageBuffer* mask, ImageBuffer* mask2, TImageFormat fmt,
                          TImageSynthParameters* params, void (*cb)(int, void*), void* ctx, int* cancel) {
  return imageSynthEx(img, mask, mask2, fmt, params, cb, ctx, cancel, nullptr, nullptr);
}

RS_EXPORT int imageSynthBatch(TResynthRequest* requests, unsigned int count, unsigned int concurrency,
                              const TResynthOptions* options, TResynthStats* stats) {
  if (!requests && count) return fail(RESYNTH_ERROR_ARGUMENT, "NULL argument");
  const auto t0 = std::chrono::steady_clock::now();
  const TResynthOptions opt = options_or_default(options);
  const unsigned workers = std::max(1u, std::min(count, concurrency ? concurrency : 8u));
  std::vector<TResynthStats> per(count);
  // Wavefront requests with a random order go through the many-request
  // launches (unless options->separateRequests); the rest through workers.
  std::vector<TResynthRequest*> multi;
  std::vector<unsigned> rest;
  for (unsigned i = 0; i < count; i++) {
    if (!opt.separateRequests && batch_eligible(requests[i], opt)) multi.push_back(&requests[i]);
    else rest.push_back(i);
  }
  // Cohorts of at most 2^28 pixels (~10 GB of device state) run one after
  // the other, so a large batch does not need all its state at once.
  TResynthStats multiStats{};
  for (size_t first = 0; first < multi.size();) {
    size_t last = first;
    unsigned long long px = 0;
    while (last < multi.size() &&
           (last == first || px + (unsigned long long)multi[last]->image->width * multi[last]->image->height <= (1ull << 28))) {
      px += (unsigned long long)multi[last]->image->width * multi[last]->image->height;
      last++;
    }
    std::vector<TResynthRequest*> cohort(multi.begin() + first, multi.begin() + last);
    const int rc = guarded("imageSynthBatch", [&] { return run_batch_wave(cohort, opt, multiStats); });
    if (rc)
      for (TResynthRequest* r : cohort) r->result = rc;
    first = last;
  }
  std::atomic<unsigned> next{0};
  auto work = [&] {
    for (unsigned j = next++; j < rest.size(); j = next++) {
      TResynthRequest& r = requests[rest[j]];
      r.result = imageSynthEx(r.image, r.mask, r.mask2, r.format, r.parameters, nullptr, nullptr, nullptr, &opt,
                              &per[rest[j]]);
    }
  };
  std::vector<std::thread> pool;
  if (!rest.empty()) {
    for (unsigned w = 1; w < std::min<unsigned>(workers, (unsigned)rest.size()); w++) pool.emplace_back(work);
    work();
  }
  for (auto& t : pool) t.join();
  int rc = 0;
  TResynthStats total = multiStats;
  for (unsigned i = 0; i < count; i++) {
    if (!rc && requests[i].result) rc = requests[i].result;
    total.visits += per[i].visits;
    total.evals += per[i].evals;
    total.terms += per[i].terms;
    total.launches += per[i].launches;
    total.deviceMs += per[i].deviceMs;
    total.h2dBytes += per[i].h2dBytes;
    total.d2hBytes += per[i].d2hBytes;
    total.passes = std::max(total.passes, per[i].passes);
  }
  total.totalMs = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (stats) *stats = total;
  return rc;
}

RS_EXPORT int engineDevice(const TImageSynthParameters* p, const TFormatIndices* f, unsigned char* dTarget,
                           unsigned int tw, unsigned int th, const unsigned char* dCorpus, unsigned int cw,
                           unsigned int ch, void* stream, void (*cb)(int, void*), void* ctx, int* cancel,
                           const TResynthOptions* options, TResynthStats* stats) {
  if (!p || !f || !dTarget || !dCorpus) return fail(RESYNTH_ERROR_ARGUMENT, "NULL argument");
  if (p->patchSize > (unsigned)rs::kMaxNeighbors) return IMAGE_SYNTH_ERROR_PATCH_SIZE_EXCEEDED;
  if (!supported_format(*f)) return fail(RESYNTH_ERROR_UNSUPPORTED, "pixel layout not supported");
  TResynthStats local{};
  TResynthStats& st = stats ? *stats : local;
  memset(&st, 0, sizeof st);
  const auto t0 = std::chrono::steady_clock::now();
  const TResynthOptions opt = options_or_default(options);
  const int rc = guarded("engineDevice", [&] {
    return run_engine_device(*p, *f, dTarget, tw, th, dCorpus, cw, ch, nullptr, (cudaStream_t)stream, cb, ctx,
                             cancel, opt, st);
  });
  st.totalMs = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return rc;
}

RS_EXPORT int resynthGetState(Coordinates* sourceOf, unsigned char* hasValue, unsigned int w, unsigned int h) {
  if (g_state.w != w || g_state.h != h || g_state.src.empty())
    return fail(RESYNTH_ERROR_ARGUMENT, "no recorded state of that size");
  if (sourceOf) memcpy(sourceOf, g_state.src.data(), g_state.src.size() * sizeof(Coordinates));
  if (hasValue) memcpy(hasValue, g_state.has.data(), g_state.has.size());
  return 0;
}

RS_EXPORT int resynthFrozenBestFit(const TImageSynthParameters* p, const TFormatIndices* f, const unsigned char* target,
                                   unsigned int tw, unsigned int th, const unsigned char* corpus, unsigned int cw,
                                   unsigned int ch, const unsigned char* hasValue, const Coordinates* sourceOf,
                                   const Coordinates* targets, unsigned int n, const unsigned int* candStart,
                                   const Coordinates* cands, unsigned int* bestSum, Coordinates* bestPoint,
                                   unsigned int* patchCount) {
  return guarded("resynthFrozenBestFit", [&] {
    return score_host(false, p, f, target, tw, th, corpus, cw, ch, hasValue, sourceOf, targets, n, candStart, cands,
                      bestSum, bestPoint, patchCount, nullptr);
  });
}

RS_EXPORT int resynthPatchNeighbours(const unsigned char* hasValue, unsigned int width, unsigned int height,
                                     unsigned int patchSize, const Coordinates* targets, unsigned int n, int useGrid,
                                     Coordinates* offsets, unsigned int* counts) {
  if (!hasValue || !targets || !offsets || !counts || !width || !height)
    return fail(RESYNTH_ERROR_ARGUMENT, "NULL argument");
  if (patchSize > (unsigned)rs::kMaxNeighbors) return IMAGE_SYNTH_ERROR_PATCH_SIZE_EXCEEDED;
  return guarded("resynthPatchNeighbours", [&] {
    Stream& st = thread_stream();
    cudaStream_t s = st.s;
    Arena ar(s);
    unsigned long long h2d = 0;
    const int w = (int)width, h = (int)height;
    const size_t npx = (size_t)w * h;
    const long long maxD2 = wave_radius2(w, h);
    const auto offsHeld = cached_offsets(w, h, maxD2);
    const std::vector<int2>& offs = *offsHeld;
    rs::Problem pb{};
    pb.tw = pb.cw = w;
    pb.th = pb.ch = h;
    pb.nc = 1;
    pb.has = ar.upload(hasValue, npx, h2d);
    int* vis = ar.alloc<int>(npx);
    CK(rs_vis_init(pb.has, (int)npx, vis, s));
    pb.vis = vis;
    pb.tpx = ar.alloc<uint32_t>(npx);
    CK(cudaMemsetAsync(pb.tpx, 0, npx * sizeof(uint32_t), s));
    pb.src = ar.alloc<int2>(npx);
    CK(cudaMemsetAsync(pb.src, 0xFF, npx * sizeof(int2), s));
    pb.offs = ar.upload(offs.data(), offs.size(), h2d);
    pb.noffs = (int)offs.size();
    pb.patchLimit = (int)std::max(patchSize, 2u);
    pb.boxW = w;
    pb.boxH = h;
    pb.maxD2 = maxD2;
    pb.cellsW = (w + rs::kCell - 1) >> rs::kCellShift;
    pb.cellsH = (h + rs::kCell - 1) >> rs::kCellShift;
    int* cellMin = ar.alloc<int>((size_t)pb.cellsW * pb.cellsH);
    CK(rs_cell_min(vis, w, h, cellMin, s));
    pb.cellMin = cellMin;
    const int2* dT = ar.upload(reinterpret_cast<const int2*>(targets), n, h2d);
    int* dOff = ar.alloc<int>((size_t)n * rs::kMaxNeighbors);
    int* dCnt = ar.alloc<int>(n);
    // valued = hasValue: stamp -1 < 0
    if (n) CK(rs_launch_patches(pb, dT, (int)n, 0, useGrid ? 1 : 0, dOff, dCnt, s));
    std::vector<int> hOff((size_t)n * rs::kMaxNeighbors), hCnt(n);
    CK(cudaMemcpyAsync(hOff.data(), dOff, hOff.size() * sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(hCnt.data(), dCnt, hCnt.size() * sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    for (unsigned t = 0; t < n; t++) {
      counts[t] = (unsigned)hCnt[t];
      for (int i = 0; i < hCnt[t]; i++) {
        const int o = hOff[(size_t)t * rs::kMaxNeighbors + i];
        offsets[(size_t)t * (rs::kMaxNeighbors - 1) + i] = Coordinates{(int)(int16_t)(o & 0xffff), o >> 16};
      }
    }
    return 0;
  });
}

RS_EXPORT int resynthOrderTargets(int matchContextType, const Coordinates* points, unsigned int n,
                                  Coordinates* ordered) {
  if (!points || !ordered || !n) return fail(RESYNTH_ERROR_ARGUMENT, "resynthOrderTargets: bad argument");
  if (matchContextType < 2 || matchContextType > 8)
    return fail(RESYNTH_ERROR_ARGUMENT, "resynthOrderTargets: matchContextType must be 2..8");
  return guarded("resynthOrderTargets", [&]() -> int {
    Stream& st = thread_stream();
    cudaStream_t s = st.s;
    Arena ar(s);
    unsigned long long h2d = 0, d2h = 0;
    unsigned launches = 0;
    const int2* dIn = ar.upload(reinterpret_cast<const int2*>(points), n, h2d);
    int2* dOut = ar.alloc<int2>(n);
    order_directional(matchContextType, dIn, (int)n, dOut, ar, st, s, h2d, d2h, launches);
    CK(cudaMemcpyAsync(ordered, dOut, (size_t)n * sizeof(int2), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return 0;
  });
}

RS_EXPORT int resynthPatchEnergy(const TImageSynthParameters* p, const TFormatIndices* f, const unsigned char* target,
                                 unsigned int tw, unsigned int th, const unsigned char* corpus, unsigned int cw,
                                 unsigned int ch, const unsigned char* hasValue, const Coordinates* sourceOf,
                                 const Coordinates* targets, unsigned int n, unsigned long long* energy,
                                 unsigned int* perTarget) {
  if (!energy) return fail(RESYNTH_ERROR_ARGUMENT, "NULL argument");
  return guarded("resynthPatchEnergy", [&] {
    return score_host(true, p, f, target, tw, th, corpus, cw, ch, hasValue, sourceOf, targets, n, nullptr, nullptr,
                      perTarget, nullptr, nullptr, energy);
  });
}
