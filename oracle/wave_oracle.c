/*
 * wave_oracle.c -- CPU restatement of the GPU engine's wavefront mode.
 *
 * TEST INFRASTRUCTURE ONLY (like resynth_oracle.c): the checker for the GPU
 * library's default mode, loaded by tests/ and never by the product.
 *
 * The wavefront mode is a deterministic schedule, so it can be restated
 * exactly (every visit order, matchContextType 0..8):
 *   - targets (selected pixels) and corpus points (mask 0xFF, opaque) in
 *     row-major order; hasValue = context (matchContextType != 0, unselected,
 *     opaque), sourceOf = (-1, -1)  (lib/engine.c:338-431 semantics);
 *   - passes over prefixes [n, n, 3n/4, ...] of one visit order (random
 *     orders: rank = a hash of the pixel; directional orders: the reference's
 *     order), stopping when betters < n/10 after at least minPasses
 *     (lib/refiner.h:42-122, lib/passes.h:67-93);
 *   - a pass is a sequence of batches: pass 0 cuts the ranks into bands of
 *     f, 2f, 4f, ... targets with f = 16, or n / 1024 when larger for a
 *     problem with context (random orders), or of equal widths of at least
 *     1024 (directional), later passes use one band, and every band is split
 *     into k x k colour phases by (x mod k, y mod k);
 *   - within a batch, targets see the state left by earlier batches only
 *     (visit stamps in pass 0, staged stores in later passes);
 *   - a target's patch is itself plus the nearest sorted offsets (radius
 *     min(box diagonal, 256)) that hold a value (lib/synthesize.h:189-241);
 *     its candidates are the deduplicated continuations of the neighbours'
 *     sources in neighbour order, then `trys` counter-hashed probes; the
 *     first strict minimum of the patch metric (lib/synthesize.h:266-400)
 *     wins and is stored if it differs from the current source.
 * Each step follows the GPU library's resynthesizer_gb300/csrc/synth_host.cpp
 * (run_engine_device) and synth_kernels.cu (wave_target); the constants are
 * the ones those files use.  Targets of one batch are independent, so they
 * are spread over worker threads.
 */
#include "resynth_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define WO_PASSES 6
#define WO_MAX_BANDS 64
#define WO_MAX_NB 64
#define WO_STAGED_LIMIT (112 * 1024)

typedef struct { int x, y; } wpt;

static uint32_t mix32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x85ebca6bu;
  x ^= x >> 13;
  x *= 0xc2b2ae35u;
  x ^= x >> 16;
  return x;
}
static uint32_t umulhi32(uint32_t a, uint32_t b) { return (uint32_t)(((uint64_t)a * b) >> 32); }
static uint32_t probe_base(uint32_t seed, uint32_t pass, uint32_t pix) {
  return mix32(seed ^ mix32(pass * 0x9E3779B9u + 0x7f4a7c15u) ^ (pix * 0x85EBCA77u));
}

typedef struct {
  /* problem */
  int tw, th, cw, ch, nc, nm, limit, tileH, tileV, boxW, boxH, fullCorpus, trys, probeShare;
  uint32_t ct[256], mt[256], clip, seed;
  uint32_t *tpx, *tmap;          /* target words (mask | colours << 8), map words */
  const uint32_t *cpx, *cmap;    /* corpus words, map words */
  wpt *src;                      /* sourceOf per target pixel */
  int *vis;                      /* visit stamp per target pixel */
  const wpt *cpts;
  int ncorpus;
  const wpt *offs;
  int noffs;
  /* the batch being run */
  const wpt *batch;
  int nslots, batchIdx, pass, visCur;
  wpt *stage;                    /* per slot: new source or (-2, -2) */
} wave;

static int wrap_or_clip(const wave *w, int *x, int *y) {
  if (*x < 0 || *x >= w->tw) {
    if (!w->tileH) return 0;
    *x %= w->tw;
    if (*x < 0) *x += w->tw;
  }
  if (*y < 0 || *y >= w->th) {
    if (!w->tileV) return 0;
    *y %= w->th;
    if (*y < 0) *y += w->th;
  }
  return 1;
}

static uint32_t absdiff8(uint32_t a, uint32_t b, int byte) {
  const int x = (int)((a >> (8 * byte)) & 0xFFu), y = (int)((b >> (8 * byte)) & 0xFFu);
  return (uint32_t)(x > y ? x - y : y - x);
}

/* One neighbour term for candidate (cx, cy): the clip penalty outside the
 * corpus or on a pixel whose mask is not 0xFF, else the colour terms (not for
 * the target itself) plus the map terms (lib/synthesize.h:266-400). */
static uint32_t term(const wave *w, int cx, int cy, int dx, int dy, uint32_t t, uint32_t tm, int self) {
  const int qx = cx + dx, qy = cy + dy;
  if (qx < 0 || qy < 0 || qx >= w->cw || qy >= w->ch) return w->clip;
  const size_t qi = (size_t)qy * w->cw + qx;
  const uint32_t s = w->cpx[qi];
  if ((s & 0xFFu) != 0xFFu) return w->clip;
  uint32_t sum = 0;
  if (!self)
    for (int c = 1; c <= w->nc; c++) sum += w->ct[absdiff8(t, s, c)];
  if (w->nm) {
    const uint32_t sm = w->cmap[qi];
    for (int m = 0; m < w->nm; m++) sum += w->mt[absdiff8(tm, sm, m)];
  }
  return sum;
}

static wpt probe_point(const wave *w, uint32_t base, uint32_t j) {
  const uint32_t h = mix32(base + j * 0x9E3779B9u);
  wpt p;
  if (w->fullCorpus) {
    p.x = (int)umulhi32(h, (uint32_t)w->cw);
    p.y = (int)umulhi32((h << 16) | (h >> 16), (uint32_t)w->ch);
    return p;
  }
  return w->cpts[umulhi32(h, (uint32_t)w->ncorpus)];
}

static int corpus_ok(const wave *w, wpt c) {
  return c.x >= 0 && c.y >= 0 && c.x < w->cw && c.y < w->ch && (w->cpx[(size_t)c.y * w->cw + c.x] & 0xFFu) == 0xFFu;
}

/* One target of the current batch (wave_target in synth_kernels.cu). */
static void visit(const wave *w, int slot) {
  const wpt pos = w->batch[slot];
  const size_t pi = (size_t)pos.y * w->tw + pos.x;
  int offx[WO_MAX_NB], offy[WO_MAX_NB];
  uint32_t px[WO_MAX_NB], pm[WO_MAX_NB];
  wpt ps[WO_MAX_NB];
  int n = 1;
  offx[0] = offy[0] = 0;
  px[0] = w->tpx[pi];
  pm[0] = w->tmap ? w->tmap[pi] : 0u;
  ps[0] = w->src[pi];
  for (int j = 1; j < w->noffs && n < w->limit; j++) {
    const wpt o = w->offs[j];
    if (abs(o.x) >= w->boxW || abs(o.y) >= w->boxH) continue;
    int qx = pos.x + o.x, qy = pos.y + o.y;
    if (!wrap_or_clip(w, &qx, &qy)) continue;
    const size_t qi = (size_t)qy * w->tw + qx;
    if (w->vis[qi] >= w->visCur) continue;
    offx[n] = o.x;
    offy[n] = o.y;
    px[n] = w->tpx[qi];
    pm[n] = w->tmap ? w->tmap[qi] : 0u;
    ps[n] = w->src[qi];
    n++;
  }
  /* continuations, first occurrence in neighbour order */
  wpt cont[WO_MAX_NB];
  int np = 0;
  for (int k = 0; k < n; k++) {
    if (ps[k].x < 0) continue;
    wpt c = {ps[k].x - offx[k], ps[k].y - offy[k]};
    if (!corpus_ok(w, c)) continue;
    int dup = 0;
    for (int e = 0; e < np && !dup; e++) dup = cont[e].x == c.x && cont[e].y == c.y;
    if (!dup) cont[np++] = c;
  }
  const uint32_t pbase =
      w->probeShare ? probe_base(w->seed ^ 0x6A09E667u, (uint32_t)w->pass,
                                 (uint32_t)w->batchIdx * 0x01000193u + ((uint32_t)slot >> 4))
                    : probe_base(w->seed, (uint32_t)w->pass, (uint32_t)pi);
  const int ncand = np + w->trys;
  uint32_t best = 0xFFFFFFFFu;
  int bestK = -1;
  wpt bestPt = {0, 0};
  for (int k = 0; k < ncand; k++) {
    const wpt c = k < np ? cont[k] : probe_point(w, pbase, (uint32_t)(k - np));
    uint32_t sum = 0;
    int i = 0;
    for (; i < n; i++) {
      sum += term(w, c.x, c.y, offx[i], offy[i], px[i], pm[i], i == 0);
      if (sum >= best) break;   /* a later candidate only wins with a smaller sum */
    }
    if (i == n && sum < best) {
      best = sum;
      bestK = k;
      bestPt = c;
      if (best == 0) break;
    }
  }
  wpt out = {-2, -2};
  if (bestK >= 0 && (w->src[pi].x != bestPt.x || w->src[pi].y != bestPt.y)) out = bestPt;
  w->stage[slot] = out;
}

typedef struct {
  wave *w;
  int tid, nthreads;
} job;

static void *run_part(void *arg) {
  job *j = (job *)arg;
  for (int s = j->tid; s < j->w->nslots; s += j->nthreads) visit(j->w, s);
  return NULL;
}

static void run_batch(wave *w, int nthreads) {
  if (nthreads <= 1 || w->nslots < 64) {
    for (int s = 0; s < w->nslots; s++) visit(w, s);
    return;
  }
  pthread_t th[64];
  job jobs[64];
  if (nthreads > 64) nthreads = 64;
  for (int t = 0; t < nthreads; t++) {
    jobs[t].w = w;
    jobs[t].tid = t;
    jobs[t].nthreads = nthreads;
    pthread_create(&th[t], NULL, run_part, &jobs[t]);
  }
  for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
}

static int cmp_u64(const void *a, const void *b) {
  const uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
  return x < y ? -1 : x > y;
}

static int phase_side(const wpt *offs, int noffs, int limit, int w, int h) {
  int taken = 0;
  wpt last = {0, 0};
  for (int i = 0; i < noffs; i++) {
    if (abs(offs[i].x) >= w || abs(offs[i].y) >= h) continue;
    last = offs[i];
    if (++taken == limit) break;
  }
  const double r = sqrt((double)last.x * last.x + (double)last.y * last.y);
  int k = (int)floor(r) + 1;
  if (k > 8) k = 8;
  if (k < 1) k = 1;
  return k;
}

/* The wavefront offset list: every offset within 256 px in ascending
 * dx^2 + dy^2, ties by descending position in the box (descending dy, then
 * descending dx) -- an order that does not depend on the box; each call cuts
 * it at min(box diagonal, 256)^2.  Built once per process. */
static pthread_once_t g_offs_once = PTHREAD_ONCE_INIT;
static wpt *g_offs_all;
static size_t g_noffs_all;

static void build_offsets(void) {
  const int W = 2 * 257 - 1;
  uint64_t *keys = malloc((size_t)W * W * sizeof *keys);
  size_t nall = 0;
  for (int y = -256; y <= 256; y++)
    for (int x = -256; x <= 256; x++) {
      const long long d2 = (long long)x * x + (long long)y * y;
      if (d2 > 65536) continue;
      const uint32_t idx = (uint32_t)((y + 256) * W + (x + 256));
      keys[nall++] = ((uint64_t)d2 << 32) | (uint32_t)~idx;
    }
  qsort(keys, nall, sizeof *keys, cmp_u64);
  g_offs_all = malloc(nall * sizeof *g_offs_all);
  for (size_t i = 0; i < nall; i++) {
    const uint32_t idx = ~(uint32_t)(keys[i] & 0xffffffffu);
    g_offs_all[i].x = (int)(idx % W) - 256;
    g_offs_all[i].y = (int)(idx / W) - 256;
  }
  g_noffs_all = nall;
  free(keys);
}

/* The wavefront engine on interleaved pixmaps (the GPU library's engine()
 * in its default mode), random orders only.  target is modified in place
 * (colours).  Returns 0, or -1 for an unsupported order.  passesOut and
 * bettersOut (WO_PASSES entries) may be NULL. */
int orc_wave_engine_ex(const orc_params *p, const orc_format *f, unsigned char *target, unsigned tw, unsigned th,
                       const unsigned char *corpus, unsigned cw, unsigned ch, unsigned seed, int nthreads,
                       const orc_wave_opts *opt, unsigned *passesOut, unsigned *bettersOut, orc_pt *sourceOut,
                       unsigned char *hasValueOut, unsigned *batchesOut) {
  static const orc_wave_opts defaults = {0, 0, 0, 0, 0};
  if (!opt) opt = &defaults;
  if (p->matchContextType < 0 || p->matchContextType > 8) return -1;
  const int randomOrder = p->matchContextType <= 1;
  const size_t tn = (size_t)tw * th, cn = (size_t)cw * ch;
  const int bpp = f->total_bpp;
  wave w;
  memset(&w, 0, sizeof w);
  w.tw = (int)tw;
  w.th = (int)th;
  w.cw = (int)cw;
  w.ch = (int)ch;
  w.nc = f->img_match_bpp;
  w.nm = f->map_match_bpp;
  w.limit = p->patchSize > 2 ? (int)p->patchSize : 2;
  w.tileH = p->tileH ? 1 : 0;
  w.tileV = p->tileV ? 1 : 0;
  w.boxW = (int)(tw < cw ? tw : cw);
  w.boxH = (int)(th < ch ? th : ch);
  w.trys = (int)p->maxProbeCount;
  w.seed = seed ? seed : 1198472u;
  unsigned short ct16[512];
  unsigned int mt32[512];
  orc_metric_tables(p->sensitivityToOutliers, p->mapWeight, ct16, mt32);
  for (int d = 0; d < 256; d++) {
    w.ct[d] = ct16[256 + d];
    w.mt[d] = mt32[256 + d];
  }
  w.clip = 65535u * (uint32_t)f->img_match_bpp + mt32[0] * (uint32_t)f->map_match_bpp;
  /* pixel words */
  uint32_t *tpx = malloc(tn * sizeof *tpx), *tmap = w.nm ? malloc(tn * sizeof *tmap) : NULL;
  uint32_t *cpx = malloc(cn * sizeof *cpx), *cmap = w.nm ? malloc(cn * sizeof *cmap) : NULL;
  for (size_t i = 0; i < tn; i++) {
    const unsigned char *q = target + i * bpp;
    uint32_t v = q[0];
    for (int c = 0; c < w.nc; c++) v |= (uint32_t)q[1 + c] << (8 * (c + 1));
    tpx[i] = v;
    if (tmap) {
      uint32_t m = 0;
      for (int c = 0; c < w.nm; c++) m |= (uint32_t)q[f->map_start_bip + c] << (8 * c);
      tmap[i] = m;
    }
  }
  for (size_t i = 0; i < cn; i++) {
    const unsigned char *q = corpus + i * bpp;
    uint32_t v = q[0];
    for (int c = 0; c < w.nc; c++) v |= (uint32_t)q[1 + c] << (8 * (c + 1));
    cpx[i] = v;
    if (cmap) {
      uint32_t m = 0;
      for (int c = 0; c < w.nm; c++) m |= (uint32_t)q[f->map_start_bip + c] << (8 * c);
      cmap[i] = m;
    }
  }
  w.tpx = tpx;
  w.tmap = tmap;
  w.cpx = cpx;
  w.cmap = cmap;
  /* targets, context, corpus points */
  wpt *targets = malloc(tn * sizeof *targets);
  wpt *cpts = malloc(cn * sizeof *cpts);
  int *vis = malloc(tn * sizeof *vis);
  wpt *src = malloc(tn * sizeof *src);
  int n = 0, ncorpus = 0, context = 0;
  for (unsigned y = 0; y < th; y++)
    for (unsigned x = 0; x < tw; x++) {
      const size_t i = (size_t)y * tw + x;
      const unsigned char *q = target + i * bpp;
      const int sel = q[0] != 0, opaque = !f->isAlphaTarget || q[f->alpha_bip] != 0;
      const int hv = p->matchContextType && !sel && opaque;
      vis[i] = hv ? -1 : 0x7fffffff;
      context |= hv;
      src[i].x = src[i].y = -1;
      if (sel) {
        targets[n].x = (int)x;
        targets[n].y = (int)y;
        n++;
      }
    }
  for (unsigned y = 0; y < ch; y++)
    for (unsigned x = 0; x < cw; x++) {
      const unsigned char *q = corpus + ((size_t)y * cw + x) * bpp;
      if (q[0] == 0xFF && (!f->isAlphaSource || q[f->alpha_bip] != 0)) {
        cpts[ncorpus].x = (int)x;
        cpts[ncorpus].y = (int)y;
        ncorpus++;
      }
    }
  w.src = src;
  w.vis = vis;
  w.cpts = cpts;
  w.ncorpus = ncorpus;
  w.fullCorpus = (size_t)ncorpus == cn;
  int rc = 0;
  if (!n || !ncorpus) {
    rc = -2;
    goto done;
  }
  {
    /* the shared offset list (build_offsets), cut at min(box diagonal, 256)^2 */
    pthread_once(&g_offs_once, build_offsets);
    long long full = (long long)(w.boxW - 1) * (w.boxW - 1) + (long long)(w.boxH - 1) * (w.boxH - 1);
    const long long maxD2 = full < 65536 ? full : 65536;
    const size_t nall = g_noffs_all;
    const wpt *offs = g_offs_all;
    int noffs = 0;
    while ((size_t)noffs < nall &&
           (long long)offs[noffs].x * offs[noffs].x + (long long)offs[noffs].y * offs[noffs].y <= maxD2)
      noffs++;
    w.offs = offs;
    w.noffs = noffs;
    const int k = opt->phaseSide ? (int)opt->phaseSide : phase_side(offs, (int)nall, w.limit, w.boxW, w.boxH);
    /* corpus staged in shared memory when it fits: then probes stay per pixel */
    const size_t padWords = (((size_t)(cw + 12) * (ch + 12)) + 3) & ~(size_t)3;
    const size_t smem = 2064 + padWords * 4 * (w.nm ? 2 : 1) + 16 * 2048;
    w.probeShare = opt->probeShare == 1 ? 1 : opt->probeShare == 2 ? 0 : smem > WO_STAGED_LIMIT ? 1 : 0;
    const int minPasses = opt->minPasses ? (int)opt->minPasses : ((!context && w.nm == 0) ? 3 : 0);
    unsigned ends[WO_PASSES];
    {
      unsigned m = (unsigned)n;
      ends[0] = m;
      for (int i = 1; i < WO_PASSES; i++) {
        ends[i] = m;
        m = m * 3 / 4;
      }
    }
    /* one visit order for every pass: random orders rank a target by a hash
     * of its pixel; the directional orders are the reference's own order
     * (lib/orderTarget.h:268-343) and rank a target by its position in it */
    const uint32_t orderSeed = w.seed ^ 0x5bd1e995u;
    int *rank = malloc((size_t)n * sizeof *rank);
    if (randomOrder) {
      for (int t = 0; t < n; t++)
        rank[t] = (int)umulhi32(mix32((uint32_t)(targets[t].y * (int)tw + targets[t].x) * 0x9E3779B1u ^ orderSeed),
                                (uint32_t)n);
    } else {
      if (orc_order_targets(p->matchContextType, (orc_pt *)targets, (unsigned)n)) {
        free(rank);
        rc = -1;
        goto done;
      }
      for (int t = 0; t < n; t++) rank[t] = t;
    }
    int *key = malloc((size_t)n * sizeof *key);
    wpt *bucket = malloc((size_t)n * sizeof *bucket);
    int *start = malloc(((size_t)WO_MAX_BANDS * k * k + 1) * sizeof *start);
    w.stage = malloc((size_t)n * sizeof *w.stage);
    unsigned bettersTotal = 0, passes = 0;
    for (int pass = 0; pass < WO_PASSES; pass++) {
      const unsigned end = ends[pass];
      int bandEnds[WO_MAX_BANDS], nb = 0;
      if (pass == 0) {
        /* random orders: 16, 32, 64, ...; directional: equal widths of at
         * least 1024 */
        /* random orders: 16, or n / 1024 when larger for problems with
         * context (wave_first_band in synth_host.cpp) */
        const unsigned firstRandom = context && (unsigned)n / 1024u > 16u ? (unsigned)n / 1024u : 16u;
        const double first = opt->firstBatch ? opt->firstBatch : (randomOrder ? (double)firstRandom : 1024.0);
        /* bands double, or quadruple with map channels (wave_band_growth) */
        const double growth = (opt->bandGrowth ? opt->bandGrowth : (w.nm ? 400u : 200u)) / 100.0;
        double size = randomOrder ? first : fmax(first, ceil((double)end / WO_MAX_BANDS)), b = 0;
        while (b < end && nb < WO_MAX_BANDS - 1) {
          b = fmin((double)end, b + fmax(1.0, size));
          bandEnds[nb++] = (int)b;
          if (randomOrder) size *= growth;
        }
        if (bandEnds[nb - 1] < (int)end) bandEnds[nb++] = (int)end;
      } else {
        bandEnds[nb++] = (int)end;
      }
      const int nkeys = nb * k * k;
      /* batch keys and stable bucketing (k_batch_keys, k_scatter) */
      memset(start, 0, ((size_t)nkeys + 1) * sizeof *start);
      for (int t = 0; t < n; t++) {
        key[t] = -1;
        if (rank[t] >= (int)end) continue;
        int band = 0;
        while (band < nb - 1 && rank[t] >= bandEnds[band]) band++;
        key[t] = band * k * k + (targets[t].y % k) * k + (targets[t].x % k);
        start[key[t] + 1]++;
        if (pass == 0) vis[(size_t)targets[t].y * tw + targets[t].x] = key[t];
      }
      for (int b = 0; b < nkeys; b++) start[b + 1] += start[b];
      {
        int *fill = malloc((size_t)nkeys * sizeof *fill);
        memcpy(fill, start, (size_t)nkeys * sizeof *fill);
        for (int t = 0; t < n; t++)
          if (key[t] >= 0) bucket[fill[key[t]]++] = targets[t];
        free(fill);
      }
      unsigned betters = 0;
      w.pass = pass;
      for (int b = 0; b < nkeys; b++) {
        w.batch = bucket + start[b];
        w.nslots = start[b + 1] - start[b];
        if (!w.nslots) continue;
        if (batchesOut) (*batchesOut)++;
        w.batchIdx = b;
        w.visCur = pass == 0 ? b : 0x7ffffffe;
        run_batch(&w, nthreads);
        for (int s = 0; s < w.nslots; s++) {
          const wpt o = w.stage[s];
          if (o.x == -2) continue;
          const size_t pi = (size_t)w.batch[s].y * tw + w.batch[s].x;
          tpx[pi] = (tpx[pi] & 0xFFu) | (cpx[(size_t)o.y * cw + o.x] & 0xFFFFFF00u);
          src[pi] = o;
          betters++;
        }
      }
      passes = (unsigned)pass + 1;
      if (bettersOut) bettersOut[pass] = betters;
      bettersTotal += betters;
      if ((double)((float)betters / (float)n) < 0.1 && pass + 1 >= minPasses) break;   /* lib/refiner.h:111 */
    }
    if (passesOut) *passesOut = passes;
    if (sourceOut)
      for (size_t i = 0; i < tn; i++) {
        sourceOut[i].x = src[i].x;
        sourceOut[i].y = src[i].y;
      }
    if (hasValueOut)
      for (size_t i = 0; i < tn; i++) hasValueOut[i] = vis[i] != 0x7fffffff;
    (void)bettersTotal;
    free(rank);
    free(key);
    free(bucket);
    free(start);
    free(w.stage);
  }
  /* colours back into the pixmap */
  for (size_t i = 0; i < tn; i++)
    for (int c = 0; c < w.nc; c++) target[i * bpp + 1 + c] = (unsigned char)(tpx[i] >> (8 * (c + 1)));
done:
  free(tpx);
  free(tmap);
  free(cpx);
  free(cmap);
  free(targets);
  free(cpts);
  free(vis);
  free(src);
  return rc;
}

int orc_wave_engine(const orc_params *p, const orc_format *f, unsigned char *target, unsigned tw, unsigned th,
                    const unsigned char *corpus, unsigned cw, unsigned ch, unsigned seed, int nthreads,
                    unsigned *passesOut, unsigned *bettersOut) {
  return orc_wave_engine_ex(p, f, target, tw, th, corpus, cw, ch, seed, nthreads, NULL, passesOut, bettersOut, NULL,
                            NULL, NULL);
}
