/*
 * resynth_oracle.c -- CPU oracle (test infrastructure only; see the header).
 *
 * A restatement, in plain C, of the reference synthesis engine:
 *   engine prep            lib/engine.c:338-497, 539-690
 *   target ordering        lib/orderTarget.h:35-343, lib/brushfire.h:62-163,
 *                          lib/engineTypes.h:51-226
 *   metric tables          lib/matchWeighting.h:49-60, 142-204
 *   passes / refiner       lib/passes.h:67-93, lib/refiner.h:42-122,
 *                          lib/refinerThreaded.h:259-381
 *   per-target synthesis   lib/synthesize.h:81-113, 158-241, 266-419, 426-642
 *   progress               lib/progress.c:53-65
 *   simple API             lib/imageSynth.c:61-216, lib/adaptSimple.h:47-354
 * The PRNG is libc srand/rand and sorting is libc qsort, as in the
 * reference's standalone build (lib/glibProxy.c:29-49, 104-116).
 */
#define _GNU_SOURCE
#include "resynth_oracle.h"

#include <limits.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

enum {
  ERR_INVALID_FORMAT = 1, ERR_MASK_MISMATCH = 2, ERR_PATCH_SIZE = 3,
  ERR_CONTEXT_TYPE = 4, ERR_EMPTY_TARGET = 5, ERR_EMPTY_CORPUS = 6
};

#define MAX_NEIGHBORS 64        /* lib/imageSynthConstants.h:26 */
#define MAX_BPP 8               /* lib/imageSynthConstants.h:58 */
#define CALLBACK_MASK 4095u     /* lib/imageSynthConstants.h:100 */
#define NPASSES 6               /* lib/passes.h:51 */
#define SEED 1198472u           /* lib/engine.c:643 */

/* ------------------------------------------------------------------ PRNG */

/* lib/glibProxy.c:36-49: lo + rand() / (RAND_MAX / (hi - lo) + 1); no draw
 * when the upper bound is below 1. */
static unsigned rand_range(unsigned lo, unsigned hi_excl, unsigned long long *draws) {
  if (hi_excl < 1) return 0;
  unsigned hi = hi_excl - 1;
  if (draws) (*draws)++;
  return lo + (unsigned)rand() / ((unsigned)RAND_MAX / (hi - lo + 1) + 1);
}

void orc_rand_stream(unsigned seed, unsigned n, int *out) {
  srand(seed);
  for (unsigned i = 0; i < n; i++) out[i] = rand();
}

/* --------------------------------------------------------- metric tables */

/* lib/matchWeighting.h:49-60 */
static double neg_ln_cauchy(double x, float c) {
  return log((x / (c * 256)) * (x / (c * 256)) + 1.0);
}

/* lib/matchWeighting.h:142-178 (float parameters, truncating casts). */
void orc_metric_tables(double sensitivity, double mapWeight,
                       unsigned short ct[512], unsigned int mt[512]) {
  float c = (float)sensitivity, w = (float)mapWeight;
  for (int i = -256; i < 256; i++) {
    double v = neg_ln_cauchy(i, c) / neg_ln_cauchy(256, c) * (float)65535;
    ct[256 + i] = (unsigned short)v;
    mt[256 + i] = (unsigned int)(i * i * w * 4.0);
  }
}

/* ---------------------------------------------------------- pixel format */

void orc_format_indices(orc_format *f, unsigned colors, unsigned mapColors,
                        int alphaT, int alphaS, int isMap) {
  memset(f, 0, sizeof *f);
  f->img_match_bpp = (unsigned char)colors;
  f->colorEndBip = (unsigned char)(1 + colors);
  if (alphaT || alphaS) {
    f->alpha_bip = f->colorEndBip;
    f->map_start_bip = (unsigned char)(f->colorEndBip + 1);
  } else {
    f->map_start_bip = f->colorEndBip;
  }
  f->map_match_bpp = (unsigned char)(isMap ? mapColors : 0);
  f->map_end_bip = (unsigned char)(f->map_start_bip + f->map_match_bpp);
  f->total_bpp = f->map_end_bip;
  f->isAlphaTarget = alphaT;
  f->isAlphaSource = alphaS;
}

/* T_RGB=0, T_RGBA=1, T_Gray=2, T_GrayA=3 (lib/imageFormat.h:36-42). */
int orc_format_from_type(orc_format *f, int t) {
  switch (t) {
    case 0: orc_format_indices(f, 3, 0, 0, 0, 0); return 0;
    case 1: orc_format_indices(f, 3, 0, 1, 1, 0); return 0;
    case 2: orc_format_indices(f, 1, 0, 0, 0, 0); return 0;
    case 3: orc_format_indices(f, 1, 0, 1, 1, 0); return 0;
    default: return ERR_INVALID_FORMAT;
  }
}

unsigned orc_pixelels_for_format(int t) {
  static const unsigned n[4] = {3, 4, 1, 2};
  return (t >= 0 && t < 4) ? n[t] : 0;
}

/* ------------------------------------------------------------- ordering */

/* Comparators never return 0 (lib/engineTypes.h:51-149): "a before b" is
 * -1, everything else +1, so tie order is whatever libc qsort makes of it. */
static int cmp_less_cartesian(const void *va, const void *vb) {
  const orc_pt *a = va, *b = vb;
  return (a->y * a->y + a->x * a->x < b->y * b->y + b->x * b->x) ? -1 : 1;
}
static int cmp_more_horizontal(const void *va, const void *vb) {
  const orc_pt *a = va, *b = vb;
  int less = (a->x * a->x < b->x * b->x) ? -1 : 1;
  return less == 1 ? -1 : 1;
}
static int cmp_less_horizontal(const void *va, const void *vb) {
  const orc_pt *a = va, *b = vb;
  return (a->x * a->x < b->x * b->x) ? -1 : 1;
}
static int cmp_more_vertical(const void *va, const void *vb) {
  const orc_pt *a = va, *b = vb;
  int less = (a->y * a->y < b->y * b->y) ? -1 : 1;
  return less == 1 ? -1 : 1;
}
static int cmp_less_vertical(const void *va, const void *vb) {
  const orc_pt *a = va, *b = vb;
  return (a->y * a->y < b->y * b->y) ? -1 : 1;
}

typedef struct { orc_pt p; float prop; } sort_elem;  /* lib/engineTypes.h:23-26 */

static int cmp_less_inward(const void *va, const void *vb) {
  const sort_elem *a = va, *b = vb;
  return (a->prop < b->prop) ? -1 : 1;
}
static int cmp_more_inward(const void *va, const void *vb) {
  return cmp_less_inward(va, vb) == 1 ? -1 : 1;
}

size_t orc_sorted_offsets(unsigned tw, unsigned th, unsigned cw, unsigned ch, orc_pt *out) {
  int w = (int)(cw < tw ? cw : tw), h = (int)(ch < th ? ch : th);
  size_t n = 0;
  for (int y = -h + 1; y < h; y++)
    for (int x = -w + 1; x < w; x++) { out[n].x = x; out[n].y = y; n++; }
  qsort(out, n, sizeof(orc_pt), cmp_less_cartesian);
  return n;
}

/* Centre of the bounding box, lib/engineTypes.h:187-226 (bounds start at
 * {INT_MAX, INT_MAX, 0, 0}). */
static orc_pt bbox_center(const orc_pt *pts, unsigned n) {
  int ulx = INT_MAX, uly = INT_MAX, lrx = 0, lry = 0;
  for (unsigned i = 0; i < n; i++) {
    if (pts[i].x < ulx) ulx = pts[i].x;
    if (pts[i].y < uly) uly = pts[i].y;
    if (pts[i].x > lrx) lrx = pts[i].x;
    if (pts[i].y > lry) lry = pts[i].y;
  }
  orc_pt c = {(lrx - ulx) / 2 + ulx, (lry - uly) / 2 + uly};
  return c;
}

static void swap_pts(orc_pt *v, unsigned i, unsigned j) {
  orc_pt t = v[i]; v[i] = v[j]; v[j] = t;
}

/* lib/orderTarget.h:58-79 */
static void band_shuffle(orc_pt *v, unsigned n) {
  int last = (int)n - 1;
  int half = (int)(n * 0.1);
  for (int i = 0; i <= last; i++) {
    int lo = i - half > 0 ? i - half : 0;
    int hi = i + half < last ? i + half : last;
    int j = lo + (int)rand_range(0, (unsigned)(hi - lo), NULL);
    swap_pts(v, (unsigned)i, (unsigned)j);
  }
}

/* lib/brushfire.h:62-67: ray index 0..400 of an offset. */
static unsigned ray_of(orc_pt a) {
  return (unsigned)(atan2((float)a.y, (float)a.x) * 200 / 3.1415926535897932384626433832795028841971693993751 + 200);
}

/* lib/brushfire.h:73-148: key = |a|^2 / max |p|^2 on the same ray. */
static sort_elem *proportion_keys(const orc_pt *offs, unsigned n) {
  unsigned maxr[401];
  memset(maxr, 0, sizeof maxr);
  for (unsigned i = 0; i < n; i++) {
    unsigned d = (unsigned)(offs[i].x * offs[i].x + offs[i].y * offs[i].y);
    unsigned r = ray_of(offs[i]);
    if (d > maxr[r]) maxr[r] = d;
  }
  sort_elem *s = malloc(sizeof(sort_elem) * (n ? n : 1));
  for (unsigned i = 0; i < n; i++) {
    s[i].p = offs[i];
    s[i].prop = (float)(offs[i].y * offs[i].y + offs[i].x * offs[i].x) / maxr[ray_of(offs[i])];
  }
  return s;
}

static void to_offsets(orc_pt *v, unsigned n, orc_pt c, int sign) {
  for (unsigned i = 0; i < n; i++) { v[i].x += sign * c.x; v[i].y += sign * c.y; }
}

int orc_order_targets(int type, orc_pt *v, unsigned n) {
  srand(SEED);
  if (type == 0 || type == 1) {                       /* lib/orderTarget.h:35-47 */
    for (unsigned i = 0; i < n; i++) swap_pts(v, i, rand_range(0, n, NULL));
    return 0;
  }
  if (type < 0 || type > 8) return ERR_CONTEXT_TYPE;
  orc_pt c = bbox_center(v, n);
  to_offsets(v, n, c, -1);
  if (type == 2 || type == 5 || type == 8) {          /* brushfire / squeeze */
    sort_elem *s = proportion_keys(v, n);
    /* Squeeze (lib/orderTarget.h:209-262) sorts the keys inward but then
     * writes the sorted array straight back, so its front/back interleave
     * is overwritten: the result equals the inward brushfire order. */
    qsort(s, n, sizeof *s, type == 5 ? cmp_less_inward : cmp_more_inward);
    for (unsigned i = 0; i < n; i++) v[i] = s[i].p;
    free(s);
  } else {                                            /* lib/orderTarget.h:154-178 */
    int (*cmp)(const void *, const void *) =
        type == 3 ? cmp_more_horizontal : type == 4 ? cmp_more_vertical
      : type == 6 ? cmp_less_horizontal : cmp_less_vertical;
    qsort(v, n, sizeof(orc_pt), cmp);
  }
  to_offsets(v, n, c, +1);
  band_shuffle(v, n);
  return 0;
}

/* ---------------------------------------------------------------- engine */

typedef struct {
  orc_pt off;
  orc_pt src;
  unsigned char px[MAX_BPP];
} neighbor;   /* TNeighbor, lib/synthesize.h:120-125 */

typedef struct {
  const orc_params *p;
  const orc_format *f;
  unsigned char *tgt; unsigned tw, th;
  const unsigned char *cor; unsigned cw, ch;
  unsigned char *hasValue;       /* tw*th */
  orc_pt *sourceOf;              /* tw*th */
  unsigned *recentProber;        /* cw*ch */
  const orc_pt *targets; unsigned ntargets;
  const orc_pt *corpusPts; unsigned ncorpus;
  const orc_pt *offs; size_t noffs;
  unsigned short ct[512];
  unsigned mt[512];
  int nthreads;
  pthread_mutex_t mutex;
  /* progress, lib/progress.h:9-23 */
  unsigned estimated, completed, prior;
  void (*progress)(int, void *); void *ctx; int *cancel;
} engine_ctx;

static const unsigned char *cpx(const engine_ctx *e, orc_pt q) {
  return e->cor + ((size_t)q.x + (size_t)q.y * e->cw) * e->f->total_bpp;
}
static unsigned char *tpx(const engine_ctx *e, orc_pt q) {
  return e->tgt + ((size_t)q.x + (size_t)q.y * e->tw) * e->f->total_bpp;
}

/* lib/engine.c:505-517: out of bounds, or corpus mask != 0xFF. */
static int clipped_or_masked(const engine_ctx *e, orc_pt q) {
  return q.x < 0 || q.y < 0 || q.x >= (int)e->cw || q.y >= (int)e->ch || cpx(e, q)[0] != 0xFF;
}

/* lib/synthesize.h:81-113 */
static int wrap_or_clip(const orc_params *p, unsigned w, unsigned h, orc_pt *q) {
  while (q->x < 0) { if (!p->tileH) return 0; q->x += (int)w; }
  while (q->x >= (int)w) { if (!p->tileH) return 0; q->x -= (int)w; }
  while (q->y < 0) { if (!p->tileV) return 0; q->y += (int)h; }
  while (q->y >= (int)h) { if (!p->tileV) return 0; q->y -= (int)h; }
  return 1;
}

static void copy_neighbor(engine_ctx *e, neighbor *nb, orc_pt off, orc_pt q, int lock) {
  nb->off = off;
  if (lock) pthread_mutex_lock(&e->mutex);
  nb->src = e->sourceOf[q.x + q.y * (int)e->tw];
  memcpy(nb->px, tpx(e, q), e->f->total_bpp);
  if (lock) pthread_mutex_unlock(&e->mutex);
}

/* lib/synthesize.h:189-241: self first, then the nearest offsets whose point
 * is in (or wraps into) the target image and has a value, until patchSize. */
static unsigned build_patch(engine_ctx *e, orc_pt pos, neighbor *nb, int lock) {
  unsigned count = 0;
  copy_neighbor(e, &nb[count++], e->offs[0], pos, lock);
  for (size_t j = 1; j < e->noffs; j++) {
    orc_pt q = {pos.x + e->offs[j].x, pos.y + e->offs[j].y};
    if (wrap_or_clip(e->p, e->tw, e->th, &q) && e->hasValue[q.x + q.y * (int)e->tw]) {
      copy_neighbor(e, &nb[count++], e->offs[j], q, lock);
      if (count >= e->p->patchSize) break;
    }
  }
  return count;
}

/* Full or early-out patch metric, lib/synthesize.h:266-400.  Returns the sum
 * reached; *stopped is set when the early-out fired (sum >= best). */
static unsigned patch_metric(const engine_ctx *e, orc_pt cand, const neighbor *nb, unsigned n,
                             unsigned best, int *stopped, unsigned long long *terms) {
  const orc_format *f = e->f;
  unsigned sum = 0;
  unsigned clipCost = 65535u * f->img_match_bpp + e->mt[0] * f->map_match_bpp;
  *stopped = 0;
  for (unsigned i = 0; i < n; i++) {
    orc_pt q = {cand.x + nb[i].off.x, cand.y + nb[i].off.y};
    if (terms) (*terms)++;
    if (clipped_or_masked(e, q)) {
      sum += clipCost;
    } else {
      const unsigned char *s = cpx(e, q), *t = nb[i].px;
      if (i) for (unsigned j = 1; j < f->colorEndBip; j++) sum += e->ct[256u + t[j] - s[j]];
      for (unsigned j = f->map_start_bip; j < f->map_end_bip; j++) sum += e->mt[256u + t[j] - s[j]];
    }
    if (sum >= best) { *stopped = 1; return sum; }
  }
  return sum;
}

/* computeBestFit: strict-less update, returns 1 on a perfect match. */
static int best_fit(const engine_ctx *e, orc_pt cand, const neighbor *nb, unsigned n,
                    unsigned *best, orc_pt *bestPt, int *bettered, unsigned long long *evals,
                    unsigned long long *terms) {
  int stopped;
  if (evals) (*evals)++;
  unsigned s = patch_metric(e, cand, nb, n, *best, &stopped, terms);
  if (stopped) return 0;
  *best = s; *bestPt = cand; *bettered = 1;
  return s == 0;
}

/* lib/progress.c:53-65 */
static void deep_progress(engine_ctx *e) {
  e->completed += CALLBACK_MASK;
  unsigned pct = (unsigned)(((float)e->completed / e->estimated) * 100);
  if (pct > e->prior) {
    e->progress((int)pct, e->ctx);
    e->prior = pct;
  }
}

typedef struct {
  engine_ctx *e;
  unsigned tid, end;
  unsigned long betters;
  unsigned long long visits, evals, terms, draws;
} synth_job;

/* lib/synthesize.h:426-642 */
static void synthesize(synth_job *job) {
  engine_ctx *e = job->e;
  const int lock = e->nthreads > 1;
  const unsigned stride = (unsigned)e->nthreads;
  neighbor nb[MAX_NEIGHBORS];
  for (unsigned t = job->tid % stride; t < job->end; t += stride) {
    if ((t & CALLBACK_MASK) == 0) {
      if (lock) pthread_mutex_lock(&e->mutex);
      deep_progress(e);
      if (lock) pthread_mutex_unlock(&e->mutex);
      if (*e->cancel) break;
    }
    job->visits++;
    orc_pt pos = e->targets[t];
    unsigned n = build_patch(e, pos, nb, lock);
    unsigned best = UINT_MAX;
    orc_pt bestPt = {0, 0};
    int bettered = 0, perfect = 0;
    /* heuristic 1: continuations of the neighbours' sources */
    for (unsigned k = 0; k < n && best != 0; k++) {
      if (nb[k].src.x == -1) continue;
      orc_pt c = {nb[k].src.x - nb[k].off.x, nb[k].src.y - nb[k].off.y};
      if (clipped_or_masked(e, c)) continue;
      unsigned *rp = &e->recentProber[c.x + c.y * (int)e->cw];
      if (*rp == t) continue;                       /* heuristic 2 */
      perfect = best_fit(e, c, nb, n, &best, &bestPt, &bettered, &job->evals, &job->terms);
      if (perfect) break;
      *rp = t;
    }
    if (!perfect) {
      for (unsigned j = 0; j < e->p->maxProbeCount; j++) {
        orc_pt c = e->corpusPts[rand_range(0, e->ncorpus, &job->draws)];
        perfect = best_fit(e, c, nb, n, &best, &bestPt, &bettered, &job->evals, &job->terms);
        if (perfect) break;
      }
    }
    size_t ti = (size_t)pos.x + (size_t)pos.y * e->tw;
    if (bettered && (e->sourceOf[ti].x != bestPt.x || e->sourceOf[ti].y != bestPt.y)) {
      job->betters++;
      if (lock) pthread_mutex_lock(&e->mutex);
      const unsigned char *s = cpx(e, bestPt);
      unsigned char *d = tpx(e, pos);
      for (unsigned j = 1; j < e->f->colorEndBip; j++) d[j] = s[j];
      e->sourceOf[ti] = bestPt;
      if (lock) pthread_mutex_unlock(&e->mutex);
    }
    e->hasValue[ti] = 1;
  }
}

static void *synth_thread(void *arg) { synthesize((synth_job *)arg); return NULL; }

static void noop_progress(int pct, void *ctx) { (void)pct; (void)ctx; }

int orc_engine(const orc_params *p, const orc_format *f,
               unsigned char *target, unsigned tw, unsigned th,
               const unsigned char *corpus, unsigned cw, unsigned ch,
               int nthreads, void (*progress)(int, void *), void *ctx, int *cancel,
               orc_stats *stats, orc_pt *sourceOut, unsigned char *hasValueOut) {
  int zero = 0;
  if (stats) memset(stats, 0, sizeof *stats);
  if (p->patchSize > MAX_NEIGHBORS) return ERR_PATCH_SIZE;         /* engine.c:591 */
  engine_ctx *e = calloc(1, sizeof *e);
  e->p = p; e->f = f; e->tgt = target; e->tw = tw; e->th = th;
  e->cor = corpus; e->cw = cw; e->ch = ch;
  e->nthreads = nthreads < 1 ? 1 : nthreads;
  e->progress = progress ? progress : noop_progress;
  e->ctx = ctx; e->cancel = cancel ? cancel : &zero;
  size_t tn = (size_t)tw * th, cn = (size_t)cw * ch;
  int rc = 0;

  /* target points + hasValue, engine.c:338-391 */
  orc_pt *targets = malloc(sizeof(orc_pt) * (tn ? tn : 1));
  e->hasValue = calloc(tn ? tn : 1, 1);
  unsigned nt = 0;
  for (unsigned y = 0; y < th; y++)
    for (unsigned x = 0; x < tw; x++) {
      const unsigned char *px = target + ((size_t)x + (size_t)y * tw) * f->total_bpp;
      int selected = px[0] != 0;
      int opaque = f->isAlphaTarget ? px[f->alpha_bip] != 0 : 1;
      e->hasValue[x + y * tw] = (p->matchContextType && !selected && opaque) ? 1 : 0;
      if (selected) { targets[nt].x = (int)x; targets[nt].y = (int)y; nt++; }
    }
  if (!nt) { rc = ERR_EMPTY_TARGET; goto done_targets; }
  e->sourceOf = malloc(sizeof(orc_pt) * tn);
  for (size_t i = 0; i < tn; i++) e->sourceOf[i].x = e->sourceOf[i].y = -1;

  /* corpus points, engine.c:400-431 */
  orc_pt *cpts = malloc(sizeof(orc_pt) * (cn ? cn : 1));
  unsigned nc = 0;
  for (unsigned y = 0; y < ch; y++)
    for (unsigned x = 0; x < cw; x++) {
      const unsigned char *px = corpus + ((size_t)x + (size_t)y * cw) * f->total_bpp;
      if (px[0] == 0xFF && (f->isAlphaSource ? px[f->alpha_bip] != 0 : 1)) {
        cpts[nc].x = (int)x; cpts[nc].y = (int)y; nc++;
      }
    }
  if (!nc) { rc = ERR_EMPTY_CORPUS; goto done_corpus; }

  /* offsets and tables, engine.c:465-497, 631-636 */
  size_t mw = cw < tw ? cw : tw, mh = ch < th ? ch : th;
  orc_pt *offs = malloc(sizeof(orc_pt) * (2 * mw - 1) * (2 * mh - 1));
  size_t noffs = orc_sorted_offsets(tw, th, cw, ch, offs);
  orc_metric_tables(p->sensitivityToOutliers, p->mapWeight, e->ct, e->mt);

  /* order (seeds the PRNG), engine.c:643-647 */
  rc = orc_order_targets(p->matchContextType, targets, nt);
  if (rc) goto done_offsets;

  e->recentProber = malloc(sizeof(unsigned) * cn);
  memset(e->recentProber, 0xFF, sizeof(unsigned) * cn);
  e->targets = targets; e->ntargets = nt;
  e->corpusPts = cpts; e->ncorpus = nc;
  e->offs = offs; e->noffs = noffs;
  pthread_mutex_init(&e->mutex, NULL);

  /* passes, lib/passes.h:67-93 */
  unsigned ends[NPASSES], n = nt, total = 0;
  ends[0] = nt; total = nt;
  for (int i = 1; i < NPASSES; i++) { ends[i] = n; total += n; n = n * 3 / 4; }
  e->estimated = total;

  for (int pass = 0; pass < NPASSES; pass++) {
    synth_job jobs[64];
    unsigned long betters = 0;
    int T = e->nthreads;
    memset(jobs, 0, sizeof(jobs));
    for (int k = 0; k < T; k++) { jobs[k].e = e; jobs[k].tid = (unsigned)k; jobs[k].end = ends[pass]; }
    if (T == 1) {
      synthesize(&jobs[0]);
    } else {
      pthread_t th_[64];
      for (int k = 0; k < T; k++) pthread_create(&th_[k], NULL, synth_thread, &jobs[k]);
      for (int k = 0; k < T; k++) pthread_join(th_[k], NULL);
    }
    for (int k = 0; k < T; k++) {
      betters += jobs[k].betters;
      if (stats) {
        stats->visits += jobs[k].visits; stats->evals += jobs[k].evals;
        stats->terms += jobs[k].terms; stats->draws += jobs[k].draws;
      }
    }
    if (stats) { stats->passes = (unsigned)pass + 1; stats->pass_len[pass] = ends[pass];
                 stats->betters[pass] = (unsigned)betters; }
    if ((float)betters / nt < 0.1) break;         /* lib/refiner.h:111 */
  }
  pthread_mutex_destroy(&e->mutex);
  if (sourceOut) memcpy(sourceOut, e->sourceOf, sizeof(orc_pt) * tn);
  if (hasValueOut) memcpy(hasValueOut, e->hasValue, tn);
  free(e->recentProber);
done_offsets:
  free(offs);
done_corpus:
  free(cpts);
  free(e->sourceOf);
done_targets:
  free(targets);
  free(e->hasValue);
  free(e);
  return rc;
}

/* ------------------------------------------------------------ simple API */

/* The engine behind a Simple API call: the reference engine (nthreads >= 1)
 * or the GPU library's wavefront mode restated (wave != 0, wave_oracle.c). */
typedef struct {
  int wave, nthreads;
  unsigned seed;
  void (*progress)(int, void *);
  void *ctx;
  int *cancel;
  orc_stats *stats;
} simple_engine;

static int run_simple_engine(const simple_engine *se, const orc_params *p, const orc_format *f,
                             unsigned char *tgt, unsigned w, unsigned h, const unsigned char *cor) {
  if (!se->wave)
    return orc_engine(p, f, tgt, w, h, cor, w, h, se->nthreads, se->progress, se->ctx, se->cancel, se->stats,
                      NULL, NULL);
  if (p->patchSize > MAX_NEIGHBORS) return ERR_PATCH_SIZE;                   /* engine.c:591 */
  const int rc = orc_wave_engine(p, f, tgt, w, h, cor, w, h, se->seed, se->nthreads, NULL, NULL);
  if (rc == -1) return ERR_CONTEXT_TYPE;
  if (rc == -2) {                                                           /* engine.c:605-627 */
    for (size_t i = 0; i < (size_t)w * h; i++)
      if (tgt[i * f->total_bpp]) return ERR_EMPTY_CORPUS;
    return ERR_EMPTY_TARGET;
  }
  return rc;
}

/* lib/imageSynth.c:61-216 with adaptSimpleAPI / antiAdaptImage
 * (lib/adaptSimple.h:47-354): the caller's row-padded image becomes two
 * unpadded pixmaps with the mask interleaved first (the corpus takes mask2,
 * or the inverted mask); the engine's colours go back into the caller's
 * buffer only on success and without cancellation. */
static int simple_api(orc_image_buffer *img, orc_image_buffer *mask, orc_image_buffer *mask2, int fmt,
                      const orc_params *p, const simple_engine *se) {
  if (img->width != mask->width || img->height != mask->height) return ERR_MASK_MISMATCH;
  orc_params defaults = {0, 0, 1, 0.5, 0.117, 30, 200};    /* lib/engineParams.c:8-19 */
  if (!p) p = &defaults;
  orc_format f;
  int rc = orc_format_from_type(&f, fmt);
  if (rc) return rc;
  unsigned bpp = orc_pixelels_for_format(fmt), w = img->width, h = img->height;
  unsigned char *tgt = malloc((size_t)w * h * (bpp + 1) + 1);
  unsigned char *cor = malloc((size_t)w * h * (bpp + 1) + 1);
  orc_image_buffer *cm = mask2 ? mask2 : mask;
  for (unsigned y = 0; y < h; y++)
    for (unsigned x = 0; x < w; x++) {
      size_t d = ((size_t)x + (size_t)y * w) * (bpp + 1);
      const unsigned char *s = img->data + y * img->rowBytes + (size_t)x * bpp;
      tgt[d] = mask->data[y * mask->rowBytes + x];
      unsigned char m = cm->data[y * cm->rowBytes + x];
      cor[d] = mask2 ? m : (unsigned char)~m;
      memcpy(tgt + d + 1, s, bpp);
      memcpy(cor + d + 1, s, bpp);
    }
  rc = run_simple_engine(se, p, &f, tgt, w, h, cor);
  if (!rc && !*se->cancel)
    for (unsigned y = 0; y < h; y++)
      for (unsigned x = 0; x < w; x++)
        memcpy(img->data + y * img->rowBytes + (size_t)x * bpp,
               tgt + ((size_t)x + (size_t)y * w) * (bpp + 1) + 1, bpp);
  free(tgt);
  free(cor);
  return rc;
}

int orc_image_synth(orc_image_buffer *img, orc_image_buffer *mask, orc_image_buffer *mask2,
                    int fmt, const orc_params *p, int nthreads,
                    void (*progress)(int, void *), void *ctx, int *cancel, orc_stats *stats) {
  int zero = 0;
  simple_engine se = {0, nthreads, 0, progress, ctx, cancel ? cancel : &zero, stats};
  return simple_api(img, mask, mask2, fmt, p, &se);
}

int orc_wave_image_synth(orc_image_buffer *img, orc_image_buffer *mask, orc_image_buffer *mask2, int fmt,
                         const orc_params *p, unsigned seed, int nthreads) {
  int zero = 0;
  simple_engine se = {1, nthreads, seed, NULL, NULL, &zero, NULL};
  return simple_api(img, mask, mask2, fmt, p, &se);
}

/* ---------------------------------------------------- frozen and energy */

static void frozen_ctx(engine_ctx *e, const orc_params *p, const orc_format *f,
                       const unsigned char *target, unsigned tw, unsigned th,
                       const unsigned char *corpus, unsigned cw, unsigned ch,
                       const unsigned char *hasValue, const orc_pt *sourceOf) {
  memset(e, 0, sizeof *e);
  e->p = p; e->f = f; e->tgt = (unsigned char *)target; e->tw = tw; e->th = th;
  e->cor = corpus; e->cw = cw; e->ch = ch;
  e->hasValue = (unsigned char *)hasValue; e->sourceOf = (orc_pt *)sourceOf;
  e->nthreads = 1;
  size_t mw = cw < tw ? cw : tw, mh = ch < th ? ch : th;
  orc_pt *offs = malloc(sizeof(orc_pt) * (2 * mw - 1) * (2 * mh - 1));
  e->noffs = orc_sorted_offsets(tw, th, cw, ch, offs);
  e->offs = offs;
  orc_metric_tables(p->sensitivityToOutliers, p->mapWeight, e->ct, e->mt);
}

void orc_frozen(const orc_params *p, const orc_format *f,
                const unsigned char *target, unsigned tw, unsigned th,
                const unsigned char *corpus, unsigned cw, unsigned ch,
                const unsigned char *hasValue, const orc_pt *sourceOf,
                const orc_pt *targets, unsigned n,
                const unsigned *candStart, const orc_pt *cands,
                unsigned *outSum, orc_pt *outPt, unsigned *outCount) {
  engine_ctx e;
  frozen_ctx(&e, p, f, target, tw, th, corpus, cw, ch, hasValue, sourceOf);
  neighbor nb[MAX_NEIGHBORS];
  for (unsigned t = 0; t < n; t++) {
    unsigned cnt = build_patch(&e, targets[t], nb, 0);
    unsigned best = UINT_MAX;
    orc_pt bp = {-1, -1};
    int bettered = 0;
    for (unsigned k = candStart[t]; k < candStart[t + 1]; k++)
      best_fit(&e, cands[k], nb, cnt, &best, &bp, &bettered, NULL, NULL);
    outSum[t] = best;
    outPt[t] = bp;
    if (outCount) outCount[t] = cnt;
  }
  free((void *)e.offs);
}

unsigned long long orc_energy(const orc_params *p, const orc_format *f,
                              const unsigned char *target, unsigned tw, unsigned th,
                              const unsigned char *corpus, unsigned cw, unsigned ch,
                              const unsigned char *hasValue, const orc_pt *sourceOf,
                              const orc_pt *targets, unsigned n, unsigned *perTarget) {
  engine_ctx e;
  frozen_ctx(&e, p, f, target, tw, th, corpus, cw, ch, hasValue, sourceOf);
  neighbor nb[MAX_NEIGHBORS];
  unsigned long long total = 0;
  for (unsigned t = 0; t < n; t++) {
    unsigned cnt = build_patch(&e, targets[t], nb, 0);
    orc_pt s = sourceOf[targets[t].x + targets[t].y * (int)tw];
    int stopped;
    unsigned v = patch_metric(&e, s, nb, cnt, UINT_MAX, &stopped, NULL);
    if (perTarget) perTarget[t] = v;
    total += v;
  }
  free((void *)e.offs);
  return total;
}
