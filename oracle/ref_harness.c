/*
 * ref_harness.c -- exposes the reference engine's internals for pinning the
 * oracle.  TEST INFRASTRUCTURE ONLY.
 *
 * Compiled by oracle/build_ref.sh against the reference sources where they
 * lie (the reference tree is never copied): this translation unit includes
 * the reference lib/engine.c, so the file-static functions it defines
 * (prepare_neighbors, computeBestFit, prepareTargetPoints, refiner, ...)
 * are callable here.  Each wrapper below repeats a call sequence of
 * lib/engine.c:539-690 or lib/synthesize.h:426-642 and returns internal state
 * that engine() itself frees.
 */
#include "engine.c"

#include <string.h>

static void ref_noop_progress(int percent, void *ctx) { (void)percent; (void)ctx; }

static void ref_map_from_bytes(Map *m, const unsigned char *src, unsigned w, unsigned h, unsigned depth) {
  new_pixmap(m, w, h, depth);
  memcpy(m->data->data, src, (size_t)w * h * depth);
}

/* The sequence of lib/engine.c:594-673 with sourceOf/hasValue returned. */
int ref_engine_state(TImageSynthParameters *params, TFormatIndices *indices,
                     unsigned char *target, unsigned tw, unsigned th,
                     const unsigned char *corpus, unsigned cw, unsigned ch,
                     Coordinates *sourceOut, unsigned char *hasValueOut) {
  TImageSynthParameters parameters = *params;
  Map targetMap, corpusMap, recentProberMap, hasValueMap, sourceOfMap;
  pointVector targetPoints, corpusPoints, sortedOffsets;
  TPixelelMetricFunc corpusTargetMetric;
  TMapPixelelMetricFunc mapMetric;
  int cancel = 0;

  if (parameters.patchSize > IMAGE_SYNTH_MAX_NEIGHBORS) return IMAGE_SYNTH_ERROR_PATCH_SIZE_EXCEEDED;
  ref_map_from_bytes(&targetMap, target, tw, th, indices->total_bpp);
  ref_map_from_bytes(&corpusMap, corpus, cw, ch, indices->total_bpp);
  prepareTargetPoints(parameters.matchContextType, indices, &targetMap, &hasValueMap, &targetPoints);
  if (!targetPoints->len) return IMAGE_SYNTH_ERROR_EMPTY_TARGET;
  prepare_target_sources(&targetMap, &sourceOfMap);
  prepareCorpusPoints(indices, &corpusMap, &corpusPoints);
  if (!corpusPoints->len) return IMAGE_SYNTH_ERROR_EMPTY_CORPUS;
  prepareSortedOffsets(&targetMap, &corpusMap, &sortedOffsets);
  quantizeMetricFuncs(parameters.sensitivityToOutliers, parameters.mapWeight, corpusTargetMetric, mapMetric);
  GRand *prng = g_rand_new_with_seed(1198472);
  int error = orderTargetPoints(&parameters, targetPoints, prng);
  if (error) return error;
  prepareRecentProber(&corpusMap, &recentProberMap);
  refiner(parameters, indices, &targetMap, &corpusMap, &recentProberMap, &hasValueMap, &sourceOfMap,
          targetPoints, corpusPoints, sortedOffsets, prng, corpusTargetMetric, mapMetric,
          ref_noop_progress, NULL, &cancel);
  memcpy(target, targetMap.data->data, (size_t)tw * th * indices->total_bpp);
  if (sourceOut) memcpy(sourceOut, sourceOfMap.data->data, sizeof(Coordinates) * tw * th);
  if (hasValueOut) memcpy(hasValueOut, hasValueMap.data->data, (size_t)tw * th);
  free_map(&recentProberMap); free_map(&hasValueMap); free_map(&sourceOfMap);
  free_map(&targetMap); free_map(&corpusMap);
  g_array_free(targetPoints, TRUE); g_array_free(corpusPoints, TRUE); g_array_free(sortedOffsets, TRUE);
  return 0;
}

/* The reference target order (lib/engine.c:608-645 then orderTargetPoints). */
int ref_order_targets(TImageSynthParameters *params, TFormatIndices *indices,
                      const unsigned char *target, unsigned tw, unsigned th,
                      Coordinates *out, unsigned *count) {
  Map targetMap, hasValueMap;
  pointVector targetPoints;
  ref_map_from_bytes(&targetMap, target, tw, th, indices->total_bpp);
  prepareTargetPoints(params->matchContextType, indices, &targetMap, &hasValueMap, &targetPoints);
  GRand *prng = g_rand_new_with_seed(1198472);
  int error = orderTargetPoints(params, targetPoints, prng);
  memcpy(out, targetPoints->data, sizeof(Coordinates) * targetPoints->len);
  *count = targetPoints->len;
  free_map(&targetMap); free_map(&hasValueMap);
  g_array_free(targetPoints, TRUE);
  return error;
}

/* The reference sorted offsets, lib/engine.c:465-497. */
unsigned ref_sorted_offsets(unsigned tw, unsigned th, unsigned cw, unsigned ch, Coordinates *out) {
  Map t, c;
  pointVector offs;
  t.width = tw; t.height = th; c.width = cw; c.height = ch;
  prepareSortedOffsets(&t, &c, &offs);
  unsigned n = offs->len;
  memcpy(out, offs->data, sizeof(Coordinates) * n);
  g_array_free(offs, TRUE);
  return n;
}

/* The reference metric tables, lib/matchWeighting.h:194-204. */
void ref_metric_tables(double sensitivity, double mapWeight, unsigned short *ct, unsigned *mt) {
  TPixelelMetricFunc a;
  TMapPixelelMetricFunc b;
  quantizeMetricFuncs(sensitivity, mapWeight, a, b);
  memcpy(ct, a, sizeof a);
  memcpy(mt, b, sizeof b);
}

/* Frozen state: the reference prepare_neighbors + computeBestFit over an
 * explicit candidate list per target. */
void ref_frozen(TImageSynthParameters *params, TFormatIndices *indices,
                const unsigned char *target, unsigned tw, unsigned th,
                const unsigned char *corpus, unsigned cw, unsigned ch,
                const unsigned char *hasValue, const Coordinates *sourceOf,
                const Coordinates *targets, unsigned n,
                const unsigned *candStart, const Coordinates *cands,
                unsigned *outSum, Coordinates *outPt, unsigned *outCount, int fullSum) {
  Map targetMap, corpusMap, hasValueMap, sourceOfMap;
  pointVector sortedOffsets;
  TPixelelMetricFunc ct;
  TMapPixelelMetricFunc mt;
  TNeighbor neighbors[IMAGE_SYNTH_MAX_NEIGHBORS];
  ref_map_from_bytes(&targetMap, target, tw, th, indices->total_bpp);
  ref_map_from_bytes(&corpusMap, corpus, cw, ch, indices->total_bpp);
  ref_map_from_bytes(&hasValueMap, hasValue, tw, th, 1);
  new_coordmap(&sourceOfMap, tw, th);
  memcpy(sourceOfMap.data->data, sourceOf, sizeof(Coordinates) * tw * th);
  prepareSortedOffsets(&targetMap, &corpusMap, &sortedOffsets);
  quantizeMetricFuncs(params->sensitivityToOutliers, params->mapWeight, ct, mt);
  for (unsigned t = 0; t < n; t++) {
    guint count = prepare_neighbors(targets[t], params, indices, &targetMap, &hasValueMap,
                                    &sourceOfMap, sortedOffsets, neighbors);
    guint best = G_MAXUINT;
    Coordinates bp = {-1, -1};
    tBettermentKind kind = NO_BETTERMENT;
    for (unsigned k = candStart[t]; k < candStart[t + 1]; k++) {
      if (fullSum) best = G_MAXUINT;
      computeBestFit(cands[k], indices, &corpusMap, &best, &bp, count, neighbors, &kind,
                     RANDOM_CORPUS, ct, mt);
    }
    outSum[t] = best;
    outPt[t] = bp;
    if (outCount) outCount[t] = count;
  }
  free_map(&targetMap); free_map(&corpusMap); free_map(&hasValueMap); free_map(&sourceOfMap);
  g_array_free(sortedOffsets, TRUE);
}
