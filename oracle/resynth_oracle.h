/*
 * resynth_oracle.h -- CPU oracle for the resynthesizer synthesis engine.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * engine (bootchk/resynthesizer, lib/engine.c and the headers it includes),
 * used as the checker for the GPU engine.  Only tests/, the smoke check in
 * __graft_entry__.py and bench.py's CPU-baseline leg may load it; the product
 * library never links or calls it.
 *
 * Parity is pinned: tests/test_oracle_pin.py runs this restatement and the
 * reference compiled from its own sources (oracle/build_ref.sh) on the same
 * inputs and requires byte-identical results.
 *
 * Struct layouts mirror the reference ABI so buffers can be shared:
 *   orc_params  == TImageSynthParameters   (lib/engineParams.h:31-86)
 *   orc_format  == TFormatIndices          (lib/imageFormatIndicies.h:46-58)
 *   orc_pt      == Coordinates             (lib/map.h:43-46)
 */
#ifndef RESYNTH_ORACLE_H
#define RESYNTH_ORACLE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int tileH;             /* isMakeSeamlesslyTileableHorizontally */
  int tileV;             /* isMakeSeamlesslyTileableVertically   */
  int matchContextType;  /* 0..8 */
  double mapWeight;
  double sensitivityToOutliers;
  unsigned int patchSize;
  unsigned int maxProbeCount;
} orc_params;

typedef struct {
  unsigned char colorEndBip, alpha_bip, map_start_bip, map_end_bip;
  unsigned char img_match_bpp, map_match_bpp, total_bpp;
  int isAlphaTarget, isAlphaSource;
} orc_format;

typedef struct { int x, y; } orc_pt;

typedef struct {
  unsigned char *data;
  unsigned int width, height;
  size_t rowBytes;
} orc_image_buffer;   /* == ImageBuffer (lib/imageBuffer.h:12-19) */

typedef struct {
  unsigned long long visits;    /* target visits over all passes */
  unsigned long long evals;     /* computeBestFit-equivalent calls */
  unsigned long long terms;     /* neighbour terms evaluated (with early-out) */
  unsigned long long draws;     /* PRNG draws for random probes */
  unsigned int passes;          /* passes run */
  unsigned int pass_len[6];     /* target indices per pass */
  unsigned int betters[6];      /* betters per pass */
} orc_stats;

/* Metric tables, lib/matchWeighting.h:142-204 (non-symmetric build). */
void orc_metric_tables(double sensitivity, double mapWeight,
                       unsigned short color_table[512], unsigned int map_table[512]);

/* Format indices, lib/imageFormat.c:116-207 and :65-113. */
void orc_format_indices(orc_format *f, unsigned colors, unsigned mapColors,
                        int alphaTarget, int alphaSource, int isMap);
int orc_format_from_type(orc_format *f, int imageFormat);
unsigned orc_pixelels_for_format(int imageFormat);

/* Sorted offsets, lib/engine.c:465-497; returns count, fills out (caller
 * allocates (2*min(w)-1)*(2*min(h)-1) entries). */
size_t orc_sorted_offsets(unsigned tw, unsigned th, unsigned cw, unsigned ch, orc_pt *out);

/* Target order, lib/orderTarget.h:268-343 (uses libc srand/rand/qsort like the
 * reference's standalone build).  Seeds the PRNG with 1198472 first.  Returns
 * 0 or the MATCH_CONTEXT_TYPE_RANGE error code. */
int orc_order_targets(int matchContextType, orc_pt *points, unsigned n);

/* The engine on interleaved pixmaps, lib/engine.c:539-690.
 * target: tw*th*total_bpp bytes, modified in place (colours only).
 * nthreads == 1: the single-threaded refiner (lib/refiner.h:42-122);
 * nthreads > 1: the threaded refiner, alternative 1 (lib/refinerThreaded.h:259-381).
 * sourceOut (tw*th) and hasValueOut (tw*th) receive the final state when non-NULL. */
int orc_engine(const orc_params *p, const orc_format *f,
               unsigned char *target, unsigned tw, unsigned th,
               const unsigned char *corpus, unsigned cw, unsigned ch,
               int nthreads,
               void (*progress)(int, void *), void *ctx, int *cancel,
               orc_stats *stats, orc_pt *sourceOut, unsigned char *hasValueOut);

/* Simple API, lib/imageSynth.c:61-137 (mask2 == NULL) and :139-216. */
int orc_image_synth(orc_image_buffer *img, orc_image_buffer *mask, orc_image_buffer *mask2,
                    int imageFormat, const orc_params *p, int nthreads,
                    void (*progress)(int, void *), void *ctx, int *cancel,
                    orc_stats *stats);

/* Frozen-state best fit: for each target, build the patch from the frozen
 * hasValue/sourceOf/target maps (lib/synthesize.h:189-241) and run
 * computeBestFit (lib/synthesize.h:266-400) over its candidate list in order,
 * starting from best = UINT_MAX.  outPt = (-1,-1) when no candidate bettered. */
void orc_frozen(const orc_params *p, const orc_format *f,
                const unsigned char *target, unsigned tw, unsigned th,
                const unsigned char *corpus, unsigned cw, unsigned ch,
                const unsigned char *hasValue, const orc_pt *sourceOf,
                const orc_pt *targets, unsigned n,
                const unsigned *candStart, const orc_pt *cands,
                unsigned *outSum, orc_pt *outPt, unsigned *outCount);

/* Patch energy: sum over targets of the full-patch metric (no early-out) at
 * each target's source, with patches built from the given final state. */
unsigned long long orc_energy(const orc_params *p, const orc_format *f,
                              const unsigned char *target, unsigned tw, unsigned th,
                              const unsigned char *corpus, unsigned cw, unsigned ch,
                              const unsigned char *hasValue, const orc_pt *sourceOf,
                              const orc_pt *targets, unsigned n, unsigned *perTarget);

/* libc rand() stream after srand(seed): fills out[n]. */
void orc_rand_stream(unsigned seed, unsigned n, int *out);

/* The GPU library's wavefront mode (its default engine() path) restated on
 * the CPU, for every visit order and default options: target
 * (tw*th*total_bpp) is modified in place.  seed 0 = the library's default.
 * Returns 0, -1 for a matchContextType outside 0..8, -2 for an empty target
 * or corpus.
 * passesOut and bettersOut (6 entries) may be NULL.  (wave_oracle.c) */
int orc_wave_engine(const orc_params *p, const orc_format *f, unsigned char *target, unsigned tw, unsigned th,
                    const unsigned char *corpus, unsigned cw, unsigned ch, unsigned seed, int nthreads,
                    unsigned *passesOut, unsigned *bettersOut);

/* Schedule options of the wavefront mode (TResynthOptions' firstBatch,
 * bandGrowth, phaseSide, minPasses; 0 = the library's default). */
typedef struct {
  unsigned int firstBatch, bandGrowth, phaseSide, minPasses;
  unsigned int probeShare;   /* 0: the library's rule, 1: always share probes by slot group, 2: never */
} orc_wave_opts;

/* orc_wave_engine with schedule options (opt may be NULL) and optional
 * outputs: the final sourceOf and hasValue (tw*th each) and the number of
 * non-empty batches run. */
int orc_wave_engine_ex(const orc_params *p, const orc_format *f, unsigned char *target, unsigned tw, unsigned th,
                       const unsigned char *corpus, unsigned cw, unsigned ch, unsigned seed, int nthreads,
                       const orc_wave_opts *opt, unsigned *passesOut, unsigned *bettersOut, orc_pt *sourceOut,
                       unsigned char *hasValueOut, unsigned *batchesOut);

/* The Simple API (lib/imageSynth.c:61-216, the reference's adapters) around
 * the wavefront restatement: what the GPU library's imageSynth / imageSynth2
 * give in wavefront mode.  mask2 NULL = imageSynth.  Returns the reference's
 * error codes. */
int orc_wave_image_synth(orc_image_buffer *img, orc_image_buffer *mask, orc_image_buffer *mask2, int imageFormat,
                         const orc_params *p, unsigned seed, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
