/*
 * resynthesizer.h -- C ABI of the GB300 synthesis engine (libresynthesizer.so).
 *
 * Drop-in for the reference's library interface: a caller compiled against
 * the reference headers (lib/imageSynth.h, lib/engine.h, lib/map.h,
 * lib/engineParams.h, lib/imageFormatIndicies.h) links against this library
 * unchanged.  Every declaration below states the reference declaration it
 * replaces; types keep the reference's memory layout.  Work runs on the
 * current CUDA device; there is no CPU fallback -- without a usable GPU the
 * synthesis entry points return RESYNTH_ERROR_DEVICE.
 */
#ifndef RESYNTHESIZER_GB300_H
#define RESYNTHESIZER_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ types */

/* lib/imageBuffer.h:12-19 */
typedef struct _ImageBuffer {
  unsigned char *data;
  unsigned int width;
  unsigned int height;
  size_t rowBytes;
} ImageBuffer;

/* lib/imageFormat.h:36-42 */
typedef enum ImageFormat { T_RGB, T_RGBA, T_Gray, T_GrayA } TImageFormat;

/* lib/engineParams.h:13-28, plus codes of this library from 100 on. */
typedef enum ImageSynthError {
  IMAGE_SYNTH_SUCCESS,
  IMAGE_SYNTH_ERROR_INVALID_IMAGE_FORMAT,
  IMAGE_SYNTH_ERROR_IMAGE_MASK_MISMATCH,
  IMAGE_SYNTH_ERROR_PATCH_SIZE_EXCEEDED,
  IMAGE_SYNTH_ERROR_MATCH_CONTEXT_TYPE_RANGE,
  IMAGE_SYNTH_ERROR_EMPTY_TARGET,
  IMAGE_SYNTH_ERROR_EMPTY_CORPUS,
  RESYNTH_ERROR_DEVICE = 100,        /* CUDA unavailable or a CUDA call failed */
  RESYNTH_ERROR_UNSUPPORTED = 101,   /* pixel layout or size outside the engine's limits */
  RESYNTH_ERROR_ARGUMENT = 102       /* NULL or inconsistent argument to an extension call */
} TImageSynthError;

/* lib/engineParams.h:31-86 */
typedef struct ImageSynthParametersStruct {
  int isMakeSeamlesslyTileableHorizontally;
  int isMakeSeamlesslyTileableVertically;
  int matchContextType;
  double mapWeight;
  double sensitivityToOutliers;
  unsigned int patchSize;
  unsigned int maxProbeCount;
} TImageSynthParameters;

/* lib/imageFormatIndicies.h:39-58 */
typedef unsigned char TPixelelIndex;
typedef struct indicesStruct {
  TPixelelIndex colorEndBip;
  TPixelelIndex alpha_bip;
  TPixelelIndex map_start_bip;
  TPixelelIndex map_end_bip;
  TPixelelIndex img_match_bpp;
  TPixelelIndex map_match_bpp;
  TPixelelIndex total_bpp;
  int isAlphaTarget;
  int isAlphaSource;
} TFormatIndices;

/* lib/glibProxy.h:86-92 (same layout as GLib's public GArray). */
typedef struct _GArray {
  char *data;
  unsigned int len;
} GArray;

/* lib/map.h:28-46 */
typedef struct {
  unsigned int width;
  unsigned int height;
  unsigned int depth;
  GArray *data;
} Map;
typedef unsigned char Pixelel;
typedef struct { int x; int y; } Coordinates;

/* ------------------------------------------------- reference entry points */

/* lib/imageSynth.h:31-40 (def lib/imageSynth.c:61-137) */
int imageSynth(ImageBuffer *imageBuffer, ImageBuffer *mask, TImageFormat imageFormat,
               TImageSynthParameters *parameters, void (*progressCallback)(int, void *),
               void *contextInfo, int *cancelFlag);

/* lib/imageSynth.h:42-52 (def lib/imageSynth.c:139-216) */
int imageSynth2(ImageBuffer *imageBuffer, ImageBuffer *mask, ImageBuffer *mask2,
                TImageFormat imageFormat, TImageSynthParameters *parameters,
                void (*progressCallback)(int, void *), void *contextInfo, int *cancelFlag);

/* lib/engine.h:3-12 (def lib/engine.c:539-690) */
int engine(TImageSynthParameters parameters, TFormatIndices *indices, Map *targetMap, Map *corpusMap,
           void (*progressCallback)(int, void *), void *contextInfo, int *cancelFlag);

/* lib/engineParams.h:91-94 (def lib/engineParams.c:8-19) */
void setDefaultParams(TImageSynthParameters *param);

/* lib/imageFormatIndicies.h:60-84 (defs lib/imageFormat.c:39-241) */
unsigned int countPixelelsPerPixelForFormat(TImageFormat format);
int prepareImageFormatIndicesFromFormatType(TFormatIndices *indices, TImageFormat format);
void prepareImageFormatIndices(TFormatIndices *indices, unsigned int count_color_channels_target,
                               unsigned int count_color_channels_map, int is_alpha_target,
                               int is_alpha_source, int isMap);
void prepareDefaultFormatIndices(TFormatIndices *formatIndices);

/* lib/map.h:49-99 (defs lib/mapOps.h:35-168) */
void free_map(Map *map);
void new_pixmap(Map *map, unsigned int width, unsigned int height, unsigned int depth);
void new_bytemap(Map *map, unsigned int width, unsigned int height);
void new_intmap(Map *map, unsigned int width, unsigned int height);
void new_coordmap(Map *map, unsigned int width, unsigned int height);
void set_bytemap(Map *map, unsigned char value);
void invert_bytemap(Map *map);
void interleave_mask(Map *pixmap, Map *mask);

/* ------------------------------------------------------------- extensions */
/* Not in the reference: mode selection, statistics, state access and the
 * device-resident path used for throughput measurement. */

typedef enum {
  /* Dependency wavefronts: each pass runs as batches of target pixels that are
   * synthesized in parallel; candidates are neighbour-source propagation plus
   * counter-based random probes.  The default. */
  RESYNTH_MODE_WAVEFRONT = 0,
  /* Sequential replay: target pixels are visited one at a time in the
   * reference's order with the reference's PRNG stream; the output is
   * byte-identical to the reference's single-threaded engine. */
  RESYNTH_MODE_REPLAY = 1
} TResynthMode;

/* Opaque objects of the learned proposal network (declared at the end). */
typedef struct TResynthNet TResynthNet;
typedef struct TResynthPairs TResynthPairs;

typedef struct {
  int mode;                   /* TResynthMode */
  unsigned int seed;          /* wavefront probe RNG seed (0 = 1198472) */
  unsigned int firstBatch;    /* wavefront: pass-0 first batch size (0 = default) */
  unsigned int refineBatches; /* wavefront: sequential batches per refinement pass (0 = default) */
  unsigned int warpsPerBlock; /* wavefront: 0 = autotuned */
  int recordState;            /* keep final sourceOf/hasValue for resynthGetState() */
  int profile;                /* time each synthesis-kernel launch with CUDA events (stats.waveMs) */
  unsigned int phaseSide;     /* wavefront: k of the k x k colour phases (0 = from the patch radius, 1 = none) */
  unsigned int bandGrowth;    /* wavefront: pass-0 band growth in percent for random orders (0 = 200) */
  unsigned int minPasses;     /* wavefront: run at least this many passes; 0 = default (3 for texture synthesis
                                 without context or map channels, else the reference's stop rule alone), 1 = the
                                 reference's stop rule alone */
  TResynthNet *net;           /* wavefront: score this network's proposals at every visit (NULL = none) */
  unsigned int proposals;     /* wavefront: how many of the network's 16 offsets are scored (0 = none) */
  TResynthPairs *dumpPairs;   /* wavefront: append (context, final source) training pairs at the end */
  unsigned int dumpStride;    /* every dumpStride-th target of the visit order gives a pair (0 = 16) */
  int graphs;                 /* wavefront: launch each pass as one captured CUDA graph */
  int separateRequests;       /* imageSynthBatch: one stream per request instead of the many-request launches */
  unsigned int bandGrowthLarge; /* wavefront: growth in percent of pass-0 bands of at least 1/64 of the pass (0 = default) */
  int batchLaunches;          /* wavefront: how passes are launched (the output is the same): 0 = chosen per
                                 problem class across calls (persistent cooperative launches with grid barriers
                                 between batches, 16 or 8 warps per CTA, or one launch per batch: the fastest
                                 over the first six calls of the class); 1 = one launch per batch; 2 = persistent */
  unsigned int proposalPasses; /* wavefront with a network: score its proposals in the first proposalPasses passes
                                 only (0 = every pass) */
  int probeShare;             /* wavefront: random probes keyed per target pixel or shared by groups of 16 batch
                                 slots: 0 = shared when the corpus is read from global memory, 1 = always
                                 shared, 2 = never */
} TResynthOptions;

typedef struct {
  unsigned long long visits;      /* target-pixel visits over all passes */
  unsigned long long evals;       /* candidate patches scored */
  unsigned long long terms;       /* neighbour terms evaluated (after early-out) */
  unsigned int passes;
  unsigned int passLength[6];
  unsigned int betters[6];
  unsigned int launches;          /* kernels launched by this call */
  double deviceMs;                /* GPU time of the synthesis kernels (CUDA events) */
  double totalMs;                 /* wall time of the call */
  unsigned long long h2dBytes, d2hBytes;
  double waveMs;                  /* profile: summed duration of the per-target synthesis kernels */
  unsigned int waveLaunches;      /* profile: how many launches waveMs covers */
  unsigned long long waveTerms;   /* profile: neighbour terms those launches evaluated */
  int launchMode;                 /* wavefront passes ran as: 0 persistent (16 warps per CTA), 1 persistent (8),
                                     2 one launch per batch, 3 persistent (the caller's warps); -1 replay */
} TResynthStats;

/* Default options (wavefront mode, or the mode named by the environment
 * variable RESYNTH_MODE=replay|wavefront). */
void resynthDefaultOptions(TResynthOptions *options);

/* Sets the mode imageSynth/imageSynth2/engine use in this process.
 * Returns the previous mode, or -1 for an unknown mode. */
int resynthSetMode(int mode);

/* engine() with options and statistics.  stats may be NULL. */
int engineEx(const TImageSynthParameters *parameters, const TFormatIndices *indices, Map *targetMap,
             Map *corpusMap, void (*progressCallback)(int, void *), void *contextInfo, int *cancelFlag,
             const TResynthOptions *options, TResynthStats *stats);

/* imageSynth() with options and statistics (mask2 may be NULL). */
int imageSynthEx(ImageBuffer *imageBuffer, ImageBuffer *mask, ImageBuffer *mask2, TImageFormat imageFormat,
                 TImageSynthParameters *parameters, void (*progressCallback)(int, void *), void *contextInfo,
                 int *cancelFlag, const TResynthOptions *options, TResynthStats *stats);

/* Final state of the last engineEx/imageSynthEx call on this thread that ran
 * with options->recordState: sourceOf (width*height Coordinates, (-1,-1) = none)
 * and hasValue (width*height bytes) of the target.  Returns 0 or an error. */
int resynthGetState(Coordinates *sourceOf, unsigned char *hasValue, unsigned int width, unsigned int height);

/* Same as engineEx on pixmaps that already live in device memory (the
 * interleaved layout of Map data).  dTarget is updated in place.  stream is a
 * cudaStream_t (NULL = the library's stream).  Progress callbacks and cancel
 * behave as in engineEx. */
int engineDevice(const TImageSynthParameters *parameters, const TFormatIndices *indices,
                 unsigned char *dTarget, unsigned int targetWidth, unsigned int targetHeight,
                 const unsigned char *dCorpus, unsigned int corpusWidth, unsigned int corpusHeight,
                 void *stream, void (*progressCallback)(int, void *), void *contextInfo, int *cancelFlag,
                 const TResynthOptions *options, TResynthStats *stats);

/* Frozen-state best fit.  For each target point, the patch is built from the
 * given frozen state exactly as the reference's prepare_neighbors
 * (lib/synthesize.h:189-241), and the candidates candidates[candStart[t] ..
 * candStart[t+1]) are scored in order with the reference's computeBestFit rule
 * (lib/synthesize.h:266-400: strict-less update from UINT_MAX).  Outputs per
 * target: bestSum (UINT_MAX if no candidate), bestPoint ((-1,-1) if none) and
 * patchCount (neighbours in the patch).  All pointers are host memory;
 * target/corpus are interleaved pixmaps, hasValue/sourceOf are target-sized. */
int resynthFrozenBestFit(const TImageSynthParameters *parameters, const TFormatIndices *indices,
                         const unsigned char *target, unsigned int targetWidth, unsigned int targetHeight,
                         const unsigned char *corpus, unsigned int corpusWidth, unsigned int corpusHeight,
                         const unsigned char *hasValue, const Coordinates *sourceOf,
                         const Coordinates *targets, unsigned int targetCount,
                         const unsigned int *candStart, const Coordinates *candidates,
                         unsigned int *bestSum, Coordinates *bestPoint, unsigned int *patchCount);

/* Patch energy of a final state: the sum over targets of the full-patch metric
 * (no early-out) at each target's source, patches built from the given state.
 * perTarget (may be NULL) receives each target's term. */
int resynthPatchEnergy(const TImageSynthParameters *parameters, const TFormatIndices *indices,
                       const unsigned char *target, unsigned int targetWidth, unsigned int targetHeight,
                       const unsigned char *corpus, unsigned int corpusWidth, unsigned int corpusHeight,
                       const unsigned char *hasValue, const Coordinates *sourceOf,
                       const Coordinates *targets, unsigned int targetCount,
                       unsigned long long *energy, unsigned int *perTarget);

/* No counterpart in the reference.  Test entry of the two pass-0 patch
 * builders of wavefront mode: for each target (a pixel without a value), the
 * offsets (dx, dy) of its patch neighbours in patch order, self excluded, as
 * prepare_neighbors (lib/synthesize.h:158-241) chooses them under the
 * wavefront offset radius, found by walking the sorted offset list (useGrid
 * 0) or from the cell grid of least visit stamps (useGrid 1).  hasValue is
 * width x height bytes; offsets receives n x 63 Coordinates, counts n. */
int resynthPatchNeighbours(const unsigned char *hasValue, unsigned int width, unsigned int height,
                           unsigned int patchSize, const Coordinates *targets, unsigned int n, int useGrid,
                           Coordinates *offsets, unsigned int *counts);

/* No counterpart in the reference.  Test entry of the device-side visit
 * order of the directional and brushfire types (matchContextType 2..8): the
 * n points (host memory, in the engine's row-major target order) reordered
 * as lib/orderTarget.h:268-343 orders them -- the sort by the type's key from
 * the bounding-box centre, then the banded shuffle drawn from the PRNG seeded
 * with 1198472 -- computed by the kernels wavefront mode uses. */
int resynthOrderTargets(int matchContextType, const Coordinates *points, unsigned int n, Coordinates *ordered);

/* No counterpart in the reference.  Frozen-state best fit, as
 * resynthFrozenBestFit, for callers that cannot let a library allocate device
 * memory -- a host application that reserves the GPU's memory up front and
 * hands out every buffer from its own pool, or a latency-critical loop that
 * cannot afford cudaMalloc's implicit device-wide synchronisation.
 *   - Every pointer is device memory owned by the caller, with the same
 *     meaning as in resynthFrozenBestFit; the call allocates nothing.
 *   - Working memory is one 8 MiB array inside the library, held by every GPU
 *     that loads the library until the process exits.  The images must fit:
 *     4 KiB + 4 * (targetWidth*targetHeight + corpusWidth*corpusHeight rounded
 *     up to 4) bytes, doubled when map channels are matched; larger images
 *     return RESYNTH_ERROR_UNSUPPORTED with the reason in resynthLastError().
 *   - Work is enqueued on `stream` (a cudaStream_t, NULL = the default stream)
 *     and the outputs are ready when the stream reaches that point.
 *   - All calls share the one working array: calls that may overlap on the GPU
 *     (on different streams without ordering between them) race and corrupt
 *     each other's results.  Every call rewrites everything it reads there.
 *   - The call enqueues kernels only (the metric tables travel as kernel
 *     arguments), so it can be captured into a CUDA graph; but the first
 *     call on each device looks up the array's device address with that
 *     device current, so make that first call before any stream capture. */
int resynthFrozenBestFitNoAlloc(const TImageSynthParameters *parameters, const TFormatIndices *indices,
                                const unsigned char *dTarget, unsigned int targetWidth, unsigned int targetHeight,
                                const unsigned char *dCorpus, unsigned int corpusWidth, unsigned int corpusHeight,
                                const unsigned char *dHasValue, const Coordinates *dSourceOf,
                                const Coordinates *dTargets, unsigned int targetCount,
                                const unsigned int *dCandStart, const Coordinates *dCandidates,
                                unsigned int *dBestSum, Coordinates *dBestPoint, unsigned int *dPatchCount,
                                void *stream);

/* One request of imageSynthBatch: the arguments of imageSynth2 (mask2 NULL =
 * imageSynth) and the request's own return code. */
typedef struct {
  ImageBuffer *image;
  ImageBuffer *mask;
  ImageBuffer *mask2;
  TImageFormat format;
  TImageSynthParameters *parameters;   /* NULL = defaults */
  int result;                          /* out: the request's return code */
} TResynthRequest;

/* No counterpart in the reference (which heals one image per call).  Runs
 * `count` independent requests of any sizes and formats.  In wavefront mode,
 * requests with a random order (matchContextType 0 or 1) are synthesized
 * together: each pass runs step b -- batch b of every request -- as one
 * launch per pixel layout.  Other requests (and all of them with
 * options->separateRequests) run on `concurrency` host workers (0 = 8), each
 * with its own CUDA stream.  Each request's result equals an imageSynthEx
 * call with the same options.  stats (may be NULL) sums all requests.
 * Returns 0, or the first nonzero request result. */
int imageSynthBatch(TResynthRequest *requests, unsigned int count, unsigned int concurrency,
                    const TResynthOptions *options, TResynthStats *stats);

/* Text of the last error on this thread ("" if none). */
const char *resynthLastError(void);

/* ------------------------------------------------------ learned proposals */

/* No counterpart in the reference.  Test entry of the tensor-core GEMM that
 * the proposal network runs on: D[M x N] = bf16(A)[M x K] . bf16(B)[N x K]^T
 * with fp32 accumulation (A, B, D host row-major; inputs rounded to nearest
 * even bf16).  N must be a multiple of 32. */
int resynthTcGemm(const float *A, const float *B, int M, int N, int K, float *D);

/* No counterpart in the reference.  Test entry of the kernels' bounded waits:
 * runs one GEMM tile whose load barrier can never complete, so its wait gives
 * up after a fixed number of polls.  Returns RESYNTH_ERROR_DEVICE ("a
 * tensor-core wait ran out") with the CUDA context still usable. */
int resynthTcWaitTimeout(void);

/* No counterpart in the reference.  Measures, on the current device, a peak
 * of one of the two on-chip resources the synthesis kernels are bound by:
 * which = 0: shared-memory load bandwidth (conflict-free 16-byte loads), in
 * GB/s over the whole GPU; which = 1: 32-bit integer ALU throughput (chains
 * of add and xor), in G ops/s.  Three warm-up launches, then the best of
 * five timed with CUDA events; *ms (may be NULL) receives that launch's time. */
int resynthMicrobench(int which, double *value, double *ms);

/* No counterpart in the reference.  Test entry of the grid barrier the
 * persistent wavefront kernel places between batches: a cooperative launch
 * (two CTAs per SM) in which every CTA meets `rounds` barriers, except CTA
 * absentCta (pass -1 for none), which leaves at once.  A barrier wait longer
 * than timeoutNs nanoseconds gives up.  *passed receives the barriers passed
 * summed over CTAs, *error the kernel's error bits (4 = a barrier wait ran
 * out).  Returns 0 when the launch completed, with the CUDA context usable. */
int resynthGridBarrierProbe(int rounds, int absentCta, long long timeoutNs, unsigned int *passed,
                            unsigned int *error);

/* No counterpart in the reference.  The proposal network reads an 11 x 11
 * context around a target pixel and emits 16 source offsets; in wavefront
 * mode (TResynthOptions.net) they join each visit's candidates next to the
 * neighbours' continuations and the random probes (lib/synthesize.h:536-604)
 * and are scored by the same exact metric, so the plain search stays both
 * fallback and arbiter.
 *
 * Context: 11 x 11 pixels x 16 bf16 channels, row-major (y, x, channel),
 * centred on the target.  Channels 0-2 colour (grey repeated) as v/255 - 0.5,
 * channel 3 = 1 where the pixel has a value (colours are 0 where it has
 * none), channel 4 = first map channel as m/255 - 0.5 (0 without maps),
 * channels 5-15 = 0; pixels outside the image are all 0.
 * Network: four 3x3 convolutions of 32 channels with ReLU (11 -> 9 -> 7 -> 5
 * -> 3), then a 3x3 convolution to 32 outputs = 16 x (dx, dy) in units of 64
 * pixels.  BF16 weights and activations, fp32 accumulation on the tensor
 * cores.  Parameters (fp32, resynthNetParamCount() of them): for each layer
 * W [32 x 9*Cin] (column (ky*3 + kx)*Cin + c, Cin = 16 then 32) then b [32].
 * Training minimises the relaxed multiple-choice loss: the offset nearest the
 * label (source - target, / 64, clipped to +-16) weighs 0.95, each other
 * 0.05/15, loss = mean of sum_k w_k |o_k - label|^2, with Adam. */
unsigned int resynthNetParamCount(void);

/* A network with He-normal weights drawn from `seed`, on the current device.
 * NULL on failure (reason in resynthLastError()). */
TResynthNet *resynthNetCreate(unsigned int seed);
void resynthNetDestroy(TResynthNet *net);
int resynthNetGetParams(TResynthNet *net, float *params);
int resynthNetSetParams(TResynthNet *net, const float *params);

/* Outputs [n x 32] for contexts [n x 11 x 11 x 16] (bf16 bits), host
 * buffers.  path 0 = the fused inference kernel, 1 = the training kernels. */
int resynthNetForward(TResynthNet *net, const unsigned short *contexts, unsigned int n, float *out, int path);

/* Loss and its gradient w.r.t. the parameters (resynthNetParamCount() floats)
 * for contexts [n x 11 x 11 x 16] and labels [n x 2]; host buffers. */
int resynthNetGradients(TResynthNet *net, const unsigned short *contexts, const float *labels, unsigned int n,
                        float *gradient, float *loss);

typedef struct {
  unsigned int steps;          /* Adam steps (0 = 2000) */
  unsigned int batch;          /* pairs per step (0 = 512) */
  float learningRate;          /* 0 = 1e-3 */
  unsigned int seed;           /* minibatch sampling */
} TResynthTrainOptions;

/* Trains on the pairs with the tensor-core forward and backward kernels.
 * lossOut (may be NULL) receives the mean loss of the last tenth of the steps. */
int resynthNetTrain(TResynthNet *net, TResynthPairs *pairs, const TResynthTrainOptions *options, float *lossOut);

/* Device-resident store of training pairs (context, label). */
TResynthPairs *resynthPairsCreate(unsigned int capacity);
void resynthPairsDestroy(TResynthPairs *pairs);
unsigned int resynthPairsCount(const TResynthPairs *pairs);
/* Appends n host pairs (contexts as above, labels [n x 2] in units of 64 px);
 * returns the number stored (the store keeps its first `capacity` pairs). */
unsigned int resynthPairsAdd(TResynthPairs *pairs, const unsigned short *contexts, const float *labels,
                             unsigned int n);
/* Copies pairs [first, first + n) to host buffers (either may be NULL). */
int resynthPairsRead(const TResynthPairs *pairs, unsigned int first, unsigned int n, unsigned short *contexts,
                     float *labels);

#ifdef __cplusplus
}
#endif
#endif
