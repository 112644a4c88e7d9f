// synth_internal.h -- structures shared by the host engine (synth_host.cpp)
// and the CUDA kernels (synth_kernels.cu).  Not part of the public ABI.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace rs {

constexpr int kMaxNeighbors = 64;     // IMAGE_SYNTH_MAX_NEIGHBORS, lib/imageSynthConstants.h:26
constexpr int kPasses = 6;            // MAX_PASSES, lib/passes.h:51
constexpr int kTable = 512;           // metric table length, lib/matchWeighting.h:132-133
constexpr int kPad = 6;               // masked border of the padded corpus copy used by the wavefront kernel

// Device view of one synthesis problem.  Pixels are repacked into 32-bit
// words: px = mask | c0 << 8 | c1 << 16 | c2 << 24 and map = m0 | m1 << 8 | m2 << 16.
// Coordinates are int2 (x, y); a source of (-1, -1) means "none".
struct Problem {
  int tw, th;                 // target size
  int cw, ch;                 // corpus size
  int nc, nm;                 // colour and map channels matched (1..3, 0..3)
  uint32_t* tpx;              // target pixels (tw*th)
  uint32_t* tmap;             // target map channels (tw*th) or null
  uint8_t* has;               // hasValue (tw*th)
  const int* vis;             // wavefront: visit stamp per pixel; a pixel has a value for batch b iff vis < b
                              // (null: use has)
  int2* src;                  // sourceOf (tw*th)
  const uint32_t* cpx;        // corpus pixels (cw*ch)
  const uint32_t* cmap;       // corpus map channels (cw*ch) or null
  const uint32_t* cpxPad;     // the corpus with a kPad-wide masked border ((cw+2kPad) x (ch+2kPad))
  const uint2* cpmPad;        // with map channels: the padded corpus as (corpus word, map word) pairs, else null
  int padW;                   // cw + 2 * kPad
  const int2* cpts;           // corpus points (selected and not transparent)
  int ncorpus;
  const int2* offs;           // sorted offsets, offs[0] == (0, 0)
  int noffs;
  int patchLimit;             // the patch stops growing at max(patchSize, 2) neighbours
  int tileH, tileV;
  int boxW, boxH;             // offsets span |dx| < boxW, |dy| < boxH (the smaller image)
  long long maxD2;            // offsets are cut at dx^2 + dy^2 <= maxD2 (wavefront: at most 256^2, which the
                              // pass-0 nearest-key lists pack into 32-bit keys)
  int fullCorpus;             // every corpus pixel is a corpus point: probes need no list
  uint32_t clipCost;          // 65535 * nc + mapTable[0] * nm
  const uint32_t* ctab;       // colour metric table (512 entries, widened to 32 bits)
  const uint32_t* mtab;       // map metric table (512)
  const int* cellMin;         // wavefront pass 0: least visit stamp of each kCell x kCell cell, or null
  int cellsW, cellsH;
};

// Side of the cells of Problem::cellMin (a power of two).
constexpr int kCellShift = 3;
constexpr int kCell = 1 << kCellShift;

// Grid-wide barrier of the persistent wavefront kernel (cooperative launch):
// zeroed by the host before every launch.
struct GridBar {
  unsigned int count;            // arrivals so far (barrier k is passed once it reaches k * CTAs)
  unsigned int stopInv;          // 0, or ~k: every CTA leaves at barrier k (the earliest requested)
  unsigned int error;            // error bits of a launch that has no Counters of its own (many requests)
  unsigned int pad;
};

// Most requests one persistent many-request launch takes (its slot prefix
// sits in shared memory).
constexpr int kMultiPersistentMaxRequests = 4096;

// Counters::error bits.
constexpr unsigned kErrStage = 1u;     // a bulk copy into shared memory did not complete
constexpr unsigned kErrBarrier = 4u;   // a grid-barrier wait ran out (a CTA never arrived)

// Device counters accumulated by the synthesis kernels.
struct Counters {
  unsigned long long evals;
  unsigned long long terms;
  unsigned long long refEvals;   // replay: computeBestFit calls the reference would make
  unsigned int betters;
  unsigned int cursor;           // replay: position in the PRNG stream
  unsigned int error;            // nonzero: a kernel gave up (bounded wait ran out)
  unsigned int pad;
};

// Sequential replay of the reference order (one CTA).
struct ReplayArgs {
  Problem pb;
  const int2* targets;           // targetPoints in the reference order
  unsigned int* recentProber;    // cw*ch, init 0xFFFFFFFF
  const int* randStream;         // libc rand() outputs after srand(1198472) and ordering
  unsigned int randCount;
  unsigned int trys;
  Counters* ctr;
};

// One wavefront batch: targets[batchStart[batch] .. batchStart[batch + 1])
// are synthesized together (the range lives in device memory, so batches can
// be enqueued without a host round trip).
struct WaveArgs {
  Problem pb;
  const int2* targets;           // this pass's targets, bucketed by batch
  const int* batchStart;         // device: batch boundaries
  int batch;
  int visCur;                    // pixels with vis < visCur have values during this batch
  int inPlace;                   // write results straight into the state (else stage for k_commit)
  int sparse;                    // allowed: patches from the valued list targets[0 .. b0)
  long long sparseLimit2;        // ... while b0 * b0 < sparseLimit2
  unsigned int trys;
  unsigned int seed, pass;
  int2* stageSrc;                // per-batch-slot new source, (-2, -2) = unchanged
  Counters* ctr;
  const volatile int* abortFlag; // host-mapped; nonzero stops the batch
  const int2* props;             // proposal network's sources, 16 per target of the band, or null
  int nprop;                     // how many of each target's 16 are scored
  int propBatch0;                // the band's first batch: props index = t - batchStart[propBatch0]
  int probeShare;                // random probes keyed by (batch, slot / 16) instead of the pixel
  int nbatches;                  // many-request steps: batches of this pass (0 = inactive)
  // Persistent kernel (one cooperative launch runs batches batch .. batchEnd - 1
  // with a grid barrier after each, and a commit phase between barriers when
  // results are staged):
  int batchEnd;
  unsigned int* queue;           // per batch: next slot to hand out (zeroed by the host), or null = static shares
  GridBar* gbar;
  long long barTimeoutNs;        // a barrier wait longer than this gives up (kErrBarrier)
};

// One request's bucketing of a pass, for rs_prep_batches_multi (the
// arguments of rs_prep_batches with its work split out; cellMin non-null =
// also the pass-0 cell minima of vis).
struct PrepJob {
  const int2* targets;
  int n, tw, th, endRank, randomOrder;
  uint32_t seed;
  const int* bandEnds;
  const int* bandPhased;
  int nbands, k;
  int* keys;
  int* counts;
  int* offsets;
  int nchunks;
  int* batchStart;
  int2* out;
  int* vis;
  int* cellMin;
};

// One Simple-API request of the many-request path, for the set-up and
// write-back kernels that serve every request of a call at once: the caller's
// buffers (uploaded as they are, row padding included), the interleaved
// pixmaps the adaption writes, the packed words, the prepared state and the
// request's first compaction chunk.
struct SetupJob {
  const uint8_t* img;
  size_t imgRow;
  const uint8_t* mask;
  size_t maskRow;
  const uint8_t* mask2;
  size_t mask2Row;
  int w, h, bpp;                 // the caller's pixel: bpp bytes
  int nc, alpha, alphaT, alphaS, useContext;
  uint8_t* target;               // interleaved pixmaps, bpp + 1 bytes per pixel
  uint8_t* corpus;
  uint32_t* tpx;
  uint32_t* cpx;
  uint32_t* cpxPad;
  int padW;
  uint8_t* has;
  int2* src;
  int* vis;
  int2* targets;
  int2* cpts;
  int chunk0;                    // first compaction chunk (rs_setup_chunks(w * h) of them)
  int writeBack;                 // write-back kernel: 1 = put the colours into img
};

// Frozen-state scoring and energy.
struct ScoreArgs {
  Problem pb;
  const int2* targets;
  int n;
  const unsigned int* candStart; // frozen: n+1 offsets into cands
  const int2* cands;
  unsigned int* outSum;
  int2* outPt;
  unsigned int* outCount;
  unsigned long long* energy;    // energy mode: total
};

}  // namespace rs

// Kernel launchers (synth_kernels.cu).  All return a cudaError_t.
extern "C" {
cudaError_t rs_launch_pack(const uint8_t* raw, int w, int h, int bpp, int colorStart, int nc, int mapStart,
                           int nm, uint32_t* px, uint32_t* map, cudaStream_t s);
cudaError_t rs_launch_pack_padded(const uint8_t* raw, int w, int h, int bpp, int nc, int mapStart, int nm,
                                  uint32_t* px, uint2* pm, cudaStream_t s);
cudaError_t rs_launch_unpack_colors(uint8_t* raw, int w, int h, int bpp, int nc, const uint32_t* px,
                                    cudaStream_t s);
cudaError_t rs_launch_replay(const rs::ReplayArgs& a, int t0, int t1, cudaStream_t s);
cudaError_t rs_launch_wave(const rs::WaveArgs& a, int warpsPerBlock, int maxCtas, cudaStream_t s);
cudaError_t rs_launch_commit(const rs::WaveArgs& a, int maxCtas, cudaStream_t s);
// Batches a.batch .. a.batchEnd - 1 of one problem in one cooperative launch
// of at most maxCtas CTAs (0 = one per resident slot of the GPU).
cudaError_t rs_launch_wave_persistent(const rs::WaveArgs& a, int warpsPerBlock, int maxCtas, cudaStream_t s);
// Whether this device can run the persistent kernel (cooperative launches).
int rs_persistent_supported();
int rs_wave_corpus_staged(const rs::Problem& pb, int warps);
cudaError_t rs_launch_wave_multi(const rs::WaveArgs* jobs, int nreq, const int* prefix, int step, int visCur, int nc,
                                 int map, int maxCtas, const volatile int* abortFlag, cudaStream_t s);
cudaError_t rs_launch_multi_prefix(const rs::WaveArgs* jobs, int nreq, int step, int* prefix, cudaStream_t s);
// Every step's slot prefix (steps x (nreq + 1) ints) for the persistent many-request pass.
cudaError_t rs_launch_multi_prefix_all(const rs::WaveArgs* jobs, int nreq, int steps, int* prefix, cudaStream_t s);
// Steps 0 .. steps - 1 of a pass of many requests of one pixel layout in one cooperative launch.
cudaError_t rs_launch_wave_multi_persistent(const rs::WaveArgs* jobs, int nreq, int steps, const int* prefix,
                                            unsigned* queue, int pass, int staged, rs::GridBar* gb,
                                            const volatile int* abortFlag, int nc, int map, long long timeoutNs,
                                            cudaStream_t s);

cudaError_t rs_launch_commit_multi(const rs::WaveArgs* jobs, int nreq, const int* prefix, int step, int maxCtas,
                                   cudaStream_t s);
cudaError_t rs_launch_frozen(const rs::ScoreArgs& a, cudaStream_t s);
cudaError_t rs_launch_energy(const rs::ScoreArgs& a, cudaStream_t s);
cudaError_t rs_prep_target(const uint8_t* raw, int w, int h, int bpp, int alpha, int hasAlpha, int useContext,
                           uint8_t* has, int2* src, int* scratch, int2* targets, int* counts, cudaStream_t s);
cudaError_t rs_prep_corpus(const uint8_t* raw, int w, int h, int bpp, int alpha, int hasAlpha, int* scratch,
                           int2* points, int* count, cudaStream_t s);
int rs_prep_scratch_ints(int w, int h);
cudaError_t rs_prep_batches(const int2* targets, int n, int tw, int endRank, int randomOrder, uint32_t seed,
                            const int* dBandEnds, const int* dBandPhased, int nbands, int k, int* work,
                            int* batchStart, int2* out, int* vis, cudaStream_t s);
size_t rs_prep_batches_ints(int n, int nkeys);
// rs_prep_batches (and pass-0 cell minima) for njobs requests in five launches:
// dJobs[njobs] in device memory, dChunk0[j] = the first bucketing chunk of
// request j (chunks of rs_prep_chunks(n) each, totalChunks in all), maxKeys =
// the largest nbands * k * k, cellBlocks = CTAs per request for the cell
// minima (0 = none).
cudaError_t rs_prep_batches_multi(const rs::PrepJob* dJobs, const int* dChunk0, int njobs, int totalChunks,
                                  int maxKeys, int cellBlocks, cudaStream_t s);
int rs_prep_chunks(int n);
// The many-request set-up for njobs requests (dJobs in device memory, dChunk0
// their first chunks, njobs + 1 entries): adaption, packing, initial state and
// visit stamps, then the compaction of targets and corpus points;
// counts[4 j .. 4 j + 2] = targets, any context, corpus points of request j
// (zeroed here).  work: rs_setup_work_ints(totalChunks, njobs) ints.
cudaError_t rs_setup_multi(const rs::SetupJob* dJobs, const int* dChunk0, int njobs, int totalChunks, int maxPx,
                           int* counts, int* work, cudaStream_t s);
int rs_setup_chunks(int npx);
size_t rs_setup_work_ints(int totalChunks, int njobs);
// The colours of every request with writeBack set back into its uploaded image.
cudaError_t rs_writeback_multi(const rs::SetupJob* dJobs, int njobs, int maxPx, cudaStream_t s);
cudaError_t rs_adapt(const uint8_t* img, size_t imgRow, const uint8_t* mask, size_t maskRow, const uint8_t* mask2,
                     size_t mask2Row, int w, int h, int bpp, uint8_t* target, uint8_t* corpus, cudaStream_t s);
cudaError_t rs_unadapt(const uint8_t* target, int w, int h, int bpp, uint8_t* img, size_t imgRow, cudaStream_t s);
// The directional and brushfire visit orders (matchContextType 2..8) on the
// device, from the row-major target list: begin (bounding box; brushfire:
// rays, listing as (index, dx, dy) the targets whose ray the host must
// recompute), rays (brushfire: the host's rays for those as (index, ray)
// pairs, the largest |q|^2 per ray, the NaN flag), finish (keys, stable radix
// sort, banded-shuffle permutation `perm` from the host).  work:
// rs_order_ints(n) ints.
size_t rs_order_ints(int n);
cudaError_t rs_order_begin(int type, const int2* targets, int n, int* work, int* flagCount, int* flags, int cap,
                           cudaStream_t s);
cudaError_t rs_order_rays(const int2* targets, int n, int* work, const int* fix, int nfix, cudaStream_t s);
int* rs_order_nan_flag(int* work, int n);
cudaError_t rs_order_finish(int type, const int2* targets, int n, int* work, const int* perm, int2* out,
                            cudaStream_t s);
cudaError_t rs_vis_init(const uint8_t* has, int npx, int* vis, cudaStream_t s);
cudaError_t rs_vis_to_has(const int* vis, int npx, uint8_t* has, cudaStream_t s);
cudaError_t rs_cell_min(const int* vis, int tw, int th, int* cellMin, cudaStream_t s);
cudaError_t rs_launch_patches(const rs::Problem& pb, const int2* targets, int n, int visCur, int useGrid, int* outOff,
                              int* outCount, cudaStream_t s);
}

// Proposal network (proposal_net.cu).
struct TResynthNet;
struct TResynthPairs;
extern "C" {
cudaError_t rs_net_propose(const TResynthNet* net, const rs::Problem& pb, const int2* targets, const int* batchStart,
                           int batch0, int batch1, int count, int visCur, int2* props, unsigned* err, cudaStream_t s);
cudaError_t rs_net_dump(TResynthPairs* pairs, const rs::Problem& pb, const int2* targets, int ntargets, unsigned stride,
                        cudaStream_t s);
}
