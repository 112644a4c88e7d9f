// tc_gemm.cuh -- BF16 GEMM on the sm_103a tensor cores (tcgen05 + TMEM).
//
//   D[M x N] (fp32) = sum over K chunks of  A[M x Kc] . B[N x Kc]^T
//
// A and B are bf16 and K-major.  Operand storage ("blocked"): a tile of Rt
// rows (Rt a multiple of 8) and Kc columns (a multiple of 16) is a run of
// core matrices of 8 rows x 8 bf16 (128 contiguous bytes, row r of the core
// at byte 16 r).  Core (rb, kb) of the tile sits at byte kb * (Rt / 8) * 128 +
// rb * 128: for each 8-column block, all row blocks back to back.  This is
// the no-swizzle K-major layout of the tcgen05 shared-memory descriptor with
// stride-dimension byte offset 128 (between row blocks) and leading-dimension
// byte offset (Rt / 8) * 128 (between column blocks), so one CTA's A tile
// (128 rows) and B tile (NT rows) are each a single bulk copy.
//
// Grid: blockIdx.x = 128-row tile of D, blockIdx.y = NT-column tile of D,
// blockIdx.z = K chunk.  Tile (x, y, z) of A starts at element
// x * aTile + z * aChunk, of B at y * bTile + z * bChunk.
#pragma once

#include <cuda_bf16.h>
#include <cstdint>

namespace rs {
namespace tc {

constexpr int kTileM = 128;
constexpr int kMaxK = 320;   // largest K chunk one CTA stages

struct GemmArgs {
  const uint16_t* A;
  const uint16_t* B;
  long long aTile, aChunk, bTile, bChunk;
  int M, N, K;               // valid rows, valid columns, K of one chunk
  const float* bias;         // per column, or null
  int relu;
  int accumulate;            // atomicAdd the tile into outF (chunked K)
  float* outF;               // row-major, leading dimension ldo, or null
  long long outChunk;        // chunked K without accumulate: chunk z writes outF + z * outChunk
  uint16_t* outH;            // bf16 bits, row-major, leading dimension ldo, or null
  int ldo;
  unsigned* err;             // bit 2: a wait ran out
  unsigned extraTx;          // test only: bytes the load barrier expects beyond the copies (0)
  int waitLimit;             // polls per barrier wait (0 = 2^20)
};

// Offset in elements of (row r, column k) in a blocked tile of Rt rows and Kc columns.
__host__ __device__ inline long long blocked_offset(int r, int k, int Rt) {
  return (long long)(k >> 3) * (Rt >> 3) * 64 + (r >> 3) * 64 + (r & 7) * 8 + (k & 7);
}

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// tcgen05 shared-memory matrix descriptor, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;   // descriptor version of tcgen05
  return d;                 // base offset 0, relative LBO, layout type 0 (no swizzle)
}

// Instruction descriptor of kind::f16: D fp32, A and B bf16, both K-major, dense.
__host__ __device__ constexpr uint32_t instr_desc(int m, int n) {
  return (1u << 4)                        // D format: f32
         | (1u << 7)                      // A format: bf16
         | (1u << 10)                     // B format: bf16
         | ((uint32_t)(n >> 3) << 17)     // N / 8
         | ((uint32_t)(m >> 4) << 24);    // M / 16
}

__device__ __forceinline__ void mbar_init1(uint64_t* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(saddr(bar)));
}

// Bounded wait on an mbarrier phase; false when the limit ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t phase, int limit) {
  for (int it = 0; it < limit; it++) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(saddr(bar)), "r"(phase)
        : "memory");
    if (ok) return true;
    if (it > 64) __nanosleep(64);
  }
  return false;
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   saddr(dst)),
               "l"(src), "r"(bytes), "r"(saddr(bar))
               : "memory");
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
      "l"(da), "l"(db), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(saddr(bar))
               : "memory");
}

// 32 consecutive fp32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&v)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
        "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
        "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
        "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

template <int COLS>
__device__ __forceinline__ void tmem_alloc(uint32_t* dst) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(dst)), "r"(COLS));
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}

template <int COLS>
__device__ __forceinline__ void tmem_free(uint32_t tmem) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(COLS));
}

// Dynamic shared memory one CTA of k_gemm<NT> needs for chunk size K.
inline size_t gemm_smem_bytes(int NT, int K) { return (size_t)(kTileM + NT) * K * 2; }

// One CTA of 128 threads computes one 128 x NT tile of D for one K chunk.
template <int NT>
__global__ void __launch_bounds__(128, 1) k_gemm(GemmArgs g) {
  static_assert(NT % 32 == 0 && NT >= 32 && NT <= 256, "tile N");
  constexpr int kCols = NT <= 32 ? 32 : NT <= 64 ? 64 : NT <= 128 ? 128 : 256;
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ __align__(8) uint64_t barLoad, barMma;
  __shared__ uint32_t tmemBase;
  const int K = g.K;
  uint16_t* sA = reinterpret_cast<uint16_t*>(sm);
  uint16_t* sB = reinterpret_cast<uint16_t*>(sm + (size_t)kTileM * K * 2);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    mbar_init1(&barLoad);
    mbar_init1(&barMma);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) tmem_alloc<kCols>(&tmemBase);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmemBase;
  const uint32_t bytesA = (uint32_t)kTileM * K * 2, bytesB = (uint32_t)NT * K * 2;
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(&barLoad)),
                 "r"(bytesA + bytesB + g.extraTx)
                 : "memory");
    bulk_g2s(sA, g.A + blockIdx.x * g.aTile + blockIdx.z * g.aChunk, bytesA, &barLoad);
    bulk_g2s(sB, g.B + blockIdx.y * g.bTile + blockIdx.z * g.bChunk, bytesB, &barLoad);
  }
  // A failed load wait leaves the copies possibly in flight: the second wait
  // below gives them the same bound again before the CTA leaves.
  const int limit = g.waitLimit > 0 ? g.waitLimit : 1 << 20;
  bool ok = mbar_wait(&barLoad, 0, limit);
  ok = __syncthreads_and(ok) != 0;
  if (ok && threadIdx.x == 0) {
    const uint32_t idesc = instr_desc(kTileM, NT);
    const uint32_t lboA = (kTileM / 8) * 128, lboB = (NT / 8) * 128;
    for (int ks = 0; ks < K / 16; ks++) {   // one K step = two 8-column blocks
      const uint64_t da = smem_desc(saddr(sA) + 2 * ks * lboA, lboA, 128);
      const uint64_t db = smem_desc(saddr(sB) + 2 * ks * lboB, lboB, 128);
      mma_bf16(tmem, da, db, idesc, ks > 0 ? 1u : 0u);
    }
    mma_commit(&barMma);
  }
  bool done = ok ? mbar_wait(&barMma, 0, limit) : (mbar_wait(&barLoad, 0, limit), false);
  done = __syncthreads_and(done) != 0;
  if (!done && threadIdx.x == 0) atomicOr(g.err, 4u);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (done) {
    const int row = blockIdx.x * kTileM + warp * 32 + lane;
    float* outF = g.outF ? g.outF + blockIdx.z * g.outChunk : nullptr;
#pragma unroll 1
    for (int c0 = 0; c0 < NT; c0 += 32) {
      uint32_t v[32];
      tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
      const int col0 = blockIdx.y * NT + c0;
      if (row < g.M) {
#pragma unroll
        for (int j = 0; j < 32; j++) {
          const int col = col0 + j;
          if (col >= g.N) break;
          float x = __uint_as_float(v[j]);
          const long long o = (long long)row * g.ldo + col;
          if (g.accumulate) {
            atomicAdd(outF + o, x);
            continue;
          }
          if (g.bias) x += g.bias[col];
          if (g.relu) x = fmaxf(x, 0.f);
          if (outF) outF[o] = x;
          if (g.outH) g.outH[o] = __bfloat16_as_ushort(__float2bfloat16_rn(x));
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) tmem_free<kCols>(tmem);
}

}  // namespace tc
}  // namespace rs
