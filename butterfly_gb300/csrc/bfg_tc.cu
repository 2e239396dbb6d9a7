// Split-BF16 apply of butterfly factors on the 5th-generation tensor cores
// (tcgen05.mma, accumulator in tensor memory, operands staged by the bulk
// copy engine).  This is the GB300 form of the reference's per-block
// cblas_zgemm (mat_dense_complex.c:1705-1766) for the FP32-vector precisions:
// the stored blocks are split into TERMS bf16 planes (hi, lo[, lo2]) once,
// each right-hand side is split the same way as it is staged, and the complex
// product is formed from real bf16 MMAs with FP32 accumulation.
//
// Complex -> real mapping for a tile of RT right-hand sides:
//   A_real (128 rows x 2n) : row m = Re a_m0, Im a_m0, Re a_m1, Im a_m1, ...
//   B      (2n x 2 RT)     : rows 2j, 2j+1 of column q    = ( Re x_jq, -Im x_jq)
//                            rows 2j, 2j+1 of column RT+q = ( Im x_jq,  Re x_jq)
//   D = A_real B           : column q = Re y_q, column RT+q = Im y_q
// so the stored block needs no duplication and the output lands in TMEM as
// one row per lane.
//
// Products kept: TERMS = 2 -> hh + hl + lh (bf16x2, ~16 significant bits);
// TERMS = 3 -> additionally h l2 + l l + l2 h (bf16x3, ~24 bits, FP32-like).
// Two tile widths: RT = 16 (up to 16 RHS) and RT = 32 (more RHS: half the
// chunk passes per right-hand side, with MMAs of N = 128).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "bfg_kernels.cuh"

namespace bfg {
namespace {

// even: stage s then only ever holds chunks of one parity, so each stage's
// barriers are waited on by one MMA thread, in order (an mbarrier parity wait
// must not run more than one phase ahead of the barrier)
constexpr int kTcStages = 4;
constexpr int kAPlaneBytes = 64 * 128;     // at most 64 core matrices per plane
constexpr uint64_t kWaitLimitNs = 1000000000ull;                          // 1 s

constexpr int32_t kTcBulkX = 1, kTcBulkW = 2;   // inputs / intermediates by bulk copy

template <int TERMS, int RT>
struct TcLayout {
  static_assert(RT == 16 || RT == 32, "RHS tile");
  static constexpr int kN = 2 * RT;        // D columns of one product group
  // B planes interleaved by k-group: k-group g holds plane 0's kN / 8
  // n-groups, then plane 1's, ... so that planes u .. TERMS-1 form one
  // N = kN (TERMS-u) operand; bytes of one plane and of one k-group:
  static constexpr int kBPlaneKGroupBytes = (kN / 8) * 128;
  static constexpr int kBKGroupBytes = TERMS * kBPlaneKGroupBytes;
  // product groups in TMEM per accumulator chain: unfolded (RT = 16), one
  // group per B plane (one MMA per A plane and k-step, N = 32 TERMS ... 32);
  // folded (RT = 32), the products with B planes 1 and 2 share one group
  // (N <= 128)
  static constexpr bool kFold = RT == 32;
  static constexpr int kGroups = kFold ? 2 : TERMS;
  static_assert(kGroups * kN <= 128, "TMEM columns of one chain");
  // TMEM: kNB accumulator buffers (chunk i uses buffer i % kNB) of kNC
  // k-step chains (k-step st adds to chain st % kNC), 128 columns each;
  // buffer b chain c at column 128 (b + kNB c).  RT = 32: four buffers of
  // one chain (two buffers of two chains: 7 % slower at 256 RHS, error
  // 4.1e-7 instead of 6.2e-7 at 65,536 points)
  static constexpr int kNB = RT == 32 ? 4 : 2, kNC = RT == 32 ? 1 : 2;
  static_assert(kNB * kNC * 128 <= 512, "TMEM columns");
  static constexpr int kXStageBytes = kTcChunkCols * RT * 8;
  // warp roles: builders (B planes), extractors (TMEM partial sums and
  // stores; 16 RHS of one TMEM lane quarter each), one bulk-copy warp and
  // the two MMA warps (the even and the odd chunks: one thread's waits and
  // descriptor work overlap the other's MMAs).  RT = 16: 4 + 4 + 1 + 2
  // warps; RT = 32: 4 + 8 + 1 + 2 warps (the extractors' accumulators of 32
  // RHS would not fit one thread's registers; measured at 256 RHS, two
  // builder warps were 12 % and one MMA warp 7 % slower)
  static constexpr int kBuilders = 128;
  static constexpr int kExtractors = RT == 16 ? 128 : 256;
  static constexpr int kMmaWarps = 2;
  static constexpr int kProducerWarp = (kBuilders + kExtractors) / 32;
  static constexpr int kMmaWarp = kProducerWarp + 1;
  static constexpr int kThreads = kBuilders + kExtractors + 32 * (1 + kMmaWarps);
  static constexpr int aBytes = TERMS * kAPlaneBytes;
  static constexpr int bBytes = (kTcChunkCols / 4) * kBKGroupBytes;
  // A planes, B planes, then the chunk's FP32 right-hand sides
  static constexpr int stageBytes = aBytes + bBytes + kXStageBytes;
  // an A descriptor spans 16 row groups and the last k-step reads up to 2 KB
  // past a short tile (rows whose outputs are discarded): 2 KB of slack
  // follow the last stage
  static constexpr int barOff = kTcStages * stageBytes + 2048;
  // fullA[S], fullB[S], empty[S], accFull[kNB], accEmpty[kNB], fullX[S],
  // TMEM slot, abort
  static constexpr int smemBytes = barOff + 8 * (4 * kTcStages + 2 * kNB) + 16;
  static_assert(smemBytes <= 232448, "shared memory per CTA");
  static_assert(kTcStages % 2 == 0, "stages must hold one chunk parity each");
};

// instruction descriptor: D f32, A and B bf16, both K-major, M = m, N = n.
// D row r lands in TMEM lane r for M = 128, and in lane 32 (r / 16) + r % 16
// for M = 64 (16 rows in each warp's lane quarter).  An MMA costs at least
// ~44 cycles whatever its size and M = 64 takes as long as M = 128, but it
// reads half the A bytes from shared memory, which bounds this kernel: items
// of at most 64 rows use M = 64.
__host__ __device__ constexpr uint32_t idesc(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ uint32_t smemAddr(void const *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// shared-memory matrix descriptor, no swizzle: core matrices of 8 rows x 16 B;
// lbo = bytes between K-adjacent cores, sbo = bytes between M/N-adjacent cores
__device__ __forceinline__ uint64_t smemDesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

__device__ __forceinline__ void mbarInit(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void fenceMbarInit() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbarExpectTx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbarTryWait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// the same test, letting the hardware suspend the thread for up to 2 us
// while the phase is incomplete (it resumes as soon as the phase completes)
__device__ __forceinline__ bool mbarTryWaitSuspend(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity), "n"(2000)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ uint64_t globalTimerNs() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// waits for the phase with the given parity; false after limitNs (the
// launch's wait limit, kWaitLimitNs unless a test lowers it) or as soon as
// another role of the CTA has given up (*abort set)
__device__ bool mbarWait(uint32_t bar, uint32_t parity, int volatile *abort, uint64_t limitNs) {
  // a zero limit (the test hook) gives up at once, as a wait on a phase that
  // never completes gives up once the limit has passed
  if (limitNs == 0) return false;
  if (mbarTryWait(bar, parity)) return true;
  uint64_t const t0 = globalTimerNs();
  for (;;) {
    // the abort flag and the clock are read every 8 suspended tests, not
    // every test: polling warps take fewer issue slots from working ones
#pragma unroll 1
    for (int k = 0; k < 8; ++k)
      if (mbarTryWaitSuspend(bar, parity)) return true;
    if (*abort || globalTimerNs() - t0 > limitNs) return false;
  }
}
// the same wait without the early exit (draining work in flight)
__device__ void mbarDrain(uint32_t bar, uint32_t parity) {
  uint64_t const t0 = globalTimerNs();
  while (!mbarTryWait(bar, parity))
    if (globalTimerNs() - t0 > kWaitLimitNs) return;
}
__device__ __forceinline__ void cpAsync8(uint32_t dst, float2 const *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cpAsyncCommit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cpAsyncWait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
__device__ __forceinline__ void mbarArrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void bulkG2S(uint32_t dst, void const *src, uint32_t bytes,
                                        uint32_t bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
      ::"r"(dst), "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void fenceProxyAsync() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// the whole tensor memory (one CTA per SM): the accumulator buffers and
// k-step chains of TcLayout, 128 columns each
__device__ __forceinline__ void tmemAlloc512(uint32_t slot) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(slot)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmemDealloc512(uint32_t taddr) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(taddr) : "memory");
}
__device__ __forceinline__ void tcFenceBefore() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tcFenceAfter() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tcMma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc,
                                      uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
      ::"r"(d), "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void tcCommit(uint32_t bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
      : "memory");
}
// v = t[0] + t[1] + ... with each t[i] the bf16 rounding of what is left
template <int TERMS>
__device__ __forceinline__ void splitD(double v, __nv_bfloat16 (&t)[TERMS]) {
  double r = v;
#pragma unroll
  for (int i = 0; i < TERMS; ++i) {
    t[i] = __double2bfloat16(r);
    r -= (double)__bfloat162float(t[i]);
  }
}
// (lo, hi) rounded to a bf16 pair, lo in the low half
__device__ __forceinline__ uint32_t cvtPack(float lo, float hi) {
  uint32_t r;
  asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
  return r;
}
// (re, im) = sum over t of the bf16 pairs p[t], each the rounding of what is left
template <int TERMS>
__device__ __forceinline__ void splitPair(float re, float im, uint32_t (&p)[TERMS]) {
#pragma unroll
  for (int t = 0; t < TERMS; ++t) {
    p[t] = cvtPack(re, im);
    re -= __uint_as_float(p[t] << 16);
    im -= __uint_as_float(p[t] & 0xFFFF0000u);
  }
}
// 8 consecutive FP32 columns of this thread's TMEM lane (no wait)
__device__ __forceinline__ void tmemLoad8(uint32_t taddr, float *v) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
                 "=r"(r[6]), "=r"(r[7])
               : "r"(taddr)
               : "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}
// 16 consecutive FP32 columns of this thread's TMEM lane (no wait)
__device__ __forceinline__ void tmemLoad16(uint32_t taddr, float *v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
      "%11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
// (a.x + b.x, a.y + b.y), both rounded to nearest: one packed FP32 add
__device__ __forceinline__ float2 add2(float2 a, float2 b) {
  uint64_t ra, rb, r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(ra) : "f"(a.x), "f"(a.y));
  asm("mov.b64 %0, {%1, %2};" : "=l"(rb) : "f"(b.x), "f"(b.y));
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(ra), "l"(rb));
  float2 o;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(o.x), "=f"(o.y) : "l"(r));
  return o;
}
__device__ __forceinline__ void tmemWaitLoads() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ uint32_t pack2(__nv_bfloat16 lo, __nv_bfloat16 hi) {
  return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

// FP64 arena -> bf16 planes of every chunk tile (one CTA per chunk, strided)
template <int TERMS>
__global__ void __launch_bounds__(256) tcFillKernel(TcFill const *__restrict__ fills,
                                                    int64_t nFills,
                                                    double2 const *__restrict__ arena,
                                                    uint8_t *__restrict__ tarena) {
  for (int64_t f = blockIdx.x; f < nFills; f += gridDim.x) {
    TcFill const d = fills[f];
    int const r8 = d.mg * 8, j4 = d.kg * 4;
    int64_t const plane = (int64_t)d.kg * d.mg * 128;
    for (int e = threadIdx.x; e < r8 * j4; e += blockDim.x) {
      int const m = e % r8, j = e / r8;
      double2 v = make_double2(0.0, 0.0);
      if (m < d.rows && j < d.nc) v = arena[d.srcOff + (int64_t)j * d.lda + m];
      __nv_bfloat16 re[TERMS], im[TERMS];
      splitD<TERMS>(v.x, re);
      splitD<TERMS>(v.y, im);
      int64_t const off =
          d.tileOff + ((int64_t)(j >> 2) * d.mg + (m >> 3)) * 128 + (m & 7) * 16 + (j & 3) * 4;
#pragma unroll
      for (int t = 0; t < TERMS; ++t)
        *reinterpret_cast<uint32_t *>(tarena + off + t * plane) = pack2(re[t], im[t]);
    }
  }
}

// Persistent CTA over its chunk stream (one apply stage, one tile of RT RHS),
// warp-specialised around mbarriers (warp numbers for RT = 16; TcLayout
// gives both layouts):
//   warp 8           once the MMAs of chunk i-4 are done (empty) bulk-copies
//                    chunk i's FP32 right-hand-side rows when they form one
//                    aligned block (fullX), then its A planes into stage
//                    i % 4 (fullA);
//   warps 0-3        otherwise copy chunk i+2's right-hand sides into its
//                    stage (cp.async); build chunk i's bf16 B planes (fullB);
//   warps 9, 10      (lane 0) issue the MMAs of the even and the odd chunks,
//                    chunk i into TMEM buffer i % kNB, once its A and B
//                    planes have landed and the buffer was read;
//   warps 4-7        read each chunk's partial sums from TMEM (accFull) into
//                    FP32 registers, release the buffer (accEmpty) and store
//                    finished items.
// Each chunk starts its TMEM buffer from zero and deals its k-steps to the
// buffer's kNC accumulator chains, so the tensor cores accumulate only a
// few k-steps before the sums move to FP32 registers (the tensor-core FP32
// accumulation loses accuracy over long chains).
// Every wait is bounded (kWaitLimitNs) and gives up when another role has;
// the CTA then waits (bounded) for the copies and MMAs it has in flight,
// frees its TMEM and reports kStatusTcTimeout.
template <int TERMS, int RT>
__global__ void __launch_bounds__(TcLayout<TERMS, RT>::kThreads, 1) applyTcKernel(
    TcChunk const *__restrict__ chunks, int64_t const *__restrict__ ctaChunk0,
    uint8_t const *__restrict__ tarena, float2 const *__restrict__ X, int64_t ldx, int64_t xTs,
    float2 *__restrict__ W, int64_t ldw, int64_t wTs, int64_t R, int32_t rhsTiles, int32_t xBulk,
    uint64_t waitLimitNs, int32_t *status) {
  using L = TcLayout<TERMS, RT>;
  constexpr int kN = L::kN;
  constexpr int kBuilders = L::kBuilders, kExtractors = L::kExtractors;
  constexpr int kProducerWarp = L::kProducerWarp, kMmaWarp = L::kMmaWarp;
  constexpr int kMmaWarps = L::kMmaWarps;
  constexpr int S = kTcStages;
  constexpr int kBKGroupBytes = L::kBKGroupBytes;
  extern __shared__ __align__(1024) uint8_t smem[];
  int const tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // CTA = (chunk stream, RHS tile), the tile varying fastest: the tiles of a
  // stream run side by side and read each A chunk from HBM once, the other
  // tiles finding it in L2
  int const stream = (int)(blockIdx.x / (unsigned)rhsTiles);
  int const tile = (int)(blockIdx.x % (unsigned)rhsTiles);
  int64_t const c0 = ctaChunk0[stream];
  int64_t const nCh = ctaChunk0[stream + 1] - c0;
  if (nCh <= 0) return;
  int64_t const r0 = (int64_t)tile * RT;
  int const nr = (R - r0) < RT ? (int)(R - r0) : RT;
  // this tile's right-hand sides: row i at Xt + i ldx (inputs), Wt + i ldw
  // (intermediates and outputs); the tile stride is RT for row-major
  // operands and rows x RT for tile-major ones
  float2 const *__restrict__ Xt = X + tile * xTs;
  float2 *__restrict__ Wt = W + tile * wTs;
  TcChunk const *ch = chunks + c0;
  // a chunk's right-hand sides arrive by one bulk copy with its A planes when
  // they form a contiguous 16-byte aligned block (a full tile of RT RHS,
  // leading dimension RT), else by the builders' cp.async (one copy per
  // 128 B row was slower: the copy engine takes small copies one at a time)
  bool const bulkX = nr == RT && (xBulk & kTcBulkX);
  bool const bulkW = nr == RT && (xBulk & kTcBulkW);

  uint32_t const sbase = smemAddr(smem);
  uint32_t const fullA = sbase + L::barOff, fullB = fullA + 8 * S, empty = fullB + 8 * S;
  constexpr int NB = L::kNB, NC = L::kNC;
  uint32_t const accFull = empty + 8 * S, accEmpty = accFull + 8 * NB;
  uint32_t const fullX = accEmpty + 8 * NB;
  uint32_t *tmemSlot = reinterpret_cast<uint32_t *>(smem + L::barOff + 8 * (4 * S + 2 * NB));
  int volatile *abortFlag = reinterpret_cast<int volatile *>(tmemSlot + 1);

  if (tid == 0) {
    for (int s = 0; s < S; ++s) {
      mbarInit(fullA + 8 * s, 1);
      mbarInit(fullX + 8 * s, 1);
      mbarInit(fullB + 8 * s, kBuilders / 32);
      mbarInit(empty + 8 * s, 1);
    }
    for (int b = 0; b < NB; ++b) {
      mbarInit(accFull + 8 * b, 1);
      mbarInit(accEmpty + 8 * b, kExtractors / 32);
    }
    *abortFlag = 0;
    fenceMbarInit();
  }
  if (warp == kMmaWarp) tmemAlloc512(smemAddr(tmemSlot));
  tcFenceBefore();
  __syncthreads();
  tcFenceAfter();
  uint32_t const tmem = *tmemSlot;

  // what each role has in flight, for the drains after an abort: the
  // producer's issued bulk copies, each MMA thread's last committed chunk
  int64_t issued = 0, lastMma = -1;
  if (warp == kProducerWarp) {
    // ---- bulk copies of the A planes and of the input rows (lane 0) ----
    // descriptors are read one chunk ahead, off the wait-issue path
    TcChunk const *cp = ch;
    int64_t off = cp->tileOff, inRow = cp->inRow;
    uint32_t plane = (uint32_t)cp->kg * cp->mg * 128;
    int32_t nc = cp->nc, inIsX = cp->inIsX;
    for (int64_t i = 0; i < nCh; ++i) {
      int const s = (int)(i % S);
      int64_t offN = 0, inRowN = 0;
      uint32_t planeN = 0;
      int32_t ncN = 0, inIsXN = 0;
      if (i + 1 < nCh) {
        offN = ch[i + 1].tileOff;
        inRowN = ch[i + 1].inRow;
        planeN = (uint32_t)ch[i + 1].kg * ch[i + 1].mg * 128;
        ncN = ch[i + 1].nc;
        inIsXN = ch[i + 1].inIsX;
      }
      int ok = 1;
      if (i >= S && lane == 0) ok = mbarWait(empty + 8 * s, (uint32_t)((i / S - 1) & 1), abortFlag, waitLimitNs);
      if (!__shfl_sync(0xffffffffu, ok, 0)) {
        if (lane == 0) *abortFlag = 1;
        break;
      }
      bool const bulk = inIsX ? bulkX : bulkW;
      if (lane == 0) {
        // the input rows first, on their own barrier (every chunk arrives on
        // it, with no bytes on the cp.async path, so its phases follow the
        // chunks): the builders convert them while the A planes stream in
        mbarExpectTx(fullX + 8 * s, bulk ? (uint32_t)nc * (RT * 8) : 0u);
        // the chunk's input rows are one contiguous block (leading dimension RT)
        if (bulk)
          bulkG2S(sbase + s * L::stageBytes + L::aBytes + L::bBytes,
                  (inIsX ? Xt : Wt) + inRow * RT, (uint32_t)nc * (RT * 8), fullX + 8 * s);
        mbarExpectTx(fullA + 8 * s, plane * TERMS);
#pragma unroll
        for (int t = 0; t < TERMS; ++t)
          bulkG2S(sbase + s * L::stageBytes + t * kAPlaneBytes, tarena + off + (int64_t)t * plane,
                  plane, fullA + 8 * s);
      }
      __syncwarp();
      issued = i + 1;
      off = offN;
      inRow = inRowN;
      plane = planeN;
      nc = ncN;
      inIsX = inIsXN;
    }
  } else if (warp >= kMmaWarp) {
    // ---- MMAs: with two MMA warps, warp kMmaWarp issues the even chunks and
    // the next warp the odd ones, so one thread's waits and bookkeeping
    // overlap the other's MMAs in the tensor pipe; chunk i uses TMEM buffer
    // i % kNB ----
    int const parity = warp - kMmaWarp;
    if (lane == 0 && parity < nCh) {

      int32_t kg = ch[parity].kg, mg = ch[parity].mg;
      for (int64_t i = parity; i < nCh; i += kMmaWarps) {
        int const s = (int)(i % S), b = (int)(i % NB);
        uint32_t const ph = (uint32_t)((i / S) & 1);
        int32_t kgN = 0, mgN = 0;
        if (i + kMmaWarps < nCh) {
          kgN = ch[i + kMmaWarps].kg;
          mgN = ch[i + kMmaWarps].mg;
        }
        if (!mbarWait(fullA + 8 * s, ph, abortFlag, waitLimitNs) || !mbarWait(fullB + 8 * s, ph, abortFlag, waitLimitNs) ||
            (i >= NB && !mbarWait(accEmpty + 8 * b, (uint32_t)((i / NB - 1) & 1), abortFlag, waitLimitNs))) {
          *abortFlag = 1;
          break;
        }
        tcFenceAfter();
        uint32_t const aS = sbase + s * L::stageBytes, bS = aS + L::aBytes;
        uint32_t const lboA = (uint32_t)mg * 128;
        int const ksteps = (kg + 1) >> 1;
        int const mRows = mg <= 8 ? 64 : 128;
        // The descriptors of k-step st are those of k-step 0 with the start
        // address advanced (the address field is the low 14 bits, in 16 B).
        uint64_t da[TERMS];
#pragma unroll
        for (int t = 0; t < TERMS; ++t) da[t] = smemDesc(aS + t * kAPlaneBytes, lboA, 128);
        uint64_t db = smemDesc(bS, kBKGroupBytes, 128);
        uint64_t const stepA = (2 * lboA) >> 4, stepB = (2 * kBKGroupBytes) >> 4;
        // B plane u of the k-group, as a descriptor offset
        constexpr uint64_t kBPlane = (uint64_t)L::kBPlaneKGroupBytes >> 4;
        uint32_t const d = tmem + 128 * b;
#pragma unroll
        for (int st = 0; st < kTcChunkCols / 8; ++st) {
          if (st >= ksteps) break;
          uint32_t const dc = d + 128 * NB * (st % NC);   // the k-step's chain
          uint32_t const acc0 = st >= NC ? 1u : 0u;       // a chain's first k-step overwrites
          if constexpr (!L::kFold) {
            // A plane t times the B planes 0 .. TERMS-1-t, side by side in
            // N: D columns 32 u .. 32 u + 31 collect the products with B
            // plane u
#pragma unroll
            for (int t = 0; t < TERMS; ++t)
              tcMma(dc, da[t], db, idesc(mRows, kN * (TERMS - t)), (acc0 || t > 0) ? 1u : 0u);
          } else if constexpr (TERMS == 3) {
            // group 0 (columns 0 .. kN-1) collects the products with B plane
            // 0, group 1 those with B planes 1 and 2 (hm + mm + hl); the
            // smallest products go first, hh last
            tcMma(dc, da[1], db, idesc(mRows, 2 * kN), acc0);             // m x (h | m)
            tcMma(dc, da[2], db, idesc(mRows, kN), 1u);                   // l x h
            tcMma(dc + kN, da[0], db + 2 * kBPlane, idesc(mRows, kN), 1u);  // h x l
            tcMma(dc, da[0], db, idesc(mRows, 2 * kN), 1u);               // h x (h | m)
          } else {
            tcMma(dc, da[0], db, idesc(mRows, 2 * kN), acc0);             // h x (h | l)
            tcMma(dc, da[1], db, idesc(mRows, kN), 1u);                   // l x h
          }
#pragma unroll
          for (int t = 0; t < TERMS; ++t) da[t] += stepA;
          db += stepB;
        }
        tcCommit(empty + 8 * s);
        tcCommit(accFull + 8 * b);
        lastMma = i;
        kg = kgN;
        mg = mgN;
      }
    }
  } else {
    struct Cd {            // builders: inputs of a chunk
      int64_t inRow;
      int32_t nc, kg, mg, inIsX;
    };
    auto loadCd = [&](int64_t i) {
      Cd d{};
      if (i < nCh) {
        TcChunk const &k = ch[i];
        d = Cd{k.inRow, k.nc, k.kg, k.mg, k.inIsX};
      }
      return d;
    };
    struct Ce {            // extractors: outputs of a chunk
      int64_t outRow;
      int32_t rows, kg, flags;
    };
    auto loadCe = [&](int64_t i) {
      Ce d{};
      if (i < nCh) {
        TcChunk const &k = ch[i];
        d = Ce{k.outRow, k.rows, k.kg, k.flags};
      }
      return d;
    };
    if (tid < kBuilders) {
      // ---- B planes ----
      // A builder converts columns j0 .. j0+3 (j0 = 4 jg: one k-group) of RHS
      // q = tid % RT, jg = tid / RT + kJgPass p for passes p: the four
      // complex values fill one 16 B core-matrix row of each B plane, and a
      // warp's stores cover 512 contiguous-in-banks bytes.  On the cp.async
      // path the thread that copies an element into the X stage is the one
      // that converts it, so the cp.async groups need no barrier.
      // Descriptors are loaded one iteration before their first use.
      constexpr int kJgPass = kBuilders / RT;               // k-groups per pass
      constexpr int kPasses = (kTcChunkCols / 4) / kJgPass;
      static_assert(kPasses * kJgPass == kTcChunkCols / 4, "builder passes");
      int const q = tid % RT, jgBase = tid / RT;
      auto issueX = [&](Cd const &d, int64_t i) {
        int64_t const xld = d.inIsX ? ldx : ldw;
        float2 const *src = (d.inIsX ? Xt : Wt) + d.inRow * xld + q;
        uint32_t const xs = sbase + (int)(i % S) * L::stageBytes + L::aBytes + L::bBytes;
        if (q < nr)
#pragma unroll
          for (int p = 0; p < kPasses; ++p)
#pragma unroll
            for (int u = 0; u < 4; ++u) {
              int const j = 4 * (jgBase + kJgPass * p) + u;
              if (j < d.nc) cpAsync8(xs + (uint32_t)(j * RT + q) * 8, src + (int64_t)j * xld);
            }
      };
      auto bulkOf = [&](Cd const &d) { return d.inIsX ? bulkX : bulkW; };
      Cd d0 = loadCd(0), d1 = loadCd(1), d2 = loadCd(2);
      // inputs of chunks 0 and 1 in flight before the loop (two cp.async groups)
      if (0 < nCh && !bulkOf(d0)) issueX(d0, 0);
      cpAsyncCommit();
      if (1 < nCh && !bulkOf(d1)) issueX(d1, 1);
      cpAsyncCommit();
      for (int64_t i = 0; i < nCh; ++i) {
        int const s = (int)(i % S);
        Cd const d3 = loadCd(i + 3);   // used from the next iteration on
        // inputs of chunk i+2 into its stage: that stage's X area last held
        // chunk i+2-S, which this thread has converted
        if (i + 2 < nCh && !bulkOf(d2)) issueX(d2, i + 2);
        cpAsyncCommit();
        // bulk inputs land on fullX, which the producer arrives on only once
        // the MMAs of chunk i-S are done; the empty wait then returns at once.
        // A warp gives up as one (a vote): were a phase to complete while
        // the abort flag is being set, some lanes could pass the wait and
        // others leave the loop, and the passing lanes' __syncwarp would
        // then wait forever for lanes already at the final barrier.
        if (bulkOf(d0) &&
            !__all_sync(0xffffffffu, mbarWait(fullX + 8 * s, (uint32_t)((i / S) & 1), abortFlag, waitLimitNs))) {
          *abortFlag = 1;
          break;
        }
        if (i >= S &&
            !__all_sync(0xffffffffu,
                        mbarWait(empty + 8 * s, (uint32_t)((i / S - 1) & 1), abortFlag, waitLimitNs))) {
          *abortFlag = 1;
          break;
        }
        cpAsyncWait<2>();   // this thread's elements of chunk i have landed
        uint8_t *stage = smem + s * L::stageBytes;
        uint8_t *bsm = stage + L::aBytes;
        float2 const *xs = reinterpret_cast<float2 const *>(stage + L::aBytes + L::bBytes);
        int const kgEven = ((d0.kg + 1) >> 1) * 2;   // k-groups the MMAs read
#pragma unroll
        for (int p = 0; p < kPasses; ++p) {
          int const jg = jgBase + kJgPass * p;
          if (jg < kgEven) {
            float2 v[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
              int const j = 4 * jg + u;
              v[u] = (j < d0.nc && q < nr) ? xs[j * RT + q] : make_float2(0.f, 0.f);
            }
            uint32_t pr[4][TERMS];
#pragma unroll
            for (int u = 0; u < 4; ++u) splitPair<TERMS>(v[u].x, v[u].y, pr[u]);
            uint32_t const offRe = (uint32_t)jg * kBKGroupBytes + (q >> 3) * 128 + (q & 7) * 16;
#pragma unroll
            for (int t = 0; t < TERMS; ++t) {
              // rows 2j, 2j+1 of column q: (Re x, -Im x); of column RT+q
              // (RT / 8 core rows further): (Im x, Re x)
              uint8_t *bp = bsm + t * L::kBPlaneKGroupBytes + offRe;
              *reinterpret_cast<uint4 *>(bp) =
                  make_uint4(pr[0][t] ^ 0x80000000u, pr[1][t] ^ 0x80000000u,
                             pr[2][t] ^ 0x80000000u, pr[3][t] ^ 0x80000000u);
              *reinterpret_cast<uint4 *>(bp + (RT / 8) * 128) =
                  make_uint4(__byte_perm(pr[0][t], 0, 0x1032), __byte_perm(pr[1][t], 0, 0x1032),
                             __byte_perm(pr[2][t], 0, 0x1032), __byte_perm(pr[3][t], 0, 0x1032));
            }
          }
        }
        // an odd k-group count leaves the second half of the last k-step unset
        // in A: zero it (B is zero there, but stale shared memory may hold NaNs)
        if (d0.kg & 1) {
          uint32_t const padOff = (uint32_t)d0.kg * d0.mg * 128, padBytes = (uint32_t)d0.mg * 128;
          for (uint32_t e = (uint32_t)tid * 16; e < padBytes; e += kBuilders * 16)
#pragma unroll
            for (int t = 0; t < TERMS; ++t)
              *reinterpret_cast<uint4 *>(stage + t * kAPlaneBytes + padOff + e) =
                  make_uint4(0, 0, 0, 0);
        }
        fenceProxyAsync();
        __syncwarp();
        if (lane == 0) mbarArrive(fullB + 8 * s);
        d0 = d1;
        d1 = d2;
        d2 = d3;
      }
      cpAsyncWait<0>();
    } else {
      // ---- TMEM partial sums, FP32 accumulation, stores ----
      // extractor warp w reads TMEM lane quarter w % 4 (item row
      // 32 (w % 4) + lane) for the 16 RHS 16 h .. 16 h + 15 of the tile,
      // h = (w - first extractor warp) / 4
      int const e = warp & 3;
      int const h = (warp - kBuilders / 32) >> 2;
      float acc[32];   // 16 real parts, then 16 imaginary parts
#pragma unroll
      for (int c = 0; c < 32; ++c) acc[c] = 0.f;
      // TMEM columns per load: 8 for three groups, 16 for two; one wait per
      // part.  Part p covers accumulator slots
      // kLoadW p ..: real parts (columns 16 h + ..) then imaginary parts
      // (columns RT + 16 h + ..)
      constexpr int kLoadW = L::kGroups == 3 ? 8 : 16, kG = L::kGroups;
      Ce dn = loadCe(0);
      for (int64_t j = 0; j < nCh; ++j) {
        Ce const d = dn;
        dn = loadCe(j + 1);
        int const b = (int)(j % NB);
        // as one warp (a vote), for the collective TMEM loads below
        if (!__all_sync(0xffffffffu, mbarWait(accFull + 8 * b, (uint32_t)((j / NB) & 1), abortFlag, waitLimitNs))) {
          *abortFlag = 1;
          break;
        }
        tcFenceAfter();
        uint32_t const tl = tmem + 128 * b + ((uint32_t)(e * 32) << 16);
        int const ksteps = (d.kg + 1) >> 1;
        int const chains = ksteps < NC ? ksteps : NC;   // the chains this chunk wrote
        for (int c = 0; c < chains; ++c) {
#pragma unroll
          for (int part = 0; part < 32 / kLoadW; ++part) {
            int const slot = kLoadW * part;
            uint32_t const col = slot < 16 ? 16 * h + slot : RT + 16 * h + (slot - 16);
            float v[kG][kLoadW];
#pragma unroll
            for (int u = 0; u < kG; ++u) {
              uint32_t const ta = tl + 128 * NB * c + kN * u + col;
              if constexpr (kLoadW == 8)
                tmemLoad8(ta, v[u]);
              else
                tmemLoad16(ta, v[u]);
            }
            tmemWaitLoads();
            // the group of the smaller products first; packed adds, the same
            // roundings as scalar ones
#pragma unroll
            for (int k = 0; k < kLoadW; k += 2) {
              float2 t = make_float2(v[kG - 1][k], v[kG - 1][k + 1]);
#pragma unroll
              for (int u = kG - 2; u >= 0; --u) t = add2(t, make_float2(v[u][k], v[u][k + 1]));
              float2 const a = add2(make_float2(acc[slot + k], acc[slot + k + 1]), t);
              acc[slot + k] = a.x;
              acc[slot + k + 1] = a.y;
            }
          }
        }
        tcFenceBefore();
        __syncwarp();
        if (lane == 0) mbarArrive(accEmpty + 8 * b);
        if (d.flags & kTcLast) {
          // M = 64 chunks (items of <= 64 rows): lanes 16..31 hold no row
          int const row = d.rows <= 64 ? (lane < 16 ? e * 16 + lane : kTcRows) : e * 32 + lane;
          if (row < d.rows) {
            float2 *out = Wt + (d.outRow + row) * ldw + 16 * h;
#pragma unroll
            for (int c = 0; c < 16; ++c)
              if (16 * h + c < nr) out[c] = make_float2(acc[c], acc[16 + c]);
          }
#pragma unroll
          for (int c = 0; c < 32; ++c) acc[c] = 0.f;
        }
      }
    }
  }

  // After an abort, whatever a role still has in flight lands before the CTA
  // frees its tensor memory and shared memory.  The drains come after a
  // barrier: a role that finished its loop may have read the abort flag
  // before another role gave up, and its copies or MMAs could then still be
  // outstanding.  The flag is final here, the same for every thread.
  tcFenceBefore();
  __syncthreads();
  if (*abortFlag) {
    if (warp == kProducerWarp && lane == 0)
      for (int64_t j = issued > S ? issued - S : 0; j < issued; ++j) {
        mbarDrain(fullX + 8 * (j % S), (uint32_t)((j / S) & 1));
        mbarDrain(fullA + 8 * (j % S), (uint32_t)((j / S) & 1));
      }
    if (warp >= kMmaWarp && lane == 0 && lastMma >= 0)
      mbarDrain(empty + 8 * (lastMma % S), (uint32_t)((lastMma / S) & 1));
  }
  tcFenceBefore();
  __syncthreads();
  if (warp == kMmaWarp) {
    __syncwarp();
    tcFenceAfter();
    tmemDealloc512(tmem);
  }
  if (tid == 0 && *abortFlag) atomicOr(status, kStatusTcTimeout);
}

}  // namespace

// the RHS tile of an apply of R right-hand sides
int32_t tcRhsTile(int64_t R) { return R > 16 ? 32 : 16; }

namespace {
template <int TERMS, int RT>
cudaError_t prepareOne(int *per) {
  cudaError_t e = cudaFuncSetAttribute(applyTcKernel<TERMS, RT>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       TcLayout<TERMS, RT>::smemBytes);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per, applyTcKernel<TERMS, RT>,
                                                       TcLayout<TERMS, RT>::kThreads,
                                                       TcLayout<TERMS, RT>::smemBytes);
}
template <int TERMS, int RT>
void launchOne(dim3 grid, cudaStream_t stream, TcChunk const *chunks, int64_t const *ctaChunk0,
               uint8_t const *tarena, float2 const *X, int64_t ldx, int64_t xTs, float2 *W,
               int64_t ldw, int64_t wTs, int64_t R, int32_t tiles, int32_t xBulk,
               uint64_t waitLimitNs, int32_t *status) {
  applyTcKernel<TERMS, RT><<<grid, TcLayout<TERMS, RT>::kThreads, TcLayout<TERMS, RT>::smemBytes,
                             stream>>>(
      chunks, ctaChunk0, tarena, X, ldx, xTs, W, ldw, wTs, R, tiles, xBulk, waitLimitNs, status);
}
}  // namespace

// resident CTAs per SM of every tile width (the smaller count)
cudaError_t tcPrepare(int32_t terms, int32_t *ctasPerSm) {
  int a = 0, b = 0;
  cudaError_t e = terms == 3 ? prepareOne<3, 16>(&a) : prepareOne<2, 16>(&a);
  if (e != cudaSuccess) return e;
  e = terms == 3 ? prepareOne<3, 32>(&b) : prepareOne<2, 32>(&b);
  if (e != cudaSuccess) return e;
  *ctasPerSm = a < b ? a : b;
  return cudaSuccess;
}

cudaError_t launchTcFill(int32_t terms, TcFill const *fills, int64_t nFills,
                         double2 const *arena64, uint8_t *tarena, cudaStream_t stream) {
  if (nFills == 0) return cudaSuccess;
  unsigned const grid = (unsigned)(nFills < 152 * 64 ? nFills : 152 * 64);
  if (terms == 3)
    tcFillKernel<3><<<grid, 256, 0, stream>>>(fills, nFills, arena64, tarena);
  else
    tcFillKernel<2><<<grid, 256, 0, stream>>>(fills, nFills, arena64, tarena);
  return cudaGetLastError();
}

cudaError_t launchApplyTc(int32_t terms, int32_t rt, TcChunk const *chunks,
                          int64_t const *ctaChunk0, int32_t ctas, uint8_t const *tarena,
                          float2 const *X, int64_t ldx, int64_t xTs, float2 *W, int64_t ldw,
                          int64_t wTs, int64_t R, int32_t *status, cudaStream_t stream,
                          uint64_t waitLimitNs) {
  if (rt != 16 && rt != 32) return cudaErrorInvalidValue;
  if (ctas == 0) return cudaSuccess;
  int64_t const tiles = (R + rt - 1) / rt;
  if (tiles > 0x7fffffff / ctas) return cudaErrorInvalidValue;
  // row-major operands hold a tile's RT columns side by side (ld >= R, tile
  // stride RT), tile-major ones one panel per tile (ld = RT, tile stride at
  // least rows x RT); a single tile is row-major
  auto const layoutOk = [&](int64_t ld, int64_t ts) {
    if (tiles == 1) return ld >= R;
    return (ld >= R && ts == rt) || (ld == rt && ts >= rt);
  };
  if (!layoutOk(ldx, xTs) || !layoutOk(ldw, wTs)) return cudaErrorInvalidValue;
  dim3 grid((unsigned)(ctas * tiles));
  // one bulk copy per chunk: RT RHS with leading dimension RT, 16-byte aligned
  int32_t const xBulk =
      ((ldx == rt && (uintptr_t)X % 16 == 0 && xTs % 2 == 0) ? kTcBulkX : 0) |
      ((ldw == rt && (uintptr_t)W % 16 == 0 && wTs % 2 == 0) ? kTcBulkW : 0);
  auto const t32 = (int32_t)tiles;
  if (terms == 3 && rt == 16)
    launchOne<3, 16>(grid, stream, chunks, ctaChunk0, tarena, X, ldx, xTs, W, ldw, wTs, R, t32, xBulk,
                     waitLimitNs, status);
  else if (terms == 3)
    launchOne<3, 32>(grid, stream, chunks, ctaChunk0, tarena, X, ldx, xTs, W, ldw, wTs, R, t32, xBulk,
                     waitLimitNs, status);
  else if (rt == 16)
    launchOne<2, 16>(grid, stream, chunks, ctaChunk0, tarena, X, ldx, xTs, W, ldw, wTs, R, t32, xBulk,
                     waitLimitNs, status);
  else
    launchOne<2, 32>(grid, stream, chunks, ctaChunk0, tarena, X, ldx, xTs, W, ldw, wTs, R, t32, xBulk,
                     waitLimitNs, status);
  return cudaGetLastError();
}

}  // namespace bfg
