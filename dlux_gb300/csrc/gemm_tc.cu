// gemm_tc.cu -- split-precision complex GEMM on the 5th-generation tensor cores.
//
//   D[b][m][n] = sum_k opA(A[b][m][k]) * B[b][n][k]
//
// Every real operand is stored as two bf16 planes, hi = rn(x) and
// lo = rn(x - hi) (layout [b][4][rows][K]: re_hi, re_lo, im_hi, im_lo), and
// every real product is formed as hi*hi + hi*lo + lo*hi with FP32
// accumulation in tensor memory (the lo*lo term, ~2^-16 relative, is
// dropped). The complex product needs four real products, so one complex
// K-step issues 12 tcgen05.mma instructions; the minus sign of Im*Im (and the
// conjugate of A) is applied with the instruction descriptor's negate-A bit.
//
// Accuracy: each MMA rounds its running FP32 accumulator, so an accumulator
// that absorbs many MMAs of a coherent sum (the bright core of a PSF) drifts
// by about one ulp of the running sum per MMA. The hi*hi products therefore
// go to a "main" accumulator (2 MMAs per complex K-step) and the ~2^-8
// smaller hi*lo + lo*hi cross products to a separate "cross" accumulator (4
// per K-step), whose rounding is 2^-8 smaller; the epilogue adds the two in
// FP32. This keeps the polychromatic PSF within 1e-5 (relative L2) of the FP64
// oracle at 512 x 512 x 512.
//
// CTA tile: 128 complex rows of A x 128 complex rows of B. The tensor core
// accumulates the transposed tile, so TMEM lane i holds output column n0 + i
// and TMEM column j output row m0 + j. The epilogue threads then each drain
// one output column, and the 32 lanes of a warp write 32 consecutive
// elements of a row: every epilogue store and side-input load is one
// contiguous segment. TMEM holds main and cross accumulators for the real and
// imaginary parts (4 x 128 fp32 columns = all 512 columns). K is staged 32
// elements at a time (64-byte rows, 64B swizzle) by TMA in a 3-stage mbarrier
// pipeline (64 KB per stage). Warp roles: warp 0 issues TMA, warp 1 issues
// MMA (one thread each), warps 4-11 drain TMEM through the shared epilogues,
// two warps per TMEM lane quarter taking alternate 32-row chunks, so that the
// epilogue's memory traffic has enough loads in flight. The MMAs of the next
// tile wait for the drain (no TMEM is left for a second accumulator set), so
// the drain must be short: each epilogue warp loads both of its chunks into
// registers and releases TMEM before its stores. The warpgroups split the
// register file unevenly (setmaxnreg): 88 per thread for TMA/MMA, 208 for the
// epilogue, which then holds its 128 drained values without spilling.
// The kernel is persistent over (batch, m-tile, n-tile)
// work items. Every mbarrier wait is bounded by a wall-clock limit; on
// expiry the CTA records DLX_ERR_TIMEOUT in a device status word, drains its
// own in-flight copies and MMAs, frees TMEM and exits.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <atomic>
#include <cstdlib>
#include <mutex>

#include "epilogue.cuh"

namespace dlx {
namespace {

constexpr int TC_BM = 128;
constexpr int TC_BN = 128;
constexpr int TC_BK = 32;
constexpr int TC_STAGES = 3;
constexpr int A_PLANE_BYTES = TC_BM * TC_BK * 2;                         // 8 KB
constexpr int B_PLANE_BYTES = TC_BN * TC_BK * 2;                         // 8 KB
constexpr int STAGE_BYTES = 4 * A_PLANE_BYTES + 4 * B_PLANE_BYTES;       // 64 KB
constexpr int SMEM_BYTES = TC_STAGES * STAGE_BYTES + 1024 + 256;
// 384 threads in three warpgroups. Warpgroup 0: warp 0 issues TMA, warp 1
// MMA, warps 2-3 idle; it gives registers back (setmaxnreg.dec to
// REG_CTRL). Warpgroups 1-2 (warps 4-11) are the 8 epilogue warps, two per
// TMEM lane quarter, raised to REG_EPI registers so that a warp holds both of
// its drained 32-row chunks without spilling.
constexpr int TC_THREADS = 384;
constexpr int TC_EPI_WARPS = 8;
constexpr int TC_EPI_W0 = 4;  // first epilogue warp
constexpr int REG_LAUNCH = 168, REG_CTRL = 88, REG_EPI = 208;
// setmaxnreg.inc waits until the block's launch registers cover the split.
static_assert(128 * REG_CTRL + 256 * REG_EPI <= TC_THREADS * REG_LAUNCH,
              "register split exceeds the launch registers");
static_assert(REG_LAUNCH * TC_THREADS <= 65536, "launch registers exceed the SM");
constexpr uint32_t TMEM_COLS = 512;
// Paired form (cta_group::2, opt-in). A cluster of two CTAs on adjacent
// n-tiles issues M = 256 MMAs from the even CTA: each CTA holds its own 128 B
// rows and half (64) of the A rows, and the tensor cores exchange the A
// halves. Per SM that is 6 KB of operand reads per MMA and 48 KB of fills per
// K block instead of 8 KB and 64 KB, a fourth pipeline stage in the same
// shared memory, and a quarter less L2 traffic. Every output element is formed
// from the same products in the same order, so results are bitwise those of
// the single-CTA form.
constexpr int TP_STAGES = 4;
constexpr int TP_A_PLANE_BYTES = (TC_BM / 2) * TC_BK * 2;                 // 4 KB
constexpr int TP_STAGE_BYTES = 4 * TP_A_PLANE_BYTES + 4 * B_PLANE_BYTES;  // 48 KB
static_assert(TP_STAGES * TP_STAGE_BYTES == TC_STAGES * STAGE_BYTES,
              "both forms use the same shared-memory layout size");
// Wall-clock limit of each mbarrier wait: the default, and the one used while
// draining after an abort (copies and MMAs already issued always complete,
// so the drain keeps the long limit whatever the caller set).
constexpr unsigned long long kTimeoutNs = 2000000000ull;  // 2 s per wait
constexpr unsigned long long kDrainNs = kTimeoutNs;

// ------------------------------- PTX wrappers -------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait. Returns false if another role aborted or the limit expired
// (then the abort flag and the device status word are set). Inlined: a call
// inside a setmaxnreg region makes ptxas run out of memory.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag,
                                       int* status, unsigned long long limit_ns,
                                       bool honour_abort = true) {
  const unsigned long long t0 = globaltimer();
  for (uint32_t it = 0;; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 63u) == 63u) {
      if (honour_abort && *abort_flag) return false;
      if (globaltimer() - t0 > limit_ns) {
        *abort_flag = 1;
        if (status) atomicExch(status, DLX_ERR_TIMEOUT);
        return false;
      }
    }
  }
}

// Warp-uniform bounded wait: lane 0 polls, the outcome is broadcast, so the
// whole warp leaves together (required before .sync.aligned tcgen05 ops).
__device__ __forceinline__ bool warp_wait(uint64_t* bar, uint32_t parity,
                                          volatile int* abort_flag, int* status,
                                          unsigned long long limit_ns) {
  int ok = 0;
  if ((threadIdx.x & 31) == 0) ok = mbar_wait(bar, parity, abort_flag, status, limit_ns) ? 1 : 0;
  ok = __shfl_sync(0xffffffffu, ok, 0);
  return ok != 0;
}

__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar,
                                            int c0, int c1, int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4, %5}], [%2];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2)
      : "memory");
}

// Paired form: the copy lands in this CTA's shared memory and completes on
// the mbarrier at cluster address `bar` (the even CTA's).
__device__ __forceinline__ void tma_load_3d_pair(void* dst, const CUtensorMap* map, uint32_t bar,
                                                 int c0, int c1, int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      ".cta_group::2 [%0], [%1, {%3, %4, %5}], [%2];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(bar), "r"(c0), "r"(c1), "r"(c2)
      : "memory");
}

__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

// Cluster address of the shared variable at the same offset in CTA `rank`.
__device__ __forceinline__ uint32_t cluster_addr(const void* local, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(smem_u32(local)), "r"(rank));
  return r;
}

__device__ __forceinline__ void mbar_arrive_cluster(uint32_t cluster_bar) {
  asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(cluster_bar)
               : "memory");
}

// Every thread of both CTAs.
__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\t"
               "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

__device__ __forceinline__ void prefetch_tmap(const CUtensorMap* map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

// PAIR: the cta_group::2 forms, issued by one warp in each CTA of the pair.
template <bool PAIR = false>
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  if constexpr (PAIR) {
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
  } else {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
}

template <bool PAIR = false>
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  if constexpr (PAIR)
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
                 : "memory");
  else
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

template <bool PAIR = false>
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc,
                                        uint32_t idesc, uint32_t accumulate) {
  if constexpr (PAIR)
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
  else
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

// Paired form: arrive on the mbarrier at this offset in every CTA of `mask`
// once the pair's MMAs issued so far have completed.
__device__ __forceinline__ void mma_commit_pair(uint64_t* bar, uint16_t mask) {
  asm volatile(
      "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64"
      " [%0], %1;" ::"r"(smem_u32(bar)),
      "h"(mask)
      : "memory");
}

// 32 lanes x 32 consecutive 32-bit TMEM columns -> 32 registers per thread.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* out) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) out[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_ld_wait();

// 32 lanes x 16 consecutive 32-bit TMEM columns -> 16 registers per thread.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* out) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) out[i] = __uint_as_float(r[i]);
}

// main + cross accumulators of 32 output rows starting at TMEM column `col`,
// loaded 16 columns at a time so that only 16 temporaries are live.
__device__ __forceinline__ void tmem_sum32(uint32_t lane_addr, uint32_t col, uint32_t cross_off,
                                           float* out) {
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    float t[16];
    tmem_ld16(lane_addr + col + 16 * h, out + 16 * h);
    tmem_ld16(lane_addr + cross_off + col + 16 * h, t);
    tmem_ld_wait();
#pragma unroll
    for (int i = 0; i < 16; ++i) out[16 * h + i] += t[i];
  }
}

__device__ __forceinline__ void tmem_ld_wait() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Shared-memory matrix descriptor: K-major, 64B swizzle, 64-byte rows, 8-row
// core groups 512 bytes apart.
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;            // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(512 >> 4) << 32;   // stride byte offset
  d |= (uint64_t)1 << 46;            // descriptor version
  d |= (uint64_t)4 << 61;            // SWIZZLE_64B
  return d;
}

// Instruction descriptor: kind::f16, A = B = BF16, D = F32, both K-major,
// optional negation of the first operand. The MMA computes the transposed
// tile D^T[n][m] = sum_k B[n][k] A[m][k]: its first operand is the B tile
// (MMA M = TC_BN rows -> TMEM lanes) and its second the A tile (MMA N = TC_BM
// -> TMEM columns). Negating either factor negates the product, so the sign
// bit serves the -Ai*Bi and conj(A) terms unchanged.
// `mrows` is the MMA M: TC_BN, or 2 TC_BN for the paired form.
__host__ __device__ constexpr uint32_t make_idesc(bool neg_a, int mrows = TC_BN) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((neg_a ? 1u : 0u) << 13) |
         ((uint32_t)(TC_BM >> 3) << 17) | ((uint32_t)(mrows >> 4) << 24);
}

// --------------------------- vectorised epilogue ----------------------------
__device__ __forceinline__ uint32_t pack_bf16(__nv_bfloat16 a, __nv_bfloat16 b) {
  return (uint32_t)__bfloat16_as_ushort(a) | ((uint32_t)__bfloat16_as_ushort(b) << 16);
}

// --------------------------------- kernel -----------------------------------
struct TcParams {
  int batch, M, N, K;
  int a_batch_div, b_batch_div;
  int mt, nt, total;   // total = batch * mt * nt * splits work items
  int splits, kbps;    // split K: each work item covers kbps K blocks of one tile
  int conj_a;
  int* status;
  unsigned long long wait_ns;  // limit of each mbarrier wait
  int withhold_copies;         // test hook: the copy warp issues nothing (waits run out)
  EpiArgs epi;
};

// Work item w of the loaded kernel: split ks of output tile (b, mt, nt), K
// blocks [kb0, kb1). Every role decodes it the same way.
struct TcWork {
  int b, mt, nt, ks, kb0, kb1;
};
__device__ __forceinline__ TcWork tc_work(const TcParams& p, int w, int nkb) {
  TcWork t;
  t.ks = w % p.splits;
  const int wt = w / p.splits;
  t.b = wt / (p.mt * p.nt);
  const int r = wt - t.b * p.mt * p.nt;
  t.mt = r / p.nt;
  t.nt = r - t.mt * p.nt;
  t.kb0 = t.ks * p.kbps;
  t.kb1 = min(nkb, t.kb0 + p.kbps);
  return t;
}
// Paired form: work item w is the n-tile pair (2 np, 2 np + 1) of (b, mt);
// CTA `rank` of the cluster takes n-tile 2 np + rank. No split K.
__device__ __forceinline__ TcWork tc_work_pair(const TcParams& p, int w, int nkb, int rank) {
  TcWork t;
  const int np = p.nt >> 1;
  t.ks = 0;
  t.b = w / (p.mt * np);
  const int r = w - t.b * p.mt * np;
  t.mt = r / np;
  t.nt = 2 * (r - t.mt * np) + rank;
  t.kb0 = 0;
  t.kb1 = nkb;
  return t;
}

// PAIR: the paired form, launched in clusters of two CTAs (work items are
// n-tile pairs, see tc_work_pair). The even CTA issues the MMAs; both CTAs
// load their operand parts against the even CTA's `full` barriers, drain
// their own TMEM and release it on the even CTA's `tempty` barrier.
template <int KIND, bool PAIR = false>
__global__ void __launch_bounds__(TC_THREADS, 1)
    tc_cgemm_kernel(const __grid_constant__ CUtensorMap tmA,
                    const __grid_constant__ CUtensorMap tmB, const TcParams p) {
  constexpr int kStages = PAIR ? TP_STAGES : TC_STAGES;
  constexpr int kStageBytes = PAIR ? TP_STAGE_BYTES : STAGE_BYTES;
  constexpr int kAPlane = PAIR ? TP_A_PLANE_BYTES : A_PLANE_BYTES;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + kStages * kStageBytes);
  uint64_t* empty = full + kStages;
  uint64_t* tfull = empty + kStages;
  uint64_t* tempty = tfull + 1;
  uint64_t* mdone = tempty + 1;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mdone + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int nkb = (p.K + TC_BK - 1) / TC_BK;
  // work items: one per CTA, or one per cluster (PAIR)
  const int rank = PAIR ? (int)cluster_rank() : 0;
  const int unit0 = PAIR ? (int)(blockIdx.x >> 1) : (int)blockIdx.x;
  const int ustep = PAIR ? (int)(gridDim.x >> 1) : (int)gridDim.x;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(tfull, 1);
    mbar_init(tempty, PAIR ? 2 * TC_EPI_WARPS : TC_EPI_WARPS);
    mbar_init(mdone, 1);
    *abort_flag = 0;
    fence_barrier_init();
    prefetch_tmap(&tmA);
    prefetch_tmap(&tmB);
  }
  if (warp == 1) tmem_alloc<PAIR>(tmem_slot, TMEM_COLS);
  tc_fence_before();
  // PAIR: the peer's barriers must be initialised and its TMEM allocated
  // before either CTA signals or writes across the pair.
  __syncwarp();
  if constexpr (PAIR) cluster_sync(); else __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  // The prologue above overlaps the previous kernel of the stream (PDL);
  // operands and outputs are touched only after it has completed.
  pdl_enter();

  if (warp < TC_EPI_W0) {
    asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;\n" ::"n"(REG_CTRL));
  if (warp == 0) {
    // ------------------------------ TMA producer ------------------------------
    // withhold_copies (tests of the bounded waits, single-CTA form only):
    // nothing is issued, so the consumers' waits run into their limit with no
    // copy in flight.
    if (lane == 0 && !p.withhold_copies) {
      int stage = 0;
      uint32_t ph = 0;
      uint32_t issued_mask = 0, issued_ph = 0;
      bool ok = true;
      for (int w = unit0; w < p.total && ok; w += ustep) {
        const TcWork t = PAIR ? tc_work_pair(p, w, nkb, rank) : tc_work(p, w, nkb);
        const int b = t.b, mt = t.mt, nt = t.nt;
        const int ab = b / p.a_batch_div;
        for (int kb = t.kb0; kb < t.kb1; ++kb) {
          if (!mbar_wait(&empty[stage], ph ^ 1u, abort_flag, p.status, p.wait_ns)) { ok = false; break; }
          uint8_t* base = smem + stage * kStageBytes;
          if constexpr (PAIR) {
            // both CTAs' parts complete on the even CTA's barrier
            const uint32_t fb = cluster_addr(&full[stage], 0);
            if (rank == 0) mbar_expect_tx(&full[stage], 2 * kStageBytes);
#pragma unroll
            for (int q = 0; q < 4; ++q)
              tma_load_3d_pair(base + q * kAPlane, &tmA, fb, kb * TC_BK,
                               mt * TC_BM + rank * (TC_BM / 2), ab * 4 + q);
#pragma unroll
            for (int q = 0; q < 4; ++q)
              tma_load_3d_pair(base + 4 * kAPlane + q * B_PLANE_BYTES, &tmB, fb, kb * TC_BK,
                               nt * TC_BN, (b / p.b_batch_div) * 4 + q);
          } else {
            mbar_expect_tx(&full[stage], STAGE_BYTES);
#pragma unroll
            for (int q = 0; q < 4; ++q)
              tma_load_3d(base + q * A_PLANE_BYTES, &tmA, &full[stage], kb * TC_BK, mt * TC_BM,
                          ab * 4 + q);
#pragma unroll
            for (int q = 0; q < 4; ++q)
              tma_load_3d(base + 4 * A_PLANE_BYTES + q * B_PLANE_BYTES, &tmB, &full[stage],
                          kb * TC_BK, nt * TC_BN, (b / p.b_batch_div) * 4 + q);
          }
          issued_mask |= 1u << stage;
          issued_ph = (issued_ph & ~(1u << stage)) | (ph << stage);
          if (++stage == kStages) { stage = 0; ph ^= 1u; }
        }
      }
      // Drain every copy this thread issued before the CTA can exit. In the
      // paired form only the even CTA sees completions (on its barriers).
      if (!ok && (!PAIR || rank == 0)) {
        for (int s = 0; s < kStages; ++s)
          if (issued_mask & (1u << s))
            mbar_wait(&full[s], (issued_ph >> s) & 1u, abort_flag, p.status, kDrainNs, false);
      }
    }
  } else if (warp == 1) {
    // ------------------------------- MMA issuer -------------------------------
    if (lane == 0 && (!PAIR || rank == 0)) {
      const uint32_t id_pos = make_idesc(false, PAIR ? 2 * TC_BN : TC_BN);
      const uint32_t id_neg = make_idesc(true, PAIR ? 2 * TC_BN : TC_BN);
      // Sign of the Ai * Bi term in Re and of the Ai * Br term in Im.
      const uint32_t id_rii = p.conj_a ? id_pos : id_neg;
      const uint32_t id_iir = p.conj_a ? id_neg : id_pos;
      // main (hi*hi) and cross (hi*lo + lo*hi) accumulators, real and imaginary
      const uint32_t m_re = tmem, m_im = tmem + TC_BM;
      const uint32_t c_re = tmem + 2 * TC_BM, c_im = tmem + 3 * TC_BM;
      int stage = 0;
      uint32_t ph = 0, acc_ph = 0;
      bool ok = true;
      for (int w = unit0; w < p.total && ok; w += ustep) {
        const TcWork t = PAIR ? tc_work_pair(p, w, nkb, rank) : tc_work(p, w, nkb);
        if (!mbar_wait(tempty, acc_ph ^ 1u, abort_flag, p.status, p.wait_ns)) { ok = false; break; }
        tc_fence_after();
        for (int kb = t.kb0; kb < t.kb1; ++kb) {
          if (!mbar_wait(&full[stage], ph, abort_flag, p.status, p.wait_ns)) { ok = false; break; }
          tc_fence_after();
          const uint32_t sa = smem_u32(smem + stage * kStageBytes);
          const uint32_t sb = sa + 4 * kAPlane;
#pragma unroll
          for (int j = 0; j < TC_BK / 16; ++j) {
            const uint32_t ko = j * 32;  // 16 bf16 = 32 bytes along K
            const uint64_t arh = make_desc(sa + 0 * kAPlane + ko);
            const uint64_t arl = make_desc(sa + 1 * kAPlane + ko);
            const uint64_t aih = make_desc(sa + 2 * kAPlane + ko);
            const uint64_t ail = make_desc(sa + 3 * kAPlane + ko);
            const uint64_t brh = make_desc(sb + 0 * B_PLANE_BYTES + ko);
            const uint64_t brl = make_desc(sb + 1 * B_PLANE_BYTES + ko);
            const uint64_t bih = make_desc(sb + 2 * B_PLANE_BYTES + ko);
            const uint64_t bil = make_desc(sb + 3 * B_PLANE_BYTES + ko);
            const uint32_t acc = (kb > t.kb0 || j > 0) ? 1u : 0u;
            // Re += Ar Br -/+ Ai Bi
            mma_bf16<PAIR>(m_re, brh, arh, id_pos, acc);
            mma_bf16<PAIR>(m_re, bih, aih, id_rii, 1u);
            mma_bf16<PAIR>(c_re, brl, arh, id_pos, acc);
            mma_bf16<PAIR>(c_re, brh, arl, id_pos, 1u);
            mma_bf16<PAIR>(c_re, bil, aih, id_rii, 1u);
            mma_bf16<PAIR>(c_re, bih, ail, id_rii, 1u);
            // Im += Ar Bi +/- Ai Br
            mma_bf16<PAIR>(m_im, bih, arh, id_pos, acc);
            mma_bf16<PAIR>(m_im, brh, aih, id_iir, 1u);
            mma_bf16<PAIR>(c_im, bil, arh, id_pos, acc);
            mma_bf16<PAIR>(c_im, bih, arl, id_pos, 1u);
            mma_bf16<PAIR>(c_im, brl, aih, id_iir, 1u);
            mma_bf16<PAIR>(c_im, brh, ail, id_iir, 1u);
          }
          if constexpr (PAIR) mma_commit_pair(&empty[stage], 0x3); else mma_commit(&empty[stage]);
          if (++stage == kStages) { stage = 0; ph ^= 1u; }
        }
        if (!ok) break;
        if constexpr (PAIR) mma_commit_pair(tfull, 0x3); else mma_commit(tfull);
        acc_ph ^= 1u;
      }
      // Wait for every MMA this thread issued before TMEM is released.
      if constexpr (PAIR) mma_commit_pair(mdone, 0x1); else mma_commit(mdone);
      mbar_wait(mdone, 0, abort_flag, p.status, kDrainNs, false);
    }
  }
  } else {
    asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;\n" ::"n"(REG_EPI));
    // -------------------------------- epilogue --------------------------------
    // TMEM lane = output column n, TMEM column = output row m (see the MMA
    // issue): each thread drains one column of the tile, 32 rows at a time.
    const int q = warp & 3;  // TMEM lane quarter this warp may access
    const int half = (warp - TC_EPI_W0) >> 2;  // the two warps of a quarter take alternate chunks
    uint32_t acc_ph = 0;
    for (int w = unit0; w < p.total; w += ustep) {
      if (!warp_wait(tfull, acc_ph, abort_flag, p.status, p.wait_ns)) break;
      tc_fence_after();
      const TcWork t = PAIR ? tc_work_pair(p, w, nkb, rank) : tc_work(p, w, nkb);
      const int b = t.b, mt = t.mt, nt = t.nt;
      const int n = nt * TC_BN + q * 32 + lane;
      const int mbase = mt * TC_BM;
      const uint32_t lane_addr = tmem + ((uint32_t)(q * 32) << 16);
      // Drain both chunks of this warp (rows c0 and c0 + 64) into registers,
      // hand TMEM back to the MMA warp, then run the epilogue from registers
      // while the next tile's MMAs proceed.
      const int c0 = half, c1 = half + 2;
      const bool has0 = mbase + c0 * 32 < p.M, has1 = mbase + c1 * 32 < p.M;  // warp-uniform
      float re0[32], im0[32], re1[32], im1[32];
      if (has0) {
        tmem_sum32(lane_addr, c0 * 32, 2 * TC_BM, re0);
        tmem_sum32(lane_addr, TC_BM + c0 * 32, 2 * TC_BM, im0);
      }
      if (has1) {
        tmem_sum32(lane_addr, c1 * 32, 2 * TC_BM, re1);
        tmem_sum32(lane_addr, TC_BM + c1 * 32, 2 * TC_BM, im1);
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) {
        if constexpr (PAIR) mbar_arrive_cluster(cluster_addr(tempty, 0));
        else mbar_arrive(tempty);
      }
      if (n < p.N) {
        if constexpr (KIND == EPI_PARTIAL) {
          // raw partial sums of split t.ks, one column per thread
          float2* o = p.epi.partial + ((long long)t.ks * p.batch + b) * p.M * p.N + n;
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const int m0 = mbase + c0 * 32 + j, m1 = mbase + c1 * 32 + j;
            if (has0 && m0 < p.M) o[(long long)m0 * p.N] = make_float2(re0[j], im0[j]);
            if (has1 && m1 < p.M) o[(long long)m1 * p.N] = make_float2(re1[j], im1[j]);
          }
        } else {
          if (has0) epi_col32<KIND>(p.epi, b, n, mbase + c0 * 32, p.M, p.N, re0, im0);
          if (has1) epi_col32<KIND>(p.epi, b, n, mbase + c1 * 32, p.M, p.N, re1, im1);
        }
      }
      acc_ph ^= 1u;
    }
  }

  tc_fence_before();
  // PAIR: neither CTA leaves (or frees TMEM) while the pair's MMAs, copies or
  // arrivals may still touch it.
  __syncwarp();
  if constexpr (PAIR) cluster_sync(); else __syncthreads();
  tc_fence_after();
  if (warp == 1) {
    __syncwarp();
    tmem_dealloc<PAIR>(tmem, TMEM_COLS);
  }
}

// ------------------ generated-A variant (DFT operand built in the CTA) -------
//
// Every A operand of the MFT/FFT GEMMs is a DFT matrix whose phase is affine
// along K for a fixed row: phase(row, k) = theta0(row) + k * delta(row)
// cycles (DftAxis, FP64 coefficients). Instead of streaming the split matrix
// from memory, four generator warps build each 128 x 32 A stage in shared
// memory: one thread per row keeps the 32 step factors cis(t * delta) in
// registers (computed once per tile), forms cis(theta0 + 32 kb delta) once per
// stage, and multiplies. Both phases are reduced with the error-free FP32
// scheme of cis_ff, so every element is within a few FP32 ulps of the cached
// matrix. Only the field operand B goes through TMA, which halves the bytes
// per stage and leaves room for a 4-deep B pipeline.
constexpr int GA_STAGES = 2;
constexpr int GB_STAGES = 4;
constexpr int G_A_BYTES = 4 * A_PLANE_BYTES;   // 32 KB
constexpr int G_B_BYTES = 4 * B_PLANE_BYTES;   // 32 KB
constexpr int G_SMEM_BYTES = GA_STAGES * G_A_BYTES + GB_STAGES * G_B_BYTES + 1024 + 256;
constexpr int G_THREADS = 320;  // TMA, MMA, 4 epilogue warps, 4 generator warps

struct TcGenParams {
  int batch, M, N, K;
  int a_batch_div, b_batch_div;
  int mt, nt, total;
  int conj_a;
  int rows_are_out;
  const DftAxis* axes;
  int* status;
  unsigned long long wait_ns;  // limit of each mbarrier wait
  EpiArgs epi;
};

// cis(2 pi (n * delta + theta)) for an integer n < 2^24 and float pairs delta,
// theta; the reduction is exact up to FP32 rounding of the final argument.
__device__ __forceinline__ float2 cis_affine(float n, FF delta, FF theta) {
  const float p = n * delta.hi;
  const float e = fmaf(n, delta.hi, -p);
  float r = (p - rintf(p)) + theta.hi;
  r = r + (fmaf(n, delta.lo, e) + theta.lo);
  r = r - rintf(r);
  float s, c;
  sincospif(2.0f * r, &s, &c);
  return make_float2(c, s);
}

__global__ void __launch_bounds__(G_THREADS, 1)
    tc_cgemm_gen_kernel(const __grid_constant__ CUtensorMap tmB, const TcGenParams p) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  uint8_t* abuf = smem;                                 // GA_STAGES x 32 KB
  uint8_t* bbuf = smem + GA_STAGES * G_A_BYTES;         // GB_STAGES x 32 KB
  uint64_t* bfull = reinterpret_cast<uint64_t*>(bbuf + GB_STAGES * G_B_BYTES);
  uint64_t* bempty = bfull + GB_STAGES;
  uint64_t* afull = bempty + GB_STAGES;
  uint64_t* aempty = afull + GA_STAGES;
  uint64_t* tfull = aempty + GA_STAGES;
  uint64_t* tempty = tfull + 1;
  uint64_t* mdone = tempty + 1;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mdone + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int nkb = (p.K + TC_BK - 1) / TC_BK;

  if (threadIdx.x == 0) {
    for (int s = 0; s < GB_STAGES; ++s) {
      mbar_init(&bfull[s], 1);
      mbar_init(&bempty[s], 1);
    }
    for (int s = 0; s < GA_STAGES; ++s) {
      mbar_init(&afull[s], 4);
      mbar_init(&aempty[s], 1);
    }
    mbar_init(tfull, 1);
    mbar_init(tempty, 4);
    mbar_init(mdone, 1);
    *abort_flag = 0;
    fence_barrier_init();
    prefetch_tmap(&tmB);
  }
  if (warp == 1) tmem_alloc(tmem_slot, TMEM_COLS);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ------------------------- TMA producer (field B) -------------------------
    if (lane == 0) {
      int stage = 0;
      uint32_t ph = 0, issued_mask = 0, issued_ph = 0;
      bool ok = true;
      for (int w = blockIdx.x; w < p.total && ok; w += gridDim.x) {
        const int b = w / (p.mt * p.nt);
        const int r = w - b * p.mt * p.nt;
        const int nt = r - (r / p.nt) * p.nt;
        for (int kb = 0; kb < nkb; ++kb) {
          if (!mbar_wait(&bempty[stage], ph ^ 1u, abort_flag, p.status, p.wait_ns)) { ok = false; break; }
          mbar_expect_tx(&bfull[stage], G_B_BYTES);
          uint8_t* base = bbuf + stage * G_B_BYTES;
#pragma unroll
          for (int q = 0; q < 4; ++q)
            tma_load_3d(base + q * B_PLANE_BYTES, &tmB, &bfull[stage], kb * TC_BK, nt * TC_BN,
                        (b / p.b_batch_div) * 4 + q);
          issued_mask |= 1u << stage;
          issued_ph = (issued_ph & ~(1u << stage)) | (ph << stage);
          if (++stage == GB_STAGES) { stage = 0; ph ^= 1u; }
        }
      }
      if (!ok)
        for (int s = 0; s < GB_STAGES; ++s)
          if (issued_mask & (1u << s))
            mbar_wait(&bfull[s], (issued_ph >> s) & 1u, abort_flag, p.status, kDrainNs, false);
    }
  } else if (warp == 1) {
    // ------------------------------- MMA issuer -------------------------------
    if (lane == 0) {
      const uint32_t id_pos = make_idesc(false);
      const uint32_t id_neg = make_idesc(true);
      const uint32_t id_rii = p.conj_a ? id_pos : id_neg;
      const uint32_t id_iir = p.conj_a ? id_neg : id_pos;
      const uint32_t m_re = tmem, m_im = tmem + TC_BM;
      const uint32_t c_re = tmem + 2 * TC_BM, c_im = tmem + 3 * TC_BM;
      int sb = 0, sa = 0;
      uint32_t phb = 0, pha = 0, acc_ph = 0;
      bool ok = true;
      for (int w = blockIdx.x; w < p.total && ok; w += gridDim.x) {
        if (!mbar_wait(tempty, acc_ph ^ 1u, abort_flag, p.status, p.wait_ns)) { ok = false; break; }
        tc_fence_after();
        for (int kb = 0; kb < nkb; ++kb) {
          if (!mbar_wait(&bfull[sb], phb, abort_flag, p.status, p.wait_ns)) { ok = false; break; }
          if (!mbar_wait(&afull[sa], pha, abort_flag, p.status, p.wait_ns)) { ok = false; break; }
          tc_fence_after();
          const uint32_t s_a = smem_u32(abuf + sa * G_A_BYTES);
          const uint32_t s_b = smem_u32(bbuf + sb * G_B_BYTES);
#pragma unroll
          for (int j = 0; j < TC_BK / 16; ++j) {
            const uint32_t ko = j * 32;
            const uint64_t arh = make_desc(s_a + 0 * A_PLANE_BYTES + ko);
            const uint64_t arl = make_desc(s_a + 1 * A_PLANE_BYTES + ko);
            const uint64_t aih = make_desc(s_a + 2 * A_PLANE_BYTES + ko);
            const uint64_t ail = make_desc(s_a + 3 * A_PLANE_BYTES + ko);
            const uint64_t brh = make_desc(s_b + 0 * B_PLANE_BYTES + ko);
            const uint64_t brl = make_desc(s_b + 1 * B_PLANE_BYTES + ko);
            const uint64_t bih = make_desc(s_b + 2 * B_PLANE_BYTES + ko);
            const uint64_t bil = make_desc(s_b + 3 * B_PLANE_BYTES + ko);
            const uint32_t acc = (kb > 0 || j > 0) ? 1u : 0u;
            mma_bf16(m_re, brh, arh, id_pos, acc);
            mma_bf16(m_re, bih, aih, id_rii, 1u);
            mma_bf16(c_re, brl, arh, id_pos, acc);
            mma_bf16(c_re, brh, arl, id_pos, 1u);
            mma_bf16(c_re, bil, aih, id_rii, 1u);
            mma_bf16(c_re, bih, ail, id_rii, 1u);
            mma_bf16(m_im, bih, arh, id_pos, acc);
            mma_bf16(m_im, brh, aih, id_iir, 1u);
            mma_bf16(c_im, bil, arh, id_pos, acc);
            mma_bf16(c_im, bih, arl, id_pos, 1u);
            mma_bf16(c_im, brl, aih, id_iir, 1u);
            mma_bf16(c_im, brh, ail, id_iir, 1u);
          }
          mma_commit(&bempty[sb]);
          mma_commit(&aempty[sa]);
          if (++sb == GB_STAGES) { sb = 0; phb ^= 1u; }
          if (++sa == GA_STAGES) { sa = 0; pha ^= 1u; }
        }
        if (!ok) break;
        mma_commit(tfull);
        acc_ph ^= 1u;
      }
      mma_commit(mdone);
      mbar_wait(mdone, 0, abort_flag, p.status, kDrainNs, false);
    }
  } else if (warp < 6) {
    // -------------------------------- epilogue --------------------------------
    const int q = warp & 3;  // column-per-thread drain, as in tc_cgemm_kernel
    uint32_t acc_ph = 0;
    for (int w = blockIdx.x; w < p.total; w += gridDim.x) {
      if (!warp_wait(tfull, acc_ph, abort_flag, p.status, p.wait_ns)) break;
      tc_fence_after();
      const int b = w / (p.mt * p.nt);
      const int r = w - b * p.mt * p.nt;
      const int mt = r / p.nt, nt = r - (r / p.nt) * p.nt;
      const int n = nt * TC_BN + q * 32 + lane;
      const int mbase = mt * TC_BM;
      const uint32_t lane_addr = tmem + ((uint32_t)(q * 32) << 16);
#pragma unroll 1
      for (int c = 0; c < TC_BM / 32; ++c) {
        if (mbase + c * 32 >= p.M) break;
        float re[32], im[32], t[32];
        tmem_ld32(lane_addr + c * 32, re);
        tmem_ld32(lane_addr + TC_BM + c * 32, im);
        tmem_ld32(lane_addr + 2 * TC_BM + c * 32, t);
        tmem_ld_wait();
#pragma unroll
        for (int i = 0; i < 32; ++i) re[i] += t[i];
        tmem_ld32(lane_addr + 3 * TC_BM + c * 32, t);
        tmem_ld_wait();
#pragma unroll
        for (int i = 0; i < 32; ++i) im[i] += t[i];
        if (n < p.N) epi_col32(p.epi, b, n, mbase + c * 32, p.M, p.N, re, im);
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(tempty);
      acc_ph ^= 1u;
    }
  } else {
    // ------------------------ A generators (one row each) ---------------------
    const int r = threadIdx.x - 192;  // 0..127
    const uint32_t swz = (uint32_t)((r >> 1) & 3);
    int sa = 0;
    uint32_t pha = 0;
    bool ok = true;
    for (int w = blockIdx.x; w < p.total && ok; w += gridDim.x) {
      const int b = w / (p.mt * p.nt);
      const int rr = w - b * p.mt * p.nt;
      const int mt = rr / p.nt;
      const DftAxis ax = p.axes[b / p.a_batch_div];
      const int R = mt * TC_BM + r;
      const bool live = R < p.M;
      // Row phase: theta0 + k * delta cycles (FP64 once per row and tile).
      double coef, delta, theta;
      if (p.rows_are_out) {
        coef = ax.a_out * (double)R + ax.b_out;
        delta = ax.sigma * coef * ax.a_in + ax.g_in;
        theta = ax.sigma * coef * ax.b_in + ax.d_in + ax.g_out * (double)R + ax.d_out;
      } else {
        coef = ax.a_in * (double)R + ax.b_in;
        delta = ax.sigma * coef * ax.a_out + ax.g_out;
        theta = ax.sigma * coef * ax.b_out + ax.d_out + ax.g_in * (double)R + ax.d_in;
      }
      const FF dff = ff_from_double(delta);
      const FF tff = ff_from_double(theta - rint(theta));
      const FF zero{0.f, 0.f};
      float2 step[32];
#pragma unroll
      for (int t = 0; t < 32; ++t) step[t] = cis_affine((float)t, dff, zero);
      for (int kb = 0; kb < nkb; ++kb) {
        if (!warp_wait(&aempty[sa], pha ^ 1u, abort_flag, p.status, p.wait_ns)) { ok = false; break; }
        const float2 base = cis_affine((float)(kb * TC_BK), dff, tff);
        uint8_t* tile = abuf + sa * G_A_BYTES + r * 64;
        const int kvalid = p.K - kb * TC_BK;  // columns beyond K must be zero
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          uint32_t rh[4], rl[4], ih[4], il[4];
#pragma unroll
          for (int h = 0; h < 4; ++h) {
            float2 v[2];
#pragma unroll
            for (int e = 0; e < 2; ++e) {
              const int t = c * 8 + h * 2 + e;
              v[e] = (live && t < kvalid) ? cmul(base, step[t]) : make_float2(0.f, 0.f);
            }
            __nv_bfloat16 h0, l0, h1, l1;
            split_bf16(v[0].x, h0, l0);
            split_bf16(v[1].x, h1, l1);
            rh[h] = pack_bf16(h0, h1);
            rl[h] = pack_bf16(l0, l1);
            split_bf16(v[0].y, h0, l0);
            split_bf16(v[1].y, h1, l1);
            ih[h] = pack_bf16(h0, h1);
            il[h] = pack_bf16(l0, l1);
          }
          // 64B swizzle: 16-byte chunk c of row r sits at chunk c ^ ((r >> 1) & 3).
          const uint32_t off = ((uint32_t)c ^ swz) << 4;
          *reinterpret_cast<uint4*>(tile + 0 * A_PLANE_BYTES + off) =
              make_uint4(rh[0], rh[1], rh[2], rh[3]);
          *reinterpret_cast<uint4*>(tile + 1 * A_PLANE_BYTES + off) =
              make_uint4(rl[0], rl[1], rl[2], rl[3]);
          *reinterpret_cast<uint4*>(tile + 2 * A_PLANE_BYTES + off) =
              make_uint4(ih[0], ih[1], ih[2], ih[3]);
          *reinterpret_cast<uint4*>(tile + 3 * A_PLANE_BYTES + off) =
              make_uint4(il[0], il[1], il[2], il[3]);
        }
        // Make the generic-proxy stores visible to the tensor core, then signal.
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncwarp();
        if (lane == 0) mbar_arrive(&afull[sa]);
        if (++sa == GA_STAGES) { sa = 0; pha ^= 1u; }
      }
    }
  }

  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) {
    __syncwarp();
    tmem_dealloc(tmem, TMEM_COLS);
  }
}

// ------------------------------- host side ----------------------------------
using LoadedKernel = void (*)(CUtensorMap, CUtensorMap, TcParams);

// One instantiation of the loaded-operand kernel per epilogue kind.
LoadedKernel loaded_kernel(int kind) {
  switch (kind) {
    case EPI_C64: return tc_cgemm_kernel<EPI_C64>;
    case EPI_SPLIT: return tc_cgemm_kernel<EPI_SPLIT>;
    case EPI_INTENSITY: return tc_cgemm_kernel<EPI_INTENSITY>;
    case EPI_GRADF: return tc_cgemm_kernel<EPI_GRADF>;
    case EPI_PUPIL: return tc_cgemm_kernel<EPI_PUPIL>;
    case EPI_PSF_GRADF: return tc_cgemm_kernel<EPI_PSF_GRADF>;
    case EPI_SPLIT2: return tc_cgemm_kernel<EPI_SPLIT2>;
    case EPI_DOT: return tc_cgemm_kernel<EPI_DOT>;
    case EPI_PARTIAL: return tc_cgemm_kernel<EPI_PARTIAL>;
    default: return nullptr;
  }
}

// The paired form per epilogue kind (split K never runs paired).
LoadedKernel loaded_kernel_pair(int kind) {
  switch (kind) {
    case EPI_C64: return tc_cgemm_kernel<EPI_C64, true>;
    case EPI_SPLIT: return tc_cgemm_kernel<EPI_SPLIT, true>;
    case EPI_INTENSITY: return tc_cgemm_kernel<EPI_INTENSITY, true>;
    case EPI_GRADF: return tc_cgemm_kernel<EPI_GRADF, true>;
    case EPI_PUPIL: return tc_cgemm_kernel<EPI_PUPIL, true>;
    case EPI_PSF_GRADF: return tc_cgemm_kernel<EPI_PSF_GRADF, true>;
    case EPI_SPLIT2: return tc_cgemm_kernel<EPI_SPLIT2, true>;
    case EPI_DOT: return tc_cgemm_kernel<EPI_DOT, true>;
    default: return nullptr;
  }
}

const void* const* loaded_kernels() {
  static const void* all[] = {
      (const void*)tc_cgemm_kernel<EPI_C64>,       (const void*)tc_cgemm_kernel<EPI_SPLIT>,
      (const void*)tc_cgemm_kernel<EPI_INTENSITY>, (const void*)tc_cgemm_kernel<EPI_GRADF>,
      (const void*)tc_cgemm_kernel<EPI_PUPIL>,     (const void*)tc_cgemm_kernel<EPI_PSF_GRADF>,
      (const void*)tc_cgemm_kernel<EPI_SPLIT2>,    (const void*)tc_cgemm_kernel<EPI_DOT>,
      (const void*)tc_cgemm_kernel<EPI_PARTIAL>,
      (const void*)tc_cgemm_kernel<EPI_C64, true>,       (const void*)tc_cgemm_kernel<EPI_SPLIT, true>,
      (const void*)tc_cgemm_kernel<EPI_INTENSITY, true>, (const void*)tc_cgemm_kernel<EPI_GRADF, true>,
      (const void*)tc_cgemm_kernel<EPI_PUPIL, true>,     (const void*)tc_cgemm_kernel<EPI_PSF_GRADF, true>,
      (const void*)tc_cgemm_kernel<EPI_SPLIT2, true>,    (const void*)tc_cgemm_kernel<EPI_DOT, true>,
      nullptr};
  return all;
}

// Paired launch: clusters of two CTAs, with programmatic dependent launch.
template <typename... KArgs, typename... Args>
cudaError_t launch_pair(void (*kernel)(KArgs...), int clusters, cudaStream_t s, Args&&... args) {
  cudaLaunchAttribute at[2];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  at[1].id = cudaLaunchAttributeClusterDimension;
  at[1].val.clusterDim.x = 2;
  at[1].val.clusterDim.y = 1;
  at[1].val.clusterDim.z = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(2 * clusters);
  cfg.blockDim = dim3(TC_THREADS);
  cfg.dynamicSmemBytes = SMEM_BYTES;
  cfg.stream = s;
  cfg.attrs = at;
  cfg.numAttrs = 2;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}
// Split-K reduction: D = sum of the partials in split order, then the GEMM's
// own epilogue element by element (the FP32 form's epilogue code).
// The splits' partial sums per element, added in split order. S > 0: the
// count known at compile time, all S loads issued before the adds (one memory
// round trip instead of S); S = 0: `splits` read at run time.
template <int S>
__global__ void splitk_reduce_kernel(const float2* __restrict__ part, int splits, int batch,
                                     int M, int N, const EpiArgs e) {
  pdl_enter();
  const long long total = (long long)batch * M * N;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  float2 v;
  if constexpr (S > 0) {
    float2 q[S];
#pragma unroll
    for (int s = 0; s < S; ++s) q[s] = __ldg(part + (long long)s * total + i);
    v = q[0];
#pragma unroll
    for (int s = 1; s < S; ++s) {
      v.x += q[s].x;
      v.y += q[s].y;
    }
  } else {
    v = part[i];
    for (int s = 1; s < splits; ++s) {
      const float2 q = part[(long long)s * total + i];
      v.x += q.x;
      v.y += q.y;
    }
  }
  const long long mn = (long long)M * N;
  const int b = (int)(i / mn);
  const long long r = i - (long long)b * mn;
  const int m = (int)(r / N);
  const int n = (int)(r - (long long)m * N);
  epi_apply(e, b, m, n, M, N, v);
}

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::once_flag g_encode_once;
int g_encode_status = DLX_OK;
void init_encode() {
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault,
                                       &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !fn) {
    g_encode_status = fail(DLX_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled is not available");
    return;
  }
  g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
}
// Paired form of the loaded-operand GEMM (dlx_set_gemm_pair, or DLX_GEMM_PAIR=1
// in the environment); off by default: on GB300 it measures the same as the
// single-CTA form (within 1-3% either way on the batched workloads), whose
// mainloop is bound by barrier hand-offs, TMA latency and the epilogue's
// memory traffic rather than by shared-memory or L2 bandwidth. Read at every
// launch, so a change also applies to existing plans (but not to CUDA graphs
// already captured).
std::atomic<int> g_pair_enabled{-1};  // -1: not yet read from the environment
// Limit of each mbarrier wait (dlx_set_wait_limit_ns), read at every launch.
std::atomic<unsigned long long> g_wait_ns{kTimeoutNs};
// Test hook (dlx_test_gemm_withhold_copies): the copy warp issues nothing.
std::atomic<int> g_withhold{0};

bool pair_enabled() {
  int v = g_pair_enabled.load();
  if (v < 0) {
    const char* e = getenv("DLX_GEMM_PAIR");
    int want = (e && atoi(e) != 0) ? 1 : 0;
    int expect = -1;
    g_pair_enabled.compare_exchange_strong(expect, want);
    v = g_pair_enabled.load();
  }
  return v != 0;
}

// State of one device: set up on first use with that device current.
struct TcDevice {
  std::once_flag once;
  int init_status = DLX_OK;
  int num_sms = 0;
  int cc = 0;
  int pair_clusters = 0;  // co-resident clusters of the paired form (0: unavailable)
  int* status = nullptr;  // DLX_ERR_TIMEOUT word read by dlx_device_status
};
TcDevice g_dev[kMaxDevices];

void init_device(TcDevice* d, int dev) {
  std::call_once(g_encode_once, init_encode);
  if (g_encode_status != DLX_OK) {
    d->init_status = g_encode_status;
    return;
  }
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) {
    d->init_status = fail(DLX_ERR_CUDA, "cudaGetDeviceProperties failed");
    return;
  }
  d->num_sms = prop.multiProcessorCount;
  d->cc = prop.major * 10 + prop.minor;
  if (cudaMalloc(&d->status, sizeof(int)) != cudaSuccess ||
      cudaMemset(d->status, 0, sizeof(int)) != cudaSuccess) {
    d->status = nullptr;
    d->init_status = fail(DLX_ERR_NOMEM, "status word allocation failed");
    return;
  }
  if (d->cc != 103) return;  // no tensor-core form on this device
  // The register split of the loaded kernels needs REG_LAUNCH registers per
  // thread at launch; refuse a build that came out with fewer.
  for (const void* const* k = loaded_kernels(); *k; ++k) {
    cudaFuncAttributes fa{};
    if (cudaFuncGetAttributes(&fa, *k) != cudaSuccess || fa.numRegs < REG_LAUNCH) {
      d->init_status = fail(DLX_ERR_UNSUPPORTED,
                            "tensor-core GEMM: the build's register count does not cover its "
                            "warpgroup register split");
      return;
    }
  }
  bool attr_ok = true;
  for (const void* const* k = loaded_kernels(); *k; ++k)
    attr_ok = attr_ok && cudaFuncSetAttribute(*k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              SMEM_BYTES) == cudaSuccess;
  if (!attr_ok ||
      cudaFuncSetAttribute(tc_cgemm_gen_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           G_SMEM_BYTES) != cudaSuccess) {
    d->init_status = fail(DLX_ERR_CUDA, "cudaFuncSetAttribute(tensor-core GEMM) failed");
    return;
  }
  // How many two-CTA clusters fit at once: the paired form's persistent grid.
  {
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = 2;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(2 * (d->num_sms / 2));
    cfg.blockDim = dim3(TC_THREADS);
    cfg.dynamicSmemBytes = SMEM_BYTES;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, (const void*)tc_cgemm_kernel<EPI_C64, true>, &cfg) !=
        cudaSuccess) {
      (void)cudaGetLastError();
      n = 0;
    }
    d->pair_clusters = n;
  }
}

// The current device's state, set up on first use; nullptr (error recorded)
// if the device cannot be queried.
TcDevice* tc_device() {
  int dev = 0;
  if (current_device(&dev) != DLX_OK) return nullptr;
  TcDevice* d = &g_dev[dev];
  std::call_once(d->once, init_device, d, dev);
  return d;
}

// Operand tiles are 64-byte rows (32 K elements); L2 promotion of 128 bytes
// measured 1.9% faster per GEMM launch than 256 bytes at 512 x 512 x 512 x 64.
// Split operand [nbatch][4][rows][split_ld(K)]: the extent along K is K, so
// TMA fills the padded columns (and a last K block past K) with zeros.
int encode_split(CUtensorMap* map, const __nv_bfloat16* base, int rows, int K, int nbatch,
                 int box_rows) {
  const cuuint64_t ld = (cuuint64_t)split_ld(K);
  cuuint64_t dims[3] = {(cuuint64_t)K, (cuuint64_t)rows, (cuuint64_t)nbatch * 4};
  cuuint64_t strides[2] = {ld * 2, (cuuint64_t)rows * ld * 2};
  cuuint32_t box[3] = {(cuuint32_t)TC_BK, (cuuint32_t)box_rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<__nv_bfloat16*>(base),
                        dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    return fail(DLX_ERR_ARG, "cuTensorMapEncodeTiled failed (code " + std::to_string((int)r) +
                                 ") for a split operand of " + std::to_string(rows) + " x " +
                                 std::to_string(K));
  return DLX_OK;
}

}  // namespace

bool tc_supported() {
  const TcDevice* d = tc_device();
  return d && d->init_status == DLX_OK && d->cc == 103;
}

// Split K (see GemmArgs::splits). Creation-time switch for plans made after
// the call (dlx_set_split_k); on by default.
std::atomic<int> g_split_k_enabled{1};
bool split_k_enabled() { return g_split_k_enabled.load() != 0; }

int split_k_count(long long tiles, int K) {
  const TcDevice* d = tc_device();
  if (!d || d->init_status != DLX_OK || d->cc != 103 || tiles <= 0) return 1;
  const int nkb = (K + TC_BK - 1) / TC_BK;
  if (nkb < 2 || tiles * 2 > d->num_sms) return 1;  // half the SMs or more are busy already
  long long s = d->num_sms / tiles;
  if (s > 8) s = 8;
  if (s > nkb) s = nkb;
  if (s < 2) return 1;
  // the count the launch will use: every split gets at least one K block
  const int kbps = (nkb + (int)s - 1) / (int)s;
  return (nkb + kbps - 1) / kbps;
}

size_t split_k_bytes(int splits, long long batch, int M, int N) {
  if (splits <= 1) return 0;
  return (size_t)splits * (size_t)batch * (size_t)M * (size_t)N * sizeof(float2);
}

int* tc_status_word() {
  TcDevice* d = tc_device();
  return d ? d->status : nullptr;
}

int launch_gemm_tc(const GemmArgs& g, cudaStream_t s) {
  const TcDevice* dev = tc_device();
  if (!dev) return DLX_ERR_CUDA;
  if (dev->init_status != DLX_OK) return dev->init_status;
  if (dev->cc != 103) return fail(DLX_ERR_UNSUPPORTED, "split-BF16 GEMM needs an sm_103 device");
  const int num_sms = dev->num_sms;
  const unsigned long long wait_ns = g_wait_ns.load();
  if (g.batch <= 0 || g.M <= 0 || g.N <= 0) return DLX_OK;
  if (g.K <= 0) return fail(DLX_ERR_SHAPE, "split-BF16 GEMM: inner size must be positive");
  const int div = g.a_batch_div > 0 ? g.a_batch_div : 1;
  const int bdiv = g.b_batch_div > 0 ? g.b_batch_div : 1;
  const int nB = (g.batch + bdiv - 1) / bdiv;
  if (g.a_axes) {
    if (!g.Bs) return fail(DLX_ERR_ARG, "split-BF16 GEMM: null operand");
    CUtensorMap tb;
    DLX_TRY(encode_split(&tb, g.Bs, g.N, g.K, nB, TC_BN));
    TcGenParams p{};
    p.batch = g.batch; p.M = g.M; p.N = g.N; p.K = g.K;
    p.a_batch_div = div;
    p.b_batch_div = bdiv;
    p.mt = (g.M + TC_BM - 1) / TC_BM;
    p.nt = (g.N + TC_BN - 1) / TC_BN;
    p.total = g.batch * p.mt * p.nt;
    p.conj_a = g.conj_a ? 1 : 0;
    p.rows_are_out = g.a_rows_are_out ? 1 : 0;
    p.axes = g.a_axes;
    p.status = dev->status;
    p.wait_ns = wait_ns;
    p.epi = g.epi;
    const int grid = p.total < num_sms ? p.total : num_sms;
    tc_cgemm_gen_kernel<<<grid, G_THREADS, G_SMEM_BYTES, s>>>(tb, p);
    DLX_LAUNCH_CHECK("tc_cgemm_gen_kernel");
    return DLX_OK;
  }
  if (!g.As || !g.Bs) return fail(DLX_ERR_ARG, "split-BF16 GEMM: null operand");
  const int nA = (g.batch + div - 1) / div;
  const int nkb = (g.K + TC_BK - 1) / TC_BK;
  const bool split = g.splits > 1 && g.split_ws != nullptr && nkb > 1;
  const int nt_tiles = (g.N + TC_BN - 1) / TC_BN;
  // Paired form: n-tiles in pairs, no split K.
  const int withhold = g_withhold.load();
  const bool want_pair = g.pair_mode == 2 || (g.pair_mode == 0 && pair_enabled());
  const bool pair = !split && nt_tiles % 2 == 0 && dev->pair_clusters > 0 && !withhold &&
                    want_pair;
  CUtensorMap ta, tb;
  DLX_TRY(encode_split(&ta, g.As, g.M, g.K, nA, pair ? TC_BM / 2 : TC_BM));
  DLX_TRY(encode_split(&tb, g.Bs, g.N, g.K, nB, TC_BN));
  TcParams p{};
  p.batch = g.batch; p.M = g.M; p.N = g.N; p.K = g.K;
  p.a_batch_div = div;
  p.b_batch_div = bdiv;
  p.mt = (g.M + TC_BM - 1) / TC_BM;
  p.nt = nt_tiles;
  p.splits = 1;
  p.kbps = nkb;
  if (split) {
    p.kbps = (nkb + g.splits - 1) / g.splits;
    p.splits = (nkb + p.kbps - 1) / p.kbps;  // every split gets at least one K block
  }
  p.total = g.batch * p.mt * p.nt * p.splits;
  p.conj_a = g.conj_a ? 1 : 0;
  p.status = dev->status;
  p.wait_ns = wait_ns;
  p.withhold_copies = withhold;
  p.epi = g.epi;
  if (split) {
    p.epi.kind = EPI_PARTIAL;
    p.epi.partial = g.split_ws;
  }
  if (pair) {
    p.total = g.batch * p.mt * (p.nt / 2);  // n-tile pairs
    LoadedKernel kern = loaded_kernel_pair(p.epi.kind);
    if (!kern) return fail(DLX_ERR_ARG, "split-BF16 GEMM: unknown epilogue kind");
    const int clusters = p.total < dev->pair_clusters ? p.total : dev->pair_clusters;
    const cudaError_t e = launch_pair(kern, clusters, s, ta, tb, p);
    if (e != cudaSuccess) return check_cuda(e, "tc_cgemm_kernel (paired)");
    note_launch();
    return DLX_OK;
  }
  const int grid = p.total < num_sms ? p.total : num_sms;
  LoadedKernel kern = loaded_kernel(p.epi.kind);
  if (!kern) return fail(DLX_ERR_ARG, "split-BF16 GEMM: unknown epilogue kind");
  DLX_PDL_LAUNCH("tc_cgemm_kernel", kern, dim3(grid), dim3(TC_THREADS), SMEM_BYTES, s, ta, tb, p);
  if (split) {
    const long long n = (long long)g.batch * g.M * g.N;
    const dim3 rgrid(ceil_div(n, 256));
    switch (p.splits) {
#define DLX_SPLITK_REDUCE(S, C)                                                             \
  case C:                                                                                   \
    DLX_PDL_LAUNCH("splitk_reduce_kernel", splitk_reduce_kernel<S>, rgrid, dim3(256), 0, s, \
                   g.split_ws, p.splits, g.batch, g.M, g.N, g.epi);                         \
    break;
      DLX_SPLITK_REDUCE(2, 2) DLX_SPLITK_REDUCE(3, 3) DLX_SPLITK_REDUCE(4, 4)
      DLX_SPLITK_REDUCE(5, 5) DLX_SPLITK_REDUCE(6, 6) DLX_SPLITK_REDUCE(7, 7)
      DLX_SPLITK_REDUCE(8, 8)
#undef DLX_SPLITK_REDUCE
      default:
        DLX_PDL_LAUNCH("splitk_reduce_kernel", splitk_reduce_kernel<0>, rgrid, dim3(256), 0, s,
                       g.split_ws, p.splits, g.batch, g.M, g.N, g.epi);
    }
  }
  return DLX_OK;
}

}  // namespace dlx

extern "C" int dlx_set_split_k(int enable) {
  dlx::g_split_k_enabled.store(enable ? 1 : 0);
  return DLX_OK;
}

extern "C" int dlx_set_gemm_pair(int enable) {
  dlx::g_pair_enabled.store(enable ? 1 : 0);
  return DLX_OK;
}

extern "C" int dlx_gemm_pair_clusters(int* clusters) {
  if (!clusters) return DLX_ERR_ARG;
  const dlx::TcDevice* d = dlx::tc_device();
  *clusters = (d && d->init_status == DLX_OK) ? d->pair_clusters : 0;
  return DLX_OK;
}

extern "C" int dlx_set_wait_limit_ns(unsigned long long limit_ns) {
  dlx::g_wait_ns.store(limit_ns ? limit_ns : dlx::kTimeoutNs);
  return DLX_OK;
}

extern "C" int dlx_test_gemm_withhold_copies(int enable) {
  dlx::g_withhold.store(enable ? 1 : 0);
  return DLX_OK;
}

extern "C" int dlx_device_status(void* stream, int* status) {
  using namespace dlx;
  if (!status) return fail(DLX_ERR_ARG, "device_status: null pointer");
  int* word = tc_status_word();
  *status = DLX_OK;
  if (!word) return DLX_OK;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  DLX_TRY_CUDA(cudaStreamSynchronize(s));
  int v = 0;
  DLX_TRY_CUDA(cudaMemcpy(&v, word, sizeof(int), cudaMemcpyDeviceToHost));
  if (v != 0) {
    DLX_TRY_CUDA(cudaMemset(word, 0, sizeof(int)));
    *status = v;
  }
  return DLX_OK;
}
