// conv_tc.cu -- root/part filter convolution on the tcgen05 tensor cores:
// BF16 operands (kind::f16) or FP8-e4m3 operands with per-filter scaling
// (kind::f8f6f4), FP32 accumulation in tensor memory.
//
// Same contraction as conv_fp32.cu (CAR_TRACKING/GPU_function.cu:302-358 and
// :630-685): C[x][y] = sum_{c, xp, yp} A[c][x+xp][y+yp] * B[c][xp][yp], here
// as an implicit GEMM without an im2col copy.  A level's features are kept as
// NQ channel planes of 16 bytes per position ([q][pos][16 B], pos = x*fs0 + y):
// four planes of 8 bf16 channels, or two planes of 16 e4m3 channels (features
// scaled by kFp8FeatScale).  The chunks of consecutive positions lie 16 bytes
// apart, exactly the row stride of the canonical K-major, no-swizzle operand
// layout, so for filter tap (xp, yp) the A operand of 128 consecutive output
// positions p is the slab rows p + xp*fs0 + yp of the staged planes: one
// shared-memory descriptor per tap, LBO = the plane stride (next chunk of
// channels), SBO = 128 B (next 8 rows).  An MMA takes two planes (K = 16 bf16
// or 32 e4m3), so a tap is 2 MMAs in BF16 and 1 in FP8.
//
// One launch covers every model of a plan.  The filters of all models share
// one bank [tap][q][row][16 B] over one tap grid (the largest part filter):
// each part filter is a row (zero weights around it in the grid), and each
// root filter is cut into blocks of the grid, one row per block.  A level's
// job multiplies its feature planes by every row the level uses in one MMA
// chain (N = all of them), so the root filters cost no extra pass over the
// features: block (a, b) of a root, evaluated at position p + a*gx*fs0 + b*gy,
// is that root's partial sum over the block's taps, and k_root_sum adds a
// root's blocks back into its map.  In BF16 mode the root blocks run on split
// operands: the features' BF16 remainder planes (f - bf16(f)) and each block's
// BF16 remainder row (w - bf16(w)) add the products hi*lo and lo*hi to hi*hi
// (a second MMA chain accumulates lo*hi into the same TMEM columns), about 16
// significant bits per operand for the roots, whose rounding decides most
// detections; part filters stay plain BF16.
//
// A CTA (12 warps) owns a run of up to 8 tiles of 128 positions of one job, each
// tile with its own TMEM accumulator.  The run's feature slab stays in shared
// memory while the bank streams through a ring of stages, one tap per stage:
// lane 0 of warp 0 bulk-copies (cp.async.bulk, mbarrier completion), lane 0
// of warp 1+i issues the tap's MMAs for tile i (one issuing thread per tile:
// one thread alone cannot issue MMAs of N = 48 as fast as the tensor pipe
// retires them) and commits them to the stage's "free" mbarrier, which
// completes when every issuer's MMAs are done, so the copy of tap t+stages
// overlaps the MMAs of tap t.  Grids wider than the slab allows are walked in column phases (the
// slab reloaded per phase).  After the last MMA the twelve warps read the
// accumulators with tcgen05.ld (warp w reads TMEM lanes 32(w%4)..+31; the three
// warps of a lane quarter take turns at the tiles and column chunks) and write
// part maps in the reference layout and root blocks by position.  Every
// mbarrier wait is bounded; a timeout sets an error bit, and the CTA waits
// (bounded) for its own copies and MMAs before it frees TMEM and leaves.
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <cuda_bf16.h>
#include <cuda_fp8.h>

#include <algorithm>
#include <cmath>

#include "runtime.h"
#include "tc_planes.h"

namespace geye {

constexpr int kTcThreads = 384;                 // 12 warps: three per TMEM lane quarter in the epilogue
constexpr int kTcM = 128;                        // positions per tile (TMEM lanes)
constexpr int kTcMaxTiles = 8;                   // tiles per CTA, at most
constexpr int kTcMaxStages = 8;                  // bank stages in the ring, at most
constexpr int kTcHead = 256;                     // mbarriers and the TMEM address
constexpr int kTcColBytes = 256 * 24;            // the job's column table (N <= 256 entries)
constexpr int kTcMaxN = 256;                     // N of an MMA, at most
constexpr int kTcTmemCols = 512;                 // tiles per CTA x N, at most
constexpr unsigned long long kWaitNs = 1000000000ull;   // a wait gives up after 1 s (then 4 s for the drain)

// mbarriers in the head: slab landed, slab free, all MMAs done, then per stage
// "landed" and "free"
constexpr int kBarSlabFull = 0, kBarSlabFree = 1, kBarDone = 2, kBarStageFull = 3,
              kBarStageFree = 3 + kTcMaxStages;

// ---------------------------------------------------------------------------
// PTX wrappers
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
// bounded wait on a phase: false once limit_ns have passed
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, unsigned long long limit_ns) {
  const unsigned long long t0 = global_ns();
  while (!mbar_try_wait(bar, parity))
    if (global_ns() - t0 > limit_ns) return false;
  return true;
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
template <int NQ>
__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                       uint32_t accumulate) {
  if constexpr (NQ == 4)
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
  else
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void tc_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tc_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
__device__ __forceinline__ void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// shared-memory operand descriptor: K-major, no swizzle; lbo = byte distance
// between the two 8-element K chunks, sbo = between 8-row groups
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;   // descriptor version of tcgen05
  return d;                 // base offset 0, relative LBO, no swizzle
}

// instruction descriptors, D = F32, both operands K-major, dense:
// kind::f16 with A = B = BF16 (format 1); kind::f8f6f4 with A = B = E4M3 (format 0)
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
__host__ __device__ constexpr uint32_t idesc_e4m3(int M, int N) {
  return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// ---------------------------------------------------------------------------
// kernel
// ---------------------------------------------------------------------------
// Chunk (job, first tile, tiles, tap columns per phase) -> one CTA.
template <int NQ>
__global__ void __launch_bounds__(kTcThreads, 1)
    k_conv_tc(const TcJob *__restrict__ jobs, const int4 *__restrict__ chunks, const TcCol *__restrict__ cols,
              const uint8_t *__restrict__ arena16, const uint8_t *__restrict__ bank, int n_stages, int tps,
              float *__restrict__ arena, int *err) {
  extern __shared__ __align__(128) uint8_t sm[];
  uint64_t *bar = reinterpret_cast<uint64_t *>(sm);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(sm + 8 * (3 + 2 * kTcMaxStages));
  const int4 ch = chunks[blockIdx.x];
  const TcJob J = jobs[ch.x];
  const int tile0 = ch.y, ntile = ch.z, cs = ch.w;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int NS = n_stages;
  // taps a stage: tps > 0 that many, 0 a filter column, < 0 every tap of a phase (the bank
  // of the phase resident at once: one copy with the slab, no refills while the MMAs run)
  const bool whole = tps < 0;
  tps = whole ? cs * J.b0 : (tps > 0 ? tps : J.b0);
  const int p_begin = tile0 * kTcM;
  const int S = ntile * kTcM + (cs - 1) * J.fs0 + (J.b0 - 1);   // slab cells per plane
  const uint32_t plane_bytes = (uint32_t)S * 16u;
  const bool split = J.n_lo > 0;
  TcCol *col_s = reinterpret_cast<TcCol *>(sm + kTcHead);          // the job's column table
  uint8_t *slab = sm + kTcHead + kTcColBytes;
  uint8_t *slab_lo = slab + (size_t)NQ * plane_bytes;
  const size_t slab_end = kTcHead + kTcColBytes + (size_t)NQ * plane_bytes * (split ? 2 : 1);
  uint8_t *stages = sm + ((slab_end + 127) & ~(size_t)127);
  const uint32_t tap_bytes = (uint32_t)NQ * (uint32_t)J.n * 16u;   // one tap of the job's bank
  const uint32_t stage_bytes = (uint32_t)tps * tap_bytes;           // room of a stage
  uint32_t ncols = 32;
  while (ncols < (uint32_t)(ntile * J.n)) ncols <<= 1;
  for (int k = threadIdx.x; k < J.n; k += kTcThreads) col_s[k] = cols[J.col_tab + k];

  // MMA issuers: warps 1 .. nis, one per tile (tiles i = w-1, w-1+nis, ...); each commits to the
  // "free" and "done" barriers, so those complete once every issuer's MMAs are done
  const int nis = min(ntile, kTcThreads / 32 - 1);
  if (threadIdx.x == 0) {
    for (int i = 0; i < 3 + 2 * kTcMaxStages; i++)
      mbar_init(&bar[i], (i == kBarSlabFree || i == kBarDone || i >= kBarStageFree) ? (uint32_t)nis : 1u);
    mbar_fence_init();
  }
  if (warp == 0) tmem_alloc(tslot, ncols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  const int phases = (J.b1 + cs - 1) / cs;
  bool ok = true;

  if (warp == 0 && lane == 0) {
    // ---- producer: the phase's slab, then one bank tap per stage
    int issued = 0, slabs = 0;
    for (int ph = 0; ph < phases && ok; ph++) {
      const int xp0 = ph * cs, ncol = min(cs, J.b1 - xp0);
      if (ph > 0 && !mbar_wait(&bar[kBarSlabFree], (uint32_t)((ph - 1) & 1), kWaitNs)) { ok = false; break; }
      mbar_expect_tx(&bar[kBarSlabFull], (uint32_t)NQ * plane_bytes * (split ? 2u : 1u));
      const size_t cell0 = (size_t)p_begin + (size_t)xp0 * J.fs0;
      for (int q = 0; q < NQ; q++)
        bulk_g2s(slab + (size_t)q * plane_bytes,
                 arena16 + 2 * (size_t)J.plane_off + ((size_t)q * J.plane_cells + cell0) * 16, plane_bytes,
                 &bar[kBarSlabFull]);
      if (split)
        for (int q = 0; q < NQ; q++)
          bulk_g2s(slab_lo + (size_t)q * plane_bytes,
                   arena16 + 2 * (size_t)J.lo_off + ((size_t)q * J.plane_cells + cell0) * 16, plane_bytes,
                   &bar[kBarSlabFull]);
      slabs++;
      // the phase's taps t = xp*b0 + yp, step to a stage (tps divides b0: no stage crosses a phase)
      const int step = whole ? ncol * J.b0 : tps;
      for (int t = xp0 * J.b0; t < (xp0 + ncol) * J.b0 && ok; t += step) {
        const int s = issued % NS;
        if (issued >= NS && !mbar_wait(&bar[kBarStageFree + s], (uint32_t)((issued / NS - 1) & 1), kWaitNs)) {
          ok = false;
          break;
        }
        mbar_expect_tx(&bar[kBarStageFull + s], (uint32_t)step * tap_bytes);
        bulk_g2s(stages + (size_t)s * stage_bytes, bank + (size_t)J.bank_off + (size_t)t * tap_bytes,
                 (uint32_t)step * tap_bytes, &bar[kBarStageFull + s]);
        issued++;
      }
    }
    if (!ok) {
      atomicOr(err, 1);
      // every copy issued lands before the CTA leaves
      if (slabs) mbar_wait(&bar[kBarSlabFull], (uint32_t)((slabs - 1) & 1), 4 * kWaitNs);
      for (int s = 0; s < NS && s < issued; s++) {
        const int last = issued - 1 - ((issued - 1 - s) % NS);
        mbar_wait(&bar[kBarStageFull + s], (uint32_t)((last / NS) & 1), 4 * kWaitNs);
      }
    }
  } else if (warp >= 1 && warp <= nis && lane == 0) {
    // ---- MMA issue: per tap, this warp's tiles' chains (and the split chain of the root blocks)
    // The start-address field of a descriptor is (address >> 4) in its low 14 bits and
    // every operand lies below 2^18 bytes, so moving an operand by a 16-byte multiple off
    // is adding off >> 4 to the descriptor: A moves by cells (16 B), B by rows (16 B).
    const uint32_t idesc = NQ == 4 ? idesc_bf16(kTcM, J.n) : idesc_e4m3(kTcM, J.n);
    const uint32_t idesc_lo = idesc_bf16(kTcM, split ? J.n_lo : 16);
    const uint64_t a_base = sdesc(smem_u32(slab), plane_bytes, 128u);
    const uint64_t alo_base = sdesc(smem_u32(slab_lo), plane_bytes, 128u);
    const uint32_t a_k1 = 2u * (uint32_t)S;     // planes 2, 3: 2 * plane_bytes >> 4
    const uint32_t b_k1 = 2u * (uint32_t)J.n;   // planes 2, 3 of a stage
    int used = 0;
    for (int ph = 0; ph < phases && ok; ph++) {
      const int xp0 = ph * cs, ncol = min(cs, J.b1 - xp0);
      if (!mbar_wait(&bar[kBarSlabFull], (uint32_t)(ph & 1), kWaitNs)) { ok = false; break; }
      const int step = whole ? ncol * J.b0 : tps;
      for (int t0 = xp0 * J.b0; t0 < (xp0 + ncol) * J.b0 && ok; t0 += step) {
        const int s = used % NS;
        if (!mbar_wait(&bar[kBarStageFull + s], (uint32_t)((used / NS) & 1), kWaitNs)) { ok = false; break; }
        tc_fence_after();
        const uint64_t stage_desc = sdesc(smem_u32(stages + (size_t)s * stage_bytes), (uint32_t)J.n * 16u, 128u);
        for (int u = 0; u < step; u++) {
          const int t = t0 + u, xp = t / J.b0, yp = t - (t / J.b0) * J.b0;
          const uint64_t b_base = stage_desc + (uint32_t)(u * NQ * J.n);   // tap u of the stage: NQ*n rows of 16 B on
          const uint32_t acc = t > 0 ? 1u : 0u;
          const uint32_t shift = (uint32_t)((xp - xp0) * J.fs0 + yp);
          for (int i = warp - 1; i < ntile; i += nis) {
            const uint32_t d = tmem + (uint32_t)(i * J.n);
            const uint64_t ad = a_base + ((uint32_t)(i * kTcM) + shift);
            tc_mma<NQ>(d, ad, b_base, idesc, acc);
            if constexpr (NQ == 4) {
              tc_mma<NQ>(d, ad + a_k1, b_base + b_k1, idesc, 1u);
              if (split) {
                const uint64_t al = alo_base + ((uint32_t)(i * kTcM) + shift);
                const uint64_t bl = b_base + (uint32_t)J.lo_row;
                tc_mma<NQ>(d + (uint32_t)J.lo_row, al, bl, idesc_lo, 1u);
                tc_mma<NQ>(d + (uint32_t)J.lo_row, al + a_k1, bl + b_k1, idesc_lo, 1u);
              }
            }
          }
        }
        tc_commit(&bar[kBarStageFree + s]);   // the stage is free once these MMAs are done
        used++;
      }
      tc_commit(&bar[kBarSlabFree]);   // and the slab once the phase's MMAs are
    }
    if (!ok) atomicOr(err, 2);
    tc_commit(&bar[kBarDone]);   // tracks every MMA issued above
  }
  __syncthreads();
  bool done = mbar_wait(&bar[kBarDone], 0u, kWaitNs);
  if (!done) {
    atomicOr(err, 4);
    mbar_wait(&bar[kBarDone], 0u, 4 * kWaitNs);   // the MMAs must finish before TMEM is read or freed
  }
  ok = __syncthreads_and(done && ok);
  tc_fence_after();
  // ---- epilogue: row r of a tile is TMEM lane r; warp w reads the rows 32*(w & 3) .. +31 of
  // the tiles, and the three warps of a lane quarter take turns at the (tile, 16-column chunk) items
  const int ncell = J.fs0 * J.fs1;
  const int quarter = warp & 3, nch = J.n >> 4;
  for (int item = warp >> 2; item < ntile * nch; item += kTcThreads / 128) {
    const int i = item / nch, c0 = (item - i * nch) * 16;
    const TcCol head = col_s[c0];               // a 16-column chunk lies inside one section
    if (head.kind == 0) continue;               // (uniform across the warp: the loads below are collective)
    const int p = p_begin + i * kTcM + quarter * 32 + lane;
    const int x = p / J.fs0, y = p - x * J.fs0;
    const uint32_t row_addr = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(i * J.n);
    uint32_t r[16], r2[16];
    __syncwarp();
    tc_ld16(row_addr + (uint32_t)c0, r);
    if (head.kind == 2 && head.pair) tc_ld16(row_addr + (uint32_t)(c0 + head.pair), r2);
    tc_wait_ld();
    if (ok && p < ncell) {
#pragma unroll
      for (int k = 0; k < 16; k++) {
        const TcCol c = col_s[c0 + k];
        float v;
        memcpy(&v, &r[k], 4);
        if (c.kind == 1) {
          if (x < c.cols && y < c.rows) arena[(size_t)c.off + (size_t)x * c.rows + y] = v * c.inv;
        } else if (c.kind == 2) {
          if (c.pair) {
            float w;
            memcpy(&w, &r2[k], 4);
            v += w;
          }
          arena[(size_t)c.off + p] = v * c.inv;
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, ncols);
}

// ---------------------------------------------------------------------------
// persistent form: one CTA per SM walks a contiguous range of units (a unit: up
// to two tiles of one job).  The bank of the units' jobs stays resident in
// shared memory while consecutive units use it (reloaded where the range moves
// to another bank), the slab of unit k+1 lands while the MMAs of unit k run
// (two slab buffers; a slab too large for one buffer takes both, and its unit
// waits for the one before), and two TMEM accumulator sets let the epilogue of
// unit k overlap the MMAs of unit k+1.  Warp 0 copies, warps 1 and 2 issue the
// MMAs (one per tile of a unit: a single thread cannot issue MMAs of N = 48
// as fast as the tensor pipe retires them), warps 3..10 drain the accumulators
// (two per TMEM lane quarter).  Every MMA of a tile runs in the same order as
// in k_conv_tc, so the two forms give the same sums.
// ---------------------------------------------------------------------------
constexpr int kTcpIssuers = 2;                   // warps 1, 2: one per tile of a unit
constexpr int kTcpWarps = 3 + 8;
constexpr int kTcpThreads = 32 * kTcpWarps;
constexpr int kTcpEpiWarps = 8;
constexpr int kTcpHead = 256;
constexpr int kTcpTiles = 2;                     // tiles per unit, at most
constexpr uint32_t kTcpCopy = 32768;             // bytes per bulk copy of a bank
// barriers: slab landed [2], unit's MMAs done [2], accumulators full [2] and
// free [2] (one arrival per epilogue warp), bank landed, every MMA done
constexpr int kPbSlabFull = 0, kPbMmaDone = 2, kPbAccFull = 4, kPbAccFree = 6, kPbBank = 8, kPbEnd = 9,
              kPbCount = 10;

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// units: (job, first tile, tiles, flags: bit 0 = the slab takes both buffers);
// ctainfo[c]: CTA c's units (first, end), bank region and slab buffer bytes
template <int NQ>
__global__ void __launch_bounds__(kTcpThreads, 1)
    k_conv_tcp(const TcJob *__restrict__ jobs, const int4 *__restrict__ units, const int4 *__restrict__ ctainfo,
               const TcCol *__restrict__ cols, const uint8_t *__restrict__ arena16, const uint8_t *__restrict__ bank,
               uint32_t colbuf, float *__restrict__ arena, int *err) {
  extern __shared__ __align__(128) uint8_t sm[];
  uint64_t *bar = reinterpret_cast<uint64_t *>(sm);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(sm + 8 * kPbCount);
  // this CTA's units, and its shared memory: the bank region, then two slab buffers
  const int4 R = ctainfo[blockIdx.x];
  const int u0 = R.x, nu = R.y - R.x;
  const uint32_t slab_half = (uint32_t)R.w;
  uint8_t *bank_s = sm + kTcpHead;
  uint8_t *slab_s = bank_s + (uint32_t)R.z;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int i = 0; i < kPbCount; i++)
      mbar_init(&bar[i], (i == kPbAccFree || i == kPbAccFree + 1)                      ? kTcpEpiWarps
                         : (i == kPbSlabFull || i == kPbSlabFull + 1 || i == kPbBank) ? 1
                                                                                       : kTcpIssuers);
    mbar_fence_init();
  }
  if (warp == 0) tmem_alloc(tslot, 2 * colbuf);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  bool ok = true;

  if (warp == 0 && lane == 0) {
    // ---- copies: a bank where the range reaches a new one, then each unit's slab
    int cur = -1, banks = 0, slabs = 0;
    auto unit_done = [&](int j) { return mbar_wait(&bar[kPbMmaDone + (j & 1)], (uint32_t)((j >> 1) & 1), kWaitNs); };
    for (int k = 0; k < nu && ok; k++) {
      const int4 U = units[u0 + k];
      const TcJob J = jobs[U.x];   // a copy: the MMA asm clobbers memory, a reference would reload every field
      const bool big = U.w & 1, prev_big = k > 0 && (units[u0 + k - 1].w & 1);
      const bool new_bank = J.bank_off != cur;
      // the buffer's last user (unit k-2), and unit k-1 where its slab or bank is overwritten
      if (k >= 2 && !unit_done(k - 2)) { ok = false; break; }
      if (k >= 1 && (big || prev_big || new_bank) && !unit_done(k - 1)) { ok = false; break; }
      if (new_bank) {
        const uint32_t bytes = (uint32_t)J.b0 * J.b1 * NQ * J.n * 16u;
        mbar_expect_tx(&bar[kPbBank], bytes);
        for (uint32_t o = 0; o < bytes; o += kTcpCopy)
          bulk_g2s(bank_s + o, bank + (size_t)J.bank_off + o, min(kTcpCopy, bytes - o), &bar[kPbBank]);
        cur = J.bank_off;
        banks++;
      }
      const int S = U.z * kTcM + (J.b1 - 1) * J.fs0 + (J.b0 - 1);
      const uint32_t plane_bytes = (uint32_t)S * 16u;
      const bool split = J.n_lo > 0;
      uint8_t *slab = slab_s + (big ? 0u : (uint32_t)(k & 1) * slab_half);
      const size_t cell0 = (size_t)U.y * kTcM;
      mbar_expect_tx(&bar[kPbSlabFull + (k & 1)], (uint32_t)NQ * plane_bytes * (split ? 2u : 1u));
      for (int q = 0; q < NQ; q++)
        bulk_g2s(slab + (size_t)q * plane_bytes,
                 arena16 + 2 * (size_t)J.plane_off + ((size_t)q * J.plane_cells + cell0) * 16, plane_bytes,
                 &bar[kPbSlabFull + (k & 1)]);
      if (split)
        for (int q = 0; q < NQ; q++)
          bulk_g2s(slab + (size_t)(NQ + q) * plane_bytes,
                   arena16 + 2 * (size_t)J.lo_off + ((size_t)q * J.plane_cells + cell0) * 16, plane_bytes,
                   &bar[kPbSlabFull + (k & 1)]);
      slabs = k + 1;
    }
    if (!ok) {
      atomicOr(err, 1);
      // every copy issued lands before the CTA leaves
      if (banks) mbar_wait(&bar[kPbBank], (uint32_t)((banks - 1) & 1), 4 * kWaitNs);
      for (int j = max(0, slabs - 2); j < slabs; j++)
        mbar_wait(&bar[kPbSlabFull + (j & 1)], (uint32_t)((j >> 1) & 1), 4 * kWaitNs);
    }
  } else if (warp >= 1 && warp <= kTcpIssuers && lane == 0) {
    // ---- MMAs: every tap of this warp's tiles of the unit into accumulator set k & 1
    int cur = -1, banks = 0;
    for (int k = 0; k < nu && ok; k++) {
      const int4 U = units[u0 + k];
      const TcJob J = jobs[U.x];   // a copy: the MMA asm clobbers memory, a reference would reload every field
      const bool big = U.w & 1, split = J.n_lo > 0;
      if (J.bank_off != cur) {
        if (!mbar_wait(&bar[kPbBank], (uint32_t)(banks & 1), kWaitNs)) { ok = false; break; }
        cur = J.bank_off;
        banks++;
      }
      if (!mbar_wait(&bar[kPbSlabFull + (k & 1)], (uint32_t)((k >> 1) & 1), kWaitNs)) { ok = false; break; }
      if (k >= 2 && !mbar_wait(&bar[kPbAccFree + (k & 1)], (uint32_t)(((k - 2) >> 1) & 1), kWaitNs)) {
        ok = false;
        break;
      }
      tc_fence_after();
      const int S = U.z * kTcM + (J.b1 - 1) * J.fs0 + (J.b0 - 1);
      const uint32_t plane_bytes = (uint32_t)S * 16u;
      const uint8_t *slab = slab_s + (big ? 0u : (uint32_t)(k & 1) * slab_half);
      const uint32_t idesc = NQ == 4 ? idesc_bf16(kTcM, J.n) : idesc_e4m3(kTcM, J.n);
      const uint32_t idesc_lo = idesc_bf16(kTcM, split ? J.n_lo : 16);
      const uint64_t a_base = sdesc(smem_u32(slab), plane_bytes, 128u);
      const uint64_t alo_base = sdesc(smem_u32(slab + (size_t)NQ * plane_bytes), plane_bytes, 128u);
      const uint64_t b_desc = sdesc(smem_u32(bank_s), (uint32_t)J.n * 16u, 128u);
      const uint32_t a_k1 = 2u * (uint32_t)S, b_k1 = 2u * (uint32_t)J.n;
      const uint32_t dbase = tmem + (uint32_t)(k & 1) * colbuf;
      const int taps = J.b0 * J.b1;
      for (int t = 0, xp = 0, yp = 0; t < taps; t++) {
        const uint64_t b_base = b_desc + (uint32_t)(t * NQ * J.n);
        const uint32_t acc = t > 0 ? 1u : 0u;
        const uint32_t shift = (uint32_t)(xp * J.fs0 + yp);
        for (int i = warp - 1; i < U.z; i += kTcpIssuers) {
          const uint32_t d = dbase + (uint32_t)(i * J.n);
          const uint64_t ad = a_base + ((uint32_t)(i * kTcM) + shift);
          tc_mma<NQ>(d, ad, b_base, idesc, acc);
          if constexpr (NQ == 4) {
            tc_mma<NQ>(d, ad + a_k1, b_base + b_k1, idesc, 1u);
            if (split) {
              const uint64_t al = alo_base + ((uint32_t)(i * kTcM) + shift);
              const uint64_t bl = b_base + (uint32_t)J.lo_row;
              tc_mma<NQ>(d + (uint32_t)J.lo_row, al, bl, idesc_lo, 1u);
              tc_mma<NQ>(d + (uint32_t)J.lo_row, al + a_k1, bl + b_k1, idesc_lo, 1u);
            }
          }
        }
        if (++yp == J.b0) { yp = 0; xp++; }
      }
      tc_commit(&bar[kPbMmaDone + (k & 1)]);   // the slab (and bank) are free once these MMAs are done
      tc_commit(&bar[kPbAccFull + (k & 1)]);   // and the accumulators full
    }
    if (!ok) atomicOr(err, 2);
    if (nu > 0) tc_commit(&bar[kPbEnd]);   // tracks every MMA issued above
  } else if (warp > kTcpIssuers) {
    // ---- epilogue: warp w reads the rows 32*(w & 3) .. +31 of the unit's tiles; the
    // two warps of a lane quarter take alternate (tile, 16-column chunk) items
    const int quarter = warp & 3, half = (warp - kTcpIssuers - 1) >> 2;
    for (int k = 0; k < nu && ok; k++) {
      const int4 U = units[u0 + k];
      const TcJob J = jobs[U.x];   // a copy: the MMA asm clobbers memory, a reference would reload every field
      if (!mbar_wait(&bar[kPbAccFull + (k & 1)], (uint32_t)((k >> 1) & 1), kWaitNs)) { ok = false; break; }
      tc_fence_after();
      const int ncell = J.fs0 * J.fs1, nch = J.n >> 4, fs0 = J.fs0;
      const TcCol *col = cols + J.col_tab;
      const uint32_t abase = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(k & 1) * colbuf;
      for (int item = half; item < U.z * nch; item += 2) {
        const int i = item / nch, c0 = (item - i * nch) * 16;
        const TcCol head = col[c0];                 // a 16-column chunk lies inside one section
        if (head.kind == 0) continue;               // (uniform across the warp: the loads below are collective)
        const int p = U.y * kTcM + i * kTcM + quarter * 32 + lane;
        const int x = p / fs0, y = p - x * fs0;
        const uint32_t row_addr = abase + (uint32_t)(i * J.n);
        uint32_t r[16], r2[16];
        __syncwarp();
        tc_ld16(row_addr + (uint32_t)c0, r);
        if (head.kind == 2 && head.pair) tc_ld16(row_addr + (uint32_t)(c0 + head.pair), r2);
        tc_wait_ld();
        if (p < ncell) {
#pragma unroll
          for (int kk = 0; kk < 16; kk++) {
            const TcCol c = col[c0 + kk];
            float v;
            memcpy(&v, &r[kk], 4);
            if (c.kind == 1) {
              if (x < c.cols && y < c.rows) arena[(size_t)c.off + (size_t)x * c.rows + y] = v * c.inv;
            } else if (c.kind == 2) {
              if (c.pair) {
                float w;
                memcpy(&w, &r2[kk], 4);
                v += w;
              }
              arena[(size_t)c.off + p] = v * c.inv;
            }
          }
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&bar[kPbAccFree + (k & 1)]);
    }
    if (!ok) atomicOr(err, 8);
  }
  __syncthreads();
  // every MMA issued is done before TMEM is freed
  if (nu > 0 && !mbar_wait(&bar[kPbEnd], 0u, kWaitNs)) {
    atomicOr(err, 4);
    mbar_wait(&bar[kPbEnd], 0u, 4 * kWaitNs);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, 2 * colbuf);
}

// Root maps from their blocks: root[x][y] = sum_k block_k[x*fs0 + y + shift_k],
// the blocks in row order.
__global__ void k_root_sum(const RootSumJob *__restrict__ jobs, float *__restrict__ arena) {
  const RootSumJob &J = jobs[blockIdx.y];
  const int r0 = J.r0, n = J.r0 * J.r1, fs0 = J.fs0, nblk = J.nblk, out = J.out_off;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    const int x = e / r0, y = e - x * r0;
    const int p = x * fs0 + y;
    float v = 0.f;
    for (int k = 0; k < nblk; k++) v += arena[(size_t)J.blk[k] + p + J.shift[k]];
    arena[(size_t)out + e] = v;
  }
}

// feature planes for a standalone call: [pos][32] float -> NQ planes [ncell + pad][16 B]
template <int NQ>
__global__ void k_feat_planes(const float *__restrict__ feat, int ncell, uint8_t *__restrict__ planes) {
  const size_t plane = ((size_t)ncell + kTcPlanePad) * 16;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ncell + kTcPlanePad; i += gridDim.x * blockDim.x) {
    float f[32];
    for (int c = 0; c < 32; c++) f[c] = i < ncell ? feat[(size_t)i * kFeatPad + c] : 0.f;
    tc_store_planes<NQ>(f, planes, plane, i);
  }
}

// ---------------------------------------------------------------------------
// host: the filter bank
// ---------------------------------------------------------------------------
static uint16_t to_bf16(float f) {   // round to nearest even
  uint32_t u;
  memcpy(&u, &f, 4);
  if ((u & 0x7f800000u) == 0x7f800000u) return (uint16_t)(u >> 16);   // inf / nan
  const uint32_t lsb = (u >> 16) & 1u;
  u += 0x7fffu + lsb;
  return (uint16_t)(u >> 16);
}
static float from_bf16(uint16_t h) {
  const uint32_t u = (uint32_t)h << 16;
  float f;
  memcpy(&f, &u, 4);
  return f;
}

static int tc_planes_of(geye_conv_mode mode) { return mode == GEYE_CONV_FP8 ? 2 : 4; }
static int pad16(int n) { return (n + 15) & ~15; }

// power of two that brings a filter's absolute maximum under e4m3's 448
static float e4m3_filter_scale(const float *F, size_t n) {
  float m = 0.f;
  for (size_t i = 0; i < n; i++) m = std::max(m, std::fabs(F[i]));
  if (!(m > 0.f)) return 1.f;
  return std::ldexp(1.0f, (int)std::floor(std::log2(448.0 / m)));
}

// One bank row: filter f ([31][fb1][fb0], element (c, x, y) at c*fb0*fb1 + x*fb0 + y)
// from its row y0, column x0 on (a whole filter: 0, 0), or the BF16 remainder of
// those weights (lo).  Padding rows have no filter.
struct BankRow {
  const float *h = nullptr;   // host copy
  const float *d = nullptr;   // device copy (FP8 banks are converted on the device)
  int fb0 = 0, fb1 = 0, y0 = 0, x0 = 0, lo = 0;
  float scale = 1.f;          // FP8: the filter's power-of-two scale
};

struct DevRow {
  const float *f;
  int fb0, fb1, y0, x0;
  float scale;
};

// e4m3 bank [tap][2][rows][16]: element (tap t = xp*b0 + yp, plane q, row r, lane k)
// = channel 16q + k of row r's filter at (x0 + xp, y0 + yp) times its scale, CUDA's
// own conversion (as for the features); zero outside the filter
__global__ void k_bank_e4m3(const DevRow *__restrict__ rows, int n_rows, int R, int b0, int taps,
                            uint8_t *__restrict__ out) {
  const size_t total = (size_t)taps * 2 * R * 16;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(e % 16), r = (int)((e / 16) % R), q = (int)((e / (16 * (size_t)R)) % 2);
    const int t = (int)(e / (32 * (size_t)R));
    const int c = 16 * q + k, xp = t / b0, yp = t - (t / b0) * b0;
    float v = 0.f;
    if (r < n_rows && c < kFeat) {
      const DevRow D = rows[r];
      const int x = D.x0 + xp, y = D.y0 + yp;
      if (D.f && x < D.fb1 && y < D.fb0) v = D.f[(size_t)c * D.fb0 * D.fb1 + (size_t)x * D.fb0 + y] * D.scale;
    }
    out[e] = (uint8_t)__nv_cvt_float_to_fp8(v, __NV_SATFINITE, __NV_E4M3);
  }
}

// A job's bank holds its own rows (first, n) contiguously, [tap][q][n][16 B], so a
// stage of consecutive taps is one bulk copy.  One buffer holds every layout.
struct BankLayout {
  int first, n;     // rows of the plan's row list
  size_t off;       // byte offset in the buffer
};
static size_t layout_bytes(int NQ, int b0, int b1, int n) { return (size_t)b0 * b1 * NQ * n * 16; }

static geye_status upload_bank(geye_ctx *ctx, const std::vector<BankRow> &rows, int NQ, int b0, int b1,
                               const std::vector<BankLayout> &layouts, size_t total, DevBuf &dst) {
  GEYE_TRY(dst.alloc(ctx, std::max<size_t>(total, 16)));
  if (NQ == 4) {
    std::vector<uint16_t> bank(total / 2, 0);
    for (const BankLayout &L : layouts) {
      uint16_t *out = bank.data() + L.off / 2;
      for (int xp = 0; xp < b1; xp++)
        for (int yp = 0; yp < b0; yp++) {
          const size_t t = (size_t)xp * b0 + yp;
          for (int r = 0; r < L.n; r++) {
            const BankRow &B = rows[L.first + r];
            const int x = B.x0 + xp, y = B.y0 + yp;
            if (!B.h || x >= B.fb1 || y >= B.fb0) continue;
            for (int c = 0; c < kFeat; c++) {
              const float w = B.h[(size_t)c * B.fb0 * B.fb1 + (size_t)x * B.fb0 + y];
              const uint16_t hi = to_bf16(w);
              out[((t * 4 + (c >> 3)) * L.n + r) * 8 + (c & 7)] = B.lo ? to_bf16(w - from_bf16(hi)) : hi;
            }
          }
        }
    }
    CUDA_TRY(cudaMemcpyAsync(dst.p, bank.data(), total, cudaMemcpyHostToDevice, ctx->stream));
    CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return GEYE_OK;
  }
  std::vector<DevRow> dr;
  for (const BankRow &B : rows) dr.push_back(DevRow{B.d, B.fb0, B.fb1, B.y0, B.x0, B.scale});
  DevBuf d_rows;
  GEYE_TRY(upload_bytes(ctx, d_rows, dr.data(), sizeof(DevRow) * std::max<size_t>(dr.size(), 1)));
  const int taps = b0 * b1;
  for (const BankLayout &L : layouts) {
    const size_t elems = (size_t)taps * 2 * L.n * 16;
    k_bank_e4m3<<<(int)std::max<size_t>(1, std::min<size_t>((elems + 255) / 256, 2048)), 256, 0, ctx->stream>>>(
        d_rows.as<DevRow>() + L.first, std::max(0, std::min(L.n, (int)dr.size() - L.first)), L.n, b0, taps,
        dst.as<uint8_t>() + L.off);
    CUDA_TRY(cudaGetLastError());
  }
  CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return GEYE_OK;
}

// one layout per distinct row range of the jobs; sets each job's bank_off
static size_t assign_layouts(std::vector<TcJob> &jobs, int NQ, int b0, int b1, std::vector<BankLayout> &layouts) {
  size_t total = 0;
  for (TcJob &J : jobs) {
    const BankLayout *hit = nullptr;
    for (const BankLayout &L : layouts)
      if (L.first == J.row0 && L.n == J.n) hit = &L;
    if (!hit) {
      layouts.push_back(BankLayout{J.row0, J.n, total});
      total += layout_bytes(NQ, b0, b1, J.n);
      hit = &layouts.back();
    }
    J.bank_off = (int)hit->off;
  }
  return total;
}

// ---------------------------------------------------------------------------
// host: chunks (tile runs) of the jobs for a tile shape
// ---------------------------------------------------------------------------
struct TcShape {
  int t_cap;        // tiles per CTA, at most
  size_t budget;    // dynamic shared memory per CTA, at most
  int stages;       // bank stages in the ring
  int col;          // a stage holds -1: every tap of a phase (the bank resident), 1: a filter column, 0: one tap
};
static const TcShape kTcShapes[] = {{4, 110 * 1024, 2, 1},  {2, 72 * 1024, 3, 0},  {4, 220 * 1024, 1, -1},
                                    {2, 220 * 1024, 1, -1}, {8, 220 * 1024, 1, -1}, {2, 110 * 1024, 1, -1},
                                    {1, 72 * 1024, 4, 0},   {4, 220 * 1024, 8, 0},  {4, 110 * 1024, 8, 0},
                                    {4, 110 * 1024, 4, 0}};
constexpr int kTcNumShapes = (int)(sizeof(kTcShapes) / sizeof(kTcShapes[0]));

// taps a stage holds for a phase of cs columns: one, a column (b0), or the whole phase
static int taps_per_stage(const TcJob &J, const TcShape &sh, int cs) {
  return sh.col < 0 ? cs * J.b0 : sh.col ? J.b0 : 1;
}
static int tps_arg(const TcShape &sh) { return sh.col < 0 ? -1 : sh.col ? 0 : 1; }

static size_t tc_need(const TcJob &J, int NQ, int T, int cs, const TcShape &sh) {
  const size_t S = (size_t)T * kTcM + (size_t)(cs - 1) * J.fs0 + (J.b0 - 1);
  const size_t slab = kTcHead + kTcColBytes + (size_t)NQ * S * 16 * (J.n_lo > 0 ? 2 : 1);
  return ((slab + 127) & ~(size_t)127) + (size_t)sh.stages * taps_per_stage(J, sh, cs) * NQ * J.n * 16;
}

static int tmem_cols(int c) {
  int n = 32;
  while (n < c) n <<= 1;
  return n;
}

// chunks of every job for a shape; false when a job fits no CTA or a slab would
// read past the planes' buffer (cells_total cells of 16 B)
static bool chunk_jobs(const std::vector<TcJob> &jobs, int NQ, const TcShape &sh, long long cells_total,
                       std::vector<int4> &chunks, size_t &max_smem) {
  chunks.clear();
  max_smem = 0;
  for (size_t j = 0; j < jobs.size(); j++) {
    const TcJob &J = jobs[j];
    const int t_max = std::max(1, std::min(sh.t_cap, kTcTmemCols / J.n));
    int T = 0, cs = 0;
    for (int Tc = t_max; Tc >= 1 && !T; Tc--)
      if (tc_need(J, NQ, Tc, J.b1, sh) <= sh.budget) { T = Tc; cs = J.b1; }
    for (int c = J.b1 - 1; c >= 1 && !T; c--)
      if (tc_need(J, NQ, 1, c, sh) <= sh.budget) { T = 1; cs = c; }
    if (!T) return false;
    // the CTAs that share an SM (by shared memory) fit their accumulators in its
    // 512 TMEM columns together, or one's allocation waits for another to end
    auto per_sm = [&](int Tc) { return std::max<size_t>(1, (228u * 1024u) / (tc_need(J, NQ, Tc, cs, sh) + 1024)); };
    while (T > 1 && (size_t)tmem_cols(T * J.n) * per_sm(T) > (size_t)kTcTmemCols) T--;
    const long long reach = (long long)(J.b1 - 1) * J.fs0 + (J.b0 - 1);
    for (int t0 = 0; t0 < J.ntiles; t0 += T) {
      const int nt = std::min(T, J.ntiles - t0);
      const long long last = (long long)(NQ - 1) * J.plane_cells + (long long)t0 * kTcM + (long long)nt * kTcM + reach;
      if ((long long)J.plane_off * 2 / 16 + last > cells_total) return false;
      if (J.lo_off >= 0 && (long long)J.lo_off * 2 / 16 + last > cells_total) return false;
      chunks.push_back(make_int4((int)j, t0, nt, cs));
      max_smem = std::max(max_smem, tc_need(J, NQ, nt, cs, sh));
    }
  }
  // heaviest first (tiles x taps x N), so the long ones start in the first wave
  auto cost = [&](const int4 &c) {
    const TcJob &J = jobs[c.x];
    return (long long)c.z * J.b0 * J.b1 * (J.n + 2 * J.n_lo);
  };
  std::stable_sort(chunks.begin(), chunks.end(), [&](const int4 &x, const int4 &y) { return cost(x) > cost(y); });
  return true;
}

// tps: taps per stage for every job of the launch (> 0 that many, 0: a filter column, < 0: a whole phase)
static void launch_conv_tc(int NQ, const TcJob *jobs, const int4 *chunks, int n_chunks, const TcCol *cols,
                           const uint8_t *planes, const uint8_t *bank, int stages, int tps, float *out, int *err,
                           size_t smem, cudaStream_t s) {
  if (n_chunks <= 0) return;
  if (NQ == 4) {
    static SmemAttr a4;
    raise_smem(a4, k_conv_tc<4>, smem);
    k_conv_tc<4><<<n_chunks, kTcThreads, smem, s>>>(jobs, chunks, cols, planes, bank, stages, tps, out, err);
  } else {
    static SmemAttr a2;
    raise_smem(a2, k_conv_tc<2>, smem);
    k_conv_tc<2><<<n_chunks, kTcThreads, smem, s>>>(jobs, chunks, cols, planes, bank, stages, tps, out, err);
  }
}

// ---------------------------------------------------------------------------
// host: units and CTA ranges of the persistent form
// ---------------------------------------------------------------------------
struct TcpLayout {
  std::vector<int4> units;   // (job, first tile, tiles, flags: 1 = the slab takes both buffers)
  std::vector<int4> ctas;    // per CTA: first unit, end unit, bank region bytes, slab buffer bytes
  uint32_t colbuf = 0;
  size_t smem = 0;
};
constexpr size_t kTcpSmemMax = 227 * 1024;

static size_t tcp_slab_bytes(const TcJob &J, int NQ, int T) {
  const size_t S = (size_t)T * kTcM + (size_t)(J.b1 - 1) * J.fs0 + (J.b0 - 1);
  return ((size_t)NQ * S * 16 * (J.n_lo > 0 ? 2 : 1) + 127) & ~(size_t)127;
}

// Units bank by bank; each bank's units get a share of the CTAs in proportion to
// their cost (no CTA holds two banks), and each CTA's shared memory is carved for
// its bank.  False when a job's bank and its slab do not fit one CTA, or a slab
// would read past the planes' buffer (cells_total cells of 16 B).
static bool tcp_layout(const std::vector<TcJob> &jobs, int NQ, int ctas, long long cells_total, TcpLayout &L) {
  L = TcpLayout{};
  if (jobs.empty() || ctas <= 0) return false;
  std::vector<int> banks;   // distinct bank offsets, ascending
  for (const TcJob &J : jobs) banks.push_back(J.bank_off);
  std::sort(banks.begin(), banks.end());
  banks.erase(std::unique(banks.begin(), banks.end()), banks.end());
  struct Group {
    int u0 = 0, u1 = 0;
    size_t bank = 0, half = 0;
    long long cost = 0;
    int ctas = 0;
  };
  std::vector<Group> G(banks.size());
  std::vector<long long> cost;
  int cmax = 0;
  for (size_t g = 0; g < banks.size(); g++) {
    Group &gr = G[g];
    std::vector<int> js;
    for (size_t j = 0; j < jobs.size(); j++)
      if (jobs[j].bank_off == banks[g]) js.push_back((int)j);
    const TcJob &J0 = jobs[js[0]];
    gr.bank = ((size_t)J0.b0 * J0.b1 * NQ * J0.n * 16 + 127) & ~(size_t)127;
    if (kTcpHead + gr.bank >= kTcpSmemMax) return false;
    const size_t half_cap = ((kTcpSmemMax - kTcpHead - gr.bank) / 2) & ~(size_t)127;
    size_t whole = 0;
    gr.u0 = (int)L.units.size();
    for (int j : js) {
      const TcJob &J = jobs[j];
      int t = std::max(1, std::min(kTcpTiles, 128 / std::max(1, J.n)));   // a unit's accumulators: t*n <= 128 columns
      while (t > 1 && tcp_slab_bytes(J, NQ, t) > half_cap) t--;
      int big = 0;
      if (tcp_slab_bytes(J, NQ, t) <= half_cap) {
        gr.half = std::max(gr.half, tcp_slab_bytes(J, NQ, t));
      } else if (tcp_slab_bytes(J, NQ, 1) <= 2 * half_cap) {
        big = 1;
        whole = std::max(whole, tcp_slab_bytes(J, NQ, 1));
      } else {
        return false;
      }
      cmax = std::max(cmax, t * J.n);
      const long long reach = (long long)(J.b1 - 1) * J.fs0 + (J.b0 - 1);
      const int taps = J.b0 * J.b1;
      for (int t0 = 0; t0 < J.ntiles; t0 += t) {
        const int nt = std::min(t, J.ntiles - t0);
        const long long last = (long long)(NQ - 1) * J.plane_cells + (long long)(t0 + nt) * kTcM + reach;
        if ((long long)J.plane_off * 2 / 16 + last > cells_total) return false;
        if (J.lo_off >= 0 && (long long)J.lo_off * 2 / 16 + last > cells_total) return false;
        L.units.push_back(make_int4(j, t0, nt, big));
        // MMA columns of the unit, and a fixed share for its slab and epilogue
        const long long c = (long long)nt * taps * (J.n + 2 * J.n_lo) + (long long)taps * 64;
        cost.push_back(c);
        gr.cost += c;
      }
    }
    gr.u1 = (int)L.units.size();
    gr.half = std::max(gr.half, (((whole + 1) / 2) + 127) & ~(size_t)127);
    if (kTcpHead + gr.bank + 2 * gr.half > kTcpSmemMax) return false;
    L.smem = std::max(L.smem, kTcpHead + gr.bank + 2 * gr.half);
  }
  uint32_t colbuf = 32;
  while ((int)colbuf < cmax) colbuf <<= 1;
  if (2 * colbuf > (uint32_t)kTcTmemCols) return false;
  L.colbuf = colbuf;
  // CTAs per bank in proportion to cost, at least one, at most its units
  long long total = 0;
  int free_ctas = ctas;
  for (Group &gr : G) total += gr.cost, free_ctas -= 1, gr.ctas = 1;
  if (free_ctas < 0) return false;
  for (Group &gr : G) {
    const int extra = (int)((double)free_ctas * (double)gr.cost / (double)std::max(1LL, total));
    gr.ctas = std::min(gr.u1 - gr.u0, 1 + extra);
  }
  // units of a bank in ranges of about equal cost, none empty
  for (const Group &gr : G) {
    const int nu = gr.u1 - gr.u0, C = std::max(1, std::min(gr.ctas, nu));
    std::vector<long long> prefix(nu + 1, 0);
    for (int u = 0; u < nu; u++) prefix[u + 1] = prefix[u] + cost[gr.u0 + u];
    int prev = 0;
    for (int c = 1, u = 0; c <= C; c++) {
      int end = nu;
      if (c < C) {
        while (u < nu && prefix[u] * C < prefix[nu] * c) u++;
        end = std::min(std::max(u, prev + 1), nu - (C - c));
      }
      L.ctas.push_back(make_int4(gr.u0 + prev, gr.u0 + end, (int)gr.bank, (int)gr.half));
      prev = end;
    }
  }
  return !L.ctas.empty();
}

static void launch_conv_tcp(int NQ, const TcJob *jobs, const int4 *units, const int4 *ctainfo, int ctas,
                            const TcCol *cols, const uint8_t *planes, const uint8_t *bank, uint32_t colbuf,
                            float *out, int *err, size_t smem, cudaStream_t s) {
  if (ctas <= 0) return;
  if (NQ == 4) {
    static SmemAttr a4;
    raise_smem(a4, k_conv_tcp<4>, smem);
    k_conv_tcp<4><<<ctas, kTcpThreads, smem, s>>>(jobs, units, ctainfo, cols, planes, bank, colbuf, out, err);
  } else {
    static SmemAttr a2;
    raise_smem(a2, k_conv_tcp<2>, smem);
    k_conv_tcp<2><<<ctas, kTcpThreads, smem, s>>>(jobs, units, ctainfo, cols, planes, bank, colbuf, out, err);
  }
}

// ---------------------------------------------------------------------------
// host: the plan's bank, jobs, column tables and root sums
// ---------------------------------------------------------------------------
// Before the arena is allocated: the rows (every model's part filters, then its
// root filters cut into blocks of the part grid, then in BF16 mode the blocks'
// remainders), one job per feature level over the rows it uses, the blocks'
// position-indexed buffers (taken from the arena) and the root sums.
geye_status plan_tc(geye_ctx *ctx, Plan &P, ArenaAlloc &A) {
  TcPlan &T = P.tc;   // a fresh plan's (default-constructed)
  const geye_conv_mode mode = ctx->conv_mode;
  const bool split = mode == GEYE_CONV_BF16;
  T.planes = tc_planes_of(mode);
  int gb0 = 0, gb1 = 0;
  for (auto &mp : P.models) {
    const HostModel &h = mp->model->h;
    for (int p = 0; p < h.NoP; p++) { gb0 = std::max(gb0, h.part_size[3 * p]); gb1 = std::max(gb1, h.part_size[3 * p + 1]); }
  }
  if (!gb0 || !gb1)   // no parts anywhere: one block per root
    for (auto &mp : P.models) {
      const HostModel &h = mp->model->h;
      for (int r = 0; r < h.NoR; r++) { gb0 = std::max(gb0, h.root_size[3 * r]); gb1 = std::max(gb1, h.root_size[3 * r + 1]); }
    }
  T.grid_b0 = gb0;
  T.grid_b1 = gb1;
  // rows
  struct PartRow { int mi, p; };
  struct RootRow { int mi, c, y0, x0; };
  std::vector<PartRow> parts;
  std::vector<RootRow> roots;
  for (int mi = 0; mi < (int)P.models.size(); mi++) {
    const HostModel &h = P.models[mi]->model->h;
    for (int p = 0; p < h.NoP; p++) parts.push_back({mi, p});
  }
  for (int mi = 0; mi < (int)P.models.size(); mi++) {
    const HostModel &h = P.models[mi]->model->h;
    for (int c = 0; c < h.numcomponent; c++) {
      const int rb0 = h.root_size[3 * c], rb1 = h.root_size[3 * c + 1];
      const int na = (rb1 + gb1 - 1) / gb1, nb = (rb0 + gb0 - 1) / gb0;
      if (na * nb > kMaxRootBlocks) {
        set_error("tensor-core conv: a root filter needs more than 16 blocks of the part grid");
        return GEYE_ERR_UNSUPPORTED;
      }
      for (int a = 0; a < na; a++)
        for (int b = 0; b < nb; b++) roots.push_back({mi, c, b * gb0, a * gb1});
    }
  }
  const int p16 = pad16((int)parts.size()), r16 = pad16((int)roots.size());
  const int RS = r16 * (split ? 2 : 1);
  if (p16 > kTcMaxN || RS > kTcMaxN) {
    set_error("tensor-core conv: more than 256 filter rows in one section");
    return GEYE_ERR_UNSUPPORTED;
  }
  T.rows = p16 + RS;
  T.rows_p16 = p16;
  T.rows_r16 = r16;
  // host bank rows (filters and FP8 scales)
  T.bank_rows.assign(T.rows, BankRowSpec{});
  std::map<std::pair<int, int>, float> root_scale;
  for (size_t j = 0; j < parts.size(); j++) {
    geye_model *m = P.models[parts[j].mi]->model;
    T.bank_rows[j] = BankRowSpec{parts[j].mi, m->h.NoR + parts[j].p, 0, 0, 0};
  }
  for (size_t j = 0; j < roots.size(); j++) {
    T.bank_rows[p16 + j] = BankRowSpec{roots[j].mi, roots[j].c, roots[j].y0, roots[j].x0, 0};
    if (split) T.bank_rows[p16 + r16 + j] = BankRowSpec{roots[j].mi, roots[j].c, roots[j].y0, roots[j].x0, 1};
  }
  auto filt_scale = [&](int mi, int f) {
    if (mode != GEYE_CONV_FP8) return 1.f;
    const HostModel &h = P.models[mi]->model->h;
    const bool root = f < h.NoR;
    const std::vector<float> &w = root ? h.rootfilter[f] : h.partfilter[f - h.NoR];
    return e4m3_filter_scale(w.data(), w.size());
  };
  for (auto &b : T.bank_rows)
    if (b.mi >= 0) b.scale = filt_scale(b.mi, b.filt);
  // jobs per feature level
  const int interval = P.interval;
  for (int l = 0; l < P.LEN; l++) {
    const LevelInfo &L = P.lv[l];
    if (L.feat16_off < 0 || L.fs0 <= 0 || L.fs1 <= 0) continue;
    std::vector<int> part_on(parts.size(), 0), root_on(roots.size(), 0);
    bool any_p = false, any_r = false;
    for (size_t j = 0; j < parts.size(); j++) {
      const ModelPlan &mp = *P.models[parts[j].mi];
      const int NoP = mp.model->h.NoP;
      const size_t i = (size_t)l * NoP + parts[j].p;
      if (i < mp.part_map_off.size() && mp.part_map_off[i] >= 0) { part_on[j] = 1; any_p = true; }
    }
    for (size_t j = 0; j < roots.size(); j++) {
      const ModelPlan &mp = *P.models[roots[j].mi];
      const size_t i = (size_t)l * mp.model->h.numcomponent + roots[j].c;
      if (l >= interval && l < mp.LEN && i < mp.root_map_off.size() && mp.root_map_off[i] >= 0) {
        root_on[j] = 1;
        any_r = true;
      }
    }
    if (!any_p && !any_r) continue;
    const int ncell = L.fs0 * L.fs1;
    std::vector<int> block_off(roots.size(), -1);
    for (size_t j = 0; j < roots.size(); j++)
      if (root_on[j]) block_off[j] = A.take((size_t)ncell);
    // root sums: each root present at this level from its blocks
    for (int mi = 0; mi < (int)P.models.size(); mi++) {
      const ModelPlan &mp = *P.models[mi];
      const int NoC = mp.model->h.numcomponent;
      for (int c = 0; c < NoC; c++) {
        RootSumJob S{};
        for (size_t j = 0; j < roots.size(); j++) {
          if (roots[j].mi != mi || roots[j].c != c || !root_on[j]) continue;
          S.blk[S.nblk] = block_off[j];
          S.shift[S.nblk] = roots[j].x0 * L.fs0 + roots[j].y0;
          S.nblk++;
        }
        if (!S.nblk) continue;
        S.out_off = mp.root_map_off[(size_t)l * NoC + c];
        S.r0 = mp.root_r0[(size_t)l * NoC + c];
        S.r1 = mp.root_r1[(size_t)l * NoC + c];
        S.fs0 = L.fs0;
        T.sums.push_back(S);
        T.sum_max_r = std::max(T.sum_max_r, S.r0 * S.r1);
      }
    }
    auto add_job = [&](int row0, int n, int lo_row, int n_lo, bool with_roots) {
      TcJob J{};
      J.plane_off = L.feat16_off;
      J.lo_off = n_lo ? L.feat16lo_off : -1;
      J.plane_cells = ncell + kTcPlanePad;
      J.fs0 = L.fs0; J.fs1 = L.fs1;
      J.b0 = gb0; J.b1 = gb1;
      J.row0 = row0; J.n = n;
      J.lo_row = lo_row; J.n_lo = n_lo;
      J.col_tab = (int)T.cols.size();
      int p_valid = 0;
      for (int k = 0; k < n; k++) {
        const int row = row0 + k;
        TcCol C{};
        C.inv = 1.f;
        if (row < p16) {
          if (row < (int)parts.size() && part_on[row]) {
            const ModelPlan &mp = *P.models[parts[row].mi];
            const size_t i = (size_t)l * mp.model->h.NoP + parts[row].p;
            C.kind = 1;
            C.off = mp.part_map_off[i];
            C.rows = mp.part_d0[i];
            C.cols = mp.part_d1[i];
            C.inv = 1.f / (T.bank_rows[row].scale * (mode == GEYE_CONV_FP8 ? kFp8FeatScale : 1.f));
            p_valid = std::max(p_valid, (C.cols - 1) * L.fs0 + C.rows);
          }
        } else if (row < p16 + r16) {
          const int j = row - p16;
          if (j < (int)roots.size() && root_on[j]) {
            C.kind = 2;
            C.off = block_off[j];
            C.pair = split ? r16 : 0;
            C.inv = 1.f / (T.bank_rows[row].scale * (mode == GEYE_CONV_FP8 ? kFp8FeatScale : 1.f));
          }
        }
        T.cols.push_back(C);
      }
      J.ntiles = ((with_roots ? ncell : p_valid) + kTcM - 1) / kTcM;
      if (J.ntiles > 0) T.jobs.push_back(J);
    };
    // parts and root blocks as separate jobs, so each job's bank can stay resident in
    // shared memory (the part filters' bank alone, the root blocks' with its remainders)
    const int n_lo = split ? r16 : 0;
    if (any_p) add_job(0, p16, 0, 0, false);
    if (any_r) add_job(p16, RS, 0, n_lo, true);
  }
  return GEYE_OK;
}

// After the arena exists: the bank, then the tile-shape autotuner (every candidate
// is chunked, timed on the plan's own arena with CUDA events after one untimed
// launch, and the fastest kept; the choice is cached per models and geometry),
// then the tables.
geye_status build_tc_plan(geye_ctx *ctx, Plan &P) {
  TcPlan &T = P.tc;
  if (!P.arena16.p || T.jobs.empty()) return GEYE_OK;
  const int NQ = T.planes;
  // the bank
  std::vector<BankRow> rows(T.rows);
  for (int r = 0; r < T.rows; r++) {
    const BankRowSpec &b = T.bank_rows[r];
    if (b.mi < 0) continue;
    geye_model *m = P.models[b.mi]->model;
    const HostModel &h = m->h;
    const bool root = b.filt < h.NoR;
    BankRow R;
    R.h = root ? h.rootfilter[b.filt].data() : h.partfilter[b.filt - h.NoR].data();
    R.d = m->d_filters + m->filt_off[b.filt];
    R.fb0 = root ? h.root_size[3 * b.filt] : h.part_size[3 * (b.filt - h.NoR)];
    R.fb1 = root ? h.root_size[3 * b.filt + 1] : h.part_size[3 * (b.filt - h.NoR) + 1];
    R.y0 = b.y0;
    R.x0 = b.x0;
    R.lo = b.lo;
    R.scale = b.scale;
    rows[r] = R;
  }
  std::vector<BankLayout> layouts;
  const size_t bank_total = assign_layouts(T.jobs, NQ, T.grid_b0, T.grid_b1, layouts);
  GEYE_TRY(upload_bank(ctx, rows, NQ, T.grid_b0, T.grid_b1, layouts, bank_total, T.d_bank));
  GEYE_TRY(upload_bytes(ctx, T.d_jobs, T.jobs.data(), sizeof(TcJob) * T.jobs.size()));
  GEYE_TRY(upload_bytes(ctx, T.d_cols, T.cols.data(), sizeof(TcCol) * std::max<size_t>(T.cols.size(), 1)));
  GEYE_TRY(upload_bytes(ctx, T.d_sums, T.sums.data(), sizeof(RootSumJob) * std::max<size_t>(T.sums.size(), 1)));
  const long long cells_total = (long long)(P.arena16.bytes / 16);
  int *err = P.d_small.as<int>() + 130;
  // a geometry these models were tuned at before reuses that choice
  std::string key = std::to_string(P.width) + "x" + std::to_string(P.height) + "/" + std::to_string(P.LEN) + "/" +
                    std::to_string((int)ctx->conv_mode);
  for (auto &mp : P.models) key += ":" + std::to_string(mp->model->id);
  geye_model *m0 = P.models[0]->model;
  int first = 0, last = kTcNumShapes + 1;   // the tile shapes, then the persistent form
  float best_ms = 0.f;
  {
    std::lock_guard<std::mutex> lk(m0->tc_mu);
    auto it = m0->tc_tuned.find(key);
    if (it != m0->tc_tuned.end()) { first = it->second.first; last = first + 1; best_ms = 3.0f * it->second.second; }
  }
  // GEYE_TC_SHAPE=<i> pins candidate i (reproducible shapes; no timing)
  if (const char *e = getenv("GEYE_TC_SHAPE")) {
    const int i = atoi(e);
    if (i >= 0 && i <= kTcNumShapes) { first = i; last = i + 1; }
  }
  const bool timed = last - first > 1;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (timed) {
    CUDA_TRY(cudaEventCreate(&e0));
    CUDA_TRY(cudaEventCreate(&e1));
  }
  std::vector<int4> best;
  size_t best_smem = 0;
  int best_shape = -1;
  int sms = 0;
  CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
  for (int si = first; si < last; si++) {
    if (si == kTcNumShapes) {
      TcpLayout L;
      if (!tcp_layout(T.jobs, NQ, sms, cells_total, L)) continue;
      DevBuf d_units, d_ranges;
      GEYE_TRY(upload_bytes(ctx, d_units, L.units.data(), sizeof(int4) * L.units.size()));
      GEYE_TRY(upload_bytes(ctx, d_ranges, L.ctas.data(), sizeof(int4) * L.ctas.size()));
      const int ctas = (int)L.ctas.size();
      auto launch = [&]() {
        launch_conv_tcp(NQ, T.d_jobs.as<TcJob>(), d_units.as<int4>(), d_ranges.as<int4>(), ctas, T.d_cols.as<TcCol>(),
                        P.arena16.as<uint8_t>(), T.d_bank.as<uint8_t>(), L.colbuf, P.arena.as<float>(), err, L.smem,
                        ctx->stream);
      };
      float ms = 0.f;
      if (timed) {
        launch();
        CUDA_TRY(cudaEventRecord(e0, ctx->stream));
        for (int r = 0; r < 3; r++) launch();
        CUDA_TRY(cudaEventRecord(e1, ctx->stream));
        CUDA_TRY(cudaEventSynchronize(e1));
        CUDA_TRY(cudaGetLastError());
        CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
      }
      if (!timed || best_shape < 0 || ms < best_ms) {
        best.clear();
        best_smem = L.smem;
        best_shape = si;
        best_ms = ms;
        // the plan takes the candidate's buffers (its previous ones are freed with the candidate's)
        std::swap(T.d_units.p, d_units.p);
        std::swap(T.d_units.bytes, d_units.bytes);
        std::swap(T.d_ranges.p, d_ranges.p);
        std::swap(T.d_ranges.bytes, d_ranges.bytes);
        T.tcp_ctas = ctas;
        T.tcp_colbuf = L.colbuf;
      }
      if (!timed) break;
      continue;
    }
    std::vector<int4> chunks;
    size_t smem = 0;
    if (!chunk_jobs(T.jobs, NQ, kTcShapes[si], cells_total, chunks, smem)) continue;
    if (!timed) {
      best = std::move(chunks);
      best_smem = smem;
      best_shape = si;
      break;
    }
    DevBuf d_chunks;
    GEYE_TRY(upload_bytes(ctx, d_chunks, chunks.data(), sizeof(int4) * chunks.size()));
    auto launch = [&]() {
      launch_conv_tc(NQ, T.d_jobs.as<TcJob>(), d_chunks.as<int4>(), (int)chunks.size(), T.d_cols.as<TcCol>(),
                     P.arena16.as<uint8_t>(), T.d_bank.as<uint8_t>(), kTcShapes[si].stages,
                     tps_arg(kTcShapes[si]), P.arena.as<float>(), err, smem, ctx->stream);
    };
    launch();
    CUDA_TRY(cudaEventRecord(e0, ctx->stream));
    for (int r = 0; r < 3; r++) launch();
    CUDA_TRY(cudaEventRecord(e1, ctx->stream));
    CUDA_TRY(cudaEventSynchronize(e1));
    CUDA_TRY(cudaGetLastError());
    float ms = 0.f;
    CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
    if (best_shape < 0 || ms < best_ms) {
      best = std::move(chunks);
      best_smem = smem;
      best_shape = si;
      best_ms = ms;
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (timed) CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), ctx->stream));
  if (best_shape < 0) {
    set_error("tensor-core conv: a level's slab and bank stages exceed shared memory or the planes' buffer");
    return GEYE_ERR_UNSUPPORTED;
  }
  if (timed) {
    std::lock_guard<std::mutex> lk(m0->tc_mu);
    m0->tc_tuned[key] = {best_shape, best_ms / 3.0f};
  }
  T.smem = best_smem;
  T.n_chunks = (int)best.size();
  T.shape = best_shape;
  if (best_shape < kTcNumShapes) {
    T.stages = kTcShapes[best_shape].stages;
    T.tps = tps_arg(kTcShapes[best_shape]);
    T.d_units.release();
    T.d_ranges.release();
    T.tcp_ctas = 0;
  }
  T.tuned_ms = best_ms / 3.0f;
  if (!best.empty()) GEYE_TRY(upload_bytes(ctx, T.d_chunks, best.data(), sizeof(int4) * best.size()));
  return GEYE_OK;
}

geye_status run_conv_tc(geye_ctx *ctx, Plan &P) {
  const TcPlan &T = P.tc;
  if (!P.arena16.p) {
    set_error("tensor-core conv: the plan has no feature planes");
    return GEYE_ERR_UNSUPPORTED;
  }
  if (T.shape == kTcNumShapes) {
    launch_conv_tcp(T.planes, T.d_jobs.as<TcJob>(), T.d_units.as<int4>(), T.d_ranges.as<int4>(), T.tcp_ctas,
                    T.d_cols.as<TcCol>(), P.arena16.as<uint8_t>(), T.d_bank.as<uint8_t>(), T.tcp_colbuf,
                    P.arena.as<float>(), P.d_small.as<int>() + 130, T.smem, ctx->stream);
  } else {
    if (T.n_chunks == 0) return GEYE_OK;
    launch_conv_tc(T.planes, T.d_jobs.as<TcJob>(), T.d_chunks.as<int4>(), T.n_chunks, T.d_cols.as<TcCol>(),
                   P.arena16.as<uint8_t>(), T.d_bank.as<uint8_t>(), T.stages, T.tps, P.arena.as<float>(),
                   P.d_small.as<int>() + 130, T.smem, ctx->stream);
  }
  ctx->launches++;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && !T.sums.empty()) {
    dim3 g((T.sum_max_r + 255) / 256, (unsigned)T.sums.size());
    k_root_sum<<<g, 256, 0, ctx->stream>>>(T.d_sums.as<RootSumJob>(), P.arena.as<float>());
    ctx->launches++;
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) {
    set_error(std::string("tensor-core conv: ") + cudaGetErrorString(e));
    return GEYE_ERR_CUDA;
  }
  return GEYE_OK;
}

// fconvsMT on the tensor cores for the stage entry point (the context's conv
// mode): d_feat is [pos][32] float on the device (a0 x a1 cells), filters on
// the host; maps go to d_out + out_off[i].  One job: every filter a row of one
// bank over the largest filter's grid.  Temporary device buffers live in tmp.
geye_status conv_tc_maps(geye_ctx *ctx, const float *d_feat, int a0, int a1, const float *const *filters,
                         const int *b_dims, int n_filters, float *d_out, const std::vector<int> &out_off,
                         std::vector<std::unique_ptr<DevBuf>> &tmp) {
  const geye_conv_mode mode = ctx->conv_mode;
  const int NQ = tc_planes_of(mode);
  auto buf = [&]() { tmp.push_back(std::make_unique<DevBuf>()); return tmp.back().get(); };
  int gb0 = 1, gb1 = 1;
  for (int i = 0; i < n_filters; i++) { gb0 = std::max(gb0, b_dims[2 * i]); gb1 = std::max(gb1, b_dims[2 * i + 1]); }
  const int R = pad16(n_filters);
  if (R > kTcMaxN) {
    set_error("tensor-core conv: more than 256 filters in one call");
    return GEYE_ERR_UNSUPPORTED;
  }
  std::vector<BankRow> rows(R);
  std::vector<TcCol> cols(R);
  int p_valid = 0;
  for (int i = 0; i < n_filters; i++) {
    const int fb0 = b_dims[2 * i], fb1 = b_dims[2 * i + 1];
    const size_t n = (size_t)fb0 * fb1 * kFeat;
    DevBuf *f = buf();
    GEYE_TRY(upload_bytes(ctx, *f, filters[i], sizeof(float) * n));
    BankRow &B = rows[i];
    B.h = filters[i];
    B.d = f->as<float>();
    B.fb0 = fb0;
    B.fb1 = fb1;
    B.scale = mode == GEYE_CONV_FP8 ? e4m3_filter_scale(filters[i], n) : 1.f;
    TcCol &C = cols[i];
    C.rows = a0 - fb0 + 1;
    C.cols = a1 - fb1 + 1;
    if (C.rows < 1 || C.cols < 1) continue;   // no map for a filter larger than the level
    C.kind = 1;
    C.off = out_off[i];
    C.inv = 1.f / (B.scale * (mode == GEYE_CONV_FP8 ? kFp8FeatScale : 1.f));
    p_valid = std::max(p_valid, (C.cols - 1) * a0 + C.rows);
  }
  if (p_valid == 0) return GEYE_OK;
  TcJob J{};
  J.plane_off = 0;
  J.lo_off = -1;
  J.plane_cells = a0 * a1 + kTcPlanePad;
  J.fs0 = a0; J.fs1 = a1;
  J.b0 = gb0; J.b1 = gb1;
  J.row0 = 0; J.n = R;
  J.ntiles = (p_valid + kTcM - 1) / kTcM;
  // planes, then a zeroed tail that slabs near the end may read (their outputs are discarded)
  const int ncell = a0 * a1;
  const size_t tail_cells = (size_t)gb1 * a0 + gb0 + (size_t)kTcMaxTiles * kTcM;
  const size_t plane_total = (size_t)NQ * (ncell + kTcPlanePad);
  std::vector<int4> chunks;
  size_t smem = 0;
  std::vector<TcJob> jobs{J};
  std::vector<BankLayout> layouts;
  const size_t bank_total = assign_layouts(jobs, NQ, gb0, gb1, layouts);
  int stages = 0, tps = 1;
  for (int si = 0; si < kTcNumShapes && !stages; si++)
    if (chunk_jobs(jobs, NQ, kTcShapes[si], (long long)(plane_total + tail_cells), chunks, smem)) {
      stages = kTcShapes[si].stages;
      tps = tps_arg(kTcShapes[si]);
    }
  if (!stages) {
    set_error("tensor-core conv: the filters' slab and bank stages exceed shared memory");
    return GEYE_ERR_UNSUPPORTED;
  }
  DevBuf *planes = buf(), *d_bank = buf(), *d_jobs = buf(), *d_chunks = buf(), *d_cols = buf(), *d_err = buf();
  GEYE_TRY(planes->alloc(ctx, (plane_total + tail_cells) * 16));
  CUDA_TRY(cudaMemsetAsync(planes->as<uint8_t>() + plane_total * 16, 0, tail_cells * 16, ctx->stream));
  GEYE_TRY(upload_bank(ctx, rows, NQ, gb0, gb1, layouts, bank_total, *d_bank));
  GEYE_TRY(upload_bytes(ctx, *d_jobs, jobs.data(), sizeof(TcJob)));
  GEYE_TRY(upload_bytes(ctx, *d_chunks, chunks.data(), sizeof(int4) * chunks.size()));
  GEYE_TRY(upload_bytes(ctx, *d_cols, cols.data(), sizeof(TcCol) * cols.size()));
  GEYE_TRY(d_err->alloc(ctx, 16));
  CUDA_TRY(cudaMemsetAsync(d_err->p, 0, 16, ctx->stream));
  const int grid = std::max(1, std::min((ncell + kTcPlanePad + 255) / 256, 1024));
  if (NQ == 4) k_feat_planes<4><<<grid, 256, 0, ctx->stream>>>(d_feat, ncell, planes->as<uint8_t>());
  else k_feat_planes<2><<<grid, 256, 0, ctx->stream>>>(d_feat, ncell, planes->as<uint8_t>());
  launch_conv_tc(NQ, d_jobs->as<TcJob>(), d_chunks->as<int4>(), (int)chunks.size(), d_cols->as<TcCol>(),
                 planes->as<uint8_t>(), d_bank->as<uint8_t>(), stages, tps, d_out, d_err->as<int>(), smem, ctx->stream);
  CUDA_TRY(cudaGetLastError());
  int errw = 0;
  CUDA_TRY(cudaMemcpyAsync(&errw, d_err->p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  if (errw) {
    set_error("tensor-core conv: a tensor-core wait ran out (error bits " + std::to_string(errw) + ")");
    return GEYE_ERR_TIMEOUT;
  }
  return GEYE_OK;
}

}  // namespace geye

geye_status geye_conv_tuning(geye_ctx *ctx, const geye_model *m, int shape[3], float *ms) {
  ARG_CHECK(ctx && m && shape && ms, "null argument");
  ARG_CHECK(ctx->last_plan, "no run yet");
  const geye::Plan &P = *ctx->last_plan;
  bool in_plan = false;
  for (auto &mp : P.models) in_plan |= mp->model == m;
  ARG_CHECK(in_plan, "the last run has no such model");
  ARG_CHECK(P.tc.shape >= 0, "the last run's plan has no tensor-core convolution");
  const bool persistent = P.tc.shape == geye::kTcNumShapes;
  shape[0] = persistent ? 0 : geye::kTcShapes[P.tc.shape].t_cap;
  shape[1] = (int)((persistent ? P.tc.smem : geye::kTcShapes[P.tc.shape].budget) / 1024);
  shape[2] = persistent ? P.tc.tcp_ctas : P.tc.n_chunks;
  *ms = P.tc.tuned_ms;
  return GEYE_OK;
}

geye_status geye_dt_tuning(geye_ctx *ctx, const geye_model *m, int *elems, float ms[3]) {
  ARG_CHECK(ctx && m && elems && ms, "null argument");
  ARG_CHECK(ctx->last_plan, "no run yet");
  for (auto &mp : ctx->last_plan->models)
    if (mp->model == m) {
      *elems = mp->dt_elems;
      for (int c = 0; c < 3; c++) ms[c] = mp->dt_ms[c];
      return GEYE_OK;
    }
  geye::set_error("the last run has no such model");
  return GEYE_ERR_ARG;
}
