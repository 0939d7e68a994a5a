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
// or 32 e4m3), so a tap is 2 MMAs in BF16 and 1 in FP8.  Positions whose
// window crosses a column edge are computed and discarded ((b0-1)/fs0 of the work).
//
// B (the filters) is precomputed per model as [tap][q][n][16 B] (N padded to 16
// or 32), one descriptor per (tap, plane pair) as well.  FP8 filters are scaled
// per filter by the power of two that brings their absolute maximum under 448;
// the epilogue multiplies by the exact inverse of both scales.
//
// A CTA (4 warps) owns a run of up to 16 tiles of 128 positions of one (level,
// filter group), each tile with its own TMEM accumulator.  The filter is walked
// in column phases whose bank columns and feature slab fit in shared memory:
// one thread bulk-copies them (cp.async.bulk, completion on an mbarrier); one
// thread per warp issues the MMAs of every fourth tile (each tile's chain from
// one thread, in order) and commits them to a second mbarrier that expects the
// four warps' commits; after the last
// phase the four warps read the accumulators with tcgen05.ld (warp w owns TMEM
// lanes 32w..32w+31) and write the maps in the reference layout.  Every
// mbarrier wait is bounded; a timeout sets an error bit and the CTA still
// waits (bounded) for its own copies and MMAs before it frees TMEM and leaves.
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

constexpr int kTcThreads = 128;
constexpr int kTcM = 128;                        // positions per tile (TMEM lanes)
constexpr int kTcMaxTiles = 16;                  // tiles per CTA, at most
constexpr size_t kTcSmemBudget = 220 * 1024;     // dynamic shared memory per CTA, at most
constexpr int kTcMaxN = 64;                      // filters per group, at most (N of an MMA)
constexpr int kTcHead = 1152;                    // barriers, TMEM address, map offsets, scales, map dims
constexpr int kTcTmemCols = 512;                 // tiles per CTA x n_pad, at most
constexpr unsigned long long kWaitNs = 1000000000ull;   // a wait gives up after 1 s (then 4 s for the drain)

struct TcJob {
  int plane_off;     // offset of plane 0 in arena16, in 2-byte units
  int plane_cells;   // cells per plane
  int fs0, fs1;      // feature rows, columns
  int b0, b1;        // filter rows, columns
  int c0, c1;        // output rows, columns computed (those of the group's smallest filter)
  int n, n_pad;      // filters; padded to 16 or 32
  int bank_off;      // byte offset of the group's bank in the model's bank buffer
  int out_tab;       // first entry of the job's map offsets
  int ntiles;        // 128-position tiles up to the last valid output
};

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
template <int NQ>
__global__ void __launch_bounds__(kTcThreads, 1) k_conv_tc(const TcJob *__restrict__ jobs, const int4 *__restrict__ chunks,
                                                           const int *__restrict__ outs,
                                                           const float *__restrict__ inv_scale,
                                                           const int2 *__restrict__ out_dims,
                                                           const uint8_t *__restrict__ arena16,
                                                           const uint8_t *__restrict__ bank, float *__restrict__ arena,
                                                           int *err) {
  extern __shared__ __align__(128) uint8_t sm[];
  uint64_t *bar_load = reinterpret_cast<uint64_t *>(sm);
  uint64_t *bar_mma = reinterpret_cast<uint64_t *>(sm + 8);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(sm + 16);
  int *out_s = reinterpret_cast<int *>(sm + 32);       // the job's map offsets (n <= kTcMaxN)
  float *scl_s = reinterpret_cast<float *>(sm + 288);   // and output scales
  int2 *dim_s = reinterpret_cast<int2 *>(sm + 544);     // and each map's rows, columns
  const int4 ch = chunks[blockIdx.x];
  const TcJob J = jobs[ch.x];
  const int tile0 = ch.y, ntile = ch.z, cs = ch.w;   // cs = filter columns per phase
  if (threadIdx.x < J.n) {
    out_s[threadIdx.x] = outs[J.out_tab + threadIdx.x];
    scl_s[threadIdx.x] = inv_scale[J.out_tab + threadIdx.x];
    dim_s[threadIdx.x] = out_dims[J.out_tab + threadIdx.x];
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int p_begin = tile0 * kTcM;
  const uint32_t bq = (uint32_t)J.n_pad * 16u;                 // one (tap, q) slice of the bank
  const uint32_t col_bytes = (uint32_t)J.b0 * NQ * bq;         // one filter column of the bank
  const uint32_t bank_room = ((uint32_t)cs * col_bytes + 127u) & ~127u;
  uint8_t *sB = sm + kTcHead;
  uint8_t *sA = sB + bank_room;
  // accumulators: tile i at TMEM columns i*n_pad .. i*n_pad + n_pad - 1
  uint32_t ncols = 32;
  while (ncols < (uint32_t)(ntile * J.n_pad)) ncols <<= 1;

  if (threadIdx.x == 0) {
    mbar_init(bar_load, 1);
    mbar_init(bar_mma, kTcThreads / 32);   // one commit per issuing warp
    mbar_fence_init();
  }
  if (warp == 0) tmem_alloc(tslot, ncols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;

  const uint32_t idesc = NQ == 4 ? idesc_bf16(kTcM, J.n_pad) : idesc_e4m3(kTcM, J.n_pad);
  const uint32_t sA_addr = smem_u32(sA), sB_addr = smem_u32(sB);
  const int phases = (J.b1 + cs - 1) / cs;
  bool ok = true;   // uniform across the CTA (every wait outcome is combined with __syncthreads_and)
  for (int ph = 0; ph < phases && ok; ph++) {
    const int xp0 = ph * cs, ncol = min(cs, J.b1 - xp0);
    const int S = ntile * kTcM + (ncol - 1) * J.fs0 + (J.b0 - 1);   // slab cells per plane this phase
    const uint32_t plane_bytes = (uint32_t)S * 16u;
    if (threadIdx.x == 0) {
      mbar_expect_tx(bar_load, (uint32_t)ncol * col_bytes + NQ * plane_bytes);
      bulk_g2s(sB, bank + J.bank_off + (size_t)xp0 * col_bytes, (uint32_t)ncol * col_bytes, bar_load);
      for (int q = 0; q < NQ; q++)
        bulk_g2s(sA + (size_t)q * plane_bytes,
                 arena16 + 2 * (size_t)J.plane_off +
                     ((size_t)q * J.plane_cells + (size_t)p_begin + (size_t)xp0 * J.fs0) * 16,
                 plane_bytes, bar_load);
    }
    bool landed = mbar_wait(bar_load, (uint32_t)(ph & 1), kWaitNs);
    if (!landed) {
      atomicOr(err, 1);
      mbar_wait(bar_load, (uint32_t)(ph & 1), 4 * kWaitNs);   // the copies must land before the CTA leaves
    }
    ok = __syncthreads_and(landed);
    if (!ok) break;
    if (lane == 0) {   // one issuing thread per warp: tiles warp, warp + 4, ... (each tile's chain in order)
      tc_fence_after();
      // The start-address field of a descriptor is (address >> 4) in its low 14 bits and
      // every operand lies below 2^18 bytes, so moving an operand by a 16-byte multiple off
      // is adding off >> 4 to the descriptor: A moves by cells (16 B), B by (tap, q) slices.
      const uint64_t a_base = sdesc(sA_addr, plane_bytes, 128u);
      const uint64_t b_base = sdesc(sB_addr, bq, 128u);
      const uint32_t a_hi = 2u * (uint32_t)S;           // planes 2, 3: 2 * plane_bytes >> 4
      const uint32_t b_tap = NQ * (uint32_t)J.n_pad;    // one tap of the bank: NQ * bq >> 4
      const uint32_t b_hi = 2u * (uint32_t)J.n_pad;     // planes 2, 3 of a tap
      for (int i = warp; i < ntile; i += kTcThreads / 32) {
        const uint32_t d = tmem + (uint32_t)(i * J.n_pad);
        uint32_t acc = ph ? 1u : 0u;
        for (int xp = 0; xp < ncol; xp++) {
          const uint32_t cell0 = (uint32_t)(i * kTcM + xp * J.fs0);
          const uint32_t tap0 = (uint32_t)(xp * J.b0) * b_tap;
          for (int yp = 0; yp < J.b0; yp++) {
            const uint64_t ad = a_base + (cell0 + (uint32_t)yp);
            const uint64_t bd = b_base + (tap0 + (uint32_t)yp * b_tap);
            tc_mma<NQ>(d, ad, bd, idesc, acc);
            if constexpr (NQ == 4) tc_mma<NQ>(d, ad + a_hi, bd + b_hi, idesc, 1u);
            acc = 1u;
          }
        }
      }
      tc_commit(bar_mma);   // tracks this thread's MMAs (an immediate arrive if it issued none)
    }
    bool done = mbar_wait(bar_mma, (uint32_t)(ph & 1), kWaitNs);
    if (!done) {
      atomicOr(err, 2);
      mbar_wait(bar_mma, (uint32_t)(ph & 1), 4 * kWaitNs);   // the MMAs must finish before smem or TMEM is reused
    }
    ok = __syncthreads_and(done);
  }
  tc_fence_after();
  // epilogue: row r of a tile is TMEM lane r; this thread owns row 32*warp + lane of every tile
  for (int i = 0; i < ntile; i++) {
    const int p = p_begin + i * kTcM + warp * 32 + lane;
    const int x = p / J.fs0, y = p - x * J.fs0;
    const bool valid = ok && x < J.c1 && y < J.c0;
    for (int c0 = 0; c0 < J.n_pad; c0 += 16) {
      uint32_t r[16];
      tc_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(i * J.n_pad + c0), r);
      tc_wait_ld();
      if (valid) {
        for (int k = 0; k < 16 && c0 + k < J.n; k++) {
          const int2 dk = dim_s[c0 + k];   // this filter's own map: rows dk.x, columns dk.y
          if (x >= dk.y || y >= dk.x) continue;
          float v;
          memcpy(&v, &r[k], 4);
          arena[(size_t)out_s[c0 + k] + (size_t)x * dk.x + y] = v * scl_s[c0 + k];
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, ncols);
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
// host: filter banks and job tables
// ---------------------------------------------------------------------------
static uint16_t to_bf16(float f) {   // round to nearest even
  uint32_t u;
  memcpy(&u, &f, 4);
  if ((u & 0x7f800000u) == 0x7f800000u) return (uint16_t)(u >> 16);   // inf / nan
  const uint32_t lsb = (u >> 16) & 1u;
  u += 0x7fffu + lsb;
  return (uint16_t)(u >> 16);
}

// e4m3 bank from FP32 filters on the device (CUDA's own conversion, as for the
// features): element (tap t = xp*b0 + yp of the group's grid, plane q, filter
// f, lane k) = channel 16q + k of filter f at (xp, yp) times scale[f], zero
// outside the filter's own b1 x b0 (fdim[f] = {b0, b1})
__global__ void k_bank_e4m3(const float *const *__restrict__ filt, const float *__restrict__ scale,
                            const int2 *__restrict__ fdim, int n, int n_pad, int b0, int taps,
                            uint8_t *__restrict__ out) {
  const int total = taps * 2 * n_pad * 16;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
    const int k = e % 16, f = (e / 16) % n_pad, q = (e / (16 * n_pad)) % 2, t = e / (32 * n_pad);
    const int c = 16 * q + k, xp = t / b0, yp = t - xp * b0;
    float v = 0.f;
    if (f < n && c < kFeat) {
      const int fb0 = fdim[f].x, fb1 = fdim[f].y;
      if (xp < fb1 && yp < fb0) v = filt[f][(size_t)c * fb0 * fb1 + xp * fb0 + yp] * scale[f];
    }
    out[e] = (uint8_t)__nv_cvt_float_to_fp8(v, __NV_SATFINITE, __NV_E4M3);
  }
}

// A group's filters share one bank [tap][q][n_pad][16 B] over the group's tap
// grid b1 x b0 (the largest of its filters); a smaller filter sits in the
// grid's first rows and columns with zero weights around it, which add
// nothing to its sums, and its map is its own size (c0, c1 of its b0, b1).
struct BankGroup {
  int b0, b1, n, n_pad, bank_off, kind;
  std::vector<int> filt;      // indices into the caller's filter list
  std::vector<int> fb0, fb1;  // each filter's own rows, columns
  std::vector<float> inv;     // per filter: factor that undoes the operand scaling
};

static int tc_planes_of(geye_conv_mode mode) { return mode == GEYE_CONV_FP8 ? 2 : 4; }

// power of two that brings a filter's absolute maximum under e4m3's 448
static float e4m3_filter_scale(const float *F, size_t n) {
  float m = 0.f;
  for (size_t i = 0; i < n; i++) m = std::max(m, std::fabs(F[i]));
  if (!(m > 0.f)) return 1.f;
  return std::ldexp(1.0f, (int)std::floor(std::log2(448.0 / m)));
}

// tensor work of a grouping: every tile issues taps MMAs of N = n_pad
static double group_cost(const std::vector<BankGroup> &gs) {
  double c = 0;
  for (auto &g : gs) c += (double)g.b0 * g.b1 * (((g.n + 15) & ~15) + 16);
  return c;
}

// groups the filters of each kind either by exact size or all together on the
// largest grid (at most 32 a group), whichever issues less tensor work; lays
// out the banks (filter f is [31][b1][b0] as conv_fp32 reads it: element
// (c, xp, yp) at c*b0*b1 + xp*b0 + yp).  BF16 banks are built here into
// bank16; for FP8 scale[f] is filled and the caller converts on the device.
static void build_banks(const std::vector<const float *> &filt, const std::vector<int> &b0s,
                        const std::vector<int> &b1s, const std::vector<int> &kinds, geye_conv_mode mode,
                        std::vector<BankGroup> &groups, std::vector<uint16_t> &bank16, std::vector<float> &scale,
                        size_t &total, int cap = 32) {
  const int NQ = tc_planes_of(mode);
  groups.clear();
  for (int kind = 0; kind <= 1; kind++) {
    std::vector<BankGroup> exact, merged;
    for (size_t f = 0; f < filt.size(); f++) {
      if (kinds[f] != kind) continue;
      bool placed = false;
      for (auto &g : exact)
        if (g.b0 == b0s[f] && g.b1 == b1s[f] && g.n < cap) {
          g.filt.push_back((int)f); g.fb0.push_back(b0s[f]); g.fb1.push_back(b1s[f]);
          g.n++;
          placed = true;
          break;
        }
      if (!placed) exact.push_back(BankGroup{b0s[f], b1s[f], 1, 0, 0, kind, {(int)f}, {b0s[f]}, {b1s[f]}, {}});
      if (merged.empty() || merged.back().n == cap) merged.push_back(BankGroup{0, 0, 0, 0, 0, kind, {}, {}, {}, {}});
      BankGroup &m = merged.back();
      m.b0 = std::max(m.b0, b0s[f]);
      m.b1 = std::max(m.b1, b1s[f]);
      m.filt.push_back((int)f); m.fb0.push_back(b0s[f]); m.fb1.push_back(b1s[f]);
      m.n++;
    }
    const auto &pick = group_cost(merged) < group_cost(exact) ? merged : exact;
    groups.insert(groups.end(), pick.begin(), pick.end());
  }
  total = 0;
  for (auto &g : groups) {
    g.n_pad = (g.n + 15) & ~15;   // N of the MMA: a multiple of 16
    g.bank_off = (int)total;
    total += (size_t)g.b0 * g.b1 * NQ * g.n_pad * 16;
  }
  scale.assign(filt.size(), 1.f);
  for (auto &g : groups)
    for (int k = 0; k < g.n; k++) {
      const int f = g.filt[k];
      if (mode == GEYE_CONV_FP8) scale[f] = e4m3_filter_scale(filt[f], (size_t)g.fb0[k] * g.fb1[k] * kFeat);
      g.inv.push_back(mode == GEYE_CONV_FP8 ? 1.0f / (scale[f] * kFp8FeatScale) : 1.0f);
    }
  if (mode == GEYE_CONV_FP8) return;
  bank16.assign(total / 2, 0);
  for (auto &g : groups) {
    uint16_t *dst = bank16.data() + g.bank_off / 2;
    for (int n = 0; n < g.n; n++) {
      const float *F = filt[g.filt[n]];
      const int fb0 = g.fb0[n], fb1 = g.fb1[n];
      for (int xp = 0; xp < fb1; xp++)
        for (int yp = 0; yp < fb0; yp++) {
          const size_t t = (size_t)xp * g.b0 + yp;
          for (int c = 0; c < kFeat; c++)
            dst[((t * 4 + (c >> 3)) * g.n_pad + n) * 8 + (c & 7)] = to_bf16(F[(size_t)c * fb0 * fb1 + xp * fb0 + yp]);
        }
    }
  }
}

// device bank of the groups (d_bank sized total); d_filt: the filters on the device
static geye_status upload_bank(const std::vector<BankGroup> &groups, geye_conv_mode mode,
                               const std::vector<uint16_t> &bank16, const std::vector<const float *> &d_filt,
                               const std::vector<float> &scale, size_t total, void *d_bank, cudaStream_t s) {
  if (mode != GEYE_CONV_FP8) {
    CUDA_TRY(cudaMemcpyAsync(d_bank, bank16.data(), total, cudaMemcpyHostToDevice, s));
    return GEYE_OK;
  }
  for (auto &g : groups) {
    std::vector<const float *> ptrs;
    std::vector<float> sc;
    std::vector<int2> dims;
    for (int k = 0; k < g.n; k++) {
      ptrs.push_back(d_filt[g.filt[k]]);
      sc.push_back(scale[g.filt[k]]);
      dims.push_back(make_int2(g.fb0[k], g.fb1[k]));
    }
    const float **d_ptrs = nullptr;
    float *d_sc = nullptr;
    int2 *d_dims = nullptr;
    CUDA_TRY(cudaMalloc(&d_ptrs, sizeof(float *) * ptrs.size()));
    cudaError_t e = cudaMalloc(&d_sc, sizeof(float) * sc.size());
    if (e == cudaSuccess) e = cudaMalloc(&d_dims, sizeof(int2) * dims.size());
    if (e == cudaSuccess) e = cudaMemcpy(d_ptrs, ptrs.data(), sizeof(float *) * ptrs.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_sc, sc.data(), sizeof(float) * sc.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_dims, dims.data(), sizeof(int2) * dims.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
      const int taps = g.b0 * g.b1, elems = taps * 2 * g.n_pad * 16;
      k_bank_e4m3<<<std::max(1, std::min((elems + 255) / 256, 1024)), 256, 0, s>>>(
          d_ptrs, d_sc, d_dims, g.n, g.n_pad, g.b0, taps, static_cast<uint8_t *>(d_bank) + g.bank_off);
      e = cudaStreamSynchronize(s);
    }
    cudaFree(d_ptrs);
    cudaFree(d_sc);
    cudaFree(d_dims);
    if (e != cudaSuccess) {
      set_error(std::string("e4m3 filter bank: ") + cudaGetErrorString(e));
      return GEYE_ERR_CUDA;
    }
  }
  return GEYE_OK;
}

struct TcTables {
  std::vector<TcJob> jobs;
  std::vector<int4> chunks;
  std::vector<int> outs;
  std::vector<float> inv;
  std::vector<int2> dims;   // each map's rows, columns
  size_t max_smem = 0;
};

// one job: group g on a level whose planes start at plane_off; map_off[k] is
// the float offset of filter k's output map.  cells_avail: cells from the
// start of plane 0 to the end of the planes' buffer (a slab may read past its
// own plane into the next one or into the buffer's tail: those cells only
// meet zero weights).  t_cap and budget: the largest tile run and shared
// memory a CTA may take (the tile-shape candidates of the autotuner below).
// False if it cannot fit in shared memory or the buffer.
static bool add_tc_job(TcTables &T, int NQ, int plane_off, int fs0, int fs1, const BankGroup &g,
                       const std::vector<int> &map_off, long long cells_avail, int t_cap = kTcMaxTiles,
                       size_t budget = kTcSmemBudget) {
  TcJob J{};
  J.plane_off = plane_off;
  J.plane_cells = fs0 * fs1 + kTcPlanePad;
  J.fs0 = fs0; J.fs1 = fs1;
  J.b0 = g.b0; J.b1 = g.b1;
  int mb0 = g.b0, mb1 = g.b1;   // the smallest filter: the most outputs
  for (int k = 0; k < g.n; k++) { mb0 = std::min(mb0, g.fb0[k]); mb1 = std::min(mb1, g.fb1[k]); }
  J.c0 = fs0 - mb0 + 1; J.c1 = fs1 - mb1 + 1;
  if (J.c0 < 1 || J.c1 < 1) return false;
  J.n = g.n; J.n_pad = g.n_pad;
  J.bank_off = g.bank_off;
  J.out_tab = (int)T.outs.size();
  for (int k = 0; k < g.n; k++) {
    const int c0k = fs0 - g.fb0[k] + 1, c1k = fs1 - g.fb1[k] + 1;
    if (c0k < 1 || c1k < 1) return false;
    T.outs.push_back(map_off[k]);
    T.inv.push_back(g.inv[k]);
    T.dims.push_back(make_int2(c0k, c1k));
  }
  const int P_valid = (J.c1 - 1) * J.fs0 + J.c0;
  J.ntiles = (P_valid + kTcM - 1) / kTcM;
  // tiles per CTA (T) and filter columns per phase (cs): one phase when the whole
  // bank and slab fit, else fewer columns per phase; every phase needs
  // head + bank columns + NQ planes of (T*128 + (cs-1)*fs0 + b0-1) cells x 16 B
  const size_t col_bytes = (size_t)g.b0 * NQ * g.n_pad * 16;
  auto need = [&](int Tc, int cs) {
    return (size_t)kTcHead + ((cs * col_bytes + 127) & ~(size_t)127) +
           ((size_t)Tc * kTcM + (size_t)(cs - 1) * fs0 + (g.b0 - 1)) * 16 * NQ;
  };
  int T_cta = 0, cs = 0;
  const int t_max = std::max(1, std::min(t_cap, kTcTmemCols / g.n_pad));   // accumulators fit TMEM
  for (int Tc = t_max; Tc >= std::min(4, t_max) && !T_cta; Tc /= 2)
    if (need(Tc, g.b1) <= budget) { T_cta = Tc; cs = g.b1; }
  for (int Tc = std::min(8, t_max); Tc >= 1 && !T_cta; Tc /= 2)
    for (int c = g.b1; c >= 1; c--)
      if (need(Tc, c) <= budget) { T_cta = Tc; cs = c; break; }
  if (!T_cta) return false;
  // the CTAs that share an SM (by shared memory) must fit their accumulators in
  // its 512 TMEM columns together, or one's allocation waits for another to end
  auto tmem_cols = [&](int Tc) {
    uint32_t c = 32;
    while (c < (uint32_t)(Tc * g.n_pad)) c <<= 1;
    return (int)c;
  };
  auto per_sm = [&](int Tc) { return std::max<size_t>(1, (size_t)(228 * 1024) / (need(Tc, cs) + 1024)); };
  while (T_cta > 1 && (size_t)tmem_cols(T_cta) * per_sm(T_cta) > (size_t)kTcTmemCols) T_cta /= 2;
  const int jid = (int)T.jobs.size();
  T.jobs.push_back(J);
  const long long reach = (long long)(g.b1 - 1) * fs0 + (g.b0 - 1);
  for (int t0 = 0; t0 < J.ntiles; t0 += T_cta) {
    const int nt = std::min(T_cta, J.ntiles - t0);
    // the last plane's slab stays inside the buffer
    if ((long long)(NQ - 1) * J.plane_cells + (long long)t0 * kTcM + nt * kTcM + reach > cells_avail) return false;
    T.chunks.push_back(make_int4(jid, t0, nt, cs));
    T.max_smem = std::max(T.max_smem, need(nt, cs));
  }
  return true;
}

static void launch_conv_tc(int NQ, const TcJob *jobs, const int4 *chunks, int n_chunks, const int *outs,
                           const float *inv, const int2 *dims, const uint8_t *planes, const uint8_t *bank, float *out,
                           int *err, size_t smem, cudaStream_t s) {
  if (NQ == 4) {
    static SmemAttr a4;
    raise_smem(a4, k_conv_tc<4>, smem);
    k_conv_tc<4><<<n_chunks, kTcThreads, smem, s>>>(jobs, chunks, outs, inv, dims, planes, bank, out, err);
  } else {
    static SmemAttr a2;
    raise_smem(a2, k_conv_tc<2>, smem);
    k_conv_tc<2><<<n_chunks, kTcThreads, smem, s>>>(jobs, chunks, outs, inv, dims, planes, bank, out, err);
  }
}

// the model's banks for a precision (built once per model and mode; roots and
// parts in separate groups)
static geye_status ensure_bank(geye_ctx *ctx, geye_model *m, geye_conv_mode mode, std::vector<BankGroup> &groups) {
  const HostModel &h = m->h;
  std::vector<const float *> filt, d_filt;
  std::vector<int> b0s, b1s, kinds;
  for (int r = 0; r < h.NoR; r++) {
    filt.push_back(h.rootfilter[r].data());
    d_filt.push_back(m->d_filters + m->filt_off[r]);
    b0s.push_back(h.root_size[3 * r]); b1s.push_back(h.root_size[3 * r + 1]); kinds.push_back(0);
  }
  for (int p = 0; p < h.NoP; p++) {
    filt.push_back(h.partfilter[p].data());
    d_filt.push_back(m->d_filters + m->filt_off[h.NoR + p]);
    b0s.push_back(h.part_size[3 * p]); b1s.push_back(h.part_size[3 * p + 1]); kinds.push_back(1);
  }
  std::vector<uint16_t> bank16;
  std::vector<float> scale;
  size_t total = 0;
  build_banks(filt, b0s, b1s, kinds, mode, groups, bank16, scale, total);
  void *&d_bank = mode == GEYE_CONV_FP8 ? m->d_bank8 : m->d_bank16;
  if (d_bank) return GEYE_OK;
  CUDA_TRY(cudaMalloc(&d_bank, std::max<size_t>(total, 16)));
  const geye_status st = upload_bank(groups, mode, bank16, d_filt, scale, total, d_bank, ctx->stream);
  CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return st;
}

// chunks ordered by cost (tiles x taps x N), heaviest first, so that the long
// ones start in the first wave
static void sort_chunks(TcTables &T) {
  auto cost = [&](const int4 &c) {
    const TcJob &J = T.jobs[c.x];
    return (long long)c.z * J.b0 * J.b1 * J.n_pad;
  };
  std::stable_sort(T.chunks.begin(), T.chunks.end(), [&](const int4 &x, const int4 &y) { return cost(x) > cost(y); });
}

// job tables of one model for a tile-shape candidate; chunks ordered by cost,
// heaviest first, so that the long ones start in the first wave
static geye_status build_tables(Plan &P, ModelPlan &mp, const std::vector<BankGroup> &groups, int NQ, int t_cap,
                                size_t budget, TcTables &T) {
  const HostModel &h = mp.model->h;
  const long long total_cells = (long long)(P.arena16.bytes / 16);
  const int NoC = h.numcomponent, NoP = h.NoP, interval = h.interval;
  for (int level = interval; level < mp.LEN; level++) {
    if (mp.skipped[level]) continue;
    const int Lv = level - interval;
    for (auto &g : groups) {
      std::vector<int> map_off;
      const bool root = g.kind == 0;
      for (int f : g.filt) map_off.push_back(root ? mp.root_map_off[level * NoC + f] : mp.part_map_off[Lv * NoP + (f - h.NoR)]);
      for (int v : map_off)
        if (v < 0) { set_error("tensor-core conv: filter map missing from the plan"); return GEYE_ERR_UNSUPPORTED; }
      const LevelInfo &L = root ? P.lv[level] : P.lv[Lv];
      const long long avail = total_cells - (long long)L.feat16_off * 2 / 16;
      if (!add_tc_job(T, NQ, L.feat16_off, L.fs0, L.fs1, g, map_off, avail, t_cap, budget)) {
        set_error("tensor-core conv: a filter bank and its feature reach exceed shared memory");
        return GEYE_ERR_UNSUPPORTED;
      }
    }
  }
  sort_chunks(T);
  return GEYE_OK;
}

// Tile-shape autotuner: every candidate (largest tile run per CTA, shared
// memory per CTA -- fewer tiles and less memory let more CTAs share an SM and
// overlap one's copies with another's MMAs) is built for this plan's levels,
// timed on the device (CUDA events, after one untimed launch) and the fastest
// kept.  Runs once per plan, before the plan's first frame.
struct TcShape {
  int t_cap;
  size_t budget;
};
static const TcShape kTcShapes[] = {{16, 220 * 1024}, {8, 220 * 1024}, {4, 220 * 1024},
                                    {8, 110 * 1024},  {4, 110 * 1024}, {4, 72 * 1024}, {2, 72 * 1024}};

geye_status build_tc_jobs(geye_ctx *ctx, Plan &P, ModelPlan &mp) {
  geye_model *m = mp.model;
  const geye_conv_mode mode = ctx->conv_mode;
  std::vector<BankGroup> groups;
  GEYE_TRY(ensure_bank(ctx, m, mode, groups));
  const int NQ = tc_planes_of(mode);
  const void *bank = NQ == 2 ? m->d_bank8 : m->d_bank16;
  mp.tc_planes = NQ;
  if (!P.arena16.p) {   // a plan built from features has no planes: run_conv_tc reports it
    mp.tc_chunks = 0;
    return GEYE_OK;
  }
  TcTables best;
  int best_shape = -1;
  float best_ms = 0.f;
  const bool tunable = P.arena16.p && P.arena.p && P.d_small.p;
  int n_shapes = tunable ? (int)(sizeof(kTcShapes) / sizeof(kTcShapes[0])) : 1;
  int first = 0;
  // a geometry this model was tuned at before reuses that choice
  const std::string key = std::to_string(P.width) + "x" + std::to_string(P.height) + "/" + std::to_string(mp.LEN) +
                          "/" + std::to_string((int)mode);
  {
    std::lock_guard<std::mutex> lk(m->tc_mu);
    auto it = m->tc_tuned.find(key);
    if (tunable && it != m->tc_tuned.end()) {
      first = it->second.first;
      n_shapes = first + 1;
      best_ms = 3.0f * it->second.second;
    }
  }
  // GEYE_TC_SHAPE=<i> pins candidate i (reproducible shapes; no timing)
  if (const char *e = getenv("GEYE_TC_SHAPE")) {
    const int i = atoi(e);
    if (i >= 0 && i < (int)(sizeof(kTcShapes) / sizeof(kTcShapes[0]))) { first = i; n_shapes = i + 1; }
  }
  const bool timed = tunable && n_shapes - first > 1;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (timed) {
    CUDA_TRY(cudaEventCreate(&e0));
    CUDA_TRY(cudaEventCreate(&e1));
  }
  for (int si = first; si < n_shapes; si++) {
    TcTables T;
    if (build_tables(P, mp, groups, NQ, kTcShapes[si].t_cap, kTcShapes[si].budget, T) != GEYE_OK) continue;
    if (!timed || T.chunks.empty()) {
      best = std::move(T);
      best_shape = si;
      break;
    }
    DevBuf jobs, chunks, outs, inv, dims;
    GEYE_TRY(upload_bytes(ctx, jobs, T.jobs.data(), sizeof(TcJob) * T.jobs.size()));
    GEYE_TRY(upload_bytes(ctx, chunks, T.chunks.data(), sizeof(int4) * T.chunks.size()));
    GEYE_TRY(upload_bytes(ctx, outs, T.outs.data(), sizeof(int) * T.outs.size()));
    GEYE_TRY(upload_bytes(ctx, inv, T.inv.data(), sizeof(float) * T.inv.size()));
    GEYE_TRY(upload_bytes(ctx, dims, T.dims.data(), sizeof(int2) * T.dims.size()));
    auto launch = [&]() {
      launch_conv_tc(NQ, jobs.as<TcJob>(), chunks.as<int4>(), (int)T.chunks.size(), outs.as<int>(), inv.as<float>(),
                     dims.as<int2>(), P.arena16.as<uint8_t>(), static_cast<const uint8_t *>(bank), P.arena.as<float>(),
                     P.d_small.as<int>() + 130, T.max_smem, ctx->stream);
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
      best = std::move(T);
      best_shape = si;
      best_ms = ms;
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (timed) CUDA_TRY(cudaMemsetAsync(P.d_small.as<int>() + 130, 0, sizeof(int), ctx->stream));
  if (best_shape < 0) return GEYE_ERR_UNSUPPORTED;   // the error of the last candidate stands
  if (timed) {
    std::lock_guard<std::mutex> lk(m->tc_mu);
    m->tc_tuned[key] = {best_shape, best_ms / 3.0f};
  }
  mp.tc_smem = best.max_smem;
  mp.tc_chunks = (int)best.chunks.size();
  mp.tc_planes = NQ;
  mp.tc_shape = best_shape;
  mp.tc_tuned_ms = best_ms / 3.0f;
  GEYE_TRY(upload_bytes(ctx, mp.d_tc_jobs, best.jobs.data(), sizeof(TcJob) * best.jobs.size()));
  GEYE_TRY(upload_bytes(ctx, mp.d_tc_chunks, best.chunks.data(), sizeof(int4) * best.chunks.size()));
  GEYE_TRY(upload_bytes(ctx, mp.d_tc_outs, best.outs.data(), sizeof(int) * best.outs.size()));
  GEYE_TRY(upload_bytes(ctx, mp.d_tc_inv, best.inv.data(), sizeof(float) * best.inv.size()));
  GEYE_TRY(upload_bytes(ctx, mp.d_tc_dims, best.dims.data(), sizeof(int2) * best.dims.size()));
  return GEYE_OK;
}

}  // namespace geye

geye_status geye_conv_tuning(geye_ctx *ctx, const geye_model *m, int shape[3], float *ms) {
  ARG_CHECK(ctx && m && shape && ms, "null argument");
  ARG_CHECK(ctx->last_plan, "no run yet");
  for (auto &mp : ctx->last_plan->models) {
    if (mp->model != m) continue;
    ARG_CHECK(mp->tc_shape >= 0, "the last run's plan has no tensor-core convolution");
    shape[0] = geye::kTcShapes[mp->tc_shape].t_cap;
    shape[1] = (int)(geye::kTcShapes[mp->tc_shape].budget / 1024);
    shape[2] = mp->tc_chunks;
    *ms = mp->tc_tuned_ms;
    return GEYE_OK;
  }
  ARG_CHECK(false, "the last run has no such model");
  return GEYE_ERR_ARG;
}

namespace geye {

geye_status run_conv_tc(geye_ctx *ctx, Plan &P, ModelPlan &mp) {
  if (!P.arena16.p) {
    set_error("tensor-core conv: the plan has no feature planes");
    return GEYE_ERR_UNSUPPORTED;
  }
  if (mp.tc_chunks == 0) return GEYE_OK;
  const void *bank = mp.tc_planes == 2 ? mp.model->d_bank8 : mp.model->d_bank16;
  launch_conv_tc(mp.tc_planes, mp.d_tc_jobs.as<TcJob>(), mp.d_tc_chunks.as<int4>(), mp.tc_chunks,
                 mp.d_tc_outs.as<int>(), mp.d_tc_inv.as<float>(), mp.d_tc_dims.as<int2>(), P.arena16.as<uint8_t>(),
                 static_cast<const uint8_t *>(bank), P.arena.as<float>(), P.d_small.as<int>() + 130, mp.tc_smem,
                 ctx->stream);
  ctx->launches++;
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(std::string("tensor-core conv: ") + cudaGetErrorString(e));
    return GEYE_ERR_CUDA;
  }
  return GEYE_OK;
}

// fconvsMT on the tensor cores for the stage entry point (the context's conv
// mode): d_feat is [pos][32] float on the device (a0 x a1 cells), filters on
// the host; maps go to d_out + out_off[i].  Temporary device buffers live in tmp.
geye_status conv_tc_maps(geye_ctx *ctx, const float *d_feat, int a0, int a1, const float *const *filters,
                         const int *b_dims, int n_filters, float *d_out, const std::vector<int> &out_off,
                         std::vector<std::unique_ptr<DevBuf>> &tmp) {
  const geye_conv_mode mode = ctx->conv_mode;
  const int NQ = tc_planes_of(mode);
  auto buf = [&]() { tmp.push_back(std::make_unique<DevBuf>()); return tmp.back().get(); };
  std::vector<const float *> filt(filters, filters + n_filters), d_filt;
  std::vector<int> b0s, b1s, kinds(n_filters, 0);
  for (int i = 0; i < n_filters; i++) { b0s.push_back(b_dims[2 * i]); b1s.push_back(b_dims[2 * i + 1]); }
  std::vector<BankGroup> groups;
  std::vector<uint16_t> bank16;
  std::vector<float> scale;
  size_t total = 0;
  build_banks(filt, b0s, b1s, kinds, mode, groups, bank16, scale, total, kTcMaxN);
  for (int i = 0; i < n_filters; i++) {   // the FP8 bank is converted on the device from FP32 copies
    DevBuf *f = buf();
    const size_t n = (size_t)b0s[i] * b1s[i] * kFeat;
    GEYE_TRY(upload_bytes(ctx, *f, filters[i], sizeof(float) * n));
    d_filt.push_back(f->as<float>());
  }
  // planes, then a zeroed tail that slabs of filters smaller than their group's grid may read
  const int ncell = a0 * a1;
  int mb0 = 1, mb1 = 1;
  for (auto &g : groups) { mb0 = std::max(mb0, g.b0); mb1 = std::max(mb1, g.b1); }
  const size_t tail_cells = (size_t)mb1 * a0 + mb0 + (size_t)kTcMaxTiles * kTcM;
  const size_t plane_total = (size_t)NQ * (ncell + kTcPlanePad);
  TcTables T;
  for (auto &g : groups) {
    std::vector<int> map_off;
    for (int f : g.filt) map_off.push_back(out_off[f]);
    if (!add_tc_job(T, NQ, 0, a0, a1, g, map_off, (long long)(plane_total + tail_cells))) {
      set_error("tensor-core conv: a filter bank and its feature reach exceed shared memory");
      return GEYE_ERR_UNSUPPORTED;
    }
  }
  DevBuf *planes = buf(), *d_bank = buf(), *d_jobs = buf(), *d_chunks = buf(), *d_outs = buf(), *d_inv = buf(),
         *d_dims = buf(), *d_err = buf();
  GEYE_TRY(planes->alloc(ctx, (plane_total + tail_cells) * 16));
  CUDA_TRY(cudaMemsetAsync(planes->as<uint8_t>() + plane_total * 16, 0, tail_cells * 16, ctx->stream));
  GEYE_TRY(d_bank->alloc(ctx, std::max<size_t>(total, 16)));
  GEYE_TRY(upload_bank(groups, mode, bank16, d_filt, scale, total, d_bank->p, ctx->stream));
  GEYE_TRY(upload_bytes(ctx, *d_jobs, T.jobs.data(), sizeof(TcJob) * T.jobs.size()));
  GEYE_TRY(upload_bytes(ctx, *d_chunks, T.chunks.data(), sizeof(int4) * T.chunks.size()));
  GEYE_TRY(upload_bytes(ctx, *d_outs, T.outs.data(), sizeof(int) * T.outs.size()));
  GEYE_TRY(upload_bytes(ctx, *d_inv, T.inv.data(), sizeof(float) * T.inv.size()));
  GEYE_TRY(upload_bytes(ctx, *d_dims, T.dims.data(), sizeof(int2) * T.dims.size()));
  GEYE_TRY(d_err->alloc(ctx, 16));
  CUDA_TRY(cudaMemsetAsync(d_err->p, 0, 16, ctx->stream));
  const int grid = std::max(1, std::min((ncell + kTcPlanePad + 255) / 256, 1024));
  if (NQ == 4) k_feat_planes<4><<<grid, 256, 0, ctx->stream>>>(d_feat, ncell, planes->as<uint8_t>());
  else k_feat_planes<2><<<grid, 256, 0, ctx->stream>>>(d_feat, ncell, planes->as<uint8_t>());
  launch_conv_tc(NQ, d_jobs->as<TcJob>(), d_chunks->as<int4>(), (int)T.chunks.size(), d_outs->as<int>(),
                 d_inv->as<float>(), d_dims->as<int2>(), planes->as<uint8_t>(), d_bank->as<uint8_t>(), d_out,
                 d_err->as<int>(), T.max_smem, ctx->stream);
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
