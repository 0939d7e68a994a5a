// nms_sort.cu -- the reference's quicksort of the detection scores
// (CAR_TRACKING/nms.cpp:70-84), every model of a frame at once, with its exact
// order for equal scores (partition argument in nms_common.h).
//
//   k_qs_load: keys, the identity order and the first segment of each model.
//   Levels (by default three times the balanced depth to kNmsSegS, plus three:
//   nms_sort_levels; a plan may launch fewer once it has seen its frames' depth), three
//   kernels each (no-ops once nothing is left):
//     k_qs_count   every segment above kNmsSegS is cut into tiles of kNmsTile
//                  elements; a block counts its tile's values <= key and >= key;
//     k_qs_scatter with the counts of the tiles before it, a block writes its
//                  tile's positions into the L and R lists;
//     k_qs_swap    a block swaps its slice of the pairs (L[k], R[k]) with
//                  L[k] < R[k]; the block holding the first k with
//                  L[k] >= R[k] (or the end of the lists) knows K and queues
//                  the two children, above kNmsSegS for the next level, the
//                  others for the shared-memory kernel.
//   k_qs_small: a block per queued segment sorts it in shared memory: block
//     partitions above kWarpSeg elements, warp partitions above kTiny, one
//     thread below.
//   k_qs_rest: one block per model finishes any segment still above kNmsSegS
//     after the launched levels (block partitions in global memory).
// No block waits on another; every hand-over is a kernel boundary.
#include <algorithm>

#include "nms_common.h"

namespace geye {

constexpr int kT = kNmsTile;     // elements per tile (4 per thread)
constexpr int kWarpSeg = 1024;   // shared-memory kernel: block partitions above this
constexpr int kWL = 256;         // its queue of warp segments
constexpr int kQ = 1024;         // k_qs_rest's block-tier queue

// ---------------------------------------------------------------------------
// load
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_qs_load(const float *__restrict__ boxes_all, const int *__restrict__ d_num,
                                                 int GL, int cap, int *si, float *sf, const int *need) {
  const int m = blockIdx.y;
  Slots S = slots(si, sf, m, cap);
  const float *boxes = boxes_all + (size_t)m * cap * GL;
  // a model that does not need the quicksort order: nothing to sort or resolve
  const int D = (need && !need[m]) ? 0 : max(0, min(d_num[m], cap));
  const int i = blockIdx.x * 256 + threadIdx.x;
  if (i < D) {
    S.val[i] = boxes[(size_t)i * GL + GL - 2];
    S.ord[i] = i;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    BatchState &st = *S.st;
    st.D = D;
    st.nwords = (D + 31) >> 5;
    st.scan_word = 0;
    st.npicks = 0;
    st.npb = 0;
    st.done = D <= 0;
    st.batches = 0;
    st.fallback = 0;
    SortState &ss = *S.ss;
    ss.big_n[0] = D > kNmsSegS ? 1 : 0;
    ss.big_n[1] = 0;
    ss.small_n = (D >= 2 && D <= kNmsSegS) ? 1 : 0;
    S.big[0][0] = make_int2(0, D - 1);
    S.small[0] = make_int2(0, D - 1);
  }
}

// ---------------------------------------------------------------------------
// grid-wide partition levels
// ---------------------------------------------------------------------------
struct TileRef {
  int e, t, tb, nt;   // segment, tile within it, first tile index of the segment, its tiles
  int lo, hi;
};

// global tile g of level buffer cur -> segment and tile; false past the end
__device__ __forceinline__ bool find_tile(const Slots &S, int cur, int n, int g, TileRef &r) {
  int tb = 0;
  for (int e = 0; e < n; e++) {
    const int2 sg = S.big[cur][e];
    const int nt = (sg.y - sg.x + 1 + kT - 1) / kT;
    if (g < tb + nt) {
      r.e = e; r.t = g - tb; r.tb = tb; r.nt = nt; r.lo = sg.x; r.hi = sg.y;
      return true;
    }
    tb += nt;
  }
  return false;
}

__device__ __forceinline__ int total_tiles(const Slots &S, int cur, int n) {
  int tb = 0;
  for (int e = 0; e < n; e++) {
    const int2 sg = S.big[cur][e];
    tb += (sg.y - sg.x + 1 + kT - 1) / kT;
  }
  return tb;
}

// block sums of two ints; every thread gets both totals
__device__ __forceinline__ int2 block_sum2(int a, int b, int2 *wbuf) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
  __syncthreads();   // wbuf free
  if (lane == 0) wbuf[warp] = make_int2(a, b);
  __syncthreads();
  int2 t = make_int2(0, 0);
  for (int w = 0; w < kNmsNT / 32; w++) {
    t.x += wbuf[w].x;
    t.y += wbuf[w].y;
  }
  return t;
}

// (<= key, >= key) counts of the tiles of one segment before tile t, and of all its tiles
__device__ __forceinline__ void tile_prefix(const Slots &S, const TileRef &r, int2 *wbuf, int2 &before, int2 &total) {
  int bl = 0, br = 0, al = 0, ar = 0;
  for (int u = threadIdx.x; u < r.nt; u += kNmsNT) {
    const int2 c = S.tiles[r.tb + u];
    al += c.x; ar += c.y;
    if (u < r.t) { bl += c.x; br += c.y; }
  }
  before = block_sum2(bl, br, wbuf);
  total = block_sum2(al, ar, wbuf);
}

__global__ void __launch_bounds__(kNmsNT) k_qs_count(int level, int cap, int *si, float *sf, int *lv_used) {
  __shared__ int2 wbuf[kNmsNT / 32];
  Slots S = slots(si, sf, blockIdx.y, cap);
  const int cur = level & 1;
  if (blockIdx.x == 0 && threadIdx.x == 0) S.ss->big_n[cur ^ 1] = 0;   // the next level's queue
  const int n = S.ss->big_n[cur];
  if (n == 0) return;
  if (lv_used && blockIdx.x == 0 && threadIdx.x == 0) atomicMax(lv_used, level + 1);   // levels with work
  const int ntot = total_tiles(S, cur, n);
  for (int g = blockIdx.x; g < ntot; g += gridDim.x) {
    TileRef r;
    if (!find_tile(S, cur, n, g, r)) break;
    const float key = S.val[(r.lo + r.hi) / 2];
    const int start = r.lo + r.t * kT, end = min(start + kT, r.hi + 1);
    int cL = 0, cR = 0;
    const int p0 = start + 4 * threadIdx.x;
    for (int p = p0; p < min(p0 + 4, end); p++) {
      const float v = S.val[p];
      cL += !(v > key);
      cR += !(v < key);
    }
    const int2 t = block_sum2(cL, cR, wbuf);
    if (threadIdx.x == 0) S.tiles[r.tb + r.t] = t;
  }
}

__global__ void __launch_bounds__(kNmsNT) k_qs_scatter(int level, int cap, int *si, float *sf) {
  __shared__ int2 wbuf[kNmsNT / 32];
  __shared__ unsigned long long wsum[kNmsNT / 32];
  Slots S = slots(si, sf, blockIdx.y, cap);
  const int cur = level & 1;
  const int n = S.ss->big_n[cur];
  if (n == 0) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int ntot = total_tiles(S, cur, n);
  for (int g = blockIdx.x; g < ntot; g += gridDim.x) {
    TileRef r;
    if (!find_tile(S, cur, n, g, r)) break;
    int2 before, total;
    tile_prefix(S, r, wbuf, before, total);
    const float key = S.val[(r.lo + r.hi) / 2];
    const int start = r.lo + r.t * kT, end = min(start + kT, r.hi + 1);
    const int p0 = start + 4 * threadIdx.x, p1 = min(p0 + 4, end);
    unsigned cL = 0, cR = 0;
    for (int p = p0; p < p1; p++) {
      const float v = S.val[p];
      cL += !(v > key);
      cR += !(v < key);
    }
    const unsigned long long mine = ((unsigned long long)cL << 32) | cR;
    const unsigned long long inc = warp_incl_scan64(mine);
    if (lane == 31) wsum[warp] = inc;
    __syncthreads();
    if (warp == 0) wsum[lane] = warp_incl_scan64(wsum[lane]);
    __syncthreads();
    const unsigned long long ex = (warp ? wsum[warp - 1] : 0ull) + inc - mine;
    int rl = before.x + (int)(ex >> 32), rr = before.y + (int)(ex & 0xffffffffu);
    const int nR = total.y;
    int *Lp = S.Lpos + r.lo, *Rp = S.Rpos + r.lo;
    for (int p = p0; p < p1; p++) {
      const float v = S.val[p];
      if (!(v > key)) Lp[rl++] = p;
      if (!(v < key)) Rp[nR - 1 - (rr++)] = p;
    }
    __syncthreads();   // wsum reused by the next tile
  }
}

__global__ void __launch_bounds__(kNmsNT) k_qs_swap(int level, int cap, int *si, float *sf, int *err) {
  __shared__ int2 wbuf[kNmsNT / 32];
  Slots S = slots(si, sf, blockIdx.y, cap);
  const int cur = level & 1, nxt = cur ^ 1;
  const int n = S.ss->big_n[cur];
  if (n == 0) return;
  const int ntot = total_tiles(S, cur, n);
  const int bcap = nms_big_cap(cap);
  for (int g = blockIdx.x; g < ntot; g += gridDim.x) {
    TileRef r;
    if (!find_tile(S, cur, n, g, r)) break;
    int2 before, total;
    tile_prefix(S, r, wbuf, before, total);
    const int nL = total.x, nR = total.y, lim = min(nL, nR);
    const int *Lp = S.Lpos + r.lo, *Rp = S.Rpos + r.lo;
    const int s = r.t * kT, e = min(s + kT, lim);
    int c = 0;
    const int k0 = s + 4 * threadIdx.x;
    for (int k = k0; k < min(k0 + 4, e); k++) {
      const int a = Lp[k], b = Rp[k];
      if (a < b) {   // a true prefix: exactly the k < K
        const float tv = S.val[a]; S.val[a] = S.val[b]; S.val[b] = tv;
        const int to = S.ord[a]; S.ord[a] = S.ord[b]; S.ord[b] = to;
        c++;
      }
    }
    const int cnt = block_sum2(c, 0, wbuf).x;
    if (threadIdx.x == 0 && s < e) {
      int K = -1;
      if (cnt < e - s) {
        if (s == 0 || Lp[s - 1] < Rp[s - 1]) K = s + cnt;
      } else if (e == lim) {
        K = lim;
      }
      if (K >= 0) {
        int i, j;
        part_bounds(Lp, Rp, K, nL, nR, i, j);
        const int2 ch[2] = {make_int2(r.lo, i - 1), make_int2(j + 1, r.hi)};
        for (int u = 0; u < 2; u++) {
          if (ch[u].x >= ch[u].y) continue;
          if (ch[u].y - ch[u].x + 1 > kNmsSegS) {
            const int idx = atomicAdd(&S.ss->big_n[nxt], 1);
            if (idx < bcap) S.big[nxt][idx] = ch[u];
            else atomicOr(err, 256);   // impossible: disjoint segments above kNmsSegS
          } else {
            const int idx = atomicAdd(&S.ss->small_n, 1);
            if (idx < cap / 2) S.small[idx] = ch[u];
            else atomicOr(err, 512);   // impossible: disjoint segments of >= 2 elements
          }
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// segments of <= kNmsSegS elements, each sorted in shared memory by one block
// ---------------------------------------------------------------------------
struct SmallSmem {
  float a[kNmsSegS];
  int o[kNmsSegS];
  uint16_t Lp[kNmsSegS], Rp[kNmsSegS];
  int2 wl[kWL];             // segments of kTiny+1..kWarpSeg elements
  int2 tiny[32][32];        // per warp: segments of <= kTiny elements
};

// per warp: queue a tiny segment; 32 queued ones are sorted at once, a lane each.
// Every lane reads the count before lane 0 changes it (the __syncwarp after the read).
__device__ __forceinline__ void tiny_push(SmallSmem &Z, int *tiny_n, int2 seg) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int cnt = tiny_n[warp];
  __syncwarp();
  if (cnt == 32) {
    const int2 t = Z.tiny[warp][lane];
    thread_qsort(Z.a, Z.o, t.x, t.y);
    __syncwarp();
    cnt = 0;
  }
  if (lane == 0) {
    Z.tiny[warp][cnt] = seg;
    tiny_n[warp] = cnt + 1;
  }
  __syncwarp();
}

__global__ void __launch_bounds__(kNmsNT) k_qs_small(int n_models, int cap, int *si, float *sf, int *err) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SmallSmem &Z = *reinterpret_cast<SmallSmem *>(smem_raw);
  __shared__ unsigned long long wsum[32];
  __shared__ int sh[8];
  __shared__ int2 bstk[64];
  __shared__ int nbs, wl_n, wl_next;
  __shared__ int tiny_n[kNmsNT / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int total = 0;
  for (int m = 0; m < n_models; m++) total += slots(si, sf, m, cap).ss->small_n;
  for (int g = blockIdx.x; g < total; g += gridDim.x) {
    int m = 0, e = g;
    for (; m < n_models; m++) {
      const int c = slots(si, sf, m, cap).ss->small_n;
      if (e < c) break;
      e -= c;
    }
    Slots S = slots(si, sf, m, cap);
    const int2 sg = S.small[e];
    const int lo = sg.x, len = sg.y - sg.x + 1;
    if (len < 2 || len > kNmsSegS) {   // impossible by construction
      if (threadIdx.x == 0) atomicOr(err, 1024);
      continue;
    }
    for (int i = threadIdx.x; i < len; i += kNmsNT) {
      Z.a[i] = S.val[lo + i];
      Z.o[i] = S.ord[lo + i];
    }
    if (lane == 0) tiny_n[warp] = 0;
    if (threadIdx.x == 0) {
      nbs = 0; wl_n = 0; wl_next = 0;
      if (len > kWarpSeg) { bstk[0] = make_int2(0, len - 1); nbs = 1; }
      else { Z.wl[0] = make_int2(0, len - 1); wl_n = 1; }
    }
    __syncthreads();
    for (int round = 0;; round++) {
      // block partitions, depth first (larger child pushed first): the stack
      // holds at most log2(kNmsSegS / kWarpSeg) + 1 segments
      while (nbs > 0 && wl_n <= kWL - 2) {
        const int2 seg = bstk[nbs - 1];
        __syncthreads();   // everyone has read nbs and the top entry
        chunk_partition<uint16_t>(Z.a, Z.o, Z.Lp, Z.Rp, seg.x, seg.y, wsum, sh);
        if (threadIdx.x == 0) {
          nbs--;
          const int i = sh[1], j = sh[2];
          int2 ch[2] = {make_int2(seg.x, i - 1), make_int2(j + 1, seg.y)};
          if (ch[0].y - ch[0].x < ch[1].y - ch[1].x) { const int2 t = ch[0]; ch[0] = ch[1]; ch[1] = t; }
          for (int u = 0; u < 2; u++) {
            if (ch[u].x >= ch[u].y) continue;
            if (ch[u].y - ch[u].x + 1 > kWarpSeg) {
              if (nbs < 64) bstk[nbs++] = ch[u];
              else atomicOr(err, 2048);   // impossible, see above
            } else {
              Z.wl[wl_n++] = ch[u];
            }
          }
        }
        __syncthreads();
      }
      // warp partitions of the queued segments, depth first per warp
      for (;;) {
        int k = 0;
        if (lane == 0) k = atomicAdd(&wl_next, 1);
        k = __shfl_sync(0xffffffffu, k, 0);
        if (k >= wl_n) break;
        const int2 w0 = Z.wl[k];
        if (w0.y - w0.x + 1 <= kTiny) {
          tiny_push(Z, tiny_n, w0);
          continue;
        }
        int stk[2 * 16];
        int sp = 0;
        stk[sp++] = w0.x;
        stk[sp++] = w0.y;
        while (sp > 0) {
          const int hi = stk[--sp], l0 = stk[--sp];
          int i, j;
          warp_part<uint16_t>(Z.a, Z.o, Z.Lp, Z.Rp, l0, hi, i, j);
          int2 ch[2] = {make_int2(l0, i - 1), make_int2(j + 1, hi)};
          if (ch[0].y - ch[0].x < ch[1].y - ch[1].x) { const int2 t = ch[0]; ch[0] = ch[1]; ch[1] = t; }
          for (int u = 0; u < 2; u++) {
            if (ch[u].x >= ch[u].y) continue;
            if (ch[u].y - ch[u].x + 1 > kTiny) {
              if (sp + 2 <= 2 * 16) { stk[sp++] = ch[u].x; stk[sp++] = ch[u].y; }
              else if (lane == 0) atomicOr(err, 4096);   // impossible: depth <= log2(kWarpSeg / kTiny) + 1
            } else {
              tiny_push(Z, tiny_n, ch[u]);
            }
          }
        }
      }
      __syncthreads();
      if (threadIdx.x == 0) { wl_n = 0; wl_next = 0; }
      __syncthreads();
      if (nbs == 0 || round > kNmsSegS) break;
    }
    // the tiny segments still queued
    if (lane < tiny_n[warp]) {
      const int2 t = Z.tiny[warp][lane];
      thread_qsort(Z.a, Z.o, t.x, t.y);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < len; i += kNmsNT) {
      S.val[lo + i] = Z.a[i];
      S.ord[lo + i] = Z.o[i];
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// segments still above kNmsSegS after the launched levels (none on ordinary
// inputs): the whole-block tiers in global memory, one block per model
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kNmsNT) k_qs_rest(int levels, int cap, int *si, float *sf, int *err,
                                                   long long *diag) {
  __shared__ unsigned long long wsum[32];
  __shared__ int sh[8];
  __shared__ int2 q[2][kQ];
  __shared__ int qn[2];
  __shared__ int segn, segnext, tinyn;
  const int m = blockIdx.x;
  Slots S = slots(si, sf, m, cap);
  const int cur = levels & 1;   // the queue the next level would have taken
  const int nbig = S.ss->big_n[cur];
  if (threadIdx.x == 0 && diag) diag[8 * m + 1] = nbig;
  if (nbig == 0) return;
  const int lane = threadIdx.x & 31;
  const int D = S.st->D;
  // the shared-memory kernel is done with S.small: reuse it for the warp and thread tiers
  int2 *segq = S.small;
  if (threadIdx.x == 0) {
    qn[0] = min(nbig, kQ); qn[1] = 0; segn = 0; segnext = 0; tinyn = 0;
    for (int k = 0; k < qn[0]; k++) q[0][k] = S.big[cur][k];
    if (nbig > kQ) atomicOr(err, 8192);
  }
  __syncthreads();
  int c = 0, rounds = 0;
  while (qn[c] > 0) {
    if (++rounds > D) {
      if (threadIdx.x == 0) atomicOr(err, 4);
      break;
    }
    const int nx = c ^ 1;
    if (threadIdx.x == 0) qn[nx] = 0;
    __syncthreads();
    const int nq = qn[c];
    for (int k = 0; k < nq; k++) {
      const int2 seg = q[c][k];
      chunk_partition<int>(S.val, S.ord, S.Lpos, S.Rpos, seg.x, seg.y, wsum, sh);
      if (threadIdx.x == 0) {
        const int i = sh[1], j = sh[2];
        const int2 ch[2] = {make_int2(seg.x, i - 1), make_int2(j + 1, seg.y)};
        for (int u = 0; u < 2; u++) {
          if (ch[u].x >= ch[u].y) continue;
          const int len = ch[u].y - ch[u].x + 1;
          if (len > 4096 && qn[nx] < kQ) q[nx][qn[nx]++] = ch[u];
          else if (len > kTiny) segq[segn++] = ch[u];
          else segq[cap / 2 - 1 - (tinyn++)] = ch[u];
        }
      }
      __syncthreads();
    }
    c = nx;
  }
  for (;;) {
    int idx = 0;
    if (lane == 0) idx = atomicAdd(&segnext, 1);
    idx = __shfl_sync(0xffffffffu, idx, 0);
    if (idx >= segn) break;
    int stk[2 * 24];
    int sp = 0;
    stk[sp++] = segq[idx].x;
    stk[sp++] = segq[idx].y;
    while (sp > 0) {
      const int hi = stk[--sp], lo = stk[--sp];
      int i, j;
      warp_part<int>(S.val, S.ord, S.Lpos, S.Rpos, lo, hi, i, j);
      const int2 ch[2] = {make_int2(lo, i - 1), make_int2(j + 1, hi)};
      const bool ok[2] = {lo < i - 1, hi > j + 1};
      const int big = (ch[0].y - ch[0].x) >= (ch[1].y - ch[1].x) ? 0 : 1;
      for (int t2 = 0; t2 < 2; t2++) {
        const int t = t2 == 0 ? big : 1 - big;
        if (!ok[t]) continue;
        if (ch[t].y - ch[t].x + 1 > kTiny) {
          if (sp + 2 > 2 * 24) {   // unreachable for segments of <= 4096 elements
            if (lane == 0) atomicOr(err, 1);
            continue;
          }
          stk[sp++] = ch[t].x;
          stk[sp++] = ch[t].y;
        } else if (lane == 0) {
          const int ti = atomicAdd(&tinyn, 1);
          segq[cap / 2 - 1 - ti] = ch[t];
        }
      }
      __syncwarp();
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < tinyn; t += kNmsNT) {
    const int2 seg = segq[cap / 2 - 1 - t];
    thread_qsort(S.val, S.ord, seg.x, seg.y);
  }
}

// the default number of grid-wide levels for cap boxes per model: quicksort
// splits are uneven (ties, runs), so three times the balanced depth to
// kNmsSegS, plus three (a level with nothing left costs three empty launches; a
// segment still above kNmsSegS afterwards costs k_qs_rest's single block per
// model far more).  Plans then fit the count to their frames' depth on the host.
int nms_sort_levels(int cap) {
  int depth = 0;
  while (((long long)kNmsSegS << depth) < cap) depth++;
  return std::max(4, std::min(30, 3 * depth + 3));
}

void launch_nms_sort(const float *boxes, const int *d_num, int n_models, int GL, int cap, int *si, float *sf,
                     int *err, long long *diag, int levels, int *lv_used, const int *need, cudaStream_t s) {
  if (levels <= 0) levels = nms_sort_levels(cap);
  k_qs_load<<<dim3((cap + 255) / 256, n_models), 256, 0, s>>>(boxes, d_num, GL, cap, si, sf, need);
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int tiles = std::max(1, std::min(nms_tile_cap(cap), std::max(1, 2 * sms / std::max(1, n_models))));
  for (int l = 0; l < levels; l++) {
    k_qs_count<<<dim3(tiles, n_models), kNmsNT, 0, s>>>(l, cap, si, sf, lv_used);
    k_qs_scatter<<<dim3(tiles, n_models), kNmsNT, 0, s>>>(l, cap, si, sf);
    k_qs_swap<<<dim3(tiles, n_models), kNmsNT, 0, s>>>(l, cap, si, sf, err);
  }
  static SmemAttr attr;
  raise_smem(attr, k_qs_small, sizeof(SmallSmem));
  k_qs_small<<<std::max(1, sms), kNmsNT, sizeof(SmallSmem), s>>>(n_models, cap, si, sf, err);
  k_qs_rest<<<n_models, kNmsNT, 0, s>>>(levels, cap, si, sf, err, diag);
}

}  // namespace geye
