// nms_common.h -- scratch layout and device routines shared by the pipeline
// NMS kernels (nms_sort.cu: the reference's quicksort; nms_batch.cu: the
// greedy suppression).  Reference: CAR_TRACKING/nms.cpp:70-217.
#pragma once
#include <stdint.h>

#include "internal.h"

namespace geye {

constexpr int kNmsNT = 1024;   // threads of the whole-block kernels
constexpr int kTiny = 32;      // sort segments finished by one thread

struct BatchState {   // greedy rounds
  int D, nwords, scan_word, npicks;
  int npb, done, batches, fallback;
};

struct SortState {    // grid-wide partition levels
  int big_n[2];       // segments above kNmsSegS, double-buffered by level parity
  int small_n;        // segments of 2..kNmsSegS elements, sorted in shared memory
  int pad[5];
};

// per-model scratch: nms_model_words(cap) ints and 5 * cap floats
struct Slots {
  float *val;        // sort keys
  int *ord;          // sorted position -> box
  int *Lpos, *Rpos;  // partition lists; Rpos holds keep flags at the end
  int2 *small;       // cap/2 sort segments for the shared-memory kernel
  int *picks;        // sorted positions of the picks, in pick order
  int *flag;         // per pick: it suppressed at least one box
  unsigned *bits;    // alive bitmap over sorted positions
  BatchState *st;
  SortState *ss;
  float *bp;         // current round's picks: y1, x1, y2, x2, area (kNmsBatch each)
  int2 *big[2];      // nms_big_cap(cap) segments each
  int2 *tiles;       // nms_tile_cap(cap) per-tile (<= key, >= key) counts
  int *hist;         // 256 * nms_rs_tiles(cap) radix-sort digit counts (nms_radix.cu)
  unsigned *sbits;   // summary of bits: bit w set while word w has an alive box
  unsigned *cmask;   // the round's picks by cell: [axis y, x][level][cell][pick word] (nms_batch.cu)
  float *y1, *x1, *y2, *x2, *ar;   // boxes in sorted order
};

__device__ __forceinline__ Slots slots(int *si, float *sf, int m, int cap) {
  int *b = si + (size_t)m * nms_model_words(cap);
  float *f = sf + (size_t)m * 5 * cap;
  Slots S;
  S.val = reinterpret_cast<float *>(b);
  S.ord = b + cap;
  S.Lpos = b + 2 * (size_t)cap;
  S.Rpos = b + 3 * (size_t)cap;
  S.small = reinterpret_cast<int2 *>(b + 4 * (size_t)cap);
  S.picks = b + 5 * (size_t)cap;
  S.flag = b + 6 * (size_t)cap;
  S.bits = reinterpret_cast<unsigned *>(b + 7 * (size_t)cap);
  int *t = b + 8 * (size_t)cap;
  S.st = reinterpret_cast<BatchState *>(t);
  S.ss = reinterpret_cast<SortState *>(t + 8);
  S.bp = reinterpret_cast<float *>(t + 64);
  int *l = t + 64 + 5 * kNmsBatch;
  const int bc = nms_big_cap(cap);
  S.big[0] = reinterpret_cast<int2 *>(l);
  S.big[1] = reinterpret_cast<int2 *>(l + 2 * bc);
  S.tiles = reinterpret_cast<int2 *>(l + 4 * bc);
  S.hist = l + 4 * bc + 2 * nms_tile_cap(cap);
  S.sbits = reinterpret_cast<unsigned *>(S.hist + 256 * (size_t)nms_rs_tiles(cap));
  S.cmask = S.sbits + nms_summary_words(cap);
  S.y1 = f;
  S.x1 = f + cap;
  S.y2 = f + 2 * (size_t)cap;
  S.x2 = f + 3 * (size_t)cap;
  S.ar = f + 4 * (size_t)cap;
  return S;
}

// ---------------------------------------------------------------------------
// Quicksort partitions.  Each reproduces one pass of nms.cpp:70-84's loop
// (key = the middle element, i stops at a[i] <= key, j at a[j] >= key, swap,
// recurse on [lo, i-1] and [j+1, hi]): with L the positions holding a value
// <= key in ascending order and R those holding a value >= key in descending
// order, the sequential loop swaps L[k] with R[k] for every k < K,
// K = #{k : L[k] < R[k]} (a prefix, since L rises and R falls), and stops at
// i = min(L[K], R[K-1]), j = max(R[K], L[K-1]) (i = L[0], j = R[0] when K = 0).
// P is the position type of the L/R lists (int in global memory, uint16_t for
// a segment in shared memory).
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long warp_incl_scan64(unsigned long long v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    unsigned long long t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

__device__ __forceinline__ void part_bounds(const int *Lp, const int *Rp, int K, int nL, int nR, int &i, int &j) {
  if (K == 0) { i = Lp[0]; j = Rp[0]; }
  else {
    i = K < nL ? min(Lp[K], Rp[K - 1]) : Rp[K - 1];
    j = K < nR ? max(Rp[K], Lp[K - 1]) : Lp[K - 1];
  }
}

// partition val[lo..hi] by the whole block (kNmsNT threads, each owning a
// contiguous chunk); result (i, j) in sh[1], sh[2]
template <class P>
__device__ void chunk_partition(float *val, int *ord, P *Lpos, P *Rpos, int lo, int hi, unsigned long long *wsum,
                                int *sh) {
  const int m = hi - lo + 1;
  const float key = val[(lo + hi) / 2];
  const int cs = (m + kNmsNT - 1) / kNmsNT;
  const int t0 = lo + threadIdx.x * cs, t1 = min(t0 + cs, hi + 1);
  unsigned cL = 0, cR = 0;
  for (int p = t0; p < t1; p++) {
    const float v = val[p];
    cL += !(v > key);
    cR += !(v < key);
  }
  // block exclusive scan of (cL, cR) packed into 64 bits
  const unsigned long long mine = ((unsigned long long)cL << 32) | cR;
  const unsigned long long inc = warp_incl_scan64(mine);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 31) wsum[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    unsigned long long w = wsum[lane];
    w = warp_incl_scan64(w);
    wsum[lane] = w;   // inclusive over warps
  }
  __syncthreads();
  const unsigned long long before = (warp ? wsum[warp - 1] : 0ull) + inc - mine;
  const unsigned long long tot = wsum[31];
  const int nL = (int)(tot >> 32), nR = (int)(tot & 0xffffffffu);
  int rl = (int)(before >> 32), rr = (int)(before & 0xffffffffu);
  P *Lp = Lpos + lo, *Rp = Rpos + lo;
  for (int p = t0; p < t1; p++) {
    const float v = val[p];
    if (!(v > key)) Lp[rl++] = (P)p;
    if (!(v < key)) Rp[nR - 1 - (rr++)] = (P)p;
  }
  __syncthreads();
  const int lim = min(nL, nR);
  int cnt = 0;
  for (int k = threadIdx.x; k < lim; k += kNmsNT) cnt += (int)Lp[k] < (int)Rp[k];
  cnt = __syncthreads_count(0) + cnt;   // barrier: all counts computed before wsum reuse
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  if (lane == 0) wsum[warp] = (unsigned long long)cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    int K = 0;
    for (int w = 0; w < kNmsNT / 32; w++) K += (int)wsum[w];
    sh[0] = K;
  }
  __syncthreads();
  const int K = sh[0];
  for (int k = threadIdx.x; k < K; k += kNmsNT) {
    const int a = Lp[k], b = Rp[k];
    const float tv = val[a]; val[a] = val[b]; val[b] = tv;
    const int to = ord[a]; ord[a] = ord[b]; ord[b] = to;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int i, j;
    if (K == 0) { i = Lp[0]; j = Rp[0]; }
    else {
      i = K < nL ? min((int)Lp[K], (int)Rp[K - 1]) : (int)Rp[K - 1];
      j = K < nR ? max((int)Rp[K], (int)Lp[K - 1]) : (int)Lp[K - 1];
    }
    sh[1] = i;
    sh[2] = j;
  }
  __syncthreads();
}

// partition val[lo..hi] by one warp
template <class P>
__device__ void warp_part(float *val, int *ord, P *Lpos, P *Rpos, int lo, int hi, int &oi, int &oj) {
  const int lane = threadIdx.x & 31;
  const float key = val[(lo + hi) / 2];
  P *Lp = Lpos + lo, *Rp = Rpos + lo;
  int nL = 0, nR = 0;
  for (int base = lo; base <= hi; base += 32) {
    const int p = base + lane;
    const int f = p <= hi && !(val[p] > key);
    const unsigned bal = __ballot_sync(0xffffffffu, f);
    if (f) Lp[nL + __popc(bal & ((1u << lane) - 1))] = (P)p;
    nL += __popc(bal);
  }
  for (int top = hi; top >= lo; top -= 32) {
    const int p = top - lane;
    const int f = p >= lo && !(val[p] < key);
    const unsigned bal = __ballot_sync(0xffffffffu, f);
    if (f) Rp[nR + __popc(bal & ((1u << lane) - 1))] = (P)p;
    nR += __popc(bal);
  }
  __syncwarp();
  const int lim = min(nL, nR);
  int K = 0;
  for (int k0 = 0; k0 < lim; k0 += 32) {
    const int k = k0 + lane;
    const unsigned bal = __ballot_sync(0xffffffffu, k < lim && (int)Lp[k] < (int)Rp[k]);
    K += __popc(bal);
    if (bal != 0xffffffffu) break;
  }
  for (int k = lane; k < K; k += 32) {
    const int a = Lp[k], b = Rp[k];
    const float tv = val[a]; val[a] = val[b]; val[b] = tv;
    const int to = ord[a]; ord[a] = ord[b]; ord[b] = to;
  }
  __syncwarp();
  if (K == 0) { oi = Lp[0]; oj = Rp[0]; }
  else {
    oi = K < nL ? min((int)Lp[K], (int)Rp[K - 1]) : (int)Rp[K - 1];
    oj = K < nR ? max((int)Rp[K], (int)Lp[K - 1]) : (int)Lp[K - 1];
  }
  __syncwarp();
}

// the reference's recursive quicksort, one thread, segment of <= kTiny elements
__device__ __forceinline__ void thread_qsort(float *a, int *ord, int lo0, int hi0) {
  int st[2 * 16];
  int sp = 0;
  st[sp++] = lo0; st[sp++] = hi0;
  while (sp > 0) {
    const int last = st[--sp], first = st[--sp];
    int i = first, j = last;
    const float key = a[(first + last) / 2];
    for (;;) {
      while (a[i] > key) i++;
      while (a[j] < key) j--;
      if (i >= j) break;
      const float tv = a[i]; a[i] = a[j]; a[j] = tv;
      const int to = ord[i]; ord[i] = ord[j]; ord[j] = to;
      i++; j--;
    }
    const bool l = first < i - 1, r = last > j + 1;
    // larger half first so the smaller is popped next: depth <= log2(kTiny) + 1
    if (l && r) {
      if (i - 1 - first > last - j - 1) { st[sp++] = first; st[sp++] = i - 1; st[sp++] = j + 1; st[sp++] = last; }
      else { st[sp++] = j + 1; st[sp++] = last; st[sp++] = first; st[sp++] = i - 1; }
    } else if (l) { st[sp++] = first; st[sp++] = i - 1; }
    else if (r) { st[sp++] = j + 1; st[sp++] = last; }
    if (sp > 2 * 16 - 4) break;   // unreachable for kTiny = 32
  }
}

// suppression test (nms.cpp:141-176); A is the kept box, B the other one
__device__ __forceinline__ bool supp(float Ay1, float Ax1, float Ay2, float Ax2, float aA, float By1, float Bx1,
                                     float By2, float Bx2, float aB, float overlap) {
  const float yy1 = Ay1 >= By1 ? Ay1 : By1;
  const float xx1 = Ax1 >= Bx1 ? Ax1 : Bx1;
  const float yy2 = Ay2 <= By2 ? Ay2 : By2;
  const float xx2 = Ax2 <= Bx2 ? Ax2 : Bx2;
  // nms.cpp adds the double 1.0 and stores a float: one rounding of the exact
  // sum, which is what the float addition gives (no FP64 in the inner loop)
  const float w = xx2 - xx1 + 1.0f;
  const float h = yy2 - yy1 + 1.0f;
  const float R_AREA = aA <= aB ? aA : aB;
  if (w > 0 && h > 0) return w * h / R_AREA > overlap;
  if (Ay1 < By1 && Ax1 < Bx1 && Ay2 > By2 && Ax2 > Bx2) return true;
  if (Ay1 > By1 && Ax1 > Bx1 && Ay2 < By2 && Ax2 < Bx2) return true;
  return false;
}

// sort stage (nms_sort.cu): leaves val/ord sorted for every model and the
// BatchState initialised; diag[8m + 1] gets the segments left to k_qs_rest.
// levels: grid-wide partition levels to launch (<= 0: nms_sort_levels(cap));
// *lv_used (optional) gets the deepest level that had a segment to partition.
// need (optional): only the models with need[m] set are sorted; the others
// are left with an empty, finished state
void launch_nms_sort(const float *boxes, const int *d_num, int n_models, int GL, int cap, int *si, float *sf,
                     int *err, long long *diag, int levels, int *lv_used, const int *need, cudaStream_t s);
// key-order sort (nms_radix.cu): val = transformed keys, ord = input index,
// BatchState initialised; need[m] set for a NaN score
void launch_nms_radix(const float *boxes, const int *d_num, int n_models, int GL, int cap, int *si, float *sf,
                      int *need, cudaStream_t s);

}  // namespace geye
