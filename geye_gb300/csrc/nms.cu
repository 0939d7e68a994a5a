// nms.cu -- greedy non-maximum suppression, one thread block per model.
//
// Reference: CAR_TRACKING/nms.cpp:70-84 (quickSort) and :94-217 (nms).
//
// Sorting.  The kept set depends on the order of equal scores, which is the
// order the reference's recursive Hoare quicksort leaves them in (key = the
// middle element, i stops at a[i] <= key, j at a[j] >= key, swap, recurse on
// [lo, i-1] and [j+1, hi]).  That order is reproduced exactly with a parallel
// partition: let L be the positions with a <= key in ascending order and R
// the positions with a >= key in descending order (original values).  The
// k-th swap of the sequential loop exchanges L[k] and R[k] for every k < K,
// K = #{k : L[k] < R[k]} (a prefix, since L rises and R falls); the scan then
// stops at i = min(L[K], R[K-1]), j = max(R[K], L[K-1]) (i = L[0], j = R[0]
// when K = 0).  Positions strictly between two swapped pairs are never touched,
// so these ranks can be taken on the unswapped segment.  Large segments are
// partitioned by the whole block, segments of <= kWarpSeg elements by one
// warp each (depth-first with a small stack).
//
// Suppression.  Standard greedy in sorted order: overlap = w*h / min(area)
// (not IoU), plus containment when the intersection is empty; the loop runs
// while cnum > 0 with cnum starting at NUM-1, so the last box that would be
// kept is never emitted.  The kept records are written in input order.
#include "internal.h"

namespace geye {

constexpr int kNmsThreads = 1024;
constexpr int kWarpSeg = 2048;
constexpr int kBigQueue = 2048;

struct NmsScratch {
  float *val;     // D
  int *ord;       // D
  int *Lpos;      // D
  int *Rpos;      // D
  float *sb;      // 5*D: sorted y1, x1, y2, x2, area
  int *checked;   // D
  int2 *wq;       // D/2+1 warp-tier segments
};

__device__ __forceinline__ NmsScratch nms_scratch(float *sf, int *si, int cap) {
  NmsScratch S;
  S.val = sf;
  S.sb = sf + cap;
  S.ord = si;
  S.Lpos = si + cap;
  S.Rpos = si + 2 * cap;
  S.checked = si + 3 * cap;
  S.wq = reinterpret_cast<int2 *>(si + 4 * cap);
  return S;
}

// block-wide exclusive scan of one flag per thread; returns the prefix, *total gets the block sum
__device__ __forceinline__ int block_scan_flag(int flag, int *warp_buf, int &total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned bal = __ballot_sync(0xffffffffu, flag);
  __syncthreads();
  if (lane == 0) warp_buf[warp] = __popc(bal);
  __syncthreads();
  int before = 0, tot = 0;
  for (int w = 0; w < kNmsThreads / 32; w++) {
    const int c = warp_buf[w];
    if (w < warp) before += c;
    tot += c;
  }
  total = tot;
  return before + __popc(bal & ((1u << lane) - 1));
}

// one partition of [lo, hi] by the whole block; returns (i, j) through smem
__device__ void block_partition(NmsScratch &S, int lo, int hi, int *warp_buf, int *sh) {
  const float key = S.val[(lo + hi) / 2];
  __syncthreads();
  int *Lp = S.Lpos + lo, *Rp = S.Rpos + lo;
  int nL = 0, nR = 0;
  for (int base = lo; base <= hi; base += kNmsThreads) {
    const int p = base + threadIdx.x;
    const int f = p <= hi && !(S.val[p] > key);
    int tot;
    const int r = block_scan_flag(f, warp_buf, tot);
    if (f) Lp[nL + r] = p;
    nL += tot;
  }
  for (int top = hi; top >= lo; top -= kNmsThreads) {
    const int p = top - threadIdx.x;
    const int f = p >= lo && !(S.val[p] < key);
    int tot;
    const int r = block_scan_flag(f, warp_buf, tot);
    if (f) Rp[nR + r] = p;
    nR += tot;
  }
  __syncthreads();
  const int lim = min(nL, nR);
  int cnt = 0;
  for (int k = threadIdx.x; k < lim; k += kNmsThreads) cnt += Lp[k] < Rp[k];
  // block reduction of cnt
  {
    int v = cnt;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) warp_buf[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
      int K = 0;
      for (int w = 0; w < kNmsThreads / 32; w++) K += warp_buf[w];
      sh[0] = K;
    }
    __syncthreads();
  }
  const int K = sh[0];
  for (int k = threadIdx.x; k < K; k += kNmsThreads) {
    const int a = Lp[k], b = Rp[k];
    const float tv = S.val[a]; S.val[a] = S.val[b]; S.val[b] = tv;
    const int to = S.ord[a]; S.ord[a] = S.ord[b]; S.ord[b] = to;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int i, j;
    if (K == 0) { i = Lp[0]; j = Rp[0]; }
    else {
      i = K < nL ? min(Lp[K], Rp[K - 1]) : Rp[K - 1];
      j = K < nR ? max(Rp[K], Lp[K - 1]) : Lp[K - 1];
    }
    sh[1] = i;
    sh[2] = j;
  }
  __syncthreads();
}

// one partition of [lo, hi] by one warp
__device__ void warp_partition(NmsScratch &S, int lo, int hi, int &oi, int &oj) {
  const int lane = threadIdx.x & 31;
  const float key = S.val[(lo + hi) / 2];
  __syncwarp();
  int *Lp = S.Lpos + lo, *Rp = S.Rpos + lo;
  int nL = 0, nR = 0;
  for (int base = lo; base <= hi; base += 32) {
    const int p = base + lane;
    const int f = p <= hi && !(S.val[p] > key);
    const unsigned bal = __ballot_sync(0xffffffffu, f);
    if (f) Lp[nL + __popc(bal & ((1u << lane) - 1))] = p;
    nL += __popc(bal);
  }
  for (int top = hi; top >= lo; top -= 32) {
    const int p = top - lane;
    const int f = p >= lo && !(S.val[p] < key);
    const unsigned bal = __ballot_sync(0xffffffffu, f);
    if (f) Rp[nR + __popc(bal & ((1u << lane) - 1))] = p;
    nR += __popc(bal);
  }
  __syncwarp();
  const int lim = min(nL, nR);
  int K = 0;
  for (int k0 = 0; k0 < lim; k0 += 32) {
    const int k = k0 + lane;
    const unsigned bal = __ballot_sync(0xffffffffu, k < lim && Lp[k] < Rp[k]);
    K += __popc(bal);
    if (bal != 0xffffffffu) break;   // the true set is a prefix
  }
  for (int k = lane; k < K; k += 32) {
    const int a = Lp[k], b = Rp[k];
    const float tv = S.val[a]; S.val[a] = S.val[b]; S.val[b] = tv;
    const int to = S.ord[a]; S.ord[a] = S.ord[b]; S.ord[b] = to;
  }
  __syncwarp();
  if (K == 0) { oi = Lp[0]; oj = Rp[0]; }
  else {
    oi = K < nL ? min(Lp[K], Rp[K - 1]) : Rp[K - 1];
    oj = K < nR ? max(Rp[K], Lp[K - 1]) : Lp[K - 1];
  }
}

__device__ __forceinline__ bool nms_suppress(float Ay1, float Ax1, float Ay2, float Ax2, float areaA, float By1,
                                             float Bx1, float By2, float Bx2, float areaB, float overlap) {
  const float yy1 = Ay1 >= By1 ? Ay1 : By1;
  const float xx1 = Ax1 >= Bx1 ? Ax1 : Bx1;
  const float yy2 = Ay2 <= By2 ? Ay2 : By2;
  const float xx2 = Ax2 <= Bx2 ? Ax2 : Bx2;
  // the reference adds the double 1.0 and stores a float: the float addition
  // rounds the same exact sum once
  const float w = xx2 - xx1 + 1.0f;
  const float h = yy2 - yy1 + 1.0f;
  const float R_AREA = areaA <= areaB ? areaA : areaB;
  if (w > 0 && h > 0) {
    const float o = w * h / R_AREA;
    return o > overlap;
  }
  if (Ay1 < By1 && Ax1 < Bx1 && Ay2 > By2 && Ax2 > Bx2) return true;
  if (Ay1 > By1 && Ax1 > Bx1 && Ay2 < By2 && Ax2 < Bx2) return true;
  return false;
}

__global__ void __launch_bounds__(kNmsThreads) k_nms(const float *__restrict__ boxes_all, const int *__restrict__ d_num,
                                                      int GL, float overlap, int cap, float *scratch_f,
                                                      int *scratch_i, float *out_all, int *d_kept, int *err) {
  __shared__ int warp_buf[kNmsThreads / 32];
  __shared__ int sh[8];
  __shared__ int2 bigq[2][kBigQueue];
  __shared__ int qn[2];
  __shared__ int wq_n, wq_next;
  // one block per model: model m's boxes, scratch and outputs are cap-strided
  const int m = blockIdx.x;
  const float *boxes = boxes_all + (size_t)m * cap * GL;
  float *out = out_all + (size_t)m * cap * GL;
  NmsScratch S = nms_scratch(scratch_f + (size_t)m * cap * 6, scratch_i + (size_t)m * cap * 5, cap);
  const int D = min(d_num[m], cap);
  if (D <= 0) {
    if (threadIdx.x == 0) d_kept[m] = 0;
    return;
  }
  for (int i = threadIdx.x; i < D; i += kNmsThreads) {
    const float *P = boxes + (size_t)i * GL;
    S.val[i] = P[GL - 2];
    S.ord[i] = i;
  }
  if (threadIdx.x == 0) {
    qn[0] = 0; qn[1] = 0; wq_n = 0; wq_next = 0;
    if (D > 1) {
      if (D > kWarpSeg) { bigq[0][0] = make_int2(0, D - 1); qn[0] = 1; }
      else { S.wq[0] = make_int2(0, D - 1); wq_n = 1; }
    }
  }
  __syncthreads();
  // ---- block tier: rounds of large segments
  int cur = 0, rounds = 0;
  while (qn[cur] > 0) {
    if (++rounds > D) {   // every round shrinks each segment; bounded by D
      if (threadIdx.x == 0) atomicOr(err, 4);
      break;
    }
    const int nxt = cur ^ 1;
    if (threadIdx.x == 0) qn[nxt] = 0;
    __syncthreads();
    for (int q = 0; q < qn[cur]; q++) {
      const int2 seg = bigq[cur][q];
      block_partition(S, seg.x, seg.y, warp_buf, sh);
      if (threadIdx.x == 0) {
        const int i = sh[1], j = sh[2];
        int2 c[2] = {make_int2(seg.x, i - 1), make_int2(j + 1, seg.y)};
        bool ok[2] = {seg.x < i - 1, seg.y > j + 1};
        for (int t = 0; t < 2; t++) {
          if (!ok[t]) continue;
          const int len = c[t].y - c[t].x + 1;
          if (len > kWarpSeg && qn[nxt] < kBigQueue) bigq[nxt][qn[nxt]++] = c[t];
          else S.wq[wq_n++] = c[t];   // (queue overflow falls back to the warp tier: still exact)
        }
      }
      __syncthreads();
    }
    cur = nxt;
    __syncthreads();
  }
  // ---- warp tier: each warp sorts whole segments depth-first
  {
    const int lane = threadIdx.x & 31;
    for (;;) {
      int idx = 0;
      if (lane == 0) idx = atomicAdd(&wq_next, 1);
      idx = __shfl_sync(0xffffffffu, idx, 0);
      if (idx >= wq_n) break;
      int stk[2 * 48];
      int sp = 0;
      stk[sp++] = S.wq[idx].x;
      stk[sp++] = S.wq[idx].y;
      while (sp > 0) {
        const int hi = stk[--sp], lo = stk[--sp];
        int i, j;
        warp_partition(S, lo, hi, i, j);
        // recursion order does not matter (disjoint segments); push the larger first
        const bool l = lo < i - 1, r = hi > j + 1;
        if (sp + 4 > 2 * 48) {
          // unreachable: with the larger half pushed first the stack holds at
          // most log2(kWarpSeg) pending segments; report instead of dropping work
          if (lane == 0) atomicOr(err, 1);
          break;
        }
        if (l && r) {
          if ((i - 1 - lo) > (hi - j - 1)) { stk[sp++] = lo; stk[sp++] = i - 1; stk[sp++] = j + 1; stk[sp++] = hi; }
          else { stk[sp++] = j + 1; stk[sp++] = hi; stk[sp++] = lo; stk[sp++] = i - 1; }
        } else if (l) { stk[sp++] = lo; stk[sp++] = i - 1; }
        else if (r) { stk[sp++] = j + 1; stk[sp++] = hi; }
      }
    }
  }
  __syncthreads();
  // ---- gather sorted boxes
  float *sy1 = S.sb, *sx1 = S.sb + cap, *sy2 = S.sb + 2 * cap, *sx2 = S.sb + 3 * cap, *sar = S.sb + 4 * cap;
  for (int k = threadIdx.x; k < D; k += kNmsThreads) {
    const float *P = boxes + (size_t)S.ord[k] * GL;
    sy1[k] = P[0]; sx1[k] = P[1]; sy2[k] = P[2]; sx2[k] = P[3];
    sar[k] = (P[3] - P[1] + 1.0) * (P[2] - P[0] + 1.0);
    S.checked[k] = 0;
  }
  __syncthreads();
  // ---- greedy suppression
  int cnum = D - 1, A = 0, iters = 0;
  while (cnum > 0) {
    // each pass removes at least one unchecked box, so D passes always suffice
    if (++iters > D) {
      if (threadIdx.x == 0) atomicOr(err, 2);
      break;
    }
    if (threadIdx.x == 0) S.checked[A] = 1;
    const float Ay1 = sy1[A], Ax1 = sx1[A], Ay2 = sy2[A], Ax2 = sx2[A], aA = sar[A];
    int supp = 0, first = 0x7fffffff;
    for (int kk = A + 1 + threadIdx.x; kk < D; kk += kNmsThreads) {
      if (S.checked[kk] != 0) continue;
      if (nms_suppress(Ay1, Ax1, Ay2, Ax2, aA, sy1[kk], sx1[kk], sy2[kk], sx2[kk], sar[kk], overlap)) {
        S.checked[kk] = -1;
        supp++;
      } else if (kk < first) first = kk;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      supp += __shfl_xor_sync(0xffffffffu, supp, o);
      first = min(first, __shfl_xor_sync(0xffffffffu, first, o));
    }
    __syncthreads();
    if ((threadIdx.x & 31) == 0) { warp_buf[threadIdx.x >> 5] = supp; bigq[0][threadIdx.x >> 5].x = first; }
    __syncthreads();
    int tot = 0, nf = 0x7fffffff;
    for (int w = 0; w < kNmsThreads / 32; w++) { tot += warp_buf[w]; nf = min(nf, bigq[0][w].x); }
    cnum = cnum - 1 - tot;
    if (nf != 0x7fffffff) A = nf;
    __syncthreads();
  }
  __syncthreads();
  // ---- keep flags back to input order, then compact the kept records
  int *keep = S.Lpos;   // reuse: input-order flags
  for (int k = threadIdx.x; k < D; k += kNmsThreads) keep[S.ord[k]] = S.checked[k] == 1;
  __syncthreads();
  int written = 0;
  for (int base = 0; base < D; base += kNmsThreads) {
    const int i = base + threadIdx.x;
    const int f = i < D && keep[i];
    int tot;
    const int r = block_scan_flag(f, warp_buf, tot);
    if (f) {
      const float *P = boxes + (size_t)i * GL;
      float *Q = out + (size_t)(written + r) * GL;
      for (int q = 0; q < GL; q++) Q[q] = P[q];
    }
    written += tot;
  }
  if (threadIdx.x == 0) d_kept[m] = written;
}

void launch_nms(const float *boxes, const int *d_num, int n_models, int GL, float overlap, int cap,
                float *scratch_f, int *scratch_i, float *out, int *d_kept, int *err, cudaStream_t s) {
  k_nms<<<n_models, kNmsThreads, 0, s>>>(boxes, d_num, GL, overlap, cap, scratch_f, scratch_i, out, d_kept, err);
}

}  // namespace geye
