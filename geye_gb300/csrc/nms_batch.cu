// nms_batch.cu -- NMS of the pipeline's detections, every model of a frame at once.
//
// Same kept set as nms.cu (CAR_TRACKING/nms.cpp:70-217): the reference's Hoare
// quicksort order for equal scores, greedy suppression by intersection over
// the smaller area or containment, and a box that is alone when its turn comes
// never emitted.  The greedy loop is restated so that most of it runs on every
// SM:
//
//  1. k_nms_sort (one block per model): the quicksort (partition argument in
//     nms.cu): segments above kSeg partitioned by the whole block, each thread
//     owning a contiguous chunk; segments of kTiny+1..kSeg by one warp each;
//     the rest by one thread each.
//  2. k_nms_gather: the boxes in sorted order (structure of arrays) and an
//     alive bitmap over sorted positions.
//  3. Rounds of two kernels, each a no-op for a model that is done:
//     k_nms_resolve (one block per model) takes the first kBatch alive boxes
//     in sorted order, computes their pairwise suppression bits and walks
//     them in order: a member is picked unless an earlier pick of the batch
//     suppresses it -- the sequential loop's decisions for these boxes, since
//     every box before them is already resolved.
//     k_nms_pass (grid) tests every other alive box against the batch's picks
//     in pick order; the first pick that suppresses it is the one the
//     sequential loop would have removed it with.
//  4. k_nms_finish (one block per model) runs any remaining rounds itself,
//     drops the final pick if it suppressed nothing (the reference's
//     `while (cnum > 0)` with cnum = NUM-1 never takes a box that is alone at
//     its turn) and writes the kept records in input order.
#include "internal.h"

namespace geye {

constexpr int kSortNT = 1024;   // threads of the sort, resolve and finish blocks
constexpr int kSeg = 4096;      // block-tier threshold of the sort
constexpr int kTiny = 32;       // thread-tier threshold of the sort
constexpr int kQ = 1024;        // block-tier queue capacity (shared memory)
constexpr int kBatch = kNmsBatch;
constexpr int kBW = kBatch / 32;   // words of a suppression row
constexpr int kPassNT = 256;
constexpr int kRounds = 8;      // resolve/pass rounds launched before the finish kernel

struct BatchState {
  int D, nwords, scan_word, npicks;
  int npb, done, batches, fallback;
};

// per-model scratch: nms_model_words(cap) ints and 5 * cap floats
struct Slots {
  float *val;        // sort keys
  int *ord;          // sorted position -> box
  int *Lpos, *Rpos;  // partition lists; Rpos holds keep flags at the end
  int2 *segq;        // cap/2 segments (warp tier from the front, thread tier from the back)
  int *picks;        // sorted positions of the picks, in pick order
  int *flag;         // per pick: it suppressed at least one box
  unsigned *bits;    // alive bitmap over sorted positions
  BatchState *st;
  float *bp;         // current batch's picks: y1, x1, y2, x2, area (kBatch each)
  const float *y1, *x1, *y2, *x2, *ar;   // boxes in sorted order
};

__device__ __forceinline__ Slots slots(int *si, float *sf, int m, int cap) {
  int *b = si + (size_t)m * nms_model_words(cap);
  float *f = sf + (size_t)m * 5 * cap;
  Slots S;
  S.val = reinterpret_cast<float *>(b);
  S.ord = b + cap;
  S.Lpos = b + 2 * (size_t)cap;
  S.Rpos = b + 3 * (size_t)cap;
  S.segq = reinterpret_cast<int2 *>(b + 4 * (size_t)cap);
  S.picks = b + 5 * (size_t)cap;
  S.flag = b + 6 * (size_t)cap;
  S.bits = reinterpret_cast<unsigned *>(b + 7 * (size_t)cap);
  S.st = reinterpret_cast<BatchState *>(b + 8 * (size_t)cap);
  S.bp = reinterpret_cast<float *>(b + 8 * (size_t)cap + 64);
  S.y1 = f;
  S.x1 = f + cap;
  S.y2 = f + 2 * (size_t)cap;
  S.x2 = f + 3 * (size_t)cap;
  S.ar = f + 4 * (size_t)cap;
  return S;
}

// ---------------------------------------------------------------------------
// sort tiers (each partition reproduces one pass of nms.cpp:70-84's loop)
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

// partition [lo, hi] by the whole block; result (i, j) in sh[1], sh[2]
__device__ void chunk_partition(Slots &S, int lo, int hi, unsigned long long *wsum, int *sh) {
  const int m = hi - lo + 1;
  const float key = S.val[(lo + hi) / 2];
  const int cs = (m + kSortNT - 1) / kSortNT;
  const int t0 = lo + threadIdx.x * cs, t1 = min(t0 + cs, hi + 1);
  unsigned cL = 0, cR = 0;
  for (int p = t0; p < t1; p++) {
    const float v = S.val[p];
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
  int *Lp = S.Lpos + lo, *Rp = S.Rpos + lo;
  for (int p = t0; p < t1; p++) {
    const float v = S.val[p];
    if (!(v > key)) Lp[rl++] = p;
    if (!(v < key)) Rp[nR - 1 - (rr++)] = p;
  }
  __syncthreads();
  const int lim = min(nL, nR);
  int cnt = 0;
  for (int k = threadIdx.x; k < lim; k += kSortNT) cnt += Lp[k] < Rp[k];
  cnt = __syncthreads_count(0) + cnt;   // barrier: all counts computed before wsum reuse
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  if (lane == 0) wsum[warp] = (unsigned long long)cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    int K = 0;
    for (int w = 0; w < kSortNT / 32; w++) K += (int)wsum[w];
    sh[0] = K;
  }
  __syncthreads();
  const int K = sh[0];
  for (int k = threadIdx.x; k < K; k += kSortNT) {
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

__device__ void warp_part(Slots &S, int lo, int hi, int &oi, int &oj) {
  const int lane = threadIdx.x & 31;
  const float key = S.val[(lo + hi) / 2];
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
    if (bal != 0xffffffffu) break;
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
  __syncwarp();
}

// the reference's recursive quicksort, one thread, segment of <= kTiny elements
__device__ void thread_qsort(float *a, int *ord, int lo0, int hi0) {
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

// ---------------------------------------------------------------------------
// 1. sort
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kSortNT) k_nms_sort(const float *__restrict__ boxes_all,
                                                      const int *__restrict__ d_num, int GL, int cap, int *si,
                                                      float *sf, int *err, long long *diag) {
  __shared__ unsigned long long wsum[32];
  __shared__ int sh[8];
  __shared__ int2 q[2][kQ];
  __shared__ int qn[2];
  __shared__ int segn, segnext, tinyn;
  const int m = blockIdx.x;
  const float *boxes = boxes_all + (size_t)m * cap * GL;
  Slots S = slots(si, sf, m, cap);
  const int D = max(0, min(d_num[m], cap));
  const int lane = threadIdx.x & 31;
  const long long t_start = clock64();
  for (int i = threadIdx.x; i < D; i += kSortNT) {
    S.val[i] = boxes[(size_t)i * GL + GL - 2];
    S.ord[i] = i;
  }
  if (threadIdx.x == 0) {
    BatchState &st = *S.st;
    st.D = D;
    st.nwords = (D + 31) >> 5;
    st.scan_word = 0;
    st.npicks = 0;
    st.npb = 0;
    st.done = D <= 0;
    st.batches = 0;
    st.fallback = 0;
    qn[0] = 0; qn[1] = 0; segn = 0; segnext = 0; tinyn = 0;
    if (D > 1) {
      if (D > kSeg) { q[0][0] = make_int2(0, D - 1); qn[0] = 1; }
      else if (D > kTiny) { S.segq[0] = make_int2(0, D - 1); segn = 1; }
      else { S.segq[cap / 2 - 1] = make_int2(0, D - 1); tinyn = 1; }
    }
  }
  __syncthreads();
  // ---- block tier
  int cur = 0, rounds = 0;
  while (qn[cur] > 0) {
    if (++rounds > D) {   // every round shrinks each segment, so D rounds always suffice
      if (threadIdx.x == 0) atomicOr(err, 4);
      break;
    }
    const int nxt = cur ^ 1;
    if (threadIdx.x == 0) qn[nxt] = 0;
    __syncthreads();
    const int nq = qn[cur];
    for (int k = 0; k < nq; k++) {
      const int2 seg = q[cur][k];
      chunk_partition(S, seg.x, seg.y, wsum, sh);
      if (threadIdx.x == 0) {
        const int i = sh[1], j = sh[2];
        const int2 c[2] = {make_int2(seg.x, i - 1), make_int2(j + 1, seg.y)};
        const bool ok[2] = {seg.x < i - 1, seg.y > j + 1};
        for (int t = 0; t < 2; t++) {
          if (!ok[t]) continue;
          const int len = c[t].y - c[t].x + 1;
          if (len > kSeg && qn[nxt] < kQ) q[nxt][qn[nxt]++] = c[t];
          else if (len > kTiny) S.segq[segn++] = c[t];
          else S.segq[cap / 2 - 1 - (tinyn++)] = c[t];
        }
      }
      __syncthreads();
    }
    cur = nxt;
  }
  // ---- warp tier: whole subtrees down to kTiny elements
  for (;;) {
    int idx = 0;
    if (lane == 0) idx = atomicAdd(&segnext, 1);
    idx = __shfl_sync(0xffffffffu, idx, 0);
    if (idx >= segn) break;
    int stk[2 * 24];
    int sp = 0;
    stk[sp++] = S.segq[idx].x;
    stk[sp++] = S.segq[idx].y;
    while (sp > 0) {
      const int hi = stk[--sp], lo = stk[--sp];
      int i, j;
      warp_part(S, lo, hi, i, j);
      const int2 c[2] = {make_int2(lo, i - 1), make_int2(j + 1, hi)};
      const bool ok[2] = {lo < i - 1, hi > j + 1};
      // push the larger child first so the smaller is popped next: depth <= log2(kSeg)
      const int big = (c[0].y - c[0].x) >= (c[1].y - c[1].x) ? 0 : 1;
      for (int t2 = 0; t2 < 2; t2++) {
        const int t = t2 == 0 ? big : 1 - big;
        if (!ok[t]) continue;
        if (c[t].y - c[t].x + 1 > kTiny) {
          if (sp + 2 > 2 * 24) {   // unreachable for kSeg = 4096
            if (lane == 0) atomicOr(err, 1);
            continue;
          }
          stk[sp++] = c[t].x;
          stk[sp++] = c[t].y;
        } else if (lane == 0) {
          const int ti = atomicAdd(&tinyn, 1);
          S.segq[cap / 2 - 1 - ti] = c[t];
        }
      }
      __syncwarp();
    }
  }
  __syncthreads();
  // ---- thread tier
  for (int t = threadIdx.x; t < tinyn; t += kSortNT) {
    const int2 seg = S.segq[cap / 2 - 1 - t];
    thread_qsort(S.val, S.ord, seg.x, seg.y);
  }
  if (threadIdx.x == 0 && diag) diag[8 * m + 0] = clock64() - t_start;
}

// ---------------------------------------------------------------------------
// suppression test (nms.cpp:141-176); A is the kept box, B the other one
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool supp(float Ay1, float Ax1, float Ay2, float Ax2, float aA, float By1, float Bx1,
                                     float By2, float Bx2, float aB, float overlap) {
  const float yy1 = Ay1 >= By1 ? Ay1 : By1;
  const float xx1 = Ax1 >= Bx1 ? Ax1 : Bx1;
  const float yy2 = Ay2 <= By2 ? Ay2 : By2;
  const float xx2 = Ax2 <= Bx2 ? Ax2 : Bx2;
  const float w = xx2 - xx1 + 1.0;
  const float h = yy2 - yy1 + 1.0;
  const float R_AREA = aA <= aB ? aA : aB;
  if (w > 0 && h > 0) return w * h / R_AREA > overlap;
  if (Ay1 < By1 && Ax1 < Bx1 && Ay2 > By2 && Ax2 > Bx2) return true;
  if (Ay1 > By1 && Ax1 > Bx1 && Ay2 < By2 && Ax2 < Bx2) return true;
  return false;
}

// ---------------------------------------------------------------------------
// 2. sorted boxes and the alive bitmap
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kPassNT) k_nms_gather(const float *__restrict__ boxes_all, int GL, int cap, int *si,
                                                        float *sf) {
  const int m = blockIdx.y;
  Slots S = slots(si, sf, m, cap);
  const float *boxes = boxes_all + (size_t)m * cap * GL;
  const int D = S.st->D;
  const int r = blockIdx.x * kPassNT + threadIdx.x;
  float *y1 = const_cast<float *>(S.y1), *x1 = const_cast<float *>(S.x1), *y2 = const_cast<float *>(S.y2),
        *x2 = const_cast<float *>(S.x2), *ar = const_cast<float *>(S.ar);
  if (r < D) {
    const float *P = boxes + (size_t)S.ord[r] * GL;
    y1[r] = P[0]; x1[r] = P[1]; y2[r] = P[2]; x2[r] = P[3];
    ar[r] = (P[3] - P[1] + 1.0) * (P[2] - P[0] + 1.0);   // nms.cpp's area expression
  }
  const unsigned bal = __ballot_sync(0xffffffffu, r < D);
  if ((threadIdx.x & 31) == 0 && (r >> 5) < ((D + 31) >> 5)) S.bits[r >> 5] = bal;
}

// ---------------------------------------------------------------------------
// 3a. resolve the next batch (whole block)
// ---------------------------------------------------------------------------
struct ResolveSmem {
  int mem_pos[kBatch];
  float my[5][kBatch];
  unsigned rows[kBatch][kBW];
  int pick_mem[kBatch];
  int pick_any[kBatch];
  int wtot[kSortNT / 32];
  int nb, np, last_word, done;
};

// Returns with R.np picks in R.pick_mem, the batch's picks appended to S.picks
// and written to S.bp, the members cleared from the bitmap and the state
// advanced; R.done set when no alive box was left.
__device__ void resolve_batch(Slots &S, float overlap, ResolveSmem &R) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  BatchState &st = *S.st;
  const int nwords = st.nwords;
  if (threadIdx.x == 0) { R.nb = 0; R.last_word = st.scan_word; }
  __syncthreads();
  // members: the first kBatch alive sorted positions from scan_word on
  for (int base = st.scan_word; base < nwords; base += kSortNT) {
    const int have = R.nb;   // uniform: written before the last barrier
    if (have >= kBatch) break;
    const int w = base + threadIdx.x;
    const unsigned word = w < nwords ? S.bits[w] : 0u;
    const int c = __popc(word);
    int inc = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += t;
    }
    if (lane == 31) R.wtot[warp] = inc;
    __syncthreads();
    int before = inc - c, tot = 0;
    for (int k = 0; k < kSortNT / 32; k++) {
      const int v = R.wtot[k];
      if (k < warp) before += v;
      tot += v;
    }
    int rank = have + before;
    unsigned rem = word;
    while (rem && rank < kBatch) {
      const int b = __ffs(rem) - 1;
      rem &= rem - 1;
      R.mem_pos[rank] = (w << 5) + b;
      if (rank == kBatch - 1) R.last_word = w;
      rank++;
    }
    __syncthreads();   // everyone has read wtot and R.nb
    if (threadIdx.x == 0) {
      const int nb = min(kBatch, have + tot);
      if (have + tot <= kBatch) R.last_word = min(base + kSortNT, nwords);   // took every alive box up to here
      R.nb = nb;
    }
    __syncthreads();
  }
  const int nb = R.nb;
  // members' boxes
  if (threadIdx.x < nb) {
    const int r = R.mem_pos[threadIdx.x];
    R.my[0][threadIdx.x] = S.y1[r];
    R.my[1][threadIdx.x] = S.x1[r];
    R.my[2][threadIdx.x] = S.y2[r];
    R.my[3][threadIdx.x] = S.x2[r];
    R.my[4][threadIdx.x] = S.ar[r];
  }
  __syncthreads();
  // suppression rows: bit j of row i = member i (kept) suppresses member j > i
  const int nwm = (nb + 31) >> 5;
  for (int item = threadIdx.x; item < nb * nwm; item += kSortNT) {
    const int i = item / nwm, w = item % nwm;
    unsigned word = 0u;
    if (32 * w + 31 > i) {
      const float a0 = R.my[0][i], a1 = R.my[1][i], a2 = R.my[2][i], a3 = R.my[3][i], a4 = R.my[4][i];
      for (int b = 0; b < 32; b++) {
        const int j = 32 * w + b;
        if (j > i && j < nb &&
            supp(a0, a1, a2, a3, a4, R.my[0][j], R.my[1][j], R.my[2][j], R.my[3][j], R.my[4][j], overlap))
          word |= 1u << b;
      }
    }
    R.rows[i][w] = word;
  }
  __syncthreads();
  // warp 0 walks the batch in order
  if (warp == 0) {
    unsigned alive = 0u;
    if (lane < nwm) alive = (lane == nwm - 1 && (nb & 31)) ? (1u << (nb & 31)) - 1u : ~0u;
    int np = 0;
    for (int guard = 0; guard < kBatch; guard++) {
      const unsigned nz = __ballot_sync(0xffffffffu, alive != 0u);
      if (!nz) break;
      const int fl = __ffs(nz) - 1;
      const unsigned fw = __shfl_sync(0xffffffffu, alive, fl);
      const int i = (fl << 5) + __ffs(fw) - 1;
      if (lane == fl) alive &= ~(1u << (i & 31));
      const unsigned row = lane < nwm ? R.rows[i][lane] : 0u;
      const bool any = __ballot_sync(0xffffffffu, (alive & row) != 0u) != 0u;
      alive &= ~row;
      if (lane == 0) {
        R.pick_mem[np] = i;
        R.pick_any[np] = any ? 1 : 0;
      }
      np++;
    }
    if (lane == 0) R.np = np;
  }
  __syncthreads();
  const int np = R.np, base = st.npicks;
  for (int k = threadIdx.x; k < np; k += kSortNT) {
    const int i = R.pick_mem[k];
    S.picks[base + k] = R.mem_pos[i];
    S.flag[base + k] = R.pick_any[k];
    for (int c = 0; c < 5; c++) S.bp[c * kBatch + k] = R.my[c][i];
  }
  for (int k = threadIdx.x; k < nb; k += kSortNT) {
    const int r = R.mem_pos[k];
    atomicAnd(&S.bits[r >> 5], ~(1u << (r & 31)));   // every member is resolved
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    st.npicks = base + np;
    st.npb = np;
    st.scan_word = R.last_word;
    st.batches += 1;
    if (nb == 0) st.done = 1;
    R.done = nb == 0;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kSortNT) k_nms_resolve(int cap, int *si, float *sf, float overlap) {
  __shared__ ResolveSmem R;
  Slots S = slots(si, sf, blockIdx.x, cap);
  if (S.st->done) return;
  resolve_batch(S, overlap, R);
}

// ---------------------------------------------------------------------------
// 3b. test the alive boxes against the batch's picks (warps own bitmap words)
// ---------------------------------------------------------------------------
__device__ void pass_words(Slots &S, const float (*pk)[kBatch], int np, int pick_base, float overlap, int gwarp,
                           int nwarps) {
  const int lane = threadIdx.x & 31;
  const int nwords = S.st->nwords;
  for (int w = S.st->scan_word + gwarp; w < nwords; w += nwarps) {
    const unsigned word = S.bits[w];
    if (!word) continue;
    const int r = (w << 5) + lane;
    const bool mine = (word >> lane) & 1u;
    const float e0 = mine ? S.y1[r] : 0.f, e1 = mine ? S.x1[r] : 0.f, e2 = mine ? S.y2[r] : 0.f,
                e3 = mine ? S.x2[r] : 0.f, e4 = mine ? S.ar[r] : 0.f;
    unsigned out = word, rem = word;
    while (rem) {
      const int b = __ffs(rem) - 1;
      rem &= rem - 1;
      const float b0 = __shfl_sync(0xffffffffu, e0, b), b1 = __shfl_sync(0xffffffffu, e1, b);
      const float b2 = __shfl_sync(0xffffffffu, e2, b), b3 = __shfl_sync(0xffffffffu, e3, b);
      const float b4 = __shfl_sync(0xffffffffu, e4, b);
      for (int t0 = 0; t0 < np; t0 += 32) {
        const int t = t0 + lane;
        const bool s = t < np && supp(pk[0][t], pk[1][t], pk[2][t], pk[3][t], pk[4][t], b0, b1, b2, b3, b4, overlap);
        const unsigned bal = __ballot_sync(0xffffffffu, s);
        if (bal) {
          out &= ~(1u << b);
          if (lane == 0) S.flag[pick_base + t0 + __ffs(bal) - 1] = 1;
          break;
        }
      }
    }
    if (lane == 0 && out != word) S.bits[w] = out;
  }
}

__global__ void __launch_bounds__(kPassNT) k_nms_pass(int cap, int *si, float *sf, float overlap) {
  __shared__ float pk[5][kBatch];
  Slots S = slots(si, sf, blockIdx.y, cap);
  if (S.st->done) return;
  const int np = S.st->npb;
  if (np <= 0) return;
  for (int k = threadIdx.x; k < np; k += kPassNT)
    for (int c = 0; c < 5; c++) pk[c][k] = S.bp[c * kBatch + k];
  __syncthreads();
  pass_words(S, pk, np, S.st->npicks - np, overlap, blockIdx.x * (kPassNT / 32) + (threadIdx.x >> 5),
             gridDim.x * (kPassNT / 32));
}

// ---------------------------------------------------------------------------
// 4. remaining rounds, final-pick rule, kept records in input order
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kSortNT) k_nms_finish(const float *__restrict__ boxes_all, int GL, int cap,
                                                        int *si, float *sf, float overlap, float *out_all,
                                                        int *d_kept, int *err, long long *diag) {
  __shared__ ResolveSmem R;
  __shared__ float pk[5][kBatch];
  __shared__ int wcnt[kSortNT / 32];
  const int m = blockIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  Slots S = slots(si, sf, m, cap);
  BatchState &st = *S.st;
  const float *boxes = boxes_all + (size_t)m * cap * GL;
  float *out = out_all + (size_t)m * cap * GL;
  const int D = st.D;
  if (!st.done) {
    if (threadIdx.x == 0) st.fallback = 1;
    for (int it = 0;; it++) {
      if (it > D + 1) {   // every round resolves at least one box
        if (threadIdx.x == 0) atomicOr(err, 2);
        break;
      }
      resolve_batch(S, overlap, R);
      if (R.done) break;
      const int np = R.np;
      for (int k = threadIdx.x; k < np; k += kSortNT)
        for (int c = 0; c < 5; c++) pk[c][k] = R.my[c][R.pick_mem[k]];
      __syncthreads();
      pass_words(S, pk, np, st.npicks - np, overlap, warp, kSortNT / 32);
      __syncthreads();
    }
  }
  const int npk = st.npicks;
  const int K = npk - ((npk > 0 && S.flag[npk - 1] == 0) ? 1 : 0);
  int *keep = S.Rpos;
  for (int i = threadIdx.x; i < D; i += kSortNT) keep[i] = 0;
  __syncthreads();
  for (int k = threadIdx.x; k < K; k += kSortNT) keep[S.ord[S.picks[k]]] = 1;
  __syncthreads();
  int written = 0;
  for (int base = 0; base < D; base += kSortNT) {
    const int i = base + threadIdx.x;
    const int f = i < D && keep[i];
    const unsigned bal = __ballot_sync(0xffffffffu, f);
    if (lane == 0) wcnt[warp] = __popc(bal);
    __syncthreads();
    int before = 0, tot = 0;
    for (int w = 0; w < kSortNT / 32; w++) {
      const int c = wcnt[w];
      if (w < warp) before += c;
      tot += c;
    }
    if (f) {
      const float *P = boxes + (size_t)i * GL;
      float *Q = out + (size_t)(written + before + __popc(bal & ((1u << lane) - 1))) * GL;
      for (int t = 0; t < GL; t++) Q[t] = P[t];
    }
    written += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    d_kept[m] = written;
    if (diag) {
      diag[8 * m + 2] = st.batches;
      diag[8 * m + 3] = npk;
      diag[8 * m + 4] = st.fallback;
    }
  }
}

void launch_nms_batch(const float *boxes, const int *d_num, int n_models, int GL, float overlap, int cap, int *si,
                      float *sf, float *out, int *d_kept, int *err, long long *diag, cudaStream_t s) {
  if (n_models <= 0) return;
  k_nms_sort<<<n_models, kSortNT, 0, s>>>(boxes, d_num, GL, cap, si, sf, err, diag);
  k_nms_gather<<<dim3((cap + kPassNT - 1) / kPassNT, n_models), kPassNT, 0, s>>>(boxes, GL, cap, si, sf);
  const int words = (cap + 31) / 32;
  const int pass_blocks = std::max(1, std::min((words + kPassNT / 32 - 1) / (kPassNT / 32), 512));
  for (int r = 0; r < kRounds; r++) {
    k_nms_resolve<<<n_models, kSortNT, 0, s>>>(cap, si, sf, overlap);
    k_nms_pass<<<dim3(pass_blocks, n_models), kPassNT, 0, s>>>(cap, si, sf, overlap);
  }
  k_nms_finish<<<n_models, kSortNT, 0, s>>>(boxes, GL, cap, si, sf, overlap, out, d_kept, err, diag);
}

}  // namespace geye
