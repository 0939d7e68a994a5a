// nms_maps.cu -- NMS of the pipeline's detections, one thread block per model.
//
// Same result as nms.cu (CAR_TRACKING/nms.cpp:70-217: the reference's Hoare
// quicksort order for equal scores, greedy suppression by intersection over
// the smaller area or containment, the last lone box not emitted), but it
// exploits what the pipeline knows about its boxes: every record is the root
// box of a position (x, y) of a (level, component) score map, so the boxes a
// pick can suppress are the positions whose boxes intersect it, a small
// rectangle of each map.
//
// Sort (exact quicksort tie order, see nms.cu for the partition argument):
//   * segments above kSeg are partitioned by the whole block, each thread
//     owning a contiguous chunk (one block scan per partition);
//   * segments of kTiny+1..kSeg elements: one warp each, depth first;
//   * segments of <= kTiny elements: one thread each, the sequential algorithm.
// Greedy: the alive set is a bitmap over map positions in shared memory.
// Boxes are taken in sorted order in batches of up to 32 alive boxes; a warp
// resolves the batch sequentially (a member is picked unless an earlier pick
// of the batch suppresses it); then every block thread walks the alive bits
// inside each pick's candidate rectangle of every map and clears the boxes
// the batch's picks suppress (credited to the first suppressing pick, as the
// sequential loop would).  The loop ends when no alive box is left; the
// reference's `while (cnum > 0)` never picks a box that is alone when its turn
// comes, so the final pick is dropped if it suppressed nothing.
#include "internal.h"

namespace geye {

constexpr int kNT = 1024;                 // threads per block
constexpr int kSeg = 4096;                // block-tier threshold
constexpr int kTiny = 32;                 // thread-tier threshold
constexpr int kQ = 1024;                  // block-tier queue capacity (smem)
constexpr int kMaxMaps = 192;
constexpr int kBatch = 32;

struct MapGeom {
  int r0, r1, pos_off, rs0, rs1;
  float scale;
};

struct NmsMapScratch {
  float *val;      // cap  sort keys
  int *ord;        // cap  sorted position -> box
  int *Lpos, *Rpos;
  int2 *segq;      // cap/2 segment queue (warp tier, then thread tier)
  int *pos2box;    // cap  position -> box (-1 below threshold)
  int *box2pos;    // cap
  int *spos;       // cap  sorted position -> position
};

__device__ __forceinline__ NmsMapScratch nmsm_scratch(int *base, int cap) {
  NmsMapScratch S;
  S.val = reinterpret_cast<float *>(base);
  S.ord = base + cap;
  S.Lpos = base + 2 * cap;
  S.Rpos = base + 3 * cap;
  S.segq = reinterpret_cast<int2 *>(base + 4 * cap);
  S.pos2box = base + 5 * cap;
  S.box2pos = base + 6 * cap;
  S.spos = base + 7 * cap;
  return S;
}

// ---------------------------------------------------------------------------
// sort tiers
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

// partition [lo, hi] (hi-lo+1 > kSeg) by the whole block; result (i, j) in sh[1], sh[2]
__device__ void chunk_partition(NmsMapScratch &S, int lo, int hi, unsigned long long *wsum, int *sh) {
  const int m = hi - lo + 1;
  const float key = S.val[(lo + hi) / 2];
  const int cs = (m + kNT - 1) / kNT;
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
  for (int k = threadIdx.x; k < lim; k += kNT) cnt += Lp[k] < Rp[k];
  cnt = __syncthreads_count(0) + cnt;   // barrier: all counts computed before wsum reuse
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  if (lane == 0) wsum[warp] = (unsigned long long)cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    int K = 0;
    for (int w = 0; w < kNT / 32; w++) K += (int)wsum[w];
    sh[0] = K;
  }
  __syncthreads();
  const int K = sh[0];
  for (int k = threadIdx.x; k < K; k += kNT) {
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

__device__ void warp_part(NmsMapScratch &S, int lo, int hi, int &oi, int &oj) {
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
// suppression test (nms.cpp:141-176)
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

__device__ __forceinline__ float box_area(const float *P) { return (P[3] - P[1] + 1.0) * (P[2] - P[0] + 1.0); }

// ---------------------------------------------------------------------------
// kernel
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kNT) k_nms_maps(const float *__restrict__ boxes_all, const int *__restrict__ d_num,
                                                  const ScoreJob *__restrict__ jobs_all, const int *__restrict__ job_start,
                                                  int GL, float overlap, int cap, int *scratch, float *out_all,
                                                  int *d_kept, int *err, long long *diag) {
  extern __shared__ unsigned bits[];       // alive bitmap over map positions
  __shared__ MapGeom maps[kMaxMaps];
  __shared__ unsigned long long wsum[32];
  __shared__ int sh[8];
  __shared__ int2 q[2][kQ];
  __shared__ int qn[2];
  __shared__ int segn, segnext, tinyn;
  __shared__ float pk[kBatch][5];          // picks of the current batch: y1, x1, y2, x2, area
  __shared__ int pkattr[kBatch];           // boxes each pick suppressed first
  __shared__ int npk, npicks, scan_pos;
  __shared__ int mem_pos[kBatch];

  const int m = blockIdx.x;
  const float *boxes = boxes_all + (size_t)m * cap * GL;
  float *out = out_all + (size_t)m * cap * GL;
  NmsMapScratch S = nmsm_scratch(scratch + (size_t)m * nms_model_words(cap), cap);
  const ScoreJob *jobs = jobs_all + job_start[m];
  const int nmaps = job_start[m + 1] - job_start[m];
  const int D = min(d_num[m], cap);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long t_start = clock64();
  if (D <= 0 || nmaps <= 0 || nmaps > kMaxMaps) {
    if (threadIdx.x == 0) {
      d_kept[m] = 0;
      if (D > 0) atomicOr(err, 8);
    }
    return;
  }
  for (int i = threadIdx.x; i < nmaps; i += kNT) {
    const ScoreJob &J = jobs[i];
    maps[i] = MapGeom{J.r0, J.r1, J.pos_off, J.rsize0, J.rsize1, J.scale};
  }
  for (int i = threadIdx.x; i < D; i += kNT) {
    S.val[i] = boxes[(size_t)i * GL + GL - 2];
    S.ord[i] = i;
  }
  if (threadIdx.x == 0) {
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
  for (int t = threadIdx.x; t < tinyn; t += kNT) {
    const int2 seg = S.segq[cap / 2 - 1 - t];
    thread_qsort(S.val, S.ord, seg.x, seg.y);
  }
  __syncthreads();

  const long long t_sorted = clock64();
  // ---- greedy over the alive bitmap
  const MapGeom &LM = maps[nmaps - 1];
  const int npos = LM.pos_off + LM.r0 * LM.r1;
  const int nwords = (npos + 31) >> 5;
  for (int w = threadIdx.x; w < nwords; w += kNT) bits[w] = 0u;
  if (threadIdx.x == 0) { npicks = 0; scan_pos = 0; }
  __syncthreads();
  for (int p = threadIdx.x; p < D; p += kNT) {
    const int qq = S.box2pos[S.ord[p]];
    S.spos[p] = qq;
    atomicOr(&bits[qq >> 5], 1u << (qq & 31));
  }
  __syncthreads();
  int *picks = S.Lpos;   // pick list in pick order (the sort is done with Lpos)
  int last_attr = 1, batches = 0;
  for (;;) {
    if (++batches > D + 1) {
      if (threadIdx.x == 0) atomicOr(err, 2);
      break;
    }
    if (warp == 0) {
      // collect up to kBatch alive boxes in sorted order into mem_pos[]
      int nb = 0, p = scan_pos;
      while (nb < kBatch && p < D) {
        const int pp = p + lane;
        int qq = -1;
        bool alive = false;
        if (pp < D) {
          qq = S.spos[pp];
          alive = (bits[qq >> 5] >> (qq & 31)) & 1u;
        }
        const unsigned bal = __ballot_sync(0xffffffffu, alive);
        const int navail = __popc(bal), take = min(navail, kBatch - nb);
        const int rank = __popc(bal & ((1u << lane) - 1));
        if (alive && rank < take) mem_pos[nb + rank] = qq;
        if (take < navail) {
          // continue right after the last taken lane: the take-th set bit of bal
          unsigned mb = bal;
          for (int u = 0; u < take - 1; u++) mb &= mb - 1;
          p += __ffs(mb);
        } else {
          p += 32;
        }
        nb += take;
      }
      p = min(p, D);
      __syncwarp();
      const int mypos = lane < nb ? mem_pos[lane] : -1;
      // resolve the batch: member i (lane i) is picked unless an earlier pick suppresses it
      float my[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
      int mybox = -1;
      if (lane < nb) {
        mybox = S.pos2box[mypos];
        const float *P = boxes + (size_t)mybox * GL;
        my[0] = P[0]; my[1] = P[1]; my[2] = P[2]; my[3] = P[3];
        my[4] = box_area(P);
      }
      bool alive = lane < nb;
      int np = 0, base = npicks;
      for (int i = 0; i < nb; i++) {
        if (!__shfl_sync(0xffffffffu, alive, i)) continue;
        const float y1 = __shfl_sync(0xffffffffu, my[0], i), x1 = __shfl_sync(0xffffffffu, my[1], i);
        const float y2 = __shfl_sync(0xffffffffu, my[2], i), x2 = __shfl_sync(0xffffffffu, my[3], i);
        const float ar = __shfl_sync(0xffffffffu, my[4], i);
        const bool sp = lane > i && alive && supp(y1, x1, y2, x2, ar, my[0], my[1], my[2], my[3], my[4], overlap);
        const unsigned sb = __ballot_sync(0xffffffffu, sp);
        if (sp) alive = false;
        if (lane == 0) {
          pk[np][0] = y1; pk[np][1] = x1; pk[np][2] = y2; pk[np][3] = x2; pk[np][4] = ar;
          pkattr[np] = __popc(sb);
        }
        if (lane == i) picks[base + np] = mybox;
        np++;
      }
      // every member leaves the alive set (picked or suppressed)
      if (lane < nb) atomicAnd(&bits[mypos >> 5], ~(1u << (mypos & 31)));
      if (lane == 0) {
        npk = np;
        npicks = base + np;
        scan_pos = p;
      }
    }
    __syncthreads();
    const int np = npk;
    if (np == 0) break;
    // candidate pass: alive boxes inside each pick's rectangle of each map.  A warp
    // takes a (pick, map) pair, its lanes take columns; a candidate's box comes from
    // the map geometry (the same expression that wrote its record), not from memory.
    for (int pm = warp; pm < np * nmaps; pm += kNT / 32) {
      const int pq = pm / nmaps, mi = pm % nmaps;
      const MapGeom G = maps[mi];
      const float s = G.scale;
      // root box of (x, y): [(y+1)s, (y+1)s + rs0*s - 1] x [(x+1)s, ...]; it can only meet
      // the pick's box [Ay1, Ay2] x [Ax1, Ax2] (inclusive, +1) inside this range, widened by a cell
      int ylo = (int)floorf((pk[pq][0] - 1.0f) / s) - G.rs0 - 2, yhi = (int)ceilf((pk[pq][2] + 1.0f) / s) + 1;
      int xlo = (int)floorf((pk[pq][1] - 1.0f) / s) - G.rs1 - 2, xhi = (int)ceilf((pk[pq][3] + 1.0f) / s) + 1;
      ylo = max(ylo, 0); xlo = max(xlo, 0);
      yhi = min(yhi, G.r0 - 1); xhi = min(xhi, G.r1 - 1);
      if (ylo > yhi) continue;
      for (int x = xlo + lane; x <= xhi; x += 32) {
        const int q0 = G.pos_off + x * G.r0 + ylo, q1 = G.pos_off + x * G.r0 + yhi;
        for (int w = q0 >> 5; w <= (q1 >> 5); w++) {
          unsigned word = bits[w];
          const int wb = w << 5;
          if (wb < q0) word &= ~0u << (q0 - wb);
          if (q1 - wb < 31) word &= (1u << (q1 - wb + 1)) - 1u;
          while (word) {
            const int bit = __ffs(word) - 1;
            word &= word - 1;
            const int y = wb + bit - G.pos_off - x * G.r0;
            float B[4];
            root_box(x, y, s, G.rs0, G.rs1, B);
            const float aB = (B[3] - B[1] + 1.0) * (B[2] - B[0] + 1.0);
            int first = -1;
            for (int t = 0; t < np; t++)
              if (supp(pk[t][0], pk[t][1], pk[t][2], pk[t][3], pk[t][4], B[0], B[1], B[2], B[3], aB, overlap)) {
                first = t;
                break;
              }
            if (first < 0) continue;
            const unsigned old = atomicAnd(&bits[w], ~(1u << bit));
            if (old & (1u << bit)) atomicAdd(&pkattr[first], 1);
          }
        }
      }
    }
    __syncthreads();
    last_attr = pkattr[np - 1];
    __syncthreads();
  }
  if (threadIdx.x == 0 && diag) {
    diag[8 * m + 0] = t_sorted - t_start;
    diag[8 * m + 1] = clock64() - t_sorted;
    diag[8 * m + 2] = batches;
    diag[8 * m + 3] = npicks;
  }
  // the reference's loop (while cnum > 0) never takes a box that is alone when
  // its turn comes: that is the final pick exactly when it suppressed nothing
  const int K = npicks - ((npicks > 0 && last_attr == 0) ? 1 : 0);
  int *keep = S.Rpos;
  for (int i = threadIdx.x; i < D; i += kNT) keep[i] = 0;
  __syncthreads();
  for (int k = threadIdx.x; k < K; k += kNT) keep[picks[k]] = 1;
  __syncthreads();
  int written = 0;
  for (int base = 0; base < D; base += kNT) {
    const int i = base + threadIdx.x;
    const int f = i < D && keep[i];
    const unsigned bal = __ballot_sync(0xffffffffu, f);
    if (lane == 0) wsum[warp] = __popc(bal);
    __syncthreads();
    int before = 0, tot = 0;
    for (int w = 0; w < kNT / 32; w++) {
      const int c = (int)wsum[w];
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
  if (threadIdx.x == 0) d_kept[m] = written;
}

void launch_nms_maps(const float *boxes, const int *d_num, int n_models, const ScoreJob *jobs, const int *job_start,
                     int GL, float overlap, int cap, int max_positions, int *scratch, float *out, int *d_kept, int *err,
                     long long *diag, cudaStream_t s) {
  const size_t smem = sizeof(unsigned) * (size_t)((max_positions + 31) / 32 + 1);
  static size_t set = 0;
  if (smem > set) {
    cudaFuncSetAttribute(k_nms_maps, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    set = smem;
  }
  k_nms_maps<<<n_models, kNT, smem, s>>>(boxes, d_num, jobs, job_start, GL, overlap, cap, scratch, out, d_kept, err,
                                         diag);
}

}  // namespace geye
