// nms_batch.cu -- NMS of the pipeline's detections, every model of a frame at once.
//
// Same kept set as nms.cu (CAR_TRACKING/nms.cpp:70-217): the reference's Hoare
// quicksort order for equal scores, greedy suppression by intersection over
// the smaller area or containment, and a box that is alone when its turn comes
// never emitted.  The greedy loop is restated so that most of it runs on every
// SM:
//
//  1. the order: score order from the radix sort (nms_radix.cu), checked for
//     the cases where the quicksort's order among equal scores could change
//     the kept set; the models that raise them go through steps 2-4 again in
//     the quicksort's order (nms_sort.cu).
//  2. k_nms_gather: the boxes in sorted order (structure of arrays), an alive
//     bitmap over sorted positions and its summary (one bit per word).
//  3. Rounds of two kernels, each a no-op for a model that is done:
//     k_nms_resolve (one block per model) takes the first kBatch alive boxes
//     in sorted order (found through the summary), computes for each member
//     which earlier members suppress it (pairs whose cell spans overlap) and
//     decides the members in parallel rounds: a member is picked when every
//     earlier member that suppresses it is decided and none is picked, and
//     removed when an earlier pick suppresses it -- the sequential loop's
//     decisions, since every box before the batch is already resolved.  It
//     then lists its picks by image cell on each axis.
//     k_nms_pass (grid) tests every other alive box against the picks that
//     share a row cell and a column cell with it, in pick order; the first
//     pick that suppresses it is the one the sequential loop would have
//     removed it with.
//  4. k_nms_finish (one block per model) runs any remaining rounds itself,
//     drops the final pick if it suppressed nothing (the reference's
//     `while (cnum > 0)` with cnum = NUM-1 never takes a box that is alone at
//     its turn) and writes the kept records in input order.
#include <algorithm>

#include "nms_common.h"

namespace geye {

constexpr int kSortNT = kNmsNT;   // threads of the resolve and finish blocks
constexpr int kBatch = kNmsBatch;
constexpr int kBW = kBatch / 32;   // words of a suppression row
constexpr int kPassNT = 256;
constexpr int kRankSortMax = 4096; // kept boxes ordered by ranking in shared memory up to this many

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
  if (r < D) {
    const float *P = boxes + (size_t)S.ord[r] * GL;
    S.y1[r] = P[0]; S.x1[r] = P[1]; S.y2[r] = P[2]; S.x2[r] = P[3];
    S.ar[r] = (P[3] - P[1] + 1.0) * (P[2] - P[0] + 1.0);   // nms.cpp's area expression
  }
  const unsigned bal = __ballot_sync(0xffffffffu, r < D);
  const int nwords = (D + 31) >> 5;
  if ((threadIdx.x & 31) == 0 && (r >> 5) < nwords) S.bits[r >> 5] = bal;
  // summary: every word below nwords starts with an alive box
  if (r < (nwords + 31) >> 5) {
    const int n = min(32, nwords - 32 * r);
    S.sbits[r] = n == 32 ? ~0u : (1u << n) - 1u;
  }
}

// clears the alive bits `clear` of word w (more than one thread may clear bits
// of the same word); the last clear of a word clears its summary bit
__device__ __forceinline__ void clear_alive(const Slots &S, int w, unsigned clear) {
  const unsigned old = atomicAnd(&S.bits[w], ~clear);
  if (old != 0u && (old & ~clear) == 0u) atomicAnd(&S.sbits[w >> 5], ~(1u << (w & 31)));
}

// cell of a coordinate on one axis of the pick masks (monotone; NaN to cell 0)
__device__ __forceinline__ int nms_cell(float v, float inv) {
  return (int)fminf(fmaxf(v * inv, 0.0f), (float)(kNmsCells - 1));
}

// ---------------------------------------------------------------------------
// 3a. resolve the next batch (whole block)
// ---------------------------------------------------------------------------
struct ResolveSmem {
  int mem_pos[kBatch + 1];
  int wl[kBatch + 1];    // non-empty words of the alive bitmap holding the members
  int run_end[kBatch];   // key order: last member with the same score
  unsigned key[kBatch + 1];   // key order: the candidates' keys
  float my[5][kBatch];
  unsigned cm[2][kNmsCells][kBW];   // the picks by cell, built for the pass
  unsigned und[kBW], pk_bits[kBW];  // undecided and picked members
  int killed_any[kBatch];           // member (a pick) removed a member alive at its turn
  unsigned span[kBatch];            // member's cell span (bytes y0, y1, x0, x1)
  int pick_mem[kBatch];
  int pick_any[kBatch];
  int wtot[kSortNT / 32];
  int nb, nw, np, last_word, done;
};

// exclusive block scan of c (kSortNT threads); *tot gets the sum
__device__ __forceinline__ int block_excl_scan(int c, int *tot, int *wtot) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int inc = c;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  __syncthreads();   // wtot free
  if (lane == 31) wtot[warp] = inc;
  __syncthreads();
  int before = inc - c, t = 0;
  for (int k = 0; k < kSortNT / 32; k++) {
    const int v = wtot[k];
    if (k < warp) before += v;
    t += v;
  }
  *tot = t;
  return before;
}

__device__ __forceinline__ unsigned sorted_key(const Slots &S, int pos) {
  return reinterpret_cast<const unsigned *>(S.val)[pos];
}

// Returns with R.np picks in R.pick_mem, the batch's picks appended to S.picks
// and written to S.bp, the members cleared from the bitmap and the state
// advanced; R.done set when no alive box was left.
// KEY_ORDER (positions in nms_radix.cu's order): a run of equal scores never
// straddles two batches (the batch ends before a run that the next alive box
// continues), and *need is raised where the order inside a run could matter:
// a pick that suppresses an alive member of its own run, or a run longer than
// a batch.
template <bool KEY_ORDER>
__device__ void resolve_batch(Slots &S, float overlap, float cell_inv, ResolveSmem &R, int *need) {
  constexpr int want = kBatch + (KEY_ORDER ? 1 : 0);   // key order: one more, to see the run at the boundary
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  BatchState &st = *S.st;
  const int nwords = st.nwords;
  if (threadIdx.x == 0) R.nw = 0;
  __syncthreads();
  // members: the first `want` alive sorted positions from scan_word on, found
  // through the summary (words before scan_word hold no alive box): the first
  // `want` non-empty words, then the first `want` alive bits of those
  const int nsw = (nwords + 31) >> 5;
  for (int sb = st.scan_word >> 5; sb < nsw; sb += kSortNT) {
    const int have = R.nw;   // uniform: written before the last barrier
    if (have >= want) break;
    const int j = sb + threadIdx.x;
    const unsigned sw = j < nsw ? S.sbits[j] : 0u;
    int tot;
    int rank = have + block_excl_scan(__popc(sw), &tot, R.wtot);
    unsigned rem = sw;
    while (rem && rank < want) {
      R.wl[rank++] = (j << 5) + __ffs(rem) - 1;
      rem &= rem - 1;
    }
    __syncthreads();   // everyone has read R.nw
    if (threadIdx.x == 0) R.nw = min(want, have + tot);
    __syncthreads();
  }
  const int nw = R.nw;
  {
    const int w = threadIdx.x < nw ? R.wl[threadIdx.x] : 0;
    const unsigned word = threadIdx.x < nw ? S.bits[w] : 0u;
    int tot;
    int rank = block_excl_scan(__popc(word), &tot, R.wtot);
    unsigned rem = word;
    while (rem && rank < want) {
      const int r = (w << 5) + __ffs(rem) - 1;
      R.mem_pos[rank] = r;
      if (KEY_ORDER) R.key[rank] = sorted_key(S, r);
      rank++;
      rem &= rem - 1;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      int nb = min(want, tot);
      // every alive box is a member: the summary was exhausted and held no more than a batch
      const bool all_taken = nw < want && tot <= kBatch;
      if (KEY_ORDER && nb == want) {   // an alive box follows the batch: end before its run
        const unsigned kb = R.key[kBatch];
        int lo = 0, hi = kBatch;   // first candidate with key kb (keys ascend): in [lo, hi]
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (R.key[mid] < kb) lo = mid + 1;
          else hi = mid;
        }
        nb = lo;
        if (nb == 0) {   // a run longer than a batch
          *need = 1;
          nb = kBatch;
        }
      }
      R.nb = nb;
      R.last_word = (all_taken || nb == 0) ? nwords : (R.mem_pos[nb - 1] >> 5);
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
    if (KEY_ORDER) {   // last member with this key (keys ascend)
      const unsigned k = R.key[threadIdx.x];
      int lo = threadIdx.x, hi = nb - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (R.key[mid] == k) lo = mid;
        else hi = mid - 1;
      }
      R.run_end[threadIdx.x] = lo;
    }
  }
  __syncthreads();
  // The batch's decisions, in parallel rounds.  Four threads per member j
  // hold its column (bit i of word w: member i < j suppresses j; thread q of
  // the group: words q and q + 4).  A round decides every undecided member
  // that an earlier pick suppresses (removed) or whose earlier suppressors
  // are all decided and none picked (picked): the sequential walk's decision
  // for it, since the members before it are decided as the walk would.  The
  // first undecided member is always decided, so the rounds end.
  const int nwm = (nb + 31) >> 5;
  const int gj = threadIdx.x >> 2, gq = threadIdx.x & 3;
  // each member's cell span, widened by two pixels (bytes y0, y1, x0, x1): two
  // boxes that can suppress each other have overlapping spans on both axes
  if (threadIdx.x < nb) {
    const int i = threadIdx.x;
    const int y0 = nms_cell(fminf(R.my[0][i], R.my[2][i]) - 2.0f, cell_inv);
    const int y1 = nms_cell(fmaxf(R.my[0][i], R.my[2][i]) + 2.0f, cell_inv);
    const int x0 = nms_cell(fminf(R.my[1][i], R.my[3][i]) - 2.0f, cell_inv);
    const int x1 = nms_cell(fmaxf(R.my[1][i], R.my[3][i]) + 2.0f, cell_inv);
    R.span[i] = (unsigned)y0 | ((unsigned)y1 << 8) | ((unsigned)x0 << 16) | ((unsigned)x1 << 24);
  }
  __syncthreads();
  unsigned col[2] = {0u, 0u};
  if (gj < nb) {
    const float b0 = R.my[0][gj], b1 = R.my[1][gj], b2 = R.my[2][gj], b3 = R.my[3][gj], b4 = R.my[4][gj];
    const unsigned sj = R.span[gj];
    const int jy0 = sj & 255, jy1 = (sj >> 8) & 255, jx0 = (sj >> 16) & 255, jx1 = sj >> 24;
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int w = gq + 4 * h;
      const int i0 = 32 * w, i1 = min(i0 + 32, gj);
      unsigned word = 0u;
      for (int i = i0; i < i1; i++) {
        const unsigned si_ = R.span[i];
        if ((int)(si_ & 255) > jy1 || (int)((si_ >> 8) & 255) < jy0 || (int)((si_ >> 16) & 255) > jx1 ||
            (int)(si_ >> 24) < jx0)
          continue;
        if (supp(R.my[0][i], R.my[1][i], R.my[2][i], R.my[3][i], R.my[4][i], b0, b1, b2, b3, b4, overlap))
          word |= 1u << (i - i0);
      }
      col[h] = word;
    }
  }
  if (threadIdx.x < kBW) {
    const int w = threadIdx.x;
    R.und[w] = w < nwm ? ((w == nwm - 1 && (nb & 31)) ? (1u << (nb & 31)) - 1u : ~0u) : 0u;
    R.pk_bits[w] = 0u;
  }
  if (threadIdx.x < kBatch) R.killed_any[threadIdx.x] = 0;
  __syncthreads();
  for (int round = 0; round <= kBatch; round++) {
    const bool mine_und = gj < nb && ((R.und[gj >> 5] >> (gj & 31)) & 1u);
    int hp = ((col[0] & R.pk_bits[gq]) | (col[1] & R.pk_bits[gq + 4])) != 0u;
    int hu = ((col[0] & R.und[gq]) | (col[1] & R.und[gq + 4])) != 0u;
    hp |= __shfl_xor_sync(0xffffffffu, hp, 1);
    hp |= __shfl_xor_sync(0xffffffffu, hp, 2);
    hu |= __shfl_xor_sync(0xffffffffu, hu, 1);
    hu |= __shfl_xor_sync(0xffffffffu, hu, 2);
    const bool decide = mine_und && (hp || !hu), pick = decide && !hp;
    __syncthreads();   // every group has read the round's state
    if (gq == 0 && decide) {
      atomicAnd(&R.und[gj >> 5], ~(1u << (gj & 31)));
      if (pick) atomicOr(&R.pk_bits[gj >> 5], 1u << (gj & 31));
    }
    __syncthreads();
    unsigned left = 0u;
#pragma unroll
    for (int w = 0; w < kBW; w++) left |= R.und[w];
    if (!left) break;
  }
  // a removed member's first suppressor among the picks removed it in the
  // walk: that pick suppressed a box alive at its turn (its flag); in key
  // order, a pick that removes a member of its own run of equal scores needs
  // the quicksort's order
  {
    const bool removed = gj < nb && !((R.pk_bits[gj >> 5] >> (gj & 31)) & 1u);
    const unsigned h0 = removed ? col[0] & R.pk_bits[gq] : 0u, h1 = removed ? col[1] & R.pk_bits[gq + 4] : 0u;
    int wfirst = h0 ? gq : (h1 ? gq + 4 : 64);   // smallest word with a suppressing pick
    wfirst = min(wfirst, __shfl_xor_sync(0xffffffffu, wfirst, 1));
    wfirst = min(wfirst, __shfl_xor_sync(0xffffffffu, wfirst, 2));
    const unsigned hw = wfirst == gq ? h0 : (wfirst == gq + 4 ? h1 : 0u);
    if (hw) {
      const int killer = 32 * wfirst + __ffs(hw) - 1;
      R.killed_any[killer] = 1;
      if (KEY_ORDER && R.key[killer] == R.key[gj]) *need = 1;
    }
  }
  __syncthreads();
  if (threadIdx.x < nb && ((R.pk_bits[threadIdx.x >> 5] >> (threadIdx.x & 31)) & 1u)) {
    int rank = __popc(R.pk_bits[threadIdx.x >> 5] & ((1u << (threadIdx.x & 31)) - 1u));
    for (int w = 0; w < (threadIdx.x >> 5); w++) rank += __popc(R.pk_bits[w]);
    R.pick_mem[rank] = threadIdx.x;
    R.pick_any[rank] = R.killed_any[threadIdx.x];
  }
  if (threadIdx.x == 0) {
    int np = 0;
    for (int w = 0; w < kBW; w++) np += __popc(R.pk_bits[w]);
    R.np = np;
  }
  __syncthreads();
  const int np = R.np, base = st.npicks;
  for (int k = threadIdx.x; k < np; k += kSortNT) {
    const int i = R.pick_mem[k];
    S.picks[base + k] = R.mem_pos[i];
    S.flag[base + k] = R.pick_any[k];
    for (int c = 0; c < 5; c++) S.bp[c * kBatch + k] = R.my[c][i];
  }
  // the picks by cell for the pass (the suppression rows are free now): a
  // pick is listed on every cell of its span widened by two pixels, so a box
  // that it can suppress (positive overlap, or containment) shares a row and a
  // column cell with it
  unsigned *cm = &R.cm[0][0][0];   // [axis][cell][kBW]
  for (int k = threadIdx.x; k < 2 * kNmsCells * kBW; k += kSortNT) cm[k] = 0u;
  __syncthreads();
  for (int k = threadIdx.x; k < np; k += kSortNT) {
    const int i = R.pick_mem[k];
    const unsigned bit = 1u << (k & 31);
    for (int a = 0; a < 2; a++) {   // a = 0: y (my[0], my[2]); 1: x (my[1], my[3])
      const float lo = fminf(R.my[a][i], R.my[a + 2][i]) - 2.0f, hi = fmaxf(R.my[a][i], R.my[a + 2][i]) + 2.0f;
      const int c1 = nms_cell(hi, cell_inv);
      for (int c = nms_cell(lo, cell_inv); c <= c1; c++) atomicOr(&cm[(a * kNmsCells + c) * kBW + (k >> 5)], bit);
    }
  }
  __syncthreads();
  for (int k = threadIdx.x; k < 2 * kNmsCells * kBW; k += kSortNT) S.cmask[k] = cm[k];
  for (int k = threadIdx.x; k < nb; k += kSortNT) {
    const int r = R.mem_pos[k];
    clear_alive(S, r >> 5, 1u << (r & 31));   // every member is resolved
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    st.npicks = base + np;
    st.npb = np;
    st.scan_word = R.last_word;
    st.batches += 1;
    // done once no alive box is left: none found, or this batch took every
    // one up to the end of the bitmap (its pass would test nothing)
    if (nb == 0 || R.last_word >= nwords) st.done = 1;
    R.done = nb == 0;
  }
  __syncthreads();
}

template <bool KEY_ORDER>
__global__ void __launch_bounds__(kSortNT) k_nms_resolve(int cap, int *si, float *sf, float overlap, float cell_inv,
                                                         int *need) {
  __shared__ ResolveSmem R;
  Slots S = slots(si, sf, blockIdx.x, cap);
  if (S.st->done) return;
  resolve_batch<KEY_ORDER>(S, overlap, cell_inv, R, need ? need + blockIdx.x : nullptr);
}

// ---------------------------------------------------------------------------
// 3b. test the alive boxes against the batch's picks (warps own bitmap words):
// each alive box is removed by the first pick, in pick order, that suppresses
// it, and that pick is flagged; sparse words take a box at a time against 32
// picks a step, dense ones a pick at a time against 32 boxes a step
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
    if (2 * __popc(word) * ((np + 31) >> 5) > np) {
      // dense word: a lane per box walks the picks in order (about np steps for
      // the warp instead of one 32-pick step per box and pick chunk)
      int first = -1;
      if (mine)
        for (int t = 0; t < np; t++)
          if (supp(pk[0][t], pk[1][t], pk[2][t], pk[3][t], pk[4][t], e0, e1, e2, e3, e4, overlap)) {
            first = t;
            break;
          }
      const unsigned gone = __ballot_sync(0xffffffffu, first >= 0);
      if (first >= 0) S.flag[pick_base + first] = 1;
      if (lane == 0 && gone) clear_alive(S, w, gone);
      continue;
    }
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
    if (lane == 0 && out != word) clear_alive(S, w, word & ~out);
  }
}

// The round's pass: a lane per alive box of a word, testing only the picks
// that share a row cell and a column cell with it (the union of the picks
// listed on its cell span, per axis, from a sparse table of spans of 2^l
// cells), in pick order; the first that suppresses it removes it and is
// flagged.
struct PassSmem {
  float pk[5][kBatch];
  unsigned tab[2][kNmsLevels][kNmsCells][kBW];
};

__global__ void __launch_bounds__(kPassNT) k_nms_pass(int cap, int *si, float *sf, float overlap, float cell_inv) {
  __shared__ PassSmem Z;
  Slots S = slots(si, sf, blockIdx.y, cap);
  const BatchState &st = *S.st;
  if (st.done) return;
  const int np = st.npb;
  if (np <= 0) return;
  const int nwarps = gridDim.x * (kPassNT / 32);
  const int w_first = st.scan_word + blockIdx.x * (kPassNT / 32);
  const int nwords = st.nwords;
  {
    // a block whose words hold no alive box leaves before it builds the tables
    // (only this block's warps change its words, so the check stays true)
    bool any = false;
    for (int k = threadIdx.x; !any; k += kPassNT) {
      const int w = w_first + (k & (kPassNT / 32 - 1)) + (k / (kPassNT / 32)) * nwarps;
      if (w >= nwords) break;
      any = S.bits[w] != 0u;
    }
    if (!__syncthreads_or(any)) return;
  }
  const int nwm = (np + 31) >> 5;
  for (int k = threadIdx.x; k < np; k += kPassNT)
    for (int c = 0; c < 5; c++) Z.pk[c][k] = S.bp[c * kBatch + k];
  for (int e = threadIdx.x; e < 2 * kNmsCells * nwm; e += kPassNT) {
    const int a = e / (kNmsCells * nwm), rem = e - a * kNmsCells * nwm, c = rem / nwm, k = rem - c * nwm;
    Z.tab[a][0][c][k] = S.cmask[(a * kNmsCells + c) * kBW + k];
  }
  __syncthreads();
  for (int l = 1; l < kNmsLevels; l++) {
    for (int e = threadIdx.x; e < 2 * kNmsCells * nwm; e += kPassNT) {
      const int a = e / (kNmsCells * nwm), rem = e - a * kNmsCells * nwm, c = rem / nwm, k = rem - c * nwm;
      Z.tab[a][l][c][k] = Z.tab[a][l - 1][c][k] | Z.tab[a][l - 1][min(c + (1 << (l - 1)), kNmsCells - 1)][k];
    }
    __syncthreads();
  }
  const int lane = threadIdx.x & 31;
  const int pick_base = st.npicks - np;
  for (int w = w_first + (threadIdx.x >> 5); w < nwords; w += nwarps) {
    const unsigned word = S.bits[w];
    if (!word) continue;
    const int r = (w << 5) + lane;
    int first = -1;
    if ((word >> lane) & 1u) {
      const float e0 = S.y1[r], e1 = S.x1[r], e2 = S.y2[r], e3 = S.x2[r], e4 = S.ar[r];
      const int cy0 = nms_cell(fminf(e0, e2), cell_inv), cy1 = nms_cell(fmaxf(e0, e2), cell_inv);
      const int cx0 = nms_cell(fminf(e1, e3), cell_inv), cx1 = nms_cell(fmaxf(e1, e3), cell_inv);
      const int ly = 31 - __clz(cy1 - cy0 + 1), lx = 31 - __clz(cx1 - cx0 + 1);
      const int cy2 = cy1 - (1 << ly) + 1, cx2 = cx1 - (1 << lx) + 1;
      for (int k = 0; k < nwm && first < 0; k++) {
        unsigned cand = (Z.tab[0][ly][cy0][k] | Z.tab[0][ly][cy2][k]) & (Z.tab[1][lx][cx0][k] | Z.tab[1][lx][cx2][k]);
        while (cand) {
          const int t = (k << 5) + __ffs(cand) - 1;
          cand &= cand - 1;
          if (supp(Z.pk[0][t], Z.pk[1][t], Z.pk[2][t], Z.pk[3][t], Z.pk[4][t], e0, e1, e2, e3, e4, overlap)) {
            first = t;
            break;
          }
        }
      }
    }
    const unsigned gone = __ballot_sync(0xffffffffu, first >= 0);
    if (first >= 0) S.flag[pick_base + first] = 1;
    if (lane == 0 && gone) {   // this warp owns word w in this kernel
      const unsigned left = word & ~gone;
      S.bits[w] = left;
      if (!left) atomicAnd(&S.sbits[w >> 5], ~(1u << (w & 31)));
    }
  }
}

// ---------------------------------------------------------------------------
// 4. remaining rounds, final-pick rule, kept records in input order
// ---------------------------------------------------------------------------
// KEY_ORDER: the key-order pass (writes every model's result; raises need[m]
// where the quicksort order could differ).  Otherwise the quicksort-order pass:
// with need given, only the models that raised it (their result replaces the
// key-order one); without, every model.
template <bool KEY_ORDER>
__global__ void __launch_bounds__(kSortNT) k_nms_finish(const float *__restrict__ boxes_all, int GL, int cap,
                                                        int *si, float *sf, float overlap, float *out_all,
                                                        int *d_kept, int *err, long long *diag, int *rounds_used,
                                                        int *need, float cell_inv) {
  __shared__ ResolveSmem R;
  __shared__ float pk[5][kBatch];
  __shared__ int wcnt[kSortNT / 32];
  const int m = blockIdx.x;
  if (!KEY_ORDER && need && !need[m]) return;
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
      resolve_batch<KEY_ORDER>(S, overlap, cell_inv, R, need ? need + m : nullptr);
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
  // the last pick shares its score with another pick: which of them is last is the quicksort's call
  if (KEY_ORDER && threadIdx.x == 0 && npk >= 2 && sorted_key(S, S.picks[npk - 1]) == sorted_key(S, S.picks[npk - 2]))
    need[m] = 1;
  const int K = npk - ((npk > 0 && S.flag[npk - 1] == 0) ? 1 : 0);
  int written = 0;
  if (K <= kRankSortMax) {
    // few kept boxes: their input indices ranked in shared memory (all distinct)
    static_assert(sizeof(ResolveSmem) >= sizeof(int) * kRankSortMax, "rank buffer");
    int *idx = reinterpret_cast<int *>(&R);   // the round's buffers are free now
    for (int k = threadIdx.x; k < K; k += kSortNT) idx[k] = S.ord[S.picks[k]];
    __syncthreads();
    for (int k = threadIdx.x; k < K; k += kSortNT) {
      const int v = idx[k];
      int rank = 0;
      for (int j = 0; j < K; j++) rank += idx[j] < v;
      const float *P = boxes + (size_t)v * GL;
      float *Q = out + (size_t)rank * GL;
      for (int t = 0; t < GL; t++) Q[t] = P[t];
    }
    written = K;
  } else {
    int *keep = S.Rpos;
    for (int i = threadIdx.x; i < D; i += kSortNT) keep[i] = 0;
    __syncthreads();
    for (int k = threadIdx.x; k < K; k += kSortNT) keep[S.ord[S.picks[k]]] = 1;
    __syncthreads();
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
  }
  if (threadIdx.x == 0) {
    d_kept[m] = written;
    if (rounds_used) atomicMax(rounds_used, st.batches);   // batches this frame took, grid rounds and any here
    if (diag) {
      diag[8 * m + 2] = st.batches;
      diag[8 * m + 3] = npk;
      diag[8 * m + 4] = st.fallback;
      diag[8 * m + 5] = need ? need[m] : 1;
    }
  }
}

// sets an if node's condition: some model raised need
__global__ void k_nms_need(cudaGraphConditionalHandle h, const int *need, int n_models) {
  unsigned any = 0;
  for (int m = 0; m < n_models; m++) any |= need[m] ? 1u : 0u;
  cudaGraphSetConditional(h, any);
}

// Inside a stream capture: a handle for a conditional node of the graph s is
// capturing (its condition reset to init at every launch of the graph)
static cudaError_t cond_handle(cudaStream_t s, unsigned init, cudaGraphConditionalHandle *h) {
  cudaStreamCaptureStatus cs;
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamGetCaptureInfo(s, &cs, nullptr, &g, nullptr, nullptr, nullptr);
  if (e != cudaSuccess) return e;
  if (cs != cudaStreamCaptureStatusActive) return cudaErrorStreamCaptureUnsupported;
  return cudaGraphConditionalHandleCreate(h, g, init, cudaGraphCondAssignDefault);
}

// the conditional node on s's current dependencies, which become the node;
// aux then captures its body (the capture is begun here, end_conditional ends it)
static cudaError_t begin_conditional(cudaStream_t s, cudaStream_t aux, cudaGraphConditionalNodeType type,
                                     cudaGraphConditionalHandle h) {
  cudaStreamCaptureStatus cs;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t *deps = nullptr;
  const cudaGraphEdgeData *ed = nullptr;
  size_t nd = 0;
  cudaError_t e = cudaStreamGetCaptureInfo(s, &cs, nullptr, &g, &deps, &ed, &nd);
  if (e != cudaSuccess) return e;
  cudaGraphNodeParams p = {};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = h;
  p.conditional.type = type;
  p.conditional.size = 1;
  cudaGraphNode_t node;
  if ((e = cudaGraphAddNode(&node, g, deps, ed, nd, &p)) != cudaSuccess) return e;
  if ((e = cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies)) != cudaSuccess)
    return e;
  return cudaStreamBeginCaptureToGraph(aux, p.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                       cudaStreamCaptureModeRelaxed);
}

static cudaError_t end_conditional(cudaStream_t aux) {
  cudaGraph_t body = nullptr;
  cudaError_t e = cudaStreamEndCapture(aux, &body);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();   // a launch inside the body
}

// gather, the greedy rounds and the finish, in the order the sort left in (val, ord)
template <bool KEY_ORDER>
static void launch_greedy(const float *boxes, int n_models, int GL, float overlap, float cell_inv, int cap, int *si,
                          float *sf, float *out, int *d_kept, int *err, long long *diag, int rounds,
                          int *rounds_used, int *need, cudaStream_t s) {
  k_nms_gather<<<dim3((cap + kPassNT - 1) / kPassNT, n_models), kPassNT, 0, s>>>(boxes, GL, cap, si, sf);
  const int words = (cap + 31) / 32;
  const int pass_blocks = std::max(1, std::min((words + kPassNT / 32 - 1) / (kPassNT / 32), 512));
  for (int r = 0; r < rounds; r++) {
    k_nms_resolve<KEY_ORDER><<<n_models, kSortNT, 0, s>>>(cap, si, sf, overlap, cell_inv, need);
    k_nms_pass<<<dim3(pass_blocks, n_models), kPassNT, 0, s>>>(cap, si, sf, overlap, cell_inv);
  }
  k_nms_finish<KEY_ORDER><<<n_models, kSortNT, 0, s>>>(boxes, GL, cap, si, sf, overlap, out, d_kept, err, diag,
                                                       rounds_used, need, cell_inv);
}

cudaError_t launch_nms_batch(const float *boxes, const int *d_num, int n_models, int GL, float overlap,
                             float extent, int cap, int *si, float *sf, float *out, int *d_kept, int *err,
                             long long *diag, int levels, int *lv_used, int rounds, int *rounds_used, int *need,
                             int order, cudaStream_t s, cudaStream_t aux) {
  const float cell_inv = (float)kNmsCells / std::max(extent, 1.0f);
  if (n_models <= 0) return cudaSuccess;
  if (rounds <= 0) rounds = kNmsRounds;
  if (order == kNmsOrderQuicksort) {
    launch_nms_sort(boxes, d_num, n_models, GL, cap, si, sf, err, diag, levels, lv_used, nullptr, s);
    launch_greedy<false>(boxes, n_models, GL, overlap, cell_inv, cap, si, sf, out, d_kept, err, diag, rounds,
                         rounds_used, nullptr, s);
    return cudaGetLastError();
  }
  launch_nms_radix(boxes, d_num, n_models, GL, cap, si, sf, need, s);
  launch_greedy<true>(boxes, n_models, GL, overlap, cell_inv, cap, si, sf, out, d_kept, err, diag, rounds,
                      rounds_used, need, s);
  // the models whose kept set could depend on the order inside a run of equal
  // scores, again in the quicksort's order: in a graph captured with aux, an
  // if node that runs only when some model needs it; otherwise launches that
  // do nothing for the models that do not
  cudaStream_t q = s;
  cudaError_t e = cudaSuccess;
  if (aux) {
    cudaGraphConditionalHandle h;
    if ((e = cond_handle(s, 0u, &h)) != cudaSuccess) return e;
    k_nms_need<<<1, 1, 0, s>>>(h, need, n_models);
    if ((e = begin_conditional(s, aux, cudaGraphCondTypeIf, h)) != cudaSuccess) return e;
    q = aux;
  }
  launch_nms_sort(boxes, d_num, n_models, GL, cap, si, sf, err, diag, levels, lv_used, need, q);
  launch_greedy<false>(boxes, n_models, GL, overlap, cell_inv, cap, si, sf, out, d_kept, err, diag, rounds,
                       rounds_used, need, q);
  if (aux) e = end_conditional(aux);
  return e == cudaSuccess ? cudaGetLastError() : e;
}

}  // namespace geye
