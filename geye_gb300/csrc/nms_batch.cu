// nms_batch.cu -- NMS of the pipeline's detections, every model of a frame at once.
//
// Same kept set as nms.cu (CAR_TRACKING/nms.cpp:70-217): the reference's Hoare
// quicksort order for equal scores, greedy suppression by intersection over
// the smaller area or containment, and a box that is alone when its turn comes
// never emitted.  The greedy loop is restated so that most of it runs on every
// SM:
//
//  1. the quicksort (nms_sort.cu).
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
  if ((threadIdx.x & 31) == 0 && (r >> 5) < ((D + 31) >> 5)) S.bits[r >> 5] = bal;
}

// ---------------------------------------------------------------------------
// 3a. resolve the next batch (whole block)
// ---------------------------------------------------------------------------
struct ResolveSmem {
  int mem_pos[kBatch + 1];
  int run_end[kBatch];   // key order: last member with the same score
  float my[5][kBatch];
  unsigned rows[kBatch][kBW];
  int pick_mem[kBatch];
  int pick_any[kBatch];
  int wtot[kSortNT / 32];
  int nb, np, last_word, done;
};

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
__device__ void resolve_batch(Slots &S, float overlap, ResolveSmem &R, int *need) {
  constexpr int want = kBatch + (KEY_ORDER ? 1 : 0);   // key order: one more, to see the run at the boundary
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  BatchState &st = *S.st;
  const int nwords = st.nwords;
  if (threadIdx.x == 0) { R.nb = 0; R.last_word = st.scan_word; }
  __syncthreads();
  // members: the first kBatch alive sorted positions from scan_word on
  for (int base = st.scan_word; base < nwords; base += kSortNT) {
    const int have = R.nb;   // uniform: written before the last barrier
    if (have >= want) break;
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
    while (rem && rank < want) {
      const int b = __ffs(rem) - 1;
      rem &= rem - 1;
      R.mem_pos[rank] = (w << 5) + b;
      if (rank == kBatch - 1) R.last_word = w;
      rank++;
    }
    __syncthreads();   // everyone has read wtot and R.nb
    if (threadIdx.x == 0) {
      const int nb = min(want, have + tot);
      if (have + tot <= want) R.last_word = min(base + kSortNT, nwords);   // took every alive box up to here
      R.nb = nb;
    }
    __syncthreads();
  }
  if (KEY_ORDER) {
    if (threadIdx.x == 0 && R.nb == want) {   // an alive box follows the batch
      const unsigned kb = sorted_key(S, R.mem_pos[kBatch]);
      int nb = kBatch;
      while (nb > 0 && sorted_key(S, R.mem_pos[nb - 1]) == kb) nb--;
      if (nb == 0) {   // a run longer than a batch
        *need = 1;
        nb = kBatch;
      }
      R.nb = nb;
      R.last_word = R.mem_pos[nb - 1] >> 5;
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
    if (KEY_ORDER) {
      const unsigned k = sorted_key(S, r);
      int e = threadIdx.x;
      while (e + 1 < nb && sorted_key(S, R.mem_pos[e + 1]) == k) e++;
      R.run_end[threadIdx.x] = e;
    }
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
      if (KEY_ORDER) {
        const int e = R.run_end[i];
        if (e > i) {   // does the pick suppress an alive member of its own run (i, e]?
          const int lo = max(i + 1, 32 * lane), hi = min(e, 32 * lane + 31);
          unsigned span = 0u;
          if (lo <= hi) span = (hi - lo == 31 ? ~0u : ((1u << (hi - lo + 1)) - 1u)) << (lo - 32 * lane);
          if (__any_sync(0xffffffffu, (alive & row & span) != 0u) && lane == 0) *need = 1;
        }
      }
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
    // done once no alive box is left: none found, or this batch took every
    // one up to the end of the bitmap (its pass would test nothing)
    if (nb == 0 || R.last_word >= nwords) st.done = 1;
    R.done = nb == 0;
  }
  __syncthreads();
}

template <bool KEY_ORDER>
__global__ void __launch_bounds__(kSortNT) k_nms_resolve(int cap, int *si, float *sf, float overlap, int *need) {
  __shared__ ResolveSmem R;
  Slots S = slots(si, sf, blockIdx.x, cap);
  if (S.st->done) return;
  resolve_batch<KEY_ORDER>(S, overlap, R, need ? need + blockIdx.x : nullptr);
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
      if (lane == 0 && gone) S.bits[w] = word & ~gone;
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
    if (lane == 0 && out != word) S.bits[w] = out;
  }
}

// loop: inside a frame graph's while node, block (0, 0) sets the node's
// condition for the next round: a model is not done and has taken fewer than
// max_batches batches (the finish kernel takes any rest)
__global__ void __launch_bounds__(kPassNT) k_nms_pass(int cap, int *si, float *sf, float overlap,
                                                      cudaGraphConditionalHandle loop, int use_loop,
                                                      int max_batches) {
  __shared__ float pk[5][kBatch];
  if (use_loop && blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) {
    unsigned more = 0;
    for (int m = 0; m < (int)gridDim.y; m++) {
      const BatchState &b = *slots(si, sf, m, cap).st;
      more |= (!b.done && b.batches < max_batches) ? 1u : 0u;
    }
    cudaGraphSetConditional(loop, more);
  }
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
// KEY_ORDER: the key-order pass (writes every model's result; raises need[m]
// where the quicksort order could differ).  Otherwise the quicksort-order pass:
// with need given, only the models that raised it (their result replaces the
// key-order one); without, every model.
template <bool KEY_ORDER>
__global__ void __launch_bounds__(kSortNT) k_nms_finish(const float *__restrict__ boxes_all, int GL, int cap,
                                                        int *si, float *sf, float overlap, float *out_all,
                                                        int *d_kept, int *err, long long *diag, int *rounds_used,
                                                        int *need) {
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
      resolve_batch<KEY_ORDER>(S, overlap, R, need ? need + m : nullptr);
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

constexpr int kNmsLoopBatches = 512;   // while-node rounds before the finish kernel takes the rest

// gather, the greedy rounds and the finish, in the order the sort left in (val, ord).
// aux non-null: s is capturing a graph, and the rounds are a while node (as many
// as the frame needs) instead of `rounds` launches
template <bool KEY_ORDER>
static cudaError_t launch_greedy(const float *boxes, int n_models, int GL, float overlap, int cap, int *si, float *sf,
                                 float *out, int *d_kept, int *err, long long *diag, int rounds, int *rounds_used,
                                 int *need, cudaStream_t s, cudaStream_t aux) {
  k_nms_gather<<<dim3((cap + kPassNT - 1) / kPassNT, n_models), kPassNT, 0, s>>>(boxes, GL, cap, si, sf);
  const int words = (cap + 31) / 32;
  const int pass_blocks = std::max(1, std::min((words + kPassNT / 32 - 1) / (kPassNT / 32), 512));
  if (aux) {
    cudaGraphConditionalHandle loop;
    cudaError_t e = cond_handle(s, 1u, &loop);
    if (e == cudaSuccess) e = begin_conditional(s, aux, cudaGraphCondTypeWhile, loop);
    if (e != cudaSuccess) return e;
    k_nms_resolve<KEY_ORDER><<<n_models, kSortNT, 0, aux>>>(cap, si, sf, overlap, need);
    k_nms_pass<<<dim3(pass_blocks, n_models), kPassNT, 0, aux>>>(cap, si, sf, overlap, loop, 1, kNmsLoopBatches);
    if ((e = end_conditional(aux)) != cudaSuccess) return e;
  } else {
    for (int r = 0; r < rounds; r++) {
      k_nms_resolve<KEY_ORDER><<<n_models, kSortNT, 0, s>>>(cap, si, sf, overlap, need);
      k_nms_pass<<<dim3(pass_blocks, n_models), kPassNT, 0, s>>>(cap, si, sf, overlap, 0, 0, 0);
    }
  }
  k_nms_finish<KEY_ORDER><<<n_models, kSortNT, 0, s>>>(boxes, GL, cap, si, sf, overlap, out, d_kept, err, diag,
                                                       rounds_used, need);
  return cudaSuccess;
}

cudaError_t launch_nms_batch(const float *boxes, const int *d_num, int n_models, int GL, float overlap, int cap,
                             int *si, float *sf, float *out, int *d_kept, int *err, long long *diag, int levels,
                             int *lv_used, int rounds, int *rounds_used, int *need, int order, cudaStream_t s,
                             cudaStream_t aux) {
  if (n_models <= 0) return cudaSuccess;
  if (rounds <= 0) rounds = kNmsRounds;
  cudaError_t e;
  if (order == kNmsOrderQuicksort) {
    launch_nms_sort(boxes, d_num, n_models, GL, cap, si, sf, err, diag, levels, lv_used, nullptr, s);
    return launch_greedy<false>(boxes, n_models, GL, overlap, cap, si, sf, out, d_kept, err, diag, rounds,
                                rounds_used, nullptr, s, aux);
  }
  launch_nms_radix(boxes, d_num, n_models, GL, cap, si, sf, need, s);
  e = launch_greedy<true>(boxes, n_models, GL, overlap, cap, si, sf, out, d_kept, err, diag, rounds, rounds_used,
                          need, s, aux);
  if (e != cudaSuccess) return e;
  // the models whose kept set could depend on the order inside a run of equal
  // scores, again in the quicksort's order: in a graph, an if node that runs
  // only when some model needs it; otherwise launches that do nothing for the others
  cudaStream_t q = s;
  if (aux) {
    cudaGraphConditionalHandle h;
    if ((e = cond_handle(s, 0u, &h)) != cudaSuccess) return e;
    k_nms_need<<<1, 1, 0, s>>>(h, need, n_models);
    if ((e = begin_conditional(s, aux, cudaGraphCondTypeIf, h)) != cudaSuccess) return e;
    q = aux;
  }
  launch_nms_sort(boxes, d_num, n_models, GL, cap, si, sf, err, diag, levels, lv_used, need, q);
  e = launch_greedy<false>(boxes, n_models, GL, overlap, cap, si, sf, out, d_kept, err, diag, rounds, rounds_used,
                           need, q, nullptr);
  if (aux) {
    const cudaError_t e2 = end_conditional(aux);
    if (e == cudaSuccess) e = e2;
  }
  return e;
}

}  // namespace geye
