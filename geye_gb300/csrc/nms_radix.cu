// nms_radix.cu -- the detections in score order for the pipeline NMS, every
// model of a frame at once: a stable least-significant-digit radix sort of the
// scores (descending) with the input index as the order among equal scores.
//
// The greedy suppression of CAR_TRACKING/nms.cpp:86-217 walks the boxes in the
// order of the reference's quicksort (nms.cpp:70-84).  That order and this one
// differ only inside runs of equal scores, and the kept set can depend on the
// order inside a run only when
//   (a) two boxes of one run are both alive when the run's turn comes and one
//       suppresses the other, or
//   (b) the last pick's run holds another pick (which of them is last decides
//       the reference's rule for a box that is alone at its turn),
// or when a score is NaN (the quicksort places it by its comparisons).  The
// greedy rounds (nms_batch.cu) check (a) and (b) as they go and raise the
// model's flag for any of them; a flagged model is then sorted again by the
// quicksort restatement (nms_sort.cu) and resolved again in that order.  The
// kept set is the reference's either way.
//
//   k_rs_load     keys (order-preserving transform of the float score, -0 as
//                 +0, complemented for descending order), indices, the greedy
//                 state; NaN raises the flag.
//   four passes of eight bits, three kernels each:
//     k_rs_count  a block per tile of nms_rs_tile(cap) keys: the digit histogram of its
//                 tile, stored digit-major (H[digit][tile]);
//     k_rs_scan   a block per model: exclusive scan of H in that order, which
//                 is each (digit, tile)'s first output position;
//     k_rs_scatter a block per tile: each key's rank among the equal digits
//                 before it in its tile (warp match, then warp prefix), so the
//                 pass is stable.
// Keys ping-pong between (val, ord) and (Lpos, Rpos); after the fourth pass
// they are back in (val, ord): val holds the transformed keys (equal keys <=>
// equal scores), ord the input index of each sorted position.
#include "nms_common.h"

namespace geye {

constexpr int kRsNT = 512;   // threads of the count and scatter blocks
constexpr int kRsWarps = kRsNT / 32;

__device__ __forceinline__ unsigned rs_key(float v, bool &nan) {
  unsigned u = __float_as_uint(v);
  if (u == 0x80000000u) u = 0u;   // -0 sorts with +0 (the quicksort's comparisons see them equal)
  nan = v != v;
  const unsigned asc = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
  return ~asc;   // ascending keys = descending scores
}

__global__ void __launch_bounds__(256) k_rs_load(const float *__restrict__ boxes_all, const int *__restrict__ d_num,
                                                 int GL, int cap, int *si, float *sf, int *need) {
  const int m = blockIdx.y;
  Slots S = slots(si, sf, m, cap);
  const float *boxes = boxes_all + (size_t)m * cap * GL;
  const int D = max(0, min(d_num[m], cap));
  const int i = blockIdx.x * 256 + threadIdx.x;
  bool nan = false;
  if (i < D) {
    const unsigned k = rs_key(boxes[(size_t)i * GL + GL - 2], nan);
    reinterpret_cast<unsigned *>(S.val)[i] = k;
    S.ord[i] = i;
  }
  if (__any_sync(0xffffffffu, nan) && (threadIdx.x & 31) == 0) need[m] = 1;
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
  }
}

// pass p reads (val, ord) for even p and (Lpos, Rpos) for odd p
__device__ __forceinline__ void rs_bufs(const Slots &S, int pass, const unsigned *&sk, const int *&si_, unsigned *&dk,
                                        int *&di) {
  unsigned *a_k = reinterpret_cast<unsigned *>(S.val), *b_k = reinterpret_cast<unsigned *>(S.Lpos);
  int *a_i = S.ord, *b_i = S.Rpos;
  if (pass & 1) {
    sk = b_k; si_ = b_i; dk = a_k; di = a_i;
  } else {
    sk = a_k; si_ = a_i; dk = b_k; di = b_i;
  }
}

__global__ void __launch_bounds__(kRsNT) k_rs_count(int pass, int cap, int *si, float *sf) {
  __shared__ int h[256];
  Slots S = slots(si, sf, blockIdx.y, cap);
  const int D = S.st->D, T = nms_rs_tile(cap);
  const int nt = (D + T - 1) / T;
  const int t = blockIdx.x;
  if (t >= nt) return;
  const unsigned *sk;
  const int *sidx;
  unsigned *dk;
  int *di;
  rs_bufs(S, pass, sk, sidx, dk, di);
  const int shift = 8 * pass;
  for (int d = threadIdx.x; d < 256; d += kRsNT) h[d] = 0;
  __syncthreads();
  const int e0 = t * T, e1 = min(e0 + T, D);
  for (int e = e0 + threadIdx.x; e < e1; e += kRsNT) atomicAdd(&h[(sk[e] >> shift) & 255u], 1);
  __syncthreads();
  for (int d = threadIdx.x; d < 256; d += kRsNT) S.hist[(size_t)d * nt + t] = h[d];
}

// exclusive scan of H (digit-major) in place, one block per model: chunks of
// kRsScanNT * kRsScanItems counts staged in shared memory with coalesced
// loads and stores, each thread scanning kRsScanItems consecutive ones
constexpr int kRsScanNT = 1024, kRsScanItems = 8, kRsScanPad = kRsScanItems + 1;
__global__ void __launch_bounds__(kRsScanNT) k_rs_scan(int cap, int *si, float *sf) {
  __shared__ int buf[kRsScanNT * kRsScanPad];   // thread t's items at t * kRsScanPad (no bank conflicts)
  __shared__ int wsum[kRsScanNT / 32];
  __shared__ int carry_s;
  Slots S = slots(si, sf, blockIdx.x, cap);
  const int D = S.st->D;
  if (D <= 0) return;
  const int n = 256 * ((D + nms_rs_tile(cap) - 1) / nms_rs_tile(cap));
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int carry = 0;
  for (int base = 0; base < n; base += kRsScanItems * kRsScanNT) {
#pragma unroll
    for (int k = 0; k < kRsScanItems; k++) {
      const int e = k * kRsScanNT + threadIdx.x;   // chunk element, coalesced
      buf[(e / kRsScanItems) * kRsScanPad + e % kRsScanItems] = base + e < n ? S.hist[base + e] : 0;
    }
    __syncthreads();
    int *mine = buf + threadIdx.x * kRsScanPad;
    int s = 0;
#pragma unroll
    for (int k = 0; k < kRsScanItems; k++) s += mine[k];
    int inc = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += y;
    }
    if (lane == 31) wsum[warp] = inc;
    __syncthreads();
    if (warp == 0) {
      int w = wsum[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += y;
      }
      wsum[lane] = w;   // inclusive over warps
      if (lane == 31) carry_s = w;
    }
    __syncthreads();
    int run = carry + (warp ? wsum[warp - 1] : 0) + inc - s;
#pragma unroll
    for (int k = 0; k < kRsScanItems; k++) {
      const int v = mine[k];
      mine[k] = run;
      run += v;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kRsScanItems; k++) {
      const int e = k * kRsScanNT + threadIdx.x;
      if (base + e < n) S.hist[base + e] = buf[(e / kRsScanItems) * kRsScanPad + e % kRsScanItems];
    }
    carry += carry_s;
    __syncthreads();   // buf, wsum and carry_s reused by the next chunk
  }
}

__global__ void __launch_bounds__(kRsNT) k_rs_scatter(int pass, int cap, int *si, float *sf) {
  __shared__ int base[256];
  __shared__ int cnt[kRsWarps][256];
  Slots S = slots(si, sf, blockIdx.y, cap);
  const int D = S.st->D, T = nms_rs_tile(cap);
  const int nt = (D + T - 1) / T;
  const int t = blockIdx.x;
  if (t >= nt) return;
  const unsigned *sk;
  const int *sidx;
  unsigned *dk;
  int *di;
  rs_bufs(S, pass, sk, sidx, dk, di);
  const int shift = 8 * pass;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int d = threadIdx.x; d < 256; d += kRsNT) base[d] = S.hist[(size_t)d * nt + t];
  const unsigned lt = (1u << lane) - 1u;
  for (int e0 = t * T; e0 < min((t + 1) * T, D); e0 += kRsNT) {
    for (int k = threadIdx.x; k < kRsWarps * 256; k += kRsNT) (&cnt[0][0])[k] = 0;
    __syncthreads();   // counters clear, base up to date
    const int e = e0 + threadIdx.x;
    const bool valid = e < D;
    const unsigned key = valid ? sk[e] : 0u;
    const int idx = valid ? sidx[e] : 0;
    const int digit = (int)((key >> shift) & 255u);
    // lanes past the end match nobody (a value no digit takes)
    const unsigned peers = __match_any_sync(0xffffffffu, valid ? digit : 256 + lane);
    const int rank = __popc(peers & lt);
    if (valid && rank == 0) cnt[warp][digit] = __popc(peers);
    __syncthreads();
    for (int d = threadIdx.x; d < 256; d += kRsNT) {
      int acc = base[d];
      for (int w = 0; w < kRsWarps; w++) {
        const int c = cnt[w][d];
        cnt[w][d] = acc;
        acc += c;
      }
      base[d] = acc;
    }
    __syncthreads();
    if (valid) {
      const int p = cnt[warp][digit] + rank;
      dk[p] = key;
      di[p] = idx;
    }
    __syncthreads();   // cnt read before the next clear
  }
}

void launch_nms_radix(const float *boxes, const int *d_num, int n_models, int GL, int cap, int *si, float *sf,
                      int *need, cudaStream_t s) {
  k_rs_load<<<dim3((cap + 255) / 256, n_models), 256, 0, s>>>(boxes, d_num, GL, cap, si, sf, need);
  const int tiles = nms_rs_tiles(cap);
  for (int p = 0; p < 4; p++) {
    k_rs_count<<<dim3(tiles, n_models), kRsNT, 0, s>>>(p, cap, si, sf);
    k_rs_scan<<<n_models, kRsScanNT, 0, s>>>(cap, si, sf);
    k_rs_scatter<<<dim3(tiles, n_models), kRsNT, 0, s>>>(p, cap, si, sf);
  }
}

}  // namespace geye
