// score.cu -- score assembly, detection records, accumulated score map and
// box regression.
//
//   score = root + offw[ridx[c]] - sum_k M_k[(ay_k-1+2y) + (ax_k-1+2x)*d0_k]
//       CAR_TRACKING/get_boxes.cpp:1022-1041 and dt.cpp:38-55, parts in order
//   threshold in column-major scan order, level by level, component by
//   component: get_boxes.cpp:185-220 (get_gmpc), :1497-1569, :1746-1762
//   root / part boxes: get_boxes.cpp:227-258
//   A_SCORE: get_boxes.cpp:265-300 (CPU form), normalised at :1765-1787
//   box regression: CAR_TRACKING/tracking.cpp:90-166 (get_new_rects)
// Records are written in the reference's order: a per-block count pass, an
// exclusive scan, and a write pass that recomputes the same flags.
#include <algorithm>

#include "internal.h"

namespace geye {

constexpr int kScoreThreads = 256;

__global__ void k_fill(float *__restrict__ p, size_t n, float v) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) p[i] = v;
}

void launch_fill(float *p, size_t n, float v, cudaStream_t s) {
  size_t b = (n + 255) / 256;
  k_fill<<<(unsigned)(b > 4096 ? 4096 : (b ? b : 1)), 256, 0, s>>>(p, n, v);
}

__device__ __forceinline__ float assemble(const ScoreJob &J, const float *__restrict__ arena, int x, int y) {
  const int i = x * J.r0 + y;
  float s = arena[J.root_off + i];
  s += J.off;
  for (int k = 0; k < J.np; k++) {
    // M at (ax - 1 + 2x, ay - 1 + 2y); compact: its class entry ((ax - 1) / 2 + x, (ay - 1) / 2 + y)
    const int cm0 = J.part_cm0[k];
    const int idx = cm0 ? ((J.ax[k] - 1) / 2 + x) * cm0 + ((J.ay[k] - 1) / 2 + y)
                        : (J.ay[k] + 2 * y - 1) + (J.ax[k] - 1 + 2 * x) * J.part_d0[k];
    s -= arena[J.part_M[k] + idx];
  }
  return s;
}

// One block per entry of `blocks` (job, block of 256 positions): exactly the
// blocks the maps need, whatever their sizes across levels.  Its count of
// positions above the threshold goes to block_counts[blockIdx.x]; the list is
// in job order, so the exclusive scan of the counts places every block's
// records in the reference's order.
__global__ void k_score(const ScoreJob *__restrict__ jobs, const int2 *__restrict__ blocks, float thresh,
                        float *__restrict__ arena, int *__restrict__ block_counts) {
  const int2 blk = blocks[blockIdx.x];
  const ScoreJob &J = jobs[blk.x];
  const int n = J.r0 * J.r1;
  const int i = blk.y * kScoreThreads + threadIdx.x;
  int flag = 0;
  if (i < n) {
    const int y = i % J.r0, x = i / J.r0;
    const float s = assemble(J, arena, x, y);
    arena[J.score_off + i] = s;
    flag = s > thresh;
  }
  const int c = __syncthreads_count(flag);
  if (threadIdx.x == 0) block_counts[blockIdx.x] = c;   // block-list order: job, then position
}

void score_block_list(const std::vector<ScoreJob> &jobs, std::vector<int2> &blocks) {
  blocks.clear();
  for (size_t j = 0; j < jobs.size(); j++)
    for (int b = 0; b * kScoreThreads < jobs[j].r0 * jobs[j].r1; b++) blocks.push_back(make_int2((int)j, b));
}

void launch_score(const ScoreJob *d_jobs, const int2 *d_blocks, int n_blocks, float thresh, float *arena,
                  int *block_counts, cudaStream_t s) {
  if (n_blocks <= 0) return;
  k_score<<<n_blocks, kScoreThreads, 0, s>>>(d_jobs, d_blocks, thresh, arena, block_counts);
}

// exclusive scan of n ints in place (one block); *total gets the sum
__global__ void k_scan(int *__restrict__ a, int n, int *__restrict__ total) {
  __shared__ int warp_sums[32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int base = 0; base < n; base += blockDim.x) {
    const int i = base + threadIdx.x;
    const int v = i < n ? a[i] : 0;
    int inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int t = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += t;
    }
    if (lane == 31) warp_sums[warp] = inc;
    __syncthreads();
    if (warp == 0) {
      int w = lane < nw ? warp_sums[lane] : 0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += t;
      }
      if (lane < nw) warp_sums[lane] = w;   // inclusive warp prefix
    }
    __syncthreads();
    const int before = carry + (warp > 0 ? warp_sums[warp - 1] : 0) + inc - v;
    if (i < n) a[i] = before;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = before + v;
    __syncthreads();
  }
  if (threadIdx.x == 0 && total) *total = carry;
}

void launch_scan_counts(int *counts, int n, int *total, cudaStream_t s) {
  k_scan<<<1, 1024, 0, s>>>(counts, n, total);
}

// Records of a block are contiguous in the output (its offset from the scan,
// then rank order), so they are built in shared memory and written out with
// coalesced stores.
//
// partbox (get_boxes.cpp:243-258) is written in double; every step of it is
// exact except the final rounding to float, so it is restated in float and
// integer arithmetic with that one rounding (the FP64 pipe is narrow here):
//   q0 = ((py - 2)/2 + 1) * scale  ==  (py * 0.5f) * scale   (exact product, one rounding)
//   q2 = q0 + psize*scale/2 - 1     ==  one rounding of the exact sum (below)

// float(q + h - 1) with the sum taken exactly.  For q, h in [0.5, 2^23) the
// double expression is exact before its rounding to float.  In float:
// s + e = q + h exactly (TwoSum; no contraction), s - 1 is exact for
// 1 <= s < 2^24 (1 is a multiple of s's unit in the last place), so
// (s - 1) + e is one correctly rounded addition of the exact q + h - 1.
// (64-bit integer conversions would run on the narrow FP64 pipe.)
__device__ __forceinline__ float sum_minus_one(float q, float h) {
  if (q >= 0.5f && h >= 0.5f && q < 8388608.0f && h < 8388608.0f) {
    const float s = q + h;
    const float bb = s - q;
    const float e = (q - (s - bb)) + (h - bb);
    return (s - 1.0f) + e;
  }
  return (float)((double)q + (double)h - 1.0);
}

__global__ void __launch_bounds__(kScoreThreads) k_boxes(const ScoreJob *__restrict__ jobs,
                                                         const int2 *__restrict__ blocks, float thresh,
                                                         const float *__restrict__ arena,
                                                         const int *__restrict__ arena_i,
                                                         const int *__restrict__ block_offsets, int GL,
                                                         float *__restrict__ boxes) {
  extern __shared__ float rec_s[];   // [count][GL]
  __shared__ int warp_cnt[kScoreThreads / 32];
  const int2 blk = blocks[blockIdx.x];
  const ScoreJob &J = jobs[blk.x];
  const int n = J.r0 * J.r1;
  const int i = blk.y * kScoreThreads + threadIdx.x;
  float s = 0.f;
  int flag = 0;
  if (i < n) {
    s = arena[J.score_off + i];
    flag = s > thresh;
  }
  const unsigned bal = __ballot_sync(0xffffffffu, flag);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) warp_cnt[warp] = __popc(bal);
  __syncthreads();
  int rank = __popc(bal & ((1u << lane) - 1)), count = 0;
  for (int w = 0; w < kScoreThreads / 32; w++) {
    if (w < warp) rank += warp_cnt[w];
    count += warp_cnt[w];
  }
  if (count == 0) return;
  if (flag) {
    const int y = i % J.r0, x = i / J.r0;
    float *P = rec_s + rank * GL;
    const float scale = J.scale;
    root_box(x, y, scale, J.rsize0, J.rsize1, P);
    float *Q = P + 4;
    for (int k = 0; k < J.np; k++) {
      const int probex = (x - 1) * 2 + J.ax[k];
      const int probey = (y - 1) * 2 + J.ay[k];
      long Pi;
      if (const int ci0 = J.part_ci0[k]) {   // compact: every probe is inside and in the stored class
        Pi = (long)(probex >> 1) * ci0 + (probey >> 1);
      } else {
        Pi = probey + (long)probex * J.part_d0[k];
        // the reference reads outside the map here (undefined); use entry 0 instead
        if (Pi < 0 || Pi >= (long)J.part_d0[k] * J.part_d1[k]) Pi = 0;
      }
      const float px = (float)arena_i[J.part_Ix[k] + Pi] + 1.0f;   // an integer: exact
      const float py = (float)arena_i[J.part_Iy[k] + Pi] + 1.0f;
      const float q0 = (py * 0.5f) * scale;
      const float q1 = (px * 0.5f) * scale;
      Q[0] = q0;
      Q[1] = q1;
      Q[2] = sum_minus_one(q0, ((float)J.psize0[k] * scale) * 0.5f);
      Q[3] = sum_minus_one(q1, ((float)J.psize1[k] * scale) * 0.5f);
      Q += 4;
    }
    Q[0] = (float)J.comp;
    Q[1] = s;
    Q[2] = scale;
  }
  __syncthreads();
  float *out = boxes + (size_t)block_offsets[blockIdx.x] * GL;
  for (int t = threadIdx.x; t < count * GL; t += kScoreThreads) out[t] = rec_s[t];
}

void launch_boxes(const ScoreJob *d_jobs, const int2 *d_blocks, int n_blocks, float thresh, const float *arena,
                  const int *arena_i, const int *block_offsets, int GL, float *boxes, cudaStream_t s) {
  if (n_blocks <= 0) return;
  const size_t smem = sizeof(float) * kScoreThreads * GL;
  static SmemAttr attr;
  raise_smem(attr, k_boxes, smem);
  k_boxes<<<n_blocks, kScoreThreads, smem, s>>>(d_jobs, d_blocks, thresh, arena, arena_i, block_offsets, GL, boxes);
}

// A_SCORE in gather form: target pixel (X, Y) takes the max over every
// (level, component) of the score at the cell that the reference's scatter
// loop maps from source pixel (X - RX, Y - RY) -- looked up in the plan's
// per-map column and row tables -- then the threshold/offset of
// get_boxes.cpp:1765-1776 and a running maximum for the normalisation.
// A block owns a 16 x 16 pixel tile and stages the tile's table entries of
// every map in shared memory, so only the score gathers touch global memory.
// The maximum is exact in any order.
constexpr int kAsTile = 16;

__global__ void __launch_bounds__(kAsTile *kAsTile) k_ascore(const int *__restrict__ col, const int *__restrict__ row,
                                                             int n_jobs, const float *__restrict__ arena,
                                                             float *__restrict__ a_score, int im_w, int im_h,
                                                             float thresh, unsigned *max_bits) {
  extern __shared__ int tab_s[];   // [job][16] column bases, then [job][16] rows
  const int X0 = blockIdx.y * kAsTile, Y0 = blockIdx.x * kAsTile;
  for (int i = threadIdx.x; i < n_jobs * kAsTile; i += blockDim.x) {
    const int j = i / kAsTile, k = i % kAsTile;
    tab_s[i] = X0 + k < im_w ? col[(size_t)j * im_w + X0 + k] : -1;
    tab_s[n_jobs * kAsTile + i] = Y0 + k < im_h ? row[(size_t)j * im_h + Y0 + k] : -1;
  }
  __syncthreads();
  const int tx = threadIdx.x / kAsTile, ty = threadIdx.x % kAsTile;
  const int X = X0 + tx, Y = Y0 + ty;
  unsigned local_max = 0;
  if (X < im_w && Y < im_h) {
    const size_t idx = (size_t)X * im_h + Y;
    float a = a_score[idx];
    const int *tc = tab_s + tx, *tr = tab_s + n_jobs * kAsTile + ty;
#pragma unroll 8   // eight gathers in flight per thread (the maximum is exact in any order)
    for (int j = 0; j < n_jobs; j++) {
      const int c = tc[j * kAsTile], r = tr[j * kAsTile];
      if ((c | r) >= 0) {
        const float sc = arena[c + r];
        if (sc > a) a = sc;
      }
    }
    const float AS_OFF = fabsf(thresh);
    if (a < thresh) a = 0.0;
    else a += AS_OFF;
    a_score[idx] = a;
    const unsigned bits = __float_as_uint(a);
    if (a > 0.0f) local_max = bits;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) local_max = max(local_max, __shfl_xor_sync(0xffffffffu, local_max, o));
  if ((threadIdx.x & 31) == 0 && local_max) atomicMax(max_bits, local_max);
}

__global__ void k_ascore_norm(float *__restrict__ a_score, int n, const unsigned *__restrict__ max_bits) {
  const float max_ac = __uint_as_float(*max_bits);
  if (!(max_ac > 0.0f)) return;
  // the reference's double reciprocal, once per warp (the FP64 pipe is narrow)
  float ac_ratio = 0.f;
  if ((threadIdx.x & 31) == 0) ac_ratio = 1.0 / max_ac;
  ac_ratio = __shfl_sync(0xffffffffu, ac_ratio, 0);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a_score[i] *= ac_ratio;
}

void launch_ascore(const int *col, const int *row, int n_jobs, const float *arena, float *a_score, int im_w,
                  int im_h, float thresh, unsigned *max_bits, cudaStream_t s) {
  dim3 grid((im_h + kAsTile - 1) / kAsTile, (im_w + kAsTile - 1) / kAsTile);
  const size_t smem = sizeof(int) * 2 * kAsTile * (size_t)std::max(n_jobs, 1);
  static SmemAttr attr;
  raise_smem(attr, k_ascore, smem);
  k_ascore<<<grid, kAsTile * kAsTile, smem, s>>>(col, row, n_jobs, arena, a_score, im_w, im_h, thresh, max_bits);
}

void launch_ascore_normalize(float *a_score, int n, const unsigned *max_bits, cudaStream_t s) {
  int blocks = (n + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  k_ascore_norm<<<blocks, 256, 0, s>>>(a_score, n, max_bits);
}

// get_new_rects on the kept records: coef = [comp][x1, y1, x2, y2][ML]
__global__ void k_new_rects(const float *__restrict__ kept, const int *__restrict__ d_kept, int GL, int np,
                            const float *__restrict__ coef, int img_w, int img_h, float ratio, int *point,
                            int *or_point, int *type, float *scale, float *score) {
  const int K = *d_kept;
  const int ML = 1 + 2 * (1 + np);
  const int LL = GL - 3;
  for (int ii = blockIdx.x * blockDim.x + threadIdx.x; ii < K; ii += gridDim.x * blockDim.x) {
    const float *P = kept + (size_t)ii * GL;
    const int CNUM = (int)P[GL - 3];
    const float *x1 = coef + ((size_t)CNUM * 4 + 0) * ML;
    const float *y1 = coef + ((size_t)CNUM * 4 + 1) * ML;
    const float *x2 = coef + ((size_t)CNUM * 4 + 2) * ML;
    const float *y2 = coef + ((size_t)CNUM * 4 + 3) * ML;
    float XP1 = 0, XP2 = 0, YP1 = 0, YP2 = 0;
    for (int kk = 0; kk < ML; kk++) {
      float av;
      if (kk == 0) av = P[3] - P[1];
      else {
        const int q = kk - 1;                 // Avec = [w, (x1, y1) of root and parts]
        const int box = q >> 1;
        av = (q & 1) ? P[4 * box] : P[4 * box + 1];
        if (4 * box >= LL) av = 0.f;
      }
      YP1 += av * y1[kk];
      YP2 += av * y2[kk];
      XP1 += av * x1[kk];
      XP2 += av * x2[kk];
    }
    int PP[4];
    PP[0] = XP1 > 0 ? (int)XP1 : 0;
    PP[1] = YP1 > 0 ? (int)YP1 : 0;
    PP[2] = XP2 < img_w ? (int)XP2 : img_w;
    PP[3] = YP2 < img_h ? (int)YP2 : img_h;
    for (int q = 0; q < 4; q++) {
      point[4 * ii + q] = PP[q];
      or_point[4 * ii + q] = (int)((float)PP[q] / ratio);
    }
    type[ii] = CNUM;
    scale[ii] = P[GL - 1];
    score[ii] = P[GL - 2];
  }
}

void launch_new_rects(const float *kept, const int *d_kept, int GL, int np, const float *coef, int img_w,
                      int img_h, float ratio, int *point, int *or_point, int *type, float *scale, float *score,
                      cudaStream_t s) {
  k_new_rects<<<16, 256, 0, s>>>(kept, d_kept, GL, np, coef, img_w, img_h, ratio, point, or_point, type, scale,
                                 score);
}

}  // namespace geye
