// dt.cu -- generalized distance transform with argmax displacements.
//
// Reference: CAR_TRACKING/dt.cpp:61-136.  dt_helper is a divide-and-conquer
// monotone argmin: for the middle d of [d1, d2] it scans s in [s1, s2]
// keeping the leftmost minimum of
//     f_d(s) = (v[s] + (a*t)*t) + b*t,  t = d - s   (float, no FMA)
// and recurses on [d1, d-1] x [s1, s*] and [d+1, d2] x [s*, s2].
//
// GPU form.  Let g(d) be the leftmost global argmin of f_d over the whole
// line.  If g is non-decreasing in d, the recursion returns g(d) for every d
// (each node's range [s1, s2] then contains g(d), and no smaller index in it
// reaches the minimum).  So every output of a line is computed in parallel.
// Where dt_monotone proves from the line's value range and (a, b) that the
// computed g cannot decrease (the usual case: a >= 8 times the rounding bound),
// nothing else is needed, and pass 2 computes only the entries it stores;
// otherwise g is checked to be non-decreasing, and only if it is not does one
// thread replay the recursion exactly (counted in *fallback_count).
//
// A block takes a tile of L consecutive lines (about `elems` outputs: the
// plan's tuned tile size, kDtElems by default) into
// shared memory, each line padded with +inf, and spreads the tile's outputs
// over its threads: a thread scans its output's window with no bounds checks
// (an inf candidate never wins a strict comparison), using per-offset terms
// (a*t)*t and b*t tabulated once per block -- the same roundings as dt_f.
//
// g(d) is searched in a window |d - s| < K.  K is chosen so that every s
// outside the window has f_d(s) > max(v) >= f_d(d): with u = 2^-24,
// f_d(s) >= v_min + (1-8u) a t^2 - (1+8u)|b t| - 8u max|v| for a > 0, and K
// is the first integer past the positive root of that bound minus v_max.
// For a <= 0 the window is the whole line.  Pass 1 (columns: many short
// lines per tile) takes one K from the whole tile's value range and, when the
// order is proven and K <= 8, scans with the per-offset terms in registers;
// pass 2 (rows: a few long lines) takes a K per line and, when the order is
// proven and every line's K <= 8, reads the terms of each line's window from
// one register table.
#include <math.h>

#include <algorithm>

#include "internal.h"

namespace geye {

constexpr int kDtThreads = 256;
// kDtElems (outputs per block, about) is in internal.h: plans tune it
constexpr int kDtPad = 64;          // largest window half-width served by the fast loop

__device__ __forceinline__ float dt_f(float v, float a, float b, int t) {
  return v + a * t * t + b * t;      // ((v + (a*t)*t) + b*t), each op rounded (no FMA)
}

// window half-width bound K for one line (a > 0); returns n when unbounded.
// Float arithmetic (the FP64 pipe is narrow on this GPU): A and B are pushed
// down and up by 2^-18 and the root up by 2^-16, far more than the few
// 2^-24 roundings of the expression, so K never falls below the exact bound.
__device__ __forceinline__ int dt_window(float vmin, float vmax, float vabs, float a, float b, int n) {
  if (!(a > 0.f)) return n;
  const float u = 8.0f * 5.9604644775390625e-08f;   // 8 * 2^-24
  const float lo = 1.0f - 3.814697265625e-06f;      // 1 - 2^-18
  const float hi = 1.0f + 3.814697265625e-06f;      // 1 + 2^-18
  const float A = (1.0f - u) * a * lo;
  const float B = (1.0f + u) * fabsf(b) * hi;
  const float R = ((vmax - vmin) * hi + u * vabs * hi) * hi + 1e-30f;
  const float root = (B + sqrtf(B * B * hi + 4.0f * A * R * hi)) / (2.0f * A) * (1.0f + 1.52587890625e-05f);
  if (!(root < (float)n)) return n;
  return (int)floorf(root) + 2;
}

// Exact replay of dt_helper for one line (one thread).
__device__ void dt_replay(const float *v, int n, float a, float b, float *out, int *arg) {
  int st[4 * 64];
  int sp = 0;
  st[sp++] = 0; st[sp++] = n - 1; st[sp++] = 0; st[sp++] = n - 1;
  while (sp > 0) {
    const int d2 = st[--sp], d1 = st[--sp], s2 = st[--sp], s1 = st[--sp];
    if (d2 < d1) continue;
    const int d = (d1 + d2) >> 1;
    int s = s1;
    float src_ss = v[s];
    for (int p = s1 + 1; p <= s2; p++) {
      int t1 = d - s, t2 = d - p;
      if (src_ss + a * t1 * t1 + b * t1 > v[p] + a * t2 * t2 + b * t2) {
        s = p;
        src_ss = v[s];
      }
    }
    const int D = d - s;
    out[d] = v[s] + a * D * D + b * D;
    arg[d] = s;
    if (sp + 8 <= 4 * 64) {
      st[sp++] = s; st[sp++] = s2; st[sp++] = d + 1; st[sp++] = d2;
      st[sp++] = s1; st[sp++] = s; st[sp++] = d1; st[sp++] = d - 1;
    }
  }
}

// lines per block: pass 1 (columns, contiguous) any count up to 64; pass 2
// (rows, strided in memory) a power of two up to 16 so that staging is coalesced
__host__ __device__ __forceinline__ int dt_lines1(int n, int elems) { return max(1, min(64, elems / max(n, 1))); }
__host__ __device__ __forceinline__ int dt_lg_lines2(int n, int elems) {
  int lg = 0;
  while (lg < 4 && (2 << lg) * n <= elems) lg++;
  return lg;
}
__host__ __device__ __forceinline__ size_t dt_smem_bytes(int L, int n) {
  return sizeof(float) * ((size_t)kDtPad + (size_t)L * (n + kDtPad) + 2 * (size_t)L * n + 2 * (2 * kDtPad - 1)) +
         sizeof(int) * (2 * (size_t)L + 1) + sizeof(float) * 3 * (kDtThreads / 32) + sizeof(int);
}

// Leftmost minimum of output d over the window |t| < KM of a padded line,
// unrolled; At/Bt: (a*t)*t and b*t tabulated in shared memory (broadcast
// reads).  KM may exceed the line's own K: candidates past K lose to f_d(d)
// anyway, so a wider window returns the same leftmost minimum.
template <int KM>
__device__ __forceinline__ int dt_scan_fixed(const float *__restrict__ line, int d, const float *__restrict__ At,
                                             const float *__restrict__ Bt, float &best) {
  const float *v = line + d - (KM - 1);   // v[i] = line[d - t], t = KM-1-i: p ascending
  best = INFINITY;
  int s = -1;
#pragma unroll
  for (int i = 0; i < 2 * KM - 1; i++) {
    const float f = (v[i] + At[KM - 1 - i]) + Bt[KM - 1 - i];
    if (f < best) { best = f; s = i; }
  }
  return s < 0 ? -1 : d - (KM - 1) + s;
}

// Leftmost minimum of output d over its line's window (K rounded up to an
// unrolled size, a loop beyond 16, a bounds-checked loop past the padding).
__device__ __forceinline__ int dt_full(const float *__restrict__ line, int d, int K, int n, float a, float b,
                                       const float *__restrict__ At, const float *__restrict__ Bt, float &best) {
  int p;
  if (K <= 3) p = dt_scan_fixed<3>(line, d, At, Bt, best);
  else if (K <= 4) p = dt_scan_fixed<4>(line, d, At, Bt, best);
  else if (K <= 5) p = dt_scan_fixed<5>(line, d, At, Bt, best);
  else if (K <= 6) p = dt_scan_fixed<6>(line, d, At, Bt, best);
  else if (K <= 8) p = dt_scan_fixed<8>(line, d, At, Bt, best);
  else if (K <= 12) p = dt_scan_fixed<12>(line, d, At, Bt, best);
  else if (K <= 16) p = dt_scan_fixed<16>(line, d, At, Bt, best);
  else if (K <= kDtPad) {
    best = INFINITY;
    p = -1;
    for (int t = K - 1; t > -K; t--) {   // p = d - t ascending
      const float f = (line[d - t] + At[t]) + Bt[t];
      if (f < best) { best = f; p = d - t; }
    }
  } else {
    const int lo = max(0, d - K + 1), hi = min(n - 1, d + K - 1);
    p = lo;
    best = dt_f(line[lo], a, b, d - lo);
    for (int q = lo + 1; q <= hi; q++) {
      const float fq = dt_f(line[q], a, b, d - q);
      if (best > fq) { best = fq; p = q; }
    }
  }
  if (p < 0) {   // every candidate was NaN: the reference keeps the window's first index
    p = max(0, d - K + 1);
    best = dt_f(line[p], a, b, d - p);
  }
  return p;
}

// Outputs d = c + q*i of every line of the tile, spread over all threads
// (e -> line e / m, slot e % m, the division by a precomputed reciprocal), each
// with its own line's window.  q = 1: every output (c = 0); q = 2: the parity
// class c of line l that pass 2 writes (par_x on rows of parity par_y, the
// other class on the other rows).
__device__ __forceinline__ void dt_scan_tile(const float *__restrict__ v_s, int stride, int n, int nl, float a,
                                             float b, const int *__restrict__ K_s, const float *__restrict__ At,
                                             const float *__restrict__ Bt, float *__restrict__ o_s,
                                             int *__restrict__ g_s, int q, int y0, int par_y, int par_x) {
  const int m = (n + q - 1) / q;
  const unsigned mg = 0xFFFFFFFFu / (unsigned)m + 1u;   // e / m for e < 2^32 / m
  for (int e = threadIdx.x; e < nl * m; e += blockDim.x) {
    const int l = __umulhi((unsigned)e, mg), i = e - l * m;
    const int c = q == 1 ? 0 : (((y0 + l) & 1) == par_y ? par_x : 1 - par_x);
    const int d = c + q * i;
    if (d >= n) continue;
    float best;
    const int p = dt_full(v_s + l * stride, d, K_s[l], n, a, b, At, Bt, best);
    o_s[l * n + d] = best;
    g_s[l * n + d] = p;
  }
}

// Outputs of the tile when the argmin order is proven (every value finite,
// one window K <= KM for the whole tile): the outputs d = c + q * i of every
// line spread over the threads as in dt_scan_tile (consecutive outputs to
// consecutive lanes: conflict-free shared-memory reads), with the per-offset
// terms (a*t)*t and b*t (the same roundings as dt_f) held in registers; each
// output is the leftmost minimum over its window, candidates in ascending order.
template <int KM, int Q>
__device__ __forceinline__ void dt_mono_tile(const float *__restrict__ v_s, int stride, int n, int nl, float a,
                                             float b, float *__restrict__ o_s, int *__restrict__ g_s, int y0,
                                             int par_y, int par_x) {
  constexpr int W = 2 * KM - 1;
  float At[W], Bt[W];
#pragma unroll
  for (int j = 0; j < W; j++) {
    const float ft = (float)(KM - 1 - j);   // t = d - p for candidate j of a window
    At[j] = a * ft * ft;
    Bt[j] = b * ft;
  }
  const int m = (n + Q - 1) / Q;
  const unsigned mg = 0xFFFFFFFFu / (unsigned)m + 1u;   // e / m for e < 2^32 / m
  for (int e = threadIdx.x; e < nl * m; e += blockDim.x) {
    const int l = __umulhi((unsigned)e, mg), i = e - l * m;
    const int c = Q == 1 ? 0 : (((y0 + l) & 1) == par_y ? par_x : 1 - par_x);
    const int d = c + Q * i;
    if (d >= n) continue;
    const float *v = v_s + l * stride + d - (KM - 1);   // padded: reads past the line see +inf
    float best = INFINITY;
    int s = 0;
#pragma unroll
    for (int j = 0; j < W; j++) {
      const float f = (v[j] + At[j]) + Bt[j];
      if (f < best) { best = f; s = j; }
    }
    o_s[l * n + d] = best;
    g_s[l * n + d] = d - (KM - 1) + s;
  }
}

// Leftmost minimum over the window |t| < KK of output d, the per-offset
// terms taken from registers At8/Bt8 (offsets t = 7 - j, j = 0..14)
template <int KK>
__device__ __forceinline__ int dt_scan_slice(const float *__restrict__ line, int d, const float (&At8)[15],
                                             const float (&Bt8)[15], float &best) {
  const float *v = line + d - (KK - 1);
  best = INFINITY;
  int s = 0;
#pragma unroll
  for (int jj = 0; jj < 2 * KK - 1; jj++) {
    const float f = (v[jj] + At8[jj + 8 - KK]) + Bt8[jj + 8 - KK];
    if (f < best) { best = f; s = jj; }
  }
  return d - (KK - 1) + s;
}

// As dt_scan_tile for a proven order with every line's window at most 8: the
// same outputs and candidates, a window per line, the per-offset terms in registers.
template <int Q>
__device__ __forceinline__ void dt_scan_tile_reg(const float *__restrict__ v_s, int stride, int n, int nl, float a,
                                                 float b, const int *__restrict__ K_s, float *__restrict__ o_s,
                                                 int *__restrict__ g_s, int y0, int par_y, int par_x) {
  float At8[15], Bt8[15];
#pragma unroll
  for (int j = 0; j < 15; j++) {
    const float ft = (float)(7 - j);
    At8[j] = a * ft * ft;
    Bt8[j] = b * ft;
  }
  const int m = (n + Q - 1) / Q;
  const unsigned mg = 0xFFFFFFFFu / (unsigned)m + 1u;
  for (int e = threadIdx.x; e < nl * m; e += blockDim.x) {
    const int l = __umulhi((unsigned)e, mg), i = e - l * m;
    const int c = Q == 1 ? 0 : (((y0 + l) & 1) == par_y ? par_x : 1 - par_x);
    const int d = c + Q * i;
    if (d >= n) continue;
    const float *line = v_s + l * stride;
    float best;
    int p;
    switch (K_s[l]) {
      case 0: case 1: case 2: p = dt_scan_slice<2>(line, d, At8, Bt8, best); break;
      case 3: p = dt_scan_slice<3>(line, d, At8, Bt8, best); break;
      case 4: p = dt_scan_slice<4>(line, d, At8, Bt8, best); break;
      case 5: p = dt_scan_slice<5>(line, d, At8, Bt8, best); break;
      case 6: p = dt_scan_slice<6>(line, d, At8, Bt8, best); break;
      case 7: p = dt_scan_slice<7>(line, d, At8, Bt8, best); break;
      default: p = dt_scan_slice<8>(line, d, At8, Bt8, best); break;
    }
    o_s[l * n + d] = best;
    g_s[l * n + d] = p;
  }
}

// True when the computed leftmost argmin g(d) of a line is certainly
// non-decreasing in d.  For s < p, the exact terms give
//   [f_d(s) - f_d(p)] - [f_{d-1}(s) - f_{d-1}(p)] = 2a(p - s) >= 2a,
// and each computed f (four roundings, no FMA) is within
// E = 4u(|v| + a t^2 + |b t|) of the exact one (u = 2^-24, |t| <= K for the
// argmins of d and d - 1, which lie in their windows).  g(d) < g(d-1) needs
// the computed bracket below zero, so 2a > 4E; a >= 8E rules it out with a
// factor 4 to spare (the 1e-37 covers subnormal roundings).  NaN or infinite
// values, a <= 0 and windows past the padding fail the test.
__device__ __forceinline__ bool dt_monotone(float vabs, float a, float b, int K) {
  if (!(a > 0.f) || K > kDtPad - 2 || !(vabs <= 3.0e38f)) return false;
  const float T = (float)(K + 1);
  const float E = 4.0f * 5.9604644775390625e-08f * (vabs + a * T * T + fabsf(b) * T) + 1e-37f;
  return a >= 8.0f * E;
}

// PASS 1: along y (dim 0) of each column x of the negated part map -> tmpM, tmpI.
// PASS 2: along x (dim 1) of each row y of tmpM -> M, Ix, Iy = tmpIy[Ix*d0 + y]
// (dt.cpp:123-133).
// One block per entry of `blocks` (job, first line of its tile): the launch covers
// exactly the tiles of every map, however their sizes differ across levels.
template <int PASS>
__global__ void __launch_bounds__(kDtThreads) k_dt(const DtJob *__restrict__ jobs, const int2 *__restrict__ blocks,
                                                    float *__restrict__ arena, int *__restrict__ arena_i,
                                                    int *fallback_count, int elems) {
  extern __shared__ float dsm[];
  const int2 blk = blocks[blockIdx.x];
  const DtJob J = jobs[blk.x];
  const int d0 = J.d0;
  const int n = PASS == 1 ? J.d0 : J.d1;           // line length
  const int nlines = PASS == 1 ? J.d1 : J.d0;
  const int lgL = PASS == 1 ? 0 : dt_lg_lines2(n, elems);
  const int L = PASS == 1 ? dt_lines1(n, elems) : (1 << lgL);
  const int line0 = blk.y;
  const int nl = min(L, nlines - line0);
  const int stride = n + kDtPad;
  float *v_s = dsm + kDtPad;                       // line l at v_s[l * stride], +inf pads between
  float *o_s = dsm + kDtPad + (size_t)L * stride;  // [L][n]
  int *g_s = reinterpret_cast<int *>(o_s + (size_t)L * n);
  float *At = reinterpret_cast<float *>(g_s + (size_t)L * n) + (kDtPad - 1);   // At[t], |t| < kDtPad
  float *Bt = At + (2 * kDtPad - 1);
  int *K_s = reinterpret_cast<int *>(Bt + kDtPad);
  int *bad_s = K_s + L;
  int *mono_s = bad_s + L;   // every line's argmin certainly non-decreasing
  const float a = PASS == 1 ? J.ay : J.ax, b = PASS == 1 ? J.by : J.bx;
  const int tid = threadIdx.x, nth = blockDim.x;
  const int cnt = nl * n;
  const unsigned magic = 0xFFFFFFFFu / (unsigned)n + 1u;   // e / n for e < 2^32 / n

  // stage the tile (pass 1: with each thread's value range), the pads and the per-offset terms
  float vmin = INFINITY, vmax = -INFINITY, vabs = 0.f;
  bool nan = false;   // fminf/fmaxf skip NaN
  if (PASS == 1) {
    const float *src = arena + J.in_off + (size_t)line0 * n;
    for (int e = tid; e < cnt; e += nth) {
      const int l = __umulhi((unsigned)e, magic), d = e - l * n;
      const float x = J.negate ? -src[e] : src[e];   // inverse_Q (GPU_function.cu:695-794)
      v_s[l * stride + d] = x;
      vmin = fminf(vmin, x); vmax = fmaxf(vmax, x); vabs = fmaxf(vabs, fabsf(x)); nan |= x != x;
    }
  } else {
    const float *tm = arena + J.tmpM_off;
    for (int e = tid; e < (n << lgL); e += nth) {
      const int l = e & (L - 1), x = e >> lgL;
      if (l < nl) {
        v_s[l * stride + x] = tm[(size_t)x * d0 + line0 + l];
      }
    }
  }
  for (int i = tid; i < (nl + 1) * kDtPad; i += nth) {
    const int l = i / kDtPad, k = i - l * kDtPad;
    v_s[l * stride - kDtPad + k] = INFINITY;   // pad before line l (l = nl: after the last line)
  }
  int *kmax_s = mono_s + 1 + 3 * (kDtThreads / 32);   // pass 2: the widest line window of the tile
  if (tid == 0) {
    *mono_s = 1;
    *kmax_s = 0;
  }
  for (int t = tid - (kDtPad - 1); t < kDtPad; t += nth) {
    const float ft = (float)t;
    At[t] = a * ft * ft;
    Bt[t] = b * ft;
  }
  __syncthreads();

  // window bounds.  Pass 1 (many short lines per tile): one bound for the
  // whole tile, from the tile's value range (a wider window than a line's own
  // returns the same leftmost minimum, and the order proof only gets more
  // conservative).  Pass 2 (a few long lines): a bound per line, each line's
  // range reduced by a warp.
  const int lane = tid & 31, warp = tid >> 5;
  int K = 0;
  if (PASS == 1) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      vmin = fminf(vmin, __shfl_xor_sync(0xffffffffu, vmin, o));
      vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
      vabs = fmaxf(vabs, __shfl_xor_sync(0xffffffffu, vabs, o));
    }
    nan = __any_sync(0xffffffffu, nan);
    float *red = reinterpret_cast<float *>(mono_s + 1);   // [3][warps]: the warps' min, max, max |x| (-1: NaN)
    if (lane == 0) {
      red[warp] = vmin;
      red[kDtThreads / 32 + warp] = vmax;
      red[2 * (kDtThreads / 32) + warp] = nan ? -1.0f : vabs;
    }
    __syncthreads();
    float mn = INFINITY, mx = -INFINITY, ab = 0.f;
    bool tile_nan = false;
    for (int w = 0; w < (nth >> 5); w++) {
      mn = fminf(mn, red[w]);
      mx = fmaxf(mx, red[kDtThreads / 32 + w]);
      const float aw = red[2 * (kDtThreads / 32) + w];
      tile_nan |= aw < 0.f;
      ab = fmaxf(ab, aw);
    }
    K = dt_window(mn, mx, ab, a, b, n);
    if (tid == 0 && (tile_nan || !dt_monotone(ab, a, b, K))) *mono_s = 0;
    for (int l = tid; l < nl; l += nth) {
      K_s[l] = K;
      bad_s[l] = 0;
    }
  } else {
    for (int l = warp; l < nl; l += nth >> 5) {
      const float *v = v_s + l * stride;
      float lmin = INFINITY, lmax = -INFINITY, labs = 0.f;
      bool lnan = false;
      for (int i = lane; i < n; i += 32) {
        const float x = v[i];
        lmin = fminf(lmin, x);
        lmax = fmaxf(lmax, x);
        labs = fmaxf(labs, fabsf(x));
        lnan |= x != x;
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        lmin = fminf(lmin, __shfl_xor_sync(0xffffffffu, lmin, o));
        lmax = fmaxf(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
        labs = fmaxf(labs, __shfl_xor_sync(0xffffffffu, labs, o));
      }
      lnan = __any_sync(0xffffffffu, lnan);
      if (lane == 0) {
        const int Kl = dt_window(lmin, lmax, labs, a, b, n);
        K_s[l] = Kl;
        bad_s[l] = 0;
        atomicMax(kmax_s, Kl);
        if (lnan || !dt_monotone(labs, a, b, Kl)) *mono_s = 0;
      }
    }
  }
  __syncthreads();

  // pass 2 computes only the entries it writes when both the score sum's and
  // the part boxes' reads are sampled: one parity class of x per row
  const int q = (PASS == 2 && J.samp_m && J.samp_i) ? 2 : 1;
  if (*mono_s) {
    // the order holds: no check, no replay
    if (PASS == 1 && K <= 8) {   // (pass 2's long lines measured faster with a window per line)
#define DT_MONO(KM)                                                                                       \
  do {                                                                                                    \
    if (q == 1) dt_mono_tile<KM, 1>(v_s, stride, n, nl, a, b, o_s, g_s, line0, J.par_y, J.par_x);          \
    else dt_mono_tile<KM, 2>(v_s, stride, n, nl, a, b, o_s, g_s, line0, J.par_y, J.par_x);                 \
  } while (0)
      if (K <= 3) DT_MONO(3);
      else if (K <= 4) DT_MONO(4);
      else if (K <= 5) DT_MONO(5);
      else if (K <= 6) DT_MONO(6);
      else DT_MONO(8);
#undef DT_MONO
    } else if (PASS == 2 && *kmax_s <= 8) {   // a window per line, the terms in registers
      if (q == 1) dt_scan_tile_reg<1>(v_s, stride, n, nl, a, b, K_s, o_s, g_s, line0, J.par_y, J.par_x);
      else dt_scan_tile_reg<2>(v_s, stride, n, nl, a, b, K_s, o_s, g_s, line0, J.par_y, J.par_x);
    } else {
      dt_scan_tile(v_s, stride, n, nl, a, b, K_s, At, Bt, o_s, g_s, q, line0, J.par_y, J.par_x);
    }
    __syncthreads();   // every output of the tile written before the stores read them
  } else {
    // every output's window, then the order check and the exact replay
    dt_scan_tile(v_s, stride, n, nl, a, b, K_s, At, Bt, o_s, g_s, 1, 0, 0, 0);
    __syncthreads();
    for (int e = tid; e < cnt; e += nth) {
      const int l = __umulhi((unsigned)e, magic), d = e - l * n;
      if (d + 1 < n && g_s[e] > g_s[e + 1]) bad_s[l] = 1;
    }
    __syncthreads();
    for (int l = tid; l < nl; l += nth)
      if (bad_s[l]) {
        dt_replay(v_s + l * stride, n, a, b, o_s + (size_t)l * n, g_s + (size_t)l * n);
        atomicAdd(fallback_count, 1);
      }
    __syncthreads();
  }

  if (PASS == 1) {
    float *tm = arena + J.tmpM_off + (size_t)line0 * n;
    int *ti = arena_i + J.tmpI_off + (size_t)line0 * n;
    for (int e = tid; e < cnt; e += nth) {
      tm[e] = o_s[e];
      ti[e] = g_s[e];
    }
  } else {
    float *M = arena + J.M_off;
    int *Ix = arena_i + J.Ix_off;
    int *Iy = arena_i + J.Iy_off;
    const int *tIy = arena_i + J.tmpI_off;
    for (int e = tid; e < (n << lgL); e += nth) {
      const int l = e & (L - 1), x = e >> lgL;
      if (l >= nl) continue;
      const int y = line0 + l;
      const bool mpos = (y & 1) == J.par_y && (x & 1) == J.par_x;
      const bool ipos = (y & 1) != J.par_y && (x & 1) != J.par_x;
      const bool wm = !J.samp_m || mpos, wi = !J.samp_i || ipos;
      const size_t o = (size_t)x * d0 + y;
      const int ix = g_s[l * n + x];
      if (wm) M[J.cm0 ? (size_t)((x - J.par_x) >> 1) * J.cm0 + ((y - J.par_y) >> 1) : o] = o_s[l * n + x];
      if (wi) {
        const size_t oi = J.ci0 ? (size_t)((x - 1 + J.par_x) >> 1) * J.ci0 + ((y - 1 + J.par_y) >> 1) : o;
        Ix[oi] = ix;
        Iy[oi] = tIy[(size_t)ix * d0 + y];
      }
    }
  }
}

void dt_block_lists(const std::vector<DtJob> &jobs, std::vector<int2> &b1, std::vector<int2> &b2, int elems) {
  b1.clear();
  b2.clear();
  for (size_t j = 0; j < jobs.size(); j++) {
    const DtJob &J = jobs[j];
    const int L1 = dt_lines1(J.d0, elems), L2 = 1 << dt_lg_lines2(J.d1, elems);
    for (int l = 0; l < J.d1; l += L1) b1.push_back(make_int2((int)j, l));
    for (int l = 0; l < J.d0; l += L2) b2.push_back(make_int2((int)j, l));
  }
  // the largest maps' tiles first, so the long blocks start in the first wave
  auto by_size = [&](const int2 &x, const int2 &y) {
    return (long long)jobs[x.x].d0 * jobs[x.x].d1 > (long long)jobs[y.x].d0 * jobs[y.x].d1;
  };
  std::stable_sort(b1.begin(), b1.end(), by_size);
  std::stable_sort(b2.begin(), b2.end(), by_size);
}

void launch_dt(const DtJob *d_jobs, const int2 *d_b1, int n_b1, const int2 *d_b2, int n_b2, int max_d0, int max_d1,
               float *arena, int *arena_i, int *fallback_count, int elems, cudaStream_t s) {
  if (n_b1 <= 0) return;
  size_t smem1 = 0, smem2 = 0;
  for (int n = 1; n <= max_d0; n++) smem1 = std::max(smem1, dt_smem_bytes(dt_lines1(n, elems), n));
  for (int n = 1; n <= max_d1; n++) smem2 = std::max(smem2, dt_smem_bytes(1 << dt_lg_lines2(n, elems), n));
  static SmemAttr a1, a2;
  raise_smem(a1, k_dt<1>, smem1);
  raise_smem(a2, k_dt<2>, smem2);
  k_dt<1><<<n_b1, kDtThreads, smem1, s>>>(d_jobs, d_b1, arena, arena_i, fallback_count, elems);
  k_dt<2><<<n_b2, kDtThreads, smem2, s>>>(d_jobs, d_b2, arena, arena_i, fallback_count, elems);
}

}  // namespace geye
