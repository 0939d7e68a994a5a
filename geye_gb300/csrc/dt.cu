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
// reaches the minimum).  So a warp per line computes g(d) for all d in
// parallel, checks that g is non-decreasing, and only if it is not does one
// lane replay the recursion exactly (counted in *fallback_count).
//
// g(d) is searched in a window |d - s| < K.  K is chosen per line so that
// every s outside the window has f_d(s) > max(v) >= f_d(d): with u = 2^-24,
// f_d(s) >= v_min + (1-8u) a t^2 - (1+8u)|b t| - 8u max|v| for a > 0, and K
// is the first integer past the positive root of that bound minus v_max.
// For a <= 0 the window is the whole line.
#include <math.h>

#include "internal.h"

namespace geye {

constexpr int kDtMaxLine = 1100;     // longest line the host lets through (shared-memory bound)
constexpr int kDtWarps = 8;

__device__ __forceinline__ float dt_f(float v, float a, float b, int t) {
  return v + a * t * t + b * t;      // ((v + (a*t)*t) + b*t), each op rounded (no FMA)
}

// window half-width bound K for one line (a > 0); returns n when unbounded
__device__ __forceinline__ int dt_window(float vmin, float vmax, float vabs, float a, float b, int n) {
  if (!(a > 0.f)) return n;
  const double u = 8.0 * 5.9604644775390625e-08;   // 8 * 2^-24
  const double A = (1.0 - u) * (double)a;
  const double B = (1.0 + u) * fabs((double)b);
  const double R = ((double)vmax - (double)vmin) + u * (double)vabs + 1e-30;
  const double root = (B + sqrt(B * B + 4.0 * A * R)) / (2.0 * A);
  if (!(root < (double)n)) return n;
  return (int)floor(root) + 2;
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

// One warp transforms one line held in shared memory v[0..n).
__device__ void dt_line_warp(const float *v, int n, float a, float b, float *out, int *arg, int *gbuf,
                             int *fallback_count) {
  const int lane = threadIdx.x & 31;
  float vmin = INFINITY, vmax = -INFINITY, vabs = 0.f;
  for (int i = lane; i < n; i += 32) {
    float x = v[i];
    vmin = fminf(vmin, x);
    vmax = fmaxf(vmax, x);
    vabs = fmaxf(vabs, fabsf(x));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    vmin = fminf(vmin, __shfl_xor_sync(0xffffffffu, vmin, o));
    vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
    vabs = fmaxf(vabs, __shfl_xor_sync(0xffffffffu, vabs, o));
  }
  const int K = dt_window(vmin, vmax, vabs, a, b, n);
  for (int d = lane; d < n; d += 32) {
    const int lo = max(0, d - K + 1), hi = min(n - 1, d + K - 1);
    int s = lo;
    float best = dt_f(v[lo], a, b, d - lo);
    for (int p = lo + 1; p <= hi; p++) {
      float fp = dt_f(v[p], a, b, d - p);
      if (best > fp) { best = fp; s = p; }
    }
    gbuf[d] = s;
    out[d] = best;
  }
  __syncwarp();
  bool bad = false;
  for (int d = lane; d + 1 < n; d += 32) bad |= gbuf[d] > gbuf[d + 1];
  bad = __any_sync(0xffffffffu, bad);
  if (bad) {
    if (lane == 0) {
      dt_replay(v, n, a, b, out, gbuf);
      atomicAdd(fallback_count, 1);
    }
    __syncwarp();
  }
  for (int d = lane; d < n; d += 32) arg[d] = gbuf[d];
  __syncwarp();
}

// Pass 1: along y (dim 0) for each column x of the negated part map.
__global__ void __launch_bounds__(kDtWarps * 32) k_dt_pass1(const DtJob *__restrict__ jobs, float *__restrict__ arena,
                                                            int *__restrict__ arena_i, int *fallback_count,
                                                            int line_cap) {
  extern __shared__ float sm1[];
  const DtJob J = jobs[blockIdx.y];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float *v_s = sm1 + (size_t)warp * 3 * line_cap;
  float *o_s = v_s + line_cap;
  int *g_s = reinterpret_cast<int *>(o_s + line_cap);
  const int n = J.d0;
  for (int x = blockIdx.x * kDtWarps + warp; x < J.d1; x += gridDim.x * kDtWarps) {
    const float *src = arena + J.in_off + (size_t)x * n;
    for (int i = lane; i < n; i += 32) v_s[i] = J.negate ? -src[i] : src[i];   // inverse_Q (GPU_function.cu:695-794)
    __syncwarp();
    dt_line_warp(v_s, n, J.ay, J.by, o_s, g_s, g_s, fallback_count);
    float *tm = arena + J.tmpM_off + (size_t)x * n;
    int *ti = arena_i + J.tmpI_off + (size_t)x * n;
    for (int i = lane; i < n; i += 32) { tm[i] = o_s[i]; ti[i] = g_s[i]; }
    __syncwarp();
  }
}

// Pass 2: along x (dim 1) for each row y.  A block stages kRows consecutive
// rows (coalesced along y), each warp transforms rows from shared memory, and
// the results go back out coalesced; Iy = tmpIy[Ix*d0 + y] (dt.cpp:123-133).
constexpr int kRows = 16;

__global__ void __launch_bounds__(kDtWarps * 32) k_dt_pass2(const DtJob *__restrict__ jobs, float *__restrict__ arena,
                                                            int *__restrict__ arena_i, int *fallback_count) {
  extern __shared__ float sm2[];
  const DtJob J = jobs[blockIdx.y];
  const int y0 = blockIdx.x * kRows;
  if (y0 >= J.d0) return;
  const int n = J.d1, d0 = J.d0;
  const int rows = min(kRows, d0 - y0);
  float *v_s = sm2;                               // [kRows][n]
  float *o_s = v_s + kRows * n;                   // [kRows][n]
  int *g_s = reinterpret_cast<int *>(o_s + kRows * n);   // [kRows][n]
  const float *tm = arena + J.tmpM_off;
  for (int i = threadIdx.x; i < rows * n; i += blockDim.x) {
    const int r = i % rows, x = i / rows;
    v_s[r * n + x] = tm[(size_t)x * d0 + y0 + r];
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5;
  for (int r = warp; r < rows; r += kDtWarps)
    dt_line_warp(v_s + r * n, n, J.ax, J.bx, o_s + r * n, g_s + r * n, g_s + r * n, fallback_count);
  __syncthreads();
  float *M = arena + J.M_off;
  int *Ix = arena_i + J.Ix_off;
  int *Iy = arena_i + J.Iy_off;
  const int *tIy = arena_i + J.tmpI_off;
  for (int i = threadIdx.x; i < rows * n; i += blockDim.x) {
    const int r = i % rows, x = i / rows;
    const size_t o = (size_t)x * d0 + y0 + r;
    const int ix = g_s[r * n + x];
    M[o] = o_s[r * n + x];
    Ix[o] = ix;
    Iy[o] = tIy[(size_t)ix * d0 + y0 + r];
  }
}

void launch_dt(const DtJob *d_jobs, int n_jobs, int max_d0, int max_d1, float *arena, int *arena_i,
               int *fallback_count, cudaStream_t s) {
  if (n_jobs <= 0) return;
  int gx1 = (max_d1 + kDtWarps - 1) / kDtWarps;
  size_t smem1 = (size_t)kDtWarps * 3 * max_d0 * sizeof(float);
  size_t smem = (size_t)kRows * max_d1 * 3 * sizeof(float);
  static size_t set1 = 0, set = 0;
  if (smem1 > set1) {
    cudaFuncSetAttribute(k_dt_pass1, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem1);
    set1 = smem1;
  }
  k_dt_pass1<<<dim3(gx1, n_jobs), kDtWarps * 32, smem1, s>>>(d_jobs, arena, arena_i, fallback_count, max_d0);
  if (smem > set) {
    cudaFuncSetAttribute(k_dt_pass2, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    set = smem;
  }
  int gx2 = (max_d0 + kRows - 1) / kRows;
  k_dt_pass2<<<dim3(gx2, n_jobs), kDtWarps * 32, smem, s>>>(d_jobs, arena, arena_i, fallback_count);
}

}  // namespace geye
