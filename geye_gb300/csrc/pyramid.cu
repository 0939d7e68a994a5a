// pyramid.cu -- frame ingest, area resize and HOG features on sm_103a.
//
// All arithmetic repeats the reference's C expressions with the same operand
// types; the library is compiled with -fmad=false so that no a*b+c is fused,
// which makes every value here bit-identical to the reference CPU path:
//   ingest  CAR_TRACKING/featurepyramid.cpp.org:461-500 (Ipl_to_FLOAT)
//   resize  CAR_TRACKING/resize.cc:68-160 (resize1dtran, resize)
//   HOG     CAR_TRACKING/featurepyramid.cpp:263-501 (calc_feature)
// The HOG histogram is computed in gather form: each histogram block sums the
// votes of its pixels in the reference's pixel order (x outer, y inner), so
// the float sums match the reference's sequential scatter exactly without
// atomics.
#include <cuda_bf16.h>

#include <algorithm>

#include "internal.h"
#include "tc_planes.h"

namespace geye {

// ----------------------------------------------------------------------------
// ingest: u8 BGR rows -> float planes R,G,B column-major [c][w][h]
// 32x32 pixel tile: rows read along x (coalesced bytes), planes written along y.
// ----------------------------------------------------------------------------
// one 32x32 tile (x0, y0) by 256 threads (tx = lane, ty = warp)
__device__ __forceinline__ void ingest_tile(const uint8_t *__restrict__ bgr, int width, int height, int width_step,
                                            float *__restrict__ planes, int x0, int y0, int tx, int ty,
                                            float (*tile)[32][33]) {
  for (int r = ty; r < 32; r += 8) {
    int y = y0 + r, x = x0 + tx;
    if (y < height && x < width) {
      const uint8_t *p = bgr + (size_t)y * width_step + 3 * x;
      tile[0][tx][r] = (float)p[2];   // R
      tile[1][tx][r] = (float)p[1];   // G
      tile[2][tx][r] = (float)p[0];   // B
    }
  }
  __syncthreads();
  const size_t SQ = (size_t)width * height;
  for (int c = ty; c < 32; c += 8) {
    int x = x0 + c, y = y0 + tx;
    if (x < width && y < height) {
      size_t o = (size_t)x * height + y;
      planes[o] = tile[0][c][tx];
      planes[SQ + o] = tile[1][c][tx];
      planes[2 * SQ + o] = tile[2][c][tx];
    }
  }
  __syncthreads();   // the tile is free for the next one
}

__global__ void __launch_bounds__(256) k_ingest(const uint8_t *__restrict__ bgr, int width, int height,
                                                int width_step, float *__restrict__ planes) {
  __shared__ float tile[3][32][33];
  ingest_tile(bgr, width, height, width_step, planes, blockIdx.x * 32, blockIdx.y * 32, threadIdx.x & 31,
              threadIdx.x >> 5, tile);
}

void launch_ingest(const uint8_t *bgr, int width, int height, int width_step, float *planes, cudaStream_t s) {
  dim3 grid((width + 31) / 32, (height + 31) / 32);
  k_ingest<<<grid, 256, 0, s>>>(bgr, width, height, width_step, planes);
}

// ----------------------------------------------------------------------------
// resize: one 1-D pass over all jobs of a phase.  Taps for destination index d
// are tap_si/tap_alpha[tap_start[d] .. tap_start[d+1]) in the reference's order.
// vertical: out[c][x][d] = sum alpha * src[c][x][si]     (src h -> dst h, same w)
// horizontal: out[c][d][y] = sum alpha * src[c][si][y]   (src w -> dst w, same h)
// A warp owns one column x of the output (all three channels), lanes along y:
// no index division per element, and each tap is loaded once for the three
// channels (vertical) or once per column (horizontal).
// ----------------------------------------------------------------------------
constexpr int kResizeWarps = 4;

// output column x of one pass (all three channels) by one warp
__device__ __forceinline__ void resize_column(const ResizeJob &J, int vertical, const int *__restrict__ tap_start,
                                              const int *__restrict__ tap_si, const float *__restrict__ tap_alpha,
                                              float *__restrict__ arena, int x) {
  const float *src = arena + J.src_off;
  float *dst = arena + J.dst_off;
  const int *ts = tap_start + J.tap_start_off;
  const int *si = tap_si + J.tap_off;
  const float *al = tap_alpha + J.tap_off;
  const int lane = threadIdx.x & 31;
  const size_t src_plane = (size_t)J.src_w * J.src_h, dst_plane = (size_t)J.dst_w * J.dst_h;
  {
    float *out = dst + (size_t)x * J.dst_h;
    if (vertical) {
      const float *col = src + (size_t)x * J.src_h;
      for (int y = lane; y < J.dst_h; y += 64) {   // two outputs per lane in flight
        const int y2 = y + 32;
        float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, c0 = 0.0f, c1 = 0.0f, c2 = 0.0f;
        const int t1 = ts[y + 1];
        const int u0 = y2 < J.dst_h ? ts[y2] : 0, u1 = y2 < J.dst_h ? ts[y2 + 1] : 0;
#pragma unroll 4
        for (int t = ts[y]; t < t1; t++) {
          const float w = al[t];
          const float *p = col + si[t];
          a0 += w * p[0];
          a1 += w * p[src_plane];
          a2 += w * p[2 * src_plane];
        }
#pragma unroll 4
        for (int t = u0; t < u1; t++) {
          const float w = al[t];
          const float *p = col + si[t];
          c0 += w * p[0];
          c1 += w * p[src_plane];
          c2 += w * p[2 * src_plane];
        }
        out[y] = a0;
        out[dst_plane + y] = a1;
        out[2 * dst_plane + y] = a2;
        if (y2 < J.dst_h) {
          out[y2] = c0;
          out[dst_plane + y2] = c1;
          out[2 * dst_plane + y2] = c2;
        }
      }
    } else {
      // taps are uniform along the column: two outputs per lane in flight
      const int t0 = ts[x], t1 = ts[x + 1];
      for (int y = lane; y < J.dst_h; y += 64) {
        const bool two = y + 32 < J.dst_h;
        float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, b0 = 0.0f, b1 = 0.0f, b2 = 0.0f;
        for (int t = t0; t < t1; t++) {
          const float w = al[t];
          const float *p = src + (size_t)si[t] * J.src_h + y;
          a0 += w * p[0];
          a1 += w * p[src_plane];
          a2 += w * p[2 * src_plane];
          if (two) {
            b0 += w * p[32];
            b1 += w * p[src_plane + 32];
            b2 += w * p[2 * src_plane + 32];
          }
        }
        out[y] = a0;
        out[dst_plane + y] = a1;
        out[2 * dst_plane + y] = a2;
        if (two) {
          out[y + 32] = b0;
          out[dst_plane + y + 32] = b1;
          out[2 * dst_plane + y + 32] = b2;
        }
      }
    }
  }
}

__global__ void __launch_bounds__(kResizeWarps * 32) k_resize_pass(const ResizeJob *__restrict__ jobs, int vertical,
                                                                   const int *__restrict__ tap_start,
                                                                   const int *__restrict__ tap_si,
                                                                   const float *__restrict__ tap_alpha,
                                                                   float *__restrict__ arena) {
  const ResizeJob J = jobs[blockIdx.y];
  for (int x = blockIdx.x * kResizeWarps + (threadIdx.x >> 5); x < J.dst_w; x += gridDim.x * kResizeWarps)
    resize_column(J, vertical, tap_start, tap_si, tap_alpha, arena, x);
}

// max_cols: the largest output column count (dst_w) of the phase's jobs
void launch_resize_pass(const ResizeJob *d_jobs, int n_jobs, int max_cols, int vertical, const int *d_tap_start,
                        const int *d_tap_si, const float *d_tap_alpha, float *arena, cudaStream_t s) {
  if (n_jobs <= 0) return;
  int bx = (max_cols + kResizeWarps - 1) / kResizeWarps;
  if (bx > 1024) bx = 1024;
  dim3 grid(bx, n_jobs);
  k_resize_pass<<<grid, kResizeWarps * 32, 0, s>>>(d_jobs, vertical, d_tap_start, d_tap_si, d_tap_alpha, arena);
}

// ----------------------------------------------------------------------------
// HOG
// ----------------------------------------------------------------------------
__constant__ float c_Hcos[9] = {1.0000f, 0.9397f, 0.7660f, 0.5000f, 0.1736f, -0.1736f, -0.5000f, -0.7660f, -0.9397f};
__constant__ float c_Hsin[9] = {0.0000f, 0.3420f, 0.6428f, 0.8660f, 0.9848f, 0.9848f, 0.8660f, 0.6428f, 0.3420f};

// strongest-channel gradient, orientation snap (featurepyramid.cpp:310-362)
__device__ __forceinline__ void hog_pixel(const float *__restrict__ img, int h, int w, int x, int y, int &bin,
                                          float &mag) {
  const size_t SQ = (size_t)w * h;
  const float *s = img + (size_t)min(x, w - 2) * h + min(y, h - 2);
  float dy = s[1] - s[-1];
  float dx = s[h] - s[-h];
  float v = dx * dx + dy * dy;
  s += SQ;
  float dy2 = s[1] - s[-1];
  float dx2 = s[h] - s[-h];
  float v2 = dx2 * dx2 + dy2 * dy2;
  s += SQ;
  float dy3 = s[1] - s[-1];
  float dx3 = s[h] - s[-h];
  float v3 = dx3 * dx3 + dy3 * dy3;
  if (v2 > v) { v = v2; dx = dx2; dy = dy2; }
  if (v3 > v) { v = v3; dx = dx3; dy = dy3; }
  float best_dot = 0;
  int best_o = 0;
#pragma unroll
  for (int o = 0; o < 9; o++) {
    float dot = c_Hcos[o] * dx + c_Hsin[o] * dy;
    if (dot > best_dot) { best_dot = dot; best_o = o; }
    else if (-dot > best_dot) { best_dot = -dot; best_o = o + 9; }
  }
  bin = best_o;
  mag = sqrtf(v);   // sqrt in double rounded to float == correctly rounded sqrtf
}

// interpolation position of pixel coordinate p (featurepyramid.cpp:365-372)
__device__ __forceinline__ void hog_interp(int p, int sbin, int &ip, float &w0, float &w1) {
  float pp = ((float)p + 0.5) / (float)sbin - 0.5;
  ip = (int)floor(pp);
  w0 = pp - ip;
  w1 = 1.0 - w0;
}

// interpolation position for a power-of-two sbin: (p + 0.5) / sbin - 0.5 and
// everything after it are exact in float, so this equals hog_interp's double form
__device__ __forceinline__ void hog_interp_pow2(int p, float inv_sbin, int &ip, float &w0, float &w1) {
  const float pp = ((float)p + 0.5f) * inv_sbin - 0.5f;
  ip = (int)floorf(pp);
  w0 = pp - (float)ip;
  w1 = 1.0f - w0;
}

// Pass 1: (orientation bin, magnitude) of every pixel that votes, once per
// image (the levels of the first octave share their images with the levels
// an octave up, at half the bin size).  A warp owns a pixel column x, lanes
// run along y; out [x * Y + y] for 1 <= x < xe, 1 <= y < ye.
constexpr int kPixWarps = 8;

__device__ __forceinline__ void hog_pix_column(const HogPixJob &J, float *__restrict__ arena, int x) {
  const float *img = arena + J.img_off;
  float *mag = arena + J.mag_off;
  uint8_t *bin = reinterpret_cast<uint8_t *>(arena + J.bin_off);
  const int lane = threadIdx.x & 31;
  {
    for (int y = 1 + lane; y < J.ye; y += 64) {   // two pixels per lane in flight
      const int y2 = y + 32;
      int b, b2 = 0;
      float m, m2 = 0.f;
      hog_pixel(img, J.h, J.w, x, y, b, m);
      if (y2 < J.ye) hog_pixel(img, J.h, J.w, x, y2, b2, m2);
      mag[(size_t)x * J.Y + y] = m;
      bin[(size_t)x * J.Y + y] = (uint8_t)b;
      if (y2 < J.ye) {
        mag[(size_t)x * J.Y + y2] = m2;
        bin[(size_t)x * J.Y + y2] = (uint8_t)b2;
      }
    }
  }
}

__global__ void __launch_bounds__(kPixWarps * 32) k_hog_pix(const HogPixJob *__restrict__ jobs,
                                                           float *__restrict__ arena) {
  const HogPixJob J = jobs[blockIdx.y];
  for (int x = 1 + blockIdx.x * kPixWarps + (threadIdx.x >> 5); x < J.xe; x += gridDim.x * kPixWarps)
    hog_pix_column(J, arena, x);
}

// Pass 2: one thread per histogram block sums its votes in the reference's
// pixel order (x outer, y inner; featurepyramid.cpp:365-416), into 18 bins
// held in shared memory ([bin][thread], conflict-free), then writes the bins
// and the block energy.  A block's votes come from pixels whose interpolation
// cell is (bx-1 or bx, by-1 or by): for a power-of-two sbin these are the
// column range [bx*sbin - sbin/2, bx*sbin + 3*sbin/2), the first half with
// weight w0 and the second with w1 (same for rows); otherwise the range is
// widened by a pixel each side and each pixel's cell is tested.
constexpr int kVoteThreads = 256;

// the vote loop for a compile-time power-of-two sbin: the 2*SB row weights of
// the block are formed once and the row loop is unrolled
template <int SB>
__device__ __forceinline__ void hog_vote_pow2(float *myh, const float *__restrict__ mag,
                                              const uint8_t *__restrict__ bin, size_t Y, int bx, int by,
                                              int visible0, int visible1) {
  const float inv = 1.0f / (float)SB;
  const int xm = bx * SB + SB / 2, ym = by * SB + SB / 2;
  const int xa = max(1, xm - SB), xb = min(visible1 - 1, xm + SB);
  const int y0 = ym - SB;
  const int ya = max(1, y0), yb = min(visible0 - 1, ym + SB);
  float wy[2 * SB];
#pragma unroll
  for (int k = 0; k < 2 * SB; k++) {
    int iyp;
    float w0, w1;
    hog_interp_pow2(y0 + k, inv, iyp, w0, w1);
    wy[k] = k < SB ? w0 : w1;
  }
  for (int x = xa; x < xb; x++) {
    int ixp;
    float wx0, wx1;
    hog_interp_pow2(x, inv, ixp, wx0, wx1);
    const float wx = x < xm ? wx0 : wx1;
    const float *mcol = mag + (size_t)x * Y + y0;
    const uint8_t *bcol = bin + (size_t)x * Y + y0;
#pragma unroll
    for (int k = 0; k < 2 * SB; k++) {
      const int y = y0 + k;
      if (y >= ya && y < yb) myh[bcol[k] * kVoteThreads] += wx * wy[k] * mcol[k];
    }
  }
}

// One CUDA block per entry of `blocks` (job, block of kVoteThreads histogram
// blocks): exactly the blocks every level needs.
// histogram block pos of one level by one thread (hist_s: the block's [18][kVoteThreads] bins)
__device__ __forceinline__ void hog_vote_one(const HogJob &J, float *__restrict__ arena, int pos, float *hist_s) {
  const int nb = J.b0 * J.b1;
  float *myh = hist_s + threadIdx.x;   // bin o at myh[o * kVoteThreads]
#pragma unroll
  for (int o = 0; o < 18; o++) myh[o * kVoteThreads] = 0.f;
  if (pos >= nb) return;
  const int bx = pos / J.b0, by = pos - bx * J.b0;
  const int sbin = J.sbin;
  const int visible0 = J.b0 * sbin, visible1 = J.b1 * sbin;
  const float *mag = arena + J.mag_off;
  const uint8_t *bin = reinterpret_cast<const uint8_t *>(arena + J.bin_off);
  const size_t Y = J.pix_Y;
  if (sbin == 8) {
    hog_vote_pow2<8>(myh, mag, bin, Y, bx, by, visible0, visible1);
  } else if (sbin == 4) {
    hog_vote_pow2<4>(myh, mag, bin, Y, bx, by, visible0, visible1);
  } else if ((sbin & (sbin - 1)) == 0) {
    const float inv = 1.0f / (float)sbin;
    const int xm = bx * sbin + sbin / 2, ym = by * sbin + sbin / 2;   // first pixel of cell bx / by
    const int xa = max(1, xm - sbin), xb = min(visible1 - 1, xm + sbin);
    const int ya = max(1, ym - sbin), yb = min(visible0 - 1, ym + sbin);
    for (int x = xa; x < xb; x++) {
      int ixp;
      float wx0, wx1;
      hog_interp_pow2(x, inv, ixp, wx0, wx1);
      const float wx = x < xm ? wx0 : wx1;   // cell bx is ixp + 1 in the first half, ixp in the second
      const float *mcol = mag + (size_t)x * Y;
      const uint8_t *bcol = bin + (size_t)x * Y;
      for (int y = ya; y < yb; y++) {
        int iyp;
        float wy0, wy1;
        hog_interp_pow2(y, inv, iyp, wy0, wy1);
        const float wy = y < ym ? wy0 : wy1;
        myh[bcol[y] * kVoteThreads] += wx * wy * mcol[y];
      }
    }
  } else {
    const int xlo = max(1, bx * sbin - sbin / 2 - 2), xhi = min(visible1 - 2, bx * sbin + (3 * sbin) / 2 + 1);
    const int ylo = max(1, by * sbin - sbin / 2 - 2), yhi = min(visible0 - 2, by * sbin + (3 * sbin) / 2 + 1);
    for (int x = xlo; x <= xhi; x++) {
      int ixp;
      float wx0, wx1, wx;
      hog_interp(x, sbin, ixp, wx0, wx1);
      if (ixp == bx) wx = wx1; else if (ixp + 1 == bx) wx = wx0; else continue;
      for (int y = ylo; y <= yhi; y++) {
        int iyp;
        float wy0, wy1, wy;
        hog_interp(y, sbin, iyp, wy0, wy1);
        if (iyp == by) wy = wy1; else if (iyp + 1 == by) wy = wy0; else continue;
        myh[bin[(size_t)x * Y + y] * kVoteThreads] += wx * wy * mag[(size_t)x * Y + y];
      }
    }
  }
  float *hist = arena + J.hist_off;
  float norm = 0.f;
#pragma unroll
  for (int o = 0; o < 18; o++) hist[(size_t)o * nb + pos] = myh[o * kVoteThreads];
#pragma unroll
  for (int o = 0; o < 9; o++) {
    float s2 = myh[o * kVoteThreads] + myh[(o + 9) * kVoteThreads];
    norm += s2 * s2;
  }
  hist[(size_t)18 * nb + pos] = norm;
}

__global__ void __launch_bounds__(kVoteThreads, 4) k_hog_vote(const HogJob *__restrict__ jobs,
                                                             const int2 *__restrict__ blocks,
                                                             float *__restrict__ arena) {
  __shared__ float hist_s[18 * kVoteThreads];
  const int2 blk = blocks[blockIdx.x];
  hog_vote_one(jobs[blk.x], arena, blk.y * kVoteThreads + threadIdx.x, hist_s);
}

// 31 features per output cell (featurepyramid.cpp:421-487), written as 32
// floats [pos][32] (channel 31 = 0), plus an optional copy as the tensor-core
// convolution's channel planes (tc_planes.h).
// Normalisation factor of every corner of 2x2 histogram blocks,
// 1 / sqrt(e(x,y) + e(x,y+1) + e(x+1,y) + e(x+1,y+1) + 0.0001) in the reference's
// expression (float sum, double root and division, rounded to float), once per
// corner: each is shared by the four output cells around it.
__device__ __forceinline__ int hog_corners(const HogJob &J) { return (J.fs0 + 1) * (J.fs1 + 1); }

__device__ __forceinline__ void hog_norm_one(const HogJob &J, float *__restrict__ arena, int i) {
  const int C0 = J.fs0 + 1;
  const int b0 = J.b0, nb = J.b0 * J.b1;
  const float *norm = arena + J.hist_off + (size_t)18 * nb;
  float *N = arena + J.corner_off;
  const int y = i % C0, x = i / C0;
  const float *p = norm + x * b0 + y;
  N[i] = 1.0 / sqrt(p[0] + p[1] + p[b0] + p[b0 + 1] + 0.0001);
}

__global__ void k_hog_norm(const HogJob *__restrict__ jobs, float *__restrict__ arena) {
  const HogJob J = jobs[blockIdx.y];
  const int nc = hog_corners(J);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += gridDim.x * blockDim.x) hog_norm_one(J, arena, i);
}

// output cell i of one level
__device__ __forceinline__ void hog_feat_one(const HogJob &J, float *__restrict__ arena,
                                             uint8_t *__restrict__ arena16, int i) {
  const int ncell = J.fs0 * J.fs1;
  const int b0 = J.b0, nb = J.b0 * J.b1;
  const float *hist = arena + J.hist_off;
  const float *N = arena + J.corner_off;
  const int C0 = J.fs0 + 1;
  float *feat = arena + J.feat_off;
  {
    const int y = i % J.fs0, x = i / J.fs0;
    float n1, n2, n3, n4;
    if (J.fast) {
      // the tensor-core modes: the four corner factors in float here (no FP64, no corner pass)
      const float *e = hist + (size_t)18 * nb;
      auto corner = [&](int cx, int cy) {
        const float *p = e + cx * b0 + cy;
        return 1.0f / sqrtf(p[0] + p[1] + p[b0] + p[b0 + 1] + 0.0001f);
      };
      n1 = corner(x + 1, y + 1);
      n2 = corner(x + 1, y);
      n3 = corner(x, y + 1);
      n4 = corner(x, y);
    } else {
      n1 = N[(x + 1) * C0 + y + 1];
      n2 = N[(x + 1) * C0 + y];
      n3 = N[x * C0 + y + 1];
      n4 = N[x * C0 + y];
    }
    const float *src = hist + (x + 1) * b0 + (y + 1);
    float out[32];
    float t1 = 0, t2 = 0, t3 = 0, t4 = 0;
#pragma unroll
    for (int o = 0; o < 18; o++) {
      const float hv = src[(size_t)o * nb];
      // min_2(v) = v <= 0.2 (double) ? v : (float)0.2  ==  v < 0.2f ? v : 0.2f
      float a = hv * n1, b = hv * n2, c = hv * n3, d = hv * n4;
      float h1 = a < 0.2f ? a : 0.2f;
      float h2 = b < 0.2f ? b : 0.2f;
      float h3 = c < 0.2f ? c : 0.2f;
      float h4 = d < 0.2f ? d : 0.2f;
      out[o] = 0.5f * (h1 + h2 + h3 + h4);
      t1 += h1; t2 += h2; t3 += h3; t4 += h4;
    }
#pragma unroll
    for (int o = 0; o < 9; o++) {
      float sum = src[(size_t)o * nb] + src[(size_t)(o + 9) * nb];
      float a = sum * n1, b = sum * n2, c = sum * n3, d = sum * n4;
      float h1 = a < 0.2f ? a : 0.2f;
      float h2 = b < 0.2f ? b : 0.2f;
      float h3 = c < 0.2f ? c : 0.2f;
      float h4 = d < 0.2f ? d : 0.2f;
      out[18 + o] = 0.5f * (h1 + h2 + h3 + h4);
    }
    if (J.fast) {
      out[27] = 0.2357f * t1;
      out[28] = 0.2357f * t2;
      out[29] = 0.2357f * t3;
      out[30] = 0.2357f * t4;
    } else {   // the reference's double product, rounded once
      out[27] = (float)(0.2357 * (double)t1);
      out[28] = (float)(0.2357 * (double)t2);
      out[29] = (float)(0.2357 * (double)t3);
      out[30] = (float)(0.2357 * (double)t4);
    }
    out[31] = 0.f;
    float4 *dst = reinterpret_cast<float4 *>(feat + (size_t)i * kFeatPad);
#pragma unroll
    for (int q = 0; q < 8; q++) dst[q] = make_float4(out[4 * q], out[4 * q + 1], out[4 * q + 2], out[4 * q + 3]);
    if (J.feat16_off >= 0 && arena16) {   // planes for the tensor-core convolution
      uint8_t *planes = arena16 + 2 * (size_t)J.feat16_off;
      const size_t plane = ((size_t)ncell + kTcPlanePad) * 16;
      if (J.tc_planes == 4) tc_store_planes<4>(out, planes, plane, i);
      else if (J.tc_planes == 2) tc_store_planes<2>(out, planes, plane, i);
      if (J.feat16lo_off >= 0) tc_store_planes_lo(out, arena16 + 2 * (size_t)J.feat16lo_off, plane, i);
    }
  }
}

__global__ void k_hog_feat(const HogJob *__restrict__ jobs, float *__restrict__ arena, uint8_t *__restrict__ arena16) {
  const HogJob J = jobs[blockIdx.y];
  const int ncell = J.fs0 * J.fs1;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ncell; i += gridDim.x * blockDim.x)
    hog_feat_one(J, arena, arena16, i);
}

// ----------------------------------------------------------------------------
// batched front end: persistent CTAs over a stage's (frame, job, chunk) items
// ----------------------------------------------------------------------------
template <int STAGE>
__global__ void __launch_bounds__(256) k_batch_front(const BatchFrame *__restrict__ frames,
                                                     const BatchItem *__restrict__ items, int n, int phase) {
  __shared__ float sm[18 * kVoteThreads];   // a vote block's bins, or an ingest tile ([3][32][33] floats)
  const int tid = threadIdx.x, warp = tid >> 5;
  for (int it = blockIdx.x; it < n; it += gridDim.x) {
    const BatchItem I = items[it];
    const BatchFrame &F = frames[I.frame];
    if (STAGE == kBatchIngest) {
      ingest_tile(F.bgr, F.width, F.height, F.width_step, F.arena + F.img0_off, 32 * I.job, 32 * I.chunk, tid & 31,
                  warp, reinterpret_cast<float (*)[32][33]>(sm));
    } else if (STAGE == kBatchResizeV || STAGE == kBatchResizeH) {
      const ResizeJob J = (STAGE == kBatchResizeV ? F.vjobs[phase] : F.hjobs[phase])[I.job];
      const int x = I.chunk * kBatchColumns + warp;
      if (x < J.dst_w) resize_column(J, STAGE == kBatchResizeV, F.tap_start, F.tap_si, F.tap_alpha, F.arena, x);
    } else if (STAGE == kBatchPix) {
      const HogPixJob J = F.pix[I.job];
      const int x = 1 + I.chunk * kBatchColumns + warp;
      if (x < J.xe) hog_pix_column(J, F.arena, x);
    } else if (STAGE == kBatchVote) {
      const int2 blk = F.vote_blocks[I.job];
      hog_vote_one(F.hog[blk.x], F.arena, blk.y * kVoteThreads + tid, sm);
    } else if (STAGE == kBatchNorm) {
      const HogJob J = F.hog[I.job];
      const int i = I.chunk * kBatchCells + tid;
      if (i < hog_corners(J)) hog_norm_one(J, F.arena, i);
    } else {
      const HogJob J = F.hog[I.job];
      const int i = I.chunk * kBatchCells + tid;
      if (i < J.fs0 * J.fs1) hog_feat_one(J, F.arena, F.arena16, i);
    }
  }
}

void launch_batch_front(int stage, const BatchFrame *d_frames, const BatchItem *d_items, int n, int phase,
                        cudaStream_t s) {
  if (n <= 0) return;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int grid = std::max(1, std::min(n, 4 * std::max(sms, 1)));   // persistent: a few CTAs per SM
  switch (stage) {
    case kBatchIngest: k_batch_front<kBatchIngest><<<grid, 256, 0, s>>>(d_frames, d_items, n, phase); break;
    case kBatchResizeV: k_batch_front<kBatchResizeV><<<grid, 256, 0, s>>>(d_frames, d_items, n, phase); break;
    case kBatchResizeH: k_batch_front<kBatchResizeH><<<grid, 256, 0, s>>>(d_frames, d_items, n, phase); break;
    case kBatchPix: k_batch_front<kBatchPix><<<grid, 256, 0, s>>>(d_frames, d_items, n, phase); break;
    case kBatchVote: k_batch_front<kBatchVote><<<grid, 256, 0, s>>>(d_frames, d_items, n, phase); break;
    case kBatchNorm: k_batch_front<kBatchNorm><<<grid, 256, 0, s>>>(d_frames, d_items, n, phase); break;
    default: k_batch_front<kBatchFeat><<<grid, 256, 0, s>>>(d_frames, d_items, n, phase); break;
  }
}

void hog_vote_blocks(const std::vector<HogJob> &jobs, std::vector<int2> &blocks) {
  blocks.clear();
  for (size_t j = 0; j < jobs.size(); j++)
    for (int b = 0; b * kVoteThreads < jobs[j].b0 * jobs[j].b1; b++) blocks.push_back(make_int2((int)j, b));
}

void launch_hog(const HogJob *d_jobs, int n_jobs, const int2 *d_vote_blocks, int n_vote_blocks, int max_b0,
                int max_b1, const HogPixJob *d_pix, int n_pix, int max_xe, float *arena, void *arena16,
                bool corners, cudaStream_t s) {
  if (n_jobs <= 0) return;
  dim3 g0((max_xe + kPixWarps - 1) / kPixWarps, n_pix);
  k_hog_pix<<<g0, kPixWarps * 32, 0, s>>>(d_pix, arena);
  k_hog_vote<<<n_vote_blocks, kVoteThreads, 0, s>>>(d_jobs, d_vote_blocks, arena);
  const int max_cells = max_b0 * max_b1;
  int bx = (max_cells + 255) / 256;
  if (bx > 512) bx = 512;
  dim3 g2(bx, n_jobs);
  if (corners) k_hog_norm<<<g2, 256, 0, s>>>(d_jobs, arena);
  k_hog_feat<<<g2, 256, 0, s>>>(d_jobs, arena, reinterpret_cast<uint8_t *>(arena16));
}

// ----------------------------------------------------------------------------
// layout conversion between the device feature layout [pos][32] and the
// reference layout [31][fs1][fs0] (stage entry points only)
// ----------------------------------------------------------------------------
__global__ void k_to_ref(const float *__restrict__ feat, int ncell, float *__restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ncell * kFeat; i += gridDim.x * blockDim.x) {
    const int f = i / ncell, pos = i % ncell;
    out[i] = feat[(size_t)pos * kFeatPad + f];
  }
}

__global__ void k_from_ref(const float *__restrict__ ref, int ncell, float *__restrict__ feat) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ncell * kFeatPad; i += gridDim.x * blockDim.x) {
    const int pos = i / kFeatPad, f = i % kFeatPad;
    feat[i] = f < kFeat ? ref[(size_t)f * ncell + pos] : 0.f;
  }
}

// flip_feat (get_boxes.cpp:121-178): output channel c, column x is source
// channel ord[c] - 1, column n1 - 1 - x (a mirror along dim 1 with the signed
// orientations reversed); a thread per output element, rows contiguous.
__constant__ int c_flip_ord[kFeat] = {10, 9,  8,  7,  6,  5,  4,  3,  2,  1,  18, 17, 16, 15, 14, 13,
                                      12, 11, 19, 27, 26, 25, 24, 23, 22, 21, 20, 30, 31, 28, 29};

__global__ void k_flip_feat(const float *__restrict__ feat, int n0, int n1, float *__restrict__ out) {
  const size_t plane = (size_t)n0 * n1, total = plane * kFeat;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(i / plane);
    const size_t r = i - (size_t)c * plane;
    const int x = (int)(r / n0), y = (int)(r - (size_t)x * n0);
    out[i] = feat[(size_t)(c_flip_ord[c] - 1) * plane + (size_t)(n1 - 1 - x) * n0 + y];
  }
}

void launch_flip_feat(const float *feat, int n0, int n1, float *out, cudaStream_t s) {
  const size_t total = (size_t)n0 * n1 * kFeat;
  const int blocks = (int)std::min<size_t>((total + 255) / 256, 4096);
  k_flip_feat<<<blocks, 256, 0, s>>>(feat, n0, n1, out);
}

void launch_to_ref_layout(const float *feat, int fs0, int fs1, float *out, cudaStream_t s) {
  int n = fs0 * fs1 * kFeat;
  if (n <= 0) return;
  k_to_ref<<<(n + 255) / 256 < 2048 ? (n + 255) / 256 : 2048, 256, 0, s>>>(feat, fs0 * fs1, out);
}

void launch_from_ref_layout(const float *ref, int fs0, int fs1, float *feat, cudaStream_t s) {
  int n = fs0 * fs1 * kFeatPad;
  if (n <= 0) return;
  k_from_ref<<<(n + 255) / 256 < 2048 ? (n + 255) / 256 : 2048, 256, 0, s>>>(ref, fs0 * fs1, feat);
}

}  // namespace geye
