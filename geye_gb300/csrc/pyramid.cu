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

#include "internal.h"
#include "tc_planes.h"

namespace geye {

// ----------------------------------------------------------------------------
// ingest: u8 BGR rows -> float planes R,G,B column-major [c][w][h]
// 32x32 pixel tile: rows read along x (coalesced bytes), planes written along y.
// ----------------------------------------------------------------------------
__global__ void k_ingest(const uint8_t *__restrict__ bgr, int width, int height, int width_step,
                         float *__restrict__ planes) {
  __shared__ float tile[3][32][33];
  const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 32;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    int y = y0 + r, x = x0 + threadIdx.x;
    if (y < height && x < width) {
      const uint8_t *p = bgr + (size_t)y * width_step + 3 * x;
      tile[0][threadIdx.x][r] = (float)p[2];   // R
      tile[1][threadIdx.x][r] = (float)p[1];   // G
      tile[2][threadIdx.x][r] = (float)p[0];   // B
    }
  }
  __syncthreads();
  const size_t SQ = (size_t)width * height;
  for (int c = threadIdx.y; c < 32; c += blockDim.y) {
    int x = x0 + c, y = y0 + threadIdx.x;
    if (x < width && y < height) {
      size_t o = (size_t)x * height + y;
      planes[o] = tile[0][c][threadIdx.x];
      planes[SQ + o] = tile[1][c][threadIdx.x];
      planes[2 * SQ + o] = tile[2][c][threadIdx.x];
    }
  }
}

void launch_ingest(const uint8_t *bgr, int width, int height, int width_step, float *planes, cudaStream_t s) {
  dim3 grid((width + 31) / 32, (height + 31) / 32), block(32, 8);
  k_ingest<<<grid, block, 0, s>>>(bgr, width, height, width_step, planes);
}

// ----------------------------------------------------------------------------
// resize: one 1-D pass over all jobs of a phase.  Taps for destination index d
// are tap_si/tap_alpha[tap_start[d] .. tap_start[d+1]) in the reference's order.
// vertical: out[c][x][d] = sum alpha * src[c][x][si]     (src h -> dst h, same w)
// horizontal: out[c][d][y] = sum alpha * src[c][si][y]   (src w -> dst w, same h)
// ----------------------------------------------------------------------------
__global__ void k_resize_pass(const ResizeJob *__restrict__ jobs, int vertical, const int *__restrict__ tap_start,
                              const int *__restrict__ tap_si, const float *__restrict__ tap_alpha,
                              float *__restrict__ arena) {
  const ResizeJob J = jobs[blockIdx.y];
  const int n = 3 * J.dst_h * J.dst_w;
  const float *src = arena + J.src_off;
  float *dst = arena + J.dst_off;
  const int *ts = tap_start + J.tap_start_off;
  const int *si = tap_si + J.tap_off;
  const float *al = tap_alpha + J.tap_off;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int y = i % J.dst_h;
    const int rest = i / J.dst_h;
    const int x = rest % J.dst_w;
    const int c = rest / J.dst_w;
    float acc = 0.0f;
    if (vertical) {
      const float *col = src + ((size_t)c * J.src_w + x) * J.src_h;
      for (int t = ts[y]; t < ts[y + 1]; t++) acc += al[t] * col[si[t]];
    } else {
      const float *pl = src + (size_t)c * J.src_w * J.src_h;
      for (int t = ts[x]; t < ts[x + 1]; t++) acc += al[t] * pl[(size_t)si[t] * J.src_h + y];
    }
    dst[i] = acc;
  }
}

void launch_resize_pass(const ResizeJob *d_jobs, int n_jobs, int max_items, int vertical, const int *d_tap_start,
                        const int *d_tap_si, const float *d_tap_alpha, float *arena, cudaStream_t s) {
  if (n_jobs <= 0) return;
  int bx = (max_items + 255) / 256;
  if (bx > 1024) bx = 1024;
  dim3 grid(bx, n_jobs);
  k_resize_pass<<<grid, 256, 0, s>>>(d_jobs, vertical, d_tap_start, d_tap_si, d_tap_alpha, arena);
}

// ----------------------------------------------------------------------------
// HOG
// ----------------------------------------------------------------------------
__constant__ float c_Hcos[9] = {1.0000f, 0.9397f, 0.7660f, 0.5000f, 0.1736f, -0.1736f, -0.5000f, -0.7660f, -0.9397f};
__constant__ float c_Hsin[9] = {0.0000f, 0.3420f, 0.6428f, 0.8660f, 0.9848f, 0.9848f, 0.8660f, 0.6428f, 0.3420f};

constexpr int kTB0 = 16;   // histogram blocks per tile along y
constexpr int kTB1 = 8;    // along x

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

// Histogram + block energy for a tile of kTB0 x kTB1 blocks.  Pixels of the
// tile region get their (bin, magnitude) once into shared memory, and each
// pixel row/column its interpolation cell and weights (the reference's double
// expression, evaluated once per tile row/column instead of per vote); then
// each thread sums its block's votes in the reference's pixel order.
__global__ void __launch_bounds__(kTB0 *kTB1) k_hog_hist(const HogJob *__restrict__ jobs, float *__restrict__ arena) {
  extern __shared__ unsigned char smem_raw[];
  const HogJob J = jobs[blockIdx.z];
  const int by0 = blockIdx.x * kTB0, bx0 = blockIdx.y * kTB1;
  if (by0 >= J.b0 || bx0 >= J.b1) return;
  const int sbin = J.sbin;
  // pixel region covering every vote into blocks [bx0, bx0+kTB1) x [by0, by0+kTB0)
  const int px0 = bx0 * sbin - sbin, py0 = by0 * sbin - sbin;
  const int PW = (kTB1 + 2) * sbin, PH = (kTB0 + 2) * sbin;
  float *mag_s = reinterpret_cast<float *>(smem_raw);
  unsigned char *bin_s = smem_raw + sizeof(float) * PW * PH;
  float *hist_s = reinterpret_cast<float *>(smem_raw + ((sizeof(float) + 1) * PW * PH + 15) / 16 * 16);
  float *wx0_s = hist_s + 18 * kTB0 * kTB1;   // per region column: vx0, vx1, ixp
  float *wx1_s = wx0_s + PW;
  int *ix_s = reinterpret_cast<int *>(wx1_s + PW);
  float *wy0_s = reinterpret_cast<float *>(ix_s + PW);   // per region row
  float *wy1_s = wy0_s + PH;
  int *iy_s = reinterpret_cast<int *>(wy1_s + PH);
  const float *img = arena + J.img_off;
  const int visible0 = J.b0 * sbin, visible1 = J.b1 * sbin;
  const int nthreads = blockDim.x;
  for (int i = threadIdx.x; i < PW * PH; i += nthreads) {
    const int ly = i % PH, lx = i / PH;
    const int x = px0 + lx, y = py0 + ly;
    int bin = 255;
    float mag = 0.f;
    if (x >= 1 && x < visible1 - 1 && y >= 1 && y < visible0 - 1) hog_pixel(img, J.h, J.w, x, y, bin, mag);
    mag_s[i] = mag;
    bin_s[i] = (unsigned char)bin;
  }
  for (int i = threadIdx.x; i < PW + PH; i += nthreads) {
    int ip; float w0, w1;
    if (i < PW) {
      hog_interp(px0 + i, sbin, ip, w0, w1);
      wx0_s[i] = w0; wx1_s[i] = w1; ix_s[i] = ip;
    } else {
      hog_interp(py0 + i - PW, sbin, ip, w0, w1);
      wy0_s[i - PW] = w0; wy1_s[i - PW] = w1; iy_s[i - PW] = ip;
    }
  }
  for (int i = threadIdx.x; i < 18 * nthreads; i += nthreads) hist_s[i] = 0.f;
  __syncthreads();

  const int ty = threadIdx.x % kTB0, tx = threadIdx.x / kTB0;
  const int by = by0 + ty, bx = bx0 + tx;
  const bool active = by < J.b0 && bx < J.b1;
  float *myh = hist_s + threadIdx.x;   // bin o at myh[o * nthreads]
  if (active) {
    // candidate pixel range: any pixel whose interpolation cell is bx-1 or bx
    const int xlo = max(1, bx * sbin - sbin), xhi = min(visible1 - 2, bx * sbin + 2 * sbin - 1);
    const int ylo = max(1, by * sbin - sbin), yhi = min(visible0 - 2, by * sbin + 2 * sbin - 1);
    for (int x = xlo; x <= xhi; x++) {
      const int lx = x - px0;
      const int ixp = ix_s[lx];
      float wx;
      if (ixp == bx) wx = wx1_s[lx]; else if (ixp + 1 == bx) wx = wx0_s[lx]; else continue;
      for (int y = ylo; y <= yhi; y++) {
        const int ly = y - py0;
        const int iyp = iy_s[ly];
        float wy;
        if (iyp == by) wy = wy1_s[ly]; else if (iyp + 1 == by) wy = wy0_s[ly]; else continue;
        const int li = lx * PH + ly;
        const int o = bin_s[li];
        myh[o * nthreads] += wx * wy * mag_s[li];
      }
    }
    const int nb = J.b0 * J.b1;
    const int pos = bx * J.b0 + by;
    float *hist = arena + J.hist_off;
    float norm = 0.f;
#pragma unroll
    for (int o = 0; o < 18; o++) hist[(size_t)o * nb + pos] = myh[o * nthreads];
#pragma unroll
    for (int o = 0; o < 9; o++) {
      float s2 = myh[o * nthreads] + myh[(o + 9) * nthreads];
      norm += s2 * s2;
    }
    hist[(size_t)18 * nb + pos] = norm;
  }
}

// 31 features per output cell (featurepyramid.cpp:421-487), written as 32
// floats [pos][32] (channel 31 = 0), plus an optional copy as the tensor-core
// convolution's channel planes (tc_planes.h).
__global__ void k_hog_feat(const HogJob *__restrict__ jobs, float *__restrict__ arena, uint8_t *__restrict__ arena16) {
  const HogJob J = jobs[blockIdx.y];
  const int ncell = J.fs0 * J.fs1;
  const int b0 = J.b0, nb = J.b0 * J.b1;
  const float *hist = arena + J.hist_off;
  const float *norm = hist + (size_t)18 * nb;
  float *feat = arena + J.feat_off;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ncell; i += gridDim.x * blockDim.x) {
    const int y = i % J.fs0, x = i / J.fs0;
    const float *p;
    float n1, n2, n3, n4;
    p = norm + (x + 1) * b0 + y + 1;
    n1 = 1.0 / sqrt(p[0] + p[1] + p[b0] + p[b0 + 1] + 0.0001);
    p = norm + (x + 1) * b0 + y;
    n2 = 1.0 / sqrt(p[0] + p[1] + p[b0] + p[b0 + 1] + 0.0001);
    p = norm + x * b0 + y + 1;
    n3 = 1.0 / sqrt(p[0] + p[1] + p[b0] + p[b0 + 1] + 0.0001);
    p = norm + x * b0 + y;
    n4 = 1.0 / sqrt(p[0] + p[1] + p[b0] + p[b0 + 1] + 0.0001);
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
    out[27] = (float)(0.2357 * (double)t1);
    out[28] = (float)(0.2357 * (double)t2);
    out[29] = (float)(0.2357 * (double)t3);
    out[30] = (float)(0.2357 * (double)t4);
    out[31] = 0.f;
    float4 *dst = reinterpret_cast<float4 *>(feat + (size_t)i * kFeatPad);
#pragma unroll
    for (int q = 0; q < 8; q++) dst[q] = make_float4(out[4 * q], out[4 * q + 1], out[4 * q + 2], out[4 * q + 3]);
    if (J.feat16_off >= 0 && arena16) {   // planes for the tensor-core convolution
      uint8_t *planes = arena16 + 2 * (size_t)J.feat16_off;
      const size_t plane = ((size_t)ncell + kTcPlanePad) * 16;
      if (J.tc_planes == 4) tc_store_planes<4>(out, planes, plane, i);
      else if (J.tc_planes == 2) tc_store_planes<2>(out, planes, plane, i);
    }
  }
}

void launch_hog(const HogJob *d_jobs, int n_jobs, int max_b0, int max_b1, float *arena, void *arena16,
                cudaStream_t s) {
  if (n_jobs <= 0) return;
  // dynamic shared memory of the widest sbin in the plan (8): 18 bins x 128 threads + pixel tile
  const int sbin_max = 8;
  const int PW = (kTB1 + 2) * sbin_max, PH = (kTB0 + 2) * sbin_max;
  size_t smem = ((sizeof(float) + 1) * PW * PH + 15) / 16 * 16 + sizeof(float) * 18 * kTB0 * kTB1 +
                sizeof(float) * 3 * (PW + PH);
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(k_hog_hist, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr_set = true;
  }
  dim3 g1((max_b0 + kTB0 - 1) / kTB0, (max_b1 + kTB1 - 1) / kTB1, n_jobs);
  k_hog_hist<<<g1, kTB0 * kTB1, smem, s>>>(d_jobs, arena);
  int max_cells = max_b0 * max_b1;
  int bx = (max_cells + 255) / 256;
  if (bx > 512) bx = 512;
  dim3 g2(bx, n_jobs);
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
