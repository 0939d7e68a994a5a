// conv_fp32.cu -- root/part filter convolution in FP32 on the CUDA cores.
//
// Arithmetic of CAR_TRACKING/GPU_function.cu:302-358 (process_root) and
// :630-685 (process_part), whose loop is the only statement of the
// reference's fconvsMT arithmetic: for each of the 31 features f,
//   val = sum_{xp} sum_{yp} A[f][x+xp][y+yp] * B[f][xp][yp]   (xp outer)
//   add_val += val
// and the output is 0 + add_val.  With -fmad=false this kernel repeats that
// order exactly, so its maps are bit-identical to the oracle's.
//
// Tiling: a block computes an (8*CR) (y) x 16 (x) output tile for G filters of
// the same size.  Features arrive 8 channels at a time ([pos][32] layout, one
// 32-byte sector per cell) into shared memory; filter slices of the same 8
// channels sit beside them and are read as warp-wide broadcasts.  Each thread
// owns CR consecutive y outputs x G filters.  Neither CR nor G changes any
// output's summation order, so every shape gives the same bits; the shape per
// plan (CR = 4 or 8, groups of up to 8 or 4 filters) is chosen by timing
// (tune_conv_fp32).
#include "internal.h"

namespace geye {

constexpr int kCTX = 16, kCYT = 8;                       // tile columns; threads along y
constexpr int kCThreads = kCYT * kCTX;                   // 128
constexpr int kChunk = 8;                               // channels per shared-memory stage

template <int G, int kCR>
__global__ void __launch_bounds__(kCThreads) k_conv_fp32(const ConvJob *__restrict__ jobs,
                                                         const float *__restrict__ filters,
                                                         const int *__restrict__ filt_off,
                                                         const float *__restrict__ arena_in,
                                                         float *__restrict__ arena_out) {
  constexpr int kCTY = kCYT * kCR;                       // tile rows
  extern __shared__ float sm[];
  const ConvJob J = jobs[blockIdx.y];
  const int tiles = J.tiles_y * J.tiles_x;
  if ((int)blockIdx.x >= tiles) return;
  const int ty0 = (blockIdx.x % J.tiles_y) * kCTY;
  const int tx0 = (blockIdx.x / J.tiles_y) * kCTX;
  const int b0 = J.b0, b1 = J.b1;
  const int RH = kCTY + b0 - 1, RW = kCTX + b1 - 1;
  const int S = RH | 1;                                  // odd column stride: conflict-free reads
  float *A_s = sm;                                       // [kChunk][RW][S]
  float *B_s = sm + kChunk * RW * S;                     // [G][kChunk][b1][b0]
  const int BSQ = b0 * b1;
  const float *feat = arena_in + J.feat_off;

  const int ty = threadIdx.x % kCYT;                     // 0..7
  const int tx = threadIdx.x / kCYT;                     // 0..15
  float add[G][kCR];
#pragma unroll
  for (int g = 0; g < G; g++)
#pragma unroll
    for (int r = 0; r < kCR; r++) add[g][r] = 0.f;

  for (int c0 = 0; c0 < kFeat; c0 += kChunk) {
    const int nc = min(kChunk, kFeat - c0);
    __syncthreads();
    // features: cells of the region, 8 channels each
    for (int i = threadIdx.x; i < RH * RW; i += kCThreads) {
      const int ly = i % RH, lx = i / RH;
      const int y = ty0 + ly, x = tx0 + lx;
      float4 v0 = make_float4(0.f, 0.f, 0.f, 0.f), v1 = v0;
      if (y < J.a0 && x < J.a1) {
        const float4 *p = reinterpret_cast<const float4 *>(feat + ((size_t)x * J.a0 + y) * kFeatPad + c0);
        v0 = p[0];
        v1 = p[1];
      }
      float *d = A_s + lx * S + ly;
      const int CS = RW * S;
      d[0] = v0.x; d[CS] = v0.y; d[2 * CS] = v0.z; d[3 * CS] = v0.w;
      d[4 * CS] = v1.x; d[5 * CS] = v1.y; d[6 * CS] = v1.z; d[7 * CS] = v1.w;
    }
    for (int i = threadIdx.x; i < G * nc * BSQ; i += kCThreads) {
      const int g = i / (nc * BSQ), rem = i % (nc * BSQ);
      float v = 0.f;
      if (g < J.n_filt) v = filters[filt_off[J.filt_base + g] + c0 * BSQ + rem];
      B_s[g * kChunk * BSQ + rem] = v;
    }
    __syncthreads();
    for (int c = 0; c < nc; c++) {
      float val[G][kCR];
#pragma unroll
      for (int g = 0; g < G; g++)
#pragma unroll
        for (int r = 0; r < kCR; r++) val[g][r] = 0.f;
      const float *Ac = A_s + c * RW * S + tx * S + ty * kCR;
      const float *Bc = B_s + c * BSQ;
      for (int xp = 0; xp < b1; xp++) {
        const float *Ax = Ac + xp * S;
        const float *Bx = Bc + xp * b0;
        for (int yp = 0; yp < b0; yp++) {
          float a[kCR];
#pragma unroll
          for (int r = 0; r < kCR; r++) a[r] = Ax[yp + r];
#pragma unroll
          for (int g = 0; g < G; g++) {
            const float b = Bx[g * kChunk * BSQ + yp];
#pragma unroll
            for (int r = 0; r < kCR; r++) val[g][r] += a[r] * b;
          }
        }
      }
#pragma unroll
      for (int g = 0; g < G; g++)
#pragma unroll
        for (int r = 0; r < kCR; r++) add[g][r] += val[g][r];
    }
  }
  const int x = tx0 + tx;
  if (x >= J.c1) return;
  const size_t MSQ = (size_t)J.c0 * J.c1;
#pragma unroll
  for (int g = 0; g < G; g++) {
    if (g >= J.n_filt) break;
    float *out = arena_out + J.out_off + g * MSQ + (size_t)x * J.c0;
#pragma unroll
    for (int r = 0; r < kCR; r++) {
      const int y = ty0 + ty * kCR + r;
      if (y < J.c0) out[y] = 0.0f + add[g][r];
    }
  }
}

static size_t conv_smem(int b0, int b1, int G, int CR) {
  const int RH = kCYT * CR + b0 - 1, RW = kCTX + b1 - 1;
  return sizeof(float) * ((size_t)kChunk * RW * (RH | 1) + (size_t)G * kChunk * b0 * b1);
}

template <int CR>
static void launch_cr(const ConvJob *d_jobs, int n_jobs, dim3 grid, const float *filters, const int *filt_off,
                      const float *arena_in, float *arena_out, int max_b0, int max_b1, int G, cudaStream_t s) {
  const size_t smem = conv_smem(max_b0, max_b1, G, CR);
  switch (G) {
    case 1:
      { static SmemAttr a; raise_smem(a, k_conv_fp32<1, CR>, smem); }
      k_conv_fp32<1, CR><<<grid, kCThreads, smem, s>>>(d_jobs, filters, filt_off, arena_in, arena_out);
      break;
    case 2:
      { static SmemAttr a; raise_smem(a, k_conv_fp32<2, CR>, smem); }
      k_conv_fp32<2, CR><<<grid, kCThreads, smem, s>>>(d_jobs, filters, filt_off, arena_in, arena_out);
      break;
    case 4:
      { static SmemAttr a; raise_smem(a, k_conv_fp32<4, CR>, smem); }
      k_conv_fp32<4, CR><<<grid, kCThreads, smem, s>>>(d_jobs, filters, filt_off, arena_in, arena_out);
      break;
    default:
      { static SmemAttr a; raise_smem(a, k_conv_fp32<8, CR>, smem); }
      k_conv_fp32<8, CR><<<grid, kCThreads, smem, s>>>(d_jobs, filters, filt_off, arena_in, arena_out);
      break;
  }
}

// rows per thread: 4 (tiles of 32 rows) or 8 (64 rows); jobs' tiles_y must be
// ceil(c0 / (8 * cr))
void launch_conv_fp32(const ConvJob *d_jobs, int n_jobs, int max_tiles_y, int max_tiles_x, const float *filters,
                      const int *filt_off, const float *arena_in, float *arena_out, int max_b0, int max_b1,
                      int max_group, cudaStream_t s, int cr) {
  if (n_jobs <= 0) return;
  dim3 grid(max_tiles_y * max_tiles_x, n_jobs);
  const int G = max_group <= 1 ? 1 : max_group <= 2 ? 2 : max_group <= 4 ? 4 : 8;
  if (cr == 8) launch_cr<8>(d_jobs, n_jobs, grid, filters, filt_off, arena_in, arena_out, max_b0, max_b1, G, s);
  else launch_cr<4>(d_jobs, n_jobs, grid, filters, filt_off, arena_in, arena_out, max_b0, max_b1, G, s);
}

}  // namespace geye
