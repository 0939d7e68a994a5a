// tc_planes.h -- the tensor-core convolution's feature planes (conv_tc.cu):
// NQ planes of 16 bytes per position, four of 8 bf16 channels or two of 16
// e4m3 channels (features times kFp8FeatScale, saturated to e4m3's range).
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp8.h>
#include <stdint.h>

#include "internal.h"

namespace geye {

constexpr float kFp8FeatScale = 256.0f;   // HOG features (<= ~1) times this stay under e4m3's 448

// writes position i's 32 channels (f[31] = 0) into the NQ planes (plane_bytes apart)
template <int NQ>
__device__ __forceinline__ void tc_store_planes(const float *f, uint8_t *planes, size_t plane_bytes, size_t i) {
  if constexpr (NQ == 4) {
#pragma unroll
    for (int q = 0; q < 4; q++) {
      __nv_bfloat162 v[4];
#pragma unroll
      for (int k = 0; k < 4; k++) v[k] = __floats2bfloat162_rn(f[8 * q + 2 * k], f[8 * q + 2 * k + 1]);
      *reinterpret_cast<uint4 *>(planes + q * plane_bytes + i * 16) = *reinterpret_cast<uint4 *>(v);
    }
  } else {
#pragma unroll
    for (int q = 0; q < 2; q++) {
      __nv_fp8x2_storage_t v[8];
#pragma unroll
      for (int k = 0; k < 8; k++)
        v[k] = __nv_cvt_float2_to_fp8x2(make_float2(f[16 * q + 2 * k] * kFp8FeatScale,
                                                    f[16 * q + 2 * k + 1] * kFp8FeatScale),
                                        __NV_SATFINITE, __NV_E4M3);
      *reinterpret_cast<uint4 *>(planes + q * plane_bytes + i * 16) = *reinterpret_cast<uint4 *>(v);
    }
  }
}

// the BF16 remainders of position i's channels, f - bf16(f), rounded to BF16
// (four planes like tc_store_planes<4>): with the high planes, a split operand
// whose two BF16 parts carry about 16 significant bits
__device__ __forceinline__ void tc_store_planes_lo(const float *f, uint8_t *planes, size_t plane_bytes, size_t i) {
#pragma unroll
  for (int q = 0; q < 4; q++) {
    __nv_bfloat162 v[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const float a = f[8 * q + 2 * k], b = f[8 * q + 2 * k + 1];
      v[k] = __floats2bfloat162_rn(a - __bfloat162float(__float2bfloat16_rn(a)),
                                   b - __bfloat162float(__float2bfloat16_rn(b)));
    }
    *reinterpret_cast<uint4 *>(planes + q * plane_bytes + i * 16) = *reinterpret_cast<uint4 *>(v);
  }
}

}  // namespace geye
