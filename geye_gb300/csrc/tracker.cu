// tracker.cu -- one frame of a stream's particle-filter tracker (model in tracker.h).
//
//   k_track_assoc (one block): gathers the frame's kept boxes of every model,
//     IoU of each live track's estimate with each detection, greedy
//     assignment in track order (highest IoU >= kAssocIoU, lowest index on
//     ties), new tracks for detections left over, ends tracks missed too long.
//   k_track_update (a block per track, a thread per particle): predict with
//     Philox-driven Gaussian noise; weight each particle, as the reference's
//     calc_part_likelihood does (tracking.cpp:403-452: confidence = A_SCORE at
//     the particle + an image likelihood), by the frame's A_SCORE at its
//     centre (the largest over the models, 0 outside the image) plus
//     exp(-|corners - detection corners|^2 / (2 kLikeScale^2)) for an assigned
//     detection (1 without one); estimate as the weighted mean and, with a
//     detection, resample systematically; a new track starts its particles
//     around its detection.
#include <math.h>
#include <string.h>

#include "tracker.h"

namespace geye {

__device__ __forceinline__ float box_iou(const float *a, const float *b) {
  const float w = fminf(a[2], b[2]) - fmaxf(a[0], b[0]);
  const float h = fminf(a[3], b[3]) - fmaxf(a[1], b[1]);
  if (w <= 0.f || h <= 0.f) return 0.f;
  const float inter = w * h;
  const float ua = (a[2] - a[0]) * (a[3] - a[1]) + (b[2] - b[0]) * (b[3] - b[1]) - inter;
  return ua > 0.f ? inter / ua : 0.f;
}

__global__ void __launch_bounds__(256) k_track_assoc(TrackState *S, const int *__restrict__ res, int max_cap,
                                                     const int *__restrict__ kept, int n_models) {
  __shared__ float iou_m[kTracks][kMaxDet];
  __shared__ float dets[kMaxDet][4];
  __shared__ int taken[kMaxDet];
  __shared__ int base[9];
  __shared__ int nd;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nm = min(n_models, 8);
  if (threadIdx.x == 0) {
    int n = 0;
    for (int m = 0; m < nm; m++) {
      base[m] = n;
      n += max(0, min(kept[m], max_cap));
    }
    base[nm] = n;
    nd = min(n, kMaxDet);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nd; i += blockDim.x) {
    int m = 0;
    while (m + 1 < nm && base[m + 1] <= i) m++;
    const int *pt = res + (size_t)m * max_cap * 11 + 4 * (size_t)(i - base[m]);
    for (int c = 0; c < 4; c++) {
      dets[i][c] = (float)pt[c];
      S->det[i][c] = (float)pt[c];
    }
    taken[i] = 0;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < kTracks * nd; e += blockDim.x) {
    const int t = e / nd, d = e % nd;
    iou_m[t][d] = S->alive[t] ? box_iou(S->est[t], dets[d]) : -1.f;
  }
  __syncthreads();
  if (warp == 0) {
    for (int t = 0; t < kTracks; t++) {
      const int alive = S->alive[t];
      if (!alive) {
        if (lane == 0) { S->assign[t] = -1; S->init[t] = 0; }
        __syncwarp();
        continue;
      }
      float bv = -1.f;
      int bi = -1;
      for (int d = lane; d < nd; d += 32) {
        const float v = iou_m[t][d];
        if (!taken[d] && v >= kAssocIoU && v > bv) { bv = v; bi = d; }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov > bv || (ov == bv && oi >= 0 && (bi < 0 || oi < bi))) { bv = ov; bi = oi; }
      }
      if (lane == 0) {
        S->assign[t] = bi;
        S->init[t] = 0;
        S->age[t]++;
        if (bi >= 0) {
          taken[bi] = 1;
          S->missed[t] = 0;
        } else if (++S->missed[t] > kMaxMissed) {
          S->alive[t] = 0;
        }
      }
      __syncwarp();
    }
    if (lane == 0) {
      int t = 0;
      for (int d = 0; d < nd; d++) {
        if (taken[d]) continue;
        while (t < kTracks && S->alive[t]) t++;
        if (t == kTracks) break;
        S->alive[t] = 1; S->missed[t] = 0; S->age[t] = 0; S->assign[t] = d; S->init[t] = 1;
        taken[d] = 1;
        t++;
      }
      int n = 0;
      for (int u = 0; u < kTracks; u++) n += S->alive[u];
      S->n_alive = n;
      S->ndet = nd;
      S->frame += 1;
    }
  }
}

// four standard normals of (particle, draw) by Box-Muller on one Philox block
__device__ __forceinline__ void normals4(int i, int draw, int frame, int t, uint32_t k0, uint32_t k1, float z[4]) {
  const Philox4 r = philox4x32_10((uint32_t)i, (uint32_t)draw, (uint32_t)frame, (uint32_t)t, k0, k1);
  const float a = sqrtf(-2.0f * logf(philox_unit(r.v[0]))), b = sqrtf(-2.0f * logf(philox_unit(r.v[2])));
  z[0] = a * cospif(2.0f * philox_unit(r.v[1]));
  z[1] = a * sinpif(2.0f * philox_unit(r.v[1]));
  z[2] = b * cospif(2.0f * philox_unit(r.v[3]));
  z[3] = b * sinpif(2.0f * philox_unit(r.v[3]));
}

__device__ __forceinline__ float block_sum512(float v, float *wbuf) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if (lane == 0) wbuf[warp] = v;
  __syncthreads();
  float t = 0.f;
  for (int w = 0; w < 16; w++) t += wbuf[w];
  return t;
}

// A_SCORE[Y + X*H] (column-major, get_boxes.cpp:265-300) at the particle centre:
// X = (int)cx and Y = (int)cy as the reference casts them, the largest over
// the n_models maps; 0 when the point is outside the image or no map is given
__device__ __forceinline__ float ascore_at(const float *__restrict__ asc, int n_models, int W, int H, float cx,
                                           float cy) {
  if (!asc || !(cx > -1.0f && cx < (float)W && cy > -1.0f && cy < (float)H)) return 0.f;
  const size_t o = (size_t)(int)cx * H + (int)cy;
  float v = asc[o];
  for (int m = 1; m < n_models; m++) v = fmaxf(v, asc[(size_t)m * W * H + o]);
  return v;
}

__global__ void __launch_bounds__(512) k_track_update(TrackState *S, uint32_t k0, uint32_t k1,
                                                       const float *__restrict__ asc, int n_models, int W, int H) {
  __shared__ float q[6][kParticles];
  __shared__ float cum[512];
  __shared__ float wbuf[16];
  const int t = blockIdx.x, i = threadIdx.x;
  if (!S->alive[t]) return;
  const int frame = S->frame;
  const bool mine = i < kParticles;
  float (*P)[kParticles] = S->p[t];
  if (S->init[t]) {   // particles around the new detection
    const float *d = S->det[S->assign[t]];
    if (mine) {
      float z[4];
      normals4(i, 0, frame, t, k0, k1, z);
      P[0][i] = 0.5f * (d[0] + d[2]) + kSigmaPos * z[0];
      P[1][i] = 0.5f * (d[1] + d[3]) + kSigmaPos * z[1];
      P[2][i] = fmaxf(4.0f, d[2] - d[0] + kSigmaPos * z[2]);
      P[3][i] = fmaxf(4.0f, d[3] - d[1] + kSigmaPos * z[3]);
      P[4][i] = 0.f;
      P[5][i] = 0.f;
    }
    if (i < 4) S->est[t][i] = d[i];
    return;
  }
  float s[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  if (mine) {   // predict: constant velocity plus Gaussian noise
    float z[4], zv[4];
    normals4(i, 0, frame, t, k0, k1, z);
    normals4(i, 1, frame, t, k0, k1, zv);
    for (int c = 0; c < 6; c++) s[c] = P[c][i];
    s[0] += s[4] + kSigmaPos * z[0];
    s[1] += s[5] + kSigmaPos * z[1];
    s[2] = fmaxf(4.0f, s[2] + kSigmaPos * z[2]);
    s[3] = fmaxf(4.0f, s[3] + kSigmaPos * z[3]);
    s[4] += kSigmaVel * zv[0];
    s[5] += kSigmaVel * zv[1];
  }
  float b[4] = {s[0] - 0.5f * s[2], s[1] - 0.5f * s[3], s[0] + 0.5f * s[2], s[1] + 0.5f * s[3]};
  const int a = S->assign[t];
  float w = 0.f;
  if (mine) {
    float pro = 1.0f;
    if (a >= 0) {
      const float *d = S->det[a];
      float d2 = 0.f;
      for (int c = 0; c < 4; c++) d2 += (b[c] - d[c]) * (b[c] - d[c]);
      pro = expf(-d2 / (2.0f * kLikeScale * kLikeScale));
    }
    w = ascore_at(asc, n_models, W, H, s[0], s[1]) + pro;
  }
  float total = block_sum512(w, wbuf);
  if (!(total > 0.f)) {   // every weight underflowed: uniform
    w = mine ? 1.0f : 0.f;
    total = (float)kParticles;
  }
  float e[4];
  for (int c = 0; c < 4; c++) e[c] = block_sum512(w * b[c], wbuf) / total;
  if (i < 4) S->est[t][i] = e[i];
  if (a < 0) {   // no detection: keep the predicted cloud
    if (mine)
      for (int c = 0; c < 6; c++) P[c][i] = s[c];
    return;
  }
  // systematic resampling over the inclusive prefix of the weights
  if (mine)
    for (int c = 0; c < 6; c++) q[c][i] = s[c];
  cum[i] = w;
  __syncthreads();
  for (int o = 1; o < 512; o <<= 1) {
    const float v = i >= o ? cum[i - o] : 0.f;
    __syncthreads();
    cum[i] += v;
    __syncthreads();
  }
  const float tot = cum[kParticles - 1];
  const Philox4 r = philox4x32_10(0u, 2u, (uint32_t)frame, (uint32_t)t, k0, k1);
  const float u0 = philox_unit(r.v[0]) - 1e-7f;
  if (mine) {
    const float target = (u0 + (float)i) * (tot / (float)kParticles);
    int lo = 0, hi = kParticles - 1;
    while (lo < hi) {   // first k with cum[k] >= target
      const int mid = (lo + hi) >> 1;
      if (cum[mid] >= target) hi = mid; else lo = mid + 1;
    }
    for (int c = 0; c < 6; c++) P[c][i] = q[c][lo];
  }
}

__global__ void k_track_clear(TrackState *S) {
  int *p = reinterpret_cast<int *>(S);
  const size_t n = sizeof(TrackState) / sizeof(int);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) p[i] = 0;
}

geye_status tracker_init(TrackerSet &T, unsigned long long seed) {
  T.seed = seed;
  CUDA_TRY(cudaMallocHost(&T.h_count, sizeof(int) * kTrackerStreams));
  memset(T.h_count, 0, sizeof(int) * kTrackerStreams);
  return GEYE_OK;
}

void tracker_free(TrackerSet &T) {
  for (auto &kv : T.d) cudaFree(kv.second);
  T.d.clear();
  if (T.h_count) cudaFreeHost(T.h_count);
  T.h_count = nullptr;
}

geye_status tracker_update(TrackerSet &T, int stream, const int *d_result, int max_cap, const int *d_kept,
                           int n_models, const float *d_ascore, int width, int height, cudaStream_t s) {
  TrackState *S = nullptr;
  auto it = T.d.find(stream);
  if (it == T.d.end()) {
    CUDA_TRY(cudaMalloc(&S, sizeof(TrackState)));
    k_track_clear<<<64, 256, 0, s>>>(S);
    T.d[stream] = S;
  } else {
    S = it->second;
  }
  const uint32_t k0 = (uint32_t)T.seed ^ (uint32_t)(stream * 0x9E3779B9u), k1 = (uint32_t)(T.seed >> 32) + (uint32_t)stream;
  k_track_assoc<<<1, 256, 0, s>>>(S, d_result, max_cap, d_kept, n_models);
  k_track_update<<<kTracks, 512, 0, s>>>(S, k0, k1, d_ascore, n_models, width, height);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(T.h_count + stream, &S->n_alive, sizeof(int), cudaMemcpyDeviceToHost, s));
  return GEYE_OK;
}

int tracker_count(const TrackerSet &T, int stream) { return T.h_count ? T.h_count[stream] : 0; }

int tracker_streams(const TrackerSet &T) { return (int)T.d.size(); }

geye_status tracker_read(TrackerSet &T, int stream, int max, float *boxes, int *n) {
  *n = 0;
  auto it = T.d.find(stream);
  if (it == T.d.end()) return GEYE_OK;
  int alive[kTracks];
  float est[kTracks][4];
  CUDA_TRY(cudaMemcpy(alive, it->second->alive, sizeof(alive), cudaMemcpyDeviceToHost));
  CUDA_TRY(cudaMemcpy(est, it->second->est, sizeof(est), cudaMemcpyDeviceToHost));
  int k = 0;
  for (int t = 0; t < kTracks; t++) {
    if (!alive[t]) continue;
    if (k < max) memcpy(boxes + 4 * k, est[t], sizeof(float) * 4);
    k++;
  }
  *n = k;
  return GEYE_OK;
}

}  // namespace geye
