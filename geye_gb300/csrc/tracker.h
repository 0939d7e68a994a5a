// tracker.h -- device-resident particle-filter tracker of the detection server.
//
// The reference tracks with OpenCV's CvConDensation on the host
// (CAR_TRACKING/tracking.cpp:321-850: 1000 particles, uniform noise, template
// likelihood).  This tracker follows the serving specification instead: per
// camera stream up to kTracks tracks of kParticles particles, state (cx, cy,
// w, h, vx, vy) in FP32, constant-velocity motion with Gaussian noise
// (sigma 4 px on position and size, 1 px/frame on velocity) drawn from a
// per-stream Philox4x32-10 stream, particle weights of A_SCORE at the
// particle plus a Gaussian likelihood on the box corners of the associated
// detection (the reference adds A_SCORE to its template likelihood,
// tracking.cpp:429-433), and systematic resampling.  Association is
// greedy by IoU (>= 0.3) in track order; detections left over start tracks;
// tracks missed kMaxMissed frames in a row end.
#pragma once
#include <stdint.h>

#include <map>
#include <vector>

#include "runtime.h"

namespace geye {

constexpr int kTrackerStreams = 256;   // stream ids 0..255
constexpr int kTracks = 32;            // tracks per stream
constexpr int kParticles = 500;        // particles per track
constexpr int kMaxDet = 256;           // detections per frame fed to the tracker
constexpr int kMaxMissed = 10;
constexpr float kSigmaPos = 4.0f, kSigmaVel = 1.0f, kLikeScale = 8.0f, kAssocIoU = 0.3f;

struct TrackState {
  int frame, n_alive, ndet, pad;
  int alive[kTracks], missed[kTracks], age[kTracks], assign[kTracks], init[kTracks];
  float est[kTracks][4];                 // x1, y1, x2, y2
  float det[kMaxDet][4];
  float p[kTracks][6][kParticles];       // cx, cy, w, h, vx, vy
};

struct TrackerSet {
  std::map<int, TrackState *> d;   // per stream, allocated on its first frame
  int *h_count = nullptr;          // pinned: live tracks per stream after its latest update
  unsigned long long seed = 0;
};

geye_status tracker_init(TrackerSet &T, unsigned long long seed);
void tracker_free(TrackerSet &T);
// one frame of `stream`: detections are the kept boxes of each model
// (point arrays of d_result, model m at m*max_cap*11, counts d_kept[m]);
// d_ascore holds the frame's n_models A_SCORE maps (width x height,
// column-major, map m at m*width*height) or is NULL
geye_status tracker_update(TrackerSet &T, int stream, const int *d_result, int max_cap, const int *d_kept,
                           int n_models, const float *d_ascore, int width, int height, cudaStream_t s);
int tracker_count(const TrackerSet &T, int stream);
int tracker_streams(const TrackerSet &T);
geye_status tracker_read(TrackerSet &T, int stream, int max, float *boxes, int *n);

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC 2011): counter (c0..c3), key (k0, k1)
struct Philox4 {
  uint32_t v[4];
};
__host__ __device__ inline void philox_mulhilo(uint32_t a, uint32_t b, uint32_t &hi, uint32_t &lo) {
  const uint64_t p = (uint64_t)a * b;
  hi = (uint32_t)(p >> 32);
  lo = (uint32_t)p;
}
__host__ __device__ inline Philox4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0,
                                                 uint32_t k1) {
  for (int r = 0; r < 10; r++) {
    uint32_t hi0, lo0, hi1, lo1;
    philox_mulhilo(0xD2511F53u, c0, hi0, lo0);
    philox_mulhilo(0xCD9E8D57u, c2, hi1, lo1);
    const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  Philox4 o;
  o.v[0] = c0; o.v[1] = c1; o.v[2] = c2; o.v[3] = c3;
  return o;
}
// uniform in (0, 1]: (x + 1) / 2^32 in float arithmetic of 24 bits
__host__ __device__ inline float philox_unit(uint32_t x) { return ((float)(x >> 8) + 1.0f) * (1.0f / 16777216.0f); }

}  // namespace geye
