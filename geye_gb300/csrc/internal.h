// internal.h -- shared declarations of libgeye_dpm (host runtime + kernels).
//
// Device layouts (all spatial maps column-major like the reference, so a
// level's stage output is a plain copy):
//   image level l:   3 float planes [c][w][h]                (x*h + y)
//   feature level l: [pos][32] float, pos = x*fs0 + y, channel 31 = 0
//   conv/DT/score maps: [x][y] float (int for argmax), per (level, filter)
// Every per-frame buffer lives in one arena sized when a plan is built.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "geye_dpm.h"

namespace geye {

constexpr int kFeat = 31;       // HOG channels
constexpr int kFeatPad = 32;    // channel stride in device feature buffers
constexpr int kMaxParts = 32;   // parts per component supported by the kernels
constexpr int kTcPlanePad = 128;   // cells after each bf16 feature plane (reach of a 128-position tile)

// Raises a kernel's dynamic shared-memory limit to at least `smem` bytes on the
// current device. The attribute belongs to the device, so the record of the largest
// size set is kept per device; raises are serialised, so a concurrent smaller raise
// never lowers a limit another thread's launch relies on.  Only a raise that
// succeeded is recorded: a failed one is tried again by the next launch, and
// its error comes back (the launch that needs the limit then fails and reports).
constexpr int kSmemAttrDevices = 64;
struct SmemAttr {
  size_t set[kSmemAttrDevices] = {};
  std::mutex mu;
};
template <typename K>
inline cudaError_t raise_smem(SmemAttr &A, K *kernel, size_t smem) {
  if (smem <= 48 * 1024) return cudaSuccess;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> g(A.mu);
  if (dev >= 0 && dev < kSmemAttrDevices && A.set[dev] >= smem) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess && dev >= 0 && dev < kSmemAttrDevices) A.set[dev] = smem;
  return e;
}

// ----------------------------------------------------------------------------
// job descriptors (device-readable, plain structs)
// ----------------------------------------------------------------------------
struct ResizeJob {         // one 1-D resize pass of one level
  int src_off;             // float offset of the source planes
  int dst_off;             // float offset of the destination planes
  int src_h, src_w;        // source dims (rows, cols)
  int dst_h, dst_w;        // destination dims of this pass
  int tap_start_off;       // int offset of tap_start[dst_len + 1] in the tap-index table
  int tap_off;             // offset of the tap (si, alpha) arrays
};

struct HogJob {
  int img_off;             // image planes [3][w][h]
  int h, w;                // image dims
  int sbin;
  int b0, b1;              // histogram blocks (rows, cols)
  int hist_off;            // [18][b1*b0] then norm [b1*b0] at hist_off + 18*b1*b0
  int fs0, fs1;            // output cells
  int feat_off;            // [pos][32] float
  int feat16_off;          // tensor-core planes (offset in 2-byte units), -1 = not written
  int feat16lo_off;        // BF16 remainder planes (root levels in BF16 mode), -1 = none
  int fast;                // 1 (tensor-core modes): float normalisation factors computed per cell,
                           // no corner pass; 0: the reference's double form, bit for bit
  int tc_planes;           // 4: bf16 planes [4][fs0*fs1 + kTcPlanePad][16 B]; 2: e4m3 planes; 0: none
  int mag_off, bin_off;    // the image's pixel magnitudes (float) and bins (u8), [x * pix_Y + y]
  int pix_Y;
  int corner_off;          // normalisation factors [(fs1 + 1) * (fs0 + 1)]
};

struct HogPixJob {         // (bin, magnitude) of the pixels of one image
  int img_off;             // image planes [3][w][h]
  int h, w;
  int xe, ye;              // pixels 1 <= x < xe, 1 <= y < ye
  int Y;                   // row stride of the outputs
  int mag_off, bin_off;    // float magnitudes; u8 bins at (uint8_t *)(arena + bin_off)
};

struct ConvJob {           // a block of outputs of one (level, filter group)
  int feat_off, a0, a1;    // feature level [pos][32], dims
  int filt_base;           // first filter index in the model's filter table
  int n_filt;              // filters in the group (same size)
  int b0, b1;              // filter dims
  int c0, c1;              // output dims
  int out_off;             // output of filter g at out_off + g*c0*c1
  int tiles_y, tiles_x;    // output tiles of this job
};

// tensor-core convolution (conv_tc.cu)
struct TcJob {             // one feature level's MMA chain over the rows of the filter bank it uses
  int plane_off;           // the level's NQ feature planes, in 2-byte units of arena16
  int lo_off;              // its BF16 remainder planes (split chain), -1: none
  int plane_cells;         // cells per plane (fs0*fs1 + kTcPlanePad)
  int fs0, fs1;            // feature rows, columns
  int b0, b1;              // tap grid
  int bank_off;            // byte offset of the job's bank [tap][q][n][16 B] (its rows, contiguous)
  int n;                   // the job's bank rows: the MMA's N columns (a multiple of 16)
  int lo_row, n_lo;        // split chain: rows lo_row .. lo_row+n_lo (0: none), accumulated into TMEM columns lo_row ..
  int col_tab;             // first entry of the job's column table (n entries)
  int ntiles;              // 128-position tiles the job covers
  int row0;                // the job's first row in the plan's row list (host bookkeeping)
};

struct TcCol {             // what the epilogue does with one MMA column of a job
  int kind;                // 0: nothing; 1: a map; 2: a root block
  int off;                 // 1: the map's float offset; 2: the block buffer's (indexed by position)
  int rows, cols;          // 1: the map's rows (c0) and columns (c1)
  int pair;                // 2: the column of the block's hi*lo products, relative (0: none)
  float inv;               // factor undoing the operand scaling (FP8), else 1
};

constexpr int kMaxRootBlocks = 16;
struct RootSumJob {        // one (level, component) root map as the sum of its blocks
  int out_off, r0, r1, fs0, nblk;
  int blk[kMaxRootBlocks];     // block buffers (position-indexed)
  int shift[kMaxRootBlocks];   // the block's position offset: x0*fs0 + y0
};

struct DtJob {             // one part map: DT of the negated map
  int in_off;              // part conv map (negated on load)
  int d0, d1;
  int tmpM_off, tmpI_off;  // pass-1 outputs
  int M_off, Ix_off, Iy_off;
  float ax, bx, ay, by;
  int negate;              // 1: run on -map (inverse_Q of the pipeline); 0: plain dt()
  // only what the pipeline reads is written (0: full maps, dt() itself):
  // samp_m: M only where the score sum reads it (rows y = par_y, columns
  // x = par_x mod 2); samp_i: Ix/Iy only where the part boxes probe (the other
  // parity in both), set when every probe falls inside the map
  int samp_m, samp_i;
  int par_y, par_x;
  // sampled entries stored compactly: M of (x, y) in its class at
  // ((x - par_x) / 2) * cm0 + (y - par_y) / 2, Ix/Iy likewise with the other
  // parity and ci0 rows (cm0 / ci0 = the class's rows; 0: full layout)
  int cm0, ci0;
};

struct ScoreJob {          // one (level, component) score map
  int root_off;            // root conv map
  int r0, r1;
  float off;               // offw[ridx[c]]
  int score_off;           // output score map
  int np;
  int comp;
  int level;               // pyramid level of the root map
  float scale;             // sbin / scales[level]
  int rsize0, rsize1;      // component root size (boxes, A_SCORE)
  int RY, RX;              // A_SCORE shifts
  int part_M[kMaxParts];   // DT outputs per part (M); Ix/Iy at M + ix_delta/iy_delta
  int part_Ix[kMaxParts];
  int part_Iy[kMaxParts];
  int part_d0[kMaxParts];
  int part_d1[kMaxParts];
  int ax[kMaxParts];       // anchor+1
  int ay[kMaxParts];
  int psize0[kMaxParts];   // part box size (component file)
  int psize1[kMaxParts];
  int part_cm0[kMaxParts]; // DtJob.cm0 / ci0: the parts' compact layouts (0: full)
  int part_ci0[kMaxParts];
};

// Root box of position (x, y) of a score map (get_boxes.cpp:227-235, pad = 0).
// (o[0] + rs0*scale) is a float sum; subtracting 1.0 in double and rounding to
// float equals the float subtraction (the double difference is exact), so the
// whole box is float arithmetic.
__host__ __device__ __forceinline__ void root_box(int x, int y, float scale, int rs0, int rs1, float *o) {
  o[0] = ((float)y - (float)0 + 1) * scale;
  o[1] = ((float)x - (float)0 + 1) * scale;
  o[2] = (o[0] + (float)rs0 * scale) - 1.0f;
  o[3] = (o[1] + (float)rs1 * scale) - 1.0f;
}

// ----------------------------------------------------------------------------
// host model
// ----------------------------------------------------------------------------
struct HostModel {
  int numcomponent = 0, sbin = 0, interval = 0, max_X = 0, max_Y = 0, padx = 0, pady = 0;
  float ratio = 1.0f;
  std::vector<int> ridx, oidx, rsize, numpart;
  std::vector<float> offw;
  std::vector<std::vector<int>> pidx, didx, psize;
  int DefL = 0;
  std::vector<float> def;
  std::vector<int> anchor;
  std::vector<std::vector<float>> x1, y1, x2, y2;
  int NoR = 0, NoP = 0;
  std::vector<int> root_size, part_size, part_partner;   // n x 3
  std::vector<std::vector<float>> rootfilter, partfilter; // [31][w][h]
};

}  // namespace geye

struct geye_model {
  geye_ctx *ctx = nullptr;
  geye::HostModel h;
  bool ini = true;         // ini_scales latch (featurepyramid.cpp:178-236)
  int max_scale = -1;
  int id = 0;
  // device filter tables, fp32 [31][w][h] per filter, roots then parts
  float *d_filters = nullptr;
  int *d_filt_off = nullptr;   // float offsets, NoR + NoP entries
  float *d_coef = nullptr;     // box regression [comp][x1, y1, x2, y2][ML]
  std::vector<int> filt_off;
  // tile shapes the autotuners chose per plan geometry (frame size, levels, mode,
  // and for the tensor-core convolution the plan's other models), shared by every
  // context that plans this model at that geometry
  std::mutex tc_mu;
  std::map<std::string, std::pair<int, float>> tc_tuned;   // candidate, ms per launch
  int gl() const { return (h.numpart[0] + 1) * 4 + 3; }
};

namespace geye {

// ----------------------------------------------------------------------------
// kernel launchers (defined in the .cu files)
// ----------------------------------------------------------------------------
void launch_fill(float *p, size_t n, float v, cudaStream_t s);
void launch_ingest(const uint8_t *bgr, int width, int height, int width_step, float *planes, cudaStream_t s);
void launch_resize_pass(const ResizeJob *d_jobs, int n_jobs, int max_cols, int vertical, const int *d_tap_start,
                        const int *d_tap_si, const float *d_tap_alpha, float *arena, cudaStream_t s);
// (job, block of histogram blocks) of every level's vote kernel
void hog_vote_blocks(const std::vector<HogJob> &jobs, std::vector<int2> &blocks);

// Batched front end (a batch of frames of any sizes): ingest, resize and HOG
// of every level of every frame, each stage one persistent launch over a
// ragged work list of (frame, job, chunk) items.  A frame's jobs are its own
// plan's (the same device functions as the single-frame kernels).
constexpr int kBatchMaxPhases = 16;
struct BatchFrame {
  const uint8_t *bgr;      // the frame on the device
  int width, height, width_step;
  float *arena;            // the frame's plan
  uint8_t *arena16;
  int img0_off;            // level-0 image planes (ingest output)
  int n_phases;
  const ResizeJob *vjobs[kBatchMaxPhases], *hjobs[kBatchMaxPhases];
  const int *tap_start, *tap_si;
  const float *tap_alpha;
  const HogPixJob *pix;
  const HogJob *hog;
  const int2 *vote_blocks;
};
struct BatchItem {
  int frame, job, chunk, pad;
};
enum BatchStage { kBatchIngest = 0, kBatchResizeV, kBatchResizeH, kBatchPix, kBatchVote, kBatchNorm, kBatchFeat };
constexpr int kBatchColumns = 8;   // resize / pixel columns per item (a warp each)
constexpr int kBatchCells = 256;   // corners / cells per item (a thread each)
// one stage (phase: the resize phase) over n items
void launch_batch_front(int stage, const BatchFrame *d_frames, const BatchItem *d_items, int n, int phase,
                        cudaStream_t s);
// corners: run the corner-factor pass (jobs with fast = 0 read its factors)
void launch_hog(const HogJob *d_jobs, int n_jobs, const int2 *d_vote_blocks, int n_vote_blocks, int max_b0,
                int max_b1, const HogPixJob *d_pix, int n_pix, int max_xe, float *arena, void *arena16,
                bool corners, cudaStream_t s);   // arena16: base of the tensor-core planes (bytes)
void launch_to_ref_layout(const float *feat, int fs0, int fs1, float *out, cudaStream_t s);
void launch_flip_feat(const float *feat, int n0, int n1, float *out, cudaStream_t s);
void launch_from_ref_layout(const float *ref, int fs0, int fs1, float *feat, cudaStream_t s);
void launch_conv_fp32(const ConvJob *d_jobs, int n_jobs, int max_tiles_y, int max_tiles_x, const float *filters,
                      const int *filt_off, const float *arena_in, float *arena_out, int max_b0, int max_b1,
                      int max_group, cudaStream_t s, int cr = 4);
// (job, first line) of every DT block, pass 1 (columns) and pass 2 (rows), largest maps first
// DT tiles of about `elems` outputs per block (kDtElems by default; a plan
// tunes it on its first frame's maps among kDtElemsChoices)
constexpr int kDtElems = 2048;
constexpr int kDtElemsChoices[3] = {1024, 2048, 4096};
void dt_block_lists(const std::vector<DtJob> &jobs, std::vector<int2> &b1, std::vector<int2> &b2, int elems);
void launch_dt(const DtJob *d_jobs, const int2 *d_b1, int n_b1, const int2 *d_b2, int n_b2, int max_d0, int max_d1,
               float *arena, int *arena_i, int *fallback_count, int elems, cudaStream_t s);
// (job, block of 256 positions) of every score map, in job order
void score_block_list(const std::vector<ScoreJob> &jobs, std::vector<int2> &blocks);
void launch_score(const ScoreJob *d_jobs, const int2 *d_blocks, int n_blocks, float thresh, float *arena,
                  int *block_counts, cudaStream_t s);
void launch_boxes(const ScoreJob *d_jobs, const int2 *d_blocks, int n_blocks, float thresh, const float *arena,
                  const int *arena_i, const int *block_offsets, int GL, float *boxes, cudaStream_t s);
void launch_scan_counts(int *counts, int n, int *total, cudaStream_t s);
void launch_ascore(const int *col, const int *row, int n_jobs, const float *arena, float *a_score, int im_w,
                  int im_h, float thresh, unsigned *max_bits, cudaStream_t s);
void launch_ascore_normalize(float *a_score, int n, const unsigned *max_bits, cudaStream_t s);
// one block per model; model m uses boxes/out at m*cap*GL, scratch at m*cap*6 floats and m*cap*5 ints
void launch_nms(const float *boxes, const int *d_num, int n_models, int GL, float overlap, int cap,
                float *scratch_f, int *scratch_i, float *out, int *d_kept, int *err, cudaStream_t s);
// pipeline NMS (nms_sort.cu, nms_batch.cu): per model nms_model_words(cap) ints
// of scratch and 5 * cap floats (the boxes in sorted order)
constexpr int kNmsBatch = 256;     // boxes resolved per round
constexpr int kNmsSegS = 16384;    // sort segments finished in shared memory (one block, ~203 KB)
constexpr int kNmsTile = 4096;     // elements per block in the sort's grid-wide partitions
__host__ __device__ inline int nms_big_cap(int cap) { return cap / kNmsSegS + 2; }
__host__ __device__ inline int nms_tile_cap(int cap) { return cap / kNmsTile + nms_big_cap(cap) + 1; }
constexpr int kNmsCells = 64;      // cells per image axis of the greedy's pick masks
constexpr int kNmsLevels = 7;      // their sparse-table levels (spans of 1..64 cells)
// elements per block in the key-order radix sort: small tiles spread a frame's
// few thousand boxes over more blocks; large ones keep the single-block digit
// scan short when a model has a million boxes
__host__ __device__ inline int nms_rs_tile(int cap) { return cap <= (1 << 18) ? 1024 : 4096; }
__host__ __device__ inline int nms_rs_tiles(int cap) { return (cap + nms_rs_tile(cap) - 1) / nms_rs_tile(cap); }
// summary bitmap: one bit per word of the alive bitmap
__host__ __device__ inline int nms_summary_words(int cap) { return ((cap + 31) / 32 + 31) / 32 + 1; }
__host__ __device__ inline size_t nms_model_words(int cap) {
  const size_t w = 8 * (size_t)cap + 64 + 5 * kNmsBatch + 4 * (size_t)nms_big_cap(cap) +
                   2 * (size_t)nms_tile_cap(cap) + 256 * (size_t)nms_rs_tiles(cap) + nms_summary_words(cap) +
                   2 * kNmsLevels * kNmsCells * (kNmsBatch / 32);
  return (w + 31) & ~(size_t)31;
}
// diag (optional): per model m, diag[8m+1..8m+5] = sort segments left to the fallback, batches, picks,
// whether the finish kernel ran rounds itself, whether the quicksort order was needed
// levels, lv_used: as for launch_nms_sort (nms_common.h); rounds: resolve/pass
// rounds launched before the finish kernel (<= 0: kNmsRounds), *rounds_used
// (optional) gets the batches the frame took, the finish kernel's included
// need: n_models ints, zero on entry; order: kNmsOrderKey (the scores in
// key order, the quicksort's order only for the models that need it: need[m]
// raised) or kNmsOrderQuicksort (the quicksort's order for every model)
constexpr int kNmsRounds = 8, kNmsMaxRounds = 64;
constexpr int kNmsOrderKey = 0, kNmsOrderQuicksort = 1;
// aux: null for plain launches on s; when s is capturing a graph, a second
// stream that captures the body of the quicksort-order pass's if node
// extent: box coordinates in [0, extent) spread over the pick masks' cells
// (any value is exact; boxes outside share the edge cells)
cudaError_t launch_nms_batch(const float *boxes, const int *d_num, int n_models, int GL, float overlap,
                             float extent, int cap, int *si, float *sf, float *out, int *d_kept, int *err,
                             long long *diag, int levels, int *lv_used, int rounds, int *rounds_used, int *need,
                             int order, cudaStream_t s, cudaStream_t aux);
int nms_sort_levels(int cap);   // the default number of grid-wide sort levels for cap boxes
void launch_new_rects(const float *kept, const int *d_kept, int GL, int np, const float *coef, int img_w,
                      int img_h, float ratio, int *point, int *or_point, int *type, float *scale, float *score,
                      cudaStream_t s);

}  // namespace geye
