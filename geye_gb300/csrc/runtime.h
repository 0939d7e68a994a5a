// runtime.h -- host-side runtime of libgeye_dpm: context, plans, pipeline.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <map>
#include <set>
#include <memory>
#include <string>
#include <vector>

#include "internal.h"

// status plumbing shared by the host translation units
#define CUDA_TRY(call)                                                   \
  do {                                                                   \
    cudaError_t e_ = (call);                                             \
    if (e_ != cudaSuccess) {                                             \
      geye::set_error(std::string(#call) + ": " + cudaGetErrorString(e_)); \
      return GEYE_ERR_CUDA;                                              \
    }                                                                    \
  } while (0)
#define GEYE_TRY(call)            \
  do {                            \
    geye_status s_ = (call);      \
    if (s_ != GEYE_OK) return s_; \
  } while (0)
#define ARG_CHECK(cond, msg)   \
  do {                         \
    if (!(cond)) {             \
      geye::set_error(msg);    \
      return GEYE_ERR_ARG;     \
    }                          \
  } while (0)
// a model's filters live on the device of the context that loaded it, and are freed
// with that context: it runs only there, and only while that context lives
#define MODEL_CHECK(m, dev)                                                          \
  do {                                                                               \
    ARG_CHECK((m), "null model");                                                    \
    ARG_CHECK((m)->ctx, "the model's context was destroyed");                        \
    ARG_CHECK((m)->ctx->device == (dev), "the model was loaded on another device");  \
  } while (0)

namespace geye {

// thread-local error text, set by every failing entry point
void set_error(const std::string &msg);

struct DevBuf;
struct Plan;
struct ModelPlan;
// copies n bytes from the host into buf (allocated to fit)
geye_status upload_bytes(geye_ctx *ctx, DevBuf &buf, const void *src, size_t n);
struct ArenaAlloc;
// tensor-core convolution of a plan's models together (conv_tc.cu): tables and
// arena space before the arena exists, bank and tuned chunks after, the launch
geye_status plan_tc(geye_ctx *ctx, Plan &P, ArenaAlloc &A);
geye_status build_tc_plan(geye_ctx *ctx, Plan &P);
geye_status run_conv_tc(geye_ctx *ctx, Plan &P);
// d_small[kSortLevelsUsed]: the deepest NMS sort level with work in the frame;
// d_small[kNmsRoundsUsed]: the greedy batches it took
constexpr int kSortLevelsUsed = 48, kNmsRoundsUsed = 49;
// d_small[kNmsNeed + m]: model m's kept set was resolved again in the quicksort's order
constexpr int kNmsNeed = 160;
void note_sort_levels(geye_ctx *ctx, Plan &P, int used, int rounds);
// tensor-core fconvsMT of one feature map ([pos][32] float on the device) for the stage entry point
geye_status conv_tc_maps(geye_ctx *ctx, const float *d_feat, int a0, int a1, const float *const *filters,
                         const int *b_dims, int n_filters, float *d_out, const std::vector<int> &out_off,
                         std::vector<std::unique_ptr<DevBuf>> &tmp);

// Bump allocator of a plan's float arena (128-byte aligned offsets, in words).
struct ArenaAlloc {
  size_t words = 0;
  int take(size_t n) {
    size_t o = (words + 31) & ~size_t(31);   // 128-byte alignment
    words = o + n;
    return (int)o;
  }
};

// Device buffer owned by a plan or context.
struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
  ~DevBuf();
  geye_status alloc(geye_ctx *ctx, size_t n);
  void release();
  template <class T> T *as() const { return reinterpret_cast<T *>(p); }
};

struct LevelInfo {
  int img_h = 0, img_w = 0;   // image of this level (aliases for [interval, 2*interval))
  int img_level = 0;          // level whose image planes are used
  int img_off = -1;           // word offset of the planes (own image only)
  int fs0 = 0, fs1 = 0;       // features
  int sbin = 0;
  float scale = 0.f;          // scales[] entry
  int feat_off = -1;          // [pos][32]
  int feat16_off = -1;        // tensor-core planes, 2-byte units
  int feat16lo_off = -1;      // BF16 remainder planes (root levels, BF16 mode), 2-byte units
  int hist_off = -1;
};

struct ModelPlan {
  geye_model *model = nullptr;
  int LEN = 0;                          // levels this model uses
  std::vector<ConvJob> root_jobs, part_jobs;
  int root_max_b0 = 0, root_max_b1 = 0, root_max_g = 1, root_tiles_y = 0, root_tiles_x = 0;
  int part_max_b0 = 0, part_max_b1 = 0, part_max_g = 1, part_tiles_y = 0, part_tiles_x = 0;
  int root_cr = 4, part_cr = 4;   // FP32 conv rows per thread (tuned per plan)
  std::vector<DtJob> dt_jobs;
  int dt_max_d0 = 0, dt_max_d1 = 0;
  std::vector<ScoreJob> score_jobs;
  int score_max_r = 0;
  int cap = 0;                          // max detections (sum of root map sizes)
  // device copies
  DevBuf d_root_jobs, d_part_jobs, d_dt_jobs, d_score_jobs, d_counts;
  DevBuf d_dt_blocks1, d_dt_blocks2;    // DT tiles of every map (dt_block_lists)
  int dt_nblocks1 = 0, dt_nblocks2 = 0;
  int dt_elems = kDtElems;              // outputs per DT block: tuned on the plan's first frame (tune_dt)
  bool dt_tuned = false;
  float dt_ms[3] = {0, 0, 0};           // the timed launch per kDtElemsChoices entry
  DevBuf d_score_blocks;                // score / box blocks of every map (score_block_list)
  int score_nblocks = 0;
  // per-(level, comp) and per-(L, part) map offsets for stage readback
  std::vector<int> root_map_off, root_r0, root_r1;     // [level*NoC + c], -1 if none
  std::vector<int> part_map_off, part_d0, part_d1;     // [L*NoP + p]
  std::vector<int> skipped;                            // per level
  double conv_flops = 0, conv_bytes = 0, dt_bytes = 0, score_bytes = 0;
  // A_SCORE lookups: [job][image column] score-map column base, [job][image row] score row
  DevBuf d_as_col, d_as_row;
};

// One row of the tensor-core convolution's filter bank (conv_tc.cu): filter
// `filt` of model `mi` (its roots, then its parts), from filter row y0 and
// column x0 on, or the BF16 remainder of those weights; mi < 0: a padding row.
struct BankRowSpec {
  int mi = -1, filt = 0, y0 = 0, x0 = 0, lo = 0;
  float scale = 1.f;   // FP8: the filter's power-of-two scale
};

// The tensor-core convolution of all of a plan's models (conv_tc.cu): bank
// rows, one job per feature level, the epilogue's column tables, the root sums.
struct TcPlan {
  int planes = 0;                       // 4: BF16 planes, 2: e4m3
  int grid_b0 = 0, grid_b1 = 0;         // the bank's tap grid
  int rows = 0, rows_p16 = 0, rows_r16 = 0;
  std::vector<BankRowSpec> bank_rows;
  std::vector<TcJob> jobs;
  std::vector<TcCol> cols;
  std::vector<RootSumJob> sums;
  int sum_max_r = 0;
  DevBuf d_bank, d_jobs, d_chunks, d_cols, d_sums;
  int n_chunks = 0, stages = 0, tps = 1;   // bank stages; taps a stage (0: a filter column, -1: a phase)
  size_t smem = 0;
  int shape = -1;                       // tile-shape candidate the autotuner chose
  float tuned_ms = 0.f;                 // its measured time per launch
  // the persistent form (shape == the candidate after the tile shapes): units, and per CTA
  // its units, bank region and slab buffer bytes
  DevBuf d_units, d_ranges;
  int tcp_ctas = 0;
  uint32_t tcp_colbuf = 0;
};

struct Plan {
  // distinct for every plan a process builds (a rebuilt plan never reuses one)
  const unsigned long long serial = next_plan_serial();
  static unsigned long long next_plan_serial() {
    static std::atomic<unsigned long long> n{0};
    return ++n;
  }
  int width = 0, height = 0;           // frame size (0 when built from features)
  int interval = 0, sbin = 0, LEN = 0;
  bool from_features = false;
  std::vector<LevelInfo> lv;
  // resize phases: each phase is two passes (vertical then horizontal)
  std::vector<std::vector<ResizeJob>> vjobs, hjobs;
  std::vector<int> v_max_items, h_max_items;   // per phase: largest output column count
  std::vector<DevBuf> d_vjobs, d_hjobs;
  DevBuf d_tap_start, d_tap_si, d_tap_alpha;
  std::vector<HogJob> hog_jobs;
  DevBuf d_hog_jobs;
  DevBuf d_hog_vote_blocks;             // vote kernel blocks of every level (hog_vote_blocks)
  int hog_vote_nblocks = 0;
  int hog_max_b0 = 0, hog_max_b1 = 0;
  std::vector<HogPixJob> pix_jobs;   // one per image
  DevBuf d_pix_jobs;
  int pix_max_xe = 0;
  std::vector<std::unique_ptr<ModelPlan>> models;
  TcPlan tc;                             // BF16 / FP8 modes
  // memory
  size_t arena_words = 0, arena16_elems = 0;
  DevBuf arena, arena16;
  DevBuf d_bgr;                          // frame upload buffer
  DevBuf d_boxes, d_kept_boxes, d_nms_f, d_nms_i, d_small, d_ascore, d_result;
  int gl = 0, max_cap = 0;
  // algorithmic bytes per stage (for roofline reporting)
  double bytes_resize = 0, bytes_hog = 0;
  // last-run results (host)
  std::vector<int> last_D, last_K;
  // the frame after its ingest, captured as CUDA graphs keyed by threshold, overlap and timing
  struct FrameGraph {
    cudaGraphExec_t exec = nullptr;
    int kernels = 0;
  };
  std::map<std::string, FrameGraph> graphs;
  // grid-wide NMS sort levels launched per frame (0: the default for max_cap),
  // adapted once to the depth the plan's frames need (note_sort_levels)
  int sort_levels = 0;
  int nms_rounds = 0;   // greedy resolve/pass rounds per frame (0: kNmsRounds), adapted to the frames
  bool sort_levels_fixed = false;
  // asynchronous submission (serve.cu): pinned frame staging, pinned result
  // block (counts, then per model kHostRes records) and the completion event
  void *h_bgr = nullptr, *h_res = nullptr;
  cudaEvent_t ev_done = nullptr;
  ~Plan() {
    for (auto &g : graphs)
      if (g.second.exec) cudaGraphExecDestroy(g.second.exec);
    if (h_bgr) cudaFreeHost(h_bgr);
    if (h_res) cudaFreeHost(h_res);
    if (ev_done) cudaEventDestroy(ev_done);
  }
};

}  // namespace geye

struct geye_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  // A_SCORE runs beside NMS on this stream (forked after the score stage,
  // joined before the frame ends)
  cudaStream_t side = nullptr;
  // captures the bodies of the frame graph's conditional nodes (NMS rounds, quicksort pass)
  cudaStream_t aux = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  geye_conv_mode conv_mode = GEYE_CONV_FP32;
  std::map<std::string, std::unique_ptr<geye::Plan>> plans;
  int next_model_id = 1;
  // timing
  bool timing = false;
  cudaEvent_t ev[GEYE_N_STAGES + 1] = {};
  float stage_ms[GEYE_N_STAGES] = {};
  double stage_bytes[GEYE_N_STAGES] = {};
  double conv_flops = 0;
  int launches = 0;
  bool use_graphs = true;   // replay the frame as a CUDA graph (GEYE_NO_GRAPHS=1 at creation: plain launches)
  int nms_order = geye::kNmsOrderKey;   // geye_ctx_set_nms_order
  // the frame graph runs the NMS quicksort-order pass as an if node (a lone
  // frame skips its launches when no model needs it); server slots and batch
  // lanes launch it plainly (its kernels return at once there), which measured
  // faster with frames of other contexts in flight
  bool nms_if_node = true;
  bool front_external = false;   // a batch's front end ran ingest, resize and HOG of the frame already
  bool capturing = false;
  // fault injection (host side)
  std::string inject_op;
  int inject_countdown = 0;
  // fallback counters etc. (device)
  geye::DevBuf d_diag;
  // pinned staging for results
  void *h_pinned = nullptr;
  size_t h_pinned_bytes = 0;
  // last device-resident run
  geye::Plan *last_plan = nullptr;
  // frame submitted with geye_detect_submit and not collected yet
  geye::Plan *pending = nullptr;
  // live models (detached when the context goes away first)
  std::set<geye_model *> models;
};
