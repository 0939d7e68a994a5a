// api.cu -- the C ABI of libgeye_dpm (include/geye_dpm.h).
//
// Each entry point replaces one reference interface (listed in the header)
// with the same argument meaning, but returns a status code instead of
// calling exit() (the reference exits on every CUDA error:
// CAR_TRACKING/fconvsMT.cpp:19-23, featurepyramid.cpp:505-509).  There is no
// CPU fallback: without a usable CUDA device every call fails.
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "runtime.h"

namespace geye {
geye_status run_frame(geye_ctx *ctx, Plan &P, const uint8_t *d_bgr, int width_step, float thresh, float overlap,
                      const float *const *h_ascore_init);
geye_status run_pyramid(geye_ctx *ctx, Plan &P, const uint8_t *d_bgr, int width_step);
geye_status run_hog(geye_ctx *ctx, Plan &P);
geye_status run_conv(geye_ctx *ctx, Plan &P, ModelPlan &mp);
geye_status run_dt(geye_ctx *ctx, Plan &P, ModelPlan &mp);
geye_status run_score(geye_ctx *ctx, Plan &P, ModelPlan &mp, int mi, float thresh);
geye_status run_ascore(geye_ctx *ctx, Plan &P, ModelPlan &mp, int mi, float thresh, const float *h_init);
geye_status collect_stage_times(geye_ctx *ctx);
geye_status frame_plan(geye_ctx *ctx, geye_model *const *models, int n, int w, int h, Plan **out);
geye_status features_plan(geye_ctx *ctx, geye_model *model, const int *ftsize, const float *scales, int n_levels,
                          int img_w, int img_h, Plan **out);
geye_status parse_model_files(const char *c, const char *r, const char *p, HostModel &m);
void launch_nms(const float *boxes, const int *d_num, int n_models, int GL, float overlap, int cap,
                float *scratch_f, int *scratch_i, float *out, int *d_kept, int *err, cudaStream_t s);
}  // namespace geye

using namespace geye;


static thread_local std::string *g_err_ptr = nullptr;

extern "C" {

const char *geye_version(void) { return "geye_dpm 0.1 (sm_103a)"; }

geye_status geye_ctx_create(int device, void *cuda_stream, geye_ctx **out) {
  ARG_CHECK(out, "out is null");
  *out = nullptr;
  int n = 0;
  CUDA_TRY(cudaGetDeviceCount(&n));
  ARG_CHECK(device >= 0 && device < n, "no such CUDA device");
  CUDA_TRY(cudaSetDevice(device));
  cudaDeviceProp prop;
  CUDA_TRY(cudaGetDeviceProperties(&prop, device));
  if (prop.major < 10) {
    set_error("libgeye_dpm is built for sm_103a (Blackwell); this device is sm_" + std::to_string(prop.major) +
              std::to_string(prop.minor));
    return GEYE_ERR_UNSUPPORTED;
  }
  geye_ctx *ctx = new geye_ctx();
  ctx->device = device;
  if (const char *e = getenv("GEYE_NO_GRAPHS")) ctx->use_graphs = !(e[0] == '1');
  if (cuda_stream) {
    ctx->stream = reinterpret_cast<cudaStream_t>(cuda_stream);
  } else {
    cudaError_t e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      delete ctx;
      set_error(std::string("cudaStreamCreate: ") + cudaGetErrorString(e));
      return GEYE_ERR_CUDA;
    }
    ctx->own_stream = true;
  }
  {
    cudaError_t e = cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->aux, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming);
    if (e != cudaSuccess) {
      if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
      if (ctx->aux) cudaStreamDestroy(ctx->aux);
      if (ctx->side) cudaStreamDestroy(ctx->side);
      if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
      delete ctx;
      set_error(std::string("side stream: ") + cudaGetErrorString(e));
      return GEYE_ERR_CUDA;
    }
  }
  geye_status s = ctx->d_diag.alloc(ctx, 256);
  if (s != GEYE_OK) { delete ctx; return s; }
  cudaMemset(ctx->d_diag.p, 0, 256);
  *out = ctx;
  return GEYE_OK;
}

geye_status geye_ctx_destroy(geye_ctx *ctx) {
  if (!ctx) return GEYE_OK;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  // the models loaded here may be read by other contexts' work in flight (server
  // slots, batch lanes): wait for the device before their filters are freed
  if (!ctx->models.empty()) cudaDeviceSynchronize();
  ctx->plans.clear();
  for (geye_model *m : ctx->models) {
    if (m->d_filters) cudaFree(m->d_filters);
    if (m->d_filt_off) cudaFree(m->d_filt_off);
    if (m->d_coef) cudaFree(m->d_coef);
    m->d_filters = nullptr; m->d_filt_off = nullptr; m->d_coef = nullptr;
    m->ctx = nullptr;
  }
  ctx->models.clear();
  ctx->d_diag.release();
  for (auto &e : ctx->ev)
    if (e) cudaEventDestroy(e);
  if (ctx->h_pinned) cudaFreeHost(ctx->h_pinned);
  if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
  if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
  if (ctx->side) {
    cudaStreamSynchronize(ctx->side);
    cudaStreamDestroy(ctx->side);
  }
  if (ctx->aux) cudaStreamDestroy(ctx->aux);
  if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return GEYE_OK;
}

geye_status geye_ctx_set_conv_mode(geye_ctx *ctx, geye_conv_mode mode) {
  ARG_CHECK(ctx, "ctx is null");
  ARG_CHECK(mode == GEYE_CONV_FP32 || mode == GEYE_CONV_BF16 || mode == GEYE_CONV_FP8, "unknown conv mode");
  ctx->conv_mode = mode;
  return GEYE_OK;
}

geye_status geye_ctx_set_nms_order(geye_ctx *ctx, int order) {
  ARG_CHECK(ctx, "ctx is null");
  ARG_CHECK(order == GEYE_NMS_ORDER_KEY || order == GEYE_NMS_ORDER_QUICKSORT, "unknown NMS order");
  ctx->nms_order = order == GEYE_NMS_ORDER_KEY ? kNmsOrderKey : kNmsOrderQuicksort;
  return GEYE_OK;
}

geye_status geye_ctx_synchronize(geye_ctx *ctx) {
  ARG_CHECK(ctx, "ctx is null");
  CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return GEYE_OK;
}

geye_status geye_ctx_enable_timing(geye_ctx *ctx, int enable) {
  ARG_CHECK(ctx, "ctx is null");
  if (enable && !ctx->ev[0])
    for (auto &e : ctx->ev) CUDA_TRY(cudaEventCreate(&e));
  ctx->timing = enable != 0;
  return GEYE_OK;
}

geye_status geye_ctx_stage_times(geye_ctx *ctx, float ms[GEYE_N_STAGES], double bytes[GEYE_N_STAGES],
                                 double *conv_flops, int *kernel_launches) {
  ARG_CHECK(ctx, "ctx is null");
  GEYE_TRY(collect_stage_times(ctx));
  for (int i = 0; i < GEYE_N_STAGES; i++) {
    if (ms) ms[i] = ctx->stage_ms[i];
    if (bytes) bytes[i] = ctx->stage_bytes[i];
  }
  if (conv_flops) *conv_flops = ctx->conv_flops;
  if (kernel_launches) *kernel_launches = ctx->launches;
  return GEYE_OK;
}

geye_status geye_debug_inject_fault(geye_ctx *ctx, const char *op, int nth) {
  ARG_CHECK(ctx, "ctx is null");
  ARG_CHECK(nth >= 0, "nth < 0");
  if (nth == 0 || !op) {
    ctx->inject_op.clear();
    ctx->inject_countdown = 0;
    return GEYE_OK;
  }
  std::string o(op);
  ARG_CHECK(o == "alloc" || o == "h2d" || o == "launch", "unknown fault point");
  ctx->inject_op = o;
  ctx->inject_countdown = nth;
  return GEYE_OK;
}

const char *geye_last_error(void);

geye_status geye_ctx_debug_counters(geye_ctx *ctx, long long *out, int n) {
  ARG_CHECK(ctx && out && n > 0 && n <= 64, "bad argument");
  ARG_CHECK(ctx->last_plan, "no run yet");
  CUDA_TRY(cudaMemcpyAsync(out, ctx->last_plan->d_small.as<int>() + 512, sizeof(long long) * n, cudaMemcpyDeviceToHost,
                           ctx->stream));
  int errw = 0;
  CUDA_TRY(cudaMemcpyAsync(&errw, ctx->last_plan->d_small.as<int>() + 128, sizeof(int), cudaMemcpyDeviceToHost,
                           ctx->stream));
  CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  if (n > 15) out[15] = errw;
  return GEYE_OK;
}

geye_status geye_score_map(geye_ctx *ctx, const geye_model *m, int level, int comp, float *out, int cap,
                           int dims[2]) {
  ARG_CHECK(ctx && m && dims, "null argument");
  ARG_CHECK(ctx->last_plan, "no run yet");
  const geye::Plan &P = *ctx->last_plan;
  for (auto &mp : P.models) {
    if (mp->model != m) continue;
    for (auto &S : mp->score_jobs) {
      if (S.level != level || S.comp != comp) continue;
      dims[0] = S.r0;
      dims[1] = S.r1;
      const size_t n = (size_t)S.r0 * S.r1;
      if (!out) return GEYE_OK;
      ARG_CHECK((size_t)cap >= n, "output buffer too small");
      CUDA_TRY(cudaMemcpyAsync(out, P.arena.as<float>() + S.score_off, sizeof(float) * n, cudaMemcpyDeviceToHost,
                               ctx->stream));
      CUDA_TRY(cudaStreamSynchronize(ctx->stream));
      return GEYE_OK;
    }
  }
  ARG_CHECK(false, "the last run has no score map for this model, level and component");
  return GEYE_ERR_ARG;
}

void geye_free(void *p) { free(p); }

// ---------------------------------------------------------------------------
// models
// ---------------------------------------------------------------------------
geye_status geye_model_load_csv(geye_ctx *ctx, const char *comp_csv, const char *root_csv, const char *part_csv,
                                float ratio, geye_model **out) {
  ARG_CHECK(ctx && comp_csv && root_csv && part_csv && out, "null argument");
  *out = nullptr;
  geye_model *m = new geye_model();
  geye_status s = parse_model_files(comp_csv, root_csv, part_csv, m->h);
  if (s != GEYE_OK) { delete m; return s; }
  m->h.ratio = ratio;
  m->ctx = ctx;
  m->id = ctx->next_model_id++;
  // filters: roots then parts, each [31][w][h] as read
  std::vector<float> all;
  std::vector<int> off;
  for (auto &f : m->h.rootfilter) { off.push_back((int)all.size()); all.insert(all.end(), f.begin(), f.end()); }
  for (auto &f : m->h.partfilter) { off.push_back((int)all.size()); all.insert(all.end(), f.begin(), f.end()); }
  m->filt_off = off;
  const int np = m->h.numpart[0];
  const int ML = 1 + 2 * (1 + np);
  std::vector<float> coef((size_t)m->h.numcomponent * 4 * ML, 0.f);
  for (int c = 0; c < m->h.numcomponent; c++)
    for (int j = 0; j < ML && j < (int)m->h.x1[c].size(); j++) {
      coef[((size_t)c * 4 + 0) * ML + j] = m->h.x1[c][j];
      coef[((size_t)c * 4 + 1) * ML + j] = m->h.y1[c][j];
      coef[((size_t)c * 4 + 2) * ML + j] = m->h.x2[c][j];
      coef[((size_t)c * 4 + 3) * ML + j] = m->h.y2[c][j];
    }
  cudaSetDevice(ctx->device);
  cudaError_t e = cudaMalloc(&m->d_filters, sizeof(float) * std::max<size_t>(all.size(), 1));
  if (e == cudaSuccess) e = cudaMalloc(&m->d_filt_off, sizeof(int) * std::max<size_t>(off.size(), 1));
  if (e == cudaSuccess) e = cudaMalloc(&m->d_coef, sizeof(float) * std::max<size_t>(coef.size(), 1));
  if (e == cudaSuccess) e = cudaMemcpy(m->d_filters, all.data(), sizeof(float) * all.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(m->d_filt_off, off.data(), sizeof(int) * off.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(m->d_coef, coef.data(), sizeof(float) * coef.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    set_error(std::string("model upload: ") + cudaGetErrorString(e));
    geye_model_free(m);
    return GEYE_ERR_CUDA;
  }
  ctx->models.insert(m);
  *out = m;
  return GEYE_OK;
}

geye_status geye_model_free(geye_model *m) {
  if (!m) return GEYE_OK;
  if (m->ctx) {
    m->ctx->models.erase(m);
    cudaSetDevice(m->ctx->device);
    cudaStreamSynchronize(m->ctx->stream);
    // drop every cached plan that refers to this model
    for (auto it = m->ctx->plans.begin(); it != m->ctx->plans.end();) {
      bool uses = false;
      for (auto &mp : it->second->models) uses |= mp->model == m;
      if (uses) {
        if (m->ctx->last_plan == it->second.get()) m->ctx->last_plan = nullptr;
        it = m->ctx->plans.erase(it);
      } else {
        ++it;
      }
    }
  }
  if (m->d_filters) cudaFree(m->d_filters);
  if (m->d_filt_off) cudaFree(m->d_filt_off);
  if (m->d_coef) cudaFree(m->d_coef);
  delete m;
  return GEYE_OK;
}

geye_status geye_model_info(const geye_model *m, int info[8]) {
  ARG_CHECK(m && info, "null argument");
  info[0] = m->h.numcomponent;
  info[1] = m->h.sbin;
  info[2] = m->h.interval;
  info[3] = m->h.numpart[0];
  info[4] = m->gl();
  info[5] = m->h.NoR;
  info[6] = m->h.NoP;
  info[7] = m->ini ? -1 : m->max_scale;
  return GEYE_OK;
}

geye_status geye_model_sym(const geye_model *m, int *rootsym, int *part_partner, int *part_sym) {
  ARG_CHECK(m, "model is null");
  for (int i = 0; rootsym && i < m->h.NoR; i++) rootsym[i] = 1;   // load_model.cpp:373
  for (int i = 0; i < m->h.NoP; i++) {
    const int p = i < (int)m->h.part_partner.size() ? m->h.part_partner[i] : 0;
    if (part_partner) part_partner[i] = p;                         // load_model.cpp:522
    if (part_sym) part_sym[i] = p == 0 ? 1 : 0;                    // load_model.cpp:523-524
  }
  return GEYE_OK;
}

geye_status geye_model_reset_scales(geye_model *m) {
  ARG_CHECK(m, "model is null");
  m->ini = true;
  m->max_scale = -1;
  return GEYE_OK;
}

// ---------------------------------------------------------------------------
// whole path
// ---------------------------------------------------------------------------
static geye_status fetch_model_result(geye_ctx *ctx, Plan &P, int mi, geye_result *out, int *D_out,
                                      float **kept_out) {
  int counts[4] = {0, 0, 0, 0};
  CUDA_TRY(cudaMemcpyAsync(&counts[0], P.d_small.as<int>() + mi, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CUDA_TRY(cudaMemcpyAsync(&counts[1], P.d_small.as<int>() + 32 + mi, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  if (mi == 0)
    CUDA_TRY(cudaMemcpyAsync(&counts[2], P.d_small.as<int>() + kSortLevelsUsed, 2 * sizeof(int),
                             cudaMemcpyDeviceToHost, ctx->stream));
  CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  const int D = counts[0], K = counts[1];
  if (mi == 0 && !P.from_features) note_sort_levels(ctx, P, counts[2], counts[3]);
  if (D_out) *D_out = D;
  P.last_D[mi] = D;
  P.last_K[mi] = K;
  if (out) {
    memset(out, 0, sizeof(*out));
    out->num = K;
    const size_t k = std::max(K, 1);
    out->point = (int *)malloc(sizeof(int) * 4 * k);
    out->or_point = (int *)malloc(sizeof(int) * 4 * k);
    out->type = (int *)malloc(sizeof(int) * k);
    out->scale = (float *)malloc(sizeof(float) * k);
    out->score = (float *)malloc(sizeof(float) * k);
    if (!out->point || !out->or_point || !out->type || !out->scale || !out->score) {
      geye_result_free(out);
      set_error("host allocation failed");
      return GEYE_ERR_NOMEM;
    }
    if (K > 0) {
      const int *res = P.d_result.as<int>() + (size_t)mi * P.max_cap * 11;
      CUDA_TRY(cudaMemcpyAsync(out->point, res, sizeof(int) * 4 * K, cudaMemcpyDeviceToHost, ctx->stream));
      CUDA_TRY(cudaMemcpyAsync(out->or_point, res + 4 * P.max_cap, sizeof(int) * 4 * K, cudaMemcpyDeviceToHost, ctx->stream));
      CUDA_TRY(cudaMemcpyAsync(out->type, res + 8 * P.max_cap, sizeof(int) * K, cudaMemcpyDeviceToHost, ctx->stream));
      CUDA_TRY(cudaMemcpyAsync(out->scale, res + 9 * P.max_cap, sizeof(float) * K, cudaMemcpyDeviceToHost, ctx->stream));
      CUDA_TRY(cudaMemcpyAsync(out->score, res + 10 * P.max_cap, sizeof(float) * K, cudaMemcpyDeviceToHost, ctx->stream));
    }
  }
  if (kept_out) {
    const int GL = P.models[mi]->model->gl();
    *kept_out = (float *)malloc(sizeof(float) * (size_t)std::max(K, 1) * GL);
    if (K > 0)
      CUDA_TRY(cudaMemcpyAsync(*kept_out, P.d_kept_boxes.as<float>() + (size_t)mi * P.max_cap * P.gl,
                               sizeof(float) * (size_t)K * GL, cudaMemcpyDeviceToHost, ctx->stream));
  }
  CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return GEYE_OK;
}

geye_status geye_detect_multi(geye_ctx *ctx, geye_model *const *models, int n_models, const uint8_t *bgr, int width,
                              int height, int width_step, float thresh, float overlap, float *const *a_scores,
                              geye_result *out) {
  ARG_CHECK(ctx && models && bgr && out, "null argument");
  ARG_CHECK(width >= 16 && height >= 16 && width_step >= 3 * width, "bad frame size");
  for (int i = 0; i < n_models; i++) MODEL_CHECK(models[i], ctx->device);
  CUDA_TRY(cudaSetDevice(ctx->device));
  Plan *P = nullptr;
  GEYE_TRY(frame_plan(ctx, models, n_models, width, height, &P));
  CUDA_TRY(cudaMemcpy2DAsync(P->d_bgr.p, (size_t)3 * width, bgr, width_step, (size_t)3 * width, height,
                             cudaMemcpyHostToDevice, ctx->stream));
  std::vector<const float *> init(n_models, nullptr);
  if (a_scores)
    for (int i = 0; i < n_models; i++) init[i] = a_scores[i];
  GEYE_TRY(run_frame(ctx, *P, P->d_bgr.as<uint8_t>(), 3 * width, thresh, overlap, init.data()));
  for (int i = 0; i < n_models; i++) {
    GEYE_TRY(fetch_model_result(ctx, *P, i, &out[i], nullptr, nullptr));
    if (a_scores && a_scores[i])
      CUDA_TRY(cudaMemcpyAsync(a_scores[i], P->d_ascore.as<float>() + (size_t)i * width * height,
                               sizeof(float) * (size_t)width * height, cudaMemcpyDeviceToHost, ctx->stream));
  }
  CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return GEYE_OK;
}

geye_status geye_car_detection(geye_ctx *ctx, geye_model *model, const uint8_t *bgr, int width, int height,
                               int width_step, float thresh, float overlap, float *a_score, geye_result *out) {
  geye_model *ms[1] = {model};
  float *as[1] = {a_score};
  return geye_detect_multi(ctx, ms, 1, bgr, width, height, width_step, thresh, overlap, a_score ? as : nullptr, out);
}

geye_status geye_result_free(geye_result *r) {
  if (!r) return GEYE_OK;
  free(r->point); free(r->or_point); free(r->type); free(r->scale); free(r->score);
  memset(r, 0, sizeof(*r));
  return GEYE_OK;
}

geye_status geye_detect_device(geye_ctx *ctx, geye_model *const *models, int n_models, const uint8_t *d_bgr,
                               int width, int height, float thresh, float overlap) {
  ARG_CHECK(ctx && models && d_bgr, "null argument");
  ARG_CHECK(width >= 16 && height >= 16, "bad frame size");
  for (int i = 0; i < n_models; i++) MODEL_CHECK(models[i], ctx->device);
  CUDA_TRY(cudaSetDevice(ctx->device));
  Plan *P = nullptr;
  GEYE_TRY(frame_plan(ctx, models, n_models, width, height, &P));
  return run_frame(ctx, *P, d_bgr, 3 * width, thresh, overlap, nullptr);
}

geye_status geye_fetch_result(geye_ctx *ctx, int model_index, geye_result *out, int *n_boxes_before_nms) {
  ARG_CHECK(ctx && ctx->last_plan, "no device-resident run to fetch");
  ARG_CHECK(model_index >= 0 && model_index < (int)ctx->last_plan->models.size(), "model index out of range");
  return fetch_model_result(ctx, *ctx->last_plan, model_index, out, n_boxes_before_nms, nullptr);
}

}  // extern "C"
