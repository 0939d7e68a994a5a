// stages.cu -- stage-level entry points of the C ABI: each one runs a single
// stage of the path on the device with the reference's host layouts, for
// callers that replace one reference function at a time and for stage parity.
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "runtime.h"

namespace geye {
geye_status run_pyramid(geye_ctx *ctx, Plan &P, const uint8_t *d_bgr, int width_step);
geye_status run_hog(geye_ctx *ctx, Plan &P);
geye_status run_conv(geye_ctx *ctx, Plan &P, ModelPlan &mp);
geye_status run_dt(geye_ctx *ctx, Plan &P, ModelPlan &mp);
geye_status run_score(geye_ctx *ctx, Plan &P, ModelPlan &mp, int mi, float thresh);
geye_status run_ascore(geye_ctx *ctx, Plan &P, ModelPlan &mp, int mi, float thresh, const float *h_init);
geye_status frame_plan(geye_ctx *ctx, geye_model *const *models, int n, int w, int h, Plan **out);
geye_status features_plan(geye_ctx *ctx, geye_model *model, const int *ftsize, const float *scales, int n_levels,
                          int img_w, int img_h, Plan **out);
void drop_plan(geye_ctx *ctx, Plan *P);
const char *last_error_cstr();
}  // namespace geye

using namespace geye;


// scoped temporary device buffers for one stage call
struct Scratch {
  geye_ctx *ctx;
  std::vector<DevBuf *> bufs;
  explicit Scratch(geye_ctx *c) : ctx(c) {}
  ~Scratch() {
    cudaStreamSynchronize(ctx->stream);
    for (auto *b : bufs) delete b;
  }
  template <class T> geye_status get(size_t n, T **out) {
    DevBuf *b = new DevBuf();
    bufs.push_back(b);
    GEYE_TRY(b->alloc(ctx, sizeof(T) * std::max<size_t>(n, 1)));
    *out = b->as<T>();
    return GEYE_OK;
  }
  template <class T> geye_status put(const T *h, size_t n, T **out) {
    GEYE_TRY(get(n, out));
    if (n) CUDA_TRY(cudaMemcpyAsync(*out, h, sizeof(T) * n, cudaMemcpyHostToDevice, ctx->stream));
    return GEYE_OK;
  }
};

static void taps(int sheight, int dheight, std::vector<int> &start, std::vector<int> &si, std::vector<float> &alpha) {
  // resize.cc:68-105, grouped by destination index (same as the plan builder)
  float scale = (float)dheight / (float)sheight;
  float invscale = (float)sheight / (float)dheight;
  for (int dy = 0; dy < dheight; dy++) {
    start.push_back((int)si.size());
    float fsy1 = dy * invscale;
    float fsy2 = fsy1 + invscale;
    int sy1 = (int)(fsy1 + 0.99);
    int sy2 = (int)fsy2;
    if (sy1 - fsy1 > 1e-3) { si.push_back(sy1 - 1); alpha.push_back((sy1 - fsy1) * scale); }
    for (int sy = sy1; sy < sy2; sy++) { si.push_back(sy); alpha.push_back(scale); }
    if (fsy2 - sy2 > 1e-3) { si.push_back(sy2); alpha.push_back((fsy2 - sy2) * scale); }
  }
  start.push_back((int)si.size());
  // float rounding could name a source row one past the end (the reference
  // would read past its buffer); keep every read inside the image
  for (auto &v : si) v = std::min(std::max(v, 0), sheight - 1);
}

extern "C" {

const char *geye_last_error(void) { return last_error_cstr(); }

geye_status geye_resize(geye_ctx *ctx, const float *src, const int *sdims, int *odims, float scale, float *dst) {
  ARG_CHECK(ctx && src && sdims && odims && dst, "null argument");
  const int h = sdims[0], w = sdims[1], c = sdims[2];
  ARG_CHECK(h > 0 && w > 0 && c == 3, "resize expects 3-channel planes");
  CUDA_TRY(cudaSetDevice(ctx->device));
  int oh, ow;
  if (scale == 1.0f) { oh = h; ow = w; }
  else { oh = (int)((float)h * scale + 0.5); ow = (int)((float)w * scale + 0.5); }
  odims[0] = oh; odims[1] = ow; odims[2] = c;
  if (scale == 1.0f) { memcpy(dst, src, sizeof(float) * (size_t)h * w * c); return GEYE_OK; }
  ARG_CHECK(oh > 0 && ow > 0, "resize to an empty image");
  Scratch S(ctx);
  std::vector<int> st, si;
  std::vector<float> al;
  taps(h, oh, st, si, al);
  const int h_start = (int)st.size(), h_tap = (int)si.size();
  taps(w, ow, st, si, al);
  float *arena;
  const size_t n_src = (size_t)3 * h * w, n_tmp = (size_t)3 * oh * w, n_dst = (size_t)3 * oh * ow;
  GEYE_TRY(S.get(n_src + n_tmp + n_dst, &arena));
  CUDA_TRY(cudaMemcpyAsync(arena, src, sizeof(float) * n_src, cudaMemcpyHostToDevice, ctx->stream));
  int *d_st, *d_si;
  float *d_al;
  GEYE_TRY(S.put(st.data(), st.size(), &d_st));
  GEYE_TRY(S.put(si.data(), si.size(), &d_si));
  GEYE_TRY(S.put(al.data(), al.size(), &d_al));
  ResizeJob jv{}, jh{};
  jv.src_off = 0; jv.dst_off = (int)n_src; jv.src_h = h; jv.src_w = w; jv.dst_h = oh; jv.dst_w = w;
  jv.tap_start_off = 0; jv.tap_off = 0;
  jh.src_off = (int)n_src; jh.dst_off = (int)(n_src + n_tmp); jh.src_h = oh; jh.src_w = w; jh.dst_h = oh; jh.dst_w = ow;
  // both tap tables share one start array whose entries index the whole si/alpha arrays
  jh.tap_start_off = h_start; jh.tap_off = 0;
  (void)h_tap;
  ResizeJob *d_jv, *d_jh;
  GEYE_TRY(S.put(&jv, 1, &d_jv));
  GEYE_TRY(S.put(&jh, 1, &d_jh));
  launch_resize_pass(d_jv, 1, w, 1, d_st, d_si, d_al, arena, ctx->stream);
  launch_resize_pass(d_jh, 1, ow, 0, d_st, d_si, d_al, arena, ctx->stream);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(dst, arena + n_src + n_tmp, sizeof(float) * n_dst, cudaMemcpyDeviceToHost, ctx->stream));
  CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return GEYE_OK;
}

geye_status geye_flip_feat(geye_ctx *ctx, const float *feat, const int *size, float **out) {
  ARG_CHECK(ctx && feat && size && out, "null argument");
  *out = nullptr;
  ARG_CHECK(size[2] == kFeat, "flip_feat takes 31 feature channels");   // the reference's ORD table has 31 entries
  ARG_CHECK(size[0] >= 0 && size[1] >= 0, "negative size");
  const size_t n = (size_t)size[0] * size[1] * kFeat;
  CUDA_TRY(cudaSetDevice(ctx->device));
  float *h = static_cast<float *>(calloc(n ? n : 1, sizeof(float)));
  ARG_CHECK(h, "host allocation failed");
  if (n == 0) { *out = h; return GEYE_OK; }
  geye_status st = GEYE_OK;
  {
    Scratch S(ctx);
    float *d_in, *d_out;
    if ((st = S.put(feat, n, &d_in)) == GEYE_OK && (st = S.get(n, &d_out)) == GEYE_OK) {
      launch_flip_feat(d_in, size[0], size[1], d_out, ctx->stream);
      cudaError_t e = cudaGetLastError();
      if (e == cudaSuccess) e = cudaMemcpyAsync(h, d_out, sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
      if (e != cudaSuccess) {
        set_error(std::string("flip_feat: ") + cudaGetErrorString(e));
        st = GEYE_ERR_CUDA;
      }
    }
  }
  if (st != GEYE_OK) { free(h); return st; }
  *out = h;
  return GEYE_OK;
}

geye_status geye_calc_feature(geye_ctx *ctx, const float *src, const int *isize, int sbin, int *ftsize, float *feat) {
  ARG_CHECK(ctx && src && isize && ftsize && feat, "null argument");
  ARG_CHECK(sbin >= 1 && sbin <= 8, "sbin must be in 1..8");
  const int h = isize[0], w = isize[1];
  ARG_CHECK(h >= 3 && w >= 3, "image too small");
  CUDA_TRY(cudaSetDevice(ctx->device));
  const int b0 = (int)floor((double)h / (double)sbin + 0.5), b1 = (int)floor((double)w / (double)sbin + 0.5);
  const int fs0 = std::max(b0 - 2, 0), fs1 = std::max(b1 - 2, 0);
  ftsize[0] = fs0;
  ftsize[1] = fs1;
  if (fs0 * fs1 == 0) return GEYE_OK;
  Scratch S(ctx);
  const size_t n_img = (size_t)3 * h * w;
  const size_t hist = ((n_img + 31) & ~size_t(31));
  const size_t feat_off = ((hist + (size_t)19 * b0 * b1 + 31) & ~size_t(31));
  HogPixJob X{};
  X.img_off = 0; X.h = h; X.w = w; X.xe = b1 * sbin - 1; X.ye = b0 * sbin - 1; X.Y = X.ye + 1;
  const size_t n_pix = (size_t)(X.xe + 1) * X.Y;
  const size_t mag_off = ((feat_off + (size_t)fs0 * fs1 * kFeatPad + 31) & ~size_t(31));
  const size_t bin_off = ((mag_off + n_pix + 31) & ~size_t(31));
  const size_t corner_off = ((bin_off + (n_pix + 3) / 4 + 31) & ~size_t(31));
  X.mag_off = (int)mag_off; X.bin_off = (int)bin_off;
  float *arena, *out;
  GEYE_TRY(S.get(corner_off + (size_t)(fs0 + 1) * (fs1 + 1), &arena));
  GEYE_TRY(S.get((size_t)fs0 * fs1 * kFeat, &out));
  CUDA_TRY(cudaMemcpyAsync(arena, src, sizeof(float) * n_img, cudaMemcpyHostToDevice, ctx->stream));
  HogJob J{};
  J.img_off = 0; J.h = h; J.w = w; J.sbin = sbin; J.b0 = b0; J.b1 = b1; J.hist_off = (int)hist;
  J.fs0 = fs0; J.fs1 = fs1; J.feat_off = (int)feat_off; J.feat16_off = -1; J.feat16lo_off = -1; J.fast = 0;
  J.mag_off = X.mag_off; J.bin_off = X.bin_off; J.pix_Y = X.Y; J.corner_off = (int)corner_off;
  HogJob *d_j;
  GEYE_TRY(S.put(&J, 1, &d_j));
  HogPixJob *d_x;
  GEYE_TRY(S.put(&X, 1, &d_x));
  std::vector<int2> vb;
  hog_vote_blocks(std::vector<HogJob>{J}, vb);
  int2 *d_vb;
  GEYE_TRY(S.put(vb.data(), vb.size(), &d_vb));
  launch_hog(d_j, 1, d_vb, (int)vb.size(), b0, b1, d_x, 1, X.xe, arena, nullptr, true, ctx->stream);
  launch_to_ref_layout(arena + feat_off, fs0, fs1, out, ctx->stream);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(feat, out, sizeof(float) * (size_t)fs0 * fs1 * kFeat, cudaMemcpyDeviceToHost, ctx->stream));
  CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return GEYE_OK;
}

geye_status geye_calc_f_pyramid(geye_ctx *ctx, geye_model *model, const uint8_t *bgr, int width, int height,
                                int width_step, int *n_levels, float **features, int **ftsize, float **scales) {
  ARG_CHECK(ctx && model && bgr && n_levels && features && ftsize && scales, "null argument");
  MODEL_CHECK(model, ctx->device);
  ARG_CHECK(width >= 16 && height >= 16 && width_step >= 3 * width, "bad frame size");
  CUDA_TRY(cudaSetDevice(ctx->device));
  geye_model *ms[1] = {model};
  Plan *P = nullptr;
  GEYE_TRY(frame_plan(ctx, ms, 1, width, height, &P));
  CUDA_TRY(cudaMemcpy2DAsync(P->d_bgr.p, (size_t)3 * width, bgr, width_step, (size_t)3 * width, height,
                             cudaMemcpyHostToDevice, ctx->stream));
  GEYE_TRY(run_pyramid(ctx, *P, P->d_bgr.as<uint8_t>(), 3 * width));
  GEYE_TRY(run_hog(ctx, *P));
  const int LEN = P->models[0]->LEN;
  size_t total = 0;
  for (int l = 0; l < LEN; l++) total += (size_t)P->lv[l].fs0 * P->lv[l].fs1 * kFeat;
  Scratch S(ctx);
  float *d_out;
  GEYE_TRY(S.get(total, &d_out));
  float *h_feat = (float *)malloc(sizeof(float) * std::max<size_t>(total, 1));
  int *h_fs = (int *)malloc(sizeof(int) * 2 * LEN);
  float *h_sc = (float *)malloc(sizeof(float) * LEN);
  if (!h_feat || !h_fs || !h_sc) {
    free(h_feat); free(h_fs); free(h_sc);
    set_error("host allocation failed");
    return GEYE_ERR_NOMEM;
  }
  size_t o = 0;
  for (int l = 0; l < LEN; l++) {
    const LevelInfo &L = P->lv[l];
    launch_to_ref_layout(P->arena.as<float>() + L.feat_off, L.fs0, L.fs1, d_out + o, ctx->stream);
    h_fs[2 * l] = L.fs0;
    h_fs[2 * l + 1] = L.fs1;
    h_sc[l] = L.scale;
    o += (size_t)L.fs0 * L.fs1 * kFeat;
  }
  cudaError_t e = cudaMemcpyAsync(h_feat, d_out, sizeof(float) * total, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    free(h_feat); free(h_fs); free(h_sc);
    set_error(std::string("pyramid readback: ") + cudaGetErrorString(e));
    return GEYE_ERR_CUDA;
  }
  *n_levels = LEN;
  *features = h_feat;
  *ftsize = h_fs;
  *scales = h_sc;
  return GEYE_OK;
}

geye_status geye_get_boxes(geye_ctx *ctx, geye_model *model, const float *features, const float *scales,
                           const int *ftsize, int n_levels, int img_width, int img_height, float thresh,
                           float *a_score, float **boxes, int *dnum) {
  ARG_CHECK(ctx && model && features && scales && ftsize && boxes && dnum, "null argument");
  MODEL_CHECK(model, ctx->device);
  ARG_CHECK(n_levels > model->h.interval, "need more levels than the interval");
  CUDA_TRY(cudaSetDevice(ctx->device));
  Plan *P = nullptr;
  GEYE_TRY(features_plan(ctx, model, ftsize, scales, n_levels, img_width, img_height, &P));
  struct Drop { geye_ctx *c; Plan *p; ~Drop() { cudaStreamSynchronize(c->stream); drop_plan(c, p); } } drop{ctx, P};
  size_t total = 0;
  for (int l = 0; l < n_levels; l++) total += (size_t)ftsize[2 * l] * ftsize[2 * l + 1] * kFeat;
  Scratch S(ctx);
  float *d_ref;
  GEYE_TRY(S.put(features, total, &d_ref));
  size_t o = 0;
  for (int l = 0; l < n_levels; l++) {
    const LevelInfo &L = P->lv[l];
    launch_from_ref_layout(d_ref + o, L.fs0, L.fs1, P->arena.as<float>() + L.feat_off, ctx->stream);
    o += (size_t)L.fs0 * L.fs1 * kFeat;
  }
  ModelPlan &mp = *P->models[0];
  CUDA_TRY(cudaMemsetAsync(P->d_small.p, 0, 4096, ctx->stream));
  GEYE_TRY(run_conv(ctx, *P, mp));
  GEYE_TRY(run_dt(ctx, *P, mp));
  GEYE_TRY(run_score(ctx, *P, mp, 0, thresh));
  if (a_score && img_width > 0 && img_height > 0) GEYE_TRY(run_ascore(ctx, *P, mp, 0, thresh, a_score));
  int D = 0;
  CUDA_TRY(cudaMemcpyAsync(&D, P->d_small.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  const int GL = model->gl();
  float *h = (float *)malloc(sizeof(float) * (size_t)std::max(D, 1) * GL);
  if (!h) { set_error("host allocation failed"); return GEYE_ERR_NOMEM; }
  cudaError_t e = cudaSuccess;
  if (D > 0) e = cudaMemcpyAsync(h, P->d_boxes.p, sizeof(float) * (size_t)D * GL, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess && a_score && img_width > 0 && img_height > 0)
    e = cudaMemcpyAsync(a_score, P->d_ascore.p, sizeof(float) * (size_t)img_width * img_height,
                        cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    free(h);
    set_error(std::string("get_boxes readback: ") + cudaGetErrorString(e));
    return GEYE_ERR_CUDA;
  }
  *boxes = h;
  *dnum = D;
  return GEYE_OK;
}

geye_status geye_nms(geye_ctx *ctx, const float *boxes, float overlap, int *num, int numpart0, float **out) {
  ARG_CHECK(ctx && num && out, "null argument");
  ARG_CHECK(numpart0 >= 0 && numpart0 <= kMaxParts, "numpart out of range");
  const int D = *num;
  const int GL = (numpart0 + 1) * 4 + 3;
  *out = nullptr;
  if (D <= 0) { *num = 0; return GEYE_OK; }   // nms.cpp:97 returns NULL for an empty list
  ARG_CHECK(boxes, "boxes is null");
  CUDA_TRY(cudaSetDevice(ctx->device));
  Scratch S(ctx);
  float *d_boxes, *d_out, *d_f;
  int *d_i, *d_small;
  GEYE_TRY(S.put(boxes, (size_t)D * GL, &d_boxes));
  GEYE_TRY(S.get((size_t)D * GL, &d_out));
  const int cap = (D + 31) & ~31;
  GEYE_TRY(S.get((size_t)cap * 6, &d_f));
  GEYE_TRY(S.get((size_t)cap * 5 + 64, &d_i));
  GEYE_TRY(S.get(64, &d_small));
  CUDA_TRY(cudaMemsetAsync(d_small, 0, 64 * sizeof(int), ctx->stream));
  CUDA_TRY(cudaMemcpyAsync(d_small, &D, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  launch_nms(d_boxes, d_small, 1, GL, overlap, cap, d_f, d_i, d_out, d_small + 1, d_small + 2, ctx->stream);
  CUDA_TRY(cudaGetLastError());
  int res[2] = {0, 0};
  CUDA_TRY(cudaMemcpyAsync(res, d_small + 1, 2 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  if (res[1]) { set_error("nms sort stack overflow"); return GEYE_ERR_UNSUPPORTED; }
  const int K = res[0];
  float *h = (float *)malloc(sizeof(float) * (size_t)std::max(K, 1) * GL);
  if (!h) { set_error("host allocation failed"); return GEYE_ERR_NOMEM; }
  if (K > 0) {
    cudaError_t e = cudaMemcpy(h, d_out, sizeof(float) * (size_t)K * GL, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) { free(h); set_error(cudaGetErrorString(e)); return GEYE_ERR_CUDA; }
  }
  *out = h;
  *num = K;
  return GEYE_OK;
}

geye_status geye_get_new_rects(geye_ctx *ctx, const geye_model *model, const float *boxes, int num, int img_width,
                               int img_height, geye_result *out) {
  ARG_CHECK(ctx && model && out, "null argument");
  ARG_CHECK(num >= 0, "num < 0");
  MODEL_CHECK(model, ctx->device);
  memset(out, 0, sizeof(*out));
  const size_t k = std::max(num, 1);
  out->num = num;
  out->point = (int *)malloc(sizeof(int) * 4 * k);
  out->or_point = (int *)malloc(sizeof(int) * 4 * k);
  out->type = (int *)malloc(sizeof(int) * k);
  out->scale = (float *)malloc(sizeof(float) * k);
  out->score = (float *)malloc(sizeof(float) * k);
  if (num == 0) return GEYE_OK;
  ARG_CHECK(boxes, "boxes is null");
  CUDA_TRY(cudaSetDevice(ctx->device));
  const int GL = model->gl();
  Scratch S(ctx);
  float *d_boxes;
  int *d_num, *d_res;
  GEYE_TRY(S.put(boxes, (size_t)num * GL, &d_boxes));
  GEYE_TRY(S.put(&num, 1, &d_num));
  GEYE_TRY(S.get((size_t)num * 11, &d_res));
  launch_new_rects(d_boxes, d_num, GL, model->h.numpart[0], model->d_coef, img_width, img_height, model->h.ratio,
                   d_res, d_res + 4 * num, d_res + 8 * num, reinterpret_cast<float *>(d_res + 9 * num),
                   reinterpret_cast<float *>(d_res + 10 * num), ctx->stream);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(out->point, d_res, sizeof(int) * 4 * num, cudaMemcpyDeviceToHost, ctx->stream));
  CUDA_TRY(cudaMemcpyAsync(out->or_point, d_res + 4 * num, sizeof(int) * 4 * num, cudaMemcpyDeviceToHost, ctx->stream));
  CUDA_TRY(cudaMemcpyAsync(out->type, d_res + 8 * num, sizeof(int) * num, cudaMemcpyDeviceToHost, ctx->stream));
  CUDA_TRY(cudaMemcpyAsync(out->scale, d_res + 9 * num, sizeof(float) * num, cudaMemcpyDeviceToHost, ctx->stream));
  CUDA_TRY(cudaMemcpyAsync(out->score, d_res + 10 * num, sizeof(float) * num, cudaMemcpyDeviceToHost, ctx->stream));
  CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return GEYE_OK;
}

geye_status geye_dt(geye_ctx *ctx, const float *vals, float ax, float bx, float ay, float by, const int *dims,
                    float *M, int *Ix, int *Iy) {
  ARG_CHECK(ctx && vals && dims && M && Ix && Iy, "null argument");
  const int d0 = dims[0], d1 = dims[1];
  ARG_CHECK(d0 > 0 && d1 > 0 && d0 <= 1100 && d1 <= 1100, "dims out of range (1..1100)");
  CUDA_TRY(cudaSetDevice(ctx->device));
  const size_t n = (size_t)d0 * d1;
  const size_t np = (n + 31) & ~size_t(31);
  Scratch S(ctx);
  float *arena;
  GEYE_TRY(S.get(np * 6, &arena));
  CUDA_TRY(cudaMemcpyAsync(arena, vals, sizeof(float) * n, cudaMemcpyHostToDevice, ctx->stream));
  DtJob J{};
  J.in_off = 0; J.d0 = d0; J.d1 = d1;
  J.tmpM_off = (int)np; J.tmpI_off = (int)(2 * np); J.M_off = (int)(3 * np); J.Ix_off = (int)(4 * np); J.Iy_off = (int)(5 * np);
  J.ax = ax; J.bx = bx; J.ay = ay; J.by = by; J.negate = 0;
  DtJob *d_j;
  GEYE_TRY(S.put(&J, 1, &d_j));
  std::vector<int2> b1, b2;
  dt_block_lists(std::vector<DtJob>{J}, b1, b2, kDtElems);
  int2 *d_b1, *d_b2;
  GEYE_TRY(S.put(b1.data(), b1.size(), &d_b1));
  GEYE_TRY(S.put(b2.data(), b2.size(), &d_b2));
  launch_dt(d_j, d_b1, (int)b1.size(), d_b2, (int)b2.size(), d0, d1, arena, reinterpret_cast<int *>(arena),
            ctx->d_diag.as<int>(), kDtElems, ctx->stream);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(M, arena + 3 * np, sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->stream));
  CUDA_TRY(cudaMemcpyAsync(Ix, arena + 4 * np, sizeof(int) * n, cudaMemcpyDeviceToHost, ctx->stream));
  CUDA_TRY(cudaMemcpyAsync(Iy, arena + 5 * np, sizeof(int) * n, cudaMemcpyDeviceToHost, ctx->stream));
  CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return GEYE_OK;
}

geye_status geye_fconv(geye_ctx *ctx, const float *feat, const int *a_dims, const float *const *filters,
                       const int *b_dims, int n_filters, float *out) {
  ARG_CHECK(ctx && feat && a_dims && filters && b_dims && out && n_filters > 0, "null argument");
  const int a0 = a_dims[0], a1 = a_dims[1];
  ARG_CHECK(a0 > 0 && a1 > 0, "empty feature map");
  CUDA_TRY(cudaSetDevice(ctx->device));
  Scratch S(ctx);
  const size_t cells = (size_t)a0 * a1;
  float *d_ref, *arena, *d_filt;
  int *d_off;
  GEYE_TRY(S.put(feat, cells * kFeat, &d_ref));
  std::vector<float> all;
  std::vector<int> off;
  std::vector<ConvJob> jobs;
  size_t out_words = 0;
  int mb0 = 0, mb1 = 0, mty = 0, mtx = 0;
  for (int i = 0; i < n_filters; i++) {
    const int b0 = b_dims[2 * i], b1 = b_dims[2 * i + 1];
    ARG_CHECK(b0 > 0 && b1 > 0 && b0 <= a0 && b1 <= a1, "filter larger than the feature map");
    off.push_back((int)all.size());
    all.insert(all.end(), filters[i], filters[i] + (size_t)b0 * b1 * kFeat);
    ConvJob J{};
    J.feat_off = 0; J.a0 = a0; J.a1 = a1; J.filt_base = i; J.n_filt = 1; J.b0 = b0; J.b1 = b1;
    J.c0 = a0 - b0 + 1; J.c1 = a1 - b1 + 1;
    J.out_off = (int)(cells * kFeatPad + out_words);
    J.tiles_y = (J.c0 + 31) / 32; J.tiles_x = (J.c1 + 15) / 16;
    out_words += (size_t)J.c0 * J.c1;
    mb0 = std::max(mb0, b0); mb1 = std::max(mb1, b1);
    mty = std::max(mty, J.tiles_y); mtx = std::max(mtx, J.tiles_x);
    jobs.push_back(J);
  }
  GEYE_TRY(S.get(cells * kFeatPad + out_words, &arena));
  GEYE_TRY(S.put(all.data(), all.size(), &d_filt));
  GEYE_TRY(S.put(off.data(), off.size(), &d_off));
  ConvJob *d_jobs;
  GEYE_TRY(S.put(jobs.data(), jobs.size(), &d_jobs));
  launch_from_ref_layout(d_ref, a0, a1, arena, ctx->stream);
  if (ctx->conv_mode != GEYE_CONV_FP32) {
    std::vector<int> out_off;
    for (auto &J : jobs) out_off.push_back(J.out_off);
    std::vector<std::unique_ptr<DevBuf>> tmp;
    GEYE_TRY(conv_tc_maps(ctx, arena, a0, a1, filters, b_dims, n_filters, arena, out_off, tmp));
  } else {
    launch_conv_fp32(d_jobs, (int)jobs.size(), mty, mtx, d_filt, d_off, arena, arena, mb0, mb1, 1, ctx->stream);
  }
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(out, arena + cells * kFeatPad, sizeof(float) * out_words, cudaMemcpyDeviceToHost,
                           ctx->stream));
  CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return GEYE_OK;
}

}  // extern "C"
