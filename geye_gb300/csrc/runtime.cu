// runtime.cu -- host runtime of libgeye_dpm: models, plans and the pipeline.
//
// Host-side arithmetic that sizes the pyramid (scale schedule, resize output
// sizes, tap tables, feature sizes, level skipping) repeats the reference's C
// expressions with the same float/double types; this file is compiled with
// -ffp-contract=off so the host compiler fuses nothing either.
//   ini_scales           CAR_TRACKING/featurepyramid.cpp:174-239
//   pyramid schedule     CAR_TRACKING/featurepyramid.cpp.org:547-661
//   resize sizes / taps  CAR_TRACKING/resize.cc:68-160
//   feature sizes        CAR_TRACKING/featurepyramid.cpp:277-281
//   level skip, conv and part-map sizes  CAR_TRACKING/fconvsMT.cpp:420-470
//   score assembly inputs                CAR_TRACKING/get_boxes.cpp:1000-1360
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <sstream>

#include "runtime.h"

namespace geye {

static thread_local std::string g_err;
void set_error(const std::string &msg) { g_err = msg; }



static bool injected(geye_ctx *ctx, const char *op) {
  if (!ctx || ctx->inject_countdown <= 0 || ctx->inject_op != op) return false;
  if (--ctx->inject_countdown == 0) {
    ctx->inject_op.clear();
    return true;
  }
  return false;
}

DevBuf::~DevBuf() { release(); }
void DevBuf::release() {
  if (p) cudaFree(p);
  p = nullptr;
  bytes = 0;
}
geye_status DevBuf::alloc(geye_ctx *ctx, size_t n) {
  if (n <= bytes && p) return GEYE_OK;
  release();
  if (injected(ctx, "alloc")) {
    set_error("injected allocation failure");
    return GEYE_ERR_INJECTED;
  }
  if (n == 0) n = 16;
  cudaError_t e = cudaMalloc(&p, n);
  if (e != cudaSuccess) {
    p = nullptr;
    set_error(std::string("cudaMalloc: ") + cudaGetErrorString(e));
    return GEYE_ERR_NOMEM;
  }
  bytes = n;
  return GEYE_OK;
}

geye_status upload_bytes(geye_ctx *ctx, DevBuf &buf, const void *src, size_t n) {
  GEYE_TRY(buf.alloc(ctx, std::max<size_t>(n, 16)));
  if (n) CUDA_TRY(cudaMemcpyAsync(buf.p, src, n, cudaMemcpyHostToDevice, ctx->stream));
  return GEYE_OK;
}

template <class T>
static geye_status upload(geye_ctx *ctx, DevBuf &buf, const std::vector<T> &v) {
  GEYE_TRY(buf.alloc(ctx, sizeof(T) * std::max<size_t>(v.size(), 1)));
  if (!v.empty()) {
    if (injected(ctx, "h2d")) {
      set_error("injected host-to-device copy failure");
      return GEYE_ERR_INJECTED;
    }
    CUDA_TRY(cudaMemcpyAsync(buf.p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, ctx->stream));
  }
  return GEYE_OK;
}

// ----------------------------------------------------------------------------
// model CSV (load_model.cpp:57-558); values are read with fscanf("%f,") like
// the reference so every weight is the same float
// ----------------------------------------------------------------------------
static int scan_f(FILE *f, float *v) { return fscanf(f, "%f,", v) == 1 ? 0 : -1; }

static geye_status parse_model(const char *comp, const char *root, const char *part, HostModel &m) {
  FILE *f = fopen(comp, "r");
  if (!f) { set_error(std::string("model component file not found: ") + comp); return GEYE_ERR_MODEL; }
  float t1, t2, t3, t4;
  int bad = 0;
  bad |= scan_f(f, &t1); m.numcomponent = (int)t1;
  bad |= scan_f(f, &t1); m.sbin = (int)t1;
  bad |= scan_f(f, &t1); m.interval = (int)t1;
  bad |= scan_f(f, &t1); m.max_Y = (int)t1;
  bad |= scan_f(f, &t1); m.max_X = (int)t1;
  const int nc = m.numcomponent;
  if (bad || nc <= 0 || nc > 64 || m.sbin <= 0 || m.interval <= 0) { fclose(f); set_error("bad component header"); return GEYE_ERR_MODEL; }
  m.ridx.resize(nc); m.oidx.resize(nc); m.offw.resize(nc); m.rsize.resize(2 * nc); m.numpart.resize(nc);
  m.pidx.resize(nc); m.didx.resize(nc); m.psize.resize(nc);
  for (int c = 0; c < nc; c++) {
    bad |= scan_f(f, &t1); m.ridx[c] = (int)t1 - 1;
    bad |= scan_f(f, &t1); m.oidx[c] = (int)t1 - 1;
    bad |= scan_f(f, &t1); m.offw[c] = t1;
    bad |= scan_f(f, &t1); bad |= scan_f(f, &t2);
    m.rsize[2 * c] = (int)t1; m.rsize[2 * c + 1] = (int)t2;
    bad |= scan_f(f, &t1); m.numpart[c] = (int)t1;
    const int np = m.numpart[c];
    if (bad || np < 0 || np > kMaxParts) { fclose(f); set_error("bad component record"); return GEYE_ERR_MODEL; }
    m.pidx[c].resize(np); m.didx[c].resize(np); m.psize[c].resize(2 * np);
    for (int k = 0; k < np; k++) {
      bad |= scan_f(f, &t1); m.pidx[c][k] = (int)t1 - 1;
      bad |= scan_f(f, &t1); m.didx[c][k] = (int)t1 - 1;
      bad |= scan_f(f, &t1); bad |= scan_f(f, &t2);
      m.psize[c][2 * k] = (int)t1; m.psize[c][2 * k + 1] = (int)t2;
    }
  }
  bad |= scan_f(f, &t1);
  m.DefL = (int)t1;
  if (bad || m.DefL < 0 || m.DefL > 4096) { fclose(f); set_error("bad deformation count"); return GEYE_ERR_MODEL; }
  m.def.resize(4 * m.DefL); m.anchor.resize(2 * m.DefL);
  for (int k = 0; k < m.DefL; k++) {
    bad |= scan_f(f, &t1); bad |= scan_f(f, &t2); bad |= scan_f(f, &t3); bad |= scan_f(f, &t4);
    m.def[4 * k] = t1; m.def[4 * k + 1] = t2; m.def[4 * k + 2] = t3; m.def[4 * k + 3] = t4;
    bad |= scan_f(f, &t1); bad |= scan_f(f, &t2);
    m.anchor[2 * k] = (int)t1; m.anchor[2 * k + 1] = (int)t2;
  }
  m.x1.resize(nc); m.y1.resize(nc); m.x2.resize(nc); m.y2.resize(nc);
  for (int c = 0; c < nc; c++) {
    const int GL = 1 + 2 * (1 + m.numpart[c]);
    for (auto *v : {&m.x1[c], &m.y1[c], &m.x2[c], &m.y2[c]}) {
      v->resize(GL);
      for (int j = 0; j < GL; j++) { bad |= scan_f(f, &t1); (*v)[j] = t1; }
    }
  }
  fclose(f);
  if (bad) { set_error("truncated component file"); return GEYE_ERR_MODEL; }
  // load_model.cpp:552-553: the pad is forced to zero
  m.padx = 0;
  m.pady = 0;

  auto read_filters = [&](const char *path, bool parts, int &n, std::vector<int> &sz,
                          std::vector<std::vector<float>> &w) -> geye_status {
    FILE *g = fopen(path, "r");
    if (!g) { set_error(std::string("filter file not found: ") + path); return GEYE_ERR_MODEL; }
    float a, b, c;
    int bd = scan_f(g, &a);
    n = (int)a;
    if (bd || n < 0 || n > 4096) { fclose(g); set_error("bad filter count"); return GEYE_ERR_MODEL; }
    sz.resize(3 * n); w.resize(n);
    if (parts) m.part_partner.resize(n);
    for (int i = 0; i < n; i++) {
      bd |= scan_f(g, &a); bd |= scan_f(g, &b); bd |= scan_f(g, &c);
      sz[3 * i] = (int)a; sz[3 * i + 1] = (int)b; sz[3 * i + 2] = (int)c;
      const int num = (int)a * (int)b * (int)c;
      if (bd || num <= 0 || (int)c != kFeat) { fclose(g); set_error("bad filter size"); return GEYE_ERR_MODEL; }
      w[i].resize(num);
      for (int j = 0; j < num; j++) { bd |= scan_f(g, &a); w[i][j] = a; }
      if (parts) { bd |= scan_f(g, &a); m.part_partner[i] = (int)a; }
    }
    fclose(g);
    if (bd) { set_error("truncated filter file"); return GEYE_ERR_MODEL; }
    return GEYE_OK;
  };
  GEYE_TRY(read_filters(root, false, m.NoR, m.root_size, m.rootfilter));
  GEYE_TRY(read_filters(part, true, m.NoP, m.part_size, m.partfilter));
  // shapes the kernels assume
  if (m.NoR < nc) { set_error("fewer root filters than components"); return GEYE_ERR_UNSUPPORTED; }
  for (int c = 1; c < nc; c++)
    if (m.numpart[c] != m.numpart[0]) {
      // get_boxes.cpp:1746 sizes every record with numpart[0]
      set_error("components with different part counts");
      return GEYE_ERR_UNSUPPORTED;
    }
  for (int c = 0; c < nc; c++)
    for (int k = 0; k < m.numpart[c]; k++)
      if (m.pidx[c][k] < 0 || m.pidx[c][k] >= m.NoP || m.didx[c][k] < 0 || m.didx[c][k] >= m.DefL) {
        set_error("part or deformation index out of range");
        return GEYE_ERR_MODEL;
      }
  if (m.sbin > 8) { set_error("sbin above 8 is not supported by the HOG kernel"); return GEYE_ERR_UNSUPPORTED; }
  return GEYE_OK;
}

// ----------------------------------------------------------------------------
// scale schedule and sizes
// ----------------------------------------------------------------------------
static int max_scale_for(const HostModel &m, int width, int height) {
  const int sbin = m.sbin, interval = m.interval;
  const float sc = pow(2.0, (1 / (double)interval));
  int max_scale = 36;
  const int L_NUM = interval + max_scale;
  float MRY = (float)m.rsize[0];
  float MRX = (float)m.rsize[1];
  for (int kk = 1; kk < m.numcomponent; kk++) {
    if (m.rsize[kk * 2] < MRY) MRY = m.rsize[kk * 2];
    if (m.rsize[kk * 2 + 1] < MRX) MRX = m.rsize[kk * 2 + 1];
  }
  MRY /= 2;
  MRX /= 2;
  float h = (float)height / (float)sbin;
  float w = (float)width / (float)sbin;
  float sc_step = 1 / sc;
  for (int kk = 0; kk < L_NUM; kk++) {
    h *= sc_step;
    w *= sc_step;
    if (h < MRY || w < MRX) { max_scale = kk - interval - 1; break; }
  }
  if (max_scale < interval) max_scale = interval;
  return max_scale;
}

static void resize_dims(int h, int w, float scale, int &oh, int &ow) {
  if (scale == 1.0f) { oh = h; ow = w; return; }
  oh = (int)((float)h * scale + 0.5);
  ow = (int)((float)w * scale + 0.5);
}

// taps of one 1-D pass (resize.cc:68-105), grouped by destination index
static void build_taps(int sheight, int dheight, std::vector<int> &start, std::vector<int> &si,
                       std::vector<float> &alpha) {
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

static void feature_dims(int h, int w, int sbin, int &b0, int &b1, int &fs0, int &fs1) {
  b0 = (int)floor((double)h / (double)sbin + 0.5);
  b1 = (int)floor((double)w / (double)sbin + 0.5);
  fs0 = std::max(b0 - 2, 0);
  fs1 = std::max(b1 - 2, 0);
}

// ----------------------------------------------------------------------------
// plan construction
// ----------------------------------------------------------------------------
static geye_status build_model_plan(geye_ctx *ctx, Plan &P, geye_model *mdl, int LEN_m, ArenaAlloc &A) {
  const HostModel &m = mdl->h;
  auto mp = std::make_unique<ModelPlan>();
  mp->model = mdl;
  mp->LEN = LEN_m;
  const int interval = m.interval, NoC = m.numcomponent, NoP = m.NoP;
  mp->root_map_off.assign((size_t)LEN_m * NoC, -1);
  mp->root_r0.assign((size_t)LEN_m * NoC, 0);
  mp->root_r1.assign((size_t)LEN_m * NoC, 0);
  mp->part_map_off.assign((size_t)LEN_m * std::max(NoP, 1), -1);
  mp->part_d0.assign((size_t)LEN_m * std::max(NoP, 1), 0);
  mp->part_d1.assign((size_t)LEN_m * std::max(NoP, 1), 0);
  mp->skipped.assign(LEN_m, 1);
  int filt_parts_base = m.NoR;
  for (int level = interval; level < LEN_m; level++) {
    const LevelInfo &L = P.lv[level];
    if (L.fs0 + 2 * m.pady < m.max_Y || L.fs1 + 2 * m.padx < m.max_X) continue;   // fconvsMT.cpp:425
    mp->skipped[level] = 0;
    // roots: filter c for component c, grouped by size
    std::vector<int> done(NoC, 0);
    for (int c = 0; c < NoC; c++) {
      if (done[c]) continue;
      const int b0 = m.root_size[3 * c], b1 = m.root_size[3 * c + 1];
      std::vector<int> grp;
      for (int c2 = c; c2 < NoC && (int)grp.size() < 8; c2++)
        if (!done[c2] && m.root_size[3 * c2] == b0 && m.root_size[3 * c2 + 1] == b1 && (grp.empty() || c2 == grp.back() + 1))
          grp.push_back(c2);
      const int c0 = L.fs0 - b0 + 1, c1 = L.fs1 - b1 + 1;
      if (c0 < 1 || c1 < 1) { set_error("root filter larger than a kept feature level"); return GEYE_ERR_UNSUPPORTED; }
      ConvJob J{};
      J.feat_off = L.feat_off; J.a0 = L.fs0; J.a1 = L.fs1;
      J.filt_base = grp[0]; J.n_filt = (int)grp.size(); J.b0 = b0; J.b1 = b1; J.c0 = c0; J.c1 = c1;
      J.out_off = A.take((size_t)c0 * c1 * grp.size());
      J.tiles_y = (c0 + 31) / 32; J.tiles_x = (c1 + 15) / 16;
      for (size_t g = 0; g < grp.size(); g++) {
        const int cc = grp[g];
        done[cc] = 1;
        mp->root_map_off[level * NoC + cc] = J.out_off + (int)g * c0 * c1;
        mp->root_r0[level * NoC + cc] = c0;
        mp->root_r1[level * NoC + cc] = c1;
        mp->conv_flops += 2.0 * c0 * c1 * b0 * b1 * kFeat;
      }
      mp->root_jobs.push_back(J);
      mp->root_max_b0 = std::max(mp->root_max_b0, b0);
      mp->root_max_b1 = std::max(mp->root_max_b1, b1);
      mp->root_max_g = std::max(mp->root_max_g, J.n_filt);
      mp->root_tiles_y = std::max(mp->root_tiles_y, J.tiles_y);
      mp->root_tiles_x = std::max(mp->root_tiles_x, J.tiles_x);
      mp->conv_bytes += 128.0 * L.fs0 * L.fs1 + 4.0 * c0 * c1 * grp.size();
    }
    // parts at L = level - interval
    const int Lv = level - interval;
    const LevelInfo &PL = P.lv[Lv];
    std::vector<int> pdone(NoP, 0);
    for (int p = 0; p < NoP; p++) {
      if (pdone[p]) continue;
      const int b0 = m.part_size[3 * p], b1 = m.part_size[3 * p + 1];
      std::vector<int> grp;
      for (int p2 = p; p2 < NoP && (int)grp.size() < 8; p2++)
        if (!pdone[p2] && m.part_size[3 * p2] == b0 && m.part_size[3 * p2 + 1] == b1 && (grp.empty() || p2 == grp.back() + 1))
          grp.push_back(p2);
      const int c0 = PL.fs0 - b0 + 1, c1 = PL.fs1 - b1 + 1;
      if (c0 < 1 || c1 < 1) { set_error("part filter larger than its feature level"); return GEYE_ERR_UNSUPPORTED; }
      ConvJob J{};
      J.feat_off = PL.feat_off; J.a0 = PL.fs0; J.a1 = PL.fs1;
      J.filt_base = filt_parts_base + grp[0]; J.n_filt = (int)grp.size(); J.b0 = b0; J.b1 = b1; J.c0 = c0; J.c1 = c1;
      J.out_off = A.take((size_t)c0 * c1 * grp.size());
      J.tiles_y = (c0 + 31) / 32; J.tiles_x = (c1 + 15) / 16;
      for (size_t g = 0; g < grp.size(); g++) {
        const int pp = grp[g];
        pdone[pp] = 1;
        mp->part_map_off[Lv * NoP + pp] = J.out_off + (int)g * c0 * c1;
        mp->part_d0[Lv * NoP + pp] = c0;
        mp->part_d1[Lv * NoP + pp] = c1;
        mp->conv_flops += 2.0 * c0 * c1 * b0 * b1 * kFeat;
      }
      mp->part_jobs.push_back(J);
      mp->part_max_b0 = std::max(mp->part_max_b0, b0);
      mp->part_max_b1 = std::max(mp->part_max_b1, b1);
      mp->part_max_g = std::max(mp->part_max_g, J.n_filt);
      mp->part_tiles_y = std::max(mp->part_tiles_y, J.tiles_y);
      mp->part_tiles_x = std::max(mp->part_tiles_x, J.tiles_x);
      mp->conv_bytes += 128.0 * PL.fs0 * PL.fs1 / std::max(1.0, (double)NoP / grp.size()) + 4.0 * c0 * c1 * grp.size();
    }
    // DT per (component, part) and score jobs per component
    for (int c = 0; c < NoC; c++) {
      ScoreJob S{};
      const int r0 = mp->root_r0[level * NoC + c], r1 = mp->root_r1[level * NoC + c];
      S.root_off = mp->root_map_off[level * NoC + c];
      S.r0 = r0; S.r1 = r1;
      S.off = m.offw[m.ridx[c]];
      S.score_off = A.take((size_t)r0 * r1);
      S.np = m.numpart[c];
      S.comp = c;
      S.level = level;
      S.scale = (float)m.sbin / P.lv[level].scale;
      S.rsize0 = m.rsize[2 * c];
      S.rsize1 = m.rsize[2 * c + 1];
      int block_pad = (int)(S.scale / 2.0);
      S.RY = (int)((float)S.rsize0 * S.scale / 2.0 - 1.0 + block_pad);
      S.RX = (int)((float)S.rsize1 * S.scale / 2.0 - 1.0 + block_pad);
      mp->cap += r0 * r1;
      mp->score_max_r = std::max(mp->score_max_r, r0 * r1);
      for (int k = 0; k < S.np; k++) {
        const int p = m.pidx[c][k], di = m.didx[c][k];
        const int d0 = mp->part_d0[Lv * NoP + p], d1 = mp->part_d1[Lv * NoP + p];
        DtJob D{};
        D.in_off = mp->part_map_off[Lv * NoP + p];
        D.d0 = d0; D.d1 = d1;
        D.tmpM_off = A.take((size_t)d0 * d1);
        D.tmpI_off = A.take((size_t)d0 * d1);
        D.ax = m.def[4 * di]; D.bx = m.def[4 * di + 1]; D.ay = m.def[4 * di + 2]; D.by = m.def[4 * di + 3];
        D.negate = 1;
        // the score sum reads M at (anchor_y + 2y, anchor_x + 2x) (dt.cpp:38-55); the
        // part boxes read Ix/Iy one row and column before (get_boxes.cpp:243-258)
        D.samp_m = 1;
        D.par_y = m.anchor[di * 2 + 1] & 1;
        D.par_x = m.anchor[di * 2] & 1;
        {   // the box probes (anchor - 1 + 2k) all inside the map: no linear wrap, no entry-0 reads
          const int ay0 = m.anchor[di * 2 + 1] - 1, ax0 = m.anchor[di * 2] - 1;
          D.samp_i = ay0 >= 0 && ax0 >= 0 && ay0 + 2 * (r0 - 1) < d0 && ax0 + 2 * (r1 - 1) < d1;
        }
        // the sampled entries, stored compactly (a quarter of the map each)
        const int qy = 1 - D.par_y, qx = 1 - D.par_x;
        D.cm0 = (d0 - D.par_y + 1) >> 1;
        D.ci0 = D.samp_i ? (d0 - qy + 1) >> 1 : 0;
        D.M_off = A.take((size_t)D.cm0 * ((d1 - D.par_x + 1) >> 1));
        const size_t ni = D.samp_i ? (size_t)D.ci0 * ((d1 - qx + 1) >> 1) : (size_t)d0 * d1;
        D.Ix_off = A.take(ni);
        D.Iy_off = A.take(ni);
        mp->dt_jobs.push_back(D);
        mp->dt_max_d0 = std::max(mp->dt_max_d0, d0);
        mp->dt_max_d1 = std::max(mp->dt_max_d1, d1);
        mp->dt_bytes += 16.0 * d0 * d1;
        S.part_M[k] = D.M_off; S.part_Ix[k] = D.Ix_off; S.part_Iy[k] = D.Iy_off;
        S.part_d0[k] = d0; S.part_d1[k] = d1;
        S.part_cm0[k] = D.cm0; S.part_ci0[k] = D.ci0;
        S.ax[k] = m.anchor[di * 2] + 1;
        S.ay[k] = m.anchor[di * 2 + 1] + 1;
        S.psize0[k] = m.psize[c][2 * k];
        S.psize1[k] = m.psize[c][2 * k + 1];
        // add_part_calculation reads M up to (ax-1+2(r1-1), ay-1+2(r0-1)); the kernels trust it
        const int xmax = S.ax[k] - 1 + 2 * (r1 - 1), ymax = S.ay[k] - 1 + 2 * (r0 - 1);
        if (S.ax[k] - 1 < 0 || S.ay[k] - 1 < 0 || xmax >= d1 || ymax >= d0) {
          set_error("part anchor places a part outside its score map");
          return GEYE_ERR_UNSUPPORTED;
        }
      }
      mp->score_bytes += 8.0 * r0 * r1 + 4.0 * S.np * r0 * r1;
      mp->score_jobs.push_back(S);
    }
  }
  if (mp->dt_max_d0 > 1100 || mp->dt_max_d1 > 1100) { set_error("frame too large for the DT kernels"); return GEYE_ERR_UNSUPPORTED; }
  GEYE_TRY(upload(ctx, mp->d_root_jobs, mp->root_jobs));
  GEYE_TRY(upload(ctx, mp->d_part_jobs, mp->part_jobs));
  GEYE_TRY(upload(ctx, mp->d_dt_jobs, mp->dt_jobs));
  {
    std::vector<int2> b1, b2;
    dt_block_lists(mp->dt_jobs, b1, b2, mp->dt_elems);
    mp->dt_nblocks1 = (int)b1.size();
    mp->dt_nblocks2 = (int)b2.size();
    GEYE_TRY(upload(ctx, mp->d_dt_blocks1, b1));
    GEYE_TRY(upload(ctx, mp->d_dt_blocks2, b2));
  }
  GEYE_TRY(upload(ctx, mp->d_score_jobs, mp->score_jobs));
  {
    std::vector<int2> sb;
    score_block_list(mp->score_jobs, sb);
    mp->score_nblocks = (int)sb.size();
    GEYE_TRY(upload(ctx, mp->d_score_blocks, sb));
  }
  GEYE_TRY(mp->d_counts.alloc(ctx, sizeof(int) * ((size_t)std::max(mp->score_nblocks, 1) + 8)));
  P.models.push_back(std::move(mp));
  return GEYE_OK;
}

// Pyramid levels of a frame: sizes (featurepyramid.cpp.org:578-628) and jobs.
static geye_status build_pyramid_plan(geye_ctx *ctx, Plan &P, int width, int height, int LEN, int interval, int sbin,
                                      ArenaAlloc &A, int tc_planes) {
  P.width = width; P.height = height; P.LEN = LEN; P.interval = interval; P.sbin = sbin;
  P.lv.assign(LEN, LevelInfo{});
  const int sbin2 = (int)floor((double)sbin / 2.0);
  const float sc = pow(2, (1.0 / (double)interval));
  // image sizes and scales
  std::vector<int> own(LEN, 0);
  for (int ii = 0; ii < interval && ii < LEN; ii++) {
    float st = 1.0 / pow(sc, ii);
    int oh, ow;
    resize_dims(height, width, st, oh, ow);
    P.lv[ii].img_h = oh; P.lv[ii].img_w = ow; P.lv[ii].img_level = ii; own[ii] = 1;
    P.lv[ii].scale = st * 2;
    if (ii + interval < LEN) {
      P.lv[ii + interval].img_h = oh; P.lv[ii + interval].img_w = ow; P.lv[ii + interval].img_level = ii;
      P.lv[ii + interval].scale = st;
    }
    int rh = oh, rw = ow;
    for (int jj = ii + interval; jj < LEN - interval; jj += interval) {
      int nh, nw;
      resize_dims(rh, rw, 0.5f, nh, nw);
      P.lv[jj + interval].img_h = nh; P.lv[jj + interval].img_w = nw; P.lv[jj + interval].img_level = jj + interval;
      own[jj + interval] = 1;
      P.lv[jj + interval].scale = 0.5 * (P.lv[jj].scale);
      rh = nh; rw = nw;
    }
  }
  for (int l = 0; l < LEN; l++) {
    LevelInfo &L = P.lv[l];
    if (L.img_h < 3 || L.img_w < 3) { set_error("frame too small for the pyramid"); return GEYE_ERR_ARG; }
    if (own[l]) L.img_off = A.take((size_t)3 * L.img_h * L.img_w);
  }
  for (int l = 0; l < LEN; l++) {
    LevelInfo &L = P.lv[l];
    if (!own[l]) L.img_off = P.lv[L.img_level].img_off;
  }
  // resize phases: phase 0 = base levels 1..interval-1 from level 0; phase k>=1 = octave k+1
  std::vector<int> tstart, tsi;
  std::vector<float> talpha;
  auto add_job = [&](std::vector<ResizeJob> &vj, std::vector<ResizeJob> &hj, int &vmax, int &hmax, int src_level,
                     int dst_level) {
    const LevelInfo &S = P.lv[src_level];
    LevelInfo &D = P.lv[dst_level];
    const int tmp = A.take((size_t)3 * D.img_h * S.img_w);
    ResizeJob v{};
    v.src_off = S.img_off; v.dst_off = tmp; v.src_h = S.img_h; v.src_w = S.img_w; v.dst_h = D.img_h; v.dst_w = S.img_w;
    v.tap_start_off = (int)tstart.size(); v.tap_off = (int)tsi.size();
    {
      std::vector<int> st, si; std::vector<float> al;
      build_taps(S.img_h, D.img_h, st, si, al);
      for (auto &x : st) tstart.push_back(x);
      tsi.insert(tsi.end(), si.begin(), si.end());
      talpha.insert(talpha.end(), al.begin(), al.end());
    }
    ResizeJob h{};
    h.src_off = tmp; h.dst_off = D.img_off; h.src_h = D.img_h; h.src_w = S.img_w; h.dst_h = D.img_h; h.dst_w = D.img_w;
    h.tap_start_off = (int)tstart.size(); h.tap_off = (int)tsi.size();
    {
      std::vector<int> st, si; std::vector<float> al;
      build_taps(S.img_w, D.img_w, st, si, al);
      for (auto &x : st) tstart.push_back(x);
      tsi.insert(tsi.end(), si.begin(), si.end());
      talpha.insert(talpha.end(), al.begin(), al.end());
    }
    vj.push_back(v);
    hj.push_back(h);
    vmax = std::max(vmax, v.dst_w);   // output columns: one warp each
    hmax = std::max(hmax, h.dst_w);
    P.bytes_resize += 4.0 * 3 * (S.img_h * S.img_w + D.img_h * S.img_w) + 4.0 * 3 * (D.img_h * S.img_w + D.img_h * D.img_w);
  };
  {
    std::vector<ResizeJob> vj, hj;
    int vm = 0, hm = 0;
    for (int ii = 1; ii < interval && ii < LEN; ii++) {
      if (P.lv[ii].img_h == P.lv[0].img_h && P.lv[ii].img_w == P.lv[0].img_w && 1.0 / pow(sc, ii) == 1.0) continue;
      add_job(vj, hj, vm, hm, 0, ii);
    }
    P.vjobs.push_back(vj); P.hjobs.push_back(hj); P.v_max_items.push_back(vm); P.h_max_items.push_back(hm);
  }
  for (int base = 2 * interval; base < LEN; base += interval) {
    std::vector<ResizeJob> vj, hj;
    int vm = 0, hm = 0;
    for (int l = base; l < std::min(base + interval, LEN); l++) add_job(vj, hj, vm, hm, P.lv[l - interval].img_level, l);
    P.vjobs.push_back(vj); P.hjobs.push_back(hj); P.v_max_items.push_back(vm); P.h_max_items.push_back(hm);
  }
  P.bytes_resize += (double)3 * width * height + 12.0 * width * height;   // ingest
  // HOG
  for (int l = 0; l < LEN; l++) {
    LevelInfo &L = P.lv[l];
    L.sbin = l < interval ? sbin2 : sbin;
    int b0, b1;
    feature_dims(L.img_h, L.img_w, L.sbin, b0, b1, L.fs0, L.fs1);
    L.feat_off = A.take((size_t)std::max(L.fs0 * L.fs1, 1) * kFeatPad);
    if (tc_planes) {   // tc_planes planes [fs0*fs1 + kTcPlanePad][16 B]
      size_t o = (P.arena16_elems + 63) & ~size_t(63);
      L.feat16_off = (int)o;
      P.arena16_elems = o + (size_t)tc_planes * ((size_t)L.fs0 * L.fs1 + kTcPlanePad) * 8;
      // root levels in BF16 mode: the BF16 remainder planes right after (root filters
      // run on split operands, conv_tc.cu)
      if (tc_planes == 4 && l >= interval) {
        L.feat16lo_off = (int)P.arena16_elems;
        P.arena16_elems += (size_t)4 * ((size_t)L.fs0 * L.fs1 + kTcPlanePad) * 8;
      }
    }
    L.hist_off = A.take((size_t)19 * std::max(b0 * b1, 1));
    if (b0 > 0 && b1 > 0) {
      HogJob J{};
      J.img_off = L.img_off; J.h = L.img_h; J.w = L.img_w; J.sbin = L.sbin; J.b0 = b0; J.b1 = b1;
      J.hist_off = L.hist_off; J.fs0 = L.fs0; J.fs1 = L.fs1; J.feat_off = L.feat_off; J.feat16_off = L.feat16_off;
      J.feat16lo_off = L.feat16lo_off;
      J.tc_planes = tc_planes;
      J.fast = tc_planes ? 1 : 0;
      J.corner_off = A.take((size_t)(L.fs0 + 1) * (L.fs1 + 1));
      J.mag_off = L.img_level;   // resolved below, once the image's pixel buffer is placed
      P.hog_jobs.push_back(J);
      P.hog_max_b0 = std::max(P.hog_max_b0, b0);
      P.hog_max_b1 = std::max(P.hog_max_b1, b1);
      P.bytes_hog += 12.0 * L.img_h * L.img_w + 124.0 * L.fs0 * L.fs1;
    }
  }
  // one (bin, magnitude) buffer per image, covering the widest visible area of its levels
  {
    std::map<int, int> pix_of;   // image level -> pix job
    for (auto &J : P.hog_jobs) {
      const int il = J.mag_off;
      auto it = pix_of.find(il);
      if (it == pix_of.end()) {
        HogPixJob X{};
        X.img_off = J.img_off; X.h = J.h; X.w = J.w;
        it = pix_of.emplace(il, (int)P.pix_jobs.size()).first;
        P.pix_jobs.push_back(X);
      }
      HogPixJob &X = P.pix_jobs[it->second];
      X.xe = std::max(X.xe, J.b1 * J.sbin - 1);
      X.ye = std::max(X.ye, J.b0 * J.sbin - 1);
    }
    for (auto &X : P.pix_jobs) {
      X.Y = X.ye + 1;
      const size_t n = (size_t)(X.xe + 1) * X.Y;
      X.mag_off = A.take(n);
      X.bin_off = A.take((n + 3) / 4);
      P.pix_max_xe = std::max(P.pix_max_xe, X.xe);
      P.bytes_hog += 5.0 * n;
    }
    for (auto &J : P.hog_jobs) {
      const HogPixJob &X = P.pix_jobs[pix_of[J.mag_off]];
      J.mag_off = X.mag_off; J.bin_off = X.bin_off; J.pix_Y = X.Y;
    }
  }
  GEYE_TRY(upload(ctx, P.d_tap_start, tstart));
  GEYE_TRY(upload(ctx, P.d_tap_si, tsi));
  GEYE_TRY(upload(ctx, P.d_tap_alpha, talpha));
  P.d_vjobs.resize(P.vjobs.size());
  P.d_hjobs.resize(P.hjobs.size());
  for (size_t i = 0; i < P.vjobs.size(); i++) {
    GEYE_TRY(upload(ctx, P.d_vjobs[i], P.vjobs[i]));
    GEYE_TRY(upload(ctx, P.d_hjobs[i], P.hjobs[i]));
  }
  GEYE_TRY(upload(ctx, P.d_hog_jobs, P.hog_jobs));
  {
    std::vector<int2> vb;
    hog_vote_blocks(P.hog_jobs, vb);
    P.hog_vote_nblocks = (int)vb.size();
    GEYE_TRY(upload(ctx, P.d_hog_vote_blocks, vb));
  }
  GEYE_TRY(upload(ctx, P.d_pix_jobs, P.pix_jobs));
  return GEYE_OK;
}

// FP32 conv shape tuner: job tables for rows per thread cr (4 or 8) and groups
// of at most gmax filters, split from the plan's groups (maps of a group are
// contiguous, so a split group writes the same places); each candidate is timed
// on the plan's arena (CUDA events after one untimed launch), the fastest kept.
// Every shape gives the same bits.
static void conv_jobs_for(const std::vector<ConvJob> &in, int cr, int gmax, std::vector<ConvJob> &out, int &mty,
                          int &mtx, int &mg) {
  out.clear();
  mty = mtx = 0;
  mg = 1;
  for (const ConvJob &J : in)
    for (int k = 0; k < J.n_filt; k += gmax) {
      ConvJob C = J;
      C.filt_base = J.filt_base + k;
      C.n_filt = std::min(gmax, J.n_filt - k);
      C.out_off = J.out_off + k * J.c0 * J.c1;
      C.tiles_y = (J.c0 + 8 * cr - 1) / (8 * cr);
      C.tiles_x = (J.c1 + 15) / 16;
      mty = std::max(mty, C.tiles_y);
      mtx = std::max(mtx, C.tiles_x);
      mg = std::max(mg, C.n_filt);
      out.push_back(C);
    }
}

static geye_status tune_conv_fp32(geye_ctx *ctx, Plan &P, ModelPlan &mp) {
  geye_model *m = mp.model;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  CUDA_TRY(cudaEventCreate(&e0));
  CUDA_TRY(cudaEventCreate(&e1));
  geye_status st = GEYE_OK;
  for (int kind = 0; kind < 2 && st == GEYE_OK; kind++) {
    std::vector<ConvJob> &jobs = kind ? mp.part_jobs : mp.root_jobs;
    if (jobs.empty()) continue;
    const int b0 = kind ? mp.part_max_b0 : mp.root_max_b0, b1 = kind ? mp.part_max_b1 : mp.root_max_b1;
    float best = 0.f;
    std::vector<ConvJob> best_jobs;
    int best_cr = 4, bty = 0, btx = 0, bg = 1, best_i = 0;
    // a geometry this model was tuned at before reuses the choice without timing
    const std::string key = std::string(kind ? "fp32p:" : "fp32r:") + std::to_string(P.width) + "x" +
                            std::to_string(P.height) + "/" + std::to_string(mp.LEN);
    int only = -1;
    {
      std::lock_guard<std::mutex> lk(m->tc_mu);
      auto it = m->tc_tuned.find(key);
      if (it != m->tc_tuned.end()) only = it->second.first;
    }
    for (int ci = 0; ci < 4; ci++) {
      if (only >= 0 && ci != only) continue;
      const int cr = ci < 2 ? 4 : 8, gmax = ci % 2 ? 4 : 8;
      {
        std::vector<ConvJob> cand;
        int mty, mtx, mg;
        conv_jobs_for(jobs, cr, gmax, cand, mty, mtx, mg);
        DevBuf d;
        st = upload(ctx, d, cand);
        if (st != GEYE_OK) break;
        auto launch = [&]() {
          launch_conv_fp32(d.as<ConvJob>(), (int)cand.size(), mty, mtx, m->d_filters, m->d_filt_off,
                           P.arena.as<float>(), P.arena.as<float>(), b0, b1, mg, ctx->stream, cr);
        };
        launch();
        if (cudaEventRecord(e0, ctx->stream) != cudaSuccess) { st = GEYE_ERR_CUDA; break; }
        for (int r = 0; r < 3; r++) launch();
        float ms = 0.f;
        cudaError_t e = cudaEventRecord(e1, ctx->stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e != cudaSuccess) {
          set_error(std::string("FP32 conv tuning: ") + cudaGetErrorString(e));
          st = GEYE_ERR_CUDA;
          break;
        }
        if (best_jobs.empty() || ms < best) {
          best = ms;
          best_jobs = cand;
          best_cr = cr; bty = mty; btx = mtx; bg = mg; best_i = ci;
        }
      }
    }
    if (st != GEYE_OK) break;
    if (only < 0) {
      std::lock_guard<std::mutex> lk(m->tc_mu);
      m->tc_tuned[key] = {best_i, best / 3.0f};
    }
    jobs = best_jobs;
    if (kind) {
      mp.part_cr = best_cr; mp.part_tiles_y = bty; mp.part_tiles_x = btx; mp.part_max_g = bg;
      st = upload(ctx, mp.d_part_jobs, mp.part_jobs);
    } else {
      mp.root_cr = best_cr; mp.root_tiles_y = bty; mp.root_tiles_x = btx; mp.root_max_g = bg;
      st = upload(ctx, mp.d_root_jobs, mp.root_jobs);
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return st;
}

static geye_status finish_plan(geye_ctx *ctx, Plan &P, ArenaAlloc &A) {
  P.arena_words = A.words + 64;
  GEYE_TRY(P.arena.alloc(ctx, P.arena_words * 4));
  if (P.arena16_elems) {
    // after the last plane, a tail that slabs of filters smaller than their group's
    // tap grid may read (the widest filter's columns of the largest level)
    int fb0 = 1, fb1 = 1, fs0 = 1;
    for (auto &mp : P.models) {
      const HostModel &h = mp->model->h;
      for (int r = 0; r < h.NoR; r++) { fb0 = std::max(fb0, h.root_size[3 * r]); fb1 = std::max(fb1, h.root_size[3 * r + 1]); }
      for (int q = 0; q < h.NoP; q++) { fb0 = std::max(fb0, h.part_size[3 * q]); fb1 = std::max(fb1, h.part_size[3 * q + 1]); }
    }
    for (auto &L : P.lv) fs0 = std::max(fs0, L.fs0);
    P.arena16_elems += ((size_t)fb1 * fs0 + fb0 + 16 * 128) * 8;
    GEYE_TRY(P.arena16.alloc(ctx, P.arena16_elems * 2));
    // plane tails are read (and their outputs discarded) but never written: keep them zero
    CUDA_TRY(cudaMemsetAsync(P.arena16.p, 0, P.arena16_elems * 2, ctx->stream));
  }
  int gl = 0, cap = 0;
  for (auto &mp : P.models) {
    gl = std::max(gl, mp->model->gl());
    cap = std::max(cap, mp->cap);
  }
  P.gl = gl;
  // multiple of 32: per-model NMS scratch (int2 queues) stays 8-byte aligned
  P.max_cap = (std::max(cap, 1) + 31) & ~31;
  const size_t nm = std::max<size_t>(P.models.size(), 1);
  GEYE_TRY(P.d_boxes.alloc(ctx, sizeof(float) * nm * P.max_cap * std::max(gl, 1)));
  GEYE_TRY(P.d_kept_boxes.alloc(ctx, sizeof(float) * nm * P.max_cap * std::max(gl, 1)));
  GEYE_TRY(P.d_nms_f.alloc(ctx, sizeof(float) * nm * P.max_cap * 6));
  GEYE_TRY(P.d_nms_i.alloc(ctx, sizeof(int) * nm * nms_model_words(P.max_cap)));
  GEYE_TRY(P.d_small.alloc(ctx, 4096));
  if (P.width > 0) {
    GEYE_TRY(P.d_ascore.alloc(ctx, sizeof(float) * nm * P.width * P.height));
    // A_SCORE lookups (get_boxes.cpp:265-300): per score map, the score column of every
    // image column X and the score row of every image row Y, or -1 where the
    // reference's loop maps nothing there; the division is the reference's float one.
    for (auto &mp : P.models) {
      const int nj = (int)mp->score_jobs.size();
      std::vector<int> col((size_t)nj * P.width), row((size_t)nj * P.height);
      for (int j = 0; j < nj; j++) {
        const ScoreJob &S = mp->score_jobs[j];
        for (int X = 0; X < P.width; X++) {
          const int ii = X - S.RX;
          const int Xn = ii < 0 ? -1 : (int)((float)ii / S.scale + 0);
          col[(size_t)j * P.width + X] = (Xn >= 0 && Xn < S.r1) ? S.score_off + Xn * S.r0 : -1;
        }
        for (int Y = 0; Y < P.height; Y++) {
          const int jj = Y - S.RY;
          const int Yn = jj < 0 ? -1 : (int)((float)jj / S.scale + 0);
          row[(size_t)j * P.height + Y] = (Yn >= 0 && Yn < S.r0) ? Yn : -1;
        }
      }
      GEYE_TRY(upload(ctx, mp->d_as_col, col));
      GEYE_TRY(upload(ctx, mp->d_as_row, row));
    }
  }
  // result arrays: point, or_point (4 ints each), type, scale, score per kept box
  GEYE_TRY(P.d_result.alloc(ctx, nm * (size_t)P.max_cap * 11 * 4));
  P.last_D.assign(nm, 0);
  P.last_K.assign(nm, 0);
  return GEYE_OK;
}

static std::string plan_key(int width, int height, geye_model *const *models, int n, const int *LENs, int mode) {
  std::ostringstream os;
  os << width << "x" << height << "m" << mode;
  for (int i = 0; i < n; i++) os << ":" << models[i]->id << "/" << LENs[i];
  return os.str();
}

static geye_status get_frame_plan(geye_ctx *ctx, geye_model *const *models, int n_models, int width, int height,
                                  Plan **out) {
  if (n_models <= 0 || n_models > 16) { set_error("n_models out of range"); return GEYE_ERR_ARG; }
  const int interval = models[0]->h.interval, sbin = models[0]->h.sbin;
  std::vector<int> LENs(n_models);
  int LEN = 0;
  for (int i = 0; i < n_models; i++) {
    geye_model *m = models[i];
    if (m->h.interval != interval || m->h.sbin != sbin) {
      set_error("models in one call must share sbin and interval");
      return GEYE_ERR_UNSUPPORTED;
    }
    // ini_scales latch (featurepyramid.cpp:178-236)
    if (m->ini) {
      m->max_scale = max_scale_for(m->h, width, height);
      m->ini = false;
    }
    LENs[i] = m->max_scale + interval;
    LEN = std::max(LEN, LENs[i]);
  }
  const int tc_planes = ctx->conv_mode == GEYE_CONV_BF16 ? 4 : ctx->conv_mode == GEYE_CONV_FP8 ? 2 : 0;
  std::string key = plan_key(width, height, models, n_models, LENs.data(), (int)ctx->conv_mode);
  auto it = ctx->plans.find(key);
  if (it != ctx->plans.end()) { *out = it->second.get(); return GEYE_OK; }
  auto P = std::make_unique<Plan>();
  ArenaAlloc A;
  GEYE_TRY(build_pyramid_plan(ctx, *P, width, height, LEN, interval, sbin, A, tc_planes));
  for (int i = 0; i < n_models; i++) GEYE_TRY(build_model_plan(ctx, *P, models[i], LENs[i], A));
  if (ctx->conv_mode != GEYE_CONV_FP32) GEYE_TRY(plan_tc(ctx, *P, A));
  GEYE_TRY(finish_plan(ctx, *P, A));
  // after the arena exists: the tile shapes are tuned on it
  if (ctx->conv_mode != GEYE_CONV_FP32)
    GEYE_TRY(build_tc_plan(ctx, *P));
  else
    for (auto &mp : P->models) GEYE_TRY(tune_conv_fp32(ctx, *P, *mp));
  GEYE_TRY(P->d_bgr.alloc(ctx, (size_t)width * height * 3 + 64));
  if (ctx->plans.size() > 32) ctx->plans.clear();
  *out = P.get();
  ctx->plans[key] = std::move(P);
  return GEYE_OK;
}

// ----------------------------------------------------------------------------
// pipeline
// ----------------------------------------------------------------------------
enum { ST_PYR = 0, ST_HOG, ST_CONV, ST_DT, ST_SCORE, ST_NMS, ST_TOTAL };

struct StageTimer {
  geye_ctx *ctx;
  explicit StageTimer(geye_ctx *c) : ctx(c) {}
  void mark(int i) {
    if (!ctx->timing) return;
    // inside a capture the record becomes an event-record node of the graph
    if (ctx->capturing) cudaEventRecordWithFlags(ctx->ev[i], ctx->stream, cudaEventRecordExternal);
    else cudaEventRecord(ctx->ev[i], ctx->stream);
  }
};

static geye_status check_launch(geye_ctx *ctx, const char *what) {
  ctx->launches++;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(std::string(what) + ": " + cudaGetErrorString(e));
    return GEYE_ERR_CUDA;
  }
  return GEYE_OK;
}

geye_status run_ingest(geye_ctx *ctx, Plan &P, const uint8_t *d_bgr, int width_step) {
  if (injected(ctx, "launch")) { set_error("injected launch failure"); return GEYE_ERR_INJECTED; }
  launch_ingest(d_bgr, P.width, P.height, width_step, P.arena.as<float>() + P.lv[0].img_off, ctx->stream);
  return check_launch(ctx, "ingest");
}

geye_status run_resize(geye_ctx *ctx, Plan &P) {
  cudaStream_t s = ctx->stream;
  float *arena = P.arena.as<float>();
  for (size_t ph = 0; ph < P.vjobs.size(); ph++) {
    if (P.vjobs[ph].empty()) continue;
    launch_resize_pass(P.d_vjobs[ph].as<ResizeJob>(), (int)P.vjobs[ph].size(), P.v_max_items[ph], 1,
                       P.d_tap_start.as<int>(), P.d_tap_si.as<int>(), P.d_tap_alpha.as<float>(), arena, s);
    GEYE_TRY(check_launch(ctx, "resize (vertical)"));
    launch_resize_pass(P.d_hjobs[ph].as<ResizeJob>(), (int)P.hjobs[ph].size(), P.h_max_items[ph], 0,
                       P.d_tap_start.as<int>(), P.d_tap_si.as<int>(), P.d_tap_alpha.as<float>(), arena, s);
    GEYE_TRY(check_launch(ctx, "resize (horizontal)"));
  }
  return GEYE_OK;
}

geye_status run_pyramid(geye_ctx *ctx, Plan &P, const uint8_t *d_bgr, int width_step) {
  GEYE_TRY(run_ingest(ctx, P, d_bgr, width_step));
  return run_resize(ctx, P);
}

geye_status run_hog(geye_ctx *ctx, Plan &P) {
  const bool fast = !P.hog_jobs.empty() && P.hog_jobs[0].fast;
  launch_hog(P.d_hog_jobs.as<HogJob>(), (int)P.hog_jobs.size(), P.d_hog_vote_blocks.as<int2>(), P.hog_vote_nblocks,
             P.hog_max_b0, P.hog_max_b1, P.d_pix_jobs.as<HogPixJob>(), (int)P.pix_jobs.size(), P.pix_max_xe,
             P.arena.as<float>(), P.arena16.p, !fast, ctx->stream);
  ctx->launches += 3;   // pixels, votes, corner norms, features
  return check_launch(ctx, "hog");
}

// FP32 conv of one model (the tensor-core modes convolve every model at once: run_conv_tc)
geye_status run_conv(geye_ctx *ctx, Plan &P, ModelPlan &mp) {
  geye_model *m = mp.model;
  float *arena = P.arena.as<float>();
  if (!mp.root_jobs.empty()) {
    launch_conv_fp32(mp.d_root_jobs.as<ConvJob>(), (int)mp.root_jobs.size(), mp.root_tiles_y, mp.root_tiles_x,
                     m->d_filters, m->d_filt_off, arena, arena, mp.root_max_b0, mp.root_max_b1, mp.root_max_g,
                     ctx->stream, mp.root_cr);
    GEYE_TRY(check_launch(ctx, "root conv"));
  }
  if (!mp.part_jobs.empty()) {
    launch_conv_fp32(mp.d_part_jobs.as<ConvJob>(), (int)mp.part_jobs.size(), mp.part_tiles_y, mp.part_tiles_x,
                     m->d_filters, m->d_filt_off, arena, arena, mp.part_max_b0, mp.part_max_b1, mp.part_max_g,
                     ctx->stream, mp.part_cr);
    GEYE_TRY(check_launch(ctx, "part conv"));
  }
  return GEYE_OK;
}

geye_status run_dt(geye_ctx *ctx, Plan &P, ModelPlan &mp) {
  if (mp.dt_jobs.empty()) return GEYE_OK;
  launch_dt(mp.d_dt_jobs.as<DtJob>(), mp.d_dt_blocks1.as<int2>(), mp.dt_nblocks1, mp.d_dt_blocks2.as<int2>(),
            mp.dt_nblocks2, mp.dt_max_d0, mp.dt_max_d1, P.arena.as<float>(),
            P.arena.as<int>(), ctx->d_diag.as<int>(), mp.dt_elems, ctx->stream);
  ctx->launches++;
  return check_launch(ctx, "dt");
}

// DT tile size of each model of a plan, timed on the maps its last frame left
// in the arena (the DT's cost depends on the values: they set the window
// bounds and whether the argmin order is proven): each of kDtElemsChoices
// runs once untimed and three times timed with CUDA events on the context's
// stream, and the fastest is kept.  A DT run rewrites its outputs from its
// inputs, so the frame's results are unchanged.  Returns true when a plan's
// block lists changed (its frame graphs must be captured again).
static bool tune_dt(geye_ctx *ctx, Plan &P) {
  bool changed = false;
  for (auto &mpp : P.models) {
    ModelPlan &mp = *mpp;
    if (mp.dt_tuned || mp.dt_jobs.empty()) continue;
    mp.dt_tuned = true;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
      if (e0) cudaEventDestroy(e0);
      return changed;
    }
    int best = -1;
    float best_ms = 0.f;
    std::vector<int2> keep1, keep2;
    for (int c = 0; c < 3; c++) {
      const int elems = kDtElemsChoices[c];
      std::vector<int2> b1, b2;
      dt_block_lists(mp.dt_jobs, b1, b2, elems);
      DevBuf t1, t2;
      if (upload(ctx, t1, b1) != GEYE_OK || upload(ctx, t2, b2) != GEYE_OK) break;
      float ms = 0.f;
      for (int rep = 0; rep < 4; rep++) {
        if (rep == 1) cudaEventRecord(e0, ctx->stream);
        launch_dt(mp.d_dt_jobs.as<DtJob>(), t1.as<int2>(), (int)b1.size(), t2.as<int2>(), (int)b2.size(),
                  mp.dt_max_d0, mp.dt_max_d1, P.arena.as<float>(), P.arena.as<int>(), ctx->d_diag.as<int>(), elems,
                  ctx->stream);
      }
      cudaEventRecord(e1, ctx->stream);
      if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) break;
      mp.dt_ms[c] = ms / 3.0f;
      if (best < 0 || mp.dt_ms[c] < best_ms) {
        best = c;
        best_ms = mp.dt_ms[c];
        keep1 = b1;
        keep2 = b2;
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaGetLastError();
    if (best >= 0 && kDtElemsChoices[best] != mp.dt_elems) {
      if (upload(ctx, mp.d_dt_blocks1, keep1) != GEYE_OK || upload(ctx, mp.d_dt_blocks2, keep2) != GEYE_OK) {
        // the old lists may be gone: rebuild them for the old size
        std::vector<int2> b1, b2;
        dt_block_lists(mp.dt_jobs, b1, b2, mp.dt_elems);
        upload(ctx, mp.d_dt_blocks1, b1);
        upload(ctx, mp.d_dt_blocks2, b2);
        continue;
      }
      mp.dt_elems = kDtElemsChoices[best];
      mp.dt_nblocks1 = (int)keep1.size();
      mp.dt_nblocks2 = (int)keep2.size();
      changed = true;
    }
  }
  return changed;
}

// score maps, detection records; model index mi writes boxes at mi*cap*GL and its count at d_small[mi]
geye_status run_score(geye_ctx *ctx, Plan &P, ModelPlan &mp, int mi, float thresh) {
  int *counts = mp.d_counts.as<int>();
  int *d_num = P.d_small.as<int>() + mi;
  const int nj = (int)mp.score_jobs.size();
  if (nj == 0) {
    CUDA_TRY(cudaMemsetAsync(d_num, 0, sizeof(int), ctx->stream));
    return GEYE_OK;
  }
  launch_score(mp.d_score_jobs.as<ScoreJob>(), mp.d_score_blocks.as<int2>(), mp.score_nblocks, thresh,
               P.arena.as<float>(), counts, ctx->stream);
  GEYE_TRY(check_launch(ctx, "score"));
  launch_scan_counts(counts, mp.score_nblocks, d_num, ctx->stream);
  GEYE_TRY(check_launch(ctx, "scan"));
  float *boxes = P.d_boxes.as<float>() + (size_t)mi * P.max_cap * P.gl;
  launch_boxes(mp.d_score_jobs.as<ScoreJob>(), mp.d_score_blocks.as<int2>(), mp.score_nblocks, thresh,
               P.arena.as<float>(), P.arena.as<int>(), counts, mp.model->gl(), boxes, ctx->stream);
  return check_launch(ctx, "boxes");
}

// A_SCORE starts from the caller's map or from ini_ac_score's -100 (detect.cpp:136-145)
static geye_status ascore_init(geye_ctx *ctx, Plan &P, int mi, const float *h_init) {
  float *a = P.d_ascore.as<float>() + (size_t)mi * P.width * P.height;
  const size_t n = (size_t)P.width * P.height;
  if (h_init) {
    if (injected(ctx, "h2d")) { set_error("injected host-to-device copy failure"); return GEYE_ERR_INJECTED; }
    CUDA_TRY(cudaMemcpyAsync(a, h_init, n * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    return GEYE_OK;
  }
  launch_fill(a, n, -100.0f, ctx->stream);
  return check_launch(ctx, "fill");
}

static geye_status ascore_compute(geye_ctx *ctx, Plan &P, ModelPlan &mp, int mi, float thresh, cudaStream_t s) {
  float *a = P.d_ascore.as<float>() + (size_t)mi * P.width * P.height;
  const size_t n = (size_t)P.width * P.height;
  unsigned *maxb = reinterpret_cast<unsigned *>(P.d_small.as<int>() + 64 + mi);
  CUDA_TRY(cudaMemsetAsync(maxb, 0, sizeof(unsigned), s));
  launch_ascore(mp.d_as_col.as<int>(), mp.d_as_row.as<int>(), (int)mp.score_jobs.size(), P.arena.as<float>(), a,
                P.width, P.height, thresh, maxb, s);
  GEYE_TRY(check_launch(ctx, "a_score"));
  launch_ascore_normalize(a, (int)n, maxb, s);
  return check_launch(ctx, "a_score normalise");
}

geye_status run_ascore(geye_ctx *ctx, Plan &P, ModelPlan &mp, int mi, float thresh, const float *h_init) {
  GEYE_TRY(ascore_init(ctx, P, mi, h_init));
  return ascore_compute(ctx, P, mp, mi, thresh, ctx->stream);
}

// After a frame of the plan has completed: `used` is the deepest grid-wide
// quicksort level that had a segment to partition (0 when no model needed the
// quicksort's order), `rounds` the greedy batches the frame took.
// Sort levels: the first frame that sorts launches the default count
// (nms_sort_levels); if it needed fewer, the plan launches three levels more
// than it needed from then on (each empty level costs three launches).  A
// frame whose last launched level still had work left its remaining segments
// to the single-block fallback (exact, slower): the plan goes back to the
// default count for good.
// Rounds: a plan launches kNmsRounds (a round with nothing left is two launches
// that return at once); a frame that took more batches than were launched (the
// rest ran in the finish kernel's single block) makes it launch half as many
// again plus two, so that a few frames settle it (each change costs a graph
// capture), and the count only grows.
// The plan's DT tile sizes are tuned here too, once, on this frame's maps
// (tune_dt).  A change drops the plan's frame graphs after its stream has
// drained; the next frame captures them again.
void note_sort_levels(geye_ctx *ctx, Plan &P, int used, int rounds) {
  const int full = nms_sort_levels(P.max_cap);
  const int launched = P.sort_levels > 0 ? P.sort_levels : full;
  const int r_launched = P.nms_rounds > 0 ? P.nms_rounds : kNmsRounds;
  int next = P.sort_levels, r_next = P.nms_rounds;
  if (used >= launched) {
    if (P.sort_levels > 0) { next = 0; P.sort_levels_fixed = true; }
  } else if (!P.sort_levels_fixed && P.sort_levels == 0 && used > 0 && used + 3 < full) {
    next = std::max(4, used + 3);
  }
  if (rounds > r_launched) r_next = std::min(kNmsMaxRounds, rounds + rounds / 2 + 2);
  const bool dt_changed = P.from_features ? false : tune_dt(ctx, P);   // (behind the frame on its stream)
  if (next == P.sort_levels && r_next == P.nms_rounds && !dt_changed) return;
  P.sort_levels = next;
  P.nms_rounds = r_next;
  cudaStreamSynchronize(ctx->stream);
  for (auto &g : P.graphs)
    if (g.second.exec) cudaGraphExecDestroy(g.second.exec);
  P.graphs.clear();
}

geye_status run_nms(geye_ctx *ctx, Plan &P, int n_models, float overlap) {
  int *d_num = P.d_small.as<int>();
  int *d_kept = d_num + 32;
  int *err = d_num + 128;
  const cudaError_t ge =
      launch_nms_batch(P.d_boxes.as<float>(), d_num, n_models, P.gl, overlap,
                       1.25f * (float)std::max(P.width, P.height), P.max_cap, P.d_nms_i.as<int>(),
                       P.d_nms_f.as<float>(), P.d_kept_boxes.as<float>(), d_kept, err,
                       reinterpret_cast<long long *>(d_num + 512), P.sort_levels, d_num + kSortLevelsUsed,
                       P.nms_rounds, d_num + kNmsRoundsUsed, d_num + kNmsNeed, ctx->nms_order, ctx->stream,
                       (ctx->capturing && ctx->nms_if_node) ? ctx->aux : nullptr);
  if (ge != cudaSuccess) {
    set_error(std::string("nms graph nodes: ") + cudaGetErrorString(ge));
    return GEYE_ERR_CUDA;
  }
  GEYE_TRY(check_launch(ctx, "nms"));
  for (int mi = 0; mi < n_models; mi++) {
    ModelPlan &mp = *P.models[mi];
    geye_model *m = mp.model;
    int *res = P.d_result.as<int>() + (size_t)mi * P.max_cap * 11;
    int *point = res, *or_point = res + 4 * P.max_cap, *type = res + 8 * P.max_cap;
    float *scale = reinterpret_cast<float *>(res + 9 * P.max_cap), *score = reinterpret_cast<float *>(res + 10 * P.max_cap);
    launch_new_rects(P.d_kept_boxes.as<float>() + (size_t)mi * P.max_cap * P.gl, d_kept + mi, m->gl(),
                     m->h.numpart[0], m->d_coef, P.width, P.height, m->h.ratio, point, or_point, type, scale, score,
                     ctx->stream);
    GEYE_TRY(check_launch(ctx, "new_rects"));
  }
  return GEYE_OK;
}

// Everything after the ingest and the A_SCORE initialisation: plan-static, so
// it is captured once per (plan, threshold, overlap, timing) as a CUDA graph.
static geye_status run_body(geye_ctx *ctx, Plan &P, float thresh, float overlap) {
  StageTimer T(ctx);
  if (!ctx->front_external) GEYE_TRY(run_resize(ctx, P));
  T.mark(1);
  if (!ctx->front_external) GEYE_TRY(run_hog(ctx, P));
  T.mark(2);
  const bool tc = ctx->conv_mode != GEYE_CONV_FP32;
  if (tc) GEYE_TRY(run_conv_tc(ctx, P));   // every model's filters in one launch
  if (ctx->timing || P.models.size() < 2) {   // stage by stage (per-stage times)
    if (!tc)
      for (auto &mp : P.models) GEYE_TRY(run_conv(ctx, P, *mp));
    T.mark(3);
    for (auto &mp : P.models) GEYE_TRY(run_dt(ctx, P, *mp));
    T.mark(4);
    for (size_t mi = 0; mi < P.models.size(); mi++) GEYE_TRY(run_score(ctx, P, *P.models[mi], (int)mi, thresh));
  } else {
    // each model's conv -> DT -> score chain reads only the shared features and
    // writes only its own maps and records: models 1.. run on the side stream
    // beside model 0 (their kernels take the context's stream, swapped while
    // they are issued), joined before NMS
    auto chain = [&](size_t mi) -> geye_status {
      if (!tc) GEYE_TRY(run_conv(ctx, P, *P.models[mi]));
      GEYE_TRY(run_dt(ctx, P, *P.models[mi]));
      return run_score(ctx, P, *P.models[mi], (int)mi, thresh);
    };
    CUDA_TRY(cudaEventRecord(ctx->ev_fork, ctx->stream));
    CUDA_TRY(cudaStreamWaitEvent(ctx->side, ctx->ev_fork, 0));
    std::swap(ctx->stream, ctx->side);
    geye_status st1 = GEYE_OK;
    for (size_t mi = 1; mi < P.models.size() && st1 == GEYE_OK; mi++) st1 = chain(mi);
    std::swap(ctx->stream, ctx->side);
    CUDA_TRY(cudaEventRecord(ctx->ev_join, ctx->side));
    const geye_status st0 = chain(0);
    CUDA_TRY(cudaStreamWaitEvent(ctx->stream, ctx->ev_join, 0));   // joined on every path
    GEYE_TRY(st0);
    GEYE_TRY(st1);
  }
  T.mark(5);
  // A_SCORE feeds nothing in the frame: it runs on the side stream beside NMS
  CUDA_TRY(cudaEventRecord(ctx->ev_fork, ctx->stream));
  CUDA_TRY(cudaStreamWaitEvent(ctx->side, ctx->ev_fork, 0));
  geye_status st = GEYE_OK;
  for (size_t mi = 0; mi < P.models.size() && st == GEYE_OK; mi++)
    st = ascore_compute(ctx, P, *P.models[mi], (int)mi, thresh, ctx->side);
  CUDA_TRY(cudaEventRecord(ctx->ev_join, ctx->side));
  if (st == GEYE_OK) st = run_nms(ctx, P, (int)P.models.size(), overlap);
  CUDA_TRY(cudaStreamWaitEvent(ctx->stream, ctx->ev_join, 0));   // joined on every path
  GEYE_TRY(st);
  T.mark(6);
  return GEYE_OK;
}

static geye_status run_body_graph(geye_ctx *ctx, Plan &P, float thresh, float overlap) {
  char key[64];
  unsigned tb, ob;
  memcpy(&tb, &thresh, 4);
  memcpy(&ob, &overlap, 4);
  snprintf(key, sizeof key, "%08x:%08x:%d:%d", tb, ob, ctx->timing ? 1 : 0, ctx->nms_order);
  Plan::FrameGraph &g = P.graphs[key];
  if (!g.exec) {
    const int before = ctx->launches;
    cudaGraph_t graph = nullptr;
    ctx->capturing = true;
    CUDA_TRY(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeRelaxed));
    const geye_status st = run_body(ctx, P, thresh, overlap);
    const cudaError_t e = cudaStreamEndCapture(ctx->stream, &graph);
    ctx->capturing = false;
    ctx->launches = before;
    if (st != GEYE_OK) {
      if (graph) cudaGraphDestroy(graph);
      P.graphs.erase(key);
      return st;
    }
    if (e != cudaSuccess) {
      P.graphs.erase(key);
      set_error(std::string("frame graph capture: ") + cudaGetErrorString(e));
      return GEYE_ERR_CUDA;
    }
    size_t n = 0;
    cudaGraphGetNodes(graph, nullptr, &n);
    std::vector<cudaGraphNode_t> nodes(n);
    if (n) cudaGraphGetNodes(graph, nodes.data(), &n);
    int kernels = 0;
    for (auto nd : nodes) {
      cudaGraphNodeType t;
      if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) kernels++;
    }
    const cudaError_t ie = cudaGraphInstantiate(&g.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) {
      g.exec = nullptr;
      P.graphs.erase(key);
      set_error(std::string("frame graph instantiate: ") + cudaGetErrorString(ie));
      return GEYE_ERR_CUDA;
    }
    g.kernels = kernels;
  }
  CUDA_TRY(cudaGraphLaunch(g.exec, ctx->stream));
  ctx->launches += g.kernels;
  return GEYE_OK;
}

// Whole path for n models on a frame already on the device.
geye_status run_frame(geye_ctx *ctx, Plan &P, const uint8_t *d_bgr, int width_step, float thresh, float overlap,
                      const float *const *h_ascore_init) {
  StageTimer T(ctx);
  ctx->launches = 0;
  CUDA_TRY(cudaMemsetAsync(P.d_small.p, 0, 4096, ctx->stream));
  T.mark(0);
  if (!ctx->front_external) GEYE_TRY(run_ingest(ctx, P, d_bgr, width_step));
  for (size_t mi = 0; mi < P.models.size(); mi++)
    GEYE_TRY(ascore_init(ctx, P, (int)mi, h_ascore_init ? h_ascore_init[mi] : nullptr));
  if (ctx->use_graphs) GEYE_TRY(run_body_graph(ctx, P, thresh, overlap));
  else GEYE_TRY(run_body(ctx, P, thresh, overlap));
  if (ctx->timing) {
    // stage bytes / flops for the roofline report
    double conv_b = 0, conv_f = 0, dt_b = 0, sc_b = 0;
    for (auto &mp : P.models) { conv_b += mp->conv_bytes; conv_f += mp->conv_flops; dt_b += mp->dt_bytes; sc_b += mp->score_bytes; }
    ctx->stage_bytes[ST_PYR] = P.bytes_resize;
    ctx->stage_bytes[ST_HOG] = P.bytes_hog;
    ctx->stage_bytes[ST_CONV] = conv_b;
    ctx->stage_bytes[ST_DT] = dt_b;
    ctx->stage_bytes[ST_SCORE] = sc_b;
    ctx->stage_bytes[ST_NMS] = 0;
    ctx->stage_bytes[ST_TOTAL] = P.bytes_resize + P.bytes_hog + conv_b + dt_b + sc_b;
    ctx->conv_flops = conv_f;
  }
  ctx->last_plan = &P;
  return GEYE_OK;
}

geye_status collect_stage_times(geye_ctx *ctx) {
  if (!ctx->timing) return GEYE_OK;
  CUDA_TRY(cudaEventSynchronize(ctx->ev[6]));
  for (int i = 0; i < 6; i++) CUDA_TRY(cudaEventElapsedTime(&ctx->stage_ms[i], ctx->ev[i], ctx->ev[i + 1]));
  CUDA_TRY(cudaEventElapsedTime(&ctx->stage_ms[6], ctx->ev[0], ctx->ev[6]));
  return GEYE_OK;
}

geye_status frame_plan(geye_ctx *ctx, geye_model *const *models, int n, int w, int h, Plan **out) {
  return get_frame_plan(ctx, models, n, w, h, out);
}

void drop_frame_plans(geye_ctx *ctx, int w, int h) {
  for (auto it = ctx->plans.begin(); it != ctx->plans.end();) {
    Plan *P = it->second.get();
    if (!P->from_features && P->width == w && P->height == h) {
      if (ctx->last_plan == P) ctx->last_plan = nullptr;
      if (ctx->pending == P) ctx->pending = nullptr;
      it = ctx->plans.erase(it);
    } else {
      ++it;
    }
  }
}

geye_status parse_model_files(const char *c, const char *r, const char *p, HostModel &m) { return parse_model(c, r, p, m); }

int model_max_scale(const HostModel &m, int w, int h) { return max_scale_for(m, w, h); }

}  // namespace geye

namespace geye {

const char *last_error_cstr() { return g_err.c_str(); }

// Plan over caller-supplied features (get_boxes stage entry point): no images,
// levels take their sizes and scales from the caller.
geye_status features_plan(geye_ctx *ctx, geye_model *model, const int *ftsize, const float *scales, int n_levels,
                          int img_w, int img_h, Plan **out) {
  const HostModel &m = model->h;
  auto P = std::make_unique<Plan>();
  P->from_features = true;
  P->width = img_w;
  P->height = img_h;
  P->interval = m.interval;
  P->sbin = m.sbin;
  P->LEN = n_levels;
  P->lv.assign(n_levels, LevelInfo{});
  ArenaAlloc A;
  for (int l = 0; l < n_levels; l++) {
    LevelInfo &L = P->lv[l];
    L.fs0 = ftsize[2 * l];
    L.fs1 = ftsize[2 * l + 1];
    L.scale = scales[l];
    L.sbin = l < m.interval ? m.sbin / 2 : m.sbin;
    L.feat_off = A.take((size_t)std::max(L.fs0 * L.fs1, 1) * kFeatPad);
  }
  GEYE_TRY(build_model_plan(ctx, *P, model, n_levels, A));
  GEYE_TRY(finish_plan(ctx, *P, A));
  std::string key = "features:" + std::to_string((uintptr_t)P.get());
  *out = P.get();
  ctx->plans[key] = std::move(P);
  return GEYE_OK;
}

void drop_plan(geye_ctx *ctx, Plan *P) {
  for (auto it = ctx->plans.begin(); it != ctx->plans.end(); ++it)
    if (it->second.get() == P) {
      if (ctx->last_plan == P) ctx->last_plan = nullptr;
      ctx->plans.erase(it);
      return;
    }
}

}  // namespace geye
