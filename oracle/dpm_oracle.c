/*
 * dpm_oracle.c -- CPU restatement of CPFL/geye's DPM detection path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: the pytest suite, the
 * smoke check in __graft_entry__.py and the cpu_baseline leg of bench.py call it
 * to decide whether the CUDA path is right, and bench.py times it as the CPU
 * baseline.  The product (libgeye_dpm.so) never links, loads or calls it.
 *
 * Every function restates, in this project's own code, the arithmetic of the
 * reference function named in its comment (paths are relative to the
 * reference project root).  Expressions keep the reference's C types and
 * evaluation order on purpose: float-vs-double promotion and the order of
 * float additions decide bit-exactness.  Build with -ffp-contract=off (no FMA
 * contraction; gcc contracts by default on aarch64) and without -ffast-math.
 *
 * Parity pins: tests/test_oracle_vs_ref.py checks each function here against
 * the reference's own translation units compiled by oracle/ref/Makefile
 * (resize.cc, dt.cpp, nms.cpp, get_boxes.cpp, featurepyramid.cpp) on seeded
 * inputs, and tests/golden/ holds vectors produced by those compiled
 * reference functions for machines without the reference sources.
 * Two stages have no CPU body in the reference and are restated from the
 * reference's GPU kernel / alternate file:
 *   - filter convolution: CAR_TRACKING/GPU_function.cu:302-358 (per-feature
 *     partial sum over (xp, yp), partials summed over the 31 features);
 *   - pyramid orchestration: CAR_TRACKING/featurepyramid.cpp.org:547-661.
 * Those two are pinned only by this restatement (no reference binary runs
 * them on the CPU).
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "dpm_oracle.h"

/* ------------------------------------------------------------------------- */
/* Model loading: CAR_TRACKING/load_model.cpp:57-244 (component file),        */
/* :250-384 (root filters), :390-530 (part filters), :541-558 (load_model,    */
/* which forces padx = pady = 0).                                             */
/* ------------------------------------------------------------------------- */

static int scan_f(FILE *f, float *v) { return fscanf(f, "%f,", v) == 1 ? 0 : -1; }

void orc_model_free(orc_model *m)
{
    if (!m) return;
    free(m->ridx); free(m->oidx); free(m->offw); free(m->rsize); free(m->numpart);
    for (int c = 0; c < m->numcomponent; c++) {
        if (m->pidx) free(m->pidx[c]);
        if (m->didx) free(m->didx[c]);
        if (m->psize) free(m->psize[c]);
        if (m->x1) free(m->x1[c]);
        if (m->y1) free(m->y1[c]);
        if (m->x2) free(m->x2[c]);
        if (m->y2) free(m->y2[c]);
    }
    free(m->pidx); free(m->didx); free(m->psize);
    free(m->x1); free(m->y1); free(m->x2); free(m->y2);
    free(m->def); free(m->anchor);
    for (int i = 0; i < m->NoR; i++) free(m->rootfilter ? m->rootfilter[i] : NULL);
    for (int i = 0; i < m->NoP; i++) free(m->partfilter ? m->partfilter[i] : NULL);
    free(m->rootfilter); free(m->partfilter);
    free(m->root_size); free(m->part_size); free(m->part_partner);
    free(m);
}

orc_model *orc_model_load(const char *comp, const char *root, const char *part, float ratio)
{
    FILE *f = fopen(comp, "r");
    if (!f) return NULL;
    orc_model *m = (orc_model *)calloc(1, sizeof(orc_model));
    float t1, t2, t3, t4;
    int bad = 0;
    bad |= scan_f(f, &t1); m->numcomponent = (int)t1;
    bad |= scan_f(f, &t1); m->sbin = (int)t1;
    bad |= scan_f(f, &t1); m->interval = (int)t1;
    bad |= scan_f(f, &t1); m->max_Y = (int)t1;
    bad |= scan_f(f, &t1); m->max_X = (int)t1;
    int nc = m->numcomponent;
    if (bad || nc <= 0 || nc > 64) { fclose(f); orc_model_free(m); return NULL; }
    m->ridx = (int *)calloc(nc, sizeof(int));
    m->oidx = (int *)calloc(nc, sizeof(int));
    m->offw = (float *)calloc(nc, sizeof(float));
    m->rsize = (int *)calloc(2 * nc, sizeof(int));
    m->numpart = (int *)calloc(nc, sizeof(int));
    m->pidx = (int **)calloc(nc, sizeof(int *));
    m->didx = (int **)calloc(nc, sizeof(int *));
    m->psize = (int **)calloc(nc, sizeof(int *));
    for (int c = 0; c < nc; c++) {
        bad |= scan_f(f, &t1); m->ridx[c] = (int)t1 - 1;
        bad |= scan_f(f, &t1); m->oidx[c] = (int)t1 - 1;
        bad |= scan_f(f, &t1); m->offw[c] = t1;
        bad |= scan_f(f, &t1); bad |= scan_f(f, &t2);
        m->rsize[2 * c] = (int)t1; m->rsize[2 * c + 1] = (int)t2;
        bad |= scan_f(f, &t1); m->numpart[c] = (int)t1;
        int np = m->numpart[c];
        if (bad || np < 0 || np > 64) { fclose(f); orc_model_free(m); return NULL; }
        m->pidx[c] = (int *)calloc(np ? np : 1, sizeof(int));
        m->didx[c] = (int *)calloc(np ? np : 1, sizeof(int));
        m->psize[c] = (int *)calloc(2 * (np ? np : 1), sizeof(int));
        for (int k = 0; k < np; k++) {
            bad |= scan_f(f, &t1); m->pidx[c][k] = (int)t1 - 1;
            bad |= scan_f(f, &t1); m->didx[c][k] = (int)t1 - 1;
            bad |= scan_f(f, &t1); bad |= scan_f(f, &t2);
            m->psize[c][2 * k] = (int)t1; m->psize[c][2 * k + 1] = (int)t2;
        }
    }
    bad |= scan_f(f, &t1);
    m->DefL = (int)t1;
    if (bad || m->DefL < 0 || m->DefL > 4096) { fclose(f); orc_model_free(m); return NULL; }
    m->def = (float *)calloc(4 * (m->DefL ? m->DefL : 1), sizeof(float));
    m->anchor = (int *)calloc(2 * (m->DefL ? m->DefL : 1), sizeof(int));
    for (int k = 0; k < m->DefL; k++) {
        bad |= scan_f(f, &t1); bad |= scan_f(f, &t2); bad |= scan_f(f, &t3); bad |= scan_f(f, &t4);
        m->def[4 * k] = t1; m->def[4 * k + 1] = t2; m->def[4 * k + 2] = t3; m->def[4 * k + 3] = t4;
        bad |= scan_f(f, &t1); bad |= scan_f(f, &t2);
        m->anchor[2 * k] = (int)t1; m->anchor[2 * k + 1] = (int)t2;
    }
    m->x1 = (float **)calloc(nc, sizeof(float *));
    m->y1 = (float **)calloc(nc, sizeof(float *));
    m->x2 = (float **)calloc(nc, sizeof(float *));
    m->y2 = (float **)calloc(nc, sizeof(float *));
    for (int c = 0; c < nc; c++) {
        int GL = 1 + 2 * (1 + m->numpart[c]);
        m->x1[c] = (float *)calloc(GL, sizeof(float));
        m->y1[c] = (float *)calloc(GL, sizeof(float));
        m->x2[c] = (float *)calloc(GL, sizeof(float));
        m->y2[c] = (float *)calloc(GL, sizeof(float));
        for (int j = 0; j < GL; j++) { bad |= scan_f(f, &t1); m->x1[c][j] = t1; }
        for (int j = 0; j < GL; j++) { bad |= scan_f(f, &t1); m->y1[c][j] = t1; }
        for (int j = 0; j < GL; j++) { bad |= scan_f(f, &t1); m->x2[c][j] = t1; }
        for (int j = 0; j < GL; j++) { bad |= scan_f(f, &t1); m->y2[c][j] = t1; }
    }
    fclose(f);
    if (bad) { orc_model_free(m); return NULL; }
    /* load_model.cpp:552-553 forces the pad to zero after load_modelinfo set it. */
    m->padx = 0;
    m->pady = 0;
    m->ini = 1;
    m->ratio = ratio;

    /* root filters */
    f = fopen(root, "r");
    if (!f) { orc_model_free(m); return NULL; }
    bad |= scan_f(f, &t1);
    m->NoR = (int)t1;
    if (bad || m->NoR <= 0 || m->NoR > 64) { fclose(f); orc_model_free(m); return NULL; }
    m->root_size = (int *)calloc(3 * m->NoR, sizeof(int));
    m->rootfilter = (float **)calloc(m->NoR, sizeof(float *));
    for (int i = 0; i < m->NoR; i++) {
        bad |= scan_f(f, &t1); bad |= scan_f(f, &t2); bad |= scan_f(f, &t3);
        m->root_size[3 * i] = (int)t1; m->root_size[3 * i + 1] = (int)t2; m->root_size[3 * i + 2] = (int)t3;
        int n = (int)t1 * (int)t2 * (int)t3;
        if (bad || n <= 0) { fclose(f); orc_model_free(m); return NULL; }
        m->rootfilter[i] = (float *)calloc(n, sizeof(float));
        for (int j = 0; j < n; j++) { bad |= scan_f(f, &t1); m->rootfilter[i][j] = t1; }
    }
    fclose(f);
    if (bad) { orc_model_free(m); return NULL; }

    /* part filters: size triple, values, then the symmetric partner */
    f = fopen(part, "r");
    if (!f) { orc_model_free(m); return NULL; }
    bad |= scan_f(f, &t1);
    m->NoP = (int)t1;
    if (bad || m->NoP < 0 || m->NoP > 4096) { fclose(f); orc_model_free(m); return NULL; }
    m->part_size = (int *)calloc(3 * (m->NoP ? m->NoP : 1), sizeof(int));
    m->partfilter = (float **)calloc(m->NoP ? m->NoP : 1, sizeof(float *));
    m->part_partner = (int *)calloc(m->NoP ? m->NoP : 1, sizeof(int));
    for (int i = 0; i < m->NoP; i++) {
        bad |= scan_f(f, &t1); bad |= scan_f(f, &t2); bad |= scan_f(f, &t3);
        m->part_size[3 * i] = (int)t1; m->part_size[3 * i + 1] = (int)t2; m->part_size[3 * i + 2] = (int)t3;
        int n = (int)t1 * (int)t2 * (int)t3;
        if (bad || n <= 0) { fclose(f); orc_model_free(m); return NULL; }
        m->partfilter[i] = (float *)calloc(n, sizeof(float));
        for (int j = 0; j < n; j++) { bad |= scan_f(f, &t1); m->partfilter[i][j] = t1; }
        bad |= scan_f(f, &t1);
        m->part_partner[i] = (int)t1;
    }
    fclose(f);
    if (bad) { orc_model_free(m); return NULL; }
    return m;
}

/* ------------------------------------------------------------------------- */
/* Image ingest: CAR_TRACKING/featurepyramid.cpp.org:461-500 (Ipl_to_FLOAT).  */
/* BGR interleaved rows (stride widthStep) -> planes R,G,B, column-major      */
/* [c][x][y].                                                                 */
/* ------------------------------------------------------------------------- */
void orc_ipl_to_float(const uint8_t *bgr, int height, int width, int width_step, float *out)
{
    const int SQ = height * width;
    float *R = out, *G = out + SQ, *B = out + 2 * SQ;
    for (int x = 0; x < width; x++) {
        int XT = x * 3;
        for (int y = 0; y < height; y++) {
            int pp = width_step * y + XT;
            *(B++) = (float)bgr[pp];
            *(G++) = (float)bgr[pp + 1];
            *(R++) = (float)bgr[pp + 2];
        }
    }
}

/* ------------------------------------------------------------------------- */
/* Resize: CAR_TRACKING/resize.cc:68-124 (resize1dtran), :135-160 (resize).    */
/* ------------------------------------------------------------------------- */
typedef struct { int si, di; float alpha; } orc_tap;

/* Builds the tap list of one 1-D pass exactly as resize1dtran does. */
int orc_resize_taps(int sheight, int dheight, int *si, int *di, float *alpha, int cap)
{
    float scale = (float)dheight / (float)sheight;
    float invscale = (float)sheight / (float)dheight;
    int k = 0;
    for (int dy = 0; dy < dheight; dy++) {
        float fsy1 = dy * invscale;
        float fsy2 = fsy1 + invscale;
        int sy1 = (int)(fsy1 + 0.99);
        int sy2 = (int)fsy2;
        if (sy1 - fsy1 > 1e-3) {
            if (k < cap) { di[k] = dy; si[k] = sy1 - 1; alpha[k] = (sy1 - fsy1) * scale; }
            k++;
        }
        for (int sy = sy1; sy < sy2; sy++) {
            if (k < cap) { di[k] = dy; si[k] = sy; alpha[k] = scale; }
            k++;
        }
        if (fsy2 - sy2 > 1e-3) {
            if (k < cap) { di[k] = dy; si[k] = sy2; alpha[k] = (fsy2 - sy2) * scale; }
            k++;
        }
    }
    return k;
}

static void resize1dtran(const float *src, int sheight, float *dst, int dheight, int width, int chan)
{
    int cap = (int)(dheight * ((float)sheight / (float)dheight) + 0.99) + 2 * dheight + 4;
    int *si = (int *)malloc(sizeof(int) * cap), *di = (int *)malloc(sizeof(int) * cap);
    float *al = (float *)malloc(sizeof(float) * cap);
    int k = orc_resize_taps(sheight, dheight, si, di, al, cap);
    if (k > cap) { fprintf(stderr, "orc: tap overflow\n"); abort(); }
    const int WD = width * dheight, WS = width * sheight;
    memset(dst, 0, sizeof(float) * (size_t)chan * WD);
    for (int c = 0; c < chan; c++) {
        const float *s = src + (size_t)c * WS;
        float *d = dst + (size_t)c * WD;
        for (int x = 0; x < width; x++) {
            for (int t = 0; t < k; t++) d[di[t] * width] += al[t] * s[si[t]];
            s += sheight;
            d++;
        }
    }
    free(si); free(di); free(al);
}

void orc_resize_dims(const int *sdims, float scale, int *odims)
{
    if (scale == 1.0f) { odims[0] = sdims[0]; odims[1] = sdims[1]; odims[2] = sdims[2]; return; }
    odims[0] = (int)((float)sdims[0] * scale + 0.5);
    odims[1] = (int)((float)sdims[1] * scale + 0.5);
    odims[2] = sdims[2];
}

/* src/dst column-major [c][x][y]; dst sized by orc_resize_dims. */
void orc_resize(const float *src, const int *sdims, int *odims, float scale, float *dst)
{
    orc_resize_dims(sdims, scale, odims);
    if (scale == 1.0f) {
        memcpy(dst, src, sizeof(float) * (size_t)odims[0] * odims[1] * odims[2]);
        return;
    }
    float *tmp = (float *)calloc((size_t)odims[0] * sdims[1] * sdims[2], sizeof(float));
    resize1dtran(src, sdims[0], tmp, odims[0], sdims[1], sdims[2]);
    resize1dtran(tmp, sdims[1], dst, odims[1], odims[0], sdims[2]);
    free(tmp);
}

/* ------------------------------------------------------------------------- */
/* HOG: CAR_TRACKING/featurepyramid.cpp:263-501 (calc_feature; the symlink    */
/* resolves to featurepyramid.cpp.new2).                                      */
/* ------------------------------------------------------------------------- */
static const float Hcos[9] = {1.0000, 0.9397, 0.7660, 0.5000, 0.1736, -0.1736, -0.5000, -0.7660, -0.9397};
static const float Hsin[9] = {0.0000, 0.3420, 0.6428, 0.8660, 0.9848, 0.9848, 0.8660, 0.6428, 0.3420};

static inline int imax(int a, int b) { return a >= b ? a : b; }
static inline int imin(int a, int b) { return a <= b ? a : b; }
static inline float min_2(float x) { return (x <= 0.2 ? x : 0.2); }

void orc_feature_dims(int height, int width, int sbin, int *ftsize)
{
    int b0 = (int)floor((double)height / (double)sbin + 0.5);
    int b1 = (int)floor((double)width / (double)sbin + 0.5);
    ftsize[0] = imax(b0 - 2, 0);
    ftsize[1] = imax(b1 - 2, 0);
}

/* Orientation bin (0..17) and squared magnitude of one pixel; exposed so the
 * tests can compare bin selection pixel by pixel.  Returns best_o; *vout gets
 * the squared magnitude before the sqrt. */
int orc_hog_pixel(const float *SRC, int height, int width, int x, int y, float *vout)
{
    const int dims[2] = {height, width};
    const float *s = SRC + imin(x, dims[1] - 2) * dims[0] + imin(y, dims[0] - 2);
    float dy = *(s + 1) - *(s - 1);
    float dx = *(s + dims[0]) - *(s - dims[0]);
    float v = dx * dx + dy * dy;
    s += dims[0] * dims[1];
    float dy2 = *(s + 1) - *(s - 1);
    float dx2 = *(s + dims[0]) - *(s - dims[0]);
    float v2 = dx2 * dx2 + dy2 * dy2;
    s += dims[0] * dims[1];
    float dy3 = *(s + 1) - *(s - 1);
    float dx3 = *(s + dims[0]) - *(s - dims[0]);
    float v3 = dx3 * dx3 + dy3 * dy3;
    if (v2 > v) { v = v2; dx = dx2; dy = dy2; }
    if (v3 > v) { v = v3; dx = dx3; dy = dy3; }
    float best_dot = 0;
    int best_o = 0;
    for (int o = 0; o < 9; o++) {
        float dot = Hcos[o] * dx + Hsin[o] * dy;
        if (dot > best_dot) { best_dot = dot; best_o = o; }
        else if (-dot > best_dot) { best_dot = -dot; best_o = o + 9; }
    }
    *vout = v;
    return best_o;
}

/* SRC column-major [3][width][height]; feat column-major [31][out1][out0]. */
void orc_calc_feature(const float *SRC, int height, int width, int sbin, int *ftsize, float *feat)
{
    const int dims[2] = {height, width};
    const int blocks[2] = {(int)floor((double)height / (double)sbin + 0.5),
                           (int)floor((double)width / (double)sbin + 0.5)};
    int out[3] = {imax(blocks[0] - 2, 0), imax(blocks[1] - 2, 0), 27 + 4};
    const int visible[2] = {blocks[0] * sbin, blocks[1] * sbin};
    float *hist = (float *)calloc((size_t)blocks[0] * blocks[1] * 18 + 1, sizeof(float));
    float *norm = (float *)calloc((size_t)blocks[0] * blocks[1] + 1, sizeof(float));
    const size_t BSQ = (size_t)blocks[0] * blocks[1];

    for (int x = 1; x < visible[1] - 1; x++) {
        for (int y = 1; y < visible[0] - 1; y++) {
            float v;
            int best_o = orc_hog_pixel(SRC, dims[0], dims[1], x, y, &v);
            float xp = ((float)x + 0.5) / (float)sbin - 0.5;
            float yp = ((float)y + 0.5) / (float)sbin - 0.5;
            int ixp = (int)floor(xp);
            int iyp = (int)floor(yp);
            float vx0 = xp - ixp;
            float vy0 = yp - iyp;
            float vx1 = 1.0 - vx0;
            float vy1 = 1.0 - vy0;
            v = sqrt(v);
            if (ixp >= 0 && iyp >= 0)
                hist[ixp * blocks[0] + iyp + best_o * BSQ] += vx1 * vy1 * v;
            if (ixp + 1 < blocks[1] && iyp >= 0)
                hist[(ixp + 1) * blocks[0] + iyp + best_o * BSQ] += vx0 * vy1 * v;
            if (ixp >= 0 && iyp + 1 < blocks[0])
                hist[ixp * blocks[0] + (iyp + 1) + best_o * BSQ] += vx1 * vy0 * v;
            if (ixp + 1 < blocks[1] && iyp + 1 < blocks[0])
                hist[(ixp + 1) * blocks[0] + (iyp + 1) + best_o * BSQ] += vx0 * vy0 * v;
        }
    }
    for (int o = 0; o < 9; o++) {
        const float *src1 = hist + o * BSQ;
        const float *src2 = hist + (o + 9) * BSQ;
        for (size_t i = 0; i < BSQ; i++) norm[i] += (src1[i] + src2[i]) * (src1[i] + src2[i]);
    }
    const size_t ODIM = (size_t)out[0] * out[1];
    for (int x = 0; x < out[1]; x++) {
        for (int y = 0; y < out[0]; y++) {
            float *dst = feat + x * out[0] + y;
            const float *src, *p;
            float n1, n2, n3, n4;
            p = norm + (x + 1) * blocks[0] + y + 1;
            n1 = 1.0 / sqrt(*p + *(p + 1) + *(p + blocks[0]) + *(p + blocks[0] + 1) + 0.0001);
            p = norm + (x + 1) * blocks[0] + y;
            n2 = 1.0 / sqrt(*p + *(p + 1) + *(p + blocks[0]) + *(p + blocks[0] + 1) + 0.0001);
            p = norm + x * blocks[0] + y + 1;
            n3 = 1.0 / sqrt(*p + *(p + 1) + *(p + blocks[0]) + *(p + blocks[0] + 1) + 0.0001);
            p = norm + x * blocks[0] + y;
            n4 = 1.0 / sqrt(*p + *(p + 1) + *(p + blocks[0]) + *(p + blocks[0] + 1) + 0.0001);
            float t1 = 0, t2 = 0, t3 = 0, t4 = 0;
            src = hist + (x + 1) * blocks[0] + (y + 1);
            for (int o = 0; o < 18; o++) {
                float h1 = min_2(*src * n1);
                float h2 = min_2(*src * n2);
                float h3 = min_2(*src * n3);
                float h4 = min_2(*src * n4);
                *dst = 0.5 * (h1 + h2 + h3 + h4);
                t1 += h1; t2 += h2; t3 += h3; t4 += h4;
                dst += ODIM;
                src += BSQ;
            }
            src = hist + (x + 1) * blocks[0] + (y + 1);
            for (int o = 0; o < 9; o++) {
                float sum = *src + *(src + 9 * BSQ);
                float h1 = min_2(sum * n1);
                float h2 = min_2(sum * n2);
                float h3 = min_2(sum * n3);
                float h4 = min_2(sum * n4);
                *dst = 0.5 * (h1 + h2 + h3 + h4);
                dst += ODIM;
                src += BSQ;
            }
            *dst = 0.2357 * t1; dst += ODIM;
            *dst = 0.2357 * t2; dst += ODIM;
            *dst = 0.2357 * t3; dst += ODIM;
            *dst = 0.2357 * t4;
        }
    }
    free(hist);
    free(norm);
    ftsize[0] = out[0];
    ftsize[1] = out[1];
}

/* ------------------------------------------------------------------------- */
/* Scale schedule: CAR_TRACKING/featurepyramid.cpp:174-239 (ini_scales).       */
/* Returns max_scale for an image of X x Y (width x height) without touching  */
/* the model's latch.                                                         */
/* ------------------------------------------------------------------------- */
int orc_max_scale(const orc_model *m, int width, int height)
{
    const int sbin = m->sbin;
    const int interval = m->interval;
    const float sc = pow(2.0, (1 / (double)interval));
    int max_scale = 36;
    const int L_NUM = interval + max_scale;
    float MRY = (float)m->rsize[0];
    float MRX = (float)m->rsize[1];
    for (int kk = 1; kk < m->numcomponent; kk++) {
        if (m->rsize[kk * 2] < MRY) MRY = m->rsize[kk * 2];
        if (m->rsize[kk * 2 + 1] < MRX) MRX = m->rsize[kk * 2 + 1];
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

/* ini_scales latch: the first image seen by a model fixes max_scale. */
int orc_ini_scales(orc_model *m, int width, int height)
{
    if (m->ini) {
        m->max_scale = orc_max_scale(m, width, height);
        m->ini = 0;
    }
    m->im_w = width;
    m->im_h = height;
    return m->max_scale;
}

/* ------------------------------------------------------------------------- */
/* Pyramid orchestration: CAR_TRACKING/featurepyramid.cpp.org:547-661.         */
/* Produces LEN = max_scale + interval levels.  Level ii (< interval) uses     */
/* sbin/2 on the image resized by 1/sc^ii; level ii+interval uses sbin on the  */
/* same image; level j+interval (j >= interval) resizes level j's image by     */
/* 0.5.  feats[l] is column-major [31][fs1][fs0]; caller frees with            */
/* orc_free_pyramid.                                                          */
/* ------------------------------------------------------------------------- */
static void pyr_level(orc_pyramid *P, int level, const float *img, const int *isize, int sbin)
{
    int fs[2];
    orc_feature_dims(isize[0], isize[1], sbin, fs);
    P->feat[level] = (float *)calloc((size_t)fs[0] * fs[1] * 31 + 1, sizeof(float));
    orc_calc_feature(img, isize[0], isize[1], sbin, fs, P->feat[level]);
    P->ftsize[2 * level] = fs[0];
    P->ftsize[2 * level + 1] = fs[1];
    P->imsize[2 * level] = isize[0];
    P->imsize[2 * level + 1] = isize[1];
}

orc_pyramid *orc_build_pyramid(const orc_model *m, int max_scale, const uint8_t *bgr,
                               int height, int width, int width_step, int nthreads)
{
    const int interval = m->interval;
    const int sbin = m->sbin;
    const int sbin2 = (int)floor((double)sbin / 2.0);
    const int LEN = max_scale + interval;
    const float sc = pow(2, (1.0 / (double)interval));
    orc_pyramid *P = (orc_pyramid *)calloc(1, sizeof(orc_pyramid));
    P->LEN = LEN;
    P->feat = (float **)calloc(LEN, sizeof(float *));
    P->ftsize = (int *)calloc(2 * LEN, sizeof(int));
    P->imsize = (int *)calloc(2 * LEN, sizeof(int));
    P->scales = (float *)calloc(LEN, sizeof(float));
    P->images = (float **)calloc(LEN, sizeof(float *));
    int INSIZE[3] = {height, width, 3};
    float *D_I = (float *)malloc(sizeof(float) * (size_t)height * width * 3);
    orc_ipl_to_float(bgr, height, width, width_step, D_I);

    /* Images: level ii and ii+interval share one image; octave chain after. */
    int *isz = (int *)calloc(3 * LEN, sizeof(int));
    for (int ii = 0; ii < interval; ii++) {
        float st = 1.0 / pow(sc, ii);
        int od[3];
        orc_resize_dims(INSIZE, st, od);
        P->images[ii] = (float *)malloc(sizeof(float) * (size_t)od[0] * od[1] * od[2] + 4);
        orc_resize(D_I, INSIZE, od, st, P->images[ii]);
        memcpy(isz + 3 * ii, od, sizeof(od));
        P->scales[ii] = st * 2;
        P->scales[ii + interval] = st;
        memcpy(isz + 3 * (ii + interval), od, sizeof(od));
        const float *RIM_T = P->images[ii];
        int RIS[3];
        memcpy(RIS, od, sizeof(od));
        for (int jj = ii + interval; jj < max_scale; jj += interval) {
            int O[3];
            orc_resize_dims(RIS, 0.5f, O);
            P->images[jj + interval] = (float *)malloc(sizeof(float) * (size_t)O[0] * O[1] * O[2] + 4);
            orc_resize(RIM_T, RIS, O, 0.5f, P->images[jj + interval]);
            memcpy(isz + 3 * (jj + interval), O, sizeof(O));
            memcpy(RIS, O, sizeof(O));
            P->scales[jj + interval] = 0.5 * (P->scales[jj]);
            RIM_T = P->images[jj + interval];
        }
    }
    free(D_I);
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads > 0 ? nthreads : 1)
#endif
    for (int l = 0; l < LEN; l++) {
        const float *img = (l >= interval && l < 2 * interval) ? P->images[l - interval] : P->images[l];
        pyr_level(P, l, img, isz + 3 * l, l < interval ? sbin2 : sbin);
    }
    (void)nthreads;
    free(isz);
    return P;
}

void orc_free_pyramid(orc_pyramid *P)
{
    if (!P) return;
    int interval_shared = 0;
    for (int l = 0; l < P->LEN; l++) {
        free(P->feat[l]);
        /* levels [interval, 2*interval) alias the base images and were never allocated */
        if (P->images[l]) free(P->images[l]);
    }
    (void)interval_shared;
    free(P->feat); free(P->ftsize); free(P->imsize); free(P->scales); free(P->images);
    free(P);
}

/* ------------------------------------------------------------------------- */
/* Filter convolution.  The reference's CPU fconvsMT body is absent           */
/* (declared at CAR_TRACKING/get_boxes_func.h:28); the arithmetic is restated */
/* from process_root/process_part, CAR_TRACKING/GPU_function.cu:302-358 and   */
/* :630-685: for each of the 31 features, val = sum over xp (outer) and yp    */
/* (inner) of A*B in that order; add_val accumulates val over the features;  */
/* the output is 0 + add_val.  Column-major everywhere:                       */
/*   A [f][x][y] (dims a0 x a1), B [f][xp][yp] (dims b0 x b1),                */
/*   C [x][y] (dims a0-b0+1 x a1-b1+1).                                       */
/* The innermost loop runs over output rows so the compiler may vectorise    */
/* across independent outputs; each output's own summation order is the     */
/* reference's.                                                              */
/* ------------------------------------------------------------------------- */
void orc_fconv(const float *A, int a0, int a1, const float *B, int b0, int b1, float *C)
{
    const int c0 = a0 - b0 + 1, c1 = a1 - b1 + 1;
    if (c0 < 1 || c1 < 1) return;
    const size_t ASQ = (size_t)a0 * a1, BSQ = (size_t)b0 * b1;
    float *val = (float *)malloc(sizeof(float) * c0);
    float *acc = (float *)malloc(sizeof(float) * c0);
    for (int x = 0; x < c1; x++) {
        for (int y = 0; y < c0; y++) acc[y] = 0;
        for (int f = 0; f < 31; f++) {
            const float *Af = A + f * ASQ;
            const float *Bf = B + f * BSQ;
            for (int y = 0; y < c0; y++) val[y] = 0;
            for (int xp = 0; xp < b1; xp++) {
                const float *Acol = Af + (size_t)(x + xp) * a0;
                for (int yp = 0; yp < b0; yp++) {
                    const float b = Bf[xp * b0 + yp];
                    const float *Ap = Acol + yp;
                    for (int y = 0; y < c0; y++) val[y] += Ap[y] * b;
                }
            }
            for (int y = 0; y < c0; y++) acc[y] += val[y];
        }
        for (int y = 0; y < c0; y++) C[(size_t)x * c0 + y] = 0.0f + acc[y];
    }
    free(val);
    free(acc);
}

/* Same loop nest in double precision, for measuring reduced-precision error. */
void orc_fconv_f64(const float *A, int a0, int a1, const float *B, int b0, int b1, double *C)
{
    const int c0 = a0 - b0 + 1, c1 = a1 - b1 + 1;
    if (c0 < 1 || c1 < 1) return;
    const size_t ASQ = (size_t)a0 * a1, BSQ = (size_t)b0 * b1;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int x = 0; x < c1; x++)
        for (int y = 0; y < c0; y++) {
            double acc = 0;
            for (int f = 0; f < 31; f++)
                for (int xp = 0; xp < b1; xp++)
                    for (int yp = 0; yp < b0; yp++)
                        acc += (double)A[f * ASQ + (size_t)(x + xp) * a0 + y + yp] * (double)B[f * BSQ + xp * b0 + yp];
            C[(size_t)x * c0 + y] = acc;
        }
}

/* Tensor-core operand emulation, for measuring what a reduced-precision      */
/* convolution does to detections (not the reference's arithmetic): each      */
/* operand is rounded to BF16 (round to nearest even), or split into a BF16   */
/* high part and the BF16 rounding of the remainder, and the products are     */
/* summed in double, then rounded to float.  mode 1: both operands BF16;      */
/* 2: both split, hi*hi + hi*lo + lo*hi; 3: features BF16, filters FP32;      */
/* 4: features split, filters BF16 (hi*b + lo*b); 5: TF32 operands (10-bit   */
/* mantissa, round to nearest even); 6: mode 2 for root filters, mode 1 for   */
/* part filters.                                                              */
static float bf16_rne(float x)
{
    uint32_t u;
    memcpy(&u, &x, 4);
    if ((u & 0x7f800000u) == 0x7f800000u) return x;
    u += 0x7fffu + ((u >> 16) & 1u);
    u &= 0xffff0000u;
    memcpy(&x, &u, 4);
    return x;
}

static float tf32_rne(float x)
{
    uint32_t u;
    memcpy(&u, &x, 4);
    if ((u & 0x7f800000u) == 0x7f800000u) return x;
    u += 0xfffu + ((u >> 13) & 1u);
    u &= 0xffffe000u;
    memcpy(&x, &u, 4);
    return x;
}

static int g_conv_emulation = 0;
void orc_set_conv_emulation(int mode) { g_conv_emulation = mode; }

static void fconv_emul(const float *A, int a0, int a1, const float *B, int b0, int b1, float *C, int mode)
{
    const int c0 = a0 - b0 + 1, c1 = a1 - b1 + 1;
    if (c0 < 1 || c1 < 1) return;
    const size_t ASQ = (size_t)a0 * a1, BSQ = (size_t)b0 * b1;
    float *Ah = (float *)malloc(sizeof(float) * 31 * ASQ), *Al = (float *)malloc(sizeof(float) * 31 * ASQ);
    float *Bh = (float *)malloc(sizeof(float) * 31 * BSQ), *Bl = (float *)malloc(sizeof(float) * 31 * BSQ);
    for (size_t i = 0; i < 31 * ASQ; i++) { Ah[i] = bf16_rne(A[i]); Al[i] = bf16_rne(A[i] - Ah[i]); }
    for (size_t i = 0; i < 31 * BSQ; i++) { Bh[i] = bf16_rne(B[i]); Bl[i] = bf16_rne(B[i] - Bh[i]); }
    for (int x = 0; x < c1; x++)
        for (int y = 0; y < c0; y++) {
            double acc = 0;
            for (int f = 0; f < 31; f++)
                for (int xp = 0; xp < b1; xp++)
                    for (int yp = 0; yp < b0; yp++) {
                        const size_t ia = f * ASQ + (size_t)(x + xp) * a0 + y + yp, ib = f * BSQ + xp * b0 + yp;
                        double p;
                        switch (mode) {
                        case 1: p = (double)Ah[ia] * Bh[ib]; break;
                        case 2: p = (double)Ah[ia] * Bh[ib] + (double)Ah[ia] * Bl[ib] + (double)Al[ia] * Bh[ib]; break;
                        case 3: p = (double)Ah[ia] * B[ib]; break;
                        case 5: p = (double)tf32_rne(A[ia]) * tf32_rne(B[ib]); break;
                        default: p = (double)Ah[ia] * Bh[ib] + (double)Al[ia] * Bh[ib]; break;
                        }
                        acc += p;
                    }
            C[(size_t)x * c0 + y] = (float)acc;
        }
    free(Ah); free(Al); free(Bh); free(Bl);
}

/* max over positions of sum |A| |B| (the magnitude that bounds rounding errors) */
static double fconv_abs_max(const float *A, int a0, int a1, const float *B, int b0, int b1)
{
    const int c0 = a0 - b0 + 1, c1 = a1 - b1 + 1;
    if (c0 < 1 || c1 < 1) return 0;
    const size_t ASQ = (size_t)a0 * a1, BSQ = (size_t)b0 * b1;
    double best = 0;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) reduction(max : best)
#endif
    for (int x = 0; x < c1; x++)
        for (int y = 0; y < c0; y++) {
            double acc = 0;
            for (int f = 0; f < 31; f++)
                for (int xp = 0; xp < b1; xp++)
                    for (int yp = 0; yp < b0; yp++)
                        acc += fabs((double)A[f * ASQ + (size_t)(x + xp) * a0 + y + yp]) * fabs((double)B[f * BSQ + xp * b0 + yp]);
            if (acc > best) best = acc;
        }
    return best;
}

/* ------------------------------------------------------------------------- */
/* Generalized distance transform: CAR_TRACKING/dt.cpp:61-85 (dt_helper),     */
/* :91-94 (dt1d), :101-136 (dt).                                              */
/* ------------------------------------------------------------------------- */
static void dt_helper(const float *src, float *dst, int *ptr, int step, int s1, int s2, int d1, int d2, float a, float b)
{
    while (d2 >= d1) {
        int d = (d1 + d2) >> 1;
        int s = s1;
        float src_ss = src[s * step];
        for (int p = s1 + 1; p <= s2; p++) {
            int t1 = d - s;
            int t2 = d - p;
            if (src_ss + a * t1 * t1 + b * t1 > src[p * step] + a * t2 * t2 + b * t2) {
                s = p;
                src_ss = src[s * step];
            }
        }
        int D = d - s;
        dst[d * step] = src[s * step] + a * D * D + b * D;
        ptr[d * step] = s;
        /* left half recursively, right half by iteration (same visiting set) */
        dt_helper(src, dst, ptr, step, s1, s, d1, d - 1, a, b);
        s1 = s;
        d1 = d + 1;
    }
}

/* vals/M/Ix/Iy column-major d0 x d1 (dims[0] = d0 rows along y). */
void orc_dt(const float *vals, float ax, float bx, float ay, float by, const int *dims, float *M, int *Ix, int *Iy)
{
    const int d0 = dims[0], d1 = dims[1];
    const size_t SQ = (size_t)d0 * d1;
    float *tmpM = (float *)malloc(sizeof(float) * SQ + 4);
    int *tmpIx = (int *)malloc(sizeof(int) * SQ + 4);
    int *tmpIy = (int *)malloc(sizeof(int) * SQ + 4);
    for (int x = 0; x < d1; x++)
        dt_helper(vals + (size_t)x * d0, tmpM + (size_t)x * d0, tmpIy + (size_t)x * d0, 1, 0, d0 - 1, 0, d0 - 1, ay, by);
    for (int y = 0; y < d0; y++)
        dt_helper(tmpM + y, M + y, tmpIx + y, d0, 0, d1 - 1, 0, d1 - 1, ax, bx);
    for (int x = 0; x < d1; x++)
        for (int y = 0; y < d0; y++) {
            size_t i = (size_t)x * d0 + y;
            Ix[i] = tmpIx[i];
            Iy[i] = tmpIy[(size_t)tmpIx[i] * d0 + y];
        }
    free(tmpM); free(tmpIx); free(tmpIy);
}

/* add_part_calculation: CAR_TRACKING/dt.cpp:38-55. */
void orc_add_part(float *score, const float *M, const int *rootsize, const int *partsize, int ax, int ay)
{
    float *S = score;
    int jj_L = ax + 2 * (rootsize[1] - 1) - 1;
    int ii_L = ay + 2 * (rootsize[0] - 1);
    int axm = ax - 1;
    for (int jj = axm; jj <= jj_L; jj += 2) {
        int L = jj * partsize[0];
        for (int ii = ay; ii <= ii_L; ii += 2) {
            *S -= M[ii + L - 1];
            S++;
        }
    }
}

/* ------------------------------------------------------------------------- */
/* Box geometry: CAR_TRACKING/get_boxes.cpp:227-235 (rootbox), :243-258       */
/* (partbox), :265-300 (calc_a_score, the CPU form; the GPU kernel at         */
/* GPU_function.cu:1176-1269 reads the wrong size words).                     */
/* ------------------------------------------------------------------------- */
void orc_rootbox(int x, int y, float scale, int padx, int pady, const int *rsize, float *Out)
{
    Out[0] = ((float)y - (float)pady + 1) * scale;
    Out[1] = ((float)x - (float)padx + 1) * scale;
    Out[2] = Out[0] + (float)rsize[0] * scale - 1.0;
    Out[3] = Out[1] + (float)rsize[1] * scale - 1.0;
}

/* Returns 0 when the probe falls inside the map; -1 when the reference would
 * read outside its buffer (the box is then filled from probe index 0). */
int orc_partbox(int x, int y, int ax, int ay, float scale, int padx, int pady, const int *psize,
                const int *lx, const int *ly, const int *ssize, float *Out)
{
    int probex = (x - 1) * 2 + ax;
    int probey = (y - 1) * 2 + ay;
    long P = probey + (long)probex * ssize[0];
    int rc = 0;
    if (P < 0 || P >= (long)ssize[0] * ssize[1]) { P = 0; rc = -1; }
    float px = (float)lx[P] + 1.0;
    float py = (float)ly[P] + 1.0;
    Out[0] = ((py - 2.0) / 2.0 + 1.0 - (float)pady) * scale;
    Out[1] = ((px - 2.0) / 2.0 + 1.0 - (float)padx) * scale;
    Out[2] = Out[0] + (float)psize[0] * scale / 2.0 - 1.0;
    Out[3] = Out[1] + (float)psize[1] * scale / 2.0 - 1.0;
    return rc;
}

void orc_calc_a_score(float *ac_score, const float *score, const int *ssize, const int *rsize,
                      int im_h, int im_w, int padx, int pady, float scale)
{
    const int IHEI = im_h, IWID = im_w;
    int block_pad = (int)(scale / 2.0);
    int RY = (int)((float)rsize[0] * scale / 2.0 - 1.0 + block_pad);
    int RX = (int)((float)rsize[1] * scale / 2.0 - 1.0 + block_pad);
    for (int ii = 0; ii < IWID; ii++) {
        int Xn = (int)((float)ii / scale + padx);
        for (int jj = 0; jj < IHEI; jj++) {
            int Yn = (int)((float)jj / scale + pady);
            if (Yn < ssize[0] && Xn < ssize[1]) {
                float sc = score[Yn + Xn * ssize[0]];
                int Im_Y = jj + RY;
                int Im_X = ii + RX;
                if (Im_Y < IHEI && Im_X < IWID) {
                    float *PP = ac_score + Im_Y + Im_X * IHEI;
                    if (sc > *PP) *PP = sc;
                }
            }
        }
    }
}

/* ------------------------------------------------------------------------- */
/* Scoring driver: CAR_TRACKING/get_boxes.cpp:583-1797 (get_boxes), CPU form. */
/* Root conv at levels [interval, LEN) (skipped when the level's features are */
/* smaller than max_Y x max_X), part conv at level-interval, score = root +   */
/* offw[ridx[c]], minus the part DT maps in part order, A_SCORE max per      */
/* level, threshold in column-major scan order, boxes, then A_SCORE offset    */
/* and normalisation.  Boxes are returned as [D][GL] with GL =               */
/* (numpart[0]+1)*4+3.  Also fills optional per-stage dumps for the tests.   */
/* ------------------------------------------------------------------------- */
static int level_skipped(const orc_model *m, const int *FSIZE, int level)
{
    return (FSIZE[level * 2] + 2 * m->pady < m->max_Y) || (FSIZE[level * 2 + 1] + 2 * m->padx < m->max_X);
}

orc_scores *orc_compute_scores(const orc_model *m, const orc_pyramid *P, int nthreads)
{
    const int interval = m->interval, LEN = P->LEN, NoC = m->numcomponent;
    const int *FSIZE = P->ftsize;
    orc_scores *S = (orc_scores *)calloc(1, sizeof(orc_scores));
    S->LEN = LEN; S->NoC = NoC; S->NoP = m->NoP; S->interval = interval;
    S->root = (float **)calloc((size_t)LEN * NoC, sizeof(float *));
    S->rsz = (int *)calloc((size_t)LEN * NoC * 2, sizeof(int));
    S->part = (float **)calloc((size_t)LEN * (m->NoP ? m->NoP : 1), sizeof(float *));
    S->psz = (int *)calloc((size_t)LEN * (m->NoP ? m->NoP : 1) * 2, sizeof(int));
    S->score = (float **)calloc((size_t)LEN * NoC, sizeof(float *));
    int maxnp = 0;
    for (int c = 0; c < NoC; c++) maxnp = imax(maxnp, m->numpart[c]);
    S->maxnp = maxnp;
    S->M = (float **)calloc((size_t)LEN * NoC * (maxnp ? maxnp : 1), sizeof(float *));
    S->Ix = (int **)calloc((size_t)LEN * NoC * (maxnp ? maxnp : 1), sizeof(int *));
    S->Iy = (int **)calloc((size_t)LEN * NoC * (maxnp ? maxnp : 1), sizeof(int *));
    S->skipped = (int *)calloc(LEN, sizeof(int));

    /* job list: (level, root filter) and (level, part filter) convolutions */
    int njobs = 0;
    int *jobs = (int *)malloc(sizeof(int) * 3 * (size_t)LEN * (NoC + m->NoP + 1));
    for (int level = interval; level < LEN; level++) {
        if (level_skipped(m, FSIZE, level)) { S->skipped[level] = 1; continue; }
        for (int j = 0; j < m->NoR && j < NoC; j++) { jobs[3 * njobs] = 0; jobs[3 * njobs + 1] = level; jobs[3 * njobs + 2] = j; njobs++; }
        for (int j = 0; j < m->NoP; j++) { jobs[3 * njobs] = 1; jobs[3 * njobs + 1] = level - interval; jobs[3 * njobs + 2] = j; njobs++; }
    }
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads > 0 ? nthreads : 1)
#endif
    for (int t = 0; t < njobs; t++) {
        int kind = jobs[3 * t], lv = jobs[3 * t + 1], j = jobs[3 * t + 2];
        const int a0 = FSIZE[2 * lv], a1 = FSIZE[2 * lv + 1];
        const int *bs = kind == 0 ? m->root_size + 3 * j : m->part_size + 3 * j;
        int c0 = a0 - bs[0] + 1, c1 = a1 - bs[1] + 1;
        if (c0 < 1 || c1 < 1) { c0 = c1 = 0; }
        float *C = (float *)calloc((size_t)(c0 > 0 ? c0 : 1) * (c1 > 0 ? c1 : 1), sizeof(float));
        if (c0 > 0 && g_conv_emulation)
            fconv_emul(P->feat[lv], a0, a1, kind == 0 ? m->rootfilter[j] : m->partfilter[j], bs[0], bs[1], C,
                       g_conv_emulation == 6 ? (kind == 0 ? 2 : 1) : g_conv_emulation);
        else if (c0 > 0)
            orc_fconv(P->feat[lv], a0, a1, kind == 0 ? m->rootfilter[j] : m->partfilter[j], bs[0], bs[1], C);
        if (kind == 0) { S->root[lv * NoC + j] = C; S->rsz[2 * (lv * NoC + j)] = c0; S->rsz[2 * (lv * NoC + j) + 1] = c1; }
        else { S->part[lv * m->NoP + j] = C; S->psz[2 * (lv * m->NoP + j)] = c0; S->psz[2 * (lv * m->NoP + j) + 1] = c1; }
    }
    free(jobs);

    /* DT jobs: (level, component, part) */
    int ndt = 0;
    int *dj = (int *)malloc(sizeof(int) * 3 * (size_t)LEN * NoC * (maxnp ? maxnp : 1) + 3);
    for (int level = interval; level < LEN; level++) {
        if (S->skipped[level]) continue;
        for (int c = 0; c < NoC; c++)
            for (int k = 0; k < m->numpart[c]; k++) { dj[3 * ndt] = level; dj[3 * ndt + 1] = c; dj[3 * ndt + 2] = k; ndt++; }
    }
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads > 0 ? nthreads : 1)
#endif
    for (int t = 0; t < ndt; t++) {
        int level = dj[3 * t], c = dj[3 * t + 1], k = dj[3 * t + 2];
        int L = level - interval;
        int pi = m->pidx[c][k], di = m->didx[c][k];
        int dims[2] = {S->psz[2 * (L * m->NoP + pi)], S->psz[2 * (L * m->NoP + pi) + 1]};
        size_t n = (size_t)dims[0] * dims[1];
        /* inverse_Q (GPU_function.cu:695-794): the DT runs on the negated map */
        float *neg = (float *)malloc(sizeof(float) * n + 4);
        const float *src = S->part[L * m->NoP + pi];
        for (size_t i = 0; i < n; i++) neg[i] = -src[i];
        size_t idx = ((size_t)level * NoC + c) * maxnp + k;
        S->M[idx] = (float *)malloc(sizeof(float) * n + 4);
        S->Ix[idx] = (int *)malloc(sizeof(int) * n + 4);
        S->Iy[idx] = (int *)malloc(sizeof(int) * n + 4);
        orc_dt(neg, m->def[4 * di], m->def[4 * di + 1], m->def[4 * di + 2], m->def[4 * di + 3], dims, S->M[idx], S->Ix[idx], S->Iy[idx]);
        free(neg);
    }
    free(dj);

    /* score assembly: root + offset, then subtract the part maps in order */
    for (int level = interval; level < LEN; level++) {
        if (S->skipped[level]) continue;
        int L = level - interval;
        for (int c = 0; c < NoC; c++) {
            int r0 = S->rsz[2 * (level * NoC + c)], r1 = S->rsz[2 * (level * NoC + c) + 1];
            size_t n = (size_t)r0 * r1;
            float *sc = (float *)malloc(sizeof(float) * n + 4);
            memcpy(sc, S->root[level * NoC + c], sizeof(float) * n);
            float off = m->offw[m->ridx[c]];
            for (size_t i = 0; i < n; i++) sc[i] += off;
            int R_S[2] = {r0, r1};
            for (int k = 0; k < m->numpart[c]; k++) {
                int pi = m->pidx[c][k], di = m->didx[c][k];
                int PS[2] = {S->psz[2 * (L * m->NoP + pi)], S->psz[2 * (L * m->NoP + pi) + 1]};
                int ax = m->anchor[di * 2] + 1, ay = m->anchor[di * 2 + 1] + 1;
                orc_add_part(sc, S->M[((size_t)level * NoC + c) * maxnp + k], R_S, PS, ax, ay);
            }
            S->score[level * NoC + c] = sc;
        }
    }
    return S;
}

/* The same lower-envelope recursion as dt_helper in double: only for measuring
 * the error of the FP32 and reduced-precision paths. */
static void dt_helper_f64(const double *src, double *dst, int step, int s1, int s2, int d1, int d2, double a, double b)
{
    while (d2 >= d1) {
        int d = (d1 + d2) >> 1;
        int s = s1;
        for (int p = s1 + 1; p <= s2; p++) {
            double t1 = d - s, t2 = d - p;
            if (src[s * step] + a * t1 * t1 + b * t1 > src[p * step] + a * t2 * t2 + b * t2) s = p;
        }
        double D = d - s;
        dst[d * step] = src[s * step] + a * D * D + b * D;
        dt_helper_f64(src, dst, step, s1, s, d1, d - 1, a, b);
        s1 = s;
        d1 = d + 1;
    }
}

int orc_score_f64(const orc_model *m, const orc_pyramid *P, int level, int c, double *out, int *dims, double *mag)
{
    const int interval = m->interval, L = level - interval;
    const int *FSIZE = P->ftsize;
    if (level < interval || level >= P->LEN || level_skipped(m, FSIZE, level)) return -1;
    const int a0 = FSIZE[2 * level], a1 = FSIZE[2 * level + 1];
    const int *rs = m->root_size + 3 * c;
    const int r0 = a0 - rs[0] + 1, r1 = a1 - rs[1] + 1;
    if (r0 < 1 || r1 < 1) return -1;
    dims[0] = r0; dims[1] = r1;
    orc_fconv_f64(P->feat[level], a0, a1, m->rootfilter[c], rs[0], rs[1], out);
    if (mag) *mag = fconv_abs_max(P->feat[level], a0, a1, m->rootfilter[c], rs[0], rs[1]);
    const double off = m->offw[m->ridx[c]];
    for (size_t i = 0; i < (size_t)r0 * r1; i++) out[i] += off;
    const int p0 = FSIZE[2 * L], p1 = FSIZE[2 * L + 1];
    for (int k = 0; k < m->numpart[c]; k++) {
        const int pi = m->pidx[c][k], di = m->didx[c][k];
        const int *ps = m->part_size + 3 * pi;
        const int d0 = p0 - ps[0] + 1, d1 = p1 - ps[1] + 1;
        const size_t n = (size_t)d0 * d1;
        double *v = (double *)malloc(sizeof(double) * n + 8);
        double *t = (double *)malloc(sizeof(double) * n + 8);
        double *M = (double *)malloc(sizeof(double) * n + 8);
        orc_fconv_f64(P->feat[L], p0, p1, m->partfilter[pi], ps[0], ps[1], v);
        if (mag) *mag += fconv_abs_max(P->feat[L], p0, p1, m->partfilter[pi], ps[0], ps[1]);
        for (size_t i = 0; i < n; i++) v[i] = -v[i];
        const double ax = m->def[4 * di], bx = m->def[4 * di + 1], ay = m->def[4 * di + 2], by = m->def[4 * di + 3];
        for (int x = 0; x < d1; x++) dt_helper_f64(v + (size_t)x * d0, t + (size_t)x * d0, 1, 0, d0 - 1, 0, d0 - 1, ay, by);
        for (int y = 0; y < d0; y++) dt_helper_f64(t + y, M + y, d0, 0, d1 - 1, 0, d1 - 1, ax, bx);
        const int pax = m->anchor[di * 2] + 1, pay = m->anchor[di * 2 + 1] + 1;
        for (int x = 0; x < r1; x++)
            for (int y = 0; y < r0; y++)
                out[(size_t)x * r0 + y] -= M[(size_t)(pax - 1 + 2 * x) * d0 + (pay - 1 + 2 * y)];
        free(v); free(t); free(M);
    }
    return 0;
}

void orc_free_scores(orc_scores *S)
{
    if (!S) return;
    size_t n1 = (size_t)S->LEN * S->NoC;
    for (size_t i = 0; i < n1; i++) { free(S->root[i]); free(S->score[i]); }
    for (size_t i = 0; i < (size_t)S->LEN * (S->NoP ? S->NoP : 1); i++) free(S->part[i]);
    for (size_t i = 0; i < n1 * (S->maxnp ? S->maxnp : 1); i++) { free(S->M[i]); free(S->Ix[i]); free(S->Iy[i]); }
    free(S->root); free(S->score); free(S->part); free(S->M); free(S->Ix); free(S->Iy);
    free(S->rsz); free(S->psz); free(S->skipped);
    free(S);
}

/* Boxes + A_SCORE from precomputed scores.  a_score (H*W, column-major)
 * must hold the caller's initial values (ini_ac_score fills -100).  Returns
 * malloc'ed [D][GL]; *Dnum gets D; *probe_oob counts partbox probes that fell
 * outside their map. */
float *orc_boxes_from_scores(const orc_model *m, const orc_pyramid *P, const orc_scores *S,
                             float thresh, float *a_score, int *Dnum, int *probe_oob)
{
    const int interval = m->interval, LEN = P->LEN, NoC = m->numcomponent;
    const int GL = (m->numpart[0] + 1) * 4 + 3;
    int D = 0, oob = 0;
    for (int level = interval; level < LEN; level++) {
        if (S->skipped[level]) continue;
        for (int c = 0; c < NoC; c++) {
            int n = S->rsz[2 * (level * NoC + c)] * S->rsz[2 * (level * NoC + c) + 1];
            const float *sc = S->score[level * NoC + c];
            for (int i = 0; i < n; i++) if (sc[i] > thresh) D++;
        }
    }
    float *boxes = (float *)calloc((size_t)(D ? D : 1) * GL, sizeof(float));
    float *T = boxes;
    for (int level = interval; level < LEN; level++) {
        if (S->skipped[level]) continue;
        int L = level - interval;
        float scale = (float)m->sbin / P->scales[level];
        for (int c = 0; c < NoC; c++) {
            int R_S[2] = {S->rsz[2 * (level * NoC + c)], S->rsz[2 * (level * NoC + c) + 1]};
            const float *sc = S->score[level * NoC + c];
            int RSIZE[2] = {m->rsize[c * 2], m->rsize[c * 2 + 1]};
            if (a_score) orc_calc_a_score(a_score, sc, R_S, RSIZE, m->im_h, m->im_w, m->padx, m->pady, scale);
        }
        for (int c = 0; c < NoC; c++) {
            int R_S[2] = {S->rsz[2 * (level * NoC + c)], S->rsz[2 * (level * NoC + c) + 1]};
            const float *sc = S->score[level * NoC + c];
            int RSIZE[2] = {m->rsize[c * 2], m->rsize[c * 2 + 1]};
            int n = R_S[0] * R_S[1];
            for (int i = 0; i < n; i++) {
                if (!(sc[i] > thresh)) continue;
                int y = i % R_S[0], x = i / R_S[0];
                orc_rootbox(x, y, scale, m->padx, m->pady, RSIZE, T);
                float *Pt = T + 4;
                for (int k = 0; k < m->numpart[c]; k++) {
                    int pi = m->pidx[c][k], di = m->didx[c][k];
                    int PB[2] = {m->psize[c][k * 2], m->psize[c][k * 2 + 1]};
                    int Is[2] = {S->psz[2 * (L * m->NoP + pi)], S->psz[2 * (L * m->NoP + pi) + 1]};
                    size_t idx = ((size_t)level * NoC + c) * S->maxnp + k;
                    if (orc_partbox(x, y, m->anchor[di * 2] + 1, m->anchor[di * 2 + 1] + 1, scale, m->padx, m->pady,
                                    PB, S->Ix[idx], S->Iy[idx], Is, Pt)) oob++;
                    Pt += 4;
                }
                *(Pt++) = (float)c;
                *(Pt++) = sc[x * R_S[0] + y];
                *Pt = scale;
                T += GL;
            }
        }
    }
    if (a_score) orc_normalize_a_score(a_score, m->im_h * m->im_w, thresh);
    *Dnum = D;
    if (probe_oob) *probe_oob = oob;
    return boxes;
}

/* get_boxes.cpp:1765-1787.  AS_OFF = abs(thresh) resolves to the float
 * overload of abs in the reference's translation unit. */
void orc_normalize_a_score(float *A, int n, float thresh)
{
    float AS_OFF = fabsf(thresh);
    float max_ac = 0.0;
    for (int i = 0; i < n; i++) {
        if (A[i] < thresh) A[i] = 0.0;
        else {
            A[i] += AS_OFF;
            if (A[i] > max_ac) max_ac = A[i];
        }
    }
    if (max_ac > 0.0) {
        float ac_ratio = 1.0 / max_ac;
        for (int i = 0; i < n; i++) A[i] *= ac_ratio;
    }
}

/* ------------------------------------------------------------------------- */
/* NMS: CAR_TRACKING/nms.cpp:70-84 (quickSort), :94-217 (nms).                 */
/* ------------------------------------------------------------------------- */
void orc_quicksort(float *ary, int *Order, int first_index, int last_index)
{
    for (;;) {
        int i = first_index, j = last_index;
        float key = ary[(first_index + last_index) / 2];
        for (;;) {
            while (ary[i] > key) i++;
            while (ary[j] < key) j--;
            if (i >= j) break;
            float tv = ary[i]; ary[i] = ary[j]; ary[j] = tv;
            int to = Order[i]; Order[i] = Order[j]; Order[j] = to;
            i++; j--;
        }
        if (first_index < i - 1) orc_quicksort(ary, Order, first_index, i - 1);
        if (last_index > j + 1) { first_index = j + 1; continue; }
        break;
    }
}

static inline float max_d(float x, float y) { return (x >= y ? x : y); }
static inline float min_d(float x, float y) { return (x <= y ? x : y); }

/* Returns the kept count; keep[] (size NUM, in input index order) gets 1 for
 * emitted boxes; order[] (optional, size NUM) gets the sorted permutation. */
int orc_nms_keep(const float *boxes, int NUM, int GL, float overlap, int *keep, int *order_out)
{
    if (NUM <= 0) return 0;
    float *area = (float *)calloc(NUM, sizeof(float));
    float *scores = (float *)calloc(NUM, sizeof(float));
    int *sorted = (int *)calloc(NUM, sizeof(int));
    int *checked = (int *)calloc(NUM, sizeof(int));
    for (int i = 0; i < NUM; i++) {
        const float *P = boxes + (size_t)GL * i;
        area[i] = (P[3] - P[1] + 1.0) * (P[2] - P[0] + 1.0);
        scores[i] = P[GL - 2];
        sorted[i] = i;
    }
    orc_quicksort(scores, sorted, 0, NUM - 1);
    if (order_out) memcpy(order_out, sorted, sizeof(int) * NUM);
    int cnum = NUM - 1, cur = 0, pi_num = 0;
    while (cnum > 0) {
        int A = sorted[cur];
        const float *P = boxes + (size_t)GL * A;
        float Ay1 = P[0], Ax1 = P[1], Ay2 = P[2], Ax2 = P[3];
        checked[A] = 1;
        cnum--;
        cur++;
        pi_num++;
        for (int kk = cur; kk < NUM; kk++) {
            int B = sorted[kk];
            if (checked[B] != 0) continue;
            P = boxes + (size_t)GL * B;
            float yy1 = max_d(Ay1, P[0]);
            float xx1 = max_d(Ax1, P[1]);
            float yy2 = min_d(Ay2, P[2]);
            float xx2 = min_d(Ax2, P[3]);
            float w = xx2 - xx1 + 1.0;
            float h = yy2 - yy1 + 1.0;
            float R_AREA = min_d(area[A], area[B]);
            if (w > 0 && h > 0) {
                float o = w * h / R_AREA;
                if (o > overlap) { checked[B] = -1; cnum--; }
            } else if (Ay1 < P[0] && Ax1 < P[1] && Ay2 > P[2] && Ax2 > P[3]) {
                checked[B] = -1; cnum--;
            } else if (Ay1 > P[0] && Ax1 > P[1] && Ay2 < P[2] && Ax2 < P[3]) {
                checked[B] = -1; cnum--;
            }
        }
        for (int kk = cur; kk < NUM; kk++)
            if (checked[sorted[kk]] == 0) { cur = kk; break; }
    }
    for (int i = 0; i < NUM; i++) keep[i] = checked[i] == 1;
    free(area); free(scores); free(sorted); free(checked);
    return pi_num;
}

/* ------------------------------------------------------------------------- */
/* Box regression: CAR_TRACKING/tracking.cpp:90-166 (get_new_rects).           */
/* point[4k..] = x1,y1,x2,y2 clamped to the image; or_point divided by ratio.  */
/* ------------------------------------------------------------------------- */
void orc_get_new_rects(const orc_model *m, const float *boxes, int NUM, int img_w, int img_h,
                       int *point, int *or_point, int *type, float *scale, float *score)
{
    const int GL = (m->numpart[0] + 1) * 4 + 3;
    const int LL = GL - 3;
    const int ML = 1 + 2 * (1 + m->numpart[0]);
    float *Avec = (float *)calloc(ML, sizeof(float));
    for (int ii = 0; ii < NUM; ii++) {
        const float *P = boxes + (size_t)GL * ii;
        float *Av = Avec;
        int CNUM = (int)(*(P + GL - 3));
        int PP[4];
        *(Av++) = P[3] - P[1];
        for (int kk = 0; kk < LL; kk += 4) { *(Av++) = P[kk + 1]; *(Av++) = P[kk]; }
        float XP1 = 0, XP2 = 0, YP1 = 0, YP2 = 0;
        const float *x1 = m->x1[CNUM], *x2 = m->x2[CNUM], *y1 = m->y1[CNUM], *y2 = m->y2[CNUM];
        for (int kk = 0; kk < ML; kk++) {
            YP1 += Avec[kk] * y1[kk]; YP2 += Avec[kk] * y2[kk];
            XP1 += Avec[kk] * x1[kk]; XP2 += Avec[kk] * x2[kk];
        }
        PP[0] = XP1 > 0 ? (int)XP1 : 0;
        PP[1] = YP1 > 0 ? (int)YP1 : 0;
        PP[2] = XP2 < img_w ? (int)XP2 : img_w;
        PP[3] = YP2 < img_h ? (int)YP2 : img_h;
        memcpy(point + 4 * ii, PP, sizeof(PP));
        scale[ii] = *(P + GL - 1);
        score[ii] = *(P + GL - 2);
        type[ii] = CNUM;
        for (int q = 0; q < 4; q++) or_point[4 * ii + q] = (int)((float)PP[q] / m->ratio);
    }
    free(Avec);
}

/* ------------------------------------------------------------------------- */
/* Whole path: CAR_TRACKING/detect.cpp:151-276 (detect + car_detection).       */
/* ------------------------------------------------------------------------- */
int orc_car_detection(orc_model *m, const uint8_t *bgr, int height, int width, int width_step,
                      float thresh, float overlap, float *a_score, int nthreads, orc_detection *out)
{
    int max_scale = orc_ini_scales(m, width, height);
    orc_pyramid *P = orc_build_pyramid(m, max_scale, bgr, height, width, width_step, nthreads);
    orc_scores *S = orc_compute_scores(m, P, nthreads);
    int D = 0, oob = 0;
    float *boxes = orc_boxes_from_scores(m, P, S, thresh, a_score, &D, &oob);
    const int GL = (m->numpart[0] + 1) * 4 + 3;
    int *keep = (int *)calloc(D ? D : 1, sizeof(int));
    int K = orc_nms_keep(boxes, D, GL, overlap, keep, NULL);
    float *kept = (float *)calloc((size_t)(K ? K : 1) * GL, sizeof(float));
    for (int i = 0, k = 0; i < D; i++)
        if (keep[i]) memcpy(kept + (size_t)GL * (k++), boxes + (size_t)GL * i, sizeof(float) * GL);
    memset(out, 0, sizeof(*out));
    out->D = D;
    out->GL = GL;
    out->boxes = boxes;
    out->K = K;
    out->kept = kept;
    out->probe_oob = oob;
    out->point = (int *)calloc(4 * (K ? K : 1), sizeof(int));
    out->or_point = (int *)calloc(4 * (K ? K : 1), sizeof(int));
    out->type = (int *)calloc(K ? K : 1, sizeof(int));
    out->scale = (float *)calloc(K ? K : 1, sizeof(float));
    out->score = (float *)calloc(K ? K : 1, sizeof(float));
    orc_get_new_rects(m, kept, K, width, height, out->point, out->or_point, out->type, out->scale, out->score);
    free(keep);
    orc_free_scores(S);
    orc_free_pyramid(P);
    return 0;
}

void orc_free_detection(orc_detection *d)
{
    if (!d) return;
    free(d->boxes); free(d->kept); free(d->point); free(d->or_point); free(d->type); free(d->scale); free(d->score);
    memset(d, 0, sizeof(*d));
}

void orc_free(void *p) { free(p); }
