/*
 * Flat C entry points over the reference's own CPU functions, so the test
 * suite can call them through ctypes.  TEST INFRASTRUCTURE ONLY: this file
 * only marshals arguments; every result comes from the reference's code.
 */
#include <stdlib.h>
#include <string.h>
#include "cv.h"
#include "MODEL_info.h"
#include "switch_float.h"

/* reference functions (C++ linkage), declared as in their translation units */
FLOAT *resize(FLOAT *src, int *sdims, int *odims, FLOAT scale);                   /* resize.cc:135 */
FLOAT *calc_feature(FLOAT *SRC, int *ISIZE, int *FTSIZE, int sbin);               /* featurepyramid.cpp:263 */
FLOAT *ini_scales(Model_info *MI, IplImage *IM, int X, int Y);                     /* featurepyramid.cpp:174 */
FLOAT *dt(FLOAT *vals, FLOAT ax, FLOAT bx, FLOAT ay, FLOAT by, int *dims, int *Ix, int *Iy); /* dt.cpp:101 */
void add_part_calculation(FLOAT *score, FLOAT *M, int *rootsize, int *partsize, int ax, int ay); /* dt.cpp:38 */
int *get_gmpc(FLOAT *score, FLOAT thresh, int *ssize, int *GMN);                  /* get_boxes.cpp:185 */
FLOAT *rootbox(int x, int y, FLOAT scale, int padx, int pady, int *rsize);        /* get_boxes.cpp:227 */
FLOAT *partbox(int x, int y, int ax, int ay, FLOAT scale, int padx, int pady, int *psize, int *lx, int *ly, int *ssize); /* :243 */
void calc_a_score(FLOAT *ac_score, FLOAT *score, int *ssize, int *rsize, Model_info *MI, FLOAT scale); /* :265 */
FLOAT *nms(FLOAT *boxes, FLOAT overlap, int *num, MODEL *MO);                      /* nms.cpp:94 */
void quickSort(FLOAT *ary, int *Order, int first_index, int last_index);          /* nms.cpp:70 */
FLOAT *flip_feat(FLOAT *feat, int *size);                                          /* get_boxes.cpp:121 */
Model_info *load_modelinfo(char *filename);                                        /* load_model.cpp:57 */
Rootfilters *load_rootfilter(char *filename);                                      /* load_model.cpp:250 */
Partfilters *load_partfilter(char *filename);                                      /* load_model.cpp:390 */
extern int sum_size_def_array;                                                     /* load_model.cpp:25, set at :178 */
RESULT *get_new_rects(IplImage *Image, MODEL *MO, FLOAT *boxes, int *NUM);         /* tracking.cpp:90 */

/* get_new_rects logs every box to this file (main.cpp opens it) */
FILE *resFP;

extern "C" {

void ref_free(void *p) { free(p); }

/* dst sized by the caller from odims computed the same way */
void ref_resize(float *src, int *sdims, int *odims, float scale, float *dst)
{
    FLOAT *r = resize(src, sdims, odims, scale);
    memcpy(dst, r, sizeof(FLOAT) * (size_t)odims[0] * odims[1] * odims[2]);
    free(r);
}

/* out holds size[0]*size[1]*size[2] floats; the reference's result is pinned
 * memory on the GPU build (cuMemHostAlloc, a calloc stub here) */
void ref_flip_feat(float *feat, int *size, float *out)
{
    FLOAT *f = flip_feat(feat, size);
    memcpy(out, f, sizeof(FLOAT) * (size_t)size[0] * size[1] * size[2]);
    free(f);
}

void ref_calc_feature(float *src, int *isize, int sbin, int *ftsize, float *feat)
{
    FLOAT *f = calc_feature(src, isize, ftsize, sbin);
    memcpy(feat, f, sizeof(FLOAT) * (size_t)ftsize[0] * ftsize[1] * 31);
    free(f);
}

int ref_max_scale(int numcomponent, int sbin, int interval, int *rsize, int width, int height)
{
    Model_info MI;
    memset(&MI, 0, sizeof(MI));
    MI.numcomponent = numcomponent;
    MI.sbin = sbin;
    MI.interval = interval;
    MI.rsize = rsize;
    MI.ini = true;
    IplImage im;
    memset(&im, 0, sizeof(im));
    im.width = width;
    im.height = height;
    FLOAT *s = ini_scales(&MI, &im, width, height);
    free(s);
    return MI.max_scale;
}

void ref_dt(float *vals, float ax, float bx, float ay, float by, int *dims, float *M, int *Ix, int *Iy)
{
    FLOAT *m = dt(vals, ax, bx, ay, by, dims, Ix, Iy);
    memcpy(M, m, sizeof(FLOAT) * (size_t)dims[0] * dims[1]);
    free(m);
}

void ref_add_part(float *score, float *M, int *rootsize, int *partsize, int ax, int ay)
{
    add_part_calculation(score, M, rootsize, partsize, ax, ay);
}

int ref_get_gmpc(float *score, float thresh, int *ssize, int *out, int cap)
{
    int n = 0;
    int *g = get_gmpc(score, thresh, ssize, &n);
    memcpy(out, g, sizeof(int) * 2 * (size_t)(n < cap ? n : cap));
    free(g);
    return n;
}

void ref_rootbox(int x, int y, float scale, int padx, int pady, int *rsize, float *out)
{
    FLOAT *b = rootbox(x, y, scale, padx, pady, rsize);
    memcpy(out, b, sizeof(FLOAT) * 4);
    free(b);
}

void ref_partbox(int x, int y, int ax, int ay, float scale, int padx, int pady, int *psize, int *lx, int *ly, int *ssize, float *out)
{
    FLOAT *b = partbox(x, y, ax, ay, scale, padx, pady, psize, lx, ly, ssize);
    memcpy(out, b, sizeof(FLOAT) * 4);
    free(b);
}

void ref_calc_a_score(float *ac, float *score, int *ssize, int *rsize, int im_h, int im_w, int padx, int pady, int sbin, float scale)
{
    Model_info MI;
    memset(&MI, 0, sizeof(MI));
    MI.IM_HEIGHT = im_h;
    MI.IM_WIDTH = im_w;
    MI.padx = padx;
    MI.pady = pady;
    MI.sbin = sbin;
    calc_a_score(ac, score, ssize, rsize, &MI, scale);
}

/* keep[] gets 1 for every input box that nms() emits (output is in input order) */
int ref_nms(float *boxes, int num, int numpart0, float overlap, int *keep)
{
    Model_info MI;
    memset(&MI, 0, sizeof(MI));
    int np = numpart0;
    MI.numpart = &np;
    MODEL MO;
    MO.MI = &MI;
    MO.RF = NULL;
    MO.PF = NULL;
    int n = num;
    const int GL = (numpart0 + 1) * 4 + 3;
    FLOAT *out = nms(boxes, overlap, &n, &MO);
    for (int i = 0; i < num; i++) keep[i] = 0;
    /* match emitted records back to their input rows (records are unique rows in order) */
    int j = 0;
    for (int i = 0; i < num && j < n; i++)
        if (memcmp(boxes + (size_t)GL * i, out + (size_t)GL * j, sizeof(FLOAT) * GL) == 0) { keep[i] = 1; j++; }
    free(out);
    return n;
}

void ref_quicksort(float *ary, int *order, int first, int last) { quickSort(ary, order, first, last); }

/* get_new_rects (tracking.cpp:90-166) on kept boxes [num][GL] of a model loaded by
 * the reference's loader; fills point/or_point (4 ints a box), type, scale, score. */
int ref_get_new_rects(const char *comp, const char *root, const char *part, float ratio, float *boxes, int num,
                      int img_w, int img_h, int *point, int *or_point, int *type, float *scale, float *score)
{
    if (!resFP) resFP = fopen("/dev/null", "w");
    MODEL MO;
    MO.MI = load_modelinfo((char *)comp);
    MO.RF = NULL;
    MO.PF = NULL;
    MO.MI->ratio = ratio;
    IplImage im;
    memset(&im, 0, sizeof(im));
    im.width = img_w;
    im.height = img_h;
    int n = num;
    RESULT *R = get_new_rects(&im, &MO, boxes, &n);
    for (int i = 0; i < R->num; i++) {
        memcpy(point + 4 * i, R->point + 4 * i, sizeof(int) * 4);
        memcpy(or_point + 4 * i, R->OR_point + 4 * i, sizeof(int) * 4);
        type[i] = R->type[i];
        scale[i] = R->scale[i];
        score[i] = R->score[i];
    }
    return R->num;
}

/* Loads a model CSV triple with the reference's own loader functions and
 * writes every parsed field, in a fixed order, into out[] as floats (the
 * integers are small, so exact):
 *   numcomponent sbin interval max_Y max_X padx pady
 *   per component: ridx oidx offw rsize[0] rsize[1] numpart,
 *                  then per part: pidx didx psize[0] psize[1]
 *   DefL, def[4*DefL], anchor[2*DefL]
 *   per component: x1[GL] y1[GL] x2[GL] y2[GL]   (GL = 1+2*(1+numpart))
 *   NoR, per root: size[3] rootsym weights[size0*size1*size2]
 *   NoP, per part: size[3] part_partner part_sym weights[...]
 * Returns the number of floats (written only while below cap). */
int ref_load_model_dump(const char *comp, const char *root, const char *part, float *out, int cap)
{
    Model_info *MI = load_modelinfo((char *)comp);
    Rootfilters *RF = load_rootfilter((char *)root);
    Partfilters *PF = load_partfilter((char *)part);
    int n = 0;
#define PUT(v) do { if (n < cap) out[n] = (float)(v); n++; } while (0)
    PUT(MI->numcomponent); PUT(MI->sbin); PUT(MI->interval); PUT(MI->max_Y); PUT(MI->max_X);
    PUT(MI->padx); PUT(MI->pady);
    for (int c = 0; c < MI->numcomponent; c++) {
        PUT(MI->ridx[c]); PUT(MI->oidx[c]); PUT(MI->offw[c]); PUT(MI->rsize[2 * c]); PUT(MI->rsize[2 * c + 1]);
        PUT(MI->numpart[c]);
        for (int k = 0; k < MI->numpart[c]; k++) {
            PUT(MI->pidx[c][k]); PUT(MI->didx[c][k]); PUT(MI->psize[c][2 * k]); PUT(MI->psize[c][2 * k + 1]);
        }
    }
    /* DefL is not kept in Model_info; the loader leaves 4*DefL floats' bytes in this global */
    const int defl = sum_size_def_array / (int)(4 * sizeof(FLOAT));
    PUT(defl);
    for (int i = 0; i < 4 * defl; i++) PUT(MI->def[i]);
    for (int i = 0; i < 2 * defl; i++) PUT(MI->anchor[i]);
    for (int c = 0; c < MI->numcomponent; c++) {
        const int GL = 1 + 2 * (1 + MI->numpart[c]);
        for (int j = 0; j < GL; j++) PUT(MI->x1[c][j]);
        for (int j = 0; j < GL; j++) PUT(MI->y1[c][j]);
        for (int j = 0; j < GL; j++) PUT(MI->x2[c][j]);
        for (int j = 0; j < GL; j++) PUT(MI->y2[c][j]);
    }
    PUT(RF->NoR);
    for (int r = 0; r < RF->NoR; r++) {
        const int *sz = RF->root_size[r];
        PUT(sz[0]); PUT(sz[1]); PUT(sz[2]); PUT(RF->rootsym[r]);
        for (int i = 0; i < sz[0] * sz[1] * sz[2]; i++) PUT(RF->rootfilter[r][i]);
    }
    PUT(PF->NoP);
    for (int p = 0; p < PF->NoP; p++) {
        const int *sz = PF->part_size[p];
        PUT(sz[0]); PUT(sz[1]); PUT(sz[2]); PUT(PF->part_partner[p]); PUT(PF->part_sym[p]);
        for (int i = 0; i < sz[0] * sz[1] * sz[2]; i++) PUT(PF->partfilter[p][i]);
    }
#undef PUT
    /* the loader's allocations are left to the process: a test helper, called a few times */
    return n;
}

}
