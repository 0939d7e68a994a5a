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

}
