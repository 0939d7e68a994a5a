/*
 * dpm_oracle.h -- CPU restatement of CPFL/geye's DPM detection path.
 * TEST INFRASTRUCTURE ONLY (the oracle); see dpm_oracle.c for the rules.
 */
#ifndef GEYE_DPM_ORACLE_H
#define GEYE_DPM_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Mirror of MODEL / Model_info / Rootfilters / Partfilters
 * (CAR_TRACKING/MODEL_info.h:75-142). */
typedef struct {
    int numcomponent, sbin, interval, max_X, max_Y, padx, pady, max_scale, im_w, im_h;
    int ini;
    float ratio;
    int *ridx, *oidx;
    float *offw;
    int *rsize, *numpart;
    int **pidx, **didx, **psize;
    int DefL;
    float *def;
    int *anchor;
    float **x1, **y1, **x2, **y2;
    int NoR;
    int *root_size;   /* NoR x 3 */
    float **rootfilter;
    int NoP;
    int *part_size;   /* NoP x 3 */
    float **partfilter;
    int *part_partner;
} orc_model;

typedef struct {
    int LEN;
    float **feat;     /* per level, column-major [31][fs1][fs0] */
    int *ftsize;      /* LEN x 2 (fs0 = rows/y, fs1 = cols/x) */
    int *imsize;      /* LEN x 2 image size (h, w) the level was computed on */
    float *scales;    /* LEN */
    float **images;   /* resized images (levels [interval,2*interval) alias) */
} orc_pyramid;

typedef struct {
    int LEN, NoC, NoP, interval, maxnp;
    float **root;     /* [level*NoC + c] root conv map, column-major */
    int *rsz;         /* [level*NoC + c] x 2 */
    float **part;     /* [L*NoP + p] part conv map at level L */
    int *psz;         /* [L*NoP + p] x 2 */
    float **M;        /* [(level*NoC + c)*maxnp + k] DT value map */
    int **Ix, **Iy;
    float **score;    /* [level*NoC + c] final score map */
    int *skipped;     /* per level */
} orc_scores;

typedef struct {
    int D, GL, K, probe_oob;
    float *boxes;     /* [D][GL] before NMS */
    float *kept;      /* [K][GL] after NMS, input order */
    int *point, *or_point, *type;
    float *scale, *score;
} orc_detection;

orc_model *orc_model_load(const char *comp, const char *root, const char *part, float ratio);
void orc_model_free(orc_model *m);

void orc_ipl_to_float(const uint8_t *bgr, int height, int width, int width_step, float *out);
int orc_resize_taps(int sheight, int dheight, int *si, int *di, float *alpha, int cap);
void orc_resize_dims(const int *sdims, float scale, int *odims);
void orc_resize(const float *src, const int *sdims, int *odims, float scale, float *dst);
void orc_feature_dims(int height, int width, int sbin, int *ftsize);
int orc_hog_pixel(const float *SRC, int height, int width, int x, int y, float *vout);
void orc_calc_feature(const float *SRC, int height, int width, int sbin, int *ftsize, float *feat);
int orc_max_scale(const orc_model *m, int width, int height);
int orc_ini_scales(orc_model *m, int width, int height);
orc_pyramid *orc_build_pyramid(const orc_model *m, int max_scale, const uint8_t *bgr,
                               int height, int width, int width_step, int nthreads);
void orc_free_pyramid(orc_pyramid *P);
void orc_fconv(const float *A, int a0, int a1, const float *B, int b0, int b1, float *C);
void orc_fconv_f64(const float *A, int a0, int a1, const float *B, int b0, int b1, double *C);
/* 0 (default): the reference's FP32 convolution; 1-4: tensor-core operand
 * emulation (BF16 / split BF16), see dpm_oracle.c; process-wide */
void orc_set_conv_emulation(int mode);
void orc_dt(const float *vals, float ax, float bx, float ay, float by, const int *dims, float *M, int *Ix, int *Iy);
void orc_add_part(float *score, const float *M, const int *rootsize, const int *partsize, int ax, int ay);
void orc_rootbox(int x, int y, float scale, int padx, int pady, const int *rsize, float *Out);
int orc_partbox(int x, int y, int ax, int ay, float scale, int padx, int pady, const int *psize,
                const int *lx, const int *ly, const int *ssize, float *Out);
void orc_calc_a_score(float *ac_score, const float *score, const int *ssize, const int *rsize,
                      int im_h, int im_w, int padx, int pady, float scale);
void orc_normalize_a_score(float *A, int n, float thresh);
orc_scores *orc_compute_scores(const orc_model *m, const orc_pyramid *P, int nthreads);
/* Score map of (level, component) in double precision from the same FP32
 * features: convolutions, distance transforms and the part sum all in double.
 * out holds r0*r1 doubles (dims = {r0, r1}); returns -1 for a skipped level.
 * mag (may be null) receives max sum|a||b| of the root plus that of each part:
 * an operand rounding of relative size u moves no score by more than u * mag,
 * since the distance transform's minimum moves no more than its input. */
int orc_score_f64(const orc_model *m, const orc_pyramid *P, int level, int c, double *out, int *dims, double *mag);
void orc_free_scores(orc_scores *S);
float *orc_boxes_from_scores(const orc_model *m, const orc_pyramid *P, const orc_scores *S,
                             float thresh, float *a_score, int *Dnum, int *probe_oob);
void orc_quicksort(float *ary, int *Order, int first_index, int last_index);
int orc_nms_keep(const float *boxes, int NUM, int GL, float overlap, int *keep, int *order_out);
void orc_get_new_rects(const orc_model *m, const float *boxes, int NUM, int img_w, int img_h,
                       int *point, int *or_point, int *type, float *scale, float *score);
int orc_car_detection(orc_model *m, const uint8_t *bgr, int height, int width, int width_step,
                      float thresh, float overlap, float *a_score, int nthreads, orc_detection *out);
void orc_free_detection(orc_detection *d);
void orc_free(void *p);

#ifdef __cplusplus
}
#endif
#endif
