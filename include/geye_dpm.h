/*
 * geye_dpm.h -- C ABI of libgeye_dpm.so, the GB300 (sm_103a) implementation
 * of CPFL/geye's DPM detection path:
 *   image resize pyramid -> 31-channel HOG pyramid -> root/part filter
 *   convolution -> generalized distance transform with argmax -> score
 *   assembly and box records -> greedy NMS -> box regression.
 *
 * Every entry point returns a geye_status (0 = success).  Plain pointers and
 * sizes only.  Array layouts are the reference's: a map of d0 rows (y) by d1
 * columns (x) is column-major (element (x, y) at x*d0 + y); a feature level
 * is [31][d1][d0]; a box record is GL = (numpart+1)*4+3 floats
 * [root y1,x1,y2,x2, part boxes..., component, score, scale].
 *
 * Reference interfaces replaced (paths relative to the reference project):
 *   init_cuda / clean_cuda        CAR_TRACKING/for_use_GPU.h:128-130
 *   load_model / free_model       CAR_TRACKING/car_det_func.h:22-23
 *   car_detection                 CAR_TRACKING/car_det_func.h:30
 *   calc_f_pyramid                CAR_TRACKING/detect_func.h:27
 *   get_boxes                     CAR_TRACKING/detect_func.h:36
 *   nms                           CAR_TRACKING/detect_func.h:45
 *   get_new_rects                 CAR_TRACKING/detect_func.h:54 (tracking.cpp:90)
 *   dt                            CAR_TRACKING/get_boxes_func.h:34
 *   fconvsMT / fconvsMT_GPU       CAR_TRACKING/get_boxes_func.h:28, for_use_GPU.h:136-160
 *   resize                        CAR_TRACKING/resize.cc:135
 *   calc_feature                  CAR_TRACKING/featurepyramid.cpp:263
 */
#ifndef GEYE_DPM_H
#define GEYE_DPM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int geye_status;
#define GEYE_OK               0
#define GEYE_ERR_ARG          1   /* bad argument (null pointer, bad size)          */
#define GEYE_ERR_CUDA         2   /* a CUDA call failed; see geye_last_error()      */
#define GEYE_ERR_MODEL        3   /* model file missing or malformed                */
#define GEYE_ERR_NOMEM        4   /* device or host allocation failed               */
#define GEYE_ERR_UNSUPPORTED  5   /* model shape outside what the kernels cover     */
#define GEYE_ERR_INJECTED     6   /* fault injected by geye_debug_inject_fault      */
#define GEYE_ERR_TIMEOUT      7   /* a bounded device-side wait gave up             */
#define GEYE_BUSY             8   /* the submitted frame is still on the GPU        */

typedef struct geye_ctx geye_ctx;       /* one device + one stream + work buffers */
typedef struct geye_model geye_model;   /* a DPM model resident on the device     */

/* Convolution arithmetic. */
typedef enum {
    GEYE_CONV_FP32 = 0,   /* CUDA-core FP32 in the reference's summation order (bit-exact) */
    GEYE_CONV_BF16 = 1,   /* tcgen05 implicit GEMM, BF16 operands, FP32 accumulation        */
    GEYE_CONV_FP8 = 2,    /* tcgen05 implicit GEMM, FP8-e4m3 operands (features x 256, each
                             filter x a power of two under 448), FP32 accumulation, scales
                             undone exactly in the epilogue                                  */
} geye_conv_mode;

/* Detection result; mirrors RESULT (CAR_TRACKING/MODEL_info.h:158-166)
 * without the per-box IplImage crops. */
typedef struct {
    int num;
    int *point;      /* num x 4: x1, y1, x2, y2 clamped to the image            */
    int *or_point;   /* num x 4: point / model ratio                            */
    int *type;       /* component index                                         */
    float *scale;
    float *score;
} geye_result;

/* ---- runtime: replaces init_cuda / clean_cuda ------------------------- */
/* stream may be NULL (the context creates its own non-blocking stream). */
geye_status geye_ctx_create(int device, void *cuda_stream, geye_ctx **out);
geye_status geye_ctx_destroy(geye_ctx *ctx);
geye_status geye_ctx_set_conv_mode(geye_ctx *ctx, geye_conv_mode mode);
geye_status geye_ctx_synchronize(geye_ctx *ctx);
const char *geye_last_error(void);
const char *geye_version(void);

/* ---- models: replaces load_model / free_model ------------------------- */
geye_status geye_model_load_csv(geye_ctx *ctx, const char *comp_csv, const char *root_csv,
                                const char *part_csv, float ratio, geye_model **out);
geye_status geye_model_free(geye_model *model);
/* numcomponent, sbin, interval, numpart[0], GL, NoR, NoP, latched max_scale (-1 if none) */
geye_status geye_model_info(const geye_model *model, int info[8]);
/* Clears the ini_scales latch so the next frame fixes max_scale again. */
geye_status geye_model_reset_scales(geye_model *model);

/* ---- whole path: replaces car_detection -------------------------------- */
/* bgr: height rows of width*3 bytes (B,G,R) at width_step bytes apart, host memory.
 * a_score: height*width floats, column-major, host, updated in place (the caller
 * fills it with -100 first, as ini_ac_score does); may be NULL.
 * out: filled with callee-allocated arrays; release with geye_result_free. */
geye_status geye_car_detection(geye_ctx *ctx, geye_model *model, const uint8_t *bgr, int width, int height,
                               int width_step, float thresh, float overlap, float *a_score, geye_result *out);
geye_status geye_result_free(geye_result *res);

/* Several models on one frame; the feature pyramid is computed once and shared.
 * out[m] receives model m's result. */
geye_status geye_detect_multi(geye_ctx *ctx, geye_model *const *models, int n_models, const uint8_t *bgr,
                              int width, int height, int width_step, float thresh, float overlap,
                              float *const *a_scores, geye_result *out);

/* ---- stage entry points (reference layouts, host buffers) --------------- */
/* calc_f_pyramid: *n_levels gets LEN; *features (callee-allocated, geye_free)
 * holds the levels back to back, level l at offset sum_{k<l} 31*fs0*fs1;
 * ftsize (2*LEN ints) and scales (LEN floats) are callee-allocated too. */
geye_status geye_calc_f_pyramid(geye_ctx *ctx, geye_model *model, const uint8_t *bgr, int width, int height,
                                int width_step, int *n_levels, float **features, int **ftsize, float **scales);

/* get_boxes: features as produced by geye_calc_f_pyramid.  *boxes is [D][GL]
 * (callee-allocated, geye_free), *dnum = D.  a_score as in geye_car_detection. */
geye_status geye_get_boxes(geye_ctx *ctx, geye_model *model, const float *features, const float *scales,
                           const int *ftsize, int n_levels, int img_width, int img_height, float thresh,
                           float *a_score, float **boxes, int *dnum);

/* nms: boxes [num][GL] -> *out [kept][GL] in input order (callee-allocated); *num updated. */
geye_status geye_nms(geye_ctx *ctx, const float *boxes, float overlap, int *num, int numpart0, float **out);

/* get_new_rects: kept boxes -> result (callee-allocated arrays, geye_result_free). */
geye_status geye_get_new_rects(geye_ctx *ctx, const geye_model *model, const float *boxes, int num,
                               int img_width, int img_height, geye_result *out);

/* dt: vals/M column-major dims[0] x dims[1]; M, Ix, Iy caller-allocated. */
geye_status geye_dt(geye_ctx *ctx, const float *vals, float ax, float bx, float ay, float by, const int *dims,
                    float *M, int *Ix, int *Iy);

/* fconvsMT for one feature level and n filters: feat [31][a1][a0] (a_dims = {a0, a1});
 * filters[i] [31][b1][b0] (b_dims 2*i, 2*i+1); out receives the n maps back to back,
 * each (a0-b0+1) x (a1-b1+1) column-major.  Uses the context's convolution mode. */
geye_status geye_fconv(geye_ctx *ctx, const float *feat, const int *a_dims, const float *const *filters,
                       const int *b_dims, int n_filters, float *out);

/* resize: src [c][w][h] with sdims = {h, w, c}; odims receives the output size;
 * dst must hold the output (size from the same rounding as the reference). */
geye_status geye_resize(geye_ctx *ctx, const float *src, const int *sdims, int *odims, float scale, float *dst);

/* calc_feature: src [3][w][h] (isize = {h, w, 3}) -> feat [31][fs1][fs0]; ftsize receives {fs0, fs1}. */
geye_status geye_calc_feature(geye_ctx *ctx, const float *src, const int *isize, int sbin, int *ftsize,
                              float *feat);

/* flip_feat (CAR_TRACKING/get_boxes.cpp:121-178): feat [size[2]][size[1]][size[0]]
 * (reference layout, size[2] = 31 channels) mirrored along dim 1, channel ii
 * taken from channel ORD[ii]-1 of the reference's table; *out is callee-allocated
 * (geye_free), as the reference allocates its result. */
geye_status geye_flip_feat(geye_ctx *ctx, const float *feat, const int *size, float **out);

/* Symmetric information of a loaded model (CAR_TRACKING/load_model.cpp:279-373,
 * 420-524): rootsym (NoR ints; the loader sets every one to 1), part_partner
 * (NoP ints, the part CSV's partner field) and part_sym (NoP ints, 1 where the
 * partner is 0).  Any pointer may be NULL. */
geye_status geye_model_sym(const geye_model *model, int *rootsym, int *part_partner, int *part_sym);

void geye_free(void *p);

/* ---- device-resident path (benchmarks, batching) ------------------------ */
/* Runs the whole path on a frame already in device memory (d_bgr, tightly packed
 * width*3 bytes per row), leaving boxes and the kept set on the device.  Results
 * can be read with geye_fetch_result.  Asynchronous on the context's stream:
 * nothing is copied between host and device. */
geye_status geye_detect_device(geye_ctx *ctx, geye_model *const *models, int n_models, const uint8_t *d_bgr,
                               int width, int height, float thresh, float overlap);
geye_status geye_fetch_result(geye_ctx *ctx, int model_index, geye_result *out, int *n_boxes_before_nms);

/* ---- allocation-free NMS --------------------------------------------------- */
/* No counterpart in the reference: an addition for callers that cannot call
 * cudaMalloc (their device memory belongs to another allocator, such as a
 * framework's caching pool or a fixed per-process budget, or they run a
 * real-time loop that cannot take cudaMalloc's latency and synchronisation).
 * Same computation as geye_nms (reference tie order and kept set) on
 * caller-owned DEVICE buffers: d_boxes [num][GL], d_out with room for
 * num*GL floats (kept records in input order), *d_kept (device int) = kept
 * count, or -1 on an internal error.  Asynchronous on cuda_stream (NULL = the
 * legacy default stream).  Allocates nothing: working memory is a fixed
 * __device__ array sized for GEYE_NMS_NOALLOC_MAX_BOXES boxes (~2.8 MB, held by
 * every GPU that loads the library until exit); num above that returns
 * GEYE_ERR_ARG.  All calls share that array and it keeps the last call's
 * contents, so calls that overlap on the GPU race.  The first call on each
 * device looks up the array's device address (cudaGetSymbolAddress); make that
 * first call before any stream capture.  The address is remembered per CUDA
 * context (its unique id), so after cudaDeviceReset, or in a caller's own
 * non-primary context, the first call there looks it up again.
 * On success *d_kept is the kept count (0 for num = 0). */
#define GEYE_NMS_NOALLOC_MAX_BOXES 65536
geye_status geye_nms_noalloc(const float *d_boxes, int num, int numpart0, float overlap, float *d_out,
                             int *d_kept, void *cuda_stream);

/* ---- asynchronous submission (no counterpart in the reference) ------------ */
/* The work of geye_detect_multi without waiting: the frame is copied (the
 * caller's buffer is free on return), staged through pinned memory, run on the
 * context's stream and its results copied back into pinned memory.  One frame
 * per context may be outstanding; geye_detect_query returns GEYE_OK when it is
 * done and GEYE_BUSY while it runs; geye_detect_collect waits for it and fills
 * out[0..n_models) (free each with geye_result_free).  Several contexts on one
 * device run their frames concurrently. */
geye_status geye_detect_submit(geye_ctx *ctx, geye_model *const *models, int n_models, const uint8_t *bgr, int width,
                               int height, int width_step, float thresh, float overlap);
geye_status geye_detect_query(geye_ctx *ctx);
geye_status geye_detect_collect(geye_ctx *ctx, geye_result *out);

/* ---- multi-stream server (no counterpart in the reference) --------------- */
/* Frames from many camera streams are admitted as they arrive into slots (one
 * context and stream each, created on demand while the device memory held by
 * slots stays within hbm_budget bytes and at most max_slots exist); frames of
 * different resolutions and streams overlap on the GPU.  Each stream's frames
 * are dispatched in submission order.  When track is nonzero every stream
 * keeps a device-resident particle-filter tracker fed with its detections.
 * The slots' streams overlap only as far as the device's hardware work
 * queues allow: a serving process should set CUDA_DEVICE_MAX_CONNECTIONS=32
 * in its environment before its first CUDA call (with CUDA's default of 8,
 * 16 slots at 640x480 run 2954 instead of 3384 frames/s end to end). */
typedef struct geye_server geye_server;   /* the models must outlive the server */
typedef struct {
    long long ticket;        /* from geye_server_submit                         */
    int stream;              /* camera stream id                                */
    int n_tracks;            /* live tracks of the stream after this frame      */
    long long queued_ns;     /* submit -> dispatch to a slot                     */
    long long latency_ns;    /* submit -> results on the host                    */
    int dropped;             /* 1: never run (admission limit, or its model's
                                context was destroyed); its results are empty  */
    int reserved;
} geye_served;
geye_status geye_server_create(int device, geye_model *const *models, int n_models, geye_conv_mode mode,
                               size_t hbm_budget, int max_slots, float thresh, float overlap, int track,
                               geye_server **out);
geye_status geye_server_destroy(geye_server *s);
/* Copies the frame and queues it; dispatches whatever fits.  *ticket identifies it. */
geye_status geye_server_submit(geye_server *s, int stream, const uint8_t *bgr, int width, int height,
                               int width_step, long long *ticket);
/* Completes finished frames and dispatches queued ones without blocking; up to
 * max finished frames are returned (info[i], and n_models results per frame in
 * results[i*n_models ...] when results is not NULL).  *n = how many. */
geye_status geye_server_poll(geye_server *s, int max, geye_served *info, geye_result *results, int *n);
/* Blocks until every submitted frame has finished (collect them with poll). */
geye_status geye_server_drain(geye_server *s);
/* Latency-aware admission, for cameras that together offer more frames than the
 * GPU serves: a stream holds at most max_queued_per_stream frames waiting for a
 * slot (a newer frame drops the stream's oldest waiting one), and a frame that
 * has waited more than max_wait_ns for a slot is dropped instead of run.  0 turns
 * a limit off (the default: every frame is served).  Dropped frames come back
 * from poll with dropped = 1 and empty results.  Before any launch, every
 * submit and poll also drops all waiting frames and returns GEYE_ERR_ARG when a
 * model's loading context has been destroyed; models must outlive the server. */
geye_status geye_server_set_admission(geye_server *s, int max_queued_per_stream, long long max_wait_ns);
/* out[0..7]: slots, busy slots, queued frames, finished not yet polled,
 * device bytes held by slots, frames completed, streams with trackers,
 * frames dropped. */
geye_status geye_server_stats(geye_server *s, long long out[8]);
/* Copies stream `stream`'s live tracks (up to max) as x1, y1, x2, y2 floats into
 * boxes[4*i]; *n = count. */
geye_status geye_server_tracks(geye_server *s, int stream, int max, float *boxes, int *n);

/* ---- batches -------------------------------------------------------------- */
/* Several frames of any sizes as one CUDA graph: each frame gets a lane (its own
 * context, stream and plan per size, created on first use) and the lanes run as
 * parallel branches of one graph between a fork and a join, the graph kept per
 * combination of lane sizes, thresh and overlap.  geye_batch_run copies the
 * frames into the lanes' pinned buffers, launches the graph, waits, and fills
 * results[i * n_models + m] (free each with geye_result_free); every result is
 * the one geye_detect_multi gives for that frame alone. */
typedef struct geye_batch geye_batch;     /* the models must outlive the batch */
geye_status geye_batch_create(int device, geye_model *const *models, int n_models, geye_conv_mode mode,
                              int max_frames, geye_batch **out);
geye_status geye_batch_destroy(geye_batch *b);
geye_status geye_batch_run(geye_batch *b, int n_frames, const uint8_t *const *bgr, const int *widths,
                           const int *heights, const int *width_steps, float thresh, float overlap,
                           geye_result *results);
/* out = {lanes, graphs built, kernels in the last graph, 0}; last_ms = device
 * time of the last graph launch (CUDA events on the batch stream). */
geye_status geye_batch_stats(geye_batch *b, int out[4], float *last_ms);

/* ---- measurement ---------------------------------------------------------- */
/* When enabled, the context records CUDA events around each stage on its stream.
 * ms receives per-stage milliseconds of the last run, in this order:
 * ingest+resize, hog, conv, dt, score, nms, total; bytes receives the
 * algorithmic bytes of each stage and flops the conv FLOPs. */
#define GEYE_N_STAGES 7
geye_status geye_ctx_enable_timing(geye_ctx *ctx, int enable);
geye_status geye_ctx_stage_times(geye_ctx *ctx, float ms[GEYE_N_STAGES], double bytes[GEYE_N_STAGES],
                                 double *conv_flops, int *kernel_launches);

/* Diagnostic counters of the last whole-path run (per model m, 8 values each:
 * [8m+1] sort segments left to the one-block quicksort tier, [8m+2] greedy
 * batches, [8m+3] picks, [8m+4] whether the finish kernel ran batches itself,
 * [8m+5] whether the model's kept set was resolved in the quicksort's order). */
geye_status geye_ctx_debug_counters(geye_ctx *ctx, long long *out, int n);

/* Order in which the whole-path NMS resolves the detections (the kept set is
 * nms.cpp's in both):
 *   GEYE_NMS_ORDER_KEY (default): score order, equal scores by input index;
 *     a model whose kept set could depend on the order among equal scores is
 *     resolved again in the order of the reference's quicksort (nms.cpp:70-84);
 *   GEYE_NMS_ORDER_QUICKSORT: the quicksort's order for every model. */
#define GEYE_NMS_ORDER_KEY 0
#define GEYE_NMS_ORDER_QUICKSORT 1
geye_status geye_ctx_set_nms_order(geye_ctx *ctx, int order);

/* Score map (root + offset - parts, before the threshold) of pyramid level
 * `level` and component `comp` of model m, from the last whole-path run on this
 * context, column-major r0 x r1 as get_boxes.cpp:1022-1041 builds it.
 * dims receives {r0, r1}; out (cap floats) may be null to ask the size only.
 * GEYE_ERR_ARG when the last run has no such map (skipped level, other model). */
geye_status geye_score_map(geye_ctx *ctx, const geye_model *m, int level, int comp, float *out, int cap,
                           int dims[2]);

/* Tile shape the tensor-core convolution's autotuner chose for model m in the
 * last run's plan: shape = {largest tile run per CTA (128 positions a tile; 0:
 * the persistent form, one CTA per SM with its filter bank resident),
 * shared-memory budget per CTA in KB, CTAs per launch}; ms = its measured time
 * per launch.  GEYE_ERR_ARG in FP32 mode or before a run. */
geye_status geye_conv_tuning(geye_ctx *ctx, const geye_model *m, int shape[3], float *ms);

/* DT tile size of model m in the last run's plan: elems = outputs per DT block,
 * chosen after the plan's first completed frame by timing 1024, 2048 and 4096
 * on that frame's part maps; ms = the timed DT launch of each (0 before the
 * tuning has run).  GEYE_ERR_ARG before a run or for a model not in it. */
geye_status geye_dt_tuning(geye_ctx *ctx, const geye_model *m, int *elems, float ms[3]);

/* ---- fault injection (host side only) ------------------------------------ */
/* The n-th subsequent call of the named operation ("alloc", "h2d", "launch")
 * fails with GEYE_ERR_INJECTED; n = 0 clears.  No device fault is ever raised. */
geye_status geye_debug_inject_fault(geye_ctx *ctx, const char *op, int nth);

#ifdef __cplusplus
}
#endif
#endif
