/* Minimal stand-in for OpenCV 2.4's cv.h: the reference's hot path only uses
 * IplImage as a pixel container (height, width, nChannels, widthStep,
 * imageData) and names CvConDensation in a struct it never touches.  The
 * tracker around get_new_rects (tracking.cpp) also names the small value
 * types and image functions declared below; nothing the oracle calls reaches
 * them, and their definitions are aborting stubs (ref_stubs.cpp). */
#pragma once
#include <math.h>
#include <string.h>
typedef struct _IplImage {
    int nChannels;
    int depth;
    int width;
    int height;
    int widthStep;
    char *imageData;
} IplImage;
typedef struct CvConDensation CvConDensation;

typedef struct { int width, height; } CvSize;
typedef struct { int x, y, width, height; } CvRect;
typedef struct { int x, y; } CvPoint;
typedef struct { double val[4]; } CvScalar;
typedef struct CvMat {
    int type;
    union { int rows; int height; };
    union { int cols; int width; };
    float *data;
} CvMat;
#define CV_32FC1 5
#define CV_BGR2GRAY 6
#define CV_TM_CCORR_NORMED 3
#define CV_WINDOW_AUTOSIZE 1
#ifdef __cplusplus
CvSize cvSize(int width, int height);
CvRect cvRect(int x, int y, int width, int height);
CvPoint cvPoint(int x, int y);
CvScalar cvScalar(double v0, double v1 = 0, double v2 = 0, double v3 = 0);
IplImage *cvCreateImage(CvSize size, int depth, int channels);
IplImage *cvCloneImage(const IplImage *image);
void cvReleaseImage(IplImage **image);
void cvSetImageROI(IplImage *image, CvRect rect);
void cvResetImageROI(IplImage *image);
void cvCopy(const void *src, void *dst, const void *mask = 0);
void cvCvtColor(const void *src, void *dst, int code);
void cvResize(const void *src, void *dst, int interpolation = 1);
CvMat *cvCreateMat(int rows, int cols, int type);
void cvReleaseMat(CvMat **mat);
void cvmSet(CvMat *mat, int row, int col, double value);
double cvmGet(const CvMat *mat, int row, int col);
void cvSetReal2D(void *arr, int idx0, int idx1, double value);
void cvMatchTemplate(const void *image, const void *templ, void *result, int method);
void cvCircle(void *img, CvPoint center, int radius, CvScalar color, int thickness = 1, int line_type = 8, int shift = 0);
void cvRectangle(void *img, CvPoint pt1, CvPoint pt2, CvScalar color, int thickness = 1, int line_type = 8, int shift = 0);
int cvNamedWindow(const char *name, int flags = 1);
void cvShowImage(const char *name, const void *image);
int cvWaitKey(int delay = 0);
void cvDestroyWindow(const char *name);
#endif
