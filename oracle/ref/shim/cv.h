/* Minimal stand-in for OpenCV 2.4's cv.h: the reference's hot path only uses
 * IplImage as a pixel container (height, width, nChannels, widthStep,
 * imageData) and names CvConDensation in a struct it never touches. */
#pragma once
#include <math.h>
typedef struct _IplImage {
    int nChannels;
    int depth;
    int width;
    int height;
    int widthStep;
    char *imageData;
} IplImage;
typedef struct CvConDensation CvConDensation;
