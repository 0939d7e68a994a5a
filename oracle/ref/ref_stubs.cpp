/*
 * Link stubs for building the reference's CPU translation units
 * (resize.cc, dt.cpp, nms.cpp, get_boxes.cpp, featurepyramid.cpp,
 * load_model.cpp, tracking.cpp) into a shared library on a machine without
 * the reference's GPU runtime or OpenCV.  TEST INFRASTRUCTURE ONLY.
 *
 * cuMemHostAlloc / cuMemFreeHost are the only driver calls reached on the CPU
 * path (get_boxes.cpp:75-114 padarray); they map to calloc/free.  Every other
 * driver entry point aborts, so a CPU-path test that strays onto the GPU path
 * fails loudly instead of silently.
 */
#include <stdio.h>
#include <stdlib.h>
#include <sys/time.h>
#include <cuda.h>
#include "cv.h"
#include "legacy.hpp"
#include "switch_float.h"

static void die(const char *what) { fprintf(stderr, "reference GPU path reached on the CPU build: %s\n", what); abort(); }

extern "C" {
CUresult cuMemHostAlloc(void **pp, size_t n, unsigned int) { *pp = calloc(1, n ? n : 1); return *pp ? CUDA_SUCCESS : CUDA_ERROR_OUT_OF_MEMORY; }
CUresult cuMemFreeHost(void *p) { free(p); return CUDA_SUCCESS; }
CUresult cuCtxSetCurrent(CUcontext) { die("cuCtxSetCurrent"); return CUDA_SUCCESS; }
CUresult cuCtxSynchronize(void) { die("cuCtxSynchronize"); return CUDA_SUCCESS; }
CUresult cuDeviceGetAttribute(int *, CUdevice_attribute, CUdevice) { die("cuDeviceGetAttribute"); return CUDA_SUCCESS; }
CUresult cuEventCreate(CUevent *, unsigned int) { die("cuEventCreate"); return CUDA_SUCCESS; }
CUresult cuEventDestroy(CUevent) { die("cuEventDestroy"); return CUDA_SUCCESS; }
CUresult cuEventElapsedTime(float *, CUevent, CUevent) { die("cuEventElapsedTime"); return CUDA_SUCCESS; }
CUresult cuEventRecord(CUevent, CUstream) { die("cuEventRecord"); return CUDA_SUCCESS; }
CUresult cuEventSynchronize(CUevent) { die("cuEventSynchronize"); return CUDA_SUCCESS; }
CUresult cuLaunchKernel(CUfunction, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, CUstream, void **, void **) { die("cuLaunchKernel"); return CUDA_SUCCESS; }
CUresult cuMemAlloc(CUdeviceptr *, size_t) { die("cuMemAlloc"); return CUDA_SUCCESS; }
CUresult cuMemFree(CUdeviceptr) { die("cuMemFree"); return CUDA_SUCCESS; }
CUresult cuMemcpyDtoH(void *, CUdeviceptr, size_t) { die("cuMemcpyDtoH"); return CUDA_SUCCESS; }
CUresult cuMemcpyHtoD(CUdeviceptr, const void *, size_t) { die("cuMemcpyHtoD"); return CUDA_SUCCESS; }
CUresult cuModuleGetTexRef(CUtexref *, CUmodule, const char *) { die("cuModuleGetTexRef"); return CUDA_SUCCESS; }
CUresult cuStreamCreate(CUstream *, unsigned int) { die("cuStreamCreate"); return CUDA_SUCCESS; }
CUresult cuStreamDestroy(CUstream) { die("cuStreamDestroy"); return CUDA_SUCCESS; }
CUresult cuStreamSynchronize(CUstream) { die("cuStreamSynchronize"); return CUDA_SUCCESS; }
CUresult cuTexRefSetAddress(size_t *, CUtexref, CUdeviceptr, size_t) { die("cuTexRefSetAddress"); return CUDA_SUCCESS; }
CUresult cuTexRefSetFlags(CUtexref, unsigned int) { die("cuTexRefSetFlags"); return CUDA_SUCCESS; }
CUresult cuTexRefSetFormat(CUtexref, CUarray_format, int) { die("cuTexRefSetFormat"); return CUDA_SUCCESS; }
char *conv(unsigned int) { return (char *)"stub"; }
FLOAT ***fconvsMT_GPU(CUdeviceptr, int, FLOAT **, int *, int, int, int *, int **, int **, int, int, int *, int, int, int, int, int) { die("fconvsMT_GPU"); return 0; }
FLOAT ****dt_GPU(int ****, int ****, int ***, int **, int, int *, int, int, int, int *, int, int, int, int, FLOAT *, int, int *, int *) { die("dt_GPU"); return 0; }
}

/* C++-linkage helpers of the GPU pyramid (resize_GPU.cc), never reached on the CPU path */
FLOAT *Ipl_to_FLOAT_forGPU(IplImage *) { die("Ipl_to_FLOAT_forGPU"); return 0; }
void *calc_resized_image_size(int *, int *, int, FLOAT, int, FLOAT *) { die("calc_resized_image_size"); return 0; }
void create_resized_image_texref(void) { die("create_resized_image_texref"); }
void cleanup_about_resize(void) { die("cleanup_about_resize"); }
FLOAT *resize_byGPU(FLOAT *, int *, int *, int, int, CUstream *) { die("resize_byGPU"); return 0; }

/* globals the reference's GPU runtime (GPU_init.cpp, fconvsMT.cpp, main.cpp) would define */
CUdevice *dev; CUcontext *ctx; CUmodule *module; int device_num;
CUfunction *func_calc_hist, *func_calc_norm, *func_calc_feat, *func_calc_a_score;
int *NR_MAXTHREADS_X, *NR_MAXTHREADS_Y;
CUdeviceptr *part_C_dev, *part_error_array_dev;
size_t size_A_SCORE;
struct timeval tv_memcpy_start, tv_memcpy_end, tv_kernel_start, tv_kernel_end;
float time_memcpy, time_kernel;

/* OpenCV image and tracker calls of tracking.cpp's tracker; get_new_rects and
 * create_result (the only tracking.cpp functions the oracle calls) reach none */
CvSize cvSize(int, int) { die("cvSize"); return CvSize{}; }
CvRect cvRect(int, int, int, int) { die("cvRect"); return CvRect{}; }
CvPoint cvPoint(int, int) { die("cvPoint"); return CvPoint{}; }
CvScalar cvScalar(double, double, double, double) { die("cvScalar"); return CvScalar{}; }
IplImage *cvCreateImage(CvSize, int, int) { die("cvCreateImage"); return 0; }
IplImage *cvCloneImage(const IplImage *) { die("cvCloneImage"); return 0; }
void cvReleaseImage(IplImage **) { die("cvReleaseImage"); }
void cvSetImageROI(IplImage *, CvRect) { die("cvSetImageROI"); }
void cvResetImageROI(IplImage *) { die("cvResetImageROI"); }
void cvCopy(const void *, void *, const void *) { die("cvCopy"); }
void cvCvtColor(const void *, void *, int) { die("cvCvtColor"); }
void cvResize(const void *, void *, int) { die("cvResize"); }
CvMat *cvCreateMat(int, int, int) { die("cvCreateMat"); return 0; }
void cvReleaseMat(CvMat **) { die("cvReleaseMat"); }
void cvmSet(CvMat *, int, int, double) { die("cvmSet"); }
double cvmGet(const CvMat *, int, int) { die("cvmGet"); return 0; }
void cvMatchTemplate(const void *, const void *, void *, int) { die("cvMatchTemplate"); }
CvConDensation *cvCreateConDensation(int, int, int) { die("cvCreateConDensation"); return 0; }
void cvReleaseConDensation(CvConDensation **) { die("cvReleaseConDensation"); }
void cvConDensInitSampleSet(CvConDensation *, CvMat *, CvMat *) { die("cvConDensInitSampleSet"); }
void cvConDensUpdateByTime(CvConDensation *) { die("cvConDensUpdateByTime"); }
void cvRandInit(CvRandState *, double, double, int, int) { die("cvRandInit"); }
