/* Stand-in for OpenCV 2.4's legacy module: the condensation (particle
 * filter) tracker's state as tracking.cpp reads it.  Only the tracker
 * (tracking.cpp:321-850) touches these, and the oracle never calls it; its
 * functions link to aborting stubs (ref_stubs.cpp). */
#pragma once
#include "cv.h"
typedef struct CvRandState { double param[4]; int disttype; } CvRandState;
struct CvConDensation {
    int MP, DP;
    float *DynamMatr;
    float *State;
    int SamplesNum;
    float **flSamples;
    float **flNewSamples;
    float *flConfidence;
    float *flCumulative;
    float *Temp;
    float *RandomSample;
    CvRandState *RandS;
};
CvConDensation *cvCreateConDensation(int dynam_params, int measure_params, int sample_count);
void cvReleaseConDensation(CvConDensation **condens);
void cvConDensInitSampleSet(CvConDensation *condens, CvMat *lower_bound, CvMat *upper_bound);
void cvConDensUpdateByTime(CvConDensation *condens);
void cvRandInit(CvRandState *state, double param1, double param2, int seed, int disttype = 0);
