/*
 * timeMeasurement.h -- timer types of the CUNFFT plan ABI.
 *
 * NFFTTimeSpec is a member of cunfft_plan (reference src/timeMeasurement.h:22-36),
 * so its field order is part of the ABI.  The helpers below give drivers the
 * same wall-clock and CUDA-event timers the reference drivers use
 * (getTimeCPU / getTimeGPU / elapsed*Time); all times are in seconds.
 * This library fills NFFTTimeSpec (time_ROC, time_FFT, time_CONV, time_COPY_IN,
 * time_COPY_OUT) on every call from events on the plan's stream.
 */
#ifndef TIMEMEASUREMENT_H_
#define TIMEMEASUREMENT_H_

#include <cuda_runtime_api.h>
#include <time.h>

typedef struct timespec Timer;
typedef cudaEvent_t GPUTimer;
typedef Timer CPUTimer;

typedef struct {
  double runTime;       /**< whole transformation */
  double time_ROC;      /**< roll-off correction step */
  double time_CONV;     /**< gridding (convolution) step, node binning included */
  double time_FFT;      /**< FFT step */
  double time_COPY_IN;  /**< host -> device copy */
  double time_COPY_OUT; /**< device -> host copy */
  double time_else;     /**< user-defined */
} NFFTTimeSpec;

static __inline__ void resetNFFTTimeSpec(NFFTTimeSpec *t)
{
  t->runTime = 0.0; t->time_ROC = 0.0; t->time_CONV = 0.0; t->time_FFT = 0.0;
  t->time_COPY_IN = 0.0; t->time_COPY_OUT = 0.0; t->time_else = 0.0;
}

static __inline__ CPUTimer getTimeCPU(void)
{
  CPUTimer t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return t;
}

static __inline__ double elapsedCPUTime(CPUTimer start, CPUTimer stop)
{
  return (double)(stop.tv_sec - start.tv_sec) + (double)(stop.tv_nsec - start.tv_nsec) * 1e-9;
}

/** Record an event on the legacy default stream. */
static __inline__ GPUTimer getTimeGPU(void)
{
  GPUTimer e;
  cudaEventCreate(&e);
  cudaEventRecord(e, 0);
  return e;
}

/** Seconds between two events; destroys both. */
static __inline__ double elapsedGPUTime(GPUTimer start, GPUTimer stop)
{
  float ms = 0.0f;
  cudaEventSynchronize(stop);
  cudaEventElapsedTime(&ms, start, stop);
  cudaEventDestroy(start);
  cudaEventDestroy(stop);
  return (double)ms / 1000.0;
}

#endif /* TIMEMEASUREMENT_H_ */
