/* Forced-include prologue for building src/prototypes/detrend.cu with CUDA 13, written for this
 * oracle build: the prototype's host code calls cudaThreadSetCacheConfig, which later CUDA
 * releases removed in favour of cudaDeviceSetCacheConfig (same arguments).  The kernel is not
 * affected. */
#pragma once
#include <cuda_runtime.h>
#define cudaThreadSetCacheConfig cudaDeviceSetCacheConfig
