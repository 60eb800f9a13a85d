/* Forced-include prologue for building src/prototypes/rfi_clipper.cu with CUDA 13, written for
 * this oracle build.  The prototype declares its kernel `__global__ __device__`, a combination
 * current nvcc rejects.  The headers the file includes are taken in first, with the runtime's
 * own qualifier macros; `__device__` is then made empty for the rest of the translation unit,
 * so the declaration reads `__global__ void rfi_clipping(...)`.  No other `__device__` appears
 * in that file. */
#pragma once
#include <cuda_runtime.h>
#include <cufft.h>
#include <sys/time.h>
#include "cutil.h"
#undef __device__
#define __device__
