/* Stand-in for the retired CUDA SDK header that the MDSM kernels include; written for this
 * oracle build.  Only the error-check macro is needed. */
#pragma once
#include <cuda_runtime.h>
#include <stdio.h>
#define cutilSafeCall(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) fprintf(stderr, "%s\n", cudaGetErrorString(e_)); } while (0)
