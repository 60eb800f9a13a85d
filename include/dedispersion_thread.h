/*
 * dedispersion_thread.h -- the reference's internal C ABI between its manager and its per-GPU
 * worker threads (src/mdsm/dedispersion_wrapper.cu:4-13, types of
 * src/mdsm/dedispersion_thread.h:9-57), implemented by this library.  A manager written
 * against the reference (src/mdsm/dedispersion_manager.cpp:269-382, 416-501) spawns
 * call_dedisperse once per device with pthread_create and drives it through the same two
 * barriers and read-write lock; the worker copies each block in, dedisperses it with this
 * library's kernels and copies the series out into the THREAD_PARAMS output buffer.  The three
 * structs keep the reference's members, order and types: they are an ABI the manager compiles
 * against.
 */
#ifndef MDSM_GB300_DEDISPERSION_THREAD_H_
#define MDSM_GB300_DEDISPERSION_THREAD_H_

#include <pthread.h>
#include <stddef.h>
#include <time.h>

#include "survey.h"

/* src/mdsm/dedispersion_thread.h:9-20 */
typedef struct {
    int multiprocessor_count;
    int constant_memory;
    int shared_memory;
    int register_count;
    int thread_count;
    int clock_rate;  /* kHz */
    int device_id;
} DEVICE_INFO;

/* src/mdsm/dedispersion_thread.h:22-29 */
typedef struct {
    int num_devices;
    unsigned long int minTotalGlobalMem;  /* KiB, the smallest selected device's memory */
    DEVICE_INFO *devices;
} DEVICES;

/* src/mdsm/dedispersion_thread.h:31-57 */
typedef struct {
    int iterations, maxiters;
    int maxshift, binsize;
    float *dmshifts;
    size_t inputsize, outputsize, dm_output, dedispersed_size;
    float *output;
    float *input;
    int device_id;
    unsigned short thread_num, num_threads, stop;
    pthread_rwlock_t *rw_lock;
    pthread_barrier_t *input_barrier;
    pthread_barrier_t *output_barrier;
    time_t start;
    SURVEY *survey;
} THREAD_PARAMS;

#ifdef __cplusplus
extern "C" {
#endif

/* src/mdsm/dedispersion_wrapper.cu:5,11-13 (initialise_devices, dedispersion_thread.cu:4-62):
 * the devices with more than 2.5 GiB of memory, restricted to survey->gpu_ids when it is set;
 * minTotalGlobalMem starts at 16 GiB (in KiB) and takes the smallest selected device's
 * memory.  Returns a malloc'd DEVICES (and devices array) the caller frees, or NULL with
 * mdsm_last_error() set (the reference prints the message and exits). */
DEVICES *call_initialise_devices(SURVEY *survey);

/* src/mdsm/dedispersion_wrapper.cu:4,7-9 (dedisperse, dedispersion_thread.cu:246-401): the
 * worker thread of one device, started by pthread_create with a THREAD_PARAMS.  Per loop:
 * from the first data block on (loop counter >= iterations) copy the block in (the whole
 * [nchans][nsamp + maxshift] float buffer once; later the previous block's last maxshift
 * samples of each channel, kept on the device, then the caller's new samples), wait at the
 * input barrier, dedisperse (brute force with the reference's L1 or opt shift arithmetic, or
 * the subband passes), wait at the output barrier, copy the thread's series into output
 * (dedispersed_size floats: brute force [tdms/num_threads][nsamp] from
 * lowdm + dmstep*tdms/num_threads*thread_num; subband, per pass and sub-DM call, calldms rows
 * of nsamp/binsize samples), then take the read lock, follow survey->nsamp and stop as the
 * reference does (after stop is set, iterations - 1 more loops, then maxiters - iterations
 * barrier pairs).  Returns thread_params.  A failing block is reported on stderr and its
 * output zeroed; the worker keeps to the barrier protocol so the other threads never wait
 * on it. */
void *call_dedisperse(void *thread_params);

#ifdef __cplusplus
}
#endif
#endif
