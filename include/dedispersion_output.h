/*
 * dedispersion_output.h -- the reference's output thread interface (src/mdsm/dedispersion_output.h:8-30),
 * implemented by this library.  A manager written against the reference
 * (src/mdsm/dedispersion_manager.cpp:331-344) starts process_output with pthread_create next to
 * its call_dedisperse workers and drives it through the same two barriers and read-write lock;
 * each block's series, as the workers left them in the shared output buffer, is searched on
 * the GPU with the reference's detectors (process_brute, with its own or the caller's noise
 * statistics; process_subband) and the candidate lines are written to the reference's files.
 * OUTPUT_PARAMS keeps the reference's members, order and types: it is an ABI the manager
 * compiles against.
 */
#ifndef MDSM_GB300_DEDISPERSION_OUTPUT_H_
#define MDSM_GB300_DEDISPERSION_OUTPUT_H_

#include <pthread.h>
#include <stddef.h>
#include <time.h>

#include "survey.h"

/* src/mdsm/dedispersion_output.h:8-28 */
typedef struct {
    int nthreads, iterations, maxiters;
    float *output_buffer;
    size_t dedispersed_size;  /* floats of one worker thread's series */
    unsigned short stop;
    pthread_rwlock_t *rw_lock;
    pthread_barrier_t *input_barrier;
    pthread_barrier_t *output_barrier;
    time_t start;
    SURVEY *survey;
} OUTPUT_PARAMS;

#ifdef __cplusplus
extern "C" {
#endif

/* src/mdsm/dedispersion_output.cpp:216-356: the output thread.  Every cycle it waits at the
 * input barrier; from cycle `iterations` on it searches the output buffer (the block handed in
 * two cycles earlier, with that block's nsamp, timestamp, blockRate and noise statistics) and
 * appends the candidate lines to the current file (survey->basedir/fileprefix.dat in single
 * file mode, else a file per secs_per_file named by the block's time); it then waits at the
 * output barrier, takes the read lock to advance those values, and leaves once `stop` is set,
 * after the remaining maxiters - iterations barrier pairs.  Device failures are reported on
 * stderr ("mdsm output: ...") and the thread keeps to the barrier protocol.  Returns its
 * argument. */
void *process_output(void *output_params);

#ifdef __cplusplus
}
#endif

#endif
