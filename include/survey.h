/*
 * survey.h -- the SURVEY observation-parameter struct, with the same members, order and types
 * as the reference's src/mdsm/survey.h:6-57, so callers written against the reference compile
 * and lay out memory identically.  (The layout is an ABI, so it is kept alike on purpose.)
 */
#ifndef MDSM_GB300_SURVEY_H_
#define MDSM_GB300_SURVEY_H_

#include <stdio.h>

#ifndef __cplusplus
#include <stdbool.h>
#endif

/* src/mdsm/survey.h:6-11 -- one subband pass of a DM plan. */
typedef struct {
    float lowdm, highdm, dmstep, sub_dmstep;
    int binsize, ndms, ncalls, calldms, mean, stddev;
} SUBBAND_PASSES;

/* src/mdsm/survey.h:13-57 */
typedef struct {
    /* data parameters */
    unsigned int nsamp, nchans, tdms, maxshift, nbits;
    float tsamp, foff, fch1;

    /* brute force vs subband */
    bool useBruteForce;
    bool useL1Cache;

    /* brute-force parameters */
    float lowdm, dmstep;

    /* subband parameters */
    SUBBAND_PASSES *pass_parameters;
    unsigned num_passes, nsubs;

    /* timing */
    double timestamp;
    double blockRate;

    /* noise definition */
    float *noiseMean;
    float *noiseRMS;

    /* samples per input chunk (for noiseMean/noiseRMS) */
    unsigned samplesPerChunk;

    /* input file for standalone mode */
    FILE *fp;

    /* output */
    char fileprefix[80], basedir[120];
    unsigned secs_per_file;
    char use_pc_time, single_file_mode;

    /* detection */
    float detection_threshold;

    /* devices */
    unsigned num_threads;
    unsigned *gpu_ids;
    unsigned num_gpus;
} SURVEY;

#endif
