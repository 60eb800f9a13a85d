/*
 * ref_host_driver.cpp -- TEST INFRASTRUCTURE ONLY.  C entry points over the reference's own
 * host code (src/mdsm/dedispersion_output.cpp and src/mdsm/file_handler.cpp), compiled from
 * the reference tree by oracle/Makefile into oracle/_ref/.  Used in this container to pin the
 * oracle (tests/golden/make_golden.py); never shipped, never part of the product.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "survey.h"
#include "file_handler.h"

/* dedispersion_output.cpp:135-136 (not declared in any reference header) */
void process_brute(float *buffer, FILE *output, SURVEY *survey, int read_nsamp, size_t size,
                   double timestamp, double blockRate, time_t start_time, float *mean, float *rms);
float medianOfFive(float n1, float n2, float n3, float n4, float n5);
/* dedispersion_output.cpp:56-57 */
void process_subband(float *buffer, FILE *output, SURVEY *survey, int read_nsamp, size_t size,
                     double timestamp, double blockRate, float *mean, float *rms);

extern "C" int ref_process_brute(float *buf, int tdms, int nsamp, float lowdm, float dmstep,
                                 float threshold, const char *outpath)
{
    SURVEY s;
    memset(&s, 0, sizeof(s));
    s.tdms = (unsigned)tdms;
    s.nsamp = (unsigned)nsamp;
    s.lowdm = lowdm;
    s.dmstep = dmstep;
    s.detection_threshold = threshold;
    s.num_threads = 1;
    s.useBruteForce = 1;
    FILE *fp = fopen(outpath, "w");
    if (!fp) return -1;
    process_brute(buf, fp, &s, nsamp, (size_t)tdms * (size_t)nsamp, 0.0, 1.0, time(NULL), NULL,
                  NULL);
    fclose(fp);
    return 0;
}

/* process_brute with caller noise statistics (mean != NULL, one value per spc samples). */
extern "C" int ref_process_brute_chunked(float *buf, int tdms, int nsamp, float lowdm,
                                         float dmstep, float threshold, int spc, float *mean,
                                         float *rms, const char *outpath)
{
    SURVEY s;
    memset(&s, 0, sizeof(s));
    s.tdms = (unsigned)tdms;
    s.nsamp = (unsigned)nsamp;
    s.lowdm = lowdm;
    s.dmstep = dmstep;
    s.detection_threshold = threshold;
    s.num_threads = 1;
    s.useBruteForce = 1;
    s.samplesPerChunk = (unsigned)spc;
    FILE *fp = fopen(outpath, "w");
    if (!fp) return -1;
    process_brute(buf, fp, &s, nsamp, (size_t)tdms * (size_t)nsamp, 0.0, 1.0, time(NULL), mean,
                  rms);
    fclose(fp);
    return 0;
}

/* process_subband for one pass (its pass loop reads the first pass's rows for every pass, so
 * one pass is the case it computes as intended) with caller noise statistics; mean == NULL
 * would dereference the null pointer at :63. */
extern "C" int ref_process_subband_chunked(float *buf, int nsamp, float lowdm, float dmstep,
                                           float sub_dmstep, int ncalls, int calldms,
                                           int binsize, float threshold, int spc, float *mean,
                                           float *rms, const char *outpath)
{
    SUBBAND_PASSES pass;
    memset(&pass, 0, sizeof(pass));
    pass.lowdm = lowdm;
    pass.dmstep = dmstep;
    pass.sub_dmstep = sub_dmstep;
    pass.ncalls = ncalls;
    pass.calldms = calldms;
    pass.binsize = binsize;
    SURVEY s;
    memset(&s, 0, sizeof(s));
    s.pass_parameters = &pass;
    s.num_passes = 1;
    s.num_threads = 1;
    s.detection_threshold = threshold;
    s.samplesPerChunk = (unsigned)spc;
    FILE *fp = fopen(outpath, "w");
    if (!fp) return -1;
    const size_t rows = (size_t)ncalls * (size_t)calldms;
    process_subband(buf, fp, &s, nsamp, rows * (size_t)(nsamp / binsize), 0.0, 1.0, mean, rms);
    fclose(fp);
    return 0;
}

extern "C" float ref_median_of_five(float a, float b, float c, float d, float e)
{
    return medianOfFive(a, b, c, d, e);
}

/* file_handler.cpp:193: read_block over a file holding the raw bytes. */
extern "C" long ref_read_block(const char *path, int nbits, float *out, unsigned long nread)
{
    FILE *fp = fopen(path, "rb");
    if (!fp) return -1;
    long n = (long)read_block(fp, nbits, out, nread);
    fclose(fp);
    return n;
}

/* file_handler.cpp:56-187 on a file: the fields the tests compare. */
extern "C" int ref_read_header(const char *path, int *ints, double *dbls, long long *total,
                               char *source)
{
    FILE *fp = fopen(path, "rb");
    if (!fp) return -1;
    FILE_HEADER *h = read_header(fp);
    fclose(fp);
    if (!h) return -2;
    ints[0] = h->nchans; ints[1] = h->nbits; ints[2] = h->nifs; ints[3] = h->machine_id;
    ints[4] = h->telescope_id; ints[5] = h->data_type; ints[6] = h->nbeams; ints[7] = h->ibeam;
    dbls[0] = h->tstart; dbls[1] = h->tsamp; dbls[2] = h->fch1; dbls[3] = h->foff;
    dbls[4] = h->src_raj; dbls[5] = h->src_dej; dbls[6] = h->refdm;
    *total = h->total_bytes;
    strcpy(source, h->source_name);
    free(h);
    return 0;
}
