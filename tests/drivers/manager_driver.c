/*
 * A manager written against the reference's internal C ABI (include/dedispersion_thread.h):
 * the thread set-up and block handshake of src/mdsm/dedispersion_manager.cpp (initialiseMDSM
 * :269-382, next_chunk :416-484, start_processing :487-501, tearDownMDSM :385-413) with an
 * output thread that follows process_output's barrier and lock pattern
 * (src/mdsm/dedispersion_output.cpp:216-356) but writes each block's series to a file instead
 * of detecting, driven block by block as src/MDSM.cpp:128-170 does from a file of time-major
 * float spectra (corner turn as readBinaryData, :100-125).  C, pthreads, no Qt.
 *
 * usage: manager_driver spectra.f32 out.f32 nchans nsamp fch1 foff tsamp brute lowdm dmstep
 *                       tdms useL1Cache
 *        manager_driver spectra.f32 out.f32 nchans nsamp fch1 foff tsamp subband nsubs
 *                       "lowdm,highdm,dmstep,sub_dmstep,ncalls,calldms,binsize;..."
 * prints "blocks B outputs O maxshift M dedispersed_size D" on success.
 *
 * Environment: MDSM_DRIVER_THREADS=N runs N workers (devices beyond the machine's repeat its
 * first); MDSM_DRIVER_OUTPUT=dir starts the library's process_output (the reference's output
 * thread, src/mdsm/dedispersion_manager.cpp:331-344) instead of the capture thread, writing
 * its candidates to dir/cands.dat at threshold MDSM_DRIVER_THRESHOLD (default 6).  Block k is
 * handed in with timestamp 1000 + k nsamp tsamp and blockRate tsamp, as next_chunk's callers
 * pass them (src/mdsm/dedispersion_manager.cpp:416-484).
 */
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "dedispersion_output.h"
#include "dedispersion_thread.h"
#include "mdsm_gb300.h"

typedef struct {
    int iterations, maxiters;
    float *output_buffer;
    size_t total;  /* floats of all threads' series */
    unsigned short stop;
    pthread_rwlock_t *rw_lock;
    pthread_barrier_t *input_barrier, *output_barrier;
    FILE *out;
    int written;
} CAPTURE;

static SURVEY survey;
static SUBBAND_PASSES passes[8];
static DEVICES *devices;
static int num_devices, loop_counter, outSwitch = 1;
static pthread_barrier_t input_barrier, output_barrier;
static pthread_rwlock_t rw_lock = PTHREAD_RWLOCK_INITIALIZER;
static pthread_t *threads, output_thread;
static THREAD_PARAMS *threads_params;
static CAPTURE capture;
static OUTPUT_PARAMS output_params;
static int use_output;
static float *input_buffer, *output_buffer, *dmshifts;
static unsigned pnsamp, ppnsamp;

static void barrier(pthread_barrier_t *b)
{
    int r = pthread_barrier_wait(b);
    if (!(r == 0 || r == PTHREAD_BARRIER_SERIAL_THREAD)) {
        fprintf(stderr, "barrier\n");
        exit(3);
    }
}

/* process_output's loop, writing the output buffer of every data iteration */
static void *capture_output(void *arg)
{
    CAPTURE *p = (CAPTURE *)arg;
    int i, iters = 0, lc = 0;
    while (1) {
        barrier(p->input_barrier);
        if (lc >= p->iterations) {
            fwrite(p->output_buffer, sizeof(float), p->total, p->out);
            p->written++;
        }
        barrier(p->output_barrier);
        pthread_rwlock_rdlock(p->rw_lock);
        if (p->stop) {
            if (iters >= p->iterations - 1) {
                pthread_rwlock_unlock(p->rw_lock);
                for (i = 0; i < p->maxiters - p->iterations; i++) {
                    barrier(p->input_barrier);
                    barrier(p->output_barrier);
                }
                break;
            }
            iters++;
        }
        pthread_rwlock_unlock(p->rw_lock);
        lc++;
    }
    return arg;
}

static float *initialise(FILE *out)
{
    int k;
    unsigned i;
    devices = call_initialise_devices(&survey);
    if (!devices) return NULL;
    const char *nthr = getenv("MDSM_DRIVER_THREADS");
    if (nthr && atoi(nthr) > devices->num_devices) {
        /* more workers than devices: the extra ones share the first device */
        int n = atoi(nthr);
        DEVICE_INFO *d = (DEVICE_INFO *)calloc((size_t)n, sizeof(DEVICE_INFO));
        for (k = 0; k < n; k++) d[k] = devices->devices[k < devices->num_devices ? k : 0];
        free(devices->devices);
        devices->devices = d;
        devices->num_devices = n;
    }
    num_devices = devices->num_devices;
    survey.num_threads = (unsigned)num_devices;
    threads = (pthread_t *)calloc((size_t)num_devices, sizeof(pthread_t));
    threads_params = (THREAD_PARAMS *)calloc((size_t)num_devices, sizeof(THREAD_PARAMS));
    dmshifts = (float *)malloc(survey.nchans * sizeof(float));
    for (i = 0; i < survey.nchans; i++)
        dmshifts[i] = mdsm_dmdelay(survey.fch1 + survey.foff * (float)i, survey.fch1);
    float hiDM = survey.useBruteForce ? survey.lowdm + survey.dmstep * (float)(survey.tdms - 1)
                                      : passes[survey.num_passes - 1].highdm;
    int maxshift = (int)(dmshifts[survey.nchans - 1] * hiDM / survey.tsamp);
    survey.maxshift = (unsigned)maxshift;
    size_t outsize = 0;
    if (survey.useBruteForce)
        outsize = (size_t)survey.nsamp * survey.tdms / (unsigned)num_devices;
    else {
        for (i = 0; i < survey.num_passes; i++)
            outsize += (size_t)(passes[i].ncalls / num_devices) * passes[i].calldms /
                       passes[i].binsize;
        outsize *= survey.nsamp;
    }
    size_t inputsize = (size_t)(survey.nsamp + maxshift) * survey.nchans * sizeof(float);
    input_buffer = (float *)calloc(1, inputsize);
    output_buffer = (float *)calloc((size_t)num_devices * outsize, sizeof(float));
    pthread_barrier_init(&input_barrier, NULL, (unsigned)num_devices + 2);
    pthread_barrier_init(&output_barrier, NULL, (unsigned)num_devices + 2);
    capture.iterations = 2;
    capture.maxiters = 2;
    capture.output_buffer = output_buffer;
    capture.total = (size_t)num_devices * outsize;
    capture.rw_lock = &rw_lock;
    capture.input_barrier = &input_barrier;
    capture.output_barrier = &output_barrier;
    capture.out = out;
    if (use_output) {
        output_params.nthreads = num_devices;
        output_params.iterations = 2;
        output_params.maxiters = 2;
        output_params.output_buffer = output_buffer;
        output_params.dedispersed_size = outsize;
        output_params.stop = 0;
        output_params.rw_lock = &rw_lock;
        output_params.input_barrier = &input_barrier;
        output_params.output_barrier = &output_barrier;
        output_params.start = time(NULL);
        output_params.survey = &survey;
        pthread_create(&output_thread, NULL, process_output, &output_params);
    } else {
        pthread_create(&output_thread, NULL, capture_output, &capture);
    }
    for (k = 0; k < num_devices; k++) {
        THREAD_PARAMS *t = &threads_params[k];
        t->iterations = 1;
        t->maxiters = 2;
        t->stop = 0;
        t->maxshift = maxshift;
        t->dedispersed_size = outsize;
        t->binsize = 1;
        t->output = &output_buffer[outsize * (size_t)k];
        t->input = input_buffer;
        t->dmshifts = dmshifts;
        t->thread_num = (unsigned short)k;
        t->num_threads = (unsigned short)num_devices;
        t->device_id = devices->devices[k].device_id;
        t->rw_lock = &rw_lock;
        t->input_barrier = &input_barrier;
        t->output_barrier = &output_barrier;
        t->start = time(NULL);
        t->survey = &survey;
        t->inputsize = inputsize;
        t->outputsize = outsize * sizeof(float);
        if (pthread_create(&threads[k], NULL, call_dedisperse, t)) return NULL;
    }
    barrier(&input_barrier);
    return input_buffer;
}

static void next_chunk(unsigned data_read, unsigned block)
{
    int k;
    pthread_rwlock_wrlock(&rw_lock);
    barrier(&output_barrier);
    ppnsamp = pnsamp;
    pnsamp = data_read;
    survey.timestamp = 1000.0 + (double)block * (double)survey.nsamp * (double)survey.tsamp;
    survey.blockRate = (double)survey.tsamp;
    if (data_read == 0) {
        capture.stop = 1;
        output_params.stop = 1;
        for (k = 0; k < num_devices; k++) threads_params[k].stop = 1;
    }
    pthread_rwlock_unlock(&rw_lock);
}

static int start_processing(unsigned data_read)
{
    if (data_read == 0 && outSwitch)
        outSwitch = 0;
    else if (data_read == 0 && !outSwitch)
        return 0;
    barrier(&input_barrier);
    return ++loop_counter;
}

static void tear_down(void)
{
    int k;
    for (k = 0; k < num_devices; k++) pthread_join(threads[k], NULL);
    pthread_join(output_thread, NULL);
    pthread_barrier_destroy(&input_barrier);
    pthread_barrier_destroy(&output_barrier);
    free(devices->devices);
    free(devices);
    free(output_buffer);
    free(threads_params);
    free(input_buffer);
    free(dmshifts);
    free(threads);
}

/* readBinaryData (src/MDSM.cpp:100-125) over float spectra */
static unsigned read_block(FILE *fp, float *buffer, unsigned counter)
{
    unsigned nch = survey.nchans, ns = survey.nsamp, ms = survey.maxshift, i, j, got = 0;
    unsigned to_read = counter == 0 ? ns + ms : ns, shift = counter == 0 ? 0 : ms;
    float *spec = (float *)malloc(nch * sizeof(float));
    for (i = 0; i < to_read; i++) {
        if (fread(spec, sizeof(float), nch, fp) != nch) break;
        for (j = 0; j < nch; j++) buffer[(size_t)j * (ns + ms) + shift + i] = spec[j];
        got++;
    }
    free(spec);
    return got;
}

int main(int argc, char **argv)
{
    if (argc < 10) {
        fprintf(stderr, "usage: see the header of this file\n");
        return 2;
    }
    memset(&survey, 0, sizeof survey);
    survey.nchans = (unsigned)atoi(argv[3]);
    survey.nsamp = (unsigned)atoi(argv[4]);
    survey.fch1 = (float)atof(argv[5]);
    survey.foff = (float)atof(argv[6]);
    survey.tsamp = (float)atof(argv[7]);
    if (!strcmp(argv[8], "brute")) {
        if (argc < 13) return 2;
        survey.useBruteForce = 1;
        survey.lowdm = (float)atof(argv[9]);
        survey.dmstep = (float)atof(argv[10]);
        survey.tdms = (unsigned)atoi(argv[11]);
        survey.useL1Cache = atoi(argv[12]) != 0;
    } else {
        char *spec = argv[10], *tok;
        survey.useBruteForce = 0;
        survey.nsubs = (unsigned)atoi(argv[9]);
        for (tok = strtok(spec, ";"); tok && survey.num_passes < 8; tok = strtok(NULL, ";")) {
            SUBBAND_PASSES *p = &passes[survey.num_passes++];
            memset(p, 0, sizeof *p);
            if (sscanf(tok, "%f,%f,%f,%f,%d,%d,%d", &p->lowdm, &p->highdm, &p->dmstep,
                       &p->sub_dmstep, &p->ncalls, &p->calldms, &p->binsize) != 7)
                return 2;
            p->ndms = p->ncalls * p->calldms;
        }
        survey.pass_parameters = passes;
        survey.tdms = 0;
        for (unsigned i = 0; i < survey.num_passes; i++)
            survey.tdms += (unsigned)passes[i].ndms;
    }
    const char *odir = getenv("MDSM_DRIVER_OUTPUT");
    if (odir && *odir) {
        use_output = 1;
        snprintf(survey.basedir, sizeof survey.basedir, "%s", odir);
        snprintf(survey.fileprefix, sizeof survey.fileprefix, "cands");
        survey.single_file_mode = 1;
        const char *thr = getenv("MDSM_DRIVER_THRESHOLD");
        survey.detection_threshold = thr ? (float)atof(thr) : 6.0f;
    }
    FILE *fp = fopen(argv[1], "rb"), *out = fopen(argv[2], "wb");
    if (!fp || !out) return 4;
    if (!initialise(out)) {
        fprintf(stderr, "initialise: %s\n", mdsm_last_error());
        return 5;
    }
    unsigned counter = 0, data_read;
    while (1) {
        if (counter == 0) {
            data_read = read_block(fp, input_buffer, counter);
            data_read = data_read < survey.maxshift ? 0 : data_read - survey.maxshift;
        } else {
            data_read = read_block(fp, input_buffer, counter);
        }
        if (data_read < survey.nsamp) data_read = 0;  /* whole blocks only */
        next_chunk(data_read, counter);
        if (!start_processing(data_read)) break;
        counter++;
    }
    tear_down();
    fclose(fp);
    fclose(out);
    printf("blocks %u outputs %d maxshift %u dedispersed_size %zu threads %d\n", counter,
           capture.written, survey.maxshift, capture.total, num_devices);
    return 0;
}
