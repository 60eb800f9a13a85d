// A caller written against the reference's stage interface, following the call sequence of the
// reference's standalone driver (src/MDSM.cpp:19-64,100-169): parse the observation file, read
// an 8-bit sigproc filterbank block by block with the corner turn into the library-owned input
// buffer, rows of nsamp + maxshift samples (the first block with its maxshift tail), then
// next_chunk / start_processing until the file ends, then tearDownMDSM.  Built against
// include/dedispersion_manager.h; no Qt, no Pelican.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "dedispersion_manager.h"

static long read_spectra(FILE *fp, int nchans, float *buffer, int nsamp, int maxshift,
                         int counter)
{
    const int to_read = counter == 0 ? nsamp + maxshift : nsamp;
    const int shift = counter == 0 ? 0 : maxshift;
    std::vector<unsigned char> spec((size_t)nchans);
    long got = 0;
    for (int i = 0; i < to_read; ++i) {
        if (fread(spec.data(), 1, spec.size(), fp) != spec.size()) break;
        for (int c = 0; c < nchans; ++c)
            buffer[(long)c * (nsamp + maxshift) + shift + i] = (float)spec[(size_t)c];
        ++got;
    }
    return got;
}

int main(int argc, char **argv)
{
    if (argc < 3) {
        fprintf(stderr, "usage: %s file.fil obs.xml\n", argv[0]);
        return 2;
    }
    mdsm_sigproc_header h;
    if (mdsm_sigproc_read_header(argv[1], &h) != MDSM_OK || h.nbits != 8) {
        fprintf(stderr, "header: %s\n", mdsm_last_error());
        return 3;
    }
    SURVEY *survey = processSurveyParameters(argv[2]);
    if (!survey) {
        fprintf(stderr, "survey: %s\n", mdsm_last_error());
        return 4;
    }
    survey->nbits = (unsigned)h.nbits;
    float *input_buffer = initialiseMDSM(survey);
    if (!input_buffer) {
        fprintf(stderr, "initialise: %s\n", mdsm_last_error());
        return 5;
    }
    FILE *fp = fopen(argv[1], "rb");
    if (!fp || fseek(fp, (long)h.header_bytes, SEEK_SET) != 0) return 6;
    unsigned counter = 0, outputs = 0;
    unsigned long total = 0;
    while (true) {
        long data_read = read_spectra(fp, h.nchans, input_buffer, (int)survey->nsamp,
                                      (int)survey->maxshift, (int)counter);
        if (counter == 0) data_read = data_read < (long)survey->maxshift
                                          ? 0 : data_read - (long)survey->maxshift;
        if (data_read < (long)survey->nsamp) data_read = 0;  // whole blocks only
        unsigned x = 0;
        float *out = next_chunk((unsigned)data_read, x, survey->tsamp * survey->nsamp * counter,
                                survey->tsamp);
        if (out && x != 0u && x != (unsigned)-1) ++outputs;
        if (!start_processing((unsigned)data_read)) break;
        total += (unsigned long)data_read;
        counter++;
    }
    fclose(fp);
    tearDownMDSM();
    printf("blocks %u outputs %u samples %lu\n", counter, outputs, total);
    return 0;
}
