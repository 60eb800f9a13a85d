/*
 * ref_sp_driver.cpp -- TEST INFRASTRUCTURE ONLY.  C entry points over the single-pulse
 * prototype's own functions (src/prototypes/singlepulse.cpp: createFFTKernel :41-67, convolve
 * :69-87, pruneRelated :90-120, pruneRelatedDownfactors :122-146), compiled from the reference
 * tree by oracle/Makefile into oracle/_ref/ against the FFTW stand-in in oracle/ref_shim/.  The
 * prototype's main() (a benchmark over an uninitialised buffer) is renamed and never called.
 * Used in this container to make the golden fixtures that pin the oracle's single-pulse mode
 * (tests/golden/make_golden.py); never shipped, never part of the product.
 */
#define main singlepulse_prototype_main
#include "singlepulse.cpp"
#undef main

/* Spectrum of the width-`factor` template of length fftlen, fftlen/2 + 1 complex bins. */
extern "C" int ref_sp_kernel(unsigned factor, unsigned fftlen, float *out)
{
    fftwf_complex *k = (fftwf_complex *)fftwf_malloc(fftlen / 2 * sizeof(fftwf_complex));
    createFFTKernel(k, factor, fftlen);
    memcpy(out, k, (fftlen / 2 + 1) * sizeof(fftwf_complex));
    fftwf_free(k);
    return 0;
}

/* One chunk convolved with the width-`factor` template as the prototype's main loop does it
 * (:199-212, :248, :257): r2c of the chunk, convolve(), c2r into the chunk buffer. */
extern "C" int ref_sp_convolve(const float *in, unsigned factor, unsigned fftlen, float *result)
{
    fftwf_complex *kern = (fftwf_complex *)fftwf_malloc(fftlen / 2 * sizeof(fftwf_complex));
    createFFTKernel(kern, factor, fftlen);
    float *chunk = (float *)fftwf_malloc(fftlen * sizeof(float));
    fftwf_complex *fc = (fftwf_complex *)fftwf_malloc(fftlen / 2 * sizeof(fftwf_complex));
    fftwf_complex *cc = (fftwf_complex *)fftwf_malloc(fftlen / 2 * sizeof(fftwf_complex));
    fftwf_plan chunkPlan = fftwf_plan_dft_r2c_1d(fftlen, chunk, fc, FFTW_ESTIMATE);
    fftwf_plan convPlan = fftwf_plan_dft_c2r_1d(fftlen, cc, chunk, FFTW_ESTIMATE);
    memcpy(chunk, in, fftlen * sizeof(float));
    fftwf_execute(chunkPlan);
    convolve(fc, kern, cc, chunk, fftlen, convPlan);
    memcpy(result, chunk, fftlen * sizeof(float));
    fftwf_destroy_plan(chunkPlan);
    fftwf_destroy_plan(convPlan);
    fftwf_free(kern);
    fftwf_free(chunk);
    fftwf_free(fc);
    fftwf_free(cc);
    return 0;
}

/* pruneRelated on one list (bins ascending); pruned entries come back as bin 0, value 0. */
extern "C" void ref_sp_prune_related(unsigned *bins, float *values, unsigned num,
                                     unsigned factor)
{
    InitialCandidate *c = (InitialCandidate *)malloc(num * sizeof(InitialCandidate));
    for (unsigned i = 0; i < num; i++) {
        c[i].bin = bins[i];
        c[i].value = values[i];
    }
    pruneRelated(c, factor, num);
    for (unsigned i = 0; i < num; i++) {
        bins[i] = c[i].bin;
        values[i] = c[i].value;
    }
    free(c);
}

/* pruneRelatedDownfactors on one DM's list, with the mask zeroed first (the prototype passes
 * an uninitialised malloc'd mask, :291).  mask[i] != 0 marks a pruned candidate. */
extern "C" void ref_sp_prune_downfactors(const long *bins, const float *values,
                                         const unsigned *downfacts, unsigned n,
                                         unsigned numDownFacts, char *mask)
{
    std::vector<Candidate> v(n);
    for (unsigned i = 0; i < n; i++) {
        v[i].dm = 0.0f;
        v[i].value = values[i];
        v[i].time = 0.0;
        v[i].bin = bins[i];
        v[i].downfact = downfacts[i];
    }
    memset(mask, 0, n);
    pruneRelatedDownfactors(v, mask, numDownFacts);
}
