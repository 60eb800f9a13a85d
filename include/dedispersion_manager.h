/*
 * dedispersion_manager.h -- the reference's stage interface under its own names
 * (src/mdsm/dedispersion_manager.h:7-12), forwarding to the C ABI in mdsm_gb300.h, so callers
 * such as the standalone driver (src/MDSM.cpp) and the Pelican MdsmModule
 * (src/pelican-mdsm/modules/MdsmModule.cpp) compile against this library unchanged.  Qt is not
 * required: processSurveyParameters takes a path string; a QString overload is provided when
 * QString is available.
 */
#ifndef DEDISPERSION_MANAGER_H_
#define DEDISPERSION_MANAGER_H_

#include "mdsm_gb300.h"
#include "survey.h"

#ifdef __cplusplus
inline SURVEY *processSurveyParameters(const char *filepath)
{
    return mdsm_processSurveyParameters(filepath);
}
#ifdef QSTRING_H
inline SURVEY *processSurveyParameters(QString filepath)
{
    return mdsm_processSurveyParameters(filepath.toUtf8().constData());
}
#endif
inline float *initialiseMDSM(SURVEY *input_survey) { return mdsm_initialiseMDSM(input_survey); }
inline float *next_chunk(unsigned int data_read, unsigned &samples, double timestamp = 0,
                         double blockRate = 0, float *mean = NULL, float *rms = NULL)
{
    return mdsm_next_chunk(data_read, &samples, timestamp, blockRate, mean, rms);
}
inline int start_processing(unsigned int data_read) { return mdsm_start_processing(data_read); }
inline void tearDownMDSM() { mdsm_tearDownMDSM(); }
#endif

#endif  // DEDISPERSION_MANAGER_H_
