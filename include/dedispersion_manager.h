/*
 * dedispersion_manager.h -- the reference's stage interface under its own names
 * (src/mdsm/dedispersion_manager.h:7-12), forwarding to the C ABI in mdsm_gb300.h, so callers
 * such as the standalone driver (src/MDSM.cpp) and the Pelican MdsmModule
 * (src/pelican-mdsm/modules/MdsmModule.cpp) compile against this library unchanged.  Qt is not
 * required: processSurveyParameters takes a path string.  Where <QString> can be included, this
 * header includes it, as the reference's does (src/mdsm/dedispersion_manager.h:5), and adds the
 * reference's QString overload, so a caller that includes this header before any Qt header and
 * calls processSurveyParameters(QString(...)) (src/MDSM.cpp:2,42,79,91) compiles.
 */
#ifndef DEDISPERSION_MANAGER_H_
#define DEDISPERSION_MANAGER_H_

#include "mdsm_gb300.h"
#include "survey.h"

#if defined(__cplusplus) && defined(__has_include)
#if __has_include(<QString>)
#include <QString>
#define MDSM_GB300_HAVE_QSTRING 1
#endif
#endif

#ifdef __cplusplus
inline SURVEY *processSurveyParameters(const char *filepath)
{
    return mdsm_processSurveyParameters(filepath);
}
#if defined(MDSM_GB300_HAVE_QSTRING) || defined(QSTRING_H)
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
