// Levelled logger with the reference's C bridge name (c_log_msg,
// ParallelFDTD src/kernels/cudaUtils.cu:6-19).  Messages at or above the
// threshold go to stderr; nothing is written to files.
#ifndef PFDTD_LOGGER_H
#define PFDTD_LOGGER_H

enum log_level { LOG_ERROR = 0, LOG_WARNING, LOG_INFO, LOG_DEBUG, LOG_VERBOSE };

void c_log_msg(log_level level, const char* fmt, ...);
void loggerInit();
void setLogLevel(log_level level);

#endif
