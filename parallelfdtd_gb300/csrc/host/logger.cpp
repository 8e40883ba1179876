// Levelled stderr logger (replaces the reference's boost::wformat logger,
// ParallelFDTD src/logger.h:46-80, which appends to a file on every message).
#include "logger.h"

#include <cstdarg>
#include <cstdio>
#include <cstdlib>

static log_level g_level = LOG_WARNING;

void setLogLevel(log_level level) { g_level = level; }

void loggerInit() {
  const char* env = std::getenv("PFDTD_LOG_LEVEL");
  if (env) g_level = (log_level)std::atoi(env);
}

void c_log_msg(log_level level, const char* fmt, ...) {
  if (level > g_level) return;
  static const char* names[] = {"ERROR", "WARNING", "INFO", "DEBUG", "VERBOSE"};
  std::fprintf(stderr, "[pfdtd %s] ", names[level]);
  va_list ap;
  va_start(ap, fmt);
  std::vfprintf(stderr, fmt, ap);
  va_end(ap);
  std::fputc('\n', stderr);
}
