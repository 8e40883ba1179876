// Levelled stderr logger (replaces the reference's boost::wformat logger,
// ParallelFDTD src/logger.h:46-80, which appends to a file on every message).
#include "logger.h"

#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cwchar>

static log_level g_level = LOG_WARNING;

void setLogLevel(log_level level) { g_level = level; }

// PFDTD_LOG_LEVEL: 0 nothing .. 6 verbose (the log_level values).
void loggerInit() {
  const char* env = std::getenv("PFDTD_LOG_LEVEL");
  if (env) g_level = (log_level)std::atoi(env);
}

void c_log_msg(log_level level, const char* fmt, ...) {
  if (level == LOG_NOTHING || level > g_level) return;
  static const char* names[] = {"", "CRITICAL", "ERROR", "WARNING", "INFO", "DEBUG", "VERBOSE"};
  std::fprintf(stderr, "[pfdtd %s] ", names[(int)level < 7 ? (int)level : 6]);
  va_list ap;
  va_start(ap, fmt);
  std::vfprintf(stderr, fmt, ap);
  va_end(ap);
  std::fputc('\n', stderr);
}

Logger::~Logger() {
  if (!live_ || level_ == LOG_NOTHING || level_ > g_level) return;
  c_log_msg(level_, "%s", format().c_str());
}

// boost::format directives: %% -> %, %N% -> argument N (1-based), a
// printf-style directive %[flags][width][.prec]type -> the next argument
// (numbers formatted with the directive, anything else as streamed).
std::string Logger::format() const {
  std::string out;
  size_t next = 0;
  auto narrow = [](const std::wstring& w) {
    std::string s;
    for (wchar_t c : w) s.push_back((c >= 0 && c < 128) ? (char)c : '?');
    return s;
  };
  const std::wstring& f = fmt_;
  for (size_t i = 0; i < f.size(); ++i) {
    if (f[i] != L'%') {
      out.push_back((f[i] >= 0 && f[i] < 128) ? (char)f[i] : '?');
      continue;
    }
    if (i + 1 < f.size() && f[i + 1] == L'%') {
      out.push_back('%');
      ++i;
      continue;
    }
    size_t j = i + 1;
    size_t num = 0;
    while (j < f.size() && f[j] >= L'0' && f[j] <= L'9') num = num * 10 + (size_t)(f[j++] - L'0');
    if (j < f.size() && f[j] == L'%' && j > i + 1) {  // %N%
      if (num >= 1 && num <= args_.size()) out += narrow(args_[num - 1].text);
      i = j;
      continue;
    }
    // printf-style: flags, width, precision, length modifiers, type
    j = i + 1;
    std::string spec = "%";
    while (j < f.size() && std::wcschr(L"-+ #0", f[j]) && f[j]) spec.push_back((char)f[j++]);
    while (j < f.size() && f[j] >= L'0' && f[j] <= L'9') spec.push_back((char)f[j++]);
    if (j < f.size() && f[j] == L'.') {
      spec.push_back('.');
      ++j;
      while (j < f.size() && f[j] >= L'0' && f[j] <= L'9') spec.push_back((char)f[j++]);
    }
    while (j < f.size() && std::wcschr(L"hlLqjzt", f[j]) && f[j]) ++j;
    if (j >= f.size()) {  // dangling %: literal
      out.push_back('%');
      continue;
    }
    const char type = (char)f[j];
    i = j;
    if (next >= args_.size()) continue;
    const Arg& a = args_[next++];
    char buf[128];
    if (std::strchr("diouxXc", type) && a.kind <= 1) {
      const std::string s = spec + "ll" + (type == 'c' ? 'd' : type);
      if (a.kind == 0) std::snprintf(buf, sizeof buf, s.c_str(), a.i);
      else std::snprintf(buf, sizeof buf, s.c_str(), a.u);
      out += buf;
    } else if (std::strchr("feEgGaA", type) && a.kind <= 2) {
      const double v = a.kind == 2 ? a.d : (a.kind == 0 ? (double)a.i : (double)a.u);
      std::snprintf(buf, sizeof buf, (spec + type).c_str(), v);
      out += buf;
    } else {
      out += narrow(a.text);
    }
  }
  return out;
}
