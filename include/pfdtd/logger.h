// Levelled logger with the reference's interface: the C bridge c_log_msg
// (ParallelFDTD src/kernels/cudaUtils.cu:6-19) and the C++
// log_msg<level>(L"format") % arg % arg ... records (src/logger.h:46-84),
// without boost: the format takes boost::format's directives (%1%, %N%,
// printf-style %d %u %f %.3f %s ..., %%).  Messages at or above the threshold
// go to stderr; nothing is written to files.  The level values are the
// reference's.
#ifndef PFDTD_LOGGER_H
#define PFDTD_LOGGER_H

enum log_level {
  LOG_NOTHING,
  LOG_CRITICAL,
  LOG_ERROR,
  LOG_WARNING,
  LOG_INFO,
  LOG_DEBUG,
  LOG_VERBOSE
};

void c_log_msg(log_level level, const char* fmt, ...);
void loggerInit();
void setLogLevel(log_level level);

#ifdef __cplusplus
#include <sstream>
#include <string>
#include <type_traits>
#include <vector>

// One log record: arguments are collected with operator% and the message is
// formatted and emitted when the record is destroyed (the end of the
// statement that made it).
class Logger {
 public:
  Logger(log_level level, const wchar_t* msg) : level_(level), fmt_(msg ? msg : L"") {}
  Logger(const Logger& other)
      : level_(other.level_), fmt_(other.fmt_), args_(other.args_) {
    other.live_ = false;  // only the last copy emits
  }
  Logger& operator=(const Logger&) = delete;
  ~Logger();

  template <typename T>
  Logger& operator%(const T& value) {
    Arg a;
    number(a, value, std::integral_constant<int, std::is_same<T, bool>::value ? 3
                                                : std::is_integral<T>::value ? 0
                                                : std::is_floating_point<T>::value ? 2 : 3>());
    std::wostringstream o;
    put(o, value);
    a.text = o.str();
    args_.push_back(a);
    return *this;
  }

 private:
  struct Arg {
    int kind = 3;  // 0 signed, 1 unsigned, 2 floating, 3 text
    long long i = 0;
    unsigned long long u = 0;
    double d = 0.0;
    std::wstring text;
  };
  template <typename T>
  static void number(Arg& a, const T& v, std::integral_constant<int, 0>) {
    a.kind = std::is_signed<T>::value ? 0 : 1;
    a.i = (long long)v;
    a.u = (unsigned long long)v;
  }
  template <typename T>
  static void number(Arg& a, const T& v, std::integral_constant<int, 2>) {
    a.kind = 2;
    a.d = (double)v;
  }
  template <typename T>
  static void number(Arg&, const T&, std::integral_constant<int, 3>) {}
  template <typename T>
  static void put(std::wostringstream& o, const T& v) { o << v; }
  static void put(std::wostringstream& o, const std::string& v) { o << v.c_str(); }
  static void put(std::wostringstream& o, const std::wstring& v) { o << v; }
  std::string format() const;

  log_level level_;
  std::wstring fmt_;
  std::vector<Arg> args_;
  mutable bool live_ = true;
};

template <log_level level>
Logger log_msg(const wchar_t* msg) {
  return Logger(level, msg);
}
#endif

#endif
