// Stand-in for <boost/format.hpp> — test infrastructure only.
//
// The reference's logger (src/logger.h:26) includes <boost/format.hpp> for
// boost::wformat, a printf-like formatter fed with operator%.  Boost is not
// installed here, so this header supplies the small part of that interface the
// reference's host sources use: construction from a (wide) format string,
// operator% to bind the next argument, and output to a stream.  It is only
// used to compile the reference's own sources for the parity checks; the
// product never includes it.
//
// Directives handled: %N% (positional), %s %d %u %f %g %e %x %i %c %p with
// optional flags/width/precision, and %%.  Anything else is copied verbatim.
#ifndef PFDTD_REF_STUB_BOOST_FORMAT_HPP
#define PFDTD_REF_STUB_BOOST_FORMAT_HPP

#include <ostream>
#include <sstream>
#include <string>
#include <vector>

namespace boost {

template <class Ch>
class basic_format {
 public:
  using string_type = std::basic_string<Ch>;
  explicit basic_format(const Ch* s) : fmt_(s ? s : string_type()) {}
  explicit basic_format(const string_type& s) : fmt_(s) {}

  template <class T>
  basic_format& operator%(const T& v) {
    std::basic_ostringstream<Ch> os;
    os << v;
    args_.push_back(os.str());
    return *this;
  }
  basic_format& operator%(const char* v) { return bind_narrow(v ? v : "(null)"); }
  basic_format& operator%(char* v) { return bind_narrow(v ? v : "(null)"); }
  basic_format& operator%(const std::string& v) { return bind_narrow(v.c_str()); }

  string_type str() const {
    string_type out;
    size_t next = 0;
    for (size_t i = 0; i < fmt_.size(); ++i) {
      Ch c = fmt_[i];
      if (c != Ch('%')) { out.push_back(c); continue; }
      if (i + 1 < fmt_.size() && fmt_[i + 1] == Ch('%')) { out.push_back(c); ++i; continue; }
      // positional %N%
      size_t j = i + 1;
      size_t num = 0;
      bool digits = false;
      while (j < fmt_.size() && fmt_[j] >= Ch('0') && fmt_[j] <= Ch('9')) {
        num = num * 10 + size_t(fmt_[j] - Ch('0'));
        ++j;
        digits = true;
      }
      if (digits && j < fmt_.size() && fmt_[j] == Ch('%')) {
        if (num >= 1 && num <= args_.size()) out += args_[num - 1];
        i = j;
        continue;
      }
      // printf-style directive: skip flags, width, precision, length, then the conversion
      j = i + 1;
      while (j < fmt_.size() && string_type(1, fmt_[j]).find_first_of(flag_chars()) == 0) ++j;
      static const char conv[] = "sdufgexicpXEG";
      bool found = false;
      while (j < fmt_.size()) {
        for (const char* k = conv; *k; ++k)
          if (fmt_[j] == Ch(*k)) found = true;
        if (found) break;
        ++j;
      }
      if (!found) { out.push_back(c); continue; }
      if (next < args_.size()) out += args_[next++];
      i = j;
    }
    return out;
  }

 private:
  static const Ch* flag_chars() {
    static const Ch f[] = {Ch('-'), Ch('+'), Ch(' '), Ch('#'), Ch('0'), Ch('1'), Ch('2'),
                           Ch('3'), Ch('4'), Ch('5'), Ch('6'), Ch('7'), Ch('8'), Ch('9'),
                           Ch('.'), Ch('l'), Ch('h'), Ch('z'), Ch(0)};
    return f;
  }
  basic_format& bind_narrow(const char* s) {
    string_type w;
    for (const char* p = s; *p; ++p) w.push_back(Ch((unsigned char)*p));
    args_.push_back(w);
    return *this;
  }
  string_type fmt_;
  std::vector<string_type> args_;
};

template <class Ch>
std::basic_ostream<Ch>& operator<<(std::basic_ostream<Ch>& os, const basic_format<Ch>& f) {
  return os << f.str();
}

using format = basic_format<char>;
using wformat = basic_format<wchar_t>;

inline std::string str(const format& f) { return f.str(); }
inline std::wstring str(const wformat& f) { return f.str(); }

}  // namespace boost

#endif
