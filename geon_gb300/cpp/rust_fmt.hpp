// Rust's float formatting where the ports of the reference's executables need
// it: `{:.Ne}` / `{:+.Ne}` (LowerExp: no exponent padding, no '+' in the
// exponent) and `{}` for the small whole and decimal values they print.
#pragma once
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

namespace rustfmt {

inline std::string exp(double v, int prec, bool sign = false) {
  char buf[64];
  std::snprintf(buf, sizeof buf, sign ? "%+.*e" : "%.*e", prec, v);
  std::string s(buf);
  const size_t e = s.find('e');
  if (e == std::string::npos) return s;  // inf / nan
  const int ex = std::atoi(s.c_str() + e + 1);
  return s.substr(0, e) + "e" + std::to_string(ex);
}

inline std::string fixed(double v, int prec) {
  char buf[64];
  std::snprintf(buf, sizeof buf, "%.*f", prec, v);
  return buf;
}

// `{}` of a finite f64: the fewest significant digits that read back to v,
// written positionally (never with an exponent), e.g. 20, 0.05, 0.00000035496.
inline std::string display(double v) {
  char buf[512];
  int p = 1;
  for (; p < 17; ++p) {
    std::snprintf(buf, sizeof buf, "%.*e", p - 1, v);
    if (std::strtod(buf, nullptr) == v) break;
  }
  std::snprintf(buf, sizeof buf, "%.*e", p - 1, v);
  const int e10 = std::atoi(std::strchr(buf, 'e') + 1);
  const int decimals = p - 1 - e10 > 0 ? p - 1 - e10 : 0;
  std::snprintf(buf, sizeof buf, "%.*f", decimals, v);
  return buf;
}

inline std::string pad_left(const std::string& s, size_t w) { return s.size() >= w ? s : std::string(w - s.size(), ' ') + s; }

// pad to w characters (UTF-8 code points, as Rust counts them)
inline std::string pad_right(const std::string& s, size_t w) {
  size_t n = 0;
  for (unsigned char c : s) n += (c & 0xC0) != 0x80;
  return n >= w ? s : s + std::string(w - n, ' ');
}

}  // namespace rustfmt
