// ffmt.cpp — Fortran edit descriptors (see ffmt.hpp).
#include "ffmt.hpp"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

namespace sodahost {

static std::string stars(int w) { return std::string(w > 0 ? w : 0, '*'); }

std::string fmt_i(long long v, int w)
{
    char b[64];
    std::snprintf(b, sizeof b, "%lld", v);
    const int n = (int)std::strlen(b);
    if (n > w) return stars(w);
    return std::string(w - n, ' ') + b;
}

std::string fmt_f(double v, int w, int d)
{
    if (!std::isfinite(v)) {
        const std::string s = std::isnan(v) ? "NaN" : (v > 0 ? "Infinity" : "-Infinity");
        return (int)s.size() > w ? stars(w) : std::string(w - s.size(), ' ') + s;
    }
    char b[512];
    std::snprintf(b, sizeof b, "%.*f", d, v);
    std::string s = b;
    // a negative value that rounds to zero keeps its sign in gfortran ("-0.00")
    if ((int)s.size() > w && s.size() >= 2 && s[0] == '0' && s[1] == '.') s = s.substr(1);   // drop optional zero
    if ((int)s.size() > w && s.size() >= 3 && s[0] == '-' && s[1] == '0' && s[2] == '.') s = "-" + s.substr(2);
    if ((int)s.size() > w) return stars(w);
    return std::string(w - s.size(), ' ') + s;
}

// Ew.d: sign, "0.", d significant digits, exponent letter and two digits
// (three digits without the letter when |exponent| > 99).
std::string fmt_e(double v, int w, int d)
{
    if (!std::isfinite(v)) {
        const std::string s = std::isnan(v) ? "NaN" : (v > 0 ? "Infinity" : "-Infinity");
        return (int)s.size() > w ? stars(w) : std::string(w - s.size(), ' ') + s;
    }
    std::string digits(d, '0');
    int exp10 = 0;
    bool neg = std::signbit(v);
    if (v != 0.0) {
        char b[128];
        std::snprintf(b, sizeof b, "%.*e", d - 1, std::fabs(v));   // x.xxxxxe+yy with d significant digits
        const char *p = b;
        std::string m;
        while (*p && *p != 'e') {
            if (*p != '.') m.push_back(*p);
            ++p;
        }
        exp10 = std::atoi(p + 1) + 1;
        digits = m;
    } else {
        neg = false;   // gfortran prints +0.0 as "0.000000E+00"
    }
    std::string s = neg ? "-" : "";
    s += "0." + digits;
    const int ae = std::abs(exp10);
    char eb[16];
    if (ae <= 99) std::snprintf(eb, sizeof eb, "E%c%02d", exp10 < 0 ? '-' : '+', ae);
    else if (ae <= 999) std::snprintf(eb, sizeof eb, "%c%03d", exp10 < 0 ? '-' : '+', ae);
    else return stars(w);
    s += eb;
    if ((int)s.size() > w && s.compare(0, 2, "0.") == 0) s = s.substr(1);
    if ((int)s.size() > w && s.compare(0, 3, "-0.") == 0) s = "-" + s.substr(2);
    if ((int)s.size() > w) return stars(w);
    return std::string(w - s.size(), ' ') + s;
}

std::string fmt_a(const std::string &s, int w, int len)
{
    std::string v = s;
    if (len >= 0) {
        if ((int)v.size() > len) v = v.substr(0, len);
        v.resize(len, ' ');
    }
    if ((int)v.size() >= w) return v.substr(0, w);
    return std::string(w - v.size(), ' ') + v;
}

void Record::put(const std::string &s)
{
    if (pend_) {   // pending positional blanks are written before the next item
        pos_ += pend_;
        pend_ = 0;
    }
    if (buf_.size() < pos_) buf_.resize(pos_, ' ');
    if (pos_ + s.size() > buf_.size()) buf_.resize(pos_ + s.size(), ' ');
    buf_.replace(pos_, s.size(), s);
    pos_ += s.size();
}

Record &Record::a(const std::string &s) { put(s); return *this; }
Record &Record::a(const std::string &s, int w, int len) { put(fmt_a(s, w, len)); return *this; }
Record &Record::i(long long v, int w) { put(fmt_i(v, w)); return *this; }
Record &Record::f(double v, int w, int d) { put(fmt_f(v, w, d)); return *this; }
Record &Record::e(double v, int w, int d) { put(fmt_e(v, w, d)); return *this; }
Record &Record::x(int n) { pos_ += n; return *this; }
Record &Record::t(int col) { pos_ = col > 0 ? (size_t)(col - 1) : 0; return *this; }
Record &Record::l(bool v) { put(v ? "T" : "F"); return *this; }

std::string Record::str() const
{
    std::string s = buf_;
    const size_t end = pos_ + pend_;
    if (pend_ && s.size() < end) s.resize(end, ' ');
    return s;
}

}  // namespace sodahost
