// ffmt.hpp — Fortran formatted-output edit descriptors, as gfortran writes
// them, for byte-compatible output files:
//   Aw  output of a CHARACTER variable of declared length `len`: the value is
//       blank-padded to `len`, then the leftmost w characters are written
//       when len >= w, otherwise it is right-justified in w;
//   Iw  right-justified integer;
//   Fw.d, Ew.d (0.ddddddE+xx form, exponents beyond 99 written as +xxx);
//   nX, Tc positioning (T overwrites, X past the end pads with blanks);
//   L   logical without width: "T" / "F".
// A Record collects one output record; str() returns it without the newline.
#pragma once
#include <cstdint>
#include <string>

namespace sodahost {

class Record {
public:
    Record &a(const std::string &s);                       // A without width
    Record &a(const std::string &s, int w, int len = -1);  // Aw; len = declared length (-1: the string's own)
    Record &i(long long v, int w);
    Record &f(double v, int w, int d);
    Record &e(double v, int w, int d);
    Record &x(int n = 1);
    Record &t(int col);                                    // column, 1-based
    Record &l(bool v);
    // a non-advancing write whose format had positional descriptors left
    // after its last item: the pending blanks count once the record ends
    Record &pending(int n = 1) { pend_ += n; return *this; }
    std::string str() const;

private:
    void put(const std::string &s);
    std::string buf_;
    size_t pos_ = 0;
    int pend_ = 0;
};

std::string fmt_i(long long v, int w);
std::string fmt_f(double v, int w, int d);
std::string fmt_e(double v, int w, int d);
std::string fmt_a(const std::string &s, int w, int len = -1);

}  // namespace sodahost
