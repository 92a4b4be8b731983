// ORACLE — test infrastructure only.
//
// An operation-counting scalar for the restatement in oracle.cpp: the sampling and
// integrand functions there are templates over their real type, and instantiating
// them with `cnt` (and its complex companion `cx`) runs the same algorithm while
// counting every floating-point operation a sample performs.  The counts give the
// algorithmic operations per sample of the reference's loop (srcs/feynman_integral.hpp:
// 162-362 with the sector draw of srcs/tropical_sampling.hpp:468-564), which the
// benchmark divides by a kernel's time for its roofline.
//
// Conventions: a real add/sub, mul or div counts one each; sqrt and each
// transcendental (pow, exp, log, sin, cos, atan2) count once in their own class;
// comparisons are counted apart and are not floating-point operations.  Complex
// operations are written out in real operations: (a+bi)(c+di) = 4 mul + 2 add,
// division = 6 mul + 3 add + 2 div, |z| = 2 mul + 1 add + 1 sqrt, arg z = 1
// transcendental, log z = |z| + 2 transcendentals, polar(r, t) = 2 transcendentals +
// 2 mul.  Sign changes, loads, integer and bitmask work are free.
#pragma once

#include <cmath>
#include <cstdint>

namespace fto {

struct op_counts {
    double add = 0, mul = 0, div = 0, sqrt = 0, trans = 0, cmp = 0;
};

op_counts& ops();   // this thread's counters

struct cnt {
    double v = 0.0;
    cnt() = default;
    cnt(double x) : v(x) {}
    explicit operator double() const { return v; }
    cnt& operator+=(cnt o) { ops().add++; v += o.v; return *this; }
    cnt& operator-=(cnt o) { ops().add++; v -= o.v; return *this; }
    cnt& operator*=(cnt o) { ops().mul++; v *= o.v; return *this; }
    cnt& operator/=(cnt o) { ops().div++; v /= o.v; return *this; }
};

inline cnt operator+(cnt a, cnt b) { ops().add++; return cnt(a.v + b.v); }
inline cnt operator-(cnt a, cnt b) { ops().add++; return cnt(a.v - b.v); }
inline cnt operator*(cnt a, cnt b) { ops().mul++; return cnt(a.v * b.v); }
inline cnt operator/(cnt a, cnt b) { ops().div++; return cnt(a.v / b.v); }
inline cnt operator-(cnt a) { return cnt(-a.v); }
inline bool operator<(cnt a, cnt b) { ops().cmp++; return a.v < b.v; }
inline bool operator>(cnt a, cnt b) { ops().cmp++; return a.v > b.v; }
inline bool operator<=(cnt a, cnt b) { ops().cmp++; return a.v <= b.v; }
inline bool operator>=(cnt a, cnt b) { ops().cmp++; return a.v >= b.v; }
inline bool operator==(cnt a, cnt b) { ops().cmp++; return a.v == b.v; }
inline bool operator!=(cnt a, cnt b) { ops().cmp++; return a.v != b.v; }

inline cnt fabs(cnt a) { return cnt(std::fabs(a.v)); }
inline cnt sqrt(cnt a) { ops().sqrt++; return cnt(std::sqrt(a.v)); }
inline cnt pow(cnt a, cnt b) { ops().trans++; return cnt(std::pow(a.v, b.v)); }
inline cnt exp(cnt a) { ops().trans++; return cnt(std::exp(a.v)); }
inline cnt log(cnt a) { ops().trans++; return cnt(std::log(a.v)); }
inline cnt cos(cnt a) { ops().trans++; return cnt(std::cos(a.v)); }
inline cnt sin(cnt a) { ops().trans++; return cnt(std::sin(a.v)); }
inline bool isfinite(cnt a) { return std::isfinite(a.v); }

// complex number of counted parts (constructors explicit, so that mixed real /
// complex expressions pick the cheaper real-operand overloads below)
struct cx {
    cnt re, im;
    cx() = default;
    explicit cx(double r, double i = 0.0) : re(r), im(i) {}
    explicit cx(cnt r, cnt i = cnt(0.0)) : re(r), im(i) {}
    cnt real() const { return re; }
    cnt imag() const { return im; }
    cx& operator+=(const cx& o) { re += o.re; im += o.im; return *this; }
    cx& operator-=(const cx& o) { re -= o.re; im -= o.im; return *this; }
    cx& operator*=(const cx& o);
    cx& operator/=(const cx& o);
};

inline cx operator-(const cx& a) { return cx(-a.re, -a.im); }
inline cx operator+(const cx& a, const cx& b) { return cx(a.re + b.re, a.im + b.im); }
inline cx operator-(const cx& a, const cx& b) { return cx(a.re - b.re, a.im - b.im); }
inline cx operator*(const cx& a, const cx& b)
{
    return cx(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
inline cx operator/(const cx& a, const cx& b)
{
    const cnt d = b.re * b.re + b.im * b.im;
    return cx((a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d);
}
inline cx& cx::operator*=(const cx& o) { return *this = *this * o; }
inline cx& cx::operator/=(const cx& o) { return *this = *this / o; }

inline cx operator*(const cx& a, cnt s) { return cx(a.re * s, a.im * s); }
inline cx operator*(cnt s, const cx& a) { return cx(s * a.re, s * a.im); }
inline cx operator*(const cx& a, double s) { return a * cnt(s); }
inline cx operator*(double s, const cx& a) { return cnt(s) * a; }
inline cx operator/(const cx& a, cnt s) { return cx(a.re / s, a.im / s); }
inline cx operator/(const cx& a, double s) { return a / cnt(s); }
inline cx operator/(double s, const cx& a) { return cx(s) / a; }
inline cx operator+(const cx& a, double s) { return cx(a.re + s, a.im); }
inline cx operator+(double s, const cx& a) { return cx(s + a.re, a.im); }
inline cx operator-(const cx& a, double s) { return cx(a.re - s, a.im); }

inline cnt abs(const cx& z) { return sqrt(z.re * z.re + z.im * z.im); }
inline cnt arg(const cx& z) { ops().trans++; return cnt(std::atan2(z.im.v, z.re.v)); }
inline cx log(const cx& z) { return cx(log(abs(z)), arg(z)); }
inline cx polar(cnt r, cnt t) { return cx(r * cos(t), r * sin(t)); }

}  // namespace fto
