// Operation-counting stand-in for `double`, used to compile raptor_port.c
// as C++ with -DPORT_COUNT_FLOPS (TEST INFRASTRUCTURE ONLY).
//
// Convention: every +, -, *, / and every libm call (sqrt, exp, log, pow,
// sin, cos, tan, acos, cbrt) is one floating-point operation; comparisons,
// fabs, fmin, fmax, negation and conversions are free.  This is the
// "algorithmic work" the roofline divides by the measured time.
#pragma once
#include <cmath>

extern "C" unsigned long long port_flop_counter;

struct cdouble {
    double v;
    cdouble() = default;
    constexpr cdouble(double x) : v(x) {}
    explicit operator double() const { return v; }
    explicit operator int() const { return (int)v; }
};

static inline cdouble tick(double x) {
    ++port_flop_counter;
    return cdouble(x);
}

#define CD_BINOP(OP)                                                                          \
    static inline cdouble operator OP(cdouble a, cdouble b) { return tick(a.v OP b.v); }      \
    static inline cdouble operator OP(cdouble a, double b) { return tick(a.v OP b); }         \
    static inline cdouble operator OP(double a, cdouble b) { return tick(a OP b.v); }         \
    static inline cdouble operator OP(cdouble a, int b) { return tick(a.v OP b); }            \
    static inline cdouble operator OP(int a, cdouble b) { return tick(a OP b.v); }            \
    static inline cdouble& operator OP##=(cdouble& a, cdouble b) { a = a OP b; return a; }    \
    static inline cdouble& operator OP##=(cdouble& a, double b) { a = a OP b; return a; }
CD_BINOP(+)
CD_BINOP(-)
CD_BINOP(*)
CD_BINOP(/)
#undef CD_BINOP

static inline cdouble operator-(cdouble a) { return cdouble(-a.v); }

#define CD_CMP(OP)                                                                     \
    static inline bool operator OP(cdouble a, cdouble b) { return a.v OP b.v; }        \
    static inline bool operator OP(cdouble a, double b) { return a.v OP b; }           \
    static inline bool operator OP(double a, cdouble b) { return a OP b.v; }           \
    static inline bool operator OP(cdouble a, int b) { return a.v OP b; }
CD_CMP(<)
CD_CMP(>)
CD_CMP(<=)
CD_CMP(>=)
CD_CMP(==)
CD_CMP(!=)
#undef CD_CMP

#define CD_FN1(F) \
    static inline cdouble F(cdouble a) { return tick(std::F(a.v)); }
CD_FN1(sqrt)
CD_FN1(exp)
CD_FN1(log)
CD_FN1(sin)
CD_FN1(cos)
CD_FN1(tan)
CD_FN1(acos)
CD_FN1(cbrt)
#undef CD_FN1
static inline cdouble pow(cdouble a, cdouble b) { return tick(std::pow(a.v, b.v)); }
static inline cdouble pow(cdouble a, double b) { return tick(std::pow(a.v, b)); }
static inline cdouble fabs(cdouble a) { return cdouble(std::fabs(a.v)); }
static inline cdouble fmin(cdouble a, cdouble b) { return cdouble(std::fmin(a.v, b.v)); }
static inline cdouble fmin(double a, cdouble b) { return cdouble(std::fmin(a, b.v)); }
static inline cdouble fmax(cdouble a, cdouble b) { return cdouble(std::fmax(a.v, b.v)); }
static inline cdouble fmax(cdouble a, double b) { return cdouble(std::fmax(a.v, b)); }
