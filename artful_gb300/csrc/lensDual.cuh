/* artful_cuda — dual numbers: a double with N directional derivatives carried along (forward-mode
 * differentiation).  Instantiating the trace's templated core (lensCore.cuh) with Dual<N> gives, for every
 * pixel, its radiance and the radiance's derivatives along N parameter directions, through exactly the
 * arithmetic the trace performs: the FP64 forward-mode reference the adjoint is checked against.
 *
 * Rules: sums and products by the chain rule; comparisons, floor and truncation act on the value (their
 * derivative is zero almost everywhere); |x| takes the value's sign; min / max select an operand, with its
 * derivative. */
#pragma once

#include "lensCore.cuh"

namespace artf {

template <int N> struct Dual {
    double v;
    double d[N];

    ARTF_HD Dual() : v(0) {
        for (int k = 0; k < N; ++k) d[k] = 0;
    }
    ARTF_HD Dual(double x) : v(x) {
        for (int k = 0; k < N; ++k) d[k] = 0;
    }
    ARTF_HD Dual(float x) : Dual((double)x) {}
    ARTF_HD Dual(int x) : Dual((double)x) {}
    ARTF_HD explicit operator double() const { return v; }
    ARTF_HD explicit operator float() const { return (float)v; }
};

#define DUAL_OP(op, value, deriv)                                                            \
    template <int N> ARTF_HD Dual<N> operator op(const Dual<N>& a, const Dual<N>& b) {      \
        Dual<N> r;                                                                           \
        r.v = value;                                                                         \
        for (int k = 0; k < N; ++k) r.d[k] = deriv;                                          \
        return r;                                                                            \
    }
DUAL_OP(+, a.v + b.v, a.d[k] + b.d[k])
DUAL_OP(-, a.v - b.v, a.d[k] - b.d[k])
DUAL_OP(*, a.v * b.v, a.d[k] * b.v + a.v * b.d[k])
DUAL_OP(/, a.v / b.v, (a.d[k] * b.v - a.v * b.d[k]) / (b.v * b.v))
#undef DUAL_OP

template <int N> ARTF_HD Dual<N> operator-(const Dual<N>& a) {
    Dual<N> r;
    r.v = -a.v;
    for (int k = 0; k < N; ++k) r.d[k] = -a.d[k];
    return r;
}
#define DUAL_CMP(op)                                                                                   \
    template <int N> ARTF_HD bool operator op(const Dual<N>& a, const Dual<N>& b) { return a.v op b.v; }
DUAL_CMP(<)
DUAL_CMP(>)
DUAL_CMP(<=)
DUAL_CMP(>=)
DUAL_CMP(==)
DUAL_CMP(!=)
#undef DUAL_CMP

/* f(a) with f' known at a */
template <int N> ARTF_HD Dual<N> chain(const Dual<N>& a, double value, double slope) {
    Dual<N> r;
    r.v = value;
    for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * slope;
    return r;
}

template <int N> ARTF_HD Dual<N> sqrtR(const Dual<N>& a) {
    const double s = sqrt(a.v);
    return chain(a, s, .5 / s);
}
template <int N> ARTF_HD Dual<N> rootR(const Dual<N>& a) { return sqrtR(a); }
template <int N> ARTF_HD Dual<N> recipR(const Dual<N>& a) { return chain(a, 1.0 / a.v, -1.0 / (a.v * a.v)); }
template <int N> ARTF_HD Dual<N> invSqrtR(const Dual<N>& a) {
    const double s = 1.0 / sqrt(a.v);
    return chain(a, s, -.5 * s / a.v);
}
template <int N> ARTF_HD Dual<N> divR(const Dual<N>& a, const Dual<N>& b) { return a / b; }
template <int N> ARTF_HD Dual<N> divSqrtR(const Dual<N>& a, const Dual<N>& x) { return a * invSqrtR(x); }
template <int N> ARTF_HD Dual<N> floorR(const Dual<N>& a) { return Dual<N>(floor(a.v)); }
template <int N> ARTF_HD Dual<N> absR(const Dual<N>& a) { return a.v < 0 ? -a : a; }
template <int N> ARTF_HD Dual<N> expR(const Dual<N>& a) {
    const double e = exp(a.v);
    return chain(a, e, e);
}
template <int N> ARTF_HD Dual<N> logR(const Dual<N>& a) { return chain(a, log(a.v), 1.0 / a.v); }
template <int N> ARTF_HD int32_t truncI(const Dual<N>& a) { return truncI(a.v); }

}  // namespace artf
