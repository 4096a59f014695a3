// Forward-mode dual numbers with the interface and arithmetic of Ceres
// Solver's ceres::Jet<T, N> (jet.h), restated for building the reference's
// pyDeform sources in oracle/_ref (Ceres is an un-vendored submodule of the
// reference).  Only the operations those sources use are provided.  Each
// operation is Ceres' published rule, one IEEE operation per component:
//   (f + g) = (f.a + g.a, f.v + g.v)      (f - g) = (f.a - g.a, f.v - g.v)
//   (f * g) = (f.a * g.a, f.a * g.v + f.v * g.a)
//   (f / g) = (f.a / g.a, (f.v - (f.a / g.a) * g.v) / g.a), with 1/g.a formed once
// and scalar operands are jets with a zero derivative folded away.
// Comparisons compare the values.  The value is the first member, as in
// Ceres (the reference reads it through a pointer cast).
#ifndef MO_REFSHIM_CERES_JET_
#define MO_REFSHIM_CERES_JET_

#include <Eigen/Core>

namespace ceres {

template <typename Tp, int N>
struct Jet {
    typedef Eigen::Matrix<Tp, N, 1> Vec;
    Jet() : a(Tp(0)) { v.setZero(); }
    explicit Jet(const Tp& value) : a(value) { v.setZero(); }
    Jet(const Tp& value, int k) : a(value) {
        v.setZero();
        v[k] = Tp(1);
    }
    Jet(const Tp& value, const Vec& dv) : a(value), v(dv) {}

    Jet& operator+=(const Jet& y) { return *this = *this + y; }
    Jet& operator-=(const Jet& y) { return *this = *this - y; }
    Jet& operator*=(const Jet& y) { return *this = *this * y; }
    Jet& operator/=(const Jet& y) { return *this = *this / y; }
    Jet& operator+=(const Tp& s) { return *this = *this + s; }
    Jet& operator-=(const Tp& s) { return *this = *this - s; }
    Jet& operator*=(const Tp& s) { return *this = *this * s; }
    Jet& operator/=(const Tp& s) { return *this = *this / s; }

    Tp a;
    Vec v;
};

template <typename Tp, int N>
inline Jet<Tp, N> operator+(const Jet<Tp, N>& f) { return f; }
template <typename Tp, int N>
inline Jet<Tp, N> operator-(const Jet<Tp, N>& f) { return Jet<Tp, N>(-f.a, -f.v); }

template <typename Tp, int N>
inline Jet<Tp, N> operator+(const Jet<Tp, N>& f, const Jet<Tp, N>& g) { return Jet<Tp, N>(f.a + g.a, f.v + g.v); }
template <typename Tp, int N>
inline Jet<Tp, N> operator+(const Jet<Tp, N>& f, Tp s) { return Jet<Tp, N>(f.a + s, f.v); }
template <typename Tp, int N>
inline Jet<Tp, N> operator+(Tp s, const Jet<Tp, N>& f) { return Jet<Tp, N>(f.a + s, f.v); }

template <typename Tp, int N>
inline Jet<Tp, N> operator-(const Jet<Tp, N>& f, const Jet<Tp, N>& g) { return Jet<Tp, N>(f.a - g.a, f.v - g.v); }
template <typename Tp, int N>
inline Jet<Tp, N> operator-(const Jet<Tp, N>& f, Tp s) { return Jet<Tp, N>(f.a - s, f.v); }
template <typename Tp, int N>
inline Jet<Tp, N> operator-(Tp s, const Jet<Tp, N>& f) { return Jet<Tp, N>(s - f.a, -f.v); }

template <typename Tp, int N>
inline Jet<Tp, N> operator*(const Jet<Tp, N>& f, const Jet<Tp, N>& g) {
    return Jet<Tp, N>(f.a * g.a, f.a * g.v + f.v * g.a);
}
template <typename Tp, int N>
inline Jet<Tp, N> operator*(const Jet<Tp, N>& f, Tp s) { return Jet<Tp, N>(f.a * s, f.v * s); }
template <typename Tp, int N>
inline Jet<Tp, N> operator*(Tp s, const Jet<Tp, N>& f) { return Jet<Tp, N>(f.a * s, f.v * s); }

template <typename Tp, int N>
inline Jet<Tp, N> operator/(const Jet<Tp, N>& f, const Jet<Tp, N>& g) {
    const Tp inv = Tp(1) / g.a;
    const Tp q = f.a * inv;
    return Jet<Tp, N>(q, (f.v - q * g.v) * inv);
}
template <typename Tp, int N>
inline Jet<Tp, N> operator/(const Jet<Tp, N>& f, Tp s) {
    const Tp inv = Tp(1) / s;
    return Jet<Tp, N>(f.a * inv, f.v * inv);
}

#define MO_REFSHIM_JET_CMP(op)                                                                       \
    template <typename Tp, int N>                                                                    \
    inline bool operator op(const Jet<Tp, N>& f, const Jet<Tp, N>& g) { return f.a op g.a; }         \
    template <typename Tp, int N>                                                                    \
    inline bool operator op(const Jet<Tp, N>& f, Tp s) { return f.a op s; }                          \
    template <typename Tp, int N>                                                                    \
    inline bool operator op(Tp s, const Jet<Tp, N>& g) { return s op g.a; }
MO_REFSHIM_JET_CMP(<)
MO_REFSHIM_JET_CMP(<=)
MO_REFSHIM_JET_CMP(>)
MO_REFSHIM_JET_CMP(>=)
MO_REFSHIM_JET_CMP(==)
MO_REFSHIM_JET_CMP(!=)
#undef MO_REFSHIM_JET_CMP

}  // namespace ceres

#endif
