/*
 * ad_tape.h -- reverse-mode automatic differentiation by operator
 * overloading, for the CPU ORACLE only (test infrastructure).
 *
 * The oracle's step is a template on its REAL type.  Instantiated with
 * adt::AD it records every arithmetic operation on a tape (the value in
 * double precision, the operand node indices and the two local partial
 * derivatives); a reverse sweep over the tape then gives the exact
 * transposed Jacobian-vector product of the restated step at the recorded
 * state.  Branches (IF tests, MIN/MAX, ABS) follow the recorded values, so
 * the product is the derivative of the branch the state selects.  This is
 * the checker for the hand-written reverse kernels of the GPU library.
 */
#ifndef ORACLE_AD_TAPE_H_
#define ORACLE_AD_TAPE_H_

#include <cmath>
#include <cstdint>
#include <vector>

namespace adt {

struct Tape {
    std::vector<int32_t> a, b;     // operand nodes (-1: none)
    std::vector<double> da, db;    // partial derivatives d(node)/d(a), d(node)/d(b)
    std::vector<double> adj;
    int32_t push(int32_t ia, double pa, int32_t ib, double pb) {
        a.push_back(ia);
        da.push_back(pa);
        b.push_back(ib);
        db.push_back(pb);
        return (int32_t)(a.size() - 1);
    }
    void clear() {
        a.clear(); b.clear(); da.clear(); db.clear(); adj.clear();
    }
    size_t size() const { return a.size(); }
    // adjoint sweep: adj must be seeded on the output nodes
    void reverse() {
        for (size_t n = a.size(); n-- > 0;) {
            double g = adj[n];
            if (g == 0.0) continue;
            if (a[n] >= 0) adj[(size_t)a[n]] += g * da[n];
            if (b[n] >= 0) adj[(size_t)b[n]] += g * db[n];
        }
    }
};

inline Tape *&tape() {
    static thread_local Tape *t = nullptr;
    return t;
}

struct AD {
    double v;
    int32_t i;    // tape node, -1 for a passive constant
    AD() : v(0.0), i(-1) {}
    AD(double x) : v(x), i(-1) {}
    AD(float x) : v((double)x), i(-1) {}
    AD(int x) : v((double)x), i(-1) {}
    AD(double x, int32_t node) : v(x), i(node) {}
    explicit operator double() const { return v; }
    explicit operator float() const { return (float)v; }
    explicit operator int() const { return (int)v; }
    explicit operator long() const { return (long)v; }
    explicit operator bool() const { return v != 0.0; }
    AD &operator+=(const AD &o);
    AD &operator-=(const AD &o);
    AD &operator*=(const AD &o);
    AD &operator/=(const AD &o);
};

// a new node from one or two active operands; passive results stay off the tape
inline AD rec1(double v, const AD &x, double dx) {
    if (x.i < 0 || !tape()) return AD(v);
    return AD(v, tape()->push(x.i, dx, -1, 0.0));
}
inline AD rec2(double v, const AD &x, double dx, const AD &y, double dy) {
    if (!tape() || (x.i < 0 && y.i < 0)) return AD(v);
    if (x.i < 0) return AD(v, tape()->push(y.i, dy, -1, 0.0));
    if (y.i < 0) return AD(v, tape()->push(x.i, dx, -1, 0.0));
    return AD(v, tape()->push(x.i, dx, y.i, dy));
}
// an independent variable
inline AD independent(double v) { return AD(v, tape()->push(-1, 0.0, -1, 0.0)); }

inline AD operator+(const AD &x, const AD &y) { return rec2(x.v + y.v, x, 1.0, y, 1.0); }
inline AD operator-(const AD &x, const AD &y) { return rec2(x.v - y.v, x, 1.0, y, -1.0); }
inline AD operator*(const AD &x, const AD &y) { return rec2(x.v * y.v, x, y.v, y, x.v); }
inline AD operator/(const AD &x, const AD &y) {
    double q = x.v / y.v;
    return rec2(q, x, 1.0 / y.v, y, -q / y.v);
}
inline AD operator-(const AD &x) { return rec1(-x.v, x, -1.0); }
inline AD operator+(const AD &x) { return x; }
inline AD &AD::operator+=(const AD &o) { return *this = *this + o; }
inline AD &AD::operator-=(const AD &o) { return *this = *this - o; }
inline AD &AD::operator*=(const AD &o) { return *this = *this * o; }
inline AD &AD::operator/=(const AD &o) { return *this = *this / o; }

inline bool operator<(const AD &x, const AD &y) { return x.v < y.v; }
inline bool operator>(const AD &x, const AD &y) { return x.v > y.v; }
inline bool operator<=(const AD &x, const AD &y) { return x.v <= y.v; }
inline bool operator>=(const AD &x, const AD &y) { return x.v >= y.v; }
inline bool operator==(const AD &x, const AD &y) { return x.v == y.v; }
inline bool operator!=(const AD &x, const AD &y) { return x.v != y.v; }

inline AD sqrt(const AD &x) {
    double s = std::sqrt(x.v);
    return rec1(s, x, s > 0.0 ? 0.5 / s : 0.0);
}
inline AD fabs(const AD &x) { return rec1(std::fabs(x.v), x, x.v < 0.0 ? -1.0 : 1.0); }
inline AD abs(const AD &x) { return fabs(x); }
inline AD log(const AD &x) { return rec1(std::log(x.v), x, 1.0 / x.v); }
inline AD log10(const AD &x) { return rec1(std::log10(x.v), x, 1.0 / (x.v * std::log(10.0))); }
inline AD exp(const AD &x) {
    double e = std::exp(x.v);
    return rec1(e, x, e);
}
inline AD sin(const AD &x) { return rec1(std::sin(x.v), x, std::cos(x.v)); }
inline AD cos(const AD &x) { return rec1(std::cos(x.v), x, -std::sin(x.v)); }
inline AD asin(const AD &x) { return rec1(std::asin(x.v), x, 1.0 / std::sqrt(1.0 - x.v * x.v)); }
inline AD tanh(const AD &x) {
    double t = std::tanh(x.v);
    return rec1(t, x, 1.0 - t * t);
}
inline AD atan2(const AD &y, const AD &x) {
    double r2 = x.v * x.v + y.v * y.v;
    return rec2(std::atan2(y.v, x.v), y, x.v / r2, x, -y.v / r2);
}
inline AD pow(const AD &x, const AD &y) {
    double p = std::pow(x.v, y.v);
    double dx = y.v == 0.0 ? 0.0 : y.v * std::pow(x.v, y.v - 1.0);
    double dy = (y.i >= 0 && x.v > 0.0) ? p * std::log(x.v) : 0.0;
    return rec2(p, x, dx, y, dy);
}
inline bool isfinite(const AD &x) { return std::isfinite(x.v); }

}  // namespace adt

#endif /* ORACLE_AD_TAPE_H_ */
