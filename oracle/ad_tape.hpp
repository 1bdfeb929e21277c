// ad_tape.hpp -- TEST INFRASTRUCTURE ONLY.
//
// A reverse-mode automatic-differentiation scalar (FP64 values, one tape per
// thread) used to derive the reference gradient of the oracle's own templated
// restatement of the trace and the mips: instantiating ClipmapTracer and
// downsample_f4_on with T = ad::Var differentiates exactly the arithmetic the
// FP64 oracle evaluates, independently of the GPU's hand-written adjoint.
//
// A Var is a constant (no dependence on the differentiated inputs), a leaf
// (input scalar k of the atlas) or a tape node with up to two parents and
// their partial derivatives.  Operations on constants record nothing, so a
// tape holds only the atlas-dependent part of a computation.  Piecewise-
// constant functions (floor, ceil, trunc) and comparisons use the value;
// min / max / clamps pass the derivative of the selected argument, which
// holds every branch (level choice, occlusion stop, clamps) at its value --
// the same convention as the GPU adjoint.
//
// The <cmath> overloads for Var are declared in namespace std so that the
// restatement's qualified calls (std::floor, std::pow, ...) instantiate
// unchanged; this header must be included before the templates that use them.
#pragma once

#include <cmath>
#include <cstdint>
#include <type_traits>
#include <vector>

namespace vcto {
namespace ad {

struct Node {
    int64_t a, b;  // parents: >= 0 tape node, <= -2 leaf (-2 - k), -1 none
    double da, db;
};

inline std::vector<Node>& tape() {
    static thread_local std::vector<Node> t;
    return t;
}

struct Var {
    double v;
    int64_t i;  // >= 0: tape node; -1: constant; <= -2: leaf scalar -2 - i
    Var() : v(0.0), i(-1) {}
    template <class N, std::enable_if_t<std::is_arithmetic_v<N>, int> = 0>
    Var(N x) : v(static_cast<double>(x)), i(-1) {}
    static Var leaf(double value, int64_t k) {
        Var r;
        r.v = value;
        r.i = -2 - k;
        return r;
    }
    explicit operator int() const { return static_cast<int>(v); }
    explicit operator float() const { return static_cast<float>(v); }
    explicit operator double() const { return v; }
};

inline Var node(double v, const Var& x, double dx, const Var& y, double dy) {
    const bool ax = x.i != -1, ay = y.i != -1;
    if (!ax && !ay) return Var(v);
    auto& t = tape();
    t.push_back({ax ? x.i : -1, ay ? y.i : -1, ax ? dx : 0.0, ay ? dy : 0.0});
    Var r;
    r.v = v;
    r.i = static_cast<int64_t>(t.size()) - 1;
    return r;
}
inline Var node(double v, const Var& x, double dx) { return node(v, x, dx, Var(), 0.0); }

inline Var operator+(const Var& a, const Var& b) { return node(a.v + b.v, a, 1.0, b, 1.0); }
inline Var operator-(const Var& a, const Var& b) { return node(a.v - b.v, a, 1.0, b, -1.0); }
inline Var operator*(const Var& a, const Var& b) { return node(a.v * b.v, a, b.v, b, a.v); }
inline Var operator/(const Var& a, const Var& b) { return node(a.v / b.v, a, 1.0 / b.v, b, -a.v / (b.v * b.v)); }
inline Var operator-(const Var& a) { return node(-a.v, a, -1.0); }
inline Var& operator+=(Var& a, const Var& b) { return a = a + b; }
inline Var& operator-=(Var& a, const Var& b) { return a = a - b; }
inline Var& operator*=(Var& a, const Var& b) { return a = a * b; }
inline bool operator<(const Var& a, const Var& b) { return a.v < b.v; }
inline bool operator>(const Var& a, const Var& b) { return a.v > b.v; }
inline bool operator<=(const Var& a, const Var& b) { return a.v <= b.v; }
inline bool operator>=(const Var& a, const Var& b) { return a.v >= b.v; }
inline bool operator==(const Var& a, const Var& b) { return a.v == b.v; }
inline bool operator!=(const Var& a, const Var& b) { return a.v != b.v; }

// Reverse sweep over the current tape.  `adj` holds one adjoint per tape node
// (seeded by the caller); leaf contributions are added to grad[k].
inline void backward(std::vector<double>& adj, double* grad) {
    auto& t = tape();
    for (int64_t k = static_cast<int64_t>(t.size()) - 1; k >= 0; --k) {
        const double g = adj[k];
        if (g == 0.0) continue;
        const Node& n = t[k];
        if (n.a >= 0) adj[n.a] += g * n.da;
        else if (n.a <= -2) grad[-2 - n.a] += g * n.da;
        if (n.b >= 0) adj[n.b] += g * n.db;
        else if (n.b <= -2) grad[-2 - n.b] += g * n.db;
    }
}

// Adds weight * d(out)/d(inputs): seeds `out` (a node, a leaf or a constant).
inline void seed(std::vector<double>& adj, double* grad, const Var& out, double weight) {
    if (out.i >= 0) adj[out.i] += weight;
    else if (out.i <= -2) grad[-2 - out.i] += weight;
}

}  // namespace ad
}  // namespace vcto

namespace std {
inline vcto::ad::Var floor(const vcto::ad::Var& x) { return vcto::ad::Var(std::floor(x.v)); }
inline vcto::ad::Var ceil(const vcto::ad::Var& x) { return vcto::ad::Var(std::ceil(x.v)); }
inline vcto::ad::Var trunc(const vcto::ad::Var& x) { return vcto::ad::Var(std::trunc(x.v)); }
inline vcto::ad::Var exp2(const vcto::ad::Var& x) {
    const double v = std::exp2(x.v);
    return vcto::ad::node(v, x, v * 0.69314718055994530942);
}
inline vcto::ad::Var log2(const vcto::ad::Var& x) {
    return vcto::ad::node(std::log2(x.v), x, 1.0 / (x.v * 0.69314718055994530942));
}
inline vcto::ad::Var tan(const vcto::ad::Var& x) {
    const double c = std::cos(x.v);
    return vcto::ad::node(std::tan(x.v), x, 1.0 / (c * c));
}
inline vcto::ad::Var sqrt(const vcto::ad::Var& x) {
    const double v = std::sqrt(x.v);
    return vcto::ad::node(v, x, 0.5 / v);
}
inline vcto::ad::Var fabs(const vcto::ad::Var& x) { return vcto::ad::node(std::fabs(x.v), x, x.v < 0.0 ? -1.0 : 1.0); }
inline vcto::ad::Var pow(const vcto::ad::Var& a, const vcto::ad::Var& b) {
    const double v = std::pow(a.v, b.v);
    const double da = b.v == 0.0 ? 0.0 : b.v * std::pow(a.v, b.v - 1.0);
    const double db = a.v > 0.0 ? v * std::log(a.v) : 0.0;
    return vcto::ad::node(v, a, da, b, db);
}
}  // namespace std
