// XPBD oracle: a CPU restatement of the reference's XPBD substep loop.
//
// TEST INFRASTRUCTURE ONLY. Nothing in the shipped library links, calls or
// executes this file; tests, the smoke check and the benchmark's CPU-baseline
// leg use it as the checker.
//
// PARITY STATUS: the physics is "parity unpinned". The reference ships no
// golden vectors, known-answer tests or stored outputs for the solver, and
// its own build needs Eigen/yaml-cpp/gmsh, which are absent, so it cannot be
// run here. The grid-mesh generator IS pinned: its output is compared with
// the reference's cube{2,4,8,16}.msh files, which the reference's own
// MeshUtils::createBeamMsh wrote. The physics is checked by known-answer
// tests derived from the formulas (rest stability, free fall, Lame
// parameters, finite-difference gradients).
//
// Every function cites the reference file:line it restates. Real is the
// template parameter: double reproduces the reference's CPU build
// (include/common/types.hpp:6-11, Real = double without HAVE_CUDA), float
// gives a same-precision oracle for the GPU kernels.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

namespace xo {

// ---------------------------------------------------------------------------
// Grid mesh: restates MeshUtils::createBeamMsh (src/utils/MeshUtils.cpp:424-660)
// with the hex counts given directly. Axis mapping follows the reference:
// width index wi -> x, length index li -> y, height index hi -> z, and vertex
// index hi + wi*(h+1) + li*(w+1)*(h+1) (MeshUtils.cpp:432-435).
// ---------------------------------------------------------------------------
struct GridDims {
    int w, l, h;  // hexes along x, y, z
    long long V() const { return (long long)(w + 1) * (l + 1) * (h + 1); }
    long long T() const { return 5LL * w * l * h; }
    long long F() const { return 4LL * w * h + 4LL * l * h + 4LL * l * w; }
};

// split = 0: the alternating 5-tet split and face diagonals of the current
// createBeamMsh source (conforming across hexes). split = 1: the revision of
// the generator that wrote the reference's resource/cube/cube2.msh and
// cube4.msh fixtures: every hex takes the first 5-tet pattern and each
// boundary quad takes its second triangulation exactly when its two in-plane
// hex indices have equal parity (inferred from those files).
inline void grid_mesh(const GridDims& d, double ex, double ey, double ez,
                      double* X, int* tets, int* faces, int split = 0) {
    const int w = d.w, l = d.l, h = d.h;
    const bool legacy = split == 1;
    auto index = [w, h](int li, int wi, int hi) { return hi + wi * (h + 1) + li * (w + 1) * (h + 1); };
    // vertices (MeshUtils.cpp:437-449)
    for (int li = 0; li < l + 1; li++)
        for (int wi = 0; wi < w + 1; wi++)
            for (int hi = 0; hi < h + 1; hi++) {
                long long i = index(li, wi, hi);
                X[3 * i + 0] = wi * ex;
                X[3 * i + 1] = li * ey;
                X[3 * i + 2] = hi * ez;
            }
    long long fi = 0;
    auto put3 = [&](int a, int b, int c) {
        faces[3 * fi + 0] = a; faces[3 * fi + 1] = b; faces[3 * fi + 2] = c; fi++;
    };
    // front/back faces, w*h (MeshUtils.cpp:451-500)
    for (int wi = 0; wi < w; wi++)
        for (int hi = 0; hi < h; hi++) {
            int f1 = index(0, wi, hi), f2 = index(0, wi + 1, hi), f3 = index(0, wi + 1, hi + 1), f4 = index(0, wi, hi + 1);
            int a = legacy ? (wi % 2 != hi % 2) : (wi % 2 == hi % 2);
            if (!a) { put3(f1, f2, f4); put3(f2, f3, f4); }
            else    { put3(f1, f2, f3); put3(f1, f3, f4); }
            int b1 = index(l, wi, hi), b2 = index(l, wi + 1, hi), b3 = index(l, wi + 1, hi + 1), b4 = index(l, wi, hi + 1);
            a = legacy ? (wi % 2 != hi % 2) : (wi % 2 == hi % 2) - l % 2;
            if (!a) { put3(b1, b4, b2); put3(b2, b4, b3); }
            else    { put3(b1, b3, b2); put3(b1, b4, b3); }
        }
    // right/left faces, l*h (MeshUtils.cpp:502-550)
    for (int hi = 0; hi < h; hi++)
        for (int li = 0; li < l; li++) {
            int r1 = index(li, w, hi), r2 = index(li + 1, w, hi), r3 = index(li + 1, w, hi + 1), r4 = index(li, w, hi + 1);
            int a = legacy ? (hi % 2 != li % 2) : (hi % 2 == li % 2) - w % 2;
            if (a) { put3(r1, r2, r3); put3(r1, r3, r4); }
            else   { put3(r1, r2, r4); put3(r2, r3, r4); }
            int l1 = index(li, 0, hi), l2 = index(li + 1, 0, hi), l3 = index(li + 1, 0, hi + 1), l4 = index(li, 0, hi + 1);
            a = legacy ? (hi % 2 != li % 2) : (hi % 2 == li % 2);
            if (!a) { put3(l1, l4, l2); put3(l2, l4, l3); }
            else    { put3(l1, l3, l2); put3(l1, l4, l3); }
        }
    // top/bottom faces, l*w (MeshUtils.cpp:552-600)
    for (int li = 0; li < l; li++)
        for (int wi = 0; wi < w; wi++) {
            int t1 = index(li, wi, h), t2 = index(li, wi + 1, h), t3 = index(li + 1, wi + 1, h), t4 = index(li + 1, wi, h);
            int a = legacy ? (li % 2 != wi % 2) : (li % 2 == wi % 2) - h % 2;
            if (a) { put3(t1, t2, t3); put3(t1, t3, t4); }
            else   { put3(t1, t2, t4); put3(t2, t3, t4); }
            int b1 = index(li, wi, 0), b2 = index(li, wi + 1, 0), b3 = index(li + 1, wi + 1, 0), b4 = index(li + 1, wi, 0);
            a = legacy ? (li % 2 != wi % 2) : (li % 2 == wi % 2);
            if (a) { put3(b1, b3, b2); put3(b1, b4, b3); }
            else   { put3(b1, b4, b2); put3(b2, b4, b3); }
        }
    // tets, 5 per hex; split selector a = (hi%2==wi%2) - li%2, where -1 is
    // truthy (MeshUtils.cpp:602-660)
    long long ti = 0;
    auto put4 = [&](int a, int b, int c, int e) {
        tets[4 * ti + 0] = a; tets[4 * ti + 1] = b; tets[4 * ti + 2] = c; tets[4 * ti + 3] = e; ti++;
    };
    for (int li = 0; li < l; li++)
        for (int wi = 0; wi < w; wi++)
            for (int hi = 0; hi < h; hi++) {
                int a = legacy ? 1 : (hi % 2 == wi % 2) - li % 2;
                int i1 = index(li, wi, hi), i2 = index(li, wi + 1, hi), i3 = index(li + 1, wi + 1, hi), i4 = index(li + 1, wi, hi);
                int i5 = index(li, wi, hi + 1), i6 = index(li, wi + 1, hi + 1), i7 = index(li + 1, wi + 1, hi + 1), i8 = index(li + 1, wi, hi + 1);
                if (a) {
                    put4(i1, i2, i3, i6); put4(i1, i3, i4, i8); put4(i1, i6, i5, i8); put4(i3, i6, i7, i8); put4(i1, i3, i6, i8);
                } else {
                    put4(i1, i4, i2, i5); put4(i2, i4, i3, i7); put4(i2, i6, i5, i7); put4(i4, i5, i8, i7); put4(i2, i4, i5, i7);
                }
            }
}

// ---------------------------------------------------------------------------
// Small 3x3 helpers (column-major, as Eigen's default Mat3r).
// ---------------------------------------------------------------------------
template <typename R>
inline R det3(const R* m) {
    // m(r,c) = m[c*3+r]; cofactor expansion down column 0
    auto M = [m](int r, int c) { return m[c * 3 + r]; };
    return M(0, 0) * (M(1, 1) * M(2, 2) - M(2, 1) * M(1, 2)) - M(1, 0) * (M(0, 1) * M(2, 2) - M(2, 1) * M(0, 2)) +
           M(2, 0) * (M(0, 1) * M(1, 2) - M(1, 1) * M(0, 2));
}

template <typename R>
inline void inv3(const R* m, R* out) {
    auto M = [m](int r, int c) { return m[c * 3 + r]; };
    R c00 = M(1, 1) * M(2, 2) - M(1, 2) * M(2, 1);
    R c10 = M(1, 2) * M(2, 0) - M(1, 0) * M(2, 2);
    R c20 = M(1, 0) * M(2, 1) - M(1, 1) * M(2, 0);
    R det = M(0, 0) * c00 + M(0, 1) * c10 + M(0, 2) * c20;
    R inv = R(1) / det;
    // out(r,c) = cofactor(c,r)/det
    out[0 * 3 + 0] = c00 * inv;
    out[0 * 3 + 1] = c10 * inv;
    out[0 * 3 + 2] = c20 * inv;
    out[1 * 3 + 0] = (M(0, 2) * M(2, 1) - M(0, 1) * M(2, 2)) * inv;
    out[1 * 3 + 1] = (M(0, 0) * M(2, 2) - M(0, 2) * M(2, 0)) * inv;
    out[1 * 3 + 2] = (M(0, 1) * M(2, 0) - M(0, 0) * M(2, 1)) * inv;
    out[2 * 3 + 0] = (M(0, 1) * M(1, 2) - M(0, 2) * M(1, 1)) * inv;
    out[2 * 3 + 1] = (M(0, 2) * M(1, 0) - M(0, 0) * M(1, 2)) * inv;
    out[2 * 3 + 2] = (M(0, 0) * M(1, 1) - M(0, 1) * M(1, 0)) * inv;
}

// ---------------------------------------------------------------------------
// Element constraint pieces.
// ---------------------------------------------------------------------------

// Q = (X0-X3, X1-X3, X2-X3)^-1 and V = |det|/6 at rest
// (include/solver/constraint/ElementConstraint.hpp:23-51).
template <typename R>
inline void rest_shape(const R* X0, const R* X1, const R* X2, const R* X3, R* Q, R* vol) {
    R X[9];
    for (int k = 0; k < 3; k++) { X[k] = X0[k] - X3[k]; X[3 + k] = X1[k] - X3[k]; X[6 + k] = X2[k] - X3[k]; }
    inv3(X, Q);
    *vol = std::abs(det3(X) / R(6));
}

// F = Ds * Q, column-major (ElementConstraint.hpp:78-119)
template <typename R>
inline void compute_F(const R* x0, const R* x1, const R* x2, const R* x3, const R* Q, R* F) {
    R X[9];
    X[0] = x0[0] - x3[0]; X[1] = x0[1] - x3[1]; X[2] = x0[2] - x3[2];
    X[3] = x1[0] - x3[0]; X[4] = x1[1] - x3[1]; X[5] = x1[2] - x3[2];
    X[6] = x2[0] - x3[0]; X[7] = x2[1] - x3[1]; X[8] = x2[2] - x3[2];
    auto q = [Q](int r, int c) { return Q[c * 3 + r]; };
    for (int c = 0; c < 3; c++) {
        F[3 * c + 0] = X[0] * q(0, c) + X[3] * q(1, c) + X[6] * q(2, c);
        F[3 * c + 1] = X[1] * q(0, c) + X[4] * q(1, c) + X[7] * q(2, c);
        F[3 * c + 2] = X[2] * q(0, c) + X[5] * q(1, c) + X[8] * q(2, c);
    }
}

template <typename R>
inline R detF(const R* F) {
    // HydrostaticConstraint.hpp:127 (same term order)
    return F[0] * F[4] * F[8] - F[0] * F[7] * F[5] - F[3] * F[1] * F[8] + F[3] * F[7] * F[2] + F[6] * F[1] * F[5] -
           F[6] * F[4] * F[2];
}

// C_h = -gamma + log J (J >= 1) or its 3-term Taylor series (J < 1)
// (include/solver/constraint/HydrostaticConstraint.hpp:123-153)
template <typename R>
inline R hyd_C(const R* F, R gamma) {
    R J = detF(F);
    if (J >= 1) return -gamma + std::log(J);
    return -gamma + (J - 1) - (J - 1) * (J - 1) / R(2) + (J - 1) * (J - 1) * (J - 1) / R(3);
}

template <typename R>
inline void cross3(const R* a, const R* b, R* c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

// grad C_h = fac * [f1 x f2, f2 x f0, f0 x f1] * Q^T, 4th = -sum
// (HydrostaticConstraint.hpp:158-221)
template <typename R>
inline void hyd_grad(const R* F, const R* Q, R* g) {
    R Fc[9];
    cross3(F + 3, F + 6, Fc);
    cross3(F + 6, F, Fc + 3);
    cross3(F, F + 3, Fc + 6);
    R J = detF(F);
    R fac = (J >= R(1.0)) ? R(1) / J : R(1) - (J - 1) + (J - 1) * (J - 1);
    auto q = [Q](int r, int c) { return Q[c * 3 + r]; };
    for (int i = 0; i < 3; i++)
        for (int k = 0; k < 3; k++) g[3 * i + k] = fac * (Fc[k] * q(i, 0) + Fc[3 + k] * q(i, 1) + Fc[6 + k] * q(i, 2));
    for (int k = 0; k < 3; k++) g[9 + k] = -g[k] - g[3 + k] - g[6 + k];
}

// C_d = ||F||_F (include/solver/constraint/DeviatoricConstraint.hpp:112-116)
template <typename R>
inline R dev_C(const R* F) {
    return std::sqrt(F[0] * F[0] + F[1] * F[1] + F[2] * F[2] + F[3] * F[3] + F[4] * F[4] + F[5] * F[5] + F[6] * F[6] +
                     F[7] * F[7] + F[8] * F[8]);
}

// grad C_d = (1/C) F Q^T, 4th = -sum (DeviatoricConstraint.hpp:121-152)
template <typename R>
inline void dev_grad(const R* F, R C, const R* Q, R* g) {
    R inv_C = R(1.0) / C;
    auto q = [Q](int r, int c) { return Q[c * 3 + r]; };
    for (int i = 0; i < 3; i++)
        for (int k = 0; k < 3; k++) g[3 * i + k] = inv_C * (F[k] * q(i, 0) + F[3 + k] * q(i, 1) + F[6 + k] * q(i, 2));
    for (int k = 0; k < 3; k++) g[9 + k] = -g[k] - g[3 + k] - g[6 + k];
}

// Combined deviatoric+hydrostatic 2x2 projection, 2nd order
// (src/solver/xpbd_projector/CombinedNeohookeanConstraintProjector.cpp:98-179).
// at[0] = alpha_d/dt^2, at[1] = alpha_h/dt^2. Writes 12 position updates.
template <typename R>
inline void project_combined(const R* x0, const R* x1, const R* x2, const R* x3, const R* w, const R* Q,
                             const R* at, R gamma, R* lam, R* dx) {
    R F[9];
    compute_F(x0, x1, x2, x3, Q, F);
    R C[2];
    R g[24];
    C[0] = dev_C(F);
    dev_grad(F, C[0], Q, g);
    C[1] = hyd_C(F, gamma);
    hyd_grad(F, Q, g + 12);
    R L[4];
    L[0] = at[0]; L[1] = 0; L[2] = 0; L[3] = at[1];
    for (int ci = 0; ci < 2; ci++) {
        const R* gi = g + 12 * ci;
        for (int cj = ci; cj < 2; cj++) {
            const R* gj = g + 12 * cj;
            for (int i = 0; i < 4; i++)
                L[cj * 2 + ci] += w[i] * (gi[3 * i] * gj[3 * i] + gi[3 * i + 1] * gj[3 * i + 1] + gi[3 * i + 2] * gj[3 * i + 2]);
            L[ci * 2 + cj] = L[cj * 2 + ci];
        }
    }
    R rhs[2] = {-C[0] - at[0] * lam[0], -C[1] - at[1] * lam[1]};
    const R det = L[0] * L[3] - L[1] * L[2];
    R dl0 = (rhs[0] * L[3] - rhs[1] * L[2]) / det;
    R dl1 = (rhs[1] * L[0] - rhs[0] * L[1]) / det;
    lam[0] += dl0;
    lam[1] += dl1;
    for (int i = 0; i < 4; i++)
        for (int k = 0; k < 3; k++) dx[3 * i + k] = w[i] * (g[3 * i + k] * dl0 + g[12 + 3 * i + k] * dl1);
}

// Scalar XPBD projection of one element constraint (Dev or Hyd) for the
// "Stable-Neohookean" (separate) configuration
// (include/solver/xpbd_projector/ConstraintProjector.hpp:111-172).
template <typename R>
inline void project_single_elem(int which, const R* x0, const R* x1, const R* x2, const R* x3, const R* w, const R* Q,
                                R at, R gamma, R* lam, R* dx) {
    R F[9], g[12], C;
    compute_F(x0, x1, x2, x3, Q, F);
    if (which == 0) { C = dev_C(F); dev_grad(F, C, Q, g); }
    else            { C = hyd_C(F, gamma); hyd_grad(F, Q, g); }
    R L = at;
    for (int i = 0; i < 4; i++) L += w[i] * (g[3 * i] * g[3 * i] + g[3 * i + 1] * g[3 * i + 1] + g[3 * i + 2] * g[3 * i + 2]);
    R rhs = -C - at * (*lam);
    R dl = rhs / L;
    *lam += dl;
    for (int i = 0; i < 4; i++)
        for (int k = 0; k < 3; k++) dx[3 * i + k] = w[i] * g[3 * i + k] * dl;
}

// ---------------------------------------------------------------------------
// Collisions.
// ---------------------------------------------------------------------------
template <typename R>
struct Contact {
    int sphere;    // which sphere produced it
    int face;      // surface face index
    int v[3];      // face vertices
    R u, v_, w;    // barycentrics
    R p[3];        // surface point
    R n[3];        // normal
    R lambda;
    bool dynamic = false;  // against a free rigid body (RigidDeformableCollisionConstraint)
};

// SphereSDF::evaluate / gradient (src/geometry/SphereSDF.cpp:16-26). Eigen's
// normalized() leaves a zero vector unchanged.
template <typename R>
inline R sphere_sdf(const R* x, const R* c, R r) {
    R d0 = x[0] - c[0], d1 = x[1] - c[1], d2 = x[2] - c[2];
    return std::sqrt(d0 * d0 + d1 * d1 + d2 * d2) - r;
}
template <typename R>
inline void sphere_grad(const R* x, const R* c, R* g) {
    R d0 = x[0] - c[0], d1 = x[1] - c[1], d2 = x[2] - c[2];
    R n2 = d0 * d0 + d1 * d1 + d2 * d2;
    if (n2 > R(0)) {
        R n = std::sqrt(n2);
        g[0] = d0 / n; g[1] = d1 / n; g[2] = d2 / n;
    } else {
        g[0] = d0; g[1] = d1; g[2] = d2;
    }
}

// Static SDF primitive of a fixed rigid object: sphere (d = radius),
// box (d = full size), cylinder (d = radius, height), at position p with
// orientation quaternion q = (x, y, z, w) (include/simobject/RigidPrimitives.hpp).
enum { PRIM_SPHERE = 0, PRIM_BOX = 1, PRIM_CYLINDER = 2 };
template <typename R>
struct Prim {
    int kind = PRIM_SPHERE;
    R p[3] = {0, 0, 0};
    R q[4] = {0, 0, 0, 1};
    R d[3] = {0, 0, 0};
};

// GeometryUtils::rotateVectorByQuat / inverseQuat (src/utils/GeometryUtils.cpp:92-102)
template <typename R>
inline void quat_rotate(const R* v, const R* q, R* out) {
    const R ud = q[0] * v[0] + q[1] * v[1] + q[2] * v[2];
    const R s = 2 * q[3] * q[3] - 1;
    const R cx = q[1] * v[2] - q[2] * v[1], cy = q[2] * v[0] - q[0] * v[2], cz = q[0] * v[1] - q[1] * v[0];
    out[0] = 2 * ud * q[0] + s * v[0] + 2 * q[3] * cx;
    out[1] = 2 * ud * q[1] + s * v[1] + 2 * q[3] * cy;
    out[2] = 2 * ud * q[2] + s * v[2] + 2 * q[3] * cz;
}
// RigidObject::globalToBody (src/simobject/RigidObject.cpp:94-97)
template <typename R>
inline void to_body(const Prim<R>& pr, const R* x, R* out) {
    const R n2 = pr.q[0] * pr.q[0] + pr.q[1] * pr.q[1] + pr.q[2] * pr.q[2] + pr.q[3] * pr.q[3];
    const R qi[4] = {-pr.q[0] / n2, -pr.q[1] / n2, -pr.q[2] / n2, pr.q[3] / n2};
    const R v[3] = {x[0] - pr.p[0], x[1] - pr.p[1], x[2] - pr.p[2]};
    quat_rotate(v, qi, out);
}
// Eigen's normalized(): unchanged when the norm is zero
template <typename R>
inline void normalize3(R* v) {
    const R n2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    if (n2 > R(0)) {
        const R n = std::sqrt(n2);
        v[0] /= n; v[1] /= n; v[2] /= n;
    }
}

// BoxSDF::evaluate / CylinderSDF::evaluate (src/geometry/BoxSDF.cpp,
// CylinderSDF.cpp); spheres as sphere_sdf
template <typename R>
inline R prim_sdf(const Prim<R>& pr, const R* x) {
    if (pr.kind == PRIM_SPHERE) return sphere_sdf(x, pr.p, pr.d[0]);
    R b[3];
    to_body(pr, x, b);
    if (pr.kind == PRIM_BOX) {
        R qv[3], o = 0;
        for (int k = 0; k < 3; k++) {
            qv[k] = std::abs(b[k]) - R(0.5) * pr.d[k];
            const R m = std::max(qv[k], R(0));
            o += m * m;
        }
        return std::sqrt(o) + std::min(std::max({qv[0], qv[1], qv[2]}), R(0));
    }
    const R xy = std::sqrt(b[0] * b[0] + b[1] * b[1]) - pr.d[0];
    const R z = std::abs(b[2]) - R(0.5) * pr.d[1];
    const R ox = std::max(xy, R(0)), oz = std::max(z, R(0));
    return std::sqrt(ox * ox + oz * oz) + std::min(std::max(xy, z), R(0));
}

template <typename R>
inline void prim_grad(const Prim<R>& pr, const R* x, R* g) {
    if (pr.kind == PRIM_SPHERE) {
        sphere_grad(x, pr.p, g);
        return;
    }
    R b[3], go[3], gi[3];
    to_body(pr, x, b);
    if (pr.kind == PRIM_BOX) {
        R qv[3];
        for (int k = 0; k < 3; k++) qv[k] = std::abs(b[k]) - pr.d[k] / R(2.0);
        const R md = std::min(std::max({qv[0], qv[1], qv[2]}), R(0));
        for (int k = 0; k < 3; k++) {
            const R sg = b[k] > 0 ? R(1) : R(-1);
            go[k] = sg * std::max(qv[k], R(0));
            gi[k] = sg * (qv[k] == md ? R(1) : R(0));
        }
        normalize3(go);
    } else {
        const R xy = std::sqrt(b[0] * b[0] + b[1] * b[1]) - pr.d[0];
        const R z = std::abs(b[2]) - R(0.5) * pr.d[1];
        const R ox = std::max(xy, R(0)), oz = std::max(z, R(0));
        const R in = std::min(std::max(xy, z), R(0));
        go[0] = b[0] * (ox > 0 ? R(1) : R(0));
        go[1] = b[1] * (ox > 0 ? R(1) : R(0));
        go[2] = b[2] * (oz > 0 ? R(1) : R(0));
        gi[0] = b[0] * (in == xy ? R(1) : R(0));
        gi[1] = b[1] * (in == xy ? R(1) : R(0));
        gi[2] = b[2] * (in == z ? R(1) : R(0));
        normalize3(go);
        normalize3(gi);
    }
    const R sum[3] = {go[0] + gi[0], go[1] + gi[1], go[2] + gi[2]};
    quat_rotate(sum, pr.q, g);
}

// CollisionScene::_frankWolfe (src/collision/CollisionScene.cpp:253-283)
template <typename R>
inline void frank_wolfe(const Prim<R>& pr, const R* p1, const R* p2, const R* p3, R* x) {
    R d1 = prim_sdf(pr, p1), d2 = prim_sdf(pr, p2), d3 = prim_sdf(pr, p3);
    const R* s0 = (d1 <= d2 && d1 <= d3) ? p1 : ((d2 <= d1 && d2 <= d3) ? p2 : p3);
    x[0] = s0[0]; x[1] = s0[1]; x[2] = s0[2];
    for (int i = 0; i < 32; i++) {
        R alpha = R(2.0) / R(i + 3);
        R g[3];
        prim_grad(pr, x, g);
        R sg1 = p1[0] * g[0] + p1[1] * g[1] + p1[2] * g[2];
        R sg2 = p2[0] * g[0] + p2[1] * g[1] + p2[2] * g[2];
        R sg3 = p3[0] * g[0] + p3[1] * g[1] + p3[2] * g[2];
        const R* s = (sg1 < sg2 && sg1 < sg3) ? p1 : ((sg2 < sg1 && sg2 < sg3) ? p2 : p3);
        for (int k = 0; k < 3; k++) x[k] = x[k] + alpha * (s[k] - x[k]);
    }
}

// GeometryUtils::barycentricCoords (src/utils/GeometryUtils.cpp:6-23)
template <typename R>
inline void barycentric(const R* p, const R* a, const R* b, const R* c, R* u, R* v, R* w) {
    R v0[3], v1[3], v2[3];
    for (int k = 0; k < 3; k++) { v0[k] = b[k] - a[k]; v1[k] = c[k] - a[k]; v2[k] = p[k] - a[k]; }
    auto dot = [](const R* x, const R* y) { return x[0] * y[0] + x[1] * y[1] + x[2] * y[2]; };
    R d00 = dot(v0, v0), d01 = dot(v0, v1), d11 = dot(v1, v1), d20 = dot(v2, v0), d21 = dot(v2, v1);
    R denom = d00 * d11 - d01 * d01;
    *v = (d11 * d20 - d01 * d21) / denom;
    *w = (d00 * d21 - d01 * d20) / denom;
    *u = 1 - *v - *w;
}

// One face against one SDF primitive: centroid cull, Frank-Wolfe, threshold,
// barycentrics, surface point (CollisionScene.cpp:171-214). Returns true and
// fills the contact when the face is in contact.
template <typename R>
inline bool collide_face(const R* p1, const R* p2, const R* p3, const Prim<R>& pr, Contact<R>* out) {
    auto sq = [](const R* a, const R* b) {
        R d0 = b[0] - a[0], d1 = b[1] - a[1], d2 = b[2] - a[2];
        return d0 * d0 + d1 * d1 + d2 * d2;
    };
    R e12 = sq(p1, p2), e13 = sq(p1, p3), e23 = sq(p2, p3);
    R max_edge = std::max({e12, e13, e23});
    R cen[3];
    for (int k = 0; k < 3; k++) cen[k] = (p1[k] + p2[k] + p3[k]) / R(3);
    R cd = prim_sdf(pr, cen);
    if (cd * cd > max_edge) return false;
    R x[3];
    frank_wolfe(pr, p1, p2, p3, x);
    const double distance = (double)prim_sdf(pr, x);
    if (!(distance <= 1e-4)) return false;
    barycentric(x, p1, p2, p3, &out->u, &out->v_, &out->w);
    R g[3];
    prim_grad(pr, x, g);
    for (int k = 0; k < 3; k++) {
        out->p[k] = (R)(x[k] - g[k] * distance);
        out->n[k] = g[k];
    }
    out->lambda = 0;
    return true;
}

// Static deformable collision projection: C = n.(u x1 + v x2 + w x3 - p),
// inequality skip when C > 0, alpha = 0
// (src/solver/constraint/StaticDeformableCollisionConstraint.cpp:20-49;
//  include/solver/xpbd_projector/ConstraintProjector.hpp:111-172).
// Returns false when skipped.
template <typename R>
inline bool project_contact(const R* x1, const R* x2, const R* x3, const R* wv, Contact<R>& ct, R* dx) {
    R a[3];
    for (int k = 0; k < 3; k++) a[k] = ct.u * x1[k] + ct.v_ * x2[k] + ct.w * x3[k];
    R C = ct.n[0] * (a[0] - ct.p[0]) + ct.n[1] * (a[1] - ct.p[1]) + ct.n[2] * (a[2] - ct.p[2]);
    if (C > 0) return false;
    R g[9];
    R b[3] = {ct.u, ct.v_, ct.w};
    for (int i = 0; i < 3; i++)
        for (int k = 0; k < 3; k++) g[3 * i + k] = b[i] * ct.n[k];
    R L = 0;  // alpha_tilde = 0 for collision constraints
    for (int i = 0; i < 3; i++) L += wv[i] * (g[3 * i] * g[3 * i] + g[3 * i + 1] * g[3 * i + 1] + g[3 * i + 2] * g[3 * i + 2]);
    R rhs = -C - R(0) * ct.lambda;
    R dl = rhs / L;
    ct.lambda += dl;
    for (int i = 0; i < 3; i++)
        for (int k = 0; k < 3; k++) dx[3 * i + k] = wv[i] * g[3 * i + k] * dl;
    return true;
}

// ---------------------------------------------------------------------------
// Free rigid bodies (RigidObject with fixed: false) and two-way coupling.
// The rigid state is double, as the reference's Real, for either precision
// of the deformable object.
// ---------------------------------------------------------------------------
// GeometryUtils::quatMult (src/utils/GeometryUtils.cpp:81-90), (x, y, z, w)
inline void quat_mult(const double* a, const double* b, double* r) {
    r[0] = a[3] * b[0] + a[0] * b[3] + a[1] * b[2] - a[2] * b[1];
    r[1] = a[3] * b[1] + a[1] * b[3] + a[2] * b[0] - a[0] * b[2];
    r[2] = a[3] * b[2] + a[2] * b[3] + a[0] * b[1] - a[1] * b[0];
    r[3] = a[3] * b[3] - a[0] * b[0] - a[1] * b[1] - a[2] * b[2];
}
// GeometryUtils::inverseQuat (src/utils/GeometryUtils.cpp:99-102)
inline void quat_inverse(const double* q, double* r) {
    const double n2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
    r[0] = -q[0] / n2; r[1] = -q[1] / n2; r[2] = -q[2] / n2; r[3] = q[3] / n2;
}
inline void cross3(const double* a, const double* b, double* r) {
    r[0] = a[1] * b[2] - a[2] * b[1];
    r[1] = a[2] * b[0] - a[0] * b[2];
    r[2] = a[0] * b[1] - a[1] * b[0];
}

// RigidObject (src/simobject/RigidObject.cpp) with a diagonal inertia (the
// primitives' _I, src/simobject/RigidPrimitives.cpp).
struct RigidBody {
    int kind = PRIM_SPHERE;
    double d[3] = {0, 0, 0};
    double p[3] = {0, 0, 0}, q[4] = {0, 0, 0, 1}, v[3] = {0, 0, 0}, w[3] = {0, 0, 0};
    double p_prev[3] = {0, 0, 0}, q_prev[4] = {0, 0, 0, 1};
    double m = 1, I[3] = {1, 1, 1}, I_inv[3] = {1, 1, 1};

    Prim<double> prim() const {
        Prim<double> pr;
        pr.kind = kind;
        for (int k = 0; k < 3; k++) { pr.p[k] = p[k]; pr.d[k] = d[k]; }
        for (int k = 0; k < 4; k++) pr.q[k] = q[k];
        return pr;
    }

    // RigidObject::update (RigidObject.cpp:41-60): gravity on v and p, the
    // body-frame Euler step of w (no external torque), q += dt/2 [w,0] q, normalised
    void update(double dt, double g) {
        const double f[3] = {0.0, 0.0, -m * g};
        for (int k = 0; k < 3; k++) v[k] = v[k] + dt * f[k] / m;
        for (int k = 0; k < 3; k++) p[k] = p[k] + dt * v[k];
        double qi[4], wb[3], Iw[3], c[3];
        quat_inverse(q, qi);
        quat_rotate(w, qi, wb);
        for (int k = 0; k < 3; k++) Iw[k] = I[k] * wb[k];
        cross3(wb, Iw, c);
        for (int k = 0; k < 3; k++) wb[k] = wb[k] + dt * I_inv[k] * (0.0 - c[k]);
        quat_rotate(wb, q, w);
        const double w4[4] = {w[0], w[1], w[2], 0.0};
        double dq[4];
        quat_mult(w4, q, dq);
        for (int k = 0; k < 4; k++) q[k] = q[k] + 0.5 * dt * dq[k];
        const double n = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
        for (int k = 0; k < 4; k++) q[k] /= n;
    }

    // RigidObject::velocityUpdate (RigidObject.cpp:62-77)
    void velocity_update(double dt) {
        for (int k = 0; k < 3; k++) v[k] = (p[k] - p_prev[k]) / dt;
        double qi[4], dq[4];
        quat_inverse(q_prev, qi);
        quat_mult(q, qi, dq);
        for (int k = 0; k < 3; k++) w[k] = 2 / dt * dq[k];
        if (dq[3] < 0)
            for (int k = 0; k < 3; k++) w[k] = -w[k];
        for (int k = 0; k < 3; k++) p_prev[k] = p[k];
        for (int k = 0; k < 4; k++) q_prev[k] = q[k];
    }

    // PositionalRigidBodyXPBDHelper::update (RigidBodyConstraint.hpp) for a
    // contact at global point pt with direction -n: position and orientation
    // increments from the body's current pose
    void contact_delta(double dlam, const double* pt, const double* n, double* dp, double* dq) const {
        const double dir[3] = {-n[0], -n[1], -n[2]};
        double qi[4], rb[3], nb[3], t[3], c[3], wb[3], ws[3];
        quat_inverse(q, qi);
        const double rel[3] = {pt[0] - p[0], pt[1] - p[1], pt[2] - p[2]};
        quat_rotate(rel, qi, rb);
        quat_rotate(dir, qi, nb);
        for (int k = 0; k < 3; k++) dp[k] = dlam * dir[k] / m;
        for (int k = 0; k < 3; k++) t[k] = dlam * nb[k];
        cross3(rb, t, c);
        for (int k = 0; k < 3; k++) wb[k] = 0.5 * I_inv[k] * c[k];
        quat_rotate(wb, q, ws);
        const double w4[4] = {ws[0], ws[1], ws[2], 0.0};
        quat_mult(w4, q, dq);
    }
};

// RigidDeformableCollisionConstraint (RigidDeformableCollisionConstraint.cpp:23-55)
// projected by RigidBodyConstraintProjector::project
// (RigidBodyConstraintProjector.hpp:97-158): C = the body's SDF at the
// contact's barycentric point (current pose), gradient (u n, v n, w n),
// inequality skip when C > 0, alpha = 0; the multiplier update uses only the
// deformable weights. Deformable arithmetic in double; dx receives the 9
// vertex updates. Returns false when skipped.
template <typename R>
inline bool project_rigid_contact(const R* x1, const R* x2, const R* x3, const R* wv, Contact<R>& ct,
                                  const RigidBody& rb, double* dx, double* dlam_out) {
    const double b[3] = {(double)ct.u, (double)ct.v_, (double)ct.w};
    double a[3];
    for (int k = 0; k < 3; k++) a[k] = b[0] * (double)x1[k] + b[1] * (double)x2[k] + b[2] * (double)x3[k];
    const double C = prim_sdf(rb.prim(), a);
    if (C > 0) return false;
    const double n[3] = {(double)ct.n[0], (double)ct.n[1], (double)ct.n[2]};
    double L = 0;
    for (int i = 0; i < 3; i++) {
        const double gx = b[i] * n[0], gy = b[i] * n[1], gz = b[i] * n[2];
        L += (double)wv[i] * (gx * gx + gy * gy + gz * gz);
    }
    const double dl = -C / L;
    ct.lambda = (R)((double)ct.lambda + dl);
    for (int i = 0; i < 3; i++)
        for (int k = 0; k < 3; k++) dx[3 * i + k] = (double)wv[i] * (b[i] * n[k]) * dl;
    *dlam_out = dl;
    return true;
}

// ---------------------------------------------------------------------------
// Self-collisions: XPBDMeshObject_::selfCollisionCheck (XPBDMeshObject.cpp:719-762)
// with Embree's queries restated, and DeformableDeformableCollisionConstraint.
// ---------------------------------------------------------------------------
// EmbreeTetMeshGeometry::isPointInTetrahedron (EmbreeTetMeshGeometry.cpp:20-47):
// p is inside when it lies on the same side of each face as the opposite
// vertex (or on the face), all in float
inline bool same_side_f(const float* p, const float* a, const float* b, const float* c, const float* d) {
    const float ab0 = b[0] - a[0], ab1 = b[1] - a[1], ab2 = b[2] - a[2];
    const float ac0 = c[0] - a[0], ac1 = c[1] - a[1], ac2 = c[2] - a[2];
    const float n0 = ab1 * ac2 - ab2 * ac1, n1 = ab2 * ac0 - ab0 * ac2, n2 = ab0 * ac1 - ab1 * ac0;
    const float sp = n0 * (p[0] - a[0]) + n1 * (p[1] - a[1]) + n2 * (p[2] - a[2]);
    const float sd = n0 * (d[0] - a[0]) + n1 * (d[1] - a[1]) + n2 * (d[2] - a[2]);
    return sp * sd >= 0;
}
inline bool point_in_tet_f(const float* p, const float* v0, const float* v1, const float* v2, const float* v3) {
    return same_side_f(p, v0, v1, v2, v3) && same_side_f(p, v0, v1, v3, v2) && same_side_f(p, v0, v2, v3, v1) &&
           same_side_f(p, v1, v2, v3, v0);
}

// Distance from p to the triangle (a, b, c), in float: the closest point by
// the Voronoi-region walk of Ericson, Real-Time Collision Detection, 5.1.5
// (the method of EmbreeMeshGeometry::_closestPointTriangle)
inline float point_triangle_distance_f(const float* p, const float* a, const float* b, const float* c) {
    auto dot = [](const float* u, const float* v) { return u[0] * v[0] + u[1] * v[1] + u[2] * v[2]; };
    const float ab[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
    const float ac[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
    const float ap[3] = {p[0] - a[0], p[1] - a[1], p[2] - a[2]};
    float o[3];
    const float d1 = dot(ab, ap), d2 = dot(ac, ap);
    const float bp[3] = {p[0] - b[0], p[1] - b[1], p[2] - b[2]};
    const float d3 = dot(ab, bp), d4 = dot(ac, bp);
    const float cp[3] = {p[0] - c[0], p[1] - c[1], p[2] - c[2]};
    const float d5 = dot(ab, cp), d6 = dot(ac, cp);
    if (d1 <= 0.f && d2 <= 0.f) {
        o[0] = a[0]; o[1] = a[1]; o[2] = a[2];
    } else if (d3 >= 0.f && d4 <= d3) {
        o[0] = b[0]; o[1] = b[1]; o[2] = b[2];
    } else if (d6 >= 0.f && d5 <= d6) {
        o[0] = c[0]; o[1] = c[1]; o[2] = c[2];
    } else {
        const float vc = d1 * d4 - d3 * d2, vb = d5 * d2 - d1 * d6, va = d3 * d6 - d5 * d4;
        if (vc <= 0.f && d1 >= 0.f && d3 <= 0.f) {
            const float v = d1 / (d1 - d3);
            for (int k = 0; k < 3; k++) o[k] = a[k] + v * ab[k];
        } else if (vb <= 0.f && d2 >= 0.f && d6 <= 0.f) {
            const float v = d2 / (d2 - d6);
            for (int k = 0; k < 3; k++) o[k] = a[k] + v * ac[k];
        } else if (va <= 0.f && (d4 - d3) >= 0.f && (d5 - d6) >= 0.f) {
            const float v = (d4 - d3) / ((d4 - d3) + (d5 - d6));
            for (int k = 0; k < 3; k++) o[k] = b[k] + v * (c[k] - b[k]);
        } else {
            const float den = 1.f / (va + vb + vc);
            const float v = vb * den, w = vc * den;
            for (int k = 0; k < 3; k++) o[k] = a[k] + v * ab[k] + w * ac[k];
        }
    }
    const float e0 = p[0] - o[0], e1 = p[1] - o[1], e2 = p[2] - o[2];
    return std::sqrt(e0 * e0 + e1 * e1 + e2 * e2);
}

// DeformableDeformableCollisionConstraint (DeformableDeformableCollisionConstraint.cpp):
// q against the face plane through p1, p2, p3, C = (q - p1).a/|a| + 1e-5 with
// a = (p2 - p1) x (p3 - p1), and its gradient as the reference writes it
// (the third face vertex's term uses q - p2); g = (q, p1, p2, p3) x 3
template <typename R>
inline R self_contact_eval(const R* q, const R* p1, const R* p2, const R* p3, R* g) {
    const R e1[3] = {p2[0] - p1[0], p2[1] - p1[1], p2[2] - p1[2]};
    const R e2[3] = {p3[0] - p1[0], p3[1] - p1[1], p3[2] - p1[2]};
    const R a[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
    const R an = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    const R u1[3] = {q[0] - p1[0], q[1] - p1[1], q[2] - p1[2]};
    const R u2[3] = {q[0] - p2[0], q[1] - p2[1], q[2] - p2[2]};
    const R C = (u1[0] * a[0] + u1[1] * a[1] + u1[2] * a[2]) / an + R(1e-5);
    // M = I/|a| - a a^T/|a|^3 (symmetric); u^T M [v]x = (M u) x v
    const R an3 = an * an * an;
    auto Mu = [&](const R* u, R* r) {
        const R ad = a[0] * u[0] + a[1] * u[1] + a[2] * u[2];
        for (int k = 0; k < 3; k++) r[k] = u[k] / an - a[k] * ad / an3;
    };
    auto cross = [](const R* x, const R* y, R* r) {
        r[0] = x[1] * y[2] - x[2] * y[1];
        r[1] = x[2] * y[0] - x[0] * y[2];
        r[2] = x[0] * y[1] - x[1] * y[0];
    };
    R r1[3], r2[3], t[3];
    Mu(u1, r1);
    Mu(u2, r2);
    for (int k = 0; k < 3; k++) g[k] = a[k] / an;
    const R d32[3] = {p3[0] - p2[0], p3[1] - p2[1], p3[2] - p2[2]};
    cross(r1, d32, t);
    for (int k = 0; k < 3; k++) g[3 + k] = -a[k] / an + t[k];
    const R d13[3] = {p1[0] - p3[0], p1[1] - p3[1], p1[2] - p3[2]};
    cross(r1, d13, t);
    for (int k = 0; k < 3; k++) g[6 + k] = t[k];
    const R d21[3] = {p2[0] - p1[0], p2[1] - p1[1], p2[2] - p1[2]};
    cross(r2, d21, t);
    for (int k = 0; k < 3; k++) g[9 + k] = t[k];
    return C;
}

// ---------------------------------------------------------------------------
// Greedy tet colouring used by the coloured Gauss-Seidel order. Tets are
// visited in index order; each takes the smallest colour not used by any tet
// already coloured that shares a vertex. Surface faces use the same rule.
// This is this project's own ordering (the reference's Gauss-Seidel order is
// plain projector index order, include/common/VariadicVectorContainer.hpp:83-223).
// ---------------------------------------------------------------------------
inline int greedy_colour(long long n_items, int arity, const int* items, long long n_vertices, int* colour_out) {
    std::vector<std::vector<uint64_t>> used(1, std::vector<uint64_t>((size_t)n_vertices, 0));
    int ncol = 0;
    for (long long t = 0; t < n_items; t++) {
        const int* it = items + arity * t;
        int c = -1;
        for (size_t word = 0; c < 0; word++) {
            if (word == used.size()) used.emplace_back((size_t)n_vertices, 0);
            uint64_t m = 0;
            for (int k = 0; k < arity; k++) m |= used[word][(size_t)it[k]];
            if (~m) c = (int)(64 * word + __builtin_ctzll(~m));
        }
        colour_out[t] = c;
        for (int k = 0; k < arity; k++) used[(size_t)c / 64][(size_t)it[k]] |= (1ULL << (c % 64));
        ncol = std::max(ncol, c + 1);
    }
    return ncol;
}

// ---------------------------------------------------------------------------
// The simulated object: XPBDMeshObject_ with a combined (or separate)
// Stable-Neo-Hookean constraint set, 2nd order.
// ---------------------------------------------------------------------------
enum SolverKind { GAUSS_SEIDEL = 0, JACOBI = 1, COLOURED_GS = 2 };
enum ConstraintKind { COMBINED = 0, SEPARATE = 1 };

template <typename R>
struct Object {
    long long V = 0, T = 0, F = 0;
    std::vector<R> x, prev, vel;     // 3V each
    std::vector<R> mass, inv_mass;   // V
    std::vector<uint8_t> fixed;      // V
    std::vector<int> tets, faces;    // 4T, 3F
    std::vector<R> Q, vol, alpha_d, alpha_h, gamma;  // 9T, T, T, T, T
    std::vector<R> lam;              // 2T: [2t]=dev, [2t+1]=hyd
    std::vector<Contact<R>> contacts;
    // attachment constraints: vertex, target (attach point + offset), lambda
    struct Attachment {
        int v;
        R t[3];
        R lambda;
    };
    std::vector<Attachment> attachments;
    // AttachmentConstraint::evaluateWithGradient (AttachmentConstraint.hpp:70-90)
    // projected by ConstraintProjector::project with alpha = 0
    // (ConstraintProjector.hpp:111-172); dx receives the vertex's 3 updates
    bool project_attachment(Attachment& at, R* dx) const {
        const R* xv = &x[3 * at.v];
        R a = xv[0] - at.t[0], b = xv[1] - at.t[1], c = xv[2] - at.t[2];
        R dist = std::sqrt(a * a + b * b + c * c);
        R g[3];
        if (dist < R(1e-12)) {
            g[0] = g[1] = g[2] = R(1e-12);
        } else {
            g[0] = a / dist; g[1] = b / dist; g[2] = c / dist;
        }
        const R w = inv_mass[at.v];
        const R L = w * (g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
        const R dl = -dist / L;
        at.lambda += dl;
        for (int k = 0; k < 3; k++) dx[k] = w * g[k] * dl;
        return true;
    }
    R dt = R(1e-3), g = R(9.81);
    double dt_host = 1e-3;           // the host loop's time step, always double
    int num_iter = 1;
    int solver = GAUSS_SEIDEL;
    int ckind = COMBINED;
    // coloured Gauss-Seidel order
    std::vector<int> tet_order;      // tets in colour order
    std::vector<int> face_colour;    // F
    int n_face_colours = 0;
    // local collision iterations (num-local-collision-iters) and, for
    // COLOURED_GS, the order of their tet passes
    int num_local_iter = 0;
    std::vector<int> local_order;
    // spheres
    std::vector<Prim<R>> prims;   // SDF primitives (fixed rigid bodies, and free ones' current poses)
    std::vector<int> prim_body;   // per primitive: index into bodies, -1 when fixed
    std::vector<RigidBody> bodies;
    // self-collisions (self-collisions: true): surface vertex against surface face
    bool self_collisions = false;
    std::vector<double> X0;        // rest positions, double (DeformableMeshSDF::_initial_vertices)
    std::vector<double> Q64;       // Dm^-1 per tet in double (TetMesh::_element_inv_undeformed_basis)
    std::vector<int> surface_verts;  // vertices of the surface faces, ascending
    struct SelfContact {
        int v, f;
        R lambda;
    };
    std::vector<SelfContact> self_contacts;
    // DeformableDeformableCollisionConstraint's compliance (its Constraint(..., 1e-8))
    static constexpr double kSelfAlpha = 1e-8;
    bool is_dynamic(int s) const { return s < (int)prim_body.size() && prim_body[s] >= 0; }
    // the detection pose of free bodies: their current state in R
    void sync_prims() {
        for (size_t s = 0; s < prim_body.size(); s++)
            if (prim_body[s] >= 0) {
                const RigidBody& b = bodies[prim_body[s]];
                for (int k = 0; k < 3; k++) prims[s].p[k] = (R)b.p[k];
                for (int k = 0; k < 4; k++) prims[s].q[k] = (R)b.q[k];
            }
    }
    void enable_self_collisions() {
        self_collisions = true;
        std::vector<char> on(V, 0);
        for (long long i = 0; i < 3 * F; i++) on[faces[i]] = 1;
        surface_verts.clear();
        for (long long v = 0; v < V; v++)
            if (on[v]) surface_verts.push_back((int)v);
    }

    // selfCollisionCheck (XPBDMeshObject.cpp:719-762): for each surface vertex,
    // the lowest-index tet that holds it without having it as a vertex
    // (EmbreeScene::tetMeshSelfCollisionQuery, a std::set ordered by index, on
    // float copies of the positions); then
    // DeformableMeshSDF::closestSurfaceFaceToPointInTet (DeformableMeshSDF.cpp:68-82):
    // the point mapped back to rest space through that tet, and the surface face
    // closest to it in the rest shape (in float; of equally close faces the
    // lowest index -- Embree's traversal order decides in the reference)
    void detect_self() {
        self_contacts.clear();
        std::vector<float> xf(3 * V), X0f(3 * V);
        for (long long i = 0; i < 3 * V; i++) {
            xf[i] = (float)x[i];
            X0f[i] = (float)X0[i];
        }
        for (int v : surface_verts) {
            int hit = -1;
            for (long long t = 0; t < T && hit < 0; t++) {
                const int* e = &tets[4 * t];
                if (e[0] == v || e[1] == v || e[2] == v || e[3] == v) continue;
                if (point_in_tet_f(&xf[3 * v], &xf[3 * e[0]], &xf[3 * e[1]], &xf[3 * e[2]], &xf[3 * e[3]]))
                    hit = (int)t;
            }
            if (hit < 0) continue;
            const int* e = &tets[4 * hit];
            double xd[5][3];
            const int ids[5] = {e[0], e[1], e[2], e[3], v};
            for (int i = 0; i < 5; i++)
                for (int k = 0; k < 3; k++) xd[i][k] = (double)x[3 * ids[i] + k];
            double Fm[9], Fi[9];
            compute_F(xd[0], xd[1], xd[2], xd[3], &Q64[9 * hit], Fm);
            if (std::abs(det3(Fm)) < 1e-8) continue;
            inv3(Fm, Fi);
            const double rel[3] = {xd[4][0] - xd[3][0], xd[4][1] - xd[3][1], xd[4][2] - xd[3][2]};
            float pm[3];
            for (int r = 0; r < 3; r++)
                pm[r] = (float)(Fi[r] * rel[0] + Fi[3 + r] * rel[1] + Fi[6 + r] * rel[2] + X0[3 * e[3] + r]);
            int best = -1;
            float bd = std::numeric_limits<float>::infinity();
            for (long long f = 0; f < F; f++) {
                const int* fv = &faces[3 * f];
                const float d = point_triangle_distance_f(pm, &X0f[3 * fv[0]], &X0f[3 * fv[1]], &X0f[3 * fv[2]]);
                if (d < bd) {
                    bd = d;
                    best = (int)f;
                }
            }
            if (best >= 0) self_contacts.push_back(SelfContact{v, best, R(0)});
        }
    }

    // ConstraintProjector::project (ConstraintProjector.hpp:111-172) for one
    // self contact: inequality skip when C > 0, alpha = 1e-8; dx gets the 12
    // updates (q, p1, p2, p3). Returns false when skipped.
    bool project_self_i(SelfContact& sc, R* dx) {
        const int* fv = &faces[3 * sc.f];
        const int ids[4] = {sc.v, fv[0], fv[1], fv[2]};
        R g[12];
        const R C = self_contact_eval(&x[3 * ids[0]], &x[3 * ids[1]], &x[3 * ids[2]], &x[3 * ids[3]], g);
        if (C > 0) return false;
        const R at = (R)kSelfAlpha / adt();
        R L = at;
        for (int i = 0; i < 4; i++)
            L += inv_mass[ids[i]] * (g[3 * i] * g[3 * i] + g[3 * i + 1] * g[3 * i + 1] + g[3 * i + 2] * g[3 * i + 2]);
        const R dl = (-C - at * sc.lambda) / L;
        sc.lambda += dl;
        for (int i = 0; i < 4; i++)
            for (int k = 0; k < 3; k++) dx[3 * i + k] = inv_mass[ids[i]] * g[3 * i + k] * dl;
        return true;
    }
    void project_self_contacts(std::vector<R>* acc) {
        R dx[12];
        for (auto& sc : self_contacts) {
            if (!project_self_i(sc, dx)) continue;
            const int* fv = &faces[3 * sc.f];
            const int ids[4] = {sc.v, fv[0], fv[1], fv[2]};
            for (int i = 0; i < 4; i++)
                for (int k = 0; k < 3; k++) {
                    if (acc) (*acc)[3 * ids[i] + k] += dx[3 * i + k];
                    else x[3 * ids[i] + k] += dx[3 * i + k];
                }
        }
    }

    // Rigid contacts, after the static ones (projector type order,
    // include/common/XPBDTypedefs.hpp:55-56), in detection order. Gauss-Seidel
    // applies each update at once; Jacobi reads one state, sums the vertex
    // updates into acc and the body increments, applied after the pass
    // (XPBDGaussSeidelSolver.hpp:61-95, XPBDJacobiSolver.hpp:79-114).
    void project_rigid_contacts(std::vector<R>* acc) {
        std::vector<double> dps(3 * bodies.size(), 0.0), dqs(4 * bodies.size(), 0.0);
        for (auto& ct : contacts) {
            if (!ct.dynamic) continue;
            RigidBody& rb = bodies[prim_body[ct.sphere]];
            R wv[3] = {inv_mass[ct.v[0]], inv_mass[ct.v[1]], inv_mass[ct.v[2]]};
            double dx[9], dl;
            if (!project_rigid_contact(&x[3 * ct.v[0]], &x[3 * ct.v[1]], &x[3 * ct.v[2]], wv, ct, rb, dx, &dl))
                continue;
            double pt[3] = {(double)ct.p[0], (double)ct.p[1], (double)ct.p[2]};
            double nn[3] = {(double)ct.n[0], (double)ct.n[1], (double)ct.n[2]};
            double dp[3], dq[4];
            rb.contact_delta(dl, pt, nn, dp, dq);
            if (acc) {
                for (int i = 0; i < 3; i++)
                    for (int k = 0; k < 3; k++) (*acc)[3 * ct.v[i] + k] += (R)dx[3 * i + k];
                const size_t bi = (size_t)prim_body[ct.sphere];
                for (int k = 0; k < 3; k++) dps[3 * bi + k] += dp[k];
                for (int k = 0; k < 4; k++) dqs[4 * bi + k] += dq[k];
            } else {
                for (int i = 0; i < 3; i++)
                    for (int k = 0; k < 3; k++) x[3 * ct.v[i] + k] = (R)((double)x[3 * ct.v[i] + k] + dx[3 * i + k]);
                for (int k = 0; k < 3; k++) rb.p[k] = rb.p[k] + dp[k];
                for (int k = 0; k < 4; k++) rb.q[k] = rb.q[k] + dq[k];
            }
        }
        if (acc)
            for (size_t bi = 0; bi < bodies.size(); bi++) {
                for (int k = 0; k < 3; k++) bodies[bi].p[k] += dps[3 * bi + k];
                for (int k = 0; k < 4; k++) bodies[bi].q[k] += dqs[4 * bi + k];
            }
    }
    // kinematic vertex group
    std::vector<int> kin_idx;
    std::vector<R> kin_rest;
    // collision cadence (Simulation.cpp:197-276), in double as the host loop
    double time = 0, last_cd = 0, cd_interval = 1e300;
    // per-iteration residual trajectory of the last update(): ||r||_2
    std::vector<double> res_history;
    // relative-residual stop of update() (0 = off) and the sweeps it ran
    double rel_tol = 0.0;
    int iters_done = 0;

    // Setup: rest shape, materials, masses (XPBDMeshObject.cpp:277-331,
    // 352-417; HydrostaticConstraint.cpp:15-16; DeviatoricConstraint.cpp:13;
    // ElasticMaterial.hpp:31-32).
    void setup(long long V_, const double* X, long long T_, const int* tets_, long long F_, const int* faces_,
               const double* E, const double* nu, const double* rho) {
        V = V_; T = T_; F = F_;
        x.assign(3 * V, 0);
        for (long long i = 0; i < 3 * V; i++) x[i] = (R)X[i];
        X0.assign(X, X + 3 * V);
        Q64.assign(9 * T_, 0.0);
        for (long long t = 0; t < T_; t++) {
            const int* e = tets_ + 4 * t;
            double v_e;
            rest_shape(&X0[3 * e[0]], &X0[3 * e[1]], &X0[3 * e[2]], &X0[3 * e[3]], &Q64[9 * t], &v_e);
        }
        prev = x;
        vel.assign(3 * V, 0);
        tets.assign(tets_, tets_ + 4 * T);
        faces.assign(faces_, faces_ + 3 * F);
        mass.assign(V, 0);
        fixed.assign(V, 0);
        Q.assign(9 * T, 0); vol.assign(T, 0); alpha_d.assign(T, 0); alpha_h.assign(T, 0); gamma.assign(T, 0);
        lam.assign(2 * T, 0);
        for (long long t = 0; t < T; t++) {
            const int* e = &tets[4 * t];
            R v_e;
            rest_shape(&x[3 * e[0]], &x[3 * e[1]], &x[3 * e[2]], &x[3 * e[3]], &Q[9 * t], &v_e);
            vol[t] = v_e;
            R mu = (R)E[t] / (2 * (1 + (R)nu[t]));
            R la = ((R)E[t] * (R)nu[t]) / ((1 + (R)nu[t]) * (1 - 2 * (R)nu[t]));
            R em = v_e * (R)rho[t];
            for (int k = 0; k < 4; k++) mass[e[k]] += em / R(4.0);
            alpha_h[t] = 1 / (la * v_e);
            gamma[t] = mu / la;
            alpha_d[t] = 1 / (mu * v_e);
        }
        inv_mass.assign(V, 0);
        for (long long i = 0; i < V; i++) inv_mass[i] = R(1.0) / mass[i];
        tet_order.clear();
        face_colour.assign(F, 0);
    }

    // 1st-order XPBD (FirstOrderXPBDMeshObject): alpha~ = alpha/dt and the
    // vertex damping B as the constraint inertia (XPBDMeshObject.cpp:333-348,
    // XPBDMeshObjectBase.hpp:131-137), with the vertex E and nu averaged over
    // the attached elements (:321-329). E and nu are per tet.
    bool first_order = false;
    std::vector<R> damping;  // B per vertex
    void set_first_order(double multiplier, bool adjust, const double* E, const double* nu) {
        first_order = true;
        std::vector<R> vvol(V, 0), vE(V, 0), vnu(V, 0);
        std::vector<int> natt(V, 0);
        for (long long t = 0; t < T; t++)
            for (int k = 0; k < 4; k++) natt[tets[4 * t + k]]++;
        for (long long t = 0; t < T; t++)
            for (int k = 0; k < 4; k++) {
                const int v = tets[4 * t + k];
                vvol[v] += vol[t] / R(4.0);
                vE[v] += (R)E[t] / natt[v];
                vnu[v] += (R)nu[t] / natt[v];
            }
        damping.assign(V, 0);
        for (long long i = 0; i < V; i++) {
            damping[i] = adjust ? vvol[i] * (R)multiplier * vE[i] / (1 + vnu[i]) : vvol[i] * (R)multiplier;
            inv_mass[i] = R(1.0) / damping[i];
        }
    }
    R adt() const { return first_order ? dt : dt * dt; }

    // _movePositionsInertially (XPBDMeshObject.cpp:446-470)
    void move_inertially() {
        for (long long i = 0; i < V; i++) {
            if (first_order) {
                x[3 * i + 2] += -g * mass[i] * dt / damping[i];
            } else {
                for (int k = 0; k < 3; k++) x[3 * i + k] += dt * vel[3 * i + k];
                x[3 * i + 2] += -g * dt * dt;
            }
        }
    }

    void use_colouring() {
        std::vector<int> col(T);
        int nc = greedy_colour(T, 4, tets.data(), V, col.data());
        tet_order.clear();
        for (int c = 0; c < nc; c++)
            for (long long t = 0; t < T; t++)
                if (col[t] == c) tet_order.push_back((int)t);
        n_face_colours = F ? greedy_colour(F, 3, faces.data(), V, face_colour.data()) : 0;
    }

    R at_d(long long t) const { return alpha_d[t] / adt(); }
    R at_h(long long t) const { return alpha_h[t] / adt(); }

    void project_tet_combined(long long t, R* dx) {
        const int* e = &tets[4 * t];
        R w[4] = {inv_mass[e[0]], inv_mass[e[1]], inv_mass[e[2]], inv_mass[e[3]]};
        R at[2] = {at_d(t), at_h(t)};
        project_combined(&x[3 * e[0]], &x[3 * e[1]], &x[3 * e[2]], &x[3 * e[3]], w, &Q[9 * t], at, gamma[t],
                         &lam[2 * t], dx);
    }
    void project_tet_single(long long t, int which, R* dx) {
        const int* e = &tets[4 * t];
        R w[4] = {inv_mass[e[0]], inv_mass[e[1]], inv_mass[e[2]], inv_mass[e[3]]};
        R at = which == 0 ? at_d(t) : at_h(t);
        project_single_elem(which, &x[3 * e[0]], &x[3 * e[1]], &x[3 * e[2]], &x[3 * e[3]], w, &Q[9 * t], at,
                            gamma[t], &lam[2 * t + which], dx);
    }
    void add_tet(long long t, const R* dx) {
        const int* e = &tets[4 * t];
        for (int i = 0; i < 4; i++)
            for (int k = 0; k < 3; k++) x[3 * e[i] + k] += dx[3 * i + k];
    }
    bool project_contact_i(Contact<R>& ct, R* dx) {
        R wv[3] = {inv_mass[ct.v[0]], inv_mass[ct.v[1]], inv_mass[ct.v[2]]};
        return project_contact(&x[3 * ct.v[0]], &x[3 * ct.v[1]], &x[3 * ct.v[2]], wv, ct, dx);
    }
    void add_contact(const Contact<R>& ct, const R* dx) {
        for (int i = 0; i < 3; i++)
            for (int k = 0; k < 3; k++) x[3 * ct.v[i] + k] += dx[3 * i + k];
    }

    // ||r||^2 over the elastic constraints, r = C + alpha_tilde*lambda
    // (include/solver/xpbd_solver/XPBDSolver.hpp:327-391)
    void constraint_residual(std::vector<R>& r) const {
        r.assign(2 * T, 0);
        for (long long t = 0; t < T; t++) {
            const int* e = &tets[4 * t];
            R F_[9];
            compute_F(&x[3 * e[0]], &x[3 * e[1]], &x[3 * e[2]], &x[3 * e[3]], &Q[9 * t], F_);
            R Cd = dev_C(F_), Ch = hyd_C(F_, gamma[t]);
            if (ckind == COMBINED) {
                r[2 * t] = Cd + alpha_d[t] / adt() * lam[2 * t];
                r[2 * t + 1] = Ch + alpha_h[t] / adt() * lam[2 * t + 1];
            } else {  // separate: all Dev residuals, then all Hyd residuals
                r[t] = Cd + alpha_d[t] / adt() * lam[2 * t];
                r[T + t] = Ch + alpha_h[t] / adt() * lam[2 * t + 1];
            }
        }
    }
    double residual_norm() const {
        std::vector<R> r;
        constraint_residual(r);
        double s = 0;
        for (R v : r) s += (double)v * (double)v;
        return std::sqrt(s);
    }

    // Sum of C^2/alpha over Dev and Hyd constraints (XPBDMeshObject.cpp:537-549)
    double total_strain_energy() const {
        double e_dev = 0, e_hyd = 0;
        for (long long t = 0; t < T; t++) {
            const int* e = &tets[4 * t];
            R F_[9];
            compute_F(&x[3 * e[0]], &x[3 * e[1]], &x[3 * e[2]], &x[3 * e[3]], &Q[9 * t], F_);
            R Cd = dev_C(F_), Ch = hyd_C(F_, gamma[t]);
            e_dev += (double)(Cd * Cd / alpha_d[t]);
            e_hyd += (double)(Ch * Ch / alpha_h[t]);
        }
        return e_dev + e_hyd;
    }

    // One solver iteration (XPBDGaussSeidelSolver.hpp:29-80,
    // XPBDJacobiSolver.hpp:79-114). Projector type order: elastic first, then
    // static collision (include/common/XPBDTypedefs.hpp, StableNeohookeanCombined
    // / StableNeohookean lists).
    void iterate() {
        R dx[12];
        if (solver == GAUSS_SEIDEL) {
            if (ckind == COMBINED) {
                for (long long t = 0; t < T; t++) { project_tet_combined(t, dx); add_tet(t, dx); }
            } else {
                for (long long t = 0; t < T; t++) { project_tet_single(t, 0, dx); add_tet(t, dx); }
                for (long long t = 0; t < T; t++) { project_tet_single(t, 1, dx); add_tet(t, dx); }
            }
            for (auto& ct : contacts)
                if (!ct.dynamic && project_contact_i(ct, dx)) add_contact(ct, dx);
            project_self_contacts(nullptr);
            project_rigid_contacts(nullptr);
            for (auto& at : attachments) {
                project_attachment(at, dx);
                for (int k = 0; k < 3; k++) x[3 * at.v + k] += dx[k];
            }
        } else if (solver == COLOURED_GS) {
            if (ckind == COMBINED) {
                for (int t : tet_order) { project_tet_combined(t, dx); add_tet(t, dx); }
            } else {
                for (int t : tet_order) { project_tet_single(t, 0, dx); add_tet(t, dx); }
                for (int t : tet_order) { project_tet_single(t, 1, dx); add_tet(t, dx); }
            }
            // contacts: face-colour order, ascending face within a colour,
            // ascending sphere within a face
            for (int k = 0; k < n_face_colours; k++)
                for (auto& ct : contacts)
                    if (face_colour[ct.face] == k && !ct.dynamic)
                        if (project_contact_i(ct, dx)) add_contact(ct, dx);
            project_self_contacts(nullptr);
            project_rigid_contacts(nullptr);
            // attachments in insertion order (the GPU's colours keep it per vertex)
            for (auto& at : attachments) {
                project_attachment(at, dx);
                for (int k = 0; k < 3; k++) x[3 * at.v + k] += dx[k];
            }
        } else {  // Jacobi: every projection reads the same x; updates summed, no averaging
            std::vector<R> acc(3 * V, 0);
            for (long long t = 0; t < T; t++) {
                const int* e = &tets[4 * t];
                if (ckind == COMBINED) {
                    project_tet_combined(t, dx);
                    for (int i = 0; i < 4; i++) for (int k = 0; k < 3; k++) acc[3 * e[i] + k] += dx[3 * i + k];
                } else {
                    project_tet_single(t, 0, dx);
                    for (int i = 0; i < 4; i++) for (int k = 0; k < 3; k++) acc[3 * e[i] + k] += dx[3 * i + k];
                    project_tet_single(t, 1, dx);
                    for (int i = 0; i < 4; i++) for (int k = 0; k < 3; k++) acc[3 * e[i] + k] += dx[3 * i + k];
                }
            }
            for (auto& ct : contacts)
                if (!ct.dynamic && project_contact_i(ct, dx))
                    for (int i = 0; i < 3; i++) for (int k = 0; k < 3; k++) acc[3 * ct.v[i] + k] += dx[3 * i + k];
            project_self_contacts(&acc);
            project_rigid_contacts(&acc);
            for (auto& at : attachments) {
                project_attachment(at, dx);
                for (int k = 0; k < 3; k++) acc[3 * at.v + k] += dx[k];
            }
            for (long long i = 0; i < 3 * V; i++) x[i] += acc[i];
        }
    }

    // _gatherProjectorsForLocalCollisionIterations (XPBDMeshObject.cpp:764-825):
    // for every contact projected with lambda != 0, for each of its three
    // vertices, every element attached to that vertex in ascending element
    // order (TetMesh.cpp:88-96) -- duplicates kept, as the reference lists them
    std::vector<int> local_tet_list() const {
        std::vector<std::vector<int>> attached(V);
        for (long long t = 0; t < T; t++)
            for (int i = 0; i < 4; i++) attached[tets[4 * t + i]].push_back((int)t);
        std::vector<int> out;
        for (const auto& ct : contacts)
            if (ct.lambda != 0 && !ct.dynamic)
                for (int i = 0; i < 3; i++)
                    for (int t : attached[ct.v[i]]) out.push_back(t);
        return out;
    }

    // Local collision iterations (XPBDMeshObject.cpp:472-505): passes over the
    // gathered projectors without re-initialising lambda, elastic projectors
    // before collision projectors (type order of the projector lists).
    //   GAUSS_SEIDEL: the reference's list order, duplicates included;
    //   COLOURED_GS : each listed tet once per pass, in local_order;
    //   JACOBI      : each listed tet once per pass, every projection from the
    //                 same x, updates summed with the contacts'.
    void local_iterations() {
        if (num_local_iter <= 0) return;
        bool any_static = false;
        for (const auto& ct : contacts) any_static |= !ct.dynamic;
        if (!any_static) return;
        const std::vector<int> list = local_tet_list();
        std::vector<char> mark(T, 0);
        for (int t : list) mark[t] = 1;
        R dx[12];
        for (int it = 0; it < num_local_iter; it++) {
            if (solver == GAUSS_SEIDEL) {
                if (ckind == COMBINED) {
                    for (int t : list) { project_tet_combined(t, dx); add_tet(t, dx); }
                } else {
                    for (int t : list) { project_tet_single(t, 0, dx); add_tet(t, dx); }
                    for (int t : list) { project_tet_single(t, 1, dx); add_tet(t, dx); }
                }
                for (auto& ct : contacts)
                    if (!ct.dynamic && project_contact_i(ct, dx)) add_contact(ct, dx);
            } else if (solver == COLOURED_GS) {
                for (int pass = 0; pass < (ckind == COMBINED ? 1 : 2); pass++)
                    for (int t : local_order) {
                        if (!mark[t]) continue;
                        if (ckind == COMBINED) project_tet_combined(t, dx);
                        else project_tet_single(t, pass, dx);
                        add_tet(t, dx);
                    }
                for (int k = 0; k < n_face_colours; k++)
                    for (auto& ct : contacts)
                        if (face_colour[ct.face] == k && !ct.dynamic)
                            if (project_contact_i(ct, dx)) add_contact(ct, dx);
            } else {
                std::vector<R> acc(3 * V, 0);
                for (long long t = 0; t < T; t++) {
                    if (!mark[t]) continue;
                    const int* e = &tets[4 * t];
                    for (int pass = 0; pass < (ckind == COMBINED ? 1 : 2); pass++) {
                        if (ckind == COMBINED) project_tet_combined(t, dx);
                        else project_tet_single(t, pass, dx);
                        for (int i = 0; i < 4; i++) for (int k = 0; k < 3; k++) acc[3 * e[i] + k] += dx[3 * i + k];
                    }
                }
                for (auto& ct : contacts)
                    if (!ct.dynamic && project_contact_i(ct, dx))
                        for (int i = 0; i < 3; i++) for (int k = 0; k < 3; k++) acc[3 * ct.v[i] + k] += dx[3 * i + k];
                for (long long i = 0; i < 3 * V; i++) x[i] += acc[i];
            }
        }
    }

    // Update from a given start (warm-start experiments, not a reference
    // feature): after the inertial move, ||r(x_pred, 0)|| is kept in
    // last_r_plain (the plain solver's normaliser), then the positions move
    // by dx0 (3V, may be empty) and the multipliers start at lam0 (2 per tet;
    // empty: 0) before the sweeps.
    double last_r_plain = 0.0;
    void update_start(const std::vector<R>& dx0, const std::vector<R>& lam0, bool record_residual) {
        prev = x;
        move_inertially();
        std::fill(lam.begin(), lam.end(), R(0));
        for (auto& ct : contacts) ct.lambda = 0;
        for (auto& at : attachments) at.lambda = 0;
        for (auto& sc : self_contacts) sc.lambda = 0;
        last_r_plain = residual_norm();
        if (!dx0.empty())
            for (long long i = 0; i < 3 * V; i++) x[i] += dx0[i];
        if (!lam0.empty()) lam = lam0;
        res_history.clear();
        iters_done = 0;
        for (int it = 0; it < num_iter; it++) {
            if (record_residual) res_history.push_back(residual_norm());
            iterate();
            iters_done = it + 1;
            // rel_tol > 0: stop at ||r|| <= rel_tol * ||r(x_pred, 0)||
            if (rel_tol > 0 && residual_norm() <= rel_tol * last_r_plain) break;
        }
        if (record_residual) res_history.push_back(residual_norm());
        local_iterations();
        for (long long i = 0; i < V; i++)
            if (fixed[i])
                for (int k = 0; k < 3; k++) x[3 * i + k] = prev[3 * i + k];
    }

    // Warm-started update: the multipliers start at lam0 (2 per tet, dev/hyd)
    // and the positions take the matching correction x += M^-1 grad C(x)^T lam0
    // (summed over tets at the predicted positions) before the sweeps; the
    // sweeps then continue from lam0 instead of 0. fallback: when the residual
    // after the correction exceeds the plain residual r(x_pred, 0), the plain
    // initialisation is restored. Returns true when the warm start was kept.
    bool update_warm(const std::vector<R>& lam0, bool record_residual, bool fallback) {
        prev = x;
        move_inertially();
        std::fill(lam.begin(), lam.end(), R(0));
        for (auto& ct : contacts) ct.lambda = 0;
        for (auto& at : attachments) at.lambda = 0;
        for (auto& sc : self_contacts) sc.lambda = 0;
        const double r_plain = residual_norm();
        const std::vector<R> x_pred = x;
        std::vector<R> acc(3 * V, 0);
        for (long long t = 0; t < T; t++) {
            const int* e = &tets[4 * t];
            R F_[9], gd[12], gh[12];
            compute_F(&x[3 * e[0]], &x[3 * e[1]], &x[3 * e[2]], &x[3 * e[3]], &Q[9 * t], F_);
            R Cd = dev_C(F_);
            dev_grad(F_, Cd, &Q[9 * t], gd);
            hyd_grad(F_, &Q[9 * t], gh);
            for (int i = 0; i < 4; i++)
                for (int k = 0; k < 3; k++)
                    acc[3 * e[i] + k] += inv_mass[e[i]] * (gd[3 * i + k] * lam0[2 * t] + gh[3 * i + k] * lam0[2 * t + 1]);
        }
        for (long long i = 0; i < 3 * V; i++) x[i] += acc[i];
        lam = lam0;
        bool kept = true;
        if (fallback && residual_norm() > r_plain) {
            x = x_pred;
            std::fill(lam.begin(), lam.end(), R(0));
            kept = false;
        }
        res_history.clear();
        for (int it = 0; it < num_iter; it++) {
            if (record_residual) res_history.push_back(residual_norm());
            iterate();
        }
        if (record_residual) res_history.push_back(residual_norm());
        local_iterations();
        for (long long i = 0; i < V; i++)
            if (fixed[i])
                for (int k = 0; k < 3; k++) x[3 * i + k] = prev[3 * i + k];
        return kept;
    }

    // XPBDMeshObject_::update = prev <- x; inertial move; project
    // (XPBDMeshObject.cpp:426-505). record_residual stores ||r|| before each
    // iteration and after the last one.
    void update(bool record_residual = false) {
        prev = x;
        move_inertially();
        // XPBDSolver::solve: lambda <- 0, num_iter sweeps (XPBDSolver.hpp:66-97)
        std::fill(lam.begin(), lam.end(), R(0));
        for (auto& ct : contacts) ct.lambda = 0;
        for (auto& at : attachments) at.lambda = 0;
        for (auto& sc : self_contacts) sc.lambda = 0;
        res_history.clear();
        // convergence measurement (not a reference feature): with rel_tol > 0
        // the sweeps stop once ||r|| <= rel_tol * ||r(x_pred, 0)||, at most
        // num_iter of them; iters_done counts the sweeps run
        const double r_first = rel_tol > 0 ? residual_norm() : 0.0;
        iters_done = 0;
        for (int it = 0; it < num_iter; it++) {
            if (record_residual) res_history.push_back(residual_norm());
            iterate();
            iters_done = it + 1;
            if (rel_tol > 0 && residual_norm() <= rel_tol * r_first) break;
        }
        if (record_residual) res_history.push_back(residual_norm());
        local_iterations();
        // fixed vertices back to previous position (XPBDMeshObject.cpp:497-503)
        for (long long i = 0; i < V; i++)
            if (fixed[i])
                for (int k = 0; k < 3; k++) x[3 * i + k] = prev[3 * i + k];
    }

    // v = (x - prev)/dt (XPBDMeshObject.cpp:507-535)
    void velocity_update() {
        for (long long i = 0; i < 3 * V; i++) vel[i] = (x[i] - prev[i]) / dt;
    }

    // clearCollisionConstraints + CollisionScene::collideObjects for the
    // object against every sphere, sphere-major then face order
    // (XPBDMeshObject.cpp:233-251; CollisionScene.cpp:32-51,171-214).
    void detect() {
        contacts.clear();
        sync_prims();
        long long S = (long long)prims.size();
        for (long long s = 0; s < S; s++)
            for (long long f = 0; f < F; f++) {
                const int* fv = &faces[3 * f];
                Contact<R> ct;
                if (collide_face(&x[3 * fv[0]], &x[3 * fv[1]], &x[3 * fv[2]], prims[s], &ct)) {
                    ct.sphere = (int)s;
                    ct.face = (int)f;
                    ct.v[0] = fv[0]; ct.v[1] = fv[1]; ct.v[2] = fv[2];
                    ct.dynamic = is_dynamic((int)s);
                    contacts.push_back(ct);
                }
            }
        // self-collision tests run after the object pairs (CollisionScene.cpp:44-50)
        if (self_collisions) detect_self();
    }

    void set_kinematic_offset(const R* off) {
        for (size_t j = 0; j < kin_idx.size(); j++)
            for (int k = 0; k < 3; k++) x[3 * kin_idx[j] + k] = kin_rest[3 * j + k] + off[k];
    }

    // Simulation::_timeStep for this object (Simulation.cpp:197-276):
    // collision detection on the strict cadence test, update, the free rigid
    // bodies' update, velocities, time.
    void time_step(bool record_residual = false) {
        bool cd = (time - last_cd > cd_interval);
        if (cd) detect();
        update(record_residual);
        // the rigid objects update after the XPBD objects, then every object's
        // velocity update runs (Simulation.cpp:245-255; object type order,
        // include/common/SimulationTypeDefs.hpp)
        for (auto& b : bodies) b.update(dt_host, (double)g);
        velocity_update();
        for (auto& b : bodies) b.velocity_update(dt_host);
        if (time - last_cd > cd_interval) last_cd = time;
        time += dt_host;
    }
};

}  // namespace xo
