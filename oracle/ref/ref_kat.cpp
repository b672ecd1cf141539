// extern "C" driver over the reference's own constraint and projector
// classes, compiled from the reference's sources by oracle/ref/Makefile into
// oracle/_ref/libref_kat.so. TEST INFRASTRUCTURE ONLY: it checks the oracle
// (oracle/xpbd_oracle.hpp) against the reference's arithmetic; nothing in the
// product links it. Real is double here (the reference's CPU build).
//
// Reference code exercised:
//   ElementConstraint (Q, rest volume, F)  include/solver/constraint/ElementConstraint.hpp:23-119
//   HydrostaticConstraint                  include/solver/constraint/HydrostaticConstraint.hpp:123-221,
//                                          src/solver/constraint/HydrostaticConstraint.cpp:15-16
//   DeviatoricConstraint                   include/solver/constraint/DeviatoricConstraint.hpp:112-152,
//                                          src/solver/constraint/DeviatoricConstraint.cpp:13
//   CombinedConstraintProjector<false, Dev, Hyd>::project
//                                          src/solver/xpbd_projector/CombinedNeohookeanConstraintProjector.cpp:98-179
//   ConstraintProjector<false, C>::project include/solver/xpbd_projector/ConstraintProjector.hpp:111-172
//   StaticDeformableCollisionConstraint    src/solver/constraint/StaticDeformableCollisionConstraint.cpp:20-49
//   ElasticMaterial (Lame parameters)      include/simobject/ElasticMaterial.hpp:31-32
// The mesh-object steps around the projectors (lumped masses, inertial move,
// Gauss-Seidel application, fixed reset, velocity) are restated below from
// src/simobject/XPBDMeshObject.cpp and XPBDGaussSeidelSolver.hpp, with the
// lines cited, because XPBDMeshObject_ itself needs the whole object layer.
#include <cmath>
#include <cstring>
#include <vector>

#include "simobject/ElasticMaterial.hpp"
#include "solver/constraint/DeviatoricConstraint.hpp"
#include "solver/constraint/HydrostaticConstraint.hpp"
#include "solver/constraint/StaticDeformableCollisionConstraint.hpp"
#include "solver/xpbd_projector/CombinedNeohookeanConstraintProjector.hpp"
#include "solver/xpbd_projector/ConstraintProjector.hpp"

using Solver::CombinedConstraintProjector;
using Solver::ConstraintProjector;
using Solver::ConstraintReference;
using Solver::CoordinateUpdate;
using Solver::DeviatoricConstraint;
using Solver::HydrostaticConstraint;
using Solver::StaticDeformableCollisionConstraint;

namespace {

// read access to the protected rest-shape members
struct DevPeek : DeviatoricConstraint {
    using DeviatoricConstraint::DeviatoricConstraint;
    const Mat3r& Q() const { return _Q; }
};
struct HydPeek : HydrostaticConstraint {
    using HydrostaticConstraint::HydrostaticConstraint;
    Real gamma() const { return _gamma; }
};

ElasticMaterial material(double E, double nu, double rho) { return ElasticMaterial("kat", rho, E, nu, 0.0, 0.0); }

using Combined = CombinedConstraintProjector<false, DeviatoricConstraint, HydrostaticConstraint>;

}  // namespace

extern "C" {

// Q = Dm^-1 (column-major, q[3c + r] = Q(r, c)), rest volume, alpha_dev,
// alpha_hyd and gamma of one tet at rest X4 (4 x 3).
void ref_rest(const double* X4, double E, double nu, double* Q, double* vol, double* alpha_dev, double* alpha_hyd,
              double* gamma) {
    double buf[12];
    std::memcpy(buf, X4, sizeof buf);
    const ElasticMaterial m = material(E, nu, 1000.0);
    DevPeek d(0, buf, 1.0, 1, buf + 3, 1.0, 2, buf + 6, 1.0, 3, buf + 9, 1.0, m);
    HydPeek h(0, buf, 1.0, 1, buf + 3, 1.0, 2, buf + 6, 1.0, 3, buf + 9, 1.0, m);
    for (int c = 0; c < 3; c++)
        for (int r = 0; r < 3; r++) Q[3 * c + r] = d.Q()(r, c);
    *vol = d.restVolume();
    *alpha_dev = d.alpha();
    *alpha_hyd = h.alpha();
    *gamma = h.gamma();
}

// C and grad C (12 values) of both constraints of a tet built at rest X4 and
// evaluated at x4.
void ref_eval(const double* X4, const double* x4, double E, double nu, double* Cd, double* Ch, double* gd,
              double* gh) {
    double buf[12];
    std::memcpy(buf, X4, sizeof buf);
    const ElasticMaterial m = material(E, nu, 1000.0);
    DeviatoricConstraint d(0, buf, 1.0, 1, buf + 3, 1.0, 2, buf + 6, 1.0, 3, buf + 9, 1.0, m);
    HydrostaticConstraint h(0, buf, 1.0, 1, buf + 3, 1.0, 2, buf + 6, 1.0, 3, buf + 9, 1.0, m);
    std::memcpy(buf, x4, sizeof buf);
    d.evaluateWithGradient(Cd, gd);
    h.evaluateWithGradient(Ch, gh);
}

// nproj successive combined projections of one tet (built at rest X4, vertex
// masses m4, started at x4, lambda initialised once), each update applied
// before the next projection: per projection the 12 updates and (lambda_dev,
// lambda_hyd) after it; x_out = the final positions.
void ref_project_combined(const double* X4, const double* x4, const double* m4, double E, double nu, double dt,
                          int nproj, double* dx, double* lam, double* x_out) {
    double buf[12];
    std::memcpy(buf, X4, sizeof buf);
    const ElasticMaterial m = material(E, nu, 1000.0);
    std::vector<DeviatoricConstraint> devs;
    std::vector<HydrostaticConstraint> hyds;
    devs.emplace_back(0, buf, m4[0], 1, buf + 3, m4[1], 2, buf + 6, m4[2], 3, buf + 9, m4[3], m);
    hyds.emplace_back(0, buf, m4[0], 1, buf + 3, m4[1], 2, buf + 6, m4[2], 3, buf + 9, m4[3], m);
    Combined p(dt, ConstraintReference<DeviatoricConstraint>(devs, 0), ConstraintReference<HydrostaticConstraint>(hyds, 0));
    std::memcpy(buf, x4, sizeof buf);
    p.initialize();
    CoordinateUpdate u[Combined::MAX_NUM_COORDINATES];
    for (int k = 0; k < nproj; k++) {
        p.project(u);
        for (int i = 0; i < p.numCoordinates(); i++) {
            dx[12 * k + i] = u[i].update;
            if (u[i].ptr) *u[i].ptr += u[i].update;
        }
        const Vec2r l = p.lambda();
        lam[2 * k] = l[0];
        lam[2 * k + 1] = l[1];
    }
    std::memcpy(x_out, buf, sizeof buf);
}

// The same with the scalar projector of one constraint (which 0: deviatoric,
// 1: hydrostatic), the Stable-Neohookean (separate) configuration; lam gets
// the single multiplier after each projection (read back through the
// update: dlambda = update / (w grad C) is not exposed, so the driver returns
// the updates and the caller checks them).
void ref_project_single(int which, const double* X4, const double* x4, const double* m4, double E, double nu,
                        double dt, int nproj, double* dx, double* x_out) {
    double buf[12];
    std::memcpy(buf, X4, sizeof buf);
    const ElasticMaterial m = material(E, nu, 1000.0);
    std::vector<DeviatoricConstraint> devs;
    std::vector<HydrostaticConstraint> hyds;
    devs.emplace_back(0, buf, m4[0], 1, buf + 3, m4[1], 2, buf + 6, m4[2], 3, buf + 9, m4[3], m);
    hyds.emplace_back(0, buf, m4[0], 1, buf + 3, m4[1], 2, buf + 6, m4[2], 3, buf + 9, m4[3], m);
    std::memcpy(buf, x4, sizeof buf);
    CoordinateUpdate u[12];
    auto run = [&](auto& p) {
        p.initialize();
        for (int k = 0; k < nproj; k++) {
            p.project(u);
            for (int i = 0; i < 12; i++) {
                dx[12 * k + i] = u[i].update;
                if (u[i].ptr) *u[i].ptr += u[i].update;
            }
        }
    };
    if (which == 0) {
        ConstraintProjector<false, DeviatoricConstraint> p(dt, ConstraintReference<DeviatoricConstraint>(devs, 0));
        run(p);
    } else {
        ConstraintProjector<false, HydrostaticConstraint> p(dt, ConstraintReference<HydrostaticConstraint>(hyds, 0));
        run(p);
    }
    std::memcpy(x_out, buf, sizeof buf);
}

// nproj successive projections of one static collision constraint on the
// face x3 (3 x 3) with masses m3, barycentrics (u, v, w), surface point p and
// normal n (an inequality: no update while C > 0).
void ref_project_collision(const double* x3, const double* m3, const double* p, const double* n, double u, double v,
                           double w, double dt, int nproj, double* dx, double* x_out) {
    double buf[9];
    std::memcpy(buf, x3, sizeof buf);
    const Vec3r pv(p[0], p[1], p[2]), nv(n[0], n[1], n[2]);
    std::vector<StaticDeformableCollisionConstraint> cs;
    cs.emplace_back(nullptr, pv, nv, 0, buf, m3[0], 1, buf + 3, m3[1], 2, buf + 6, m3[2], u, v, w);
    ConstraintProjector<false, StaticDeformableCollisionConstraint> pr(
        dt, ConstraintReference<StaticDeformableCollisionConstraint>(cs, 0));
    pr.initialize();
    CoordinateUpdate up[9];
    for (int k = 0; k < nproj; k++) {
        pr.project(up);
        for (int i = 0; i < 9; i++) {
            dx[9 * k + i] = up[i].update;
            if (up[i].ptr) *up[i].ptr += up[i].update;
        }
    }
    std::memcpy(x_out, buf, sizeof buf);
}

// nsteps substeps of a second-order XPBD mesh object with combined
// constraints and the sequential Gauss-Seidel solver, built from the
// reference's constraint and projector classes:
//   masses      XPBDMeshObject.cpp:277-331 (rho * elementVolume / 4 per vertex,
//               TetMesh.cpp:153-166), passed as vertexConstraintInertia
//               (XPBDMeshObjectBase.hpp:131-137)
//   constraints XPBDMeshObject.cpp:352-417 (combined: Dev and Hyd per element,
//               one projector per element in element order)
//   update      XPBDMeshObject.cpp:426-505 (prev <- x, x += dt v, z -= g dt^2,
//               solve, fixed vertices back to prev)
//   solve       XPBDSolver.hpp:66-97 (initialize, num_iter sweeps) with
//               XPBDGaussSeidelSolver.hpp:29-80 (project, apply non-null updates)
//   velocity    XPBDMeshObject.cpp:507-535 (v = (x - prev) / dt)
// X (V x 3) rest = initial state unless x0 is given; x_out (V x 3) and lam
// (T x 2, dev/hyd) receive the final state.
void ref_gs_steps(long long V, const double* X, const double* x0, long long T, const int* tets, const double* E,
                  const double* nu, const double* rho, const unsigned char* fixed, double dt, double g, int num_iter,
                  int nsteps, double* x_out, double* lam) {
    std::vector<double> x(X, X + 3 * V), prev(3 * V), vel(3 * V, 0.0), mass(V, 0.0);
    for (long long e = 0; e < T; e++) {
        const int* t = tets + 4 * e;
        Mat3r D;
        for (int c = 0; c < 3; c++)
            for (int k = 0; k < 3; k++) D(k, c) = x[3 * t[c] + k] - x[3 * t[3] + k];
        const double vol = std::abs(D.determinant() / 6.0);
        const double em = vol * rho[e];
        for (int q = 0; q < 4; q++) mass[t[q]] += em / 4.0;
    }
    std::vector<ElasticMaterial> mats;
    mats.reserve(T);
    std::vector<DeviatoricConstraint> devs;
    std::vector<HydrostaticConstraint> hyds;
    devs.reserve(T);
    hyds.reserve(T);
    std::vector<Combined> projs;
    projs.reserve(T);
    for (long long e = 0; e < T; e++) {
        const int* t = tets + 4 * e;
        mats.push_back(material(E[e], nu[e], rho[e]));
        double* p[4] = {&x[3 * t[0]], &x[3 * t[1]], &x[3 * t[2]], &x[3 * t[3]]};
        hyds.emplace_back(t[0], p[0], mass[t[0]], t[1], p[1], mass[t[1]], t[2], p[2], mass[t[2]], t[3], p[3],
                          mass[t[3]], mats.back());
        devs.emplace_back(t[0], p[0], mass[t[0]], t[1], p[1], mass[t[1]], t[2], p[2], mass[t[2]], t[3], p[3],
                          mass[t[3]], mats.back());
        projs.emplace_back(dt, ConstraintReference<DeviatoricConstraint>(devs, (int)e),
                           ConstraintReference<HydrostaticConstraint>(hyds, (int)e));
    }
    if (x0) std::memcpy(x.data(), x0, sizeof(double) * 3 * V);
    CoordinateUpdate u[Combined::MAX_NUM_COORDINATES];
    for (int s = 0; s < nsteps; s++) {
        prev = x;
        for (long long i = 0; i < 3 * V; i++) x[i] += dt * vel[i];
        for (long long i = 0; i < V; i++) x[3 * i + 2] += -g * dt * dt;
        for (auto& p : projs) p.initialize();
        for (int it = 0; it < num_iter; it++)
            for (auto& p : projs) {
                p.project(u);
                for (int i = 0; i < p.numCoordinates(); i++)
                    if (u[i].ptr) *u[i].ptr += u[i].update;
            }
        for (long long i = 0; i < V; i++)
            if (fixed[i])
                for (int k = 0; k < 3; k++) x[3 * i + k] = prev[3 * i + k];
        for (long long i = 0; i < 3 * V; i++) vel[i] = (x[i] - prev[i]) / dt;
    }
    std::memcpy(x_out, x.data(), sizeof(double) * 3 * V);
    for (long long e = 0; e < T; e++) {
        const Vec2r l = projs[e].lambda();
        lam[2 * e] = l[0];
        lam[2 * e + 1] = l[1];
    }
}

}  // extern "C"
