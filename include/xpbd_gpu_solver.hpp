// xpbd_gpu_solver.hpp -- C++ host mirror of the reference's XPBDSolver
// surface over the C ABI in xpbd_gpu.h.
//
// Drop-in for the solver member of XPBDMeshObject_<false, SolverType, ...>
// (include/simobject/XPBDMeshObject.hpp:229 in the reference). The member
// functions keep the reference's names and argument meaning:
//
//   GPUXPBDSolver(obj, num_iter, residual_policy)   XPBDSolver.hpp:47-51
//   setup()                                         XPBDSolver.hpp:56-61
//   solve()                                         XPBDSolver.hpp:66-97
//   solveLocal(num_iter) = solve(refs, num_iter,    XPBDSolver.hpp:106-125
//     false) over the local collision set
//   constraintResidual()                            XPBDSolver.hpp:135
//   numIterations()                                 XPBDSolver.hpp:139
//   addStaticCollisionConstraint(...)               XPBDMeshObject.cpp:180-206
//   clearCollisionConstraints()                     XPBDMeshObject.cpp:233-251
//
// ObjectT is duck-typed so this header builds without Eigen: it needs
//   obj->mesh()->numVertices(), obj->mesh()->vertices().data() (3 x V, Real),
//   obj->tetMesh()->numElements(), obj->tetMesh()->elements().data() (4 x T, int),
//   obj->mesh()->numFaces(), obj->mesh()->faces().data() (3 x F, int),
//   obj->vertexFixed(i), and per-element material accessors supplied by the
//   caller through MaterialFn (E, nu, density of element i).
//
// solve() means what the reference's does: every projector's lambda <- 0,
// then num_iter sweeps over the mesh's current positions -- no inertial move
// and no fixed-vertex reset, which XPBDMeshObject_::update and
// _projectConstraints do around it (XPBDMeshObject.cpp:426-505). The
// reference's solver works on the mesh in place; this one owns a device copy,
// so solve() uploads the mesh's positions, solves on the device and writes
// the result back into the mesh. A binding dropped in at
// XPBDMeshObject.cpp:476 therefore keeps the host's inertial move before it
// and the host's fixed-vertex loop after it. solveLocal(n) is the
// solve(refs, n, false) call that follows (XPBDMeshObject.cpp:483).
//
// updateOnDevice() runs the whole of XPBDMeshObject_::update (prediction,
// projection, local passes, fixed reset) on the device; callers that keep the
// state there use it or step() and read back only when needed.
#pragma once

#include <cstdint>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

#include "xpbd_gpu.h"

namespace xpbd_gpu {

class Error : public std::runtime_error {
   public:
    Error(int status, const std::string& what) : std::runtime_error(what), status_(status) {}
    int status() const { return status_; }

   private:
    int status_;
};

struct Material {
    double E, nu, density;
};

template <typename ObjectT>
class GPUXPBDSolver {
   public:
    using MaterialFn = std::function<Material(int element)>;

    // residual_policy: 0 Never, 1 Every-Substep, 2 Every-Iteration
    GPUXPBDSolver(ObjectT* obj, int num_iter, int residual_policy, int solver_type = XPBD_SOLVER_GAUSS_SEIDEL)
        : obj_(obj) {
        xpbd_default_params(&params_);
        params_.num_iters = num_iter;
        params_.residual_policy = residual_policy;
        params_.solver_type = solver_type;
    }
    GPUXPBDSolver(const GPUXPBDSolver&) = delete;
    GPUXPBDSolver& operator=(const GPUXPBDSolver&) = delete;
    ~GPUXPBDSolver() {
        if (ctx_) xpbd_destroy(ctx_);
    }

    xpbd_params& params() { return params_; }

    // Uploads the object's mesh; the object's current state is its rest state.
    void setup(double dt, double g_accel, const MaterialFn& material) {
        params_.dt = dt;
        params_.g_accel = g_accel;
        auto* mesh = obj_->mesh();
        auto* tm = obj_->tetMesh();
        const int64_t V = mesh->numVertices(), T = tm->numElements(), F = mesh->numFaces();
        std::vector<double> X(3 * V), E(T), nu(T), rho(T);
        const auto* xv = mesh->vertices().data();
        for (int64_t i = 0; i < 3 * V; i++) X[i] = (double)xv[i];
        std::vector<int32_t> tets(4 * T), faces(3 * F);
        const auto* ev = tm->elements().data();
        for (int64_t i = 0; i < 4 * T; i++) tets[i] = (int32_t)ev[i];
        const auto* fv = mesh->faces().data();
        for (int64_t i = 0; i < 3 * F; i++) faces[i] = (int32_t)fv[i];
        for (int64_t t = 0; t < T; t++) {
            const Material m = material((int)t);
            E[t] = m.E; nu[t] = m.nu; rho[t] = m.density;
        }
        xpbd_mesh_desc d{V, T, F, X.data(), tets.data(), F ? faces.data() : nullptr, E.data(), nu.data(), rho.data()};
        check(xpbd_create(&d, &params_, &ctx_), nullptr);
        std::vector<uint8_t> fixed(V);
        for (int64_t i = 0; i < V; i++) fixed[i] = obj_->vertexFixed((int)i) ? 1 : 0;
        check(xpbd_set_fixed(ctx_, fixed.data()));
        V_ = V;
        T_ = T;
    }

    // XPBDSolver::solve() (XPBDSolver.hpp:66-97) on the mesh's positions.
    void solve() {
        upload_positions();
        check(xpbd_solve(ctx_));
        download_positions();
    }
    // XPBDSolver::solve(refs, num_iter, false) over the local collision set
    // (XPBDMeshObject.cpp:483, 764-825); the context needs
    // params().num_local_collision_iters > 0 before setup().
    void solveLocal(int num_iter) {
        upload_positions();
        check(xpbd_solve_local(ctx_, num_iter));
        download_positions();
    }

    // device-resident variants: XPBDMeshObject_::update on the device
    void updateOnDevice() { check(xpbd_update(ctx_)); }
    void velocityUpdate() { check(xpbd_velocity_update(ctx_)); }
    void step(int n) { check(xpbd_step(ctx_, n)); }
    void upload_positions() {
        const auto* xv = obj_->mesh()->vertices().data();
        host_.resize(3 * V_);
        for (int64_t i = 0; i < 3 * V_; i++) host_[i] = (double)xv[i];
        check(xpbd_set_positions(ctx_, host_.data()));
    }
    void download_positions() {
        host_.resize(3 * V_);
        check(xpbd_get_positions(ctx_, host_.data()));
        auto* xv = obj_->mesh()->vertices().data();
        for (int64_t i = 0; i < 3 * V_; i++) xv[i] = (std::remove_reference_t<decltype(*xv)>)host_[i];
    }

    std::vector<double> constraintResidual() {
        std::vector<double> r(2 * T_);
        check(xpbd_get_constraint_residual(ctx_, r.data(), (int64_t)r.size()));
        return r;
    }
    int numIterations() const { return params_.num_iters; }

    void addStaticCollisionConstraint(const double* surface_point, const double* normal, int face, double u,
                                      double v, double w) {
        check(xpbd_add_static_collision(ctx_, face, u, v, w, surface_point, normal));
    }
    void clearCollisionConstraints() { check(xpbd_clear_collisions(ctx_)); }
    // a free rigid body in SDF slot `slot` (RigidObject with fixed: false); its
    // contacts are the reference's RigidDeformableCollisionConstraints, created
    // by the device detection (addRigidDeformableCollisionConstraint has no
    // host-side counterpart)
    void setRigidBody(int slot, double mass, const double* inertia3, const double* velocity3,
                      const double* angular_velocity3) {
        check(xpbd_set_rigid_body(ctx_, 0, slot, mass, inertia3, velocity3, angular_velocity3));
    }
    // position[3], orientation (x, y, z, w)[4], velocity[3], angular velocity[3]
    void rigidBodyState(int slot, double* state13) { check(xpbd_get_rigid_body(ctx_, 0, slot, state13)); }

    xpbd_ctx* context() { return ctx_; }

   private:
    void check(int st) { check(st, ctx_); }
    static void check(int st, xpbd_ctx* c) {
        if (st != XPBD_OK) throw Error(st, std::string("xpbd: ") + (c ? xpbd_last_error(c) : xpbd_status_string(st)));
    }

    ObjectT* obj_;
    xpbd_params params_{};
    xpbd_ctx* ctx_ = nullptr;
    int64_t V_ = 0, T_ = 0;
    std::vector<double> host_;
};

}  // namespace xpbd_gpu
