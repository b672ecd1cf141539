// extern "C" surface of the XPBD oracle for the Python test suite and the
// benchmark's CPU-baseline leg. TEST INFRASTRUCTURE ONLY: the shipped library
// never links or calls this. See xpbd_oracle.hpp for the parity status.
#include <chrono>
#include <cstdint>

#include "xpbd_oracle.hpp"

namespace {

struct Handle {
    int precision;  // 32 or 64
    xo::Object<float> f;
    xo::Object<double> d;
};

template <typename Fn>
auto with(Handle* h, Fn fn) {
    if (h->precision == 32) return fn(h->f);
    return fn(h->d);
}

template <typename R>
void put_vec(std::vector<R>& dst, const double* src, long long n) {
    for (long long i = 0; i < n; i++) dst[i] = (R)src[i];
}
template <typename R>
void get_vec(const std::vector<R>& src, double* dst, long long n) {
    for (long long i = 0; i < n; i++) dst[i] = (double)src[i];
}

}  // namespace

extern "C" {

void xo_grid_counts(int w, int l, int h, long long* V, long long* T, long long* F) {
    xo::GridDims d{w, l, h};
    *V = d.V(); *T = d.T(); *F = d.F();
}

void xo_grid_mesh(int w, int l, int h, double ex, double ey, double ez, double* X, int* tets, int* faces, int split) {
    xo::grid_mesh(xo::GridDims{w, l, h}, ex, ey, ez, X, tets, faces, split);
}

int xo_greedy_colour(long long n, int arity, const int* items, long long nv, int* colour_out) {
    return xo::greedy_colour(n, arity, items, nv, colour_out);
}

void* xo_create(int precision, long long V, const double* X, long long T, const int* tets, long long F,
                const int* faces, const double* E, const double* nu, const double* rho, double dt, double g,
                int num_iter, int solver, int ckind) {
    Handle* h = new Handle();
    h->precision = precision == 32 ? 32 : 64;
    with(h, [&](auto& o) {
        using R = typename std::decay_t<decltype(o.x)>::value_type;
        o.dt = (R)dt;
        o.dt_host = dt;
        o.g = (R)g;
        o.num_iter = num_iter;
        o.solver = solver;
        o.ckind = ckind;
        o.setup(V, X, T, tets, F, faces, E, nu, rho);
        if (solver == xo::COLOURED_GS) o.use_colouring();
        return 0;
    });
    return h;
}

void xo_destroy(void* p) { delete (Handle*)p; }

void xo_set_collision_rate(void* p, double rate) {
    with((Handle*)p, [&](auto& o) { o.cd_interval = 1.0 / rate; return 0; });
}

void xo_set_num_iter(void* p, int n) {
    with((Handle*)p, [&](auto& o) { o.num_iter = n; return 0; });
}

void xo_set_positions(void* p, const double* x) {
    with((Handle*)p, [&](auto& o) { put_vec(o.x, x, 3 * o.V); return 0; });
}
void xo_get_positions(void* p, double* x) {
    with((Handle*)p, [&](auto& o) { get_vec(o.x, x, 3 * o.V); return 0; });
}
void xo_get_prev_positions(void* p, double* x) {
    with((Handle*)p, [&](auto& o) { get_vec(o.prev, x, 3 * o.V); return 0; });
}
void xo_set_velocities(void* p, const double* v) {
    with((Handle*)p, [&](auto& o) { put_vec(o.vel, v, 3 * o.V); return 0; });
}
void xo_get_velocities(void* p, double* v) {
    with((Handle*)p, [&](auto& o) { get_vec(o.vel, v, 3 * o.V); return 0; });
}
void xo_set_fixed(void* p, const uint8_t* m) {
    with((Handle*)p, [&](auto& o) { for (long long i = 0; i < o.V; i++) o.fixed[i] = m[i] ? 1 : 0; return 0; });
}
void xo_get_masses(void* p, double* m) {
    with((Handle*)p, [&](auto& o) { get_vec(o.mass, m, o.V); return 0; });
}
// per tet: Q (9, column-major), vol, alpha_d, alpha_h, gamma
void xo_get_tet_data(void* p, double* Q, double* vol, double* ad, double* ah, double* gm) {
    with((Handle*)p, [&](auto& o) {
        get_vec(o.Q, Q, 9 * o.T); get_vec(o.vol, vol, o.T); get_vec(o.alpha_d, ad, o.T);
        get_vec(o.alpha_h, ah, o.T); get_vec(o.gamma, gm, o.T);
        return 0;
    });
}
void xo_get_lambda(void* p, double* lam) {
    with((Handle*)p, [&](auto& o) { get_vec(o.lam, lam, 2 * o.T); return 0; });
}
void xo_set_lambda(void* p, const double* lam) {
    with((Handle*)p, [&](auto& o) { put_vec(o.lam, lam, 2 * o.T); return 0; });
}

void xo_set_spheres(void* p, int n, const double* c, const double* r) {
    with((Handle*)p, [&](auto& o) {
        using R = typename std::decay_t<decltype(o.x)>::value_type;
        o.prims.assign(n, xo::Prim<R>{});
        for (int i = 0; i < n; i++) {
            o.prims[i].kind = xo::PRIM_SPHERE;
            for (int k = 0; k < 3; k++) o.prims[i].p[k] = (R)c[3 * i + k];
            o.prims[i].d[0] = (R)r[i];
        }
        return 0;
    });
}

// SDF primitives: kind[n] (0 sphere, 1 box, 2 cylinder), pos 3n, quat 4n
// (x, y, z, w), dims 3n (radius | full size | radius, height)
void xo_set_prims(void* p, int n, const int* kind, const double* pos, const double* quat, const double* dims) {
    with((Handle*)p, [&](auto& o) {
        using R = typename std::decay_t<decltype(o.x)>::value_type;
        o.prims.assign(n, xo::Prim<R>{});
        for (int i = 0; i < n; i++) {
            o.prims[i].kind = kind[i];
            for (int k = 0; k < 3; k++) o.prims[i].p[k] = (R)pos[3 * i + k];
            for (int k = 0; k < 4; k++) o.prims[i].q[k] = (R)quat[4 * i + k];
            for (int k = 0; k < 3; k++) o.prims[i].d[k] = (R)dims[3 * i + k];
        }
        o.prim_body.assign(n, -1);
        o.bodies.clear();
        return 0;
    });
}

// self-collisions on (XPBDMeshObjectConfig self-collisions)
void xo_enable_self_collisions(void* p) {
    with((Handle*)p, [&](auto& o) {
        o.enable_self_collisions();
        return 0;
    });
}

int xo_num_self_contacts(void* p) {
    return with((Handle*)p, [&](auto& o) { return (int)o.self_contacts.size(); });
}

// rows of (vertex, face, lambda)
void xo_get_self_contacts(void* p, double* rows) {
    with((Handle*)p, [&](auto& o) {
        for (size_t i = 0; i < o.self_contacts.size(); i++) {
            rows[3 * i] = o.self_contacts[i].v;
            rows[3 * i + 1] = o.self_contacts[i].f;
            rows[3 * i + 2] = (double)o.self_contacts[i].lambda;
        }
        return 0;
    });
}

// C and gradient (12) of one self contact at the object's current positions
double xo_self_contact_eval(void* p, int v, int f, double* g12) {
    return with((Handle*)p, [&](auto& o) {
        using R = typename std::decay_t<decltype(o.x)>::value_type;
        const int* fv = &o.faces[3 * f];
        R g[12];
        const R C = xo::self_contact_eval(&o.x[3 * v], &o.x[3 * fv[0]], &o.x[3 * fv[1]], &o.x[3 * fv[2]], g);
        for (int i = 0; i < 12; i++) g12[i] = (double)g[i];
        return (double)C;
    });
}

// primitive `prim` becomes a free rigid body with the given pose (double),
// mass, diagonal inertia, velocity and angular velocity
void xo_set_rigid_body(void* p, int prim, const double* pos3, const double* quat4, double mass,
                       const double* inertia3, const double* vel3, const double* omega3) {
    with((Handle*)p, [&](auto& o) {
        xo::RigidBody b;
        b.kind = o.prims[prim].kind;
        for (int k = 0; k < 3; k++) {
            b.d[k] = (double)o.prims[prim].d[k];
            b.p[k] = b.p_prev[k] = pos3[k];
            b.v[k] = vel3[k];
            b.w[k] = omega3[k];
            b.I[k] = inertia3[k];
            b.I_inv[k] = 1.0 / inertia3[k];
        }
        for (int k = 0; k < 4; k++) b.q[k] = b.q_prev[k] = quat4[k];
        b.m = mass;
        if (o.prim_body[prim] >= 0) {
            o.bodies[o.prim_body[prim]] = b;
        } else {
            o.prim_body[prim] = (int)o.bodies.size();
            o.bodies.push_back(b);
        }
        o.sync_prims();
        return 0;
    });
}

// out = p[3], q[4], v[3], w[3] of primitive `prim`'s rigid body
void xo_get_rigid_body(void* p, int prim, double* out) {
    with((Handle*)p, [&](auto& o) {
        const xo::RigidBody& b = o.bodies[o.prim_body[prim]];
        for (int k = 0; k < 3; k++) out[k] = b.p[k];
        for (int k = 0; k < 4; k++) out[3 + k] = b.q[k];
        for (int k = 0; k < 3; k++) out[7 + k] = b.v[k];
        for (int k = 0; k < 3; k++) out[10 + k] = b.w[k];
        return 0;
    });
}

// one SDF value and gradient (test hook): out = (sdf, gx, gy, gz)
void xo_prim_eval(int precision, int kind, const double* pos, const double* quat, const double* dims,
                  const double* x, double* out) {
    auto run = [&](auto zero) {
        using R = decltype(zero);
        xo::Prim<R> pr;
        pr.kind = kind;
        for (int k = 0; k < 3; k++) { pr.p[k] = (R)pos[k]; pr.d[k] = (R)dims[k]; }
        for (int k = 0; k < 4; k++) pr.q[k] = (R)quat[k];
        const R xx[3] = {(R)x[0], (R)x[1], (R)x[2]};
        R g[3];
        out[0] = (double)xo::prim_sdf(pr, xx);
        xo::prim_grad(pr, xx, g);
        for (int k = 0; k < 3; k++) out[1 + k] = (double)g[k];
    };
    if (precision == 32) run(0.0f);
    else run(0.0);
}

// kinematic vertices are fixed vertices driven to rest + offset
void xo_set_kinematic_group(void* p, int n, const int* idx) {
    with((Handle*)p, [&](auto& o) {
        o.kin_idx.assign(idx, idx + n);
        o.kin_rest.assign(3 * n, 0);
        for (int j = 0; j < n; j++) {
            o.fixed[idx[j]] = 1;
            for (int k = 0; k < 3; k++) o.kin_rest[3 * j + k] = o.x[3 * idx[j] + k];
        }
        return 0;
    });
}
void xo_set_kinematic_offset(void* p, const double* off) {
    with((Handle*)p, [&](auto& o) {
        using R = typename std::decay_t<decltype(o.x)>::value_type;
        R of[3] = {(R)off[0], (R)off[1], (R)off[2]};
        o.set_kinematic_offset(of);
        return 0;
    });
}

int xo_detect(void* p) {
    return with((Handle*)p, [&](auto& o) { o.detect(); return (int)o.contacts.size(); });
}
int xo_num_contacts(void* p) {
    return with((Handle*)p, [&](auto& o) { return (int)o.contacts.size(); });
}
// contact row: sphere, face, u, v, w, p0..2, n0..2, lambda  (12 doubles)
void xo_get_contacts(void* p, double* out) {
    with((Handle*)p, [&](auto& o) {
        for (size_t i = 0; i < o.contacts.size(); i++) {
            auto& c = o.contacts[i];
            double* r = out + 12 * i;
            r[0] = c.sphere; r[1] = c.face; r[2] = c.u; r[3] = c.v_; r[4] = c.w;
            for (int k = 0; k < 3; k++) { r[5 + k] = c.p[k]; r[8 + k] = c.n[k]; }
            r[11] = c.lambda;
        }
        return 0;
    });
}
// replace the contact list (rows as above, lambda ignored)
void xo_set_contacts(void* p, int n, const double* rows) {
    with((Handle*)p, [&](auto& o) {
        using R = typename std::decay_t<decltype(o.x)>::value_type;
        o.contacts.clear();
        for (int i = 0; i < n; i++) {
            const double* r = rows + 12 * i;
            xo::Contact<R> c;
            c.sphere = (int)r[0]; c.face = (int)r[1];
            for (int k = 0; k < 3; k++) c.v[k] = o.faces[3 * c.face + k];
            c.u = (R)r[2]; c.v_ = (R)r[3]; c.w = (R)r[4];
            for (int k = 0; k < 3; k++) { c.p[k] = (R)r[5 + k]; c.n[k] = (R)r[8 + k]; }
            c.lambda = 0;
            o.contacts.push_back(c);
        }
        return 0;
    });
}

int xo_update_warm(void* p, const double* lam0, int record, int fallback) {
    return with((Handle*)p, [&](auto& o) {
        using R = typename std::decay_t<decltype(o.x)>::value_type;
        std::vector<R> l(2 * o.T);
        for (long long i = 0; i < 2 * o.T; i++) l[i] = (R)lam0[i];
        return o.update_warm(l, record != 0, fallback != 0) ? 1 : 0;
    });
}

void xo_update_start(void* p, const double* dx0, const double* lam0, int record) {
    with((Handle*)p, [&](auto& o) {
        using R = typename std::decay_t<decltype(o.x)>::value_type;
        std::vector<R> d, l;
        if (dx0) d.assign(dx0, dx0 + 3 * o.V);
        if (lam0) l.assign(lam0, lam0 + 2 * o.T);
        o.update_start(d, l, record != 0);
        return 0;
    });
}
double xo_last_r_plain(void* p) {
    return with((Handle*)p, [&](auto& o) { return o.last_r_plain; });
}
void xo_set_rel_tol(void* p, double tol) {
    with((Handle*)p, [&](auto& o) { o.rel_tol = tol; return 0; });
}
int xo_iters_done(void* p) {
    return with((Handle*)p, [&](auto& o) { return o.iters_done; });
}
void xo_update(void* p, int record) {
    with((Handle*)p, [&](auto& o) { o.update(record != 0); return 0; });
}
void xo_velocity_update(void* p) {
    with((Handle*)p, [&](auto& o) { o.velocity_update(); return 0; });
}
void xo_iterate(void* p) {
    with((Handle*)p, [&](auto& o) { o.iterate(); return 0; });
}
// full time steps; returns wall seconds spent
double xo_time_steps(void* p, int n, int record) {
    auto t0 = std::chrono::steady_clock::now();
    with((Handle*)p, [&](auto& o) { for (int i = 0; i < n; i++) o.time_step(record != 0); return 0; });
    auto t1 = std::chrono::steady_clock::now();
    return std::chrono::duration<double>(t1 - t0).count();
}
double xo_time(void* p) {
    return with((Handle*)p, [&](auto& o) { return o.time; });
}
int xo_res_history(void* p, double* out) {
    return with((Handle*)p, [&](auto& o) {
        if (out) for (size_t i = 0; i < o.res_history.size(); i++) out[i] = o.res_history[i];
        return (int)o.res_history.size();
    });
}
double xo_residual_norm(void* p) {
    return with((Handle*)p, [&](auto& o) { return o.residual_norm(); });
}
void xo_constraint_residual(void* p, double* out) {
    with((Handle*)p, [&](auto& o) {
        using R = typename std::decay_t<decltype(o.x)>::value_type;
        std::vector<R> r;
        o.constraint_residual(r);
        get_vec(r, out, (long long)r.size());
        return 0;
    });
}
double xo_strain_energy(void* p) {
    return with((Handle*)p, [&](auto& o) { return o.total_strain_energy(); });
}
// replace the coloured Gauss-Seidel order (a permutation of the tets), e.g.
// with the sweep order the GPU library reports
// num-local-collision-iters and (optional, n == T) the tet order of the
// coloured local passes
int xo_set_local(void* p, int iters, int n, const int* order) {
    return with((Handle*)p, [&](auto& o) {
        if (iters < 0 || (n && n != (int)o.T)) return 1;
        o.num_local_iter = iters;
        if (n) o.local_order.assign(order, order + n);
        if (o.face_colour.size() != (size_t)o.F || (o.F && o.n_face_colours == 0))
            o.n_face_colours = o.F ? xo::greedy_colour(o.F, 3, o.faces.data(), o.V, o.face_colour.data()) : 0;
        return 0;
    });
}

// the tets the reference gathers for local collision passes (with duplicates);
// returns the count, writes them when out != NULL
int xo_local_tets(void* p, int* out) {
    return with((Handle*)p, [&](auto& o) {
        const std::vector<int> l = o.local_tet_list();
        if (out) std::copy(l.begin(), l.end(), out);
        return (int)l.size();
    });
}

// 1st-order XPBD with the given damping multiplier (E, nu per tet)
void xo_set_first_order(void* p, double multiplier, int adjust, const double* E, const double* nu) {
    with((Handle*)p, [&](auto& o) {
        o.set_first_order(multiplier, adjust != 0, E, nu);
        return 0;
    });
}

// attachment constraint on vertex v with target point (attach point + offset)
void xo_add_attachment(void* p, int v, const double* target3) {
    with((Handle*)p, [&](auto& o) {
        using A = typename std::decay_t<decltype(o.attachments)>::value_type;
        A a;
        a.v = v;
        for (int k = 0; k < 3; k++) a.t[k] = target3[k];
        a.lambda = 0;
        o.attachments.push_back(a);
        return 0;
    });
}

void xo_set_attachment_target(void* p, int id, const double* target3) {
    with((Handle*)p, [&](auto& o) {
        for (int k = 0; k < 3; k++) o.attachments[id].t[k] = target3[k];
        return 0;
    });
}

int xo_set_order(void* p, int n, const int* order) {
    return with((Handle*)p, [&](auto& o) {
        if (n != (int)o.T) return 1;
        std::vector<int> seen(o.T, 0);
        for (int i = 0; i < n; i++) {
            if (order[i] < 0 || order[i] >= (int)o.T || seen[order[i]]++) return 1;
        }
        o.tet_order.assign(order, order + n);
        if (o.face_colour.size() != (size_t)o.F || (o.F && o.n_face_colours == 0))
            o.n_face_colours = o.F ? xo::greedy_colour(o.F, 3, o.faces.data(), o.V, o.face_colour.data()) : 0;
        return 0;
    });
}

// the coloured Gauss-Seidel order actually used (tets in colour order)
int xo_tet_order(void* p, int* out) {
    return with((Handle*)p, [&](auto& o) {
        if (out) for (size_t i = 0; i < o.tet_order.size(); i++) out[i] = o.tet_order[i];
        return (int)o.tet_order.size();
    });
}

// ---- per-element kernels exposed for unit tests (double precision) ----
void xo_rest_shape(const double* X4, double* Q, double* vol) {
    xo::rest_shape(X4, X4 + 3, X4 + 6, X4 + 9, Q, vol);
}
void xo_elem_eval(const double* x4, const double* Q, double gamma, double* F, double* Cd, double* Ch, double* gd,
                  double* gh) {
    xo::compute_F(x4, x4 + 3, x4 + 6, x4 + 9, Q, F);
    *Cd = xo::dev_C(F);
    xo::dev_grad(F, *Cd, Q, gd);
    *Ch = xo::hyd_C(F, gamma);
    xo::hyd_grad(F, Q, gh);
}
void xo_project_combined(const double* x4, const double* w, const double* Q, const double* at, double gamma,
                         double* lam, double* dx) {
    xo::project_combined(x4, x4 + 3, x4 + 6, x4 + 9, w, Q, at, gamma, lam, dx);
}
void xo_project_single(int which, const double* x4, const double* w, const double* Q, double at, double gamma,
                       double* lam, double* dx) {
    xo::project_single_elem(which, x4, x4 + 3, x4 + 6, x4 + 9, w, Q, at, gamma, lam, dx);
}
// one static contact projection on face x3 (3 x 3); returns 0 when skipped
// (C > 0), else 1 with the 9 updates in dx
int xo_project_contact(const double* x3, const double* w, double u, double v, double wb, const double* p,
                       const double* n, double* lam, double* dx) {
    xo::Contact<double> ct{};
    ct.u = u; ct.v_ = v; ct.w = wb;
    for (int k = 0; k < 3; k++) { ct.p[k] = p[k]; ct.n[k] = n[k]; }
    ct.lambda = *lam;
    const bool on = xo::project_contact(x3, x3 + 3, x3 + 6, w, ct, dx);
    *lam = ct.lambda;
    return on ? 1 : 0;
}

}  // extern "C"
