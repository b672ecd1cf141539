// Free rigid bodies on the device (RigidObject with fixed: false and the
// two-way RigidDeformableCollisionConstraint): FP64 body records, their SDF
// table, contact compaction, the contact projections in slot order and the
// body update / velocity update.
//   src/simobject/RigidObject.cpp:41-77
//   src/solver/constraint/RigidDeformableCollisionConstraint.cpp:23-55
//   include/solver/xpbd_projector/RigidBodyConstraintProjector.hpp:97-158
#include "xpbd_device.cuh"

namespace xg {

namespace {

// ---- free rigid bodies: two-way coupling (FP64, one thread) ----
// GeometryUtils quatMult / rotateVectorByQuat / inverseQuat
// (src/utils/GeometryUtils.cpp:81-102), quaternions (x, y, z, w)
__device__ __forceinline__ void dquat_mult(const double* a, const double* b, double* r) {
    r[0] = a[3] * b[0] + a[0] * b[3] + a[1] * b[2] - a[2] * b[1];
    r[1] = a[3] * b[1] + a[1] * b[3] + a[2] * b[0] - a[0] * b[2];
    r[2] = a[3] * b[2] + a[2] * b[3] + a[0] * b[1] - a[1] * b[0];
    r[3] = a[3] * b[3] - a[0] * b[0] - a[1] * b[1] - a[2] * b[2];
}
__device__ __forceinline__ void dquat_rotate(const double* v, const double* q, double* o) {
    const double ud = q[0] * v[0] + q[1] * v[1] + q[2] * v[2];
    const double s = 2 * q[3] * q[3] - 1;
    const double cx = q[1] * v[2] - q[2] * v[1], cy = q[2] * v[0] - q[0] * v[2], cz = q[0] * v[1] - q[1] * v[0];
    o[0] = 2 * ud * q[0] + s * v[0] + 2 * q[3] * cx;
    o[1] = 2 * ud * q[1] + s * v[1] + 2 * q[3] * cy;
    o[2] = 2 * ud * q[2] + s * v[2] + 2 * q[3] * cz;
}
__device__ __forceinline__ void dquat_inverse(const double* q, double* r) {
    const double n2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
    r[0] = -q[0] / n2; r[1] = -q[1] / n2; r[2] = -q[2] / n2; r[3] = q[3] / n2;
}
__device__ __forceinline__ void dcross(const double* a, const double* b, double* r) {
    r[0] = a[1] * b[2] - a[2] * b[1];
    r[1] = a[2] * b[0] - a[0] * b[2];
    r[2] = a[0] * b[1] - a[1] * b[0];
}

// The body's SDF at its current pose (SphereSDF / BoxSDF / CylinderSDF::evaluate;
// RigidObject::globalToBody): the orientation may be off unit length inside a
// solve, and the rotation formula is applied to it as it stands
__device__ double sdf_body(const double* rb, const double* x) {
    const double* p = rb + RB_P;
    const int kind = (int)rb[RB_KIND];
    const double* d = rb + RB_D;
    if (kind == 0) {
        const double a = x[0] - p[0], b = x[1] - p[1], c = x[2] - p[2];
        return sqrt(a * a + b * b + c * c) - d[0];
    }
    double qi[4], b[3];
    dquat_inverse(rb + RB_Q, qi);
    const double rel[3] = {x[0] - p[0], x[1] - p[1], x[2] - p[2]};
    dquat_rotate(rel, qi, b);
    if (kind == 1) {
        double o = 0, mq = -1e300;
        for (int k = 0; k < 3; k++) {
            const double q = fabs(b[k]) - 0.5 * d[k];
            const double m = fmax(q, 0.0);
            o += m * m;
            mq = fmax(mq, q);
        }
        return sqrt(o) + fmin(mq, 0.0);
    }
    const double xy = sqrt(b[0] * b[0] + b[1] * b[1]) - d[0];
    const double z = fabs(b[2]) - 0.5 * d[1];
    const double ox = fmax(xy, 0.0), oz = fmax(z, 0.0);
    return sqrt(ox * ox + oz * oz) + fmin(fmax(xy, z), 0.0);
}

// PositionalRigidBodyXPBDHelper::update (RigidBodyConstraint.hpp): the body's
// increments for a contact at pt pushing along -n, from its current pose
__device__ void rigid_contact_delta(const double* rb, double dlam, const double* pt, const double* n, double* dp,
                                    double* dq) {
    const double dir[3] = {-n[0], -n[1], -n[2]};
    double qi[4], rbody[3], nb[3], t[3], cr[3], wb[3], ws[3];
    dquat_inverse(rb + RB_Q, qi);
    const double rel[3] = {pt[0] - rb[RB_P], pt[1] - rb[RB_P + 1], pt[2] - rb[RB_P + 2]};
    dquat_rotate(rel, qi, rbody);
    dquat_rotate(dir, qi, nb);
    for (int k = 0; k < 3; k++) dp[k] = dlam * dir[k] / rb[RB_M];
    for (int k = 0; k < 3; k++) t[k] = dlam * nb[k];
    dcross(rbody, t, cr);
    for (int k = 0; k < 3; k++) wb[k] = 0.5 * rb[RB_II + k] * cr[k];
    dquat_rotate(wb, rb + RB_Q, ws);
    const double w4[4] = {ws[0], ws[1], ws[2], 0.0};
    dquat_mult(w4, rb + RB_Q, dq);
}

// table entries of the free bodies from their poses (the detection's view)
__global__ void k_rigid_sync_table(const double* __restrict__ rb, int nb, float4* __restrict__ table) {
    pdl_wait_then_release();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb) return;
    const double* r = rb + (size_t)i * kRigidRec;
    const size_t e = (size_t)r[RB_ENTRY];
    table[3 * e] = make_float4((float)r[RB_P], (float)r[RB_P + 1], (float)r[RB_P + 2], table[3 * e].w);
    table[3 * e + 1] = make_float4((float)r[RB_Q], (float)r[RB_Q + 1], (float)r[RB_Q + 2], (float)r[RB_Q + 3]);
}

// slots of the rigid contacts (active = 2) in slot order, one block
__global__ void __launch_bounds__(kCompactThreads) k_rigid_compact(ContactArrays c, int* __restrict__ list,
                                                                   int* __restrict__ count) {
    __shared__ int warp_tot[kCompactThreads / 32];
    __shared__ int base;
    pdl_wait_then_release();
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int ns = c.S * c.F;
    if (tid == 0) base = 0;
    __syncthreads();
    for (int b0 = 0; b0 < ns; b0 += kCompactThreads) {
        const int slot = b0 + tid;
        const bool hit = slot < ns && c.bary[slot].w == 2.f;
        const unsigned m = __ballot_sync(0xffffffffu, hit);
        if (lane == 0) warp_tot[wid] = __popc(m);
        __syncthreads();
        int off = base;
        for (int w = 0; w < wid; w++) off += warp_tot[w];
        if (hit) list[off + __popc(m & ((1u << lane) - 1u))] = slot;
        __syncthreads();
        if (tid == 0) {
            int t = 0;
            for (int w = 0; w < kCompactThreads / 32; w++) t += warp_tot[w];
            base += t;
        }
        __syncthreads();
    }
    if (tid == 0) *count = base;
}

// RigidDeformableCollisionConstraint projected by RigidBodyConstraintProjector
// (RigidDeformableCollisionConstraint.cpp:35-55, RigidBodyConstraintProjector.hpp:97-158):
// C = the body's SDF at the barycentric point, gradient (u n, v n, w n),
// skipped when C > 0, alpha = 0, the multiplier from the deformable weights
// alone; the vertices and the body move by the increments. Every contact
// moves the body that the next one reads, so one thread walks the list.
// Gauss-Seidel applies each update at once; Jacobi reads one state, adds the
// vertex updates to dx and sums the body increments, applied at the end
// (XPBDGaussSeidelSolver.hpp:61-95, XPBDJacobiSolver.hpp:79-114).
__global__ void k_rigid_contacts(ContactArrays c, const int* __restrict__ list, const int* __restrict__ count,
                                 const float4* __restrict__ table, const int* __restrict__ face_inst,
                                 double* __restrict__ rb, int nb, float4* __restrict__ x, float4* __restrict__ dx,
                                 bool jacobi, bool first, Flags* flags) {
    pdl_wait_then_release();
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    if (jacobi)
        for (int i = 0; i < nb; i++)
            for (int k = 0; k < 7; k++) rb[(size_t)i * kRigidRec + RB_ACC + k] = 0.0;
    const int n = *count;
    for (int j = 0; j < n; j++) {
        const int slot = list[j];
        const int f = slot % c.F, sl = slot / c.F;
        const size_t e = (size_t)face_inst[f] * c.S + sl;
        const int body = (int)table[3 * e + 2].w - 1;
        if (body < 0 || body >= nb) continue;  // the host resets the list when bodies change
        double* r = rb + (size_t)body * kRigidRec;
        const int4 fv = c.faces[f];
        const int vi[3] = {fv.x, fv.y, fv.z};
        const float4 xs[3] = {x[fv.x], x[fv.y], x[fv.z]};
        const float4 bb = c.bary[slot];
        const double b[3] = {(double)bb.x, (double)bb.y, (double)bb.z};
        float lam = first ? 0.f : c.lam[slot];
        double a[3];
        a[0] = b[0] * (double)xs[0].x + b[1] * (double)xs[1].x + b[2] * (double)xs[2].x;
        a[1] = b[0] * (double)xs[0].y + b[1] * (double)xs[1].y + b[2] * (double)xs[2].y;
        a[2] = b[0] * (double)xs[0].z + b[1] * (double)xs[1].z + b[2] * (double)xs[2].z;
        const double C = sdf_body(r, a);
        if (!(C > 0)) {
            const float4 nf = c.n[slot];
            const double nn[3] = {(double)nf.x, (double)nf.y, (double)nf.z};
            double L = 0;
            for (int i = 0; i < 3; i++) {
                const double gx = b[i] * nn[0], gy = b[i] * nn[1], gz = b[i] * nn[2];
                L += (double)fabsf(xs[i].w) * (gx * gx + gy * gy + gz * gz);
            }
            const double dl = -C / L;
            if (!isfinite(dl)) {
                atomicAdd(&flags->nonfinite, 1ull);
            } else {
                lam = (float)((double)lam + dl);
                for (int i = 0; i < 3; i++) {
                    const double w = (double)fabsf(xs[i].w);
                    const double d0 = w * (b[i] * nn[0]) * dl, d1 = w * (b[i] * nn[1]) * dl,
                                 d2 = w * (b[i] * nn[2]) * dl;
                    if (jacobi) {
                        float4 a4 = dx[vi[i]];
                        a4.x += (float)d0; a4.y += (float)d1; a4.z += (float)d2;
                        dx[vi[i]] = a4;
                    } else {
                        x[vi[i]] = make_float4((float)((double)xs[i].x + d0), (float)((double)xs[i].y + d1),
                                               (float)((double)xs[i].z + d2), xs[i].w);
                    }
                }
                const float4 pf = c.p[slot];
                const double pt[3] = {(double)pf.x, (double)pf.y, (double)pf.z};
                double dp[3], dq[4];
                rigid_contact_delta(r, dl, pt, nn, dp, dq);
                if (jacobi) {
                    for (int k = 0; k < 3; k++) r[RB_ACC + k] += dp[k];
                    for (int k = 0; k < 4; k++) r[RB_ACC + 3 + k] += dq[k];
                } else {
                    for (int k = 0; k < 3; k++) r[RB_P + k] = r[RB_P + k] + dp[k];
                    for (int k = 0; k < 4; k++) r[RB_Q + k] = r[RB_Q + k] + dq[k];
                }
            }
        }
        c.lam[slot] = lam;
    }
    if (jacobi)
        for (int i = 0; i < nb; i++) {
            double* r = rb + (size_t)i * kRigidRec;
            for (int k = 0; k < 3; k++) r[RB_P + k] += r[RB_ACC + k];
            for (int k = 0; k < 4; k++) r[RB_Q + k] += r[RB_ACC + 3 + k];
        }
}

// RigidObject::update (src/simobject/RigidObject.cpp:41-60)
__global__ void k_rigid_update(double* __restrict__ rb, int nb, double dt, double g) {
    pdl_wait_then_release();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb) return;
    double* r = rb + (size_t)i * kRigidRec;
    const double m = r[RB_M];
    const double f[3] = {0.0, 0.0, -m * g};
    for (int k = 0; k < 3; k++) r[RB_V + k] = r[RB_V + k] + dt * f[k] / m;
    for (int k = 0; k < 3; k++) r[RB_P + k] = r[RB_P + k] + dt * r[RB_V + k];
    double qi[4], wb[3], Iw[3], cr[3], w[3];
    dquat_inverse(r + RB_Q, qi);
    dquat_rotate(r + RB_W, qi, wb);
    for (int k = 0; k < 3; k++) Iw[k] = r[RB_I + k] * wb[k];
    dcross(wb, Iw, cr);
    for (int k = 0; k < 3; k++) wb[k] = wb[k] + dt * r[RB_II + k] * (0.0 - cr[k]);
    dquat_rotate(wb, r + RB_Q, w);
    for (int k = 0; k < 3; k++) r[RB_W + k] = w[k];
    const double w4[4] = {w[0], w[1], w[2], 0.0};
    double dq[4];
    dquat_mult(w4, r + RB_Q, dq);
    double q[4];
    for (int k = 0; k < 4; k++) q[k] = r[RB_Q + k] + 0.5 * dt * dq[k];
    const double nq = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
    for (int k = 0; k < 4; k++) r[RB_Q + k] = q[k] / nq;
}

// RigidObject::velocityUpdate (src/simobject/RigidObject.cpp:62-77)
__global__ void k_rigid_velocity(double* __restrict__ rb, int nb, double dt) {
    pdl_wait_then_release();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb) return;
    double* r = rb + (size_t)i * kRigidRec;
    for (int k = 0; k < 3; k++) r[RB_V + k] = (r[RB_P + k] - r[RB_PP + k]) / dt;
    double qi[4], dq[4];
    dquat_inverse(r + RB_QP, qi);
    dquat_mult(r + RB_Q, qi, dq);
    const double sg = dq[3] < 0 ? -1.0 : 1.0;
    for (int k = 0; k < 3; k++) r[RB_W + k] = sg * (2 / dt * dq[k]);
    for (int k = 0; k < 3; k++) r[RB_PP + k] = r[RB_P + k];
    for (int k = 0; k < 4; k++) r[RB_QP + k] = r[RB_Q + k];
}

}  // namespace

void launch_rigid_sync_table(const Launch& s, const double* rb, int nb, float4* table) {
    if (nb > 0) go(k_rigid_sync_table, nblk(nb, 32), 32, s, rb, nb, table);
}

void launch_rigid_compact(const Launch& s, const ContactArrays& c, int* list, int* count) {
    go(k_rigid_compact, 1, kCompactThreads, s, c, list, count);
}

void launch_rigid_contacts(const Launch& s, const ContactArrays& c, const int* list, const int* count,
                           const float4* table, const int* face_inst, double* rb, int nb, float4* x, float4* dx,
                           bool jacobi, bool first, Flags* flags) {
    if (nb > 0) go(k_rigid_contacts, 1, 32, s, c, list, count, table, face_inst, rb, nb, x, dx, jacobi, first, flags);
}

void launch_rigid_update(const Launch& s, double* rb, int nb, double dt, double g) {
    if (nb > 0) go(k_rigid_update, nblk(nb, 32), 32, s, rb, nb, dt, g);
}

void launch_rigid_velocity(const Launch& s, double* rb, int nb, double dt) {
    if (nb > 0) go(k_rigid_velocity, nblk(nb, 32), 32, s, rb, nb, dt);
}

}  // namespace xg
