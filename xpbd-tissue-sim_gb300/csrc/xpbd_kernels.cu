// sm_103a kernels of the XPBD substep: prediction, Stable-Neo-Hookean
// tetrahedral projection (combined 2x2 and separate scalar forms), Jacobi
// scatter/apply, coloured Gauss-Seidel sweeps, SDF sphere collision detection
// and projection, fixed-vertex reset + velocity update, and FP64-finished
// residual/energy reductions.
//
// Semantics follow the reference's CPU path:
//   projection   src/solver/xpbd_projector/CombinedNeohookeanConstraintProjector.cpp:98-179
//                include/solver/xpbd_projector/ConstraintProjector.hpp:111-172
//   constraints  include/solver/constraint/{Hydrostatic,Deviatoric}Constraint.hpp
//   Jacobi       include/solver/xpbd_solver/XPBDJacobiSolver.hpp:79-114 (plain sum)
//   predict      src/simobject/XPBDMeshObject.cpp:446-470
//   fixed/vel    src/simobject/XPBDMeshObject.cpp:497-535
//   collisions   src/collision/CollisionScene.cpp:171-214,253-283
//                src/solver/constraint/StaticDeformableCollisionConstraint.cpp:20-49
// Every kernel is memory-bound; see the HBM layout in xpbd_kernels.cuh.
#include <cuda_runtime.h>

#include <utility>

#include "xpbd_kernels.cuh"

namespace xg {

namespace {

constexpr float kDegenerateJ = 1e-3f;  // |det F| below this takes the FP64 path

// Programmatic dependent launch: a kernel may start while its predecessor on
// the stream still runs; it must wait before touching anything the
// predecessor writes. Dependents are released only after this kernel's own
// wait, so a pre-wait prologue overlaps at most the direct predecessor.
__device__ __forceinline__ void pdl_wait_then_release() {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 900
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
#endif
}

// ---- TMA (bulk async copy) + mbarrier helpers ----
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// 1-D bulk copy global -> shared; both addresses 16-byte aligned, bytes a
// multiple of 16; completion is counted on the mbarrier.
__device__ __forceinline__ void tma_load_1d(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait for phase `parity` of the barrier: false after `limit` tries.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity, unsigned limit) {
    for (unsigned i = 0; i < limit; i++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

constexpr unsigned kWaitLimit = 1u << 20;

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Fixed-order block sum: FP32 inside a warp, FP64 across warps.
__device__ __forceinline__ void block_sum_store(float v, double* slot) {
    __shared__ double sw[32];
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) sw[wid] = (double)v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        const int nw = (blockDim.x + 31) >> 5;
        for (int i = 0; i < nw; i++) s += sw[i];
        *slot = s;
    }
}

__device__ __forceinline__ void add_vec4(float4* addr, float a, float b, float c) {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 900
    atomicAdd(addr, make_float4(a, b, c, 0.f));  // one 16-byte vector reduction at L2
#else
    atomicAdd(&addr->x, a);
    atomicAdd(&addr->y, b);
    atomicAdd(&addr->z, c);
#endif
}

// ---------------------------------------------------------------------------
// Per-tet math, templated on the arithmetic type (float fast path, double for
// near-degenerate elements).
// ---------------------------------------------------------------------------
template <typename R>
struct TetState {
    R p[4][3];
    R w[4];
    R q[9];  // Q column-major: q[3c + r] = Q(r, c)
    R atd, ath, gam;
};

template <typename R>
__device__ __forceinline__ R dev_log(R v) { return log(v); }
template <>
__device__ __forceinline__ float dev_log<float>(float v) { return logf(v); }
template <typename R>
__device__ __forceinline__ R dev_sqrt(R v) { return sqrt(v); }
template <>
__device__ __forceinline__ float dev_sqrt<float>(float v) { return sqrtf(v); }

// F = Ds Q (ElementConstraint.hpp:78-119), its Frobenius norm (C_dev) and det.
template <typename R>
__device__ __forceinline__ void tet_F(const TetState<R>& s, R F[9]) {
    R X[9];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int k = 0; k < 3; k++) X[3 * i + k] = s.p[i][k] - s.p[3][k];
#pragma unroll
    for (int c = 0; c < 3; c++)
#pragma unroll
        for (int k = 0; k < 3; k++)
            F[3 * c + k] = X[k] * s.q[3 * c + 0] + X[3 + k] * s.q[3 * c + 1] + X[6 + k] * s.q[3 * c + 2];
}

template <typename R>
__device__ __forceinline__ R tet_detF(const R F[9]) {
    return F[0] * F[4] * F[8] - F[0] * F[7] * F[5] - F[3] * F[1] * F[8] + F[3] * F[7] * F[2] + F[6] * F[1] * F[5] -
           F[6] * F[4] * F[2];
}

// Values and gradients of both constraints (HydrostaticConstraint.hpp:123-221,
// DeviatoricConstraint.hpp:112-152). gd/gh hold vertices 0..2; vertex 3 is
// minus their sum.
template <typename R>
__device__ __forceinline__ void tet_eval(const TetState<R>& s, R& Cd, R& Ch, R gd[9], R gh[9], R& J) {
    R F[9];
    tet_F(s, F);
    R ss = 0;
#pragma unroll
    for (int i = 0; i < 9; i++) ss += F[i] * F[i];
    Cd = dev_sqrt(ss);
    const R invC = R(1) / Cd;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int k = 0; k < 3; k++)
            gd[3 * i + k] = invC * (F[k] * s.q[i] + F[3 + k] * s.q[3 + i] + F[6 + k] * s.q[6 + i]);
    J = tet_detF(F);
    R fac;
    if (J >= R(1)) {
        Ch = -s.gam + dev_log(J);
        fac = R(1) / J;
    } else {
        const R d = J - R(1);
        Ch = -s.gam + d - d * d / R(2) + d * d * d / R(3);
        fac = R(1) - d + d * d;
    }
    R Fc[9];
    Fc[0] = F[4] * F[8] - F[5] * F[7]; Fc[1] = F[5] * F[6] - F[3] * F[8]; Fc[2] = F[3] * F[7] - F[4] * F[6];
    Fc[3] = F[7] * F[2] - F[8] * F[1]; Fc[4] = F[8] * F[0] - F[6] * F[2]; Fc[5] = F[6] * F[1] - F[7] * F[0];
    Fc[6] = F[1] * F[5] - F[2] * F[4]; Fc[7] = F[2] * F[3] - F[0] * F[5]; Fc[8] = F[0] * F[4] - F[1] * F[3];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int k = 0; k < 3; k++)
            gh[3 * i + k] = fac * (Fc[k] * s.q[i] + Fc[3 + k] * s.q[3 + i] + Fc[6 + k] * s.q[6 + i]);
}

__device__ __forceinline__ float dot3(const float* a, const float* b) {
    return fmaf(a[0], b[0], fmaf(a[1], b[1], a[2] * b[2]));
}

// FP32 fast path of the combined 2x2 projection (same contract as
// tet_project_combined below), with a shorter dependency chain:
// - the gradients are formed unscaled, G_i = F q_i and H_i = cof(F) q_i (q_i
//   the rows of Q, q_3 = -q_0 - q_1 - q_2), so they do not wait for 1/||F||
//   (rsqrt) or the hydrostatic factor; both scales enter the 2x2 system and
//   the update as scalars: grad C_dev,i = G_i / ||F||, grad C_hyd,i = fac H_i
//   (DeviatoricConstraint.hpp:112-152, HydrostaticConstraint.hpp:123-221);
// - tree-shaped sums, 1/||F|| from rsqrt, 1/J and 1/det from the hardware
//   reciprocal; det F from the cofactors the gradient uses.
// Results differ from tet_project_combined only by FP32 rounding (a few ulp);
// near-degenerate elements never use it.
__device__ __forceinline__ void tet_project_combined_fast(const TetState<float>& s, float lam0, float lam1, float& r0,
                                                          float& r1, float& dl0, float& dl1, float d[4][3], float& J) {
    float F[9];
    tet_F(s, F);
    const float ss = ((fmaf(F[0], F[0], F[1] * F[1]) + fmaf(F[2], F[2], F[3] * F[3])) +
                      (fmaf(F[4], F[4], F[5] * F[5]) + fmaf(F[6], F[6], F[7] * F[7]))) + F[8] * F[8];
    const float invC = rsqrtf(ss);
    const float Cd = ss * invC;
    float Fc[9];
    Fc[0] = F[4] * F[8] - F[5] * F[7]; Fc[1] = F[5] * F[6] - F[3] * F[8]; Fc[2] = F[3] * F[7] - F[4] * F[6];
    Fc[3] = F[7] * F[2] - F[8] * F[1]; Fc[4] = F[8] * F[0] - F[6] * F[2]; Fc[5] = F[6] * F[1] - F[7] * F[0];
    Fc[6] = F[1] * F[5] - F[2] * F[4]; Fc[7] = F[2] * F[3] - F[0] * F[5]; Fc[8] = F[0] * F[4] - F[1] * F[3];
    J = fmaf(F[0], Fc[0], fmaf(F[1], Fc[1], F[2] * Fc[2]));
    float Ch, fac;
    if (J >= 1.f) {
        Ch = -s.gam + logf(J);
        fac = __frcp_rn(J);
    } else {
        const float dd = J - 1.f;
        Ch = -s.gam + dd - dd * dd * 0.5f + dd * dd * dd * (1.f / 3.f);
        fac = fmaf(dd, dd, 1.f - dd);
    }
    float G[12], H[12];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int k = 0; k < 3; k++) {
            G[3 * i + k] = fmaf(F[k], s.q[i], fmaf(F[3 + k], s.q[3 + i], F[6 + k] * s.q[6 + i]));
            H[3 * i + k] = fmaf(Fc[k], s.q[i], fmaf(Fc[3 + k], s.q[3 + i], Fc[6 + k] * s.q[6 + i]));
        }
#pragma unroll
    for (int k = 0; k < 3; k++) {
        G[9 + k] = -(G[k] + G[3 + k]) - G[6 + k];
        H[9 + k] = -(H[k] + H[3 + k]) - H[6 + k];
    }
    float gg[4], gh[4], hh[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        gg[i] = dot3(G + 3 * i, G + 3 * i);
        gh[i] = dot3(G + 3 * i, H + 3 * i);
        hh[i] = dot3(H + 3 * i, H + 3 * i);
    }
    const float sgg = fmaf(s.w[0], gg[0], s.w[1] * gg[1]) + fmaf(s.w[2], gg[2], s.w[3] * gg[3]);
    const float sgh = fmaf(s.w[0], gh[0], s.w[1] * gh[1]) + fmaf(s.w[2], gh[2], s.w[3] * gh[3]);
    const float shh = fmaf(s.w[0], hh[0], s.w[1] * hh[1]) + fmaf(s.w[2], hh[2], s.w[3] * hh[3]);
    const float L00 = fmaf(invC * invC, sgg, s.atd);
    const float L01 = (invC * fac) * sgh;
    const float L11 = fmaf(fac * fac, shh, s.ath);
    r0 = fmaf(s.atd, lam0, Cd);
    r1 = fmaf(s.ath, lam1, Ch);
    const float inv_det = __frcp_rn(fmaf(L00, L11, -L01 * L01));
    dl0 = fmaf(-r0, L11, r1 * L01) * inv_det;
    dl1 = fmaf(-r1, L00, r0 * L01) * inv_det;
    const float a = invC * dl0, b = fac * dl1;
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int k = 0; k < 3; k++) d[i][k] = s.w[i] * fmaf(G[3 * i + k], a, H[3 * i + k] * b);
}

// Combined 2x2 projection. Returns the pre-update residuals r = C + at*lam and
// the lambda increments; writes the 4 vertex updates to d[4][3].
template <typename R>
__device__ __forceinline__ void tet_project_combined(const TetState<R>& s, R lam0, R lam1, R& r0, R& r1, R& dl0,
                                                     R& dl1, R d[4][3], R& J) {
    R Cd, Ch, gd[9], gh[9];
    tet_eval(s, Cd, Ch, gd, gh, J);
    R gd3[3], gh3[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        gd3[k] = -gd[k] - gd[3 + k] - gd[6 + k];
        gh3[k] = -gh[k] - gh[3 + k] - gh[6 + k];
    }
    R L00 = s.atd, L01 = 0, L11 = s.ath;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const R* a = i < 3 ? gd + 3 * i : gd3;
        const R* b = i < 3 ? gh + 3 * i : gh3;
        L00 += s.w[i] * (a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
        L01 += s.w[i] * (a[0] * b[0] + a[1] * b[1] + a[2] * b[2]);
        L11 += s.w[i] * (b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
    }
    r0 = Cd + s.atd * lam0;
    r1 = Ch + s.ath * lam1;
    const R det = L00 * L11 - L01 * L01;
    dl0 = (-r0 * L11 + r1 * L01) / det;
    dl1 = (-r1 * L00 + r0 * L01) / det;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const R* a = i < 3 ? gd + 3 * i : gd3;
        const R* b = i < 3 ? gh + 3 * i : gh3;
#pragma unroll
        for (int k = 0; k < 3; k++) d[i][k] = s.w[i] * (a[k] * dl0 + b[k] * dl1);
    }
}

// Scalar projection of one element constraint (which = 0 dev, 1 hyd).
template <typename R>
__device__ __forceinline__ void tet_project_single(const TetState<R>& s, int which, R lam, R& r, R& dl, R d[4][3],
                                                   R& J) {
    R Cd, Ch, gd[9], gh[9];
    tet_eval(s, Cd, Ch, gd, gh, J);
    const R* g = which == 0 ? gd : gh;
    const R at = which == 0 ? s.atd : s.ath;
    const R C = which == 0 ? Cd : Ch;
    R g3[3];
#pragma unroll
    for (int k = 0; k < 3; k++) g3[k] = -g[k] - g[3 + k] - g[6 + k];
    R L = at;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const R* a = i < 3 ? g + 3 * i : g3;
        L += s.w[i] * (a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    }
    r = C + at * lam;
    dl = -r / L;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const R* a = i < 3 ? g + 3 * i : g3;
#pragma unroll
        for (int k = 0; k < 3; k++) d[i][k] = s.w[i] * a[k] * dl;
    }
}

// Static per-tet data (indices, Dm^-1, compliances): never written while the
// solver runs, so it may be loaded before the dependency wait.
__device__ __forceinline__ void load_tet_static(const TetArrays& t, int slot, int4& e, TetState<float>& s) {
    e = __ldg(t.idx + slot);
    const float4 a = __ldg(t.q0 + slot), b = __ldg(t.q1 + slot), c = __ldg(t.q2 + slot);
    s.q[0] = a.x; s.q[1] = a.y; s.q[2] = a.z; s.q[3] = a.w;
    s.q[4] = b.x; s.q[5] = b.y; s.q[6] = b.z; s.q[7] = b.w;
    s.q[8] = c.x; s.atd = c.y; s.ath = c.z; s.gam = c.w;
}

// A vertex moved by a projection's update. The adds are not contracted with
// the update's last multiply, so every Gauss-Seidel kernel variant rounds the
// same way and their results agree bit for bit.
__device__ __forceinline__ float4 moved(const float4& p, const float* d) {
    return make_float4(__fadd_rn(p.x, d[0]), __fadd_rn(p.y, d[1]), __fadd_rn(p.z, d[2]), p.w);
}

__device__ __forceinline__ void gather_tet(const float4* __restrict__ x, const int4& e, TetState<float>& s,
                                           float4 xp[4]) {
    xp[0] = x[e.x]; xp[1] = x[e.y]; xp[2] = x[e.z]; xp[3] = x[e.w];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        s.p[i][0] = xp[i].x; s.p[i][1] = xp[i].y; s.p[i][2] = xp[i].z;
        s.w[i] = fabsf(xp[i].w);
    }
}

// FP64 guard path for near-degenerate / inverted elements. Kept out of line
// so the FP32 path keeps its register budget; everything crosses the call by
// value (static tet data is re-read by slot) so no caller array needs an
// address.
struct Fp64Out {
    float r0, r1, dl0, dl1;
    float d[12];
};

__device__ __forceinline__ TetState<double> fp64_state(const TetArrays& t, int slot, float4 p0, float4 p1, float4 p2,
                                                       float4 p3) {
    TetState<double> s;
    const float4 ps[4] = {p0, p1, p2, p3};
    for (int i = 0; i < 4; i++) {
        s.p[i][0] = ps[i].x; s.p[i][1] = ps[i].y; s.p[i][2] = ps[i].z;
        s.w[i] = fabsf(ps[i].w);
    }
    const float4 a = __ldg(t.q0 + slot), b = __ldg(t.q1 + slot), c = __ldg(t.q2 + slot);
    s.q[0] = a.x; s.q[1] = a.y; s.q[2] = a.z; s.q[3] = a.w;
    s.q[4] = b.x; s.q[5] = b.y; s.q[6] = b.z; s.q[7] = b.w;
    s.q[8] = c.x; s.atd = c.y; s.ath = c.z; s.gam = c.w;
    return s;
}

__device__ __noinline__ Fp64Out project_combined_fp64(TetArrays t, int slot, float4 p0, float4 p1, float4 p2,
                                                      float4 p3, float lam0, float lam1) {
    const TetState<double> s = fp64_state(t, slot, p0, p1, p2, p3);
    double r0, r1, dl0, dl1, dd[4][3], J;
    tet_project_combined(s, (double)lam0, (double)lam1, r0, r1, dl0, dl1, dd, J);
    Fp64Out o;
    o.r0 = (float)r0; o.r1 = (float)r1; o.dl0 = (float)dl0; o.dl1 = (float)dl1;
    for (int i = 0; i < 4; i++)
        for (int k = 0; k < 3; k++) o.d[3 * i + k] = (float)dd[i][k];
    return o;
}

__device__ __noinline__ Fp64Out project_single_fp64(TetArrays t, int slot, float4 p0, float4 p1, float4 p2, float4 p3,
                                                    int which, float lam) {
    const TetState<double> s = fp64_state(t, slot, p0, p1, p2, p3);
    double rr, dl, dd[4][3], J;
    tet_project_single(s, which, (double)lam, rr, dl, dd, J);
    Fp64Out o;
    o.r0 = (float)rr; o.r1 = 0.f; o.dl0 = (float)dl; o.dl1 = 0.f;
    for (int i = 0; i < 4; i++)
        for (int k = 0; k < 3; k++) o.d[3 * i + k] = (float)dd[i][k];
    return o;
}

// One tet projection in the chosen constraint form. On return d holds the
// vertex updates, lam the updated multipliers and rsq the squared residual of
// the state the projection saw. Returns false when the update is non-finite
// (then nothing may be applied).
template <bool SEPARATE>
__device__ __forceinline__ bool project_one(const TetState<float>& s, const TetArrays& t, int slot, const float4 xp[4],
                                            float2& lam, float d[4][3], float& rsq, Flags* flags) {
    float J;
    if (!SEPARATE) {
        float r0, r1, dl0, dl1;
        tet_project_combined_fast(s, lam.x, lam.y, r0, r1, dl0, dl1, d, J);
        if (fabsf(J) < kDegenerateJ) {
            const Fp64Out o = project_combined_fp64(t, slot, xp[0], xp[1], xp[2], xp[3], lam.x, lam.y);
            r0 = o.r0; r1 = o.r1; dl0 = o.dl0; dl1 = o.dl1;
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int k = 0; k < 3; k++) d[i][k] = o.d[3 * i + k];
            atomicAdd(&flags->degenerate, 1ull);
        }
        rsq = r0 * r0 + r1 * r1;
        if (!(isfinite(dl0) && isfinite(dl1))) {
            atomicAdd(&flags->nonfinite, 1ull);
            return false;
        }
        lam.x += dl0;
        lam.y += dl1;
    } else {
        // Jacobi form of the separate configuration: Dev and Hyd both see the
        // same positions, their updates are summed.
        float r0, r1, dl0, dl1, d1[4][3];
        tet_project_single(s, 0, lam.x, r0, dl0, d, J);
        tet_project_single(s, 1, lam.y, r1, dl1, d1, J);
        if (fabsf(J) < kDegenerateJ) {
            const Fp64Out a = project_single_fp64(t, slot, xp[0], xp[1], xp[2], xp[3], 0, lam.x);
            const Fp64Out b = project_single_fp64(t, slot, xp[0], xp[1], xp[2], xp[3], 1, lam.y);
            r0 = a.r0; dl0 = a.dl0; r1 = b.r0; dl1 = b.dl0;
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    d[i][k] = a.d[3 * i + k];
                    d1[i][k] = b.d[3 * i + k];
                }
            atomicAdd(&flags->degenerate, 1ull);
        }
        rsq = r0 * r0 + r1 * r1;
        if (!(isfinite(dl0) && isfinite(dl1))) {
            atomicAdd(&flags->nonfinite, 1ull);
            return false;
        }
        lam.x += dl0;
        lam.y += dl1;
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
            for (int k = 0; k < 3; k++) d[i][k] += d1[i][k];
    }
    return true;
}

// ---------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------

__global__ void k_predict(float4* __restrict__ x, float4* __restrict__ prev, const float4* __restrict__ vel, int V,
                          float dt, float dz) {
    pdl_wait_then_release();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V) return;
    const float4 p = x[i];
    const float4 v = vel[i];
    prev[i] = p;
    x[i] = make_float4(p.x + dt * v.x, p.y + dt * v.y, (p.z + dt * v.z) + dz, p.w);
}

// 1st-order inertial move: no velocity term, gravity scaled by m / B per
// vertex (XPBDMeshObject.cpp:449-456)
__global__ void k_predict_first_order(float4* __restrict__ x, float4* __restrict__ prev, const float* __restrict__ gdz,
                                      int V) {
    pdl_wait_then_release();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V) return;
    const float4 p = x[i];
    prev[i] = p;
    x[i] = make_float4(p.x, p.y, p.z + __ldg(gdz + i), p.w);
}

__global__ void k_kinematic(float4* __restrict__ x, const int* __restrict__ idx, const float4* __restrict__ rest,
                            int n, float ox, float oy, float oz) {
    pdl_wait_then_release();
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int i = idx[j];
    const float4 r = rest[j];
    const float w = x[i].w;
    x[i] = make_float4(r.x + ox, r.y + oy, r.z + oz, w);
}

// Jacobi sweep: every tet reads the same x, its updates are summed into dx by
// 16-byte vector reductions (XPBDJacobiSolver.hpp:79-114, plain summation).
template <bool FIRST, bool SEPARATE, bool RES>
__global__ void __launch_bounds__(256) k_project_jacobi(TetArrays t, int T, const float4* __restrict__ x,
                                                        float4* __restrict__ dx, ResidualSink res, Flags* flags) {
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    float rsq = 0.f;
    int4 e;
    TetState<float> s;
    if (slot < T) load_tet_static(t, slot, e, s);
    pdl_wait_then_release();
    if (slot < T) {
        float4 xp[4];
        gather_tet(x, e, s, xp);
        float2 lam = FIRST ? make_float2(0.f, 0.f) : t.lam[slot];
        float d[4][3];
        if (project_one<SEPARATE>(s, t, slot, xp, lam, d, rsq, flags)) {
            add_vec4(dx + e.x, d[0][0], d[0][1], d[0][2]);
            add_vec4(dx + e.y, d[1][0], d[1][1], d[1][2]);
            add_vec4(dx + e.z, d[2][0], d[2][1], d[2][2]);
            add_vec4(dx + e.w, d[3][0], d[3][1], d[3][2]);
        }
        t.lam[slot] = lam;
    }
    if (RES) block_sum_store(rsq, res.partial + (size_t)res.row * res.stride + res.offset + blockIdx.x);
}

// Deterministic Jacobi variant, pass 1: per-tet updates to a [T][3] float4
// buffer (12 floats per tet).
template <bool FIRST, bool SEPARATE, bool RES>
__global__ void __launch_bounds__(256) k_project_jacobi_write(TetArrays t, int T, const float4* __restrict__ x,
                                                              float4* __restrict__ dxt, ResidualSink res,
                                                              Flags* flags) {
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    float rsq = 0.f;
    int4 e;
    TetState<float> s;
    if (slot < T) load_tet_static(t, slot, e, s);
    pdl_wait_then_release();
    if (slot < T) {
        float4 xp[4];
        gather_tet(x, e, s, xp);
        float2 lam = FIRST ? make_float2(0.f, 0.f) : t.lam[slot];
        float d[4][3];
        if (!project_one<SEPARATE>(s, t, slot, xp, lam, d, rsq, flags)) {
#pragma unroll
            for (int i = 0; i < 4; i++) d[i][0] = d[i][1] = d[i][2] = 0.f;
        }
        dxt[3 * (size_t)slot + 0] = make_float4(d[0][0], d[0][1], d[0][2], d[1][0]);
        dxt[3 * (size_t)slot + 1] = make_float4(d[1][1], d[1][2], d[2][0], d[2][1]);
        dxt[3 * (size_t)slot + 2] = make_float4(d[2][2], d[3][0], d[3][1], d[3][2]);
        t.lam[slot] = lam;
    }
    if (RES) block_sum_store(rsq, res.partial + (size_t)res.row * res.stride + res.offset + blockIdx.x);
}

// Fixed vertices go back to their previous position (XPBDMeshObject.cpp:497-503);
// with write_vel the velocity update v = (x - prev)/dt (XPBDMeshObject.cpp:507-535)
// is fused in.
__device__ __forceinline__ void finalize_vertex(float4* __restrict__ x, const float4* __restrict__ prev,
                                                float4* __restrict__ vel, int i, float4 xx, float dt,
                                                bool write_vel) {
    const float4 p = prev[i];
    if (p.w < 0.f) xx = p;
    x[i] = xx;
    if (write_vel) vel[i] = make_float4((xx.x - p.x) / dt, (xx.y - p.y) / dt, (xx.z - p.z) / dt, 0.f);
}

// Pass 2: each vertex sums its tets' updates in CSR (ascending tet) order.
template <bool FINAL>
__global__ void k_gather_apply(float4* __restrict__ x, const float* __restrict__ dxt, const int* __restrict__ off,
                               const int* __restrict__ ent, float4* __restrict__ dx, int V,
                               const float4* __restrict__ prev, float4* __restrict__ vel, float dt, bool write_vel) {
    pdl_wait_then_release();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V) return;
    float sx = 0.f, sy = 0.f, sz = 0.f;
    const int b = off[i], e = off[i + 1];
    for (int j = b; j < e; j++) {
        const int code = ent[j];  // slot * 4 + local vertex
        const float* p = dxt + 12 * (size_t)(code >> 2) + 3 * (code & 3);
        sx += p[0]; sy += p[1]; sz += p[2];
    }
    // contact updates arrive through dx
    const float4 dc = dx[i];
    dx[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 xx = x[i];
    xx.x += sx + dc.x; xx.y += sy + dc.y; xx.z += sz + dc.z;
    if (FINAL) finalize_vertex(x, prev, vel, i, xx, dt, write_vel);
    else x[i] = xx;
}

template <bool FINAL>
__global__ void k_apply(float4* __restrict__ x, float4* __restrict__ dx, int V, const float4* __restrict__ prev,
                        float4* __restrict__ vel, float dt, bool write_vel) {
    pdl_wait_then_release();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V) return;
    float4 xx = x[i];
    const float4 d = dx[i];
    xx.x += d.x; xx.y += d.y; xx.z += d.z;
    dx[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (FINAL) finalize_vertex(x, prev, vel, i, xx, dt, write_vel);
    else x[i] = xx;
}

// Coloured Gauss-Seidel over patches: a patch is a run of up to
// kMaxPatchTets consecutive tets on at most kMaxPatchVerts vertices. Patches of
// one colour share no vertex, so each thread owns one patch: it stages the
// patch's vertices in shared memory, projects the patch's tets in order on
// them, and writes the vertices back once. One launch per patch colour. A
// patch of one tet is plain per-tet colouring.
template <bool FIRST, int WHICH, int MINB>
__global__ void __launch_bounds__(kPatchBlock, MINB) k_project_patch(TetArrays t, PatchArrays pa, int pbegin, int pend,
                                                               float4* __restrict__ x, Flags* flags) {
    // the block's patches own the contiguous slot range [s0, s1): their static
    // tet records arrive by three bulk copies (q0, q1, q2) before the
    // dependency wait, costing no registers
    __shared__ __align__(128) float4 sq[3][kPatchBlock * kMaxPatchTets];
    __shared__ float4 sv[kMaxPatchVerts][kPatchBlock];
    __shared__ __align__(8) unsigned long long bar;
    __shared__ int s_first;
    const int tid = threadIdx.x;
    const int p0 = pbegin + blockIdx.x * kPatchBlock;
    const int p = p0 + tid;
    const bool active = p < pend;
    if (tid == 0) mbar_init(&bar, 1);
    __syncthreads();
    if (tid == 0) {
        const int plast = min(p0 + kPatchBlock - 1, pend - 1);
        const int4 m0 = __ldg(pa.meta + p0), m1 = __ldg(pa.meta + plast);
        const int s0 = m0.x, s1 = m1.x + (m1.y & 0xff);
        const unsigned bytes = (unsigned)(s1 - s0) * 16u;
        s_first = s0;
        mbar_arrive_expect_tx(&bar, 3u * bytes);
        tma_load_1d(sq[0], t.q0 + s0, bytes, &bar);
        tma_load_1d(sq[1], t.q1 + s0, bytes, &bar);
        tma_load_1d(sq[2], t.q2 + s0, bytes, &bar);
    }
    int4 meta = make_int4(0, 0, 0, 0), va = make_int4(0, 0, 0, 0), vb = make_int4(0, 0, 0, 0);
    int ntets = 0, nverts = 0;
    if (active) {
        meta = __ldg(pa.meta + p);
        va = __ldg(pa.verts + 2 * (size_t)p);
        vb = __ldg(pa.verts + 2 * (size_t)p + 1);
        ntets = meta.y & 0xff;
        nverts = meta.y >> 8;
    }
    pdl_wait_then_release();
    // one round trip: all vertex and multiplier loads are issued together
    const int vid[kMaxPatchVerts] = {va.x, va.y, va.z, va.w, vb.x, vb.y, vb.z, vb.w};
    float2 lams[kMaxPatchTets];
#pragma unroll
    for (int i = 0; i < kMaxPatchTets; i++)
        lams[i] = (!FIRST && i < ntets) ? t.lam[meta.x + i] : make_float2(0.f, 0.f);
#pragma unroll
    for (int k = 0; k < kMaxPatchVerts; k++)
        if (k < nverts) sv[k][tid] = x[vid[k]];
    __syncthreads();  // s_first visible
    const bool staged = mbar_wait_bounded(&bar, 0, kWaitLimit);
    if (!staged) {
        // the copies never completed: record it, give them a second bounded
        // chance to land before the block exits, and change nothing
        if (tid == 0) {
            atomicAdd(&flags->timeouts, 1ull);
            mbar_wait_bounded(&bar, 0, kWaitLimit);
        }
        return;
    }
    if (!active) return;
    const int base = meta.x - s_first;
    const unsigned long long loc = (unsigned long long)(unsigned)meta.z | ((unsigned long long)(unsigned)meta.w << 32);
#pragma unroll
    for (int i = 0; i < kMaxPatchTets; i++) {
        if (i >= ntets) break;
        const int slot = meta.x + i;
        TetState<float> st;
        {
            const float4 a = sq[0][base + i], b = sq[1][base + i], c = sq[2][base + i];
            st.q[0] = a.x; st.q[1] = a.y; st.q[2] = a.z; st.q[3] = a.w;
            st.q[4] = b.x; st.q[5] = b.y; st.q[6] = b.z; st.q[7] = b.w;
            st.q[8] = c.x; st.atd = c.y; st.ath = c.z; st.gam = c.w;
        }
        int l[4];
        float4 xp[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            l[j] = (int)((loc >> (12 * i + 3 * j)) & 7ull);
            xp[j] = sv[l[j]][tid];
            st.p[j][0] = xp[j].x; st.p[j][1] = xp[j].y; st.p[j][2] = xp[j].z;
            st.w[j] = fabsf(xp[j].w);
        }
        float2 lam = lams[i];
        float d[4][3];
        bool ok;
        if (WHICH == 2) {
            float rsq;
            ok = project_one<false>(st, t, slot, xp, lam, d, rsq, flags);
        } else {
            float J, r, dl;
            const float lw = WHICH == 0 ? lam.x : lam.y;
            tet_project_single(st, WHICH, lw, r, dl, d, J);
            if (fabsf(J) < kDegenerateJ) {
                const Fp64Out o = project_single_fp64(t, slot, xp[0], xp[1], xp[2], xp[3], WHICH, lw);
                r = o.r0; dl = o.dl0;
#pragma unroll
                for (int a = 0; a < 4; a++)
#pragma unroll
                    for (int k = 0; k < 3; k++) d[a][k] = o.d[3 * a + k];
                atomicAdd(&flags->degenerate, 1ull);
            }
            ok = isfinite(dl);
            if (!ok) atomicAdd(&flags->nonfinite, 1ull);
            else if (WHICH == 0) lam.x += dl;
            else lam.y += dl;
        }
        if (ok) {
#pragma unroll
            for (int j = 0; j < 4; j++)
                sv[l[j]][tid] = moved(xp[j], d[j]);
        }
        t.lam[slot] = lam;
    }
#pragma unroll
    for (int k = 0; k < kMaxPatchVerts; k++)
        if (k < nverts) x[vid[k]] = sv[k][tid];
}

// One lane per patch, static tet records prefetched into registers before the
// dependency wait (shortest prologue; for latency-bound sweeps).
template <bool FIRST, int WHICH>
__global__ void __launch_bounds__(kPatchBlock) k_project_patch_reg(TetArrays t, PatchArrays pa, int pbegin, int pend,
                                                               float4* __restrict__ x, Flags* flags) {
    __shared__ float4 sv[kMaxPatchVerts][kPatchBlock];
    const int tid = threadIdx.x;
    const int p = pbegin + blockIdx.x * kPatchBlock + tid;
    const bool active = p < pend;
    int4 meta = make_int4(0, 0, 0, 0), va = make_int4(0, 0, 0, 0), vb = make_int4(0, 0, 0, 0);
    TetState<float> st[kMaxPatchTets];
    int ntets = 0, nverts = 0;
    if (active) {
        meta = __ldg(pa.meta + p);
        va = __ldg(pa.verts + 2 * (size_t)p);
        vb = __ldg(pa.verts + 2 * (size_t)p + 1);
        ntets = meta.y & 0xff;
        nverts = meta.y >> 8;
        // static tet data does not depend on the predecessor: load it before the wait
#pragma unroll
        for (int i = 0; i < kMaxPatchTets; i++) {
            if (i < ntets) {
                int4 dummy;
                load_tet_static(t, meta.x + i, dummy, st[i]);
            }
        }
    }
    pdl_wait_then_release();
    if (!active) return;
    // one round trip: all vertex and multiplier loads are issued together
    const int vid[kMaxPatchVerts] = {va.x, va.y, va.z, va.w, vb.x, vb.y, vb.z, vb.w};
    float2 lams[kMaxPatchTets];
#pragma unroll
    for (int i = 0; i < kMaxPatchTets; i++)
        lams[i] = (!FIRST && i < ntets) ? t.lam[meta.x + i] : make_float2(0.f, 0.f);
#pragma unroll
    for (int k = 0; k < kMaxPatchVerts; k++)
        if (k < nverts) sv[k][tid] = x[vid[k]];
    const unsigned long long loc = (unsigned long long)(unsigned)meta.z | ((unsigned long long)(unsigned)meta.w << 32);
#pragma unroll
    for (int i = 0; i < kMaxPatchTets; i++) {
        if (i >= ntets) break;
        const int slot = meta.x + i;
        int l[4];
        float4 xp[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            l[j] = (int)((loc >> (12 * i + 3 * j)) & 7ull);
            xp[j] = sv[l[j]][tid];
            st[i].p[j][0] = xp[j].x; st[i].p[j][1] = xp[j].y; st[i].p[j][2] = xp[j].z;
            st[i].w[j] = fabsf(xp[j].w);
        }
        float2 lam = lams[i];
        float d[4][3];
        bool ok;
        if (WHICH == 2) {
            float rsq;
            ok = project_one<false>(st[i], t, slot, xp, lam, d, rsq, flags);
        } else {
            float J, r, dl;
            const float lw = WHICH == 0 ? lam.x : lam.y;
            tet_project_single(st[i], WHICH, lw, r, dl, d, J);
            if (fabsf(J) < kDegenerateJ) {
                const Fp64Out o = project_single_fp64(t, slot, xp[0], xp[1], xp[2], xp[3], WHICH, lw);
                r = o.r0; dl = o.dl0;
#pragma unroll
                for (int a = 0; a < 4; a++)
#pragma unroll
                    for (int k = 0; k < 3; k++) d[a][k] = o.d[3 * a + k];
                atomicAdd(&flags->degenerate, 1ull);
            }
            ok = isfinite(dl);
            if (!ok) atomicAdd(&flags->nonfinite, 1ull);
            else if (WHICH == 0) lam.x += dl;
            else lam.y += dl;
        }
        if (ok) {
#pragma unroll
            for (int j = 0; j < 4; j++)
                sv[l[j]][tid] = moved(xp[j], d[j]);
        }
        t.lam[slot] = lam;
    }
#pragma unroll
    for (int k = 0; k < kMaxPatchVerts; k++)
        if (k < nverts) x[vid[k]] = sv[k][tid];
}


// Static collision projection of one contact slot: C = n.(u x1 + v x2 + w x3 - p),
// skipped when C > 0, alpha = 0. Returns false when skipped.
__device__ __forceinline__ bool contact_update(const ContactArrays& c, int slot, const float4 xs[3], float d[3][3],
                                               float& lam) {
    const float4 b = c.bary[slot];
    const float4 p = c.p[slot];
    const float4 n = c.n[slot];
    const float a0 = b.x * xs[0].x + b.y * xs[1].x + b.z * xs[2].x;
    const float a1 = b.x * xs[0].y + b.y * xs[1].y + b.z * xs[2].y;
    const float a2 = b.x * xs[0].z + b.y * xs[1].z + b.z * xs[2].z;
    const float C = n.x * (a0 - p.x) + n.y * (a1 - p.y) + n.z * (a2 - p.z);
    if (C > 0.f) return false;
    const float bb[3] = {b.x, b.y, b.z};
    float L = 0.f;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const float gx = bb[i] * n.x, gy = bb[i] * n.y, gz = bb[i] * n.z;
        L += fabsf(xs[i].w) * (gx * gx + gy * gy + gz * gz);
    }
    const float dl = -C / L;
    if (!isfinite(dl)) return false;
    lam += dl;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const float wi = fabsf(xs[i].w);
        d[i][0] = wi * (bb[i] * n.x) * dl;
        d[i][1] = wi * (bb[i] * n.y) * dl;
        d[i][2] = wi * (bb[i] * n.z) * dl;
    }
    return true;
}

template <bool FIRST>
__global__ void k_contacts_jacobi(ContactArrays c, const float4* __restrict__ x, float4* __restrict__ dx) {
    pdl_wait_then_release();
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= c.S * c.F) return;
    if (c.bary[slot].w != 1.f) return;  // empty, or against a free rigid body
    const int f = slot % c.F;
    const int4 fv = c.faces[f];
    const float4 xs[3] = {x[fv.x], x[fv.y], x[fv.z]};
    float lam = FIRST ? 0.f : c.lam[slot];
    float d[3][3];
    if (contact_update(c, slot, xs, d, lam)) {
        add_vec4(dx + fv.x, d[0][0], d[0][1], d[0][2]);
        add_vec4(dx + fv.y, d[1][0], d[1][1], d[1][2]);
        add_vec4(dx + fv.z, d[2][0], d[2][1], d[2][2]);
    }
    c.lam[slot] = lam;
}

// Gauss-Seidel contacts of one face: its slots in order, positions updated in
// place (faces of one colour share no vertex)
__device__ __forceinline__ void contact_face_gs(const ContactArrays& c, int f, float4* __restrict__ x, bool first) {
    const int4 fv = c.faces[f];
    for (int s = 0; s < c.S; s++) {
        const int slot = s * c.F + f;
        if (c.bary[slot].w != 1.f) continue;  // empty, or against a free rigid body
        float4 xs[3] = {x[fv.x], x[fv.y], x[fv.z]};
        float lam = first ? 0.f : c.lam[slot];
        float d[3][3];
        if (contact_update(c, slot, xs, d, lam)) {
            x[fv.x] = make_float4(xs[0].x + d[0][0], xs[0].y + d[0][1], xs[0].z + d[0][2], xs[0].w);
            x[fv.y] = make_float4(xs[1].x + d[1][0], xs[1].y + d[1][1], xs[1].z + d[1][2], xs[1].w);
            x[fv.z] = make_float4(xs[2].x + d[2][0], xs[2].y + d[2][1], xs[2].z + d[2][2], xs[2].w);
        }
        c.lam[slot] = lam;
    }
}

// After a detection: per instance and face colour, the faces holding an
// active static contact, in face-list order. One block per instance; ifl
// lists the faces by (instance, colour, index) with ranges
// ifo_off[k * (ncol + 1) + colour]; act_faces reuses the same positions.
__global__ void __launch_bounds__(kContactListThreads) k_contact_lists(ContactArrays c, const int* __restrict__ ifl,
                                                                       const int* __restrict__ ifo_off, int ncol,
                                                                       int* __restrict__ act_faces,
                                                                       int* __restrict__ act_off) {
    __shared__ int warp_tot[kContactListThreads / 32];
    __shared__ int out;
    pdl_wait_then_release();
    const int k = blockIdx.x, tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int* off = ifo_off + (size_t)k * (ncol + 1);
    int* aoff = act_off + (size_t)k * (ncol + 1);
    if (tid == 0) out = off[0];
    __syncthreads();
    for (int col = 0; col < ncol; col++) {
        if (tid == 0) aoff[col] = out;
        for (int b0 = off[col]; b0 < off[col + 1]; b0 += kContactListThreads) {
            const int j = b0 + tid;
            bool hit = false;
            int f = 0;
            if (j < off[col + 1]) {
                f = ifl[j];
                for (int s = 0; s < c.S; s++) hit |= c.bary[s * c.F + f].w == 1.f;
            }
            const unsigned m = __ballot_sync(0xffffffffu, hit);
            if (lane == 0) warp_tot[wid] = __popc(m);
            __syncthreads();
            int o = out;
            for (int w = 0; w < wid; w++) o += warp_tot[w];
            if (hit) act_faces[o + __popc(m & ((1u << lane) - 1u))] = f;
            __syncthreads();
            if (tid == 0) {
                int t = 0;
                for (int w = 0; w < kContactListThreads / 32; w++) t += warp_tot[w];
                out += t;
            }
            __syncthreads();
        }
    }
    if (tid == 0) aoff[ncol] = out;
}

constexpr int kMaxListColours = 63;  // colour offsets staged in shared memory up to this many

// Gauss-Seidel contacts of every face colour in one launch: one block per
// instance (instances share no vertex), the colours in order with a block
// barrier between them (the faces of a colour share no vertex)
__global__ void __launch_bounds__(kContactListThreads) k_contacts_gs_lists(ContactArrays c,
                                                                           const int* __restrict__ act_faces,
                                                                           const int* __restrict__ act_off, int ncol,
                                                                           float4* __restrict__ x, bool first) {
    __shared__ int soff[kMaxListColours + 1];
    pdl_wait_then_release();
    const int* aoff = act_off + (size_t)blockIdx.x * (ncol + 1);
    const bool staged = ncol <= kMaxListColours;
    if (staged)
        for (int i = threadIdx.x; i <= ncol; i += blockDim.x) soff[i] = aoff[i];
    __syncthreads();
    for (int col = 0; col < ncol; col++) {
        const int lo = staged ? soff[col] : aoff[col], hi = staged ? soff[col + 1] : aoff[col + 1];
        if (lo == hi) continue;  // uniform: the bounds are the block's
        for (int j = lo + threadIdx.x; j < hi; j += blockDim.x) contact_face_gs(c, act_faces[j], x, first);
        __syncthreads();
    }
}

// ---- collision detection (one thread per (sphere slot, face)) ----
// SDF primitive of a fixed rigid object, three float4 per table entry:
// a = (position, kind: 0 sphere, 1 box, 2 cylinder, < 0 empty),
// q = orientation quaternion (x, y, z, w), d = radius | full size | (radius, height).
struct Prim {
    float4 a, q, d;
};

__device__ __forceinline__ Prim load_prim(const float4* __restrict__ table, size_t e) {
    return Prim{table[3 * e], table[3 * e + 1], table[3 * e + 2]};
}

// GeometryUtils::rotateVectorByQuat (src/utils/GeometryUtils.cpp:92-97)
__device__ __forceinline__ void quat_rotate(const float v[3], float qx, float qy, float qz, float qw, float o[3]) {
    const float ud = qx * v[0] + qy * v[1] + qz * v[2];
    const float s = 2.f * qw * qw - 1.f;
    const float cx = qy * v[2] - qz * v[1], cy = qz * v[0] - qx * v[2], cz = qx * v[1] - qy * v[0];
    o[0] = 2.f * ud * qx + s * v[0] + 2.f * qw * cx;
    o[1] = 2.f * ud * qy + s * v[1] + 2.f * qw * cy;
    o[2] = 2.f * ud * qz + s * v[2] + 2.f * qw * cz;
}

// RigidObject::globalToBody (src/simobject/RigidObject.cpp:94-97)
__device__ __forceinline__ void to_body(const Prim& P, float px, float py, float pz, float b[3]) {
    const float n2 = P.q.x * P.q.x + P.q.y * P.q.y + P.q.z * P.q.z + P.q.w * P.q.w;
    const float v[3] = {px - P.a.x, py - P.a.y, pz - P.a.z};
    quat_rotate(v, -P.q.x / n2, -P.q.y / n2, -P.q.z / n2, P.q.w / n2, b);
}

__device__ __forceinline__ void normalize3(float v[3]) {
    const float n2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    if (n2 > 0.f) {
        const float n = sqrtf(n2);
        v[0] /= n; v[1] /= n; v[2] /= n;
    }
}

// SphereSDF / BoxSDF / CylinderSDF::evaluate (src/geometry/*SDF.cpp)
__device__ __forceinline__ float sdf_prim(float px, float py, float pz, const Prim& P) {
    if (P.a.w == 0.f) {
        const float a = px - P.a.x, b = py - P.a.y, c = pz - P.a.z;
        return sqrtf(a * a + b * b + c * c) - P.d.x;
    }
    float b[3];
    to_body(P, px, py, pz, b);
    if (P.a.w == 1.f) {
        const float q0 = fabsf(b[0]) - 0.5f * P.d.x, q1 = fabsf(b[1]) - 0.5f * P.d.y, q2 = fabsf(b[2]) - 0.5f * P.d.z;
        const float m0 = fmaxf(q0, 0.f), m1 = fmaxf(q1, 0.f), m2 = fmaxf(q2, 0.f);
        return sqrtf(m0 * m0 + m1 * m1 + m2 * m2) + fminf(fmaxf(fmaxf(q0, q1), q2), 0.f);
    }
    const float xy = sqrtf(b[0] * b[0] + b[1] * b[1]) - P.d.x;
    const float z = fabsf(b[2]) - 0.5f * P.d.y;
    const float ox = fmaxf(xy, 0.f), oz = fmaxf(z, 0.f);
    return sqrtf(ox * ox + oz * oz) + fminf(fmaxf(xy, z), 0.f);
}

// ...::gradient; a zero vector stays zero when normalised (Eigen)
__device__ __forceinline__ void grad_prim(float px, float py, float pz, const Prim& P, float g[3]) {
    if (P.a.w == 0.f) {
        const float a = px - P.a.x, b = py - P.a.y, c = pz - P.a.z;
        const float n2 = a * a + b * b + c * c;
        if (n2 > 0.f) {
            const float n = sqrtf(n2);
            g[0] = a / n; g[1] = b / n; g[2] = c / n;
        } else {
            g[0] = a; g[1] = b; g[2] = c;
        }
        return;
    }
    float b[3], go[3], gi[3];
    to_body(P, px, py, pz, b);
    if (P.a.w == 1.f) {
        const float dd[3] = {P.d.x, P.d.y, P.d.z};
        float q[3];
#pragma unroll
        for (int k = 0; k < 3; k++) q[k] = fabsf(b[k]) - dd[k] / 2.f;
        const float md = fminf(fmaxf(fmaxf(q[0], q[1]), q[2]), 0.f);
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const float sg = b[k] > 0.f ? 1.f : -1.f;
            go[k] = sg * fmaxf(q[k], 0.f);
            gi[k] = sg * (q[k] == md ? 1.f : 0.f);
        }
        normalize3(go);
    } else {
        const float xy = sqrtf(b[0] * b[0] + b[1] * b[1]) - P.d.x;
        const float z = fabsf(b[2]) - 0.5f * P.d.y;
        const float in = fminf(fmaxf(xy, z), 0.f);
        const float fo = fmaxf(xy, 0.f) > 0.f ? 1.f : 0.f, fz = fmaxf(z, 0.f) > 0.f ? 1.f : 0.f;
        go[0] = b[0] * fo; go[1] = b[1] * fo; go[2] = b[2] * fz;
        const float ix = in == xy ? 1.f : 0.f, iz = in == z ? 1.f : 0.f;
        gi[0] = b[0] * ix; gi[1] = b[1] * ix; gi[2] = b[2] * iz;
        normalize3(go);
        normalize3(gi);
    }
    const float sum[3] = {go[0] + gi[0], go[1] + gi[1], go[2] + gi[2]};
    quat_rotate(sum, P.q.x, P.q.y, P.q.z, P.q.w, g);
}

// one primitive's SDF value and gradient at points (test hook)
__global__ void k_prim_eval(const float4* __restrict__ prim, const float4* __restrict__ pts, int n,
                            float4* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Prim P = load_prim(prim, 0);
    const float4 p = pts[i];
    float g[3];
    grad_prim(p.x, p.y, p.z, P, g);
    out[i] = make_float4(sdf_prim(p.x, p.y, p.z, P), g[0], g[1], g[2]);
}

__global__ void k_detect(ContactArrays c, const float4* __restrict__ x, const float4* __restrict__ table,
                         const int* __restrict__ face_inst) {
    pdl_wait_then_release();
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= c.S * c.F) return;
    const int s = slot / c.F, f = slot - s * c.F;
    float4 bary = make_float4(0.f, 0.f, 0.f, 0.f);
    const Prim S = load_prim(table, (size_t)face_inst[f] * c.S + s);
    if (S.a.w >= 0.f) {
        const int4 fv = c.faces[f];
        const float4 q1 = x[fv.x], q2 = x[fv.y], q3 = x[fv.z];
        const float p1[3] = {q1.x, q1.y, q1.z}, p2[3] = {q2.x, q2.y, q2.z}, p3[3] = {q3.x, q3.y, q3.z};
        auto sq = [](const float* a, const float* b) {
            const float d0 = b[0] - a[0], d1 = b[1] - a[1], d2 = b[2] - a[2];
            return d0 * d0 + d1 * d1 + d2 * d2;
        };
        const float me = fmaxf(fmaxf(sq(p1, p2), sq(p1, p3)), sq(p2, p3));
        const float cd = sdf_prim((p1[0] + p2[0] + p3[0]) / 3.f, (p1[1] + p2[1] + p3[1]) / 3.f,
                                    (p1[2] + p2[2] + p3[2]) / 3.f, S);
        if (!(cd * cd > me)) {
            // Frank-Wolfe over the triangle, 32 iterations, from the vertex of
            // smallest SDF (CollisionScene.cpp:253-283)
            const float d1 = sdf_prim(p1[0], p1[1], p1[2], S), d2 = sdf_prim(p2[0], p2[1], p2[2], S),
                        d3 = sdf_prim(p3[0], p3[1], p3[2], S);
            const float* s0 = (d1 <= d2 && d1 <= d3) ? p1 : ((d2 <= d1 && d2 <= d3) ? p2 : p3);
            float xx[3] = {s0[0], s0[1], s0[2]};
            for (int i = 0; i < 32; i++) {
                const float alpha = 2.0f / (float)(i + 3);
                float g[3];
                grad_prim(xx[0], xx[1], xx[2], S, g);
                const float sg1 = p1[0] * g[0] + p1[1] * g[1] + p1[2] * g[2];
                const float sg2 = p2[0] * g[0] + p2[1] * g[1] + p2[2] * g[2];
                const float sg3 = p3[0] * g[0] + p3[1] * g[1] + p3[2] * g[2];
                const float* sv = (sg1 < sg2 && sg1 < sg3) ? p1 : ((sg2 < sg1 && sg2 < sg3) ? p2 : p3);
#pragma unroll
                for (int k = 0; k < 3; k++) xx[k] = xx[k] + alpha * (sv[k] - xx[k]);
            }
            const float dist = sdf_prim(xx[0], xx[1], xx[2], S);
            if ((double)dist <= 1e-4) {
                // barycentrics (GeometryUtils.cpp:6-23)
                float v0[3], v1[3], v2[3];
                for (int k = 0; k < 3; k++) { v0[k] = p2[k] - p1[k]; v1[k] = p3[k] - p1[k]; v2[k] = xx[k] - p1[k]; }
                auto dot = [](const float* a, const float* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; };
                const float d00 = dot(v0, v0), d01 = dot(v0, v1), d11 = dot(v1, v1), d20 = dot(v2, v0),
                            d21 = dot(v2, v1);
                const float den = d00 * d11 - d01 * d01;
                const float bv = (d11 * d20 - d01 * d21) / den;
                const float bw = (d00 * d21 - d01 * d20) / den;
                const float bu = 1.f - bv - bw;
                float g[3];
                grad_prim(xx[0], xx[1], xx[2], S, g);
                bary = make_float4(bu, bv, bw, S.d.w > 0.f ? 2.f : 1.f);
                c.p[slot] = make_float4(xx[0] - g[0] * dist, xx[1] - g[1] * dist, xx[2] - g[2] * dist, 0.f);
                c.n[slot] = make_float4(g[0], g[1], g[2], 0.f);
                c.lam[slot] = 0.f;
            }
        }
    }
    c.bary[slot] = bary;
}

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
constexpr int kCompactThreads = 1024;
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

// ---- self-collisions: detection (selfCollisionCheck, XPBDMeshObject.cpp:719-762)
// and DeformableDeformableCollisionConstraint ----

// exclusive scan of n ints in three launches (block sums, their scan, the
// blocks' scans with offsets); out[n] = total
constexpr int kScanThreads = 1024, kScanItems = 4, kScanChunk = kScanThreads * kScanItems;

__device__ __forceinline__ int block_excl_scan(int v, int* total) {
    __shared__ int wsum[kScanThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) wsum[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        int w = lane < kScanThreads / 32 ? wsum[lane] : 0;
        int wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += y;
        }
        if (lane < kScanThreads / 32) wsum[lane] = wi - w;  // exclusive warp offsets
    }
    __syncthreads();
    const int res = wsum[wid] + incl - v;
    if (total) {
        __shared__ int tot;
        if (threadIdx.x == kScanThreads - 1) tot = res + v;
        __syncthreads();
        *total = tot;
    }
    __syncthreads();
    return res;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_partials(const int* __restrict__ in, int n, int* __restrict__ part) {
    pdl_wait_then_release();
    const int base = blockIdx.x * kScanChunk + threadIdx.x * kScanItems;
    int s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; i++)
        if (base + i < n) s += in[base + i];
    int total = 0;
    block_excl_scan(s, &total);
    if (threadIdx.x == 0) part[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_part_single(int* __restrict__ part, int nb) {
    pdl_wait_then_release();
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int b0 = 0; b0 < nb; b0 += kScanThreads) {
        const int i = b0 + threadIdx.x;
        const int v = i < nb ? part[i] : 0;
        int total = 0;
        const int ex = block_excl_scan(v, &total);
        if (i < nb) part[i] = carry + ex;
        __syncthreads();
        if (threadIdx.x == 0) carry += total;
        __syncthreads();
    }
    if (threadIdx.x == 0) part[nb] = carry;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_apply(const int* __restrict__ in, int n,
                                                             const int* __restrict__ part, int* __restrict__ out,
                                                             int nb) {
    pdl_wait_then_release();
    const int base = blockIdx.x * kScanChunk + threadIdx.x * kScanItems;
    int v[kScanItems], s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; i++) {
        v[i] = base + i < n ? in[base + i] : 0;
        s += v[i];
    }
    int run = part[blockIdx.x] + block_excl_scan(s, nullptr);
#pragma unroll
    for (int i = 0; i < kScanItems; i++) {
        if (base + i < n) out[base + i] = run;
        run += v[i];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) out[n] = part[nb];
}

__device__ __forceinline__ int grid_cell1(float v, float o, float cell, int n) {
    float f = (v - o) / cell;
    f = fminf(fmaxf(f, 0.f), (float)(n - 1));  // NaN gives 0
    return (int)f;
}

// each tet in the cell of its centroid, or in the overflow list when its box
// is wider than a cell in some axis
__global__ void k_self_bin_count(SelfArrays a, SelfGrid g, const float4* __restrict__ x) {
    pdl_wait_then_release();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.T) return;
    const int4 e = a.tets[t];
    const float4 p0 = x[e.x], p1 = x[e.y], p2 = x[e.z], p3 = x[e.w];
    const float ex = fmaxf(fmaxf(p0.x, p1.x), fmaxf(p2.x, p3.x)) - fminf(fminf(p0.x, p1.x), fminf(p2.x, p3.x));
    const float ey = fmaxf(fmaxf(p0.y, p1.y), fmaxf(p2.y, p3.y)) - fminf(fminf(p0.y, p1.y), fminf(p2.y, p3.y));
    const float ez = fmaxf(fmaxf(p0.z, p1.z), fmaxf(p2.z, p3.z)) - fminf(fminf(p0.z, p1.z), fminf(p2.z, p3.z));
    int c = -1;
    if (ex <= g.cell && ey <= g.cell && ez <= g.cell) {
        const int cx = grid_cell1(0.25f * (p0.x + p1.x + p2.x + p3.x), g.ox, g.cell, g.nx);
        const int cy = grid_cell1(0.25f * (p0.y + p1.y + p2.y + p3.y), g.oy, g.cell, g.ny);
        const int cz = grid_cell1(0.25f * (p0.z + p1.z + p2.z + p3.z), g.oz, g.cell, g.nz);
        c = (cz * g.ny + cy) * g.nx + cx;
        atomicAdd(a.cell_count + c, 1);
    } else {
        a.overflow[atomicAdd(a.n_overflow, 1)] = t;
    }
    a.tet_cell[t] = c;
}

__global__ void k_self_bin_fill(SelfArrays a) {
    pdl_wait_then_release();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.T) return;
    const int c = a.tet_cell[t];
    if (c < 0) return;
    a.cell_tets[a.cell_off[c] + atomicAdd(a.cell_fill + c, 1)] = t;
}

// EmbreeTetMeshGeometry::isPointInTetrahedron (EmbreeTetMeshGeometry.cpp:20-47),
// float, with every product and sum rounded on its own (no contraction), as
// the host computes it
__device__ __forceinline__ bool same_side_f(const float* p, const float* a, const float* b, const float* c,
                                            const float* d) {
    const float ab0 = __fsub_rn(b[0], a[0]), ab1 = __fsub_rn(b[1], a[1]), ab2 = __fsub_rn(b[2], a[2]);
    const float ac0 = __fsub_rn(c[0], a[0]), ac1 = __fsub_rn(c[1], a[1]), ac2 = __fsub_rn(c[2], a[2]);
    const float n0 = __fsub_rn(__fmul_rn(ab1, ac2), __fmul_rn(ab2, ac1));
    const float n1 = __fsub_rn(__fmul_rn(ab2, ac0), __fmul_rn(ab0, ac2));
    const float n2 = __fsub_rn(__fmul_rn(ab0, ac1), __fmul_rn(ab1, ac0));
    const float sp = __fadd_rn(__fadd_rn(__fmul_rn(n0, __fsub_rn(p[0], a[0])), __fmul_rn(n1, __fsub_rn(p[1], a[1]))),
                               __fmul_rn(n2, __fsub_rn(p[2], a[2])));
    const float sd = __fadd_rn(__fadd_rn(__fmul_rn(n0, __fsub_rn(d[0], a[0])), __fmul_rn(n1, __fsub_rn(d[1], a[1]))),
                               __fmul_rn(n2, __fsub_rn(d[2], a[2])));
    return __fmul_rn(sp, sd) >= 0.f;
}

// EmbreeScene::tetMeshSelfCollisionQuery: the lowest-index tet holding the
// surface vertex among those that do not have it as a vertex
__global__ void k_self_query(SelfArrays a, SelfGrid g, const float4* __restrict__ x) {
    pdl_wait_then_release();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.n_surf) return;
    const int v = a.surf[k];
    const float4 pv = x[v];
    const float p[3] = {pv.x, pv.y, pv.z};
    int best = INT_MAX;
    auto test = [&](int t) {
        if (t >= best) return;
        const int4 e = a.tets[t];
        if (e.x == v || e.y == v || e.z == v || e.w == v) return;
        const float4 q0 = x[e.x], q1 = x[e.y], q2 = x[e.z], q3 = x[e.w];
        const float v0[3] = {q0.x, q0.y, q0.z}, v1[3] = {q1.x, q1.y, q1.z}, v2[3] = {q2.x, q2.y, q2.z},
                    v3[3] = {q3.x, q3.y, q3.z};
        if (same_side_f(p, v0, v1, v2, v3) && same_side_f(p, v0, v1, v3, v2) && same_side_f(p, v0, v2, v3, v1) &&
            same_side_f(p, v1, v2, v3, v0))
            best = t;
    };
    const int cx = grid_cell1(p[0], g.ox, g.cell, g.nx), cy = grid_cell1(p[1], g.oy, g.cell, g.ny),
              cz = grid_cell1(p[2], g.oz, g.cell, g.nz);
    for (int z = max(cz - 1, 0); z <= min(cz + 1, g.nz - 1); z++)
        for (int y = max(cy - 1, 0); y <= min(cy + 1, g.ny - 1); y++)
            for (int xx = max(cx - 1, 0); xx <= min(cx + 1, g.nx - 1); xx++) {
                const int c = (z * g.ny + y) * g.nx + xx;
                for (int i = a.cell_off[c]; i < a.cell_off[c + 1]; i++) test(a.cell_tets[i]);
            }
    const int no = *a.n_overflow;
    for (int i = 0; i < no; i++) test(a.overflow[i]);
    a.hit_tet[k] = best == INT_MAX ? -1 : best;
}

// the surface indices with a hit, ascending (one block)
__global__ void __launch_bounds__(kCompactThreads) k_self_compact(SelfArrays a) {
    __shared__ int warp_tot[kCompactThreads / 32];
    __shared__ int base;
    pdl_wait_then_release();
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    if (tid == 0) base = 0;
    __syncthreads();
    for (int b0 = 0; b0 < a.n_surf; b0 += kCompactThreads) {
        const int k = b0 + tid;
        const bool hit = k < a.n_surf && a.hit_tet[k] >= 0;
        const unsigned m = __ballot_sync(0xffffffffu, hit);
        if (lane == 0) warp_tot[wid] = __popc(m);
        __syncthreads();
        int off = base;
        for (int w = 0; w < wid; w++) off += warp_tot[w];
        if (hit) a.hit_list[off + __popc(m & ((1u << lane) - 1u))] = k;
        __syncthreads();
        if (tid == 0) {
            int t = 0;
            for (int w = 0; w < kCompactThreads / 32; w++) t += warp_tot[w];
            base += t;
        }
        __syncthreads();
    }
    if (tid == 0) *a.n_hits = base;
}

// Distance from p to triangle (a, b, c) in float: Ericson, Real-Time Collision
// Detection 5.1.5 (the method EmbreeMeshGeometry::_closestPointTriangle uses)
__device__ float point_triangle_distance_f(const float* p, const float* a, const float* b, const float* c) {
    auto dot = [](const float* u, const float* v) {
        return __fadd_rn(__fadd_rn(__fmul_rn(u[0], v[0]), __fmul_rn(u[1], v[1])), __fmul_rn(u[2], v[2]));
    };
    const float ab[3] = {__fsub_rn(b[0], a[0]), __fsub_rn(b[1], a[1]), __fsub_rn(b[2], a[2])};
    const float ac[3] = {__fsub_rn(c[0], a[0]), __fsub_rn(c[1], a[1]), __fsub_rn(c[2], a[2])};
    const float ap[3] = {__fsub_rn(p[0], a[0]), __fsub_rn(p[1], a[1]), __fsub_rn(p[2], a[2])};
    const float bp[3] = {__fsub_rn(p[0], b[0]), __fsub_rn(p[1], b[1]), __fsub_rn(p[2], b[2])};
    const float cp[3] = {__fsub_rn(p[0], c[0]), __fsub_rn(p[1], c[1]), __fsub_rn(p[2], c[2])};
    const float d1 = dot(ab, ap), d2 = dot(ac, ap), d3 = dot(ab, bp), d4 = dot(ac, bp), d5 = dot(ab, cp),
                d6 = dot(ac, cp);
    float o[3];
    if (d1 <= 0.f && d2 <= 0.f) {
        o[0] = a[0]; o[1] = a[1]; o[2] = a[2];
    } else if (d3 >= 0.f && d4 <= d3) {
        o[0] = b[0]; o[1] = b[1]; o[2] = b[2];
    } else if (d6 >= 0.f && d5 <= d6) {
        o[0] = c[0]; o[1] = c[1]; o[2] = c[2];
    } else {
        const float vc = __fsub_rn(__fmul_rn(d1, d4), __fmul_rn(d3, d2));
        const float vb = __fsub_rn(__fmul_rn(d5, d2), __fmul_rn(d1, d6));
        const float va = __fsub_rn(__fmul_rn(d3, d6), __fmul_rn(d5, d4));
        if (vc <= 0.f && d1 >= 0.f && d3 <= 0.f) {
            const float v = __fdiv_rn(d1, __fsub_rn(d1, d3));
            for (int k = 0; k < 3; k++) o[k] = __fadd_rn(a[k], __fmul_rn(v, ab[k]));
        } else if (vb <= 0.f && d2 >= 0.f && d6 <= 0.f) {
            const float v = __fdiv_rn(d2, __fsub_rn(d2, d6));
            for (int k = 0; k < 3; k++) o[k] = __fadd_rn(a[k], __fmul_rn(v, ac[k]));
        } else if (va <= 0.f && __fsub_rn(d4, d3) >= 0.f && __fsub_rn(d5, d6) >= 0.f) {
            const float v = __fdiv_rn(__fsub_rn(d4, d3), __fadd_rn(__fsub_rn(d4, d3), __fsub_rn(d5, d6)));
            for (int k = 0; k < 3; k++) o[k] = __fadd_rn(b[k], __fmul_rn(v, __fsub_rn(c[k], b[k])));
        } else {
            const float den = __fdiv_rn(1.f, __fadd_rn(__fadd_rn(va, vb), vc));
            const float v = __fmul_rn(vb, den), w = __fmul_rn(vc, den);
            for (int k = 0; k < 3; k++) o[k] = __fadd_rn(__fadd_rn(a[k], __fmul_rn(v, ab[k])), __fmul_rn(w, ac[k]));
        }
    }
    const float e0 = __fsub_rn(p[0], o[0]), e1 = __fsub_rn(p[1], o[1]), e2 = __fsub_rn(p[2], o[2]);
    return __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(e0, e0), __fmul_rn(e1, e1)), __fmul_rn(e2, e2)));
}

// DeformableMeshSDF::closestSurfaceFaceToPointInTet (DeformableMeshSDF.cpp:68-82),
// one warp per hit: the vertex mapped to rest space through the tet it is in
// (F = Ds Dm^-1 in double, none when |det F| < 1e-8), then the closest face of
// the rest surface (float; of equally close faces the lowest index)
__global__ void k_self_face(SelfArrays a, const float4* __restrict__ x, const int4* __restrict__ faces) {
    pdl_wait_then_release();
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= *a.n_hits) return;
    const int k = a.hit_list[w];
    const int v = a.surf[k], t = a.hit_tet[k];
    const int4 e = a.tets[t];
    const int ids[5] = {e.x, e.y, e.z, e.w, v};
    double xd[5][3];
    for (int i = 0; i < 5; i++) {
        const float4 q = x[ids[i]];
        xd[i][0] = q.x; xd[i][1] = q.y; xd[i][2] = q.z;
    }
    // F = Ds Q (column-major), as the host's compute_F
    const double* Q = a.Q + 9 * (size_t)t;
    double D[9], F[9];
    for (int i = 0; i < 3; i++)
        for (int r = 0; r < 3; r++) D[3 * i + r] = xd[i][r] - xd[3][r];
    for (int c = 0; c < 3; c++)
        for (int r = 0; r < 3; r++) F[3 * c + r] = D[r] * Q[3 * c] + D[3 + r] * Q[3 * c + 1] + D[6 + r] * Q[3 * c + 2];
    auto M = [&F](int r, int c) { return F[c * 3 + r]; };
    const double c00 = M(1, 1) * M(2, 2) - M(1, 2) * M(2, 1);
    const double c10 = M(1, 2) * M(2, 0) - M(1, 0) * M(2, 2);
    const double c20 = M(1, 0) * M(2, 1) - M(1, 1) * M(2, 0);
    const double det = M(0, 0) * c00 + M(0, 1) * c10 + M(0, 2) * c20;
    int face = -1;
    if (!(fabs(det) < 1e-8)) {
        const double inv = 1.0 / det;
        double Fi[9];
        Fi[0] = c00 * inv; Fi[1] = c10 * inv; Fi[2] = c20 * inv;
        Fi[3] = (M(0, 2) * M(2, 1) - M(0, 1) * M(2, 2)) * inv;
        Fi[4] = (M(0, 0) * M(2, 2) - M(0, 2) * M(2, 0)) * inv;
        Fi[5] = (M(0, 1) * M(2, 0) - M(0, 0) * M(2, 1)) * inv;
        Fi[6] = (M(0, 1) * M(1, 2) - M(0, 2) * M(1, 1)) * inv;
        Fi[7] = (M(0, 2) * M(1, 0) - M(0, 0) * M(1, 2)) * inv;
        Fi[8] = (M(0, 0) * M(1, 1) - M(0, 1) * M(1, 0)) * inv;
        const double rel[3] = {xd[4][0] - xd[3][0], xd[4][1] - xd[3][1], xd[4][2] - xd[3][2]};
        float pm[3];
        for (int r = 0; r < 3; r++)
            pm[r] = (float)(Fi[r] * rel[0] + Fi[3 + r] * rel[1] + Fi[6 + r] * rel[2] + a.X0[3 * (size_t)e.w + r]);
        float bd = INFINITY;
        int bf = INT_MAX;
        for (int f = lane; f < a.F; f += 32) {
            const int4 fv = faces[f];
            const float4 A = a.X0f[fv.x], B = a.X0f[fv.y], Cc = a.X0f[fv.z];
            const float pa[3] = {A.x, A.y, A.z}, pb[3] = {B.x, B.y, B.z}, pc[3] = {Cc.x, Cc.y, Cc.z};
            const float d = point_triangle_distance_f(pm, pa, pb, pc);
            if (d < bd) {
                bd = d;
                bf = f;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float od = __shfl_xor_sync(0xffffffffu, bd, o);
            const int of = __shfl_xor_sync(0xffffffffu, bf, o);
            if (od < bd || (od == bd && of < bf)) {
                bd = od;
                bf = of;
            }
        }
        face = bf == INT_MAX ? -1 : bf;
    }
    if (lane == 0) a.contact[w] = make_int2(v, face);
}

// DeformableDeformableCollisionConstraint::evaluate / gradient
// (DeformableDeformableCollisionConstraint.cpp): C = (q - p1).a/|a| + 1e-5,
// a = (p2 - p1) x (p3 - p1); the gradient as the reference writes it (the
// third face vertex's term uses q - p2). g: q, p1, p2, p3 x 3
__device__ float self_contact_eval(const float* q, const float* p1, const float* p2, const float* p3, float* g) {
    const float e1[3] = {p2[0] - p1[0], p2[1] - p1[1], p2[2] - p1[2]};
    const float e2[3] = {p3[0] - p1[0], p3[1] - p1[1], p3[2] - p1[2]};
    const float av[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
    const float an = sqrtf(av[0] * av[0] + av[1] * av[1] + av[2] * av[2]);
    const float u1[3] = {q[0] - p1[0], q[1] - p1[1], q[2] - p1[2]};
    const float u2[3] = {q[0] - p2[0], q[1] - p2[1], q[2] - p2[2]};
    const float C = (u1[0] * av[0] + u1[1] * av[1] + u1[2] * av[2]) / an + 1e-5f;
    const float an3 = an * an * an;
    float r1[3], r2[3];
    const float ad1 = av[0] * u1[0] + av[1] * u1[1] + av[2] * u1[2];
    const float ad2 = av[0] * u2[0] + av[1] * u2[1] + av[2] * u2[2];
    for (int k = 0; k < 3; k++) {
        r1[k] = u1[k] / an - av[k] * ad1 / an3;
        r2[k] = u2[k] / an - av[k] * ad2 / an3;
    }
    auto cross = [](const float* x, const float* y, float* r) {
        r[0] = x[1] * y[2] - x[2] * y[1];
        r[1] = x[2] * y[0] - x[0] * y[2];
        r[2] = x[0] * y[1] - x[1] * y[0];
    };
    float t[3];
    for (int k = 0; k < 3; k++) g[k] = av[k] / an;
    const float d32[3] = {p3[0] - p2[0], p3[1] - p2[1], p3[2] - p2[2]};
    cross(r1, d32, t);
    for (int k = 0; k < 3; k++) g[3 + k] = -av[k] / an + t[k];
    const float d13[3] = {p1[0] - p3[0], p1[1] - p3[1], p1[2] - p3[2]};
    cross(r1, d13, t);
    for (int k = 0; k < 3; k++) g[6 + k] = t[k];
    const float d21[3] = {p2[0] - p1[0], p2[1] - p1[1], p2[2] - p1[2]};
    cross(r2, d21, t);
    for (int k = 0; k < 3; k++) g[9 + k] = t[k];
    return C;
}

// ConstraintProjector::project (ConstraintProjector.hpp:111-172) of self
// contact j: skipped when C > 0; alpha~ = 1e-8/dt^2 (or /dt)
__device__ bool self_update(const SelfArrays& a, int j, const int4* __restrict__ faces, const float4* x, bool first,
                            float at, int ids[4], float4 xs[4], float d[4][3], Flags* flags) {
    const int2 ct = a.contact[j];
    if (ct.y < 0) return false;
    const int4 fv = faces[ct.y];
    ids[0] = ct.x; ids[1] = fv.x; ids[2] = fv.y; ids[3] = fv.z;
    float p[4][3];
    for (int i = 0; i < 4; i++) {
        xs[i] = x[ids[i]];
        p[i][0] = xs[i].x; p[i][1] = xs[i].y; p[i][2] = xs[i].z;
    }
    float g[12];
    const float C = self_contact_eval(p[0], p[1], p[2], p[3], g);
    float lam = first ? 0.f : a.lam[j];
    bool ok = false;
    if (!(C > 0.f)) {
        float L = at;
        for (int i = 0; i < 4; i++)
            L += fabsf(xs[i].w) * (g[3 * i] * g[3 * i] + g[3 * i + 1] * g[3 * i + 1] + g[3 * i + 2] * g[3 * i + 2]);
        const float dl = (-C - at * lam) / L;
        if (!isfinite(dl)) {
            atomicAdd(&flags->nonfinite, 1ull);
        } else {
            lam += dl;
            for (int i = 0; i < 4; i++)
                for (int k = 0; k < 3; k++) d[i][k] = fabsf(xs[i].w) * g[3 * i + k] * dl;
            ok = true;
        }
    }
    a.lam[j] = lam;
    return ok;
}

// Gauss-Seidel: the contacts in detection (vertex) order, one thread
__global__ void k_self_contacts_gs(SelfArrays a, const int4* __restrict__ faces, float4* __restrict__ x, bool first,
                                   float at, Flags* flags) {
    pdl_wait_then_release();
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    const int n = *a.n_hits;
    for (int j = 0; j < n; j++) {
        int ids[4];
        float4 xs[4];
        float d[4][3];
        if (!self_update(a, j, faces, x, first, at, ids, xs, d, flags)) continue;
        for (int i = 0; i < 4; i++) {
            const float4 c = x[ids[i]];  // a vertex may repeat: add to the current value
            x[ids[i]] = make_float4(c.x + d[i][0], c.y + d[i][1], c.z + d[i][2], c.w);
        }
    }
}

// Jacobi: every contact from the same positions, updates summed into dx
__global__ void k_self_contacts_jacobi(SelfArrays a, const int4* __restrict__ faces, const float4* __restrict__ x,
                                       float4* __restrict__ dx, bool first, float at, Flags* flags) {
    pdl_wait_then_release();
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= *a.n_hits) return;
    int ids[4];
    float4 xs[4];
    float d[4][3];
    if (!self_update(a, j, faces, x, first, at, ids, xs, d, flags)) return;
    for (int i = 0; i < 4; i++) add_vec4(dx + ids[i], d[i][0], d[i][1], d[i][2]);
}

// ---- host arrays the device addresses directly (coherent pageable memory
// on a Grace-Blackwell system): 3 values per vertex, converted here ----
// A block moves its 256 vertices' 3 x 256 values through shared memory, so the
// host side is read and written in whole 16-byte pieces covering full cache
// lines (when the block's run of the array is 16-byte aligned).
constexpr int kHostIoThreads = 256;

template <typename H>
__global__ void __launch_bounds__(kHostIoThreads) k_xyz_from_host(float4* __restrict__ x, const H* __restrict__ h,
                                                                  int V, bool keep_w) {
    __shared__ __align__(16) H buf[3 * kHostIoThreads];
    const int tid = threadIdx.x, v0 = blockIdx.x * kHostIoThreads;
    const int n = min(kHostIoThreads, V - v0), nv = 3 * n;
    const H* src = h + 3 * (size_t)v0;
    constexpr int kPer16 = 16 / (int)sizeof(H);
    if (((uintptr_t)src & 15) == 0) {
        for (int i = tid; i < nv / kPer16; i += kHostIoThreads)
            reinterpret_cast<uint4*>(buf)[i] = __ldcv(reinterpret_cast<const uint4*>(src) + i);
        for (int i = nv / kPer16 * kPer16 + tid; i < nv; i += kHostIoThreads) buf[i] = src[i];
    } else {
        for (int i = tid; i < nv; i += kHostIoThreads) buf[i] = src[i];
    }
    __syncthreads();
    if (tid < n) {
        const int i = v0 + tid;
        const float w = keep_w ? x[i].w : 0.f;  // inverse mass and fixed sign stay
        x[i] = make_float4((float)buf[3 * tid], (float)buf[3 * tid + 1], (float)buf[3 * tid + 2], w);
    }
}

template <typename H>
__global__ void __launch_bounds__(kHostIoThreads) k_xyz_to_host(H* __restrict__ h, const float4* __restrict__ x,
                                                                int V) {
    __shared__ __align__(16) H buf[3 * kHostIoThreads];
    const int tid = threadIdx.x, v0 = blockIdx.x * kHostIoThreads;
    const int n = min(kHostIoThreads, V - v0), nv = 3 * n;
    if (tid < n) {
        const float4 p = x[v0 + tid];
        buf[3 * tid] = (H)p.x;
        buf[3 * tid + 1] = (H)p.y;
        buf[3 * tid + 2] = (H)p.z;
    }
    __syncthreads();
    H* dst = h + 3 * (size_t)v0;
    constexpr int kPer16 = 16 / (int)sizeof(H);
    if (((uintptr_t)dst & 15) == 0) {
        for (int i = tid; i < nv / kPer16; i += kHostIoThreads)
            reinterpret_cast<uint4*>(dst)[i] = reinterpret_cast<const uint4*>(buf)[i];
        for (int i = nv / kPer16 * kPer16 + tid; i < nv; i += kHostIoThreads) dst[i] = buf[i];
    } else {
        for (int i = tid; i < nv; i += kHostIoThreads) dst[i] = buf[i];
    }
}

__global__ void k_finalize(float4* __restrict__ x, const float4* __restrict__ prev, float4* __restrict__ vel, int V,
                           float dt, bool write_vel) {
    pdl_wait_then_release();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V) return;
    finalize_vertex(x, prev, vel, i, x[i], dt, write_vel);
}

// v = (x - prev)/dt alone (XPBDMeshObject_::velocityUpdate)
__global__ void k_velocity(const float4* __restrict__ x, const float4* __restrict__ prev, float4* __restrict__ vel,
                           int V, float dt) {
    pdl_wait_then_release();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V) return;
    const float4 xx = x[i], p = prev[i];
    vel[i] = make_float4((xx.x - p.x) / dt, (xx.y - p.y) / dt, (xx.z - p.z) / dt, 0.f);
}

// Exact residual / energy at the current state. rvec (optional) receives the
// per-constraint residuals in the reference's order via the slot->tet map.
__global__ void __launch_bounds__(256) k_residual(TetArrays t, int T, const float4* __restrict__ x, bool separate,
                                                  const int* __restrict__ perm, float* __restrict__ rvec,
                                                  ResidualSink res, double* __restrict__ energy_partial, float dt2,
                                                  bool zero_lam) {
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    float rsq = 0.f, en = 0.f;
    int4 e;
    TetState<float> s;
    if (slot < T) load_tet_static(t, slot, e, s);
    pdl_wait_then_release();
    if (slot < T) {
        float4 xp[4];
        gather_tet(x, e, s, xp);
        const float2 lam = zero_lam ? make_float2(0.f, 0.f) : t.lam[slot];
        float Cd, Ch, gd[9], gh[9], J;
        tet_eval(s, Cd, Ch, gd, gh, J);
        const float r0 = Cd + s.atd * lam.x, r1 = Ch + s.ath * lam.y;
        rsq = r0 * r0 + r1 * r1;
        en = Cd * Cd / (s.atd * dt2) + Ch * Ch / (s.ath * dt2);
        if (rvec) {
            const int tt = perm ? perm[slot] : slot;
            if (!separate) { rvec[2 * (size_t)tt] = r0; rvec[2 * (size_t)tt + 1] = r1; }
            else { rvec[tt] = r0; rvec[(size_t)T + tt] = r1; }
        }
    }
    if (res.partial) block_sum_store(rsq, res.partial + (size_t)res.row * res.stride + res.offset + blockIdx.x);
    if (energy_partial) {
        __syncthreads();
        block_sum_store(en, energy_partial + blockIdx.x);
    }
}

// ---- dataflow Gauss-Seidel: all iterations and colours in one cooperative launch ----


__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void red_release_add_u32(unsigned* p, unsigned v) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// One warp per task, the warp's tasks in (iteration, colour, index) order. The
// smallest unfinished task always has its dependencies done and its warp at
// it (all blocks are co-resident), so the waits end; each is bounded anyway,
// and a wait that gives up sets abort_flag so that every other waiter leaves.
// A task's epoch counts lane releases (32 per iteration): every lane's
// red.release orders its own position and multiplier stores before it.
// The projections, their order and their arithmetic are those of
// k_project_patch_reg, so results equal the colour-by-colour launches.
template <bool FIRST_ZERO, int MINB>
__global__ void __launch_bounds__(kPatchBlock, MINB) k_sweep_dataflow(TetArrays t, PatchArrays pa, TaskArrays ta,
                                                                  int iters, float4* __restrict__ x, Flags* flags) {
    __shared__ float4 sv[kMaxPatchVerts][kPatchBlock];
    const int tid = threadIdx.x, lane = tid & 31;
    const int gw = (blockIdx.x * blockDim.x + tid) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    pdl_wait_then_release();
    for (int it = 0; it < iters; it++) {
        for (int j = gw; j < ta.ntasks; j += nw) {
            const int4 tk = __ldg(ta.task + j);
            const int p = tk.x + lane;
            const bool active = lane < tk.y;
            // static data first: it does not depend on other tasks
            int4 meta = make_int4(0, 0, 0, 0), va = make_int4(0, 0, 0, 0), vb = make_int4(0, 0, 0, 0);
            float4 r0[kMaxPatchTets], r1[kMaxPatchTets], r2[kMaxPatchTets];  // q0, q1, q2 records
            int ntets = 0, nverts = 0;
            if (active) {
                meta = __ldg(pa.meta + p);
                va = __ldg(pa.verts + 2 * (size_t)p);
                vb = __ldg(pa.verts + 2 * (size_t)p + 1);
                ntets = meta.y & 0xff;
                nverts = meta.y >> 8;
#pragma unroll
                for (int i = 0; i < kMaxPatchTets; i++) {
                    if (i < ntets) {
                        r0[i] = __ldg(t.q0 + meta.x + i);
                        r1[i] = __ldg(t.q1 + meta.x + i);
                        r2[i] = __ldg(t.q2 + meta.x + i);
                    }
                }
            }
            // dependencies: lower colours at it + 1, higher colours at it
            bool ok = true;
            const int d1 = __ldg(ta.dep_off + j + 1);
            for (int d = __ldg(ta.dep_off + j) + lane; d < d1 && ok; d += 32) {
                const int e = __ldg(ta.dep + d);
                const unsigned need = 32u * ((e & 1) ? (unsigned)it : (unsigned)it + 1u);
                const unsigned* f = ta.epoch + (e >> 1);
                unsigned n = 0;
                while (ld_acquire_u32(f) < need) {
                    if (++n > ta.poll_limit || ((n & 63) == 0 && *(volatile unsigned*)ta.abort_flag)) {
                        ok = false;
                        break;
                    }
                    __nanosleep(32);
                }
            }
            if (!__all_sync(0xffffffffu, ok)) {
                if (lane == 0) {
                    atomicExch(ta.abort_flag, 1u);
                    atomicAdd(&flags->timeouts, 1ull);
                }
                return;
            }
            __syncwarp();
            if (active) {
                const int vid[kMaxPatchVerts] = {va.x, va.y, va.z, va.w, vb.x, vb.y, vb.z, vb.w};
                float2 lams[kMaxPatchTets];
#pragma unroll
                for (int i = 0; i < kMaxPatchTets; i++)
                    lams[i] = (!(FIRST_ZERO && it == 0) && i < ntets) ? __ldcg(t.lam + meta.x + i)
                                                                      : make_float2(0.f, 0.f);
                // positions other warps wrote: read past L1
#pragma unroll
                for (int k = 0; k < kMaxPatchVerts; k++)
                    if (k < nverts) sv[k][tid] = __ldcg(x + vid[k]);
                const unsigned long long loc =
                    (unsigned long long)(unsigned)meta.z | ((unsigned long long)(unsigned)meta.w << 32);
#pragma unroll
                for (int i = 0; i < kMaxPatchTets; i++) {
                    if (i >= ntets) break;
                    const int slot = meta.x + i;
                    TetState<float> st;
                    st.q[0] = r0[i].x; st.q[1] = r0[i].y; st.q[2] = r0[i].z; st.q[3] = r0[i].w;
                    st.q[4] = r1[i].x; st.q[5] = r1[i].y; st.q[6] = r1[i].z; st.q[7] = r1[i].w;
                    st.q[8] = r2[i].x; st.atd = r2[i].y; st.ath = r2[i].z; st.gam = r2[i].w;
                    int l[4];
                    float4 xp[4];
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        l[q] = (int)((loc >> (12 * i + 3 * q)) & 7ull);
                        xp[q] = sv[l[q]][tid];
                        st.p[q][0] = xp[q].x; st.p[q][1] = xp[q].y; st.p[q][2] = xp[q].z;
                        st.w[q] = fabsf(xp[q].w);
                    }
                    float2 lam = lams[i];
                    float d[4][3], rsq;
                    if (project_one<false>(st, t, slot, xp, lam, d, rsq, flags)) {
#pragma unroll
                        for (int q = 0; q < 4; q++)
                            sv[l[q]][tid] = moved(xp[q], d[q]);
                    }
                    t.lam[slot] = lam;
                }
#pragma unroll
                for (int k = 0; k < kMaxPatchVerts; k++)
                    if (k < nverts) x[vid[k]] = sv[k][tid];
            }
            // each lane releases its own stores: the task's epoch counts lanes,
            // 32 per completed iteration
            red_release_add_u32(ta.epoch + j, 1u);
        }
    }
}

// Dataflow sweep with the task's static tet records staged in shared memory:
// lane 0 issues three bulk copies (q0, q1, q2 over the task's contiguous slot
// range) before the dependency wait; each warp owns its staging buffer and
// mbarrier. Same projections, order and arithmetic as k_sweep_dataflow.
constexpr int kFlowWarps = kPatchBlock / 32;
constexpr int kTaskSlots = kTaskPatches * kMaxPatchTets;

template <bool FIRST_ZERO>
__global__ void __launch_bounds__(kPatchBlock, 6) k_sweep_dataflow_staged(TetArrays t, PatchArrays pa, TaskArrays ta,
                                                                         int iters, float4* __restrict__ x,
                                                                         Flags* flags) {
    __shared__ __align__(128) float4 sq[kFlowWarps][3][kTaskSlots];
    __shared__ float4 sv[kMaxPatchVerts][kPatchBlock];
    __shared__ __align__(8) unsigned long long bar[kFlowWarps];
    const int tid = threadIdx.x, lane = tid & 31, wib = tid >> 5;
    const int gw = (blockIdx.x * blockDim.x + tid) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    if (lane == 0) mbar_init(&bar[wib], 1);
    __syncwarp();
    unsigned phase = 0;
    pdl_wait_then_release();
    for (int it = 0; it < iters; it++) {
        for (int j = gw; j < ta.ntasks; j += nw) {
            const int4 tk = __ldg(ta.task + j);
            if (lane == 0) {
                // the previous task's reads of sq are done (syncwarp below)
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                const unsigned bytes = (unsigned)tk.w * 16u;
                mbar_arrive_expect_tx(&bar[wib], 3u * bytes);
                tma_load_1d(sq[wib][0], t.q0 + tk.z, bytes, &bar[wib]);
                tma_load_1d(sq[wib][1], t.q1 + tk.z, bytes, &bar[wib]);
                tma_load_1d(sq[wib][2], t.q2 + tk.z, bytes, &bar[wib]);
            }
            const int p = tk.x + lane;
            const bool active = lane < tk.y;
            int4 meta = make_int4(0, 0, 0, 0), va = make_int4(0, 0, 0, 0), vb = make_int4(0, 0, 0, 0);
            int ntets = 0, nverts = 0;
            if (active) {
                meta = __ldg(pa.meta + p);
                va = __ldg(pa.verts + 2 * (size_t)p);
                vb = __ldg(pa.verts + 2 * (size_t)p + 1);
                ntets = meta.y & 0xff;
                nverts = meta.y >> 8;
            }
            bool ok = true;
            const int d1 = __ldg(ta.dep_off + j + 1);
            for (int d = __ldg(ta.dep_off + j) + lane; d < d1 && ok; d += 32) {
                const int e = __ldg(ta.dep + d);
                const unsigned need = (e & 1) ? (unsigned)it : (unsigned)it + 1u;
                const unsigned* f = ta.epoch + (e >> 1);
                unsigned n = 0;
                while (ld_acquire_u32(f) < need) {
                    if (++n > ta.poll_limit || ((n & 63) == 0 && *(volatile unsigned*)ta.abort_flag)) {
                        ok = false;
                        break;
                    }
                    __nanosleep(32);
                }
            }
            ok = __all_sync(0xffffffffu, ok) != 0;
            const int vid[kMaxPatchVerts] = {va.x, va.y, va.z, va.w, vb.x, vb.y, vb.z, vb.w};
            float2 lams[kMaxPatchTets];
            if (ok && active) {
#pragma unroll
                for (int i = 0; i < kMaxPatchTets; i++)
                    lams[i] = (!(FIRST_ZERO && it == 0) && i < ntets) ? __ldcg(t.lam + meta.x + i)
                                                                      : make_float2(0.f, 0.f);
#pragma unroll
                for (int k = 0; k < kMaxPatchVerts; k++)
                    if (k < nverts) sv[k][tid] = __ldcg(x + vid[k]);
            }
            // the copies land (or not) whatever happened above
            const bool staged = __all_sync(0xffffffffu, mbar_wait_bounded(&bar[wib], phase, kWaitLimit)) != 0;
            phase ^= 1u;
            if (!ok || !staged) {
                if (lane == 0) {
                    atomicExch(ta.abort_flag, 1u);
                    atomicAdd(&flags->timeouts, 1ull);
                    if (!staged) mbar_wait_bounded(&bar[wib], phase ^ 1u, kWaitLimit);
                }
                __syncwarp();
                return;
            }
            if (active) {
                const int base = meta.x - tk.z;
                const unsigned long long loc =
                    (unsigned long long)(unsigned)meta.z | ((unsigned long long)(unsigned)meta.w << 32);
#pragma unroll
                for (int i = 0; i < kMaxPatchTets; i++) {
                    if (i >= ntets) break;
                    const int slot = meta.x + i;
                    TetState<float> st;
                    {
                        const float4 a = sq[wib][0][base + i], b = sq[wib][1][base + i], c = sq[wib][2][base + i];
                        st.q[0] = a.x; st.q[1] = a.y; st.q[2] = a.z; st.q[3] = a.w;
                        st.q[4] = b.x; st.q[5] = b.y; st.q[6] = b.z; st.q[7] = b.w;
                        st.q[8] = c.x; st.atd = c.y; st.ath = c.z; st.gam = c.w;
                    }
                    int l[4];
                    float4 xp[4];
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        l[q] = (int)((loc >> (12 * i + 3 * q)) & 7ull);
                        xp[q] = sv[l[q]][tid];
                        st.p[q][0] = xp[q].x; st.p[q][1] = xp[q].y; st.p[q][2] = xp[q].z;
                        st.w[q] = fabsf(xp[q].w);
                    }
                    float2 lam = lams[i];
                    float d[4][3], rsq;
                    if (project_one<false>(st, t, slot, xp, lam, d, rsq, flags)) {
#pragma unroll
                        for (int q = 0; q < 4; q++) sv[l[q]][tid] = moved(xp[q], d[q]);
                    }
                    t.lam[slot] = lam;
                }
#pragma unroll
                for (int k = 0; k < kMaxPatchVerts; k++)
                    if (k < nverts) x[vid[k]] = sv[k][tid];
            }
            __threadfence();
            __syncwarp();
            if (lane == 0) st_release_u32(ta.epoch + j, (unsigned)it + 1u);
        }
    }
}

// ---- dataflow Gauss-Seidel on version-stamped vertices ----
// The sweep works on its own copy xv of the positions whose w word holds the
// vertex's version: how many patch projections have written it in this
// launch. In one iteration a vertex is written by each patch containing it,
// in colour order, so the patch of colour c reads vertex v once its version
// is it * deg(v) + pre(v, c) (deg: patches containing v, pre: those of a lower
// colour) -- the state the colour-by-colour launches give it. A writer stores
// position and version as one aligned 16-byte vector, so a reader that sees
// the version also sees the position written with it: the poll is the load,
// and no fence or task counter sits between two phases.

__device__ __forceinline__ float4 ld_relaxed_f4(const float4* p) {
    float4 v;
    asm volatile("ld.relaxed.gpu.global.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "l"(p)
                 : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed_f4(float4* p, float4 v) {
    asm volatile("st.relaxed.gpu.global.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(v.x), "f"(v.y), "f"(v.z),
                 "f"(v.w)
                 : "memory");
}

// Positions at version 0, and per patch the inverse masses of its 8 vertex
// slots (two float4: the sweep reads them with its other per-patch records).
__global__ void k_versions_in(float4* __restrict__ xv, float4* __restrict__ pw, const float4* __restrict__ x,
                              PatchArrays pa, int V, int P) {
    pdl_wait_then_release();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < V) {
        const float4 p = x[i];
        xv[i] = make_float4(p.x, p.y, p.z, __int_as_float(0));
    }
    if (i < P) {
        const int nv = __ldg(&pa.meta[i].y) >> 8;
        const int4 va = __ldg(pa.verts + 2 * (size_t)i), vb = __ldg(pa.verts + 2 * (size_t)i + 1);
        const int vid[kMaxPatchVerts] = {va.x, va.y, va.z, va.w, vb.x, vb.y, vb.z, vb.w};
        float w[kMaxPatchVerts];
#pragma unroll
        for (int k = 0; k < kMaxPatchVerts; k++) w[k] = k < nv ? x[vid[k]].w : 0.f;
        pw[2 * (size_t)i] = make_float4(w[0], w[1], w[2], w[3]);
        pw[2 * (size_t)i + 1] = make_float4(w[4], w[5], w[6], w[7]);
    }
}

__global__ void k_versions_out(float4* __restrict__ x, const float4* __restrict__ xv, int V) {
    pdl_wait_then_release();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V) return;
    const float4 p = xv[i];
    x[i] = make_float4(p.x, p.y, p.z, x[i].w);
}

// Warp w runs the w-th task of every colour (the task layout of
// k_sweep_dataflow). A lane's patch reads its vertices when their versions
// are due and writes them back one version later. The smallest unfinished
// task always has its vertices due and its warp at it (all blocks are
// co-resident), so the waits end; each is bounded anyway, and one that gives
// up sets abort_flag so that every other waiter leaves. Inverse masses come
// from the per-patch copy pw. Projections, order and arithmetic are those of
// k_project_patch_reg.
template <bool FIRST_ZERO, int MINB>
__global__ void __launch_bounds__(kFlowBlock, MINB)
    k_sweep_versioned(TetArrays t, PatchArrays pa, const int4* __restrict__ pver, TaskArrays ta, int iters,
                      const float4* __restrict__ pw, float4* __restrict__ xv, Flags* flags) {
    __shared__ float4 sv[kMaxPatchVerts][kFlowBlock];
    const int tid = threadIdx.x, lane = tid & 31;
    const int gw = (blockIdx.x * blockDim.x + tid) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    pdl_wait_then_release();
    for (int it = 0; it < iters; it++) {
        for (int j = gw; j < ta.ntasks; j += nw) {
            const int4 tk = __ldg(ta.task + j);
            const int p = tk.x + lane;
            bool ok = true;
            if (lane < tk.y) {
                const int4 meta = __ldg(pa.meta + p);
                const int4 va = __ldg(pa.verts + 2 * (size_t)p), vb = __ldg(pa.verts + 2 * (size_t)p + 1);
                const int4 vr = __ldg(pver + p);
                const float4 wa = __ldg(pw + 2 * (size_t)p), wb = __ldg(pw + 2 * (size_t)p + 1);
                const float wv[kMaxPatchVerts] = {wa.x, wa.y, wa.z, wa.w, wb.x, wb.y, wb.z, wb.w};
                const int ntets = meta.y & 0xff, nverts = meta.y >> 8;
                float4 r0[kMaxPatchTets], r1[kMaxPatchTets], r2[kMaxPatchTets];  // q0, q1, q2 records
                float2 lams[kMaxPatchTets];
#pragma unroll
                for (int i = 0; i < kMaxPatchTets; i++) {
                    if (i < ntets) {
                        r0[i] = __ldg(t.q0 + meta.x + i);
                        r1[i] = __ldg(t.q1 + meta.x + i);
                        r2[i] = __ldg(t.q2 + meta.x + i);
                        // this lane alone writes these multipliers
                        lams[i] = (FIRST_ZERO && it == 0) ? make_float2(0.f, 0.f) : t.lam[meta.x + i];
                    }
                }
                const int vid[kMaxPatchVerts] = {va.x, va.y, va.z, va.w, vb.x, vb.y, vb.z, vb.w};
                const int vw[4] = {vr.x, vr.y, vr.z, vr.w};
                int due[kMaxPatchVerts];
                unsigned pending = 0;
#pragma unroll
                for (int k = 0; k < kMaxPatchVerts; k++) {
                    const int h = (vw[k >> 1] >> (16 * (k & 1))) & 0xffff;  // deg << 8 | pre
                    due[k] = it * (h >> 8) + (h & 0xff);
                    if (k < nverts) {
                        const float4 v = ld_relaxed_f4(xv + vid[k]);
                        sv[k][tid] = make_float4(v.x, v.y, v.z, wv[k]);
                        if (__float_as_int(v.w) < due[k]) pending |= 1u << k;
                    }
                }
                unsigned n = 0;
                while (pending) {
                    if (++n > ta.poll_limit || ((n & 63) == 0 && *(volatile unsigned*)ta.abort_flag)) {
                        ok = false;
                        break;
                    }
                    __nanosleep(1024);  // polls cost L2 bandwidth the writers need
#pragma unroll
                    for (int k = 0; k < kMaxPatchVerts; k++) {
                        if (pending & (1u << k)) {
                            const float4 v = ld_relaxed_f4(xv + vid[k]);
                            if (__float_as_int(v.w) >= due[k]) {
                                sv[k][tid].x = v.x;
                                sv[k][tid].y = v.y;
                                sv[k][tid].z = v.z;
                                pending &= ~(1u << k);
                            }
                        }
                    }
                }
                if (ok) {
                    const unsigned long long loc =
                        (unsigned long long)(unsigned)meta.z | ((unsigned long long)(unsigned)meta.w << 32);
#pragma unroll
                    for (int i = 0; i < kMaxPatchTets; i++) {
                        if (i >= ntets) break;
                        const int slot = meta.x + i;
                        TetState<float> st;
                        st.q[0] = r0[i].x; st.q[1] = r0[i].y; st.q[2] = r0[i].z; st.q[3] = r0[i].w;
                        st.q[4] = r1[i].x; st.q[5] = r1[i].y; st.q[6] = r1[i].z; st.q[7] = r1[i].w;
                        st.q[8] = r2[i].x; st.atd = r2[i].y; st.ath = r2[i].z; st.gam = r2[i].w;
                        int l[4];
                        float4 xp[4];
#pragma unroll
                        for (int q = 0; q < 4; q++) {
                            l[q] = (int)((loc >> (12 * i + 3 * q)) & 7ull);
                            xp[q] = sv[l[q]][tid];
                            st.p[q][0] = xp[q].x; st.p[q][1] = xp[q].y; st.p[q][2] = xp[q].z;
                            st.w[q] = fabsf(xp[q].w);
                        }
                        float2 lam = lams[i];
                        float d[4][3], rsq;
                        if (project_one<false>(st, t, slot, xp, lam, d, rsq, flags)) {
#pragma unroll
                            for (int q = 0; q < 4; q++) sv[l[q]][tid] = moved(xp[q], d[q]);
                        }
                        t.lam[slot] = lam;
                    }
                    // every vertex goes out one version later, moved or not
#pragma unroll
                    for (int k = 0; k < kMaxPatchVerts; k++) {
                        if (k < nverts) {
                            const float4 s = sv[k][tid];
                            st_relaxed_f4(xv + vid[k], make_float4(s.x, s.y, s.z, __int_as_float(due[k] + 1)));
                        }
                    }
                }
            }
            if (!__all_sync(0xffffffffu, ok)) {
                if (lane == 0) {
                    atomicExch(ta.abort_flag, 1u);
                    atomicAdd(&flags->timeouts, 1ull);
                }
                return;
            }
        }
    }
}

// ---- attachment constraints (AttachmentConstraint.hpp:15-100) ----
// C = |x - target|, grad C = (x - target) / C (1e-12 per component when C <
// 1e-12), alpha = 0, an equality constraint projected by the scalar rule of
// ConstraintProjector::project (ConstraintProjector.hpp:111-172).
__device__ __forceinline__ void attach_update(const float4 xv, const float4 tg, float lam, float& dlam, float d[3]) {
    const float a = xv.x - tg.x, b = xv.y - tg.y, c = xv.z - tg.z;
    const float dist = sqrtf(a * a + b * b + c * c);
    float g0, g1, g2;
    if (dist < 1e-12f) {
        g0 = g1 = g2 = 1e-12f;
    } else {
        g0 = a / dist; g1 = b / dist; g2 = c / dist;
    }
    const float w = fabsf(xv.w);
    const float L = w * (g0 * g0 + g1 * g1 + g2 * g2);
    dlam = -dist / L;
    d[0] = w * g0 * dlam;
    d[1] = w * g1 * dlam;
    d[2] = w * g2 * dlam;
    (void)lam;  // alpha~ = 0: lambda does not enter the update
}

// Gauss-Seidel: one colour of attachments (no two share a vertex), in place
__global__ void k_attach_gs(const int* __restrict__ vert, const float4* __restrict__ target,
                            float* __restrict__ lam, const int* __restrict__ order, int begin, int end,
                            float4* __restrict__ x, bool first) {
    pdl_wait_then_release();
    const int i = begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= end) return;
    const int a = order[i];
    const int v = vert[a];
    const float4 xv = x[v];
    float l = first ? 0.f : lam[a];
    float dl, d[3];
    attach_update(xv, target[a], l, dl, d);
    if (isfinite(dl)) {
        lam[a] = l + dl;
        x[v] = moved(xv, d);
    } else {
        lam[a] = l;
    }
}

// Jacobi: every attachment from the same x, updates summed into dx
__global__ void k_attach_jacobi(const int* __restrict__ vert, const float4* __restrict__ target,
                                float* __restrict__ lam, int n, const float4* __restrict__ x,
                                float4* __restrict__ dx, bool first) {
    pdl_wait_then_release();
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    const int v = vert[a];
    float l = first ? 0.f : lam[a];
    float dl, d[3];
    attach_update(x[v], target[a], l, dl, d);
    if (isfinite(dl)) {
        lam[a] = l + dl;
        add_vec4(dx + v, d[0], d[1], d[2]);
    } else {
        lam[a] = l;
    }
}

// ---- local collision iterations (XPBDMeshObject.cpp:472-505, 764-825) ----
// Vertices of every contact that was projected (lambda != 0) in the global
// solve; vmask must be cleared first.
__global__ void k_mark_contact_verts(ContactArrays c, unsigned char* __restrict__ vmask) {
    pdl_wait_then_release();
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= c.S * c.F) return;
    // static contacts only: the local passes gather no rigid-body projector
    if (c.bary[slot].w != 1.f || c.lam[slot] == 0.f) return;
    const int4 fv = c.faces[slot % c.F];
    vmask[fv.x] = 1;
    vmask[fv.y] = 1;
    vmask[fv.z] = 1;
}

// Tets attached to a marked vertex (TetMesh::vertexAttachedElements)
__global__ void k_mark_tets(const int4* __restrict__ idx, int T, const unsigned char* __restrict__ vmask,
                            unsigned char* __restrict__ tmask) {
    pdl_wait_then_release();
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= T) return;
    const int4 e = __ldg(idx + slot);
    tmask[slot] = vmask[e.x] | vmask[e.y] | vmask[e.z] | vmask[e.w];
}

// Gauss-Seidel over the marked tets of one colour of the local order
// (order[i] = slot), in place; which: 2 combined, 0 Dev, 1 Hyd.
__global__ void k_project_local_gs(TetArrays t, const int* __restrict__ order, int begin, int end,
                                   const unsigned char* __restrict__ tmask, float4* __restrict__ x, int which,
                                   Flags* flags) {
    pdl_wait_then_release();
    const int i = begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= end) return;
    const int slot = __ldg(order + i);
    if (!tmask[slot]) return;
    int4 e;
    TetState<float> s;
    load_tet_static(t, slot, e, s);
    float4 xp[4];
    gather_tet(x, e, s, xp);
    float2 lam = t.lam[slot];
    float d[4][3];
    bool ok;
    if (which == 2) {
        float rsq;
        ok = project_one<false>(s, t, slot, xp, lam, d, rsq, flags);
    } else {
        float J, r, dl;
        const float lw = which == 0 ? lam.x : lam.y;
        tet_project_single(s, which, lw, r, dl, d, J);
        if (fabsf(J) < kDegenerateJ) {
            const Fp64Out o = project_single_fp64(t, slot, xp[0], xp[1], xp[2], xp[3], which, lw);
            dl = o.dl0;
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int k = 0; k < 3; k++) d[a][k] = o.d[3 * a + k];
            atomicAdd(&flags->degenerate, 1ull);
        }
        ok = isfinite(dl);
        if (!ok) atomicAdd(&flags->nonfinite, 1ull);
        else if (which == 0) lam.x += dl;
        else lam.y += dl;
    }
    if (ok) {
        const int v[4] = {e.x, e.y, e.z, e.w};
#pragma unroll
        for (int j = 0; j < 4; j++)
            x[v[j]] = moved(xp[j], d[j]);
    }
    t.lam[slot] = lam;
}

// Jacobi over the marked tets: updates from the same x summed into dx
template <bool SEPARATE>
__global__ void k_project_local_jacobi(TetArrays t, int T, const unsigned char* __restrict__ tmask,
                                       const float4* __restrict__ x, float4* __restrict__ dx, Flags* flags) {
    pdl_wait_then_release();
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= T || !tmask[slot]) return;
    int4 e;
    TetState<float> s;
    load_tet_static(t, slot, e, s);
    float4 xp[4];
    gather_tet(x, e, s, xp);
    float2 lam = t.lam[slot];
    float d[4][3], rsq;
    if (project_one<SEPARATE>(s, t, slot, xp, lam, d, rsq, flags)) {
        add_vec4(dx + e.x, d[0][0], d[0][1], d[0][2]);
        add_vec4(dx + e.y, d[1][0], d[1][1], d[1][2]);
        add_vec4(dx + e.z, d[2][0], d[2][1], d[2][2]);
        add_vec4(dx + e.w, d[3][0], d[3][1], d[3][2]);
    }
    t.lam[slot] = lam;
}

// ---- learned warm start ----
// Features of the tets in slots [s0, s0 + n) at the current (predicted)
// positions: F (9, column-major), the previous multipliers scaled to
// alpha_tilde * lambda (dimensionless), log10(E)/5, nu, dt * 1e3.
__global__ void k_mlp_features(TetArrays t, const float4* __restrict__ x, const float2* __restrict__ mat, float dt_feat,
                               int s0, int n, __nv_bfloat16* __restrict__ X) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    pdl_wait_then_release();
    if (i >= n) return;
    const int slot = s0 + i;
    int4 e;
    TetState<float> st;
    load_tet_static(t, slot, e, st);
    float4 xp[4];
    gather_tet(x, e, st, xp);
    float F[9];
    tet_F(st, F);
    const float2 lam = t.lam[slot];
    const float2 m = mat[slot];
    float f[16];
#pragma unroll
    for (int k = 0; k < 9; k++) f[k] = F[k];
    f[9] = st.atd * lam.x;
    f[10] = st.ath * lam.y;
    f[11] = m.x;
    f[12] = m.y;
    f[13] = dt_feat;
    f[14] = 0.f;
    f[15] = 0.f;
    __nv_bfloat162 h[8];
#pragma unroll
    for (int k = 0; k < 8; k++) h[k] = __floats2bfloat162_rn(f[2 * k], f[2 * k + 1]);
    uint4* dst = reinterpret_cast<uint4*>(X + (size_t)i * 16);
    dst[0] = reinterpret_cast<const uint4*>(h)[0];
    dst[1] = reinterpret_cast<const uint4*>(h)[1];
}

// Training targets: the solved multipliers, scaled as the features.
__global__ void k_mlp_targets(TetArrays t, int s0, int n, float* __restrict__ Y) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    pdl_wait_then_release();
    if (i >= n) return;
    const int slot = s0 + i;
    const float4 c = __ldg(t.q2 + slot);
    const float2 lam = t.lam[slot];
    Y[2 * (size_t)i] = c.y * lam.x;
    Y[2 * (size_t)i + 1] = c.z * lam.y;
}

// Warm start: lambda <- lambda0 and x += M^-1 grad C(x)^T lambda0 summed over
// tets (into dx; applied by k_apply). lambda0 comes from the network output
// (scaled, pred != nullptr) or from the multipliers already in place (the
// previous step's, pred == nullptr).
__global__ void k_warm_start(TetArrays t, int T, const float* __restrict__ pred, const float4* __restrict__ x,
                             float4* __restrict__ dx) {
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    pdl_wait_then_release();
    if (slot >= T) return;
    int4 e;
    TetState<float> st;
    load_tet_static(t, slot, e, st);
    float4 xp[4];
    gather_tet(x, e, st, xp);
    float2 lam;
    if (pred) {
        lam = make_float2(pred[2 * (size_t)slot] / st.atd, pred[2 * (size_t)slot + 1] / st.ath);
        if (!(isfinite(lam.x) && isfinite(lam.y))) lam = make_float2(0.f, 0.f);
        t.lam[slot] = lam;
    } else {
        lam = t.lam[slot];
    }
    float Cd, Ch, gd[9], gh[9], J;
    tet_eval(st, Cd, Ch, gd, gh, J);
    float d[4][3];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const float a = i < 3 ? gd[3 * i + k] : -gd[k] - gd[3 + k] - gd[6 + k];
            const float b = i < 3 ? gh[3 * i + k] : -gh[k] - gh[3 + k] - gh[6 + k];
            d[i][k] = st.w[i] * (a * lam.x + b * lam.y);
        }
    add_vec4(dx + e.x, d[0][0], d[0][1], d[0][2]);
    add_vec4(dx + e.y, d[1][0], d[1][1], d[1][2]);
    add_vec4(dx + e.z, d[2][0], d[2][1], d[2][2]);
    add_vec4(dx + e.w, d[3][0], d[3][1], d[3][2]);
}

// Residual-triggered fallback: rows[0] = ||r(x_pred, 0)||^2, rows[1] =
// ||r(x_warm, lambda0)||^2. When the warm start made the residual worse, the
// predicted positions and lambda = 0 are restored. stats[0] counts kept warm
// starts, stats[1] rejected ones.
__global__ void k_warm_fallback(const double* __restrict__ rows, float4* __restrict__ x,
                                const float4* __restrict__ x_pred, float2* __restrict__ lam, int V, int T,
                                unsigned long long* __restrict__ stats) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    pdl_wait_then_release();
    const bool reject = rows[1] > rows[0];
    if (i == 0) atomicAdd(&stats[reject ? 1 : 0], 1ull);
    if (!reject) return;
    if (i < V) x[i] = x_pred[i];
    if (i < T) lam[i] = make_float2(0.f, 0.f);
}

// One block per row: FP64 sum of `stride` partials, fixed order.
__global__ void k_reduce_rows(const double* __restrict__ partial, int stride, double* __restrict__ out) {
    pdl_wait_then_release();
    __shared__ double sh[256];
    const int row = blockIdx.x;
    double s = 0.0;
    for (int i = threadIdx.x; i < stride; i += blockDim.x) s += partial[(size_t)row * stride + i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[row] = sh[0];
}

inline int nblk(long long n, int b) { return (int)((n + b - 1) / b); }

// cudaLaunchKernelEx with programmatic stream serialization when L.pdl.
template <typename... KArgs, typename... Args>
void go(void (*kernel)(KArgs...), int grid, int block, const Launch& L, Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = L.s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = L.pdl ? 1 : 0;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

}  // namespace

int residual_blocks(int T, int block) { return nblk(T, block); }

void launch_predict_first_order(const Launch& s, float4* x, float4* prev, const float* gdz, int V) {
    if (V > 0) go(k_predict_first_order, nblk(V, 256), 256, s, x, prev, gdz, V);
}

void launch_predict(const Launch& s, float4* x, float4* prev, const float4* vel, int V, float dt, float dz) {
    if (V > 0) go(k_predict, nblk(V, 256), 256, s, x, prev, vel, V, dt, dz);
}

void launch_kinematic(const Launch& s, float4* x, const int* idx, const float4* rest, int n, float ox, float oy,
                      float oz) {
    if (n > 0) go(k_kinematic, nblk(n, 256), 256, s, x, idx, rest, n, ox, oy, oz);
}

// FIRST x SEPARATE x RES instantiations of the tet sweep kernels
#define XG_SWEEP(KERNEL, GRID, BLOCK, ...)                                                      \
    do {                                                                                        \
        const bool _r = res.partial != nullptr;                                                 \
        if (first) {                                                                            \
            if (separate) {                                                                     \
                if (_r) go(KERNEL<true, true, true>, GRID, BLOCK, s, __VA_ARGS__);              \
                else go(KERNEL<true, true, false>, GRID, BLOCK, s, __VA_ARGS__);                \
            } else {                                                                            \
                if (_r) go(KERNEL<true, false, true>, GRID, BLOCK, s, __VA_ARGS__);             \
                else go(KERNEL<true, false, false>, GRID, BLOCK, s, __VA_ARGS__);               \
            }                                                                                   \
        } else {                                                                                \
            if (separate) {                                                                     \
                if (_r) go(KERNEL<false, true, true>, GRID, BLOCK, s, __VA_ARGS__);             \
                else go(KERNEL<false, true, false>, GRID, BLOCK, s, __VA_ARGS__);               \
            } else {                                                                            \
                if (_r) go(KERNEL<false, false, true>, GRID, BLOCK, s, __VA_ARGS__);            \
                else go(KERNEL<false, false, false>, GRID, BLOCK, s, __VA_ARGS__);              \
            }                                                                                   \
        }                                                                                       \
    } while (0)

void launch_project_jacobi(const Launch& s, int block, const TetArrays& t, int T, const float4* x, float4* dx,
                           bool first, bool separate, ResidualSink res, Flags* flags) {
    if (T <= 0) return;
    XG_SWEEP(k_project_jacobi, nblk(T, block), block, t, T, x, dx, res, flags);
}

void launch_project_jacobi_gather_write(const Launch& s, int block, const TetArrays& t, int T, const float4* x,
                                        float4* dxt, bool first, bool separate, ResidualSink res, Flags* flags) {
    if (T <= 0) return;
    XG_SWEEP(k_project_jacobi_write, nblk(T, block), block, t, T, x, dxt, res, flags);
}

void launch_gather_apply(const Launch& s, float4* x, const float4* dxt, const int* csr_off, const int* csr_ent,
                         float4* dx, int V, float4* prev, float4* vel, bool final_step, float dt, bool write_vel) {
    if (V <= 0) return;
    const float* d = (const float*)dxt;
    if (final_step) go(k_gather_apply<true>, nblk(V, 256), 256, s, x, d, csr_off, csr_ent, dx, V, prev, vel, dt, write_vel);
    else go(k_gather_apply<false>, nblk(V, 256), 256, s, x, d, csr_off, csr_ent, dx, V, prev, vel, dt, write_vel);
}

void launch_apply(const Launch& s, float4* x, float4* dx, int V, float4* prev, float4* vel, bool final_step,
                  float dt, bool write_vel) {
    if (V <= 0) return;
    if (final_step) go(k_apply<true>, nblk(V, 256), 256, s, x, dx, V, prev, vel, dt, write_vel);
    else go(k_apply<false>, nblk(V, 256), 256, s, x, dx, V, prev, vel, dt, write_vel);
}

void launch_project_patches(const Launch& s, const TetArrays& t, const PatchArrays& pa, int pbegin, int pend,
                            float4* x, bool first, int which, Flags* flags, int min_blocks, int variant) {
    const int n = pend - pbegin;
    if (n <= 0) return;
    const int g = nblk(n, kPatchBlock);
    if (variant == 0) {
#define XG_PATCHR(F, W) go(k_project_patch_reg<F, W>, g, kPatchBlock, s, t, pa, pbegin, pend, x, flags)
        if (which == 2) { if (first) XG_PATCHR(true, 2); else XG_PATCHR(false, 2); }
        else if (which == 0) { if (first) XG_PATCHR(true, 0); else XG_PATCHR(false, 0); }
        else { if (first) XG_PATCHR(true, 1); else XG_PATCHR(false, 1); }
#undef XG_PATCHR
        return;
    }
#define XG_PATCH(F, W, M) go(k_project_patch<F, W, M>, g, kPatchBlock, s, t, pa, pbegin, pend, x, flags)
#define XG_PATCH_M(F, W) do { if (min_blocks == 8) XG_PATCH(F, W, 8); else XG_PATCH(F, W, 6); } while (0)
    if (which == 2) { if (first) XG_PATCH_M(true, 2); else XG_PATCH_M(false, 2); }
    else if (which == 0) { if (first) XG_PATCH_M(true, 0); else XG_PATCH_M(false, 0); }
    else { if (first) XG_PATCH_M(true, 1); else XG_PATCH_M(false, 1); }
#undef XG_PATCH_M
#undef XG_PATCH
}

void launch_contacts_jacobi(const Launch& s, const ContactArrays& c, const float4* x, float4* dx, bool first) {
    const int n = c.S * c.F;
    if (n <= 0) return;
    if (first) go(k_contacts_jacobi<true>, nblk(n, 256), 256, s, c, x, dx);
    else go(k_contacts_jacobi<false>, nblk(n, 256), 256, s, c, x, dx);
}

void launch_contact_lists(const Launch& s, const ContactArrays& c, const int* ifl, const int* ifo_off, int ncol,
                          int n_inst, int* act_faces, int* act_off) {
    if (n_inst > 0 && c.F > 0) go(k_contact_lists, n_inst, kContactListThreads, s, c, ifl, ifo_off, ncol, act_faces, act_off);
}

void launch_contacts_gs_lists(const Launch& s, const ContactArrays& c, const int* act_faces, const int* act_off,
                              int ncol, int n_inst, float4* x, bool first) {
    if (n_inst > 0 && c.F > 0 && ncol > 0)
        go(k_contacts_gs_lists, n_inst, kContactListThreads, s, c, act_faces, act_off, ncol, x, first);
}

void launch_prim_eval(cudaStream_t s, const float4* prim, const float4* pts, int n, float4* out) {
    if (n > 0) k_prim_eval<<<nblk(n, 128), 128, 0, s>>>(prim, pts, n, out);
}

void launch_detect(const Launch& s, const ContactArrays& c, const float4* x, const float4* sphere_table,
                   const int* face_inst) {
    const int n = c.S * c.F;
    if (n <= 0) return;
    go(k_detect, nblk(n, 128), 128, s, c, x, sphere_table, face_inst);
}

void launch_finalize(const Launch& s, float4* x, const float4* prev, float4* vel, int V, float dt, bool write_vel) {
    if (V > 0) go(k_finalize, nblk(V, 256), 256, s, x, prev, vel, V, dt, write_vel);
}

void launch_velocity(const Launch& s, const float4* x, const float4* prev, float4* vel, int V, float dt) {
    if (V > 0) go(k_velocity, nblk(V, 256), 256, s, x, prev, vel, V, dt);
}

void launch_residual(const Launch& s, int block, const TetArrays& t, int T, const float4* x, bool separate,
                     const int* perm, float* rvec, ResidualSink res, double* energy_partial, float dt2,
                     bool zero_lam) {
    if (T <= 0) return;
    go(k_residual, nblk(T, block), block, s, t, T, x, separate, perm, rvec, res, energy_partial, dt2, zero_lam);
}

int sweep_dataflow_blocks_per_sm(bool staged, int min_blocks) {
    int n = 0, m = 0;
    cudaError_t e;
    if (staged) {
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_sweep_dataflow_staged<true>, kPatchBlock, 0);
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&m, k_sweep_dataflow_staged<false>, kPatchBlock, 0);
    } else if (min_blocks == 8) {
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_sweep_dataflow<true, 8>, kFlowBlock, 0);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&m, k_sweep_dataflow<false, 8>, kFlowBlock, 0);
    } else if (min_blocks == 6) {
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_sweep_dataflow<true, 6>, kFlowBlock, 0);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&m, k_sweep_dataflow<false, 6>, kFlowBlock, 0);
    } else {
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_sweep_dataflow<true, 1>, kFlowBlock, 0);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&m, k_sweep_dataflow<false, 1>, kFlowBlock, 0);
    }
    if (e != cudaSuccess) return 0;
    return n < m ? n : m;
}

cudaError_t launch_sweep_dataflow(const Launch& s, const TetArrays& t, const PatchArrays& pa, const TaskArrays& ta,
                                  int iters, bool first_zero, float4* x, Flags* flags, int grid, bool staged,
                                  int min_blocks) {
    if (iters <= 0 || ta.ntasks <= 0) return cudaSuccess;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(staged ? kPatchBlock : kFlowBlock);
    cfg.stream = s.s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (staged) {
        if (first_zero) return cudaLaunchKernelEx(&cfg, k_sweep_dataflow_staged<true>, t, pa, ta, iters, x, flags);
        return cudaLaunchKernelEx(&cfg, k_sweep_dataflow_staged<false>, t, pa, ta, iters, x, flags);
    }
#define XG_FLOW(F, M) return cudaLaunchKernelEx(&cfg, k_sweep_dataflow<F, M>, t, pa, ta, iters, x, flags)
    if (min_blocks == 8) { if (first_zero) XG_FLOW(true, 8); else XG_FLOW(false, 8); }
    if (min_blocks == 6) { if (first_zero) XG_FLOW(true, 6); else XG_FLOW(false, 6); }
    if (first_zero) XG_FLOW(true, 1);
    XG_FLOW(false, 1);
#undef XG_FLOW
}

int sweep_versioned_blocks_per_sm(int min_blocks) {
    int n = 0, m = 0;
    cudaError_t e;
#define XG_VOCC(M)                                                                                 \
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_sweep_versioned<true, M>, kFlowBlock, 0); \
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&m, k_sweep_versioned<false, M>, kFlowBlock, 0)
    if (min_blocks == 8) { XG_VOCC(8); }
    else if (min_blocks == 6) { XG_VOCC(6); }
    else { XG_VOCC(1); }
#undef XG_VOCC
    if (e != cudaSuccess) return 0;
    return n < m ? n : m;
}

cudaError_t launch_sweep_versioned(const Launch& s, const TetArrays& t, const PatchArrays& pa, const int4* pver,
                                   const TaskArrays& ta, int iters, bool first_zero, float4* x, float4* xv,
                                   float4* pw, int V, int P, Flags* flags, int grid, int min_blocks) {
    if (iters <= 0 || ta.ntasks <= 0) return cudaSuccess;
    go(k_versions_in, nblk(V > P ? V : P, 256), 256, s, xv, pw, (const float4*)x, pa, V, P);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(kFlowBlock);
    cfg.stream = s.s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const float4* pwc = pw;
    cudaError_t e;
#define XG_VER(F, M) e = cudaLaunchKernelEx(&cfg, k_sweep_versioned<F, M>, t, pa, pver, ta, iters, pwc, xv, flags)
    if (min_blocks == 8) { if (first_zero) XG_VER(true, 8); else XG_VER(false, 8); }
    else if (min_blocks == 6) { if (first_zero) XG_VER(true, 6); else XG_VER(false, 6); }
    else if (first_zero) XG_VER(true, 1);
    else XG_VER(false, 1);
#undef XG_VER
    if (e != cudaSuccess) return e;
    go(k_versions_out, nblk(V, 256), 256, s, x, (const float4*)xv, V);
    return cudaSuccess;
}

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

void launch_self_detect(const Launch& s, const SelfArrays& a, const SelfGrid& g, const float4* x, const int4* faces) {
    if (a.n_surf <= 0 || a.T <= 0) return;
    const int ncells = g.nx * g.ny * g.nz;
    cudaMemsetAsync(a.cell_count, 0, sizeof(int) * (size_t)ncells, s.s);
    cudaMemsetAsync(a.cell_fill, 0, sizeof(int) * (size_t)ncells, s.s);
    cudaMemsetAsync(a.n_overflow, 0, sizeof(int), s.s);
    go(k_self_bin_count, nblk(a.T, 256), 256, s, a, g, x);
    const int nb = (ncells + kScanChunk - 1) / kScanChunk;
    go(k_scan_partials, nb, kScanThreads, s, (const int*)a.cell_count, ncells, a.scan_part);
    go(k_scan_part_single, 1, kScanThreads, s, a.scan_part, nb);
    go(k_scan_apply, nb, kScanThreads, s, (const int*)a.cell_count, ncells, (const int*)a.scan_part, a.cell_off, nb);
    go(k_self_bin_fill, nblk(a.T, 256), 256, s, a);
    go(k_self_query, nblk(a.n_surf, 128), 128, s, a, g, x);
    go(k_self_compact, 1, kCompactThreads, s, a);
    go(k_self_face, nblk(32 * a.n_surf, 256), 256, s, a, x, faces);
}

void launch_self_contacts(const Launch& s, const SelfArrays& a, const int4* faces, float4* x, float4* dx,
                          bool jacobi, bool first, float alpha_tilde, Flags* flags) {
    if (a.n_surf <= 0) return;
    if (jacobi) go(k_self_contacts_jacobi, nblk(a.n_surf, 128), 128, s, a, faces, (const float4*)x, dx, first,
                   alpha_tilde, flags);
    else go(k_self_contacts_gs, 1, 32, s, a, faces, x, first, alpha_tilde, flags);
}

void launch_xyz_from_host(cudaStream_t s, float4* x, const double* h, int V, bool keep_w) {
    if (V > 0) k_xyz_from_host<double><<<nblk(V, kHostIoThreads), kHostIoThreads, 0, s>>>(x, h, V, keep_w);
}
void launch_xyz_from_host(cudaStream_t s, float4* x, const float* h, int V, bool keep_w) {
    if (V > 0) k_xyz_from_host<float><<<nblk(V, kHostIoThreads), kHostIoThreads, 0, s>>>(x, h, V, keep_w);
}
void launch_xyz_to_host(cudaStream_t s, double* h, const float4* x, int V) {
    if (V > 0) k_xyz_to_host<double><<<nblk(V, kHostIoThreads), kHostIoThreads, 0, s>>>(h, x, V);
}
void launch_xyz_to_host(cudaStream_t s, float* h, const float4* x, int V) {
    if (V > 0) k_xyz_to_host<float><<<nblk(V, kHostIoThreads), kHostIoThreads, 0, s>>>(h, x, V);
}

void launch_attach_gs(const Launch& s, const int* vert, const float4* target, float* lam, const int* order, int begin,
                      int end, float4* x, bool first) {
    if (end > begin) go(k_attach_gs, nblk(end - begin, 128), 128, s, vert, target, lam, order, begin, end, x, first);
}

void launch_attach_jacobi(const Launch& s, const int* vert, const float4* target, float* lam, int n, const float4* x,
                          float4* dx, bool first) {
    if (n > 0) go(k_attach_jacobi, nblk(n, 128), 128, s, vert, target, lam, n, x, dx, first);
}

void launch_mark_local(const Launch& s, const ContactArrays& c, const TetArrays& t, int T, unsigned char* vmask,
                       unsigned char* tmask) {
    const int n = c.S * c.F;
    if (n > 0) go(k_mark_contact_verts, nblk(n, 256), 256, s, c, vmask);
    if (T > 0) go(k_mark_tets, nblk(T, 256), 256, s, t.idx, T, (const unsigned char*)vmask, tmask);
}

void launch_project_local_gs(const Launch& s, const TetArrays& t, const int* order, int begin, int end,
                             const unsigned char* tmask, float4* x, int which, Flags* flags) {
    if (end > begin) go(k_project_local_gs, nblk(end - begin, 128), 128, s, t, order, begin, end, tmask, x, which, flags);
}

void launch_project_local_jacobi(const Launch& s, const TetArrays& t, int T, const unsigned char* tmask,
                                 const float4* x, float4* dx, bool separate, Flags* flags) {
    if (T <= 0) return;
    if (separate) go(k_project_local_jacobi<true>, nblk(T, 256), 256, s, t, T, tmask, x, dx, flags);
    else go(k_project_local_jacobi<false>, nblk(T, 256), 256, s, t, T, tmask, x, dx, flags);
}

void launch_mlp_features(const Launch& s, const TetArrays& t, const float4* x, const float2* mat, float dt_feat,
                         int s0, int n, __nv_bfloat16* X) {
    if (n > 0) go(k_mlp_features, nblk(n, 256), 256, s, t, x, mat, dt_feat, s0, n, X);
}

void launch_mlp_targets(const Launch& s, const TetArrays& t, int s0, int n, float* Y) {
    if (n > 0) go(k_mlp_targets, nblk(n, 256), 256, s, t, s0, n, Y);
}

void launch_warm_start(const Launch& s, const TetArrays& t, int T, const float* pred, const float4* x, float4* dx) {
    if (T > 0) go(k_warm_start, nblk(T, 256), 256, s, t, T, pred, x, dx);
}

void launch_warm_fallback(const Launch& s, const double* rows, float4* x, const float4* x_pred, float2* lam, int V,
                          int T, unsigned long long* stats) {
    const int n = V > T ? V : T;
    go(k_warm_fallback, nblk(n, 256), 256, s, rows, x, x_pred, lam, V, T, stats);
}

void launch_reduce_rows(const Launch& s, const double* partial, int rows, int stride, double* out) {
    if (rows > 0) go(k_reduce_rows, rows, 256, s, partial, stride, out);
}

}  // namespace xg
