// Device code shared by the kernel translation units of the XPBD substep:
// programmatic-dependent-launch and TMA/mbarrier helpers, the per-tet
// Stable-Neo-Hookean arithmetic (FP32 fast path and FP64 guard path), the
// projection of one tet in either constraint form, and the launch helper.
//
// Semantics follow the reference's CPU path:
//   projection   src/solver/xpbd_projector/CombinedNeohookeanConstraintProjector.cpp:98-179
//                include/solver/xpbd_projector/ConstraintProjector.hpp:111-172
//   constraints  include/solver/constraint/{Hydrostatic,Deviatoric}Constraint.hpp
#pragma once
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

// FP64 butterfly over the warp (each step is two 32-bit shuffles).
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Fixed-order block sum in FP64 from the lane up: the caller widens each
// lane's term before squaring, the warp and the block add in double.
__device__ __forceinline__ void block_sum_store(double v, double* slot) {
    __shared__ double sw[32];
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) sw[wid] = v;
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

// Constraint values only (no gradients): C_dev = ||F||_F and C_hyd
// (DeviatoricConstraint.hpp:112-116, HydrostaticConstraint.hpp:123-153).
template <typename R>
__device__ __forceinline__ void tet_C(const TetState<R>& s, R& Cd, R& Ch) {
    R F[9];
    tet_F(s, F);
    R ss = 0;
#pragma unroll
    for (int i = 0; i < 9; i++) ss += F[i] * F[i];
    Cd = dev_sqrt(ss);
    const R J = tet_detF(F);
    if (J >= R(1)) {
        Ch = -s.gam + dev_log(J);
    } else {
        const R d = J - R(1);
        Ch = -s.gam + d - d * d / R(2) + d * d * d / R(3);
    }
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
// the state the projection saw (squared and added in FP64). Returns false when the update is non-finite
// (then nothing may be applied).
template <bool SEPARATE>
__device__ __forceinline__ bool project_one(const TetState<float>& s, const TetArrays& t, int slot, const float4 xp[4],
                                            float2& lam, float d[4][3], double& rsq, Flags* flags) {
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
        rsq = fma((double)r0, (double)r0, (double)r1 * (double)r1);
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
        rsq = fma((double)r0, (double)r0, (double)r1 * (double)r1);
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

// threads of the one-block compaction kernels (rigid contacts, self contacts)
constexpr int kCompactThreads = 1024;

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

}  // namespace xg
