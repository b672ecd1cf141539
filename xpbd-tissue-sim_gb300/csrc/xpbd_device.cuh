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

// Copies with an L2 eviction-priority policy (createpolicy): data a kernel
// reads or writes once per pass can go evict-first, so that it passes through
// the L2 without pushing out what the pass keeps reusing; evict-normal is the
// default priority.
__device__ __forceinline__ unsigned long long l2_policy(bool evict_first) {
    unsigned long long p;
    if (evict_first)
        asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    else
        asm volatile("createpolicy.fractional.L2::evict_normal.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ void tma_load_1d_hint(void* dst, const void* src, unsigned bytes, unsigned long long* bar,
                                                 unsigned long long pol) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::
            "r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar)), "l"(pol)
        : "memory");
}
// 16-byte asynchronous copy global -> shared (cp.async, cache-global); with
// src_bytes = 0 nothing is read and the 16 bytes are zero-filled. Completion
// (cp_async_wait_all) makes the data visible to the issuing thread.
__device__ __forceinline__ void cp_async16_hint(void* dst, const void* src, unsigned src_bytes,
                                                unsigned long long pol) {
    asm volatile("cp.async.cg.shared.global.L2::cache_hint [%0], [%1], 16, %2, %3;" ::"r"(smem_u32(dst)), "l"(src),
                 "r"(src_bytes), "l"(pol)
                 : "memory");
}
__device__ __forceinline__ float2 ld_f2_hint(const float2* p, unsigned long long pol) {
    float2 v;
    asm volatile("ld.global.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;" : "=f"(v.x), "=f"(v.y) : "l"(p), "l"(pol));
    return v;
}
__device__ __forceinline__ void st_f2_hint(float2* p, float2 v, unsigned long long pol) {
    asm volatile("st.global.L2::cache_hint.v2.f32 [%0], {%1, %2}, %3;" ::"l"(p), "f"(v.x), "f"(v.y), "l"(pol)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

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
//
// The static record of a tet holds M = Q Q^T and det Q (Q = Dm^-1) instead of
// Q. With the edges X_i = p_i - p_3 (i < 3), F = [X_0 X_1 X_2] Q
// (ElementConstraint.hpp:78-119) and q_i the rows of Q (q_3 = -q_0 - q_1 -
// q_2), everything the two constraints need follows exactly:
//   G_i = F q_i         = sum_j M_ij X_j
//   ||F||^2             = sum_i X_i . G_i
//   cof(F) q_i          = det Q N_i,  N_0 = X_1 x X_2, N_1 = X_2 x X_0, N_2 = X_0 x X_1
//   det F               = det Q (X_0 . N_0)
//   G_i . cof(F) q_i    = det F |q_i|^2 = det F M_ii   (F^T cof F = det F I)
// so grad C_dev,i = G_i / ||F|| (DeviatoricConstraint.hpp:112-152) and
// grad C_hyd,i = fac det Q N_i (HydrostaticConstraint.hpp:123-221). F itself
// is never formed; the results agree with the F-based evaluation to rounding.
// ---------------------------------------------------------------------------
template <typename R>
struct TetState {
    R p[4][3];
    R w[4];
    R m[6];  // M00 M11 M22 M01 M02 M12
    R dq;    // det Q
    R atd, ath, gam;
    R msum;  // |q_3|^2 = sum of all entries of M (q_3 = -q_0 - q_1 - q_2)
};

template <typename R>
__device__ __forceinline__ R dev_log(R v) { return log(v); }
template <>
__device__ __forceinline__ float dev_log<float>(float v) { return logf(v); }
template <typename R>
__device__ __forceinline__ R dev_sqrt(R v) { return sqrt(v); }
template <>
__device__ __forceinline__ float dev_sqrt<float>(float v) { return sqrtf(v); }

// Edges X_i, G_i = F q_i and the face normals N_i (cof(F) q_i / det Q).
template <typename R>
__device__ __forceinline__ void tet_geom(const TetState<R>& s, R X[3][3], R G[3][3], R N[3][3]) {
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int k = 0; k < 3; k++) X[i][k] = s.p[i][k] - s.p[3][k];
    const R M[3][3] = {{s.m[0], s.m[3], s.m[4]}, {s.m[3], s.m[1], s.m[5]}, {s.m[4], s.m[5], s.m[2]}};
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int k = 0; k < 3; k++) G[i][k] = M[i][0] * X[0][k] + M[i][1] * X[1][k] + M[i][2] * X[2][k];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const R* a = X[(i + 1) % 3];
        const R* b = X[(i + 2) % 3];
        N[i][0] = a[1] * b[2] - a[2] * b[1];
        N[i][1] = a[2] * b[0] - a[0] * b[2];
        N[i][2] = a[0] * b[1] - a[1] * b[0];
    }
}

// C_hyd and the scale fac of its gradient, both branches of
// HydrostaticConstraint.hpp:123-221 (log J for J >= 1, its cubic Taylor
// polynomial below).
template <typename R>
__device__ __forceinline__ R tet_hyd(R J, R gam, R& fac) {
    if (J >= R(1)) {
        fac = R(1) / J;
        return -gam + dev_log(J);
    }
    const R d = J - R(1);
    fac = R(1) - d + d * d;
    return -gam + d - d * d / R(2) + d * d * d / R(3);
}

// Values and gradients of both constraints. gd/gh hold vertices 0..2; vertex
// 3 is minus their sum.
template <typename R>
__device__ __forceinline__ void tet_eval(const TetState<R>& s, R& Cd, R& Ch, R gd[9], R gh[9], R& J) {
    R X[3][3], G[3][3], N[3][3];
    tet_geom(s, X, G, N);
    R ss = 0;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int k = 0; k < 3; k++) ss += X[i][k] * G[i][k];
    Cd = dev_sqrt(ss);
    const R invC = R(1) / Cd;
    J = s.dq * (X[0][0] * N[0][0] + X[0][1] * N[0][1] + X[0][2] * N[0][2]);
    R fac;
    Ch = tet_hyd(J, s.gam, fac);
    const R fh = fac * s.dq;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int k = 0; k < 3; k++) {
            gd[3 * i + k] = invC * G[i][k];
            gh[3 * i + k] = fh * N[i][k];
        }
}

// Constraint values only (no gradients): C_dev = ||F||_F and C_hyd
// (DeviatoricConstraint.hpp:112-116, HydrostaticConstraint.hpp:123-153).
template <typename R>
__device__ __forceinline__ void tet_C(const TetState<R>& s, R& Cd, R& Ch) {
    R X[3][3], G[3][3], N[3][3];
    tet_geom(s, X, G, N);
    R ss = 0;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int k = 0; k < 3; k++) ss += X[i][k] * G[i][k];
    Cd = dev_sqrt(ss);
    const R J = s.dq * (X[0][0] * N[0][0] + X[0][1] * N[0][1] + X[0][2] * N[0][2]);
    R fac;
    Ch = tet_hyd(J, s.gam, fac);
}

// One-instruction hardware approximations (PTX rsqrt.approx, rcp.approx,
// lg2.approx) for the FP32 fast path. Their error is about an ulp of the
// result; for log J near 1 it is an absolute error below an ulp of C_hyd,
// which is dominated by -gamma.
__device__ __forceinline__ float rsqrt_approx(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rcp_approx(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float log_approx(float x) {
    float y;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y * 0.693147180559945f;  // ln 2
}
__device__ __forceinline__ float2 splat2(float v) { return make_float2(v, v); }

// FP32 fast path of the combined 2x2 projection (same contract as
// tet_project_combined below), written for issue slots, the limit of the
// Gauss-Seidel chain:
// - the edge / face-normal form above: no F, no cofactor matrix, and the
//   cross term sum_i w_i grad C_dev,i . grad C_hyd,i = J sum_i w_i M_ii / ||F||
//   * fac without a dot product;
// - (G_ik, N_ik) held as float2 pairs, so their squares, sums and the vertex
//   updates run as packed FP32x2 instructions (FFMA2 / FADD2 / FMUL2);
// - the hydrostatic term without a branch (both forms are a few
//   instructions), 1/||F||, 1/J and 1/det from single MUFU approximations.
// Near-degenerate elements never use it.
__device__ __forceinline__ void tet_project_combined_fast(const TetState<float>& s, float lam0, float lam1, float& r0,
                                                          float& r1, float& dl0, float& dl1, float d[4][3], float& J) {
    float X[3][3];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int k = 0; k < 3; k++) X[i][k] = s.p[i][k] - s.p[3][k];
    const float M[3][3] = {{s.m[0], s.m[3], s.m[4]}, {s.m[3], s.m[1], s.m[5]}, {s.m[4], s.m[5], s.m[2]}};
    float2 GN[3][3];  // (G_ik, N_ik)
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int k = 0; k < 3; k++) GN[i][k].x = fmaf(M[i][0], X[0][k], fmaf(M[i][1], X[1][k], M[i][2] * X[2][k]));
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const float* a = X[(i + 1) % 3];
        const float* b = X[(i + 2) % 3];
        GN[i][0].y = a[1] * b[2] - a[2] * b[1];
        GN[i][1].y = a[2] * b[0] - a[0] * b[2];
        GN[i][2].y = a[0] * b[1] - a[1] * b[0];
    }
    const float ss = (fmaf(X[0][0], GN[0][0].x, fmaf(X[0][1], GN[0][1].x, X[0][2] * GN[0][2].x)) +
                      fmaf(X[1][0], GN[1][0].x, fmaf(X[1][1], GN[1][1].x, X[1][2] * GN[1][2].x))) +
                     fmaf(X[2][0], GN[2][0].x, fmaf(X[2][1], GN[2][1].x, X[2][2] * GN[2][2].x));
    const float invC = rsqrt_approx(ss);
    const float Cd = ss * invC;
    J = s.dq * fmaf(X[0][0], GN[0][0].y, fmaf(X[0][1], GN[0][1].y, X[0][2] * GN[0][2].y));
    const float dd = J - 1.f;
    const bool ge = J >= 1.f;
    const float Ch = -s.gam + (ge ? log_approx(J) : dd - dd * dd * 0.5f + dd * dd * dd * (1.f / 3.f));
    const float fac = ge ? rcp_approx(J) : fmaf(dd, dd, 1.f - dd);
    const float fh = fac * s.dq;  // grad C_hyd,i = fh N_i
    float2 S[3];                  // -(G_3, N_3)
#pragma unroll
    for (int k = 0; k < 3; k++) S[k] = __fadd2_rn(__fadd2_rn(GN[0][k], GN[1][k]), GN[2][k]);
    float2 sq[4];  // (|G_i|^2, |N_i|^2)
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const float2* v = i < 3 ? GN[i] : S;
        sq[i] = __ffma2_rn(v[0], v[0], __ffma2_rn(v[1], v[1], __fmul2_rn(v[2], v[2])));
    }
    const float2 s01 = __ffma2_rn(splat2(s.w[0]), sq[0], __fmul2_rn(splat2(s.w[1]), sq[1]));
    const float2 s23 = __ffma2_rn(splat2(s.w[2]), sq[2], __fmul2_rn(splat2(s.w[3]), sq[3]));
    const float2 sgn = __fadd2_rn(s01, s23);  // (sum w |G|^2, sum w |N|^2)
    const float sw = fmaf(s.w[0], s.m[0], s.w[1] * s.m[1]) + fmaf(s.w[2], s.m[2], s.w[3] * s.msum);
    const float L00 = fmaf(invC * invC, sgn.x, s.atd);
    const float L01 = (invC * fac) * (J * sw);
    const float L11 = fmaf(fh * fh, sgn.y, s.ath);
    r0 = fmaf(s.atd, lam0, Cd);
    r1 = fmaf(s.ath, lam1, Ch);
    const float inv_det = rcp_approx(fmaf(L00, L11, -L01 * L01));
    dl0 = fmaf(-r0, L11, r1 * L01) * inv_det;
    dl1 = fmaf(-r1, L00, r0 * L01) * inv_det;
    const float2 ab = make_float2(invC * dl0, fh * dl1);
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const float2* v = i < 3 ? GN[i] : S;
        const float2 abi = __fmul2_rn(splat2(i < 3 ? s.w[i] : -s.w[3]), ab);
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const float2 t = __fmul2_rn(v[k], abi);
            d[i][k] = t.x + t.y;
        }
    }
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

// The static record (m0, m1, m2) into a tet state.
template <typename R>
__device__ __forceinline__ void unpack_static(const float4& a, const float4& b, const float4& c, TetState<R>& s) {
    s.m[0] = a.x; s.m[1] = a.y; s.m[2] = a.z; s.m[3] = a.w;
    s.m[4] = b.x; s.m[5] = b.y; s.dq = b.z; s.atd = b.w;
    s.ath = c.x; s.gam = c.y; s.msum = c.z;
}

// Static per-tet data (indices, M and det Q, compliances): never written
// while the solver runs, so it may be loaded before the dependency wait.
__device__ __forceinline__ void load_tet_static(const TetArrays& t, int slot, int4& e, TetState<float>& s) {
    e = __ldg(t.idx + slot);
    unpack_static(__ldg(t.m0 + slot), __ldg(t.m1 + slot), __ldg(t.m2 + slot), s);
}

// A vertex moved by a projection's update. The adds are not contracted with
// the update's last multiply, so every Gauss-Seidel kernel variant rounds the
// same way and their results agree bit for bit.
__device__ __forceinline__ float4 moved(const float4& p, const float* d) {
    const float2 xy = __fadd2_rn(make_float2(p.x, p.y), make_float2(d[0], d[1]));
    return make_float4(xy.x, xy.y, __fadd_rn(p.z, d[2]), p.w);
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
    unpack_static(__ldg(t.m0 + slot), __ldg(t.m1 + slot), __ldg(t.m2 + slot), s);
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
