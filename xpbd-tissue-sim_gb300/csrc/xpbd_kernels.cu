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
#include "xpbd_device.cuh"

namespace xg {

namespace {

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
// Four blocks per SM (64 registers, a few bytes spilled): the launch waits on
// its gathers and reductions, and 32 warps per SM hide more of that than 16.
template <bool FIRST, bool SEPARATE, bool RES>
__global__ void __launch_bounds__(256, 4) k_project_jacobi(TetArrays t, int T, const float4* __restrict__ x,
                                                           float4* __restrict__ dx, ResidualSink res, Flags* flags) {
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    double rsq = 0.0;
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
    double rsq = 0.0;
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
    // tet records arrive by three bulk copies (m0, m1, m2) before the
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
        tma_load_1d(sq[0], t.m0 + s0, bytes, &bar);
        tma_load_1d(sq[1], t.m1 + s0, bytes, &bar);
        tma_load_1d(sq[2], t.m2 + s0, bytes, &bar);
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
        unpack_static(sq[0][base + i], sq[1][base + i], sq[2][base + i], st);
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
            double rsq;
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
            double rsq;
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
// The face's static contacts in slot order. The slots' active flags are read
// together and the face's vertices once: each contact moves them in registers
// for the next, and they are stored once (no other thread touches them while
// this colour runs: the faces of a colour share no vertex).
__device__ __forceinline__ void contact_face_gs(const ContactArrays& c, int f, float4* __restrict__ x, bool first) {
    const int4 fv = c.faces[f];
    unsigned act = 0;
    for (int s = 0; s < c.S; s++)
        if (c.bary[s * c.F + f].w == 1.f) act |= 1u << s;  // not empty, not against a free rigid body
    if (!act) return;
    float4 xs[3] = {x[fv.x], x[fv.y], x[fv.z]};
    bool moved_any = false;
    for (int s = 0; s < c.S; s++) {
        if (!(act & (1u << s))) continue;
        const int slot = s * c.F + f;
        float lam = first ? 0.f : c.lam[slot];
        float d[3][3];
        if (contact_update(c, slot, xs, d, lam)) {
#pragma unroll
            for (int i = 0; i < 3; i++) xs[i] = moved(xs[i], d[i]);
            moved_any = true;
        }
        c.lam[slot] = lam;
    }
    if (moved_any) {
        x[fv.x] = xs[0];
        x[fv.y] = xs[1];
        x[fv.z] = xs[2];
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

// Exact residual / energy at the current state: C in FP32 (tet_C), then
// r = C + alpha~ lambda, r^2 and the sums in FP64 (the product of the two
// floats is exact in double), so the reduction that decides convergence adds
// no FP32 rounding of its own; GB300's FP64 rate is low, so C itself stays
// FP32. rvec (optional) receives the per-constraint residuals (rounded to
// float) in the reference's order via the slot->tet map.
__global__ void __launch_bounds__(256) k_residual(TetArrays t, int T, const float4* __restrict__ x, bool separate,
                                                  const int* __restrict__ perm, float* __restrict__ rvec,
                                                  ResidualSink res, double* __restrict__ energy_partial, float dt2,
                                                  bool zero_lam) {
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    double rsq = 0.0, en = 0.0;
    int4 e;
    TetState<float> s;
    if (slot < T) load_tet_static(t, slot, e, s);
    pdl_wait_then_release();
    if (slot < T) {
        float4 xp[4];
        gather_tet(x, e, s, xp);
        const float2 lam = zero_lam ? make_float2(0.f, 0.f) : t.lam[slot];
        float Cf, Chf;
        tet_C(s, Cf, Chf);
        const double Cd = Cf, Ch = Chf;
        const double r0 = fma((double)s.atd, (double)lam.x, Cd), r1 = fma((double)s.ath, (double)lam.y, Ch);
        rsq = fma(r0, r0, r1 * r1);
        en = Cd * Cd / ((double)s.atd * dt2) + Ch * Ch / ((double)s.ath * dt2);
        if (rvec) {
            const int tt = perm ? perm[slot] : slot;
            if (!separate) { rvec[2 * (size_t)tt] = (float)r0; rvec[2 * (size_t)tt + 1] = (float)r1; }
            else { rvec[tt] = (float)r0; rvec[(size_t)T + tt] = (float)r1; }
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
            float4 r0[kMaxPatchTets], r1[kMaxPatchTets], r2[kMaxPatchTets];  // m0, m1, m2 records
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
                        r0[i] = __ldg(t.m0 + meta.x + i);
                        r1[i] = __ldg(t.m1 + meta.x + i);
                        r2[i] = __ldg(t.m2 + meta.x + i);
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
                    unpack_static(r0[i], r1[i], r2[i], st);
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
                    float d[4][3];
                    double rsq;
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
// lane 0 issues three bulk copies (m0, m1, m2 over the task's contiguous slot
// range) before the dependency wait; each warp owns its staging buffer and
// mbarrier. Same projections, order and arithmetic as k_sweep_dataflow.
constexpr int kFlowWarps = kPatchBlock / 32;
constexpr int kTaskSlots = kTaskPatches * kMaxPatchTets;
static_assert(kTaskSlots % 32 == 0, "whole multiplier records per lane");
constexpr int kLamPerLane = kTaskSlots / 32;  // a task's multipliers per lane

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
                tma_load_1d(sq[wib][0], t.m0 + tk.z, bytes, &bar[wib]);
                tma_load_1d(sq[wib][1], t.m1 + tk.z, bytes, &bar[wib]);
                tma_load_1d(sq[wib][2], t.m2 + tk.z, bytes, &bar[wib]);
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
                    unpack_static(sq[wib][0][base + i], sq[wib][1][base + i], sq[wib][2][base + i], st);
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
                    float d[4][3];
                    double rsq;
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
// The sweep works on its own copy xv of the positions, one 32-byte record per
// vertex (VerRec): the words (x, ver), (y, ver), (z, ver), (w, 0), where ver
// is the vertex's version -- how many patch projections have written it in
// this launch. In one iteration a vertex is written by each patch containing
// it, in colour order, so the patch of colour c reads vertex v once its
// version is it * deg(v) + pre(v, c) (deg: patches containing v, pre: those
// of a lower colour) -- the state the colour-by-colour launches give it.
// Each coordinate travels in one aligned 64-bit word with the version it was
// written with, and the PTX memory model makes an aligned 64-bit access
// single-copy atomic (a vector access counts as one access per element): a
// reader that sees the due version in all three words holds the three
// coordinates written with it, and a read that met a write half-way shows an
// older version in some word and is polled again. A record is one 32-byte
// L2 sector, read and written by one 256-bit vector access (.v4.b64). The
// poll is the load; no fence or task counter sits between two phases.

__device__ __forceinline__ void ld_ver(const VerRec* p, unsigned long long& a, unsigned long long& b,
                                       unsigned long long& c, unsigned long long& d) {
    asm volatile("ld.relaxed.gpu.global.v4.b64 {%0, %1, %2, %3}, [%4];"
                 : "=l"(a), "=l"(b), "=l"(c), "=l"(d)
                 : "l"(p)
                 : "memory");
}
// the fourth word (the inverse mass) is written back unchanged
__device__ __forceinline__ void st_ver(VerRec* p, float x, float y, float z, float w, unsigned ver) {
    const unsigned long long hi = (unsigned long long)ver << 32;
    const unsigned long long a = hi | __float_as_uint(x), b = hi | __float_as_uint(y), c = hi | __float_as_uint(z);
    const unsigned long long d = __float_as_uint(w);
    asm volatile("st.relaxed.gpu.global.v4.b64 [%0], {%1, %2, %3, %4};" ::"l"(p), "l"(a), "l"(b), "l"(c), "l"(d)
                 : "memory");
}
__device__ __forceinline__ float ver_val(unsigned long long w) { return __uint_as_float((unsigned)w); }
__device__ __forceinline__ int ver_of(unsigned long long w) { return (int)(w >> 32); }
__device__ __forceinline__ int ver_min(unsigned long long a, unsigned long long b, unsigned long long c) {
    return min(ver_of(a), min(ver_of(b), ver_of(c)));
}

// The device clock in ns (%globaltimer).
__device__ __forceinline__ unsigned long long clock_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t)::"memory");
    return t;
}

__global__ void k_stamp(unsigned long long* p) {
    pdl_wait_then_release();
    *p = clock_ns();
}

// Positions at version 0, the inverse mass in the fourth word; record vperm[i]
// holds vertex i (the sweep's numbering).
__global__ void k_versions_in(VerRec* __restrict__ xv, const float4* __restrict__ x, const int* __restrict__ vperm,
                              int V) {
    pdl_wait_then_release();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V) return;
    const float4 p = x[i];
    xv[vperm[i]] = VerRec{__float_as_uint(p.x), __float_as_uint(p.y), __float_as_uint(p.z), __float_as_uint(p.w)};
}

__global__ void k_versions_out(float4* __restrict__ x, const VerRec* __restrict__ xv, const int* __restrict__ vperm,
                               int V) {
    pdl_wait_then_release();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V) return;
    const VerRec r = xv[vperm[i]];
    x[i] = make_float4(ver_val(r.x), ver_val(r.y), ver_val(r.z), x[i].w);
}

// One lane's patch task of k_sweep_versioned after its first polls went out:
// wait for the vertices still short of their due versions, for the task's
// bulk-copied records and staged multipliers, project the patch's tets in
// order and write every vertex back one version later. HEX: the patch is a
// grid hex in the canonical layout kHexLocA (five tets on eight vertices), so
// the layout is known at compile time and the vertices stay in registers;
// otherwise the layout comes from the record and the vertices sit in shared
// memory (sv).
// The tets go through one straight FP32 pass. A near-degenerate element or a
// non-finite update anywhere in the patch (rare) sends the lane through the
// careful pass, which starts again from the patch's state before the task --
// the vertex records still hold it (nothing else writes them before this
// task's stores) and so does lam in global memory -- with the per-tet rule of
// every other sweep kernel (FP64 guard, non-finite updates skipped).
template <bool FIRST_ZERO, bool CONTACT_DEG, bool HEX>
__device__ __forceinline__ void versioned_patch(const TetArrays& t, const TaskArrays& ta, const FlowContacts& fc,
                                                VerRec* __restrict__ xv, Flags* flags, const int4& meta,
                                                const int (&vid)[kMaxPatchVerts], const int4& vr, int it, int s0,
                                                int ns, bool copy, float4 (*sv)[kFlowBlock],
                                                const float4 (*srec)[kTaskSlots], float2* slam,
                                                const float2 (&lt)[kLamPerLane], unsigned long long* bar,
                                                unsigned& phase, bool& ok,
                                                const unsigned long long (&pw)[kMaxPatchVerts][4]) {
    const int tid = threadIdx.x, lane = tid & 31;
    const bool active = (meta.y >> 8) > 0;
    const int ntets = HEX ? kMaxPatchTets : (meta.y & 0xff);
    const int nverts = HEX ? kMaxPatchVerts : (meta.y >> 8);
    float4 pv[kMaxPatchVerts] = {};  // HEX: the patch's vertices
    auto vget = [&](int l) -> float4 { return HEX ? pv[l] : sv[l][tid]; };
    auto vset = [&](int l, const float4& p) {
        if (HEX) pv[l] = p;
        else sv[l][tid] = p;
    };
    int due[kMaxPatchVerts];
    if (active) {
        const int vw[4] = {vr.x, vr.y, vr.z, vr.w};
        unsigned pending = 0;
#pragma unroll
        for (int k2 = 0; k2 < kMaxPatchVerts; k2++) {
            const int h = (vw[k2 >> 1] >> (16 * (k2 & 1))) & 0xffff;  // deg << 8 | pre
            int deg = h >> 8;
            if (CONTACT_DEG && k2 < nverts) deg += __ldg(fc.vdegc + vid[k2]);
            due[k2] = it * deg + (h & 0xff);
            if (k2 < nverts) {
                vset(k2, make_float4(ver_val(pw[k2][0]), ver_val(pw[k2][1]), ver_val(pw[k2][2]), ver_val(pw[k2][3])));
                if (ver_min(pw[k2][0], pw[k2][1], pw[k2][2]) < due[k2]) pending |= 1u << k2;
            }
        }
        unsigned n = 0;
        while (pending) {
            if (++n > ta.poll_limit || ((n & 63) == 0 && *(volatile unsigned*)ta.abort_flag)) {
                ok = false;
                break;
            }
            __nanosleep(ta.poll_ns);  // polls cost L2 bandwidth the writers need
#pragma unroll
            for (int k2 = 0; k2 < kMaxPatchVerts; k2++) {
                if (pending & (1u << k2)) {
                    unsigned long long a, b, c, d;
                    ld_ver(xv + vid[k2], a, b, c, d);
                    if (ver_min(a, b, c) >= due[k2]) {
                        vset(k2, make_float4(ver_val(a), ver_val(b), ver_val(c), ver_val(d)));
                        pending &= ~(1u << k2);
                    }
                }
            }
        }
    }
#pragma unroll
    for (int u = 0; u < kLamPerLane; u++)
        if (lane + 32 * u < ns) slam[lane + 32 * u] = lt[u];
    __syncwarp();  // slam filled
    if (copy) {
        // the copies land (or not) whatever happened above
        const bool staged = __all_sync(0xffffffffu, mbar_wait_bounded(bar, phase, kWaitLimit)) != 0;
        phase ^= 1u;
        if (!staged) {
            ok = false;
            if (lane == 0) mbar_wait_bounded(bar, phase ^ 1u, kWaitLimit);
        }
    }
    if (!(active && ok)) return;
    const unsigned long long loc =
        HEX ? kHexLocA : ((unsigned long long)(unsigned)meta.z | ((unsigned long long)(unsigned)meta.w << 32));
    bool careful = false;
#pragma unroll
    for (int i = 0; i < kMaxPatchTets; i++) {
        if (!HEX && i >= ntets) break;
        const int r = meta.x + i - s0;
        TetState<float> st;
        unpack_static(srec[0][r], srec[1][r], srec[2][r], st);
        int l[4];
        float4 xp[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            l[q] = (int)((loc >> (12 * i + 3 * q)) & 7ull);
            xp[q] = vget(l[q]);
            st.p[q][0] = xp[q].x; st.p[q][1] = xp[q].y; st.p[q][2] = xp[q].z;
            st.w[q] = fabsf(xp[q].w);
        }
        float2 lam = slam[r];
        float d[4][3], r0, r1, dl0, dl1, J;
        tet_project_combined_fast(st, lam.x, lam.y, r0, r1, dl0, dl1, d, J);
        careful |= !(fabsf(J) >= kDegenerateJ && isfinite(dl0) && isfinite(dl1));
        lam.x += dl0;
        lam.y += dl1;
#pragma unroll
        for (int q = 0; q < 4; q++) vset(l[q], moved(xp[q], d[q]));
        slam[r] = lam;
    }
    if (careful) {
#pragma unroll
        for (int k2 = 0; k2 < kMaxPatchVerts; k2++) {
            if (k2 < nverts) {
                unsigned long long a, b, c, d;
                ld_ver(xv + vid[k2], a, b, c, d);
                vset(k2, make_float4(ver_val(a), ver_val(b), ver_val(c), ver_val(d)));
            }
        }
        for (int i = 0; i < ntets; i++)
            slam[meta.x + i - s0] = (FIRST_ZERO && it == 0) ? make_float2(0.f, 0.f) : t.lam[meta.x + i];
#pragma unroll
        for (int i = 0; i < kMaxPatchTets; i++) {
            if (!HEX && i >= ntets) break;
            const int slot = meta.x + i;
            const int r = slot - s0;
            TetState<float> st;
            unpack_static(srec[0][r], srec[1][r], srec[2][r], st);
            int l[4];
            float4 xp[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                l[q] = (int)((loc >> (12 * i + 3 * q)) & 7ull);
                xp[q] = vget(l[q]);
                st.p[q][0] = xp[q].x; st.p[q][1] = xp[q].y; st.p[q][2] = xp[q].z;
                st.w[q] = fabsf(xp[q].w);
            }
            float2 lam = slam[r];
            float d[4][3];
            double rsq;
            if (project_one<false>(st, t, slot, xp, lam, d, rsq, flags)) {
#pragma unroll
                for (int q = 0; q < 4; q++) vset(l[q], moved(xp[q], d[q]));
            }
            slam[r] = lam;
        }
    }
    // every vertex goes out one version later, moved or not
#pragma unroll
    for (int k2 = 0; k2 < kMaxPatchVerts; k2++) {
        if (k2 < nverts) {
            const float4 sp = vget(k2);
            st_ver(xv + vid[k2], sp.x, sp.y, sp.z, sp.w, (unsigned)(due[k2] + 1));
        }
    }
}

// Warp w runs the w-th task of every colour (the task layout of
// k_sweep_dataflow). A lane's patch reads its vertices when their versions
// are due and writes them back one version later. The smallest unfinished
// task always has its vertices due and its warp at it (all blocks are
// co-resident), so the waits end; each is bounded anyway, and one that gives
// up sets abort_flag so that every other waiter leaves. The projections and
// their order are those of the colour launches; the results equal
// k_sweep_dataflow's bit for bit.
// RESIDENT: the warp's tasks' topology (patch record, vertex ids, version
// words: four int4 per lane and task) is read once into shared memory, before
// the wait on the previous kernel, so a phase's first poll does not wait for
// the task, patch and vertex-id loads.
// ta.l2_first: the tet records' bulk copies, the patch records' cp.async and
// the multiplier loads and stores carry an evict-first L2 policy (the build
// sets it when these streams and the vertex records outgrow the L2), so the
// vertex records, which every patch around a vertex polls and writes, stay.
// CONTACTS: after every iteration's patch tasks come the contact tasks
// (FlowContacts): a lane takes one face with an active static contact,
// polls its three vertices, projects the face's contacts in slot order
// (contact_face_gs) and writes the vertices back one version later; a
// vertex's writes per iteration then include its active faces (vdegc).
template <bool FIRST_ZERO, bool RESIDENT, bool CONTACTS, int MINB>
__global__ void __launch_bounds__(kFlowBlock, MINB)
    k_sweep_versioned(TetArrays t, PatchArrays pa, const int4* __restrict__ pver, TaskArrays ta, int iters,
                      VerRec* __restrict__ xv, Flags* flags, ContactArrays ca, FlowContacts fc) {
    static_assert(kFlowBlock == 32, "one warp per block: the topology is indexed by lane");
    extern __shared__ int4 topo[];  // RESIDENT: [task k][meta, verts a, verts b, versions][lane]
    __shared__ float4 sv[kMaxPatchVerts][kFlowBlock];
    __shared__ __align__(128) float4 srec[3][kTaskSlots];  // the task's m0, m1, m2 records
    __shared__ float2 slam[kTaskSlots];                   // and its multipliers
    __shared__ __align__(8) unsigned long long bar;
    // !RESIDENT: the next patch task's records (meta, verts a, verts b, versions) per lane
    __shared__ __align__(16) int4 ring[RESIDENT ? 1 : 2][4][kFlowBlock];
    const int tid = threadIdx.x, lane = tid & 31;
    const int gw = (blockIdx.x * blockDim.x + tid) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    if (lane == 0) mbar_init(&bar, 1);
    __syncwarp();
    unsigned phase = 0;
    // L2 priority of what every sweep streams once (ta.l2_first)
    const unsigned long long pol = l2_policy(ta.l2_first != 0);
    if (RESIDENT) {
        int k = 0;
        for (int j = gw; j < ta.ntasks; j += nw, k++) {
            const int4 tk = __ldg(ta.task + j);
            int4 meta = make_int4(0, 0, 0, 0), va = meta, vb = meta, vr = meta;
            if (lane < tk.y) {
                const int p = tk.x + lane;
                meta = __ldg(pa.meta + p);
                va = __ldg(pa.verts + 2 * (size_t)p);
                vb = __ldg(pa.verts + 2 * (size_t)p + 1);
                vr = __ldg(pver + p);
            }
            topo[(4 * k + 0) * 32 + lane] = meta;
            topo[(4 * k + 1) * 32 + lane] = va;
            topo[(4 * k + 2) * 32 + lane] = vb;
            topo[(4 * k + 3) * 32 + lane] = vr;
        }
        __syncwarp();
    }
    pdl_wait_then_release();
    if (RESIDENT && CONTACTS) {
        // this detection's active faces add to each vertex's writes per iteration
        int k = 0;
        for (int j = gw; j < ta.ntasks; j += nw, k++) {
            const int nv = topo[(4 * k + 0) * 32 + lane].y >> 8;
            const int4 va = topo[(4 * k + 1) * 32 + lane], vb = topo[(4 * k + 2) * 32 + lane];
            const int4 vr = topo[(4 * k + 3) * 32 + lane];
            const int vid[kMaxPatchVerts] = {va.x, va.y, va.z, va.w, vb.x, vb.y, vb.z, vb.w};
            int vw[4] = {vr.x, vr.y, vr.z, vr.w};
#pragma unroll
            for (int k2 = 0; k2 < kMaxPatchVerts; k2++)
                if (k2 < nv) vw[k2 >> 1] += (int)__ldg(fc.vdegc + vid[k2]) << (8 + 16 * (k2 & 1));
            topo[(4 * k + 3) * 32 + lane] = make_int4(vw[0], vw[1], vw[2], vw[3]);
        }
        __syncwarp();
    }
    const int ntot = ta.ntasks + (CONTACTS ? *fc.ntasks : 0);
    // !RESIDENT: software pipeline over this warp's patch tasks. While a task
    // runs, the next one's patch records are on their way into shared memory
    // (cp.async, one ring slot per task, lanes without a patch zero-filled)
    // and the descriptor of the one after that into a register, so a task
    // starts polling without a dependent load. (Each warp cycles through the
    // same tasks every iteration: after its last patch task of an iteration
    // comes its first one, gw.)
    auto next_patch_task = [&](int j) { return j + nw < ta.ntasks ? j + nw : gw; };
    int4 tk_next = make_int4(0, 0, 0, 0);  // descriptor of the task after the next
    int rs = 0;                            // ring slot of the next task's records
    auto stage_records = [&](int4 tk, int slot) {
        const bool on = lane < tk.y;
        const size_t p = on ? (size_t)(tk.x + lane) : 0;
        const unsigned nb = on ? 16u : 0u;
        cp_async16_hint(&ring[slot][0][lane], pa.meta + p, nb, pol);
        cp_async16_hint(&ring[slot][1][lane], pa.verts + 2 * p, nb, pol);
        cp_async16_hint(&ring[slot][2][lane], pa.verts + 2 * p + 1, nb, pol);
        cp_async16_hint(&ring[slot][3][lane], pver + p, nb, pol);
        cp_async_commit();
    };
    auto load_desc = [&](int j) { return __ldg(ta.task + j); };
    if (!RESIDENT && gw < ta.ntasks) {
        stage_records(load_desc(gw), 0);
        tk_next = load_desc(next_patch_task(gw));
    }
    for (int it = 0; it < iters; it++) {
        int k = 0;
        for (int j = gw; j < ntot; j += nw) {
          bool ok = true;
          if (j < ta.ntasks) {
            int4 meta, va, vb, vr;
            if (RESIDENT) {
                meta = topo[(4 * k + 0) * 32 + lane];
                va = topo[(4 * k + 1) * 32 + lane];
                vb = topo[(4 * k + 2) * 32 + lane];
                vr = topo[(4 * k + 3) * 32 + lane];
            } else {
                cp_async_wait_all();  // this task's records (staged one task earlier)
                const int s = RESIDENT ? 0 : rs;
                meta = ring[s][0][lane];
                va = ring[s][1][lane];
                vb = ring[s][2][lane];
                vr = ring[s][3][lane];
                const int jn = next_patch_task(j);
                stage_records(tk_next, s ^ 1);
                tk_next = load_desc(next_patch_task(jn));
                rs ^= 1;
            }
            k++;
            const int ntets = meta.y & 0xff, nverts = meta.y >> 8;
            const int vid[kMaxPatchVerts] = {va.x, va.y, va.z, va.w, vb.x, vb.y, vb.z, vb.w};
            // The first polls go out before anything else the task issues:
            // their round trip is the phase's critical path.
            unsigned long long pw[kMaxPatchVerts][4];
#pragma unroll
            for (int k2 = 0; k2 < kMaxPatchVerts; k2++)
                if (k2 < nverts) ld_ver(xv + vid[k2], pw[k2][0], pw[k2][1], pw[k2][2], pw[k2][3]);
            // The task's static records (a contiguous slot range of at most
            // kTaskSlots) arrive in shared memory by three bulk copies that
            // do not pass through the load/store pipe the polls use.
            // Padding tasks (colour runs are padded to the warp count) have no
            // patch and copy nothing; a range longer than the buffer (never
            // built) is refused without a copy.
            const int s0 = __reduce_min_sync(0xffffffffu, nverts > 0 ? meta.x : INT_MAX);
            const int s1 = __reduce_max_sync(0xffffffffu, nverts > 0 ? meta.x + ntets : 0);
            const bool copy = s1 > s0 && s1 - s0 <= kTaskSlots;
            if (s1 > s0 && !copy) ok = false;
            __syncwarp();  // the previous task's reads of srec are done
            if (copy && lane == 0) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                const unsigned bytes = (unsigned)(s1 - s0) * 16u;
                mbar_arrive_expect_tx(&bar, 3u * bytes);
                tma_load_1d_hint(srec[0], t.m0 + s0, bytes, &bar, pol);
                tma_load_1d_hint(srec[1], t.m1 + s0, bytes, &bar, pol);
                tma_load_1d_hint(srec[2], t.m2 + s0, bytes, &bar, pol);
            }
            // The task's multipliers, read and (after the task) written back by
            // coalesced accesses; only this warp touches them meanwhile. The
            // loads are in flight during the polls and land in slam after them.
            const int ns = copy ? s1 - s0 : 0;
            float2 lt[kLamPerLane];
#pragma unroll
            for (int u = 0; u < kLamPerLane; u++) {
                const int r = lane + 32 * u;
                lt[u] = make_float2(0.f, 0.f);
                if (!(FIRST_ZERO && it == 0) && r < ns) lt[u] = ld_f2_hint(t.lam + s0 + r, pol);
            }
            // Grid hexes (after the build's canonical corner order every one has
            // the layout kHexLocA) keep the patch's vertices in registers.
            const unsigned long long loc =
                (unsigned long long)(unsigned)meta.z | ((unsigned long long)(unsigned)meta.w << 32);
            if (__all_sync(0xffffffffu, nverts == 0 || (ntets == 5 && nverts == 8 && loc == kHexLocA)))
                versioned_patch<FIRST_ZERO, CONTACTS && !RESIDENT, true>(t, ta, fc, xv, flags, meta, vid, vr, it, s0,
                                                                          ns, copy, sv, srec, slam, lt, &bar, phase,
                                                                          ok, pw);
            else
                versioned_patch<FIRST_ZERO, CONTACTS && !RESIDENT, false>(t, ta, fc, xv, flags, meta, vid, vr, it, s0,
                                                                           ns, copy, sv, srec, slam, lt, &bar, phase,
                                                                           ok, pw);
            __syncwarp();  // every lane's multipliers are in slam
#pragma unroll
            for (int u = 0; u < kLamPerLane; u++)
                if (lane + 32 * u < ns) lt[u] = slam[lane + 32 * u];
#pragma unroll
            for (int u = 0; u < kLamPerLane; u++)
                if (lane + 32 * u < ns) st_f2_hint(t.lam + s0 + lane + 32 * u, lt[u], pol);
          } else if (CONTACTS) {
            const int2 ct = fc.task[j - ta.ntasks];
            if (lane < ct.y) {
                const int4 e = fc.face[ct.x + lane];
                const int4 fv = __ldg(fc.vfaces + e.x);  // the sweep's vertex numbering
                const int vid3[3] = {fv.x, fv.y, fv.z};
                const int dw[3] = {e.y & 0xffff, (e.y >> 16) & 0xffff, e.z & 0xffff};
                int due3[3];
                float4 xs[3];
                unsigned pending = 0;
#pragma unroll
                for (int q = 0; q < 3; q++) {
                    due3[q] = it * (dw[q] & 0xff) + (dw[q] >> 8);
                    unsigned long long a, b, c, d;
                    ld_ver(xv + vid3[q], a, b, c, d);
                    xs[q] = make_float4(ver_val(a), ver_val(b), ver_val(c), ver_val(d));
                    if (ver_min(a, b, c) < due3[q]) pending |= 1u << q;
                }
                unsigned n = 0;
                while (pending) {
                    if (++n > ta.poll_limit || ((n & 63) == 0 && *(volatile unsigned*)ta.abort_flag)) {
                        ok = false;
                        break;
                    }
                    __nanosleep(ta.poll_ns);
#pragma unroll
                    for (int q = 0; q < 3; q++) {
                        if (pending & (1u << q)) {
                            unsigned long long a, b, c, d;
                            ld_ver(xv + vid3[q], a, b, c, d);
                            if (ver_min(a, b, c) >= due3[q]) {
                                xs[q].x = ver_val(a);
                                xs[q].y = ver_val(b);
                                xs[q].z = ver_val(c);
                                pending &= ~(1u << q);
                            }
                        }
                    }
                }
                if (ok) {
                    // the face's contacts in slot order (contact_face_gs)
                    for (int sl = 0; sl < ca.S; sl++) {
                        const int slot = sl * ca.F + e.x;
                        if (ca.bary[slot].w != 1.f) continue;
                        float lam = it == 0 ? 0.f : ca.lam[slot];
                        float d[3][3];
                        if (contact_update(ca, slot, xs, d, lam)) {
#pragma unroll
                            for (int q = 0; q < 3; q++) xs[q] = moved(xs[q], d[q]);
                        }
                        ca.lam[slot] = lam;
                    }
#pragma unroll
                    for (int q = 0; q < 3; q++)
                        st_ver(xv + vid3[q], xs[q].x, xs[q].y, xs[q].z, xs[q].w, (unsigned)(due3[q] + 1));
                }
            }
          }
            if (ta.stamp && it == iters - 1) {
                __syncwarp();  // the task's stores are issued
                if (lane == 0) ta.stamp[2 + j] = clock_ns();
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
        double rsq;
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
    float d[4][3];
    double rsq;
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
    // F = [X_0 X_1 X_2] Q (ElementConstraint.hpp:78-119), Q column-major
    const float4 qa = __ldg(t.q0 + slot), qb = __ldg(t.q1 + slot), qc = __ldg(t.q2 + slot);
    const float q[9] = {qa.x, qa.y, qa.z, qa.w, qb.x, qb.y, qb.z, qb.w, qc.x};
    float Ds[9];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int k = 0; k < 3; k++) Ds[3 * i + k] = st.p[i][k] - st.p[3][k];
    const float2 lam = t.lam[slot];
    const float2 m = mat[slot];
    float f[16];
#pragma unroll
    for (int c = 0; c < 3; c++)
#pragma unroll
        for (int k = 0; k < 3; k++) f[3 * c + k] = Ds[k] * q[3 * c] + Ds[3 + k] * q[3 * c + 1] + Ds[6 + k] * q[3 * c + 2];
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
    const float atd = __ldg(t.m1 + slot).w, ath = __ldg(t.m2 + slot).x;
    const float2 lam = t.lam[slot];
    Y[2 * (size_t)i] = atd * lam.x;
    Y[2 * (size_t)i + 1] = ath * lam.y;
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

int sweep_versioned_blocks_per_sm(int min_blocks, int tasks_per_warp, bool contacts) {
    int n = 0, m = 0;
    cudaError_t e = cudaSuccess;
    const size_t smem = sweep_versioned_smem(tasks_per_warp);
    const bool res = tasks_per_warp > 0;
#define XG_VOCC(R, C, M)                                                                                             \
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_sweep_versioned<true, R, C, M>, kFlowBlock, smem);       \
    if (e == cudaSuccess)                                                                                            \
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&m, k_sweep_versioned<false, R, C, M>, kFlowBlock, smem)
#define XG_VOCC_M(R, C)                         \
    if (min_blocks == 8) { XG_VOCC(R, C, 8); }   \
    else if (min_blocks == 6) { XG_VOCC(R, C, 6); } \
    else { XG_VOCC(R, C, 1); }
    if (res) {
        if (contacts) { XG_VOCC_M(true, true) } else { XG_VOCC_M(true, false) }
    } else {
        if (contacts) { XG_VOCC_M(false, true) } else { XG_VOCC_M(false, false) }
    }
#undef XG_VOCC_M
#undef XG_VOCC
    if (e != cudaSuccess) return 0;
    return n < m ? n : m;
}

cudaError_t launch_sweep_versioned(const Launch& s, const TetArrays& t, const PatchArrays& pa, const int4* pver,
                                   const TaskArrays& ta, int iters, bool first_zero, float4* x, VerRec* xv, int V,
                                   const int* vperm, Flags* flags, int grid, int min_blocks, bool resident,
                                   const ContactArrays& ca, const FlowContacts& fc) {
    if (iters <= 0 || ta.ntasks <= 0) return cudaSuccess;
    go(k_versions_in, nblk(V, 256), 256, s, xv, (const float4*)x, vperm, V);
    const int warps = grid * (kFlowBlock / 32);
    const int per_warp = (ta.ntasks + warps - 1) / warps;
    const bool contacts = fc.task != nullptr;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(kFlowBlock);
    cfg.dynamicSmemBytes = resident ? sweep_versioned_smem(per_warp) : 0;
    cfg.stream = s.s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e = cudaSuccess;
#define XG_VER(F, R, C, M) \
    e = cudaLaunchKernelEx(&cfg, k_sweep_versioned<F, R, C, M>, t, pa, pver, ta, iters, xv, flags, ca, fc)
#define XG_VER_M(F, R, C)                       \
    if (min_blocks == 8) { XG_VER(F, R, C, 8); } \
    else if (min_blocks == 6) { XG_VER(F, R, C, 6); } \
    else { XG_VER(F, R, C, 1); }
#define XG_VER_C(F, R)                              \
    if (contacts) { XG_VER_M(F, R, true) } else { XG_VER_M(F, R, false) }
    if (resident) {
        if (first_zero) { XG_VER_C(true, true) } else { XG_VER_C(false, true) }
    } else {
        if (first_zero) { XG_VER_C(true, false) } else { XG_VER_C(false, false) }
    }
#undef XG_VER_C
#undef XG_VER_M
#undef XG_VER
    if (e != cudaSuccess) return e;
    go(k_versions_out, nblk(V, 256), 256, s, x, (const VerRec*)xv, vperm, V);
    return cudaSuccess;
}

// ---- the versioned sweep's contact tables (after each detection) ----
// faces holding at least one active static contact
__global__ void k_face_active(ContactArrays c, unsigned char* __restrict__ factive) {
    pdl_wait_then_release();
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= c.F) return;
    unsigned char a = 0;
    for (int s = 0; s < c.S; s++) a |= c.bary[(size_t)s * c.F + f].w == 1.f;
    factive[f] = a;
}

// active faces containing each vertex
__global__ void k_vertex_contact_degree(const int* __restrict__ vface_off, const int* __restrict__ vface,
                                        const unsigned char* __restrict__ factive, unsigned char* __restrict__ vdegc,
                                        const int* __restrict__ vperm, int V) {
    pdl_wait_then_release();
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V) return;
    int n = 0;
    for (int e = vface_off[v]; e < vface_off[v + 1]; e++) n += factive[vface[e]];
    vdegc[vperm[v]] = (unsigned char)n;  // in the sweep's vertex numbering
}

constexpr int kScanThreads = 1024;

// Colour-major offsets of the active faces (colour, instance) from the
// per-instance lists, and the contact tasks: per colour, runs of up to 32.
// One block.
__global__ void __launch_bounds__(kScanThreads) k_contact_task_table(const int* __restrict__ act_off, int ncol,
                                                                    int n_inst, int* __restrict__ cm_off,
                                                                    int2* __restrict__ ctask,
                                                                    int* __restrict__ n_ctasks) {
    __shared__ int part[kScanThreads];
    __shared__ int col_tasks_off[kMaxFlowFaceColours + 1];
    pdl_wait_then_release();
    const int tid = threadIdx.x;
    const int n = ncol * n_inst;
    const int per = (n + kScanThreads - 1) / kScanThreads;
    const int lo = min(n, tid * per), hi = min(n, lo + per);
    auto count = [&](int i) {
        const int col = i / n_inst, k = i % n_inst;
        const int* a = act_off + (size_t)k * (ncol + 1);
        return a[col + 1] - a[col];
    };
    int sum = 0;
    for (int i = lo; i < hi; i++) sum += count(i);
    part[tid] = sum;
    __syncthreads();
    if (tid == 0) {
        int run = 0;
        for (int i = 0; i < kScanThreads; i++) {
            const int v = part[i];
            part[i] = run;
            run += v;
        }
    }
    __syncthreads();
    int run = part[tid];
    for (int i = lo; i < hi; i++) {
        cm_off[i] = run;
        run += count(i);
    }
    if (tid == kScanThreads - 1) cm_off[n] = run;
    __syncthreads();
    if (tid == 0) {
        int t = 0;
        for (int col = 0; col < ncol; col++) {
            col_tasks_off[col] = t;
            const int tot = cm_off[(col + 1) * n_inst] - cm_off[col * n_inst];
            t += (tot + 31) / 32;
        }
        col_tasks_off[ncol] = t;
        *n_ctasks = t;
    }
    __syncthreads();
    for (int col = 0; col < ncol; col++) {
        const int base = cm_off[col * n_inst], tot = cm_off[(col + 1) * n_inst] - base;
        const int t0 = col_tasks_off[col], nt = col_tasks_off[col + 1] - t0;
        for (int i = tid; i < nt; i += kScanThreads) ctask[t0 + i] = make_int2(base + 32 * i, min(32, tot - 32 * i));
    }
}

// The colour-major face entries with, per face vertex, its writes per
// iteration (patches + active faces) and those before this face (patches +
// active faces of a lower colour). One block per instance.
__global__ void k_contact_faces_fill(ContactArrays c, const int* __restrict__ act_faces,
                                     const int* __restrict__ act_off, int ncol, int n_inst,
                                     const int* __restrict__ cm_off, const int* __restrict__ vface_off,
                                     const int* __restrict__ vface, const int* __restrict__ fcol,
                                     const unsigned char* __restrict__ vdegp,
                                     const unsigned char* __restrict__ factive, int4* __restrict__ cface) {
    pdl_wait_then_release();
    const int k = blockIdx.x;
    const int* a = act_off + (size_t)k * (ncol + 1);
    for (int col = 0; col < ncol; col++) {
        const int dst0 = cm_off[col * n_inst + k];
        for (int i = a[col] + threadIdx.x; i < a[col + 1]; i += blockDim.x) {
            const int f = act_faces[i];
            const int4 fv = c.faces[f];
            const int vs[3] = {fv.x, fv.y, fv.z};
            int w[3];
            for (int q = 0; q < 3; q++) {
                const int v = vs[q];
                int deg = 0, pre = 0;
                for (int e = vface_off[v]; e < vface_off[v + 1]; e++) {
                    const int g = vface[e];
                    if (factive[g]) {
                        deg++;
                        pre += fcol[g] < col;
                    }
                }
                w[q] = (vdegp[v] + deg) | ((vdegp[v] + pre) << 8);
            }
            cface[dst0 + (i - a[col])] = make_int4(f, w[0] | (w[1] << 16), w[2], 0);
        }
    }
}

void launch_stamp(const Launch& s, unsigned long long* p) { go(k_stamp, 1, 1, s, p); }

void launch_flow_contact_tables(const Launch& s, const ContactArrays& ca, const int* act_faces, const int* act_off,
                                int ncol, int n_inst, const int* vface_off, const int* vface, const int* fcol,
                                const unsigned char* vdegp, unsigned char* factive, int* cm_off, int2* ctask,
                                int* n_ctasks, int4* cface, unsigned char* vdegc, const int* vperm, int V) {
    go(k_face_active, nblk(ca.F, 256), 256, s, ca, factive);
    go(k_vertex_contact_degree, nblk(V, 256), 256, s, vface_off, vface, (const unsigned char*)factive, vdegc, vperm,
       V);
    go(k_contact_task_table, 1, kScanThreads, s, act_off, ncol, n_inst, cm_off, ctask, n_ctasks);
    go(k_contact_faces_fill, n_inst, 256, s, ca, act_faces, act_off, ncol, n_inst, (const int*)cm_off, vface_off,
       vface, fcol, vdegp, (const unsigned char*)factive, cface);
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
