// Self-collisions on the device: grid binning of the tets, the point-in-tet
// query of the surface vertices, the closest rest face, and the
// DeformableDeformableCollisionConstraint projections.
//   src/simobject/XPBDMeshObject.cpp:719-762 (selfCollisionCheck)
//   src/geometry/embree/EmbreeScene.cpp:369-393, EmbreeTetMeshGeometry.cpp:20-47
//   src/geometry/DeformableMeshSDF.cpp:68-82
#include "xpbd_device.cuh"

namespace xg {

namespace {

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

}  // namespace

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

}  // namespace xg
