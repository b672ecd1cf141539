// Private host-side state of one solver context (the opaque xpbd_ctx of
// include/xpbd_gpu.h) and the error / profiling helpers shared by the C ABI
// translation units.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/xpbd_gpu.h"
#include "xpbd_kernels.cuh"

namespace xg {

template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    cudaError_t alloc(size_t count) {
        n = count;
        if (count == 0) return cudaSuccess;
        return cudaMalloc((void**)&p, count * sizeof(T));
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

struct Prof {
    bool on = false;
    std::vector<cudaEvent_t> pool;
    std::vector<int> ids;  // kernel id per recorded pair
    size_t used = 0;
};

}  // namespace xg

using xg::DevBuf;
using xg::Flags;
using xg::Launch;
using xg::PatchArrays;
using xg::Prof;
using xg::TetArrays;
using xg::ContactArrays;

struct xpbd_ctx {
    xpbd_params prm{};
    int V = 0, T = 0, F = 0;
    int block = 256;
    cudaStream_t stream = nullptr;
    std::string err;
    long long launches = 0;

    // host mirrors
    std::vector<double> inv_mass_h;     // V, positive
    std::vector<uint8_t> fixed_h;       // V
    std::vector<double> mass_h;         // V
    std::vector<int> tet_of_slot;       // T
    std::vector<int> tets_h, faces_h;   // 4T, 3F (original order)
    std::vector<int> tet_colour;        // T, by original index
    std::vector<int> fcol_off;          // face colour ranges over face_list
    int n_tet_colours = 1, n_face_colours = 0;
    std::vector<float> alpha_t_d, alpha_t_h;  // per slot, for energy

    // device state
    DevBuf<float4> x, prev, vel, dx, dxt;
    DevBuf<int4> tet_idx;
    DevBuf<float4> m0, m1, m2;  // projection records (M = Q Q^T, det Q, compliances)
    DevBuf<float4> q0, q1, q2;  // Q, for the network features
    DevBuf<float2> lam;
    DevBuf<int> perm, csr_off, csr_ent;
    DevBuf<int4> faces;
    DevBuf<int> face_list;
    DevBuf<int4> patch_meta, patch_verts;
    std::vector<int> pcol_off;           // patch colour ranges (Gauss-Seidel)
    // local collision iterations: slots in per-tet colour order, masks
    std::vector<int> lcol_off;           // colour ranges over local_slots
    std::vector<int> local_tets_h;       // the same order as tet indices
    DevBuf<int> local_slots;
    DevBuf<unsigned char> vmask, tmask;
    DevBuf<float> gdz;                   // 1st order: per-vertex inertial z move
    // attachment constraints: vertex, attach point + offset (host, double),
    // the device copies, and a colouring so no colour repeats a vertex
    std::vector<int> att_v;
    std::vector<double> att_point, att_offset;  // 3 per attachment
    std::vector<int> att_order, att_col_off;
    bool att_struct_dirty = false, att_target_dirty = false;
    DevBuf<int> d_att_v, d_att_order;
    DevBuf<float4> d_att_target;
    DevBuf<float> d_att_lam;
    // dataflow Gauss-Seidel (sweep variants 2-4): tasks, dependencies, epochs
    int ntasks = 0, flow_grid = 0;
    DevBuf<int4> flow_tasks;
    DevBuf<int> flow_dep_off, flow_dep;
    DevBuf<unsigned> flow_epoch;  // ntasks epochs + the abort flag
    DevBuf<int4> patch_ver;       // variant 4: per patch, 8 x 16-bit deg << 8 | pre
    DevBuf<xg::VerRec> xv;        // variant 4: version-stamped vertex records, in the sweep's numbering:
    DevBuf<int> vperm;            //   vertex -> record (a task's lanes touch neighbouring records)
    DevBuf<int4> pverts_v;        //   patch vertices and
    DevBuf<int4> faces_v;         //   surface faces in that numbering
    bool flow_resident = false;   // variant 4: task topology kept in shared memory
    // variant 4 with static contacts inside the sweep (FlowContacts)
    bool flow_contacts = false;
    DevBuf<unsigned char> vdeg_p, vdeg_c, factive;  // patches / active faces per vertex, face flags
    DevBuf<int> vface_off, vface, fcol_d, cm_off, n_ctasks;
    DevBuf<int2> ctask;
    DevBuf<int4> cface;
    int npatches = 0;
    bool flow_versioned = false;  // variant 4 tables built (else variant 2 runs)
    std::vector<int4> patch_ver_h;  // host copy of patch_ver
    unsigned flow_poll_limit = xg::kFlowLimit;
    unsigned flow_poll_ns = xg::kPollNs;
    bool flow_l2_first = false;  // variant 4: streamed records evict-first (gs_l2_stream)
    // per-instance latency stamps (xpbd_set_latency_stamps): [0] substep start,
    // [1] substep end, [2 + j] task j's end of its last iteration
    DevBuf<unsigned long long> lat;
    bool lat_on = false, lat_have = false;
    std::vector<int2> task_inst_h;  // patch task -> first and last instance it touches
    std::vector<int> vperm_h;       // the versioned sweep's vertex numbering (vertex -> record)
    DevBuf<float4> c_bary, c_p, c_n;
    DevBuf<float> c_lam;
    int S = 4;
    // instances (batched objects): offsets into the concatenated arrays
    int n_inst = 1;
    std::vector<int64_t> voff, toff, foff;
    std::vector<float4> sphere_tab_h;  // [n_inst * S] SDF primitives, 3 float4 each (kind < 0 = empty)
    DevBuf<float4> sphere_tab;
    std::vector<double> sdf_pose_h;    // [n_inst * S] * 10: position, quaternion, dims as given (double)
    // free rigid bodies (two-way coupling): FP64 records (xg::kRigidRec each)
    int nbodies = 0;
    std::vector<double> body_h;        // host copy, current after pull_bodies
    DevBuf<double> rb;                 // capacity n_inst * S records
    DevBuf<int> rc_list, rc_count;     // rigid contacts in slot order, their count
    // static contacts by instance and face colour: all faces (ifl, ifo_off) and,
    // after each detection, those with an active contact (act_faces, act_off)
    DevBuf<int> ifl, ifo_off, act_faces, act_off;
    bool contact_lists_dirty = true;
    // self-collisions: grid, binning, hits and contacts (xg::SelfArrays)
    bool self_on = false;
    int n_surf = 0, ncells = 0;
    xg::SelfGrid sgrid{};
    DevBuf<int4> s_tets;
    DevBuf<int2> s_contact;
    DevBuf<double> s_Q, s_X0;
    DevBuf<float4> s_X0f;
    DevBuf<float> s_lam;
    DevBuf<int> s_surf, s_cell_count, s_cell_off, s_cell_fill, s_cell_tets, s_tet_cell, s_overflow, s_n_overflow,
        s_hit_tet, s_hit_list, s_n_hits, s_scan_part;
    DevBuf<int> face_inst;
    bool sphere_dirty = true;
    int n_spheres_total = 0;
    DevBuf<int> kin_idx;
    DevBuf<float4> kin_rest;
    int nkin = 0;
    DevBuf<Flags> flags;
    DevBuf<double> res_partial, res_rows, energy_partial;
    DevBuf<float> rvec;
    int res_stride = 0;   // doubles per residual row
    bool have_rvec = false;
    std::vector<int> api_slots;  // contacts added through the API per face

    // pinned staging
    float4* h_stage = nullptr;
    // the device addresses pageable host memory coherently (Grace-Blackwell):
    // positions cross the boundary by kernels on the caller's own arrays
    bool host_direct = false;
    double* h_rows = nullptr;
    int h_rows_cap = 0;
    int last_rows = 0;
    bool rows_pending = false;

    // host simulation clock (Simulation.cpp:197-276)
    double time = 0, last_cd = 0;

    // graphs: [write_vel]
    // captured substep bodies: update, step (update + velocities), solve only
    cudaGraphExec_t gexec[3] = {nullptr, nullptr, nullptr};
    long long graph_kernels[3] = {0, 0, 0};  // kernels captured in each graph
    bool graph_dirty = true;

    Prof prof;

    // learned warm start (MLP on the tensor cores) and its online training
    int warm_mode = 0;                 // XPBD_WARM_*
    bool record = false;               // keep (features, solved multipliers) of each substep
    bool recorded = false;             // a substep has been recorded since record was set
    bool mlp_ready = false;            // parameters initialised and packed
    int adam_t = 0;                    // Adam steps taken
    DevBuf<float> mlp_p, mlp_m, mlp_v, mlp_g, mlp_w4f;  // kMlpParams each (w4f: 128)
    DevBuf<__nv_bfloat16> mlp_tiles;   // packed operand tiles W1|W2|W3|W4|W2t|W3t
    DevBuf<float2> mat;                // per slot: log10(E)/5, nu
    DevBuf<__nv_bfloat16> feat;        // [T][16] features of the last substep
    DevBuf<float> pred, target;        // [T][2] network output, recorded targets
    DevBuf<float4> x_pred;             // V: predicted positions (fallback restore)
    DevBuf<unsigned long long> warm_stats;  // kept, rejected warm starts
    DevBuf<double> warm_rows, mse;     // 2 residual sums; loss accumulator
    int cache_rows = 0;                // training cache capacity (rows)
    DevBuf<float> cache_z, cache_out;
    DevBuf<__nv_bfloat16> cache_a;

    xg::MlpNet net() {
        __nv_bfloat16* b = mlp_tiles.p;
        const int w1 = 64 * 16, w2 = 64 * 64, w4 = 16 * 64;
        return xg::MlpNet{b,           b + w1,          b + w1 + w2, b + w1 + 2 * w2, b + w1 + 2 * w2 + w4,
                          b + w1 + 3 * w2 + w4, mlp_p.p + xg::kOffB1, mlp_p.p + xg::kOffB2, mlp_p.p + xg::kOffB3,
                          mlp_p.p + xg::kOffB4, mlp_w4f.p};
    }

    xg::TaskArrays tasks() {
        return xg::TaskArrays{flow_tasks.p,       flow_dep_off.p, flow_dep.p,      flow_epoch.p,
                              flow_epoch.p + ntasks, ntasks,        flow_poll_limit, flow_poll_ns,
                              lat_on ? lat.p : nullptr, flow_l2_first ? 1u : 0u};
    }
    xg::FlowContacts flowc() {
        return xg::FlowContacts{ctask.p, cface.p, n_ctasks.p, vdeg_c.p, faces_v.p};
    }
    xg::SelfArrays selfs() {
        return xg::SelfArrays{s_tets.p,        s_Q.p,          s_X0.p,         s_X0f.p,      s_surf.p,
                              n_surf,          s_cell_count.p, s_cell_off.p,   s_cell_fill.p, s_cell_tets.p,
                              s_tet_cell.p,    s_overflow.p,   s_n_overflow.p, s_hit_tet.p,  s_hit_list.p,
                              s_n_hits.p,      s_contact.p,    s_lam.p,        s_scan_part.p, T,
                              F};
    }
    TetArrays tets() {
        return TetArrays{tet_idx.p, m0.p, m1.p, m2.p, lam.p, q0.p, q1.p, q2.p};
    }
    Launch L() const { return Launch{stream, prm.use_pdl != 0}; }
    PatchArrays patches() const { return PatchArrays{patch_meta.p, patch_verts.p}; }
    PatchArrays patches_v() const { return PatchArrays{patch_meta.p, pverts_v.p}; }  // the versioned sweep's
    ContactArrays contacts() {
        return ContactArrays{c_bary.p, c_p.p, c_n.p, c_lam.p, faces.p, F, S};
    }
};

namespace xg {

inline int fail(xpbd_ctx* c, int code, const char* fmt, ...) {
    if (c) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        c->err = buf;
    }
    return code;
}

inline int cuda_check(xpbd_ctx* c, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return XPBD_OK;
    return fail(c, XPBD_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define XPBD_CU(ctx, call)                                         \
    do {                                                           \
        int _st = cuda_check((ctx), (call), #call);                \
        if (_st != XPBD_OK) return _st;                            \
    } while (0)

inline int after_launches(xpbd_ctx* c, const char* what) {
    return cuda_check(c, cudaGetLastError(), what);
}

// ---- profiling brackets (only when prof.on) ----
inline void prof_begin(xpbd_ctx* c, int id) {
    if (!c->prof.on) return;
    if (c->prof.used + 2 > c->prof.pool.size()) {
        size_t old = c->prof.pool.size();
        c->prof.pool.resize(std::max<size_t>(256, old * 2));
        for (size_t i = old; i < c->prof.pool.size(); i++) cudaEventCreate(&c->prof.pool[i]);
    }
    cudaEventRecord(c->prof.pool[c->prof.used], c->stream);
    c->prof.ids.push_back(id);
}
inline void prof_end(xpbd_ctx* c) {
    if (!c->prof.on) return;
    cudaEventRecord(c->prof.pool[c->prof.used + 1], c->stream);
    c->prof.used += 2;
}

struct Scope {
    xpbd_ctx* c;
    Scope(xpbd_ctx* c_, int id) : c(c_) {
        prof_begin(c, id);
        c->launches++;
    }
    ~Scope() { prof_end(c); }
};

}  // namespace xg
