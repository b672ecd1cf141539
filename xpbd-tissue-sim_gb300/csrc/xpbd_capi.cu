// C ABI of the GB300 XPBD solver (declared in include/xpbd_gpu.h).
//
// Host side of one XPBDMeshObject_ + XPBDSolver pair: builds the device
// layout (rest shapes, compliances, lumped masses, colouring, CSR), drives the
// substep on one CUDA stream, captures the substep into a CUDA graph, and
// reports errors as status codes instead of the reference's assert(0)
// (include/gpu/resource/GPUResource.hpp:8-19).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/xpbd_gpu.h"
#include "xpbd_ctx.cuh"
#include "xpbd_kernels.cuh"

using namespace xg;

namespace {

bool valid_params(const xpbd_params& p) {
    return p.dt > 0 && std::isfinite(p.dt) && std::isfinite(p.g_accel) && p.num_iters >= 0 &&
           (p.solver_type == XPBD_SOLVER_GAUSS_SEIDEL || p.solver_type == XPBD_SOLVER_JACOBI) &&
           (p.constraint_type == XPBD_CONSTRAINT_COMBINED || p.constraint_type == XPBD_CONSTRAINT_SEPARATE) &&
           p.residual_policy >= XPBD_RESIDUAL_NEVER && p.residual_policy <= XPBD_RESIDUAL_EVERY_ITERATION &&
           (p.jacobi_variant == XPBD_JACOBI_ATOMIC || p.jacobi_variant == XPBD_JACOBI_GATHER) &&
           (p.block_size == 0 || (p.block_size >= 32 && p.block_size <= 256 && p.block_size % 32 == 0)) &&
           p.max_contacts_per_face >= 0 && p.max_contacts_per_face <= kMaxSpheres &&
           (p.use_graphs == 0 || p.use_graphs == 1) && (p.use_pdl == 0 || p.use_pdl == 1) &&
           p.gs_patch_tets >= 0 && p.gs_patch_tets <= kMaxPatchTets &&
           (p.gs_min_blocks == 0 || p.gs_min_blocks == 6 || p.gs_min_blocks == 8) &&
           p.gs_variant >= 0 && p.gs_variant <= 4 && p.num_local_collision_iters >= 0 &&
           p.num_local_collision_iters <= 1000 && (p.first_order == 0 || p.first_order == 1) &&
           (p.adjust_damping_to_material == 0 || p.adjust_damping_to_material == 1) &&
           (p.first_order == 0 || (p.damping_multiplier > 0 && std::isfinite(p.damping_multiplier))) &&
           (p.self_collisions == 0 || p.self_collisions == 1);
}

// The colour-launch kernel that stands in for a GS variant where the one-launch
// sweeps do not apply (contacts, attachments, residual every iteration):
// 0 = registers, 1 = staged records.
int patch_kernel_variant(int gs_variant) { return gs_variant == 1 || gs_variant == 3 ? 1 : 0; }

// Gauss-Seidel patch: a run of consecutive tets on at most kMaxPatchVerts
// vertices, each tet sharing a vertex with the run.
struct HostPatch {
    int first = 0, n = 0, nv = 0;
    int v[kMaxPatchVerts] = {-1, -1, -1, -1, -1, -1, -1, -1};
    unsigned long long loc = 0;
    int local(int vert) const {
        for (int k = 0; k < nv; k++)
            if (v[k] == vert) return k;
        return -1;
    }
};

std::vector<HostPatch> build_patches(const std::vector<int>& tets, int T, int cap) {
    std::vector<HostPatch> out;
    HostPatch cur;
    for (int t = 0; t < T; t++) {
        const int* e = &tets[4 * (size_t)t];
        bool fits = cur.n > 0 && cur.n < cap;
        if (fits) {
            int fresh = 0;
            bool shares = false;
            for (int k = 0; k < 4; k++) {
                if (cur.local(e[k]) >= 0) shares = true;
                else fresh++;
            }
            fits = shares && cur.nv + fresh <= kMaxPatchVerts;
        }
        if (!fits && cur.n > 0) {
            out.push_back(cur);
            cur = HostPatch();
        }
        if (cur.n == 0) cur.first = t;
        for (int k = 0; k < 4; k++) {
            int l = cur.local(e[k]);
            if (l < 0) {
                l = cur.nv;
                cur.v[cur.nv++] = e[k];
            }
            cur.loc |= (unsigned long long)l << (12 * cur.n + 3 * k);
        }
        cur.n++;
    }
    if (cur.n > 0) out.push_back(cur);
    return out;
}

// greedy vertex-disjoint colouring in item order (smallest free colour);
// entries < 0 in an item are padding
int greedy_colour(long long n, int arity, const int* items, long long nv, int* out) {
    std::vector<std::vector<uint64_t>> used;
    used.emplace_back((size_t)nv, 0);
    int ncol = 0;
    for (long long t = 0; t < n; t++) {
        const int* it = items + (size_t)arity * t;
        int c = -1;
        for (size_t w = 0; c < 0; w++) {
            if (w == used.size()) used.emplace_back((size_t)nv, 0);
            uint64_t m = 0;
            for (int k = 0; k < arity; k++)
                if (it[k] >= 0) m |= used[w][(size_t)it[k]];
            if (~m) c = (int)(64 * w) + __builtin_ctzll(~m);
        }
        out[t] = c;
        for (int k = 0; k < arity; k++)
            if (it[k] >= 0) used[(size_t)c / 64][(size_t)it[k]] |= 1ull << (c % 64);
        ncol = std::max(ncol, c + 1);
    }
    return ncol;
}

// ---- residual bookkeeping ----
bool tracking(const xpbd_ctx* c) { return c->prm.residual_policy != XPBD_RESIDUAL_NEVER; }

ResidualSink no_sink() { return ResidualSink{nullptr, 0, 0, 0}; }
ResidualSink sink(xpbd_ctx* c, int row, int offset) { return ResidualSink{c->res_partial.p, row, c->res_stride, offset}; }

// Residual scratch: `rows` rows of per-block partials, their FP64 sums and a
// pinned host copy. Growing a buffer invalidates captured graphs, which hold
// its address.
int ensure_residual_rows(xpbd_ctx* c, int rows) {
    const size_t need = (size_t)rows * c->res_stride;
    if (c->res_partial.n < need) {
        XPBD_CU(c, cudaStreamSynchronize(c->stream));
        c->res_partial.release();
        XPBD_CU(c, c->res_partial.alloc(need));
        c->graph_dirty = true;
    }
    if (c->res_rows.n < (size_t)rows) {
        XPBD_CU(c, cudaStreamSynchronize(c->stream));
        c->res_rows.release();
        XPBD_CU(c, c->res_rows.alloc(rows));
        c->graph_dirty = true;
    }
    if (c->h_rows_cap < rows) {
        XPBD_CU(c, cudaStreamSynchronize(c->stream));
        double* nh = nullptr;
        XPBD_CU(c, cudaMallocHost((void**)&nh, sizeof(double) * rows));
        std::fill(nh, nh + rows, 0.0);
        if (c->h_rows) {
            std::copy(c->h_rows, c->h_rows + c->h_rows_cap, nh);
            cudaFreeHost(c->h_rows);
        }
        c->h_rows = nh;
        c->h_rows_cap = rows;
        c->graph_dirty = true;
    }
    return XPBD_OK;
}

void exact_residual_row(xpbd_ctx* c, int row, bool with_vec) {
    Scope s(c, K_RESIDUAL);
    launch_residual(c->L(), c->block, c->tets(), c->T, c->x.p, c->prm.constraint_type == XPBD_CONSTRAINT_SEPARATE,
                    c->perm.p, with_vec ? c->rvec.p : nullptr, sink(c, row, 0), nullptr,
                    (float)(c->prm.dt * c->prm.dt));
}

// r(x, 0): the residual at the current positions with every multiplier 0
void zero_lambda_residual_row(xpbd_ctx* c, int row) {
    Scope s(c, K_RESIDUAL);
    launch_residual(c->L(), c->block, c->tets(), c->T, c->x.p, c->prm.constraint_type == XPBD_CONSTRAINT_SEPARATE,
                    c->perm.p, nullptr, sink(c, row, 0), nullptr, (float)(c->prm.dt * c->prm.dt), true);
}

// network features of every tet at the predicted positions
void enqueue_features(xpbd_ctx* c) {
    Scope sc(c, K_WARM);
    launch_mlp_features(c->L(), c->tets(), c->x.p, c->mat.p, (float)(c->prm.dt * 1e3), 0, c->T, c->feat.p);
}

// Warm start of one substep (after prediction): lambda_0 from the network or
// the previous substep, x += M^-1 grad C^T lambda_0, and the residual-triggered
// fallback to (x_pred, lambda = 0) when ||r(x_warm, lambda_0)|| > ||r(x_pred, 0)||.
void enqueue_warm_start(xpbd_ctx* c) {
    cudaStream_t s = c->stream;
    const bool mlp = c->warm_mode == XPBD_WARM_MLP;
    const int r0 = c->prm.num_iters + 2;  // two scratch rows past the history
    double* rows = c->res_partial.p + (size_t)r0 * c->res_stride;
    cudaMemsetAsync(rows, 0, sizeof(double) * 2 * (size_t)c->res_stride, s);
    if (mlp || c->record) enqueue_features(c);
    if (mlp) {
        Scope sc(c, K_MLP);
        launch_mlp_forward(s, c->feat.p, c->T, c->net(), c->pred.p, nullptr, &c->flags.p->timeouts);
    }
    zero_lambda_residual_row(c, r0);
    cudaMemcpyAsync(c->x_pred.p, c->x.p, sizeof(float4) * (size_t)c->V, cudaMemcpyDeviceToDevice, s);
    {
        Scope sc(c, K_WARM);
        launch_warm_start(c->L(), c->tets(), c->T, mlp ? c->pred.p : nullptr, c->x.p, c->dx.p);
    }
    {
        Scope sc(c, K_APPLY);
        launch_apply(c->L(), c->x.p, c->dx.p, c->V, c->prev.p, c->vel.p, false, (float)c->prm.dt, false);
    }
    exact_residual_row(c, r0 + 1, false);
    {
        Scope sc(c, K_REDUCE);
        launch_reduce_rows(c->L(), rows, 2, c->res_stride, c->warm_rows.p);
    }
    Scope sc(c, K_WARM);
    launch_warm_fallback(c->L(), c->warm_rows.p, c->x.p, c->x_pred.p, c->lam.p, c->V, c->T, c->warm_stats.p);
}

// Local collision iterations after the global solve
// (XPBDMeshObject_::_projectConstraints, XPBDMeshObject.cpp:472-505, with
// _gatherProjectorsForLocalCollisionIterations, :764-825): every contact plus
// the tets attached to a vertex of a contact projected with lambda != 0, for
// num_local_collision_iters passes without re-initialising lambda, elastic
// projectors before collision projectors (the projector type order). A tet
// the reference lists once per incident contact vertex is projected once per
// pass here, in per-tet colour order (Gauss-Seidel) or from the same x
// (Jacobi).
void enqueue_local_collision_iters(xpbd_ctx* c) {
    const xpbd_params& p = c->prm;
    const bool separate = p.constraint_type == XPBD_CONSTRAINT_SEPARATE;
    const ContactArrays ca = c->contacts();
    cudaMemsetAsync(c->vmask.p, 0, (size_t)c->V, c->stream);
    {
        Scope sc(c, K_LOCAL);
        launch_mark_local(c->L(), ca, c->tets(), c->T, c->vmask.p, c->tmask.p);
    }
    const int ncol = (int)c->lcol_off.size() - 1;
    for (int it = 0; it < p.num_local_collision_iters; it++) {
        if (p.solver_type == XPBD_SOLVER_GAUSS_SEIDEL) {
            for (int pass = 0; pass < (separate ? 2 : 1); pass++)
                for (int col = 0; col < ncol; col++) {
                    Scope sc(c, K_PROJECT_GS);
                    launch_project_local_gs(c->L(), c->tets(), c->local_slots.p, c->lcol_off[col], c->lcol_off[col + 1],
                                            c->tmask.p, c->x.p, separate ? pass : 2, c->flags.p);
                }
            {
                Scope sc(c, K_CONTACT);
                launch_contacts_gs_lists(c->L(), ca, c->act_faces.p, c->act_off.p, c->n_face_colours, c->n_inst,
                                         c->x.p, false);
            }
        } else {
            {
                Scope sc(c, K_PROJECT_JACOBI);
                launch_project_local_jacobi(c->L(), c->tets(), c->T, c->tmask.p, c->x.p, c->dx.p, separate, c->flags.p);
            }
            {
                Scope sc(c, K_CONTACT);
                launch_contacts_jacobi(c->L(), ca, c->x.p, c->dx.p, false);
            }
            Scope sc(c, K_APPLY);
            launch_apply(c->L(), c->x.p, c->dx.p, c->V, c->prev.p, c->vel.p, false, (float)p.dt, false);
        }
    }
}

// ---- the substep body (XPBDMeshObject_::update, XPBDMeshObject.cpp:426-505) ----
// DeformableDeformableCollisionConstraint's alpha = 1e-8 (its Constraint
// base, DeformableDeformableCollisionConstraint.cpp:12-18) over dt^2 (or dt)
float self_alpha_tilde(const xpbd_ctx* c) {
    return (float)(1e-8 / (c->prm.first_order ? c->prm.dt : c->prm.dt * c->prm.dt));
}

int enqueue_update(xpbd_ctx* c, bool write_vel) {
    const xpbd_params& p = c->prm;
    const int iters = p.num_iters;
    const bool track = tracking(c);
    const bool every_iter = p.residual_policy == XPBD_RESIDUAL_EVERY_ITERATION;
    const bool separate = p.constraint_type == XPBD_CONSTRAINT_SEPARATE;
    const float dt = (float)p.dt;
    const float dz = (float)(-p.g_accel * p.dt * p.dt);
    cudaStream_t s = c->stream;
    const ContactArrays ca = c->contacts();
    const bool have_faces = c->F > 0;
    {
        Scope sc(c, K_PREDICT);
        if (p.first_order) launch_predict_first_order(c->L(), c->x.p, c->prev.p, c->gdz.p, c->V);
        else launch_predict(c->L(), c->x.p, c->prev.p, c->vel.p, c->V, dt, dz);
    }
    const bool warm = c->warm_mode != XPBD_WARM_NONE;
    if (track) cudaMemsetAsync(c->res_partial.p, 0, sizeof(double) * (size_t)c->res_stride * (iters + 1), s);
    if (warm) {
        // r(x_pred, 0) before the warm start moves anything
        // (record 0 of the history, also under the every-iteration policy, so
        // relative residuals share the plain start's denominator)
        if (track) zero_lambda_residual_row(c, 0);
        enqueue_warm_start(c);
    } else {
        // features read the previous substep's multipliers: before the reset
        if (c->record) enqueue_features(c);
        // lambda <- 0 (XPBDSolver.hpp:71-77) before the r(x_pred, 0) evaluation
        if (track) cudaMemsetAsync(c->lam.p, 0, sizeof(float2) * (size_t)c->T, s);
    }
    const bool jacobi = p.solver_type == XPBD_SOLVER_JACOBI;
    const bool local = have_faces && p.num_local_collision_iters > 0 && c->local_slots.p;
    const bool fuse_final = !track && !local;
    if (jacobi) {
        const bool gather = p.jacobi_variant == XPBD_JACOBI_GATHER;
        if (track && !every_iter && !warm) exact_residual_row(c, 0, false);
        for (int it = 0; it < iters; it++) {
            // a warm start keeps its multipliers: no iteration treats lambda as 0
            const bool first = it == 0 && !warm;
            const bool first_contact = it == 0;
            const ResidualSink rs = every_iter && !(warm && it == 0) ? sink(c, it, 0) : no_sink();
            const bool last = it == iters - 1;
            if (gather) {
                {
                    Scope sc(c, K_PROJECT_JACOBI);
                    launch_project_jacobi_gather_write(c->L(), c->block, c->tets(), c->T, c->x.p, c->dxt.p, first,
                                                       separate, rs, c->flags.p);
                }
                if (have_faces) {
                    Scope sc(c, K_CONTACT);
                    launch_contacts_jacobi(c->L(), ca, c->x.p, c->dx.p, first_contact);
                }
                if (c->self_on) {
                    Scope sc(c, K_CONTACT);
                    launch_self_contacts(c->L(), c->selfs(), c->faces.p, c->x.p, c->dx.p, true, first_contact,
                                         self_alpha_tilde(c), c->flags.p);
                }
                if (c->nbodies) {
                    Scope sc(c, K_CONTACT);
                    launch_rigid_contacts(c->L(), ca, c->rc_list.p, c->rc_count.p, c->sphere_tab.p, c->face_inst.p,
                                          c->rb.p, c->nbodies, c->x.p, c->dx.p, true, first_contact, c->flags.p);
                }
                if (!c->att_v.empty()) {
                    Scope sc(c, K_CONTACT);
                    launch_attach_jacobi(c->L(), c->d_att_v.p, c->d_att_target.p, c->d_att_lam.p,
                                         (int)c->att_v.size(), c->x.p, c->dx.p, first_contact);
                }
                Scope sc(c, K_GATHER);
                launch_gather_apply(c->L(), c->x.p, c->dxt.p, c->csr_off.p, c->csr_ent.p, c->dx.p, c->V, c->prev.p,
                                    c->vel.p, last && fuse_final, dt, write_vel);
            } else {
                {
                    Scope sc(c, K_PROJECT_JACOBI);
                    launch_project_jacobi(c->L(), c->block, c->tets(), c->T, c->x.p, c->dx.p, first, separate, rs,
                                          c->flags.p);
                }
                if (have_faces) {
                    Scope sc(c, K_CONTACT);
                    launch_contacts_jacobi(c->L(), ca, c->x.p, c->dx.p, first_contact);
                }
                if (c->self_on) {
                    Scope sc(c, K_CONTACT);
                    launch_self_contacts(c->L(), c->selfs(), c->faces.p, c->x.p, c->dx.p, true, first_contact,
                                         self_alpha_tilde(c), c->flags.p);
                }
                if (c->nbodies) {
                    Scope sc(c, K_CONTACT);
                    launch_rigid_contacts(c->L(), ca, c->rc_list.p, c->rc_count.p, c->sphere_tab.p, c->face_inst.p,
                                          c->rb.p, c->nbodies, c->x.p, c->dx.p, true, first_contact, c->flags.p);
                }
                if (!c->att_v.empty()) {
                    Scope sc(c, K_CONTACT);
                    launch_attach_jacobi(c->L(), c->d_att_v.p, c->d_att_target.p, c->d_att_lam.p,
                                         (int)c->att_v.size(), c->x.p, c->dx.p, first_contact);
                }
                Scope sc(c, K_APPLY);
                launch_apply(c->L(), c->x.p, c->dx.p, c->V, c->prev.p, c->vel.p, last && fuse_final, dt, write_vel);
            }
        }
    } else if (!separate && !every_iter && !have_faces && c->att_v.empty() &&
               (p.gs_variant == 2 || p.gs_variant == 3 || p.gs_variant == 4) && c->ntasks > 0) {
        // every iteration and colour in one cooperative launch
        if (track && !warm) exact_residual_row(c, 0, false);
        const bool versioned = p.gs_variant == 4 && c->flow_versioned;
        if (versioned) {
            // the abort flag (after the epochs, which variant 4 does not use)
            cudaMemsetAsync(c->flow_epoch.p + c->ntasks, 0, sizeof(unsigned), s);
        } else {
            cudaMemsetAsync(c->flow_epoch.p, 0, sizeof(unsigned) * (size_t)(c->ntasks + 1), s);
        }
        Scope sc(c, K_PROJECT_GS);
        if (versioned) {
            launch_sweep_versioned(c->L(), c->tets(), c->patches(), c->patch_ver.p, c->tasks(), iters, !warm, c->x.p,
                                   c->xv.p, c->patch_w.p, c->V, c->npatches, c->flags.p, c->flow_grid,
                                   p.gs_min_blocks);
            c->launches += 2;  // the copies into and out of the versioned positions
        } else
            launch_sweep_dataflow(c->L(), c->tets(), c->patches(), c->tasks(), iters, !warm, c->x.p, c->flags.p,
                                  c->flow_grid, p.gs_variant == 3, p.gs_min_blocks);
    } else {
        if (track && !every_iter && !warm) exact_residual_row(c, 0, false);
        for (int it = 0; it < iters; it++) {
            const bool first = it == 0;
            if (every_iter && !(warm && it == 0)) exact_residual_row(c, it, false);
            const int passes = separate ? 2 : 1;
            for (int pass = 0; pass < passes; pass++) {
                const int which = separate ? pass : 2;
                // in the separate form the second pass (Hyd) of iteration 0
                // must not re-zero the Dev multipliers updated by pass 0
                const bool f = first && !warm && (!separate || pass == 0);
                for (int col = 0; col < c->n_tet_colours; col++) {
                    Scope sc(c, K_PROJECT_GS);
                    launch_project_patches(c->L(), c->tets(), c->patches(), c->pcol_off[col], c->pcol_off[col + 1],
                                           c->x.p, f, which, c->flags.p, c->prm.gs_min_blocks ? c->prm.gs_min_blocks : 6,
                                           patch_kernel_variant(c->prm.gs_variant));
                }
            }
            if (have_faces) {
                Scope sc(c, K_CONTACT);
                launch_contacts_gs_lists(c->L(), ca, c->act_faces.p, c->act_off.p, c->n_face_colours, c->n_inst,
                                         c->x.p, first);
            }
            // then the self contacts and the rigid-body contacts (projector type order)
            if (c->self_on) {
                Scope sc(c, K_CONTACT);
                launch_self_contacts(c->L(), c->selfs(), c->faces.p, c->x.p, nullptr, false, first,
                                     self_alpha_tilde(c), c->flags.p);
            }
            if (c->nbodies) {
                Scope sc(c, K_CONTACT);
                launch_rigid_contacts(c->L(), ca, c->rc_list.p, c->rc_count.p, c->sphere_tab.p, c->face_inst.p,
                                      c->rb.p, c->nbodies, c->x.p, nullptr, false, first, c->flags.p);
            }
            // attachments last: the projector type order (XPBDTypedefs.hpp:55-56)
            for (int ac = 0; ac + 1 < (int)c->att_col_off.size(); ac++) {
                Scope sc(c, K_CONTACT);
                launch_attach_gs(c->L(), c->d_att_v.p, c->d_att_target.p, c->d_att_lam.p, c->d_att_order.p,
                                 c->att_col_off[ac], c->att_col_off[ac + 1], c->x.p, first);
            }
        }
    }
    if (c->record) {
        Scope sc(c, K_WARM);
        launch_mlp_targets(c->L(), c->tets(), 0, c->T, c->target.p);
    }
    if (track) {
        exact_residual_row(c, iters, true);
        {
            Scope sc(c, K_REDUCE);
            launch_reduce_rows(c->L(), c->res_partial.p, iters + 1, c->res_stride, c->res_rows.p);
        }
        cudaMemcpyAsync(c->h_rows, c->res_rows.p, sizeof(double) * (iters + 1), cudaMemcpyDeviceToHost, s);
    }
    if (local) enqueue_local_collision_iters(c);
    if (!jacobi || !fuse_final || iters == 0) {
        Scope sc(c, K_FINALIZE);
        launch_finalize(c->L(), c->x.p, c->prev.p, c->vel.p, c->V, dt, write_vel);
    }
    if (c->nbodies) {
        // the rigid objects update after the XPBD objects (Simulation.cpp:245-255,
        // object type order of include/common/SimulationTypeDefs.hpp)
        Scope sc(c, K_FINALIZE);
        launch_rigid_update(c->L(), c->rb.p, c->nbodies, p.dt, p.g_accel);
    }
    if (c->nbodies && write_vel) {
        Scope sc(c, K_VELOCITY);
        launch_rigid_velocity(c->L(), c->rb.p, c->nbodies, p.dt);
    }
    return XPBD_OK;
}

// device copies of the attachments: structure (vertices, colours) when
// attachments were added or cleared, targets whenever an attach point moved
int sync_attachments(xpbd_ctx* c) {
    const int n = (int)c->att_v.size();
    if (c->att_struct_dirty) {
        XPBD_CU(c, cudaStreamSynchronize(c->stream));
        if ((size_t)n > c->d_att_v.n) {
            const size_t cap = std::max<size_t>(64, 2 * (size_t)n);
            c->d_att_v.release(); c->d_att_order.release(); c->d_att_target.release(); c->d_att_lam.release();
            XPBD_CU(c, c->d_att_v.alloc(cap));
            XPBD_CU(c, c->d_att_order.alloc(cap));
            XPBD_CU(c, c->d_att_target.alloc(cap));
            XPBD_CU(c, c->d_att_lam.alloc(cap));
        }
        // greedy colouring by vertex, in insertion order: attachments on one
        // vertex keep their order across colours
        std::vector<int> col(n);
        std::unordered_map<int, int> seen;
        int ncol = 0;
        for (int a = 0; a < n; a++) {
            col[a] = seen[c->att_v[a]]++;
            ncol = std::max(ncol, col[a] + 1);
        }
        c->att_col_off.assign(n ? ncol + 1 : 0, 0);
        for (int a = 0; a < n; a++) c->att_col_off[col[a] + 1]++;
        for (int k = 0; k < ncol; k++) c->att_col_off[k + 1] += c->att_col_off[k];
        c->att_order.assign(n, 0);
        std::vector<int> fill(c->att_col_off.begin(), c->att_col_off.end() - (n ? 1 : 0));
        for (int a = 0; a < n; a++) c->att_order[fill[col[a]]++] = a;
        if (n) {
            XPBD_CU(c, cudaMemcpy(c->d_att_v.p, c->att_v.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
            XPBD_CU(c, cudaMemcpy(c->d_att_order.p, c->att_order.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
            XPBD_CU(c, cudaMemset(c->d_att_lam.p, 0, sizeof(float) * n));
        }
        c->att_struct_dirty = false;
        c->att_target_dirty = true;
        c->graph_dirty = true;
    }
    if (c->att_target_dirty && n) {
        std::vector<float4> tg(n);
        for (int a = 0; a < n; a++)
            tg[a] = make_float4((float)(c->att_point[3 * a] + c->att_offset[3 * a]),
                                (float)(c->att_point[3 * a + 1] + c->att_offset[3 * a + 1]),
                                (float)(c->att_point[3 * a + 2] + c->att_offset[3 * a + 2]), 0.f);
        // pageable source: staged before the call returns, ordered on the stream
        XPBD_CU(c, cudaMemcpyAsync(c->d_att_target.p, tg.data(), sizeof(float4) * n, cudaMemcpyHostToDevice,
                                   c->stream));
    }
    c->att_target_dirty = false;
    return XPBD_OK;
}

int prepare_update(xpbd_ctx* c) {
    int ast = sync_attachments(c);
    if (ast) return ast;
    if (c->F && c->contact_lists_dirty) {
        // the faces with active static contacts, after the contacts changed
        Scope sc(c, K_DETECT);
        launch_contact_lists(c->L(), c->contacts(), c->ifl.p, c->ifo_off.p, c->n_face_colours, c->n_inst,
                             c->act_faces.p, c->act_off.p);
        c->contact_lists_dirty = false;
    }
    if (tracking(c) || c->warm_mode != XPBD_WARM_NONE) {
        // one extra row for on-demand residual queries, two for the warm start
        int st = ensure_residual_rows(c, c->prm.num_iters + 4);
        if (st) return st;
    }
    return XPBD_OK;
}

void drop_graphs(xpbd_ctx* c) {
    for (auto& g : c->gexec)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    c->graph_kernels[0] = c->graph_kernels[1] = 0;
    c->graph_dirty = false;
}

int run_update(xpbd_ctx* c, bool write_vel) {
    int st = prepare_update(c);
    if (st) return st;
    if (c->graph_dirty) drop_graphs(c);
    if (c->prm.use_graphs && !c->prof.on) {
        cudaGraphExec_t& ge = c->gexec[write_vel ? 1 : 0];
        if (!ge) {
            cudaGraph_t g = nullptr;
            XPBD_CU(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
            const long long before = c->launches;
            enqueue_update(c, write_vel);
            c->graph_kernels[write_vel ? 1 : 0] = c->launches - before;
            c->launches = before;
            cudaError_t e = cudaStreamEndCapture(c->stream, &g);
            if (e != cudaSuccess) return cuda_check(c, e, "cudaStreamEndCapture");
            e = cudaGraphInstantiate(&ge, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) {
                ge = nullptr;
                return cuda_check(c, e, "cudaGraphInstantiate");
            }
        }
        XPBD_CU(c, cudaGraphLaunch(ge, c->stream));
        c->launches += c->graph_kernels[write_vel ? 1 : 0];
    } else {
        enqueue_update(c, write_vel);
    }
    c->rows_pending = tracking(c);
    c->last_rows = c->prm.num_iters + 1;
    if (c->record) c->recorded = true;
    if (tracking(c)) c->have_rvec = true;
    return after_launches(c, "update");
}

// ---- free rigid bodies ----
// device records -> body_h (the device state is the current one once steps ran)
int pull_bodies(xpbd_ctx* c) {
    c->body_h.resize((size_t)c->nbodies * kRigidRec);
    if (!c->nbodies) return XPBD_OK;
    XPBD_CU(c, cudaStreamSynchronize(c->stream));
    XPBD_CU(c, cudaMemcpy(c->body_h.data(), c->rb.p, sizeof(double) * c->body_h.size(), cudaMemcpyDeviceToHost));
    return XPBD_OK;
}

// body_h -> device records, and every table entry's body mark (d.w = index + 1)
int push_bodies(xpbd_ctx* c) {
    c->nbodies = (int)(c->body_h.size() / kRigidRec);
    for (size_t e = 0; e < c->sphere_tab_h.size(); e += 3) c->sphere_tab_h[e + 2].w = 0.f;
    for (int i = 0; i < c->nbodies; i++) {
        const size_t e = (size_t)c->body_h[(size_t)i * kRigidRec + RB_ENTRY];
        c->sphere_tab_h[3 * e + 2].w = (float)(i + 1);
    }
    if (c->nbodies)
        XPBD_CU(c, cudaMemcpyAsync(c->rb.p, c->body_h.data(), sizeof(double) * c->body_h.size(),
                                   cudaMemcpyHostToDevice, c->stream));
    // the rigid contacts found so far may name bodies that moved or ended:
    // none is projected before the next detection
    if (c->rc_count.p) XPBD_CU(c, cudaMemsetAsync(c->rc_count.p, 0, sizeof(int), c->stream));
    XPBD_CU(c, cudaStreamSynchronize(c->stream));
    c->sphere_dirty = true;
    c->graph_dirty = true;  // the body count is baked into captured launches
    return XPBD_OK;
}

int detect(xpbd_ctx* c) {
    if (c->F == 0) return XPBD_OK;
    if (c->n_spheres_total == 0) {
        // no SDFs: the object pairs add nothing; self-collisions may
        int st = xpbd_clear_collisions(c);
        if (st) return st;
        if (c->self_on) {
            Scope sc(c, K_DETECT);
            launch_self_detect(c->L(), c->selfs(), c->sgrid, c->x.p, c->faces.p);
        }
        return after_launches(c, "detect");
    }
    if (c->sphere_dirty) {
        // pageable source: the copy is staged before the call returns, so the
        // host table may change right after; the upload is stream-ordered
        XPBD_CU(c, cudaMemcpyAsync(c->sphere_tab.p, c->sphere_tab_h.data(), sizeof(float4) * c->sphere_tab_h.size(),
                                   cudaMemcpyHostToDevice, c->stream));
        c->sphere_dirty = false;
    }
    if (c->nbodies) {
        // free bodies are detected at their current poses
        Scope sc(c, K_DETECT);
        launch_rigid_sync_table(c->L(), c->rb.p, c->nbodies, c->sphere_tab.p);
    }
    {
        Scope sc(c, K_DETECT);
        launch_detect(c->L(), c->contacts(), c->x.p, c->sphere_tab.p, c->face_inst.p);
    }
    if (c->nbodies) {
        Scope sc(c, K_DETECT);
        launch_rigid_compact(c->L(), c->contacts(), c->rc_list.p, c->rc_count.p);
    }
    // self-collision tests run after the object pairs (CollisionScene.cpp:44-50)
    if (c->self_on) {
        Scope sc(c, K_DETECT);
        launch_self_detect(c->L(), c->selfs(), c->sgrid, c->x.p, c->faces.p);
    }
    std::fill(c->api_slots.begin(), c->api_slots.end(), -1);  // unknown until read back
    c->contact_lists_dirty = true;
    return after_launches(c, "detect");
}

int stage_positions_to_device(xpbd_ctx* c, const double* x3v, const float* x3f) {
    for (int i = 0; i < c->V; i++) {
        const float w = (float)c->inv_mass_h[i] * (c->fixed_h[i] ? -1.f : 1.f);
        if (x3v)
            c->h_stage[i] = make_float4((float)x3v[3 * i], (float)x3v[3 * i + 1], (float)x3v[3 * i + 2], w);
        else
            c->h_stage[i] = make_float4(x3f[3 * i], x3f[3 * i + 1], x3f[3 * i + 2], w);
    }
    XPBD_CU(c, cudaMemcpyAsync(c->x.p, c->h_stage, sizeof(float4) * c->V, cudaMemcpyHostToDevice, c->stream));
    XPBD_CU(c, cudaStreamSynchronize(c->stream));
    return XPBD_OK;
}

int fetch(xpbd_ctx* c, const float4* src) {
    XPBD_CU(c, cudaMemcpyAsync(c->h_stage, src, sizeof(float4) * c->V, cudaMemcpyDeviceToHost, c->stream));
    XPBD_CU(c, cudaStreamSynchronize(c->stream));
    return XPBD_OK;
}

void release(xpbd_ctx* c) {
    drop_graphs(c);
    for (auto e : c->prof.pool) cudaEventDestroy(e);
    c->x.release(); c->prev.release(); c->vel.release(); c->dx.release(); c->dxt.release();
    c->tet_idx.release(); c->q0.release(); c->q1.release(); c->q2.release(); c->lam.release();
    c->perm.release(); c->csr_off.release(); c->csr_ent.release(); c->faces.release(); c->face_list.release();
    c->c_bary.release(); c->c_p.release(); c->c_n.release(); c->c_lam.release();
    c->kin_idx.release(); c->kin_rest.release(); c->flags.release();
    c->sphere_tab.release(); c->face_inst.release();
    c->rb.release(); c->rc_list.release(); c->rc_count.release();
    c->ifl.release(); c->ifo_off.release(); c->act_faces.release(); c->act_off.release();
    c->s_tets.release(); c->s_contact.release(); c->s_Q.release(); c->s_X0.release(); c->s_X0f.release();
    c->s_lam.release(); c->s_surf.release(); c->s_cell_count.release(); c->s_cell_off.release();
    c->s_cell_fill.release(); c->s_cell_tets.release(); c->s_tet_cell.release(); c->s_overflow.release();
    c->s_n_overflow.release(); c->s_hit_tet.release(); c->s_hit_list.release(); c->s_n_hits.release();
    c->s_scan_part.release();
    c->patch_meta.release(); c->patch_verts.release();
    c->local_slots.release(); c->vmask.release(); c->tmask.release(); c->gdz.release();
    c->d_att_v.release(); c->d_att_order.release(); c->d_att_target.release(); c->d_att_lam.release();
    c->flow_tasks.release(); c->flow_dep_off.release(); c->flow_dep.release(); c->flow_epoch.release();
    c->patch_ver.release(); c->xv.release(); c->patch_w.release();
    c->res_partial.release(); c->res_rows.release(); c->energy_partial.release(); c->rvec.release();
    c->mlp_p.release(); c->mlp_m.release(); c->mlp_v.release(); c->mlp_g.release(); c->mlp_w4f.release();
    c->mlp_tiles.release(); c->mat.release(); c->feat.release(); c->pred.release(); c->target.release();
    c->x_pred.release(); c->warm_stats.release(); c->warm_rows.release(); c->mse.release();
    c->cache_z.release(); c->cache_out.release(); c->cache_a.release();
    if (c->h_stage) cudaFreeHost(c->h_stage);
    if (c->h_rows) cudaFreeHost(c->h_rows);
    c->h_stage = nullptr;
    c->h_rows = nullptr;
    if (c->stream) cudaStreamDestroy(c->stream);
    c->stream = nullptr;
}

// Dataflow tasks: runs of up to kTaskPatches consecutive patches of one colour
// (tasks therefore in colour order), and for each task the tasks sharing a
// vertex with it, flagged when theirs is the higher colour.
int build_flow_tasks(xpbd_ctx* c, const std::vector<int4>& pmeta, const std::vector<int4>& pverts) {
    const int P = (int)pmeta.size(), V = c->V;
    std::vector<int4> tasks;
    std::vector<int> tcol, task_of(P);
    for (int col = 0; col < c->n_tet_colours; col++)
        for (int q = c->pcol_off[col]; q < c->pcol_off[col + 1]; q += kTaskPatches) {
            const int n = std::min(kTaskPatches, c->pcol_off[col + 1] - q);
            int slots = 0;
            for (int k = 0; k < n; k++) {
                task_of[q + k] = (int)tasks.size();
                // the task's tets form one contiguous slot range (bulk-copied whole)
                if (pmeta[q + k].x != pmeta[q].x + slots)
                    return fail(c, XPBD_ERR_STATE, "dataflow: patch %d does not continue its task's slots", q + k);
                slots += pmeta[q + k].y & 0xff;
            }
            tasks.push_back(make_int4(q, n, pmeta[q].x, slots));
            tcol.push_back(col);
        }
    const int NT = (int)tasks.size();
    auto pv = [&](int q, int k) {
        const int4& a = pverts[2 * (size_t)q + (k >> 2)];
        const int kk = k & 3;
        return kk == 0 ? a.x : (kk == 1 ? a.y : (kk == 2 ? a.z : a.w));
    };
    // vertex -> tasks (CSR, deduplicated)
    std::vector<int> voff(V + 1, 0);
    for (int q = 0; q < P; q++)
        for (int k = 0; k < (pmeta[q].y >> 8); k++) voff[pv(q, k) + 1]++;
    for (int v = 0; v < V; v++) voff[v + 1] += voff[v];
    std::vector<int> vt(voff[V]), fill(voff.begin(), voff.end() - 1);
    for (int q = 0; q < P; q++)
        for (int k = 0; k < (pmeta[q].y >> 8); k++) vt[fill[pv(q, k)]++] = task_of[q];
    // per-task dependency lists
    std::vector<int> doff(NT + 1, 0), dep;
    std::vector<int> scratch;
    for (int j = 0; j < NT; j++) {
        scratch.clear();
        for (int q = tasks[j].x; q < tasks[j].x + tasks[j].y; q++)
            for (int k = 0; k < (pmeta[q].y >> 8); k++) {
                const int v = pv(q, k);
                for (int e = voff[v]; e < voff[v + 1]; e++)
                    if (vt[e] != j) scratch.push_back(vt[e]);
            }
        std::sort(scratch.begin(), scratch.end());
        scratch.erase(std::unique(scratch.begin(), scratch.end()), scratch.end());
        for (int d : scratch) {
            if (tcol[d] == tcol[j]) return fail(c, XPBD_ERR_STATE, "dataflow: tasks %d and %d share a colour and a vertex", j, d);
            dep.push_back((d << 1) | (tcol[d] > tcol[j] ? 1 : 0));
        }
        doff[j + 1] = (int)dep.size();
    }
    const bool staged = c->prm.gs_variant == 3;
    // variant 4 may fall back to variant 2 (below), so its grid fits both
    const int per_sm = c->prm.gs_variant == 4 ? std::min(sweep_versioned_blocks_per_sm(c->prm.gs_min_blocks),
                                                         sweep_dataflow_blocks_per_sm(false, c->prm.gs_min_blocks))
                                              : sweep_dataflow_blocks_per_sm(staged, c->prm.gs_min_blocks);
    int dev = 0, sms = 0;
    XPBD_CU(c, cudaGetDevice(&dev));
    XPBD_CU(c, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    if (per_sm <= 0 || sms <= 0) return fail(c, XPBD_ERR_CUDA, "dataflow sweep: no co-resident blocks");
    c->flow_grid = per_sm * sms;
    if (!staged) {
        // no more warps than the largest colour has tasks
        int maxc = 0;
        for (int j0 = 0; j0 < NT;) {
            int j1 = j0;
            while (j1 < NT && tcol[j1] == tcol[j0]) j1++;
            maxc = std::max(maxc, j1 - j0);
            j0 = j1;
        }
        const int wpb = kFlowBlock / 32;
        c->flow_grid = std::max(1, std::min(c->flow_grid, (maxc + wpb - 1) / wpb));
        // Warp w runs tasks w, w + W, w + 2W, ... (W warps). Each colour's run
        // of tasks is padded with empty tasks to a multiple of W, so warp w
        // gets the k-th task of every colour with k = w mod W: the same part of
        // the mesh colour after colour, whose dependencies are its own earlier
        // tasks and its neighbours'.
        const int W = c->flow_grid * (kFlowBlock / 32);
        std::vector<int> newpos(NT);
        int padded = 0;
        for (int j0 = 0; j0 < NT;) {
            int j1 = j0;
            while (j1 < NT && tcol[j1] == tcol[j0]) j1++;
            for (int j = j0; j < j1; j++) newpos[j] = padded + (j - j0);
            padded += (j1 - j0 + W - 1) / W * W;
            j0 = j1;
        }
        std::vector<int4> tp(padded, make_int4(0, 0, 0, 0));
        std::vector<int> real(padded, -1);
        for (int j = 0; j < NT; j++) {
            tp[newpos[j]] = tasks[j];
            real[newpos[j]] = j;
        }
        std::vector<int> dp_off(padded + 1, 0), dp;
        for (int i = 0; i < padded; i++) {
            if (real[i] >= 0)
                for (int e = doff[real[i]]; e < doff[real[i] + 1]; e++) {
                    const int d = newpos[dep[e] >> 1];
                    // the same warp ran that task earlier (this iteration for a
                    // lower colour, the previous one for a higher): program
                    // order and the warp barrier before the loads cover it
                    if (d % W == i % W) continue;
                    dp.push_back((d << 1) | (dep[e] & 1));
                }
            dp_off[i + 1] = (int)dp.size();
        }
        tasks.swap(tp);
        doff.swap(dp_off);
        dep.swap(dp);
    }
    const int NTP = (int)tasks.size();
    c->ntasks = NTP;
    XPBD_CU(c, c->flow_tasks.alloc(NTP));
    XPBD_CU(c, c->flow_dep_off.alloc(NTP + 1));
    XPBD_CU(c, c->flow_dep.alloc(std::max<size_t>(dep.size(), 1)));
    XPBD_CU(c, c->flow_epoch.alloc(NTP + 1));
    XPBD_CU(c, cudaMemcpy(c->flow_tasks.p, tasks.data(), sizeof(int4) * NTP, cudaMemcpyHostToDevice));
    XPBD_CU(c, cudaMemcpy(c->flow_dep_off.p, doff.data(), sizeof(int) * (NTP + 1), cudaMemcpyHostToDevice));
    if (!dep.empty()) XPBD_CU(c, cudaMemcpy(c->flow_dep.p, dep.data(), sizeof(int) * dep.size(), cudaMemcpyHostToDevice));
    XPBD_CU(c, cudaMemset(c->flow_epoch.p, 0, sizeof(unsigned) * (NTP + 1)));
    c->flow_versioned = false;
    if (c->prm.gs_variant == 4) {
        // per patch and vertex slot: deg << 8 | pre, deg = patches containing
        // the vertex, pre = those of a lower colour
        std::vector<int> pcol(P);
        for (int col = 0; col < c->n_tet_colours; col++)
            for (int q = c->pcol_off[col]; q < c->pcol_off[col + 1]; q++) pcol[q] = col;
        std::vector<int> vp_off(V + 1, 0);
        for (int q = 0; q < P; q++)
            for (int k = 0; k < (pmeta[q].y >> 8); k++) vp_off[pv(q, k) + 1]++;
        for (int v = 0; v < V; v++) vp_off[v + 1] += vp_off[v];
        std::vector<int> vcol(vp_off[V]), vfill(vp_off.begin(), vp_off.end() - 1);
        for (int q = 0; q < P; q++)
            for (int k = 0; k < (pmeta[q].y >> 8); k++) vcol[vfill[pv(q, k)]++] = pcol[q];
        std::vector<int4> ver(P, make_int4(0, 0, 0, 0));
        for (int q = 0; q < P; q++) {
            int w[4] = {0, 0, 0, 0};
            for (int k = 0; k < (pmeta[q].y >> 8); k++) {
                const int v = pv(q, k), deg = vp_off[v + 1] - vp_off[v];
                int pre = 0, same = 0;
                for (int e = vp_off[v]; e < vp_off[v + 1]; e++) {
                    pre += vcol[e] < pcol[q];
                    same += vcol[e] == pcol[q];
                }
                if (same != 1) return fail(c, XPBD_ERR_STATE, "dataflow: vertex %d in two patches of colour %d", v, pcol[q]);
                // a vertex in more than 255 patches does not fit the 8-bit
                // fields: this context runs the task-counter sweep (variant 2),
                // whose task layout and co-residency this grid also satisfies
                if (deg > 255) return XPBD_OK;
                w[k >> 1] |= ((deg << 8) | pre) << (16 * (k & 1));
            }
            ver[q] = make_int4(w[0], w[1], w[2], w[3]);
        }
        c->flow_versioned = true;
        c->patch_ver_h = ver;
        XPBD_CU(c, c->patch_ver.alloc(P));
        XPBD_CU(c, c->xv.alloc(V));
        XPBD_CU(c, c->patch_w.alloc(2 * (size_t)P));
        c->npatches = P;
        XPBD_CU(c, cudaMemcpy(c->patch_ver.p, ver.data(), sizeof(int4) * P, cudaMemcpyHostToDevice));
    }
    return XPBD_OK;
}

// Self-collision data: the surface vertices, tets in index order, Dm^-1 and
// rest positions in double, and a uniform grid over the rest bounding box
// padded by a quarter of its extent, cells 1.1x the widest tet box at rest
// (a tet whose box outgrows a cell goes to the overflow list), at most
// 2^22 cells.
int build_self_collisions(xpbd_ctx* c, const std::vector<double>& X, const std::vector<double>& Q) {
    const int V = c->V, T = c->T, F = c->F;
    std::vector<char> on(V, 0);
    for (size_t i = 0; i < c->faces_h.size(); i++) on[c->faces_h[i]] = 1;
    std::vector<int> surf;
    for (int v = 0; v < V; v++)
        if (on[v]) surf.push_back(v);
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300}, wmax = 0;
    for (int v = 0; v < V; v++)
        for (int k = 0; k < 3; k++) {
            lo[k] = std::min(lo[k], X[3 * (size_t)v + k]);
            hi[k] = std::max(hi[k], X[3 * (size_t)v + k]);
        }
    std::vector<int4> tt(T);
    for (int t = 0; t < T; t++) {
        const int* e = &c->tets_h[4 * (size_t)t];
        tt[t] = make_int4(e[0], e[1], e[2], e[3]);
        for (int k = 0; k < 3; k++) {
            double a = 1e300, b = -1e300;
            for (int i = 0; i < 4; i++) {
                a = std::min(a, X[3 * (size_t)e[i] + k]);
                b = std::max(b, X[3 * (size_t)e[i] + k]);
            }
            wmax = std::max(wmax, b - a);
        }
    }
    double ext = 0;
    for (int k = 0; k < 3; k++) ext = std::max(ext, hi[k] - lo[k]);
    double cell = std::max(1.1 * wmax, 1e-9 * std::max(ext, 1.0));
    int n[3];
    for (;;) {
        long long cells = 1;
        for (int k = 0; k < 3; k++) {
            const double w = (hi[k] - lo[k]) + 0.5 * ext;
            n[k] = std::max(1, (int)std::ceil(w / cell));
            cells *= n[k];
        }
        if (cells <= (1LL << 22)) break;
        cell *= 1.25;
    }
    xg::SelfGrid g;
    g.ox = (float)(lo[0] - 0.25 * ext);
    g.oy = (float)(lo[1] - 0.25 * ext);
    g.oz = (float)(lo[2] - 0.25 * ext);
    g.cell = (float)cell;
    g.nx = n[0]; g.ny = n[1]; g.nz = n[2];
    c->sgrid = g;
    c->ncells = n[0] * n[1] * n[2];
    c->n_surf = (int)surf.size();
    std::vector<float4> X0f(V);
    for (int v = 0; v < V; v++)
        X0f[v] = make_float4((float)X[3 * (size_t)v], (float)X[3 * (size_t)v + 1], (float)X[3 * (size_t)v + 2], 0.f);
    const int ns = std::max(c->n_surf, 1);
    XPBD_CU(c, c->s_tets.alloc(T));
    XPBD_CU(c, c->s_Q.alloc(9 * (size_t)T));
    XPBD_CU(c, c->s_X0.alloc(3 * (size_t)V));
    XPBD_CU(c, c->s_X0f.alloc(V));
    XPBD_CU(c, c->s_surf.alloc(ns));
    XPBD_CU(c, c->s_cell_count.alloc(c->ncells));
    XPBD_CU(c, c->s_cell_fill.alloc(c->ncells));
    XPBD_CU(c, c->s_cell_off.alloc(c->ncells + 1));
    XPBD_CU(c, c->s_cell_tets.alloc(T));
    XPBD_CU(c, c->s_tet_cell.alloc(T));
    XPBD_CU(c, c->s_overflow.alloc(T));
    XPBD_CU(c, c->s_n_overflow.alloc(1));
    XPBD_CU(c, c->s_hit_tet.alloc(ns));
    XPBD_CU(c, c->s_hit_list.alloc(ns));
    XPBD_CU(c, c->s_n_hits.alloc(1));
    XPBD_CU(c, c->s_contact.alloc(ns));
    XPBD_CU(c, c->s_lam.alloc(ns));
    XPBD_CU(c, c->s_scan_part.alloc(c->ncells / 4096 + 2));
    XPBD_CU(c, cudaMemcpy(c->s_tets.p, tt.data(), sizeof(int4) * T, cudaMemcpyHostToDevice));
    XPBD_CU(c, cudaMemcpy(c->s_Q.p, Q.data(), sizeof(double) * 9 * (size_t)T, cudaMemcpyHostToDevice));
    XPBD_CU(c, cudaMemcpy(c->s_X0.p, X.data(), sizeof(double) * 3 * (size_t)V, cudaMemcpyHostToDevice));
    XPBD_CU(c, cudaMemcpy(c->s_X0f.p, X0f.data(), sizeof(float4) * V, cudaMemcpyHostToDevice));
    if (!surf.empty()) XPBD_CU(c, cudaMemcpy(c->s_surf.p, surf.data(), sizeof(int) * surf.size(), cudaMemcpyHostToDevice));
    XPBD_CU(c, cudaMemset(c->s_n_hits.p, 0, sizeof(int)));
    c->self_on = true;
    return XPBD_OK;
}

int build(xpbd_ctx* c, const xpbd_mesh_desc* ms, int n_inst) {
    const int V = c->V, T = c->T, F = c->F;
    const xpbd_params& p = c->prm;
    c->block = p.block_size ? p.block_size : 256;
    c->S = p.max_contacts_per_face ? p.max_contacts_per_face : 4;
    // concatenate the instances; indices are shifted by the vertex offsets
    c->n_inst = n_inst;
    c->voff.assign(n_inst + 1, 0);
    c->toff.assign(n_inst + 1, 0);
    c->foff.assign(n_inst + 1, 0);
    for (int k = 0; k < n_inst; k++) {
        c->voff[k + 1] = c->voff[k] + ms[k].num_vertices;
        c->toff[k + 1] = c->toff[k] + ms[k].num_tets;
        c->foff[k + 1] = c->foff[k] + ms[k].num_faces;
    }
    std::vector<double> Xcat(3 * (size_t)V), Ecat(T), nucat(T), rhocat(T);
    c->tets_h.resize(4 * (size_t)T);
    c->faces_h.resize(3 * (size_t)F);
    std::vector<int> finst(F);
    for (int k = 0; k < n_inst; k++) {
        const xpbd_mesh_desc& m = ms[k];
        const int64_t vo = c->voff[k], to = c->toff[k], fo = c->foff[k];
        std::copy(m.vertices, m.vertices + 3 * m.num_vertices, Xcat.begin() + 3 * vo);
        std::copy(m.tet_E, m.tet_E + m.num_tets, Ecat.begin() + to);
        std::copy(m.tet_nu, m.tet_nu + m.num_tets, nucat.begin() + to);
        std::copy(m.tet_density, m.tet_density + m.num_tets, rhocat.begin() + to);
        for (int64_t i = 0; i < 4 * m.num_tets; i++) {
            const int v = m.tets[i];
            if (v < 0 || v >= m.num_vertices)
                return fail(c, XPBD_ERR_INVALID, "instance %d: tet vertex index %d out of range [0,%lld)", k, v,
                            (long long)m.num_vertices);
            c->tets_h[4 * to + i] = (int)(v + vo);
        }
        for (int64_t i = 0; i < 3 * m.num_faces; i++) {
            const int v = m.faces[i];
            if (v < 0 || v >= m.num_vertices)
                return fail(c, XPBD_ERR_INVALID, "instance %d: face vertex index %d out of range [0,%lld)", k, v,
                            (long long)m.num_vertices);
            c->faces_h[3 * fo + i] = (int)(v + vo);
        }
        for (int64_t f = 0; f < m.num_faces; f++) finst[fo + f] = k;
    }
    c->sphere_tab_h.assign(3 * (size_t)n_inst * c->S, make_float4(0.f, 0.f, 0.f, -1.f));
    c->sdf_pose_h.assign(10 * (size_t)n_inst * c->S, 0.0);

    // rest shape, compliance, lumped mass (ElementConstraint.hpp:23-51;
    // HydrostaticConstraint.cpp:15-16; DeviatoricConstraint.cpp:13;
    // ElasticMaterial.hpp:31-32; XPBDMeshObject.cpp:277-331)
    const double* X = Xcat.data();
    std::vector<double> Q(9 * (size_t)T), ad(T), ah(T), gm(T);
    c->mass_h.assign(V, 0.0);
    std::vector<double> vvol(V, 0.0);  // vertex volumes (1st-order damping)
    for (int t = 0; t < T; t++) {
        const int* e = &c->tets_h[4 * (size_t)t];
        double D[9];
        for (int i = 0; i < 3; i++)
            for (int k = 0; k < 3; k++) D[3 * i + k] = X[3 * (size_t)e[i] + k] - X[3 * (size_t)e[3] + k];
        auto M = [&D](int r, int cc) { return D[cc * 3 + r]; };
        const double c00 = M(1, 1) * M(2, 2) - M(1, 2) * M(2, 1);
        const double c10 = M(1, 2) * M(2, 0) - M(1, 0) * M(2, 2);
        const double c20 = M(1, 0) * M(2, 1) - M(1, 1) * M(2, 0);
        const double det = M(0, 0) * c00 + M(0, 1) * c10 + M(0, 2) * c20;
        if (!(std::fabs(det) > 0) || !std::isfinite(det))
            return fail(c, XPBD_ERR_INVALID, "tet %d is degenerate at rest (det = %g)", t, det);
        const double inv = 1.0 / det;
        double* q = &Q[9 * (size_t)t];
        q[0] = c00 * inv; q[1] = c10 * inv; q[2] = c20 * inv;
        q[3] = (M(0, 2) * M(2, 1) - M(0, 1) * M(2, 2)) * inv;
        q[4] = (M(0, 0) * M(2, 2) - M(0, 2) * M(2, 0)) * inv;
        q[5] = (M(0, 1) * M(2, 0) - M(0, 0) * M(2, 1)) * inv;
        q[6] = (M(0, 1) * M(1, 2) - M(0, 2) * M(1, 1)) * inv;
        q[7] = (M(0, 2) * M(1, 0) - M(0, 0) * M(1, 2)) * inv;
        q[8] = (M(0, 0) * M(1, 1) - M(0, 1) * M(1, 0)) * inv;
        const double vol = std::fabs(det / 6.0);
        const double E = Ecat[t], nu = nucat[t], rho = rhocat[t];
        if (!(E > 0) || !(nu > -1 && nu < 0.5) || !(rho > 0))
            return fail(c, XPBD_ERR_INVALID, "tet %d has invalid material E=%g nu=%g rho=%g", t, E, nu, rho);
        const double mu = E / (2 * (1 + nu));
        const double la = (E * nu) / ((1 + nu) * (1 - 2 * nu));
        ad[t] = 1 / (mu * vol);
        ah[t] = 1 / (la * vol);
        gm[t] = mu / la;
        const double em = vol * rho;
        for (int k = 0; k < 4; k++) c->mass_h[e[k]] += em / 4.0;
        for (int k = 0; k < 4; k++) vvol[e[k]] += vol / 4.0;
    }
    c->inv_mass_h.assign(V, 0.0);
    for (int i = 0; i < V; i++) {
        if (!(c->mass_h[i] > 0))
            return fail(c, XPBD_ERR_INVALID, "vertex %d belongs to no tet (zero mass)", i);
        c->inv_mass_h[i] = 1.0 / c->mass_h[i];
    }
    if (p.first_order) {
        // per-vertex damping B is the constraint inertia of 1st-order XPBD
        // (XPBDMeshObject.cpp:333-348, XPBDMeshObjectBase.hpp:131-137); the
        // vertex E and nu average the attached elements' (:321-329)
        std::vector<double> vE(V, 0.0), vnu(V, 0.0);
        std::vector<int> natt(V, 0);
        for (int t = 0; t < T; t++)
            for (int k = 0; k < 4; k++) natt[c->tets_h[4 * (size_t)t + k]]++;
        for (int t = 0; t < T; t++)
            for (int k = 0; k < 4; k++) {
                const int v = c->tets_h[4 * (size_t)t + k];
                vE[v] += Ecat[t] / natt[v];
                vnu[v] += nucat[t] / natt[v];
            }
        std::vector<float> gdz(V);
        for (int i = 0; i < V; i++) {
            const double B = p.adjust_damping_to_material ? vvol[i] * p.damping_multiplier * vE[i] / (1 + vnu[i])
                                                          : vvol[i] * p.damping_multiplier;
            c->inv_mass_h[i] = 1.0 / B;
            // _movePositionsInertially, 1st order (XPBDMeshObject.cpp:449-456)
            gdz[i] = (float)(-p.g_accel * c->mass_h[i] * p.dt / B);
        }
        XPBD_CU(c, c->gdz.alloc(V));
        XPBD_CU(c, cudaMemcpy(c->gdz.p, gdz.data(), sizeof(float) * V, cudaMemcpyHostToDevice));
    }
    c->fixed_h.assign(V, 0);

    // slot order: Gauss-Seidel sorts patches by colour (tets of a patch stay
    // consecutive); Jacobi keeps the tet order
    c->tet_colour.assign(T, 0);
    c->tet_of_slot.resize(T);
    std::vector<int4> pmeta, pverts;
    if (p.solver_type == XPBD_SOLVER_GAUSS_SEIDEL) {
        const int cap = p.gs_patch_tets ? p.gs_patch_tets : kMaxPatchTets;
        const std::vector<HostPatch> patches = build_patches(c->tets_h, T, cap);
        const int P = (int)patches.size();
        std::vector<int> plist((size_t)P * kMaxPatchVerts), pcol(P);
        for (int q = 0; q < P; q++)
            for (int k = 0; k < kMaxPatchVerts; k++) plist[(size_t)q * kMaxPatchVerts + k] = patches[q].v[k];
        c->n_tet_colours = greedy_colour(P, kMaxPatchVerts, plist.data(), V, pcol.data());
        c->pcol_off.assign(c->n_tet_colours + 1, 0);
        for (int q = 0; q < P; q++) c->pcol_off[pcol[q] + 1]++;
        for (int k = 0; k < c->n_tet_colours; k++) c->pcol_off[k + 1] += c->pcol_off[k];
        std::vector<int> sorted(P), fill(c->pcol_off.begin(), c->pcol_off.end() - 1);
        for (int q = 0; q < P; q++) sorted[fill[pcol[q]]++] = q;
        pmeta.resize(P);
        pverts.resize(2 * (size_t)P);
        int slot = 0;
        for (int r = 0; r < P; r++) {
            const HostPatch& hp = patches[sorted[r]];
            pmeta[r] = make_int4(slot, hp.n | (hp.nv << 8), (int)(unsigned)(hp.loc & 0xffffffffull),
                                 (int)(unsigned)(hp.loc >> 32));
            pverts[2 * (size_t)r] = make_int4(hp.v[0], hp.v[1], hp.v[2], hp.v[3]);
            pverts[2 * (size_t)r + 1] = make_int4(hp.v[4], hp.v[5], hp.v[6], hp.v[7]);
            for (int i = 0; i < hp.n; i++) {
                c->tet_of_slot[slot++] = hp.first + i;
                c->tet_colour[hp.first + i] = pcol[sorted[r]];
            }
        }
    } else {
        for (int t = 0; t < T; t++) c->tet_of_slot[t] = t;
        c->n_tet_colours = 1;
    }
    // alpha~ = alpha / dt^2 (2nd order) or alpha / dt (1st order,
    // CombinedNeohookeanConstraintProjector.cpp:35, ConstraintProjector.hpp:133-140)
    const double dt2 = p.first_order ? p.dt : p.dt * p.dt;
    std::vector<int4> hidx(T);
    std::vector<float4> h0(T), h1(T), h2(T);
    std::vector<float2> hmat(T);
    c->alpha_t_d.resize(T);
    c->alpha_t_h.resize(T);
    for (int sidx = 0; sidx < T; sidx++) {
        const int t = c->tet_of_slot[sidx];
        const int* e = &c->tets_h[4 * (size_t)t];
        const double* q = &Q[9 * (size_t)t];
        hidx[sidx] = make_int4(e[0], e[1], e[2], e[3]);
        const float atd = (float)(ad[t] / dt2), ath = (float)(ah[t] / dt2);
        h0[sidx] = make_float4((float)q[0], (float)q[1], (float)q[2], (float)q[3]);
        h1[sidx] = make_float4((float)q[4], (float)q[5], (float)q[6], (float)q[7]);
        h2[sidx] = make_float4((float)q[8], atd, ath, (float)gm[t]);
        c->alpha_t_d[sidx] = atd;
        c->alpha_t_h[sidx] = ath;
        hmat[sidx] = make_float2((float)(std::log10(Ecat[t]) / 5.0), (float)nucat[t]);
    }

    // faces and their colouring (Gauss-Seidel contact order)
    std::vector<int4> hf(F);
    for (int f = 0; f < F; f++) hf[f] = make_int4(c->faces_h[3 * f], c->faces_h[3 * f + 1], c->faces_h[3 * f + 2], 0);
    std::vector<int> fcol(F, 0), flist(F);
    c->n_face_colours = F ? greedy_colour(F, 3, c->faces_h.data(), V, fcol.data()) : 0;
    c->fcol_off.assign(c->n_face_colours + 1, 0);
    for (int f = 0; f < F; f++) c->fcol_off[fcol[f] + 1]++;
    for (int k = 0; k < c->n_face_colours; k++) c->fcol_off[k + 1] += c->fcol_off[k];
    {
        std::vector<int> fill(c->fcol_off.begin(), c->fcol_off.end() - 1);
        for (int f = 0; f < F; f++) flist[fill[fcol[f]]++] = f;
    }
    // faces by (instance, colour, index) for the per-instance contact lists
    const int nfc = c->n_face_colours;
    std::vector<int> ifl(F), ifo((size_t)n_inst * (nfc + 1), 0);
    {
        std::vector<int> cnt((size_t)n_inst * nfc, 0);
        for (int f = 0; f < F; f++) cnt[(size_t)finst[f] * nfc + fcol[f]]++;
        int run = 0;
        for (int k = 0; k < n_inst; k++) {
            for (int col = 0; col < nfc; col++) {
                ifo[(size_t)k * (nfc + 1) + col] = run;
                run += cnt[(size_t)k * nfc + col];
            }
            ifo[(size_t)k * (nfc + 1) + nfc] = run;
        }
        std::vector<int> pos(ifo.begin(), ifo.end());
        for (int f = 0; f < F; f++) ifl[pos[(size_t)finst[f] * (nfc + 1) + fcol[f]]++] = f;
    }
    c->api_slots.assign(F, 0);

    // local collision iterations: a per-tet greedy colouring in tet index
    // order; the local order lists the slots colour by colour, ascending tet
    // index within a colour
    std::vector<int> lslots;
    if (F && p.num_local_collision_iters > 0) {
        std::vector<int> tcol(T), slot_of(T);
        const int nc = greedy_colour(T, 4, c->tets_h.data(), V, tcol.data());
        c->lcol_off.assign(nc + 1, 0);
        for (int t = 0; t < T; t++) c->lcol_off[tcol[t] + 1]++;
        for (int k = 0; k < nc; k++) c->lcol_off[k + 1] += c->lcol_off[k];
        for (int s = 0; s < T; s++) slot_of[c->tet_of_slot[s]] = s;
        std::vector<int> fill(c->lcol_off.begin(), c->lcol_off.end() - 1);
        lslots.resize(T);
        c->local_tets_h.resize(T);
        for (int t = 0; t < T; t++) {
            const int j = fill[tcol[t]]++;
            lslots[j] = slot_of[t];
            c->local_tets_h[j] = t;
        }
    }

    // CSR vertex -> (slot, local vertex) for the gather variant
    std::vector<int> off(V + 1, 0), ent(4 * (size_t)T);
    if (p.solver_type == XPBD_SOLVER_JACOBI && p.jacobi_variant == XPBD_JACOBI_GATHER) {
        for (int sidx = 0; sidx < T; sidx++) {
            const int4 e = hidx[sidx];
            off[e.x + 1]++; off[e.y + 1]++; off[e.z + 1]++; off[e.w + 1]++;
        }
        for (int i = 0; i < V; i++) off[i + 1] += off[i];
        std::vector<int> fill(off.begin(), off.end() - 1);
        for (int sidx = 0; sidx < T; sidx++) {
            const int4 e = hidx[sidx];
            const int vs[4] = {e.x, e.y, e.z, e.w};
            for (int k = 0; k < 4; k++) ent[fill[vs[k]]++] = 4 * sidx + k;
        }
    }

    // device allocation + upload
    XPBD_CU(c, cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    {
        // coherent access to pageable host memory (Grace-Blackwell C2C): the
        // position transfers run as kernels on the caller's arrays
        int dev = 0, pma = 0;
        XPBD_CU(c, cudaGetDevice(&dev));
        if (cudaDeviceGetAttribute(&pma, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) {
            cudaGetLastError();
            pma = 0;
        }
        c->host_direct = pma == 1;
    }
    XPBD_CU(c, c->x.alloc(V));
    XPBD_CU(c, c->prev.alloc(V));
    XPBD_CU(c, c->vel.alloc(V));
    XPBD_CU(c, c->dx.alloc(V));
    XPBD_CU(c, c->tet_idx.alloc(T));
    XPBD_CU(c, c->q0.alloc(T));
    XPBD_CU(c, c->q1.alloc(T));
    XPBD_CU(c, c->q2.alloc(T));
    XPBD_CU(c, c->lam.alloc(T));
    XPBD_CU(c, c->perm.alloc(T));
    XPBD_CU(c, c->flags.alloc(1));
    XPBD_CU(c, c->mat.alloc(T));
    XPBD_CU(c, c->warm_stats.alloc(2));
    XPBD_CU(c, c->warm_rows.alloc(2));
    XPBD_CU(c, c->mse.alloc(1));
    XPBD_CU(c, c->rvec.alloc(2 * (size_t)T));
    XPBD_CU(c, c->energy_partial.alloc(residual_blocks(T, c->block) + 1));
    XPBD_CU(c, cudaMallocHost((void**)&c->h_stage, sizeof(float4) * (size_t)std::max(V, 1)));
    XPBD_CU(c, c->sphere_tab.alloc(c->sphere_tab_h.size()));
    if (F) {
        XPBD_CU(c, c->face_inst.alloc(F));
        XPBD_CU(c, cudaMemcpy(c->face_inst.p, finst.data(), sizeof(int) * F, cudaMemcpyHostToDevice));
        XPBD_CU(c, c->faces.alloc(F));
        XPBD_CU(c, c->face_list.alloc(F));
        const size_t ns = (size_t)c->S * F;
        XPBD_CU(c, c->c_bary.alloc(ns));
        XPBD_CU(c, c->c_p.alloc(ns));
        XPBD_CU(c, c->c_n.alloc(ns));
        XPBD_CU(c, c->c_lam.alloc(ns));
        XPBD_CU(c, cudaMemset(c->c_bary.p, 0, sizeof(float4) * ns));
        XPBD_CU(c, cudaMemset(c->c_lam.p, 0, sizeof(float) * ns));
        XPBD_CU(c, cudaMemcpy(c->faces.p, hf.data(), sizeof(int4) * F, cudaMemcpyHostToDevice));
        XPBD_CU(c, cudaMemcpy(c->face_list.p, flist.data(), sizeof(int) * F, cudaMemcpyHostToDevice));
        XPBD_CU(c, c->ifl.alloc(F));
        XPBD_CU(c, c->ifo_off.alloc(ifo.size()));
        XPBD_CU(c, c->act_faces.alloc(F));
        XPBD_CU(c, c->act_off.alloc(ifo.size()));
        XPBD_CU(c, cudaMemcpy(c->ifl.p, ifl.data(), sizeof(int) * F, cudaMemcpyHostToDevice));
        XPBD_CU(c, cudaMemcpy(c->ifo_off.p, ifo.data(), sizeof(int) * ifo.size(), cudaMemcpyHostToDevice));
        XPBD_CU(c, cudaMemset(c->act_off.p, 0, sizeof(int) * ifo.size()));
        XPBD_CU(c, c->rb.alloc((size_t)kRigidRec * n_inst * c->S));
        XPBD_CU(c, c->rc_list.alloc(ns));
        XPBD_CU(c, c->rc_count.alloc(1));
        XPBD_CU(c, cudaMemset(c->rc_count.p, 0, sizeof(int)));
        if (p.self_collisions) {
            int st = build_self_collisions(c, Xcat, Q);
            if (st) return st;
        }
    }
    if (!lslots.empty()) {
        XPBD_CU(c, c->local_slots.alloc(T));
        XPBD_CU(c, c->vmask.alloc(V));
        XPBD_CU(c, c->tmask.alloc(T));
        XPBD_CU(c, cudaMemcpy(c->local_slots.p, lslots.data(), sizeof(int) * T, cudaMemcpyHostToDevice));
    }
    // (faces allow contacts, which the dataflow sweep leaves to the launches)
    if (!pmeta.empty() && p.solver_type == XPBD_SOLVER_GAUSS_SEIDEL && p.gs_variant >= 2 &&
        F == 0) {
        int st = build_flow_tasks(c, pmeta, pverts);
        if (st) return st;
    }
    if (!pmeta.empty()) {
        XPBD_CU(c, c->patch_meta.alloc(pmeta.size()));
        XPBD_CU(c, c->patch_verts.alloc(pverts.size()));
        XPBD_CU(c, cudaMemcpy(c->patch_meta.p, pmeta.data(), sizeof(int4) * pmeta.size(), cudaMemcpyHostToDevice));
        XPBD_CU(c, cudaMemcpy(c->patch_verts.p, pverts.data(), sizeof(int4) * pverts.size(), cudaMemcpyHostToDevice));
    }
    if (p.solver_type == XPBD_SOLVER_JACOBI && p.jacobi_variant == XPBD_JACOBI_GATHER) {
        XPBD_CU(c, c->dxt.alloc(3 * (size_t)T));
        XPBD_CU(c, c->csr_off.alloc(V + 1));
        XPBD_CU(c, c->csr_ent.alloc(4 * (size_t)T));
        XPBD_CU(c, cudaMemcpy(c->csr_off.p, off.data(), sizeof(int) * (V + 1), cudaMemcpyHostToDevice));
        XPBD_CU(c, cudaMemcpy(c->csr_ent.p, ent.data(), sizeof(int) * 4 * (size_t)T, cudaMemcpyHostToDevice));
    }
    XPBD_CU(c, cudaMemcpy(c->tet_idx.p, hidx.data(), sizeof(int4) * T, cudaMemcpyHostToDevice));
    XPBD_CU(c, cudaMemcpy(c->q0.p, h0.data(), sizeof(float4) * T, cudaMemcpyHostToDevice));
    XPBD_CU(c, cudaMemcpy(c->q1.p, h1.data(), sizeof(float4) * T, cudaMemcpyHostToDevice));
    XPBD_CU(c, cudaMemcpy(c->q2.p, h2.data(), sizeof(float4) * T, cudaMemcpyHostToDevice));
    XPBD_CU(c, cudaMemcpy(c->perm.p, c->tet_of_slot.data(), sizeof(int) * T, cudaMemcpyHostToDevice));
    XPBD_CU(c, cudaMemcpy(c->mat.p, hmat.data(), sizeof(float2) * T, cudaMemcpyHostToDevice));
    XPBD_CU(c, cudaMemset(c->warm_stats.p, 0, 2 * sizeof(unsigned long long)));
    XPBD_CU(c, cudaMemset(c->lam.p, 0, sizeof(float2) * T));
    XPBD_CU(c, cudaMemset(c->dx.p, 0, sizeof(float4) * V));
    XPBD_CU(c, cudaMemset(c->vel.p, 0, sizeof(float4) * V));
    XPBD_CU(c, cudaMemset(c->flags.p, 0, sizeof(Flags)));
    c->res_stride = residual_blocks(T, c->block) + 1;
    int st = stage_positions_to_device(c, X, nullptr);
    if (st) return st;
    XPBD_CU(c, cudaMemcpy(c->prev.p, c->x.p, sizeof(float4) * V, cudaMemcpyDeviceToDevice));
    return XPBD_OK;
}

}  // namespace

extern "C" {

int xpbd_abi_version(void) { return XPBD_ABI_VERSION; }

const char* xpbd_status_string(int st) {
    switch (st) {
        case XPBD_OK: return "ok";
        case XPBD_ERR_INVALID: return "invalid argument";
        case XPBD_ERR_CUDA: return "CUDA error";
        case XPBD_ERR_NUMERIC: return "non-finite projection update";
        case XPBD_ERR_NO_DEVICE: return "no CUDA device";
        case XPBD_ERR_STATE: return "invalid state";
        case XPBD_ERR_CAPACITY: return "capacity exceeded";
        case XPBD_ERR_TIMEOUT: return "a bounded device wait timed out";
        default: return "unknown status";
    }
}

int xpbd_default_params(xpbd_params* p) {
    if (!p) return XPBD_ERR_INVALID;
    std::memset(p, 0, sizeof(*p));
    p->dt = 1e-3;
    p->g_accel = 9.81;
    p->collision_rate = 100.0;
    p->num_iters = 1;
    p->solver_type = XPBD_SOLVER_GAUSS_SEIDEL;
    p->constraint_type = XPBD_CONSTRAINT_COMBINED;
    p->residual_policy = XPBD_RESIDUAL_NEVER;
    p->jacobi_variant = XPBD_JACOBI_ATOMIC;
    p->block_size = 0;
    p->max_contacts_per_face = 0;
    p->use_graphs = 1;
    p->use_pdl = 1;
    p->gs_patch_tets = 0;
    p->gs_min_blocks = 0;
    p->gs_variant = 4;
    p->num_local_collision_iters = 0;
    p->first_order = 0;
    p->adjust_damping_to_material = 0;
    p->damping_multiplier = 1.0;
    return XPBD_OK;
}

int xpbd_colour_items(int64_t n, int32_t arity, const int32_t* items, int64_t nv, int32_t* out) {
    if (n < 0 || nv <= 0 || arity < 1 || arity > 8 || (n > 0 && (!items || !out))) return -XPBD_ERR_INVALID;
    for (int64_t i = 0; i < n * arity; i++)
        if (items[i] < 0 || items[i] >= nv) return -XPBD_ERR_INVALID;
    return n ? greedy_colour(n, arity, items, nv, out) : 0;
}

int xpbd_create(const xpbd_mesh_desc* m, const xpbd_params* p, xpbd_ctx** out) {
    return xpbd_create_batch(m, 1, p, out);
}

int xpbd_create_batch(const xpbd_mesh_desc* ms, int32_t n_inst, const xpbd_params* p, xpbd_ctx** out) {
    if (!out) return XPBD_ERR_INVALID;
    *out = nullptr;
    if (!ms || !p || n_inst <= 0) return XPBD_ERR_INVALID;
    long long V = 0, T = 0, F = 0;
    for (int k = 0; k < n_inst; k++) {
        const xpbd_mesh_desc* m = ms + k;
        if (!m->vertices || !m->tets || !m->tet_E || !m->tet_nu || !m->tet_density) return XPBD_ERR_INVALID;
        if (m->num_vertices <= 0 || m->num_tets <= 0 || m->num_faces < 0 || (m->num_faces > 0 && !m->faces))
            return XPBD_ERR_INVALID;
        V += m->num_vertices;
        T += m->num_tets;
        F += m->num_faces;
    }
    if (V > (1LL << 30) || T > (1LL << 29) || F > (1LL << 28)) return XPBD_ERR_CAPACITY;
    if (!valid_params(*p)) return XPBD_ERR_INVALID;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return XPBD_ERR_NO_DEVICE;
    }
    xpbd_ctx* c = new (std::nothrow) xpbd_ctx();
    if (!c) return XPBD_ERR_CAPACITY;
    c->prm = *p;
    c->V = (int)V;
    c->T = (int)T;
    c->F = (int)F;
    int st = build(c, ms, n_inst);
    if (st) {
        fprintf(stderr, "xpbd_create: %s\n", c->err.c_str());
        release(c);
        delete c;
        return st;
    }
    *out = c;
    return XPBD_OK;
}

int xpbd_destroy(xpbd_ctx* c) {
    if (!c) return XPBD_ERR_INVALID;
    if (c->stream) cudaStreamSynchronize(c->stream);
    release(c);
    delete c;
    return XPBD_OK;
}

const char* xpbd_last_error(const xpbd_ctx* c) { return c ? c->err.c_str() : "null context"; }

int xpbd_set_num_iters(xpbd_ctx* c, int32_t n) {
    if (!c || n < 0) return XPBD_ERR_INVALID;
    if (n != c->prm.num_iters) {
        c->prm.num_iters = n;
        c->graph_dirty = true;
    }
    return XPBD_OK;
}

}  // extern "C"

namespace {
// the device reads or writes the caller's array itself; returns after the
// transfer, so the caller may reuse the array
template <typename H>
int host_direct_in(xpbd_ctx* c, float4* dst, const H* h, bool keep_w) {
    launch_xyz_from_host(c->stream, dst, h, c->V, keep_w);
    XPBD_CU(c, cudaGetLastError());
    XPBD_CU(c, cudaStreamSynchronize(c->stream));
    return XPBD_OK;
}
template <typename H>
int host_direct_out(xpbd_ctx* c, H* h, const float4* src) {
    launch_xyz_to_host(c->stream, h, src, c->V);
    XPBD_CU(c, cudaGetLastError());
    XPBD_CU(c, cudaStreamSynchronize(c->stream));
    return XPBD_OK;
}
}  // namespace

extern "C" {

int xpbd_set_positions(xpbd_ctx* c, const double* x) {
    if (!c || !x) return XPBD_ERR_INVALID;
    if (c->host_direct) return host_direct_in(c, c->x.p, x, true);
    return stage_positions_to_device(c, x, nullptr);
}

int xpbd_set_positions_f32(xpbd_ctx* c, const float* x) {
    if (!c || !x) return XPBD_ERR_INVALID;
    if (c->host_direct) return host_direct_in(c, c->x.p, x, true);
    return stage_positions_to_device(c, nullptr, x);
}

static int get_xyz(xpbd_ctx* c, const float4* src, double* out) {
    if (c->host_direct) return host_direct_out(c, out, src);
    int st = fetch(c, src);
    if (st) return st;
    for (int i = 0; i < c->V; i++) {
        out[3 * i] = c->h_stage[i].x;
        out[3 * i + 1] = c->h_stage[i].y;
        out[3 * i + 2] = c->h_stage[i].z;
    }
    return XPBD_OK;
}

int xpbd_get_positions(xpbd_ctx* c, double* x) {
    if (!c || !x) return XPBD_ERR_INVALID;
    return get_xyz(c, c->x.p, x);
}

int xpbd_get_positions_f32(xpbd_ctx* c, float* x) {
    if (!c || !x) return XPBD_ERR_INVALID;
    if (c->host_direct) return host_direct_out(c, x, c->x.p);
    int st = fetch(c, c->x.p);
    if (st) return st;
    for (int i = 0; i < c->V; i++) {
        x[3 * i] = c->h_stage[i].x;
        x[3 * i + 1] = c->h_stage[i].y;
        x[3 * i + 2] = c->h_stage[i].z;
    }
    return XPBD_OK;
}

int xpbd_get_prev_positions(xpbd_ctx* c, double* x) {
    if (!c || !x) return XPBD_ERR_INVALID;
    return get_xyz(c, c->prev.p, x);
}

int xpbd_set_velocities(xpbd_ctx* c, const double* v) {
    if (!c || !v) return XPBD_ERR_INVALID;
    if (c->host_direct) return host_direct_in(c, c->vel.p, v, false);
    for (int i = 0; i < c->V; i++)
        c->h_stage[i] = make_float4((float)v[3 * i], (float)v[3 * i + 1], (float)v[3 * i + 2], 0.f);
    XPBD_CU(c, cudaMemcpyAsync(c->vel.p, c->h_stage, sizeof(float4) * c->V, cudaMemcpyHostToDevice, c->stream));
    XPBD_CU(c, cudaStreamSynchronize(c->stream));
    return XPBD_OK;
}

int xpbd_get_velocities(xpbd_ctx* c, double* v) {
    if (!c || !v) return XPBD_ERR_INVALID;
    return get_xyz(c, c->vel.p, v);
}

int xpbd_get_masses(xpbd_ctx* c, double* m) {
    if (!c || !m) return XPBD_ERR_INVALID;
    std::copy(c->mass_h.begin(), c->mass_h.end(), m);
    return XPBD_OK;
}

int xpbd_set_fixed(xpbd_ctx* c, const uint8_t* mask) {
    if (!c || !mask) return XPBD_ERR_INVALID;
    // the fixed flag lives in the sign of x.w (and prev.w): re-stage both
    int st = fetch(c, c->x.p);
    if (st) return st;
    for (int i = 0; i < c->V; i++) {
        c->fixed_h[i] = mask[i] ? 1 : 0;
        c->h_stage[i].w = (float)c->inv_mass_h[i] * (c->fixed_h[i] ? -1.f : 1.f);
    }
    XPBD_CU(c, cudaMemcpyAsync(c->x.p, c->h_stage, sizeof(float4) * c->V, cudaMemcpyHostToDevice, c->stream));
    XPBD_CU(c, cudaStreamSynchronize(c->stream));
    st = fetch(c, c->prev.p);
    if (st) return st;
    for (int i = 0; i < c->V; i++) c->h_stage[i].w = (float)c->inv_mass_h[i] * (c->fixed_h[i] ? -1.f : 1.f);
    XPBD_CU(c, cudaMemcpyAsync(c->prev.p, c->h_stage, sizeof(float4) * c->V, cudaMemcpyHostToDevice, c->stream));
    XPBD_CU(c, cudaStreamSynchronize(c->stream));
    return XPBD_OK;
}

int xpbd_set_kinematic_group(xpbd_ctx* c, int32_t n, const int32_t* idx) {
    if (!c || n < 0 || (n > 0 && !idx)) return XPBD_ERR_INVALID;
    for (int j = 0; j < n; j++)
        if (idx[j] < 0 || idx[j] >= c->V) return fail(c, XPBD_ERR_INVALID, "kinematic index %d out of range", idx[j]);
    std::vector<uint8_t> mask(c->fixed_h);
    for (int j = 0; j < n; j++) mask[idx[j]] = 1;
    int st = xpbd_set_fixed(c, mask.data());
    if (st) return st;
    st = fetch(c, c->x.p);
    if (st) return st;
    std::vector<float4> rest(n);
    for (int j = 0; j < n; j++) rest[j] = c->h_stage[idx[j]];
    c->kin_idx.release();
    c->kin_rest.release();
    c->nkin = n;
    if (n) {
        XPBD_CU(c, c->kin_idx.alloc(n));
        XPBD_CU(c, c->kin_rest.alloc(n));
        XPBD_CU(c, cudaMemcpy(c->kin_idx.p, idx, sizeof(int) * n, cudaMemcpyHostToDevice));
        XPBD_CU(c, cudaMemcpy(c->kin_rest.p, rest.data(), sizeof(float4) * n, cudaMemcpyHostToDevice));
    }
    return XPBD_OK;
}

int xpbd_set_kinematic_offset(xpbd_ctx* c, const double* off) {
    if (!c || !off) return XPBD_ERR_INVALID;
    if (c->nkin == 0) return XPBD_OK;
    {
        Scope sc(c, K_KINEMATIC);
        launch_kinematic(c->L(), c->x.p, c->kin_idx.p, c->kin_rest.p, c->nkin, (float)off[0], (float)off[1],
                         (float)off[2]);
    }
    return after_launches(c, "kinematic offset");
}

int xpbd_set_instance_spheres(xpbd_ctx* c, int32_t inst, int32_t n, const double* ctr, const double* rad) {
    if (!c) return XPBD_ERR_INVALID;
    if (inst < 0 || inst >= c->n_inst) return fail(c, XPBD_ERR_INVALID, "instance %d out of range", inst);
    if (n < 0 || n > kMaxSpheres || (n > 0 && (!ctr || !rad)))
        return fail(c, XPBD_ERR_INVALID, "sphere count %d outside [0,%d]", n, kMaxSpheres);
    if (n > c->S) return fail(c, XPBD_ERR_CAPACITY, "%d spheres exceed %d contact slots per face", n, c->S);
    for (int i = 0; i < n; i++)
        if (!(rad[i] >= 0) || !std::isfinite(ctr[3 * i]) || !std::isfinite(ctr[3 * i + 1]) ||
            !std::isfinite(ctr[3 * i + 2]))
            return fail(c, XPBD_ERR_INVALID, "sphere %d has a bad centre or radius", i);
    std::vector<int32_t> kind(n, XPBD_SDF_SPHERE);
    std::vector<double> quat(4 * (size_t)n, 0.0), dims(3 * (size_t)n, 0.0);
    for (int i = 0; i < n; i++) {
        quat[4 * i + 3] = 1.0;
        dims[3 * i] = rad[i];
    }
    return xpbd_set_instance_sdfs(c, inst, n, kind.data(), ctr, quat.data(), dims.data());
}

int xpbd_set_instance_sdfs(xpbd_ctx* c, int32_t inst, int32_t n, const int32_t* kind, const double* pos,
                           const double* quat, const double* dims) {
    if (!c) return XPBD_ERR_INVALID;
    if (inst < 0 || inst >= c->n_inst) return fail(c, XPBD_ERR_INVALID, "instance %d out of range", inst);
    if (n < 0 || n > kMaxSpheres || (n > 0 && (!kind || !pos || !quat || !dims)))
        return fail(c, XPBD_ERR_INVALID, "SDF count %d outside [0,%d]", n, kMaxSpheres);
    if (n > c->S) return fail(c, XPBD_ERR_CAPACITY, "%d SDFs exceed %d contact slots per face", n, c->S);
    for (int i = 0; i < n; i++) {
        bool ok = kind[i] >= XPBD_SDF_SPHERE && kind[i] <= XPBD_SDF_CYLINDER;
        for (int k = 0; k < 3; k++) ok = ok && std::isfinite(pos[3 * i + k]) && dims[3 * i + k] >= 0;
        double qn = 0;
        for (int k = 0; k < 4; k++) qn += quat[4 * i + k] * quat[4 * i + k];
        ok = ok && qn > 0 && std::isfinite(qn);
        if (!ok) return fail(c, XPBD_ERR_INVALID, "SDF %d has a bad kind, position, orientation or size", i);
    }
    // free bodies of this instance end here (the caller marks them again)
    if (c->nbodies) {
        int st = pull_bodies(c);
        if (st) return st;
        std::vector<double> keep;
        for (int i = 0; i < c->nbodies; i++) {
            const double* r = &c->body_h[(size_t)i * kRigidRec];
            if ((int)r[RB_ENTRY] / c->S != inst) keep.insert(keep.end(), r, r + kRigidRec);
        }
        c->body_h.swap(keep);
    }
    double* pose = &c->sdf_pose_h[10 * (size_t)inst * c->S];
    for (int k = 0; k < c->S; k++)
        for (int j = 0; j < 10; j++)
            pose[10 * k + j] = k >= n ? 0.0 : (j < 3 ? pos[3 * k + j] : (j < 7 ? quat[4 * k + j - 3] : dims[3 * k + j - 7]));
    float4* row = &c->sphere_tab_h[3 * (size_t)inst * c->S];
    for (int k = 0; k < c->S; k++) {
        if (k < n) {
            row[3 * k] = make_float4((float)pos[3 * k], (float)pos[3 * k + 1], (float)pos[3 * k + 2], (float)kind[k]);
            row[3 * k + 1] = make_float4((float)quat[4 * k], (float)quat[4 * k + 1], (float)quat[4 * k + 2],
                                         (float)quat[4 * k + 3]);
            row[3 * k + 2] = make_float4((float)dims[3 * k], (float)dims[3 * k + 1], (float)dims[3 * k + 2], 0.f);
        } else {
            row[3 * k] = make_float4(0.f, 0.f, 0.f, -1.f);
            row[3 * k + 1] = make_float4(0.f, 0.f, 0.f, 1.f);
            row[3 * k + 2] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
    c->n_spheres_total = 0;
    for (size_t e = 0; e < c->sphere_tab_h.size(); e += 3) c->n_spheres_total += c->sphere_tab_h[e].w >= 0.f ? 1 : 0;
    c->sphere_dirty = true;
    return push_bodies(c);
}

int xpbd_set_sdfs(xpbd_ctx* c, int32_t n, const int32_t* kind, const double* pos, const double* quat,
                  const double* dims) {
    return xpbd_set_instance_sdfs(c, 0, n, kind, pos, quat, dims);
}

int xpbd_set_rigid_body(xpbd_ctx* c, int32_t inst, int32_t slot, double mass, const double* inertia3,
                        const double* vel3, const double* omega3) {
    if (!c || !inertia3 || !vel3 || !omega3) return XPBD_ERR_INVALID;
    if (!c->F) return fail(c, XPBD_ERR_STATE, "free rigid bodies need the surface faces (collisions)");
    if (inst < 0 || inst >= c->n_inst || slot < 0 || slot >= c->S)
        return fail(c, XPBD_ERR_INVALID, "instance %d / SDF slot %d out of range", inst, slot);
    const size_t e = (size_t)inst * c->S + slot;
    if (c->sphere_tab_h[3 * e].w < 0.f) return fail(c, XPBD_ERR_STATE, "SDF slot %d of instance %d is empty", slot, inst);
    bool ok = mass > 0 && std::isfinite(mass);
    for (int k = 0; k < 3; k++)
        ok = ok && inertia3[k] > 0 && std::isfinite(inertia3[k]) && std::isfinite(vel3[k]) && std::isfinite(omega3[k]);
    if (!ok) return fail(c, XPBD_ERR_INVALID, "rigid body: bad mass, inertia or velocity");
    int st = pull_bodies(c);
    if (st) return st;
    std::vector<double> r(kRigidRec, 0.0);
    const double* pose = &c->sdf_pose_h[10 * e];
    for (int k = 0; k < 3; k++) {
        r[RB_P + k] = r[RB_PP + k] = pose[k];
        r[RB_V + k] = vel3[k];
        r[RB_W + k] = omega3[k];
        r[RB_I + k] = inertia3[k];
        r[RB_II + k] = 1.0 / inertia3[k];
        r[RB_D + k] = pose[7 + k];
    }
    for (int k = 0; k < 4; k++) r[RB_Q + k] = r[RB_QP + k] = pose[3 + k];
    r[RB_M] = mass;
    r[RB_KIND] = (double)c->sphere_tab_h[3 * e].w;
    r[RB_ENTRY] = (double)e;
    bool replaced = false;
    for (int i = 0; i < c->nbodies && !replaced; i++)
        if ((size_t)c->body_h[(size_t)i * kRigidRec + RB_ENTRY] == e) {
            std::copy(r.begin(), r.end(), c->body_h.begin() + (size_t)i * kRigidRec);
            replaced = true;
        }
    if (!replaced) c->body_h.insert(c->body_h.end(), r.begin(), r.end());
    return push_bodies(c);
}

int xpbd_get_rigid_body(xpbd_ctx* c, int32_t inst, int32_t slot, double* state13) {
    if (!c || !state13) return XPBD_ERR_INVALID;
    if (inst < 0 || inst >= c->n_inst || slot < 0 || slot >= c->S)
        return fail(c, XPBD_ERR_INVALID, "instance %d / SDF slot %d out of range", inst, slot);
    int st = pull_bodies(c);
    if (st) return st;
    const size_t e = (size_t)inst * c->S + slot;
    for (int i = 0; i < c->nbodies; i++) {
        const double* r = &c->body_h[(size_t)i * kRigidRec];
        if ((size_t)r[RB_ENTRY] != e) continue;
        std::copy(r + RB_P, r + RB_P + 3, state13);
        std::copy(r + RB_Q, r + RB_Q + 4, state13 + 3);
        std::copy(r + RB_V, r + RB_V + 3, state13 + 7);
        std::copy(r + RB_W, r + RB_W + 3, state13 + 10);
        return XPBD_OK;
    }
    return fail(c, XPBD_ERR_STATE, "SDF slot %d of instance %d is not a free rigid body", slot, inst);
}

int xpbd_sdf_eval(int32_t kind, const double* pos, const double* quat, const double* dims, int64_t n,
                  const double* pts, double* out) {
    if (!pos || !quat || !dims || n < 0 || (n > 0 && (!pts || !out)) || kind < XPBD_SDF_SPHERE ||
        kind > XPBD_SDF_CYLINDER)
        return XPBD_ERR_INVALID;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return XPBD_ERR_NO_DEVICE;
    }
    std::vector<float4> h(3 + 2 * (size_t)n);
    h[0] = make_float4((float)pos[0], (float)pos[1], (float)pos[2], (float)kind);
    h[1] = make_float4((float)quat[0], (float)quat[1], (float)quat[2], (float)quat[3]);
    h[2] = make_float4((float)dims[0], (float)dims[1], (float)dims[2], 0.f);
    for (int64_t i = 0; i < n; i++) h[3 + i] = make_float4((float)pts[3 * i], (float)pts[3 * i + 1], (float)pts[3 * i + 2], 0.f);
    float4* d = nullptr;
    if (cudaMalloc((void**)&d, sizeof(float4) * h.size()) != cudaSuccess) return XPBD_ERR_CUDA;
    cudaError_t e = cudaMemcpy(d, h.data(), sizeof(float4) * (3 + n), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        launch_prim_eval(0, d, d + 3, (int)n, d + 3 + n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(h.data() + 3 + n, d + 3 + n, sizeof(float4) * n, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return XPBD_ERR_CUDA;
    for (int64_t i = 0; i < n; i++) {
        const float4 r = h[3 + n + i];
        out[4 * i] = r.x; out[4 * i + 1] = r.y; out[4 * i + 2] = r.z; out[4 * i + 3] = r.w;
    }
    return XPBD_OK;
}

int xpbd_set_spheres(xpbd_ctx* c, int32_t n, const double* ctr, const double* rad) {
    return xpbd_set_instance_spheres(c, 0, n, ctr, rad);
}

int xpbd_num_instances(xpbd_ctx* c, int32_t* n) {
    if (!c || !n) return XPBD_ERR_INVALID;
    *n = c->n_inst;
    return XPBD_OK;
}

int xpbd_instance_offsets(xpbd_ctx* c, int64_t* voff, int64_t* toff, int64_t* foff) {
    if (!c) return XPBD_ERR_INVALID;
    if (voff) std::copy(c->voff.begin(), c->voff.end(), voff);
    if (toff) std::copy(c->toff.begin(), c->toff.end(), toff);
    if (foff) std::copy(c->foff.begin(), c->foff.end(), foff);
    return XPBD_OK;
}

int xpbd_clear_collisions(xpbd_ctx* c) {
    if (!c) return XPBD_ERR_INVALID;
    if (c->F) {
        XPBD_CU(c, cudaMemsetAsync(c->c_bary.p, 0, sizeof(float4) * (size_t)c->S * c->F, c->stream));
        XPBD_CU(c, cudaMemsetAsync(c->c_lam.p, 0, sizeof(float) * (size_t)c->S * c->F, c->stream));
        XPBD_CU(c, cudaMemsetAsync(c->rc_count.p, 0, sizeof(int), c->stream));
        if (c->self_on) XPBD_CU(c, cudaMemsetAsync(c->s_n_hits.p, 0, sizeof(int), c->stream));
        c->contact_lists_dirty = true;
    }
    std::fill(c->api_slots.begin(), c->api_slots.end(), 0);
    return XPBD_OK;
}

int xpbd_detect_collisions(xpbd_ctx* c) {
    if (!c) return XPBD_ERR_INVALID;
    return detect(c);
}

int xpbd_add_static_collision(xpbd_ctx* c, int32_t face, double u, double v, double w, const double* p3,
                              const double* n3) {
    if (!c || !p3 || !n3) return XPBD_ERR_INVALID;
    if (face < 0 || face >= c->F) return fail(c, XPBD_ERR_INVALID, "face %d out of range", face);
    if (c->api_slots[face] < 0) {
        // slots were filled by a detection: count the active ones
        std::vector<float4> b((size_t)c->S * c->F);
        XPBD_CU(c, cudaMemcpyAsync(b.data(), c->c_bary.p, sizeof(float4) * b.size(), cudaMemcpyDeviceToHost,
                                   c->stream));
        XPBD_CU(c, cudaStreamSynchronize(c->stream));
        for (int f = 0; f < c->F; f++) {
            int k = 0;
            for (int s = 0; s < c->S; s++)
                if (b[(size_t)s * c->F + f].w != 0.f) k = s + 1;
            c->api_slots[f] = k;
        }
    }
    const int s = c->api_slots[face];
    if (s >= c->S) return fail(c, XPBD_ERR_CAPACITY, "face %d already has %d contacts", face, c->S);
    const size_t slot = (size_t)s * c->F + face;
    const float4 b = make_float4((float)u, (float)v, (float)w, 1.f);
    const float4 pp = make_float4((float)p3[0], (float)p3[1], (float)p3[2], 0.f);
    const float4 nn = make_float4((float)n3[0], (float)n3[1], (float)n3[2], 0.f);
    const float z = 0.f;
    XPBD_CU(c, cudaMemcpy(c->c_p.p + slot, &pp, sizeof pp, cudaMemcpyHostToDevice));
    XPBD_CU(c, cudaMemcpy(c->c_n.p + slot, &nn, sizeof nn, cudaMemcpyHostToDevice));
    XPBD_CU(c, cudaMemcpy(c->c_lam.p + slot, &z, sizeof z, cudaMemcpyHostToDevice));
    XPBD_CU(c, cudaMemcpy(c->c_bary.p + slot, &b, sizeof b, cudaMemcpyHostToDevice));
    c->api_slots[face] = s + 1;
    c->contact_lists_dirty = true;
    return XPBD_OK;
}

int xpbd_add_attachment(xpbd_ctx* c, int32_t vertex, const double* point3, const double* offset3, int32_t* id) {
    if (!c || !point3) return XPBD_ERR_INVALID;
    if (vertex < 0 || vertex >= c->V) return fail(c, XPBD_ERR_INVALID, "vertex %d out of range", vertex);
    for (int k = 0; k < 3; k++)
        if (!std::isfinite(point3[k]) || (offset3 && !std::isfinite(offset3[k])))
            return fail(c, XPBD_ERR_INVALID, "attachment point or offset is not finite");
    c->att_v.push_back(vertex);
    for (int k = 0; k < 3; k++) {
        c->att_point.push_back(point3[k]);
        c->att_offset.push_back(offset3 ? offset3[k] : 0.0);
    }
    if (id) *id = (int32_t)c->att_v.size() - 1;
    c->att_struct_dirty = true;
    return XPBD_OK;
}

int xpbd_set_attachment_point(xpbd_ctx* c, int32_t id, const double* point3) {
    if (!c || !point3) return XPBD_ERR_INVALID;
    if (id < 0 || id >= (int)c->att_v.size()) return fail(c, XPBD_ERR_INVALID, "attachment %d does not exist", id);
    for (int k = 0; k < 3; k++) {
        if (!std::isfinite(point3[k])) return fail(c, XPBD_ERR_INVALID, "attachment point is not finite");
        c->att_point[3 * id + k] = point3[k];
    }
    c->att_target_dirty = true;
    return XPBD_OK;
}

int xpbd_clear_attachments(xpbd_ctx* c) {
    if (!c) return XPBD_ERR_INVALID;
    if (!c->att_v.empty()) c->att_struct_dirty = true;
    c->att_v.clear();
    c->att_point.clear();
    c->att_offset.clear();
    return XPBD_OK;
}

int xpbd_num_attachments(xpbd_ctx* c, int32_t* n) {
    if (!c || !n) return XPBD_ERR_INVALID;
    *n = (int32_t)c->att_v.size();
    return XPBD_OK;
}

int xpbd_get_collisions(xpbd_ctx* c, int32_t max_rows, double* rows, int32_t* n_out) {
    if (!c || !n_out || max_rows < 0 || (max_rows > 0 && !rows)) return XPBD_ERR_INVALID;
    *n_out = 0;
    if (!c->F) return XPBD_OK;
    const size_t ns = (size_t)c->S * c->F;
    std::vector<float4> b(ns), pp(ns), nn(ns);
    std::vector<float> l(ns);
    XPBD_CU(c, cudaMemcpyAsync(b.data(), c->c_bary.p, sizeof(float4) * ns, cudaMemcpyDeviceToHost, c->stream));
    XPBD_CU(c, cudaMemcpyAsync(pp.data(), c->c_p.p, sizeof(float4) * ns, cudaMemcpyDeviceToHost, c->stream));
    XPBD_CU(c, cudaMemcpyAsync(nn.data(), c->c_n.p, sizeof(float4) * ns, cudaMemcpyDeviceToHost, c->stream));
    XPBD_CU(c, cudaMemcpyAsync(l.data(), c->c_lam.p, sizeof(float) * ns, cudaMemcpyDeviceToHost, c->stream));
    XPBD_CU(c, cudaStreamSynchronize(c->stream));
    int k = 0;
    for (size_t sl = 0; sl < ns; sl++) {
        if (b[sl].w == 0.f) continue;
        if (k < max_rows) {
            double* r = rows + 12 * (size_t)k;
            r[0] = (double)(sl / c->F); r[1] = (double)(sl % c->F);
            r[2] = b[sl].x; r[3] = b[sl].y; r[4] = b[sl].z;
            r[5] = pp[sl].x; r[6] = pp[sl].y; r[7] = pp[sl].z;
            r[8] = nn[sl].x; r[9] = nn[sl].y; r[10] = nn[sl].z;
            r[11] = l[sl];
        }
        k++;
    }
    *n_out = k;
    return XPBD_OK;
}

int xpbd_get_self_contacts(xpbd_ctx* c, int32_t max_rows, int32_t* vf, double* lam, int32_t* n_out) {
    if (!c || !n_out || max_rows < 0 || (max_rows > 0 && !vf)) return XPBD_ERR_INVALID;
    *n_out = 0;
    if (!c->self_on) return XPBD_OK;
    int n = 0;
    XPBD_CU(c, cudaMemcpyAsync(&n, c->s_n_hits.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    XPBD_CU(c, cudaStreamSynchronize(c->stream));
    const int k = std::min(n, (int)max_rows);
    if (k > 0) {
        std::vector<int2> ct(k);
        std::vector<float> l(k);
        XPBD_CU(c, cudaMemcpy(ct.data(), c->s_contact.p, sizeof(int2) * k, cudaMemcpyDeviceToHost));
        XPBD_CU(c, cudaMemcpy(l.data(), c->s_lam.p, sizeof(float) * k, cudaMemcpyDeviceToHost));
        for (int i = 0; i < k; i++) {
            vf[2 * i] = ct[i].x;
            vf[2 * i + 1] = ct[i].y;
            if (lam) lam[i] = l[i];
        }
    }
    *n_out = n;
    return XPBD_OK;
}

int xpbd_update(xpbd_ctx* c) {
    if (!c) return XPBD_ERR_INVALID;
    return run_update(c, false);
}

int xpbd_velocity_update(xpbd_ctx* c) {
    if (!c) return XPBD_ERR_INVALID;
    {
        Scope sc(c, K_VELOCITY);
        launch_velocity(c->L(), c->x.p, c->prev.p, c->vel.p, c->V, (float)c->prm.dt);
    }
    if (c->nbodies) {
        Scope sc(c, K_VELOCITY);
        launch_rigid_velocity(c->L(), c->rb.p, c->nbodies, c->prm.dt);
    }
    return after_launches(c, "velocity update");
}

int xpbd_step(xpbd_ctx* c, int32_t nsteps) {
    if (!c || nsteps < 0) return XPBD_ERR_INVALID;
    const double interval = c->prm.collision_rate > 0 ? 1.0 / c->prm.collision_rate : 1e300;
    for (int k = 0; k < nsteps; k++) {
        const bool cd = (c->time - c->last_cd > interval);
        if (cd && (c->n_spheres_total > 0 || c->self_on)) {
            int st = detect(c);
            if (st) return st;
        } else if (cd) {
            int st = xpbd_clear_collisions(c);
            if (st) return st;
        }
        int st = run_update(c, true);
        if (st) return st;
        if (c->time - c->last_cd > interval) c->last_cd = c->time;
        c->time += c->prm.dt;
    }
    return XPBD_OK;
}

int xpbd_synchronize(xpbd_ctx* c) {
    if (!c) return XPBD_ERR_INVALID;
    XPBD_CU(c, cudaStreamSynchronize(c->stream));
    Flags f{};
    XPBD_CU(c, cudaMemcpy(&f, c->flags.p, sizeof f, cudaMemcpyDeviceToHost));
    if (f.timeouts)
        return fail(c, XPBD_ERR_TIMEOUT, "%llu bounded device waits gave up (their work was skipped)", f.timeouts);
    if (f.nonfinite) return fail(c, XPBD_ERR_NUMERIC, "%llu projections produced non-finite updates", f.nonfinite);
    return XPBD_OK;
}

int xpbd_get_time(xpbd_ctx* c, double* t) {
    if (!c || !t) return XPBD_ERR_INVALID;
    *t = c->time;
    return XPBD_OK;
}

int xpbd_residual_history(xpbd_ctx* c, double* out, int32_t max_n, int32_t* n_out) {
    if (!c || !n_out || max_n < 0 || (max_n > 0 && !out)) return XPBD_ERR_INVALID;
    *n_out = 0;
    if (!c->rows_pending && c->last_rows == 0) return XPBD_OK;
    XPBD_CU(c, cudaStreamSynchronize(c->stream));
    if (!tracking(c)) return XPBD_OK;
    const int n = c->last_rows;
    if (c->prm.residual_policy == XPBD_RESIDUAL_EVERY_SUBSTEP) {
        // only r(x_pred, 0) and the final residual are evaluated
        if (max_n > 0) out[0] = std::sqrt(c->h_rows[0]);
        if (max_n > 1) out[1] = std::sqrt(c->h_rows[n - 1]);
        *n_out = std::min(2, max_n);
        return XPBD_OK;
    }
    for (int i = 0; i < n && i < max_n; i++) out[i] = std::sqrt(c->h_rows[i]);
    *n_out = std::min(n, max_n);
    return XPBD_OK;
}

int xpbd_residual(xpbd_ctx* c, double* abs_norm, double* rel) {
    if (!c || !abs_norm) return XPBD_ERR_INVALID;
    // exact residual at the current state into a scratch row past the history
    const int row = std::max(c->last_rows, c->prm.num_iters + 1);
    int st = ensure_residual_rows(c, row + 1);
    if (st) return st;
    XPBD_CU(c, cudaMemsetAsync(c->res_partial.p + (size_t)row * c->res_stride, 0, sizeof(double) * c->res_stride,
                               c->stream));
    exact_residual_row(c, row, false);
    launch_reduce_rows(c->L(), c->res_partial.p + (size_t)row * c->res_stride, 1, c->res_stride,
                       c->res_rows.p + row);
    double v = 0;
    XPBD_CU(c, cudaMemcpyAsync(&v, c->res_rows.p + row, sizeof v, cudaMemcpyDeviceToHost, c->stream));
    XPBD_CU(c, cudaStreamSynchronize(c->stream));
    *abs_norm = std::sqrt(v);
    if (rel) {
        *rel = -1.0;
        if (tracking(c) && c->last_rows > 0) {
            const double r0 = std::sqrt(c->h_rows[0]);
            *rel = r0 > 0 ? *abs_norm / r0 : 0.0;
        }
    }
    return after_launches(c, "residual");
}

int xpbd_get_constraint_residual(xpbd_ctx* c, double* r, int64_t n) {
    if (!c || !r || n < 2LL * c->T) return XPBD_ERR_INVALID;
    if (!c->have_rvec) {
        // no stored residual: evaluate at the current state
        launch_residual(c->L(), c->block, c->tets(), c->T, c->x.p,
                        c->prm.constraint_type == XPBD_CONSTRAINT_SEPARATE, c->perm.p, c->rvec.p, no_sink(), nullptr,
                        (float)(c->prm.dt * c->prm.dt));
    }
    std::vector<float> h(2 * (size_t)c->T);
    XPBD_CU(c, cudaMemcpyAsync(h.data(), c->rvec.p, sizeof(float) * h.size(), cudaMemcpyDeviceToHost, c->stream));
    XPBD_CU(c, cudaStreamSynchronize(c->stream));
    for (size_t i = 0; i < h.size(); i++) r[i] = h[i];
    return after_launches(c, "constraint residual");
}

int xpbd_get_lambda(xpbd_ctx* c, double* lam) {
    if (!c || !lam) return XPBD_ERR_INVALID;
    std::vector<float2> h(c->T);
    XPBD_CU(c, cudaMemcpyAsync(h.data(), c->lam.p, sizeof(float2) * c->T, cudaMemcpyDeviceToHost, c->stream));
    XPBD_CU(c, cudaStreamSynchronize(c->stream));
    for (int sidx = 0; sidx < c->T; sidx++) {
        const int t = c->tet_of_slot[sidx];
        lam[2 * (size_t)t] = h[sidx].x;
        lam[2 * (size_t)t + 1] = h[sidx].y;
    }
    return XPBD_OK;
}

int xpbd_total_strain_energy(xpbd_ctx* c, double* e) {
    if (!c || !e) return XPBD_ERR_INVALID;
    const int nb = residual_blocks(c->T, c->block);
    launch_residual(c->L(), c->block, c->tets(), c->T, c->x.p, c->prm.constraint_type == XPBD_CONSTRAINT_SEPARATE,
                    c->perm.p, nullptr, no_sink(), c->energy_partial.p, (float)(c->prm.dt * c->prm.dt));
    launch_reduce_rows(c->L(), c->energy_partial.p, 1, nb, c->energy_partial.p + nb);
    double v = 0;
    XPBD_CU(c, cudaMemcpyAsync(&v, c->energy_partial.p + nb, sizeof v, cudaMemcpyDeviceToHost, c->stream));
    XPBD_CU(c, cudaStreamSynchronize(c->stream));
    *e = v;
    return after_launches(c, "strain energy");
}

int xpbd_debug_stall_vertex(xpbd_ctx* c, int32_t vertex, int32_t poll_limit) {
    if (!c) return XPBD_ERR_INVALID;
    if (!c->flow_versioned || c->patch_ver_h.empty())
        return fail(c, XPBD_ERR_STATE, "no versioned dataflow sweep in this context");
    if (vertex >= c->V || (vertex >= 0 && poll_limit <= 0)) return XPBD_ERR_INVALID;
    XPBD_CU(c, cudaStreamSynchronize(c->stream));  // no sweep in flight reads the tables
    std::vector<int4> ver = c->patch_ver_h;
    if (vertex >= 0) {
        const int P = c->npatches;
        std::vector<int4> meta(P), verts(2 * (size_t)P);
        XPBD_CU(c, cudaMemcpy(meta.data(), c->patch_meta.p, sizeof(int4) * P, cudaMemcpyDeviceToHost));
        XPBD_CU(c, cudaMemcpy(verts.data(), c->patch_verts.p, sizeof(int4) * 2 * (size_t)P, cudaMemcpyDeviceToHost));
        for (int q = 0; q < P; q++) {
            const int4 a = verts[2 * (size_t)q], b = verts[2 * (size_t)q + 1];
            const int vid[kMaxPatchVerts] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
            int* w = &ver[q].x;
            for (int k = 0; k < (meta[q].y >> 8); k++)
                if (vid[k] == vertex) w[k >> 1] |= 0xff << (16 * (k & 1));  // pre = 255
        }
        c->flow_poll_limit = (unsigned)poll_limit;
    } else {
        c->flow_poll_limit = kFlowLimit;
    }
    XPBD_CU(c, cudaMemcpy(c->patch_ver.p, ver.data(), sizeof(int4) * ver.size(), cudaMemcpyHostToDevice));
    c->graph_dirty = true;  // the poll limit is a launch argument
    return XPBD_OK;
}

int xpbd_health(xpbd_ctx* c, int64_t* nonfinite, int64_t* degenerate) {
    if (!c) return XPBD_ERR_INVALID;
    XPBD_CU(c, cudaStreamSynchronize(c->stream));
    Flags f{};
    XPBD_CU(c, cudaMemcpy(&f, c->flags.p, sizeof f, cudaMemcpyDeviceToHost));
    XPBD_CU(c, cudaMemset(c->flags.p, 0, sizeof f));
    if (nonfinite) *nonfinite = (int64_t)f.nonfinite;
    if (degenerate) *degenerate = (int64_t)f.degenerate;
    return XPBD_OK;
}

int xpbd_num_colours(xpbd_ctx* c, int32_t* nt, int32_t* nf) {
    if (!c) return XPBD_ERR_INVALID;
    if (nt) *nt = c->n_tet_colours;
    if (nf) *nf = c->n_face_colours;
    return XPBD_OK;
}

int xpbd_get_tet_colours(xpbd_ctx* c, int32_t* col) {
    if (!c || !col) return XPBD_ERR_INVALID;
    std::copy(c->tet_colour.begin(), c->tet_colour.end(), col);
    return XPBD_OK;
}

int xpbd_get_sweep_order(xpbd_ctx* c, int32_t* order) {
    if (!c || !order) return XPBD_ERR_INVALID;
    std::copy(c->tet_of_slot.begin(), c->tet_of_slot.end(), order);
    return XPBD_OK;
}

int xpbd_get_local_order(xpbd_ctx* c, int32_t* order, int32_t* colour_offsets, int32_t max_colours,
                         int32_t* n_colours) {
    if (!c || !order || !n_colours) return XPBD_ERR_INVALID;
    if (c->local_tets_h.empty())
        return fail(c, XPBD_ERR_STATE, "no local collision iterations (needs faces and num_local_collision_iters > 0)");
    const int nc = (int)c->lcol_off.size() - 1;
    *n_colours = nc;
    std::copy(c->local_tets_h.begin(), c->local_tets_h.end(), order);
    if (colour_offsets) {
        if (max_colours < nc + 1) return fail(c, XPBD_ERR_CAPACITY, "need %d colour offsets", nc + 1);
        std::copy(c->lcol_off.begin(), c->lcol_off.end(), colour_offsets);
    }
    return XPBD_OK;
}

static const char* kNames[K_COUNT] = {"predict",  "project_jacobi", "apply",    "project_gs",
                                      "contacts", "detect",         "finalize", "residual",
                                      "reduce",   "kinematic",      "gather_apply", "velocity",
                                      "warm_start", "mlp", "local_mark"};

const char* xpbd_kernel_name(int32_t id) { return (id >= 0 && id < K_COUNT) ? kNames[id] : "?"; }

int xpbd_profile_steps(xpbd_ctx* c, int32_t nsteps, int32_t max_k, double* avg_ms, int64_t* launches) {
    if (!c || nsteps < 0 || max_k < 0 || (max_k > 0 && (!avg_ms || !launches))) return XPBD_ERR_INVALID;
    XPBD_CU(c, cudaStreamSynchronize(c->stream));
    c->prof.on = true;
    c->prof.used = 0;
    c->prof.ids.clear();
    int st = xpbd_step(c, nsteps);
    c->prof.on = false;
    if (st) return st;
    XPBD_CU(c, cudaStreamSynchronize(c->stream));
    std::vector<double> tot(K_COUNT, 0.0);
    std::vector<long long> cnt(K_COUNT, 0);
    for (size_t i = 0; i < c->prof.ids.size(); i++) {
        float ms = 0;
        XPBD_CU(c, cudaEventElapsedTime(&ms, c->prof.pool[2 * i], c->prof.pool[2 * i + 1]));
        tot[c->prof.ids[i]] += ms;
        cnt[c->prof.ids[i]]++;
    }
    for (int k = 0; k < max_k; k++) {
        avg_ms[k] = (k < K_COUNT && cnt[k]) ? tot[k] / cnt[k] : 0.0;
        launches[k] = k < K_COUNT ? cnt[k] : 0;
    }
    return XPBD_OK;
}

int xpbd_launch_count(xpbd_ctx* c, int64_t* n) {
    if (!c || !n) return XPBD_ERR_INVALID;
    *n = c->launches;
    return XPBD_OK;
}

// Autotuner: times candidate launch configurations on trial contexts built
// from the caller's meshes and keeps the fastest. Trials start from the rest
// state with gravity off, so every candidate does the same, stable work.
int xpbd_autotune(const xpbd_mesh_desc* meshes, int32_t n_inst, xpbd_params* params, int32_t trial_steps,
                  char* report, int32_t report_len) {
    if (!meshes || n_inst <= 0 || !params || trial_steps <= 0 || (report_len > 0 && !report)) return XPBD_ERR_INVALID;
    if (!valid_params(*params)) return XPBD_ERR_INVALID;
    std::vector<xpbd_params> cands;
    xpbd_params base = *params;
    base.g_accel = 0.0;
    base.residual_policy = XPBD_RESIDUAL_NEVER;
    base.use_graphs = 1;
    if (base.solver_type == XPBD_SOLVER_GAUSS_SEIDEL) {
        for (int patch : {1, 2, 3, 5})
            for (int pdl : {0, 1})
                // variant x min blocks: (0,-) (1,6) (1,8) (2,uncapped) (3,-) (4,uncapped)
                for (int var_minb : {6, 16, 18, 20, 30, 40}) {
                    xpbd_params q = base;
                    q.gs_patch_tets = patch;
                    q.use_pdl = pdl;
                    q.gs_variant = var_minb / 10;
                    q.gs_min_blocks = var_minb % 10;
                    cands.push_back(q);
                }
    } else {
        for (int block : {64, 128, 256})
            for (int variant : {XPBD_JACOBI_ATOMIC, XPBD_JACOBI_GATHER})
                for (int pdl : {0, 1}) {
                    xpbd_params q = base;
                    q.block_size = block;
                    q.jacobi_variant = variant;
                    q.use_pdl = pdl;
                    cands.push_back(q);
                }
    }
    std::string rep = "[";
    double best = 1e300;
    int best_i = -1;
    for (size_t i = 0; i < cands.size(); i++) {
        xpbd_ctx* c = nullptr;
        int st = xpbd_create_batch(meshes, n_inst, &cands[i], &c);
        if (st) return st;
        double ms = -1;
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        if (cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess &&
            xpbd_step(c, 2) == XPBD_OK && cudaStreamSynchronize(c->stream) == cudaSuccess) {
            cudaEventRecord(e0, c->stream);
            st = xpbd_step(c, trial_steps);
            cudaEventRecord(e1, c->stream);
            float f = 0;
            if (st == XPBD_OK && cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(&f, e0, e1) == cudaSuccess)
                ms = f / trial_steps;
        }
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        xpbd_destroy(c);
        char buf[256];
        snprintf(buf, sizeof buf,
                 "%s{\"gs_patch_tets\":%d,\"gs_variant\":%d,\"gs_min_blocks\":%d,\"block_size\":%d,"
                 "\"jacobi_variant\":%d,\"use_pdl\":%d,\"ms_per_step\":%.6f}",
                 i ? "," : "", cands[i].gs_patch_tets, cands[i].gs_variant, cands[i].gs_min_blocks,
                 cands[i].block_size, cands[i].jacobi_variant, cands[i].use_pdl, ms);
        rep += buf;
        if (ms > 0 && ms < best) {
            best = ms;
            best_i = (int)i;
        }
    }
    rep += "]";
    if (report_len > 0) {
        std::strncpy(report, rep.c_str(), (size_t)report_len - 1);
        report[report_len - 1] = 0;
    }
    if (best_i < 0) return XPBD_ERR_CUDA;
    const xpbd_params& w = cands[best_i];
    params->gs_patch_tets = w.gs_patch_tets;
    params->block_size = w.block_size;
    params->jacobi_variant = w.jacobi_variant;
    params->use_pdl = w.use_pdl;
    params->gs_min_blocks = w.gs_min_blocks;
    params->gs_variant = w.gs_variant;
    return XPBD_OK;
}

int xpbd_get_stream(xpbd_ctx* c, void** stream) {
    if (!c || !stream) return XPBD_ERR_INVALID;
    *stream = (void*)c->stream;
    return XPBD_OK;
}

}  // extern "C"
