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
#include "xpbd_host.cuh"
#include "xpbd_kernels.cuh"

using namespace xg;
using namespace xg::host;

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
           (p.self_collisions == 0 || p.self_collisions == 1) && p.gs_poll_ns >= 0 && p.gs_poll_ns <= 1000000 &&
           (p.gs_topology_reload == 0 || p.gs_topology_reload == 1) && p.gs_l2_stream >= -1 && p.gs_l2_stream <= 1;
}

// The colour-launch kernel that stands in for a GS variant where the one-launch
// sweeps do not apply (contacts, attachments, residual every iteration):
// 0 = registers, 1 = staged records.
int patch_kernel_variant(int gs_variant) { return gs_variant == 1 || gs_variant == 3 ? 1 : 0; }

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
void enqueue_local_collision_iters(xpbd_ctx* c, int passes) {
    const xpbd_params& p = c->prm;
    const bool separate = p.constraint_type == XPBD_CONSTRAINT_SEPARATE;
    const ContactArrays ca = c->contacts();
    cudaMemsetAsync(c->vmask.p, 0, (size_t)c->V, c->stream);
    {
        Scope sc(c, K_LOCAL);
        launch_mark_local(c->L(), ca, c->tets(), c->T, c->vmask.p, c->tmask.p);
    }
    const int ncol = (int)c->lcol_off.size() - 1;
    for (int it = 0; it < passes; it++) {
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

// solve_only: XPBDSolver::solve() alone (XPBDSolver.hpp:66-97) -- lambda <- 0
// and num_iters sweeps on the current positions, with no inertial move, no
// local collision passes, no fixed reset and no rigid-body update.
int enqueue_update(xpbd_ctx* c, bool write_vel, bool solve_only) {
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
    if (!solve_only) {
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
    const bool local = !solve_only && have_faces && p.num_local_collision_iters > 0 && c->local_slots.p;
    const bool fuse_final = !track && !local && !solve_only;
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
    } else if (!separate && !every_iter && c->att_v.empty() &&
               (!have_faces || (p.gs_variant == 4 && c->flow_versioned && c->flow_contacts && !c->self_on &&
                                !c->nbodies)) &&
               (p.gs_variant == 2 || p.gs_variant == 3 || p.gs_variant == 4) && c->ntasks > 0) {
        // every iteration and colour in one cooperative launch (with faces:
        // the versioned sweep, static contacts after each iteration's patches)
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
            const xg::FlowContacts fc =
                have_faces ? c->flowc() : xg::FlowContacts{nullptr, nullptr, nullptr, nullptr, nullptr};
            launch_sweep_versioned(c->L(), c->tets(), c->patches_v(), c->patch_ver.p, c->tasks(), iters, !warm, c->x.p,
                                   c->xv.p, c->V, c->vperm.p, c->flags.p, c->flow_grid, p.gs_min_blocks,
                                   c->flow_resident, ca, fc);
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
    if (solve_only) return XPBD_OK;
    if (local) enqueue_local_collision_iters(c, p.num_local_collision_iters);
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
        if (c->flow_contacts)
            launch_flow_contact_tables(c->L(), c->contacts(), c->act_faces.p, c->act_off.p, c->n_face_colours,
                                       c->n_inst, c->vface_off.p, c->vface.p, c->fcol_d.p, c->vdeg_p.p,
                                       c->factive.p, c->cm_off.p, c->ctask.p, c->n_ctasks.p, c->cface.p,
                                       c->vdeg_c.p, c->vperm.p, c->V);
        c->contact_lists_dirty = false;
    }
    if (tracking(c) || c->warm_mode != XPBD_WARM_NONE) {
        // one extra row for on-demand residual queries, two for the warm start
        int st = ensure_residual_rows(c, c->prm.num_iters + 4);
        if (st) return st;
    }
    return XPBD_OK;
}

int run_update(xpbd_ctx* c, bool write_vel, bool solve_only) {
    int st = prepare_update(c);
    if (st) return st;
    if (c->graph_dirty) drop_graphs(c);
    const int gi = solve_only ? 2 : (write_vel ? 1 : 0);
    if (c->prm.use_graphs && !c->prof.on) {
        cudaGraphExec_t& ge = c->gexec[gi];
        if (!ge) {
            cudaGraph_t g = nullptr;
            XPBD_CU(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
            const long long before = c->launches;
            enqueue_update(c, write_vel, solve_only);
            c->graph_kernels[gi] = c->launches - before;
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
        c->launches += c->graph_kernels[gi];
    } else {
        enqueue_update(c, write_vel, solve_only);
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

int fetch(xpbd_ctx* c, const float4* src) {
    XPBD_CU(c, cudaMemcpyAsync(c->h_stage, src, sizeof(float4) * c->V, cudaMemcpyDeviceToHost, c->stream));
    XPBD_CU(c, cudaStreamSynchronize(c->stream));
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
    c->flow_poll_ns = p->gs_poll_ns > 0 ? (unsigned)p->gs_poll_ns : kPollNs;
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

int xpbd_set_latency_stamps(xpbd_ctx* c, int32_t on) {
    if (!c || (on != 0 && on != 1)) return XPBD_ERR_INVALID;
    if (on && !(c->flow_versioned && c->ntasks > 0))
        return fail(c, XPBD_ERR_STATE, "latency stamps need the persistent versioned sweep (gs_variant 4)");
    if (on && !c->lat.p) {
        // every patch task, and at most one contact task per face plus one per face colour
        XPBD_CU(c, c->lat.alloc(2 + (size_t)c->ntasks + (size_t)c->F + kMaxFlowFaceColours));
        XPBD_CU(c, cudaMemset(c->lat.p, 0, sizeof(unsigned long long) * c->lat.n));
    }
    if (on && c->task_inst_h.empty()) {
        // the instances each patch task's slot range touches
        std::vector<int4> tk(c->ntasks);
        XPBD_CU(c, cudaMemcpy(tk.data(), c->flow_tasks.p, sizeof(int4) * tk.size(), cudaMemcpyDeviceToHost));
        c->task_inst_h.assign(c->ntasks, make_int2(-1, -1));
        for (int j = 0; j < c->ntasks; j++) {
            if (tk[j].y <= 0) continue;  // padding task
            int lo = c->n_inst, hi = -1;
            for (int sl = tk[j].z; sl < tk[j].z + tk[j].w; sl++) {
                const int64_t t = c->tet_of_slot[sl];
                const int k = (int)(std::upper_bound(c->toff.begin(), c->toff.end(), t) - c->toff.begin()) - 1;
                lo = std::min(lo, k);
                hi = std::max(hi, k);
            }
            c->task_inst_h[j] = make_int2(lo, hi);
        }
    }
    if ((bool)on != c->lat_on) c->graph_dirty = true;  // the stamp pointer is a launch argument
    c->lat_on = on != 0;
    c->lat_have = false;
    return XPBD_OK;
}

int xpbd_instance_latencies(xpbd_ctx* c, double* ms, double* batch_ms) {
    if (!c || !ms) return XPBD_ERR_INVALID;
    if (!c->lat_on || !c->lat_have) return fail(c, XPBD_ERR_STATE, "no stamped substep since the stamps were turned on");
    XPBD_CU(c, cudaStreamSynchronize(c->stream));
    int nct = 0;
    if (c->F && c->flow_contacts) XPBD_CU(c, cudaMemcpy(&nct, c->n_ctasks.p, sizeof(int), cudaMemcpyDeviceToHost));
    const size_t ntot = (size_t)c->ntasks + nct;
    std::vector<unsigned long long> st(2 + ntot);
    XPBD_CU(c, cudaMemcpy(st.data(), c->lat.p, sizeof(unsigned long long) * st.size(), cudaMemcpyDeviceToHost));
    std::vector<unsigned long long> done(c->n_inst, 0);
    for (int j = 0; j < c->ntasks; j++) {
        const int2 r = c->task_inst_h[j];
        for (int k = r.x; k >= 0 && k <= r.y; k++) done[k] = std::max(done[k], st[2 + j]);
    }
    if (nct > 0) {
        // contact task -> its faces -> their instances
        std::vector<int2> ct(nct);
        XPBD_CU(c, cudaMemcpy(ct.data(), c->ctask.p, sizeof(int2) * nct, cudaMemcpyDeviceToHost));
        const int ne = ct.back().x + ct.back().y;
        std::vector<int4> fe(std::max(ne, 0));
        if (ne > 0) XPBD_CU(c, cudaMemcpy(fe.data(), c->cface.p, sizeof(int4) * ne, cudaMemcpyDeviceToHost));
        for (int j = 0; j < nct; j++)
            for (int e = ct[j].x; e < ct[j].x + ct[j].y; e++) {
                const int f = fe[e].x;
                const int k = (int)(std::upper_bound(c->foff.begin(), c->foff.end(), (int64_t)f) - c->foff.begin()) - 1;
                done[k] = std::max(done[k], st[2 + c->ntasks + j]);
            }
    }
    for (int k = 0; k < c->n_inst; k++) ms[k] = done[k] > st[0] ? (double)(done[k] - st[0]) * 1e-6 : 0.0;
    if (batch_ms) *batch_ms = st[1] > st[0] ? (double)(st[1] - st[0]) * 1e-6 : 0.0;
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
    if (c->lat_on) launch_stamp(c->L(), c->lat.p);
    int st = run_update(c, false, false);
    if (st) return st;
    if (c->lat_on) {
        launch_stamp(c->L(), c->lat.p + 1);
        c->lat_have = true;
    }
    return XPBD_OK;
}

int xpbd_solve(xpbd_ctx* c) {
    if (!c) return XPBD_ERR_INVALID;
    return run_update(c, false, true);
}

int xpbd_solve_local(xpbd_ctx* c, int32_t num_iter) {
    if (!c || num_iter < 0) return XPBD_ERR_INVALID;
    if (!c->F || !c->local_slots.p)
        return fail(c, XPBD_ERR_STATE,
                    "xpbd_solve_local: the context has no local collision passes (surface faces and "
                    "num_local_collision_iters > 0 at creation)");
    int st = prepare_update(c);
    if (st) return st;
    if (num_iter > 0 && c->F > 0) enqueue_local_collision_iters(c, num_iter);
    return after_launches(c, "local collision passes");
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
        if (c->lat_on) launch_stamp(c->L(), c->lat.p);
        if (cd && (c->n_spheres_total > 0 || c->self_on)) {
            int st = detect(c);
            if (st) return st;
        } else if (cd) {
            int st = xpbd_clear_collisions(c);
            if (st) return st;
        }
        int st = run_update(c, true, false);
        if (st) return st;
        if (c->lat_on) {
            launch_stamp(c->L(), c->lat.p + 1);
            c->lat_have = true;
        }
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
