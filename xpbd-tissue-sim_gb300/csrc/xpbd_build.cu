// Context construction for the C ABI: uploads one or more meshes, computes rest
// shapes Q = Dm^-1, volumes, compliances and lumped masses in FP64
// (ElementConstraint.hpp:23-51, HydrostaticConstraint.cpp:15-16,
// DeviatoricConstraint.cpp:13, ElasticMaterial.hpp:31-32,
// XPBDMeshObject.cpp:277-331), and builds the Gauss-Seidel patches and
// colours, the dataflow tasks, the Jacobi CSR, the contact tables and the
// self-collision grid.
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

namespace xg {
namespace host {

namespace {

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
}  // namespace

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


void release(xpbd_ctx* c) {
    drop_graphs(c);
    for (auto e : c->prof.pool) cudaEventDestroy(e);
    c->x.release(); c->prev.release(); c->vel.release(); c->dx.release(); c->dxt.release();
    c->tet_idx.release(); c->q0.release(); c->q1.release(); c->q2.release(); c->m0.release(); c->m1.release(); c->m2.release(); c->lam.release();
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
    c->patch_ver.release(); c->xv.release(); c->vperm.release(); c->pverts_v.release(); c->faces_v.release();
    c->vdeg_p.release(); c->vdeg_c.release(); c->factive.release(); c->vface_off.release(); c->vface.release();
    c->fcol_d.release(); c->cm_off.release(); c->n_ctasks.release(); c->ctask.release(); c->cface.release();
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
    const bool with_faces = c->F > 0;  // variant 4 may then run the contacts inside the sweep
    const int per_sm =
        c->prm.gs_variant == 4
            ? std::min(std::min(sweep_versioned_blocks_per_sm(c->prm.gs_min_blocks, 0, false),
                                with_faces ? sweep_versioned_blocks_per_sm(c->prm.gs_min_blocks, 0, true) : 1 << 20),
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
        // The sweep's own vertex numbering: records in the order in which the
        // tasks' lanes first touch the vertices (task by task, corner by
        // corner, lane by lane), so the 32 lanes of one poll or store mostly
        // hit consecutive 32-byte records -- eight 128-byte lines instead of
        // up to 32 -- on the L1 data path that bounds the phase.
        std::vector<int> vperm(V, -1);
        int next_rec = 0;
        for (int j = 0; j < NTP; j++) {
            const int4 tk = tasks[j];
            for (int k = 0; k < kMaxPatchVerts; k++)
                for (int L = 0; L < tk.y; L++) {
                    const int q = tk.x + L;
                    if (k >= (pmeta[q].y >> 8)) continue;
                    const int v = pv(q, k);
                    if (vperm[v] < 0) vperm[v] = next_rec++;
                }
        }
        for (int v = 0; v < V; v++)
            if (vperm[v] < 0) vperm[v] = next_rec++;
        std::vector<int4> pvv(pverts.size());
        for (int q = 0; q < P; q++) {
            int r[kMaxPatchVerts];
            for (int k = 0; k < kMaxPatchVerts; k++) r[k] = k < (pmeta[q].y >> 8) ? vperm[pv(q, k)] : -1;
            pvv[2 * (size_t)q] = make_int4(r[0], r[1], r[2], r[3]);
            pvv[2 * (size_t)q + 1] = make_int4(r[4], r[5], r[6], r[7]);
        }
        c->flow_versioned = true;
        c->patch_ver_h = ver;
        c->vperm_h = vperm;
        XPBD_CU(c, c->patch_ver.alloc(P));
        XPBD_CU(c, c->xv.alloc(V));
        XPBD_CU(c, c->vperm.alloc(V));
        XPBD_CU(c, c->pverts_v.alloc(pvv.size()));
        XPBD_CU(c, cudaMemcpy(c->vperm.p, vperm.data(), sizeof(int) * V, cudaMemcpyHostToDevice));
        XPBD_CU(c, cudaMemcpy(c->pverts_v.p, pvv.data(), sizeof(int4) * pvv.size(), cudaMemcpyHostToDevice));
        c->npatches = P;
        // the task topology stays in shared memory when every warp owns few
        // enough tasks and the grid stays co-resident with that memory
        const int W = c->flow_grid * (kFlowBlock / 32);
        const int per_warp = (NTP + W - 1) / W;
        c->flow_resident = false;
        if (per_warp <= kResidentTasks && !c->prm.gs_topology_reload) {
            int res_sm = sweep_versioned_blocks_per_sm(c->prm.gs_min_blocks, per_warp, false);
            if (with_faces) res_sm = std::min(res_sm, sweep_versioned_blocks_per_sm(c->prm.gs_min_blocks, per_warp, true));
            c->flow_resident = (long long)res_sm * sms >= c->flow_grid;
        }
        // Each sweep streams the tet records (48 B), the multipliers (8 B)
        // and, without the resident topology, the patch records (64 B) once;
        // the vertex records (32 B) are polled and written by every patch
        // around the vertex. When all of it is larger than 3/4 of the L2, the
        // streams go evict-first so that they pass through the L2 without
        // evicting the vertex records.
        int l2 = 0;
        XPBD_CU(c, cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev));
        const double streamed = 56.0 * c->T + (c->flow_resident ? 0.0 : 64.0 * P) + 32.0 * V;
        c->flow_l2_first = c->prm.gs_l2_stream > 0 || (c->prm.gs_l2_stream == 0 && streamed > 0.75 * l2);
        XPBD_CU(c, cudaMemcpy(c->patch_ver.p, ver.data(), sizeof(int4) * P, cudaMemcpyHostToDevice));
    }
    return XPBD_OK;
}

// Static tables of the versioned sweep's contact phases: per vertex its
// patch count and its surface faces (CSR), per face its colour, and room for
// the per-detection tables. Needs every vertex's writes per iteration --
// patches plus the faces containing it -- to fit the 8-bit fields, and at
// most 64 face colours; otherwise the contacts keep their own launches.
int build_flow_contacts(xpbd_ctx* c, const std::vector<int4>& pmeta, const std::vector<int4>& pverts,
                        const std::vector<int>& fcol) {
    c->flow_contacts = false;
    const int V = c->V, F = c->F, P = (int)pmeta.size();
    if (!c->flow_versioned || F == 0 || c->n_face_colours > kMaxFlowFaceColours) return XPBD_OK;
    std::vector<int> degp(V, 0);
    for (int q = 0; q < P; q++)
        for (int k = 0; k < (pmeta[q].y >> 8); k++) {
            const int4& a = pverts[2 * (size_t)q + (k >> 2)];
            const int kk = k & 3;
            degp[kk == 0 ? a.x : (kk == 1 ? a.y : (kk == 2 ? a.z : a.w))]++;
        }
    std::vector<int> off(V + 1, 0);
    for (int f = 0; f < F; f++)
        for (int q = 0; q < 3; q++) off[c->faces_h[3 * f + q] + 1]++;
    for (int v = 0; v < V; v++) off[v + 1] += off[v];
    std::vector<int> ent(std::max(off[V], 1)), fill(off.begin(), off.end() - 1);
    for (int f = 0; f < F; f++)
        for (int q = 0; q < 3; q++) ent[fill[c->faces_h[3 * f + q]]++] = f;
    std::vector<unsigned char> dp(V);
    for (int v = 0; v < V; v++) {
        if (degp[v] + (off[v + 1] - off[v]) > 255) return XPBD_OK;
        dp[v] = (unsigned char)degp[v];
    }
    const size_t ncm = (size_t)c->n_face_colours * c->n_inst + 1;
    XPBD_CU(c, c->vdeg_p.alloc(V));
    XPBD_CU(c, c->vdeg_c.alloc(V));
    XPBD_CU(c, c->factive.alloc(F));
    XPBD_CU(c, c->vface_off.alloc(V + 1));
    XPBD_CU(c, c->vface.alloc(ent.size()));
    XPBD_CU(c, c->fcol_d.alloc(F));
    XPBD_CU(c, c->cm_off.alloc(ncm));
    XPBD_CU(c, c->n_ctasks.alloc(1));
    XPBD_CU(c, c->ctask.alloc((size_t)F / 32 + c->n_face_colours + 1));
    XPBD_CU(c, c->cface.alloc(F));
    {
        std::vector<int4> fv(F);
        for (int f = 0; f < F; f++)
            fv[f] = make_int4(c->vperm_h[c->faces_h[3 * f]], c->vperm_h[c->faces_h[3 * f + 1]],
                              c->vperm_h[c->faces_h[3 * f + 2]], 0);
        XPBD_CU(c, c->faces_v.alloc(F));
        XPBD_CU(c, cudaMemcpy(c->faces_v.p, fv.data(), sizeof(int4) * F, cudaMemcpyHostToDevice));
    }
    XPBD_CU(c, cudaMemcpy(c->vdeg_p.p, dp.data(), V, cudaMemcpyHostToDevice));
    XPBD_CU(c, cudaMemset(c->vdeg_c.p, 0, V));
    XPBD_CU(c, cudaMemset(c->n_ctasks.p, 0, sizeof(int)));
    XPBD_CU(c, cudaMemcpy(c->vface_off.p, off.data(), sizeof(int) * (V + 1), cudaMemcpyHostToDevice));
    XPBD_CU(c, cudaMemcpy(c->vface.p, ent.data(), sizeof(int) * ent.size(), cudaMemcpyHostToDevice));
    XPBD_CU(c, cudaMemcpy(c->fcol_d.p, fcol.data(), sizeof(int) * F, cudaMemcpyHostToDevice));
    c->flow_contacts = true;
    return XPBD_OK;
}

// Self-collision data: the surface vertices, tets in index order, Dm^-1 and
// rest positions in double, and a uniform grid over the rest bounding box
// padded by a quarter of its extent, cells 1.1x the widest tet box at rest
// (a tet whose box outgrows a cell goes to the overflow list), at most
// 2^22 cells.
int build_self_collisions(xpbd_ctx* c, const std::vector<double>& X, const std::vector<double>& Q) {
    const int V = c->V, T = c->T;
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

    // Canonical corner order of the grid generator's five-tet hexes: in a
    // patch of split B (layout kHexLocB) tet 0's corners (a,b,c,d) become
    // (c,a,b,d) and tet 2's (a,b,c,d) become (a,c,b,d). Its layout is then
    // kHexLocA, so every grid hex takes the sweep's register path. A tet's
    // corner order changes neither its element (F = Ds Dm^-1 is the same) nor
    // its constraints; the rest shapes below follow the new order.
    if (p.solver_type == XPBD_SOLVER_GAUSS_SEIDEL) {
        const int cap = p.gs_patch_tets ? p.gs_patch_tets : kMaxPatchTets;
        for (const HostPatch& hp : build_patches(c->tets_h, T, cap)) {
            if (hp.n != 5 || hp.nv != 8 || hp.loc != kHexLocB) continue;
            int* a = &c->tets_h[4 * (size_t)hp.first];
            const int t0[4] = {a[2], a[0], a[1], a[3]};
            std::copy(t0, t0 + 4, a);
            int* b = &c->tets_h[4 * ((size_t)hp.first + 2)];
            std::swap(b[1], b[2]);
        }
    }

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
    std::vector<float4> h0(T), h1(T), h2(T), hm0(T), hm1(T), hm2(T);
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
        h2[sidx] = make_float4((float)q[8], 0.f, 0.f, 0.f);
        {
            // M = Q Q^T (q[3c + r] = Q(r, c)) and det Q, in FP64
            double M[3][3];
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) M[i][j] = q[i] * q[j] + q[3 + i] * q[3 + j] + q[6 + i] * q[6 + j];
            const double dq = q[0] * (q[4] * q[8] - q[7] * q[5]) - q[3] * (q[1] * q[8] - q[7] * q[2]) +
                              q[6] * (q[1] * q[5] - q[4] * q[2]);
            hm0[sidx] = make_float4((float)M[0][0], (float)M[1][1], (float)M[2][2], (float)M[0][1]);
            hm1[sidx] = make_float4((float)M[0][2], (float)M[1][2], (float)dq, atd);
            const double msum = M[0][0] + M[1][1] + M[2][2] + 2.0 * (M[0][1] + M[0][2] + M[1][2]);  // |q_3|^2
            hm2[sidx] = make_float4(ath, (float)gm[t], (float)msum, 0.f);
        }
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
    XPBD_CU(c, c->m0.alloc(T));
    XPBD_CU(c, c->m1.alloc(T));
    XPBD_CU(c, c->m2.alloc(T));
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
    // with faces only the versioned sweep (variant 4) takes the contacts into
    // its phases; variants 2 and 3 leave them to the launches
    if (!pmeta.empty() && p.solver_type == XPBD_SOLVER_GAUSS_SEIDEL && p.gs_variant >= 2 &&
        (F == 0 || (p.gs_variant == 4 && p.constraint_type == XPBD_CONSTRAINT_COMBINED && !p.self_collisions))) {
        int st = build_flow_tasks(c, pmeta, pverts);
        if (st) return st;
        if (F > 0) {
            st = build_flow_contacts(c, pmeta, pverts, fcol);
            if (st) return st;
        }
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
    XPBD_CU(c, cudaMemcpy(c->m0.p, hm0.data(), sizeof(float4) * T, cudaMemcpyHostToDevice));
    XPBD_CU(c, cudaMemcpy(c->m1.p, hm1.data(), sizeof(float4) * T, cudaMemcpyHostToDevice));
    XPBD_CU(c, cudaMemcpy(c->m2.p, hm2.data(), sizeof(float4) * T, cudaMemcpyHostToDevice));
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

void drop_graphs(xpbd_ctx* c) {
    for (auto& g : c->gexec)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    c->graph_kernels[0] = c->graph_kernels[1] = c->graph_kernels[2] = 0;
    c->graph_dirty = false;
}

}  // namespace host
}  // namespace xg
