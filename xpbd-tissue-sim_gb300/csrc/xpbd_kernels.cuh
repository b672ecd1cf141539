// Device data layout and kernel launchers of the GB300 XPBD solver.
//
// HBM layout (all arrays 16-byte aligned, structure-of-arrays):
//   x      float4[V]  position xyz, w = inverse mass; w < 0 marks a fixed vertex
//   prev   float4[V]  position at the start of the substep (w copied from x)
//   vel    float4[V]  velocity xyz
//   dx     float4[V]  Jacobi accumulator (zero between sweeps)
//   tet_idx int4[T]   vertex indices, in solver slot order
//   tet_m0  float4[T] M00 M11 M22 M01                  (M = Q Q^T, Q = Dm^-1)
//   tet_m1  float4[T] M02 M12 det(Q) alpha_tilde_dev
//   tet_m2  float4[T] alpha_tilde_hyd gamma |q_3|^2 0   (q_3 = -q_0 - q_1 - q_2)
//   lam     float2[T] (lambda_dev, lambda_hyd)
//   tet_q0  float4[T] Q(0,0) Q(1,0) Q(2,0) Q(0,1)      (Q column-major; read only
//   tet_q1  float4[T] Q(1,1) Q(2,1) Q(0,2) Q(1,2)       for the warm-start network's
//   tet_q2  float4[T] Q(2,2) 0 0 0                      deformation-gradient features)
// One tet costs 16 + 48 + 8 (+8 write) = 80 bytes of streamed data per sweep.
#pragma once

#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace xg {

// kernel ids for per-kernel profiling
enum KernelId {
    K_PREDICT = 0,
    K_PROJECT_JACOBI,
    K_APPLY,
    K_PROJECT_GS,
    K_CONTACT,
    K_DETECT,
    K_FINALIZE,
    K_RESIDUAL,
    K_REDUCE,
    K_KINEMATIC,
    K_GATHER,
    K_VELOCITY,
    K_WARM,
    K_MLP,
    K_LOCAL,
    K_COUNT
};

struct TetArrays {
    const int4* idx;
    const float4* m0;
    const float4* m1;
    const float4* m2;
    float2* lam;
    const float4* q0;
    const float4* q1;
    const float4* q2;
};

struct ContactArrays {
    float4* bary;   // u, v, w, active (1/0)           [S*F]
    float4* p;      // surface point                    [S*F]
    float4* n;      // normal                           [S*F]
    float* lam;     //                                  [S*F]
    const int4* faces;  // face vertex indices (w unused) [F]
    int F;
    int S;
};

// Gauss-Seidel patches: up to kMaxPatchTets consecutive tets on at most
// kMaxPatchVerts vertices, one thread each.
constexpr int kMaxPatchTets = 5;
constexpr int kMaxPatchVerts = 8;
// The local layout (the 60-bit word of a patch record, 3 bits per tet corner)
// of a grid hex of five tets under the patch builder's first-appearance
// numbering: tets (0,1,2,3), (0,2,4,5), (0,3,6,5), (2,3,7,5), (0,2,3,5). The
// grid generator's split A gives it directly; split B gives kHexLocB until
// the build reorders two of its tets' corners (tet 0: (a,b,c,d) -> (c,a,b,d),
// tet 2: (a,b,c,d) -> (a,c,b,d)), which leaves every tet's geometry as it is.
constexpr unsigned long long kHexLocA = 0xad0bdab98b10688ull;
constexpr unsigned long long kHexLocB = 0xacabd9af2b0a688ull;
constexpr int kPatchBlock = 64;
// Gauss-Seidel sweep kernels: 0 one lane per patch, static tet records
// prefetched into registers; 1 one lane per patch, records staged in shared
// memory by bulk copies; 2 four lanes per patch (one per tet corner), staged.
constexpr int kGsVariants = 2;
struct PatchArrays {
    const int4* meta;   // [P] x: first slot, y: ntets | nverts << 8, z/w: local vertex ids, 3 bits per
                        //     (tet i, corner j) at bit 12 i + 3 j of the 64-bit word (z low, w high)
    const int4* verts;  // [2P] the patch's vertex indices
};

constexpr int kMaxSpheres = 16;  // sphere slots per instance

// Free rigid bodies (RigidObject with fixed: false), one FP64 record each.
// Their SDF table entries carry body index + 1 in d.w (0: fixed), and their
// contacts are marked active = 2 by the detection.
constexpr int kRigidRec = 40;
enum RigidField {
    RB_P = 0,      // position [3]
    RB_Q = 3,      // orientation (x, y, z, w) [4]
    RB_V = 7,      // velocity [3]
    RB_W = 10,     // angular velocity [3]
    RB_PP = 13,    // position at the last velocity update [3]
    RB_QP = 16,    // orientation at the last velocity update [4]
    RB_M = 20,     // mass
    RB_I = 21,     // diagonal inertia [3]
    RB_II = 24,    // its inverse [3]
    RB_KIND = 27,  // SDF kind (0 sphere, 1 box, 2 cylinder)
    RB_D = 28,     // SDF dimensions [3]
    RB_ACC = 31,   // Jacobi sums of position [3] and orientation [4] increments
    RB_ENTRY = 38  // SDF table entry (instance * S + slot)
};

// Dataflow Gauss-Seidel (sweep variant 2): every iteration and colour in one
// cooperative launch. A task is up to 32 consecutive patches of one colour,
// run by one warp; a task waits until every task sharing a vertex with it has
// reached the right iteration (lower colours: this one, higher colours: the
// previous one), which is exactly the order of the colour-by-colour launches.
constexpr int kTaskPatches = 32;
constexpr unsigned kFlowLimit = 1u << 21;  // default polls of one dependency before giving up
// threads per block of the (register-prefetch) dataflow launch: one warp, so
// the warps spread evenly over the SMs
constexpr int kFlowBlock = 32;
struct TaskArrays {
    const int4* task;     // [ntasks] first patch, patch count, first slot, slot count;
                          // tasks in colour order
    const int* dep_off;   // [ntasks + 1] CSR into dep
    const int* dep;       // (task << 1) | 1 when that task has the higher colour
    unsigned* epoch;      // [ntasks] progress (variant 2: 32 lane releases per iteration,
                          // variant 3: iterations); zeroed before each launch
    unsigned* abort_flag; // set when a wait gives up; every waiter then leaves
    int ntasks;
    unsigned poll_limit;  // polls of one wait before it gives up
    unsigned poll_ns;     // variant 4: back-off between two polls of a vertex not yet due
    unsigned long long* stamp;  // variant 4, optional: stamp[2 + j] = device clock (ns) when
                                // task j ends its last iteration
    unsigned l2_first;    // variant 4: what a sweep streams once (tet records, multipliers,
                          // patch records) is loaded and stored evict-first in L2
};

// Variant 4's vertex record: four aligned 64-bit words (x, ver), (y, ver),
// (z, ver), (w, 0); low 32 bits the float's bits, high 32 bits the version
// (projections that wrote the vertex in this launch). w is the inverse mass,
// which the sweep reads and writes back unchanged. 32-byte aligned: one
// 256-bit access moves a record.
struct alignas(32) VerRec {
    unsigned long long x, y, z, w;
};
// face colours the versioned sweep's contact phases handle (more keep their own launches)
constexpr int kMaxFlowFaceColours = 64;
constexpr unsigned kPollNs = 128;  // default back-off of variant 4's polls

// Static contacts inside variant 4's sweep: after each detection, the faces
// with an active static contact in colour-major order (colour, instance,
// index), cut into tasks of up to 32 faces of one colour that follow the
// patch tasks of every iteration. A vertex is then written per iteration by
// each patch containing it and then by each active face containing it, in
// face-colour order; vdegc[v] counts those faces, and face[i] carries, per
// face vertex, its writes per iteration and the writes before this face's.
struct FlowContacts {
    const int2* task;         // [*ntasks] (first entry of face[], faces in the task)
    const int4* face;         // (face, due words of vertices 0-1, vertex 2, 0): per vertex
                              // (writes per iteration) | (writes before this face) << 8
    const int* ntasks;        // contact tasks per iteration (written after each detection)
    const unsigned char* vdegc;  // [V] active contact faces containing the vertex (sweep numbering)
    const int4* vfaces;       // [F] face vertices in the sweep's numbering
};
// variant 4 keeps the topology of a warp's tasks (patch records, vertex ids,
// version words: 64 B per lane and task) in shared memory across iterations
// when the warp owns at most this many tasks per iteration
constexpr int kResidentTasks = 10;

// Self-collisions (DeformableDeformableCollisionConstraint): a uniform grid
// over the positions, each tet in the cell of its centroid, queries over the
// 27 cells around a point; tets larger than a cell in some axis go to an
// overflow list that every query scans.
struct SelfGrid {
    float ox, oy, oz, cell;  // origin and cell size
    int nx, ny, nz;
};
struct SelfArrays {
    const int4* tets;       // [T] vertex indices in tet index order
    const double* Q;        // [9T] Dm^-1, column-major, double
    const double* X0;       // [3V] rest positions, double
    const float4* X0f;      // [V] rest positions, float
    const int* surf;        // [n_surf] surface vertices, ascending
    int n_surf;
    int* cell_count;        // [ncells] (zeroed before binning)
    int* cell_off;          // [ncells + 1]
    int* cell_fill;         // [ncells] (zeroed before binning)
    int* cell_tets;         // [T]
    int* tet_cell;          // [T] each tet's cell, -1 in the overflow list
    int* overflow;          // [T]
    int* n_overflow;        // [1] (zeroed before binning)
    int* hit_tet;           // [n_surf] lowest tet holding the vertex, -1 none
    int* hit_list;          // [n_surf] surface indices with a hit, ascending
    int* n_hits;            // [1]
    int2* contact;          // [n_surf] (vertex, face; face -1 = none), in hit order
    float* lam;             // [n_surf]
    int* scan_part;         // scan scratch, [ncells / 4096 + 2]
    int T, F;
};

struct Flags {
    unsigned long long nonfinite;
    unsigned long long degenerate;
    unsigned long long timeouts;  // bounded waits that gave up (the work was skipped)
};

// residual partial sums: one double per block per record row
struct ResidualSink {
    double* partial;  // nullptr = off
    int row;          // record row (iteration)
    int stride;       // doubles per row
    int offset;       // first slot of this launch in the row
};

// Where and how to launch: the stream, and whether the kernel may start
// before its predecessor finishes (programmatic dependent launch).
struct Launch {
    cudaStream_t s;
    bool pdl;
};

// ---- warm-start MLP (14 -> 64 -> 64 -> 64 -> 2, SiLU), BF16 tensor cores ----
// Flat FP32 parameter vector: W_k row-major (out x in), then b_k.
constexpr int kMlpIn = 16;  // 14 features, zero padded
constexpr int kMlpHid = 64;
constexpr int kOffW1 = 0;                    // 64 x 16
constexpr int kOffB1 = kOffW1 + 64 * 16;     // 64
constexpr int kOffW2 = kOffB1 + 64;          // 64 x 64
constexpr int kOffB2 = kOffW2 + 64 * 64;     // 64
constexpr int kOffW3 = kOffB2 + 64;          // 64 x 64
constexpr int kOffB3 = kOffW3 + 64 * 64;     // 64
constexpr int kOffW4 = kOffB3 + 64;          // 2 x 64
constexpr int kOffB4 = kOffW4 + 2 * 64;      // 2
constexpr int kMlpParams = kOffB4 + 2;

struct MlpNet {
    __nv_bfloat16 *w1, *w2, *w3, *w4, *w2t, *w3t;  // packed K-major operand tiles
    const float *b1, *b2, *b3, *b4;                // into the FP32 parameter vector
    float* w4f;                                    // BF16-rounded W4 as FP32 (2 x 64), backward pass
};

struct MlpCache {
    float* z[3];            // pre-activations of the hidden layers, [n][64]
    __nv_bfloat16* a[3];    // their BF16 activations, [n][64]
};

cudaError_t mlp_prepare_kernels();
int mlp_forward_smem();
int mlp_backward_smem();
void launch_mlp_pack(cudaStream_t s, const float* params, const MlpNet& net);
void launch_mlp_forward(cudaStream_t s, const __nv_bfloat16* X, int n, const MlpNet& net, float* out,
                        const MlpCache* cache, unsigned long long* err);
void launch_mlp_backward(cudaStream_t s, const __nv_bfloat16* X, const float* Y, int n, const MlpNet& net,
                         const MlpCache& cache, const float* out, float* grad, unsigned long long* err);
void launch_mse(cudaStream_t s, const float* out, const float* Y, int n, double* acc);
void launch_adam(cudaStream_t s, float* p, const float* g, float* m, float* v, int n, float lr, int step);

// ---- launchers (all asynchronous on L.s) ----
void launch_predict_first_order(const Launch& s, float4* x, float4* prev, const float* gdz, int V);
void launch_predict(const Launch& s, float4* x, float4* prev, const float4* vel, int V, float dt, float dz);
void launch_kinematic(const Launch& s, float4* x, const int* idx, const float4* rest, int n, float ox, float oy,
                      float oz);
void launch_project_jacobi(const Launch& s, int block, const TetArrays& t, int T, const float4* x, float4* dx,
                           bool first, bool separate, ResidualSink res, Flags* flags);
void launch_project_jacobi_gather_write(const Launch& s, int block, const TetArrays& t, int T, const float4* x,
                                        float4* dxt, bool first, bool separate, ResidualSink res, Flags* flags);
void launch_gather_apply(const Launch& s, float4* x, const float4* dxt, const int* csr_off, const int* csr_ent,
                         float4* dx, int V, float4* prev, float4* vel, bool final_step, float dt, bool write_vel);
void launch_apply(const Launch& s, float4* x, float4* dx, int V, float4* prev, float4* vel, bool final_step,
                  float dt, bool write_vel);
void launch_project_patches(const Launch& s, const TetArrays& t, const PatchArrays& pa, int pbegin, int pend,
                            float4* x, bool first, int which, Flags* flags, int min_blocks, int variant);
// returns the launch's status (cooperative launches can be refused)
// staged = true: the task's static tet records arrive in shared memory by bulk
// copies issued before the dependency wait (fewer registers, more warps)
cudaError_t launch_sweep_dataflow(const Launch& s, const TetArrays& t, const PatchArrays& pa, const TaskArrays& ta,
                                  int iters, bool first_zero, float4* x, Flags* flags, int grid, bool staged,
                                  int min_blocks);
// min_blocks (variant 2): 0 = no register cap, 6 or 8 blocks per SM
int sweep_dataflow_blocks_per_sm(bool staged, int min_blocks);
// Variant 4: the dataflow sweep on version-stamped vertices. Copies x into
// the records xv (version 0), runs every iteration and colour in one
// cooperative launch and copies the positions back; pver holds per patch and
// vertex slot the 16-bit deg << 8 | pre of that vertex (patches containing
// it, those of a lower colour). resident: each warp's task topology stays in
// shared memory (ntasks / warps <= kResidentTasks; sweep_versioned_smem bytes
// per block).
// fc.task != nullptr: the static contacts of ca run inside the sweep (FlowContacts).
// The sweep numbers the vertices its own way (vperm: vertex -> record of xv,
// chosen so that a task's lanes touch neighbouring records); pa.verts and
// fc.vfaces are in that numbering.
cudaError_t launch_sweep_versioned(const Launch& s, const TetArrays& t, const PatchArrays& pa, const int4* pver,
                                   const TaskArrays& ta, int iters, bool first_zero, float4* x, VerRec* xv, int V,
                                   const int* vperm, Flags* flags, int grid, int min_blocks, bool resident,
                                   const ContactArrays& ca, const FlowContacts& fc);
// blocks per SM of the versioned sweep with the dynamic shared memory it
// needs when each warp owns `tasks_per_warp` tasks (0: not resident), with or
// without the contact phases
int sweep_versioned_blocks_per_sm(int min_blocks, int tasks_per_warp, bool contacts);
// After a detection (the per-instance active lists built): the sweep's
// contact tables. vface_off/vface/fcol/vdegp are static: per vertex its
// surface faces (CSR) and patch count, per face its colour.
// one thread writes the device clock (ns) to *p once the stream's earlier work is done
void launch_stamp(const Launch& s, unsigned long long* p);
void launch_flow_contact_tables(const Launch& s, const ContactArrays& ca, const int* act_faces, const int* act_off,
                                int ncol, int n_inst, const int* vface_off, const int* vface, const int* fcol,
                                const unsigned char* vdegp, unsigned char* factive, int* cm_off, int2* ctask,
                                int* n_ctasks, int4* cface, unsigned char* vdegc, const int* vperm, int V);
inline size_t sweep_versioned_smem(int tasks_per_warp) { return (size_t)tasks_per_warp * 4 * 32 * sizeof(int4); }
void launch_contacts_jacobi(const Launch& s, const ContactArrays& c, const float4* x, float4* dx, bool first);
// after a detection: per instance and face colour, the faces with an active
// static contact (ifl: faces by instance, colour, index; ifo_off its ranges)
constexpr int kContactListThreads = 512;
void launch_contact_lists(const Launch& s, const ContactArrays& c, const int* ifl, const int* ifo_off, int ncol,
                          int n_inst, int* act_faces, int* act_off);
// every colour's Gauss-Seidel contacts in one launch, one block per instance
void launch_contacts_gs_lists(const Launch& s, const ContactArrays& c, const int* act_faces, const int* act_off,
                              int ncol, int n_inst, float4* x, bool first);
// prim: one 3-float4 primitive entry; out[i] = (sdf, gradient) at pts[i]
void launch_prim_eval(cudaStream_t s, const float4* prim, const float4* pts, int n, float4* out);
// sphere_table: 3 float4 per (instance, slot) primitive entry
void launch_detect(const Launch& s, const ContactArrays& c, const float4* x, const float4* sphere_table,
                   const int* face_inst);
void launch_finalize(const Launch& s, float4* x, const float4* prev, float4* vel, int V, float dt, bool write_vel);
void launch_velocity(const Launch& s, const float4* x, const float4* prev, float4* vel, int V, float dt);
void launch_residual(const Launch& s, int block, const TetArrays& t, int T, const float4* x, bool separate,
                     const int* perm, float* rvec, ResidualSink res, double* energy_partial, float dt2,
                     bool zero_lam = false);
// free rigid bodies: table entries from the bodies' poses; the ordered list of
// rigid contacts; their projection (Gauss-Seidel in list order, or Jacobi from
// one state with summed increments); RigidObject::update and velocityUpdate
void launch_rigid_sync_table(const Launch& s, const double* rb, int nb, float4* table);
void launch_rigid_compact(const Launch& s, const ContactArrays& c, int* list, int* count);
void launch_rigid_contacts(const Launch& s, const ContactArrays& c, const int* list, const int* count,
                           const float4* table, const int* face_inst, double* rb, int nb, float4* x, float4* dx,
                           bool jacobi, bool first, Flags* flags);
void launch_rigid_update(const Launch& s, double* rb, int nb, double dt, double g);
void launch_rigid_velocity(const Launch& s, double* rb, int nb, double dt);
// self-collision detection (after the SDF contacts) and projection
void launch_self_detect(const Launch& s, const SelfArrays& a, const SelfGrid& g, const float4* x, const int4* faces);
void launch_self_contacts(const Launch& s, const SelfArrays& a, const int4* faces, float4* x, float4* dx,
                          bool jacobi, bool first, float alpha_tilde, Flags* flags);
// positions and velocities from / to host arrays the device can address
// (keep_w: the float4's w is left as it is; else 0)
void launch_xyz_from_host(cudaStream_t s, float4* x, const double* h, int V, bool keep_w);
void launch_xyz_from_host(cudaStream_t s, float4* x, const float* h, int V, bool keep_w);
void launch_xyz_to_host(cudaStream_t s, double* h, const float4* x, int V);
void launch_xyz_to_host(cudaStream_t s, float* h, const float4* x, int V);
void launch_attach_gs(const Launch& s, const int* vert, const float4* target, float* lam, const int* order, int begin,
                      int end, float4* x, bool first);
void launch_attach_jacobi(const Launch& s, const int* vert, const float4* target, float* lam, int n, const float4* x,
                          float4* dx, bool first);
void launch_mark_local(const Launch& s, const ContactArrays& c, const TetArrays& t, int T, unsigned char* vmask,
                       unsigned char* tmask);
void launch_project_local_gs(const Launch& s, const TetArrays& t, const int* order, int begin, int end,
                             const unsigned char* tmask, float4* x, int which, Flags* flags);
void launch_project_local_jacobi(const Launch& s, const TetArrays& t, int T, const unsigned char* tmask,
                                 const float4* x, float4* dx, bool separate, Flags* flags);
void launch_mlp_features(const Launch& s, const TetArrays& t, const float4* x, const float2* mat, float dt_feat,
                         int s0, int n, __nv_bfloat16* X);
void launch_mlp_targets(const Launch& s, const TetArrays& t, int s0, int n, float* Y);
void launch_warm_start(const Launch& s, const TetArrays& t, int T, const float* pred, const float4* x, float4* dx);
void launch_warm_fallback(const Launch& s, const double* rows, float4* x, const float4* x_pred, float2* lam, int V,
                          int T, unsigned long long* stats);
void launch_reduce_rows(const Launch& s, const double* partial, int rows, int stride, double* out);
int residual_blocks(int T, int block);

}  // namespace xg
