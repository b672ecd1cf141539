/*
 * xpbd_gpu.h -- C ABI of the GB300 (sm_103a) XPBD substep solver.
 *
 * The reference (MAVYWAVY902/xpbd-tissue-sim) has no FFI: its solver seam is
 * the compile-time template interface XPBDSolver<IsFirstOrder, Projectors...>
 * owned by XPBDMeshObject_ (include/simobject/XPBDMeshObject.hpp:229), chosen
 * by the YAML key `solver-type` (include/config/simobject/XPBDMeshObjectConfig.hpp:26-34)
 * in XPBDObjectFactory (include/simobject/XPBDObjectFactory.hpp:53-77). Each
 * entry point below names the member of that surface it replaces.
 *
 * Conventions
 *  - Every call returns an int status (XPBD_OK = 0) and never aborts; the
 *    reference instead asserts (include/gpu/resource/GPUResource.hpp:8-19).
 *    xpbd_last_error() gives a message for the last failing call on a context.
 *  - Vertex arrays are 3 x V column-major doubles (x0,y0,z0,x1,...), the layout
 *    of Geometry::Mesh::VerticesMat (include/geometry/Mesh.hpp:29).
 *  - Tets are 4 x T int32, faces 3 x F int32, 0-based, as TetMesh stores them.
 *  - One context = one deformable object on one CUDA stream. A context is not
 *    thread-safe; distinct contexts are independent (the reference drives its
 *    solver from the single Simulation::update thread, Simulation.cpp:332-336).
 *  - The device computes in FP32; residual and energy reductions finish in FP64.
 */
#ifndef XPBD_GPU_H
#define XPBD_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define XPBD_ABI_VERSION 8

/* status codes */
#define XPBD_OK 0
#define XPBD_ERR_INVALID 1      /* bad argument or size                        */
#define XPBD_ERR_CUDA 2         /* a CUDA runtime call failed                  */
#define XPBD_ERR_NUMERIC 3      /* a projection produced a non-finite update   */
#define XPBD_ERR_NO_DEVICE 4    /* no CUDA device / extension not usable       */
#define XPBD_ERR_STATE 5        /* call not valid in the context's state       */
#define XPBD_ERR_CAPACITY 6     /* a fixed capacity was exceeded               */
#define XPBD_ERR_TIMEOUT 7      /* a bounded device wait gave up (work skipped) */

/* solver-type (XPBDObjectSolverTypeEnum, include/common/XPBDEnumTypes.hpp:6-11).
 * "Gauss-Seidel" maps to the graph-coloured Gauss-Seidel, "Jacobi" and
 * "Parallel-Jacobi" to the GPU Jacobi solver. */
#define XPBD_SOLVER_GAUSS_SEIDEL 0
#define XPBD_SOLVER_JACOBI 1

/* constraint-type (XPBDMeshObjectConstraintConfigurationEnum) */
#define XPBD_CONSTRAINT_COMBINED 0   /* "Stable-Neohookean-Combined" (2x2 solve)   */
#define XPBD_CONSTRAINT_SEPARATE 1   /* "Stable-Neohookean" (Dev, then Hyd)        */

/* residual-policy (XPBDSolverResidualPolicyEnum) */
#define XPBD_RESIDUAL_NEVER 0
#define XPBD_RESIDUAL_EVERY_SUBSTEP 1
#define XPBD_RESIDUAL_EVERY_ITERATION 2  /* records ||r|| before every iteration */

/* Jacobi scatter variant */
#define XPBD_JACOBI_ATOMIC 0   /* warp-level vector atomics into a delta buffer  */
#define XPBD_JACOBI_GATHER 1   /* per-tet deltas + vertex->tet CSR gather        */

typedef struct xpbd_ctx xpbd_ctx;

/* Mesh and per-element material, the data XPBDMeshObject_::setup() derives
 * from the loaded TetMesh and its ElasticMaterial list
 * (src/simobject/XPBDMeshObject.cpp:103-160, 277-417). */
typedef struct {
    int64_t num_vertices;
    int64_t num_tets;
    int64_t num_faces;        /* surface faces used by collision detection, may be 0 */
    const double* vertices;   /* 3 x V, column-major, rest = initial state           */
    const int32_t* tets;      /* 4 x T                                               */
    const int32_t* faces;     /* 3 x F or NULL                                       */
    const double* tet_E;      /* T Young's moduli [Pa]                               */
    const double* tet_nu;     /* T Poisson ratios                                    */
    const double* tet_density;/* T densities [kg/m^3]                                */
} xpbd_mesh_desc;

/* Solver parameters (Simulation + XPBDMeshObjectConfig keys). */
typedef struct {
    double dt;                 /* time-step [s]                                    */
    double g_accel;            /* g-accel [m/s^2], acts along -z                   */
    double collision_rate;     /* collision-rate [Hz]; <= 0 disables the cadence  */
    int32_t num_iters;         /* num-solver-iters                                 */
    int32_t solver_type;       /* XPBD_SOLVER_*                                    */
    int32_t constraint_type;   /* XPBD_CONSTRAINT_*                                */
    int32_t residual_policy;   /* XPBD_RESIDUAL_*                                  */
    int32_t jacobi_variant;    /* XPBD_JACOBI_*                                    */
    int32_t block_size;        /* threads per block for tet kernels; 0 = default   */
    int32_t max_contacts_per_face; /* contact slots per surface face; 0 = 4        */
    int32_t use_graphs;        /* capture each substep in a CUDA graph (1) or not  */
    int32_t use_pdl;           /* programmatic dependent launch between kernels    */
    int32_t gs_patch_tets;     /* Gauss-Seidel patch size in tets (1..5); 0 = 5;   */
                               /* 1 = plain per-tet colouring                      */
    int32_t gs_min_blocks;     /* variant-1 occupancy target, blocks/SM: 6 or 8   */
                               /* (8 caps registers at 128); 0 = 6                 */
    int32_t gs_variant;        /* sweep kernel: 0 one lane per patch, tet records  */
                               /* prefetched into registers; 1 one lane, records   */
                               /* staged in shared memory by bulk (TMA) copies;    */
                               /* 2 dataflow: every iteration and colour in one    */
                               /* cooperative launch, warps ordered by per-task    */
                               /* dependency counters (combined constraints, no    */
                               /* faces, no per-iteration residual; else as 0);    */
                               /* 3 dataflow with records staged by bulk copies    */
                               /* (else as 1); 4 dataflow on version-stamped       */
                               /* vertices: a patch polls the versions of its own  */
                               /* vertices, no task counters or fences (else as 0);*/
                               /* default 4                                        */
    int32_t num_local_collision_iters; /* num-local-collision-iters: passes    */
                               /* after the global solve over every contact    */
                               /* and the tets touching a vertex of a contact  */
                               /* projected with lambda != 0; 0 = off          */
    int32_t first_order;       /* 1: FirstOrderXPBDMeshObject -- alpha~ = alpha/dt, */
                               /* vertex damping B as the constraint inertia,   */
                               /* x_z += -g m dt / B as the inertial move       */
    int32_t adjust_damping_to_material; /* adjust-damping-to-material          */
    double damping_multiplier; /* damping-multiplier: B = V_vertex * this       */
                               /* (* E_v / (1 + nu_v) when adjusted); default 1 */
    int32_t self_collisions;   /* self-collisions (XPBDMeshObjectConfig.hpp:66):  */
                               /* each detection tests every surface vertex for   */
                               /* a tet it is inside (selfCollisionCheck,        */
                               /* XPBDMeshObject.cpp:719-762) and adds a          */
                               /* DeformableDeformableCollisionConstraint with    */
                               /* the closest rest-surface face; needs faces     */
    int32_t gs_poll_ns;        /* versioned sweep (gs_variant 4): back-off in ns  */
                               /* between two polls of a vertex that is not yet   */
                               /* due; 0 = 128                                    */
    int32_t gs_topology_reload;/* versioned sweep: 1 reloads each task's patch    */
                               /* records from global memory every phase; 0 keeps */
                               /* a warp's task topology in shared memory when it */
                               /* fits (default)                                  */
    int32_t gs_l2_stream;      /* versioned sweep: L2 priority of what it streams */
                               /* once per sweep (tet records, multipliers, patch */
                               /* records): 0 = evict-first when these and the    */
                               /* vertex records exceed 3/4 of the L2, so that the*/
                               /* vertex records stay (default); 1 = always       */
                               /* evict-first; -1 = never                         */
} xpbd_params;

/* Fills p with the reference's defaults (XPBDMeshObjectConfig.hpp:117-125,
 * SimulationConfig.hpp:185-195): dt 1e-3, g 9.81, collision-rate 100 Hz,
 * 1 iteration, Gauss-Seidel, combined constraints, residual Never. */
int xpbd_default_params(xpbd_params* p);

int xpbd_abi_version(void);
const char* xpbd_status_string(int status);

/* Host-only utility (no GPU needed): greedy vertex-disjoint colouring in item
 * order, the order the coloured Gauss-Seidel uses. arity = 4 for tets, 3 for
 * faces. Returns the number of colours (> 0) or -XPBD_ERR_INVALID. */
int xpbd_colour_items(int64_t n_items, int32_t arity, const int32_t* items, int64_t n_vertices,
                      int32_t* colour_out);

/* Host-only utility (no GPU needed): hexahedral grid of nx x ny x nz hexes
 * with spacing (hx, hy, hz), five tets per hex, and its boundary triangles, as
 * MeshUtils::createBeamMsh builds them (src/utils/MeshUtils.cpp:424-660; x =
 * width, y = length, z = height). split = 0: the alternating split of the
 * current generator; split = 1: the uniform split of the revision that wrote
 * resource/cube/cube{2,4}.msh. X is 3 x V, tets 4 x T, faces 3 x F with the
 * counts from xpbd_grid_counts. */
int xpbd_grid_counts(int32_t nx, int32_t ny, int32_t nz, int64_t* nv, int64_t* nt, int64_t* nf);
int xpbd_grid_mesh(int32_t nx, int32_t ny, int32_t nz, double hx, double hy, double hz, int32_t split, double* X,
                   int32_t* tets, int32_t* faces);

/* Context lifetime: XPBDMeshObject_ ctor + setup() + XPBDSolver ctor/setup()
 * (XPBDMeshObject.cpp:60-160; XPBDSolver.hpp:47-61). Uploads the mesh, builds
 * rest shapes, masses, compliances and the colouring. */
int xpbd_create(const xpbd_mesh_desc* mesh, const xpbd_params* params, xpbd_ctx** out);
/* Batched instances: n independent objects (one XPBDMeshObject_ each, as a
 * Simulation holding many objects steps them, Simulation.cpp:246-255) advanced
 * together by the same kernel launches. Instance k's vertices, tets and faces
 * follow instance k-1's in the context's arrays (xpbd_instance_offsets); state
 * transfer, fixing and kinematic groups use these concatenated indices. */
int xpbd_create_batch(const xpbd_mesh_desc* meshes, int32_t n_instances, const xpbd_params* params,
                      xpbd_ctx** out);
int xpbd_num_instances(xpbd_ctx* ctx, int32_t* n);
/* offsets of each instance into the concatenated arrays, n + 1 entries each
 * (any pointer may be NULL) */
int xpbd_instance_offsets(xpbd_ctx* ctx, int64_t* vertex_offsets, int64_t* tet_offsets, int64_t* face_offsets);
/* Per-instance completion times of a batched substep (GPU-side measurement,
 * no reference counterpart). With stamps on, each xpbd_step / xpbd_update
 * substep records the device clock when it starts, when each task of the
 * persistent sweep (gs_variant 4) finishes its last iteration, and when the
 * substep's last kernel ends. xpbd_instance_latencies then gives, for the
 * last substep, ms[k] = start -> the end of instance k's last sweep task (its
 * final projections written; n_instances entries) and *batch_ms = start ->
 * end of the substep (after the batch-wide copy-out and velocity update).
 * XPBD_ERR_STATE without a persistent versioned sweep or before a stamped
 * substep; stamps cost one clock read and store per task and substep. */
int xpbd_set_latency_stamps(xpbd_ctx* ctx, int32_t on);
int xpbd_instance_latencies(xpbd_ctx* ctx, double* ms, double* batch_ms);
int xpbd_destroy(xpbd_ctx* ctx);
const char* xpbd_last_error(const xpbd_ctx* ctx);

/* Iteration count (XPBDSolver::_num_iter, XPBDSolver.hpp:139). */
int xpbd_set_num_iters(xpbd_ctx* ctx, int32_t num_iters);

/* State transfer between the host mesh (Mesh::vertices()) and the device. */
int xpbd_set_positions(xpbd_ctx* ctx, const double* x3v);
int xpbd_get_positions(xpbd_ctx* ctx, double* x3v);
int xpbd_get_prev_positions(xpbd_ctx* ctx, double* x3v);
int xpbd_set_velocities(xpbd_ctx* ctx, const double* v3v);
int xpbd_get_velocities(xpbd_ctx* ctx, double* v3v);
/* float32 xyz-interleaved variants (3*V floats) for callers that keep FP32 */
int xpbd_set_positions_f32(xpbd_ctx* ctx, const float* x3v);
int xpbd_get_positions_f32(xpbd_ctx* ctx, float* x3v);
/* lumped vertex masses (XPBDMeshObject.cpp:277-331) */
int xpbd_get_masses(xpbd_ctx* ctx, double* m);

/* XPBDMeshObject_Base_::fixVertex (include/simobject/XPBDMeshObjectBase.hpp:97-99):
 * mask[i] != 0 fixes vertex i (reset to its previous position after solve). */
int xpbd_set_fixed(xpbd_ctx* ctx, const uint8_t* mask);

/* Kinematic vertex group: fixed vertices driven to rest + offset, the pattern
 * of fixVertex + a cursor setPosition (src/simulation/GraspingSimulation.cpp:155,241).
 * set_group records the current positions of idx as their rest positions and
 * fixes them; set_offset moves them (stream-ordered, before the next step). */
int xpbd_set_kinematic_group(xpbd_ctx* ctx, int32_t n, const int32_t* idx);
int xpbd_set_kinematic_offset(xpbd_ctx* ctx, const double* offset3);

/* Rigid spheres (RigidSphere + SphereSDF, src/geometry/SphereSDF.cpp:16-26),
 * treated as fixed: detection emits static collision constraints. */
int xpbd_set_spheres(xpbd_ctx* ctx, int32_t n, const double* centers3n, const double* radii);
/* the same for one instance of a batch (xpbd_set_spheres addresses instance 0) */
int xpbd_set_instance_spheres(xpbd_ctx* ctx, int32_t instance, int32_t n, const double* centers3n,
                              const double* radii);
/* Fixed rigid primitives as SDFs: spheres, boxes and cylinders
 * (SphereSDF / BoxSDF / CylinderSDF, src/geometry/{Sphere,Box,Cylinder}SDF.cpp) at a position with
 * an orientation quaternion (x, y, z, w), as RigidSphere / RigidBox /
 * RigidCylinder hold them (RigidObject::globalToBody, RigidObject.cpp:94-97).
 * dims: sphere (radius, -, -), box (full size x, y, z), cylinder (radius,
 * height, -). Slot k of the contact table belongs to primitive k; at most
 * max_contacts_per_face primitives. The sphere setters above fill the same
 * table. */
#define XPBD_SDF_SPHERE 0
#define XPBD_SDF_BOX 1
#define XPBD_SDF_CYLINDER 2
int xpbd_set_sdfs(xpbd_ctx* ctx, int32_t n, const int32_t* kind, const double* pos3n, const double* quat4n,
                  const double* dims3n);
int xpbd_set_instance_sdfs(xpbd_ctx* ctx, int32_t instance, int32_t n, const int32_t* kind, const double* pos3n,
                           const double* quat4n, const double* dims3n);
/* Free rigid bodies: SDF slot `slot` of `instance` becomes a RigidObject
 * with fixed: false (src/simobject/RigidObject.cpp) -- mass, diagonal inertia
 * (RigidPrimitives.cpp formulas are the caller's), velocity and angular
 * velocity; the pose is the one last given to xpbd_set_instance_sdfs (double).
 * Detection then makes its contacts RigidDeformableCollisionConstraints
 * (CollisionScene.cpp:204-210), projected after the static contacts by
 * RigidBodyConstraintProjector (RigidBodyConstraintProjector.hpp:97-158): the
 * multiplier from the deformable weights alone, the body moved by
 * PositionalRigidBodyXPBDHelper::update (RigidBodyConstraint.hpp), all
 * contacts in slot order by one device thread (each moves the body the next
 * one reads). Each xpbd_step then runs RigidObject::update (gravity, the
 * Euler step of the angular velocity, normalised orientation) and
 * velocityUpdate after the deformable update. Setting SDFs for an instance
 * drops its free bodies. State: FP64 on the device. Needs surface faces. */
int xpbd_set_rigid_body(xpbd_ctx* ctx, int32_t instance, int32_t slot, double mass, const double* inertia3,
                        const double* velocity3, const double* angular_velocity3);
/* state13 = position[3], orientation (x, y, z, w)[4], velocity[3], angular velocity[3] */
int xpbd_get_rigid_body(xpbd_ctx* ctx, int32_t instance, int32_t slot, double* state13);
/* SDF value and gradient of one primitive at n points on the device
 * (out: n x (sdf, gx, gy, gz)); a test and tooling hook, no context needed */
int xpbd_sdf_eval(int32_t kind, const double* pos3, const double* quat4, const double* dims3, int64_t n,
                  const double* pts3n, double* out4n);

/* The self contacts of the last detection (no counterpart in the reference's
 * API; its constraint list holds them): rows of (surface vertex, face; face -1
 * when the tet it is in was degenerate) into vf2n, their multipliers into
 * lam (may be NULL); n_out = the count. */
int xpbd_get_self_contacts(xpbd_ctx* ctx, int32_t max_rows, int32_t* vf2n, double* lam, int32_t* n_out);

/* clearCollisionConstraints (XPBDMeshObject.cpp:233-251). */
int xpbd_clear_collisions(xpbd_ctx* ctx);
/* clear + CollisionScene::collideObjects against the spheres
 * (src/collision/CollisionScene.cpp:171-214, 253-283). */
int xpbd_detect_collisions(xpbd_ctx* ctx);
/* addStaticCollisionConstraint (XPBDMeshObject.cpp:180-206). */
int xpbd_add_static_collision(xpbd_ctx* ctx, int32_t face, double u, double v, double w, const double* p3,
                              const double* n3);
/* Active contacts, rows of 12 doubles: slot, face, u, v, w, p(3), n(3), lambda.
 * *n_out receives the count; at most max_rows rows are written. */
int xpbd_get_collisions(xpbd_ctx* ctx, int32_t max_rows, double* rows, int32_t* n_out);

/* Attachment constraints (AttachmentConstraint, include/solver/constraint/
 * AttachmentConstraint.hpp; XPBDMeshObject_::addAttachmentConstraint /
 * clearAttachmentConstraints, XPBDMeshObject.cpp:254-275): C = |x_v - (point +
 * offset)|, alpha = 0, projected after the contacts of every iteration (the
 * projector type order). The point can move between steps (a grasping tool);
 * the offset is fixed. Attachments do not enter the residual. The reference's
 * update writes 3 of its 4 coordinate slots and applies the fourth stale slot;
 * here only the vertex's 3 coordinates change. */
int xpbd_add_attachment(xpbd_ctx* ctx, int32_t vertex, const double* point3, const double* offset3, int32_t* id);
int xpbd_set_attachment_point(xpbd_ctx* ctx, int32_t id, const double* point3);
int xpbd_clear_attachments(xpbd_ctx* ctx);
int xpbd_num_attachments(xpbd_ctx* ctx, int32_t* n);

/* XPBDMeshObject_::update (XPBDMeshObject.cpp:426-505): prev <- x, inertial
 * move, solve (lambda <- 0, num_iters sweeps), fixed reset. Asynchronous. */
int xpbd_update(xpbd_ctx* ctx);
/* XPBDSolver::solve() (XPBDSolver.hpp:66-97) alone: every projector's lambda
 * <- 0, then num_iters sweeps over all constraints on the device positions as
 * they stand (set them with xpbd_set_positions after a host-side inertial
 * move). No inertial move, no local collision passes, no fixed-vertex reset:
 * XPBDMeshObject_::_projectConstraints (XPBDMeshObject.cpp:472-505) does those
 * around its solve() call. The residual is recorded as the policy asks.
 * Asynchronous. */
int xpbd_solve(xpbd_ctx* ctx);
/* XPBDSolver::solve(projector_references, num_iter, false) (XPBDSolver.hpp:106-125)
 * over the set XPBDMeshObject_::_gatherProjectorsForLocalCollisionIterations
 * builds (XPBDMeshObject.cpp:764-825): num_iter passes over the static contacts
 * and the elastic projectors of every tet touching a vertex of a contact with
 * lambda != 0, with no re-initialisation of the multipliers. Needs surface
 * faces and num_local_collision_iters > 0 at creation (XPBD_ERR_STATE
 * otherwise). Asynchronous. */
int xpbd_solve_local(xpbd_ctx* ctx, int32_t num_iter);
/* XPBDMeshObject_::velocityUpdate (XPBDMeshObject.cpp:507-535). */
int xpbd_velocity_update(xpbd_ctx* ctx);
/* Simulation::_timeStep for this object, n times (Simulation.cpp:197-276):
 * collision detection on the strict cadence test t - t_last > 1/rate,
 * update, velocity update, t += dt. Asynchronous. */
int xpbd_step(xpbd_ctx* ctx, int32_t nsteps);
/* waits for the context's stream; reports CUDA errors, device waits that
 * timed out (XPBD_ERR_TIMEOUT) and non-finite projections (XPBD_ERR_NUMERIC) */
int xpbd_synchronize(xpbd_ctx* ctx);
int xpbd_get_time(xpbd_ctx* ctx, double* t);

/* ||r||_2 of the elastic constraint residual r = C + alpha_tilde*lambda at the
 * current state (XPBDSolver::_calculateConstraintResidual, XPBDSolver.hpp:327-391),
 * and its ratio to ||r(x_pred, 0)|| of the last update. FP64 reduction. */
int xpbd_residual(xpbd_ctx* ctx, double* abs_norm, double* rel);
/* lastConstraintResidual(): 2T values in the reference's order (combined:
 * [dev_0, hyd_0, dev_1, ...]; separate: all dev, then all hyd). */
int xpbd_get_constraint_residual(xpbd_ctx* ctx, double* r, int64_t n);
/* Per-iteration ||r|| of the last update when residual_policy is
 * EVERY_ITERATION: num_iters + 1 exact state residuals (before each sweep,
 * after the last); EVERY_SUBSTEP: 2 values (||r(x_pred, 0)||, the final one).
 * Writes at most max_n values; *n_out = the number written. */
int xpbd_residual_history(xpbd_ctx* ctx, double* out, int32_t max_n, int32_t* n_out);
/* Lagrange multipliers, T x 2 (dev, hyd) in tet order. */
int xpbd_get_lambda(xpbd_ctx* ctx, double* lam);
/* totalStrainEnergy: sum of C^2/alpha over Dev and Hyd (XPBDMeshObject.cpp:537-549). */
int xpbd_total_strain_energy(xpbd_ctx* ctx, double* e);
/* Counters since the last call: projections with a non-finite update (skipped)
 * and projections that took the FP64 near-degenerate path (|det F| < 1e-3). */
int xpbd_health(xpbd_ctx* ctx, int64_t* nonfinite, int64_t* degenerate);

/* Test hook for the bounded waits of the versioned dataflow sweep (gs_variant
 * 4; no counterpart in the reference). vertex >= 0: every patch containing
 * that vertex waits for a version the sweep never writes (unreachable while
 * num_iters x (patches per vertex) < 255), and each wait gives up after
 * poll_limit polls; the next update then skips that work, xpbd_synchronize
 * returns XPBD_ERR_TIMEOUT and xpbd_health clears the count. vertex < 0 puts the
 * tables and the default limit back. XPBD_ERR_STATE without the versioned
 * sweep. Stalls no GPU: every wait is bounded and the kernel returns. */
int xpbd_debug_stall_vertex(xpbd_ctx* ctx, int32_t vertex, int32_t poll_limit);
/* Colouring in use (coloured Gauss-Seidel). Tets are grouped into patches
 * (runs of up to gs_patch_tets consecutive tets on at most 8 vertices) and the
 * patches are coloured so that patches of one colour share no vertex; each
 * colour is one kernel launch. n_tet_colours is the number of these sweep
 * colours, colour_of_tet the colour of each tet's patch; contacts follow the
 * surface-face colouring. */
int xpbd_num_colours(xpbd_ctx* ctx, int32_t* n_tet_colours, int32_t* n_face_colours);
int xpbd_get_tet_colours(xpbd_ctx* ctx, int32_t* colour_of_tet);
/* The order in which one Gauss-Seidel sweep projects the tets (T tet indices):
 * colour by colour, patch by patch, tets of a patch in index order. The FP64
 * oracle replays this order for parity. */
int xpbd_get_sweep_order(xpbd_ctx* ctx, int32_t* order);
/* The order of the Gauss-Seidel local collision passes: T tet indices, colour
 * by colour (a greedy per-tet colouring in tet index order), ascending tet
 * index within a colour; colour_offsets (n_colours + 1 entries, may be NULL)
 * delimit the colours. XPBD_ERR_STATE without faces or local passes. */
int xpbd_get_local_order(xpbd_ctx* ctx, int32_t* order, int32_t* colour_offsets, int32_t max_colours,
                         int32_t* n_colours);

/* Per-kernel timing with CUDA events on the context's stream over n substeps
 * (no graphs). Fills up to max_k entries: average milliseconds per launch and
 * launches, for kernel ids 0..max_k-1 (see xpbd_kernel_name). */
int xpbd_profile_steps(xpbd_ctx* ctx, int32_t nsteps, int32_t max_k, double* avg_ms, int64_t* launches);
const char* xpbd_kernel_name(int32_t id);
/* number of kernel launches issued by the library since creation */
int xpbd_launch_count(xpbd_ctx* ctx, int64_t* n);
/* Autotuner: builds trial contexts from the meshes, times trial_steps substeps
 * (CUDA events, graphs on) for each candidate launch configuration -- Gauss-
 * Seidel: patch size (tet colours folded into one launch) x sweep kernel
 * variant and occupancy x programmatic dependent launch; Jacobi: block size x
 * scatter/gather variant x programmatic
 * dependent launch -- and writes the fastest into *params. report (if
 * report_len > 0) receives a JSON list of the candidates and their ms/step. */
int xpbd_autotune(const xpbd_mesh_desc* meshes, int32_t n_instances, xpbd_params* params, int32_t trial_steps,
                  char* report, int32_t report_len);
/* the context's CUDA stream (a cudaStream_t), for callers that time or order
 * their own work against the solver's */
int xpbd_get_stream(xpbd_ctx* ctx, void** stream);

/* ---- Learned warm start (no counterpart in the reference) ----
 * A per-tet network, 14 -> 64 -> 64 -> 64 -> 2 with SiLU, maps features taken
 * right after position prediction -- F (9, column-major), alpha~_d lambda_d
 * and alpha~_h lambda_h of the previous substep, log10(E)/5, nu, 1e3 dt
 * (alpha~ = alpha / dt^2) -- to alpha~ lambda of this substep's solution. It
 * runs on the tensor cores (BF16 operands, FP32 accumulation) and trains online
 * with Adam on (features, solved multipliers) pairs recorded from the
 * solver's own substeps.
 * A warm start sets lambda_0 and moves the predicted positions by
 * M^-1 grad C(x_pred)^T lambda_0; when that leaves a larger constraint residual
 * than the plain start, ||r(x_warm, lambda_0)|| > ||r(x_pred, 0)||, the substep
 * falls back on the device to (x_pred, lambda = 0). With a residual policy
 * other than "never", record 0 of the history stays ||r(x_pred, 0)|| so
 * relative residuals compare with the plain solver's. */
#define XPBD_MLP_INPUTS 16    /* feature row: 14 features + 2 zero pads       */
#define XPBD_MLP_PARAMS 9538  /* W1 64x16, b1, W2 64x64, b2, W3 64x64, b3,   */
                              /* W4 2x64, b4; each W row-major (out x in)     */
#define XPBD_WARM_NONE 0      /* lambda_0 = 0 (the reference's start)         */
#define XPBD_WARM_PREVIOUS 1  /* lambda_0 = the previous substep's lambda     */
#define XPBD_WARM_MLP 2       /* lambda_0 = the network's prediction          */
/* He-normal initial parameters from seed; resets the Adam state */
int xpbd_mlp_init(xpbd_ctx* ctx, uint64_t seed);
int xpbd_mlp_set_params(xpbd_ctx* ctx, const float* params, int64_t n);  /* n = XPBD_MLP_PARAMS */
int xpbd_mlp_get_params(xpbd_ctx* ctx, float* params, int64_t n);
/* network output (n x 2) for host feature rows (n x XPBD_MLP_INPUTS, rounded
 * to BF16 on upload) */
int xpbd_mlp_forward(xpbd_ctx* ctx, const float* X, int64_t n, float* out);
/* mean squared error over n rows and its gradient (XPBD_MLP_PARAMS floats,
 * either output may be NULL); the gradient stays on the device for
 * xpbd_mlp_adam_step(ctx, NULL, lr) */
int xpbd_mlp_loss_grad(xpbd_ctx* ctx, const float* X, const float* Y, int64_t n, double* loss, float* grad);
/* one Adam step (beta 0.9 / 0.999, eps 1e-8) with grad, or with the device
 * gradient of the last loss evaluation when grad is NULL */
int xpbd_mlp_adam_step(xpbd_ctx* ctx, const float* grad, float lr);
/* on = 1: every substep keeps its features and solved alpha~ lambda (the
 * training pairs of the last substep) */
int xpbd_mlp_record(xpbd_ctx* ctx, int32_t on);
/* the recorded pairs in tet order: X (T x XPBD_MLP_INPUTS), Y (T x 2); either may be NULL */
int xpbd_mlp_get_samples(xpbd_ctx* ctx, float* X, float* Y);
/* epochs of minibatch Adam over the recorded pairs (batch rows per step);
 * *loss = mean squared error of the last epoch, taken before each step */
int xpbd_mlp_train(xpbd_ctx* ctx, int32_t epochs, int32_t batch, float lr, double* loss);
int xpbd_set_warm_start(xpbd_ctx* ctx, int32_t mode);
/* warm starts kept / rejected by the residual test since creation */
int xpbd_warm_start_stats(xpbd_ctx* ctx, int64_t* kept, int64_t* rejected);

/* ---- Residual without allocation (no counterpart in the reference) ----
 * ||r(x, lambda)||_2 at the current state, the abs_norm of xpbd_residual, for
 * callers that must not allocate device or pinned host memory: a real-time
 * control or haptics thread, where cudaMalloc / cudaFree may synchronise the
 * device and take unbounded time. xpbd_residual grows context buffers on
 * demand; this call instead uses a fixed 128 KiB scratch array inside the
 * library, one per device, and so handles at most 16384 x block tets
 * (4,194,304 at the default block of 256): larger meshes get
 * XPBD_ERR_CAPACITY. The first call on each device resolves the scratch's
 * address (cudaGetSymbolAddress) with that device current: make that first
 * call before any stream capture. All contexts on a device share the scratch,
 * so calls that overlap in time race: serialise them. */
int xpbd_residual_noalloc(xpbd_ctx* ctx, double* abs_norm);

#ifdef __cplusplus
}
#endif

#endif /* XPBD_GPU_H */
