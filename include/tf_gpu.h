/*
 * tf_gpu.h -- C ABI of the GB300 implicit prism time step.
 *
 * Drop-in for the reference's NewtonRaphsonSolver call sequence as driven by
 * Simulation::updateStepNR (TissueFolding/TissueFolding/SourceCode/
 * Simulation.cpp:6449-6590).  Every entry point returns a tf_status; none of
 * them exits or throws.  Plain pointers and sizes only: host arrays are
 * read/written in the reference's layouts (DOF index = 3*node + dim, prism
 * nodes 0-2 basal and 3-5 apical, row-major 3x3 tensors).
 *
 * Citations below are relative to TissueFolding/TissueFolding/SourceCode/.
 */
#ifndef TF_GPU_H
#define TF_GPU_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define TF_API __attribute__((visibility("default")))
#else
#define TF_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum tf_status {
    TF_OK = 0,
    TF_NOT_CONVERGED = 1,        /* Newton hit its iteration cap; the reference prints
                                    "did not converge" and carries on (Simulation.cpp:6568-6571) */
    TF_KRYLOV_NOT_CONVERGED = 2, /* linear solve stopped at its iteration cap */
    TF_KRYLOV_BREAKDOWN = 3,     /* a Krylov recurrence divided by zero / lost positivity */
    TF_NAN_DETECTED = 4,         /* non-finite residual or update (the reference only prints) */
    TF_BAD_INPUT = 5,            /* invalid argument, mesh or size */
    TF_CUDA_ERROR = 6,           /* a CUDA runtime call failed; see tf_last_error() */
    TF_NO_DEVICE = 7,            /* no usable GB300 device */
    TF_OUT_OF_MEMORY = 8
} tf_status;

typedef struct tf_handle tf_handle;

/* Mesh and node data, as the reference holds them in Simulation::Nodes /
 * Elements after initiateSystem (Simulation.cpp:546-715). */
typedef struct tf_mesh {
    int32_t n_nodes;
    int32_t n_elems;
    const double* node_pos;        /* [3*n_nodes] reference (initial) positions, Node::Position */
    const int32_t* conn;           /* [6*n_elems] prism node ids, ShapeBase::NodeIds */
    const uint8_t* fixed;          /* [3*n_nodes] Node::FixedPos */
    const double* ext_visc;        /* [3*n_nodes] Node::externalViscosity */
    const int32_t* node_placement; /* [n_nodes] Node::tissuePlacement (0 basal, 1 apical, 2 mid) */
    const double* ref_pos;         /* [18*n_elems] reference (stress-free) prism shapes, 6 x 3 per prism
                                      (ShapeBase::ReferenceShape->Positions as read from a mesh file,
                                      ShapeBase.cpp:935-944); NULL: the node positions */
} tf_mesh;

/* Per-element material, Prism::setElasticProperties (Prism.cpp:491-516) and
 * ShapeBase::setViscosity (ShapeBase.cpp:871-873). */
typedef struct tf_material {
    const double* E;   /* [n_elems] Young's modulus */
    const double* nu;  /* [n_elems] Poisson ratio (clamped to [0, 0.5] as the reference does) */
    const double* eta; /* [n_elems] internal viscosity */
} tf_material;

/* Solver controls.  Zero-initialised fields take the defaults shown. */
typedef struct tf_options {
    double newton_tol;    /* 1e-8: |du|_2 threshold, NewtonRaphsonSolver.cpp:17 */
    int32_t newton_max_iter; /* 20: Simulation.cpp:6451 (the loop allows max_iter+1 solves) */
    double krylov_rtol;   /* 1e-8: relative residual of each linear solve (keeps the Newton
                             iteration counts of an exact solve on the benchmark sheets) */
    int32_t krylov_max_iter; /* 20000 */
    int32_t krylov_method;   /* 0 auto (CG when every eta is 0, else BiCGStab), 1 CG, 2 BiCGStab */
    int32_t deterministic;   /* 1: order-fixed assembly (no atomics); 0: atomic scatter */
    int32_t device;          /* CUDA device ordinal */
    int32_t autotune_off;    /* 1: keep 16 prisms per CTA instead of timing 8/16/32 on the mesh */
    int32_t precond;         /* 0 auto (smoothed-aggregation multigrid from 20,000 nodes on,
                                else block-Jacobi), 1 block-Jacobi, 2 smoothed-aggregation
                                multigrid, 3 plain-aggregation multigrid (no reference
                                counterpart for 2 and 3); other values: TF_BAD_INPUT */
    double update_atol;      /* tf_newton_step / tf_batch_step only: absolute accuracy (um, 2-norm)
                                each Newton update needs.  A linear solve stops at the looser of
                                krylov_rtol and the relative residual that bounds the update's
                                error by update_atol (through the largest |du| / |g| seen so far,
                                relative residual at most 0.1); late Newton iterations, whose
                                update is orders of magnitude below newton_tol, then need a few
                                Krylov iterations instead of a full solve.  Such a solve never
                                decides the Newton test alone: when its |du| lies within
                                max(1e3 update_atol, 1e-3 newton_tol) of newton_tol the system is
                                solved again to krylov_rtol first.
                                0: newton_tol x 1e-4; negative: off (every solve to krylov_rtol).
                                tf_solve ignores it. */
    int32_t host_loops;      /* 1: the Krylov iterations run as host-checked CUDA-graph chunks and
                                every Newton iteration is host-driven, instead of the device-side
                                while loops (for profilers that cannot see kernels inside conditional
                                graph nodes); same results.  No reference counterpart. */
    int32_t multigrid_reuse_steps; /* multigrid only: the coarse levels (aggregates' prolongators,
                                Galerkin operators, smoother weights) built at a time step's first
                                solve are kept for up to k further time steps, the level-0 smoother
                                always using the current matrix; they are rebuilt at the next step
                                once a step's first solve needs more than 1.25 x (+2) the Krylov
                                iterations of the first solve after the last rebuild, and at once
                                when a solve with kept levels does not converge.  Changes Krylov
                                counts only (every solve meets the same tolerance).  tf_set_Fg and
                                tf_set_dof_bindings drop kept levels; tf_set_positions does not.
                                The adjoint (tf_adj_forward, tf_adj_backward) rebuilds at every
                                step.  0: the default, k = 4; negative: rebuilt at every time step.
                                No reference counterpart. */
} tf_options;

/* Statistics of one time step (tf_newton_step). */
typedef struct tf_step_stats {
    int32_t newton_iters;       /* number of linear solves performed */
    int32_t krylov_iters_total; /* summed over the step */
    int32_t krylov_iters_max;
    int32_t converged;          /* 1 if |du| <= tol before the cap */
    double dunorm[32];          /* |du|_2 of each Newton iteration (first 32) */
    double final_relres;        /* relative residual of the last linear solve */
    float ms_assemble;          /* device time spent in assembly (all iterations) */
    float ms_solve;             /* device time spent in linear solves */
    float ms_total;             /* device time of the whole step */
    int32_t device_iters;       /* Newton iterations run by the device-side loop (one graph launch for the
                                   iterations after the step's first; the rest ran host-driven) */
    int32_t device_handback;    /* why that loop handed an iteration back to the host: 0 it did not,
                                   1 a loosened solve's |du| near newton_tol, 3 a non-finite update,
                                   10 + the Krylov flag (11 converged is not used, 12 breakdown, 13 NaN,
                                   10 still running at the iteration cap) for a solve that did not converge */
} tf_step_stats;

TF_API const char* tf_status_string(tf_status s);
/* Message of the last failure on this thread (never NULL). */
TF_API const char* tf_last_error(void);

/* Replaces `new NewtonRaphsonSolver(3, nNodes)` (Simulation.cpp:689) plus the
 * per-element set-up of initiateSystem: reference shape-function derivatives
 * (Prism::calculateElementShapeFunctionDerivatives, Prism.cpp:705-728),
 * tissue placement and exposed surfaces (ShapeBase.cpp:705-770,
 * Prism.cpp:2674-2742).  Builds the block sparsity pattern and the
 * element-slot -> block map once.  `opts` may be NULL. */
TF_API tf_status tf_create(const tf_mesh* mesh, const tf_material* mat, const tf_options* opts, tf_handle** out);
/* Replaces `delete NRSolver` (Simulation.cpp:93). */
TF_API tf_status tf_destroy(tf_handle* h);

/* Node positions (Node::Position), host <-> device. */
TF_API tf_status tf_set_positions(tf_handle* h, const double* pos);
TF_API tf_status tf_get_positions(tf_handle* h, double* pos);
/* Growth tensors (ShapeBase::setFg, ShapeBase.cpp:858-868): Fg[9*n_elems]. */
TF_API tf_status tf_set_Fg(tf_handle* h, const double* Fg);
TF_API tf_status tf_get_Fg(tf_handle* h, double* Fg, double* invFg);
/* Per-element growth rates in 1/s, [3*n_elems] (x, y, z), applied at each
 * tf_begin_step as ShapeBase::calculateFgFromRates + growShapeByFg
 * (ShapeBase.cpp:396-421, :1215-1251).  NULL clears them. */
TF_API tf_status tf_set_growth_rates(tf_handle* h, const double* rates);

/* --- the NewtonRaphsonSolver call sequence ------------------------------ */

/* Start of a time step: growth update (per-element rates and the growth
 * functions active at the handle's time, see tf_add_uniform_growth), node
 * viscosity surfaces (Simulation::updateNodeViscositySurfaces :7563-7581),
 * packing detection when on, then
 * setMatricesToZeroAtTheBeginningOfIteration + constructUnMatrix +
 * initialteUkMatrix (NewtonRaphsonSolver.cpp:102-146). */
TF_API tf_status tf_begin_step(tf_handle* h, double dt);
/* One Newton assembly: calculateDisplacementMatrix, the element loop
 * calculateForcesAndJacobianMatrixNR, writeForcesTogeAndgvInternal,
 * writeImplicitElementalKToJacobian, calculateExternalViscousForcesForNR,
 * addImplicitKViscousExternalToJacobian, calculateSumOfInternalForces,
 * addExernalForces and calcutateFixedK (NewtonRaphsonSolver.cpp:148-378). */
TF_API tf_status tf_assemble(tf_handle* h);
/* Adds host forces to the right-hand side after tf_assemble, at DOFs that are
 * not fixed -- the gExt hook of addMyosinForces/addPackingForces
 * (Simulation.cpp:6506-6540). */
TF_API tf_status tf_add_external_forces(tf_handle* h, const double* gext);
/* Adds n entries to K after tf_assemble -- the hook of the writers that add
 * to NRSolver->K directly, e.g. Simulation::calculatePackingJacobian3D
 * (Simulation.cpp:7205-7290): K(rows[k], cols[k]) += vals[k], DOF indices.
 * Entries in a fixed DOF's row or column are dropped (calcutateFixedK runs
 * after these writers).  Node pairs outside the element pattern are kept as
 * extra blocks that the linear solve's products include (the multigrid
 * preconditioner does not); their positions persist, their values are
 * cleared by the next tf_assemble.  tf_export_csr includes them. */
TF_API tf_status tf_add_K_triplets(tf_handle* h, int64_t n, const int32_t* rows, const int32_t* cols,
                                   const double* vals);
/* Bound DOF couples, NRSolver->slaveMasterList (Simulation.cpp:505-513):
 * before each solve K_bound = N^T K N + I and g_bound = N^T g couple by couple
 * (calculateBoundKWithSlavesMasterDoF, NewtonRaphsonSolver.cpp:154-235), after
 * it du[slave] = du[master] (equateSlaveDisplacementsToMasters, :237-251).
 * DOF indices (3*node + dim); n = 0 removes them. */
TF_API tf_status tf_set_dof_bindings(tf_handle* h, int32_t n, const int32_t* slave_dofs, const int32_t* master_dofs);
/* Implicit packing between tissue surfaces (implicitPacking, Simulation.cpp:37).
 * enable = 1: every tf_begin_step detects the node couples at the step's start
 * shape on the device -- Simulation::detectPacingNodes (Simulation.cpp:8167-8440)
 * with the node masses of updateNodeMasses (:7552-7561), no fold-initiation
 * branch and no collapsed nodes -- and every tf_assemble adds their forces to g
 * and their Jacobian to K (calculatePackingForcesImplicit3D :7149-7203,
 * calculatePackingJacobian3D :7205-7300, addPackingForces :8869-8900).
 * flags bit 0 (TF_PACKING_REFERENCE_MERGE): leave out the couples found from
 * the last of 16 node segments, as the reference's merge loop does (:8426).
 * Single-mesh handles only; enable = 0 switches packing off. */
#define TF_PACKING_REFERENCE_MERGE 1
TF_API tf_status tf_set_packing(tf_handle* h, int32_t enable, int32_t flags);
/* Couples of the last detection (pacingNodeCouples0/1, initialWeightPoint):
 * their number in *n; node ids (2 per couple, first < second), weights (3 per
 * couple, the unit vector from the second node to the first at detection),
 * mean node masses, the force threshold (packingThreshold) and the detection
 * distance.  Array arguments may be NULL. */
TF_API tf_status tf_get_packing(tf_handle* h, int64_t* n, int32_t* nodes, double* weights, double* mbar,
                                double* threshold, double* detect_distance);
/* Node masses of the last detection (Node::mass), n_nodes values. */
TF_API tf_status tf_packing_masses(tf_handle* h, double* mass);

/* --- growth functions (GrowthFunctionBase types 1-3) --------------------- */
/* Growth functions of the reference (GrowthFunctionTypes.h), applied at every
 * tf_begin_step at simulation time t, in the order they were added, after the
 * per-element rates of tf_set_growth_rates: Simulation::calculateGrowth
 * (Simulation.cpp:9651-9666) -- each active function (init_time <= t <
 * end_time, both kept as float as GrowthFunctionBase does) multiplies the
 * growth increment of every prism whose initial relative z (0 apical,
 * 1 basal; assignInitialZPositions, Simulation.cpp:3367-3371) is within
 * [zmin, zmax] (ShapeBase::isGrowthRateApplicable, ShapeBase.cpp:277-300),
 * and Fg <- increment Fg (growShapeByFg, ShapeBase.cpp:1215-1251).  Rates in
 * 1/s (x, y, z).  Columnar prisms; single-mesh handles; at most 16 functions.
 * The initial relative z, the prism columns and the pinned grid positions come
 * from the mesh given to tf_create. */
/* Type 1, UniformGrowthFunction (GrowthFunctionTypes.h:14-100) applied by
 * calculateGrowthUniform (Simulation.cpp:9757-9799): R diag(exp(rate dt)) R^T,
 * R the rotation by angle_rad about z (ShapeBase::calculateFgFromRates,
 * ShapeBase.cpp:396-421). */
TF_API tf_status tf_add_uniform_growth(tf_handle* h, const double* rates, double angle_rad, double init_time,
                                       double end_time, double zmin, double zmax);
/* Type 2, RingGrowthFunction (GrowthFunctionTypes.h:150-264) applied by
 * calculateGrowthRing (Simulation.cpp:9801-9885): for prisms whose centre lies
 * at an xy distance d from (centre_x, centre_y) with r_in^2 < d^2 < r_out^2,
 * the uniform increment of rates x (1 - (d - r_in)/(r_out - r_in)); centre,
 * radii and d in single precision as the reference reads them. */
TF_API tf_status tf_add_ring_growth(tf_handle* h, double centre_x, double centre_y, double inner_radius,
                                    double outer_radius, const double* rates, double angle_rad, double init_time,
                                    double end_time, double zmin, double zmax);
/* Type 3, GridBasedGrowthFunction (GrowthFunctionTypes.h:266-609, read by
 * ModelInputObject::readGrowthOptions): an nx x ny grid of rates,
 * rates[3*(i*ny + j) + k] for grid point (i, j) and axis k, and xy angles in
 * degrees, angles_deg[i*ny + j] (NULL: all 0), over the tissue's bounding box;
 * Simulation::calculateGrowthGridBased (Simulation.cpp:10065-10114) with
 * ShapeBase::calculateFgFromGridCorners (ShapeBase.cpp:432-562), positions
 * from Simulation.cpp:5833-5843. */
TF_API tf_status tf_add_grid_growth(tf_handle* h, int32_t nx, int32_t ny, const double* rates,
                                    const double* angles_deg, double init_time, double end_time, double zmin,
                                    double zmax);
/* Removes every growth function (the per-element rates stay). */
TF_API tf_status tf_clear_growth_functions(tf_handle* h);
/* gridGrowthsInterpolationType (0 nearest grid point, 1 bilinear; default 1)
 * and GridGrowthsPinnedOnInitialMesh (default 0: the positions of each step's
 * start shape), Simulation.cpp:144-146. */
TF_API tf_status tf_set_grid_growth_mode(tf_handle* h, int32_t interpolation, int32_t pinned_on_initial_mesh);
/* Simulation::updatePinningPositions (Simulation.cpp:6018-6023): the current
 * shape's bounding-box positions become the pinned ones. */
TF_API tf_status tf_repin_grid_growth(tf_handle* h);
/* Per prism: initial relative z [n_elems], pinned positions [2*n_elems] and
 * the current shape's positions [2*n_elems] (x block, then y block) in the
 * bounding box, after the column rule of
 * Simulation::updateRelativePositionsToApicalPositioning (:5987-6003).
 * Any argument may be NULL. */
TF_API tf_status tf_grid_growth_positions(tf_handle* h, double* rel_z, double* rel_pinned, double* rel_current);
/* Simulation time in seconds (currSimTimeSec, starts at 0); tf_end_step
 * advances it by the step's dt (Simulation.cpp:5969). */
TF_API tf_status tf_set_time(tf_handle* h, double time_sec);
TF_API tf_status tf_get_time(tf_handle* h, double* time_sec);
/* solveForDeltaU (NewtonRaphsonSolver.cpp:382-404): solves K^T du = g, the
 * transposed system Pardiso is asked for (iparm[11] = 1, :639). */
TF_API tf_status tf_solve(tf_handle* h, int32_t* iters, double* relres);
/* checkConvergenceViaDeltaU + updateUkInIteration (:727-761). */
TF_API tf_status tf_update(tf_handle* h, int32_t* converged, double* dunorm);
/* updateNodePositionsNR at the end of the step (Simulation.cpp:6576). */
TF_API tf_status tf_end_step(tf_handle* h);
/* The whole of updateStepNR, device-resident: tf_begin_step, then
 * assemble / solve / update until |du| <= tol or the iteration cap, then
 * tf_end_step.  Returns TF_NOT_CONVERGED when the cap was hit (the state is
 * still advanced, as in the reference). */
TF_API tf_status tf_newton_step(tf_handle* h, double dt, tf_step_stats* stats);

/* --- batches of independent tissues ---------------------------------------
 * No counterpart in the reference (it simulates one tissue per process).
 * n_instances meshes are held by one handle as one block-diagonal system:
 * one element-kernel launch and one Krylov launch sequence cover every
 * instance (ragged node / element offsets), with separate Krylov scalars,
 * convergence flags and Newton iteration counts per instance; an instance
 * that has converged is masked out of later assemblies and solves.  All other
 * calls act on the concatenation (positions, Fg and rates of instance i
 * start at its node / element offset, see tf_get_instances). */
TF_API tf_status tf_batch_create(const tf_mesh* meshes, const tf_material* mats, int32_t n_instances,
                                 const tf_options* opts, tf_handle** out);
/* One implicit time step of every instance.  newton_iters and converged
 * ([n_instances], may be NULL) receive the per-instance counts.  Returns
 * TF_NOT_CONVERGED when any instance hit the iteration cap. */
TF_API tf_status tf_batch_step(tf_handle* h, double dt, int32_t* newton_iters, int32_t* converged,
                               tf_step_stats* stats);
/* Instance count and offsets ([n+1] each, may be NULL). */
TF_API tf_status tf_get_instances(tf_handle* h, int32_t* n_instances, int32_t* node_offsets, int32_t* elem_offsets);
/* Prisms per CTA of the element kernel chosen by the autotuner (8, 16, 32). */
TF_API int32_t tf_elements_per_cta(tf_handle* h);
/* The solve's kernel variants the autotuner chose by timing them on the
 * handle's own matrix before its first solve: block rows' slots in flight per
 * lane in the FP64 SpMV (1, 2, 4) and in the multigrid's level-0 smoother
 * (2, 4, 8; 0 without multigrid).  No reference counterpart. */
TF_API tf_status tf_solve_variants(tf_handle* h, int32_t* spmv_unroll, int32_t* smoother_unroll);

/* --- inspection (parity tests) ------------------------------------------ */

/* gSum after the last tf_assemble (fixed DOFs zero), [3*n_nodes]. */
TF_API tf_status tf_get_residual(tf_handle* h, double* g);
/* deltaU of the last tf_solve, [3*n_nodes]. */
TF_API tf_status tf_get_delta_u(tf_handle* h, double* du);
/* Node::viscositySurface after the last tf_begin_step, [n_nodes]. */
TF_API tf_status tf_get_viscosity_surfaces(tf_handle* h, double* area);
TF_API tf_status tf_set_viscosity_surfaces(tf_handle* h, const double* area);
/* Sets the Newton state directly: uk (current) and un (start of step). */
TF_API tf_status tf_set_state(tf_handle* h, const double* uk, const double* un, double dt);
/* The last assembled Jacobian exactly as the reference hands it to Pardiso
 * (constructiaForPardiso, NewtonRaphsonSolver.cpp:686-707): K (not
 * transposed), fixed rows/columns applied, entries with |v| <= drop_tol
 * removed, 0-based CSR.  With ia == NULL only *nnz is written. */
TF_API tf_status tf_export_csr(tf_handle* h, double drop_tol, int32_t* ia, int32_t* ja, double* a, int64_t* nnz);
/* Per-element 18x18 elastic and viscous tangents (TriPointKe/TriPointKv,
 * row-major, reference orientation) and 6x3 element forces
 * (ElementalElasticSystemForces / ElementalInternalViscousSystemForces) at
 * the current state, for elements [e0, e0+count).  Any output may be NULL. */
TF_API tf_status tf_element_eval(tf_handle* h, int32_t e0, int32_t count, double* Ke, double* Kv, double* fe, double* fv);
/* Sizes: nodes, elements, nonzero 3x3 blocks of the structural pattern. */
TF_API tf_status tf_get_sizes(tf_handle* h, int64_t* n_nodes, int64_t* n_elems, int64_t* n_blocks);
/* The CUDA stream all work of this handle runs on (a cudaStream_t). */
TF_API void* tf_get_stream(tf_handle* h);
/* Kernel launches issued by this handle since creation (all kernels). */
TF_API int64_t tf_launch_count(tf_handle* h);
/* Runs `iters` back-to-back assemblies at the current state and returns the
 * device time per assembly and per element-kernel launch (CUDA events on the
 * handle's stream). */
TF_API tf_status tf_time_assembly(tf_handle* h, int32_t iters, float* ms_per_assembly, float* ms_per_element_kernel);

/* HBM bandwidth of three access patterns on `device`, measured with kernels of
 * this library (no counterpart in the reference): a read stream of 16-byte
 * loads (eight in flight per thread), a read stream of 32 KB bulk (TMA)
 * copies into shared memory, and a copy (read + write bytes counted); best
 * of `reps` timed runs each, in GB/s.  `bytes` per buffer (a multiple of
 * 32 KB, at least 152 chunks); allocates two such buffers for the duration
 * of the call.  These are the denominators of the read-dominated solve
 * kernels' rooflines. */
TF_API tf_status tf_measure_bandwidth(int32_t device, int64_t bytes, int32_t reps, double* read_gbs, double* bulk_gbs,
                                      double* copy_gbs);

/* --- solve without device allocation --------------------------------------
 * No counterpart in the reference: this is an addition for callers that may
 * not call cudaMalloc (a host that owns every device allocation, a fixed
 * memory budget).
 * Solves A x = b for a caller-owned 3x3 block-sparse matrix on the current
 * device with block-Jacobi preconditioned BiCGStab in FP64; every pointer is
 * a device pointer the caller owns (rowptr[n+1], colidx[nnzb], val[9*nnzb]
 * row-major blocks, b and x [3n]).  Work space is one static device array of
 * this library (about 4.3 MB, held by every GPU that loads it until exit),
 * so n_block_rows is limited to 16384; larger systems return TF_BAD_INPUT.
 * The first call on a device (and the first after its context changes, e.g.
 * after cudaDeviceReset) looks the array up.  Every call synchronises
 * `stream` and reads scalars back, so it must never be made on a stream that
 * is being captured: it then returns TF_BAD_INPUT.  Calls share the array:
 * overlapping calls race, so serialise them.  `stream` is a cudaStream_t
 * (NULL: the default stream). */
TF_API tf_status tf_solve_bsr_static(int32_t n_block_rows, const int32_t* rowptr, const int32_t* colidx,
                                     const double* val, const double* b, double* x, double rtol, int32_t max_iter,
                                     void* stream, int32_t* iters, double* relres);

/* The reference's mesh input file (.mesh; Simulation.cpp:2074-2239): node
 * positions, tissue placement / type / circumference flags, prism node ids
 * (after Prism::checkRotationConsistency3D, Prism.cpp:364-410) and the 6 x 3
 * reference positions per prism.  Call with NULL arrays to get the sizes,
 * then again with arrays of those sizes.  Host only (no device work). */
TF_API tf_status tf_read_mesh_file(const char* path, int32_t* n_nodes, int32_t* n_elems, double* pos, int32_t* conn,
                                   int32_t* placement, int32_t* tissue_type, int32_t* at_circumference,
                                   double* ref_pos);
/* One save frame in the reference's format (Simulation::saveStep header,
 * writeNodes, writeElements, footer; Simulation.cpp:9265-9356), written to
 * `path` (appended when `append` != 0).  Host only. */
TF_API tf_status tf_write_frame(const char* path, int32_t append, double time_sec, int32_t n_nodes, const double* pos,
                                const int32_t* placement, const int32_t* tissue_type,
                                const int32_t* at_circumference, int32_t n_elems, const int32_t* conn,
                                const double* ref_pos);

/* Multigrid hierarchy of the handle (tf_options.precond): number of levels
 * (0 when block-Jacobi is used), nodes per level and the smoother weights
 * of the last numeric set-up (4 / (3 lambda_max(D^-1 A)) per level; arrays of
 * at least 10 entries, either may be NULL).  No reference counterpart. */
TF_API tf_status tf_multigrid_info(tf_handle* h, int32_t* levels, int32_t* nodes, double* weights);
/* Matrix blocks (3x3 at level 0, 6x6 below) and prolongator blocks to the
 * next level, per level of the hierarchy (arrays of at least 10 entries;
 * nothing is written when block-Jacobi is used).  No reference counterpart. */
TF_API tf_status tf_multigrid_blocks(tf_handle* h, int64_t* blocks, int64_t* prolongator_blocks);

/* ---- discrete adjoint (no counterpart in the reference) ------------------
 * Gradients of a shape loss after n implicit steps with respect to per-element
 * in-plane growth rates r_e (rates (r_e, r_e, 0), Fg starting at I) and log
 * Young's moduli.  loss_params = {cx, cy, amp, w}:
 *   L = sum over apical nodes (z - amp exp(-((x-cx)^2 + (y-cy)^2) / (2 w^2)))^2.
 * tf_adj_forward overwrites the handle's Fg, growth rates and elastic
 * moduli (E_e = exp(logE_e), Poisson ratios kept), runs n_steps Newton steps
 * of length dt from the current positions and keeps the state every `every`
 * steps in *saved.  tf_adj_backward recomputes each span of `every` steps
 * from its saved state and solves A^T lambda = rhs per step (to a relative
 * residual of min(krylov_rtol, 1e-12): the errors of these solves are carried
 * through the earlier steps), scaling dL by dloss; it leaves the handle at the
 * final state.  Single-mesh handles only. */
typedef struct tf_adjoint tf_adjoint;
TF_API tf_status tf_adj_forward(tf_handle* h, const double* rate, const double* logE, int32_t n_steps, double dt,
                                int32_t every, const double* loss_params, double* loss, tf_adjoint** saved);
TF_API tf_status tf_adj_backward(tf_handle* h, tf_adjoint* saved, double dloss, double* grad_rate,
                                 double* grad_logE);
TF_API tf_status tf_adj_free(tf_adjoint* saved);

#ifdef __cplusplus
}
#endif
#endif /* TF_GPU_H */
