/*
 * tf_oracle: CPU restatement, in plain C, of the reference's implicit prism
 * time step.  TEST INFRASTRUCTURE ONLY.  It is the test oracle for the
 * CUDA path (tests, __graft_entry__.smoke) and the timed CPU baseline of
 * bench.py; the product never links, loads or calls it.  Each routine follows
 * the reference function named beside it, in the reference's operation order
 * (paths relative to TissueFolding/TissueFolding/SourceCode/):
 *
 *   Prism.cpp:102-150, :655-703, :705-728   Gauss points, dN, dX/dxi per GP
 *   Prism.cpp:749-874                        per-GP forces (calculateCurrNodalForces)
 *   ShapeBase.cpp:2184-2235                  Gauss sum of element forces
 *   ShapeBase.cpp:2284-2341                  neo-Hookean S, D81, Cauchy stress
 *   ShapeBase.cpp:2619-2705, :2786-3053     elastic / viscous 18x18 tangents
 *   ShapeBase.cpp:2148-2180, :2707-2758     scatter into g and K
 *   NewtonRaphsonSolver.cpp:237-378          BCs, external viscosity, sums
 *   NewtonRaphsonSolver.cpp:686-707          value-filtered CSR (|K| > 1e-13)
 *   NewtonRaphsonSolver.cpp:418-683          transposed solve (banded-LU stand-in)
 *   Simulation.cpp:6449-6590                 the Newton loop (updateStepNR)
 *   Simulation.cpp:7563-7581, Prism.cpp:2424-2503  viscosity surfaces
 *   ShapeBase.cpp:396-421, :1215-1251        growth increment, Fg update
 *
 * Parity of this restatement is pinned against the reference's own sources
 * compiled in oracle/_ref (see tests/golden/make_golden.py).
 */
#ifndef TF_ORACLE_H
#define TF_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct tfo_model tfo_model;

/* Element-tangent evaluation modes. */
#define TFO_LITERAL 0 /* the reference's 3^6 contraction with D81 (ShapeBase.cpp:2786-2856) */
#define TFO_CLOSED 1  /* the push-forward identity Fe C^-1 Fe^T = I, same maths, fewer flops */

tfo_model* tfo_create(int n_nodes, int n_elems, const double* pos0, const int* conn,
                      const unsigned char* fixed, const double* ext_visc, const int* node_placement,
                      const double* E, const double* nu, const double* eta);
void tfo_destroy(tfo_model* m);
/* Reference (stress-free) prism shapes different from the node positions the
 * model was created with: ref_pos[18*n_elems], 6 x 3 per prism. */
void tfo_set_reference_shapes(tfo_model* m, const double* ref_pos);
void tfo_set_threads(int n);
int tfo_get_threads(void);

void tfo_set_Fg(tfo_model* m, const double* Fg);
void tfo_get_Fg(const tfo_model* m, double* Fg, double* invFg);
void tfo_set_positions(tfo_model* m, const double* pos);
void tfo_get_positions(const tfo_model* m, double* pos);
void tfo_get_lame(const tfo_model* m, double* lam, double* mu);
void tfo_get_placement(const tfo_model* m, int* placement);
void tfo_get_ref_geometry(const tfo_model* m, double* detdXde, double* invdXde);

void tfo_grow(tfo_model* m, double dt, const double* rates);
void tfo_update_viscosity_surfaces(tfo_model* m, double* area_out);
void tfo_set_viscosity_surfaces(tfo_model* m, const double* area);

/* Per-element 18x18 Ke, Kv (row-major) and 6x3 element forces for elements
 * [e0, e0+count) at state (uk, un). Any output may be NULL. */
void tfo_element_eval(tfo_model* m, const double* uk, const double* un, double dt, int mode,
                      int e0, int count, double* Ke, double* Kv, double* fe, double* fv);

/* Full assembly at (uk, un) into the structural CSR of the reference's K
 * (rows = DOF 3*node+dim) and the right-hand side gSum, in the reference's
 * summation order.  Returns the number of structural entries. */
long tfo_assemble(tfo_model* m, const double* uk, const double* un, double dt, int mode);
long tfo_structure_nnz(const tfo_model* m);
/* Element loop over the first `count` prisms plus their serial scatter: a
 * bounded sample of one K+f assembly, used to time the CPU baseline. */
long tfo_assemble_sample(tfo_model* m, const double* uk, const double* un, double dt, int mode, int count);
void tfo_get_structure(const tfo_model* m, int* ia, int* ja);
void tfo_get_values(const tfo_model* m, double* a, double* g);
/* The reference's value-filtered CSR of the last assembly (fixed rows and
 * columns applied, |v| <= drop removed).  With ia == NULL only counts. */
long tfo_export_filtered(const tfo_model* m, double drop, int* ia, int* ja, double* a);
/* Residual g only (no tangent), for size-independent checks on big meshes. */
void tfo_residual(tfo_model* m, const double* uk, const double* un, double dt, double* g);

/* Solve K^T du = g for the last assembly (banded LU stand-in for Pardiso). */
int tfo_solve(tfo_model* m, double* du);

/* One time step (growth, viscosity surfaces, Newton loop).  Returns 1 when
 * the Newton loop hit its iteration cap, 0 when it converged, <0 on error. */
int tfo_step(tfo_model* m, double dt, const double* rates, int mode, int* iters,
             double* dunorm_hist, int max_hist);

#ifdef __cplusplus
}
#endif
#endif
