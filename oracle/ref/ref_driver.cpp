// C API over the reference's own element and Newton-Raphson classes.
// TEST INFRASTRUCTURE ONLY: linked into oracle/_ref/libtfref.so together with
// the reference's unmodified translation units (ShapeBase.cpp, Prism.cpp,
// Node.cpp, ReferenceShapeBase.cpp, NewtonRaphsonSolver.cpp) and the
// project-written GSL/uBLAS/Pardiso stand-ins.  It replaces the parts of
// Simulation.cpp that the implicit step needs:
//   * mesh set-up (Simulation::initiateNodesFromMeshInput :2074-2095,
//     initiatePrismFromMeshInput :2222-2239, assignInitialZPositions :3367,
//     calculateShapeFunctionDerivatives :3381, assignPhysicalParameters
//     :4012-4131, assignElementalSurfaceAreaIndices :1231);
//   * the per-step growth (cleanUpGrowthRates :9688-9694, a uniform growth
//     function :9757-9800 with per-element rates, growShapeByFg
//     ShapeBase.cpp:1215-1251);
//   * updateNodeViscositySurfaces (Simulation.cpp:7563-7581);
//   * updateStepNR (Simulation.cpp:6449-6590), restated call for call with
//     packing, myosin, pipette and random forces switched off as in every
//     configuration this build targets.
#include <cmath>
#include <cstring>
#include <iostream>
#include <sstream>
#include <vector>

#include "NewtonRaphsonSolver.h"
#include "Node.h"
#include "Prism.h"

namespace {

class PrismRef : public Prism {
public:
    using Prism::Prism;
    gsl_matrix* ke() { return TriPointKe; }
    gsl_matrix* kv() { return TriPointKv; }
    gsl_matrix* elasticForces() { return ElementalElasticSystemForces; }
    gsl_matrix* viscousForces() { return ElementalInternalViscousSystemForces; }
    void exposeSurfaces(std::vector<Node*>& nodes) { assignExposedSurfaceAreaIndices(nodes); }
    double lambdaValue() const { return lambda; }
    double muValue() const { return mu; }
};

struct RefSim {
    std::vector<Node*> nodes;
    std::vector<ShapeBase*> elements;
    NewtonRaphsonSolver* nr = nullptr;
    double** systemForces = nullptr;
    double** fixedNodeForces = nullptr;
    std::vector<int> ablated;
    int nNodes = 0, nElems = 0;
};

struct QuietCout {
    std::stringstream sink;
    std::streambuf* old;
    QuietCout() : old(std::cout.rdbuf(sink.rdbuf())) {}
    ~QuietCout() { std::cout.rdbuf(old); }
};

void copyUkToPositions(RefSim* s) {
    // Simulation::updateElementPositionsinNR :6635-6649 and
    // updateNodePositionsNR :6625-6633.
    for (auto* e : s->elements) {
        int* ids = e->getNodeIds();
        for (int j = 0; j < 6; ++j)
            for (int d = 0; d < 3; ++d) e->Positions[j][d] = gsl_matrix_get(s->nr->uk, 3 * ids[j] + d, 0);
    }
    for (int i = 0; i < s->nNodes; ++i)
        for (int d = 0; d < 3; ++d) s->nodes[i]->Position[d] = gsl_matrix_get(s->nr->uk, 3 * i + d, 0);
}

}  // namespace

extern "C" {

void* tfr_create(int n_nodes, int n_elems, const double* pos, const int* conn,
                 const unsigned char* fixed, const double* ext_visc, const int* node_placement,
                 const double* E, const double* nu, const double* eta) {
    QuietCout q;
    RefSim* s = new RefSim;
    s->nNodes = n_nodes;
    s->nElems = n_elems;
    for (int i = 0; i < n_nodes; ++i) {
        double p[3] = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
        Node* nd = new Node(i, 3, p, node_placement[i], 0);
        for (int d = 0; d < 3; ++d) {
            nd->FixedPos[d] = fixed[3 * i + d] != 0;
            nd->externalViscosity[d] = ext_visc[3 * i + d];
            nd->initialExternalViscosity[d] = ext_visc[3 * i + d];
        }
        s->nodes.push_back(nd);
    }
    double zmin = 1e300, zmax = -1e300;
    for (int i = 0; i < n_nodes; ++i) {
        zmin = std::min(zmin, pos[3 * i + 2]);
        zmax = std::max(zmax, pos[3 * i + 2]);
    }
    for (int e = 0; e < n_elems; ++e) {
        int ids[6];
        for (int a = 0; a < 6; ++a) ids[a] = conn[6 * e + a];
        PrismRef* p = new PrismRef(ids, s->nodes, e, false);
        // Prism::~Prism deletes this array, which only the column-neighbour
        // set-up (Prism::setBasalNeigElementId) allocates.
        p->elementsIdsOnSameColumn = nullptr;
        p->checkRotationConsistency3D();
        p->setElasticProperties(E[e], E[e], E[e], E[e], nu[e]);
        p->setViscosity(eta[e]);
        s->elements.push_back(p);
    }
    for (auto* e : s->elements) {
        e->setInitialZPosition(zmin, zmax - zmin);
        e->calculateElementShapeFunctionDerivatives();
        static_cast<PrismRef*>(e)->exposeSurfaces(s->nodes);
    }
    s->nr = new NewtonRaphsonSolver(3, n_nodes);
    s->systemForces = new double*[n_nodes];
    s->fixedNodeForces = new double*[n_nodes];
    for (int i = 0; i < n_nodes; ++i) {
        s->systemForces[i] = new double[3]();
        s->fixedNodeForces[i] = new double[3]();
    }
    return s;
}

void tfr_destroy(void* h) {
    QuietCout q;
    RefSim* s = static_cast<RefSim*>(h);
    delete s->nr;
    for (int i = 0; i < s->nNodes; ++i) {
        delete[] s->systemForces[i];
        delete[] s->fixedNodeForces[i];
    }
    delete[] s->systemForces;
    delete[] s->fixedNodeForces;
    for (auto* e : s->elements) delete e;
    for (auto* n : s->nodes) delete n;
    delete s;
}

void tfr_get_conn(void* h, int* conn) {
    RefSim* s = static_cast<RefSim*>(h);
    for (int e = 0; e < s->nElems; ++e)
        for (int a = 0; a < 6; ++a) conn[6 * e + a] = s->elements[e]->getNodeIds()[a];
}

void tfr_get_lame(void* h, double* lam, double* mu) {
    RefSim* s = static_cast<RefSim*>(h);
    for (int e = 0; e < s->nElems; ++e) {
        lam[e] = static_cast<PrismRef*>(s->elements[e])->lambdaValue();
        mu[e] = static_cast<PrismRef*>(s->elements[e])->muValue();
    }
}

void tfr_get_placement(void* h, int* placement) {
    RefSim* s = static_cast<RefSim*>(h);
    for (int e = 0; e < s->nElems; ++e) placement[e] = s->elements[e]->tissuePlacement;
}

void tfr_set_Fg(void* h, const double* Fg) {
    QuietCout q;
    RefSim* s = static_cast<RefSim*>(h);
    gsl_matrix* m = gsl_matrix_alloc(3, 3);
    for (int e = 0; e < s->nElems; ++e) {
        for (int k = 0; k < 9; ++k) gsl_matrix_set(m, k / 3, k % 3, Fg[9 * e + k]);
        s->elements[e]->setFg(m);
    }
    gsl_matrix_free(m);
}

void tfr_get_Fg(void* h, double* Fg, double* invFg) {
    RefSim* s = static_cast<RefSim*>(h);
    for (int e = 0; e < s->nElems; ++e)
        for (int k = 0; k < 9; ++k) {
            if (Fg) Fg[9 * e + k] = gsl_matrix_get(s->elements[e]->getFg(), k / 3, k % 3);
            if (invFg) invFg[9 * e + k] = gsl_matrix_get(s->elements[e]->getInvFg(), k / 3, k % 3);
        }
}

void tfr_set_positions(void* h, const double* pos) {
    RefSim* s = static_cast<RefSim*>(h);
    for (int i = 0; i < s->nNodes; ++i)
        for (int d = 0; d < 3; ++d) s->nodes[i]->Position[d] = pos[3 * i + d];
    for (auto* e : s->elements) {
        int* ids = e->getNodeIds();
        for (int j = 0; j < 6; ++j)
            for (int d = 0; d < 3; ++d) e->Positions[j][d] = pos[3 * ids[j] + d];
    }
}

void tfr_get_positions(void* h, double* pos) {
    RefSim* s = static_cast<RefSim*>(h);
    for (int i = 0; i < s->nNodes; ++i)
        for (int d = 0; d < 3; ++d) pos[3 * i + d] = s->nodes[i]->Position[d];
}

// Per-element growth for one step from per-element rates (1/s), as a single
// uniform-type growth function applied with the identity rotation.
void tfr_grow(void* h, double dt, const double* rates) {
    QuietCout q;
    RefSim* s = static_cast<RefSim*>(h);
    gsl_matrix* rot = gsl_matrix_alloc(3, 3);
    gsl_matrix* inc = gsl_matrix_alloc(3, 3);
    gsl_matrix* peri = gsl_matrix_alloc(3, 3);
    gsl_matrix_set_identity(rot);
    for (int e = 0; e < s->nElems; ++e) {
        ShapeBase* el = s->elements[e];
        el->setGrowthRate(dt, 0.0, 0.0, 0.0);
        el->updateGrowthIncrementFromRate();
        gsl_matrix_set_identity(inc);
        gsl_matrix_set_identity(peri);
        el->calculateFgFromRates(dt, rates[3 * e], rates[3 * e + 1], rates[3 * e + 2], rot, inc, 0, 0.0, 1.0);
        el->updateGrowthIncrement(inc, peri);
        el->growShapeByFg();
    }
    gsl_matrix_free(rot);
    gsl_matrix_free(inc);
    gsl_matrix_free(peri);
}

void tfr_update_viscosity_surfaces(void* h, double* area_out) {
    RefSim* s = static_cast<RefSim*>(h);
    for (auto* e : s->elements)
        if (!e->IsAblated) e->calculateViscositySurfaces();
    for (auto* n : s->nodes) n->viscositySurface = 0;
    for (auto* e : s->elements)
        if (!e->IsAblated) e->assignViscositySurfaceAreaToNodes(s->nodes);
    if (area_out)
        for (int i = 0; i < s->nNodes; ++i) area_out[i] = s->nodes[i]->viscositySurface;
}

// Element quantities at state (uk, un): 18x18 Ke and Kv (row-major, as the
// reference stores TriPointKe / TriPointKv) and the 6x3 element elastic and
// internal viscous forces (ElementalElasticSystemForces, ...).
void tfr_element_eval(void* h, const double* uk, const double* un, double dt,
                      double* Ke, double* Kv, double* fe, double* fv) {
    QuietCout q;
    RefSim* s = static_cast<RefSim*>(h);
    NewtonRaphsonSolver* nr = s->nr;
    for (int i = 0; i < 3 * s->nNodes; ++i) {
        gsl_matrix_set(nr->uk, i, 0, uk[i]);
        gsl_matrix_set(nr->un, i, 0, un[i]);
    }
    copyUkToPositions(s);
    nr->calculateDisplacementMatrix(dt);
    nr->calculateForcesAndJacobianMatrixNR(s->nodes, s->elements, dt, false, s->fixedNodeForces);
    for (int e = 0; e < s->nElems; ++e) {
        PrismRef* p = static_cast<PrismRef*>(s->elements[e]);
        for (int r = 0; r < 18; ++r)
            for (int c = 0; c < 18; ++c) {
                if (Ke) Ke[324L * e + 18 * r + c] = gsl_matrix_get(p->ke(), r, c);
                if (Kv) Kv[324L * e + 18 * r + c] = gsl_matrix_get(p->kv(), r, c);
            }
        for (int a = 0; a < 6; ++a)
            for (int d = 0; d < 3; ++d) {
                if (fe) fe[18L * e + 3 * a + d] = gsl_matrix_get(p->elasticForces(), a, d);
                if (fv) fv[18L * e + 3 * a + d] = gsl_matrix_get(p->viscousForces(), a, d);
            }
    }
}

// One assembly of the Newton system at (uk, un): everything updateStepNR does
// before solveForDeltaU.  Returns the number of entries of the reference's
// value-filtered CSR (constructiaForPardiso, |K| > 1e-13).
long tfr_assemble(void* h, const double* uk, const double* un, double dt) {
    QuietCout q;
    RefSim* s = static_cast<RefSim*>(h);
    NewtonRaphsonSolver* nr = s->nr;
    nr->setMatricesToZeroAtTheBeginningOfIteration(false);
    for (int i = 0; i < 3 * s->nNodes; ++i) {
        gsl_matrix_set(nr->uk, i, 0, uk[i]);
        gsl_matrix_set(nr->un, i, 0, un[i]);
    }
    copyUkToPositions(s);
    for (int i = 0; i < s->nNodes; ++i)
        for (int d = 0; d < 3; ++d) s->systemForces[i][d] = 0.0;
    nr->setMatricesToZeroInsideIteration();
    nr->calculateDisplacementMatrix(dt);
    nr->calculateForcesAndJacobianMatrixNR(s->nodes, s->elements, dt, false, s->fixedNodeForces);
    nr->writeForcesTogeAndgvInternal(s->nodes, s->elements, s->systemForces);
    nr->writeImplicitElementalKToJacobian(s->elements);
    nr->calculateExternalViscousForcesForNR(s->nodes);
    nr->addImplicitKViscousExternalToJacobian(s->nodes, dt);
    nr->checkJacobianForAblatedNodes(s->ablated);
    nr->calculateSumOfInternalForces();
    nr->addExernalForces();
    nr->calcutateFixedK(s->nodes);
    nr->calculateBoundKWithSlavesMasterDoF();
    long n = 0;
    const int N3 = 3 * s->nNodes;
    for (int i = 0; i < N3; ++i)
        for (int j = 0; j < N3; ++j) {
            double v = gsl_matrix_get(nr->K, i, j);
            if (v > 1E-13 || v < -1E-13) ++n;
        }
    return n;
}

// The reference's CSR of the last assembly (constructiaForPardiso :686-707)
// and its right-hand side gSum.
void tfr_get_system(void* h, int* ia, int* ja, double* a, double* g) {
    RefSim* s = static_cast<RefSim*>(h);
    NewtonRaphsonSolver* nr = s->nr;
    const int N3 = 3 * s->nNodes;
    std::vector<int> jv;
    std::vector<double> av;
    nr->constructiaForPardiso(ia, N3, jv, av);
    for (size_t p = 0; p < jv.size(); ++p) {
        ja[p] = jv[p];
        a[p] = av[p];
    }
    for (int i = 0; i < N3; ++i) g[i] = gsl_vector_get(nr->gSum, i);
}

// One time step: growth, viscosity surfaces, then updateStepNR restated.
// Writes the number of Newton solves and the |du| of each into iters / dunorm
// (capacity max_hist).  Returns 1 when the reference's non-convergence branch
// was taken, else 0.
// NRSolver->slaveMasterList and boundNodesWithSlaveMasterDefinition as
// Simulation::initiateSystem sets them for bound nodes (Simulation.cpp:505-513).
void tfr_set_bindings(void* h, int n, const int* slave_dofs, const int* master_dofs) {
    RefSim* s = static_cast<RefSim*>(h);
    s->nr->slaveMasterList.clear();
    for (int k = 0; k < n; ++k) s->nr->slaveMasterList.push_back({slave_dofs[k], master_dofs[k]});
    s->nr->boundNodesWithSlaveMasterDefinition = n > 0;
}

int tfr_step(void* h, double dt, const double* rates, int* iters, double* dunorm, int max_hist) {
    RefSim* s = static_cast<RefSim*>(h);
    if (rates) tfr_grow(h, dt, rates);
    tfr_update_viscosity_surfaces(h, nullptr);
    QuietCout q;
    std::ostringstream err;
    std::streambuf* oldErr = std::cerr.rdbuf(err.rdbuf());
    NewtonRaphsonSolver* nr = s->nr;
    int iteratorK = 0;
    const int maxIteration = 20;
    bool converged = false;
    int notConverged = 0;
    nr->setMatricesToZeroAtTheBeginningOfIteration(false);
    nr->constructUnMatrix(s->nodes);
    nr->initialteUkMatrix();
    while (!converged) {
        for (int i = 0; i < s->nNodes; ++i)
            for (int d = 0; d < 3; ++d) s->systemForces[i][d] = 0.0;
        nr->setMatricesToZeroInsideIteration();
        nr->calculateDisplacementMatrix(dt);
        nr->calculateForcesAndJacobianMatrixNR(s->nodes, s->elements, dt, false, s->fixedNodeForces);
        nr->writeForcesTogeAndgvInternal(s->nodes, s->elements, s->systemForces);
        nr->writeImplicitElementalKToJacobian(s->elements);
        nr->calculateExternalViscousForcesForNR(s->nodes);
        nr->addImplicitKViscousExternalToJacobian(s->nodes, dt);
        nr->checkJacobianForAblatedNodes(s->ablated);
        nr->calculateSumOfInternalForces();
        nr->addExernalForces();
        nr->calcutateFixedK(s->nodes);
        nr->calculateBoundKWithSlavesMasterDoF();
        nr->solveForDeltaU();
        if (iteratorK < max_hist) dunorm[iteratorK] = gsl_blas_dnrm2(nr->deltaU);
        converged = nr->checkConvergenceViaDeltaU();
        nr->updateUkInIteration();
        copyUkToPositions(s);
        iteratorK++;
        if (!converged && iteratorK > maxIteration) {
            notConverged = 1;
            converged = true;
        }
    }
    copyUkToPositions(s);
    std::cerr.rdbuf(oldErr);
    *iters = iteratorK;
    return notConverged;
}

}  // extern "C"
