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
//     myosin, pipette and random forces switched off as in every
//     benchmark configuration;
//   * implicit packing between tissue surfaces when switched on
//     (tfr_set_packing): calculateBoundingBox :9148-9185 and the elements'
//     bounding-box positions :5833-5843, updateNodeMasses :7552-7561,
//     getAverageSideLength :3205-3265, detectPacingNodes :8167-8440 (without
//     the fold-initiation branch, which needs emergent-ellipse marking or
//     peripodial adhesion, and with no collapsed nodes),
//     calculatePackingForcesImplicit3D :7149-7203,
//     calculatePackingJacobian3D :7205-7300 and addPackingForces :8869-8900,
//     in the order runOneStep / updateStepNR call them;
//   * growth functions (tfr_add_*_growth): the reference's own
//     UniformGrowthFunction, RingGrowthFunction and GridBasedGrowthFunction
//     (GrowthFunctionTypes.h) applied as calculateGrowth does
//     (Simulation.cpp:9651-9666): calculateGrowthUniform :9757-9799,
//     calculateGrowthRing :9801-9885 and calculateGrowthGridBased
//     :10065-10114 (ShapeBase::calculateFgFromRates /
//     calculateFgFromGridCorners), the growth turned with each prism's
//     rotation (updateGrowthRotationMatrices :4459-4466), with calculateTissueHeight
//     :3280-3330, assignInitialZPositions :3367-3371, fillInElementColumnLists
//     :7612-7624, the bounding-box positions of initiateSystem :630-645 and of
//     runOneStep :5833-5843, and updateRelativePositionsToApicalPositioning
//     :5987-6003.
//   The reference's tissue alignment (alignTissueDVToXPositive), a rigid
//   rotation outside the step, is not applied.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <fstream>  // GrowthFunctionTypes.h writes summaries to std::ofstream without including it
#include <iostream>
#include <sstream>
#include <vector>

#include "GrowthFunctionTypes.h"
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
    double relZ() const { return initialRelativePositionInZ; }
};

// Growth functions and the simulation time (Simulation's GrowthFunctions,
// gridGrowthsInterpolationType,
// GridGrowthsPinnedOnInitialMesh, TissueHeight(DiscretisationLayers),
// currSimTimeSec).
struct GridRef {
    std::vector<GrowthFunctionBase*> fns;
    int interp = 1;
    bool pinned = false;
    bool setUp = false;
    int layers = 0;
    double height = 0.0;
    double time = 0.0;
};

// State of the packing restatement (Simulation's packing members).
struct PackingRef {
    bool on = false;
    bool dropLastSegment = true;   // the reference's merge loop (Simulation.cpp:8426) skips the last segment
    double bb[2][3] = {{0, 0, 0}, {0, 0, 0}};
    double bbSize[3] = {0, 0, 0};
    double threshold = 0.0;        // packingThreshold
    double detect = 0.0;           // detection distance of a master node in grid cell [0][0]
    double multiplier = 5000.0;    // packingMultiplier
    double saturation = 5.0;       // sigmoidSaturationForPacking
    std::vector<int> c0, c1;       // pacingNodeCouples0 / 1
    std::vector<double> wx, wy, wz;  // initialWeightPointx / y / z
    std::vector<double> force;     // PackingForces, 3 per node
};

struct RefSim {
    PackingRef pk;
    GridRef grid;
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

// Simulation::calculateBoundingBox (Simulation.cpp:9148-9185): every node
// counts (no ECM-mimicking elements), no y symmetry; note the running
// "else if": a node that lowers the minimum is not tested for the maximum.
void refBoundingBox(RefSim* s) {
    PackingRef& p = s->pk;
    for (int i = 0; i < 3; ++i) {
        p.bb[0][i] = 100000.0;
        p.bb[1][i] = -100000.0;
    }
    for (Node* n : s->nodes)
        for (int i = 0; i < 3; ++i) {
            if (n->Position[i] < p.bb[0][i]) p.bb[0][i] = n->Position[i];
            else if (n->Position[i] > p.bb[1][i]) p.bb[1][i] = n->Position[i];
        }
    for (int i = 0; i < 3; ++i) p.bbSize[i] = p.bb[1][i] - p.bb[0][i];
    for (ShapeBase* e : s->elements)
        e->calculateRelativePosInBoundingBox(p.bb[0][0], p.bb[0][1], p.bbSize[0], p.bbSize[1]);
}

// Simulation::updateNodeMasses (Simulation.cpp:7552-7561)
void refNodeMasses(RefSim* s) {
    for (Node* n : s->nodes) n->mass = 0;
    for (ShapeBase* e : s->elements)
        if (!e->IsAblated) e->assignVolumesToNodes(s->nodes);
}

// Simulation::getAverageSideLength (Simulation.cpp:3205-3265) for a tissue of
// columnar elements only: returns colAverageSideLength and fills the 10 x 5
// detection grid.  (The reference declares its counter grid [10][4] while
// indexing it [10][5]; both grids are 10 x 5 here.)
double refAverageSideLength(RefSim* s, double grid[10][5]) {
    double cnt[10][5];
    for (int i = 0; i < 10; ++i)
        for (int j = 0; j < 5; ++j) grid[i][j] = cnt[i][j] = 0.0;
    double dsum = 0.0;
    int n = 0;
    for (ShapeBase* e : s->elements) {
        if (e->IsAblated || e->tissueType != 0) continue;
        double v = e->getApicalSideLengthAverage();
        if (v > 0) {
            dsum += v;
            n++;
        }
        if (e->tissuePlacement == 0 || e->spansWholeTissue) {
            v = e->getBasalSideLengthAverage();
            if (v > 0) {
                dsum += v;
                n++;
            }
        }
        double rel[2];
        e->getRelativePosInBoundingBox(rel);
        int rx = static_cast<int>(std::floor(rel[0])), ry = static_cast<int>(std::floor(rel[1] / 2.0));
        rx = std::min(std::max(rx, 0), 9);
        ry = std::min(std::max(ry, 0), 4);
        grid[rx][ry] += v;
        cnt[rx][ry] += 1.0;
    }
    for (int i = 0; i < 10; ++i)
        for (int j = 0; j < 5; ++j)
            if (cnt[i][j] > 0) grid[i][j] /= cnt[i][j];
    return dsum / static_cast<double>(n);
}

// Simulation::detectPacingNodes (Simulation.cpp:8167-8440) without the
// fold-initiation branch and with no collapsed nodes.
void refDetectPacking(RefSim* s) {
    PackingRef& p = s->pk;
    double grid[10][5], gridSq[10][5];
    const double col = refAverageSideLength(s, grid);
    for (int i = 0; i < 10; ++i)
        for (int j = 0; j < 5; ++j) {
            grid[i][j] = 0.4 * grid[i][j];
            gridSq[i][j] = grid[i][j] * grid[i][j];
        }
    p.threshold = 0.4 * col;
    p.detect = grid[0][0];
    p.c0.clear();
    p.c1.clear();
    p.wx.clear();
    p.wy.clear();
    p.wz.clear();
    const int nNodes = s->nNodes;
    int segSize = nNodes / 16;
    if (segSize < 1) segSize = 1;
    const int nSeg = nNodes / segSize;
    const int lastStart = (nSeg - 1) * segSize;
    for (int a = 0; a < nNodes; ++a) {
        Node* m = s->nodes[a];
        if (!m->checkIfNodeHasPacking()) continue;
        if (p.dropLastSegment && a >= lastStart) continue;  // found, then dropped by the merge loop
        const int gx = static_cast<int>(std::floor((m->Position[0] - p.bb[0][0]) / p.bbSize[0]));
        const int gy = static_cast<int>(std::floor((m->Position[1] - p.bb[0][1]) / p.bbSize[1]));
        // the reference indexes its 10 x 5 grid unchecked; no node lies outside it here
        const double t2 = (gx >= 0 && gx < 10 && gy >= 0 && gy < 5) ? gridSq[gx][gy] : 0.0;
        for (int b = a + 1; b < nNodes; ++b) {
            Node* sl = s->nodes[b];
            if (!sl->checkIfNodeHasPacking()) continue;
            if (m->tissuePlacement != sl->tissuePlacement) continue;
            if (m->isMyNeig(sl->Id)) continue;
            const double dx = m->Position[0] - sl->Position[0];
            const double dy = m->Position[1] - sl->Position[1];
            const double dz = m->Position[2] - sl->Position[2];
            const double d2 = dx * dx + dy * dy + dz * dz;
            if (d2 < t2) {
                const double d = std::pow(d2, 0.5);
                p.c0.push_back(m->Id);
                p.c1.push_back(sl->Id);
                p.wx.push_back(dx / d);
                p.wy.push_back(dy / d);
                p.wz.push_back(dz / d);
            }
        }
    }
}

// calculatePackingForcesImplicit3D (Simulation.cpp:7149-7203) after the
// iteration's resetForces(true) (:6466), then calculatePackingJacobian3D
// (:7205-7300) into K.
void refPackingForcesAndJacobian(RefSim* s) {
    PackingRef& p = s->pk;
    std::fill(p.force.begin(), p.force.end(), 0.0);
    const size_t n = p.c0.size();
    for (size_t i = 0; i < n; ++i) {
        const int a = p.c0[i], b = p.c1[i];
        const double mbar = 0.5 * (s->nodes[a]->mass + s->nodes[b]->mass);
        const double w[3] = {p.wx[i], p.wy[i], p.wz[i]};
        for (int d = 0; d < 3; ++d) {
            double dd = s->nodes[a]->Position[d] - s->nodes[b]->Position[d];
            if (w[d] > 0) dd *= -1.0;
            double F = p.multiplier * mbar / (1 + std::exp(p.saturation / p.threshold * (-1.0 * dd)));
            F *= w[d];
            p.force[3 * a + d] += F;
            p.force[3 * b + d] -= F;
        }
    }
    gsl_matrix* K = s->nr->K;
    for (size_t i = 0; i < n; ++i) {
        const int a = p.c0[i], b = p.c1[i];
        const double mbar = 0.5 * (s->nodes[a]->mass + s->nodes[b]->mass);
        const double w[3] = {p.wx[i], p.wy[i], p.wz[i]};
        for (int d = 0; d < 3; ++d) {
            double dd = s->nodes[a]->Position[d] - s->nodes[b]->Position[d];
            if (w[d] > 0) dd *= -1.0;
            const double sig = 1 / (1 + std::exp(p.saturation / p.threshold * (-1.0 * dd)));
            double d0 = sig * (1 - sig) * p.multiplier * mbar * w[d] * (p.saturation / p.threshold);
            double d1 = -1.0 * d0;
            if (w[d] > 0) {
                d0 *= -1.0;
                d1 *= -1.0;
            }
            const int ra = 3 * a + d, rb = 3 * b + d;
            gsl_matrix_set(K, ra, ra, gsl_matrix_get(K, ra, ra) - d0);
            gsl_matrix_set(K, ra, rb, gsl_matrix_get(K, ra, rb) - d1);
            gsl_matrix_set(K, rb, rb, gsl_matrix_get(K, rb, rb) - d0);
            gsl_matrix_set(K, rb, ra, gsl_matrix_get(K, rb, ra) - d1);
        }
    }
}

// Simulation::addPackingForces (Simulation.cpp:8869-8900)
void refAddPackingForces(RefSim* s) {
    for (int j = 0; j < s->nNodes; ++j)
        for (int d = 0; d < 3; ++d)
            gsl_matrix_set(s->nr->gExt, 3 * j + d, 0,
                           s->pk.force[3 * j + d] + gsl_matrix_get(s->nr->gExt, 3 * j + d, 0));
}

// Start-of-step packing work of runOneStep (Simulation.cpp:5833-5843,
// 5911, 5920): bounding box and element positions in it, node masses,
// couple detection.  Growth has already updated the element volumes.
void refPackingStepStart(RefSim* s) {
    refBoundingBox(s);
    refNodeMasses(s);
    refDetectPacking(s);
}

// Simulation::updateRelativePositionsToApicalPositioning (Simulation.cpp:5987-6003)
void refApicalPositioning(RefSim* s) {
    for (ShapeBase* e : s->elements) {
        if (e->tissuePlacement != 1 || e->tissueType != 0 || !e->elementsIdsOnSameColumn) continue;
        double rel[2];
        e->getRelativePosInBoundingBox(rel);
        for (int i = 0; i < s->grid.layers - 2; ++i)
            s->elements[e->elementsIdsOnSameColumn[i]]->setRelativePosInBoundingBox(rel[0], rel[1]);
    }
}

// Once, at the first grid function, from the current (initial) shape:
// Simulation::calculateTissueHeight (Simulation.cpp:3280-3330),
// calculateBoundingBox + assignInitialZPositions (:573-576),
// fillInElementColumnLists (:7612-7624), then the element positions in the
// bounding box, moved to the apical ones and kept as the pinned positions
// (:631-645).
void refGridSetup(RefSim* s) {
    GridRef& g = s->grid;
    g.setUp = true;
    int cur = -1;
    for (Node* n : s->nodes)
        if (n->tissueType == 0 && n->tissuePlacement == 0) {
            cur = n->Id;
            break;
        }
    for (int guard = 0; cur >= 0 && s->nodes[cur]->tissuePlacement != 1 && guard <= s->nElems; ++guard) {
        ShapeBase* owner = nullptr;
        for (ShapeBase* e : s->elements)
            if (e->IsThisNodeMyBasal(cur)) {
                owner = e;
                break;
            }
        if (!owner) break;
        g.height += owner->getElementHeight();
        g.layers++;
        cur = owner->getCorrecpondingApical(cur);
    }
    refBoundingBox(s);
    for (ShapeBase* e : s->elements) e->setInitialZPosition(s->pk.bb[0][2], g.height);
    if (g.layers > 0)
        for (ShapeBase* e : s->elements)
            if (!e->IsAblated && e->tissueType == 0 && e->tissuePlacement == 0)
                e->constructElementStackList(g.layers, s->elements);
    refApicalPositioning(s);
    for (ShapeBase* e : s->elements) e->setInitialRelativePosInBoundingBox();
}

// Simulation::calculateGrowthRing (Simulation.cpp:9801-9885) for one
// element: false when its centre is outside the ring, else the increment of
// the scaled rates.
bool refRingIncrement(ShapeBase* el, GrowthFunctionBase* f, double dt, gsl_matrix* inc) {
    float centre[2];
    f->getCentre(centre[0], centre[1]);
    float innerRadius = f->getInnerRadius();
    float outerRadius = f->getOuterRadius();
    double maxValues[3];
    f->getGrowthRate(maxValues);
    float innerRadius2 = innerRadius * innerRadius;
    float outerRadius2 = outerRadius * outerRadius;
    double* c = el->getCentre();
    double d[2] = {centre[0] - c[0], centre[1] - c[1]};
    delete[] c;
    double dmag2 = d[0] * d[0] + d[1] * d[1];
    if (!(dmag2 > innerRadius2 && dmag2 < outerRadius2)) return false;
    float distance = pow(dmag2, 0.5);
    double sf = (1.0 - (distance - innerRadius) / (outerRadius - innerRadius));
    double growthscale[3] = {maxValues[0] * sf, maxValues[1] * sf, maxValues[2] * sf};
    el->calculateFgFromRates(dt, growthscale[0], growthscale[1], growthscale[2], f->getShearAngleRotationMatrix(),
                             inc, 0, f->zMin, f->zMax);
    return true;
}

// The growth of one step: cleanUpGrowthRates, the per-element rates as a
// uniform function, then (with_functions) the growth functions active at the
// current time in their order (calculateGrowth, Simulation.cpp:9651-9666,
// after the bounding-box positions of :5833-5843), and growShapeByFg.
void refGrow(RefSim* s, double dt, const double* rates, bool with_functions) {
    QuietCout q;
    GridRef& g = s->grid;
    std::vector<GrowthFunctionBase*> active;
    bool grid = false;
    if (with_functions)
        for (GrowthFunctionBase* f : g.fns)
            if (g.time >= f->initTime && g.time < f->endTime) {
                active.push_back(f);
                grid |= f->Type == 3;
            }
    if (grid) {
        refBoundingBox(s);
        refApicalPositioning(s);
    }
    // Simulation::updateGrowthRotationMatrices (Simulation.cpp:4459-4466),
    // called by runOneStep whenever growth functions exist (:5872-5876)
    if (with_functions && !g.fns.empty())
        for (ShapeBase* el : s->elements)
            if (!el->IsAblated) el->CalculateGrowthRotationByF();
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
        for (GrowthFunctionBase* f : active) {
            gsl_matrix_set_identity(inc);
            gsl_matrix_set_identity(peri);
            if (f->Type == 1) {
                double r[3];
                f->getGrowthRate(r);
                el->calculateFgFromRates(dt, r[0], r[1], r[2], f->getShearAngleRotationMatrix(), inc, 0, f->zMin,
                                         f->zMax);
            } else if (f->Type == 2) {
                if (!refRingIncrement(el, f, dt, inc)) continue;
            } else {
                GridBasedGrowthFunction* gf = static_cast<GridBasedGrowthFunction*>(f);
                int ix = 0, iy = 0;
                double fx = 1.0, fy = 1.0;
                if (g.pinned)
                    el->getInitialRelativePositionInTissueInGridIndex(gf->getGridX(), gf->getGridY(), ix, iy, fx, fy);
                else
                    el->getRelativePositionInTissueInGridIndex(gf->getGridX(), gf->getGridY(), ix, iy, fx, fy);
                el->calculateFgFromGridCorners(g.interp, dt, gf, inc, 0, ix, iy, fx, fy);
            }
            el->updateGrowthIncrement(inc, peri);
        }
        el->growShapeByFg();
    }
    gsl_matrix_free(rot);
    gsl_matrix_free(inc);
    gsl_matrix_free(peri);
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
    // Simulation::fillInNodeNeighbourhood (Simulation.cpp:7595-7600)
    for (auto* e : s->elements) e->fillNodeNeighbourhood(s->nodes);
    s->pk.force.assign(3 * (size_t)n_nodes, 0.0);
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

// The growth of one step: per-element rates (1/s) as a single uniform-type
// growth function with the identity rotation, then the grid functions active
// at the current time.
void tfr_grow(void* h, double dt, const double* rates) { refGrow(static_cast<RefSim*>(h), dt, rates, true); }

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
    if (s->pk.on) refPackingForcesAndJacobian(s);
    nr->checkJacobianForAblatedNodes(s->ablated);
    nr->calculateSumOfInternalForces();
    if (s->pk.on) refAddPackingForces(s);
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
    if (rates) {
        tfr_grow(h, dt, rates);
    } else if (s->pk.on || !s->grid.fns.empty()) {
        // runOneStep calls growShapeByFg on every element at every step
        // (Simulation.cpp:5901-5906), which sets the volumes the node masses
        // are made of (the Prism constructor leaves them 0, Prism.cpp:218)
        std::vector<double> zero(3 * (size_t)s->nElems, 0.0);
        tfr_grow(h, dt, zero.data());
    }
    tfr_update_viscosity_surfaces(h, nullptr);
    if (s->pk.on) refPackingStepStart(s);
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
        if (s->pk.on) refPackingForcesAndJacobian(s);
        nr->checkJacobianForAblatedNodes(s->ablated);
        nr->calculateSumOfInternalForces();
        if (s->pk.on) refAddPackingForces(s);
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
    s->grid.time += dt;  // runOneStep: currSimTimeSec += dt (Simulation.cpp:5969)
    return notConverged;
}

// Packing on / off; drop_last_segment reproduces the reference's merge of
// its 16 detection segments (Simulation.cpp:8426), which leaves out the
// couples found from the nodes of the last segment.
void tfr_set_packing(void* h, int on, int drop_last_segment) {
    RefSim* s = static_cast<RefSim*>(h);
    s->pk.on = on != 0;
    s->pk.dropLastSegment = drop_last_segment != 0;
}

// The start-of-step packing work at the current positions and growth (a
// zero-rate growShapeByFg first, as every step of runOneStep does).
void tfr_pack_detect(void* h) {
    RefSim* s = static_cast<RefSim*>(h);
    std::vector<double> zero(3 * (size_t)s->nElems, 0.0);
    refGrow(s, 1.0, zero.data(), false);
    QuietCout q;
    refPackingStepStart(s);
}

long tfr_pack_count(void* h) { return static_cast<long>(static_cast<RefSim*>(h)->pk.c0.size()); }

// Couples of the last detection: node ids (2 per couple), weights (3),
// average masses, the force threshold and the detection distance.
void tfr_pack_get(void* h, int* nodes, double* w, double* mbar, double* threshold, double* detect) {
    RefSim* s = static_cast<RefSim*>(h);
    const PackingRef& p = s->pk;
    for (size_t i = 0; i < p.c0.size(); ++i) {
        if (nodes) {
            nodes[2 * i] = p.c0[i];
            nodes[2 * i + 1] = p.c1[i];
        }
        if (w) {
            w[3 * i] = p.wx[i];
            w[3 * i + 1] = p.wy[i];
            w[3 * i + 2] = p.wz[i];
        }
        if (mbar) mbar[i] = 0.5 * (s->nodes[p.c0[i]]->mass + s->nodes[p.c1[i]]->mass);
    }
    if (threshold) *threshold = p.threshold;
    if (detect) *detect = p.detect;
}

void tfr_node_masses(void* h, double* mass) {
    RefSim* s = static_cast<RefSim*>(h);
    for (int i = 0; i < s->nNodes; ++i) mass[i] = s->nodes[i]->mass;
}

// PackingForces of the last assembly (3 per node).
void tfr_pack_forces(void* h, double* f) {
    RefSim* s = static_cast<RefSim*>(h);
    std::copy(s->pk.force.begin(), s->pk.force.end(), f);
}

// A UniformGrowthFunction over the columnar layer: rates (1/s), xy angle (rad).
void tfr_add_uniform_growth(void* h, const double* rates, double angle, double t0, double t1, double zmin,
                            double zmax) {
    RefSim* s = static_cast<RefSim*>(h);
    QuietCout q;
    if (!s->grid.setUp) refGridSetup(s);
    UniformGrowthFunction* f = new UniformGrowthFunction(static_cast<int>(s->grid.fns.size()), 1, t0, t1, true,
                                                         false, false, false, rates[0], rates[1], rates[2], angle);
    f->zMin = zmin;
    f->zMax = zmax;
    s->grid.fns.push_back(f);
}

// A RingGrowthFunction over the columnar layer.
void tfr_add_ring_growth(void* h, double cx, double cy, double r_in, double r_out, const double* rates,
                         double angle, double t0, double t1, double zmin, double zmax) {
    RefSim* s = static_cast<RefSim*>(h);
    QuietCout q;
    if (!s->grid.setUp) refGridSetup(s);
    RingGrowthFunction* f = new RingGrowthFunction(static_cast<int>(s->grid.fns.size()), 2, t0, t1, true, false,
                                                   false, false, cx, cy, r_in, r_out, rates[0], rates[1], rates[2],
                                                   angle);
    f->zMin = zmin;
    f->zMax = zmax;
    s->grid.fns.push_back(f);
}

void tfr_clear_growth_functions(void* h) { static_cast<RefSim*>(h)->grid.fns.clear(); }

// A GridBasedGrowthFunction over the columnar layer: rates[3*(i*ny + j) + k]
// (1/s), angles_deg[i*ny + j] (NULL: 0), its time window and z range.
void tfr_add_grid_growth(void* h, int nx, int ny, const double* rates, const double* angles_deg, double t0,
                         double t1, double zmin, double zmax) {
    RefSim* s = static_cast<RefSim*>(h);
    QuietCout q;
    if (!s->grid.setUp) refGridSetup(s);
    double*** G = new double**[nx];
    double** A = new double*[nx];
    for (int i = 0; i < nx; ++i) {
        G[i] = new double*[ny];
        A[i] = new double[ny];
        for (int j = 0; j < ny; ++j) {
            G[i][j] = new double[3];
            for (int k = 0; k < 3; ++k) G[i][j][k] = rates[3 * ((size_t)i * ny + j) + k];
            A[i][j] = angles_deg ? angles_deg[(size_t)i * ny + j] : 0.0;
        }
    }
    GridBasedGrowthFunction* f = new GridBasedGrowthFunction(static_cast<int>(s->grid.fns.size()), 3, t0, t1, true,
                                                             false, false, false, nx, ny, G, A);
    f->zMin = zmin;
    f->zMax = zmax;
    s->grid.fns.push_back(f);
    for (int i = 0; i < nx; ++i) {
        for (int j = 0; j < ny; ++j) delete[] G[i][j];
        delete[] G[i];
        delete[] A[i];
    }
    delete[] G;
    delete[] A;
}

void tfr_set_grid_mode(void* h, int interp, int pinned) {
    RefSim* s = static_cast<RefSim*>(h);
    s->grid.interp = interp;
    s->grid.pinned = pinned != 0;
}

// Simulation::updatePinningPositions (Simulation.cpp:6018-6023) at the
// current shape.
void tfr_repin_grid_growth(void* h) {
    RefSim* s = static_cast<RefSim*>(h);
    QuietCout q;
    refBoundingBox(s);
    refApicalPositioning(s);
    for (ShapeBase* e : s->elements) e->setInitialRelativePosInBoundingBox();
}

void tfr_set_time(void* h, double t) { static_cast<RefSim*>(h)->grid.time = t; }
double tfr_get_time(void* h) { return static_cast<RefSim*>(h)->grid.time; }

// Initial relative z, pinned positions and the current shape's positions
// ([2][n_elems] each, x block then y block).
void tfr_grid_positions(void* h, double* relz, double* rel0, double* rel) {
    RefSim* s = static_cast<RefSim*>(h);
    QuietCout q;
    refBoundingBox(s);
    refApicalPositioning(s);
    const int ne = s->nElems;
    for (int e = 0; e < ne; ++e) {
        double r[2], r0[2];
        s->elements[e]->getRelativePosInBoundingBox(r);
        s->elements[e]->getInitialRelativePosInBoundingBox(r0);
        if (relz) relz[e] = static_cast<PrismRef*>(s->elements[e])->relZ();
        if (rel0) {
            rel0[e] = r0[0];
            rel0[ne + e] = r0[1];
        }
        if (rel) {
            rel[e] = r[0];
            rel[ne + e] = r[1];
        }
    }
}

}  // extern "C"
