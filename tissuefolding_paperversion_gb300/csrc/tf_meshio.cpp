// The reference's mesh input file and save-frame formats, host side.
//
//   * .mesh input (Simulation::initiateNodesFromMeshInput /
//     initiateElementsFromMeshInput / initiatePrismFromMeshInput,
//     Simulation.cpp:2074-2239): the node count, then per node
//     "x y z tissuePlacement tissueType atCircumference"; the element count,
//     then per element the shape type (1 = prism), six node ids and the 6 x 3
//     reference positions (ShapeBase::updateReferencePositionMatrixFromSave,
//     ShapeBase.cpp:935-944); an optional tissue-weights block follows
//     (Simulation.cpp:2972-2976, 3016-3023).  Each prism goes through the
//     reference's orientation check (Prism::checkRotationConsistency3D,
//     Prism.cpp:364-410): node ids 1<->2 and 4<->5 are swapped when the basal
//     triangle is clockwise seen from the apical side.
//   * save frames (Simulation::saveStep -> writeSaveFileStepHeader,
//     writeNodes, writeElements, writeSaveFileStepFooter,
//     Simulation.cpp:9265-9356): the same records with the reference's field
//     widths and precisions, so its viewer and analysis tools read them.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "../../include/tf_gpu.h"

namespace tf {
void set_error(const std::string& msg);
}

namespace {

struct MeshFile {
    std::vector<double> pos, ref;
    std::vector<int32_t> conn, placement, type, circ;
    std::vector<double> weights;
    int32_t nn = 0, ne = 0;
};

bool parse(const char* path, MeshFile& m, std::string& err) {
    std::ifstream f(path);
    if (!f.is_open()) {
        err = std::string("cannot open the mesh file ") + path;
        return false;
    }
    long long n = 0;
    if (!(f >> n) || n < 0 || n > (1LL << 30)) {
        err = "mesh file: bad node count";
        return false;
    }
    m.nn = static_cast<int32_t>(n);
    m.pos.resize(3 * (size_t)n);
    m.placement.resize(n);
    m.type.resize(n);
    m.circ.resize(n);
    for (long long i = 0; i < n; ++i) {
        if (!(f >> m.pos[3 * i] >> m.pos[3 * i + 1] >> m.pos[3 * i + 2] >> m.placement[i] >> m.type[i] >> m.circ[i])) {
            err = "mesh file: truncated node record " + std::to_string(i);
            return false;
        }
    }
    long long e = 0;
    if (!(f >> e) || e < 0 || e > (1LL << 30)) {
        err = "mesh file: bad element count";
        return false;
    }
    m.ne = static_cast<int32_t>(e);
    m.conn.resize(6 * (size_t)e);
    m.ref.resize(18 * (size_t)e);
    for (long long k = 0; k < e; ++k) {
        int shape = 0;
        if (!(f >> shape)) {
            err = "mesh file: truncated element record " + std::to_string(k);
            return false;
        }
        if (shape != 1) {
            err = "mesh file: element " + std::to_string(k) + " has shape type " + std::to_string(shape) +
                  " (only prisms, type 1, are read)";
            return false;
        }
        for (int a = 0; a < 6; ++a)
            if (!(f >> m.conn[6 * k + a]) || m.conn[6 * k + a] < 0 || m.conn[6 * k + a] >= m.nn) {
                err = "mesh file: element " + std::to_string(k) + " has a bad node id";
                return false;
            }
        for (int q = 0; q < 18; ++q)
            if (!(f >> m.ref[18 * k + q])) {
                err = "mesh file: truncated reference positions of element " + std::to_string(k);
                return false;
            }
        // orientation: view from apical to basal, basal triangle counter-clockwise
        const int32_t* c = &m.conn[6 * k];
        double v1[3], v2[3], view[3];
        for (int d = 0; d < 3; ++d) {
            v1[d] = m.pos[3 * (size_t)c[1] + d] - m.pos[3 * (size_t)c[0] + d];
            v2[d] = m.pos[3 * (size_t)c[2] + d] - m.pos[3 * (size_t)c[0] + d];
            view[d] = m.pos[3 * (size_t)c[0] + d] - m.pos[3 * (size_t)c[3] + d];
        }
        const double nrm[3] = {v1[1] * v2[2] - v1[2] * v2[1], v1[2] * v2[0] - v1[0] * v2[2],
                               v1[0] * v2[1] - v1[1] * v2[0]};
        if (view[0] * nrm[0] + view[1] * nrm[1] + view[2] * nrm[2] > 0) {
            int32_t* cc = &m.conn[6 * k];
            std::swap(cc[1], cc[2]);
            std::swap(cc[4], cc[5]);
            double* r = &m.ref[18 * k];
            for (int d = 0; d < 3; ++d) {
                std::swap(r[3 * 1 + d], r[3 * 2 + d]);
                std::swap(r[3 * 4 + d], r[3 * 5 + d]);
            }
        }
    }
    int flag = 0;
    if (f >> flag && flag) {
        m.weights.resize(e);
        for (long long k = 0; k < e; ++k)
            if (!(f >> m.weights[k])) {
                err = "mesh file: truncated tissue weights";
                return false;
            }
    }
    return true;
}

}  // namespace

extern "C" {

TF_API tf_status tf_read_mesh_file(const char* path, int32_t* n_nodes, int32_t* n_elems, double* pos, int32_t* conn,
                                   int32_t* placement, int32_t* tissue_type, int32_t* at_circumference,
                                   double* ref_pos) {
    if (!path || !n_nodes || !n_elems) {
        tf::set_error("tf_read_mesh_file: bad arguments");
        return TF_BAD_INPUT;
    }
    MeshFile m;
    std::string err;
    if (!parse(path, m, err)) {
        tf::set_error(err);
        return TF_BAD_INPUT;
    }
    const bool fill = pos || conn || placement || tissue_type || at_circumference || ref_pos;
    if (fill && (*n_nodes != m.nn || *n_elems != m.ne)) {
        tf::set_error("tf_read_mesh_file: the arrays are sized for a different mesh (call with NULL arrays first)");
        return TF_BAD_INPUT;
    }
    *n_nodes = m.nn;
    *n_elems = m.ne;
    if (pos) std::memcpy(pos, m.pos.data(), m.pos.size() * sizeof(double));
    if (conn) std::memcpy(conn, m.conn.data(), m.conn.size() * sizeof(int32_t));
    if (placement) std::memcpy(placement, m.placement.data(), m.placement.size() * sizeof(int32_t));
    if (tissue_type) std::memcpy(tissue_type, m.type.data(), m.type.size() * sizeof(int32_t));
    if (at_circumference) std::memcpy(at_circumference, m.circ.data(), m.circ.size() * sizeof(int32_t));
    if (ref_pos) std::memcpy(ref_pos, m.ref.data(), m.ref.size() * sizeof(double));
    return TF_OK;
}

TF_API tf_status tf_write_frame(const char* path, int32_t append, double time_sec, int32_t n_nodes, const double* pos,
                                const int32_t* placement, const int32_t* tissue_type,
                                const int32_t* at_circumference, int32_t n_elems, const int32_t* conn,
                                const double* ref_pos) {
    if (!path || n_nodes < 0 || n_elems < 0 || (n_nodes && (!pos || !placement || !tissue_type || !at_circumference)) ||
        (n_elems && (!conn || !ref_pos))) {
        tf::set_error("tf_write_frame: bad arguments");
        return TF_BAD_INPUT;
    }
    FILE* f = std::fopen(path, append ? "a" : "w");
    if (!f) {
        tf::set_error(std::string("tf_write_frame: cannot open ") + path);
        return TF_BAD_INPUT;
    }
    // writeSaveFileStepHeader: precision 6, width 10
    std::fprintf(f, "=============== TIME: %10.6g===================================================\n", time_sec);
    // writeNodes: count, then per node 3 x (precision 10, width 20) and 3 x width 4
    std::fprintf(f, "%d\n", n_nodes);
    for (int32_t i = 0; i < n_nodes; ++i)
        std::fprintf(f, "%20.10g%20.10g%20.10g%4d%4d%4d\n", pos[3 * (size_t)i], pos[3 * (size_t)i + 1],
                     pos[3 * (size_t)i + 2], placement[i], tissue_type[i], at_circumference[i]);
    // writeElements: count, then shape type (width 4), IsAblated (width 4),
    // node ids (width 9), reference positions (precision 4, width 15)
    std::fprintf(f, "%d\n", n_elems);
    for (int32_t e = 0; e < n_elems; ++e) {
        std::fprintf(f, "%4d%4d", 1, 0);
        for (int a = 0; a < 6; ++a) std::fprintf(f, "%9d", conn[6 * (size_t)e + a]);
        for (int q = 0; q < 18; ++q) std::fprintf(f, "%15.4g", ref_pos[18 * (size_t)e + q]);
        std::fprintf(f, "\n");
    }
    // writeSaveFileStepFooter
    std::fprintf(f, "=============== END OF TIME: %10.6g============================================\n", time_sec);
    const bool ok = std::fflush(f) == 0;
    std::fclose(f);
    if (!ok) {
        tf::set_error(std::string("tf_write_frame: write failed on ") + path);
        return TF_BAD_INPUT;
    }
    return TF_OK;
}

}  // extern "C"
