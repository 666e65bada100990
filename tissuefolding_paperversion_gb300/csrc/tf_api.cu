// C ABI of the GB300 implicit prism step (declared in include/tf_gpu.h):
// set-up of the device-resident mesh, the block-sparse pattern and the
// element-slot map, and the host side of the NewtonRaphsonSolver call
// sequence driven by Simulation::updateStepNR
// (TissueFolding/TissueFolding/SourceCode/Simulation.cpp:6449-6590).
#include <algorithm>
#include <array>
#include <map>
#include <set>
#include <tuple>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "tf_internal.cuh"

namespace tf {

namespace {
thread_local std::string g_last_error = "no error";

// Gauss points (eta, nu, zeta), weight 1/6 each: Prism.cpp:123-146.
// Shape-function derivatives dN (3x6): Prism::setShapeFunctionDerivatives,
// Prism.cpp:655-680.
void shape_derivatives(int gp, double dN[3][6]) {
    const double s = 1.0 / std::sqrt(3.0);
    const double pts[6][3] = {{1.0 / 6.0, 1.0 / 6.0, s}, {2.0 / 3.0, 1.0 / 6.0, s}, {1.0 / 6.0, 2.0 / 3.0, s},
                              {1.0 / 6.0, 1.0 / 6.0, -s}, {2.0 / 3.0, 1.0 / 6.0, -s}, {1.0 / 6.0, 2.0 / 3.0, -s}};
    const double eta = pts[gp][0], nu = pts[gp][1], zeta = pts[gp][2];
    const double alpha = (1 - zeta) / 2, beta = (1 + zeta) / 2, lambda = 1 - eta - nu;
    const double d[3][6] = {{-alpha, alpha, 0, -beta, beta, 0},
                            {-alpha, 0, alpha, -beta, 0, beta},
                            {-lambda / 2, -eta / 2, -nu / 2, lambda / 2, eta / 2, nu / 2}};
    std::memcpy(dN, d, sizeof(d));
}

bool inverse3(const double M[9], double inv[9], double* det_out) {
    const double c0 = M[4] * M[8] - M[5] * M[7];
    const double c1 = M[5] * M[6] - M[3] * M[8];
    const double c2 = M[3] * M[7] - M[4] * M[6];
    const double det = M[0] * c0 + M[1] * c1 + M[2] * c2;
    *det_out = det;
    if (det == 0.0 || !std::isfinite(det)) return false;
    const double r = 1.0 / det;
    inv[0] = c0 * r;
    inv[1] = (M[2] * M[7] - M[1] * M[8]) * r;
    inv[2] = (M[1] * M[5] - M[2] * M[4]) * r;
    inv[3] = c1 * r;
    inv[4] = (M[0] * M[8] - M[2] * M[6]) * r;
    inv[5] = (M[2] * M[3] - M[0] * M[5]) * r;
    inv[6] = c2 * r;
    inv[7] = (M[1] * M[6] - M[0] * M[7]) * r;
    inv[8] = (M[0] * M[4] - M[1] * M[3]) * r;
    return true;
}

// Prism::calculateReferenceVolume (Prism.cpp:876-908) with
// ShapeBase::calculateVolumeForInputShapeStructure (ShapeBase.cpp:3362-3395):
// 8 triangles (2 bases, 3 split quads), each the base of a tetrahedron with
// the prism's centre.
double prism_volume(const double X[6][3]) {
    static const int faces[8][3] = {{0, 1, 2}, {3, 4, 5}, {0, 1, 3}, {1, 3, 4},
                                    {1, 2, 4}, {2, 4, 5}, {0, 2, 3}, {2, 3, 5}};
    double c[3] = {0.0, 0.0, 0.0};
    for (int a = 0; a < 6; ++a)
        for (int k = 0; k < 3; ++k) c[k] += X[a][k];
    for (int k = 0; k < 3; ++k) c[k] /= 6;
    double vol = 0.0;
    for (const auto& f : faces) {
        double v1[3], v2[3], vm[3];
        for (int k = 0; k < 3; ++k) {
            v1[k] = X[f[1]][k] - X[f[0]][k];
            v2[k] = X[f[2]][k] - X[f[0]][k];
            vm[k] = c[k] - X[f[0]][k];
        }
        const double b[3] = {v1[1] * v2[2] - v1[2] * v2[1], v1[2] * v2[0] - v1[0] * v2[2],
                             v1[0] * v2[1] - v1[1] * v2[0]};
        const double nb = std::sqrt(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
        double hgt = (vm[0] * b[0] + vm[1] * b[1] + vm[2] * b[2]) / nb;
        if (hgt < 0) hgt *= -1.0;
        vol += 1.0 / 3.0 * (hgt * (nb / 2));
    }
    return vol;
}

template <class T>
tf_status dev_alloc(T** p, size_t n) {
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), n * sizeof(T));
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        set_error("device allocation of " + std::to_string(n * sizeof(T)) + " bytes failed");
        return TF_OUT_OF_MEMORY;
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
    return TF_OK;
}

template <class T>
tf_status upload(T** p, const std::vector<T>& v) {
    tf_status s = dev_alloc(p, v.size());
    if (s != TF_OK) return s;
    TF_CUDA(cudaMemcpy(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return TF_OK;
}

void free_all(tf_handle* h) {
    Device& d = h->d;
    void* ptrs[] = {d.conn, d.gx, d.wdet, d.detdxde, d.Fg, d.invFg, d.rates, d.lam, d.mu, d.eta, d.exposure,
                    d.aptr, d.alist, d.farea, d.fixed, d.ext_visc, d.area, d.rowptr, d.colidx, d.diag, d.rowof,
                    d.slot, d.bofs, d.wslot0, d.scol, d.val, d.eblk, d.ef, d.gptr, d.glist, d.fptr, d.flist, d.uk, d.un, d.vel, d.g,
                    d.du, d.dinv, d.r, d.p, d.z, d.q, d.rhat, d.s, d.t, d.sh, d.scal, d.part, d.tickets,
                    d.seg_node0, d.elem_seg, d.cta_seg, d.cta_node0, d.cta_node1, d.seg_cta0, d.seg_active, d.seg_solve,
                    d.tblk, d.valT, d.lamv, d.carry, d.dldu, d.gr, d.ge, d.nu, d.apical, d.xrow, d.xcol, d.xval,
                    d.check};
    destroy_graphs(h);
    if (h->kloop_ctl) cudaFree(h->kloop_ctl);
    if (h->kloop_host) cudaFreeHost(h->kloop_host);
    h->kloop_ctl = nullptr;
    h->kloop_host = nullptr;
    if (h->du0) cudaFree(h->du0);
    h->du0 = nullptr;
    h->have_du0 = false;
    if (h->nd) cudaFree(h->nd);
    if (h->nd_host) cudaFreeHost(h->nd_host);
    if (h->nd_seg) cudaFree(h->nd_seg);
    if (h->nd_seg_host) cudaFreeHost(h->nd_seg_host);
    if (h->cap_stream) cudaStreamDestroy(h->cap_stream);
    h->nd = nullptr;
    h->nd_host = nullptr;
    h->nd_seg = nullptr;
    h->nd_seg_host = nullptr;
    h->cap_stream = nullptr;
    if (h->amg) {
        amg_free(h->amg);
        h->amg = nullptr;
    }
    if (h->pk) {
        packing_free(h->pk);
        h->pk = nullptr;
    }
    if (h->growth) {
        growth_free(h->growth);
        h->growth = nullptr;
    }
    bind_free(h);
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (d.host_scal) cudaFreeHost(d.host_scal);
    for (auto& e : h->ev)
        if (e) cudaEventDestroy(e);
    if (h->stream) cudaStreamDestroy(h->stream);
}

#define TF_TRY(expr)                       \
    do {                                   \
        tf_status _s = (expr);             \
        if (_s != TF_OK) return _s;        \
    } while (0)

tf_status check_handle(tf_handle* h) {
    if (!h) {
        set_error("null handle");
        return TF_BAD_INPUT;
    }
    TF_CUDA(cudaSetDevice(h->device));
    return TF_OK;
}

// CTA tables of the node-parallel kernels: every CTA covers up to
// kNodeThreads consecutive nodes of one instance.
tf_status setup_instances(tf_handle* h, const std::vector<int>& seg_node0, const std::vector<int>& seg_elem0) {
    Device& d = h->d;
    const int nseg = static_cast<int>(seg_node0.size()) - 1;
    d.nseg = nseg;
    std::vector<int> cta_seg, cta0, cta1, seg_cta0(nseg + 1, 0), elem_seg(d.ne);
    for (int g = 0; g < nseg; ++g) {
        seg_cta0[g] = static_cast<int>(cta_seg.size());
        for (int n0 = seg_node0[g]; n0 < seg_node0[g + 1]; n0 += kNodeThreads) {
            cta_seg.push_back(g);
            cta0.push_back(n0);
            cta1.push_back(std::min(n0 + kNodeThreads, seg_node0[g + 1]));
        }
        for (int e = seg_elem0[g]; e < seg_elem0[g + 1]; ++e) elem_seg[e] = g;
    }
    seg_cta0[nseg] = static_cast<int>(cta_seg.size());
    d.ncta = static_cast<int>(cta_seg.size());
    TF_TRY(upload(&d.seg_node0, seg_node0));
    TF_TRY(upload(&d.elem_seg, elem_seg));
    TF_TRY(upload(&d.cta_seg, cta_seg));
    TF_TRY(upload(&d.cta_node0, cta0));
    TF_TRY(upload(&d.cta_node1, cta1));
    TF_TRY(upload(&d.seg_cta0, seg_cta0));
    h->h_active.assign(nseg, 1);
    TF_TRY(upload(&d.seg_active, h->h_active));
    TF_TRY(upload(&d.seg_solve, h->h_active));
    TF_TRY(dev_alloc(&d.tickets, nseg));
    TF_TRY(dev_alloc(&d.check, 1));
    TF_CUDA(cudaMemset(d.check, 0, sizeof(int)));
    TF_CUDA(cudaMemset(d.tickets, 0, sizeof(unsigned) * (size_t)nseg));
    TF_TRY(dev_alloc(&d.scal, (size_t)nseg * S_COUNT));
    TF_CUDA(cudaMemset(d.scal, 0, sizeof(double) * (size_t)nseg * S_COUNT));
    TF_TRY(dev_alloc(&d.part, 3 * (size_t)d.ncta));
    TF_CUDA(cudaMallocHost(reinterpret_cast<void**>(&d.host_scal), sizeof(double) * (size_t)nseg * S_COUNT));
    h->h_seg_node0 = seg_node0;
    h->h_seg_elem0 = seg_elem0;
    return TF_OK;
}

tf_status build(tf_handle* h, const tf_mesh* m, const tf_material* mat, const std::vector<int>& seg_node0,
                const std::vector<int>& seg_elem0) {
    Device& d = h->d;
    const int nn = m->n_nodes, ne = m->n_elems;
    d.nn = nn;
    d.ne = ne;
    // ---- connectivity (SoA) and placement ---------------------------------
    h->h_conn.assign(m->conn, m->conn + 6 * (size_t)ne);
    std::vector<int> conn_soa(6 * (size_t)ne);
    for (int e = 0; e < ne; ++e)
        for (int a = 0; a < 6; ++a) conn_soa[(size_t)a * ne + e] = m->conn[6 * (size_t)e + a];
    // ShapeBase::setTissuePlacement (ShapeBase.cpp:705-770) and
    // Prism::assignExposedSurfaceAreaIndices (Prism.cpp:2674-2742) for
    // columnar elements: bit0 apical face exposed, bit1 basal face exposed.
    std::vector<int> exposure(ne);
    for (int e = 0; e < ne; ++e) {
        bool hasA = false, hasB = false, hasL = false;
        for (int a = 0; a < 6; ++a) {
            int p = m->node_placement[m->conn[6 * (size_t)e + a]];
            if (p == 1) hasA = true;
            else if (p == 0) hasB = true;
            else if (p == 3) hasL = true;
        }
        int ex = 0;
        if (!hasL) {
            if (hasA && hasB) ex = 3;
            else if (hasA) ex = 1;
            else if (hasB) ex = 2;
        }
        exposure[e] = ex;
    }
    // ---- reference geometry: dN_X per Gauss point --------------------------
    std::vector<double> gx(18 * 6 * (size_t)ne), wdet(6 * (size_t)ne), detd(6 * (size_t)ne);
    h->h_vref.assign(ne, 0.0);
    double dN[6][3][6];
    for (int gp = 0; gp < 6; ++gp) shape_derivatives(gp, dN[gp]);
    for (int e = 0; e < ne; ++e) {
        double X[6][3];  // the reference shape (ReferenceShape->Positions)
        for (int a = 0; a < 6; ++a)
            for (int c = 0; c < 3; ++c)
                X[a][c] = m->ref_pos ? m->ref_pos[18 * (size_t)e + 3 * a + c]
                                     : m->node_pos[3 * (size_t)m->conn[6 * (size_t)e + a] + c];
        h->h_vref[e] = prism_volume(X);
        for (int gp = 0; gp < 6; ++gp) {
            // dX/dxi = (dN X)^T   (Prism.cpp:705-728)
            double J[9];
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) {
                    double acc = 0.0;
                    for (int a = 0; a < 6; ++a) acc += dN[gp][j][a] * X[a][i];
                    J[3 * i + j] = acc;
                }
            double inv[9], det;
            if (!inverse3(J, inv, &det) || !(det > 0.0)) {
                set_error("element " + std::to_string(e) + " has a degenerate or inverted reference shape");
                return TF_BAD_INPUT;
            }
            const size_t q = 6 * (size_t)e + gp;
            detd[q] = det;
            wdet[q] = (1.0 / 6.0) * det;
            for (int a = 0; a < 6; ++a)
                for (int k = 0; k < 3; ++k) {
                    double acc = 0.0;
                    for (int j = 0; j < 3; ++j) acc += inv[3 * j + k] * dN[gp][j][a];
                    gx[(size_t)(3 * a + k) * (6 * (size_t)ne) + q] = acc;
                }
        }
    }
    // ---- material (Prism::setElasticProperties, Prism.cpp:491-516) ----------
    std::vector<double> lam(ne), mu(ne), eta(ne);
    d.any_visc = false;
    h->h_nu.resize(ne);
    h->h_apical.resize(nn);
    for (int i = 0; i < nn; ++i) h->h_apical[i] = m->node_placement[i] == 1 ? 1 : 0;
    h->h_place.assign(m->node_placement, m->node_placement + nn);
    h->h_pos0.assign(m->node_pos, m->node_pos + 3 * (size_t)nn);
    for (int e = 0; e < ne; ++e) {
        double v = mat->nu[e];
        if (v > 0.5) v = 0.5;
        else if (v < 0.0) v = 0.0;
        h->h_nu[e] = v;
        const double E = mat->E[e];
        lam[e] = E * v / (1 + v) / (1 - 2.0 * v);
        mu[e] = E / 2.0 / (1 + v);
        eta[e] = mat->eta[e];
        if (eta[e] != 0.0) d.any_visc = true;
        if (!std::isfinite(lam[e]) || !std::isfinite(mu[e]) || !std::isfinite(eta[e])) {
            set_error("element " + std::to_string(e) + " has non-finite material parameters (nu = 0.5 is incompressible)");
            return TF_BAD_INPUT;
        }
    }
    // ---- node adjacency -> block pattern of A ---------------------------------
    std::vector<int> cnt(nn + 1, 0);
    for (int e = 0; e < ne; ++e)
        for (int a = 0; a < 6; ++a) cnt[m->conn[6 * (size_t)e + a]] += 6;
    std::vector<int64_t> off(nn + 1, 0);
    for (int i = 0; i < nn; ++i) off[i + 1] = off[i] + cnt[i];
    std::vector<int> tmp(off[nn]);
    std::vector<int64_t> fill(off.begin(), off.end() - 1);
    for (int e = 0; e < ne; ++e)
        for (int a = 0; a < 6; ++a) {
            const int A = m->conn[6 * (size_t)e + a];
            for (int b = 0; b < 6; ++b) tmp[fill[A]++] = m->conn[6 * (size_t)e + b];
        }
    std::vector<int> rowptr(nn + 1, 0);
    std::vector<int> colidx;
    colidx.reserve(off[nn] / 2);
    for (int i = 0; i < nn; ++i) {
        auto b = tmp.begin() + off[i], en = tmp.begin() + off[i + 1];
        std::sort(b, en);
        auto u = std::unique(b, en);
        colidx.insert(colidx.end(), b, u);
        rowptr[i + 1] = static_cast<int>(colidx.size());
        if (colidx.size() > (size_t)INT32_MAX / 9) {
            set_error("mesh too large for 32-bit block indices");
            return TF_BAD_INPUT;
        }
    }
    tmp.clear();
    tmp.shrink_to_fit();
    const int64_t nnzb = static_cast<int64_t>(colidx.size());
    d.nnzb = nnzb;
    std::vector<int> diag(nn), rowof(nnzb);
    for (int i = 0; i < nn; ++i) {
        for (int p = rowptr[i]; p < rowptr[i + 1]; ++p) rowof[p] = i;
        auto it = std::lower_bound(colidx.begin() + rowptr[i], colidx.begin() + rowptr[i + 1], i);
        diag[i] = static_cast<int>(it - colidx.begin());
    }
    auto find_block = [&](int r, int c) {
        auto it = std::lower_bound(colidx.begin() + rowptr[r], colidx.begin() + rowptr[r + 1], c);
        return static_cast<int>(it - colidx.begin());
    };
    std::vector<int> slot(36 * (size_t)ne);
    for (int e = 0; e < ne; ++e)
        for (int a = 0; a < 6; ++a)
            for (int b = 0; b < 6; ++b)
                slot[(size_t)(6 * a + b) * ne + e] = find_block(m->conn[6 * (size_t)e + a], m->conn[6 * (size_t)e + b]);
    // ---- node -> exposed faces (viscosity surfaces) ---------------------------
    std::vector<int> aptr(nn + 1, 0), alist;
    {
        std::vector<std::vector<int>> per(nn);
        for (int e = 0; e < ne; ++e) {
            if (exposure[e] & 1)
                for (int a = 3; a < 6; ++a) per[m->conn[6 * (size_t)e + a]].push_back(0 * ne + e);
            if (exposure[e] & 2)
                for (int a = 0; a < 3; ++a) per[m->conn[6 * (size_t)e + a]].push_back(1 * ne + e);
        }
        for (int i = 0; i < nn; ++i) {
            alist.insert(alist.end(), per[i].begin(), per[i].end());
            aptr[i + 1] = static_cast<int>(alist.size());
        }
    }
    // ---- uploads -----------------------------------------------------------------
    TF_TRY(upload(&d.conn, conn_soa));
    TF_TRY(upload(&d.gx, gx));
    TF_TRY(upload(&d.wdet, wdet));
    TF_TRY(upload(&d.detdxde, detd));
    TF_TRY(upload(&d.lam, lam));
    TF_TRY(upload(&d.mu, mu));
    TF_TRY(upload(&d.eta, eta));
    TF_TRY(upload(&d.exposure, exposure));
    TF_TRY(upload(&d.aptr, aptr));
    TF_TRY(upload(&d.alist, alist));
    TF_TRY(dev_alloc(&d.farea, 2 * (size_t)ne));
    h->h_fixed.assign(m->fixed, m->fixed + 3 * (size_t)nn);
    TF_TRY(upload(&d.fixed, h->h_fixed));
    TF_TRY(upload(&d.ext_visc, std::vector<double>(m->ext_visc, m->ext_visc + 3 * (size_t)nn)));
    TF_TRY(dev_alloc(&d.area, nn));
    TF_CUDA(cudaMemset(d.area, 0, sizeof(double) * (size_t)nn));
    TF_TRY(upload(&d.rowptr, rowptr));
    TF_TRY(upload(&d.colidx, colidx));
    TF_TRY(upload(&d.rowof, rowof));
    std::vector<double> ident(9 * (size_t)ne, 0.0);
    for (int k : {0, 4, 8})
        for (int e = 0; e < ne; ++e) ident[(size_t)k * ne + e] = 1.0;
    TF_TRY(upload(&d.Fg, ident));
    TF_TRY(upload(&d.invFg, ident));
    TF_TRY(upload(&d.rates, std::vector<double>(3 * (size_t)ne, 0.0)));
    const size_t n3 = 3 * (size_t)nn;
    std::vector<double> pos(m->node_pos, m->node_pos + n3);
    TF_TRY(upload(&d.uk, pos));
    TF_TRY(upload(&d.un, pos));
    double** vecs[] = {&d.vel, &d.g, &d.du, &d.r, &d.p, &d.z, &d.q, &d.rhat, &d.s, &d.t, &d.sh};
    for (double** v : vecs) {
        TF_TRY(dev_alloc(v, n3));
        TF_CUDA(cudaMemset(*v, 0, n3 * sizeof(double)));
    }
    TF_TRY(dev_alloc(&d.dinv, 9 * (size_t)nn));
    TF_TRY(setup_instances(h, seg_node0, seg_elem0));
    // ---- sliced value storage ----------------------------------------------------
    // Warp w of CTA c covers rows cta0[c] + 32 w ... (as in the node-parallel
    // kernels); its slots are as many as its longest row.
    std::vector<int> bofs(nnzb), scol, wslot0;
    {
        std::vector<int> cta0;
        std::vector<int> cta1;
        for (size_t g = 0; g + 1 < seg_node0.size(); ++g)
            for (int n0 = seg_node0[g]; n0 < seg_node0[g + 1]; n0 += kNodeThreads) {
                cta0.push_back(n0);
                cta1.push_back(std::min(n0 + kNodeThreads, seg_node0[g + 1]));
            }
        const size_t nwarp = cta0.size() * kWarps;
        wslot0.assign(nwarp + 1, 0);
        int64_t nslots = 0;
        for (size_t c = 0; c < cta0.size(); ++c)
            for (int w = 0; w < kWarps; ++w) {
                const int r0 = cta0[c] + 32 * w, r1 = std::min(r0 + 32, cta1[c]);
                int W = 0;
                for (int i = r0; i < r1; ++i) W = std::max(W, rowptr[i + 1] - rowptr[i]);
                wslot0[c * kWarps + w] = static_cast<int>(nslots);
                nslots += W;
                if (nslots * kSlotDoubles > (int64_t)INT32_MAX) {
                    set_error("mesh too large for 32-bit value offsets");
                    return TF_BAD_INPUT;
                }
                for (int i = r0; i < r1; ++i)
                    for (int p = rowptr[i]; p < rowptr[i + 1]; ++p)
                        bofs[p] = (wslot0[c * kWarps + w] + (p - rowptr[i])) * kSlotDoubles + (i - r0);
            }
        wslot0[nwarp] = static_cast<int>(nslots);
        scol.assign(nslots * kSlice, 0);
        for (size_t c = 0; c < cta0.size(); ++c)
            for (int w = 0; w < kWarps; ++w) {
                const int r0 = cta0[c] + 32 * w, r1 = std::min(r0 + 32, cta1[c]);
                const int s0 = wslot0[c * kWarps + w], s1 = wslot0[c * kWarps + w + 1];
                for (int l = 0; l < 32; ++l) {
                    const int i = r0 + l;
                    const int len = i < r1 ? rowptr[i + 1] - rowptr[i] : 0;
                    for (int sl = s0; sl < s1; ++sl) {
                        const int k = sl - s0;
                        // padding: own row (or the warp's first row), value 0
                        scol[(size_t)sl * kSlice + l] = k < len ? colidx[rowptr[i] + k] : (i < r1 ? i : r0);
                    }
                }
            }
        d.nval = nslots * kSlotDoubles;
    }
    std::vector<int> slot_ofs(slot.size()), diag_ofs(nn);
    for (size_t q = 0; q < slot.size(); ++q) slot_ofs[q] = bofs[slot[q]];
    for (int i = 0; i < nn; ++i) diag_ofs[i] = bofs[diag[i]];
    TF_TRY(upload(&d.diag, diag_ofs));
    TF_TRY(upload(&d.slot, slot_ofs));
    TF_TRY(upload(&d.bofs, bofs));
    TF_TRY(upload(&d.wslot0, wslot0));
    TF_TRY(upload(&d.scol, scol));
    TF_TRY(dev_alloc(&d.val, d.nval));
    TF_CUDA(cudaMemset(d.val, 0, sizeof(double) * (size_t)d.nval));
    // ---- order-fixed assembly lists ----------------------------------------------
    if (h->opt.deterministic) {
        std::vector<int> gptr(nnzb + 1, 0), glist(36 * (size_t)ne);
        for (int e = 0; e < ne; ++e)
            for (int p = 0; p < 36; ++p) gptr[slot[(size_t)p * ne + e] + 1]++;
        for (int64_t b = 0; b < nnzb; ++b) gptr[b + 1] += gptr[b];
        std::vector<int> gf(gptr.begin(), gptr.end() - 1);
        for (int e = 0; e < ne; ++e)
            for (int p = 0; p < 36; ++p) glist[gf[slot[(size_t)p * ne + e]]++] = p * ne + e;
        std::vector<int> fptr(nn + 1, 0), flist(6 * (size_t)ne);
        for (int e = 0; e < ne; ++e)
            for (int a = 0; a < 6; ++a) fptr[m->conn[6 * (size_t)e + a] + 1]++;
        for (int i = 0; i < nn; ++i) fptr[i + 1] += fptr[i];
        std::vector<int> ff(fptr.begin(), fptr.end() - 1);
        for (int e = 0; e < ne; ++e)
            for (int a = 0; a < 6; ++a) flist[ff[m->conn[6 * (size_t)e + a]]++] = a * ne + e;
        TF_TRY(upload(&d.gptr, gptr));
        TF_TRY(upload(&d.glist, glist));
        TF_TRY(upload(&d.fptr, fptr));
        TF_TRY(upload(&d.flist, flist));
        TF_TRY(dev_alloc(&d.eblk, 9 * 36 * (size_t)ne));
        TF_TRY(dev_alloc(&d.ef, 18 * (size_t)ne));
    }
    h->h_rowptr = std::move(rowptr);
    h->h_colidx = std::move(colidx);
    h->h_bofs = std::move(bofs);
    h->method = h->opt.krylov_method == 0 ? (d.any_visc ? 2 : 1) : h->opt.krylov_method;
    return TF_OK;
}

tf_status validate(const tf_mesh* m, const tf_material* mat) {
    if (!m || !mat) {
        set_error("mesh and material are required");
        return TF_BAD_INPUT;
    }
    if (m->n_nodes <= 0 || m->n_elems <= 0 || !m->node_pos || !m->conn || !m->fixed || !m->ext_visc ||
        !m->node_placement || !mat->E || !mat->nu || !mat->eta) {
        set_error("empty mesh or missing array");
        return TF_BAD_INPUT;
    }
    if ((int64_t)m->n_nodes * 3 > INT32_MAX / 2 || (int64_t)m->n_elems * 36 > INT32_MAX) {
        set_error("mesh exceeds the 32-bit index range of the library");
        return TF_BAD_INPUT;
    }
    for (int64_t k = 0; k < 6 * (int64_t)m->n_elems; ++k)
        if (m->conn[k] < 0 || m->conn[k] >= m->n_nodes) {
            set_error("connectivity entry " + std::to_string(k) + " is out of range");
            return TF_BAD_INPUT;
        }
    for (int64_t k = 0; k < 3 * (int64_t)m->n_nodes; ++k)
        if (!std::isfinite(m->node_pos[k])) {
            set_error("non-finite node position");
            return TF_NAN_DETECTED;
        }
    return TF_OK;
}

tf_status sync(tf_handle* h) {
    TF_CUDA(cudaStreamSynchronize(h->stream));
    return TF_OK;
}

}  // namespace

void set_error(const std::string& msg) { g_last_error = msg; }

tf_status cuda_fail(cudaError_t e, const char* what) {
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return TF_CUDA_ERROR;
}


// Meshes from this many nodes on use the multigrid preconditioner by default.
constexpr int kAutoMultigridNodes = 20000;
// Time steps the multigrid's coarse levels are kept for by default.
constexpr int kDefaultMultigridReuse = 4;

tf_status create_handle(const tf_mesh* mesh, const tf_material* mat, const tf_options* opts,
                        const std::vector<int>& seg_node0, const std::vector<int>& seg_elem0, tf_handle** out) {
    if (opts && (opts->precond < 0 || opts->precond > 3 || opts->krylov_method < 0 || opts->krylov_method > 2)) {
        set_error("tf_options: precond must be 0..3 and krylov_method 0..2");
        return TF_BAD_INPUT;
    }
    tf_handle* h = new tf_handle;
    if (opts) h->opt = *opts;
    if (h->opt.newton_tol <= 0) h->opt.newton_tol = 1e-8;
    if (h->opt.newton_max_iter <= 0) h->opt.newton_max_iter = 20;
    // coarse levels kept across time steps: on the 320,000-prism sheet a step
    // with kept levels takes ~3 ms less (no Galerkin products, prolongator
    // smoothing or power iterations) with the same Krylov counts to +-1
    if (h->opt.multigrid_reuse_steps == 0) h->opt.multigrid_reuse_steps = kDefaultMultigridReuse;
    else if (h->opt.multigrid_reuse_steps < 0) h->opt.multigrid_reuse_steps = 0;
    if (h->opt.krylov_rtol <= 0) h->opt.krylov_rtol = 1e-8;
    if (h->opt.krylov_max_iter <= 0) h->opt.krylov_max_iter = 20000;
    if (h->opt.update_atol == 0.0) h->opt.update_atol = 1e-4 * h->opt.newton_tol;
    if (h->opt.update_atol < 0.0) h->opt.update_atol = 0.0;
    h->device = h->opt.device;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= h->device) {
        cudaGetLastError();
        delete h;
        set_error("no CUDA device available");
        return TF_NO_DEVICE;
    }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, h->device) != cudaSuccess || prop.major != 10 || prop.minor != 3) {
        delete h;
        set_error("this library is built for sm_103 (GB300) only");
        return TF_NO_DEVICE;
    }
    cudaError_t e = cudaSetDevice(h->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    for (auto& ev : h->ev)
        if (e == cudaSuccess) e = cudaEventCreate(&ev);
    if (e != cudaSuccess) {
        tf_status s = cuda_fail(e, "stream/event creation");
        free_all(h);
        delete h;
        return s;
    }
    tf_status s = build(h, mesh, mat, seg_node0, seg_elem0);
    const bool amg = h->opt.precond >= 2 || (h->opt.precond == 0 && mesh->n_nodes >= kAutoMultigridNodes);
    if (s == TF_OK && amg) s = amg_build(h, mesh->node_pos);
    if (s != TF_OK) {
        free_all(h);
        delete h;
        return s;
    }
    *out = h;
    return TF_OK;
}

// Newton loop of updateStepNR (Simulation.cpp:6449-6590) over every
// instance of the handle: an instance leaves the loop once |du| <= tol or
// after max_iter+1 solves; the others continue.  Per-instance iteration
// counts and convergence go to iters / conv (may be NULL).
tf_status newton_run(tf_handle* h, double dt, tf_step_stats* stats, int32_t* iters, int32_t* conv) {
    NvtxRange nvtx_range("tf newton step");
    Device& d = h->d;
    tf_step_stats st;
    std::memset(&st, 0, sizeof(st));
    TF_CUDA(cudaEventRecord(h->ev[0], h->stream));
    TF_TRY(tf_begin_step(h, dt));
    std::vector<int> it(d.nseg, 0), cv(d.nseg, 0), capped(d.nseg, 0);
    std::vector<double> du2(d.nseg);
    float ms_asm = 0.f;
    int k = 0;
    bool device_tried = false;
    bool assembled_tight = false;  // the device loop handed back an assembled iteration to solve tightly
    while (true) {
        TF_CUDA(cudaEventRecord(h->ev[2], h->stream));
        if (!assembled_tight) TF_TRY(tf_assemble(h));
        TF_CUDA(cudaEventRecord(h->ev[3], h->stream));
        int kit = 0;
        double rr = 0.0;
        h->solve_atol = assembled_tight ? 0.0 : h->opt.update_atol;
        h->newton_index = k;
        const long rebuilds0 = amg_rebuilds(h);
        tf_status s = tf_solve(h, &kit, &rr);
        h->solve_atol = 0.0;
        h->newton_index = -1;
        if (amg_rebuilds(h) != rebuilds0) {  // this solve rebuilt the coarse levels
            h->mg_kept = 0;
            h->mg_ref_iters = k == 0 ? kit : -1;
        } else if (k == 0 && h->opt.multigrid_reuse_steps > 0 && h->mg_ref_iters >= 0 &&
                   4 * kit > 5 * h->mg_ref_iters + 8) {
            h->mg_force = true;  // the kept levels have aged: rebuild at the next step
        }
        assembled_tight = false;
        if (s != TF_OK && s != TF_KRYLOV_NOT_CONVERGED) return s;
        float ms = 0.f;
        TF_CUDA(cudaEventElapsedTime(&ms, h->ev[2], h->ev[3]));
        ms_asm += ms;
        st.krylov_iters_total += kit;
        st.krylov_iters_max = std::max(st.krylov_iters_max, kit);
        // |du| before the update is applied.  An inexact solve must not decide
        // the Newton test: when a solve stopped at the update accuracy (a stop
        // test looser than krylov_rtol) and |du| lands near newton_tol
        // (near_newton_tol), the active instances are solved again to krylov_rtol.
        TF_TRY(launch_update_norm(h));
        TF_CUDA(cudaMemcpy2DAsync(du2.data(), sizeof(double), d.scal + S_DU2, sizeof(double) * S_COUNT,
                                  sizeof(double), d.nseg, cudaMemcpyDeviceToHost, h->stream));
        TF_TRY(sync(h));
        if (h->opt.update_atol > 0.0) {
            const double rt2 = h->opt.krylov_rtol * h->opt.krylov_rtol;
            bool redo = false;
            for (int g = 0; g < d.nseg && !redo; ++g) {
                if (!h->h_active[g]) continue;
                const double dn = std::sqrt(du2[g]);
                redo = d.host_scal[(size_t)g * S_COUNT + S_TOL2] > rt2 &&
                       near_newton_tol(dn, h->opt.newton_tol, h->opt.update_atol);
            }
            if (redo) {
                int kit2 = 0;
                s = tf_solve(h, &kit2, &rr);
                if (s != TF_OK && s != TF_KRYLOV_NOT_CONVERGED) return s;
                st.krylov_iters_total += kit2;
                st.final_relres = rr;
                TF_TRY(launch_update_norm(h));
                TF_CUDA(cudaMemcpy2DAsync(du2.data(), sizeof(double), d.scal + S_DU2, sizeof(double) * S_COUNT,
                                          sizeof(double), d.nseg, cudaMemcpyDeviceToHost, h->stream));
                TF_TRY(sync(h));
            }
        }
        if (k == 0) {  // the start of the next step's first solve
            if (!h->du0) TF_CUDA(cudaMalloc(&h->du0, sizeof(double) * 3 * (size_t)d.nn));
            TF_CUDA(cudaMemcpyAsync(h->du0, d.du, sizeof(double) * 3 * (size_t)d.nn, cudaMemcpyDeviceToDevice,
                                    h->stream));
            h->have_du0 = true;
        }
        TF_TRY(launch_update(h));
        double dmax = 0.0;
        bool any_active = false;
        for (int g = 0; g < d.nseg; ++g) {
            if (!h->h_active[g]) continue;
            const double dn = std::sqrt(du2[g]);
            if (!std::isfinite(dn)) return set_error("non-finite Newton update"), TF_NAN_DETECTED;
            dmax = std::max(dmax, dn);
            ++it[g];
            if (!(dn > h->opt.newton_tol)) {
                cv[g] = 1;
                h->h_active[g] = 0;
            } else if (it[g] > h->opt.newton_max_iter) {
                capped[g] = 1;
                h->h_active[g] = 0;
            } else {
                any_active = true;
            }
        }
        if (k < 32) st.dunorm[k] = dmax;
        ++k;
        if (!any_active) break;
        TF_CUDA(cudaMemcpyAsync(d.seg_active, h->h_active.data(), sizeof(int) * (size_t)d.nseg,
                                cudaMemcpyHostToDevice, h->stream));
        if (!device_tried) {
            // the rest of the step's iterations as one graph on the device; an
            // iteration it hands back (exc) continues on this host path
            device_tried = true;
            bool ran = false, exc = false;
            TF_TRY(newton_device_loop(h, it.data(), cv.data(), capped.data(), &k, &st, &ms_asm, &ran, &exc));
            if (ran && !exc) break;
            // handed back because a loosened solve's |du| came near newton_tol:
            // the iteration's assembly is in place, only its solve is redone
            if (ran && st.device_handback == 1) assembled_tight = true;
        }
    }
    std::fill(h->h_active.begin(), h->h_active.end(), 1);
    TF_CUDA(cudaMemcpyAsync(d.seg_active, h->h_active.data(), sizeof(int) * (size_t)d.nseg, cudaMemcpyHostToDevice,
                            h->stream));
    TF_TRY(tf_end_step(h));
    TF_CUDA(cudaEventRecord(h->ev[1], h->stream));
    TF_TRY(sync(h));
    float total = 0.f;
    TF_CUDA(cudaEventElapsedTime(&total, h->ev[0], h->ev[1]));
    int ncap = 0;
    for (int g = 0; g < d.nseg; ++g) {
        ncap += capped[g];
        if (iters) iters[g] = it[g];
        if (conv) conv[g] = cv[g];
    }
    st.newton_iters = k;
    st.converged = ncap == 0 ? 1 : 0;
    st.ms_assemble = ms_asm;
    st.ms_total = total;
    st.ms_solve = total - ms_asm;
    if (stats) *stats = st;
    if (ncap) {
        set_error("Newton iteration reached its cap without |du| <= tol in " + std::to_string(ncap) + " instance(s)");
        return TF_NOT_CONVERGED;
    }
    return TF_OK;
}

// val[off[k]] += v[k]: K entries added at node pairs of the element pattern
__global__ void k_add_entries(int n, const int* __restrict__ off, const double* __restrict__ v,
                              double* __restrict__ val) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) atomicAdd(&val[off[k]], v[k]);
}

// Checked build: a failed index check of the last kernels becomes
// TF_CUDA_ERROR (with the site) and the word is cleared; a no-op otherwise.
tf_status take_check(tf_handle* h) {
#ifdef TF_CHECKED
    int code = 0;
    TF_CUDA(cudaMemcpyAsync(&code, h->d.check, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    TF_CUDA(cudaStreamSynchronize(h->stream));
    if (code == 0) return TF_OK;
    TF_CUDA(cudaMemset(h->d.check, 0, sizeof(int)));
    static const char* site[] = {"", "prism node id", "element scatter offset", "Krylov product column",
                                 "extra block column", "level-0 smoother column", "restriction row",
                                 "prolongation column", "packing couple node", "packing extra block"};
    set_error(std::string("index check failed: ") + (code > 0 && code < 10 ? site[code] : "unknown site"));
    return TF_CUDA_ERROR;
#else
    (void)h;
    return TF_OK;
#endif
}

// The extra-block values of the current assembly back to the host copy
// (needed before a host-side change or read when the device wrote some of
// them: the packing Jacobian, the bound-DOF merges).
tf_status sync_extra_to_host(tf_handle* h) {
    if (h->d.nxb == 0 || (!h->pk && !h->bound_applied)) return TF_OK;
    TF_CUDA(cudaMemcpyAsync(h->h_xval.data(), h->d.xval, sizeof(double) * 9 * (size_t)h->d.nxb,
                            cudaMemcpyDeviceToHost, h->stream));
    return sync(h);
}

// Adds block (J, I) to the user's extra pattern (kept apart from the
// packing blocks, which change every step).
void note_user_block(tf_handle* h, int J, int I) {
    if (h->h_xuser.empty()) h->h_xuser.resize(h->d.nn);
    std::vector<int>& xu = h->h_xuser[J];
    auto it = std::lower_bound(xu.begin(), xu.end(), I);
    if (it == xu.end() || *it != I) xu.insert(it, I);
}

// Re-uploads the extra blocks (pattern and values) after a change.
tf_status upload_extra(tf_handle* h, bool pattern_changed) {
    Device& d = h->d;
    if (pattern_changed) {
        cudaFree(d.xrow);
        cudaFree(d.xcol);
        cudaFree(d.xval);
        d.xrow = d.xcol = nullptr;
        d.xval = nullptr;
        std::vector<int> col;
        h->h_xrow.assign(d.nn + 1, 0);
        for (int i = 0; i < d.nn; ++i) {
            col.insert(col.end(), h->h_xcols[i].begin(), h->h_xcols[i].end());
            h->h_xrow[i + 1] = static_cast<int>(col.size());
        }
        d.nxb = static_cast<int64_t>(col.size());
        TF_TRY(upload(&d.xrow, h->h_xrow));
        TF_TRY(upload(&d.xcol, col));
        TF_TRY(dev_alloc(&d.xval, 9 * (size_t)d.nxb));
        destroy_graphs(h);  // the captured Krylov chunks hold the extra-block pointers
        TF_TRY(packing_relink(h));
        h->extra_version++;
        amg_mark_stale(h, 2);  // the coarse images of the extra blocks follow the new layout
    }
    TF_CUDA(cudaMemcpyAsync(d.xval, h->h_xval.data(), sizeof(double) * 9 * (size_t)d.nxb, cudaMemcpyHostToDevice,
                            h->stream));
    return sync(h);
}

// ---- bound DOFs ------------------------------------------------------------
//
// K_bound = N^T K N + I, g_bound = N^T g couple by couple, as
// NewtonRaphsonSolver::calculateBoundKWithSlavesMasterDoF
// (NewtonRaphsonSolver.cpp:154-235) does on its dense K: g[m] += g[s],
// g[s] = 0; the slave row is added to the master row and zeroed, then the
// slave column to the master column, then K(s, s) = 1.  In A = K^T a row of
// K is a column of A.
//
// Which entries move where depends only on the couples and the block
// pattern, so the host turns the couples into a device program once (a
// "plan"): per couple three waves -- the moves of the column merge, the
// moves of the row merge, the unit diagonal -- each a list of entry
// addresses.  Every entry of the blocks in the involved rows and columns is
// moved (moving a zero adds nothing), so the blocks a merge can create
// outside the element pattern are known up front and join the extra blocks
// once.  One CTA runs the waves in order with a barrier between them; within
// a wave the sources and destinations are disjoint and every destination has
// one source, so its moves are independent.  The plan is rebuilt when the
// couples or the extra-block layout change; a solve with bindings then does
// no host transfer and no allocation.

struct BindPlan {
    int ncouple = 0;
    int nwave = 0;
    int64_t nop = 0;
    int64_t* dst = nullptr;   // entry addresses: >= 0 pattern value offset, < 0: -(1 + extra value index)
    int64_t* src = nullptr;   // kSetOne: the destination is set to 1
    int* wave = nullptr;      // [nwave + 1] op ranges
    int* slave = nullptr;     // [ncouple] DOFs
    int* master = nullptr;
    int64_t extra_version = -1;
};

constexpr int64_t kSetOne = INT64_MIN;

void bind_free(tf_handle* h) {
    if (!h->bind) return;
    cudaFree(h->bind->dst);
    cudaFree(h->bind->src);
    cudaFree(h->bind->wave);
    cudaFree(h->bind->slave);
    cudaFree(h->bind->master);
    delete h->bind;
    h->bind = nullptr;
}

__device__ __forceinline__ double* bind_entry(int64_t a, double* val, double* xval) {
    return a >= 0 ? val + a : xval + (-1 - a);
}

// The merges of all couples, in their order (one CTA; the first thread also
// merges the right-hand side, couple by couple).
__global__ void __launch_bounds__(1024) k_bind_apply(int ncouple, const int* __restrict__ slave,
                                                     const int* __restrict__ master, int nwave,
                                                     const int* __restrict__ wave, const int64_t* __restrict__ dst,
                                                     const int64_t* __restrict__ src, double* val, double* xval,
                                                     double* g) {
    if (threadIdx.x == 0)
        for (int k = 0; k < ncouple; ++k) {
            g[master[k]] += g[slave[k]];
            g[slave[k]] = 0.0;
        }
    for (int w = 0; w < nwave; ++w) {
        for (int q = wave[w] + threadIdx.x; q < wave[w + 1]; q += blockDim.x) {
            double* d = bind_entry(dst[q], val, xval);
            if (src[q] == kSetOne) {
                *d = 1.0;
            } else {
                double* sp = bind_entry(src[q], val, xval);
                *d += *sp;
                *sp = 0.0;
            }
        }
        __syncthreads();
    }
}

// du[slave] = du[master], couple by couple in their order
// (NewtonRaphsonSolver::equateSlaveDisplacementsToMasters, NewtonRaphsonSolver.cpp:237-251)
__global__ void k_equate(int n, const int* __restrict__ slave, const int* __restrict__ master, double* du) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    for (int k = 0; k < n; ++k) du[slave[k]] = du[master[k]];
}

// Builds the plan for the current couples and extra-block layout.
tf_status bind_build(tf_handle* h) {
    Device& d = h->d;
    bind_free(h);
    const int nc = static_cast<int>(h->bind_slave.size());
    using Key = std::pair<int, int>;  // block (J, I) of A
    auto find_block = [&](int r, int c) -> int64_t {
        auto b = h->h_colidx.begin() + h->h_rowptr[r], en = h->h_colidx.begin() + h->h_rowptr[r + 1];
        auto it = std::lower_bound(b, en, c);
        return (it != en && *it == c) ? static_cast<int64_t>(it - h->h_colidx.begin()) : -1;
    };
    // the blocks in the rows and columns of the involved nodes
    std::vector<char> involved(d.nn, 0);
    for (int k = 0; k < nc; ++k) {
        involved[h->bind_slave[k] / 3] = 1;
        involved[h->bind_master[k] / 3] = 1;
    }
    std::set<Key> keys;
    for (int X = 0; X < d.nn; ++X) {
        if (!involved[X]) continue;
        for (int p = h->h_rowptr[X]; p < h->h_rowptr[X + 1]; ++p) {
            keys.insert({X, h->h_colidx[p]});
            keys.insert({h->h_colidx[p], X});
        }
    }
    if (!h->h_xcols.empty())
        for (int J = 0; J < d.nn; ++J)
            for (int I : h->h_xcols[J])
                if (involved[J] || involved[I]) keys.insert({J, I});
    // symbolic pass: the blocks the merges reach
    struct Move {
        Key dk, sk;
        int de, se;  // entries 3 r + c within the blocks; se < 0: set to one
    };
    std::vector<std::vector<Move>> waves;
    for (int k = 0; k < nc; ++k) {
        const int sd = h->bind_slave[k], md = h->bind_master[k];
        const int S = sd / 3, M = md / 3, ds = sd % 3, dm = md % 3;
        // K row m += K row s: column S of A into column M
        std::vector<Move> wa, wb;
        std::vector<Key> colS, rowS;
        for (const Key& key : keys)
            if (key.second == S) colS.push_back(key);
        for (const Key& key : colS)
            for (int dc = 0; dc < 3; ++dc) wa.push_back({{key.first, M}, key, 3 * dc + dm, 3 * dc + ds});
        for (const Move& m : wa) keys.insert(m.dk);
        // K column m += K column s: row S of A into row M
        for (const Key& key : keys)
            if (key.first == S) rowS.push_back(key);
        for (const Key& key : rowS)
            for (int dr = 0; dr < 3; ++dr) wb.push_back({{M, key.second}, key, 3 * dm + dr, 3 * ds + dr});
        for (const Move& m : wb) keys.insert(m.dk);
        keys.insert({S, S});
        waves.push_back(std::move(wa));
        waves.push_back(std::move(wb));
        waves.push_back({Move{{S, S}, {S, S}, 3 * ds + ds, -1}});
    }
    // blocks outside the element pattern join the extra blocks (values kept)
    bool changed = false;
    for (const Key& key : keys) {
        if (find_block(key.first, key.second) >= 0) continue;
        if (h->h_xcols.empty()) h->h_xcols.resize(d.nn);
        std::vector<int>& xc = h->h_xcols[key.first];
        auto jt = std::lower_bound(xc.begin(), xc.end(), key.second);
        if (jt != xc.end() && *jt == key.second) continue;
        if (!changed) TF_TRY(sync_extra_to_host(h));
        note_user_block(h, key.first, key.second);
        xc.insert(jt, key.second);
        changed = true;
    }
    if (changed) {
        std::vector<int> row(d.nn + 1, 0);
        for (int i = 0; i < d.nn; ++i) row[i + 1] = row[i] + static_cast<int>(h->h_xcols[i].size());
        std::vector<double> nv(9 * (size_t)row[d.nn], 0.0);
        if (!h->h_xrow.empty())
            for (int i = 0; i < d.nn; ++i)
                for (int p = h->h_xrow[i]; p < h->h_xrow[i + 1]; ++p) {
                    const auto& xc = h->h_xcols[i];
                    const int q = row[i] + static_cast<int>(std::lower_bound(xc.begin(), xc.end(),
                                                                             h->h_xcol_prev[p]) - xc.begin());
                    for (int t = 0; t < 9; ++t) nv[9 * (size_t)q + t] = h->h_xval[9 * (size_t)p + t];
                }
        h->h_xval.swap(nv);
        h->h_xcol_prev.clear();
        for (const auto& xc : h->h_xcols) h->h_xcol_prev.insert(h->h_xcol_prev.end(), xc.begin(), xc.end());
        TF_TRY(upload_extra(h, true));
    }
    // entry addresses
    auto addr = [&](const Key& key, int e) -> int64_t {
        const int64_t b = find_block(key.first, key.second);
        const int r = e / 3, c = e - 3 * (e / 3);
        if (b >= 0) return static_cast<int64_t>(h->h_bofs[b]) + kSlice * (3 * r + c);
        const auto& xc = h->h_xcols[key.first];
        const int q = h->h_xrow[key.first] + static_cast<int>(std::lower_bound(xc.begin(), xc.end(), key.second) -
                                                              xc.begin());
        return -1 - (9 * static_cast<int64_t>(q) + e);
    };
    std::vector<int64_t> vdst, vsrc;
    std::vector<int> vwave{0};
    for (const auto& w : waves) {
        for (const Move& m : w) {
            vdst.push_back(addr(m.dk, m.de));
            vsrc.push_back(m.se < 0 ? kSetOne : addr(m.sk, m.se));
        }
        vwave.push_back(static_cast<int>(vdst.size()));
    }
    BindPlan* P = new BindPlan;
    h->bind = P;
    P->ncouple = nc;
    P->nwave = static_cast<int>(waves.size());
    P->nop = static_cast<int64_t>(vdst.size());
    if (P->nop > 0) {
        TF_TRY(upload(&P->dst, vdst));
        TF_TRY(upload(&P->src, vsrc));
    }
    TF_TRY(upload(&P->wave, vwave));
    TF_TRY(upload(&P->slave, h->bind_slave));
    TF_TRY(upload(&P->master, h->bind_master));
    P->extra_version = h->extra_version;
    return TF_OK;
}

tf_status apply_bindings(tf_handle* h) {
    if (!h->bind || h->bind->extra_version != h->extra_version) TF_TRY(bind_build(h));
    const BindPlan& P = *h->bind;
    const Device& d = h->d;
    k_bind_apply<<<1, 1024, 0, h->stream>>>(P.ncouple, P.slave, P.master, P.nwave, P.wave, P.dst, P.src, d.val,
                                            d.xval, d.g);
    TF_LAUNCH_CHECK(h);
    h->bound_applied = true;
    amg_mark_stale(h, 1);
    return TF_OK;
}

tf_status equate_bound(tf_handle* h) {
    const BindPlan& P = *h->bind;
    k_equate<<<1, 1, 0, h->stream>>>(P.ncouple, P.slave, P.master, h->d.du);
    TF_LAUNCH_CHECK(h);
    return TF_OK;
}

}  // namespace tf

using namespace tf;

extern "C" {

tf_status tf_set_packing(tf_handle* h, int32_t enable, int32_t flags) {
    TF_TRY(check_handle(h));
    if (flags & ~1) return set_error("tf_set_packing: unknown flags"), TF_BAD_INPUT;
    if (h->d.nseg != 1) return set_error("tf_set_packing: packing works on single-mesh handles"), TF_BAD_INPUT;
    TF_CUDA(cudaSetDevice(h->device));
    TF_CUDA(cudaStreamSynchronize(h->stream));
    if (h->pk) {
        packing_free(h->pk);
        h->pk = nullptr;
    }
    if (enable) {
        const tf_status s = packing_setup(h, flags);
        if (s != TF_OK) {
            packing_free(h->pk);
            h->pk = nullptr;
            return s;
        }
    } else if (!h->h_xuser.empty() || !h->h_xcols.empty()) {
        // back to the user's extra blocks only
        if (h->h_xuser.empty()) h->h_xuser.resize(h->d.nn);
        h->h_xcols = h->h_xuser;
        int64_t nxb = 0;
        for (const auto& xc : h->h_xcols) nxb += (int64_t)xc.size();
        h->h_xval.assign(9 * (size_t)nxb, 0.0);
        h->h_xcol_prev.clear();
        for (const auto& xc : h->h_xcols) h->h_xcol_prev.insert(h->h_xcol_prev.end(), xc.begin(), xc.end());
        TF_TRY(upload_extra(h, true));
    }
    return TF_OK;
}

tf_status tf_get_packing(tf_handle* h, int64_t* n, int32_t* nodes, double* weights, double* mbar, double* threshold,
                         double* detect_distance) {
    TF_TRY(check_handle(h));
    if (!n) return set_error("tf_get_packing: n is required"), TF_BAD_INPUT;
    TF_CUDA(cudaSetDevice(h->device));
    return packing_get(h, n, nodes, weights, mbar, threshold, detect_distance);
}

tf_status tf_packing_masses(tf_handle* h, double* mass) {
    TF_TRY(check_handle(h));
    if (!mass) return set_error("tf_packing_masses: bad arguments"), TF_BAD_INPUT;
    TF_CUDA(cudaSetDevice(h->device));
    return packing_masses(h, mass);
}

namespace {

// Common checks of the tf_add_*_growth calls; sets the growth tables up at
// the first function.
tf_status growth_prologue(tf_handle* h, const char* what, const double* rates, double t0, double t1, double zmin,
                          double zmax) {
    TF_TRY(check_handle(h));
    const std::string w(what);
    if (h->d.nseg != 1) return set_error(w + ": growth functions work on single-mesh handles"), TF_BAD_INPUT;
    if (!rates) return set_error(w + ": null rates"), TF_BAD_INPUT;
    if (std::isnan(t0) || std::isnan(t1) || !std::isfinite(zmin) || !std::isfinite(zmax))
        return set_error(w + ": bad time window or z range"), TF_BAD_INPUT;
    if (growth_count(h) >= kMaxGrowthFunctions)
        return set_error(w + ": at most 16 growth functions per handle"), TF_BAD_INPUT;
    TF_CUDA(cudaStreamSynchronize(h->stream));
    if (!h->growth) {
        const tf_status s = growth_setup(h);
        if (s != TF_OK) {
            growth_free(h->growth);
            h->growth = nullptr;
            return s;
        }
    }
    return TF_OK;
}

bool all_finite(const double* v, int64_t n) {
    for (int64_t k = 0; k < n; ++k)
        if (!std::isfinite(v[k])) return false;
    return true;
}

}  // namespace

tf_status tf_add_uniform_growth(tf_handle* h, const double* rates, double angle_rad, double init_time,
                                double end_time, double zmin, double zmax) {
    TF_TRY(growth_prologue(h, "tf_add_uniform_growth", rates, init_time, end_time, zmin, zmax));
    if (!all_finite(rates, 3) || !std::isfinite(angle_rad))
        return set_error("tf_add_uniform_growth: non-finite rate or angle"), TF_BAD_INPUT;
    return growth_add_uniform(h, rates, angle_rad, init_time, end_time, zmin, zmax);
}

tf_status tf_add_ring_growth(tf_handle* h, double centre_x, double centre_y, double inner_radius,
                             double outer_radius, const double* rates, double angle_rad, double init_time,
                             double end_time, double zmin, double zmax) {
    TF_TRY(growth_prologue(h, "tf_add_ring_growth", rates, init_time, end_time, zmin, zmax));
    if (!all_finite(rates, 3) || !std::isfinite(angle_rad) || !std::isfinite(centre_x) || !std::isfinite(centre_y) ||
        !(inner_radius >= 0.0) || !(outer_radius > inner_radius) || !std::isfinite(outer_radius))
        return set_error("tf_add_ring_growth: needs finite values and 0 <= inner radius < outer radius"),
               TF_BAD_INPUT;
    return growth_add_ring(h, centre_x, centre_y, inner_radius, outer_radius, rates, angle_rad, init_time, end_time,
                           zmin, zmax);
}

tf_status tf_add_grid_growth(tf_handle* h, int32_t nx, int32_t ny, const double* rates, const double* angles_deg,
                             double init_time, double end_time, double zmin, double zmax) {
    if (nx < 2 || ny < 2 || (int64_t)nx * ny > (1 << 24))
        return set_error("tf_add_grid_growth: needs a grid of at least 2 x 2 points"), TF_BAD_INPUT;
    if (rates && !all_finite(rates, 3 * (int64_t)nx * ny))
        return set_error("tf_add_grid_growth: non-finite rate"), TF_BAD_INPUT;
    if (angles_deg && !all_finite(angles_deg, (int64_t)nx * ny))
        return set_error("tf_add_grid_growth: non-finite angle"), TF_BAD_INPUT;
    TF_TRY(growth_prologue(h, "tf_add_grid_growth", rates, init_time, end_time, zmin, zmax));
    return growth_add_grid(h, nx, ny, rates, angles_deg, init_time, end_time, zmin, zmax);
}

tf_status tf_clear_growth_functions(tf_handle* h) {
    TF_TRY(check_handle(h));
    TF_CUDA(cudaStreamSynchronize(h->stream));
    growth_clear(h);
    return TF_OK;
}

tf_status tf_set_grid_growth_mode(tf_handle* h, int32_t interpolation, int32_t pinned_on_initial_mesh) {
    TF_TRY(check_handle(h));
    if ((interpolation != 0 && interpolation != 1) || (pinned_on_initial_mesh != 0 && pinned_on_initial_mesh != 1))
        return set_error("tf_set_grid_growth_mode: interpolation and pinning are 0 or 1"), TF_BAD_INPUT;
    if (!h->growth) return set_error("tf_set_grid_growth_mode: no growth function added"), TF_BAD_INPUT;
    growth_set_mode(h, interpolation, pinned_on_initial_mesh);
    return TF_OK;
}

tf_status tf_repin_grid_growth(tf_handle* h) {
    TF_TRY(check_handle(h));
    if (!h->growth) return set_error("tf_repin_grid_growth: no growth function added"), TF_BAD_INPUT;
    TF_CUDA(cudaSetDevice(h->device));
    TF_TRY(growth_repin(h));
    return sync(h);
}

tf_status tf_grid_growth_positions(tf_handle* h, double* rel_z, double* rel_pinned, double* rel_current) {
    TF_TRY(check_handle(h));
    if (!h->growth) return set_error("tf_grid_growth_positions: no growth function added"), TF_BAD_INPUT;
    TF_CUDA(cudaSetDevice(h->device));
    return growth_positions(h, rel_z, rel_pinned, rel_current);
}

tf_status tf_set_time(tf_handle* h, double time_sec) {
    TF_TRY(check_handle(h));
    if (std::isnan(time_sec)) return set_error("tf_set_time: NaN time"), TF_BAD_INPUT;
    h->time = time_sec;
    return TF_OK;
}

tf_status tf_get_time(tf_handle* h, double* time_sec) {
    TF_TRY(check_handle(h));
    if (!time_sec) return set_error("tf_get_time: null output"), TF_BAD_INPUT;
    *time_sec = h->time;
    return TF_OK;
}

tf_status tf_set_dof_bindings(tf_handle* h, int32_t n, const int32_t* slave_dofs, const int32_t* master_dofs) {
    TF_TRY(check_handle(h));
    if (n < 0 || (n > 0 && (!slave_dofs || !master_dofs))) return set_error("tf_set_dof_bindings: bad arguments"), TF_BAD_INPUT;
    const int64_t n3 = 3 * (int64_t)h->d.nn;
    for (int k = 0; k < n; ++k)
        if (slave_dofs[k] < 0 || slave_dofs[k] >= n3 || master_dofs[k] < 0 || master_dofs[k] >= n3 ||
            slave_dofs[k] == master_dofs[k])
            return set_error("tf_set_dof_bindings: couple " + std::to_string(k) + " is invalid"), TF_BAD_INPUT;
    h->bind_slave.assign(slave_dofs, slave_dofs + n);
    h->bind_master.assign(master_dofs, master_dofs + n);
    h->bound_applied = false;
    bind_free(h);
    amg_mark_stale(h, 2);  // a new operator: no kept coarse levels
    return TF_OK;
}


tf_status tf_add_K_triplets(tf_handle* h, int64_t n, const int32_t* rows, const int32_t* cols, const double* vals) {
    TF_TRY(check_handle(h));
    if (n < 0 || (n > 0 && (!rows || !cols || !vals))) return set_error("tf_add_K_triplets: bad arguments"), TF_BAD_INPUT;
    if (!h->assembled) return set_error("tf_add_K_triplets called before tf_assemble"), TF_BAD_INPUT;
    Device& d = h->d;
    const int64_t n3 = 3 * (int64_t)d.nn;
    if (h->h_xcols.empty()) h->h_xcols.resize(d.nn);
    TF_TRY(sync_extra_to_host(h));
    std::vector<int> off;
    std::vector<double> v;
    struct Pending {
        int J, I, e;
        double v;
    };
    std::vector<Pending> extra;
    bool changed = false;
    for (int64_t k = 0; k < n; ++k) {
        const int64_t r = rows[k], c = cols[k];
        if (r < 0 || r >= n3 || c < 0 || c >= n3)
            return set_error("tf_add_K_triplets: entry " + std::to_string(k) + " is out of range"), TF_BAD_INPUT;
        if (h->h_fixed[r] || h->h_fixed[c]) continue;  // calcutateFixedK runs after these writers
        // K(r, c) is A(c, r): block (J, I) = (c/3, r/3), entry (c%3, r%3)
        const int J = static_cast<int>(c / 3), I = static_cast<int>(r / 3);
        const int e = static_cast<int>(3 * (c % 3) + (r % 3));
        auto b = h->h_colidx.begin() + h->h_rowptr[J], en = h->h_colidx.begin() + h->h_rowptr[J + 1];
        auto it = std::lower_bound(b, en, I);
        if (it != en && *it == I) {
            off.push_back(h->h_bofs[it - h->h_colidx.begin()] + kSlice * e);
            v.push_back(vals[k]);
        } else {
            note_user_block(h, J, I);
            std::vector<int>& xc = h->h_xcols[J];
            auto jt = std::lower_bound(xc.begin(), xc.end(), I);
            if (jt == xc.end() || *jt != I) {
                xc.insert(jt, I);
                changed = true;
            }
            extra.push_back({J, I, e, vals[k]});
        }
    }
    if (changed) {
        // new layout; the values accumulated so far in this assembly move with their blocks
        int64_t nxb = 0;
        for (const auto& xc : h->h_xcols) nxb += (int64_t)xc.size();
        std::vector<double> nv(9 * (size_t)nxb, 0.0);
        std::vector<int> row(d.nn + 1, 0);
        for (int i = 0; i < d.nn; ++i) row[i + 1] = row[i] + static_cast<int>(h->h_xcols[i].size());
        if (!h->h_xrow.empty())
            for (int i = 0; i < d.nn; ++i)
                for (int p = h->h_xrow[i]; p < h->h_xrow[i + 1]; ++p) {
                    const auto& xc = h->h_xcols[i];
                    const int q = row[i] + static_cast<int>(
                                               std::lower_bound(xc.begin(), xc.end(), h->h_xcol_prev[p]) - xc.begin());
                    for (int t = 0; t < 9; ++t) nv[9 * (size_t)q + t] = h->h_xval[9 * (size_t)p + t];
                }
        h->h_xval.swap(nv);
        h->h_xcol_prev.clear();
        for (const auto& xc : h->h_xcols) h->h_xcol_prev.insert(h->h_xcol_prev.end(), xc.begin(), xc.end());
    }
    if (!extra.empty() || changed) {
        std::vector<int> row(d.nn + 1, 0);
        for (int i = 0; i < d.nn; ++i) row[i + 1] = row[i] + static_cast<int>(h->h_xcols[i].size());
        for (const Pending& q : extra) {
            const auto& xc = h->h_xcols[q.J];
            const int p = row[q.J] + static_cast<int>(std::lower_bound(xc.begin(), xc.end(), q.I) - xc.begin());
            h->h_xval[9 * (size_t)p + q.e] += q.v;
        }
        TF_TRY(upload_extra(h, changed));
    }
    if (!off.empty()) {
        int* doff = nullptr;
        double* dv = nullptr;
        TF_TRY(upload(&doff, off));
        const tf_status s = upload(&dv, v);
        if (s != TF_OK) {
            cudaFree(doff);
            return s;
        }
        const int m = static_cast<int>(off.size());
        k_add_entries<<<cdiv(m, 256), 256, 0, h->stream>>>(m, doff, dv, d.val);
        const cudaError_t e1 = cudaGetLastError();
        const cudaError_t e2 = cudaStreamSynchronize(h->stream);
        cudaFree(doff);
        cudaFree(dv);
        if (e1 != cudaSuccess) return cuda_fail(e1, "k_add_entries");
        if (e2 != cudaSuccess) return cuda_fail(e2, "k_add_entries");
        h->launches++;
    }
    amg_mark_stale(h, 1);
    return TF_OK;
}


const char* tf_status_string(tf_status s) {
    switch (s) {
        case TF_OK: return "ok";
        case TF_NOT_CONVERGED: return "Newton iteration did not converge";
        case TF_KRYLOV_NOT_CONVERGED: return "linear solve did not converge";
        case TF_KRYLOV_BREAKDOWN: return "Krylov breakdown";
        case TF_NAN_DETECTED: return "non-finite value detected";
        case TF_BAD_INPUT: return "bad input";
        case TF_CUDA_ERROR: return "CUDA error";
        case TF_NO_DEVICE: return "no usable device";
        case TF_OUT_OF_MEMORY: return "out of device memory";
    }
    return "unknown status";
}

const char* tf_last_error(void) { return g_last_error.c_str(); }

tf_status tf_create(const tf_mesh* mesh, const tf_material* mat, const tf_options* opts, tf_handle** out) {
    if (!out) {
        set_error("null output handle");
        return TF_BAD_INPUT;
    }
    *out = nullptr;
    TF_TRY(validate(mesh, mat));
    return create_handle(mesh, mat, opts, {0, mesh->n_nodes}, {0, mesh->n_elems}, out);
}

tf_status tf_batch_create(const tf_mesh* meshes, const tf_material* mats, int32_t n, const tf_options* opts,
                          tf_handle** out) {
    if (!out || !meshes || !mats || n <= 0) {
        set_error("tf_batch_create: bad arguments");
        return TF_BAD_INPUT;
    }
    *out = nullptr;
    int64_t nn = 0, ne = 0;
    for (int i = 0; i < n; ++i) {
        const tf_status s = validate(&meshes[i], &mats[i]);
        if (s != TF_OK) {
            set_error("instance " + std::to_string(i) + ": " + g_last_error);
            return s;
        }
        nn += meshes[i].n_nodes;
        ne += meshes[i].n_elems;
    }
    if (nn * 3 > INT32_MAX / 2 || ne * 36 > INT32_MAX) {
        set_error("tf_batch_create: the batch exceeds the 32-bit index range of the library");
        return TF_BAD_INPUT;
    }
    std::vector<double> pos, ev, E, nu, eta, ref;
    std::vector<int32_t> conn, placement;
    std::vector<uint8_t> fixed;
    std::vector<int> node0{0}, elem0{0};
    pos.reserve(3 * nn);
    conn.reserve(6 * ne);
    bool any_ref = false;
    for (int i = 0; i < n; ++i) any_ref |= meshes[i].ref_pos != nullptr;
    for (int i = 0; i < n; ++i) {
        const tf_mesh& m = meshes[i];
        const int off = node0.back();
        if (any_ref) {
            for (int64_t e = 0; e < m.n_elems; ++e)
                for (int a = 0; a < 6; ++a)
                    for (int c = 0; c < 3; ++c)
                        ref.push_back(m.ref_pos ? m.ref_pos[18 * e + 3 * a + c]
                                                : m.node_pos[3 * (size_t)m.conn[6 * e + a] + c]);
        }
        pos.insert(pos.end(), m.node_pos, m.node_pos + 3 * (size_t)m.n_nodes);
        ev.insert(ev.end(), m.ext_visc, m.ext_visc + 3 * (size_t)m.n_nodes);
        fixed.insert(fixed.end(), m.fixed, m.fixed + 3 * (size_t)m.n_nodes);
        placement.insert(placement.end(), m.node_placement, m.node_placement + m.n_nodes);
        for (int64_t k = 0; k < 6 * (int64_t)m.n_elems; ++k) conn.push_back(m.conn[k] + off);
        E.insert(E.end(), mats[i].E, mats[i].E + m.n_elems);
        nu.insert(nu.end(), mats[i].nu, mats[i].nu + m.n_elems);
        eta.insert(eta.end(), mats[i].eta, mats[i].eta + m.n_elems);
        node0.push_back(off + m.n_nodes);
        elem0.push_back(elem0.back() + m.n_elems);
    }
    tf_mesh all{static_cast<int32_t>(nn), static_cast<int32_t>(ne), pos.data(), conn.data(), fixed.data(), ev.data(),
                placement.data(), any_ref ? ref.data() : nullptr};
    tf_material mat{E.data(), nu.data(), eta.data()};
    return create_handle(&all, &mat, opts, node0, elem0, out);
}

tf_status tf_batch_step(tf_handle* h, double dt, int32_t* newton_iters, int32_t* converged, tf_step_stats* stats) {
    TF_TRY(check_handle(h));
    return newton_run(h, dt, stats, newton_iters, converged);
}

tf_status tf_get_instances(tf_handle* h, int32_t* n_instances, int32_t* node_offsets, int32_t* elem_offsets) {
    if (!h) return set_error("null handle"), TF_BAD_INPUT;
    if (n_instances) *n_instances = h->d.nseg;
    for (int i = 0; i <= h->d.nseg; ++i) {
        if (node_offsets) node_offsets[i] = h->h_seg_node0[i];
        if (elem_offsets) elem_offsets[i] = h->h_seg_elem0[i];
    }
    return TF_OK;
}

int32_t tf_elements_per_cta(tf_handle* h) { return h ? h->elem_cta : 0; }

tf_status tf_solve_variants(tf_handle* h, int32_t* spmv_unroll, int32_t* smoother_unroll) {
    TF_TRY(check_handle(h));
    if (spmv_unroll) *spmv_unroll = h->spmv_unroll;
    if (smoother_unroll) *smoother_unroll = amg_smoother_unroll(h);
    return TF_OK;
}

tf_status tf_destroy(tf_handle* h) {
    if (!h) return TF_OK;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    free_all(h);
    delete h;
    return TF_OK;
}

tf_status tf_set_positions(tf_handle* h, const double* pos) {
    TF_TRY(check_handle(h));
    if (!pos) return set_error("null positions"), TF_BAD_INPUT;
    TF_CUDA(cudaMemcpyAsync(h->d.uk, pos, sizeof(double) * 3 * (size_t)h->d.nn, cudaMemcpyHostToDevice, h->stream));
    return sync(h);
}

tf_status tf_get_positions(tf_handle* h, double* pos) {
    TF_TRY(check_handle(h));
    if (!pos) return set_error("null positions"), TF_BAD_INPUT;
    TF_CUDA(cudaMemcpyAsync(pos, h->d.uk, sizeof(double) * 3 * (size_t)h->d.nn, cudaMemcpyDeviceToHost, h->stream));
    return sync(h);
}

tf_status tf_set_Fg(tf_handle* h, const double* Fg) {
    TF_TRY(check_handle(h));
    if (!Fg) return set_error("null Fg"), TF_BAD_INPUT;
    const int ne = h->d.ne;
    std::vector<double> f(9 * (size_t)ne), inv(9 * (size_t)ne);
    for (int e = 0; e < ne; ++e) {
        double M[9], I[9], det;
        for (int k = 0; k < 9; ++k) M[k] = Fg[9 * (size_t)e + k];
        if (!inverse3(M, I, &det)) {
            set_error("Fg of element " + std::to_string(e) + " is singular");
            return TF_BAD_INPUT;
        }
        for (int k = 0; k < 9; ++k) {
            f[(size_t)k * ne + e] = M[k];
            inv[(size_t)k * ne + e] = I[k];
        }
    }
    TF_CUDA(cudaMemcpyAsync(h->d.Fg, f.data(), f.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    TF_CUDA(cudaMemcpyAsync(h->d.invFg, inv.data(), inv.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    amg_mark_stale(h, 2);  // the tangent may differ from the kept coarse levels' by more than a step's change
    return sync(h);
}

tf_status tf_get_Fg(tf_handle* h, double* Fg, double* invFg) {
    TF_TRY(check_handle(h));
    const int ne = h->d.ne;
    std::vector<double> f(9 * (size_t)ne);
    for (int which = 0; which < 2; ++which) {
        double* out = which == 0 ? Fg : invFg;
        if (!out) continue;
        TF_CUDA(cudaMemcpyAsync(f.data(), which == 0 ? h->d.Fg : h->d.invFg, f.size() * sizeof(double),
                                cudaMemcpyDeviceToHost, h->stream));
        TF_TRY(sync(h));
        for (int e = 0; e < ne; ++e)
            for (int k = 0; k < 9; ++k) out[9 * (size_t)e + k] = f[(size_t)k * ne + e];
    }
    return TF_OK;
}

tf_status tf_set_growth_rates(tf_handle* h, const double* rates) {
    TF_TRY(check_handle(h));
    const int ne = h->d.ne;
    std::vector<double> r(3 * (size_t)ne, 0.0);
    h->have_rates = rates != nullptr;
    if (rates)
        for (int e = 0; e < ne; ++e)
            for (int d = 0; d < 3; ++d) r[(size_t)d * ne + e] = rates[3 * (size_t)e + d];
    TF_CUDA(cudaMemcpyAsync(h->d.rates, r.data(), r.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    return sync(h);
}

tf_status tf_begin_step(tf_handle* h, double dt) {
    NvtxRange nvtx_range("tf begin_step");
    TF_TRY(check_handle(h));
    if (!(dt > 0.0) || !std::isfinite(dt)) return set_error("dt must be positive"), TF_BAD_INPUT;
    h->dt = dt;
    // a new time step: rebuild the multigrid hierarchy at its first solve, or
    // keep its coarse levels for up to multigrid_reuse_steps steps (the
    // level-0 copies follow every assembly either way)
    const int keep = h->opt.multigrid_reuse_steps;
    if (keep > 0 && !h->mg_force && h->mg_kept < keep && h->mg_ref_iters >= 0) {
        amg_mark_stale(h, 1);
        ++h->mg_kept;
    } else {
        amg_mark_stale(h, 2);
        h->mg_force = false;
    }
    // calculateGrowth (Simulation.cpp:9651-9666): the per-element rates, then
    // the growth functions active at this time, in one increment per prism
    bool grown = false;
    TF_TRY(launch_growth_functions(h, &grown));
    if (!grown && h->have_rates) TF_TRY(launch_growth(h));
    h->in_step = true;
    TF_TRY(launch_viscosity_surfaces(h));
    TF_CUDA(cudaMemcpyAsync(h->d.un, h->d.uk, sizeof(double) * 3 * (size_t)h->d.nn, cudaMemcpyDeviceToDevice,
                            h->stream));
    h->assembled = false;
    if (h->pk) TF_TRY(packing_detect(h));  // runOneStep: detectPacingNodes after growth (Simulation.cpp:5920)
    return take_check(h);
}

tf_status tf_assemble(tf_handle* h) {
    NvtxRange nvtx_range("tf assemble");
    TF_TRY(check_handle(h));
    amg_mark_stale(h, 1);
    h->bound_applied = false;
    if (h->d.nxb > 0) {  // K entries added outside the element pattern belong to one assembly
        std::fill(h->h_xval.begin(), h->h_xval.end(), 0.0);
        TF_CUDA(cudaMemsetAsync(h->d.xval, 0, sizeof(double) * 9 * (size_t)h->d.nxb, h->stream));
    }
    TF_TRY(autotune_element(h));
    TF_TRY(launch_prepare(h));
    TF_TRY(launch_element(h));
    if (h->opt.deterministic) TF_TRY(launch_deterministic_gather(h));
    if (h->pk) TF_TRY(packing_assemble(h));  // after addImplicitKViscousExternalToJacobian (Simulation.cpp:6489-6493)
    TF_TRY(take_check(h));
    h->assembled = true;
    return TF_OK;
}

tf_status tf_add_external_forces(tf_handle* h, const double* gext) {
    TF_TRY(check_handle(h));
    if (!gext) return set_error("null forces"), TF_BAD_INPUT;
    const size_t n3 = 3 * (size_t)h->d.nn;
    std::vector<double> g(n3);
    TF_CUDA(cudaMemcpyAsync(g.data(), h->d.g, n3 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    TF_TRY(sync(h));
    for (size_t k = 0; k < n3; ++k)
        if (!h->h_fixed[k]) g[k] = g[k] + gext[k];
    TF_CUDA(cudaMemcpyAsync(h->d.g, g.data(), n3 * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    return sync(h);
}

tf_status tf_solve(tf_handle* h, int32_t* iters, double* relres) {
    NvtxRange nvtx_range("tf solve");
    TF_TRY(check_handle(h));
    if (!h->assembled) return set_error("tf_solve called before tf_assemble"), TF_BAD_INPUT;
    if (!h->bind_slave.empty() && !h->bound_applied) TF_TRY(apply_bindings(h));
    int it = 0;
    double rr = 0.0;
    tf_status s = krylov_solve(h, &it, &rr);
    TF_TRY(take_check(h));
    if (!h->bind_slave.empty() && (s == TF_OK || s == TF_KRYLOV_NOT_CONVERGED)) TF_TRY(equate_bound(h));
    if (iters) *iters = it;
    if (relres) *relres = rr;
    return s;
}

tf_status tf_update(tf_handle* h, int32_t* converged, double* dunorm) {
    TF_TRY(check_handle(h));
    TF_TRY(launch_update(h));
    Device& d = h->d;
    std::vector<double> du2(d.nseg);
    TF_CUDA(cudaMemcpy2DAsync(du2.data(), sizeof(double), d.scal + S_DU2, sizeof(double) * S_COUNT, sizeof(double),
                              d.nseg, cudaMemcpyDeviceToHost, h->stream));
    TF_TRY(sync(h));
    double dn = 0.0;
    for (double v : du2) dn = std::max(dn, std::sqrt(v));
    if (dunorm) *dunorm = dn;
    if (converged) *converged = !(dn > h->opt.newton_tol);
    if (!std::isfinite(dn)) return set_error("non-finite Newton update"), TF_NAN_DETECTED;
    return TF_OK;
}

tf_status tf_end_step(tf_handle* h) {
    TF_TRY(check_handle(h));
    if (h->in_step) h->time += h->dt;  // runOneStep: currSimTimeSec += dt (Simulation.cpp:5969)
    h->in_step = false;
    return sync(h);
}

tf_status tf_newton_step(tf_handle* h, double dt, tf_step_stats* stats) {
    TF_TRY(check_handle(h));
    return newton_run(h, dt, stats, nullptr, nullptr);
}

tf_status tf_get_residual(tf_handle* h, double* g) {
    TF_TRY(check_handle(h));
    if (!g) return set_error("null output"), TF_BAD_INPUT;
    TF_CUDA(cudaMemcpyAsync(g, h->d.g, sizeof(double) * 3 * (size_t)h->d.nn, cudaMemcpyDeviceToHost, h->stream));
    return sync(h);
}

tf_status tf_get_delta_u(tf_handle* h, double* du) {
    TF_TRY(check_handle(h));
    if (!du) return set_error("null output"), TF_BAD_INPUT;
    TF_CUDA(cudaMemcpyAsync(du, h->d.du, sizeof(double) * 3 * (size_t)h->d.nn, cudaMemcpyDeviceToHost, h->stream));
    return sync(h);
}

tf_status tf_get_viscosity_surfaces(tf_handle* h, double* area) {
    TF_TRY(check_handle(h));
    if (!area) return set_error("null output"), TF_BAD_INPUT;
    TF_CUDA(cudaMemcpyAsync(area, h->d.area, sizeof(double) * (size_t)h->d.nn, cudaMemcpyDeviceToHost, h->stream));
    return sync(h);
}

tf_status tf_set_viscosity_surfaces(tf_handle* h, const double* area) {
    TF_TRY(check_handle(h));
    if (!area) return set_error("null input"), TF_BAD_INPUT;
    TF_CUDA(cudaMemcpyAsync(h->d.area, area, sizeof(double) * (size_t)h->d.nn, cudaMemcpyHostToDevice, h->stream));
    return sync(h);
}

tf_status tf_set_state(tf_handle* h, const double* uk, const double* un, double dt) {
    TF_TRY(check_handle(h));
    if (!uk || !un || !(dt > 0.0)) return set_error("bad state"), TF_BAD_INPUT;
    h->dt = dt;
    const size_t n3 = 3 * (size_t)h->d.nn;
    TF_CUDA(cudaMemcpyAsync(h->d.uk, uk, n3 * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    TF_CUDA(cudaMemcpyAsync(h->d.un, un, n3 * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    h->assembled = false;
    return sync(h);
}

tf_status tf_export_csr(tf_handle* h, double drop_tol, int32_t* ia, int32_t* ja, double* a, int64_t* nnz) {
    TF_TRY(check_handle(h));
    if (!h->assembled) return set_error("tf_export_csr called before tf_assemble"), TF_BAD_INPUT;
    if (!nnz || (ia && (!ja || !a))) return set_error("bad output arrays"), TF_BAD_INPUT;
    const Device& d = h->d;
    TF_TRY(sync_extra_to_host(h));
    std::vector<double> val((size_t)d.nval);
    TF_CUDA(cudaMemcpyAsync(val.data(), d.val, val.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    TF_TRY(sync(h));
    const std::vector<int>& rp = h->h_rowptr;
    const std::vector<int>& ci = h->h_colidx;
    auto find_block = [&](int r, int c) {
        auto it = std::lower_bound(ci.begin() + rp[r], ci.begin() + rp[r + 1], c);
        return static_cast<int64_t>(it - ci.begin());
    };
    // extra blocks A(J, I) from tf_add_K_triplets, listed by the K row I they touch
    std::vector<std::vector<std::pair<int, int64_t>>> xby(d.nn);
    if (d.nxb > 0)
        for (int J = 0; J < d.nn; ++J)
            for (int p = h->h_xrow[J]; p < h->h_xrow[J + 1]; ++p) xby[h->h_xcol_prev[p]].push_back({J, p});
    for (auto& v : xby) std::sort(v.begin(), v.end());
    // K(3i+di, 3j+dj) = A(3j+dj, 3i+di): block (j, i) of A, entry (dj, di).
    int64_t q = 0;
    if (ia) ia[0] = 0;
    for (int i = 0; i < d.nn; ++i)
        for (int di = 0; di < 3; ++di) {
            const int r = 3 * i + di;
            size_t xk = 0;
            const auto& xi = xby[i];
            auto emit = [&](int j, const double* blk, int stride) {
                for (int dj = 0; dj < 3; ++dj) {
                    const int c = 3 * j + dj;
                    double v;
                    if (h->h_fixed[r] || h->h_fixed[c]) v = (r == c) ? 1.0 : 0.0;
                    else v = blk[stride * (3 * dj + di)];
                    if (v > drop_tol || v < -drop_tol) {
                        if (ia) {
                            ja[q] = c;
                            a[q] = v;
                        }
                        ++q;
                    }
                }
            };
            for (int p = rp[i]; p < rp[i + 1]; ++p) {
                const int j = ci[p];
                for (; xk < xi.size() && xi[xk].first < j; ++xk)
                    emit(xi[xk].first, &h->h_xval[9 * (size_t)xi[xk].second], 1);
                emit(j, &val[(size_t)h->h_bofs[find_block(j, i)]], kSlice);
            }
            for (; xk < xi.size(); ++xk) emit(xi[xk].first, &h->h_xval[9 * (size_t)xi[xk].second], 1);
            if (ia) ia[r + 1] = static_cast<int32_t>(q);
        }
    *nnz = q;
    return TF_OK;
}

tf_status tf_element_eval(tf_handle* h, int32_t e0, int32_t count, double* Ke, double* Kv, double* fe, double* fv) {
    TF_TRY(check_handle(h));
    if (e0 < 0 || count < 0 || (int64_t)e0 + count > h->d.ne) return set_error("element range"), TF_BAD_INPUT;
    if (count == 0) return TF_OK;
    // velocity of the current state, as tf_assemble computes it
    const Device& d = h->d;
    double *dKe = nullptr, *dKv = nullptr, *dfe = nullptr, *dfv = nullptr;
    tf_status s = TF_OK;
    if (Ke) s = dev_alloc(&dKe, 324 * (size_t)count);
    if (s == TF_OK && Kv) s = dev_alloc(&dKv, 324 * (size_t)count);
    if (s == TF_OK && fe) s = dev_alloc(&dfe, 18 * (size_t)count);
    if (s == TF_OK && fv) s = dev_alloc(&dfv, 18 * (size_t)count);
    if (s == TF_OK) s = launch_prepare(h);
    if (s == TF_OK) s = launch_element_eval(h, e0, count, dKe, dKv, dfe, dfv);
    struct Out {
        double* dev;
        double* host;
        size_t n;
    } outs[] = {{dKe, Ke, 324 * (size_t)count}, {dKv, Kv, 324 * (size_t)count},
                {dfe, fe, 18 * (size_t)count}, {dfv, fv, 18 * (size_t)count}};
    for (auto& o : outs)
        if (s == TF_OK && o.dev) {
            cudaError_t e = cudaMemcpyAsync(o.host, o.dev, o.n * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
            if (e != cudaSuccess) s = cuda_fail(e, "cudaMemcpyAsync");
        }
    if (s == TF_OK) s = sync(h);
    for (auto& o : outs)
        if (o.dev) cudaFree(o.dev);
    (void)d;
    h->assembled = false;  // launch_prepare reset the block values
    return s;
}

tf_status tf_get_sizes(tf_handle* h, int64_t* n_nodes, int64_t* n_elems, int64_t* n_blocks) {
    if (!h) return set_error("null handle"), TF_BAD_INPUT;
    if (n_nodes) *n_nodes = h->d.nn;
    if (n_elems) *n_elems = h->d.ne;
    if (n_blocks) *n_blocks = h->d.nnzb;
    return TF_OK;
}

void* tf_get_stream(tf_handle* h) { return h ? reinterpret_cast<void*>(h->stream) : nullptr; }

int64_t tf_launch_count(tf_handle* h) { return h ? h->launches : 0; }

tf_status tf_time_assembly(tf_handle* h, int32_t iters, float* ms_per_assembly, float* ms_per_element_kernel) {
    TF_TRY(check_handle(h));
    if (iters <= 0) return set_error("iters must be positive"), TF_BAD_INPUT;
    float asm_ms = 0.f, elem_ms = 0.f;
    for (int i = 0; i < iters; ++i) {
        TF_CUDA(cudaEventRecord(h->ev[4], h->stream));
        TF_TRY(launch_prepare(h));
        TF_CUDA(cudaEventRecord(h->ev[5], h->stream));
        TF_TRY(launch_element(h));
        TF_CUDA(cudaEventRecord(h->ev[6], h->stream));
        if (h->opt.deterministic) TF_TRY(launch_deterministic_gather(h));
        TF_CUDA(cudaEventRecord(h->ev[7], h->stream));
        TF_TRY(sync(h));
        float a = 0.f, b = 0.f;
        TF_CUDA(cudaEventElapsedTime(&a, h->ev[4], h->ev[7]));
        TF_CUDA(cudaEventElapsedTime(&b, h->ev[5], h->ev[6]));
        asm_ms += a;
        elem_ms += b;
    }
    h->assembled = true;
    if (ms_per_assembly) *ms_per_assembly = asm_ms / iters;
    if (ms_per_element_kernel) *ms_per_element_kernel = elem_ms / iters;
    return TF_OK;
}

}  // extern "C"
