// fem_xtk.cpp -- XFEM input for the cut-cell path: decomposition of a uniform
// level-0 HEX8 mesh by a nodal level set into tetrahedral integration cells,
// Heaviside enrichment of the B-spline bases, interface facets and
// face-oriented ghost facets.
//
// This is the host preprocessing that feeds the cut-cluster and double-sided
// kernels; it stands in for the reference's XTK pipeline
// (XTK/src/cl_XTK_Model.cpp:690 decompose, cl_XTK_Regular_Subdivision_
// Interface.hpp:225 24-tet subdivision, cl_XTK_Integration_Mesh_Generator.cpp:
// 53, cl_XTK_Enrichment.cpp:1148-2362, cl_XTK_Ghost_Stabilization.cpp:45) for
// one level set:
//
//  * a cell is cut when its corner level-set values change sign (phase 1 where
//    phi < 0, phase 0 where phi >= 0);
//  * a cut cell is split into 24 tetrahedra around its centre and face centres
//    (the regular subdivision); the level set at a face centre is the mean of
//    its four corners, at the cell centre the mean of the eight corners
//    (derived nodes interpolate their parent cell);
//  * every tetrahedron whose vertices change sign is cut by the plane phi = 0
//    (linear along each edge, Intersection_Node_Linear, GEN/src/PDV/
//    cl_GEN_Intersection_Node_Linear.cpp:46-57): a lone vertex gives one tet
//    plus a wedge, two against two give two wedges; wedges are split into
//    three tets; the cut plane gives the interface triangles, oriented with
//    the normal pointing out of phase 0 (the leader);
//  * enrichment: for every background basis and phase, the cells of its
//    support that hold the phase are grouped into face-connected components
//    and each component is one enriched basis (numbered by basis, then phase,
//    then component); each enriched cell (cell, phase) has its own unzipped
//    vertices whose extraction rows point at the enriched bases;
//  * ghost facets: for every phase, every face between two cells that both
//    hold the phase, at least one of them cut; the lower cell is the leader.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <unordered_map>
#include <vector>

#include "fem_internal.hpp"
#include "fem_xtk.hpp"

namespace fem {
const int kHexSides[6][4] = {{1, 5, 4, 0}, {1, 2, 6, 5}, {3, 7, 6, 2}, {0, 4, 7, 3}, {0, 3, 2, 1}, {4, 5, 6, 7}};
const double kHexXi[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                             {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
}  // namespace fem

namespace {

struct Tet {
    int32_t v[4];     // IG vertex ids
    double xi[4][3];  // parametric coordinates in the IP cell
};

struct Facet {
    int32_t v[3];
    double xi[3][3];
};

struct CutCell {
    int64_t cell;
    std::vector<Tet> tets[2];
    std::vector<Facet> facets;
};

uint64_t edge_key(int32_t a, int32_t b) {
    if (a > b) std::swap(a, b);
    return (uint64_t)(uint32_t)a << 32 | (uint32_t)b;
}

double signed_det(const double* x0, const double* x1, const double* x2, const double* x3) {
    // det of [x0-x2; x1-x2; x3-x2] (the Tet4 Jacobian with vertex order xi1, xi2, 1-sum, xi3)
    double a[3], b[3], c[3];
    for (int d = 0; d < 3; ++d) {
        a[d] = x0[d] - x2[d];
        b[d] = x1[d] - x2[d];
        c[d] = x3[d] - x2[d];
    }
    return a[0] * (b[1] * c[2] - b[2] * c[1]) - a[1] * (b[0] * c[2] - b[2] * c[0]) + a[2] * (b[0] * c[1] - b[1] * c[0]);
}

}  // namespace

using namespace fem;

extern "C" {

fem_gpu_status fem_xtk_decompose(const int32_t* num_elements, const double* lengths, int32_t p,
                                 const double* node_phi, fem_xtk_model** out) {
    if (!num_elements || !lengths || !node_phi || !out || p < 1 || p > 3) return FEM_GPU_BAD_ARG;
    for (int d = 0; d < 3; ++d)
        if (num_elements[d] < 1 || !(lengths[d] > 0.0)) return FEM_GPU_BAD_ARG;
    fem_hmr_mesh* bg = nullptr;
    fem_gpu_status st = fem_hmr_uniform_mesh(3, num_elements, lengths, p, &bg);
    if (st != FEM_GPU_OK) return st;
    int64_t nnodes, ncells, nbases, tnz;
    fem_hmr_mesh_sizes(bg, &nnodes, &ncells, &nbases, &tnz);
    std::vector<double> bx(nnodes * 3), bw(tnz);
    std::vector<int32_t> bc(ncells * 8), bb(tnz);
    std::vector<int64_t> boff(nnodes + 1);
    fem_hmr_mesh_arrays(bg, bx.data(), bc.data(), boff.data(), bb.data(), bw.data());
    fem_hmr_mesh_free(bg);
    for (int64_t n = 0; n < nnodes; ++n)
        if (!std::isfinite(node_phi[n])) return FEM_GPU_NONFINITE;

    auto* m = new fem_xtk_model;
    m->p = p;
    for (int d = 0; d < 3; ++d) {
        m->ne[d] = num_elements[d];
        m->nn[d] = num_elements[d] + 1;
        m->nbk[d] = num_elements[d] + p;
    }
    const int64_t* ne = m->ne;
    auto phase_of = [](double phi) { return phi < 0.0 ? 1 : 0; };

    // ---- cell phases ------------------------------------------------------
    std::vector<uint8_t> has(ncells * 2, 0), is_cut(ncells, 0);
    for (int64_t c = 0; c < ncells; ++c) {
        for (int a = 0; a < 8; ++a) has[c * 2 + phase_of(node_phi[bc[c * 8 + a]])] = 1;
        is_cut[c] = has[c * 2] && has[c * 2 + 1];
    }

    // ---- IG vertices and the decomposition of cut cells -----------------------
    std::vector<int32_t> node_vid(nnodes, -1);
    std::unordered_map<uint64_t, int32_t> face_vid, edge_vid;
    auto add_vertex = [&](const IgVertex& v) {
        m->verts.push_back(v);
        return (int32_t)(m->verts.size() - 1);
    };
    auto bg_vertex = [&](int32_t n) {
        if (node_vid[n] < 0) {
            IgVertex v{};
            v.kind = 0;
            for (int k = 0; k < 8; ++k) v.parents[k] = -1;
            v.parents[0] = n;
            for (int d = 0; d < 3; ++d) v.x[d] = bx[(int64_t)n * 3 + d];
            v.value = node_phi[n];
            node_vid[n] = add_vertex(v);
        }
        return node_vid[n];
    };
    std::vector<CutCell> cutcells;
    for (int64_t c = 0; c < ncells; ++c) {
        if (!is_cut[c]) continue;
        CutCell cc;
        cc.cell = c;
        const int32_t* cn = &bc[c * 8];
        int32_t cv[8];
        for (int a = 0; a < 8; ++a) cv[a] = bg_vertex(cn[a]);
        // cell centre
        IgVertex ctr{};
        ctr.kind = 2;
        ctr.value = 0.0;
        for (int a = 0; a < 8; ++a) {
            ctr.parents[a] = cn[a];
            ctr.value += node_phi[cn[a]];
            for (int d = 0; d < 3; ++d) ctr.x[d] += bx[(int64_t)cn[a] * 3 + d];
        }
        ctr.value /= 8.0;
        for (int d = 0; d < 3; ++d) ctr.x[d] /= 8.0;
        const int32_t vc = add_vertex(ctr);
        // local vertex table of the cell: 8 corners, 6 face centres, centre
        int32_t lv[15];
        double lxi[15][3];
        for (int a = 0; a < 8; ++a) {
            lv[a] = cv[a];
            for (int d = 0; d < 3; ++d) lxi[a][d] = kHexXi[a][d];
        }
        for (int f = 0; f < 6; ++f) {
            int32_t fn[4];
            for (int k = 0; k < 4; ++k) fn[k] = cn[kHexSides[f][k]];
            const int32_t mn = *std::min_element(fn, fn + 4);
            const int axis = (f == 1 || f == 3) ? 0 : (f == 0 || f == 2) ? 1 : 2;
            const uint64_t key = (uint64_t)mn * 3 + axis;
            auto it = face_vid.find(key);
            if (it == face_vid.end()) {
                IgVertex v{};
                v.kind = 1;
                for (int k = 0; k < 8; ++k) v.parents[k] = k < 4 ? fn[k] : -1;
                v.value = 0.0;
                for (int k = 0; k < 4; ++k) {
                    v.value += node_phi[fn[k]];
                    for (int d = 0; d < 3; ++d) v.x[d] += bx[(int64_t)fn[k] * 3 + d];
                }
                v.value /= 4.0;
                for (int d = 0; d < 3; ++d) v.x[d] /= 4.0;
                it = face_vid.emplace(key, add_vertex(v)).first;
            }
            lv[8 + f] = it->second;
            for (int d = 0; d < 3; ++d) {
                double s = 0.0;
                for (int k = 0; k < 4; ++k) s += kHexXi[kHexSides[f][k]][d];
                lxi[8 + f][d] = s / 4.0;
            }
        }
        lv[14] = vc;
        for (int d = 0; d < 3; ++d) lxi[14][d] = 0.0;
        // intersection vertex on the IG edge (va, vb), parametric point by the same t
        auto cut_vertex = [&](int la, int lb, double* xi_out) {
            const int32_t va = lv[la], vb = lv[lb];
            const uint64_t key = edge_key(va, vb);
            const int32_t lo = std::min(va, vb), hi = std::max(va, vb);
            const double pl = m->verts[lo].value, ph = m->verts[hi].value;
            const double t = pl / (pl - ph);
            auto it = edge_vid.find(key);
            if (it == edge_vid.end()) {
                IgVertex v{};
                v.kind = 3;
                for (int k = 0; k < 8; ++k) v.parents[k] = -1;
                v.parents[0] = lo;
                v.parents[1] = hi;
                v.value = t;
                for (int d = 0; d < 3; ++d) v.x[d] = m->verts[lo].x[d] + t * (m->verts[hi].x[d] - m->verts[lo].x[d]);
                it = edge_vid.emplace(key, add_vertex(v)).first;
            }
            const int llo = lo == va ? la : lb, lhi = lo == va ? lb : la;
            for (int d = 0; d < 3; ++d) xi_out[d] = lxi[llo][d] + t * (lxi[lhi][d] - lxi[llo][d]);
            return it->second;
        };
        auto emit_tet = [&](int ph, const int32_t* v, const double (*xi)[3]) {
            Tet t;
            for (int k = 0; k < 4; ++k) {
                t.v[k] = v[k];
                for (int d = 0; d < 3; ++d) t.xi[k][d] = xi[k][d];
            }
            if (signed_det(m->verts[t.v[0]].x, m->verts[t.v[1]].x, m->verts[t.v[2]].x, m->verts[t.v[3]].x) < 0.0) {
                std::swap(t.v[0], t.v[1]);
                for (int d = 0; d < 3; ++d) std::swap(t.xi[0][d], t.xi[1][d]);
            }
            cc.tets[ph].push_back(t);
        };
        // wedge A0 A1 A2 / B0 B1 B2 with lateral edges Ak-Bk -> three tets
        auto emit_wedge = [&](int ph, const int32_t* A, const double (*xa)[3], const int32_t* B, const double (*xb)[3]) {
            const int32_t t1[4] = {A[0], A[1], A[2], B[0]}, t2[4] = {A[1], A[2], B[0], B[1]}, t3[4] = {A[2], B[0], B[1], B[2]};
            const double x1[4][3] = {{xa[0][0], xa[0][1], xa[0][2]}, {xa[1][0], xa[1][1], xa[1][2]},
                                     {xa[2][0], xa[2][1], xa[2][2]}, {xb[0][0], xb[0][1], xb[0][2]}};
            const double x2[4][3] = {{xa[1][0], xa[1][1], xa[1][2]}, {xa[2][0], xa[2][1], xa[2][2]},
                                     {xb[0][0], xb[0][1], xb[0][2]}, {xb[1][0], xb[1][1], xb[1][2]}};
            const double x3[4][3] = {{xa[2][0], xa[2][1], xa[2][2]}, {xb[0][0], xb[0][1], xb[0][2]},
                                     {xb[1][0], xb[1][1], xb[1][2]}, {xb[2][0], xb[2][1], xb[2][2]}};
            emit_tet(ph, t1, x1);
            emit_tet(ph, t2, x2);
            emit_tet(ph, t3, x3);
        };
        // interface triangle, normal (x0-x2) x (x1-x2) out of phase 0
        auto emit_facet = [&](const int32_t* v, const double (*xi)[3], const double* inside0) {
            Facet f;
            for (int k = 0; k < 3; ++k) {
                f.v[k] = v[k];
                for (int d = 0; d < 3; ++d) f.xi[k][d] = xi[k][d];
            }
            const double* x0 = m->verts[f.v[0]].x;
            const double* x1 = m->verts[f.v[1]].x;
            const double* x2 = m->verts[f.v[2]].x;
            double a[3], b[3], n[3];
            for (int d = 0; d < 3; ++d) {
                a[d] = x0[d] - x2[d];
                b[d] = x1[d] - x2[d];
            }
            n[0] = a[1] * b[2] - a[2] * b[1];
            n[1] = a[2] * b[0] - a[0] * b[2];
            n[2] = a[0] * b[1] - a[1] * b[0];
            double s = 0.0;
            for (int d = 0; d < 3; ++d) s += n[d] * (inside0[d] - x2[d]);
            if (s > 0.0) {
                std::swap(f.v[0], f.v[1]);
                for (int d = 0; d < 3; ++d) std::swap(f.xi[0][d], f.xi[1][d]);
            }
            cc.facets.push_back(f);
        };
        for (int f = 0; f < 6; ++f)
            for (int k = 0; k < 4; ++k) {
                const int l[4] = {14, 8 + f, kHexSides[f][k], kHexSides[f][(k + 1) % 4]};
                int ph[4], n1 = 0;
                for (int q = 0; q < 4; ++q) {
                    ph[q] = phase_of(m->verts[lv[l[q]]].value);
                    n1 += ph[q];
                }
                int32_t v[4];
                double xi[4][3];
                for (int q = 0; q < 4; ++q) {
                    v[q] = lv[l[q]];
                    for (int d = 0; d < 3; ++d) xi[q][d] = lxi[l[q]][d];
                }
                if (n1 == 0 || n1 == 4) {
                    emit_tet(ph[0], v, xi);
                    continue;
                }
                if (n1 == 1 || n1 == 3) {
                    const int lone_ph = n1 == 1 ? 1 : 0;
                    int L = 0;
                    while (ph[L] != lone_ph) ++L;
                    int O[3], no = 0;
                    for (int q = 0; q < 4; ++q)
                        if (q != L) O[no++] = q;
                    int32_t I[3];
                    double xI[3][3];
                    for (int k2 = 0; k2 < 3; ++k2) I[k2] = cut_vertex(l[L], l[O[k2]], xI[k2]);
                    const int32_t tv[4] = {v[L], I[0], I[1], I[2]};
                    const double tx[4][3] = {{xi[L][0], xi[L][1], xi[L][2]}, {xI[0][0], xI[0][1], xI[0][2]},
                                             {xI[1][0], xI[1][1], xI[1][2]}, {xI[2][0], xI[2][1], xI[2][2]}};
                    emit_tet(lone_ph, tv, tx);
                    const int32_t A[3] = {v[O[0]], v[O[1]], v[O[2]]};
                    const double xa[3][3] = {{xi[O[0]][0], xi[O[0]][1], xi[O[0]][2]},
                                             {xi[O[1]][0], xi[O[1]][1], xi[O[1]][2]},
                                             {xi[O[2]][0], xi[O[2]][1], xi[O[2]][2]}};
                    emit_wedge(1 - lone_ph, A, xa, I, xI);
                    const double* in0 = lone_ph == 0 ? m->verts[v[L]].x : m->verts[v[O[0]]].x;
                    emit_facet(I, xI, in0);
                } else {
                    int P[2], Q[2], np = 0, nq = 0;
                    for (int q = 0; q < 4; ++q) {
                        if (ph[q] == 1) P[np++] = q;
                        else Q[nq++] = q;
                    }
                    const int a = P[0], b = P[1], c2 = Q[0], d2 = Q[1];
                    double xac[3], xad[3], xbc[3], xbd[3];
                    const int32_t Iac = cut_vertex(l[a], l[c2], xac), Iad = cut_vertex(l[a], l[d2], xad);
                    const int32_t Ibc = cut_vertex(l[b], l[c2], xbc), Ibd = cut_vertex(l[b], l[d2], xbd);
                    {
                        const int32_t A[3] = {v[a], Iac, Iad}, B[3] = {v[b], Ibc, Ibd};
                        const double xa[3][3] = {{xi[a][0], xi[a][1], xi[a][2]}, {xac[0], xac[1], xac[2]},
                                                 {xad[0], xad[1], xad[2]}};
                        const double xb[3][3] = {{xi[b][0], xi[b][1], xi[b][2]}, {xbc[0], xbc[1], xbc[2]},
                                                 {xbd[0], xbd[1], xbd[2]}};
                        emit_wedge(1, A, xa, B, xb);
                    }
                    {
                        const int32_t A[3] = {v[c2], Iac, Ibc}, B[3] = {v[d2], Iad, Ibd};
                        const double xa[3][3] = {{xi[c2][0], xi[c2][1], xi[c2][2]}, {xac[0], xac[1], xac[2]},
                                                 {xbc[0], xbc[1], xbc[2]}};
                        const double xb[3][3] = {{xi[d2][0], xi[d2][1], xi[d2][2]}, {xad[0], xad[1], xad[2]},
                                                 {xbd[0], xbd[1], xbd[2]}};
                        emit_wedge(0, A, xa, B, xb);
                    }
                    const double* in0 = m->verts[v[c2]].x;
                    const int32_t f1[3] = {Iac, Iad, Ibd}, f2[3] = {Iac, Ibd, Ibc};
                    const double x1[3][3] = {{xac[0], xac[1], xac[2]}, {xad[0], xad[1], xad[2]}, {xbd[0], xbd[1], xbd[2]}};
                    const double x2[3][3] = {{xac[0], xac[1], xac[2]}, {xbd[0], xbd[1], xbd[2]}, {xbc[0], xbc[1], xbc[2]}};
                    emit_facet(f1, x1, in0);
                    emit_facet(f2, x2, in0);
                }
            }
        cutcells.push_back(std::move(cc));
    }

    // ---- enrichment ---------------------------------------------------------
    const int pp = p + 1, nloc = pp * pp * pp;
    const int64_t nb0 = m->nbk[0], nb1 = m->nbk[1];
    // ebase[(cell*2 + phase)*nloc + l]: enriched basis id (-1 where the phase is absent)
    std::vector<int64_t> ncomp(nbases, 0);
    std::vector<int32_t> comp((size_t)ncells * 2 * nloc, -1);
    for (int64_t b = 0; b < nbases; ++b) {
        const int64_t bi = b % nb0, bj = (b / nb0) % nb1, bk = b / (nb0 * nb1);
        int64_t sc[64];
        int nsc = 0;
        for (int l2 = 0; l2 < pp; ++l2)
            for (int l1 = 0; l1 < pp; ++l1)
                for (int l0 = 0; l0 < pp; ++l0) {
                    const int64_t ci = bi - l0, cj = bj - l1, ck = bk - l2;
                    if (ci < 0 || cj < 0 || ck < 0 || ci >= ne[0] || cj >= ne[1] || ck >= ne[2]) continue;
                    sc[nsc++] = ci + ne[0] * (cj + ne[1] * ck);
                }
        std::sort(sc, sc + nsc);
        int next = 0;
        for (int ph = 0; ph < 2; ++ph) {
            int lab[64];
            for (int k = 0; k < nsc; ++k) lab[k] = -1;
            for (int k0 = 0; k0 < nsc; ++k0) {
                if (!has[sc[k0] * 2 + ph] || lab[k0] >= 0) continue;
                // flood fill over face neighbours inside the support
                int stack[64], top = 0;
                stack[top++] = k0;
                lab[k0] = next;
                while (top) {
                    const int k = stack[--top];
                    const int64_t c = sc[k];
                    const int64_t ci = c % ne[0], cj = (c / ne[0]) % ne[1], ck = c / (ne[0] * ne[1]);
                    for (int q = 0; q < nsc; ++q) {
                        if (lab[q] >= 0 || !has[sc[q] * 2 + ph]) continue;
                        const int64_t c2 = sc[q];
                        const int64_t qi = c2 % ne[0], qj = (c2 / ne[0]) % ne[1], qk = c2 / (ne[0] * ne[1]);
                        if (std::llabs(qi - ci) + std::llabs(qj - cj) + std::llabs(qk - ck) != 1) continue;
                        lab[q] = next;
                        stack[top++] = q;
                    }
                }
                ++next;
            }
            for (int k = 0; k < nsc; ++k) {
                if (lab[k] < 0) continue;
                const int64_t c = sc[k];
                const int64_t ci = c % ne[0], cj = (c / ne[0]) % ne[1], ck = c / (ne[0] * ne[1]);
                const int l = (int)((bi - ci) + pp * ((bj - cj) + pp * (bk - ck)));
                comp[(size_t)(c * 2 + ph) * nloc + l] = lab[k];
            }
        }
        ncomp[b] = next;
    }
    std::vector<int64_t> eoff(nbases + 1, 0);
    for (int64_t b = 0; b < nbases; ++b) eoff[b + 1] = eoff[b] + ncomp[b];
    m->num_enriched_bases = eoff[nbases];

    // ---- enriched cells and unzipped vertices ----------------------------------
    std::vector<int64_t> ecell_of((size_t)ncells * 2, -1);
    for (int64_t c = 0; c < ncells; ++c)
        for (int ph = 0; ph < 2; ++ph)
            if (has[c * 2 + ph]) {
                ecell_of[c * 2 + ph] = (int64_t)m->cell_bg.size();
                m->cell_bg.push_back((int32_t)c);
                m->cell_phase.push_back(ph);
            }
    const int64_t nec = (int64_t)m->cell_bg.size();
    m->cells.resize(nec * 8);
    std::vector<std::vector<int32_t>> node_uv(nnodes);
    m->t_off.push_back(0);
    std::vector<int32_t> row;
    std::vector<double> roww;
    for (int64_t e = 0; e < nec; ++e) {
        const int64_t c = m->cell_bg[e];
        const int ph = m->cell_phase[e];
        const int64_t ci = c % ne[0], cj = (c / ne[0]) % ne[1], ck = c / (ne[0] * ne[1]);
        for (int a = 0; a < 8; ++a) {
            const int32_t n = bc[c * 8 + a];
            row.clear();
            roww.clear();
            for (int64_t k = boff[n]; k < boff[n + 1]; ++k) {
                const int64_t b = bb[k];
                const int64_t bi = b % nb0, bj = (b / nb0) % nb1, bk = b / (nb0 * nb1);
                const int l = (int)((bi - ci) + pp * ((bj - cj) + pp * (bk - ck)));
                const int32_t cp = comp[(size_t)(c * 2 + ph) * nloc + l];
                if (cp < 0) {
                    delete m;
                    return FEM_GPU_UNSUPPORTED;
                }
                row.push_back((int32_t)(eoff[b] + cp));
                roww.push_back(bw[k]);
            }
            int32_t vid = -1;
            for (int32_t cand : node_uv[n]) {
                const int64_t o = m->t_off[cand], len = m->t_off[cand + 1] - o;
                if (len == (int64_t)row.size() && std::equal(row.begin(), row.end(), m->t_bases.begin() + o)) {
                    vid = cand;
                    break;
                }
            }
            if (vid < 0) {
                vid = (int32_t)(m->t_off.size() - 1);
                for (int d = 0; d < 3; ++d) m->coords.push_back(bx[(int64_t)n * 3 + d]);
                m->t_bases.insert(m->t_bases.end(), row.begin(), row.end());
                m->t_w.insert(m->t_w.end(), roww.begin(), roww.end());
                m->t_off.push_back((int64_t)m->t_bases.size());
                node_uv[n].push_back(vid);
            }
            m->cells[e * 8 + a] = vid;
        }
    }

    // ---- clusters -------------------------------------------------------------
    for (int64_t c = 0; c < ncells; ++c)
        if (!is_cut[c])
            for (int ph = 0; ph < 2; ++ph)
                if (has[c * 2 + ph]) m->uncut[ph].push_back((int32_t)ecell_of[c * 2 + ph]);
    for (int ph = 0; ph < 2; ++ph) m->ig_off[ph].push_back(0);
    m->if_off.push_back(0);
    for (const CutCell& cc : cutcells) {
        for (int ph = 0; ph < 2; ++ph) {
            m->cut[ph].push_back((int32_t)ecell_of[cc.cell * 2 + ph]);
            for (const Tet& t : cc.tets[ph])
                for (int k = 0; k < 4; ++k) {
                    m->ig_v[ph].push_back(t.v[k]);
                    for (int d = 0; d < 3; ++d) {
                        m->ig_x[ph].push_back(m->verts[t.v[k]].x[d]);
                        m->ig_xi[ph].push_back(t.xi[k][d]);
                    }
                }
            m->ig_off[ph].push_back((int64_t)m->ig_v[ph].size() / 4);
        }
        m->if_leader.push_back((int32_t)ecell_of[cc.cell * 2 + 0]);
        m->if_follower.push_back((int32_t)ecell_of[cc.cell * 2 + 1]);
        for (const Facet& f : cc.facets)
            for (int k = 0; k < 3; ++k) {
                m->if_v.push_back(f.v[k]);
                for (int d = 0; d < 3; ++d) {
                    m->if_x.push_back(m->verts[f.v[k]].x[d]);
                    m->if_xi.push_back(f.xi[k][d]);
                }
            }
        m->if_off.push_back((int64_t)m->if_v.size() / 3);
    }
    // ghost facets: faces towards the +x, +y, +z neighbour
    const int side_of_axis[3] = {1, 2, 5};
    for (int ph = 0; ph < 2; ++ph)
        for (int64_t c = 0; c < ncells; ++c) {
            if (!has[c * 2 + ph]) continue;
            const int64_t ijk[3] = {c % ne[0], (c / ne[0]) % ne[1], c / (ne[0] * ne[1])};
            for (int ax = 0; ax < 3; ++ax) {
                if (ijk[ax] + 1 >= ne[ax]) continue;
                const int64_t c2 = c + (ax == 0 ? 1 : ax == 1 ? ne[0] : ne[0] * ne[1]);
                if (!has[c2 * 2 + ph] || !(is_cut[c] || is_cut[c2])) continue;
                m->gh_leader[ph].push_back((int32_t)ecell_of[c * 2 + ph]);
                m->gh_follower[ph].push_back((int32_t)ecell_of[c2 * 2 + ph]);
                const int s = side_of_axis[ax];
                for (int k = 0; k < 4; ++k) {
                    const int a = kHexSides[s][k];
                    const int32_t n = bc[c * 8 + a];
                    for (int d = 0; d < 3; ++d) {
                        m->gh_x[ph].push_back(bx[(int64_t)n * 3 + d]);
                        m->gh_xi_l[ph].push_back(kHexXi[a][d]);
                        m->gh_xi_f[ph].push_back(d == ax ? -1.0 : kHexXi[a][d]);
                    }
                }
            }
        }
    *out = m;
    return FEM_GPU_OK;
}

fem_gpu_status fem_xtk_get_sizes(const fem_xtk_model* m, fem_xtk_sizes* s) {
    if (!m || !s) return FEM_GPU_BAD_ARG;
    std::memset(s, 0, sizeof(*s));
    s->num_nodes = (int64_t)m->coords.size() / 3;
    s->num_cells = (int64_t)m->cell_bg.size();
    s->num_bases = m->num_enriched_bases;
    s->t_nnz = (int64_t)m->t_bases.size();
    for (int ph = 0; ph < 2; ++ph) {
        s->num_uncut[ph] = (int64_t)m->uncut[ph].size();
        s->num_cut[ph] = (int64_t)m->cut[ph].size();
        s->num_ig_cells[ph] = m->ig_off[ph].back();
        s->num_ghost[ph] = (int64_t)m->gh_leader[ph].size();
    }
    s->num_interface = (int64_t)m->if_leader.size();
    s->num_interface_facets = m->if_off.back();
    s->num_ig_vertices = (int64_t)m->verts.size();
    return FEM_GPU_OK;
}

fem_gpu_status fem_xtk_get_ip_mesh(const fem_xtk_model* m, double* coords, int32_t* cell_nodes, int64_t* t_off,
                                   int32_t* t_bases, double* t_w, int32_t* cell_background, int32_t* cell_phase) {
    if (!m) return FEM_GPU_BAD_ARG;
    if (coords) std::memcpy(coords, m->coords.data(), m->coords.size() * sizeof(double));
    if (cell_nodes) std::memcpy(cell_nodes, m->cells.data(), m->cells.size() * sizeof(int32_t));
    if (t_off) std::memcpy(t_off, m->t_off.data(), m->t_off.size() * sizeof(int64_t));
    if (t_bases) std::memcpy(t_bases, m->t_bases.data(), m->t_bases.size() * sizeof(int32_t));
    if (t_w) std::memcpy(t_w, m->t_w.data(), m->t_w.size() * sizeof(double));
    if (cell_background) std::memcpy(cell_background, m->cell_bg.data(), m->cell_bg.size() * sizeof(int32_t));
    if (cell_phase) std::memcpy(cell_phase, m->cell_phase.data(), m->cell_phase.size() * sizeof(int32_t));
    return FEM_GPU_OK;
}

fem_gpu_status fem_xtk_get_bulk(const fem_xtk_model* m, int32_t phase, int32_t* uncut_cells, int32_t* cut_cells,
                                int64_t* ig_offsets, double* ig_coords, double* ig_param, int32_t* ig_vertices) {
    if (!m || phase < 0 || phase > 1) return FEM_GPU_BAD_ARG;
    const int ph = phase;
    if (uncut_cells) std::memcpy(uncut_cells, m->uncut[ph].data(), m->uncut[ph].size() * sizeof(int32_t));
    if (cut_cells) std::memcpy(cut_cells, m->cut[ph].data(), m->cut[ph].size() * sizeof(int32_t));
    if (ig_offsets) std::memcpy(ig_offsets, m->ig_off[ph].data(), m->ig_off[ph].size() * sizeof(int64_t));
    if (ig_coords) std::memcpy(ig_coords, m->ig_x[ph].data(), m->ig_x[ph].size() * sizeof(double));
    if (ig_param) std::memcpy(ig_param, m->ig_xi[ph].data(), m->ig_xi[ph].size() * sizeof(double));
    if (ig_vertices) std::memcpy(ig_vertices, m->ig_v[ph].data(), m->ig_v[ph].size() * sizeof(int32_t));
    return FEM_GPU_OK;
}

fem_gpu_status fem_xtk_get_interface(const fem_xtk_model* m, int32_t* leader, int32_t* follower, int64_t* offsets,
                                     double* coords, double* param, int32_t* vertices) {
    if (!m) return FEM_GPU_BAD_ARG;
    if (leader) std::memcpy(leader, m->if_leader.data(), m->if_leader.size() * sizeof(int32_t));
    if (follower) std::memcpy(follower, m->if_follower.data(), m->if_follower.size() * sizeof(int32_t));
    if (offsets) std::memcpy(offsets, m->if_off.data(), m->if_off.size() * sizeof(int64_t));
    if (coords) std::memcpy(coords, m->if_x.data(), m->if_x.size() * sizeof(double));
    if (param) std::memcpy(param, m->if_xi.data(), m->if_xi.size() * sizeof(double));
    if (vertices) std::memcpy(vertices, m->if_v.data(), m->if_v.size() * sizeof(int32_t));
    return FEM_GPU_OK;
}

fem_gpu_status fem_xtk_get_ghost(const fem_xtk_model* m, int32_t phase, int32_t* leader, int32_t* follower,
                                 double* coords, double* leader_param, double* follower_param) {
    if (!m || phase < 0 || phase > 1) return FEM_GPU_BAD_ARG;
    const int ph = phase;
    if (leader) std::memcpy(leader, m->gh_leader[ph].data(), m->gh_leader[ph].size() * sizeof(int32_t));
    if (follower) std::memcpy(follower, m->gh_follower[ph].data(), m->gh_follower[ph].size() * sizeof(int32_t));
    if (coords) std::memcpy(coords, m->gh_x[ph].data(), m->gh_x[ph].size() * sizeof(double));
    if (leader_param) std::memcpy(leader_param, m->gh_xi_l[ph].data(), m->gh_xi_l[ph].size() * sizeof(double));
    if (follower_param) std::memcpy(follower_param, m->gh_xi_f[ph].data(), m->gh_xi_f[ph].size() * sizeof(double));
    return FEM_GPU_OK;
}

fem_gpu_status fem_xtk_get_vertices(const fem_xtk_model* m, int32_t* kind, int32_t* parents, double* coords,
                                    double* value) {
    if (!m) return FEM_GPU_BAD_ARG;
    for (size_t i = 0; i < m->verts.size(); ++i) {
        const IgVertex& v = m->verts[i];
        if (kind) kind[i] = v.kind;
        if (parents)
            for (int k = 0; k < 8; ++k) parents[i * 8 + k] = v.parents[k];
        if (coords)
            for (int d = 0; d < 3; ++d) coords[i * 3 + d] = v.x[d];
        if (value) value[i] = v.value;
    }
    return FEM_GPU_OK;
}

void fem_xtk_free(fem_xtk_model* m) { delete m; }

}  // extern "C"
