// fem_host.cpp -- host side of libfem_gpu.so: the HMR-equivalent uniform
// mesh generator, context and set bookkeeping, and the MSI work of
// fem_gpu_finalize (adof numbering, element extraction operators, sparsity
// graph and the compact scatter maps the assembly kernels use).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>

#include "fem_internal.hpp"

namespace fem {

fem_gpu_status fail(fem_gpu_ctx* c, fem_gpu_status s, const std::string& msg) {
    if (c) c->err = msg;
    return s;
}

namespace {

int hw_threads() {
    unsigned n = std::thread::hardware_concurrency();
    return n == 0 ? 1 : (int)std::min(n, 64u);
}

// run f(i) for i in [0, n) on all host threads, in contiguous chunks
// threads parallel_for uses for n items
int range_threads(int64_t n) { return (int)std::min<int64_t>(hw_threads(), std::max<int64_t>(1, n / 256)); }

// f(t, begin, end) on nt = range_threads(n) threads, thread t taking the
// contiguous range [n t / nt, n (t + 1) / nt)
template <class F>
void parallel_ranges(int64_t n, int nt, F f) {
    if (nt <= 1) {
        f(0, (int64_t)0, n);
        return;
    }
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t) th.emplace_back([=]() { f(t, n * t / nt, n * (t + 1) / nt); });
    for (auto& x : th) x.join();
}

template <class F>
void parallel_for(int64_t n, F f) {
    const int nt = range_threads(n);
    if (nt <= 1) {
        for (int64_t i = 0; i < n; ++i) f(i);
        return;
    }
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t)
        th.emplace_back([=]() {
            const int64_t b = n * t / nt, e = n * (t + 1) / nt;
            for (int64_t i = b; i < e; ++i) f(i);
        });
    for (auto& x : th) x.join();
}

// runs the callables on threads of their own: the large per-set arrays are
// filled concurrently, so their first-touch page faults overlap
template <class... F>
void concurrently(F&&... fs) {
    std::vector<std::thread> th;
    (th.emplace_back(std::forward<F>(fs)), ...);
    for (auto& t : th) t.join();
}

// Cox-de Boor evaluation of one B-spline basis of an element, in element
// parametric coordinates [-1, 1] with knots at 2(i-p)-1 (the reference's
// HMR/src/fn_HMR_bspline_shape.cpp:20-58 convention: basis number j of the
// element spans the knot interval [2(j-p)-1, 2(j+1)-1)).
double bspline_value(int p, int j, double xi) {
    double N[8] = {0};
    double kn[10];
    for (int i = 0; i < 2 * (p + 1); ++i) kn[i] = 2.0 * (i - p) - 1.0;
    for (int q = 0; q <= p; ++q) N[q] = (kn[q + j] <= xi && xi < kn[q + j + 1]) ? 1.0 : 0.0;
    for (int q = 1; q <= p; ++q)
        for (int i = 0; i <= p - q; ++i) {
            const double a = xi - kn[i + j];
            const double b = kn[i + j + q + 1] - xi;
            N[i] = 0.5 * (a * N[i] + b * N[i + 1]) / (double)q;
        }
    return N[0];
}

}  // namespace
}  // namespace fem

using namespace fem;

extern "C" {

int32_t fem_gpu_abi_version(void) { return FEM_GPU_ABI_VERSION; }

// Set::get_auto_integration_order (FEM/INT/src/CORE/cl_FEM_Set.cpp:2983-3185):
// rule tables per (set kind, integration geometry, interpolation order); -1
// where the reference's choice is not a rule of this library
fem_gpu_status fem_gpu_auto_integration_rule(int32_t set_kind, int32_t cell, int32_t order, int32_t* rule) {
    if (!rule || order < 1 || order > 3) return FEM_GPU_BAD_ARG;
    const int o = order - 1;
    // entries: linear, quadratic, cubic
    static const int bulk_line[3] = {FEM_GPU_RULE_BAR_3, -1, -1};           // BAR_3, BAR_4, BAR_5
    static const int bulk_quad[3] = {FEM_GPU_RULE_QUAD_2x2, -1, -1};        // QUAD_2x2, QUAD_3x3, QUAD_5x5
    static const int bulk_hex[3] = {FEM_GPU_RULE_HEX_2x2x2, FEM_GPU_RULE_HEX_3x3x3, -1};  // ..., HEX_4x4x4
    static const int bulk_tri[3] = {FEM_GPU_RULE_TRI_7, -1, -1};            // TRI_7, TRI_12, TRI_25
    static const int bulk_tet[3] = {FEM_GPU_RULE_TET_11, -1, -1};           // TET_11, TET_35, TET_56
    static const int side_line[3] = {FEM_GPU_RULE_BAR_3, -1, -1};           // BAR_3, BAR_4, BAR_5
    static const int side_quad[3] = {FEM_GPU_RULE_QUAD_2x2, -1, -1};        // QUAD_2x2, QUAD_4x4, QUAD_5x5
    static const int side_tri[3] = {FEM_GPU_RULE_TRI_7, -1, -1};            // TRI_7, TRI_12, TRI_25
    const int* t = nullptr;
    if (set_kind == FEM_GPU_SET_BULK) {
        switch (cell) {
            case FEM_GPU_CELL_LINE2: t = bulk_line; break;
            case FEM_GPU_CELL_QUAD4: t = bulk_quad; break;
            case FEM_GPU_CELL_HEX8: t = bulk_hex; break;
            case FEM_GPU_CELL_TRI3: t = bulk_tri; break;
            case FEM_GPU_CELL_TET4: t = bulk_tet; break;
            default: return FEM_GPU_BAD_ARG;
        }
    } else if (set_kind == FEM_GPU_SET_SIDESET || set_kind == FEM_GPU_SET_DOUBLE_SIDESET) {
        switch (cell) {
            case FEM_GPU_CELL_LINE2: t = side_line; break;
            case FEM_GPU_CELL_QUAD4: t = side_quad; break;
            case FEM_GPU_CELL_TRI3: t = side_tri; break;
            default: return FEM_GPU_BAD_ARG;
        }
    } else {
        return FEM_GPU_BAD_ARG;
    }
    if (t[o] < 0) return FEM_GPU_UNSUPPORTED;
    *rule = t[o];
    return FEM_GPU_OK;
}

const char* fem_gpu_status_string(fem_gpu_status s) {
    switch (s) {
        case FEM_GPU_OK: return "ok";
        case FEM_GPU_BAD_ARG: return "bad argument";
        case FEM_GPU_OOB_INDEX: return "index out of range";
        case FEM_GPU_NONFINITE: return "non-finite value";
        case FEM_GPU_DETJ_NEGATIVE: return "negative Jacobian determinant";
        case FEM_GPU_TIMEOUT: return "device wait timed out";
        case FEM_GPU_CUDA_ERROR: return "CUDA error";
        case FEM_GPU_NOT_FINALIZED: return "context not finalized";
        case FEM_GPU_UNSUPPORTED: return "unsupported combination";
        case FEM_GPU_OUT_OF_MEMORY: return "out of memory";
        case FEM_GPU_NOT_CONVERGED: return "not converged";
        case FEM_GPU_NO_DEVICE: return "no CUDA device";
    }
    return "unknown status";
}

/* Uniform level-0 mesh as HMR builds it for a tensor grid: elements and
   bases numbered i-fastest (HMR/src/cl_HMR_BSpline_Mesh.hpp:474-535),
   Lagrange QUAD4/HEX8 nodes on the grid points, each node's extraction row
   T = L evaluated by the first element that visits the node, entries with
   |T| <= 1e-12 dropped (HMR/src/cl_HMR_T_Matrix_Base.cpp:306-457,
   cl_HMR_T_Matrix.hpp:433-463). */
fem_gpu_status fem_hmr_uniform_mesh(int32_t dim, const int32_t* ne_in, const double* len, int32_t p,
                                    fem_hmr_mesh** out) {
    if (!out || !ne_in || !len || (dim != 2 && dim != 3) || p < 1 || p > 3) return FEM_GPU_BAD_ARG;
    int64_t ne[3] = {1, 1, 1}, nn[3] = {1, 1, 1}, nb[3] = {1, 1, 1};
    for (int d = 0; d < dim; ++d) {
        if (ne_in[d] < 1) return FEM_GPU_BAD_ARG;
        ne[d] = ne_in[d];
        nn[d] = ne[d] + 1;
        nb[d] = ne[d] + p;
    }
    auto* m = new fem_hmr_mesh;
    m->dim = dim;
    const int64_t num_nodes = nn[0] * nn[1] * nn[2];
    const int64_t num_cells = ne[0] * ne[1] * ne[2];
    m->num_bases = nb[0] * nb[1] * nb[2];
    m->coords.resize(num_nodes * dim);
    for (int64_t n = 0; n < num_nodes; ++n) {
        const int64_t ijk[3] = {n % nn[0], (n / nn[0]) % nn[1], n / (nn[0] * nn[1])};
        for (int d = 0; d < dim; ++d) m->coords[n * dim + d] = len[d] * (double)ijk[d] / (double)ne[d];
    }
    const int npe = dim == 2 ? 4 : 8;
    const int cell = dim == 2 ? FEM_GPU_CELL_QUAD4 : FEM_GPU_CELL_HEX8;
    double xih[24];
    cell_param_coords(cell, xih);
    // element-local 1D basis values at the two element ends
    double v1[4][2];
    for (int j = 0; j <= p; ++j)
        for (int s = 0; s < 2; ++s) v1[j][s] = bspline_value(p, j, s ? 1.0 : -1.0);
    m->cells.resize(num_cells * npe);
    // owner element of each node: the first element (i-fastest) containing it
    std::vector<int64_t> owner(num_nodes, -1);
    std::vector<int8_t> owner_corner(num_nodes, -1);
    for (int64_t e = 0; e < num_cells; ++e) {
        const int64_t eijk[3] = {e % ne[0], (e / ne[0]) % ne[1], e / (ne[0] * ne[1])};
        for (int a = 0; a < npe; ++a) {
            int64_t nijk[3] = {0, 0, 0};
            for (int d = 0; d < dim; ++d) nijk[d] = eijk[d] + (xih[a * dim + d] > 0 ? 1 : 0);
            const int64_t nid = nijk[0] + nn[0] * (nijk[1] + nn[1] * nijk[2]);
            m->cells[e * npe + a] = (int32_t)nid;
            if (owner[nid] < 0) {
                owner[nid] = e;
                owner_corner[nid] = (int8_t)a;
            }
        }
    }
    const int nlb = dim == 2 ? (p + 1) * (p + 1) : (p + 1) * (p + 1) * (p + 1);
    std::vector<int32_t> cnt(num_nodes, 0);
    std::vector<std::vector<std::pair<int32_t, double>>> rows(num_nodes);
    parallel_for(num_nodes, [&](int64_t nid) {
        const int64_t e = owner[nid];
        const int a = owner_corner[nid];
        const int64_t eijk[3] = {e % ne[0], (e / ne[0]) % ne[1], e / (ne[0] * ne[1])};
        auto& row = rows[nid];
        for (int lb = 0; lb < nlb; ++lb) {
            const int l[3] = {lb % (p + 1), (lb / (p + 1)) % (p + 1), lb / ((p + 1) * (p + 1))};
            double w = 1.0;
            for (int d = 0; d < dim; ++d) w *= v1[l[d]][xih[a * dim + d] > 0 ? 1 : 0];
            if (std::abs(w) > 1e-12) {
                int64_t b = 0, stride = 1;
                for (int d = 0; d < dim; ++d) {
                    b += (eijk[d] + l[d]) * stride;
                    stride *= nb[d];
                }
                row.push_back({(int32_t)b, w});
            }
        }
    });
    m->t_off.assign(num_nodes + 1, 0);
    for (int64_t n = 0; n < num_nodes; ++n) m->t_off[n + 1] = m->t_off[n] + (int64_t)rows[n].size();
    m->t_bases.resize(m->t_off[num_nodes]);
    m->t_w.resize(m->t_off[num_nodes]);
    parallel_for(num_nodes, [&](int64_t n) {
        for (size_t k = 0; k < rows[n].size(); ++k) {
            m->t_bases[m->t_off[n] + k] = rows[n][k].first;
            m->t_w[m->t_off[n] + k] = rows[n][k].second;
        }
    });
    *out = m;
    return FEM_GPU_OK;
}

/* Tensor-product B-spline field on a uniform grid (the GEN B-spline level
   set): basis values at arbitrary points, HMR element / basis numbering. */
fem_gpu_status fem_gen_bspline_tmatrix(const int32_t* num_coefs, const double* len, int32_t p, int64_t np,
                                       const double* pts, int32_t* cols, double* vals) {
    if (!num_coefs || !len || !pts || !cols || !vals || p < 1 || p > 3 || np < 0) return FEM_GPU_BAD_ARG;
    int64_t ne[3], nb[3];
    for (int d = 0; d < 3; ++d) {
        nb[d] = num_coefs[d];
        ne[d] = nb[d] - p;
        if (ne[d] < 1 || !(len[d] > 0.0)) return FEM_GPU_BAD_ARG;
    }
    const int pp = p + 1, w = pp * pp * pp;
    for (int64_t k = 0; k < np; ++k) {
        int64_t el[3];
        double b[3][4];
        for (int d = 0; d < 3; ++d) {
            const double x = pts[k * 3 + d] / len[d] * (double)ne[d];
            if (!std::isfinite(x)) return FEM_GPU_NONFINITE;
            int64_t e = (int64_t)std::floor(x);
            e = std::min<int64_t>(std::max<int64_t>(e, 0), ne[d] - 1);
            const double xi = 2.0 * (x - (double)e) - 1.0;  // element coordinate in [-1, 1]
            el[d] = e;
            for (int j = 0; j < pp; ++j) {
                // the right end of the last element belongs to it (half-open intervals otherwise)
                const double xe = (xi >= 1.0 && e == ne[d] - 1) ? 1.0 - 1e-15 : xi;
                b[d][j] = bspline_value(p, j, xe);
            }
        }
        int q = 0;
        for (int l2 = 0; l2 < pp; ++l2)
            for (int l1 = 0; l1 < pp; ++l1)
                for (int l0 = 0; l0 < pp; ++l0, ++q) {
                    cols[k * w + q] = (int32_t)((el[0] + l0) + nb[0] * ((el[1] + l1) + nb[1] * (el[2] + l2)));
                    vals[k * w + q] = b[0][l0] * b[1][l1] * b[2][l2];
                }
    }
    return FEM_GPU_OK;
}

fem_gpu_status fem_hmr_mesh_sizes(const fem_hmr_mesh* m, int64_t* nn, int64_t* nc, int64_t* nb, int64_t* nz) {
    if (!m || !nn || !nc || !nb || !nz) return FEM_GPU_BAD_ARG;
    const int npe = m->dim == 2 ? 4 : 8;
    *nn = (int64_t)m->coords.size() / m->dim;
    *nc = (int64_t)m->cells.size() / npe;
    *nb = m->num_bases;
    *nz = (int64_t)m->t_bases.size();
    return FEM_GPU_OK;
}

fem_gpu_status fem_hmr_mesh_arrays(const fem_hmr_mesh* m, double* coords, int32_t* cells, int64_t* t_off,
                                   int32_t* t_b, double* t_w) {
    if (!m || !coords || !cells || !t_off || !t_b || !t_w) return FEM_GPU_BAD_ARG;
    std::memcpy(coords, m->coords.data(), m->coords.size() * sizeof(double));
    std::memcpy(cells, m->cells.data(), m->cells.size() * sizeof(int32_t));
    std::memcpy(t_off, m->t_off.data(), m->t_off.size() * sizeof(int64_t));
    std::memcpy(t_b, m->t_bases.data(), m->t_bases.size() * sizeof(int32_t));
    std::memcpy(t_w, m->t_w.data(), m->t_w.size() * sizeof(double));
    return FEM_GPU_OK;
}

fem_gpu_status fem_hmr_mesh_free(fem_hmr_mesh* m) {
    delete m;
    return FEM_GPU_OK;
}

fem_gpu_status fem_gpu_create(const fem_gpu_mesh_desc* d, fem_gpu_ctx** out) {
    if (!d || !out) return FEM_GPU_BAD_ARG;
    *out = nullptr;
    if (d->spatial_dim != 2 && d->spatial_dim != 3) return FEM_GPU_BAD_ARG;
    if ((d->spatial_dim == 2 && d->ip_cell_type != FEM_GPU_CELL_QUAD4) ||
        (d->spatial_dim == 3 && d->ip_cell_type != FEM_GPU_CELL_HEX8))
        return FEM_GPU_UNSUPPORTED;
    if (d->cell_shape != FEM_GPU_SHAPE_RECTANGULAR && d->cell_shape != FEM_GPU_SHAPE_GENERAL) return FEM_GPU_BAD_ARG;
    if (d->num_nodes <= 0 || d->num_cells <= 0 || d->num_bases <= 0 || !d->node_coords || !d->cell_nodes ||
        !d->t_offsets || !d->t_bases || !d->t_weights)
        return FEM_GPU_BAD_ARG;
    auto* c = new fem_gpu_ctx;
    c->dim = d->spatial_dim;
    c->ip_cell = d->ip_cell_type;
    c->shape = d->cell_shape;
    c->npe = cell_num_nodes(c->ip_cell);
    c->num_nodes = d->num_nodes;
    c->num_cells = d->num_cells;
    c->num_bases = d->num_bases;
    c->coords.assign(d->node_coords, d->node_coords + d->num_nodes * c->dim);
    c->cells.assign(d->cell_nodes, d->cell_nodes + d->num_cells * c->npe);
    c->t_off.assign(d->t_offsets, d->t_offsets + d->num_nodes + 1);
    if (c->t_off[0] != 0) {
        delete c;
        return FEM_GPU_BAD_ARG;
    }
    for (int64_t n = 0; n < d->num_nodes; ++n)
        if (c->t_off[n + 1] < c->t_off[n]) {
            delete c;
            return FEM_GPU_BAD_ARG;
        }
    const int64_t tn = c->t_off[d->num_nodes];
    c->t_bases.assign(d->t_bases, d->t_bases + tn);
    c->t_w.assign(d->t_weights, d->t_weights + tn);
    for (auto v : c->cells)
        if (v < 0 || v >= c->num_nodes) {
            delete c;
            return FEM_GPU_OOB_INDEX;
        }
    for (auto b : c->t_bases)
        if (b < 0 || b >= c->num_bases) {
            delete c;
            return FEM_GPU_OOB_INDEX;
        }
    for (double x : c->coords)
        if (!std::isfinite(x)) {
            delete c;
            return FEM_GPU_NONFINITE;
        }
    for (double x : c->t_w)
        if (!std::isfinite(x)) {
            delete c;
            return FEM_GPU_NONFINITE;
        }
    *out = c;
    return FEM_GPU_OK;
}

fem_gpu_status fem_gpu_destroy(fem_gpu_ctx* c) {
    if (!c) return FEM_GPU_BAD_ARG;
    device_release(c);
    delete c;
    return FEM_GPU_OK;
}

fem_gpu_status fem_gpu_add_bulk_set(fem_gpu_ctx* c, const fem_gpu_bulk_set_desc* d, int32_t* idx) {
    if (!c || !d) return FEM_GPU_BAD_ARG;
    if (c->host_final) return fail(c, FEM_GPU_BAD_ARG, "sets must be added before finalize");
    if (d->iwg_type != FEM_GPU_IWG_STRUC_LINEAR_BULK) return fail(c, FEM_GPU_UNSUPPORTED, "bulk iwg type");
    // an empty set (no clusters, as on a processor or mesh without cut cells) is
    // kept so that set indices stay those of the caller, and does no work
    if (d->num_clusters < 0 || (d->num_clusters > 0 && (!d->cluster_ip_cell || !d->youngs_modulus)))
        return fail(c, FEM_GPU_BAD_ARG, "bulk set arrays");
    const int igc = d->ig_cell_type;
    int rule = d->integration_rule;
    if (rule == FEM_GPU_RULE_AUTO && fem_gpu_auto_integration_rule(FEM_GPU_SET_BULK, igc, 1, &rule) != FEM_GPU_OK)
        return fail(c, FEM_GPU_BAD_ARG, "no automatic integration rule for this integration cell");
    const Rule r = gauss_rule(rule);
    if (r.n == 0 || cell_num_nodes(igc) == 0 || r.dim != cell_param_dim(igc))
        return fail(c, FEM_GPU_BAD_ARG, "integration rule does not match the integration cell");
    if (cell_param_dim(igc) != c->dim) return fail(c, FEM_GPU_BAD_ARG, "integration cell dimension");
    if (c->dim == 3 && d->model_type != FEM_GPU_MODEL_3D) return fail(c, FEM_GPU_BAD_ARG, "3D model type");
    if (c->dim == 2 && d->model_type == FEM_GPU_MODEL_3D) return fail(c, FEM_GPU_BAD_ARG, "2D model type");
    if (!d->ig_offsets && igc != c->ip_cell && d->num_clusters > 0)
        return fail(c, FEM_GPU_BAD_ARG, "trivial clusters need IG == IP cell");
    if (!(d->poisson_ratio > -1.0 && d->poisson_ratio < 0.5)) return fail(c, FEM_GPU_BAD_ARG, "poisson ratio");
    SetData s;
    s.kind = 0;
    s.bulk = *d;
    s.bulk.integration_rule = rule;
    s.neq = d->num_clusters;
    s.ip_cell.assign(d->cluster_ip_cell, d->cluster_ip_cell + s.neq);
    for (auto v : s.ip_cell)
        if (v < 0 || v >= c->num_cells) return fail(c, FEM_GPU_OOB_INDEX, "cluster interpolation cell");
    s.E.assign(d->youngs_modulus, d->youngs_modulus + s.neq);
    for (double e : s.E)
        if (!std::isfinite(e)) return fail(c, FEM_GPU_NONFINITE, "youngs modulus");
    // the Thickness property multiplies w* of every term of this linear
    // elastic set (stiffness, residual, strain energy, their derivatives), which
    // is the same as multiplying E
    if (d->thickness < 0.0 || !std::isfinite(d->thickness)) return fail(c, FEM_GPU_BAD_ARG, "bulk set thickness");
    if (d->thickness > 0.0) {
        s.bulk_thickness = d->thickness;
        for (double& e : s.E) e *= d->thickness;
    }
    if (d->ig_offsets || igc != c->ip_cell) {
        if (d->ig_offsets) s.ig_off.assign(d->ig_offsets, d->ig_offsets + s.neq + 1);
        else s.ig_off.assign(1, 0);
        const int64_t nig = s.ig_off[s.neq];
        if (nig > 0 && (!d->ig_coords || !d->ig_param_coords))
            return fail(c, FEM_GPU_BAD_ARG, "integration cell arrays");
        const int64_t per = (int64_t)cell_num_nodes(igc) * c->dim;
        s.ig_coords.assign(d->ig_coords, d->ig_coords + nig * per);
        s.ig_param.assign(d->ig_param_coords, d->ig_param_coords + nig * per);
        if (s.ig_off[0] != 0) return fail(c, FEM_GPU_BAD_ARG, "integration cell offsets must start at 0");
        for (int64_t i = 0; i < s.neq; ++i)
            if (s.ig_off[i + 1] < s.ig_off[i]) return fail(c, FEM_GPU_BAD_ARG, "integration cell offsets");
        for (int64_t k = 0; k < nig * per; ++k)
            if (!std::isfinite(s.ig_coords[k]) || !std::isfinite(s.ig_param[k]))
                return fail(c, FEM_GPU_NONFINITE, "integration cell coordinates");
        if (d->ig_vertex_ids) s.vid.assign(d->ig_vertex_ids, d->ig_vertex_ids + nig * cell_num_nodes(igc));
    }
    if (d->node_density) {
        if (!std::isfinite(d->density_exponent)) return fail(c, FEM_GPU_BAD_ARG, "density exponent");
        s.node_rho.assign(d->node_density, d->node_density + c->num_nodes);
        for (double r : s.node_rho)
            if (!std::isfinite(r) || r < 0.0) return fail(c, FEM_GPU_NONFINITE, "node density must be finite and >= 0");
    }
    s.bulk.node_density = nullptr;
    s.bulk.cluster_ip_cell = nullptr;
    s.bulk.ig_offsets = nullptr;
    s.bulk.ig_coords = nullptr;
    s.bulk.ig_param_coords = nullptr;
    s.bulk.youngs_modulus = nullptr;
    s.bulk.ig_vertex_ids = nullptr;
    c->sets.push_back(std::move(s));
    if (idx) *idx = (int32_t)c->sets.size() - 1;
    return FEM_GPU_OK;
}

fem_gpu_status fem_gpu_add_side_set(fem_gpu_ctx* c, const fem_gpu_side_set_desc* d, int32_t* idx) {
    if (!c || !d) return FEM_GPU_BAD_ARG;
    if (c->host_final) return fail(c, FEM_GPU_BAD_ARG, "sets must be added before finalize");
    if (d->iwg_type != FEM_GPU_IWG_STRUC_LINEAR_NEUMANN &&
        d->iwg_type != FEM_GPU_IWG_STRUC_LINEAR_DIRICHLET_SYMMETRIC_NITSCHE &&
        d->iwg_type != FEM_GPU_IWG_STRUC_LINEAR_DIRICHLET_UNSYMMETRIC_NITSCHE)
        return fail(c, FEM_GPU_UNSUPPORTED, "side iwg type");
    if (d->num_sides < 0 || (d->num_sides > 0 && (!d->side_ip_cell || !d->side_ordinal || !d->youngs_modulus)))
        return fail(c, FEM_GPU_BAD_ARG, "side set arrays");
    int rule = d->integration_rule;
    if (rule == FEM_GPU_RULE_AUTO)
        fem_gpu_auto_integration_rule(FEM_GPU_SET_SIDESET, c->dim == 2 ? FEM_GPU_CELL_LINE2 : FEM_GPU_CELL_QUAD4, 1,
                                      &rule);
    const Rule r = gauss_rule(rule);
    if (r.n == 0 || r.dim != c->dim - 1) return fail(c, FEM_GPU_BAD_ARG, "side integration rule");
    SetData s;
    s.kind = 1;
    s.side = *d;
    s.side.integration_rule = rule;
    if (d->thickness < 0.0 || !std::isfinite(d->thickness)) return fail(c, FEM_GPU_BAD_ARG, "side set thickness");
    s.side_thickness = d->thickness > 0.0 ? d->thickness : 1.0;
    if (d->select_matrix) {
        if (d->iwg_type == FEM_GPU_IWG_STRUC_LINEAR_NEUMANN)
            return fail(c, FEM_GPU_BAD_ARG, "a Select matrix applies to Dirichlet sets only");
        for (int k = 0; k < 9; ++k) s.side_select[k] = 0.0;
        for (int i = 0; i < c->dim; ++i)
            for (int j = 0; j < c->dim; ++j) {
                const double v = d->select_matrix[i * c->dim + j];
                if (!std::isfinite(v)) return fail(c, FEM_GPU_NONFINITE, "select matrix");
                s.side_select[i * 3 + j] = v;
            }
    }
    s.side.select_matrix = nullptr;
    s.neq = d->num_sides;
    s.ip_cell.assign(d->side_ip_cell, d->side_ip_cell + s.neq);
    s.ordinal.assign(d->side_ordinal, d->side_ordinal + s.neq);
    s.E.assign(d->youngs_modulus, d->youngs_modulus + s.neq);
    for (int64_t i = 0; i < s.neq; ++i) {
        int nf = 0;
        if (s.ip_cell[i] < 0 || s.ip_cell[i] >= c->num_cells) return fail(c, FEM_GPU_OOB_INDEX, "side cell");
        if (!facet_vertices(c->ip_cell, s.ordinal[i], &nf)) return fail(c, FEM_GPU_OOB_INDEX, "side ordinal");
    }
    s.side.side_ip_cell = nullptr;
    s.side.side_ordinal = nullptr;
    s.side.youngs_modulus = nullptr;
    c->sets.push_back(std::move(s));
    if (idx) *idx = (int32_t)c->sets.size() - 1;
    return FEM_GPU_OK;
}

fem_gpu_status fem_gpu_add_double_side_set(fem_gpu_ctx* c, const fem_gpu_double_side_set_desc* d, int32_t* idx) {
    if (!c || !d) return FEM_GPU_BAD_ARG;
    if (c->host_final) return fail(c, FEM_GPU_BAD_ARG, "sets must be added before finalize");
    if (d->iwg_type != FEM_GPU_IWG_STRUC_LINEAR_INTERFACE_SYMMETRIC_NITSCHE &&
        d->iwg_type != FEM_GPU_IWG_STRUC_LINEAR_INTERFACE_UNSYMMETRIC_NITSCHE &&
        !is_ghost_iwg(d->iwg_type))
        return fail(c, FEM_GPU_UNSUPPORTED, "double-sided iwg type");
    if (c->dim != 3 || c->ip_cell != FEM_GPU_CELL_HEX8 || d->model_type != FEM_GPU_MODEL_3D)
        return fail(c, FEM_GPU_UNSUPPORTED, "double-sided sets need a 3D HEX8 model");
    if (d->facet_cell_type != FEM_GPU_CELL_TRI3 && d->facet_cell_type != FEM_GPU_CELL_QUAD4)
        return fail(c, FEM_GPU_BAD_ARG, "facet cell type");
    int rule = d->integration_rule;
    if (rule == FEM_GPU_RULE_AUTO)
        fem_gpu_auto_integration_rule(FEM_GPU_SET_DOUBLE_SIDESET, d->facet_cell_type, 1, &rule);
    const Rule r = gauss_rule(rule);
    if (r.n == 0 || r.dim != 2 || r.n > 9) return fail(c, FEM_GPU_BAD_ARG, "facet integration rule");
    const bool tri_rule = rule == FEM_GPU_RULE_TRI_3 || rule == FEM_GPU_RULE_TRI_7;
    if (tri_rule != (d->facet_cell_type == FEM_GPU_CELL_TRI3))
        return fail(c, FEM_GPU_BAD_ARG, "integration rule does not match the facet cell");
    if (d->num_clusters < 0 ||
        (d->num_clusters > 0 && (!d->leader_ip_cell || !d->follower_ip_cell || !d->facet_offsets ||
                                 !d->facet_coords || !d->leader_param_coords || !d->follower_param_coords ||
                                 !d->leader_youngs_modulus || !d->follower_youngs_modulus)))
        return fail(c, FEM_GPU_BAD_ARG, "double-sided set arrays");
    if (!(d->poisson_ratio > -1.0 && d->poisson_ratio < 0.5)) return fail(c, FEM_GPU_BAD_ARG, "poisson ratio");
    if (!std::isfinite(d->alpha)) return fail(c, FEM_GPU_NONFINITE, "alpha");
    SetData s;
    s.kind = 2;
    s.dside = *d;
    s.dside.integration_rule = rule;
    s.neq = d->num_clusters;
    s.nfv = cell_num_nodes(d->facet_cell_type);
    s.ip_cell.assign(d->leader_ip_cell, d->leader_ip_cell + s.neq);
    s.fcell.assign(d->follower_ip_cell, d->follower_ip_cell + s.neq);
    for (int64_t i = 0; i < s.neq; ++i)
        if (s.ip_cell[i] < 0 || s.ip_cell[i] >= c->num_cells || s.fcell[i] < 0 || s.fcell[i] >= c->num_cells)
            return fail(c, FEM_GPU_OOB_INDEX, "double-sided cluster cell");
    if (s.neq) s.fc_off.assign(d->facet_offsets, d->facet_offsets + s.neq + 1);
    else s.fc_off.assign(1, 0);
    if (s.fc_off[0] != 0) return fail(c, FEM_GPU_BAD_ARG, "facet offsets must start at 0");
    for (int64_t i = 0; i < s.neq; ++i)
        if (s.fc_off[i + 1] <= s.fc_off[i]) return fail(c, FEM_GPU_BAD_ARG, "every cluster needs a facet");
    const int64_t nv = s.fc_off[s.neq] * s.nfv * 3;
    s.fc_x.assign(d->facet_coords, d->facet_coords + nv);
    s.fc_xl.assign(d->leader_param_coords, d->leader_param_coords + nv);
    s.fc_xf.assign(d->follower_param_coords, d->follower_param_coords + nv);
    for (int64_t k = 0; k < nv; ++k)
        if (!std::isfinite(s.fc_x[k]) || !std::isfinite(s.fc_xl[k]) || !std::isfinite(s.fc_xf[k]))
            return fail(c, FEM_GPU_NONFINITE, "facet coordinates");
    s.E.assign(d->leader_youngs_modulus, d->leader_youngs_modulus + s.neq);
    s.EF.assign(d->follower_youngs_modulus, d->follower_youngs_modulus + s.neq);
    if (d->facet_vertex_ids) s.vid.assign(d->facet_vertex_ids, d->facet_vertex_ids + s.fc_off[s.neq] * s.nfv);
    for (int64_t i = 0; i < s.neq; ++i)
        if (!(s.E[i] > 0.0) || !(s.EF[i] > 0.0) || !std::isfinite(s.E[i]) || !std::isfinite(s.EF[i]))
            return fail(c, FEM_GPU_NONFINITE, "youngs modulus must be finite and > 0");
    s.dside.leader_ip_cell = s.dside.follower_ip_cell = nullptr;
    s.dside.facet_offsets = nullptr;
    s.dside.facet_coords = s.dside.leader_param_coords = s.dside.follower_param_coords = nullptr;
    s.dside.leader_youngs_modulus = s.dside.follower_youngs_modulus = nullptr;
    s.dside.facet_vertex_ids = nullptr;
    c->sets.push_back(std::move(s));
    if (idx) *idx = (int32_t)c->sets.size() - 1;
    return FEM_GPU_OK;
}

}  // extern "C"

namespace fem {
double ip_cell_measure(const fem_gpu_ctx* c, int64_t cell) {
    const Rule r = gauss_rule(c->dim == 2 ? FEM_GPU_RULE_QUAD_2x2 : FEM_GPU_RULE_HEX_2x2x2);
    const int npe = c->npe, d = c->dim;
    double vol = 0.0;
    for (int q = 0; q < r.n; ++q) {
        double N[8], dN[24], J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        lagrange(c->ip_cell, &r.pts[(size_t)q * r.dim], N, dN);
        for (int i = 0; i < d; ++i)
            for (int j = 0; j < d; ++j)
                for (int a = 0; a < npe; ++a) J[i][j] += dN[i * npe + a] * c->coords[(int64_t)c->cells[cell * npe + a] * d + j];
        const double det = d == 2 ? J[0][0] * J[1][1] - J[0][1] * J[1][0]
                                  : J[0][0] * (J[1][1] * J[2][2] - J[2][1] * J[1][2]) -
                                        J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                                        J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
        vol += r.w[q] * det;
    }
    return vol;
}

fem_gpu_status interface_volumes(fem_gpu_ctx* c) {
    const int dim = c->dim;
    // cluster volumes per IP cell (bulk clusters), for the interface parameter
    std::vector<double> cell_vol;
    bool need_vol = false;
    for (auto& s : c->sets)
        need_vol |= s.kind == 2 && !is_ghost_iwg(s.dside.iwg_type);
    if (need_vol) {
        // only the cells that interface clusters name need a volume
        std::vector<char> needed(c->num_cells, 0);
        for (auto& s : c->sets) {
            if (s.kind != 2 || is_ghost_iwg(s.dside.iwg_type)) continue;
            for (auto v : s.ip_cell) needed[v] = 1;
            for (auto v : s.fcell) needed[v] = 1;
        }
        cell_vol.assign(c->num_cells, 0.0);
        for (auto& s : c->sets) {
            if (s.kind != 0) continue;
            for (int64_t i = 0; i < s.neq; ++i) {
                if (!needed[s.ip_cell[i]]) continue;
                double v = 0.0;
                if (s.ig_off.empty()) {
                    v = ip_cell_measure(c, s.ip_cell[i]);
                } else {
                    const int ign = cell_num_nodes(s.bulk.ig_cell_type);
                    for (int64_t g = s.ig_off[i]; g < s.ig_off[i + 1]; ++g) {
                        const double* x = &s.ig_coords[(size_t)g * ign * dim];
                        if (s.bulk.ig_cell_type == FEM_GPU_CELL_TET4) {
                            double a[3], b[3], cc[3];
                            for (int k = 0; k < 3; ++k) {
                                a[k] = x[0 * 3 + k] - x[2 * 3 + k];
                                b[k] = x[1 * 3 + k] - x[2 * 3 + k];
                                cc[k] = x[3 * 3 + k] - x[2 * 3 + k];
                            }
                            v += std::abs(a[0] * (b[1] * cc[2] - b[2] * cc[1]) - a[1] * (b[0] * cc[2] - b[2] * cc[0]) +
                                          a[2] * (b[0] * cc[1] - b[1] * cc[0])) /
                                 6.0;
                        }
                    }
                }
                cell_vol[s.ip_cell[i]] += v;
            }
        }
    }
    for (auto& s : c->sets) {
        if (s.kind != 2 || is_ghost_iwg(s.dside.iwg_type)) continue;
        s.vol.resize(s.neq * 2);
        for (int64_t i = 0; i < s.neq; ++i) {
            s.vol[i * 2] = cell_vol[s.ip_cell[i]];
            s.vol[i * 2 + 1] = cell_vol[s.fcell[i]];
            if (!(s.vol[i * 2] > 0.0) || !(s.vol[i * 2 + 1] > 0.0))
                return fail(c, FEM_GPU_BAD_ARG, "interface cluster without bulk clusters on its cells");
        }
    }
    return FEM_GPU_OK;
}
}  // namespace fem

extern "C" {

/* MSI work of Model_Solver_Interface::finalize and build_graph:
   - used bases (referenced by a node of a cell of any set) ranked in basis
     order; adof id = type * n_used + rank (Dof_Manager::set_owned_adofs_ids_
     by_type, FEM/MSI/src/cl_MSI_Dof_Manager.cpp:703-744);
   - per equation object the ascending unique basis ranks and the dense
     element extraction T (build_PADofMap, cl_MSI_Equation_Object.cpp:333-364);
   - graph: row (type f, basis b) holds, for every type g, the columns
     g * n_used + U(b), U(b) = union of the basis lists of all equation objects
     containing b (compute_sparsity_pattern, cl_MSI_Solver_Interface.cpp:
     309-588), so each row is ascending and type-major;
   - scatter slots: sidx[e][i][j] = position of basis j inside U(basis i), so
     the CSR position of element entry (f,i; g,j) is
     rowptr[f*n_used + b_i] + g * |U(b_i)| + sidx[e][i][j]. */
fem_gpu_status fem_gpu_finalize_host(fem_gpu_ctx* c) {
    if (!c) return FEM_GPU_BAD_ARG;
    if (c->host_final) return FEM_GPU_OK;
    if (c->sets.empty()) return fail(c, FEM_GPU_BAD_ARG, "no sets");
    int64_t total_eq = 0;
    for (const auto& s : c->sets) total_eq += s.neq;
    if (total_eq == 0) return fail(c, FEM_GPU_BAD_ARG, "no equation objects in any set");
    const int npe = c->npe, dim = c->dim;
    std::vector<char> cell_used(c->num_cells, 0);
    for (auto& s : c->sets) {
        for (auto v : s.ip_cell) cell_used[v] = 1;
        for (auto v : s.fcell) cell_used[v] = 1;
    }
    std::vector<char> used(c->num_bases, 0);
    for (int64_t e = 0; e < c->num_cells; ++e) {
        if (!cell_used[e]) continue;
        for (int a = 0; a < npe; ++a) {
            const int32_t n = c->cells[e * npe + a];
            for (int64_t k = c->t_off[n]; k < c->t_off[n + 1]; ++k) used[c->t_bases[k]] = 1;
        }
    }
    c->basis_rank.assign(c->num_bases, -1);
    int64_t nu = 0;
    for (int64_t b = 0; b < c->num_bases; ++b)
        if (used[b]) c->basis_rank[b] = nu++;
    c->num_used = nu;
    if (nu * dim >= INT32_MAX) return fail(c, FEM_GPU_UNSUPPORTED, "adof count exceeds 32-bit ids");
    // unique sorted basis ranks per used cell
    std::vector<int64_t> cb_off(c->num_cells + 1, 0);
    for (int64_t e = 0; e < c->num_cells; ++e) {
        int64_t n = 0;
        if (cell_used[e])
            for (int a = 0; a < npe; ++a) {
                const int32_t nd = c->cells[e * npe + a];
                n += c->t_off[nd + 1] - c->t_off[nd];
            }
        cb_off[e + 1] = cb_off[e] + n;
    }
    std::vector<int32_t> cb(cb_off[c->num_cells]);
    std::vector<int32_t> cb_len(c->num_cells, 0);
    parallel_for(c->num_cells, [&](int64_t e) {
        if (!cell_used[e]) return;
        int32_t* b = cb.data() + cb_off[e];
        int64_t n = 0;
        for (int a = 0; a < npe; ++a) {
            const int32_t nd = c->cells[e * npe + a];
            for (int64_t k = c->t_off[nd]; k < c->t_off[nd + 1]; ++k) b[n++] = (int32_t)c->basis_rank[c->t_bases[k]];
        }
        std::sort(b, b + n);
        cb_len[e] = (int32_t)(std::unique(b, b + n) - b);
    });
    // basis -> cells adjacency
    std::vector<int64_t> adj_off(nu + 1, 0);
    for (int64_t e = 0; e < c->num_cells; ++e)
        for (int32_t k = 0; k < cb_len[e]; ++k) adj_off[cb[cb_off[e] + k] + 1]++;
    for (int64_t b = 0; b < nu; ++b) adj_off[b + 1] += adj_off[b];
    std::vector<int64_t> adj(adj_off[nu]);
    {
        std::vector<int64_t> fillp(adj_off.begin(), adj_off.end() - 1);
        for (int64_t e = 0; e < c->num_cells; ++e)
            for (int32_t k = 0; k < cb_len[e]; ++k) adj[fillp[cb[cb_off[e] + k]]++] = e;
    }
    // cells coupled to a cell through a double-sided equation object
    std::vector<int64_t> pt_off(c->num_cells + 1, 0);
    for (auto& s : c->sets)
        if (s.kind == 2)
            for (int64_t i = 0; i < s.neq; ++i) {
                pt_off[s.ip_cell[i] + 1]++;
                pt_off[s.fcell[i] + 1]++;
            }
    for (int64_t e = 0; e < c->num_cells; ++e) pt_off[e + 1] += pt_off[e];
    std::vector<int32_t> partners(pt_off[c->num_cells]);
    {
        std::vector<int64_t> fillp(pt_off.begin(), pt_off.end() - 1);
        for (auto& s : c->sets)
            if (s.kind == 2)
                for (int64_t i = 0; i < s.neq; ++i) {
                    partners[fillp[s.ip_cell[i]]++] = s.fcell[i];
                    partners[fillp[s.fcell[i]]++] = s.ip_cell[i];
                }
    }
    // union lists U(b): bases of every equation object that contains b.  Each
    // thread appends the lists of its contiguous basis range to one arena, which
    // then is a contiguous piece of ucols (no per-basis allocations)
    const int unt = range_threads(nu);
    std::vector<std::vector<int32_t>> arena(unt);
    c->ulen.resize(nu);
    parallel_ranges(nu, unt, [&](int t, int64_t b0, int64_t b1) {
        std::vector<int32_t>& out = arena[t];
        std::vector<int32_t> u;
        for (int64_t b = b0; b < b1; ++b) {
            u.clear();
            for (int64_t k = adj_off[b]; k < adj_off[b + 1]; ++k) {
                const int64_t e = adj[k];
                u.insert(u.end(), cb.begin() + cb_off[e], cb.begin() + cb_off[e] + cb_len[e]);
                for (int64_t q = pt_off[e]; q < pt_off[e + 1]; ++q) {
                    const int64_t e2 = partners[q];
                    u.insert(u.end(), cb.begin() + cb_off[e2], cb.begin() + cb_off[e2] + cb_len[e2]);
                }
            }
            std::sort(u.begin(), u.end());
            u.erase(std::unique(u.begin(), u.end()), u.end());
            c->ulen[b] = (int32_t)u.size();
            out.insert(out.end(), u.begin(), u.end());
        }
    });
    c->uoff.assign(nu + 1, 0);
    for (int64_t b = 0; b < nu; ++b) c->uoff[b + 1] = c->uoff[b] + c->ulen[b];
    c->ucols.resize(c->uoff[nu]);
    parallel_ranges(nu, unt, [&](int t, int64_t b0, int64_t) {
        std::copy(arena[t].begin(), arena[t].end(), c->ucols.begin() + c->uoff[b0]);
    });
    arena.clear();
    const int64_t nad = nu * dim;
    c->rowptr.assign(nad + 1, 0);
    int64_t acc = 0;
    for (int f = 0; f < dim; ++f)
        for (int64_t b = 0; b < nu; ++b) {
            c->rowptr[f * nu + b] = (int32_t)acc;
            acc += (int64_t)dim * c->ulen[b];
            if (acc >= INT32_MAX) return fail(c, FEM_GPU_UNSUPPORTED, "nnz exceeds 32-bit offsets");
        }
    c->rowptr[nad] = (int32_t)acc;
    c->nnz = acc;
    // per set element data
    for (auto& s : c->sets) {
        if (s.kind == 2) {
            int maxnb = 0;
            for (int64_t i = 0; i < s.neq; ++i)
                maxnb = std::max(maxnb, std::max(cb_len[s.ip_cell[i]], cb_len[s.fcell[i]]));
            if (2 * maxnb > 255) return fail(c, FEM_GPU_UNSUPPORTED, "more than 255 bases per element");
            s.maxnb = maxnb;
            const int W2 = 2 * maxnb;
            concurrently([&] { s.nb.assign(s.neq * 2, 0); s.bases.assign(s.neq * 2 * maxnb, -1); },
                         [&] { s.T.assign(s.neq * 2 * npe * maxnb, 0.0); },
                         [&] { s.sidx.assign(s.neq * W2 * W2, 0); },
                         [&] { s.xe.resize(s.neq * 2 * npe * dim); });

            std::atomic<bool> bad{false};
            parallel_for(s.neq, [&](int64_t i) {
                int32_t all[512];
                int nall = 0;
                for (int side = 0; side < 2; ++side) {
                    const int64_t e = side == 0 ? s.ip_cell[i] : s.fcell[i];
                    const int32_t n = cb_len[e];
                    const int32_t* b = cb.data() + cb_off[e];
                    s.nb[i * 2 + side] = n;
                    std::copy(b, b + n, s.bases.begin() + (i * 2 + side) * maxnb);
                    for (int k = 0; k < n; ++k) all[nall++] = b[k];
                    for (int k = n; k < maxnb; ++k) all[nall++] = -1;
                    for (int a = 0; a < npe; ++a) {
                        const int32_t nd = c->cells[e * npe + a];
                        for (int d = 0; d < dim; ++d)
                            s.xe[((i * 2 + side) * npe + a) * dim + d] = c->coords[(int64_t)nd * dim + d];
                        for (int64_t k = c->t_off[nd]; k < c->t_off[nd + 1]; ++k) {
                            const int32_t r = (int32_t)c->basis_rank[c->t_bases[k]];
                            const int32_t j = (int32_t)(std::lower_bound(b, b + n, r) - b);
                            s.T[(((i * 2 + side) * npe) + a) * maxnb + j] += c->t_w[k];
                        }
                    }
                }
                for (int ii = 0; ii < W2; ++ii) {
                    if (all[ii] < 0) continue;
                    const int32_t* u = c->ucols.data() + c->uoff[all[ii]];
                    const int32_t ul = c->ulen[all[ii]];
                    for (int jj = 0; jj < W2; ++jj) {
                        if (all[jj] < 0) continue;
                        const int32_t pos = (int32_t)(std::lower_bound(u, u + ul, all[jj]) - u);
                        if (pos >= ul || u[pos] != all[jj] || pos > 65535) bad = true;
                        s.sidx[(i * W2 + ii) * W2 + jj] = (uint16_t)pos;
                    }
                }
            });
            if (bad) return fail(c, FEM_GPU_UNSUPPORTED, "scatter slot does not fit 16 bits");
            continue;
        }
        int maxnb = 0;
        for (int64_t i = 0; i < s.neq; ++i) maxnb = std::max(maxnb, cb_len[s.ip_cell[i]]);
        if (maxnb > 255) return fail(c, FEM_GPU_UNSUPPORTED, "more than 255 bases per element");
        s.maxnb = maxnb;
        concurrently([&] { s.nb.resize(s.neq); s.bases.assign(s.neq * maxnb, -1); },
                     [&] { s.T.assign(s.neq * npe * maxnb, 0.0); },
                     [&] { s.sidx.assign(s.neq * maxnb * maxnb, 0); },
                     [&] { s.xe.resize(s.neq * npe * dim); if (!s.node_rho.empty()) s.rhoe.resize(s.neq * npe); });
        std::atomic<bool> bad{false};
        parallel_for(s.neq, [&](int64_t i) {
            const int64_t e = s.ip_cell[i];
            const int32_t n = cb_len[e];
            const int32_t* b = cb.data() + cb_off[e];
            s.nb[i] = n;
            std::copy(b, b + n, s.bases.begin() + i * maxnb);
            for (int a = 0; a < npe; ++a) {
                const int32_t nd = c->cells[e * npe + a];
                for (int d = 0; d < dim; ++d) s.xe[(i * npe + a) * dim + d] = c->coords[(int64_t)nd * dim + d];
                if (!s.rhoe.empty()) s.rhoe[i * npe + a] = s.node_rho[nd];
                for (int64_t k = c->t_off[nd]; k < c->t_off[nd + 1]; ++k) {
                    const int32_t r = (int32_t)c->basis_rank[c->t_bases[k]];
                    const int32_t j = (int32_t)(std::lower_bound(b, b + n, r) - b);
                    s.T[(i * npe + a) * maxnb + j] += c->t_w[k];
                }
            }
            for (int ii = 0; ii < n; ++ii) {
                const int32_t* u = c->ucols.data() + c->uoff[b[ii]];
                const int32_t ul = c->ulen[b[ii]];
                for (int jj = 0; jj < n; ++jj) {
                    const int32_t pos = (int32_t)(std::lower_bound(u, u + ul, b[jj]) - u);
                    if (pos >= ul || u[pos] != b[jj] || pos > 65535) bad = true;
                    s.sidx[(i * maxnb + ii) * maxnb + jj] = (uint16_t)pos;
                }
            }
        });
        if (bad) return fail(c, FEM_GPU_UNSUPPORTED, "scatter slot does not fit 16 bits");
    }
    fem_gpu_status vst = interface_volumes(c);
    if (vst != FEM_GPU_OK) return vst;
    c->host_final = true;
    return FEM_GPU_OK;
}

fem_gpu_status fem_gpu_get_sizes(const fem_gpu_ctx* c, int64_t* nad, int64_t* nnz, int32_t* nsets) {
    if (!c) return FEM_GPU_BAD_ARG;
    if (!c->host_final) return FEM_GPU_NOT_FINALIZED;
    if (nad) *nad = c->num_used * c->dim;
    if (nnz) *nnz = c->nnz;
    if (nsets) *nsets = (int32_t)c->sets.size();
    return FEM_GPU_OK;
}

fem_gpu_status fem_gpu_get_num_equation_objects(const fem_gpu_ctx* c, int32_t set, int64_t* n) {
    if (!c || !n || set < 0 || set >= (int32_t)c->sets.size()) return FEM_GPU_BAD_ARG;
    *n = c->sets[set].neq;
    return FEM_GPU_OK;
}

fem_gpu_status fem_gpu_get_max_element_adofs(const fem_gpu_ctx* c, int32_t set, int32_t* n) {
    if (!c || !n || set < 0 || set >= (int32_t)c->sets.size()) return FEM_GPU_BAD_ARG;
    if (!c->host_final) return FEM_GPU_NOT_FINALIZED;
    *n = c->sets[set].maxnb * c->dim * (c->sets[set].kind == 2 ? 2 : 1);
    return FEM_GPU_OK;
}

fem_gpu_status fem_gpu_get_element_topology(const fem_gpu_ctx* c, int32_t set, int64_t eq, int32_t* ids,
                                            int32_t* n) {
    if (!c || !ids || !n || set < 0 || set >= (int32_t)c->sets.size()) return FEM_GPU_BAD_ARG;
    if (!c->host_final) return FEM_GPU_NOT_FINALIZED;
    const SetData& s = c->sets[set];
    if (eq < 0 || eq >= s.neq) return FEM_GPU_OOB_INDEX;
    int k = 0;
    const int sides = s.kind == 2 ? 2 : 1;
    for (int side = 0; side < sides; ++side) {
        const int64_t row = eq * sides + side;
        const int nb = s.nb[row];
        for (int f = 0; f < c->dim; ++f)
            for (int j = 0; j < nb; ++j) ids[k++] = (int32_t)(f * c->num_used + s.bases[row * s.maxnb + j]);
    }
    *n = k;
    return FEM_GPU_OK;
}

const char* fem_gpu_last_error(const fem_gpu_ctx* c) { return c ? c->err.c_str() : "null context"; }

int64_t fem_gpu_launch_count(const fem_gpu_ctx* c) { return c ? c->launches : 0; }

}  // extern "C"
