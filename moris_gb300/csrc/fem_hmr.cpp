// fem_hmr.cpp -- hierarchical (refined) HMR B-spline meshes on the host.
//
// A refined tensor-product B-spline hierarchy with HMR's rules, and the
// Lagrange (QUAD4 / HEX8) interpolation mesh of its active elements with the
// extraction row of every node -- the input the element kernels take for the
// uniform level-0 mesh (fem_hmr_uniform_mesh), now on graded meshes.
//
//  * background mesh: ne domain elements per direction and `padding`
//    elements around them (HMR/src/cl_HMR_Parameters.cpp:418-423); padding
//    elements are never active and count as refined, but have children only
//    where they were refined (Background_Element_Base::set_padding_flag,
//    cl_HMR_Background_Element_Base.hpp:225-249);
//  * refinement (Background_Mesh_Base::perform_refinement, cl_HMR_Background_
//    Mesh_Base.cpp:648-737): the queued elements, the padding test of every
//    queued domain element (cl_HMR_Background_Mesh.hpp:1101-1145), the
//    staircase buffer (cl_HMR_Background_Mesh_Base.cpp:1383-1495), repeated
//    until the queue stops growing;
//  * basis states (BSpline_Mesh::determine_basis_state, cl_HMR_BSpline_Mesh.
//    hpp:738-807): a basis is deactivated unless every element of its support
//    exists and is active or refined, active if any of them is active,
//    refined otherwise;
//  * element T matrices (T_Matrix_Base::calculate_untruncated_t_matrix /
//    calculate_truncated_t_matrix, cl_HMR_T_Matrix_Base.cpp:58-248) from the
//    uniform two-scale relation of degree-p B-splines (children 2m-p+j,
//    weights 2^-p C(p+1, j)), in the element-local basis order of HMR's
//    B-spline elements;
//  * node rows (T_Matrix_Base::evaluate, cl_HMR_T_Matrix_Base.cpp:306-457):
//    the element T at the element's corner nodes, |t| <= 1e-12 dropped, set by
//    the first element that visits the node.
//
// Element and basis indices are kept per level in "mesh" coordinates counted
// from the first padding element (a level-l basis m has the support elements
// m-p .. m per direction); the C ABI uses domain-relative indices.

#include <algorithm>
#include <cmath>
#include <cstring>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "fem_internal.hpp"

namespace {

constexpr int kMaxLevel = 15;
constexpr int kIdxBits = 20;  // per direction and level: up to 2^20 elements

// element-local basis order of HMR's B-spline elements (Quad4/9/16, Hex8/27/64):
// the ijk offsets of local basis k, as digits
const char* local_order_string(int dim, int p) {
    if (dim == 2) {
        if (p == 1) return "00 10 11 01";
        if (p == 2) return "00 20 22 02 10 21 12 01 11";
        if (p == 3) return "00 30 33 03 10 20 31 32 23 13 02 01 11 21 22 12";
    } else {
        if (p == 1) return "000 100 110 010 001 101 111 011";
        if (p == 2)
            return "000 200 220 020 002 202 222 022 100 210 120 010 001 201 221 021 102 212 122 012 111 110 112 "
                   "011 211 101 121";
        if (p == 3)
            return "000 300 330 030 003 303 333 033 100 200 010 020 001 002 310 320 301 302 230 130 331 332 031 "
                   "032 103 203 013 023 313 323 233 133 110 120 220 210 101 201 202 102 011 012 022 021 311 321 "
                   "322 312 231 131 132 232 113 213 223 123 111 211 221 121 112 212 222 122";
    }
    return nullptr;
}

struct Idx {
    int64_t v[3] = {0, 0, 0};
};

inline uint64_t pack(const Idx& e) {
    return (uint64_t)e.v[0] | ((uint64_t)e.v[1] << kIdxBits) | ((uint64_t)e.v[2] << (2 * kIdxBits));
}

double cardinal(int p, double t) {
    // uniform cardinal B-spline of degree p on [0, p + 1] (Cox-de Boor, half-open spans)
    if (p == 0) return (t >= 0.0 && t < 1.0) ? 1.0 : 0.0;
    return (t * cardinal(p - 1, t) + (p + 1 - t) * cardinal(p - 1, t - 1.0)) / p;
}

}  // namespace

struct fem_hmr_refined {
    int dim = 0, p = 0, buffer = 0, half_buffer = 0, pad = 0, pr = 0;
    int64_t ne[3] = {1, 1, 1};
    double len[3] = {1, 1, 1};
    std::vector<std::unordered_set<uint64_t>> refined = std::vector<std::unordered_set<uint64_t>>(kMaxLevel + 1);
    std::vector<Idx> local;  // element-local basis offsets
    int nloc = 0;

    int64_t count(int l, int k) const { return (ne[k] + 2 * pad) << l; }
    bool inside(int l, const Idx& e) const {
        for (int k = 0; k < dim; ++k)
            if (e.v[k] < 0 || e.v[k] >= count(l, k)) return false;
        return true;
    }
    Idx parent(const Idx& e) const {
        Idx q;
        for (int k = 0; k < dim; ++k) q.v[k] = e.v[k] >> 1;
        return q;
    }
    bool is_refined(int l, const Idx& e) const { return refined[l].count(pack(e)) != 0; }
    bool exists(int l, const Idx& e) const { return inside(l, e) && (l == 0 || is_refined(l - 1, parent(e))); }
    bool padding(int l, const Idx& e) const {
        for (int k = 0; k < dim; ++k)
            if (e.v[k] < ((int64_t)pad << l) || e.v[k] >= ((pad + ne[k]) << l)) return true;
        return false;
    }
    bool active(int l, const Idx& e) const { return exists(l, e) && !is_refined(l, e) && !padding(l, e); }

    template <class F>
    void neighbours(int l, const Idx& e, int r, F&& f) const {
        const int span = 2 * r + 1;
        int tot = 1;
        for (int k = 0; k < dim; ++k) tot *= span;
        for (int c = 0; c < tot; ++c) {
            Idx n;
            int rem = c;
            bool self = true;
            for (int k = 0; k < dim; ++k) {
                const int o = rem % span - r;
                rem /= span;
                n.v[k] = e.v[k] + o;
                self &= o == 0;
            }
            if (!self && exists(l, n)) f(n);
        }
    }

    // 0 deactivated, 1 active, 2 refined
    int basis_state(int l, const Idx& m) const {
        int tot = 1;
        for (int k = 0; k < dim; ++k) tot *= p + 1;
        bool any_active = false;
        for (int c = 0; c < tot; ++c) {
            Idx e;
            int rem = c;
            for (int k = 0; k < dim; ++k) {
                e.v[k] = m.v[k] - rem % (p + 1);
                rem /= p + 1;
            }
            if (!exists(l, e)) return 0;
            any_active |= active(l, e);
        }
        return any_active ? 1 : 2;
    }

    Idx local_basis(const Idx& e, int k) const {
        Idx m;
        for (int d = 0; d < dim; ++d) m.v[d] = e.v[d] + local[k].v[d];
        return m;
    }
};

namespace {

// the children of basis m (level l) on level l + 1 with their weights
void basis_children(const fem_hmr_refined* h, const Idx& m, std::vector<std::pair<Idx, double>>& out) {
    out.clear();
    const int n = h->p + 2;
    std::vector<double> w1(n);
    for (int j = 0; j < n; ++j) {
        double c = 1.0;  // C(p+1, j)
        for (int i = 1; i <= j; ++i) c = c * (h->p + 2 - i) / i;
        w1[j] = c / std::pow(2.0, h->p);
    }
    int tot = 1;
    for (int k = 0; k < h->dim; ++k) tot *= n;
    for (int c = 0; c < tot; ++c) {
        Idx ch;
        double w = 1.0;
        int rem = c;
        for (int k = 0; k < h->dim; ++k) {
            const int j = rem % n;
            rem /= n;
            ch.v[k] = 2 * m.v[k] - h->p + j;
            w *= w1[j];
        }
        out.push_back({ch, w});
    }
}

// C[i][k] (nloc x nloc, row-major): local basis i of child element e (level l)
// in the parent element's local basis k
void child_matrix(const fem_hmr_refined* h, int l, const Idx& e, std::vector<double>& C) {
    const int B = h->nloc;
    C.assign((size_t)B * B, 0.0);
    std::unordered_map<uint64_t, int> idx;
    for (int i = 0; i < B; ++i) idx[pack(h->local_basis(e, i))] = i;
    const Idx par = h->parent(e);
    std::vector<std::pair<Idx, double>> ch;
    for (int k = 0; k < B; ++k) {
        basis_children(h, h->local_basis(par, k), ch);
        for (auto& c : ch) {
            auto it = idx.find(pack(c.first));
            if (it != idx.end()) C[(size_t)it->second * B + k] += c.second;
        }
    }
    (void)l;
}

struct Dof {
    int level;
    Idx m;
};

// element T (nloc x ndof, column-major by dof) and its dofs
void element_t(const fem_hmr_refined* h, int l, const Idx& e, bool truncate, std::vector<double>& T,
               std::vector<Dof>& dofs) {
    const int B = h->nloc;
    T.clear();
    dofs.clear();
    if (!truncate) {
        std::vector<double> cur((size_t)B * B, 0.0), C, nxt;
        for (int i = 0; i < B; ++i) cur[(size_t)i * B + i] = 1.0;
        Idx el = e;
        for (int lev = l; lev >= 0; --lev) {
            for (int k = 0; k < B; ++k) {
                const Idx m = h->local_basis(el, k);
                if (h->basis_state(lev, m) == 1) {
                    for (int i = 0; i < B; ++i) T.push_back(cur[(size_t)i * B + k]);
                    dofs.push_back({lev, m});
                }
            }
            if (lev > 0) {
                child_matrix(h, lev, el, C);
                nxt.assign((size_t)B * B, 0.0);
                for (int i = 0; i < B; ++i)
                    for (int j = 0; j < B; ++j) {
                        double s = 0.0;
                        for (int k = 0; k < B; ++k) s += cur[(size_t)i * B + k] * C[(size_t)k * B + j];
                        nxt[(size_t)i * B + j] = s;
                    }
                cur.swap(nxt);
                el = h->parent(el);
            }
        }
        return;
    }
    std::unordered_map<uint64_t, int> idx;
    for (int k = 0; k < B; ++k) {
        const Idx m = h->local_basis(e, k);
        idx[pack(m)] = k;
        if (h->basis_state(l, m) == 1) {
            for (int i = 0; i < B; ++i) T.push_back(i == k ? 1.0 : 0.0);
            dofs.push_back({l, m});
        }
    }
    if (l == 0) return;
    const Idx par = h->parent(e);
    std::vector<std::pair<Idx, double>> ch;
    std::vector<double> col(B);
    for (int k = 0; k < B; ++k) {
        const Idx m = h->local_basis(par, k);
        if (h->basis_state(l - 1, m) != 1) continue;
        std::fill(col.begin(), col.end(), 0.0);
        basis_children(h, m, ch);
        for (auto& c : ch) {
            auto it = idx.find(pack(c.first));
            if (it != idx.end() && h->basis_state(l, c.first) == 0) col[it->second] += c.second;
        }
        double lo = 0.0, hi = 0.0;
        for (double v : col) {
            lo = std::min(lo, v);
            hi = std::max(hi, v);
        }
        if (lo < -1e-12 || hi > 1e-12) {
            T.insert(T.end(), col.begin(), col.end());
            dofs.push_back({l - 1, m});
        }
    }
}

void refine(fem_hmr_refined* h, std::vector<std::pair<int, Idx>> queue) {
    std::unordered_set<uint64_t> queued[kMaxLevel + 1];
    auto push = [&](int l, const Idx& e) {
        if (queued[l].insert(pack(e)).second) queue.push_back({l, e});
    };
    std::vector<std::pair<int, Idx>> init;
    init.swap(queue);
    for (auto& q : init) push(q.first, q.second);
    auto padding_test = [&]() {
        const size_t n = queue.size();
        for (size_t i = 0; i < n; ++i) {
            const int l = queue[i].first;
            const Idx e = queue[i].second;
            if (h->padding(l, e)) continue;  // padding elements belong to no processor
            bool near = false;
            for (int k = 0; k < h->dim; ++k) {
                const int64_t lo = (int64_t)h->pad << l, hi = ((h->pad + h->ne[k]) << l) - 1;
                near |= e.v[k] < lo + h->pr || e.v[k] > hi - h->pr;
            }
            if (!near) continue;
            h->neighbours(l, e, h->pr, [&](const Idx& f) {
                if (h->padding(l, f)) push(l, f);
            });
        }
    };
    // staircase buffer: active coarser neighbours of the parent near the element
    std::vector<std::pair<int, Idx>> stack;
    auto staircase = [&](int l0, const Idx& e0) {
        stack.push_back({l0, e0});
        while (!stack.empty()) {
            const int l = stack.back().first;
            const Idx e = stack.back().second;
            stack.pop_back();
            if (l == 0) continue;
            h->neighbours(l - 1, h->parent(e), h->half_buffer, [&](const Idx& f) {
                if (!h->active(l - 1, f) || queued[l - 1].count(pack(f))) return;
                int64_t dist = 0;
                for (int k = 0; k < h->dim; ++k) {
                    const int64_t ni = 2 * f.v[k];
                    dist = std::max(dist, ni >= e.v[k] ? ni - e.v[k] : e.v[k] - ni - 1);
                }
                if (dist <= h->buffer) {
                    push(l - 1, f);
                    stack.push_back({l - 1, f});
                }
            });
        }
    };
    padding_test();
    for (;;) {
        const size_t n = queue.size();
        for (size_t i = 0; i < n; ++i) staircase(queue[i].first, queue[i].second);
        padding_test();
        if (queue.size() == n) break;
    }
    for (auto& q : queue) h->refined[q.first].insert(pack(q.second));
}

int max_level(const fem_hmr_refined* h) {
    int L = 0;
    for (int l = 0; l < kMaxLevel; ++l)
        if (!h->refined[l].empty()) L = l + 1;
    return L;
}

// active domain elements: coarsest domain elements (x fastest), each followed
// by its active descendants in child order (x fastest)
void leaves(const fem_hmr_refined* h, std::vector<std::pair<int, Idx>>& out) {
    out.clear();
    std::vector<std::pair<int, Idx>> stack;
    int64_t n0 = 1;
    for (int k = 0; k < h->dim; ++k) n0 *= h->ne[k];
    for (int64_t c = 0; c < n0; ++c) {
        Idx e;
        int64_t rem = c;
        for (int k = 0; k < h->dim; ++k) {
            e.v[k] = h->pad + rem % h->ne[k];
            rem /= h->ne[k];
        }
        stack.push_back({0, e});
        while (!stack.empty()) {
            const int l = stack.back().first;
            const Idx x = stack.back().second;
            stack.pop_back();
            if (!h->is_refined(l, x)) {
                out.push_back({l, x});
                continue;
            }
            const int nch = 1 << h->dim;
            for (int ci = nch - 1; ci >= 0; --ci) {  // reversed: child 0 is visited first
                Idx y;
                for (int k = 0; k < h->dim; ++k) y.v[k] = 2 * x.v[k] + ((ci >> k) & 1);
                stack.push_back({l + 1, y});
            }
        }
    }
}

// the hierarchy in the device's form (sorted keys per refined level)
fem::HmrDevice device_form(const fem_hmr_refined* h) {
    fem::HmrDevice d;
    d.dim = h->dim;
    d.p = h->p;
    d.pad = h->pad;
    d.nloc = h->nloc;
    d.levels = max_level(h);
    for (int k = 0; k < 3; ++k) d.ne[k] = h->ne[k];
    for (int b = 0; b < h->nloc; ++b)
        for (int k = 0; k < 3; ++k) d.local[b][k] = (int)h->local[b].v[k];
    d.koff.push_back(0);
    for (int l = 0; l < d.levels; ++l) {
        std::vector<uint64_t> ks(h->refined[l].begin(), h->refined[l].end());
        std::sort(ks.begin(), ks.end());
        d.keys.insert(d.keys.end(), ks.begin(), ks.end());
        d.koff.push_back((int64_t)d.keys.size());
    }
    return d;
}

// element T matrices of a list of elements on the GPU: per element its
// columns (column-major by dof) and dofs
fem_gpu_status element_t_device(const fem_hmr_refined* h, const std::vector<std::pair<int, Idx>>& els,
                                bool truncate, std::vector<std::vector<double>>& Ts,
                                std::vector<std::vector<Dof>>& Ds) {
    const int64_t n = (int64_t)els.size();
    const fem::HmrDevice d = device_form(h);
    std::vector<int32_t> lv(n), nd(n);
    std::vector<int64_t> ix((size_t)n * 3), toff(n + 1, 0);
    for (int64_t i = 0; i < n; ++i) {
        lv[i] = els[i].first;
        for (int k = 0; k < 3; ++k) ix[i * 3 + k] = els[i].second.v[k];
    }
    fem_gpu_status st = fem::hmr_element_t_device(d, truncate, n, lv.data(), ix.data(), nd.data(), nullptr,
                                                  nullptr, nullptr);
    if (st != FEM_GPU_OK) return st;
    for (int64_t i = 0; i < n; ++i) toff[i + 1] = toff[i] + (int64_t)nd[i] * h->nloc;
    std::vector<double> T((size_t)std::max<int64_t>(toff[n], 1));
    std::vector<int64_t> dofs((size_t)std::max<int64_t>(toff[n] / h->nloc, 1) * 4);
    st = fem::hmr_element_t_device(d, truncate, n, lv.data(), ix.data(), nd.data(), toff.data(), T.data(),
                                   dofs.data());
    if (st != FEM_GPU_OK) return st;
    Ts.assign(n, {});
    Ds.assign(n, {});
    for (int64_t i = 0; i < n; ++i) {
        Ts[i].assign(T.begin() + toff[i], T.begin() + toff[i + 1]);
        const int64_t d0 = toff[i] / h->nloc;
        for (int j = 0; j < nd[i]; ++j) {
            Dof df;
            df.level = (int)dofs[(d0 + j) * 4];
            for (int k = 0; k < 3; ++k) df.m.v[k] = dofs[(d0 + j) * 4 + 1 + k];
            Ds[i].push_back(df);
        }
    }
    return FEM_GPU_OK;
}

fem_gpu_status check_ijk(const fem_hmr_refined* h, int level, const int32_t* ijk, Idx& e) {
    if (level < 0 || level >= kMaxLevel || !ijk) return FEM_GPU_BAD_ARG;
    for (int k = 0; k < h->dim; ++k) e.v[k] = (int64_t)ijk[k] + ((int64_t)h->pad << level);
    return h->exists(level, e) ? FEM_GPU_OK : FEM_GPU_OOB_INDEX;
}

}  // namespace

extern "C" {

fem_gpu_status fem_hmr_refined_create(int32_t dim, const int32_t* num_elements, const double* lengths,
                                      int32_t order, int32_t staircase_buffer, int32_t padding_refinement,
                                      fem_hmr_refined** out) {
    if (!out || !num_elements || !lengths || (dim != 2 && dim != 3) || order < 1 || order > 3 ||
        staircase_buffer < 0 || padding_refinement < 0)
        return FEM_GPU_BAD_ARG;
    *out = nullptr;
    auto* h = new fem_hmr_refined;
    h->dim = dim;
    h->p = order;
    h->buffer = staircase_buffer;
    h->half_buffer = (staircase_buffer + 1) / 2;
    h->pad = std::max(staircase_buffer, order);
    h->pr = padding_refinement;
    for (int k = 0; k < dim; ++k) {
        if (num_elements[k] < 1 || !(lengths[k] > 0.0) ||
            ((int64_t)num_elements[k] + 2 * h->pad) >= ((int64_t)1 << (kIdxBits - kMaxLevel))) {
            delete h;
            return FEM_GPU_BAD_ARG;
        }
        h->ne[k] = num_elements[k];
        h->len[k] = lengths[k];
    }
    const char* s = local_order_string(dim, order);
    for (const char* c = s; *c;) {
        Idx o;
        for (int k = 0; k < dim; ++k) o.v[k] = c[k] - '0';
        h->local.push_back(o);
        c += dim;
        while (*c == ' ') ++c;
    }
    h->nloc = (int)h->local.size();
    *out = h;
    return FEM_GPU_OK;
}

fem_gpu_status fem_hmr_refined_free(fem_hmr_refined* h) {
    delete h;
    return FEM_GPU_OK;
}

fem_gpu_status fem_hmr_refined_refine(fem_hmr_refined* h, int64_t count, const int32_t* levels, const int32_t* ijk) {
    if (!h || count < 0 || (count > 0 && (!levels || !ijk))) return FEM_GPU_BAD_ARG;
    std::vector<std::pair<int, Idx>> q;
    for (int64_t i = 0; i < count; ++i) {
        Idx e;
        const fem_gpu_status st = check_ijk(h, levels[i], ijk + i * h->dim, e);
        if (st != FEM_GPU_OK) return st;
        if (levels[i] + 1 >= kMaxLevel) return FEM_GPU_UNSUPPORTED;
        if (!h->active(levels[i], e)) return FEM_GPU_BAD_ARG;  // only active domain elements are refined
        q.push_back({levels[i], e});
    }
    refine(h, std::move(q));
    return FEM_GPU_OK;
}

fem_gpu_status fem_hmr_refined_active_elements(const fem_hmr_refined* h, int64_t* count, int32_t* levels,
                                               int32_t* ijk) {
    if (!h || !count) return FEM_GPU_BAD_ARG;
    std::vector<std::pair<int, Idx>> lv;
    leaves(h, lv);
    if (levels && ijk)
        for (size_t i = 0; i < lv.size(); ++i) {
            levels[i] = lv[i].first;
            for (int k = 0; k < h->dim; ++k)
                ijk[i * h->dim + k] = (int32_t)(lv[i].second.v[k] - ((int64_t)h->pad << lv[i].first));
        }
    *count = (int64_t)lv.size();
    return FEM_GPU_OK;
}

fem_gpu_status fem_hmr_refined_element_t_matrix(const fem_hmr_refined* h, int32_t level, const int32_t* ijk,
                                                int32_t truncate, int32_t capacity, int32_t* ndof, double* T,
                                                int32_t* dof_level, int32_t* dof_ijk) {
    if (!h || !ndof) return FEM_GPU_BAD_ARG;
    Idx e;
    const fem_gpu_status st = check_ijk(h, level, ijk, e);
    if (st != FEM_GPU_OK) return st;
    std::vector<double> t;
    std::vector<Dof> dofs;
    element_t(h, level, e, truncate != 0, t, dofs);
    *ndof = (int32_t)dofs.size();
    if (!T && !dof_level && !dof_ijk) return FEM_GPU_OK;  // size query
    if ((int32_t)dofs.size() > capacity) return FEM_GPU_BAD_ARG;
    const int B = h->nloc, nd = (int)dofs.size();
    for (int j = 0; j < nd; ++j) {
        if (T)
            for (int i = 0; i < B; ++i) T[(size_t)i * nd + j] = t[(size_t)j * B + i];  // row-major [B][nd]
        if (dof_level) dof_level[j] = dofs[j].level;
        if (dof_ijk)
            for (int k = 0; k < h->dim; ++k)
                dof_ijk[j * h->dim + k] = (int32_t)(dofs[j].m.v[k] - ((int64_t)h->pad << dofs[j].level));
    }
    return FEM_GPU_OK;
}

// The Lagrange mesh of the active elements with the node rows, the element T
// matrices and node rows computed on the host or on the GPU (the same
// numbers: see fem_hmr_device.cu)
static fem_gpu_status build_mesh(const fem_hmr_refined* h, bool truncate, bool device, fem_hmr_mesh** out) {
    if (!h || !out) return FEM_GPU_BAD_ARG;
    *out = nullptr;
    const int D = h->dim, L = max_level(h), npe = D == 2 ? 4 : 8, B = h->nloc;
    std::vector<std::pair<int, Idx>> lv;
    leaves(h, lv);
    // element T matrices and the active bases they use, numbered by (level, ijk x fastest)
    std::vector<std::vector<double>> Ts(lv.size());
    std::vector<std::vector<Dof>> Ds(lv.size());
    if (device) {
        const fem_gpu_status st = element_t_device(h, lv, truncate, Ts, Ds);
        if (st != FEM_GPU_OK) return st;
    } else {
        for (size_t i = 0; i < lv.size(); ++i) element_t(h, lv[i].first, lv[i].second, truncate, Ts[i], Ds[i]);
    }
    std::vector<std::pair<uint64_t, Dof>> used;
    std::unordered_set<uint64_t> seen;
    auto dof_key = [&](const Dof& d) {
        uint64_t key = (uint64_t)d.level;
        for (int k = D - 1; k >= 0; --k) key = (key << kIdxBits) | (uint64_t)d.m.v[k];
        return key;  // level, then z, y, x
    };
    for (size_t i = 0; i < lv.size(); ++i)
        for (auto& d : Ds[i])
            if (seen.insert(dof_key(d)).second) used.push_back({dof_key(d), d});
    std::sort(used.begin(), used.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
    std::unordered_map<uint64_t, int32_t> bid;
    for (size_t i = 0; i < used.size(); ++i) bid[used[i].first] = (int32_t)i;
    auto* m = new fem_hmr_mesh;
    m->dim = D;
    m->num_bases = (int64_t)used.size();
    m->t_off.push_back(0);
    // nodes by first visit; the first visit evaluates the node's row
    std::unordered_map<uint64_t, int32_t> node;
    std::vector<int64_t> first_elem;
    const int corner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
    for (size_t i = 0; i < lv.size(); ++i) {
        const int l = lv[i].first;
        const Idx& e = lv[i].second;
        for (int a = 0; a < npe; ++a) {
            Idx key;
            for (int k = 0; k < D; ++k) key.v[k] = (e.v[k] + corner[a][k]) << (L - l);
            auto it = node.find(pack(key));
            if (it == node.end()) {
                const int32_t id = (int32_t)(m->coords.size() / D);
                it = node.emplace(pack(key), id).first;
                for (int k = 0; k < D; ++k) {
                    const double hL = h->len[k] / h->ne[k] / std::pow(2.0, L);
                    m->coords.push_back((double)(key.v[k] - ((int64_t)h->pad << L)) * hL);
                }
                first_elem.push_back((int64_t)i);
            }
            m->cells.push_back(it->second);
        }
    }
    const int64_t nn = (int64_t)first_elem.size();
    // the rows: the element's local B-splines at the node, times its T
    std::vector<int64_t> roff(nn + 1, 0);
    for (int64_t k = 0; k < nn; ++k) roff[k + 1] = roff[k] + (int64_t)Ds[first_elem[k]].size();
    std::vector<double> rows((size_t)std::max<int64_t>(roff[nn], 1));
    if (device) {
        std::vector<int32_t> lvl(lv.size()), nd(lv.size());
        std::vector<int64_t> ix(lv.size() * 3), toff(lv.size() + 1, 0);
        for (size_t i = 0; i < lv.size(); ++i) {
            lvl[i] = lv[i].first;
            nd[i] = (int32_t)Ds[i].size();
            for (int k = 0; k < 3; ++k) ix[i * 3 + k] = lv[i].second.v[k];
            toff[i + 1] = toff[i] + (int64_t)Ts[i].size();
        }
        std::vector<double> Tflat((size_t)std::max<int64_t>(toff[lv.size()], 1));
        for (size_t i = 0; i < lv.size(); ++i) std::copy(Ts[i].begin(), Ts[i].end(), Tflat.begin() + toff[i]);
        const fem::HmrDevice d = device_form(h);
        const fem_gpu_status st =
            fem::hmr_node_rows_device(d, h->len, nn, first_elem.data(), m->coords.data(), lvl.data(), ix.data(),
                                      nd.data(), toff.data(), Tflat.data(), roff.data(), rows.data());
        if (st != FEM_GPU_OK) {
            delete m;
            return st;
        }
    } else {
        for (int64_t k = 0; k < nn; ++k) {
            const size_t i = (size_t)first_elem[k];
            const int l = lv[i].first;
            const Idx& e = lv[i].second;
            const double* x = m->coords.data() + k * D;
            std::vector<double> lag(B);
            for (int b = 0; b < B; ++b) {
                const Idx mb = h->local_basis(e, b);
                double v = 1.0;
                for (int kk = 0; kk < D; ++kk) {
                    const double hl = h->len[kk] / h->ne[kk] / std::pow(2.0, l);
                    const double t = (x[kk] + h->pad * h->len[kk] / h->ne[kk]) / hl - (double)(mb.v[kk] - h->p);
                    v *= cardinal(h->p, t);
                }
                lag[b] = v;
            }
            const int nd = (int)Ds[i].size();
            for (int j = 0; j < nd; ++j) {
                double s = 0.0;
                for (int b = 0; b < B; ++b) s += lag[b] * Ts[i][(size_t)j * B + b];
                rows[roff[k] + j] = s;
            }
        }
    }
    for (int64_t k = 0; k < nn; ++k) {
        const auto& Di = Ds[first_elem[k]];
        for (size_t j = 0; j < Di.size(); ++j) {
            const double s = rows[roff[k] + j];
            if (std::abs(s) > 1e-12) {
                m->t_bases.push_back(bid[dof_key(Di[j])]);
                m->t_w.push_back(s);
            }
        }
        m->t_off.push_back((int64_t)m->t_bases.size());
    }
    *out = m;
    return FEM_GPU_OK;
}

fem_gpu_status fem_hmr_refined_mesh(const fem_hmr_refined* h, int32_t truncate, fem_hmr_mesh** out) {
    return build_mesh(h, truncate != 0, false, out);
}

fem_gpu_status fem_hmr_refined_mesh_device(const fem_hmr_refined* h, int32_t truncate, fem_hmr_mesh** out) {
    return build_mesh(h, truncate != 0, true, out);
}

fem_gpu_status fem_hmr_refined_element_t_matrices_device(const fem_hmr_refined* h, int32_t truncate, int64_t count,
                                                         const int32_t* levels, const int32_t* ijk,
                                                         int32_t capacity, int32_t* ndof, double* T,
                                                         int32_t* dof_level, int32_t* dof_ijk) {
    if (!h || count < 0 || (count > 0 && (!levels || !ijk || !ndof))) return FEM_GPU_BAD_ARG;
    std::vector<std::pair<int, Idx>> els;
    for (int64_t i = 0; i < count; ++i) {
        Idx e;
        const fem_gpu_status st = check_ijk(h, levels[i], ijk + i * h->dim, e);
        if (st != FEM_GPU_OK) return st;
        els.push_back({levels[i], e});
    }
    std::vector<std::vector<double>> Ts;
    std::vector<std::vector<Dof>> Ds;
    const fem_gpu_status st = element_t_device(h, els, truncate != 0, Ts, Ds);
    if (st != FEM_GPU_OK) return st;
    const int B = h->nloc;
    bool fits = true;
    for (int64_t i = 0; i < count; ++i) {
        const int nd = (int)Ds[i].size();
        ndof[i] = nd;
        if (nd > capacity) {
            fits = false;
            continue;
        }
        for (int j = 0; j < nd; ++j) {
            if (T)
                for (int b = 0; b < B; ++b) T[((size_t)i * B + b) * capacity + j] = Ts[i][(size_t)j * B + b];
            if (dof_level) dof_level[i * capacity + j] = Ds[i][j].level;
            if (dof_ijk)
                for (int k = 0; k < h->dim; ++k)
                    dof_ijk[(i * capacity + j) * h->dim + k] =
                        (int32_t)(Ds[i][j].m.v[k] - ((int64_t)h->pad << Ds[i][j].level));
        }
    }
    if (!T && !dof_level && !dof_ijk) return FEM_GPU_OK;  // size query
    return fits ? FEM_GPU_OK : FEM_GPU_BAD_ARG;
}

}  // extern "C"
