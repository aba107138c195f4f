// fem_xtk_device.cu -- the XFEM decomposition of fem_xtk.cpp on the device.
//
// Same input and the same fem_xtk_model, array for array, as
// fem_xtk_decompose; every per-cell and per-basis step runs on the GPU and the
// numberings that the host builds by first touch are rebuilt with stable sorts:
//  1. cells: phases present, cut flag (a thread per cell); cut cells compacted
//     in cell order;
//  2. face centres: the host takes a face centre's level set and position from
//     the first cut cell that touches it (in that cell's corner order); every
//     cut cell emits its six face keys, a stable sort groups them, and the
//     first entry of a group (the lowest cut cell) computes the face;
//  3. per cut cell (a thread): the 24-tet subdivision and the conformal cut,
//     first counting tets, facets and vertex requests, then writing the
//     requests in the host's visiting order (corners, centre, faces, cut edges
//     in subdivision order);
//  4. IG vertex ids: a stable sort of the requests by entity gives every entity
//     its first touch, a sort of the entities by first touch its id (the host
//     hands out ids in first-touch order);
//  5. the vertex table: kinds 0-2 from their parents, then the intersection
//     vertices, whose edge coordinate runs from the lower id to the higher;
//  6. per cut cell again: tets and interface facets with ids, parametric
//     coordinates and orientation, at the cell's offsets;
//  7. enrichment: a thread per basis, flood fill of its support per phase;
//  8. unzipped vertices: the enriched extraction row of every (enriched cell,
//     corner), deduplicated by a sort on a hash of (node, row) with an exact
//     comparison, numbered by first touch;
//  9. clusters and ghost facets by compaction in the host's loop order.
// The file is compiled without FMA contraction, like the host code, so the
// floating-point results are the host's bit for bit.
#include <cub/cub.cuh>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "fem_internal.hpp"
#include "fem_xtk.hpp"

using fem::IgVertex;

namespace {

__constant__ int c_sides[6][4];
__constant__ double c_xi[8][3];

// self-checks: the first failed check records (code, index) and the access is skipped
__device__ unsigned long long g_fault[2];
__device__ inline bool ok_or_record(bool ok, int code, int64_t index) {
    if (!ok && atomicCAS(&g_fault[0], 0ull, (unsigned long long)code) == 0ull) g_fault[1] = (unsigned long long)index;
    return ok;
}

enum : uint64_t { kNode = 0, kFace = 1, kCell = 2, kEdge = 3 };
constexpr int kIdBits = 29;  // ids of nodes, faces (3 x nodes) and cells

__host__ __device__ inline uint64_t vcode(uint64_t kind, uint64_t id) { return (kind << kIdBits) | id; }
__host__ __device__ inline uint64_t ekey_of_code(uint64_t code) {
    return ((code >> kIdBits) << 62) | (code & ((1ull << kIdBits) - 1));
}
__device__ inline uint64_t edge_key(uint64_t ca, uint64_t cb) {
    const uint64_t lo = ca < cb ? ca : cb, hi = ca < cb ? cb : ca;
    return (kEdge << 62) | (lo << 31) | hi;
}
__device__ inline int phase_of(double phi) { return phi < 0.0 ? 1 : 0; }

template <typename T>
struct DevVec {
    T* p = nullptr;
    size_t n = 0;
    DevVec() = default;
    DevVec(const DevVec&) = delete;
    ~DevVec() { cudaFree(p); }
    bool alloc(size_t count) {
        cudaFree(p);
        p = nullptr;
        n = count;
        return cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)) == cudaSuccess;
    }
    bool upload(const T* h, size_t count) {
        return alloc(count) && cudaMemcpy(p, h, count * sizeof(T), cudaMemcpyHostToDevice) == cudaSuccess;
    }
    bool download(std::vector<T>& h, size_t count) const {
        h.resize(count);
        return count == 0 || cudaMemcpy(h.data(), p, count * sizeof(T), cudaMemcpyDeviceToHost) == cudaSuccess;
    }
};

// CUB two-phase calls with a scratch buffer
template <typename F>
bool cub_run(F f) {
    size_t bytes = 0;
    if (f(nullptr, bytes) != cudaSuccess) return false;
    void* tmp = nullptr;
    if (cudaMalloc(&tmp, std::max<size_t>(bytes, 16)) != cudaSuccess) return false;
    const bool ok = f(tmp, bytes) == cudaSuccess;
    cudaFree(tmp);
    return ok;
}

template <typename T>
bool exclusive_scan(const T* in, T* out, int64_t n) {
    return cub_run([&](void* t, size_t& b) { return cub::DeviceScan::ExclusiveSum(t, b, in, out, (int)n); });
}

// stable sort of (key, value) pairs
template <typename K, typename V>
bool sort_pairs(const K* kin, K* kout, const V* vin, V* vout, int64_t n) {
    return cub_run([&](void* t, size_t& b) {
        return cub::DeviceRadixSort::SortPairs(t, b, kin, kout, vin, vout, (int)n);
    });
}

__global__ void k_iota(int32_t* a, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        a[i] = (int32_t)i;
}

// order-preserving selection of the indices i < n with flags[i] != 0
bool select_indices(const uint8_t* flags, int64_t n, DevVec<int32_t>& out, int64_t& count) {
    DevVec<int32_t> idx;
    DevVec<int32_t> cnt;
    if (!idx.alloc(n) || !out.alloc(n) || !cnt.alloc(1)) return false;
    k_iota<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)fem::sm_count() * 64)), 256>>>(idx.p, n);
    if (!cub_run([&](void* t, size_t& b) {
            return cub::DeviceSelect::Flagged(t, b, idx.p, flags, out.p, cnt.p, (int)n);
        }))
        return false;
    int32_t h = 0;
    if (cudaMemcpy(&h, cnt.p, sizeof(int32_t), cudaMemcpyDeviceToHost) != cudaSuccess) return false;
    count = h;
    return true;
}

unsigned grid(int64_t n, int tpb = 256) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + tpb - 1) / tpb, (int64_t)fem::sm_count() * 64));
}
#define GRID_STRIDE(i, n) for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (n); \
                               i += (int64_t)gridDim.x * blockDim.x)

struct Mesh {
    const double* phi;
    const double* x;     // [nnodes][3]
    const int32_t* bc;   // [ncells][8]
    int64_t ncells, nnodes;
};

__global__ void k_classify(Mesh m, uint8_t* has, uint8_t* cut) {
    GRID_STRIDE(c, m.ncells) {
        int h0 = 0, h1 = 0;
        for (int a = 0; a < 8; ++a) {
            if (phase_of(m.phi[m.bc[c * 8 + a]])) h1 = 1;
            else h0 = 1;
        }
        has[c * 2] = (uint8_t)h0;
        has[c * 2 + 1] = (uint8_t)h1;
        cut[c] = (uint8_t)(h0 && h1);
    }
}

__device__ inline void face_nodes(const Mesh& m, int64_t c, int f, int32_t fn[4]) {
    for (int k = 0; k < 4; ++k) fn[k] = m.bc[c * 8 + c_sides[f][k]];
}
__device__ inline uint64_t face_id(const int32_t fn[4], int f) {
    int32_t mn = fn[0];
    for (int k = 1; k < 4; ++k) mn = min(mn, fn[k]);
    const int axis = (f == 1 || f == 3) ? 0 : (f == 0 || f == 2) ? 1 : 2;
    return (uint64_t)mn * 3 + axis;
}

__global__ void k_face_requests(Mesh m, const int32_t* cutc, int64_t ncut, uint64_t* key, int32_t* idx) {
    GRID_STRIDE(t, ncut * 6) {
        const int64_t j = t / 6;
        const int f = (int)(t % 6);
        int32_t fn[4];
        face_nodes(m, cutc[j], f, fn);
        key[t] = face_id(fn, f);
        idx[t] = (int32_t)t;
    }
}

__global__ void k_heads(const uint64_t* key, int64_t n, int32_t* head) {
    GRID_STRIDE(i, n) head[i] = (i == 0 || key[i] != key[i - 1]) ? 1 : 0;
}

// unique faces: key, level set, position, parents in the first cut cell's order
struct Faces {
    uint64_t* key;
    double* val;
    double* x;       // [nf][3]
    int32_t* par;    // [nf][4]
    int64_t n;
};

__global__ void k_faces(Mesh m, const int32_t* cutc, const uint64_t* skey, const int32_t* sidx, const int32_t* head,
                        const int32_t* hpos, int64_t nreq, Faces F) {
    GRID_STRIDE(i, nreq) {
        if (!head[i]) continue;
        const int64_t u = hpos[i];
        const int32_t r = sidx[i];
        if (!ok_or_record(u >= 0 && u < F.n, 1, i)) continue;
        const int64_t c = cutc[r / 6];
        const int f = r % 6;
        int32_t fn[4];
        face_nodes(m, c, f, fn);
        double v = 0.0, x[3] = {0.0, 0.0, 0.0};
        for (int k = 0; k < 4; ++k) {
            v += m.phi[fn[k]];
            for (int d = 0; d < 3; ++d) x[d] += m.x[(int64_t)fn[k] * 3 + d];
        }
        F.key[u] = skey[i];
        F.val[u] = v / 4.0;
        for (int d = 0; d < 3; ++d) F.x[u * 3 + d] = x[d] / 4.0;
        for (int k = 0; k < 4; ++k) F.par[u * 4 + k] = fn[k];
    }
}

template <typename K>
__device__ inline int64_t bsearch_key(const K* a, int64_t n, K k) {
    int64_t lo = 0, hi = n - 1;
    while (lo <= hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (a[mid] == k) return mid;
        if (a[mid] < k) lo = mid + 1;
        else hi = mid - 1;
    }
    return -1;
}

// local vertex table of a cut cell: 8 corners, 6 face centres, the centre
struct Local {
    int64_t c;
    int32_t cn[8];
    uint64_t code[15];
    double val[15];
    double xi[15][3];
};

__device__ void local_table(const Mesh& m, int64_t c, const Faces& F, Local& L) {
    L.c = c;
    double cv = 0.0;
    for (int a = 0; a < 8; ++a) {
        L.cn[a] = m.bc[c * 8 + a];
        L.code[a] = vcode(kNode, (uint64_t)L.cn[a]);
        L.val[a] = m.phi[L.cn[a]];
        cv += m.phi[L.cn[a]];
        for (int d = 0; d < 3; ++d) L.xi[a][d] = c_xi[a][d];
    }
    for (int f = 0; f < 6; ++f) {
        int32_t fn[4];
        face_nodes(m, c, f, fn);
        const uint64_t id = face_id(fn, f);
        const int64_t u = bsearch_key(F.key, F.n, id);
        ok_or_record(u >= 0, 2, (int64_t)id);
        L.code[8 + f] = vcode(kFace, id);
        L.val[8 + f] = u >= 0 ? F.val[u] : 0.0;
        for (int d = 0; d < 3; ++d) {
            double s = 0.0;
            for (int k = 0; k < 4; ++k) s += c_xi[c_sides[f][k]][d];
            L.xi[8 + f][d] = s / 4.0;
        }
    }
    L.code[14] = vcode(kCell, (uint64_t)c);
    L.val[14] = cv / 8.0;
    for (int d = 0; d < 3; ++d) L.xi[14][d] = 0.0;
}

// the 24 sub-tets (centre, face centre, two corners of the face edge) and
// their cut cases, in the host's order; Visit receives
//   whole(ph, l[4])                      an uncut tet,
//   lone(lone_ph, l[4], L, O[3])          one vertex against three,
//   pair(l[4], a, b, c2, d2)              two against two (a, b in phase 1)
template <typename Visit>
__device__ void subdivide(const Local& L, Visit& vis) {
    for (int f = 0; f < 6; ++f)
        for (int k = 0; k < 4; ++k) {
            const int l[4] = {14, 8 + f, c_sides[f][k], c_sides[f][(k + 1) % 4]};
            int ph[4], n1 = 0;
            for (int q = 0; q < 4; ++q) {
                ph[q] = phase_of(L.val[l[q]]);
                n1 += ph[q];
            }
            if (n1 == 0 || n1 == 4) {
                vis.whole(ph[0], l);
            } else if (n1 == 1 || n1 == 3) {
                const int lone_ph = n1 == 1 ? 1 : 0;
                int Lq = 0;
                while (ph[Lq] != lone_ph) ++Lq;
                int O[3], no = 0;
                for (int q = 0; q < 4; ++q)
                    if (q != Lq) O[no++] = q;
                vis.lone(lone_ph, l, Lq, O);
            } else {
                int P[2], Q[2], np = 0, nq = 0;
                for (int q = 0; q < 4; ++q) {
                    if (ph[q] == 1) P[np++] = q;
                    else Q[nq++] = q;
                }
                vis.pair(l, P[0], P[1], Q[0], Q[1]);
            }
        }
}

struct Counter {
    int ntet[2] = {0, 0}, nfac = 0, ncut = 0;
    __device__ void whole(int ph, const int*) { ntet[ph] += 1; }
    __device__ void lone(int lph, const int*, int, const int*) {
        ntet[lph] += 1;
        ntet[1 - lph] += 3;
        nfac += 1;
        ncut += 3;
    }
    __device__ void pair(const int*, int, int, int, int) {
        ntet[0] += 3;
        ntet[1] += 3;
        nfac += 2;
        ncut += 4;
    }
};

__global__ void k_count(Mesh m, const int32_t* cutc, int64_t ncut, Faces F, int64_t* nt0, int64_t* nt1,
                        int64_t* nfac, int64_t* nreq) {
    GRID_STRIDE(j, ncut) {
        Local L;
        local_table(m, cutc[j], F, L);
        Counter cnt;
        subdivide(L, cnt);
        nt0[j] = cnt.ntet[0];
        nt1[j] = cnt.ntet[1];
        nfac[j] = cnt.nfac;
        nreq[j] = 15 + cnt.ncut;
    }
}

struct Requester {
    const Local* L;
    uint64_t* key;
    int64_t pos, end;
    __device__ void cut(int la, int lb) {
        if (ok_or_record(pos < end, 3, pos)) key[pos] = edge_key(L->code[la], L->code[lb]);
        ++pos;
    }
    __device__ void whole(int, const int*) {}
    __device__ void lone(int, const int* l, int Lq, const int* O) {
        for (int k2 = 0; k2 < 3; ++k2) cut(l[Lq], l[O[k2]]);
    }
    __device__ void pair(const int* l, int a, int b, int c2, int d2) {
        cut(l[a], l[c2]);
        cut(l[a], l[d2]);
        cut(l[b], l[c2]);
        cut(l[b], l[d2]);
    }
};

__global__ void k_requests(Mesh m, const int32_t* cutc, int64_t ncut, Faces F, const int64_t* oreq, uint64_t* key,
                           int64_t* idx) {
    GRID_STRIDE(j, ncut) {
        Local L;
        local_table(m, cutc[j], F, L);
        const int64_t o = oreq[j];
        // the host's visiting order: corners, centre, faces, then the cut edges
        for (int a = 0; a < 8; ++a) key[o + a] = ekey_of_code(L.code[a]);
        key[o + 8] = ekey_of_code(L.code[14]);
        for (int f = 0; f < 6; ++f) key[o + 9 + f] = ekey_of_code(L.code[8 + f]);
        Requester rq{&L, key, o + 15, oreq[j + 1]};
        subdivide(L, rq);
        for (int64_t i = o; i < rq.pos && i < oreq[j + 1]; ++i) idx[i] = i;
    }
}

// unique entities: key (sorted) and first request; rank by first request = id
__global__ void k_entities(const uint64_t* skey, const int64_t* sidx, const int32_t* head, const int32_t* hpos,
                           int64_t n, int64_t nv_max, uint64_t* ekey, int64_t* efirst, int32_t* eu) {
    GRID_STRIDE(i, n) {
        if (!head[i]) continue;
        const int64_t u = hpos[i];
        if (!ok_or_record(u >= 0 && u < nv_max, 4, i)) continue;
        ekey[u] = skey[i];
        efirst[u] = sidx[i];
        eu[u] = (int32_t)u;
    }
}

__global__ void k_scatter_ids(const int32_t* u_of_id, int64_t n, int32_t* id_of_u) {
    GRID_STRIDE(id, n) {
        if (ok_or_record(u_of_id[id] >= 0 && u_of_id[id] < n, 5, id)) id_of_u[u_of_id[id]] = (int32_t)id;
    }
}

struct Ids {
    const uint64_t* ekey;
    const int32_t* id_of_u;
    int64_t n;
    __device__ int32_t operator()(uint64_t key) const {
        const int64_t u = bsearch_key(ekey, n, key);
        return u >= 0 ? id_of_u[u] : -1;
    }
};

struct Verts {
    int32_t* kind;
    int32_t* par;  // [nv][8]
    double* x;     // [nv][3]
    double* val;
};

__global__ void k_verts_base(Mesh m, Faces F, const uint64_t* ekey, const int32_t* u_of_id, int64_t nv, Verts V) {
    GRID_STRIDE(id, nv) {
        const uint64_t key = ekey[u_of_id[id]];
        const int kind = (int)(key >> 62);
        const uint64_t v = key & ((1ull << 62) - 1);
        if (kind == (int)kEdge) continue;
        for (int k = 0; k < 8; ++k) V.par[id * 8 + k] = -1;
        V.kind[id] = kind;
        if (kind == (int)kNode) {
            V.par[id * 8] = (int32_t)v;
            for (int d = 0; d < 3; ++d) V.x[id * 3 + d] = m.x[v * 3 + d];
            V.val[id] = m.phi[v];
        } else if (kind == (int)kFace) {
            const int64_t u = bsearch_key(F.key, F.n, v);
            if (!ok_or_record(u >= 0, 6, id)) continue;
            for (int k = 0; k < 4; ++k) V.par[id * 8 + k] = F.par[u * 4 + k];
            for (int d = 0; d < 3; ++d) V.x[id * 3 + d] = F.x[u * 3 + d];
            V.val[id] = F.val[u];
        } else {
            double s = 0.0, x[3] = {0.0, 0.0, 0.0};
            for (int a = 0; a < 8; ++a) {
                const int32_t n = m.bc[v * 8 + a];
                V.par[id * 8 + a] = n;
                s += m.phi[n];
                for (int d = 0; d < 3; ++d) x[d] += m.x[(int64_t)n * 3 + d];
            }
            V.val[id] = s / 8.0;
            for (int d = 0; d < 3; ++d) V.x[id * 3 + d] = x[d] / 8.0;
        }
    }
}

__global__ void k_verts_edges(const uint64_t* ekey, const int32_t* u_of_id, int64_t nv, Ids ids, Verts V) {
    GRID_STRIDE(id, nv) {
        const uint64_t key = ekey[u_of_id[id]];
        if ((int)(key >> 62) != (int)kEdge) continue;
        const uint64_t ca = (key >> 31) & ((1ull << 31) - 1), cb = key & ((1ull << 31) - 1);
        const int32_t ia = ids(ekey_of_code(ca)), ib = ids(ekey_of_code(cb));
        if (!ok_or_record(ia >= 0 && ib >= 0 && ia < nv && ib < nv, 7, id)) continue;
        const int32_t lo = min(ia, ib), hi = max(ia, ib);
        const double pl = V.val[lo], ph = V.val[hi];
        const double t = pl / (pl - ph);
        V.kind[id] = 3;
        for (int k = 0; k < 8; ++k) V.par[id * 8 + k] = -1;
        V.par[id * 8] = lo;
        V.par[id * 8 + 1] = hi;
        V.val[id] = t;
        for (int d = 0; d < 3; ++d) V.x[id * 3 + d] = V.x[lo * 3 + d] + t * (V.x[hi * 3 + d] - V.x[lo * 3 + d]);
    }
}

__device__ double signed_det(const double* x0, const double* x1, const double* x2, const double* x3) {
    double a[3], b[3], c[3];
    for (int d = 0; d < 3; ++d) {
        a[d] = x0[d] - x2[d];
        b[d] = x1[d] - x2[d];
        c[d] = x3[d] - x2[d];
    }
    return a[0] * (b[1] * c[2] - b[2] * c[1]) - a[1] * (b[0] * c[2] - b[2] * c[0]) + a[2] * (b[0] * c[1] - b[1] * c[0]);
}

struct Out {
    int32_t* tv[2];    // [tet][4]
    double* txi[2];    // [tet][4][3]
    double* tx[2];     // [tet][4][3]
    int32_t* fv;       // [facet][3]
    double* fxi;       // [facet][3][3]
    double* fx;        // [facet][3][3]
};

struct Emitter {
    const Local* L;
    const Ids* ids;
    const Verts* V;
    Out o;
    int64_t t[2], fc;
    int32_t lv[15];

    int64_t tend[2], fend, nv;
    bool bad = false;
    __device__ int32_t cut(int la, int lb, double* xi) {
        const int32_t va = lv[la], vb = lv[lb];
        if (!ok_or_record(va >= 0 && vb >= 0, 8, L->c)) {
            bad = true;
            for (int d = 0; d < 3; ++d) xi[d] = 0.0;
            return 0;
        }
        const int32_t lo = min(va, vb), hi = max(va, vb);
        const double pl = V->val[lo], ph = V->val[hi];
        const double tt = pl / (pl - ph);
        const int llo = lo == va ? la : lb, lhi = lo == va ? lb : la;
        for (int d = 0; d < 3; ++d) xi[d] = L->xi[llo][d] + tt * (L->xi[lhi][d] - L->xi[llo][d]);
        const int32_t id = (*ids)(edge_key(L->code[la], L->code[lb]));
        if (!ok_or_record(id >= 0 && id < nv, 9, L->c)) {
            bad = true;
            return 0;
        }
        return id;
    }
    __device__ void tet(int ph, const int32_t* v, const double (*xi)[3]) {
        if (!ok_or_record(!bad && t[ph] < tend[ph], 10, L->c)) {
            ++t[ph];
            return;
        }
        int32_t w[4] = {v[0], v[1], v[2], v[3]};
        int s0 = 0, s1 = 1;
        if (signed_det(V->x + (int64_t)w[0] * 3, V->x + (int64_t)w[1] * 3, V->x + (int64_t)w[2] * 3,
                       V->x + (int64_t)w[3] * 3) < 0.0) {
            const int32_t tmp = w[0];
            w[0] = w[1];
            w[1] = tmp;
            s0 = 1;
            s1 = 0;
        }
        const int src[4] = {s0, s1, 2, 3};
        const int64_t n = t[ph]++;
        for (int k = 0; k < 4; ++k) {
            o.tv[ph][n * 4 + k] = w[k];
            for (int d = 0; d < 3; ++d) {
                o.txi[ph][(n * 4 + k) * 3 + d] = xi[src[k]][d];
                o.tx[ph][(n * 4 + k) * 3 + d] = V->x[(int64_t)w[k] * 3 + d];
            }
        }
    }
    __device__ void wedge(int ph, const int32_t* A, const double (*xa)[3], const int32_t* B, const double (*xb)[3]) {
        const int32_t t1[4] = {A[0], A[1], A[2], B[0]}, t2[4] = {A[1], A[2], B[0], B[1]},
                      t3[4] = {A[2], B[0], B[1], B[2]};
        double x1[4][3], x2[4][3], x3[4][3];
        for (int d = 0; d < 3; ++d) {
            x1[0][d] = xa[0][d]; x1[1][d] = xa[1][d]; x1[2][d] = xa[2][d]; x1[3][d] = xb[0][d];
            x2[0][d] = xa[1][d]; x2[1][d] = xa[2][d]; x2[2][d] = xb[0][d]; x2[3][d] = xb[1][d];
            x3[0][d] = xa[2][d]; x3[1][d] = xb[0][d]; x3[2][d] = xb[1][d]; x3[3][d] = xb[2][d];
        }
        tet(ph, t1, x1);
        tet(ph, t2, x2);
        tet(ph, t3, x3);
    }
    __device__ void facet(const int32_t* v, const double (*xi)[3], const double* in0) {
        if (!ok_or_record(!bad && fc < fend, 11, L->c)) {
            ++fc;
            return;
        }
        int32_t w[3] = {v[0], v[1], v[2]};
        const double* x0 = V->x + (int64_t)w[0] * 3;
        const double* x1 = V->x + (int64_t)w[1] * 3;
        const double* x2 = V->x + (int64_t)w[2] * 3;
        double a[3], b[3], nn[3];
        for (int d = 0; d < 3; ++d) {
            a[d] = x0[d] - x2[d];
            b[d] = x1[d] - x2[d];
        }
        nn[0] = a[1] * b[2] - a[2] * b[1];
        nn[1] = a[2] * b[0] - a[0] * b[2];
        nn[2] = a[0] * b[1] - a[1] * b[0];
        double s = 0.0;
        for (int d = 0; d < 3; ++d) s += nn[d] * (in0[d] - x2[d]);
        int src[3] = {0, 1, 2};
        if (s > 0.0) {
            const int32_t tmp = w[0];
            w[0] = w[1];
            w[1] = tmp;
            src[0] = 1;
            src[1] = 0;
        }
        const int64_t n = fc++;
        for (int k = 0; k < 3; ++k) {
            o.fv[n * 3 + k] = w[k];
            for (int d = 0; d < 3; ++d) {
                o.fxi[(n * 3 + k) * 3 + d] = xi[src[k]][d];
                o.fx[(n * 3 + k) * 3 + d] = V->x[(int64_t)w[k] * 3 + d];
            }
        }
    }
    __device__ void whole(int ph, const int* l) {
        int32_t v[4];
        double xi[4][3];
        for (int q = 0; q < 4; ++q) {
            v[q] = lv[l[q]];
            for (int d = 0; d < 3; ++d) xi[q][d] = L->xi[l[q]][d];
        }
        tet(ph, v, xi);
    }
    __device__ void lone(int lone_ph, const int* l, int Lq, const int* O) {
        int32_t v[4];
        double xi[4][3];
        for (int q = 0; q < 4; ++q) {
            v[q] = lv[l[q]];
            for (int d = 0; d < 3; ++d) xi[q][d] = L->xi[l[q]][d];
        }
        int32_t I[3];
        double xI[3][3];
        for (int k2 = 0; k2 < 3; ++k2) I[k2] = cut(l[Lq], l[O[k2]], xI[k2]);
        const int32_t tv[4] = {v[Lq], I[0], I[1], I[2]};
        double tx[4][3];
        for (int d = 0; d < 3; ++d) {
            tx[0][d] = xi[Lq][d];
            for (int k2 = 0; k2 < 3; ++k2) tx[1 + k2][d] = xI[k2][d];
        }
        tet(lone_ph, tv, tx);
        const int32_t A[3] = {v[O[0]], v[O[1]], v[O[2]]};
        double xa[3][3];
        for (int k2 = 0; k2 < 3; ++k2)
            for (int d = 0; d < 3; ++d) xa[k2][d] = xi[O[k2]][d];
        wedge(1 - lone_ph, A, xa, I, xI);
        const double* in0 = lone_ph == 0 ? V->x + (int64_t)v[Lq] * 3 : V->x + (int64_t)v[O[0]] * 3;
        facet(I, xI, in0);
    }
    __device__ void pair(const int* l, int a, int b, int c2, int d2) {
        int32_t v[4];
        double xi[4][3];
        for (int q = 0; q < 4; ++q) {
            v[q] = lv[l[q]];
            for (int d = 0; d < 3; ++d) xi[q][d] = L->xi[l[q]][d];
        }
        double xac[3], xad[3], xbc[3], xbd[3];
        const int32_t Iac = cut(l[a], l[c2], xac), Iad = cut(l[a], l[d2], xad);
        const int32_t Ibc = cut(l[b], l[c2], xbc), Ibd = cut(l[b], l[d2], xbd);
        {
            const int32_t A[3] = {v[a], Iac, Iad}, B[3] = {v[b], Ibc, Ibd};
            double xa[3][3], xb[3][3];
            for (int d = 0; d < 3; ++d) {
                xa[0][d] = xi[a][d]; xa[1][d] = xac[d]; xa[2][d] = xad[d];
                xb[0][d] = xi[b][d]; xb[1][d] = xbc[d]; xb[2][d] = xbd[d];
            }
            wedge(1, A, xa, B, xb);
        }
        {
            const int32_t A[3] = {v[c2], Iac, Ibc}, B[3] = {v[d2], Iad, Ibd};
            double xa[3][3], xb[3][3];
            for (int d = 0; d < 3; ++d) {
                xa[0][d] = xi[c2][d]; xa[1][d] = xac[d]; xa[2][d] = xbc[d];
                xb[0][d] = xi[d2][d]; xb[1][d] = xad[d]; xb[2][d] = xbd[d];
            }
            wedge(0, A, xa, B, xb);
        }
        const double* in0 = V->x + (int64_t)v[c2] * 3;
        const int32_t f1[3] = {Iac, Iad, Ibd}, f2[3] = {Iac, Ibd, Ibc};
        double x1[3][3], x2[3][3];
        for (int d = 0; d < 3; ++d) {
            x1[0][d] = xac[d]; x1[1][d] = xad[d]; x1[2][d] = xbd[d];
            x2[0][d] = xac[d]; x2[1][d] = xbd[d]; x2[2][d] = xbc[d];
        }
        facet(f1, x1, in0);
        facet(f2, x2, in0);
    }
};

__global__ void k_emit(Mesh m, const int32_t* cutc, int64_t ncut, Faces F, Ids ids, Verts V, Out o,
                       const int64_t* ot0, const int64_t* ot1, const int64_t* ofac) {
    GRID_STRIDE(j, ncut) {
        Local L;
        local_table(m, cutc[j], F, L);
        Emitter em{&L, &ids, &V, o, {ot0[j], ot1[j]}, ofac[j], {}, {ot0[j + 1], ot1[j + 1]}, ofac[j + 1], ids.n};
        for (int q = 0; q < 15; ++q) {
            em.lv[q] = ids(ekey_of_code(L.code[q]));
            if (!ok_or_record(em.lv[q] >= 0, 12, L.c)) em.bad = true;
        }
        if (!em.bad) subdivide(L, em);
    }
}

// enrichment: components of every basis support per phase (the host's flood fill)
struct Enrich {
    int64_t ne[3], nb0, nb1, nbases;
    int p;
    const uint8_t* has;
    int32_t* comp;    // [(cell*2 + phase)*nloc + l]
    int64_t* ncomp;   // [nbases]
};

__global__ void k_enrich(Enrich E) {
    const int pp = E.p + 1, nloc = pp * pp * pp;
    GRID_STRIDE(b, E.nbases) {
        const int64_t bi = b % E.nb0, bj = (b / E.nb0) % E.nb1, bk = b / (E.nb0 * E.nb1);
        int64_t sc[64];
        int nsc = 0;
        for (int l2 = 0; l2 < pp; ++l2)
            for (int l1 = 0; l1 < pp; ++l1)
                for (int l0 = 0; l0 < pp; ++l0) {
                    const int64_t ci = bi - l0, cj = bj - l1, ck = bk - l2;
                    if (ci < 0 || cj < 0 || ck < 0 || ci >= E.ne[0] || cj >= E.ne[1] || ck >= E.ne[2]) continue;
                    sc[nsc++] = ci + E.ne[0] * (cj + E.ne[1] * ck);
                }
        for (int i = 1; i < nsc; ++i)  // ascending cell order (insertion sort)
            for (int k = i; k > 0 && sc[k - 1] > sc[k]; --k) {
                const int64_t t = sc[k];
                sc[k] = sc[k - 1];
                sc[k - 1] = t;
            }
        int next = 0;
        for (int ph = 0; ph < 2; ++ph) {
            int lab[64];
            for (int k = 0; k < nsc; ++k) lab[k] = -1;
            for (int k0 = 0; k0 < nsc; ++k0) {
                if (!E.has[sc[k0] * 2 + ph] || lab[k0] >= 0) continue;
                int stack[64], top = 0;
                stack[top++] = k0;
                lab[k0] = next;
                while (top) {
                    const int k = stack[--top];
                    const int64_t c = sc[k];
                    const int64_t ci = c % E.ne[0], cj = (c / E.ne[0]) % E.ne[1], ck = c / (E.ne[0] * E.ne[1]);
                    for (int q = 0; q < nsc; ++q) {
                        if (lab[q] >= 0 || !E.has[sc[q] * 2 + ph]) continue;
                        const int64_t c2 = sc[q];
                        const int64_t qi = c2 % E.ne[0], qj = (c2 / E.ne[0]) % E.ne[1], qk = c2 / (E.ne[0] * E.ne[1]);
                        const int64_t dist = llabs(qi - ci) + llabs(qj - cj) + llabs(qk - ck);
                        if (dist != 1) continue;
                        lab[q] = next;
                        stack[top++] = q;
                    }
                }
                ++next;
            }
            for (int k = 0; k < nsc; ++k) {
                if (lab[k] < 0) continue;
                const int64_t c = sc[k];
                const int64_t ci = c % E.ne[0], cj = (c / E.ne[0]) % E.ne[1], ck = c / (E.ne[0] * E.ne[1]);
                const int l = (int)((bi - ci) + pp * ((bj - cj) + pp * (bk - ck)));
                E.comp[(c * 2 + ph) * nloc + l] = lab[k];
            }
        }
        E.ncomp[b] = next;
    }
}

__global__ void k_ecell_flags(const uint8_t* has, int64_t n, int64_t* f) { GRID_STRIDE(i, n) f[i] = has[i]; }

__global__ void k_ecells(const uint8_t* has, const int64_t* eoff, int64_t n, int32_t* cell_bg, int32_t* cell_ph,
                         int64_t* ecell_of) {
    GRID_STRIDE(i, n) {
        ecell_of[i] = has[i] ? eoff[i] : -1;
        if (has[i]) {
            cell_bg[eoff[i]] = (int32_t)(i / 2);
            cell_ph[eoff[i]] = (int32_t)(i % 2);
        }
    }
}

// unzipping: the enriched row of (enriched cell e, corner a)
struct Unzip {
    int64_t ne[3], nb0, nb1;
    int p;
    const int32_t* bc;
    const int64_t* boff;
    const int32_t* bb;
    const int32_t* cell_bg;
    const int32_t* cell_ph;
    const int32_t* comp;
    const int64_t* eoff;
    int* err;
    int64_t nec, ncells, nnodes, nbases;
};

__device__ inline int32_t unzip_entry(const Unzip& U, int64_t c, int ph, int64_t k) {
    const int pp = U.p + 1, nloc = pp * pp * pp;
    const int64_t ci = c % U.ne[0], cj = (c / U.ne[0]) % U.ne[1], ck = c / (U.ne[0] * U.ne[1]);
    const int64_t b = U.bb[k];
    if (!ok_or_record(b >= 0 && b < U.nbases, 20, k)) return -1;
    const int64_t bi = b % U.nb0, bj = (b / U.nb0) % U.nb1, bk = b / (U.nb0 * U.nb1);
    const int l = (int)((bi - ci) + pp * ((bj - cj) + pp * (bk - ck)));
    if (!ok_or_record(l >= 0 && l < nloc && c >= 0 && c < U.ncells && (ph == 0 || ph == 1), 21, c)) return -1;
    const int32_t cp = U.comp[(c * 2 + ph) * nloc + l];
    if (cp < 0) {
        atomicOr(U.err, 1);
        return -1;
    }
    return (int32_t)(U.eoff[b] + cp);
}

__global__ void k_unzip_keys(Unzip U, int64_t nitems, uint64_t* key, int64_t* idx) {
    GRID_STRIDE(it, nitems) {
        const int64_t e = it / 8;
        const int a = (int)(it % 8);
        const int64_t c = U.cell_bg[e];
        const int ph = U.cell_ph[e];
        key[it] = 0;
        idx[it] = it;
        if (!ok_or_record(e < U.nec && c >= 0 && c < U.ncells, 22, it)) continue;
        const int32_t n = U.bc[c * 8 + a];
        if (!ok_or_record(n >= 0 && n < U.nnodes, 23, it)) continue;
        uint64_t h = 1469598103934665603ull ^ (uint64_t)n;  // FNV-1a over (node, row)
        h *= 1099511628211ull;
        for (int64_t k = U.boff[n]; k < U.boff[n + 1]; ++k) {
            h ^= (uint64_t)(uint32_t)unzip_entry(U, c, ph, k);
            h *= 1099511628211ull;
        }
        key[it] = h;
        idx[it] = it;
    }
}

// equal hashes must be equal (node, row): checked against the group head
__global__ void k_unzip_check(Unzip U, const uint64_t* skey, const int64_t* sidx, int64_t n, const int32_t* head,
                              const int32_t* hpos, int64_t* gfirst) {
    GRID_STRIDE(i, n) {
        if (head[i]) gfirst[hpos[i]] = sidx[i];
    }
}
// group of sorted item i: the exclusive scan of the head flags counts the heads
// before i, so a head sits at its group's index and the others one past it
__device__ inline int64_t group_of(const int32_t* head, const int32_t* hpos, int64_t i) { return hpos[i] + head[i] - 1; }

__global__ void k_unzip_verify(Unzip U, const int64_t* sidx, int64_t n, const int32_t* head, const int32_t* hpos,
                               const int64_t* gfirst) {
    GRID_STRIDE(i, n) {
        const int64_t it = sidx[i], h = gfirst[group_of(head, hpos, i)];
        if (it == h) continue;
        if (!ok_or_record(it >= 0 && it < n && h >= 0 && h < n, 24, i)) continue;
        const int64_t e1 = it / 8, e2 = h / 8;
        const int32_t n1 = U.bc[(int64_t)U.cell_bg[e1] * 8 + it % 8], n2 = U.bc[(int64_t)U.cell_bg[e2] * 8 + h % 8];
        bool same = n1 == n2;
        for (int64_t k = U.boff[n1]; same && k < U.boff[n1 + 1]; ++k)
            same = unzip_entry(U, U.cell_bg[e1], U.cell_ph[e1], k) == unzip_entry(U, U.cell_bg[e2], U.cell_ph[e2], k);
        if (!same) atomicOr(U.err, 2);
    }
}

__global__ void k_unzip_ids(const int64_t* sidx, int64_t n, const int32_t* head, const int32_t* hpos,
                            const int32_t* gid_of_group, int32_t* cells) {
    GRID_STRIDE(i, n) {
        if (ok_or_record(sidx[i] >= 0 && sidx[i] < n, 13, i)) cells[sidx[i]] = gid_of_group[group_of(head, hpos, i)];
    }
}

__global__ void k_unzip_len(Unzip U, const int64_t* first_of_vid, int64_t nv, int64_t* len) {
    GRID_STRIDE(v, nv) {
        const int64_t it = first_of_vid[v];
        len[v] = 0;
        if (!ok_or_record(it >= 0 && it < U.nec * 8, 25, v)) continue;
        const int32_t n = U.bc[(int64_t)U.cell_bg[it / 8] * 8 + it % 8];
        len[v] = U.boff[n + 1] - U.boff[n];
    }
}

__global__ void k_unzip_rows(Unzip U, const double* bw, const double* bx, const int64_t* first_of_vid, int64_t nv,
                             const int64_t* toff, double* coords, int32_t* tb, double* tw) {
    GRID_STRIDE(v, nv) {
        const int64_t it = first_of_vid[v];
        const int64_t e = it / 8;
        const int64_t c = U.cell_bg[e];
        const int32_t n = U.bc[c * 8 + it % 8];
        for (int d = 0; d < 3; ++d) coords[v * 3 + d] = bx[(int64_t)n * 3 + d];
        int64_t o = toff[v];
        for (int64_t k = U.boff[n]; k < U.boff[n + 1]; ++k, ++o) {
            tb[o] = unzip_entry(U, c, U.cell_ph[e], k);
            tw[o] = bw[k];
        }
    }
}

// ghost facet candidates in the host's order (phase, cell, axis)
__global__ void k_ghost_flags(const uint8_t* has, const uint8_t* cut, int64_t ne0, int64_t ne1, int64_t ne2,
                              uint8_t* flag) {
    const int64_t ncells = ne0 * ne1 * ne2;
    GRID_STRIDE(t, 2 * ncells * 3) {
        const int ph = (int)(t / (ncells * 3));
        const int64_t c = (t / 3) % ncells;
        const int ax = (int)(t % 3);
        const int64_t ijk[3] = {c % ne0, (c / ne0) % ne1, c / (ne0 * ne1)};
        const int64_t nax = ax == 0 ? ne0 : ax == 1 ? ne1 : ne2;
        bool ok = has[c * 2 + ph] && ijk[ax] + 1 < nax;
        if (ok) {
            const int64_t c2 = c + (ax == 0 ? 1 : ax == 1 ? ne0 : ne0 * ne1);
            ok = has[c2 * 2 + ph] && (cut[c] || cut[c2]);
        }
        flag[t] = ok ? 1 : 0;
    }
}

__global__ void k_ghosts(const int32_t* sel, int64_t nsel, int64_t ncells, int64_t ne0, int64_t ne1, Mesh m,
                         const int64_t* ecell_of, int32_t* leader, int32_t* follower, double* gx, double* gxl,
                         double* gxf) {
    GRID_STRIDE(g, nsel) {
        const int64_t t = sel[g];
        const int ph = (int)(t / (ncells * 3));
        const int64_t c = (t / 3) % ncells;
        const int ax = (int)(t % 3);
        const int64_t c2 = c + (ax == 0 ? 1 : ax == 1 ? ne0 : ne0 * ne1);
        leader[g] = (int32_t)ecell_of[c * 2 + ph];
        follower[g] = (int32_t)ecell_of[c2 * 2 + ph];
        const int side_of_axis[3] = {1, 2, 5};
        const int s = side_of_axis[ax];
        for (int k = 0; k < 4; ++k) {
            const int a = c_sides[s][k];
            const int32_t n = m.bc[c * 8 + a];
            for (int d = 0; d < 3; ++d) {
                gx[(g * 4 + k) * 3 + d] = m.x[(int64_t)n * 3 + d];
                gxl[(g * 4 + k) * 3 + d] = c_xi[a][d];
                gxf[(g * 4 + k) * 3 + d] = d == ax ? -1.0 : c_xi[a][d];
            }
        }
    }
}

__global__ void k_gather_i32(const int32_t* idx, int64_t n, const int64_t* src, int stride, int off, int32_t* out) {
    GRID_STRIDE(i, n) out[i] = (int32_t)src[(int64_t)idx[i] * stride + off];
}

}  // namespace

using namespace fem;

extern "C" {

fem_gpu_status fem_xtk_decompose_device(const int32_t* num_elements, const double* lengths, int32_t p,
                                        const double* node_phi, fem_xtk_model** out) {
    if (!num_elements || !lengths || !node_phi || !out || p < 1 || p > 3) return FEM_GPU_BAD_ARG;
    *out = nullptr;
    for (int d = 0; d < 3; ++d)
        if (num_elements[d] < 1 || !(lengths[d] > 0.0)) return FEM_GPU_BAD_ARG;
    // background mesh and its extraction rows (host generator, as the host path)
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
    if (3 * nnodes >= (1ll << kIdBits) || ncells >= (1ll << kIdBits)) return FEM_GPU_UNSUPPORTED;
    cudaMemcpyToSymbol(c_sides, kHexSides, sizeof(kHexSides));
    cudaMemcpyToSymbol(c_xi, kHexXi, sizeof(kHexXi));

    auto m = new fem_xtk_model;
    auto fail_out = [&](fem_gpu_status s) {
        delete m;
        return s;
    };
    const unsigned long long zero2[2] = {0ull, 0ull};
    cudaMemcpyToSymbol(g_fault, zero2, sizeof(zero2));
    const char* stage = "setup";
    // a failed CUDA call or device self-check names its stage on stderr
    auto report = [&](fem_gpu_status s) {
        unsigned long long f[2] = {0ull, 0ull};
        cudaMemcpyFromSymbol(f, g_fault, sizeof(f));
        fprintf(stderr, "fem_xtk_decompose_device: stage %s: %s (check %llu at %llu)\n", stage,
                cudaGetErrorString(cudaGetLastError()), f[0], f[1]);
        return fail_out(s);
    };
#define CK(x) \
    if (!(x)) return report(FEM_GPU_CUDA_ERROR)
#define STAGE(name)                                                                                        \
    do {                                                                                                   \
        if (cudaDeviceSynchronize() != cudaSuccess || cudaGetLastError() != cudaSuccess) return report(FEM_GPU_CUDA_ERROR); \
        unsigned long long f0 = 0ull;                                                                      \
        cudaMemcpyFromSymbol(&f0, g_fault, sizeof(f0));                                                    \
        if (f0) return report(FEM_GPU_UNSUPPORTED);                                                        \
        stage = name;                                                                                      \
    } while (0)
    m->p = p;
    for (int d = 0; d < 3; ++d) {
        m->ne[d] = num_elements[d];
        m->nn[d] = num_elements[d] + 1;
        m->nbk[d] = num_elements[d] + p;
    }
    const int64_t* ne = m->ne;
    DevVec<double> dphi, dx, dbw;
    DevVec<int32_t> dbc, dbb;
    DevVec<int64_t> dboff;
    CK(dphi.upload(node_phi, nnodes) && dx.upload(bx.data(), bx.size()) && dbc.upload(bc.data(), bc.size()) &&
       dboff.upload(boff.data(), boff.size()) && dbb.upload(bb.data(), bb.size()) && dbw.upload(bw.data(), bw.size()));
    Mesh M{dphi.p, dx.p, dbc.p, ncells, nnodes};

    // 1. cells
    DevVec<uint8_t> has, cut;
    CK(has.alloc(ncells * 2) && cut.alloc(ncells));
    k_classify<<<grid(ncells), 256>>>(M, has.p, cut.p);
    DevVec<int32_t> cutc;
    int64_t ncut = 0;
    CK(select_indices(cut.p, ncells, cutc, ncut));

    STAGE("faces");
    // 2. face centres
    Faces F{};
    DevVec<uint64_t> fkey, fkey_s, ukey;
    DevVec<int32_t> fidx, fidx_s, fhead, fpos;
    DevVec<double> fval, fxv;
    DevVec<int32_t> fpar;
    const int64_t nfr = ncut * 6;
    CK(fkey.alloc(nfr) && fkey_s.alloc(nfr) && fidx.alloc(nfr) && fidx_s.alloc(nfr) && fhead.alloc(nfr) &&
       fpos.alloc(nfr));
    if (ncut) {
        k_face_requests<<<grid(nfr), 256>>>(M, cutc.p, ncut, fkey.p, fidx.p);
        CK(sort_pairs(fkey.p, fkey_s.p, fidx.p, fidx_s.p, nfr));
        k_heads<<<grid(nfr), 256>>>(fkey_s.p, nfr, fhead.p);
        CK(exclusive_scan(fhead.p, fpos.p, nfr));
    }
    int32_t last_h = 0, last_p = 0;
    if (nfr) {
        CK(cudaMemcpy(&last_h, fhead.p + nfr - 1, 4, cudaMemcpyDeviceToHost) == cudaSuccess);
        CK(cudaMemcpy(&last_p, fpos.p + nfr - 1, 4, cudaMemcpyDeviceToHost) == cudaSuccess);
    }
    F.n = nfr ? last_p + last_h : 0;
    CK(ukey.alloc(F.n) && fval.alloc(F.n) && fxv.alloc(F.n * 3) && fpar.alloc(F.n * 4));
    F.key = ukey.p;
    F.val = fval.p;
    F.x = fxv.p;
    F.par = fpar.p;
    if (nfr) k_faces<<<grid(nfr), 256>>>(M, cutc.p, fkey_s.p, fidx_s.p, fhead.p, fpos.p, nfr, F);

    STAGE("counts");
    // 3. counts and requests per cut cell
    DevVec<int64_t> nt0, nt1, nfc, nrq, ot0, ot1, ofc, orq;
    CK(nt0.alloc(ncut + 1) && nt1.alloc(ncut + 1) && nfc.alloc(ncut + 1) && nrq.alloc(ncut + 1) &&
       ot0.alloc(ncut + 1) && ot1.alloc(ncut + 1) && ofc.alloc(ncut + 1) && orq.alloc(ncut + 1));
    cudaMemset(nt0.p, 0, (ncut + 1) * 8);
    cudaMemset(nt1.p, 0, (ncut + 1) * 8);
    cudaMemset(nfc.p, 0, (ncut + 1) * 8);
    cudaMemset(nrq.p, 0, (ncut + 1) * 8);
    if (ncut) k_count<<<grid(ncut, 128), 128>>>(M, cutc.p, ncut, F, nt0.p, nt1.p, nfc.p, nrq.p);
    CK(exclusive_scan(nt0.p, ot0.p, ncut + 1) && exclusive_scan(nt1.p, ot1.p, ncut + 1) &&
       exclusive_scan(nfc.p, ofc.p, ncut + 1) && exclusive_scan(nrq.p, orq.p, ncut + 1));
    int64_t tot[4];
    CK(cudaMemcpy(&tot[0], ot0.p + ncut, 8, cudaMemcpyDeviceToHost) == cudaSuccess);
    CK(cudaMemcpy(&tot[1], ot1.p + ncut, 8, cudaMemcpyDeviceToHost) == cudaSuccess);
    CK(cudaMemcpy(&tot[2], ofc.p + ncut, 8, cudaMemcpyDeviceToHost) == cudaSuccess);
    CK(cudaMemcpy(&tot[3], orq.p + ncut, 8, cudaMemcpyDeviceToHost) == cudaSuccess);
    const int64_t nreq = tot[3];
    DevVec<uint64_t> rkey, rkey_s, ekey;
    DevVec<int64_t> ridx, ridx_s, efirst, efirst_s;
    DevVec<int32_t> rhead, rpos, eu, u_of_id, id_of_u;
    CK(rkey.alloc(nreq) && rkey_s.alloc(nreq) && ridx.alloc(nreq) && ridx_s.alloc(nreq) && rhead.alloc(nreq) &&
       rpos.alloc(nreq));
    if (ncut) k_requests<<<grid(ncut, 128), 128>>>(M, cutc.p, ncut, F, orq.p, rkey.p, ridx.p);

    STAGE("ids");
    // 4. ids by first touch
    int64_t nv = 0;
    if (nreq) {
        CK(sort_pairs(rkey.p, rkey_s.p, ridx.p, ridx_s.p, nreq));
        k_heads<<<grid(nreq), 256>>>(rkey_s.p, nreq, rhead.p);
        CK(exclusive_scan(rhead.p, rpos.p, nreq));
        CK(cudaMemcpy(&last_h, rhead.p + nreq - 1, 4, cudaMemcpyDeviceToHost) == cudaSuccess);
        CK(cudaMemcpy(&last_p, rpos.p + nreq - 1, 4, cudaMemcpyDeviceToHost) == cudaSuccess);
        nv = last_p + last_h;
    }
    CK(ekey.alloc(nv) && efirst.alloc(nv) && efirst_s.alloc(nv) && eu.alloc(nv) && u_of_id.alloc(nv) &&
       id_of_u.alloc(nv));
    if (nreq) {
        k_entities<<<grid(nreq), 256>>>(rkey_s.p, ridx_s.p, rhead.p, rpos.p, nreq, nv, ekey.p, efirst.p, eu.p);
        CK(sort_pairs(efirst.p, efirst_s.p, eu.p, u_of_id.p, nv));
        k_scatter_ids<<<grid(nv), 256>>>(u_of_id.p, nv, id_of_u.p);
    }
    const Ids ids{ekey.p, id_of_u.p, nv};

    STAGE("vertices");
    // 5. vertex table
    DevVec<int32_t> vkind, vpar;
    DevVec<double> vx, vval;
    CK(vkind.alloc(nv) && vpar.alloc(nv * 8) && vx.alloc(nv * 3) && vval.alloc(nv));
    const Verts V{vkind.p, vpar.p, vx.p, vval.p};
    if (nv) {
        k_verts_base<<<grid(nv), 256>>>(M, F, ekey.p, u_of_id.p, nv, V);
        k_verts_edges<<<grid(nv), 256>>>(ekey.p, u_of_id.p, nv, ids, V);
    }

    STAGE("emit");
    // 6. tets and facets
    DevVec<int32_t> tv0, tv1, fv;
    DevVec<double> txi0, txi1, tx0, tx1, fxi, fx;
    CK(tv0.alloc(tot[0] * 4) && tv1.alloc(tot[1] * 4) && fv.alloc(tot[2] * 3) && txi0.alloc(tot[0] * 12) &&
       txi1.alloc(tot[1] * 12) && tx0.alloc(tot[0] * 12) && tx1.alloc(tot[1] * 12) && fxi.alloc(tot[2] * 9) &&
       fx.alloc(tot[2] * 9));
    Out o{{tv0.p, tv1.p}, {txi0.p, txi1.p}, {tx0.p, tx1.p}, fv.p, fxi.p, fx.p};
    if (ncut) k_emit<<<grid(ncut, 64), 64>>>(M, cutc.p, ncut, F, ids, V, o, ot0.p, ot1.p, ofc.p);

    STAGE("enrichment");
    // 7. enrichment
    const int pp = p + 1, nloc = pp * pp * pp;
    DevVec<int32_t> comp;
    DevVec<int64_t> ncomp, eoffb;
    CK(comp.alloc((size_t)ncells * 2 * nloc) && ncomp.alloc(nbases + 1) && eoffb.alloc(nbases + 1));
    cudaMemset(comp.p, 0xff, (size_t)ncells * 2 * nloc * sizeof(int32_t));
    cudaMemset(ncomp.p, 0, (nbases + 1) * 8);
    Enrich E{{ne[0], ne[1], ne[2]}, m->nbk[0], m->nbk[1], nbases, p, has.p, comp.p, ncomp.p};
    k_enrich<<<grid(nbases, 64), 64>>>(E);
    CK(exclusive_scan(ncomp.p, eoffb.p, nbases + 1));
    CK(cudaMemcpy(&m->num_enriched_bases, eoffb.p + nbases, 8, cudaMemcpyDeviceToHost) == cudaSuccess);

    STAGE("enriched cells");
    // enriched cells
    DevVec<int64_t> ef, eoffc, ecell_of;
    CK(ef.alloc(ncells * 2 + 1) && eoffc.alloc(ncells * 2 + 1) && ecell_of.alloc(ncells * 2));
    cudaMemset(ef.p, 0, (ncells * 2 + 1) * 8);
    k_ecell_flags<<<grid(ncells * 2), 256>>>(has.p, ncells * 2, ef.p);
    CK(exclusive_scan(ef.p, eoffc.p, ncells * 2 + 1));
    int64_t nec = 0;
    CK(cudaMemcpy(&nec, eoffc.p + ncells * 2, 8, cudaMemcpyDeviceToHost) == cudaSuccess);
    DevVec<int32_t> cell_bg, cell_ph;
    CK(cell_bg.alloc(nec) && cell_ph.alloc(nec));
    k_ecells<<<grid(ncells * 2), 256>>>(has.p, eoffc.p, ncells * 2, cell_bg.p, cell_ph.p, ecell_of.p);

    STAGE("unzip");
    // 8. unzipped vertices
    DevVec<int> derr;
    CK(derr.alloc(1));
    cudaMemset(derr.p, 0, sizeof(int));
    Unzip U{{ne[0], ne[1], ne[2]}, m->nbk[0], m->nbk[1], p, dbc.p, dboff.p, dbb.p, cell_bg.p, cell_ph.p, comp.p,
            eoffb.p, derr.p, nec, ncells, nnodes, nbases};
    const int64_t nit = nec * 8;
    DevVec<uint64_t> zkey, zkey_s;
    DevVec<int64_t> zidx, zidx_s, gfirst, gfirst_s, first_of_vid, zlen, ztoff;
    DevVec<int32_t> zhead, zpos, gidx, grp_of_vid, vid_of_grp, dcells;
    CK(zkey.alloc(nit) && zkey_s.alloc(nit) && zidx.alloc(nit) && zidx_s.alloc(nit) && zhead.alloc(nit) &&
       zpos.alloc(nit) && dcells.alloc(nit));
    int64_t nuv = 0;
    if (nit) {
        k_unzip_keys<<<grid(nit), 256>>>(U, nit, zkey.p, zidx.p);
        STAGE("unzip keys");
        CK(sort_pairs(zkey.p, zkey_s.p, zidx.p, zidx_s.p, nit));
        STAGE("unzip sort");
        k_heads<<<grid(nit), 256>>>(zkey_s.p, nit, zhead.p);
        CK(exclusive_scan(zhead.p, zpos.p, nit));
        CK(cudaMemcpy(&last_h, zhead.p + nit - 1, 4, cudaMemcpyDeviceToHost) == cudaSuccess);
        CK(cudaMemcpy(&last_p, zpos.p + nit - 1, 4, cudaMemcpyDeviceToHost) == cudaSuccess);
        nuv = last_p + last_h;
    }
    CK(gfirst.alloc(nuv) && gfirst_s.alloc(nuv) && gidx.alloc(nuv) && grp_of_vid.alloc(nuv) &&
       vid_of_grp.alloc(nuv) && first_of_vid.alloc(nuv) && zlen.alloc(nuv + 1) && ztoff.alloc(nuv + 1));
    if (nit) {
        k_unzip_check<<<grid(nit), 256>>>(U, zkey_s.p, zidx_s.p, nit, zhead.p, zpos.p, gfirst.p);
        k_unzip_verify<<<grid(nit), 256>>>(U, zidx_s.p, nit, zhead.p, zpos.p, gfirst.p);
        // groups in first-touch order -> vertex ids
        k_iota<<<grid(nuv), 256>>>(gidx.p, nuv);
        CK(sort_pairs(gfirst.p, gfirst_s.p, gidx.p, grp_of_vid.p, nuv));
        CK(cudaMemcpy(first_of_vid.p, gfirst_s.p, nuv * 8, cudaMemcpyDeviceToDevice) == cudaSuccess);
        k_scatter_ids<<<grid(nuv), 256>>>(grp_of_vid.p, nuv, vid_of_grp.p);
        k_unzip_ids<<<grid(nit), 256>>>(zidx_s.p, nit, zhead.p, zpos.p, vid_of_grp.p, dcells.p);
        cudaMemset(zlen.p, 0, (nuv + 1) * 8);
        k_unzip_len<<<grid(nuv), 256>>>(U, first_of_vid.p, nuv, zlen.p);
        CK(exclusive_scan(zlen.p, ztoff.p, nuv + 1));
    }
    STAGE("unzip groups");
    int herr = 0;
    CK(cudaMemcpy(&herr, derr.p, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess);
    if (herr) {  // a corner row without its phase, or a hash collision
        fprintf(stderr, "fem_xtk_decompose_device: unzip error %d\n", herr);
        return fail_out(FEM_GPU_UNSUPPORTED);
    }
    int64_t ntb = 0;
    if (nuv) CK(cudaMemcpy(&ntb, ztoff.p + nuv, 8, cudaMemcpyDeviceToHost) == cudaSuccess);
    DevVec<double> zcoords, ztw;
    DevVec<int32_t> ztb;
    CK(zcoords.alloc(nuv * 3) && ztb.alloc(ntb) && ztw.alloc(ntb));
    if (nuv) k_unzip_rows<<<grid(nuv), 256>>>(U, dbw.p, dx.p, first_of_vid.p, nuv, ztoff.p, zcoords.p, ztb.p, ztw.p);

    STAGE("clusters");
    // 9. clusters and ghost facets
    DevVec<uint8_t> uflag;
    CK(uflag.alloc(ncells));
    for (int ph = 0; ph < 2; ++ph) {
        std::vector<uint8_t> hh(ncells * 2), hc(ncells), fl(ncells);
        CK(cudaMemcpy(hh.data(), has.p, ncells * 2, cudaMemcpyDeviceToHost) == cudaSuccess);
        CK(cudaMemcpy(hc.data(), cut.p, ncells, cudaMemcpyDeviceToHost) == cudaSuccess);
        for (int64_t c = 0; c < ncells; ++c) fl[c] = (!hc[c] && hh[c * 2 + ph]) ? 1 : 0;
        CK(cudaMemcpy(uflag.p, fl.data(), ncells, cudaMemcpyHostToDevice) == cudaSuccess);
        DevVec<int32_t> sel, outc;
        int64_t ns = 0;
        CK(select_indices(uflag.p, ncells, sel, ns));
        CK(outc.alloc(ns));
        if (ns) k_gather_i32<<<grid(ns), 256>>>(sel.p, ns, ecell_of.p, 2, ph, outc.p);
        CK(outc.download(m->uncut[ph], ns));
        DevVec<int32_t> cutl;
        CK(cutl.alloc(ncut));
        if (ncut) k_gather_i32<<<grid(ncut), 256>>>(cutc.p, ncut, ecell_of.p, 2, ph, cutl.p);
        CK(cutl.download(m->cut[ph], ncut));
    }
    m->if_leader = m->cut[0];
    m->if_follower = m->cut[1];
    DevVec<uint8_t> gflag;
    CK(gflag.alloc(2 * ncells * 3));
    k_ghost_flags<<<grid(2 * ncells * 3), 256>>>(has.p, cut.p, ne[0], ne[1], ne[2], gflag.p);
    DevVec<int32_t> gsel;
    int64_t ngs = 0;
    CK(select_indices(gflag.p, 2 * ncells * 3, gsel, ngs));
    DevVec<int32_t> gl, gf;
    DevVec<double> gxx, gxl, gxf;
    CK(gl.alloc(ngs) && gf.alloc(ngs) && gxx.alloc(ngs * 12) && gxl.alloc(ngs * 12) && gxf.alloc(ngs * 12));
    if (ngs) k_ghosts<<<grid(ngs), 256>>>(gsel.p, ngs, ncells, ne[0], ne[1], M, ecell_of.p, gl.p, gf.p, gxx.p, gxl.p,
                                          gxf.p);
    STAGE("results");

    // results to the host model
    std::vector<int32_t> gsel_h, gl_h, gf_h;
    std::vector<double> gxx_h, gxl_h, gxf_h;
    CK(gsel.download(gsel_h, ngs) && gl.download(gl_h, ngs) && gf.download(gf_h, ngs) &&
       gxx.download(gxx_h, ngs * 12) && gxl.download(gxl_h, ngs * 12) && gxf.download(gxf_h, ngs * 12));
    for (int64_t g = 0; g < ngs; ++g) {
        const int ph = (int)(gsel_h[g] / (ncells * 3));
        m->gh_leader[ph].push_back(gl_h[g]);
        m->gh_follower[ph].push_back(gf_h[g]);
        for (int k = 0; k < 12; ++k) {
            m->gh_x[ph].push_back(gxx_h[g * 12 + k]);
            m->gh_xi_l[ph].push_back(gxl_h[g * 12 + k]);
            m->gh_xi_f[ph].push_back(gxf_h[g * 12 + k]);
        }
    }
    CK(zcoords.download(m->coords, nuv * 3) && dcells.download(m->cells, nit) && ztb.download(m->t_bases, ntb) &&
       ztw.download(m->t_w, ntb) && ztoff.download(m->t_off, nuv + 1) && cell_bg.download(m->cell_bg, nec) &&
       cell_ph.download(m->cell_phase, nec));
    CK(tv0.download(m->ig_v[0], tot[0] * 4) && tv1.download(m->ig_v[1], tot[1] * 4) &&
       txi0.download(m->ig_xi[0], tot[0] * 12) && txi1.download(m->ig_xi[1], tot[1] * 12) &&
       tx0.download(m->ig_x[0], tot[0] * 12) && tx1.download(m->ig_x[1], tot[1] * 12) &&
       fv.download(m->if_v, tot[2] * 3) && fxi.download(m->if_xi, tot[2] * 9) && fx.download(m->if_x, tot[2] * 9));
    CK(ot0.download(m->ig_off[0], ncut + 1) && ot1.download(m->ig_off[1], ncut + 1) &&
       ofc.download(m->if_off, ncut + 1));
    std::vector<int32_t> hk, hp;
    std::vector<double> hx, hv;
    CK(vkind.download(hk, nv) && vpar.download(hp, nv * 8) && vx.download(hx, nv * 3) && vval.download(hv, nv));
    m->verts.resize(nv);
    for (int64_t i = 0; i < nv; ++i) {
        IgVertex& v = m->verts[i];
        v.kind = hk[i];
        for (int k = 0; k < 8; ++k) v.parents[k] = hp[i * 8 + k];
        for (int d = 0; d < 3; ++d) v.x[d] = hx[i * 3 + d];
        v.value = hv[i];
    }
#undef CK
#undef STAGE
    *out = m;
    return FEM_GPU_OK;
}

}  // extern "C"
