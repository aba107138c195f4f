// fem_vis.cpp -- field output as an Exodus II file (the reference's VIS output
// path: VIS::Output_Manager::write_mesh / write_field, FEM/VIS/src/
// cl_VIS_Output_Manager.cpp:244-785, through mtk::Writer_Exodus, MTK/src/io/
// cl_MTK_Writer_Exodus.cpp:112-420, which calls the SEACAS exodus library).
//
// The exodus library is not available here, so the file is written directly
// in the netCDF classic format with 64-bit offsets (CDF-2) that Exodus II
// files use, with the Exodus II names: one element block (id 1), coordinates
// coordx / coordy / coordz, connectivity connect1 with its elem_type
// attribute (1-based node numbers), nodal variables vals_nod_var<k> named in
// name_nod_var, and one time step in time_whole.  Host code.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "fem_internal.hpp"

namespace {

enum NcType { NC_CHAR = 2, NC_INT = 4, NC_FLOAT = 5, NC_DOUBLE = 6 };
constexpr int kLenName = 33;

struct Buf {
    std::vector<unsigned char> b;
    void u32(uint32_t v) {
        for (int s = 24; s >= 0; s -= 8) b.push_back((unsigned char)(v >> s));
    }
    void u64(uint64_t v) {
        for (int s = 56; s >= 0; s -= 8) b.push_back((unsigned char)(v >> s));
    }
    void f64(double v) {
        uint64_t u;
        std::memcpy(&u, &v, 8);
        u64(u);
    }
    void f32(float v) {
        uint32_t u;
        std::memcpy(&u, &v, 4);
        u32(u);
    }
    void pad() {
        while (b.size() % 4) b.push_back(0);
    }
    void name(const std::string& s) {
        u32((uint32_t)s.size());
        b.insert(b.end(), s.begin(), s.end());
        pad();
    }
};

struct Dim {
    std::string name;
    uint64_t len;  // 0: the record (unlimited) dimension
};
struct Att {
    std::string name;
    int type;
    std::string text;   // NC_CHAR
    double num = 0.0;   // NC_INT / NC_FLOAT / NC_DOUBLE, one value
};
struct Var {
    std::string name;
    std::vector<int> dims;
    std::vector<Att> atts;
    int type;
    std::vector<unsigned char> data;  // big-endian values (one record for record variables)
    bool record = false;
    uint64_t vsize = 0, begin = 0;
};

void put_atts(Buf& h, const std::vector<Att>& atts) {
    if (atts.empty()) {
        h.u32(0);
        h.u32(0);
        return;
    }
    h.u32(0x0C);
    h.u32((uint32_t)atts.size());
    for (const Att& a : atts) {
        h.name(a.name);
        h.u32((uint32_t)a.type);
        if (a.type == NC_CHAR) {
            h.u32((uint32_t)a.text.size());
            h.b.insert(h.b.end(), a.text.begin(), a.text.end());
        } else {
            h.u32(1);
            if (a.type == NC_INT) h.u32((uint32_t)(int32_t)a.num);
            else if (a.type == NC_FLOAT) h.f32((float)a.num);
            else h.f64(a.num);
        }
        h.pad();
    }
}

int type_size(int t) { return t == NC_CHAR ? 1 : t == NC_INT || t == NC_FLOAT ? 4 : 8; }

std::vector<unsigned char> chars(const std::vector<std::string>& names, int width) {
    std::vector<unsigned char> d((size_t)names.size() * width, 0);
    for (size_t i = 0; i < names.size(); ++i)
        std::memcpy(&d[i * width], names[i].data(), std::min<size_t>(names[i].size(), width - 1));
    return d;
}

}  // namespace

using namespace fem;

extern "C" {

fem_gpu_status fem_vis_write_exodus(const char* path, int32_t dim, int64_t num_nodes, const double* coords,
                                    int64_t num_cells, int32_t nodes_per_cell, const int32_t* cell_nodes,
                                    const char* elem_type, int32_t num_fields, const char* const* field_names,
                                    const double* field_values, double time) {
    if (!path || dim < 1 || dim > 3 || num_nodes < 1 || !coords || num_cells < 1 || nodes_per_cell < 1 ||
        !cell_nodes || !elem_type || num_fields < 0 || (num_fields && (!field_names || !field_values)))
        return FEM_GPU_BAD_ARG;
    for (int64_t i = 0; i < num_cells * nodes_per_cell; ++i)
        if (cell_nodes[i] < 0 || cell_nodes[i] >= num_nodes) return FEM_GPU_OOB_INDEX;
    std::vector<Dim> dims = {{"len_string", 33},     {"len_line", 81},         {"four", 4},
                             {"len_name", kLenName}, {"time_step", 0},         {"num_dim", (uint64_t)dim},
                             {"num_nodes", (uint64_t)num_nodes},  {"num_elem", (uint64_t)num_cells},
                             {"num_el_blk", 1},      {"num_el_in_blk1", (uint64_t)num_cells},
                             {"num_nod_per_el1", (uint64_t)nodes_per_cell}};
    auto dim_id = [&](const char* n) {
        for (size_t i = 0; i < dims.size(); ++i)
            if (dims[i].name == n) return (int)i;
        return -1;
    };
    if (num_fields) dims.push_back({"num_nod_var", (uint64_t)num_fields});
    std::vector<Att> gatts = {{"api_version", NC_FLOAT, "", 8.03},
                              {"version", NC_FLOAT, "", 8.03},
                              {"floating_point_word_size", NC_INT, "", 8},
                              {"file_size", NC_INT, "", 1},
                              {"maximum_name_length", NC_INT, "", 32},
                              {"int64_status", NC_INT, "", 0},
                              {"title", NC_CHAR, "moris_gb300", 0}};
    std::vector<Var> vars;
    auto be_f64 = [](const double* v, int64_t n, int64_t stride) {
        Buf b;
        for (int64_t i = 0; i < n; ++i) b.f64(v[i * stride]);
        return b.b;
    };
    {
        Var v{"time_whole", {dim_id("time_step")}, {}, NC_DOUBLE, be_f64(&time, 1, 1), true};
        vars.push_back(v);
    }
    {
        Buf b;
        b.u32(1);
        vars.push_back(Var{"eb_status", {dim_id("num_el_blk")}, {}, NC_INT, b.b});
        Buf p;
        p.u32(1);
        vars.push_back(Var{"eb_prop1", {dim_id("num_el_blk")}, {{"name", NC_CHAR, "ID", 0}}, NC_INT, p.b});
    }
    const char* axes[3] = {"coordx", "coordy", "coordz"};
    for (int d = 0; d < dim; ++d)
        vars.push_back(Var{axes[d], {dim_id("num_nodes")}, {}, NC_DOUBLE, be_f64(coords + d, num_nodes, dim)});
    {
        std::vector<std::string> cn = {"x", "y", "z"};
        cn.resize(dim);
        vars.push_back(Var{"coor_names", {dim_id("num_dim"), dim_id("len_name")}, {}, NC_CHAR, chars(cn, kLenName)});
        vars.push_back(
            Var{"eb_names", {dim_id("num_el_blk"), dim_id("len_name")}, {}, NC_CHAR, chars({"block_1"}, kLenName)});
    }
    {
        Buf b;
        for (int64_t i = 0; i < num_cells * nodes_per_cell; ++i) b.u32((uint32_t)(cell_nodes[i] + 1));
        vars.push_back(Var{"connect1", {dim_id("num_el_in_blk1"), dim_id("num_nod_per_el1")},
                           {{"elem_type", NC_CHAR, elem_type, 0}}, NC_INT, b.b});
    }
    if (num_fields) {
        std::vector<std::string> fn(field_names, field_names + num_fields);
        vars.push_back(
            Var{"name_nod_var", {dim_id("num_nod_var"), dim_id("len_name")}, {}, NC_CHAR, chars(fn, kLenName)});
        for (int k = 0; k < num_fields; ++k) {
            Var v{"vals_nod_var" + std::to_string(k + 1), {dim_id("time_step"), dim_id("num_nodes")}, {}, NC_DOUBLE,
                  be_f64(field_values + (int64_t)k * num_nodes, num_nodes, 1), true};
            vars.push_back(v);
        }
    }
    // sizes and offsets: non-record variables first in list order, then the records
    for (Var& v : vars) {
        uint64_t n = type_size(v.type);
        for (int d : v.dims)
            if (dims[d].len) n *= dims[d].len;
        v.vsize = (n + 3) / 4 * 4;
    }
    auto header = [&]() {
        Buf h;
        h.b = {'C', 'D', 'F', 2};
        h.u32(1);  // numrecs
        h.u32(0x0A);
        h.u32((uint32_t)dims.size());
        for (const Dim& d : dims) {
            h.name(d.name);
            h.u32((uint32_t)d.len);
        }
        put_atts(h, gatts);
        h.u32(0x0B);
        h.u32((uint32_t)vars.size());
        for (const Var& v : vars) {
            h.name(v.name);
            h.u32((uint32_t)v.dims.size());
            for (int d : v.dims) h.u32((uint32_t)d);
            put_atts(h, v.atts);
            h.u32((uint32_t)v.type);
            h.u32((uint32_t)v.vsize);
            h.u64(v.begin);
        }
        return h.b;
    };
    uint64_t off = header().size();
    for (Var& v : vars)
        if (!v.record) {
            v.begin = off;
            off += v.vsize;
        }
    for (Var& v : vars)
        if (v.record) {
            v.begin = off;
            off += v.vsize;
        }
    const std::vector<unsigned char> h = header();
    FILE* f = std::fopen(path, "wb");
    if (!f) return FEM_GPU_BAD_ARG;
    bool ok = std::fwrite(h.data(), 1, h.size(), f) == h.size();
    for (int pass = 0; pass < 2 && ok; ++pass)
        for (const Var& v : vars) {
            if (v.record != (pass == 1)) continue;
            ok = ok && std::fwrite(v.data.data(), 1, v.data.size(), f) == v.data.size();
            static const unsigned char zeros[4] = {0, 0, 0, 0};
            const size_t padn = v.vsize - v.data.size();
            ok = ok && (padn == 0 || std::fwrite(zeros, 1, padn, f) == padn);
        }
    ok = (std::fclose(f) == 0) && ok;
    return ok ? FEM_GPU_OK : FEM_GPU_BAD_ARG;
}

}  // extern "C"
