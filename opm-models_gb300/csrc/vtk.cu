// VTK output of a context's state: one XML UnstructuredGrid file (.vtu) per
// time step with the fields the reference's VTK output modules write, and
// the collection file (.pvd) that lists the time steps.
//
// The reference (VtkMultiWriter, opm/models/io/vtkmultiwriter.hh:64-540)
// hands element buffers filled by VtkPrimaryVarsModule
// (vtkprimaryvarsmodule.hh:54-170) and VtkMultiPhaseModule
// (vtkmultiphasemodule.hh:84-460) to dune-grid's VTK writer.  Here the
// quantities come from the device in one pass (gbfv_output_fields: the
// intensive-quantity kernel with its values written out), are copied to the
// host once and formatted by several host threads; the file follows the
// published VTK XML format with the reference's field names and order, its
// default field set (the VtkWrite* parameters) and its ASCII default
// (fvbasediscretization.hh:237-238).  Every value is rounded to float first,
// as VtkScalarFunction::evaluate does (vtkscalarfunction.hh:76-110), and
// printed with 9 significant digits, which reads back to the same float.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/gbfv.h"
#include "gbfv_internal.cuh"

namespace gbfv {
void setLastError(const std::string& s);  // gbfv.cu: the message gbfv_last_error returns
}

namespace {

// the reference's phase and primary-variable names: FluidSystem::phaseName
// (opm-common's two-phase immiscible and black-oil fluid systems) and
// primaryVarName (immisciblemodel.hh:257-277, blackoilmodel.hh:345-367)
const char* phaseName(int b, int a)
{
    static const char* two[2] = {"w", "n"};
    static const char* three[3] = {"water", "oil", "gas"};
    return b == 2 ? two[a] : three[a];
}
const char* pvName(int b, int e)
{
    static const char* two[2] = {"pressure_w", "saturation_w"};
    static const char* three[3] = {"water_switching", "pressure_switching", "composition_switching"};
    return b == 2 ? two[e] : three[e];
}

// n values formatted as text, `perLine` per line, by up to 16 host threads
// working on contiguous ranges (the order is kept)
template <class F>
std::string formatValues(size_t n, int perLine, F&& one)
{
    const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    const size_t chunks = std::min<size_t>(hw, std::max<size_t>(1, n / 4096));
    std::vector<std::string> parts(chunks);
    auto work = [&](size_t c) {
        const size_t lo = n * c / chunks, hi = n * (c + 1) / chunks;
        std::string& s = parts[c];
        s.reserve((hi - lo) * 16);
        char buf[64];
        for (size_t i = lo; i < hi; ++i) {
            const int len = one(i, buf, sizeof(buf));
            s.append(buf, (size_t)len);
            s.push_back(((i + 1) % (size_t)perLine == 0 || i + 1 == n) ? '\n' : ' ');
        }
    };
    std::vector<std::thread> th;
    for (size_t c = 1; c < chunks; ++c) th.emplace_back(work, c);
    work(0);
    for (auto& t : th) t.join();
    std::string all;
    size_t total = 0;
    for (auto& p : parts) total += p.size();
    all.reserve(total);
    for (auto& p : parts) all += p;
    return all;
}

std::string floatArray(const char* name, int comps, size_t n, const float* v)
{
    std::string s = "        <DataArray type=\"Float32\" Name=\"" + std::string(name) + "\" NumberOfComponents=\"" +
                    std::to_string(comps) + "\" format=\"ascii\">\n";
    s += formatValues(n * (size_t)comps, 6 * comps, [&](size_t i, char* buf, size_t cap) {
        return std::snprintf(buf, cap, "%.9g", (double)v[i]);
    });
    s += "        </DataArray>\n";
    return s;
}

template <class I>
std::string intArray(const char* type, const char* name, size_t n, const I* v)
{
    std::string s = "        <DataArray type=\"" + std::string(type) + "\" Name=\"" + std::string(name) +
                    "\" NumberOfComponents=\"1\" format=\"ascii\">\n";
    s += formatValues(n, 12, [&](size_t i, char* buf, size_t cap) {
        return std::snprintf(buf, cap, "%lld", (long long)v[i]);
    });
    s += "        </DataArray>\n";
    return s;
}

bool writeFile(const char* path, const std::string& text)
{
    FILE* f = std::fopen(path, "wb");
    if (!f) return false;
    const bool ok = std::fwrite(text.data(), 1, text.size(), f) == text.size();
    return std::fclose(f) == 0 && ok;
}

}  // namespace

extern "C" {

int gbfv_write_vtk(gbfv_ctx* ctx, const gbfv_vtk_grid* g, int32_t fields, const char* path)
{
    if (!ctx || !g || !path || !g->points || !g->cell_vertices || g->num_points <= 0 ||
        (g->vertices_per_cell != 4 && g->vertices_per_cell != 8) || fields < 0 || fields > 511) {
        gbfv::setLastError("gbfv_write_vtk: null pointer, no points, vertices_per_cell other than 4 or 8, or "
                           "unknown field bits");
        return GBFV_ERR_ARG;
    }
    int N = 0, b = 0, nnz = 0;
    int st = gbfv_dims(ctx, &N, &b, &nnz);
    if (st) return st;
    // a vertex-centred grid: the degrees of freedom are the points
    const bool pointData = g->num_cells > 0;
    if (g->num_cells < 0 || (pointData && g->num_points != N)) {
        gbfv::setLastError("gbfv_write_vtk: num_cells < 0, or vertex data with num_points other than the "
                           "context's degrees of freedom");
        return GBFV_ERR_ARG;
    }
    const int NC = pointData ? g->num_cells : N;
    const size_t vpc = (size_t)g->vertices_per_cell;
    for (size_t k = 0; k < (size_t)NC * vpc; ++k)
        if (g->cell_vertices[k] < 0 || g->cell_vertices[k] >= g->num_points) {
            gbfv::setLastError("gbfv_write_vtk: cell vertex index out of range at entry " + std::to_string(k));
            return GBFV_ERR_ARG;
        }
    std::vector<double> out((size_t)GBFV_OUTPUT_PLANES * N);
    if ((st = gbfv_output_fields(ctx, out.data()))) return st;
    const int np = b == 3 ? 3 : 2;
    std::string cells;
    std::vector<float> f(N);
    std::string first;
    auto plane = [&](int q) {
        for (int i = 0; i < N; ++i) f[i] = (float)out[(size_t)q * N + i];
    };
    auto add = [&](const std::string& name) {
        if (first.empty()) first = name;
        cells += floatArray(name.c_str(), 1, (size_t)N, f.data());
    };
    // VtkPrimaryVarsModule (attached first by the model), then VtkMultiPhaseModule
    if (fields & GBFV_VTK_PRIMARY_VARS) {
        std::vector<double> pv((size_t)N * b);
        if ((st = gbfv_get_solution(ctx, pv.data(), nullptr))) return st;
        for (int e = 0; e < b; ++e) {
            for (int i = 0; i < N; ++i) f[i] = (float)pv[(size_t)i * b + e];
            add(std::string("PV_") + pvName(b, e));
        }
    }
    if (fields & GBFV_VTK_DOF_INDEX) {
        for (int i = 0; i < N; ++i) f[i] = (float)i;
        add("DOF index");
    }
    const struct {
        int bit, q;
        const char* pattern;
    } phaseFields[] = {{GBFV_VTK_PRESSURE, 0, "pressure_"},  {GBFV_VTK_DENSITY, 1, "density_"},
                       {GBFV_VTK_SATURATION, 2, "saturation_"}, {GBFV_VTK_MOBILITY, 3, "mobility_"},
                       {GBFV_VTK_RELPERM, 4, "relativePerm_"}, {GBFV_VTK_VISCOSITY, 5, "viscosity_"}};
    for (const auto& pf : phaseFields) {
        if (!(fields & pf.bit)) continue;
        for (int a = 0; a < np; ++a) {
            plane(3 * pf.q + a);
            add(std::string(pf.pattern) + phaseName(b, a));
        }
    }
    if (fields & GBFV_VTK_POROSITY) {
        plane(18);
        add("porosity");
    }
    std::vector<float> pts((size_t)g->num_points * 3);
    for (size_t k = 0; k < pts.size(); ++k) pts[k] = (float)g->points[k];
    std::vector<int32_t> offsets(NC);
    std::vector<uint8_t> types(NC, (uint8_t)(vpc == 4 ? 9 : 12));  // VTK_QUAD, VTK_HEXAHEDRON
    for (int i = 0; i < NC; ++i) offsets[i] = (int32_t)((size_t)(i + 1) * vpc);
    std::string doc = "<?xml version=\"1.0\"?>\n"
                      "<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\">\n"
                      "  <UnstructuredGrid>\n"
                      "    <Piece NumberOfCells=\"" + std::to_string(NC) + "\" NumberOfPoints=\"" +
                      std::to_string(g->num_points) + "\">\n";
    const char* section = pointData ? "PointData" : "CellData";
    if (!first.empty())
        doc += std::string("      <") + section + " Scalars=\"" + first + "\">\n" + cells + "      </" + section + ">\n";
    doc += "      <Points>\n" + floatArray("Coordinates", 3, (size_t)g->num_points, pts.data()) + "      </Points>\n";
    doc += "      <Cells>\n";
    doc += intArray("Int32", "connectivity", (size_t)NC * vpc, g->cell_vertices);
    doc += intArray("Int32", "offsets", (size_t)NC, offsets.data());
    doc += intArray("UInt8", "types", (size_t)NC, types.data());
    doc += "      </Cells>\n    </Piece>\n  </UnstructuredGrid>\n</VTKFile>\n";
    if (!writeFile(path, doc)) {
        gbfv::setLastError(std::string("gbfv_write_vtk: cannot write ") + path);
        return GBFV_ERR_ARG;
    }
    return GBFV_OK;
}

int gbfv_vtk_file_name(const char* sim_name, int32_t writer_num, char* buf, size_t cap)
{
    if (!buf || writer_num < 0) return GBFV_ERR_ARG;
    const char* s = (sim_name && *sim_name) ? sim_name : "sim";
    const int n = std::snprintf(buf, cap, "%s-%05d.vtu", s, (int)writer_num);
    return (n < 0 || (size_t)n >= cap) ? GBFV_ERR_ARG : GBFV_OK;
}

int gbfv_write_pvd(const char* path, int32_t n, const double* times, const char* const* files)
{
    if (!path || n < 0 || (n > 0 && (!times || !files))) return GBFV_ERR_ARG;
    std::string doc = "<?xml version=\"1.0\"?>\n"
                      "<VTKFile type=\"Collection\"\n"
                      "         version=\"0.1\"\n"
                      "         byte_order=\"LittleEndian\"\n"
                      "         compressor=\"vtkZLibDataCompressor\">\n"
                      " <Collection>\n";
    char buf[64];
    for (int i = 0; i < n; ++i) {
        if (!files[i]) return GBFV_ERR_ARG;
        std::snprintf(buf, sizeof(buf), "%.16g", times[i]);
        doc += std::string("   <DataSet timestep=\"") + buf + "\" file=\"" + files[i] + "\"/>\n";
    }
    doc += " </Collection>\n</VTKFile>\n";
    if (!writeFile(path, doc)) {
        gbfv::setLastError(std::string("gbfv_write_pvd: cannot write ") + path);
        return GBFV_ERR_ARG;
    }
    return GBFV_OK;
}

}  // extern "C"
