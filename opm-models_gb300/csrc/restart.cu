// Restart files of a context's state in the reference's text format, so a
// run can be stopped on the device and continued by either side.
//
// Layout (Opm::Restart, opm/models/io/restart.hh:101-265): sections, each a
// cookie line, its content and one closing "\n" (serializeSectionBegin/End,
// restart.hh:125-135), in the order Simulator::serialize writes them
// (opm/models/utils/simulator.hh:906-962):
//   1. the magic cookie (restart.hh:57-75), empty content;
//   2. "Simulator": episodeIdx episodeStartTime episodeLength startTime time
//      timeStepIdx, each followed by one blank (simulator.hh:930-943);
//   3. "VTKMultiWriter" when the problem writes VTK output (fvbaseproblem.hh:
//      755-760, vtkmultiwriter.hh:408-437): the writer count, then the
//      length and position of the .pvd meta file (two blanks between) and
//      its bytes; this library writes no meta file, so both are 0;
//   4. "Entities: Codim 0" (ECFV: one line per element in grid order,
//      ecfvdiscretization.hh:212-226, restart.hh:141-160): the primary
//      variables, each followed by a blank (fvbasediscretization.hh:
//      1440-1454); black-oil adds the gas, water and pressure meanings and
//      the PVT region index (blackoilmodel.hh:468-493).
// Numbers are written as an std::ostream with precision(20) writes them
// (restart.hh:115): "%.20g" for floating point, plain integers.  That is
// enough digits for every double to read back to the same bits.
//
// Text formatting is host work (the state is copied out once); large
// states are formatted by several threads, one contiguous range of cells
// each, and concatenated in order.
#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/gbfv.h"

namespace gbfv {
void setLastError(const std::string& s);
// the context's restart entities: codim 0 (cells) or, on a vertex-centred
// grid, its dimension (vertices) and the element count
void entitiesOf(const gbfv_ctx* ctx, int32_t& codim, int32_t& numElements);
}

namespace {

// the entities are the cells (codim 0) or, on a vertex-centred grid, the
// vertices; the cookie's element count follows
int numElementsOf(const gbfv_restart_info& in, int numCells)
{
    return in.entity_codim > 0 ? in.num_elements : numCells;
}

std::string entitiesLine(const gbfv_restart_info& in)
{
    return "Entities: Codim " + std::to_string(in.entity_codim);
}

std::string cookie(const gbfv_restart_info& in, int numCells)
{
    char buf[256];
    snprintf(buf, sizeof buf,
             "eWoms restart file: gridName='blubb' numCPUs=%d myRank=%d numElements=%d numEdges=%d numVertices=%d",
             in.num_cpus, in.rank, numElementsOf(in, numCells), in.num_edges, in.num_vertices);
    return buf;
}

void putG(std::string& s, double v)
{
    char buf[40];
    const int n = snprintf(buf, sizeof buf, "%.20g", v);
    s.append(buf, (size_t)n);
}

void putI(std::string& s, long long v)
{
    char buf[24];
    const int n = snprintf(buf, sizeof buf, "%lld", v);
    s.append(buf, (size_t)n);
}

// the entity lines of cells [c0, c1)
void entityLines(std::string& s, int c0, int c1, int b, const double* pv, const int32_t* gas)
{
    for (int c = c0; c < c1; ++c) {
        for (int e = 0; e < b; ++e) {
            putG(s, pv[(size_t)c * b + e]);
            s += ' ';
        }
        if (gas) {  // gas, water (Sw = 0) and pressure (Po = 0) meanings, PVT region 0
            putI(s, gas[c]);
            s += " 0 0 0 ";
        }
        s += '\n';
    }
}

std::string formatRestart(const gbfv_restart_info& in, int numCells, int b, const double* pv, const int32_t* gas)
{
    std::string s = cookie(in, numCells);
    s += "\n\n";
    s += "Simulator\n";
    putI(s, in.episode_index);
    s += ' ';
    putG(s, in.episode_start_time);
    s += ' ';
    putG(s, in.episode_length);
    s += ' ';
    putG(s, in.start_time);
    s += ' ';
    putG(s, in.time);
    s += ' ';
    putI(s, in.time_step_index);
    s += " \n";
    if (in.vtk_section) {
        s += "VTKMultiWriter\n";
        putI(s, in.vtk_writer_num);
        s += "\n0  0\n\n";
    }
    s += entitiesLine(in) + "\n";
    const int nt = numCells < 65536 ? 1
                                    : (int)std::min<unsigned>(16u, std::max(1u, std::thread::hardware_concurrency()));
    std::vector<std::string> part(nt);
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t) {
        const int c0 = (int)((long long)numCells * t / nt), c1 = (int)((long long)numCells * (t + 1) / nt);
        if (nt == 1)
            entityLines(part[t], c0, c1, b, pv, gas);
        else
            th.emplace_back([&part, t, c0, c1, b, pv, gas] { entityLines(part[t], c0, c1, b, pv, gas); });
    }
    for (auto& x : th) x.join();
    for (auto& p : part) s += p;
    s += '\n';
    return s;
}

// a line-oriented reader over the text
struct Reader {
    const char* p;
    const char* end;
    bool line(std::string& out)
    {
        if (p >= end) return false;
        const char* q = static_cast<const char*>(memchr(p, '\n', (size_t)(end - p)));
        if (!q) q = end;
        out.assign(p, (size_t)(q - p));
        p = q < end ? q + 1 : end;
        return true;
    }
};

bool expectLine(Reader& r, const std::string& want, const char* what)
{
    std::string l;
    if (!r.line(l) || l != want) {
        gbfv::setLastError(std::string("restart file: expected ") + what + " '" + want + "'");
        return false;
    }
    return true;
}

// end of a section: a line of blanks only (deserializeSectionEnd, restart.hh:220-229)
bool sectionEnd(Reader& r, const char* what)
{
    std::string l;
    if (!r.line(l) || l.find_first_not_of(" \t\r\f\v") != std::string::npos) {
        gbfv::setLastError(std::string("restart file: unread values at the end of ") + what);
        return false;
    }
    return true;
}

// `count` numbers of one line (strtod), nothing but blanks after them
bool numbers(const std::string& l, int count, double* d)
{
    const char* s = l.c_str();
    for (int k = 0; k < count; ++k) {
        char* e = nullptr;
        errno = 0;
        d[k] = strtod(s, &e);
        if (e == s) return false;
        s = e;
    }
    while (*s == ' ') ++s;
    return *s == '\0';
}

// a parsed number as an integer in [lo, hi]: false for NaN, fractions and
// values outside the range, whose bare conversion to int would be undefined
bool asInt(double v, double lo, double hi, int32_t& out)
{
    if (!(v >= lo && v <= hi) || v != std::floor(v)) return false;
    out = (int32_t)v;
    return true;
}

constexpr double kIntMin = -2147483648.0, kIntMax = 2147483647.0;

int parseRestart(const char* text, size_t len, const gbfv_restart_info& expect, int numCells, int b, double* pv,
                 int32_t* gas, gbfv_restart_info& out)
{
    Reader r{text, text + len};
    std::string l;
    if (!expectLine(r, cookie(expect, numCells), "cookie") || !sectionEnd(r, "the cookie section") ||
        !expectLine(r, "Simulator", "section"))
        return GBFV_ERR_ARG;
    // the section's values and its end share a line (simulator.hh:951-962)
    double sim[6];
    int32_t episode = 0, step = 0;
    if (!r.line(l) || !numbers(l, 6, sim) || !asInt(sim[0], kIntMin, kIntMax, episode) ||
        !asInt(sim[5], kIntMin, kIntMax, step)) {
        gbfv::setLastError("restart file: bad Simulator section");
        return GBFV_ERR_ARG;
    }
    out = expect;
    out.episode_index = episode;
    out.episode_start_time = sim[1];
    out.episode_length = sim[2];
    out.start_time = sim[3];
    out.time = sim[4];
    out.time_step_index = step;
    out.vtk_section = 0;
    if (!r.line(l)) {
        gbfv::setLastError("restart file: truncated");
        return GBFV_ERR_ARG;
    }
    if (l == "VTKMultiWriter") {
        double w[1], fl[2];
        int32_t writer = 0, metaLen = 0;
        std::string l2;
        // the meta file's length: an integer no larger than what is left
        if (!r.line(l2) || !numbers(l2, 1, w) || !asInt(w[0], kIntMin, kIntMax, writer) || !r.line(l2) ||
            !numbers(l2, 2, fl) || !asInt(fl[0], 0.0, std::min((double)(r.end - r.p), kIntMax), metaLen)) {
            gbfv::setLastError("restart file: bad VTKMultiWriter section");
            return GBFV_ERR_ARG;
        }
        out.vtk_section = 1;
        out.vtk_writer_num = writer;
        r.p += (size_t)metaLen;  // the meta file's bytes
        if (!sectionEnd(r, "the VTKMultiWriter section") || !r.line(l)) return GBFV_ERR_ARG;
    }
    if (l != entitiesLine(expect)) {
        gbfv::setLastError("restart file: expected section '" + entitiesLine(expect) + "'");
        return GBFV_ERR_ARG;
    }
    // the entity lines: located in one pass, parsed by several threads
    std::vector<const char*> start((size_t)numCells + 1);
    for (int c = 0; c < numCells; ++c) {
        if (r.p >= r.end) {
            gbfv::setLastError("restart file: truncated at entity line " + std::to_string(c));
            return GBFV_ERR_ARG;
        }
        start[(size_t)c] = r.p;
        const char* q = static_cast<const char*>(memchr(r.p, '\n', (size_t)(r.end - r.p)));
        r.p = q ? q + 1 : r.end;
    }
    start[(size_t)numCells] = r.p;
    const int per = b + (gas ? 4 : 0);
    const int nt = numCells < 65536 ? 1
                                    : (int)std::min<unsigned>(16u, std::max(1u, std::thread::hardware_concurrency()));
    std::vector<int> bad(nt, -1), badKind(nt, 0);
    auto work = [&](int t) {
        const int c0 = (int)((long long)numCells * t / nt), c1 = (int)((long long)numCells * (t + 1) / nt);
        std::vector<double> v((size_t)per);
        std::string line;
        for (int c = c0; c < c1; ++c) {
            const char* a = start[(size_t)c];
            const char* e = start[(size_t)c + 1];
            if (e > a && e[-1] == '\n') --e;
            line.assign(a, (size_t)(e - a));
            if (!numbers(line, per, v.data())) {
                bad[t] = c;
                badKind[t] = GBFV_ERR_ARG;
                return;
            }
            for (int k = 0; k < b; ++k) pv[(size_t)c * b + k] = v[(size_t)k];
            if (gas) {
                // the reference's enums (blackoilprimaryvariables.hh:125-143):
                // gas Sg Rs Rv Disabled, water Sw Rvw Rsw Disabled, pressure
                // Po Pg Pw; a PVT region index >= 0
                int32_t gm = 0, wm = 0, pm = 0, reg = 0;
                if (!asInt(v[(size_t)b], 0, 3, gm) || !asInt(v[(size_t)b + 1], 0, 3, wm) ||
                    !asInt(v[(size_t)b + 2], 0, 2, pm) || !asInt(v[(size_t)b + 3], 0, kIntMax, reg)) {
                    bad[t] = c;
                    badKind[t] = GBFV_ERR_ARG;
                    return;
                }
                if (gm == 3 || wm != 0 || pm != 0 || reg != 0) {
                    bad[t] = c;
                    badKind[t] = GBFV_ERR_UNSUPPORTED;
                    return;
                }
                gas[c] = gm;
            }
        }
    };
    if (nt == 1)
        work(0);
    else {
        std::vector<std::thread> th;
        for (int t = 0; t < nt; ++t) th.emplace_back(work, t);
        for (auto& x : th) x.join();
    }
    for (int t = 0; t < nt; ++t)
        if (bad[t] >= 0) {
            gbfv::setLastError(badKind[t] == GBFV_ERR_UNSUPPORTED
                                   ? "restart file: disabled gas, water/pressure meaning or PVT region other than 0 "
                                     "(not supported)"
                                   : "restart file: bad entity line " + std::to_string(bad[t]));
            return badKind[t];
        }
    if (!sectionEnd(r, "the Entities section")) return GBFV_ERR_ARG;
    return GBFV_OK;
}

bool readFile(const char* path, std::string& out)
{
    FILE* f = fopen(path, "rb");
    if (!f) return false;
    char buf[1 << 16];
    size_t n;
    out.clear();
    while ((n = fread(buf, 1, sizeof buf, f)) > 0) out.append(buf, n);
    const bool ok = !ferror(f);
    fclose(f);
    return ok;
}

}  // namespace

extern "C" {

int gbfv_format_restart(const gbfv_restart_info* info, int32_t num_cells, int32_t b, const double* pv,
                        const int32_t* gas_meaning, char* buf, size_t cap, size_t* len)
{
    if (!info || num_cells < 0 || b < 1 || b > 8 || (num_cells > 0 && !pv) || !len || info->entity_codim < 0 ||
        info->entity_codim > 3)
        return GBFV_ERR_ARG;
    const std::string s = formatRestart(*info, num_cells, b, pv, gas_meaning);
    *len = s.size();
    if (buf) {
        if (cap < s.size()) return GBFV_ERR_ARG;
        memcpy(buf, s.data(), s.size());
    }
    return GBFV_OK;
}

int gbfv_parse_restart(const char* text, size_t len, const gbfv_restart_info* expect, int32_t num_cells, int32_t b,
                       double* pv, int32_t* gas_meaning, gbfv_restart_info* out)
{
    if (!text || !expect || num_cells < 0 || b < 1 || b > 8 || (num_cells > 0 && !pv) || !out ||
        expect->entity_codim < 0 || expect->entity_codim > 3)
        return GBFV_ERR_ARG;
    return parseRestart(text, len, *expect, num_cells, b, pv, gas_meaning, *out);
}

int gbfv_restart_file_name(const char* output_dir, const char* sim_name, double time, int32_t rank, char* buf,
                           size_t cap)
{
    if (!sim_name || !buf) return GBFV_ERR_ARG;
    // restartFileName_ (restart.hh:80-95): "." means the current directory;
    // the time as an std::ostream writes it by default ("%g")
    std::string dir = output_dir ? output_dir : "";
    if (dir == ".")
        dir.clear();
    else if (!dir.empty() && dir.back() != '/')
        dir += '/';
    char t[64];
    snprintf(t, sizeof t, "%g", time);
    const std::string s = dir + sim_name + "_time=" + t + "_rank=" + std::to_string(rank) + ".ers";
    if (cap < s.size() + 1) return GBFV_ERR_ARG;
    memcpy(buf, s.c_str(), s.size() + 1);
    return GBFV_OK;
}

int gbfv_write_restart(gbfv_ctx* ctx, const char* path, const gbfv_restart_info* infoIn)
{
    if (!ctx || !path || !infoIn) return GBFV_ERR_ARG;
    int n = 0, b = 0, nnz = 0;
    int st = gbfv_dims(ctx, &n, &b, &nnz);
    if (st) return st;
    gbfv_restart_info in = *infoIn;
    gbfv::entitiesOf(ctx, in.entity_codim, in.num_elements);
    const gbfv_restart_info* info = &in;
    std::vector<double> pv((size_t)n * b);
    std::vector<int32_t> gas(b == 3 ? n : 0);
    if ((st = gbfv_get_solution(ctx, pv.data(), b == 3 ? gas.data() : nullptr))) return st;
    const std::string s = formatRestart(*info, n, b, pv.data(), b == 3 ? gas.data() : nullptr);
    FILE* f = fopen(path, "wb");
    if (!f) {
        gbfv::setLastError(std::string("gbfv_write_restart: cannot open ") + path);
        return GBFV_ERR_ARG;
    }
    const bool ok = fwrite(s.data(), 1, s.size(), f) == s.size();
    if (fclose(f) != 0 || !ok) {
        gbfv::setLastError(std::string("gbfv_write_restart: write failed: ") + path);
        return GBFV_ERR_ARG;
    }
    return GBFV_OK;
}

int gbfv_read_restart(gbfv_ctx* ctx, const char* path, gbfv_restart_info* info)
{
    if (!ctx || !path || !info) return GBFV_ERR_ARG;
    int n = 0, b = 0, nnz = 0;
    int st = gbfv_dims(ctx, &n, &b, &nnz);
    if (st) return st;
    gbfv::entitiesOf(ctx, info->entity_codim, info->num_elements);
    std::string text;
    if (!readFile(path, text)) {
        gbfv::setLastError(std::string("gbfv_read_restart: cannot read ") + path);
        return GBFV_ERR_ARG;
    }
    std::vector<double> pv((size_t)n * b);
    std::vector<int32_t> gas(b == 3 ? n : 0);
    gbfv_restart_info out;
    if ((st = parseRestart(text.data(), text.size(), *info, n, b, pv.data(), b == 3 ? gas.data() : nullptr, out)))
        return st;
    // deserialize: solution(0) from the file, solution(1) = solution(0)
    // (blackoilmodel.hh:555-576); both are set by gbfv_set_solution
    if ((st = gbfv_set_solution(ctx, pv.data(), b == 3 ? gas.data() : nullptr))) return st;
    *info = out;
    return GBFV_OK;
}

}  // extern "C"
