// Mutation sweep over the restart-file parser, built with the library's
// restart unit alone (host code) under AddressSanitizer and
// UndefinedBehaviorSanitizer.  Every mutated text is handed over in a heap
// buffer of exactly its length, so a read past the end is reported; every
// parse must end in GBFV_OK, GBFV_ERR_ARG or GBFV_ERR_UNSUPPORTED.
// Exit status 0 when all parses behaved, 1 otherwise (the sanitizers abort
// on their own reports).
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "gbfv.h"

// the restart unit's links into the rest of the library: the error text and
// the context calls of gbfv_write_restart / gbfv_read_restart (not used here)
namespace gbfv {
void setLastError(const std::string&) {}
void entitiesOf(const gbfv_ctx*, int32_t& codim, int32_t& numElements)
{
    codim = 0;
    numElements = 0;
}
}
extern "C" {
int gbfv_dims(const gbfv_ctx*, int*, int*, int*) { return GBFV_ERR_ARG; }
int gbfv_set_solution(gbfv_ctx*, const double*, const int32_t*) { return GBFV_ERR_ARG; }
int gbfv_get_solution(gbfv_ctx*, double*, int32_t*) { return GBFV_ERR_ARG; }
}

namespace {

uint64_t g_rng = 0x9e3779b97f4a7c15ull;
uint64_t next()
{
    g_rng ^= g_rng << 13;
    g_rng ^= g_rng >> 7;
    g_rng ^= g_rng << 17;
    return g_rng;
}

struct Case {
    gbfv_restart_info info;
    int n, b;
    bool gas;
    std::string text;
};

Case makeCase(int n, int b, bool gas, bool vtk)
{
    Case c{};
    c.info.num_cpus = 1;
    c.info.num_edges = 2 * n + 3;
    c.info.num_vertices = n + 7;
    c.info.time = 86400.0 * 3;
    c.info.time_step_index = 3;
    c.info.vtk_section = vtk;
    c.info.vtk_writer_num = vtk ? 4 : 0;
    c.n = n;
    c.b = b;
    c.gas = gas;
    std::vector<double> pv((size_t)n * b);
    std::vector<int32_t> gm((size_t)n);
    for (auto& v : pv) v = ((double)(next() % 2000001) - 1e6) * 1e-3;
    for (auto& m : gm) m = (int32_t)(next() % 3);
    size_t len = 0;
    if (gbfv_format_restart(&c.info, n, b, pv.data(), gas ? gm.data() : nullptr, nullptr, 0, &len)) abort();
    c.text.resize(len);
    if (gbfv_format_restart(&c.info, n, b, pv.data(), gas ? gm.data() : nullptr, &c.text[0], len, &len)) abort();
    return c;
}

long g_parses = 0, g_ok = 0, g_bad = 0;

int parse(const Case& c, const std::string& t)
{
    // exactly t.size() bytes on the heap (one byte for an empty text, with
    // length 0), so the sanitizer sees any read beyond the text
    char* buf = static_cast<char*>(malloc(t.empty() ? 1 : t.size()));
    if (!t.empty()) memcpy(buf, t.data(), t.size());
    std::vector<double> pv((size_t)c.n * c.b);
    std::vector<int32_t> gm((size_t)c.n);
    gbfv_restart_info out{};
    const int st = gbfv_parse_restart(buf, t.size(), &c.info, c.n, c.b, pv.data(), c.gas ? gm.data() : nullptr, &out);
    free(buf);
    ++g_parses;
    if (st == GBFV_OK) ++g_ok;
    if (st != GBFV_OK && st != GBFV_ERR_ARG && st != GBFV_ERR_UNSUPPORTED) {
        fprintf(stderr, "unexpected status %d\n", st);
        ++g_bad;
    }
    return st;
}

void expect(const Case& c, const std::string& t, int want, const char* what)
{
    const int st = parse(c, t);
    if (st != want) {
        fprintf(stderr, "%s: status %d, expected %d\n", what, st, want);
        ++g_bad;
    }
}

// the text with the k-th blank-separated field of line `line` replaced
std::string withField(const std::string& t, int line, int k, const std::string& v)
{
    size_t a = 0;
    for (int i = 0; i < line; ++i) a = t.find('\n', a) + 1;
    size_t e = t.find('\n', a);
    std::string l = t.substr(a, e - a);
    size_t f = 0;
    for (int i = 0; i < k; ++i) f = l.find(' ', f) + 1;
    size_t fe = l.find(' ', f);
    if (fe == std::string::npos) fe = l.size();
    l.replace(f, fe - f, v);
    return t.substr(0, a) + l + t.substr(e);
}

int lineOf(const std::string& t, const char* head)
{
    size_t p = t.find(head);
    int n = 0;
    for (size_t i = 0; i < p; ++i) n += t[i] == '\n';
    return n;
}

}  // namespace

int main()
{
    const char* specials[] = {"nan", "-nan", "inf", "-inf", "1e300", "-1e300", "2.5", "-1", "4294967296",
                              "2147483648", "-2147483649", "0x10", "", "1e", "--1", "3", "7"};
    std::vector<Case> cases = {makeCase(40, 3, true, false), makeCase(40, 3, true, true),
                               makeCase(30, 2, false, false), makeCase(30, 2, false, true)};
    for (const Case& c : cases) {
        expect(c, c.text, GBFV_OK, "unchanged text");
        // every prefix
        for (size_t k = 0; k < c.text.size(); ++k) parse(c, c.text.substr(0, k));
        // single bytes replaced, deleted, inserted
        const std::string alpha = "0123456789.-+eEnaix \n\t";
        for (int i = 0; i < 6000; ++i) {
            std::string t = c.text;
            const size_t at = next() % t.size();
            const char ch = (next() & 3) ? alpha[next() % alpha.size()] : (char)(next() & 0xff);
            switch (next() % 3) {
            case 0: t[at] = ch; break;
            case 1: t.erase(at, 1); break;
            default: t.insert(at, 1, ch); break;
            }
            parse(c, t);
        }
        // chunks cut out or repeated
        for (int i = 0; i < 1500; ++i) {
            std::string t = c.text;
            const size_t at = next() % t.size(), n = 1 + next() % 64;
            if (next() & 1)
                t.erase(at, n);
            else
                t.insert(at, t.substr(at, n));
            parse(c, t);
        }
        // special numbers in every field of the Simulator, VTK and first entity lines
        const int sim = lineOf(c.text, "Simulator\n") + 1;
        const int ent = lineOf(c.text, "Entities: Codim 0") + 1;
        std::vector<std::pair<int, int>> fields;
        for (int k = 0; k < 6; ++k) fields.push_back({sim, k});
        if (c.info.vtk_section) {
            const int vtk = lineOf(c.text, "VTKMultiWriter") + 1;
            fields.push_back({vtk, 0});
            fields.push_back({vtk + 1, 0});
        }
        for (int k = 0; k < c.b + (c.gas ? 4 : 0); ++k) fields.push_back({ent, k});
        for (auto f : fields)
            for (const char* s : specials) parse(c, withField(c.text, f.first, f.second, s));
    }
    // the outcomes the parser promises for malformed integer fields
    const Case& bo = cases[1];
    const int sim = lineOf(bo.text, "Simulator\n") + 1;
    const int vtk = lineOf(bo.text, "VTKMultiWriter") + 1;
    const int ent = lineOf(bo.text, "Entities: Codim 0") + 1;
    expect(bo, withField(bo.text, sim, 0, "1e300"), GBFV_ERR_ARG, "episode index out of range");
    expect(bo, withField(bo.text, sim, 5, "2.5"), GBFV_ERR_ARG, "fractional time step index");
    expect(bo, withField(bo.text, vtk, 0, "nan"), GBFV_ERR_ARG, "writer count NaN");
    expect(bo, withField(bo.text, vtk + 1, 0, "nan"), GBFV_ERR_ARG, "meta length NaN");
    expect(bo, withField(bo.text, vtk + 1, 0, "1e300"), GBFV_ERR_ARG, "meta length past the end");
    expect(bo, withField(bo.text, ent, 3, "3"), GBFV_ERR_UNSUPPORTED, "gas meaning Disabled");
    expect(bo, withField(bo.text, ent, 3, "7"), GBFV_ERR_ARG, "gas meaning out of range");
    expect(bo, withField(bo.text, ent, 3, "1.5"), GBFV_ERR_ARG, "fractional gas meaning");
    expect(bo, withField(bo.text, ent, 4, "2"), GBFV_ERR_UNSUPPORTED, "water meaning Rsw");
    expect(bo, withField(bo.text, ent, 5, "3"), GBFV_ERR_ARG, "pressure meaning out of range");
    expect(bo, withField(bo.text, ent, 6, "1"), GBFV_ERR_UNSUPPORTED, "second PVT region");
    expect(bo, withField(bo.text, ent, 6, "-1"), GBFV_ERR_ARG, "negative PVT region");
    // a large state: the threaded entity parser
    Case big = makeCase(70000, 3, true, false);
    expect(big, big.text, GBFV_OK, "large unchanged text");
    expect(big, big.text.substr(0, big.text.size() - 40), GBFV_ERR_ARG, "large text truncated");
    printf("parses %ld ok %ld unexpected %ld\n", g_parses, g_ok, g_bad);
    return g_bad ? 1 : 0;
}
