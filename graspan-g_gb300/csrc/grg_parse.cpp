// grg_parse.cpp -- text formats of the reference (host side of the boundary).
//
// Grammar (readAndTransferRules, src/main.cpp:60-97): lines starting with '#'
// are skipped; the first data line is numRules; each rule line is
// "LHS[\tRHS1[\tRHS2]]"; labels are numbered 1,2,... in order of first
// appearance; a missing RHS is 0.
// Graph (getGraphInfo/readEdges, src/main.cpp:106-139, 177-221): first data
// line "numEdges\tnumVars", then numEdges lines "src\tdst\tlabel".
// Differences, all on inputs where the reference has undefined behaviour:
// unknown labels and ids >= numVars are errors instead of silent corruption,
// edges need not be sorted by src, and a trailing '\r' is ignored.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "grg.h"

namespace {

struct LineReader {
    FILE *f = nullptr;
    char *buf = nullptr;
    size_t cap = 0;
    explicit LineReader(const char *path) { f = fopen(path, "r"); }
    ~LineReader()
    {
        if (f) fclose(f);
        free(buf);
    }
    // next line not starting with '#' (skipComments, src/main.cpp:60-67)
    bool next(std::string &out)
    {
        for (;;) {
            ssize_t n = getline(&buf, &cap, f);
            if (n < 0) return false;
            while (n > 0 && (buf[n - 1] == '\n' || buf[n - 1] == '\r')) buf[--n] = 0;
            if (buf[0] == '#') continue;
            out.assign(buf, (size_t)n);
            return true;
        }
    }
};

int find_label(const char *names, int n, const std::string &s)
{
    for (int i = 0; i < n; i++)
        if (strncmp(names + (size_t)i * GRG_NAME_LEN, s.c_str(), GRG_NAME_LEN) == 0) return i + 1;
    return 0;
}

}  // namespace

extern "C" {

int grg_parse_grammar(const char *path, int *num_rules, int *rules, int *num_labels, char *names)
{
    if (!path || !num_rules || !rules || !num_labels || !names) return GRG_E_ARG;
    LineReader in(path);
    if (!in.f) return GRG_E_IO;
    std::string line;
    if (!in.next(line)) return GRG_E_IO;
    int nr = atoi(line.c_str());
    if (nr < 0 || nr > GRG_MAX_RULES) return GRG_E_RANGE;
    memset(rules, 0, sizeof(int) * 3 * GRG_MAX_RULES);
    memset(names, 0, (size_t)GRG_MAX_LABELS * GRG_NAME_LEN);
    int nl = 0;
    for (int r = 0; r < nr; r++) {
        if (!in.next(line)) return GRG_E_IO;
        size_t pos = 0;
        int j = 0;
        while (j < 3) {
            size_t tab = line.find('\t', pos);
            std::string item = line.substr(pos, tab == std::string::npos ? std::string::npos : tab - pos);
            if (item.empty() && tab == std::string::npos) break;   // end of line
            int id = find_label(names, nl, item);
            if (!id) {
                if (nl >= GRG_MAX_LABELS || item.size() >= GRG_NAME_LEN) return GRG_E_RANGE;
                memcpy(names + (size_t)nl * GRG_NAME_LEN, item.c_str(), item.size());
                id = ++nl;
            }
            rules[3 * r + j++] = id;
            if (tab == std::string::npos) break;
            pos = tab + 1;
        }
        if (rules[3 * r] == 0) return GRG_E_IO;
    }
    *num_rules = nr;
    *num_labels = nl;
    return GRG_OK;
}

int grg_parse_graph_header(const char *path, uint64_t *num_edges, uint32_t *num_vars)
{
    if (!path || !num_edges || !num_vars) return GRG_E_ARG;
    LineReader in(path);
    if (!in.f) return GRG_E_IO;
    std::string line;
    if (!in.next(line)) return GRG_E_IO;
    char *end = nullptr;
    *num_edges = strtoull(line.c_str(), &end, 10);
    size_t tab = line.find('\t');
    if (tab == std::string::npos) return GRG_E_IO;
    unsigned long long v = strtoull(line.c_str() + tab + 1, nullptr, 10);
    if (v > 0xFFFFFFFFull) return GRG_E_RANGE;
    *num_vars = (uint32_t)v;
    return GRG_OK;
}

int grg_parse_graph(const char *path, int num_labels, const char *names, uint64_t num_edges, uint32_t num_vars,
                    uint32_t *src, uint32_t *dst, uint8_t *label)
{
    if (!path || !names || (num_edges && (!src || !dst || !label))) return GRG_E_ARG;
    LineReader in(path);
    if (!in.f) return GRG_E_IO;
    std::string line;
    if (!in.next(line)) return GRG_E_IO;
    for (uint64_t e = 0; e < num_edges; e++) {
        if (!in.next(line)) return GRG_E_IO;
        const char *p = line.c_str();
        const char *t1 = strchr(p, '\t');
        if (!t1) return GRG_E_IO;
        const char *t2 = strchr(t1 + 1, '\t');
        if (!t2) return GRG_E_IO;
        const char *t3 = strchr(t2 + 1, '\t');
        std::string lab = t3 ? std::string(t2 + 1, t3) : std::string(t2 + 1);
        unsigned long long s = strtoull(p, nullptr, 10), d = strtoull(t1 + 1, nullptr, 10);
        if (s >= num_vars || d >= num_vars) return GRG_E_RANGE;
        int id = find_label(names, num_labels, lab);
        if (!id) return GRG_E_LABEL;
        src[e] = (uint32_t)s;
        dst[e] = (uint32_t)d;
        label[e] = (uint8_t)id;
    }
    return GRG_OK;
}

}  // extern "C"
