// comp.cpp -- drop-in `comp` entry point (the reference's src/main.cpp:860-921).
//
//   comp <grammar_file> <graph_file> <filter_flag> [--heap-gb G] [--device D] [--quiet]
//
// The reference reads the grammar from argv[1] and the graph from argv[2]
// (src/main.cpp:869-871) while its README documents the opposite order; both
// orders are accepted here: the grammar's first data line holds one integer,
// the graph's holds two. The filter flag is required (the reference crashes
// without it). The reference's stdout lines are kept verbatim and per-label
// counts are added.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "grg.h"

static bool first_data_line_has_tab(const char *path, bool *ok)
{
    FILE *f = fopen(path, "r");
    *ok = f != nullptr;
    if (!f) return false;
    char buf[4096];
    bool tab = false;
    while (fgets(buf, sizeof buf, f)) {
        if (buf[0] == '#') continue;
        tab = strchr(buf, '\t') != nullptr;
        break;
    }
    fclose(f);
    return tab;
}

static int die(const char *what, int st, grg_ctx *ctx = nullptr)
{
    fprintf(stderr, "%s failed: %s %s\n", what, grg_error_string(st), ctx ? grg_last_error(ctx) : "");
    if (ctx) grg_destroy(ctx);
    return 1;
}

int main(int argc, char **argv)
{
    if (argc < 4) {
        fprintf(stderr, "usage: %s <grammar_file> <graph_file> <filter_flag> [--heap-gb G] [--device D]\n", argv[0]);
        return 2;
    }
    const char *gram = argv[1], *graph = argv[2];
    bool ok1, ok2;
    bool tab1 = first_data_line_has_tab(argv[1], &ok1), tab2 = first_data_line_has_tab(argv[2], &ok2);
    if (!ok1 || !ok2) {
        fprintf(stderr, "cannot open input files\n");
        return 2;
    }
    if (tab1 && !tab2) { gram = argv[2]; graph = argv[1]; }
    const int filter = atoi(argv[3]);
    double heap_gb = 0;
    int device = -1;
    for (int i = 4; i < argc; i++) {
        if (!strcmp(argv[i], "--heap-gb") && i + 1 < argc) heap_gb = atof(argv[++i]);
        else if (!strcmp(argv[i], "--device") && i + 1 < argc) device = atoi(argv[++i]);
    }
    auto t0 = std::chrono::steady_clock::now();
    printf("===== PREPROCESSING INFO =====\n");
    grg_ctx *ctx = nullptr;
    int st = grg_create(&ctx, device);
    if (st) return die("grg_create", st);
    printf("SELECTED DEVICE: %d\n", grg_device(ctx));

    int num_rules = 0, num_labels = 0;
    std::vector<int> rules(3 * GRG_MAX_RULES);
    std::vector<char> names((size_t)GRG_MAX_LABELS * GRG_NAME_LEN);
    st = grg_parse_grammar(gram, &num_rules, rules.data(), &num_labels, names.data());
    if (st) return die("grammar", st, ctx);
    printf("NUM RULES: %d\n", num_rules);
    printf("NUM LABELS: %d\n", num_labels);
    st = grg_transfer_rules(ctx, num_rules, rules.data(), num_labels);
    if (st) return die("grg_transfer_rules", st, ctx);

    uint64_t num_edges = 0;
    uint32_t num_vars = 0;
    st = grg_parse_graph_header(graph, &num_edges, &num_vars);
    if (st) return die("graph header", st, ctx);
    printf("NUM VERTICES: %u\n", num_vars);
    printf("INITIAL NUM EDGES: %llu\n", (unsigned long long)num_edges);
    std::vector<uint32_t> src(num_edges), dst(num_edges);
    std::vector<uint8_t> lab(num_edges);
    st = grg_parse_graph(graph, num_labels, names.data(), num_edges, num_vars, src.data(), dst.data(), lab.data());
    if (st) return die("graph", st, ctx);

    st = grg_allocate_pool(ctx, (uint64_t)(heap_gb * 1073741824.0));
    if (st) return die("grg_allocate_pool", st, ctx);
    st = grg_load_edges(ctx, num_vars, num_edges, src.data(), dst.data(), lab.data(), 0);
    if (st) return die("grg_load_edges", st, ctx);
    printf("INITIAL NUM PARTITIONS: 1\n");
    grg_stats stats;
    st = grg_closure(ctx, (uint32_t)filter, &stats);
    if (st) return die("grg_closure", st, ctx);
    std::vector<uint64_t> counts(num_labels);
    st = grg_label_counts(ctx, counts.data());
    if (st) return die("grg_label_counts", st, ctx);
    auto t1 = std::chrono::steady_clock::now();
    double secs = std::chrono::duration<double>(t1 - t0).count();
    printf("===== SPAGPU FINISHED =====\n");
    printf("NUM SUPERSTEPS: %llu\n", (unsigned long long)stats.rounds);
    printf("FINAL NUM PARTITIONS: 1\n");
    printf("FINAL NUM EDGES: %llu\n", (unsigned long long)stats.total_edges);
    for (int l = 0; l < num_labels; l++)
        printf("LABEL %s EDGES: %llu\n", names.data() + (size_t)l * GRG_NAME_LEN, (unsigned long long)counts[l]);
    printf("TIME TO FIXPOINT: %.3f ms\n", stats.closure_ms);
    printf("CLOSURE EDGES/S: %.4g\n", stats.closure_ms > 0 ? stats.total_edges / (stats.closure_ms * 1e-3) : 0.0);
    printf("TOTAL SPAGPU TIME: %.3f s\n", secs);
    grg_destroy(ctx);
    return 0;
}
