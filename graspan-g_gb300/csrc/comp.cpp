// comp.cpp -- drop-in `comp` entry point (the reference's src/main.cpp:860-921).
//
//   comp <grammar_file> <graph_file> <filter_flag> [--heap-gb G] [--device D]
//        [--partitions P] [--checkpoint FILE [--checkpoint-every N]] [--resume FILE]
//        [--out FILE]
//
// --partitions P closes the graph out of core over P vertex-range partitions
// (the reference always partitions, src/main.cpp:141-175); --checkpoint saves
// the partition set to FILE after every N device runs (default 1) and at the
// end; --resume continues from such a file (the graph file is then not read,
// the grammar must be the same). --out writes the closure as the reference's
// compressed edge stream (5 bytes per edge, storeElements_c,
// src/main.cpp:541-596) to FILE and the edges per source vertex (uint32) to
// FILE.degree; out of core, partition by partition.
//
// The reference reads the grammar from argv[1] and the graph from argv[2]
// (src/main.cpp:869-871) while its README documents the opposite order; both
// orders are accepted here: the grammar's first data line holds one integer,
// the graph's holds two. The filter flag is required (the reference crashes
// without it). The reference's stdout lines are kept verbatim and per-label
// counts are added.
#include <algorithm>
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
        fprintf(stderr,
                "usage: %s <grammar_file> <graph_file> <filter_flag> [--heap-gb G] [--device D] [--partitions P]\n"
                "          [--checkpoint FILE [--checkpoint-every N]] [--resume FILE] [--out FILE]\n",
                argv[0]);
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
    uint32_t parts = 0, ckpt_every = 1;
    const char *ckpt = nullptr, *resume = nullptr, *out = nullptr;
    for (int i = 4; i < argc; i++) {
        if (!strcmp(argv[i], "--heap-gb") && i + 1 < argc) heap_gb = atof(argv[++i]);
        else if (!strcmp(argv[i], "--device") && i + 1 < argc) device = atoi(argv[++i]);
        else if (!strcmp(argv[i], "--partitions") && i + 1 < argc) parts = (uint32_t)atoi(argv[++i]);
        else if (!strcmp(argv[i], "--checkpoint") && i + 1 < argc) ckpt = argv[++i];
        else if (!strcmp(argv[i], "--checkpoint-every") && i + 1 < argc) ckpt_every = (uint32_t)atoi(argv[++i]);
        else if (!strcmp(argv[i], "--resume") && i + 1 < argc) resume = argv[++i];
        else if (!strcmp(argv[i], "--out") && i + 1 < argc) out = argv[++i];
        else {
            fprintf(stderr, "unknown option %s\n", argv[i]);
            return 2;
        }
    }
    if ((ckpt || resume) && !parts) parts = 2;
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

    st = grg_allocate_pool(ctx, (uint64_t)(heap_gb * 1073741824.0));
    if (st) return die("grg_allocate_pool", st, ctx);
    uint64_t num_edges = 0;
    uint32_t num_vars = 0;
    std::vector<uint32_t> src, dst;
    std::vector<uint8_t> lab;
    if (!resume) {
        st = grg_parse_graph_header(graph, &num_edges, &num_vars);
        if (st) return die("graph header", st, ctx);
        printf("NUM VERTICES: %u\n", num_vars);
        printf("INITIAL NUM EDGES: %llu\n", (unsigned long long)num_edges);
        src.resize(num_edges);
        dst.resize(num_edges);
        lab.resize(num_edges);
        st = grg_parse_graph(graph, num_labels, names.data(), num_edges, num_vars, src.data(), dst.data(), lab.data());
        if (st) return die("graph", st, ctx);
    }
    std::vector<uint64_t> counts(num_labels);
    uint64_t total = 0, steps = 0;
    uint32_t final_parts = 1;
    double fix_ms = 0;
    std::vector<uint8_t> stream;
    std::vector<uint32_t> degree;
    auto take_stream = [&](int s2, uint64_t n, std::vector<uint8_t> &bytes, std::vector<uint32_t> &deg,
                           auto call) -> int {
        if (s2 != GRG_OK && s2 != GRG_E_RANGE) return s2;
        bytes.resize(n * 5);
        return call(n, bytes.data(), deg.data());
    };
    if (!parts) {
        st = grg_load_edges(ctx, num_vars, num_edges, src.data(), dst.data(), lab.data(), 0);
        if (st) return die("grg_load_edges", st, ctx);
        printf("INITIAL NUM PARTITIONS: 1\n");
        grg_stats stats;
        st = grg_closure(ctx, (uint32_t)filter, &stats);
        if (st) return die("grg_closure", st, ctx);
        st = grg_label_counts(ctx, counts.data());
        if (st) return die("grg_label_counts", st, ctx);
        total = stats.total_edges;
        steps = stats.rounds;
        fix_ms = stats.closure_ms;
        if (out) {
            uint64_t n = 0;
            degree.resize(num_vars);
            st = take_stream(grg_export_csr5(ctx, 0, num_vars, 0, nullptr, nullptr, &n), n, stream, degree,
                             [&](uint64_t m, uint8_t *b, uint32_t *d) {
                                 return grg_export_csr5(ctx, 0, num_vars, m, b, d, &m);
                             });
            if (st) return die("grg_export_csr5", st, ctx);
        }
    } else {
        grg_part *part = nullptr;
        if (resume) {
            st = grg_part_restore(&part, ctx, resume);
            if (st) return die("grg_part_restore", st, ctx);
        } else {
            st = grg_part_create(&part, ctx, num_vars, parts);
            if (!st) st = grg_part_load_edges(part, num_edges, src.data(), dst.data(), lab.data());
            if (st) return die("partitioned load", st, ctx);
        }
        uint32_t np = 0;
        grg_part_bounds(part, 0, nullptr, &np);
        printf("INITIAL NUM PARTITIONS: %u\n", np);
        if (ckpt) grg_part_set_checkpoint(part, ckpt, ckpt_every);
        grg_part_stats ps{};
        uint64_t h = 0;
        st = grg_part_label_counts(part, counts.data(), &h);      // a restored closed set
        if (st == GRG_E_STATE) {
            st = grg_part_run(part, (uint32_t)filter, &ps);
            if (st) return die("grg_part_run", st, ctx);
            st = grg_part_label_counts(part, counts.data(), &h);
        }
        if (st) return die("grg_part_label_counts", st, ctx);
        for (uint64_t c : counts) total += c;
        steps = ps.supersteps;
        fix_ms = ps.ms;
        grg_part_bounds(part, 0, nullptr, &final_parts);
        if (out) {
            std::vector<uint32_t> b(final_parts + 1);
            grg_part_bounds(part, (uint32_t)b.size(), b.data(), &final_parts);
            num_vars = b[final_parts];
            degree.resize(num_vars);
            for (uint32_t k = 0; k < final_parts && !st; k++) {
                uint64_t n = 0;
                std::vector<uint8_t> piece;
                std::vector<uint32_t> dk(b[k + 1] - b[k]);
                st = take_stream(grg_part_export_csr5(part, k, 0, nullptr, nullptr, &n), n, piece, dk,
                                 [&](uint64_t m, uint8_t *bb, uint32_t *d) {
                                     return grg_part_export_csr5(part, k, m, bb, d, &m);
                                 });
                stream.insert(stream.end(), piece.begin(), piece.end());
                std::copy(dk.begin(), dk.end(), degree.begin() + b[k]);
            }
            if (st) return die("grg_part_export_csr5", st, ctx);
        }
        grg_part_destroy(part);
    }
    if (out) {
        const std::string dpath = std::string(out) + ".degree";
        FILE *f = fopen(out, "wb");
        FILE *g = fopen(dpath.c_str(), "wb");
        bool ok = f && g && fwrite(stream.data(), 1, stream.size(), f) == stream.size() &&
                  fwrite(degree.data(), 4, degree.size(), g) == degree.size();
        if (f && fclose(f) != 0) ok = false;
        if (g && fclose(g) != 0) ok = false;
        if (!ok) return die("writing the edge stream", GRG_E_IO, ctx);
    }
    auto t1 = std::chrono::steady_clock::now();
    double secs = std::chrono::duration<double>(t1 - t0).count();
    printf("===== SPAGPU FINISHED =====\n");
    printf("NUM SUPERSTEPS: %llu\n", (unsigned long long)steps);
    printf("FINAL NUM PARTITIONS: %u\n", final_parts);
    printf("FINAL NUM EDGES: %llu\n", (unsigned long long)total);
    for (int l = 0; l < num_labels; l++)
        printf("LABEL %s EDGES: %llu\n", names.data() + (size_t)l * GRG_NAME_LEN, (unsigned long long)counts[l]);
    printf("TIME TO FIXPOINT: %.3f ms\n", fix_ms);
    printf("CLOSURE EDGES/S: %.4g\n", fix_ms > 0 ? total / (fix_ms * 1e-3) : 0.0);
    printf("TOTAL SPAGPU TIME: %.3f s\n", secs);
    grg_destroy(ctx);
    return 0;
}
