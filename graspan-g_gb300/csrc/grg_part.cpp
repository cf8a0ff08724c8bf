// grg_part.cpp -- out-of-core closure over vertex-range partitions.
//
// The reference always runs partitioned (src/main.cpp:141-175: at least two
// vertex-range partitions), spilling partition pools to files and computing
// supersteps over all partition pairs until no pair has new edges
// (precomputation / run_computation, src/main.cpp:764-858), splitting a
// partition that overflows the GPU heap (src/main.cpp:633-762). Here the
// in-core closure (grg_closure) is the normal path -- the GPU's memory holds
// graphs the reference had to partition -- and this scheduler takes over when
// a graph's closure does not fit the context's pool limit. It is host code on
// the C ABI: partition images live in host memory (the spill files), the
// device closes one partition or one pair at a time.
//
// Two schedules:
//   stream  every binary rule's second symbol is never derived, so a row's
//           closure needs only its own rows and static rows: the static
//           labels of the whole graph stay in the load, each partition's rows
//           are closed once, in turn (no supersteps).
//   pairs   otherwise: supersteps over pairs (a, b). A join A(i,j) <- B(i,k)
//           C(k,j) involves rows i and k only, so a run that holds a closes
//           a's own rows, and a pair (a, b) adds something only if a B-edge
//           crosses between them (each partition's reach set, computed on the
//           device after every run; the reference's data-dependence manager,
//           src/ddm.cpp:9-132, never called there). Every element carries a
//           stamp (the run that last gave it bits); a run marks as round-1
//           deltas exactly the elements stamped after the last run that held
//           the same partitions, and is skipped when none is newer. A
//           superstep without a run is the fixpoint.
// A run that does not fit (GRG_E_NOMEM) splits the larger partition at its
// median element and is repeated.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <map>
#include <utility>
#include <vector>

#include "grg.h"

namespace {

constexpr uint32_t KEY_SHIFT = 25;

// Growable array in page-locked host memory (pageable if pinning fails): images
// live here, so device<->host copies of them need no staging copy.
struct HostVec {
    uint32_t *p = nullptr;
    uint64_t n = 0, cap = 0;
    bool pinned = false;
    HostVec() = default;
    HostVec(const HostVec &) = delete;
    HostVec &operator=(const HostVec &) = delete;
    HostVec(HostVec &&o) noexcept : p(o.p), n(o.n), cap(o.cap), pinned(o.pinned) { o.p = nullptr; o.n = o.cap = 0; }
    HostVec &operator=(HostVec &&o) noexcept
    {
        if (this != &o) {
            release();
            p = o.p; n = o.n; cap = o.cap; pinned = o.pinned;
            o.p = nullptr; o.n = o.cap = 0;
        }
        return *this;
    }
    ~HostVec() { release(); }
    void release()
    {
        if (p) {
            if (pinned) cudaFreeHost(p); else free(p);
        }
        p = nullptr;
        n = cap = 0;
    }
    bool reserve(uint64_t c)       // keeps the contents
    {
        if (c <= cap) return true;
        const uint64_t nc = std::max<uint64_t>(c + c / 4, 256);
        uint32_t *q = nullptr;
        bool pin = true;
        if (cudaHostAlloc((void **)&q, nc * 4, cudaHostAllocDefault) != cudaSuccess) {
            cudaGetLastError();
            pin = false;
            q = (uint32_t *)malloc(nc * 4);
            if (!q) return false;
        }
        if (n) memcpy(q, p, n * 4);
        const uint64_t keep = n;
        release();
        p = q; n = keep; cap = nc; pinned = pin;
        return true;
    }
    bool resize(uint64_t m)
    {
        if (!reserve(m)) return false;
        n = m;
        return true;
    }
    bool append(const uint32_t *src, uint64_t m)
    {
        if (!reserve(n + m)) return false;
        memcpy(p + n, src, m * 4);
        n += m;
        return true;
    }
    uint32_t *data() { return p; }
    const uint32_t *data() const { return p; }
    uint64_t size() const { return n; }
    uint32_t &operator[](uint64_t i) { return p[i]; }
    uint32_t operator[](uint64_t i) const { return p[i]; }
    uint32_t *begin() { return p; }
    uint32_t *end() { return p + n; }
    const uint32_t *begin() const { return p; }
    const uint32_t *end() const { return p + n; }
};

struct Image {
    uint32_t id = 0;                 // unique per partition (splits make new ids)
    uint32_t lo = 0, hi = 0;         // source vertices [lo, hi)
    HostVec rec;                     // 8 words per element
    HostVec st;                      // stamp per element
    uint32_t max_stamp = 0;
    uint32_t last_run = 0;           // last run that held this partition
    bool counted = false;            // counts/hash are those of the current image
    std::vector<uint32_t> reach;     // ids of partitions this one's B-edges may end in (sorted)
    std::vector<uint64_t> counts;
    uint64_t hash = 0;

    uint64_t size() const { return st.size(); }
    void refresh()
    {
        max_stamp = 0;
        for (uint32_t s : st) max_stamp = std::max(max_stamp, s);
    }
};

// Pinned staging buffer for records and stamps.
struct Pinned {
    uint32_t *rec = nullptr;
    uint32_t *st = nullptr;
    uint64_t cap = 0;
    ~Pinned() { release(); }
    void release()
    {
        if (rec) cudaFreeHost(rec);
        if (st) cudaFreeHost(st);
        rec = st = nullptr;
        cap = 0;
    }
    int ensure(uint64_t n)
    {
        if (n <= cap) return GRG_OK;
        release();
        const uint64_t c = std::max<uint64_t>(n + n / 4, 1024);
        if (cudaHostAlloc((void **)&rec, c * 32, cudaHostAllocDefault) != cudaSuccess ||
            cudaHostAlloc((void **)&st, c * 4, cudaHostAllocDefault) != cudaSuccess) {
            cudaGetLastError();
            release();
            return GRG_E_NOMEM;
        }
        cap = c;
        return GRG_OK;
    }
};

}  // namespace

struct grg_part {
    grg_ctx *ctx = nullptr;
    uint32_t V = 0;
    int R = 0, L = 0;
    int rules[3 * GRG_MAX_RULES] = {0};
    std::vector<Image> parts;                                  // ordered by lo
    std::map<std::pair<uint32_t, uint32_t>, uint32_t> seen;    // (id, id) -> run after which the pair is closed
    uint32_t next_id = 1;
    uint32_t run_id = 1;                                       // stamps of loaded edges are 1
    bool loaded = false;
    bool closed = false;
    Pinned in;                       // run inputs assembled for the device
    grg_part_stats S{};
    uint64_t bmask = 0;              // labels that are a binary rule's first symbol
};

namespace {

std::pair<uint32_t, uint32_t> pkey(uint32_t a, uint32_t b) { return a < b ? std::make_pair(a, b) : std::make_pair(b, a); }

// Adds the wall time of its scope to a stats field.
struct Timer {
    double &acc;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    explicit Timer(double &a) : acc(a) {}
    ~Timer() { acc += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count(); }
};

// Labels any rule can add edges to under the filter (epsilon rules count: they
// add edges at the load), as the engine classifies them.
void derivable_labels(const grg_part *p, uint32_t filter, bool *der)
{
    for (int l = 0; l <= GRG_MAX_LABELS; l++) der[l] = false;
    for (int q = 0; q < p->R; q++) {
        const int *r = &p->rules[3 * q];
        const bool unary = r[1] && !r[2];
        if (!(filter && unary)) der[r[0]] = true;
    }
}

// Export rows [lo, hi) of the loaded graph into img (records + device stamps).
int export_image(grg_part *p, Image &img)
{
    Timer tm(p->S.export_ms);
    // straight into the image's own (pinned) arrays; regrown once when they are too small
    uint64_t cap = std::min(img.rec.cap / 8, img.st.cap), n2 = 0;
    img.rec.n = img.st.n = 0;
    int st = grg_export_elements(p->ctx, img.lo, img.hi, cap, img.rec.data(), img.st.data(), &n2);
    if (st == GRG_E_RANGE && n2 > cap) {
        if (!img.rec.reserve(n2 * 8) || !img.st.reserve(n2)) return GRG_E_NOMEM;
        cap = std::min(img.rec.cap / 8, img.st.cap);
        st = grg_export_elements(p->ctx, img.lo, img.hi, cap, img.rec.data(), img.st.data(), &n2);
    }
    if (st) return st;
    img.rec.n = n2 * 8;
    img.st.n = n2;
    p->S.d2h_bytes += n2 * 36;
    return GRG_OK;
}

int count_image(grg_part *p, Image &img)
{
    Timer tm(p->S.count_ms);
    img.counts.assign(p->L, 0);
    int st = grg_range_counts(p->ctx, img.lo, img.hi, img.counts.data(), &img.hash);
    if (st) return st;
    img.counted = true;
    return GRG_OK;
}

// Reach set of parts[i] over the current partition bounds (graph loaded on the device).
int reach_image(grg_part *p, size_t i)
{
    Timer tm(p->S.count_ms);
    const size_t m = p->parts.size();
    std::vector<uint32_t> bounds(m + 1);
    for (size_t q = 0; q < m; q++) bounds[q] = p->parts[q].lo;
    bounds[m] = p->parts[m - 1].hi;
    std::vector<uint8_t> r(m);
    Image &x = p->parts[i];
    int st = grg_range_reach(p->ctx, x.lo, x.hi, p->bmask, (uint32_t)m, bounds.data(), r.data());
    if (st) return st;
    x.reach.clear();
    for (size_t q = 0; q < m; q++)
        if (r[q]) x.reach.push_back(p->parts[q].id);
    std::sort(x.reach.begin(), x.reach.end());
    return GRG_OK;
}

// Split parts[i] at its median element (by source row); false when it is one row.
bool split(grg_part *p, size_t i)
{
    Image &x = p->parts[i];
    if (x.hi - x.lo < 2) return false;
    std::vector<uint64_t> per(x.hi - x.lo, 0);
    for (uint64_t e = 0; e < x.size(); e++) per[x.rec[8 * e + 7] - x.lo]++;
    uint64_t half = x.size() / 2, acc = 0;
    uint32_t mid = x.lo + (x.hi - x.lo) / 2;
    if (x.size()) {
        for (uint32_t v = x.lo; v < x.hi; v++) {
            acc += per[v - x.lo];
            if (acc >= half) { mid = v + 1; break; }
        }
        mid = std::min(std::max(mid, x.lo + 1), x.hi - 1);
    }
    Image a, b;
    a.id = p->next_id++;
    b.id = p->next_id++;
    a.lo = x.lo; a.hi = mid;
    b.lo = mid; b.hi = x.hi;
    uint64_t na = 0;
    for (uint64_t e = 0; e < x.size(); e++) na += x.rec[8 * e + 7] < mid;
    a.rec.reserve(na * 8);
    a.st.reserve(na);
    b.rec.reserve((x.size() - na) * 8);
    b.st.reserve(x.size() - na);
    for (uint64_t e = 0; e < x.size(); e++) {
        Image &t = x.rec[8 * e + 7] < mid ? a : b;
        t.rec.append(x.rec.data() + 8 * e, 8);
        t.st.append(&x.st[e], 1);
    }
    a.refresh();
    b.refresh();
    a.last_run = b.last_run = x.last_run;
    // the halves have seen what the whole had seen, with every other partition and with each other
    std::map<std::pair<uint32_t, uint32_t>, uint32_t> add;
    for (const auto &kv : p->seen) {
        uint32_t other = kv.first.first == x.id ? kv.first.second : kv.first.second == x.id ? kv.first.first : 0;
        if (!other) continue;
        if (other == x.id) continue;
        add[pkey(a.id, other)] = kv.second;
        add[pkey(b.id, other)] = kv.second;
    }
    for (const auto &kv : add) p->seen[kv.first] = kv.second;
    p->seen[pkey(a.id, b.id)] = x.last_run;
    p->seen[pkey(a.id, a.id)] = p->seen.count(pkey(x.id, x.id)) ? p->seen[pkey(x.id, x.id)] : 0;
    p->seen[pkey(b.id, b.id)] = p->seen[pkey(a.id, a.id)];
    // reach: what reached x (or x itself) may now reach either half
    auto widen = [&](std::vector<uint32_t> &r) {
        if (std::binary_search(r.begin(), r.end(), x.id)) {
            r.push_back(a.id);
            r.push_back(b.id);
            std::sort(r.begin(), r.end());
        }
    };
    a.reach = x.reach;
    widen(a.reach);
    b.reach = a.reach;
    for (Image &y : p->parts)
        if (y.id != x.id) widen(y.reach);
    p->parts[i] = std::move(a);
    p->parts.insert(p->parts.begin() + i + 1, std::move(b));
    p->S.splits++;
    return true;
}

// Load one partition's image (nothing marked) and count its rows.
int recount(grg_part *p, Image &x)
{
    int st = p->in.ensure(x.size());
    if (st) return st;
    memcpy(p->in.rec, x.rec.data(), x.size() * 32);
    memcpy(p->in.st, x.st.data(), x.size() * 4);
    p->S.h2d_bytes += x.size() * 36;
    if ((st = grg_load_elements(p->ctx, p->V, x.size(), p->in.rec, p->in.st, ~0u, 0))) return st;
    return count_image(p, x);
}

// One device run over the given partitions; the load holds `extra` first (static
// records of the stream schedule, stamps as given) then the partitions' images.
// Partitions' records are marked when their stamp is above mark_after.
int run_once(grg_part *p, uint32_t filter, const std::vector<size_t> &idx, const Image *extra,
             const bool *keep_label, uint32_t mark_after, uint32_t run_stamp)
{
    uint64_t n = extra ? extra->size() : 0;
    int st;
    {
        Timer tm(p->S.stage_ms);
        for (size_t i : idx) {
            if (!keep_label) {
                n += p->parts[i].size();
                continue;
            }
            for (uint64_t e = 0; e < p->parts[i].size(); e++)
                if (keep_label[p->parts[i].rec[8 * e + 6] >> KEY_SHIFT]) n++;
        }
        if ((st = p->in.ensure(n))) return st;
        uint64_t k = 0;
        if (extra && extra->size()) {
            memcpy(p->in.rec, extra->rec.data(), extra->size() * 32);
            memcpy(p->in.st, extra->st.data(), extra->size() * 4);
            k = extra->size();
        }
        for (size_t i : idx) {
            const Image &x = p->parts[i];
            if (!keep_label) {               // whole images: one copy each
                memcpy(p->in.rec + 8 * k, x.rec.data(), x.size() * 32);
                memcpy(p->in.st + k, x.st.data(), x.size() * 4);
                k += x.size();
                continue;
            }
            for (uint64_t e = 0; e < x.size(); e++) {
                if (!keep_label[x.rec[8 * e + 6] >> KEY_SHIFT]) continue;
                memcpy(p->in.rec + 8 * k, x.rec.data() + 8 * e, 32);
                p->in.st[k] = x.st[e];
                k++;
            }
        }
    }
    p->S.h2d_bytes += n * 36;
    {
        Timer tm(p->S.load_ms);
        if ((st = grg_load_elements(p->ctx, p->V, n, p->in.rec, p->in.st, mark_after, 0))) return st;
    }
    grg_stats cs;
    {
        Timer tm(p->S.closure_ms);
        if ((st = grg_closure_ex(p->ctx, filter, run_stamp, &cs))) return st;
    }
    p->S.runs++;
    p->S.rounds += cs.rounds;
    return GRG_OK;
}

int run_stream(grg_part *p, uint32_t filter, const bool *der)
{
    bool derived[GRG_MAX_LABELS + 1];
    for (int l = 0; l <= GRG_MAX_LABELS; l++) derived[l] = der[l];
    // static records of every partition (never inserted into, so built once; again after
    // a split), in partition order; seg[j] = where partition j's begin. A run marks only
    // its own partition's segment.
    Image stat;
    std::vector<uint64_t> seg;
    bool stale = true;
    for (size_t i = 0; i < p->parts.size();) {
        if (stale) {
            uint64_t ns = 0;
            for (const Image &x : p->parts)
                for (uint64_t e = 0; e < x.size(); e++) ns += !derived[x.rec[8 * e + 6] >> KEY_SHIFT];
            stat.rec.n = stat.st.n = 0;
            if (!stat.rec.reserve(ns * 8) || !stat.st.reserve(ns)) return GRG_E_NOMEM;
            seg.assign(1, 0);
            const uint32_t zero = 0;
            for (const Image &x : p->parts) {
                for (uint64_t e = 0; e < x.size(); e++) {
                    if (derived[x.rec[8 * e + 6] >> KEY_SHIFT]) continue;
                    stat.rec.append(x.rec.data() + 8 * e, 8);
                    stat.st.append(&zero, 1);
                }
                seg.push_back(stat.size());
            }
            stale = false;
        }
        for (uint64_t e = seg[i]; e < seg[i + 1]; e++) stat.st[e] = 1;
        Image &x = p->parts[i];
        for (uint32_t &s : x.st) s = 1;
        const int st = run_once(p, filter, {i}, &stat, derived, 0, 0);
        for (uint64_t e = seg[i]; e < seg[i + 1]; e++) stat.st[e] = 0;
        if (st == GRG_E_NOMEM) {
            if (!split(p, i)) return GRG_E_NOMEM;
            stale = true;
            continue;
        }
        if (st) return st;
        int s2 = export_image(p, p->parts[i]);
        if (s2) return s2;
        if ((s2 = count_image(p, p->parts[i]))) return s2;
        i++;
    }
    return GRG_OK;
}

uint32_t seen_of(grg_part *p, uint32_t a, uint32_t b)
{
    auto it = p->seen.find(pkey(a, b));
    return it == p->seen.end() ? 0 : it->second;
}

bool reaches(const Image &a, const Image &b)
{
    return std::binary_search(a.reach.begin(), a.reach.end(), b.id) ||
           std::binary_search(b.reach.begin(), b.reach.end(), a.id);
}

int run_pairs(grg_part *p, uint32_t filter)
{
    for (;;) {
        bool ran = false, restart = false;
        // pairs whose B-edges cross, then partitions no run has closed since their last change
        std::vector<std::pair<size_t, size_t>> order;
        const size_t m = p->parts.size();
        for (size_t i = 0; i < m; i++)
            for (size_t j = i + 1; j < m; j++) order.emplace_back(i, j);
        for (size_t i = 0; i < m; i++) order.emplace_back(i, i);
        for (const auto &ij : order) {
            const size_t i = ij.first, j = ij.second;
            Image &a = p->parts[i], &b = p->parts[j];
            const uint32_t t = seen_of(p, a.id, b.id);
            bool need;
            if (i == j)
                need = a.max_stamp > t;
            else
                need = reaches(a, b) && (a.max_stamp > t || b.max_stamp > t);
            if (!need) {
                p->S.skipped++;
                continue;
            }
            const uint32_t r = ++p->run_id;
            std::vector<size_t> idx = {i};
            if (j != i) idx.push_back(j);
            const int st = run_once(p, filter, idx, nullptr, nullptr, t, r);
            if (st == GRG_E_NOMEM) {
                const size_t big = (j != i && b.size() > a.size()) ? j : i;
                if (!split(p, big)) return GRG_E_NOMEM;
                restart = true;
                break;
            }
            if (st) return st;
            for (size_t q : idx) {
                int s2 = export_image(p, p->parts[q]);
                if (s2) return s2;
                if ((s2 = count_image(p, p->parts[q]))) return s2;
                if ((s2 = reach_image(p, q))) return s2;
                Image &x = p->parts[q];
                x.refresh();
                x.last_run = r;
                p->seen[pkey(x.id, x.id)] = r;   // a run that holds x closes x's own rows
            }
            p->seen[pkey(a.id, b.id)] = r;
            ran = true;
        }
        if (restart) continue;
        p->S.supersteps++;
        if (!ran) return GRG_OK;
    }
}

}  // namespace

extern "C" {

int grg_part_create(grg_part **out, grg_ctx *ctx, uint32_t num_vars, uint32_t num_parts)
{
    if (!out || !ctx || num_parts == 0) return GRG_E_ARG;
    *out = nullptr;
    grg_part *p = new grg_part;
    p->ctx = ctx;
    p->V = num_vars;
    int st = grg_get_rules(ctx, &p->R, p->rules, &p->L);
    if (st) {
        delete p;
        return st;
    }
    for (int q = 0; q < p->R; q++)
        if (p->rules[3 * q + 1] && p->rules[3 * q + 2]) p->bmask |= 1ull << (p->rules[3 * q + 1] - 1);
    const uint32_t m = std::max<uint32_t>(1, std::min<uint32_t>(num_parts, std::max<uint32_t>(num_vars, 1)));
    for (uint32_t i = 0; i < m; i++) {
        Image x;
        x.id = p->next_id++;
        x.lo = (uint32_t)((uint64_t)num_vars * i / m);
        x.hi = (uint32_t)((uint64_t)num_vars * (i + 1) / m);
        p->parts.push_back(std::move(x));
    }
    *out = p;
    return GRG_OK;
}

void grg_part_destroy(grg_part *p) { delete p; }

int grg_part_load_edges(grg_part *p, uint64_t num_edges, const uint32_t *src, const uint32_t *dst,
                        const uint8_t *label)
{
    if (!p || (num_edges && (!src || !dst || !label))) return GRG_E_ARG;
    for (uint64_t e = 0; e < num_edges; e++)
        if (src[e] >= p->V || dst[e] >= p->V) return GRG_E_RANGE;
    // bucket the edges by source partition, then build each image on the device
    struct Bucket { std::vector<uint32_t> s, d; std::vector<uint8_t> l; };
    std::vector<Bucket> bk(p->parts.size());
    std::vector<uint32_t> lo;
    for (const Image &x : p->parts) lo.push_back(x.lo);
    for (uint64_t e = 0; e < num_edges; e++) {
        const size_t i = std::upper_bound(lo.begin(), lo.end(), src[e]) - lo.begin() - 1;
        bk[i].s.push_back(src[e]);
        bk[i].d.push_back(dst[e]);
        bk[i].l.push_back(label[e]);
    }
    for (size_t i = 0; i < p->parts.size();) {
        Image &x = p->parts[i];
        Bucket &b0 = bk[i];
        int st = grg_load_edges(p->ctx, p->V, b0.s.size(), b0.s.data(), b0.d.data(), b0.l.data(), 0);
        if (st == GRG_E_NOMEM) {
            // halve the vertex range (its image does not exist yet)
            if (x.hi - x.lo < 2) return GRG_E_NOMEM;
            Image b;
            b.id = p->next_id++;
            b.lo = x.lo + (x.hi - x.lo) / 2;
            b.hi = x.hi;
            x.hi = b.lo;
            Bucket lo_b, hi_b;
            for (size_t e = 0; e < b0.s.size(); e++) {
                Bucket &t = b0.s[e] < b.lo ? lo_b : hi_b;
                t.s.push_back(b0.s[e]);
                t.d.push_back(b0.d[e]);
                t.l.push_back(b0.l[e]);
            }
            bk[i] = std::move(lo_b);
            bk.insert(bk.begin() + i + 1, std::move(hi_b));
            // partitions already loaded that reach x may reach its upper half
            for (Image &y : p->parts)
                if (std::binary_search(y.reach.begin(), y.reach.end(), x.id)) {
                    y.reach.push_back(b.id);
                    std::sort(y.reach.begin(), y.reach.end());
                }
            p->parts.insert(p->parts.begin() + i + 1, std::move(b));
            p->S.splits++;
            continue;
        }
        if (st) return st;
        p->S.h2d_bytes += b0.s.size() * 9;
        if ((st = export_image(p, p->parts[i]))) return st;
        if ((st = reach_image(p, i))) return st;
        Image &y = p->parts[i];
        for (uint32_t &t : y.st) t = 1;
        y.refresh();
        y.counted = false;
        i++;
    }
    p->loaded = true;
    p->closed = false;
    return GRG_OK;
}

int grg_part_run(grg_part *p, uint32_t filter, grg_part_stats *stats)
{
    if (!p || filter > 1) return GRG_E_ARG;
    if (!p->loaded) return GRG_E_STATE;
    if (p->closed) return GRG_E_STATE;
    const auto t0 = std::chrono::steady_clock::now();
    const uint64_t splits0 = p->S.splits;
    p->S = grg_part_stats{};
    p->S.splits = splits0;
    bool der[GRG_MAX_LABELS + 1];
    derivable_labels(p, filter, der);
    bool coupled = false;
    for (int q = 0; q < p->R; q++) {
        const int *r = &p->rules[3 * q];
        if (r[1] && r[2] && der[r[2]]) coupled = true;
    }
    p->S.schedule = coupled ? 1 : 0;
    int st = coupled ? run_pairs(p, filter) : run_stream(p, filter, der);
    if (st) return st;
    // partitions whose counts predate a split are counted from their images
    for (size_t i = 0; i < p->parts.size(); i++) {
        Image &x = p->parts[i];
        if (x.counted) continue;
        if ((st = recount(p, x))) return st;
    }
    for (const Image &x : p->parts)
        for (int l = 0; l < p->L; l++) p->S.total_edges += x.counts[l];
    p->S.num_parts = (uint32_t)p->parts.size();
    p->S.ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    p->closed = true;
    if (stats) *stats = p->S;
    return GRG_OK;
}

int grg_part_label_counts(grg_part *p, uint64_t *counts, uint64_t *hash)
{
    if (!p || !counts) return GRG_E_ARG;
    if (!p->closed) return GRG_E_STATE;
    uint64_t h = 0;
    for (int l = 0; l < p->L; l++) counts[l] = 0;
    for (const Image &x : p->parts) {
        for (int l = 0; l < p->L; l++) counts[l] += x.counts[l];
        h += x.hash;
    }
    if (hash) *hash = h;
    return GRG_OK;
}

int grg_part_bounds(grg_part *p, uint32_t cap, uint32_t *bounds, uint32_t *num_parts)
{
    if (!p || !num_parts) return GRG_E_ARG;
    *num_parts = (uint32_t)p->parts.size();
    if (cap < p->parts.size() + 1 || !bounds) return cap ? GRG_E_RANGE : GRG_OK;
    for (size_t i = 0; i < p->parts.size(); i++) bounds[i] = p->parts[i].lo;
    bounds[p->parts.size()] = p->parts.empty() ? 0 : p->parts.back().hi;
    return GRG_OK;
}

}  // extern "C"
