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
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <thread>
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
    bool done = false;               // stream schedule: this partition's rows are closed
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

// The next device run's input, prepared while the current run computes: a
// helper thread assembles it in page-locked memory and copies it to the device
// on a copy stream of its own, and allocates ahead the page-locked buffers that
// the coming exports fill (pinning host memory costs about as much as copying
// it). A run whose input was prepared loads it from the device.
struct Ahead {
    std::thread th;
    bool active = false;             // a helper thread was started for `key`
    int status = GRG_OK;             // the helper's CUDA status
    std::vector<uint64_t> key;       // the run it prepares: partition ids, kind, marks
    uint64_t n = 0;                  // records
    Pinned pin;                      // page-locked staging
    uint32_t *d_rec = nullptr, *d_st = nullptr;   // device copy
    uint64_t dcap = 0;
    cudaStream_t cs = nullptr;
    cudaEvent_t ev = nullptr;
    ~Ahead()
    {
        if (th.joinable()) th.join();
        if (ev) cudaEventDestroy(ev);
        if (cs) cudaStreamDestroy(cs);
        cudaFree(d_rec);
        cudaFree(d_st);
    }
};

struct grg_part {
    grg_ctx *ctx = nullptr;
    Ahead ahead;                     // the next run's input (see Ahead)
    double grow = 0;                 // largest closed/loaded image size ratio seen (export buffer sizing)
    uint64_t prefetched = 0, prefetch_hits = 0;
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
    // checkpoint / run budget
    std::string ckpt_path;           // empty = no automatic checkpoints
    uint32_t ckpt_every = 0;         // save after every this many runs of a call
    uint64_t run_budget = 0;         // runs per grg_part_run call (0 = unbounded)
    uint64_t runs_call = 0;          // runs made by the current call
    int run_filter = -1;             // filter of a paused run (-1 = none)
    bool window_pinned = false;      // the first tuned run's join window holds for the other runs
    uint64_t cursor = 0;             // pairs schedule: position in the paused superstep's pair order
    bool cursor_ran = false;         // a run happened in that superstep before the pause
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

// ---- checkpoint file: the partition set's whole state, with a checksum over
// every byte before it (64-bit words, FNV-1a style). Native byte order.

constexpr char CKPT_MAGIC[8] = {'G', 'R', 'G', 'P', 'A', 'R', 'T', '1'};
constexpr uint32_t CKPT_VERSION = 1;

struct Hasher {
    uint64_t h = 1469598103934665603ull, pend = 0;
    int npend = 0;
    void byte(uint8_t b)
    {
        pend |= (uint64_t)b << (8 * npend);
        if (++npend == 8) word();
    }
    void word()
    {
        h = (h ^ pend) * 1099511628211ull;
        pend = 0;
        npend = 0;
    }
    void mix(const void *p, size_t n)
    {
        const uint8_t *b = (const uint8_t *)p;
        while (n && npend) { byte(*b++); n--; }
        for (; n >= 8; n -= 8, b += 8) {
            memcpy(&pend, b, 8);
            word();
        }
        while (n) { byte(*b++); n--; }
    }
    uint64_t final_value()
    {
        if (npend) word();
        return h;
    }
};

struct Writer {
    FILE *f = nullptr;
    Hasher hs;
    bool ok = true;
    void put(const void *p, size_t n)
    {
        if (!ok || !n) return;
        if (fwrite(p, 1, n, f) != n) ok = false;
        hs.mix(p, n);
    }
    template <class T> void val(T v) { put(&v, sizeof v); }
};

struct Reader {
    FILE *f = nullptr;
    Hasher hs;
    uint64_t left = 0;               // bytes of the file not read yet
    bool ok = true;
    bool get(void *p, size_t n)
    {
        if (!ok) return false;
        if (n > left || (n && fread(p, 1, n, f) != n)) return ok = false;
        left -= n;
        hs.mix(p, n);
        return true;
    }
    template <class T> bool val(T &v) { return get(&v, sizeof v); }
};

int save_state(grg_part *p, const char *path)
{
    const std::string tmp = std::string(path) + ".tmp";
    Writer w;
    w.f = fopen(tmp.c_str(), "wb");
    if (!w.f) return GRG_E_IO;
    w.put(CKPT_MAGIC, 8);
    w.val(CKPT_VERSION);
    w.val(p->V);
    w.val(p->R);
    w.val(p->L);
    w.put(p->rules, sizeof(int) * 3 * p->R);
    w.val(p->run_id);
    w.val(p->next_id);
    w.val(p->run_filter);
    w.val((uint8_t)p->loaded);
    w.val((uint8_t)p->closed);
    w.val((uint64_t)p->S.splits);
    w.val(p->cursor);
    w.val((uint8_t)p->cursor_ran);
    w.val((uint64_t)p->parts.size());
    for (const Image &x : p->parts) {
        w.val(x.id); w.val(x.lo); w.val(x.hi); w.val(x.max_stamp); w.val(x.last_run);
        w.val((uint8_t)x.counted);
        w.val((uint8_t)x.done);
        w.val((uint64_t)x.reach.size());
        w.put(x.reach.data(), 4 * x.reach.size());
        w.val((uint64_t)x.counts.size());
        w.put(x.counts.data(), 8 * x.counts.size());
        w.val(x.hash);
        w.val((uint64_t)x.size());
        w.put(x.rec.data(), 32 * x.size());
        w.put(x.st.data(), 4 * x.size());
    }
    w.val((uint64_t)p->seen.size());
    for (const auto &kv : p->seen) {
        w.val(kv.first.first);
        w.val(kv.first.second);
        w.val(kv.second);
    }
    const uint64_t sum = w.hs.final_value();
    if (w.ok && fwrite(&sum, 8, 1, w.f) != 1) w.ok = false;
    if (fflush(w.f) != 0) w.ok = false;
    if (fclose(w.f) != 0) w.ok = false;
    if (!w.ok || rename(tmp.c_str(), path) != 0) {
        remove(tmp.c_str());
        return GRG_E_IO;
    }
    return GRG_OK;
}

// Reads a checkpoint into p (created on the right context, without partitions).
int read_state(grg_part *p, FILE *f, uint64_t size)
{
    Reader r;
    r.f = f;
    if (size < 8) return GRG_E_IO;
    r.left = size - 8;               // the checksum is not part of the hashed bytes
    char magic[8];
    uint32_t ver = 0, V = 0;
    int R = 0, L = 0;
    if (!r.get(magic, 8) || memcmp(magic, CKPT_MAGIC, 8) != 0) return GRG_E_IO;
    if (!r.val(ver) || ver != CKPT_VERSION) return GRG_E_IO;
    if (!r.val(V) || !r.val(R) || !r.val(L)) return GRG_E_IO;
    if (V != p->V || R != p->R || L != p->L) return GRG_E_IO;
    int rules[3 * GRG_MAX_RULES];
    if (!r.get(rules, sizeof(int) * 3 * R) || memcmp(rules, p->rules, sizeof(int) * 3 * R) != 0) return GRG_E_IO;
    uint8_t loaded = 0, closed = 0, cran = 0;
    uint64_t splits = 0, nparts = 0;
    if (!r.val(p->run_id) || !r.val(p->next_id) || !r.val(p->run_filter) || !r.val(loaded) || !r.val(closed) ||
        !r.val(splits) || !r.val(p->cursor) || !r.val(cran) || !r.val(nparts))
        return GRG_E_IO;
    p->cursor_ran = cran != 0;
    if (nparts == 0 || nparts > (uint64_t)V + 1 || p->run_filter < -1 || p->run_filter > 1) return GRG_E_IO;
    p->parts.clear();
    uint32_t expect_lo = 0;
    for (uint64_t q = 0; q < nparts; q++) {
        Image x;
        uint8_t counted = 0, done = 0;
        uint64_t nreach = 0, ncounts = 0, n = 0;
        if (!r.val(x.id) || !r.val(x.lo) || !r.val(x.hi) || !r.val(x.max_stamp) || !r.val(x.last_run) ||
            !r.val(counted) || !r.val(done) || !r.val(nreach))
            return GRG_E_IO;
        if (x.lo != expect_lo || x.hi <= x.lo || x.hi > V || x.id >= p->next_id) return GRG_E_IO;
        expect_lo = x.hi;
        if (nreach > r.left / 4) return GRG_E_IO;
        x.reach.resize(nreach);
        if (!r.get(x.reach.data(), 4 * nreach) || !r.val(ncounts)) return GRG_E_IO;
        if (ncounts != 0 && ncounts != (uint64_t)L) return GRG_E_IO;
        x.counts.resize(ncounts);
        if (!r.get(x.counts.data(), 8 * ncounts) || !r.val(x.hash) || !r.val(n)) return GRG_E_IO;
        if (n > r.left / 36) return GRG_E_IO;
        if (!x.rec.resize(8 * n) || !x.st.resize(n)) return GRG_E_NOMEM;
        if (!r.get(x.rec.data(), 32 * n) || !r.get(x.st.data(), 4 * n)) return GRG_E_IO;
        for (uint64_t e = 0; e < n; e++) {
            const uint32_t row = x.rec[8 * e + 7], lab = x.rec[8 * e + 6] >> KEY_SHIFT;
            if (row < x.lo || row >= x.hi || lab < 1 || lab > (uint32_t)L) return GRG_E_IO;
        }
        x.counted = counted != 0;
        x.done = done != 0;
        if (x.counted && ncounts != (uint64_t)L) return GRG_E_IO;
        p->parts.push_back(std::move(x));
    }
    if (expect_lo != V) return GRG_E_IO;
    uint64_t nseen = 0;
    if (!r.val(nseen) || nseen > r.left / 12) return GRG_E_IO;
    p->seen.clear();
    for (uint64_t q = 0; q < nseen; q++) {
        uint32_t a = 0, b = 0, t = 0;
        if (!r.val(a) || !r.val(b) || !r.val(t)) return GRG_E_IO;
        p->seen[std::make_pair(a, b)] = t;
    }
    uint64_t want = 0;
    if (r.left != 0 || fread(&want, 8, 1, f) != 1 || want != r.hs.final_value()) return GRG_E_IO;
    p->loaded = loaded != 0;
    p->closed = closed != 0;
    p->S = grg_part_stats{};
    p->S.splits = splits;
    return GRG_OK;
}

// Bookkeeping after each completed device run: count it, checkpoint when due.
int ahead_join(grg_part *p);

int after_run(grg_part *p)
{
    p->runs_call++;
    if (p->ckpt_every && !p->ckpt_path.empty() && p->runs_call % p->ckpt_every == 0) {
        // the helper thread may be growing an image's buffers: let it finish first
        const int st = ahead_join(p);
        if (st) return st;
        return save_state(p, p->ckpt_path.c_str());
    }
    return GRG_OK;
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

// A device run's input: `extra` first (the stream schedule's static records,
// stamped 1 in [mark_lo, mark_hi) and 0 elsewhere, so that only the run's own
// partition's static rows are marked), then the partitions' images (only labels
// in keep_label when given; with own_one, their stamps count as 1).
struct RunInput {
    std::vector<size_t> idx;
    const Image *extra = nullptr;
    uint64_t mark_lo = 0, mark_hi = 0;
    const bool *keep_label = nullptr;
    bool own_one = false;
    uint32_t mark_after = 0;
};

uint64_t input_size(const grg_part *p, const RunInput &in)
{
    uint64_t n = in.extra ? in.extra->size() : 0;
    for (size_t i : in.idx) {
        const Image &x = p->parts[i];
        if (!in.keep_label) {
            n += x.size();
            continue;
        }
        for (uint64_t e = 0; e < x.size(); e++)
            if (in.keep_label[x.rec[8 * e + 6] >> KEY_SHIFT]) n++;
    }
    return n;
}

void stage_input(const grg_part *p, const RunInput &in, uint32_t *rec, uint32_t *st)
{
    uint64_t k = 0;
    if (in.extra && in.extra->size()) {
        const Image &x = *in.extra;
        memcpy(rec, x.rec.data(), x.size() * 32);
        memset(st, 0, x.size() * 4);
        for (uint64_t e = in.mark_lo; e < in.mark_hi; e++) st[e] = 1;
        k = x.size();
    }
    for (size_t i : in.idx) {
        const Image &x = p->parts[i];
        if (!in.keep_label) {                // whole images: one copy each
            memcpy(rec + 8 * k, x.rec.data(), x.size() * 32);
            if (in.own_one)
                for (uint64_t e = 0; e < x.size(); e++) st[k + e] = 1;
            else
                memcpy(st + k, x.st.data(), x.size() * 4);
            k += x.size();
            continue;
        }
        for (uint64_t e = 0; e < x.size(); e++) {
            if (!in.keep_label[x.rec[8 * e + 6] >> KEY_SHIFT]) continue;
            memcpy(rec + 8 * k, x.rec.data() + 8 * e, 32);
            st[k] = in.own_one ? 1u : x.st[e];
            k++;
        }
    }
}

// Identity of a run's input: what it holds and how it is marked.
std::vector<uint64_t> input_key(const grg_part *p, const RunInput &in)
{
    std::vector<uint64_t> k = {in.extra ? 1ull : 0ull, in.mark_lo, in.mark_hi, in.keep_label ? 1ull : 0ull,
                               in.own_one ? 1ull : 0ull, in.mark_after};
    for (size_t i : in.idx) {
        k.push_back(p->parts[i].id);
        k.push_back(p->parts[i].size());
    }
    return k;
}

// Waits for the helper thread; the prepared input stays for a run with its key.
int ahead_join(grg_part *p)
{
    Ahead &a = p->ahead;
    if (a.th.joinable()) a.th.join();
    return a.status;
}

void ahead_drop(grg_part *p)
{
    ahead_join(p);
    p->ahead.active = false;
    p->ahead.key.clear();
}

// Starts preparing `next` on the helper thread (the partitions it holds must not be
// changed before the next ahead_join). Image buffers of its partitions are grown
// ahead to the size their closure is expected to reach.
int ahead_start(grg_part *p, const RunInput &next)
{
    Ahead &a = p->ahead;
    ahead_drop(p);
    const uint64_t n = input_size(p, next);
    if (!n) return GRG_OK;
    // page-locked and device buffers are sized here, on the calling thread
    int st = a.pin.ensure(n);
    if (st) return GRG_OK;                   // no room to prepare: the run stages its input itself
    if (a.dcap < n) {
        cudaFree(a.d_rec);
        cudaFree(a.d_st);
        a.d_rec = a.d_st = nullptr;
        a.dcap = 0;
        const uint64_t c = n + n / 4;
        if (cudaMalloc(&a.d_rec, c * 32) != cudaSuccess || cudaMalloc(&a.d_st, c * 4) != cudaSuccess) {
            cudaGetLastError();
            cudaFree(a.d_rec);
            cudaFree(a.d_st);
            a.d_rec = a.d_st = nullptr;
            return GRG_OK;
        }
        a.dcap = c;
    }
    if (!a.cs && cudaStreamCreateWithFlags(&a.cs, cudaStreamNonBlocking) != cudaSuccess) return GRG_E_CUDA;
    if (!a.ev && cudaEventCreateWithFlags(&a.ev, cudaEventDisableTiming) != cudaSuccess) return GRG_E_CUDA;
    int dev = 0;
    cudaGetDevice(&dev);
    a.key = input_key(p, next);
    a.n = n;
    a.active = true;
    a.status = GRG_OK;
    std::vector<size_t> grow_idx;
    if (p->grow > 1.0) grow_idx = next.idx;
    const double grow = p->grow;
    a.th = std::thread([p, next, n, dev, grow_idx, grow]() {
        Ahead &h = p->ahead;
        cudaSetDevice(dev);
        stage_input(p, next, h.pin.rec, h.pin.st);
        if (cudaMemcpyAsync(h.d_rec, h.pin.rec, n * 32, cudaMemcpyHostToDevice, h.cs) != cudaSuccess ||
            cudaMemcpyAsync(h.d_st, h.pin.st, n * 4, cudaMemcpyHostToDevice, h.cs) != cudaSuccess ||
            cudaEventRecord(h.ev, h.cs) != cudaSuccess) {
            cudaGetLastError();
            h.status = GRG_E_CUDA;
            return;
        }
        // the coming export of these partitions finds page-locked room already there
        for (size_t i : grow_idx) {
            Image &x = p->parts[i];
            const uint64_t want = (uint64_t)((double)x.size() * grow * 1.1) + 1024;
            if (!x.rec.reserve(want * 8) || !x.st.reserve(want)) break;
        }
    });
    p->prefetched++;
    return GRG_OK;
}

// One device run over the given partitions; `next` (may be null) is the run the
// helper thread prepares meanwhile. Partitions' records are marked when their
// stamp is above mark_after.
int run_once(grg_part *p, uint32_t filter, const RunInput &in, uint32_t run_stamp, const RunInput *next)
{
    int st;
    uint64_t n = 0;
    const uint32_t *rec = nullptr, *stp = nullptr;
    int on_device = 0;
    {
        Timer tm(p->S.stage_ms);
        Ahead &a = p->ahead;
        if (a.active) {
            if ((st = ahead_join(p))) return st;
            if (a.key == input_key(p, in)) {
                if (cudaEventSynchronize(a.ev) != cudaSuccess) return GRG_E_CUDA;
                n = a.n;
                rec = a.d_rec;
                stp = a.d_st;
                on_device = 1;
                p->prefetch_hits++;
            }
            a.active = false;
        }
        if (!on_device) {
            n = input_size(p, in);
            if ((st = p->in.ensure(n))) return st;
            stage_input(p, in, p->in.rec, p->in.st);
            rec = p->in.rec;
            stp = p->in.st;
        }
    }
    p->S.h2d_bytes += n * 36;
    {
        Timer tm(p->S.load_ms);
        if ((st = grg_load_elements(p->ctx, p->V, n, rec, stp, in.mark_after, on_device))) return st;
    }
    // the input is on the device: the next run's can be prepared while this one computes
    if (next && (st = ahead_start(p, *next))) return st;
    grg_stats cs;
    {
        Timer tm(p->S.closure_ms);
        if ((st = grg_closure_ex(p->ctx, filter, run_stamp, &cs))) return st;
    }
    // partitions of one graph share its degree distribution: the window the first tuned
    // run chose holds for the rest (no trial per partition)
    if (cs.window_tuned && !p->window_pinned) {
        grg_set_join_window(p->ctx, cs.wide_window ? 1 : 0);
        grg_set_join_items(p->ctx, cs.join_elements ? 1 : 0);
        p->window_pinned = true;
    }
    p->S.runs++;
    p->S.rounds += cs.rounds;
    return GRG_OK;
}

// Largest growth of an image from its run input to its exported closure (sizes the
// page-locked buffers allocated ahead).
void note_growth(grg_part *p, uint64_t before, uint64_t after)
{
    if (before) p->grow = std::max(p->grow, (double)after / (double)before);
}

// Every way out of a schedule waits for the helper thread first (it reads the
// schedule's partitions and static records).
struct AheadGuard {
    grg_part *p;
    ~AheadGuard() { ahead_drop(p); }
};

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
    AheadGuard guard{p};                 // declared after stat: joins the helper before stat goes
    auto input_of = [&](size_t i) {
        RunInput in;
        in.idx = {i};
        in.extra = &stat;
        in.mark_lo = seg[i];
        in.mark_hi = seg[i + 1];
        in.keep_label = derived;
        in.own_one = true;                   // every derived record of the partition is marked
        in.mark_after = 0;
        return in;
    };
    for (size_t i = 0; i < p->parts.size();) {
        if (p->parts[i].done) {          // closed before a pause
            i++;
            continue;
        }
        if (p->run_budget && p->runs_call >= p->run_budget) {
            ahead_drop(p);
            return GRG_PAUSED;
        }
        if (stale) {
            ahead_drop(p);               // the prepared input holds the old static records
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
        // the next partition to close, prepared while this one computes
        size_t i2 = i + 1;
        while (i2 < p->parts.size() && p->parts[i2].done) i2++;
        const bool has_next = i2 < p->parts.size() && !(p->run_budget && p->runs_call + 1 >= p->run_budget);
        const RunInput in = input_of(i);
        RunInput nx;
        if (has_next) nx = input_of(i2);
        const uint64_t before = input_size(p, in) - stat.size();
        const int st = run_once(p, filter, in, 0, has_next ? &nx : nullptr);
        if (st == GRG_E_NOMEM) {
            ahead_drop(p);
            if (!split(p, i)) return GRG_E_NOMEM;
            stale = true;
            continue;
        }
        if (st) {
            ahead_drop(p);
            return st;
        }
        int s2 = export_image(p, p->parts[i]);
        if (s2) return s2;
        note_growth(p, before, p->parts[i].size());
        if ((s2 = count_image(p, p->parts[i]))) return s2;
        p->parts[i].done = true;
        if ((s2 = after_run(p))) return s2;
        i++;
    }
    ahead_drop(p);
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
    AheadGuard guard{p};
    for (;;) {
        bool ran = false, restart = false;
        // pairs whose B-edges cross, then partitions no run has closed since their last change
        std::vector<std::pair<size_t, size_t>> order;
        const size_t m = p->parts.size();
        for (size_t i = 0; i < m; i++)
            for (size_t j = i + 1; j < m; j++) order.emplace_back(i, j);
        for (size_t i = 0; i < m; i++) order.emplace_back(i, i);
        auto needed = [&](size_t k) {
            const size_t i = order[k].first, j = order[k].second;
            const Image &a = p->parts[i], &b = p->parts[j];
            const uint32_t t = seen_of(p, a.id, b.id);
            if (i == j) return a.max_stamp > t;
            return reaches(a, b) && (a.max_stamp > t || b.max_stamp > t);
        };
        auto input_of = [&](size_t k) {
            RunInput in;
            in.idx = {order[k].first};
            if (order[k].second != order[k].first) in.idx.push_back(order[k].second);
            in.mark_after = seen_of(p, p->parts[order[k].first].id, p->parts[order[k].second].id);
            return in;
        };
        // a paused superstep continues where it stopped (later pairs are not starved by a restart)
        size_t k0 = 0;
        if (p->cursor && p->cursor < order.size()) {
            k0 = (size_t)p->cursor;
            ran = p->cursor_ran;
        }
        p->cursor = 0;
        p->cursor_ran = false;
        for (size_t k = k0; k < order.size(); k++) {
            const size_t i = order[k].first, j = order[k].second;
            Image &a = p->parts[i], &b = p->parts[j];
            const uint32_t t = seen_of(p, a.id, b.id);
            if (!needed(k)) {
                p->S.skipped++;
                continue;
            }
            if (p->run_budget && p->runs_call >= p->run_budget) {
                ahead_drop(p);
                p->cursor = k;
                p->cursor_ran = ran;
                return GRG_PAUSED;
            }
            // the next pair this superstep runs, prepared meanwhile when it shares no
            // partition with this one (this run changes nothing it reads)
            RunInput nx;
            bool has_next = false;
            if (!(p->run_budget && p->runs_call + 1 >= p->run_budget))
                for (size_t k2 = k + 1; k2 < order.size(); k2++) {
                    if (!needed(k2)) continue;
                    const size_t i2 = order[k2].first, j2 = order[k2].second;
                    if (i2 != i && i2 != j && j2 != i && j2 != j) {
                        nx = input_of(k2);
                        has_next = true;
                    }
                    break;
                }
            const uint32_t r = ++p->run_id;
            const RunInput in = input_of(k);
            const uint64_t before = input_size(p, in);
            const int st = run_once(p, filter, in, r, has_next ? &nx : nullptr);
            if (st == GRG_E_NOMEM) {
                ahead_drop(p);
                const size_t big = (j != i && b.size() > a.size()) ? j : i;
                if (!split(p, big)) return GRG_E_NOMEM;
                restart = true;
                break;
            }
            if (st) {
                ahead_drop(p);
                return st;
            }
            uint64_t after = 0;
            for (size_t q : in.idx) {
                int s2 = export_image(p, p->parts[q]);
                if (s2) return s2;
                after += p->parts[q].size();
                if ((s2 = count_image(p, p->parts[q]))) return s2;
                if ((s2 = reach_image(p, q))) return s2;
                Image &x = p->parts[q];
                x.refresh();
                x.last_run = r;
                p->seen[pkey(x.id, x.id)] = r;   // a run that holds x closes x's own rows
            }
            note_growth(p, before, after);
            p->seen[pkey(a.id, b.id)] = r;
            (void)t;
            ran = true;
            const int s3 = after_run(p);
            if (s3) return s3;
        }
        if (restart) continue;
        p->S.supersteps++;
        if (!ran) {
            ahead_drop(p);
            return GRG_OK;
        }
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
    // partition images are rows by source: the context loads every label that way
    grg_set_layout(ctx, 0);
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
    if (p->run_filter >= 0 && (uint32_t)p->run_filter != filter) return GRG_E_ARG;   // a paused run's filter
    const auto t0 = std::chrono::steady_clock::now();
    const uint64_t splits0 = p->S.splits;
    p->S = grg_part_stats{};
    p->S.splits = splits0;
    p->runs_call = 0;
    bool der[GRG_MAX_LABELS + 1];
    derivable_labels(p, filter, der);
    bool coupled = false;
    for (int q = 0; q < p->R; q++) {
        const int *r = &p->rules[3 * q];
        if (r[1] && r[2] && der[r[2]]) coupled = true;
    }
    p->S.schedule = coupled ? 1 : 0;
    p->prefetched = p->prefetch_hits = 0;
    int st = coupled ? run_pairs(p, filter) : run_stream(p, filter, der);
    p->S.prefetched = p->prefetched;
    p->S.prefetch_hits = p->prefetch_hits;
    if (p->window_pinned) {                // the context tunes again after this run
        grg_set_join_window(p->ctx, 2);
        grg_set_join_items(p->ctx, 2);
        p->window_pinned = false;
    }
    if (st == GRG_PAUSED) {
        p->run_filter = (int)filter;
        p->S.num_parts = (uint32_t)p->parts.size();
        if (!p->ckpt_path.empty() && (st = save_state(p, p->ckpt_path.c_str()))) return st;
        p->S.ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (stats) *stats = p->S;
        return GRG_PAUSED;
    }
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
    p->closed = true;
    p->run_filter = -1;
    if (!p->ckpt_path.empty() && (st = save_state(p, p->ckpt_path.c_str()))) return st;
    p->S.ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
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

int grg_part_export_csr5(grg_part *p, uint32_t index, uint64_t cap, uint8_t *edges, uint32_t *degree,
                         uint64_t *num_edges)
{
    if (!p || !num_edges) return GRG_E_ARG;
    if (!p->closed) return GRG_E_STATE;
    if (index >= p->parts.size()) return GRG_E_RANGE;
    Image &x = p->parts[index];
    uint64_t total = 0;
    for (uint64_t c : x.counts) total += c;
    *num_edges = total;
    if (total > cap) return total ? GRG_E_RANGE : GRG_OK;
    int st = p->in.ensure(x.size());
    if (st) return st;
    memcpy(p->in.rec, x.rec.data(), x.size() * 32);
    memcpy(p->in.st, x.st.data(), x.size() * 4);
    if ((st = grg_load_elements(p->ctx, p->V, x.size(), p->in.rec, p->in.st, ~0u, 0))) return st;
    return grg_export_csr5(p->ctx, x.lo, x.hi, cap, edges, degree, num_edges);
}

int grg_part_save(grg_part *p, const char *path)
{
    if (!p || !path) return GRG_E_ARG;
    if (!p->loaded) return GRG_E_STATE;
    return save_state(p, path);
}

int grg_part_restore(grg_part **out, grg_ctx *ctx, const char *path)
{
    if (!out || !ctx || !path) return GRG_E_ARG;
    *out = nullptr;
    FILE *f = fopen(path, "rb");
    if (!f) return GRG_E_IO;
    uint64_t size = 0;
    if (fseek(f, 0, SEEK_END) == 0) {
        const long e = ftell(f);
        size = e > 0 ? (uint64_t)e : 0;
    }
    fseek(f, 0, SEEK_SET);
    grg_part *p = new grg_part;
    p->ctx = ctx;
    grg_set_layout(ctx, 0);                 // partition images are rows by source
    int st = grg_get_rules(ctx, &p->R, p->rules, &p->L);
    if (!st) {
        for (int q = 0; q < p->R; q++)
            if (p->rules[3 * q + 1] && p->rules[3 * q + 2]) p->bmask |= 1ull << (p->rules[3 * q + 1] - 1);
        // the vertex count is the file's; read it first so read_state can compare the rest
        uint32_t V = 0;
        char magic[8];
        uint32_t ver = 0;
        if (fread(magic, 1, 8, f) != 8 || fread(&ver, 4, 1, f) != 1 || fread(&V, 4, 1, f) != 1) st = GRG_E_IO;
        fseek(f, 0, SEEK_SET);
        p->V = V;
        if (!st) st = read_state(p, f, size);
    }
    fclose(f);
    if (st) {
        delete p;
        return st;
    }
    *out = p;
    return GRG_OK;
}

int grg_part_set_checkpoint(grg_part *p, const char *path, uint32_t every_runs)
{
    if (!p) return GRG_E_ARG;
    p->ckpt_path = path ? path : "";
    p->ckpt_every = path ? every_runs : 0;
    return GRG_OK;
}

int grg_part_set_run_budget(grg_part *p, uint64_t max_runs)
{
    if (!p) return GRG_E_ARG;
    p->run_budget = max_runs;
    return GRG_OK;
}

}  // extern "C"
