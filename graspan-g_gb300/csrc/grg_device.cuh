// grg_device.cuh -- device-side data layout and primitives of the closure engine.
//
// Storage ("sparse bit-vector", the reference's element unit, src/kernel.h:32-44):
// every (label slot, row) owns an open-addressing hash table of 32-byte
// elements in one device pool. Element words 0..5 are a bitmap of 192
// consecutive destination ids, word 6 is the key (slot << 25 | base, base =
// dst / 192), word 7 the row (source vertex). The reference links elements of
// a row into a sorted list (word 7 = NEXT, src/kernel.cu:165-202); here a
// row's elements are hashed by base, so a lookup is one or two probes instead
// of a list walk and rows never need re-sorting.
//
// Deltas: a parallel pool of 32-byte delta bitmaps (words 0..5 = bits that
// became set this round; words 6..7 = the slot's key and row, written when the
// slot is filled, so the gather reads one sector per record) and a dirty
// bitmap with one bit per pool slot. An
// insert that sets new bits ORs them into the slot's delta bitmap and sets the
// slot's dirty bit, both fire-and-forget; the next round's gather scans the
// dirty bitmap and emits one delta record per dirty slot, in slot order (so a
// row's records come out together). Nothing is appended to a shared list, so
// no counter is contended and no capacity can be exceeded. This replaces the reference's tmp region and the
// diff/merge kernels (src/kernel.cu:841-985): new edges are found by atomicOr
// on the stored element, which returns exactly the bits that were new.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace grg {

constexpr int EW = 6;                    // bitmap words per element
constexpr uint32_t EIDS = 192;           // ids per element
constexpr uint32_t EMPTY = 0xFFFFFFFFu;  // free slot key
constexpr int KEY_SHIFT = 25;
constexpr uint32_t BASE_MASK = (1u << KEY_SHIFT) - 1;
constexpr int MAX_LABELS = 63;
constexpr int MAX_SLOTS = 2 * MAX_LABELS;  // label slots 1..L, reverse-index slots L+1..2L
constexpr int MAX_RULES = 64;
constexpr uint32_t OL_SLOT0 = 64;          // label slots >= 64 in a delta record: old-left rule (slot - 64)

// device counter block indices
enum : int {
    C_POOL_TOP = 0,   // bump allocator (elements)
    C_DIRTY_N = 1,    // delta records gathered this round
    C_RETRY_N = 2,    // retry-list length (delta records to re-run)
    C_GROW_N = 3,     // grow-list length
    C_ERR = 4,        // error bits
    C_LEFT = 5,       // left-operand elements of binary joins
    C_RIGHT = 6,      // right-operand elements of binary joins
    C_INSERTS = 7,    // global element inserts issued
    C_TOTAL = 8,      // edge count (count kernel)
    C_HASH = 9,       // edge-set hash (hash kernel)
    C_EXPORT = 10,    // export cursor
    C_PH0 = 11,       // join phase cycle counters (built with -DGRG_PHASE_TIMERS): 11..15
    C_CAND_N = 16,    // candidate elements written by joins for k_apply
    C_AFAIL = 17,     // candidates k_apply could not insert (tables to grow)
    C_VN = 18,        // virtual old-left records written
    C_HALT = 19,      // device-driven rounds: why the round loop stopped (0 = running)
    C_ITERS = 20,     // device-driven round iterations started
    C_GROUNDS = 21,   // device-driven rounds that had delta records
    C_GDSUM = 22,     // delta records of those rounds
    C_JNS = 23,       // join-pass nanoseconds of those rounds (with kernel timing)
    C_LABEL0 = 24,    // per-label edge counts: C_LABEL0 + slot
    C_JT0 = C_LABEL0 + MAX_SLOTS + 2,   // start time of the current join pass (device-driven rounds)
    C_MAXR = C_LABEL0 + MAX_SLOTS + 3,  // rounds a device-driven launch may run (0 = until the fixpoint)
    C_WOUT = C_LABEL0 + MAX_SLOTS + 4,  // right-hand items the join's dense window could not hold
    C_SPLIT_N = C_LABEL0 + MAX_SLOTS + 5,  // sub-records of a small round (k_split)
    C_JN1 = C_LABEL0 + MAX_SLOTS + 6,   // records the join reads from the gathered buffer this round
    C_JN2 = C_LABEL0 + MAX_SLOTS + 7,   // records the join reads from the virtual-record buffer this round
    C_GT0 = C_LABEL0 + MAX_SLOTS + 8,   // start time of the current gather (kernel timing)
    C_GNS = C_LABEL0 + MAX_SLOTS + 9,   // gather nanoseconds (kernel timing)
    C_BADIN = C_LABEL0 + MAX_SLOTS + 10, // input edges refused: ERR_IN_LABEL / ERR_IN_RANGE bits
    C_DH0 = C_LABEL0 + MAX_SLOTS + 11,   // 8 counters: tables by log2 of their elements (tuning key)
    C_CHECK = C_LABEL0 + MAX_SLOTS + 19, // first failed bounds check of the push kernels: id << 56 | value
    C_JQ = C_LABEL0 + MAX_SLOTS + 20,    // work queue of a join or push launch: next 32-record batch (zeroed before each launch)
    C_NOSLOT = C_LABEL0 + MAX_SLOTS + 21, // of C_WOUT: items of a run of records left without a window slot
    C_CANDS = C_LABEL0 + MAX_SLOTS + 22,  // candidates k_apply inserted over the closure
    NCTR = C_LABEL0 + MAX_SLOTS + 23
};
// error bits of C_ERR; ERR_IN_* (in C_BADIN) flag input edges that were refused
// (label outside 1..L, vertex id outside the graph) and never touched a table
enum : unsigned long long { ERR_POOL = 1, ERR_LOAD = 2, ERR_INTERNAL = 4, ERR_IN_LABEL = 8, ERR_IN_RANGE = 16 };

struct RuleTable {
    int L;                                   // labels
    // binary rules A ::= B C grouped by B
    uint8_t bin_start[MAX_LABELS + 2];
    uint8_t bin_A[MAX_RULES], bin_C[MAX_RULES];
    // unary rules A ::= B grouped by B (empty under filter 1)
    uint8_t un_start[MAX_LABELS + 2];
    uint8_t un_A[MAX_RULES];
    // old-left joins O_B o D_C of rules A ::= B C whose C is derivable (filter 0):
    // rule q (0..nol-1) = (ol_A[q], ol_B[q], ol_C[q]); a virtual delta record
    // with label slot OL_SLOT0 + q carries an O_B element masked to the
    // vertices k whose row C[k] has deltas this round
    int nol;
    uint8_t ol_A[MAX_RULES], ol_B[MAX_RULES], ol_C[MAX_RULES];
    uint8_t dindex[MAX_LABELS + 1];          // label C: index this round's deltas per row
    uint8_t track[MAX_SLOTS + 2];            // slot: new bits become deltas
    // labels stored by destination: the table of (label, row j) holds the sources
    // i of edges (i, j), as 192-id elements over i. A binary rule A ::= B C whose
    // B and A are stored so and whose C is never derived is then joined by pushing
    // each delta element of B at column k, whole, into A's column j for every
    // edge (k, j) of C -- bit-parallel over the sources, where the join by source
    // rows visits every source-intermediate pair. Chosen per label when the
    // grammar allows it (see plan_columns); C stays stored by source.
    uint8_t tpose[MAX_LABELS + 1];
    // labels never inserted into after the load that are a rule's second
    // symbol also get a CSR copy (row pointers + destination ids): joins read
    // 4 bytes per edge instead of a 32-byte element per 192-id block
    const uint2 *csr_row[MAX_LABELS + 1];    // {first edge, degree | min(elements,255) << 24}
    const uint32_t *csr_col[MAX_LABELS + 1];
    uint32_t csr_n[MAX_LABELS + 1];          // destination ids in each CSR copy
};

// A failed bounds check (id >= 1): the access is skipped and the first
// failure's check id and offending value are kept in C_CHECK; the host then
// returns GRG_E_INTERNAL with them instead of touching memory out of bounds.
__device__ __forceinline__ bool check_failed(unsigned long long *ctr, unsigned id, unsigned long long value)
{
    atomicCAS(&ctr[C_CHECK], 0ull, ((unsigned long long)id << 56) | (value & ((1ull << 56) - 1)));
    return true;
}

struct Dev {
    uint32_t *elems;          // pool: 8 words per slot
    uint32_t *dbits;          // delta bitmaps: 8 words per slot
    uint64_t *desc;           // [(slot-1)*V + row] = cap << 32 | offset
    uint32_t *cnt;            // occupied slots per table
    uint32_t *want;           // failed inserts per table since its last growth
    uint32_t *dmap;           // dirty bitmap: bit s = slot s has delta bits
    uint32_t *grow;           // grow list (table indices)
    uint4 *cand;              // candidate elements (32 B: bits[6], key, row) for k_apply; may be null
    uint64_t cand_cap;        // candidates
    uint64_t retry_cap;       // records a join's retry list holds (more are counted, not written)
    // this round's delta index (labels with dindex): records [drs, drs+drc) of
    // the gathered delta buffer drec belong to table (label, row); dvm = vertex
    // bitmap per label of rows with deltas (vwords words per label)
    uint32_t *drs;
    uint32_t *drc;
    uint32_t *dvm;
    const uint4 *drec;
    uint32_t vwords;
    // per-slot stamps of a graph loaded from element images (null otherwise):
    // the run in which the element last gained bits, carried through growth,
    // compaction and export; the out-of-core schedule marks deltas from them
    uint32_t *stamp;
    // labels whose small tables (capacity <= PREFIX_CAP) are filled as a prefix
    // (probing from slot 0), so a join reading the row as right-hand items reads
    // only its occupied slots: bit l-1 = label l
    unsigned long long prefix_mask;
    unsigned long long *ctr;  // counter block
    uint32_t V;
    uint32_t pool_cap;        // elements
    // the context's grammar under this closure's filter. It travels with every
    // launch (kernel parameters live in the constant bank, so reads cost what a
    // __constant__ table costs), so contexts with different grammars can run
    // on one device, on one stream or several, without sharing any table
    RuleTable rt;
};

__device__ __forceinline__ uint32_t hash_slot(uint32_t base, uint32_t lg)
{
    return lg ? (base * 0x9E3779B1u) >> (32 - lg) : 0u;
}
__device__ __forceinline__ uint32_t max_load(uint32_t cap) { return cap - (cap >> 2); }

// Table layout: a hashed table (Fibonacci hash, linear probing, load <= 3/4),
// or -- for labels in prefix_mask while their capacity is at most PREFIX_CAP --
// a prefix-filled one: probing starts at slot 0 and a table may fill up, so its
// occupied slots are always slots [0, count). Layout follows from the label and
// capacity alone, so every kernel that places or finds an element agrees.
constexpr uint32_t PREFIX_CAP = 16;
__device__ __forceinline__ bool prefix_table(const Dev &d, uint32_t slot, uint32_t cap)
{
    return cap <= PREFIX_CAP && ((d.prefix_mask >> (slot - 1)) & 1ull);
}
__device__ __forceinline__ uint32_t table_start(const Dev &d, uint32_t slot, uint32_t base, uint32_t cap)
{
    return prefix_table(d, slot, cap) ? 0u : hash_slot(base, 31 - __clz(cap));
}
__device__ __forceinline__ uint32_t table_limit(const Dev &d, uint32_t slot, uint32_t cap)
{
    return prefix_table(d, slot, cap) ? cap : max_load(cap);
}

struct Bits { uint32_t w[EW]; };

#ifndef GRG_LD256
#define GRG_LD256 1   // 32-byte elements and records move with one 256-bit access (0: two 128-bit ones)
#endif
// One 32-byte element or record: every such address is a 32-byte offset into an allocation
// aligned to at least 256 bytes. ld32 is a plain load, ld32_cg one that skips L1 (for
// elements other threads update), st32 a plain store.
__device__ __forceinline__ void ld32(const void *p, uint4 &a, uint4 &b)
{
#if GRG_LD256
    asm volatile("ld.global.v8.u32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(a.x), "=r"(a.y), "=r"(a.z), "=r"(a.w), "=r"(b.x), "=r"(b.y), "=r"(b.z), "=r"(b.w)
                 : "l"(p));
#else
    a = reinterpret_cast<const uint4 *>(p)[0];
    b = reinterpret_cast<const uint4 *>(p)[1];
#endif
}
__device__ __forceinline__ void ld32_cg(const void *p, uint4 &a, uint4 &b)
{
#if GRG_LD256
    asm volatile("ld.global.cg.v8.u32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(a.x), "=r"(a.y), "=r"(a.z), "=r"(a.w), "=r"(b.x), "=r"(b.y), "=r"(b.z), "=r"(b.w)
                 : "l"(p));
#else
    a = __ldcg(reinterpret_cast<const uint4 *>(p));
    b = __ldcg(reinterpret_cast<const uint4 *>(p) + 1);
#endif
}
__device__ __forceinline__ void st32(void *p, const uint4 a, const uint4 b)
{
#if GRG_LD256
    asm volatile("st.global.v8.u32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(p), "r"(a.x), "r"(a.y),
                 "r"(a.z), "r"(a.w), "r"(b.x), "r"(b.y), "r"(b.z), "r"(b.w)
                 : "memory");
#else
    reinterpret_cast<uint4 *>(p)[0] = a;
    reinterpret_cast<uint4 *>(p)[1] = b;
#endif
}

__device__ __forceinline__ uint64_t splitmix64(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
__device__ __forceinline__ uint64_t edge_hash(uint32_t l, uint32_t s, uint32_t d)
{
    return splitmix64(splitmix64(((uint64_t)s << 32) | d) ^ ((uint64_t)l * 0x9E3779B97F4A7C15ull));
}

// OR `b` into the element in pool slot s. With `track`, the bits that were new
// go to its delta bitmap and its dirty bit is set (both without waiting).
// OR `b` into slot s whose bitmap words were read as c0 (words 0-3) and c1.x/.y
// (words 4-5). Words whose candidate bits are all present already need no
// atomic: bits are only ever set during a round, so a stale read can only show
// fewer of them.
__device__ __forceinline__ bool g_or_cur(const Dev &d, uint32_t s, const Bits b, bool track, const uint4 c0,
                                         const uint4 c1)
{
    uint32_t *e = d.elems + (size_t)s * 8;
    const uint32_t cur[EW] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y};
    Bits nb;
    uint32_t any = 0;
#pragma unroll
    for (int w = 0; w < EW; w++) {
        nb.w[w] = 0;
        if (b.w[w] & ~cur[w]) {
            const uint32_t old = atomicOr(&e[w], b.w[w]);
            nb.w[w] = b.w[w] & ~old;
            any |= nb.w[w];
        }
    }
    if (track && any) {
        uint32_t *db = d.dbits + (size_t)s * 8;
#pragma unroll
        for (int w = 0; w < EW; w++)
            if (nb.w[w]) atomicOr(&db[w], nb.w[w]);
        atomicOr(&d.dmap[s >> 5], 1u << (s & 31));
    }
    return true;
}

__device__ __forceinline__ bool g_or_into(const Dev &d, uint32_t s, const Bits b, bool track)
{
    const uint32_t *e = d.elems + (size_t)s * 8;
    uint4 c0, c1;
    ld32_cg(e, c0, c1);
    return g_or_cur(d, s, b, track, c0, c1);
}

// OR `b` into element (slot, row, base). Returns false when the table is full
// or absent; the failure is recorded so the table grows before a retry. With
// `track`, the bits that were new are ORed into the element's delta bitmap and
// its dirty bit is set (both without waiting for a reply). WHOLE: a probe of a
// hashed table reads the whole 32-byte element (one sector), so a key found at
// its probe brings the bitmap words for the pre-check without a second round
// trip (prefix-filled tables, scanned from slot 0, read keys only).
template <bool WHOLE>
__device__ __forceinline__ bool g_insert_t(const Dev &d, uint32_t slot, uint32_t row, uint32_t base, const Bits b,
                                           bool track)
{
    const size_t ti = (size_t)(slot - 1) * d.V + row;
    const uint64_t de = d.desc[ti];
    const uint32_t off = (uint32_t)de, cap = (uint32_t)(de >> 32);
    const uint32_t key = (slot << KEY_SHIFT) | base;
    uint32_t s = EMPTY;
    bool have = false;                        // c0 / c1 hold slot s's bitmap words (or zeros)
    uint4 c0 = make_uint4(0, 0, 0, 0), c1 = make_uint4(0, 0, 0, 0);
    if (cap != 0 && (cap & (cap - 1)) == 0) {
        const uint32_t h = table_start(d, slot, base, cap), lim = table_limit(d, slot, cap);
        const bool whole = WHOLE && !prefix_table(d, slot, cap);
        for (uint32_t p = 0; p < cap; p++) {
            const uint32_t q = off + ((h + p) & (cap - 1));
            uint32_t *kp = d.elems + (size_t)q * 8 + 6;
            uint32_t k;
            if (whole) {
                ld32_cg(d.elems + (size_t)q * 8, c0, c1);
                k = c1.z;
            } else {
                k = __ldcg(kp);
            }
            if (k == key) { s = q; have = whole; break; }
            if (k != EMPTY) continue;
            if (atomicAdd(&d.cnt[ti], 1u) >= lim) { atomicSub(&d.cnt[ti], 1u); break; }
            const uint32_t prev = atomicCAS(kp, EMPTY, key);
            // a slot claimed here, or by a concurrent insert of the same key, is ORed
            // into without a pre-check (its words read as zero)
            c0 = c1 = make_uint4(0, 0, 0, 0);
            if (prev == EMPTY) {
                d.elems[(size_t)q * 8 + 7] = row;
                // the delta bitmap's spare words carry the slot's key and row for the gather
                reinterpret_cast<uint2 *>(d.dbits + (size_t)q * 8)[3] = make_uint2(key, row);
                s = q;
                have = true;
                break;
            }
            atomicSub(&d.cnt[ti], 1u);
            if (prev == key) { s = q; have = true; break; }
        }
    }
    if (s == EMPTY) {
        if (atomicAdd(&d.want[ti], 1u) == 0) {
            const unsigned long long g = atomicAdd(&d.ctr[C_GROW_N], 1ull);
            d.grow[g] = (uint32_t)ti;
        }
        return false;
    }
    return have ? g_or_cur(d, s, b, track, c0, c1) : g_or_into(d, s, b, track);
}

__device__ __forceinline__ bool g_insert(const Dev &d, uint32_t slot, uint32_t row, uint32_t base, const Bits b,
                                         bool track)
{
    return g_insert_t<false>(d, slot, row, base, b, track);
}

}  // namespace grg
