// grg_engine.cu -- CUDA kernels and the C ABI of the closure engine (sm_103a).
//
// Hot path (reference: src/kernel.cu):
//   k_join    binary joins A ::= B C for a round's delta records, delta-left
//             (D_B o O_C) and old-left (O_B o D_C, pulled through this round's
//             delta index: virtual records from k_oldleft),
//             unary rules A ::= B, and dedup of every candidate against the
//             stored rows. Replaces compute11/compute10 (src/kernel.cu:403-442)
//             and diff/merge (src/kernel.cu:841-985).
//             Its delta records come straight from the last round's dirty list
//             (the reference's Delta region, mergeAndDiff src/kernel.cu:943-985).
//   k_grow    re-hashes tables that overflowed; their delta records are re-run
//             (the reference instead repartitions on overflow, src/main.cpp:633-762).
// Loader (createGraph, src/main.cpp:223-333): k_load_hist/k_load_alloc/
// k_load_insert/k_eps_insert/k_compact_static/k_mark_all.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "grg.h"
#include "grg_device.cuh"
#include "grg_format.h"

namespace grg {

// Rule table of a grammar under a filter (filter semantics: src/kernel.cu:490-494,
// 499-503): binary rules by first symbol, unary rules (filter 0 only), old-left
// joins for binary rules whose second symbol is derivable (filter 0; refused
// under filter 1), tracked and delta-indexed labels.
static int make_rule_table(const int *rules, int R, int L, uint32_t filter, RuleTable &rt, bool *derivable)
{
    memset(&rt, 0, sizeof rt);
    rt.L = L;
    for (int l = 0; l <= MAX_LABELS; l++) derivable[l] = false;
    for (int q = 0; q < R; q++) {
        const int *r = &rules[3 * q];
        const bool unary = r[1] && !r[2];
        if (!(filter && unary)) derivable[r[0]] = true;
    }
    int nol = 0;
    for (int q = 0; q < R; q++) {
        const int *r = &rules[3 * q];
        if (r[1] && r[2] && derivable[r[2]]) {
            if (filter) return GRG_E_FILTER;
            rt.ol_A[nol] = (uint8_t)r[0];
            rt.ol_B[nol] = (uint8_t)r[1];
            rt.ol_C[nol] = (uint8_t)r[2];
            rt.dindex[r[2]] = 1;
            rt.track[r[2]] = 1;
            nol++;
        }
    }
    rt.nol = nol;
    int k = 0;
    for (int B = 1; B <= L + 1; B++) {
        rt.bin_start[B] = (uint8_t)k;
        if (B > L) break;
        for (int q = 0; q < R; q++)
            if (rules[3 * q + 1] == B && rules[3 * q + 2]) {
                rt.bin_A[k] = (uint8_t)rules[3 * q];
                rt.bin_C[k] = (uint8_t)rules[3 * q + 2];
                k++;
            }
    }
    k = 0;
    for (int B = 1; B <= L + 1; B++) {
        rt.un_start[B] = (uint8_t)k;
        if (B > L || filter) continue;
        for (int q = 0; q < R; q++)
            if (rules[3 * q + 1] == B && !rules[3 * q + 2]) rt.un_A[k++] = (uint8_t)rules[3 * q];
    }
    // tracked labels: left operand of an active binary/unary rule, or right operand of an old-left join
    for (int q = 0; q < R; q++) {
        const int *r = &rules[3 * q];
        const bool unary = r[1] && !r[2];
        if (r[1] && !(filter && unary)) rt.track[r[1]] = 1;
    }
    return GRG_OK;
}

// Labels that can be stored by destination (bit l-1 = label l; see RuleTable::tpose).
// Decided from the grammar alone, so the layout chosen at the load holds under
// either filter. Start from every label a rule derives and drop labels until:
//  - a binary rule A ::= B C whose C is derived needs old-left joins, which read
//    rows of B and C by source: A, B and C stay by source;
//  - a binary rule A ::= B C with a C that is never derived joins by pushing B's
//    columns along C's source rows: A and B are stored alike (both or neither);
//  - a unary rule A ::= B keeps the orientation (A and B alike), except that A may
//    be stored by destination when B is never derived: B's loaded edges are then
//    turned around once, in round 1;
//  - a label read as a rule's second symbol is never derived here, so it stays by
//    source (its rows, or their CSR copy, are what a push walks).
// Labels no rule derives stay by source (they are inputs: read as second symbols
// or unary sources by source rows).
static uint64_t plan_columns(const int *rules, int R, int L)
{
    bool der[MAX_LABELS + 1] = {false};
    for (int q = 0; q < R; q++) der[rules[3 * q]] = true;
    uint64_t t = 0;
    for (int l = 1; l <= L; l++)
        if (der[l]) t |= 1ull << (l - 1);
    auto in = [&](int l) { return l >= 1 && ((t >> (l - 1)) & 1ull); };
    auto drop = [&](int l) { if (l >= 1) t &= ~(1ull << (l - 1)); };
    for (bool changed = true; changed;) {
        const uint64_t before = t;
        for (int q = 0; q < R; q++) {
            const int A = rules[3 * q], B = rules[3 * q + 1], C = rules[3 * q + 2];
            if (B && C) {
                if (der[C]) { drop(A); drop(B); drop(C); }
                else if (in(A) != in(B)) { drop(A); drop(B); }
            } else if (B) {
                if (in(B) && !in(A)) drop(B);
                if (in(A) && !in(B) && der[B]) drop(A);
            }
        }
        changed = t != before;
    }
    return t;
}

static void set_columns(RuleTable &rt, uint64_t tmask, int L)
{
    for (int l = 1; l <= L; l++) rt.tpose[l] = (uint8_t)((tmask >> (l - 1)) & 1ull);
}


// Join tuning (compile-time; -DGRG_... overrides for sweeps)
#ifndef GRG_JOIN_WARPS
#define GRG_JOIN_WARPS 4
#endif
#ifndef GRG_WIN
#define GRG_WIN 8
#endif
#ifndef GRG_WIN_LO
#define GRG_WIN_LO 3
#endif
#ifndef GRG_ACC_LG
#define GRG_ACC_LG 6
#endif
#ifndef GRG_JOIN_MINB
#define GRG_JOIN_MINB 6
#endif
#ifndef GRG_GATHER_GR
#define GRG_GATHER_GR 4           // delta records per thread per step of the gather's record pass
#endif
#ifndef GRG_RUN_PASSES
#define GRG_RUN_PASSES 1          // 1: a batch of more runs than window slots joins in passes, every run with a slot
#endif
#ifndef GRG_WIN_PRECHECK
#define GRG_WIN_PRECHECK 1        // items of derivable right-hand labels (2: of every label) OR only the
#endif                            // window words they add to (1M alias closure 230.6 -> 209.4 ms; 2M
                                  // dataflow closure 52.5 ms either way, 53.2 with every label)
#ifndef GRG_APPLY_MINB
#define GRG_APPLY_MINB 6          // k_apply blocks of 256 threads a SM (its grid: this many per SM); at 6
#endif                            // its 36 registers need no spills (8: 32 and spills; 2M dataflow closure
                                  // 53.0 / 53.2 ms at 8 against 52.3 / 52.3 at 6 on two boxes)
#ifndef GRG_JOIN_MINB_WIDE
#define GRG_JOIN_MINB_WIDE 8      // wide join blocks a SM: 8 at 64 registers (with spills) measured 51.3 /
#endif                            // 195.3 ms on the 2M dataflow / 1M alias closures against 52.5 / 207.7 at 7
#ifdef GRG_PHASE_TIMERS
#define PH_MARK(i)                                   \
    do {                                             \
        const long long t_ = clock64();              \
        ph[i] += (unsigned long long)(t_ - ph_t);    \
        ph_t = t_;                                   \
    } while (0)
#else
#define PH_MARK(i) do { } while (0)
#endif
constexpr int JOIN_WARPS = GRG_JOIN_WARPS;  // warps per join block
constexpr int RB = 32;            // delta records per warp batch (one per lane)
constexpr int WIN = GRG_WIN;      // dense accumulator window: elements base-WIN_LO .. base+WIN-1-WIN_LO
constexpr int WIN_LO = GRG_WIN_LO;
#ifndef GRG_WIN2
#define GRG_WIN2 12               // measured with 8 slots a warp (dataflow / alias, ms): 10 53.6 / 263.5,
#endif                            // 11 52.6 / 254.3, 12 52.5 / 250.9, 16 52.8 / 264.1
#ifndef GRG_WIN2_LO
#define GRG_WIN2_LO 5
#endif
constexpr int WIN2 = GRG_WIN2;    // wide window: rows whose destinations spread over many elements
constexpr int WIN2_LO = GRG_WIN2_LO;
constexpr int ACC_LG = GRG_ACC_LG;
#ifndef GRG_WIN_SLOTS
#define GRG_WIN_SLOTS 8
#endif
// dense windows per warp: one per run of a row's records; a batch of more runs joins in passes
// of NSLOT runs (measured, 2M-vertex dataflow / 1M alias closure: 16 slots 54.8 / 272.5 ms,
// 12 slots 53.4 / 269.7 ms, 8 slots 54.1 / 263.7 ms; 16 slots with runs past the 16th sent to
// the hash instead of a second pass: 53.9 / 311.5 ms)
constexpr int NSLOT = GRG_WIN_SLOTS;
constexpr uint32_t NO_SLOT = 0xFFu;
constexpr int ACC = 1 << ACC_LG;  // per-warp hash accumulator entries (candidates outside the window)
constexpr int ACC_MAX = ACC * 3 / 4;

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31; }

// ---------------------------------------------------------------- loader

__global__ void k_init_region(uint32_t *elems, uint32_t *dbits, uint32_t *stamp, uint64_t begin, uint64_t end)
{
    for (uint64_t s = begin + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < end;
         s += (uint64_t)gridDim.x * blockDim.x) {
        uint4 *e = reinterpret_cast<uint4 *>(elems + s * 8);
        e[0] = make_uint4(0, 0, 0, 0);
        e[1] = make_uint4(0, 0, EMPTY, 0);
        uint4 *b = reinterpret_cast<uint4 *>(dbits + s * 8);
        b[0] = make_uint4(0, 0, 0, 0);
        b[1] = make_uint4(0, 0, 0, 0);
        if (stamp) stamp[s] = 0;
    }
}

// Input ids are local to a vertex range starting at `base` (0 for a whole graph).
__global__ void k_fill_u32(uint32_t *p, uint64_t n, uint32_t v)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        p[i] = v;
}

// Input edges are checked where they are first read: a label outside 1..L or a
// vertex id outside [0, nv) is flagged and skipped here and in k_load_insert.
__device__ __forceinline__ bool edge_ok(Dev d, uint32_t s, uint32_t t, uint32_t l, uint32_t nv, uint32_t L, bool flag)
{
    if (l - 1u >= L) {
        if (flag) atomicOr(&d.ctr[C_BADIN], (unsigned long long)ERR_IN_LABEL);
        return false;
    }
    if (s >= nv || t >= nv) {
        if (flag) atomicOr(&d.ctr[C_BADIN], (unsigned long long)ERR_IN_RANGE);
        return false;
    }
    return true;
}

// tmask: labels stored by destination (bit l-1): their edges go to the table of
// the destination, as the source's bit.
__global__ void k_load_hist(Dev d, const uint32_t *src, const uint32_t *dst, const uint8_t *lab, uint64_t n,
                            uint32_t base, uint32_t nv, uint32_t L, unsigned long long tmask)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t s = src[i], t = dst[i], l = lab[i];
        if (!edge_ok(d, s, t, l, nv, L, true)) continue;
        const uint32_t row = ((tmask >> (l - 1)) & 1ull) ? t : s;
        atomicAdd(&d.cnt[(size_t)(l - 1) * d.V + base + row], 1u);
    }
}

__global__ void k_eps_hist(Dev d, uint32_t slot, uint32_t first, uint32_t nv)
{
    for (uint32_t v = first + blockIdx.x * blockDim.x + threadIdx.x; v < first + nv; v += gridDim.x * blockDim.x)
        atomicAdd(&d.cnt[(size_t)(slot - 1) * d.V + v], 1u);
}

// Minimum table capacity per label (0 = none): tables of labels that rules
// derive start large enough to rarely grow, so they stay in row order.
struct MinCap { uint32_t cap[MAX_LABELS + 1]; };

// One thread per table of labels 1..L over rows [first, first + nv): size from
// the edge histogram (held in cnt), bump-allocate. rowmark (nullable, 1 bit per
// row): the minimum capacities apply only to marked rows -- an element image
// holds a few partitions' rows, and rows it does not hold never gain edges.
__global__ void k_load_alloc(Dev d, uint32_t first, uint32_t nv, uint32_t L, MinCap mc,
                             const uint32_t *__restrict__ rowmark)
{
    const uint64_t ntables = (uint64_t)L * nv;
    for (uint64_t u = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; u < ((ntables + 31) & ~31ull);
         u += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t lab = u < ntables ? (uint32_t)(u / nv) + 1 : 1;
        const uint64_t t = (uint64_t)(lab - 1) * d.V + first + (u < ntables ? u % nv : 0);
        uint32_t h = u < ntables ? d.cnt[t] : 0;
        uint32_t cap = u < ntables ? mc.cap[lab] : 0;
        if (rowmark && cap) {
            const uint32_t row = first + (uint32_t)(u % nv);
            if (!((rowmark[row >> 5] >> (row & 31)) & 1u)) cap = 0;
        }
        if (h) {
            const uint32_t need = h + h / 3 + 1;
            if (cap < 4) cap = 4;
            while (cap < need) cap <<= 1;
        }
        // warp-aggregated bump allocation
        uint32_t incl = cap;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane_id() >= (uint32_t)o) incl += y;
        }
        uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
        unsigned long long base = 0;
        if (lane_id() == 31 && total) base = atomicAdd(&d.ctr[C_POOL_TOP], (unsigned long long)total);
        base = __shfl_sync(0xffffffffu, base, 31);
        if (u < ntables) {
            uint64_t off = base + incl - cap;
            if (cap && off + cap > d.pool_cap) {
                atomicOr(&d.ctr[C_ERR], (unsigned long long)ERR_POOL);
                cap = 0;
            }
            d.desc[t] = cap ? ((uint64_t)cap << 32) | (uint32_t)off : 0ull;
            d.cnt[t] = 0;
        }
    }
}

__global__ void k_load_insert(Dev d, const uint32_t *src, const uint32_t *dst, const uint8_t *lab, uint64_t n,
                              uint32_t vbase, uint32_t nv, uint32_t L, unsigned long long tmask)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t l = lab[i];
        if (!edge_ok(d, src[i], dst[i], l, nv, L, false)) continue;
        const bool by_dst = (tmask >> (l - 1)) & 1ull;
        const uint32_t row = vbase + (by_dst ? dst[i] : src[i]);
        const uint32_t v = vbase + (by_dst ? src[i] : dst[i]);
        Bits b;
        const uint32_t o = v % EIDS;
#pragma unroll
        for (int w = 0; w < EW; w++) b.w[w] = (uint32_t)w == (o >> 5) ? 1u << (o & 31) : 0u;
        if (!g_insert(d, l, row, v / EIDS, b, false)) atomicOr(&d.ctr[C_ERR], (unsigned long long)ERR_LOAD);
    }
}

// Epsilon rules A ::= eps: (v, v, A) for every vertex (compute00, src/kernel.cu:445-464).
__global__ void k_eps_insert(Dev d, uint32_t slot, uint32_t first, uint32_t nv)
{
    for (uint32_t v = first + blockIdx.x * blockDim.x + threadIdx.x; v < first + nv; v += gridDim.x * blockDim.x) {
        Bits b;
        const uint32_t o = v % EIDS;
#pragma unroll
        for (int w = 0; w < EW; w++) b.w[w] = (uint32_t)w == (o >> 5) ? 1u << (o & 31) : 0u;
        if (!g_insert(d, slot, v, v / EIDS, b, false)) atomicOr(&d.ctr[C_ERR], (unsigned long long)ERR_LOAD);
    }
}

// Rows of labels that are never inserted into after the load are packed:
// occupied slots moved to the front, capacity = count (no empty slots to scan).
__global__ void k_compact_static(Dev d, uint32_t slot, uint32_t first, uint32_t nv)
{
    for (uint32_t v = first + blockIdx.x * blockDim.x + threadIdx.x; v < first + nv; v += gridDim.x * blockDim.x) {
        const size_t ti = (size_t)(slot - 1) * d.V + v;
        const uint64_t de = d.desc[ti];
        const uint32_t off = (uint32_t)de, cap = (uint32_t)(de >> 32);
        if (!cap) continue;
        uint32_t wpos = 0;
        for (uint32_t j = 0; j < cap; j++) {
            uint4 *e = reinterpret_cast<uint4 *>(d.elems + (size_t)(off + j) * 8);
            uint4 e1 = e[1];
            if (e1.z == EMPTY) continue;
            if (j != wpos) {
                const uint64_t os = (uint64_t)off + j, ns = (uint64_t)off + wpos;
                uint4 *t = reinterpret_cast<uint4 *>(d.elems + ns * 8);
                t[0] = e[0];
                t[1] = e1;
                e[0] = make_uint4(0, 0, 0, 0);
                e[1] = make_uint4(0, 0, EMPTY, 0);
                if (d.stamp) d.stamp[ns] = d.stamp[os];
                // a delta mark set at the load (element images) moves with its element
                if ((d.dmap[os >> 5] >> (os & 31)) & 1u) {
                    uint4 *ob = reinterpret_cast<uint4 *>(d.dbits + os * 8);
                    uint4 *nbp = reinterpret_cast<uint4 *>(d.dbits + ns * 8);
                    nbp[0] = ob[0];
                    nbp[1] = ob[1];
                    ob[0] = make_uint4(0, 0, 0, 0);
                    ob[1] = make_uint4(0, 0, 0, 0);
                    atomicAnd(&d.dmap[os >> 5], ~(1u << (os & 31)));
                    atomicOr(&d.dmap[ns >> 5], 1u << (ns & 31));
                }
                reinterpret_cast<uint2 *>(d.dbits + ns * 8)[3] = make_uint2(e1.z, e1.w);
            }
            wpos++;
        }
        d.desc[ti] = wpos ? ((uint64_t)wpos << 32) | off : 0ull;
        d.cnt[ti] = wpos;
    }
}

// Every loaded element of a tracked label becomes a delta of round 1. A warp
// covers 32 consecutive slots, so it owns one dirty-bitmap word.
__global__ void k_mark_all(Dev d, uint64_t begin, uint64_t end)   // begin: multiple of 32
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t b0 = begin + blockIdx.x * (uint64_t)blockDim.x + (threadIdx.x & ~31u); b0 < end; b0 += stride) {
        const uint64_t s = b0 + lane_id();
        bool mark = false;
        if (s < end) {
            const uint4 *e = reinterpret_cast<const uint4 *>(d.elems + s * 8);
            const uint4 e1 = e[1];
            if (e1.z != EMPTY && d.rt.track[e1.z >> KEY_SHIFT]) {
                const uint4 e0 = e[0];
                uint4 *b = reinterpret_cast<uint4 *>(d.dbits + s * 8);
                b[0] = e0;
                b[1] = e1;                 // words 6-7: key and row
                mark = true;
            }
        }
        const unsigned m = __ballot_sync(0xffffffffu, mark);
        if (lane_id() == 0) d.dmap[b0 >> 5] = m;
    }
}

// ---------------------------------------------------------------- rounds

// Dirty records per chunk of 1024 slots (one warp per chunk of 32 bitmap words).
// Dirty-bitmap words below the pool top. Launches recorded once and replayed
// (round graphs, dyn != 0) read the top from the device counter, bounded by
// nwords = the words the buffers were sized for; others get the host's figure.
__device__ __forceinline__ uint64_t dyn_words(uint64_t nwords, const unsigned long long *ctr, int dyn)
{
    return dyn ? min(nwords, (uint64_t)(ctr[C_POOL_TOP] + 31) / 32) : nwords;
}

__global__ void k_dcount(Dev d, uint64_t nwords, uint32_t *chunk_cnt, int dyn)
{
    if (d.ctr[C_HALT]) return;
    nwords = dyn_words(nwords, d.ctr, dyn);
    const uint64_t nchunks = (nwords + 31) / 32;
    const uint64_t nwarps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for (uint64_t c = blockIdx.x * (uint64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); c < nchunks; c += nwarps) {
        const uint64_t wi = c * 32 + lane_id();
        uint32_t n = wi < nwords ? __popc(d.dmap[wi]) : 0;
        for (int o = 16; o; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
        if (lane_id() == 0) chunk_cnt[c] = n;
    }
}

// Position of the n-th (0-based) set bit of a 32-bit word (broadword select, no loop).
__device__ __forceinline__ uint32_t select32(uint32_t w, uint32_t n)
{
    uint32_t pos = 0, c;
    c = __popc(w & 0xFFFFu); if (n >= c) { n -= c; pos += 16; w >>= 16; }
    c = __popc(w & 0xFFu);   if (n >= c) { n -= c; pos += 8;  w >>= 8; }
    c = __popc(w & 0xFu);    if (n >= c) { n -= c; pos += 4;  w >>= 4; }
    c = __popc(w & 0x3u);    if (n >= c) { n -= c; pos += 2;  w >>= 2; }
    c = w & 1u;              if (n >= c) { pos += 1; }
    return pos;
}

// Dirty slots -> delta records (32 B: bits[6], key, row) in slot order at the
// chunk offsets; clears the delta bitmaps and the dirty bitmap. One warp per
// chunk of 32 bitmap words; lanes take consecutive dirty slots of the chunk, so
// the copies of a warp are independent and mostly coalesced.
// Gather, pass 1: the dirty slots of the round, in slot order (a table's
// records stay contiguous), as a dense array of slot ids; the dirty bits are
// cleared. Lanes walk their own bitmap word: stores only, nothing to wait for.
__global__ void k_gather_slots(Dev d, uint64_t nwords, const uint32_t *__restrict__ chunk_off, uint32_t *slots,
                               int dyn)
{
    if (d.ctr[C_HALT]) return;
    nwords = dyn_words(nwords, d.ctr, dyn);
    const uint64_t nchunks = (nwords + 31) / 32;
    const uint64_t nwarps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    const uint32_t lane = lane_id();
    for (uint64_t c = blockIdx.x * (uint64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); c < nchunks; c += nwarps) {
        const uint64_t wi = c * 32 + lane;
        uint32_t m = wi < nwords ? d.dmap[wi] : 0;
        const uint64_t base_pos = chunk_off[c];
        const uint32_t cnt = __popc(m);
        uint32_t incl = cnt;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= (uint32_t)o) incl += y;
        }
        if (m) d.dmap[wi] = 0;
        uint32_t *sp = slots + base_pos + incl - cnt;
        while (m) {
            *sp++ = (uint32_t)(wi * 32 + (__ffs(m) - 1));
            m &= m - 1;
        }
    }
}

// Gather, pass 2: one thread per record. The slot's delta bitmap (words 0-5:
// bits new since the last gather; 6-7: the slot's key and row) becomes the
// record and is cleared; the delta index and per-job counts are filled.
// n_ctr >= 0: the record count is device counter n_ctr (round graphs).
__global__ void k_gather_recs(Dev d, const uint32_t *__restrict__ slots, uint4 *out, uint64_t n, int n_ctr,
                              const uint32_t *__restrict__ row_job, uint32_t *job_cnt, uint32_t run_stamp)
{
    if (d.ctr[C_HALT]) return;
    if (n_ctr >= 0) n = d.ctr[n_ctr];
    // GR records per thread per step, their random delta reads issued together
    constexpr int GR = GRG_GATHER_GR;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i0 < n; i0 += stride * GR) {
        uint64_t sl[GR];
        uint4 b0[GR], b1[GR];
#pragma unroll
        for (int u = 0; u < GR; u++) {
            const uint64_t i = i0 + u * stride;
            sl[u] = i < n ? slots[i] : 0;
        }
#pragma unroll
        for (int u = 0; u < GR; u++) {
            if (i0 + u * stride < n) ld32(d.dbits + sl[u] * 8, b0[u], b1[u]);
        }
#pragma unroll
        for (int u = 0; u < GR; u++) {
            const uint64_t i = i0 + u * stride;
            if (i >= n) continue;
            const uint64_t s = sl[u];
            // words 0-5 cleared; 6-7 keep the slot's key and row
            st32(d.dbits + s * 8, make_uint4(0, 0, 0, 0), make_uint4(0, 0, b1[u].z, b1[u].w));
            if (run_stamp) d.stamp[s] = run_stamp;     // gained bits during this run
            st32(out + 2 * i, b0[u], b1[u]);
            const uint32_t lab = b1[u].z >> KEY_SHIFT, row = b1[u].w;
            if (lab <= (uint32_t)MAX_LABELS && d.rt.dindex[lab]) {
                const size_t ti = (size_t)(lab - 1) * d.V + row;
                atomicMin(&d.drs[ti], (uint32_t)i);
                atomicAdd(&d.drc[ti], 1u);
                atomicOr(&d.dvm[(size_t)(lab - 1) * d.vwords + (row >> 5)], 1u << (row & 31));
            }
            if (row_job) {
                // batched jobs: records per job (a job with none has reached its fixpoint)
                const uint32_t job = row_job[row];
                const unsigned act = __activemask();
                const unsigned g = __match_any_sync(act, job);
                if (job != EMPTY && lane_id() == (uint32_t)(__ffs(g) - 1)) atomicAdd(&job_cnt[job], (uint32_t)__popc(g));
            }
        }
    }
}

// Device-driven rounds: clear the delta index entries the previous round's gather
// set (its records are still in recs, n_ctr counts them), instead of clearing
// every vertex.
__global__ void k_dindex_clear(Dev d, const uint4 *__restrict__ recs, int n_ctr)
{
    if (d.ctr[C_HALT]) return;
    const uint64_t n = d.ctr[n_ctr];
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint4 b1 = recs[2 * i + 1];
        const uint32_t lab = b1.z >> KEY_SHIFT, row = b1.w;
        if (lab > (uint32_t)MAX_LABELS || !d.rt.dindex[lab]) continue;
        const size_t ti = (size_t)(lab - 1) * d.V + row;
        d.drs[ti] = EMPTY;
        d.drc[ti] = 0;
        d.dvm[(size_t)(lab - 1) * d.vwords + (row >> 5)] = 0;
    }
}

// Old-left join q (A ::= B C, C derivable): every element of every row of B,
// masked to the vertices k whose row C[k] has deltas this round, becomes a
// virtual delta record (label slot OL_SLOT0 + q). The 192 ids of an element are
// exactly 6 words of the dirty-vertex bitmap. Records past cap are counted only.
__global__ void k_oldleft(Dev d, uint32_t q, uint4 *out, uint64_t cap, const uint32_t *__restrict__ row_job,
                          const uint32_t *__restrict__ job_cnt)
{
    if (d.ctr[C_HALT]) return;
    const uint32_t B = d.rt.ol_B[q], C = d.rt.ol_C[q];
    const uint32_t *dv = d.dvm + (size_t)(C - 1) * d.vwords;
    const uint32_t vkey = (OL_SLOT0 + q) << KEY_SHIFT;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t b0 = blockIdx.x * (uint64_t)blockDim.x + (threadIdx.x & ~31u); b0 < d.V; b0 += stride) {
        const uint64_t v = b0 + lane_id();
        const uint64_t de = v < d.V ? d.desc[(size_t)(B - 1) * d.V + v] : 0ull;
        const uint32_t off = (uint32_t)de;
        uint32_t cap_v = (uint32_t)(de >> 32);
        if (v < d.V && prefix_table(d, B, cap_v)) cap_v = min(cap_v, d.cnt[(size_t)(B - 1) * d.V + v]);
        // batched jobs: a job without delta records this round adds no virtual records
        if (row_job && cap_v) {
            const uint32_t job = row_job[v];
            if (job == EMPTY || job_cnt[job] == 0) cap_v = 0;
        }
        const uint32_t maxc = __reduce_max_sync(0xffffffffu, cap_v);
        for (uint32_t j = 0; j < maxc; j++) {
            Bits m;
            uint32_t any = 0, base = 0;
            if (j < cap_v) {
                const uint4 *e = reinterpret_cast<const uint4 *>(d.elems + (size_t)(off + j) * 8);
                const uint4 e0 = e[0], e1 = e[1];
                if (e1.z != EMPTY) {
                    base = e1.z & BASE_MASK;
                    const uint64_t w0 = (uint64_t)base * EW;
                    const uint32_t ew[EW] = {e0.x, e0.y, e0.z, e0.w, e1.x, e1.y};
#pragma unroll
                    for (int x = 0; x < EW; x++) {
                        m.w[x] = (w0 + x < d.vwords) ? ew[x] & __ldg(dv + w0 + x) : 0u;
                        any |= m.w[x];
                    }
                }
            }
            const unsigned em = __ballot_sync(0xffffffffu, any != 0);
            if (!em) continue;
            unsigned long long p0 = 0;
            const int leader = __ffs(em) - 1;
            if ((int)lane_id() == leader) p0 = atomicAdd(&d.ctr[C_VN], (unsigned long long)__popc(em));
            p0 = __shfl_sync(0xffffffffu, p0, leader);
            if (any) {
                const uint64_t p = p0 + __popc(em & ((1u << lane_id()) - 1u));
                if (p < cap) {
                    out[2 * p] = make_uint4(m.w[0], m.w[1], m.w[2], m.w[3]);
                    out[2 * p + 1] = make_uint4(m.w[4], m.w[5], vkey | base, (uint32_t)v);
                }
            }
        }
    }
}

// Per-warp shared memory of the join, for a dense window of W elements per
// record covering bases rbase-LO .. rbase+W-1-LO.
template <int W, int LO>
struct __align__(16) WarpSmemT {
    static constexpr int kWin = W, kLo = LO;
    uint32_t win[NSLOT][W][EW];   // dense window accumulators, one per run of a row's records
    uint32_t slot_rec[NSLOT];     // the first record of each window's run
    uint32_t acc_bits[ACC][EW];   // hash accumulator: OR of candidate bitmaps
    uint32_t acc_key[ACC];        // key = record << 25 | base (EMPTY = free)
    uint32_t rbits[RB][EW];       // the batch's delta records
    uint32_t rrow[RB];
    uint32_t rbase[RB];
    uint32_t rA[RB];              // per record: output label of the current rule pass
    uint32_t rpk[RB];             // per record, packed: the first record of its run with the same row
                                  // and label (bits 0-7), the current rule's right operand label
                                  // (8-15), where that label's rows come from (16-23: 0 tables, 1 CSR
                                  // copy, 2 delta records of a virtual old-left record; +4 when its
                                  // items pre-check the window) and the run's window slot (24-31,
                                  // NO_SLOT: the hash only)
    uint32_t kpre[RB + 1];        // exclusive prefix of per-record task counts
    uint8_t own[32];              // per chunk of 32 tasks (items): lane whose record (task) starts there
    uint32_t acc_n;
    uint32_t fail;                // records with a failed insert (retry after growth)
};

// One right-hand item of a join, loaded: ok (an occupied element or an id), its base,
// the id within the element (EMPTY for an element) and the element's bits.
struct Item {
    bool ok;
    uint32_t b2, ob;
    Bits ib;
};

__device__ __forceinline__ uint32_t popc6(const Bits &b)
{
    uint32_t c = 0;
#pragma unroll
    for (int x = 0; x < EW; x++) c += __popc(b.w[x]);
    return c;
}

// Position (0..191) of the idx-th set bit of a record's bitmap in shared memory.
__device__ __forceinline__ uint32_t select_bit(const uint32_t *bits, uint32_t idx)
{
    uint32_t pos = 0, wsel = 0, found = 0;
#pragma unroll
    for (int x = 0; x < EW; x++) {
        const uint32_t bw = bits[x];
        const uint32_t c = __popc(bw);
        const bool here = !found && idx < c;
        if (here) { wsel = bw; pos = x * 32; found = 1; }
        else if (!found) idx -= c;
    }
    return pos + select32(wsel, idx);
}

// Exclusive warp prefix of per-lane task counts into kpre[0..RB]; returns the total.
template <class WS>
__device__ __forceinline__ uint32_t warp_tasks(WS &w, uint32_t cnt)
{
    const uint32_t lane = lane_id();
    uint32_t incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (uint32_t)o) incl += y;
    }
    w.kpre[lane] = incl - cnt;
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    if (lane == 31) w.kpre[RB] = total;
    __syncwarp();
    return total;
}

// Owner of position `lane` of a chunk of 32 flattened tasks (or items): every
// lane whose run of positions starts in the chunk (starts, at offset pos) marks
// it; a position belongs to the highest mark at or below it, or to `carry`
// (the owner running into the chunk) when there is none. carry is updated to
// the owner of the chunk's last position. Warp-uniform; one OR-reduction and
// one shared-memory read instead of a 5-step dependent search.
template <class WS>
__device__ __forceinline__ uint32_t chunk_owner(WS &w, bool starts, uint32_t pos, uint32_t &carry)
{
    const uint32_t lane = lane_id();
    if (starts) w.own[pos] = (uint8_t)lane;
    const uint32_t m = __reduce_or_sync(0xffffffffu, starts ? 1u << pos : 0u);
    __syncwarp();
    const uint32_t below = m & (0xFFFFFFFFu >> (31 - lane));
    const uint32_t o = below ? w.own[31 - __clz(below)] : carry;
    const uint32_t last = m ? w.own[31 - __clz(m)] : carry;
    __syncwarp();
    carry = last;
    return o;
}

// OR (key, b) into the warp's hash accumulator; false when it is full.
template <class WS>
__device__ __forceinline__ bool acc_insert(WS &w, uint32_t key, const Bits b)
{
    volatile uint32_t *keys = w.acc_key;
    const uint32_t h = (key * 0x9E3779B1u) >> (32 - ACC_LG);
    for (int p = 0; p < ACC; p++) {
        const uint32_t q = (h + p) & (ACC - 1);
        const uint32_t k = keys[q];
        if (k == key) {
#pragma unroll
            for (int x = 0; x < EW; x++)
                if (b.w[x]) atomicOr(&w.acc_bits[q][x], b.w[x]);
            return true;
        }
        if (k != EMPTY) continue;
        if (atomicAdd(&w.acc_n, 1u) >= (uint32_t)ACC_MAX) {
            atomicSub(&w.acc_n, 1u);
            return false;
        }
        const uint32_t prev = atomicCAS(&w.acc_key[q], EMPTY, key);
        if (prev != EMPTY) atomicSub(&w.acc_n, 1u);
        if (prev == EMPTY || prev == key) {
#pragma unroll
            for (int x = 0; x < EW; x++)
                if (b.w[x]) atomicOr(&w.acc_bits[q][x], b.w[x]);
            return true;
        }
    }
    return false;
}

// Reserve cnt candidate slots per lane (warp-uniform). Returns the lane's first
// slot, or ~0 for every lane when the buffer cannot take the warp's total (the
// caller then inserts directly); slots of a reservation that straddles the end
// of the buffer are filled with empty records.
__device__ __forceinline__ uint64_t cand_reserve(const Dev &d, uint32_t cnt)
{
    const uint32_t lane = lane_id();
    uint32_t incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (uint32_t)o) incl += y;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    if (!total || !d.cand) return d.cand ? 0 : ~0ull;
    unsigned long long base = 0;
    if (lane == 31) base = atomicAdd(&d.ctr[C_CAND_N], (unsigned long long)total);
    base = __shfl_sync(0xffffffffu, base, 31);
    if (base + total <= d.cand_cap) return base + incl - cnt;
    for (uint64_t i = base + incl - cnt; i < base + incl && i < d.cand_cap; i++) {
        d.cand[2 * i] = make_uint4(0, 0, 0, 0);
        d.cand[2 * i + 1] = make_uint4(0, 0, EMPTY, 0);
    }
    return ~0ull;
}

__device__ __forceinline__ void cand_write(const Dev &d, uint64_t i, const Bits &b, uint32_t key, uint32_t row)
{
    st32(d.cand + 2 * i, make_uint4(b.w[0], b.w[1], b.w[2], b.w[3]), make_uint4(b.w[4], b.w[5], key, row));
}

// Flush the hash accumulator: entry (r, base) goes to row (rA[r], rrow[r]),
// as a candidate for k_apply or, when the candidate buffer is full, by a
// direct insert. Warp-uniform.
template <class WS>
__device__ __forceinline__ void acc_flush(const Dev &d, WS &w, uint32_t &inserts)
{
    __syncwarp();
    uint32_t nz = 0;
#pragma unroll
    for (int it = 0; it < ACC / 32; it++)
        if (w.acc_key[it * 32 + lane_id()] != EMPTY) nz |= 1u << it;
    uint64_t ci = cand_reserve(d, __popc(nz));
#pragma unroll 1
    for (int it = 0; it < ACC / 32; it++) {
        const int j = it * 32 + (int)lane_id();
        const uint32_t k = w.acc_key[j];
        if (k != EMPTY) {
            Bits b;
#pragma unroll
            for (int x = 0; x < EW; x++) { b.w[x] = w.acc_bits[j][x]; w.acc_bits[j][x] = 0; }
            w.acc_key[j] = EMPTY;
            const uint32_t r = k >> KEY_SHIFT, A = w.rA[r];
            if (ci != ~0ull) {
                cand_write(d, ci++, b, (A << KEY_SHIFT) | (k & BASE_MASK), w.rrow[r]);
            } else {
                if (!g_insert(d, A, w.rrow[r], k & BASE_MASK, b, d.rt.track[A])) atomicOr(&w.fail, 1u << r);
                inserts++;
            }
        }
    }
    __syncwarp();
    if (lane_id() == 0) w.acc_n = 0;
    __syncwarp();
}

// Flush every record's window into row (rA[r], rrow[r]) and clear it. Warp-uniform.
template <class WS>
__device__ __forceinline__ void win_flush(const Dev &d, WS &w, uint32_t &inserts)
{
    constexpr int WIN = WS::kWin, WIN_LO = WS::kLo;
    constexpr int NPOS = (NSLOT * WIN + 31) / 32;
    __syncwarp();
    uint32_t nz = 0;
#pragma unroll
    for (int it = 0; it < NPOS; it++) {
        const uint32_t p = it * 32 + lane_id();
        if (p >= (uint32_t)(NSLOT * WIN)) continue;
        const uint32_t sl = p / WIN, dd = p % WIN;
        uint32_t any = 0;
#pragma unroll
        for (int x = 0; x < EW; x++) any |= w.win[sl][dd][x];
        if (any) nz |= 1u << it;
    }
    uint64_t ci = cand_reserve(d, __popc(nz));
#pragma unroll 1
    for (int it = 0; it < NPOS; it++) {
        const uint32_t p = it * 32 + lane_id();
        const uint32_t sl = p / WIN, dd = p % WIN;
        if ((nz >> it) & 1u) {
            const uint32_t r = w.slot_rec[sl];
            Bits b;
#pragma unroll
            for (int x = 0; x < EW; x++) { b.w[x] = w.win[sl][dd][x]; w.win[sl][dd][x] = 0; }
            const uint32_t A = w.rA[r], base = w.rbase[r] + dd - WIN_LO;
            if (ci != ~0ull) {
                cand_write(d, ci++, b, (A << KEY_SHIFT) | base, w.rrow[r]);
            } else {
                if (!g_insert(d, A, w.rrow[r], base, b, d.rt.track[A])) atomicOr(&w.fail, 1u << r);
                inserts++;
            }
        }
    }
    __syncwarp();
}

// Insert candidate elements (label, row, base, bits) written by k_join. One
// thread per candidate: thousands of independent insert chains per SM.
// Candidates whose table is full go to fail_out (C_AFAIL) for a retry after growth.
__global__ void __launch_bounds__(256, GRG_APPLY_MINB) k_apply(Dev d, const uint4 *__restrict__ cand, uint4 *fail_out)
{
    if (d.ctr[C_HALT]) return;
    // the candidate count is read on the device, so the host need not wait for the join
    const uint64_t n = min((uint64_t)d.ctr[C_CAND_N], d.cand_cap);
    if (blockIdx.x == 0 && threadIdx.x == 0 && n) atomicAdd(&d.ctr[C_CANDS], (unsigned long long)n);
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        uint4 a, b;
        ld32(cand + 2 * i, a, b);
        if (b.z == EMPTY) continue;
        Bits bits;
        bits.w[0] = a.x; bits.w[1] = a.y; bits.w[2] = a.z; bits.w[3] = a.w; bits.w[4] = b.x; bits.w[5] = b.y;
        const uint32_t A = b.z >> KEY_SHIFT;
        if (!g_insert_t<true>(d, A, b.w, b.z & BASE_MASK, bits, d.rt.track[A])) {
            const unsigned long long f = atomicAdd(&d.ctr[C_AFAIL], 1ull);
            fail_out[2 * f] = a;
            fail_out[2 * f + 1] = b;
        }
    }
}

// Delta records of labels stored by destination (RuleTable::tpose). A record
// (label B, column k, base, bits = sources i of new edges (i, k)) is pushed
// whole: a unary rule A ::= B puts it into A's column k, a binary rule A ::= B C
// into A's column j for every edge (k, j) of C (C's CSR copy, or its table
// elements by source) -- one element insert per edge of C, for up to 192
// sources at once. The kernel also turns around the records of a label stored
// by source that a unary rule A ::= B copies into a destination-stored A (B's
// loaded edges, in round 1): one single-bit insert per edge. One thread per
// record; a record with an insert into a full table goes to the retry list,
// as in k_join (pushing a record again adds nothing twice).
// n_ctr >= 0: the record count is device counter n_ctr (round graphs).
__global__ void __launch_bounds__(256, 4) k_push(Dev d, const uint4 *__restrict__ recs, uint64_t n, int n_ctr,
                                                  uint4 *retry_out)
{
    if (d.ctr[C_HALT]) return;
    if (n_ctr >= 0) n = d.ctr[n_ctr];
    unsigned long long n_left = 0, n_right = 0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    // i0 is the same for every thread of a block, so each warp runs the ballot together
    for (uint64_t i0 = blockIdx.x * (uint64_t)blockDim.x; i0 < n; i0 += stride) {
        const uint64_t i = i0 + threadIdx.x;
        bool failed = false;
        uint4 a = make_uint4(0, 0, 0, 0), b = make_uint4(0, 0, EMPTY, 0);
        if (i < n) {
            a = recs[2 * i];
            b = recs[2 * i + 1];
        }
        const uint32_t B = b.z >> KEY_SHIFT, base = b.z & BASE_MASK, row = b.w;
        bool valid = i < n && B >= 1 && B <= (uint32_t)d.rt.L;
        if (valid && (row >= d.V || (uint64_t)base * EIDS >= d.V)) valid = !check_failed(d.ctr, 1, row);
        if (valid) {
            Bits bits;
            bits.w[0] = a.x; bits.w[1] = a.y; bits.w[2] = a.z; bits.w[3] = a.w; bits.w[4] = b.x; bits.w[5] = b.y;
            bool ok = true;
            if (d.rt.tpose[B]) {
                for (uint32_t u = d.rt.un_start[B]; u < d.rt.un_start[B + 1]; u++) {
                    const uint32_t A = d.rt.un_A[u];
                    ok &= g_insert_t<true>(d, A, row, base, bits, d.rt.track[A]);
                }
                for (uint32_t q = d.rt.bin_start[B]; q < d.rt.bin_start[B + 1]; q++) {
                    const uint32_t A = d.rt.bin_A[q], C = d.rt.bin_C[q];
                    const bool tr = d.rt.track[A];
                    n_left++;
                    const uint2 *cr = d.rt.csr_row[C];
                    if (cr) {
                        const uint2 rw = __ldg(cr + row);
                        const uint32_t *col = d.rt.csr_col[C] + rw.x;
                        uint32_t cnt = rw.y & 0xFFFFFFu;
                        if ((uint64_t)rw.x + cnt > d.rt.csr_n[C]) cnt = check_failed(d.ctr, 5, rw.x) ? 0 : cnt;
                        n_right += cnt;
                        for (uint32_t t = 0; t < cnt; t++) {
                            const uint32_t j = __ldg(col + t);
                            if (j >= d.V || A < 1 || A > (uint32_t)d.rt.L) { check_failed(d.ctr, 7, j); continue; }
                            ok &= g_insert_t<true>(d, A, j, base, bits, tr);
                        }
                    } else {
                        const size_t ti = (size_t)(C - 1) * d.V + row;
                        const uint64_t de = __ldg(d.desc + ti);
                        const uint32_t off = (uint32_t)de;
                        uint32_t cap = (uint32_t)(de >> 32);
                        if (prefix_table(d, C, cap)) cap = min(cap, __ldcg(d.cnt + ti));
                        if ((uint64_t)off + cap > d.pool_cap) cap = check_failed(d.ctr, 2, off) ? 0 : cap;
                        for (uint32_t t = 0; t < cap; t++) {
                            const uint32_t *e = d.elems + (size_t)(off + t) * 8;
                            const uint32_t ek = __ldcg(e + 6);
                            if (ek == EMPTY) continue;
                            const uint32_t eb = (ek & BASE_MASK) * EIDS;
#pragma unroll 1
                            for (int x = 0; x < EW; x++) {
                                uint32_t w = __ldcg(e + x);
                                while (w) {
                                    const uint32_t j = eb + x * 32 + (__ffs(w) - 1);
                                    w &= w - 1;
                                    n_right++;
                                    if (j >= d.V) { check_failed(d.ctr, 3, j); continue; }
                                    ok &= g_insert_t<true>(d, A, j, base, bits, tr);
                                }
                            }
                        }
                    }
                }
            } else {
                for (uint32_t u = d.rt.un_start[B]; u < d.rt.un_start[B + 1]; u++) {
                    const uint32_t A = d.rt.un_A[u];
                    if (!d.rt.tpose[A]) continue;
                    Bits one;
                    const uint32_t o = row % EIDS;
#pragma unroll
                    for (int x = 0; x < EW; x++) one.w[x] = (uint32_t)x == (o >> 5) ? 1u << (o & 31) : 0u;
#pragma unroll 1
                    for (int x = 0; x < EW; x++) {
                        uint32_t w = bits.w[x];
                        while (w) {
                            const uint32_t j = base * EIDS + x * 32 + (__ffs(w) - 1);
                            w &= w - 1;
                            if (j >= d.V) { check_failed(d.ctr, 4, j); continue; }
                            ok &= g_insert(d, A, j, row / EIDS, one, d.rt.track[A]);
                        }
                    }
                }
            }
            failed = !ok;
        }
        const unsigned fm = __ballot_sync(0xffffffffu, failed);
        if (fm) {
            const uint32_t lane = lane_id();
            unsigned long long p = 0;
            if (lane == (uint32_t)(__ffs(fm) - 1)) p = atomicAdd(&d.ctr[C_RETRY_N], (unsigned long long)__popc(fm));
            p = __shfl_sync(0xffffffffu, p, __ffs(fm) - 1);
            const uint64_t o = p + __popc(fm & ((1u << lane) - 1u));
            if (failed && o < d.retry_cap) {
                retry_out[2 * o] = a;
                retry_out[2 * o + 1] = b;
            }
        }
    }
    for (int o = 16; o; o >>= 1) {
        n_left += __shfl_xor_sync(0xffffffffu, n_left, o);
        n_right += __shfl_xor_sync(0xffffffffu, n_right, o);
    }
    if (lane_id() == 0) {
        if (n_left) atomicAdd(&d.ctr[C_LEFT], n_left);
        if (n_right) atomicAdd(&d.ctr[C_RIGHT], n_right);
    }
}

// k_push with the pushes along CSR rows flattened over the lanes: a warp takes
// 32 records, and the edges of C that their binary rules walk are dealt out
// one per lane, so a record whose row of C is long (Zipf-distributed degrees)
// does not hold its warp while the other lanes idle. Each lane takes its edge's
// record (output label, base, bits) from the record's lane. Everything else --
// unary rules, C without a CSR copy, records turned around for a unary rule --
// stays in the record's own lane, as in k_push. Same results, same retry list.
constexpr int PUSH_WARPS = 8;
__global__ void __launch_bounds__(PUSH_WARPS * 32, 4) k_push_flat(Dev d, const uint4 *__restrict__ recs, uint64_t n,
                                                                  int n_ctr, uint4 *retry_out)
{
    if (d.ctr[C_HALT]) return;
    if (n_ctr >= 0) n = d.ctr[n_ctr];
    __shared__ uint8_t own_s[PUSH_WARPS][32];
    __shared__ uint32_t fail_s[PUSH_WARPS];
    const uint32_t lane = lane_id(), wi = threadIdx.x >> 5;
    uint8_t *own = own_s[wi];
    unsigned long long n_left = 0, n_right = 0;
    // warps pull batches of 32 records from the launch's device queue (C_JQ, zeroed before it)
    const uint64_t nbatch = (n + 31) / 32;
    uint64_t bt = 0;
    if (lane == 0) bt = atomicAdd(&d.ctr[C_JQ], 1ull);
    bt = __shfl_sync(0xffffffffu, bt, 0);
    for (; bt < nbatch; bt = __shfl_sync(0xffffffffu, lane == 0 ? atomicAdd(&d.ctr[C_JQ], 1ull) : 0ull, 0)) {
        const uint64_t i = bt * 32 + lane;
        const bool have = i < n;
        uint4 a = make_uint4(0, 0, 0, 0), b = make_uint4(0, 0, EMPTY, 0);
        if (have) {
            a = recs[2 * i];
            b = recs[2 * i + 1];
        }
        if (lane == 0) fail_s[wi] = 0;
        __syncwarp();
        const uint32_t B = b.z >> KEY_SHIFT, base = b.z & BASE_MASK, row = b.w;
        bool valid = have && B >= 1 && B <= (uint32_t)d.rt.L;
        if (valid && (row >= d.V || (uint64_t)base * EIDS >= d.V)) valid = !check_failed(d.ctr, 1, row);
        const bool col = valid && d.rt.tpose[B];
        Bits bits;
        bits.w[0] = a.x; bits.w[1] = a.y; bits.w[2] = a.z; bits.w[3] = a.w; bits.w[4] = b.x; bits.w[5] = b.y;
        bool ok = true;
        // the record's own lane: everything but pushes along CSR rows
        if (col) {
            for (uint32_t u = d.rt.un_start[B]; u < d.rt.un_start[B + 1]; u++) {
                const uint32_t A = d.rt.un_A[u];
                ok &= g_insert_t<true>(d, A, row, base, bits, d.rt.track[A]);
            }
            for (uint32_t q = d.rt.bin_start[B]; q < d.rt.bin_start[B + 1]; q++) {
                const uint32_t A = d.rt.bin_A[q], C = d.rt.bin_C[q];
                if (d.rt.csr_row[C]) continue;
                n_left++;
                const size_t ti = (size_t)(C - 1) * d.V + row;
                const uint64_t de = __ldg(d.desc + ti);
                const uint32_t off = (uint32_t)de;
                uint32_t cap = (uint32_t)(de >> 32);
                if (prefix_table(d, C, cap)) cap = min(cap, __ldcg(d.cnt + ti));
                if ((uint64_t)off + cap > d.pool_cap) cap = check_failed(d.ctr, 2, off) ? 0 : cap;
                for (uint32_t t = 0; t < cap; t++) {
                    const uint32_t *e = d.elems + (size_t)(off + t) * 8;
                    const uint32_t ek = __ldcg(e + 6);
                    if (ek == EMPTY) continue;
                    const uint32_t eb = (ek & BASE_MASK) * EIDS;
#pragma unroll 1
                    for (int x = 0; x < EW; x++) {
                        uint32_t w = __ldcg(e + x);
                        while (w) {
                            const uint32_t j = eb + x * 32 + (__ffs(w) - 1);
                            w &= w - 1;
                            n_right++;
                            if (j >= d.V || A < 1 || A > (uint32_t)d.rt.L) { check_failed(d.ctr, 3, j); continue; }
                            ok &= g_insert_t<true>(d, A, j, base, bits, d.rt.track[A]);
                        }
                    }
                }
            }
        } else if (valid) {
            for (uint32_t u = d.rt.un_start[B]; u < d.rt.un_start[B + 1]; u++) {
                const uint32_t A = d.rt.un_A[u];
                if (!d.rt.tpose[A]) continue;
                Bits one;
                const uint32_t o = row % EIDS;
#pragma unroll
                for (int x = 0; x < EW; x++) one.w[x] = (uint32_t)x == (o >> 5) ? 1u << (o & 31) : 0u;
#pragma unroll 1
                for (int x = 0; x < EW; x++) {
                    uint32_t w = bits.w[x];
                    while (w) {
                        const uint32_t j = base * EIDS + x * 32 + (__ffs(w) - 1);
                        w &= w - 1;
                        if (j >= d.V) { check_failed(d.ctr, 4, j); continue; }
                        ok &= g_insert(d, A, j, row / EIDS, one, d.rt.track[A]);
                    }
                }
            }
        }
        // pushes along CSR rows of C, one rule position at a time, edges dealt over the lanes
        const uint32_t nb = col ? d.rt.bin_start[B + 1] - d.rt.bin_start[B] : 0;
        const uint32_t maxb = __reduce_max_sync(0xffffffffu, nb);
        for (uint32_t rho = 0; rho < maxb; rho++) {
            uint32_t A = 0, C = 0, beg = 0, cnt = 0;
            if (rho < nb) {
                const uint32_t q = d.rt.bin_start[B] + rho;
                A = d.rt.bin_A[q];
                C = d.rt.bin_C[q];
                if (d.rt.csr_row[C]) {
                    const uint2 rw = __ldg(d.rt.csr_row[C] + row);
                    beg = rw.x;
                    cnt = rw.y & 0xFFFFFFu;
                    if ((uint64_t)beg + cnt > d.rt.csr_n[C]) cnt = check_failed(d.ctr, 5, beg) ? 0 : cnt;
                    n_left++;
                    n_right += cnt;
                }
            }
            uint32_t incl = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= (uint32_t)o) incl += y;
            }
            const uint32_t total = __shfl_sync(0xffffffffu, incl, 31), st = incl - cnt;
            const uint32_t adj = beg - st;                   // edge f of this lane's record: col[f + adj]
            uint32_t carry = 0;
            for (uint32_t f0 = 0; f0 < total; f0 += 32) {
                // owner of position f: the last lane with edges whose first position is at or below f
                const bool starts = cnt != 0 && st - f0 < 32u;
                if (starts) own[st - f0] = (uint8_t)lane;
                const uint32_t m = __reduce_or_sync(0xffffffffu, starts ? 1u << (st - f0) : 0u);
                __syncwarp();
                const uint32_t below = m & (0xFFFFFFFFu >> (31 - lane));
                const uint32_t o = below ? own[31 - __clz(below)] : carry;
                const uint32_t last = m ? own[31 - __clz(m)] : carry;
                __syncwarp();
                carry = last;
                const uint32_t f = f0 + lane;
                const uint32_t oA = __shfl_sync(0xffffffffu, A, o), oC = __shfl_sync(0xffffffffu, C, o);
                const uint32_t oadj = __shfl_sync(0xffffffffu, adj, o), obase = __shfl_sync(0xffffffffu, base, o);
                Bits ob;
#pragma unroll
                for (int x = 0; x < EW; x++) ob.w[x] = __shfl_sync(0xffffffffu, bits.w[x], o);
                if (f < total) {
                    const uint32_t ci = f + oadj;
                    if (oC < 1 || oC > (uint32_t)d.rt.L || ci >= d.rt.csr_n[oC]) {
                        check_failed(d.ctr, 6, ((uint64_t)oC << 32) | ci);
                    } else {
                        const uint32_t j = __ldg(d.rt.csr_col[oC] + ci);
                        if (j >= d.V || oA < 1 || oA > (uint32_t)d.rt.L)
                            check_failed(d.ctr, 7, ((uint64_t)oA << 32) | j);
                        else if (!g_insert_t<true>(d, oA, j, obase, ob, d.rt.track[oA]))
                            atomicOr(&fail_s[wi], 1u << o);
                    }
                }
            }
        }
        __syncwarp();
        const bool failed = have && (!ok || ((fail_s[wi] >> lane) & 1u));
        const unsigned fm = __ballot_sync(0xffffffffu, failed);
        if (fm) {
            unsigned long long p = 0;
            if (lane == (uint32_t)(__ffs(fm) - 1)) p = atomicAdd(&d.ctr[C_RETRY_N], (unsigned long long)__popc(fm));
            p = __shfl_sync(0xffffffffu, p, __ffs(fm) - 1);
            const uint64_t o = p + __popc(fm & ((1u << lane) - 1u));
            if (failed && o < d.retry_cap) {
                retry_out[2 * o] = a;
                retry_out[2 * o + 1] = b;
            }
        }
        __syncwarp();
    }
    for (int o = 16; o; o >>= 1) {
        n_left += __shfl_xor_sync(0xffffffffu, n_left, o);
        n_right += __shfl_xor_sync(0xffffffffu, n_right, o);
    }
    if (lane == 0) {
        if (n_left) atomicAdd(&d.ctr[C_LEFT], n_left);
        if (n_right) atomicAdd(&d.ctr[C_RIGHT], n_right);
    }
}

// Small rounds: a warp joins 32 records, so a round of few, dense records (alias
// rows reach a whole block) leaves most SMs idle. Below SPLIT_MAX records the
// round's gathered and virtual records are cut into sub-records of at most
// SPLIT_BITS bits each (the union over a record's bits is the union over its
// parts), which the join reads instead; above it the join reads the records
// as they are. The choice is made here, on the device: the joins read their
// counts from C_JN1 / C_JN2 / C_SPLIT_N.
constexpr uint32_t SPLIT_MAX = 32768;
constexpr uint32_t SPLIT_BITS = 8;
constexpr uint32_t SPLIT_PARTS = (EIDS + SPLIT_BITS - 1) / SPLIT_BITS;

__global__ void k_split(Dev d, const uint4 *__restrict__ grecs, const uint4 *__restrict__ vrecs, uint4 *out)
{
    if (d.ctr[C_HALT]) return;
    const uint64_t nd = d.ctr[C_DIRTY_N], nv = d.ctr[C_VN];
    const bool split = nd + nv < SPLIT_MAX;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        d.ctr[C_JN1] = split ? 0 : nd;
        d.ctr[C_JN2] = split ? 0 : nv;
    }
    if (!split) return;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nd + nv;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint4 *r = i < nd ? grecs + 2 * i : vrecs + 2 * (i - nd);
        const uint4 a = r[0], b = r[1];
        const uint32_t w[EW] = {a.x, a.y, a.z, a.w, b.x, b.y};
        uint32_t p = 0;
#pragma unroll
        for (int x = 0; x < EW; x++) p += __popc(w[x]);
        const uint32_t lab = b.z >> KEY_SHIFT;
        if (p && lab <= (uint32_t)MAX_LABELS && d.rt.tpose[lab]) {
            // a column's record is pushed whole (its bits cost nothing extra): never split
            const uint64_t pos = atomicAdd(&d.ctr[C_SPLIT_N], 1ull);
            out[2 * pos] = a;
            out[2 * pos + 1] = b;
            continue;
        }
        const uint32_t parts = (p + SPLIT_BITS - 1) / SPLIT_BITS;
        if (!parts) continue;
        uint64_t pos = atomicAdd(&d.ctr[C_SPLIT_N], (unsigned long long)parts);
        uint32_t cur[EW] = {0, 0, 0, 0, 0, 0}, c = 0;
#pragma unroll
        for (int x = 0; x < EW; x++) {
            uint32_t m = w[x];
            while (m) {
                const uint32_t bit = m & (0u - m);
                m ^= bit;
                cur[x] |= bit;
                if (++c == SPLIT_BITS) {
                    out[2 * pos] = make_uint4(cur[0], cur[1], cur[2], cur[3]);
                    out[2 * pos + 1] = make_uint4(cur[4], cur[5], b.z, b.w);
                    pos++;
                    c = 0;
#pragma unroll
                    for (int y = 0; y < EW; y++) cur[y] = 0;
                }
            }
        }
        if (c) {                      // the last, partial part
            out[2 * pos] = make_uint4(cur[0], cur[1], cur[2], cur[3]);
            out[2 * pos + 1] = make_uint4(cur[4], cur[5], b.z, b.w);
        }
    }
}

// One warp per batch of RB delta records (label B, row i, base, bits); lane r
// owns record r for per-record work, and (record, k) tasks and their right-hand
// items are flattened over the lanes so every phase keeps 32 independent memory
// operations in flight.
// n_ctr >= 0: the record count is device counter n_ctr (round graphs).
// W, LO: the dense window (instantiated for narrow and wide rows; see join_wide).
template <int W, int LO>
__global__ void __launch_bounds__(JOIN_WARPS * 32, (W <= 8 ? GRG_JOIN_MINB : GRG_JOIN_MINB_WIDE))
    k_join(Dev d, const uint4 *__restrict__ recs, uint64_t n, int n_ctr, uint4 *retry_out)
{
    constexpr int WIN = W, WIN_LO = LO;
    using WarpSmem = WarpSmemT<W, LO>;
    if (d.ctr[C_HALT]) return;
    if (n_ctr >= 0) n = d.ctr[n_ctr];
    __shared__ WarpSmem smem[JOIN_WARPS];
    WarpSmem &w = smem[threadIdx.x >> 5];
    const uint32_t lane = lane_id();
    for (int j = lane; j < ACC; j += 32) {
        w.acc_key[j] = EMPTY;
#pragma unroll
        for (int x = 0; x < EW; x++) w.acc_bits[j][x] = 0;
    }
    for (int j = lane; j < NSLOT * WIN * EW; j += 32) (&w.win[0][0][0])[j] = 0;
    if (lane == 0) w.acc_n = 0;
    __syncwarp();
    // per-lane work counters, added into the device counters when one nears 2^30 and at the end
    uint32_t n_left = 0, n_right = 0, n_out = 0, n_noslot = 0, inserts = 0;
    auto flush_counters = [&]() {
        unsigned long long s[5] = {inserts, n_left, n_right, n_out, n_noslot};
#pragma unroll
        for (int i = 0; i < 5; i++)
            for (int o = 16; o; o >>= 1) s[i] += __shfl_xor_sync(0xffffffffu, s[i], o);
        if (lane == 0) {
            if (s[0]) atomicAdd(&d.ctr[C_INSERTS], s[0]);
            if (s[1]) atomicAdd(&d.ctr[C_LEFT], s[1]);
            if (s[2]) atomicAdd(&d.ctr[C_RIGHT], s[2]);
            if (s[3]) atomicAdd(&d.ctr[C_WOUT], s[3]);
            if (s[4]) atomicAdd(&d.ctr[C_NOSLOT], s[4]);
        }
        inserts = n_left = n_right = n_out = n_noslot = 0;
    };
#ifdef GRG_PHASE_TIMERS
    unsigned long long ph[5] = {0, 0, 0, 0, 0};
    long long ph_t = clock64();
#endif
    // a persistent grid: each warp pulls its next batch of 32 records from the launch's
    // device queue (C_JQ, zeroed before the launch), so warps that drew light batches take
    // more of them instead of idling behind the ones that drew heavy records
    const uint64_t nbatch = (n + RB - 1) / RB;
    uint64_t bt = 0;
    if (lane == 0) bt = atomicAdd(&d.ctr[C_JQ], 1ull);
    bt = __shfl_sync(0xffffffffu, bt, 0);
    for (; bt < nbatch; bt = __shfl_sync(0xffffffffu, lane == 0 ? atomicAdd(&d.ctr[C_JQ], 1ull) : 0ull, 0)) {
        const uint64_t ri = bt * RB + lane;
        const bool have = ri < n;
        Bits rb;
        uint32_t key = EMPTY, row = 0;
        if (have) {
            uint4 a, b;
            ld32(recs + 2 * ri, a, b);
            rb.w[0] = a.x; rb.w[1] = a.y; rb.w[2] = a.z; rb.w[3] = a.w; rb.w[4] = b.x; rb.w[5] = b.y;
            key = b.z;
            row = b.w;
        } else {
#pragma unroll
            for (int x = 0; x < EW; x++) rb.w[x] = 0;
        }
        // records of labels stored by destination are pushed by k_push, not joined here
        const uint32_t B = (have && !((key >> KEY_SHIFT) <= (uint32_t)MAX_LABELS && d.rt.tpose[key >> KEY_SHIFT]))
                               ? key >> KEY_SHIFT : 0,
                       base = key & BASE_MASK;
#pragma unroll
        for (int x = 0; x < EW; x++) w.rbits[lane][x] = rb.w[x];
        w.rrow[lane] = row;
        w.rbase[lane] = base;
        // a row's records of one label are contiguous (a table's slots are, and the gather
        // keeps slot order): a run of them shares the window and hash entries of its first
        // record, so their candidates for one output element merge into one
        const uint32_t prow = __shfl_up_sync(0xffffffffu, row, 1), pB = __shfl_up_sync(0xffffffffu, B, 1);
        const bool start = lane == 0 || !have || B == 0 || prow != row || pB != B;
        const unsigned sm = __ballot_sync(0xffffffffu, start);
        const uint32_t lead = 31 - __clz(sm & (0xFFFFFFFFu >> (31 - lane)));
        // runs are numbered in batch order; records past the end of the input come last, so
        // the batch's runs are those of its valid records. A batch of more runs than a warp has
        // window slots joins its runs in passes of NSLOT runs, each run with a slot of its own.
        const uint32_t run = __popc(sm & ((1u << lead) - 1u));
        const uint32_t nruns = __popc(sm & __ballot_sync(0xffffffffu, have));
#if GRG_RUN_PASSES
        const uint32_t npass = nruns > (uint32_t)NSLOT ? (nruns + NSLOT - 1) / NSLOT : 1u;
#else
        const uint32_t npass = 1;
        (void)nruns;
#endif
        if (lane == 0) w.fail = 0;
        __syncwarp();
        bool ok = true;
        const uint32_t nbits = popc6(rb);

        PH_MARK(0);
        // unary rules A ::= B (compute10): the delta itself joins row (A, row)
        // a record names a label 1..L or an old-left rule; anything else joins nothing
        const bool virt = have && B >= OL_SLOT0 && B < OL_SLOT0 + (uint32_t)d.rt.nol;
        const bool real = have && B >= 1 && B <= (uint32_t)d.rt.L;
        const uint32_t nu = real ? d.rt.un_start[B + 1] - d.rt.un_start[B] : 0;
        const uint32_t maxu = __reduce_max_sync(0xffffffffu, nu);
        for (uint32_t u = 0; u < maxu; u++) {
            if (u < nu) {
                const uint32_t A = d.rt.un_A[d.rt.un_start[B] + u];
                if (!d.rt.tpose[A]) {          // into a label stored by destination: k_push turns it around
                    ok &= g_insert(d, A, row, base, rb, d.rt.track[A]);
                    inserts++;
                }
            }
        }

        PH_MARK(1);
        // binary rules A ::= B C: union of rows C[k] into row (A, row). Delta-left
        // (D_B o O_C): right rows from the tables (or their CSR copy). Old-left
        // (O_B o D_C, virtual record of rule q): right rows are this round's delta
        // records of C[k], found through the delta index.
        const uint32_t qv = virt ? B - OL_SLOT0 : 0;
        const uint32_t nbr_rec = virt ? 1 : real ? d.rt.bin_start[B + 1] - d.rt.bin_start[B] : 0;
        for (uint32_t pass = 0; pass < npass; pass++) {
#if GRG_RUN_PASSES
            const bool act = run / (uint32_t)NSLOT == pass;
            if (start && act) w.slot_rec[run % NSLOT] = lane;
            w.rpk[lane] = lead | ((act ? run % NSLOT : NO_SLOT) << 24);
#else
            const bool act = true;
            if (start && run < (uint32_t)NSLOT) w.slot_rec[run] = lane;
            w.rpk[lane] = lead | ((run < (uint32_t)NSLOT ? run : NO_SLOT) << 24);
#endif
            __syncwarp();
            const uint32_t nbr = act ? nbr_rec : 0;
            const uint32_t maxb = __reduce_max_sync(0xffffffffu, nbr);
            for (uint32_t rho = 0; rho < maxb; rho++) {
                const bool hr = rho < nbr;
                const uint32_t q = virt ? qv : d.rt.bin_start[B] + rho;
                w.rA[lane] = !hr ? 0 : virt ? d.rt.ol_A[q] : d.rt.bin_A[q];
                {
                    const uint32_t Cr = !hr ? 0 : virt ? d.rt.ol_C[q] : d.rt.bin_C[q];
                    // item source 0 table, 1 CSR, 2 delta records; +4: a derivable right-hand
                    // label, whose dense rows mostly OR bits the window already holds
                    const bool pre = GRG_WIN_PRECHECK == 2 || (GRG_WIN_PRECHECK == 1 && d.rt.track[Cr]);
                    const uint32_t src = (virt ? 2u : (hr && d.rt.csr_row[Cr]) ? 1u : 0u) | (hr && pre ? 4u : 0u);
                    w.rpk[lane] = (w.rpk[lane] & 0xFF0000FFu) | (Cr << 8) | (src << 16);
                }
                n_left += hr;
                const uint32_t my_cnt = hr ? nbits : 0;
                const uint32_t total = warp_tasks(w, my_cnt);
                const uint32_t my_st = w.kpre[lane];
                uint32_t carry_r = 0;
                // task (record r, intermediate k) -> items of row C[k]. The record of task t is the
                // last record that starts at or before t: records starting in a chunk of 32 tasks
                // mark their start position, a lane takes the highest mark at or below it
                auto task_of = [&](uint32_t tq, uint32_t &rq, uint32_t &kq) {
                    rq = chunk_owner(w, my_cnt != 0 && my_st - tq < 32u, my_st - tq, carry_r);
                    const uint32_t r_st = __shfl_sync(0xffffffffu, my_st, rq);
                    kq = tq + lane < total ? w.rbase[rq] * EIDS + select_bit(w.rbits[rq], tq + lane - r_st) : 0u;
                };
                for (uint32_t t0 = 0; t0 < total; t0 += 32) {
                    const uint32_t t = t0 + lane;
                    uint32_t rr, k;
                    task_of(t0, rr, k);
                    // the task's record, packed: its run's first record tr, right label C, item
                    // source csr (low bits 0 table, 1 CSR, 2 delta records; +4 window pre-check)
                    // and run window slot ts
                    const uint32_t pk = t < total ? w.rpk[rr] : 0u;
                    const uint32_t tr = pk & 0xFFu, C = (pk >> 8) & 0xFFu, csr = (pk >> 16) & 0xFFu, ts = pk >> 24;
                    uint32_t beg = 0, cnt = 0;
                    if (t < total) {
                        if ((csr & 3u) == 2) {
                            const size_t ti = (size_t)(C - 1) * d.V + k;
                            const uint32_t s0 = __ldg(d.drs + ti);
                            beg = s0;
                            cnt = s0 == EMPTY ? 0 : __ldg(d.drc + ti);
                        } else if ((csr & 3u) == 1) {
                            const uint2 rw = __ldg(d.rt.csr_row[C] + k);
                            beg = rw.x;
                            cnt = rw.y & 0xFFFFFFu;
                            n_right += rw.y >> 24;
                        } else {
                            const size_t ti = (size_t)(C - 1) * d.V + k;
                            // a prefix-filled table: only slots [0, count) can be occupied. The
                            // count of a label with such tables loads beside the descriptor.
                            const bool pl = (d.prefix_mask >> (C - 1)) & 1ull;
                            const uint64_t de = __ldg(d.desc + ti);
                            const uint32_t used = pl ? __ldcg(d.cnt + ti) : 0u;
                            beg = (uint32_t)de;
                            cnt = (uint32_t)(de >> 32);
                            if (pl && cnt <= PREFIX_CAP) cnt = min(cnt, used);
                        }
                    }
                    // one right-hand item: a CSR destination id (csr 1), a table element (0) or a
                    // delta record of row C[k] (2). fetch loads it; put ORs it into its run's window
                    // or, outside the window, the shared hash (every lane calls put together: the
                    // hash needs the warp).
                    auto fetch = [&](bool valid, uint32_t o_C, uint32_t o_csr, uint32_t item, Item &it) {
                        it.ok = false;
                        it.b2 = 0;
                        it.ob = EMPTY;
#pragma unroll
                        for (int x = 0; x < EW; x++) it.ib.w[x] = 0;
                        if (valid) {
                            if ((o_csr & 3u) == 1) {
                                const uint32_t dst = __ldg(d.rt.csr_col[o_C] + item);
                                it.b2 = dst / EIDS;
                                it.ob = dst % EIDS;
                                it.ok = true;
                            } else {
                                const uint4 *ep =
                                    (o_csr & 3u) == 2 ? d.drec + 2 * (size_t)item
                                               : reinterpret_cast<const uint4 *>(d.elems + (size_t)item * 8);
                                uint4 e0, e1;
                                ld32(ep, e0, e1);
                                it.ok = e1.z != EMPTY;
                                it.b2 = e1.z & BASE_MASK;
                                it.ib.w[0] = e0.x; it.ib.w[1] = e0.y; it.ib.w[2] = e0.z; it.ib.w[3] = e0.w;
                                it.ib.w[4] = e1.x; it.ib.w[5] = e1.y;
                                n_right += it.ok ? 1 : 0;
                            }
                        }
                    };
                    auto put = [&](Item &it, uint32_t o_r, uint32_t o_s, bool pre) {
                        bool pending = false;
                        uint32_t ckey = 0;
                        if (it.ok) {
                            const int dd = (int)it.b2 - (int)w.rbase[o_r] + WIN_LO;
                            if ((unsigned)dd < (unsigned)WIN && o_s != NO_SLOT) {
                                if (it.ob != EMPTY) {
                                    // one destination id: one word of the window
                                    atomicOr(&w.win[o_s][dd][it.ob >> 5], 1u << (it.ob & 31));
                                } else if (pre) {
                                    // only the words with bits the window lacks (a stale read
                                    // costs an atomic, never a bit: bits stay until the flush)
                                    const uint2 *wp = reinterpret_cast<const uint2 *>(&w.win[o_s][dd][0]);
                                    const uint2 q0 = wp[0], q1 = wp[1], q2 = wp[2];
                                    const uint32_t cur[EW] = {q0.x, q0.y, q1.x, q1.y, q2.x, q2.y};
#pragma unroll
                                    for (int x = 0; x < EW; x++)
                                        if (it.ib.w[x] & ~cur[x]) atomicOr(&w.win[o_s][dd][x], it.ib.w[x]);
                                } else {
#pragma unroll
                                    for (int x = 0; x < EW; x++)
                                        if (it.ib.w[x]) atomicOr(&w.win[o_s][dd][x], it.ib.w[x]);
                                }
                            } else {
                                pending = true;
                                n_out++;                   // an item the dense windows could not hold
                                n_noslot += o_s == NO_SLOT;
                                ckey = (o_r << KEY_SHIFT) | it.b2;
                                if (it.ob != EMPTY) {
#pragma unroll
                                    for (int x = 0; x < EW; x++)
                                        it.ib.w[x] = (uint32_t)x == (it.ob >> 5) ? 1u << (it.ob & 31) : 0u;
                                }
                            }
                        }
                        while (__any_sync(0xffffffffu, pending)) {
                            if (pending) pending = !acc_insert(w, ckey, it.ib);
                            if (__any_sync(0xffffffffu, pending)) acc_flush(d, w, inserts);
                        }
                    };
                    // the first item of every task in the task's own lane (no search, no
                    // broadcast), then the rest flattened over the lanes. (A second item in the
                    // own lane before flattening measured slower: 53.2 -> 58.7 ms on the 2M-vertex
                    // dataflow closure, 252.4 -> 268.3 ms on the 1M alias closure.)
                    Item it;
                    fetch(cnt > 0, C, csr, beg, it);
                    put(it, tr, ts, (csr & 4u) != 0);
                    constexpr uint32_t OWN = 1;
                    const uint32_t cnt1 = cnt > OWN ? cnt - OWN : 0;
                    if (__any_sync(0xffffffffu, cnt1 != 0)) {
                        uint32_t incl = cnt1;
#pragma unroll
                        for (int o = 1; o < 32; o <<= 1) {
                            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
                            if (lane >= (uint32_t)o) incl += y;
                        }
                        const uint32_t nitems = __shfl_sync(0xffffffffu, incl, 31);
                        // per task: item f sits at beg + OWN + f - (first f of the task); record,
                        // label and source packed
                        const uint32_t s1 = incl - cnt1;         // the task's first flattened item
                        const uint32_t adj = beg + OWN - s1;
                        uint32_t carry_o = 0;
                        for (uint32_t f0 = 0; f0 < nitems; f0 += 32) {
                            const uint32_t f = f0 + lane;
                            // owner lane of flattened item f: the last task whose items start at
                            // or before f
                            const uint32_t lo = chunk_owner(w, cnt1 != 0 && s1 - f0 < 32u, s1 - f0, carry_o);
                            const uint32_t o_adj = __shfl_sync(0xffffffffu, adj, lo);
                            const uint32_t o_pk = __shfl_sync(0xffffffffu, pk, lo);
                            fetch(f < nitems, (o_pk >> 8) & 0xFFu, (o_pk >> 16) & 0xFFu, f + o_adj, it);
                            put(it, o_pk & 0xFFu, o_pk >> 24, ((o_pk >> 16) & 4u) != 0);
                        }
                    }
                }
                PH_MARK(2);
                win_flush(d, w, inserts);
                acc_flush(d, w, inserts);
                PH_MARK(3);
            }
        }

        __syncwarp();
        // a failed insert of a run's merged window re-runs every record of the run
        const bool failed = have && (!ok || ((w.fail >> (w.rpk[lane] & 0xFFu)) & 1u));
        const unsigned fm = __ballot_sync(0xffffffffu, failed);
        if (fm) {
            unsigned long long p = 0;
            if (lane == (uint32_t)(__ffs(fm) - 1)) p = atomicAdd(&d.ctr[C_RETRY_N], (unsigned long long)__popc(fm));
            p = __shfl_sync(0xffffffffu, p, __ffs(fm) - 1);
            const uint64_t o = p + __popc(fm & ((1u << lane) - 1u));
            if (failed && o < d.retry_cap) {
                const uint32_t *rw = w.rbits[lane];
                retry_out[2 * o] = make_uint4(rw[0], rw[1], rw[2], rw[3]);
                retry_out[2 * o + 1] = make_uint4(rw[4], rw[5], key, row);
            }
        }
        if (__any_sync(0xffffffffu, (n_left | n_right | n_out | inserts) >> 30)) flush_counters();
        __syncwarp();
        PH_MARK(4);
    }
#ifdef GRG_PHASE_TIMERS

    if (lane == 0)
        for (int i = 0; i < 5; i++) atomicAdd(&d.ctr[C_PH0 + i], ph[i]);
#endif
    flush_counters();
}

// Tables of labels 1..L by log2 of their occupied elements (buckets 0..7, the
// last open-ended) into C_DH0..C_DH0+7: the degree distribution that keys the
// join-window tuning.
__global__ void k_degree_hist(Dev d, uint32_t L)
{
    __shared__ unsigned long long h[8];
    if (threadIdx.x < 8) h[threadIdx.x] = 0;
    __syncthreads();
    const uint64_t nt = (uint64_t)L * d.V;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < nt; t += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t c = d.cnt[t];
        if (c) atomicAdd(&h[min(31 - __clz(c), 7)], 1ull);
    }
    __syncthreads();
    if (threadIdx.x < 8 && h[threadIdx.x]) atomicAdd(&d.ctr[C_DH0 + threadIdx.x], h[threadIdx.x]);
}

// ------------------------------------------------------------ CSR of static rows

// Edges per row of a packed (static) label: deg[v], and row[v].y = deg | min(elements,255) << 24.
__global__ void k_csr_count(Dev d, uint32_t slot, uint32_t *deg, uint2 *row)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < d.V; v += gridDim.x * blockDim.x) {
        const uint64_t de = d.desc[(size_t)(slot - 1) * d.V + v];
        const uint32_t off = (uint32_t)de, cap = (uint32_t)(de >> 32);
        uint32_t c = 0, nel = 0;
        for (uint32_t j = 0; j < cap; j++) {
            const uint32_t *p = d.elems + (size_t)(off + j) * 8;
            if (p[6] == EMPTY) continue;
            nel++;
            for (int x = 0; x < EW; x++) c += __popc(p[x]);
        }
        deg[v] = c;
        row[v].y = (c & 0xFFFFFFu) | (min(nel, 255u) << 24);
        if (c > 0xFFFFFFu) atomicOr(&d.ctr[C_ERR], (unsigned long long)ERR_INTERNAL);
    }
}

// Block-wise exclusive scan of n values (1024 per block); block totals to sums.
// dyn != null: a scan of the gather's chunk counts whose length follows the
// pool top in the device counters (round graphs), at most n; blocks past it return.
__device__ __forceinline__ uint64_t dyn_chunks(uint64_t n, const unsigned long long *dyn)
{
    return dyn ? min(n, (uint64_t)(dyn[C_POOL_TOP] + 1023) / 1024) : n;
}

__global__ void k_scan_blocks(const uint32_t *in, uint32_t *out, uint32_t *sums, uint64_t n,
                              const unsigned long long *dyn)
{
    if (dyn && dyn[C_HALT]) return;
    n = dyn_chunks(n, dyn);
    if (blockIdx.x * 1024ull >= n && n) return;
    __shared__ uint32_t wsum[32];
    const uint64_t i = blockIdx.x * 1024ull + threadIdx.x;
    const uint32_t v = i < n ? in[i] : 0;
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t incl = v;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (uint32_t)o) incl += y;
    }
    if (lane == 31) wsum[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        uint32_t s = wsum[lane], si = s;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, si, o);
            if (lane >= (uint32_t)o) si += y;
        }
        wsum[lane] = si - s;
        if (lane == 31) sums[blockIdx.x] = si;
    }
    __syncthreads();
    if (i < n) out[i] = incl - v + wsum[wid];
}

// Exclusive scan of the block totals (one block, sequential over chunks of 1024); total at sums[nb].
__global__ void k_scan_sums(uint32_t *sums, uint64_t nb, const unsigned long long *dyn)
{
    if (dyn && dyn[C_HALT]) return;
    if (dyn) nb = min(nb, (dyn_chunks(~0ull, dyn) + 1023) / 1024);
    __shared__ uint32_t wsum[32];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (uint64_t c0 = 0; c0 < nb; c0 += 1024) {
        const uint64_t i = c0 + threadIdx.x;
        const uint32_t v = i < nb ? sums[i] : 0;
        uint32_t incl = v;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= (uint32_t)o) incl += y;
        }
        if (lane == 31) wsum[wid] = incl;
        __syncthreads();
        if (wid == 0) {
            uint32_t s = wsum[lane], si = s;
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, si, o);
                if (lane >= (uint32_t)o) si += y;
            }
            wsum[lane] = si - s;
        }
        __syncthreads();
        const uint32_t base = carry;
        if (i < nb) sums[i] = base + incl - v + wsum[wid];
        __syncthreads();
        if (threadIdx.x == 1023) carry = base + wsum[wid] + incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) sums[nb] = carry;
}

__global__ void k_scan_add(uint32_t *out, const uint32_t *sums, uint64_t n, const unsigned long long *dyn)
{
    if (dyn && dyn[C_HALT]) return;
    n = dyn_chunks(n, dyn);
    const uint64_t i = blockIdx.x * 1024ull + threadIdx.x;
    if (i < n) out[i] += sums[blockIdx.x];
}

// Destination ids of every row of a packed label at ptr[v]; row[v].x = ptr[v].
__global__ void k_csr_fill(Dev d, uint32_t slot, const uint32_t *ptr, uint2 *row, uint32_t *col)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < d.V; v += gridDim.x * blockDim.x) {
        const uint64_t de = d.desc[(size_t)(slot - 1) * d.V + v];
        const uint32_t off = (uint32_t)de, cap = (uint32_t)(de >> 32);
        uint32_t pos = ptr[v];
        row[v].x = pos;
        for (uint32_t j = 0; j < cap; j++) {
            const uint32_t *p = d.elems + (size_t)(off + j) * 8;
            const uint32_t k = p[6];
            if (k == EMPTY) continue;
            const uint32_t b = k & BASE_MASK;
            for (int x = 0; x < EW; x++) {
                uint32_t bw = p[x];
                while (bw) {
                    const int bit = __ffs(bw) - 1;
                    bw &= bw - 1;
                    col[pos++] = b * EIDS + x * 32 + bit;
                }
            }
        }
    }
}

// One warp per table that overflowed: allocate a larger table, re-hash.
__global__ void k_grow(Dev d, uint64_t n)
{
    const uint32_t lane = lane_id();
    const uint64_t nwarps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for (uint64_t g = blockIdx.x * (uint64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); g < n; g += nwarps) {
        const uint32_t ti = d.grow[g];
        const uint32_t want = d.want[ti];
        if (!want) continue;
        const uint64_t de = d.desc[ti];
        const uint32_t off = (uint32_t)de, cap = (uint32_t)(de >> 32);
        const uint32_t need = d.cnt[ti] + want;
        uint32_t ncap = 4;
        while (ncap < 2 * cap || max_load(ncap) < need) ncap <<= 1;
        unsigned long long nb = 0;
        if (lane == 0) {
            nb = atomicAdd(&d.ctr[C_POOL_TOP], (unsigned long long)ncap);
            if (nb + ncap > d.pool_cap) {
                atomicOr(&d.ctr[C_ERR], (unsigned long long)ERR_POOL);
                nb = ~0ull;
            }
        }
        nb = __shfl_sync(0xffffffffu, nb, 0);
        if (nb == ~0ull) continue;
        const uint32_t row = (uint32_t)(ti % d.V);
        for (uint32_t t = lane; t < ncap; t += 32) {
            uint4 *e = reinterpret_cast<uint4 *>(d.elems + (nb + t) * 8);
            e[0] = make_uint4(0, 0, 0, 0);
            e[1] = make_uint4(0, 0, EMPTY, row);
            uint4 *b = reinterpret_cast<uint4 *>(d.dbits + (nb + t) * 8);
            b[0] = make_uint4(0, 0, 0, 0);
            b[1] = make_uint4(0, 0, 0, 0);
            if (d.stamp) d.stamp[nb + t] = 0;
        }
        __syncwarp();
        const uint32_t lab = (uint32_t)(ti / d.V) + 1;
        for (uint32_t t = lane; t < cap; t += 32) {
            const uint4 *e = reinterpret_cast<const uint4 *>(d.elems + (size_t)(off + t) * 8);
            const uint4 e0 = e[0], e1 = e[1];
            if (e1.z == EMPTY) continue;
            const uint32_t h = table_start(d, lab, e1.z & BASE_MASK, ncap);
            for (uint32_t p = 0; p < ncap; p++) {
                const uint64_t q = nb + ((h + p) & (ncap - 1));
                if (atomicCAS(d.elems + q * 8 + 6, EMPTY, e1.z) == EMPTY) {
                    uint4 *t2 = reinterpret_cast<uint4 *>(d.elems + q * 8);
                    t2[0] = e0;
                    d.elems[q * 8 + 4] = e1.x;
                    d.elems[q * 8 + 5] = e1.y;
                    // pending delta bits move along, so a table's delta records stay contiguous
                    const uint64_t os = (uint64_t)off + t;
                    if (d.stamp) d.stamp[q] = d.stamp[os];
                    reinterpret_cast<uint2 *>(d.dbits + q * 8)[3] = make_uint2(e1.z, e1.w);
                    if ((d.dmap[os >> 5] >> (os & 31)) & 1u) {
                        uint4 *ob = reinterpret_cast<uint4 *>(d.dbits + os * 8);
                        uint4 *nbp = reinterpret_cast<uint4 *>(d.dbits + q * 8);
                        nbp[0] = ob[0];
                        nbp[1] = ob[1];
                        ob[0] = make_uint4(0, 0, 0, 0);
                        ob[1] = make_uint4(0, 0, 0, 0);
                        atomicAnd(&d.dmap[os >> 5], ~(1u << (os & 31)));
                        atomicOr(&d.dmap[q >> 5], 1u << (q & 31));
                    }
                    break;
                }
            }
        }
        __syncwarp();
        if (lane == 0) {
            d.desc[ti] = ((uint64_t)ncap << 32) | (uint32_t)nb;
            d.want[ti] = 0;
        }
    }
}

// ---------------------------------------------------------------- results

// One warp per table of a label slot: edge/element counts, optional degree and hash.
// by_dst: the label is stored by destination (rows are destinations), which only
// turns the hash terms around; degrees need tables by source.
__global__ void k_count(Dev d, uint32_t slot, uint32_t *deg_edges, uint32_t *deg_elems, uint32_t first,
                        uint32_t last, int do_hash, uint32_t r0, uint32_t r1, uint32_t hash_base, uint32_t id0,
                        int by_dst)
{
    const uint32_t lane = lane_id();
    const uint64_t nwarps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    unsigned long long my_edges = 0, my_hash = 0;
    for (uint64_t v = r0 + blockIdx.x * (uint64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); v < r1; v += nwarps) {
        const uint64_t de = d.desc[(size_t)(slot - 1) * d.V + v];
        const uint32_t off = (uint32_t)de, cap = (uint32_t)(de >> 32);
        uint32_t e = 0, el = 0;
        for (uint32_t t = lane; t < cap; t += 32) {
            const uint32_t *p = d.elems + (size_t)(off + t) * 8;
            const uint32_t k = p[6];
            if (k == EMPTY) continue;
            el++;
            const uint32_t hb = k & BASE_MASK;
            for (int x = 0; x < EW; x++) {
                uint32_t bw = p[x];
                e += __popc(bw);
                if (do_hash)
                    while (bw) {
                        const int bit = __ffs(bw) - 1;
                        bw &= bw - 1;
                    {
                        const uint32_t a = (uint32_t)v - id0, b = hb * EIDS + x * 32 + bit - id0;
                        my_hash += by_dst ? edge_hash(slot - hash_base, b, a) : edge_hash(slot - hash_base, a, b);
                    }
                    }
            }
        }
        for (int o = 16; o; o >>= 1) {
            e += __shfl_xor_sync(0xffffffffu, e, o);
            el += __shfl_xor_sync(0xffffffffu, el, o);
        }
        my_edges += e;
        if (lane == 0 && deg_edges && v >= first && v <= last) {
            deg_edges[v - first] += e;
            deg_elems[v - first] += el;
        }
    }
    if (lane == 0 && my_edges) atomicAdd(&d.ctr[C_LABEL0 + slot], my_edges);
    for (int o = 16; o; o >>= 1) my_hash += __shfl_xor_sync(0xffffffffu, my_hash, o);
    if (lane == 0 && my_hash) atomicAdd(&d.ctr[C_HASH], my_hash);
}

__global__ void k_export(Dev d, uint32_t slot, uint32_t *src, uint32_t *dst, uint8_t *lab, uint64_t cap_out, int by_dst)
{
    const uint64_t n = (uint64_t)d.V;
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t de = d.desc[(size_t)(slot - 1) * d.V + v];
        const uint32_t off = (uint32_t)de, cap = (uint32_t)(de >> 32);
        for (uint32_t t = 0; t < cap; t++) {
            const uint32_t *p = d.elems + (size_t)(off + t) * 8;
            const uint32_t k = p[6];
            if (k == EMPTY) continue;
            const uint32_t hb = k & BASE_MASK;
            uint32_t c = 0;
            for (int x = 0; x < EW; x++) c += __popc(p[x]);
            unsigned long long pos = atomicAdd(&d.ctr[C_EXPORT], (unsigned long long)c);
            for (int x = 0; x < EW; x++) {
                uint32_t bw = p[x];
                while (bw) {
                    const int bit = __ffs(bw) - 1;
                    bw &= bw - 1;
                    if (pos < cap_out) {
                        const uint32_t o = hb * EIDS + x * 32 + bit;
                        src[pos] = by_dst ? o : (uint32_t)v;
                        dst[pos] = by_dst ? (uint32_t)v : o;
                        lab[pos] = (uint8_t)slot;
                    }
                    pos++;
                }
            }
        }
    }
}

// ---------------------------------------------------------------- element images
//
// An element image is the list of a vertex range's occupied elements, 32 bytes
// each (words 0-5 bitmap, word 6 key = label << 25 | base, word 7 row), with
// a stamp per element: the reference's partition pool dump (transferElements
// / transferBackElements, src/kernel.cu:42-52, src/main.cpp:477-483) with its
// linked-list words replaced by the key, and the stamps that let an
// out-of-core schedule mark only what a pair of partitions has not seen.

__device__ __forceinline__ bool elem_ok(const Dev &d, uint32_t L, uint32_t key, uint32_t row)
{
    const uint32_t lab = key >> KEY_SHIFT, base = key & BASE_MASK;
    return lab >= 1 && lab <= L && row < d.V && (uint64_t)base * EIDS < d.V;
}

// rowmark (nullable): rows that hold a record get their bit set
__global__ void k_elem_hist(Dev d, const uint4 *recs, uint64_t n, uint32_t L, uint32_t *rowmark)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint4 e1 = recs[2 * i + 1];
        if (!elem_ok(d, L, e1.z, e1.w)) {
            atomicOr(&d.ctr[C_ERR], (unsigned long long)ERR_LOAD);
            continue;
        }
        atomicAdd(&d.cnt[(size_t)((e1.z >> KEY_SHIFT) - 1) * d.V + e1.w], 1u);
        if (rowmark) {
            const uint32_t bit = 1u << (e1.w & 31);
            uint32_t *w = rowmark + (e1.w >> 5);
            if (!(__ldcg(w) & bit)) atomicOr(w, bit);
        }
    }
}

// Place every record in its (fresh, histogram-sized) table; records stamped
// after mark_after become deltas of round 1.
__global__ void k_elem_insert(Dev d, const uint4 *recs, const uint32_t *stamps, uint64_t n, uint32_t mark_after,
                              uint32_t L)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint4 e0 = recs[2 * i], e1 = recs[2 * i + 1];
        if (!elem_ok(d, L, e1.z, e1.w)) {
            atomicOr(&d.ctr[C_ERR], (unsigned long long)ERR_LOAD);
            continue;
        }
        const uint32_t lab = e1.z >> KEY_SHIFT, base = e1.z & BASE_MASK;
        const size_t ti = (size_t)(lab - 1) * d.V + e1.w;
        const uint64_t de = d.desc[ti];
        const uint32_t off = (uint32_t)de, cap = (uint32_t)(de >> 32);
        uint32_t q = EMPTY;
        if (cap && (cap & (cap - 1)) == 0) {
            const uint32_t h = table_start(d, lab, base, cap);
            for (uint32_t p = 0; p < cap; p++) {
                const uint32_t t = off + ((h + p) & (cap - 1));
                const uint32_t prev = atomicCAS(d.elems + (size_t)t * 8 + 6, EMPTY, e1.z);
                if (prev == EMPTY) { q = t; break; }
                if (prev == e1.z) break;               // repeated record
            }
        }
        if (q == EMPTY) {
            atomicOr(&d.ctr[C_ERR], (unsigned long long)ERR_LOAD);
            continue;
        }
        uint4 *e = reinterpret_cast<uint4 *>(d.elems + (size_t)q * 8);
        e[0] = e0;
        d.elems[(size_t)q * 8 + 4] = e1.x;
        d.elems[(size_t)q * 8 + 5] = e1.y;
        d.elems[(size_t)q * 8 + 7] = e1.w;
        atomicAdd(&d.cnt[ti], 1u);
        const uint32_t st = stamps[i];
        d.stamp[q] = st;
        uint4 *b = reinterpret_cast<uint4 *>(d.dbits + (size_t)q * 8);
        if (st > mark_after) {
            b[0] = e0;
            b[1] = e1;                     // words 6-7: key and row
            atomicOr(&d.dmap[q >> 5], 1u << (q & 31));
        } else {
            reinterpret_cast<uint2 *>(b)[3] = make_uint2(e1.z, e1.w);
        }
    }
}

// Image of rows [v0, v1): one warp per table (label, row); out == null counts only.
__global__ void k_export_elems(Dev d, uint32_t v0, uint32_t v1, uint32_t L, uint4 *out, uint32_t *st_out,
                               uint64_t cap_out)
{
    const uint32_t lane = lane_id();
    const uint64_t nv = v1 - v0, ntab = (uint64_t)L * nv;
    const uint64_t nwarps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for (uint64_t u = blockIdx.x * (uint64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); u < ntab; u += nwarps) {
        const uint32_t lab = (uint32_t)(u / nv) + 1, row = v0 + (uint32_t)(u % nv);
        const uint64_t de = d.desc[(size_t)(lab - 1) * d.V + row];
        const uint32_t off = (uint32_t)de, cap = (uint32_t)(de >> 32);
        for (uint32_t t0 = 0; t0 < cap; t0 += 32) {
            const uint32_t t = t0 + lane;
            uint4 e0 = make_uint4(0, 0, 0, 0), e1 = make_uint4(0, 0, EMPTY, 0);
            if (t < cap) {
                const uint4 *e = reinterpret_cast<const uint4 *>(d.elems + (size_t)(off + t) * 8);
                e1 = e[1];
                if (e1.z != EMPTY) e0 = e[0];
            }
            const bool have = e1.z != EMPTY;
            const unsigned m = __ballot_sync(0xffffffffu, have);
            if (!m) continue;
            unsigned long long p0 = 0;
            if (lane == 0) p0 = atomicAdd(&d.ctr[C_EXPORT], (unsigned long long)__popc(m));
            p0 = __shfl_sync(0xffffffffu, p0, 0);
            if (have && out) {
                const uint64_t p = p0 + __popc(m & ((1u << lane) - 1u));
                if (p < cap_out) {
                    out[2 * p] = e0;
                    out[2 * p + 1] = make_uint4(e1.x, e1.y, e1.z, row);
                    st_out[p] = d.stamp ? d.stamp[off + t] : 0u;
                }
            }
        }
    }
}

// Partitions that rows [v0, v1) reach through labels in label_mask:
// flags[p] = 1 when an element's destinations overlap [bounds[p], bounds[p+1])
// (every partition between an element's lowest and highest destination: a
// superset, which only ever schedules a pair too many).
__global__ void k_range_reach(Dev d, uint32_t v0, uint32_t v1, uint32_t L, unsigned long long label_mask,
                              const uint32_t *bounds, uint32_t np, uint32_t *flags)
{
    const uint32_t lane = lane_id();
    const uint64_t nv = v1 - v0, ntab = (uint64_t)L * nv;
    const uint64_t nwarps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for (uint64_t u = blockIdx.x * (uint64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); u < ntab; u += nwarps) {
        const uint32_t lab = (uint32_t)(u / nv) + 1, row = v0 + (uint32_t)(u % nv);
        if (!((label_mask >> (lab - 1)) & 1ull)) continue;
        const uint64_t de = d.desc[(size_t)(lab - 1) * d.V + row];
        const uint32_t off = (uint32_t)de, cap = (uint32_t)(de >> 32);
        for (uint32_t t = lane; t < cap; t += 32) {
            const uint32_t *e = d.elems + (size_t)(off + t) * 8;
            const uint32_t key = e[6];
            if (key == EMPTY) continue;
            int lo = -1, hi = -1;
#pragma unroll
            for (int x = 0; x < EW; x++) {
                const uint32_t w = e[x];
                if (w && lo < 0) lo = x * 32 + __ffs(w) - 1;
                if (w) hi = x * 32 + 31 - __clz(w);
            }
            if (lo < 0) continue;
            const uint64_t b0 = (uint64_t)(key & BASE_MASK) * EIDS;
            const uint64_t dmin = b0 + lo, dmax = b0 + hi;
            // last p with bounds[p] <= dest
            uint32_t a = 0, z = np;
            while (z - a > 1) {
                const uint32_t m = (a + z) / 2;
                if (bounds[m] <= dmin) a = m; else z = m;
            }
            uint32_t p = a;
            for (; p < np && bounds[p] <= dmax; p++)
                if (!flags[p]) flags[p] = 1;
        }
    }
}

}  // namespace grg

// ====================================================================== host

using namespace grg;

struct grg_ctx {
    int device = 0;
    int sms = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    std::string err;
    bool timing = false;
    cudaEvent_t ev_a = nullptr, ev_b = nullptr, ev_c = nullptr, ev_d = nullptr;
    // grammar
    bool have_rules = false;
    int L = 0, R = 0;
    int rules[3 * GRG_MAX_RULES] = {0};
    // graph
    bool loaded = false;
    bool closed = false;
    uint32_t V = 0;
    uint64_t ntables = 0;          // L * V (label slots 1..L)
    uint64_t ntables_alloc = 0;    // table entries allocated (>= L * V)
    uint64_t dvm_alloc = 0;        // dirty-vertex bitmap words allocated
    // device memory
    uint64_t pool_bytes_req = 0;
    uint64_t pool_cap = 0;         // elements
    uint32_t *elems = nullptr;
    uint32_t *dbits = nullptr;                 // delta bitmaps (32 B per slot)
    uint32_t *dmap = nullptr;                  // dirty bitmap (1 bit per slot)
    uint32_t *chunk = nullptr;                 // dirty counts / offsets per 1024 slots (+ scan sums)
    uint64_t chunk_cap = 0;
    uint64_t *desc = nullptr;
    uint32_t *cnt = nullptr, *want = nullptr, *grow = nullptr;
    uint4 *rbuf[2] = {nullptr, nullptr};       // delta records of retry passes
    uint64_t rbuf_cap = 0;                     // records
    uint4 *gbuf = nullptr;                     // gathered delta records of the round
    uint64_t gbuf_cap = 0;
    uint32_t *gslot = nullptr;                 // their slot ids (gather pass 1)
    uint64_t gslot_cap = 0;
    uint4 *vbuf = nullptr;                     // virtual records of old-left joins
    uint64_t vbuf_cap = 0;
    uint4 *sbuf = nullptr;                     // sub-records of small rounds (k_split)
    uint32_t *drs = nullptr, *drc = nullptr, *dvm = nullptr;   // delta index (per label x row / vertex bitmap)
    uint4 *cand[2] = {nullptr, nullptr};       // join candidates for k_apply / failed candidates
    uint64_t cand_cap = 0;
    int cb = 0;                                // candidate buffer the joins write
    unsigned long long *ctr = nullptr;
    unsigned long long *h_ctr = nullptr;   // pinned
    uint32_t *d_in32 = nullptr;            // staged input edges (src, dst)
    uint8_t *d_in8 = nullptr;
    uint64_t in_cap = 0;
    // element images (out-of-core partitions): graph loaded from element records with stamps
    bool stamp_on = false;                 // the pool carries a stamp per slot
    bool elem_loaded = false;              // the current graph came from grg_load_elements
    uint32_t *stamp = nullptr;             // per-slot stamps (pool_cap entries)
    uint32_t *rowmark = nullptr;           // rows an element image holds (1 bit per vertex)
    uint64_t rowmark_cap = 0;
    uint32_t run_stamp = 0;                // stamp given to elements that gain bits in this closure
    uint4 *xbuf = nullptr;                 // staged element records (load input / export output)
    uint32_t *xst = nullptr;               // staged stamps
    uint64_t xcap = 0;
    uint64_t pool_limit = 0;               // maximum pool slots (0 = what the device holds)
    uint64_t retry_min = 1ull << 20;       // smallest retry list (records; GRG_RETRY_ROOM)
    uint64_t prefix_mask = 0;              // labels with prefix-filled small tables (Dev::prefix_mask)
    // join window: narrow (WIN) or wide (WIN2, the default)
    bool join_wide = true;
    int join_window_mode = 2;              // 0 narrow, 1 wide, 2 tuned per degree key, 3 re-measured
    bool tuned_wide = true;                // the tuned choice for the current closure
    // right-hand items of CSR-copied labels: destination ids (the CSR copy) or whole
    // 192-id elements of the label's table
    int items_mode = 2;                    // 0 ids, 1 elements, 2 tuned per degree key, 3 re-measured
    bool join_elems = false;               // the form of this closure
    bool tuned_elems = false;
    float items_ms[2] = {0, 0};            // measured (ids, elements) when tuned in this closure
    bool tune_pending = false;             // measure both windows in the first large round
    uint64_t tune_key = 0;
    int tune_source = 0;                   // grg_stats.window_tuned
    float tune_ms[2] = {0, 0};
    cudaEvent_t ev_t0 = nullptr, ev_t1 = nullptr;
    // device-driven rounds: a CUDA graph whose WHILE node repeats one closure round
    bool device_rounds = true;
    cudaStream_t cap_stream = nullptr;     // stream the round graph is recorded on
    cudaGraph_t rg_graph = nullptr;
    cudaGraphExec_t rg_exec = nullptr;
    std::vector<uint64_t> rg_key;          // pointers and sizes the recorded launches hold
    int rg_kernels = 0;                    // kernels per recorded round
    RuleTable rt{};
    // labels stored by destination in the loaded graph (bit l-1), and whether loads
    // may choose that layout (grg_set_layout)
    uint64_t tmask = 0;
    int layout_mode = 0;
    // kernels a join pass needs under the current rule table: k_join for records
    // joined by source rows, k_push for records of destination-stored labels
    bool need_join = true, need_push = false;
    // push kernel: one lane per record (k_push) or edges dealt over the lanes (k_push_flat)
    int push_mode = 2;                     // 0 per record, 1 flattened, 2 tuned per degree key, 3 re-measured
    bool push_flat = true;                 // the kernel of this closure
    bool tuned_flat = true;
    bool push_pending = false;             // measure both push kernels in the first large round
    int push_source = 0;                   // grg_stats.push_tuned
    float push_ms[2] = {0, 0};
    uint64_t launches = 0;
    // CSR copies of static labels, per label; reused by later closures while they fit
    struct CsrBuf {
        uint32_t *ptr = nullptr, *sums = nullptr, *col = nullptr;
        uint2 *row = nullptr;
        uint64_t vcap = 0, colcap = 0;
    } csr[MAX_LABELS + 1];
    // batched jobs (continuous batching): each job owns a vertex range
    uint32_t *row_job = nullptr;           // vertex -> job slot (EMPTY = free)
    uint32_t *job_cnt = nullptr;           // delta records per job slot in the last gather
    uint32_t max_jobs = 0;
    bool batch = false;
    uint32_t filter = 0;
    // pending: delta records of the job in the last gather (UINT32_MAX until a step has run)
    struct JobRange { uint32_t base = 0, nv = 0; bool active = false; uint32_t pending = 0xFFFFFFFFu; };
    std::vector<JobRange> jobs;
};

static void free_round_graph(grg_ctx *c);

namespace {

const char *status_text(int s)
{
    switch (s) {
    case GRG_OK: return "ok";
    case GRG_NEED_REPARTITION: return "partition needs repartitioning";
    case GRG_PAUSED: return "paused at the run budget";
    case GRG_E_ARG: return "invalid argument";
    case GRG_E_CUDA: return "CUDA error";
    case GRG_E_NOMEM: return "out of memory";
    case GRG_E_FILTER: return "filter_flag=1 is schedule-dependent for this grammar (a binary rule's second symbol is derivable)";
    case GRG_E_IO: return "I/O or format error";
    case GRG_E_LABEL: return "graph label not in grammar";
    case GRG_E_RANGE: return "value out of range";
    case GRG_E_STATE: return "call out of order";
    case GRG_E_NODEV: return "no CUDA device";
    case GRG_E_INTERNAL: return "internal limit or consistency check failed";
    default: return "unknown status";
    }
}

int fail(grg_ctx *c, int st, const std::string &msg)
{
    if (c) c->err = msg;
    return st;
}

#define GRG_CUDA(c, call)                                                                        \
    do {                                                                                         \
        cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess) return fail((c), GRG_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

int grid_for(const grg_ctx *c, uint64_t n, int block, int per_sm = 8)
{
    uint64_t g = (n + block - 1) / block;
    uint64_t cap = (uint64_t)c->sms * per_sm;
    if (g > cap) g = cap;
    return (int)std::max<uint64_t>(g, 1);
}

Dev make_dev(const grg_ctx *c)
{
    Dev d;
    d.elems = c->elems;
    d.dbits = c->dbits;
    d.dmap = c->dmap;
    d.desc = c->desc;
    d.cnt = c->cnt;
    d.want = c->want;
    d.cand = c->cand[c->cb];
    d.cand_cap = c->cand_cap;
    d.retry_cap = c->rbuf_cap;
    d.drs = c->drs;
    d.drc = c->drc;
    d.dvm = c->dvm;
    d.drec = c->gbuf;
    d.vwords = (c->V + 31) / 32;
    d.grow = c->grow;
    d.ctr = c->ctr;
    d.V = c->V;
    d.pool_cap = (uint32_t)c->pool_cap;
    d.stamp = c->elem_loaded ? c->stamp : nullptr;
    d.prefix_mask = c->prefix_mask;
    d.rt = c->rt;
    return d;
}

void free_csr(grg_ctx *c)
{
    for (auto &b : c->csr) {
        cudaFree(b.ptr);
        cudaFree(b.sums);
        cudaFree(b.col);
        cudaFree(b.row);
        b = grg_ctx::CsrBuf();
    }
}

void free_graph(grg_ctx *c)
{
    free_csr(c);
    cudaFree(c->drs); c->drs = nullptr;
    cudaFree(c->drc); c->drc = nullptr;
    cudaFree(c->dvm); c->dvm = nullptr;
    c->dvm_alloc = 0;
    cudaFree(c->row_job); c->row_job = nullptr;
    cudaFree(c->job_cnt); c->job_cnt = nullptr;
    c->max_jobs = 0;
    c->batch = false;
    c->jobs.clear();
    cudaFree(c->desc); c->desc = nullptr;
    cudaFree(c->cnt); c->cnt = nullptr;
    cudaFree(c->want); c->want = nullptr;
    cudaFree(c->grow); c->grow = nullptr;
    c->ntables_alloc = 0;
}

void free_pool(grg_ctx *c)
{
    cudaFree(c->elems); c->elems = nullptr;
    cudaFree(c->dbits); c->dbits = nullptr;
    cudaFree(c->dmap); c->dmap = nullptr;
    cudaFree(c->stamp); c->stamp = nullptr;
    c->pool_cap = 0;
}

int read_ctr(grg_ctx *c)
{
    GRG_CUDA(c, cudaMemcpyAsync(c->h_ctr, c->ctr, sizeof(unsigned long long) * NCTR, cudaMemcpyDeviceToHost, c->stream));
    GRG_CUDA(c, cudaStreamSynchronize(c->stream));
    return GRG_OK;
}

// Device staging of num_edges input edges (src and dst in d_in32, labels in d_in8).
static int ensure_input(grg_ctx *c, uint64_t num_edges)
{
    if (c->in_cap >= num_edges) return GRG_OK;
    cudaFree(c->d_in32); cudaFree(c->d_in8);
    c->d_in32 = nullptr; c->d_in8 = nullptr;
    c->in_cap = 0;
    GRG_CUDA(c, cudaMalloc(&c->d_in32, num_edges * 8));
    GRG_CUDA(c, cudaMalloc(&c->d_in8, num_edges));
    c->in_cap = num_edges;
    return GRG_OK;
}

// Status for input edges the load kernels refused (counters already read).
int input_status(grg_ctx *c)
{
    const unsigned long long b = c->h_ctr[C_BADIN];
    if (b & ERR_IN_LABEL) return fail(c, GRG_E_LABEL, "edge label outside 1..numLabels");
    if (b & ERR_IN_RANGE) return fail(c, GRG_E_RANGE, "edge vertex id >= numVars");
    return GRG_OK;
}


constexpr uint64_t POOL_BYTES_PER_SLOT = 32 + 32 + 1;
constexpr uint32_t DERIVED_MIN_CAP = 16;   // element, delta bitmap, dirty bit (rounded up)

// Pool of `elems` 32-byte slots + their delta bitmaps + the dirty bitmap.
int alloc_pool(grg_ctx *c, uint64_t elems)
{
    if (elems > 0xFFFFFFE0ull) elems = 0xFFFFFFE0ull;
    const uint64_t words = elems / 32 + 2;
    uint32_t *e = nullptr, *b = nullptr, *m = nullptr, *t = nullptr;
    if (cudaMalloc(&e, elems * 32) != cudaSuccess || cudaMalloc(&b, elems * 32) != cudaSuccess ||
        cudaMalloc(&m, words * 4) != cudaSuccess || (c->stamp_on && cudaMalloc(&t, elems * 4) != cudaSuccess)) {
        cudaGetLastError();
        cudaFree(e); cudaFree(b); cudaFree(m); cudaFree(t);
        return fail(c, GRG_E_NOMEM, "cannot allocate element pool of " + std::to_string(elems) + " slots");
    }
    GRG_CUDA(c, cudaMemsetAsync(m, 0, words * 4, c->stream));
    if (c->elems) {
        // grow: keep the used part, its delta bitmaps, dirty bits and stamps
        int st = read_ctr(c);
        if (st) { cudaFree(e); cudaFree(b); cudaFree(m); cudaFree(t); return st; }
        const uint64_t used = std::min<uint64_t>(c->h_ctr[C_POOL_TOP], c->pool_cap);
        GRG_CUDA(c, cudaMemcpyAsync(e, c->elems, used * 32, cudaMemcpyDeviceToDevice, c->stream));
        GRG_CUDA(c, cudaMemcpyAsync(b, c->dbits, used * 32, cudaMemcpyDeviceToDevice, c->stream));
        GRG_CUDA(c, cudaMemcpyAsync(m, c->dmap, (used / 32 + 1) * 4, cudaMemcpyDeviceToDevice, c->stream));
        if (t && c->stamp) GRG_CUDA(c, cudaMemcpyAsync(t, c->stamp, used * 4, cudaMemcpyDeviceToDevice, c->stream));
        GRG_CUDA(c, cudaStreamSynchronize(c->stream));
        free_pool(c);
    }
    c->elems = e;
    c->dbits = b;
    c->dmap = m;
    c->stamp = t;
    c->pool_cap = elems;
    return GRG_OK;
}

// Chunk counters of the dirty-bitmap gather: one per 1024 slots, plus scan sums.
int ensure_chunks(grg_ctx *c, uint64_t nchunks)
{
    const uint64_t need = 2 * (nchunks + 1) + (nchunks + 1023) / 1024 + 2;
    if (need <= c->chunk_cap) return GRG_OK;
    cudaFree(c->chunk);
    c->chunk = nullptr;
    GRG_CUDA(c, cudaMalloc(&c->chunk, need * 2 * 4));
    c->chunk_cap = need * 2;
    return GRG_OK;
}

int grow_pool(grg_ctx *c, uint64_t min_elems)
{
    uint64_t want = std::max<uint64_t>(c->pool_cap * 2, min_elems);
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    uint64_t fit = (uint64_t)((double)fr * 0.9) / POOL_BYTES_PER_SLOT;
    if (want > fit) want = fit;
    if (c->pool_limit && want > c->pool_limit) want = c->pool_limit;
    if (want <= c->pool_cap) return fail(c, GRG_E_NOMEM, "element pool exhausted and device memory is full");
    return alloc_pool(c, want);
}

// Where a join's merged elements go: candidates that k_apply inserts after the join
// (write-behind), or straight into the tables from the join. Direct inserts let the
// joins of a round read right-hand rows that other joins of the same round have just
// grown, which pays when right-hand labels are derivable (old-left rules): the 1M alias
// closure needed 12% fewer delta elements and took 242 instead of 252 ms. With static
// right-hand rows nothing is gained and the join's warps wait on the inserts: the 2M
// dataflow closure took 56.3 instead of 52.8 ms. Environment GRG_DIRECT_INSERTS=0 / 1
// overrides the choice.
static bool direct_inserts(const grg_ctx *c)
{
    const char *e = getenv("GRG_DIRECT_INSERTS");
    if (e && (e[0] == '0' || e[0] == '1')) return e[0] == '1';
    return c->rt.nol > 0;
}

// Candidate buffers of a round (4 per delta record; a full buffer falls back to direct inserts).
int ensure_cand(grg_ctx *c, uint64_t nd)
{
    if (direct_inserts(c)) {
        if (c->cand_cap) {
            cudaFree(c->cand[0]);
            cudaFree(c->cand[1]);
            c->cand[0] = c->cand[1] = nullptr;
            c->cand_cap = 0;
        }
        return GRG_OK;
    }
    // capped at 2^26 candidates (2 GiB a buffer): past it, joins insert directly
    const uint64_t want = std::min<uint64_t>(std::max<uint64_t>(4 * nd, 1 << 20), 1ull << 26);
    if (want <= c->cand_cap) return GRG_OK;
    const uint64_t cap = std::min<uint64_t>(want + want / 2, 1ull << 26);
    cudaFree(c->cand[0]);
    cudaFree(c->cand[1]);
    c->cand[0] = c->cand[1] = nullptr;
    c->cand_cap = 0;
    if (cudaMalloc(&c->cand[0], cap * 32) != cudaSuccess || cudaMalloc(&c->cand[1], cap * 32) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(c->cand[0]);
        cudaFree(c->cand[1]);
        c->cand[0] = c->cand[1] = nullptr;
        return GRG_OK;   // no candidate buffers: joins insert directly
    }
    c->cand_cap = cap;
    return GRG_OK;
}

// Grow a record buffer (32 B per record) to hold n records (contents not kept).
int ensure_buf(grg_ctx *c, uint4 **buf, uint64_t *cap, uint64_t n)
{
    if (n <= *cap) return GRG_OK;
    const uint64_t nc = std::max<uint64_t>(n + n / 2, 1 << 16);
    cudaFree(*buf);
    *buf = nullptr;
    *cap = 0;
    GRG_CUDA(c, cudaMalloc(buf, nc * 32));
    *cap = nc;
    return GRG_OK;
}

// Gathered records and their slot ids, room for n.
int ensure_gather(grg_ctx *c, uint64_t n)
{
    int st = ensure_buf(c, &c->gbuf, &c->gbuf_cap, n);
    if (st) return st;
    if (c->gslot_cap >= c->gbuf_cap) return GRG_OK;
    cudaFree(c->gslot);
    c->gslot = nullptr;
    c->gslot_cap = 0;
    GRG_CUDA(c, cudaMalloc(&c->gslot, c->gbuf_cap * 4));
    c->gslot_cap = c->gbuf_cap;
    return GRG_OK;
}

// Retry buffers: every delta record of a pass may fail once, so n records each.
int ensure_rbuf(grg_ctx *c, uint64_t n)
{
    if (n <= c->rbuf_cap) return GRG_OK;
    const uint64_t cap = std::max<uint64_t>(n + n / 2, 1 << 16);
    for (int i = 0; i < 2; i++) {
        cudaFree(c->rbuf[i]);
        c->rbuf[i] = nullptr;
    }
    c->rbuf_cap = 0;
    for (int i = 0; i < 2; i++) GRG_CUDA(c, cudaMalloc(&c->rbuf[i], cap * 32));
    c->rbuf_cap = cap;
    return GRG_OK;
}

// Delta index of the labels old-left joins read: table start/count and vertex bitmap.
int alloc_dindex(grg_ctx *c)
{
    const uint64_t nt = (uint64_t)c->L * c->V, vw = (uint64_t)c->L * ((c->V + 31) / 32);
    c->dvm_alloc = std::max<uint64_t>(vw, 1);
    GRG_CUDA(c, cudaMalloc(&c->drs, std::max<uint64_t>(nt, 1) * 4));
    GRG_CUDA(c, cudaMalloc(&c->drc, std::max<uint64_t>(nt, 1) * 4));
    GRG_CUDA(c, cudaMalloc(&c->dvm, std::max<uint64_t>(vw, 1) * 4));
    GRG_CUDA(c, cudaMemsetAsync(c->drs, 0xFF, std::max<uint64_t>(nt, 1) * 4, c->stream));
    GRG_CUDA(c, cudaMemsetAsync(c->drc, 0, std::max<uint64_t>(nt, 1) * 4, c->stream));
    GRG_CUDA(c, cudaMemsetAsync(c->dvm, 0, std::max<uint64_t>(vw, 1) * 4, c->stream));
    return GRG_OK;
}

// Rule table of the context's grammar for a filter.
int build_rules(grg_ctx *c, uint32_t filter, RuleTable &rt)
{
    bool derivable[MAX_LABELS + 1];
    const int st = make_rule_table(c->rules, c->R, c->L, filter, rt, derivable);
    if (st) return fail(c, st, status_text(st));
    set_columns(rt, c->tmask, c->L);
    return GRG_OK;
}

}  // namespace

extern "C" {

const char *grg_error_string(int status) { return status_text(status); }
const char *grg_last_error(const grg_ctx *ctx) { return ctx ? ctx->err.c_str() : ""; }

int grg_create(grg_ctx **out, int device)
{
    if (!out) return GRG_E_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) { cudaGetLastError(); return GRG_E_NODEV; }
    if (device >= n) return GRG_E_ARG;
    if (device < 0) {
        int best = -1;
        for (int i = 0; i < n; i++) {
            int sm = 0;
            cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, i);
            if (sm > best) { best = sm; device = i; }
        }
    }
    grg_ctx *c = new grg_ctx();
    c->device = device;
    if (cudaSetDevice(device) != cudaSuccess) { delete c; return GRG_E_CUDA; }
    cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device);
    if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&c->ctr, sizeof(unsigned long long) * NCTR) != cudaSuccess ||
        cudaMallocHost(&c->h_ctr, sizeof(unsigned long long) * NCTR) != cudaSuccess ||
        cudaEventCreate(&c->ev_a) != cudaSuccess || cudaEventCreate(&c->ev_b) != cudaSuccess ||
        cudaEventCreate(&c->ev_c) != cudaSuccess || cudaEventCreate(&c->ev_d) != cudaSuccess) {
        grg_destroy(c);
        return GRG_E_CUDA;
    }
    c->stream = c->own_stream;
    const char *dr = getenv("GRG_DEVICE_ROUNDS");      // "0": every round driven from the host
    c->device_rounds = !(dr && dr[0] == '0');
    const char *rr = getenv("GRG_RETRY_ROOM");         // smallest retry list, in records
    if (rr && atoll(rr) > 0) c->retry_min = (uint64_t)atoll(rr);
    const char *jw = getenv("GRG_JOIN_WINDOW");        // "narrow" / "wide"; otherwise chosen per closure
    if (jw) c->join_window_mode = !strcmp(jw, "narrow") ? 0 : !strcmp(jw, "wide") ? 1 : 2;
    const char *ly = getenv("GRG_LAYOUT");             // "columns": labels the grammar allows by destination
    if (ly) c->layout_mode = !strcmp(ly, "columns") ? 1 : 0;
    const char *ji = getenv("GRG_JOIN_ITEMS");         // "ids" / "elements"; otherwise chosen per closure
    if (ji) c->items_mode = !strcmp(ji, "ids") ? 0 : !strcmp(ji, "elements") ? 1 : 2;
    const char *pm = getenv("GRG_PUSH");               // "lane" / "flat"; otherwise chosen per closure
    if (pm) c->push_mode = !strcmp(pm, "lane") ? 0 : !strcmp(pm, "flat") ? 1 : 2;
    *out = c;
    return GRG_OK;
}

void grg_destroy(grg_ctx *c)
{
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    free_graph(c);
    free_pool(c);
    for (int i = 0; i < 2; i++) cudaFree(c->rbuf[i]);
    cudaFree(c->gbuf);
    cudaFree(c->gslot);
    cudaFree(c->vbuf);
    cudaFree(c->sbuf);
    cudaFree(c->xbuf);
    cudaFree(c->xst);
    cudaFree(c->rowmark);
    cudaFree(c->cand[0]);
    cudaFree(c->cand[1]);
    cudaFree(c->chunk);
    cudaFree(c->ctr);
    cudaFree(c->d_in32);
    cudaFree(c->d_in8);
    if (c->h_ctr) cudaFreeHost(c->h_ctr);
    if (c->ev_a) cudaEventDestroy(c->ev_a);
    if (c->ev_b) cudaEventDestroy(c->ev_b);
    if (c->ev_c) cudaEventDestroy(c->ev_c);
    if (c->ev_d) cudaEventDestroy(c->ev_d);
    if (c->ev_t0) cudaEventDestroy(c->ev_t0);
    if (c->ev_t1) cudaEventDestroy(c->ev_t1);
    free_round_graph(c);
    if (c->cap_stream) cudaStreamDestroy(c->cap_stream);
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
    delete c;
}

int grg_device(const grg_ctx *c) { return c ? c->device : -1; }

int grg_set_stream(grg_ctx *c, void *stream)
{
    if (!c) return GRG_E_ARG;
    c->stream = stream ? (cudaStream_t)stream : c->own_stream;
    return GRG_OK;
}

int grg_set_join_window(grg_ctx *c, int mode)
{
    if (!c || mode < 0 || mode > 3) return GRG_E_ARG;
    c->join_window_mode = mode;
    return GRG_OK;
}

int grg_set_device_rounds(grg_ctx *c, int on)
{
    if (!c) return GRG_E_ARG;
    c->device_rounds = on != 0;
    return GRG_OK;
}

int grg_set_join_items(grg_ctx *c, int mode)
{
    if (!c || mode < 0 || mode > 3) return GRG_E_ARG;
    c->items_mode = mode;
    return GRG_OK;
}

int grg_set_push(grg_ctx *c, int mode)
{
    if (!c || mode < 0 || mode > 3) return GRG_E_ARG;
    c->push_mode = mode;
    return GRG_OK;
}

int grg_set_layout(grg_ctx *c, int mode)
{
    if (!c || mode < 0 || mode > 1) return GRG_E_ARG;
    c->layout_mode = mode;
    return GRG_OK;
}

int grg_set_kernel_timing(grg_ctx *c, int on)
{
    if (!c) return GRG_E_ARG;
    c->timing = on != 0;
    return GRG_OK;
}

int grg_transfer_rules(grg_ctx *c, int num_rules, const int *rules, int num_labels)
{
    if (!c || num_rules < 0 || (num_rules && !rules)) return GRG_E_ARG;
    if (num_rules > GRG_MAX_RULES || num_labels < 1 || num_labels > GRG_MAX_LABELS)
        return fail(c, GRG_E_RANGE, "too many rules or labels");
    for (int q = 0; q < num_rules; q++) {
        const int *r = &rules[3 * q];
        if (r[0] < 1 || r[0] > num_labels || r[1] < 0 || r[1] > num_labels || r[2] < 0 || r[2] > num_labels ||
            (r[1] == 0 && r[2] != 0))
            return fail(c, GRG_E_ARG, "malformed rule " + std::to_string(q));
    }
    c->R = num_rules;
    c->L = num_labels;
    memset(c->rules, 0, sizeof c->rules);
    memcpy(c->rules, rules, sizeof(int) * 3 * (size_t)num_rules);
    // prefix-filled small tables for the labels joins read as table rows: a binary
    // rule's derivable second symbol (delta-left items) and that rule's first
    // symbol (old-left virtual records scan its rows). A static second symbol's
    // tables are compacted after the load (k_compact_static), so their rows hold
    // no empty slots either.
    bool der[GRG_MAX_LABELS + 1] = {false};
    for (int q = 0; q < num_rules; q++) der[rules[3 * q]] = true;
    c->prefix_mask = 0;
    for (int q = 0; q < num_rules; q++) {
        const int *r = &rules[3 * q];
        if (r[1] && r[2] && der[r[2]]) c->prefix_mask |= (1ull << (r[2] - 1)) | (1ull << (r[1] - 1));
    }
    const char *pt = getenv("GRG_PREFIX_TABLES");    // "0": every table hashed
    if (pt && pt[0] == '0') c->prefix_mask = 0;
    c->have_rules = true;
    c->loaded = false;
    return GRG_OK;
}

int grg_get_rules(const grg_ctx *c, int *num_rules, int *rules, int *num_labels)
{
    if (!c || !num_rules || !rules || !num_labels) return GRG_E_ARG;
    if (!c->have_rules) return GRG_E_STATE;
    *num_rules = c->R;
    *num_labels = c->L;
    memcpy(rules, c->rules, sizeof(int) * 3 * c->R);
    return GRG_OK;
}

int grg_allocate_pool(grg_ctx *c, uint64_t pool_bytes)
{
    if (!c) return GRG_E_ARG;
    cudaSetDevice(c->device);
    c->pool_bytes_req = pool_bytes;
    uint64_t elems;
    if (pool_bytes) {
        elems = pool_bytes / POOL_BYTES_PER_SLOT;
    } else {
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        elems = (uint64_t)(fr / 8) / POOL_BYTES_PER_SLOT;   // start at 1/8 of free memory; grows on demand
    }
    if (elems < 1024) elems = 1024;
    if (c->pool_limit && elems > c->pool_limit) elems = c->pool_limit;
    if (c->elems && c->pool_cap >= elems) return GRG_OK;
    free_pool(c);
    return alloc_pool(c, elems);
}

}  // extern "C"

namespace {

// Tables for a new graph of num_vars vertices: descriptors, counts and the
// delta index (re)allocated when the size changes, everything cleared.
int setup_tables(grg_ctx *c, uint32_t num_vars)
{
    if (!c->elems) {
        int st = grg_allocate_pool(c, c->pool_bytes_req);
        if (st) return st;
    }
    if ((uint64_t)num_vars * (uint64_t)c->L >= 0xFFFFFFFFull)
        return fail(c, GRG_E_RANGE, "numVars x numLabels must stay below 2^32");
    c->V = num_vars;
    c->ntables = (uint64_t)c->L * num_vars;
    const uint64_t nt_all = c->ntables;
    // table arrays are kept while a graph needs no more than they hold
    if (c->ntables_alloc < nt_all || c->batch ||
        c->dvm_alloc < (uint64_t)c->L * ((num_vars + 31) / 32)) {
        free_graph(c);
        GRG_CUDA(c, cudaMalloc(&c->desc, std::max<uint64_t>(nt_all, 1) * 8));
        GRG_CUDA(c, cudaMalloc(&c->cnt, std::max<uint64_t>(nt_all, 1) * 4));
        GRG_CUDA(c, cudaMalloc(&c->want, std::max<uint64_t>(nt_all, 1) * 4));
        GRG_CUDA(c, cudaMalloc(&c->grow, std::max<uint64_t>(nt_all, 1) * 4));
        c->ntables_alloc = nt_all;
        int st0 = alloc_dindex(c);
        if (st0) return st0;
    }
    cudaStream_t s = c->stream;
    GRG_CUDA(c, cudaMemsetAsync(c->desc, 0, nt_all * 8, s));
    GRG_CUDA(c, cudaMemsetAsync(c->cnt, 0, nt_all * 4, s));
    GRG_CUDA(c, cudaMemsetAsync(c->want, 0, nt_all * 4, s));
    GRG_CUDA(c, cudaMemsetAsync(c->ctr, 0, sizeof(unsigned long long) * NCTR, s));
    c->loaded = false;
    c->closed = false;
    return GRG_OK;
}

// Labels on a rule's left-hand side get tables of DERIVED_MIN_CAP slots when
// that fits in half of the pool (fewer growths, rows stay in allocation order).
MinCap derived_min_cap(const grg_ctx *c)
{
    MinCap mc;
    memset(&mc, 0, sizeof mc);
    int nder = 0;
    bool lhs[MAX_LABELS + 1] = {false};
    for (int q = 0; q < c->R; q++) lhs[c->rules[3 * q]] = true;
    for (int l = 1; l <= c->L; l++) nder += lhs[l];
    if ((uint64_t)nder * c->V * DERIVED_MIN_CAP <= c->pool_cap / 2)
        for (int l = 1; l <= c->L; l++) mc.cap[l] = lhs[l] ? DERIVED_MIN_CAP : 0;
    return mc;
}

// Size and bump-allocate every table from the histogram that `hist` builds in
// cnt; the pool grows (and the histogram is rebuilt) until the tables fit.
// Clears the allocated region. Returns the pool top in *top.
template <class Hist>
int alloc_tables(grg_ctx *c, const MinCap &mc, Hist hist, uint64_t *top, const uint32_t *rowmark = nullptr)
{
    cudaStream_t s = c->stream;
    hist(make_dev(c));
    for (int attempt = 0;; attempt++) {
        GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_POOL_TOP, 0, 8, s));
        GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_ERR, 0, 8, s));
        k_load_alloc<<<grid_for(c, c->ntables, 256), 256, 0, s>>>(make_dev(c), 0, c->V, (uint32_t)c->L, mc, rowmark);
        c->launches++;
        int st = read_ctr(c);
        if (st) return st;
        if (!(c->h_ctr[C_ERR] & ERR_POOL)) break;
        if (attempt > 8) return fail(c, GRG_E_NOMEM, "element pool too small for the input graph");
        // the histogram was consumed: rebuild it after growing the pool
        st = grow_pool(c, c->h_ctr[C_POOL_TOP] + c->h_ctr[C_POOL_TOP] / 2);
        if (st) return st;
        GRG_CUDA(c, cudaMemsetAsync(c->cnt, 0, c->ntables * 4, s));
        hist(make_dev(c));
    }
    *top = c->h_ctr[C_POOL_TOP];
    GRG_CUDA(c, cudaMemsetAsync(c->dmap, 0, (c->pool_cap / 32 + 2) * 4, s));
    if (*top) {
        k_init_region<<<grid_for(c, *top, 256), 256, 0, s>>>(c->elems, c->dbits, c->elem_loaded ? c->stamp : nullptr,
                                                             0, *top);
        c->launches++;
    }
    return GRG_OK;
}

}  // namespace

extern "C" {

int grg_load_edges(grg_ctx *c, uint32_t num_vars, uint64_t num_edges, const uint32_t *src, const uint32_t *dst,
                   const uint8_t *label, int on_device)
{
    if (!c || (num_edges && (!src || !dst || !label))) return GRG_E_ARG;
    if (!c->have_rules) return fail(c, GRG_E_STATE, "grg_transfer_rules must come first");
    cudaSetDevice(c->device);
    c->elem_loaded = false;
    int st = setup_tables(c, num_vars);
    if (st) return st;
    c->tmask = c->layout_mode ? plan_columns(c->rules, c->R, c->L) : 0;
    cudaStream_t s = c->stream;
    const uint32_t *dsrc = src, *ddst = dst;
    const uint8_t *dlab = label;
    if (!on_device && num_edges) {
        st = ensure_input(c, num_edges);
        if (st) return st;
        GRG_CUDA(c, cudaMemcpyAsync(c->d_in32, src, num_edges * 4, cudaMemcpyHostToDevice, s));
        GRG_CUDA(c, cudaMemcpyAsync(c->d_in32 + num_edges, dst, num_edges * 4, cudaMemcpyHostToDevice, s));
        GRG_CUDA(c, cudaMemcpyAsync(c->d_in8, label, num_edges, cudaMemcpyHostToDevice, s));
        dsrc = c->d_in32;
        ddst = c->d_in32 + num_edges;
        dlab = c->d_in8;
    }
    c->launches = 0;
    auto hist = [&](Dev d) {
        if (num_edges) {
            k_load_hist<<<grid_for(c, num_edges, 256), 256, 0, s>>>(d, dsrc, ddst, dlab, num_edges, 0, num_vars, (uint32_t)c->L,
                                                                    c->tmask);
            c->launches++;
        }
        for (int q = 0; q < c->R; q++)
            if (c->rules[3 * q + 1] == 0) {
                k_eps_hist<<<grid_for(c, num_vars, 256), 256, 0, s>>>(d, (uint32_t)c->rules[3 * q], 0, num_vars);
                c->launches++;
            }
    };
    // derived rows start presized when the device can hold them: grow the pool for it
    {
        int nder = 0;
        bool lhs[MAX_LABELS + 1] = {false};
        for (int q = 0; q < c->R; q++) lhs[c->rules[3 * q]] = true;
        for (int l = 1; l <= c->L; l++) nder += lhs[l];
        const uint64_t want = 2ull * nder * num_vars * DERIVED_MIN_CAP + 2 * num_edges;
        if (want > c->pool_cap) {
            size_t fr = 0, tot = 0;
            cudaMemGetInfo(&fr, &tot);
            const uint64_t fit = (uint64_t)((double)fr * 0.6) / (POOL_BYTES_PER_SLOT + 4);
            if (fit > c->pool_cap && (!c->pool_limit || c->pool_limit > c->pool_cap)) {
                st = grow_pool(c, std::min(want, fit));
                if (st) return st;
            }
        }
    }
    uint64_t top = 0;
    st = alloc_tables(c, derived_min_cap(c), hist, &top);
    if (st) return st;
    if ((st = input_status(c))) return st;
    Dev d = make_dev(c);
    if (num_edges) {
        k_load_insert<<<grid_for(c, num_edges, 256), 256, 0, s>>>(d, dsrc, ddst, dlab, num_edges, 0, num_vars, (uint32_t)c->L,
                                                                  c->tmask);
        c->launches++;
    }
    for (int q = 0; q < c->R; q++)
        if (c->rules[3 * q + 1] == 0) {
            k_eps_insert<<<grid_for(c, num_vars, 256), 256, 0, s>>>(d, (uint32_t)c->rules[3 * q], 0, num_vars);
            c->launches++;
        }
    GRG_CUDA(c, cudaGetLastError());
    st = read_ctr(c);
    if (st) return st;
    if (c->h_ctr[C_ERR]) return fail(c, GRG_E_INTERNAL, "internal error while loading edges");
    c->loaded = true;
    c->closed = false;
    return GRG_OK;
}

int grg_load_elements(grg_ctx *c, uint32_t num_vars, uint64_t num_elems, const uint32_t *elems,
                      const uint32_t *stamps, uint32_t mark_after, int on_device)
{
    if (!c || (num_elems && (!elems || !stamps))) return GRG_E_ARG;
    if (!c->have_rules) return fail(c, GRG_E_STATE, "grg_transfer_rules must come first");
    cudaSetDevice(c->device);
    if (!c->stamp_on) {
        // the pool gains a stamp per slot from now on
        c->stamp_on = true;
        if (c->elems && !c->stamp) {
            if (cudaMalloc(&c->stamp, c->pool_cap * 4) != cudaSuccess) {
                cudaGetLastError();
                c->stamp = nullptr;
                c->stamp_on = false;
                return fail(c, GRG_E_NOMEM, "cannot allocate element stamps");
            }
        }
    }
    c->elem_loaded = true;
    int st = setup_tables(c, num_vars);
    if (st) return st;
    c->tmask = 0;                         // element images are rows by source
    cudaStream_t s = c->stream;
    const uint4 *drec = reinterpret_cast<const uint4 *>(elems);
    const uint32_t *dst_ = stamps;
    if (!on_device && num_elems) {
        if (c->xcap < num_elems) {
            cudaFree(c->xbuf); cudaFree(c->xst);
            c->xbuf = nullptr; c->xst = nullptr;
            c->xcap = 0;
            const uint64_t cap = num_elems + num_elems / 4;
            GRG_CUDA(c, cudaMalloc(&c->xbuf, cap * 32));
            GRG_CUDA(c, cudaMalloc(&c->xst, cap * 4));
            c->xcap = cap;
        }
        GRG_CUDA(c, cudaMemcpyAsync(c->xbuf, elems, num_elems * 32, cudaMemcpyHostToDevice, s));
        GRG_CUDA(c, cudaMemcpyAsync(c->xst, stamps, num_elems * 4, cudaMemcpyHostToDevice, s));
        drec = c->xbuf;
        dst_ = c->xst;
    }
    c->launches = 0;
    // rows the image holds: only those get presized derived rows
    const uint64_t mwords = ((uint64_t)num_vars + 31) / 32 + 1;
    if (c->rowmark_cap < mwords) {
        cudaFree(c->rowmark);
        c->rowmark = nullptr;
        c->rowmark_cap = 0;
        GRG_CUDA(c, cudaMalloc(&c->rowmark, mwords * 4));
        c->rowmark_cap = mwords;
    }
    auto hist = [&](Dev d) {
        GRG_CUDA(c, cudaMemsetAsync(c->rowmark, 0, mwords * 4, s));
        if (num_elems) {
            k_elem_hist<<<grid_for(c, num_elems, 256), 256, 0, s>>>(d, drec, num_elems, (uint32_t)c->L, c->rowmark);
            c->launches++;
        }
        return GRG_OK;
    };
    uint64_t top = 0;
    st = alloc_tables(c, derived_min_cap(c), hist, &top, c->rowmark);
    if (st) return st;
    if (num_elems) {
        k_elem_insert<<<grid_for(c, num_elems, 256), 256, 0, s>>>(make_dev(c), drec, dst_, num_elems, mark_after,
                                                                  (uint32_t)c->L);
        c->launches++;
    }
    GRG_CUDA(c, cudaGetLastError());
    st = read_ctr(c);
    if (st) return st;
    if (c->h_ctr[C_ERR]) return fail(c, GRG_E_ARG, "element records out of range or repeated");
    c->loaded = true;
    c->closed = false;
    return GRG_OK;
}

}  // extern "C"

// Kernel timing of a phase (join pass, gather): the global nanosecond timer at its start
// (t0_slot) and the elapsed time added at its end (acc_slot).
__global__ void k_tmark(unsigned long long *ctr, int t0_slot, int acc_slot, int end)
{
    if (threadIdx.x != 0 || ctr[C_HALT]) return;
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    if (!end)
        ctr[t0_slot] = t;
    else
        ctr[acc_slot] += t - ctr[t0_slot];
}

// Semi-naive rounds on the host's side: gather the dirty slots of the last
// round into delta records, join them, insert the candidates, re-run what did
// not fit after growing its tables. The pieces are separate so a round the
// device-driven loop hands back can be finished where it stopped.

// Window of this closure's joins. Measured on dataflow, alias, points-to and
// small alias jobs, the wide window was fastest or within 1.5% on every one, so
// it is the default; the narrow window stays selectable. Wide is 12 elements
// (5 below the run's base). A warp has 8 window slots, one per run of a row's
// records, and joins a batch of more runs in passes; a block takes 22 KB of
// shared memory, and at 64 registers a thread (some bytes spilled) 8 blocks fit
// an SM. Earlier layouts, measured on one box (2M-vertex dataflow / 1M alias
// closure): 16 slots with runs past the 16th in the hash, 10-element windows, 7
// blocks 54.4 / 317 ms; 32 slots (one per record) at 5 blocks 66.3 / 334 ms.
static void choose_window(grg_ctx *c)
{
    c->join_wide = c->join_window_mode >= 2 ? c->tuned_wide : c->join_window_mode != 0;
    c->join_elems = c->items_mode >= 2 ? c->tuned_elems : c->items_mode != 0;
    c->push_flat = c->push_mode >= 2 ? c->tuned_flat : c->push_mode != 0;
}

// The join kernel in the window chosen for this closure (join_wide), reading the
// right-hand rows of CSR-copied labels as ids or (join_elems) as table elements.
static void launch_join(const grg_ctx *c, int grid, cudaStream_t s, const Dev &d, const uint4 *recs, uint64_t n,
                        int n_ctr, uint4 *retry_out)
{
    const Dev *dp = &d;
    Dev de;
    if (c->join_elems) {
        de = d;
        for (int l = 0; l <= MAX_LABELS; l++) de.rt.csr_row[l] = nullptr;
        dp = &de;
    }
    // the launch's work queue starts at batch 0; the grid is what the SMs hold at once
    cudaMemsetAsync(d.ctr + C_JQ, 0, 8, s);
    const int resident = c->sms * (c->join_wide ? GRG_JOIN_MINB_WIDE : GRG_JOIN_MINB);
    if (grid > resident) grid = resident;
    if (c->join_wide)
        k_join<WIN2, WIN2_LO><<<grid, JOIN_WARPS * 32, 0, s>>>(*dp, recs, n, n_ctr, retry_out);
    else
        k_join<WIN, WIN_LO><<<grid, JOIN_WARPS * 32, 0, s>>>(*dp, recs, n, n_ctr, retry_out);
}

static bool any_csr(const grg_ctx *c)
{
    for (int l = 1; l <= c->L; l++)
        if (c->rt.csr_row[l]) return true;
    return false;
}

// Which pass kernels the rule table needs: k_join unless every record it could
// see belongs to a destination-stored label (pushed) or only feeds unary rules
// into one; k_push when a destination-stored label has records, or a unary rule
// turns a source-stored label into one.
static void set_passes(grg_ctx *c)
{
    const RuleTable &rt = c->rt;
    c->need_join = rt.nol > 0;
    c->need_push = false;
    for (int B = 1; B <= c->L; B++) {
        if (!rt.track[B]) continue;
        if (rt.tpose[B]) {
            c->need_push = true;
            continue;
        }
        if (rt.bin_start[B + 1] > rt.bin_start[B]) c->need_join = true;
        for (int u = rt.un_start[B]; u < rt.un_start[B + 1]; u++) {
            if (rt.tpose[rt.un_A[u]]) c->need_push = true;
            else c->need_join = true;
        }
    }
}

// One join pass over n records (or the device count n_ctr): the kernels the rule
// table needs, each taking its own records and skipping the others'.
static void launch_pass(grg_ctx *c, int grid, cudaStream_t s, const Dev &d, const uint4 *recs, uint64_t n, int n_ctr,
                        uint4 *retry_out, uint64_t &joins)
{
    if (c->need_join) {
        launch_join(c, grid, s, d, recs, n, n_ctr, retry_out);
        c->launches++;
        joins++;
    }
    if (c->need_push) {
        if (c->push_flat) {
            cudaMemsetAsync(d.ctr + C_JQ, 0, 8, s);
            k_push_flat<<<c->sms * 4, PUSH_WARPS * 32, 0, s>>>(d, recs, n, n_ctr, retry_out);
        } else
            k_push<<<c->sms * 8, 256, 0, s>>>(d, recs, n, n_ctr, retry_out);
        c->launches++;
        joins++;
    }
}

// ---------------------------------------------------------------- join-window tuning
//
// A closure's input is keyed by grammar, filter, vertex count and the share of
// its tables in each log2 size bucket (eighths). The first closure of a key
// whose first round is large enough to time joins a slice of that round's
// records in each window, keeps the faster window for the round, the rest of
// the closure and later closures with the key. Joining a record more than once
// is harmless: a join pass only appends candidates and retry records, and
// applying a candidate or re-running a record twice adds nothing.

static std::mutex g_tune_mu;
struct JoinChoice { bool wide, elems; };
static std::map<uint64_t, JoinChoice> g_tune_cache;    // degree key -> the faster window and item form
static std::map<uint64_t, bool> g_push_cache;          // degree key -> flattened push faster
constexpr uint64_t TUNE_MIN_RECORDS = 1u << 16;        // smaller first rounds are not timed
// The narrow window replaces the wide default only when the wide trial pass takes at least
// this long: the 1M-vertex alias closure's trials take ~26 us each, where the two windows
// swap places by more than the 10% margin from run to run, and the narrow window then
// costs ~11% over the closure
constexpr float TUNE_WINDOW_MIN_MS = 0.25f;

static int degree_key(grg_ctx *c, uint32_t filter, uint64_t *key)
{
    cudaStream_t s = c->stream;
    GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_DH0, 0, 8 * 8, s));
    if (c->V) k_degree_hist<<<grid_for(c, (uint64_t)c->L * c->V, 256), 256, 0, s>>>(make_dev(c), (uint32_t)c->L);
    c->launches++;
    int st = read_ctr(c);
    if (st) return st;
    uint64_t h = 1469598103934665603ull, tot = 0;
    auto mix = [&](uint64_t v) { h = (h ^ v) * 1099511628211ull; };
    mix((uint64_t)c->L);
    mix(filter);
    for (int q = 0; q < 3 * c->R; q++) mix((uint64_t)c->rules[q]);
    uint32_t vb = 0;
    while ((1ull << vb) < c->V) vb++;
    mix(vb);
    for (int b = 0; b < 8; b++) tot += c->h_ctr[C_DH0 + b];
    for (int b = 0; b < 8; b++) mix(tot ? c->h_ctr[C_DH0 + b] * 8 / tot : 0);
    *key = h;
    return GRG_OK;
}

// Sets the closure's window from the cache, or marks it for measurement.
static int tune_begin(grg_ctx *c, uint32_t filter)
{
    c->tune_pending = c->push_pending = false;
    c->tune_source = c->push_source = 0;
    c->tune_ms[0] = c->tune_ms[1] = 0;
    c->items_ms[0] = c->items_ms[1] = 0;
    c->push_ms[0] = c->push_ms[1] = 0;
    // only the choices this closure's pass kernels make are tuned (the window is
    // k_join's; the push kernel is timed only when the pass is pushes alone)
    const bool tune_window = (c->join_window_mode >= 2 || c->items_mode >= 2) && c->need_join;
    const bool tune_push = c->push_mode >= 2 && c->need_push && !c->need_join;
    if (!tune_window && !tune_push) return GRG_OK;
    int st = degree_key(c, filter, &c->tune_key);
    if (st) return st;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    if (tune_window) {
        auto it = g_tune_cache.find(c->tune_key);
        if (it != g_tune_cache.end() && c->join_window_mode != 3 && c->items_mode != 3) {
            c->tuned_wide = it->second.wide;
            c->tuned_elems = it->second.elems;
            c->tune_source = 2;
        } else {
            c->tuned_wide = true;
            c->tuned_elems = false;
            c->tune_pending = true;
        }
    }
    if (tune_push) {
        auto it = g_push_cache.find(c->tune_key);
        if (it != g_push_cache.end() && c->push_mode == 2) {
            c->tuned_flat = it->second;
            c->push_source = 2;
        } else {
            c->tuned_flat = true;
            c->push_pending = true;
        }
    }
    return GRG_OK;
}

static void first_pass_joins(grg_ctx *c, const Dev &d, uint64_t nd, uint64_t nv, bool split, uint64_t &joins);

// The first pass of a round with its window measured (see above): both windows
// are timed twice, interleaved, on a slice of the round's records (an eighth, at
// least TUNE_MIN_RECORDS), after an untimed pass over the slice that warms the
// caches; narrow is taken only when its best time beats wide's by 10% (slices
// of one round differ by a few percent between runs). Then the whole round
// runs in the chosen window.
static int tune_first_pass(grg_ctx *c, const Dev &d, uint64_t nd, uint64_t nv, uint64_t &joins)
{
    cudaStream_t s = c->stream;
    if (!c->ev_t0) GRG_CUDA(c, cudaEventCreate(&c->ev_t0));
    if (!c->ev_t1) GRG_CUDA(c, cudaEventCreate(&c->ev_t1));
    int st = read_ctr(c);
    if (st) return st;
    const int kept[5] = {C_LEFT, C_RIGHT, C_WOUT, C_NOSLOT, C_INSERTS};
    unsigned long long keep[5];
    for (int i = 0; i < 5; i++) keep[i] = c->h_ctr[kept[i]];
    const uint64_t nt = std::min(nd, std::max<uint64_t>(TUNE_MIN_RECORDS, nd / 8));
    const int grid = grid_for(c, (nt + RB - 1) / RB, JOIN_WARPS, 16);
    // the choices open in this closure: windows unless fixed, item forms unless fixed or no
    // right-hand label has a CSR copy; an untimed pass, then every combination twice,
    // interleaved, keeping each one's best time
    const bool tw = c->join_window_mode >= 2, ti = c->items_mode >= 2 && any_csr(c);
    const bool fix_wide = c->join_wide, fix_elems = c->join_elems;
    float best[2][2] = {{1e30f, 1e30f}, {1e30f, 1e30f}};        // [wide][elems]
    for (int rep = -1; rep < 2; rep++)
        for (int w = 0; w < 2; w++)
            for (int e = 0; e < 2; e++) {
                if ((!tw && w != (int)fix_wide) || (!ti && e != (int)fix_elems)) continue;
                if (rep < 0 && !(w == 1 || !tw)) continue;         // one untimed (wide) pass per item form
                c->join_wide = w == 1;
                c->join_elems = e == 1;
                if (rep >= 0) GRG_CUDA(c, cudaEventRecord(c->ev_t0, s));
                launch_join(c, grid, s, d, c->gbuf, nt, -1, c->rbuf[0]);
                c->launches++;
                joins++;
                if (rep < 0) continue;
                float ms = 0;
                GRG_CUDA(c, cudaEventRecord(c->ev_t1, s));
                GRG_CUDA(c, cudaEventSynchronize(c->ev_t1));
                GRG_CUDA(c, cudaEventElapsedTime(&ms, c->ev_t0, c->ev_t1));
                best[w][e] = std::min(best[w][e], ms);
            }
    // the statistics count the round's own pass only
    for (int i = 0; i < 5; i++) {
        c->h_ctr[kept[i]] = keep[i];
        GRG_CUDA(c, cudaMemcpyAsync(c->ctr + kept[i], c->h_ctr + kept[i], 8, cudaMemcpyHostToDevice, s));
    }
    // the trial passes' retry records and candidates are dropped: the round's own pass
    // below joins every record again. Tables they queued for growth stay queued (their
    // want counters are set, so the real pass would not queue them a second time).
    GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_RETRY_N, 0, 8, s));
    GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_CAND_N, 0, 16, s));    // candidates + failed candidates
    // per item form, the wide window is the measured default (faster on every workload
    // swept): narrow must win by a margin the trial's noise cannot produce; then the faster
    // item form with its window
    bool wide_of[2];
    float t_of[2];
    for (int e = 0; e < 2; e++) {
        wide_of[e] = tw ? !(best[0][e] < 0.9f * best[1][e] && best[1][e] >= TUNE_WINDOW_MIN_MS) : fix_wide;
        t_of[e] = best[wide_of[e] ? 1 : 0][e];
    }
    const bool elems = ti ? t_of[1] < t_of[0] : fix_elems;
    const bool wide = wide_of[elems ? 1 : 0];
    c->tune_ms[0] = best[0][elems ? 1 : 0] < 1e29f ? best[0][elems ? 1 : 0] : 0.f;
    c->tune_ms[1] = best[1][elems ? 1 : 0] < 1e29f ? best[1][elems ? 1 : 0] : 0.f;
    c->items_ms[0] = ti ? t_of[0] : 0.f;
    c->items_ms[1] = ti ? t_of[1] : 0.f;
    c->tuned_wide = c->join_wide = wide;
    c->tuned_elems = c->join_elems = elems;
    c->tune_pending = false;
    c->tune_source = 1;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_cache[c->tune_key] = JoinChoice{wide, elems};
    }
    first_pass_joins(c, d, nd, nv, false, joins);
    return GRG_OK;
}

// The first pass of a round whose join pass is pushes only, with the push kernel
// measured: one lane per record and edges dealt over the lanes, each timed twice,
// interleaved, on a slice of the round's records after an untimed pass; the
// faster is kept for this closure and later closures with the degree key.
// Pushing a record again adds nothing twice.
static int tune_push_pass(grg_ctx *c, const Dev &d, uint64_t nd, uint64_t nv, uint64_t &joins)
{
    cudaStream_t s = c->stream;
    if (!c->ev_t0) GRG_CUDA(c, cudaEventCreate(&c->ev_t0));
    if (!c->ev_t1) GRG_CUDA(c, cudaEventCreate(&c->ev_t1));
    int st = read_ctr(c);
    if (st) return st;
    const int kept[2] = {C_LEFT, C_RIGHT};
    unsigned long long keep[2];
    for (int i = 0; i < 2; i++) keep[i] = c->h_ctr[kept[i]];
    const uint64_t nt = std::min(nd, std::max<uint64_t>(TUNE_MIN_RECORDS, nd / 8));
    c->push_ms[0] = c->push_ms[1] = 1e30f;
    for (int it = -1; it < 4; it++) {
        const int k = it < 0 ? 1 : it & 1;     // 0 one lane per record, 1 flattened
        c->push_flat = k == 1;
        if (it >= 0) GRG_CUDA(c, cudaEventRecord(c->ev_t0, s));
        launch_pass(c, 0, s, d, c->gbuf, nt, -1, c->rbuf[0], joins);
        if (it < 0) continue;
        float ms = 0;
        GRG_CUDA(c, cudaEventRecord(c->ev_t1, s));
        GRG_CUDA(c, cudaEventSynchronize(c->ev_t1));
        GRG_CUDA(c, cudaEventElapsedTime(&ms, c->ev_t0, c->ev_t1));
        c->push_ms[k] = std::min(c->push_ms[k], ms);
    }
    for (int i = 0; i < 2; i++) {
        c->h_ctr[kept[i]] = keep[i];
        GRG_CUDA(c, cudaMemcpyAsync(c->ctr + kept[i], c->h_ctr + kept[i], 8, cudaMemcpyHostToDevice, s));
    }
    // the trial passes' retry records are dropped: the round's own pass pushes every record again
    GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_RETRY_N, 0, 8, s));
    const bool flat = c->push_ms[1] <= c->push_ms[0];
    c->tuned_flat = c->push_flat = flat;
    c->push_pending = false;
    c->push_source = 1;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_push_cache[c->tune_key] = flat;
    }
    first_pass_joins(c, d, nd, nv, false, joins);
    return GRG_OK;
}

// Round head: count and gather the dirty slots (rs: stamp for elements that
// gained bits, 0 = none). *nd = delta records (0 = fixpoint).
static int round_head(grg_ctx *c, uint32_t rs, grg_stats &S, uint64_t *nd_out)
{
    cudaStream_t s = c->stream;
    if (c->job_cnt) GRG_CUDA(c, cudaMemsetAsync(c->job_cnt, 0, (size_t)c->max_jobs * 4, s));
    // the pool top is the one read after the last growth
    const uint64_t nwords = (c->h_ctr[C_POOL_TOP] + 31) / 32;
    const uint64_t nchunks = (nwords + 31) / 32;
    int st = ensure_chunks(c, nchunks);
    if (st) return st;
    uint32_t *ccnt = c->chunk, *coff = c->chunk + nchunks + 1, *csum = c->chunk + 2 * (nchunks + 1);
    const uint64_t nb = (nchunks + 1023) / 1024;
    Dev d = make_dev(c);
    if (c->timing) k_tmark<<<1, 32, 0, s>>>(c->ctr, C_GT0, C_GNS, 0);
    k_dcount<<<grid_for(c, nchunks * 32, 256), 256, 0, s>>>(d, nwords, ccnt, 0);
    k_scan_blocks<<<(unsigned)std::max<uint64_t>(nb, 1), 1024, 0, s>>>(ccnt, coff, csum, nchunks, nullptr);
    k_scan_sums<<<1, 1024, 0, s>>>(csum, nb, nullptr);
    k_scan_add<<<(unsigned)std::max<uint64_t>(nb, 1), 1024, 0, s>>>(coff, csum, nchunks, nullptr);
    c->launches += 4;
    GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_DIRTY_N, 0, 8, s));
    GRG_CUDA(c, cudaMemcpyAsync(c->ctr + C_DIRTY_N, csum + nb, 4, cudaMemcpyDeviceToDevice, s));
    GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_RETRY_N, 0, 16, s));   // retry + grow counters
    GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_CAND_N, 0, 16, s));    // candidates + failed candidates
    st = read_ctr(c);
    if (st) return st;
    const uint64_t nd = c->h_ctr[C_DIRTY_N];
    *nd_out = nd;
    if (nd == 0) return GRG_OK;
    st = ensure_gather(c, nd);
    if (st) return st;
    st = ensure_cand(c, nd);
    if (st) return st;
    S.rounds++;
    S.delta_elems += nd;
    c->cb = 0;
    d = make_dev(c);
    // the delta index of the last round is cleared for the labels old-left joins read
    for (int l = 1; l <= c->L; l++)
        if (c->rt.dindex[l]) {
            const size_t t0 = (size_t)(l - 1) * c->V, vw = (c->V + 31) / 32;
            GRG_CUDA(c, cudaMemsetAsync(c->drs + t0, 0xFF, (size_t)c->V * 4, s));
            GRG_CUDA(c, cudaMemsetAsync(c->drc + t0, 0, (size_t)c->V * 4, s));
            GRG_CUDA(c, cudaMemsetAsync(c->dvm + (size_t)(l - 1) * vw, 0, vw * 4, s));
        }
    k_gather_slots<<<grid_for(c, nchunks * 32, 256), 256, 0, s>>>(d, nwords, coff, c->gslot, 0);
    k_gather_recs<<<grid_for(c, nd, 256), 256, 0, s>>>(d, c->gslot, c->gbuf, nd, -1, c->row_job, c->job_cnt, rs);
    c->launches += 2;
    if (c->timing) k_tmark<<<1, 32, 0, s>>>(c->ctr, C_GT0, C_GNS, 1);
    return GRG_OK;
}

// Old-left joins: virtual records of O_B masked to the vertices with deltas of C.
static int round_oldleft(grg_ctx *c, uint64_t *nv_out)
{
    cudaStream_t s = c->stream;
    uint64_t nv = 0;
    if (c->rt.nol) {
        for (int attempt = 0; attempt < 2; attempt++) {
            Dev d = make_dev(c);
            GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_VN, 0, 8, s));
            for (int q = 0; q < c->rt.nol; q++) {
                k_oldleft<<<grid_for(c, c->V, 256), 256, 0, s>>>(d, (uint32_t)q, c->vbuf, c->vbuf_cap, c->row_job,
                                                                 c->job_cnt);
                c->launches++;
            }
            int st = read_ctr(c);
            if (st) return st;
            nv = c->h_ctr[C_VN];
            if (nv <= c->vbuf_cap) break;
            st = ensure_buf(c, &c->vbuf, &c->vbuf_cap, nv);
            if (st) return st;
        }
    }
    *nv_out = nv;
    return GRG_OK;
}

// Tables that overflowed grow (the pool too, when it is full); then the failed
// records (rbuf[0]) and failed candidates (cand[cb ^ 1]) of the round's first
// pass are re-run until nothing fails.
// Retry list size for a round of n records: retries come only from tables at
// their load limit, a small share; a round with more is re-run whole.
static uint64_t retry_room(const grg_ctx *c, uint64_t n) { return std::max<uint64_t>(c->retry_min, n / 8); }

// The first join pass of a round over its records: the parts of a small round
// (sub-records in sbuf, count on the device) or the gathered and virtual records.
static void first_pass_joins(grg_ctx *c, const Dev &d, uint64_t nd, uint64_t nv, bool split, uint64_t &joins)
{
    cudaStream_t s = c->stream;
    if (split) {
        launch_pass(c, grid_for(c, ((nd + nv) * SPLIT_PARTS + RB - 1) / RB, JOIN_WARPS, 16), s, d, c->sbuf, 0,
                    C_SPLIT_N, c->rbuf[0], joins);
        return;
    }
    launch_pass(c, grid_for(c, (nd + RB - 1) / RB, JOIN_WARPS, 16), s, d, c->gbuf, nd, -1, c->rbuf[0], joins);
    if (nv) {
        // virtual old-left records: joined by source rows only
        launch_join(c, grid_for(c, (nv + RB - 1) / RB, JOIN_WARPS, 16), s, d, c->vbuf, nv, -1, c->rbuf[0]);
        c->launches++;
        joins++;
    }
}

// Tables that overflowed grow (the pool too, when it is full); then the failed
// records (rbuf[0]) and failed candidates (cand[cb ^ 1]) of the round's first
// pass are re-run until nothing fails. When more records failed than the retry
// list holds, the round's whole first pass is re-run instead (joining a record
// again adds nothing twice).
static int round_retries(grg_ctx *c, uint64_t nr, uint64_t nf, grg_stats &S, double &join_ms, uint64_t &joins,
                         uint64_t nd, uint64_t nv, bool split)
{
    cudaStream_t s = c->stream;
    int rb = 0;    // the failed records of the last pass are in rbuf[rb]
    for (int pass = 1;; pass++) {
        if (nr == 0 && nf == 0) return GRG_OK;
        S.retry_records += nr + nf;
        const bool rerun_all = nr > c->rbuf_cap;
        Dev d = make_dev(c);
        for (int gtry = 0;; gtry++) {
            const uint64_t ng = c->h_ctr[C_GROW_N];
            GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_ERR, 0, 8, s));
            k_grow<<<grid_for(c, ng * 32, 256), 256, 0, s>>>(d, ng);
            c->launches++;
            S.grow_rows += ng;
            int st = read_ctr(c);
            if (st) return st;
            if (!(c->h_ctr[C_ERR] & ERR_POOL)) break;
            if (gtry > 16) return fail(c, GRG_E_NOMEM, "element pool exhausted");
            st = grow_pool(c, c->pool_cap * 2);
            if (st) return st;
            d = make_dev(c);
        }
        if (pass > 64) return fail(c, GRG_E_INTERNAL, "table growth did not converge in 64 passes");
        // failed candidates (in cand[cb^1]) become the candidate list; join retries append to it
        c->cb ^= 1;
        d = make_dev(c);
        c->h_ctr[C_CAND_N] = nf;
        GRG_CUDA(c, cudaMemcpyAsync(c->ctr + C_CAND_N, c->h_ctr + C_CAND_N, 8, cudaMemcpyHostToDevice, s));
        GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_AFAIL, 0, 8, s));
        GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_RETRY_N, 0, 16, s));
        if (c->timing) GRG_CUDA(c, cudaEventRecord(c->ev_c, s));
        if (rerun_all) {
            first_pass_joins(c, d, nd, nv, split, joins);
            rb = 0;
        } else if (nr) {
            launch_pass(c, grid_for(c, (nr + RB - 1) / RB, JOIN_WARPS, 16), s, d, c->rbuf[rb], nr, -1, c->rbuf[rb ^ 1],
                        joins);
            rb ^= 1;
        }
        if (c->cand_cap) {
            k_apply<<<c->sms * GRG_APPLY_MINB, 256, 0, s>>>(d, c->cand[c->cb], c->cand[c->cb ^ 1]);
            c->launches++;
        }
        if (c->timing) GRG_CUDA(c, cudaEventRecord(c->ev_d, s));
        GRG_CUDA(c, cudaGetLastError());
        int st = read_ctr(c);
        if (st) return st;
        if (c->timing) {
            float ms = 0;
            cudaEventElapsedTime(&ms, c->ev_c, c->ev_d);
            join_ms += ms;
        }
        nr = c->h_ctr[C_RETRY_N];
        nf = c->cand_cap ? c->h_ctr[C_AFAIL] : 0;
    }
}

// First join pass of a round over its nd gathered and nv virtual records, then retries.
static int ensure_sbuf(grg_ctx *c)
{
    if (c->sbuf) return GRG_OK;
    GRG_CUDA(c, cudaMalloc(&c->sbuf, (size_t)SPLIT_MAX * SPLIT_PARTS * 32));
    return GRG_OK;
}

static int round_joins(grg_ctx *c, uint64_t nd, uint64_t nv, grg_stats &S, double &join_ms, uint64_t &joins)
{
    cudaStream_t s = c->stream;
    const bool split = nd + nv < SPLIT_MAX;
    int st = ensure_rbuf(c, retry_room(c, nd + nv));
    if (st) return st;
    if (split && (st = ensure_sbuf(c))) return st;
    Dev d = make_dev(c);
    if (c->timing) GRG_CUDA(c, cudaEventRecord(c->ev_c, s));
    if (split) {
        // few records: their parts spread the join over more warps
        GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_SPLIT_N, 0, 8, s));
        k_split<<<grid_for(c, nd + nv, 256), 256, 0, s>>>(d, c->gbuf, c->vbuf, c->sbuf);
        c->launches++;
    }
    if (c->tune_pending && c->need_join && !split && nd >= TUNE_MIN_RECORDS) {
        if ((st = tune_first_pass(c, d, nd, nv, joins))) return st;
    } else if (c->push_pending && c->need_push && !c->need_join && !split && nd >= TUNE_MIN_RECORDS) {
        if ((st = tune_push_pass(c, d, nd, nv, joins))) return st;
    } else {
        first_pass_joins(c, d, nd, nv, split, joins);
    }
    // insert the candidates the joins wrote (count read on the device)
    if (c->cand_cap) {
        k_apply<<<c->sms * GRG_APPLY_MINB, 256, 0, s>>>(d, c->cand[c->cb], c->cand[c->cb ^ 1]);
        c->launches++;
    }
    if (c->timing) GRG_CUDA(c, cudaEventRecord(c->ev_d, s));
    GRG_CUDA(c, cudaGetLastError());
    st = read_ctr(c);
    if (st) return st;
    if (c->timing) {
        float ms = 0;
        cudaEventElapsedTime(&ms, c->ev_c, c->ev_d);
        join_ms += ms;
    }
    return round_retries(c, c->h_ctr[C_RETRY_N], c->cand_cap ? c->h_ctr[C_AFAIL] : 0, S, join_ms, joins, nd, nv,
                         split);
}

// ---------------------------------------------------------------- device-driven rounds
//
// After the first round, closure rounds run from a CUDA graph whose WHILE node
// repeats one round -- count/scan/gather, old-left records, joins, apply --
// with every size read on the device, so the host neither waits nor launches
// per round. Gate kernels end the loop when the host is needed: the fixpoint,
// a buffer too small for the round, or tables to grow (the rare retry path);
// the host then finishes that round with the functions above and relaunches.

enum : unsigned long long {
    HALT_FIXPOINT = 1, HALT_CAPACITY = 2, HALT_OLDLEFT = 3, HALT_RETRY = 4, HALT_LIMIT = 5, HALT_ROUNDS = 6
};
constexpr uint64_t GATE_MAX_ITERS = 1u << 20;   // iterations of one graph launch; past it the host takes over

__global__ void k_gate_gather(unsigned long long *ctr, const uint32_t *csum, uint64_t max_chunks, uint64_t gbuf_cap,
                              uint64_t max_iters, cudaGraphConditionalHandle h)
{
    if (threadIdx.x != 0) return;
    const unsigned long long it = ++ctr[C_ITERS];
    if (ctr[C_HALT] || it > max_iters) {
        if (!ctr[C_HALT]) ctr[C_HALT] = HALT_LIMIT;
        cudaGraphSetConditional(h, 0);
        return;
    }
    const uint64_t nb = (dyn_chunks(max_chunks, ctr) + 1023) / 1024;
    const uint64_t nd = csum[nb];
    ctr[C_DIRTY_N] = nd;
    const unsigned long long halt = nd == 0 ? HALT_FIXPOINT : nd > gbuf_cap ? HALT_CAPACITY : 0;
    if (halt) {
        ctr[C_HALT] = halt;                  // later kernels of this iteration return at once
        cudaGraphSetConditional(h, 0);
        return;
    }
    ctr[C_GROUNDS]++;
    ctr[C_GDSUM] += nd;
}

__global__ void k_gate_oldleft(unsigned long long *ctr, uint64_t vbuf_cap, cudaGraphConditionalHandle h)
{
    if (threadIdx.x != 0 || ctr[C_HALT]) return;
    const uint64_t nv = ctr[C_VN];
    if (nv > vbuf_cap) {
        ctr[C_HALT] = HALT_OLDLEFT;
        cudaGraphSetConditional(h, 0);
    }
}

__global__ void k_gate_end(unsigned long long *ctr, cudaGraphConditionalHandle h)
{
    if (threadIdx.x != 0 || ctr[C_HALT]) return;
    if (ctr[C_RETRY_N] || ctr[C_AFAIL]) {
        ctr[C_HALT] = HALT_RETRY;
        cudaGraphSetConditional(h, 0);
    } else if (ctr[C_MAXR] && ctr[C_GROUNDS] >= ctr[C_MAXR]) {
        // the round budget of this launch is spent; per-job counts of this round stay for the host
        ctr[C_HALT] = HALT_ROUNDS;
        cudaGraphSetConditional(h, 0);
    }
}


static void free_round_graph(grg_ctx *c)
{
    if (c->rg_exec) cudaGraphExecDestroy(c->rg_exec);
    if (c->rg_graph) cudaGraphDestroy(c->rg_graph);
    c->rg_exec = nullptr;
    c->rg_graph = nullptr;
    c->rg_key.clear();
}

// Everything the recorded launches hold by value.
static std::vector<uint64_t> round_graph_key(const grg_ctx *c, uint32_t rs, uint64_t nchunks)
{
    std::vector<uint64_t> k = {(uint64_t)c->elems, (uint64_t)c->dbits, (uint64_t)c->dmap, (uint64_t)c->stamp,
                               (uint64_t)c->desc, (uint64_t)c->cnt, (uint64_t)c->want, (uint64_t)c->grow,
                               (uint64_t)c->gbuf, c->gbuf_cap, (uint64_t)c->gslot, (uint64_t)c->vbuf, c->vbuf_cap,
                               (uint64_t)c->rbuf[0], (uint64_t)c->rbuf[1], c->rbuf_cap, (uint64_t)c->cand[0],
                               (uint64_t)c->cand[1], c->cand_cap, (uint64_t)c->chunk, nchunks, (uint64_t)c->drs,
                               (uint64_t)c->drc, (uint64_t)c->dvm, c->pool_cap, c->V, rs, (uint64_t)c->timing,
                               (uint64_t)c->elem_loaded, (uint64_t)c->rt.nol, (uint64_t)c->row_job,
                               (uint64_t)c->job_cnt, c->max_jobs, (uint64_t)c->join_wide, (uint64_t)c->sbuf,
                               (uint64_t)c->need_join, (uint64_t)c->need_push, (uint64_t)c->push_flat,
                               (uint64_t)c->join_elems};
    for (int l = 1; l <= c->L; l++) k.push_back(c->rt.dindex[l]);
    // the rule table is a parameter of every recorded launch
    uint64_t w[(sizeof(RuleTable) + 7) / 8] = {0};
    memcpy(w, &c->rt, sizeof(RuleTable));
    k.insert(k.end(), w, w + (sizeof(RuleTable) + 7) / 8);
    return k;
}

static int build_round_graph(grg_ctx *c, uint32_t rs)
{
    const uint64_t nwords = c->pool_cap / 32 + 2, nchunks = (nwords + 31) / 32, nb = (nchunks + 1023) / 1024;
    int st = ensure_chunks(c, nchunks);
    if (st) return st;
    std::vector<uint64_t> key = round_graph_key(c, rs, nchunks);
    if (c->rg_exec && key == c->rg_key) return GRG_OK;
    free_round_graph(c);
    if (!c->cap_stream) GRG_CUDA(c, cudaStreamCreateWithFlags(&c->cap_stream, cudaStreamNonBlocking));
    cudaStream_t s = c->cap_stream;
    GRG_CUDA(c, cudaGraphCreate(&c->rg_graph, 0));
    cudaGraphConditionalHandle h;
    GRG_CUDA(c, cudaGraphConditionalHandleCreate(&h, c->rg_graph, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams p = {};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = h;
    p.conditional.type = cudaGraphCondTypeWhile;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    GRG_CUDA(c, cudaGraphAddNode(&node, c->rg_graph, nullptr, nullptr, 0, &p));
    cudaGraph_t body = p.conditional.phGraph_out[0];
    GRG_CUDA(c, cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    const int saved_cb = c->cb;
    c->cb = 0;
    Dev d = make_dev(c);
    c->cb = saved_cb;
    uint32_t *ccnt = c->chunk, *coff = c->chunk + nchunks + 1, *csum = c->chunk + 2 * (nchunks + 1);
    unsigned long long *ctr = c->ctr;
    int nk = 0;
    bool any_dindex = false;
    for (int l = 1; l <= c->L; l++) any_dindex |= c->rt.dindex[l] != 0;
    if (any_dindex) {
        // first in the body: C_DIRTY_N still counts the previous round's records in gbuf
        k_dindex_clear<<<grid_for(c, c->gbuf_cap, 256), 256, 0, s>>>(d, c->gbuf, C_DIRTY_N);
        nk++;
    }
    cudaMemsetAsync(ctr + C_RETRY_N, 0, 16, s);
    cudaMemsetAsync(ctr + C_CAND_N, 0, 16, s);
    if (c->job_cnt) cudaMemsetAsync(c->job_cnt, 0, (size_t)c->max_jobs * 4, s);
    if (c->timing) {
        k_tmark<<<1, 32, 0, s>>>(ctr, C_GT0, C_GNS, 0);
        nk++;
    }
    k_dcount<<<grid_for(c, nchunks * 32, 256), 256, 0, s>>>(d, nwords, ccnt, 1);
    k_scan_blocks<<<(unsigned)std::max<uint64_t>(nb, 1), 1024, 0, s>>>(ccnt, coff, csum, nchunks, ctr);
    k_scan_sums<<<1, 1024, 0, s>>>(csum, nb, ctr);
    k_scan_add<<<(unsigned)std::max<uint64_t>(nb, 1), 1024, 0, s>>>(coff, csum, nchunks, ctr);
    k_gate_gather<<<1, 32, 0, s>>>(ctr, csum, nchunks, c->gbuf_cap, GATE_MAX_ITERS, h);
    nk += 5;
    cudaMemsetAsync(ctr + C_VN, 0, 8, s);
    k_gather_slots<<<grid_for(c, nchunks * 32, 256), 256, 0, s>>>(d, nwords, coff, c->gslot, 1);
    k_gather_recs<<<grid_for(c, c->gbuf_cap, 256), 256, 0, s>>>(d, c->gslot, c->gbuf, 0, C_DIRTY_N, c->row_job,
                                                                c->job_cnt, rs);
    nk += 2;
    if (c->timing) {
        k_tmark<<<1, 32, 0, s>>>(ctr, C_GT0, C_GNS, 1);
        nk++;
    }
    if (c->rt.nol) {
        for (int q = 0; q < c->rt.nol; q++)
            k_oldleft<<<grid_for(c, c->V, 256), 256, 0, s>>>(d, (uint32_t)q, c->vbuf, c->vbuf_cap, c->row_job,
                                                             c->job_cnt);
        k_gate_oldleft<<<1, 32, 0, s>>>(ctr, c->vbuf_cap, h);
        nk += c->rt.nol + 1;
    }
    if (c->timing) {
        k_tmark<<<1, 32, 0, s>>>(ctr, C_JT0, C_JNS, 0);
        nk++;
    }
    const int jgrid = grid_for(c, ~0u, JOIN_WARPS, 16);
    cudaMemsetAsync(ctr + C_SPLIT_N, 0, 8, s);
    k_split<<<grid_for(c, SPLIT_MAX, 256), 256, 0, s>>>(d, c->gbuf, c->vbuf, c->sbuf);
    nk++;
    {
        const uint64_t launches0 = c->launches;
        uint64_t unused = 0;
        launch_pass(c, jgrid, s, d, c->gbuf, 0, C_JN1, c->rbuf[0], unused);
        launch_pass(c, jgrid, s, d, c->sbuf, 0, C_SPLIT_N, c->rbuf[0], unused);
        nk += (int)(c->launches - launches0);
        c->launches = launches0;
    }
    if (c->rt.nol) {
        launch_join(c, jgrid, s, d, c->vbuf, 0, C_JN2, c->rbuf[0]);
        nk++;
    }
    if (c->cand_cap) {
        k_apply<<<c->sms * GRG_APPLY_MINB, 256, 0, s>>>(d, c->cand[0], c->cand[1]);
        nk++;
    }
    if (c->timing) {
        k_tmark<<<1, 32, 0, s>>>(ctr, C_JT0, C_JNS, 1);
        nk++;
    }
    k_gate_end<<<1, 32, 0, s>>>(ctr, h);
    nk++;
    cudaGraph_t captured = body;
    const cudaError_t ce = cudaStreamEndCapture(s, &captured);
    if (ce != cudaSuccess) {
        free_round_graph(c);
        return fail(c, GRG_E_CUDA, std::string("round graph capture: ") + cudaGetErrorString(ce));
    }
    GRG_CUDA(c, cudaGraphInstantiate(&c->rg_exec, c->rg_graph, 0));
    c->rg_key = key;
    c->rg_kernels = nk;
    return GRG_OK;
}

// Rounds until the fixpoint (max_rounds = 0) or max_rounds rounds with work;
// *idle = the last gather found no delta.
static int run_rounds(grg_ctx *c, uint64_t max_rounds, grg_stats &S, double &join_ms, uint64_t &joins, bool *idle)
{
    cudaStream_t s = c->stream;
    int st = read_ctr(c);
    if (st) return st;
    *idle = false;
    uint64_t done_rounds = 0;
    bool graphs = c->device_rounds && max_rounds != 1 && c->V > 0;
    for (;;) {
        if (max_rounds && done_rounds >= max_rounds) break;
        // elements that gain bits in this run get its stamp; round 1 gathers the load marks
        const uint32_t rs = (c->elem_loaded && done_rounds > 0) ? c->run_stamp : 0u;
        choose_window(c);
        if (!graphs || done_rounds == 0) {
            uint64_t nd = 0, nv = 0;
            if ((st = round_head(c, rs, S, &nd))) return st;
            if (nd == 0) {
                *idle = true;
                break;
            }
            done_rounds++;
            if ((st = round_oldleft(c, &nv))) return st;
            if ((st = round_joins(c, nd, nv, S, join_ms, joins))) return st;
            continue;
        }
        // device-driven rounds: buffers sized with room to grow, then the graph loop. A round
        // has at most one record per used slot (and one virtual record per old-left rule and
        // element), so up to 16M records the buffers take what can never overflow and the
        // recorded graph survives the whole closure.
        const uint64_t nd_last = std::max<uint64_t>(c->h_ctr[C_DIRTY_N], 1);
        const uint64_t top = c->h_ctr[C_POOL_TOP], floor_cap = 1ull << 24;
        if ((st = ensure_gather(c, std::max(2 * nd_last, std::min(top, floor_cap))))) return st;
        if (c->rt.nol &&
            (st = ensure_buf(c, &c->vbuf, &c->vbuf_cap,
                             std::max<uint64_t>(2 * std::max<uint64_t>(c->h_ctr[C_VN], 1),
                                                std::min<uint64_t>((uint64_t)c->rt.nol * top, floor_cap)))))
            return st;
        if ((st = ensure_cand(c, 2 * nd_last))) return st;    // a full candidate buffer falls back to direct inserts
        if ((st = ensure_rbuf(c, retry_room(c, c->gbuf_cap + (c->rt.nol ? c->vbuf_cap : 0))))) return st;
        if ((st = ensure_sbuf(c))) return st;
        if ((st = build_round_graph(c, rs))) return st;
        c->cb = 0;
        // the delta index starts clear: inside the graph each round clears what the previous
        // round's records set, and those records may not have survived a buffer regrowth
        for (int l = 1; l <= c->L; l++)
            if (c->rt.dindex[l]) {
                const size_t t0 = (size_t)(l - 1) * c->V, vw = (c->V + 31) / 32;
                GRG_CUDA(c, cudaMemsetAsync(c->drs + t0, 0xFF, (size_t)c->V * 4, s));
                GRG_CUDA(c, cudaMemsetAsync(c->drc + t0, 0, (size_t)c->V * 4, s));
                GRG_CUDA(c, cudaMemsetAsync(c->dvm + (size_t)(l - 1) * vw, 0, vw * 4, s));
            }
        GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_DIRTY_N, 0, 8, s));
        GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_HALT, 0, 8 * 5, s));   // halt, iterations, rounds, deltas, join ns
        c->h_ctr[C_MAXR] = max_rounds ? max_rounds - done_rounds : 0;
        GRG_CUDA(c, cudaMemcpyAsync(c->ctr + C_MAXR, c->h_ctr + C_MAXR, 8, cudaMemcpyHostToDevice, s));
        GRG_CUDA(c, cudaGraphLaunch(c->rg_exec, s));
        if ((st = read_ctr(c))) return st;
        const unsigned long long halt = c->h_ctr[C_HALT], rounds = c->h_ctr[C_GROUNDS];
        S.rounds += rounds;
        S.delta_elems += c->h_ctr[C_GDSUM];
        joins += rounds * ((c->need_join ? 1 : 0) + (c->need_push ? 1 : 0) + (c->rt.nol ? 1 : 0));
        c->launches += c->h_ctr[C_ITERS] * c->rg_kernels;
        join_ms += c->h_ctr[C_JNS] * 1e-6;
        done_rounds += rounds;
        GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_HALT, 0, 8, s));
        c->h_ctr[C_HALT] = 0;
        if (halt == HALT_FIXPOINT) {
            *idle = true;
            break;
        }
        if (halt == HALT_ROUNDS) continue;      // the loop head ends the step
        if (halt == HALT_CAPACITY) {
            // this round's dirty bits are untouched: the host runs it from the start
            uint64_t nd = 0, nv = 0;
            if ((st = round_head(c, rs, S, &nd))) return st;
            if (nd == 0) {
                *idle = true;
                break;
            }
            done_rounds++;
            if ((st = round_oldleft(c, &nv))) return st;
            if ((st = round_joins(c, nd, nv, S, join_ms, joins))) return st;
        } else if (halt == HALT_OLDLEFT) {
            // gathered and indexed: the host redoes the virtual records with more room, then joins
            uint64_t nv = 0;
            if ((st = ensure_buf(c, &c->vbuf, &c->vbuf_cap, c->h_ctr[C_VN]))) return st;
            if ((st = round_oldleft(c, &nv))) return st;
            if ((st = round_joins(c, c->h_ctr[C_DIRTY_N], nv, S, join_ms, joins))) return st;
        } else if (halt == HALT_RETRY) {
            const uint64_t nd = c->h_ctr[C_DIRTY_N], nv = c->h_ctr[C_VN];
            if ((st = round_retries(c, c->h_ctr[C_RETRY_N], c->cand_cap ? c->h_ctr[C_AFAIL] : 0, S, join_ms, joins,
                                    nd, nv, nd + nv < SPLIT_MAX)))
                return st;
        } else if (halt == HALT_LIMIT) {
            // a launch that ran this long without a halt is not trusted: host-driven rounds from here
            c->device_rounds = false;
            graphs = false;
        } else {
            return fail(c, GRG_E_INTERNAL, "device-driven rounds stopped without a reason");
        }
    }
    return GRG_OK;
}

extern "C" {

int grg_closure(grg_ctx *c, uint32_t filter, grg_stats *stats) { return grg_closure_ex(c, filter, 0, stats); }

int grg_closure_ex(grg_ctx *c, uint32_t filter, uint32_t run_stamp, grg_stats *stats)
{
    if (!c || filter > 1) return GRG_E_ARG;
    if (!c->loaded) return fail(c, GRG_E_STATE, "grg_load_edges must come first");
    c->run_stamp = run_stamp;
    choose_window(c);
    if (c->closed) return fail(c, GRG_E_STATE, "closure already computed; reload the graph");
    cudaSetDevice(c->device);
    RuleTable rt;
    int st = build_rules(c, filter, rt);
    if (st) return st;
    c->rt = rt;
    set_passes(c);                         // which pass kernels run (the CSR copies do not change it)
    cudaStream_t s = c->stream;
    grg_stats S;
    memset(&S, 0, sizeof S);
    GRG_CUDA(c, cudaEventRecord(c->ev_a, s));
    if ((st = tune_begin(c, filter))) return st;
    choose_window(c);
    Dev d = make_dev(c);
    // labels never inserted into after the load are packed
    bool derivable[MAX_LABELS + 1] = {false};
    for (int q = 0; q < c->R; q++) {
        const int *r = &c->rules[3 * q];
        bool unary = r[1] && !r[2];
        if (!(filter && unary)) derivable[r[0]] = true;
    }
    for (int l = 1; l <= c->L; l++)
        if (!derivable[l]) {
            k_compact_static<<<grid_for(c, c->V, 256), 256, 0, s>>>(d, (uint32_t)l, 0, c->V);
            c->launches++;
        }
    // CSR copies of static labels that are a binary rule's second symbol (buffers kept per label)
    for (int l = 1; l <= c->L; l++) {
        bool rhs2 = false;
        for (int q = 0; q < c->R; q++)
            if (c->rules[3 * q + 1] && c->rules[3 * q + 2] == l) rhs2 = true;
        if (derivable[l] || !rhs2 || c->V == 0) continue;
        grg_ctx::CsrBuf &cb = c->csr[l];
        const uint64_t nb = (c->V + 1023) / 1024;
        if (cb.vcap < (uint64_t)c->V + 1) {
            cudaFree(cb.ptr); cudaFree(cb.row); cudaFree(cb.sums);
            cb.ptr = cb.sums = nullptr;
            cb.row = nullptr;
            cb.vcap = 0;
            const uint64_t vc = (uint64_t)c->V + 1 + c->V / 4;
            GRG_CUDA(c, cudaMalloc(&cb.ptr, vc * 4));
            GRG_CUDA(c, cudaMalloc(&cb.row, vc * 8));
            GRG_CUDA(c, cudaMalloc(&cb.sums, ((vc + 1023) / 1024 + 1) * 4));
            cb.vcap = vc;
        }
        uint32_t *ptr = cb.ptr, *sums = cb.sums;
        uint2 *row = cb.row;
        GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_ERR, 0, 8, s));
        k_csr_count<<<grid_for(c, c->V, 256), 256, 0, s>>>(d, (uint32_t)l, ptr, row);
        k_scan_blocks<<<(unsigned)nb, 1024, 0, s>>>(ptr, ptr, sums, c->V, nullptr);
        k_scan_sums<<<1, 1024, 0, s>>>(sums, nb, nullptr);
        k_scan_add<<<(unsigned)nb, 1024, 0, s>>>(ptr, sums, c->V, nullptr);
        st = read_ctr(c);
        if (st) return st;
        if (c->h_ctr[C_ERR]) continue;                 // a row too long for the packed CSR: keep elements
        uint32_t total = 0;
        GRG_CUDA(c, cudaMemcpyAsync(&total, sums + nb, 4, cudaMemcpyDeviceToHost, s));
        GRG_CUDA(c, cudaStreamSynchronize(s));
        if (cb.colcap < std::max<uint64_t>(total, 1)) {
            cudaFree(cb.col);
            cb.col = nullptr;
            cb.colcap = 0;
            const uint64_t cc = std::max<uint64_t>(total, 1) + total / 4;
            GRG_CUDA(c, cudaMalloc(&cb.col, cc * 4));
            cb.colcap = cc;
        }
        k_csr_fill<<<grid_for(c, c->V, 256), 256, 0, s>>>(d, (uint32_t)l, ptr, row, cb.col);
        c->launches += 6;
        rt.csr_row[l] = row;
        rt.csr_col[l] = cb.col;
        rt.csr_n[l] = total;
    }
    c->rt = rt;
    set_passes(c);
    st = read_ctr(c);
    if (st) return st;
    const uint64_t top = c->h_ctr[C_POOL_TOP];
    // every loaded element of a tracked label is a delta of round 1 (element images
    // carry their own marks instead)
    d = make_dev(c);
    if (top && !c->elem_loaded) {
        k_mark_all<<<grid_for(c, top, 256), 256, 0, s>>>(d, 0, top);
        c->launches++;
    }
    double join_ms = 0;
    uint64_t joins = 0;
    bool idle = false;
    st = run_rounds(c, 0, S, join_ms, joins, &idle);
    if (st) return st;
    if ((st = read_ctr(c))) return st;
    if (c->h_ctr[C_CHECK])
        return fail(c, GRG_E_INTERNAL, "bounds check " + std::to_string(c->h_ctr[C_CHECK] >> 56) + " failed (value " +
                                           std::to_string(c->h_ctr[C_CHECK] & ((1ull << 56) - 1)) + ")");
    GRG_CUDA(c, cudaEventRecord(c->ev_b, s));
    GRG_CUDA(c, cudaEventSynchronize(c->ev_b));
    float ms = 0;
    cudaEventElapsedTime(&ms, c->ev_a, c->ev_b);
    S.closure_ms = ms;
    S.join_ms = join_ms;
    S.join_launches = joins;
    S.left_elems = c->h_ctr[C_LEFT];
    S.window_out_elems = c->h_ctr[C_WOUT];
    S.window_noslot_items = c->h_ctr[C_NOSLOT];
    S.candidates = c->h_ctr[C_CANDS];
    S.join_inserts = c->h_ctr[C_INSERTS];
    S.direct_inserts = c->cand_cap == 0;
    S.gather_ms = c->h_ctr[C_GNS] * 1e-6;
    S.wide_window = c->join_wide ? 1 : 0;
    S.window_tuned = (uint64_t)c->tune_source;
    S.window_trial_ms[0] = c->tune_ms[0];
    S.window_trial_ms[1] = c->tune_ms[1];
    S.column_labels = c->tmask;
    S.join_elements = c->need_join && c->join_elems && any_csr(c) ? 1 : 0;
    S.items_trial_ms[0] = c->items_ms[0];
    S.items_trial_ms[1] = c->items_ms[1];
    S.push_flat = c->need_push && c->push_flat ? 1 : 0;
    S.push_tuned = (uint64_t)c->push_source;
    S.push_trial_ms[0] = c->push_ms[0];
    S.push_trial_ms[1] = c->push_ms[1];
    c->tune_pending = c->push_pending = false;   // an untimed closure leaves its key for the next one
    S.right_elems = c->h_ctr[C_RIGHT];
    S.out_elems = S.delta_elems;
    S.pool_elems_used = c->h_ctr[C_POOL_TOP];
    S.pool_elems_cap = c->pool_cap;
    for (int i = 0; i < 5; i++) S.join_phase_cycles[i] = c->h_ctr[C_PH0 + i];
    c->closed = true;
    // total edge count
    uint64_t counts[MAX_LABELS];
    st = grg_label_counts(c, counts);
    if (st) return st;
    for (int l = 0; l < c->L; l++) S.total_edges += counts[l];
    S.kernel_launches = c->launches;
    if (stats) *stats = S;
    return GRG_OK;
}

static int count_pass(grg_ctx *c, uint32_t *deg_e, uint32_t *deg_el, uint32_t first, uint32_t last, int do_hash)
{
    cudaStream_t s = c->stream;
    Dev d = make_dev(c);
    GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_LABEL0, 0, sizeof(unsigned long long) * (MAX_SLOTS + 2), s));
    GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_HASH, 0, 8, s));
    for (int l = 1; l <= c->L; l++)
        k_count<<<grid_for(c, (uint64_t)c->V * 32, 256), 256, 0, s>>>(d, (uint32_t)l, deg_e, deg_el, first, last, do_hash,
                                                                       0, c->V, 0, 0, (int)((c->tmask >> (l - 1)) & 1));
    GRG_CUDA(c, cudaGetLastError());
    return read_ctr(c);
}

int grg_label_counts(grg_ctx *c, uint64_t *counts)
{
    if (!c || !counts) return GRG_E_ARG;
    if (!c->loaded) return fail(c, GRG_E_STATE, "no graph loaded");
    cudaSetDevice(c->device);
    int st = count_pass(c, nullptr, nullptr, 0, 0, 0);
    if (st) return st;
    for (int l = 1; l <= c->L; l++) counts[l - 1] = c->h_ctr[C_LABEL0 + l];
    return GRG_OK;
}

int grg_set_hash(grg_ctx *c, uint64_t *hash)
{
    if (!c || !hash) return GRG_E_ARG;
    if (!c->loaded) return fail(c, GRG_E_STATE, "no graph loaded");
    cudaSetDevice(c->device);
    int st = count_pass(c, nullptr, nullptr, 0, 0, 1);
    if (st) return st;
    *hash = c->h_ctr[C_HASH];
    return GRG_OK;
}

static int stage_elements(grg_ctx *c, uint32_t v_begin, uint32_t v_end, uint64_t *n_out);

// Labels stored by destination are turned back into rows by source; every entry
// point that reads rows by source (degrees, element images, ranges, streams)
// calls this first. The graph's element records are staged, the
// destination-stored ones transposed on the device, 192 x 192 tiles at a time,
// and everything is reloaded as an element image with no deltas marked. A closed
// graph stays closed. Not available on a batch context.
static int rows_by_source(grg_ctx *c)
{
    if (!c->tmask || !c->loaded) return GRG_OK;
    if (c->batch) return fail(c, GRG_E_STATE, "rows by source are not available on a batch context");
    const bool closed = c->closed;
    uint64_t n = 0;
    int st = stage_elements(c, 0, c->V, &n);
    if (st) return st;
    uint4 *rows = nullptr;
    uint32_t *stamps = nullptr;
    uint64_t m = 0;
    cudaError_t e = grg_fmt_columns_to_rows(c->xbuf, n, c->tmask, &rows, &m, c->stream);
    if (e == cudaSuccess) e = cudaMalloc(&stamps, std::max<uint64_t>(m, 1) * 4);
    if (e == cudaSuccess) e = cudaMemsetAsync(stamps, 0, std::max<uint64_t>(m, 1) * 4, c->stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        cudaFree(rows);
        cudaFree(stamps);
        return fail(c, e == cudaErrorMemoryAllocation ? GRG_E_NOMEM : GRG_E_CUDA,
                    std::string("turning columns into rows: ") + cudaGetErrorString(e));
    }
    st = grg_load_elements(c, c->V, m, reinterpret_cast<const uint32_t *>(rows), stamps, ~0u, 1);
    cudaFree(rows);
    cudaFree(stamps);
    if (st) return st;
    c->closed = closed;
    return GRG_OK;
}

int grg_get_degree(grg_ctx *c, uint32_t first_var, uint32_t last_var, uint32_t *degree)
{
    if (!c || !degree || last_var < first_var) return GRG_E_ARG;
    if (!c->loaded) return fail(c, GRG_E_STATE, "no graph loaded");
    if (last_var >= c->V) return fail(c, GRG_E_RANGE, "vertex range beyond numVars");
    cudaSetDevice(c->device);
    if (int rs = rows_by_source(c)) return rs;
    const uint64_t n = (uint64_t)last_var - first_var + 1;
    uint32_t *dd = nullptr;
    GRG_CUDA(c, cudaMalloc(&dd, n * 8));
    GRG_CUDA(c, cudaMemsetAsync(dd, 0, n * 8, c->stream));
    int st = count_pass(c, dd, dd + n, first_var, last_var, 0);
    if (st) { cudaFree(dd); return st; }
    memset(degree, 0, sizeof(uint32_t) * n * 6);
    cudaError_t e1 = cudaMemcpy(degree, dd, n * 4, cudaMemcpyDeviceToHost);
    cudaError_t e2 = cudaMemcpy(degree + 3 * n, dd + n, n * 4, cudaMemcpyDeviceToHost);
    cudaFree(dd);
    if (e1 != cudaSuccess || e2 != cudaSuccess) return fail(c, GRG_E_CUDA, "degree copy failed");
    return GRG_OK;
}

int grg_export_edges(grg_ctx *c, uint64_t cap, uint32_t *src, uint32_t *dst, uint8_t *label, uint64_t *num_out)
{
    if (!c || !num_out || (cap && (!src || !dst || !label))) return GRG_E_ARG;
    if (!c->loaded) return fail(c, GRG_E_STATE, "no graph loaded");
    cudaSetDevice(c->device);
    cudaStream_t s = c->stream;
    uint32_t *d32 = nullptr;
    uint8_t *d8 = nullptr;
    if (cap) {
        GRG_CUDA(c, cudaMalloc(&d32, cap * 8));
        GRG_CUDA(c, cudaMalloc(&d8, cap));
    }
    GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_EXPORT, 0, 8, s));
    Dev d = make_dev(c);
    for (int l = 1; l <= c->L; l++)
        k_export<<<grid_for(c, c->V, 256), 256, 0, s>>>(d, (uint32_t)l, d32, d32 ? d32 + cap : nullptr, d8, cap,
                                                         (int)((c->tmask >> (l - 1)) & 1));
    int st = read_ctr(c);
    if (st) { cudaFree(d32); cudaFree(d8); return st; }
    *num_out = c->h_ctr[C_EXPORT];
    if (cap) {
        uint64_t m = std::min<uint64_t>(cap, *num_out);
        cudaMemcpy(src, d32, m * 4, cudaMemcpyDeviceToHost);
        cudaMemcpy(dst, d32 + cap, m * 4, cudaMemcpyDeviceToHost);
        cudaMemcpy(label, d8, m, cudaMemcpyDeviceToHost);
        cudaFree(d32);
        cudaFree(d8);
    }
    GRG_CUDA(c, cudaGetLastError());
    return GRG_OK;
}

int grg_export_elements(grg_ctx *c, uint32_t v_begin, uint32_t v_end, uint64_t cap, uint32_t *elems,
                        uint32_t *stamps, uint64_t *num_out)
{
    if (!c || v_begin > v_end || (cap && (!elems || !stamps))) return GRG_E_ARG;
    if (!c->loaded) return fail(c, GRG_E_STATE, "no graph loaded");
    if (v_end > c->V) return fail(c, GRG_E_RANGE, "vertex range beyond the graph");
    cudaSetDevice(c->device);
    if (int rs = rows_by_source(c)) return rs;
    cudaStream_t s = c->stream;
    Dev d = make_dev(c);
    const uint64_t ntab = (uint64_t)c->L * (v_end - v_begin);
    // count first: nothing is staged when the caller's buffer is too small
    GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_EXPORT, 0, 8, s));
    if (ntab) k_export_elems<<<grid_for(c, ntab * 32, 256), 256, 0, s>>>(d, v_begin, v_end, (uint32_t)c->L, nullptr, nullptr, 0);
    int st = read_ctr(c);
    if (st) return st;
    uint64_t n = c->h_ctr[C_EXPORT];
    if (num_out) *num_out = n;
    if (n > cap) return fail(c, GRG_E_RANGE, "export buffer too small");
    if (!n) return GRG_OK;
    if ((st = stage_elements(c, v_begin, v_end, &n))) return st;
    GRG_CUDA(c, cudaMemcpyAsync(elems, c->xbuf, n * 32, cudaMemcpyDeviceToHost, s));
    GRG_CUDA(c, cudaMemcpyAsync(stamps, c->xst, n * 4, cudaMemcpyDeviceToHost, s));
    GRG_CUDA(c, cudaStreamSynchronize(s));
    GRG_CUDA(c, cudaGetLastError());
    return GRG_OK;
}

// Records of rows [v_begin, v_end) into the staging buffer xbuf (8 words each,
// any order; stamps into xst). *n = their number.
static int stage_elements(grg_ctx *c, uint32_t v_begin, uint32_t v_end, uint64_t *n_out)
{
    cudaStream_t s = c->stream;
    Dev d = make_dev(c);
    const uint64_t ntab = (uint64_t)c->L * (v_end - v_begin);
    GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_EXPORT, 0, 8, s));
    if (ntab) k_export_elems<<<grid_for(c, ntab * 32, 256), 256, 0, s>>>(d, v_begin, v_end, (uint32_t)c->L, nullptr, nullptr, 0);
    int st = read_ctr(c);
    if (st) return st;
    const uint64_t n = c->h_ctr[C_EXPORT];
    *n_out = n;
    if (!n) return GRG_OK;
    if (c->xcap < n) {
        cudaFree(c->xbuf); cudaFree(c->xst);
        c->xbuf = nullptr; c->xst = nullptr;
        c->xcap = 0;
        const uint64_t xc = n + n / 4;
        GRG_CUDA(c, cudaMalloc(&c->xbuf, xc * 32));
        GRG_CUDA(c, cudaMalloc(&c->xst, xc * 4));
        c->xcap = xc;
    }
    GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_EXPORT, 0, 8, s));
    k_export_elems<<<grid_for(c, ntab * 32, 256), 256, 0, s>>>(d, v_begin, v_end, (uint32_t)c->L, c->xbuf, c->xst, n);
    GRG_CUDA(c, cudaGetLastError());
    return GRG_OK;
}


// Elements of rows [a, b) (a count-only pass of the element export).
static int count_elements(grg_ctx *c, uint32_t a, uint32_t b, uint64_t *n)
{
    cudaStream_t s = c->stream;
    const uint64_t ntab = (uint64_t)c->L * (b - a);
    GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_EXPORT, 0, 8, s));
    if (ntab) k_export_elems<<<grid_for(c, ntab * 32, 256), 256, 0, s>>>(make_dev(c), a, b, (uint32_t)c->L, nullptr,
                                                                          nullptr, 0);
    int st = read_ctr(c);
    if (st) return st;
    *n = c->h_ctr[C_EXPORT];
    return GRG_OK;
}

// One piece of a stream export: rows [v_begin, v_end), `total` edges, into host
// buffers edges / degree.
static int export_csr5_piece(grg_ctx *c, uint32_t v_begin, uint32_t v_end, uint64_t total, uint8_t *edges,
                             uint32_t *degree)
{
    const uint32_t nrows = v_end - v_begin;
    if (!nrows) return GRG_OK;
    uint64_t n = 0;
    int st = stage_elements(c, v_begin, v_end, &n);
    if (st) return st;
    uint8_t *dbytes = nullptr;
    uint32_t *ddeg = nullptr;
    cudaError_t e = cudaMalloc(&ddeg, (size_t)nrows * 4);
    if (e == cudaSuccess && total) e = cudaMalloc(&dbytes, total * 5);
    if (e == cudaSuccess) e = grg_fmt_records_to_csr5(c->xbuf, n, v_begin, nrows, total, dbytes, ddeg, c->stream);
    if (e == cudaSuccess && total) e = cudaMemcpy(edges, dbytes, total * 5, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(degree, ddeg, (size_t)nrows * 4, cudaMemcpyDeviceToHost);
    cudaFree(dbytes);
    cudaFree(ddeg);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(c, e == cudaErrorMemoryAllocation ? GRG_E_NOMEM : GRG_E_CUDA,
                    std::string("compressed export: ") + cudaGetErrorString(e));
    }
    return GRG_OK;
}

// Device bytes one piece needs: its stream (5 B per edge) and, per element, the
// staged record and stamp (36 B), sort keys and indices in and out (24 B), the
// counts and offsets (16 B) and the sort's own room (~12 B).
static uint64_t csr5_footprint(uint64_t edges, uint64_t elems) { return 5 * edges + 88 * elems; }

// Rows [a, b) with `total` edges: halved by rows until a piece fits `budget`
// bytes of device memory; pieces go out in row order, so their streams and row
// lengths concatenate into the range's.
static int export_csr5_split(grg_ctx *c, uint32_t a, uint32_t b, uint64_t total, uint64_t budget, uint8_t *edges,
                             uint32_t *degree)
{
    uint64_t n = 0;
    int st = count_elements(c, a, b, &n);
    if (st) return st;
    if (csr5_footprint(total, n) <= budget || b - a <= 1) return export_csr5_piece(c, a, b, total, edges, degree);
    const uint32_t mid = a + (b - a) / 2;
    std::vector<uint64_t> counts(c->L + 1, 0);
    uint64_t h = 0, t1 = 0;
    if ((st = grg_range_counts(c, a, mid, counts.data(), &h))) return st;
    for (int l = 0; l < c->L; l++) t1 += counts[l];
    if ((st = export_csr5_split(c, a, mid, t1, budget, edges, degree))) return st;
    return export_csr5_split(c, mid, b, total - t1, budget, edges + t1 * 5, degree + (mid - a));
}

int grg_export_csr5(grg_ctx *c, uint32_t v_begin, uint32_t v_end, uint64_t cap, uint8_t *edges, uint32_t *degree,
                    uint64_t *num_edges)
{
    if (!c || v_begin > v_end || !num_edges || (cap && (!edges || !degree))) return GRG_E_ARG;
    if (!c->loaded) return fail(c, GRG_E_STATE, "no graph loaded");
    if (v_end > c->V) return fail(c, GRG_E_RANGE, "vertex range beyond the graph");
    cudaSetDevice(c->device);
    if (int rs = rows_by_source(c)) return rs;
    // the stream's length is the range's popcount
    std::vector<uint64_t> counts(c->L + 1, 0);
    uint64_t h = 0, total = 0;
    int st = grg_range_counts(c, v_begin, v_end, counts.data(), &h);
    if (st) return st;
    for (int l = 0; l < c->L; l++) total += counts[l];
    *num_edges = total;
    if (total > cap) return total ? fail(c, GRG_E_RANGE, "stream buffer too small") : GRG_OK;
    if (v_end == v_begin) return GRG_OK;
    // pieces take at most half of the free device memory (at least 256 MiB)
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    uint64_t budget = std::max<uint64_t>(fr / 2, 256ull << 20);
    const char *eb = getenv("GRG_CSR5_BUDGET");         // bytes; smaller budgets split (tests)
    if (eb && atoll(eb) > 0) budget = (uint64_t)atoll(eb);
    return export_csr5_split(c, v_begin, v_end, total, budget, edges, degree);
}

int grg_load_csr5(grg_ctx *c, uint32_t num_vars, uint32_t v_begin, uint32_t v_end, const uint32_t *degree,
                  uint64_t num_edges, const uint8_t *edges, int on_device)
{
    if (!c || v_begin > v_end || (v_end > v_begin && !degree) || (num_edges && !edges)) return GRG_E_ARG;
    if (!c->have_rules) return fail(c, GRG_E_STATE, "grg_transfer_rules must come first");
    if (v_end > num_vars) return fail(c, GRG_E_RANGE, "vertex range beyond numVars");
    cudaSetDevice(c->device);
    const uint32_t nrows = v_end - v_begin;
    if (num_edges && !nrows) return fail(c, GRG_E_ARG, "edges without rows");
    cudaError_t e = cudaSuccess;
    uint64_t sum = 0, n = 0;
    unsigned bad = 0;
    uint4 *recs = nullptr;
    uint32_t *stamps = nullptr;
    if (on_device) {
        e = grg_fmt_csr5_to_records(edges, num_edges, degree, v_begin, nrows, num_vars, (uint32_t)c->L, nullptr,
                                    nullptr, 0, &recs, &stamps, &n, &sum, &bad, c->stream);
    } else {
        // host stream: its lengths are checked here, then it goes to the device in row
        // pieces. A piece's stream bytes (5 per edge) and its records (at most one
        // 32-byte record and a 4-byte stamp per edge) fit a quarter of the free device
        // memory. With more than one piece, a first pass counts each piece's records,
        // the joined record buffer is allocated once, and a second pass builds every
        // piece's records at its own offset, so no second copy is ever held.
        for (uint32_t r = 0; r < nrows; r++) sum += degree[r];
        if (sum != num_edges) return fail(c, GRG_E_ARG, "row lengths do not add up to num_edges");
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        uint64_t budget = std::max<uint64_t>(fr / 4, 64ull << 20);
        const char *eb = getenv("GRG_CSR5_BUDGET");     // bytes; smaller budgets split (tests)
        if (eb && atoll(eb) > 0) budget = (uint64_t)atoll(eb);
        constexpr uint64_t PIECE_BYTES_PER_EDGE = 5 + 32 + 4;
        struct Piece { uint32_t r0, r1; uint64_t e0, ne, n; };
        std::vector<Piece> pieces;
        uint64_t max_ne = 0;
        uint64_t e0 = 0;
        for (uint32_t r0 = 0; r0 < nrows;) {
            uint32_t r1 = r0;
            uint64_t pe = 0;
            while (r1 < nrows && (r1 == r0 || (pe + degree[r1]) * PIECE_BYTES_PER_EDGE <= budget)) pe += degree[r1++];
            pieces.push_back({r0, r1, e0, pe, 0});
            max_ne = std::max(max_ne, pe);
            e0 += pe;
            r0 = r1;
        }
        uint8_t *sbytes = nullptr;
        uint32_t *sdeg = nullptr;
        uint32_t max_rows = 0;
        for (const Piece &q : pieces) max_rows = std::max(max_rows, q.r1 - q.r0);
        if (max_ne) e = cudaMalloc(&sbytes, max_ne * 5);
        if (e == cudaSuccess) e = cudaMalloc(&sdeg, (size_t)std::max<uint32_t>(max_rows, 1) * 4);
        auto upload = [&](const Piece &q) {
            cudaError_t r = cudaSuccess;
            if (q.ne) r = cudaMemcpyAsync(sbytes, edges + q.e0 * 5, q.ne * 5, cudaMemcpyHostToDevice, c->stream);
            if (r == cudaSuccess)
                r = cudaMemcpyAsync(sdeg, degree + q.r0, (size_t)(q.r1 - q.r0) * 4, cudaMemcpyHostToDevice, c->stream);
            return r;
        };
        uint64_t psum = 0;
        if (pieces.size() == 1) {
            if (e == cudaSuccess) e = upload(pieces[0]);
            if (e == cudaSuccess)
                e = grg_fmt_csr5_to_records(sbytes, pieces[0].ne, sdeg, v_begin, nrows, num_vars, (uint32_t)c->L,
                                            nullptr, nullptr, 0, &recs, &stamps, &n, &psum, &bad, c->stream);
        } else {
            for (Piece &q : pieces) {                 // pass 1: records per piece
                if (e != cudaSuccess || bad) break;
                e = upload(q);
                if (e == cudaSuccess)
                    e = grg_fmt_csr5_to_records(sbytes, q.ne, sdeg, v_begin + q.r0, q.r1 - q.r0, num_vars,
                                                (uint32_t)c->L, nullptr, nullptr, 0, nullptr, nullptr, &q.n, &psum,
                                                &bad, c->stream);
                n += q.n;
            }
            if (e == cudaSuccess && !bad && n) {
                e = cudaMalloc(&recs, n * 32);
                if (e == cudaSuccess) e = cudaMalloc(&stamps, n * 4);
            }
            uint64_t o = 0;
            for (const Piece &q : pieces) {           // pass 2: each piece at its offset
                if (e != cudaSuccess || bad || !n) break;
                uint64_t qn = 0;
                e = upload(q);
                if (e == cudaSuccess && q.n)
                    e = grg_fmt_csr5_to_records(sbytes, q.ne, sdeg, v_begin + q.r0, q.r1 - q.r0, num_vars,
                                                (uint32_t)c->L, recs + 2 * o, stamps + o, q.n, nullptr, nullptr,
                                                &qn, &psum, &bad, c->stream);
                o += q.n;
            }
        }
        cudaFree(sbytes);
        cudaFree(sdeg);
    }
    int st = GRG_OK;
    if (e != cudaSuccess) {
        cudaGetLastError();
        st = fail(c, e == cudaErrorMemoryAllocation ? GRG_E_NOMEM : GRG_E_CUDA,
                  std::string("compressed load: ") + cudaGetErrorString(e));
    } else if (sum != num_edges) {
        st = fail(c, GRG_E_ARG, "row lengths do not add up to num_edges");
    } else if (bad & 1u) {
        st = fail(c, GRG_E_LABEL, "edge label outside 1..numLabels");
    } else if (bad & 2u) {
        st = fail(c, GRG_E_RANGE, "edge vertex id >= numVars");
    }
    if (st) {
        cudaFree(recs);
        cudaFree(stamps);
        return st;
    }
    // a stream is a spilled image: it already holds its epsilon edges, and every
    // element is a delta of round 1 of the next closure
    st = grg_load_elements(c, num_vars, n, reinterpret_cast<const uint32_t *>(recs), stamps, 0, 1);
    cudaFree(recs);
    cudaFree(stamps);
    return st;
}

int grg_range_counts(grg_ctx *c, uint32_t v_begin, uint32_t v_end, uint64_t *counts, uint64_t *hash)
{
    if (!c || !counts || v_begin > v_end) return GRG_E_ARG;
    if (!c->loaded) return fail(c, GRG_E_STATE, "no graph loaded");
    if (v_end > c->V) return fail(c, GRG_E_RANGE, "vertex range beyond the graph");
    cudaSetDevice(c->device);
    if (int rs = rows_by_source(c)) return rs;
    cudaStream_t s = c->stream;
    Dev d = make_dev(c);
    GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_LABEL0, 0, sizeof(unsigned long long) * (MAX_SLOTS + 2), s));
    GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_HASH, 0, 8, s));
    if (v_end > v_begin)
        for (int l = 1; l <= c->L; l++)
            k_count<<<grid_for(c, (uint64_t)(v_end - v_begin) * 32, 256), 256, 0, s>>>(
                d, (uint32_t)l, nullptr, nullptr, 0, 0, hash ? 1 : 0, v_begin, v_end, 0, 0, 0);
    GRG_CUDA(c, cudaGetLastError());
    int st = read_ctr(c);
    if (st) return st;
    for (int l = 1; l <= c->L; l++) counts[l - 1] = c->h_ctr[C_LABEL0 + l];
    if (hash) *hash = c->h_ctr[C_HASH];
    return GRG_OK;
}

int grg_range_reach(grg_ctx *c, uint32_t v_begin, uint32_t v_end, uint64_t label_mask, uint32_t num_parts,
                    const uint32_t *bounds, uint8_t *reach)
{
    if (!c || v_begin > v_end || num_parts == 0 || !bounds || !reach) return GRG_E_ARG;
    if (!c->loaded) return fail(c, GRG_E_STATE, "no graph loaded");
    if (v_end > c->V) return fail(c, GRG_E_RANGE, "vertex range beyond the graph");
    for (uint32_t p = 0; p < num_parts; p++)
        if (bounds[p] > bounds[p + 1]) return fail(c, GRG_E_ARG, "partition bounds must not decrease");
    cudaSetDevice(c->device);
    if (int rs = rows_by_source(c)) return rs;
    cudaStream_t s = c->stream;
    uint32_t *db = nullptr;                      // bounds, then one flag per partition
    GRG_CUDA(c, cudaMallocAsync((void **)&db, (2 * (size_t)num_parts + 1) * 4, s));
    GRG_CUDA(c, cudaMemcpyAsync(db, bounds, ((size_t)num_parts + 1) * 4, cudaMemcpyHostToDevice, s));
    GRG_CUDA(c, cudaMemsetAsync(db + num_parts + 1, 0, (size_t)num_parts * 4, s));
    const uint64_t ntab = (uint64_t)c->L * (v_end - v_begin);
    if (ntab)
        k_range_reach<<<grid_for(c, ntab * 32, 256), 256, 0, s>>>(make_dev(c), v_begin, v_end, (uint32_t)c->L,
                                                                  label_mask, db, num_parts, db + num_parts + 1);
    std::vector<uint32_t> f(num_parts);
    GRG_CUDA(c, cudaMemcpyAsync(f.data(), db + num_parts + 1, (size_t)num_parts * 4, cudaMemcpyDeviceToHost, s));
    GRG_CUDA(c, cudaFreeAsync(db, s));
    GRG_CUDA(c, cudaStreamSynchronize(s));
    GRG_CUDA(c, cudaGetLastError());
    for (uint32_t p = 0; p < num_parts; p++) reach[p] = f[p] ? 1 : 0;
    return GRG_OK;
}

int grg_set_pool_limit(grg_ctx *c, uint64_t pool_bytes)
{
    if (!c) return GRG_E_ARG;
    cudaSetDevice(c->device);
    c->pool_limit = pool_bytes ? std::max<uint64_t>(pool_bytes / (POOL_BYTES_PER_SLOT + 4), 1024) : 0;
    if (c->pool_limit && c->elems && c->pool_cap > c->pool_limit) {
        // the pool shrinks on the next load; the loaded graph is dropped
        free_pool(c);
        c->loaded = false;
        c->closed = false;
    }
    return GRG_OK;
}

}  // extern "C"

// ====================================================================== batched jobs

extern "C" {

int grg_batch_begin(grg_ctx *c, uint32_t max_vars, uint32_t max_jobs, int num_rules, const int *rules,
                    int num_labels, uint32_t filter)
{
    if (!c || filter > 1 || max_jobs == 0 || max_vars == 0) return GRG_E_ARG;
    int st = grg_transfer_rules(c, num_rules, rules, num_labels);
    if (st) return st;
    cudaSetDevice(c->device);
    c->elem_loaded = false;
    c->tmask = c->layout_mode ? plan_columns(c->rules, c->R, c->L) : 0;
    RuleTable rt;
    st = build_rules(c, filter, rt);
    if (st) return st;
    if (!c->elems) {
        st = grg_allocate_pool(c, c->pool_bytes_req);
        if (st) return st;
    }
    if ((uint64_t)max_vars * (uint64_t)c->L >= 0xFFFFFFFFull)
        return fail(c, GRG_E_RANGE, "max_vars x 2 x numLabels must stay below 2^32");
    free_graph(c);
    cudaStream_t s = c->stream;
    c->V = max_vars;
    c->ntables = (uint64_t)c->L * max_vars;
    const uint64_t nt_all = (uint64_t)c->L * max_vars;
    GRG_CUDA(c, cudaMalloc(&c->desc, nt_all * 8));
    GRG_CUDA(c, cudaMalloc(&c->cnt, nt_all * 4));
    GRG_CUDA(c, cudaMalloc(&c->want, nt_all * 4));
    GRG_CUDA(c, cudaMalloc(&c->grow, nt_all * 4));
    c->ntables_alloc = nt_all;
    st = alloc_dindex(c);
    if (st) return st;
    GRG_CUDA(c, cudaMalloc(&c->row_job, (uint64_t)max_vars * 4));
    GRG_CUDA(c, cudaMalloc(&c->job_cnt, (uint64_t)max_jobs * 4));
    c->max_jobs = max_jobs;
    c->jobs.assign(max_jobs, grg_ctx::JobRange());
    GRG_CUDA(c, cudaMemsetAsync(c->desc, 0, nt_all * 8, s));
    GRG_CUDA(c, cudaMemsetAsync(c->cnt, 0, nt_all * 4, s));
    GRG_CUDA(c, cudaMemsetAsync(c->want, 0, nt_all * 4, s));
    GRG_CUDA(c, cudaMemsetAsync(c->row_job, 0xFF, (uint64_t)max_vars * 4, s));
    GRG_CUDA(c, cudaMemsetAsync(c->job_cnt, 0, (uint64_t)max_jobs * 4, s));
    GRG_CUDA(c, cudaMemsetAsync(c->ctr, 0, sizeof(unsigned long long) * NCTR, s));
    GRG_CUDA(c, cudaMemsetAsync(c->dmap, 0, (c->pool_cap / 32 + 2) * 4, s));
    c->rt = rt;   // batch mode keeps every label in hash tables (no CSR copies)
    set_passes(c);
    c->batch = true;
    c->filter = filter;
    c->loaded = true;
    c->closed = false;
    return read_ctr(c);
}

int grg_batch_admit(grg_ctx *c, uint32_t job, uint32_t base, uint32_t num_vars, uint64_t num_edges,
                    const uint32_t *src, const uint32_t *dst, const uint8_t *label, int on_device, uint64_t eps_mask)
{
    if (!c || (num_edges && (!src || !dst || !label))) return GRG_E_ARG;
    if (!c->batch) return fail(c, GRG_E_STATE, "grg_batch_begin must come first");
    if (job >= c->max_jobs || c->jobs[job].active) return fail(c, GRG_E_ARG, "job slot in use or out of range");
    if (num_vars == 0 || (uint64_t)base + num_vars > c->V) return fail(c, GRG_E_RANGE, "vertex range outside max_vars");
    for (const auto &j : c->jobs)
        if (j.active && base < j.base + j.nv && j.base < base + num_vars)
            return fail(c, GRG_E_ARG, "vertex range overlaps an admitted job");
    cudaSetDevice(c->device);
    cudaStream_t s = c->stream;
    const uint32_t *dsrc = src, *ddst = dst;
    const uint8_t *dlab = label;
    if (!on_device && num_edges) {
        const int se = ensure_input(c, num_edges);
        if (se) return se;
        GRG_CUDA(c, cudaMemcpyAsync(c->d_in32, src, num_edges * 4, cudaMemcpyHostToDevice, s));
        GRG_CUDA(c, cudaMemcpyAsync(c->d_in32 + num_edges, dst, num_edges * 4, cudaMemcpyHostToDevice, s));
        GRG_CUDA(c, cudaMemcpyAsync(c->d_in8, label, num_edges, cudaMemcpyHostToDevice, s));
        dsrc = c->d_in32;
        ddst = c->d_in32 + num_edges;
        dlab = c->d_in8;
    }
    // room for the job's tables: edges x 4/3 plus presized derived rows -- only of the
    // labels the job's own edges can derive (host inputs), else of every derived label
    MinCap mc;
    memset(&mc, 0, sizeof mc);
    bool lhs[MAX_LABELS + 1] = {false};
    int nder = 0;
    if (!on_device) {
        bool have[MAX_LABELS + 1] = {false};
        for (uint64_t e = 0; e < num_edges; e++)
            if (label[e] >= 1 && label[e] <= c->L) have[label[e]] = true;
        for (int l = 1; l <= c->L; l++)
            if ((eps_mask >> (l - 1)) & 1ull) have[l] = true;
        for (bool grew = true; grew;) {
            grew = false;
            for (int q = 0; q < c->R; q++) {
                const int *r = &c->rules[3 * q];
                if (r[1] && have[r[1]] && (!r[2] || have[r[2]]) && !have[r[0]]) have[r[0]] = grew = true;
            }
        }
        for (int q = 0; q < c->R; q++)
            if (have[c->rules[3 * q]]) lhs[c->rules[3 * q]] = true;
    } else {
        for (int q = 0; q < c->R; q++) lhs[c->rules[3 * q]] = true;
    }
    for (int l = 1; l <= c->L; l++) nder += lhs[l];
    int st = read_ctr(c);
    if (st) return st;
    const uint64_t top0 = (c->h_ctr[C_POOL_TOP] + 31) & ~31ull;   // the job's slots start on a dirty-bitmap word
    const uint64_t est = 2 * num_edges + (uint64_t)num_vars * (64 + 4 * __builtin_popcountll(eps_mask)) +
                         (uint64_t)nder * num_vars * DERIVED_MIN_CAP;
    if (top0 + est > c->pool_cap) {
        st = grow_pool(c, top0 + est + c->pool_cap / 2);
        if (st) return st;
    }
    if ((uint64_t)nder * num_vars * DERIVED_MIN_CAP <= (c->pool_cap - top0) / 4)
        for (int l = 1; l <= c->L; l++) mc.cap[l] = lhs[l] ? DERIVED_MIN_CAP : 0;
    c->h_ctr[C_POOL_TOP] = top0;
    GRG_CUDA(c, cudaMemcpyAsync(c->ctr + C_POOL_TOP, c->h_ctr + C_POOL_TOP, 8, cudaMemcpyHostToDevice, s));
    GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_ERR, 0, 8, s));
    GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_BADIN, 0, 8, s));
    Dev d = make_dev(c);
    if (num_edges)
        k_load_hist<<<grid_for(c, num_edges, 256), 256, 0, s>>>(d, dsrc, ddst, dlab, num_edges, base, num_vars, (uint32_t)c->L,
                                                                c->tmask);
    for (int l = 1; l <= c->L; l++)
        if ((eps_mask >> (l - 1)) & 1ull) k_eps_hist<<<grid_for(c, num_vars, 256), 256, 0, s>>>(d, (uint32_t)l, base, num_vars);
    k_load_alloc<<<grid_for(c, (uint64_t)c->L * num_vars, 256), 256, 0, s>>>(d, base, num_vars, (uint32_t)c->L, mc,
                                                                              nullptr);
    st = read_ctr(c);
    if (st) return st;
    if (c->h_ctr[C_BADIN]) {
        // refused input: the job's tables are given back (rows cleared as a release clears them)
        for (int slot = 1; slot <= c->L; slot++) {
            const size_t t0 = (size_t)(slot - 1) * c->V + base;
            GRG_CUDA(c, cudaMemsetAsync(c->desc + t0, 0, (size_t)num_vars * 8, s));
            GRG_CUDA(c, cudaMemsetAsync(c->cnt + t0, 0, (size_t)num_vars * 4, s));
        }
        c->h_ctr[C_POOL_TOP] = top0;
        GRG_CUDA(c, cudaMemcpyAsync(c->ctr + C_POOL_TOP, c->h_ctr + C_POOL_TOP, 8, cudaMemcpyHostToDevice, s));
        GRG_CUDA(c, cudaStreamSynchronize(s));
        return input_status(c);
    }
    if (c->h_ctr[C_ERR] & ERR_POOL) return fail(c, GRG_E_NOMEM, "element pool too small for the job");
    const uint64_t top1 = c->h_ctr[C_POOL_TOP];
    if (top1 > top0) k_init_region<<<grid_for(c, top1 - top0, 256), 256, 0, s>>>(c->elems, c->dbits, nullptr, top0, top1);
    if (num_edges)
        k_load_insert<<<grid_for(c, num_edges, 256), 256, 0, s>>>(d, dsrc, ddst, dlab, num_edges, base, num_vars,
                                                                  (uint32_t)c->L, c->tmask);
    for (int l = 1; l <= c->L; l++)
        if ((eps_mask >> (l - 1)) & 1ull) k_eps_insert<<<grid_for(c, num_vars, 256), 256, 0, s>>>(d, (uint32_t)l, base, num_vars);
    // rows of labels that no active rule derives are packed (as grg_closure does)
    bool derivable[MAX_LABELS + 1] = {false};
    for (int q = 0; q < c->R; q++) {
        const int *r = &c->rules[3 * q];
        const bool unary = r[1] && !r[2];
        if (!(c->filter && unary)) derivable[r[0]] = true;
    }
    for (int l = 1; l <= c->L; l++)
        if (!derivable[l]) k_compact_static<<<grid_for(c, num_vars, 256), 256, 0, s>>>(d, (uint32_t)l, base, num_vars);
    if (top1 > top0) k_mark_all<<<grid_for(c, top1 - top0, 256), 256, 0, s>>>(d, top0, top1);
    k_fill_u32<<<grid_for(c, num_vars, 256), 256, 0, s>>>(c->row_job + base, num_vars, job);
    GRG_CUDA(c, cudaGetLastError());
    st = read_ctr(c);
    if (st) return st;
    if (c->h_ctr[C_ERR]) return fail(c, GRG_E_INTERNAL, "internal error while admitting a job");
    c->jobs[job].base = base;
    c->jobs[job].nv = num_vars;
    c->jobs[job].active = true;
    c->jobs[job].pending = 0xFFFFFFFFu;
    return GRG_OK;
}

int grg_batch_step(grg_ctx *c, uint32_t max_rounds, uint32_t *job_records, uint64_t *rounds_run)
{
    if (!c) return GRG_E_ARG;
    if (!c->batch) return fail(c, GRG_E_STATE, "grg_batch_begin must come first");
    cudaSetDevice(c->device);
    grg_stats S;
    memset(&S, 0, sizeof S);
    double join_ms = 0;
    uint64_t joins = 0;
    bool idle = false;
    int st = run_rounds(c, max_rounds, S, join_ms, joins, &idle);
    if (st) return st;
    std::vector<uint32_t> cnt(c->max_jobs, 0);
    if (!idle) GRG_CUDA(c, cudaMemcpy(cnt.data(), c->job_cnt, sizeof(uint32_t) * c->max_jobs, cudaMemcpyDeviceToHost));
    for (uint32_t j = 0; j < c->max_jobs; j++)
        if (c->jobs[j].active) c->jobs[j].pending = cnt[j];
    if (job_records) memcpy(job_records, cnt.data(), sizeof(uint32_t) * c->max_jobs);
    if (rounds_run) *rounds_run = S.rounds;
    return GRG_OK;
}

int grg_batch_result(grg_ctx *c, uint32_t job, uint32_t label_offset, uint32_t num_labels, uint64_t *counts,
                     uint64_t *hash)
{
    if (!c || !counts) return GRG_E_ARG;
    if (!c->batch || job >= c->max_jobs || !c->jobs[job].active) return fail(c, GRG_E_STATE, "no such job");
    if (label_offset + num_labels > (uint32_t)c->L) return GRG_E_RANGE;
    cudaSetDevice(c->device);
    cudaStream_t s = c->stream;
    Dev d = make_dev(c);
    const uint32_t r0 = c->jobs[job].base, r1 = r0 + c->jobs[job].nv;
    GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_LABEL0, 0, sizeof(unsigned long long) * (MAX_SLOTS + 2), s));
    GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_HASH, 0, 8, s));
    for (uint32_t l = label_offset + 1; l <= label_offset + num_labels; l++)
        k_count<<<grid_for(c, (uint64_t)(r1 - r0) * 32, 256), 256, 0, s>>>(d, l, nullptr, nullptr, 0, 0, hash ? 1 : 0,
                                                                           r0, r1, label_offset, r0,
                                                                           (int)((c->tmask >> (l - 1)) & 1));
    GRG_CUDA(c, cudaGetLastError());
    int st = read_ctr(c);
    if (st) return st;
    for (uint32_t l = 0; l < num_labels; l++) counts[l] = c->h_ctr[C_LABEL0 + label_offset + 1 + l];
    if (hash) *hash = c->h_ctr[C_HASH];
    return GRG_OK;
}

int grg_batch_release(grg_ctx *c, uint32_t job)
{
    if (!c) return GRG_E_ARG;
    if (!c->batch || job >= c->max_jobs || !c->jobs[job].active) return fail(c, GRG_E_STATE, "no such job");
    if (c->jobs[job].pending != 0)
        return fail(c, GRG_E_STATE, "job has not reached its fixpoint (its last step gathered delta records)");
    cudaSetDevice(c->device);
    cudaStream_t s = c->stream;
    const uint32_t base = c->jobs[job].base, nv = c->jobs[job].nv;
    for (int slot = 1; slot <= c->L; slot++) {
        const size_t t0 = (size_t)(slot - 1) * c->V + base;
        GRG_CUDA(c, cudaMemsetAsync(c->desc + t0, 0, (size_t)nv * 8, s));
        GRG_CUDA(c, cudaMemsetAsync(c->cnt + t0, 0, (size_t)nv * 4, s));
        GRG_CUDA(c, cudaMemsetAsync(c->want + t0, 0, (size_t)nv * 4, s));
    }
    GRG_CUDA(c, cudaMemsetAsync(c->row_job + base, 0xFF, (size_t)nv * 4, s));
    GRG_CUDA(c, cudaStreamSynchronize(s));
    c->jobs[job].active = false;
    return GRG_OK;
}

}  // extern "C"

// ====================================================================== allocation-free closure
//
// grg_closure_noalloc runs the same kernels as grg_load_edges + grg_closure,
// but every scratch buffer they need (element pool, delta bitmaps, dirty and
// retry lists, delta records, table descriptors, counters) lives in one
// file-scope device array of fixed size instead of cudaMalloc'd memory. It is
// for callers that cannot allocate device memory while they run: a serving
// loop whose device memory is owned by another allocator or budget, or a
// process that must not let cudaMalloc/cudaFree synchronize the device while
// other jobs are in flight. Every GPU that loads this library reserves the
// array until the process exits.

namespace grg {

constexpr size_t NOALLOC_SCRATCH_BYTES = 64ull << 20;   // GRG_NOALLOC_SCRATCH_BYTES in grg.h
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

// Device address of g_noalloc_scratch per device ordinal, looked up once per
// device with that device current (the host-side symbol is not a device address).
static void *g_noalloc_addr[256];

static inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace grg

#define NA_CUDA(call)                                   \
    do {                                                \
        if ((call) != cudaSuccess) return GRG_E_CUDA;   \
    } while (0)

static int na_read(unsigned long long *h, const unsigned long long *ctr, cudaStream_t s)
{
    // pageable destination: no pinned buffer is needed (or allocated) by this path
    NA_CUDA(cudaMemcpyAsync(h, ctr, sizeof(unsigned long long) * NCTR, cudaMemcpyDeviceToHost, s));
    NA_CUDA(cudaStreamSynchronize(s));
    return GRG_OK;
}

namespace {
// restores the caller's current device on every return path
struct DeviceGuard {
    int prev = -1;
    ~DeviceGuard()
    {
        if (prev >= 0) cudaSetDevice(prev);
    }
};
}  // namespace

extern "C" int grg_closure_noalloc(int device, void *stream, int num_rules, const int *rules, int num_labels,
                                   uint32_t filter, uint32_t num_vars, uint64_t num_edges, const uint32_t *d_src,
                                   const uint32_t *d_dst, const uint8_t *d_label, uint64_t *d_label_counts,
                                   uint64_t *d_set_hash, uint64_t *rounds_out)
{
    if (device < 0 || device >= 256 || num_rules < 0 || num_rules > GRG_MAX_RULES || (num_rules && !rules) ||
        num_labels < 1 || num_labels > GRG_MAX_LABELS || filter > 1 || !d_label_counts ||
        (num_edges && (!d_src || !d_dst || !d_label)))
        return GRG_E_ARG;
    for (int q = 0; q < num_rules; q++) {
        const int *r = &rules[3 * q];
        if (r[0] < 1 || r[0] > num_labels || r[1] < 0 || r[1] > num_labels || r[2] < 0 || r[2] > num_labels ||
            (r[1] == 0 && r[2] != 0))
            return GRG_E_ARG;
    }
    // scratch layout: counters | descriptors | cnt | want | grow | delta index | pool arrays
    // (198 B per element slot: element, delta bitmap, dirty bit, slot id, four delta-record buffers) |
    // gather chunk counters. A round has at most one delta record per slot, old-left virtual
    // records at most one per (old-left rule, element), retries at most one per record.
    const uint64_t ntab = (uint64_t)num_labels * num_vars, vwords = (num_vars + 31) / 32;
    size_t off = 0;
    const size_t o_ctr = off; off = align256(off + sizeof(unsigned long long) * NCTR);
    const size_t o_desc = off; off = align256(off + ntab * 8);
    const size_t o_cnt = off; off = align256(off + ntab * 4);
    const size_t o_want = off; off = align256(off + ntab * 4);
    const size_t o_grow = off; off = align256(off + ntab * 4);
    const size_t o_drs = off; off = align256(off + ntab * 4);
    const size_t o_drc = off; off = align256(off + ntab * 4);
    const size_t o_dvm = off; off = align256(off + (uint64_t)num_labels * vwords * 4);
    if (off >= NOALLOC_SCRATCH_BYTES) return GRG_E_RANGE;            // tables alone exceed the scratch
    uint64_t pool = (NOALLOC_SCRATCH_BYTES - off - 16 * 256) / 198;
    if (pool < 4096 || num_edges > pool / 2) return GRG_E_RANGE;    // graph too large for the scratch
    const uint64_t pwords = pool / 32 + 2, pchunks = (pwords + 31) / 32, pnb = (pchunks + 1023) / 1024;
    const size_t o_elems = off; off = align256(off + pool * 32);
    const size_t o_dbits = off; off = align256(off + pool * 32);
    const size_t o_dmap = off; off = align256(off + pwords * 4);
    const size_t o_gslot = off; off = align256(off + pool * 4);
    const size_t o_gbuf = off; off = align256(off + pool * 32);
    const size_t o_vbuf = off; off = align256(off + pool * 32);
    const size_t o_rbuf0 = off; off = align256(off + pool * 32);
    const size_t o_rbuf1 = off; off = align256(off + pool * 32);
    const size_t o_chunk = off; off = align256(off + (2 * (pchunks + 1) + pnb + 2) * 4);
    if (off > NOALLOC_SCRATCH_BYTES) return GRG_E_RANGE;

    RuleTable rt;
    bool derivable[MAX_LABELS + 1];
    int st = make_rule_table(rules, num_rules, num_labels, filter, rt, derivable);
    if (st) return st;

    DeviceGuard guard;
    NA_CUDA(cudaGetDevice(&guard.prev));
    NA_CUDA(cudaSetDevice(device));
    if (!g_noalloc_addr[device]) {                 // set-up, once per device, with the device current
        void *p = nullptr;
        NA_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_noalloc_addr[device] = p;
    }
    unsigned char *base = (unsigned char *)g_noalloc_addr[device];
    cudaStream_t s = (cudaStream_t)stream;
    int sms = 0;
    NA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    auto grid = [&](uint64_t n, int block, int per_sm) {
        uint64_t g = (n + block - 1) / block, cap = (uint64_t)sms * per_sm;
        return (int)std::max<uint64_t>(std::min(g, cap), 1);
    };

    Dev d;
    d.ctr = (unsigned long long *)(base + o_ctr);
    d.desc = (uint64_t *)(base + o_desc);
    d.cnt = (uint32_t *)(base + o_cnt);
    d.want = (uint32_t *)(base + o_want);
    d.grow = (uint32_t *)(base + o_grow);
    d.elems = (uint32_t *)(base + o_elems);
    d.dbits = (uint32_t *)(base + o_dbits);
    d.dmap = (uint32_t *)(base + o_dmap);
    d.V = num_vars;
    d.pool_cap = (uint32_t)pool;
    d.cand = nullptr;          // no candidate buffer: joins insert directly
    d.cand_cap = 0;
    d.retry_cap = pool;        // a round's records (and so its retries) never exceed the pool
    d.drs = (uint32_t *)(base + o_drs);
    d.drc = (uint32_t *)(base + o_drc);
    d.dvm = (uint32_t *)(base + o_dvm);
    d.vwords = (uint32_t)vwords;
    d.stamp = nullptr;
    d.prefix_mask = 0;         // every table hashed
    d.rt = rt;                 // the grammar travels with every launch (no shared table)
    uint4 *gbuf = (uint4 *)(base + o_gbuf), *vbuf = (uint4 *)(base + o_vbuf);
    uint32_t *gslot = (uint32_t *)(base + o_gslot);
    d.drec = gbuf;
    uint4 *rbuf[2] = {(uint4 *)(base + o_rbuf0), (uint4 *)(base + o_rbuf1)};
    uint32_t *chunk = (uint32_t *)(base + o_chunk);
    unsigned long long h[NCTR];

    // the array keeps the previous call's contents: clear everything that must start at zero
    NA_CUDA(cudaMemsetAsync(d.ctr, 0, sizeof(unsigned long long) * NCTR, s));
    NA_CUDA(cudaMemsetAsync(d.desc, 0, ntab * 8, s));
    NA_CUDA(cudaMemsetAsync(d.cnt, 0, ntab * 4, s));
    NA_CUDA(cudaMemsetAsync(d.want, 0, ntab * 4, s));
    NA_CUDA(cudaMemsetAsync(d.dmap, 0, pwords * 4, s));
    NA_CUDA(cudaMemsetAsync(d.drs, 0xFF, ntab * 4, s));
    NA_CUDA(cudaMemsetAsync(d.drc, 0, ntab * 4, s));
    NA_CUDA(cudaMemsetAsync(d.dvm, 0, (uint64_t)num_labels * vwords * 4, s));

    // load (grg_load_edges)
    const uint64_t nlab = (uint64_t)num_labels * num_vars;
    if (num_edges) k_load_hist<<<grid(num_edges, 256, 8), 256, 0, s>>>(d, d_src, d_dst, d_label, num_edges, 0, num_vars, (uint32_t)num_labels, 0ull);
    for (int q = 0; q < num_rules; q++)
        if (rules[3 * q + 1] == 0) k_eps_hist<<<grid(num_vars, 256, 8), 256, 0, s>>>(d, (uint32_t)rules[3 * q], 0, num_vars);
    MinCap mc;
    memset(&mc, 0, sizeof mc);
    k_load_alloc<<<grid(nlab, 256, 8), 256, 0, s>>>(d, 0, num_vars, (uint32_t)num_labels, mc, nullptr);
    if ((st = na_read(h, d.ctr, s))) return st;
    if (h[C_BADIN] & ERR_IN_LABEL) return GRG_E_LABEL;
    if (h[C_BADIN] & ERR_IN_RANGE) return GRG_E_RANGE;
    if (h[C_ERR] & ERR_POOL) return GRG_E_NOMEM;
    const uint64_t top0 = h[C_POOL_TOP];
    if (top0) k_init_region<<<grid(top0, 256, 8), 256, 0, s>>>(d.elems, d.dbits, nullptr, 0, top0);
    if (num_edges) k_load_insert<<<grid(num_edges, 256, 8), 256, 0, s>>>(d, d_src, d_dst, d_label, num_edges, 0, num_vars, (uint32_t)num_labels, 0ull);
    for (int q = 0; q < num_rules; q++)
        if (rules[3 * q + 1] == 0) k_eps_insert<<<grid(num_vars, 256, 8), 256, 0, s>>>(d, (uint32_t)rules[3 * q], 0, num_vars);
    for (int l = 1; l <= num_labels; l++)
        if (!derivable[l]) k_compact_static<<<grid(num_vars, 256, 8), 256, 0, s>>>(d, (uint32_t)l, 0, num_vars);
    if (top0) k_mark_all<<<grid(top0, 256, 8), 256, 0, s>>>(d, 0, top0);
    NA_CUDA(cudaGetLastError());
    if ((st = na_read(h, d.ctr, s))) return st;
    if (h[C_ERR] & ERR_POOL) return GRG_E_NOMEM;
    if (h[C_ERR]) return GRG_E_INTERNAL;

    // semi-naive rounds (grg_closure); the pool cannot grow here
    uint64_t rounds = 0;
    for (;;) {
        if ((st = na_read(h, d.ctr, s))) return st;
        const uint64_t nwords = (h[C_POOL_TOP] + 31) / 32, nchunks = (nwords + 31) / 32;
        const uint64_t nb = (nchunks + 1023) / 1024;
        uint32_t *ccnt = chunk, *coff = chunk + nchunks + 1, *csum = chunk + 2 * (nchunks + 1);
        k_dcount<<<grid(nchunks * 32, 256, 8), 256, 0, s>>>(d, nwords, ccnt, 0);
        k_scan_blocks<<<(unsigned)std::max<uint64_t>(nb, 1), 1024, 0, s>>>(ccnt, coff, csum, nchunks, nullptr);
        k_scan_sums<<<1, 1024, 0, s>>>(csum, nb, nullptr);
        k_scan_add<<<(unsigned)std::max<uint64_t>(nb, 1), 1024, 0, s>>>(coff, csum, nchunks, nullptr);
        uint32_t nd32 = 0;
        NA_CUDA(cudaMemcpyAsync(&nd32, csum + nb, 4, cudaMemcpyDeviceToHost, s));
        NA_CUDA(cudaStreamSynchronize(s));
        const uint64_t nd = nd32;
        if (nd == 0) break;
        rounds++;
        for (int l = 1; l <= num_labels; l++)
            if (rt.dindex[l]) {
                NA_CUDA(cudaMemsetAsync(d.drs + (size_t)(l - 1) * num_vars, 0xFF, (size_t)num_vars * 4, s));
                NA_CUDA(cudaMemsetAsync(d.drc + (size_t)(l - 1) * num_vars, 0, (size_t)num_vars * 4, s));
                NA_CUDA(cudaMemsetAsync(d.dvm + (size_t)(l - 1) * vwords, 0, vwords * 4, s));
            }
        k_gather_slots<<<grid(nchunks * 32, 256, 8), 256, 0, s>>>(d, nwords, coff, gslot, 0);
        k_gather_recs<<<grid(nd, 256, 8), 256, 0, s>>>(d, gslot, gbuf, nd, -1, nullptr, nullptr, 0);
        uint64_t nv = 0;
        if (rt.nol) {
            NA_CUDA(cudaMemsetAsync(d.ctr + C_VN, 0, 8, s));
            for (int q = 0; q < rt.nol; q++)
                k_oldleft<<<grid(num_vars, 256, 8), 256, 0, s>>>(d, (uint32_t)q, vbuf, pool, nullptr, nullptr);
            if ((st = na_read(h, d.ctr, s))) return st;
            nv = h[C_VN];
            if (nd + nv > pool) return GRG_E_NOMEM;                // records (and their retries) outgrew the scratch
        }
        NA_CUDA(cudaMemsetAsync(d.ctr + C_RETRY_N, 0, 16, s));
        uint64_t n = nd;
        int rb = 0;
        for (int pass = 0;; pass++) {
            const int g = grid((n + RB - 1) / RB, JOIN_WARPS, 16);
            // each join launch pulls 32-record batches from a queue that starts at 0
            if (pass == 0) {
                NA_CUDA(cudaMemsetAsync(d.ctr + C_JQ, 0, 8, s));
                k_join<WIN, WIN_LO><<<g, JOIN_WARPS * 32, 0, s>>>(d, gbuf, nd, -1, rbuf[0]);
                if (nv) {
                    NA_CUDA(cudaMemsetAsync(d.ctr + C_JQ, 0, 8, s));
                    k_join<WIN, WIN_LO><<<grid((nv + RB - 1) / RB, JOIN_WARPS, 16), JOIN_WARPS * 32, 0, s>>>(d, vbuf, nv,
                                                                                                        -1, rbuf[0]);
                }
            } else {
                NA_CUDA(cudaMemsetAsync(d.ctr + C_JQ, 0, 8, s));
                k_join<WIN, WIN_LO><<<g, JOIN_WARPS * 32, 0, s>>>(d, rbuf[rb], n, -1, rbuf[rb ^ 1]);
            }
            NA_CUDA(cudaGetLastError());
            if ((st = na_read(h, d.ctr, s))) return st;
            const uint64_t nr = h[C_RETRY_N];
            if (nr == 0) break;
            NA_CUDA(cudaMemsetAsync(d.ctr + C_ERR, 0, 8, s));
            k_grow<<<grid(h[C_GROW_N] * 32, 256, 8), 256, 0, s>>>(d, h[C_GROW_N]);
            if ((st = na_read(h, d.ctr, s))) return st;
            if (h[C_ERR] & ERR_POOL) return GRG_E_NOMEM;          // closure outgrew the scratch
            if (pass > 64) return GRG_E_INTERNAL;             // table growth did not converge
            rb = pass == 0 ? 0 : rb ^ 1;
            n = nr;
            NA_CUDA(cudaMemsetAsync(d.ctr + C_RETRY_N, 0, 16, s));
        }
    }

    // per-label counts and edge-set hash into the caller's device buffers
    NA_CUDA(cudaMemsetAsync(d.ctr + C_LABEL0, 0, sizeof(unsigned long long) * (MAX_SLOTS + 2), s));
    NA_CUDA(cudaMemsetAsync(d.ctr + C_HASH, 0, 8, s));
    for (int l = 1; l <= num_labels; l++)
        k_count<<<grid((uint64_t)num_vars * 32, 256, 8), 256, 0, s>>>(d, (uint32_t)l, nullptr, nullptr, 0, 0, d_set_hash ? 1 : 0, 0, num_vars, 0, 0, 0);
    NA_CUDA(cudaMemcpyAsync(d_label_counts, d.ctr + C_LABEL0 + 1, sizeof(uint64_t) * num_labels,
                            cudaMemcpyDeviceToDevice, s));
    if (d_set_hash) NA_CUDA(cudaMemcpyAsync(d_set_hash, d.ctr + C_HASH, 8, cudaMemcpyDeviceToDevice, s));
    NA_CUDA(cudaGetLastError());
    NA_CUDA(cudaStreamSynchronize(s));
    if (rounds_out) *rounds_out = rounds;
    return GRG_OK;
}
