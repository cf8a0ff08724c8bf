// grg_engine.cu -- CUDA kernels and the C ABI of the closure engine (sm_103a).
//
// Hot path (reference: src/kernel.cu):
//   k_join    binary joins A ::= B C for a round's delta records, delta-left
//             (D_B o O_C) and old-left (O_B o D_C through a reverse index),
//             unary rules A ::= B, and dedup of every candidate against the
//             stored rows. Replaces compute11/compute10 (src/kernel.cu:403-442)
//             and diff/merge (src/kernel.cu:841-985).
//   k_gather  turns the dirty list of the last round into delta records
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
#include <string>
#include <vector>

#include "grg.h"
#include "grg_device.cuh"

namespace grg {

__constant__ RuleTable c_rt;

constexpr int JOIN_WARPS = 8;     // warps per join block
constexpr int ACC = 64;           // per-warp accumulator entries
constexpr int ACC_MAX = ACC * 3 / 4;

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31; }

// ---------------------------------------------------------------- loader

__global__ void k_init_region(uint32_t *elems, uint32_t *dbits, uint64_t begin, uint64_t end)
{
    for (uint64_t s = begin + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < end;
         s += (uint64_t)gridDim.x * blockDim.x) {
        uint4 *e = reinterpret_cast<uint4 *>(elems + s * 8);
        e[0] = make_uint4(0, 0, 0, 0);
        e[1] = make_uint4(0, 0, EMPTY, 0);
        uint4 *b = reinterpret_cast<uint4 *>(dbits + s * 8);
        b[0] = make_uint4(0, 0, 0, 0);
        b[1] = make_uint4(0, 0, 0, 0);
    }
}

__global__ void k_load_hist(Dev d, const uint32_t *src, const uint8_t *lab, uint64_t n)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        atomicAdd(&d.cnt[(size_t)(lab[i] - 1) * d.V + src[i]], 1u);
}

__global__ void k_eps_hist(Dev d, uint32_t slot)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < d.V; v += gridDim.x * blockDim.x)
        atomicAdd(&d.cnt[(size_t)(slot - 1) * d.V + v], 1u);
}

// One thread per table: size from the edge histogram (held in cnt), bump-allocate.
__global__ void k_load_alloc(Dev d, uint64_t ntables)
{
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < ((ntables + 31) & ~31ull);
         t += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t h = t < ntables ? d.cnt[t] : 0;
        uint32_t cap = 0;
        if (h) {
            uint32_t need = h + h / 3 + 1;
            cap = 4;
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
        if (t < ntables) {
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

__global__ void k_load_insert(Dev d, const uint32_t *src, const uint32_t *dst, const uint8_t *lab, uint64_t n)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t v = dst[i];
        Bits b;
#pragma unroll
        for (int w = 0; w < EW; w++) b.w[w] = 0;
        uint32_t o = v % EIDS;
        b.w[o >> 5] = 1u << (o & 31);
        if (!g_insert(d, lab[i], src[i], v / EIDS, b, false)) atomicOr(&d.ctr[C_ERR], (unsigned long long)ERR_LOAD);
    }
}

// Epsilon rules A ::= eps: (v, v, A) for every vertex (compute00, src/kernel.cu:445-464).
__global__ void k_eps_insert(Dev d, uint32_t slot)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < d.V; v += gridDim.x * blockDim.x) {
        Bits b;
#pragma unroll
        for (int w = 0; w < EW; w++) b.w[w] = 0;
        uint32_t o = v % EIDS;
        b.w[o >> 5] = 1u << (o & 31);
        if (!g_insert(d, slot, v, v / EIDS, b, false)) atomicOr(&d.ctr[C_ERR], (unsigned long long)ERR_LOAD);
    }
}

// Rows of labels that are never inserted into after the load are packed:
// occupied slots moved to the front, capacity = count (no empty slots to scan).
__global__ void k_compact_static(Dev d, uint32_t slot)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < d.V; v += gridDim.x * blockDim.x) {
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
                uint4 *t = reinterpret_cast<uint4 *>(d.elems + (size_t)(off + wpos) * 8);
                t[0] = e[0];
                t[1] = e1;
                e[0] = make_uint4(0, 0, 0, 0);
                e[1] = make_uint4(0, 0, EMPTY, 0);
            }
            wpos++;
        }
        d.desc[ti] = wpos ? ((uint64_t)wpos << 32) | off : 0ull;
        d.cnt[ti] = wpos;
    }
}

// Every loaded element of a tracked label becomes a delta of round 1.
__global__ void k_mark_all(Dev d, uint64_t end)
{
    for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < end; s += (uint64_t)gridDim.x * blockDim.x) {
        const uint4 *e = reinterpret_cast<const uint4 *>(d.elems + s * 8);
        uint4 e1 = e[1];
        if (e1.z == EMPTY || !c_rt.track[e1.z >> KEY_SHIFT]) continue;
        uint4 e0 = e[0];
        uint4 *b = reinterpret_cast<uint4 *>(d.dbits + s * 8);
        b[0] = e0;
        b[1] = make_uint4(e1.x, e1.y, 1u, 0u);
        append_dirty(d, (uint32_t)s);
    }
}

// ---------------------------------------------------------------- rounds

// Dirty slots -> delta records (32 B: bits[6], key, row); clears the delta bitmap.
__global__ void k_gather(Dev d, uint64_t n, uint4 *delta)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t s = d.dirty[i];
        uint4 *b = reinterpret_cast<uint4 *>(d.dbits + (size_t)s * 8);
        const uint4 b0 = b[0], b1 = b[1];
        const uint4 e1 = reinterpret_cast<const uint4 *>(d.elems + (size_t)s * 8)[1];
        b[0] = make_uint4(0, 0, 0, 0);
        b[1] = make_uint4(0, 0, 0, 0);
        delta[2 * i] = b0;
        delta[2 * i + 1] = make_uint4(b1.x, b1.y, e1.z, e1.w);
    }
}

struct __align__(16) WarpSmem {
    uint32_t acc_bits[ACC][EW];
    uint32_t acc_key[ACC];
    uint32_t klist[EIDS];
    uint32_t koff[EIDS];
    uint32_t kpre[EIDS + 1];
    uint32_t acc_n;
};

__device__ __forceinline__ bool acc_insert(WarpSmem &w, uint32_t base, const Bits &b)
{
    volatile uint32_t *keys = w.acc_key;
    uint32_t h = (base * 0x9E3779B1u) >> (32 - 6);
    for (int p = 0; p < ACC; p++) {
        uint32_t q = (h + p) & (ACC - 1);
        uint32_t k = keys[q];
        if (k == base) {
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
        uint32_t prev = atomicCAS(&w.acc_key[q], EMPTY, base);
        if (prev != EMPTY) atomicSub(&w.acc_n, 1u);
        if (prev == EMPTY || prev == base) {
#pragma unroll
            for (int x = 0; x < EW; x++)
                if (b.w[x]) atomicOr(&w.acc_bits[q][x], b.w[x]);
            return true;
        }
    }
    return false;
}

// Flush the warp's accumulator into row (A, row). Returns false if any insert failed.
__device__ __forceinline__ bool acc_flush(const Dev &d, WarpSmem &w, uint32_t A, uint32_t row, bool track,
                                          uint32_t &inserts)
{
    __syncwarp();
    bool ok = true;
    for (int j = lane_id(); j < ACC; j += 32) {
        uint32_t k = w.acc_key[j];
        if (k == EMPTY) continue;
        Bits b;
#pragma unroll
        for (int x = 0; x < EW; x++) { b.w[x] = w.acc_bits[j][x]; w.acc_bits[j][x] = 0; }
        w.acc_key[j] = EMPTY;
        ok &= g_insert(d, A, row, k, b, track);
        inserts++;
    }
    __syncwarp();
    if (lane_id() == 0) w.acc_n = 0;
    __syncwarp();
    return ok;
}

// One warp per delta record (label B, row i, base, bits).
__global__ void __launch_bounds__(JOIN_WARPS * 32) k_join(Dev d, const uint4 *__restrict__ delta, uint64_t n,
                                                          const uint32_t *__restrict__ idx, uint32_t *retry_out)
{
    __shared__ WarpSmem smem[JOIN_WARPS];
    WarpSmem &w = smem[threadIdx.x >> 5];
    const uint32_t lane = lane_id();
    for (int j = lane; j < ACC; j += 32) {
        w.acc_key[j] = EMPTY;
#pragma unroll
        for (int x = 0; x < EW; x++) w.acc_bits[j][x] = 0;
    }
    if (lane == 0) { w.acc_n = 0; w.kpre[0] = 0; }
    __syncwarp();
    unsigned long long n_left = 0, n_right = 0;
    uint32_t inserts = 0;
    const uint64_t nwarps = (uint64_t)gridDim.x * JOIN_WARPS;
    for (uint64_t r = blockIdx.x * (uint64_t)JOIN_WARPS + (threadIdx.x >> 5); r < n; r += nwarps) {
        const uint64_t ri = idx ? idx[r] : r;
        const uint32_t *rec = reinterpret_cast<const uint32_t *>(delta + 2 * ri);
        uint32_t word = lane < 8 ? rec[lane] : 0u;
        Bits rb;
#pragma unroll
        for (int x = 0; x < EW; x++) rb.w[x] = __shfl_sync(0xffffffffu, word, x);
        const uint32_t key = __shfl_sync(0xffffffffu, word, 6);
        const uint32_t row = __shfl_sync(0xffffffffu, word, 7);
        const uint32_t B = key >> KEY_SHIFT, base = key & BASE_MASK;
        bool ok = true;

        // unary rules A ::= B (compute10): the delta itself joins row (A, row)
        for (int q = c_rt.un_start[B]; q < c_rt.un_start[B + 1]; q++)
            if (lane == 0) { ok &= g_insert(d, c_rt.un_A[q], row, base, rb, c_rt.track[c_rt.un_A[q]]); inserts++; }

        // decode the intermediate vertices k of this record
        uint32_t nk = 0;
#pragma unroll
        for (int x = 0; x < EW; x++) {
            const uint32_t bw = rb.w[x];
            if ((bw >> lane) & 1u) w.klist[nk + __popc(bw & ((1u << lane) - 1u))] = base * EIDS + x * 32 + lane;
            nk += __popc(bw);
        }
        __syncwarp();

        // reverse index of B (needed by old-left joins): rev_B[k] gets row
        const uint32_t rs = c_rt.rev_slot[B];
        if (rs) {
            Bits ib;
#pragma unroll
            for (int x = 0; x < EW; x++) ib.w[x] = 0;
            const uint32_t o = row % EIDS;
            ib.w[o >> 5] = 1u << (o & 31);
            for (uint32_t j = lane; j < nk; j += 32) { ok &= g_insert(d, rs, w.klist[j], row / EIDS, ib, false); inserts++; }
        }

        // binary rules A ::= B C, delta-left: union of rows C[k] into row (A, row)
        for (int q = c_rt.bin_start[B]; q < c_rt.bin_start[B + 1]; q++) {
            const uint32_t A = c_rt.bin_A[q], C = c_rt.bin_C[q];
            const bool trk = c_rt.track[A];
            uint32_t total = 0;
            for (uint32_t j0 = 0; j0 < nk; j0 += 32) {
                const uint32_t j = j0 + lane;
                uint32_t cap = 0, off = 0;
                if (j < nk) {
                    const uint64_t de = d.desc[(size_t)(C - 1) * d.V + w.klist[j]];
                    off = (uint32_t)de;
                    cap = (uint32_t)(de >> 32);
                }
                uint32_t incl = cap;
                for (int o = 1; o < 32; o <<= 1) {
                    uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= (uint32_t)o) incl += y;
                }
                if (j < nk) { w.koff[j] = off; w.kpre[j + 1] = total + incl; }
                total += __shfl_sync(0xffffffffu, incl, 31);
            }
            __syncwarp();
            n_left++;
            for (uint32_t t0 = 0; t0 < total; t0 += 32) {
                const uint32_t t = t0 + lane;
                bool pending = false;
                uint32_t ebase = 0;
                Bits eb;
                if (t < total) {
                    // largest j with kpre[j] <= t
                    uint32_t lo = 0, hi = nk;
                    while (lo < hi) {
                        uint32_t mid = (lo + hi + 1) >> 1;
                        if (w.kpre[mid] <= t) lo = mid; else hi = mid - 1;
                    }
                    const uint32_t s = w.koff[lo] + (t - w.kpre[lo]);
                    const uint4 *ep = reinterpret_cast<const uint4 *>(d.elems + (size_t)s * 8);
                    const uint4 e0 = ep[0], e1 = ep[1];
                    if (e1.z != EMPTY) {
                        pending = true;
                        ebase = e1.z & BASE_MASK;
                        eb.w[0] = e0.x; eb.w[1] = e0.y; eb.w[2] = e0.z; eb.w[3] = e0.w;
                        eb.w[4] = e1.x; eb.w[5] = e1.y;
                    }
                }
                n_right += __popc(__ballot_sync(0xffffffffu, pending)) * (lane == 0);
                while (__any_sync(0xffffffffu, pending)) {
                    if (pending) pending = !acc_insert(w, ebase, eb);
                    if (__any_sync(0xffffffffu, pending)) ok &= acc_flush(d, w, A, row, trk, inserts);
                }
            }
            ok &= acc_flush(d, w, A, row, trk, inserts);
        }

        // old-left joins A ::= Bp B (this record is a delta of B at vertex `row`):
        // every h with Bp(h, row) gets the record's bits in row (A, h)
        for (int q = c_rt.ol_start[B]; q < c_rt.ol_start[B + 1]; q++) {
            const uint32_t A = c_rt.ol_A[q], rv = c_rt.ol_rev[q];
            const bool trk = c_rt.track[A];
            const uint64_t de = d.desc[(size_t)(rv - 1) * d.V + row];
            const uint32_t off = (uint32_t)de, cap = (uint32_t)(de >> 32);
            for (uint32_t t = lane; t < cap; t += 32) {
                const uint4 *ep = reinterpret_cast<const uint4 *>(d.elems + (size_t)(off + t) * 8);
                const uint4 e0 = ep[0], e1 = ep[1];
                if (e1.z == EMPTY) continue;
                const uint32_t hb = e1.z & BASE_MASK;
                const uint32_t hw[EW] = {e0.x, e0.y, e0.z, e0.w, e1.x, e1.y};
#pragma unroll
                for (int x = 0; x < EW; x++) {
                    uint32_t bw = hw[x];
                    while (bw) {
                        const int bit = __ffs(bw) - 1;
                        bw &= bw - 1;
                        ok &= g_insert(d, A, hb * EIDS + x * 32 + bit, base, rb, trk);
                        inserts++;
                    }
                }
            }
        }

        if (__any_sync(0xffffffffu, !ok) && lane == 0) {
            unsigned long long p = atomicAdd(&d.ctr[C_RETRY_N], 1ull);
            retry_out[p] = (uint32_t)ri;
        }
    }
    // per-warp work counters
    for (int o = 16; o; o >>= 1) inserts += __shfl_xor_sync(0xffffffffu, inserts, o);
    if (lane == 0) {
        if (n_left) atomicAdd(&d.ctr[C_LEFT], n_left);
        if (n_right) atomicAdd(&d.ctr[C_RIGHT], n_right);
        if (inserts) atomicAdd(&d.ctr[C_INSERTS], (unsigned long long)inserts);
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
        }
        __syncwarp();
        const uint32_t lg = 31 - __clz(ncap);
        for (uint32_t t = lane; t < cap; t += 32) {
            const uint4 *e = reinterpret_cast<const uint4 *>(d.elems + (size_t)(off + t) * 8);
            const uint4 e0 = e[0], e1 = e[1];
            if (e1.z == EMPTY) continue;
            uint32_t h = hash_slot(e1.z & BASE_MASK, lg);
            for (uint32_t p = 0; p < ncap; p++) {
                const uint64_t q = nb + ((h + p) & (ncap - 1));
                if (atomicCAS(d.elems + q * 8 + 6, EMPTY, e1.z) == EMPTY) {
                    uint4 *t2 = reinterpret_cast<uint4 *>(d.elems + q * 8);
                    t2[0] = e0;
                    d.elems[q * 8 + 4] = e1.x;
                    d.elems[q * 8 + 5] = e1.y;
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
__global__ void k_count(Dev d, uint32_t slot, uint32_t *deg_edges, uint32_t *deg_elems, uint32_t first,
                        uint32_t last, int do_hash)
{
    const uint32_t lane = lane_id();
    const uint64_t nwarps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    unsigned long long my_edges = 0, my_hash = 0;
    for (uint64_t v = blockIdx.x * (uint64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); v < d.V; v += nwarps) {
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
                        my_hash += edge_hash(slot, (uint32_t)v, hb * EIDS + x * 32 + bit);
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

__global__ void k_export(Dev d, uint32_t slot, uint32_t *src, uint32_t *dst, uint8_t *lab, uint64_t cap_out)
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
                        src[pos] = (uint32_t)v;
                        dst[pos] = hb * EIDS + x * 32 + bit;
                        lab[pos] = (uint8_t)slot;
                    }
                    pos++;
                }
            }
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
    uint64_t ntables_alloc = 0;    // 2L * V (with reverse slots)
    // device memory
    uint64_t pool_bytes_req = 0;
    uint64_t pool_cap = 0;         // elements
    uint32_t *elems = nullptr, *dbits = nullptr, *dirty = nullptr;
    uint64_t *desc = nullptr;
    uint32_t *cnt = nullptr, *want = nullptr, *grow = nullptr;
    uint4 *delta = nullptr;
    uint64_t delta_cap = 0;        // records
    uint32_t *retry[2] = {nullptr, nullptr};
    uint64_t retry_cap = 0;
    unsigned long long *ctr = nullptr;
    unsigned long long *h_ctr = nullptr;   // pinned
    uint32_t *d_in32 = nullptr;            // staged input edges (src, dst)
    uint8_t *d_in8 = nullptr;
    uint64_t in_cap = 0;
    RuleTable rt{};
    uint64_t launches = 0;
};

namespace {

const char *status_text(int s)
{
    switch (s) {
    case GRG_OK: return "ok";
    case GRG_NEED_REPARTITION: return "partition needs repartitioning";
    case GRG_E_ARG: return "invalid argument";
    case GRG_E_CUDA: return "CUDA error";
    case GRG_E_NOMEM: return "out of memory";
    case GRG_E_FILTER: return "filter_flag=1 is schedule-dependent for this grammar (a binary rule's second symbol is derivable)";
    case GRG_E_IO: return "I/O or format error";
    case GRG_E_LABEL: return "graph label not in grammar";
    case GRG_E_RANGE: return "value out of range";
    case GRG_E_STATE: return "call out of order";
    case GRG_E_NODEV: return "no CUDA device";
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
    d.desc = c->desc;
    d.cnt = c->cnt;
    d.want = c->want;
    d.dirty = c->dirty;
    d.grow = c->grow;
    d.ctr = c->ctr;
    d.V = c->V;
    d.pool_cap = (uint32_t)c->pool_cap;
    return d;
}

void free_graph(grg_ctx *c)
{
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
    cudaFree(c->dirty); c->dirty = nullptr;
    c->pool_cap = 0;
}

int read_ctr(grg_ctx *c)
{
    GRG_CUDA(c, cudaMemcpyAsync(c->h_ctr, c->ctr, sizeof(unsigned long long) * NCTR, cudaMemcpyDeviceToHost, c->stream));
    GRG_CUDA(c, cudaStreamSynchronize(c->stream));
    return GRG_OK;
}


// Pool of `elems` 32-byte slots + delta bitmaps + dirty list (68 bytes per slot).
int alloc_pool(grg_ctx *c, uint64_t elems)
{
    if (elems > 0xFFFFFFF0ull) elems = 0xFFFFFFF0ull;
    uint32_t *e = nullptr, *b = nullptr, *dl = nullptr;
    if (cudaMalloc(&e, elems * 32) != cudaSuccess || cudaMalloc(&b, elems * 32) != cudaSuccess ||
        cudaMalloc(&dl, elems * 4) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(e); cudaFree(b); cudaFree(dl);
        return fail(c, GRG_E_NOMEM, "cannot allocate element pool of " + std::to_string(elems) + " slots");
    }
    if (c->elems) {
        // grow: keep the used part and the pending dirty list
        int st = read_ctr(c);
        if (st) { cudaFree(e); cudaFree(b); cudaFree(dl); return st; }
        uint64_t used = std::min<uint64_t>(c->h_ctr[C_POOL_TOP], c->pool_cap);
        uint64_t nd = c->h_ctr[C_DIRTY_N];
        GRG_CUDA(c, cudaMemcpyAsync(e, c->elems, used * 32, cudaMemcpyDeviceToDevice, c->stream));
        GRG_CUDA(c, cudaMemcpyAsync(b, c->dbits, used * 32, cudaMemcpyDeviceToDevice, c->stream));
        GRG_CUDA(c, cudaMemcpyAsync(dl, c->dirty, nd * 4, cudaMemcpyDeviceToDevice, c->stream));
        GRG_CUDA(c, cudaStreamSynchronize(c->stream));
        free_pool(c);
    }
    c->elems = e;
    c->dbits = b;
    c->dirty = dl;
    c->pool_cap = elems;
    return GRG_OK;
}

int grow_pool(grg_ctx *c, uint64_t min_elems)
{
    uint64_t want = std::max<uint64_t>(c->pool_cap * 2, min_elems);
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    uint64_t fit = (uint64_t)((double)fr * 0.9) / 68;
    if (want > fit) want = fit;
    if (want <= c->pool_cap) return fail(c, GRG_E_NOMEM, "element pool exhausted and device memory is full");
    return alloc_pool(c, want);
}

int ensure_delta(grg_ctx *c, uint64_t n)
{
    if (n <= c->delta_cap) return GRG_OK;
    uint64_t cap = std::max<uint64_t>(n + n / 2, 1 << 16);
    cudaFree(c->delta);
    cudaFree(c->retry[0]);
    cudaFree(c->retry[1]);
    c->delta = nullptr; c->retry[0] = c->retry[1] = nullptr;
    GRG_CUDA(c, cudaMalloc(&c->delta, cap * 32));
    GRG_CUDA(c, cudaMalloc(&c->retry[0], cap * 4));
    GRG_CUDA(c, cudaMalloc(&c->retry[1], cap * 4));
    c->delta_cap = cap;
    return GRG_OK;
}

// Build the rule table for a filter (filter semantics: src/kernel.cu:490-494, 499-503 ...).
int build_rules(grg_ctx *c, uint32_t filter, RuleTable &rt)
{
    memset(&rt, 0, sizeof rt);
    const int L = c->L;
    rt.L = L;
    bool derivable[MAX_LABELS + 1] = {false};
    for (int q = 0; q < c->R; q++) {
        const int *r = &c->rules[3 * q];
        bool unary = r[1] && !r[2];
        if (!(filter && unary)) derivable[r[0]] = true;
    }
    bool need_ol[GRG_MAX_RULES] = {false};
    for (int q = 0; q < c->R; q++) {
        const int *r = &c->rules[3 * q];
        if (r[1] && r[2] && derivable[r[2]]) {
            if (filter) return fail(c, GRG_E_FILTER, status_text(GRG_E_FILTER));
            need_ol[q] = true;
        }
    }
    int next_rev = L + 1;
    for (int q = 0; q < c->R; q++)
        if (need_ol[q] && !rt.rev_slot[c->rules[3 * q + 1]]) rt.rev_slot[c->rules[3 * q + 1]] = (uint8_t)next_rev++;
    rt.num_slots = next_rev - 1;
    // binary rules grouped by RHS1
    int k = 0;
    for (int B = 1; B <= L + 1; B++) {
        rt.bin_start[B] = (uint8_t)k;
        if (B > L) break;
        for (int q = 0; q < c->R; q++) {
            const int *r = &c->rules[3 * q];
            if (r[1] == B && r[2]) { rt.bin_A[k] = (uint8_t)r[0]; rt.bin_C[k] = (uint8_t)r[2]; k++; }
        }
    }
    rt.bin_start[0] = 0;
    k = 0;
    for (int B = 1; B <= L + 1; B++) {
        rt.un_start[B] = (uint8_t)k;
        if (B > L) break;
        if (filter) continue;
        for (int q = 0; q < c->R; q++) {
            const int *r = &c->rules[3 * q];
            if (r[1] == B && !r[2]) rt.un_A[k++] = (uint8_t)r[0];
        }
    }
    k = 0;
    for (int C = 1; C <= L + 1; C++) {
        rt.ol_start[C] = (uint8_t)k;
        if (C > L) break;
        for (int q = 0; q < c->R; q++) {
            const int *r = &c->rules[3 * q];
            if (need_ol[q] && r[2] == C) { rt.ol_A[k] = (uint8_t)r[0]; rt.ol_rev[k] = rt.rev_slot[r[1]]; k++; }
        }
    }
    // tracked labels: left operand of an active binary/unary rule, or right operand of an old-left join
    for (int q = 0; q < c->R; q++) {
        const int *r = &c->rules[3 * q];
        bool unary = r[1] && !r[2];
        if (r[1] && !(filter && unary)) rt.track[r[1]] = 1;
        if (need_ol[q]) rt.track[r[2]] = 1;
    }
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
    cudaFree(c->delta);
    cudaFree(c->retry[0]);
    cudaFree(c->retry[1]);
    cudaFree(c->ctr);
    cudaFree(c->d_in32);
    cudaFree(c->d_in8);
    if (c->h_ctr) cudaFreeHost(c->h_ctr);
    if (c->ev_a) cudaEventDestroy(c->ev_a);
    if (c->ev_b) cudaEventDestroy(c->ev_b);
    if (c->ev_c) cudaEventDestroy(c->ev_c);
    if (c->ev_d) cudaEventDestroy(c->ev_d);
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
    c->have_rules = true;
    c->loaded = false;
    return GRG_OK;
}

int grg_allocate_pool(grg_ctx *c, uint64_t pool_bytes)
{
    if (!c) return GRG_E_ARG;
    cudaSetDevice(c->device);
    c->pool_bytes_req = pool_bytes;
    uint64_t elems;
    if (pool_bytes) {
        elems = pool_bytes / 68;
    } else {
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        elems = (uint64_t)(fr / 8) / 68;   // start at 1/8 of free memory; grows on demand
    }
    if (elems < 1024) elems = 1024;
    if (c->elems && c->pool_cap >= elems) return GRG_OK;
    free_pool(c);
    return alloc_pool(c, elems);
}

int grg_load_edges(grg_ctx *c, uint32_t num_vars, uint64_t num_edges, const uint32_t *src, const uint32_t *dst,
                   const uint8_t *label, int on_device)
{
    if (!c || (num_edges && (!src || !dst || !label))) return GRG_E_ARG;
    if (!c->have_rules) return fail(c, GRG_E_STATE, "grg_transfer_rules must come first");
    cudaSetDevice(c->device);
    if (!c->elems) {
        int st = grg_allocate_pool(c, c->pool_bytes_req);
        if (st) return st;
    }
    if ((uint64_t)num_vars * (uint64_t)(2 * c->L) >= 0xFFFFFFFFull)
        return fail(c, GRG_E_RANGE, "numVars x 2 x numLabels must stay below 2^32");
    c->V = num_vars;
    c->ntables = (uint64_t)c->L * num_vars;
    const uint64_t nt_all = (uint64_t)(2 * c->L) * num_vars;
    if (c->ntables_alloc != nt_all) {
        free_graph(c);
        GRG_CUDA(c, cudaMalloc(&c->desc, std::max<uint64_t>(nt_all, 1) * 8));
        GRG_CUDA(c, cudaMalloc(&c->cnt, std::max<uint64_t>(nt_all, 1) * 4));
        GRG_CUDA(c, cudaMalloc(&c->want, std::max<uint64_t>(nt_all, 1) * 4));
        GRG_CUDA(c, cudaMalloc(&c->grow, std::max<uint64_t>(nt_all, 1) * 4));
        c->ntables_alloc = nt_all;
    }
    cudaStream_t s = c->stream;
    GRG_CUDA(c, cudaMemsetAsync(c->desc, 0, nt_all * 8, s));
    GRG_CUDA(c, cudaMemsetAsync(c->cnt, 0, nt_all * 4, s));
    GRG_CUDA(c, cudaMemsetAsync(c->want, 0, nt_all * 4, s));
    GRG_CUDA(c, cudaMemsetAsync(c->ctr, 0, sizeof(unsigned long long) * NCTR, s));
    const uint32_t *dsrc = src, *ddst = dst;
    const uint8_t *dlab = label;
    if (!on_device && num_edges) {
        if (c->in_cap < num_edges) {
            cudaFree(c->d_in32); cudaFree(c->d_in8);
            c->d_in32 = nullptr; c->d_in8 = nullptr;
            GRG_CUDA(c, cudaMalloc(&c->d_in32, num_edges * 8));
            GRG_CUDA(c, cudaMalloc(&c->d_in8, num_edges));
            c->in_cap = num_edges;
        }
        GRG_CUDA(c, cudaMemcpyAsync(c->d_in32, src, num_edges * 4, cudaMemcpyHostToDevice, s));
        GRG_CUDA(c, cudaMemcpyAsync(c->d_in32 + num_edges, dst, num_edges * 4, cudaMemcpyHostToDevice, s));
        GRG_CUDA(c, cudaMemcpyAsync(c->d_in8, label, num_edges, cudaMemcpyHostToDevice, s));
        dsrc = c->d_in32;
        ddst = c->d_in32 + num_edges;
        dlab = c->d_in8;
    }
    Dev d = make_dev(c);
    c->launches = 0;
    if (num_edges) {
        k_load_hist<<<grid_for(c, num_edges, 256), 256, 0, s>>>(d, dsrc, dlab, num_edges);
        c->launches++;
    }
    for (int q = 0; q < c->R; q++)
        if (c->rules[3 * q + 1] == 0) {
            k_eps_hist<<<grid_for(c, num_vars, 256), 256, 0, s>>>(d, (uint32_t)c->rules[3 * q]);
            c->launches++;
        }
    for (int attempt = 0;; attempt++) {
        GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_POOL_TOP, 0, 8, s));
        GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_ERR, 0, 8, s));
        k_load_alloc<<<grid_for(c, c->ntables, 256), 256, 0, s>>>(d, c->ntables);
        c->launches++;
        int st = read_ctr(c);
        if (st) return st;
        if (!(c->h_ctr[C_ERR] & ERR_POOL)) break;
        if (attempt > 8) return fail(c, GRG_E_NOMEM, "element pool too small for the input graph");
        // histogram was consumed: rebuild it after growing the pool
        st = grow_pool(c, c->h_ctr[C_POOL_TOP] + c->h_ctr[C_POOL_TOP] / 2);
        if (st) return st;
        d = make_dev(c);
        GRG_CUDA(c, cudaMemsetAsync(c->cnt, 0, nt_all * 4, s));
        if (num_edges) k_load_hist<<<grid_for(c, num_edges, 256), 256, 0, s>>>(d, dsrc, dlab, num_edges);
        for (int q = 0; q < c->R; q++)
            if (c->rules[3 * q + 1] == 0)
                k_eps_hist<<<grid_for(c, num_vars, 256), 256, 0, s>>>(d, (uint32_t)c->rules[3 * q]);
    }
    uint64_t top = c->h_ctr[C_POOL_TOP];
    if (top) {
        k_init_region<<<grid_for(c, top, 256), 256, 0, s>>>(c->elems, c->dbits, 0, top);
        c->launches++;
    }
    if (num_edges) {
        k_load_insert<<<grid_for(c, num_edges, 256), 256, 0, s>>>(d, dsrc, ddst, dlab, num_edges);
        c->launches++;
    }
    for (int q = 0; q < c->R; q++)
        if (c->rules[3 * q + 1] == 0) {
            k_eps_insert<<<grid_for(c, num_vars, 256), 256, 0, s>>>(d, (uint32_t)c->rules[3 * q]);
            c->launches++;
        }
    GRG_CUDA(c, cudaGetLastError());
    int st = read_ctr(c);
    if (st) return st;
    if (c->h_ctr[C_ERR]) return fail(c, GRG_E_CUDA, "internal error while loading edges");
    c->loaded = true;
    c->closed = false;
    return GRG_OK;
}

int grg_closure(grg_ctx *c, uint32_t filter, grg_stats *stats)
{
    if (!c || filter > 1) return GRG_E_ARG;
    if (!c->loaded) return fail(c, GRG_E_STATE, "grg_load_edges must come first");
    if (c->closed) return fail(c, GRG_E_STATE, "closure already computed; reload the graph");
    cudaSetDevice(c->device);
    RuleTable rt;
    int st = build_rules(c, filter, rt);
    if (st) return st;
    c->rt = rt;
    cudaStream_t s = c->stream;
    GRG_CUDA(c, cudaMemcpyToSymbolAsync(c_rt, &rt, sizeof rt, 0, cudaMemcpyHostToDevice, s));
    grg_stats S;
    memset(&S, 0, sizeof S);
    GRG_CUDA(c, cudaEventRecord(c->ev_a, s));
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
            k_compact_static<<<grid_for(c, c->V, 256), 256, 0, s>>>(d, (uint32_t)l);
            c->launches++;
        }
    st = read_ctr(c);
    if (st) return st;
    const uint64_t top = c->h_ctr[C_POOL_TOP];
    GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_DIRTY_N, 0, 8, s));
    if (top) {
        k_mark_all<<<grid_for(c, top, 256), 256, 0, s>>>(d, top);
        c->launches++;
    }
    double join_ms = 0;
    uint64_t joins = 0;
    for (;;) {
        st = read_ctr(c);
        if (st) return st;
        const uint64_t nd = c->h_ctr[C_DIRTY_N];
        if (nd == 0) break;
        st = ensure_delta(c, nd);
        if (st) return st;
        S.rounds++;
        S.delta_elems += nd;
        k_gather<<<grid_for(c, nd, 256), 256, 0, s>>>(d, nd, c->delta);
        c->launches++;
        GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_DIRTY_N, 0, 8, s));
        GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_RETRY_N, 0, 16, s));   // retry + grow counters
        const uint32_t *idx = nullptr;
        uint64_t n = nd;
        int rb = 0;
        for (int pass = 0;; pass++) {
            const int jgrid = grid_for(c, n, JOIN_WARPS, 16);
            if (c->timing) GRG_CUDA(c, cudaEventRecord(c->ev_c, s));
            k_join<<<jgrid, JOIN_WARPS * 32, 0, s>>>(d, c->delta, n, idx, c->retry[rb]);
            c->launches++;
            joins++;
            if (c->timing) GRG_CUDA(c, cudaEventRecord(c->ev_d, s));
            GRG_CUDA(c, cudaGetLastError());
            st = read_ctr(c);
            if (st) return st;
            if (c->timing) {
                float ms = 0;
                cudaEventElapsedTime(&ms, c->ev_c, c->ev_d);
                join_ms += ms;
            }
            const uint64_t nr = c->h_ctr[C_RETRY_N];
            if (nr == 0) break;
            S.retry_records += nr;
            // grow every table that overflowed, then re-run the failed records
            for (int gtry = 0;; gtry++) {
                const uint64_t ng = c->h_ctr[C_GROW_N];
                GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_ERR, 0, 8, s));
                k_grow<<<grid_for(c, ng * 32, 256), 256, 0, s>>>(d, ng);
                c->launches++;
                S.grow_rows += ng;
                st = read_ctr(c);
                if (st) return st;
                if (!(c->h_ctr[C_ERR] & ERR_POOL)) break;
                if (gtry > 16) return fail(c, GRG_E_NOMEM, "element pool exhausted");
                st = grow_pool(c, c->pool_cap * 2);
                if (st) return st;
                d = make_dev(c);
            }
            if (pass > 64) return fail(c, GRG_E_CUDA, "table growth did not converge");
            idx = c->retry[rb];
            n = nr;
            rb ^= 1;
            GRG_CUDA(c, cudaMemsetAsync(c->ctr + C_RETRY_N, 0, 16, s));
        }
    }
    GRG_CUDA(c, cudaEventRecord(c->ev_b, s));
    GRG_CUDA(c, cudaEventSynchronize(c->ev_b));
    float ms = 0;
    cudaEventElapsedTime(&ms, c->ev_a, c->ev_b);
    S.closure_ms = ms;
    S.join_ms = join_ms;
    S.join_launches = joins;
    S.left_elems = c->h_ctr[C_LEFT];
    S.right_elems = c->h_ctr[C_RIGHT];
    S.out_elems = S.delta_elems;
    S.pool_elems_used = c->h_ctr[C_POOL_TOP];
    S.pool_elems_cap = c->pool_cap;
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
        k_count<<<grid_for(c, (uint64_t)c->V * 32, 256), 256, 0, s>>>(d, (uint32_t)l, deg_e, deg_el, first, last, do_hash);
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

int grg_get_degree(grg_ctx *c, uint32_t first_var, uint32_t last_var, uint32_t *degree)
{
    if (!c || !degree || last_var < first_var) return GRG_E_ARG;
    if (!c->loaded) return fail(c, GRG_E_STATE, "no graph loaded");
    if (last_var >= c->V) return fail(c, GRG_E_RANGE, "vertex range beyond numVars");
    cudaSetDevice(c->device);
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
        k_export<<<grid_for(c, c->V, 256), 256, 0, s>>>(d, (uint32_t)l, d32, d32 ? d32 + cap : nullptr, d8, cap);
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

// Rule table for the allocation-free path (same rules as build_rules, without a context).
static int noalloc_rules(const int *rules, int R, int L, uint32_t filter, RuleTable &rt, bool *derivable)
{
    memset(&rt, 0, sizeof rt);
    rt.L = L;
    for (int l = 0; l <= MAX_LABELS; l++) derivable[l] = false;
    for (int q = 0; q < R; q++) {
        const int *r = &rules[3 * q];
        const bool unary = r[1] && !r[2];
        if (!(filter && unary)) derivable[r[0]] = true;
    }
    bool need_ol[GRG_MAX_RULES] = {false};
    for (int q = 0; q < R; q++) {
        const int *r = &rules[3 * q];
        if (r[1] && r[2] && derivable[r[2]]) {
            if (filter) return GRG_E_FILTER;
            need_ol[q] = true;
        }
    }
    int next_rev = L + 1;
    for (int q = 0; q < R; q++)
        if (need_ol[q] && !rt.rev_slot[rules[3 * q + 1]]) rt.rev_slot[rules[3 * q + 1]] = (uint8_t)next_rev++;
    rt.num_slots = next_rev - 1;
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
    k = 0;
    for (int C = 1; C <= L + 1; C++) {
        rt.ol_start[C] = (uint8_t)k;
        if (C > L) break;
        for (int q = 0; q < R; q++)
            if (need_ol[q] && rules[3 * q + 2] == C) {
                rt.ol_A[k] = (uint8_t)rules[3 * q];
                rt.ol_rev[k] = rt.rev_slot[rules[3 * q + 1]];
                k++;
            }
    }
    for (int q = 0; q < R; q++) {
        const int *r = &rules[3 * q];
        const bool unary = r[1] && !r[2];
        if (r[1] && !(filter && unary)) rt.track[r[1]] = 1;
        if (need_ol[q]) rt.track[r[2]] = 1;
    }
    return GRG_OK;
}

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
    // scratch layout: counters | descriptors | cnt | want | grow | pool arrays (108 B per element)
    const uint64_t ntab = (uint64_t)(2 * num_labels) * num_vars;
    size_t off = 0;
    const size_t o_ctr = off; off = align256(off + sizeof(unsigned long long) * NCTR);
    const size_t o_desc = off; off = align256(off + ntab * 8);
    const size_t o_cnt = off; off = align256(off + ntab * 4);
    const size_t o_want = off; off = align256(off + ntab * 4);
    const size_t o_grow = off; off = align256(off + ntab * 4);
    if (off >= NOALLOC_SCRATCH_BYTES) return GRG_E_RANGE;            // tables alone exceed the scratch
    uint64_t pool = (NOALLOC_SCRATCH_BYTES - off - 6 * 256) / 108;
    if (pool < 4096 || num_edges > pool / 2) return GRG_E_RANGE;    // graph too large for the scratch
    const size_t o_elems = off; off = align256(off + pool * 32);
    const size_t o_dbits = off; off = align256(off + pool * 32);
    const size_t o_dirty = off; off = align256(off + pool * 4);
    const size_t o_delta = off; off = align256(off + pool * 32);
    const size_t o_retry0 = off; off = align256(off + pool * 4);
    const size_t o_retry1 = off; off = align256(off + pool * 4);
    if (off > NOALLOC_SCRATCH_BYTES) return GRG_E_RANGE;

    RuleTable rt;
    bool derivable[MAX_LABELS + 1];
    int st = noalloc_rules(rules, num_rules, num_labels, filter, rt, derivable);
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
    d.dirty = (uint32_t *)(base + o_dirty);
    d.V = num_vars;
    d.pool_cap = (uint32_t)pool;
    uint4 *delta = (uint4 *)(base + o_delta);
    uint32_t *retry[2] = {(uint32_t *)(base + o_retry0), (uint32_t *)(base + o_retry1)};
    unsigned long long h[NCTR];

    // the array keeps the previous call's contents: clear everything that must start at zero
    NA_CUDA(cudaMemsetAsync(d.ctr, 0, sizeof(unsigned long long) * NCTR, s));
    NA_CUDA(cudaMemsetAsync(d.desc, 0, ntab * 8, s));
    NA_CUDA(cudaMemsetAsync(d.cnt, 0, ntab * 4, s));
    NA_CUDA(cudaMemsetAsync(d.want, 0, ntab * 4, s));
    NA_CUDA(cudaMemcpyToSymbolAsync(c_rt, &rt, sizeof rt, 0, cudaMemcpyHostToDevice, s));

    // load (grg_load_edges)
    const uint64_t nlab = (uint64_t)num_labels * num_vars;
    if (num_edges) k_load_hist<<<grid(num_edges, 256, 8), 256, 0, s>>>(d, d_src, d_label, num_edges);
    for (int q = 0; q < num_rules; q++)
        if (rules[3 * q + 1] == 0) k_eps_hist<<<grid(num_vars, 256, 8), 256, 0, s>>>(d, (uint32_t)rules[3 * q]);
    k_load_alloc<<<grid(nlab, 256, 8), 256, 0, s>>>(d, nlab);
    if ((st = na_read(h, d.ctr, s))) return st;
    if (h[C_ERR] & ERR_POOL) return GRG_E_NOMEM;
    const uint64_t top0 = h[C_POOL_TOP];
    if (top0) k_init_region<<<grid(top0, 256, 8), 256, 0, s>>>(d.elems, d.dbits, 0, top0);
    if (num_edges) k_load_insert<<<grid(num_edges, 256, 8), 256, 0, s>>>(d, d_src, d_dst, d_label, num_edges);
    for (int q = 0; q < num_rules; q++)
        if (rules[3 * q + 1] == 0) k_eps_insert<<<grid(num_vars, 256, 8), 256, 0, s>>>(d, (uint32_t)rules[3 * q]);
    for (int l = 1; l <= num_labels; l++)
        if (!derivable[l]) k_compact_static<<<grid(num_vars, 256, 8), 256, 0, s>>>(d, (uint32_t)l);
    if (top0) k_mark_all<<<grid(top0, 256, 8), 256, 0, s>>>(d, top0);
    NA_CUDA(cudaGetLastError());
    if ((st = na_read(h, d.ctr, s))) return st;
    if (h[C_ERR]) return GRG_E_CUDA;

    // semi-naive rounds (grg_closure); the pool cannot grow here
    uint64_t rounds = 0;
    for (;;) {
        if ((st = na_read(h, d.ctr, s))) return st;
        const uint64_t nd = h[C_DIRTY_N];
        if (nd == 0) break;
        rounds++;
        k_gather<<<grid(nd, 256, 8), 256, 0, s>>>(d, nd, delta);
        NA_CUDA(cudaMemsetAsync(d.ctr + C_DIRTY_N, 0, 8, s));
        NA_CUDA(cudaMemsetAsync(d.ctr + C_RETRY_N, 0, 16, s));
        const uint32_t *idx = nullptr;
        uint64_t n = nd;
        int rb = 0;
        for (int pass = 0;; pass++) {
            k_join<<<grid(n, JOIN_WARPS, 16), JOIN_WARPS * 32, 0, s>>>(d, delta, n, idx, retry[rb]);
            NA_CUDA(cudaGetLastError());
            if ((st = na_read(h, d.ctr, s))) return st;
            const uint64_t nr = h[C_RETRY_N];
            if (nr == 0) break;
            NA_CUDA(cudaMemsetAsync(d.ctr + C_ERR, 0, 8, s));
            k_grow<<<grid(h[C_GROW_N] * 32, 256, 8), 256, 0, s>>>(d, h[C_GROW_N]);
            if ((st = na_read(h, d.ctr, s))) return st;
            if (h[C_ERR] & ERR_POOL) return GRG_E_NOMEM;          // closure outgrew the scratch
            if (pass > 64) return GRG_E_CUDA;
            idx = retry[rb];
            n = nr;
            rb ^= 1;
            NA_CUDA(cudaMemsetAsync(d.ctr + C_RETRY_N, 0, 16, s));
        }
    }

    // per-label counts and edge-set hash into the caller's device buffers
    NA_CUDA(cudaMemsetAsync(d.ctr + C_LABEL0, 0, sizeof(unsigned long long) * (MAX_SLOTS + 2), s));
    NA_CUDA(cudaMemsetAsync(d.ctr + C_HASH, 0, 8, s));
    for (int l = 1; l <= num_labels; l++)
        k_count<<<grid((uint64_t)num_vars * 32, 256, 8), 256, 0, s>>>(d, (uint32_t)l, nullptr, nullptr, 0, 0,
                                                                     d_set_hash ? 1 : 0);
    NA_CUDA(cudaMemcpyAsync(d_label_counts, d.ctr + C_LABEL0 + 1, sizeof(uint64_t) * num_labels,
                            cudaMemcpyDeviceToDevice, s));
    if (d_set_hash) NA_CUDA(cudaMemcpyAsync(d_set_hash, d.ctr + C_HASH, 8, cudaMemcpyDeviceToDevice, s));
    NA_CUDA(cudaGetLastError());
    NA_CUDA(cudaStreamSynchronize(s));
    if (rounds_out) *rounds_out = rounds;
    return GRG_OK;
}
