// grg_format.cu -- the reference's compressed edge stream on the device.
//
// The reference spills partitions as a CSR byte stream (storeElements_c /
// elements2Edges, src/main.cpp:510-596) and reads them back with
// readElements_c / edges2Elements (src/main.cpp:335-445): per source vertex in
// order, per label 1..L, the row's destinations ascending, 5 bytes each
// (little-endian uint32 destination, uint8 label id), with the row lengths kept
// in a separate degree array. Here both directions run on the device:
//   records -> stream: sort the element records by (row, label, base) with a
//     64-bit radix sort, prefix-sum their popcounts into edge offsets, then
//     one thread per (element, bitmap word) writes its edges' bytes;
//   stream -> edges: prefix-sum the row lengths, then each thread expands a
//     run of 16 consecutive edges, finding its first row by binary search.
// Both are HBM-streaming passes over the records / the stream.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <vector>

#include "grg_format.h"

namespace {

constexpr uint32_t KEY_BITS = 32;          // word 6: label << 25 | base
constexpr uint32_t EIDS = 192;
constexpr uint32_t BASE_MASK = (1u << 25) - 1;
constexpr uint32_t EXPAND_RUN = 16;        // edges per thread in the expansion

int grid_of(uint64_t n, int block)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint64_t g = (n + block - 1) / block, cap = (uint64_t)(sms > 0 ? sms : 1) * 16;
    return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

__global__ void k_fmt_keys(const uint4 *__restrict__ rec, uint64_t n, uint32_t v_begin, uint64_t *key, uint32_t *idx)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint4 b = rec[2 * i + 1];
        key[i] = ((uint64_t)(b.w - v_begin) << KEY_BITS) | b.z;
        idx[i] = (uint32_t)i;
    }
}

__device__ __forceinline__ uint32_t popc6(uint4 a, uint4 b)
{
    return __popc(a.x) + __popc(a.y) + __popc(a.z) + __popc(a.w) + __popc(b.x) + __popc(b.y);
}

// Edge count of each sorted element (for the offsets) and of each row.
__global__ void k_fmt_count(const uint4 *__restrict__ rec, const uint32_t *__restrict__ idx, uint64_t n,
                            uint32_t v_begin, uint64_t *cnt, uint32_t *degree)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t j = idx[i];
        const uint4 a = rec[2 * j], b = rec[2 * j + 1];
        const uint32_t c = popc6(a, b);
        cnt[i] = c;
        if (c) atomicAdd(&degree[b.w - v_begin], c);
    }
}

// One thread per (sorted element, bitmap word): the word's ids ascending, 5 bytes each.
__global__ void k_fmt_write(const uint4 *__restrict__ rec, const uint32_t *__restrict__ idx,
                            const uint64_t *__restrict__ off, uint64_t n, uint8_t *out)
{
    const uint64_t total = n * 6;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total; t += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t i = t / 6;
        const uint32_t w = (uint32_t)(t - i * 6);
        const uint32_t j = idx[i];
        const uint4 a = rec[2 * j], b = rec[2 * j + 1];
        const uint32_t words[6] = {a.x, a.y, a.z, a.w, b.x, b.y};
        uint64_t o = off[i];
        for (uint32_t q = 0; q < w; q++) o += __popc(words[q]);
        uint32_t bits = words[w];
        const uint32_t lab = b.z >> 25, first = (b.z & BASE_MASK) * EIDS + w * 32;
        while (bits) {
            const uint32_t dst = first + (__ffs(bits) - 1);
            bits &= bits - 1;
            uint8_t *q = out + o * 5;
            q[0] = (uint8_t)dst;
            q[1] = (uint8_t)(dst >> 8);
            q[2] = (uint8_t)(dst >> 16);
            q[3] = (uint8_t)(dst >> 24);
            q[4] = (uint8_t)lab;
            o++;
        }
    }
}

// roff[r] = degree[r] widened (roff[nrows] = 0), for the exclusive scan.
__global__ void k_fmt_widen(const uint32_t *__restrict__ degree, uint32_t nrows, uint64_t *roff)
{
    for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r <= nrows; r += (uint64_t)gridDim.x * blockDim.x)
        roff[r] = r < nrows ? degree[r] : 0;
}

// Walks the EXPAND_RUN consecutive edges of run u: f(row, label, dst, starts)
// per edge, where `starts` says the edge begins a new element -- the first edge
// of a row, or one whose label or 192-id base differs from the edge before it
// (the stream is sorted by label, then destination, within a row). The run's
// first row is the last r with start[r] <= e0 (rows of length 0 share their
// start with the next row).
template <class F>
__device__ __forceinline__ void walk_run(const uint8_t *__restrict__ bytes, const uint64_t *__restrict__ start,
                                         uint32_t nrows, uint64_t m, uint64_t u, F f)
{
    const uint64_t e0 = u * EXPAND_RUN;
    uint32_t lo = 0, hi = nrows;                 // start[lo] <= e0 < start[hi]
    while (hi - lo > 1) {
        const uint32_t mid = lo + (hi - lo) / 2;
        if (start[mid] <= e0) lo = mid; else hi = mid;
    }
    uint32_t r = lo, plab = 0, pbase = 0;
    bool have_prev = false;
    if (e0 > start[r]) {                         // the edge before e0 is in the same row
        const uint8_t *q = bytes + (e0 - 1) * 5;
        plab = q[4];
        pbase = ((uint32_t)q[0] | ((uint32_t)q[1] << 8) | ((uint32_t)q[2] << 16) | ((uint32_t)q[3] << 24)) / EIDS;
        have_prev = true;
    }
    const uint64_t e1 = e0 + EXPAND_RUN < m ? e0 + EXPAND_RUN : m;
    for (uint64_t e = e0; e < e1; e++) {
        while (r + 1 < nrows && start[r + 1] <= e) {
            r++;
            have_prev = false;
        }
        const uint8_t *q = bytes + e * 5;
        const uint32_t dst = (uint32_t)q[0] | ((uint32_t)q[1] << 8) | ((uint32_t)q[2] << 16) | ((uint32_t)q[3] << 24);
        const uint32_t lab = q[4], base = dst / EIDS;
        f(r, lab, dst, !have_prev || lab != plab || base != pbase);
        have_prev = true;
        plab = lab;
        pbase = base;
    }
}

// Pass 1: elements starting in each run; labels outside 1..L and destinations
// >= num_vars set bits 1 and 2 of *bad.
__global__ void k_fmt_starts(const uint8_t *__restrict__ bytes, const uint64_t *__restrict__ start, uint32_t nrows,
                             uint64_t m, uint32_t num_vars, uint32_t L, uint64_t *run_cnt, unsigned *bad)
{
    const uint64_t runs = (m + EXPAND_RUN - 1) / EXPAND_RUN;
    for (uint64_t u = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; u < runs; u += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t c = 0;
        unsigned b = 0;
        walk_run(bytes, start, nrows, m, u, [&](uint32_t, uint32_t lab, uint32_t dst, bool starts) {
            if (lab - 1u >= L) b |= 1u;
            if (dst >= num_vars) b |= 2u;
            c += starts;
        });
        run_cnt[u] = c;
        if (b) atomicOr(bad, b);
    }
}

// Pass 2: ORs each edge's bit into its element (id = elements started before
// it); the element's first edge writes its key and row. Bits gather in
// registers while consecutive edges share an element.
__global__ void k_fmt_build(const uint8_t *__restrict__ bytes, const uint64_t *__restrict__ start, uint32_t nrows,
                            uint64_t m, uint32_t v_begin, const uint64_t *__restrict__ run_off, uint32_t *rec)
{
    const uint64_t runs = (m + EXPAND_RUN - 1) / EXPAND_RUN;
    for (uint64_t u = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; u < runs; u += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t id = run_off[u] - 1;            // the element the run's first edge continues, if it does
        uint32_t acc[6] = {0, 0, 0, 0, 0, 0};
        bool open = false;
        auto flush = [&]() {
            if (!open) return;
#pragma unroll
            for (int w = 0; w < 6; w++)
                if (acc[w]) atomicOr(&rec[id * 8 + w], acc[w]);
#pragma unroll
            for (int w = 0; w < 6; w++) acc[w] = 0;
        };
        walk_run(bytes, start, nrows, m, u, [&](uint32_t r, uint32_t lab, uint32_t dst, bool starts) {
            if (starts) {
                flush();
                id++;
                rec[id * 8 + 6] = (lab << 25) | (dst / EIDS);
                rec[id * 8 + 7] = v_begin + r;
            }
            open = true;
            const uint32_t o = dst % EIDS;
#pragma unroll
            for (int w = 0; w < 6; w++)
                if ((o >> 5) == (uint32_t)w) acc[w] |= 1u << (o & 31);
        });
        flush();
    }
}

__global__ void k_fmt_fill(uint32_t *p, uint64_t n, uint32_t v)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        p[i] = v;
}

int bit_width(uint64_t x)
{
    int b = 0;
    while (x) { b++; x >>= 1; }
    return b;
}

}  // namespace

#define FMT_CHECK(x)                      \
    do {                                  \
        cudaError_t e_ = (x);             \
        if (e_ != cudaSuccess) {          \
            err = e_;                     \
            goto done;                    \
        }                                 \
    } while (0)

cudaError_t grg_fmt_records_to_csr5(const uint4 *rec, uint64_t n, uint32_t v_begin, uint32_t nrows,
                                    uint64_t total_edges, uint8_t *out_bytes, uint32_t *degree, cudaStream_t s)
{
    cudaError_t err = cudaSuccess;
    uint64_t *key = nullptr, *cnt = nullptr;
    uint32_t *idx = nullptr;
    void *tmp = nullptr;
    size_t tsort = 0, tscan = 0;
    const int end_bit = (int)KEY_BITS + (nrows > 1 ? bit_width(nrows - 1) : 0);
    FMT_CHECK(cudaMemsetAsync(degree, 0, (size_t)nrows * 4, s));
    if (!n) return cudaStreamSynchronize(s);
    // key[0..n) / key[n..2n): radix sort input and output; idx the same; cnt then offsets
    FMT_CHECK(cudaMalloc(&key, n * 16));
    FMT_CHECK(cudaMalloc(&idx, n * 8));
    FMT_CHECK(cudaMalloc(&cnt, n * 16));
    FMT_CHECK(cub::DeviceRadixSort::SortPairs(nullptr, tsort, key, key + n, idx, idx + n, n, 0, end_bit, s));
    FMT_CHECK(cub::DeviceScan::ExclusiveSum(nullptr, tscan, cnt, cnt + n, n, s));
    FMT_CHECK(cudaMalloc(&tmp, tsort > tscan ? tsort : tscan));
    k_fmt_keys<<<grid_of(n, 256), 256, 0, s>>>(rec, n, v_begin, key, idx);
    FMT_CHECK(cub::DeviceRadixSort::SortPairs(tmp, tsort, key, key + n, idx, idx + n, n, 0, end_bit, s));
    k_fmt_count<<<grid_of(n, 256), 256, 0, s>>>(rec, idx + n, n, v_begin, cnt, degree);
    FMT_CHECK(cub::DeviceScan::ExclusiveSum(tmp, tscan, cnt, cnt + n, n, s));
    // the stream is written only when the records' popcount is the length the caller sized it for
    {
        uint64_t last[2] = {0, 0};
        FMT_CHECK(cudaMemcpyAsync(&last[0], cnt + n - 1, 8, cudaMemcpyDeviceToHost, s));
        FMT_CHECK(cudaMemcpyAsync(&last[1], cnt + 2 * n - 1, 8, cudaMemcpyDeviceToHost, s));
        FMT_CHECK(cudaStreamSynchronize(s));
        if (last[0] + last[1] != total_edges) {
            err = cudaErrorInvalidValue;
            goto done;
        }
    }
    if (total_edges) k_fmt_write<<<grid_of(n * 6, 256), 256, 0, s>>>(rec, idx + n, cnt + n, n, out_bytes);
    FMT_CHECK(cudaGetLastError());
    FMT_CHECK(cudaStreamSynchronize(s));
done:
    cudaFree(tmp);
    cudaFree(cnt);
    cudaFree(idx);
    cudaFree(key);
    return err;
}

cudaError_t grg_fmt_csr5_to_records(const uint8_t *bytes, uint64_t num_edges, const uint32_t *degree,
                                    uint32_t v_begin, uint32_t nrows, uint32_t num_vars, uint32_t L, uint4 *into,
                                    uint32_t *into_st, uint64_t into_cap, uint4 **recs, uint32_t **stamps,
                                    uint64_t *n_elems, uint64_t *sum, unsigned *bad, cudaStream_t s)
{
    cudaError_t err = cudaSuccess;
    uint64_t *roff = nullptr, *start = nullptr, *rcnt = nullptr, *roffs = nullptr;
    unsigned *dbad = nullptr;
    void *tmp = nullptr;
    size_t tscan = 0, tscan2 = 0;
    const uint64_t runs = (num_edges + EXPAND_RUN - 1) / EXPAND_RUN;
    uint32_t *rec = nullptr, *st = nullptr;
    if (recs) *recs = nullptr;
    if (stamps) *stamps = nullptr;
    *n_elems = 0;
    *sum = 0;
    *bad = 0;
    if (!nrows) return cudaSuccess;
    FMT_CHECK(cudaMalloc(&roff, ((uint64_t)nrows + 1) * 16));
    start = roff + nrows + 1;
    FMT_CHECK(cudaMalloc(&rcnt, (runs + 1) * 16 + 16));
    roffs = rcnt + runs + 1;
    dbad = (unsigned *)(roffs + runs + 1);
    FMT_CHECK(cub::DeviceScan::ExclusiveSum(nullptr, tscan, roff, start, (uint64_t)nrows + 1, s));
    FMT_CHECK(cub::DeviceScan::ExclusiveSum(nullptr, tscan2, rcnt, roffs, runs + 1, s));
    FMT_CHECK(cudaMalloc(&tmp, tscan > tscan2 ? tscan : tscan2));
    k_fmt_widen<<<grid_of((uint64_t)nrows + 1, 256), 256, 0, s>>>(degree, nrows, roff);
    FMT_CHECK(cub::DeviceScan::ExclusiveSum(tmp, tscan, roff, start, (uint64_t)nrows + 1, s));
    FMT_CHECK(cudaMemcpyAsync(sum, start + nrows, 8, cudaMemcpyDeviceToHost, s));
    FMT_CHECK(cudaStreamSynchronize(s));
    if (*sum != num_edges || !num_edges) goto done;
    FMT_CHECK(cudaMemsetAsync(rcnt, 0, (runs + 1) * 8, s));
    FMT_CHECK(cudaMemsetAsync(dbad, 0, 4, s));
    k_fmt_starts<<<grid_of(runs, 256), 256, 0, s>>>(bytes, start, nrows, num_edges, num_vars, L, rcnt, dbad);
    FMT_CHECK(cub::DeviceScan::ExclusiveSum(tmp, tscan2, rcnt, roffs, runs + 1, s));
    FMT_CHECK(cudaMemcpyAsync(bad, dbad, 4, cudaMemcpyDeviceToHost, s));
    FMT_CHECK(cudaMemcpyAsync(n_elems, roffs + runs, 8, cudaMemcpyDeviceToHost, s));
    FMT_CHECK(cudaStreamSynchronize(s));
    if (*bad || !*n_elems || (!into && !recs)) goto done;
    if (into) {
        if (*n_elems > into_cap) {
            err = cudaErrorInvalidValue;
            goto done;
        }
        rec = reinterpret_cast<uint32_t *>(into);
        st = into_st;
    } else {
        FMT_CHECK(cudaMalloc(&rec, *n_elems * 32));
        FMT_CHECK(cudaMalloc(&st, *n_elems * 4));
    }
    FMT_CHECK(cudaMemsetAsync(rec, 0, *n_elems * 32, s));
    k_fmt_fill<<<grid_of(*n_elems, 256), 256, 0, s>>>(st, *n_elems, 1u);
    // run u's edges belong to elements run_off[u] - 1 (continued) and run_off[u] .. run_off[u+1] - 1
    k_fmt_build<<<grid_of(runs, 256), 256, 0, s>>>(bytes, start, nrows, num_edges, v_begin, roffs, rec);
    FMT_CHECK(cudaGetLastError());
    FMT_CHECK(cudaStreamSynchronize(s));
    if (!into) {
        *recs = reinterpret_cast<uint4 *>(rec);
        *stamps = st;
    }
    rec = nullptr;
    st = nullptr;
done:
    if (!into) {
        cudaFree(rec);
        cudaFree(st);
    }
    cudaFree(tmp);
    cudaFree(rcnt);
    cudaFree(roff);
    return err;
}

// ------------------------------------------------------------------ columns -> rows
//
// Labels stored by destination keep, per (label, destination j), elements over
// the sources i. Their records are turned into records by source here, 192 x 192
// tiles at a time: the records of one label whose destinations share a 192-id
// block jb and whose source elements share a base ib form one tile (at most 192
// records, one per destination of the block); a warp loads the tile into shared
// memory and transposes it one 32 x 32 bit block at a time with warp ballots.

namespace {

constexpr int TILE_WARPS = 4;
constexpr uint64_t NOT_COLUMN = 1ull << 56;   // sort key of records that are copied as they are

__global__ void k_col_keys(const uint4 *__restrict__ rec, uint64_t n, unsigned long long tmask, uint64_t *key,
                           uint32_t *idx)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint4 b = rec[2 * i + 1];
        const uint32_t lab = b.z >> 25;
        const bool col = lab >= 1 && lab <= 63 && ((tmask >> (lab - 1)) & 1ull);
        key[i] = col ? ((uint64_t)lab << 50) | ((uint64_t)(b.w / EIDS) << 25) | (b.z & BASE_MASK) : NOT_COLUMN;
        idx[i] = (uint32_t)i;
    }
}

// head[i] = 1 where a tile starts among the first nt (column) sorted keys
__global__ void k_col_heads(const uint64_t *__restrict__ key, uint64_t nt, uint32_t *head)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nt; i += (uint64_t)gridDim.x * blockDim.x)
        head[i] = (i == 0 || key[i] != key[i - 1]) ? 1u : 0u;
}

__global__ void k_col_starts(const uint32_t *__restrict__ head, const uint32_t *__restrict__ pos, uint64_t nt,
                             uint32_t *start)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nt; i += (uint64_t)gridDim.x * blockDim.x)
        if (head[i]) start[pos[i]] = (uint32_t)i;
}

// One warp per tile. EMIT = false: cnt[t] = records the tile yields; true: they
// are written at off[t] (sources ascending within a tile).
template <bool EMIT>
__global__ void __launch_bounds__(TILE_WARPS * 32) k_col_tiles(const uint4 *__restrict__ rec, const uint64_t *__restrict__ key,
                                                            const uint32_t *__restrict__ idx,
                                                            const uint32_t *__restrict__ start, uint64_t ntiles,
                                                            uint64_t nt, uint32_t *cnt, const uint64_t *__restrict__ off,
                                                            uint4 *out)
{
    __shared__ uint32_t M[TILE_WARPS][EIDS][7];   // 7 words a row: conflict-free column reads
    const uint32_t w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint32_t(*m)[7] = M[w];
    for (uint64_t t = blockIdx.x * (uint64_t)TILE_WARPS + w; t < ntiles; t += (uint64_t)gridDim.x * TILE_WARPS) {
        const uint64_t a = start[t], z = t + 1 < ntiles ? start[t + 1] : nt;
        for (uint32_t u = lane; u < EIDS * 7; u += 32) (&m[0][0])[u] = 0;
        __syncwarp();
        const uint64_t k = key[a];
        const uint32_t lab = (uint32_t)(k >> 50), jb = (uint32_t)(k >> 25) & BASE_MASK, ib = (uint32_t)k & BASE_MASK;
        for (uint64_t r = a + lane; r < z; r += 32) {
            const uint32_t j = idx[r];
            const uint4 e0 = rec[2 * j], e1 = rec[2 * j + 1];
            const uint32_t jo = e1.w - jb * EIDS;      // < 192: the tile's destinations share block jb
            if (jo < EIDS) {
                m[jo][0] = e0.x; m[jo][1] = e0.y; m[jo][2] = e0.z; m[jo][3] = e0.w; m[jo][4] = e1.x; m[jo][5] = e1.y;
            }
        }
        __syncwarp();
        uint64_t made = 0;
        for (int iw = 0; iw < 6; iw++) {
            uint32_t o[6];
#pragma unroll
            for (int jw = 0; jw < 6; jw++) {
                const uint32_t v = m[jw * 32 + lane][iw];   // lane = destination jw*32+lane, bits over 32 sources
                uint32_t res = 0;
                if (__any_sync(0xffffffffu, v != 0)) {
#pragma unroll 4
                    for (int b = 0; b < 32; b++) {
                        const uint32_t col = __ballot_sync(0xffffffffu, (v >> b) & 1u);
                        if ((int)lane == b) res = col;   // source iw*32+b: its destinations in word jw
                    }
                }
                o[jw] = res;
            }
            const bool any = (o[0] | o[1] | o[2] | o[3] | o[4] | o[5]) != 0;
            const unsigned msk = __ballot_sync(0xffffffffu, any);
            if (EMIT && any) {
                const uint64_t p = off[t] + made + __popc(msk & ((1u << lane) - 1u));
                out[2 * p] = make_uint4(o[0], o[1], o[2], o[3]);
                out[2 * p + 1] = make_uint4(o[4], o[5], (lab << 25) | jb, ib * EIDS + iw * 32 + lane);
            }
            made += __popc(msk);
        }
        if (!EMIT && lane == 0) cnt[t] = (uint32_t)made;
        __syncwarp();
    }
}

// sorted records [from, n) copied as they are to out[dst0 + (i - from)]
__global__ void k_col_copy(const uint4 *__restrict__ rec, const uint32_t *__restrict__ idx, uint64_t from, uint64_t n,
                           uint4 *out, uint64_t dst0)
{
    for (uint64_t i = from + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t j = idx[i];
        const uint64_t o = dst0 + (i - from);
        out[2 * o] = rec[2 * j];
        out[2 * o + 1] = rec[2 * j + 1];
    }
}

__global__ void k_widen32(const uint32_t *in, uint64_t n, uint64_t *out)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = in[i];
}

}  // namespace

cudaError_t grg_fmt_columns_to_rows(const uint4 *rec, uint64_t n, uint64_t tmask, uint4 **out, uint64_t *n_out,
                                    cudaStream_t s)
{
    cudaError_t err = cudaSuccess;
    uint64_t *key = nullptr, *toff = nullptr;
    uint32_t *idx = nullptr, *head = nullptr, *tcnt = nullptr;
    void *tmp = nullptr;
    uint4 *res = nullptr;
    size_t tsort = 0, tscan = 0, tscan2 = 0;
    uint64_t nt = 0, ntiles = 0, made = 0;
    *out = nullptr;
    *n_out = 0;
    if (!n) return cudaSuccess;
    FMT_CHECK(cudaMalloc(&key, n * 16));
    FMT_CHECK(cudaMalloc(&idx, n * 8));
    FMT_CHECK(cub::DeviceRadixSort::SortPairs(nullptr, tsort, key, key + n, idx, idx + n, n, 0, 57, s));
    FMT_CHECK(cub::DeviceScan::ExclusiveSum(nullptr, tscan, idx, idx, n + 1, s));
    FMT_CHECK(cub::DeviceScan::ExclusiveSum(nullptr, tscan2, key, key, n + 1, s));
    if (tscan2 > tscan) tscan = tscan2;
    FMT_CHECK(cudaMalloc(&tmp, tsort > tscan ? tsort : tscan));
    k_col_keys<<<grid_of(n, 256), 256, 0, s>>>(rec, n, tmask, key, idx);
    FMT_CHECK(cub::DeviceRadixSort::SortPairs(tmp, tsort, key, key + n, idx, idx + n, n, 0, 57, s));
    {
        // column records come first; nt = their number (the first key >= NOT_COLUMN)
        uint64_t lo = 0, hi = n;
        std::vector<uint64_t> probe(1);
        while (lo < hi) {          // binary search on the sorted keys, one 8-byte read a step
            const uint64_t mid = (lo + hi) / 2;
            FMT_CHECK(cudaMemcpyAsync(probe.data(), key + n + mid, 8, cudaMemcpyDeviceToHost, s));
            FMT_CHECK(cudaStreamSynchronize(s));
            if (probe[0] >= NOT_COLUMN) hi = mid; else lo = mid + 1;
        }
        nt = lo;
    }
    if (nt) {
        // tile starts: heads -> their positions -> start[]
        FMT_CHECK(cudaMalloc(&head, (nt + 1) * 12));
        uint32_t *pos = head + nt + 1, *start = pos + nt + 1;
        FMT_CHECK(cudaMemsetAsync(head + nt, 0, 4, s));
        k_col_heads<<<grid_of(nt, 256), 256, 0, s>>>(key + n, nt, head);
        FMT_CHECK(cub::DeviceScan::ExclusiveSum(tmp, tscan, head, pos, nt + 1, s));
        uint32_t nt32 = 0;
        FMT_CHECK(cudaMemcpyAsync(&nt32, pos + nt, 4, cudaMemcpyDeviceToHost, s));
        FMT_CHECK(cudaStreamSynchronize(s));
        ntiles = nt32;
        k_col_starts<<<grid_of(nt, 256), 256, 0, s>>>(head, pos, nt, start);
        // records per tile, their offsets, then the records
        FMT_CHECK(cudaMalloc(&tcnt, (ntiles + 1) * 4));
        FMT_CHECK(cudaMalloc(&toff, (ntiles + 1) * 16));
        FMT_CHECK(cudaMemsetAsync(tcnt + ntiles, 0, 4, s));
        const int tg = grid_of((ntiles + TILE_WARPS - 1) / TILE_WARPS, 1);
        k_col_tiles<false><<<tg, TILE_WARPS * 32, 0, s>>>(rec, key + n, idx + n, start, ntiles, nt, tcnt, nullptr,
                                                           nullptr);
        k_widen32<<<grid_of(ntiles + 1, 256), 256, 0, s>>>(tcnt, ntiles + 1, toff + ntiles + 1);
        FMT_CHECK(cub::DeviceScan::ExclusiveSum(tmp, tscan, toff + ntiles + 1, toff, ntiles + 1, s));
        FMT_CHECK(cudaMemcpyAsync(&made, toff + ntiles, 8, cudaMemcpyDeviceToHost, s));
        FMT_CHECK(cudaStreamSynchronize(s));
        FMT_CHECK(cudaMalloc(&res, (made + (n - nt)) * 32 + 32));
        k_col_tiles<true><<<tg, TILE_WARPS * 32, 0, s>>>(rec, key + n, idx + n, start, ntiles, nt, nullptr, toff, res);
    } else {
        FMT_CHECK(cudaMalloc(&res, n * 32 + 32));
    }
    // records stored by source follow, as they are (out index made + (i - nt))
    if (n > nt) k_col_copy<<<grid_of(n - nt, 256), 256, 0, s>>>(rec, idx + n, nt, n, res, made);
    FMT_CHECK(cudaGetLastError());
    FMT_CHECK(cudaStreamSynchronize(s));
    *out = res;
    *n_out = made + (n - nt);
    res = nullptr;
done:
    cudaFree(res);
    cudaFree(toff);
    cudaFree(tcnt);
    cudaFree(head);
    cudaFree(tmp);
    cudaFree(idx);
    cudaFree(key);
    return err;
}
