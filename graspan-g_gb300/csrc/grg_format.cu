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
