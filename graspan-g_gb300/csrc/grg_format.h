// grg_format.h -- device conversions between element records and the
// reference's compressed edge stream (5 bytes per edge: little-endian uint32
// destination, then the uint8 label id; rows back to back, each row's edges by
// label, then destination). Internal to libgrg: the C ABI entry points are
// grg_export_csr5 / grg_load_csr5 in grg_engine.cu.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

// Stream of the n element records rec (8 words each: bitmap words 0-5, word 6 =
// label << 25 | base, word 7 = source row; any order) whose rows lie in
// [v_begin, v_begin + nrows). Writes the stream (total_edges x 5 bytes) to
// out_bytes and each row's edge count to degree (nrows entries, device memory).
// total_edges must be the records' popcount (cudaErrorInvalidValue, nothing
// written, otherwise). Temporary device memory is
// allocated and freed here; the call returns when the stream is complete.
cudaError_t grg_fmt_records_to_csr5(const uint4 *rec, uint64_t n, uint32_t v_begin, uint32_t nrows,
                                    uint64_t total_edges, uint8_t *out_bytes, uint32_t *degree, cudaStream_t s);

// Element records of a stream of num_edges edges for rows [v_begin, v_begin +
// nrows) with row lengths degree (device memory): consecutive edges of a row
// with the same label and 192-id base form one record (8 words: bitmap words
// 0-5, label << 25 | base, source row), each with stamp 1. *sum = the sum of
// degree; nothing else is done unless it equals num_edges. *bad = 1 (a label
// outside 1..L) | 2 (a destination >= num_vars); nothing is built then.
// Otherwise *n_elems = the number of records, and where they go depends on the
// outputs given:
//   into != null: written to into / into_st (room for into_cap records;
//                 cudaErrorInvalidValue, nothing written, when they do not fit);
//   recs != null: *recs / *stamps = new device arrays of *n_elems entries that
//                 the caller frees with cudaFree;
//   neither:      only counted.
// Returns after the records are complete.
cudaError_t grg_fmt_csr5_to_records(const uint8_t *bytes, uint64_t num_edges, const uint32_t *degree,
                                    uint32_t v_begin, uint32_t nrows, uint32_t num_vars, uint32_t L, uint4 *into,
                                    uint32_t *into_st, uint64_t into_cap, uint4 **recs, uint32_t **stamps,
                                    uint64_t *n_elems, uint64_t *sum, unsigned *bad, cudaStream_t s);

// Records of a graph whose labels in tmask (bit l-1 = label l) are stored by
// destination -- record (row j, label << 25 | base of the sources, bits over
// sources) -- turned into records by source: (row i, label << 25 | base of the
// destinations, bits over destinations). Records of other labels are copied as
// they are. *out is a new device array of *n_out records (the caller frees it
// with cudaFree). Returns after it is complete.
cudaError_t grg_fmt_columns_to_rows(const uint4 *rec, uint64_t n, uint64_t tmask, uint4 **out, uint64_t *n_out,
                                    cudaStream_t s);
