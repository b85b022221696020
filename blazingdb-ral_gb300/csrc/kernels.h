// kernels.h — launchers of the ahead-of-time kernels in kernels.cu.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace ral {

// Adds the number of set bits among the first n bits of `valid` to *out.
cudaError_t launch_count_valid(const uint32_t* valid, int64_t n, unsigned long long* out, cudaStream_t st);

// out[i] = in[idx[i]] for 0 <= idx[i] < n_in (elements of `width` bytes,
// indices of `idx_width` bytes; other indices leave out[i] untouched);
// out_valid (optional) gets bit i = in bit idx[i] (0 for an index outside
// [0, n_in), 1 when in_valid is null); valid_count (optional) gets the number
// of set output bits added.
cudaError_t launch_gather(int width, const void* in, const uint32_t* in_valid, int64_t n_in, const void* idx,
                          int idx_width, int64_t n_out, void* out, uint32_t* out_valid, unsigned long long* valid_count,
                          cudaStream_t st);

// ---- many columns gathered by one index column (joins, order-by) ----------------------------

constexpr int kMaxGatherColumns = 64;

struct GatherColumn {
    const void* in;            // n_in elements of `width` bytes
    const uint32_t* in_valid;  // optional
    void* out;                 // n_out elements
    uint32_t* out_valid;       // optional: bit i = in bit idx[i] (0 outside [0, n_in); 1 if in_valid is null)
    int32_t width;             // 1, 2, 4 or 8
    int32_t pad;
};

struct GatherColumnsParams {
    GatherColumn col[kMaxGatherColumns];
    const void* idx;
    int64_t n_in;
    int64_t n_out;
    unsigned long long* valid_counts;  // one counter per column with out_valid (zeroed), or null
    int32_t num_columns;
    int32_t idx_width;  // 1, 2, 4 or 8
};

// out_c[i] = in_c[idx[i]] for every column c, reading each index once; other indices leave
// out_c[i] untouched.  Output validity words are built by ballot, 32 rows at a time, and their
// set bits counted into valid_counts[c].
cudaError_t launch_gather_columns(const GatherColumnsParams& p, cudaStream_t st);

// ---- line index of a delimited text buffer (the text scan) ---------------------------------

// Each block handles kTextTileBytes bytes of the buffer: 16 steps of 256 threads x 16 bytes.
constexpr int64_t kTextStepBytes = 4096;
constexpr int64_t kTextTileBytes = 16 * kTextStepBytes;
inline int64_t text_tiles(int64_t n_bytes) { return (n_bytes + kTextTileBytes - 1) / kTextTileBytes; }

// counts[t] = line terminators in tile t of data[0, n).
cudaError_t launch_text_term_counts(const char* data, int64_t n, char term, uint32_t* counts, cudaStream_t st);
// offsets[t] = counts[0] + .. + counts[t-1] for t <= tiles (offsets[tiles] = the total), one block.
cudaError_t launch_exclusive_scan_u32(const uint32_t* counts, int64_t tiles, unsigned long long* offsets,
                                      cudaStream_t st);
// ends[k] = position of the k-th line terminator of data[0, n), in order.
cudaError_t launch_text_term_positions(const char* data, int64_t n, char term, const unsigned long long* offsets,
                                       long long* ends, cudaStream_t st);

// *count += lines i in [skip, lines) that are not blank (a '\r' before the terminator dropped);
// line i spans (ends[i - 1], ends[i]), the last one (i == nterm) ending at n.
cudaError_t launch_text_present_count(const char* data, int64_t n, const long long* ends, int64_t nterm, int64_t lines,
                                      int64_t skip, unsigned long long* count, cudaStream_t st);

// ---- Parquet data pages ------------------------------------------------------------------

// One uncompressed data page (v1 or v2) of a projected column, in memory the kernels read.
struct ParquetPage {
    int64_t row_start;      // the page's first row in the table
    int64_t data;           // device-visible address of the page's (uncompressed) data
    int64_t dict;           // dictionary-encoded pages: address of the chunk's dictionary (PLAIN values)
    int32_t rows;           // values in the page, nulls included
    int32_t data_bytes;     // the data's length
    int32_t column;         // output column
    int32_t optional;       // definition levels (bit width 1, RLE / bit-packed hybrid) come first
    int32_t lev_off;        // optional pages: offset of the level runs in the data (v1 4, v2 0)
    int32_t levels;         // optional pages: bytes of the level runs (-1: read from the data's first 4 bytes)
    int32_t values_off;     // offset of the values: PLAIN values, or the bit width and the indices
    int32_t item0;          // the page's first item (kParquetItemRows rows of a page per item)
    int32_t dict_count;     // entries of the dictionary; 0: PLAIN values
    int32_t idx0;           // dictionary-encoded pages: first slot of their indices in idx
};
struct ParquetColumnOut {
    void* data;             // rows x width
    uint32_t* valid;        // zeroed; bit r = value present
    int32_t width;
    int32_t pad;
};
constexpr int kParquetMaxColumns = 64;
constexpr int kParquetItemRows = 8192;
struct ParquetDecodeParams {
    ParquetPage* pages;
    ParquetColumnOut out[kParquetMaxColumns];
    unsigned long long* status;  // [0] malformed pages (levels, indices or values past their data), [1..] valid counts
    uint32_t* item_base;         // per item of an optional page: its page's present rows before it (zeroed)
    uint32_t* page_present;      // per page: present rows (written for optional pages by the levels kernel)
    uint32_t* idx;               // dictionary indices of the present rows of dictionary-encoded pages
    int32_t page_lo, page_hi;    // the pages of this launch
    int32_t item_lo, item_hi;    // their items
};
// One Snappy-compressed page body (a Parquet page of a SNAPPY column chunk): `prefix` raw bytes
// (a v2 page's levels, stored uncompressed before the values) are copied from src - prefix, then
// the raw Snappy stream src[0, src_bytes) is decompressed after them; its length must be dst_bytes.
struct SnappyJob {
    const uint8_t* src;
    uint8_t* dst;
    int32_t src_bytes;
    int32_t dst_bytes;
    int32_t prefix;
    int32_t pad;
};
// One warp per job; a malformed stream or a length mismatch adds one to *status.
cudaError_t launch_snappy_decompress(const SnappyJob* jobs, int32_t n_jobs, unsigned long long* status, cudaStream_t st);

// Byte copies gathered into one launch (one block per job): small pieces of a page-locked file
// (dictionaries) brought into device memory.
struct CopyJob {
    const uint8_t* src;
    uint8_t* dst;
    int64_t bytes;
};
cudaError_t launch_copy_jobs(const CopyJob* jobs, int32_t n_jobs, cudaStream_t st);

// Pages of [page_lo, page_hi) whose level length is -1 (Snappy v1 pages): the length from the
// first 4 bytes of their decompressed data, and their values' offset after it.
cudaError_t launch_parquet_level_lengths(const ParquetDecodeParams& p, cudaStream_t st);
// Optional pages of [page_lo, page_hi): validity bits from the definition levels, each item's
// first value index in item_base, the present rows in status[1 + column].
cudaError_t launch_parquet_levels(const ParquetDecodeParams& p, cudaStream_t st);
// Dictionary-encoded pages of [page_lo, page_hi): the index of every present row (RLE / bit-packed
// hybrid of the page's bit width) into idx, checked against the dictionary's size.  After
// launch_parquet_levels for optional pages.
cudaError_t launch_parquet_dict_indices(const ParquetDecodeParams& p, cudaStream_t st);
// Items [item_lo, item_hi): values of the present rows in row order (null rows 0).  Optional
// pages' levels and dictionary pages' indices must have been decoded by the launches above.
cudaError_t launch_parquet_values(const ParquetDecodeParams& p, cudaStream_t st);

// codes[i] += 1 where codes[i] >= pos: a string inserted at rank pos of a category dictionary.
cudaError_t launch_category_insert(int32_t* codes, int64_t n, int32_t pos, cudaStream_t st);
// codes[i] = table[codes[i]] for codes in [0, table_n): codes moved to a merged dictionary.
cudaError_t launch_category_remap(int32_t* codes, int64_t n, const int32_t* table, int32_t table_n, cudaStream_t st);

}  // namespace ral

namespace ral {

// Scratch layout of the single-pass compaction (one zeroed block per call):
//   word 0: tile ticket counter, word 1: error flag (1 = a look-back wait gave up),
//   word 2: kept-row total, words 3.. : one status word per tile.
constexpr int64_t kCompactTileRows = 4096;  // 256 threads x 16 rows
inline int64_t compact_scratch_words(int64_t n) { return 3 + (n + kCompactTileRows - 1) / kCompactTileRows; }

// cudf::apply_boolean_mask over the row-index column (CalciteInterpreter.cpp:531-543):
// writes the indices of rows whose stencil byte is nonzero and whose stencil
// valid bit is set (stencil_valid may be null) to out_idx, in row order, and the
// count to scratch[2].  `scratch` must hold compact_scratch_words(n) zeroed words.
cudaError_t launch_compact_stencil(const int8_t* stencil, const uint32_t* stencil_valid, int64_t n, int32_t* out_idx,
                                   unsigned long long* scratch, cudaStream_t st);

}  // namespace ral
