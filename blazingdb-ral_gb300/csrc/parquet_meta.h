// parquet_meta.h — the parts of a Parquet file's metadata the scan reads (Apache Parquet format:
// a footer and page headers in Thrift's compact protocol), parsed on the host.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace ral {
namespace pq {

struct ColumnChunkMeta {
    int32_t type = -1;             // physical type: 1 INT32, 2 INT64, 4 FLOAT, 5 DOUBLE, ...
    int32_t codec = 0;             // 0 UNCOMPRESSED
    int64_t num_values = 0;
    int64_t data_page_offset = -1;
    int64_t dictionary_page_offset = -1;
    int64_t total_compressed_size = 0;
};

struct RowGroupMeta {
    int64_t num_rows = 0;
    std::vector<ColumnChunkMeta> columns;
};

struct SchemaLeaf {
    std::string name;
    int32_t type = -1;
    int32_t repetition = 0;        // 0 REQUIRED, 1 OPTIONAL, 2 REPEATED
    int32_t converted_type = -1;   // 6 DATE, 9 TIMESTAMP_MILLIS, ...
};

struct FileMeta {
    int64_t num_rows = 0;
    std::vector<SchemaLeaf> leaves;  // the root's children, in order
    std::vector<RowGroupMeta> row_groups;
};

struct PageHeader {
    int32_t type = -1;             // 0 DATA_PAGE, 2 DICTIONARY_PAGE, 3 DATA_PAGE_V2
    int32_t uncompressed_size = 0;
    int32_t compressed_size = 0;
    int32_t num_values = 0;        // data pages: values (nulls included); dictionary pages: entries
    int32_t encoding = -1;         // of the values: 0 PLAIN, 2 PLAIN_DICTIONARY, 8 RLE_DICTIONARY
    int32_t def_encoding = -1;     // v1: 3 RLE
    // DATA_PAGE_V2: the levels' lengths (never compressed, no length prefix), and whether the
    // values section is compressed
    int32_t num_nulls = 0;
    int32_t def_bytes = 0;
    int32_t rep_bytes = 0;
    bool v2_compressed = true;
    int64_t header_bytes = 0;      // length of the header itself
};

// Parses the footer of file[0, n); returns an empty string or the reason it cannot be read.
std::string read_file_meta(const uint8_t* file, int64_t n, FileMeta& meta);
// Parses the page header at file[at, n).
std::string read_page_header(const uint8_t* file, int64_t n, int64_t at, PageHeader& ph);

}  // namespace pq
}  // namespace ral
