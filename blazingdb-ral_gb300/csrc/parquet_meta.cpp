// parquet_meta.cpp — Thrift compact protocol reader for the Parquet footer and page headers.
//
// Compact protocol (Apache Thrift): a struct is a sequence of fields, each introduced by a byte
// whose high nibble is the field-id delta (0: the id follows as a zigzag varint) and whose low
// nibble is the type (1/2 bool true/false, 3 byte, 4 i16, 5 i32, 6 i64, 7 double, 8 binary,
// 9 list, 10 set, 11 map, 12 struct), ended by a 0 byte; integers are zigzag varints; a list
// header is (size << 4 | element type), or 0xF? followed by the size as a varint.  Field ids are
// those of parquet.thrift.
#include "parquet_meta.h"

#include <stdexcept>

namespace ral {
namespace pq {

namespace {

struct Reader {
    const uint8_t* p;
    const uint8_t* e;
    std::vector<int16_t> last{0};

    uint8_t byte() {
        if (p >= e) throw std::runtime_error("truncated metadata");
        return *p++;
    }
    uint64_t varint() {
        uint64_t v = 0;
        for (int shift = 0; shift < 64; shift += 7) {
            const uint8_t b = byte();
            v |= (uint64_t)(b & 0x7f) << shift;
            if (!(b & 0x80)) return v;
        }
        throw std::runtime_error("bad varint");
    }
    int64_t zigzag() {
        const uint64_t v = varint();
        return (int64_t)(v >> 1) ^ -(int64_t)(v & 1);
    }
    // next field of the current struct: false at its end
    bool field(int16_t& id, int& type) {
        const uint8_t h = byte();
        if (h == 0) return false;
        type = h & 0x0f;
        const int delta = h >> 4;
        id = delta ? (int16_t)(last.back() + delta) : (int16_t)zigzag();
        last.back() = id;
        return true;
    }
    void begin() { last.push_back(0); }
    void end() { last.pop_back(); }
    std::string binary() {
        const uint64_t n = varint();
        if ((uint64_t)(e - p) < n) throw std::runtime_error("truncated metadata");
        std::string s((const char*)p, (size_t)n);
        p += n;
        return s;
    }
    void list_header(int& etype, uint64_t& n) {
        const uint8_t h = byte();
        etype = h & 0x0f;
        n = h >> 4;
        if (n == 15) n = varint();
    }
    void skip(int type) {
        switch (type) {
        case 1: case 2: return;
        case 3: byte(); return;
        case 4: case 5: case 6: varint(); return;
        case 7: for (int k = 0; k < 8; k++) byte(); return;
        case 8: binary(); return;
        case 9: case 10: {
            int et;
            uint64_t n;
            list_header(et, n);
            for (uint64_t k = 0; k < n; k++) skip(et);
            return;
        }
        case 11: {
            const uint64_t n = varint();
            if (n == 0) return;
            const uint8_t kv = byte();
            for (uint64_t k = 0; k < n; k++) {
                skip(kv >> 4);
                skip(kv & 0x0f);
            }
            return;
        }
        case 12: {
            begin();
            int16_t id;
            int t;
            while (field(id, t)) skip(t);
            end();
            return;
        }
        default: throw std::runtime_error("unknown thrift type");
        }
    }
};

void read_schema_element(Reader& r, SchemaLeaf& s, int32_t& num_children) {
    r.begin();
    int16_t id;
    int t;
    num_children = 0;
    while (r.field(id, t)) {
        if (id == 1 && t == 5) s.type = (int32_t)r.zigzag();
        else if (id == 3 && t == 5) s.repetition = (int32_t)r.zigzag();
        else if (id == 4 && t == 8) s.name = r.binary();
        else if (id == 5 && t == 5) num_children = (int32_t)r.zigzag();
        else if (id == 6 && t == 5) s.converted_type = (int32_t)r.zigzag();
        else r.skip(t);
    }
    r.end();
}

void read_column_meta(Reader& r, ColumnChunkMeta& c) {
    r.begin();
    int16_t id;
    int t;
    while (r.field(id, t)) {
        if (id == 1 && t == 5) c.type = (int32_t)r.zigzag();
        else if (id == 4 && t == 5) c.codec = (int32_t)r.zigzag();
        else if (id == 5 && t == 6) c.num_values = r.zigzag();
        else if (id == 7 && t == 6) c.total_compressed_size = r.zigzag();
        else if (id == 9 && t == 6) c.data_page_offset = r.zigzag();
        else if (id == 11 && t == 6) c.dictionary_page_offset = r.zigzag();
        else r.skip(t);
    }
    r.end();
}

void read_row_group(Reader& r, RowGroupMeta& g) {
    r.begin();
    int16_t id;
    int t;
    while (r.field(id, t)) {
        if (id == 1 && t == 9) {
            int et;
            uint64_t n;
            r.list_header(et, n);
            for (uint64_t k = 0; k < n; k++) {
                ColumnChunkMeta c;
                r.begin();
                int16_t cid;
                int ct;
                while (r.field(cid, ct)) {
                    if (cid == 3 && ct == 12) read_column_meta(r, c);
                    else r.skip(ct);
                }
                r.end();
                g.columns.push_back(c);
            }
        } else if (id == 3 && t == 6) {
            g.num_rows = r.zigzag();
        } else {
            r.skip(t);
        }
    }
    r.end();
}

}  // namespace

std::string read_file_meta(const uint8_t* file, int64_t n, FileMeta& meta) {
    if (n < 12 || file[0] != 'P' || file[1] != 'A' || file[2] != 'R' || file[3] != '1' || file[n - 4] != 'P' ||
        file[n - 3] != 'A' || file[n - 2] != 'R' || file[n - 1] != '1')
        return "not a Parquet file (no PAR1 magic)";
    const uint32_t len = (uint32_t)file[n - 8] | (uint32_t)file[n - 7] << 8 | (uint32_t)file[n - 6] << 16 |
                         (uint32_t)file[n - 5] << 24;
    if ((int64_t)len > n - 12) return "bad footer length";
    try {
        Reader r{file + n - 8 - len, file + n - 8};
        int16_t id;
        int t;
        std::vector<SchemaLeaf> elems;
        std::vector<int32_t> children;
        while (r.field(id, t)) {
            if (id == 2 && t == 9) {
                int et;
                uint64_t cnt;
                r.list_header(et, cnt);
                for (uint64_t k = 0; k < cnt; k++) {
                    SchemaLeaf s;
                    int32_t nc = 0;
                    read_schema_element(r, s, nc);
                    elems.push_back(s);
                    children.push_back(nc);
                }
            } else if (id == 3 && t == 6) {
                meta.num_rows = r.zigzag();
            } else if (id == 4 && t == 9) {
                int et;
                uint64_t cnt;
                r.list_header(et, cnt);
                for (uint64_t k = 0; k < cnt; k++) {
                    RowGroupMeta g;
                    read_row_group(r, g);
                    meta.row_groups.push_back(std::move(g));
                }
            } else {
                r.skip(t);
            }
        }
        if (elems.empty()) return "empty schema";
        // a flat schema: the root, then its leaves
        if (children[0] != (int32_t)elems.size() - 1) return "nested schemas are not supported";
        for (size_t k = 1; k < elems.size(); k++) {
            if (children[k] != 0) return "nested schemas are not supported";
            meta.leaves.push_back(elems[k]);
        }
        for (const RowGroupMeta& g : meta.row_groups)
            if (g.columns.size() != meta.leaves.size()) return "a row group's column count differs from the schema's";
    } catch (const std::exception& ex) {
        return std::string("Parquet footer: ") + ex.what();
    }
    return "";
}

std::string read_page_header(const uint8_t* file, int64_t n, int64_t at, PageHeader& ph) {
    if (at < 0 || at >= n) return "page offset outside the file";
    try {
        Reader r{file + at, file + n};
        int16_t id;
        int t;
        while (r.field(id, t)) {
            if (id == 1 && t == 5) ph.type = (int32_t)r.zigzag();
            else if (id == 2 && t == 5) ph.uncompressed_size = (int32_t)r.zigzag();
            else if (id == 3 && t == 5) ph.compressed_size = (int32_t)r.zigzag();
            else if (id == 5 && t == 12) {  // DataPageHeader
                r.begin();
                int16_t did;
                int dt;
                while (r.field(did, dt)) {
                    if (did == 1 && dt == 5) ph.num_values = (int32_t)r.zigzag();
                    else if (did == 2 && dt == 5) ph.encoding = (int32_t)r.zigzag();
                    else if (did == 3 && dt == 5) ph.def_encoding = (int32_t)r.zigzag();
                    else r.skip(dt);
                }
                r.end();
            } else if (id == 7 && t == 12) {  // DictionaryPageHeader
                r.begin();
                int16_t did;
                int dt;
                while (r.field(did, dt)) {
                    if (did == 1 && dt == 5) ph.num_values = (int32_t)r.zigzag();
                    else if (did == 2 && dt == 5) ph.encoding = (int32_t)r.zigzag();
                    else r.skip(dt);
                }
                r.end();
            } else if (id == 8 && t == 12) {  // DataPageHeaderV2
                r.begin();
                int16_t did;
                int dt;
                while (r.field(did, dt)) {
                    if (did == 1 && dt == 5) ph.num_values = (int32_t)r.zigzag();
                    else if (did == 2 && dt == 5) ph.num_nulls = (int32_t)r.zigzag();
                    else if (did == 4 && dt == 5) ph.encoding = (int32_t)r.zigzag();
                    else if (did == 5 && dt == 5) ph.def_bytes = (int32_t)r.zigzag();
                    else if (did == 6 && dt == 5) ph.rep_bytes = (int32_t)r.zigzag();
                    else if (did == 7 && (dt == 1 || dt == 2)) ph.v2_compressed = dt == 1;
                    else r.skip(dt);
                }
                r.end();
            } else {
                r.skip(t);
            }
        }
        ph.header_bytes = (int64_t)(r.p - (file + at));
    } catch (const std::exception& ex) {
        return std::string("Parquet page header: ") + ex.what();
    }
    return "";
}

}  // namespace pq
}  // namespace ral
