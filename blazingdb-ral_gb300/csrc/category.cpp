// category.cpp — string-category dictionaries and string literals in predicates.
//
// A GDF_STRING_CATEGORY column holds int32 codes; its dtype_info.category points at the
// dictionary (NVCategory in the reference).  The dictionary keeps its distinct strings sorted by
// byte value and a code is the rank of its string, so comparing codes compares strings.  The
// reference resolves a string literal on the right of a binary operator whose left operand is such
// a column (src/LogicalFilter.cpp:150-194): the literal's code when the dictionary has it;
// otherwise a new dictionary with the string added, the column's codes rewritten to the new ranks,
// the column pointed at the new dictionary, and the new string's code.  ral_category is that
// dictionary here; the rewrite of the codes is one elementwise kernel.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <iterator>
#include <string>
#include <vector>

#include "engine.h"
#include "frontend.h"
#include "kernels.h"
#include "ral/ral_c.h"

struct ral_category_s {
    std::vector<std::string> keys;  // sorted by byte value, distinct
};

namespace ral {

namespace {

// std::string::compare orders by unsigned byte value (char_traits<char>::compare is memcmp-like)
int32_t find_key(const ral_category* c, const std::string& s) {
    auto it = std::lower_bound(c->keys.begin(), c->keys.end(), s);
    if (it == c->keys.end() || *it != s) return -1;
    return (int32_t)(it - c->keys.begin());
}

thread_local CategoryScope* t_scope = nullptr;
thread_local bool t_types_only = false;

}  // namespace

int32_t resolve_and_grow(CategoryScope* sc, int col, const std::string& str);

// The resolver the front end calls for a string literal compared with frame column `col`.
int32_t resolve_category_literal(int col, const std::string& str) {
    CategoryScope* sc = t_scope;
    if (!sc) {
        // planning for output types only: the code does not matter
        if (t_types_only) return 0;
        throw ParseError("string literal '" + str + "': string-category columns are resolved by the entry points "
                         "that take the frame");
    }
    if (sc->replaying) {
        auto it = sc->codes.find(sc->current);
        size_t& k = sc->next[sc->current];
        if (it == sc->codes.end() || k >= it->second.size())
            throw ParseError("string literal '" + str + "' was not resolved before planning");
        return it->second[k++];
    }
    const int32_t code = resolve_and_grow(sc, col, str);
    sc->codes[sc->current].push_back(code);
    return code;
}

int32_t resolve_and_grow(CategoryScope* sc, int col, const std::string& str) {
    if (col < 0 || col >= sc->ncols || !sc->frame[col])
        throw ParseError("string literal '" + str + "': column reference out of range");
    gdf_column* c = sc->frame[col];
    if (c->dtype != GDF_STRING_CATEGORY || !c->dtype_info.category)
        throw ParseError("string literal '" + str + "' compared with a column that is not a string category");
    const ral_category* cat = static_cast<const ral_category*>(c->dtype_info.category);
    int32_t code = find_key(cat, str);
    if (code >= 0) return code;
    if (sc->read_only)
        throw ParseError("string literal '" + str + "' is not in the column's dictionary: adding it rewrites the "
                         "column's codes, which needs the column in device memory");
    // add the string: codes at or above its rank move up by one
    auto* grown = new ral_category_s{cat->keys};
    auto it = std::lower_bound(grown->keys.begin(), grown->keys.end(), str);
    const int32_t pos = (int32_t)(it - grown->keys.begin());
    grown->keys.insert(it, str);
    if (c->size > 0) {
        if (!c->data) {
            delete grown;
            throw ParseError("string category column without data");
        }
        cudaStream_t st = cudaStreamPerThread;
        cudaError_t e = launch_category_insert(static_cast<int32_t*>(c->data), c->size, pos, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            delete grown;
            throw ParseError(std::string("rewriting the category codes: ") + cudaGetErrorString(e));
        }
    }
    c->dtype_info.category = grown;
    return pos;
}

namespace {
// codes of column c moved from its dictionary to `merged` (a superset): one table upload and one
// remap kernel
void remap_to(gdf_column* c, const ral_category* merged) {
    const ral_category* old = static_cast<const ral_category*>(c->dtype_info.category);
    std::vector<int32_t> table(old->keys.size());
    for (size_t k = 0; k < old->keys.size(); k++) table[k] = find_key(merged, old->keys[k]);
    if (c->size > 0 && !table.empty()) {
        if (!c->data) throw ParseError("string category column without data");
        cudaStream_t st = cudaStreamPerThread;
        int32_t* d = nullptr;
        cudaError_t e = cudaMallocAsync((void**)&d, table.size() * sizeof(int32_t), st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(d, table.data(), table.size() * sizeof(int32_t), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = launch_category_remap(static_cast<int32_t*>(c->data), c->size, d, (int32_t)table.size(), st);
        if (d) cudaFreeAsync(d, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) throw ParseError(std::string("remapping category codes: ") + cudaGetErrorString(e));
    }
}
}  // namespace

// Two string-category columns compared with each other share one dictionary afterwards
// (sync_column_categories, called from src/LogicalFilter.cpp:203-211): the union of their strings,
// each column's codes remapped to it.  Each column gets its own copy of the merged dictionary.
void sync_category_columns(int a, int b) {
    CategoryScope* sc = t_scope;
    if (!sc || sc->replaying || a < 0 || b < 0 || a >= sc->ncols || b >= sc->ncols || a == b) return;
    gdf_column* ca = sc->frame[a];
    gdf_column* cb = sc->frame[b];
    if (!ca || !cb || ca->dtype != GDF_STRING_CATEGORY || cb->dtype != GDF_STRING_CATEGORY) return;
    const ral_category* ka = static_cast<const ral_category*>(ca->dtype_info.category);
    const ral_category* kb = static_cast<const ral_category*>(cb->dtype_info.category);
    if (!ka || !kb) throw ParseError("string category column without a dictionary");
    if (ka == kb || ka->keys == kb->keys) return;  // codes already comparable
    if (sc->read_only)
        throw ParseError("two string-category columns with different dictionaries: merging them rewrites their codes, "
                         "which needs the columns in device memory");
    std::vector<std::string> u;
    std::set_union(ka->keys.begin(), ka->keys.end(), kb->keys.begin(), kb->keys.end(), std::back_inserter(u));
    auto* ma = new ral_category_s{u};
    auto* mb = new ral_category_s{u};
    try {
        remap_to(ca, ma);
        remap_to(cb, mb);
    } catch (...) {
        delete ma;
        delete mb;
        throw;
    }
    ca->dtype_info.category = ma;
    cb->dtype_info.category = mb;
}

bool frame_has_category(gdf_column* const* frame, int ncols) {
    for (int c = 0; c < ncols; c++)
        if (frame[c] && frame[c]->dtype == GDF_STRING_CATEGORY) return true;
    return false;
}

TypesOnlyScope::TypesOnlyScope() : prev(t_types_only) { t_types_only = true; }
TypesOnlyScope::~TypesOnlyScope() { t_types_only = prev; }

CategoryScope::CategoryScope(gdf_column* const* f, int n) : frame(f), ncols(n), prev(t_scope) { t_scope = this; }
CategoryScope::~CategoryScope() { t_scope = prev; }
void CategoryScope::planning(const std::string& text) { current = text; }
void category_planning(const std::string& text) {
    if (t_scope) t_scope->planning(text);
}
void CategoryScope::replay() {
    replaying = true;
    next.clear();
}
std::string CategoryScope::recorded_key() const {
    std::string k;
    for (const auto& [text, v] : codes) {
        if (v.empty()) continue;
        k += "{";
        for (int32_t c : v) k += std::to_string(c) + ",";
        k += "}";
    }
    return k;
}

bool has_string_literal(const char* text) { return text && std::strchr(text, '\'') != nullptr; }

std::string category_key(gdf_column* const* frame, int ncols) {
    std::string k;
    char buf[32];
    for (int c = 0; c < ncols; c++)
        if (frame[c] && frame[c]->dtype == GDF_STRING_CATEGORY) {
            snprintf(buf, sizeof buf, "%d:%p;", c, frame[c]->dtype_info.category);
            k += buf;
        }
    return k;
}

}  // namespace ral

extern "C" {

int ral_category_create(const char* const* strings, int64_t n, ral_category** category, int32_t* codes_out) {
    using namespace ral;
    if (!category || n < 0 || (n > 0 && !strings)) return set_error(kInvalidArgument, "null argument");
    try {
        auto* c = new ral_category_s;
        for (int64_t i = 0; i < n; i++) {
            if (!strings[i]) {
                delete c;
                return set_error(kInvalidArgument, "null string at " + std::to_string(i));
            }
            c->keys.emplace_back(strings[i]);
        }
        std::sort(c->keys.begin(), c->keys.end());
        c->keys.erase(std::unique(c->keys.begin(), c->keys.end()), c->keys.end());
        if (c->keys.size() > (size_t)INT32_MAX) {
            delete c;
            return set_error(kInvalidArgument, "too many distinct strings for int32 codes");
        }
        if (codes_out)
            for (int64_t i = 0; i < n; i++) codes_out[i] = find_key(c, strings[i]);
        *category = c;
        return kSuccess;
    } catch (const std::exception& e) {
        return set_error(kInvalidArgument, e.what());
    }
}

int ral_category_size(const ral_category* category, int64_t* num_keys) {
    using namespace ral;
    if (!category || !num_keys) return set_error(kInvalidArgument, "null argument");
    *num_keys = (int64_t)category->keys.size();
    return kSuccess;
}

int ral_category_get_value(const ral_category* category, const char* str, int32_t* code) {
    using namespace ral;
    if (!category || !str || !code) return set_error(kInvalidArgument, "null argument");
    *code = find_key(category, str);
    return kSuccess;
}

int ral_category_key(const ral_category* category, int32_t code, char* buf, int64_t capacity, int64_t* length) {
    using namespace ral;
    if (!category) return set_error(kInvalidArgument, "null argument");
    if (code < 0 || (size_t)code >= category->keys.size()) return set_error(kInvalidArgument, "code out of range");
    const std::string& k = category->keys[code];
    if (length) *length = (int64_t)k.size();
    if (buf && capacity > 0) {
        const size_t m = std::min<size_t>(k.size(), (size_t)capacity - 1);
        std::memcpy(buf, k.data(), m);
        buf[m] = 0;
    }
    return kSuccess;
}

int ral_category_destroy(ral_category* category) {
    delete category;
    return ral::kSuccess;
}

}  // extern "C"
