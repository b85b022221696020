// program.cpp — validation and type inference of register programs.
#include "program.h"

#include <cstring>
#include <sstream>

namespace ral {

bool dtype_is_signed(gdf_dtype t) {
    switch (t) {
    case GDF_INT8: case GDF_INT16: case GDF_INT32: case GDF_INT64: case GDF_FLOAT32:
    case GDF_FLOAT64: case GDF_DATE32: case GDF_DATE64: case GDF_TIMESTAMP: return true;
    default: return false;
    }
}
bool dtype_is_float(gdf_dtype t) { return t == GDF_FLOAT32 || t == GDF_FLOAT64; }
bool dtype_is_date(gdf_dtype t) { return t == GDF_DATE32 || t == GDF_DATE64 || t == GDF_TIMESTAMP; }

// interpreter_ops.cuh:177-187: the dtypes a literal of which becomes an int64 register
static bool scalar_is_int(gdf_dtype t) {
    switch (t) {
    case GDF_INT8: case GDF_INT16: case GDF_INT32: case GDF_INT64: case GDF_DATE32:
    case GDF_DATE64: case GDF_TIMESTAMP: case GDF_STRING_CATEGORY: return true;
    default: return false;
    }
}

bool dtype_readable(gdf_dtype t) {
    switch (t) {
    case GDF_INT8: case GDF_INT16: case GDF_INT32: case GDF_INT64: case GDF_FLOAT32:
    case GDF_FLOAT64: case GDF_DATE32: case GDF_DATE64: case GDF_TIMESTAMP:
    case GDF_STRING_CATEGORY: return true;
    default: return false;  // BOOL8 and others: read_data has no branch for them
    }
}
bool dtype_writable(gdf_dtype t) { return dtype_readable(t); }

gdf_dtype result_type_unary(gdf_dtype in, int32_t op) {
    if (dtype_is_date(in)) return GDF_INT16;
    switch (op) {
    case BLZ_SIN: case BLZ_COS: case BLZ_ASIN: case BLZ_ACOS: case BLZ_TAN: case BLZ_COTAN:
    case BLZ_ATAN: case BLZ_LOG: case BLZ_LN:
        return dtype_is_float(in) ? in : GDF_FLOAT64;
    case BLZ_IS_NULL: case BLZ_IS_NOT_NULL:
        return GDF_INT8;
    default:
        return in;
    }
}

gdf_dtype result_type_binary(gdf_dtype l, gdf_dtype r, int32_t op) {
    if (!dtype_is_signed(l) || !dtype_is_signed(r)) return GDF_invalid;
    switch (op) {
    case GDF_ADD: case GDF_SUB: case GDF_MUL: case GDF_DIV: case GDF_MOD: {
        const bool lf = dtype_is_float(l), rf = dtype_is_float(r);
        if (lf && rf) return gdf_dtype_size(l) >= gdf_dtype_size(r) ? l : r;
        if (lf) return l;
        if (rf) return r;
        return gdf_dtype_size(l) >= gdf_dtype_size(r) ? l : r;
    }
    case GDF_EQUAL: case GDF_NOT_EQUAL: case GDF_LESS: case GDF_GREATER: case GDF_LESS_EQUAL:
    case GDF_GREATER_EQUAL:
        return GDF_INT8;
    case GDF_POW:
        return (dtype_is_float(l) || dtype_is_float(r)) ? GDF_FLOAT64 : GDF_INT64;
    case GDF_COALESCE:
        return l;
    default:
        return GDF_invalid;
    }
}

static Kind kind_of(gdf_dtype t) { return dtype_is_float(t) ? Kind::F64 : Kind::I64; }

// The 64-bit slot a literal occupies (interpreter_ops.cuh:156-175).  Floats keep
// their value (the double's bit pattern); float_literal_compat reproduces the
// shipped value-to-int64 conversion.
static uint64_t literal_slot(const gdf_scalar& s, bool compat) {
    int64_t v = 0;
    switch (s.dtype) {
    case GDF_INT8: v = s.data.si08; break;
    case GDF_INT16: v = s.data.si16; break;
    case GDF_INT32: case GDF_STRING_CATEGORY: v = s.data.si32; break;
    case GDF_DATE32: v = s.data.dt32; break;
    case GDF_INT64: v = s.data.si64; break;
    case GDF_DATE64: v = s.data.dt64; break;
    case GDF_TIMESTAMP: v = s.data.tmst; break;
    case GDF_FLOAT32: {
        if (compat) { v = (int64_t)s.data.fp32; break; }
        double d = (double)s.data.fp32;
        std::memcpy(&v, &d, 8);
        break;
    }
    case GDF_FLOAT64: {
        if (compat) { v = (int64_t)s.data.fp64; break; }
        std::memcpy(&v, &s.data.fp64, 8);
        break;
    }
    default: v = 0; break;
    }
    return (uint64_t)v;
}

static bool binary_op_supported(int32_t b) {
    switch (b) {
    case GDF_ADD: case GDF_SUB: case GDF_MUL: case GDF_DIV: case GDF_FLOOR_DIV: case GDF_MOD:
    case GDF_POW: case GDF_EQUAL: case GDF_NOT_EQUAL: case GDF_LESS: case GDF_GREATER:
    case GDF_LESS_EQUAL: case GDF_GREATER_EQUAL: case GDF_COALESCE: return true;
    default: return false;  // process_operator_3 has no branch: the register would keep stale data
    }
}

bool Program::build(const std::vector<ColumnDesc>& in_cols, const std::vector<gdf_dtype>& out_types,
                    const std::vector<bool>& out_valid, const int16_t* left, const int16_t* right,
                    const int16_t* outs, int n_ops, const int16_t* final_positions, const int32_t* bops,
                    const int32_t* uops, const gdf_scalar* lscalars, const gdf_scalar* rscalars,
                    std::string& err) {
    inputs = in_cols;
    n_in = (int)in_cols.size();
    n_out = (int)out_types.size();
    out_dtypes = out_types;
    out_has_valid = out_valid;
    final_pos.assign(final_positions, final_positions + n_out);
    ops.clear();
    if (n_in == 0) { err = "perform_operation needs at least one input column"; return false; }
    if (n_out == 0) { err = "perform_operation needs at least one output column"; return false; }
    if (n_ops < 0 || n_ops > 4096) { err = "operation count out of range"; return false; }
    for (int c = 0; c < n_in; c++) {
        if (!dtype_readable(in_cols[c].dtype)) {
            err = "input column " + std::to_string(c) + " has a dtype the interpreter cannot read";
            return false;
        }
    }
    for (int o = 0; o < n_out; o++) {
        if (!dtype_writable(out_types[o])) {
            err = "output column " + std::to_string(o) + " has a dtype the interpreter cannot write";
            return false;
        }
    }

    const int kMaxReg = 1024;
    std::vector<gdf_dtype> reg_type(kMaxReg, GDF_invalid);
    std::vector<bool> reg_written(kMaxReg, false);
    for (int c = 0; c < n_in; c++) reg_written[c] = true;

    auto operand_type = [&](int idx, const gdf_scalar& s, uint64_t& slot, bool& ok) -> gdf_dtype {
        ok = true;
        if (idx >= 0 && idx < n_in) return in_cols[idx].dtype;
        if (idx == SCALAR_NULL_INDEX) return s.dtype;
        if (idx == SCALAR_INDEX) {
            slot = literal_slot(s, float_literal_compat);
            return scalar_is_int(s.dtype) ? GDF_INT64 : GDF_FLOAT64;
        }
        if (idx >= n_in && idx < kMaxReg && reg_written[idx]) return reg_type[idx];
        ok = false;
        return GDF_invalid;
    };

    for (int k = 0; k < n_ops; k++) {
        Op op{};
        op.left = left[k];
        op.right = right[k];
        op.out = outs[k];
        op.bop = bops[k];
        op.uop = uops[k];
        op.unary = (op.right == UNARY_RIGHT_INDEX);
        op.lscalar = op.rscalar = 0;
        const std::string where = "operation " + std::to_string(k) + ": ";
        bool ok = true;
        if (op.unary) {
            if (op.left < 0) { err = where + "unary operator on a literal is not supported"; return false; }
            if (op.uop < 0 || op.uop > BLZ_INVALID_UNARY) { err = where + "unknown unary operator"; return false; }
            if ((op.uop == BLZ_IS_NULL || op.uop == BLZ_IS_NOT_NULL) && op.left >= n_in) {
                err = where + "IS_NULL / IS_NOT_NULL must read an input column";
                return false;
            }
        } else {
            if (!binary_op_supported(op.bop)) { err = where + "binary operator not supported by the interpreter"; return false; }
            if (op.left < SCALAR_NULL_INDEX || op.left == UNARY_RIGHT_INDEX || op.right < SCALAR_NULL_INDEX) {
                err = where + "bad operand index";
                return false;
            }
            if (op.bop == GDF_COALESCE && !(op.left >= 0 && op.left < n_in)) {
                err = where + "COALESCE must take an input column on the left";
                return false;
            }
        }
        op.ltype = operand_type(op.left, lscalars[k], op.lscalar, ok);
        if (!ok) { err = where + "left operand register read before it is written"; return false; }
        if (op.unary) {
            op.rtype = GDF_invalid;
        } else {
            op.rtype = operand_type(op.right, rscalars[k], op.rscalar, ok);
            if (!ok) { err = where + "right operand register read before it is written"; return false; }
        }
        const gdf_dtype t = op.unary ? result_type_unary(op.ltype, op.uop)
                                     : result_type_binary(op.ltype, op.rtype, op.bop);
        if (dtype_is_signed(t) && !dtype_is_float(t)) op.otype = GDF_INT64;
        else if (dtype_is_float(t)) op.otype = GDF_FLOAT64;
        else op.otype = GDF_invalid;  // computed as int64, like the reference
        op.lk = kind_of(op.ltype);
        op.rk = kind_of(op.rtype);
        op.ok = kind_of(op.otype);
        if (op.out < n_in || op.out >= kMaxReg) {
            err = where + "output register overlaps the inputs or is out of range";
            return false;
        }
        reg_type[op.out] = op.otype;
        reg_written[op.out] = true;
        ops.push_back(op);
    }
    for (int o = 0; o < n_out; o++) {
        const int r = final_pos[o];
        if (r < 0 || r >= kMaxReg || !reg_written[r]) {
            err = "final output " + std::to_string(o) + " reads a register that is never written";
            return false;
        }
    }

    // Validity pass column flags (interpreter_ops.cuh:1314): the pass indexes the
    // unary operator array by COLUMN number.  Past the end of that array it reads
    // the int16 position arrays that follow it in the reference's temp space
    // (interpreter_ops.cuh:1028-1039), two at a time as one 32-bit enum value.
    std::vector<int16_t> tail;
    tail.reserve(3 * ops.size() + final_pos.size());
    for (const Op& op : ops) tail.push_back(op.left);
    for (const Op& op : ops) tail.push_back(op.right);
    for (const Op& op : ops) tail.push_back(op.out);
    for (int16_t f : final_pos) tail.push_back(f);
    force_valid.assign(n_in, false);
    for (int c = 0; c < n_in; c++) {
        int32_t u;
        if (c < (int)ops.size()) {
            u = ops[c].uop;
        } else {
            const size_t j = 2 * (size_t)(c - (int)ops.size());
            if (j + 1 >= tail.size()) continue;
            u = (int32_t)((uint32_t)(uint16_t)tail[j] | ((uint32_t)(uint16_t)tail[j + 1] << 16));
        }
        force_valid[c] = (u == BLZ_IS_NULL || u == BLZ_IS_NOT_NULL);
    }
    return true;
}

std::vector<bool> Program::inputs_referenced() const {
    std::vector<bool> r(n_in, false);
    for (const Op& op : ops) {
        if (op.left >= 0 && op.left < n_in) r[op.left] = true;
        if (!op.unary && op.right >= 0 && op.right < n_in) r[op.right] = true;
    }
    for (int16_t f : final_pos)
        if (f >= 0 && f < n_in) r[f] = true;
    return r;
}

std::vector<bool> Program::inputs_raw_valid() const {
    std::vector<bool> r(n_in, false);
    for (const Op& op : ops) {
        if (op.unary && (op.uop == BLZ_IS_NULL || op.uop == BLZ_IS_NOT_NULL)) r[op.left] = true;
        if (!op.unary && op.bop == GDF_COALESCE) r[op.left] = true;
    }
    return r;
}

std::string Program::structure_key() const {
    std::ostringstream s;
    s << "i" << n_in << "o" << n_out << "|";
    for (int c = 0; c < n_in; c++)
        s << (int)inputs[c].dtype << (inputs[c].has_valid ? "v" : "") << (inputs[c].nulls_possible ? "n" : "")
          << (force_valid[c] ? "f" : "") << ",";
    s << "|";
    for (int o = 0; o < n_out; o++) s << (int)out_dtypes[o] << (out_has_valid[o] ? "v" : "") << "@" << final_pos[o] << ",";
    s << "|";
    for (const Op& op : ops) {
        s << op.left << ":" << op.right << ":" << op.out << ":" << op.bop << ":" << op.uop << ":"
          << (int)op.ltype << ":" << (int)op.rtype << ":" << (int)op.otype << ";";
    }
    return s.str();
}

}  // namespace ral
