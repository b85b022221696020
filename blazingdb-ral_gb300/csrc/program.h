// program.h — the register program of the RAL interpreter, validated and typed.
//
// A program arrives as the reference's parallel vectors (left / right / output
// register per op, binary and unary operator per op, left and right scalar per
// op, final output registers), exactly as perform_operation receives them
// (src/Interpreter/interpreter_cpp.h:25-37).  Register numbering follows
// src/Interpreter/interpreter_cpp.cu:56-58: inputs 0..n_in-1, the final output
// registers n_in..n_in+n_out-1, temporaries above.
//
// Program::build() performs what the reference does in the InterpreterFunctor
// constructor (src/Interpreter/interpreter_ops.cuh:1095-1178): per-op operand
// and result types, the 64-bit encoding of literals, and the validity-pass
// column flags of interpreter_ops.cuh:1314.  It also rejects programs the
// reference cannot execute deterministically (reads of unwritten registers,
// unsupported operators, unreadable dtypes) instead of running them.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "ral/gdf_compat.h"

namespace ral {

// Register kind: every integer-like value lives in an int64 register and every
// float (FP32 included) in a double register (interpreter_ops.cuh:215-218).
enum class Kind : uint8_t { I64 = 0, F64 = 1 };

struct Op {
    int16_t left, right, out;
    int32_t bop, uop;
    bool unary;                    // right == -1
    gdf_dtype ltype, rtype, otype; // inferred dtypes (otype is GDF_INT64, GDF_FLOAT64 or GDF_invalid)
    Kind lk, rk, ok;               // register kinds the op computes with
    uint64_t lscalar, rscalar;     // 64-bit slot encoding of SCALAR_INDEX operands
};

struct ColumnDesc {
    gdf_dtype dtype;
    bool has_valid;       // valid pointer non-null
    bool nulls_possible;  // has_valid && null_count != 0 (the validity pass reads the mask)
};

class Program {
public:
    int n_in = 0;
    int n_out = 0;
    std::vector<Op> ops;
    std::vector<int16_t> final_pos;
    std::vector<ColumnDesc> inputs;
    std::vector<gdf_dtype> out_dtypes;
    std::vector<bool> out_has_valid;
    std::vector<bool> force_valid;  // input column treated as all-valid by the validity pass
    bool float_literal_compat = false;

    // Build from the reference's vectors.  Returns false and sets err on a
    // program that cannot be run.
    bool build(const std::vector<ColumnDesc>& in_cols, const std::vector<gdf_dtype>& out_types,
               const std::vector<bool>& out_valid, const int16_t* left, const int16_t* right,
               const int16_t* outs, int n_ops, const int16_t* final_positions, const int32_t* bops,
               const int32_t* uops, const gdf_scalar* lscalars, const gdf_scalar* rscalars,
               std::string& err);

    // A string that identifies everything the generated kernel depends on
    // except the literal values (those travel as kernel arguments).
    std::string structure_key() const;

    // Input columns whose data the program reads.
    std::vector<bool> inputs_referenced() const;
    // Input columns whose raw validity bits the data pass reads (IS_NULL, COALESCE).
    std::vector<bool> inputs_raw_valid() const;
};

// Output-type rules of src/CalciteExpressionParsing.cpp:21-42,177-270.
bool dtype_is_signed(gdf_dtype t);
bool dtype_is_float(gdf_dtype t);
bool dtype_is_date(gdf_dtype t);
gdf_dtype result_type_unary(gdf_dtype in, int32_t op);
gdf_dtype result_type_binary(gdf_dtype l, gdf_dtype r, int32_t op);

// Dtypes the interpreter can read into a register / write from a register.
bool dtype_readable(gdf_dtype t);
bool dtype_writable(gdf_dtype t);

}  // namespace ral
