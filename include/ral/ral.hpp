// ral.hpp — C++ entry points with the reference's signatures, over the C ABI.
//
// Header-only.  Each function takes the same arguments as the reference
// function it replaces and throws std::runtime_error on failure, as the
// reference does (its CheckCudaErrors / CUDF_CALL macros, src/Utils.cuh:25-55).
//
//   ral::perform_operation     <- src/Interpreter/interpreter_cpp.h:25-37
//   ral::evaluate_expression   <- src/LogicalFilter.h:20-23 (output by pointer:
//                                 the reference takes a gdf_column_cpp&)
//   ral::process_filter        <- src/CalciteInterpreter.cpp:509 (frame and
//                                 output columns passed explicitly)
//   ral::execute_project_plan  <- src/CalciteInterpreter.h:61
//   ral::materialize_column    <- src/ColumnManipulation.cuh:16-18
//   ral::materialize_columns   <- the per-column materialize_column loops of joins and order-by
//   ral::add_expression_to_plan<- src/LogicalFilter.h:26-42
#ifndef RAL_HPP_
#define RAL_HPP_

#include <stdexcept>
#include <string>
#include <vector>

#include "ral/ral_c.h"

namespace ral {

inline void check(int rc) {
    if (rc != RAL_SUCCESS) throw std::runtime_error(std::string("ralgpu: ") + ral_last_error());
}

inline void perform_operation(std::vector<gdf_column*> output_columns, std::vector<gdf_column*> input_columns,
                              std::vector<column_index_type>& left_inputs,
                              std::vector<column_index_type>& right_inputs,
                              std::vector<column_index_type>& outputs,
                              std::vector<column_index_type>& final_output_positions,
                              std::vector<gdf_binary_operator>& operators,
                              std::vector<gdf_unary_operator>& unary_operators,
                              std::vector<gdf_scalar>& left_scalars, std::vector<gdf_scalar>& right_scalars,
                              std::vector<column_index_type> new_input_indices) {
    std::vector<int32_t> ops(operators.begin(), operators.end());
    std::vector<int32_t> uops(unary_operators.begin(), unary_operators.end());
    check(ral_perform_operation(output_columns.data(), (int32_t)output_columns.size(), input_columns.data(),
                                (int32_t)input_columns.size(), left_inputs.data(), right_inputs.data(),
                                outputs.data(), (int32_t)left_inputs.size(), final_output_positions.data(),
                                ops.data(), uops.data(), left_scalars.data(), right_scalars.data(),
                                new_input_indices.data(), (int32_t)new_input_indices.size()));
}

inline void evaluate_expression(const std::vector<gdf_column*>& frame, const std::string& expression,
                                gdf_column* output) {
    check(ral_evaluate_expression(frame.data(), (int32_t)frame.size(), expression.c_str(), output));
}

// Returns the kept row count; out_columns as documented for ral_process_filter.
inline gdf_size_type process_filter(const std::vector<gdf_column*>& frame, const std::string& query_part,
                                    const std::vector<gdf_column*>& out_columns) {
    gdf_size_type n = 0;
    check(ral_process_filter(frame.data(), (int32_t)frame.size(), query_part.c_str(), out_columns.data(), &n));
    return n;
}

inline void execute_project_plan(const std::vector<gdf_column*>& frame, const std::string& query_part,
                                 const std::vector<gdf_column*>& out_columns) {
    check(ral_execute_project_plan(frame.data(), (int32_t)frame.size(), query_part.c_str(), out_columns.data(),
                                   (int32_t)out_columns.size()));
}

inline void materialize_column(gdf_column* input, gdf_column* output, gdf_column* row_indices) {
    check(ral_materialize_column(input, output, row_indices));
}

// Every column of a table gathered by one index column (the per-column loops of
// JoinOperator.cpp:130,135 and OrderBy.cpp:66 in one call).
inline void materialize_columns(const std::vector<gdf_column*>& inputs, const std::vector<gdf_column*>& outputs,
                                gdf_column* row_indices) {
    if (inputs.size() != outputs.size()) throw std::runtime_error("materialize_columns: inputs and outputs differ in count");
    check(ral_materialize_columns(inputs.data(), outputs.data(), (int32_t)inputs.size(), row_indices));
}

inline void add_expression_to_plan(const std::string& expression, column_index_type expression_position,
                                   column_index_type num_outputs, column_index_type num_inputs,
                                   std::vector<column_index_type>& left_inputs,
                                   std::vector<column_index_type>& right_inputs,
                                   std::vector<column_index_type>& outputs,
                                   std::vector<gdf_binary_operator>& operators,
                                   std::vector<gdf_unary_operator>& unary_operators,
                                   std::vector<gdf_scalar>& left_scalars, std::vector<gdf_scalar>& right_scalars,
                                   std::vector<column_index_type>& new_input_indices) {
    const int32_t cap = (int32_t)left_inputs.size() + 512;
    int32_t n = (int32_t)left_inputs.size();
    std::vector<column_index_type> l(left_inputs), r(right_inputs), o(outputs);
    std::vector<int32_t> b(operators.begin(), operators.end()), u(unary_operators.begin(), unary_operators.end());
    std::vector<gdf_scalar> ls(left_scalars), rs(right_scalars);
    l.resize(cap); r.resize(cap); o.resize(cap); b.resize(cap); u.resize(cap); ls.resize(cap); rs.resize(cap);
    check(ral_add_expression_to_plan(expression.c_str(), expression_position, num_outputs, num_inputs,
                                     new_input_indices.data(), (int32_t)new_input_indices.size(), l.data(),
                                     r.data(), o.data(), b.data(), u.data(), ls.data(), rs.data(), &n, cap));
    left_inputs.assign(l.begin(), l.begin() + n);
    right_inputs.assign(r.begin(), r.begin() + n);
    outputs.assign(o.begin(), o.begin() + n);
    operators.clear();
    unary_operators.clear();
    for (int32_t k = 0; k < n; k++) {
        operators.push_back((gdf_binary_operator)b[k]);
        unary_operators.push_back((gdf_unary_operator)u[k]);
    }
    left_scalars.assign(ls.begin(), ls.begin() + n);
    right_scalars.assign(rs.begin(), rs.begin() + n);
}

}  // namespace ral

#endif  // RAL_HPP_
