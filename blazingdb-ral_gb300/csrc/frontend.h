// frontend.h — Calcite RexNode text -> register program.
//
// Accepts the expression language of src/CalciteExpressionParsing.cpp and
// emits exactly the program src/LogicalFilter.cpp:44-268 emits for it (same op
// order, same temp registers), because the program layout is observable: the
// validity pass's column flags depend on op positions
// (src/Interpreter/interpreter_ops.cuh:1314).
#pragma once

#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "ral/gdf_compat.h"

namespace ral {

struct ProgramVectors {
    std::vector<int16_t> left, right, outs, final_pos;
    std::vector<int32_t> bops, uops;
    std::vector<gdf_scalar> lscalars, rscalars;
};

struct ParseError : std::exception {
    std::string msg;
    explicit ParseError(std::string m) : msg(std::move(m)) {}
    const char* what() const noexcept override { return msg.c_str(); }
};

struct Expr {
    enum Kind { Column, Literal, Call } kind = Literal;
    int column = -1;                 // frame column index for Column
    std::string text;                // literal text, or operator name for Call
    std::vector<std::unique_ptr<Expr>> args;
};

// Applies the reference's textual rewrites (CASE(IS NOT NULL(x), x, y) ->
// COALESCE(x, y), IS [NOT] NULL -> IS_[NOT_]NULL, CAST removal, EXTRACT ->
// BL_*, FLOOR -> BL_FLOUR), then parses.  N-ary AND/OR become left-nested
// binary calls.  Throws ParseError.
std::unique_ptr<Expr> parse_expression(const std::string& text);

// Frame column indices referenced by the expression.
void collect_columns(const Expr& e, std::vector<bool>& used);

// add_expression_to_plan: appends the ops of `e` to `pv`.  new_input_indices
// maps frame column -> input register.  Throws ParseError.
void emit_expression(const Expr& e, int expression_position, int num_outputs, int num_inputs,
                     const std::vector<int>& new_input_indices, ProgramVectors& pv);

// get_output_type_expression (literals count as "invalid" and take the other
// operand's type).  Throws ParseError.
gdf_dtype expression_output_type(const Expr& e, const std::vector<gdf_dtype>& frame_dtypes);

// True when the expression text contains an evaluation (contains_evaluation).
bool contains_evaluation(const std::string& expr_text);
// get_index of a bare "$k" reference.
int column_reference_index(const std::string& expr_text);

// get_named_expression(query_part, name)
std::string named_expression(const std::string& query_part, const std::string& name);

// Splits "LogicalProject(a=[e1], b=[e2])" into (name, expression text) pairs
// (get_expressions_from_expression_list + the substr logic of parse_project_plan).
std::vector<std::pair<std::string, std::string>> project_expressions(const std::string& query_part);

// Plan for evaluate_expression: the "$k" clone shortcut or a one-output program.
struct ExpressionPlan {
    bool clone = false;
    int clone_column = -1;
    std::vector<int> input_columns;  // frame columns in register order
    ProgramVectors pv;
};
ExpressionPlan plan_expression(const std::string& expression, int num_frame_columns);

// Plan for a LogicalProject.
struct ProjectPlan {
    std::vector<int> input_columns;
    ProgramVectors pv;
    std::vector<gdf_dtype> eval_dtypes;        // per evaluated expression
    std::vector<std::pair<bool, int>> columns; // per projected column: (evaluated, k or frame column)
    std::vector<std::string> names;
};
ProjectPlan plan_project(const std::string& query_part, const std::vector<gdf_dtype>& frame_dtypes);

// ---- string literals against string-category columns (category.cpp) -------------------------
// A string literal on the right of a binary operator whose left operand is a frame column of dtype
// GDF_STRING_CATEGORY becomes an INT32 scalar: the literal's code in the column's dictionary, the
// string inserted (and the column's codes rewritten) when it is missing, as
// src/LogicalFilter.cpp:150-194 does.  The frame is the one the calling entry point holds: a
// CategoryScope makes it visible to the front end on this thread for the duration of a call.
//
// The reference resolves each literal once, in its emission order, against the dictionary as it is
// at that moment (a later insertion leaves an earlier literal's code as it was).  An entry point
// that plans a text more than once (a resolving pass ahead of its plan caches) records the codes
// of the first pass per text and replays them in order afterwards; the recorded codes are part of
// the cache keys.
struct CategoryScope {
    CategoryScope(gdf_column* const* frame, int ncols);
    ~CategoryScope();
    void planning(const std::string& text);  // the text whose literals resolve next
    void replay();                           // later resolutions return the recorded codes
    std::string recorded_key() const;
    gdf_column* const* frame;
    int ncols;
    CategoryScope* prev;
    std::map<std::string, std::vector<int32_t>> codes;
    std::map<std::string, size_t> next;
    std::string current;
    bool replaying = false;
    bool read_only = false;  // columns in host memory: a rewrite of codes is refused
};
// Planning that only asks for output types (no frame): string literals resolve to a placeholder.
struct TypesOnlyScope {
    TypesOnlyScope();
    ~TypesOnlyScope();
    bool prev;
};
int32_t resolve_category_literal(int frame_column, const std::string& str);
// CategoryScope::planning on this thread's active scope, if any.
void category_planning(const std::string& text);
// Two category columns compared with each other: both moved to one merged dictionary.
void sync_category_columns(int frame_column_a, int frame_column_b);
bool frame_has_category(gdf_column* const* frame, int ncols);
bool has_string_literal(const char* text);
// The dictionaries of a frame's category columns, for plan-cache keys.
std::string category_key(gdf_column* const* frame, int ncols);

// Plan for a LogicalAggregate (process_aggregate, src/operators/GroupBy.cpp:531-590): the GROUP BY
// columns, and per aggregation its operator (get_aggregation_operation,
// CalciteExpressionParsing.cpp:483-507) and input, the text between the outer parentheses
// (get_string_between_outer_parentheses, :756-767).  An input that contains an evaluation is an
// output of ONE program over every evaluated input (the reference evaluates each into a column of
// its own; data does not depend on op positions); any other input is a frame column (get_index,
// an empty text -- COUNT() -- meaning column 0).
struct AggregatePlan {
    std::vector<int> group_columns;
    std::vector<int> input_columns;         // program inputs: frame columns in register order
    ProgramVectors pv;
    std::vector<gdf_dtype> eval_dtypes;     // per evaluated input: get_output_type_expression
    struct Aggregation {
        std::string name;
        int op = 0;                         // gdf_agg_op
        bool evaluated = false;
        int index = -1;                     // evaluated input number, or frame column
    };
    std::vector<Aggregation> aggregations;
};
AggregatePlan plan_aggregate(const std::string& query_part, const std::vector<gdf_dtype>& frame_dtypes);

}  // namespace ral
