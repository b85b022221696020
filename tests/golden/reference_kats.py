"""Known-answer tests restated from the reference's own test files.

Each case gives the inputs, the program or RexNode text, and the expected
output exactly as the cited reference test states them (literal tables, or the
host loop the test computes its expectation with).  They pin the CPU oracle
(tests/test_oracle_golden.py) and the GPU library (tests/test_gpu_golden.py).

Reference comparisons print values with ostream's default 6 significant digits
(tests/utils/gdf/library/column.h:166-179); cases marked ``fmt6`` are compared
that way, everything else exactly.
"""
from __future__ import annotations

import numpy as np

# dtype / operator codes (include/ral/gdf_compat.h)
INT8, INT16, INT32, INT64, FLOAT32, FLOAT64 = 1, 2, 3, 4, 5, 6
ADD, SUB, MUL, DIV, MOD = 0, 1, 2, 3, 6
INVALID_BINARY = 21
FLOOR, SIN = 0, 2
INVALID_UNARY = 21

# -- tests/interpreter/interpreter_tests.cu: direct perform_operation programs ----------------

PROGRAM_KATS = [
    dict(
        name="TEST_00",  # interpreter_tests.cu:68-156
        inputs=[(INT32, [i * 2 for i in range(10)]), (INT32, [i * 10 for i in range(10)]),
                (INT32, [i * 20 for i in range(10)])],
        outputs=[INT32, INT32],
        left=[0, 5, 5, 1], right=[1, 2, 1, -2], outs=[5, 5, 3, 4], final=[3, 4],
        ops=[ADD, MUL, ADD, ADD], uops=[INVALID_UNARY] * 4,
        lscalars=[(INT32, 0)] * 4, rscalars=[(INT32, 0), (INT32, 0), (INT32, 0), (INT32, 2)],
        expected=[[0, 250, 980, 2190, 3880, 6050, 8700, 11830, 15440, 19530],
                  [2, 12, 22, 32, 42, 52, 62, 72, 82, 92]],
        fmt6=False,
    ),
    dict(
        name="TEST_FLOATS",  # interpreter_tests.cu:161-244
        inputs=[(FLOAT32, [1.1, 3.6, 5.3, 7.9, 9.35]), (FLOAT32, [1, 1, 1, 1, 1]),
                (FLOAT32, [0, 2, 4, 6, 8])],
        outputs=[FLOAT32, FLOAT32],
        left=[2, 0], right=[0, 1], outs=[3, 4], final=[3, 4],
        ops=[MUL, ADD], uops=[INVALID_UNARY] * 2,
        lscalars=[(INT32, 0)] * 2, rscalars=[(INT32, 0)] * 2,
        expected=[[0, 7.2, 21.2, 47.4, 74.8], [2.1, 4.6, 6.3, 8.9, 10.35]],
        fmt6=False,
    ),
    dict(
        name="TEST_SCALAR_ADD",  # interpreter_tests.cu:248-330
        inputs=[(INT32, [1, 3, 5, 7, 9]), (INT32, [1, 1, 1, 1, 1]), (INT32, [0, 2, 4, 6, 8])],
        outputs=[INT32],
        left=[0], right=[-2], outs=[3], final=[3],
        ops=[ADD], uops=[INVALID_UNARY],
        lscalars=[(INT32, 0)], rscalars=[(INT32, 1)],
        expected=[[2, 4, 6, 8, 10]],
        fmt6=False,
    ),
    dict(
        name="TEST_01_Unary_Operators",  # interpreter_tests.cu:334-417
        inputs=[(FLOAT32, [1.1, 3.6, 5.3, 7.9, 9.35]), (FLOAT32, [0, 2, 4, 6, 8]),
                (FLOAT32, [0, 2, 4, 6, 8])],
        outputs=[FLOAT32, FLOAT32],
        left=[0, 1], right=[-1, -1], outs=[3, 4], final=[3, 4],
        ops=[INVALID_BINARY] * 2, uops=[FLOOR, SIN],
        lscalars=[(INT32, 0)] * 2, rscalars=[(INT32, 0)] * 2,
        expected=[[1, 3, 5, 7, 9], [0, 0.9092974268, -0.7568024953, -0.2794154982, 0.9893582466]],
        fmt6=False,
    ),
    dict(
        name="TEST_02",  # interpreter_tests.cu:434-514 (float literal 2.33 as a FLOAT32 scalar)
        inputs=[(FLOAT32, [(i + 1) * 2.0 for i in range(10)]), (FLOAT32, [(i + 1) * 10.0 for i in range(10)]),
                (INT32, [(i + 1) * 20 for i in range(10)])],
        outputs=[FLOAT32, FLOAT32],
        left=[0, 5, 5, 1, 5], right=[1, 2, 1, -1, -2], outs=[5, 5, 3, 5, 4], final=[3, 4],
        ops=[ADD, MUL, ADD, INVALID_BINARY, ADD],
        uops=[INVALID_UNARY, INVALID_UNARY, INVALID_UNARY, SIN, INVALID_UNARY],
        lscalars=[(FLOAT32, 0.0)] * 5,
        rscalars=[(FLOAT32, 0.0)] * 4 + [(FLOAT32, 2.33)],
        expected=[[250.0, 980.0, 2190.0, 3880.0, 6050.0, 8700.0, 11830.0, 15440.0, 19530.0, 24100.0],
                  [1.78598, 3.24295, 1.34197, 3.07511, 2.06763, 2.02519, 3.10389, 1.33611, 3.224, 1.82363]],
        fmt6=True,
    ),
]

# -- tests/logical-filter/logical_filter-test.cu: evaluate_expression over four INT8 columns --

_N = 32
_in1 = np.array([1 if i % 2 == 0 else i for i in range(_N)], dtype=np.int64)   # :31-36
_in2 = np.arange(_N, dtype=np.int64)
_in3 = np.arange(_N, dtype=np.int64) % 2
_in4 = np.arange(_N, dtype=np.int64) + 1
LOGICAL_FILTER_FRAME = [(INT8, _in1), (INT8, _in2), (INT8, _in3), (INT8, _in4)]


def _b(x):
    return np.asarray(x, dtype=np.int64)


# (expression, host-loop expectation) pairs, logical_filter-test.cu:93-366
LOGICAL_FILTER_KATS = [
    (">($1, 5)", _b(_in2 > 5)),
    ("+(*($1, $0), $2)", (_in1 * _in2) + _in3),
    ("=(=($1, $0), $2)", _b((_b(_in1 == _in2)) == _in3)),
    ("*($0, $0)", _in1 * _in1),
    ("=(*($0, $0), 1))", _b(_in1 * _in1 == 1)),
    ("=($1, $2)", _b(_in2 == _in3)),
    ("AND(=(*($0, $0), 1), =($1, 2))", _b((_in1 * _in1 == 1) & (_in2 == 2))),
    ("AND(=(*($0, $0), 1), =($1, 2), >($2, 0))", _b((_in1 * _in1 == 1) & (_in2 == 2) & (_in3 > 0))),
    ("AND(=($0, 1), >($1, 5), >($2, 0))", _b((_in1 == 1) & (_in2 > 5) & (_in3 > 0))),
    ("AND(=($0, 1), >($1, 5), >($3, 10))", _b((_in1 == 1) & (_in2 > 5) & (_in4 > 10))),
    ("AND(=($0, 1), >($1, 5))", _b((_in1 == 1) & (_in2 > 5))),
    ("AND(>($1, 5), >($2, 0)))", _b((_in2 > 5) & (_in3 > 0))),
    ("AND(>($1, 50), >($2, 0)))", _b((_in2 > 50) & (_in3 > 0))),
    ("AND(>($1, 5), >($2, 100)))", _b((_in2 > 5) & (_in3 > 100))),
    ("AND(=($0, 1), >($1, 5), =($2, 0), >($3, 5))", _b((_in1 == 1) & (_in2 > 5) & (_in3 == 0) & (_in4 > 5))),
    ("AND(=($0, 1), >($1, 5), =($2, 1), >($3, 5))", _b((_in1 == 1) & (_in2 > 5) & (_in3 == 1) & (_in4 > 5))),
]

# -- tests/calcite-interpreter/calcite_interpreter-where-test.cu: filter + gather -------------

_x = np.array([i if i % 2 else 1 for i in range(_N)], dtype=np.int64)   # :37-46
_y = np.arange(_N, dtype=np.int64)
_z = np.ones(_N, dtype=np.int64)
WHERE_FRAME = [(INT32, _x), (INT32, _y), (INT32, _z)]

# (condition, projected frame columns, row mask from the test's host loop)
WHERE_KATS = [
    (">($1, 5)", [1], _y > 5),                                   # :99-124
    ("=($0, $1)", [2], _x == _y),                                # :126-151
    ("=(MOD($1, 5), 0)", [1], _y % 5 == 0),                      # :175-200
    ("AND(=($1, $0), >($0, 4))", [2], (_x == _y) & (_x > 4)),    # :202-227
    ("<>($0, 1)", [0], _x != 1),                                 # :229-254
    ("AND(=($0, $2), >=(4, $1))", [0, 1, 2], (_x == _z) & (4 >= _y)),   # :257-286
    ("AND(=(1, $0), >=(4, $1))", [0, 2], (_x == 1) & (4 >= _y)),        # :289-315
]

# -- tests/where/where-test.cpp: FLOAT64 compares against +-1 ---------------------------------

SWINGS = np.array([1, 2, 3, 4, 5, 6, 7], dtype=np.float64)      # :24-36
TRACTIONS = np.array([1, 0, 1, 0, -1, 0, -1], dtype=np.float64)
WHERE_F64_KATS = [                                                 # :63-118
    ("=($1, 1)", [1, 3]),
    ("<($1, 1)", [2, 4, 5, 6, 7]),
    (">($1, 1)", []),
    ("=($1, -1)", [5, 7]),
    ("<($1, -1)", []),
    (">($1, -1)", [1, 2, 3, 4, 6]),
]

# -- tests/evaluate_query/evaluate_query.cu: IS NULL / IS NOT NULL through the filter ---------

IS_NULL_KATS = [
    dict(  # :44-72
        name="TEST_IS_NULL", condition="IS NULL($0)",
        frame=[(INT32, [1, 2, 3, 4, 5, 6, 7, 8, 9, 1], [0, 1, 1, 1, 0, 0, 0, 0, 1, 1]),
               (INT32, [10, 20, 30, 40, 50, 60, 70, 80, 90, 10], [1] * 10)],
        expected=[([1, 5, 6, 7, 8], [0, 0, 0, 0, 0]), ([10, 50, 60, 70, 80], [1] * 5)],
    ),
    dict(  # :74-102
        name="TEST_IS_NOT_NULL", condition="IS NOT NULL($0)",
        frame=[(INT32, [1, 2, 3, 4, 5, 6, 7, 8, 9, 1], [0, 1, 1, 1, 0, 0, 0, 0, 1, 1]),
               (INT32, [10, 20, 30, 40, 50, 60, 70, 80, 90, 10], [1, 1, 1, 1, 0, 0, 0, 0, 1, 1])],
        expected=[([2, 3, 4, 9, 1], [1] * 5), ([20, 30, 40, 90, 10], [1] * 5)],
    ),
]

# -- tests/interpreter/process_project_tests.cu and interops_coalesce_test.cu -----------------
# These two reference tests print but do not assert values; the expectations below follow the
# interpreter's documented rules (data = row arithmetic, valid = AND; COALESCE valid = OR).

EMPS = [(INT32, [1, 2, 3, 4, 5, 6, 7, 8, 9, 1], [0, 1, 1, 1, 0, 0, 0, 0, 1, 1]),
        (INT32, [10, 20, 10, 20, 10, 20, 10, 20, 10, 2], [1, 1, 1, 1, 0, 0, 0, 0, 1, 1]),
        (INT32, [9000, 8000, 7000, 6000, 5000, 4000, 3000, 2000, 1000, 0], [1] * 10)]
PROJECT_KATS = [
    ("LogicalProject(EXPR$0=[+($0, $2)])",                         # process_project_tests.cu:34-46
     [([9001, 8002, 7003, 6004, 5005, 4006, 3007, 2008, 1009, 1],
       [0, 1, 1, 1, 0, 0, 0, 0, 1, 1])]),
    ("LogicalProject(EXPR$0=[CASE(IS NOT NULL($0), $0, -1)])",     # interops_coalesce_test.cu:36
     [([-1, 2, 3, 4, -1, -1, -1, -1, 9, 1], [1] * 10)]),
]

# tests/integration/aggregation-without-group-by/test-aggregation-without-group-by.cpp: main.part
# with p_partkey = 1..200 (INT32, no nulls).  TEST_01 (:66-118) aggregates the table; TEST_03
# (:121-177) aggregates it behind LogicalFilter(<($0, 0)), i.e. over zero rows: COUNT is a valid 0,
# the others are null (valid_result {1, 0, 0, 0, 0}).  Values are compared, as the test's
# CHECK_RESULT compares printed values (MIN / MAX keep the INT32 input type,
# CalciteExpressionParsing.cpp:103-106).
PARTKEY = [(INT32, list(range(1, 201)), None)]
AGG_QUERY = ("LogicalAggregate(group=[{}], EXPR$0=[COUNT()], EXPR$1=[SUM($0)], EXPR$2=[AVG($0)], "
             "EXPR$3=[MAX($0)], EXPR$4=[MIN($0)])")
AGG_KATS = [
    {"name": "TEST_01", "filter": None,
     "expected": [(INT64, True, 200), (INT64, True, 20100), (FLOAT64, True, 100.5), (INT32, True, 200),
                  (INT32, True, 1)]},
    {"name": "TEST_03", "filter": "LogicalFilter(condition=[<($0, 0)])",
     "expected": [(INT64, True, 0), (INT64, False, None), (FLOAT64, False, None), (INT32, False, None),
                  (INT32, False, None)]},
]

# tests/nvcategory/nvcategory-test.cu: string-category filters.  x INT32, y STRING_CATEGORY over the
# strings below; LogicalFilter(<($1, 'e')) with 'e' in the dictionary (:363-402) and <($1, 'f') with
# 'f' missing (:404-443, the dictionary grows); expected: the x of the rows whose y sorts below the
# literal.  The test draws x at random; any x values give the same kept rows.
CATEGORY_STRINGS = ["a", "b", "c", "d", "e", "g", "h", "i", "j", "k"]
CATEGORY_KATS = [("LogicalFilter(condition=[<($1, 'e')])", "e"),
                 ("LogicalFilter(condition=[<($1, 'f')])", "f")]
