"""ORACLE front end (test infrastructure only): Calcite RexNode text -> register program.

A restatement of the reference's text pipeline, used by the tests to check the
library's own C++ front end and, together with the C++ oracle VM, to produce
expected results.  Nothing in the product imports this module.

Reference files (paths relative to the reference project root):
  * src/CalciteExpressionParsing.cpp
      clean_calcite_expression :705-754, expand_if_logical_op :629-694,
      find_closing_char :769-811, get_expressions_from_expression_list :814-898,
      get_tokens_in_reverse_order :589-594, is_operator_token :596-598,
      get_index :601-608, is_string/is_literal/is_number :576-587,
      is_date :272-276, get_type_from_string :323-335,
      get_scalar_from_string :337-417, operator maps :509-556,
      get_output_type(unary/binary) :177-270, get_output_type_expression :420-481,
      contains_evaluation :900-903, clean_project_expression :697-703.
  * src/LogicalFilter.cpp
      add_expression_to_plan :44-268, get_first_open_position :30-38,
      evaluate_expression :271-371.
  * src/CalciteInterpreter.cpp
      parse_project_plan :123-309, get_named_expression :426-436,
      process_filter :509-573.

Where the reference silently emits a misaligned program (unary operator on a
literal, literal-op-literal, unknown or `null` tokens, string literals) or
throws, this front end raises FrontendError; the library rejects the same inputs.
Date and timestamp literals, which the reference cannot run (its "%Y-%m-%d %H:%M:%S" parse rejects
a bare date and its space split cuts a timestamp in two), are read as the DATE64 milliseconds that
get_scalar_from_string intends, in both front ends.
StringUtil::splitNotInQuotes (blazingdb-io, not in the reference tree) is
taken to drop empty tokens, since is_operator_token would read past an empty
string otherwise.
"""
from __future__ import annotations

import re
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

# dtype / operator codes (same numbering as include/ral/gdf_compat.h)
GDF_invalid, GDF_INT8, GDF_INT16, GDF_INT32, GDF_INT64, GDF_FLOAT32, GDF_FLOAT64, GDF_BOOL8, \
    GDF_DATE32, GDF_DATE64, GDF_TIMESTAMP, GDF_CATEGORY, GDF_STRING, GDF_STRING_CATEGORY = range(14)

(GDF_ADD, GDF_SUB, GDF_MUL, GDF_DIV, GDF_TRUE_DIV, GDF_FLOOR_DIV, GDF_MOD, GDF_POW, GDF_EQUAL,
 GDF_NOT_EQUAL, GDF_LESS, GDF_GREATER, GDF_LESS_EQUAL, GDF_GREATER_EQUAL, GDF_BITWISE_AND,
 GDF_BITWISE_OR, GDF_BITWISE_XOR, GDF_LOGICAL_AND, GDF_LOGICAL_OR, GDF_COALESCE,
 GDF_GENERIC_BINARY, GDF_INVALID_BINARY) = range(22)

(BLZ_FLOOR, BLZ_CEIL, BLZ_SIN, BLZ_COS, BLZ_ASIN, BLZ_ACOS, BLZ_TAN, BLZ_COTAN, BLZ_ATAN, BLZ_ABS,
 BLZ_NOT, BLZ_LN, BLZ_LOG, BLZ_YEAR, BLZ_MONTH, BLZ_DAY, BLZ_HOUR, BLZ_MINUTE, BLZ_SECOND,
 BLZ_IS_NULL, BLZ_IS_NOT_NULL, BLZ_INVALID_UNARY) = range(22)

SCALAR_INDEX = -2
SCALAR_NULL_INDEX = -3

UNARY_MAP = {
    "NOT": BLZ_NOT, "SIN": BLZ_SIN, "ASIN": BLZ_ASIN, "COS": BLZ_COS, "ACOS": BLZ_ACOS,
    "TAN": BLZ_TAN, "ATAN": BLZ_ATAN, "BL_FLOUR": BLZ_FLOOR, "CEIL": BLZ_CEIL, "ABS": BLZ_ABS,
    "LOG10": BLZ_LOG, "LN": BLZ_LN, "BL_YEAR": BLZ_YEAR, "BL_MONTH": BLZ_MONTH, "BL_DAY": BLZ_DAY,
    "BL_HOUR": BLZ_HOUR, "BL_MINUTE": BLZ_MINUTE, "BL_SECOND": BLZ_SECOND,
    "IS_NULL": BLZ_IS_NULL, "IS_NOT_NULL": BLZ_IS_NOT_NULL,
}
BINARY_MAP = {
    "=": GDF_EQUAL, "<>": GDF_NOT_EQUAL, ">": GDF_GREATER, ">=": GDF_GREATER_EQUAL, "<": GDF_LESS,
    "<=": GDF_LESS_EQUAL, "+": GDF_ADD, "-": GDF_SUB, "*": GDF_MUL, "/": GDF_DIV, "POWER": GDF_POW,
    "MOD": GDF_MOD, "AND": GDF_MUL, "OR": GDF_ADD, "COALESCE": GDF_COALESCE,
}

WIDTH = {GDF_INT8: 1, GDF_BOOL8: 1, GDF_INT16: 2, GDF_INT32: 4, GDF_FLOAT32: 4, GDF_DATE32: 4,
         GDF_CATEGORY: 4, GDF_STRING_CATEGORY: 4, GDF_INT64: 8, GDF_FLOAT64: 8, GDF_DATE64: 8,
         GDF_TIMESTAMP: 8}


class FrontendError(ValueError):
    pass


_COALESCE_RE = re.compile(r"CASE\(IS NOT NULL\((\W\(.+?\)|.+)\), \1, (\W\(.+?\)|.+)\)", re.I)
_COUNT_DISTINCT_RE = re.compile(r"COUNT\(DISTINCT (\W\(.+?\)|.+)\)", re.I)
_INT_RE = re.compile(r"^[-+]?[0-9]+$")
_FLOAT_RE = re.compile(r"^[-+]?[0-9]*\.?[0-9]+([eE][-+]?[0-9]+)?$")
_DATE_RE = re.compile(r"[12]\d{3}-(0[1-9]|1[0-2])-(0[1-9]|[12]\d|3[01])")
_TIME_RE = re.compile(r"([01]\d|2[0-3]):[0-5]\d:[0-5]\d")
_DATETIME_RE = re.compile(r"([12]\d{3}-(?:0[1-9]|1[0-2])-(?:0[1-9]|[12]\d|3[01])) (([01]\d|2[0-3]):[0-5]\d:[0-5]\d)")


def _quoted_vector(s: str) -> List[bool]:
    out, inq = [], False
    for ch in s:
        if ch == "'":
            inq = not inq
            out.append(True)
        else:
            out.append(inq)
    return out


def _find_first_not_in_quotes(s: str, pat: str, start: int, quoted: List[bool]) -> int:
    pos = s.find(pat, max(start, 0))
    while pos >= 0:
        if not quoted[pos]:
            return pos
        pos = s.find(pat, pos + 1)
    return -1


def find_closing_char(expression: str, start: int) -> int:
    open_ch = expression[start]
    if open_ch == "(":
        close_ch = ")"
    elif open_ch == "[":
        close_ch = "]"
    else:
        return -1
    cur, depth, inq = start + 1, 1, False
    while cur < len(expression):
        ch = expression[cur]
        if inq:
            if ch == "'" and not (cur + 1 < len(expression) and expression[cur + 1] == "'"):
                inq = False
        else:
            if ch == "'":
                inq = True
            elif ch == open_ch:
                depth += 1
            elif ch == close_ch:
                depth -= 1
                if depth == 0:
                    return cur
        cur += 1
    return -1


def _common_rewrites(s: str) -> str:
    s = _COALESCE_RE.sub(r"COALESCE(\1, \2)", s)
    s = _COUNT_DISTINCT_RE.sub(r"COUNT_DISTINCT(\1)", s)
    for a, b in ((" NOT NULL", ""), ("):DOUBLE", ""), ("CAST(", ""),
                 ("EXTRACT(FLAG(YEAR), ", "BL_YEAR("), ("EXTRACT(FLAG(MONTH), ", "BL_MONTH("),
                 ("EXTRACT(FLAG(DAY), ", "BL_DAY("), ("FLOOR(", "BL_FLOUR(")):
        s = s.replace(a, b)
    return s


def get_expressions_from_expression_list(combined: str, trim: bool = True) -> List[str]:
    combined = _common_rewrites(combined)
    exprs: List[str] = []
    cur, start, inq, pdepth, sdepth = 0, 0, False, 0, 0
    while cur < len(combined):
        ch = combined[cur]
        if inq:
            if ch == "'" and not (cur + 1 < len(combined) and combined[cur + 1] == "'"):
                inq = False
        else:
            if ch == "'":
                inq = True
            elif ch == "(":
                pdepth += 1
            elif ch == ")":
                pdepth -= 1
            elif ch == "[":
                sdepth += 1
            elif ch == "]":
                sdepth -= 1
            elif ch == "," and pdepth == 0 and sdepth == 0:
                e = combined[start:cur]
                exprs.append(e.lstrip() if trim else e)
                start = cur + 1
        cur += 1
    if start < len(combined):
        e = combined[start:cur]
        exprs.append(e.strip() if trim else e)
    return [_common_rewrites(e) for e in exprs]


def expand_if_logical_op(expression: str) -> str:
    output = expression
    start_pos = 0
    while start_pos < len(expression):
        quoted = _quoted_vector(expression)
        first_and = _find_first_not_in_quotes(expression, "AND(", start_pos, quoted)
        first_or = _find_first_not_in_quotes(expression, "OR(", start_pos, quoted)
        if first_and >= 0:
            if 0 <= first_or < first_and:
                first, op = first_or, "OR("
            else:
                first, op = first_and, "AND("
        else:
            first, op = first_or, "OR("
        if first < 0:
            return output
        expr_start = first + len(op) - 1
        expr_end = find_closing_char(expression, expr_start)
        if expr_end < 0:
            raise FrontendError("unbalanced parentheses in logical operator")
        rest = expression[expr_start + 1:expr_end]
        processed = get_expressions_from_expression_list(rest, False)
        if len(processed) == 2:
            start_pos = expr_start
            continue
        start_pos = first
        output = expression[:first]
        for _ in range(len(processed) - 1):
            output += op
            start_pos += len(op)
        output += processed[0] + ","
        for i in range(1, len(processed) - 1):
            output += processed[i] + "),"
        output += processed[-1] + ")"
        if expr_end < len(expression) - 1:
            output += expression[expr_end + 1:]
        expression = output
    return output


def clean_calcite_expression(expression: str) -> str:
    expression = _COALESCE_RE.sub(r"COALESCE(\1, \2)", expression)
    for a, b in (("IS NOT NULL", "IS_NOT_NULL"), ("IS NULL", "IS_NULL"), (" NOT NULL", ""),
                 ("):DOUBLE", ""), ("CAST(", ""),
                 ("EXTRACT(FLAG(YEAR), ", "BL_YEAR("), ("EXTRACT(FLAG(MONTH), ", "BL_MONTH("),
                 ("EXTRACT(FLAG(DAY), ", "BL_DAY("), ("EXTRACT(FLAG(HOUR), ", "BL_HOUR("),
                 ("EXTRACT(FLAG(MINUTE), ", "BL_MINUTE("), ("EXTRACT(FLAG(SECOND), ", "BL_SECOND("),
                 ("FLOOR(", "BL_FLOUR(")):
        expression = expression.replace(a, b)
    expression = expand_if_logical_op(expression)
    out = []
    for ch in expression:
        if ch == "(":
            out.append(" ")
        elif ch != "," and ch != ")":
            out.append(ch)
    # a TIMESTAMP literal keeps its time part in the same token (the reference's space split would
    # separate it; this restatement joins it with a "T", which get_scalar_from_string reads back)
    return _DATETIME_RE.sub(r"\1T\2", "".join(out))


def clean_project_expression(expression: str) -> str:
    return expression.replace("CAST(", "").replace("):BIGINT", "")


def contains_evaluation(expression: str) -> bool:
    return "(" in clean_project_expression(expression)


def _split_not_in_quotes(s: str) -> List[str]:
    toks, cur, inq = [], [], False
    for ch in s:
        if ch == "'":
            inq = not inq
            cur.append(ch)
        elif ch == " " and not inq:
            toks.append("".join(cur))
            cur = []
        else:
            cur.append(ch)
    toks.append("".join(cur))
    return [t for t in toks if t != ""]


def get_tokens_in_reverse_order(expression: str) -> List[str]:
    return list(reversed(_split_not_in_quotes(expression)))


def is_string(op: str) -> bool:
    return len(op) > 0 and op[0] == "'" and op[-1] == "'"


def is_literal(op: str) -> bool:
    return op[0] != "$"


def is_number(s: str) -> bool:
    return _FLOAT_RE.match(s) is not None


def is_date(s: str) -> bool:
    """is_date (CalciteExpressionParsing.cpp:272-276), also taking the joined "DATE" + "T" + "TIME"
    token of a TIMESTAMP literal."""
    if _DATE_RE.fullmatch(s) is not None:
        return True
    return len(s) == 19 and s[10] == "T" and _DATE_RE.fullmatch(s[:10]) is not None and \
        _TIME_RE.fullmatch(s[11:]) is not None


def is_operator_token(op: str) -> bool:
    return op[0] != "$" and not is_number(op) and not is_date(op) and not is_string(op)


def get_index(operand: str) -> int:
    cleaned = clean_calcite_expression(operand)
    if len(cleaned) == 0:
        return 0
    return int(cleaned if is_literal(cleaned) else cleaned[1:])


def get_type_from_string(s: str) -> int:
    if _INT_RE.match(s):
        return GDF_INT64
    if _FLOAT_RE.match(s):
        return GDF_FLOAT64
    return GDF_DATE64


@dataclass
class Scalar:
    dtype: int
    value: float | int
    is_valid: bool = True


JUNK = Scalar(GDF_INT32, 0, True)   # the tests' "junk" placeholder scalar


def get_scalar_from_string(s: str, dtype: int) -> Scalar:
    if s == "null":
        return Scalar(GDF_INT8, 0, False)
    if dtype == GDF_INT64:
        v = int(s)
        if not (-(1 << 63) <= v < (1 << 63)):
            raise FrontendError("integer literal out of range")
        return Scalar(GDF_INT64, v)
    if dtype == GDF_FLOAT64:
        return Scalar(GDF_FLOAT64, float(s))
    if dtype == GDF_DATE64 and is_date(s):
        # get_date_64_from_string (:293-305): "%Y-%m-%d %H:%M:%S" into a zeroed std::tm (tm_isdst 0),
        # mktime in the local time zone, milliseconds; a bare date is taken at 00:00:00
        import time
        d, t = (s[:10], s[11:]) if len(s) == 19 else (s, "00:00:00")
        y, mo, da = (int(x) for x in d.split("-"))
        h, mi, se = (int(x) for x in t.split(":"))
        return Scalar(GDF_DATE64, int(time.mktime((y, mo, da, h, mi, se, 0, 0, 0))) * 1000)
    raise FrontendError("Invalid datetime format")


@dataclass
class Plan:
    """The five parallel vectors plus scalars that perform_operation consumes."""
    left: List[int] = field(default_factory=list)
    right: List[int] = field(default_factory=list)
    outputs: List[int] = field(default_factory=list)
    final_output_positions: List[int] = field(default_factory=list)
    operators: List[int] = field(default_factory=list)
    unary_operators: List[int] = field(default_factory=list)
    left_scalars: List[Scalar] = field(default_factory=list)
    right_scalars: List[Scalar] = field(default_factory=list)
    new_input_indices: List[int] = field(default_factory=list)


# Set by the oracle's entry points while they plan over a frame: (frame column, string) -> code,
# and (frame column, frame column) -> None for two category columns compared with each other.
CATEGORY_RESOLVER = None
CATEGORY_SYNC = None


def add_expression_to_plan(expression: str, expression_position: int, num_outputs: int,
                           num_inputs: int, plan: Plan, new_input_indices: Sequence[int]) -> None:
    start = num_inputs + num_outputs
    clean = clean_calcite_expression(expression)
    stack: List[tuple] = []
    free = [True] * 512
    for i in range(start):
        free[i] = False
    tokens = get_tokens_in_reverse_order(clean)
    if not tokens:
        raise FrontendError("empty expression")

    def first_open() -> int:
        for i in range(start, len(free)):
            if free[i]:
                free[i] = False
                return i
        raise FrontendError("out of registers")

    for ti, tok in enumerate(tokens):
        if is_operator_token(tok):
            if tok in BINARY_MAP:
                if len(stack) < 2:
                    raise FrontendError("binary operator with fewer than two operands")
                lt, lpos = stack.pop()
                if not is_literal(lt) and lpos >= start:
                    free[lpos] = True
                rt, rpos = stack.pop()
                if not is_literal(rt) and rpos >= start:
                    free[rpos] = True
                op = BINARY_MAP[tok]
                if is_literal(lt) and is_literal(rt):
                    raise FrontendError("operator on two literals is not supported")
                if is_string(lt):
                    raise FrontendError("a string literal on the left of an operator is not supported")
                plan.operators.append(op)
                plan.unary_operators.append(BLZ_INVALID_UNARY)
                if is_literal(lt):
                    sc = get_scalar_from_string(lt, get_type_from_string(lt))
                    plan.left_scalars.append(sc)
                    plan.right_scalars.append(JUNK)
                    plan.left.append(SCALAR_INDEX if sc.is_valid else SCALAR_NULL_INDEX)
                    plan.right.append(get_index(rt))
                elif is_string(rt):
                    # LogicalFilter.cpp:150-194: the string's code in the left column's dictionary,
                    # the string added (and the column's codes rewritten) when it is missing
                    dense = get_index(lt)
                    if CATEGORY_RESOLVER is None or not lt.startswith("$") or dense not in new_input_indices:
                        raise FrontendError("a string literal must be compared with a string-category column")
                    sc = Scalar(GDF_INT32, CATEGORY_RESOLVER(list(new_input_indices).index(dense), rt[1:-1]))
                    plan.right_scalars.append(sc)
                    plan.left_scalars.append(JUNK)
                    plan.right.append(SCALAR_INDEX)
                    plan.left.append(dense)
                elif is_literal(rt):
                    sc = get_scalar_from_string(rt, get_type_from_string(rt))
                    plan.right_scalars.append(sc)
                    plan.left_scalars.append(JUNK)
                    plan.right.append(SCALAR_INDEX if sc.is_valid else SCALAR_NULL_INDEX)
                    plan.left.append(get_index(lt))
                else:
                    li, ri = get_index(lt), get_index(rt)
                    # two input columns: string-category columns move to one merged dictionary
                    # (sync_column_categories, LogicalFilter.cpp:196-211)
                    if CATEGORY_SYNC is not None and li < num_inputs and ri < num_inputs:
                        idx = list(new_input_indices)
                        if li in idx and ri in idx:
                            CATEGORY_SYNC(idx.index(li), idx.index(ri))
                    plan.left.append(li)
                    plan.right.append(ri)
                    plan.left_scalars.append(JUNK)
                    plan.right_scalars.append(JUNK)
            elif tok in UNARY_MAP:
                if len(stack) < 1:
                    raise FrontendError("unary operator without operand")
                lt, lpos = stack.pop()
                if not is_literal(lt) and lpos >= start:
                    free[lpos] = True
                if is_literal(lt):
                    raise FrontendError("unary operator on a literal is not supported")
                plan.operators.append(GDF_INVALID_BINARY)
                plan.unary_operators.append(UNARY_MAP[tok])
                plan.left.append(get_index(lt))
                plan.right.append(-1)
                plan.left_scalars.append(JUNK)
                plan.right_scalars.append(JUNK)
            else:
                raise FrontendError("unsupported token: " + tok)
            if ti == len(tokens) - 1:
                plan.outputs.append(expression_position + num_inputs)
            else:
                pos = first_open()
                plan.outputs.append(pos)
                stack.append(("$" + str(pos), pos))
        else:
            if is_literal(tok) or is_string(tok):
                stack.append((tok, SCALAR_INDEX))
            else:
                idx = new_input_indices[get_index(tok)]
                stack.append(("$" + str(idx), idx))
    if len(plan.outputs) == 0 or plan.outputs[-1] != expression_position + num_inputs:
        raise FrontendError("expression has no operator")
    if stack:
        raise FrontendError("dangling operands in expression")


# --- output types (CalciteExpressionParsing.cpp:21-42,177-270,420-481) ----------------------

def is_type_signed(t: int) -> bool:
    return t in (GDF_INT8, GDF_INT16, GDF_INT32, GDF_INT64, GDF_FLOAT32, GDF_FLOAT64, GDF_DATE32,
                 GDF_DATE64, GDF_TIMESTAMP)


def is_type_float(t: int) -> bool:
    return t in (GDF_FLOAT32, GDF_FLOAT64)


def is_date_type(t: int) -> bool:
    return t in (GDF_DATE32, GDF_DATE64, GDF_TIMESTAMP)


def output_type_unary(t: int, op: int) -> int:
    if is_date_type(t):
        return GDF_INT16
    if op in (BLZ_SIN, BLZ_COS, BLZ_ASIN, BLZ_ACOS, BLZ_TAN, BLZ_COTAN, BLZ_ATAN, BLZ_LOG, BLZ_LN):
        return t if is_type_float(t) else GDF_FLOAT64
    if op in (BLZ_IS_NULL, BLZ_IS_NOT_NULL):
        return GDF_INT8
    return t


def output_type_binary(l: int, r: int, op: int) -> int:
    if not is_type_signed(l) or not is_type_signed(r):
        return GDF_invalid
    if op in (GDF_ADD, GDF_SUB, GDF_MUL, GDF_DIV, GDF_MOD):
        if is_type_float(l) or is_type_float(r):
            if is_type_float(l) and is_type_float(r):
                return l if WIDTH[l] >= WIDTH[r] else r
            return l if is_type_float(l) else r
        return l if WIDTH[l] >= WIDTH[r] else r
    if op in (GDF_EQUAL, GDF_NOT_EQUAL, GDF_GREATER, GDF_GREATER_EQUAL, GDF_LESS, GDF_LESS_EQUAL):
        return GDF_INT8
    if op == GDF_POW:
        return GDF_FLOAT64 if (is_type_float(l) or is_type_float(r)) else GDF_INT64
    if op == GDF_COALESCE:
        return l
    return GDF_invalid


def get_output_type_expression(frame_dtypes: Sequence[int], expression: str) -> int:
    clean = clean_calcite_expression(expression)
    st: List[int] = []
    for tok in get_tokens_in_reverse_order(clean):
        if is_operator_token(tok):
            if tok in BINARY_MAP:
                if len(st) < 2:
                    raise FrontendError("operator on fewer than two operands")
                l, r = st.pop(), st.pop()
                if l == GDF_invalid:
                    if r == GDF_invalid:
                        raise FrontendError("invalid operands")
                    l = r
                elif r == GDF_invalid:
                    r = l
                st.append(output_type_binary(l, r, BINARY_MAP[tok]))
            elif tok in UNARY_MAP:
                st.append(output_type_unary(st.pop(), UNARY_MAP[tok]))
            else:
                raise FrontendError("unsupported operator token, " + tok)
        else:
            if is_literal(tok) or is_string(tok):
                st.append(GDF_invalid)
            else:
                st.append(frame_dtypes[get_index(tok)])
    return st[-1]


# --- plan builders for the three entry points ---------------------------------------------------

def plan_evaluate_expression(num_frame_columns: int, expression: str):
    """Returns ('clone', index) for the "$n" shortcut, else ('program', Plan, used_columns)."""
    if expression[0] == "$":
        return ("clone", get_index(expression))
    clean = clean_calcite_expression(expression)
    used = [False] * num_frame_columns
    for tok in get_tokens_in_reverse_order(clean):
        if not is_operator_token(tok) and not is_literal(tok) and not is_string(tok):
            idx = get_index(tok)
            if idx >= num_frame_columns:
                raise FrontendError("column index out of range")
            used[idx] = True
    new_idx, cols = [], []
    for i, u in enumerate(used):
        if u:
            new_idx.append(len(cols))
            cols.append(i)
        else:
            new_idx.append(-1)
    plan = Plan(new_input_indices=new_idx)
    plan.final_output_positions = [len(cols)]
    add_expression_to_plan(expression, 0, 1, len(cols), plan, new_idx)
    return ("program", plan, cols)


@dataclass
class ProjectPlan:
    plan: Plan
    input_columns: List[int]          # frame indices, dense order
    output_types: List[int]           # dtype of each evaluated expression, in order
    columns: List[tuple]              # per projected column: ('expr', k) or ('pass', frame index)
    names: List[str]


def parse_project_plan(frame_dtypes: Sequence[int], query_part: str) -> ProjectPlan:
    combined = query_part[query_part.find("(") + 1:query_part.rfind(")")]
    exprs = get_expressions_from_expression_list(combined)
    ncols = len(frame_dtypes)
    used = [False] * ncols
    bodies, names, out_types = [], [], []
    n_eval = 0
    for e in exprs:
        p = e.find("=[")
        body = e[p + 2:len(e) - 1]
        bodies.append(body)
        names.append(e[:p])
        if contains_evaluation(body):
            out_types.append(get_output_type_expression(frame_dtypes, body))
            for tok in get_tokens_in_reverse_order(clean_calcite_expression(body)):
                if not is_operator_token(tok) and not is_literal(tok):
                    used[get_index(tok)] = True
            n_eval += 1
    new_idx, cols = [], []
    for i, u in enumerate(used):
        if u:
            new_idx.append(len(cols))
            cols.append(i)
        else:
            new_idx.append(-1)
    plan = Plan(new_input_indices=new_idx)
    plan.final_output_positions = [len(cols) + k for k in range(n_eval)]
    columns, k = [], 0
    for body in bodies:
        if contains_evaluation(body):
            add_expression_to_plan(body, k, n_eval, len(cols), plan, new_idx)
            columns.append(("expr", k))
            k += 1
        else:
            columns.append(("pass", get_index(body)))
    return ProjectPlan(plan, cols, out_types, columns, names)


GDF_SUM, GDF_MIN, GDF_MAX, GDF_AVG, GDF_COUNT, GDF_COUNT_DISTINCT = range(6)
AGG_OPS = {"SUM": GDF_SUM, "MIN": GDF_MIN, "MAX": GDF_MAX, "AVG": GDF_AVG, "COUNT": GDF_COUNT,
           "COUNT_DISTINCT": GDF_COUNT_DISTINCT}


def get_string_between_outer_parentheses(s: str) -> str:
    """src/CalciteExpressionParsing.cpp:756-767."""
    a, b = s.find("("), s.rfind(")")
    if a < 0 or b < 0 or b < a:
        return ""
    return s[a + 1:b]


def get_aggregation_operation(expression: str) -> int:
    """src/CalciteExpressionParsing.cpp:483-507: the text between "=[" and the first "]", up to "("."""
    start = expression.find("=[") + 2
    end = expression.find("]")
    op = expression[start:] if end < 0 else expression[start:end]
    op = op[:op.find("(")] if "(" in op else op
    if op not in AGG_OPS:
        raise ValueError("aggregation type not supported: " + op)
    return AGG_OPS[op]


def parse_aggregate(query_part: str):
    """process_aggregate's parse, src/operators/GroupBy.cpp:531-569: the GROUP BY columns and, per
    aggregation, (name, gdf_agg_op, input expression text).  The combined expression drops the
    character before the last ')' (the closing ']'), as the reference's substr does."""
    a = query_part.find("(")
    combined = query_part[a + 1:a + 1 + (query_part.rfind(")") - a - 1) - 1]
    groups: List[int] = []
    aggs = []
    for e in get_expressions_from_expression_list(combined):
        e = re.sub(r"^ +| +$|( ) +", r"\1", e)
        if "group=" in e:
            body = e[e.find("{") + 1:e.find("}")]
            groups = [int(x) for x in body.replace(" ", "").split(",") if x != ""]
            continue
        aggs.append((e[:e.find("=[")], get_aggregation_operation(e), get_string_between_outer_parentheses(e)))
    return groups, aggs


def get_aggregation_output_type(t: int, op: int) -> int:
    """src/CalciteExpressionParsing.cpp:92-116, without a GROUP BY."""
    if op in (GDF_COUNT, GDF_COUNT_DISTINCT):
        return GDF_INT64
    if op == GDF_SUM:
        return GDF_FLOAT64 if is_type_float(t) else GDF_INT64
    if op in (GDF_MIN, GDF_MAX):
        return t
    return GDF_FLOAT64


def get_named_expression(query_part: str, name: str) -> str:
    if query_part.find(name + "=[") < 0:
        return ""
    if query_part.find(name + "=[[") >= 0:
        start = query_part.find(name + "=[[") + 3 + len(name)
    else:
        start = query_part.find(name + "=[") + 2 + len(name)
    end = query_part.find("]", start)
    return query_part[start:end]


def get_condition_expression(query_part: str) -> str:
    return get_named_expression(query_part, "condition")
