// frontend.cpp — Calcite RexNode text -> register program.
//
// The reference turns the text into a reversed token stream and runs a stack
// machine over it (src/LogicalFilter.cpp:44-268).  Reversing prefix notation
// and popping "left" first means: the right operand's ops are emitted before
// the left operand's, then the op itself; temporaries come from a free list
// that starts at num_inputs + num_outputs, operands are released before the
// result register is taken, and the expression's last op writes register
// num_inputs + expression_position.  This file builds a syntax tree and emits
// in that order with that allocator, so programs are identical to the
// reference's for every expression both accept.
#include "frontend.h"
#include "program.h"

#include <algorithm>
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <regex>
#include <sstream>
#include <iomanip>
#include <ctime>

namespace ral {

namespace {

const std::map<std::string, int32_t>& binary_ops() {
    // src/CalciteExpressionParsing.cpp:540-556; AND/OR are integer multiply/add
    static const std::map<std::string, int32_t> m = {
        {"=", GDF_EQUAL}, {"<>", GDF_NOT_EQUAL}, {">", GDF_GREATER}, {">=", GDF_GREATER_EQUAL},
        {"<", GDF_LESS}, {"<=", GDF_LESS_EQUAL}, {"+", GDF_ADD}, {"-", GDF_SUB}, {"*", GDF_MUL},
        {"/", GDF_DIV}, {"POWER", GDF_POW}, {"MOD", GDF_MOD}, {"AND", GDF_MUL}, {"OR", GDF_ADD},
        {"COALESCE", GDF_COALESCE}};
    return m;
}
const std::map<std::string, int32_t>& unary_ops() {
    // src/CalciteExpressionParsing.cpp:509-530
    static const std::map<std::string, int32_t> m = {
        {"NOT", BLZ_NOT}, {"SIN", BLZ_SIN}, {"ASIN", BLZ_ASIN}, {"COS", BLZ_COS}, {"ACOS", BLZ_ACOS},
        {"TAN", BLZ_TAN}, {"ATAN", BLZ_ATAN}, {"BL_FLOUR", BLZ_FLOOR}, {"CEIL", BLZ_CEIL},
        {"ABS", BLZ_ABS}, {"LOG10", BLZ_LOG}, {"LN", BLZ_LN}, {"BL_YEAR", BLZ_YEAR},
        {"BL_MONTH", BLZ_MONTH}, {"BL_DAY", BLZ_DAY}, {"BL_HOUR", BLZ_HOUR}, {"BL_MINUTE", BLZ_MINUTE},
        {"BL_SECOND", BLZ_SECOND}, {"IS_NULL", BLZ_IS_NULL}, {"IS_NOT_NULL", BLZ_IS_NOT_NULL}};
    return m;
}

void replace_all(std::string& s, const std::string& a, const std::string& b) {
    if (a.empty()) return;
    size_t pos = 0;
    while ((pos = s.find(a, pos)) != std::string::npos) {
        s.replace(pos, a.size(), b);
        pos += b.size();
    }
}

const std::regex& coalesce_re() {
    static const std::regex re{R"(CASE\(IS NOT NULL\((\W\(.+?\)|.+)\), \1, (\W\(.+?\)|.+)\))",
                               std::regex_constants::icase};
    return re;
}

// CAST(x):TYPE [NOT NULL] -> x, for any TYPE.  The reference strips "CAST(" and
// "):DOUBLE" textually; this keeps the operand for the other type names too.
std::string strip_casts(std::string s) {
    for (;;) {
        size_t p = s.find("CAST(");
        if (p == std::string::npos) return s;
        int depth = 0;
        size_t q = p + 4;
        for (; q < s.size(); q++) {
            if (s[q] == '(') depth++;
            else if (s[q] == ')' && --depth == 0) break;
        }
        if (q >= s.size()) throw ParseError("unbalanced CAST(");
        std::string inner = s.substr(p + 5, q - (p + 5));
        size_t e = q + 1;
        if (e < s.size() && s[e] == ':') {
            e++;
            while (e < s.size() && (std::isalnum((unsigned char)s[e]) || s[e] == '_')) e++;
            // optional precision "(p, s)" and " NOT NULL"
            if (e < s.size() && s[e] == '(') {
                size_t c = s.find(')', e);
                if (c != std::string::npos) e = c + 1;
            }
            if (s.compare(e, 9, " NOT NULL") == 0) e += 9;
        }
        s = s.substr(0, p) + inner + s.substr(e);
    }
}

std::string rewrite(std::string s) {
    // clean_calcite_expression's rewrites, CalciteExpressionParsing.cpp:705-722
    s = std::regex_replace(s, coalesce_re(), "COALESCE($1, $2)");
    replace_all(s, "IS NOT NULL", "IS_NOT_NULL");
    replace_all(s, "IS NULL", "IS_NULL");
    s = strip_casts(s);
    replace_all(s, " NOT NULL", "");
    replace_all(s, "):DOUBLE", "");
    replace_all(s, "EXTRACT(FLAG(YEAR), ", "BL_YEAR(");
    replace_all(s, "EXTRACT(FLAG(MONTH), ", "BL_MONTH(");
    replace_all(s, "EXTRACT(FLAG(DAY), ", "BL_DAY(");
    replace_all(s, "EXTRACT(FLAG(HOUR), ", "BL_HOUR(");
    replace_all(s, "EXTRACT(FLAG(MINUTE), ", "BL_MINUTE(");
    replace_all(s, "EXTRACT(FLAG(SECOND), ", "BL_SECOND(");
    replace_all(s, "FLOOR(", "BL_FLOUR(");
    return s;
}

bool is_int_literal(const std::string& s) {
    static const std::regex re{R"(^[-+]?[0-9]+$)"};
    return std::regex_match(s, re);
}
bool is_number_literal(const std::string& s) {
    static const std::regex re{R"(^[-+]?[0-9]*\.?[0-9]+([eE][-+]?[0-9]+)?$)"};
    return std::regex_match(s, re);
}
bool is_date_literal(const std::string& s) {
    static const std::regex re{R"([12]\d{3}-(0[1-9]|1[0-2])-(0[1-9]|[12]\d|3[01]))"};
    return std::regex_match(s, re);
}
bool is_time_of_day(const std::string& s) {
    static const std::regex re{R"(([01]\d|2[0-3]):[0-5]\d:[0-5]\d)"};
    return std::regex_match(s, re);
}

// get_date_64_from_string (CalciteExpressionParsing.cpp:293-305): "%Y-%m-%d %H:%M:%S" read into a
// zeroed std::tm (so tm_isdst = 0) and converted by mktime, i.e. in the process's local time zone,
// then to milliseconds.  A date without a time of day is taken at 00:00:00 (the reference's
// format would reject it).
int64_t date64_from_string(const std::string& t) {
    std::tm tm = {};
    std::istringstream ss(t.size() == 10 ? t + " 00:00:00" : t);
    if (!(ss >> std::get_time(&tm, "%Y-%m-%d %H:%M:%S"))) throw ParseError("Invalid datetime format: " + t);
    const int64_t secs = (int64_t)std::mktime(&tm);
    return secs * 1000;
}

struct Parser {
    const std::string& s;
    size_t i = 0;
    explicit Parser(const std::string& str) : s(str) {}
    void ws() { while (i < s.size() && s[i] == ' ') i++; }
    bool delim(char c) const { return c == '(' || c == ')' || c == ',' || c == ' '; }

    std::unique_ptr<Expr> parse() {
        ws();
        if (i >= s.size()) throw ParseError("unexpected end of expression");
        auto e = std::make_unique<Expr>();
        if (s[i] == '\'') {
            // a string literal, '' standing for one quote inside it
            size_t j = i + 1;
            for (;;) {
                if (j >= s.size()) throw ParseError("unterminated string literal");
                if (s[j] == '\'') {
                    if (j + 1 < s.size() && s[j + 1] == '\'') { j += 2; continue; }
                    break;
                }
                j++;
            }
            e->kind = Expr::Literal;
            e->text = s.substr(i, j + 1 - i);
            i = j + 1;
            return e;
        }
        if (s[i] == '$') {
            size_t j = i + 1;
            while (j < s.size() && std::isdigit((unsigned char)s[j])) j++;
            if (j == i + 1) throw ParseError("bad column reference");
            if (j < s.size() && !delim(s[j])) throw ParseError("bad column reference: " + s.substr(i, j - i + 1));
            e->kind = Expr::Column;
            e->column = std::atoi(s.substr(i + 1, j - i - 1).c_str());
            e->text = s.substr(i, j - i);
            i = j;
            return e;
        }
        size_t j = i;
        while (j < s.size() && !delim(s[j])) j++;
        std::string word = s.substr(i, j - i);
        i = j;
        if (i < s.size() && s[i] == '(') {
            i++;
            e->kind = Expr::Call;
            e->text = word;
            ws();
            if (i < s.size() && s[i] == ')') throw ParseError("call without arguments: " + word);
            for (;;) {
                e->args.push_back(parse());
                ws();
                if (i >= s.size()) throw ParseError("missing ')' after arguments of " + word);
                if (s[i] == ',') { i++; continue; }
                if (s[i] == ')') { i++; break; }
                throw ParseError("unexpected character in arguments of " + word);
            }
            return e;
        }
        if (word.empty()) throw ParseError("empty operand");
        // a TIMESTAMP literal "YYYY-MM-DD HH:MM:SS": the time part after the space is part of it
        if (is_date_literal(word) && i + 9 <= s.size() && s[i] == ' ' && is_time_of_day(s.substr(i + 1, 8)) &&
            (i + 9 == s.size() || delim(s[i + 9]))) {
            word += s.substr(i, 9);
            i += 9;
        }
        e->kind = Expr::Literal;
        e->text = word;
        return e;
    }
};

// N-ary AND/OR -> left-nested binary (expand_if_logical_op,
// CalciteExpressionParsing.cpp:629-694); arity checks for everything else.
void normalise(std::unique_ptr<Expr>& e) {
    if (e->kind != Expr::Call) return;
    for (auto& a : e->args) normalise(a);
    const bool logical = e->text == "AND" || e->text == "OR";
    if (logical && e->args.size() > 2) {
        std::vector<std::unique_ptr<Expr>> args = std::move(e->args);
        std::unique_ptr<Expr> acc = std::move(args[0]);
        for (size_t k = 1; k < args.size(); k++) {
            auto n = std::make_unique<Expr>();
            n->kind = Expr::Call;
            n->text = e->text;
            n->args.push_back(std::move(acc));
            n->args.push_back(std::move(args[k]));
            acc = std::move(n);
        }
        e = std::move(acc);
        return;
    }
    if (binary_ops().count(e->text)) {
        if (e->args.size() != 2)
            throw ParseError("operator " + e->text + " takes two operands (got " + std::to_string(e->args.size()) + ")");
    } else if (unary_ops().count(e->text)) {
        if (e->args.size() != 1) throw ParseError("operator " + e->text + " takes one operand");
    } else {
        throw ParseError("unsupported operator: " + e->text);
    }
}

bool is_literal_node(const Expr& e) { return e.kind == Expr::Literal; }
bool is_string_node(const Expr& e) { return e.kind == Expr::Literal && !e.text.empty() && e.text[0] == '\''; }

// The literal between its outer quotes, as the reference takes it (substr(1, size - 2)).
std::string unquote(const std::string& t) { return t.size() >= 2 ? t.substr(1, t.size() - 2) : std::string(); }

// A string literal compared with a string-category column: its INT32 code in the column's
// dictionary (src/LogicalFilter.cpp:150-194).
gdf_scalar category_scalar(const Expr& column, const Expr& literal) {
    if (column.kind != Expr::Column)
        throw ParseError("a string literal must be compared with a string-category column: " + literal.text);
    gdf_scalar sc;
    std::memset(&sc, 0, sizeof sc);
    sc.dtype = GDF_INT32;
    sc.is_valid = true;
    sc.data.si32 = resolve_category_literal(column.column, unquote(literal.text));
    return sc;
}

gdf_scalar literal_scalar(const std::string& t) {
    // get_type_from_string + get_scalar_from_string, CalciteExpressionParsing.cpp:323-417
    gdf_scalar s;
    std::memset(&s, 0, sizeof s);
    s.is_valid = true;
    if (is_date_literal(t.substr(0, 10)) && (t.size() == 10 || (t.size() == 19 && is_time_of_day(t.substr(11))))) {
        // get_type_from_string: neither an integer nor a float -> GDF_DATE64
        s.dtype = GDF_DATE64;
        s.data.dt64 = date64_from_string(t);
        return s;
    }
    if (!is_number_literal(t)) throw ParseError("unsupported token: " + t);
    if (is_int_literal(t)) {
        errno = 0;
        char* end = nullptr;
        long long v = std::strtoll(t.c_str(), &end, 10);
        if (errno == ERANGE) throw ParseError("integer literal out of range: " + t);
        s.dtype = GDF_INT64;
        s.data.si64 = v;
    } else {
        errno = 0;
        char* end = nullptr;
        double v = std::strtod(t.c_str(), &end);
        if (errno == ERANGE && (v == HUGE_VAL || v == -HUGE_VAL)) throw ParseError("float literal out of range: " + t);
        s.dtype = GDF_FLOAT64;
        s.data.fp64 = v;
    }
    return s;
}

gdf_scalar junk_scalar() {
    gdf_scalar s;
    std::memset(&s, 0, sizeof s);
    s.dtype = GDF_INT32;  // placeholder, never read
    s.is_valid = true;
    return s;
}

struct Emitter {
    int start;  // first temporary register
    std::vector<bool> busy;
    const std::vector<int>& remap;
    ProgramVectors& pv;
    Emitter(int st, const std::vector<int>& r, ProgramVectors& p) : start(st), busy(512, false), remap(r), pv(p) {
        for (int k = 0; k < st && k < 512; k++) busy[k] = true;
    }
    int take() {
        for (int k = start; k < 512; k++)
            if (!busy[k]) { busy[k] = true; return k; }
        throw ParseError("expression needs more than 512 registers");
    }
    void release(int reg) {
        if (reg >= start && reg < 512) busy[reg] = false;
    }
    int column_reg(const Expr& e) {
        if (e.column < 0 || e.column >= (int)remap.size() || remap[e.column] < 0)
            throw ParseError("column reference out of range: " + e.text);
        return remap[e.column];
    }
    // Emits e's ops; returns the register holding its value (or -2 for a literal).
    int emit(const Expr& e, int final_reg) {
        if (e.kind == Expr::Column) return column_reg(e);
        if (e.kind == Expr::Literal) return SCALAR_INDEX;
        const bool is_bin = binary_ops().count(e.text) > 0;
        if (is_bin) {
            const Expr& L = *e.args[0];
            const Expr& R = *e.args[1];
            if (is_literal_node(L) && is_literal_node(R)) throw ParseError("operator on two literals is not supported");
            if (is_string_node(L))
                throw ParseError("a string literal on the left of an operator is not supported (as in the reference)");
            // resolved before any op is emitted: a missing string rewrites the column's codes
            gdf_scalar rstring{};
            if (is_string_node(R)) rstring = category_scalar(L, R);
            if (L.kind == Expr::Column && R.kind == Expr::Column) sync_category_columns(L.column, R.column);
            const int rreg = emit(R, -1);
            const int lreg = emit(L, -1);
            release(lreg);
            release(rreg);
            pv.bops.push_back(binary_ops().at(e.text));
            pv.uops.push_back(BLZ_INVALID_UNARY);
            if (is_literal_node(L)) {
                pv.lscalars.push_back(literal_scalar(L.text));
                pv.rscalars.push_back(junk_scalar());
                pv.left.push_back(SCALAR_INDEX);
                pv.right.push_back((int16_t)rreg);
            } else if (is_literal_node(R)) {
                pv.rscalars.push_back(is_string_node(R) ? rstring : literal_scalar(R.text));
                pv.lscalars.push_back(junk_scalar());
                pv.right.push_back(SCALAR_INDEX);
                pv.left.push_back((int16_t)lreg);
            } else {
                pv.left.push_back((int16_t)lreg);
                pv.right.push_back((int16_t)rreg);
                pv.lscalars.push_back(junk_scalar());
                pv.rscalars.push_back(junk_scalar());
            }
        } else {
            const Expr& L = *e.args[0];
            if (is_literal_node(L)) throw ParseError("unary operator on a literal is not supported");
            const int lreg = emit(L, -1);
            release(lreg);
            pv.bops.push_back(GDF_INVALID_BINARY);
            pv.uops.push_back(unary_ops().at(e.text));
            pv.left.push_back((int16_t)lreg);
            pv.right.push_back(UNARY_RIGHT_INDEX);
            pv.lscalars.push_back(junk_scalar());
            pv.rscalars.push_back(junk_scalar());
        }
        const int out = final_reg >= 0 ? final_reg : take();
        pv.outs.push_back((int16_t)out);
        return out;
    }
};

}  // namespace

std::unique_ptr<Expr> parse_expression(const std::string& text) {
    const std::string s = rewrite(text);
    Parser p(s);
    auto e = p.parse();
    p.ws();
    // the reference drops every ')' and ',' after the expression; tolerate stray ')'
    while (p.i < s.size() && (s[p.i] == ')' || s[p.i] == ' ')) p.i++;
    if (p.i != s.size()) throw ParseError("trailing text after expression: " + s.substr(p.i));
    normalise(e);
    return e;
}

void collect_columns(const Expr& e, std::vector<bool>& used) {
    if (e.kind == Expr::Column) {
        if (e.column < 0 || e.column >= (int)used.size()) throw ParseError("column reference out of range: " + e.text);
        used[e.column] = true;
        return;
    }
    for (const auto& a : e.args) collect_columns(*a, used);
}

void emit_expression(const Expr& e, int expression_position, int num_outputs, int num_inputs,
                     const std::vector<int>& new_input_indices, ProgramVectors& pv) {
    if (e.kind != Expr::Call) throw ParseError("expression has no operator");
    Emitter em(num_inputs + num_outputs, new_input_indices, pv);
    em.emit(e, num_inputs + expression_position);
}

static gdf_dtype out_type_rec(const Expr& e, const std::vector<gdf_dtype>& frame);

gdf_dtype expression_output_type(const Expr& e, const std::vector<gdf_dtype>& frame) { return out_type_rec(e, frame); }

static gdf_dtype out_type_rec(const Expr& e, const std::vector<gdf_dtype>& frame) {
    if (e.kind == Expr::Literal) return GDF_invalid;
    if (e.kind == Expr::Column) {
        if (e.column < 0 || e.column >= (int)frame.size()) throw ParseError("column reference out of range");
        return frame[e.column];
    }
    if (binary_ops().count(e.text)) {
        gdf_dtype l = out_type_rec(*e.args[0], frame);
        gdf_dtype r = out_type_rec(*e.args[1], frame);
        if (l == GDF_invalid) {
            if (r == GDF_invalid) throw ParseError("invalid operands");
            l = r;
        } else if (r == GDF_invalid) {
            r = l;
        }
        return result_type_binary(l, r, binary_ops().at(e.text));
    }
    return result_type_unary(out_type_rec(*e.args[0], frame), unary_ops().at(e.text));
}

bool contains_evaluation(const std::string& expr) {
    std::string s = expr;
    replace_all(s, "CAST(", "");
    replace_all(s, "):BIGINT", "");
    return s.find('(') != std::string::npos;
}

int column_reference_index(const std::string& expr) {
    std::string s = rewrite(expr);
    size_t a = s.find_first_not_of(' ');
    if (a == std::string::npos || s[a] != '$') throw ParseError("not a column reference: " + expr);
    size_t b = a + 1;
    while (b < s.size() && std::isdigit((unsigned char)s[b])) b++;
    if (b == a + 1) throw ParseError("not a column reference: " + expr);
    return std::atoi(s.substr(a + 1, b - a - 1).c_str());
}

std::string named_expression(const std::string& q, const std::string& name) {
    if (q.find(name + "=[") == std::string::npos) return "";
    size_t start;
    if (q.find(name + "=[[") != std::string::npos) start = q.find(name + "=[[") + 3 + name.size();
    else start = q.find(name + "=[") + 2 + name.size();
    size_t end = q.find(']', start);
    if (end == std::string::npos) return q.substr(start);
    return q.substr(start, end - start);
}

std::vector<std::pair<std::string, std::string>> project_expressions(const std::string& q) {
    const size_t open = q.find('(');
    const size_t close = q.rfind(')');
    if (open == std::string::npos || close == std::string::npos || close <= open)
        throw ParseError("not a LogicalProject: " + q);
    std::string all = q.substr(open + 1, close - open - 1);
    // get_expressions_from_expression_list's rewrites, CalciteExpressionParsing.cpp:818-830, in its
    // order: after the CASE(IS NOT NULL ...) -> COALESCE rewrite it drops every " NOT NULL", so an
    // IS NOT NULL left in a projection becomes the unknown operator "IS" and is rejected, as there
    all = std::regex_replace(all, coalesce_re(), "COALESCE($1, $2)");
    replace_all(all, " NOT NULL", "");
    std::vector<std::string> parts;
    int pd = 0, sd = 0;
    bool inq = false;
    size_t st = 0;
    for (size_t i = 0; i < all.size(); i++) {
        const char c = all[i];
        if (inq) {
            if (c == '\'' && !(i + 1 < all.size() && all[i + 1] == '\'')) inq = false;
            continue;
        }
        if (c == '\'') inq = true;
        else if (c == '(') pd++;
        else if (c == ')') pd--;
        else if (c == '[') sd++;
        else if (c == ']') sd--;
        else if (c == ',' && pd == 0 && sd == 0) {
            parts.push_back(all.substr(st, i - st));
            st = i + 1;
        }
    }
    if (st < all.size()) parts.push_back(all.substr(st));
    std::vector<std::pair<std::string, std::string>> out;
    for (auto& p : parts) {
        size_t a = p.find_first_not_of(' ');
        size_t b = p.find_last_not_of(' ');
        p = a == std::string::npos ? std::string() : p.substr(a, b - a + 1);
        const size_t eq = p.find("=[");
        if (eq == std::string::npos || p.empty() || p.back() != ']') throw ParseError("bad projection: " + p);
        out.emplace_back(p.substr(0, eq), p.substr(eq + 2, p.size() - eq - 3));
    }
    return out;
}

ExpressionPlan plan_expression(const std::string& expression, int n_frame) {
    ExpressionPlan ep;
    if (!expression.empty() && expression[0] == '$') {
        ep.clone = true;
        ep.clone_column = column_reference_index(expression);
        if (ep.clone_column < 0 || ep.clone_column >= n_frame) throw ParseError("column reference out of range");
        return ep;
    }
    auto e = parse_expression(expression);
    std::vector<bool> used(n_frame, false);
    collect_columns(*e, used);
    std::vector<int> remap(n_frame, -1);
    for (int c = 0; c < n_frame; c++)
        if (used[c]) { remap[c] = (int)ep.input_columns.size(); ep.input_columns.push_back(c); }
    const int n_in = (int)ep.input_columns.size();
    ep.pv.final_pos.push_back((int16_t)n_in);
    emit_expression(*e, 0, 1, n_in, remap, ep.pv);
    return ep;
}

ProjectPlan plan_project(const std::string& q, const std::vector<gdf_dtype>& frame) {
    ProjectPlan pp;
    const int n_frame = (int)frame.size();
    auto exprs = project_expressions(q);
    std::vector<std::unique_ptr<Expr>> trees(exprs.size());
    std::vector<bool> used(n_frame, false);
    int n_eval = 0;
    for (size_t i = 0; i < exprs.size(); i++) {
        pp.names.push_back(exprs[i].first);
        if (contains_evaluation(exprs[i].second)) {
            trees[i] = parse_expression(exprs[i].second);
            pp.eval_dtypes.push_back(expression_output_type(*trees[i], frame));
            collect_columns(*trees[i], used);
            n_eval++;
        }
    }
    std::vector<int> remap(n_frame, -1);
    for (int c = 0; c < n_frame; c++)
        if (used[c]) { remap[c] = (int)pp.input_columns.size(); pp.input_columns.push_back(c); }
    const int n_in = (int)pp.input_columns.size();
    for (int k = 0; k < n_eval; k++) pp.pv.final_pos.push_back((int16_t)(n_in + k));
    int k = 0;
    for (size_t i = 0; i < exprs.size(); i++) {
        if (trees[i]) {
            emit_expression(*trees[i], k, n_eval, n_in, remap, pp.pv);
            pp.columns.emplace_back(true, k);
            k++;
        } else {
            const int c = column_reference_index(exprs[i].second);
            if (c < 0 || c >= n_frame) throw ParseError("column reference out of range");
            pp.columns.emplace_back(false, c);
        }
    }
    return pp;
}

AggregatePlan plan_aggregate(const std::string& q, const std::vector<gdf_dtype>& frame) {
    AggregatePlan ap;
    const int n_frame = (int)frame.size();
    if (q.find("LogicalAggregate") == std::string::npos) throw ParseError("not a LogicalAggregate: " + q);
    auto exprs = project_expressions(q);
    std::vector<std::unique_ptr<Expr>> trees;
    std::vector<bool> used(n_frame, false);
    for (auto& [name, text] : exprs) {
        if (name == "group") {
            // group=[{0, 1}]: the GROUP BY columns (get_group_columns)
            for (size_t i = 0; i < text.size(); i++)
                if (std::isdigit((unsigned char)text[i])) {
                    size_t j = i;
                    while (j < text.size() && std::isdigit((unsigned char)text[j])) j++;
                    ap.group_columns.push_back(std::atoi(text.substr(i, j - i).c_str()));
                    i = j;
                }
            continue;
        }
        AggregatePlan::Aggregation a;
        a.name = name;
        const std::string op = text.substr(0, text.find('('));
        if (op == "SUM") a.op = GDF_SUM;
        else if (op == "MIN") a.op = GDF_MIN;
        else if (op == "MAX") a.op = GDF_MAX;
        else if (op == "AVG") a.op = GDF_AVG;
        else if (op == "COUNT") a.op = GDF_COUNT;
        else if (op == "COUNT_DISTINCT") throw ParseError("COUNT_DISTINCT is not supported without a group by");
        else throw ParseError("aggregation type not supported: " + op);
        const size_t open = text.find('('), close = text.rfind(')');
        const std::string input = (open == std::string::npos || close == std::string::npos || close < open)
                                      ? std::string()
                                      : text.substr(open + 1, close - open - 1);
        if (contains_evaluation(input)) {
            trees.push_back(parse_expression(input));
            ap.eval_dtypes.push_back(expression_output_type(*trees.back(), frame));
            collect_columns(*trees.back(), used);
            a.evaluated = true;
            a.index = (int)trees.size() - 1;
        } else {
            bool blank = true;
            for (char c : input) blank = blank && c == ' ';
            a.index = blank ? 0 : column_reference_index(input);
            if (a.index < 0 || a.index >= n_frame) throw ParseError("column reference out of range");
        }
        ap.aggregations.push_back(a);
    }
    std::vector<int> remap(n_frame, -1);
    for (int c = 0; c < n_frame; c++)
        if (used[c]) { remap[c] = (int)ap.input_columns.size(); ap.input_columns.push_back(c); }
    const int n_in = (int)ap.input_columns.size();
    const int n_eval = (int)trees.size();
    for (int k = 0; k < n_eval; k++) ap.pv.final_pos.push_back((int16_t)(n_in + k));
    for (int k = 0; k < n_eval; k++) emit_expression(*trees[k], k, n_eval, n_in, remap, ap.pv);
    return ap;
}

}  // namespace ral
