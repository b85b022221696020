// codegen.cpp — emits one CUDA kernel per register program.
#include "codegen.h"

#include <algorithm>
#include <functional>
#include <cstdlib>
#include <sstream>
#include <stdexcept>

namespace ral {

const char* element_ctype(gdf_dtype t) {
    switch (t) {
    case GDF_INT8: case GDF_BOOL8: return "signed char";
    case GDF_INT16: return "short";
    case GDF_INT32: case GDF_DATE32: case GDF_CATEGORY: case GDF_STRING_CATEGORY: return "int";
    case GDF_INT64: case GDF_DATE64: case GDF_TIMESTAMP: return "long long";
    case GDF_FLOAT32: return "float";
    case GDF_FLOAT64: return "double";
    default: throw std::runtime_error("no element type for dtype");
    }
}

static Kind dtype_kind(gdf_dtype t) { return dtype_is_float(t) ? Kind::F64 : Kind::I64; }
static const char* kind_ctype(Kind k) { return k == Kind::F64 ? "double" : "ral_i64"; }

int max_width(const Program& p) {
    int w = 1;
    auto ref = p.inputs_referenced();
    for (int c = 0; c < p.n_in; c++)
        if (ref[c]) w = std::max(w, gdf_dtype_size(p.inputs[c].dtype));
    for (int o = 0; o < p.n_out; o++) w = std::max(w, gdf_dtype_size(p.out_dtypes[o]));
    return w;
}

Shape default_shape(const Program& p) {
    Shape s;
    s.G = 16 / max_width(p);
    s.J = std::max(1, 4 / s.G);
    // 32 resident warps (at most 64 registers a thread): the latency of the loads and of the
    // integer-pipe double operations is hidden by more warps, not by more registers.  As two
    // blocks of 512 threads rather than four of 256: the 12-op projection over 200M rows ran
    // 2.554 ms against 2.663 (same registers, same warps per SM; 20M rows: 274 against 281 us).
    s.threads = 512;
    s.min_blocks = 2;
    return s;
}

void apply_shape_tune(Shape& sh, const std::string& t) {
    size_t i = 0;
    while (i < t.size()) {
        size_t e = t.find(',', i);
        if (e == std::string::npos) e = t.size();
        const std::string kv = t.substr(i, e - i);
        const size_t eq = kv.find('=');
        if (eq != std::string::npos) {
            const std::string k = kv.substr(0, eq);
            const int v = std::atoi(kv.c_str() + eq + 1);
            if (k == "J" && v >= 1 && v * sh.G <= 2048) sh.J = v;
            else if (k == "U" && v >= 1 && v <= 64) sh.unroll = v;
            else if (k == "T" && (v == 128 || v == 256 || v == 512)) sh.threads = v;
            else if (k == "B" && v >= 1 && v <= 16) sh.min_blocks = v;
            else if (k == "S") sh.stage = v != 0;
            else if (k == "P" && v >= 0 && v <= 64) sh.prefetch = v;
            else if (k == "D" && v >= -1 && v <= 1) sh.dense = v;
            else if (k == "K" && v >= 1 && v <= 2) sh.dense_unroll = v;
            else if (k == "M" && v >= 0 && v <= 8 && v != 1) sh.tma_stages = v;
            else if (k == "R" && v >= 0 && v <= 64) sh.grid_k = v;
        }
        i = e + 1;
    }
}

namespace {

std::string conv(const std::string& x, Kind from, Kind to) {
    if (from == to) return x;
    if (from == Kind::I64) return "ral_i2d(" + x + ")";
    return "ral_d2i(" + x + ")";
}
std::string to_d(const std::string& x, Kind k) { return conv(x, k, Kind::F64); }
std::string to_i(const std::string& x, Kind k) { return conv(x, k, Kind::I64); }
std::string conv_bool(const std::string& b, Kind to) {
    return to == Kind::F64 ? "ral_b2d(" + b + ")" : "((ral_i64)(" + b + "))";
}

// Data-path op emission shared by every kernel kind.
struct OpEmitter {
    const Program& p;
    const ParamLayout& L;
    std::vector<std::string> name;   // current SSA value of each register
    std::vector<Kind> kind;
    // registers whose current value is 0 or 1 (comparisons, NOT, IS [NOT] NULL, products of two
    // such): converted to double by a select, and a double product with one skips the multiply
    std::vector<bool> b01;
    // ABS results not yet emitted: the operand's expression.  A double add, subtract or multiply
    // reads fabs(operand), which the compiler folds into the instruction as a free modifier; any
    // other reader (a stored output, a comparison, a division) gets the integer-pipe version,
    // emitted once where first needed.
    std::vector<std::string> absrc;

    // integer division / remainder by a column take the divisors' reciprocals from the kernel's
    // shared table (ral_rcp_of; eval kernels of such programs declare and fill it)
    bool rcp = false;

    OpEmitter(const Program& prog, const ParamLayout& layout) : p(prog), L(layout) {
        int maxreg = p.n_in;
        for (const Op& op : p.ops) maxreg = std::max<int>(maxreg, op.out);
        for (int16_t f : p.final_pos) maxreg = std::max<int>(maxreg, f);
        name.assign(maxreg + 1, "");
        kind.assign(maxreg + 1, Kind::I64);
        b01.assign(maxreg + 1, false);
        absrc.assign(maxreg + 1, "");
        for (int c = 0; c < p.n_in; c++) {
            name[c] = "x" + std::to_string(c);
            kind[c] = dtype_kind(p.inputs[c].dtype);
        }
    }

    // Emits the statements of every op; afterwards name[] holds the final values.
    void emit(std::ostream& os, const std::string& indent) {
        for (size_t k = 0; k < p.ops.size(); k++) {
            const Op& op = p.ops[k];
            std::string l, r;
            Kind lk = op.lk, rk = op.rk;
            const bool l01 = op.left >= 0 && b01[op.left];
            const bool r01 = !op.unary && op.right >= 0 && b01[op.right];
            // operands a deferred ABS may reach as fabs(): double add / subtract / multiply
            // (not a multiply by a 0/1 value, which is integer work)
            const bool farith = !op.unary && (lk == Kind::F64 || rk == Kind::F64) &&
                                (op.bop == GDF_ADD || op.bop == GDF_SUB || (op.bop == GDF_MUL && l01 == r01));
            auto fetch = [&](int reg, bool fold) -> std::string {
                if (!absrc[reg].empty()) {
                    if (fold) return "fabs(" + absrc[reg] + ")";
                    const std::string t = "ta" + std::to_string(k) + "_" + std::to_string(reg);
                    os << indent << "const double " << t << " = ral_dfabs(" << absrc[reg] << ");\n";
                    name[reg] = t;
                    absrc[reg].clear();
                }
                return name[reg];
            };
            const bool abs_op = op.unary && op.uop == BLZ_ABS && op.left >= 0 && lk == Kind::F64 && op.ok == Kind::F64;
            if (op.left >= 0) {
                l = fetch(op.left, (farith && lk == Kind::F64) || abs_op);
            } else if (op.left == SCALAR_INDEX) {
                l = "sl" + std::to_string(k);
                os << indent << "const " << kind_ctype(lk) << " " << l << " = "
                   << (lk == Kind::F64 ? "ral_bits_d((ral_i64)P.s[" : "((ral_i64)P.s[") << L.lscalar_slot[k]
                   << "]);\n";
            } else {
                l = lk == Kind::F64 ? "0.0" : "((ral_i64)0)";
            }
            if (abs_op) {  // deferred: see absrc
                absrc[op.out] = l;
                name[op.out].clear();
                kind[op.out] = Kind::F64;
                b01[op.out] = false;
                continue;
            }
            if (!op.unary) {
                if (op.right >= 0) {
                    r = fetch(op.right, farith && rk == Kind::F64);
                } else if (op.right == SCALAR_INDEX) {
                    r = "sr" + std::to_string(k);
                    os << indent << "const " << kind_ctype(rk) << " " << r << " = "
                       << (rk == Kind::F64 ? "ral_bits_d((ral_i64)P.s[" : "((ral_i64)P.s[")
                       << L.rscalar_slot[k] << "]);\n";
                } else {
                    r = rk == Kind::F64 ? "0.0" : "((ral_i64)0)";
                }
            }
            const Kind ok = op.ok;
            std::string e;
            bool res01 = false;
            if (!op.unary) {
                const bool f = (lk == Kind::F64) || (rk == Kind::F64);
                // a 0/1 operand as a double, and as a truth value
                auto d01 = [&](const std::string& v, Kind k) {
                    return k == Kind::I64 ? "ral_b2d((" + v + ") != 0)" : v;
                };
                auto t01 = [&](const std::string& v, Kind k) {
                    return k == Kind::I64 ? "((" + v + ") != 0)" : "(!ral_dzero(" + v + "))";
                };
                // the precomputed multiplier and shift of a literal integer divisor
                auto divider = [&](size_t j) {
                    const std::string m = std::to_string(L.rdiv_slot[j]);
                    return "(ral_i64)P.s[" + m + "], (ral_i64)P.s[" + m + " + 1]";
                };
                const std::string ld = l01 ? d01(l, lk) : to_d(l, lk);
                const std::string rd = r01 ? d01(r, rk) : to_d(r, rk);
                auto arith = [&](const char* dop, const char* iop) {
                    if (f) return conv(std::string(dop) + "(" + ld + ", " + rd + ")", Kind::F64, ok);
                    return conv(std::string(iop) + "(" + l + ", " + r + ")", Kind::I64, ok);
                };
                // double comparisons go through the prelude's ral_d* functions (integer-pipe
                // versions unless RAL_SOFT_FP is 0)
                auto cmp = [&](const char* c, const char* dfn) {
                    res01 = true;
                    if (f) return conv_bool(std::string(dfn) + "(" + ld + ", " + rd + ")", ok);
                    return conv_bool(l + " " + c + " " + r, ok);
                };
                switch (op.bop) {
                case GDF_ADD: e = arith("__dadd_rn", "ral_addi"); break;
                case GDF_SUB: e = arith("__dsub_rn", "ral_subi"); break;
                case GDF_MUL:
                    if (f && l01 && !r01) e = conv("ral_dmul01(" + t01(l, lk) + ", " + rd + ")", Kind::F64, ok);
                    else if (f && r01 && !l01) e = conv("ral_dmul01(" + t01(r, rk) + ", " + ld + ")", Kind::F64, ok);
                    else e = arith("__dmul_rn", "ral_muli");
                    res01 = l01 && r01;
                    break;
                case GDF_DIV: case GDF_FLOOR_DIV:
                    if (L.rdiv_slot.size() > k && L.rdiv_slot[k] >= 0)
                        e = conv("ral_sf_divc(" + l + ", " + r + ", " + divider(k) + ")", Kind::I64, ok);
                    else if (rcp && !f && op.right >= 0)
                        e = conv("ral_divi_m(" + l + ", " + r + ", ral_rcp_of(" + r + "))", Kind::I64, ok);
                    else
                        e = arith("ral_ddiv", "ral_divi");
                    break;
                case GDF_MOD:
                    if (L.rdiv_slot.size() > k && L.rdiv_slot[k] >= 0)
                        e = conv("ral_sf_modc(" + to_i(l, lk) + ", " + r + ", " + divider(k) + ")", Kind::I64, ok);
                    else if (rcp && op.right >= 0)
                        e = conv("ral_modi_m(" + to_i(l, lk) + ", " + to_i(r, rk) + ", ral_rcp_of(" + to_i(r, rk) + "))", Kind::I64, ok);
                    else
                        e = conv("ral_modi(" + to_i(l, lk) + ", " + to_i(r, rk) + ")", Kind::I64, ok);
                    break;
                case GDF_POW:
                    if (dtype_is_float(op.ltype) || dtype_is_float(op.rtype))
                        e = conv("pow(" + to_d(l, lk) + ", " + to_d(r, rk) + ")", Kind::F64, ok);
                    else
                        e = conv("ral_powi(" + l + ", " + r + ")", Kind::I64, ok);
                    break;
                case GDF_EQUAL: e = cmp("==", "ral_deq"); break;
                case GDF_NOT_EQUAL: e = cmp("!=", "ral_dne"); break;
                case GDF_LESS: e = cmp("<", "ral_dlt"); break;
                case GDF_GREATER: e = cmp(">", "ral_dgt"); break;
                case GDF_LESS_EQUAL: e = cmp("<=", "ral_dle"); break;
                case GDF_GREATER_EQUAL: e = cmp(">=", "ral_dge"); break;
                case GDF_COALESCE:
                    e = "(rb" + std::to_string(op.left) + " ? " + conv(l, lk, ok) + " : " + conv(r, rk, ok) + ")";
                    break;
                default: throw std::runtime_error("codegen: unsupported binary operator");
                }
            } else {
                const std::string d = l01 && lk == Kind::I64 ? "ral_b2d((" + l + ") != 0)" : to_d(l, lk);
                const bool d32 = op.ltype == GDF_DATE32;
                auto math = [&](const std::string& fn) { return conv(fn + "(" + d + ")", Kind::F64, ok); };
                switch (op.uop) {
                case BLZ_FLOOR: e = math("ral_dfloor"); break;
                case BLZ_CEIL: e = math("ral_dceil"); break;
                case BLZ_SIN: e = math("ral_dsin"); break;
                case BLZ_COS: e = math("ral_dcos"); break;
                case BLZ_ASIN: e = math("asin"); break;
                case BLZ_ACOS: e = math("acos"); break;
                case BLZ_TAN: e = math("tan"); break;
                case BLZ_COTAN: e = conv("ral_ddiv(ral_dcos(" + d + "), ral_dsin(" + d + "))", Kind::F64, ok); break;
                case BLZ_ATAN: e = math("atan"); break;
                case BLZ_ABS: e = math("ral_dfabs"); break;
                case BLZ_LN: e = math("log"); break;
                case BLZ_LOG: e = math("log10"); break;
                case BLZ_NOT: e = conv_bool(lk == Kind::F64 ? "ral_dzero(" + l + ")" : "(" + l + " == 0)", ok); res01 = true; break;
                case BLZ_YEAR: e = conv(std::string(d32 ? "ral_year32(" : "ral_year64(") + to_i(l, lk) + ")", Kind::I64, ok); break;
                case BLZ_MONTH: e = conv(std::string(d32 ? "ral_month32(" : "ral_month64(") + to_i(l, lk) + ")", Kind::I64, ok); break;
                case BLZ_DAY: e = conv(std::string(d32 ? "ral_day32(" : "ral_day64(") + to_i(l, lk) + ")", Kind::I64, ok); break;
                case BLZ_HOUR: e = d32 ? conv("((ral_i64)0)", Kind::I64, ok) : conv("ral_hour64(" + to_i(l, lk) + ")", Kind::I64, ok); break;
                case BLZ_MINUTE: e = d32 ? conv("((ral_i64)0)", Kind::I64, ok) : conv("ral_minute64(" + to_i(l, lk) + ")", Kind::I64, ok); break;
                case BLZ_SECOND: e = d32 ? conv("((ral_i64)0)", Kind::I64, ok) : conv("ral_second64(" + to_i(l, lk) + ")", Kind::I64, ok); break;
                case BLZ_IS_NULL: e = conv_bool("rb" + std::to_string(op.left) + " == 0u", ok); res01 = true; break;
                case BLZ_IS_NOT_NULL: e = conv_bool("rb" + std::to_string(op.left) + " != 0u", ok); res01 = true; break;
                default: e = conv(l, lk, ok); res01 = l01; break;  // copy with conversion
                }
            }
            const std::string t = "t" + std::to_string(k);
            os << indent << "const " << kind_ctype(ok) << " " << t << " = " << e << ";\n";
            name[op.out] = t;
            kind[op.out] = ok;
            b01[op.out] = res01;
            absrc[op.out].clear();
        }
        // deferred ABS values that are outputs of the program
        for (int16_t f : p.final_pos) {
            if (f < 0 || absrc[f].empty()) continue;
            const std::string t = "tf" + std::to_string(f);
            os << indent << "const double " << t << " = ral_dfabs(" << absrc[f] << ");\n";
            name[f] = t;
            absrc[f].clear();
        }
    }
};

// Validity-word emission: 32 rows per word, the same AND/OR over registers as
// the reference's 64-row pass (interpreter_ops.cuh:508-571).
struct ValidEmitter {
    const Program& p;
    std::vector<std::string> name;
    explicit ValidEmitter(const Program& prog) : p(prog) {
        int maxreg = p.n_in;
        for (const Op& op : p.ops) maxreg = std::max<int>(maxreg, op.out);
        for (int16_t f : p.final_pos) maxreg = std::max<int>(maxreg, f);
        name.assign(maxreg + 1, "0xffffffffu");
    }
    bool loads(int c) const {
        return p.inputs[c].has_valid && p.inputs[c].nulls_possible && !p.force_valid[c];
    }
    void emit(std::ostream& os, const std::string& indent, const std::function<std::string(int)>& word_of_input) {
        auto ref = p.inputs_referenced();
        for (int c = 0; c < p.n_in; c++) {
            if (!ref[c]) continue;
            if (loads(c)) {
                name[c] = "vw" + std::to_string(c);
                os << indent << "const ral_u32 " << name[c] << " = " << word_of_input(c) << ";\n";
            } else {
                name[c] = "0xffffffffu";
            }
        }
        for (size_t k = 0; k < p.ops.size(); k++) {
            const Op& op = p.ops[k];
            auto operand = [&](int idx) -> std::string {
                if (idx >= 0) return name[idx];
                return idx == SCALAR_NULL_INDEX ? "0u" : "0xffffffffu";
            };
            std::string e;
            if (op.unary) e = operand(op.left);
            else if (op.bop == GDF_COALESCE) e = "(" + operand(op.left) + " | " + operand(op.right) + ")";
            else e = "(" + operand(op.left) + " & " + operand(op.right) + ")";
            const std::string t = "vt" + std::to_string(k);
            os << indent << "const ral_u32 " << t << " = " << e << ";\n";
            name[op.out] = t;
        }
    }
};

std::string widen(const std::string& x, gdf_dtype t) {
    if (t == GDF_FLOAT32) return "ral_f2d(" + x + ")";
    return dtype_is_float(t) ? "((double)(" + x + "))" : "((ral_i64)(" + x + "))";
}

// Register value -> column element, as write_data does it (interpreter_ops.cuh:317-381):
// integer columns take the slot's int64 bits, float columns its double bits.
std::string narrow(const std::string& v, Kind k, gdf_dtype t) {
    const std::string et = element_ctype(t);
    if (dtype_is_float(t)) {
        std::string d = k == Kind::F64 ? v : "ral_bits_d(" + v + ")";
        if (t == GDF_FLOAT32) return "ral_d2f(" + d + ")";
        return d;
    }
    std::string bits = k == Kind::I64 ? v : "ral_d_bits(" + v + ")";
    return "((" + et + ")(" + bits + "))";
}

uint64_t fnv1a(const std::string& s) {
    uint64_t h = 1469598103934665603ull;
    for (unsigned char c : s) { h ^= c; h *= 1099511628211ull; }
    return h;
}

ParamLayout make_layout(const Program& p, int extra_slots_before_scalars) {
    ParamLayout L;
    int s = 0;
    L.n_rows = s++;
    L.in_data = s; s += p.n_in;
    L.in_valid = s; s += p.n_in;
    L.out_data = s; s += p.n_out;
    L.out_valid = s; s += p.n_out;
    L.counts = s++;
    s += extra_slots_before_scalars;
    assign_scalar_slots(p, L, s);
    L.total = s;
    return L;
}


// The row function: one row through the program, typed registers in, final
// register values out.
void emit_row_function(std::ostream& os, const Program& p, const ParamLayout& L, const char* fname,
                       bool rcp = false) {
    auto ref = p.inputs_referenced();
    auto raw = p.inputs_raw_valid();
    os << "RAL_FI void " << fname << "(const RalParams& P";
    for (int c = 0; c < p.n_in; c++)
        if (ref[c]) os << ", const " << kind_ctype(dtype_kind(p.inputs[c].dtype)) << " x" << c;
    for (int c = 0; c < p.n_in; c++)
        if (raw[c]) os << ", const ral_u32 rb" << c;
    OpEmitter em(p, L);
    em.rcp = rcp;
    std::ostringstream body;
    em.emit(body, "    ");
    for (int o = 0; o < p.n_out; o++) os << ", " << kind_ctype(em.kind[p.final_pos[o]]) << "& y" << o;
    os << ") {\n" << body.str();
    for (int o = 0; o < p.n_out; o++) os << "    y" << o << " = " << em.name[p.final_pos[o]] << ";\n";
    os << "}\n";
}

// Whether a program divides integers by a column (its eval kernel then keeps a reciprocal table).
bool divides_by_column(const Program& p) {
    for (const Op& op : p.ops) {
        if (op.unary || op.right < 0) continue;
        if (op.bop == GDF_MOD) return true;
        if ((op.bop == GDF_DIV || op.bop == GDF_FLOOR_DIV) && op.lk == Kind::I64 && op.rk == Kind::I64) return true;
    }
    return false;
}

std::vector<Kind> final_kinds(const Program& p, const ParamLayout& L) {
    OpEmitter em(p, L);
    std::ostringstream sink;
    em.emit(sink, "");
    std::vector<Kind> k;
    for (int o = 0; o < p.n_out; o++) k.push_back(em.kind[p.final_pos[o]]);
    return k;
}

}  // namespace

bool divides_by_int_literal(const Op& op) {
    if (op.unary || op.right != SCALAR_INDEX || op.rk != Kind::I64) return false;
    if (op.bop == GDF_MOD) return true;  // both operands are taken as int64
    return (op.bop == GDF_DIV || op.bop == GDF_FLOOR_DIV) && op.lk == Kind::I64;
}

void assign_scalar_slots(const Program& p, ParamLayout& L, int& slot) {
    L.lscalar_slot.assign(p.ops.size(), -1);
    L.rscalar_slot.assign(p.ops.size(), -1);
    L.rdiv_slot.assign(p.ops.size(), -1);
    for (size_t k = 0; k < p.ops.size(); k++) {
        if (p.ops[k].left == SCALAR_INDEX) L.lscalar_slot[k] = slot++;
        if (!p.ops[k].unary && p.ops[k].right == SCALAR_INDEX) L.rscalar_slot[k] = slot++;
        if (divides_by_int_literal(p.ops[k])) {
            L.rdiv_slot[k] = slot;
            slot += 2;
        }
    }
}

namespace {

// Layout of one stage of a staged eval kernel: every referenced input's tile, then the masks the
// kernel reads (validity pass or raw bits), each region a multiple of 16 bytes.
struct StageLayout {
    std::vector<int> data_off, mask_off;  // -1: not staged
    int bytes = 0;
    bool masks_staged = false;
};

StageLayout stage_layout(const Program& p, const Shape& s) {
    StageLayout st;
    const int64_t tile = (int64_t)32 * s.G * s.J;
    const auto ref = p.inputs_referenced();
    const auto raw = p.inputs_raw_valid();
    ValidEmitter ve(p);
    st.data_off.assign(p.n_in, -1);
    st.mask_off.assign(p.n_in, -1);
    int off = 0;
    for (int c = 0; c < p.n_in; c++) {
        if (!ref[c]) continue;
        const int64_t b = tile * gdf_dtype_size(p.inputs[c].dtype);
        if (b % 16) return StageLayout{};
        st.data_off[c] = off;
        off += (int)b;
    }
    // masks: 4 bytes per 32 rows; a multiple of 16 bytes when the tile is a multiple of 128 rows
    st.masks_staged = tile % 128 == 0;
    if (st.masks_staged)
        for (int c = 0; c < p.n_in; c++)
            if (p.inputs[c].has_valid && ((ref[c] && ve.loads(c)) || raw[c])) {
                st.mask_off[c] = off;
                off += (int)(tile / 8);
            }
    st.bytes = off;
    return st;
}

}  // namespace

int eval_stage_bytes_per_warp(const Program& p, const Shape& s) {
    if (s.tma_stages < 2) return 0;
    const StageLayout st = stage_layout(p, s);
    if (st.bytes == 0) return 0;
    return 128 + s.tma_stages * st.bytes;  // barriers padded to 128 bytes, then the stages
}

GeneratedKernel generate_eval_kernel(const Program& p, const Shape& s) {
    GeneratedKernel gk;
    gk.shape = s;
    const int warp_smem = eval_stage_bytes_per_warp(p, s);
    gk.layout = make_layout(p, warp_smem > 0 ? 1 : 0);  // staged kernels: an error word
    const ParamLayout& L = gk.layout;
    const auto ref = p.inputs_referenced();
    const auto raw = p.inputs_raw_valid();
    const auto fk = final_kinds(p, L);
    std::vector<int> vouts;  // outputs that carry a valid mask
    for (int o = 0; o < p.n_out; o++)
        if (p.out_has_valid[o]) vouts.push_back(o);
    const int NOV = (int)vouts.size();

    const bool staged = warp_smem > 0;
    const StageLayout SL = staged ? stage_layout(p, s) : StageLayout{};
    std::ostringstream key;
    key << "eval|" << p.structure_key() << "|G" << s.G << "J" << s.J << "T" << s.threads << "B" << s.min_blocks;
    if (staged) key << "M" << s.tma_stages;
    char hex[32];
    snprintf(hex, sizeof hex, "%016llx", (unsigned long long)fnv1a(key.str()));
    gk.name = std::string("ral_eval_") + hex;

    std::ostringstream os;
    os << "// generated: " << key.str() << "\n";
    os << "#define RAL_G " << s.G << "\n#define RAL_J " << s.J << "\n#define RAL_THREADS " << s.threads << "\n";
    os << "struct RalParams { ral_u64 s[" << L.total << "]; };\n\n";
    const bool rcp = divides_by_column(p);
    if (rcp) {
        os << "__shared__ unsigned ral_rcp_tab[RAL_RCP_TAB];\n";
        os << "RAL_FI unsigned ral_rcp_of(ral_i64 b) {\n"
              "    const ral_u64 ub = b < 0 ? 0ull - (ral_u64)b : (ral_u64)b;\n"
              "    return ub < RAL_RCP_TAB ? ral_rcp_tab[ub] : 0u;\n}\n";
    }
    emit_row_function(os, p, L, "ral_row", rcp);

    // validity word function
    if (NOV > 0) {
        os << "RAL_FI void ral_vword(const RalParams& P, const ral_i64 w, ral_u32* vo) {\n";
        ValidEmitter ve(p);
        ve.emit(os, "    ", [&](int c) {
            return "__ldg(((const ral_u32*)P.s[" + std::to_string(L.in_valid + c) + "]) + w)";
        });
        for (int i = 0; i < NOV; i++) os << "    vo[" << i << "] = " << ve.name[p.final_pos[vouts[i]]] << ";\n";
        os << "}\n";
    }

    os << "\nextern \"C\" __global__ void __launch_bounds__(RAL_THREADS, " << s.min_blocks << ") " << gk.name
       << "(const __grid_constant__ RalParams P) {\n";
    os << "    const ral_i64 n = (ral_i64)P.s[" << L.n_rows << "];\n";
    if (rcp) {
        os << "    for (int i = threadIdx.x; i < RAL_RCP_TAB; i += RAL_THREADS) ral_rcp_tab[i] = i ? 0xffffffffu / (unsigned)i : 0u;\n";
        os << "    __syncthreads();\n";
    }
    for (int c = 0; c < p.n_in; c++) {
        if (ref[c])
            os << "    const " << element_ctype(p.inputs[c].dtype) << "* __restrict__ pin" << c << " = (const "
               << element_ctype(p.inputs[c].dtype) << "*)P.s[" << L.in_data + c << "];\n";
        if (raw[c] && p.inputs[c].has_valid)
            os << "    const ral_u32* __restrict__ pvr" << c << " = (const ral_u32*)P.s[" << L.in_valid + c << "];\n";
    }
    for (int o = 0; o < p.n_out; o++) {
        os << "    " << element_ctype(p.out_dtypes[o]) << "* __restrict__ pout" << o << " = ("
           << element_ctype(p.out_dtypes[o]) << "*)P.s[" << L.out_data + o << "];\n";
    }
    for (int i = 0; i < NOV; i++)
        os << "    ral_u32* __restrict__ pvo" << i << " = (ral_u32*)P.s[" << L.out_valid + vouts[i] << "];\n";
    os << "    const int lane = threadIdx.x & 31;\n";
    os << "    const ral_i64 gwarp = ((ral_i64)blockIdx.x * RAL_THREADS + threadIdx.x) >> 5;\n";
    os << "    const ral_i64 nwarp = ((ral_i64)gridDim.x * RAL_THREADS) >> 5;\n";
    os << "    const ral_i64 TILE = 32 * RAL_G * RAL_J;\n";
    os << "    const ral_i64 ntiles = n / TILE;\n";
    if (NOV > 0) os << "    ral_u64 vcnt[" << NOV << "];\n    for (int i = 0; i < " << NOV << "; ++i) vcnt[i] = 0;\n";

    // full tiles
    if (staged) {
        // per warp: S barriers (128 bytes), then S stages; lane 0 fills a stage with one bulk copy per
        // staged column / mask of the tile and the warp waits on the stage's barrier
        const int S = s.tma_stages;
        os << "    extern __shared__ __align__(128) unsigned char ral_smem[];\n";
        os << "    const int RAL_S = " << S << ", STAGE = " << SL.bytes << ", WARP_SMEM = " << warp_smem << ";\n";
        os << "    unsigned char* wsm = ral_smem + (threadIdx.x >> 5) * WARP_SMEM;\n";
        os << "    ral_u64* bars = (ral_u64*)wsm;\n";
        os << "    unsigned char* stages = wsm + 128;\n";
        os << "    ral_u64* err = (ral_u64*)P.s[" << L.counts << " + 1];\n";
        os << "    if (lane == 0) { for (int q = 0; q < RAL_S; ++q) ral_mbar_init(bars + q, 1); ral_mbar_init_fence(); }\n";
        os << "    __syncwarp();\n";
        os << "    auto fill = [&](int q, ral_i64 t) {\n";
        os << "        unsigned char* st = stages + q * STAGE;\n";
        os << "        ral_mbar_expect_tx(bars + q, STAGE);\n";
        for (int c = 0; c < p.n_in; c++) {
            if (SL.data_off[c] >= 0) {
                const int w = gdf_dtype_size(p.inputs[c].dtype);
                os << "        ral_bulk_g2s(st + " << SL.data_off[c] << ", pin" << c << " + t * TILE, (unsigned)(TILE * " << w
                   << "), bars + q);\n";
            }
            if (SL.mask_off[c] >= 0)
                os << "        ral_bulk_g2s(st + " << SL.mask_off[c] << ", ((const ral_u32*)P.s[" << L.in_valid + c
                   << "]) + t * (TILE / 32), (unsigned)(TILE / 8), bars + q);\n";
        }
        os << "    };\n";
        os << "    if (lane == 0)\n";
        os << "        for (int q = 0; q < RAL_S; ++q)\n";
        os << "            if (gwarp + (ral_i64)q * nwarp < ntiles) fill(q, gwarp + (ral_i64)q * nwarp);\n";
        os << "    bool ok = true;\n";
        os << "    long k = 0;\n";
        os << "    for (ral_i64 t = gwarp; t < ntiles; t += nwarp, ++k) {\n";
        os << "        const int q = (int)(k % RAL_S);\n";
        os << "        if (!ral_mbar_wait(bars + q, (unsigned)((k / RAL_S) & 1))) { ok = false; break; }\n";
        os << "        const unsigned char* st = stages + q * STAGE;\n";
        os << "        const ral_i64 base = t * TILE;\n";
        os << "#pragma unroll\n";
        os << "        for (int j = 0; j < RAL_J; ++j) {\n";
        os << "            const int lr = j * 32 * RAL_G + lane * RAL_G;\n";
        os << "            const ral_i64 r = base + lr;\n";
        for (int c = 0; c < p.n_in; c++) {
            if (!ref[c]) continue;
            const char* et = element_ctype(p.inputs[c].dtype);
            os << "            " << et << " a" << c << "[RAL_G]; ral_lds<" << et << ", RAL_G>((const " << et << "*)(st + "
               << SL.data_off[c] << "), lr, a" << c << ");\n";
        }
        for (int c = 0; c < p.n_in; c++) {
            if (!raw[c]) continue;
            if (p.inputs[c].has_valid && SL.mask_off[c] >= 0)
                os << "            const ral_u32 rw" << c << " = ((const ral_u32*)(st + " << SL.mask_off[c] << "))[lr >> 5];\n";
            else if (p.inputs[c].has_valid)
                os << "            const ral_u32 rw" << c << " = __ldg(pvr" << c << " + (r >> 5));\n";
            else
                os << "            const ral_u32 rw" << c << " = 0xffffffffu;\n";
        }
    } else {
    os << "    for (ral_i64 t = gwarp; t < ntiles; t += nwarp) {\n";
    os << "        const ral_i64 base = t * TILE;\n";
    os << "#pragma unroll\n";
    os << "        for (int j = 0; j < RAL_J; ++j) {\n";
    os << "            const ral_i64 r = base + (ral_i64)j * 32 * RAL_G + lane * RAL_G;\n";
    for (int c = 0; c < p.n_in; c++) {
        if (!ref[c]) continue;
        const char* et = element_ctype(p.inputs[c].dtype);
        os << "            " << et << " a" << c << "[RAL_G]; ral_ldg<" << et << ", RAL_G>(pin" << c << ", r, a" << c << ");\n";
    }
    for (int c = 0; c < p.n_in; c++) {
        if (!raw[c]) continue;
        if (p.inputs[c].has_valid) os << "            const ral_u32 rw" << c << " = __ldg(pvr" << c << " + (r >> 5));\n";
        else os << "            const ral_u32 rw" << c << " = 0xffffffffu;\n";
    }
    }
    for (int o = 0; o < p.n_out; o++)
        os << "            " << element_ctype(p.out_dtypes[o]) << " b" << o << "[RAL_G];\n";
    os << "#pragma unroll\n";
    os << "            for (int g = 0; g < RAL_G; ++g) {\n";
    for (int o = 0; o < p.n_out; o++) os << "                " << kind_ctype(fk[o]) << " y" << o << ";\n";
    os << "                ral_row(P";
    for (int c = 0; c < p.n_in; c++)
        if (ref[c]) os << ", " << widen("a" + std::to_string(c) + "[g]", p.inputs[c].dtype);
    for (int c = 0; c < p.n_in; c++)
        if (raw[c]) os << ", (rw" << c << " >> ((int)(r & 31) + g)) & 1u";
    for (int o = 0; o < p.n_out; o++) os << ", y" << o;
    os << ");\n";
    for (int o = 0; o < p.n_out; o++)
        os << "                b" << o << "[g] = " << narrow("y" + std::to_string(o), fk[o], p.out_dtypes[o]) << ";\n";
    os << "            }\n";
    for (int o = 0; o < p.n_out; o++)
        os << "            ral_stg<" << element_ctype(p.out_dtypes[o]) << ", RAL_G>(pout" << o << ", r, b" << o << ");\n";
    os << "        }\n";
    if (NOV > 0) {
        os << "        for (int wl = lane; wl < RAL_G * RAL_J; wl += 32) {\n";
        os << "            const ral_i64 w = (base >> 5) + wl;\n";
        if (staged && SL.masks_staged) {
            // the validity pass over the staged mask words of the tile
            os << "            ral_u32 vo[" << NOV << "];\n";
            os << "            {\n";
            ValidEmitter ve(p);
            std::ostringstream vb;
            ve.emit(vb, "                ", [&](int c) {
                if (SL.mask_off[c] >= 0) return "((const ral_u32*)(st + " + std::to_string(SL.mask_off[c]) + "))[wl]";
                return "__ldg(((const ral_u32*)P.s[" + std::to_string(L.in_valid + c) + "]) + w)";
            });
            os << vb.str();
            for (int i = 0; i < NOV; i++) os << "                vo[" << i << "] = " << ve.name[p.final_pos[vouts[i]]] << ";\n";
            os << "            }\n";
        } else {
            os << "            ral_u32 vo[" << NOV << "]; ral_vword(P, w, vo);\n";
        }
        for (int i = 0; i < NOV; i++) os << "            pvo" << i << "[w] = vo[" << i << "]; vcnt[" << i << "] += __popc(vo[" << i << "]);\n";
        os << "        }\n";
    }
    if (staged) {
        // every lane is done with the stage: lane 0 refills it with the warp's tile S steps ahead
        os << "        __syncwarp();\n";
        os << "        if (lane == 0 && t + (ral_i64)RAL_S * nwarp < ntiles) {\n";
        os << "            asm volatile(\"fence.proxy.async.shared::cta;\" ::: \"memory\");\n";
        os << "            fill(q, t + (ral_i64)RAL_S * nwarp);\n";
        os << "        }\n";
    }
    os << "    }\n";
    if (staged) {
        // a wait that gave up: record it; before the warp exits, wait (bounded) for the copies it
        // issued so that none lands in shared memory after the block has finished
        os << "    if (!ok) {\n";
        os << "        if (lane == 0) atomicExch((unsigned long long*)err, 1ull);\n";
        os << "        for (ral_i64 t = gwarp + k * nwarp; t < ntiles && t < gwarp + (k + RAL_S) * nwarp; t += nwarp, ++k)\n";
        os << "            ral_mbar_wait(bars + (int)(k % RAL_S), (unsigned)((k / RAL_S) & 1));\n";
        os << "    }\n";
    }

    // tail rows and words, one warp
    os << "    const ral_i64 tail0 = ntiles * TILE;\n";
    os << "    if (tail0 < n && gwarp == (ntiles % nwarp)) {\n";
    os << "        for (ral_i64 r = tail0 + lane; r < n; r += 32) {\n";
    for (int c = 0; c < p.n_in; c++) {
        if (!raw[c]) continue;
        if (p.inputs[c].has_valid) os << "            const ral_u32 rw" << c << " = __ldg(pvr" << c << " + (r >> 5));\n";
        else os << "            const ral_u32 rw" << c << " = 0xffffffffu;\n";
    }
    for (int o = 0; o < p.n_out; o++) os << "            " << kind_ctype(fk[o]) << " y" << o << ";\n";
    os << "            ral_row(P";
    for (int c = 0; c < p.n_in; c++)
        if (ref[c]) os << ", " << widen("pin" + std::to_string(c) + "[r]", p.inputs[c].dtype);
    for (int c = 0; c < p.n_in; c++)
        if (raw[c]) os << ", (rw" << c << " >> (int)(r & 31)) & 1u";
    for (int o = 0; o < p.n_out; o++) os << ", y" << o;
    os << ");\n";
    for (int o = 0; o < p.n_out; o++)
        os << "            pout" << o << "[r] = " << narrow("y" + std::to_string(o), fk[o], p.out_dtypes[o]) << ";\n";
    os << "        }\n";
    if (NOV > 0) {
        os << "        const ral_i64 wend = (n + 31) >> 5;\n";
        os << "        for (ral_i64 w = (tail0 >> 5) + lane; w < wend; w += 32) {\n";
        os << "            ral_u32 vo[" << NOV << "]; ral_vword(P, w, vo);\n";
        os << "            const ral_i64 rem = n - (w << 5);\n";
        os << "            const ral_u32 m = rem >= 32 ? 0xffffffffu : ((1u << rem) - 1u);\n";
        for (int i = 0; i < NOV; i++) os << "            pvo" << i << "[w] = vo[" << i << "]; vcnt[" << i << "] += __popc(vo[" << i << "] & m);\n";
        os << "        }\n";
    }
    os << "    }\n";

    // valid-bit counts: warp -> block -> one atomic per block and output
    if (NOV > 0) {
        os << "    ral_u64* counts = (ral_u64*)P.s[" << L.counts << "];\n";
        os << "    if (counts) {\n";
        os << "        __shared__ ral_u64 red[RAL_THREADS / 32][" << NOV << "];\n";
        os << "        for (int i = 0; i < " << NOV << "; ++i) {\n";
        os << "            ral_u64 v = vcnt[i];\n";
        os << "            for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);\n";
        os << "            if (lane == 0) red[threadIdx.x >> 5][i] = v;\n";
        os << "        }\n";
        os << "        __syncthreads();\n";
        os << "        const int vmap[" << NOV << "] = {";
        for (int i = 0; i < NOV; i++) os << (i ? ", " : "") << vouts[i];
        os << "};\n";
        os << "        if (threadIdx.x < " << NOV << ") {\n";
        os << "            ral_u64 v = 0;\n";
        os << "            for (int k = 0; k < RAL_THREADS / 32; ++k) v += red[k][threadIdx.x];\n";
        os << "            if (v) atomicAdd((unsigned long long*)(counts + vmap[threadIdx.x]), (unsigned long long)v);\n";
        os << "        }\n";
        os << "    }\n";
    }
    os << "}\n";
    gk.source = os.str();
    if (staged) gk.dyn_smem = warp_smem * (s.threads / 32);
    return gk;
}

namespace {

bool slot_float(const AggregateSlot& a) { return dtype_is_float(a.dtype); }

// cudf's reduction identities in the reduced column's type (numeric_limits max / lowest), as
// literals of the accumulator type
std::string slot_identity(const AggregateSlot& a) {
    if (a.op == GDF_SUM) return slot_float(a) ? "0.0" : "0ll";
    const bool mn = a.op == GDF_MIN;
    switch (a.dtype) {
    case GDF_FLOAT32: return mn ? "3.4028234663852886e+38" : "-3.4028234663852886e+38";
    case GDF_FLOAT64: return mn ? "1.7976931348623157e+308" : "-1.7976931348623157e+308";
    case GDF_INT8: case GDF_BOOL8: return mn ? "127ll" : "-128ll";
    case GDF_INT16: return mn ? "32767ll" : "-32768ll";
    case GDF_INT32: case GDF_DATE32: case GDF_CATEGORY: case GDF_STRING_CATEGORY:
        return mn ? "2147483647ll" : "(-2147483647ll - 1)";
    default: return mn ? "9223372036854775807ll" : "(-9223372036854775807ll - 1)";
    }
}

// acc = fold(acc, v): wrapping int64 add, IEEE double add, or std::min / std::max (which keep the
// accumulator unless the new value compares below / above it)
std::string slot_fold(const AggregateSlot& a, const std::string& acc, const std::string& v) {
    const bool f = slot_float(a);
    if (a.op == GDF_SUM)
        return f ? "__dadd_rn(" + acc + ", " + v + ")" : "ral_addi(" + acc + ", " + v + ")";
    if (a.op == GDF_MIN)
        return f ? "(ral_dlt(" + v + ", " + acc + ") ? " + v + " : " + acc + ")" : "(" + v + " < " + acc + " ? " + v + " : " + acc + ")";
    return f ? "(ral_dlt(" + acc + ", " + v + ") ? " + v + " : " + acc + ")" : "(" + acc + " < " + v + " ? " + v + " : " + acc + ")";
}

// A column element as the accumulator's type: ints sign-extended to int64, floats to double.
std::string slot_value(const std::string& elem, gdf_dtype t) {
    if (t == GDF_FLOAT32) return "ral_f2d(" + elem + ")";
    if (t == GDF_FLOAT64) return "(" + elem + ")";
    return "((ral_i64)(" + elem + "))";
}

}  // namespace

GeneratedKernel generate_aggregate_kernel(const Program& p, const std::vector<AggregateSlot>& slots,
                                          const std::vector<ColumnDesc>& bare, const Shape& s) {
    GeneratedKernel gk;
    gk.shape = s;
    const int NB = (int)bare.size();
    gk.layout = make_layout(p, 1 + 2 * NB);
    const ParamLayout& L = gk.layout;
    const int scratch_slot = L.counts + 1;
    const int bare_data = scratch_slot + 1, bare_valid = bare_data + NB;
    const int S = (int)slots.size();
    const bool has_prog = p.n_out > 0;
    const std::vector<bool> load = has_prog ? p.inputs_referenced() : std::vector<bool>(p.n_in, false);
    const auto raw = has_prog ? p.inputs_raw_valid() : std::vector<bool>(p.n_in, false);
    std::vector<bool> mask(NB, false);  // bare columns whose null rows are skipped
    for (const auto& a : slots)
        if (!a.evaluated && a.skip_nulls) mask[a.index] = true;
    const auto fk = has_prog ? final_kinds(p, L) : std::vector<Kind>();

    std::ostringstream key;
    key << "agg|" << (has_prog ? p.structure_key() : std::string("-")) << "|";
    for (const auto& b : bare) key << (int)b.dtype << (b.has_valid ? "v" : "n") << ",";
    key << "|";
    for (const auto& a : slots)
        key << a.op << (a.evaluated ? "e" : "c") << a.index << ":" << (int)a.dtype << (a.skip_nulls ? "s" : "") << ";";
    key << "|G" << s.G << "J" << s.J << "T" << s.threads << "B" << s.min_blocks;
    char hex[32];
    snprintf(hex, sizeof hex, "%016llx", (unsigned long long)fnv1a(key.str()));
    gk.name = std::string("ral_agg_") + hex;

    std::ostringstream os;
    os << "// generated: " << key.str() << "\n";
    os << "#define RAL_G " << s.G << "\n#define RAL_J " << s.J << "\n#define RAL_THREADS " << s.threads << "\n";
    os << "struct RalParams { ral_u64 s[" << L.total << "]; };\n\n";
    if (has_prog) emit_row_function(os, p, L, "ral_row");
    auto acc_t = [&](const AggregateSlot& a) { return slot_float(a) ? "double" : "ral_i64"; };
    auto to_u64 = [&](const AggregateSlot& a, const std::string& v) {
        return slot_float(a) ? "(ral_u64)__double_as_longlong(" + v + ")" : "(ral_u64)(" + v + ")";
    };
    auto from_u64 = [&](const AggregateSlot& a, const std::string& v) {
        return slot_float(a) ? "__longlong_as_double((long long)(" + v + "))" : "(ral_i64)(" + v + ")";
    };
    // the per-row fold: elem / bit give a program input's element and raw validity bit, belem /
    // bbit a bare column's
    auto emit_folds = [&](const std::string& ind, const std::function<std::string(int)>& elem,
                          const std::function<std::string(int)>& bit, const std::function<std::string(int)>& belem,
                          const std::function<std::string(int)>& bbit) {
        std::ostringstream o;
        if (has_prog) {
            for (int q = 0; q < p.n_out; q++) o << ind << kind_ctype(fk[q]) << " y" << q << ";\n";
            o << ind << "ral_row(P";
            for (int c = 0; c < p.n_in; c++)
                if (p.inputs_referenced()[c]) o << ", " << widen(elem(c), p.inputs[c].dtype);
            for (int c = 0; c < p.n_in; c++)
                if (raw[c]) o << ", " << bit(c);
            for (int q = 0; q < p.n_out; q++) o << ", y" << q;
            o << ");\n";
        }
        for (int k = 0; k < S; k++) {
            const auto& a = slots[k];
            std::string v;
            if (a.evaluated)
                v = slot_value(narrow("y" + std::to_string(a.index), fk[a.index], a.dtype), a.dtype);
            else
                v = slot_value(belem(a.index), a.dtype);
            const std::string acc = "acc" + std::to_string(k);
            if (!a.evaluated && a.skip_nulls)
                o << ind << "if (" << bbit(a.index) << ") " << acc << " = " << slot_fold(a, acc, v) << ";\n";
            else
                o << ind << acc << " = " << slot_fold(a, acc, v) << ";\n";
        }
        return o.str();
    };

    os << "\nextern \"C\" __global__ void __launch_bounds__(RAL_THREADS, " << s.min_blocks << ") " << gk.name
       << "(const __grid_constant__ RalParams P) {\n";
    os << "    const ral_i64 n = (ral_i64)P.s[" << L.n_rows << "];\n";
    for (int c = 0; c < p.n_in; c++) {
        if (load[c])
            os << "    const " << element_ctype(p.inputs[c].dtype) << "* __restrict__ pin" << c << " = (const "
               << element_ctype(p.inputs[c].dtype) << "*)P.s[" << L.in_data + c << "];\n";
        if (raw[c] && p.inputs[c].has_valid)
            os << "    const ral_u32* __restrict__ pvr" << c << " = (const ral_u32*)P.s[" << L.in_valid + c << "];\n";
    }
    for (int c = 0; c < NB; c++) {
        os << "    const " << element_ctype(bare[c].dtype) << "* __restrict__ pbx" << c << " = (const "
           << element_ctype(bare[c].dtype) << "*)P.s[" << bare_data + c << "];\n";
        if (mask[c] && bare[c].has_valid)
            os << "    const ral_u32* __restrict__ pbv" << c << " = (const ral_u32*)P.s[" << bare_valid + c << "];\n";
    }
    for (int k = 0; k < S; k++) os << "    " << acc_t(slots[k]) << " acc" << k << " = " << slot_identity(slots[k]) << ";\n";
    os << "    const int lane = threadIdx.x & 31;\n";
    os << "    const ral_i64 gwarp = ((ral_i64)blockIdx.x * RAL_THREADS + threadIdx.x) >> 5;\n";
    os << "    const ral_i64 nwarp = ((ral_i64)gridDim.x * RAL_THREADS) >> 5;\n";
    os << "    const ral_i64 TILE = 32 * RAL_G * RAL_J;\n";
    os << "    const ral_i64 ntiles = n / TILE;\n";
    os << "    for (ral_i64 t = gwarp; t < ntiles; t += nwarp) {\n";
    os << "        const ral_i64 base = t * TILE;\n";
    os << "#pragma unroll\n";
    os << "        for (int j = 0; j < RAL_J; ++j) {\n";
    os << "            const ral_i64 r = base + (ral_i64)j * 32 * RAL_G + lane * RAL_G;\n";
    for (int c = 0; c < p.n_in; c++) {
        if (!load[c]) continue;
        const char* et = element_ctype(p.inputs[c].dtype);
        os << "            " << et << " a" << c << "[RAL_G]; ral_ldg<" << et << ", RAL_G>(pin" << c << ", r, a" << c << ");\n";
    }
    for (int c = 0; c < NB; c++) {
        const char* et = element_ctype(bare[c].dtype);
        os << "            " << et << " e" << c << "[RAL_G]; ral_ldg<" << et << ", RAL_G>(pbx" << c << ", r, e" << c << ");\n";
    }
    for (int c = 0; c < p.n_in; c++) {
        if (!raw[c]) continue;
        if (p.inputs[c].has_valid) os << "            const ral_u32 rw" << c << " = __ldg(pvr" << c << " + (r >> 5));\n";
        else os << "            const ral_u32 rw" << c << " = 0xffffffffu;\n";
    }
    for (int c = 0; c < NB; c++) {
        if (!mask[c]) continue;
        if (bare[c].has_valid) os << "            const ral_u32 bw" << c << " = __ldg(pbv" << c << " + (r >> 5));\n";
        else os << "            const ral_u32 bw" << c << " = 0xffffffffu;\n";
    }
    os << "#pragma unroll\n";
    os << "            for (int g = 0; g < RAL_G; ++g) {\n";
    os << emit_folds("                ", [](int c) { return "a" + std::to_string(c) + "[g]"; },
                     [](int c) { return "((rw" + std::to_string(c) + " >> ((int)(r & 31) + g)) & 1u)"; },
                     [](int c) { return "e" + std::to_string(c) + "[g]"; },
                     [](int c) { return "((bw" + std::to_string(c) + " >> ((int)(r & 31) + g)) & 1u)"; });
    os << "            }\n";
    os << "        }\n";
    os << "    }\n";
    // tail rows, one warp
    os << "    const ral_i64 tail0 = ntiles * TILE;\n";
    os << "    if (tail0 < n && gwarp == (ntiles % nwarp)) {\n";
    os << "        for (ral_i64 r = tail0 + lane; r < n; r += 32) {\n";
    for (int c = 0; c < p.n_in; c++) {
        if (!raw[c]) continue;
        if (p.inputs[c].has_valid) os << "            const ral_u32 rw" << c << " = __ldg(pvr" << c << " + (r >> 5));\n";
        else os << "            const ral_u32 rw" << c << " = 0xffffffffu;\n";
    }
    for (int c = 0; c < NB; c++) {
        if (!mask[c]) continue;
        if (bare[c].has_valid) os << "            const ral_u32 bw" << c << " = __ldg(pbv" << c << " + (r >> 5));\n";
        else os << "            const ral_u32 bw" << c << " = 0xffffffffu;\n";
    }
    os << emit_folds("            ", [](int c) { return "pin" + std::to_string(c) + "[r]"; },
                     [](int c) { return "((rw" + std::to_string(c) + " >> (int)(r & 31)) & 1u)"; },
                     [](int c) { return "pbx" + std::to_string(c) + "[r]"; },
                     [](int c) { return "((bw" + std::to_string(c) + " >> (int)(r & 31)) & 1u)"; });
    os << "        }\n";
    os << "    }\n";
    // warp -> block -> block partials -> the last block folds them in block order
    os << "    __shared__ ral_u64 red[RAL_THREADS / 32][" << S << "];\n";
    os << "    __shared__ int s_last;\n";
    for (int k = 0; k < S; k++) {
        const auto& a = slots[k];
        const std::string acc = "acc" + std::to_string(k);
        os << "    for (int off = 16; off > 0; off >>= 1) { const " << acc_t(a) << " o = __shfl_down_sync(0xffffffffu, "
           << acc << ", off); " << acc << " = " << slot_fold(a, acc, "o") << "; }\n";
        os << "    if (lane == 0) red[threadIdx.x >> 5][" << k << "] = " << to_u64(a, acc) << ";\n";
    }
    os << "    __syncthreads();\n";
    os << "    ral_u64* scratch = (ral_u64*)P.s[" << scratch_slot << "];\n";
    os << "    ral_u64* partials = scratch + 1 + " << S << ";\n";
    os << "    if (threadIdx.x == 0) {\n";
    for (int k = 0; k < S; k++) {
        const auto& a = slots[k];
        os << "        {\n";
        os << "            " << acc_t(a) << " v = " << from_u64(a, "red[0][" + std::to_string(k) + "]") << ";\n";
        os << "            for (int w = 1; w < RAL_THREADS / 32; ++w) { const " << acc_t(a) << " o = "
           << from_u64(a, "red[w][" + std::to_string(k) + "]") << "; v = " << slot_fold(a, "v", "o") << "; }\n";
        os << "            partials[(ral_i64)blockIdx.x * " << S << " + " << k << "] = " << to_u64(a, "v") << ";\n";
        os << "        }\n";
    }
    os << "        __threadfence();\n";
    os << "        const unsigned done = atomicAdd((unsigned*)scratch, 1u);\n";
    os << "        s_last = done == gridDim.x - 1;\n";
    os << "    }\n";
    os << "    __syncthreads();\n";
    os << "    if (s_last && threadIdx.x < " << S << ") {\n";
    os << "        __threadfence();\n";
    os << "        const int k = threadIdx.x;\n";
    for (int k = 0; k < S; k++) {
        const auto& a = slots[k];
        os << "        if (k == " << k << ") {\n";
        os << "            " << acc_t(a) << " v = " << from_u64(a, "__ldcg(partials + " + std::to_string(k) + ")") << ";\n";
        os << "            for (unsigned b = 1; b < gridDim.x; ++b) { const " << acc_t(a) << " o = "
           << from_u64(a, "__ldcg(partials + (ral_i64)b * " + std::to_string(S) + " + " + std::to_string(k) + ")")
           << "; v = " << slot_fold(a, "v", "o") << "; }\n";
        os << "            scratch[1 + " << k << "] = " << to_u64(a, "v") << ";\n";
        os << "        }\n";
    }
    os << "    }\n";
    os << "}\n";
    gk.source = os.str();
    return gk;
}

int filter_max_width(const FilterSpec& f) {
    int w = 1;
    if (f.clone_stencil) w = std::max(w, gdf_dtype_size(f.frame_dtypes[f.clone_column]));
    if (f.predicate) {
        auto ref = f.predicate->inputs_referenced();
        for (size_t c = 0; c < f.predicate_cols.size(); c++)
            if (ref[c]) w = std::max(w, gdf_dtype_size(f.frame_dtypes[f.predicate_cols[c]]));
    }
    if (f.project) {
        auto ref = f.project->inputs_referenced();
        for (size_t c = 0; c < f.project_cols.size(); c++)
            if (ref[c]) w = std::max(w, gdf_dtype_size(f.frame_dtypes[f.project_cols[c]]));
    }
    for (const FilterOutput& o : f.outputs) w = std::max(w, gdf_dtype_size(o.dtype));
    return w;
}

GeneratedKernel generate_filter_kernel(const FilterSpec& f, const Shape& s, bool item) {
    if (s.G * s.J > 4096) throw std::runtime_error("filter kernel shape: G*J out of range");
    if (item && s.stage) throw std::runtime_error("filter item functions take no shared-memory stage");
    GeneratedKernel gk;
    gk.shape = s;
    ParamLayout& L = gk.layout;
    const int NF = f.n_frame;
    const int NO = (int)f.outputs.size();
    int slot = 0;
    L.n_rows = slot++;
    L.in_data = slot; slot += NF;
    L.in_valid = slot; slot += NF;
    L.out_data = slot; slot += NO;
    L.out_valid = slot; slot += NO;
    L.scratch = slot++;
    ParamLayout PL, QL;  // scalar slots of the predicate and projection programs
    if (f.predicate) {
        assign_scalar_slots(*f.predicate, PL, slot);
    }
    if (f.project) {
        assign_scalar_slots(*f.project, QL, slot);
    }
    L.lscalar_slot = PL.lscalar_slot;
    L.rscalar_slot = PL.rscalar_slot;
    L.rdiv_slot = PL.rdiv_slot;
    gk.layout_project_lscalar = QL.lscalar_slot;
    gk.layout_project_rscalar = QL.rscalar_slot;
    gk.layout_project_rdiv = QL.rdiv_slot;
    if (!item) L.obase = slot++;
    if (!item && s.grid_k > 0) {
        L.epoch = slot++;
        L.hostmap = slot++;
    }
    L.total = slot;

    std::vector<int> vouts;  // outputs with a mask
    for (int k = 0; k < NO; k++)
        if (f.outputs[k].has_valid) vouts.push_back(k);
    const int NVO = (int)vouts.size();
    bool any_proj_valid = false;
    for (int k : vouts) any_proj_valid |= f.outputs[k].from_project;

    // which frame columns the kernel dereferences
    std::vector<bool> f_data(NF, false), f_valid(NF, false);
    auto pred_ref = f.predicate ? f.predicate->inputs_referenced() : std::vector<bool>();
    auto pred_raw = f.predicate ? f.predicate->inputs_raw_valid() : std::vector<bool>();
    auto proj_ref = f.project ? f.project->inputs_referenced() : std::vector<bool>();
    auto proj_raw = f.project ? f.project->inputs_raw_valid() : std::vector<bool>();
    if (f.clone_stencil) {
        f_data[f.clone_column] = true;
        f_valid[f.clone_column] = f.frame_has_valid[f.clone_column];
    }
    // masks the kernel body reads directly (the validity-word functions read theirs through P)
    for (size_t c = 0; c < f.predicate_cols.size(); c++) {
        if (pred_ref[c]) f_data[f.predicate_cols[c]] = true;
        if (pred_raw[c] && f.frame_has_valid[f.predicate_cols[c]]) f_valid[f.predicate_cols[c]] = true;
    }
    for (size_t c = 0; c < f.project_cols.size(); c++) {
        if (proj_ref[c]) f_data[f.project_cols[c]] = true;
        if (proj_raw[c] && f.frame_has_valid[f.project_cols[c]]) f_valid[f.project_cols[c]] = true;
    }
    for (const FilterOutput& o : f.outputs) {
        if (o.from_project) continue;
        f_data[o.index] = true;
        if (o.has_valid) f_valid[o.index] = true;
    }

    std::ostringstream key;
    key << "filter|n" << NF << "|";
    for (int c = 0; c < NF; c++) key << (int)f.frame_dtypes[c] << (f.frame_has_valid[c] ? "v" : "") << ",";
    key << "|clone" << (f.clone_stencil ? f.clone_column : -1) << "|";
    if (f.predicate) {
        key << "P" << f.predicate->structure_key() << "@";
        for (int c : f.predicate_cols) key << c << ",";
    }
    if (f.project) {
        key << "|Q" << f.project->structure_key() << "@";
        for (int c : f.project_cols) key << c << ",";
    }
    key << "|O";
    for (const FilterOutput& o : f.outputs) key << (o.from_project ? "p" : "g") << o.index << ":" << (int)o.dtype << (o.has_valid ? "v" : "") << ",";
    // dense pass 2 (see Shape::dense): per warp a u16 list of the chunk's kept rows and the
    // projection's validity words of the chunk; kept to blocks whose static shared memory fits
    bool any_gather = false, any_proj = false;
    for (const FilterOutput& o : f.outputs) (o.from_project ? any_proj : any_gather) = true;
    int n_proj_vouts = 0;
    for (int k : vouts) n_proj_vouts += f.outputs[k].from_project ? 1 : 0;
    bool dense = s.dense != 0;
    if (32 * s.G * s.J > 65536) dense = false;
    {
        const long per_warp = (long)NVO * (s.G * s.J + 2) * 4 + (dense ? (long)n_proj_vouts * s.G * s.J * 4 + 64L * s.G * s.J : 0);
        if (dense && per_warp * (s.threads / 32) > 47 * 1024) dense = false;
    }
    key << "|G" << s.G << "J" << s.J << "T" << s.threads << "B" << s.min_blocks << "U" << s.unroll << "S" << s.stage
        << "P" << s.prefetch << "D" << (dense ? 1 : 0) << "K" << s.dense_unroll;
    if (!item && s.grid_k > 0) key << "R" << s.grid_k;
    if (item) key << "|item" << (s.soft ? "s" : "");
    char hex[32];
    snprintf(hex, sizeof hex, "%016llx", (unsigned long long)fnv1a(key.str()));
    gk.name = std::string(item ? "ral_fitem_" : "ral_filter_") + hex;
    gk.soft_fp = item ? s.soft : true;

    std::ostringstream os;
    os << "// generated: " << key.str() << "\n";
    os << "#define RAL_G " << s.G << "\n#define RAL_J " << s.J << "\n#define RAL_THREADS " << s.threads << "\n";
    os << "#define RAL_WARPS (RAL_THREADS / 32)\n";
    if (!item && s.grid_k > 0) os << "#define RAL_K " << s.grid_k << "\n";
    os << "struct RalParams { ral_u64 s[" << L.total << "]; };\n\n";
    auto fdata = [&](int c) { return "f" + std::to_string(c); };
    auto fvalid = [&](int c) { return "fv" + std::to_string(c); };

    std::vector<Kind> pred_kind, proj_kind;
    if (f.predicate) {
        emit_row_function(os, *f.predicate, PL, "ral_pred_row");
        pred_kind = final_kinds(*f.predicate, PL);
        os << "RAL_FI ral_u32 ral_pred_vword(const RalParams& P, const ral_i64 w) {\n";
        ValidEmitter ve(*f.predicate);
        ve.emit(os, "    ", [&](int c) {
            return "__ldg(((const ral_u32*)P.s[" + std::to_string(L.in_valid + f.predicate_cols[c]) + "]) + w)";
        });
        os << "    return " << ve.name[f.predicate->final_pos[0]] << ";\n}\n";
    }
    std::vector<int> proj_vouts;  // projection outputs with a mask, in output order
    if (f.project) {
        emit_row_function(os, *f.project, QL, "ral_proj_row");
        proj_kind = final_kinds(*f.project, QL);
        for (int k : vouts)
            if (f.outputs[k].from_project) proj_vouts.push_back(f.outputs[k].index);
        if (!proj_vouts.empty()) {
            os << "RAL_FI void ral_proj_vword(const RalParams& P, const ral_i64 w, ral_u32* vo) {\n";
            ValidEmitter ve(*f.project);
            ve.emit(os, "    ", [&](int c) {
                return "__ldg(((const ral_u32*)P.s[" + std::to_string(L.in_valid + f.project_cols[c]) + "]) + w)";
            });
            for (size_t i = 0; i < proj_vouts.size(); i++)
                os << "    vo[" << i << "] = " << ve.name[f.project->final_pos[proj_vouts[i]]] << ";\n";
            os << "}\n";
        }
    }

    // ---- kernel: warp-sized chunks of 32*G*J rows taken by ticket, no block-wide barriers.
    // Pass 1 evaluates the predicate over a chunk into keep bits; the warp publishes the chunk's
    // kept count and looks back over the preceding chunks for its output offset; pass 2 writes
    // every output.  Pass 2 walks the chunk's kept-row list, 32 kept rows per step (dense, the
    // default), or takes each slice's rows lane by lane from packed keep bits (D=0).  Dense full
    // kernels with chunks of at most 32 mask words hold two chunks per warp: the next chunk's
    // pass 1 and published count come before the look-back and pass 2 of the last one.
    // Columns the predicate reads are loaded with normal eviction, so that a second read by the
    // gather or the projection hits in cache instead of DRAM.
    std::vector<bool> pred_col(NF, false);
    if (f.clone_stencil) pred_col[f.clone_column] = true;
    for (size_t c = 0; c < f.predicate_cols.size(); c++)
        if (pred_ref[c]) pred_col[f.predicate_cols[c]] = true;
    // loads of a frame column for the G rows at r (vector in full chunks, guarded otherwise)
    auto load = [&](std::ostream& o, const std::string& ind, int c, const std::string& arr) {
        const char* et = element_ctype(f.frame_dtypes[c]);
        o << ind << et << " " << arr << "[RAL_G];\n";
        o << ind << "if (full) " << (pred_col[c] ? "ral_ldg_keep<" : "ral_ldg<") << et << ", RAL_G>(" << fdata(c)
          << ", r, " << arr << ");\n";
        o << ind << "else {\n" << ind << "#pragma unroll\n" << ind << "    for (int g = 0; g < RAL_G; ++g) " << arr
          << "[g] = (r + g < n) ? " << fdata(c) << "[r + g] : (" << et << ")0;\n" << ind << "}\n";
    };
    auto raw_word = [&](int c) {
        if (!f.frame_has_valid[c]) return std::string("0xffffffffu");
        return "((r < n) ? __ldg(" + fvalid(c) + " + (r >> 5)) : 0xffffffffu)";
    };
    // With the dense pass 2 the kept-row list decouples pass 1 from pass 2's slices: pass 1 then
    // takes G1 = 16 / (widest column it reads) rows per lane and slice (4 for an int32 predicate
    // column against pass 2's 2 for int64 / double outputs), reads the chunk's stencil validity
    // words once (one per lane; a chunk of at most 32 words), and indexes the chunk with 32-bit
    // offsets.
    int p1_width = 0;
    if (f.clone_stencil) p1_width = gdf_dtype_size(f.frame_dtypes[f.clone_column]);
    for (size_t c = 0; c < f.predicate_cols.size(); c++)
        if (!f.clone_stencil && pred_ref[c]) p1_width = std::max(p1_width, gdf_dtype_size(f.frame_dtypes[f.predicate_cols[c]]));
    const int G1 = (s.G > 1 && p1_width > 0) ? 16 / p1_width : s.G;
    const bool wide_p1 = dense && s.G * s.J <= 32 && G1 >= 1 && G1 <= 16 && (s.G * s.J) % G1 == 0;
    // Pipelined chunks (a full kernel with the wide pass 1): a warp evaluates the predicate of its
    // next chunk B and publishes B's count before it looks back for the chunk A it evaluated the
    // round before, so A's predecessors have long published and the look-back rarely waits.
    // Pass 1 then records the keep bits as the chunk's 32 mask words (two chunks per warp in
    // shared memory) and pass 2 turns A's words into its kept-row list.
    // Grid mode (Shape::grid_k): static chunks, pass 1 of all of a warp's chunks, one grid barrier,
    // then pass 2 with offsets summed from block, warp and chunk counts -- no look-back chain,
    // which at a few thousand small chunks costs more than the rows themselves.
    const bool grid = wide_p1 && !item && s.grid_k > 0;
    const bool pipe = wide_p1 && !item && !grid;
    gk.shape.grid_k = grid ? s.grid_k : 0;
    const int KBW = (s.G * s.J + 31) / 32;  // packed keep-bit words per lane
    if (item) {
        // one chunk of a batched request: the dispatcher hands over the chunk index and this
        // warp's shared-memory area (masks staged per output)
        os << "\nextern \"C\" __device__ __noinline__ void " << gk.name
           << "(const ral_u64* __restrict__ slots, const ral_i64 chunk_index, ral_u32* __restrict__ wsm) {\n";
        os << "    const RalParams& P = *reinterpret_cast<const RalParams*>(slots);\n";
        if (NVO) os << "    ral_u32 (*const s_vbw)[RAL_G * RAL_J + 2] = reinterpret_cast<ral_u32 (*)[RAL_G * RAL_J + 2]>(wsm);\n";
        int words = NVO * (s.G * s.J + 2);
        if (dense) {
            if (n_proj_vouts)
                os << "    ral_u32 (*const s_pvw)[RAL_G * RAL_J] = reinterpret_cast<ral_u32 (*)[RAL_G * RAL_J]>(wsm + " << words << ");\n";
            words += n_proj_vouts * s.G * s.J;
            os << "    unsigned short* const s_lst = reinterpret_cast<unsigned short*>(wsm + " << words << ");\n";
            words += 16 * s.G * s.J;
        }
        gk.item_smem_words = words;
    } else {
        os << "\nextern \"C\" __global__ void __launch_bounds__(RAL_THREADS, " << std::max(1, s.min_blocks) << ") " << gk.name
           << "(const __grid_constant__ RalParams P) {\n";
        if (NVO) os << "    __shared__ ral_u32 s_vb[RAL_WARPS][" << NVO << "][RAL_G * RAL_J + 2];\n";
        if (dense) {
            if (n_proj_vouts) os << "    __shared__ ral_u32 s_pv[RAL_WARPS][" << n_proj_vouts << "][RAL_G * RAL_J];\n";
            os << "    __shared__ unsigned short s_ls[RAL_WARPS][32 * RAL_G * RAL_J];\n";
        }
        if (pipe) os << "    __shared__ ral_u32 s_kp[RAL_WARPS][2][32];\n";
        if (grid) {
            os << "    __shared__ ral_u32 s_kp[RAL_WARPS][RAL_K][32];\n";
            os << "    __shared__ ral_u32 s_ct[RAL_WARPS][RAL_K];\n";
            os << "    __shared__ ral_u32 s_wt[RAL_WARPS];\n";
            os << "    __shared__ ral_u64 s_bpre;\n";
        }
    }
    // per-warp staging of one slice's compacted values, so that stores are contiguous
    if (s.stage) os << "    __shared__ ral_u64 s_stage[RAL_WARPS][32 * RAL_G];\n";
    os << "    const ral_i64 n = (ral_i64)P.s[" << L.n_rows << "];\n";
    if (L.obase >= 0) os << "    const ral_u64 RAL_OBASE = (ral_u64)P.s[" << L.obase << "];\n";
    else os << "    const ral_u64 RAL_OBASE = 0ull;\n";
    os << "    ral_u64* const scratch = (ral_u64*)P.s[" << L.scratch << "];\n";
    os << "    ral_u64* const status = scratch + " << filter_scratch_header(NO) << ";\n";
    for (int c = 0; c < NF; c++) {
        if (f_data[c])
            os << "    const " << element_ctype(f.frame_dtypes[c]) << "* __restrict__ " << fdata(c) << " = (const "
               << element_ctype(f.frame_dtypes[c]) << "*)P.s[" << L.in_data + c << "];\n";
        if (f_valid[c])
            os << "    const ral_u32* __restrict__ " << fvalid(c) << " = (const ral_u32*)P.s[" << L.in_valid + c << "];\n";
    }
    for (int k = 0; k < NO; k++) {
        os << "    " << element_ctype(f.outputs[k].dtype) << "* __restrict__ o" << k << " = ("
           << element_ctype(f.outputs[k].dtype) << "*)P.s[" << L.out_data + k << "];\n";
        if (f.outputs[k].has_valid)
            os << "    ral_u32* __restrict__ ov" << k << " = (ral_u32*)P.s[" << L.out_valid + k << "];\n";
    }
    os << "    const int lane = threadIdx.x & 31;\n";
    if (!item) {
        os << "    const int warp = threadIdx.x >> 5;\n";
        if (NVO) os << "    ral_u32 (*const s_vbw)[RAL_G * RAL_J + 2] = s_vb[warp];\n";
        if (s.stage) os << "    ral_u64* const s_stw = s_stage[warp];\n";
        if (dense) {
            if (n_proj_vouts) os << "    ral_u32 (*const s_pvw)[RAL_G * RAL_J] = s_pv[warp];\n";
            os << "    unsigned short* const s_lst = s_ls[warp];\n";
        }
        if (pipe || grid) os << "    ral_u32 (*const s_kpw)[32] = s_kp[warp];\n";
        if (grid) os << "    ral_u32* const s_ctw = s_ct[warp];\n";
    }
    os << "    const ral_i64 WT = 32 * RAL_G * RAL_J;\n";
    os << "    const ral_i64 nchunks = (n + WT - 1) / WT;\n";
    os << "    const ral_u32 GMASK = (RAL_G == 32) ? 0xffffffffu : ((1u << RAL_G) - 1u);\n";
    if (NVO) os << "    ral_u32 vcnt[" << NVO << "];\n    for (int i = 0; i < " << NVO << "; ++i) vcnt[i] = 0;\n";
    if (grid) {
        os << "    const ral_u64 RAL_EPOCH = (ral_u64)P.s[" << L.epoch << "];\n";
        os << "    const ral_i64 gw = (ral_i64)blockIdx.x * RAL_WARPS + warp;\n";
        os << "    for (int kc = 0; kc < RAL_K; ++kc) {\n";
        os << "        const ral_i64 chunk = gw * RAL_K + kc;\n";
        os << "        if (chunk >= nchunks) { if (lane == 0) s_ctw[kc] = 0u; continue; }\n";
        os << "        ral_u32* const kp = s_kpw[kc];\n";
        os << "        kp[lane] = 0u;\n";
        os << "        __syncwarp();\n";
    } else if (pipe) {
        os << "    int chunkA = -1;\n    ral_u32 totalA = 0;\n    int bufA = 0;\n";
        os << "    for (;;) {\n";
        os << "        ral_u32 ticket = 0;\n";
        os << "        if (lane == 0) ticket = atomicAdd((unsigned int*)scratch, 1u);\n";
        os << "        const int chunkB = (int)__shfl_sync(0xffffffffu, ticket, 0);\n";
        os << "        const bool moreB = (ral_i64)chunkB < nchunks;\n";
        os << "        const int bufB = bufA ^ 1;\n";
        os << "        ral_u32 totalB = 0;\n";
        os << "        if (moreB) {\n";
        os << "        const ral_i64 chunk = chunkB;\n";
        os << "        ral_u32* const kp = s_kpw[bufB];\n";
        os << "        kp[lane] = 0u;\n";
        os << "        __syncwarp();\n";
    } else if (item) {
        os << "    do {\n";
        os << "        const ral_i64 chunk = chunk_index;\n";
    } else {
        os << "    for (;;) {\n";
        os << "        ral_u32 ticket = 0;\n";
        os << "        if (lane == 0) ticket = atomicAdd((unsigned int*)scratch, 1u);\n";
        os << "        const ral_i64 chunk = __shfl_sync(0xffffffffu, ticket, 0);\n";
        os << "        if (chunk >= nchunks) break;\n";
    }
    os << "        const ral_i64 base = chunk * WT;\n";
    os << "        const bool full = base + WT <= n;\n";
    if (!dense) {
        os << "        ral_u32 kbw[" << KBW << "];\n";
        os << "        for (int q = 0; q < " << KBW << "; ++q) kbw[q] = 0u;\n";
    }
    os << "        ral_u32 total = 0;\n";

    // ---- pass 1: predicate
    if (wide_p1) {
        os << "        ral_u32 swc = 0;\n";
        os << "        if (lane < RAL_G * RAL_J) {\n";
        os << "            const ral_i64 w = (base >> 5) + lane;\n";
        if (f.clone_stencil) {
            if (f.frame_has_valid[f.clone_column]) os << "            if ((w << 5) < n) swc = __ldg(" << fvalid(f.clone_column) << " + w);\n";
            else os << "            if ((w << 5) < n) swc = 0xffffffffu;\n";
        } else {
            os << "            if ((w << 5) < n) swc = ral_pred_vword(P, w);\n";
        }
        os << "        }\n";
        os << "#pragma unroll " << std::max(1, s.unroll) << "\n        for (int j = 0; j < (RAL_G * RAL_J) / " << G1 << "; ++j) {\n";
        os << "            const ral_u32 lr = (ral_u32)j * " << 32 * G1 << "u + (ral_u32)lane * " << G1 << "u;\n";
        os << "            const ral_i64 r = base + lr;\n";
        auto load1 = [&](int c, const std::string& arr) {
            const char* et = element_ctype(f.frame_dtypes[c]);
            os << "            " << et << " " << arr << "[" << G1 << "];\n";
            os << "            if (full) ral_ldg_keep<" << et << ", " << G1 << ">(" << fdata(c) << ", r, " << arr << ");\n";
            os << "            else {\n#pragma unroll\n                for (int g = 0; g < " << G1 << "; ++g) " << arr << "[g] = (r + g < n) ? "
               << fdata(c) << "[r + g] : (" << et << ")0;\n            }\n";
        };
        if (f.clone_stencil) {
            load1(f.clone_column, "sa");
        } else {
            for (size_t c = 0; c < f.predicate_cols.size(); c++)
                if (pred_ref[c]) load1(f.predicate_cols[c], "pa" + std::to_string(c));
            for (size_t c = 0; c < f.predicate_cols.size(); c++)
                if (pred_raw[c]) os << "            const ral_u32 rw" << c << " = " << raw_word(f.predicate_cols[c]) << ";\n";
        }
        os << "            ral_u32 bits = 0;\n";
        os << "#pragma unroll\n            for (int g = 0; g < " << G1 << "; ++g) {\n";
        if (f.clone_stencil) {
            os << "                const signed char sv = (signed char)sa[g];\n";
        } else {
            os << "                " << kind_ctype(pred_kind[0]) << " y0;\n";
            os << "                ral_pred_row(P";
            for (size_t c = 0; c < f.predicate_cols.size(); c++)
                if (pred_ref[c]) os << ", " << widen("pa" + std::to_string(c) + "[g]", f.frame_dtypes[f.predicate_cols[c]]);
            for (size_t c = 0; c < f.predicate_cols.size(); c++)
                if (pred_raw[c]) os << ", (rw" << c << " >> ((int)(r & 31) + g)) & 1u";
            os << ", y0);\n";
            os << "                const signed char sv = " << narrow("y0", pred_kind[0], GDF_INT8) << ";\n";
        }
        os << "                bits |= (sv != 0 ? 1u : 0u) << g;\n";
        os << "            }\n";
        os << "            const ral_u32 word = __shfl_sync(0xffffffffu, swc, (int)(lr >> 5));\n";
        os << "            bits &= (word >> (lr & 31u)) & " << (G1 == 32 ? "0xffffffffu" : std::to_string((1u << G1) - 1u) + "u") << ";\n";
        os << "            if (!full) {\n#pragma unroll\n                for (int g = 0; g < " << G1 << "; ++g) if (r + g >= n) bits &= ~(1u << g);\n            }\n";
        if (pipe || grid) {
            os << "            if (bits) atomicOr(kp + (lr >> 5), bits << (lr & 31u));\n";
            os << "            total += __reduce_add_sync(0xffffffffu, __popc(bits));\n";
        } else {
            os << "            {\n";
            os << "                const ral_u32 c = __popc(bits);\n";
            os << "                ral_u32 inc = c;\n";
            os << "                for (int off = 1; off < 32; off <<= 1) {\n";
            os << "                    const ral_u32 t = __shfl_up_sync(0xffffffffu, inc, off);\n";
            os << "                    if (lane >= off) inc += t;\n                }\n";
            os << "                ral_u32 q = total + inc - c;\n";
            os << "#pragma unroll\n                for (int g = 0; g < " << G1 << "; ++g)\n";
            os << "                    if ((bits >> g) & 1u) s_lst[q++] = (unsigned short)(lr + g);\n";
            os << "                total += __shfl_sync(0xffffffffu, inc, 31);\n";
            os << "            }\n";
        }
        os << "        }\n";
    } else {
    os << "#pragma unroll " << std::max(1, s.unroll) << "\n        for (int j = 0; j < RAL_J; ++j) {\n";
    os << "            const ral_i64 r = base + (ral_i64)j * 32 * RAL_G + lane * RAL_G;\n";
    // stencil validity word of this slice for the lane's rows
    os << "            ral_u32 sw = 0;\n";
    os << "            if (lane < RAL_G) {\n";
    os << "                const ral_i64 w = (base >> 5) + (ral_i64)j * RAL_G + lane;\n";
    if (f.clone_stencil) {
        if (f.frame_has_valid[f.clone_column]) os << "                if ((w << 5) < n) sw = __ldg(" << fvalid(f.clone_column) << " + w);\n";
        else os << "                if ((w << 5) < n) sw = 0xffffffffu;\n";
    } else {
        os << "                if ((w << 5) < n) sw = ral_pred_vword(P, w);\n";
    }
    os << "            }\n";
    if (f.clone_stencil) {
        load(os, "            ", f.clone_column, "sa");
    } else {
        for (size_t c = 0; c < f.predicate_cols.size(); c++)
            if (pred_ref[c]) load(os, "            ", f.predicate_cols[c], "pa" + std::to_string(c));
        for (size_t c = 0; c < f.predicate_cols.size(); c++)
            if (pred_raw[c]) os << "            const ral_u32 rw" << c << " = " << raw_word(f.predicate_cols[c]) << ";\n";
    }
    os << "            ral_u32 bits = 0;\n";
    os << "#pragma unroll\n            for (int g = 0; g < RAL_G; ++g) {\n";
    if (f.clone_stencil) {
        os << "                const signed char sv = (signed char)sa[g];\n";
    } else {
        os << "                " << kind_ctype(pred_kind[0]) << " y0;\n";
        os << "                ral_pred_row(P";
        for (size_t c = 0; c < f.predicate_cols.size(); c++)
            if (pred_ref[c]) os << ", " << widen("pa" + std::to_string(c) + "[g]", f.frame_dtypes[f.predicate_cols[c]]);
        for (size_t c = 0; c < f.predicate_cols.size(); c++)
            if (pred_raw[c]) os << ", (rw" << c << " >> ((int)(r & 31) + g)) & 1u";
        os << ", y0);\n";
        os << "                const signed char sv = " << narrow("y0", pred_kind[0], GDF_INT8) << ";\n";
    }
    os << "                bits |= (sv != 0 ? 1u : 0u) << g;\n";
    os << "            }\n";
    os << "            const ral_u32 word = __shfl_sync(0xffffffffu, sw, (lane * RAL_G) >> 5);\n";
    os << "            bits &= (word >> (int)(r & 31)) & GMASK;\n";
    os << "            if (!full) {\n#pragma unroll\n                for (int g = 0; g < RAL_G; ++g) if (r + g >= n) bits &= ~(1u << g);\n            }\n";
    if (dense) {
        // the lane's kept rows go to the chunk's list at their rank: rows of earlier slices,
        // then of lower lanes in this slice
        os << "            {\n";
        os << "                const ral_u32 c = __popc(bits);\n";
        os << "                ral_u32 inc = c;\n";
        os << "                for (int off = 1; off < 32; off <<= 1) {\n";
        os << "                    const ral_u32 t = __shfl_up_sync(0xffffffffu, inc, off);\n";
        os << "                    if (lane >= off) inc += t;\n                }\n";
        os << "                ral_u32 q = total + inc - c;\n";
        os << "#pragma unroll\n                for (int g = 0; g < RAL_G; ++g)\n";
        os << "                    if ((bits >> g) & 1u) s_lst[q++] = (unsigned short)(j * 32 * RAL_G + lane * RAL_G + g);\n";
        os << "                total += __shfl_sync(0xffffffffu, inc, 31);\n";
        os << "            }\n";
    } else {
        os << "            kbw[(j * RAL_G) >> 5] |= bits << ((j * RAL_G) & 31);\n";
        os << "            total += __reduce_add_sync(0xffffffffu, __popc(bits));\n";
    }
    os << "        }\n";
    }  // pass 1 with pass 2's slices
    if (dense && s.prefetch > 0 && s.G > 1) {
        // the chunk's rows of the columns pass 2 reads (not the predicate's, which pass 1 just
        // read) are prefetched into L2 while the warp waits in its look-back, when the chunk keeps
        // at least an eighth of its rows; one cp.async.bulk.prefetch per column, one lane each
        std::vector<bool> want(NF, false);
        for (const FilterOutput& o : f.outputs)
            if (!o.from_project) want[o.index] = true;
        for (size_t c = 0; c < f.project_cols.size(); c++)
            if (proj_ref[c]) want[f.project_cols[c]] = true;
        std::vector<int> cols;
        for (int c = 0; c < NF; c++)
            if (want[c] && !pred_col[c] && (int)cols.size() < 32) cols.push_back(c);
        if (!cols.empty()) {
            os << "        if ((ral_u64)total * 8u >= (ral_u64)WT) {\n";
            os << "            const ral_i64 rows = (n - base) < WT ? (n - base) : WT;\n";
            for (size_t i = 0; i < cols.size(); i++) {
                const int c = cols[i];
                os << "            if (lane == " << i << ") ral_prefetch_l2(" << fdata(c) << " + base, (unsigned)((rows * "
                   << gdf_dtype_size(f.frame_dtypes[c]) << ") & ~15ll));\n";
            }
            os << "        }\n";
        }
    }
    if (grid) {
        os << "        if (lane == 0) s_ctw[kc] = total;\n";
        os << "    }\n";  // pass-1 chunk loop
        // before the barrier: this block's share of the output mask words zeroed (pass 2 ORs the
        // words it shares with neighbouring chunks), block 0 zeroes the valid counts, and the
        // block's kept count goes to its status word
        os << "    {\n";
        os << "        const ral_i64 mw = (n + (ral_i64)RAL_OBASE + 31) >> 5;\n";
        os << "        for (ral_i64 q = (ral_i64)blockIdx.x * RAL_THREADS + threadIdx.x; q < mw; q += (ral_i64)gridDim.x * RAL_THREADS) {\n";
        for (int k : vouts) os << "            ov" << k << "[q] = 0u;\n";
        os << "        }\n";
        os << "        if (blockIdx.x == 0 && threadIdx.x < " << NO << ") scratch[3 + threadIdx.x] = 0ull;\n";
        os << "    }\n";
        os << "    __syncwarp();\n";
        os << "    if (lane == 0) {\n";
        os << "        ral_u32 t = 0;\n";
        os << "        for (int kc = 0; kc < RAL_K; ++kc) t += s_ctw[kc];\n";
        os << "        s_wt[warp] = t;\n";
        os << "    }\n";
        os << "    __syncthreads();\n";
        os << "    if (threadIdx.x == 0) {\n";
        os << "        ral_u64 bt = 0;\n";
        os << "        for (int w = 0; w < RAL_WARPS; ++w) bt += s_wt[w];\n";
        os << "        ral_st_status(status + blockIdx.x, bt);\n";
        os << "        ral_grid_barrier(scratch, RAL_EPOCH + gridDim.x, scratch + 1);\n";
        os << "    }\n";
        os << "    __syncthreads();\n";
        // the block's offset: the counts of the blocks before it
        os << "    if (warp == 0) {\n";
        os << "        ral_u64 acc = 0;\n";
        os << "        for (ral_i64 b = lane; b < (ral_i64)blockIdx.x; b += 32) acc += ral_ld_status(status + b);\n";
        os << "        for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);\n";
        os << "        if (lane == 0) s_bpre = acc;\n";
        os << "    }\n";
        os << "    __syncthreads();\n";
        os << "    ral_u64 wpre = s_bpre;\n";
        os << "    for (int w = 0; w < warp; ++w) wpre += s_wt[w];\n";
        os << "    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) {\n";
        os << "        ral_u64 bt = 0;\n";
        os << "        for (int w = 0; w < RAL_WARPS; ++w) bt += s_wt[w];\n";
        os << "        scratch[2] = s_bpre + bt;\n";
        os << "    }\n";
        os << "    for (int kc = 0; kc < RAL_K; ++kc) {\n";
        os << "        const ral_i64 chunk = gw * RAL_K + kc;\n";
        os << "        if (chunk >= nchunks) break;\n";
        os << "        const ral_u32 total = s_ctw[kc];\n";
        os << "        const ral_i64 base = chunk * WT;\n";
        os << "        const ral_u64 excl = wpre + RAL_OBASE;\n";
        os << "        wpre += total;\n";
        os << "        if (total != 0u) {\n";
        os << "        {\n";
        os << "            const ral_u32 kw = (lane < RAL_G * RAL_J) ? s_kpw[kc][lane] : 0u;\n";
        os << "            const ral_u32 c = __popc(kw);\n";
        os << "            ral_u32 inc = c;\n";
        os << "            for (int off = 1; off < 32; off <<= 1) {\n";
        os << "                const ral_u32 t = __shfl_up_sync(0xffffffffu, inc, off);\n";
        os << "                if (lane >= off) inc += t;\n            }\n";
        os << "            ral_u32 q = inc - c;\n";
        os << "            for (ral_u32 m = kw; m; m &= m - 1u) s_lst[q++] = (unsigned short)(lane * 32 + __ffs(m) - 1);\n";
        os << "        }\n";
    } else if (pipe) {
        os << "        ral_lookback_publish(status, chunk, total);\n";
        os << "        totalB = total;\n";
        os << "        }\n";  // chunk B
        os << "        if (chunkA >= 0) {\n";
        os << "        const ral_i64 chunk = chunkA;\n";
        os << "        const ral_u32 total = totalA;\n";
        os << "        const ral_i64 base = chunk * WT;\n";
        os << "        const ral_u64 excl0 = ral_lookback_published(status, chunk, total, scratch + 1);\n";
        os << "        if (chunk == nchunks - 1 && lane == 0) scratch[2] = excl0 + total;\n";
        os << "        const ral_u64 excl = excl0 + RAL_OBASE;\n";
        os << "        if (total != 0u) {\n";
        // A's kept-row list from its mask words: lane w holds word w, ranks by a warp scan
        os << "        {\n";
        os << "            const ral_u32 kw = (lane < RAL_G * RAL_J) ? s_kpw[bufA][lane] : 0u;\n";
        os << "            const ral_u32 c = __popc(kw);\n";
        os << "            ral_u32 inc = c;\n";
        os << "            for (int off = 1; off < 32; off <<= 1) {\n";
        os << "                const ral_u32 t = __shfl_up_sync(0xffffffffu, inc, off);\n";
        os << "                if (lane >= off) inc += t;\n            }\n";
        os << "            ral_u32 q = inc - c;\n";
        os << "            for (ral_u32 m = kw; m; m &= m - 1u) s_lst[q++] = (unsigned short)(lane * 32 + __ffs(m) - 1);\n";
        os << "        }\n";
    } else {
        os << "        const ral_u64 excl0 = ral_lookback(status, chunk, total, scratch + 1);\n";
        os << "        if (chunk == nchunks - 1 && lane == 0) scratch[2] = excl0 + total;\n";
        os << "        const ral_u64 excl = excl0 + RAL_OBASE;\n";
        os << "        if (total == 0u) continue;\n";
    }

    // ---- pass 2: ranks and outputs
    if (NVO) {
        for (int i = 0; i < NVO; i++) os << "        if (lane < RAL_G * RAL_J + 2) s_vbw[" << i << "][lane] = 0u;\n";
        os << "        if (RAL_G * RAL_J + 2 > 32) {\n";
        os << "            for (int q = 32 + lane; q < RAL_G * RAL_J + 2; q += 32) {\n";
        for (int i = 0; i < NVO; i++) os << "                s_vbw[" << i << "][q] = 0u;\n";
        os << "            }\n        }\n";
        os << "        __syncwarp();\n";
        os << "        const ral_u64 a0 = excl & ~31ull;\n";
    }
    if (dense) {
        // Dense pass 2: lane k of step k0 takes the chunk's kept row k0 + k from the list, so
        // every lane evaluates a kept row (the last step excepted) and the stores of a step are
        // contiguous.  The projection's validity words of the chunk are staged first; each masked
        // output's bits of a step are one ballot, placed at the step's output positions.
        if (n_proj_vouts) {
            os << "        for (int wl = lane; wl < RAL_G * RAL_J; wl += 32) {\n";
            os << "            const ral_i64 w = (base >> 5) + wl;\n";
            os << "            ral_u32 pv[" << n_proj_vouts << "];\n";
            os << "            for (int i = 0; i < " << n_proj_vouts << "; ++i) pv[i] = 0u;\n";
            os << "            if ((w << 5) < n) ral_proj_vword(P, w, pv);\n";
            for (int i = 0; i < n_proj_vouts; i++) os << "            s_pvw[" << i << "][wl] = pv[" << i << "];\n";
            os << "        }\n";
        }
        os << "        __syncwarp();\n";
        // one step's row and loads (suffix sx; the step's first list position kx)
        auto step_loads = [&](const std::string& sx, const std::string& kx, const std::string& guard) {
            os << "            const ral_u32 k" << sx << " = " << kx << " + lane;\n";
            os << "            const bool act" << sx << " = " << guard << "k" << sx << " < total;\n";
            // an idle lane works on the step's first row and stores nothing
            os << "            const ral_u32 off" << sx << " = s_lst[act" << sx << " ? k" << sx << " : " << kx << "];\n";
            os << "            const ral_i64 row" << sx << " = base + off" << sx << ";\n";
            for (int k = 0; k < NO; k++) {
                if (f.outputs[k].from_project) continue;
                const int c = f.outputs[k].index;
                os << "            const " << element_ctype(f.frame_dtypes[c]) << " gv" << k << sx << " = " << fdata(c) << "[row"
                   << sx << "];\n";
            }
            if (any_proj) {
                for (size_t c = 0; c < f.project_cols.size(); c++)
                    if (proj_ref[c])
                        os << "            const " << element_ctype(f.frame_dtypes[f.project_cols[c]]) << " qa" << c << sx
                           << " = " << fdata(f.project_cols[c]) << "[row" << sx << "];\n";
                for (size_t c = 0; c < f.project_cols.size(); c++)
                    if (proj_raw[c]) {
                        const int fc = f.project_cols[c];
                        if (f.frame_has_valid[fc])
                            os << "            const ral_u32 qw" << c << sx << " = __ldg(" << fvalid(fc) << " + (row" << sx << " >> 5));\n";
                        else
                            os << "            const ral_u32 qw" << c << sx << " = 0xffffffffu;\n";
                    }
            }
        };
        // the step's outputs and validity bits
        auto step_outputs = [&](const std::string& sx, const std::string& kx, const std::string& ind) {
            os << ind << "const ral_u64 pos" << sx << " = excl + k" << sx << ";\n";
            os << ind << "if (act" << sx << ") {\n";
            for (int k = 0; k < NO; k++)
                if (!f.outputs[k].from_project) os << ind << "    o" << k << "[pos" << sx << "] = gv" << k << sx << ";\n";
            os << ind << "}\n";
            if (any_proj) {
                os << ind << "{\n";
                for (int o = 0; o < f.project->n_out; o++) os << ind << "    " << kind_ctype(proj_kind[o]) << " y" << o << ";\n";
                os << ind << "    ral_proj_row(P";
                for (size_t c = 0; c < f.project_cols.size(); c++)
                    if (proj_ref[c]) os << ", " << widen("qa" + std::to_string(c) + sx, f.frame_dtypes[f.project_cols[c]]);
                for (size_t c = 0; c < f.project_cols.size(); c++)
                    if (proj_raw[c]) os << ", (qw" << c << sx << " >> (int)(row" << sx << " & 31)) & 1u";
                for (int o = 0; o < f.project->n_out; o++) os << ", y" << o;
                os << ");\n";
                os << ind << "    if (act" << sx << ") {\n";
                for (int k = 0; k < NO; k++) {
                    if (!f.outputs[k].from_project) continue;
                    const int o = f.outputs[k].index;
                    os << ind << "        o" << k << "[pos" << sx << "] = " << narrow("y" + std::to_string(o), proj_kind[o], f.outputs[k].dtype)
                       << ";\n";
                }
                os << ind << "    }\n" << ind << "}\n";
            }
            for (int i = 0; i < NVO; i++) {
                const int k = vouts[i];
                const FilterOutput& o = f.outputs[k];
                os << ind << "{\n";
                if (o.from_project) {
                    int pi = 0;
                    for (size_t q = 0; q < proj_vouts.size(); q++)
                        if (proj_vouts[q] == o.index) pi = (int)q;
                    os << ind << "    const ral_u32 vw = s_pvw[" << pi << "][off" << sx << " >> 5];\n";
                } else {
                    os << ind << "    const ral_u32 vw = __ldg(" << fvalid(o.index) << " + (row" << sx << " >> 5));\n";
                }
                os << ind << "    const ral_u32 bal = __ballot_sync(0xffffffffu, act" << sx << " && ((vw >> (off" << sx << " & 31u)) & 1u));\n";
                os << ind << "    if (lane == 0 && bal) {\n";
                os << ind << "        vcnt[" << i << "] += __popc(bal);\n";
                os << ind << "        const ral_u64 X = (ral_u64)bal << (excl & 31u);\n";
                os << ind << "        s_vbw[" << i << "][(" << kx << ") >> 5] |= (ral_u32)X;\n";
                os << ind << "        s_vbw[" << i << "][((" << kx << ") >> 5) + 1] |= (ral_u32)(X >> 32);\n";
                os << ind << "    }\n";
                os << ind << "}\n";
            }
        };
        if (s.dense_unroll >= 2) {
            // two steps per iteration: both steps' loads are in flight before either computes; the
            // second step computes only when it holds rows (a warp-uniform test)
            os << "        for (ral_u32 k0 = 0; k0 < total; k0 += 64) {\n";
            os << "            const bool two = k0 + 32u < total;\n";
            os << "            const ral_u32 k1 = two ? k0 + 32u : k0;\n";
            step_loads("A", "k0", "");
            step_loads("B", "k1", "two && ");
            step_outputs("A", "k0", "            ");
            os << "            if (two) {\n";
            step_outputs("B", "k1", "                ");
            os << "            }\n";
        } else {
            os << "        for (ral_u32 k0 = 0; k0 < total; k0 += 32) {\n";
            step_loads("A", "k0", "");
            step_outputs("A", "k0", "            ");
        }
        os << "        }\n";
    } else {
        if (any_proj && !proj_vouts.empty()) os << "        ral_u32 pw[" << proj_vouts.size() << "];\n";
        // L2 prefetch of the columns pass 2 reads (not the predicate's, which pass 1 just read), a
        // block of PF slices ahead, when the chunk keeps enough rows for the data to be needed: one
        // cp.async.bulk.prefetch per column and block, issued by one lane each
        std::vector<int> pf_cols;
        if (s.prefetch > 0 && s.G > 1) {
            std::vector<bool> want(NF, false);
            for (const FilterOutput& o : f.outputs)
                if (!o.from_project) want[o.index] = true;
            for (size_t c = 0; c < f.project_cols.size(); c++)
                if (proj_ref[c]) want[f.project_cols[c]] = true;
            for (int c = 0; c < NF; c++)
                if (want[c] && !pred_col[c]) pf_cols.push_back(c);
            if ((int)pf_cols.size() > 32) pf_cols.resize(32);
        }
        const int PF = s.prefetch;
        auto emit_prefetch = [&](const std::string& ind, const std::string& first_slice) {
            if (pf_cols.empty()) return;
            os << ind << "if (pf_on) {\n";
            os << ind << "    const ral_i64 s0 = base + (ral_i64)(" << first_slice << ") * 32 * RAL_G;\n";
            os << ind << "    if (s0 < n) {\n";
            os << ind << "        const ral_i64 rows = (n - s0) < (ral_i64)" << PF << " * 32 * RAL_G ? (n - s0) : (ral_i64)" << PF
               << " * 32 * RAL_G;\n";
            for (size_t i = 0; i < pf_cols.size(); i++) {
                const int c = pf_cols[i];
                const int w = gdf_dtype_size(f.frame_dtypes[c]);
                os << ind << "        if (lane == " << i << ") ral_prefetch_l2(" << fdata(c) << " + s0, (unsigned)((rows * " << w
                   << ") & ~15ll));\n";
            }
            os << ind << "    }\n" << ind << "}\n";
        };
        os << "        ral_u64 sbase = excl;\n";
        if (!pf_cols.empty()) {
            os << "        const bool pf_on = (ral_u64)total * 8u >= (ral_u64)WT;\n";
            emit_prefetch("        ", "0");
            emit_prefetch("        ", std::to_string(PF));
        }
        os << "#pragma unroll 2\n        for (int j = 0; j < RAL_J; ++j) {\n";
        if (!pf_cols.empty()) {
            os << "            if (j % " << PF << " == 0 && j + " << 2 * PF << " < RAL_J) {\n";
            emit_prefetch("                ", "j + " + std::to_string(2 * PF));
            os << "            }\n";
        }
        os << "            const ral_u32 kb = (kbw[(j * RAL_G) >> 5] >> ((j * RAL_G) & 31)) & GMASK;\n";
        os << "            const ral_u32 c = __popc(kb);\n";
        os << "            ral_u32 inc = c;\n";
        os << "            for (int off = 1; off < 32; off <<= 1) {\n";
        os << "                const ral_u32 t = __shfl_up_sync(0xffffffffu, inc, off);\n";
        os << "                if (lane >= off) inc += t;\n            }\n";
        os << "            const ral_u32 stot = __shfl_sync(0xffffffffu, inc, 31);\n";
        os << "            if (stot == 0u) continue;\n";
        os << "            const ral_u64 pos0 = sbase + inc - c;\n";
        os << "            const ral_i64 r = base + (ral_i64)j * 32 * RAL_G + lane * RAL_G;\n";
        if (any_gather) {
            // every gathered column of the slice is loaded first (all loads in flight together);
            // a slice that keeps many rows is then written through the warp's stage as one
            // contiguous run per column, a sparse slice with direct stores
            for (int k = 0; k < NO; k++) {
                if (f.outputs[k].from_project) continue;
                const int c = f.outputs[k].index;
                const char* et = element_ctype(f.frame_dtypes[c]);
                os << "            " << et << " ga" << k << "[RAL_G];\n";
                os << "            if (kb) {\n";
                os << "                if (full) " << (pred_col[c] ? "ral_ldg_keep<" : "ral_ldg<") << et << ", RAL_G>(" << fdata(c)
                   << ", r, ga" << k << ");\n";
                os << "                else {\n#pragma unroll\n                    for (int g = 0; g < RAL_G; ++g) ga" << k
                   << "[g] = (r + g < n) ? " << fdata(c) << "[r + g] : (" << et << ")0;\n                }\n";
                os << "            }\n";
            }
            if (s.stage) {
                os << "            if (stot >= 16u) {\n";
                for (int k = 0; k < NO; k++) {
                    if (f.outputs[k].from_project) continue;
                    const char* et = element_ctype(f.frame_dtypes[f.outputs[k].index]);
                    os << "                {\n";
                    os << "                    " << et << "* const st = reinterpret_cast<" << et << "*>(s_stw);\n";
                    os << "                    ral_u32 q = inc - c;\n";
                    os << "#pragma unroll\n                    for (int g = 0; g < RAL_G; ++g)\n";
                    os << "                        if ((kb >> g) & 1u) st[q++] = ga" << k << "[g];\n";
                    os << "                    __syncwarp();\n";
                    os << "                    for (ral_u32 m = lane; m < stot; m += 32) o" << k << "[sbase + m] = st[m];\n";
                    os << "                    __syncwarp();\n";
                    os << "                }\n";
                }
                os << "            } else\n";
            }
            os << "            if (kb) {\n";
            for (int k = 0; k < NO; k++) {
                if (f.outputs[k].from_project) continue;
                os << "                {\n                    ral_u64 pos = pos0;\n";
                os << "#pragma unroll\n                    for (int g = 0; g < RAL_G; ++g)\n";
                os << "                        if ((kb >> g) & 1u) o" << k << "[pos++] = ga" << k << "[g];\n";
                os << "                }\n";
            }
            os << "            }\n";
        }
        if (any_proj) {
            if (!proj_vouts.empty()) {
                os << "            for (int i = 0; i < " << proj_vouts.size() << "; ++i) pw[i] = 0u;\n";
                os << "            if (lane < RAL_G) {\n";
                os << "                const ral_i64 w = (base >> 5) + (ral_i64)j * RAL_G + lane;\n";
                os << "                if ((w << 5) < n) ral_proj_vword(P, w, pw);\n";
                os << "            }\n";
            }
            os << "            if (kb) {\n";
            for (size_t c = 0; c < f.project_cols.size(); c++)
                if (proj_ref[c]) load(os, "                ", f.project_cols[c], "qa" + std::to_string(c));
            for (size_t c = 0; c < f.project_cols.size(); c++)
                if (proj_raw[c]) os << "                const ral_u32 qw" << c << " = " << raw_word(f.project_cols[c]) << ";\n";
            os << "                ral_u64 pos = pos0;\n";
            os << "#pragma unroll\n                for (int g = 0; g < RAL_G; ++g) {\n";
            os << "                    if (((kb >> g) & 1u) == 0u) continue;\n";
            for (int o = 0; o < f.project->n_out; o++) os << "                    " << kind_ctype(proj_kind[o]) << " y" << o << ";\n";
            os << "                    ral_proj_row(P";
            for (size_t c = 0; c < f.project_cols.size(); c++)
                if (proj_ref[c]) os << ", " << widen("qa" + std::to_string(c) + "[g]", f.frame_dtypes[f.project_cols[c]]);
            for (size_t c = 0; c < f.project_cols.size(); c++)
                if (proj_raw[c]) os << ", (qw" << c << " >> ((int)(r & 31) + g)) & 1u";
            for (int o = 0; o < f.project->n_out; o++) os << ", y" << o;
            os << ");\n";
            for (int k = 0; k < NO; k++) {
                if (!f.outputs[k].from_project) continue;
                const int o = f.outputs[k].index;
                os << "                    o" << k << "[pos] = " << narrow("y" + std::to_string(o), proj_kind[o], f.outputs[k].dtype) << ";\n";
            }
            os << "                    ++pos;\n                }\n";
            os << "            }\n";
        }
        // validity of the masked outputs for this slice, staged in the warp's shared-memory buffer
        for (int i = 0; i < NVO; i++) {
            const int k = vouts[i];
            const FilterOutput& o = f.outputs[k];
            os << "            {\n";
            if (o.from_project) {
                int pi = 0;
                for (size_t q = 0; q < proj_vouts.size(); q++)
                    if (proj_vouts[q] == o.index) pi = (int)q;
                os << "                const ral_u32 vw = __shfl_sync(0xffffffffu, pw[" << pi << "], (lane * RAL_G) >> 5);\n";
            } else {
                os << "                const ral_u32 vw = kb ? __ldg(" << fvalid(o.index) << " + (r >> 5)) : 0u;\n";
            }
            os << "                ral_u32 lb = 0, t = 0;\n";
            os << "#pragma unroll\n                for (int g = 0; g < RAL_G; ++g)\n";
            os << "                    if ((kb >> g) & 1u) { lb |= ((vw >> ((int)(r & 31) + g)) & 1u) << t; ++t; }\n";
            os << "                vcnt[" << i << "] += __popc(lb);\n";
            os << "                const ral_u32 q = (ral_u32)(pos0 - a0);\n";
            os << "                const ral_u64 X = (ral_u64)lb << (q & 31);\n";
            os << "                const ral_u32 qw = q >> 5;\n";
            os << "                const ral_u32 first = (ral_u32)(sbase - a0) >> 5;\n";
            os << "#pragma unroll\n                for (int kk = 0; kk <= RAL_G; ++kk) {\n";
            os << "                    const ral_u32 W = first + kk;\n";
            os << "                    const ral_u32 part = (t == 0u) ? 0u : (qw == W ? (ral_u32)X : (qw + 1u == W ? (ral_u32)(X >> 32) : 0u));\n";
            os << "                    const ral_u32 v = __reduce_or_sync(0xffffffffu, part);\n";
            os << "                    if (lane == 0 && v) s_vbw[" << i << "][W] |= v;\n";
            os << "                }\n";
            os << "            }\n";
        }
        os << "            sbase += stot;\n";
        os << "        }\n";
    }
    // flush the staged masks: edge words may be shared with neighbouring chunks
    if (NVO) {
        os << "        __syncwarp();\n";
        os << "        const ral_u32 nw = (ral_u32)(((excl - a0) + total + 31) >> 5);\n";
        for (int i = 0; i < NVO; i++) {
            const int k = vouts[i];
            os << "        for (ral_u32 q = lane; q < nw; q += 32) {\n";
            os << "            const ral_u32 v = s_vbw[" << i << "][q];\n";
            os << "            ral_u32* dst = ov" << k << " + (a0 >> 5) + q;\n";
            os << "            if (q == 0 || q == nw - 1) { if (v) atomicOr(dst, v); }\n";
            os << "            else *dst = v;\n";
            os << "        }\n";
        }
        os << "        __syncwarp();\n";
    }
    // the next chunk's pass 1 rewrites the list the lanes have just read
    if (dense && !NVO) os << "        __syncwarp();\n";
    if (grid) {
        os << "        }\n";  // total != 0
        os << "    }\n";      // pass-2 chunk loop
    } else if (pipe) {
        os << "        }\n";  // total != 0
        os << "        }\n";  // chunk A
        os << "        if (!moreB) break;\n";
        os << "        chunkA = chunkB;\n        totalA = totalB;\n        bufA = bufB;\n";
        os << "    }\n";
    } else {
        os << (item ? "    } while (0);\n" : "    }\n");  // chunk loop
    }

    // ---- valid-bit counts: one atomic per warp and masked output
    if (NVO) {
        os << "    const int vmap[" << NVO << "] = {";
        for (int i = 0; i < NVO; i++) os << (i ? ", " : "") << vouts[i];
        os << "};\n";
        os << "    for (int i = 0; i < " << NVO << "; ++i) {\n";
        os << "        const ral_u32 v = __reduce_add_sync(0xffffffffu, vcnt[i]);\n";
        os << "        if (lane == 0 && v) atomicAdd((unsigned long long*)(scratch + 3 + vmap[i]), (unsigned long long)v);\n";
        os << "    }\n";
    }
    if (grid) {
        // the grid counter takes a second step per block at the end (the launch moves it by twice
        // the grid); the block that completes it copies the header -- error count, kept count,
        // valid counts -- to the caller's host-mapped header and then writes the counter's final
        // value as the completion tag, so the host sees the result without a copy back
        os << "    __syncthreads();\n";
        os << "    if (threadIdx.x == 0) {\n";
        os << "        __threadfence();\n";
        os << "        const ral_u64 fin = RAL_EPOCH + 2ull * gridDim.x;\n";
        os << "        if (atomicAdd((unsigned long long*)scratch, 1ull) + 1ull == fin) {\n";
        os << "            __threadfence();\n";
        os << "            volatile ral_u64* const hm = (volatile ral_u64*)P.s[" << L.hostmap << "];\n";
        os << "            for (int i = 1; i < " << 3 + NO << "; ++i) hm[i] = ral_ld_status(scratch + i);\n";
        os << "            __threadfence_system();\n";
        os << "            hm[0] = fin;\n";
        os << "        }\n";
        os << "    }\n";
    }
    os << "}\n";
    gk.source = os.str();
    return gk;
}

// ---- delimited-text scan fused with its filter ---------------------------------------------
// One warp per chunk of 32 J lines (ticket order).  Pass 1: lane t of slice j takes line
// base + 32 j + t, finds its fields, parses the predicate's and evaluates the predicate (a blank
// or skipped line keeps nothing); the slice's keep bits are one ballot word.  The warp looks back
// for the chunk's output offset, turns the words into the kept-line list and, 32 kept lines per
// step, parses every projected field of line list[k] in lane k and stores it at offset + k; each
// output's validity bits of the step are one ballot, OR-ed in at the step's bit offset.
extern "C" const char* const ral_textscan_source;

GeneratedKernel generate_text_scan_kernel(const TextScanSpec& t, const Shape& s) {
    if (s.J < 1 || s.J > 32) throw std::runtime_error("text scan kernel shape: J out of range");
    GeneratedKernel gk;
    gk.shape = s;
    ParamLayout& L = gk.layout;
    const int NP = (int)t.dtypes.size();
    int slot = kTextScanFixedSlots;
    L.n_rows = 0;
    L.out_data = slot; slot += NP;
    L.out_valid = slot; slot += NP;
    L.scratch = slot++;
    const Program* pred = t.predicate;
    if (pred) {
        assign_scalar_slots(*pred, L, slot);
    }
    L.total = slot;

    // the file fields each pass needs: pass 1 the predicate's, pass 2 every projection's
    std::vector<bool> pred_ref = pred ? pred->inputs_referenced() : std::vector<bool>();
    std::vector<bool> pred_raw = pred ? pred->inputs_raw_valid() : std::vector<bool>();
    std::vector<int> f1, f2;  // sorted distinct file columns
    if (pred)
        for (size_t c = 0; c < t.predicate_cols.size(); c++)
            if (pred_ref[c] || pred_raw[c]) f1.push_back(t.file_cols[t.predicate_cols[c]]);
    for (int q = 0; q < NP; q++) f2.push_back(t.file_cols[q]);
    auto uniq = [](std::vector<int>& v) {
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
    };
    uniq(f1);
    uniq(f2);
    auto slot_of = [](const std::vector<int>& v, int fc) {
        return (int)(std::lower_bound(v.begin(), v.end(), fc) - v.begin());
    };

    std::ostringstream key;
    key << "textscan|";
    for (int q = 0; q < NP; q++) key << (int)t.dtypes[q] << "@" << t.file_cols[q] << ",";
    if (pred) {
        key << "|P" << pred->structure_key() << "@";
        for (int c : t.predicate_cols) key << c << ",";
    }
    key << "|J" << s.J << "T" << s.threads << "B" << s.min_blocks;
    char hex[32];
    snprintf(hex, sizeof hex, "%016llx", (unsigned long long)fnv1a(key.str()));
    gk.name = std::string("ral_textscan_") + hex;
    gk.soft_fp = true;

    std::ostringstream os;
    os << ral_textscan_source << "\n";
    os << "// generated: " << key.str() << "\n";
    os << "#define RAL_J " << s.J << "\n#define RAL_THREADS " << s.threads << "\n";
    os << "#define RAL_WARPS (RAL_THREADS / 32)\n";
    os << "struct RalParams { ral_u64 s[" << L.total << "]; };\n\n";
    std::vector<Kind> pred_kind;
    if (pred) {
        emit_row_function(os, *pred, L, "ral_pred_row");
        pred_kind = final_kinds(*pred, L);
        os << "RAL_FI ral_u32 ral_pred_vrow(const ral_u32* fv) {\n";
        ValidEmitter ve(*pred);
        ve.emit(os, "    ", [&](int c) { return "fv[" + std::to_string(c) + "]"; });
        os << "    return " << ve.name[pred->final_pos[0]] << ";\n}\n";
    }
    os << "RAL_FI void ral_text_line(const char* d, const ral_i64* ends, ral_i64 nterm, ral_i64 nb, ral_i64 i,\n"
          "                          ral_i64& s, ral_i64& e) {\n"
          "    s = i == 0 ? 0 : ends[i - 1] + 1;\n"
          "    e = i < nterm ? ends[i] : nb;\n"
          "    if (e > s && d[e - 1] == '\\r') --e;\n"
          "}\n";
    // The text [S, E) of up to 32 lines copied into the warp's stage by all lanes (16-byte loads
    // where the text allows, never past its end), so that the lanes' byte-by-byte parsing reads
    // shared memory instead of 32 lines' worth of global addresses per instruction.  Returns the
    // pointer through which text position p reads its staged copy, or the text itself when the
    // span does not fit.
    os << "#define RAL_STAGE 4096\n";
    os << "RAL_FI const char* ral_text_stage(const char* d, ral_i64 nb, ral_i64 S, ral_i64 E, char* stage, int lane) {\n"
          "    const ral_i64 a = S & ~15ll;\n"
          "    if (E <= S || E - a > RAL_STAGE) return d;\n"
          "    __syncwarp();\n"
          "    if ((((unsigned long long)d) & 15ull) == 0ull) {\n"
          "        for (ral_i64 o = a + 16 * lane; o < E; o += 512) {\n"
          "            if (o + 16 <= nb) {\n"
          "                *reinterpret_cast<uint4*>(stage + (o - a)) = __ldcs(reinterpret_cast<const uint4*>(d + o));\n"
          "            } else {\n"
          "                for (ral_i64 k = o; k < nb; ++k) stage[k - a] = d[k];\n"
          "            }\n"
          "        }\n"
          "    } else {\n"
          "        for (ral_i64 o = a + lane; o < E; o += 32) stage[o - a] = d[o];\n"
          "    }\n"
          "    __syncwarp();\n"
          "    return stage - a;\n"
          "}\n";
    // field finders: the bounds of each needed field of a line (-1 where the line is shorter)
    auto finder = [&](const char* name, const std::vector<int>& fields) {
        os << "RAL_FI void " << name << "(const char* d, ral_i64 s, ral_i64 e, char delim, ral_i64* fs, ral_i64* fe) {\n";
        os << "#pragma unroll\n    for (int k = 0; k < " << fields.size() << "; ++k) { fs[k] = -1; fe[k] = -1; }\n";
        os << "    int f = 0;\n    ral_i64 p0 = s;\n";
        os << "    for (ral_i64 p = s;; ++p) {\n";
        os << "        const bool end = p >= e;\n";
        os << "        if (end || d[p] == delim) {\n";
        os << "            switch (f) {\n";
        for (size_t k = 0; k < fields.size(); k++)
            os << "            case " << fields[k] << ": fs[" << k << "] = p0; fe[" << k << "] = p; break;\n";
        os << "            default: break;\n            }\n";
        os << "            if (end || f >= " << fields.back() << ") break;\n";
        os << "            ++f;\n            p0 = p + 1;\n";
        os << "        }\n    }\n}\n";
    };
    if (!f1.empty()) finder("ral_fields_pred", f1);
    finder("ral_fields_all", f2);
    // parse of one field into a register value (column value widened) and a validity word
    // (a refusal is counted where `counts` holds: idle lanes of pass 2 parse a kept line twice)
    auto parse = [&](const std::string& ind, gdf_dtype dt, const std::string& k, const std::string& v,
                     const std::string& vw, const std::string& counts) {
        const bool isf = dt == GDF_FLOAT32 || dt == GDF_FLOAT64;
        os << ind << (isf ? "double " : "ral_i64 ") << v << " = 0;\n";
        os << ind << "ral_u32 " << vw << " = 0u;\n";
        os << ind << "if (fs[" << k << "] >= 0) {\n";
        if (isf) os << ind << "    double t = 0.0;\n" << ind << "    const int st = ral_tx_parse_double(ds, fs[" << k << "], fe[" << k << "], &t);\n";
        else if (dt == GDF_DATE32 || dt == GDF_DATE64)
            os << ind << "    long long t = 0;\n" << ind << "    const int st = ral_tx_parse_date(ds, fs[" << k << "], fe[" << k
               << "], " << (dt == GDF_DATE64 ? "true" : "false") << ", &t);\n";
        else os << ind << "    long long t = 0;\n" << ind << "    const int st = ral_tx_parse_int(ds, fs[" << k << "], fe[" << k << "], &t);\n";
        os << ind << "    if (st == RAL_TX_REFUSED && " << counts << ") ++refused;\n";
        os << ind << "    if (st == RAL_TX_OK) {\n";
        os << ind << "        " << vw << " = 0xffffffffu;\n";
        switch (dt) {
        case GDF_INT8: os << ind << "        " << v << " = (ral_i64)(signed char)t;\n"; break;
        case GDF_INT16: os << ind << "        " << v << " = (ral_i64)(short)t;\n"; break;
        case GDF_INT32: case GDF_DATE32: os << ind << "        " << v << " = (ral_i64)(int)t;\n"; break;
        case GDF_FLOAT32: os << ind << "        " << v << " = (double)(float)t;\n"; break;
        default: os << ind << "        " << v << " = t;\n"; break;
        }
        os << ind << "    }\n" << ind << "}\n";
    };

    os << "\nextern \"C\" __global__ void __launch_bounds__(RAL_THREADS, " << std::max(1, s.min_blocks) << ") " << gk.name
       << "(const __grid_constant__ RalParams P) {\n";
    os << "    __shared__ ral_u32 s_kp[RAL_WARPS][32];\n";
    os << "    __shared__ unsigned short s_ls[RAL_WARPS][32 * RAL_J];\n";
    os << "    __shared__ __align__(16) char s_tx[RAL_WARPS][RAL_STAGE];\n";
    os << "    const ral_i64 T = (ral_i64)P.s[0];\n";
    os << "    const char* const d = (const char*)P.s[1];\n";
    os << "    const ral_i64 nb = (ral_i64)P.s[2];\n";
    os << "    const ral_i64* const ends = (const ral_i64*)P.s[3];\n";
    os << "    const ral_i64 nterm = (ral_i64)P.s[4];\n";
    os << "    const ral_i64 skip = (ral_i64)P.s[5];\n";
    os << "    const char delim = (char)P.s[6];\n";
    os << "    const ral_u64 cap = (ral_u64)P.s[7];\n";
    os << "    const ral_u64 obase = (ral_u64)P.s[8];\n";
    os << "    ral_u64* const scratch = (ral_u64*)P.s[" << L.scratch << "];\n";
    os << "    ral_u64* const status = scratch + " << text_scan_header(NP) << ";\n";
    for (int q = 0; q < NP; q++) {
        os << "    " << element_ctype(t.dtypes[q]) << "* __restrict__ o" << q << " = (" << element_ctype(t.dtypes[q])
           << "*)P.s[" << L.out_data + q << "];\n";
        os << "    ral_u32* __restrict__ ov" << q << " = (ral_u32*)P.s[" << L.out_valid + q << "];\n";
    }
    os << "    const int lane = threadIdx.x & 31;\n    const int warp = threadIdx.x >> 5;\n";
    os << "    ral_u32* const s_kpw = s_kp[warp];\n    unsigned short* const s_lst = s_ls[warp];\n";
    os << "    char* const s_txw = s_tx[warp];\n";
    os << "    const ral_i64 CL = 32 * RAL_J;\n    const ral_i64 nchunks = (T + CL - 1) / CL;\n";
    os << "    ral_u32 vcnt[" << NP << "];\n    for (int q = 0; q < " << NP << "; ++q) vcnt[q] = 0u;\n";
    os << "    ral_u32 refused = 0, over = 0;\n";
    os << "    for (;;) {\n";
    os << "        ral_u32 ticket = 0;\n";
    os << "        if (lane == 0) ticket = atomicAdd((unsigned int*)scratch, 1u);\n";
    os << "        const ral_i64 chunk = __shfl_sync(0xffffffffu, ticket, 0);\n";
    os << "        if (chunk >= nchunks) break;\n";
    os << "        const ral_i64 base = chunk * CL;\n";
    os << "        ral_u32 total = 0;\n";
    os << "        for (int j = 0; j < RAL_J; ++j) {\n";
    os << "            const ral_i64 i0 = base + (ral_i64)j * 32;\n";
    os << "            if (i0 >= T) {\n";
    os << "                if (lane == j) s_kpw[j] = 0u;\n";
    os << "                continue;\n";
    os << "            }\n";
    os << "            const ral_i64 i = i0 + lane;\n";
    os << "            const char* ds = d;\n";
    if (pred) {
        // the slice's lines staged only when the condition has fields to parse
        os << "            {\n";
        os << "                const ral_i64 i1 = i0 + 31 < T ? i0 + 31 : T - 1;\n";
        os << "                const ral_i64 S = i0 == 0 ? 0 : ends[i0 - 1] + 1;\n";
        os << "                const ral_i64 E = i1 < nterm ? ends[i1] : nb;\n";
        os << "                ds = ral_text_stage(d, nb, S, E, s_txw, lane);\n";
        os << "            }\n";
    }
    os << "            bool keep = false;\n";
    os << "            if (i < T && i >= skip) {\n";
    os << "                ral_i64 s, e;\n";
    os << "                ral_text_line(ds, ends, nterm, nb, i, s, e);\n";
    os << "                keep = e > s;\n";
    if (pred) {
        os << "                if (keep) {\n";
        if (!f1.empty()) {
            os << "                    ral_i64 fs[" << f1.size() << "], fe[" << f1.size() << "];\n";
            os << "                    ral_fields_pred(ds, s, e, delim, fs, fe);\n";
        }
        os << "                    ral_u32 fv[" << std::max<size_t>(1, t.predicate_cols.size()) << "];\n";
        for (size_t c = 0; c < t.predicate_cols.size(); c++) {
            const int q = t.predicate_cols[c];
            if (!(pred_ref[c] || pred_raw[c])) {
                os << "                    fv[" << c << "] = 0xffffffffu;\n";
                continue;
            }
            parse("                    ", t.dtypes[q], std::to_string(slot_of(f1, t.file_cols[q])), "x" + std::to_string(c),
                  "w" + std::to_string(c), "true");
            os << "                    fv[" << c << "] = w" << c << ";\n";
        }
        os << "                    " << kind_ctype(pred_kind[0]) << " y0;\n";
        os << "                    ral_pred_row(P";
        for (size_t c = 0; c < t.predicate_cols.size(); c++)
            if (pred_ref[c]) os << ", x" << c;
        for (size_t c = 0; c < t.predicate_cols.size(); c++)
            if (pred_raw[c]) os << ", w" << c << " & 1u";
        os << ", y0);\n";
        os << "                    keep = (ral_pred_vrow(fv) & 1u) != 0u && " << narrow("y0", pred_kind[0], GDF_INT8)
           << " != 0;\n";
        os << "                }\n";
    }
    os << "            }\n";
    os << "            const ral_u32 w = __ballot_sync(0xffffffffu, keep);\n";
    os << "            if (lane == j) s_kpw[j] = w;\n";
    os << "            total += __popc(w);\n";
    os << "        }\n";
    os << "        __syncwarp();\n";
    os << "        const ral_u64 excl = ral_lookback(status, chunk, total, scratch + 1);\n";
    os << "        if (chunk == nchunks - 1 && lane == 0) scratch[2] = excl + total;\n";
    os << "        if (total == 0u) continue;\n";
    os << "        {\n";
    os << "            const ral_u32 kw = lane < RAL_J ? s_kpw[lane] : 0u;\n";
    os << "            const ral_u32 c = __popc(kw);\n";
    os << "            ral_u32 inc = c;\n";
    os << "            for (int off = 1; off < 32; off <<= 1) {\n";
    os << "                const ral_u32 u = __shfl_up_sync(0xffffffffu, inc, off);\n";
    os << "                if (lane >= off) inc += u;\n            }\n";
    os << "            ral_u32 q = inc - c;\n";
    os << "            for (ral_u32 m = kw; m; m &= m - 1u) s_lst[q++] = (unsigned short)(lane * 32 + __ffs(m) - 1);\n";
    os << "        }\n";
    os << "        __syncwarp();\n";
    os << "        for (ral_u32 k0 = 0; k0 < total; k0 += 32) {\n";
    os << "            const ral_u32 kA = k0 + lane;\n";
    os << "            const bool act = kA < total;\n";
    os << "            const ral_i64 i = base + s_lst[act ? kA : k0];\n";
    os << "            const char* ds = d;\n";
    os << "            {\n";
    os << "                const ral_i64 i0 = base + s_lst[k0];\n";
    os << "                const ral_i64 i1 = base + s_lst[k0 + 31u < total ? k0 + 31u : total - 1u];\n";
    os << "                const ral_i64 S = i0 == 0 ? 0 : ends[i0 - 1] + 1;\n";
    os << "                const ral_i64 E = i1 < nterm ? ends[i1] : nb;\n";
    os << "                ds = ral_text_stage(d, nb, S, E, s_txw, lane);\n";
    os << "            }\n";
    os << "            ral_i64 s, e;\n";
    os << "            ral_text_line(ds, ends, nterm, nb, i, s, e);\n";
    os << "            ral_i64 fs[" << f2.size() << "], fe[" << f2.size() << "];\n";
    os << "            ral_fields_all(ds, s, e, delim, fs, fe);\n";
    os << "            const ral_u64 pos0 = excl + kA;\n";
    os << "            const bool put = act && pos0 < cap;\n";
    os << "            if (act && !put) ++over;\n";
    os << "            const ral_u64 pos = pos0 + obase;\n";
    os << "            const ral_u64 b = excl + k0 + obase;\n";
    for (int q = 0; q < NP; q++) {
        os << "            {\n";
        parse("                ", t.dtypes[q], std::to_string(slot_of(f2, t.file_cols[q])), "v", "vw", "act");
        os << "                if (put) o" << q << "[pos] = (" << element_ctype(t.dtypes[q]) << ")v;\n";
        os << "                const ral_u32 bal = __ballot_sync(0xffffffffu, put && vw != 0u);\n";
        os << "                if (lane == 0 && bal) {\n";
        os << "                    vcnt[" << q << "] += __popc(bal);\n";
        os << "                    const ral_u64 X = (ral_u64)bal << (b & 31u);\n";
        os << "                    atomicOr(ov" << q << " + (b >> 5), (ral_u32)X);\n";
        os << "                    if ((ral_u32)(X >> 32)) atomicOr(ov" << q << " + (b >> 5) + 1, (ral_u32)(X >> 32));\n";
        os << "                }\n";
        os << "            }\n";
    }
    os << "        }\n";
    os << "        __syncwarp();\n";
    os << "    }\n";
    // counts: one atomic per warp and counter
    os << "    for (int q = 0; q < " << NP << "; ++q) {\n";
    os << "        const ral_u32 v = __reduce_add_sync(0xffffffffu, vcnt[q]);\n";
    os << "        if (lane == 0 && v) atomicAdd((unsigned long long*)(scratch + 3 + q), (unsigned long long)v);\n";
    os << "    }\n";
    os << "    const ral_u32 rf = __reduce_add_sync(0xffffffffu, refused);\n";
    os << "    const ral_u32 ov = __reduce_add_sync(0xffffffffu, over);\n";
    os << "    if (lane == 0 && rf) atomicAdd((unsigned long long*)(scratch + " << 3 + NP << "), (unsigned long long)rf);\n";
    os << "    if (lane == 0 && ov) atomicAdd((unsigned long long*)(scratch + " << 4 + NP << "), (unsigned long long)ov);\n";
    os << "}\n";
    gk.source = os.str();
    return gk;
}

GeneratedKernel generate_batch_item(const Program& p, const Shape& sh) {
    GeneratedKernel gk;
    gk.shape = sh;
    gk.layout = make_layout(p, 0);
    const ParamLayout& L = gk.layout;
    std::ostringstream key;
    key << "item|" << p.structure_key() << "#" << sh.G << "/" << sh.J << "/" << sh.unroll << (sh.soft ? "/s" : "");
    char hex[32];
    snprintf(hex, sizeof hex, "%016llx", (unsigned long long)fnv1a(key.str()));
    gk.name = std::string("ral_item_") + hex;
    gk.soft_fp = sh.soft;
    const std::string sfx = hex;

    std::ostringstream os;
    os << "// generated: one warp tile of a batched program\n";
    os << "struct RalParams { ral_u64 s[" << L.total << "]; };\n\n";
    const auto ref = p.inputs_referenced();
    const auto raw = p.inputs_raw_valid();
    const auto fk = final_kinds(p, L);
    std::vector<int> vouts;
    for (int o = 0; o < p.n_out; o++)
        if (p.out_has_valid[o]) vouts.push_back(o);
    const int NOV = (int)vouts.size();
    emit_row_function(os, p, L, ("ral_row_" + sfx).c_str());
    if (NOV > 0) {
        os << "RAL_FI void ral_vword_" << sfx << "(const RalParams& P, const ral_i64 w, ral_u32* vo) {\n";
        ValidEmitter ve(p);
        ve.emit(os, "    ", [&](int c) {
            return "__ldg(((const ral_u32*)P.s[" + std::to_string(L.in_valid + c) + "]) + w)";
        });
        for (int i = 0; i < NOV; i++) os << "    vo[" << i << "] = " << ve.name[p.final_pos[vouts[i]]] << ";\n";
        os << "}\n";
    }
    // one warp tile of this program
    os << "extern \"C\" __device__ __noinline__ void " << gk.name
       << "(const ral_u64* __restrict__ slots, const ral_i64 t) {\n";
    os << "    const RalParams& P = *reinterpret_cast<const RalParams*>(slots);\n";
    os << "    const int G = " << sh.G << ", J = " << sh.J << ";\n";
    os << "    const int lane = threadIdx.x & 31;\n";
    os << "    const ral_i64 n = (ral_i64)P.s[" << L.n_rows << "];\n";
    for (int c = 0; c < p.n_in; c++) {
        if (ref[c])
            os << "    const " << element_ctype(p.inputs[c].dtype) << "* __restrict__ pin" << c << " = (const "
               << element_ctype(p.inputs[c].dtype) << "*)P.s[" << L.in_data + c << "];\n";
        if (raw[c] && p.inputs[c].has_valid)
            os << "    const ral_u32* __restrict__ pvr" << c << " = (const ral_u32*)P.s[" << L.in_valid + c << "];\n";
    }
    for (int o = 0; o < p.n_out; o++)
        os << "    " << element_ctype(p.out_dtypes[o]) << "* __restrict__ pout" << o << " = ("
           << element_ctype(p.out_dtypes[o]) << "*)P.s[" << L.out_data + o << "];\n";
    for (int i = 0; i < NOV; i++)
        os << "    ral_u32* __restrict__ pvo" << i << " = (ral_u32*)P.s[" << L.out_valid + vouts[i] << "];\n";
    os << "    const ral_i64 TILE = 32 * G * J;\n";
    os << "    const ral_i64 base = t * TILE;\n";
    os << "    if (base + TILE <= n) {\n";
    os << "#pragma unroll " << std::max(1, std::min(sh.unroll, sh.J)) << "\n        for (int j = 0; j < J; ++j) {\n";
    os << "            const ral_i64 r = base + (ral_i64)j * 32 * G + lane * G;\n";
    for (int c = 0; c < p.n_in; c++) {
        if (!ref[c]) continue;
        const char* et = element_ctype(p.inputs[c].dtype);
        os << "            " << et << " a" << c << "[" << sh.G << "]; ral_ldg<" << et << ", " << sh.G << ">(pin" << c
           << ", r, a" << c << ");\n";
    }
    for (int c = 0; c < p.n_in; c++) {
        if (!raw[c]) continue;
        if (p.inputs[c].has_valid) os << "            const ral_u32 rw" << c << " = __ldg(pvr" << c << " + (r >> 5));\n";
        else os << "            const ral_u32 rw" << c << " = 0xffffffffu;\n";
    }
    for (int o = 0; o < p.n_out; o++)
        os << "            " << element_ctype(p.out_dtypes[o]) << " b" << o << "[" << sh.G << "];\n";
    os << "#pragma unroll\n            for (int g = 0; g < G; ++g) {\n";
    for (int o = 0; o < p.n_out; o++) os << "                " << kind_ctype(fk[o]) << " y" << o << ";\n";
    os << "                ral_row_" << sfx << "(P";
    for (int c = 0; c < p.n_in; c++)
        if (ref[c]) os << ", " << widen("a" + std::to_string(c) + "[g]", p.inputs[c].dtype);
    for (int c = 0; c < p.n_in; c++)
        if (raw[c]) os << ", (rw" << c << " >> ((int)(r & 31) + g)) & 1u";
    for (int o = 0; o < p.n_out; o++) os << ", y" << o;
    os << ");\n";
    for (int o = 0; o < p.n_out; o++)
        os << "                b" << o << "[g] = " << narrow("y" + std::to_string(o), fk[o], p.out_dtypes[o]) << ";\n";
    os << "            }\n";
    for (int o = 0; o < p.n_out; o++)
        os << "            ral_stg<" << element_ctype(p.out_dtypes[o]) << ", " << sh.G << ">(pout" << o << ", r, b" << o << ");\n";
    os << "        }\n";
    if (NOV > 0) {
        os << "        for (int wl = lane; wl < G * J; wl += 32) {\n";
        os << "            const ral_i64 w = (base >> 5) + wl;\n";
        os << "            ral_u32 vo[" << NOV << "]; ral_vword_" << sfx << "(P, w, vo);\n";
        for (int i = 0; i < NOV; i++) os << "            pvo" << i << "[w] = vo[" << i << "];\n";
        os << "        }\n";
    }
    os << "    } else {\n";
    os << "        for (ral_i64 r = base + lane; r < n; r += 32) {\n";
    for (int c = 0; c < p.n_in; c++) {
        if (!raw[c]) continue;
        if (p.inputs[c].has_valid) os << "            const ral_u32 rw" << c << " = __ldg(pvr" << c << " + (r >> 5));\n";
        else os << "            const ral_u32 rw" << c << " = 0xffffffffu;\n";
    }
    for (int o = 0; o < p.n_out; o++) os << "            " << kind_ctype(fk[o]) << " y" << o << ";\n";
    os << "            ral_row_" << sfx << "(P";
    for (int c = 0; c < p.n_in; c++)
        if (ref[c]) os << ", " << widen("pin" + std::to_string(c) + "[r]", p.inputs[c].dtype);
    for (int c = 0; c < p.n_in; c++)
        if (raw[c]) os << ", (rw" << c << " >> (int)(r & 31)) & 1u";
    for (int o = 0; o < p.n_out; o++) os << ", y" << o;
    os << ");\n";
    for (int o = 0; o < p.n_out; o++)
        os << "            pout" << o << "[r] = " << narrow("y" + std::to_string(o), fk[o], p.out_dtypes[o]) << ";\n";
    os << "        }\n";
    if (NOV > 0) {
        os << "        const ral_i64 wend = (n + 31) >> 5;\n";
        os << "        for (ral_i64 w = (base >> 5) + lane; w < wend; w += 32) {\n";
        os << "            ral_u32 vo[" << NOV << "]; ral_vword_" << sfx << "(P, w, vo);\n";
        for (int i = 0; i < NOV; i++) os << "            pvo" << i << "[w] = vo[" << i << "];\n";
        os << "        }\n";
    }
    os << "    }\n";
    os << "}\n\n";
    gk.source = os.str();
    return gk;
}

GeneratedKernel generate_batch_dispatch(const std::vector<DispatchEntry>& items, int smem_words_per_warp, int grab) {
    GeneratedKernel gk;
    grab = std::max(1, std::min(grab, 64));
    std::ostringstream key;
    key << "dispatch|" << smem_words_per_warp << "|g" << grab << "|";
    for (const auto& it : items) key << it.name << (it.filter ? "f" : "") << ";";
    char hex[32];
    snprintf(hex, sizeof hex, "%016llx", (unsigned long long)fnv1a(key.str()));
    gk.name = std::string("ral_batch_") + hex;
    const int NF = (int)items.size();
    std::ostringstream os;
    os << "// generated: persistent dispatcher over " << NF << " item functions\n";
    for (const auto& it : items) {
        if (it.filter)
            os << "extern \"C\" __device__ void " << it.name
               << "(const ral_u64* __restrict__ slots, const ral_i64 t, ral_u32* __restrict__ wsm);\n";
        else
            os << "extern \"C\" __device__ void " << it.name << "(const ral_u64* __restrict__ slots, const ral_i64 t);\n";
    }
    os << "#define RAL_BATCH_GRAB " << grab << "\n";
    // dynamic shared memory: item prefix (n_programs + 1 long longs), one function index per
    // program, then each warp's area for filter items
    os << "extern \"C\" __global__ void __launch_bounds__(256) " << gk.name
       << "(const ral_u64* __restrict__ descs, const int stride, const long long* __restrict__ item_prefix, "
          "const long long* __restrict__ item_base, const int* __restrict__ fn_index, const int np, "
          "unsigned int* counter, const long long total_items) {\n";
    os << "    extern __shared__ long long s_prefix[];\n";
    os << "    long long* s_base = s_prefix + np + 1;\n";
    os << "    int* s_fn = reinterpret_cast<int*>(s_base + np);\n";
    os << "    for (int i = threadIdx.x; i <= np; i += blockDim.x) s_prefix[i] = item_prefix[i];\n";
    // item t of entry q is the entry's tile / chunk item_base[q] + t (0 without item_base)
    os << "    for (int i = threadIdx.x; i < np; i += blockDim.x) s_base[i] = item_base ? item_base[i] : 0;\n";
    os << "    for (int i = threadIdx.x; i < np; i += blockDim.x) s_fn[i] = fn_index[i];\n";
    os << "    __syncthreads();\n";
    os << "    const int lane = threadIdx.x & 31;\n";
    if (smem_words_per_warp > 0) {
        os << "    const size_t head = ((size_t)(np + 1) * 8 + (size_t)np * 12 + 15) & ~(size_t)15;\n";
        os << "    ral_u32* const wsm = reinterpret_cast<ral_u32*>(reinterpret_cast<char*>(s_prefix) + head) + "
              "(threadIdx.x >> 5) * " << smem_words_per_warp << ";\n";
    }
    os << "    for (;;) {\n";
    os << "        unsigned int got = 0;\n";
    os << "        if (lane == 0) got = atomicAdd(counter, (unsigned int)RAL_BATCH_GRAB);\n";
    os << "        const long long first = (long long)__shfl_sync(0xffffffffu, got, 0);\n";
    os << "        if (first >= total_items) break;\n";
    os << "        const long long last = first + RAL_BATCH_GRAB < total_items ? first + RAL_BATCH_GRAB : total_items;\n";
    os << "        int lo = 0;\n";
    os << "        for (long long item = first; item < last; ++item) {\n";
    // largest q with s_prefix[q] <= item; items of one grab are consecutive, so start from the last q
    os << "            if (s_prefix[lo + 1] <= item) {\n";
    os << "                int hi = np;\n";
    os << "                while (hi - lo > 1) { const int mid = (lo + hi) >> 1; if (s_prefix[mid] <= item) lo = mid; else hi = mid; }\n";
    os << "            }\n";
    os << "            const ral_i64 t = item - s_prefix[lo] + s_base[lo];\n";
    os << "            const ral_u64* slots = descs + (size_t)lo * stride;\n";
    os << "            switch (s_fn[lo]) {\n";
    for (int f = 0; f < NF; f++)
        os << "            case " << f << ": " << items[f].name << (items[f].filter ? "(slots, t, wsm)" : "(slots, t)")
           << "; break;\n";
    os << "            default: break;\n";
    os << "            }\n";
    os << "        }\n";
    os << "    }\n";
    os << "}\n";
    gk.source = os.str();
    return gk;
}

}  // namespace ral
