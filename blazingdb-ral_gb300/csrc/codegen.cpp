// codegen.cpp — emits one CUDA kernel per register program.
#include "codegen.h"

#include <algorithm>
#include <functional>
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
    s.threads = 256;
    s.min_blocks = 1;
    return s;
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
    return to == Kind::F64 ? "((double)(" + b + "))" : "((ral_i64)(" + b + "))";
}

// Data-path op emission shared by every kernel kind.
struct OpEmitter {
    const Program& p;
    const ParamLayout& L;
    std::vector<std::string> name;   // current SSA value of each register
    std::vector<Kind> kind;

    OpEmitter(const Program& prog, const ParamLayout& layout) : p(prog), L(layout) {
        int maxreg = p.n_in;
        for (const Op& op : p.ops) maxreg = std::max<int>(maxreg, op.out);
        for (int16_t f : p.final_pos) maxreg = std::max<int>(maxreg, f);
        name.assign(maxreg + 1, "");
        kind.assign(maxreg + 1, Kind::I64);
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
            if (op.left >= 0) {
                l = name[op.left];
            } else if (op.left == SCALAR_INDEX) {
                l = "sl" + std::to_string(k);
                os << indent << "const " << kind_ctype(lk) << " " << l << " = "
                   << (lk == Kind::F64 ? "ral_bits_d((ral_i64)P.s[" : "((ral_i64)P.s[") << L.lscalar_slot[k]
                   << "]);\n";
            } else {
                l = lk == Kind::F64 ? "0.0" : "((ral_i64)0)";
            }
            if (!op.unary) {
                if (op.right >= 0) {
                    r = name[op.right];
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
            if (!op.unary) {
                const bool f = (lk == Kind::F64) || (rk == Kind::F64);
                auto arith = [&](const char* dop, const char* iop) {
                    if (f) return conv(std::string(dop) + "(" + to_d(l, lk) + ", " + to_d(r, rk) + ")", Kind::F64, ok);
                    return conv(std::string(iop) + "(" + l + ", " + r + ")", Kind::I64, ok);
                };
                auto cmp = [&](const char* c) {
                    if (f) return conv_bool(to_d(l, lk) + " " + c + " " + to_d(r, rk), ok);
                    return conv_bool(l + " " + c + " " + r, ok);
                };
                switch (op.bop) {
                case GDF_ADD: e = arith("__dadd_rn", "ral_addi"); break;
                case GDF_SUB: e = arith("__dsub_rn", "ral_subi"); break;
                case GDF_MUL: e = arith("__dmul_rn", "ral_muli"); break;
                case GDF_DIV: case GDF_FLOOR_DIV: e = arith("__ddiv_rn", "ral_divi"); break;
                case GDF_MOD: e = conv("ral_modi(" + to_i(l, lk) + ", " + to_i(r, rk) + ")", Kind::I64, ok); break;
                case GDF_POW:
                    if (dtype_is_float(op.ltype) || dtype_is_float(op.rtype))
                        e = conv("pow(" + to_d(l, lk) + ", " + to_d(r, rk) + ")", Kind::F64, ok);
                    else
                        e = conv("ral_powi(" + l + ", " + r + ")", Kind::I64, ok);
                    break;
                case GDF_EQUAL: e = cmp("=="); break;
                case GDF_NOT_EQUAL: e = cmp("!="); break;
                case GDF_LESS: e = cmp("<"); break;
                case GDF_GREATER: e = cmp(">"); break;
                case GDF_LESS_EQUAL: e = cmp("<="); break;
                case GDF_GREATER_EQUAL: e = cmp(">="); break;
                case GDF_COALESCE:
                    e = "(rb" + std::to_string(op.left) + " ? " + conv(l, lk, ok) + " : " + conv(r, rk, ok) + ")";
                    break;
                default: throw std::runtime_error("codegen: unsupported binary operator");
                }
            } else {
                const std::string d = to_d(l, lk);
                const bool d32 = op.ltype == GDF_DATE32;
                auto math = [&](const std::string& fn) { return conv(fn + "(" + d + ")", Kind::F64, ok); };
                switch (op.uop) {
                case BLZ_FLOOR: e = math("floor"); break;
                case BLZ_CEIL: e = math("ceil"); break;
                case BLZ_SIN: e = math("sin"); break;
                case BLZ_COS: e = math("cos"); break;
                case BLZ_ASIN: e = math("asin"); break;
                case BLZ_ACOS: e = math("acos"); break;
                case BLZ_TAN: e = math("tan"); break;
                case BLZ_COTAN: e = conv("__ddiv_rn(cos(" + d + "), sin(" + d + "))", Kind::F64, ok); break;
                case BLZ_ATAN: e = math("atan"); break;
                case BLZ_ABS: e = math("fabs"); break;
                case BLZ_LN: e = math("log"); break;
                case BLZ_LOG: e = math("log10"); break;
                case BLZ_NOT: e = conv_bool(lk == Kind::F64 ? "(" + l + " == 0.0)" : "(" + l + " == 0)", ok); break;
                case BLZ_YEAR: e = conv(std::string(d32 ? "ral_year32(" : "ral_year64(") + to_i(l, lk) + ")", Kind::I64, ok); break;
                case BLZ_MONTH: e = conv(std::string(d32 ? "ral_month32(" : "ral_month64(") + to_i(l, lk) + ")", Kind::I64, ok); break;
                case BLZ_DAY: e = conv(std::string(d32 ? "ral_day32(" : "ral_day64(") + to_i(l, lk) + ")", Kind::I64, ok); break;
                case BLZ_HOUR: e = d32 ? conv("((ral_i64)0)", Kind::I64, ok) : conv("ral_hour64(" + to_i(l, lk) + ")", Kind::I64, ok); break;
                case BLZ_MINUTE: e = d32 ? conv("((ral_i64)0)", Kind::I64, ok) : conv("ral_minute64(" + to_i(l, lk) + ")", Kind::I64, ok); break;
                case BLZ_SECOND: e = d32 ? conv("((ral_i64)0)", Kind::I64, ok) : conv("ral_second64(" + to_i(l, lk) + ")", Kind::I64, ok); break;
                case BLZ_IS_NULL: e = conv_bool("rb" + std::to_string(op.left) + " == 0u", ok); break;
                case BLZ_IS_NOT_NULL: e = conv_bool("rb" + std::to_string(op.left) + " != 0u", ok); break;
                default: e = conv(l, lk, ok); break;  // copy with conversion
                }
            }
            const std::string t = "t" + std::to_string(k);
            os << indent << "const " << kind_ctype(ok) << " " << t << " = " << e << ";\n";
            name[op.out] = t;
            kind[op.out] = ok;
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
    return dtype_is_float(t) ? "((double)(" + x + "))" : "((ral_i64)(" + x + "))";
}

// Register value -> column element, as write_data does it (interpreter_ops.cuh:317-381):
// integer columns take the slot's int64 bits, float columns its double bits.
std::string narrow(const std::string& v, Kind k, gdf_dtype t) {
    const std::string et = element_ctype(t);
    if (dtype_is_float(t)) {
        std::string d = k == Kind::F64 ? v : "ral_bits_d(" + v + ")";
        if (t == GDF_FLOAT32) return "__double2float_rn(" + d + ")";
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
    L.lscalar_slot.assign(p.ops.size(), -1);
    L.rscalar_slot.assign(p.ops.size(), -1);
    for (size_t k = 0; k < p.ops.size(); k++) {
        if (p.ops[k].left == SCALAR_INDEX) L.lscalar_slot[k] = s++;
        if (!p.ops[k].unary && p.ops[k].right == SCALAR_INDEX) L.rscalar_slot[k] = s++;
    }
    L.total = s;
    return L;
}

// The row function: one row through the program, typed registers in, final
// register values out.
void emit_row_function(std::ostream& os, const Program& p, const ParamLayout& L, const char* fname) {
    auto ref = p.inputs_referenced();
    auto raw = p.inputs_raw_valid();
    os << "RAL_FI void " << fname << "(const RalParams& P";
    for (int c = 0; c < p.n_in; c++)
        if (ref[c]) os << ", const " << kind_ctype(dtype_kind(p.inputs[c].dtype)) << " x" << c;
    for (int c = 0; c < p.n_in; c++)
        if (raw[c]) os << ", const ral_u32 rb" << c;
    OpEmitter em(p, L);
    std::ostringstream body;
    em.emit(body, "    ");
    for (int o = 0; o < p.n_out; o++) os << ", " << kind_ctype(em.kind[p.final_pos[o]]) << "& y" << o;
    os << ") {\n" << body.str();
    for (int o = 0; o < p.n_out; o++) os << "    y" << o << " = " << em.name[p.final_pos[o]] << ";\n";
    os << "}\n";
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

GeneratedKernel generate_eval_kernel(const Program& p, const Shape& s) {
    GeneratedKernel gk;
    gk.shape = s;
    gk.layout = make_layout(p, 0);
    const ParamLayout& L = gk.layout;
    const auto ref = p.inputs_referenced();
    const auto raw = p.inputs_raw_valid();
    const auto fk = final_kinds(p, L);
    std::vector<int> vouts;  // outputs that carry a valid mask
    for (int o = 0; o < p.n_out; o++)
        if (p.out_has_valid[o]) vouts.push_back(o);
    const int NOV = (int)vouts.size();

    std::ostringstream key;
    key << "eval|" << p.structure_key() << "|G" << s.G << "J" << s.J << "T" << s.threads << "B" << s.min_blocks;
    char hex[32];
    snprintf(hex, sizeof hex, "%016llx", (unsigned long long)fnv1a(key.str()));
    gk.name = std::string("ral_eval_") + hex;

    std::ostringstream os;
    os << "// generated: " << key.str() << "\n";
    os << "#define RAL_G " << s.G << "\n#define RAL_J " << s.J << "\n#define RAL_THREADS " << s.threads << "\n";
    os << "struct RalParams { ral_u64 s[" << L.total << "]; };\n\n";
    emit_row_function(os, p, L, "ral_row");

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
        os << "        if (lane < RAL_G * RAL_J) {\n";
        os << "            const ral_i64 w = (base >> 5) + lane;\n";
        os << "            ral_u32 vo[" << NOV << "]; ral_vword(P, w, vo);\n";
        for (int i = 0; i < NOV; i++) os << "            pvo" << i << "[w] = vo[" << i << "]; vcnt[" << i << "] += __popc(vo[" << i << "]);\n";
        os << "        }\n";
    }
    os << "    }\n";

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
    return gk;
}

GeneratedKernel generate_filter_kernel(const FilterSpec& f, const Shape& s) {
    (void)f; (void)s;
    throw std::runtime_error("filter kernel generation not built yet");
}

}  // namespace ral
