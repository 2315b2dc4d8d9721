// Generated right-hand side: the GPU counterpart of the straight-line f! that
// ModelingToolkit compiles for a discretised system (src/MOL_discretization.jl:171-201).
//
// From a validated descriptor the library writes CUDA C++ for one problem
// *structure*: the pointwise program becomes SSA statements, every derivative
// term becomes a function with an interior fast path (compile-time tap offsets,
// direct strided loads, structural zero weights dropped) and the generic
// boundary path (tap tables, wrap, observed boundary rows), and the reverse
// sweep of the same statements gives the vector-Jacobian product.  Grid sizes,
// weights, parameters and aux arrays stay runtime data, so one compiled module
// serves every grid size of a structure (and every member of an ensemble).
// The module is compiled with NVRTC for sm_103a and loaded through the CUDA
// runtime's library API; the hand-written kernel templates of mol_kernels.cuh
// are instantiated with the generated cell.
#include <cuda_runtime.h>
#include <dlfcn.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
#include <set>
#include <sstream>
#include <string>
#include <vector>

#include "mol_codegen.h"

#include "mol_embedded.inc"  // kEmbedNames / kEmbedTexts: the device headers, embedded at build time

namespace mol {

bool nonlinlap_fold(const mol_problem_desc* d, int k) {
    if (k < 0 || k >= d->nterms) return false;
    const mol_term& tm = d->terms[k];
    if (tm.kind != MOL_TERM_NONLINLAP) return false;
    const char* env = getenv("MOL_JIT_FOLD");
    if (env && env[0] == '0') return false;
    const mol_op1d& oo = d->ops[tm.op];
    const mol_op1d& oi = d->ops[tm.op2];
    const mol_op1d& op = d->ops[tm.op3];
    if (oo.nrows || oi.nrows || op.nrows || oo.L != 2 || oi.L != 2) return false;
    const double* w = d->weights;
    auto anti = [&](const mol_op1d& o) { return w[o.w_int] != 0.0 && w[o.w_int] == -w[o.w_int + 1]; };
    return anti(oo) && anti(oi);
}

namespace {

std::string lit(double v) {
    if (!std::isfinite(v)) return "";
    char buf[64];
    std::snprintf(buf, sizeof buf, "T(%a)", v);
    return buf;
}

struct Emitter {
    std::ostringstream o;
    template <class X>
    Emitter& operator<<(const X& x) {
        o << x;
        return *this;
    }
};

std::string v(int pc) { return "v" + std::to_string(pc); }
std::string a(int pc) { return "a" + std::to_string(pc); }

// Register program -> SSA: for each instruction the SSA ids of its register operands.
struct SSA {
    std::vector<mol_instr> ins;
    std::vector<int> ia, ib, ic;
    bool ok = true;
};

SSA to_ssa(const mol_problem_desc* d, int prog) {
    SSA s;
    const int start = d->prog_ranges[2 * prog], len = d->prog_ranges[2 * prog + 1];
    std::vector<int> last(MOL_MAX_REGS, -1);
    for (int pc = 0; pc < len; ++pc) {
        const mol_instr in = d->code[start + pc];
        s.ins.push_back(in);
        auto rd = [&](int r) { return (r >= 0 && r < MOL_MAX_REGS) ? last[r] : -1; };
        int A = -1, B = -1, C = -1;
        switch (in.op) {
            case MOL_OP_NEG: case MOL_OP_POWI: case MOL_OP_FN: case MOL_OP_OUT: case MOL_OP_UPWIND:
                A = rd(in.a);
                break;
            case MOL_OP_ADD: case MOL_OP_SUB: case MOL_OP_MUL: case MOL_OP_DIV: case MOL_OP_POW: case MOL_OP_CMP:
                A = rd(in.a);
                B = rd(in.b);
                break;
            case MOL_OP_IFELSE:
                A = rd(in.a);
                B = rd(in.b);
                C = rd(in.c);
                break;
            default:
                break;
        }
        if ((A == -2) || (B == -2) || (C == -2)) s.ok = false;
        s.ia.push_back(A);
        s.ib.push_back(B);
        s.ic.push_back(C);
        if (in.op != MOL_OP_OUT) last[in.dst] = pc;
    }
    return s;
}

// Value of a node built from constants only (CONST, NEG, ADD, SUB, MUL, DIV), or false.
bool const_value(const mol_problem_desc* d, const SSA& s, int pc, double* out) {
    if (pc < 0) return false;
    const mol_instr& in = s.ins[pc];
    double a = 0, b = 0;
    switch (in.op) {
        case MOL_OP_CONST: *out = d->consts[in.imm]; return std::isfinite(*out);
        case MOL_OP_NEG:
            if (!const_value(d, s, s.ia[pc], &a)) return false;
            *out = -a;
            return true;
        case MOL_OP_ADD: case MOL_OP_SUB: case MOL_OP_MUL: case MOL_OP_DIV:
            if (!const_value(d, s, s.ia[pc], &a) || !const_value(d, s, s.ib[pc], &b)) return false;
            *out = in.op == MOL_OP_ADD ? a + b : in.op == MOL_OP_SUB ? a - b : in.op == MOL_OP_MUL ? a * b : a / b;
            return std::isfinite(*out);
        default: return false;
    }
}

}  // namespace

std::vector<FoldGroup> const_linear_groups(const mol_problem_desc* d) {
    std::vector<FoldGroup> groups;
    const char* env = getenv("MOL_JIT_CFOLD");
    if ((env && env[0] == '0') || d->cell_prog < 0) return groups;
    const SSA s = to_ssa(d, d->cell_prog);
    if (!s.ok) return groups;
    const int n = (int)s.ins.size();
    std::vector<int> uses(n, 0);
    for (int pc = 0; pc < n; ++pc)
        for (int x : {s.ia[pc], s.ib[pc], s.ic[pc]})
            if (x >= 0) uses[x]++;
    auto nz = [&](long long off) { return d->weights[off] != 0.0; };
    // a first-derivative stencil term of compile-time weights
    auto first_deriv = [&](int k) {
        if (k < 0 || k >= d->nterms) return false;
        const mol_term& tm = d->terms[k];
        if (tm.kind == MOL_TERM_MIXED) return d->ops[tm.op].nrows == 0 && d->ops[tm.op2].nrows == 0;
        if (tm.kind != MOL_TERM_LINEAR) return false;
        const mol_op1d& o = d->ops[tm.op];
        if (o.nrows) return false;
        for (int m = 0; m < o.L; ++m)
            if (d->weights[o.w_int + m] != -d->weights[o.w_int + o.L - 1 - m]) return false;
        return true;
    };
    // a nonlinear Laplacian in its folded form whose face coefficient depends on the
    // coordinates only: the face program reads aux arrays and constants (no field, parameter,
    // time or term), so its per-cell stencil weights are fixed for the plan's life
    auto var_deriv = [&](int k) {
        if (!nonlinlap_fold(d, k)) return false;
        const mol_term& tm = d->terms[k];
        if (tm.prog < 0) return true;
        if (tm.prog >= d->nprogs) return false;
        const int start = d->prog_ranges[2 * tm.prog], len = d->prog_ranges[2 * tm.prog + 1];
        for (int pc = start; pc < start + len; ++pc) {
            switch (d->code[pc].op) {
                case MOL_OP_CONST: case MOL_OP_AUX: case MOL_OP_ADD: case MOL_OP_SUB: case MOL_OP_MUL:
                case MOL_OP_DIV: case MOL_OP_NEG: case MOL_OP_POWI: case MOL_OP_POW: case MOL_OP_FN:
                case MOL_OP_CMP: case MOL_OP_IFELSE: case MOL_OP_OUT:
                    break;
                default:
                    return false;
            }
        }
        return true;
    };
    auto is_uniform_const = [&](int pc, double* c) { return const_value(d, s, pc, c); };
    // a foldable leaf: (term, coefficient, subtree pcs)
    struct Leaf {
        int term;
        double coef;
        std::vector<int> nodes;
    };
    std::function<bool(int, Leaf*)> leaf = [&](int pc, Leaf* L) -> bool {
        const mol_instr& in = s.ins[pc];
        if (uses[pc] != 1) return false;
        if (in.op == MOL_OP_TERM && (first_deriv(in.imm) || var_deriv(in.imm))) {
            *L = Leaf{in.imm, 1.0, {pc}};
            return true;
        }
        if (in.op == MOL_OP_UPWIND) {
            double c;
            if (!is_uniform_const(s.ia[pc], &c)) return false;
            const int k = c < 0 ? in.b : in.c;
            if (k < 0 || k >= d->nterms || d->terms[k].kind != MOL_TERM_LINEAR || d->ops[d->terms[k].op].nrows)
                return false;
            *L = Leaf{k, c, {pc}};
            return true;
        }
        if (in.op == MOL_OP_MUL) {
            double c;
            for (int side = 0; side < 2; ++side) {
                const int cp = side ? s.ib[pc] : s.ia[pc], xp = side ? s.ia[pc] : s.ib[pc];
                if (!is_uniform_const(cp, &c)) continue;
                Leaf inner;
                if (xp >= 0 && leaf(xp, &inner)) {
                    inner.coef *= c;
                    inner.nodes.push_back(pc);
                    *L = inner;
                    return true;
                }
            }
        }
        return false;
    };
    for (int pc = 0; pc < n; ++pc) {
        if (s.ins[pc].op != MOL_OP_OUT || s.ia[pc] < 0) continue;
        FoldGroup g;
        g.out_pc = pc;
        // flatten the output's sum: ADD / SUB / NEG nodes used once (the root included)
        std::vector<std::pair<double, int>> adds;
        std::vector<int> chain;
        std::function<void(int, double, bool)> flat = [&](int q, double sg, bool root) {
            const mol_instr& in = s.ins[q];
            double cv;
            const bool varying = !is_uniform_const(q, &cv);
            if (varying && (root || uses[q] == 1) && (in.op == MOL_OP_ADD || in.op == MOL_OP_SUB)) {
                chain.push_back(q);
                flat(s.ia[q], sg, false);
                flat(s.ib[q], in.op == MOL_OP_SUB ? -sg : sg, false);
                return;
            }
            if (varying && (root || uses[q] == 1) && in.op == MOL_OP_NEG) {
                chain.push_back(q);
                flat(s.ia[q], -sg, false);
                return;
            }
            adds.push_back({sg, q});
        };
        flat(s.ia[pc], 1.0, true);
        std::vector<Leaf> leaves;
        for (auto& a : adds) {
            Leaf L;
            if (leaf(a.second, &L) && (g.field < 0 || d->terms[L.term].field == g.field)) {
                g.field = d->terms[L.term].field;
                L.coef *= a.first;
                g.folded.push_back(a);
                leaves.push_back(L);
            } else {
                g.rest.push_back(a);
            }
        }
        // worth it: two or more stencils, one with a coefficient to fold, or a variable member
        bool any_var = false;
        for (auto& L : leaves) any_var |= d->terms[L.term].kind == MOL_TERM_NONLINLAP;
        if (leaves.empty() ||
            (!any_var && leaves.size() == 1 && leaves[0].nodes.size() == 1 && std::fabs(leaves[0].coef) == 1.0))
            continue;
        g.absorbed = chain;
        for (auto& L : leaves)
            for (int q : L.nodes) {
                g.absorbed.push_back(q);
                g.leaf_nodes.push_back(q);
            }
        std::sort(g.leaf_nodes.begin(), g.leaf_nodes.end());
        // the term whose reserved2 holds the weights' offset: one not already keying a group
        g.key_term = -1;
        for (auto& L : leaves) {
            bool taken = false;
            for (auto& h : groups) taken |= h.key_term == L.term;
            if (!taken && (g.key_term < 0 || L.term < g.key_term)) g.key_term = L.term;
        }
        if (g.key_term < 0) continue;
        auto add_part = [&](int o0, int o1, int o2, const FoldPart& p) {
            for (auto& t : g.taps)
                if (t.o[0] == o0 && t.o[1] == o1 && t.o[2] == o2) {
                    t.parts.push_back(p);
                    return;
                }
            FoldTap t;
            t.o[0] = o0;
            t.o[1] = o1;
            t.o[2] = o2;
            t.parts.push_back(p);
            g.taps.push_back(t);
        };
        for (auto& L : leaves) {
            const mol_term& tm = d->terms[L.term];
            if (tm.kind == MOL_TERM_LINEAR) {
                const mol_op1d& o = d->ops[tm.op];
                for (int m = 0; m < o.L; ++m) {
                    if (!nz(o.w_int + m)) continue;
                    int off[3] = {0, 0, 0};
                    off[tm.dim] = o.omin + m;
                    add_part(off[0], off[1], off[2], FoldPart{L.term, m, L.coef});
                }
            } else if (tm.kind == MOL_TERM_NONLINLAP) {
                // folded form: W (F(face 1) - F(face 0)), F(face m) = a_m (u[r_m + oi.omin + 1] -
                // u[r_m + oi.omin]) at the outer stencil's half point r_m = oo.omin + m - 1
                const mol_op1d& oo = d->ops[tm.op];
                const mol_op1d& oi = d->ops[tm.op2];
                const double W = d->weights[oo.w_int + 1] * d->weights[oi.w_int + 1];
                for (int m = 0; m < 2; ++m) {
                    const int r = oo.omin + m - 1;
                    const double sg = m == 1 ? 1.0 : -1.0;
                    for (int side = 0; side < 2; ++side) {
                        int off[3] = {0, 0, 0};
                        off[tm.dim] = r + oi.omin + side;
                        add_part(off[0], off[1], off[2],
                                 FoldPart{L.term, m, L.coef * W * sg * (side ? 1.0 : -1.0), m});
                    }
                }
                g.variable = true;
            } else {
                const mol_op1d& o1 = d->ops[tm.op];
                const mol_op1d& o2 = d->ops[tm.op2];
                for (int x = 0; x < o1.L; ++x)
                    for (int y = 0; y < o2.L; ++y) {
                        if (!nz(o1.w_int + x) || !nz(o2.w_int + y)) continue;
                        int off[3] = {0, 0, 0};
                        off[tm.dim] += o1.omin + x;
                        off[tm.dim2] += o2.omin + y;
                        add_part(off[0], off[1], off[2], FoldPart{L.term, x * o2.L + y, L.coef});
                    }
            }
        }
        if (g.variable) {
            // tap modes: in the difference form every off-centre tap with a variable part is
            // applied to (u[tap] - u[centre]) and reads a coefficient array; the centre keeps a
            // uniform weight.  Expanded: every tap with a variable part reads an array.
            const bool expanded = (d->flags & MOL_FLAG_EXPAND_STENCILS) != 0;
            bool has_centre = false;
            for (auto& t : g.taps) has_centre |= t.o[0] == 0 && t.o[1] == 0 && t.o[2] == 0;
            if (!has_centre) {
                FoldTap t;
                t.o[0] = t.o[1] = t.o[2] = 0;
                g.taps.push_back(t);
            }
            for (auto& t : g.taps) {
                bool var = false;
                for (auto& p : t.parts) var |= p.face >= 0;
                const bool centre = t.o[0] == 0 && t.o[1] == 0 && t.o[2] == 0;
                if (!var || (centre && !expanded)) continue;
                t.diff = !centre && !expanded;
                t.arr = g.narr++;
            }
            int base = 0;
            for (auto& h : groups) base += h.narr;
            g.arr0 = base;
            // a reaction k u^2 in the cell's own unknown joins the expanded centre tap:
            // (c_0 + k u) u is one FMA fewer than c_0 u + k (u u)
            bool centre_arr = false;
            for (auto& t : g.taps) centre_arr |= t.arr >= 0 && !t.o[0] && !t.o[1] && !t.o[2];
            std::function<bool(int)> uniform = [&](int q) -> bool {
                if (q < 0) return false;
                const mol_instr& in = s.ins[q];
                switch (in.op) {
                    case MOL_OP_CONST: case MOL_OP_PARAM: case MOL_OP_TIME: return true;
                    case MOL_OP_ADD: case MOL_OP_SUB: case MOL_OP_MUL: case MOL_OP_DIV: case MOL_OP_POW:
                    case MOL_OP_CMP:
                        return uniform(s.ia[q]) && uniform(s.ib[q]);
                    case MOL_OP_NEG: case MOL_OP_POWI: case MOL_OP_FN: return uniform(s.ia[q]);
                    case MOL_OP_IFELSE: return uniform(s.ia[q]) && uniform(s.ib[q]) && uniform(s.ic[q]);
                    default: return false;
                }
            };
            // the square of the group's field at the cell: POWI(F, 2) or MUL(F, F) of one FIELD
            // node used by nothing else
            auto square = [&](int q, std::vector<int>* nodes) -> bool {
                if (q < 0 || uses[q] != 1) return false;
                const mol_instr& in = s.ins[q];
                int f = -1;
                if (in.op == MOL_OP_POWI && in.imm == 2) f = s.ia[q];
                else if (in.op == MOL_OP_MUL && s.ia[q] == s.ib[q]) f = s.ia[q];
                if (f < 0 || s.ins[f].op != MOL_OP_FIELD || s.ins[f].imm != g.field) return false;
                if (uses[f] != (in.op == MOL_OP_MUL ? 2 : 1)) return false;
                *nodes = {f, q};
                return true;
            };
            for (size_t i = 0; expanded && centre_arr && i < g.rest.size(); ++i) {
                const int q = g.rest[i].second;
                if (s.ins[q].op != MOL_OP_MUL || uses[q] != 1) continue;
                std::vector<int> nodes;
                int k = -1;
                if (uniform(s.ia[q]) && square(s.ib[q], &nodes)) k = s.ia[q];
                else if (uniform(s.ib[q]) && square(s.ia[q], &nodes)) k = s.ib[q];
                if (k < 0) continue;
                g.quad_coef = k;
                g.quad_sign = g.rest[i].first;
                nodes.push_back(q);
                for (int x : nodes) {
                    g.absorbed.push_back(x);
                    g.leaf_nodes.push_back(x);
                }
                std::sort(g.leaf_nodes.begin(), g.leaf_nodes.end());
                g.folded.push_back(g.rest[i]);
                g.rest.erase(g.rest.begin() + i);
                break;
            }
        }
        groups.push_back(g);
    }
    return groups;
}

int fold_coef_arrays(const std::vector<FoldGroup>& groups) {
    int n = 0;
    for (auto& g : groups) n += g.narr;
    return n;
}

bool nonlinlap_all_in_groups(const mol_problem_desc* d, const std::vector<FoldGroup>& groups) {
    for (int k = 0; k < d->nterms; ++k) {
        if (d->terms[k].kind != MOL_TERM_NONLINLAP) continue;
        bool found = false;
        for (auto& g : groups)
            for (auto& t : g.taps)
                for (auto& p : t.parts) found |= p.term == k && p.face >= 0;
        if (!found) return false;
    }
    return true;
}

// The fused weights of `g`: per tap the sum over its constant parts of coefficient * weight
// (MIXED: the product of the two interior weights), in part order; the difference form's
// centre then gains the differenced taps' constant parts.
std::vector<double> fold_weights(const mol_problem_desc* d, const FoldGroup& g) {
    std::vector<double> w;
    for (const FoldTap& t : g.taps) {
        double acc = 0.0;
        bool first = true;
        for (const FoldPart& p : t.parts) {
            if (p.face >= 0) continue;   // coordinate-dependent part: added per cell by k_coef_t
            const mol_term& tm = d->terms[p.term];
            double wk;
            if (tm.kind == MOL_TERM_LINEAR) {
                wk = d->weights[d->ops[tm.op].w_int + p.m];
            } else {
                const mol_op1d& o2 = d->ops[tm.op2];
                wk = d->weights[d->ops[tm.op].w_int + p.m / o2.L] * d->weights[o2.w_int + p.m % o2.L];
            }
            acc = first ? p.coef * wk : acc + p.coef * wk;
            first = false;
        }
        w.push_back(acc);
    }
    // difference form: c_k (u_k - u_0) for the differenced taps moves c_k's constant part off
    // the centre (the variable parts of the centre cancel identically and are not formed)
    for (size_t i = 0; i < g.taps.size(); ++i) {
        const FoldTap& t = g.taps[i];
        if (t.o[0] || t.o[1] || t.o[2]) continue;
        for (size_t j = 0; j < g.taps.size(); ++j)
            if (g.taps[j].diff) w[i] += w[j];
    }
    return w;
}

namespace {

// How leaves of a program are read and how their adjoints are written.
struct Leaves {
    // forward expressions
    virtual std::string field(int f) const = 0;
    virtual std::string aux(int k) const = 0;
    virtual std::string coord(int d) const = 0;
    virtual std::string term(int k) const = 0;
    // reverse statements (adjoint value given as expression `g`)
    virtual std::string field_adj(int f, const std::string& g) const = 0;
    virtual std::string aux_adj(int k, const std::string& g) const = 0;
    virtual std::string term_adj(int k, const std::string& g) const = 0;
    virtual ~Leaves() {}
};

std::string fn_expr(int fn, const std::string& x) {
    static const char* names[] = {"sin", "cos", "tan", "exp", "log", "sqrt", "fabs", "tanh", "sinh", "cosh", "atan"};
    return std::string(names[fn]) + "(" + x + ")";
}

// d fn(x)/dx given x and r = fn(x)
std::string fn_deriv(int fn, const std::string& x, const std::string& r) {
    switch (fn) {
        case MOL_FN_SIN: return "cos(" + x + ")";
        case MOL_FN_COS: return "(-sin(" + x + "))";
        case MOL_FN_TAN: return "(T(1) + " + r + " * " + r + ")";
        case MOL_FN_EXP: return r;
        case MOL_FN_LOG: return "(T(1) / " + x + ")";
        case MOL_FN_SQRT: return "(T(0.5) / " + r + ")";
        case MOL_FN_ABS: return "((" + x + ") < T(0) ? T(-1) : T(1))";
        case MOL_FN_TANH: return "(T(1) - " + r + " * " + r + ")";
        case MOL_FN_SINH: return "cosh(" + x + ")";
        case MOL_FN_COSH: return "sinh(" + x + ")";
        case MOL_FN_ATAN: return "(T(1) / (T(1) + " + x + " * " + x + "))";
    }
    return "T(0)";
}

// Forward statements of an SSA program; `outs` receives the OUT assignments.
void emit_forward(Emitter& e, const mol_problem_desc* d, const SSA& s, const Leaves& L, const std::string& pre,
                  std::vector<std::pair<int, int>>* outs, bool keep_terms) {
    for (size_t pc = 0; pc < s.ins.size(); ++pc) {
        const mol_instr& in = s.ins[pc];
        const std::string V = pre + v((int)pc);
        const std::string A = s.ia[pc] >= 0 ? pre + v(s.ia[pc]) : "";
        const std::string B = s.ib[pc] >= 0 ? pre + v(s.ib[pc]) : "";
        const std::string C = s.ic[pc] >= 0 ? pre + v(s.ic[pc]) : "";
        switch (in.op) {
            case MOL_OP_CONST: {
                std::string l = lit(d->consts[in.imm]);
                if (l.empty()) l = "P.consts[" + std::to_string(in.imm) + "]";
                e << "    const T " << V << " = " << l << ";\n";
                break;
            }
            case MOL_OP_PARAM: e << "    const T " << V << " = p[" << in.imm << "];\n"; break;
            case MOL_OP_FIELD: e << "    const T " << V << " = " << L.field(in.imm) << ";\n"; break;
            case MOL_OP_AUX: e << "    const T " << V << " = " << L.aux(in.imm) << ";\n"; break;
            case MOL_OP_COORD: e << "    const T " << V << " = " << L.coord(in.imm) << ";\n"; break;
            case MOL_OP_TIME: e << "    const T " << V << " = t;\n"; break;
            case MOL_OP_TERM: e << "    const T " << V << " = " << L.term(in.imm) << ";\n"; break;
            case MOL_OP_UPWIND:
                e << "    const T " << pre << "tv" << pc << " = (" << A << " < T(0)) ? " << L.term(in.b) << " : "
                  << L.term(in.c) << ";\n";
                e << "    const T " << V << " = " << A << " * " << pre << "tv" << pc << ";\n";
                break;
            case MOL_OP_ADD: e << "    const T " << V << " = " << A << " + " << B << ";\n"; break;
            case MOL_OP_SUB: e << "    const T " << V << " = " << A << " - " << B << ";\n"; break;
            case MOL_OP_MUL: e << "    const T " << V << " = " << A << " * " << B << ";\n"; break;
            case MOL_OP_DIV: e << "    const T " << V << " = " << A << " / " << B << ";\n"; break;
            case MOL_OP_NEG: e << "    const T " << V << " = -" << A << ";\n"; break;
            case MOL_OP_POWI:
                if (in.imm == 2) e << "    const T " << V << " = " << A << " * " << A << ";\n";
                else if (in.imm == 3) e << "    const T " << V << " = " << A << " * " << A << " * " << A << ";\n";
                else if (in.imm == 1) e << "    const T " << V << " = " << A << ";\n";
                else if (in.imm == 0) e << "    const T " << V << " = T(1);\n";
                else e << "    const T " << V << " = powi(" << A << ", " << in.imm << ");\n";
                break;
            case MOL_OP_POW: e << "    const T " << V << " = pow(" << A << ", " << B << ");\n"; break;
            case MOL_OP_FN: e << "    const T " << V << " = " << fn_expr(in.imm, A) << ";\n"; break;
            case MOL_OP_CMP: {
                static const char* ops[] = {"<=", "<", ">=", ">", "=="};
                e << "    const T " << V << " = (" << A << " " << ops[in.imm] << " " << B << ") ? T(1) : T(0);\n";
                break;
            }
            case MOL_OP_IFELSE:
                e << "    const T " << V << " = (" << A << " != T(0)) ? " << B << " : " << C << ";\n";
                break;
            case MOL_OP_OUT:
                if (outs) outs->push_back({in.imm, s.ia[pc]});
                break;
            default: break;
        }
        (void)keep_terms;
    }
}

// Reverse sweep.  `seed(k)` is the adjoint expression of output k.
template <class SeedFn>
void emit_reverse(Emitter& e, const SSA& s, const Leaves& L, const std::string& pre, SeedFn seed) {
    const int n = (int)s.ins.size();
    for (int pc = 0; pc < n; ++pc)
        if (s.ins[pc].op != MOL_OP_OUT) e << "    T " << pre << a(pc) << " = T(0);\n";
    for (int pc = n - 1; pc >= 0; --pc) {
        const mol_instr& in = s.ins[pc];
        const std::string G = pre + a(pc);
        const std::string V = pre + v(pc);
        const std::string A = s.ia[pc] >= 0 ? pre + v(s.ia[pc]) : "";
        const std::string B = s.ib[pc] >= 0 ? pre + v(s.ib[pc]) : "";
        const std::string GA = s.ia[pc] >= 0 ? pre + a(s.ia[pc]) : "";
        const std::string GB = s.ib[pc] >= 0 ? pre + a(s.ib[pc]) : "";
        const std::string GC = s.ic[pc] >= 0 ? pre + a(s.ic[pc]) : "";
        switch (in.op) {
            case MOL_OP_OUT: e << "    " << GA << " += " << seed(in.imm) << ";\n"; break;
            case MOL_OP_PARAM: e << "    lp[" << in.imm << "] += " << G << ";\n"; break;
            case MOL_OP_FIELD: e << L.field_adj(in.imm, G); break;
            case MOL_OP_AUX: e << L.aux_adj(in.imm, G); break;
            case MOL_OP_TERM: e << L.term_adj(in.imm, G); break;
            case MOL_OP_UPWIND:
                e << "    " << GA << " += " << G << " * " << pre << "tv" << pc << ";\n";
                e << "    if (" << A << " < T(0)) {\n" << L.term_adj(in.b, G + " * " + A) << "    } else {\n"
                  << L.term_adj(in.c, G + " * " + A) << "    }\n";
                break;
            case MOL_OP_ADD: e << "    " << GA << " += " << G << "; " << GB << " += " << G << ";\n"; break;
            case MOL_OP_SUB: e << "    " << GA << " += " << G << "; " << GB << " -= " << G << ";\n"; break;
            case MOL_OP_MUL:
                e << "    " << GA << " += " << G << " * " << B << "; " << GB << " += " << G << " * " << A << ";\n";
                break;
            case MOL_OP_DIV:
                e << "    " << GA << " += " << G << " / " << B << "; " << GB << " -= " << G << " * " << V << " / " << B
                  << ";\n";
                break;
            case MOL_OP_NEG: e << "    " << GA << " -= " << G << ";\n"; break;
            case MOL_OP_POWI:
                if (in.imm == 0) break;
                e << "    " << GA << " += " << G << " * T(" << in.imm << ") * powi(" << A << ", " << (in.imm - 1)
                  << ");\n";
                break;
            case MOL_OP_POW:
                e << "    " << GA << " += " << G << " * " << B << " * pow(" << A << ", " << B << " - T(1));\n";
                e << "    " << GB << " += " << G << " * " << V << " * log(" << A << ");\n";
                break;
            case MOL_OP_FN: e << "    " << GA << " += " << G << " * " << fn_deriv(in.imm, A, V) << ";\n"; break;
            case MOL_OP_IFELSE:
                e << "    if (" << A << " != T(0)) " << GB << " += " << G << "; else " << GC << " += " << G << ";\n";
                break;
            default: break;
        }
    }
}

bool zero_w(const mol_problem_desc* d, long long off) { return d->weights[off] == 0.0; }

// Largest tap count of an operator over its interior and boundary tables.
int max_taps(const mol_op1d& o) { return std::max(1, std::max(o.L, std::max(o.bLlo, o.bLhi))); }

// "true" when a boundary row of field f along dimension dim has program coefficients.
const char* dyn_bc(const mol_problem_desc* d, int f, int dim) {
    if (f < 0 || f >= d->nfields || dim < 0 || dim >= d->ndim) return "true";
    for (int side = 0; side < 2; ++side) {
        const mol_bc& b = d->bc[f][dim][side];
        if (b.kind == MOL_BC_ROBIN && b.prog >= 0) return "true";
    }
    return "false";
}

// Warp-shuffle aggregation of contiguous-axis VJP scatters (MOL_JIT_WARP_SCATTER=0 turns it off).
bool warp_scatter() {
    const char* w = getenv("MOL_JIT_WARP_SCATTER");
    return !(w && w[0] == '0');
}

// Leaves of the cell program.
struct CellLeaves : Leaves {
    std::string field(int f) const override { return "u[(long long)" + std::to_string(f) + " * P.ncell + c]"; }
    std::string aux(int k) const override { return "P.aux[P.aux_off[" + std::to_string(k) + "] + c]"; }
    std::string coord(int dd) const override {
        return "P.coords[" + std::to_string(dd) + "][I[" + std::to_string(dd) + "] - 1]";
    }
    std::string term(int k) const override { return "gt" + std::to_string(k) + "<T>(P, u, c, I, t, p)"; }
    // inside the cell VJP the own-cell share of field f collects in own<f>
    const mol_problem_desc* d = nullptr;
    std::string field_adj(int f, const std::string& g) const override {
        return "    own" + std::to_string(f) + " += " + g + ";\n";
    }
    std::string aux_adj(int k, const std::string& g) const override {
        return "    if (lam_aux) atomicAdd(lam_aux + P.aux_off[" + std::to_string(k) + "] + c, " + g + ");\n";
    }
    std::string term_adj(int k, const std::string& g) const override {
        return "    gt" + std::to_string(k) + "_vjp<T>(P, u, c, I, t, p, " + g + ", lam_u, lp, lam_aux, own" +
               std::to_string(d->terms[k].field) + ");\n";
    }
};

// Leaves of the cell program inside the cell VJP: WENO terms named in `split` use
// their split forward/backward pair, which share the partials in fwK/gwK.
struct VjpCellLeaves : CellLeaves {
    std::vector<int> split;
    // members of coefficient-stencil groups (term -> group): on the group path their adjoints
    // are scattered by the group (emit_group_vjp), so their own statements are left out
    std::map<int, int> var_member;
    bool omit_members = false;
    bool is_split(int k) const { return std::find(split.begin(), split.end(), k) != split.end(); }
    std::string term(int k) const override {
        if (!is_split(k)) return CellLeaves::term(k);
        const std::string K = std::to_string(k);
        return "gt" + K + "_fg<T>(P, u, c, I, t, p, fw" + K + ", gw" + K + ")";
    }
    std::string term_adj(int k, const std::string& g) const override {
        if (omit_members && var_member.count(k)) return "";
        if (!is_split(k)) return CellLeaves::term_adj(k, g);
        const std::string K = std::to_string(k);
        return "    gt" + K + "_bg<T>(P, u, c, I, t, p, " + g + ", fw" + K + ", gw" + K + ", lam_u, lp, lam_aux, own" +
               std::to_string(d->terms[k].field) + ");\n";
    }
};

// Leaves of a nonlinear-Laplacian face program: fields are the interpolated
// values uf<f>, aux arrays the face values fa<k>.
struct FaceLeaves : Leaves {
    std::string tag;
    explicit FaceLeaves(std::string t) : tag(std::move(t)) {}
    std::string field(int f) const override { return tag + "uf" + std::to_string(f); }
    std::string aux(int k) const override { return tag + "fa" + std::to_string(k); }
    std::string coord(int) const override { return "T(0)"; }
    std::string term(int) const override { return "T(0)"; }
    std::string field_adj(int f, const std::string& g) const override {
        return "    " + tag + "guf" + std::to_string(f) + " += " + g + ";\n";
    }
    std::string aux_adj(int k, const std::string& g) const override {
        return "    " + tag + "gfa" + std::to_string(k) + " += " + g + ";\n";
    }
    std::string term_adj(int, const std::string&) const override { return ""; }
};

// True when field f is periodic along dimension dim (interior weights everywhere).
bool periodic_dim(const mol_problem_desc* d, int f, int dim) {
    return f >= 0 && f < d->nfields && dim >= 0 && dim < d->ndim && d->bc[f][dim][0].kind == MOL_BC_PERIODIC;
}

// Largest |offset| of an operator's interior taps.
int reach_of(const mol_op1d& o) { return std::max(std::abs(o.omin), std::abs(o.omin + o.L - 1)); }

// Linear stencil term.  Along a periodic dimension every cell uses the interior weights
// with wrapped offsets (one uniform branch, no edge path); otherwise interior cells use
// compile-time offsets and cells near an edge the line helpers.
void emit_linear(Emitter& e, const mol_problem_desc* d, int k) {
    const mol_term& tm = d->terms[k];
    const mol_op1d& o = d->ops[tm.op];
    const std::string K = std::to_string(k), F = std::to_string(tm.field), D = std::to_string(tm.dim);
    // taps whose weight is zero in every interior row are left out
    std::vector<int> nz;
    for (int m = 0; m < o.L; ++m) {
        bool z = true;
        for (int r = 0; r < std::max(1, o.nrows) && z; ++r) z = zero_w(d, o.w_int + (int64_t)r * o.L + m);
        if (!z) nz.push_back(m);
    }
    const bool per = periodic_dim(d, tm.field, tm.dim);
    // nonuniform grid: the interior row of the cell's own point (never periodic)
    const std::string wrow = o.nrows > 0 ? " + (long long)(I[" + D + "] - " + std::to_string(o.nlo + 1) + ") * " +
                                               std::to_string(o.L)
                                         : std::string();
    const std::string cond = per ? "wrap_line_ok(P, " + F + ", " + D + ", " + std::to_string(reach_of(o)) + ")"
                                 : "warp_all(fast_line(P, P.ops[" + std::to_string(tm.op) + "], " + F + ", " + D +
                                       ", I[" + D + "]))";
    auto off = [&](int m) {
        const int of = o.omin + m;
        return per ? "(long long)wrap_off(I[" + D + "], " + std::to_string(of) + ", P.n[" + D + "]) * s"
                   : "(long long)(" + std::to_string(of) + ") * s";
    };
    e << "template <class T>\n__device__ __forceinline__ T gt" << K
      << "(const DevProb<T>& P, const T* __restrict__ u, long long c, const int* I, T t, const T* __restrict__ p) {\n"
      << "    if (" << cond << ") {\n"
      << "        const T* __restrict__ w = P.w + P.ops[" << tm.op << "].w_int" << wrow << ";\n"
      << "        const T* __restrict__ b = u + (long long)" << F << " * P.ncell + c;\n"
      << "        const long long s = gstride(P, " << D << ");\n";
    if (nz.empty()) {
        e << "        return T(0);\n";
    } else {
        for (size_t q = 0; q < nz.size(); ++q) {
            const int m = nz[q];
            const std::string tap = "b[" + off(m) + "]";
            if (q == 0) e << "        T acc = w[" << m << "] * " << tap << ";\n";
            else e << "        acc = fma(w[" << m << "], " << tap << ", acc);\n";
        }
        e << "        return acc;\n";
    }
    const std::string DY = dyn_bc(d, tm.field, tm.dim);
    e << "    }\n    return apply_op_line<T, " << D << ", " << max_taps(o) << ", " << DY << ">(P, P.ops[" << tm.op
      << "], u, " << F << ", I, c, I[" << D << "], P.n[" << D << "], t, p);\n}\n";
    // vjp
    e << "template <class T>\n__device__ __forceinline__ void gt" << K
      << "_vjp(const DevProb<T>& P, const T* __restrict__ u, long long c, const int* I, T t, const T* __restrict__ p, "
         "T g, T* lam_u, T* lp, T* lam_aux, T& own) {\n"
      << "    if (" << cond << ") {\n"
      << "        const T* __restrict__ w = P.w + P.ops[" << tm.op << "].w_int" << wrow << ";\n"
      << "        T* b = lam_u + (long long)" << F << " * P.ncell + c;\n"
      << "        const long long s = gstride(P, " << D << ");\n";
    if (!nz.empty()) {
        e << "        const T vv[" << o.L << "] = {";
        for (int m = 0; m < o.L; ++m) {
            const bool z = std::find(nz.begin(), nz.end(), m) == nz.end();
            e << (m ? ", " : "") << (z ? std::string("T(0)") : "g * w[" + std::to_string(m) + "]");
        }
        const char* W = warp_scatter() ? "true" : "false";
        if (per)
            e << "};\n        scatter_taps_wrap<T, " << o.L << ", " << o.omin << ", " << W << ">(b, c, I[" << D
              << "], P.n[" << D << "], s, vv, own);\n";
        else
            e << "};\n        scatter_taps<T, " << o.L << ", " << o.omin << ", " << W << ">(b, c, s, vv, own);\n";
    }
    e << "        return;\n    }\n    scatter_op_line<T, " << D << ", " << max_taps(o) << ", " << DY << ">(P, P.ops["
      << tm.op << "], lam_u, " << F << ", I, c, I[" << D << "], P.n[" << D << "], g, t, p);\n}\n";
}

void emit_mixed(Emitter& e, const mol_problem_desc* d, int k) {
    const mol_term& tm = d->terms[k];
    const mol_op1d& o1 = d->ops[tm.op];
    const mol_op1d& o2 = d->ops[tm.op2];
    const std::string K = std::to_string(k), F = std::to_string(tm.field);
    const std::string D1 = std::to_string(tm.dim), D2 = std::to_string(tm.dim2);
    std::vector<std::pair<int, int>> nz;
    for (int x = 0; x < o1.L; ++x)
        for (int y = 0; y < o2.L; ++y)
            if (!zero_w(d, o1.w_int + x) && !zero_w(d, o2.w_int + y)) nz.push_back({x, y});
    // both dimensions periodic: wrapped offsets everywhere (uniform branch)
    const bool per = periodic_dim(d, tm.field, tm.dim) && periodic_dim(d, tm.field, tm.dim2);
    // per-point rows (nonuniform grid): the precomputed product table is one row's, so every
    // cell takes apply_mixed, whose tap selection picks each position's row
    const bool rows = o1.nrows > 0 || o2.nrows > 0;
    const std::string cond =
        rows ? std::string("false")
        : per ? "wrap_line_ok(P, " + F + ", " + D1 + ", " + std::to_string(reach_of(o1)) + ") && wrap_line_ok(P, " + F +
                  ", " + D2 + ", " + std::to_string(reach_of(o2)) + ")"
            : "warp_all(fast_line(P, P.ops[" + std::to_string(tm.op) + "], " + F + ", " + D1 + ", I[" + D1 +
                  "]) && fast_line(P, P.ops[" + std::to_string(tm.op2) + "], " + F + ", " + D2 + ", I[" + D2 + "]))";
    // the product weights sit in the pool at term.reserved0 (filled by the library), row-major [L1][L2]
    auto body = [&](bool vjp) {
        e << "    if (" << cond << ") {\n"
          << "        const T* __restrict__ ww = P.w + P.terms[" << k << "].reserved0;\n"
          << "        const long long s1 = gstride(P, " << D1 << "), s2 = gstride(P, " << D2 << ");\n";
        if (!vjp) e << "        const T* __restrict__ b = u + (long long)" << F << " * P.ncell + c;\n";
        else e << "        T* b = lam_u + (long long)" << F << " * P.ncell + c;\n";
        for (size_t q = 0; q < nz.size(); ++q) {
            const int x = nz[q].first, y = nz[q].second;
            const std::string W = "ww[" + std::to_string(x * o2.L + y) + "]";
            const std::string a1 = std::to_string(o1.omin + x), a2 = std::to_string(o2.omin + y);
            const std::string off =
                per ? "(long long)wrap_off(I[" + D1 + "], " + a1 + ", P.n[" + D1 + "]) * s1 + (long long)wrap_off(I[" + D2 +
                          "], " + a2 + ", P.n[" + D2 + "]) * s2"
                    : "(long long)(" + a1 + ") * s1 + (long long)(" + a2 + ") * s2";
            if (vjp) e << "        atomicAdd(b + " << off << ", g * " << W << ");\n";
            else if (q == 0) e << "        T acc = " << W << " * b[" << off << "];\n";
            else e << "        acc = fma(" << W << ", b[" << off << "], acc);\n";
        }
        if (vjp) e << "        return;\n    }\n";
        else e << "        return " << (nz.empty() ? "T(0)" : "acc") << ";\n    }\n";
    };
    e << "template <class T>\n__device__ __forceinline__ T gt" << K
      << "(const DevProb<T>& P, const T* __restrict__ u, long long c, const int* I, T t, const T* __restrict__ p) {\n";
    body(false);
    e << "    return apply_mixed(P, P.terms[" << k << "], u, I, t, p);\n}\n";
    e << "template <class T>\n__device__ __forceinline__ void gt" << K
      << "_vjp(const DevProb<T>& P, const T* __restrict__ u, long long c, const int* I, T t, const T* __restrict__ p, "
         "T g, T* lam_u, T* lp, T* lam_aux, T& own) {\n";
    body(true);
    e << "    scatter_mixed(P, P.terms[" << k << "], lam_u, I, g, t, p);\n}\n";
}

// WENO5 term.  Only the tap loads (and, in the VJP, the scatters) differ between
// interior cells and cells near an edge; the FP64 arithmetic is emitted once after
// the branch so a warp that straddles the edge runs it converged.
void emit_weno(Emitter& e, const mol_problem_desc* d, int k) {
    const mol_term& tm = d->terms[k];
    const std::string K = std::to_string(k), F = std::to_string(tm.field), D = std::to_string(tm.dim);
    if (tm.variant == 1) {
        // nonuniform dimension: per-point geometry rows, taps through the line helpers
        const std::string DYN = dyn_bc(d, tm.field, tm.dim);
        e << "template <class T>\n__device__ __forceinline__ T gt" << K
          << "(const DevProb<T>& P, const T* __restrict__ u, long long c, const int* I, T t, const T* __restrict__ p) "
             "{\n    return weno_nu_line<T, "
          << D << ", " << DYN << ">(P, P.terms[" << K << "], u, " << F << ", I, c, t, p);\n}\n";
        e << "template <class T>\n__device__ __forceinline__ void gt" << K
          << "_vjp(const DevProb<T>& P, const T* __restrict__ u, long long c, const int* I, T t, "
             "const T* __restrict__ p, T g, T* lam_u, T* lp, T* lam_aux, T& own) {\n    weno_nu_line_vjp<T, "
          << D << ", " << DYN << ">(P, P.terms[" << K << "], u, " << F << ", I, c, t, p, g, lam_u);\n}\n";
        return;
    }
    const std::string cond = "warp_all(fast_weno(P, " + F + ", " + D + ", I[" + D + "]))";
    const char* W = warp_scatter() ? "true" : "false";
    const std::string DY = dyn_bc(d, tm.field, tm.dim);
    const std::string sig = "(const DevProb<T>& P, const T* __restrict__ u, long long c, const int* I, T t, "
                            "const T* __restrict__ p";
    const std::string load =
        "    T v[5];\n"
        "    if (" + cond + ") {\n"
        "        const T* __restrict__ b = u + (long long)" + F + " * P.ncell + c;\n"
        "        const long long s = gstride(P, " + D + ");\n"
        "        v[0] = b[-2 * s]; v[1] = b[-s]; v[2] = b[0]; v[3] = b[s]; v[4] = b[2 * s];\n"
        "    } else {\n"
        "        weno_taps_line<T, " + D + ", " + DY + ">(P, " + F + ", u, I, c, t, p, v);\n"
        "    }\n";
    const std::string args = "v[0], v[1], v[2], v[3], v[4], T(P.terms[" + K + "].eps), T(P.terms[" + K + "].dx)";
    // scatter of vv[5] (already multiplied by the adjoint seed) on the path `fastexpr` picks
    auto scatter = [&](const std::string& fastexpr) {
        return "    if (" + fastexpr + ") {\n"
               "        T* lb = lam_u + (long long)" + F + " * P.ncell + c;\n"
               "        scatter_taps<T, 5, -2, " + W + ">(lb, c, gstride(P, " + D + "), vv, own);\n"
               "    } else {\n"
               "        scatter_weno_taps_line<T, " + D + ", " + DY + ">(P, " + F + ", lam_u, I, c, vv, t, p);\n"
               "    }\n";
    };
    e << "template <class T>\n__device__ __forceinline__ T gt" << K << sig << ") {\n"
      << load << "    return weno5_point<T>(" << args << ");\n}\n";
    e << "template <class T>\n__device__ __forceinline__ void gt" << K << "_vjp" << sig
      << ", T g, T* lam_u, T* lp, T* lam_aux, T& own) {\n"
      << load << "    T gr[5];\n    weno5_grad<T>(" << args << ", gr);\n"
      << "    const T vv[5] = {g * gr[0], g * gr[1], g * gr[2], g * gr[3], g * gr[4]};\n"
      << scatter(cond) << "}\n";
    // split form for the cell VJP: the forward keeps the five partials in registers,
    // the backward only scatters them (one reciprocal per cell instead of two)
    e << "template <class T>\n__device__ __forceinline__ T gt" << K << "_fg" << sig << ", bool& fast, T* gr) {\n"
      << "    fast = " << cond << ";\n"
      << load << "    return weno5_valgrad<T>(" << args << ", gr);\n}\n";
    e << "template <class T>\n__device__ __forceinline__ void gt" << K << "_bg" << sig
      << ", T g, bool fast, const T* gr, T* lam_u, T* lp, T* lam_aux, T& own) {\n"
      << "    const T vv[5] = {g * gr[0], g * gr[1], g * gr[2], g * gr[3], g * gr[4]};\n"
      << scatter("fast") << "}\n";
}

// Nonlinear Laplacian.  The face value a(x~, u~) * (D_inner u) at half point Ih
// is emitted twice: with compile-time offsets for interior cells and with
// runtime tap tables for the rest.
void emit_nonlinlap(Emitter& e, const mol_problem_desc* d, int k, int face_slot) {
    const mol_term& tm = d->terms[k];
    const mol_op1d& oo = d->ops[tm.op];
    const mol_op1d& oi = d->ops[tm.op2];
    const mol_op1d& op = d->ops[tm.op3];
    const std::string K = std::to_string(k), F = std::to_string(tm.field), D = std::to_string(tm.dim);
    SSA fs;
    bool has_prog = tm.prog >= 0;
    std::vector<int> used_fields, used_aux;
    if (has_prog) {
        fs = to_ssa(d, tm.prog);
        for (auto& in : fs.ins) {
            if (in.op == MOL_OP_FIELD && std::find(used_fields.begin(), used_fields.end(), in.imm) == used_fields.end())
                used_fields.push_back(in.imm);
            if (in.op == MOL_OP_AUX && std::find(used_aux.begin(), used_aux.end(), in.imm) == used_aux.end())
                used_aux.push_back(in.imm);
        }
    }
    std::vector<int> nzo;
    for (int m = 0; m < oo.L; ++m)
        if (!zero_w(d, oo.w_int + m)) nzo.push_back(m);
    std::vector<int> nzi, nzp;
    for (int m = 0; m < oi.L; ++m)
        if (!zero_w(d, oi.w_int + m)) nzi.push_back(m);
    for (int m = 0; m < op.L; ++m)
        if (!zero_w(d, op.w_int + m)) nzp.push_back(m);
    const std::string opi = std::to_string(tm.op2), opp = std::to_string(tm.op3), opo = std::to_string(tm.op);
    // folded form (nonlinlap_fold): forward faces are a * (u[+] - u[-]), the cell scales the
    // difference of its two faces by wo[1] wi[1] (P.w[reserved0]); 1 / wi[1] is at reserved0 + 1
    const bool fold = nonlinlap_fold(d, k);
    const std::string FOLDC = "P.w[P.terms[" + K + "].reserved0]", RWI = "P.w[P.terms[" + K + "].reserved0 + 1]";

    // face program (forward), given uf*/fa* variables named with `tag`, result in `tag`a
    auto face_forward = [&](const std::string& tag) {
        if (!has_prog) {
            e << "    const T " << tag << "a = T(1);\n";
            return;
        }
        FaceLeaves L(tag);
        std::vector<std::pair<int, int>> outs;
        emit_forward(e, d, fs, L, tag, &outs, false);
        e << "    const T " << tag << "a = " << (outs.empty() ? "T(1)" : tag + v(outs[0].second)) << ";\n";
    };

    // generic face (runtime taps)
    const std::string NTI = std::to_string(max_taps(oi)), NTP = std::to_string(max_taps(op)),
                      NTO = std::to_string(max_taps(oo));
    e << "template <class T>\n__device__ __forceinline__ T gface" << K
      << "(const DevProb<T>& P, const T* __restrict__ u, long long c, const int* I, int Ih, T t, const T* __restrict__ "
         "p) {\n"
      << "    const T du = apply_op_line<T, " << D << ", " << NTI << ", " << dyn_bc(d, tm.field, tm.dim) << ">(P, P.ops["
      << opi << "], u, " << F << ", I, c, Ih, P.n[" << D << "], t, p);\n";
    for (int f : used_fields)
        e << "    const T uf" << f << " = apply_op_line<T, " << D << ", " << NTP << ", " << dyn_bc(d, f, tm.dim)
          << ">(P, P.ops[" << opp << "], u, " << f << ", I, c, Ih, P.n[" << D << "], t, p);\n";
    for (int j : used_aux)
        e << "    const T fa" << j << " = P.aux[P.aux_off[P.terms[" << K << "].aux0 + " << j << "] + face_index(P, " << D
          << ", Ih, I)];\n";
    face_forward("");
    e << "    return a * du;\n}\n";

    // generic face adjoint
    e << "template <class T>\n__device__ __forceinline__ void gface" << K
      << "_vjp(const DevProb<T>& P, const T* __restrict__ u, long long c, const int* I, int Ih, T t, const T* "
         "__restrict__ p, T g, T* lam_u, T* lp, T* lam_aux) {\n"
      << "    const T du = apply_op_line<T, " << D << ", " << NTI << ", " << dyn_bc(d, tm.field, tm.dim) << ">(P, P.ops["
      << opi << "], u, " << F << ", I, c, Ih, P.n[" << D << "], t, p);\n";
    for (int f : used_fields)
        e << "    const T uf" << f << " = apply_op_line<T, " << D << ", " << NTP << ", " << dyn_bc(d, f, tm.dim)
          << ">(P, P.ops[" << opp << "], u, " << f << ", I, c, Ih, P.n[" << D << "], t, p);\n    T guf" << f
          << " = T(0);\n";
    for (int j : used_aux)
        e << "    const long long fi" << j << " = P.aux_off[P.terms[" << K << "].aux0 + " << j << "] + face_index(P, "
          << D << ", Ih, I);\n    const T fa" << j << " = P.aux[fi" << j << "];\n    T gfa" << j << " = T(0);\n";
    face_forward("");
    e << "    scatter_op_line<T, " << D << ", " << NTI << ", " << dyn_bc(d, tm.field, tm.dim) << ">(P, P.ops[" << opi
      << "], lam_u, " << F << ", I, c, Ih, P.n[" << D << "], g * a, t, p);\n";
    if (has_prog) {
        FaceLeaves L("");
        emit_reverse(e, fs, L, "", [&](int) { return std::string("g * du"); });
        for (int f : used_fields)
            e << "    scatter_op_line<T, " << D << ", " << NTP << ", " << dyn_bc(d, f, tm.dim) << ">(P, P.ops[" << opp
              << "], lam_u, " << f << ", I, c, Ih, P.n[" << D << "], guf" << f << ", t, p);\n";
        for (int j : used_aux) e << "    if (lam_aux) atomicAdd(lam_aux + fi" << j << ", gfa" << j << ");\n";
    }
    e << "}\n";

    // Along a periodic dimension (this field and every interpolated one) all cells use the
    // interior weights with wrapped tap offsets; face indices stay unwrapped as on the
    // edge path.
    bool per = periodic_dim(d, tm.field, tm.dim);
    for (int f : used_fields) per = per && periodic_dim(d, f, tm.dim);
    int reach = 0;
    for (int m : nzo) {
        const int r = oo.omin + m - 1;
        for (int t_ : nzi) reach = std::max(reach, std::abs(r + oi.omin + t_));
        for (int t_ : nzp) reach = std::max(reach, std::abs(r + op.omin + t_));
    }
    auto toff = [&](int x) {
        return per ? "(long long)wrap_off(I[" + D + "], " + std::to_string(x) + ", P.n[" + D + "]) * s"
                   : "(long long)(" + std::to_string(x) + ") * s";
    };
    // Folded form: the stored face value F' of half point Ih from runtime positions, with the
    // fast paths' arithmetic where the face's stencils are interior (so the face pass, the
    // ensemble's window and the cells' own evaluation agree bit for bit), else the generic
    // face divided by wi[1].  The edge path of the cell reads faces through it.
    int reach_l = 0;
    for (int t_ : nzi) reach_l = std::max(reach_l, std::abs(-1 + oi.omin + t_));
    for (int t_ : nzp) reach_l = std::max(reach_l, std::abs(-1 + op.omin + t_));
    if (fold) {
        std::string gc;
        if (per) {
            gc = "wrap_line_ok(P, " + F + ", " + D + ", " + std::to_string(reach_l) + ")";
            for (int f : used_fields)
                if (f != tm.field)
                    gc += " && wrap_line_ok(P, " + std::to_string(f) + ", " + D + ", " + std::to_string(reach_l) + ")";
        } else {
            gc = "fast_line(P, P.ops[" + opi + "], " + F + ", " + D + ", Ih) && fast_line(P, P.ops[" + opp + "], " + F +
                 ", " + D + ", Ih)";
        }
        auto lp = [&](int f, const std::string& pos) {
            return "line_pt<T, " + D + ", " + dyn_bc(d, f, tm.dim) + ">(P, u, " + std::to_string(f) + ", I, c, " + pos +
                   ", t, p)";
        };
        e << "template <class T>\n__device__ __forceinline__ T gfacef" << K
          << "(const DevProb<T>& P, const T* __restrict__ u, long long c, const int* I, int Ih, T t, const T* "
             "__restrict__ p) {\n"
          << "    if (" << gc << ") {\n"
          << "    const T* __restrict__ wp = P.w + P.ops[" << opp << "].w_int;\n"
          << "    const T gf_du = " << lp(tm.field, "Ih + (" + std::to_string(oi.omin + 1) + ")") << " - "
          << lp(tm.field, "Ih + (" + std::to_string(oi.omin) + ")") << ";\n";
        for (int f : used_fields) {
            for (size_t q = 0; q < nzp.size(); ++q) {
                const int t_ = nzp[q];
                const std::string tap = lp(f, "Ih + (" + std::to_string(op.omin + t_) + ")");
                if (q == 0) e << "    T gf_uf" << f << " = wp[" << t_ << "] * " << tap << ";\n";
                else e << "    gf_uf" << f << " = fma(wp[" << t_ << "], " << tap << ", gf_uf" << f << ");\n";
            }
            if (nzp.empty()) e << "    T gf_uf" << f << " = T(0);\n";
        }
        for (int j : used_aux)
            e << "    const T gf_fa" << j << " = P.aux[P.aux_off[P.terms[" << K << "].aux0 + " << j
              << "] + face_index(P, " << D << ", Ih, I)];\n";
        face_forward("gf_");
        e << "    return mulrn(gf_a, gf_du);\n    }\n"
          << "    return gface" << K << "<T>(P, u, c, I, Ih, t, p) * " << RWI << ";\n}\n";
    }
    // fast path helpers: relative face offsets r = omin_outer + m - 1 (outer stencil sits at II - 1)
    // statements computing the face at relative half point r: tag du, tag uf<f>, the face
    // program; leaves tag a and tag du
    auto face_body = [&](int r, const std::string& tag, bool vjp) {
        // inner derivative (folded: the plain difference, its weight wi[1] moves to the cell)
        if (fold && !vjp)
            e << "    const T " << tag << "du = bF[" << toff(r + oi.omin + 1) << "] - bF[" << toff(r + oi.omin + 0)
              << "];\n";
        for (size_t q = 0; q < nzi.size() && !(fold && !vjp); ++q) {
            const int t_ = nzi[q];
            const std::string tap = "bF[" + toff(r + oi.omin + t_) + "]";
            if (q == 0) e << "    T " << tag << "du = wi[" << t_ << "] * " << tap << ";\n";
            else e << "    " << tag << "du = fma(wi[" << t_ << "], " << tap << ", " << tag << "du);\n";
        }
        if (nzi.empty() && !(fold && !vjp)) e << "    T " << tag << "du = T(0);\n";
        for (int f : used_fields) {
            e << "    const T* __restrict__ bf" << f << " = u + (long long)" << f << " * P.ncell + c;\n";
            for (size_t q = 0; q < nzp.size(); ++q) {
                const int t_ = nzp[q];
                const std::string tap = "bf" + std::to_string(f) + "[" + toff(r + op.omin + t_) + "]";
                if (q == 0) e << "    T " << tag << "uf" << f << " = wp[" << t_ << "] * " << tap << ";\n";
                else e << "    " << tag << "uf" << f << " = fma(wp[" << t_ << "], " << tap << ", " << tag << "uf" << f
                       << ");\n";
            }
            if (nzp.empty()) e << "    T " << tag << "uf" << f << " = T(0);\n";
            if (vjp) e << "    T " << tag << "guf" << f << " = T(0);\n";
        }
        for (int j : used_aux) {
            e << "    const long long " << tag << "fi" << j << " = P.aux_off[P.terms[" << K << "].aux0 + " << j
              << "] + face_index(P, " << D << ", I[" << D << "] + (" << r << "), I);\n";
            e << "    const T " << tag << "fa" << j << " = P.aux[" << tag << "fi" << j << "];\n";
            if (vjp) e << "    T " << tag << "gfa" << j << " = T(0);\n";
        }
        face_forward(tag);
    };
    // face r of this cell from the face pass: the left face of cell I + r + 1 along D, when that
    // cell is an unknown reached without a wrap
    const std::string FQ = std::to_string(face_slot);
    auto from_pass = [&](int r) {
        const std::string cf = "c + (long long)(" + std::to_string(r + 1) + ") * s";
        return "P.faces && I[" + D + "] + (" + std::to_string(r + 1) + ") > P.lo[" + D + "] && I[" + D + "] + (" +
               std::to_string(r + 1) + ") <= P.n[" + D + "] - P.up[" + D + "] && " + cf + " >= P.fbeg && " + cf +
               " < P.fend";
    };
    auto fast_face = [&](int m, bool vjp) {
        const int r = oo.omin + m - 1;
        const std::string tag = "f" + std::to_string(m) + "_";
        e << "    {\n";
        if (!vjp && fold) {
            // the two faces go to F0 / F1 declared by the caller
            face_body(r, tag, false);
            e << "    F" << m << " = mulrn(" << tag << "a, " << tag << "du);\n";
        } else if (!vjp) {
            face_body(r, tag, false);
            e << "    const T " << tag << "F = " << tag << "a * " << tag << "du;\n";
            e << "    acc = started ? fma(wo[" << m << "], " << tag << "F, acc) : wo[" << m << "] * " << tag << "F;\n"
              << "    started = true;\n";
        } else {
            face_body(r, tag, true);
            e << "    const T " << tag << "g = g * wo[" << m << "];\n";
            e << "    { const T gd = " << tag << "g * " << tag << "a;\n";
            for (int t_ : nzi)
                e << "      atomicAdd(lF + " << toff(r + oi.omin + t_) << ", gd * wi[" << t_ << "]);\n";
            e << "    }\n";
            if (has_prog) {
                FaceLeaves L(tag);
                const std::string seed = tag + "g * " + tag + "du";
                emit_reverse(e, fs, L, tag, [&](int) { return seed; });
                for (int f : used_fields)
                    for (int t_ : nzp)
                        e << "    atomicAdd(lam_u + (long long)" << f << " * P.ncell + c + " << toff(r + op.omin + t_)
                          << ", " << tag << "guf" << f << " * wp[" << t_ << "]);\n";
                for (int j : used_aux)
                    e << "    if (lam_aux) atomicAdd(lam_aux + " << tag << "fi" << j << ", " << tag << "gfa" << j
                      << ");\n";
            }
        }
        e << "    }\n";
    };
    std::string cond = "warp_all(fast_nonlinlap(P, P.ops[" + opo + "], P.ops[" + opi + "], P.ops[" + opp + "], " + F +
                       ", " + D + ", I[" + D + "]))";
    if (per) {
        cond = "wrap_line_ok(P, " + F + ", " + D + ", " + std::to_string(reach) + ")";
        for (int f : used_fields)
            if (f != tm.field) cond += " && wrap_line_ok(P, " + std::to_string(f) + ", " + D + ", " + std::to_string(reach) + ")";
    }
    // per-point rows (nonuniform grid): the compile-time fast path reads one interior row, so
    // every cell takes the runtime-tap path, whose tap selection picks each position's row
    const bool rows = oo.nrows > 0 || oi.nrows > 0 || op.nrows > 0;
    if (rows) cond = "false";
    for (int vjp = 0; vjp < 2; ++vjp) {
        if (!vjp)
            e << "template <class T>\n__device__ __forceinline__ T gt" << K
              << "(const DevProb<T>& P, const T* __restrict__ u, long long c, const int* I, T t, const T* __restrict__ "
                 "p) {\n";
        else
            e << "template <class T>\n__device__ __forceinline__ void gt" << K
              << "_vjp(const DevProb<T>& P, const T* __restrict__ u, long long c, const int* I, T t, const T* "
                 "__restrict__ p, T g, T* lam_u, T* lp, T* lam_aux, T& own) {\n";
        e << "    if (" << cond << ") {\n"
          << "    const T* __restrict__ wo = P.w + P.ops[" << opo << "].w_int;\n"
          << "    const T* __restrict__ wi = P.w + P.ops[" << opi << "].w_int;\n"
          << "    const T* __restrict__ wp = P.w + P.ops[" << opp << "].w_int;\n"
          << "    const T* __restrict__ bF = u + (long long)" << F << " * P.ncell + c;\n"
          << "    const long long s = gstride(P, " << D << ");\n";
        if (!vjp) {
            // every face of the warp's cells from the face pass: a warp-uniform branch, so the
            // face arithmetic below is not issued at all (FP64 instructions cost the same
            // predicated off)
            std::string all_owned = "P.faces";
            for (int m : nzo) all_owned += " && " + from_pass(oo.omin + m - 1);
            e << "    if (warp_all(" << all_owned << ")) {\n"
              << "    const T* __restrict__ fq = P.faces + (long long)" << FQ << " * P.fstride + c;\n";
            if (fold) {
                e << "    return " << FOLDC << " * (fq[(long long)(" << (oo.omin + 1) << ") * s] - fq[(long long)("
                  << oo.omin << ") * s]);\n    }\n";
                e << "    T F0, F1;\n";
            } else {
                bool first = true;
                for (int m : nzo) {
                    const int r = oo.omin + m - 1;
                    const std::string Fv = "fq[(long long)(" + std::to_string(r + 1) + ") * s]";
                    if (first) e << "    T acc = wo[" << m << "] * " << Fv << ";\n";
                    else e << "    acc = fma(wo[" << m << "], " << Fv << ", acc);\n";
                    first = false;
                }
                e << "    return " << (nzo.empty() ? "T(0)" : "acc") << ";\n    }\n";
                e << "    T acc = T(0);\n    bool started = false;\n";
            }
        } else {
            e << "    T* lF = lam_u + (long long)" << F << " * P.ncell + c;\n";
        }
        for (int m : nzo) fast_face(m, vjp);
        if (!vjp && fold) e << "    return " << FOLDC << " * (F1 - F0);\n    }\n";
        else if (!vjp) e << "    return acc;\n    }\n";
        else e << "    return;\n    }\n";
        // generic path: runtime outer taps
        e << "    const bool per = (P.permask[" << F << "] >> " << D << ") & 1;\n"
          << "    const TapSel so = select_taps(P.ops[" << opo << "], I[" << D << "] - 1, P.n[" << D << "] - 1, per);\n";
        if (!vjp) e << "    T acc = T(0);\n    bool started = false;\n";
        e << "#pragma unroll\n    for (int q = 0; q < " << NTO << "; ++q) {\n"
          << "        if (q >= so.cnt) break;\n"
          << "        const T w_ = P.w[so.woff + q];\n        if (w_ == T(0)) continue;\n";
        if (!vjp)
            e << "        const int Ih = so.first + q;\n"
              << "        T F_;\n"
              << "        const long long cf_ = c + (long long)(Ih + 1 - I[" << D << "]) * gstride(P, " << D << ");\n"
              << "        if (P.faces && Ih + 1 > P.lo[" << D << "] && Ih + 1 <= P.n[" << D << "] - P.up[" << D
              << "] && cf_ >= P.fbeg && cf_ < P.fend)\n"
              << "            F_ = P.faces[(long long)" << FQ << " * P.fstride + cf_]"
              << (fold ? " * P.w[P.ops[" + opi + "].w_int + 1]" : "") << ";\n"
              << "        else\n"
              << (fold ? "            F_ = gfacef" + K + "<T>(P, u, c, I, Ih, t, p) * P.w[P.ops[" + opi +
                             "].w_int + 1];\n"
                       : "            F_ = gface" + K + "<T>(P, u, c, I, Ih, t, p);\n")
              << "        acc = started ? fma(w_, F_, acc) : w_ * F_;\n        started = true;\n    }\n    return acc;\n";
        else
            e << "        gface" << K << "_vjp<T>(P, u, c, I, so.first + q, t, p, g * w_, lam_u, lp, lam_aux);\n    }\n";
        e << "}\n";
    }
    // the face pass: the left face (half point I - 1/2) of this cell
    int reach_left = 0;
    for (int t_ : nzi) reach_left = std::max(reach_left, std::abs(-1 + oi.omin + t_));
    for (int t_ : nzp) reach_left = std::max(reach_left, std::abs(-1 + op.omin + t_));
    std::string lcond;
    if (per) {
        lcond = "wrap_line_ok(P, " + F + ", " + D + ", " + std::to_string(reach_left) + ")";
        for (int f : used_fields)
            if (f != tm.field)
                lcond += " && wrap_line_ok(P, " + std::to_string(f) + ", " + D + ", " + std::to_string(reach_left) + ")";
    } else {
        lcond = "warp_all(fast_line(P, P.ops[" + opi + "], " + F + ", " + D + ", I[" + D + "] - 1) && fast_line(P, P.ops[" +
                opp + "], " + F + ", " + D + ", I[" + D + "] - 1))";
    }
    if (rows) lcond = "false";
    e << "template <class T>\n__device__ __forceinline__ T gfl" << K
      << "(const DevProb<T>& P, const T* __restrict__ u, long long c, const int* I, T t, const T* __restrict__ p) {\n"
      << "    if (" << lcond << ") {\n"
      << "    const T* __restrict__ wi = P.w + P.ops[" << opi << "].w_int;\n"
      << "    const T* __restrict__ wp = P.w + P.ops[" << opp << "].w_int;\n"
      << "    const T* __restrict__ bF = u + (long long)" << F << " * P.ncell + c;\n"
      << "    const long long s = gstride(P, " << D << ");\n";
    face_body(-1, "fl_", false);
    e << "    return " << (fold ? "mulrn(fl_a, fl_du)" : "fl_a * fl_du") << ";\n    }\n"
      << "    return " << (fold ? "gfacef" : "gface") << K << "<T>(P, u, c, I, I[" << D << "] - 1, t, p);\n}\n";
}

}  // namespace

// ----------------------------------------------------------------------------
// The cell function: uniform hoisting and linear-stencil fusion.
//
// Values that depend only on constants, parameters and time are computed once per
// thread (gen_uniform) instead of once per cell.  A linear combination of LINEAR /
// MIXED terms of one field with uniform coefficients (e.g. alpha*(Dxx u + Dyy u)) is
// evaluated, where every member term is on its interior fast path, as ONE stencil over
// the union of the taps with pre-combined weights (shared centre tap, coefficient
// folded in); elsewhere the original statements run.  On GB300 this removes FP64
// operations, the binding resource.
// ----------------------------------------------------------------------------

// Where a group's fused stencil applies: every member on its interior (or wrapped periodic)
// path; a variable group also needs the plan's coefficient arrays (batches have none).
static std::string group_cond(const mol_problem_desc* d, const FoldGroup& g) {
    const std::string F = std::to_string(g.field);
    std::set<int> members;
    int reach[3] = {0, 0, 0};
    for (const FoldTap& t : g.taps) {
        for (const FoldPart& p : t.parts) members.insert(p.term);
        for (int q = 0; q < 3; ++q) reach[q] = std::max(reach[q], std::abs(t.o[q]));
    }
    std::string cond_u, cond_w;   // uniform (periodic wrap) and per-cell (interior) parts
    for (int q = 0; q < 3; ++q) {
        if (!reach[q]) continue;
        if (periodic_dim(d, g.field, q)) {
            cond_u += (cond_u.empty() ? "" : " && ") + std::string("wrap_line_ok(P, ") + F + ", " + std::to_string(q) +
                      ", " + std::to_string(reach[q]) + ")";
            continue;
        }
        for (int k : members) {
            const mol_term& tm = d->terms[k];
            if (tm.kind == MOL_TERM_NONLINLAP) {
                // the variable member's own interior condition (outer, inner and interpolation
                // stencils all on their interior weights)
                if (tm.dim == q)
                    cond_w += (cond_w.empty() ? "" : " && ") + std::string("fast_nonlinlap(P, P.ops[") +
                              std::to_string(tm.op) + "], P.ops[" + std::to_string(tm.op2) + "], P.ops[" +
                              std::to_string(tm.op3) + "], " + F + ", " + std::to_string(q) + ", I[" +
                              std::to_string(q) + "])";
                continue;
            }
            const int op = tm.dim == q ? tm.op : (tm.kind == MOL_TERM_MIXED && tm.dim2 == q ? tm.op2 : -1);
            if (op < 0) continue;
            cond_w += (cond_w.empty() ? "" : " && ") + std::string("fast_line(P, P.ops[") + std::to_string(op) + "], " +
                      F + ", " + std::to_string(q) + ", I[" + std::to_string(q) + "])";
        }
    }
    std::string cond = cond_u.empty() ? "true" : cond_u;
    if (g.variable) cond = "P.cw && " + cond;
    if (!cond_w.empty()) cond += " && warp_all(" + cond_w + ")";
    return cond;
}

// Offset of a group tap from the cell (wrapped along periodic dimensions).
static std::string group_tap_off(const mol_problem_desc* d, const FoldGroup& g, const FoldTap& t) {
    std::string off;
    for (int q = 0; q < 3; ++q) {
        if (!t.o[q]) continue;
        const std::string oq = std::to_string(t.o[q]);
        const std::string term = periodic_dim(d, g.field, q)
                                     ? "(long long)wrap_off(I[" + std::to_string(q) + "], " + oq + ", P.n[" +
                                           std::to_string(q) + "]) * gstride(P, " + std::to_string(q) + ")"
                                     : "(long long)(" + oq + ") * gstride(P, " + std::to_string(q) + ")";
        off += (off.empty() ? "" : " + ") + term;
    }
    return off.empty() ? "0" : off;
}

struct LinInfo {
    bool ok = false;
    int field = -1;
    std::map<int, std::string> coef;  // term -> coefficient expression (uniform)
    std::vector<int> members;         // non-uniform pcs of the tree (terms included)
};

static void emit_cell_fused(Emitter& e, const mol_problem_desc* d, const SSA& s, const std::string& cell_attr) {
    const int n = (int)s.ins.size();
    std::vector<char> uni(n, 0);
    std::vector<int> uses(n, 0);
    for (int pc = 0; pc < n; ++pc) {
        const mol_instr& in = s.ins[pc];
        for (int x : {s.ia[pc], s.ib[pc], s.ic[pc]})
            if (x >= 0) uses[x]++;
        switch (in.op) {
            case MOL_OP_CONST: case MOL_OP_PARAM: case MOL_OP_TIME: uni[pc] = 1; break;
            case MOL_OP_ADD: case MOL_OP_SUB: case MOL_OP_MUL: case MOL_OP_DIV: case MOL_OP_POW: case MOL_OP_CMP:
                uni[pc] = uni[s.ia[pc]] && uni[s.ib[pc]];
                break;
            case MOL_OP_NEG: case MOL_OP_POWI: case MOL_OP_FN: uni[pc] = uni[s.ia[pc]]; break;
            case MOL_OP_IFELSE: uni[pc] = uni[s.ia[pc]] && uni[s.ib[pc]] && uni[s.ic[pc]]; break;
            default: uni[pc] = 0;
        }
    }
    auto name = [&](int pc) { return uni[pc] ? "U.u" + std::to_string(pc) : v(pc); };
    // constant-coefficient fusion of first-derivative stencils (const_linear_groups): the
    // nodes a group absorbs are emitted on its fallback path only
    const std::vector<FoldGroup> cgroups = const_linear_groups(d);
    std::vector<char> cabs(n, 0);
    std::map<int, int> cgroup_at;
    for (size_t gi = 0; gi < cgroups.size(); ++gi) {
        for (int q : cgroups[gi].absorbed) cabs[q] = 1;
        cgroup_at[cgroups[gi].out_pc] = (int)gi;
    }
    // linear analysis
    std::vector<LinInfo> lin(n);
    for (int pc = 0; pc < n; ++pc) {
        const mol_instr& in = s.ins[pc];
        LinInfo L;
        if (in.op == MOL_OP_TERM) {
            const mol_term& tm = d->terms[in.imm];
            // per-point rows (nonuniform grid) have no compile-time tap weights: not fused
            if ((tm.kind == MOL_TERM_LINEAR && d->ops[tm.op].nrows == 0) ||
                (tm.kind == MOL_TERM_MIXED && d->ops[tm.op].nrows == 0 && d->ops[tm.op2].nrows == 0)) {
                L.ok = true;
                L.field = tm.field;
                L.coef[in.imm] = "T(1)";
                L.members = {pc};
            }
        } else if ((in.op == MOL_OP_ADD || in.op == MOL_OP_SUB) && !uni[pc]) {
            const LinInfo& A = lin[s.ia[pc]];
            const LinInfo& B = lin[s.ib[pc]];
            if (A.ok && B.ok && A.field == B.field && uses[s.ia[pc]] == 1 && uses[s.ib[pc]] == 1) {
                L = A;
                for (auto& kv : B.coef) {
                    const std::string c = in.op == MOL_OP_SUB ? "(-" + kv.second + ")" : kv.second;
                    L.coef[kv.first] = L.coef.count(kv.first) ? "(" + L.coef[kv.first] + " + " + c + ")" : c;
                }
                L.members.insert(L.members.end(), B.members.begin(), B.members.end());
                L.members.push_back(pc);
            }
        } else if (in.op == MOL_OP_MUL && !uni[pc]) {
            const int a = s.ia[pc], b = s.ib[pc];
            const int li = lin[a].ok ? a : (lin[b].ok ? b : -1);
            const int ui = li == a ? b : a;
            if (li >= 0 && uni[ui] && uses[li] == 1) {
                L = lin[li];
                for (auto& kv : L.coef) kv.second = "(" + kv.second + " * " + name(ui) + ")";
                L.members.push_back(pc);
            }
        } else if (in.op == MOL_OP_NEG && !uni[pc]) {
            if (lin[s.ia[pc]].ok && uses[s.ia[pc]] == 1) {
                L = lin[s.ia[pc]];
                for (auto& kv : L.coef) kv.second = "(-" + kv.second + ")";
                L.members.push_back(pc);
            }
        }
        lin[pc] = L;
    }
    // roots: linear nodes whose single user is not linear in them, with >= 2 terms or a scaling
    std::vector<int> user(n, -1);
    for (int pc = 0; pc < n; ++pc)
        for (int x : {s.ia[pc], s.ib[pc], s.ic[pc]})
            if (x >= 0) user[x] = pc;
    std::vector<char> root(n, 0), absorbed(n, 0);
    // Off by default: on GB300 the fused stencil's extra live weights cost more occupancy than
    // the FP64 operations it saves (measured); MOL_JIT_FUSE=1 turns it on.
    const char* fz = getenv("MOL_JIT_FUSE");
    const bool fuse = fz && fz[0] == '1' && cgroups.empty();
    for (int pc = n - 1; pc >= 0 && fuse; --pc) {
        if (!lin[pc].ok || absorbed[pc]) continue;
        if (s.ins[pc].op == MOL_OP_TERM) continue;  // a lone term gains nothing
        const int u = user[pc];
        const bool extends = u >= 0 && lin[u].ok && std::find(lin[u].members.begin(), lin[u].members.end(), pc) !=
                                                       lin[u].members.end();
        if (extends) continue;
        root[pc] = 1;
        for (int m : lin[pc].members)
            if (m != pc) absorbed[m] = 1;
    }
    // tap unions of the roots
    struct Tap {
        int o[3];
        std::vector<std::pair<int, std::string>> parts;  // (term k, weight expression)
    };
    std::map<int, std::vector<Tap>> taps;
    for (int pc = 0; pc < n; ++pc) {
        if (!root[pc]) continue;
        std::vector<Tap>& T = taps[pc];
        auto add = [&](int o0, int o1, int o2, int k, const std::string& w) {
            for (auto& t : T)
                if (t.o[0] == o0 && t.o[1] == o1 && t.o[2] == o2) {
                    t.parts.push_back({k, w});
                    return;
                }
            Tap t;
            t.o[0] = o0;
            t.o[1] = o1;
            t.o[2] = o2;
            t.parts.push_back({k, w});
            T.push_back(t);
        };
        for (auto& kv : lin[pc].coef) {
            const mol_term& tm = d->terms[kv.first];
            if (tm.kind == MOL_TERM_LINEAR) {
                const mol_op1d& o = d->ops[tm.op];
                for (int m = 0; m < o.L; ++m) {
                    if (zero_w(d, o.w_int + m)) continue;
                    int off[3] = {0, 0, 0};
                    off[tm.dim] = o.omin + m;
                    add(off[0], off[1], off[2], kv.first,
                        "P.w[P.ops[" + std::to_string(tm.op) + "].w_int + " + std::to_string(m) + "]");
                }
            } else {
                const mol_op1d& o1 = d->ops[tm.op];
                const mol_op1d& o2 = d->ops[tm.op2];
                for (int x = 0; x < o1.L; ++x)
                    for (int y = 0; y < o2.L; ++y) {
                        if (zero_w(d, o1.w_int + x) || zero_w(d, o2.w_int + y)) continue;
                        int off[3] = {0, 0, 0};
                        off[tm.dim] += o1.omin + x;
                        off[tm.dim2] += o2.omin + y;
                        add(off[0], off[1], off[2], kv.first,
                            "P.w[P.terms[" + std::to_string(kv.first) + "].reserved0 + " +
                                std::to_string(x * o2.L + y) + "]");
                    }
            }
        }
    }
    // uniform struct and its initialiser
    e << "template <class T>\nstruct GenUniform {\n    T _pad;\n";
    for (int pc = 0; pc < n; ++pc)
        if (uni[pc]) e << "    T u" << pc << ";\n";
    for (auto& kv : taps)
        for (size_t i = 0; i < kv.second.size(); ++i) e << "    T fw" << kv.first << "_" << i << ";\n";
    e << "};\n";
    e << "template <class T>\n__device__ __forceinline__ void gen_uniform(const DevProb<T>& P, T t, const T* __restrict__ "
         "p, GenUniform<T>& U) {\n    U._pad = T(0);\n";
    for (int pc = 0; pc < n; ++pc) {
        if (!uni[pc]) continue;
        const mol_instr& in = s.ins[pc];
        const std::string A = s.ia[pc] >= 0 ? name(s.ia[pc]) : "", B = s.ib[pc] >= 0 ? name(s.ib[pc]) : "",
                          C = s.ic[pc] >= 0 ? name(s.ic[pc]) : "";
        std::string rhs;
        switch (in.op) {
            case MOL_OP_CONST: {
                rhs = lit(d->consts[in.imm]);
                if (rhs.empty()) rhs = "P.consts[" + std::to_string(in.imm) + "]";
                break;
            }
            case MOL_OP_PARAM: rhs = "p[" + std::to_string(in.imm) + "]"; break;
            case MOL_OP_TIME: rhs = "t"; break;
            case MOL_OP_ADD: rhs = A + " + " + B; break;
            case MOL_OP_SUB: rhs = A + " - " + B; break;
            case MOL_OP_MUL: rhs = A + " * " + B; break;
            case MOL_OP_DIV: rhs = A + " / " + B; break;
            case MOL_OP_NEG: rhs = "-" + A; break;
            case MOL_OP_POWI:
                rhs = in.imm == 2 ? A + " * " + A : (in.imm == 3 ? A + " * " + A + " * " + A
                                                                  : "powi(" + A + ", " + std::to_string(in.imm) + ")");
                break;
            case MOL_OP_POW: rhs = "pow(" + A + ", " + B + ")"; break;
            case MOL_OP_FN: rhs = fn_expr(in.imm, A); break;
            case MOL_OP_CMP: {
                static const char* ops[] = {"<=", "<", ">=", ">", "=="};
                rhs = "(" + A + " " + ops[in.imm] + " " + B + ") ? T(1) : T(0)";
                break;
            }
            case MOL_OP_IFELSE: rhs = "(" + A + " != T(0)) ? " + B + " : " + C; break;
            default: rhs = "T(0)";
        }
        e << "    U.u" << pc << " = " << rhs << ";\n";
    }
    for (auto& kv : taps) {
        const int r = kv.first;
        for (size_t i = 0; i < kv.second.size(); ++i) {
            std::string ex;
            for (auto& part : kv.second[i].parts) {
                const std::string term = lin[r].coef.at(part.first) + " * " + part.second;
                ex = ex.empty() ? term : ex + " + " + term;
            }
            e << "    U.fw" << r << "_" << i << " = " << ex << ";\n";
        }
    }
    e << "}\n";
    // the cell
    CellLeaves CL;
    e << "template <class T>\n__device__ " << cell_attr
      << " void gen_cell(const DevProb<T>& P, const T* __restrict__ u, long long c, const int* I, T t, "
         "const T* __restrict__ p, const GenUniform<T>& U, T* out) {\n";
    auto stmt = [&](int pc) -> std::string {
        const mol_instr& in = s.ins[pc];
        const std::string V = v(pc);
        const std::string A = s.ia[pc] >= 0 ? name(s.ia[pc]) : "", B = s.ib[pc] >= 0 ? name(s.ib[pc]) : "",
                          C = s.ic[pc] >= 0 ? name(s.ic[pc]) : "";
        switch (in.op) {
            case MOL_OP_FIELD: return "const T " + V + " = " + CL.field(in.imm) + ";";
            case MOL_OP_AUX: return "const T " + V + " = " + CL.aux(in.imm) + ";";
            case MOL_OP_COORD: return "const T " + V + " = " + CL.coord(in.imm) + ";";
            case MOL_OP_TERM: return "const T " + V + " = " + CL.term(in.imm) + ";";
            case MOL_OP_UPWIND:
                return "const T tv" + std::to_string(pc) + " = (" + A + " < T(0)) ? " + CL.term(in.b) + " : " +
                       CL.term(in.c) + ";\n    const T " + V + " = " + A + " * tv" + std::to_string(pc) + ";";
            case MOL_OP_ADD: return "const T " + V + " = " + A + " + " + B + ";";
            case MOL_OP_SUB: return "const T " + V + " = " + A + " - " + B + ";";
            case MOL_OP_MUL: return "const T " + V + " = " + A + " * " + B + ";";
            case MOL_OP_DIV: return "const T " + V + " = " + A + " / " + B + ";";
            case MOL_OP_NEG: return "const T " + V + " = -" + A + ";";
            case MOL_OP_POWI:
                if (in.imm == 2) return "const T " + V + " = " + A + " * " + A + ";";
                if (in.imm == 3) return "const T " + V + " = " + A + " * " + A + " * " + A + ";";
                return "const T " + V + " = powi(" + A + ", " + std::to_string(in.imm) + ");";
            case MOL_OP_POW: return "const T " + V + " = pow(" + A + ", " + B + ");";
            case MOL_OP_FN: return "const T " + V + " = " + fn_expr(in.imm, A) + ";";
            case MOL_OP_CMP: {
                static const char* ops[] = {"<=", "<", ">=", ">", "=="};
                return "const T " + V + " = (" + A + " " + ops[in.imm] + " " + B + ") ? T(1) : T(0);";
            }
            case MOL_OP_IFELSE: return "const T " + V + " = (" + A + " != T(0)) ? " + B + " : " + C + ";";
            default: return "";
        }
    };
    // one constant-coefficient group: the fused stencil where every member is on its interior
    // (or wrapped periodic) path, the original terms elsewhere, then the output's other addends
    auto emit_cgroup = [&](int gi, int out_field) {
        const FoldGroup& g = cgroups[gi];
        const std::string G = "fg" + std::to_string(gi), F = std::to_string(g.field);
        const std::string cond = group_cond(d, g);
        e << "    T " << G << ";\n    if (" << cond << ") {\n"
          << "        const T* __restrict__ fw = P.w + P.terms[" << g.key_term << "].reserved2;\n"
          << "        const T* __restrict__ fb = u + (long long)" << F << " * P.ncell + c;\n";
        if (g.variable) {
            e << "        const T* __restrict__ cw = P.cw + (long long)" << g.arr0 << " * P.ncell + c;\n";
            bool anydiff = g.quad_coef >= 0;
            for (const FoldTap& t : g.taps) anydiff |= t.diff;
            if (anydiff) e << "        const T u0 = fb[0];\n";
        }
        const std::vector<double> fwv = fold_weights(d, g);
        bool started = false;
        for (size_t i = 0; i < g.taps.size(); ++i) {
            // a uniform weight that is exactly zero (the difference form's centre when the
            // differenced constant parts cancel it) is left out
            if (g.variable && g.taps[i].arr < 0 && fwv[i] == 0.0) continue;
            const std::string off = group_tap_off(d, g, g.taps[i]);
            const FoldTap& tp = g.taps[i];
            const std::string wv = tp.arr >= 0 ? (tp.arr == 0 ? std::string("cw[0]")
                                                              : "cw[(long long)" + std::to_string(tp.arr) + " * P.ncell]")
                                               : "fw[" + std::to_string(i) + "]";
            std::string xv = tp.diff ? "(fb[" + off + "] - u0)" : "fb[" + off + "]";
            std::string wq = wv;
            if (g.quad_coef >= 0 && tp.arr >= 0 && !tp.o[0] && !tp.o[1] && !tp.o[2]) {
                // the reaction k u^2 on the centre tap: (c_0 + k u) u
                wq = "fma(" + std::string(g.quad_sign < 0 ? "-" : "") + name(g.quad_coef) + ", u0, " + wv + ")";
                xv = "u0";
            }
            if (!started) e << "        T acc = " << wq << " * " << xv << ";\n";
            else e << "        acc = fma(" << wq << ", " << xv << ", acc);\n";
            started = true;
        }
        e << "        " << G << " = " << (started ? "acc" : "T(0)") << ";\n    } else {\n";
        for (int q : g.leaf_nodes) e << "        " << stmt(q) << "\n";
        std::string fsum;
        for (auto& a : g.folded) {
            const std::string x = name(a.second);
            fsum = fsum.empty() ? (a.first < 0 ? "-" + x : x) : fsum + (a.first < 0 ? " - " : " + ") + x;
        }
        e << "        " << G << " = " << fsum << ";\n    }\n";
        std::string sum;
        for (auto& a : g.rest) {
            const std::string x = name(a.second);
            sum = sum.empty() ? (a.first < 0 ? "-" + x : x) : sum + (a.first < 0 ? " - " : " + ") + x;
        }
        e << "    out[" << out_field << "] = " << (sum.empty() ? G : "(" + sum + ") + " + G) << ";\n";
    };
    for (int pc = 0; pc < n; ++pc) {
        const mol_instr& in = s.ins[pc];
        if (in.op == MOL_OP_OUT) {
            auto it = cgroup_at.find(pc);
            if (it != cgroup_at.end()) emit_cgroup(it->second, in.imm);
            else e << "    out[" << in.imm << "] = " << name(s.ia[pc]) << ";\n";
            continue;
        }
        if (uni[pc] || absorbed[pc] || cabs[pc]) continue;
        if (!root[pc]) {
            e << "    " << stmt(pc) << "\n";
            continue;
        }
        // fused root
        std::string cond;
        for (auto& kv : lin[pc].coef) {
            const mol_term& tm = d->terms[kv.first];
            const std::string F = std::to_string(tm.field);
            std::string c1 = "fast_line(P, P.ops[" + std::to_string(tm.op) + "], " + F + ", " + std::to_string(tm.dim) +
                             ", I[" + std::to_string(tm.dim) + "])";
            if (tm.kind == MOL_TERM_MIXED)
                c1 += " && fast_line(P, P.ops[" + std::to_string(tm.op2) + "], " + F + ", " + std::to_string(tm.dim2) +
                      ", I[" + std::to_string(tm.dim2) + "])";
            cond = cond.empty() ? c1 : cond + " && " + c1;
        }
        e << "    T " << v(pc) << ";\n    if (" << cond << ") {\n"
          << "        const T* __restrict__ b = u + (long long)" << lin[pc].field << " * P.ncell + c;\n"
          << "        const long long s1 = gstride(P, 1), s2 = gstride(P, 2);\n";
        const std::vector<Tap>& T = taps[pc];
        for (size_t i = 0; i < T.size(); ++i) {
            const std::string off = "(long long)(" + std::to_string(T[i].o[0]) + ") + (long long)(" +
                                    std::to_string(T[i].o[1]) + ") * s1 + (long long)(" + std::to_string(T[i].o[2]) +
                                    ") * s2";
            if (i == 0) e << "        T acc = U.fw" << pc << "_" << i << " * b[" << off << "];\n";
            else e << "        acc = fma(U.fw" << pc << "_" << i << ", b[" << off << "], acc);\n";
        }
        if (T.empty()) e << "        T acc = T(0);\n";
        e << "        " << v(pc) << " = acc;\n    } else {\n";
        std::vector<int> mem = lin[pc].members;
        std::sort(mem.begin(), mem.end());
        for (int m : mem)
            if (m != pc) e << "        " << stmt(m) << "\n";
        std::string st = stmt(pc);
        // turn "const T vX = expr;" into "vX = expr;"
        const std::string head = "const T " + v(pc) + " = ";
        if (st.compare(0, head.size(), head) == 0) st = v(pc) + " = " + st.substr(head.size());
        e << "        " << st << "\n    }\n";
    }
    e << "}\n";
}

// The coefficient arrays of the variable groups at cell c (k_coef_t, once per plan): per tap
// with an array, its uniform constant part plus, for every variable part, coef * a(face) with
// a the term's face program at the outer stencil's half point.
static void emit_coef(Emitter& e, const mol_problem_desc* d, const std::vector<FoldGroup>& groups) {
    e << "template <class T>\n__device__ __forceinline__ void gen_coef(const DevProb<T>& P, long long c, const int* I, "
         "T* out) {\n";
    std::set<std::pair<int, int>> faces;   // (term, outer face)
    for (const FoldGroup& g : groups)
        for (const FoldTap& t : g.taps)
            if (t.arr >= 0)
                for (const FoldPart& p : t.parts)
                    if (p.face >= 0) faces.insert({p.term, p.face});
    for (auto& fk : faces) {
        const int k = fk.first, m = fk.second;
        const mol_term& tm = d->terms[k];
        const int r = d->ops[tm.op].omin + m - 1;
        const std::string tag = "c" + std::to_string(k) + "_" + std::to_string(m) + "_";
        const std::string D = std::to_string(tm.dim);
        e << "    T " << tag << "a;\n    {\n";
        if (tm.prog < 0) {
            e << "    " << tag << "a = T(1);\n";
        } else {
            const SSA fs = to_ssa(d, tm.prog);
            std::set<int> used_aux;
            for (auto& in : fs.ins)
                if (in.op == MOL_OP_AUX) used_aux.insert(in.imm);
            for (int j : used_aux)
                e << "    const T " << tag << "fa" << j << " = P.aux[P.aux_off[P.terms[" << k << "].aux0 + " << j
                  << "] + face_index(P, " << D << ", I[" << D << "] + (" << r << "), I)];\n";
            FaceLeaves L(tag);
            std::vector<std::pair<int, int>> outs;
            emit_forward(e, d, fs, L, tag, &outs, false);
            e << "    " << tag << "a = " << (outs.empty() ? "T(1)" : tag + v(outs[0].second)) << ";\n";
        }
        e << "    }\n";
    }
    for (const FoldGroup& g : groups) {
        if (!g.variable) continue;
        e << "    {\n    const T* __restrict__ fw = P.w + P.terms[" << g.key_term << "].reserved2;\n";
        for (size_t i = 0; i < g.taps.size(); ++i) {
            const FoldTap& t = g.taps[i];
            if (t.arr < 0) continue;
            std::string ex = "fw[" + std::to_string(i) + "]";
            for (const FoldPart& p : t.parts)
                if (p.face >= 0)
                    ex += " + " + lit(p.coef) + " * c" + std::to_string(p.term) + "_" + std::to_string(p.face) + "_a";
            e << "    out[" << (g.arr0 + t.arr) << "] = " << ex << ";\n";
        }
        e << "    }\n";
    }
    e << "}\n";
}

// Vector-Jacobian product of a coefficient-stencil group where its stencil applies: the
// output's seed g times each tap's weight scattered to the tap (the difference form's taps
// also take it off the cell itself), and for each variable member's face the derivative of the
// output with respect to its coefficient a, g * sum(coef * u[tap]), through the face program
// into the aux arrays it reads.
static void emit_group_vjp(Emitter& e, const mol_problem_desc* d, const FoldGroup& g, int gi, int out_field) {
    const std::string F = std::to_string(g.field);
    e << "    if (cgv" << gi << ") {\n"
      << "        const T g = seed[" << out_field << "];\n"
      << "        const T* __restrict__ fw = P.w + P.terms[" << g.key_term << "].reserved2;\n"
      << "        const T* __restrict__ cw = P.cw + (long long)" << g.arr0 << " * P.ncell + c;\n"
      << "        const T* __restrict__ fb = u + (long long)" << F << " * P.ncell + c;\n"
      << "        T* lb = lam_u + (long long)" << F << " * P.ncell + c;\n";
    const std::vector<double> fwv = fold_weights(d, g);
    for (size_t i = 0; i < g.taps.size(); ++i) {
        const FoldTap& t = g.taps[i];
        if (t.arr < 0 && fwv[i] == 0.0) continue;
        const std::string wv = t.arr >= 0 ? (t.arr == 0 ? std::string("cw[0]")
                                                        : "cw[(long long)" + std::to_string(t.arr) + " * P.ncell]")
                                          : "fw[" + std::to_string(i) + "]";
        const std::string off = group_tap_off(d, g, t);
        e << "        {\n        const T gw = g * " << wv << ";\n";
        if (off == "0") {
            e << "        own" << F << " += gw;\n";
        } else {
            e << "        atomicAdd(lb + " << off << ", gw);\n";
            if (t.diff) e << "        own" << F << " -= gw;\n";
        }
        e << "        }\n";
    }
    std::map<std::pair<int, int>, std::vector<std::pair<const FoldTap*, double>>> faces;
    for (const FoldTap& t : g.taps)
        for (const FoldPart& p : t.parts)
            if (p.face >= 0) faces[{p.term, p.face}].push_back({&t, p.coef});
    if (!faces.empty()) e << "        if (lam_aux) {\n";
    // a face whose two parts are c (u[a] - u[b]) with c > 0 (the folded nonlinear Laplacian's
    // faces): g * c is computed once for every face with that c
    auto paired = [&](const std::vector<std::pair<const FoldTap*, double>>& pr) {
        return pr.size() == 2 && pr[0].second == -pr[1].second && pr[0].second != 0.0;
    };
    std::map<double, std::string> scales;
    for (auto& fk : faces) {
        if (d->terms[fk.first.first].prog < 0 || !paired(fk.second)) continue;
        const double c = std::fabs(fk.second[0].second);
        if (scales.count(c)) continue;
        const std::string nm = "gs" + std::to_string(scales.size());
        e << "        const T " << nm << " = g * " << lit(c) << ";\n";
        scales[c] = nm;
    }
    for (auto& fk : faces) {
        const int k = fk.first.first, m = fk.first.second;
        const mol_term& tm = d->terms[k];
        if (tm.prog < 0) continue;   // a = 1: no coefficient to differentiate
        const std::string D = std::to_string(tm.dim);
        const int r = d->ops[tm.op].omin + m - 1;
        const std::string tag = "va" + std::to_string(k) + "_" + std::to_string(m) + "_";
        e << "        {\n";
        const auto& pr = fk.second;
        if (paired(pr)) {
            const int ia = pr[0].second > 0 ? 0 : 1;
            e << "        const T " << tag << "ga = " << scales.at(std::fabs(pr[0].second)) << " * (fb["
              << group_tap_off(d, g, *pr[ia].first) << "] - fb[" << group_tap_off(d, g, *pr[1 - ia].first)
              << "]);\n";
        } else {
            e << "        T " << tag << "s = T(0);\n";
            for (auto& tc : pr)
                e << "        " << tag << "s = fma(" << lit(tc.second) << ", fb[" << group_tap_off(d, g, *tc.first)
                  << "], " << tag << "s);\n";
            e << "        const T " << tag << "ga = g * " << tag << "s;\n";
        }
        const SSA fs = to_ssa(d, tm.prog);
        std::set<int> used_aux;
        for (auto& in : fs.ins)
            if (in.op == MOL_OP_AUX) used_aux.insert(in.imm);
        for (int j : used_aux)
            e << "        const long long " << tag << "fi" << j << " = P.aux_off[P.terms[" << k << "].aux0 + " << j
              << "] + face_index(P, " << D << ", I[" << D << "] + (" << r << "), I);\n"
              << "        const T " << tag << "fa" << j << " = P.aux[" << tag << "fi" << j << "];\n"
              << "        T " << tag << "gfa" << j << " = T(0);\n";
        FaceLeaves L(tag);
        std::vector<std::pair<int, int>> outs;
        emit_forward(e, d, fs, L, tag, &outs, false);
        emit_reverse(e, fs, L, tag, [&](int) { return tag + "ga"; });
        for (int j : used_aux)
            e << "        atomicAdd(lam_aux + " << tag << "fi" << j << ", " << tag << "gfa" << j << ");\n";
        e << "        }\n";
    }
    if (!faces.empty()) e << "        }\n";
    e << "    }\n";
}

// True when some boundary program uses an elementary function, a power, a comparison or a
// select (the generated module then compiles those cases into run_bc_prog).
bool bc_full_ops(const mol_problem_desc* d) {
    for (int f = 0; f < d->nfields; ++f)
        for (int q = 0; q < d->ndim; ++q)
            for (int s = 0; s < 2; ++s) {
                const mol_bc& b = d->bc[f][q][s];
                if (b.prog < 0 || b.prog >= d->nprogs) continue;
                const int start = d->prog_ranges[2 * b.prog], len = d->prog_ranges[2 * b.prog + 1];
                for (int pc = start; pc < start + len; ++pc) {
                    const int op = d->code[pc].op;
                    if (op == MOL_OP_POWI || op == MOL_OP_POW || op == MOL_OP_FN || op == MOL_OP_CMP ||
                        op == MOL_OP_IFELSE)
                        return true;
                }
            }
    return false;
}

std::string generate_source(const mol_problem_desc* d, std::string& why) {
    Emitter e;
    e << "// generated by libmolgpu for one problem structure\n";
    if (bc_full_ops(d)) e << "#define MOL_BC_FULL_OPS 1\n";
    bool edge_rows = false, extrap_rows = false;
    for (int f = 0; f < d->nfields; ++f)
        for (int q = 0; q < d->ndim; ++q)
            for (int s = 0; s < 2; ++s) {
                edge_rows |= d->bc[f][q][s].kind == MOL_BC_EDGE;
                extrap_rows |= d->bc[f][q][s].extrap > 0;
            }
    if (edge_rows) e << "#define MOL_HAS_EDGE_ROWS 1\n";
    if (extrap_rows) e << "#define MOL_HAS_EXTRAP_ROWS 1\n";
    e << "#include \"mol_kernels.cuh\"\n"
      << "namespace mol {\n";
    int nface = 0;  // nonlinear-Laplacian terms: slots of the face pass
    for (int k = 0; k < d->nterms; ++k) {
        switch (d->terms[k].kind) {
            case MOL_TERM_LINEAR: emit_linear(e, d, k); break;
            case MOL_TERM_MIXED: emit_mixed(e, d, k); break;
            case MOL_TERM_WENO: emit_weno(e, d, k); break;
            case MOL_TERM_NONLINLAP: emit_nonlinlap(e, d, k, nface++); break;
            default: why = "unknown term"; return "";
        }
    }
    SSA cs = to_ssa(d, d->cell_prog);
    if (!cs.ok) {
        why = "program reads an undefined register";
        return "";
    }
    CellLeaves L;
    // one out-of-line copy of the cell per precision, shared by every kernel template
    // (inlined into every kernel; MOL_JIT_INLINE_CELL=0 keeps one out-of-line copy instead)
    const char* inl = getenv("MOL_JIT_INLINE_CELL");
    const std::string cell_attr = (inl && inl[0] == '0') ? "__noinline__" : "__forceinline__";
    emit_cell_fused(e, d, cs, cell_attr);
    const std::vector<FoldGroup> coef_groups = const_linear_groups(d);
    const int ncoef = fold_coef_arrays(coef_groups);
    emit_coef(e, d, coef_groups);
    // The cell VJP.  With coefficient stencils it is two functions: the group path (the members'
    // adjoints scattered by the groups, emit_group_vjp) inline, for warps where every group's
    // stencil applies, and the full reverse sweep out of line (__noinline__) for the others (the
    // boundary planes), so the rarely taken sweep does not set the register budget of the kernel.
    bool any_var = false;
    for (auto& g : coef_groups) any_var |= g.variable;
    const std::string vjp_sig = "(const DevProb<T>& P, const T* __restrict__ u, long long c, const int* I, T t, "
                                "const T* __restrict__ p, const T* seed, T* lam_u, T* lp, T* lam_aux)";
    auto vjp_body = [&](bool fast) {
        VjpCellLeaves VL;
        VL.d = d;
        VL.omit_members = fast;
        for (int f = 0; f < d->nfields; ++f) e << "    T own" << f << " = T(0);\n";
        if (fast)
            for (size_t gi = 0; gi < coef_groups.size(); ++gi) {
                const FoldGroup& g = coef_groups[gi];
                if (!g.variable) continue;
                for (const FoldTap& t : g.taps)
                    for (const FoldPart& pp : t.parts) VL.var_member[pp.term] = (int)gi;
            }
        {
            // WENO terms read by exactly one TERM instruction (and by no upwind select)
            std::vector<int> refs(d->nterms, 0);
            for (auto& in : cs.ins) {
                if (in.op == MOL_OP_TERM && in.imm >= 0 && in.imm < d->nterms) refs[in.imm] += 1;
                if (in.op == MOL_OP_UPWIND) {
                    if (in.b < d->nterms) refs[in.b] += 2;
                    if (in.c < d->nterms) refs[in.c] += 2;
                }
            }
            for (int k = 0; k < d->nterms; ++k)
                if (d->terms[k].kind == MOL_TERM_WENO && d->terms[k].variant == 0 && refs[k] == 1) {
                    VL.split.push_back(k);
                    e << "    bool fw" << k << " = false;\n    T gw" << k << "[5];\n";
                }
        }
        emit_forward(e, d, cs, VL, "", nullptr, true);
        emit_reverse(e, cs, VL, "", [&](int k) { return "seed[" + std::to_string(k) + "]"; });
        if (fast)
            for (size_t gi = 0; gi < coef_groups.size(); ++gi)
                if (coef_groups[gi].variable)
                    emit_group_vjp(e, d, coef_groups[gi], (int)gi, cs.ins[coef_groups[gi].out_pc].imm);
        for (int f = 0; f < d->nfields; ++f)
            e << "    atomicAdd(lam_u + (long long)" << f << " * P.ncell + c, own" << f << ");\n";
    };
    if (any_var) {
        e << "template <class T>\n__device__ __noinline__ void gen_cell_vjp_full" << vjp_sig << " {\n";
        vjp_body(false);
        e << "}\n";
    }
    e << "template <class T>\n__device__ __forceinline__ void gen_cell_vjp" << vjp_sig << " {\n";
    if (any_var) {
        std::string all;
        for (size_t gi = 0; gi < coef_groups.size(); ++gi) {
            const FoldGroup& g = coef_groups[gi];
            if (!g.variable) continue;
            e << "    const bool cgv" << gi << " = " << group_cond(d, g) << ";\n";
            all += (all.empty() ? "" : " && ") + std::string("cgv") + std::to_string(gi);
        }
        e << "    if (!(" << all << ")) {\n        gen_cell_vjp_full<T>(P, u, c, I, t, p, seed, lam_u, lp, lam_aux);\n"
          << "        return;\n    }\n";
    }
    vjp_body(any_var);
    e << "}\n";
    // the face pass: left faces of every nonlinear-Laplacian term, slot order = term order
    e << "template <class T>\n__device__ __forceinline__ void gen_faces(const DevProb<T>& P, const T* __restrict__ u, "
         "long long c, const int* I, T t, const T* __restrict__ p, T* out) {\n";
    {
        int q = 0;
        for (int k = 0; k < d->nterms; ++k)
            if (d->terms[k].kind == MOL_TERM_NONLINLAP)
                e << "    out[" << q++ << "] = gfl" << k << "<T>(P, u, c, I, t, p);\n";
    }
    e << "}\n";
    e << "struct GenCell {\n"
      << "static constexpr int kFields = " << d->nfields << ";\n"
      << "static constexpr int kFaceTerms = " << nface << ";\n"
      << "static constexpr int kCoefArrays = " << ncoef << ";\n"
      << "template <class T>\nstatic __device__ __forceinline__ void coefs(const DevProb<T>& P, long long c, const int* I, "
         "T* out) { gen_coef<T>(P, c, I, out); }\n"
      << "template <class T>\nstatic __device__ __forceinline__ void faces(const DevProb<T>& P, const T* __restrict__ u, "
         "long long c, const int* I, T t, const T* __restrict__ p, T* out) { gen_faces<T>(P, u, c, I, t, p, out); }\n"
         "template <class T> using Uniform = GenUniform<T>;\n"
         "template <class T>\nstatic __device__ __forceinline__ void uniform(const DevProb<T>& P, T t, const T* "
         "__restrict__ p, GenUniform<T>& U) { gen_uniform<T>(P, t, p, U); }\n"
         "template <class T>\nstatic __device__ __forceinline__ void cell(const DevProb<T>& P, const T* __restrict__ u, "
         "long long c, const int* I, T t, const T* __restrict__ p, const GenUniform<T>& U, T* out) { "
         "gen_cell<T>(P, u, c, I, t, p, U, out); }\n"
         "template <class T>\nstatic __device__ __forceinline__ void cell_vjp(const DevProb<T>& P, const T* __restrict__ "
         "u, long long c, const int* I, T t, const T* __restrict__ p, const T* seed, T* lam_u, T* lp, T* lam_aux) "
         "{ gen_cell_vjp<T>(P, u, c, I, t, p, seed, lam_u, lp, lam_aux); }\n};\n}  // namespace mol\n";
    return e.o.str();
}

// ---------------------------------------------------------------------------
// NVRTC (loaded at run time) and the runtime library API
// ---------------------------------------------------------------------------

namespace {

typedef int nvrtcResult_t;
typedef struct _nvrtcProgram* nvrtcProgram_t;
struct Nvrtc {
    bool ok = false;
    std::string err;
    nvrtcResult_t (*create)(nvrtcProgram_t*, const char*, const char*, int, const char* const*, const char* const*);
    nvrtcResult_t (*compile)(nvrtcProgram_t, int, const char* const*);
    nvrtcResult_t (*logsize)(nvrtcProgram_t, size_t*);
    nvrtcResult_t (*log)(nvrtcProgram_t, char*);
    nvrtcResult_t (*cubinsize)(nvrtcProgram_t, size_t*);
    nvrtcResult_t (*cubin)(nvrtcProgram_t, char*);
    nvrtcResult_t (*destroy)(nvrtcProgram_t*);
    nvrtcResult_t (*addname)(nvrtcProgram_t, const char*);
    nvrtcResult_t (*lowered)(nvrtcProgram_t, const char*, const char**);
};

Nvrtc& nvrtc() {
    static Nvrtc N;
    static std::once_flag once;
    std::call_once(once, [] {
        const char* names[] = {"libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so.13",
                               "/usr/local/cuda/lib64/libnvrtc.so"};
        void* h = nullptr;
        for (const char* n : names)
            if ((h = dlopen(n, RTLD_NOW | RTLD_LOCAL))) break;
        if (!h) {
            N.err = "libnvrtc not found";
            return;
        }
        auto sym = [&](const char* s) { return dlsym(h, s); };
        N.create = (decltype(N.create))sym("nvrtcCreateProgram");
        N.compile = (decltype(N.compile))sym("nvrtcCompileProgram");
        N.logsize = (decltype(N.logsize))sym("nvrtcGetProgramLogSize");
        N.log = (decltype(N.log))sym("nvrtcGetProgramLog");
        N.cubinsize = (decltype(N.cubinsize))sym("nvrtcGetCUBINSize");
        N.cubin = (decltype(N.cubin))sym("nvrtcGetCUBIN");
        N.destroy = (decltype(N.destroy))sym("nvrtcDestroyProgram");
        N.addname = (decltype(N.addname))sym("nvrtcAddNameExpression");
        N.lowered = (decltype(N.lowered))sym("nvrtcGetLoweredName");
        N.ok = N.create && N.compile && N.logsize && N.log && N.cubinsize && N.cubin && N.destroy && N.addname &&
               N.lowered;
        if (!N.ok) N.err = "libnvrtc lacks required symbols";
    });
    return N;
}

struct CacheEntry {
    cudaLibrary_t lib = nullptr;
    std::vector<cudaKernel_t> kernels;
};
std::mutex g_cache_mu;
std::map<std::string, CacheEntry> g_cache;

}  // namespace

// NVRTC options.  MOL_JIT_MIN_BLOCKS sets the CTAs per SM the register allocator must allow
// for the right-hand-side kernels; MOL_JIT_MAXRREG caps registers per thread.
constexpr int kDefaultMinBlocks = 2;
// Resident CTAs per SM for the VJP of a module whose cell VJP has a coefficient-stencil path
// (the full reverse sweep out of line): its group path holds few values, and the 256^3 ADR VJP
// measured 1.708 / 1.374 / 1.364 ms at 2 / 3 / 4 CTAs per SM (long-scoreboard bound at 2).
constexpr int kCoefVjpMinBlocks = 3;
int vjp_min_blocks_of(const std::string& src) {
    return src.find("gen_cell_vjp_full") != std::string::npos ? kCoefVjpMinBlocks : 0;
}

// Resident CTAs per SM for the Float32-state group: its cells hold half-width values, its
// kernels are bound by memory latency rather than the FP64 pipe, and the 256^3 ADR FP32 step
// measured 1.028 / 0.828 / 0.675 / 0.728 ms at 3 / 4 / 6 / 8 CTAs per SM.
constexpr int kF32MinBlocks = 6;

std::vector<std::string> jit_options(int min_blocks, int vjp_min_blocks, int group) {
    std::vector<std::string> o = {"--gpu-architecture=sm_103a", "-std=c++17", "-lineinfo", "--fmad=true",
                                  "-default-device", "-DMOL_JIT=1"};
    const char* r = getenv("MOL_JIT_MAXRREG");
    if (r && atoi(r) > 0) o.push_back(std::string("--maxrregcount=") + std::to_string(atoi(r)));
    const char* mb = getenv("MOL_JIT_MIN_BLOCKS");
    const int minb = (mb && atoi(mb) > 0) ? atoi(mb)
                     : group == JIT_FWD32 ? kF32MinBlocks
                                         : (min_blocks > 0 ? min_blocks : kDefaultMinBlocks);
    o.push_back("-DMOL_MIN_BLOCKS=" + std::to_string(minb));
    // the face pass at three resident CTAs per SM more than the stage kernels: the 256^3 ADR
    // step measured 3.18 / 3.00 / 2.91 / 2.86 / 2.93 ms with the face kernel at 3 / 4 / 5 / 6 / 8
    // CTAs per SM (it spills some from 5 on, but needs the warps); MOL_FACE_MIN_BLOCKS overrides
    const char* fmb = getenv("MOL_FACE_MIN_BLOCKS");
    const int fminb = (fmb && atoi(fmb) > 0) ? atoi(fmb) : std::min(8, minb + 3);
    o.push_back("-DMOL_FACE_MIN_BLOCKS=" + std::to_string(fminb));
    // the VJP at no more than two resident CTAs (the face-form ADR cell VJP took 128 registers:
    // 44 bytes of spills instead of 2.2 KB at 80), or the coefficient-stencil budget above;
    // MOL_VJP_MIN_BLOCKS overrides
    const char* vmb = getenv("MOL_VJP_MIN_BLOCKS");
    const int vminb = (vmb && atoi(vmb) > 0) ? atoi(vmb) : (vjp_min_blocks > 0 ? vjp_min_blocks : std::min(minb, 2));
    o.push_back("-DMOL_VJP_MIN_BLOCKS=" + std::to_string(vminb));
    // MOL_BATCH_MIN_BLOCKS: the same bound for the ensemble kernels (default 1: no cap)
    const char* bmb = getenv("MOL_BATCH_MIN_BLOCKS");
    if (bmb && atoi(bmb) > 0) o.push_back("-DMOL_BATCH_MIN_BLOCKS=" + std::to_string(atoi(bmb)));
    // MOL_JIT_VERBOSE=1: ptxas resource report (registers, stack, spills) on stderr
    if (getenv("MOL_JIT_VERBOSE")) o.push_back("--ptxas-options=-v");
    // MOL_JIT_DEFINES="A B=1": extra preprocessor definitions for the generated modules
    if (const char* defs = getenv("MOL_JIT_DEFINES")) {
        std::string all(defs), tok;
        for (size_t i = 0; i <= all.size(); ++i) {
            if (i == all.size() || all[i] == ' ') {
                if (!tok.empty()) o.push_back("-D" + tok);
                tok.clear();
            } else {
                tok += all[i];
            }
        }
    }
    return o;
}

// Compiled modules are kept on disk (MOL_CACHE_DIR, else $HOME/.cache/molgpu) keyed by a
// hash of the generated source, the compile options and the kernel list.
std::string disk_cache_path(const std::string& src, int nparams, int min_blocks, int group) {
    const char* dir = getenv("MOL_CACHE_DIR");
    std::string base;
    if (dir && dir[0]) base = dir;
    else if (getenv("HOME")) base = std::string(getenv("HOME")) + "/.cache/molgpu";
    else return "";
    if (getenv("MOL_NO_DISK_CACHE")) return "";
    uint64_t h = 1469598103934665603ull;  // FNV-1a
    auto mix = [&](const std::string& x) {
        for (unsigned char ch : x) {
            h ^= ch;
            h *= 1099511628211ull;
        }
    };
    mix(src);
    for (auto& o : jit_options(min_blocks, vjp_min_blocks_of(src), group)) mix(o);
    mix("v4|" + std::to_string(nparams));
    for (int i = 0; i < (int)(sizeof(kEmbedTexts) / sizeof(kEmbedTexts[0])); ++i) mix(kEmbedTexts[i]);
    char name[64];
    std::snprintf(name, sizeof name, "/%016llx.molmod", (unsigned long long)h);
    return base + name;
}

bool disk_cache_load(const std::string& path, size_t nnames, std::vector<char>* cubin,
                     std::vector<std::string>* lowered) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    bool ok = true;
    uint64_t n = 0, sz = 0;
    ok = std::fread(&n, 8, 1, f) == 1 && n == nnames;
    lowered->clear();
    for (uint64_t i = 0; ok && i < n; ++i) {
        uint64_t l = 0;
        ok = std::fread(&l, 8, 1, f) == 1 && l < 4096;
        std::string s(l, '\0');
        if (ok && l) ok = std::fread(&s[0], 1, l, f) == l;
        lowered->push_back(s);
    }
    if (ok) ok = std::fread(&sz, 8, 1, f) == 1 && sz > 0 && sz < (1ull << 30);
    if (ok) {
        cubin->resize(sz);
        ok = std::fread(cubin->data(), 1, sz, f) == sz;
    }
    std::fclose(f);
    return ok;
}

void disk_cache_store(const std::string& path, const std::vector<char>& cubin, const std::vector<std::string>& lowered) {
    const std::string dir = path.substr(0, path.rfind('/'));
    std::string cmd_dir;
    // create the directory chain (no shell)
    for (size_t pos = 1; pos != std::string::npos && pos <= dir.size(); pos = dir.find('/', pos + 1)) {
        const std::string sub = dir.substr(0, pos == std::string::npos ? dir.size() : pos);
        mkdir(sub.c_str(), 0755);
        if (pos == std::string::npos) break;
    }
    mkdir(dir.c_str(), 0755);
    const std::string tmp = path + ".tmp" + std::to_string((long long)getpid());
    FILE* f = std::fopen(tmp.c_str(), "wb");
    if (!f) return;
    uint64_t n = lowered.size();
    bool ok = std::fwrite(&n, 8, 1, f) == 1;
    for (auto& s : lowered) {
        uint64_t l = s.size();
        ok = ok && std::fwrite(&l, 8, 1, f) == 1 && (l == 0 || std::fwrite(s.data(), 1, l, f) == l);
    }
    uint64_t sz = cubin.size();
    ok = ok && std::fwrite(&sz, 8, 1, f) == 1 && std::fwrite(cubin.data(), 1, sz, f) == sz;
    std::fclose(f);
    if (ok) std::rename(tmp.c_str(), path.c_str());
    else std::remove(tmp.c_str());
}

std::vector<std::string> jit_kernel_names(int nparams, int group) {
    const std::string NP = std::to_string(nparams > 0 ? nparams : 0);
    std::vector<std::string> n;
    switch (group) {
        case JIT_FWD64:
            n = {"&mol::k_rhs_t<double, mol::GenCell>", "&mol::k_ssprk_t<double, mol::GenCell, 1>",
                 "&mol::k_ssprk_t<double, mol::GenCell, 2>", "&mol::k_ssprk_t<double, mol::GenCell, 3>",
                 "&mol::k_tsit_stage_t<double, mol::GenCell>", "&mol::k_faces_t<double, mol::GenCell>",
                 "&mol::k_coef_t<mol::GenCell>", "&mol::k_tsit_small_t<double, mol::GenCell>"};
            break;
        case JIT_FWD32:
            n = {"&mol::k_rhs_t<float, mol::GenCell>", "&mol::k_ssprk_t<float, mol::GenCell, 1>",
                 "&mol::k_ssprk_t<float, mol::GenCell, 2>", "&mol::k_ssprk_t<float, mol::GenCell, 3>",
                 "&mol::k_faces_t<float, mol::GenCell>"};
            break;
        case JIT_BATCH:
            n = {"&mol::k_batch_ssprk_t<double, mol::GenCell>", "&mol::k_batch_ssprk_t<float, mol::GenCell>",
                 "&mol::k_batch_tiles_t<double, mol::GenCell>", "&mol::k_batch_tiles_t<float, mol::GenCell>"};
            break;
        case JIT_VJP:
            n = {"&mol::k_vjp_t<double, mol::GenCell, " + NP + ">"};
            break;
    }
    return n;
}

int nvrtc_compile(const std::string& src, int nparams, int group, std::vector<char>* cubin,
                  std::vector<std::string>* lowered, std::string& err, int min_blocks) {
    const std::vector<std::string> names = jit_kernel_names(nparams, group);
    Nvrtc& N = nvrtc();
    if (!N.ok) {
        err = "nvrtc: " + N.err;
        return MOL_ERR_UNSUPPORTED;
    }
    nvrtcProgram_t prog;
    const int nh = (int)(sizeof(kEmbedNames) / sizeof(kEmbedNames[0]));
    if (N.create(&prog, src.c_str(), "mol_generated.cu", nh, kEmbedTexts, kEmbedNames) != 0) {
        err = "nvrtcCreateProgram failed";
        return MOL_ERR_CUDA;
    }
    for (auto& n : names) N.addname(prog, n.c_str());
    std::vector<std::string> ostr = jit_options(min_blocks, vjp_min_blocks_of(src), group);
    std::vector<const char*> opts;
    for (auto& o : ostr) opts.push_back(o.c_str());
    const int rc = N.compile(prog, (int)opts.size(), opts.data());
    if (rc != 0) {
        size_t ls = 0;
        N.logsize(prog, &ls);
        std::string log(ls, '\0');
        if (ls) N.log(prog, &log[0]);
        N.destroy(&prog);
        err = "nvrtc compile failed: " + log.substr(0, 6000);
        return MOL_ERR_UNSUPPORTED;
    }
    if (getenv("MOL_JIT_VERBOSE")) {
        size_t ls = 0;
        N.logsize(prog, &ls);
        std::string log(ls, '\0');
        if (ls) N.log(prog, &log[0]);
        fprintf(stderr, "[molgpu jit group %d]\n%s\n", group, log.c_str());
    }
    size_t cs = 0;
    N.cubinsize(prog, &cs);
    if (cubin) {
        cubin->resize(cs);
        N.cubin(prog, cubin->data());
    }
    if (lowered) {
        lowered->clear();
        for (auto& n : names) {
            const char* l = nullptr;
            N.lowered(prog, n.c_str(), &l);
            lowered->push_back(l ? l : "");
        }
    }
    N.destroy(&prog);
    return MOL_OK;
}

int jit_load_group(const std::string& src, int nparams, int group, JitKernels* k, std::string& err) {
    const std::vector<std::string> names = jit_kernel_names(nparams, group);
    const std::string key = src + "\n//group " + std::to_string(group) + " minblocks " + std::to_string(k->min_blocks);
    std::vector<cudaKernel_t> got;
    {
        std::lock_guard<std::mutex> g(g_cache_mu);
        auto it = g_cache.find(key);
        if (it != g_cache.end()) got = it->second.kernels;
    }
    if (got.empty()) {
        std::vector<char> cubin;
        std::vector<std::string> lowered;
        const std::string cache_path = disk_cache_path(key, nparams, k->min_blocks, group);
        if (!(cache_path.size() && disk_cache_load(cache_path, names.size(), &cubin, &lowered))) {
            int st = nvrtc_compile(src, nparams, group, &cubin, &lowered, err, k->min_blocks);
            if (st) return st;
            if (cache_path.size()) disk_cache_store(cache_path, cubin, lowered);
        }
        cudaLibrary_t lib;
        cudaError_t ce = cudaLibraryLoadData(&lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
        if (ce != cudaSuccess) {
            err = std::string("cudaLibraryLoadData: ") + cudaGetErrorString(ce);
            cudaGetLastError();
            return MOL_ERR_CUDA;
        }
        for (size_t i = 0; i < names.size(); ++i) {
            cudaKernel_t kk;
            ce = cudaLibraryGetKernel(&kk, lib, lowered[i].c_str());
            if (ce != cudaSuccess) {
                err = "cudaLibraryGetKernel(" + names[i] + "): " + cudaGetErrorString(ce);
                cudaGetLastError();
                return MOL_ERR_CUDA;
            }
            got.push_back(kk);
        }
        std::lock_guard<std::mutex> g(g_cache_mu);
        g_cache[key] = CacheEntry{lib, got};
    }
    switch (group) {
        case JIT_FWD64:
            k->rhs64 = got[0];
            k->ssp64[0] = got[1];
            k->ssp64[1] = got[2];
            k->ssp64[2] = got[3];
            k->tsit64 = got[4];
            k->faces64 = got[5];
            k->coef64 = got[6];
            k->tsitsmall64 = got[7];
            break;
        case JIT_FWD32:
            k->rhs32 = got[0];
            k->ssp32[0] = got[1];
            k->ssp32[1] = got[2];
            k->ssp32[2] = got[3];
            k->faces32 = got[4];
            break;
        case JIT_BATCH:
            k->batch64 = got[0];
            k->batch32 = got[1];
            k->tiles64 = got[2];
            k->tiles32 = got[3];
            break;
        case JIT_VJP:
            k->vjp64 = got[0];
            break;
    }
    k->loaded |= 1u << group;
    return MOL_OK;
}

int jit_compile(const mol_problem_desc* d, JitKernels* out, std::string& err, std::string* src_out, int min_blocks) {
    std::string why;
    std::string src = generate_source(d, why);
    if (src.empty()) {
        err = "codegen: " + why;
        return MOL_ERR_UNSUPPORTED;
    }
    if (src_out) *src_out = src;
    JitKernels k;
    k.src = src;
    k.nparams = d->nparams;
    k.min_blocks = min_blocks;
    int st = jit_load_group(src, d->nparams, JIT_FWD64, &k, err);
    if (st) return st;
    k.ok = true;
    *out = k;
    return MOL_OK;
}

int jit_ensure(JitKernels* k, int group, std::string& err) {
    if (!k->ok) return MOL_ERR_UNSUPPORTED;
    if (k->loaded & (1u << group)) return MOL_OK;
    return jit_load_group(k->src, k->nparams, group, k, err);
}

}  // namespace mol
