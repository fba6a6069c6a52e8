// Seeded synthetic Pareas programs as flattened post-order AST arrays (ptl_synth.h).
//
// Build with -ffp-contract=off: the lognormal sizes use only IEEE-exact operations so
// that a seed names the same program on every host.
#include "ptl_synth.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {

// Pareas NodeType (subprojects/pareas-ast/include/codegen/astnode.hpp:11-56)
enum : uint8_t {
    N_INVALID = 0, N_STATEMENT_LIST, N_EMPTY_STAT, N_FUNC_DECL, N_FUNC_ARG, N_FUNC_ARG_LIST,
    N_EXPR_STAT, N_IF_STAT, N_IF_ELSE_STAT, N_WHILE_STAT, N_FUNC_CALL_EXPR, N_FUNC_CALL_ARG,
    N_FUNC_CALL_ARG_LIST, N_ADD, N_SUB, N_MUL, N_DIV, N_MOD, N_BITAND, N_BITOR, N_BITXOR,
    N_LSHIFT, N_RSHIFT, N_URSHIFT, N_LAND, N_LOR, N_EQ, N_NEQ, N_LESS, N_GREAT, N_LESSEQ,
    N_GREATEQ, N_BITNOT, N_LNOT, N_NEG, N_LIT, N_CAST, N_DEREF, N_ASSIGN, N_DECL, N_ID,
    N_WHILE_DUMMY, N_FUNC_DECL_DUMMY, N_RETURN,
};
// Pareas DataType (datatype.hpp:7-14)
enum : uint8_t { D_INVALID = 0, D_VOID, D_INT, D_FLOAT, D_INT_REF, D_FLOAT_REF };

// splitmix64 stream
struct Rng {
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    uint32_t u32() { return static_cast<uint32_t>(next() >> 32); }
    // uniform in [0, 1) with 53 bits
    double unit() { return static_cast<double>(next() >> 11) * (1.0 / 9007199254740992.0); }
    uint32_t below(uint32_t n) { return n ? static_cast<uint32_t>((static_cast<uint64_t>(u32()) * n) >> 32) : 0; }
    bool chance(double p) { return unit() < p; }
};

// exp() from +, -, *, / only: x = k ln2 + r, |r| <= ln2/2, Taylor series of e^r.
double exact_exp(double x) {
    const double ln2 = 0.6931471805599453;
    if (x > 700) x = 700;
    if (x < -700) x = -700;
    double kf = x / ln2;
    long k = static_cast<long>(kf < 0 ? kf - 0.5 : kf + 0.5);
    double r = x - static_cast<double>(k) * ln2;
    double term = 1.0, sum = 1.0;
    for (int i = 1; i < 20; ++i) {
        term = term * r / static_cast<double>(i);
        sum = sum + term;
    }
    double p = 1.0;
    if (k > 0) { for (long i = 0; i < k; ++i) p = p * 2.0; }
    else { for (long i = 0; i < -k; ++i) p = p * 0.5; }
    return sum * p;
}

// Standard normal by the Irwin-Hall sum of 12 uniforms (exact additions only).
double normal(Rng& r) {
    double s = 0;
    for (int i = 0; i < 12; ++i) s = s + r.unit();
    return s - 6.0;
}

struct Var {
    uint32_t id;
    uint8_t ref;  // D_INT_REF or D_FLOAT_REF
};

class Synth {
public:
    explicit Synth(const ptl_synth_params& p) : P(p) { rng.s = p.seed; }

    void run() {
        const uint32_t F = P.n_functions ? P.n_functions : 1;
        // Function signatures first: a call may name any function declared so far.
        fn_ret.reserve(F);
        std::vector<int32_t> decls;
        decls.reserve(F);
        for (uint32_t f = 0; f < F; ++f) {
            double z = normal(rng);
            double size = P.median_fn_nodes * (P.sigma > 0 ? exact_exp(P.sigma * z) : 1.0);
            if (size < P.min_fn_nodes) size = P.min_fn_nodes;
            if (P.max_fn_nodes && size > P.max_fn_nodes) size = P.max_fn_nodes;
            const uint32_t r = rng.below(3);
            const uint8_t ret = r == 0 ? D_INT : (r == 1 ? D_FLOAT : D_VOID);
            fn_ret.push_back(ret);
            decls.push_back(function(f, ret, static_cast<int64_t>(size), rng.chance(P.spill_frac)));
        }
        const int32_t root = node(N_STATEMENT_LIST, D_INVALID, 0, decls);
        parent[root] = -1;
        child_idx[root] = -1;
    }

    const ptl_synth_params P;
    Rng rng;
    std::vector<uint8_t> type, rtype;
    std::vector<int32_t> parent, child_idx;
    std::vector<uint32_t> data;
    std::string src;

private:
    std::vector<uint8_t> fn_ret;
    std::vector<std::vector<Var>> scopes;
    uint32_t next_sym = 0;
    uint32_t cur_fn = 0;
    uint8_t cur_ret = D_VOID;
    int64_t budget = 0;

    bool text() const { return P.emit_source != 0; }
    void put(const char* s) { if (text()) src += s; }
    void put(const std::string& s) { if (text()) src += s; }

    int32_t node(uint8_t t, uint8_t rt, uint32_t d, const std::vector<int32_t>& kids) {
        const int32_t idx = static_cast<int32_t>(type.size());
        type.push_back(t);
        rtype.push_back(rt);
        data.push_back(d);
        parent.push_back(-1);
        child_idx.push_back(-1);
        for (size_t j = 0; j < kids.size(); ++j) {
            parent[kids[j]] = idx;
            child_idx[kids[j]] = static_cast<int32_t>(j);
        }
        --budget;
        return idx;
    }
    int32_t leaf(uint8_t t, uint8_t rt, uint32_t d) { return node(t, rt, d, {}); }

    uint32_t declare(uint8_t ref) {
        const uint32_t id = next_sym++;
        scopes.back().push_back({id, ref});
        return id;
    }

    const Var* pick_var(uint8_t ref) {
        // Uniform over visible variables of the type, scanning from a random scope.
        size_t total = 0;
        for (const auto& s : scopes) for (const auto& v : s) total += v.ref == ref;
        if (!total) return nullptr;
        size_t k = rng.below(static_cast<uint32_t>(total));
        for (const auto& s : scopes) for (const auto& v : s) {
            if (v.ref != ref) continue;
            if (k-- == 0) return &v;
        }
        return nullptr;
    }

    static std::string vname(uint32_t id) { return "v" + std::to_string(id); }
    static std::string fname(uint32_t id) { return "f" + std::to_string(id); }

    // ---------------------------------------------------------------- expressions
    struct Val { int32_t idx; uint8_t t; };

    Val literal(uint8_t t) {
        if (t == D_INT) {
            const uint32_t v = rng.u32();
            if (v < 0x80000000u) {
                put(std::to_string(v));
                return {leaf(N_LIT, D_INT, v), D_INT};
            }
            const uint32_t mag = 0u - v;  // in (0, 2^31]
            put("(-(" + std::to_string(mag) + "))");
            const int32_t l = leaf(N_LIT, D_INT, mag);
            return {node(N_NEG, D_INT, 0, {l}), D_INT};
        }
        const float f = static_cast<float>(rng.u32() >> 8) * (1000.0f / 16777216.0f);
        uint32_t bits;
        std::memcpy(&bits, &f, 4);
        const bool neg = rng.chance(0.5);
        if (text()) {
            char buf[96];
            std::snprintf(buf, sizeof buf, "%.40f", static_cast<double>(f));
            put(neg ? std::string("(-(") + buf + "))" : std::string(buf));
        }
        const int32_t l = leaf(N_LIT, D_FLOAT, bits);
        if (!neg) return {l, D_FLOAT};
        return {node(N_NEG, D_FLOAT, 0, {l}), D_FLOAT};
    }

    Val variable(const Var& v) {
        put(vname(v.id));
        const int32_t id = leaf(N_ID, v.ref, v.id);
        const uint8_t val = v.ref == D_INT_REF ? D_INT : D_FLOAT;
        return {node(N_DEREF, val, 0, {id}), val};
    }

    // A call: FUNC_CALL_EXPR{FUNC_CALL_ARG_LIST{FUNC_CALL_ARG{value}...}}
    int32_t call(uint32_t callee, int arg_depth) {
        put(fname(callee) + "(");
        const uint32_t nargs = rng.below(7);
        std::vector<int32_t> args;
        uint32_t n_int = 0;
        for (uint32_t i = 0; i < nargs; ++i) {
            if (i) put(", ");
            const uint8_t t = rng.chance(P.float_frac) ? D_FLOAT : D_INT;
            Val v = value(t, arg_depth);
            const uint32_t arg_idx = t == D_INT ? n_int++ : i - n_int;
            args.push_back(node(N_FUNC_CALL_ARG, t, arg_idx, {v.idx}));
        }
        put(")");
        const int32_t list = node(N_FUNC_CALL_ARG_LIST, D_INVALID, 0, args);
        return node(N_FUNC_CALL_EXPR, fn_ret[callee], callee, {list});
    }

    Val leaf_value(uint8_t t) {
        const uint8_t ref = t == D_INT ? D_INT_REF : D_FLOAT_REF;
        const double r = rng.unit();
        if (r < 0.45) {
            if (const Var* v = pick_var(ref)) return variable(*v);
        } else if (r < 0.50 && budget > 40) {
            // a call to an already declared function returning t
            const uint32_t start = rng.below(cur_fn + 1);
            for (uint32_t k = 0; k <= cur_fn; ++k) {
                const uint32_t f = (start + k) % (cur_fn + 1);
                if (fn_ret[f] == t) return {call(f, 1), t};
            }
        }
        return literal(t);
    }

    Val binary(uint8_t nt, uint8_t rt, uint8_t ct, const char* op, int depth) {
        put("(");
        Val a = value(ct, depth - 1);
        put(" ");
        put(op);
        put(" ");
        Val b = value(ct, depth - 1);
        put(")");
        return {node(nt, rt, 0, {a.idx, b.idx}), rt};
    }

    Val unary(uint8_t nt, uint8_t t, const char* op, int depth) {
        put("(");
        put(op);
        put("(");
        Val a = value(t, depth - 1);
        put("))");
        return {node(nt, t, 0, {a.idx}), t};
    }

    Val cast(uint8_t to, int depth) {
        const uint8_t from = to == D_INT ? D_FLOAT : D_INT;
        put("(");
        Val a = value(from, depth - 1);
        put(to == D_INT ? ")@int" : ")@float");
        return {node(N_CAST, to, 0, {a.idx}), to};
    }

    Val value(uint8_t t, int depth) {
        if (depth <= 1 || budget <= 0 || rng.chance(0.32)) return leaf_value(t);
        if (t == D_FLOAT) {
            static const struct { uint8_t nt; const char* op; } fops[] = {
                {N_ADD, "+"}, {N_SUB, "-"}, {N_MUL, "*"}, {N_DIV, "/"}};
            const double r = rng.unit();
            if (r < 0.80) {
                const auto& o = fops[rng.below(4)];
                return binary(o.nt, D_FLOAT, D_FLOAT, o.op, depth);
            }
            if (r < 0.90) return unary(N_NEG, D_FLOAT, "-", depth);
            return cast(D_FLOAT, depth);
        }
        static const struct { uint8_t nt; const char* op; } iops[] = {
            {N_ADD, "+"}, {N_SUB, "-"}, {N_MUL, "*"}, {N_DIV, "/"}, {N_MOD, "%"},
            {N_BITAND, "&"}, {N_BITOR, "|"}, {N_BITXOR, "^"}, {N_LSHIFT, "<<"},
            {N_RSHIFT, ">>"}, {N_URSHIFT, ">>>"}};
        static const struct { uint8_t nt; const char* op; } cops[] = {
            {N_EQ, "=="}, {N_NEQ, "!="}, {N_LESS, "<"}, {N_GREAT, ">"}, {N_LESSEQ, "<="},
            {N_GREATEQ, ">="}};
        const double r = rng.unit();
        if (r < 0.55) {
            const auto& o = iops[rng.below(11)];
            return binary(o.nt, D_INT, D_INT, o.op, depth);
        }
        if (r < 0.75) {
            const auto& o = cops[rng.below(6)];
            const uint8_t ct = rng.chance(P.float_frac) ? D_FLOAT : D_INT;
            return binary(o.nt, D_INT, ct, o.op, depth);
        }
        if (r < 0.85) return rng.chance(0.5) ? binary(N_LAND, D_INT, D_INT, "&&", depth)
                                             : binary(N_LOR, D_INT, D_INT, "||", depth);
        if (r < 0.95) {
            const uint32_t u = rng.below(3);
            if (u == 0) return unary(N_NEG, D_INT, "-", depth);
            if (u == 1) return unary(N_LNOT, D_INT, "!", depth);
            return unary(N_BITNOT, D_INT, "~", depth);
        }
        return cast(D_INT, depth);
    }

    uint8_t pick_type() { return rng.chance(P.float_frac) ? D_FLOAT : D_INT; }

    // A right-nested chain a + (b + (c + ...)): every left operand stays live until
    // the innermost sum is formed.
    Val chain(uint8_t t, int len) {
        if (len <= 1) return leaf_value(t);
        put("(");
        Val a = leaf_value(t);
        put(" + ");
        Val b = chain(t, len - 1);
        put(")");
        return {node(N_ADD, t, 0, {a.idx, b.idx}), t};
    }

    // ---------------------------------------------------------------- statements
    void indent(int level) { if (text()) src.append(static_cast<size_t>(level) * 2 + 2, ' '); }

    int32_t assign(int level, bool spill) {
        indent(level);
        const uint8_t t = spill ? static_cast<uint8_t>(D_INT) : pick_type();
        const uint8_t ref = t == D_INT ? D_INT_REF : D_FLOAT_REF;
        const Var* existing = (!spill && rng.chance(0.5)) ? pick_var(ref) : nullptr;
        int32_t lhs;
        bool fresh = false;
        Var nv{};
        if (existing) {
            put(vname(existing->id));
            lhs = leaf(N_ID, existing->ref, existing->id);
        } else {
            nv = {next_sym++, ref};
            fresh = true;
            put(vname(nv.id) + (t == D_INT ? ": int" : ": float"));
            lhs = leaf(N_DECL, ref, nv.id);
        }
        put(" = ");
        Val v = spill ? chain(t, 40) : value(t, static_cast<int>(P.max_expr_depth));
        put(";\n");
        if (fresh) scopes.back().push_back(nv);
        const int32_t a = node(N_ASSIGN, t, 0, {lhs, v.idx});
        return node(N_EXPR_STAT, D_INVALID, 0, {a});
    }

    int32_t cond() {
        put("(");
        Val c = value(D_INT, static_cast<int>(P.max_expr_depth));
        put(")");
        return c.idx;
    }

    int32_t block(int level, int64_t quota) {
        put("{\n");
        scopes.emplace_back();
        std::vector<int32_t> stmts;
        const int64_t stop = budget - quota;
        do {
            stmts.push_back(statement(level + 1));
        } while (budget > stop && budget > 0);
        scopes.pop_back();
        indent(level);
        put("}");
        return node(N_STATEMENT_LIST, D_INVALID, 0, stmts);
    }

    int64_t nested_quota() {
        const int64_t q = static_cast<int64_t>(static_cast<double>(budget) * (0.05 + 0.3 * rng.unit()));
        return q < 8 ? 8 : q;
    }

    int32_t statement(int level) {
        double r = rng.unit();
        const bool can_nest = level < static_cast<int>(P.max_nesting) && budget > 30;
        if (!can_nest && r >= 0.40 && r < 0.80) r = 0.0;  // nesting exhausted: assign
        if (r < 0.40) return assign(level, false);
        if (r < 0.60) {
            indent(level);
            put("if ");
            const int32_t c = cond();
            put(" ");
            const int32_t b = block(level, nested_quota());
            put("\n");
            return node(N_IF_STAT, D_VOID, 0, {c, b});
        }
        if (r < 0.70) {
            indent(level);
            put("if ");
            const int32_t c = cond();
            put(" ");
            const int32_t b1 = block(level, nested_quota());
            put(" else ");
            const int32_t b2 = block(level, nested_quota());
            put("\n");
            return node(N_IF_ELSE_STAT, D_VOID, 0, {c, b1, b2});
        }
        if (r < 0.80) {
            indent(level);
            put("while ");
            const int32_t dummy = leaf(N_WHILE_DUMMY, D_INVALID, 0);
            const int32_t c = cond();
            put(" ");
            const int32_t b = block(level, nested_quota());
            put("\n");
            return node(N_WHILE_STAT, D_VOID, 0, {dummy, c, b});
        }
        if (r < 0.90) {
            indent(level);
            const int32_t c = call(rng.below(cur_fn + 1), 2);
            put(";\n");
            return node(N_EXPR_STAT, D_INVALID, 0, {c});
        }
        indent(level);
        if (cur_ret == D_VOID) {
            put("return;\n");
            return node(N_RETURN, D_VOID, cur_fn, {});
        }
        put("return ");
        Val v = value(cur_ret, static_cast<int>(P.max_expr_depth));
        put(";\n");
        return node(N_RETURN, v.t, cur_fn, {v.idx});
    }

    int32_t function(uint32_t f, uint8_t ret, int64_t size, bool spill) {
        cur_fn = f;
        cur_ret = ret;
        budget = size;
        scopes.clear();
        scopes.emplace_back();
        put("function " + fname(f) + "(");
        const int32_t dummy = leaf(N_FUNC_DECL_DUMMY, D_INVALID, 0);
        const uint32_t nargs = rng.below(7);
        std::vector<int32_t> args;
        uint32_t n_int = 0;
        for (uint32_t i = 0; i < nargs; ++i) {
            if (i) put(", ");
            const uint8_t ref = rng.chance(P.float_frac) ? D_FLOAT_REF : D_INT_REF;
            const uint32_t id = declare(ref);
            put(vname(id) + (ref == D_INT_REF ? ": int" : ": float"));
            const int32_t d = leaf(N_DECL, ref, id);
            const uint32_t arg_idx = ref == D_INT_REF ? n_int++ : i - n_int;
            args.push_back(node(N_FUNC_ARG, ref, arg_idx, {d}));
        }
        put(ret == D_INT ? "): int {\n" : (ret == D_FLOAT ? "): float {\n" : "): void {\n"));
        const int32_t arglist = node(N_FUNC_ARG_LIST, D_INVALID, 0, args);
        std::vector<int32_t> stmts;
        const int64_t spill_at = spill ? static_cast<int64_t>(rng.below(static_cast<uint32_t>(size > 1 ? size : 1))) : -1;
        bool spilled = false;
        do {
            if (spill && !spilled && budget <= size - spill_at) {
                stmts.push_back(assign(0, true));
                spilled = true;
            } else {
                stmts.push_back(statement(0));
            }
        } while (budget > 0);
        if (spill && !spilled) stmts.push_back(assign(0, true));
        put("}\n\n");
        const int32_t body = node(N_STATEMENT_LIST, D_INVALID, 0, stmts);
        return node(N_FUNC_DECL, ret, f, {dummy, arglist, body});
    }
};

template <typename T>
T* dup(const std::vector<T>& v) {
    T* p = static_cast<T*>(std::malloc(v.size() * sizeof(T) + 1));
    if (!v.empty()) std::memcpy(p, v.data(), v.size() * sizeof(T));
    return p;
}

}  // namespace

extern "C" void ptl_synth_default_params(ptl_synth_params* p) {
    p->seed = 0x50544C00ull;
    p->n_functions = 16;
    p->median_fn_nodes = 1250;
    p->sigma = 0;
    p->min_fn_nodes = 16;
    p->max_fn_nodes = 0;
    p->max_expr_depth = 6;
    p->float_frac = 0.30;
    p->max_nesting = 8;
    p->spill_frac = 0;
    p->emit_source = 0;
}

extern "C" int ptl_synth_generate(const ptl_synth_params* p, ptl_synth_program* out) {
    std::memset(out, 0, sizeof(*out));
    try {
        Synth s(*p);
        s.run();
        const size_t n = s.type.size();
        std::vector<int32_t> depth(n, 0);
        size_t max_depth = 0;
        for (size_t k = n; k-- > 0;) {
            const int32_t par = s.parent[k];
            depth[k] = par < 0 ? 0 : depth[static_cast<size_t>(par)] + 1;
            if (static_cast<size_t>(depth[k]) > max_depth) max_depth = static_cast<size_t>(depth[k]);
        }
        out->n = n;
        out->max_depth = max_depth;
        out->type = dup(s.type);
        out->rtype = dup(s.rtype);
        out->parent = dup(s.parent);
        out->depth = dup(depth);
        out->child_idx = dup(s.child_idx);
        out->data = dup(s.data);
        if (p->emit_source) {
            out->source = static_cast<char*>(std::malloc(s.src.size() + 1));
            std::memcpy(out->source, s.src.c_str(), s.src.size() + 1);
            out->source_len = s.src.size();
        }
        return 0;
    } catch (...) {
        return 1;
    }
}

extern "C" void ptl_synth_free(ptl_synth_program* prog) {
    std::free(prog->type);
    std::free(prog->rtype);
    std::free(prog->parent);
    std::free(prog->depth);
    std::free(prog->child_idx);
    std::free(prog->data);
    std::free(prog->source);
    std::memset(prog, 0, sizeof(*prog));
}
