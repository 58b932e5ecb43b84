// Parser and in-memory form of the lemma IR written by the front end
// (include/ivarp/sid_fe/compile.hpp). Host-only C++17; used by the engine
// and by the code generator's consumers.
//
// Layout of a lemma:
//  * nargs variables with compile-time bounds (fixed point, denominator 1e6);
//  * the split configuration (dynamic prefix, static suffix);
//  * constants with outward double / float roundings;
//  * a node DAG in topological order (children before parents); every node carries
//    its compile-time bounds, which select sign-specialised interval operations;
//  * the runtime bound table: bound k applies function node fn[k] to variable target[k];
//  * update lists (which bounds to re-run after a variable's lb / ub / both changed);
//  * constraints (predicate nodes) and per-variable constraint rows.
#pragma once

#include <cstdint>
#include <cstdlib>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace sid {

enum class NodeOp : std::uint8_t {
    Arg, Const, BoolConst, Neg, Add, Sub, Mul, Div, Sqrt, Pow, Acos, Asin, Min, Max, Ite,
    Lt, Le, Gt, Ge, Eq, Ne, OrSeq, AndSeq, Or, And, Not
};

inline bool node_is_pred(NodeOp o) {
    switch(o) {
        case NodeOp::BoolConst: case NodeOp::Lt: case NodeOp::Le: case NodeOp::Gt: case NodeOp::Ge:
        case NodeOp::Eq: case NodeOp::Ne: case NodeOp::OrSeq: case NodeOp::AndSeq: case NodeOp::Or:
        case NodeOp::And: case NodeOp::Not:
            return true;
        default:
            return false;
    }
}

constexpr std::int64_t kFxpMax = INT64_C(9223372036854775807);
constexpr std::int64_t kFxpMin = -kFxpMax;

struct IrConst {
    double dlo, dhi;
    float flo, fhi;
    bool undefined;
};

struct IrNode {
    NodeOp op;
    std::int64_t lb, ub;      // expression: fixed-point bounds; predicate: 0/1 (definitely, possibly)
    std::int64_t aux;         // Arg: index; Const: constant id; Pow: exponent
    std::vector<int> ch;
};

struct IrBound {
    int target;
    int dir;                  // 1 = leq, 2 = geq, 3 = both
    int fn;
    bool defined;             // the function has a finite compile-time bound, so it is never "undefined"
};

struct IrSplit {
    int arg;
    std::uint32_t initial, subdivisions;
    bool dynamic;
};

struct LemmaIR {
    std::string name;
    std::string numtype;      // "f64" / "f32"
    int nargs = 0;
    std::vector<std::string> arg_names;
    std::vector<std::int64_t> ct_lb, ct_ub;
    std::vector<IrSplit> splits;
    std::vector<IrConst> consts;
    std::vector<IrNode> nodes;
    std::vector<IrBound> bounds;
    std::vector<std::vector<int>> upd_lb, upd_ub, upd_both;
    std::vector<int> constraints;           // node id per constraint
    std::vector<std::vector<int>> rows;     // constraint indices per row
    std::uint64_t fingerprint = 0;          // FNV-1a of the IR text without the name line

    std::vector<IrSplit> dynamic_splits() const {
        std::vector<IrSplit> r;
        for(const auto& s : splits) if(s.dynamic) r.push_back(s);
        return r;
    }
    std::vector<IrSplit> static_splits() const {
        std::vector<IrSplit> r;
        for(const auto& s : splits) if(!s.dynamic) r.push_back(s);
        return r;
    }
};

inline NodeOp parse_op(const std::string& s) {
    static const char* names[] = {"arg", "const", "bconst", "neg", "add", "sub", "mul", "div", "sqrt", "pow",
                                  "acos", "asin", "min", "max", "ite", "lt", "le", "gt", "ge", "eq", "ne",
                                  "orseq", "andseq", "or", "and", "not"};
    for(int i = 0; i < int(sizeof(names) / sizeof(names[0])); ++i) {
        if(s == names[i]) return NodeOp(i);
    }
    throw std::invalid_argument("lemma IR: unknown node operation " + s);
}

inline std::string unescape_token(const std::string& s) {
    if(s == "%") return {};
    std::string r;
    for(std::size_t i = 0; i < s.size(); ++i) {
        if(s[i] == '%' && i + 2 < s.size()) {
            r += char(std::strtol(s.substr(i + 1, 2).c_str(), nullptr, 16));
            i += 2;
        } else {
            r += s[i];
        }
    }
    return r;
}

inline std::uint64_t ir_fingerprint(const std::string& text) {
    std::uint64_t h = 1469598103934665603ull;
    std::istringstream in(text);
    std::string line;
    while(std::getline(in, line)) {
        if(line.compare(0, 5, "name ") == 0) continue;
        for(unsigned char c : line) { h ^= c; h *= 1099511628211ull; }
        h ^= '\n';
        h *= 1099511628211ull;
    }
    return h;
}

inline LemmaIR parse_lemma_ir(const std::string& text) {
    LemmaIR L;
    std::istringstream in(text);
    std::string line;
    bool header = false, ended = false;
    auto fail = [](const std::string& what) { throw std::invalid_argument("lemma IR: " + what); };
    while(std::getline(in, line)) {
        if(line.empty()) continue;
        std::istringstream ls(line);
        std::string kw;
        ls >> kw;
        if(kw == "sidir") {
            int v = 0;
            ls >> v;
            if(v != 1) fail("unsupported version");
            header = true;
        } else if(kw == "name") {
            std::string t; ls >> t; L.name = unescape_token(t);
        } else if(kw == "numtype") {
            ls >> L.numtype;
        } else if(kw == "nargs") {
            ls >> L.nargs;
            if(L.nargs <= 0 || L.nargs > 32) fail("bad nargs");
            L.arg_names.resize(std::size_t(L.nargs));
            L.ct_lb.resize(std::size_t(L.nargs));
            L.ct_ub.resize(std::size_t(L.nargs));
            L.upd_lb.resize(std::size_t(L.nargs));
            L.upd_ub.resize(std::size_t(L.nargs));
            L.upd_both.resize(std::size_t(L.nargs));
            L.rows.resize(std::size_t(L.nargs));
        } else if(kw == "arg") {
            int i; std::string nm; std::int64_t lo, hi;
            ls >> i >> nm >> lo >> hi;
            if(i < 0 || i >= L.nargs) fail("bad arg index");
            L.arg_names[std::size_t(i)] = unescape_token(nm);
            L.ct_lb[std::size_t(i)] = lo;
            L.ct_ub[std::size_t(i)] = hi;
        } else if(kw == "split") {
            IrSplit s; int dyn;
            ls >> s.arg >> s.initial >> s.subdivisions >> dyn;
            s.dynamic = dyn != 0;
            L.splits.push_back(s);
        } else if(kw == "const") {
            int id; std::string a, b, c, d; int und;
            ls >> id >> a >> b >> c >> d >> und;
            if(id != int(L.consts.size())) fail("constants out of order");
            L.consts.push_back(IrConst{std::strtod(a.c_str(), nullptr), std::strtod(b.c_str(), nullptr),
                                       float(std::strtod(c.c_str(), nullptr)), float(std::strtod(d.c_str(), nullptr)),
                                       und != 0});
        } else if(kw == "node") {
            int id; std::string op; IrNode n; int nc;
            ls >> id >> op >> n.lb >> n.ub >> n.aux >> nc;
            if(id != int(L.nodes.size())) fail("nodes out of order");
            n.op = parse_op(op);
            for(int k = 0; k < nc; ++k) {
                int c; ls >> c;
                if(c < 0 || c >= id) fail("node child not defined before its parent");
                n.ch.push_back(c);
            }
            L.nodes.push_back(n);
        } else if(kw == "bound") {
            int id; IrBound b; std::string dir; int def;
            ls >> id >> b.target >> dir >> b.fn >> def;
            b.dir = dir == "leq" ? 1 : dir == "geq" ? 2 : dir == "both" ? 3 : 0;
            if(b.dir == 0) fail("bad bound direction");
            b.defined = def != 0;
            if(id != int(L.bounds.size())) fail("bounds out of order");
            L.bounds.push_back(b);
        } else if(kw == "update") {
            int a; std::string kind; int n;
            ls >> a >> kind >> n;
            std::vector<int> v(static_cast<std::size_t>(n));
            for(auto& x : v) ls >> x;
            if(kind == "lb") L.upd_lb.at(std::size_t(a)) = v;
            else if(kind == "ub") L.upd_ub.at(std::size_t(a)) = v;
            else if(kind == "both") L.upd_both.at(std::size_t(a)) = v;
            else fail("bad update kind");
        } else if(kw == "constraint") {
            int id, node; ls >> id >> node;
            if(id != int(L.constraints.size())) fail("constraints out of order");
            L.constraints.push_back(node);
        } else if(kw == "row") {
            int r, n; ls >> r >> n;
            std::vector<int> v(static_cast<std::size_t>(n));
            for(auto& x : v) ls >> x;
            L.rows.at(std::size_t(r)) = v;
        } else if(kw == "end") {
            ended = true;
            break;
        } else {
            fail("unknown line: " + line);
        }
        if(ls.fail()) fail("malformed line: " + line);
    }
    if(!header || !ended) fail("missing header or end");
    if(int(L.splits.size()) != L.nargs) fail("split count does not match nargs");
    for(const auto& b : L.bounds) {
        if(b.target < 0 || b.target >= L.nargs || b.fn < 0 || b.fn >= int(L.nodes.size())) fail("bad bound");
    }
    for(int c : L.constraints) if(c < 0 || c >= int(L.nodes.size())) fail("bad constraint node");
    for(const auto& n : L.nodes) {
        if(n.op == NodeOp::Const && (n.aux < 0 || n.aux >= std::int64_t(L.consts.size()))) fail("bad const id");
        if(n.op == NodeOp::Arg && (n.aux < 0 || n.aux >= L.nargs)) fail("bad arg id");
    }
    L.fingerprint = ir_fingerprint(text);
    return L;
}

} // namespace sid
