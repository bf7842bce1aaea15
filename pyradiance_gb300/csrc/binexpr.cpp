/*
 * binexpr.cpp -- compiles rcontrib bin expressions into the device byte
 * code (gbcommon.h).
 *
 * The reference evaluates -b expressions with its interpreted calcomp
 * language (common/calexpr.c, common/caldefn.c) once per contributing ray
 * (rt/rcontrib.c:301-304).  Here the expression is parsed once on the host:
 * numbers, Dx/Dy/Dz, + - * /, unary minus, parentheses, if(a,b,c),
 * floor(x), PI, constants from -p settings and variables from -e
 * definitions (name=expr or name:expr), and the Reinhart sky bins of
 * util/reinhartb.cal (rbin, Nrbins; parameters MF, RHS, rNx..rNz, Ux..Uz).
 * Anything else is rejected with a message naming the construct.
 */
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "binexpr.h"

namespace {

struct Node {
    enum Kind { NUM, DX, DY, DZ, ADD, SUB, MUL, DIV, NEG, IF, FLOOR, RBIN } k;
    double v = 0;
    std::vector<std::shared_ptr<Node>> a;
};
using NP = std::shared_ptr<Node>;

NP num(double v) { auto n = std::make_shared<Node>(); n->k = Node::NUM; n->v = v; return n; }
NP op(Node::Kind k, std::vector<NP> a) { auto n = std::make_shared<Node>(); n->k = k; n->a = std::move(a); return n; }

struct Ctx {
    std::map<std::string, std::string> defs;   /* name -> expression text */
    bool reinhart = false;
    std::string err;
    int depth = 0;
};

struct Parser {
    Ctx &C;
    const char *s;
    explicit Parser(Ctx &c, const char *t) : C(c), s(t) {}
    void ws() { while (*s && isspace((unsigned char)*s)) s++; }
    bool eat(char c) { ws(); if (*s == c) { s++; return true; } return false; }
    NP fail(const std::string &m) { if (C.err.empty()) C.err = m; return nullptr; }

    NP expr()
    {
        NP l = term();
        if (!l) return nullptr;
        for (;;) {
            if (eat('+')) { NP r = term(); if (!r) return nullptr; l = op(Node::ADD, {l, r}); }
            else if (eat('-')) { NP r = term(); if (!r) return nullptr; l = op(Node::SUB, {l, r}); }
            else return l;
        }
    }
    NP term()
    {
        NP l = unary();
        if (!l) return nullptr;
        for (;;) {
            if (eat('*')) { NP r = unary(); if (!r) return nullptr; l = op(Node::MUL, {l, r}); }
            else if (eat('/')) { NP r = unary(); if (!r) return nullptr; l = op(Node::DIV, {l, r}); }
            else return l;
        }
    }
    NP unary()
    {
        if (eat('-')) { NP x = unary(); return x ? op(Node::NEG, {x}) : nullptr; }
        if (eat('+')) return unary();
        NP p = primary();
        ws();
        if (*s == '^')
            return fail("'^' is not supported in bin expressions");
        return p;
    }
    NP primary()
    {
        ws();
        if (eat('(')) { NP e = expr(); if (!e) return nullptr; if (!eat(')')) return fail("missing ')'"); return e; }
        if (isdigit((unsigned char)*s) || *s == '.') {
            char *e;
            double v = strtod(s, &e);
            if (e == s) return fail("bad number");
            s = e;
            return num(v);
        }
        if (isalpha((unsigned char)*s) || *s == '_') {
            const char *b = s;
            while (isalnum((unsigned char)*s) || *s == '_' || *s == '.') s++;
            std::string name(b, s);
            ws();
            if (*s == '(') {
                s++;
                std::vector<NP> args;
                if (!eat(')')) {
                    for (;;) {
                        NP e = expr();
                        if (!e) return nullptr;
                        args.push_back(e);
                        if (eat(')')) break;
                        if (!eat(',')) return fail("expected ',' in call to " + name);
                    }
                }
                if (name == "if" && args.size() == 3) return op(Node::IF, args);
                if (name == "floor" && args.size() == 1) return op(Node::FLOOR, args);
                return fail("function '" + name + "' is not supported in bin expressions");
            }
            return var(name);
        }
        return fail(std::string("unexpected '") + (*s ? std::string(1, *s) : std::string("end")) + "'");
    }
    NP var(const std::string &name)
    {
        if (name == "Dx") return op(Node::DX, {});
        if (name == "Dy") return op(Node::DY, {});
        if (name == "Dz") return op(Node::DZ, {});
        if (name == "PI") return num(M_PI);
        if (C.reinhart && name == "rbin") {
            /* parameters evaluated as constants */
            const char *pn[8] = {"MF", "RHS", "rNx", "rNy", "rNz", "Ux", "Uy", "Uz"};
            auto n = std::make_shared<Node>();
            n->k = Node::RBIN;
            for (int i = 0; i < 8; i++) {
                NP v = var(pn[i]);
                if (!v) return nullptr;
                double d;
                if (!constant(v, d)) return fail(std::string("Reinhart parameter ") + pn[i] + " must be constant");
                n->a.push_back(num(d));
            }
            return n;
        }
        if (C.reinhart && name == "Nrbins") {
            NP mf = var("MF");
            double m;
            if (!mf || !constant(mf, m)) return fail("MF must be constant");
            return num(reinhart_nbins(m));
        }
        auto it = C.defs.find(name);
        if (it != C.defs.end()) {
            if (++C.depth > 64) return fail("recursive definition of " + name);
            Parser q(C, it->second.c_str());
            NP e = q.expr();
            C.depth--;
            return e;
        }
        if (C.reinhart) {
            static const std::map<std::string, double> dflt = {
                {"MF", 1}, {"RHS", 1}, {"rNx", 0}, {"rNy", 0}, {"rNz", -1}, {"Ux", 0}, {"Uy", 1}, {"Uz", 0}};
            auto d = dflt.find(name);
            if (d != dflt.end()) return num(d->second);
        }
        return fail("undefined variable '" + name + "' in bin expression");
    }
    static bool constant(const NP &n, double &v)
    {
        switch (n->k) {
        case Node::NUM: v = n->v; return true;
        case Node::NEG: { double a; if (!constant(n->a[0], a)) return false; v = -a; return true; }
        case Node::ADD: case Node::SUB: case Node::MUL: case Node::DIV: {
            double a, b;
            if (!constant(n->a[0], a) || !constant(n->a[1], b)) return false;
            v = n->k == Node::ADD ? a + b : n->k == Node::SUB ? a - b : n->k == Node::MUL ? a * b : a / b;
            return true;
        }
        case Node::IF: {
            double a, b, c;
            if (!constant(n->a[0], a) || !constant(n->a[1], b) || !constant(n->a[2], c)) return false;
            v = a > 0 ? b : c;
            return true;
        }
        case Node::FLOOR: { double a; if (!constant(n->a[0], a)) return false; v = floor(a); return true; }
        default: return false;
        }
    }
};

void emit(const NP &n, std::vector<gb_binins> &out)
{
    double c;
    if (Parser::constant(n, c)) {
        out.push_back({(float)GB_OP_CONST, (float)c, 0.f, 0.f});
        return;
    }
    switch (n->k) {
    case Node::DX: out.push_back({(float)GB_OP_DX, 0, 0, 0}); return;
    case Node::DY: out.push_back({(float)GB_OP_DY, 0, 0, 0}); return;
    case Node::DZ: out.push_back({(float)GB_OP_DZ, 0, 0, 0}); return;
    case Node::NEG: emit(n->a[0], out); out.push_back({(float)GB_OP_NEG, 0, 0, 0}); return;
    case Node::FLOOR: emit(n->a[0], out); out.push_back({(float)GB_OP_FLOOR, 0, 0, 0}); return;
    case Node::ADD: case Node::SUB: case Node::MUL: case Node::DIV:
        emit(n->a[0], out);
        emit(n->a[1], out);
        out.push_back({(float)(n->k == Node::ADD ? GB_OP_ADD : n->k == Node::SUB ? GB_OP_SUB
                                : n->k == Node::MUL ? GB_OP_MUL : GB_OP_DIV), 0, 0, 0});
        return;
    case Node::IF:
        emit(n->a[0], out);
        emit(n->a[1], out);
        emit(n->a[2], out);
        out.push_back({(float)GB_OP_IF, 0, 0, 0});
        return;
    case Node::RBIN: {
        float p[8];
        for (int i = 0; i < 8; i++) p[i] = (float)n->a[i]->v;
        out.push_back({(float)GB_OP_RBIN, 0, 0, 0});
        out.push_back({p[0], p[1], p[2], p[3]});
        out.push_back({p[4], p[5], p[6], p[7]});
        return;
    }
    default: return;
    }
}

void add_defs(Ctx &C, const char *text)
{
    /* statements "name = expr" / "name : expr" separated by ';' (comments
     * in braces are skipped) */
    std::string t;
    int brace = 0;
    for (const char *p = text; *p; p++) {
        if (*p == '{') { brace++; continue; }
        if (*p == '}') { brace--; continue; }
        if (!brace) t += *p;
    }
    size_t i = 0;
    while (i < t.size()) {
        size_t j = t.find(';', i);
        if (j == std::string::npos) j = t.size();
        std::string st = t.substr(i, j - i);
        size_t e = st.find_first_of("=:");
        if (e != std::string::npos) {
            std::string name = st.substr(0, e);
            size_t a = name.find_first_not_of(" \t\r\n"), b = name.find_last_not_of(" \t\r\n");
            if (a != std::string::npos && name.find('(') == std::string::npos)
                C.defs[name.substr(a, b - a + 1)] = st.substr(e + 1);
            else if (a != std::string::npos && C.err.empty())
                C.err = "function definitions are not supported: " + name.substr(a, b - a + 1);
        }
        i = j + 1;
    }
}

}  // namespace

double reinhart_nbins(double MF)
{
    /* Nrbins = raccum(7*MF+1) (util/reinhartb.cal:39-47) */
    static const double tnaz[7] = {30, 30, 24, 24, 18, 12, 6};
    double acc = 0;
    int last = (int)(7 * MF + 1);
    for (int r = 0; r < last; r++) {
        if (r - (7 * MF - .5) > 0) acc += 1;
        else {
            int k = (int)floor((r + .5) / MF);
            acc += MF * tnaz[k < 0 ? 0 : (k > 6 ? 6 : k)];
        }
    }
    return acc;
}

int gb_compile_bin(const char *binv, const char *params, const char *calfile, const char *expr,
                   const char *nbins_expr, std::vector<gb_binins> &prog, int *nbins, std::string &err)
{
    Ctx C;
    if (calfile && *calfile) {
        const char *b = strrchr(calfile, '/');
        b = b ? b + 1 : calfile;
        if (!strcmp(b, "reinhartb.cal") || !strcmp(b, "reinhart.cal"))
            C.reinhart = true;
        else {
            FILE *fp = fopen(calfile, "r");
            if (!fp) { err = std::string("cannot open function file \"") + calfile + "\""; return -1; }
            std::string text;
            char buf[4096];
            size_t n;
            while ((n = fread(buf, 1, sizeof buf, fp)) > 0) text.append(buf, n);
            fclose(fp);
            add_defs(C, text.c_str());
        }
    }
    if (expr && *expr) add_defs(C, expr);
    if (params && *params) {
        std::string p(params);
        for (char &ch : p) if (ch == ',') ch = ';';
        add_defs(C, p.c_str());
    }
    if (!C.err.empty()) { err = C.err; return -1; }
    const char *bv = (binv && *binv) ? binv : "0";
    Parser P(C, bv);
    NP root = P.expr();
    P.ws();
    if (!root || *P.s) {
        err = C.err.empty() ? std::string("cannot parse bin expression \"") + bv + "\"" : C.err;
        return -1;
    }
    double cv;
    bool isconst = Parser::constant(root, cv);
    int nb = *nbins;
    if (nbins_expr && *nbins_expr) {
        Parser Q(C, nbins_expr);
        NP ne = Q.expr();
        double v;
        if (!ne || !Parser::constant(ne, v)) { err = C.err.empty() ? "bad bin count expression" : C.err; return -1; }
        nb = (int)(v + .5);
    }
    if (isconst) {
        /* rt/rcontrib.c:124-131: a constant bin must be 0 */
        if ((int)(cv + 1.5) != 1) { err = std::string("illegal non-zero constant for bin (") + bv + ")"; return -1; }
        nb = 1;
    } else if (nb <= 0) {
        err = "unspecified or illegal bin count for modifier";
        return -1;
    }
    prog.clear();
    emit(root, prog);
    prog.push_back({(float)GB_OP_END, 0, 0, 0});
    if (prog.size() > GB_BINPROG_MAX) { err = "bin expression too long"; return -1; }
    *nbins = nb;
    return 0;
}
