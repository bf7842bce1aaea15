/*
 * binexpr.cpp -- compiles rcontrib bin expressions into the device byte
 * code (gbcommon.h).
 *
 * The reference evaluates -b expressions with its interpreted calcomp
 * language (common/calexpr.c, common/caldefn.c, common/calfunc.c) once per
 * contributing ray (rt/rcontrib.c:301-304).  Here the expression and the
 * definitions it uses (-f function files, -e and -p definitions) are
 * compiled once on the host into a stack program that the kernels run:
 *
 *  - the calcomp grammar (common/calexpr.c:672-860): + - * / and a right
 *    associative ^ whose left operand may carry one sign (-x^2 is (-x)^2),
 *    numbers, variables, calls, parentheses;
 *  - definitions "name = expr;" and "name : expr;", with arguments
 *    "f(a, b) = expr;"; comments in braces;
 *  - the built-in functions of common/calfunc.c:56-73 except rand: if,
 *    select, floor, ceil, sqrt, exp, log, log10, sin, cos, tan, asin, acos,
 *    atan, atan2, max, min;
 *  - the ray direction Dx, Dy, Dz and PI;
 *  - the Reinhart sky bins of util/reinhartb.cal (rbin, Nrbins) built in;
 *  - the LBNL/Klems full, half and quarter bases of util/klems_full.cal,
 *    klems_half.cal and klems_quarter.cal (kbin, khbin, kqbin with their bin
 *    counts) built in: rfluxmtx receivers name these files;
 *  - the Shirley-Chiu square bins of util/disk2square.cal (scbin, with
 *    SCdim and the frame parameters) built in;
 *  - the CIE sky scanner bins of util/cieskyscan.cal (cbin, Ncbins, with
 *    the frame parameters) built in.
 *
 * Calls are expanded where they are used (partial evaluation): arguments
 * that are constants are substituted and folded, so recursion on constant
 * arguments (as in the Klems and Tregenza function files) unrolls, and an
 * if() or select() with a constant selector keeps only the branch taken; an
 * argument that stays an expression of the ray is computed once into a
 * temporary.  Anything else is rejected with a message naming it.
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

struct Node;
using NP = std::shared_ptr<Node>;

struct Node {
    enum Kind {
        NUM, DX, DY, DZ, NEG, ADD, SUB, MUL, DIV, POW, IF, FN1, ATAN2, MAXN, MINN, SELECT, FLOOR, RBIN, KBIN, SCBIN, CBIN,
        TEMP, LET,              /* residual only: temporary t, and let t = a[0] in a[1] */
        VAR, CALL               /* parsed only */
    } k;
    double v = 0;               /* NUM value; FN1 function; TEMP/LET temporary index */
    std::string name;           /* VAR, CALL */
    std::vector<NP> a;
};

NP mk(Node::Kind k, std::vector<NP> a = {}, double v = 0)
{
    auto n = std::make_shared<Node>();
    n->k = k;
    n->a = std::move(a);
    n->v = v;
    return n;
}
NP num(double v) { return mk(Node::NUM, {}, v); }
bool isnum(const NP &n) { return n->k == Node::NUM; }

struct Def {
    std::vector<std::string> params;
    NP body;
};

struct Ctx {
    std::map<std::string, Def> defs;
    bool reinhart = false;
    int klems = 0;              /* 1, 2, 4: built-in full, half, quarter Klems bins */
    bool shirchiu = false;      /* built-in Shirley-Chiu bins (scbin) */
    bool cie = false;           /* built-in CIE sky scanner bins (cbin) */
    std::string err;
    int temps = 0;
    NP fail(const std::string &m)
    {
        if (err.empty())
            err = m;
        return nullptr;
    }
};

/* ------------------------------------------------------------- parsing */

struct Parser {
    Ctx &C;
    const char *s;
    Parser(Ctx &c, const char *t) : C(c), s(t) {}
    void ws() { while (*s && isspace((unsigned char)*s)) s++; }
    bool eat(char c)
    {
        ws();
        if (*s == c) {
            s++;
            return true;
        }
        return false;
    }
    NP e1()                                   /* E1 -> E1 ADDOP E2 */
    {
        NP l = e2();
        while (l) {
            if (eat('+')) { NP r = e2(); if (!r) return nullptr; l = mk(Node::ADD, {l, r}); }
            else if (eat('-')) { NP r = e2(); if (!r) return nullptr; l = mk(Node::SUB, {l, r}); }
            else break;
        }
        return l;
    }
    NP e2()                                   /* E2 -> E2 MULOP E3 */
    {
        NP l = e3();
        while (l) {
            if (eat('*')) { NP r = e3(); if (!r) return nullptr; l = mk(Node::MUL, {l, r}); }
            else if (eat('/')) { NP r = e3(); if (!r) return nullptr; l = mk(Node::DIV, {l, r}); }
            else break;
        }
        return l;
    }
    NP e3()                                   /* E3 -> E4 ^ E3 */
    {
        NP l = e4();
        if (l && eat('^')) {
            NP r = e3();
            return r ? mk(Node::POW, {l, r}) : nullptr;
        }
        return l;
    }
    NP e4()                                   /* E4 -> ADDOP E5 */
    {
        if (eat('-')) {
            NP x = e5();
            return x ? mk(Node::NEG, {x}) : nullptr;
        }
        if (eat('+'))
            return e5();
        return e5();
    }
    NP e5()
    {
        ws();
        if (eat('(')) {
            NP e = e1();
            if (!e) return nullptr;
            if (!eat(')')) return C.fail("missing ')'");
            return e;
        }
        if (isdigit((unsigned char)*s) || *s == '.') {
            char *e;
            double v = strtod(s, &e);
            if (e == s) return C.fail("bad number");
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
                auto call = mk(Node::CALL);
                call->name = name;
                if (!eat(')')) {
                    for (;;) {
                        NP e = e1();
                        if (!e) return nullptr;
                        call->a.push_back(e);
                        if (eat(')')) break;
                        if (!eat(',')) return C.fail("expected ',' in call to " + name);
                    }
                }
                return call;
            }
            auto v = mk(Node::VAR);
            v->name = name;
            return v;
        }
        return C.fail(std::string("unexpected '") + (*s ? std::string(1, *s) : std::string("end")) + "'");
    }
};

/* statements "name = expr;", "name : expr;", "f(a,b) = expr;" (comments
 * in braces skipped) */
void add_defs(Ctx &C, const char *text)
{
    std::string t;
    int brace = 0;
    for (const char *p = text; *p; p++) {
        if (*p == '{') { brace++; continue; }
        if (*p == '}') { brace--; continue; }
        if (!brace) t += *p;
    }
    size_t i = 0;
    while (i < t.size() && C.err.empty()) {
        size_t j = t.find(';', i);
        if (j == std::string::npos) j = t.size();
        std::string st = t.substr(i, j - i);
        i = j + 1;
        size_t e = st.find_first_of("=:");
        if (e == std::string::npos) {
            if (st.find_first_not_of(" \t\r\n") != std::string::npos)
                C.err = "cannot parse definition \"" + st + "\"";
            continue;
        }
        std::string head = st.substr(0, e);
        Def d;
        size_t lp = head.find('(');
        std::string name = lp == std::string::npos ? head : head.substr(0, lp);
        size_t a = name.find_first_not_of(" \t\r\n"), b = name.find_last_not_of(" \t\r\n");
        if (a == std::string::npos) {
            C.err = "definition without a name";
            continue;
        }
        name = name.substr(a, b - a + 1);
        if (lp != std::string::npos) {
            size_t rp = head.find(')', lp);
            if (rp == std::string::npos) {
                C.err = "bad argument list in definition of " + name;
                continue;
            }
            std::string args = head.substr(lp + 1, rp - lp - 1);
            size_t q = 0;
            while (q <= args.size()) {
                size_t c = args.find(',', q);
                if (c == std::string::npos) c = args.size();
                std::string an = args.substr(q, c - q);
                size_t x = an.find_first_not_of(" \t\r\n"), y = an.find_last_not_of(" \t\r\n");
                if (x != std::string::npos) d.params.push_back(an.substr(x, y - x + 1));
                q = c + 1;
            }
        }
        Parser P(C, st.c_str() + e + 1);
        d.body = P.e1();
        P.ws();
        if (!d.body || *P.s) {
            if (C.err.empty()) C.err = "cannot parse the definition of " + name;
            continue;
        }
        C.defs[name] = d;
    }
}

/* ---------------------------------------------------- partial evaluation */

using Env = std::map<std::string, NP>;

struct Eval {
    Ctx &C;
    int depth = 0;
    explicit Eval(Ctx &c) : C(c) {}

    /* an expression needing no temporary: a constant, a ray component or a
     * temporary already */
    static bool trivial(const NP &n)
    {
        return n->k == Node::NUM || n->k == Node::DX || n->k == Node::DY || n->k == Node::DZ ||
               n->k == Node::TEMP;
    }

    NP pe(const NP &n, const Env &env)
    {
        if (!n || !C.err.empty())
            return nullptr;
        if (++depth > 400) {
            depth--;
            return C.fail("bin expression nests or recurses too deeply");
        }
        NP r = pe1(n, env);
        depth--;
        return r;
    }

    NP pe1(const NP &n, const Env &env)
    {
        switch (n->k) {
        case Node::NUM: case Node::DX: case Node::DY: case Node::DZ: case Node::TEMP:
            return n;
        case Node::VAR: return var(n->name, env);
        case Node::CALL: return call(n, env);
        case Node::NEG: {
            NP x = pe(n->a[0], env);
            if (!x) return nullptr;
            return isnum(x) ? num(-x->v) : mk(Node::NEG, {x});
        }
        case Node::ADD: case Node::SUB: case Node::MUL: case Node::DIV: case Node::POW: {
            NP x = pe(n->a[0], env), y = pe(n->a[1], env);
            if (!x || !y) return nullptr;
            if (isnum(x) && isnum(y)) {
                double a = x->v, b = y->v;
                switch (n->k) {
                case Node::ADD: return num(a + b);
                case Node::SUB: return num(a - b);
                case Node::MUL: return num(a * b);
                case Node::DIV: return num(a / b);
                default: return num(pow(a, b));
                }
            }
            return mk(n->k, {x, y});
        }
        default:
            return n;
        }
    }

    static std::string klems_fn(int kind) { return kind == 1 ? "kbin" : kind == 2 ? "khbin" : "kqbin"; }

    /* A Klems bin of the built-in basis for a constant normal and up vector;
     * RHS (+1 right-handed, -1 left-handed) comes from the parameters. */
    NP klems_node(const std::vector<NP> &a)
    {
        NP rhs = C.defs.count("RHS") ? var("RHS", Env()) : num(1);
        if (!rhs) return nullptr;
        if (!isnum(rhs)) return C.fail("RHS must be constant");
        NP n = mk(Node::KBIN);
        n->a.push_back(num(C.klems));
        n->a.push_back(rhs);
        for (auto &x : a) n->a.push_back(x);
        return n;
    }

    NP var(const std::string &name, const Env &env)
    {
        auto e = env.find(name);
        if (e != env.end()) return e->second;
        if (name == "Dx") return mk(Node::DX);
        if (name == "Dy") return mk(Node::DY);
        if (name == "Dz") return mk(Node::DZ);
        if (name == "PI") return num(M_PI);
        if ((C.reinhart && name == "rbin") || (C.shirchiu && name == "scbin" && !C.defs.count(name))) {
            const bool sc = name == "scbin";
            static const char *rn[8] = {"MF", "RHS", "rNx", "rNy", "rNz", "Ux", "Uy", "Uz"};
            static const char *sn[8] = {"SCdim", "RHS", "rNx", "rNy", "rNz", "Ux", "Uy", "Uz"};
            const char *const *pn = sc ? sn : rn;
            NP n = mk(sc ? Node::SCBIN : Node::RBIN);
            for (int i = 0; i < 8; i++) {
                NP v = var(pn[i], Env());
                if (!v) return nullptr;
                if (!isnum(v)) return C.fail(std::string("Reinhart parameter ") + pn[i] + " must be constant");
                n->a.push_back(v);
            }
            return n;
        }
        if (C.cie && !C.defs.count(name) && (name == "cbin" || name == "Ncbins")) {
            if (name == "Ncbins")
                return num(145);
            static const char *cn[7] = {"RHS", "rNx", "rNy", "rNz", "Ux", "Uy", "Uz"};
            static const double dflt[7] = {1, 0, 0, -1, 0, 1, 0};   /* +Y north, normal down */
            NP n = mk(Node::CBIN);
            n->a.push_back(num(0));
            for (int i = 0; i < 7; i++) {
                NP v = C.defs.count(cn[i]) ? var(cn[i], Env()) : num(dflt[i]);
                if (!v) return nullptr;
                if (!isnum(v)) return C.fail(std::string("CIE bin parameter ") + cn[i] + " must be constant");
                n->a.push_back(v);
            }
            return n;
        }
        if (C.klems && !C.defs.count(name)) {
            /* Nkbins / Nkhbins / Nkqbins, and the full basis's kbinN, kbinE,
             * kbinS, kbinW (walls, up +Z) and kbinD (skylight, up +Y) */
            const std::string fn = klems_fn(C.klems);
            if (name == "N" + fn + "s") return num(C.klems == 1 ? 145 : C.klems == 2 ? 77 : 41);
            static const struct { const char *suf; double v[6]; } pre[5] = {
                {"N", {0, -1, 0, 0, 0, 1}}, {"E", {-1, 0, 0, 0, 0, 1}}, {"S", {0, 1, 0, 0, 0, 1}},
                {"W", {1, 0, 0, 0, 0, 1}}, {"D", {0, 0, -1, 0, 1, 0}}};
            for (auto &q : pre)
                if (C.klems == 1 && name == fn + q.suf) {
                    std::vector<NP> a;
                    for (double v : q.v) a.push_back(num(v));
                    return klems_node(a);
                }
        }
        if (C.reinhart && name == "Nrbins") {
            NP mf = var("MF", Env());
            if (!mf || !isnum(mf)) return C.fail("MF must be constant");
            return num(reinhart_nbins(mf->v));
        }
        auto d = C.defs.find(name);
        if (d != C.defs.end()) {
            if (!d->second.params.empty())
                return C.fail("function " + name + " used without arguments");
            return pe(d->second.body, Env());
        }
        if (C.shirchiu) {
            static const std::map<std::string, double> dflt = {
                {"RHS", 1}, {"rNx", 0}, {"rNy", 0}, {"rNz", -1}, {"Ux", 0}, {"Uy", 1}, {"Uz", 0}};
            auto f = dflt.find(name);
            if (f != dflt.end()) return num(f->second);
        }
        if (C.reinhart) {
            static const std::map<std::string, double> dflt = {
                {"MF", 1}, {"RHS", 1}, {"rNx", 0}, {"rNy", 0}, {"rNz", -1}, {"Ux", 0}, {"Uy", 1}, {"Uz", 0}};
            auto f = dflt.find(name);
            if (f != dflt.end()) return num(f->second);
        }
        return C.fail("undefined variable '" + name + "' in bin expression");
    }

    NP call(const NP &n, const Env &env)
    {
        const std::string &f = n->name;
        const size_t na = n->a.size();
        if (f == "if") {
            if (na != 3) return C.fail("if() takes three arguments");
            NP c = pe(n->a[0], env);
            if (!c) return nullptr;
            if (isnum(c)) return pe(n->a[c->v > 0 ? 1 : 2], env);
            NP x = pe(n->a[1], env), y = pe(n->a[2], env);
            return x && y ? mk(Node::IF, {c, x, y}) : nullptr;
        }
        if (f == "select") {
            if (na < 2) return C.fail("select() takes an index and at least one value");
            NP i = pe(n->a[0], env);
            if (!i) return nullptr;
            if (isnum(i)) {
                int k = (int)(i->v + .5);
                if (k == 0) return num((double)(na - 1));
                if (k < 0 || k > (int)na - 1) return C.fail("illegal index in select()");
                return pe(n->a[k], env);
            }
            NP s = mk(Node::SELECT, {i});
            for (size_t j = 1; j < na; j++) {
                NP x = pe(n->a[j], env);
                if (!x) return nullptr;
                s->a.push_back(x);
            }
            return s;
        }
        static const std::map<std::string, int> fn1 = {
            {"sqrt", GB_FN_SQRT}, {"sin", GB_FN_SIN}, {"cos", GB_FN_COS}, {"tan", GB_FN_TAN},
            {"asin", GB_FN_ASIN}, {"acos", GB_FN_ACOS}, {"atan", GB_FN_ATAN}, {"exp", GB_FN_EXP},
            {"log", GB_FN_LOG}, {"log10", GB_FN_LOG10}, {"ceil", GB_FN_CEIL}};
        std::vector<NP> args;
        auto eval_args = [&]() -> bool {
            for (auto &a : n->a) {
                NP x = pe(a, env);
                if (!x) return false;
                args.push_back(x);
            }
            return true;
        };
        auto allnum = [&]() {
            for (auto &a : args) if (!isnum(a)) return false;
            return true;
        };
        auto f1 = fn1.find(f);
        if (f1 != fn1.end() || f == "floor") {
            if (na != 1) return C.fail(f + "() takes one argument");
            if (!eval_args()) return nullptr;
            if (allnum()) {
                const double x = args[0]->v;
                if (f == "floor") return num(floor(x));
                static double (*const tab[])(double) = {sqrt, sin, cos, tan, asin, acos, atan, exp, log, log10, ceil};
                return num(tab[f1->second](x));
            }
            if (f == "floor") return mk(Node::FLOOR, args);
            return mk(Node::FN1, args, f1->second);
        }
        if (f == "atan2") {
            if (na != 2) return C.fail("atan2() takes two arguments");
            if (!eval_args()) return nullptr;
            if (allnum()) return num(atan2(args[0]->v, args[1]->v));
            return mk(Node::ATAN2, args);
        }
        if (f == "max" || f == "min") {
            if (na < 1) return C.fail(f + "() takes at least one argument");
            if (!eval_args()) return nullptr;
            if (allnum()) {
                double m = args[0]->v;
                for (auto &a : args) m = f == "max" ? fmax(m, a->v) : fmin(m, a->v);
                return num(m);
            }
            return mk(f == "max" ? Node::MAXN : Node::MINN, args);
        }
        if (f == "rand")
            return C.fail("rand() is not supported in bin expressions");
        if (C.klems && f == klems_fn(C.klems) && !C.defs.count(f)) {
            if (na != 6) return C.fail(f + "() takes a normal and an up vector");
            if (!eval_args()) return nullptr;
            if (!allnum()) return C.fail(f + "() needs constant normal and up vectors");
            return klems_node(args);
        }
        auto d = C.defs.find(f);
        if (d == C.defs.end())
            return C.fail("function '" + f + "' is not defined");
        const Def &def = d->second;
        if (def.params.size() != na)
            return C.fail("function " + f + " called with the wrong number of arguments");
        if (!eval_args()) return nullptr;
        /* bind the arguments; one that stays an expression of the ray is
         * computed once, into a temporary */
        Env inner;
        std::vector<std::pair<int, NP>> lets;
        for (size_t j = 0; j < na; j++) {
            if (trivial(args[j])) {
                inner[def.params[j]] = args[j];
            } else {
                if (C.temps >= GB_BINTEMPS) return C.fail("bin expression needs too many temporaries");
                const int t = C.temps++;
                inner[def.params[j]] = mk(Node::TEMP, {}, t);
                lets.emplace_back(t, args[j]);
            }
        }
        NP body = pe(def.body, inner);
        if (!body) return nullptr;
        for (auto it = lets.rbegin(); it != lets.rend(); ++it)
            body = mk(Node::LET, {it->second, body}, it->first);
        return body;
    }
};

/* --------------------------------------------------------------- emission */

struct Emitter {
    std::vector<gb_binins> &out;
    int sp = 0, maxsp = 0;
    explicit Emitter(std::vector<gb_binins> &o) : out(o) {}
    void put(int op, float a = 0.f, int push = 0)
    {
        out.push_back({(float)op, a, 0.f, 0.f});
        sp += push;
        if (sp > maxsp) maxsp = sp;
    }
    void emit(const NP &n)
    {
        switch (n->k) {
        case Node::NUM: put(GB_OP_CONST, (float)n->v, 1); return;
        case Node::DX: put(GB_OP_DX, 0, 1); return;
        case Node::DY: put(GB_OP_DY, 0, 1); return;
        case Node::DZ: put(GB_OP_DZ, 0, 1); return;
        case Node::TEMP: put(GB_OP_LOAD, (float)n->v, 1); return;
        case Node::LET: emit(n->a[0]); put(GB_OP_STORE, (float)n->v, -1); emit(n->a[1]); return;
        case Node::NEG: emit(n->a[0]); put(GB_OP_NEG); return;
        case Node::FLOOR: emit(n->a[0]); put(GB_OP_FLOOR); return;
        case Node::FN1: emit(n->a[0]); put(GB_OP_FN1, (float)n->v); return;
        case Node::ADD: case Node::SUB: case Node::MUL: case Node::DIV: case Node::POW: case Node::ATAN2: {
            emit(n->a[0]);
            emit(n->a[1]);
            const int op = n->k == Node::ADD ? GB_OP_ADD : n->k == Node::SUB ? GB_OP_SUB
                         : n->k == Node::MUL ? GB_OP_MUL : n->k == Node::DIV ? GB_OP_DIV
                         : n->k == Node::POW ? GB_OP_POW : GB_OP_ATAN2;
            put(op, 0, -1);
            return;
        }
        case Node::IF:
            emit(n->a[0]);
            emit(n->a[1]);
            emit(n->a[2]);
            put(GB_OP_IF, 0, -2);
            return;
        case Node::MAXN: case Node::MINN: case Node::SELECT: {
            for (auto &a : n->a) emit(a);
            const int k = (int)n->a.size();
            put(n->k == Node::MAXN ? GB_OP_MAXN : n->k == Node::MINN ? GB_OP_MINN : GB_OP_SELECT,
                (float)(n->k == Node::SELECT ? k - 1 : k), 1 - k);
            return;
        }
        case Node::RBIN: case Node::KBIN: case Node::SCBIN: case Node::CBIN: {
            float p[8];
            for (int i = 0; i < 8; i++) p[i] = (float)n->a[i]->v;
            put(n->k == Node::RBIN ? GB_OP_RBIN : n->k == Node::KBIN ? GB_OP_KBIN
                : n->k == Node::SCBIN ? GB_OP_SCBIN : GB_OP_CBIN, 0, 1);
            out.push_back({p[0], p[1], p[2], p[3]});
            out.push_back({p[4], p[5], p[6], p[7]});
            return;
        }
        default:
            return;
        }
    }
};

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
        else if (!strcmp(b, "disk2square.cal"))
            C.shirchiu = true;
        else if (!strcmp(b, "cieskyscan.cal"))
            C.cie = true;
        else if (!strcmp(b, "klems_full.cal"))
            C.klems = 1;
        else if (!strcmp(b, "klems_half.cal"))
            C.klems = 2;
        else if (!strcmp(b, "klems_quarter.cal"))
            C.klems = 4;
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
    NP tree = P.e1();
    P.ws();
    if (!tree || *P.s) {
        err = C.err.empty() ? std::string("cannot parse bin expression \"") + bv + "\"" : C.err;
        return -1;
    }
    Eval E(C);
    NP root = E.pe(tree, Env());
    if (!root) { err = C.err; return -1; }
    int nb = *nbins;
    if (nbins_expr && *nbins_expr) {
        Parser Q(C, nbins_expr);
        NP ne = Q.e1();
        NP v = ne ? E.pe(ne, Env()) : nullptr;
        if (!v || !isnum(v)) { err = C.err.empty() ? "bad bin count expression" : C.err; return -1; }
        nb = (int)(v->v + .5);
    }
    if (isnum(root)) {
        /* rt/rcontrib.c:124-131: a constant bin must be 0 */
        if ((int)(root->v + 1.5) != 1) { err = std::string("illegal non-zero constant for bin (") + bv + ")"; return -1; }
        nb = 1;
    } else if (nb <= 0) {
        err = "unspecified or illegal bin count for modifier";
        return -1;
    }
    prog.clear();
    Emitter M(prog);
    M.emit(root);
    prog.push_back({(float)GB_OP_END, 0, 0, 0});
    if (prog.size() > GB_BINPROG_MAX) { err = "bin expression too long"; return -1; }
    if (M.maxsp > GB_BINSTACK - 1) { err = "bin expression nests too deeply"; return -1; }
    *nbins = nb;
    return 0;
}
